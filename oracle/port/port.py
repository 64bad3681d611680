"""ctypes binding of the oracle (the CPU restatement in ode_port.c).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libode_port.so")
SRC = os.path.join(HERE, "ode_port.c")


def build(force: bool = False) -> str:
    """Compile the oracle with the flags that keep the reference's float order."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "ode_port.h"))):
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-o", LIB, SRC,
                               "-lm"])
    return LIB


_F = ctypes.POINTER(ctypes.c_float)
_I = ctypes.POINTER(ctypes.c_int)
_D = ctypes.POINTER(ctypes.c_double)


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32).ctypes.data_as(_F)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32).ctypes.data_as(_I)


class Port:
    def __init__(self):
        self.lib = ctypes.CDLL(build())
        L = self.lib
        L.port_collide.restype = ctypes.c_int
        L.port_boxbox_code.restype = ctypes.c_int
        L.port_hash_pairs.restype = ctypes.c_int
        L.port_world_create.restype = ctypes.c_void_p
        L.port_world_create.argtypes = [ctypes.c_int, _F, _F, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.port_world_destroy.argtypes = [ctypes.c_void_p]
        L.port_world_get.argtypes = [ctypes.c_void_p, _F]
        L.port_world_set_state.argtypes = [ctypes.c_void_p, _F]
        L.port_world_set_dyn.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_float]
        L.port_world_set_threads.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.port_world_quickstep.argtypes = [ctypes.c_void_p, ctypes.c_int, _I, _I, _F, _F, _F, _I]
        L.port_sim_create.restype = ctypes.c_void_p
        L.port_sim_create.argtypes = [ctypes.c_void_p, ctypes.c_int, _I, _I, _F, _F, _F, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, _F]
        L.port_sim_destroy.argtypes = [ctypes.c_void_p]
        L.port_sim_step.argtypes = [ctypes.c_void_p]
        L.port_sim_last_contacts.argtypes = [ctypes.c_void_p, _I, _F, ctypes.c_int]
        L.port_world_quickstep_map.argtypes = [ctypes.c_void_p, ctypes.c_int, _I, _I, _F, _F, _F, _I, _I]
        L.port_world_set_residual.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.port_sim_last_stats.argtypes = [ctypes.c_void_p, _D]
        L.port_world_last_residual.argtypes = [ctypes.c_void_p, _D]
        L.port_lcp_residual.restype = ctypes.c_double
        L.port_lcp_residual.argtypes = [ctypes.c_int, _F, ctypes.c_int, _D, _D, _F, _D]
        L.port_rand_set_seed.argtypes = [ctypes.c_ulong]

    # ---------------------------------------------------------------- collide
    def collide(self, cls1, pos1, R1, dims1, cls2, pos2, R2, dims2, flags):
        out = np.zeros((8, 8), np.float32)
        keep = [np.ascontiguousarray(x, dtype=np.float32) for x in (pos1, R1, dims1, pos2, R2, dims2)]
        n = self.lib.port_collide(int(cls1), *[k.ctypes.data_as(_F) for k in keep[:3]], int(cls2),
                                  *[k.ctypes.data_as(_F) for k in keep[3:]], int(flags), out.ctypes.data_as(_F))
        return n, out[:n]

    def boxbox_code(self, p1, R1, s1, p2, R2, s2, flags):
        keep = [np.ascontiguousarray(x, dtype=np.float32) for x in (p1, R1, s1, p2, R2, s2)]
        return self.lib.port_boxbox_code(*[k.ctypes.data_as(_F) for k in keep], int(flags))

    def hash_pairs(self, cls, body, pos, R, dims, order, minlevel=-3, maxlevel=10):
        n = len(cls)
        cap = max(16, 64 * n)
        pairs = np.zeros((cap, 2), np.int32)
        keep = [np.ascontiguousarray(cls, np.int32), np.ascontiguousarray(body, np.int32),
                np.ascontiguousarray(pos, np.float32), np.ascontiguousarray(R, np.float32),
                np.ascontiguousarray(dims, np.float32), np.ascontiguousarray(order, np.int32)]
        np_ = self.lib.port_hash_pairs(n, keep[0].ctypes.data_as(_I), keep[1].ctypes.data_as(_I),
                                       keep[2].ctypes.data_as(_F), keep[3].ctypes.data_as(_F),
                                       keep[4].ctypes.data_as(_F), keep[5].ctypes.data_as(_I),
                                       int(minlevel), int(maxlevel), pairs.ctypes.data_as(_I), cap)
        assert np_ <= cap
        return pairs[:np_]

    # ---------------------------------------------------------------- world
    def world(self, bodies_in, params, iterations, dyn=0, reorder=0):
        return PortWorld(self, bodies_in, params, iterations, dyn, reorder)

    def lcp_residual(self, rows, invm, invI, lam):
        m = rows.shape[0]
        ce = ctypes.c_double(0)
        rows = np.ascontiguousarray(rows, np.float32)
        invm = np.ascontiguousarray(invm, np.float64)
        invI = np.ascontiguousarray(invI, np.float64)
        lam = np.ascontiguousarray(lam, np.float32)
        r = self.lib.port_lcp_residual(m, rows.ctypes.data_as(_F), invm.shape[0], invm.ctypes.data_as(_D),
                                       invI.ctypes.data_as(_D), lam.ctypes.data_as(_F), ctypes.byref(ce))
        return r, ce.value


class PortWorld:
    def __init__(self, port: Port, bodies_in, params, iterations, dyn, reorder):
        self.port = port
        self.nb = bodies_in.shape[0]
        self._keep = [np.ascontiguousarray(bodies_in, np.float32), np.ascontiguousarray(params, np.float32)]
        self.h = port.lib.port_world_create(self.nb, self._keep[0].ctypes.data_as(_F),
                                            self._keep[1].ctypes.data_as(_F), int(iterations), int(dyn),
                                            int(reorder))
        self.sim = None

    def __del__(self):
        try:
            if self.sim:
                self.port.lib.port_sim_destroy(self.sim)
            self.port.lib.port_world_destroy(self.h)
        except Exception:
            pass

    def state(self):
        out = np.zeros((self.nb, 25), np.float32)
        self.port.lib.port_world_get(self.h, out.ctypes.data_as(_F))
        return out

    def set_state(self, st):
        st = np.ascontiguousarray(st, np.float32)
        self.port.lib.port_world_set_state(self.h, st.ctypes.data_as(_F))

    def set_dyn(self, premature, factor, extra_delta):
        self.port.lib.port_world_set_dyn(self.h, premature, factor, extra_delta)

    def set_threads(self, threads: int, min_rows: int = 4096):
        """SOR sweeps of islands with at least `min_rows` rows on `threads`
        host threads (same multipliers as one thread, to the bit)."""
        self.port.lib.port_world_set_threads(self.h, int(threads), int(min_rows))

    def quickstep(self, cb, mode, cs, want_rows=False):
        nc = cb.shape[0]
        lam = np.zeros((max(nc, 1), 3), np.float32)
        rows = np.zeros((max(3 * nc, 1) * 2, 20), np.float32) if want_rows else None
        nrows = ctypes.c_int(0)
        cb = np.ascontiguousarray(cb, np.int32)
        mode = np.ascontiguousarray(mode, np.int32)
        cs = np.ascontiguousarray(cs, np.float32)
        self.port.lib.port_world_quickstep(self.h, nc, cb.ctypes.data_as(_I), mode.ctypes.data_as(_I),
                                           cs.ctypes.data_as(_F), lam.ctypes.data_as(_F),
                                           rows.ctypes.data_as(_F) if want_rows else None, ctypes.byref(nrows))
        if want_rows:
            return lam[:nc], rows[:nrows.value]
        return lam[:nc]

    def quickstep_contact_rows(self, cb, mode, cs):
        """One quickstep with the rows recorded and put in contact order (3
        rows per contact: normal, friction 1, friction 2; findex and body
        columns renumbered to that order).  Returns (lambda [nc,3], rows [3nc,20])."""
        nc = cb.shape[0]
        lam = np.zeros((max(nc, 1), 3), np.float32)
        rows = np.zeros((max(3 * nc, 1) * 2, 20), np.float32)
        slot = np.full(max(3 * nc, 1) * 2, -1, np.int32)
        nrows = ctypes.c_int(0)
        cb = np.ascontiguousarray(cb, np.int32)
        mode = np.ascontiguousarray(mode, np.int32)
        cs = np.ascontiguousarray(cs, np.float32)
        self.port.lib.port_world_quickstep_map(self.h, nc, cb.ctypes.data_as(_I), mode.ctypes.data_as(_I),
                                               cs.ctypes.data_as(_F), lam.ctypes.data_as(_F),
                                               rows.ctypes.data_as(_F), ctypes.byref(nrows),
                                               slot.ctypes.data_as(_I))
        m = nrows.value
        assert m == 3 * nc, "contact rows in three-row form only"
        slot = slot[:m]
        out = np.zeros((m, 20), np.float32)
        out[slot] = rows[:m]
        f = out[:, 18] >= 0
        out[f, 18] = slot[out[f, 18].astype(np.int64)]
        return lam[:nc], out

    def attach_space(self, geom_cls, geom_body, geom_pos, geom_R, geom_dims, levels, maxc, mode, surface):
        self._gkeep = [np.ascontiguousarray(geom_cls, np.int32), np.ascontiguousarray(geom_body, np.int32),
                       np.ascontiguousarray(geom_pos, np.float32), np.ascontiguousarray(geom_R, np.float32),
                       np.ascontiguousarray(geom_dims, np.float32), np.ascontiguousarray(surface, np.float32)]
        k = self._gkeep
        self.ng = len(geom_cls)
        self.sim = self.port.lib.port_sim_create(self.h, self.ng, k[0].ctypes.data_as(_I), k[1].ctypes.data_as(_I),
                                                 k[2].ctypes.data_as(_F), k[3].ctypes.data_as(_F),
                                                 k[4].ctypes.data_as(_F), levels[0], levels[1], maxc, mode,
                                                 k[5].ctypes.data_as(_F))

    def sim_step(self):
        return self.port.lib.port_sim_step(self.sim)

    def set_residual(self, on: bool = True):
        """Evaluate every step's FP64 LCP residual while stepping."""
        self.port.lib.port_world_set_residual(self.h, 1 if on else 0)

    def last_residual(self):
        """(FP64 residual, max |lambda|) of the last quickstep (set_residual on)."""
        out = np.zeros(2, np.float64)
        self.port.lib.port_world_last_residual(self.h, out.ctypes.data_as(_D))
        return float(out[0]), float(out[1])

    def last_stats(self):
        """Of the last sim_step: (collision s, quickstep s, FP64 residual,
        max |lambda|); the residual is relative after dividing by
        max(1, max |lambda|)."""
        out = np.zeros(4, np.float64)
        self.port.lib.port_sim_last_stats(self.sim, out.ctypes.data_as(_D))
        return float(out[0]), float(out[1]), float(out[2]), float(out[3])

    def last_contacts(self):
        n = self.port.lib.port_sim_last_contacts(self.sim, None, None, 0)
        cb = np.zeros((max(n, 1), 2), np.int32)
        cs = np.zeros((max(n, 1), 16), np.float32)
        self.port.lib.port_sim_last_contacts(self.sim, cb.ctypes.data_as(_I), cs.ctypes.data_as(_F), n)
        return cb[:n], cs[:n]


def world_inv_inertia(state, bodies_in):
    """World-frame inverse inertia R * I^-1 * R^T (float64) from a [nb,25]
    state and the body-frame inertias of a [nb,20] body table."""
    nb = state.shape[0]
    R = state[:, 7:19].reshape(nb, 3, 4)[:, :, :3].astype(np.float64)
    I = np.zeros((nb, 3, 3))
    I[:, 0, 0], I[:, 1, 1], I[:, 2, 2] = bodies_in[:, 14], bodies_in[:, 15], bodies_in[:, 16]
    I[:, 0, 1] = I[:, 1, 0] = bodies_in[:, 17]
    I[:, 0, 2] = I[:, 2, 0] = bodies_in[:, 18]
    I[:, 1, 2] = I[:, 2, 1] = bodies_in[:, 19]
    invI = np.linalg.inv(I)
    return np.einsum("bij,bjk,blk->bil", R, invI, R).reshape(nb, 9), 1.0 / bodies_in[:, 13].astype(np.float64)
