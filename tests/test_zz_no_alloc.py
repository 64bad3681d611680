"""gbodeCollidePairsNoAlloc -- the narrow phase for callers that must not
allocate device memory while they run (programs that reserve all their GPU
memory up front and manage it themselves) -- against dCollide, the library's
ordinary entry point for the same colliders, through the C ABI.

The batch is the reference's collider corpus (every class pair of sphere,
box, capsule and plane).  Two calls in a row with different batches (pairs
in both orders, different contact caps and batch sizes) must each match
dCollide: counts exactly, contact position, normal and depth within 1e-5 --
so nothing left in the shared fixed scratch by one call leaks into the next.
This file is collected last on purpose.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POS_TOL = 1e-5  # contact position / normal / depth (FP32), as the dCollide tests

PAIR_GEOM = np.dtype([("cls", np.int32), ("body", np.int32), ("pad", np.int32, 2), ("dims", np.float32, 4),
                      ("pos", np.float32, 4), ("R", np.float32, 12)])


def _plane_unit(d):
    """dCreatePlane normalises (a, b, c, d) by |(a, b, c)|."""
    d = np.asarray(d, np.float32)
    l = np.float32(1.0) / np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    return d * l


def _records(g):
    n = len(g["count"])
    rec = np.zeros(2 * n, PAIR_GEOM)
    for k in range(n):
        for s in range(2):
            r = rec[2 * k + s]
            c = int(g["cls"][k, s])
            r["cls"] = c
            r["body"] = -1
            r["dims"] = _plane_unit(g["dims"][k, s]) if c == 4 else g["dims"][k, s]
            r["pos"][:3] = g["pos"][k, s]
            r["R"] = g["R"][k, s]
    assert PAIR_GEOM.itemsize == 96
    return rec


def _api_geom(L, cls, pos, R, dims):
    if cls == 0:
        h = L.dCreateSphere(None, float(dims[0]))
    elif cls == 1:
        h = L.dCreateBox(None, float(dims[0]), float(dims[1]), float(dims[2]))
    elif cls == 2:
        h = L.dCreateCapsule(None, float(dims[0]), float(dims[1]))
    else:
        return L.dCreatePlane(None, *[float(x) for x in dims])
    L.dGeomSetPosition(h, *[float(x) for x in pos])
    Rm = np.ascontiguousarray(R, np.float32)
    L.dGeomSetRotation(h, Rm.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return h


def _no_alloc(L, torch, rec, pairs, flags, capacity):
    dev = torch.device("cuda", 0)
    geoms_d = torch.from_numpy(rec.view(np.uint8).copy()).to(dev)
    pairs_d = torch.from_numpy(np.ascontiguousarray(pairs, np.int32)).to(dev)
    out_d = torch.full((capacity, 8), float("nan"), dtype=torch.float32, device=dev)
    first_d = torch.full((len(pairs) + 1,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    ok = L.gbodeCollidePairsNoAlloc(geoms_d.data_ptr(), len(rec), pairs_d.data_ptr(), len(pairs), flags,
                                    out_d.data_ptr(), capacity, first_d.data_ptr(), stream.cuda_stream)
    assert ok == 1, L.gbodeGetLastError()
    stream.synchronize()
    return out_d.cpu().numpy(), first_d.cpu().numpy()


def _check_against_dcollide(L, g, pairs, flags, out, first):
    from ode_gb300 import ode
    buf = (ode.dContactGeom * 8)()
    worst = 0.0
    total = 0
    for p, (ia, ib) in enumerate(pairs):
        ka, sa = divmod(int(ia), 2)
        kb, sb = divmod(int(ib), 2)
        a = _api_geom(L, g["cls"][ka, sa], g["pos"][ka, sa], g["R"][ka, sa], g["dims"][ka, sa])
        b = _api_geom(L, g["cls"][kb, sb], g["pos"][kb, sb], g["R"][kb, sb], g["dims"][kb, sb])
        n = L.dCollide(a, b, flags, ctypes.addressof(buf), ctypes.sizeof(ode.dContactGeom))
        assert first[p + 1] - first[p] == n, (p, int(first[p + 1] - first[p]), n)
        for i in range(n):
            row = out[first[p] + i]
            err = max(np.abs(row[0:3] - np.array(buf[i].pos[:3])).max(),
                      np.abs(row[4:7] - np.array(buf[i].normal[:3])).max(), abs(row[3] - buf[i].depth))
            worst = max(worst, err)
        total += n
        L.dGeomDestroy(a)
        L.dGeomDestroy(b)
    assert first[len(pairs)] == total
    assert worst <= POS_TOL, worst
    return total, worst


def test_no_alloc_collide_matches_dcollide_twice(gblib, golden):
    import torch
    L = gblib
    g = golden("colliders.npz")
    rec = _records(g)
    n = len(g["count"])
    # call 1: every corpus pair in its own order, up to 4 contacts per pair
    pairs1 = np.stack([2 * np.arange(n), 2 * np.arange(n) + 1], axis=1)
    out1, first1 = _no_alloc(L, torch, rec, pairs1, 4, 8 * n)
    t1, w1 = _check_against_dcollide(L, g, pairs1, 4, out1, first1)
    # call 2, straight after: a smaller batch, pairs reversed, up to 8 contacts
    sel = np.arange(0, n, 2)
    pairs2 = np.stack([2 * sel + 1, 2 * sel], axis=1)
    out2, first2 = _no_alloc(L, torch, rec, pairs2, 8, 8 * len(sel))
    t2, w2 = _check_against_dcollide(L, g, pairs2, 8, out2, first2)
    assert t1 > 1000 and t2 > 500
    print(f"no-alloc narrow phase: {n} pairs -> {t1} contacts (worst {w1:.3g}); "
          f"{len(sel)} reversed pairs -> {t2} contacts (worst {w2:.3g})")


def test_no_alloc_collide_leaves_free_memory_unchanged(gblib, golden):
    """The property the entry point is named for: once the buffers exist, a
    call takes no device memory (the device's free bytes are the same before
    and after it)."""
    import torch
    L = gblib
    g = golden("colliders.npz")
    rec = _records(g)
    n = len(g["count"])
    dev = torch.device("cuda", 0)
    geoms_d = torch.from_numpy(rec.view(np.uint8).copy()).to(dev)
    pairs = np.stack([2 * np.arange(n), 2 * np.arange(n) + 1], axis=1).astype(np.int32)
    pairs_d = torch.from_numpy(pairs).to(dev)
    out_d = torch.zeros((8 * n, 8), dtype=torch.float32, device=dev)
    first_d = torch.zeros((n + 1,), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def call():
        ok = L.gbodeCollidePairsNoAlloc(geoms_d.data_ptr(), len(rec), pairs_d.data_ptr(), n, 4, out_d.data_ptr(),
                                        8 * n, first_d.data_ptr(), stream.cuda_stream)
        assert ok == 1, L.gbodeGetLastError()
        stream.synchronize()

    call()  # the first call on the device may do its one-time set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dev)
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0, (free0, free1)
    assert int(first_d[n].item()) > 1000


def test_no_alloc_collide_rejects_misaligned_pairs(gblib):
    """A pair is read as one 8-byte load: a pairs pointer that is only 4-byte
    aligned is refused on the host before anything is launched."""
    import torch
    L = gblib
    dev = torch.device("cuda", 0)
    buf = torch.zeros(8, dtype=torch.int32, device=dev)
    geoms = torch.zeros(96, dtype=torch.uint8, device=dev)
    out = torch.zeros((8, 8), dtype=torch.float32, device=dev)
    first = torch.zeros(2, dtype=torch.int32, device=dev)
    assert L.gbodeCollidePairsNoAlloc(geoms.data_ptr(), 1, buf.data_ptr() + 4, 1, 4, out.data_ptr(), 8,
                                      first.data_ptr(), None) == 0
    assert "aligned" in L.gbodeGetLastError().decode()


def test_no_alloc_collide_rejects_oversized_batch(gblib):
    L = gblib
    from ode_gb300 import ode
    too_many = ode.GBODE_NOALLOC_MAX_PAIRS + 1
    # rejected before anything touches the (null) buffers
    assert L.gbodeCollidePairsNoAlloc(None, 0, None, too_many, 4, None, 0, None, None) == 0
    msg = L.gbodeGetLastError().decode()
    assert str(ode.GBODE_NOALLOC_MAX_PAIRS) in msg and "pairs" in msg
