"""GPU narrow and broad phase against the reference's golden vectors and the
oracle, through the C ABI (dCollide, dBoxBox, dSpaceCollide,
gbodeSpaceCollideContacts)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POS_TOL = 1e-5   # contact position / normal / depth (FP32)


def make_geom(L, space, cls, pos, R, dims):
    if cls == 0:
        g = L.dCreateSphere(space, float(dims[0]))
    elif cls == 1:
        g = L.dCreateBox(space, float(dims[0]), float(dims[1]), float(dims[2]))
    elif cls == 2:
        g = L.dCreateCapsule(space, float(dims[0]), float(dims[1]))
    else:
        return L.dCreatePlane(space, *[float(x) for x in dims])
    L.dGeomSetPosition(g, *[float(x) for x in pos])
    Rm = np.ascontiguousarray(R, np.float32)
    L.dGeomSetRotation(g, Rm.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return g


def test_dcollide_matches_reference(gblib, golden):
    from ode_gb300 import ode
    L = gblib
    g = golden("colliders.npz")
    n = len(g["count"])
    buf = (ode.dContactGeom * 8)()
    exact = 0
    worst = 0.0
    for k in range(n):
        c1, c2 = g["cls"][k]
        a = make_geom(L, None, c1, g["pos"][k, 0], g["R"][k, 0], g["dims"][k, 0])
        b = make_geom(L, None, c2, g["pos"][k, 1], g["R"][k, 1], g["dims"][k, 1])
        cnt = L.dCollide(a, b, int(g["flags"][k]), ctypes.addressof(buf), ctypes.sizeof(ode.dContactGeom))
        assert cnt == g["count"][k], (k, c1, c2, cnt, g["count"][k])
        same = True
        for i in range(cnt):
            p = np.array(buf[i].pos[:3]); nrm = np.array(buf[i].normal[:3]); d = buf[i].depth
            err = max(np.abs(p - g["cpos"][k, i]).max(), np.abs(nrm - g["cnrm"][k, i]).max(), abs(d - g["cdep"][k, i]))
            worst = max(worst, err)
            same &= err == 0
            assert buf[i].g1 == a and buf[i].g2 == b
        exact += same
        L.dGeomDestroy(a)
        L.dGeomDestroy(b)
    assert worst <= POS_TOL, worst
    print(f"dCollide: {n} cases, bit-exact {exact}/{n}, worst abs error {worst:.3g}")


def test_boxbox_feature_codes(gblib, golden):
    from ode_gb300 import ode
    L = gblib
    g = golden("colliders.npz")
    F = ctypes.POINTER(ctypes.c_float)
    buf = (ode.dContactGeom * 8)()
    checked = 0
    for k in np.nonzero((g["cls"][:, 0] == 1) & (g["cls"][:, 1] == 1))[0]:
        arrs = [np.zeros(4, np.float32) for _ in range(4)] + [np.zeros(12, np.float32) for _ in range(2)]
        p1, p2, s1, s2, R1, R2 = arrs
        p1[:3], p2[:3] = g["pos"][k, 0], g["pos"][k, 1]
        s1[:3], s2[:3] = g["dims"][k, 0][:3], g["dims"][k, 1][:3]
        R1[:], R2[:] = g["R"][k, 0], g["R"][k, 1]
        nrm = np.zeros(4, np.float32)
        depth = ctypes.c_float(0)
        code = ctypes.c_int(-1)
        n = L.dBoxBox(p1.ctypes.data_as(F), R1.ctypes.data_as(F), s1.ctypes.data_as(F), p2.ctypes.data_as(F),
                      R2.ctypes.data_as(F), s2.ctypes.data_as(F), nrm.ctypes.data_as(F), ctypes.byref(depth),
                      ctypes.byref(code), int(g["flags"][k]), ctypes.addressof(buf), ctypes.sizeof(ode.dContactGeom))
        assert n == g["count"][k]
        if n:
            assert code.value == g["code"][k], (k, code.value, g["code"][k])
        checked += 1
    assert checked > 0


def test_hash_space_pairs_match_reference(gblib, golden):
    L = gblib
    s = golden("space.npz")
    found = []
    cb = __import__("ode_gb300.ode", fromlist=["dNearCallback"]).dNearCallback(
        lambda data, o1, o2: found.append((L.dGeomGetData(o1) or 0, L.dGeomGetData(o2) or 0)))
    for ci in range(int(s["ncases"][0])):
        sp = L.dHashSpaceCreate(None)
        lv = s[f"c{ci}_levels"]
        L.dHashSpaceSetLevels(sp, int(lv[0]), int(lv[1]))
        cls = s[f"c{ci}_cls"]
        for i in range(len(cls)):
            gg = make_geom(L, sp, cls[i], s[f"c{ci}_pos"][i], s[f"c{ci}_R"][i], s[f"c{ci}_dims"][i])
            L.dGeomSetData(gg, ctypes.c_void_p(i))
        found.clear()
        L.dSpaceCollide(sp, None, cb)
        mine = {(min(a, b), max(a, b)) for a, b in found}
        assert len(mine) == len(found), "a pair was reported twice"
        ref = set(map(tuple, s[f"c{ci}_pairs"].tolist()))
        assert mine == ref, (ci, len(mine ^ ref))
        L.dSpaceDestroy(sp)


def _space_from_arrays(L, cls, pos, R, dims):
    sp = L.dHashSpaceCreate(None)
    for i in range(len(cls)):
        gg = make_geom(L, sp, cls[i], pos[i], R[i], dims[i])
        L.dGeomSetData(gg, ctypes.c_void_p(i))
    return sp


@pytest.mark.parametrize("exact", [0, 1])
def test_hash_space_settled_pile(gblib, golden, exact):
    """Reference mode reproduces the reference's pair set on a settled pile
    (including the overlapping pairs its unsigned bucket arithmetic drops);
    exact mode reports every AABB-overlapping pair."""
    from ode_gb300 import ode
    L = gblib
    g = golden("space_pile.npz")
    sp = _space_from_arrays(L, g["cls"], g["pos"], g["R"], g["dims"])
    L.gbodeHashSpaceSetExactPairs(sp, exact)
    found = []
    cb = ode.dNearCallback(lambda data, o1, o2: found.append((L.dGeomGetData(o1) or 0, L.dGeomGetData(o2) or 0)))
    L.dSpaceCollide(sp, None, cb)
    mine = {(min(a, b), max(a, b)) for a, b in found}
    ref = {tuple(p) for p in g["pairs"].tolist()}
    if not exact:
        assert mine == ref
    else:
        # make_golden.py counted 3 AABB-overlapping pairs the reference drops
        assert ref < mine and len(mine - ref) == 3
    L.dSpaceDestroy(sp)


def test_fused_contacts_match_oracle_on_a_pile(gblib, port):
    """Full-size broad + narrow phase (gbodeSpaceCollideContacts) on a settled
    32,768-body pile versus the oracle's hash space + dCollide on the same
    poses: the same contact set, counts bit-exact, geometry within 1e-5."""
    from ode_gb300 import scenes, sim
    sc = scenes.pile(32768, seed=1)
    w = sim.GBWorld(sc)
    for _ in range(150):
        w.step_fused()
    w.sync()
    st = w.state()
    L = gblib
    ng = sc.ng
    # broad phase: the GPU's candidate pairs (dSpaceCollide, GPU orientation)
    # against the oracle's hash space on the same poses, as unordered sets
    found = []
    from ode_gb300 import ode
    cb = ode.dNearCallback(lambda data, o1, o2: found.append((L.dGeomGetData(o1) or 0, L.dGeomGetData(o2) or 0)))
    L.dSpaceCollide(w.space, None, cb)
    n = sc.nb
    cls = sc.geom_cls
    pos = np.zeros((ng, 3), np.float32)
    R = np.zeros((ng, 12), np.float32)
    pos[:n] = st[:, 0:3]
    R[:n] = st[:, 7:19]
    R[n:, [0, 5, 10]] = 1
    pairs = port.hash_pairs(cls, sc.geom_body, pos, R, sc.geom_dims, np.arange(ng)[::-1].copy())
    assert {(min(a, b), max(a, b)) for a, b in found} == {(min(a, b), max(a, b)) for a, b in pairs.tolist()}
    # narrow phase: fused contacts against the oracle's dCollide in the GPU's orientation
    assert L.gbodeSpaceCollideContacts(w.space, w.w, w.group, ctypes.byref(w.surface), sc.maxc) == 1
    gc = w.contacts()
    L.dJointGroupEmpty(w.group)
    assert len(gc) > 10000
    mine = {}
    for c in gc:
        mine.setdefault((ng - 1 - int(c[7]), ng - 1 - int(c[8])), []).append(c)
    worst, exact, total = 0.0, 0, 0
    for a, b in found:
        cnt, out = port.collide(cls[a], pos[a], R[a], sc.geom_dims[a], cls[b], pos[b], R[b], sc.geom_dims[b], sc.maxc)
        lst = mine.get((a, b), [])
        assert cnt == len(lst), (a, b, cnt, len(lst))
        for c, o in zip(lst, out):
            e = max(np.abs(c[0:3] - o[0:3]).max(), np.abs(c[3:6] - o[3:6]).max(), abs(c[6] - o[6]))
            worst = max(worst, e)
            exact += e == 0
            total += 1
    assert total == len(gc)
    assert worst <= POS_TOL, worst
    print(f"pile: {len(found)} candidate pairs, {len(gc)} contacts, bit-exact {exact}, worst {worst:.3g}")
    w.close()
