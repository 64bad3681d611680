"""Edge cases of the device path through the C ABI: a world with no bodies, a
space with static geoms only, and bodies with no geoms or joints (free fall:
the step reduces to the reference's integration, quickstep.cpp:3299-3439 and
util.cpp:583-692: v += h g, then x += h v)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _surface():
    from ode_gb300 import ode, scenes
    s = ode.dSurfaceParameters()
    s.mode = scenes.dContactApprox1_1 | scenes.dContactApprox1_2 | scenes.dContactApprox1_N
    s.mu = 0.5
    return s


def test_empty_world_steps(gblib):
    """No bodies, no geoms: both steppers and the fused step return 1 and
    leave no error."""
    L = gblib
    w = L.dWorldCreate()
    sp = L.dHashSpaceCreate(None)
    grp = L.dJointGroupCreate(0)
    assert L.dWorldQuickStep(w, 0.01) == 1, L.gbodeGetLastError()
    assert L.dWorldStep(w, 0.01) == 1, L.gbodeGetLastError()
    s = _surface()
    assert L.gbodeSpaceCollideContacts(sp, w, grp, ctypes.byref(s), 4) == 1, L.gbodeGetLastError()
    assert L.dWorldQuickStep(w, 0.01) == 1, L.gbodeGetLastError()
    L.dJointGroupEmpty(grp)
    assert L.gbodeWorldSynchronize(w) == 1, L.gbodeGetLastError()
    L.dJointGroupDestroy(grp)
    L.dSpaceDestroy(sp)
    L.dWorldDestroy(w)


def test_static_geoms_only(gblib, port):
    """Five static planes (an open box) and no bodies.  The reference's hash
    space tests static geoms against each other too (collideAABBs skips only
    two geoms of one body, collision_space_internal.h:44-79; the big-box loop,
    collision_space.cpp:596-601): the near callback gets the plane pairs whose
    half-space AABBs overlap, the oracle's pair set, and dCollide finds no
    contact between planes; the device collision makes no contacts."""
    from ode_gb300 import ode, scenes
    L = gblib
    w = L.dWorldCreate()
    sp = L.dHashSpaceCreate(None)
    grp = L.dJointGroupCreate(0)
    planes = np.array([[0, 0, 1, 0], [1, 0, 0, 0], [-1, 0, 0, -5], [0, 1, 0, 0], [0, -1, 0, -5]], np.float32)
    for i, (a, b, c, d) in enumerate(planes):
        g = L.dCreatePlane(sp, float(a), float(b), float(c), float(d))
        L.dGeomSetData(g, ctypes.c_void_p(i + 1))
    calls, made = [], []
    contacts = (ode.dContact * 4)()

    def near(data, o1, o2):  # an exception here would not reach the test: record, check after
        calls.append(tuple(sorted((L.dGeomGetData(o1) - 1, L.dGeomGetData(o2) - 1))))
        made.append(L.dCollide(o1, o2, 4, ctypes.addressof(contacts[0].geom), ctypes.sizeof(ode.dContact)))
    cb = ode.dNearCallback(near)
    L.dSpaceCollide(sp, None, cb)
    assert all(k == 0 for k in made)
    n = len(planes)
    R = np.zeros((n, 12), np.float32)
    R[:, [0, 5, 10]] = 1
    expect = port.hash_pairs(np.full(n, scenes.PLANE, np.int32), np.full(n, -1, np.int32), np.zeros((n, 3), np.float32),
                             R, planes, np.arange(n)[::-1].copy())
    assert sorted(calls) == sorted(tuple(sorted(p)) for p in expect.tolist())
    s = _surface()
    assert L.gbodeSpaceCollideContacts(sp, w, grp, ctypes.byref(s), 4) == 1, L.gbodeGetLastError()
    assert L.dWorldQuickStep(w, 0.01) == 1, L.gbodeGetLastError()
    L.dJointGroupEmpty(grp)
    st = ode.gbodeStepStats()
    L.gbodeWorldGetStepStats(w, ctypes.byref(st))
    assert st.contacts == 0 and st.rows == 0
    L.dJointGroupDestroy(grp)
    L.dSpaceDestroy(sp)
    L.dWorldDestroy(w)


def test_free_fall(gblib):
    """Three bodies of different masses with no geoms or joints, one step of
    0.01 s under gravity -9.81: lvel z = h * (1/m) * (m g) and
    z = z0 + h * lvel z, as the reference integrates them; x, y and the
    rotation do not change."""
    from ode_gb300 import ode
    L = gblib
    w = L.dWorldCreate()
    L.dWorldSetGravity(w, 0.0, 0.0, -9.81)
    bodies = []
    for k, mass in enumerate((0.5, 2.0, 30.0)):
        b = L.dBodyCreate(w)
        m = ode.dMass()
        L.dMassSetBoxTotal(ctypes.byref(m), mass, 1.0, 1.0, 1.0)
        L.dBodySetMass(b, ctypes.byref(m))
        L.dBodySetPosition(b, float(k), 0.0, 10.0)
        bodies.append((b, mass))
    h = np.float32(0.01)
    assert L.dWorldQuickStep(w, float(h)) == 1, L.gbodeGetLastError()
    for k, (b, mass) in enumerate(bodies):
        m32, g = np.float32(mass), np.float32(-9.81)
        v = h * (np.float32(1) / m32) * (m32 * g)
        z = np.float32(10.0) + h * v
        lv = L.dBodyGetLinearVel(b)
        p = L.dBodyGetPosition(b)
        assert abs(lv[2] - v) <= 1e-6 and abs(lv[0]) == 0 and abs(lv[1]) == 0
        assert abs(p[2] - z) <= 2e-6 and p[0] == float(k) and p[1] == 0.0
        q = L.dBodyGetQuaternion(b)
        assert list(q[:4]) == [1.0, 0.0, 0.0, 0.0]
    L.dWorldDestroy(w)
