"""Host-side behaviour of the C ABI that needs no GPU: joint geometry set and
read on the host (anchors, axes, hinge angle with an axis offset), world
defaults copied into new bodies, and the error returns of calls without the
state they need.  The hinge cases restate the reference's own unit tests
(tests/joints/hinge.cpp:103-784): a hinge between two bodies, or one body
and the static environment, an axis along +X or -X, one body turned about
X; the angle reads back the turn with the sign the axis and the body give,
dJointSetHingeAxisOffset with that angle keeps it, and turning the body back
reads 0 (tolerance 1e-4, as there)."""
from __future__ import annotations

import ctypes
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def L():
    from ode_gb300 import build, ode
    return ode.load(build.build())


def _vec(n=4):
    return (ctypes.c_float * n)()


def _turn(L, body, angle):
    R = _vec(12)
    L.dRFromAxisAndAngle(R, 1.0, 0.0, 0.0, angle)
    L.dBodySetRotation(body, R)


# (bodies attached, axis x, turned body, turn angle, angle read back);
# "b1b2": dJointAttach(j, b1, b2), "b1": (j, b1, NULL), "b2": (j, NULL, b2)
HALF_PI = math.pi / 2
HINGE_CASES = [
    ("b1b2", +1, "b2", +HALF_PI, -HALF_PI),
    ("b1b2", +1, "b2", -HALF_PI, +HALF_PI),
    ("b1b2", +1, "b1", +0.23, +0.23),
    ("b1b2", +1, "b1", -0.23, -0.23),
    ("b1b2", -1, "b2", +HALF_PI, +HALF_PI),
    ("b1b2", -1, "b2", -HALF_PI, -HALF_PI),
    ("b1b2", -1, "b1", +0.23, -0.23),
    ("b1b2", -1, "b1", -0.23, +0.23),
    ("b1", +1, "b1", +HALF_PI, +HALF_PI),
    ("b1", +1, "b1", -0.23, -0.23),
    ("b1", -1, "b1", +HALF_PI, -HALF_PI),
    ("b1", -1, "b1", -0.23, +0.23),
    ("b2", +1, "b2", +HALF_PI, -HALF_PI),
    ("b2", +1, "b2", -0.23, +0.23),
]


@pytest.mark.parametrize("attach,ax,turned,angle,expect", HINGE_CASES)
def test_hinge_angle_and_axis_offset(L, attach, ax, turned, angle, expect):
    w = L.dWorldCreate()
    b1 = L.dBodyCreate(w) if "b1" in attach else None
    b2 = L.dBodyCreate(w) if "b2" in attach else None
    if b1:
        L.dBodySetPosition(b1, 0.0, -1.0 if b2 else 0.0, 0.0)
    if b2:
        L.dBodySetPosition(b2, 0.0, 1.0 if b1 else 0.0, 0.0)
    j = L.dJointCreateHinge(w, None)
    L.dJointAttach(j, b1, b2)
    L.dJointSetHingeAnchor(j, 0.0, 0.0, 0.0)
    L.dJointSetHingeAxis(j, float(ax), 0.0, 0.0)
    body = b1 if turned == "b1" else b2
    assert abs(L.dJointGetHingeAngle(j)) < 1e-4
    _turn(L, body, angle)
    assert abs(L.dJointGetHingeAngle(j) - expect) < 1e-4
    L.dJointSetHingeAxisOffset(j, float(ax), 0.0, 0.0, expect)
    assert abs(L.dJointGetHingeAngle(j) - expect) < 1e-4
    _turn(L, body, 0.0)
    assert abs(L.dJointGetHingeAngle(j)) < 1e-4
    L.dWorldDestroy(w)


def test_hinge_default_axis_is_x(L):
    """tests/joints/hinge.cpp:103-133: without dJointSetHingeAxis the axis is
    +X (hinge.cpp:46-63); turning the second body by +90 deg reads -90."""
    w = L.dWorldCreate()
    b1, b2 = L.dBodyCreate(w), L.dBodyCreate(w)
    L.dBodySetPosition(b1, 0.0, -1.0, 0.0)
    j = L.dJointCreateHinge(w, None)
    L.dJointAttach(j, b1, b2)
    L.dJointSetHingeAnchor(j, 0.0, 0.0, 0.0)
    _turn(L, b2, HALF_PI)
    assert abs(L.dJointGetHingeAngle(j) + HALF_PI) < 1e-4
    L.dJointSetHingeAxisOffset(j, 1.0, 0.0, 0.0, -HALF_PI)
    assert abs(L.dJointGetHingeAngle(j) + HALF_PI) < 1e-4
    _turn(L, b2, 0.0)
    assert abs(L.dJointGetHingeAngle(j)) < 1e-4
    L.dWorldDestroy(w)


def _turned_pair(L, w):
    """tests/joints/ball.cpp:41-90, hinge2.cpp:36-85: two bodies at
    (-1, -2, -3) and (11, 22, 33), each turned 27 deg about its own axis."""
    a, b = L.dBodyCreate(w), L.dBodyCreate(w)
    L.dBodySetPosition(a, -1.0, -2.0, -3.0)
    L.dBodySetPosition(b, 11.0, 22.0, 33.0)
    for body, axis in ((a, (0.53, -0.71, 0.43)), (b, (1.2, 0.87, -0.33))):
        v = _vec(4)
        v[0], v[1], v[2] = axis
        L.dNormalize3(v)
        R = _vec(12)
        L.dRFromAxisAndAngle(R, v[0], v[1], v[2], 0.47123)
        L.dBodySetRotation(body, R)
    return a, b


def test_ball_anchor_set_to_itself(L):
    """A ball joint's anchor read back and set again reads the same anchor and
    leaves the bodies where they were (the set-up of tests/joints/ball.cpp)."""
    w = L.dWorldCreate()
    a, b = _turned_pair(L, w)
    j = L.dJointCreateBall(w, None)
    L.dJointAttach(j, a, b)
    q0 = np.array(L.dBodyGetQuaternion(a)[:4]), np.array(L.dBodyGetQuaternion(b)[:4])
    anc = _vec()
    L.dJointGetBallAnchor(j, anc)
    L.dJointSetBallAnchor(j, anc[0], anc[1], anc[2])
    anc2 = _vec()
    L.dJointGetBallAnchor(j, anc2)
    assert np.allclose(anc[:3], anc2[:3], atol=1e-4)
    assert np.allclose(q0[0], L.dBodyGetQuaternion(a)[:4]) and np.allclose(q0[1], L.dBodyGetQuaternion(b)[:4])
    L.dWorldDestroy(w)


def test_hinge2_axes_set_to_themselves(L):
    """tests/joints/hinge2.cpp:101-114: a hinge2's anchor and axes read back
    and set again (both axes, the first alone, the second alone) read the
    same; the axes are unit vectors in world coordinates."""
    w = L.dWorldCreate()
    a, b = _turned_pair(L, w)
    j = L.dJointCreateHinge2(w, None)
    L.dJointAttach(j, a, b)
    L.dJointSetHinge2Axis1(j, 0.0, 0.0, 1.0)
    L.dJointSetHinge2Axis2(j, 0.0, 1.0, 0.0)
    anc = _vec()
    L.dJointGetHinge2Anchor(j, anc)
    L.dJointSetHinge2Anchor(j, anc[0], anc[1], anc[2])
    x1, x2 = _vec(), _vec()
    L.dJointGetHinge2Axis1(j, x1)
    L.dJointGetHinge2Axis2(j, x2)
    assert np.allclose(x1[:3], [0, 0, 1], atol=1e-5) and np.allclose(x2[:3], [0, 1, 0], atol=1e-5)
    for first, second in ((x1, x2), (x1, None), (None, x2)):
        L.dJointSetHinge2Axes(j, first, second)
        y1, y2 = _vec(), _vec()
        L.dJointGetHinge2Axis1(j, y1)
        L.dJointGetHinge2Axis2(j, y2)
        assert np.allclose(y1[:3], x1[:3], atol=1e-5) and np.allclose(y2[:3], x2[:3], atol=1e-5)
    L.dWorldDestroy(w)


def test_safe_normalize3(L):
    """odemath.cpp:95-165: unit length by the largest component, sign kept;
    a zero vector stays zero and returns 0."""
    v = _vec()
    v[0], v[1], v[2] = 3.0, -4.0, 0.0
    assert L.dSafeNormalize3(v) == 1
    assert np.allclose(v[:3], [0.6, -0.8, 0.0], atol=1e-6)
    z = _vec()
    assert L.dSafeNormalize3(z) == 0 and list(z[:3]) == [0.0, 0.0, 0.0]


def test_world_defaults_reach_new_bodies(L):
    """A body takes the world's auto-disable and damping settings when it is
    created (objects.cpp:55-69, ode.cpp:265-285 dBodySetAutoDisableDefaults,
    dBodySetDampingDefaults); bodies made before keep theirs."""
    w = L.dWorldCreate()
    before = L.dBodyCreate(w)
    L.dWorldSetAutoDisableFlag(w, 1)
    L.dWorldSetAutoDisableSteps(w, 7)
    L.dWorldSetLinearDamping(w, 0.25)
    L.dWorldSetAngularDamping(w, 0.5)
    after = L.dBodyCreate(w)
    assert L.dBodyGetAutoDisableFlag(before) == 0 and L.dBodyGetAutoDisableFlag(after) == 1
    assert L.dBodyGetAutoDisableSteps(after) == 7
    assert abs(L.dBodyGetLinearDamping(after) - 0.25) < 1e-7 and abs(L.dBodyGetAngularDamping(after) - 0.5) < 1e-7
    assert L.dBodyGetLinearDamping(before) == 0.0
    L.dWorldDestroy(w)


def test_connected_bodies(L):
    """ode.cpp dAreConnected / dAreConnectedExcluding through a ball joint."""
    w = L.dWorldCreate()
    a, b, c = L.dBodyCreate(w), L.dBodyCreate(w), L.dBodyCreate(w)
    j = L.dJointCreateBall(w, None)
    L.dJointAttach(j, a, b)
    assert L.dAreConnected(a, b) and L.dAreConnected(b, a) and not L.dAreConnected(a, c)
    from ode_gb300 import ode
    assert not L.dAreConnectedExcluding(a, b, ode.dJointTypeBall)
    assert L.dAreConnectedExcluding(a, b, ode.dJointTypeContact)
    L.dWorldDestroy(w)


def test_snapshot_calls_without_a_snapshot(L):
    """gbodeWorldRestoreSnapshot without a saved snapshot (or without a world)
    returns 0 with a message and touches nothing."""
    w = L.dWorldCreate()
    assert L.gbodeWorldRestoreSnapshot(w) == 0
    assert b"no snapshot" in L.gbodeGetLastError()
    assert L.gbodeWorldRestoreSnapshot(None) == 0
    L.gbodeWorldDropSnapshot(w)
    L.gbodeWorldDropSnapshot(None)
    L.dWorldDestroy(w)


def test_hinge_axis_and_anchor_set_to_themselves(L):
    """tests/joints/hinge.cpp:848-865: a hinge between two turned bodies with
    its axis and anchor read back and set again keeps the bodies' poses, the
    axis, the anchor and a zero angle (the stepping half of that test needs
    the device)."""
    w = L.dWorldCreate()
    a, b = _turned_pair(L, w)
    j = L.dJointCreateHinge(w, None)
    L.dJointAttach(j, a, b)
    q0 = [np.array(L.dBodyGetQuaternion(x)[:4]) for x in (a, b)]
    ax, anc = _vec(), _vec()
    L.dJointGetHingeAxis(j, ax)
    L.dJointSetHingeAxis(j, ax[0], ax[1], ax[2])
    L.dJointGetHingeAnchor(j, anc)
    L.dJointSetHingeAnchor(j, anc[0], anc[1], anc[2])
    ax2, anc2 = _vec(), _vec()
    L.dJointGetHingeAxis(j, ax2)
    L.dJointGetHingeAnchor(j, anc2)
    assert np.allclose(ax[:3], ax2[:3], atol=1e-6) and np.allclose(anc[:3], anc2[:3], atol=1e-5)
    assert abs(np.linalg.norm(np.array(ax2[:3])) - 1.0) < 1e-6
    for x, q in zip((a, b), q0):
        assert np.allclose(L.dBodyGetQuaternion(x)[:4], q, atol=1e-6)
    assert abs(L.dJointGetHingeAngle(j)) < 1e-4
    L.dWorldDestroy(w)


def test_attach_takes_relative_values(L):
    """dJointAttach recomputes a joint's body-frame anchor and axes from their
    world values with the bodies just attached (ode.cpp:1434-1438,
    setRelativeValues in ball.cpp:178-183, hinge.cpp:362-372,
    hinge2.cpp:521-545): a joint attached with nothing set has its anchor at
    the first body's centre (the second body's anchor is set to the same
    point), and the hinge axis is the first body's x axis; the initial
    relative rotation is the bodies' current one (angle 0)."""
    w = L.dWorldCreate()
    a, b = _turned_pair(L, w)
    pa = np.array(L.dBodyGetPosition(a)[:3])
    for create, get_anchor in ((L.dJointCreateBall, L.dJointGetBallAnchor),
                               (L.dJointCreateHinge, L.dJointGetHingeAnchor),
                               (L.dJointCreateHinge2, L.dJointGetHinge2Anchor)):
        j = create(w, None)
        L.dJointAttach(j, a, b)
        anc = _vec()
        get_anchor(j, anc)
        assert np.allclose(anc[:3], pa, atol=1e-5)
    h = L.dJointCreateHinge(w, None)
    L.dJointAttach(h, a, b)
    ax = _vec()
    L.dJointGetHingeAxis(h, ax)
    Ra = np.array(L.dBodyGetRotation(a)[:12]).reshape(3, 4)
    assert np.allclose(ax[:3], Ra[:, 0], atol=1e-6)
    assert abs(L.dJointGetHingeAngle(h)) < 1e-6
    L.dWorldDestroy(w)


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("value", [1.0, 0.1, 1e-20, -1.0, -0.1, -1e-20])
def test_safe_normalize3_axis_vectors(L, axis, value):
    """The reference's dSafeNormalize3 unit test (tests/odemath.cpp:31-182):
    a vector along one axis, of length 1, 0.1 or 1e-20 and either sign,
    becomes that axis's unit vector with the sign kept, of length exactly 1
    in single precision."""
    v = _vec()
    v[axis] = value
    assert L.dSafeNormalize3(v) == 1
    e = np.zeros(3, np.float32)
    e[axis] = math.copysign(1.0, value)
    assert list(v[:3]) == list(e)
    x = np.array(v[:3], np.float32)
    assert np.sqrt(np.float32(x @ x)) == np.float32(1.0)


def test_safe_normalize3_large_components(L):
    """tests/odemath.cpp:164-181: (1e10, 0, 1e-20) normalises to length
    exactly 1; (1e10, 9999, 9) to length 1 within 1e-3."""
    v = _vec()
    v[0], v[1], v[2] = 9999999999.0, 0.0, 1e-20
    L.dSafeNormalize3(v)
    x = np.array(v[:3], np.float32)
    assert np.sqrt(np.float32(x @ x)) == np.float32(1.0)
    v[0], v[1], v[2] = 9999999999.0, 9999.0, 9.0
    L.dSafeNormalize3(v)
    x = np.array(v[:3], np.float32)
    assert abs(float(np.sqrt(x @ x)) - 1.0) < 1e-3


def test_reattach_with_one_or_no_body(L):
    """tests/joint.cpp:2986-3053 (host half): a hinge attached to two bodies
    is attached again to the first body alone, to the second alone and to
    none; each attach takes the joint's relative values from its current
    anchor (the stepping half needs the device)."""
    w = L.dWorldCreate()
    b1, b2 = L.dBodyCreate(w), L.dBodyCreate(w)
    L.dBodySetPosition(b1, 0.0, -1.0, 0.0)
    L.dBodySetPosition(b2, 0.0, 1.0, 0.0)
    j = L.dJointCreateHinge(w, None)
    L.dJointAttach(j, b1, b2)
    anc = _vec()
    for first, second, body in ((b1, None, b1), (None, b2, b2)):
        L.dJointAttach(j, first, second)
        assert L.dJointGetBody(j, 0) == body and not L.dJointGetBody(j, 1)
        L.dJointGetHingeAnchor(j, anc)
        assert all(math.isfinite(x) for x in anc[:3])
        assert abs(L.dJointGetHingeAngle(j)) < 1e-6
    L.dJointAttach(j, None, None)
    assert not L.dJointGetBody(j, 0) and not L.dJointGetBody(j, 1)
    L.dWorldDestroy(w)


def test_rotation_helpers_agree(L):
    """rotation.cpp: dRFromAxisAndAngle is dRfromQ of dQFromAxisAndAngle
    (rotation.cpp:160-188, 236-254) and equals Rodrigues' formula; a body
    given that rotation reports a unit quaternion of the same rotation
    (dBodySetRotation -> dQfromR, rotation.cpp:257-307)."""
    rng = np.random.default_rng(7)
    w = L.dWorldCreate()
    b = L.dBodyCreate(w)
    for _ in range(20):
        ax = rng.normal(size=3)
        ang = float(rng.uniform(-3.0, 3.0))
        R = _vec(12)
        L.dRFromAxisAndAngle(R, *map(float, ax), ang)
        q = _vec(4)
        L.dQFromAxisAndAngle(q, *map(float, ax), ang)
        R2 = _vec(12)
        L.dRfromQ(R2, q)
        assert np.allclose(R[:12], R2[:12], atol=1e-6)
        k = ax / np.linalg.norm(ax)
        K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
        rod = np.eye(3) + math.sin(ang) * K + (1 - math.cos(ang)) * K @ K
        assert np.allclose(np.array(R[:12]).reshape(3, 4)[:, :3], rod, atol=2e-6)
        L.dBodySetRotation(b, R)
        qb = np.array(L.dBodyGetQuaternion(b)[:4])
        assert abs(np.linalg.norm(qb) - 1.0) < 1e-6
        R3 = _vec(12)
        L.dRfromQ(R3, (ctypes.c_float * 4)(*map(float, qb)))
        assert np.allclose(R3[:12], R[:12], atol=2e-6)
    L.dWorldDestroy(w)


def test_geom_aabbs(L):
    """dGeomGetAABB as the reference's computeAABB gives it: sphere
    (sphere.cpp), box with a rotation (box.cpp: half sides through |R|),
    capsule along its z axis (capsule.cpp), and planes (plane.cpp:80-107:
    the half space below an axis-aligned plane, else unbounded)."""
    inf = float("inf")
    sp = L.dHashSpaceCreate(None)
    a = _vec(6)
    g = L.dCreateSphere(sp, 0.5)
    L.dGeomSetPosition(g, 1.0, 2.0, 3.0)
    L.dGeomGetAABB(g, a)
    assert list(a[:6]) == [0.5, 1.5, 1.5, 2.5, 2.5, 3.5]
    R = _vec(12)
    L.dRFromAxisAndAngle(R, 0.0, 0.0, 1.0, 0.5)
    g = L.dCreateBox(sp, 1.0, 2.0, 3.0)
    L.dGeomSetRotation(g, R)
    L.dGeomGetAABB(g, a)
    Rm = np.abs(np.array(R[:12]).reshape(3, 4)[:, :3])
    half = 0.5 * Rm @ np.array([1.0, 2.0, 3.0])
    assert np.allclose(a[1:6:2], half, atol=1e-6) and np.allclose(a[0:6:2], -half, atol=1e-6)
    g = L.dCreateCapsule(sp, 0.1, 0.8)
    L.dGeomSetRotation(g, R)
    L.dGeomGetAABB(g, a)
    ext = Rm[:, 2] * 0.4 + 0.1
    assert np.allclose(a[1:6:2], ext, atol=1e-6)
    for (pa, pb, pc, pd), want in (((0, 0, 1, 0), [-inf, inf, -inf, inf, -inf, 0.0]),
                                   ((-1, 0, 0, -5), [5.0, inf, -inf, inf, -inf, inf]),
                                   ((0, 2, 0, 4), [-inf, inf, -inf, 2.0, -inf, inf]),
                                   ((1, 1, 0, 0), [-inf, inf, -inf, inf, -inf, inf])):
        g = L.dCreatePlane(sp, float(pa), float(pb), float(pc), float(pd))
        L.dGeomGetAABB(g, a)
        assert list(a[:6]) == want
    L.dSpaceDestroy(sp)


def test_body_quaternion_is_normalised(L):
    """ode.cpp:379-387 dBodySetQuaternion: the quaternion is normalised and
    the rotation matrix derived from it."""
    w = L.dWorldCreate()
    b = L.dBodyCreate(w)
    L.dBodySetQuaternion(b, (ctypes.c_float * 4)(2.0, 0.0, 0.0, 0.0))
    assert list(L.dBodyGetQuaternion(b)[:4]) == [1.0, 0.0, 0.0, 0.0]
    L.dBodySetQuaternion(b, (ctypes.c_float * 4)(0.0, 0.0, 0.0, 3.0))
    assert list(L.dBodyGetQuaternion(b)[:4]) == [0.0, 0.0, 0.0, 1.0]
    R = np.array(L.dBodyGetRotation(b)[:12]).reshape(3, 4)[:, :3]
    assert np.allclose(R, np.diag([-1.0, -1.0, 1.0]), atol=1e-7)
    L.dWorldDestroy(w)


def test_sweep_momentum_setting(L):
    """gbodeWorldSetSweepMomentum: off by default, negative values read 0,
    values above 0.95 are clamped to 0.95; the setting needs no device."""
    w = L.dWorldCreate()
    assert L.gbodeWorldGetSweepMomentum(w) == 0.0
    for value, expect in ((0.8, 0.8), (-1.0, 0.0), (2.0, 0.95), (0.0, 0.0)):
        L.gbodeWorldSetSweepMomentum(w, value)
        assert L.gbodeWorldGetSweepMomentum(w) == pytest.approx(expect)
    L.dWorldDestroy(w)
