"""The stepping halves of the reference's joint unit tests, on the device.

tests/joints/ball.cpp:111-145, hinge.cpp:848-895 and hinge2.cpp:111-160 build
two identical pairs of bodies -- at (-1, -2, -3) and (11, 22, 33), each turned
27 degrees about its own axis -- joined by a ball, hinge or hinge2 joint, read
the second joint's anchor (and axes) back and set them again, and check that
four dWorldStep(0.5) steps move both pairs the same way: quaternions and
positions within 1e-4 (ball, hinge2) and 1e-6 (hinge).  hinge.cpp:899-921
drives a hinge between two bodies at the origin, axis along X, with an
unbounded motor (dParamFMax = dInfinity, dParamVel = 100) and checks that one
dWorldStep(0.001) brings the bodies' relative angular velocity to (100, 0, 0)
within 1e-2 of the target (the dSINGLE tolerance).  The host halves (the
get/set round trips without stepping) are in tests/test_host_api.py."""
from __future__ import annotations

import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _vec(n=4):
    return (ctypes.c_float * n)()


def _turned_pair(L, w):
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


def _reset_to_itself(L, kind, j):
    """The second joint's anchor (and axes) read back and set again."""
    anc = _vec()
    if kind == "ball":
        L.dJointGetBallAnchor(j, anc)
        L.dJointSetBallAnchor(j, anc[0], anc[1], anc[2])
    elif kind == "hinge":
        ax = _vec()
        L.dJointGetHingeAxis(j, ax)
        L.dJointSetHingeAxis(j, ax[0], ax[1], ax[2])
        L.dJointGetHingeAnchor(j, anc)
        L.dJointSetHingeAnchor(j, anc[0], anc[1], anc[2])
    else:
        L.dJointGetHinge2Anchor(j, anc)
        L.dJointSetHinge2Anchor(j, anc[0], anc[1], anc[2])
        x1, x2 = _vec(), _vec()
        L.dJointGetHinge2Axis1(j, x1)
        L.dJointGetHinge2Axis2(j, x2)
        L.dJointSetHinge2Axes(j, x1, x2)
        L.dJointSetHinge2Axes(j, x1, None)
        L.dJointSetHinge2Axes(j, None, x2)


@pytest.mark.parametrize("kind,tol", [("ball", 1e-4), ("hinge", 1e-6), ("hinge2", 1e-4)])
def test_joint_set_to_itself_steps_like_the_original(gblib, kind, tol):
    L = gblib
    w = L.dWorldCreate()
    if kind == "hinge":
        L.dWorldSetGravity(w, 0.0, 0.0, 0.0)  # hinge.cpp:793
    create = {"ball": L.dJointCreateBall, "hinge": L.dJointCreateHinge, "hinge2": L.dJointCreateHinge2}[kind]
    pairs, joints = [], []
    for _ in range(2):
        a, b = _turned_pair(L, w)
        j = create(w, None)
        L.dJointAttach(j, a, b)
        pairs.append((a, b))
        joints.append(j)
    _reset_to_itself(L, kind, joints[1])

    def pose(body):
        return np.array(L.dBodyGetQuaternion(body)[:4]), np.array(L.dBodyGetPosition(body)[:3])
    for b in range(2):
        assert np.allclose(pose(pairs[0][b])[0], pose(pairs[1][b])[0], atol=tol)
    for _ in range(4):
        assert L.dWorldStep(w, 0.5) == 1, L.gbodeGetLastError()
    moved = 0.0
    for b in range(2):
        (qa, pa), (qb, pb) = pose(pairs[0][b]), pose(pairs[1][b])
        assert np.allclose(qa, qb, atol=tol), (kind, b, qa, qb)
        assert np.allclose(pa, pb, atol=tol), (kind, b, pa, pb)
        moved = max(moved, float(np.abs(pa - np.array([[-1.0, -2.0, -3.0], [11.0, 22.0, 33.0]][b])).max()))
    print(f"{kind}: the pairs agree within {tol}; the joint moved the bodies by up to {moved:.3g} m")
    L.dWorldDestroy(w)


def test_hinge_motor_reaches_its_velocity_in_one_step(gblib):
    L = gblib
    from ode_gb300 import ode
    w = L.dWorldCreate()
    a, b = L.dBodyCreate(w), L.dBodyCreate(w)
    L.dBodySetPosition(a, 0.0, 0.0, 0.0)
    L.dBodySetPosition(b, 0.0, 0.0, 0.0)
    j = L.dJointCreateHinge(w, None)
    L.dJointAttach(j, a, b)
    L.dJointSetHingeAnchor(j, 0.0, 0.0, 0.0)
    target = 100.0
    L.dJointSetHingeParam(j, ode.dParamFMax, math.inf)
    L.dJointSetHingeParam(j, ode.dParamVel, target)
    assert L.dWorldStep(w, 0.001) == 1, L.gbodeGetLastError()
    v1, v2 = np.array(L.dBodyGetAngularVel(a)[:3]), np.array(L.dBodyGetAngularVel(b)[:3])
    rvel = v1 - v2
    print(f"relative angular velocity after one step: {rvel}")
    assert np.allclose(rvel, [target, 0.0, 0.0], atol=target * 1e-2)
    L.dWorldDestroy(w)
