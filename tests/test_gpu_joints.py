"""Ball and hinge joints (with hinge limits) on the GPU, through the C ABI,
against the reference.

The golden trajectory (tests/golden/chain.npz) is the reference (no-reorder
build) stepping hanging capsule chains -- hinge joints limited to +-60 deg
alternating with ball joints, the first link hung from the environment by a
ball joint -- with 200 SOR iterations per step, a converged solve.  The GPU
steps the same joints (created through dJointCreateBall/Hinge and the
anchor/axis/limit setters) with the coloured solver iterated to an FP32
residual of 1e-7: both follow the same converged dynamics, so body positions
agree to 5e-5 m and hinge angles (dJointGetHingeAngle) to 5e-4 rad over the
first 60 steps (0.25 s; the chains are chaotic double-pendulum-like systems
and the two FP32 solvers diverge slowly after that).
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POS_TOL = 5e-5
ANGLE_TOL = 5e-4
HORIZON = 60


def _chain_scene(g):
    from ode_gb300 import scenes
    p = g["params"]
    z = np.zeros(0, np.int32)
    return scenes.Scene("chain", g["bodies"], z, z, np.zeros((0, 3), np.float32), np.zeros((0, 12), np.float32),
                        np.zeros((0, 4), np.float32), dt=float(p[0]), gravity=tuple(float(x) for x in p[1:4]),
                        erp=float(p[4]), cfm=float(p[5]), w=float(p[6]), iterations=int(g["ints"][0]),
                        joints=g["joints"],
                        damping=tuple(float(x) for x in g["damping"]) if "damping" in g.files
                        else (0.0, 0.0, 0.01, 0.01, float("inf")))


def test_hanging_chains_follow_reference(gblib, golden):
    from ode_gb300 import sim
    L = gblib
    g = golden("chain.npz")
    sc = _chain_scene(g)
    w = sim.GBWorld(sc)
    L.dWorldSetQuickStepW(w.w, 1.0)
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    L.gbodeWorldSetResidualTarget(w.w, 1e-7, 5, 3000)
    hinges = [j for j, row in zip(w.joints, sc.joints) if int(row[0]) == 2]
    worst_p, worst_a = 0.0, 0.0
    for s in range(HORIZON):
        assert w.step_fused() == 1
        st = w.state()
        worst_p = max(worst_p, float(np.abs(st[:, 0:3] - g["traj"][s, :, 0:3]).max()))
        ang = np.array([L.dJointGetHingeAngle(h) for h in hinges])
        worst_a = max(worst_a, float(np.abs(ang - g["angles"][s]).max()))
    print(f"chains: {sc.nb} bodies, {len(sc.joints)} joints; over {HORIZON} steps max position difference "
          f"{worst_p:.2e} m, max hinge angle difference {worst_a:.2e} rad")
    assert worst_p <= POS_TOL
    assert worst_a <= ANGLE_TOL
    w.close()


def test_joint_rows_and_residual(gblib, golden):
    """Rows of every joint are present (3 per ball, 5 or 6 per hinge), the
    FP64 LCP residual of the solve meets the target, and the joint anchors
    stay together."""
    from ode_gb300 import sim
    L = gblib
    g = golden("chain.npz")
    sc = _chain_scene(g)
    w = sim.GBWorld(sc)
    L.dWorldSetQuickStepW(w.w, 1.0)
    L.gbodeWorldSetResidualTarget(w.w, 1e-6, 5, 3000)
    for _ in range(30):
        w.step_fused()
    w.sync()
    st = w.stats()
    nball = int((sc.joints[:, 0] == 1).sum())
    nhinge = int((sc.joints[:, 0] == 2).sum())
    assert 3 * nball + 5 * nhinge <= st.rows <= 3 * nball + 6 * nhinge
    r64, _, ml = w.last_residual()
    assert r64 / max(1.0, ml) <= 1.5e-6
    a1 = np.zeros(4, np.float32)
    F = ctypes.POINTER(ctypes.c_float)
    for j, row in zip(w.joints, sc.joints):
        if int(row[0]) == 1:
            L.dJointGetBallAnchor(j, a1.ctypes.data_as(F))
            assert np.all(np.isfinite(a1))
    w.close()


def test_dropped_chains_rest_on_the_ground(gblib):
    """Chains with ground contacts on the fused path (jointed neighbours do
    not collide): finite, above the floor, hinge angles near their limits at
    most, every step at the residual target."""
    from ode_gb300 import scenes, sim
    L = gblib
    sc = scenes.chains(64, seed=5)
    w = sim.GBWorld(sc)
    L.dWorldSetQuickStepW(w.w, 1.0)
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    L.gbodeWorldSetResidualTarget(w.w, 1e-4, 5, 3000)
    for _ in range(240):
        w.step_fused()
        assert w.stats().residual <= 1e-4
    st = w.state()
    assert np.isfinite(st).all()
    assert st[:, 2].min() > 0.0
    hinges = [j for j, row in zip(w.joints, sc.joints) if int(row[0]) == 2]
    ang = np.array([L.dJointGetHingeAngle(h) for h in hinges])
    assert np.abs(ang).max() < np.pi / 3 + 0.15
    print(f"dropped chains: {sc.nb} bodies, {w.stats().contacts} contacts, max |hinge angle| {np.abs(ang).max():.3f}")
    w.close()


def test_graph_replay_matches_plain_steps(gblib):
    """gbodeWorldStepFused with a CUDA graph gives the same states, to the
    bit, as the same steps issued one call at a time (chains with joints and
    ground contacts, residual-target sweeps)."""
    from ode_gb300 import scenes, sim
    L = gblib
    sc = scenes.chains(32, seed=9)
    worlds = [sim.GBWorld(sc), sim.GBWorld(sc)]
    for w in worlds:
        L.dWorldSetQuickStepW(w.w, 1.0)
        L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
        L.gbodeWorldSetResidualTarget(w.w, 1e-4, 5, 3000)
    for _ in range(40):
        worlds[0].step_fused()
        worlds[1].step_graph()
    a, b = worlds[0].state(), worlds[1].state()
    assert np.isfinite(a).all()
    assert np.array_equal(a, b), float(np.abs(a - b).max())
    assert worlds[1].stats().iterations > 0
    for w in worlds:
        w.close()


def test_hanging_vehicles_hinge2_follow_reference(gblib, golden):
    """Hinge2 joints (suspension ERP/CFM, steering locked by lo = hi stop,
    motored axles) on vehicles hung from the environment: the GPU follows
    the reference's converged trajectory (tests/golden/hinge2.npz), and
    dJointGetHinge2Angle1 matches."""
    from ode_gb300 import ode, sim
    L = gblib
    g = golden("hinge2.npz")
    sc = _chain_scene(g)
    w = sim.GBWorld(sc)
    L.dWorldSetQuickStepW(w.w, 1.0)
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    L.gbodeWorldSetResidualTarget(w.w, 1e-7, 5, 3000)
    h2 = [j for j, row in zip(w.joints, sc.joints) if int(row[0]) == 6]
    assert all(L.dJointGetType(j) == ode.dJointTypeHinge2 for j in h2)
    worst_p, worst_a = 0.0, 0.0
    for s in range(HORIZON):
        assert w.step_fused() == 1
        st = w.state()
        worst_p = max(worst_p, float(np.abs(st[:, 0:3] - g["traj"][s, :, 0:3]).max()))
        ang = np.array([L.dJointGetHinge2Angle1(j) for j in h2])
        worst_a = max(worst_a, float(np.abs(ang - g["angles"][s]).max()))
    print(f"hinge2 vehicles: {sc.nb} bodies; over {HORIZON} steps max position difference {worst_p:.2e} m, "
          f"max steering angle difference {worst_a:.2e} rad")
    assert worst_p <= POS_TOL
    assert worst_a <= ANGLE_TOL
    w.close()


def test_vehicles_drive_among_obstacles(gblib):
    """Vehicles with hinge2 wheels on the plane among static box obstacles
    (fused path): finite, wheels on the ground, every step at the residual
    target, the motored wheels spinning."""
    from ode_gb300 import scenes, sim
    L = gblib
    sc = scenes.vehicles(64, seed=6)
    w = sim.GBWorld(sc)
    L.dWorldSetQuickStepW(w.w, 1.0)
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    L.gbodeWorldSetResidualTarget(w.w, 1e-4, 5, 3000)
    for _ in range(120):
        w.step_fused()
        assert w.stats().residual <= 1e-4
    st = w.state()
    assert np.isfinite(st).all()
    wheels = np.arange(sc.nb) % 5 != 0
    assert st[wheels, 2].min() > 0.2 and st[wheels, 2].max() < 0.45
    assert np.abs(st[wheels, 22:25]).max() > 1.0  # angular velocity of the motored wheels
    print(f"vehicles: {sc.nb} bodies, {w.stats().contacts} contacts, wheel z in "
          f"[{st[wheels, 2].min():.3f}, {st[wheels, 2].max():.3f}]")
    w.close()


def test_damped_chains_follow_reference(gblib, golden):
    """World damping (linear and angular scales above their thresholds) and
    the angular speed cap, copied into the bodies at dBodyCreate, applied by
    the integration kernel: the GPU follows the reference's damped chains
    (tests/golden/damped.npz) as closely as the undamped ones."""
    from ode_gb300 import sim
    L = gblib
    g = golden("damped.npz")
    sc = _chain_scene(g)
    assert sc.damping[4] < float("inf")
    w = sim.GBWorld(sc)
    L.dWorldSetQuickStepW(w.w, 1.0)
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    L.gbodeWorldSetResidualTarget(w.w, 1e-7, 5, 3000)
    b0 = w.bodies[0]
    assert abs(L.dBodyGetLinearDamping(b0) - sc.damping[0]) < 1e-7
    assert abs(L.dBodyGetAngularDampingThreshold(b0) - sc.damping[3]) < 1e-6
    assert L.dBodyGetMaxAngularSpeed(b0) == np.float32(sc.damping[4])
    hinges = [j for j, row in zip(w.joints, sc.joints) if int(row[0]) == 2]
    worst_p, worst_a, wmax = 0.0, 0.0, 0.0
    for s in range(HORIZON):
        assert w.step_fused() == 1
        st = w.state()
        worst_p = max(worst_p, float(np.abs(st[:, 0:3] - g["traj"][s, :, 0:3]).max()))
        ang = np.array([L.dJointGetHingeAngle(h) for h in hinges])
        worst_a = max(worst_a, float(np.abs(ang - g["angles"][s]).max()))
        wmax = max(wmax, float(np.linalg.norm(st[:, 22:25], axis=1).max()))
    print(f"damped chains: over {HORIZON} steps max position difference {worst_p:.2e} m, max hinge angle "
          f"difference {worst_a:.2e} rad, max angular speed {wmax:.3f} (cap {sc.damping[4]})")
    assert worst_p <= POS_TOL
    assert worst_a <= ANGLE_TOL
    # the cap holds after the step, up to the angular damping applied after it
    assert wmax <= sc.damping[4] * (1 + 1e-5)
    w.close()


def test_damping_api_round_trip(gblib):
    """World and body damping setters and getters (thresholds are stored
    squared and returned as their square roots), dBodySetDampingDefaults,
    and the max angular speed default (infinity)."""
    L = gblib
    L.dInitODE2(0)
    w = L.dWorldCreate()
    assert L.dWorldGetMaxAngularSpeed(w) == float("inf")
    assert abs(L.dWorldGetLinearDampingThreshold(w) - 0.01) < 1e-7
    L.dWorldSetDamping(w, 0.1, 0.2)
    L.dWorldSetLinearDampingThreshold(w, 0.3)
    L.dWorldSetAngularDampingThreshold(w, 0.4)
    L.dWorldSetMaxAngularSpeed(w, 5.0)
    b = L.dBodyCreate(w)
    assert abs(L.dBodyGetLinearDamping(b) - 0.1) < 1e-7 and abs(L.dBodyGetAngularDamping(b) - 0.2) < 1e-7
    assert abs(L.dBodyGetLinearDampingThreshold(b) - 0.3) < 1e-6
    assert abs(L.dBodyGetAngularDampingThreshold(b) - 0.4) < 1e-6
    assert L.dBodyGetMaxAngularSpeed(b) == 5.0
    L.dBodySetLinearDamping(b, 0.0)
    L.dBodySetAngularDampingThreshold(b, 2.0)
    assert L.dBodyGetLinearDamping(b) == 0.0 and abs(L.dBodyGetAngularDampingThreshold(b) - 2.0) < 1e-6
    L.dBodySetDampingDefaults(b)
    assert abs(L.dBodyGetLinearDamping(b) - 0.1) < 1e-7
    assert abs(L.dBodyGetAngularDampingThreshold(b) - 0.4) < 1e-6
    L.dWorldDestroy(w)


def test_autotune_keeps_a_candidate(gblib):
    """gbodeWorldAutotune times every candidate on the running chains from
    the same saved state and leaves the fastest one set; the world comes out
    exactly as one plain fused step leaves it (a twin world checks this to the
    bit) and keeps stepping at the residual target."""
    from ode_gb300 import scenes, sim
    L = gblib
    sc = scenes.chains(64, seed=2)
    w, twin = sim.GBWorld(sc), sim.GBWorld(sc)
    for x in (w, twin):
        L.dWorldSetQuickStepW(x.w, 1.0)
        L.gbodeWorldSetWarmStart(x.w, 1, 1.0)
        for _ in range(60):
            x.step_fused()
        L.gbodeWorldSetResidualTarget(x.w, 1e-4, 5, 3000)
    t = w.autotune(steps=2, graph=True)
    twin.step_fused()
    assert np.array_equal(w.state(), twin.state())
    twin.close()
    assert t.candidates == 14 and t.ms_per_step > 0
    assert t.passes in (1, 2) and t.check_every in (5, 10)
    assert t.threads in (128, 256) and t.chunk_rows in (400, 800) and t.two_level in (0, 2)
    assert L.gbodeWorldGetManifoldPasses(w.w) == t.passes
    assert L.gbodeWorldGetSolverBlocks(w.w) == t.blocks
    assert L.gbodeWorldGetTwoLevelSweep(w.w) == t.two_level
    import ctypes
    th, ch = ctypes.c_int(0), ctypes.c_int(0)
    L.gbodeWorldGetSolverTiles(w.w, ctypes.byref(th), ctypes.byref(ch))
    assert (th.value, ch.value) == (t.threads, t.chunk_rows)
    for _ in range(20):
        w.step_graph()
    w.sync()
    assert w.stats().residual <= 1e-4
    print(f"autotune: blocks {t.blocks}, passes {t.passes}, check every {t.check_every}, threads {t.threads}, "
          f"staged rows {t.chunk_rows}, two-level {t.two_level}, {t.ms_per_step:.3f} ms/step")
    w.close()


def test_joint_feedback_of_a_hanging_chain(gblib):
    """dJointFeedback on ball joints (quickstep.cpp:3108-3181), in a static
    case: four spheres hanging straight down from the environment, each ball
    joint carries the weight below it -- f1 (on the upper sphere) is +m g of
    the spheres below and the joint's own sphere, f2 the opposite -- for plain
    steps and graph-replayed steps."""
    from ode_gb300 import ode, scenes, sim
    L = gblib
    n = 4
    masses = np.array([1.0, 2.0, 1.5, 0.5], np.float32)
    pos = np.zeros((n, 3), np.float32)
    pos[:, 2] = 5.0 - 0.5 * np.arange(n)
    q = np.tile(np.array([1, 0, 0, 0], np.float32), (n, 1))
    bodies = np.zeros((n, 20), np.float32)
    bodies[:, 0:3], bodies[:, 3:7], bodies[:, 13] = pos, q, masses
    bodies[:, 14:17] = 0.4 * masses[:, None] * 0.1 ** 2
    joints = np.zeros((n, scenes.JOINT_COLS), np.float32)
    for k in range(n):
        joints[k, 0:3] = (1, k, k - 1 if k > 0 else -1)
        joints[k, 3:6] = (0.0, 0.0, pos[k, 2] + 0.25)
    z = np.zeros(0, np.int32)
    sc = scenes.Scene("hanging", bodies, z, z, np.zeros((0, 3), np.float32), np.zeros((0, 12), np.float32),
                      np.zeros((0, 4), np.float32), dt=1 / 240, iterations=20, joints=joints)
    w = sim.GBWorld(sc)
    L.dWorldSetQuickStepW(w.w, 1.0)
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    L.gbodeWorldSetResidualTarget(w.w, 1e-7, 5, 3000)
    fbs = [ode.dJointFeedback() for _ in w.joints]
    for j, fb in zip(w.joints, fbs):
        L.dJointSetFeedback(j, ctypes.byref(fb))
    g = abs(sc.gravity[2])
    for label, stepper in (("plain", w.step_fused), ("graph", w.step_graph)):
        for _ in range(60):
            stepper()
        for k, fb in enumerate(fbs):
            below = float(masses[k:].sum()) * g
            print(f"{label}: joint {k} f1 z {fb.f1[2]:.4f} N, f2 z {fb.f2[2]:.4f} N, weight carried {below:.4f} N")
            # joint k attaches sphere k (body 1) to sphere k-1 above (body 2)
            assert abs(fb.f1[2] - below) <= 1e-3 * below
            if k > 0:
                assert abs(fb.f2[2] + below) <= 1e-3 * below
            assert abs(fb.f1[0]) < 1e-3 and abs(fb.f1[1]) < 1e-3
    w.close()
