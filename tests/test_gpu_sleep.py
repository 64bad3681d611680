"""Auto-disable (sleeping bodies) on the GPU, through the C ABI, against the
reference's loop (tests/golden/sleep.npz).

The scene: two stacks of three unit boxes and a box dropped onto the first
stack.  The reference (no-reorder build, dSpaceCollide + near callback +
dWorldQuickStep) recorded poses and dBodyIsEnabled per step for two sets of
auto-disable parameters: (a) instantaneous velocity, thresholds 0.15, 10 idle
steps; (b) a 4-sample average, thresholds 0.02 / 0.05, 5 idle steps and
0.05 s.  In both, the stacks fall asleep, the struck one wakes when the box
lands, and everything is asleep at the end.

The enable state is a threshold decision on velocities the two FP32 solvers
compute in different row orders, so a body may cross a threshold a step
earlier or later: transitions are compared within TRANSITION_STEPS steps.
While a component sleeps its bodies do not move at all, which the tests
check exactly.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TRANSITION_STEPS = 3
NSTEPS = 300


def _transitions(en):
    """[(step, body, new state)] of a [steps, bodies] enable record."""
    out = []
    for s in range(1, len(en)):
        for b in np.nonzero(en[s] != en[s - 1])[0]:
            out.append((s, int(b), int(en[s, b])))
    return out


def _run(L, w, stepper, nsteps=NSTEPS):
    en = np.zeros((nsteps, len(w.bodies)), np.int32)
    traj = np.zeros((nsteps, len(w.bodies), 3), np.float32)
    for s in range(nsteps):
        assert stepper() == 1
        traj[s] = w.state()[:, 0:3]
        en[s] = [L.dBodyIsEnabled(b) for b in w.bodies]
    return en, traj


def _compare(tag, en, traj, g, calmer=False, pos_tol=0.02):
    """Same transitions (body, new state) in the same order per body, each
    within TRANSITION_STEPS steps of the reference's; with `calmer` (a solver
    converged further than the reference's 20 sweeps, whose resting contacts
    jitter less) a body may fall asleep any number of steps earlier."""
    ref_en, ref_traj = g[f"{tag}_enabled"], g[f"{tag}_traj"]
    got, ref = _transitions(en), _transitions(ref_en)
    print(f"[{tag}] reference transitions {ref}")
    print(f"[{tag}] GPU transitions       {got}")
    assert len(got) == len(ref), (got, ref)
    for (s1, b1, v1), (s2, b2, v2) in zip(sorted(got, key=lambda t: (t[1], t[0])),
                                          sorted(ref, key=lambda t: (t[1], t[0]))):
        assert b1 == b2 and v1 == v2, ((s1, b1, v1), (s2, b2, v2))
        if calmer and v2 == 0:
            assert s1 <= s2 + TRANSITION_STEPS, ((s1, b1, v1), (s2, b2, v2))
        else:
            assert abs(s1 - s2) <= TRANSITION_STEPS, ((s1, b1, v1), (s2, b2, v2))
    assert en[-1].sum() == 0 and ref_en[-1].sum() == 0
    # a sleeping body does not move
    for s in range(1, len(en)):
        still = (en[s] == 0) & (en[s - 1] == 0)
        assert np.array_equal(traj[s, still], traj[s - 1, still])
    err = float(np.abs(traj[-1] - ref_traj[-1, :, 0:3]).max())
    print(f"[{tag}] final position difference {err:.3g} m")
    assert err <= pos_tol


@pytest.mark.parametrize("tag", ["a", "b"])
def test_sleep_reference_order_loop(gblib, golden, tag):
    """The reference's user loop (dSpaceCollide -> near callback ->
    dJointCreateContact -> dWorldQuickStep) with the reference-order solver:
    the sleep stage runs on the device and the host-built islands hold the
    contacts of awake components only."""
    from ode_gb300 import ode, scenes, sim
    g = golden("sleep.npz")
    sc = scenes.sleep_stacks(seed=0, adis=tuple(float(x) for x in g[f"{tag}_adis"]))
    w = sim.GBWorld(sc, solver=ode.GBODE_SOLVER_REFERENCE_ORDER)
    b0 = w.bodies[0]
    assert gblib.dBodyGetAutoDisableFlag(b0) == 1
    assert gblib.dBodyGetAutoDisableAverageSamplesCount(b0) == int(sc.adis[5])
    en, traj = _run(gblib, w, w.step_compat)
    _compare(tag, en, traj, g)
    w.close()


@pytest.mark.parametrize("tag", ["a", "b"])
def test_sleep_fused_coloured(gblib, golden, tag):
    """The fused path (device contacts, coloured solver to an FP32 residual of
    1e-6): the same sleep and wake transitions; the struck stack wakes within
    a few steps of the reference's wake.  The converged solve leaves resting
    stacks with less jitter than the reference's 20 sweeps, so a stack may
    fall asleep earlier.  At the end the solver's contact list is empty:
    every component sleeps."""
    from ode_gb300 import scenes, sim
    L = gblib
    g = golden("sleep.npz")
    sc = scenes.sleep_stacks(seed=0, adis=tuple(float(x) for x in g[f"{tag}_adis"]))
    w = sim.GBWorld(sc)
    L.dWorldSetQuickStepW(w.w, 1.3)
    L.gbodeWorldSetResidualTarget(w.w, 1e-6, 5, 2000)
    en, traj = _run(L, w, w.step_fused)
    _compare(tag, en, traj, g, calmer=True, pos_tol=0.05)
    w.sync()
    st = w.stats()
    assert st.sleeping == len(w.bodies) and st.rows == 0 and st.contacts > 0
    w.close()


def test_sleeping_chain_wakes_on_enable(gblib):
    """A chain of jointed capsules hanging at rest (no contacts) falls asleep
    through its joints: no rows, no motion, multipliers kept; dBodyEnable on
    one link wakes the whole chain through the joint graph, and a graph
    replayed step (gbodeWorldStepFused) sleeps the same way."""
    from ode_gb300 import scenes, sim
    L = gblib
    sc = scenes.chains(4, seed=3, nmin=3, nmax=5, hang=True)
    sc.adis = (1, 0.05, 0.05, 5, 0.0, 1)
    sc.damping = (0.05, 0.05, 0.0, 0.0, float("inf"))  # settles the swing quickly
    w = sim.GBWorld(sc)
    L.dWorldSetQuickStepW(w.w, 1.0)
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    L.gbodeWorldSetResidualTarget(w.w, 1e-6, 5, 3000)
    asleep_at = None
    for s in range(1500):
        w.step_graph()
        if s % 25 == 24:
            w.sync()
            if w.stats().sleeping == len(w.bodies):
                asleep_at = s
                break
    assert asleep_at is not None, "the chains never fell asleep"
    st0 = w.state()
    for _ in range(10):
        w.step_graph()
    w.sync()
    assert w.stats().rows == 0
    assert np.array_equal(w.state(), st0)
    assert all(L.dBodyIsEnabled(b) == 0 for b in w.bodies)
    # wake the first chain's last link: its chain wakes, the others sleep on
    chain_bodies = {int(sc.joints[0, 1])}
    grown = True
    while grown:
        n0 = len(chain_bodies)
        for row in sc.joints:
            if int(row[1]) in chain_bodies or int(row[2]) in chain_bodies:
                chain_bodies.update(int(x) for x in row[1:3] if int(x) >= 0)
        grown = len(chain_bodies) > n0
    last = max(chain_bodies)
    L.dBodyEnable(w.bodies[last])
    L.dBodySetLinearVel(w.bodies[last], 0.5, 0.0, 0.0)
    w.step_fused()
    w.sync()
    st = w.stats()
    assert st.sleeping == len(w.bodies) - len(chain_bodies), (st.sleeping, len(chain_bodies))
    assert st.rows > 0
    en = np.array([L.dBodyIsEnabled(b) for b in w.bodies])
    assert en[sorted(chain_bodies)].all() and en.sum() == len(chain_bodies)
    print(f"chains asleep after {asleep_at + 1} steps; woke {len(chain_bodies)} linked bodies")
    w.close()


def test_auto_disable_api_round_trip(gblib):
    """World defaults, body setters and getters (thresholds stored squared),
    dBodySetAutoDisableFlag(0) restoring the world's steps, time and samples,
    dBodyDisable / dBodyEnable, and the reference's flag bit from
    dWorldGetAutoDisableFlag."""
    L = gblib
    L.dInitODE2(0)
    w = L.dWorldCreate()
    assert L.dWorldGetAutoDisableFlag(w) == 0
    assert L.dWorldGetAutoDisableSteps(w) == 10 and L.dWorldGetAutoDisableAverageSamplesCount(w) == 1
    assert abs(L.dWorldGetAutoDisableLinearThreshold(w) - 0.01) < 1e-7
    L.dWorldSetAutoDisableFlag(w, 1)
    assert L.dWorldGetAutoDisableFlag(w) == 16
    L.dWorldSetAutoDisableSteps(w, 7)
    L.dWorldSetAutoDisableTime(w, 0.25)
    L.dWorldSetAutoDisableAverageSamplesCount(w, 3)
    L.dWorldSetAutoDisableLinearThreshold(w, 0.2)
    b = L.dBodyCreate(w)
    assert L.dBodyGetAutoDisableFlag(b) == 1 and L.dBodyGetAutoDisableSteps(b) == 7
    assert abs(L.dBodyGetAutoDisableTime(b) - 0.25) < 1e-7
    assert L.dBodyGetAutoDisableAverageSamplesCount(b) == 3
    assert abs(L.dBodyGetAutoDisableLinearThreshold(b) - 0.2) < 1e-6
    L.dBodySetAutoDisableSteps(b, 2)
    L.dBodySetAutoDisableAverageSamplesCount(b, 9)
    L.dBodyDisable(b)
    assert L.dBodyIsEnabled(b) == 0
    L.dBodySetAutoDisableFlag(b, 0)  # also enables the body and restores the world's counts
    assert L.dBodyIsEnabled(b) == 1 and L.dBodyGetAutoDisableSteps(b) == 7
    assert L.dBodyGetAutoDisableAverageSamplesCount(b) == 3
    L.dBodyDisable(b)
    L.dBodyEnable(b)
    assert L.dBodyIsEnabled(b) == 1
    L.dWorldDestroy(w)


def test_disabled_body_keeps_forces_and_pose(gblib):
    """A body disabled by the caller and touching nothing is not stepped: no
    gravity, no motion, its accumulated force kept for when it wakes."""
    L = gblib
    L.dInitODE2(0)
    w = L.dWorldCreate()
    L.dWorldSetGravity(w, 0, 0, -9.81)
    a, b = L.dBodyCreate(w), L.dBodyCreate(w)
    L.dBodySetPosition(a, 0, 0, 5)
    L.dBodySetPosition(b, 3, 0, 5)
    L.dBodyDisable(a)
    L.dBodyAddForce(a, 1.0, 2.0, 3.0)
    for _ in range(5):
        assert L.dWorldQuickStep(w, 0.01) == 1
    pa, pb = L.dBodyGetPosition(a), L.dBodyGetPosition(b)
    assert (pa[0], pa[1], pa[2]) == (0.0, 0.0, 5.0)
    assert pb[2] < 5.0
    f = L.dBodyGetForce(a)
    assert (f[0], f[1], f[2]) == (1.0, 2.0, 3.0)
    L.dBodyEnable(a)
    assert L.dWorldQuickStep(w, 0.01) == 1
    v = L.dBodyGetLinearVel(a)
    assert abs(v[0] - 0.01) < 1e-6 and abs(v[1] - 0.02) < 1e-6  # the kept force, once, with unit mass
    L.dWorldDestroy(w)


def test_contact_feedback_skips_sleeping_contacts(gblib):
    """dJointFeedback of a contact joint in a sleeping component is left as
    the caller set it; a contact of an awake body gets its J^T lambda."""
    from ode_gb300 import ode
    L = gblib
    L.dInitODE2(0)
    w = L.dWorldCreate()
    L.dWorldSetGravity(w, 0, 0, -9.81)
    grp = L.dJointGroupCreate(0)
    a, b = L.dBodyCreate(w), L.dBodyCreate(w)
    L.dBodySetPosition(a, 0, 0, 0.5)
    L.dBodySetPosition(b, 3, 0, 0.5)
    L.dBodyDisable(a)
    fbs = []
    for body, x in ((a, 0.0), (b, 3.0)):
        c = ode.dContact()
        c.surface.mode = 0
        c.surface.mu = 0.0
        c.geom.pos[0], c.geom.pos[1], c.geom.pos[2] = x, 0.0, 0.0
        c.geom.normal[2] = 1.0
        c.geom.depth = 0.001
        j = L.dJointCreateContact(w, grp, ctypes.byref(c))
        L.dJointAttach(j, body, None)
        fb = ode.dJointFeedback()
        fb.f1[2] = 123.0
        L.dJointSetFeedback(j, ctypes.byref(fb))
        fbs.append(fb)
    assert L.dWorldQuickStep(w, 0.01) == 1
    assert fbs[0].f1[2] == 123.0  # the sleeping body's contact: untouched
    assert 5.0 < fbs[1].f1[2] < 20.0  # about m g for the awake unit-mass body
    assert L.dBodyIsEnabled(a) == 0
    L.dJointGroupDestroy(grp)
    L.dWorldDestroy(w)
