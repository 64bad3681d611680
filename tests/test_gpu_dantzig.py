"""dWorldStep on the GPU (a dense LCP per island, FP64, dantzig.cu) against
the reference's dWorldStep, through the C ABI.

Goldens: every snapshot of the step goldens (box stack, 256-body pile,
96-capsule pile) holds the recorded contacts and the reference's dWorldStep
multipliers, from its single-precision build (lambda_dantzig32) and its
double-precision build (lambda_dantzig), and the post-step state.  The
device solves the same box-constrained LCP exactly (its solution is unique
for each of the reference's two phases, see dantzig.cu), in FP64 from the
FP32 rows; the reference's two precisions differ from each other by up to
1.1e-3 of max |lambda| on the 10-box stack (an ill-conditioned island) and
1.2e-5 on the piles.  Tolerances: lambda within 1e-4 of max(1, max|lambda|)
of the double-precision reference (measured: 8e-6 on the stack, 1.4e-6 and
3.2e-6 on the piles), positions after
the step within 1e-4 m.  Where the reference's own solver gave up (its "LCP
internal error, s <= 0", recorded in the golden: the first box-stack
snapshot, whose four coplanar contacts per face make the matrix nearly
singular, after which the reference zeroes the multipliers it has not
reached) the device's solution is checked against the LCP conditions and
statics instead.  tests/golden/chain_step.npz is the reference's dWorldStep
on hanging chains of ball and limited hinge joints.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_step import contact_lambdas, snapshot_scene

pytestmark = pytest.mark.gpu

LAMBDA_RTOL = {"box_stack": 1e-4, "pile256": 1e-4, "capsule_pile96": 1e-4}
POS_ATOL = 1e-4


@pytest.mark.parametrize("name", ["box_stack", "pile256", "capsule_pile96"])
def test_dantzig_matches_reference_step(gblib, golden, name):
    from ode_gb300 import sim
    g = golden(f"step_{name}.npz")
    mode = int(g["ints"][2])
    worst, worst32, worst_p = 0.0, 0.0, 0.0
    for k in range(len(g["snaps"])):
        pre, cb, cs = g[f"s{k}_pre"], g[f"s{k}_cb"], g[f"s{k}_cs"]
        w = sim.GBWorld(snapshot_scene(g, pre, name))
        assert sim.step_contacts(w, cb, cs, mode, stepper=True) == 1, w.L.gbodeGetLastError()
        w.sync()
        lam = contact_lambdas(w.last_rows(), len(cb))
        if g[f"s{k}_dantzig_lcp_error"][1]:
            w.L.dJointGroupEmpty(w.group)
            w.close()
            continue
        ref, ref32 = g[f"s{k}_lambda_dantzig"], g[f"s{k}_lambda_dantzig32"]
        scale = max(1.0, float(np.abs(ref).max()))
        d = float(np.abs(lam - ref).max()) / scale
        worst = max(worst, d)
        worst32 = max(worst32, float(np.abs(lam - ref32).max()) / scale)
        assert d <= LAMBDA_RTOL[name], (k, d)
        post = w.state()
        dp = float(np.abs(post[:, 0:3] - g[f"s{k}_post_dantzig"][:, 0:3]).max())
        worst_p = max(worst_p, dp)
        assert dp <= POS_ATOL, (k, dp)
        w.L.dJointGroupEmpty(w.group)
        w.close()
    print(f"{name}: lambda vs double reference {worst:.2e}, vs single reference {worst32:.2e} of max|lambda|; "
          f"positions {worst_p:.2e} m")


def test_dantzig_stack_statics(gblib, golden):
    """The first box-stack snapshot, where the reference's solver gives up:
    the device's multipliers satisfy the LCP conditions (FP64 natural-map
    residual of its own rows ~1e-7 of max|lambda|; PGS at 20 sweeps leaves
    ~1e-2) and carry the stack: the normal forces of the ten interfaces sum
    to the weight each interface holds up, 9.81 x (1 + ... + 10) = 539.6 N
    (the reference returns 2.45 N)."""
    from ode_gb300 import sim
    g = golden("step_box_stack.npz")
    mode = int(g["ints"][2])
    assert g["s0_dantzig_lcp_error"][1] == 1
    w = sim.GBWorld(snapshot_scene(g, g["s0_pre"], "box_stack"))
    assert sim.step_contacts(w, g["s0_cb"], g["s0_cs"], mode, stepper=True) == 1
    w.sync()
    r64, ce, ml = w.last_residual()
    lam = contact_lambdas(w.last_rows(), len(g["s0_cb"]))
    total = float(lam[:, 0].sum())
    print(f"box stack dWorldStep: FP64 residual {r64 / max(1.0, ml):.2e}, complementarity {ce:.2e}, "
          f"sum of normal forces {total:.1f} N (reference {float(g['s0_lambda_dantzig'][:, 0].sum()):.2f} N)")
    assert r64 / max(1.0, ml) <= 1e-5
    assert abs(total - 9.81 * 55) <= 0.02 * 9.81 * 55
    w.L.dJointGroupEmpty(w.group)
    w.close()


def test_dantzig_chains_follow_reference(gblib, golden):
    """Ball and hinge joints (limits) stepped by dWorldStep: the reference's
    trajectory (tests/golden/chain_step.npz) to 5e-5 m over 60 steps."""
    from ode_gb300 import sim
    from test_gpu_joints import HORIZON, POS_TOL, ANGLE_TOL, _chain_scene
    L = gblib
    g = golden("chain_step.npz")
    sc = _chain_scene(g)
    w = sim.GBWorld(sc)
    hinges = [j for j, row in zip(w.joints, sc.joints) if int(row[0]) == 2]
    worst_p, worst_a = 0.0, 0.0
    for s in range(HORIZON):
        assert w.step_dantzig() == 1, L.gbodeGetLastError()
        st = w.state()
        worst_p = max(worst_p, float(np.abs(st[:, 0:3] - g["traj"][s, :, 0:3]).max()))
        ang = np.array([L.dJointGetHingeAngle(h) for h in hinges])
        worst_a = max(worst_a, float(np.abs(ang - g["angles"][s]).max()))
    assert w.sync() is None
    print(f"dWorldStep chains: over {HORIZON} steps max position difference {worst_p:.2e} m, "
          f"hinge angle {worst_a:.2e} rad")
    assert worst_p <= POS_TOL
    assert worst_a <= ANGLE_TOL
    w.close()


def test_dantzig_device_contacts_match_contact_joints(gblib):
    """dWorldStep on contacts made on the device (gbodeSpaceCollideContacts)
    against dWorldStep on the same collisions made as contact joints
    (dSpaceCollide, dCollide, dJointCreateContact): a 128-body pile settled
    by 90 quick steps, then 8 steps where both worlds start from the same
    state.  Both give each island the same rows in the same order (contacts
    by geom pair, then the joints), so the states after each step agree to
    the bit (measured: 1819 contacts, difference 0); the bound is 1e-5 m and
    1e-4 m/s, what an island's unique LCP solution (CFM > 0) would allow for
    a different row order."""
    from ode_gb300 import scenes, sim
    L = gblib
    sc = scenes.pile(128, seed=5)
    a, b = sim.GBWorld(sc), sim.GBWorld(sc)
    for _ in range(90):
        assert a.step_compat() == 1, L.gbodeGetLastError()
    worst_p, worst_v, ncont = 0.0, 0.0, 0
    for _ in range(8):
        pre = a.state()
        b.set_state(pre)
        assert a.step_dantzig("host") == 1, L.gbodeGetLastError()
        ncont += len(a.made)
        assert b.step_dantzig("device") == 1, L.gbodeGetLastError()
        pa, pb = a.state(), b.state()
        worst_p = max(worst_p, float(np.abs(pa[:, 0:3] - pb[:, 0:3]).max()))
        worst_v = max(worst_v, float(np.abs(pa[:, 19:25] - pb[:, 19:25]).max()))
    print(f"dWorldStep, device contacts vs contact joints: {ncont} contacts over 8 steps, "
          f"positions {worst_p:.2e} m, velocities {worst_v:.2e} m/s")
    assert ncont > 8 * 64
    assert worst_p <= 1e-5
    assert worst_v <= 1e-4
    a.close()
    b.close()


def _ptr(a):
    return a.ctypes.data if a is not None else None


def test_lcp_batch_random_problems(gblib):
    """The reference's LCP self-test (dTestSolveLCP, lcp.cpp:1205-1335)
    restated: random positive definite problems A = A2 A2^T (n = 100, A2
    uniform in [-1, 1]), b = A x0 + U(-0.1, 0.1), 50 unbounded variables and
    the rest in [-(U(0,1) + 0.01), U(0,1) + 0.01]; every solution satisfies
    A x = b + w and the complementarity conditions (FP64 tolerances scaled by
    the problem)."""
    L = gblib
    rng = np.random.default_rng(1205)
    count, n, nub = 16, 100, 50
    A2 = rng.uniform(-1, 1, (count, n, n))
    A = np.einsum("pij,pkj->pik", A2, A2)
    x0 = rng.uniform(-1, 1, (count, n))
    b = np.einsum("pij,pj->pi", A, x0) + rng.uniform(-0.1, 0.1, (count, n))
    lo = np.full((count, n), -np.inf)
    hi = np.full((count, n), np.inf)
    lo[:, nub:] = -(rng.uniform(0, 1, (count, n - nub)) + 0.01)
    hi[:, nub:] = rng.uniform(0, 1, (count, n - nub)) + 0.01
    A, b, lo, hi = [np.ascontiguousarray(v) for v in (A, b, lo, hi)]
    x = np.zeros((count, n))
    w = np.zeros((count, n))
    assert L.gbodeSolveLCPBatch(count, n, _ptr(A), _ptr(b), _ptr(lo), _ptr(hi), nub, None, _ptr(x), _ptr(w)) == 1, \
        L.gbodeGetLastError()
    worst_eq, worst_c = 0.0, 0.0
    nl = nh = nc = 0
    for p in range(count):
        scale = max(1.0, float(np.abs(b[p]).max()))
        r = np.einsum("ij,j->i", A[p], x[p]) - (b[p] + w[p])
        worst_eq = max(worst_eq, float(np.abs(r).max()) / scale)
        tx, tw = 1e-9 * max(1.0, float(np.abs(x[p]).max())), 1e-8 * scale
        for i in range(n):
            if abs(x[p, i] - lo[p, i]) <= tx and w[p, i] >= -tw:
                nl += 1
            elif abs(x[p, i] - hi[p, i]) <= tx and w[p, i] <= tw:
                nh += 1
            else:
                assert lo[p, i] - tx <= x[p, i] <= hi[p, i] + tx and abs(w[p, i]) <= tw, (p, i, x[p, i], w[p, i])
                nc += 1
                worst_c = max(worst_c, abs(w[p, i]) / scale)
    print(f"{count} random LCPs (n {n}, nub {nub}): |A x - b - w| {worst_eq:.2e}, free |w| {worst_c:.2e}; "
          f"at lo {nl}, at hi {nh}, free {nc}")
    assert worst_eq <= 1e-9
    assert nl > 0 and nh > 0


def test_lcp_batch_friction_rule(gblib):
    """findex: a normal row and two friction rows whose bounds are
    +-mu x_normal of the problem solved without them (lcp.cpp:889-917),
    against the same two-phase rule computed by enumeration on the host."""
    L = gblib
    rng = np.random.default_rng(7)
    n = 6  # two contacts: (normal, friction, friction) x 2
    count = 8
    J = rng.normal(size=(count, n, 6))
    A = np.einsum("pik,pjk->pij", J, J) + 0.05 * np.eye(n)
    b = rng.normal(size=(count, n))
    b[:, 0] = np.abs(b[:, 0]) + 0.5
    b[:, 3] = np.abs(b[:, 3]) + 0.5
    mu = 0.4
    lo = np.tile(np.array([0, -mu, -mu, 0, -mu, -mu], float), (count, 1))
    hi = np.tile(np.array([np.inf, mu, mu, np.inf, mu, mu]), (count, 1))
    findex = np.tile(np.array([-1, 0, 0, -1, 3, 3], np.int32), (count, 1))
    A, b, lo, hi = [np.ascontiguousarray(v) for v in (A, b, lo, hi)]
    x = np.zeros((count, n))
    w = np.zeros((count, n))
    assert L.gbodeSolveLCPBatch(count, n, _ptr(A), _ptr(b), _ptr(lo), _ptr(hi), 0, _ptr(findex), _ptr(x), _ptr(w)) == 1

    def box_lcp(A, b, lo, hi, free_mask):
        # enumerate active sets (tiny problems): the unique solution
        m = len(b)
        import itertools
        for states in itertools.product(range(3), repeat=m):
            xs = np.zeros(m)
            F = [i for i in range(m) if free_mask[i] and states[i] == 0]
            for i in range(m):
                if not free_mask[i]:
                    xs[i] = 0.0
                elif states[i] == 1:
                    if not np.isfinite(lo[i]):
                        break
                    xs[i] = lo[i]
                elif states[i] == 2:
                    if not np.isfinite(hi[i]):
                        break
                    xs[i] = hi[i]
            else:
                if F:
                    N = [i for i in range(m) if i not in F]
                    xs[F] = np.linalg.solve(A[np.ix_(F, F)], b[F] - A[np.ix_(F, N)] @ xs[N])
                ws = A @ xs - b
                ok = True
                for i in range(m):
                    if not free_mask[i]:
                        continue
                    if states[i] == 0:
                        ok &= lo[i] - 1e-12 <= xs[i] <= hi[i] + 1e-12
                    elif states[i] == 1:
                        ok &= ws[i] >= -1e-12
                    else:
                        ok &= ws[i] <= 1e-12
                if ok:
                    return xs
        raise AssertionError("no solution found")

    for p in range(count):
        normal = findex[p] < 0
        x1 = box_lcp(A[p], b[p], lo[p], hi[p], normal)
        lo2, hi2 = lo[p].copy(), hi[p].copy()
        for i in range(n):
            if findex[p, i] >= 0:
                hi2[i] = abs(mu * x1[findex[p, i]])
                lo2[i] = -hi2[i]
        fixed = np.array([findex[p, i] >= 0 and hi2[i] == 0 for i in range(n)])
        x2 = box_lcp(A[p], b[p], lo2, hi2, ~fixed)
        assert np.abs(x[p] - x2).max() <= 1e-9 * max(1.0, np.abs(x2).max()), (p, x[p], x2)
    print("friction rule: 8 two-contact problems match the host enumeration")
