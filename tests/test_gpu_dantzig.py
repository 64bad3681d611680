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
