"""Momentum between the coloured solver's sweeps (gbodeWorldSetSweepMomentum)
through the C ABI.

The sweeps' multipliers and body accumulators move on by beta times their
change over the previous sweep.  A solution of the step's LCP is a fixed point
of that map as of the plain sweep, so the checks are those of the plain
solver: the residual target is reached (FP32 in the kernel, FP64 on the
device), the solution agrees with the plain solver's of the same step within
1e-3 m of position (both are solutions to a residual of 1e-4), the result is
the same to the bit run after run and under either sweep-sync mode, and on the
FP64 oracle's snapshots the result meets the same bounds as the plain
solver's (test_gpu_step.py)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BETA = 0.5


def landed_pile(L, n_worlds, nb=8192, seed=7):
    from ode_gb300 import scenes, sim
    sc = scenes.pile(nb, seed=seed)
    worlds = [sim.GBWorld(sc) for _ in range(n_worlds)]
    for w in worlds:
        L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
        L.dWorldSetQuickStepW(w.w, 1.0)
        L.dWorldSetQuickStepNumIterations(w.w, 30)
    for _ in range(300):
        for w in worlds:
            w.step_fused()
    return worlds


@pytest.mark.parametrize("two_level,classes,beta", [(0, 0, 0.5), (2, 4, 0.5), (2, 0, 0.8)])
def test_momentum_on_a_pile(gblib, two_level, classes, beta):
    """An 8,192-body pile that has landed, four steps to a residual of 1e-4:
    world 0 plain, worlds 1-3 with momentum (world 3 under grid barriers on
    the two-level sweep, whose default is neighbour waits): the one-level
    sweep, the two-level sweep with 4 split classes, and the two-level sweep
    with exact crossing colours at the benchmark's beta 0.8.  Every step
    reaches the target; the FP64 residual of the last step confirms it; the
    momentum worlds agree with each other to the bit, and after the first
    step with the plain world's positions within 1e-3 m (two solutions at a
    residual of 1e-4; later steps start from different states); the mean
    sweeps of both are printed."""
    from ode_gb300 import ode
    L = gblib
    worlds = landed_pile(L, 4)
    for i, w in enumerate(worlds):
        L.gbodeWorldSetTwoLevelSweep(w.w, two_level)
        if two_level:
            L.gbodeWorldSetCrossClasses(w.w, classes)
            L.gbodeWorldSetSweepSync(w.w, ode.GBODE_SYNC_GRID if i == 3 else ode.GBODE_SYNC_NEIGHBOURS)
        L.gbodeWorldSetSweepMomentum(w.w, beta if i else 0.0)
        L.gbodeWorldSetResidualTarget(w.w, 1e-4, 5, 3000)
    assert L.gbodeWorldGetSweepMomentum(worlds[1].w) == pytest.approx(beta)
    sweeps = {0: [], 1: []}
    for step in range(4):
        for w in worlds:
            assert w.step_fused() == 1, L.gbodeGetLastError()
        st = [w.stats() for w in worlds]
        for s in st:
            assert s.residual <= 1e-4, (step, s.residual, s.iterations)
        assert st[0].momentum == 0.0 and 0.0 <= st[1].momentum <= np.float32(beta)
        assert len({(s.iterations, s.rows, s.momentum) for s in st[1:]}) == 1, step
        a, b, c = (w.state() for w in worlds[1:])
        assert np.array_equal(a, b) and np.array_equal(a, c), step
        sweeps[0].append(st[0].iterations)
        sweeps[1].append(st[1].iterations)
        if step == 0:
            dpos = float(np.abs(worlds[0].state()[:, 0:3] - a[:, 0:3]).max())
    # the residual checks of the last step: the sweeps done at each, in order, the last at the solve's end
    import ctypes
    hist = np.zeros(256, np.float32)
    at = np.zeros(256, np.int32)
    n = L.gbodeWorldGetResidualHistory(worlds[1].w, hist.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 256)
    assert L.gbodeWorldGetResidualSweeps(worlds[1].w, at.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), 256) == n > 0
    assert np.all(np.diff(at[:n]) >= 0) and at[n - 1] == st[1].iterations and hist[n - 1] <= 1e-4
    r64, _, ml = worlds[1].last_residual()
    print(f"{'two' if two_level else 'one'}-level: sweeps plain {np.mean(sweeps[0]):.1f}, momentum "
          f"{np.mean(sweeps[1]):.1f} (beta at the end {st[1].momentum}); FP64 residual {r64 / max(1.0, ml):.2e}; "
          f"positions after the first step differ by {dpos:.2e} m")
    assert r64 / max(1.0, ml) <= 1.5e-4
    assert dpos <= 1e-3
    for w in worlds:
        w.close()


@pytest.mark.parametrize("beta", [BETA, 0.8])
@pytest.mark.parametrize("two_level", [0, 1])
@pytest.mark.parametrize("name", ["box_stack", "pile256", "capsule_pile96"])
def test_momentum_against_fp64_dantzig(gblib, golden, name, two_level, beta):
    """The momentum solver (beta 0.5 and 0.8) on every snapshot of the step goldens, solved to an
    FP32 residual of 1e-6, against the exact FP64 solution of quickstep's LCP
    (tests/golden/lcp_exact.npz, continued from the reference's dDOUBLE
    Dantzig multipliers): residual and complementarity relative to
    max|lambda_dantzig| within 1e-5, lambda within 2e-2 of max|lambda_exact|,
    M^-1 J^T lambda within 2e-3 -- the plain solver's bounds
    (test_coloured_solver_against_fp64_dantzig).  The snapshot on which the
    manifold row order cycles keeps its 3e-3 residual bound."""
    from oracle import lcp_exact as X
    from oracle.port.port import world_inv_inertia
    from ode_gb300 import sim
    from test_gpu_step import (CYCLING, EXACT_DV_TOL, EXACT_LAMBDA_TOL, FP64_RESID_TOL, FP64_TARGET,
                               snapshot_scene)
    L = gblib
    g = golden(f"step_{name}.npz")
    ex = golden("lcp_exact.npz")
    mode = int(g["ints"][2])
    report = []
    for k in range(len(g["snaps"])):
        if g[f"s{k}_dantzig_lcp_error"][1]:
            continue
        pre, cb, cs = g[f"s{k}_pre"], g[f"s{k}_cb"], g[f"s{k}_cs"]
        sc = snapshot_scene(g, pre, name)
        w = sim.GBWorld(sc)
        L.dWorldSetQuickStepW(w.w, 1.0)
        L.gbodeWorldSetTwoLevelSweep(w.w, two_level)
        L.gbodeWorldSetSweepMomentum(w.w, beta)
        cyc = CYCLING.get((name, k))
        L.gbodeWorldSetResidualTarget(w.w, FP64_TARGET, 10, 5000 if cyc else 40000)
        assert sim.step_contacts(w, cb, cs, mode) == 1, L.gbodeGetLastError()
        w.sync()
        st = w.stats()
        rows = w.last_rows()
        lam = rows[:, 19].astype(np.float64)
        invI, invm = world_inv_inertia(pre, sc.bodies)
        A, b, lo, hi, fi = X.dense_problem(rows, invm, invI)
        ref = g[f"s{k}_lambda_dantzig"].reshape(-1).astype(np.float64)
        exact = ex[f"{name}_s{k}_exact"].reshape(-1)
        scale = max(1.0, float(np.abs(ref).max()))
        r = X.natural_residual(A, b, lo, hi, fi, lam) / scale
        c = X.complementarity(A, b, lo, hi, fi, lam) / scale
        escale = max(1.0, float(np.abs(exact).max()))
        d_exact = float(np.abs(lam - exact).max()) / escale
        nb = len(invm)
        b1, b2 = rows[:, 16].astype(int), rows[:, 17].astype(int)

        def dv(x):
            f = np.zeros((nb, 6))
            np.add.at(f, b1, rows[:, 0:6] * x[:, None])
            m2 = b2 >= 0
            np.add.at(f, b2[m2], rows[m2, 6:12] * x[m2, None])
            v = np.empty_like(f)
            v[:, 0:3] = f[:, 0:3] * invm[:, None]
            v[:, 3:6] = np.einsum("bij,bj->bi", invI.reshape(-1, 3, 3), f[:, 3:6])
            return v
        dv_exact = dv(exact)
        d_dv = float(np.abs(dv(lam) - dv_exact).max()) / max(1e-12, float(np.abs(dv_exact).max()))
        report.append(f"s{k}: {len(lam)} rows, {st.iterations} sweeps (beta {st.momentum}), residual {r:.1e}, "
                      f"complementarity {c:.1e}, lambda vs exact {d_exact:.1e} (dv {d_dv:.1e})"
                      + (" [cycling order]" if cyc else ""))
        L.dJointGroupEmpty(w.group)
        w.close()
        if cyc:
            assert r <= cyc, report[-1]
            continue
        assert r <= FP64_RESID_TOL, report[-1]
        assert c <= FP64_RESID_TOL, report[-1]
        assert d_exact <= EXACT_LAMBDA_TOL, report[-1]
        assert d_dv <= EXACT_DV_TOL, report[-1]
    print(f"{name}:\n  " + "\n  ".join(report))


def test_momentum_on_batched_chains(gblib):
    """Momentum on jointed worlds: 256 capsule chains (hinge rows with limits
    and ball rows, the staged plain groups) landed on a plane, four steps to a
    residual of 1e-4 with momentum 0.8 (two worlds) and without: every step
    at the target, the FP64 residual of the last step confirms it, the two
    momentum worlds agree to the bit."""
    from ode_gb300 import scenes, sim
    L = gblib
    sc = scenes.chains(256, seed=3)
    worlds = [sim.GBWorld(sc) for _ in range(3)]
    for w in worlds:
        L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
        L.dWorldSetQuickStepW(w.w, 1.0)
    for _ in range(120):
        for w in worlds:
            w.step_fused()
    for i, w in enumerate(worlds):
        L.gbodeWorldSetSweepMomentum(w.w, 0.8 if i else 0.0)
        L.gbodeWorldSetResidualTarget(w.w, 1e-4, 5, 3000)
    sweeps = {0: [], 1: []}
    for step in range(4):
        for w in worlds:
            assert w.step_fused() == 1, L.gbodeGetLastError()
        st = [w.stats() for w in worlds]
        for s in st:
            assert s.residual <= 1e-4, (step, s.residual, s.iterations)
        assert (st[1].iterations, st[1].rows) == (st[2].iterations, st[2].rows)
        assert np.array_equal(worlds[1].state(), worlds[2].state()), step
        sweeps[0].append(st[0].iterations)
        sweeps[1].append(st[1].iterations)
    r64, _, ml = worlds[1].last_residual()
    print(f"chains: sweeps plain {np.mean(sweeps[0]):.1f}, momentum {np.mean(sweeps[1]):.1f}; "
          f"FP64 residual {r64 / max(1.0, ml):.2e}")
    assert r64 / max(1.0, ml) <= 1.5e-4
    for w in worlds:
        w.close()
