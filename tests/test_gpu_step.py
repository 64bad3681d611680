"""GPU dWorldQuickStep against the reference's golden snapshots and the
oracle, through the C ABI.

Tolerances (FP32 solver):
* reference-order solver, one step from a recorded state with the recorded
  contact joints: lambda within 1e-3 relative to max(1, max|lambda|) of the
  reference with row reordering disabled; body positions within 1e-4 m.
* coloured solver: the FP64 LCP residual (natural map, relative to
  max(1, max|lambda|)) of the returned lambda at or below the requested
  target, checked by the oracle's independent FP64 evaluator too.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAMBDA_RTOL = 1e-3
POS_ATOL = 1e-4


def snapshot_scene(g, pre, name):
    from ode_gb300 import scenes
    bodies = g["bodies0"].copy()
    bodies[:, 0:3], bodies[:, 3:7] = pre[:, 0:3], pre[:, 3:7]
    bodies[:, 7:10], bodies[:, 10:13] = pre[:, 19:22], pre[:, 22:25]
    p = g["params"]
    iters, maxc, mode, _ = [int(x) for x in g["ints"]]
    return scenes.Scene(name, bodies, g["geom_cls"], g["geom_body"], g["geom_pos"], g["geom_R"], g["geom_dims"],
                        dt=float(p[0]), gravity=tuple(float(x) for x in p[1:4]), erp=float(p[4]), cfm=float(p[5]),
                        w=float(p[6]), iterations=iters, max_vel=float(p[7]), min_depth=float(p[8]),
                        surface_mode=mode, maxc=maxc)


def contact_lambdas(rows, nc):
    """rows are assembled in contact order, 3 rows per contact (mu > 0)."""
    return rows[:, 19].reshape(nc, 3)


@pytest.mark.parametrize("name", ["box_stack", "pile256", "capsule_pile96"])
def test_reference_order_lambda_parity(gblib, golden, name):
    from ode_gb300 import ode, sim
    g = golden(f"step_{name}.npz")
    mode = int(g["ints"][2])
    for k in range(len(g["snaps"])):
        pre, cb, cs = g[f"s{k}_pre"], g[f"s{k}_cb"], g[f"s{k}_cs"]
        w = sim.GBWorld(snapshot_scene(g, pre, name), solver=ode.GBODE_SOLVER_REFERENCE_ORDER)
        assert sim.step_contacts(w, cb, cs, mode) == 1
        w.sync()
        rows = w.last_rows()
        lam = contact_lambdas(rows, len(cb))
        ref = g[f"s{k}_lambda"]
        scale = max(1.0, float(np.abs(ref).max()))
        assert np.abs(lam - ref).max() / scale <= LAMBDA_RTOL, (k, np.abs(lam - ref).max() / scale)
        post = w.state()
        assert np.abs(post[:, 0:3] - g[f"s{k}_post"][:, 0:3]).max() <= POS_ATOL
        w.L.dJointGroupEmpty(w.group)
        w.close()


@pytest.mark.parametrize("name", ["box_stack", "pile256", "capsule_pile96"])
def test_reference_order_dynamic_iterations(gblib, golden, name):
    """The reference's dynamic iteration rule (quickstep.cpp:1823-1856,
    :3253-3285) in the reference-order solver (k_islands), rows not
    reordered, on every step snapshot under three parameter sets: the
    defaults (every solve runs its extra sweeps), and two under which solves
    exit early (the box stack after 4-14 of 20 sweeps) or stop between the
    regular and the doubled count (the 256-body pile after 47 of 30 + 30).
    lambda within 1e-3 of max(1, max|lambda|) of the reference, positions
    within 1e-4 m, and the sweeps performed (the largest island's) equal to the
    reference's (tests/golden/make_golden.py gen_steps_dyn: the fixed sweep
    count whose multipliers equal the dynamic solve's to the bit)."""
    import ctypes
    from ode_gb300 import ode, sim
    g = golden(f"step_{name}.npz")
    mode = int(g["ints"][2])
    report = []
    for tag in ("dyn", "dyn2", "dyn3"):
        worst, sweeps = 0.0, []
        for k in range(len(g["snaps"])):
            pre, cb, cs = g[f"s{k}_pre"], g[f"s{k}_cb"], g[f"s{k}_cs"]
            w = sim.GBWorld(snapshot_scene(g, pre, name), solver=ode.GBODE_SOLVER_REFERENCE_ORDER, dyn=True)
            if tag != "dyn":
                pe, mf, ed = (ctypes.c_float(float(x)) for x in g[f"{tag}_params"])
                w.L.dWorldSetQuickStepDynamicIterationParameters(w.w, ctypes.byref(pe), ctypes.byref(mf),
                                                                 ctypes.byref(ed))
            assert sim.step_contacts(w, cb, cs, mode) == 1
            w.sync()
            lam = contact_lambdas(w.last_rows(), len(cb))
            ref = g[f"s{k}_lambda_{tag}"]
            d = float(np.abs(lam - ref).max()) / max(1.0, float(np.abs(ref).max()))
            worst = max(worst, d)
            assert d <= LAMBDA_RTOL, (tag, k, d)
            assert np.abs(w.state()[:, 0:3] - g[f"s{k}_post_{tag}"][:, 0:3]).max() <= POS_ATOL
            ref_sweeps = int(g[f"s{k}_sweeps_{tag}"].max())
            sweeps.append((w.stats().iterations, ref_sweeps))
            assert w.stats().iterations == ref_sweeps, (tag, k, w.stats().iterations, ref_sweeps)
            w.L.dJointGroupEmpty(w.group)
            w.close()
        report.append(f"{tag}: sweeps (device, reference) {sweeps}, lambda within {worst:.1e}")
    print(f"{name}: " + "; ".join(report))


@pytest.mark.parametrize("name", ["box_stack", "pile256"])
def test_reference_order_matches_oracle_bitwise(gblib, port, golden, name):
    """The device relaxes rows in the reference's order with the reference's
    float operation order: its lambda equals the oracle's to the bit."""
    from ode_gb300 import ode, sim
    g = golden(f"step_{name}.npz")
    iters, maxc, mode, _ = [int(x) for x in g["ints"]]
    k = len(g["snaps"]) - 1
    pre, cb, cs = g[f"s{k}_pre"], g[f"s{k}_cb"], g[f"s{k}_cs"]
    sc = snapshot_scene(g, pre, name)
    w = sim.GBWorld(sc, solver=ode.GBODE_SOLVER_REFERENCE_ORDER)
    sim.step_contacts(w, cb, cs, mode)
    w.sync()
    lam = contact_lambdas(w.last_rows(), len(cb))
    pw = port.world(sc.bodies, g["params"], iters, dyn=0, reorder=0)
    plam = pw.quickstep(cb, np.full(len(cb), mode, np.int32), cs)
    diff = np.abs(lam - plam).max() / max(1.0, float(np.abs(plam).max()))
    print(f"{name}: max relative lambda difference GPU vs oracle {diff:.3g}")
    assert diff <= 1e-5
    np.testing.assert_allclose(w.state()[:, 0:3], pw.state()[:, 0:3], atol=1e-6)
    w.L.dJointGroupEmpty(w.group)
    w.close()


def test_compat_loop_box_stack(gblib, golden):
    """The reference's user loop through the C ABI (dSpaceCollide with a near
    callback -> dCollide -> dJointCreateContact -> dWorldQuickStep) for 300
    steps of the 10-box stack: the stack stands and tracks the reference."""
    from ode_gb300 import ode, scenes, sim
    g = golden("step_box_stack.npz")
    w = sim.GBWorld(scenes.box_stack(seed=0), solver=ode.GBODE_SOLVER_REFERENCE_ORDER)
    traj, traj_stock = g["traj"], g["traj_stock"]
    for s in range(300):
        assert w.step_compat() == 1
    st = w.state()
    err = np.abs(st[:, 0:3] - traj[299, :, 0:3]).max()
    # contacts arrive in another pair order than the reference's hash table, so
    # rows relax in another order; the reference's own two row orders (no
    # reordering vs. random reordering) already differ this much at step 299
    spread = np.abs(traj[299, :, 0:3] - traj_stock[299, :, 0:3]).max()
    print(f"box stack after 300 steps: max position difference {err:.3g} m (reference order spread {spread:.3g} m)")
    assert err <= 2 * spread
    assert np.abs(st[:, 2] - traj[299, :, 2]).max() < 0.01
    assert np.all(st[:, 2] > np.arange(10) + 0.45)
    w.close()


@pytest.mark.parametrize("target", [1e-4])
def test_coloured_solver_reaches_residual(gblib, port, golden, target):
    from oracle.port.port import world_inv_inertia
    from ode_gb300 import sim
    g = golden("step_pile256.npz")
    mode = int(g["ints"][2])
    k = len(g["snaps"]) - 1
    pre, cb, cs = g[f"s{k}_pre"], g[f"s{k}_cb"], g[f"s{k}_cs"]
    sc = snapshot_scene(g, pre, "pile256")
    w = sim.GBWorld(sc)
    w.L.gbodeWorldSetResidualTarget(w.w, target, 10, 5000)
    sim.step_contacts(w, cb, cs, mode)
    w.sync()
    st = w.stats()
    r64, ce, ml = w.last_residual()
    rel = r64 / max(1.0, ml)
    rows = w.last_rows()
    invI, invm = world_inv_inertia(pre, sc.bodies)
    r_oracle, _ = port.lcp_residual(rows, invm, invI, rows[:, 19])
    rel_oracle = r_oracle / max(1.0, float(np.abs(rows[:, 19]).max()))
    print(f"coloured: {st.iterations} sweeps, {st.colours} colours, FP32 residual {st.residual:.3g}, "
          f"FP64 device {rel:.3g}, FP64 oracle {rel_oracle:.3g}")
    assert st.colours > 0 and st.iterations > 0
    assert rel <= 1.5 * target
    assert abs(rel - rel_oracle) <= 1e-5 + 1e-2 * rel_oracle
    w.L.dJointGroupEmpty(w.group)
    w.close()


# coloured solver against the FP64 oracle (see the test's docstring)
FP64_TARGET = 1e-6          # FP32 in-kernel residual target of the solve
FP64_RESID_TOL = 1e-5       # section 8(d) residual of the result, relative to max|lambda_dantzig|
EXACT_LAMBDA_TOL = 2e-2     # |lambda - lambda_exact| / max|lambda_exact| (redundant contacts)
EXACT_DV_TOL = 2e-3         # |M^-1 J^T (lambda - lambda_exact)| / max|M^-1 J^T lambda_exact|
# Snapshots where projected Gauss-Seidel in the solver's row order (a
# manifold's normal rows, then its friction rows) does not converge but
# cycles: the same iteration on the oracle's rows on the CPU cycles there in
# FP64 too (residual 6e-4 after 1,000 sweeps, 1.2e-3 after 2,000), while
# contact-by-contact order converges.  Only the residual's bound is checked.
CYCLING = {("capsule_pile96", 2): 3e-3}


@pytest.mark.parametrize("two_level", [0, 1])
@pytest.mark.parametrize("name", ["box_stack", "pile256", "capsule_pile96"])
def test_coloured_solver_against_fp64_dantzig(gblib, golden, name, two_level):
    """The throughput solver (coloured PGS, k_pgs) against the FP64 oracle on
    every snapshot of the step goldens (except the one where the reference's
    Dantzig solver itself gave up).

    The oracle is the reference's dDOUBLE dWorldStep (Dantzig,
    lcp.cpp:836-1160) on the same contacts (`s{k}_lambda_dantzig`).  Dantzig
    sets the friction rows' bounds once, from the normal multipliers of a
    first pass with friction held at zero, while quickstep's LCP -- the one
    PGS solves -- bounds friction by the final normals
    (quickstep.cpp:2972-2978).  The two solutions therefore differ wherever
    friction acts; tests/golden/lcp_exact.npz holds, per snapshot, the
    reference's two-phase solution restated in FP64 (oracle/lcp_exact.py,
    within 8e-6 of the reference's own multipliers) and that solution
    continued to an exact solution of quickstep's LCP (natural-map residual
    <= 1e-9).  Checked here, with lambda_oracle = the reference's Dantzig
    multipliers as the section 8(d) normalisation:
    * residual r(lambda) / max(1, max|lambda_oracle|) <= 1e-5 after a solve
      to an FP32 residual of 1e-6, and the complementarity error (in the
      units of lambda) likewise;
    * lambda within 2e-2 of max|lambda_exact| of the exact solution, and the
      velocity change M^-1 J^T lambda within 2e-3 of its largest entry (the
      piles and the stack have four coplanar contacts per face, redundant
      rows whose split PGS converges slowly, while the net force on each
      body converges fast);
    * against the reference's Dantzig multipliers lambda differs by no more
      than the exact solution does (the friction-bound model) plus that
      solver tolerance.
    Run with the one-level sweep and with the two-level sweep
    (gbodeWorldSetTwoLevelSweep), which solves the same LCP in another order."""
    from oracle import lcp_exact as X
    from oracle.port.port import world_inv_inertia
    from ode_gb300 import sim
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
        # velocity change per body: M^-1 J^T lambda, from A's off-diagonal-free pieces
        J = np.zeros((len(lam), 6 * len(invm)))
        b1, b2 = rows[:, 16].astype(int), rows[:, 17].astype(int)
        for i in range(len(lam)):
            J[i, 6 * b1[i]:6 * b1[i] + 6] = rows[i, 0:6]
            if b2[i] >= 0:
                J[i, 6 * b2[i]:6 * b2[i] + 6] = rows[i, 6:12]

        def dv(x):
            f = (J.T @ x).reshape(-1, 6)
            v = np.empty_like(f)
            v[:, 0:3] = f[:, 0:3] * invm[:, None]
            v[:, 3:6] = np.einsum("bij,bj->bi", invI.reshape(-1, 3, 3), f[:, 3:6])
            return v
        dv_exact = dv(exact)
        d_dv = float(np.abs(dv(lam) - dv_exact).max()) / max(1e-12, float(np.abs(dv_exact).max()))
        d_ref = float(np.abs(lam - ref).max()) / scale
        d_model = float(np.abs(exact - ref).max()) / scale
        dp = float(np.abs(w.state()[:, 0:3] - g[f"s{k}_post_dantzig"][:, 0:3]).max())
        report.append(f"s{k}: {len(lam)} rows, {st.iterations} sweeps, residual {r:.1e}, complementarity {c:.1e}, "
                      f"lambda vs exact {d_exact:.1e} (dv {d_dv:.1e}), vs reference Dantzig {d_ref:.2e} "
                      f"(exact vs reference {d_model:.2e}), positions vs reference Dantzig {dp:.1e} m, "
                      f"interior rows {st.interior_rows}" + (" [cycling order]" if cyc else ""))
        if cyc:
            assert r <= cyc, report[-1]
            L.dJointGroupEmpty(w.group)
            w.close()
            continue
        assert r <= FP64_RESID_TOL, report[-1]
        assert c <= FP64_RESID_TOL, report[-1]
        assert d_exact <= EXACT_LAMBDA_TOL, report[-1]
        assert d_dv <= EXACT_DV_TOL, report[-1]
        assert d_ref <= d_model + EXACT_LAMBDA_TOL * escale / scale, report[-1]
        L.dJointGroupEmpty(w.group)
        w.close()
    print(f"{name}:\n  " + "\n  ".join(report))


def test_fused_pile_steps_are_sane(gblib):
    """Full-size pile, fused path: finite state, bodies stay in the container,
    contact and row counts in the expected range, colours valid."""
    from ode_gb300 import scenes, sim
    sc = scenes.pile(32768, seed=1)
    w = sim.GBWorld(sc)
    for _ in range(200):
        w.step_fused()
    w.sync()
    st = w.state()
    s = w.stats()
    assert np.isfinite(st).all()
    L = -float(sc.geom_dims[-3, 3])  # far wall x = L (plane -x = -L)
    assert st[:, 2].min() > -0.3 and st[:, 0].min() > -0.3 and st[:, 0].max() < L + 0.3
    assert s.rows == 3 * s.contacts and s.contacts > 20000
    assert 2 <= s.colours <= 128
    w.close()


def test_staging_waves_give_the_same_solution(gblib):
    """The coloured solver on one thread block instead of one per SM: every
    colour of a 2,048-body pile is then cut into many waves of at most 256
    slots and 800 staged rows (block barriers between them) instead of one
    wave per block.  A colour's manifolds share no body, so the order within a
    colour cannot change the result: the states after 250 steps (the pile
    landed, ~15k rows) are equal to the bit."""
    from ode_gb300 import scenes, sim
    L = gblib
    sc = scenes.pile(2048, seed=7)
    worlds = [sim.GBWorld(sc), sim.GBWorld(sc)]
    L.gbodeWorldSetSolverBlocks(worlds[1].w, 1)
    assert L.gbodeWorldGetSolverBlocks(worlds[1].w) == 1
    for w in worlds:
        L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
        L.dWorldSetQuickStepW(w.w, 1.0)
        L.dWorldSetQuickStepNumIterations(w.w, 30)
    for _ in range(250):
        for w in worlds:
            w.step_fused()
    a, b = worlds[0].state(), worlds[1].state()
    s0, s1 = worlds[0].stats(), worlds[1].stats()
    print(f"one block vs {L.gbodeWorldGetSolverBlocks(worlds[0].w)}: {s1.iterations} vs {s0.iterations} sweeps, "
          f"{s0.rows} rows, {s0.colours} colours")
    assert np.isfinite(a).all() and s0.rows > 10000
    assert np.array_equal(a, b), float(np.abs(a - b).max())
    for w in worlds:
        w.close()


@pytest.mark.parametrize("two_level", [0, 2])
def test_solver_tiles_give_the_same_solution(gblib, two_level):
    """gbodeWorldSetSolverTiles: 128 threads a block and 400 staged rows a
    buffer instead of 256 and 800 cut every colour into other waves (more of
    them, relaxed by other threads); a colour's manifolds share no body, so
    the states after 150 steps of a 2,048-body pile are equal to the bit, with
    the one-level and with the two-level sweep."""
    from ode_gb300 import scenes, sim
    import ctypes
    L = gblib
    sc = scenes.pile(2048, seed=7)
    worlds = [sim.GBWorld(sc), sim.GBWorld(sc)]
    L.gbodeWorldSetSolverTiles(worlds[1].w, 128, 400)
    t, c = ctypes.c_int(0), ctypes.c_int(0)
    L.gbodeWorldGetSolverTiles(worlds[1].w, ctypes.byref(t), ctypes.byref(c))
    assert (t.value, c.value) == (128, 400)
    for w in worlds:
        L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
        L.dWorldSetQuickStepW(w.w, 1.0)
        L.dWorldSetQuickStepNumIterations(w.w, 30)
        L.gbodeWorldSetTwoLevelSweep(w.w, two_level)
    for _ in range(150):
        for w in worlds:
            w.step_fused()
    a, b = worlds[0].state(), worlds[1].state()
    s0 = worlds[0].stats()
    assert np.isfinite(a).all() and s0.rows > 10000
    assert np.array_equal(a, b), float(np.abs(a - b).max())
    for w in worlds:
        w.close()


def test_snapshot_reruns_the_same_steps(gblib):
    """gbodeWorldSaveSnapshot / gbodeWorldRestoreSnapshot: a 2,048-body pile
    with the warm-start cache on, 60 fused steps, a snapshot, 10 steps; the
    restore and the same 10 steps again give the same state to the bit (the
    fused step is deterministic and the snapshot holds the bodies and the
    warm-start cache).  A restore after a body was added fails with a message
    and changes nothing."""
    from ode_gb300 import scenes, sim
    L = gblib
    sc = scenes.pile(2048, seed=7)
    w = sim.GBWorld(sc)
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    for _ in range(60):
        w.step_fused()
    assert L.gbodeWorldSaveSnapshot(w.w) == 1, L.gbodeGetLastError()
    start = w.state()
    for _ in range(10):
        w.step_fused()
    a = w.state()
    assert L.gbodeWorldRestoreSnapshot(w.w) == 1, L.gbodeGetLastError()
    np.testing.assert_array_equal(w.state(), start)
    for _ in range(10):
        w.step_fused()
    b = w.state()
    assert np.abs(a - start).max() > 1e-4  # the pile moved
    np.testing.assert_array_equal(a, b)
    L.dBodyCreate(w.w)
    assert L.gbodeWorldRestoreSnapshot(w.w) == 0
    assert b"changed" in L.gbodeGetLastError()
    L.gbodeWorldDropSnapshot(w.w)
    w.close()


@pytest.mark.parametrize("target", [1e-4, 0.0])
def test_neighbour_waits_match_grid_barriers(gblib, target):
    """The two-level sweep with neighbour waits (GBODE_SYNC_NEIGHBOURS: a
    block waits only for the blocks that touch the same bodies, and not at
    all in a colour where it has no manifold) against a grid barrier after
    every step (GBODE_SYNC_GRID), on an 8,192-body pile that has landed: the
    same sweeps, multipliers and bodies to the bit, step after step -- with a
    residual target (checks every 5 sweeps under grid barriers) and with a
    fixed 30 sweeps (no grid barrier at all in the neighbour mode)."""
    from ode_gb300 import ode, scenes, sim
    L = gblib
    sc = scenes.pile(8192, seed=7)
    worlds = [sim.GBWorld(sc) for _ in range(2)]
    for w in worlds:
        L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
        L.dWorldSetQuickStepW(w.w, 1.0)
        L.dWorldSetQuickStepNumIterations(w.w, 30)
    for _ in range(300):
        for w in worlds:
            w.step_fused()
    for w, mode in zip(worlds, (ode.GBODE_SYNC_GRID, ode.GBODE_SYNC_NEIGHBOURS)):
        L.gbodeWorldSetTwoLevelSweep(w.w, 2)
        L.gbodeWorldSetSweepSync(w.w, mode)
        assert L.gbodeWorldGetSweepSync(w.w) == mode
        if target > 0:
            L.gbodeWorldSetResidualTarget(w.w, target, 5, 3000)
    for step in range(4):
        for w in worlds:
            assert w.step_fused() == 1, L.gbodeGetLastError()
        g, n = (w.stats() for w in worlds)
        assert g.neighbour_waits == 0 and n.neighbour_waits == 1
        assert g.interior_rows > g.rows // 2 and g.colours >= 4
        assert (g.iterations, g.rows, g.contacts) == (n.iterations, n.rows, n.contacts), step
        a, b = (w.state() for w in worlds)
        assert np.array_equal(a, b), f"step {step}: bodies differ by {np.abs(a - b).max():.3e}"
    print(f"{'residual target' if target else '30 sweeps'}: {n.iterations} sweeps, {n.colours} cross colours, "
          f"{n.interior_rows} of {n.rows} rows interior; the two modes agree to the bit")
    for w in worlds:
        w.close()


def test_split_classes_on_a_pile(gblib):
    """Split classes (gbodeWorldSetCrossClasses): the two-level sweep's
    crossing colours merged into 5 classes, each relaxed at once with mass
    splitting, on an 8,192-body pile that has landed.  Every step reaches the
    residual target, and its FP64 residual evaluated on the device confirms
    the last one (1.5e-4: an FP32 solution at 1e-4); the class sums are integers, so two
    worlds agree to the bit, and neighbour waits agree with grid barriers to
    the bit; positions agree with the exact colours' solution of the same
    steps within 1e-3 m (both are solutions to a residual of 1e-4)."""
    from ode_gb300 import ode, scenes, sim
    L = gblib
    sc = scenes.pile(8192, seed=7)
    worlds = [sim.GBWorld(sc) for _ in range(4)]
    for w in worlds:
        L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
        L.dWorldSetQuickStepW(w.w, 1.0)
        L.dWorldSetQuickStepNumIterations(w.w, 30)
    for _ in range(300):
        for w in worlds:
            w.step_fused()
    for w, k, mode in zip(worlds, (0, 5, 5, 5), (0, 0, 0, ode.GBODE_SYNC_GRID)):
        L.gbodeWorldSetTwoLevelSweep(w.w, 2)
        L.gbodeWorldSetCrossClasses(w.w, k)
        assert L.gbodeWorldGetCrossClasses(w.w) == k
        L.gbodeWorldSetSweepSync(w.w, mode)
        L.gbodeWorldSetResidualTarget(w.w, 1e-4, 5, 3000)
    for step in range(3):
        for w in worlds:
            assert w.step_fused() == 1, L.gbodeGetLastError()
        ex, a, b, c = (w.stats() for w in worlds)
        assert ex.cross_classes == 0 and a.cross_classes == 5 and c.cross_classes == 5
        assert a.residual <= 1e-4 and (a.iterations, a.rows) == (b.iterations, b.rows) == (c.iterations, c.rows)
        sa, sb, scc = worlds[1].state(), worlds[2].state(), worlds[3].state()
        assert np.array_equal(sa, sb) and np.array_equal(sa, scc), step
    r64, _, ml = worlds[1].last_residual()
    print(f"split classes: {a.iterations} sweeps ({ex.iterations} with exact colours, {ex.colours} colours), "
          f"{a.colours} classes; FP64 residual {r64 / max(1.0, ml):.2e}; positions differ from the exact colours' "
          f"by {np.abs(worlds[0].state()[:, 0:3] - sa[:, 0:3]).max():.2e} m")
    assert r64 / max(1.0, ml) <= 1.5e-4
    assert np.abs(worlds[0].state()[:, 0:3] - sa[:, 0:3]).max() <= 1e-3
    for w in worlds:
        w.close()


def test_two_level_sweep_on_a_pile(gblib):
    """The two-level sweep (gbodeWorldSetTwoLevelSweep) on an 8,192-body
    pile that has landed: most rows are interior to a column and relaxed from
    shared memory; the step reaches the residual target (FP64 residual checked
    on the device), its positions agree with the one-level sweep's solution of
    the same step within 1e-3 m (both are solutions to a residual of 1e-4),
    and two worlds stepped the same way agree to the bit (the sweep order is
    fixed)."""
    from ode_gb300 import scenes, sim
    L = gblib
    sc = scenes.pile(8192, seed=7)
    worlds = [sim.GBWorld(sc) for _ in range(3)]
    for w in worlds:
        L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
        L.dWorldSetQuickStepW(w.w, 1.0)
        L.dWorldSetQuickStepNumIterations(w.w, 30)
    for _ in range(300):
        for w in worlds:
            w.step_fused()
    for w, two in zip(worlds, (0, 1, 1)):
        L.gbodeWorldSetTwoLevelSweep(w.w, two)
        L.gbodeWorldSetResidualTarget(w.w, 1e-4, 5, 3000)
    for w in worlds:
        assert w.step_fused() == 1, L.gbodeGetLastError()
    for w in worlds:
        w.sync()
    s0, s1 = worlds[0].stats(), worlds[1].stats()
    r64, _, ml = worlds[1].last_residual()
    a, b, c = (w.state() for w in worlds)
    print(f"one level: {s0.iterations} sweeps, {s0.colours} colours; two level: {s1.iterations} sweeps, "
          f"{s1.colours} cross colours, {s1.interior_colours} interior colours, "
          f"{s1.interior_rows} of {s1.rows} rows interior; FP64 residual {r64 / max(1.0, ml):.2e}; "
          f"positions differ by {np.abs(a[:, 0:3] - b[:, 0:3]).max():.2e} m")
    assert s1.rows > 20000 and s1.interior_rows > s1.rows // 2
    assert s1.residual <= 1e-4 and r64 / max(1.0, ml) <= 1.5e-4
    assert np.abs(a[:, 0:3] - b[:, 0:3]).max() <= 1e-3
    assert np.array_equal(b, c)
    for w in worlds:
        w.close()
