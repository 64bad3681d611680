"""The exact FP64 LCP oracle (oracle/lcp_exact.py) pinned to the reference.

* Its restatement of the reference's Dantzig treatment of friction rows
  (lcp.cpp:836-1160) reproduces the reference's dDOUBLE dWorldStep
  multipliers in the step goldens (s{k}_lambda_dantzig) within 1e-4 of
  max|lambda| (measured 2e-7 .. 8e-6) on the snapshots up to 700 rows here
  (the larger ones are checked by tests/golden/make_lcp_exact.py when the
  fixture is made).
* The committed exact solutions (tests/golden/lcp_exact.npz) solve quickstep's
  findex LCP of the same rows: natural-map residual <= 1e-8 of max|lambda|,
  complementarity likewise -- while the reference's Dantzig multipliers, whose
  friction bounds come from a first pass without friction, leave a residual
  of several per cent of max|lambda| on the piles in that LCP.
* The box-LCP solver meets the LCP conditions on random strictly monotone
  problems.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

NAMES = ("box_stack", "pile256", "capsule_pile96")


def _snapshots(golden):
    for name in NAMES:
        g = golden(f"step_{name}.npz")
        for k in range(len(g["snaps"])):
            if not g[f"s{k}_dantzig_lcp_error"][1]:
                yield name, g, k


def test_box_lcp_meets_the_conditions():
    from oracle import lcp_exact as X
    rng = np.random.default_rng(5)
    for n in (1, 7, 40, 120):
        Q = rng.normal(size=(n, n))
        A = Q @ Q.T + 1e-3 * np.eye(n)
        b = rng.normal(size=n) * 10
        lo = -rng.uniform(0, 2, n)
        hi = rng.uniform(0, 2, n)
        lo[::5] = 0.0
        hi[::7] = np.inf
        x = X.box_lcp(A, b, lo, hi)
        w = A @ x - b
        tol = 1e-8 * max(1.0, np.abs(b).max())
        assert np.all(x >= lo - 1e-12) and np.all(x <= hi + 1e-12)
        inside = (x > lo + 1e-12) & (x < hi - 1e-12)
        assert np.abs(w[inside]).max(initial=0) <= tol
        assert np.all(w[x <= lo + 1e-12] >= -tol)
        assert np.all(w[x >= hi - 1e-12] <= tol)


def test_two_phase_restatement_reproduces_reference_dantzig(port, golden):
    from make_lcp_exact import snapshot_rows
    from oracle import lcp_exact as X
    worst, n = 0.0, 0
    for name, g, k in _snapshots(golden):
        if 3 * len(g[f"s{k}_cb"]) > 700:
            continue
        rows, invm, invI = snapshot_rows(port, g, k)
        A, b, lo, hi, fi = X.dense_problem(rows, invm, invI)
        x = X.dantzig_two_phase(A, b, lo, hi, fi)
        ref = g[f"s{k}_lambda_dantzig"].reshape(-1)
        d = float(np.abs(x - ref).max()) / max(1.0, float(np.abs(ref).max()))
        worst = max(worst, d)
        n += 1
        assert d <= 1e-4, (name, k, d)
    print(f"two-phase restatement vs reference dDOUBLE dWorldStep: worst {worst:.2e} of max|lambda| over {n} snapshots")
    assert n >= 10


def test_exact_solutions_solve_quickstep_lcp(port, golden):
    from make_lcp_exact import snapshot_rows
    from oracle import lcp_exact as X
    ex = golden("lcp_exact.npz")
    for name, g, k in _snapshots(golden):
        rows, invm, invI = snapshot_rows(port, g, k)
        A, b, lo, hi, fi = X.dense_problem(rows, invm, invI)
        x = ex[f"{name}_s{k}_exact"].reshape(-1)
        ref = g[f"s{k}_lambda_dantzig"].reshape(-1).astype(np.float64)
        s = max(1.0, float(np.abs(x).max()))
        r = X.natural_residual(A, b, lo, hi, fi, x) / s
        c = X.complementarity(A, b, lo, hi, fi, x) / s
        r_ref = X.natural_residual(A, b, lo, hi, fi, ref) / max(1.0, float(np.abs(ref).max()))
        assert r <= 1e-8 and c <= 1e-8, (name, k, r, c)
        if name != "box_stack":
            # friction acts in the piles: the reference's bounds from the first pass miss
            assert r_ref >= 1e-3, (name, k, r_ref)
