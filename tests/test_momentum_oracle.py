"""Momentum between projected Gauss-Seidel sweeps (the rule of the coloured
solver's gbodeWorldSetSweepMomentum), restated here in FP64 on the dense LCP
of the step goldens' snapshots, independently of the GPU.

Each sweep relaxes the rows in the solver's manifold order (a manifold's
normal rows, then its friction pairs; quickstep.cpp:2917-3033 per row, the
friction bounds from the contact's normal multiplier, quickstep.cpp:2972-2978);
after a sweep the multipliers move on to y_k + beta (y_k - y_{k-1}).  The
first sweep and every checked sweep (one in CHECK) are plain; a check whose
residual rose halves beta, and below an eighth of the value set the sweeps go
on plain.  Checked on every snapshot of the box stack, the 256-body pile and
the capsule pile up to 400 rows, to a natural-map residual of 1e-5 of
max|lambda| (FP64):
* both the plain and the momentum sweeps reach it, and their multipliers are
  as close to the exact FP64 solution of quickstep's LCP
  (tests/golden/lcp_exact.npz) as each other (within 5e-3 of max|lambda|;
  the stack's redundant coplanar contacts leave individual multipliers a few
  per cent from it at this residual either way);
* summed over the snapshots, momentum needs fewer sweeps (measured: 21,370
  against 30,240).
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

BETA = 0.8
CHECK = 10
TARGET = 1e-5
MAX_SWEEPS = 20000


def manifold_order(rows):
    """Rows in contact order, three a contact; consecutive contacts on the same
    body pair form a manifold: its normal rows first, then its friction pairs."""
    nc = len(rows) // 3
    b1, b2 = rows[0::3, 16].astype(int), rows[0::3, 17].astype(int)
    order, c = [], 0
    while c < nc:
        e = c + 1
        while e < nc and b1[e] == b1[c] and b2[e] == b2[c]:
            e += 1
        order += [3 * i for i in range(c, e)]
        for i in range(c, e):
            order += [3 * i + 1, 3 * i + 2]
        c = e
    return order


def _sweep(A, b, lo, hi, findex, x, order, D):
    for i in order:
        if findex[i] >= 0:
            h = abs(hi[i] * x[findex[i]])
            lo_i, hi_i = -h, h
        else:
            lo_i, hi_i = lo[i], hi[i]
        x[i] = min(max(x[i] + (b[i] - A[i] @ x) / D[i], lo_i), hi_i)


def solve(A, b, lo, hi, findex, order, beta):
    from oracle import lcp_exact as X
    D = np.diag(A)
    x = np.zeros(len(b))
    prev = x.copy()
    mom, r_prev = beta, None
    for k in range(1, MAX_SWEEPS + 1):
        _sweep(A, b, lo, hi, findex, x, order, D)
        out = x.copy()
        if k % CHECK == 0:
            r = X.natural_residual(A, b, lo, hi, findex, x) / max(1.0, float(np.abs(x).max()))
            if r <= TARGET:
                return x, k
            if r_prev is not None and r > r_prev and mom > 0:
                mom = 0.0 if 0.5 * mom < beta / 8 else 0.5 * mom
            r_prev = r
        elif k > 1 and mom > 0:
            x = out + mom * (out - prev)
        prev = out
    raise AssertionError(f"no convergence in {MAX_SWEEPS} sweeps (beta {beta})")


def test_momentum_reaches_the_same_solution_in_fewer_sweeps(port, golden):
    from make_lcp_exact import snapshot_rows
    from oracle import lcp_exact as X
    ex = golden("lcp_exact.npz")
    totals = {"plain": 0, "momentum": 0}
    report = []
    for name in ("box_stack", "pile256", "capsule_pile96"):
        g = golden(f"step_{name}.npz")
        for k in range(len(g["snaps"])):
            if g[f"s{k}_dantzig_lcp_error"][1] or 3 * len(g[f"s{k}_cb"]) > 400:
                continue
            rows, invm, invI = snapshot_rows(port, g, k)
            A, b, lo, hi, fi = X.dense_problem(rows, invm, invI)
            order = manifold_order(rows)
            exact = ex[f"{name}_s{k}_exact"].reshape(-1)
            scale = max(1.0, float(np.abs(exact).max()))
            got = {}
            for label, beta in (("plain", 0.0), ("momentum", BETA)):
                x, n = solve(A, b, lo, hi, fi, order, beta)
                got[label] = (n, float(np.abs(x - exact).max()) / scale)
                totals[label] += n
            assert got["momentum"][1] <= got["plain"][1] + 5e-3, (name, k, got)
            report.append(f"{name} s{k}: {len(b)} rows, sweeps plain {got['plain'][0]}, momentum "
                          f"{got['momentum'][0]}; lambda vs exact {got['plain'][1]:.3f} / {got['momentum'][1]:.3f}")
    print("\n".join(report))
    print(f"total sweeps: plain {totals['plain']}, momentum {totals['momentum']}")
    assert len(report) >= 6 and totals["momentum"] < totals["plain"]
