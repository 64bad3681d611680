"""Exact FP64 solutions of the step's LCP, for the checks of the iterative
solvers.  Test infrastructure only (imported by tests/, never by the product).

The rows are those quickstep forms (quickstep.cpp:1486-1747, before the Ad
scaling of :2251-2316): row i couples bodies b1, b2 through J_i, with
right-hand side rhs_i, constraint force mixing cfm_i, bounds lo_i / hi_i and
findex_i.  The LCP is A x = b + w with A = J M^-1 J^T + diag(cfm) and
b = rhs, and per row

    x_i = lo_i and w_i >= 0,  or  x_i = hi_i and w_i <= 0,  or  lo_i < x_i < hi_i and w_i = 0,

where a row with findex_i = f >= 0 (a friction row) has the bounds
hi_i = |hi_i * x_f|, lo_i = -hi_i (quickstep.cpp:2972-2978).  A is symmetric
positive definite (cfm > 0), so with the bounds fixed the problem is a
box-constrained convex QP with exactly one solution (`box_lcp`).

Two solutions of the same rows are given here:

* `dantzig_two_phase` restates what the reference's Dantzig solver does with
  friction rows (lcp.cpp:836-1160): findex rows are moved to the end and held
  at zero while the other rows are solved; when the first friction row is
  reached, every friction row's bounds are set once from the normal
  multipliers found so far (lcp.cpp:927-950), and the solve continues with
  those bounds fixed.  The result is the exact solution of phase 2, whose
  friction bounds come from phase 1's normals -- so it is generally NOT a
  solution of the LCP above, whose bounds follow the final normals.
* `findex_fixed_point` continues from there: the friction bounds are set from
  the current normals (damped), the box LCP is solved again, until the
  bounds agree with the solution.  Its limit is an exact solution of the
  findex LCP, the problem projected Gauss-Seidel (quickstep's SOR_LCP)
  converges to.

The box LCPs are solved by block principal pivoting (Judice and Pires,
"A block principal pivoting algorithm for large-scale strictly monotone
linear complementarity problems", Computers & OR 21, 1994) with Murty's
single-index rule once the count of infeasible indices stops falling, which
guarantees termination for a P-matrix.
"""
from __future__ import annotations

import numpy as np


def dense_problem(rows: np.ndarray, invm: np.ndarray, invI: np.ndarray):
    """A (FP64), b, lo, hi, findex from rows in the 20-column layout
    (J1 0-5, J2 6-11, rhs 12, cfm 13, lo 14, hi 15, body1 16, body2 17,
    findex 18, lambda 19), body inverse masses invm [nb] and world-frame
    inverse inertias invI [nb][9]."""
    m = rows.shape[0]
    nb = invm.shape[0]
    b1 = rows[:, 16].astype(np.int64)
    b2 = rows[:, 17].astype(np.int64)
    J1 = rows[:, 0:6].astype(np.float64)
    J2 = rows[:, 6:12].astype(np.float64)
    Iw = invI.reshape(nb, 3, 3).astype(np.float64)

    def minv(J, b):  # M^-1 J^T per row
        out = np.empty_like(J)
        out[:, 0:3] = J[:, 0:3] * invm[b][:, None]
        out[:, 3:6] = np.einsum("rij,rj->ri", Iw[b], J[:, 3:6])
        return out

    has2 = b2 >= 0
    M1 = minv(J1, b1)
    M2 = np.zeros_like(J2)
    M2[has2] = minv(J2[has2], b2[has2])
    A = np.zeros((m, m))
    # rows sharing a body couple through that body's block
    for side_i, (Ji, bi) in enumerate(((J1, b1), (J2, b2))):
        for side_j, (Mj, bj) in enumerate(((M1, b1), (M2, b2))):
            vi = bi >= 0
            vj = bj >= 0
            same = (bi[:, None] == bj[None, :]) & vi[:, None] & vj[None, :]
            if same.any():
                A += np.where(same, Ji @ Mj.T, 0.0)
    A[np.diag_indices(m)] += rows[:, 13].astype(np.float64)
    b = rows[:, 12].astype(np.float64)
    lo = rows[:, 14].astype(np.float64)
    hi = rows[:, 15].astype(np.float64)
    findex = rows[:, 18].astype(np.int64)
    return A, b, lo, hi, findex


def box_lcp(A, b, lo, hi, max_pivots: int = 20000):
    """The box-constrained LCP with fixed bounds, exactly (FP64).  Rows with
    lo = hi are held there.  Returns x; raises if pivoting does not finish."""
    n = b.shape[0]
    fixed = lo == hi
    state = np.zeros(n, np.int8)  # 0 free, -1 at lo, +1 at hi
    state[fixed] = -1
    best, stalls, murty = n + 1, 0, False
    scale_b = np.maximum(1.0, np.abs(b).max() if n else 1.0)
    for _ in range(max_pivots):
        x = np.where(state < 0, lo, np.where(state > 0, hi, 0.0))
        F = state == 0
        if F.any():
            rhs = b[F] - A[np.ix_(F, ~F)] @ x[~F]
            x[F] = np.linalg.solve(A[np.ix_(F, F)], rhs)
        w = A @ x - b
        tol_x = 1e-13 * np.maximum(1.0, np.abs(x))
        tol_w = 1e-12 * scale_b
        below = F & (x < lo - tol_x)
        above = F & (x > hi + tol_x)
        bad_lo = (state < 0) & ~fixed & (w < -tol_w)
        bad_hi = (state > 0) & ~fixed & (w > tol_w)
        bad = below | above | bad_lo | bad_hi
        nbad = int(bad.sum())
        if nbad == 0:
            return np.clip(x, lo, hi)
        if nbad < best:
            best, stalls = nbad, 0
        else:
            stalls += 1
            if stalls > 3:
                murty = True
        idx = np.nonzero(bad)[0]
        if murty:
            idx = idx[-1:]
        for i in idx:
            if below[i]:
                state[i] = -1
            elif above[i]:
                state[i] = 1
            else:
                state[i] = 0
    raise RuntimeError("box_lcp: pivoting did not finish")


def friction_bounds(lo, hi, findex, x):
    """Bounds of every row with the friction rows' set from x (the
    quickstep.cpp:2972-2978 rule; a zero normal gives lo = hi = 0, as
    lcp.cpp:940-943)."""
    lo2, hi2 = lo.copy(), hi.copy()
    f = findex >= 0
    h = np.abs(hi[f] * x[findex[f]])
    hi2[f], lo2[f] = h, -h
    return lo2, hi2


def dantzig_two_phase(A, b, lo, hi, findex):
    """The reference's dWorldStep multipliers (lcp.cpp:836-1160 with
    findex): friction rows held at zero, then their bounds fixed from those
    normals for the full solve."""
    f = findex >= 0
    lo1, hi1 = lo.copy(), hi.copy()
    lo1[f] = 0.0
    hi1[f] = 0.0
    x1 = box_lcp(A, b, lo1, hi1)
    lo2, hi2 = friction_bounds(lo, hi, findex, x1)
    return box_lcp(A, b, lo2, hi2)


def findex_fixed_point(A, b, lo, hi, findex, x0=None, damping: float = 0.5, max_outer: int = 2000,
                       tol: float = 1e-10):
    """An exact solution of the findex LCP: friction bounds from the current
    normals (a damped average of the iterates), the box LCP solved again,
    until the iterates agree to tol x max|x|.  Returns (x, outer iterations);
    raises if it does not settle."""
    x = dantzig_two_phase(A, b, lo, hi, findex) if x0 is None else x0.copy()
    xb = x.copy()
    for k in range(max_outer):
        lo2, hi2 = friction_bounds(lo, hi, findex, xb)
        xn = box_lcp(A, b, lo2, hi2)
        d = np.abs(xn - x).max()
        x = xn
        xb = damping * xb + (1.0 - damping) * x
        if d <= tol * max(1.0, np.abs(x).max()) and natural_residual(A, b, lo, hi, findex, x) <= \
                1e-9 * max(1.0, np.abs(x).max()):
            return x, k + 1
    raise RuntimeError("findex_fixed_point: the friction bounds did not settle")


def natural_residual(A, b, lo, hi, findex, x):
    """max_i |x_i - proj_[lo_i(x), hi_i(x)](x_i - (A x - b)_i / A_ii)|, the
    natural-map residual with the friction bounds following x (unnormalised)."""
    lo2, hi2 = friction_bounds(lo, hi, findex, x)
    w = A @ x - b
    t = np.clip(x - w / np.diag(A), lo2, hi2)
    return float(np.abs(x - t).max()) if x.size else 0.0


def complementarity(A, b, lo, hi, findex, x):
    """The min-map complementarity error in the units of x,
    max_i max(min(x_i - lo_i, w_i+ / A_ii), min(hi_i - x_i, w_i- / A_ii)),
    w = A x - b, w+ = max(w, 0), w- = max(-w, 0), with the friction bounds
    following x (unnormalised)."""
    lo2, hi2 = friction_bounds(lo, hi, findex, x)
    w = A @ x - b
    D = np.diag(A)
    wp = np.maximum(w, 0.0) / D
    wm = np.maximum(-w, 0.0) / D
    c = np.maximum(np.minimum(x - lo2, wp), np.minimum(hi2 - x, wm))
    return float(np.abs(c).max()) if x.size else 0.0
