"""Exact FP64 solutions of the step goldens' LCPs (tests/golden/lcp_exact.npz).

For every snapshot of step_box_stack / step_pile256 / step_capsule_pile96 the
oracle forms the quickstep rows of the recorded contacts (oracle/port, bit-exact
with the reference's dSINGLE rows) and oracle/lcp_exact.py solves them in FP64:

* `{name}_s{k}_two_phase`: the reference's Dantzig treatment of friction rows
  (lcp.cpp:836-1160), checked here against the reference's own dDOUBLE
  dWorldStep multipliers in the golden (`s{k}_lambda_dantzig`);
* `{name}_s{k}_exact`: that solution continued to an exact solution of the
  findex LCP quickstep's SOR_LCP solves (friction bounds following the final
  normals), natural-map residual <= 1e-9 of max|lambda|.

Multipliers are in contact order, [nc, 3] (normal, friction 1, friction 2).
The snapshot where the reference's Dantzig solver gave up (its "LCP internal
error") is skipped.  Takes a few minutes (dense pivoting on up to ~1,800 rows):

    python tests/golden/make_lcp_exact.py
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

NAMES = ("box_stack", "pile256", "capsule_pile96")


def snapshot_rows(P, g, k):
    """Contact-order rows of snapshot k, body inverse masses and inertias."""
    from oracle.port.port import world_inv_inertia
    iters, _, mode, _ = [int(x) for x in g["ints"]]
    pre, cb, cs = g[f"s{k}_pre"], g[f"s{k}_cb"], g[f"s{k}_cs"]
    b = g["bodies0"].copy()
    b[:, 0:3], b[:, 3:7], b[:, 7:10], b[:, 10:13] = pre[:, 0:3], pre[:, 3:7], pre[:, 19:22], pre[:, 22:25]
    _, rows = P.world(b, g["params"], iters, dyn=0, reorder=0).quickstep_contact_rows(
        cb, np.full(len(cb), mode, np.int32), cs)
    invI, invm = world_inv_inertia(pre, b)
    return rows, invm, invI


def main():
    from oracle import lcp_exact as X
    from oracle.port.port import Port
    P = Port()
    out = {}
    for name in NAMES:
        g = np.load(os.path.join(HERE, f"step_{name}.npz"))
        for k in range(len(g["snaps"])):
            if g[f"s{k}_dantzig_lcp_error"][1]:
                continue
            t0 = time.perf_counter()
            rows, invm, invI = snapshot_rows(P, g, k)
            A, b, lo, hi, fi = X.dense_problem(rows, invm, invI)
            x2 = X.dantzig_two_phase(A, b, lo, hi, fi)
            ref = g[f"s{k}_lambda_dantzig"].reshape(-1)
            scale = max(1.0, float(np.abs(ref).max()))
            d2 = float(np.abs(x2 - ref).max()) / scale
            assert d2 <= 1e-4, (name, k, d2)
            xf, outer = X.findex_fixed_point(A, b, lo, hi, fi, x0=x2)
            rf = X.natural_residual(A, b, lo, hi, fi, xf) / max(1.0, float(np.abs(xf).max()))
            nc = len(g[f"s{k}_cb"])
            out[f"{name}_s{k}_two_phase"] = x2.reshape(nc, 3)
            out[f"{name}_s{k}_exact"] = xf.reshape(nc, 3)
            print(f"{name} s{k}: {len(b)} rows, two-phase vs reference dDOUBLE {d2:.2e}, exact after {outer} "
                  f"outer solves (residual {rf:.1e}), exact vs reference "
                  f"{float(np.abs(xf - ref).max()) / scale:.2e} of max|lambda|, {time.perf_counter() - t0:.0f} s",
                  flush=True)
    np.savez_compressed(os.path.join(HERE, "lcp_exact.npz"), **out)


if __name__ == "__main__":
    main()
