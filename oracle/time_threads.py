"""Times the reference's own multi-threaded stepping against the oracle's
restatement of it, on this machine's cores: a check that the CPU legs of the
benchmark (which run the oracle, since the compiled reference does not travel
to other machines) are not slower than the reference itself would be.

Scene: the settled 32,768-body pile (ode_gb300/data/pile32768_settled.npz),
the full user loop (dSpaceCollide -> near callback -> dCollide -> contact
joints -> dWorldQuickStep, stock random row reordering) with --sweeps SOR
sweeps per step.  The reference runs through tests/golden/gen_golden.cpp's
`timing` mode, linked against oracle/_ref/single/libode.a (built from the
reference's sources by oracle/ref_build/Makefile; x86 only, so this runs
where the reference sources are), with its built-in thread pool attached by
dWorldSetStepThreadingImplementation; the oracle with port_world_set_threads.

    python oracle/time_threads.py --threads 1 8 --steps 2 --sweeps 200

Test infrastructure only: it measures the checker, never the product.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from ode_gb300 import scenes  # noqa: E402

SETTLED = os.path.join(ROOT, "ode_gb300", "data", "pile32768_settled.npz")


def settled_pile():
    sc = scenes.pile(32768, seed=1)
    bodies = sc.bodies.copy()
    with np.load(SETTLED) as z:
        bodies[:, 0:3], bodies[:, 3:7], bodies[:, 7:10], bodies[:, 10:13] = z["pos"], z["q"], z["lvel"], z["avel"]
    return sc, bodies


def reference_exe(ref: str) -> str:
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden
    return make_golden.build(ref)["single"]


def time_reference(exe, sc, bodies, threads, steps, sweeps):
    hdr = np.array([sc.nb, sc.ng, steps + 1, sweeps, threads, sc.maxc, sc.surface_mode, sc.hash_levels[0],
                    sc.hash_levels[1]], np.int32)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            for a in (hdr, sc.world_params(), sc.surface(), bodies.astype(np.float32), sc.geom_cls, sc.geom_body,
                      sc.geom_pos, sc.geom_R, sc.geom_dims):
                f.write(np.ascontiguousarray(a).tobytes())
        subprocess.run([exe, "timing", fin, fout], check=True)
        t = np.fromfile(fout, dtype=np.float64, count=3 * (steps + 1)).reshape(steps + 1, 3)
    return t[1:]  # the first step warms the allocator and the thread pool


def time_oracle(sc, bodies, threads, steps, sweeps):
    from oracle.port.port import Port
    P = Port()
    P.lib.port_rand_set_seed(0)
    w = P.world(bodies, sc.world_params(), sweeps, dyn=0, reorder=1)
    w.set_threads(threads)
    w.attach_space(sc.geom_cls, sc.geom_body, sc.geom_pos, sc.geom_R, sc.geom_dims, sc.hash_levels, sc.maxc,
                   sc.surface_mode, sc.surface())
    w.sim_step()
    out = []
    for _ in range(steps):
        t0 = time.perf_counter()
        nc = w.sim_step()
        out.append((time.perf_counter() - t0, nc))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ODE_REFERENCE_DIR"),
                    help="reference source tree (default: $ODE_REFERENCE_DIR)")
    ap.add_argument("--threads", type=int, nargs="+", default=[1, 8])
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--sweeps", type=int, default=200)
    args = ap.parse_args()
    if not args.ref:
        ap.error("--ref or ODE_REFERENCE_DIR must name the reference source tree")
    exe = reference_exe(args.ref)
    sc, bodies = settled_pile()
    print(f"pile{sc.nb}, {args.sweeps} sweeps per step, {args.steps} timed steps after one untimed")
    print("threads | reference: collide s, quickstep s, step s | oracle: step s | oracle/reference")
    for T in args.threads:
        r = time_reference(exe, sc, bodies, T, args.steps, args.sweeps)
        o = time_oracle(sc, bodies, T, args.steps, args.sweeps)
        rc, rq = float(np.mean(r[:, 0])), float(np.mean(r[:, 1]))
        os_ = float(np.mean([x[0] for x in o]))
        print(f"{T:7d} | {rc:8.3f} {rq:8.3f} {rc + rq:8.3f} | {os_:8.3f} | {os_ / (rc + rq):5.2f}  "
              f"(contacts {int(r[0, 2])} / {o[0][1]})")


if __name__ == "__main__":
    main()
