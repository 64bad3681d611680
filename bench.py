"""Benchmark: body-steps/s of the rigid-body step on the 32,768-body pile at
LCP residual <= 1e-4 (one GB300).

Workload (`pile32768`): 32,768 bodies (50 % spheres r~U[0.05,0.25] m, 50 %
boxes sides ~U[0.1,0.5] m, density ~U[500,2000]) dropped on a jittered 32^3
grid into an open box of 5 static planes; dt 1/120, mu 0.6, dContactApprox1,
<= 4 contacts per pair, hash-space broad phase.  The pile first settles for
--settle steps (900: the top of the grid falls 19 m, about 2 s) with the
configured 30 sweeps per step (untimed), then W warm-up and K timed steps run.

A step is the fused path: gbodeSpaceCollideContacts (broad phase, narrow
phase, contact joints on the device) + dWorldQuickStep with the coloured PGS
(two-level sweep: column interiors in shared memory, crossing manifolds in
global colours; momentum 0.8 between sweeps), warm-started from the previous
step's multipliers (contact cache keyed by geom pair and slot), W = 1.0,
iterating until the natural-map LCP residual (relative to max(1,
max|lambda|)) is <= 1e-4 -- checks at least 5 sweeps apart, at half the
predicted distance to the target -- or 3000 sweeps.  `value` counts only
steps that reached the target.  Timing: CUDA events on the world's stream
around each step, an L2 flush (256 MB write) before every timed step, outside
the events.  `e2e` runs the same steps through the C ABI with host buffers:
the full body state is set from host memory before and read back after every
step, wall-clock timed.  The line also carries the same steps rerun without
momentum (`without_momentum`) and with the library's default sweep
(`dropin_defaults`), the learned warm start on them (`learned`), the batched
capsule-chain and vehicle worlds (`batched`), the CPU baseline, the roofline
of the sweep kernel and the SM clocks sampled during the timed steps.

--impl reference times the reference algorithm on the host CPU (the oracle
port of ODE's dSpaceCollide + dWorldQuickStep: random row reordering every 8
sweeps, no warm start, --ref-sweeps sweeps per step, the sweeps on every
usable core as the reference's opt-in multi-threaded stepping runs them) from
the same settled pile, W warm-up and K timed steps like the GPU arm, and
counts only steps whose own FP64 residual reaches the target.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "body-steps/s at LCP residual \u22641e-4: plain GPU PGS vs learned warm start, 1 GB300"
B_ROW = 132        # algorithmic bytes per PGS row-iteration
B_ROW_CHECK = 80   # bytes per row of a residual sweep (J 64 + lambda + findex + bodies)
B_ROW_MOM = 8      # momentum between sweeps: a row's previous result read and written
B_BODY_MOM = 128   # momentum between sweeps: a body's accumulators and their previous values, read and written
# DRAM bytes (read + write) per launch of the sweep kernel on the settled 32,768-body pile,
# measured with ncu (dram__bytes_read.sum + dram__bytes_write.sum, mean of two launches):
# k_pgs_slab (two-level sweep, exact crossing colours, momentum 0.8, kernel of commit 4fcd219):
# 80.0 and 79.0 MB; k_pgs (one-level, no momentum): 240.4 and 204.2 MB.  The rows stay in L2 /
# shared memory across sweeps.
PGS_TRAFFIC = {"gb::k_pgs_slab": 7.953e7, "gb::k_pgs": 2.223e8}
PGS_TRAFFIC_SOURCE = {"gb::k_pgs_slab": "kernel of commit 4fcd219, momentum 0.8, exact crossing colours",
                      "gb::k_pgs": "kernel of commit 53e9ef8, one-level sweep without momentum"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbode", choices=["gbode", "reference"])
    ap.add_argument("--n", type=int, default=32768)
    ap.add_argument("--settle", type=int, default=900)
    ap.add_argument("--target", type=float, default=1e-4)
    ap.add_argument("--check-every", type=int, default=5,
                    help="residual checks at least this many sweeps apart (every this many with --checks fixed)")
    ap.add_argument("--checks", choices=("predicted", "fixed"), default="predicted",
                    help="residual-check schedule (gbodeWorldSetResidualChecks)")
    ap.add_argument("--reform-every", type=int, default=0,
                    help="sweeps between re-formed body accumulators (0: the library's default, 500)")
    ap.add_argument("--sor-w", type=float, default=1.0,
                    help="SOR relaxation W (dWorldSetQuickStepW); the reference's default 1.3 stalls when warm-started")
    ap.add_argument("--max-iters", type=int, default=3000)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--warm-scale", type=float, default=1.0,
                    help="previous-step lambda warm start from the contact cache (0 = cold start)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--profile-steps", type=int, default=0, help="run N steps only (for ncu), no JSON")
    ap.add_argument("--curve", action="store_true",
                    help="after the warm-up, one step from the same state with and without momentum: print the "
                         "residual at each check and the sweeps done by then (one JSON line each), no bench line")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-warm-start leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched capsule-chain leg")
    ap.add_argument("--chains", type=int, default=8192, help="batched leg: independent capsule chains")
    ap.add_argument("--vehicles", type=int, default=65536, help="batched leg: independent vehicle worlds (0: skip)")
    ap.add_argument("--save-settled", default=None, help="write the settled state (.npz) and exit")
    ap.add_argument("--pgs-blocks", type=int, default=0, help="thread blocks of the PGS kernel (0: one per SM)")
    ap.add_argument("--passes", type=int, default=1, help="passes over a manifold's rows per visit")
    ap.add_argument("--two-level", type=int, default=2,
                    help="two-level sweep of the pile's solver with this many interior phases a sweep "
                         "(gbodeWorldSetTwoLevelSweep; 0: off)")
    ap.add_argument("--cross-classes", type=int, default=0,
                    help="two-level sweep: crossing colours merged into this many mass-split classes "
                         "(gbodeWorldSetCrossClasses; 0: exact colours)")
    ap.add_argument("--momentum", type=float, default=0.8,
                    help="momentum between the coloured solver's sweeps in the residual-target legs "
                         "(gbodeWorldSetSweepMomentum; 0: plain sweeps)")
    ap.add_argument("--sweep-sync", choices=("neighbours", "grid"), default="neighbours",
                    help="two-level sweep: blocks wait on the blocks sharing their bodies, or on a grid barrier "
                         "after every step (gbodeWorldSetSweepSync)")
    ap.add_argument("--from-settled", action="store_true",
                    help="start the pile from ode_gb300/data/pile32768_settled.npz instead of settling (profiling)")
    ap.add_argument("--ref-sweeps", type=int, default=1500,
                    help="reference arm: SOR sweeps per step (cold starts need ~1000-1500 to reach the target)")
    ap.add_argument("--weights", default=None, help="learned warm start parameters (.npz)")
    ap.add_argument("--ref-threads", type=int, default=0,
                    help="CPU legs: SOR threads (0: every core this process may run on; 1: the reference's "
                         "default self-threaded stepping)")
    return ap.parse_args()


def host_threads(args) -> int:
    """SOR threads of the CPU legs: --ref-threads, else every usable core."""
    if args.ref_threads > 0:
        return args.ref_threads
    try:
        n = len(os.sched_getaffinity(0))
    except AttributeError:
        n = os.cpu_count() or 1
    # a CPU quota below the visible cores (cgroup v2 cpu.max "quota period")
    # would deschedule spinning threads: stay within it
    try:
        with open("/sys/fs/cgroup/cpu.max") as f:
            quota, period = f.read().split()[:2]
        if quota != "max":
            n = min(n, max(1, int(int(quota) // int(period))))
    except (OSError, ValueError):
        pass
    return max(1, n)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index: int = 0):
        self.index, self.samples, self.proc, self.thread = index, [], None, None

    def start(self):
        cmd = ["nvidia-smi", f"--id={self.index}",
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx = max(mx, float(s[1]))
                for k, nm in enumerate(names):
                    if s[4 + k].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gbode" else "gloo"
        dist.init_process_group(backend=backend)
    return ws, rank, local


def dist_max(x: float, ws: int, device) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(x: float, ws: int, device) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------- reference arm
SETTLED = os.path.join(ROOT, "ode_gb300", "data", "pile32768_settled.npz")


def _port_pile(P, sc, bodies, sweeps, threads):
    """The oracle's world of the pile (stock random reordering, no warm
    start), SOR sweeps on `threads` host threads, residual evaluated per step."""
    w = P.world(bodies, sc.world_params(), sweeps, dyn=0, reorder=1)
    w.set_threads(threads)
    w.set_residual(True)
    w.attach_space(sc.geom_cls, sc.geom_body, sc.geom_pos, sc.geom_R, sc.geom_dims, sc.hash_levels, sc.maxc,
                   sc.surface_mode, sc.surface())
    return w


def _port_steps(w, steps, target):
    """`steps` oracle steps: wall time, collision / quickstep seconds, and
    per step the FP64 residual relative to max(1, max|lambda|)."""
    t0 = time.perf_counter()
    coll, quick, rel, nc = [], [], [], 0
    for _ in range(steps):
        nc += w.sim_step()
        tc, tq, r, lm = w.last_stats()
        coll.append(tc)
        quick.append(tq)
        rel.append(r / max(1.0, lm))
    return time.perf_counter() - t0, coll, quick, rel, nc


def run_reference(args, ws, rank):
    """The reference algorithm on the host CPU (the oracle port of ODE's
    collide + quickstep, stock random row reordering, no warm start -- the
    reference compiles it out) from the settled pile the GPU arm times
    (ode_gb300/data/pile32768_settled.npz, written by `bench.py
    --save-settled`), --ref-sweeps SOR sweeps per step on every usable core
    (the reference's opt-in multi-threaded stepping), W warm-up steps and K
    timed steps like the GPU arm.  Every step's FP64 LCP residual is
    evaluated on its own rows; the value counts only steps at the target."""
    if rank != 0:
        return
    from oracle.port.port import Port
    from ode_gb300 import scenes
    P = Port()
    sc = scenes.pile(args.n, seed=1)
    bodies = sc.bodies.copy()
    t0 = time.perf_counter()
    settle_note = "settled state from the fixture"
    fixture = SETTLED if args.n == 32768 else None
    if fixture and os.path.exists(fixture):
        with np.load(fixture) as z:
            bodies[:, 0:3], bodies[:, 3:7], bodies[:, 7:10], bodies[:, 10:13] = z["pos"], z["q"], z["lvel"], z["avel"]
    P.lib.port_rand_set_seed(0)
    threads = host_threads(args)
    w = _port_pile(P, sc, bodies, args.ref_sweeps, threads)
    if not (fixture and os.path.exists(fixture)):
        settle_note = f"{args.settle} CPU settle steps"
        for _ in range(args.settle):
            w.sim_step()
    for _ in range(args.warmup):
        w.sim_step()
    setup_s = time.perf_counter() - t0
    dt, coll, quick, rel, nc = _port_steps(w, args.steps, args.target)
    ok = sum(1 for r in rel if r <= args.target)
    value = sc.nb * ok / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"pile{sc.nb}", "bodies": sc.nb, "dt": sc.dt, "sweeps_per_step": args.ref_sweeps,
                       "solver": "reference quickstep (oracle port of collide + quickstep), stock random "
                                 "row reordering, no warm start (compiled out in the reference), "
                                 f"multi-threaded SOR sweeps on {threads} threads",
                       "sor_threads": threads,
                       "threads_note": "the oracle's threaded sweeps (levels of rows that share no body, a "
                                       "barrier between levels) give the single-threaded result to the bit "
                                       "and ran 5.3x faster on 8 cores than the reference's own threaded "
                                       "mode at its best (one thread) where the reference compiles",
                       "start": settle_note, "contacts_per_step": nc / args.steps,
                       "collide_ms_per_step": 1e3 * float(np.mean(coll)),
                       "quickstep_ms_per_step": 1e3 * float(np.mean(quick)),
                       "fp64_residual_max": float(max(rel)), "fp64_residual_median": float(np.median(rel)),
                       "steps_at_target": ok, "residual_target": args.target,
                       "same_steps_as_gpu_arm": "yes: the same --steps and --warmup",
                       "body_steps_per_s_regardless_of_residual": sc.nb * args.steps / dt},
            "cpu_baseline": {"value": value, "unit": "body-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} steps of pile{sc.nb} ({args.ref_sweeps} sweeps each) after "
                                       f"{args.warmup} warm-up steps and {setup_s:.0f} s of set-up, SOR sweeps "
                                       f"on {threads} host threads (collision and row assembly on one)"},
            "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------- gbode arm
def run_gbode(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from ode_gb300 import build, ode, scenes, sim
    build.build()
    L = ode.load()
    stream = torch.cuda.Stream(device=dev)
    sc = scenes.pile(args.n, seed=1 + rank)
    w = sim.GBWorld(sc, stream=ctypes.c_void_p(stream.cuda_stream))
    if args.warm_scale > 0:
        L.gbodeWorldSetWarmStart(w.w, 1, args.warm_scale)
    L.dWorldSetQuickStepW(w.w, args.sor_w)
    if args.pgs_blocks:
        L.gbodeWorldSetSolverBlocks(w.w, args.pgs_blocks)
    L.gbodeWorldSetManifoldPasses(w.w, args.passes)
    if args.from_settled:
        with np.load(SETTLED) as z:
            st = w.state()
            st[:, 0:3], st[:, 3:7], st[:, 19:22], st[:, 22:25] = z["pos"], z["q"], z["lvel"], z["avel"]
            st[:, 7:19] = scenes.quat_to_R(z["q"])
        w.set_state(st)
    else:
        # settle with the configured 30 sweeps per step (untimed)
        for _ in range(args.settle):
            w.step_fused()
    w.sync()
    L.gbodeWorldSetResidualTarget(w.w, args.target, args.check_every, args.max_iters)
    L.gbodeWorldSetResidualChecks(w.w, ode.GBODE_CHECKS_FIXED if args.checks == "fixed" else ode.GBODE_CHECKS_PREDICTED,
                                  args.reform_every)
    L.gbodeWorldSetTwoLevelSweep(w.w, args.two_level)
    L.gbodeWorldSetSweepSync(w.w, ode.GBODE_SYNC_GRID if args.sweep_sync == "grid" else ode.GBODE_SYNC_NEIGHBOURS)
    L.gbodeWorldSetCrossClasses(w.w, args.cross_classes)
    L.gbodeWorldSetSweepMomentum(w.w, args.momentum)
    L.gbodeWorldSetTiming(w.w, 1)
    if args.profile_steps:
        for _ in range(args.profile_steps):
            w.step_fused()
        w.sync()
        return
    for _ in range(args.warmup):
        w.step_fused()
    w.sync()
    settled = w.state()
    # the e2e and learned legs rerun the timed steps from this state (bodies
    # and warm-start cache, gbodeWorldSaveSnapshot)
    if not args.save_settled and L.gbodeWorldSaveSnapshot(w.w) != 1:
        raise RuntimeError(L.gbodeGetLastError().decode())
    if args.save_settled:
        np.savez_compressed(args.save_settled, pos=settled[:, 0:3], q=settled[:, 3:7], lvel=settled[:, 19:22],
                            avel=settled[:, 22:25], seed=1 + rank, settle=args.settle + args.warmup)
        return
    if args.curve:
        residual_curves(args, L, w)
        return
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    peak, peak_kind = measured_peak()
    launches0 = L.gbodeKernelLaunchCount()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    T = timed_steps(w, stream, flush, args.steps)
    clk = clocks.stop()
    launches = L.gbodeKernelLaunchCount() - launches0
    step_ms, solve_ms, sweeps, resid, rows, contacts, colours = (T[k] for k in (
        "step_ms", "solve_ms", "sweeps", "resid", "rows", "contacts", "colours"))
    total_ms = sum(step_ms)
    ok_steps = sum(1 for r in resid if r <= args.target)
    total_ms_max = dist_max(total_ms, ws, dev)
    body_steps = dist_sum(sc.nb * ok_steps, ws, dev)
    value = body_steps / (total_ms_max / 1e3)
    # FP64 residual of the last step's solution, evaluated on the device
    r64, ce, ml = w.last_residual()
    fp64_rel = r64 / max(1.0, ml)
    # roofline of the dominant kernel (the persistent PGS sweep kernel): every
    # row relaxation counts B_ROW, the interior rows of the two-level sweep once
    # per interior phase
    checks = T["checks"]
    extra = max(0, args.two_level - 1)
    # momentum: every sweep but the first and the checked ones moves the rows and bodies on
    mom_bytes = sum(max(0, s - c - 1) * (m * B_ROW_MOM + sc.nb * B_BODY_MOM)
                    for s, m, c in zip(sweeps, rows, checks)) if args.momentum > 0 else 0
    pgs_bytes = mom_bytes + sum(s * (m + extra * mi) * B_ROW + c * m * B_ROW_CHECK
                    for s, m, mi, c in zip(sweeps, rows, T["interior_rows"], checks))
    pgs_s = sum(solve_ms) / 1e3
    achieved = pgs_bytes / pgs_s / 1e9 if pgs_s > 0 else 0.0
    # e2e through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        restore_snapshot(L, w)
        host = w.state()
        h2d = 112 * sc.nb   # pos, q, R, lvel, avel (gbodeWorldSetState's pinned upload)
        d2h = 112 * sc.nb   # pos, q, R, lvel, avel (gbodeWorldGetState's pinned download)
        n_ok, t0 = 0, time.perf_counter()
        for _ in range(args.steps):
            w.set_state(host)
            w.step_fused()
            host = w.state()
            if w.stats().residual <= args.target:
                n_ok += 1
        e2e_s = dist_max(time.perf_counter() - t0, ws, dev)
        e2e = {"value": dist_sum(sc.nb * n_ok, ws, dev) / e2e_s, "unit": "body-steps/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h}
    # the same steps without momentum between sweeps, and with the library's
    # defaults (one-level sweep, no momentum): the plain drop-in at the target
    def guarded(two_level, momentum):
        try:
            return rerun_leg(args, w, L, stream, flush, sc.nb, ws, dev, two_level, momentum)
        except RuntimeError as e:  # a failed step: the leg is reported, the bench line still printed
            L.gbodeWorldSetTwoLevelSweep(w.w, args.two_level)
            L.gbodeWorldSetSweepMomentum(w.w, args.momentum)
            return {"unavailable": str(e)}
    no_mom = guarded(args.two_level, 0.0) if args.momentum > 0 else None
    dropin = guarded(0, 0.0)
    dropin["settings"] = ("the library's default sweep (one-level coloured, no two-level sweep, no momentum) at the "
                          "residual target, with the other legs' previous-step warm start, W and check schedule")
    # learned warm start: the same settled state, the same timed loop
    learned = None
    if not args.no_learned:
        learned = learned_leg(args, w, L, stream, flush, T, sc.nb, ws, dev)
        if "value" in learned and dropin.get("value", 0) > 0:
            # the learned form against the plain drop-in at the same residual
            learned["vs_dropin_defaults"] = learned["value"] / dropin["value"]
    # batched independent worlds: capsule chains with hinge/ball joints
    batched = None
    if not args.no_batched and ws == 1:
        batched = {"chains": batched_leg(args, L, stream, dev, "chains")}
        if args.vehicles > 0:
            try:
                batched["vehicles"] = batched_leg(args, L, stream, dev, "vehicles")
            except RuntimeError as e:
                batched["vehicles"] = {"unavailable": str(e)}
    # CPU baseline: the oracle port from the same settled state, same sweep count
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sc, w, args, host_threads(args))
    if rank != 0:
        return
    m_mean = float(np.mean(rows))
    line = {
        "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"pile{sc.nb}", "bodies": sc.nb, "dt": sc.dt, "mu": sc.mu, "maxc": sc.maxc,
                   "settle_steps": args.settle, "residual_target": args.target, "check_every": args.check_every,
                   "checks": (f"predicted (half the predicted distance, {args.check_every}-64 sweeps apart)"
                              if args.checks == "predicted" else f"every {args.check_every} sweeps"),
                   "checks_per_step": float(np.mean(T["checks"])),
                   "max_sweeps": args.max_iters, "l2": "256 MB flush before every timed step (outside the events)",
                   "parallelism": f"replicas{ws}" if ws > 1 else "single",
                   "solver": f"coloured PGS (W {args.sor_w}), persistent cooperative kernel"
                             + (f", two-level sweep ({args.two_level} interior phases a sweep, "
                                + ("neighbour waits" if min(T["neighbour_waits"]) else "grid barriers")
                                + (f", crossing colours in {min(T['cross_classes'])} mass-split classes"
                                   if min(T["cross_classes"]) else "") + ")"
                                if args.two_level else "")
                             + (f", momentum {args.momentum} between sweeps (at the end of a step: min "
                                f"{min(T['momentum']):.3g}, max {max(T['momentum']):.3g})" if args.momentum > 0 else ""),
                   "interior_rows_per_step": float(np.mean(T["interior_rows"])),
                   "interior_colours": int(np.median(T["interior_colours"])),
                   "warm_start": f"previous-step lambda x {args.warm_scale}" if args.warm_scale > 0 else "cold",
                   "rows_per_step": m_mean, "contacts_per_step": float(np.mean(contacts)),
                   "colours": int(np.median(colours)), "sweeps_per_step": float(np.mean(sweeps)),
                   "steps_at_target": ok_steps, "fp32_residual_max": float(max(resid)),
                   "fp64_residual_last_step": fp64_rel,
                   "complementarity_last_step": ce / max(1.0, ml),
                   "normalisation": "residual and complementarity (min-map form, in the units of lambda) "
                                    "relative to max(1, max|lambda|) of the step's own solution",
                   "contact_rows_per_s": float(np.sum(rows)) / (total_ms / 1e3),
                   "solve_share": pgs_s * 1e3 / total_ms},
        "roofline": {"bound": "hbm", "kernel": "gb::k_pgs_slab" if args.two_level else "gb::k_pgs",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": PGS_TRAFFIC["gb::k_pgs_slab" if args.two_level else "gb::k_pgs"],
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, mean of two launches "
                                       "of the same kernel from the settled pile ("
                                       + PGS_TRAFFIC_SOURCE["gb::k_pgs_slab" if args.two_level else "gb::k_pgs"] + ")",
                     "algorithmic_bytes_per_launch": pgs_bytes / args.steps},
        "clocks": clk,
        "gpu_launches": launches,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "without_momentum": no_mom,
        "dropin_defaults": dropin,
        "learned": learned,
        "batched": batched,
    }
    print(json.dumps(line))


def residual_curves(args, L, w):
    """One step from the saved state with the configured solver, with and
    without momentum: the FP32 residual at every check and the sweeps done by
    then (gbodeWorldGetResidualHistory / gbodeWorldGetResidualSweeps)."""
    hist = np.zeros(256, np.float32)
    at = np.zeros(256, np.int32)
    for beta in sorted({0.0, args.momentum}):
        restore_snapshot(L, w)
        L.gbodeWorldSetSweepMomentum(w.w, beta)
        w.step_fused()
        w.sync()
        st = w.stats()
        n = L.gbodeWorldGetResidualHistory(w.w, hist.ctypes.data_as(ode_f32p()), 256)
        L.gbodeWorldGetResidualSweeps(w.w, at.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), 256)
        print(json.dumps({"momentum": beta, "two_level": args.two_level, "cross_classes": args.cross_classes,
                          "sweeps": st.iterations, "residual": st.residual, "momentum_at_end": st.momentum,
                          "checks": [[int(a), float(h)] for a, h in zip(at[:n], hist[:n])]}))


def restore_snapshot(L, w):
    if L.gbodeWorldRestoreSnapshot(w.w) != 1:
        raise RuntimeError(L.gbodeGetLastError().decode())


def batched_leg(args, L, stream, dev, kind):
    """Thousands of independent worlds as islands of one step, stepped by one
    fused step (one persistent PGS launch) and timed like the pile:
    chains -- articulated capsule chains (N log-uniform in [2, 32], hinge +-60
    deg limits alternating with ball joints) dropped onto a plane, dt 1/240;
    vehicles -- a box chassis on four hinge2-suspended, motored sphere wheels
    among 0-16 static box obstacles per world, dt 1/120."""
    import torch
    from ode_gb300 import scenes, sim
    t0 = time.perf_counter()
    if kind == "chains":
        sc, settle = scenes.chains(args.chains, seed=3), 240
    else:
        sc, settle = scenes.vehicles(args.vehicles, seed=4), 120
    w = sim.GBWorld(sc, stream=ctypes.c_void_p(stream.cuda_stream))
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    L.dWorldSetQuickStepW(w.w, 1.0)
    for _ in range(settle):  # fall and land with the configured 20 iterations
        if not w.step_fused():
            raise RuntimeError(L.gbodeGetLastError().decode())
    w.sync()
    # every leg runs the same steps: from this state (gbodeWorldSaveSnapshot)
    if L.gbodeWorldSaveSnapshot(w.w) != 1:
        raise RuntimeError(L.gbodeGetLastError().decode())
    setup_s = time.perf_counter() - t0
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    out = {"workload": f"{kind}{args.chains if kind == 'chains' else args.vehicles}", "bodies": sc.nb,
           "geoms": sc.ng, "joints": int(len(sc.joints)), "dt": sc.dt, "setup_s": round(setup_s, 1)}
    L.gbodeWorldSetTiming(w.w, 0)
    for label, target, graph in (("iterations20", 0.0, False), ("iterations20_graph", 0.0, True),
                                 ("residual", args.target, False), ("residual_graph", args.target, True)):
        if target > 0:
            L.gbodeWorldSetResidualTarget(w.w, target, args.check_every, args.max_iters)
            L.gbodeWorldSetSweepMomentum(w.w, args.momentum)
        restore_snapshot(L, w)
        for _ in range(args.warmup):
            if graph:
                w.step_graph()
            else:
                w.step_fused()
        w.sync()
        T = timed_steps(w, stream, flush, args.steps, graph=graph)
        ms = sum(T["step_ms"])
        ok = sum(1 for r in T["resid"] if target == 0 or r <= target)
        out[label] = {"body_steps_per_s": sc.nb * ok / (ms / 1e3), "ms_per_step": ms / args.steps,
                      "sweeps_per_step": float(np.mean(T["sweeps"])), "rows_per_step": float(np.mean(T["rows"])),
                      "contacts_per_step": float(np.mean(T["contacts"])), "colours": int(np.median(T["colours"])),
                      "steps_at_target": ok}
    # solver settings tuned on the running world (gbodeWorldAutotune), then the residual leg again
    restore_snapshot(L, w)
    tu = w.autotune(steps=3, graph=True)
    restore_snapshot(L, w)
    for _ in range(args.warmup):
        w.step_graph()
    w.sync()
    T = timed_steps(w, stream, flush, args.steps, graph=True)
    ms = sum(T["step_ms"])
    ok = sum(1 for r in T["resid"] if r <= args.target)
    out["residual_tuned_graph"] = {"body_steps_per_s": sc.nb * ok / (ms / 1e3), "ms_per_step": ms / args.steps,
                                   "sweeps_per_step": float(np.mean(T["sweeps"])), "steps_at_target": ok,
                                   "tuning": {"blocks": tu.blocks, "passes": tu.passes,
                                              "check_every": tu.check_every, "threads_per_block": tu.threads,
                                              "staged_rows_per_buffer": tu.chunk_rows, "two_level": tu.two_level,
                                              "momentum": round(tu.momentum, 3),
                                              "candidates": tu.candidates}}
    if kind == "vehicles" and not args.no_learned:
        out["residual_learned_tuned_graph"] = learned_batched(args, L, w, stream, flush, sc.nb)
    r64, _, ml = w.last_residual()
    out["fp64_residual_last_step"] = r64 / max(1.0, ml)
    out["note"] = ("value counts steps at the residual target (residual) or every step at the configured 20 "
                   "sweeps (iterations20); the chains are islands of one world, solved by the same coloured "
                   "persistent kernel; *_graph: the fused step replayed from a CUDA graph (gbodeWorldStepFused); "
                   "*_tuned: after gbodeWorldAutotune chose threads a block (colour-group tile), staged rows a "
                   "buffer, the two-level sweep, solver blocks, passes per group and check interval; "
                   "*_learned_*: the learned warm start with the plain start as fallback (per step, whichever "
                   "start has the lower residual), on the tuned settings; "
                   "every leg starts from the same state (gbodeWorldRestoreSnapshot): W warm-up steps, then the "
                   "same K timed steps")
    w.close()
    return out


def learned_batched(args, L, w, stream, flush, nb):
    """The residual leg of a batched workload with the learned warm start
    (the plain previous-step start as fallback), graph-replayed: like the
    other legs, the world's snapshot restored, W untimed steps (they also
    record the graph), then the same K timed steps."""
    import ctypes as C
    from ode_gb300 import learned
    path = args.weights or learned.WEIGHTS
    if not os.path.exists(path):
        return {"unavailable": f"no trained parameters at {os.path.relpath(path, ROOT)}"}
    params = learned.load(path)
    try:
        restore_snapshot(L, w)
        if L.gbodeWorldSetLearnedWarmStart(w.w, params.ctypes.data_as(C.POINTER(C.c_float)), 1) != 1:
            return {"unavailable": L.gbodeGetLastError().decode()}
        for _ in range(args.warmup):
            w.step_graph()
        w.sync()
        st = np.zeros(3, np.float32)
        chosen = []
        T = {k: [] for k in ("step_ms", "sweeps", "resid")}
        for _ in range(args.steps):
            t = timed_steps(w, stream, flush, 1, graph=True)
            for k in T:
                T[k] += t[k]
            L.gbodeWorldGetLearnedStats(w.w, st.ctypes.data_as(C.POINTER(C.c_float)))
            chosen.append(float(st[0]))
    except RuntimeError as e:
        return {"unavailable": str(e)}
    finally:
        L.gbodeWorldSetLearnedWarmStart(w.w, None, 0)
    ms = sum(T["step_ms"])
    ok = sum(1 for r in T["resid"] if r <= args.target)
    return {"body_steps_per_s": nb * ok / (ms / 1e3), "ms_per_step": ms / args.steps,
            "sweeps_per_step": float(np.mean(T["sweeps"])), "steps_at_target": ok,
            "mlp_start_chosen": float(np.mean(chosen)), "weights": os.path.relpath(path, ROOT)}


def ode_f32p():
    import ctypes as C
    return C.POINTER(C.c_float)


def timed_steps(w, stream, flush, steps, graph=False):
    """`steps` fused steps, each bracketed by CUDA events on the world's stream
    (L2 flushed before each, outside the events); per-step statistics."""
    import torch
    out = {k: [] for k in ("step_ms", "solve_ms", "sweeps", "resid", "rows", "contacts", "colours",
                           "interior_rows", "interior_colours", "neighbour_waits", "checks", "cross_classes",
                           "momentum")}
    hist = np.zeros(256, np.float32)
    torch.cuda.nvtx.range_push("timed")
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        if graph:
            w.step_graph()
        else:
            w.step_fused()
        e1.record(stream)
        stream.synchronize()
        st = w.stats()
        out["step_ms"].append(e0.elapsed_time(e1))
        out["solve_ms"].append(st.solve_ms)
        out["sweeps"].append(st.iterations)
        out["resid"].append(st.residual)
        out["rows"].append(st.rows)
        out["contacts"].append(st.contacts)
        out["colours"].append(st.colours)
        out["interior_rows"].append(st.interior_rows)
        out["interior_colours"].append(st.interior_colours)
        out["neighbour_waits"].append(st.neighbour_waits)
        out["cross_classes"].append(st.cross_classes)
        out["momentum"].append(st.momentum)
        out["checks"].append(w.L.gbodeWorldGetResidualHistory(w.w, hist.ctypes.data_as(ode_f32p()), 256))
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    return out


def learned_leg(args, w, L, stream, flush, plain, nb, ws, dev):
    """Learned warm start on the plain leg's timed steps: W untimed steps
    with the network, then the world's snapshot of the plain leg's start
    (bodies and warm-start cache) is restored and the same timed loop runs;
    residual target and counting rules unchanged."""
    import ctypes as C
    from ode_gb300 import learned
    path = args.weights or learned.WEIGHTS
    if not os.path.exists(path):
        return {"unavailable": f"no trained parameters at {os.path.relpath(path, ROOT)}"}
    params = learned.load(path)
    restore_snapshot(L, w)
    if L.gbodeWorldSetLearnedWarmStart(w.w, params.ctypes.data_as(C.POINTER(C.c_float)), 1) != 1:
        return {"unavailable": L.gbodeGetLastError().decode()}
    for _ in range(args.warmup):
        w.step_fused()
    w.sync()
    restore_snapshot(L, w)
    chosen, r_mlp, r_plain = [], [], []
    st = np.zeros(3, np.float32)
    T = {k: [] for k in ("step_ms", "solve_ms", "sweeps", "resid", "rows", "contacts", "colours")}
    for _ in range(args.steps):
        t = timed_steps(w, stream, flush, 1)
        for k in T:
            T[k] += t[k]
        L.gbodeWorldGetLearnedStats(w.w, st.ctypes.data_as(C.POINTER(C.c_float)))
        chosen.append(float(st[0]))
        r_mlp.append(float(st[1]))
        r_plain.append(float(st[2]))
    L.gbodeWorldSetLearnedWarmStart(w.w, None, 0)
    total_ms_max = dist_max(sum(T["step_ms"]), ws, dev)
    ok = sum(1 for r in T["resid"] if r <= args.target)
    value = dist_sum(nb * ok, ws, dev) / (total_ms_max / 1e3)
    plain_ms = sum(plain["step_ms"])
    plain_ok = sum(1 for r in plain["resid"] if r <= args.target)
    plain_value = nb * plain_ok / (plain_ms / 1e3)
    return {"value": value, "unit": "body-steps/s", "ms_per_step": total_ms_max / args.steps,
            "vs_plain": value / plain_value if plain_value > 0 else None,
            "sweeps_per_step": float(np.mean(T["sweeps"])), "plain_sweeps_per_step": float(np.mean(plain["sweeps"])),
            "steps_at_target": ok, "mlp_start_chosen": float(np.mean(chosen)),
            "start_residual_mlp": float(np.median(r_mlp)), "start_residual_plain": float(np.median(r_plain)),
            "weights": os.path.relpath(path, ROOT),
            "note": "the network's start is used only when its residual beats the previous-step start's"}


def rerun_leg(args, w, L, stream, flush, nb, ws, dev, two_level, momentum):
    """The pile's timed steps again with other solver settings (the two-level
    sweep's interior phases, momentum between sweeps; everything else as the
    plain leg): W untimed steps, the snapshot of the plain leg's start
    restored, the same timed loop and counting rules; the plain leg's
    settings are put back afterwards."""
    L.gbodeWorldSetTwoLevelSweep(w.w, two_level)
    L.gbodeWorldSetSweepMomentum(w.w, momentum)
    restore_snapshot(L, w)
    for _ in range(args.warmup):
        w.step_fused()
    w.sync()
    restore_snapshot(L, w)
    T = timed_steps(w, stream, flush, args.steps)
    L.gbodeWorldSetTwoLevelSweep(w.w, args.two_level)
    L.gbodeWorldSetSweepMomentum(w.w, args.momentum)
    total_ms_max = dist_max(sum(T["step_ms"]), ws, dev)
    ok = sum(1 for r in T["resid"] if r <= args.target)
    return {"value": dist_sum(nb * ok, ws, dev) / (total_ms_max / 1e3), "unit": "body-steps/s",
            "ms_per_step": total_ms_max / args.steps, "sweeps_per_step": float(np.mean(T["sweeps"])),
            "steps_at_target": ok}


def cpu_baseline(sc, w, args, threads):
    """The reference algorithm on the host CPU from the GPU-settled state, as
    the reference arm runs it (--ref-sweeps sweeps, stock random reordering,
    no warm start), bounded: --cpu-steps steps with the SOR sweeps on
    `threads` threads, counting only steps whose own FP64 residual reaches
    the target; and the reference's default single-threaded stepping, timed
    on two short steps (100 and 200 sweeps) whose linear fit gives a
    --ref-sweeps step (one thread gives the threaded result to the bit, so the
    residual is the threaded leg's)."""
    from oracle.port.port import Port
    P = Port()
    st = w.state()
    bodies = sc.bodies.copy()
    bodies[:, 0:3], bodies[:, 3:7], bodies[:, 7:10], bodies[:, 10:13] = st[:, 0:3], st[:, 3:7], st[:, 19:22], st[:, 22:25]
    P.lib.port_rand_set_seed(0)
    pw = _port_pile(P, sc, bodies, args.ref_sweeps, threads)
    dt, coll, quick, rel, _ = _port_steps(pw, args.cpu_steps, args.target)
    ok = sum(1 for r in rel if r <= args.target)
    one = {}
    for sweeps in (100, 200):
        w1 = _port_pile(P, sc, bodies, sweeps, 1)
        _, c1, q1, _, _ = _port_steps(w1, 1, args.target)
        one[sweeps] = (c1[0], q1[0])
    per_sweep = (one[200][1] - one[100][1]) / 100.0
    q1500 = one[100][1] + per_sweep * (args.ref_sweeps - 100)
    c1 = 0.5 * (one[100][0] + one[200][0])
    t1 = c1 + q1500
    frac_ok = ok / args.cpu_steps
    return {"value": sc.nb * ok / dt, "unit": "body-steps/s", "cores": threads, "kind": "port",
            "sample": f"{args.cpu_steps} steps of pile{sc.nb} from the GPU-settled state, {args.ref_sweeps} SOR sweeps "
                      f"per step, stock random reordering, no warm start, sweeps on {threads} host threads, "
                      f"{dt:.1f} s; counted steps reach FP64 residual <= {args.target}",
            "steps_at_target": ok, "fp64_residual_max": float(max(rel)),
            "collide_ms_per_step": 1e3 * float(np.mean(coll)), "quickstep_ms_per_step": 1e3 * float(np.mean(quick)),
            "one_thread": {"value": sc.nb * frac_ok / t1, "unit": "body-steps/s", "cores": 1,
                           "collide_ms_per_step": 1e3 * c1, "quickstep_ms_per_step": 1e3 * q1500,
                           "sample": f"one thread (the reference's default stepping): steps of 100 and 200 sweeps "
                                     f"took {one[100][1]:.2f} and {one[200][1]:.2f} s of quickstep; their line "
                                     f"gives {q1500:.1f} s for {args.ref_sweeps} sweeps; steps counted at the "
                                     f"threaded leg's rate of reaching the target"}}


def main():
    args = parse()
    ws, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_gbode(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
