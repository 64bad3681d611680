"""Learned warm start: data collection, training and evaluation drivers over
the C ABI (gbodeWorldSetLearnCapture / gbodeWorldGetLearnSamples,
gbodeMlpTrain, gbodeWorldSetLearnedWarmStart).

The network predicts each contact's three starting multipliers (normal and
two friction rows) in units of the contact's weight scale s = m_eff * |g|
from twelve local features (see include/gbode.h).  Training targets are the
multipliers the plain coloured solver converges to (LCP residual 1e-6,
started from the previous step's multipliers) on seeded scenes: box stacks,
8,192-body piles and a 32,768-body pile (seeds other than the benchmark's).
Training runs on the GPU with the library's own kernels: 96 epochs of Adam
at learning rate 3e-4, batches of 1,024.

    python -m ode_gb300.learned train   # writes ode_gb300/data/warmstart_mlp.npz
"""
from __future__ import annotations

import argparse
import ctypes
import os
import time

import numpy as np

from . import ode, scenes, sim

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "data", "warmstart_mlp.npz")
NI, NH, NO = 12, 128, 3
_F = ctypes.POINTER(ctypes.c_float)


def _fp(a):
    return a.ctypes.data_as(_F)


def collect_world(w: sim.GBWorld, steps: int, iterations: int = 200, target: float = 0.0):
    """Step `w` (fused path) `steps` times with `iterations` plain sweeps per
    step (or, with `target` > 0, sweeps until the LCP residual reaches it, at
    most 5000), previous-step warm start and feature capture on; returns X
    [n][12] raw features and Y [n][3] final multipliers / s of the triplet
    contacts."""
    L = w.L
    L.gbodeWorldSetLearnCapture(w.w, 1)
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    if target > 0:
        L.gbodeWorldSetResidualTarget(w.w, target, 10, 5000)
    else:
        L.gbodeWorldSetResidualTarget(w.w, 0.0, 10, 0)
        L.dWorldSetQuickStepNumIterations(w.w, iterations)
    xs, ys = [], []
    buf = np.zeros((0, 17), np.float32)
    for _ in range(steps):
        w.step_fused()
        n = L.gbodeWorldGetLearnSamples(w.w, None, 0)
        if n > len(buf):
            buf = np.zeros((n, 17), np.float32)
        n = L.gbodeWorldGetLearnSamples(w.w, _fp(buf), len(buf))
        s = buf[:n]
        ok = (s[:, 16] == 1) & (s[:, 12] > 0) & np.isfinite(s).all(axis=1)
        xs.append(s[ok, :12].copy())
        ys.append(s[ok, 13:16] / s[ok, 12:13])
    L.gbodeWorldSetLearnCapture(w.w, 0)
    return np.concatenate(xs), np.concatenate(ys).astype(np.float32)


def init_params(seed: int, mean, std):
    rng = np.random.default_rng(seed)
    parts = [np.asarray(mean, np.float64), np.asarray(std, np.float64)]
    for fan_in, fan_out in ((NI, NH), (NH, NH), (NH, NH), (NH, NO)):
        lim = np.sqrt(6.0 / fan_in) * (0.5 if fan_out == NO else 1.0)
        parts += [rng.uniform(-lim, lim, fan_in * fan_out), np.zeros(fan_out)]
    return np.concatenate(parts).astype(np.float32)


def fit(X, Y, epochs: int = 4, batch: int = 1024, lr: float = 1e-3, seed: int = 0, losses: list | None = None):
    """Standardise on X, initialise, train on the GPU; returns the parameters."""
    L = ode.load()
    X = np.ascontiguousarray(X, np.float32)
    Y = np.ascontiguousarray(Y, np.float32)
    mean = X.mean(axis=0)
    std = np.maximum(X.std(axis=0), 1e-3)
    p = init_params(seed, mean, std)
    lp = np.zeros(epochs, np.float32)
    if L.gbodeMlpTrain(_fp(X), _fp(Y), len(X), epochs, batch, lr, seed, _fp(p), _fp(lp)) != 1:
        raise RuntimeError(L.gbodeGetLastError().decode())
    if losses is not None:
        losses.extend(float(v) for v in lp)
    return p


def training_scenes():
    """Seeded training scenes: piles of the benchmark's mix (held-out seeds
    >= 100 for training; the benchmark pile uses seed 1) and box stacks."""
    return [("pile", 8192, s) for s in (101, 102, 103, 104)] + [("box_stack", 10, s) for s in range(100, 116)]


def collect(settle: int = 600, steps: int = 40, target: float = 0.0, big: bool = False, log=print):
    xs, ys = [], []
    scenes_ = training_scenes() + ([("pile", 32768, 102)] if big else [])
    for kind, n, seed in scenes_:
        t0 = time.time()
        sc = scenes.pile(n, seed=seed) if kind == "pile" else scenes.box_stack(seed=seed)
        w = sim.GBWorld(sc)
        w.L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
        w.L.dWorldSetQuickStepW(w.w, 1.0)
        for _ in range(settle if kind == "pile" else 100):
            w.step_fused()
        X, Y = collect_world(w, steps, target=target)
        w.close()
        xs.append(X)
        ys.append(Y)
        log(f"{kind}{n} seed {seed}: {len(X)} contacts ({3 * len(X)} rows) in {time.time() - t0:.1f} s")
    return np.concatenate(xs), np.concatenate(ys)


def save(path: str, params, meta: dict):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez_compressed(path, params=np.asarray(params, np.float32), **{k: np.asarray(v) for k, v in meta.items()})


def load(path: str = WEIGHTS):
    """The trained parameters (float32 [GBODE_MLP_NPARAMS])."""
    with np.load(path) as z:
        p = z["params"].astype(np.float32)
    if p.size != ode.GBODE_MLP_NPARAMS:
        raise ValueError(f"{path}: {p.size} parameters, expected {ode.GBODE_MLP_NPARAMS}")
    return p


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--out", default=WEIGHTS)
    t.add_argument("--epochs", type=int, default=96)
    t.add_argument("--steps", type=int, default=40)
    t.add_argument("--target", type=float, default=1e-6,
                   help="targets from solves to this LCP residual (0: 200 sweeps)")
    t.add_argument("--small", action="store_true", help="leave out the 32,768-body pile (seed 102)")
    t.add_argument("--data", default=None, help="samples (.npy pair prefix): reused if present, else written")
    t.add_argument("--lr", type=float, default=3e-4)
    args = ap.parse_args(argv)
    if args.cmd == "train":
        t0 = time.time()
        if args.data and os.path.exists(args.data + "_X.npy"):
            X, Y = np.load(args.data + "_X.npy"), np.load(args.data + "_Y.npy")
        else:
            X, Y = collect(steps=args.steps, target=args.target, big=not args.small)
            if args.data:
                np.save(args.data + "_X.npy", X)
                np.save(args.data + "_Y.npy", Y)
        print(f"{len(X)} samples ({3 * len(X)} rows) collected in {time.time() - t0:.0f} s")
        t1 = time.time()
        losses = []
        p = fit(X, Y, epochs=args.epochs, lr=args.lr, losses=losses)
        print(f"trained in {time.time() - t1:.0f} s; loss per epoch {losses}")
        save(args.out, p, {"samples": len(X), "epochs": args.epochs, "loss": np.asarray(losses),
                           "target": args.target, "big": int(not args.small), "lr": args.lr})
        print("wrote", args.out)


if __name__ == "__main__":
    main()
