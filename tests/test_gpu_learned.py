"""Learned warm start on the GPU, through the C ABI: the training kernels'
loss and gradient against the FP64 oracle (oracle/mlp_ref.py), the
tensor-core inference kernel against the oracle's forward pass, training
progress, and the residual-judged start inside dWorldQuickStep.

Tolerances: gradient entries within 2e-3 of the largest gradient magnitude
of their parameter block plus 1e-3 relative (FP32 kernels, atomics in any
order); inference outputs within 3e-2 x (1 + |y|) (BF16 weights and
activations, FP32 accumulation).
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu

F = ctypes.POINTER(ctypes.c_float)


def fp(a):
    return np.ascontiguousarray(a, np.float32).ctypes.data_as(F)


def _data(seed, n):
    rng = np.random.default_rng(seed)
    mean = rng.normal(size=12)
    std = rng.uniform(0.5, 2.0, 12)
    X = (mean + std * rng.normal(size=(n, 12))).astype(np.float32)
    Y = rng.normal(size=(n, 3)).astype(np.float32)
    p = mlp_ref.init_params(seed, mean=mean, std=std)
    return p, X, Y


def _blocks():
    NI, NH, NO = 12, 128, 3
    sizes = [NH * NI, NH, NH * NH, NH, NH * NH, NH, NO * NH, NO]
    o = 2 * NI
    for s in sizes:
        yield slice(o, o + s)
        o += s


def test_loss_and_gradient_match_oracle(gblib):
    L = gblib
    p, X, Y = _data(5, 333)  # not a multiple of the 32-row blocks
    grad = np.zeros(mlp_ref.NPARAMS, np.float32)
    loss = np.zeros(1, np.float32)
    assert L.gbodeMlpLossGrad(fp(p), fp(X), fp(Y), len(X), grad.ctypes.data_as(F), loss.ctypes.data_as(F)) == 1
    ref_loss, ref_grad = mlp_ref.loss_grad(p, X, Y)
    assert abs(loss[0] - ref_loss) <= 1e-4 * (1 + ref_loss), (loss[0], ref_loss)
    assert np.all(grad[:24] == 0)
    worst = 0.0
    for sl in _blocks():
        g, r = grad[sl].astype(np.float64), ref_grad[sl]
        err = np.abs(g - r)
        bound = 2e-3 * np.abs(r).max() + 1e-3 * np.abs(r)
        worst = max(worst, float((err / (np.abs(r).max() + 1e-30)).max()))
        assert np.all(err <= bound + 1e-9), (sl, float(err.max()), float(np.abs(r).max()))
    print(f"gradient vs FP64 oracle: worst error {worst:.2e} of the block's largest entry")


def test_tensor_core_inference_matches_oracle(gblib):
    L = gblib
    p, X, _ = _data(7, 1000)  # not a multiple of the 128-row tiles
    Y = np.zeros((len(X), 3), np.float32)
    assert L.gbodeMlpPredict(fp(p), fp(X), len(X), Y.ctypes.data_as(F)) == 1, L.gbodeGetLastError()
    ref = mlp_ref.forward(p, X)
    err = np.abs(Y - ref)
    print(f"tcgen05 BF16 inference vs FP64: max abs error {err.max():.3g}, output scale {np.abs(ref).max():.3g}")
    assert np.all(err <= 3e-2 * (1 + np.abs(ref)))
    # a second call gives the same result (no state carried between launches)
    Y2 = np.zeros_like(Y)
    assert L.gbodeMlpPredict(fp(p), fp(X), len(X), Y2.ctypes.data_as(F)) == 1
    assert np.array_equal(Y, Y2)


def test_training_reduces_loss(gblib):
    L = gblib
    rng = np.random.default_rng(11)
    X = rng.normal(size=(20000, 12)).astype(np.float32)
    Y = np.stack([np.tanh(X[:, 0] + 0.5 * X[:, 1]), X[:, 2] * X[:, 3] * 0.3, np.sin(X[:, 4])], 1).astype(np.float32)
    p = mlp_ref.init_params(2)
    l0, _ = mlp_ref.loss_grad(p, X[:2000], Y[:2000])
    losses = np.zeros(4, np.float32)
    assert L.gbodeMlpTrain(fp(X), fp(Y), len(X), 4, 256, 2e-3, 1, p.ctypes.data_as(F), losses.ctypes.data_as(F)) == 1
    l1, _ = mlp_ref.loss_grad(p, X[:2000], Y[:2000])
    print(f"training: loss {l0:.4f} -> {l1:.4f}; per epoch {losses}")
    assert l1 < 0.2 * l0 and losses[-1] < losses[0]


def test_learned_start_is_residual_judged(gblib):
    """A pile steps with the learned start enabled: the start chosen each
    step has a residual no higher than the plain start's, and every step
    reaches the residual target."""
    from ode_gb300 import learned, scenes, sim
    L = gblib
    sc = scenes.pile(2048, seed=7)
    w = sim.GBWorld(sc)
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    L.dWorldSetQuickStepW(w.w, 1.0)
    for _ in range(300):
        w.step_fused()
    X, Y = learned.collect_world(w, steps=20)
    assert len(X) > 1000
    params = learned.fit(X, Y, epochs=3, seed=0)
    assert L.gbodeWorldSetLearnedWarmStart(w.w, fp(params), 1) == 1
    L.gbodeWorldSetResidualTarget(w.w, 1e-4, 5, 3000)
    st = np.zeros(3, np.float32)
    used = 0
    for _ in range(5):
        w.step_fused()
        w.sync()
        L.gbodeWorldGetLearnedStats(w.w, st.ctypes.data_as(F))
        assert st[1] > 0 and st[2] > 0
        if st[0] == 1:
            assert st[1] < st[2]
            used += 1
        else:
            assert st[2] <= st[1]
        assert w.stats().residual <= 1e-4
    print(f"learned start chosen in {used} of 5 steps; last residuals mlp {st[1]:.3g} plain {st[2]:.3g}")
    w.close()


# measured on the held-out pile below (one GB300): plain 380.2 mean sweeps to
# the target, learned 337.0 (11.4 % fewer; the network's start chosen in every
# step); the test asks for at least GAIN_MIN
GAIN_MIN = 0.05
GAIN_MIN_MOMENTUM = 0.02  # with momentum 0.8 (measured 4.4 %: 117.5 -> 112.3 sweeps)


@pytest.mark.parametrize("momentum,gain_min", [(0.0, GAIN_MIN), (0.8, GAIN_MIN_MOMENTUM)])
def test_committed_network_gains_on_a_held_out_pile(gblib, momentum, gain_min):
    """What the trained network (ode_gb300/data/warmstart_mlp.npz) gains over
    the method without it: an 8,192-body pile of a seed no training scene
    used (7; training used 101-104, 102 and box stacks 100-115; the benchmark
    seed 1), settled, saved (gbodeWorldSaveSnapshot); 12 steps to LCP residual
    1e-4 with the plain previous-step start, the snapshot restored, the same
    12 steps with the learned start (the plain start stays the fallback each
    step).  Every step reaches the target either way; the learned start cuts
    the mean sweeps by at least GAIN_MIN -- and by GAIN_MIN_MOMENTUM with
    momentum 0.8 between sweeps (gbodeWorldSetSweepMomentum) on both runs."""
    from ode_gb300 import learned, scenes, sim
    L = gblib
    sc = scenes.pile(8192, seed=7)
    w = sim.GBWorld(sc)
    L.gbodeWorldSetWarmStart(w.w, 1, 1.0)
    L.dWorldSetQuickStepW(w.w, 1.0)
    L.gbodeWorldSetTwoLevelSweep(w.w, 2)
    L.dWorldSetQuickStepNumIterations(w.w, 30)
    for _ in range(600):
        w.step_fused()
    L.gbodeWorldSetResidualTarget(w.w, 1e-4, 5, 3000)
    L.gbodeWorldSetSweepMomentum(w.w, momentum)
    for _ in range(3):
        w.step_fused()
    w.sync()
    assert L.gbodeWorldSaveSnapshot(w.w) == 1, L.gbodeGetLastError()
    params = learned.load()
    sweeps = {}
    chosen = []
    st = np.zeros(3, np.float32)
    for mode in ("plain", "learned"):
        assert L.gbodeWorldRestoreSnapshot(w.w) == 1
        if mode == "learned":
            assert L.gbodeWorldSetLearnedWarmStart(w.w, fp(params), 1) == 1
        sweeps[mode] = []
        for _ in range(12):
            w.step_fused()
            w.sync()
            s = w.stats()
            assert s.residual <= 1e-4
            sweeps[mode].append(s.iterations)
            if mode == "learned":
                L.gbodeWorldGetLearnedStats(w.w, st.ctypes.data_as(F))
                chosen.append(float(st[0]))
    L.gbodeWorldSetLearnedWarmStart(w.w, None, 0)
    p, q = float(np.mean(sweeps["plain"])), float(np.mean(sweeps["learned"]))
    gain = 1.0 - q / p
    print(f"held-out pile8192, momentum {momentum}: mean sweeps to 1e-4 plain {p:.1f}, learned {q:.1f} (gain {gain:.1%}, "
          f"network's start chosen in {np.mean(chosen):.0%} of the steps)")
    assert gain >= gain_min, (p, q)
    w.close()
