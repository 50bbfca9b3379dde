"""GPU kernels of the rank surrogate against the CPU oracle, and what the trained
network gains in construction.

Bars: gradient (bf_surrogate_grad) within 1e-4 (2-norm, relative) of the
oracle's FP32 gradient with the same BF16 rounding; predictions within 1e-4;
three full-batch Adam steps on the GPU match the oracle's Adam within 1e-4;
training lowers the loss tenfold on a smooth synthetic target.  Then the
network trained on rank records of two builds seeds the construction of a
held-out geometry: fewer sampled kernel entries than the oversampling
estimator at the same accuracy against dense far-field rows.
"""
import math

import numpy as np
import pytest

import bfgpu
from bfgpu import geometry as G
from bfgpu.surrogate import RankSurrogate, features_targets
from bfgpu.verify import far_dense_rows, sample_rows
from oracle import surrogate as S

pytestmark = pytest.mark.gpu


def _data(n, seed=0):
    rng = np.random.default_rng(seed)
    F = np.stack([rng.integers(0, 6, n), rng.uniform(1, 60, n), rng.uniform(1, 4, n),
                  np.log1p(rng.integers(8, 4000, n))], axis=1).astype(np.float32)
    T = np.log(5 + 0.3 * F[:, 1] + 2 * F[:, 0]).astype(np.float32)
    return F, T


def rel(a, b):
    a = np.asarray(a)
    return float(np.linalg.norm(a.astype(np.result_type(a, np.float64)) - b) / np.linalg.norm(b))


def test_gradient_and_prediction_match_oracle(ctx):
    F, T = _data(1000)
    model = RankSurrogate.init(F, seed=4)
    w = model.weights.copy()
    w[8:] += 0.05 * np.random.default_rng(5).standard_normal(S.NW - 8).astype(np.float32)
    model = RankSurrogate(w)
    loss, g = model.loss_and_grad(F, T, ctx)
    lref, gref = S.loss_and_grad(w, F, T, round_bf16=True, dtype=np.float32)
    assert abs(loss - lref) <= 1e-5 * abs(lref)
    assert rel(g, gref) <= 1e-4
    yref, _ = S.forward(w, F)
    assert np.max(np.abs(model.predict(F, ctx) - yref)) <= 1e-4


def test_adam_steps_match_oracle(ctx):
    F, T = _data(512, seed=6)
    m0 = RankSurrogate.init(F, seed=7)
    trained, hist = RankSurrogate.train(F, T, ctx, epochs=3, batch=512, lr=1e-3, init=m0)
    w = m0.weights.copy()
    m, v = np.zeros_like(w), np.zeros_like(w)
    for t in range(1, 4):
        _, g = S.loss_and_grad(w, F, T)
        S.adam_step(w, g, m, v, t, lr=1e-3)
    assert rel(trained.weights, w) <= 1e-4
    assert len(hist) == 3


def test_training_lowers_loss(ctx):
    F, T = _data(20000, seed=8)
    model, hist = RankSurrogate.train(F, T, ctx, epochs=20, batch=1024, lr=3e-3, seed=1)
    assert hist[-1] < 0.1 * hist[0]
    assert np.sqrt(2 * hist[-1]) < 0.05  # RMS log-rank error under 5%


def _build(pts, tree, k, surrogate=None, ctx=None):
    return bfgpu.PetrovGalerkinBF(pts, pts, tree, tree, k, tol=1e-4, ctx=ctx,
                                  rank_mode=1 if surrogate is not None else 0,
                                  surrogate=surrogate)


def test_surrogate_seeded_build_gains(ctx):
    # training records: two geometries at ~100 points per wavelength^2
    recs = []
    for shape, n in (("sphere", 8192), ("cube", 8192)):
        pts, area = G.shape_points(shape, n, seed=1)
        k = G.wavenumber(n, area)
        tr = bfgpu.Tree.build(pts, max_points=32)
        recs.append(_build(pts, tr, k, ctx=ctx).rank_log())
    F, T = features_targets(np.concatenate(recs))
    model, hist = RankSurrogate.train(F, T, ctx, epochs=25, batch=2048, lr=3e-3, seed=2)
    model.calibrate_margin(F, T, ctx, quantile=0.98)
    # held-out geometry: ellipsoid with semi-axes 1, 0.5, 0.25
    n = 16384
    pts, area = G.shape_points("ellipsoid", n, seed=3)
    k = G.wavenumber(n, area)
    tr = bfgpu.Tree.build(pts, max_points=32)
    plain = _build(pts, tr, k, ctx=ctx)
    seeded = _build(pts, tr, k, surrogate=model, ctx=ctx)
    sp, ss = plain.stats(), seeded.stats()
    # same compressions, fewer sampled kernel entries, few fallbacks
    assert ss["compressions"] == sp["compressions"]
    assert ss["kernel_entries"] < 0.9 * sp["kernel_entries"]
    assert ss["surrogate_fallbacks"] <= 0.01 * ss["compressions"]
    # same accuracy against dense far-field rows
    far, _ = bfgpu.nearandfar(tr, tr, 1.0)
    rows = sample_rows(n, 96, seed=9)
    x = G.complex_gaussian(n, 10)
    ref = far_dense_rows(pts, pts, tr, tr, far, k, rows, x)[:, 0]
    ep = rel((plain @ x)[rows], ref)
    es = rel((seeded @ x)[rows], ref)
    print(f"\nplain: entries {sp['kernel_entries']} retries {sp['retries']} "
          f"build {sp['build_seconds']:.2f}s err {ep:.2e}; surrogate: entries "
          f"{ss['kernel_entries']} retries {ss['retries']} fallbacks "
          f"{ss['surrogate_fallbacks']} build {ss['build_seconds']:.2f}s err {es:.2e}; "
          f"margin {model.margin:.3f} final loss {hist[-1]:.4f}")
    assert es < 10 * 1e-4 and es < 2.0 * ep + 1e-5
