"""Learned rank surrogate: records -> training on the GPU -> surrogate-seeded builds.

The rank records that every build logs (``Operator.rank_log``, columns 14-17
are the features, column 9 the final rank) train a 4 -> 64 -> 64 -> 1 MLP
on the GPU (``bf_surrogate_train``: the library's own forward, backward and
Adam kernels).  ``PetrovGalerkinBF(..., rank_mode=1, surrogate=model)`` then
asks the network for each compression's rank and samples
ceil(exp(pred + margin) / 0.8) + 2 rows, so the partial QR rarely needs the
adaptive doubling of src/ButterflyFactorization/compressors.jl:134-151; a
compression whose rank still exceeds 0.8 x rows falls back to the oversampling
estimator (rankestimation.jl:93-98) and is counted in
``stats()["surrogate_fallbacks"]``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import SUR_NW, TrainOpts, check, load

RANK_COL, FEAT_COLS = 9, slice(14, 18)


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def features_targets(records: np.ndarray):
    """(features n x 4 float32, targets = log(max(rank, 1)) float32) of rank records."""
    rec = np.asarray(records, np.float64)
    F = np.ascontiguousarray(rec[:, FEAT_COLS], np.float32)
    T = np.ascontiguousarray(np.log(np.maximum(rec[:, RANK_COL], 1.0)), np.float32)
    return F, T


class RankSurrogate:
    """A trained weight vector plus the sampling margin used by the builder."""

    def __init__(self, weights, margin: float = 0.15):
        w = np.ascontiguousarray(weights, np.float32)
        if w.size != SUR_NW:
            raise ValueError(f"surrogate needs {SUR_NW} weights, got {w.size}")
        self.weights = w
        self.margin = float(margin)

    @classmethod
    def init(cls, F, seed: int = 0):
        F = np.ascontiguousarray(F, np.float32)
        w = np.zeros(SUR_NW, np.float32)
        check(load().bf_surrogate_init(_fp(F), F.shape[0], int(seed), _fp(w)),
              "bf_surrogate_init")
        return cls(w)

    @classmethod
    def train(cls, F, T, ctx, epochs: int = 30, batch: int = 4096, lr: float = 3e-3,
              seed: int = 0, init=None):
        """Adam on the GPU; returns (model, mean batch loss per epoch)."""
        F = np.ascontiguousarray(F, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        model = init if init is not None else cls.init(F, seed)
        w = model.weights.copy()
        o = TrainOpts()
        load().bf_train_opts_default(C.byref(o))
        o.epochs, o.batch, o.lr, o.seed = int(epochs), int(batch), float(lr), int(seed)
        hist = np.zeros(max(int(epochs), 1), np.float32)
        check(load().bf_surrogate_train(ctx._h, _fp(F), _fp(T), F.shape[0], C.byref(o), _fp(w),
                                        _fp(hist)), "bf_surrogate_train")
        return cls(w, model.margin), hist[:int(epochs)]

    def predict(self, F, ctx) -> np.ndarray:
        F = np.ascontiguousarray(F, np.float32)
        out = np.zeros(F.shape[0], np.float32)
        check(load().bf_surrogate_predict(ctx._h, _fp(self.weights), _fp(F), F.shape[0],
                                          _fp(out)), "bf_surrogate_predict")
        return out

    def loss_and_grad(self, F, T, ctx):
        F = np.ascontiguousarray(F, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        g = np.zeros(SUR_NW, np.float32)
        loss = np.zeros(1, np.float32)
        check(load().bf_surrogate_grad(ctx._h, _fp(self.weights), _fp(F), _fp(T), F.shape[0],
                                       _fp(g), _fp(loss)), "bf_surrogate_grad")
        return float(loss[0]), g

    def calibrate_margin(self, F, T, ctx, quantile: float = 0.98) -> float:
        """Margin = the quantile of the log-rank under-prediction on (F, T)."""
        r = np.asarray(T, np.float64) - self.predict(F, ctx)
        self.margin = float(max(0.0, np.quantile(r, quantile)))
        return self.margin
