"""Sampled dense far-field rows in FP64 (NumPy, host): the accuracy yardstick.

For observer point i the far field is the sum, over every far pair (O, S)
with i in O, of G(x_i, y_j) x_j for the points j of S (the sum the
butterflies approximate, src/matrixalgebra/matrixvector.jl:8-65 without the
near part).  ``far_dense_rows`` evaluates that sum directly for a seeded
sample of rows and any number of right-hand sides, with the point Helmholtz
kernel G(r) = exp(-i k r) / (4 pi r).
"""
from __future__ import annotations

import numpy as np


def _parents(tree) -> np.ndarray:
    par = np.full(tree.n_nodes, -1, np.int64)
    for v in range(tree.n_nodes):
        for c in tree.children(v):
            par[c] = v
    return par


def far_dense_rows(obs: np.ndarray, src: np.ndarray, tree_o, tree_s, far: np.ndarray, k: float,
                   rows: np.ndarray, X: np.ndarray, chunk: int = 128) -> np.ndarray:
    """Rows ``rows`` of (far-field operator) @ X, FP64, shape (len(rows), nrhs)."""
    X = np.asarray(X, np.complex128)
    if X.ndim == 1:
        X = X[:, None]
    ptr_o, idx_o = tree_o.values_csr()
    ptr_s, idx_s = tree_s.values_csr()
    par = _parents(tree_o)
    # point -> deepest observer node holding it (a leaf)
    leaf_of = np.full(len(obs), -1, np.int64)
    for v in range(tree_o.n_nodes):
        if tree_o.isleaf(v):
            leaf_of[idx_o[ptr_o[v]:ptr_o[v + 1]]] = v
    by_obs: dict[int, list[int]] = {}
    for o, s in far:
        by_obs.setdefault(int(o), []).append(int(s))
    rows = np.asarray(rows, np.int64)
    out = np.zeros((len(rows), X.shape[1]), np.complex128)
    for c0 in range(0, len(rows), chunk):
        rr = rows[c0:c0 + chunk]
        D = np.zeros((len(rr), len(src)), np.complex128)
        for q, i in enumerate(rr):
            mask = np.zeros(len(src), bool)
            v = leaf_of[i]
            while v >= 0:
                for s in by_obs.get(int(v), ()):
                    mask[idx_s[ptr_s[s]:ptr_s[s + 1]]] = True
                v = par[v]
            cols = np.nonzero(mask)[0]
            if len(cols) == 0:
                continue
            d = src[cols] - obs[i]
            r = np.sqrt(np.einsum("ij,ij->i", d, d))
            D[q, cols] = np.exp(-1j * k * r) / (4.0 * np.pi * r)
        out[c0:c0 + len(rr)] = D @ X
    return out


def sample_rows(n: int, count: int, seed: int) -> np.ndarray:
    """Seeded sample of distinct row indices."""
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=min(count, n), replace=False))
