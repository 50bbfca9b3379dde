"""One GPU compression against one call of the oracle's PartialQR on identical rows.

``bf_compress_block`` runs the device launches of the build (row sampling,
Helmholtz kernel sampling, pivoted partial QR, interpolation solve) for one
compression; ``oracle.bfref.partial_qr`` restates the reference compressor
(src/ButterflyFactorization/compressors.jl:81-165) in FP64 with LAPACK's
pivoted QR standing in for LowRankApprox.pqr.  Both sample their rows with the
same keyed bijection, so the comparison is on identical inputs:

* sampled rows: bit-identical;
* kernel entries G(r) = exp(-ikr)/(4 pi r): within 2e-6 relative, entry by
  entry, against FP64 -- including k = 228 (the 524,288-point ellipsoid) with
  k*r up to ~450, where an FP32 phase would be off by ~3e-5;
* rank: equal, unless the oracle's R diagonal sits within 1% of the cut;
* skeleton: equal pivots for every step whose two leading residual column
  norms differ by more than 2e-5 (relative) in FP64; a nearer tie may go
  either way, since the GPU sees the FP32-rounded kernel block;
* T: with equal skeletons, Z[:, skel] T agrees with the oracle's to 1e-5 of
  |Z|, and either interpolation reproduces Z to the compression tolerance.
"""
import math

import numpy as np
import pytest
from scipy.linalg import qr as sp_qr

import bfgpu
from bfgpu import geometry as G
from oracle import bfref as O

pytestmark = pytest.mark.gpu


def pivot_gaps(Z, r):
    """FP64 column-pivoted Gram-Schmidt: the relative gap between the two largest
    residual column norms at each of the first r steps."""
    A = np.array(Z, np.complex128)
    m = A.shape[1]
    Q = np.zeros((A.shape[0], 0), np.complex128)
    left = list(range(m))
    gaps = []
    for _ in range(r):
        R = A[:, left] - Q @ (Q.conj().T @ A[:, left])
        nr = np.linalg.norm(R, axis=0)
        order = np.argsort(-nr, kind="stable")
        n1 = nr[order[0]]
        n2 = nr[order[1]] if len(order) > 1 else 0.0
        gaps.append((n1 - n2) / n1 if n1 > 0 else 0.0)
        j = order[0]
        q = R[:, j] / n1
        Q = np.concatenate([Q, q[:, None]], axis=1)
        left.pop(j)
    return np.array(gaps)


def compare(obs, src, obs_index, src_index, n_rows, k, eps, key, ctx):
    kern = O.HelmholtzKernel(obs, src, k)
    g = bfgpu.compress_block(obs, src, obs_index, src_index, n_rows, key, k, eps, ctx)
    rows = np.asarray(obs_index)[O.sample_positions(0, n_rows, len(obs_index), key)]
    assert np.array_equal(g["rows"], rows)
    Zd = kern(rows, src_index)
    rel = np.abs(g["Z"] - Zd) / np.abs(Zd)
    assert rel.max() <= 2e-6, rel.max()
    T, skel, r = O.partial_qr(kern, src_index, obs_index, n_rows, eps, adaptive=False, key=key,
                              min_samples=1)
    # where the oracle's diagonal sits relative to the cut
    _, Rf, _ = sp_qr(Zd, mode="economic", pivoting=True)
    d = np.abs(np.diag(Rf))
    near_cut = np.any(np.abs(d / (eps * d[0]) - 1.0) < 0.01)
    if not near_cut:
        assert g["rank"] == r, (g["rank"], r)
    else:
        assert abs(g["rank"] - r) <= 1
    rr = min(g["rank"], r)
    gaps = pivot_gaps(Zd, rr)
    sep = int(np.argmax(gaps < 2e-5)) if np.any(gaps < 2e-5) else rr
    assert np.array_equal(g["skeleton"][:sep], skel[:sep]), (sep, g["skeleton"][:sep], skel[:sep])
    zn = np.linalg.norm(Zd)
    pos = {int(s): i for i, s in enumerate(src_index)}
    gsk = [pos[int(s)] for s in g["skeleton"]]
    err_gpu = np.linalg.norm(Zd - Zd[:, gsk] @ g["T"]) / zn
    assert err_gpu <= 10 * eps, err_gpu
    if g["rank"] == r and sep == r:
        osk = [pos[int(s)] for s in skel]
        assert osk == gsk
        diff = np.linalg.norm(Zd[:, osk] @ (g["T"] - T)) / zn
        assert diff <= 1e-5, diff
    return dict(rank=g["rank"], oracle_rank=r, sep=sep)


def test_q_stage_compression_plane_pair(ctx):
    """A source leaf against all observers of the 4,096-point plane pair (k = 16 pi)."""
    obs, src = G.plane_pair(4096, seed=1)
    k = 2 * math.pi / 0.125
    ts = O.build_tree(src, max_depth=4)
    leaves = [i for i in range(ts.n_nodes) if ts.isleaf(i)]
    eps = 1e-4 / 5
    n_est = O.estimate_rank_butterfly(eps, 4.0)
    full = 0
    for q, leaf in enumerate(leaves[:12]):
        out = compare(obs, src, np.arange(4096), ts.values(leaf), n_est, k, eps,
                      O.task_key(3, 0, 0, 0, leaf), ctx)
        full += out["sep"] == out["rank"]
    assert full >= 6  # most compressions have well separated pivots throughout


@pytest.mark.parametrize("n_rows", [24, 64])
def test_wide_compressions_plane_pair(ctx, n_rows):
    """Sampled rows against a few hundred columns (an R-stage shape)."""
    obs, src = G.plane_pair(4096, seed=2)
    k = 2 * math.pi / 0.125
    to = O.build_tree(obs, max_depth=4)
    ts = O.build_tree(src, max_depth=4)
    lvl = [i for i in range(ts.n_nodes) if ts.level[i] == 2][:3]
    olvl = [i for i in range(to.n_nodes) if to.level[i] == 2][:2]
    for s in lvl:
        for o in olvl:
            compare(obs, src, to.values(o), ts.values(s), n_rows, k, 2e-5,
                    O.task_key(5, 1, 2, o, s), ctx)


def test_high_wavenumber_sampling(ctx):
    """k = 228 (the 524,288-point ellipsoid at ~100 points per wavelength^2) between two
    clusters ~2 apart: k*r reaches ~450, where the FP64 range reduction matters."""
    rng = np.random.default_rng(9)
    src = rng.uniform(-0.02, 0.02, (300, 3))
    obs = rng.uniform(-0.05, 0.05, (3000, 3)) + np.array([1.97, 0.0, 0.0])
    k = 228.3
    d = np.linalg.norm(obs[:, None, :] - src[None, :, :], axis=2)
    assert k * d.max() > 440
    out = compare(obs, src, np.arange(3000), np.arange(300), 120, k, 2e-5, 1234567, ctx)
    assert 5 <= out["rank"] < 120
