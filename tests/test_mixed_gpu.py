"""Tensor-core many-RHS path (bf_matvec_mixed) against the FP64 path and the oracle.

The mixed path rounds factors and level vectors to complex FP32 and contracts
BF16 hi/lo splits in three passes with FP32 accumulation, so each level adds
a relative error of order 1e-5.  Bar: relative 2-norm error <= 1e-4 against
the FP64-accurate GPU matvec on the same factors (itself pinned to the oracle
at 1e-12), per right-hand side; and the same tolerance-level agreement with
the dense far-field product as the FP64 path.
"""
import math

import numpy as np
import pytest

import bfgpu
from bfgpu import geometry as G
from oracle import bfref as O
from _util import import_oracle, relerr

pytestmark = pytest.mark.gpu
MIXED_TOL = 1e-4


def colerr(Y, R):
    return max(relerr(Y[:, j], R[:, j]) for j in range(Y.shape[1]))


@pytest.fixture(scope="module")
def c1(ctx):
    obs, src = G.plane_pair(4096, seed=1)
    k = 2 * math.pi / 0.125
    to = O.build_tree(obs, max_depth=4)
    ts = O.build_tree(src, max_depth=4)
    kern = O.HelmholtzKernel(obs, src, k)
    bf = O.assemble_bf(kern, to, ts, 0, 0, k, 1e-4, c_tau=4.0, seed=3)
    op = import_oracle([bf], 4096, 4096, to, ts, ctx)
    return dict(bf=bf, op=op, kern=kern)


@pytest.fixture(scope="module")
def sphere(ctx):
    n = 4096
    pts = G.fibonacci_sphere(n)
    k = G.wavenumber(n, 4 * math.pi)
    tr = bfgpu.Tree.build(pts, max_points=32)
    op = bfgpu.PetrovGalerkinBF(pts, pts, tr, tr, k, tol=1e-4, ctx=ctx)
    return dict(op=op, pts=pts, k=k)


@pytest.mark.parametrize("nrhs", [1, 7, 128, 131])
def test_forward_vs_fp64_c1(c1, nrhs):
    X = G.complex_gaussian(4096, 40 + nrhs, nrhs=nrhs)
    ref = c1["op"].matvec(X)
    Y = c1["op"].matvec(X, mixed=True)
    assert Y.shape == ref.shape
    assert colerr(Y.reshape(4096, -1), ref.reshape(4096, -1)) <= MIXED_TOL


def test_adjoint_transpose_vs_fp64_c1(c1):
    X = G.complex_gaussian(4096, 51, nrhs=9)
    for view in (c1["op"].adjoint(), c1["op"].transpose()):
        ref = view.matvec(X)
        Y = view.matvec(X, mixed=True)
        assert colerr(Y, ref) <= MIXED_TOL


def test_alpha_beta_mixed(c1):
    X = G.complex_gaussian(4096, 52, nrhs=3)
    Y0 = G.complex_gaussian(4096, 53, nrhs=3)
    alpha, beta = 0.5 - 2j, 1.5 + 0.25j
    Y = Y0.copy(order="F")
    c1["op"].matvec(X, y=Y, alpha=alpha, beta=beta, mixed=True)
    ref = beta * Y0 + alpha * c1["op"].matvec(X)
    assert colerr(Y, ref) <= MIXED_TOL


def test_mixed_vs_dense_c1(c1):
    """Mixed result within the compression tolerance of the dense product."""
    x = G.complex_gaussian(4096, 54)
    cols = np.arange(4096)
    dense = np.concatenate([c1["kern"](np.arange(r, r + 512), cols) @ x
                            for r in range(0, 4096, 512)])
    y = c1["op"].matvec(x, mixed=True)
    y64 = c1["op"].matvec(x)
    assert relerr(y, dense) < 10 * 1e-4
    assert abs(relerr(y, dense) - relerr(y64, dense)) < 1e-4


def test_sphere_forward_adjoint_vs_fp64(sphere):
    """Full far field of a sphere: many tasks, identity (copy) blocks, several levels."""
    op = sphere["op"]
    n = op.shape[0]
    X = np.concatenate([G.plane_waves(sphere["pts"], sphere["k"], 4, seed=5),
                        G.complex_gaussian(n, 55, nrhs=60)], axis=1)
    X = np.asfortranarray(X)
    for view in (op, op.adjoint(), op.transpose()):
        ref = view.matvec(X)
        Y = view.matvec(X, mixed=True)
        assert colerr(Y, ref) <= MIXED_TOL


def test_device_pointers_mixed(c1):
    torch = pytest.importorskip("torch")
    X = G.complex_gaussian(4096, 56, nrhs=5)
    ref = c1["op"].matvec(X)
    xd = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()   # column j contiguous
    yd = torch.zeros_like(xd)
    stream = torch.cuda.current_stream().cuda_stream
    c1["op"].matvec_device(xd.data_ptr(), 4096, yd.data_ptr(), 4096, nrhs=5, stream=stream,
                           mixed=True)
    torch.cuda.synchronize()
    Y = yd.cpu().numpy().T
    assert colerr(Y, ref) <= MIXED_TOL


def test_profile_and_info(c1):
    info = c1["op"].mixed_info()
    assert info["factor_bytes"] > 0 and info["work_units"] > 0
    ms, by, fl, nk = c1["op"].profile_mixed(nrep=2)
    assert len(ms) == c1["op"].stats()["n_stages"]
    assert (ms > 0).all() and (by > 0).all() and (fl > 0).all() and nk >= len(ms)


def test_invalid_arguments_mixed(c1):
    lib = bfgpu._lib.load()
    rc = lib.bf_matvec_mixed(c1["op"]._h, 7, 1, None, 1, None, 1, None, None, 0, None)
    assert rc == bfgpu._lib.BF_EINVAL
    # nrhs == 0 is a no-op
    rc = lib.bf_matvec_mixed(c1["op"]._h, 0, 0, None, 4096, None, 4096, None, None, 0, None)
    assert rc == bfgpu._lib.BF_OK


def test_rank_zero_operator_is_zero(ctx):
    """With tol >= 1 every compression stops at rank 0 (the first pivot already
    meets pn <= eps*r00): every P task then has no input columns and every Q
    task no rows.  Both paths and both directions must return exact zeros
    (tensor-core work units without input entries issue no MMA)."""
    n = 4096
    pts = G.fibonacci_sphere(n)
    tr = bfgpu.Tree.build(pts, max_points=32)
    op = bfgpu.PetrovGalerkinBF(pts, pts, tr, tr, G.wavenumber(n, 4 * math.pi), tol=10.0,
                                ctx=ctx)
    assert op.stats()["n_bf"] > 0
    X = G.complex_gaussian(n, 61, nrhs=3)
    for view in (op, op.adjoint()):
        assert not np.any(view.matvec(X))
        assert not np.any(view.matvec(X, mixed=True))
