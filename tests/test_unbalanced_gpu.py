"""PetrovGalerkinBF with unbalancedints (src/Matrixassembly/intlists.jl:121-149):
the traversal splits only the larger node of a pair, so far pairs join nodes of
different levels.  The GPU build of those butterflies must meet the reference's
acceptance criterion (< 10 tol against dense products, test_subroutines.jl:
174-182), with the GPU lists equal to the host ones and, with the near field
attached, the whole product against dense kernel rows."""
import math

import numpy as np
import pytest

import bfgpu
from bfgpu import geometry as G
from bfgpu.verify import far_dense_rows, sample_rows
from _util import relerr

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.mark.parametrize("case", ["sphere", "planes"])
def test_unbalanced_far_field_against_dense_rows(ctx, case):
    if case == "sphere":
        n = 8000
        obs = src = G.fibonacci_sphere(n)
        k = G.wavenumber(n, 4 * math.pi)
        to = ts = bfgpu.Tree.build(obs, max_points=32)
    else:
        obs, src = G.plane_pair(4000, 7, z_obs=0.5)
        n = 4000
        k = 2 * math.pi / 0.125
        to, ts = bfgpu.Tree.build(obs, max_points=12), bfgpu.Tree.build(src, max_points=60)
    far, _ = bfgpu.nearandfar(to, ts, 1.0, unbalancedints=True)
    lv = to.level[far[:, 0]] - ts.level[far[:, 1]]
    assert np.any(lv != 0)  # pairs of different levels
    far_d, _ = bfgpu.nearandfar_gpu(to, ts, 1.0, unbalancedints=True, ctx=ctx)
    assert np.array_equal(far, far_d)
    op = bfgpu.PetrovGalerkinBF(obs, src, to, ts, k, tol=TOL, unbalancedints=True, ctx=ctx)
    assert op.stats()["n_bf"] == len(far)
    x = G.complex_gaussian(n, 3)
    rows = sample_rows(n, 96, seed=4)
    ref = far_dense_rows(obs, src, to, ts, far, k, rows, x)[:, 0]
    y = op.matvec(x)
    assert relerr(y[rows], ref) < 10 * TOL
    # adjoint: the kernel depends on the distance only, so the far field with the
    # roles swapped is A^T, and A^H x = conj(A^T conj(x))
    ya = op.adjoint().matvec(x)
    refa = np.conj(far_dense_rows(src, obs, ts, to, far[:, ::-1], k, rows, np.conj(x))[:, 0])
    assert relerr(ya[rows], refa) < 10 * TOL


def test_unbalanced_full_product_against_dense_kernel_rows(ctx):
    n = 4000
    pts = G.fibonacci_sphere(n)
    k = G.wavenumber(n, 4 * math.pi)
    tree = bfgpu.Tree.build(pts, max_points=32)
    op = bfgpu.PetrovGalerkinBF(pts, pts, tree, tree, k, tol=TOL, unbalancedints=True,
                                farfieldonly=False, ctx=ctx)
    assert op.stats()["near_pairs"] > 0
    x = G.complex_gaussian(n, 5)
    rows = sample_rows(n, 64, seed=6)
    d = np.linalg.norm(pts[rows][:, None, :] - pts[None, :, :], axis=2)
    with np.errstate(divide="ignore", invalid="ignore"):
        K = np.where(d > 0, np.exp(-1j * k * d) / (4 * np.pi * d), 0.0)
    assert relerr(op.matvec(x)[rows], K @ x) < 10 * TOL
