"""Batched operators (bf_batch_*): one CUDA-graph launch sequence for several
operators with different right-hand-side counts must give the same products as
one bf_matvec per operator (relative 2-norm <= 1e-12 per column: same
float-float arithmetic, same task routines), for every autotuner candidate.
"""
import math

import numpy as np
import pytest

import bfgpu
from bfgpu import geometry as G
from bfgpu.batch import Batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ops(ctx):
    out = []
    for shape, n, seed in (("sphere", 4096, 1), ("cube", 3000, 2), ("ellipsoid", 6144, 3)):
        pts, area = G.shape_points(shape, n, seed)
        k = G.wavenumber(n, area)
        tr = bfgpu.Tree.build(pts, max_points=32)
        out.append(bfgpu.PetrovGalerkinBF(pts, pts, tr, tr, k, tol=1e-4, ctx=ctx))
    return out


def colerr(Y, R):
    return max(np.linalg.norm(Y[:, j] - R[:, j]) / np.linalg.norm(R[:, j])
               for j in range(R.shape[1]))


def test_batch_matches_single_operator_matvecs(ops, ctx):
    nrhs = [1, 11, 5]
    b = Batch(ops, nrhs, ctx, rhs_chunk=4)
    xs = [G.complex_gaussian(o.shape[1], 30 + i, nrhs=r) for i, (o, r) in enumerate(zip(ops, nrhs))]
    ys = b.matvec(xs)
    for o, x, y in zip(ops, xs, ys):
        assert colerr(y, o.matvec(x)) <= 1e-12
    info = b.info()
    assert info["rhs_chunks"] == 3 and info["graph_nodes"] > 0 and info["work_items"] > 0
    # replay: same result
    ys2 = b.matvec(xs)
    for y, y2 in zip(ys, ys2):
        assert np.array_equal(y, y2)


def test_autotuner_keeps_results(ops, ctx):
    nrhs = [3, 2, 7]
    b = Batch(ops, nrhs, ctx, rhs_chunk=8)
    xs = [G.complex_gaussian(o.shape[1], 40 + i, nrhs=r) for i, (o, r) in enumerate(zip(ops, nrhs))]
    ms, cfg = b.autotune(nrep=2)
    assert ms > 0 and cfg["flat_mmax"] in (64, 96, 128) and cfg["ctas_per_sm"] in (2, 4, 6)
    for o, x, y in zip(ops, xs, b.matvec(xs)):
        assert colerr(y, o.matvec(x)) <= 1e-12


def test_batch_device_pointers(ops, ctx):
    import ctypes as C
    torch = pytest.importorskip("torch")
    nrhs = [2, 1, 1]
    b = Batch(ops, nrhs, ctx)
    xs = [G.complex_gaussian(o.shape[1], 50 + i, nrhs=r) for i, (o, r) in enumerate(zip(ops, nrhs))]
    xd = [torch.from_numpy(np.ascontiguousarray(x.T)).cuda() for x in xs]  # column j contiguous
    yd = [torch.zeros((r, o.shape[0]), dtype=torch.complex128, device="cuda")
          for o, r in zip(ops, nrhs)]
    torch.cuda.synchronize()
    xp = (C.c_void_p * 3)(*[t.data_ptr() for t in xd])
    yp = (C.c_void_p * 3)(*[t.data_ptr() for t in yd])
    lib = bfgpu._lib.load()
    assert lib.bf_batch_matvec(b._h, xp, None, yp, None, bfgpu.BF_PTR_DEVICE, None) == 0
    torch.cuda.synchronize()
    for o, x, y in zip(ops, xs, yd):
        assert colerr(y.cpu().numpy().T, o.matvec(x)) <= 1e-12
    assert b.buffers(0)[0] != 0
