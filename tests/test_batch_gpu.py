"""Batched operators (bf_batch_*) against the oracle.

One CUDA-graph launch sequence applies several operators -- forward, adjoint
and transpose, each with its own number of right-hand sides -- and every
column must match the oracle's reference-order product on the same factors
(oracle.bfref.matvec_flat over the far blocks, with the materialised adjoint of
src/Butterflyalgebra/bfadjtr.jl:13-67 for op = C / T) to relative 2-norm
1e-12, for every autotuner candidate.  Operators: the golden fixtures
(float-float factors imported from the oracle) and small GPU-built operators
(complex FP32 factors, exported to the oracle exactly).
"""
import os

import numpy as np
import pytest

import bfgpu
from bfgpu import geometry as G
from bfgpu.batch import Batch
from _util import CsrTree, export_to_oracle, oracle_apply

pytestmark = pytest.mark.gpu
PARITY = 1e-12
HERE = os.path.dirname(os.path.abspath(__file__))


def golden(name, ctx):
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    op = bfgpu.import_blocks(int(g["n_rows"]), int(g["n_cols"]), g["bf"], g["stage"],
                             g["obs_out"], g["src_out"], g["obs_in"], g["src_in"], g["rows"],
                             g["cols"], g["identity"], g["data_off"], g["data"],
                             (g["obs_ptr"], g["obs_idx"]), (g["src_ptr"], g["src_idx"]), ctx)
    ex = {k: g[k] for k in ("bf", "stage", "obs_out", "src_out", "obs_in", "src_in", "rows",
                            "cols", "identity", "data_off", "data")}
    bfs = export_to_oracle(ex, CsrTree(g["obs_ptr"], g["obs_idx"]),
                           CsrTree(g["src_ptr"], g["src_idx"]))
    return op, bfs


def view(op, d):
    return op if d == "N" else op.adjoint() if d == "C" else op.transpose()


def check(ops, bfs, dirs, nrhs, ctx, seed, rhs_chunk=8, tune=False):
    views = [view(o, d) for o, d in zip(ops, dirs)]
    b = Batch(views, nrhs, ctx, rhs_chunk=rhs_chunk)
    if tune:
        ms, cfg = b.autotune(nrep=1)
        assert ms > 0 and cfg["nr_max"] in (1, 4) and cfg["ctas_per_sm"] in (2, 4, 6)
    xs = [G.complex_gaussian(v.shape[1], seed + i, nrhs=r)
          for i, (v, r) in enumerate(zip(views, nrhs))]
    ys = b.matvec(xs)
    for v, bf, d, x, y in zip(views, bfs, dirs, xs, ys):
        for j in range(x.shape[1]):
            ref = oracle_apply(bf, x[:, j], v.shape[0], d)
            err = np.linalg.norm(y[:, j] - ref) / np.linalg.norm(ref)
            assert err <= PARITY, (d, j, err)
    return b, xs, ys


@pytest.fixture(scope="module")
def fixtures(ctx):
    return [golden(n, ctx) for n in ("plane_single", "sphere_far", "plane_unbalanced")]


@pytest.fixture(scope="module")
def built(ctx):
    out = []
    # small enough for the Python oracle (tens of thousands of far blocks each)
    for shape, n, seed in (("sphere", 2048, 1), ("cube", 1536, 2), ("ellipsoid", 2560, 3)):
        pts, area = G.shape_points(shape, n, seed)
        k = G.wavenumber(n, area)
        tr = bfgpu.Tree.build(pts, max_points=32)
        op = bfgpu.PetrovGalerkinBF(pts, pts, tr, tr, k, tol=1e-4, ctx=ctx)
        csr = CsrTree(*tr.values_csr())
        out.append((op, export_to_oracle(op.export_blocks(), csr, csr)))
    return out


@pytest.mark.parametrize("dirs", [("N", "N", "N"), ("C", "T", "N"), ("T", "N", "C")])
def test_golden_operators_mixed_directions(fixtures, ctx, dirs):
    ops = [o for o, _ in fixtures]
    bfs = [b for _, b in fixtures]
    # 5 and 11 right-hand sides in chunks of 8: sub-groups of 4, 2 and 1
    check(ops, bfs, dirs, [1, 5, 11], ctx, seed=10)


def test_built_operators_and_chunks(built, ctx):
    ops = [o for o, _ in built]
    bfs = [b for _, b in built]
    # 9 right-hand sides in chunks of 4: sub-groups of 4, then a single one
    b, xs, ys = check(ops, bfs, ("N", "C", "N"), [9, 3, 6], ctx, seed=20, rhs_chunk=4)
    info = b.info()
    assert info["rhs_chunks"] == 3 and info["graph_nodes"] > 0 and info["work_items"] > 0
    # replay: same result, bit for bit
    for y, y2 in zip(ys, b.matvec(xs)):
        assert np.array_equal(y, y2)


def test_autotuner_keeps_results(built, ctx):
    ops = [o for o, _ in built]
    bfs = [b for _, b in built]
    check(ops, bfs, ("T", "N", "C"), [3, 7, 7], ctx, seed=40, tune=True)


def test_batch_device_pointers(built, ctx):
    import ctypes as C
    torch = pytest.importorskip("torch")
    ops = [o for o, _ in built]
    bfs = [b for _, b in built]
    nrhs = [2, 1, 3]
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
    for o, bf, x, y in zip(ops, bfs, xs, yd):
        Y = y.cpu().numpy().T
        for j in range(x.shape[1]):
            ref = oracle_apply(bf, x[:, j], o.shape[0])
            assert np.linalg.norm(Y[:, j] - ref) / np.linalg.norm(ref) <= PARITY
    assert b.buffers(0)[0] != 0


def test_batch_matches_single_operator_path(built, ctx):
    """The same products as one bf_matvec per operator (same arithmetic)."""
    ops = [o for o, _ in built]
    views = [view(o, d) for o, d in zip(ops, ("N", "C", "T"))]
    b = Batch(views, [4, 4, 4], ctx, rhs_chunk=4)
    xs = [G.complex_gaussian(v.shape[1], 60 + i, nrhs=4) for i, v in enumerate(views)]
    for v, x, y in zip(views, xs, b.matvec(xs)):
        ref = v.matvec(x)
        assert np.linalg.norm(y - ref) / np.linalg.norm(ref) <= PARITY
