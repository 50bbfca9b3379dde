"""Materialised adjoint and transpose (bf_op_adjoint_copy), the reference's
adjoint(BF) / transpose(BF) (src/Butterflyalgebra/bfadjtr.jl:13-67): the copy's
forward product must equal the oracle's adjoint product on the golden fixtures
and the library's own adjoint view on GPU-built operators, to the FP64 parity
bar, with the factor storage kept."""
import glob
import math
import os

import numpy as np
import pytest

import bfgpu
from bfgpu import geometry as G
from _util import relerr

pytestmark = pytest.mark.gpu
PARITY = 1e-12
HERE = os.path.dirname(os.path.abspath(__file__))


def golden(name, ctx):
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    op = bfgpu.import_blocks(int(g["n_rows"]), int(g["n_cols"]), g["bf"], g["stage"],
                             g["obs_out"], g["src_out"], g["obs_in"], g["src_in"], g["rows"],
                             g["cols"], g["identity"], g["data_off"], g["data"],
                             (g["obs_ptr"], g["obs_idx"]), (g["src_ptr"], g["src_idx"]), ctx)
    return g, op


@pytest.mark.parametrize("name", ["plane_single", "plane_unbalanced", "sphere_far"])
def test_copy_matches_oracle_adjoint(ctx, name):
    g, op = golden(name, ctx)
    c = op.adjoint_copy(bfgpu.BF_OP_C)
    t = op.adjoint_copy(bfgpu.BF_OP_T)
    assert c.shape == (op.shape[1], op.shape[0])
    assert relerr(c @ g["xa"], g["ya"]) <= PARITY
    # transpose(A) conj(xa) = conj(A^H xa)
    assert relerr(t @ np.conj(g["xa"]), np.conj(g["ya"])) <= PARITY
    # the copy's own adjoint view is A again
    assert relerr(c.adjoint() @ g["x"], g["y"]) <= PARITY
    assert c.stats()["factor_entries"] == op.stats()["factor_entries"]
    assert c.stats()["factor_bytes"] == op.stats()["factor_bytes"]


@pytest.mark.parametrize("storage", [bfgpu.BF_STORE_C32, bfgpu.BF_STORE_FF])
def test_copy_of_built_operator(ctx, storage):
    n = 4096
    pts = G.fibonacci_sphere(n)
    tree = bfgpu.Tree.build(pts, max_points=32)
    op = bfgpu.PetrovGalerkinBF(pts, pts, tree, tree, G.wavenumber(n, 4 * math.pi), tol=1e-4,
                                factor_storage=storage, ctx=ctx)
    X = G.complex_gaussian(n, 31, nrhs=3)
    c = op.adjoint_copy()
    assert c.stats()["factor_bytes"] == op.stats()["factor_bytes"]
    assert relerr(c.matvec(X), op.adjoint().matvec(X)) <= PARITY
    t = op.adjoint_copy(bfgpu.BF_OP_T)
    assert relerr(t.matvec(X), op.transpose().matvec(X)) <= PARITY
    # twice: the forward operator again
    cc = c.adjoint_copy()
    assert relerr(cc.matvec(X), op.matvec(X)) <= PARITY
    # many right-hand sides through the copy's forward chunks
    Y = G.complex_gaussian(n, 32, nrhs=9)
    assert relerr(c.matvec(Y), op.adjoint().matvec(Y)) <= PARITY


def test_refusals(ctx):
    g, op = golden("plane_single", ctx)
    with pytest.raises(bfgpu.BFError):
        op.adjoint_copy(bfgpu.BF_OP_N)
    obs, src = G.plane_pair(3000, 7, z_obs=0.2)
    to = bfgpu.Tree.build(obs, max_points=32)
    ts = bfgpu.Tree.build(src, max_points=32)
    full = bfgpu.PetrovGalerkinBF(obs, src, to, ts, 2 * math.pi / 0.25, tol=1e-4,
                                  farfieldonly=False, ctx=ctx)
    with pytest.raises(bfgpu.BFError, match="near field"):
        full.adjoint_copy()


def test_copy_of_recompressed_and_persisted(ctx, tmp_path):
    # the features compose: recompress, materialise the adjoint, save, load
    obs, src = G.plane_pair(4096, seed=1)
    k = 2 * math.pi / 0.125
    to, ts = bfgpu.Tree.build(obs, max_depth=4), bfgpu.Tree.build(src, max_depth=4)
    op = bfgpu.assemble_BF(obs, src, to, ts, 0, 0, k, 1e-4, c_tau=4.0, seed=3, ctx=ctx)
    rop = op.recompress(1e-2)
    c = rop.adjoint_copy()
    path = str(tmp_path / "c.bfop")
    c.save(path)
    back = bfgpu.load_operator(path, ctx)
    X = G.complex_gaussian(4096, 33, nrhs=2)
    assert np.array_equal(back.matvec(X), c.matvec(X))
    assert relerr(back.matvec(X), rop.adjoint().matvec(X)) <= PARITY
    assert relerr(back.adjoint().matvec(X), op.matvec(X)) < 10 * 1e-2


def test_recompression_at_extreme_tolerances(ctx):
    obs, src = G.plane_pair(4096, seed=1)
    k = 2 * math.pi / 0.125
    to, ts = bfgpu.Tree.build(obs, max_depth=4), bfgpu.Tree.build(src, max_depth=4)
    op = bfgpu.assemble_BF(obs, src, to, ts, 0, 0, k, 1e-4, c_tau=4.0, seed=3, ctx=ctx)
    X = G.complex_gaussian(4096, 34)
    y = op.matvec(X)
    # far above the build tolerance: ranks collapse, the product is still an operator
    coarse = op.recompress(0.5)
    assert coarse.stats()["factor_entries"] < op.stats()["factor_entries"]
    assert np.all(np.isfinite(coarse.matvec(X)))
    # far below it: little to take, the product within FP32 arithmetic of the input
    fine = op.recompress(1e-7)
    assert fine.stats()["factor_entries"] <= op.stats()["factor_entries"]
    assert relerr(fine.matvec(X), y) < 1e-4
