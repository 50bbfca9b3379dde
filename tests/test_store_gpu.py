"""Persisted operators (bf_op_save / bf_op_load).

An operator written to disk and read back must give bit-identical products
(forward, adjoint, transpose, tensor-core path), the same statistics and the
same exported blocks; a file with a flipped byte in the factors or in the
tables, a truncated file, a foreign file and another format version must be
refused with an error, never uploaded.
"""
import math
import os

import numpy as np
import pytest

import bfgpu
from bfgpu import _lib
from bfgpu import geometry as G

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def built(ctx):
    n = 4096
    pts = G.fibonacci_sphere(n)
    tree = bfgpu.Tree.build(pts, max_points=32)
    return bfgpu.PetrovGalerkinBF(pts, pts, tree, tree, G.wavenumber(n, 4 * math.pi), tol=1e-4,
                                  ctx=ctx)


def golden_op(ctx):
    g = np.load(os.path.join(HERE, "golden", "sphere_far.npz"))
    return bfgpu.import_blocks(int(g["n_rows"]), int(g["n_cols"]), g["bf"], g["stage"],
                               g["obs_out"], g["src_out"], g["obs_in"], g["src_in"], g["rows"],
                               g["cols"], g["identity"], g["data_off"], g["data"],
                               (g["obs_ptr"], g["obs_idx"]), (g["src_ptr"], g["src_idx"]), ctx)


def same_operator(a, b):
    sa, sb = a.stats(), b.stats()
    for key in ("n_bf", "n_stages", "n_tasks", "factor_entries", "factor_bytes",
                "workspace_entries", "map_entries", "alg_bytes_fwd", "compressions"):
        assert sa[key] == sb[key], key
    n = a.shape[1]
    X = G.complex_gaussian(n, 3, nrhs=2)
    for va, vb in ((a, b), (a.adjoint(), b.adjoint()), (a.transpose(), b.transpose())):
        assert np.array_equal(va.matvec(X), vb.matvec(X))
    ea, eb = a.export_blocks(), b.export_blocks()
    for key in ea:
        assert np.array_equal(ea[key], eb[key]), key
    assert np.array_equal(a.rank_log(), b.rank_log())


@pytest.mark.parametrize("storage", [bfgpu.BF_STORE_C32, bfgpu.BF_STORE_FF])
def test_round_trip_built(ctx, tmp_path, storage):
    n = 4096
    pts = G.fibonacci_sphere(n)
    tree = bfgpu.Tree.build(pts, max_points=32)
    op = bfgpu.PetrovGalerkinBF(pts, pts, tree, tree, G.wavenumber(n, 4 * math.pi), tol=1e-4,
                                ctx=ctx, factor_storage=storage)
    path = str(tmp_path / "op.bfgpu")
    op.save(path)
    back = bfgpu.load_operator(path, ctx)
    same_operator(op, back)
    # the tensor-core path packs its planes from the loaded factors
    X = G.complex_gaussian(n, 4, nrhs=3)
    assert np.array_equal(op.matvec(X, mixed=True), back.matvec(X, mixed=True))


def test_round_trip_imported(ctx, tmp_path):
    op = golden_op(ctx)
    path = str(tmp_path / "golden.bfgpu")
    op.save(path)
    same_operator(op, bfgpu.load_operator(path, ctx))


def _refused(path, ctx, status, text):
    with pytest.raises(bfgpu.BFError) as e:
        bfgpu.load_operator(path, ctx)
    assert e.value.status == status, str(e.value)
    assert text in str(e.value), str(e.value)


def test_corrupt_files_are_refused(built, ctx, tmp_path):
    path = tmp_path / "op.bfgpu"
    built.save(str(path))
    raw = bytearray(path.read_bytes())
    fbytes = built.stats()["factor_bytes"]
    # a flipped bit in the middle of the factor array (after the tables)
    bad = bytearray(raw)
    bad[len(raw) - 24 - fbytes // 2] ^= 0x10
    (tmp_path / "f.bfgpu").write_bytes(bytes(bad))
    _refused(str(tmp_path / "f.bfgpu"), ctx, _lib.BF_EINVAL, "fail their check")
    # a flipped bit in the routing tables (far from the header)
    bad = bytearray(raw)
    bad[len(raw) - 24 - fbytes - 4096] ^= 0x01
    (tmp_path / "t.bfgpu").write_bytes(bytes(bad))
    with pytest.raises(bfgpu.BFError) as e:
        bfgpu.load_operator(str(tmp_path / "t.bfgpu"), ctx)
    assert e.value.status == _lib.BF_EINVAL
    # truncated
    (tmp_path / "s.bfgpu").write_bytes(bytes(raw[:len(raw) // 2]))
    with pytest.raises(bfgpu.BFError) as e:
        bfgpu.load_operator(str(tmp_path / "s.bfgpu"), ctx)
    assert e.value.status == _lib.BF_EINVAL
    # not an operator file / another format version
    (tmp_path / "n.bfgpu").write_bytes(b"hello world" * 100)
    _refused(str(tmp_path / "n.bfgpu"), ctx, _lib.BF_EINVAL, "not a saved operator")
    bad = bytearray(raw)
    bad[8] = 99  # version word
    (tmp_path / "v.bfgpu").write_bytes(bytes(bad))
    _refused(str(tmp_path / "v.bfgpu"), ctx, _lib.BF_ENOTSUP, "format version")
    _refused(str(tmp_path / "missing.bfgpu"), ctx, _lib.BF_EINVAL, "cannot open")
    # the good file still loads
    same_operator(built, bfgpu.load_operator(str(path), ctx))
