"""Near field on the GPU (bf_op_add_near) against the oracle.

With the near blocks attached, one bf_matvec applies near + far, as the
reference's mul! on a full PetrovGalerkinBF (src/matrixalgebra/
matrixvector.jl:28-33; blocks assembled at src/Matrixassembly/
petrovgalerkinbf.jl:57-119).  Checks, for forward, adjoint and transpose:
the product matches the oracle (reference-order far matvec on the exported
factors + the oracle's near BlockSparse product in FP64) to 1e-12; near + far
covers the whole matrix (the dense product, self-term r = 0 left out, within
the compression tolerance); non-leaf near pairs (leafcomp / leafimbalance
off) split correctly over leaves; the near field survives save / load, runs
on the allocation-free entry and under the tensor-core path (within 1e-4).
"""
import ctypes as C
import math

import numpy as np
import pytest

import bfgpu
from bfgpu import _lib
from bfgpu import geometry as G
from oracle import bfref as O
from _util import CsrTree, export_to_oracle, oracle_apply

pytestmark = pytest.mark.gpu
PARITY = 1e-12


def relerr(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def view(op, d):
    return op if d == "N" else op.adjoint() if d == "C" else op.transpose()


def reference(case, x, d):
    """oracle far (exported factors) + oracle near, op(A) x"""
    n_out = case["n_obs"] if d == "N" else case["n_src"]
    y = oracle_apply(case["bfs"], x, n_out, d)
    return y + O.near_matvec(case["kern"], case["to"], case["ts"], case["near"], x, d, n_out)


def make_case(ctx, obs, src, k, tol=1e-4, max_o=32, max_s=32, **opts):
    to, ts = O.build_tree(obs, max_points=max_o), O.build_tree(src, max_points=max_s)
    bo, bs = bfgpu.Tree.build(obs, max_points=max_o), bfgpu.Tree.build(src, max_points=max_s)
    op = bfgpu.PetrovGalerkinBF(obs, src, bo, bs, k, tol=tol, ctx=ctx, farfieldonly=False,
                                **opts)
    _, near = O.nearandfar(to, ts, 1.0, **{q: v for q, v in opts.items()
                                           if q in ("minbflvl", "leafcomp", "leafimbalance")})
    bfs = export_to_oracle(op.export_blocks(), CsrTree(*bo.values_csr()),
                           CsrTree(*bs.values_csr()))
    return dict(op=op, bfs=bfs, near=near, to=to, ts=ts, kern=O.HelmholtzKernel(obs, src, k),
                n_obs=len(obs), n_src=len(src), obs=obs, src=src, k=k, tol=tol)


@pytest.fixture(scope="module")
def sphere(ctx):
    n = 2048
    pts = G.fibonacci_sphere(n)
    return make_case(ctx, pts, pts, G.wavenumber(n, 4 * math.pi))


@pytest.mark.parametrize("d", ["N", "C", "T"])
def test_near_plus_far_matches_oracle(sphere, d):
    st = sphere["op"].stats()
    assert st["near_pairs"] == len(sphere["near"]) > 0 and st["near_entries"] > 0
    x = G.complex_gaussian(sphere["n_src"] if d == "N" else sphere["n_obs"], 5)
    assert relerr(view(sphere["op"], d).matvec(x), reference(sphere, x, d)) <= PARITY


def test_near_plus_far_is_the_whole_matrix(sphere):
    """Against the dense kernel matrix (self-term r = 0 left out): within 10 tol."""
    pts, n = sphere["obs"], sphere["n_obs"]
    D = O.near_block(sphere["kern"], np.arange(n), np.arange(n))
    x = G.complex_gaussian(n, 6)
    assert relerr(sphere["op"] @ x, D @ x) <= 10 * sphere["tol"]
    assert relerr(sphere["op"].adjoint() @ x, D.conj().T @ x) <= 10 * sphere["tol"]


def test_alpha_beta_multi_rhs_and_device(sphere, ctx):
    torch = pytest.importorskip("torch")
    op, n = sphere["op"], sphere["n_obs"]
    X = G.complex_gaussian(n, 7, nrhs=3)
    Y0 = G.complex_gaussian(n, 8, nrhs=3)
    alpha, beta = 0.5 - 2j, 1.5 + 0.25j
    Y = Y0.copy(order="F")
    bfgpu.mul(Y, op, X, alpha, beta)
    for j in range(3):
        ref = alpha * reference(sphere, X[:, j], "N") + beta * Y0[:, j]
        assert relerr(Y[:, j], ref) <= PARITY
    xd = torch.from_numpy(X[:, 0].copy()).cuda()
    yd = torch.zeros(n, dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    op.matvec_device(xd.data_ptr(), n, yd.data_ptr(), n)
    op.check()
    assert relerr(yd.cpu().numpy(), reference(sphere, X[:, 0], "N")) <= PARITY


@pytest.mark.parametrize("opts", [dict(minbflvl=2, leafcomp=False), dict(leafimbalance=False)])
def test_non_leaf_near_pairs_unbalanced_trees(ctx, opts):
    """Plane pair 0.2 apart, observer leaves <= 12 points, source leaves <= 60: near pairs
    with non-leaf nodes, split over the leaves below them."""
    obs, src = G.plane_pair(3000, 7, z_obs=0.2)
    case = make_case(ctx, obs, src, 2 * math.pi / 0.25, max_o=12, max_s=60, **opts)
    assert any(not (case["to"].isleaf(o) and case["ts"].isleaf(s)) for o, s in case["near"])
    for d in ("N", "C", "T"):
        x = G.complex_gaussian(case["n_src"] if d == "N" else case["n_obs"], 9)
        assert relerr(view(case["op"], d).matvec(x), reference(case, x, d)) <= PARITY, d


def test_save_load_with_near(sphere, ctx, tmp_path):
    path = str(tmp_path / "full.bfgpu")
    sphere["op"].save(path)
    back = bfgpu.load_operator(path, ctx)
    assert back.stats()["near_pairs"] == sphere["op"].stats()["near_pairs"]
    x = G.complex_gaussian(sphere["n_obs"], 10)
    for d in ("N", "C", "T"):
        assert np.array_equal(view(back, d).matvec(x), view(sphere["op"], d).matvec(x))


def test_noalloc_with_near(sphere):
    torch = pytest.importorskip("torch")
    op, n = sphere["op"], sphere["n_obs"]
    assert op.stats()["workspace_entries"] <= (1 << 20)
    lib = _lib.load()
    x = G.complex_gaussian(n, 11)
    xd = torch.from_numpy(x).cuda()
    yd = torch.full((n,), float("nan"), dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    _lib.check(lib.bf_matvec_noalloc(op._h, _lib.BF_OP_N, 1, C.c_void_p(xd.data_ptr()), n,
                                     C.c_void_p(yd.data_ptr()), n, None, None, None),
               "bf_matvec_noalloc")
    op.check()
    assert relerr(yd.cpu().numpy(), reference(sphere, x, "N")) <= PARITY


def test_mixed_path_adds_the_near_field(sphere):
    X = G.complex_gaussian(sphere["n_obs"], 12, nrhs=4)
    for d in ("N", "C"):
        v = view(sphere["op"], d)
        assert relerr(v.matvec(X, mixed=True), v.matvec(X)) <= 1e-4


def test_near_field_only_once_and_not_in_batches(sphere, ctx):
    from bfgpu.batch import Batch
    with pytest.raises(bfgpu.BFError) as e:
        sphere["op"].add_near(sphere["obs"], sphere["src"],
                              bfgpu.Tree.build(sphere["obs"], max_points=32),
                              bfgpu.Tree.build(sphere["src"], max_points=32), sphere["k"])
    assert e.value.status == _lib.BF_ESTATE
    with pytest.raises(bfgpu.BFError) as e:
        Batch([sphere["op"]], [1], ctx)
    assert e.value.status == _lib.BF_ENOTSUP
