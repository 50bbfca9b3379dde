"""GPU parity of the FP64-accurate matvec against the oracle on identical factors.

Bar: relative 2-norm error <= 1e-12 against the reference-order CPU matvec
(src/Butterflyalgebra/bfvector.jl:200-296 restated in oracle/bfref.py);
summation order differs, so bit equality is not expected.
"""
import math

import numpy as np
import pytest

import bfgpu
from bfgpu import geometry as G
from oracle import bfref as O
from _util import import_oracle, relerr

pytestmark = pytest.mark.gpu
PARITY = 1e-12


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


def test_forward_parity_c1(c1):
    x = G.complex_gaussian(4096, 21)
    ref = O.matvec_flat(c1["bf"], x, np.zeros(4096, complex))
    y = c1["op"] @ x
    assert relerr(y, ref) <= PARITY


def test_adjoint_and_transpose_parity_c1(c1):
    x = G.complex_gaussian(4096, 22)
    refa = O.matvec_flat(O.adjoint_bf(c1["bf"], "C"), x, np.zeros(4096, complex))
    reft = O.matvec_flat(O.adjoint_bf(c1["bf"], "T"), x, np.zeros(4096, complex))
    assert relerr(c1["op"].adjoint() @ x, refa) <= PARITY
    assert relerr(c1["op"].transpose() @ x, reft) <= PARITY


def test_alpha_beta_and_multi_rhs(c1):
    X = G.complex_gaussian(4096, 23, nrhs=3)
    Y0 = G.complex_gaussian(4096, 24, nrhs=3)
    alpha, beta = 0.5 - 2j, 1.5 + 0.25j
    Y = Y0.copy(order="F")
    bfgpu.mul(Y, c1["op"], X, alpha, beta)
    for j in range(3):
        ref = O.matvec_flat(c1["bf"], X[:, j], Y0[:, j].copy(), alpha, beta)
        assert relerr(Y[:, j], ref) <= PARITY


@pytest.mark.parametrize("d", ["N", "C", "T"])
def test_many_rhs_chunks(c1, d):
    """19 right-hand sides: forward, two chunks of 8 through the operator's one-operator
    batch and three columns one by one (adjoint and transpose: column by column);
    alpha/beta, host and device pointers."""
    torch = pytest.importorskip("torch")
    op = {"N": c1["op"], "C": c1["op"].adjoint(), "T": c1["op"].transpose()}[d]
    bf = c1["bf"] if d == "N" else O.adjoint_bf(c1["bf"], d)
    X = G.complex_gaussian(4096, 26, nrhs=19)
    Y0 = G.complex_gaussian(4096, 27, nrhs=19)
    alpha, beta = 0.75 + 1j, -0.5 + 0.125j
    refs = [O.matvec_flat(bf, X[:, j], Y0[:, j].copy(), alpha, beta) for j in range(19)]
    Y = Y0.copy(order="F")
    bfgpu.mul(Y, op, X, alpha, beta)
    for j in range(19):
        assert relerr(Y[:, j], refs[j]) <= PARITY, j
    # device pointers with leading dimensions above the sizes; beta = 0 reads no y
    ld = 4100
    xd = torch.zeros((19, ld), dtype=torch.complex128, device="cuda")
    xd[:, :4096] = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
    yd = torch.full((19, ld), float("nan"), dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    op.matvec_device(xd.data_ptr(), ld, yd.data_ptr(), ld, nrhs=19, alpha=alpha)
    torch.cuda.synchronize()
    Yd = yd[:, :4096].cpu().numpy().T
    for j in range(19):
        ref = O.matvec_flat(bf, X[:, j], np.zeros(4096, complex), alpha, 0.0)
        assert relerr(Yd[:, j], ref) <= PARITY, j
    assert torch.isnan(yd[:, 4096:]).all()  # nothing past each column's end is written


def test_device_pointers(c1):
    torch = pytest.importorskip("torch")
    x = G.complex_gaussian(4096, 25)
    ref = O.matvec_flat(c1["bf"], x, np.zeros(4096, complex))
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros(4096, dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    c1["op"].matvec_device(xd.data_ptr(), 4096, yd.data_ptr(), 4096)
    torch.cuda.synchronize()
    assert relerr(yd.cpu().numpy(), ref) <= PARITY


@pytest.mark.parametrize("deep_obs", [True, False])
def test_unbalanced_trees_parity(ctx, deep_obs):
    obs, src = G.plane_pair(1500, seed=4, z_obs=2.5)
    k = 2 * math.pi / 0.25
    to = O.build_tree(obs, max_points=12 if deep_obs else 200)
    ts = O.build_tree(src, max_points=200 if deep_obs else 12)
    kern = O.HelmholtzKernel(obs, src, k)
    bf = O.assemble_bf(kern, to, ts, 0, 0, k, 1e-4, seed=1)
    op = import_oracle([bf], 1500, 1500, to, ts, ctx)
    x = G.complex_gaussian(1500, 1)
    assert relerr(op @ x, O.matvec_flat(bf, x, np.zeros(1500, complex))) <= PARITY
    assert relerr(op.adjoint() @ x,
                  O.matvec_flat(O.adjoint_bf(bf), x, np.zeros(1500, complex))) <= PARITY


def test_global_far_operator_parity(ctx):
    n = 2500
    pts = G.fibonacci_sphere(n)
    k = G.wavenumber(n, 4 * math.pi)
    t = O.build_tree(pts, max_points=24)
    kern = O.HelmholtzKernel(pts, pts, k)
    far = O.assemble_far(kern, t, t, k, 1e-4)
    op = import_oracle(far.bfs, n, n, t, t, ctx)
    x = G.complex_gaussian(n, 3)
    assert relerr(op @ x, O.far_matvec(far, x)) <= PARITY
    assert relerr(op.adjoint() @ x, O.far_matvec(far, x, adjoint=True)) <= PARITY
    st = op.stats()
    assert st["n_bf"] == len(far.bfs)
    assert st["factor_entries"] >= sum(O.factor_entries(b) for b in far.bfs)


def test_golden_fixtures(ctx):
    import glob
    import os
    from _util import tree_csr
    files = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
    assert files, "no golden fixtures"
    for f in files:
        g = np.load(f)
        op = bfgpu.import_blocks(int(g["n_rows"]), int(g["n_cols"]), g["bf"], g["stage"],
                                 g["obs_out"], g["src_out"], g["obs_in"], g["src_in"], g["rows"],
                                 g["cols"], g["identity"], g["data_off"], g["data"],
                                 (g["obs_ptr"], g["obs_idx"]), (g["src_ptr"], g["src_idx"]), ctx)
        assert relerr(op @ g["x"], g["y"]) <= PARITY, f
        assert relerr(op.adjoint() @ g["xa"], g["ya"]) <= PARITY, f


def test_golden_fixtures_any_block_order(ctx):
    """Imported blocks may come in any order: the packer groups R-level blocks
    per far pair only when they arrive grouped, and otherwise in one pass."""
    import glob
    import os
    from _util import tree_csr
    files = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
    rng = np.random.default_rng(11)
    for f in files:
        g = np.load(f)
        p = rng.permutation(len(g["bf"]))
        sel = {k: np.asarray(g[k])[p] for k in ("bf", "stage", "obs_out", "src_out", "obs_in",
                                               "src_in", "rows", "cols", "identity", "data_off")}
        op = bfgpu.import_blocks(int(g["n_rows"]), int(g["n_cols"]), sel["bf"], sel["stage"],
                                 sel["obs_out"], sel["src_out"], sel["obs_in"], sel["src_in"],
                                 sel["rows"], sel["cols"], sel["identity"], sel["data_off"],
                                 g["data"], (g["obs_ptr"], g["obs_idx"]),
                                 (g["src_ptr"], g["src_idx"]), ctx)
        assert relerr(op @ g["x"], g["y"]) <= PARITY, f
        assert relerr(op.adjoint() @ g["xa"], g["ya"]) <= PARITY, f
