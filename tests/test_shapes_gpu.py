"""Level kernels at the edges of their task-shape classes.

One synthetic butterfly with one R level whose Q, R and P tasks take the
shapes at which the packer and the level kernels split their work:

* small (M <= 32): lane groups G = 32/M that leave lanes idle (M = 5, 7, 11,
  17, 31) or none (1, 2, 16, 32), column counts below, at and just above one
  load batch (1, 3, 4, 7, 8, 9, 33, 63, 64, 100);
* flat (32 < M <= 128, n <= 256): M = 33, 40, 63, 64, 65, 127, 128;
* tall (64-row panels): M = 129 and 300 (a partial last panel), 150 and 200,
  and M <= 128 with more than 256 columns (M = 40, 64);
* wide (M <= 32, n > 2M, n >= 128: the bulk-copy pipeline): 1 x 1500,
  5 x 130, 5 x 200, 20 x 779, 32 x 300.

Every task is one block set as the packer forms them (bf_pack.cpp): a Q task
per source leaf, an R task per connected set of slots, a P task per observer
leaf.  The factors are FP64 (float-float storage, true low parts).  Forward,
adjoint and transpose are held against the oracle's flat matvec on the same
blocks (the restatement of bfvector.jl:200-296) at 1e-12; the materialised
adjoint and the mixed tensor-core path run on the same shapes.
"""
import numpy as np
import pytest

from oracle import bfref as O

PARITY = 1e-12

# Q tasks (rows = rank of the slot, columns = points of the source leaf)
Q_SHAPES = [(1, 1), (2, 3), (3, 7), (5, 8), (7, 9), (11, 33), (16, 1), (17, 100), (31, 4),
            (32, 64), (129, 1), (200, 9), (300, 17), (150, 300), (33, 5), (63, 40), (64, 256),
            (65, 7), (127, 1), (128, 100), (40, 257), (5, 130), (32, 300), (1, 1500)]
# R tasks: rows of the output slot, the Q slots read (disjoint: one task each)
R_TASKS = [(3, [0, 1, 2, 3]), (40, [4, 5]), (200, [6, 7]), (1, [8, 9]),
           (20, [10, 11, 12, 13]), (64, [14, 15, 16, 17, 18, 19]), (33, [20]),
           (32, [21, 22, 23])]
# P tasks: points of the observer leaf reading R slot i
P_ROWS = [129, 2, 5, 1, 7, 64, 300, 17]


def synthetic(seed=0):
    """Blocks in the export layout, the two node -> values maps and the dense
    matrix they compose."""
    rng = np.random.default_rng(seed)
    n_src = sum(n for _, n in Q_SHAPES)
    n_obs = sum(P_ROWS)
    src_perm = rng.permutation(n_src)  # leaf values scattered over the point ids
    obs_perm = rng.permutation(n_obs)
    sptr = np.concatenate([[0], np.cumsum([n for _, n in Q_SHAPES])]).astype(np.int64)
    optr = np.concatenate([[0], np.cumsum(P_ROWS)]).astype(np.int64)
    blocks = []  # (stage, oo, so, oi, si, data)

    def mat(r, c):
        return (rng.standard_normal((r, c)) + 1j * rng.standard_normal((r, c))) / np.sqrt(c)

    Q = [mat(r, n) for r, n in Q_SHAPES]
    for j, (r, n) in enumerate(Q_SHAPES):  # slot key (j, 1000 + j), source leaf j
        blocks.append((0, j, 1000 + j, 0, j, Q[j]))
    R = []
    for i, (m, ins) in enumerate(R_TASKS):  # slot key (2000 + i, 3000 + i)
        R.append([mat(m, Q_SHAPES[j][0]) for j in ins])
        for j, Rij in zip(ins, R[i]):
            blocks.append((1, 2000 + i, 3000 + i, j, 1000 + j, Rij))
    P = [mat(p, R_TASKS[i][0]) for i, p in enumerate(P_ROWS)]
    for i in range(len(P_ROWS)):  # observer leaf i
        blocks.append((-1, i, 0, 2000 + i, 3000 + i, P[i]))
    ex = dict(bf=[], stage=[], obs_out=[], src_out=[], obs_in=[], src_in=[], rows=[], cols=[],
              identity=[], data_off=[])
    data = []
    off = 0
    for st, oo, so, oi, si, d in blocks:
        for k, v in zip(("bf", "stage", "obs_out", "src_out", "obs_in", "src_in", "rows", "cols",
                         "identity", "data_off"),
                        (0, st, oo, so, oi, si, d.shape[0], d.shape[1], 0, off)):
            ex[k].append(v)
        data.append(d.reshape(-1, order="F"))
        off += d.size
    ex = {k: np.asarray(v) for k, v in ex.items()}
    ex["data"] = np.concatenate(data)
    svals = (sptr, src_perm.astype(np.int64))
    ovals = (optr, obs_perm.astype(np.int64))
    # dense: y[obs(i)] += P_i sum_j R_ij Q_j x[src(j)]
    A = np.zeros((n_obs, n_src), np.complex128)
    for i, (m, ins) in enumerate(R_TASKS):
        rows = obs_perm[optr[i]:optr[i + 1]]
        for j, Rij in zip(ins, R[i]):
            cols = src_perm[sptr[j]:sptr[j + 1]]
            A[np.ix_(rows, cols)] += P[i] @ Rij @ Q[j]
    return dict(ex=ex, svals=svals, ovals=ovals, n_obs=n_obs, n_src=n_src, dense=A)


def relerr(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def syn():
    return synthetic(0)


def test_fixture_composes_like_the_oracle(syn):
    # the fixture's own dense product and the oracle's flat matvec agree
    bfs = O.from_blocks(syn["ex"], O.CsrTree(*syn["ovals"]), O.CsrTree(*syn["svals"]))
    rng = np.random.default_rng(1)
    x = rng.standard_normal(syn["n_src"]) + 1j * rng.standard_normal(syn["n_src"])
    assert relerr(O.apply_far(bfs, x, syn["n_obs"]), syn["dense"] @ x) < 1e-13
    xa = rng.standard_normal(syn["n_obs"]) + 1j * rng.standard_normal(syn["n_obs"])
    assert relerr(O.apply_far(bfs, xa, syn["n_src"], "C"), syn["dense"].conj().T @ xa) < 1e-13


@pytest.fixture(scope="module")
def gop(syn, ctx):
    import bfgpu
    ex = syn["ex"]
    return bfgpu.import_blocks(syn["n_obs"], syn["n_src"], ex["bf"], ex["stage"], ex["obs_out"],
                               ex["src_out"], ex["obs_in"], ex["src_in"], ex["rows"], ex["cols"],
                               ex["identity"], ex["data_off"], ex["data"], syn["ovals"],
                               syn["svals"], ctx)


def _oracle(syn):
    return O.from_blocks(syn["ex"], O.CsrTree(*syn["ovals"]), O.CsrTree(*syn["svals"]))


@pytest.mark.gpu
def test_tasks_cover_every_shape_class(gop):
    stage, kind, M, n = gop.task_shapes()
    dense = kind == 0
    got = {(int(s), int(a), int(b)) for s, a, b in zip(stage[dense], M[dense], n[dense])}
    want = {(0, r, c) for r, c in Q_SHAPES}
    want |= {(1, m, sum(Q_SHAPES[j][0] for j in ins)) for m, ins in R_TASKS}
    want |= {(2, p, R_TASKS[i][0]) for i, p in enumerate(P_ROWS)}
    assert want <= got, sorted(want - got)
    # every class is present: small, flat, tall, wide
    small = (M <= 32) & ~((n > 2 * M) & (n >= 128))
    wide = (M <= 32) & (n > 2 * M) & (n >= 128)
    flat = (M > 32) & (M <= 128) & (n <= 256)
    tall = ~small & ~wide & ~flat
    for cls in (small, flat, tall, wide):
        assert np.any(cls & dense)


@pytest.mark.gpu
@pytest.mark.parametrize("op_kind", ["N", "C", "T"])
def test_parity_against_the_oracle(syn, gop, op_kind):
    bfs = _oracle(syn)
    rng = np.random.default_rng(2)
    view = {"N": gop, "C": gop.adjoint(), "T": gop.transpose()}[op_kind]
    nin, nout = view.shape[1], view.shape[0]
    x = rng.standard_normal(nin) + 1j * rng.standard_normal(nin)
    y = view.matvec(x)
    assert relerr(y, O.apply_far(bfs, x, nout, op_kind)) <= PARITY
    A = {"N": syn["dense"], "C": syn["dense"].conj().T, "T": syn["dense"].T}[op_kind]
    assert relerr(y, A @ x) <= PARITY


@pytest.mark.gpu
@pytest.mark.parametrize("nrhs", [3, 8, 13])
def test_many_right_hand_sides(syn, gop, nrhs):
    # 3: the column loop; 8 and 13: the forward chunks of the one-operator batch
    rng = np.random.default_rng(3)
    X = rng.standard_normal((syn["n_src"], nrhs)) + 1j * rng.standard_normal((syn["n_src"], nrhs))
    Y = gop.matvec(X)
    assert relerr(Y, syn["dense"] @ X) <= PARITY
    Xa = rng.standard_normal((syn["n_obs"], nrhs)) + 1j * rng.standard_normal((syn["n_obs"], nrhs))
    assert relerr(gop.adjoint().matvec(Xa), syn["dense"].conj().T @ Xa) <= PARITY


@pytest.mark.gpu
def test_materialised_adjoint_runs_the_transposed_shapes(syn, gop):
    import bfgpu
    rng = np.random.default_rng(4)
    xa = rng.standard_normal(syn["n_obs"]) + 1j * rng.standard_normal(syn["n_obs"])
    for trans, A in ((bfgpu.BF_OP_C, syn["dense"].conj().T), (bfgpu.BF_OP_T, syn["dense"].T)):
        cp = gop.adjoint_copy(trans)
        assert cp.shape == (syn["n_src"], syn["n_obs"])
        assert relerr(cp.matvec(xa), A @ xa) <= PARITY


@pytest.mark.gpu
def test_mixed_path_on_the_same_shapes(syn, gop):
    rng = np.random.default_rng(5)
    X = rng.standard_normal((syn["n_src"], 4)) + 1j * rng.standard_normal((syn["n_src"], 4))
    assert relerr(gop.matvec(X, mixed=True), syn["dense"] @ X) <= 1e-4
    Xa = rng.standard_normal((syn["n_obs"], 4)) + 1j * rng.standard_normal((syn["n_obs"], 4))
    assert relerr(gop.adjoint().matvec(Xa, mixed=True), syn["dense"].conj().T @ Xa) <= 1e-4
