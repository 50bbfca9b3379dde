"""NumPy/SciPy restatement of the ButterflyFactorizations.jl far-field hot path.

Test infrastructure only (see ``oracle/__init__.py``): the GPU library never
imports this module.  Parity status: parity unpinned (no Julia in this image,
no golden vectors in the reference); pinned instead on the reference tests'
tolerance criteria and on LAPACK ``zgeqp3``.

Indexing is 0-based throughout; node ids, level lists and point indices are the
0-based images of the reference's 1-based ones.

Sampling of observer rows (reference: ``obs_index[randperm(n_obs)]``,
``src/ButterflyFactorization/compressors.jl:101``) draws from Julia's unseeded
global RNG, so it cannot be reproduced.  Here, and in the GPU library, the row
order is a keyed bijection of ``[0, n_obs)`` (a 4-round Feistel network with
cycle walking, keyed by ``task_key``), so that the oracle and the GPU build
sample the same rows for the same compression.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
from scipy.linalg import qr as _sp_qr, solve_triangular

M64 = (1 << 64) - 1

# --------------------------------------------------------------------------
# Keyed hashing / sampling (shared specification with csrc/bf_host.cpp)
# --------------------------------------------------------------------------


def mix64(z: int) -> int:
    """SplitMix64 finaliser on a Python int (mod 2^64)."""
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def task_key(seed: int, *vals: int) -> int:
    """Key of one compression: chained SplitMix64 over (seed, bf, stage, o, s)."""
    h = mix64(seed & M64)
    for v in vals:
        h = mix64(h ^ (int(v) & M64))
    return h


def _mix64_np(z):
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def sample_positions(j0: int, j1: int, n: int, key: int) -> np.ndarray:
    """Positions pi(j) for j in [j0, j1) of the keyed bijection pi on [0, n).

    Stands in for ``randperm(n_obs)[j0+1:j1]`` (compressors.jl:101): a balanced
    4-round Feistel network on [0, 4^h) (4^h >= n > 4^h / 4) with cycle walking.
    """
    if n <= 0 or j1 <= j0:
        return np.zeros(0, dtype=np.int64)
    if n == 1:
        return np.zeros(j1 - j0, dtype=np.int64)
    bits = (n - 1).bit_length()
    h = (bits + 1) // 2
    mask = np.uint64((1 << h) - 1)
    hh = np.uint64(h)
    kk = np.uint64(key & M64)
    x = np.arange(j0, j1, dtype=np.uint64)
    out = np.empty(j1 - j0, dtype=np.uint64)
    pending = np.arange(j1 - j0)
    nn = np.uint64(n)
    while pending.size:
        v = x[pending]
        L = v >> hh
        R = v & mask
        for rnd in range(4):
            F = _mix64_np(kk ^ np.uint64((rnd + 1) << 56) ^ R) & mask
            L, R = R, L ^ F
        v = (L << hh) | R
        ok = v < nn
        out[pending[ok]] = v[ok]
        x[pending[~ok]] = v[~ok]
        pending = pending[~ok]
    return out.astype(np.int64)


# --------------------------------------------------------------------------
# Cluster tree (2^d tree on a bounding cube) -- stands in for H2Trees.TwoNTree
# --------------------------------------------------------------------------


@dataclass
class Tree:
    """0-based BFS-numbered 2^3 tree.  ``values(node) = perm[begin:end]``.

    Interface follows the reference tree contract (``src/treeinterface.jl:39-164``):
    center, radius (= halfsize * sqrt(3), ``ext/BFH2Trees/BFH2Trees.jl:15-16``),
    children, isleaf, root, values, parent, levels.
    """

    center: np.ndarray
    halfsize: np.ndarray
    level: np.ndarray
    parent: np.ndarray
    first_child: np.ndarray
    n_child: np.ndarray
    begin: np.ndarray
    end: np.ndarray
    perm: np.ndarray

    @property
    def n_nodes(self) -> int:
        return len(self.halfsize)

    def values(self, node: int) -> np.ndarray:
        return self.perm[self.begin[node]:self.end[node]]

    def children(self, node: int):
        f = int(self.first_child[node])
        return range(f, f + int(self.n_child[node]))

    def isleaf(self, node: int) -> bool:
        return self.n_child[node] == 0

    def radius(self, node: int) -> float:
        return float(self.halfsize[node]) * math.sqrt(3.0)

    def root(self) -> int:
        return 0

    def levels(self):
        nl = int(self.level.max()) + 1
        return [np.nonzero(self.level == l)[0] for l in range(nl)]


def build_tree(points: np.ndarray, max_points: int | None = None,
               max_depth: int | None = None) -> Tree:
    """Breadth-first 2^3 tree on the bounding cube of ``points``.

    A node is a leaf when it holds <= ``max_points`` points, or sits at depth
    ``max_depth`` (root depth 0), or holds a single point.  Children are the
    non-empty octants in order ``(x>=cx) + 2(y>=cy) + 4(z>=cz)``; points are
    stably partitioned so each node's values are a contiguous range of ``perm``.
    Same rule as ``bf_tree_build`` in the library.
    """
    pts = np.ascontiguousarray(points, dtype=np.float64)
    n = pts.shape[0]
    lo = pts.min(axis=0)
    hi = pts.max(axis=0)
    c0 = (lo + hi) * 0.5
    h0 = float(np.max(hi - lo)) * 0.5
    perm = np.arange(n, dtype=np.int64)
    center = [c0]
    half = [h0]
    level = [0]
    parent = [-1]
    begin = [0]
    end = [n]
    first_child = [0]
    n_child = [0]
    current = [0]
    while current:
        nxt = []
        for nd in current:
            b, e = begin[nd], end[nd]
            cnt = e - b
            leaf = cnt <= 1
            if max_points is not None and cnt <= max_points:
                leaf = True
            if max_depth is not None and level[nd] >= max_depth:
                leaf = True
            if half[nd] <= 0.0:
                leaf = True
            if leaf:
                first_child[nd] = len(center)
                n_child[nd] = 0
                continue
            c = center[nd]
            p = pts[perm[b:e]]
            octv = ((p[:, 0] >= c[0]).astype(np.int64)
                    + 2 * (p[:, 1] >= c[1]).astype(np.int64)
                    + 4 * (p[:, 2] >= c[2]).astype(np.int64))
            order = np.argsort(octv, kind="stable")
            perm[b:e] = perm[b:e][order]
            counts = np.bincount(octv, minlength=8)
            hc = half[nd] * 0.5
            first_child[nd] = len(center)
            nc = 0
            off = b
            for o in range(8):
                if counts[o] == 0:
                    continue
                cc = np.array([c[0] + (hc if (o & 1) else -hc),
                               c[1] + (hc if (o & 2) else -hc),
                               c[2] + (hc if (o & 4) else -hc)])
                center.append(cc)
                half.append(hc)
                level.append(level[nd] + 1)
                parent.append(nd)
                begin.append(off)
                end.append(off + int(counts[o]))
                first_child.append(0)
                n_child.append(0)
                nxt.append(len(center) - 1)
                off += int(counts[o])
                nc += 1
            n_child[nd] = nc
        current = nxt
    return Tree(center=np.array(center), halfsize=np.array(half), level=np.array(level),
                parent=np.array(parent), first_child=np.array(first_child),
                n_child=np.array(n_child), begin=np.array(begin), end=np.array(end),
                perm=perm)


def treelevels(tree: Tree, root: int):
    """BFS levels below ``root`` (``src/auxillaries.jl:263-281``)."""
    levels = []
    current = [root]
    while current:
        levels.append(list(current))
        nxt = []
        for node in current:
            if not tree.isleaf(node):
                nxt.extend(tree.children(node))
        current = nxt
    return levels


def traverseandpad(tree: Tree, root: int):
    """Levels with shallow leaves pushed down to the deepest level.

    ``src/auxillaries.jl:340-350``: for levels 2..end-1 (1-based) every leaf is
    appended to the next level, after that level's real nodes.
    """
    lv = treelevels(tree, root)
    for l in range(1, len(lv) - 1):
        for node in list(lv[l]):
            if tree.isleaf(node):
                lv[l + 1].append(node)
    return lv


# --------------------------------------------------------------------------
# Admissibility and interaction lists
# --------------------------------------------------------------------------


def is_far(tree_s: Tree, tree_o: Tree, snode: int, onode: int, alpha: float) -> bool:
    """AABB admissibility ``ext/BFH2Trees/h2admissible.jl:11-45``."""
    oc = tree_o.center[onode]
    ol = tree_o.radius(onode)
    sc = tree_s.center[snode]
    sl = tree_s.radius(snode)
    W = max(sl, ol)
    target = alpha * W
    mind_sq = 0.0
    for i in range(3):
        d = abs(oc[i] - sc[i]) - (sl + ol)
        if d > 0.0:
            mind_sq += d * d
    if mind_sq < 1e-10:
        return False
    return math.sqrt(mind_sq) > target


def nearandfar(tree_o: Tree, tree_s: Tree, alpha: float = 1.0, minbflvl: int = 3,
               leafcomp: bool = True, leafimbalance: bool = True, unbalancedints: bool = False):
    """Dual-tree traversal ``src/Matrixassembly/intlists.jl:30-217``: balanced splitting,
    or with ``unbalancedints`` only the larger node of a pair splits (``:121-149``,
    ``largernode`` = radius comparison, ``src/treeinterface.jl:153-154``).

    Returns ``(far, near)`` lists of ``(observer_node, source_node)`` in the
    reference's depth-first order.
    """
    far, near = [], []
    height0 = min(int(tree_o.level.max()) + 1, int(tree_s.level.max()) + 1)
    stack = [(0, 0, height0)]
    while stack:
        no, ns, h = stack.pop()
        lo = tree_o.isleaf(no)
        ls = tree_s.isleaf(ns)
        adm = is_far(tree_s, tree_o, ns, no, alpha)
        if h <= minbflvl and not leafcomp:
            near.append((no, ns))
            continue
        if adm:
            if (lo or ls) and not leafcomp:
                near.append((no, ns))
            else:
                far.append((no, ns))
            continue
        if (lo and ls) or ((lo or ls) and not leafimbalance):
            near.append((no, ns))
            continue
        kids = []
        if unbalancedints:
            if (tree_o.radius(no) >= tree_s.radius(ns) and not lo) or ls:
                kids = [(co, ns) for co in tree_o.children(no)]
            else:
                kids = [(no, cs) for cs in tree_s.children(ns)]
        elif lo:
            kids = [(no, cs) for cs in tree_s.children(ns)]
        elif ls:
            kids = [(co, ns) for co in tree_o.children(no)]
        else:
            kids = [(co, cs) for co in tree_o.children(no) for cs in tree_s.children(ns)]
        for co, cs in reversed(kids):
            stack.append((co, cs, h - 1))
    return far, near


# --------------------------------------------------------------------------
# Kernel, rank estimate, compressor
# --------------------------------------------------------------------------


class HelmholtzKernel:
    """Point Helmholtz kernel G(r) = exp(-i k r) / (4 pi r).

    Plays the role of the kernel functor ``(km)(Z, rows, cols)``
    (``ext/BFBEAST/kernelmatrix.jl:74-82``); the reference has no point kernel.
    """

    def __init__(self, obs_pts: np.ndarray, src_pts: np.ndarray, k: float):
        self.obs = np.asarray(obs_pts, dtype=np.float64)
        self.src = np.asarray(src_pts, dtype=np.float64)
        self.k = float(k)

    def __call__(self, rows, cols) -> np.ndarray:
        rows = np.asarray(rows, dtype=np.int64)
        cols = np.asarray(cols, dtype=np.int64)
        d = self.obs[rows][:, None, :] - self.src[cols][None, :, :]
        r = np.sqrt(np.einsum("ijk,ijk->ij", d, d))
        return np.exp(-1j * self.k * r) / (4.0 * np.pi * r)


def estimate_rank_butterfly(eps: float, c_tau: float, rmin: int = 10) -> int:
    """``src/ButterflyFactorization/rankestimation.jl:93-98``."""
    return max(int(math.ceil(c_tau * math.log(1.0 / eps))), rmin)


def estimate_rank_3d(k: float, tree_s: Tree, tree_o: Tree, snode: int, onode: int, eps: float,
                     C: float = 1.5, Ceps: float = 1.5, Rmin: int = 3) -> int:
    """``GeometricRankEstimator`` (``rankestimation.jl:13-25``) with the tree method of
    ``ext/BFH2Trees/h2rankest.jl:8-38``: x1 = (k a_s a_o / max(d, 1e-4))^2 from the node
    radii and the center distance, x2 = log(1/eps), max(ceil(C x1 + Ceps x2), Rmin)."""
    d2 = 0.0
    for a in range(3):
        dd = float(tree_s.center[snode, a]) - float(tree_o.center[onode, a])
        d2 += dd * dd
    d = max(math.sqrt(d2), 1e-4)
    g = k * (tree_s.radius(snode) * tree_o.radius(onode)) / d
    return max(int(math.ceil(C * (g * g) + Ceps * math.log(1.0 / eps))), Rmin)


def pqr_rank(R: np.ndarray, rtol: float) -> int:
    """Rank of a column-pivoted QR truncated at |R_ii| <= rtol |R_00|.

    Restates ``LowRankApprox.pqr(Z; rtol)`` (third-party, ``Project.toml:33``
    compat 0.5, version unpinned, called at ``compressors.jl:129``): pivoted
    Householder QR that stops once the next pivot column norm falls to
    ``rtol`` times the first.
    """
    d = np.abs(np.diag(R))
    if d.size == 0 or d[0] == 0.0:
        return 0
    thr = rtol * d[0]
    r = 0
    while r < d.size and d[r] > thr:
        r += 1
    return r


@dataclass
class CompressionRecord:
    key: int
    rows_evaluated: int
    n_obs: int
    n_src: int
    rank: int
    retries: int


def partial_qr(kern, src_index, obs_index, n_est: int, eps: float, adaptive: bool,
               key: int, min_samples: int = 10, log: list | None = None):
    """PartialQR compressor ``src/ButterflyFactorization/compressors.jl:81-165``.

    Returns ``(T, skeleton, r)`` with ``T`` (r x n_src) the interpolation
    matrix ``R11^-1 Q1^H Z`` and ``skeleton = src_index[P[:r]]``.
    """
    src_index = np.asarray(src_index, dtype=np.int64)
    obs_index = np.asarray(obs_index, dtype=np.int64)
    n_obs = len(obs_index)
    n_src = len(src_index)
    if n_obs == 0 or n_src == 0:
        return np.zeros((0, n_src), dtype=np.complex128), np.zeros(0, dtype=np.int64), 0
    n = min(max(n_est, min_samples), n_obs)
    rows = obs_index[sample_positions(0, n, n_obs, key)]
    Z = kern(rows, src_index)
    rows_eval = n
    retries = 0
    while True:
        Qf, Rf, P = _sp_qr(Z, mode="economic", pivoting=True)
        r = pqr_rank(Rf, eps)
        if adaptive and r > math.floor(0.8 * rows_eval) and rows_eval < n_obs:
            new_target = min(rows_eval * 2, n_obs)
            extra = obs_index[sample_positions(rows_eval, new_target, n_obs, key)]
            Z = np.vstack([Z, kern(extra, src_index)])
            rows_eval = new_target
            retries += 1
            continue
        if log is not None:
            log.append(CompressionRecord(key, rows_eval, n_obs, n_src, r, retries))
        Q1 = Qf[:, :r]
        R11 = Rf[:r, :r]
        T = solve_triangular(R11, Q1.conj().T @ Z, lower=False) if r > 0 else \
            np.zeros((0, n_src), dtype=np.complex128)
        return T, src_index[P[:r]], r


# --------------------------------------------------------------------------
# Butterfly factorisation (dictionary format) and assembly
# --------------------------------------------------------------------------


@dataclass
class Block:
    """``ButterflyBlock`` (``bfstructs.jl:21-29``); ``data is None`` means identity."""

    obs_out: int
    src_out: int
    obs_in: int
    src_in: int
    data: np.ndarray | None
    out_ptr: int = -1
    in_ptr: int = -1


@dataclass
class BF:
    """``ButterflyFactorization`` (``bfstructs.jl:91-146``) with pointer wiring."""

    Q: list
    R: list
    P: list
    tree_o: Tree
    tree_s: Tree
    k: float
    tau: float
    no: int = 0
    ns: int = 0
    slot_len: list = field(default_factory=list)

    def wire(self):
        """One pointer map per level (``bfstructs.jl:107-143``), 0-based."""
        nlev = len(self.R) + 1
        maps = [dict() for _ in range(nlev)]

        def ptr(l, key):
            m = maps[l]
            if key not in m:
                m[key] = len(m)
            return m[key]

        for b in self.Q:
            b.out_ptr = ptr(0, (b.obs_out, b.src_out))
            b.in_ptr = -1
        for l, lvl in enumerate(self.R):
            for b in lvl:
                b.in_ptr = ptr(l, (b.obs_in, b.src_in))
                b.out_ptr = ptr(l + 1, (b.obs_out, b.src_out))
        for b in self.P:
            b.in_ptr = ptr(nlev - 1, (b.obs_in, b.src_in))
            b.out_ptr = -1
        self.nslots = [len(m) for m in maps]
        return self


def assemble_bf(kern, tree_o: Tree, tree_s: Tree, no: int, ns: int, k: float, tau: float,
                c_tau: float = 4.0, adaptive: bool = True, seed: int = 0, bf_id: int = 0,
                min_samples: int = 10, log: list | None = None, geometric=None) -> BF:
    """``assemble_BF`` (``src/ButterflyFactorization/bfassembly.jl:48-200``).

    ``c_tau`` is the ButterflyRankEstimator constant (default ``Ctau=4.0``,
    ``bfassembly.jl:55-57`` with ``ext/BFH2Trees/h2parameters.jl:22-24``).
    Compression task keys are ``task_key(seed, bf_id, stage, obs_node, src_node)``
    with stage 0 for Q and l for R level l.
    """
    treeS = traverseandpad(tree_s, ns)
    treeO = traverseandpad(tree_o, no)
    LS, LO = len(treeS), len(treeO)
    L = max(LS, LO)
    eps = tau / L
    n_est = estimate_rank_butterfly(eps, c_tau)
    K = {}

    def comp(src, obs, stage, onode, snode):
        # geometric = (C, Ceps, Rmin): the GeometricRankEstimator at every call site
        # (the reference calls rankestimator(k, trialT, testT, Snode, Onode, tau_scaled))
        est = n_est if geometric is None else estimate_rank_3d(k, tree_s, tree_o, snode, onode,
                                                               eps, *geometric)
        return partial_qr(kern, src, obs, est, eps, adaptive,
                          task_key(seed, bf_id, stage, onode, snode), min_samples, log)

    # Q stage (bfassembly.jl:82-102)
    Q = []
    obs_root = tree_o.values(no)
    for Sleaf in treeS[-1]:
        T, skel, _ = comp(tree_s.values(Sleaf), obs_root, 0, no, Sleaf)
        Q.append(Block(no, Sleaf, no, Sleaf, T))
        K[(Sleaf, no)] = skel

    def build_U(s_level, o_level):
        # bfassembly.jl:206-230
        U = {}
        for Svert in s_level:
            for Overt in o_level:
                if not tree_s.isleaf(Svert):
                    U[(Svert, Overt)] = np.concatenate(
                        [K[(Sc, Overt)] for Sc in tree_s.children(Svert)])
                else:
                    U[(Svert, Overt)] = K[(Svert, Overt)]
        return U

    def split(T, Svert, Overt, obs_out, src_out, blocks):
        last = 0
        for Sc in tree_s.children(Svert):
            ks = len(K[(Sc, Overt)])
            blocks.append(Block(obs_out, src_out, Overt, Sc, T[:, last:last + ks].copy()))
            last += ks

    R = []
    for l in range(1, L):
        s_frozen = l >= LS
        o_frozen = l >= LO
        if s_frozen and o_frozen:
            break
        blocks, upd = [], []
        if not s_frozen and not o_frozen:
            # build_nonfrozen_R_blocks (bfassembly.jl:232-349)
            o_lvl, s_lvl = treeO[l - 1], treeS[LS - l - 1]
            U = build_U(s_lvl, o_lvl)
            for Svert in s_lvl:
                for Overt in o_lvl:
                    if not tree_o.isleaf(Overt):
                        for Oc in tree_o.children(Overt):
                            T, skel, _ = comp(U[(Svert, Overt)], tree_o.values(Oc), l, Oc, Svert)
                            upd.append((Svert, Oc, skel))
                            if not tree_s.isleaf(Svert):
                                split(T, Svert, Overt, Oc, Svert, blocks)
                            else:
                                blocks.append(Block(Oc, Svert, Overt, Svert, T))
                    else:
                        if not tree_s.isleaf(Svert):
                            T, skel, _ = comp(U[(Svert, Overt)], tree_o.values(Overt), l,
                                              Overt, Svert)
                            split(T, Svert, Overt, Overt, Svert, blocks)
                            upd.append((Svert, Overt, skel))
                        else:
                            blocks.append(Block(Overt, Svert, Overt, Svert, None))
                            upd.append((Svert, Overt, K[(Svert, Overt)]))
        elif s_frozen and not o_frozen:
            # build_sourcefrozen_R_blocks (bfassembly.jl:351-412)
            Svert = ns
            for Overt in treeO[l - 1]:
                if not tree_o.isleaf(Overt):
                    for Oc in tree_o.children(Overt):
                        T, skel, _ = comp(K[(Svert, Overt)], tree_o.values(Oc), l, Oc, Svert)
                        blocks.append(Block(Oc, Svert, Overt, Svert, T))
                        upd.append((Svert, Oc, skel))
                else:
                    blocks.append(Block(Overt, Svert, Overt, Svert, None))
                    upd.append((Svert, Overt, K[(Svert, Overt)]))
        else:
            # build_observerfrozen_R_blocks (bfassembly.jl:414-481)
            o_lvl, s_lvl = treeO[LO - 1], treeS[LS - l - 1]
            U = build_U(s_lvl, o_lvl)
            for Svert in s_lvl:
                for Overt in o_lvl:
                    if not tree_s.isleaf(Svert):
                        T, skel, _ = comp(U[(Svert, Overt)], tree_o.values(Overt), l,
                                          Overt, Svert)
                        split(T, Svert, Overt, Overt, Svert, blocks)
                        upd.append((Svert, Overt, skel))
                    else:
                        blocks.append(Block(Overt, Svert, Overt, Svert, None))
                        upd.append((Svert, Overt, K[(Svert, Overt)]))
        R.append(blocks)
        for s, o, skel in upd:
            K[(s, o)] = skel

    # P stage (bfassembly.jl:186-197)
    P = []
    for Oleaf in treeO[-1]:
        col = K[(ns, Oleaf)]
        row = tree_o.values(Oleaf)
        P.append(Block(Oleaf, ns, Oleaf, ns, kern(row, col)))
    return BF(Q, R, P, tree_o, tree_s, k, tau, no, ns).wire()


# --------------------------------------------------------------------------
# Matvecs
# --------------------------------------------------------------------------


def matvec_flat(bf: BF, x: np.ndarray, y: np.ndarray, alpha=1.0, beta=0.0) -> np.ndarray:
    """Flat-array matvec ``src/Butterflyalgebra/bfvector.jl:200-296``."""
    if beta != 1:
        y[:] = 0 if beta == 0 else y * beta
    nlev = len(bf.R) + 1
    bufs = [dict() for _ in range(nlev)]
    for b in bf.Q:
        v = x[bf.tree_s.values(b.src_in)]
        bufs[0][b.out_ptr] = v.copy() if b.data is None else b.data @ v
    for l, lvl in enumerate(bf.R):
        bin_, bout = bufs[l], bufs[l + 1]
        for b in lvl:
            n = len(bin_[b.in_ptr]) if b.data is None else b.data.shape[0]
            bout[b.out_ptr] = np.zeros(n, dtype=np.complex128)
        for b in lvl:
            vin = bin_[b.in_ptr]
            if b.data is None:
                bout[b.out_ptr] += vin
            else:
                bout[b.out_ptr] += b.data @ vin
    last = bufs[nlev - 1]
    for b in bf.P:
        vin = last[b.in_ptr]
        idx = bf.tree_o.values(b.obs_out)
        y[idx] += alpha * (vin if b.data is None else b.data @ vin)
    return y


def matvec_dict(bf: BF, x: np.ndarray, y: np.ndarray, alpha=1.0, beta=0.0) -> np.ndarray:
    """Dictionary matvec ``src/Butterflyalgebra/bfvector.jl:16-79``."""
    if beta != 1:
        y[:] = 0 if beta == 0 else y * beta
    nxt = {}
    for b in bf.Q:
        v = x[bf.tree_s.values(b.src_in)]
        nxt[(b.obs_out, b.src_out)] = v.copy() if b.data is None else b.data @ v
    for lvl in bf.R:
        cur, nxt = nxt, {}
        for b in lvl:
            vin = cur[(b.obs_in, b.src_in)]
            part = vin.copy() if b.data is None else b.data @ vin
            key = (b.obs_out, b.src_out)
            if key in nxt:
                nxt[key] = nxt[key] + part
            else:
                nxt[key] = part
    for b in bf.P:
        vin = nxt[(b.obs_in, b.src_in)]
        idx = bf.tree_o.values(b.obs_out)
        y[idx] += alpha * (vin if b.data is None else b.data @ vin)
    return y


def adjoint_bf(bf: BF, op: str = "C") -> BF:
    """Materialised adjoint / transpose ``src/Butterflyalgebra/bfadjtr.jl:13-67``."""
    f = (lambda d: d.conj().T.copy()) if op == "C" else (lambda d: d.T.copy())

    def tb(b):
        return Block(b.src_in, b.obs_in, b.src_out, b.obs_out,
                     None if b.data is None else f(b.data))

    Q = [tb(b) for b in bf.P]
    R = [[tb(b) for b in lvl] for lvl in reversed(bf.R)]
    P = [tb(b) for b in bf.Q]
    return BF(Q, R, P, bf.tree_s, bf.tree_o, bf.k, bf.tau, bf.ns, bf.no).wire()


def factor_entries(bf: BF) -> int:
    n = sum(b.data.size for b in bf.Q if b.data is not None)
    n += sum(b.data.size for lvl in bf.R for b in lvl if b.data is not None)
    n += sum(b.data.size for b in bf.P if b.data is not None)
    return n


# --------------------------------------------------------------------------
# Exchange with the C-ABI block layout (bf_op_export_blocks / bf_factor_desc)
# --------------------------------------------------------------------------


class CsrTree:
    """The part of the tree contract the matvecs use (``values(node)``), from a
    node -> values CSR map (ptr, idx)."""

    def __init__(self, ptr, idx):
        self.ptr = np.asarray(ptr, np.int64)
        self.idx = np.asarray(idx, np.int64)

    def values(self, node):
        return self.idx[self.ptr[node]:self.ptr[node + 1]]


def from_blocks(ex, tree_o, tree_s, k: float = 0.0, tau: float = 0.0) -> list:
    """Exported block arrays (keys, stage, shapes, identity flags, column-major data)
    -> one pointer-wired BF per far block; stage 0 = Q, -1 = P, l = R level l."""
    nbf = int(ex["bf"].max()) + 1 if len(ex["bf"]) else 0
    per = [dict(Q=[], R={}, P=[]) for _ in range(nbf)]
    for b in range(len(ex["bf"])):
        f, st = int(ex["bf"][b]), int(ex["stage"][b])
        if ex["identity"][b]:
            data = None
        else:
            r, c, off = int(ex["rows"][b]), int(ex["cols"][b]), int(ex["data_off"][b])
            data = ex["data"][off:off + r * c].reshape((r, c), order="F")
        blk = Block(int(ex["obs_out"][b]), int(ex["src_out"][b]), int(ex["obs_in"][b]),
                    int(ex["src_in"][b]), data)
        if st == 0:
            per[f]["Q"].append(blk)
        elif st < 0:
            per[f]["P"].append(blk)
        else:
            per[f]["R"].setdefault(st, []).append(blk)
    out = []
    for f in range(nbf):
        d = per[f]
        R = [d["R"][lv] for lv in sorted(d["R"])]
        no = d["Q"][0].obs_out if d["Q"] else 0
        ns = d["P"][0].src_out if d["P"] else 0
        out.append(BF(d["Q"], R, d["P"], tree_o, tree_s, k, tau, no, ns).wire())
    return out


def apply_far(bfs: list, x: np.ndarray, n_out: int, op: str = "N") -> np.ndarray:
    """op(A) x over a list of BFs: the reference-order flat matvec of each, through
    the materialised adjoint / transpose for "C" / "T"."""
    y = np.zeros(n_out, np.complex128)
    for bf in bfs:
        b = bf if op == "N" else adjoint_bf(bf, op)
        matvec_flat(b, x, y, 1.0, 1.0)
    return y


# --------------------------------------------------------------------------
# Algebraic recompression (src/Butterflyalgebra/algrecomp.jl)
# --------------------------------------------------------------------------


def pqr(A: np.ndarray, rtol: float):
    """``LowRankApprox.pqr(A; rtol)`` as called at ``algrecomp.jl:83``: Q (m x r)
    with orthonormal columns, R (r x n) upper trapezoidal in pivoted column
    order, and the pivots p, truncated by :func:`pqr_rank`."""
    Q, R, p = _sp_qr(A, mode="economic", pivoting=True)
    r = pqr_rank(R, rtol)
    return Q[:, :r], R[:r, :], p


def recompress_right(bf: BF, tau: float, stats: dict | None = None) -> BF:
    """``recompress_BF_right`` (``algrecomp.jl:45-148``).

    For the R levels from the last to the second (``lold = lr - l + 1``,
    ``algrecomp.jl:59-61``): the blocks sharing a column key
    ``(obs_in, src_in)`` are stacked in key order (``:63-78``), the stack is
    compressed by pivoted QR at rtol ``tau`` (``:83``), its row slices of Q
    replace the blocks (``:89-101``) and ``T = R[:, invperm(p)]`` (``:86``)
    multiplies every block of the previous level whose row key
    ``(obs_out, src_out)`` is that column key (``:115-132``).

    Identity blocks (padding of uneven trees, ``bfassembly.jl:340``) pass one
    node through unchanged and are alone in their column groups; such a group
    is left as it is, which is what the pivoted QR of an identity gives
    (Q = I, T = I).  An identity in the previous level becomes ``T * I = T``.
    """
    R = [[Block(b.obs_out, b.src_out, b.obs_in, b.src_in,
                None if b.data is None else b.data.copy()) for b in lvl] for lvl in bf.R]
    lr = len(R)
    for l in range(1, lr):
        lold = lr - l  # 0-based index of R_factors[lr - l + 1]
        cur = R[lold]
        groups: dict = {}
        for i, b in enumerate(cur):
            groups.setdefault((b.obs_in, b.src_in), []).append(i)
        Ru = {}
        for key in sorted(groups):
            idx = groups[key]
            if any(cur[i].data is None for i in idx):
                continue
            A = np.vstack([cur[i].data for i in idx])
            Qm, Rm, p = pqr(A, tau)
            Ru[key] = Rm[:, np.argsort(p)]
            row = 0
            for i in idx:
                h = cur[i].data.shape[0]
                cur[i].data = Qm[row:row + h, :].copy()
                row += h
            if stats is not None:
                stats["groups"] = stats.get("groups", 0) + 1
        for b in R[lold - 1]:
            T = Ru.get((b.obs_out, b.src_out))
            if T is not None:
                b.data = T.copy() if b.data is None else T @ b.data
    return BF([Block(b.obs_out, b.src_out, b.obs_in, b.src_in, b.data) for b in bf.Q], R,
              [Block(b.obs_out, b.src_out, b.obs_in, b.src_in, b.data) for b in bf.P],
              bf.tree_o, bf.tree_s, bf.k, bf.tau, bf.no, bf.ns).wire()


def recompress_bf(bf: BF, tau: float, stats: dict | None = None) -> BF:
    """``recompress_BF`` (``algrecomp.jl:19-31``): the right pass, then the
    right pass of the adjoint, adjoined back (the left pass)."""
    right = recompress_right(bf, tau, stats)
    return adjoint_bf(recompress_right(adjoint_bf(right, "C"), tau, stats), "C")


# --------------------------------------------------------------------------
# Global far-field operator (PetrovGalerkinBF far part)
# --------------------------------------------------------------------------


@dataclass
class FarOperator:
    """Far-field part of ``PetrovGalerkinBF`` (``petrovgalerkinbf.jl:121-151``)."""

    bfs: list
    pairs: list
    n_rows: int
    n_cols: int


def assemble_far(kern, tree_o: Tree, tree_s: Tree, k: float, tol: float, alpha: float = 1.0,
                 c_tau: float = 2.9592, adaptive: bool = True, seed: int = 0,
                 minbflvl: int = 3, log: list | None = None,
                 unbalancedints: bool = False) -> FarOperator:
    """One ``assemble_BF`` per admissible pair (``petrovgalerkinbf.jl:129-151``).

    ``c_tau = 2.9592`` is the TwoNTree + isFarFunctor constant
    (``ext/BFH2Trees/h2parameters.jl:44-48``) that ``PetrovGalerkinBF`` uses.
    """
    far, _ = nearandfar(tree_o, tree_s, alpha=alpha, minbflvl=minbflvl,
                        unbalancedints=unbalancedints)
    bfs = [assemble_bf(kern, tree_o, tree_s, no, ns, k, tol, c_tau, adaptive, seed, i, log=log)
           for i, (no, ns) in enumerate(far)]
    return FarOperator(bfs, far, len(tree_o.perm), len(tree_s.perm))


def far_matvec(op: FarOperator, x, alpha=1.0, beta=0.0, y=None, adjoint: bool = False):
    """``mul!(y, A::PetrovGalerkinBF, x, alpha, beta)`` far part (``matrixvector.jl:8-65``).

    Each BF is applied into a zeroed accumulator and the accumulator is added
    with ``alpha`` (the per-thread buffer + reduction of the reference).
    ``adjoint=True`` applies ``adjoint(A)`` (``matrix_adj_tr.jl:8-25``).
    """
    nr, nc = (op.n_cols, op.n_rows) if adjoint else (op.n_rows, op.n_cols)
    if y is None:
        y = np.zeros(nr, dtype=np.complex128)
    if beta == 0:
        y[:] = 0
    elif beta != 1:
        y *= beta
    acc = np.zeros(nr, dtype=np.complex128)
    for bf in op.bfs:
        b = adjoint_bf(bf) if adjoint else bf
        matvec_flat(b, x, acc, 1.0, 1.0)
    y += alpha * acc
    return y


def near_block(kern: HelmholtzKernel, rows, cols) -> np.ndarray:
    """One near block K(rows, cols) (the blocks of ``petrovgalerkinbf.jl:57-119``) for the
    point kernel; the singular self-term r = 0 (a point with itself) is left out (zero)."""
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    d = kern.obs[rows][:, None, :] - kern.src[cols][None, :, :]
    r = np.sqrt(np.einsum("ijk,ijk->ij", d, d))
    out = np.zeros(r.shape, dtype=np.complex128)
    nz = r > 0
    out[nz] = np.exp(-1j * kern.k * r[nz]) / (4.0 * np.pi * r[nz])
    return out


def near_matvec(kern: HelmholtzKernel, tree_o: Tree, tree_s: Tree, near, x, op: str = "N",
                n_out: int | None = None):
    """Near-field BlockSparseMatrix product (assembled at ``petrovgalerkinbf.jl:57-119``,
    applied by ``mul!`` at ``matrixvector.jl:28-33``): y[values(o)] += K_os x[values(s)] over
    the near pairs; "C" / "T" apply the adjoint / transpose of every block."""
    if n_out is None:
        n_out = len(tree_o.perm) if op == "N" else len(tree_s.perm)
    y = np.zeros(n_out, dtype=np.complex128)
    for o, s in near:
        ro, cs = tree_o.values(o), tree_s.values(s)
        B = near_block(kern, ro, cs)
        if op == "N":
            y[ro] += B @ x[cs]
        elif op == "C":
            y[cs] += B.conj().T @ x[ro]
        else:
            y[cs] += B.T @ x[ro]
    return y


def dense_far(kern, op: FarOperator) -> np.ndarray:
    """Dense far-field matrix: sum over admissible pairs of K[values(NO), values(NS)]."""
    A = np.zeros((op.n_rows, op.n_cols), dtype=np.complex128)
    for bf in op.bfs:
        ro = bf.tree_o.values(bf.no)
        cs = bf.tree_s.values(bf.ns)
        A[np.ix_(ro, cs)] += kern(ro, cs)
    return A
