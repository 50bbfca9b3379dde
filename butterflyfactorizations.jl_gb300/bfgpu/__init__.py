"""bfgpu -- Python host mirror of the ButterflyFactorizations.jl far-field interface.

The functions mirror the reference's operator interface on top of the C ABI of
``libbfgpu.so``:

=====================================  =============================================
reference (Julia)                      here
=====================================  =============================================
``assemble_BF(km, blktree, no, ns,     ``assemble_BF(obs, src, tree_o, tree_s, no,
k, tau; ...)`` (bfassembly.jl:48)      ns, k, tau, ...)`` -> ``Operator``
``PetrovGalerkinBF(op, X, Y, tree,     ``PetrovGalerkinBF(obs, src, tree_o, tree_s, k,
k; tol, ...)`` far part                 tol=1e-3, ...)`` -> ``Operator``
(petrovgalerkinbf.jl:33)
``mul!(y, A, x, alpha, beta)``         ``mul(y, A, x, alpha, beta)``
(matrixvector.jl:8)
``A * x``                              ``A @ x``
``adjoint(A)``, ``transpose(A)``       ``A.adjoint()``, ``A.transpose()`` (lazy; no copy)
``size(A)``                            ``A.shape``
``nearandfar(tree, alpha)``            ``nearandfar(tree_o, tree_s, alpha)``
=====================================  =============================================

All compute runs in ``libbfgpu.so`` on the GPU; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import (BF_OP_C, BF_OP_N, BF_OP_T, BF_PTR_DEVICE, BF_PTR_HOST, BF_STORE_C32,
                   BF_STORE_FF, RANK_REC_LEN, SUR_NW, BFError, BuildOpts, FactorDesc, OpStats,
                   check, load)

__all__ = ["Tree", "Context", "Operator", "nearandfar", "assemble_BF", "PetrovGalerkinBF",
           "import_blocks", "load_operator", "compress_block", "near_pairs", "nearandfar_gpu", "mul", "BFError",
           "GeometricRankEstimator",
           "load"]


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class Tree:
    """2^3 cluster tree built by the library (``bf_tree_build``)."""

    def __init__(self, handle, points=None):
        self._h = C.c_void_p(handle)
        self.points = points
        lib = load()
        nn, npnt, depth = C.c_int64(), C.c_int64(), C.c_int32()
        check(lib.bf_tree_size(self._h, C.byref(nn), C.byref(npnt), C.byref(depth)), "tree_size")
        n, m = nn.value, npnt.value
        self.center = np.zeros((n, 3))
        self.halfsize = np.zeros(n)
        self.level = np.zeros(n, np.int32)
        self.parent = np.zeros(n, np.int32)
        self.first_child = np.zeros(n, np.int32)
        self.n_child = np.zeros(n, np.int32)
        self.begin = np.zeros(n, np.int64)
        self.end = np.zeros(n, np.int64)
        self.perm = np.zeros(m, np.int64)
        check(lib.bf_tree_export(self._h, _p(self.center, C.c_double), _p(self.halfsize, C.c_double),
                                 _p(self.level, C.c_int32), _p(self.parent, C.c_int32),
                                 _p(self.first_child, C.c_int32), _p(self.n_child, C.c_int32),
                                 _p(self.begin, C.c_int64), _p(self.end, C.c_int64),
                                 _p(self.perm, C.c_int64)), "tree_export")
        self.depth = depth.value

    @classmethod
    def build(cls, points, max_points: int | None = None, max_depth: int | None = None):
        lib = load()
        pts = np.ascontiguousarray(points, dtype=np.float64)
        h = C.c_void_p()
        check(lib.bf_tree_build(_p(pts, C.c_double), pts.shape[0],
                                -1 if max_points is None else int(max_points),
                                -1 if max_depth is None else int(max_depth), C.byref(h)),
              "bf_tree_build")
        return cls(h.value, pts)

    @classmethod
    def build_gpu(cls, points, max_points: int | None = None, max_depth: int | None = None,
                  ctx: "Context | None" = None):
        """The same tree as ``build``, with the point partitioning on the GPU."""
        lib = load()
        ctx = ctx or default_context()
        pts = np.ascontiguousarray(points, dtype=np.float64)
        h = C.c_void_p()
        check(lib.bf_tree_build_gpu(ctx._h, _p(pts, C.c_double), pts.shape[0],
                                    -1 if max_points is None else int(max_points),
                                    -1 if max_depth is None else int(max_depth), C.byref(h)),
              "bf_tree_build_gpu")
        return cls(h.value, pts)

    @property
    def n_nodes(self):
        return len(self.halfsize)

    def values(self, node):
        return self.perm[self.begin[node]:self.end[node]]

    def children(self, node):
        f = int(self.first_child[node])
        return range(f, f + int(self.n_child[node]))

    def isleaf(self, node):
        return self.n_child[node] == 0

    def values_csr(self):
        """node -> values map as CSR (ptr, idx) over all nodes."""
        lens = (self.end - self.begin).astype(np.int64)
        ptr = np.zeros(self.n_nodes + 1, np.int64)
        np.cumsum(lens, out=ptr[1:])
        idx = np.concatenate([self.values(i) for i in range(self.n_nodes)]).astype(np.int64)
        return ptr, idx

    def __del__(self):
        try:
            if self._h and self._h.value:
                load().bf_tree_destroy(self._h)
        except Exception:
            pass


def nearandfar(tree_o: Tree, tree_s: Tree, alpha: float = 1.0, minbflvl: int = 3,
               leafcomp: bool = True, leafimbalance: bool = True, unbalancedints: bool = False):
    """Far pairs (n_far, 2) [observer node, source node] and the near-pair count."""
    lib = load()
    nf, nn = C.c_int64(), C.c_int64()
    args = (tree_o._h, tree_s._h, float(alpha), int(minbflvl), int(leafcomp), int(leafimbalance),
            int(unbalancedints))
    check(lib.bf_nearandfar(*args, None, None, 0, C.byref(nf), C.byref(nn)), "bf_nearandfar")
    fo = np.zeros(max(nf.value, 1), np.int64)
    fs = np.zeros(max(nf.value, 1), np.int64)
    check(lib.bf_nearandfar(*args, _p(fo, C.c_int64), _p(fs, C.c_int64), max(nf.value, 1),
                            C.byref(nf), C.byref(nn)), "bf_nearandfar")
    return np.stack([fo[:nf.value], fs[:nf.value]], axis=1), nn.value


def near_pairs(tree_o: Tree, tree_s: Tree, alpha: float = 1.0, minbflvl: int = 3,
               leafcomp: bool = True, leafimbalance: bool = True, unbalancedints: bool = False):
    """Near pairs (n_near, 2) [observer node, source node] of the same traversal."""
    lib = load()
    nn = C.c_int64()
    args = (tree_o._h, tree_s._h, float(alpha), int(minbflvl), int(leafcomp), int(leafimbalance),
            int(unbalancedints))
    check(lib.bf_near_pairs(*args, None, None, 0, C.byref(nn)), "bf_near_pairs")
    fo = np.zeros(max(nn.value, 1), np.int64)
    fs = np.zeros(max(nn.value, 1), np.int64)
    check(lib.bf_near_pairs(*args, _p(fo, C.c_int64), _p(fs, C.c_int64), max(nn.value, 1),
                            C.byref(nn)), "bf_near_pairs")
    return np.stack([fo[:nn.value], fs[:nn.value]], axis=1)


def nearandfar_gpu(tree_o: Tree, tree_s: Tree, alpha: float = 1.0, minbflvl: int = 3,
                   leafcomp: bool = True, leafimbalance: bool = True,
                   unbalancedints: bool = False, ctx=None):
    """Far and near pairs, (n, 2) arrays each, traversed on the GPU (same order as
    ``nearandfar`` / ``near_pairs``)."""
    lib = load()
    ctx = ctx or default_context()
    nf, nn = C.c_int64(), C.c_int64()
    args = (ctx._h, tree_o._h, tree_s._h, float(alpha), int(minbflvl), int(leafcomp),
            int(leafimbalance), int(unbalancedints))
    check(lib.bf_nearandfar_gpu(*args, None, None, 0, None, None, 0, C.byref(nf), C.byref(nn)),
          "bf_nearandfar_gpu")
    a = [np.zeros(max(v, 1), np.int64) for v in (nf.value, nf.value, nn.value, nn.value)]
    check(lib.bf_nearandfar_gpu(*args, _p(a[0], C.c_int64), _p(a[1], C.c_int64), len(a[0]),
                                _p(a[2], C.c_int64), _p(a[3], C.c_int64), len(a[2]),
                                C.byref(nf), C.byref(nn)), "bf_nearandfar_gpu")
    far = np.stack([a[0][:nf.value], a[1][:nf.value]], axis=1)
    near = np.stack([a[2][:nn.value], a[3][:nn.value]], axis=1)
    return far, near


class Context:
    """One CUDA device (``bf_ctx_create``)."""

    def __init__(self, device: int = 0):
        lib = load()
        h = C.c_void_p()
        check(lib.bf_ctx_create(int(device), C.byref(h)), "bf_ctx_create")
        self._h = h
        self.device = device

    def __del__(self):
        try:
            if self._h and self._h.value:
                load().bf_ctx_destroy(self._h)
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class Operator:
    """Device-resident far-field butterfly operator (a LinearMap-like object)."""

    def __init__(self, handle, ctx: Context, trans: int = BF_OP_N, parent=None):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle
        self.ctx = ctx
        self.trans = trans
        self._parent = parent  # keeps the owner alive for lazy adjoint views
        lib = load()
        r, c = C.c_int64(), C.c_int64()
        check(lib.bf_op_size(self._h, C.byref(r), C.byref(c)), "bf_op_size")
        self._nr, self._nc = r.value, c.value

    @property
    def shape(self):
        return (self._nr, self._nc) if self.trans == BF_OP_N else (self._nc, self._nr)

    def adjoint(self):
        if self.trans == BF_OP_N:
            return Operator(self._h, self.ctx, BF_OP_C, self)
        if self.trans == BF_OP_C:
            return Operator(self._h, self.ctx, BF_OP_N, self)
        raise ValueError("adjoint of a transpose view is not supported")

    H = property(adjoint)

    def transpose(self):
        if self.trans == BF_OP_N:
            return Operator(self._h, self.ctx, BF_OP_T, self)
        if self.trans == BF_OP_T:
            return Operator(self._h, self.ctx, BF_OP_N, self)
        raise ValueError("transpose of an adjoint view is not supported")

    T = property(transpose)

    def stats(self) -> dict:
        s = OpStats()
        check(load().bf_op_stats_get(self._h, C.byref(s)), "bf_op_stats_get")
        return {k: getattr(s, k) for k, _ in OpStats._fields_}

    def matvec(self, x, y=None, alpha=1.0, beta=0.0, mixed: bool = False):
        """y = beta*y + alpha*op(A)*x for host complex128 arrays (n,) or (n, nrhs)."""
        lib = load()
        x = np.asarray(x)
        vec = x.ndim == 1
        X = np.asfortranarray(x.reshape(x.shape[0], -1).astype(np.complex128, copy=False))
        nin = self.shape[1]
        nout = self.shape[0]
        if X.shape[0] != nin:
            raise ValueError(f"x has {X.shape[0]} rows, operator needs {nin}")
        nrhs = X.shape[1]
        if y is None:
            Y = np.zeros((nout, nrhs), dtype=np.complex128, order="F")
            beta = 0.0
        else:
            Y = y.reshape(nout, -1)
            if not (Y.dtype == np.complex128 and Y.flags.f_contiguous):
                raise ValueError("y must be a Fortran-ordered complex128 array")
        a = (C.c_double * 2)(complex(alpha).real, complex(alpha).imag)
        b = (C.c_double * 2)(complex(beta).real, complex(beta).imag)
        fn = lib.bf_matvec_mixed if mixed else lib.bf_matvec
        check(fn(self._h, self.trans, nrhs, X.ctypes.data, X.shape[0], Y.ctypes.data, Y.shape[0],
                 a, b, BF_PTR_HOST, None), "bf_matvec_mixed" if mixed else "bf_matvec")
        if y is not None:
            return y
        return Y[:, 0] if vec else Y

    def matvec_device(self, x_ptr: int, ldx: int, y_ptr: int, ldy: int, nrhs: int = 1,
                      alpha=1.0, beta=0.0, stream: int = 0, mixed: bool = False):
        """Stream-ordered matvec on device pointers (complex128 column-major)."""
        lib = load()
        a = (C.c_double * 2)(complex(alpha).real, complex(alpha).imag)
        b = (C.c_double * 2)(complex(beta).real, complex(beta).imag)
        fn = lib.bf_matvec_mixed if mixed else lib.bf_matvec
        check(fn(self._h, self.trans, int(nrhs), C.c_void_p(x_ptr), int(ldx), C.c_void_p(y_ptr),
                 int(ldy), a, b, BF_PTR_DEVICE, C.c_void_p(stream) if stream else None),
              "bf_matvec(device)")

    def matvec_ptr(self, x_ptr: int, ldx: int, y_ptr: int, ldy: int, nrhs: int = 1,
                   alpha=1.0, beta=0.0, ptr_mode: int = BF_PTR_HOST, stream: int = 0,
                   mixed: bool = False):
        """Raw-pointer matvec; ptr_mode BF_PTR_HOST copies x/y inside the call."""
        lib = load()
        a = (C.c_double * 2)(complex(alpha).real, complex(alpha).imag)
        b = (C.c_double * 2)(complex(beta).real, complex(beta).imag)
        fn = lib.bf_matvec_mixed if mixed else lib.bf_matvec
        check(fn(self._h, self.trans, int(nrhs), C.c_void_p(x_ptr), int(ldx), C.c_void_p(y_ptr),
                 int(ldy), a, b, int(ptr_mode), C.c_void_p(stream) if stream else None),
              "bf_matvec(ptr)")

    def __matmul__(self, x):
        return self.matvec(x)

    def check(self, stream: int = 0):
        """Synchronise ``stream`` (0: the operator's own) and raise BFError(BF_ETIMEOUT) if a
        bounded device-side wait of an asynchronous matvec gave up since the last check."""
        check(load().bf_op_check(self._h, C.c_void_p(stream) if stream else None),
              "bf_op_check")

    def set_wait_limit(self, polls: int):
        """Test hook: polls of a bounded wait in the plain path (< 0: the default)."""
        check(load().bf_op_set_wait_limit(self._h, int(polls)), "bf_op_set_wait_limit")

    def export_blocks(self, bf_begin: int = 0, bf_end: int | None = None,
                      as_float32: bool = False):
        """Factors of far blocks [bf_begin, bf_end) as reference-style block arrays."""
        lib = load()
        if bf_end is None:
            bf_end = self.stats()["n_bf"]
        nb, nd = C.c_int64(), C.c_int64()
        N = None
        check(lib.bf_op_export_blocks(self._h, bf_begin, bf_end, C.byref(nb), C.byref(nd),
                                      *([N] * 11), 0), "export")
        n = nb.value
        out = dict(bf=np.zeros(n, np.int32), stage=np.zeros(n, np.int32),
                   obs_out=np.zeros(n, np.int64), src_out=np.zeros(n, np.int64),
                   obs_in=np.zeros(n, np.int64), src_in=np.zeros(n, np.int64),
                   rows=np.zeros(n, np.int32), cols=np.zeros(n, np.int32),
                   identity=np.zeros(n, np.int8), data_off=np.zeros(n, np.int64),
                   data=np.zeros(max(nd.value, 1), np.complex64 if as_float32 else np.complex128))
        check(lib.bf_op_export_blocks(
            self._h, bf_begin, bf_end, C.byref(nb), C.byref(nd), _p(out["bf"], C.c_int32),
            _p(out["stage"], C.c_int32), _p(out["obs_out"], C.c_int64),
            _p(out["src_out"], C.c_int64), _p(out["obs_in"], C.c_int64),
            _p(out["src_in"], C.c_int64), _p(out["rows"], C.c_int32), _p(out["cols"], C.c_int32),
            _p(out["identity"], C.c_int8), _p(out["data_off"], C.c_int64),
            C.c_void_p(out["data"].ctypes.data), int(as_float32)), "export")
        return out

    def rank_log(self) -> np.ndarray:
        """Per-compression rank records of the build, (n, 18) float64 (see bfgpu.h):
        columns 0-13 as the reference RankLogger fields, 14-17 the surrogate features."""
        lib = load()
        n = C.c_int64()
        check(lib.bf_op_rank_log(self._h, C.byref(n), None), "rank_log")
        rec = np.zeros((max(n.value, 1), RANK_REC_LEN))
        check(lib.bf_op_rank_log(self._h, C.byref(n), _p(rec, C.c_double)), "rank_log")
        return rec[:n.value]

    def task_shapes(self):
        """(stage, kind, M, n) int32 arrays of the packed level tasks."""
        lib = load()
        n = C.c_int64()
        check(lib.bf_op_task_shapes(self._h, C.byref(n), None, None, None, None), "task_shapes")
        a = [np.zeros(max(n.value, 1), np.int32) for _ in range(4)]
        check(lib.bf_op_task_shapes(self._h, C.byref(n), *[_p(v, C.c_int32) for v in a]),
              "task_shapes")
        return tuple(v[:n.value] for v in a)

    def profile(self, nrep: int = 5):
        """Per-level launch times (ms), algorithmic bytes and kernels per matvec."""
        lib = load()
        ns = self.stats()["n_stages"]
        ms = np.zeros(ns)
        by = np.zeros(ns, np.int64)
        nk = C.c_int64()
        check(lib.bf_op_profile(self._h, self.trans, int(nrep), _p(ms, C.c_double),
                                _p(by, C.c_int64), C.byref(nk)), "bf_op_profile")
        return ms, by, nk.value

    def profile_mixed(self, nrep: int = 3):
        """Mixed path, one 128-RHS chunk: per-level ms, bytes, useful flops, kernels."""
        lib = load()
        ns = self.stats()["n_stages"]
        ms = np.zeros(ns)
        by = np.zeros(ns, np.int64)
        fl = np.zeros(ns)
        nk = C.c_int64()
        check(lib.bf_op_profile_mixed(self._h, self.trans, int(nrep), _p(ms, C.c_double),
                                      _p(by, C.c_int64), _p(fl, C.c_double), C.byref(nk)),
              "bf_op_profile_mixed")
        return ms, by, fl, nk.value

    def mixed_info(self) -> dict:
        """BF16 factor bytes, workspace bytes and work units of the mixed path."""
        f, w, u = C.c_int64(), C.c_int64(), C.c_int64()
        check(load().bf_op_mixed_info(self._h, C.byref(f), C.byref(w), C.byref(u)),
              "bf_op_mixed_info")
        return dict(factor_bytes=f.value, workspace_bytes=w.value, work_units=u.value)

    def add_near(self, obs, src, tree_o: Tree, tree_s: Tree, k: float, pairs=None,
                 alpha: float = 1.0, minbflvl: int = 3, leafcomp: bool = True,
                 leafimbalance: bool = True, unbalancedints: bool = False):
        """Attach the near field (``bf_op_add_near``): afterwards every matvec applies
        near + far, as the reference's ``mul!`` on a full ``PetrovGalerkinBF``."""
        if pairs is None:
            pairs = near_pairs(tree_o, tree_s, alpha, minbflvl, leafcomp, leafimbalance,
                               unbalancedints)
        obs = np.ascontiguousarray(obs, np.float64)
        src = np.ascontiguousarray(src, np.float64)
        pairs = np.asarray(pairs, np.int64).reshape(-1, 2)
        no = np.ascontiguousarray(pairs[:, 0])
        ns = np.ascontiguousarray(pairs[:, 1])
        check(load().bf_op_add_near(self._h, _p(obs, C.c_double), obs.shape[0],
                                    _p(src, C.c_double), src.shape[0], tree_o._h, tree_s._h,
                                    _p(no, C.c_int64), _p(ns, C.c_int64), len(no), float(k)),
              "bf_op_add_near")
        return self

    def recompress(self, tau: float) -> "Operator":
        """``recompress_BF(BF, tau)`` of every far block (``bf_op_recompress``): a new
        operator with lower ranks; this one is unchanged."""
        h = C.c_void_p()
        check(load().bf_op_recompress(self._h, float(tau), C.byref(h)), "bf_op_recompress")
        return Operator(h.value, self.ctx)

    def adjoint_copy(self, trans: int = BF_OP_C) -> "Operator":
        """The reference's materialised ``adjoint(BF)`` (``trans=BF_OP_C``) or
        ``transpose(BF)`` (``BF_OP_T``) of every far block (``bf_op_adjoint_copy``): a new
        operator whose forward product is op(A) x."""
        h = C.c_void_p()
        check(load().bf_op_adjoint_copy(self._h, int(trans), C.byref(h)), "bf_op_adjoint_copy")
        return Operator(h.value, self.ctx)

    def save(self, path: str):
        """Write the operator to ``path`` (``bf_op_save``): packed layout and factors."""
        check(load().bf_op_save(self._h, os.fsencode(path)), "bf_op_save")

    def close(self):
        if self._parent is None and self._h and self._h.value:
            load().bf_op_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_operator(path: str, ctx: Context | None = None) -> Operator:
    """Read an operator written by ``Operator.save`` onto ``ctx``'s device (``bf_op_load``)."""
    ctx = ctx or default_context()
    h = C.c_void_p()
    check(load().bf_op_load(ctx._h, os.fsencode(path), C.byref(h)), "bf_op_load")
    return Operator(h.value, ctx)


def mul(y, A: Operator, x, alpha=1.0, beta=0.0):
    """``mul!(y, A, x, alpha, beta)``: y <- beta*y + alpha*A*x (in place, returns y)."""
    return A.matvec(x, y=y, alpha=alpha, beta=beta)


def compress_block(obs, src, obs_index, src_index, n_rows: int, key: int, k: float, eps: float,
                   ctx: Context | None = None) -> dict:
    """One GPU compression (``bf_compress_block``): one ``PartialQR`` call
    (compressors.jl:81-165) on ``n_rows`` observer points sampled from
    ``obs_index`` by the keyed bijection, against the points ``src_index``."""
    ctx = ctx or default_context()
    obs = np.ascontiguousarray(obs, np.float64)
    src = np.ascontiguousarray(src, np.float64)
    oi = np.ascontiguousarray(obs_index, np.int64)
    si = np.ascontiguousarray(src_index, np.int64)
    m = len(si)
    rows = np.zeros(n_rows, np.int32)
    Z = np.zeros((m, n_rows), np.complex64)  # column-major n_rows x m
    rank = C.c_int32()
    perm = np.zeros(m, np.int32)
    kmax = min(n_rows, m)
    skel = np.zeros(max(kmax, 1), np.int32)
    T = np.zeros(max(kmax * m, 1), np.complex64)
    check(load().bf_compress_block(
        ctx._h, _p(obs, C.c_double), obs.shape[0], _p(src, C.c_double), src.shape[0],
        _p(oi, C.c_int64), len(oi), _p(si, C.c_int64), m, int(n_rows),
        int(key) & ((1 << 64) - 1), float(k), float(eps), _p(rows, C.c_int32),
        Z.ctypes.data_as(C.POINTER(C.c_float)), C.byref(rank), _p(perm, C.c_int32),
        _p(skel, C.c_int32), T.ctypes.data_as(C.POINTER(C.c_float))), "bf_compress_block")
    r = rank.value
    return dict(rows=rows.astype(np.int64), Z=Z.T.copy(), rank=r, perm=perm.astype(np.int64),
                skeleton=skel[:r].astype(np.int64),
                T=T[:r * m].reshape((m, r)).T.copy() if r > 0 else np.zeros((0, m), np.complex64))


def import_blocks(n_rows, n_cols, bf, stage, obs_out, src_out, obs_in, src_in, rows, cols,
                  identity, data_off, data, obs_csr, src_csr, ctx: Context | None = None):
    """Upload reference-style factors (``bf_import_factors``) -> ``Operator``."""
    ctx = ctx or default_context()
    keep = dict(
        bf=np.ascontiguousarray(bf, np.int32), stage=np.ascontiguousarray(stage, np.int32),
        obs_out=np.ascontiguousarray(obs_out, np.int64),
        src_out=np.ascontiguousarray(src_out, np.int64),
        obs_in=np.ascontiguousarray(obs_in, np.int64), src_in=np.ascontiguousarray(src_in, np.int64),
        rows=np.ascontiguousarray(rows, np.int32), cols=np.ascontiguousarray(cols, np.int32),
        identity=np.ascontiguousarray(identity, np.int8),
        data_off=np.ascontiguousarray(data_off, np.int64),
        data=np.ascontiguousarray(data, np.complex128),
        optr=np.ascontiguousarray(obs_csr[0], np.int64), oidx=np.ascontiguousarray(obs_csr[1], np.int64),
        sptr=np.ascontiguousarray(src_csr[0], np.int64), sidx=np.ascontiguousarray(src_csr[1], np.int64))
    d = FactorDesc()
    d.n_rows, d.n_cols, d.n_blocks = int(n_rows), int(n_cols), len(keep["bf"])
    d.bf = _p(keep["bf"], C.c_int32)
    d.stage = _p(keep["stage"], C.c_int32)
    d.obs_out = _p(keep["obs_out"], C.c_int64)
    d.src_out = _p(keep["src_out"], C.c_int64)
    d.obs_in = _p(keep["obs_in"], C.c_int64)
    d.src_in = _p(keep["src_in"], C.c_int64)
    d.rows = _p(keep["rows"], C.c_int32)
    d.cols = _p(keep["cols"], C.c_int32)
    d.identity = _p(keep["identity"], C.c_int8)
    d.data_off = _p(keep["data_off"], C.c_int64)
    d.data = keep["data"].ctypes.data_as(C.POINTER(C.c_double))
    d.n_obs_nodes = len(keep["optr"]) - 1
    d.obs_ptr = _p(keep["optr"], C.c_int64)
    d.obs_idx = _p(keep["oidx"], C.c_int64)
    d.n_src_nodes = len(keep["sptr"]) - 1
    d.src_ptr = _p(keep["sptr"], C.c_int64)
    d.src_idx = _p(keep["sidx"], C.c_int64)
    h = C.c_void_p()
    check(load().bf_import_factors(ctx._h, C.byref(d), C.byref(h)), "bf_import_factors")
    return Operator(h.value, ctx)


class GeometricRankEstimator:
    """``GeometricRankEstimator(C, Cε; Rmin=3)`` (``rankestimation.jl:13-25``, tree method
    ``ext/BFH2Trees/h2rankest.jl:8-38``): sample counts
    ``max(ceil(C (k a_s a_o / d)^2 + Cε log(1/ε)), Rmin)`` from the node radii and the
    center distance.  Pass it as ``rank_estimator`` to ``PetrovGalerkinBF`` /
    ``assemble_BF``; without one the ButterflyRankEstimator(``c_tau``) is used."""

    def __init__(self, C: float = 1.5, Ceps: float = 1.5, Rmin: int = 3):
        self.C, self.Ceps, self.Rmin = float(C), float(Ceps), int(Rmin)


def _build(obs, src, tree_o: Tree, tree_s: Tree, pairs, k, tol, c_tau, adaptive, seed,
           min_samples, rank_mode, surrogate, keep_mixed, ctx, factor_storage=BF_STORE_C32,
           rank_estimator=None):
    lib = load()
    ctx = ctx or default_context()
    obs = np.ascontiguousarray(obs, np.float64)
    src = np.ascontiguousarray(src, np.float64)
    pairs = np.asarray(pairs, np.int64).reshape(-1, 2)
    fo = np.ascontiguousarray(pairs[:, 0])
    fs = np.ascontiguousarray(pairs[:, 1])
    o = BuildOpts()
    lib.bf_build_opts_default(C.byref(o))
    o.c_tau = float(c_tau)
    o.min_samples = int(min_samples)
    o.adaptive = int(bool(adaptive))
    o.seed = int(seed) & ((1 << 64) - 1)
    o.rank_mode = int(rank_mode)
    o.keep_mixed = int(bool(keep_mixed))
    o.factor_storage = int(factor_storage)
    if rank_estimator is not None:
        o.estimator = _lib.BF_EST_GEOMETRIC
        o.geo_c, o.geo_ceps, o.geo_rmin = rank_estimator.C, rank_estimator.Ceps, rank_estimator.Rmin
    w = None
    if surrogate is not None:
        # a bfgpu.surrogate.RankSurrogate (weights + margin) or a bare weight vector
        if hasattr(surrogate, "weights"):
            o.surrogate_margin = float(surrogate.margin)
            surrogate = surrogate.weights
        w = np.ascontiguousarray(surrogate, np.float32)
        o.surrogate_weights = w.ctypes.data_as(C.POINTER(C.c_float))
        o.surrogate_nweights = w.size
    h = C.c_void_p()
    check(lib.bf_build(ctx._h, _p(obs, C.c_double), obs.shape[0], _p(src, C.c_double), src.shape[0],
                       tree_o._h, tree_s._h, _p(fo, C.c_int64), _p(fs, C.c_int64), len(fo),
                       float(k), float(tol), C.byref(o), C.byref(h)), "bf_build")
    return Operator(h.value, ctx)


def assemble_BF(obs, src, tree_o: Tree, tree_s: Tree, no: int, ns: int, k: float, tau: float,
                c_tau: float = 4.0, adaptive: bool = True, seed: int = 0, min_samples: int = 10,
                rank_mode: int = 0, surrogate=None, keep_mixed: bool = True,
                ctx: Context | None = None, factor_storage: int = BF_STORE_C32,
                rank_estimator: GeometricRankEstimator | None = None) -> Operator:
    """``assemble_BF(kernel, blktree, no, ns, k, tau)`` on the GPU (one far block).
    ``factor_storage``: BF_STORE_C32 (complex FP32, 8 B per entry) or BF_STORE_FF
    (float-float, 16 B per entry, the width of the reference's ComplexF64)."""
    return _build(obs, src, tree_o, tree_s, [(no, ns)], k, tau, c_tau, adaptive, seed,
                  min_samples, rank_mode, surrogate, keep_mixed, ctx, factor_storage,
                  rank_estimator)


def PetrovGalerkinBF(obs, src, tree_o: Tree, tree_s: Tree, k: float, tol: float = 1e-3,
                     alpha: float = 1.0, c_tau: float = 2.9592, adaptive: bool = True,
                     seed: int = 0, minbflvl: int = 3, leafcomp: bool = True,
                     min_samples: int = 10, rank_mode: int = 0, surrogate=None,
                     keep_mixed: bool = True, ctx: Context | None = None,
                     factor_storage: int = BF_STORE_C32,
                     farfieldonly: bool = True, leafimbalance: bool = True,
                     unbalancedints: bool = False,
                     rank_estimator: GeometricRankEstimator | None = None) -> Operator:
    """``PetrovGalerkinBF`` on the GPU: the far field (``farfieldonly=True``, the default
    here) or near + far (``farfieldonly=False``, the reference's default; the near blocks
    leave out the singular self-term r = 0).  ``unbalancedints``: the traversal splits only
    the larger node of a pair (``intlists.jl:121-149``)."""
    far, _ = nearandfar(tree_o, tree_s, alpha, minbflvl, leafcomp, leafimbalance,
                        unbalancedints)
    op = _build(obs, src, tree_o, tree_s, far, k, tol, c_tau, adaptive, seed, min_samples,
                rank_mode, surrogate, keep_mixed, ctx, factor_storage, rank_estimator)
    if not farfieldonly:
        op.add_near(obs, src, tree_o, tree_s, k, alpha=alpha, minbflvl=minbflvl,
                    leafcomp=leafcomp, leafimbalance=leafimbalance,
                    unbalancedints=unbalancedints)
    return op
