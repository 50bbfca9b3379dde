"""Many operators, many right-hand sides, one CUDA-graph launch (bf_batch_*)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import BF_PTR_DEVICE, BF_PTR_HOST, check, load


class Batch:
    """FP64-accurate matvecs of several operators in one launch sequence.

    ``ops`` are ``bfgpu.Operator`` objects or their ``adjoint()`` / ``transpose()``
    views (same factor storage); ``nrhs[i]`` right-hand sides for operator i.
    ``matvec(xs)`` takes a list of (n_i, nrhs_i) complex128 arrays and returns
    the list of products.
    """

    def __init__(self, ops, nrhs, ctx, rhs_chunk: int = 8):
        lib = load()
        self.ops = list(ops)           # keeps the operators alive
        self.nrhs = [int(r) for r in nrhs]
        self.ctx = ctx
        hs = (C.c_void_p * len(self.ops))(*[o._h.value for o in self.ops])
        tr = (C.c_int32 * len(self.ops))(*[int(o.trans) for o in self.ops])
        nr = (C.c_int32 * len(self.nrhs))(*self.nrhs)
        h = C.c_void_p()
        check(lib.bf_batch_create_op(ctx._h, hs, tr, nr, len(self.ops), int(rhs_chunk),
                                     C.byref(h)), "bf_batch_create_op")
        self._h = h

    def buffers(self, i: int):
        x, y = C.c_void_p(), C.c_void_p()
        check(load().bf_batch_buffers(self._h, int(i), C.byref(x), C.byref(y)), "bf_batch_buffers")
        return x.value, y.value

    def run(self, stream: int = 0):
        check(load().bf_batch_run(self._h, C.c_void_p(stream) if stream else None), "bf_batch_run")

    def matvec(self, xs):
        lib = load()
        X = [np.asfortranarray(np.asarray(x, np.complex128).reshape(x.shape[0], -1)) for x in xs]
        Y = [np.zeros((o.shape[0], r), np.complex128, order="F") for o, r in zip(self.ops, self.nrhs)]
        for x, o, r in zip(X, self.ops, self.nrhs):
            if x.shape != (o.shape[1], r):
                raise ValueError(f"x has shape {x.shape}, expected {(o.shape[1], r)}")
        n = len(X)
        xp = (C.c_void_p * n)(*[x.ctypes.data for x in X])
        yp = (C.c_void_p * n)(*[y.ctypes.data for y in Y])
        check(lib.bf_batch_matvec(self._h, xp, None, yp, None, BF_PTR_HOST, None),
              "bf_batch_matvec")
        return Y

    def autotune(self, nrep: int = 3):
        ms = C.c_double()
        cfg = (C.c_int32 * 3)()
        check(load().bf_batch_autotune(self._h, int(nrep), C.byref(ms), cfg), "bf_batch_autotune")
        return ms.value, dict(nr_max=cfg[0], order=cfg[1], ctas_per_sm=cfg[2])

    def info(self) -> dict:
        g, w, b = C.c_int64(), C.c_int64(), C.c_int64()
        ch = C.c_int32()
        check(load().bf_batch_info(self._h, C.byref(g), C.byref(w), C.byref(b), C.byref(ch)),
              "bf_batch_info")
        return dict(graph_nodes=g.value, work_items=w.value, workspace_bytes=b.value,
                    rhs_chunks=ch.value)

    def close(self):
        if self._h and self._h.value:
            load().bf_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["Batch", "BF_PTR_DEVICE", "BF_PTR_HOST"]
