"""ctypes binding of the oracle's C restatement of the far-field matvec.

Test infrastructure only: used by tests/ as a checker and by bench.py's CPU
baseline leg as the timed reference-algorithm port.
"""
import ctypes as C
import os

import numpy as np

from . import build_c

_lib = None


def load():
    global _lib
    if _lib is None:
        path = build_c.LIB
        if not os.path.exists(path):
            path = build_c.build()
        lib = C.CDLL(path)
        vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int32
        lib.bfref_plan_create.restype = vp
        lib.bfref_plan_create.argtypes = [i64, i64, i64] + [vp] * 15
        lib.bfref_plan_destroy.argtypes = [vp]
        lib.bfref_matvec.restype = C.c_int
        lib.bfref_matvec.argtypes = [vp, vp, vp, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_int, i64, i64]
        lib.bfref_plan_nbf.restype = i64
        lib.bfref_plan_nbf.argtypes = [vp]
        _lib = lib
    return _lib


class CRefOperator:
    """Far-field operator on the CPU (reference flat matvec, OpenMP)."""

    def __init__(self, n_rows, n_cols, blocks: dict, obs_csr, src_csr):
        lib = load()
        self._keep = dict(
            bf=np.ascontiguousarray(blocks["bf"], np.int32),
            stage=np.ascontiguousarray(blocks["stage"], np.int32),
            oo=np.ascontiguousarray(blocks["obs_out"], np.int64),
            so=np.ascontiguousarray(blocks["src_out"], np.int64),
            oi=np.ascontiguousarray(blocks["obs_in"], np.int64),
            si=np.ascontiguousarray(blocks["src_in"], np.int64),
            rows=np.ascontiguousarray(blocks["rows"], np.int32),
            cols=np.ascontiguousarray(blocks["cols"], np.int32),
            ident=np.ascontiguousarray(blocks["identity"], np.int8),
            off=np.ascontiguousarray(blocks["data_off"], np.int64),
            data=np.ascontiguousarray(blocks["data"], np.complex128),
            optr=np.ascontiguousarray(obs_csr[0], np.int64),
            oidx=np.ascontiguousarray(obs_csr[1], np.int64),
            sptr=np.ascontiguousarray(src_csr[0], np.int64),
            sidx=np.ascontiguousarray(src_csr[1], np.int64))
        k = self._keep
        self.n_rows, self.n_cols = int(n_rows), int(n_cols)
        args = [k[n].ctypes.data for n in ["bf", "stage", "oo", "so", "oi", "si", "rows", "cols",
                                           "ident", "off", "data", "optr", "oidx", "sptr",
                                           "sidx"]]
        self._h = lib.bfref_plan_create(self.n_rows, self.n_cols, len(k["bf"]), *args)
        if not self._h:
            raise ValueError("malformed factor description")
        self.n_bf = lib.bfref_plan_nbf(self._h)

    def matvec(self, x, y=None, alpha=1.0, beta=0.0, nthreads=0, bf_begin=0, bf_end=-1):
        x = np.ascontiguousarray(x, np.complex128)
        if y is None:
            y = np.zeros(self.n_rows, np.complex128)
            beta = 0.0
        a, b = complex(alpha), complex(beta)
        s = load().bfref_matvec(self._h, x.ctypes.data, y.ctypes.data, a.real, a.imag, b.real,
                                b.imag, int(nthreads), int(bf_begin), int(bf_end))
        if s != 0:
            raise RuntimeError(f"bfref_matvec failed ({s})")
        return y

    def __del__(self):
        try:
            if self._h:
                load().bfref_plan_destroy(self._h)
        except Exception:
            pass
