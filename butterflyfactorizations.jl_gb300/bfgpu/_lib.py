"""ctypes binding of libbfgpu.so (the C ABI declared in include/bfgpu.h)."""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbfgpu.so")

BF_OK, BF_EINVAL, BF_ENOMEM, BF_ECUDA, BF_ETIMEOUT, BF_ENOTSUP, BF_ESTATE = range(7)
BF_OP_N, BF_OP_C, BF_OP_T = 0, 1, 2
BF_EST_BUTTERFLY, BF_EST_GEOMETRIC = 0, 1
BF_PTR_HOST, BF_PTR_DEVICE = 0, 1
BF_STORE_C32, BF_STORE_FF = 0, 1
RANK_REC_LEN = 18  # BF_RANK_REC_LEN
SUR_NW = 4553      # rank-surrogate weight count (bf_surrogate_nweights)

i32, i64, u64, f64, vp = C.c_int32, C.c_int64, C.c_uint64, C.c_double, C.c_void_p
P = C.POINTER


class BuildOpts(C.Structure):
    _fields_ = [("c_tau", f64), ("min_samples", i32), ("adaptive", i32), ("seed", u64),
                ("rank_mode", i32), ("keep_mixed", i32), ("surrogate_weights", P(C.c_float)),
                ("surrogate_nweights", i64), ("surrogate_margin", f64),
                ("factor_storage", i32), ("estimator", i32), ("geo_rmin", i32),
                ("geo_c", f64), ("geo_ceps", f64)]


class TrainOpts(C.Structure):
    _fields_ = [("epochs", i32), ("batch", i32), ("lr", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("eps", C.c_float), ("seed", u64)]


class FactorDesc(C.Structure):
    _fields_ = [("n_rows", i64), ("n_cols", i64), ("n_blocks", i64), ("bf", P(i32)),
                ("stage", P(i32)), ("obs_out", P(i64)), ("src_out", P(i64)), ("obs_in", P(i64)),
                ("src_in", P(i64)), ("rows", P(i32)), ("cols", P(i32)), ("identity", P(C.c_int8)),
                ("data_off", P(i64)), ("data", P(f64)), ("n_obs_nodes", i64),
                ("obs_ptr", P(i64)), ("obs_idx", P(i64)), ("n_src_nodes", i64),
                ("src_ptr", P(i64)), ("src_idx", P(i64))]


class OpStats(C.Structure):
    _fields_ = [("n_bf", i64), ("n_stages", i64), ("n_tasks", i64), ("factor_entries", i64),
                ("factor_bytes", i64), ("workspace_entries", i64), ("map_entries", i64),
                ("alg_bytes_fwd", i64), ("max_rank", i64), ("build_seconds", f64),
                ("compressions", i64), ("retries", i64), ("kernel_entries", i64),
                ("build_compress_seconds", f64), ("build_pack_seconds", f64),
                ("build_upload_seconds", f64), ("surrogate_fallbacks", i64),
                ("near_pairs", i64), ("near_entries", i64), ("near_bytes_fwd", i64)]


# (name, restype, argtypes): every function declared in include/bfgpu.h
SIGNATURES = [
    ("bf_version", C.c_int, []),
    ("bf_status_string", C.c_char_p, [C.c_int]),
    ("bf_last_error", C.c_char_p, []),
    ("bf_ctx_create", C.c_int, [C.c_int, P(vp)]),
    ("bf_ctx_destroy", C.c_int, [vp]),
    ("bf_tree_build", C.c_int, [P(f64), i64, i32, i32, P(vp)]),
    ("bf_tree_from_arrays", C.c_int, [i64, i64, P(f64), P(f64), P(i32), P(i32), P(i32), P(i64),
                                      P(i64), P(i64), P(vp)]),
    ("bf_tree_size", C.c_int, [vp, P(i64), P(i64), P(i32)]),
    ("bf_tree_export", C.c_int, [vp, P(f64), P(f64), P(i32), P(i32), P(i32), P(i32), P(i64),
                                 P(i64), P(i64)]),
    ("bf_tree_destroy", C.c_int, [vp]),
    ("bf_nearandfar", C.c_int, [vp, vp, f64, i32, i32, i32, i32, P(i64), P(i64), i64, P(i64),
                                P(i64)]),
    ("bf_near_pairs", C.c_int, [vp, vp, f64, i32, i32, i32, i32, P(i64), P(i64), i64, P(i64)]),
    ("bf_tree_build_gpu", C.c_int, [vp, P(f64), i64, i32, i32, P(vp)]),
    ("bf_nearandfar_gpu", C.c_int, [vp, vp, vp, f64, i32, i32, i32, i32, P(i64), P(i64), i64, P(i64),
                                    P(i64), i64, P(i64), P(i64)]),
    ("bf_build_opts_default", None, [P(BuildOpts)]),
    ("bf_train_opts_default", None, [P(TrainOpts)]),
    ("bf_surrogate_nweights", C.c_int, []),
    ("bf_surrogate_init", C.c_int, [P(C.c_float), i64, u64, P(C.c_float)]),
    ("bf_surrogate_grad", C.c_int, [vp, P(C.c_float), P(C.c_float), P(C.c_float), i64,
                                    P(C.c_float), P(C.c_float)]),
    ("bf_surrogate_train", C.c_int, [vp, P(C.c_float), P(C.c_float), i64, P(TrainOpts),
                                     P(C.c_float), P(C.c_float)]),
    ("bf_surrogate_predict", C.c_int, [vp, P(C.c_float), P(C.c_float), i64, P(C.c_float)]),
    ("bf_build", C.c_int, [vp, P(f64), i64, P(f64), i64, vp, vp, P(i64), P(i64), i64, f64, f64,
                           P(BuildOpts), P(vp)]),
    ("bf_compress_block", C.c_int, [vp, P(f64), i64, P(f64), i64, P(i64), i32, P(i64), i32, i32,
                                    u64, f64, f64, P(i32), P(C.c_float), P(i32), P(i32), P(i32),
                                    P(C.c_float)]),
    ("bf_op_add_near", C.c_int, [vp, P(f64), i64, P(f64), i64, vp, vp, P(i64), P(i64), i64,
                                 f64]),
    ("bf_import_factors", C.c_int, [vp, P(FactorDesc), P(vp)]),
    ("bf_matvec", C.c_int, [vp, C.c_int, i64, vp, i64, vp, i64, P(f64), P(f64), C.c_int, vp]),
    ("bf_matvec_mixed", C.c_int, [vp, C.c_int, i64, vp, i64, vp, i64, P(f64), P(f64), C.c_int,
                                  vp]),
    ("bf_matvec_noalloc", C.c_int, [vp, C.c_int, i64, vp, i64, vp, i64, P(f64), P(f64), vp]),
    ("bf_op_check", C.c_int, [vp, vp]),
    ("bf_op_set_wait_limit", C.c_int, [vp, i64]),
    ("bf_op_size", C.c_int, [vp, P(i64), P(i64)]),
    ("bf_op_stats_get", C.c_int, [vp, P(OpStats)]),
    ("bf_op_export_blocks", C.c_int, [vp, i64, i64, P(i64), P(i64), P(i32), P(i32), P(i64),
                                      P(i64), P(i64), P(i64), P(i32), P(i32), P(C.c_int8),
                                      P(i64), vp, i32]),
    ("bf_op_rank_log", C.c_int, [vp, P(i64), P(f64)]),
    ("bf_op_profile", C.c_int, [vp, C.c_int, i32, P(f64), P(i64), P(i64)]),
    ("bf_op_profile_mixed", C.c_int, [vp, C.c_int, i32, P(f64), P(i64), P(f64), P(i64)]),
    ("bf_op_mixed_info", C.c_int, [vp, P(i64), P(i64), P(i64)]),
    ("bf_op_task_shapes", C.c_int, [vp, P(i64), P(i32), P(i32), P(i32), P(i32)]),
    ("bf_op_recompress", C.c_int, [vp, f64, P(vp)]),
    ("bf_op_adjoint_copy", C.c_int, [vp, C.c_int, P(vp)]),
    ("bf_op_save", C.c_int, [vp, C.c_char_p]),
    ("bf_op_load", C.c_int, [vp, C.c_char_p, P(vp)]),
    ("bf_op_destroy", C.c_int, [vp]),
    ("bf_batch_create", C.c_int, [vp, P(vp), P(i32), i32, i32, P(vp)]),
    ("bf_batch_create_op", C.c_int, [vp, P(vp), P(i32), P(i32), i32, i32, P(vp)]),
    ("bf_batch_buffers", C.c_int, [vp, i32, P(vp), P(vp)]),
    ("bf_batch_run", C.c_int, [vp, vp]),
    ("bf_batch_matvec", C.c_int, [vp, P(vp), P(i64), P(vp), P(i64), C.c_int, vp]),
    ("bf_batch_autotune", C.c_int, [vp, i32, P(f64), P(i32)]),
    ("bf_batch_info", C.c_int, [vp, P(i64), P(i64), P(i64), P(i32)]),
    ("bf_batch_destroy", C.c_int, [vp]),
]

_lib = None


def load():
    """Load libbfgpu.so; raises if the extension has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libbfgpu.so not built at {LIB_PATH}; run build_ext.py "
                          "(there is no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class BFError(RuntimeError):
    def __init__(self, status: int, what: str):
        lib = load()
        msg = lib.bf_last_error().decode(errors="replace")
        name = lib.bf_status_string(status).decode()
        super().__init__(f"{what}: {name}: {msg}")
        self.status = status


def check(status: int, what: str):
    if status != BF_OK:
        raise BFError(status, what)
