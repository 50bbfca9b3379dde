"""Allocation-free matvec (bf_matvec_noalloc) against the regular entry point
and against the oracle.

bf_matvec_noalloc serves callers that cannot allocate device memory when they
apply the operator -- a callback that runs while the caller's memory pool is
locked or exhausted, or a real-time loop with a fixed allocation budget: its
level workspace is a fixed 16 MiB device array inside the library, shared by
every call.  The checks: two calls in a row match bf_matvec (1e-12) and the
oracle's products stored in the golden fixtures, for the forward, adjoint and
transpose; operators that take turns on the shared array do not see each
other's leftovers.  This file is collected last so that a run stopping at the
first failure has already run every other test; it also passes on its own in a
fresh process.
"""
import ctypes as C
import os

import numpy as np
import pytest

import bfgpu
from bfgpu import _lib

pytestmark = pytest.mark.gpu
PARITY = 1e-12
HERE = os.path.dirname(os.path.abspath(__file__))


def _golden_operator(name, ctx):
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    op = bfgpu.import_blocks(int(g["n_rows"]), int(g["n_cols"]), g["bf"], g["stage"],
                             g["obs_out"], g["src_out"], g["obs_in"], g["src_in"], g["rows"],
                             g["cols"], g["identity"], g["data_off"], g["data"],
                             (g["obs_ptr"], g["obs_idx"]), (g["src_ptr"], g["src_idx"]), ctx)
    return g, op


def _relerr(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _inputs(g, trans):
    """Right-hand side and the oracle's product for op(A) from a golden fixture.
    The fixture holds y = A x and ya = A^H xa; transpose(A) conj(xa) = conj(ya)."""
    if trans == _lib.BF_OP_N:
        return g["x"], g["y"]
    if trans == _lib.BF_OP_C:
        return g["xa"], g["ya"]
    return np.conj(g["xa"]), np.conj(g["ya"])


def _noalloc(lib, op, trans, x, n_in, n_out):
    import torch
    one = (C.c_double * 2)(1.0, 0.0)
    zero = (C.c_double * 2)(0.0, 0.0)
    # start from garbage: beta = 0 must not read y, and the shared workspace
    # keeps the previous call's contents
    y = torch.full((n_out,), float("nan"), dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    _lib.check(lib.bf_matvec_noalloc(op._h, trans, 1, C.c_void_p(x.data_ptr()), n_in,
                                     C.c_void_p(y.data_ptr()), n_out, one, zero, None),
               "bf_matvec_noalloc")
    _lib.check(lib.bf_op_check(op._h, None), "bf_op_check")
    return y.cpu().numpy()


@pytest.mark.parametrize("name", ["plane_single", "sphere_far"])
@pytest.mark.parametrize("trans", [_lib.BF_OP_N, _lib.BF_OP_C, _lib.BF_OP_T])
def test_noalloc_matches_bf_matvec_twice(ctx, name, trans):
    torch = pytest.importorskip("torch")
    g, op = _golden_operator(name, ctx)
    lib = _lib.load()
    n_in = int(g["n_cols"] if trans == _lib.BF_OP_N else g["n_rows"])
    n_out = int(g["n_rows"] if trans == _lib.BF_OP_N else g["n_cols"])
    xh, oracle_y = _inputs(g, trans)
    x = torch.from_numpy(np.ascontiguousarray(xh)).cuda()
    assert x.numel() == n_in
    one = (C.c_double * 2)(1.0, 0.0)
    zero = (C.c_double * 2)(0.0, 0.0)
    y_ref = torch.zeros(n_out, dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    _lib.check(lib.bf_matvec(op._h, trans, 1, C.c_void_p(x.data_ptr()), n_in,
                             C.c_void_p(y_ref.data_ptr()), n_out, one, zero,
                             _lib.BF_PTR_DEVICE, None), "bf_matvec")
    torch.cuda.synchronize()
    ref = y_ref.cpu().numpy()
    assert _relerr(ref, oracle_y) <= PARITY
    for call in range(2):
        got = _noalloc(lib, op, trans, x, n_in, n_out)
        assert np.all(np.isfinite(got)), call
        assert _relerr(got, ref) <= PARITY, call
        assert _relerr(got, oracle_y) <= PARITY, call


def test_noalloc_operators_take_turns_on_the_shared_array(ctx):
    """A, then B, then A again (and the adjoint of each) through the one shared
    workspace: every result matches its oracle product, so no call reads a slot
    the previous operator left behind."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    ops = {n: _golden_operator(n, ctx) for n in ("plane_single", "sphere_far",
                                                  "plane_unbalanced")}
    order = ["plane_single", "sphere_far", "plane_single", "plane_unbalanced", "sphere_far"]
    for name in order:
        g, op = ops[name]
        for trans in (_lib.BF_OP_N, _lib.BF_OP_C):
            n_in = int(g["n_cols"] if trans == _lib.BF_OP_N else g["n_rows"])
            n_out = int(g["n_rows"] if trans == _lib.BF_OP_N else g["n_cols"])
            xh, oracle_y = _inputs(g, trans)
            x = torch.from_numpy(np.ascontiguousarray(xh)).cuda()
            got = _noalloc(lib, op, trans, x, n_in, n_out)
            assert _relerr(got, oracle_y) <= PARITY, (name, trans)


def test_noalloc_rejects_operators_above_the_limit(ctx):
    import math
    from bfgpu import geometry as G
    n = 16384
    pts = G.fibonacci_sphere(n)
    tree = bfgpu.Tree.build(pts, max_points=32)
    op = bfgpu.PetrovGalerkinBF(pts, pts, tree, tree, G.wavenumber(n, 4 * math.pi), tol=1e-4,
                                ctx=ctx)
    assert op.stats()["workspace_entries"] > (1 << 20)
    torch = pytest.importorskip("torch")
    x = torch.zeros(n, dtype=torch.complex128, device="cuda")
    y = torch.zeros(n, dtype=torch.complex128, device="cuda")
    lib = _lib.load()
    s = lib.bf_matvec_noalloc(op._h, _lib.BF_OP_N, 1, C.c_void_p(x.data_ptr()), n,
                              C.c_void_p(y.data_ptr()), n, None, None, None)
    assert s == _lib.BF_EINVAL
    assert b"at most" in lib.bf_last_error()
