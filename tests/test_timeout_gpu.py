"""Bounded device-side waits that run out are reported, not swallowed.

The plain path's bulk-copy level kernel (the P stage of a built sphere
operator) waits on shared-memory barriers with a bounded poll count.
``bf_op_set_wait_limit(op, 0)`` makes every such wait give up at once; the
kernel then records the error, lets the copies it has issued land and
returns.  The library must report BF_ETIMEOUT -- a host-pointer call from the
call itself, a device-pointer call from ``bf_op_check`` or from the next call
on the handle -- and once the default limit is back, the next matvec must
succeed and match the CPU restatement of the reference matvec on the same
factors.
"""
import ctypes as C
import math

import numpy as np
import pytest

import bfgpu
from bfgpu import _lib
from bfgpu import geometry as G
from oracle.cbind import CRefOperator

pytestmark = pytest.mark.gpu
PARITY = 1e-12
N = 16384


@pytest.fixture(scope="module")
def sphere(ctx):
    pts = G.fibonacci_sphere(N)
    tree = bfgpu.Tree.build(pts, max_points=32)
    op = bfgpu.PetrovGalerkinBF(pts, pts, tree, tree, G.wavenumber(N, 4 * math.pi), tol=1e-4,
                                ctx=ctx)
    csr = tree.values_csr()
    cref = CRefOperator(N, N, op.export_blocks(), csr, csr)
    x = G.complex_gaussian(N, 7)
    return dict(op=op, cref=cref, x=x, ref=cref.matvec(x))


def _relerr(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_p_stage_uses_the_bulk_copy_kernel(sphere):
    # the last level holds short wide tasks (M <= 32, n >= 128): the bulk-copy pipeline
    stage, kind, M, n = sphere["op"].task_shapes()
    last = stage == stage.max()
    assert np.any((kind[last] == 0) & (M[last] <= 32) & (n[last] >= 128))


def test_host_call_reports_timeout_then_recovers(sphere):
    op, x = sphere["op"], sphere["x"]
    assert _relerr(op @ x, sphere["ref"]) <= PARITY
    op.set_wait_limit(0)
    try:
        with pytest.raises(bfgpu.BFError) as e:
            op @ x
        assert e.value.status == _lib.BF_ETIMEOUT
        assert "gave up" in str(e.value)
    finally:
        op.set_wait_limit(-1)
    # the error was collected by the failing call: the next one runs clean
    assert _relerr(op @ x, sphere["ref"]) <= PARITY
    op.check()


def test_device_call_reports_timeout_through_check_and_next_call(sphere):
    torch = pytest.importorskip("torch")
    op, x = sphere["op"], sphere["x"]
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros_like(xd)
    torch.cuda.synchronize()
    op.set_wait_limit(0)
    try:
        # asynchronous: returns before the kernels ran
        op.matvec_device(xd.data_ptr(), N, yd.data_ptr(), N)
        with pytest.raises(bfgpu.BFError) as e:
            op.check()
        assert e.value.status == _lib.BF_ETIMEOUT
        op.check()  # collected once
        op.matvec_device(xd.data_ptr(), N, yd.data_ptr(), N)
        torch.cuda.synchronize()
        # not collected by a check: the next call reports it and does no work
        lib = _lib.load()
        one = (C.c_double * 2)(1.0, 0.0)
        s = lib.bf_matvec(op._h, _lib.BF_OP_N, 1, C.c_void_p(xd.data_ptr()), N,
                          C.c_void_p(yd.data_ptr()), N, one, None, _lib.BF_PTR_DEVICE, None)
        assert s == _lib.BF_ETIMEOUT
    finally:
        op.set_wait_limit(-1)
    op.matvec_device(xd.data_ptr(), N, yd.data_ptr(), N)
    op.check()
    assert _relerr(yd.cpu().numpy(), sphere["ref"]) <= PARITY


def test_timeout_does_not_leak_into_the_mixed_path(sphere):
    op, x = sphere["op"], sphere["x"]
    op.set_wait_limit(0)
    try:
        with pytest.raises(bfgpu.BFError):
            op @ x
    finally:
        op.set_wait_limit(-1)
    # the tensor-core path shares the device error word; it must start clean
    X = G.complex_gaussian(N, 8, nrhs=2)
    Y = op.matvec(X, mixed=True)
    R = np.stack([sphere["cref"].matvec(np.ascontiguousarray(X[:, j])) for j in range(2)], 1)
    assert _relerr(Y, R) <= 1e-4
