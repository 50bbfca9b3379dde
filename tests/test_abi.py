"""CPU tests of the C ABI: the library loads, exports every declared symbol, and
its host-side tree / interaction-list code agrees exactly with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import bfgpu
from bfgpu import _lib
from bfgpu import geometry as G
from oracle import bfref as O

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "bfgpu.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"BF_API\s+[\w\s\*]+?\b(bf_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    # the ctypes signature table covers the header exactly
    assert sorted(s[0] for s in _lib.SIGNATURES) == names


def test_status_strings_and_errors():
    lib = _lib.load()
    assert lib.bf_status_string(_lib.BF_EINVAL) == b"BF_EINVAL"
    h = C.c_void_p()
    s = lib.bf_tree_build(None, 0, 8, -1, C.byref(h))
    assert s == _lib.BF_EINVAL
    assert b"empty" in lib.bf_last_error()
    with pytest.raises(bfgpu.BFError):
        bfgpu.Tree.build(np.zeros((0, 3)))


def test_no_cpu_fallback_without_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(bfgpu.BFError) as e:
        bfgpu.Context(0)
    assert e.value.status == _lib.BF_ECUDA


@pytest.mark.parametrize("case", ["sphere", "plane", "cube", "ellipsoid"])
def test_tree_bit_exact_with_oracle(case):
    if case == "sphere":
        pts, kw = G.fibonacci_sphere(20000), dict(max_points=32)
    elif case == "plane":
        pts, kw = G.plane_pair(4096, 1)[0], dict(max_depth=4)
    elif case == "cube":
        pts, kw = G.cube_surface(5000, 3), dict(max_points=20)
    else:
        pts, kw = G.fibonacci_sphere(8000, (1.0, 0.5, 0.25)), dict(max_points=16)
    a = O.build_tree(pts, **kw)
    b = bfgpu.Tree.build(pts, **kw)
    for f in ["center", "halfsize", "level", "parent", "first_child", "n_child", "begin", "end",
              "perm"]:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    far, near = O.nearandfar(a, a, 1.0)
    fo, nn = bfgpu.nearandfar(b, b, 1.0)
    assert nn == len(near)
    assert np.array_equal(np.asarray(far, np.int64).reshape(-1, 2), fo)
    assert np.array_equal(np.asarray(near, np.int64).reshape(-1, 2), bfgpu.near_pairs(b, b, 1.0))


@pytest.mark.parametrize("opts", [dict(leafcomp=False), dict(leafimbalance=False),
                                  dict(minbflvl=2, leafcomp=False), dict(unbalancedints=True),
                                  dict(unbalancedints=True, leafimbalance=False)])
def test_near_and_far_lists_options(opts):
    """Near and far pairs of the dual traversal under the non-default options
    (intlists.jl:30-217), unbalanced trees: bit-exact with the oracle."""
    obs, src = G.plane_pair(3000, 7, z_obs=0.2)
    a_o, a_s = O.build_tree(obs, max_points=12), O.build_tree(src, max_points=60)
    b_o, b_s = bfgpu.Tree.build(obs, max_points=12), bfgpu.Tree.build(src, max_points=60)
    far, near = O.nearandfar(a_o, a_s, 1.0, **opts)
    fo, nn = bfgpu.nearandfar(b_o, b_s, 1.0, **opts)
    assert np.array_equal(np.asarray(far, np.int64).reshape(-1, 2), fo)
    assert np.array_equal(np.asarray(near, np.int64).reshape(-1, 2),
                          bfgpu.near_pairs(b_o, b_s, 1.0, **opts))
    assert nn == len(near) > 0


def test_tree_from_arrays_roundtrip():
    pts = G.cube_surface(2000, 5)
    b = bfgpu.Tree.build(pts, max_points=16)
    lib = _lib.load()
    h = C.c_void_p()
    p = lambda a, t: a.ctypes.data_as(C.POINTER(t))
    _lib.check(lib.bf_tree_from_arrays(b.n_nodes, len(b.perm), p(b.center, C.c_double),
                                       p(b.halfsize, C.c_double), p(b.parent, C.c_int32),
                                       p(b.first_child, C.c_int32), p(b.n_child, C.c_int32),
                                       p(b.begin, C.c_int64), p(b.end, C.c_int64),
                                       p(b.perm, C.c_int64), C.byref(h)), "from_arrays")
    c = bfgpu.Tree(h.value)
    for f in ["center", "halfsize", "level", "first_child", "n_child", "begin", "end", "perm"]:
        assert np.array_equal(getattr(b, f), getattr(c, f)), f
    bad = b.perm.copy()
    bad[0] = len(bad) + 5
    s = lib.bf_tree_from_arrays(b.n_nodes, len(b.perm), p(b.center, C.c_double),
                                p(b.halfsize, C.c_double), p(b.parent, C.c_int32),
                                p(b.first_child, C.c_int32), p(b.n_child, C.c_int32),
                                p(b.begin, C.c_int64), p(b.end, C.c_int64), p(bad, C.c_int64),
                                C.byref(h))
    assert s == _lib.BF_EINVAL
