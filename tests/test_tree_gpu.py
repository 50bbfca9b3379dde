"""Trees and interaction lists built on the GPU (bf_tree_build_gpu,
bf_nearandfar_gpu) against the host versions, which the CPU tests pin to the
oracle: every tree array and every far / near pair, in order, must be equal.
Geometries: spheres (up to 262,144 points), the plane pair at depth 4, a cube
surface, an ellipsoid and an unbalanced plane pair under the non-default
traversal options."""
import numpy as np
import pytest

import bfgpu
from bfgpu import geometry as G

pytestmark = pytest.mark.gpu
FIELDS = ["center", "halfsize", "level", "parent", "first_child", "n_child", "begin", "end",
          "perm"]


def same_tree(a, b):
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


@pytest.mark.parametrize("case", ["sphere", "sphere262k", "plane", "cube", "ellipsoid"])
def test_gpu_tree_and_lists_equal_host(ctx, case):
    if case == "sphere":
        pts, kw = G.fibonacci_sphere(20000), dict(max_points=32)
    elif case == "sphere262k":
        pts, kw = G.fibonacci_sphere(262144), dict(max_points=32)
    elif case == "plane":
        pts, kw = G.plane_pair(4096, 1)[0], dict(max_depth=4)
    elif case == "cube":
        pts, kw = G.cube_surface(5000, 3), dict(max_points=20)
    else:
        pts, kw = G.fibonacci_sphere(8000, (1.0, 0.5, 0.25)), dict(max_points=16)
    host = bfgpu.Tree.build(pts, **kw)
    dev = bfgpu.Tree.build_gpu(pts, ctx=ctx, **kw)
    same_tree(host, dev)
    far_h, _ = bfgpu.nearandfar(host, host, 1.0)
    near_h = bfgpu.near_pairs(host, host, 1.0)
    far_d, near_d = bfgpu.nearandfar_gpu(dev, dev, 1.0, ctx=ctx)
    assert np.array_equal(far_h, far_d)
    assert np.array_equal(near_h, near_d)


@pytest.mark.parametrize("opts", [dict(), dict(leafcomp=False), dict(leafimbalance=False),
                                  dict(minbflvl=2, leafcomp=False), dict(alpha=2.0),
                                  dict(unbalancedints=True)])
def test_gpu_lists_unbalanced_trees(ctx, opts):
    obs, src = G.plane_pair(3000, 7, z_obs=0.2)
    to, ts = bfgpu.Tree.build(obs, max_points=12), bfgpu.Tree.build(src, max_points=60)
    same_tree(to, bfgpu.Tree.build_gpu(obs, max_points=12, ctx=ctx))
    same_tree(ts, bfgpu.Tree.build_gpu(src, max_points=60, ctx=ctx))
    alpha = opts.pop("alpha", 1.0)
    far_h, _ = bfgpu.nearandfar(to, ts, alpha, **opts)
    near_h = bfgpu.near_pairs(to, ts, alpha, **opts)
    far_d, near_d = bfgpu.nearandfar_gpu(to, ts, alpha, ctx=ctx, **opts)
    assert np.array_equal(far_h, far_d)
    assert np.array_equal(near_h, near_d)


def test_gpu_tree_rejects_bad_points(ctx):
    pts = G.fibonacci_sphere(1000)
    pts[17, 1] = np.nan
    with pytest.raises(bfgpu.BFError) as e:
        bfgpu.Tree.build_gpu(pts, max_points=32, ctx=ctx)
    assert e.value.status == bfgpu._lib.BF_EINVAL
