"""Generate the golden fixtures under tests/golden/ from the CPU oracle.

Each fixture holds one operator's factors in the C-ABI block layout
(bf_factor_desc), the node->values maps, a seeded right-hand side and the
oracle's forward and adjoint products.  Regenerate with
``python tests/golden/make_golden.py`` (deterministic).
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "butterflyfactorizations.jl_gb300"), os.path.dirname(HERE)]

from bfgpu import geometry as G  # noqa: E402
from oracle import bfref as O  # noqa: E402
from _util import oracle_blocks, tree_csr  # noqa: E402

CASES = {
    # name: (kind, params)
    "plane_single": dict(kind="plane", n=512, seed=11, z=4.0, lam=0.25, depth=3, tol=1e-4),
    "plane_unbalanced": dict(kind="plane_unb", n=600, seed=12, z=2.5, lam=0.25, tol=1e-4),
    "sphere_far": dict(kind="sphere", n=400, max_points=12, tol=1e-4),
}


def build(name):
    c = CASES[name]
    if c["kind"] == "plane":
        obs, src = G.plane_pair(c["n"], c["seed"], c["z"])
        k = 2 * math.pi / c["lam"]
        to = O.build_tree(obs, max_depth=c["depth"])
        ts = O.build_tree(src, max_depth=c["depth"])
        kern = O.HelmholtzKernel(obs, src, k)
        bfs = [O.assemble_bf(kern, to, ts, 0, 0, k, c["tol"], c_tau=4.0, seed=1)]
        far = O.FarOperator(bfs, [(0, 0)], c["n"], c["n"])
    elif c["kind"] == "plane_unb":
        obs, src = G.plane_pair(c["n"], c["seed"], c["z"])
        k = 2 * math.pi / c["lam"]
        to = O.build_tree(obs, max_points=10)
        ts = O.build_tree(src, max_points=120)
        kern = O.HelmholtzKernel(obs, src, k)
        bfs = [O.assemble_bf(kern, to, ts, 0, 0, k, c["tol"], seed=2)]
        far = O.FarOperator(bfs, [(0, 0)], c["n"], c["n"])
    else:
        pts = G.fibonacci_sphere(c["n"])
        k = G.wavenumber(c["n"], 4 * math.pi)
        to = ts = O.build_tree(pts, max_points=c["max_points"])
        kern = O.HelmholtzKernel(pts, pts, k)
        far = O.assemble_far(kern, to, ts, k, c["tol"])
    return far, to, ts


def main():
    for name in CASES:
        far, to, ts = build(name)
        d = oracle_blocks(far.bfs)
        x = G.complex_gaussian(far.n_cols, 100)
        xa = G.complex_gaussian(far.n_rows, 101)
        y = O.far_matvec(far, x)
        ya = O.far_matvec(far, xa, adjoint=True)
        optr, oidx = tree_csr(to)
        sptr, sidx = tree_csr(ts)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), n_rows=far.n_rows,
                            n_cols=far.n_cols, obs_ptr=optr, obs_idx=oidx, src_ptr=sptr,
                            src_idx=sidx, x=x, y=y, xa=xa, ya=ya, **d)
        print(name, "blocks", len(d["bf"]), "entries", d["data"].size)


if __name__ == "__main__":
    main()
