"""CPU check of the sampled dense far-field rows used as the accuracy yardstick
(bfgpu.verify) against the oracle's dense far-field matrix
(sum over admissible pairs, src/PetrovGalerkin/petrovgalerkinbf.jl:121-151)."""
import math

import numpy as np

import bfgpu
from bfgpu import geometry as G
from bfgpu.verify import far_dense_rows, sample_rows
from oracle import bfref as O


def test_far_dense_rows_match_oracle_dense_far():
    n = 1536
    pts = G.fibonacci_sphere(n)
    k = G.wavenumber(n, 4 * math.pi)
    tr = bfgpu.Tree.build(pts, max_points=24)
    far, _ = bfgpu.nearandfar(tr, tr, 1.0)
    ot = O.build_tree(pts, max_points=24)
    ofar, _ = O.nearandfar(ot, ot, 1.0)
    assert sorted(map(tuple, far.tolist())) == sorted(map(tuple, np.asarray(ofar).tolist()))
    kern = O.HelmholtzKernel(pts, pts, k)
    D = O.dense_far(kern, O.FarOperator([O.BF([], [], [], ot, ot, k, 1e-4, o, s)
                                         for o, s in ofar], ofar, n, n))
    rows = sample_rows(n, 40, seed=3)
    X = G.complex_gaussian(n, 5, nrhs=3)
    Y = far_dense_rows(pts, pts, tr, tr, far, k, rows, X, chunk=16)
    ref = (D @ X)[rows]
    assert np.linalg.norm(Y - ref) <= 1e-12 * np.linalg.norm(ref)
