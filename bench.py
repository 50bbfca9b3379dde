#!/usr/bin/env python
"""Far-field butterfly matvec throughput on GB300.

Default workload (one GPU): the plain FP64 far-field operator of a
262,144-point Fibonacci sphere at ~100 points per wavelength^2 (k ~ 90.8),
octree with <= 32 points per leaf, isFar(alpha=1) admissibility, tol 1e-4,
one complex Gaussian right-hand side.  Factors are built on the GPU by
bf_build before timing and stored as float-float entries (16 bytes per complex
entry, the width of the reference's ComplexF64 factors); a step is one forward
far-field matvec over all far blocks.  The factor stream (~67 GB) is far
larger than L2, so no explicit L2 flush is needed between steps.

The same run measures
  * the batched mixed-precision path on the same operator: 256 right-hand
    sides (128 plane waves exp(-ik d.x) + 128 complex Gaussians) per step
    through bf_matvec_mixed, its error against the FP64 GPU matvec and against
    FP64 dense far-field rows on 2,048 seeded rows (bfgpu.verify);
  * the CPU restatement of the reference matvec on a bounded sample of the far
    blocks, and the GPU matvec on the same sample (parity on identical factors);
  * the same operator with complex FP32 factor storage (8 bytes per entry, an
    extra key: half the bytes, exact for the build's FP32 values).
``--workload sphere65k`` is the 65,536-point sphere (k ~ 45.4, 256 dense rows).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--storage ff|c32] [--no-mixed] [--no-cpu]

N > 1 runs independent replicas (one per rank, launched by torch.distributed.run);
the path has no cross-GPU exchange on a single operator.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "butterflyfactorizations.jl_gb300")]

import numpy as np  # noqa: E402

METRIC = "far-field matvecs/s & HBM GB/s: plain FP64 vs batched mixed, rel.err≤1e-4"
UNIT = "matvec/s"

WORKLOADS = {
    # name: (n points, max points per leaf, tol)
    "sphere262k": (262144, 32, 1e-4),
    "sphere65k": (65536, 32, 1e-4),
    "sphere16k": (16384, 32, 1e-4),
    "sphere4k": (4096, 32, 1e-4),
}
DENSE_ROWS = {"sphere262k": 2048}  # sampled dense rows per workload (default 256)
BATCH = {"batch32": 32, "batch4": 4}  # operator-batch workloads: number of operators
SURROGATE = {"surrogate524k": 524288}  # held-out ellipsoid size of the surrogate study
ROWS = {"rows": "GPU trees and lists (262,144-point sphere), persisted operator (65,536-point "
                "sphere), recompression of one far block (plane pairs of 16,384 and 65,536 points)"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload",
                    choices=sorted(WORKLOADS) + sorted(BATCH) + sorted(SURROGATE) + sorted(ROWS),
                    default="sphere262k")
    ap.add_argument("--storage", choices=["ff", "c32"], default="ff",
                    help="factor storage of the headline operator: float-float (16 B per "
                         "entry) or complex FP32 (8 B)")
    ap.add_argument("--no-c32", action="store_true",
                    help="skip the extra complex-FP32-storage leg")
    ap.add_argument("--no-near", action="store_true",
                    help="skip the near + far (full operator) leg")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision leg")
    ap.add_argument("--mixed-rhs", type=int, default=256)
    ap.add_argument("--mixed-steps", type=int, default=5)
    ap.add_argument("--ncu-case", action="store_true",
                    help="no timing: build, then 2 plain forward matvecs and 2 mixed forward "
                         "128-RHS chunks (a short, predictable launch sequence for ncu)")
    ap.add_argument("--ncu-adjoint", action="store_true",
                    help="with --ncu-case: the plain matvecs through the adjoint view")
    ap.add_argument("--ncu-near", action="store_true",
                    help="with --ncu-case: attach the near field first, so that the plain "
                         "matvecs apply near + far")
    return ap.parse_args()


def batch_operators(count, seed, ctx, storage="c32"):
    """Seeded mix of spheres, ellipsoids (1, 0.5, 0.25) and cube surfaces; N log-uniform in
    [8192, 131072] at ~100 points per wavelength^2; 1-64 right-hand sides each."""
    import bfgpu
    from bfgpu import geometry as G
    rng = np.random.default_rng(seed)
    shapes = ["sphere", "ellipsoid", "cube"]
    out = []
    for i in range(count):
        shape = shapes[int(rng.integers(0, 3))]
        n = int(round(math.exp(rng.uniform(math.log(8192), math.log(131072)))))
        nrhs = int(rng.integers(1, 65))
        pts, area = G.shape_points(shape, n, seed=int(rng.integers(0, 1 << 30)))
        k = G.wavenumber(n, area)
        tree = bfgpu.Tree.build(pts, max_points=32)
        op = bfgpu.PetrovGalerkinBF(pts, pts, tree, tree, k, tol=1e-4, ctx=ctx,
                                    factor_storage=STORAGE[storage])
        out.append(dict(shape=shape, n=n, nrhs=nrhs, k=k, pts=pts, tree=tree, op=op))
    return out


def run_batch(args, rank, world, local):
    """Operator batch: all operators and right-hand sides in one CUDA-graph launch."""
    import torch
    import bfgpu
    from bfgpu import geometry as G
    from bfgpu.batch import Batch
    torch.cuda.set_device(local)
    ctx = bfgpu.Context(local)
    t0 = time.perf_counter()
    # complex FP32 factors: the 32 operators' float-float factors do not fit in one
    # GPU's memory next to the batch workspace
    storage = "c32"
    ops = batch_operators(BATCH[args.workload], seed=3 + rank, ctx=ctx, storage=storage)
    build_s = time.perf_counter() - t0
    nrhs = [o["nrhs"] for o in ops]
    total_rhs = sum(nrhs)
    b = Batch([o["op"] for o in ops], nrhs, ctx, rhs_chunk=8)
    t0 = time.perf_counter()
    tune_ms, cfg = b.autotune(nrep=2)
    tune_s = time.perf_counter() - t0
    xs = [G.complex_gaussian(o["n"], 100 + i, nrhs=o["nrhs"]) for i, o in enumerate(ops)]
    # inputs resident: copy once into the batch buffers, then time graph replays
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ys = b.matvec(xs)  # copies in, one run, copies out (also the accuracy sample)
    for _ in range(max(args.warmup, 3)):
        b.run(stream.cuda_stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = ClockSampler(local)
    clk.start()
    b.run(stream.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        b.run(stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world)
    # unbatched: the reference's structure, one bf_matvec per operator and column
    # (bfmatrix.jl:10-75 applies each operator column by column), device pointers
    xd = [torch.from_numpy(np.ascontiguousarray(x.T)).cuda() for x in xs]
    yd = [torch.zeros_like(x) for x in xd]

    def unbatched():
        for o, x, y in zip(ops, xd, yd):
            for c in range(o["nrhs"]):
                o["op"].matvec_ptr(x[c].data_ptr(), o["n"], y[c].data_ptr(), o["n"], nrhs=1,
                                   ptr_mode=bfgpu.BF_PTR_DEVICE, stream=stream.cuda_stream)
    unbatched()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(max(1, args.steps // 4)):
        unbatched()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_unb = e0.elapsed_time(e1) / max(1, args.steps // 4)
    err = max(float(np.linalg.norm(ys[i] - yd[i].cpu().numpy().T) / np.linalg.norm(ys[i]))
              for i in range(len(ops)))
    # e2e: host buffers through bf_batch_matvec (copies inside the timed region)
    t0 = time.perf_counter()
    for _ in range(3):
        b.matvec(xs)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / 3, world)
    info = b.info()
    line = {
        "metric": METRIC, "value": world * total_rhs * 1000.0 / ms, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": f"f64 (float-float vectors and sums on FP32 pipes; {STORAGE_NAME[storage]})",
        "data": "synthetic",
        "config": {"workload": f"{args.workload}: {len(ops)} operators (seeded mix of spheres, "
                               f"ellipsoids 1/0.5/0.25, cube surfaces), N log-uniform in "
                               f"[8192, 131072], ~100 points per wavelength^2, tol 1e-4, "
                               f"1-64 complex Gaussian RHS each ({total_rhs} in total)",
                   "operators": [{"shape": o["shape"], "n": o["n"], "nrhs": o["nrhs"]}
                                 for o in ops],
                   "parallelism": f"replicas x{world}", "rhs_chunk": 8,
                   "l2": "no flush: factor streams per step >> L2",
                   "build_seconds_total": round(build_s, 2),
                   "autotune": {"seconds": round(tune_s, 2), "best_ms": tune_ms, **cfg}},
        "graph": info,
        "unbatched": {"value": world * total_rhs * 1000.0 / ms_unb, "unit": UNIT,
                      "ms_per_step": ms_unb,
                      "what": "one bf_matvec per operator and column, same device buffers"},
        "max_rel_diff_vs_unbatched": err,
        "e2e": {"value": world * total_rhs / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": int(sum(16 * o["n"] * o["nrhs"] for o in ops)),
                "d2h_bytes_per_step": int(sum(16 * o["n"] * o["nrhs"] for o in ops))},
        "gpu_launches": int(info["graph_nodes"] * args.steps),
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu:
        try:
            from oracle.cbind import CRefOperator
            threads = os.cpu_count() or 1
            sample = sorted(range(len(ops)), key=lambda i: ops[i]["n"])[:4]
            crefs = []
            for i in sample:
                csr = ops[i]["tree"].values_csr()
                crefs.append((i, CRefOperator(ops[i]["n"], ops[i]["n"],
                                              ops[i]["op"].export_blocks(), csr, csr)))
            cnt = 0
            t0 = time.perf_counter()
            for i, cref in crefs:
                for j in range(ops[i]["nrhs"]):
                    cref.matvec(np.ascontiguousarray(xs[i][:, j]), nthreads=threads)
                    cnt += 1
            dt = time.perf_counter() - t0
            line["cpu_baseline"] = {
                "value": cnt / dt, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"the 4 smallest operators of the batch, all their RHS ({cnt} "
                          f"matvecs), C port of the reference flat matvec, {threads} threads"}
        except Exception as e:  # report, do not fail the GPU measurement
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 0, "kind": "port",
                                    "sample": f"failed: {e}"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_surrogate(args, rank, world, local):
    """Learned rank surrogate: records from builds of the single-block, sphere and batch
    geometries train the MLP on the GPU; the held-out ellipsoid is built with the
    oversampling estimator and with the surrogate (construction time, sampled work,
    fallbacks, accuracy against FP64 dense far-field rows)."""
    import torch
    import bfgpu
    from bfgpu import geometry as G
    from bfgpu.surrogate import RankSurrogate, features_targets
    from bfgpu.verify import far_dense_rows, sample_rows
    torch.cuda.set_device(local)
    ctx = bfgpu.Context(local)
    t0 = time.perf_counter()
    recs = []
    # single block: two parallel unit squares 4 apart, k = 2 pi / 0.125, quadtree depth 4
    obs, src = G.plane_pair(4096, seed=1)
    to, ts = bfgpu.Tree.build(obs, max_depth=4), bfgpu.Tree.build(src, max_depth=4)
    op = bfgpu.assemble_BF(obs, src, to, ts, 0, 0, 2 * math.pi / 0.125, 1e-4, c_tau=4.0,
                           seed=3, ctx=ctx)
    recs.append(op.rank_log())
    del op
    # full far field of the 65,536-point sphere
    pts = G.fibonacci_sphere(65536)
    tr = bfgpu.Tree.build(pts, max_points=32)
    op = bfgpu.PetrovGalerkinBF(pts, pts, tr, tr, G.wavenumber(65536, 4 * math.pi), tol=1e-4,
                                ctx=ctx)
    recs.append(op.rank_log())
    del op
    # eight operators of the seeded batch mix
    for o in batch_operators(8, seed=3, ctx=ctx):
        recs.append(o["op"].rank_log())
        del o
    rec = np.concatenate(recs)
    n_all = len(rec)
    rng = np.random.default_rng(5)
    if n_all > 1_000_000:
        rec = rec[np.sort(rng.choice(n_all, 1_000_000, replace=False))]
    records_s = time.perf_counter() - t0
    F, T = features_targets(rec)
    t0 = time.perf_counter()
    model, hist = RankSurrogate.train(F, T, ctx, epochs=20, batch=4096, lr=3e-3, seed=7)
    train_s = time.perf_counter() - t0
    margin = model.calibrate_margin(F, T, ctx, quantile=0.98)
    # held-out geometry
    n = SURROGATE[args.workload]
    pts, area = G.shape_points("ellipsoid", n, seed=11)
    k = G.wavenumber(n, area)
    tr = bfgpu.Tree.build(pts, max_points=32)
    far, _ = bfgpu.nearandfar(tr, tr, 1.0)
    rows = sample_rows(n, 256, seed=13)
    x = G.complex_gaussian(n, 17)
    ref = far_dense_rows(pts, pts, tr, tr, far, k, rows, x)[:, 0]
    out = {}
    for name, sur in (("oversampling", None), ("surrogate", model)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op = bfgpu.PetrovGalerkinBF(pts, pts, tr, tr, k, tol=1e-4, ctx=ctx,
                                    rank_mode=0 if sur is None else 1, surrogate=sur)
        wall = time.perf_counter() - t0
        s = op.stats()
        y = op @ x
        out[name] = {"build_seconds": round(wall, 3),
                     "compress_seconds": round(s["build_compress_seconds"], 3),
                     "pack_seconds": round(s["build_pack_seconds"], 3),
                     "compressions": s["compressions"], "retries": s["retries"],
                     "surrogate_fallbacks": s["surrogate_fallbacks"],
                     "kernel_entries": s["kernel_entries"],
                     "rel_err_vs_dense_rows": float(np.linalg.norm(y[rows] - ref) /
                                                    np.linalg.norm(ref))}
        del op
    p, q = out["oversampling"], out["surrogate"]
    line = {
        "metric": "construction seconds (surrogate-seeded vs oversampling) at the same residual",
        "value": q["build_seconds"], "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 0,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "construction: FP32 with FP64 k.r reduction and QR norms/pivots; MLP bf16 "
                 "weights, fp32 accumulation",
        "data": "synthetic",
        "config": {"workload": f"{args.workload}: held-out ellipsoid (1, 0.5, 0.25), N={n}, "
                               f"k={k:.1f} (~100 points per wavelength^2), tol 1e-4; "
                               f"training records from the 4,096-point plane pair, the "
                               f"65,536-point sphere and 8 operators of the batch mix",
                   "records_total": int(n_all), "records_used": int(len(rec)),
                   "records_seconds": round(records_s, 1), "train_seconds": round(train_s, 2),
                   "epochs": 20, "final_loss": float(hist[-1]), "margin": margin,
                   "dense_rows": 256},
        "oversampling": p, "surrogate": q,
        "speedup": p["build_seconds"] / q["build_seconds"],
        "compress_speedup": p["compress_seconds"] / max(q["compress_seconds"], 1e-9),
        "kernel_entry_ratio": q["kernel_entries"] / max(p["kernel_entries"], 1),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def _median_time(fn, reps=3, warmup=1):
    """Median wall time of fn() over reps calls after warmup calls (fn synchronises)."""
    for _ in range(warmup):
        fn()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts)


def run_rows(args, rank, world, local):
    """The widening rows next to the matvec, each timed beside its CPU counterpart:
    cluster tree + near/far lists (GPU vs the host C++ versions, which restate
    bisection_tree.jl / intlists.jl), a persisted operator (write and read back), and
    butterfly recompression of one far block (GPU vs the oracle's restatement of
    recompress_BF on the same blocks)."""
    import tempfile as _tf
    import torch
    import bfgpu
    from bfgpu import geometry as G
    from oracle import bfref as O
    torch.cuda.set_device(local)
    if rank != 0:
        return
    ctx = bfgpu.Context(local)
    line = {"metric": "GPU tree + near/far lists, 262,144-point sphere (ms)", "unit": "ms",
            "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
            "config": {"workload": ROWS[args.workload]}}
    # trees and lists (the call a user makes: points in, host arrays out)
    n = 262144
    pts = G.fibonacci_sphere(n)
    t_host = _median_time(lambda: bfgpu.Tree.build(pts, max_points=32))
    t_gpu = _median_time(lambda: bfgpu.Tree.build_gpu(pts, max_points=32, ctx=ctx))
    th, tg = bfgpu.Tree.build(pts, max_points=32), bfgpu.Tree.build_gpu(pts, max_points=32, ctx=ctx)
    same_tree = all(np.array_equal(getattr(th, k), getattr(tg, k)) for k in
                    ("center", "halfsize", "level", "parent", "first_child", "n_child", "perm",
                     "begin", "end"))

    def host_lists():
        far, _ = bfgpu.nearandfar(th, th)
        return far, bfgpu.near_pairs(th, th)
    l_host = _median_time(host_lists)
    l_gpu = _median_time(lambda: bfgpu.nearandfar_gpu(th, th, ctx=ctx))
    fh, nh = host_lists()
    fg, ng = bfgpu.nearandfar_gpu(th, th, ctx=ctx)
    line["value"] = 1e3 * (t_gpu + l_gpu)
    line["trees_lists"] = {
        "tree_ms": {"gpu": 1e3 * t_gpu, "host": 1e3 * t_host}, "identical_tree": bool(same_tree),
        "lists_ms": {"gpu": 1e3 * l_gpu, "host": 1e3 * l_host},
        "identical_lists": bool(np.array_equal(fh, fg) and np.array_equal(nh, ng)),
        "far_pairs": int(len(fg)), "near_pairs": int(len(ng)),
        "host_threads": os.cpu_count(),
        "what": "host: bf_tree_build + bf_nearandfar + bf_near_pairs (each list call counts, "
                "then fills); gpu: bf_tree_build_gpu + bf_nearandfar_gpu"}
    # persisted operator: the 65,536-point sphere's far field, complex FP32 factors
    n2 = 65536
    p2 = G.fibonacci_sphere(n2)
    t2 = bfgpu.Tree.build(p2, max_points=32)
    op = bfgpu.PetrovGalerkinBF(p2, p2, t2, t2, G.wavenumber(n2, 4 * math.pi), tol=1e-4, ctx=ctx)
    x = G.complex_gaussian(n2, 3)
    y0 = op.matvec(x)
    with _tf.TemporaryDirectory() as d:
        path = os.path.join(d, "sphere65k.bfop")
        t0 = time.perf_counter()
        op.save(path)
        t_save = time.perf_counter() - t0
        size = os.path.getsize(path)
        t0 = time.perf_counter()
        back = bfgpu.load_operator(path, ctx)
        t_load = time.perf_counter() - t0
        same = bool(np.array_equal(back.matvec(x), y0))
        del back
    # materialised adjoint of the same operator against its adjoint view
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros_like(xd)
    stream = torch.cuda.Stream()
    t0 = time.perf_counter()
    cop = op.adjoint_copy()
    t_copy = time.perf_counter() - t0
    ms_view = time_plain(op.adjoint(), xd, yd, n2, stream, 10, 3)
    ms_copy = time_plain(cop, xd, yd, n2, stream, 10, 3)
    ya = op.adjoint().matvec(x)
    line["adjoint_copy"] = {
        "operator": "sphere65k far field, complex FP32 factors", "copy_s": t_copy,
        "adjoint_view_ms": ms_view, "copy_forward_ms": ms_copy, "speedup": ms_view / ms_copy,
        "rel_diff": float(np.linalg.norm(cop.matvec(x) - ya) / np.linalg.norm(ya))}
    del cop
    line["persisted"] = {"operator": "sphere65k far field, complex FP32 factors",
                         "file_bytes": int(size), "save_s": t_save, "load_s": t_load,
                         "save_gbs": size / t_save / 1e9, "load_gbs": size / t_load / 1e9,
                         "bit_identical_matvec": same,
                         "load_checks": "chunk hashes, every offset and length, pair alignment"}
    del op
    # recompression of one far block (two parallel unit squares 4 apart)
    rec = {}
    for npl, depth, lam, with_cpu in ((16384, 5, 0.0625, True), (65536, 6, 0.03125, False)):
        obs, src = G.plane_pair(npl, seed=1)
        to, ts = bfgpu.Tree.build(obs, max_depth=depth), bfgpu.Tree.build(src, max_depth=depth)
        op = bfgpu.assemble_BF(obs, src, to, ts, 0, 0, 2 * math.pi / lam, 1e-4, c_tau=4.0,
                               seed=3, ctx=ctx)
        e0 = op.stats()["factor_entries"]
        r = {"points": npl, "quadtree_depth": depth, "wavelength": lam, "tol_build": 1e-4,
             "tau": 1e-2, "r_levels": int(op.stats()["n_stages"]) - 2}
        holder = {}

        def gpu_rc():
            holder["op"] = op.recompress(1e-2)
            torch.cuda.synchronize()
        r["gpu_s"] = _median_time(gpu_rc)
        rop = holder["op"]
        xs = G.complex_gaussian(npl, 4)
        ya = op.matvec(xs)
        r["factor_entries"] = {"built": int(e0), "recompressed": int(rop.stats()["factor_entries"])}
        r["rel_diff_vs_built"] = float(np.linalg.norm(rop.matvec(xs) - ya) / np.linalg.norm(ya))
        if with_cpu:
            bfs = O.from_blocks(op.export_blocks(), O.CsrTree(*to.values_csr()),
                                O.CsrTree(*ts.values_csr()))
            # CPU baseline and checker: the oracle's restatement of recompress_BF on the
            # same exported blocks (outside any GPU timing)
            t0 = time.perf_counter()
            rbs = [O.recompress_bf(bf, 1e-2) for bf in bfs]
            r["cpu_baseline"] = {"value": time.perf_counter() - t0, "unit": "s", "cores": 1,
                                 "kind": "port",
                                 "sample": "the whole far block: recompress_BF restated in "
                                           "NumPy/SciPy (LAPACK pivoted QR)"}
            r["factor_entries"]["oracle"] = int(sum(O.factor_entries(b) for b in rbs))
            yo = O.apply_far(rbs, xs, npl)
            r["rel_diff_vs_oracle"] = float(np.linalg.norm(rop.matvec(xs) - yo) / np.linalg.norm(yo))
        rec[f"plane{npl // 1024}k"] = r
        del op, rop
    line["recompression"] = rec
    print(json.dumps(line), flush=True)


def run_ncu_case(args, local):
    import torch
    import bfgpu
    from bfgpu import geometry as G
    torch.cuda.set_device(local)
    if args.workload in BATCH:  # build the batch, replay its graph twice
        from bfgpu.batch import Batch
        ctx = bfgpu.Context(local)
        ops = batch_operators(BATCH[args.workload], seed=3, ctx=ctx)
        b = Batch([o["op"] for o in ops], [o["nrhs"] for o in ops], ctx, rhs_chunk=8)
        b.run()
        b.run()
        print(json.dumps({"ncu_case": args.workload, **b.info()}), flush=True)
        return
    w = build_workload(args.workload, local, args.storage)
    op, n = w["op"], w["n"]
    if args.ncu_near:
        op.add_near(w["pts"], w["pts"], w["tree"], w["tree"], w["k"])
    view = op.adjoint() if args.ncu_adjoint else op
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    xd = torch.from_numpy(w["x"]).cuda()
    yd = torch.zeros_like(xd)
    for _ in range(2):
        view.matvec_ptr(xd.data_ptr(), n, yd.data_ptr(), n, ptr_mode=bfgpu.BF_PTR_DEVICE,
                        stream=sp)
    torch.cuda.synchronize()
    view.check(sp)
    out = {"ncu_case": args.workload, "levels": op.stats()["n_stages"],
           "direction": "adjoint" if args.ncu_adjoint else "forward",
           # algorithmic bytes per level (its launches come after the two matvecs)
           "stage_bytes": [int(v) for v in view.profile(nrep=1)[1]]}
    if not args.no_mixed:
        op.mixed_info()
        X = np.ascontiguousarray(G.complex_gaussian(n, 12, nrhs=128).T)
        xm = torch.from_numpy(X).cuda()
        ym = torch.zeros_like(xm)
        for _ in range(2):
            op.matvec_ptr(xm.data_ptr(), n, ym.data_ptr(), n, nrhs=128,
                          ptr_mode=bfgpu.BF_PTR_DEVICE, stream=sp, mixed=True)
        torch.cuda.synchronize()
    print(json.dumps(out), flush=True)


def dist_setup(n_gpus, backend="nccl"):
    """Rank, world size and local rank from the torchrun environment; one process group
    for the barrier and the max over ranks (NCCL on the GPUs; gloo for the CPU tests)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


STORAGE = {"ff": 1, "c32": 0}  # bfgpu.BF_STORE_FF / BF_STORE_C32
STORAGE_NAME = {"ff": "float-float factors, 16 B per complex entry (the width of ComplexF64)",
                "c32": "complex FP32 factors, 8 B per complex entry (exact for the build)"}


def workload_config(name, w):
    return (f"{name}: Fibonacci sphere N={w['n']}, k={w['k']:.2f}, octree<=32/leaf, isFar(1.0), "
            f"tol={w['tol']}, 1 complex Gaussian RHS")


def geometry(name):
    import bfgpu
    from bfgpu import geometry as G
    n, leaf, tol = WORKLOADS[name]
    pts = G.fibonacci_sphere(n)
    k = G.wavenumber(n, 4.0 * math.pi)
    tree = bfgpu.Tree.build(pts, max_points=leaf)
    far, n_near = bfgpu.nearandfar(tree, tree, 1.0)
    x = G.complex_gaussian(n, 1234)
    return dict(pts=pts, k=k, tree=tree, far=far, n_near=n_near, x=x, n=n, tol=tol)


def build_op(w, ctx, storage):
    import bfgpu
    t0 = time.perf_counter()
    op = bfgpu.PetrovGalerkinBF(w["pts"], w["pts"], w["tree"], w["tree"], w["k"], tol=w["tol"],
                                ctx=ctx, factor_storage=STORAGE[storage])
    return op, time.perf_counter() - t0


def build_workload(name, device, storage="ff"):
    import bfgpu
    w = geometry(name)
    w["ctx"] = bfgpu.Context(device)
    w["op"], w["build_s"] = build_op(w, w["ctx"], storage)
    w["storage"] = storage
    return w


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks(key="hbm_gbs"):
    fallback = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p[key]), "measured"
    except (OSError, KeyError, ValueError):
        return fallback[key], "fallback"


def run_mixed(args, w, stream, world):
    """256-RHS tensor-core matvecs through bf_matvec_mixed: throughput, accuracy, roofline."""
    import torch
    import bfgpu
    from bfgpu import geometry as G
    from bfgpu.verify import far_dense_rows, sample_rows
    op, n, sp = w["op"], w["n"], stream.cuda_stream
    nr = args.mixed_rhs
    X = np.asfortranarray(np.concatenate(
        [G.plane_waves(w["pts"], w["k"], nr // 2, seed=11),
         G.complex_gaussian(n, 12, nrhs=nr - nr // 2)], axis=1))
    xd = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()  # column j contiguous
    yd = torch.zeros_like(xd)
    t0 = time.perf_counter()
    info = op.mixed_info()  # packs the BF16 factors on first use
    setup_s = time.perf_counter() - t0

    def timed(view, steps):
        def step():
            view.matvec_ptr(xd.data_ptr(), n, yd.data_ptr(), n, nrhs=nr,
                            ptr_mode=bfgpu.BF_PTR_DEVICE, stream=sp, mixed=True)
        for _ in range(3):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    ms_adj = timed(op.adjoint(), max(2, args.mixed_steps // 2))
    ms = timed(op, args.mixed_steps)
    ms = max_over_ranks(ms, world)
    Y = yd.cpu().numpy().T  # forward result of the last timed step
    # FP64 GPU matvec on 8 columns (4 plane waves, 4 Gaussians)
    cols = [0, 1, 2, 3, nr - 4, nr - 3, nr - 2, nr - 1]
    x8 = xd[cols].contiguous()
    y8 = torch.zeros_like(x8)
    op.matvec_ptr(x8.data_ptr(), n, y8.data_ptr(), n, nrhs=8, ptr_mode=bfgpu.BF_PTR_DEVICE,
                  stream=sp)
    torch.cuda.synchronize()
    Y8 = y8.cpu().numpy().T
    err64 = max(float(np.linalg.norm(Y[:, c] - Y8[:, i]) / np.linalg.norm(Y8[:, i]))
                for i, c in enumerate(cols))
    # FP64 dense far-field rows on a seeded sample, all right-hand sides (rank 0 only:
    # the replicas hold the same operator, and the host work is a minute at 262k)
    rows = sample_rows(n, DENSE_ROWS.get(args.workload, 256), seed=2048)
    lead = world <= 1 or torch.distributed.get_rank() == 0
    err_dense = err_dense_col = err_dense_64 = None
    dense_s = 0.0
    if lead:
        t0 = time.perf_counter()
        R = far_dense_rows(w["pts"], w["pts"], w["tree"], w["tree"], w["far"], w["k"], rows, X)
        dense_s = time.perf_counter() - t0
        err_dense = float(np.linalg.norm(Y[rows] - R) / np.linalg.norm(R))
        err_dense_col = float(max(np.linalg.norm(Y[rows, j] - R[:, j]) / np.linalg.norm(R[:, j])
                                  for j in range(nr)))
        err_dense_64 = float(np.linalg.norm(Y8[rows] - R[:, cols]) / np.linalg.norm(R[:, cols]))
    # e2e: pinned host X and Y, copies inside the call
    xh = torch.from_numpy(np.ascontiguousarray(X.T)).pin_memory()
    yh = torch.zeros_like(xh).pin_memory()
    op.matvec_ptr(xh.data_ptr(), n, yh.data_ptr(), n, nrhs=nr, ptr_mode=bfgpu.BF_PTR_HOST,
                  mixed=True)
    t0 = time.perf_counter()
    e2e_steps = max(2, args.mixed_steps // 2)
    for _ in range(e2e_steps):
        op.matvec_ptr(xh.data_ptr(), n, yh.data_ptr(), n, nrhs=nr, ptr_mode=bfgpu.BF_PTR_HOST,
                      mixed=True)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_s = max_over_ranks(e2e_s, world)
    # per-level roofline (one 128-RHS chunk, CUDA events in the library)
    sms, sby, sfl, nk = op.profile_mixed(nrep=2)
    dom = int(np.argmax(sms))
    hbm, hbm_kind = peaks("hbm_gbs")
    tc, tc_kind = peaks("bf16_tflops")
    ach_gbs = float(sby[dom] / (sms[dom] * 1e-3) / 1e9)
    useful_tf = float(sfl[dom] / (sms[dom] * 1e-3) / 1e12)
    tot_bytes = float(sby.sum()) * math.ceil(nr / 128)
    return {
        "value": world * nr * 1000.0 / ms, "unit": UNIT, "rhs_per_step": nr,
        "ms_per_step": ms, "dtype": "bf16 hi/lo x3 on tcgen05, fp32 accumulate",
        "rhs": f"{nr // 2} plane waves exp(-ik d.x) + {nr - nr // 2} complex Gaussians",
        "rel_err_vs_fp64_gpu": err64,
        "rel_err_vs_dense_rows": err_dense, "max_col_rel_err_vs_dense_rows": err_dense_col,
        "fp64_rel_err_vs_dense_rows": err_dense_64, "dense_rows": int(len(rows)),
        "dense_rows_seconds": round(dense_s, 2),
        "adjoint": {"value": world * nr * 1000.0 / ms_adj, "unit": UNIT, "ms_per_step": ms_adj},
        "hbm_gbs": tot_bytes / (ms * 1e-3) / 1e9,
        "e2e": {"value": world * nr / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 16 * n * nr,
                "d2h_bytes_per_step": 16 * n * nr},
        "roofline": {"bound": "hbm", "achieved": ach_gbs, "peak": hbm, "unit": "GB/s",
                     "frac": ach_gbs / hbm, "peak_source": f"{hbm_kind} hbm_gbs",
                     "traffic": scaled_traffic("mixed", dom, len(sms), sby[dom]),
                     "traffic_source": TRAFFIC_SOURCE,
                     "kernel": f"mx_level_kernel, level {dom} of {len(sms)}, one 128-RHS chunk, "
                               f"{sms[dom]:.3f} ms",
                     "tensor_useful_tflops": useful_tf,
                     "tensor_pipe_tflops": 3.0 * useful_tf,
                     "tensor_peak_tflops": tc, "tensor_peak_source": f"{tc_kind} bf16_tflops",
                     "tensor_pipe_frac": 3.0 * useful_tf / tc,
                     "stage_ms": [round(float(v), 4) for v in sms],
                     "stage_bytes": [int(v) for v in sby],
                     "stage_useful_tflop": [round(float(v) / 1e12, 4) for v in sfl]},
        "factor_bytes_bf16": info["factor_bytes"], "workspace_bytes": info["workspace_bytes"],
        "work_units": info["work_units"], "setup_seconds": round(setup_s, 2),
        "gpu_launches": int(nk * math.ceil(nr / 128) * args.mixed_steps),
    }


# DRAM bytes per level launch over the level's algorithmic bytes, by path and
# level kind, measured with ncu (dram__bytes_read.sum + dram__bytes_write.sum)
# on the 16,384-point sphere (a capture small enough for a multi-pass ncu
# run).  Traffic grows with the algorithmic bytes (every factor entry and slot
# is moved once), so a level's traffic at another size is this ratio times its
# algorithmic bytes.  The R ratio is the one of the largest R level.
TRAFFIC_RATIO = {"plain_c32": {"Q": 0.979, "R": 0.990, "P": 1.002},
                 "plain_ff": {"Q": 1.013, "R": 1.006, "P": 1.001},
                 "mixed": {"Q": 0.975, "R": 0.982, "P": 1.000}}
TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum per level launch at 16,384 "
                  "points, as a ratio to the level's algorithmic bytes, times this level's "
                  "algorithmic bytes")


def level_kind(dom, n_levels):
    return "Q" if dom == 0 else "P" if dom == n_levels - 1 else "R"


def scaled_traffic(path, dom, n_levels, alg_bytes):
    """DRAM bytes per launch of level dom, scaled from the 16k-point capture (None when
    that path has no capture)."""
    r = TRAFFIC_RATIO.get(path)
    if r is None:
        return None
    return int(round(r[level_kind(dom, n_levels)] * float(alg_bytes)))


# CPU sample: the far blocks [0, bf_end) whose ComplexF64 factors come to about
# this many bytes (host memory and export time stay bounded at any size)
CPU_SAMPLE_BYTES = 6 << 30
CPU_SAMPLE_SECONDS = 10.0


def cpu_sample(w, ctx):
    """A contiguous prefix of the far blocks (depth-first far-pair order) with about
    CPU_SAMPLE_BYTES of ComplexF64 factors: the exported blocks, the C port of the
    reference matvec on them, and the same blocks imported back as a GPU operator."""
    import bfgpu
    from oracle.cbind import CRefOperator
    op = w["op"]
    n_bf = op.stats()["n_bf"]
    lib = bfgpu.load()
    nb, nd = ctypes.c_int64(), ctypes.c_int64()

    def data_bytes(end):
        bfgpu.check(lib.bf_op_export_blocks(op._h, 0, end, ctypes.byref(nb), ctypes.byref(nd),
                                            *([None] * 11), 0), "export query")
        return 16 * nd.value

    total = data_bytes(n_bf)
    lo, hi = 1, n_bf
    if total > CPU_SAMPLE_BYTES:
        while lo < hi:  # smallest prefix reaching the byte budget
            mid = (lo + hi) // 2
            if data_bytes(mid) >= CPU_SAMPLE_BYTES:
                hi = mid
            else:
                lo = mid + 1
        end = lo
    else:
        end = n_bf
    ex = op.export_blocks(0, end)
    csr = w["tree"].values_csr()
    cref = CRefOperator(w["n"], w["n"], ex, csr, csr)
    sub = bfgpu.import_blocks(w["n"], w["n"], ex["bf"], ex["stage"], ex["obs_out"],
                              ex["src_out"], ex["obs_in"], ex["src_in"], ex["rows"], ex["cols"],
                              ex["identity"], ex["data_off"], ex["data"], csr, csr, ctx)
    sample_bytes = data_bytes(end)
    del ex
    return dict(cref=cref, sub=sub, bf_end=end, n_bf=n_bf, frac=sample_bytes / total,
                sample_bytes=sample_bytes, total_bytes=total)


def time_cpu(cs, x, seconds=CPU_SAMPLE_SECONDS, warmup=1, min_reps=3):
    """Median time of the C port over the sample, repeated for about `seconds`."""
    threads = os.cpu_count() or 1
    y = np.zeros(len(x), np.complex128)
    for _ in range(max(warmup, 1)):
        cs["cref"].matvec(x, y, nthreads=threads)
    ts = []
    t_end = time.perf_counter() + seconds
    while len(ts) < min_reps or time.perf_counter() < t_end:
        t0 = time.perf_counter()
        cs["cref"].matvec(x, y, nthreads=threads)
        ts.append(time.perf_counter() - t0)
        if len(ts) >= 1000:
            break
    return statistics.median(ts), len(ts), threads, y


def sample_text(cs, reps, threads):
    return (f"far blocks 0..{cs['bf_end'] - 1} of {cs['n_bf']} (a depth-first prefix; "
            f"{cs['sample_bytes'] / 1e9:.2f} GB of ComplexF64 factors = {100 * cs['frac']:.1f}% "
            f"of the operator's factor bytes), median of {reps} matvecs, {threads} OpenMP "
            f"threads; matvecs/s scaled to the whole operator by the factor-byte fraction")


def cpu_baseline(w, ctx):
    """Reference flat matvec (oracle C port, OpenMP) on a bounded sample of the same
    factors, and parity of the GPU matvec on that sample (imported, identical factors)."""
    import torch
    cs = cpu_sample(w, ctx)
    t, reps, threads, ycpu = time_cpu(cs, w["x"])
    ygpu = cs["sub"] @ w["x"]
    torch.cuda.synchronize()
    parity = float(np.linalg.norm(ygpu - ycpu) / np.linalg.norm(ycpu))
    cb = dict(value=cs["frac"] / t, unit=UNIT, cores=threads, kind="port",
              sample=sample_text(cs, reps, threads))
    return cb, parity, cs["bf_end"]


def run_reference(args, rank, world, local):
    if rank != 0:
        return
    if args.workload in BATCH:
        print(json.dumps({"impl": "reference", "unavailable":
                          "operator batches have no reference counterpart; the batch line's "
                          "cpu_baseline times the reference flat matvec on a sample of it"}))
        return
    import torch
    torch.cuda.set_device(local)
    w = build_workload(args.workload, local, args.storage)
    cs = cpu_sample(w, w["ctx"])
    threads = os.cpu_count() or 1
    x = w["x"]
    y = np.zeros(w["n"], np.complex128)
    for _ in range(args.warmup):
        cs["cref"].matvec(x, y, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cs["cref"].matvec(x, y, nthreads=threads)
    dt = (time.perf_counter() - t0) / args.steps
    v = cs["frac"] / dt  # whole-operator matvecs/s
    st = w["op"].stats()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": workload_config(args.workload, w), "global_batch": 1,
                   "n_far": st["n_bf"], "parallelism": "cpu-openmp"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "each step: the C restatement of bfvector.jl:200-296 + "
                                   "matrixvector.jl:8-65 over " +
                                   sample_text(cs, args.steps, threads) +
                                   "; factors built by bf_build, exported as ComplexF64"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_plain(op, xd, yd, n, stream, steps, warmup):
    """CUDA-event time per forward (or adjoint view) matvec on device pointers."""
    import torch
    import bfgpu
    sp = stream.cuda_stream

    def step():
        op.matvec_ptr(xd.data_ptr(), n, yd.data_ptr(), n, ptr_mode=bfgpu.BF_PTR_DEVICE, stream=sp)

    for _ in range(max(warmup, 3)):
        step()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    op.check(sp)
    return e0.elapsed_time(e1) / steps


def plain_roofline(op, storage):
    """Dominant level launch: algorithmic bytes over its CUDA-event time (inside the
    library, on the operator's stream), and the whole-matvec rate from the same pass."""
    stage_ms, stage_bytes, kernels = op.profile(nrep=5)
    dom = int(np.argmax(stage_ms))
    achieved = stage_bytes[dom] / (stage_ms[dom] * 1e-3) / 1e9
    peak, peak_kind = peaks()
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak,
            "traffic": scaled_traffic(f"plain_{storage}", dom, len(stage_ms), stage_bytes[dom]),
            "traffic_source": TRAFFIC_SOURCE,
            "kernel": f"level launch {dom} of {len(stage_ms)} "
                      f"({level_kind(dom, len(stage_ms))} stage), {stage_ms[dom]:.3f} ms",
            "peak_source": f"{peak_kind} hbm_gbs",
            "whole_matvec_gbs": float(stage_bytes.sum() / (stage_ms.sum() * 1e-3) / 1e9),
            "whole_matvec_frac": float(stage_bytes.sum() / (stage_ms.sum() * 1e-3) / 1e9 / peak),
            "stage_ms": [round(float(v), 4) for v in stage_ms],
            "stage_bytes": [int(v) for v in stage_bytes]}, kernels


def run_ours(args, rank, world, local):
    import gc
    import torch
    import bfgpu
    from bfgpu import geometry as G
    torch.cuda.set_device(local)
    w = build_workload(args.workload, local, args.storage)
    op = w["op"]
    n = w["n"]
    st = op.stats()
    # a dedicated stream: the legacy default stream has handle 0, which the C ABI
    # reads as "use the operator's own stream"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    xd = torch.from_numpy(w["x"]).to(f"cuda:{local}")
    yd = torch.zeros_like(xd)

    def step():
        op.matvec_ptr(xd.data_ptr(), n, yd.data_ptr(), n, ptr_mode=bfgpu.BF_PTR_DEVICE, stream=sp)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    for _ in range(2):  # bring clocks back up after the sampler's start-up pause
        step()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    clocks = clk.stop()
    op.check(sp)  # no bounded device wait gave up during the timed steps
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ms, world)
    value = world * 1000.0 / ms
    y = yd.cpu().numpy()

    # adjoint throughput (same timing method)
    opa = op.adjoint()
    ms_adj = time_plain(opa, xd, yd, n, stream, args.steps, 3)

    # e2e through the public C ABI with pinned host buffers (copies inside the call)
    xh = torch.from_numpy(w["x"]).pin_memory()
    yh = torch.zeros_like(xh).pin_memory()
    for _ in range(3):
        op.matvec_ptr(xh.data_ptr(), n, yh.data_ptr(), n, ptr_mode=bfgpu.BF_PTR_HOST)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        op.matvec_ptr(xh.data_ptr(), n, yh.data_ptr(), n, ptr_mode=bfgpu.BF_PTR_HOST)
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(e2e_s, world)

    # 32 right-hand sides in one bf_matvec call (forward chunks of 8 through the
    # handle's one-operator batch), CUDA events around the call
    NR = 32
    xm = torch.from_numpy(np.ascontiguousarray(G.complex_gaussian(n, 41, nrhs=NR).T)).cuda()
    ym = torch.zeros_like(xm)

    def step_multi():
        op.matvec_ptr(xm.data_ptr(), n, ym.data_ptr(), n, nrhs=NR,
                      ptr_mode=bfgpu.BF_PTR_DEVICE, stream=sp)
    for _ in range(2):
        step_multi()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(max(2, args.steps // 8)):
        step_multi()
    e1.record(stream)
    torch.cuda.synchronize()
    op.check(sp)
    ms_multi = e0.elapsed_time(e1) / max(2, args.steps // 8)
    del xm, ym

    # roofline of the dominant level launch (CUDA events inside the library)
    adj_stage_ms, _, _ = opa.profile(nrep=3)
    roof, kernels = plain_roofline(op, w["storage"])

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": f"f64 (float-float vectors and sums on FP32 pipes; {STORAGE_NAME[w['storage']]})",
        "data": "synthetic",
        "config": {
            "workload": workload_config(args.workload, w),
            "global_batch": world, "n_far": st["n_bf"], "parallelism": f"replicas x{world}",
            "l2": "no flush: factor stream per step > L2 (129 MB)",
            "factor_storage": w["storage"],
            "factor_bytes": st["factor_bytes"], "alg_bytes_per_matvec": st["alg_bytes_fwd"],
            "build_seconds": round(w["build_s"], 3), "compressions": st["compressions"],
            "retries": st["retries"]},
        "hbm_gbs": st["alg_bytes_fwd"] / (ms * 1e-3) / 1e9,
        "adjoint": {"value": world * 1000.0 / ms_adj, "unit": UNIT, "ms_per_step": ms_adj,
                    "stage_ms": [round(float(v), 4) for v in adj_stage_ms],
                    "hbm_gbs": st["alg_bytes_fwd"] / (ms_adj * 1e-3) / 1e9},
        "e2e": {"value": world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 16 * n,
                "d2h_bytes_per_step": 16 * n},
        "multi_rhs": {"value": world * NR * 1000.0 / ms_multi, "unit": UNIT, "rhs_per_call": NR,
                      "ms_per_call": ms_multi, "over_single": ms * NR / ms_multi,
                      "what": "one FP64 bf_matvec call with 32 columns: chunks of 8 through "
                              "the handle's one-operator batch"},
        "roofline": roof,
        "gpu_launches": int(kernels * args.steps),
        "clocks": clocks,
    }
    # CPU sample first: its imported GPU copy is freed before the mixed path allocates
    if rank == 0 and not args.no_cpu:
        try:
            cb, parity, end = cpu_baseline(w, w["ctx"])
            line["cpu_baseline"] = cb
            line["parity_vs_cpu_port"] = parity
            line["parity_sample"] = f"far blocks 0..{end - 1}, imported as ComplexF64"
        except Exception as e:  # report, do not fail the GPU measurement
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 0, "kind": "port",
                                    "sample": f"failed: {e}"}
        gc.collect()
    if not args.no_near:
        # the full PetrovGalerkinBF product: near blocks attached to the same operator,
        # near + far in one device pass
        t0 = time.perf_counter()
        op.add_near(w["pts"], w["pts"], w["tree"], w["tree"], w["k"])
        near_build_s = time.perf_counter() - t0
        ms_full = max_over_ranks(time_plain(op, xd, yd, n, stream, args.steps, 3), world)
        ms_full_adj = time_plain(op.adjoint(), xd, yd, n, stream, args.steps, 3)
        sn = op.stats()
        near_ms = max(ms_full - ms, 1e-6)
        line["near_far"] = {
            "value": world * 1000.0 / ms_full, "unit": UNIT, "ms_per_step": ms_full,
            "what": "full PetrovGalerkinBF product: near blocks (complex FP64 entries and FP64 "
                    "sums, self-term r=0 left out) + far butterflies in one device pass",
            "adjoint": {"value": world * 1000.0 / ms_full_adj, "ms_per_step": ms_full_adj},
            "near_pairs": sn["near_pairs"], "near_entries_both_directions": sn["near_entries"],
            "near_bytes_per_matvec": sn["near_bytes_fwd"],
            "near_ms_per_matvec": near_ms,
            "near_hbm_gbs": sn["near_bytes_fwd"] / (near_ms * 1e-3) / 1e9,
            "near_fp64_tflops": 8.0 * sn["near_entries"] / 2 / (near_ms * 1e-3) / 1e12,
            "near_setup_seconds": round(near_build_s, 3)}
    if w["storage"] == "ff" and (not args.no_c32 or not args.no_mixed):
        # the same operator with complex FP32 factor storage (half the bytes).  It
        # holds the same factor values (the float-float entries' low parts are
        # zero), and the mixed path packs its BF16 planes from them: at 262,144
        # points the 128-RHS mixed workspace alone is ~143 GB, which does not fit
        # beside the float-float operator, so that one is freed first.
        del op, opa, w["op"]
        gc.collect()
        torch.cuda.synchronize()
        w["op"], b2 = build_op(w, w["ctx"], "c32")
        w["storage"] = "c32"
        op2 = w["op"]
        ms2 = max_over_ranks(time_plain(op2, xd, yd, n, stream, args.steps, args.warmup), world)
        y2 = yd.cpu().numpy()
        ms2a = time_plain(op2.adjoint(), xd, yd, n, stream, args.steps, 3)
        roof2, _ = plain_roofline(op2, "c32")
        st2 = op2.stats()
        line["c32"] = {"value": world * 1000.0 / ms2, "unit": UNIT, "ms_per_step": ms2,
                       "storage": STORAGE_NAME["c32"], "factor_bytes": st2["factor_bytes"],
                       "alg_bytes_per_matvec": st2["alg_bytes_fwd"],
                       "hbm_gbs": st2["alg_bytes_fwd"] / (ms2 * 1e-3) / 1e9,
                       "adjoint": {"value": world * 1000.0 / ms2a, "ms_per_step": ms2a},
                       "roofline": roof2, "build_seconds": round(b2, 3),
                       "rel_diff_vs_ff": float(np.linalg.norm(y2 - y) / np.linalg.norm(y))}
    if not args.no_mixed:
        line["mixed"] = run_mixed(args, w, stream, world)
        line["mixed"]["over_plain"] = line["mixed"]["value"] / value
        line["mixed"]["factors_from"] = STORAGE_NAME[w["storage"]]
        if "c32" in line:
            line["mixed"]["over_plain_c32"] = line["mixed"]["value"] / line["c32"]["value"]
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_setup(args.gpus)
    if args.ncu_case:
        run_ncu_case(args, local)
    elif args.workload in BATCH and args.impl != "reference":
        run_batch(args, rank, world, local)
    elif args.workload in ROWS:
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference's trees, lists and recompression are Julia; the "
                              "rows line times their CPU restatements beside the GPU"}))
        else:
            run_rows(args, rank, world, local)
    elif args.workload in SURROGATE:
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "the rank surrogate has no reference counterpart"}))
        else:
            run_surrogate(args, rank, world, local)
    elif args.impl == "reference":
        run_reference(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
