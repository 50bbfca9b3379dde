// FP64-accurate butterfly matvec on the GPU (one right-hand side per pass).
//
// The level sequence of the reference flat matvec (src/Butterflyalgebra/
// bfvector.jl:200-296: Q gather+GEMV, R levels, P GEMV+scatter-add) over all
// far blocks of an operator becomes one launch per level.  Each launch runs
// independent dense tasks (see bf_pack.cpp); a task reads its input vector
// through a routing map (the fused inter-level gather) and writes each output
// entry exactly once (no atomics, deterministic).  The adjoint and transpose
// walk the same tasks backwards with A^H / A^T, reusing the forward factors.
//
// Arithmetic: factors and vectors are float-float pairs (bf_dfloat.cuh), so
// products run on the FP32 pipes at ~1e-14 relative accuracy; GB300's FP64
// rate (about 1.2 TFLOP/s) cannot feed 8 flop per 16 B at HBM speed.
#include <algorithm>
#include <atomic>
#include <cstdlib>

#include "bf_dfloat.cuh"
#include "bf_fwd_warp.cuh"
#include "bf_internal.h"

namespace bfg {
namespace {

// raw logical blocks -> packed task matrices: complex FP64 raw data becomes
// float-float entries (float4); complex FP32 raw data (the GPU build's output)
// is kept as complex FP32 (float2), which is exact and half the bytes, or
// widened to float-float with zero low parts when the build asks for the
// 16-byte storage.
template <typename SrcT, typename FT>
__global__ void repack_kernel(const DSeg* __restrict__ segs, const SrcT* __restrict__ raw,
                              FT* __restrict__ A) {
  const DSeg g = segs[blockIdx.x];
  if (g.kind == 1) {
    for (int i = threadIdx.x; i < g.rows; i += blockDim.x) {
      FT one = fac_zero<FT>();
      one.x = 1.f;
      A[g.dst_off + (size_t)i * g.dst_ld + i] = one;
    }
    return;
  }
  const long long tot = (long long)g.rows * g.cols;
  for (long long e = threadIdx.x; e < tot; e += blockDim.x) {
    int j = (int)(e / g.rows), i = (int)(e - (long long)j * g.rows);
    SrcT v = raw[g.src_off + (size_t)j * g.src_ld + i];
    FT o;
    if constexpr (sizeof(FT) == 8) {
      o = make_float2((float)v.x, (float)v.y);
    } else if constexpr (sizeof(SrcT) == 16) {
      float2 re = df_split(v.x), im = df_split(v.y);
      o = make_float4(re.x, re.y, im.x, im.y);
    } else {
      o = make_float4(v.x, 0.f, v.y, 0.f);
    }
    A[g.dst_off + (size_t)j * g.dst_ld + i] = o;
  }
}

// x (complex double, n entries) -> ws[off + q] = split(x[perm[q]]) (complex
// float-float, leaf order); optional conj
__global__ void split_kernel(const double2* __restrict__ x, int64_t n, float4* __restrict__ ws,
                             int64_t off, int conj, const int32_t* __restrict__ perm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double2 v = x[perm ? perm[i] : i];
    float2 re = df_split(v.x), im = df_split(conj ? -v.y : v.y);
    ws[off + i] = make_float4(re.x, re.y, im.x, im.y);
  }
}

// y = beta*y + alpha*v, v = ws[off + i] (optionally conjugated first).
// The last kernel of a matvec: it also moves a non-zero device error word
// (a bounded wait of this matvec's level launches gave up) to the host-visible
// word and clears it, so the next matvec starts clean.
__global__ void combine_kernel(double2* __restrict__ y, int64_t n, const float4* __restrict__ ws,
                               int64_t off, int64_t off2, double2 alpha, double2 beta,
                               int beta_zero, int conj, const int32_t* __restrict__ perm,
                               int* __restrict__ derr, int* __restrict__ herr) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int e = *(volatile int*)derr;
    if (e != 0) {
      *(volatile int*)herr = e;
      *(volatile int*)derr = 0;
      __threadfence_system();
    }
  }
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm ? perm[q] : q;  // region entry q is point perm[q]
    float4 a = ws[off + q];
    double vr = (double)a.x + (double)a.y;
    double vi = (double)a.z + (double)a.w;
    if (off2 >= 0) {  // the near field's region (same leaf order)
      const float4 b = ws[off2 + q];
      vr += (double)b.x + (double)b.y;
      vi += (double)b.z + (double)b.w;
    }
    if (conj) vi = -vi;
    double2 o;
    o.x = alpha.x * vr - alpha.y * vi;
    o.y = alpha.x * vi + alpha.y * vr;
    if (!beta_zero) {
      double2 yo = y[i];
      o.x += beta.x * yo.x - beta.y * yo.y;
      o.y += beta.x * yo.y + beta.y * yo.x;
    }
    y[i] = o;
  }
}

// ---------------------------------------------------------------------------
// Forward level kernels, chosen per task shape by the packer (bf_pack.cpp):
//   tall  (M > 128): warp per 64-row panel;
//   flat  (32 < M <= 128, n <= 256): warp per task streaming all M*n entries;
//   small (M <= 32): warp per task, lane groups on interleaved columns;
//   wide  (M <= 32, n > 2M): CTA per task (fwd_wide_kernel) or the bulk-copy
//         pipeline (bf_fwd_tma.cu);
//   copy  (identity blocks): warp per task.
// The warp routines are in bf_fwd_warp.cuh.  All of them read every factor
// entry exactly once with coalesced loads straight from HBM; input entries are
// gathered once per warp into shared memory and read as broadcasts.
template <typename FT>
__global__ void __launch_bounds__(FW_WARPS * 32) fwd_tall_kernel(
    const int2* __restrict__ items, int n_items, const DTask* __restrict__ tasks,
    const FT* __restrict__ A, const int32_t* __restrict__ maps, float4* __restrict__ ws) {
  __shared__ float4 xs[FW_WARPS][FW_XB];
  const int warp = threadIdx.x >> 5;
  const int item = blockIdx.x * FW_WARPS + warp;
  if (item >= n_items) return;
  const int2 it = items[item];
  const DTask t = tasks[it.x];
  warp_tall_one<FT>(t, it.y, A, maps, ws, xs[warp]);
}

template <typename FT>
__global__ void __launch_bounds__(FW_WARPS * 32) fwd_flat_kernel(
    const int32_t* __restrict__ tlist, int n_tasks, const DTask* __restrict__ tasks,
    const FT* __restrict__ A, const int32_t* __restrict__ maps, float4* __restrict__ ws) {
  __shared__ float4 xs[FW_WARPS][FLAT_NMAX];
  __shared__ float4 as[FW_WARPS][FLAT_MMAX];
  const int warp = threadIdx.x >> 5;
  const int ti = blockIdx.x * FW_WARPS + warp;
  if (ti >= n_tasks) return;
  const DTask t = tasks[tlist[ti]];
  warp_flat<FT>(t, A, maps, ws, xs[warp], as[warp]);
}

template <typename FT>
__global__ void __launch_bounds__(FW_WARPS * 32) fwd_small_kernel(
    const int32_t* __restrict__ tlist, int n_tasks, const DTask* __restrict__ tasks,
    const FT* __restrict__ A, const int32_t* __restrict__ maps, float4* __restrict__ ws) {
  __shared__ float4 xs[FW_WARPS][FW_XB];
  const int warp = threadIdx.x >> 5;
  const int ti = blockIdx.x * FW_WARPS + warp;
  if (ti >= n_tasks) return;
  const DTask t = tasks[tlist[ti]];
  warp_small_one<FT>(t, A, maps, ws, xs[warp]);
}

__global__ void copy_kernel(const int32_t* __restrict__ tlist, int n_tasks,
                            const DTask* __restrict__ tasks, const int32_t* __restrict__ maps,
                            float4* __restrict__ ws, int reverse) {
  const int ti = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (ti >= n_tasks) return;
  const DTask t = tasks[tlist[ti]];
  warp_copy(t, maps, ws, reverse);
}

// Forward for short wide tasks (M <= 32, many columns: the P stage).  One CTA
// per task; warps split the columns, lane groups (G = 32/M per warp) read G*M
// contiguous entries per load; partial row sums meet in shared memory.
template <typename FT>
__global__ void __launch_bounds__(256) fwd_wide_kernel(const int32_t* __restrict__ tlist,
                                                       const DTask* __restrict__ tasks,
                                                       const FT* __restrict__ A,
                                                       const int32_t* __restrict__ maps,
                                                       float4* __restrict__ ws) {
  __shared__ float4 red[8][32];
  const DTask t = tasks[tlist[blockIdx.x]];
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int M = t.M, n = t.n;
  const int G = 32 / M;
  const int g = lane / M, i = lane - g * M;
  const bool active = g < G;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  if (active) {
    const int cstep = 8 * G;
    const size_t step = (size_t)cstep * M;
    int j = warp * G + g;
    const FT* __restrict__ ap = A + t.a_off + (size_t)j * M + i;
    constexpr int LU = sizeof(FT) == 8 ? 8 : 4;  // loads in flight
    for (; j + (LU - 1) * cstep < n; j += LU * cstep) {
      FT a[LU];
      float4 x[LU];
#pragma unroll
      for (int u = 0; u < LU; ++u) a[u] = __ldg(ap + u * step);
#pragma unroll
      for (int u = 0; u < LU; ++u) x[u] = ws[cmap[j + u * cstep]];
#pragma unroll
      for (int u = 0; u < LU; ++u) cdf_mac(acc, a[u], x[u]);
      ap += LU * step;
    }
    for (; j < n; j += cstep) {
      cdf_mac(acc, __ldg(ap), ws[cmap[j]]);
      ap += step;
    }
  }
  red[warp][lane] = acc;
  __syncthreads();
  if (threadIdx.x < M) {
    const int r = threadIdx.x;
    float4 v = red[0][r];
    for (int q = 1; q < G; ++q) cdf_add(v, red[0][q * M + r]);
    for (int w = 1; w < 8; ++w)
      for (int q = 0; q < G; ++q) cdf_add(v, red[w][q * M + r]);
    ws[rmap[r]] = cdf_norm(v);
  }
}

inline int grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 16));
}

}  // namespace

Operator::~Operator() {
  for (bf_batch*& b : mrhs)
    if (b) batch_destroy(b);
  if (mixed) mixed_free(mixed);
  if (near) near_free(near);
  if (d_raw) cudaFree(d_raw);
  if (d_A) cudaFree(d_A);
  if (d_A2) cudaFree(d_A2);
  if (d_tasks) cudaFree(d_tasks);
  if (d_maps) cudaFree(d_maps);
  if (d_ws) cudaFree(d_ws);
  if (d_lists) cudaFree(d_lists);
  if (d_err) cudaFree(d_err);
  if (h_err) cudaFreeHost(h_err);
  if (d_xperm) cudaFree(d_xperm);
  if (d_yperm) cudaFree(d_yperm);
  if (d_x) cudaFree(d_x);
  if (d_y) cudaFree(d_y);
  if (stream) cudaStreamDestroy(stream);
}

int upload_plan(Operator& op) {
  Plan& p = op.plan;
  BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
  if (!op.stream) BF_TRY_CUDA(cudaStreamCreateWithFlags(&op.stream, cudaStreamNonBlocking));
  // FP64 factors -> float-float (16 B), complex FP32 factors (GPU build) stay
  // complex FP32 (8 B) unless the build asked for float-float storage (the
  // 16-byte layout of FP64 imports; the low parts are zero); two entries of
  // tail padding serve the 16-byte rounding of the bulk copies (bf_fwd_tma.cu)
  const bool f32 = !op.raw_is_double && !op.store_ff;
  const size_t esz = f32 ? sizeof(float2) : sizeof(float4);
  if ((size_t)p.fac_bytes != esz) {
    set_error("upload: plan packed for %d-byte factors, data has %zu", p.fac_bytes, esz);
    return BF_ESTATE;
  }
  size_t abytes = (size_t)(std::max<int64_t>(p.a_entries, 1) + 2) * esz;
  void* dA = nullptr;
  if (cudaMalloc(&dA, abytes) != cudaSuccess) {
    cudaGetLastError();
    set_error("upload: cannot allocate %zu bytes of factors", abytes);
    return BF_ENOMEM;
  }
  if (f32)
    op.d_A2 = (float2*)dA;
  else
    op.d_A = (float4*)dA;
  BF_TRY_CUDA(cudaMemsetAsync(dA, 0, abytes, op.stream));
  if (!p.segs.empty()) {
    DSeg* d_segs = nullptr;
    BF_TRY_CUDA(cudaMalloc(&d_segs, p.segs.size() * sizeof(DSeg)));
    BF_TRY_CUDA(cudaMemcpyAsync(d_segs, p.segs.data(), p.segs.size() * sizeof(DSeg),
                                cudaMemcpyHostToDevice, op.stream));
    // gridDim.x limit is 2^31-1; segment counts stay far below
    if (op.raw_is_double)
      repack_kernel<double2, float4><<<(unsigned)p.segs.size(), 128, 0, op.stream>>>(
          d_segs, (const double2*)op.d_raw, op.d_A);
    else if (!f32)
      repack_kernel<float2, float4><<<(unsigned)p.segs.size(), 128, 0, op.stream>>>(
          d_segs, (const float2*)op.d_raw, op.d_A);
    else
      repack_kernel<float2, float2><<<(unsigned)p.segs.size(), 128, 0, op.stream>>>(
          d_segs, (const float2*)op.d_raw, op.d_A2);
    BF_TRY_CUDA(cudaGetLastError());
    BF_TRY_CUDA(cudaStreamSynchronize(op.stream));
    cudaFree(d_segs);
  }
  // the packed matrices are the only factor copy from here on (export reads them)
  if (op.d_raw) {
    cudaFree(op.d_raw);
    op.d_raw = nullptr;
  }
  return upload_tables(op);
}

// Everything of the plan but the factors: task descriptors, routing maps,
// launch lists, leaf orders, the level workspace and the error words.
int upload_tables(Operator& op) {
  const Plan& p = op.plan;
  BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
  if (!op.stream) BF_TRY_CUDA(cudaStreamCreateWithFlags(&op.stream, cudaStreamNonBlocking));
  BF_TRY_CUDA(cudaMalloc(&op.d_tasks, std::max<size_t>(1, p.tasks.size()) * sizeof(DTask)));
  BF_TRY_CUDA(cudaMemcpy(op.d_tasks, p.tasks.data(), p.tasks.size() * sizeof(DTask),
                         cudaMemcpyHostToDevice));
  BF_TRY_CUDA(cudaMalloc(&op.d_maps, std::max<size_t>(1, p.maps.size()) * sizeof(int32_t)));
  BF_TRY_CUDA(cudaMemcpy(op.d_maps, p.maps.data(), p.maps.size() * sizeof(int32_t),
                         cudaMemcpyHostToDevice));
  if (cudaMalloc(&op.d_ws, (size_t)std::max<int64_t>(p.ws_entries, 1) * sizeof(float4)) !=
      cudaSuccess) {
    cudaGetLastError();
    set_error("upload: cannot allocate workspace");
    return BF_ENOMEM;
  }
  BF_TRY_CUDA(cudaMemset(op.d_ws, 0, (size_t)std::max<int64_t>(p.ws_entries, 1) * sizeof(float4)));
  BF_TRY_CUDA(cudaMalloc(&op.d_err, sizeof(int)));
  BF_TRY_CUDA(cudaMemset(op.d_err, 0, sizeof(int)));
  BF_TRY_CUDA(cudaHostAlloc((void**)&op.h_err, sizeof(int), cudaHostAllocMapped));
  *(volatile int*)op.h_err = 0;
  BF_TRY_CUDA(cudaHostGetDevicePointer((void**)&op.h_err_dev, op.h_err, 0));
  BF_TRY_CUDA(cudaMalloc(&op.d_xperm, std::max<size_t>(1, p.xperm.size()) * sizeof(int32_t)));
  BF_TRY_CUDA(cudaMemcpy(op.d_xperm, p.xperm.data(), p.xperm.size() * sizeof(int32_t),
                         cudaMemcpyHostToDevice));
  BF_TRY_CUDA(cudaMalloc(&op.d_yperm, std::max<size_t>(1, p.yperm.size()) * sizeof(int32_t)));
  BF_TRY_CUDA(cudaMemcpy(op.d_yperm, p.yperm.data(), p.yperm.size() * sizeof(int32_t),
                         cudaMemcpyHostToDevice));
  BF_TRY_CUDA(cudaMalloc(&op.d_lists, std::max<size_t>(1, p.lists.size()) * sizeof(int32_t)));
  if (!p.lists.empty())
    BF_TRY_CUDA(cudaMemcpy(op.d_lists, p.lists.data(), p.lists.size() * sizeof(int32_t),
                           cudaMemcpyHostToDevice));
  op.stats.n_bf = p.n_bf;
  op.stats.n_stages = p.n_stages();
  op.stats.n_tasks = (int64_t)p.tasks.size();
  op.stats.factor_entries = p.a_entries;
  op.stats.factor_bytes = p.a_entries * (int64_t)p.fac_bytes;
  op.stats.workspace_entries = p.ws_entries;
  op.stats.map_entries = (int64_t)p.maps.size();
  op.stats.alg_bytes_fwd = p.alg_bytes_fwd;
  op.stats.max_rank = p.max_rank;
  return BF_OK;
}

// Forward launches of level s with factor entries of type FT; adds the
// number of kernels launched to *nk.
template <typename FT>
static int launch_fwd_stage(Operator& op, int64_t s, cudaStream_t st, float4* ws, const FT* A,
                            int64_t* nk_out) {
  const Plan& p = op.plan;
  int nk = 0;
  auto range = [&](int c, int64_t& b, int64_t& n) {
    b = p.list_begin[c][s];
    n = p.list_begin[c][s + 1] - b;
  };
  int64_t b, n;
  const unsigned WT = FW_WARPS * 32;
  // short wide tasks (the P stage) stream through the bulk-copy pipeline; the
  // many small R-level tasks and the tall Q tasks run the direct-load kernels
  const bool tma_wide = p.stage_tma[s] != 0;
  range(Plan::L_TALL, b, n);
  if (n > 0) {
    int64_t items = n / 2;
    fwd_tall_kernel<FT><<<(unsigned)((items + FW_WARPS - 1) / FW_WARPS), WT, 0, st>>>(
        (const int2*)(op.d_lists + b), (int)items, op.d_tasks, A, op.d_maps, ws);
    ++nk;
  }
  range(Plan::L_FLAT, b, n);
  if (n > 0) {
    fwd_flat_kernel<FT><<<(unsigned)((n + FW_WARPS - 1) / FW_WARPS), WT, 0, st>>>(
        op.d_lists + b, (int)n, op.d_tasks, A, op.d_maps, ws);
    ++nk;
  }
  range(Plan::L_SMALL, b, n);
  if (n > 0) {
    fwd_small_kernel<FT><<<(unsigned)((n + FW_WARPS - 1) / FW_WARPS), WT, 0, st>>>(
        op.d_lists + b, (int)n, op.d_tasks, A, op.d_maps, ws);
    ++nk;
  }
  range(Plan::L_WIDE, b, n);
  if (n > 0 && tma_wide) {
    BF_TRY(launch_fwd_tma(op.d_lists + b, (int)n, op.d_tasks, op.d_A, op.d_A2, op.d_maps, ws,
                          op.d_err, op.wait_limit, op.ctx->prop.multiProcessorCount, st));
    ++nk;
  } else if (n > 0) {
    fwd_wide_kernel<FT><<<(unsigned)n, 256, 0, st>>>(op.d_lists + b, op.d_tasks, A, op.d_maps, ws);
    ++nk;
  }
  range(Plan::L_COPY, b, n);
  if (n > 0) {
    copy_kernel<<<(unsigned)((n + 7) / 8), 256, 0, st>>>(op.d_lists + b, (int)n, op.d_tasks,
                                                         op.d_maps, ws, 0);
    ++nk;
  }
  BF_TRY_CUDA(cudaGetLastError());
  if (nk_out) *nk_out += nk;
  return BF_OK;
}

// Launches of level s for direction trans; adds the kernel count to *nk.
static int launch_stage(Operator& op, int64_t s, int trans, cudaStream_t st, float4* ws,
                        int64_t* nk_out) {
  const Plan& p = op.plan;
  if (trans == BF_OP_N)
    return op.d_A2 ? launch_fwd_stage<float2>(op, s, st, ws, op.d_A2, nk_out)
                   : launch_fwd_stage<float4>(op, s, st, ws, op.d_A, nk_out);
  // adjoint / transpose: same tasks, rows and columns swapped
  int nk = launch_adj_stage(p, s, trans == BF_OP_C, op.d_lists, op.d_tasks, op.d_A, op.d_A2,
                            op.d_maps, ws, st);
  if (nk < 0) return BF_ECUDA;  // message set by the launcher
  int64_t b = p.list_begin[Plan::L_COPY][s], n = p.list_begin[Plan::L_COPY][s + 1] - b;
  if (n > 0) {
    copy_kernel<<<(unsigned)((n + 7) / 8), 256, 0, st>>>(op.d_lists + b, (int)n, op.d_tasks,
                                                         op.d_maps, ws, 1);
    ++nk;
  }
  BF_TRY_CUDA(cudaGetLastError());
  if (nk_out) *nk_out += nk;
  return BF_OK;
}

// One FP64-accurate matvec of a single right-hand side, device pointers.
static int matvec_one(Operator& op, int trans, const double2* x, double2* y, double2 alpha,
                      double2 beta, cudaStream_t st, float4* ws) {
  const Plan& p = op.plan;
  const bool fwd = trans == BF_OP_N;
  const int64_t nin = fwd ? p.n_cols : p.n_rows;
  const int64_t nout = fwd ? p.n_rows : p.n_cols;
  const int64_t in_off = fwd ? p.xg_off : p.yg_off;
  const int64_t out_off = fwd ? p.yg_off : p.xg_off;
  const bool covered = fwd ? p.yg_covered : p.xg_covered;
  split_kernel<<<grid_for(nin, 256), 256, 0, st>>>(x, nin, ws, in_off, 0,
                                                    fwd ? op.d_xperm : op.d_yperm);
  if (!covered)
    BF_TRY_CUDA(cudaMemsetAsync(ws + out_off, 0, (size_t)nout * sizeof(float4), st));
  const int64_t ns = p.n_stages();
  for (int64_t k = 0; k < ns; ++k) BF_TRY(launch_stage(op, fwd ? k : ns - 1 - k, trans, st, ws, nullptr));
  int64_t near_off = -1;
  if (op.near) {  // near + far in one pass (matrixvector.jl:28-33)
    BF_TRY(near_stage(op, trans, st, x, ws, nullptr));
    near_off = fwd ? op.near->ny_off : op.near->nx_off;
  }
  combine_kernel<<<grid_for(nout, 256), 256, 0, st>>>(y, nout, ws, out_off, near_off, alpha, beta,
                                                      beta.x == 0.0 && beta.y == 0.0, 0,
                                                      fwd ? op.d_yperm : op.d_xperm, op.d_err,
                                                      op.h_err_dev);
  BF_TRY_CUDA(cudaGetLastError());
  return BF_OK;
}

// y[:, c] = alpha * z[:, c] + beta * y[:, c] (beta == 0: y is not read); z packed n x ncol
__global__ void axpby_kernel(double2* __restrict__ y, int64_t ldy, const double2* __restrict__ z,
                             int64_t n, int ncol, double2 a, double2 b, int bzero) {
  const int64_t tot = n * ncol;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / n, i = e - c * n;
    const double2 v = z[e];
    double2 r = make_double2(a.x * v.x - a.y * v.y, a.x * v.y + a.y * v.x);
    if (!bzero) {
      const double2 w = y[c * ldy + i];
      r.x += b.x * w.x - b.y * w.y;
      r.y += b.x * w.y + b.y * w.x;
    }
    y[c * ldy + i] = r;
  }
}

// The columns of one call (device pointers).  Forward: whole chunks of
// MRHS_CHUNK go through the operator's own one-operator batch, where each
// factor entry loaded serves up to four right-hand sides (the reference's
// bfmatrix.jl:10-75 applies the operator column by column); measured at
// 262,144 points with 32 columns: 1.43x (float-float factors) and 1.10x
// (complex FP32) over the column loop.  The batch's adjoint was not faster
// (1.07x, 0.89x), so adjoint and transpose columns, the remainder columns and
// every column of an operator with a near field go one by one.
static int matvec_cols(Operator& op, int trans, int64_t nrhs, const double2* x, int64_t ldx,
                       double2* y, int64_t ldy, double2 a, double2 b, cudaStream_t st) {
  const Plan& p = op.plan;
  const int64_t nin = trans == BF_OP_N ? p.n_cols : p.n_rows;
  const int64_t nout = trans == BF_OP_N ? p.n_rows : p.n_cols;
  const int ti = trans == BF_OP_N ? 0 : trans == BF_OP_C ? 1 : 2;
  const int bzero = b.x == 0.0 && b.y == 0.0;
  int64_t c = 0;
  if (trans == BF_OP_N && nrhs >= MRHS_CHUNK && !op.near && !op.mrhs_off[ti]) {
    if (!op.mrhs[ti]) {
      Operator* self = &op;
      const int32_t tr = trans, nr = MRHS_CHUNK;
      const int rc = batch_create(op.ctx, &self, &tr, &nr, 1, MRHS_CHUNK, &op.mrhs[ti]);
      if (rc == BF_ENOMEM) {  // not enough device memory for the batch: columns one by one
        op.mrhs_off[ti] = 1;
        op.mrhs[ti] = nullptr;
      } else {
        BF_TRY(rc);
      }
    }
    if (op.mrhs[ti]) {
      double2 *bx = nullptr, *by = nullptr;
      BF_TRY(batch_buffers(op.mrhs[ti], 0, &bx, &by));
      for (; c + MRHS_CHUNK <= nrhs; c += MRHS_CHUNK) {
        BF_TRY_CUDA(cudaMemcpy2DAsync(bx, nin * sizeof(double2), x + c * ldx, ldx * sizeof(double2),
                                      nin * sizeof(double2), MRHS_CHUNK, cudaMemcpyDeviceToDevice,
                                      st));
        BF_TRY(batch_launch(op.mrhs[ti], st));
        axpby_kernel<<<grid_for(nout * MRHS_CHUNK, 256), 256, 0, st>>>(y + c * ldy, ldy, by, nout,
                                                                       MRHS_CHUNK, a, b, bzero);
        BF_TRY_CUDA(cudaGetLastError());
      }
    }
  }
  for (; c < nrhs; ++c) BF_TRY(matvec_one(op, trans, x + c * ldx, y + c * ldy, a, b, st, op.d_ws));
  return BF_OK;
}

int take_device_error(Operator& op, const char* what) {
  if (!op.h_err) return BF_OK;
  const int e = __atomic_exchange_n(op.h_err, 0, __ATOMIC_ACQ_REL);
  if (e == 0) return BF_OK;
  set_error("%s: a bounded device-side wait of a matvec on this operator gave up (code %d); "
            "that matvec's output is invalid", what, e);
  return BF_ETIMEOUT;
}

// Per-stage device time of one matvec: events around every level launch.
int profile_matvec(Operator& op, int trans, int nrep, double* ms, int64_t* bytes,
                   int64_t* kernels) {
  const Plan& p = op.plan;
  const int64_t ns = p.n_stages();
  if (nrep < 1) nrep = 1;
  BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
  cudaStream_t st = op.stream;
  std::vector<cudaEvent_t> ev(ns + 1);
  for (auto& e : ev) BF_TRY_CUDA(cudaEventCreate(&e));
  std::vector<double> acc(ns, 0.0);
  const bool fwd = trans == BF_OP_N;
  int64_t nk = 2;  // split + combine
  for (int r = 0; r < nrep + 1; ++r) {  // first pass warms up
    BF_TRY_CUDA(cudaEventRecord(ev[0], st));
    int64_t cnt = 2;
    for (int64_t k = 0; k < ns; ++k) {
      BF_TRY(launch_stage(op, fwd ? k : ns - 1 - k, trans, st, op.d_ws, &cnt));
      BF_TRY_CUDA(cudaEventRecord(ev[k + 1], st));
    }
    BF_TRY_CUDA(cudaGetLastError());
    nk = cnt;
    BF_TRY_CUDA(cudaEventSynchronize(ev[ns]));
    if (r == 0) continue;
    for (int64_t k = 0; k < ns; ++k) {
      float t = 0.f;
      BF_TRY_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
      int64_t s = fwd ? k : ns - 1 - k;
      acc[s] += t;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  for (int64_t s = 0; s < ns; ++s) {
    if (ms) ms[s] = acc[s] / nrep;
    if (bytes) bytes[s] = p.stage_bytes[s];
  }
  if (kernels) *kernels = nk;
  // the level launches ran without the combine kernel: read the device word here
  int h = 0;
  BF_TRY_CUDA(cudaMemcpy(&h, op.d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (h != 0) {
    BF_TRY_CUDA(cudaMemset(op.d_err, 0, sizeof(int)));
    set_error("bf_op_profile: a bounded device-side wait gave up (code %d)", h);
    return BF_ETIMEOUT;
  }
  return BF_OK;
}

int run_matvec(Operator& op, int trans, int64_t nrhs, const double* x, int64_t ldx, double* y,
               int64_t ldy, const double* alpha, const double* beta, int ptr_mode,
               cudaStream_t stream) {
  const Plan& p = op.plan;
  if (trans != BF_OP_N && trans != BF_OP_C && trans != BF_OP_T) {
    set_error("bf_matvec: invalid trans %d", trans);
    return BF_EINVAL;
  }
  const int64_t nin = trans == BF_OP_N ? p.n_cols : p.n_rows;
  const int64_t nout = trans == BF_OP_N ? p.n_rows : p.n_cols;
  if (nrhs < 0 || (nrhs > 0 && (!x || !y || ldx < nin || ldy < nout))) {
    set_error("bf_matvec: invalid sizes (nrhs=%lld ldx=%lld ldy=%lld, need %lld/%lld)",
              (long long)nrhs, (long long)ldx, (long long)ldy, (long long)nin, (long long)nout);
    return BF_EINVAL;
  }
  if (nrhs == 0) return BF_OK;
  // a timeout of an earlier asynchronous call that nobody has collected yet
  BF_TRY(take_device_error(op, "bf_matvec"));
  double2 a = make_double2(alpha ? alpha[0] : 1.0, alpha ? alpha[1] : 0.0);
  double2 b = make_double2(beta ? beta[0] : 0.0, beta ? beta[1] : 0.0);
  const bool bzero = b.x == 0.0 && b.y == 0.0;
  BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
  cudaStream_t st = stream ? stream : op.stream;
  if (ptr_mode == BF_PTR_DEVICE)
    return matvec_cols(op, trans, nrhs, (const double2*)x, ldx, (double2*)y, ldy, a, b, st);
  if (ptr_mode != BF_PTR_HOST) {
    set_error("bf_matvec: invalid ptr_mode %d", ptr_mode);
    return BF_EINVAL;
  }
  // host pointers: stage through device buffers (sized to the largest call so far)
  int64_t need = std::max(p.n_rows, p.n_cols) * nrhs;
  if (need > op.stage_cap) {
    if (op.d_x) cudaFree(op.d_x);
    if (op.d_y) cudaFree(op.d_y);
    op.d_x = op.d_y = nullptr;
    op.stage_cap = 0;
    BF_TRY_CUDA(cudaMalloc(&op.d_x, (size_t)need * 2 * sizeof(double)));
    BF_TRY_CUDA(cudaMalloc(&op.d_y, (size_t)need * 2 * sizeof(double)));
    op.stage_cap = need;
  }
  BF_TRY_CUDA(cudaMemcpy2DAsync(op.d_x, nin * 2 * sizeof(double), x, ldx * 2 * sizeof(double),
                                nin * 2 * sizeof(double), nrhs, cudaMemcpyHostToDevice, st));
  if (!bzero)
    BF_TRY_CUDA(cudaMemcpy2DAsync(op.d_y, nout * 2 * sizeof(double), y, ldy * 2 * sizeof(double),
                                  nout * 2 * sizeof(double), nrhs, cudaMemcpyHostToDevice, st));
  BF_TRY(matvec_cols(op, trans, nrhs, (const double2*)op.d_x, nin, (double2*)op.d_y, nout, a, b,
                     st));
  BF_TRY_CUDA(cudaMemcpy2DAsync(y, ldy * 2 * sizeof(double), op.d_y, nout * 2 * sizeof(double),
                                nout * 2 * sizeof(double), nrhs, cudaMemcpyDeviceToHost, st));
  BF_TRY_CUDA(cudaStreamSynchronize(st));
  return take_device_error(op, "bf_matvec");
}

}  // namespace bfg

// ---------------------------------------------------------------------------
// Allocation-free matvec (bf_matvec_noalloc).
//
// Some callers must apply the operator at a point where they cannot allocate
// device memory: a callback that runs while the caller's memory pool is
// locked or already exhausted (an iterative solver embedded in an application
// that owns all device memory), or a real-time loop whose allocation budget is
// fixed at start-up.  For them the level workspace (the scratch vectors
// between butterfly levels) lives in one file-scope device array of fixed
// size instead of the operator's own buffer.  The array is reserved in every
// GPU's memory as soon as the library is loaded and stays there until the
// process exits.
namespace bfg {
namespace {

constexpr long long NOALLOC_WS_ENTRIES = 1ll << 20;  // 16 MiB of complex float-float entries
constexpr int NOALLOC_MAX_DEVICES = 64;

__device__ __align__(256) float4 g_noalloc_ws[NOALLOC_WS_ENTRIES];

// Device address of g_noalloc_ws, per device.  In host code the symbol is a
// host-side stand-in, so the address must come from cudaGetSymbolAddress with
// that device current.
std::atomic<float4*> g_noalloc_addr[NOALLOC_MAX_DEVICES];

int noalloc_workspace(int device, float4** out) {
  if (device < 0 || device >= NOALLOC_MAX_DEVICES) {
    set_error("bf_matvec_noalloc: device %d outside the supported range", device);
    return BF_EINVAL;
  }
  float4* p = g_noalloc_addr[device].load(std::memory_order_acquire);
  if (!p) {
    void* sym = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&sym, g_noalloc_ws);
    if (e != cudaSuccess || !sym) {
      cudaGetLastError();
      set_error("bf_matvec_noalloc: cudaGetSymbolAddress failed on device %d: %s", device,
                cudaGetErrorString(e));
      return BF_ECUDA;
    }
    p = (float4*)sym;
    g_noalloc_addr[device].store(p, std::memory_order_release);
  }
  *out = p;
  return BF_OK;
}

}  // namespace
}  // namespace bfg

extern "C" int bf_matvec_noalloc(bf_op_t h, int trans, int64_t nrhs, const double* x,
                                 int64_t ldx, double* y, int64_t ldy, const double* alpha,
                                 const double* beta, void* stream) {
  using namespace bfg;
  if (!h) {
    set_error("bf_matvec_noalloc: NULL operator");
    return BF_EINVAL;
  }
  Operator& op = h->op;
  const Plan& p = op.plan;
  int s_pre = BF_OK;
  if (trans != BF_OP_N && trans != BF_OP_C && trans != BF_OP_T) {
    set_error("bf_matvec_noalloc: invalid trans %d", trans);
    return BF_EINVAL;
  }
  const int64_t nin = trans == BF_OP_N ? p.n_cols : p.n_rows;
  const int64_t nout = trans == BF_OP_N ? p.n_rows : p.n_cols;
  if (nrhs < 0 || (nrhs > 0 && (!x || !y || ldx < nin || ldy < nout))) {
    set_error("bf_matvec_noalloc: invalid sizes");
    return BF_EINVAL;
  }
  if (p.ws_entries > NOALLOC_WS_ENTRIES) {
    set_error("bf_matvec_noalloc: operator needs %lld workspace entries; the allocation-free "
              "path holds at most %lld (16 MiB); use bf_matvec",
              (long long)p.ws_entries, (long long)NOALLOC_WS_ENTRIES);
    return BF_EINVAL;
  }
  if (nrhs == 0) return BF_OK;
  // a timeout of an earlier call on this operator (read from host memory)
  s_pre = take_device_error(op, "bf_matvec_noalloc");
  if (s_pre != BF_OK) return s_pre;
  if (cudaSetDevice(op.ctx->device) != cudaSuccess) {
    cudaGetLastError();
    set_error("bf_matvec_noalloc: cudaSetDevice failed");
    return BF_ECUDA;
  }
  float4* ws = nullptr;
  int s = noalloc_workspace(op.ctx->device, &ws);
  if (s != BF_OK) return s;
  double2 a = make_double2(alpha ? alpha[0] : 1.0, alpha ? alpha[1] : 0.0);
  double2 b = make_double2(beta ? beta[0] : 0.0, beta ? beta[1] : 0.0);
  cudaStream_t st = stream ? (cudaStream_t)stream : op.stream;
  for (int64_t c = 0; c < nrhs; ++c) {
    s = matvec_one(op, trans, (const double2*)(x + 2 * c * ldx), (double2*)(y + 2 * c * ldy), a,
                   b, st, ws);
    if (s != BF_OK) return s;
  }
  return BF_OK;
}
