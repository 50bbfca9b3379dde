// Many independent far-field operators, many right-hand sides each, in one
// launch sequence (bf_batch_*).
//
// The reference applies operators one at a time, one column at a time
// (src/Butterflyalgebra/bfmatrix.jl:10-75 inside each mul!).  Here the level
// sequences of all operators are merged: merged level s holds level s of every
// operator that has one.  A level is ONE persistent launch
// (batch_level_kernel): warps take work items (operator, task, row panel) from
// an atomic queue in longest-first order and run FP64-accurate warp routines
// (the bt_* routines below, same arithmetic as bf_fwd_warp.cuh) for every
// right-hand side of the current chunk in turn.  A task matrix is read from HBM once per chunk and re-read from L1/L2
// for the chunk's other right-hand sides.  Each operator has one workspace per
// right-hand side of a chunk.  Chunks of `rhs_chunk` right-hand sides run one
// after the other.
//
// The whole sequence -- per chunk: one batched split (all operators and
// right-hand sides), the merged levels, one batched combine -- is captured once
// into a CUDA graph and replayed by bf_batch_run, so a batch matvec costs a
// single graph launch.  The work-queue counters are reset by memset nodes
// inside the graph.
//
// Autotuner (bf_batch_autotune): the task-shape cut between the flat routine
// and tall row panels (flat_mmax), the item order (longest first over all
// shapes, or bucketed by shape and then longest first) and the persistent
// grid size (CTAs per SM) are chosen by timing graph replays of the actual
// batch for every candidate; the fastest is kept.
#include <algorithm>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>

#include "bf_dfloat.cuh"
#include "bf_fwd_warp.cuh"
#include "bf_internal.h"

namespace bfg {
namespace {

enum : int32_t { BC_TALL = 0, BC_FLAT = 1, BC_SMALL = 2, BC_COPY = 3 };

struct alignas(16) BatchItem {
  int32_t op, task, r0, cls;
};

struct BatchOpDev {
  const DTask* tasks;
  const void* A;          // float2 or float4 entries (one type per batch)
  const int32_t* maps;
  float4* ws;             // rhs_chunk workspaces of ws_entries each
  const int32_t* xperm;
  const int32_t* yperm;
  const double2* X;       // n_cols x nrhs, column-major
  double2* Y;             // n_rows x nrhs
  long long ws_entries, xg_off, yg_off, n_rows, n_cols;
  int nrhs, yg_covered;
};

struct BatchCfg {
  int flat_mmax;    // 64, 96 or 128
  int bucketed;     // 0 = longest first over all shapes, 1 = by shape then longest first
  int ctas_per_sm;  // persistent grid = ctas_per_sm x SMs
};

// The batch kernel's own task routines.  Same arithmetic and traversal as
// the level routines of bf_fwd_warp.cuh, without their early first-batch loads
// and predicated tails: here a task matrix comes from HBM for the first
// right-hand side of a chunk and from L2 for the others, and the persistent
// kernel holds all three routines, so fewer live registers (3 CTAs per SM
// without spills) matter more than fewer serial HBM latencies (measured).
template <typename FT>
__device__ __forceinline__ void bt_tall(const DTask& t, int r0, const FT* __restrict__ A,
                                        const int32_t* __restrict__ maps,
                                        float4* __restrict__ ws, float4* __restrict__ xw) {
  const int lane = threadIdx.x & 31;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int M = t.M, n = t.n;
  if (r0 >= M) return;
  // the input block is staged once when it fits (n <= FW_XB, the Q-stage case)
  const bool one_block = n <= FW_XB;
  if (one_block) {
    for (int j = lane; j < n; j += 32) xw[j] = ws_in(t, cmap, ws, j);
    __syncwarp();
  }
  float4 acc[TALL_RPL];
#pragma unroll
  for (int q = 0; q < TALL_RPL; ++q) acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  bool act[TALL_RPL];
#pragma unroll
  for (int q = 0; q < TALL_RPL; ++q) act[q] = r0 + lane + 32 * q < M;
  for (int cb = 0; cb < n; cb += FW_XB) {
    const int nb = min(FW_XB, n - cb);
    if (!one_block) {
      for (int j = lane; j < nb; j += 32) xw[j] = ws_in(t, cmap, ws, cb + j);
      __syncwarp();
    }
    const FT* __restrict__ ap = A + t.a_off + (size_t)cb * M + r0 + lane;
    int j = 0;
    // columns per iteration: 128 bytes of loads in flight per lane (eight
    // float-float or sixteen complex FP32 entries)
    constexpr int CPI = (sizeof(FT) == 8 ? 16 : 8) / TALL_RPL;
    for (; j + CPI - 1 < nb; j += CPI) {
      FT a[CPI][TALL_RPL];
#pragma unroll
      for (int c = 0; c < CPI; ++c)
#pragma unroll
        for (int q = 0; q < TALL_RPL; ++q)
          a[c][q] = act[q] ? __ldg(ap + (size_t)c * M + 32 * q) : fac_zero<FT>();
#pragma unroll
      for (int c = 0; c < CPI; ++c) {
        const float4 xc = xw[j + c];
#pragma unroll
        for (int q = 0; q < TALL_RPL; ++q) cdf_mac(acc[q], a[c][q], xc);
      }
      ap += CPI * (size_t)M;
    }
    for (; j < nb; j += 1) {
      const float4 x0 = xw[j];
#pragma unroll
      for (int q = 0; q < TALL_RPL; ++q)
        if (act[q]) cdf_mac(acc[q], __ldg(ap + 32 * q), x0);
      ap += M;
    }
    __syncwarp();
  }
#pragma unroll
  for (int q = 0; q < TALL_RPL; ++q)
    if (act[q]) ws[rmap[r0 + lane + 32 * q]] = cdf_norm(acc[q]);
  __syncwarp();
}

// One warp streams a whole task flat: lane l reads entry e = l + 32k of the
// column-major M x n matrix.  With M > 32 the 32 entries of one warp load
// belong to 32 distinct rows, so each lane adds its product into a per-row
// accumulator in warp-private shared memory without conflicts.
template <typename FT>
__device__ __forceinline__ void bt_flat(const DTask& t, const FT* __restrict__ A,
                                        const int32_t* __restrict__ maps,
                                        float4* __restrict__ ws, float4* __restrict__ xw,
                                        float4* __restrict__ aw) {
  const int lane = threadIdx.x & 31;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int M = t.M, n = t.n;
  for (int j = lane; j < n; j += 32) xw[j] = ws_in(t, cmap, ws, j);
  for (int i = lane; i < M; i += 32) aw[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  __syncwarp();
  const long long tot = (long long)M * n;
  const FT* __restrict__ ap = A + t.a_off;
  int row = lane, col = 0;  // entry lane: row lane of column 0 (M > 32)
  long long e = lane;
  constexpr int LU = sizeof(FT) == 8 ? 8 : 4;  // loads in flight: 64 bytes per lane
  for (; e - lane + 32 * LU <= tot; e += 32 * LU) {  // warp-uniform: whole warp steps fit
    FT v[LU];
#pragma unroll
    for (int u = 0; u < LU; ++u) v[u] = __ldg(ap + e + 32 * u);
    // lane a at step u+1 can hit the row that lane a-(M-32) updates at step
    // u: the warp barrier orders the two read-modify-writes
#pragma unroll
    for (int u = 0; u < LU; ++u) {
      float4 s = aw[row];
      cdf_mac(s, v[u], xw[col]);
      aw[row] = s;
      __syncwarp();
      row += 32;
      if (row >= M) {
        row -= M;
        ++col;
      }
    }
  }
  for (; e - lane < tot; e += 32) {  // warp-uniform trip count
    if (e < tot) {
      float4 s = aw[row];
      cdf_mac(s, __ldg(ap + e), xw[col]);
      aw[row] = s;
    }
    __syncwarp();
    row += 32;
    if (row >= M) {
      row -= M;
      ++col;
    }
  }
  __syncwarp();
  for (int i = lane; i < M; i += 32) ws[rmap[i]] = cdf_norm(aw[i]);
  __syncwarp();
}

// M <= 32: G = 32/M lane groups walk interleaved columns (one warp load reads
// G*M contiguous entries); the groups meet in shared memory at the end.
template <typename FT>
__device__ __forceinline__ void bt_small(const DTask& t, const FT* __restrict__ A,
                                         const int32_t* __restrict__ maps,
                                         float4* __restrict__ ws, float4* __restrict__ xw) {
  const int lane = threadIdx.x & 31;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int M = t.M, n = t.n;
  const int G = 32 / M;
  const int g = lane / M, i = lane - g * M;
  const bool active = g < G;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int cb = 0; cb < n; cb += FW_XB) {
    const int nb = min(FW_XB, n - cb);
    for (int j = lane; j < nb; j += 32) xw[j] = ws_in(t, cmap, ws, cb + j);
    __syncwarp();
    if (active) {
      const size_t step = (size_t)G * M;
      const FT* __restrict__ ap = A + t.a_off + (size_t)(cb + g) * M + i;
      int j = g;
      constexpr int LU = sizeof(FT) == 8 ? 8 : 4;  // loads in flight
      for (; j + (LU - 1) * G < nb; j += LU * G) {
        FT a[LU];
#pragma unroll
        for (int u = 0; u < LU; ++u) a[u] = __ldg(ap + u * step);
#pragma unroll
        for (int u = 0; u < LU; ++u) cdf_mac(acc, a[u], xw[j + u * G]);
        ap += LU * step;
      }
      for (; j < nb; j += G) {
        cdf_mac(acc, __ldg(ap), xw[j]);
        ap += step;
      }
    }
    __syncwarp();
  }
  if (G > 1) {
    xw[lane] = acc;  // reuse the staging buffer for the group reduction
    __syncwarp();
    if (active && g == 0) {
      for (int q = 1; q < G; ++q) cdf_add(acc, xw[q * M + i]);
      ws[rmap[i]] = cdf_norm(acc);
    }
  } else if (active) {
    ws[rmap[i]] = cdf_norm(acc);
  }
  __syncwarp();
}

template <typename FT>
__global__ void __launch_bounds__(FW_WARPS * 32) batch_level_kernel(
    const BatchItem* __restrict__ items, int n_items, int* __restrict__ counter,
    const BatchOpDev* __restrict__ ops, int rhs_base, int rhs_chunk) {
  __shared__ float4 xs[FW_WARPS][FW_XB];
  __shared__ float4 as[FW_WARPS][FLAT_MMAX];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    int i = 0;
    if (lane == 0) i = atomicAdd(counter, 1);
    i = __shfl_sync(0xffffffffu, i, 0);
    if (i >= n_items) break;
    const BatchItem it = items[i];
    const BatchOpDev& o = ops[it.op];
    const int nr = min(rhs_chunk, o.nrhs - rhs_base);
    if (nr <= 0) continue;
    const DTask t = o.tasks[it.task];
    const FT* A = static_cast<const FT*>(o.A);
    for (int r = 0; r < nr; ++r) {
      float4* ws = o.ws + (size_t)r * o.ws_entries;
      switch (it.cls) {
        case BC_TALL: bt_tall<FT>(t, it.r0, A, o.maps, ws, xs[warp]); break;
        case BC_FLAT: bt_flat<FT>(t, A, o.maps, ws, xs[warp], as[warp]); break;
        case BC_SMALL: bt_small<FT>(t, A, o.maps, ws, xs[warp]); break;
        default: warp_copy(t, o.maps, ws, 0); __syncwarp(); break;
      }
    }
  }
}

// x of every (operator, right-hand side) pair of the chunk -> the x region of
// its workspace (float-float, leaf order); zeroes y regions that no P task
// covers.  blockIdx.y = pair (int2 {op, local rhs}).
__global__ void batch_split_kernel(const int2* __restrict__ pairs, const BatchOpDev* __restrict__ ops,
                                   int rhs_base) {
  const int2 pr = pairs[blockIdx.y];
  const BatchOpDev& o = ops[pr.x];
  float4* ws = o.ws + (size_t)pr.y * o.ws_entries;
  const double2* x = o.X + (size_t)(rhs_base + pr.y) * o.n_cols;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < o.n_cols;
       q += (long long)gridDim.x * blockDim.x) {
    const double2 v = x[o.xperm[q]];
    const float2 re = df_split(v.x), im = df_split(v.y);
    ws[o.xg_off + q] = make_float4(re.x, re.y, im.x, im.y);
  }
  if (!o.yg_covered)
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < o.n_rows;
         q += (long long)gridDim.x * blockDim.x)
      ws[o.yg_off + q] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void batch_combine_kernel(const int2* __restrict__ pairs,
                                     const BatchOpDev* __restrict__ ops, int rhs_base) {
  const int2 pr = pairs[blockIdx.y];
  const BatchOpDev& o = ops[pr.x];
  const float4* ws = o.ws + (size_t)pr.y * o.ws_entries;
  double2* y = o.Y + (size_t)(rhs_base + pr.y) * o.n_rows;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < o.n_rows;
       q += (long long)gridDim.x * blockDim.x) {
    const float4 a = ws[o.yg_off + q];
    y[o.yperm[q]] = make_double2((double)a.x + (double)a.y, (double)a.z + (double)a.w);
  }
}

}  // namespace

struct BatchState {
  Context* ctx = nullptr;
  std::vector<Operator*> ops;
  std::vector<int32_t> nrhs;
  int rhs_chunk = 8;
  bool f32 = true;
  int n_levels = 0, n_chunks = 0;
  std::vector<BatchOpDev> hops;
  BatchOpDev* d_ops = nullptr;
  std::vector<void*> allocs;  // workspaces, X, Y
  std::vector<int2*> d_pairs;  // per chunk
  std::vector<int> n_pairs;
  int64_t max_n = 0;
  // work items per merged level for the current configuration
  BatchItem* d_items = nullptr;
  std::vector<int64_t> item_begin;  // n_levels + 1
  int* d_counters = nullptr;        // n_chunks * n_levels
  BatchCfg cfg{128, 0, 4};
  cudaStream_t st = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t graph_nodes = 0;
  int64_t ws_bytes = 0;
  ~BatchState() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void* p : allocs) cudaFree(p);
    for (int2* p : d_pairs) cudaFree(p);
    if (d_ops) cudaFree(d_ops);
    if (d_items) cudaFree(d_items);
    if (d_counters) cudaFree(d_counters);
    if (st) cudaStreamDestroy(st);
  }
};

namespace {

// work items of every merged level for configuration c (longest first)
int build_items(BatchState& b, const BatchCfg& c) {
  std::vector<std::pair<int64_t, BatchItem>> all;
  std::vector<BatchItem> flat;
  b.item_begin.assign(b.n_levels + 1, 0);
  for (int s = 0; s < b.n_levels; ++s) {
    all.clear();
    for (size_t oi = 0; oi < b.ops.size(); ++oi) {
      const Plan& p = b.ops[oi]->plan;
      if (s >= p.n_stages()) continue;
      const int64_t w = b.nrhs[oi];
      for (int64_t ti = p.stage_begin[s]; ti < p.stage_begin[s + 1]; ++ti) {
        const DTask& t = p.tasks[ti];
        if (t.M <= 0) continue;
        BatchItem it{(int32_t)oi, (int32_t)ti, 0, 0};
        if (t.kind == TASK_COPY) {
          it.cls = BC_COPY;
          all.push_back({(int64_t)t.M * w, it});
        } else if (t.M <= 32) {
          it.cls = BC_SMALL;
          all.push_back({(int64_t)t.M * t.n * w, it});
        } else if (t.M <= c.flat_mmax && t.n <= FLAT_NMAX) {
          it.cls = BC_FLAT;
          all.push_back({(int64_t)t.M * t.n * w, it});
        } else {
          it.cls = BC_TALL;
          for (int r0 = 0; r0 < t.M; r0 += TALL_ROWS) {
            it.r0 = r0;
            all.push_back({(int64_t)std::min(TALL_ROWS, t.M - r0) * t.n * w, it});
          }
        }
      }
    }
    if (c.bucketed)
      std::stable_sort(all.begin(), all.end(), [](const auto& a, const auto& x) {
        return a.second.cls != x.second.cls ? a.second.cls < x.second.cls : a.first > x.first;
      });
    else
      std::stable_sort(all.begin(), all.end(),
                       [](const auto& a, const auto& x) { return a.first > x.first; });
    b.item_begin[s] = (int64_t)flat.size();
    for (auto& a : all) flat.push_back(a.second);
  }
  b.item_begin[b.n_levels] = (int64_t)flat.size();
  if (flat.size() > (size_t)INT32_MAX) {
    set_error("batch: too many work items");
    return BF_EINVAL;
  }
  if (b.d_items) cudaFree(b.d_items);
  b.d_items = nullptr;
  BF_TRY_CUDA(cudaMalloc(&b.d_items, std::max<size_t>(1, flat.size()) * sizeof(BatchItem)));
  BF_TRY_CUDA(cudaMemcpy(b.d_items, flat.data(), flat.size() * sizeof(BatchItem),
                         cudaMemcpyHostToDevice));
  return BF_OK;
}

// capture the whole batch matvec (all chunks) into a CUDA graph
int capture(BatchState& b, const BatchCfg& c) {
  if (b.exec) cudaGraphExecDestroy(b.exec);
  if (b.graph) cudaGraphDestroy(b.graph);
  b.exec = nullptr;
  b.graph = nullptr;
  const int sms = b.ctx->prop.multiProcessorCount;
  BF_TRY_CUDA(cudaStreamBeginCapture(b.st, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  e = cudaMemsetAsync(b.d_counters, 0, (size_t)b.n_chunks * b.n_levels * sizeof(int), b.st);
  for (int ch = 0; ch < b.n_chunks && e == cudaSuccess; ++ch) {
    const int base = ch * b.rhs_chunk;
    const unsigned gx = (unsigned)std::min<int64_t>((b.max_n + 255) / 256, 4 * sms);
    batch_split_kernel<<<dim3(gx, b.n_pairs[ch]), 256, 0, b.st>>>(b.d_pairs[ch], b.d_ops, base);
    for (int s = 0; s < b.n_levels; ++s) {
      const int64_t n = b.item_begin[s + 1] - b.item_begin[s];
      if (n == 0) continue;
      const int grid = (int)std::min<int64_t>((n + FW_WARPS - 1) / FW_WARPS, (int64_t)c.ctas_per_sm * sms);
      int* cnt = b.d_counters + (size_t)ch * b.n_levels + s;
      if (b.f32)
        batch_level_kernel<float2><<<grid, FW_WARPS * 32, 0, b.st>>>(
            b.d_items + b.item_begin[s], (int)n, cnt, b.d_ops, base, b.rhs_chunk);
      else
        batch_level_kernel<float4><<<grid, FW_WARPS * 32, 0, b.st>>>(
            b.d_items + b.item_begin[s], (int)n, cnt, b.d_ops, base, b.rhs_chunk);
    }
    batch_combine_kernel<<<dim3(gx, b.n_pairs[ch]), 256, 0, b.st>>>(b.d_pairs[ch], b.d_ops, base);
    e = cudaGetLastError();
  }
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(b.st, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    set_error("batch: graph capture failed: %s",
              cudaGetErrorString(e != cudaSuccess ? e : e2));
    return BF_ECUDA;
  }
  b.graph = g;
  size_t nn = 0;
  BF_TRY_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
  b.graph_nodes = (int64_t)nn;
  BF_TRY_CUDA(cudaGraphInstantiate(&b.exec, g, 0));
  return BF_OK;
}

int configure(BatchState& b, const BatchCfg& c) {
  BF_TRY(build_items(b, c));
  BF_TRY(capture(b, c));
  b.cfg = c;
  return BF_OK;
}

}  // namespace
}  // namespace bfg

struct bf_batch {
  bfg::BatchState s;
};

using namespace bfg;

extern "C" {

int bf_batch_create(bf_ctx_t ctx, bf_op_t const* ops, const int32_t* nrhs, int32_t n_ops,
                    int32_t rhs_chunk, bf_batch_t* out) {
  try {
    if (!ctx || !ops || !nrhs || n_ops <= 0 || !out) {
      set_error("bf_batch_create: invalid arguments");
      return BF_EINVAL;
    }
    if (rhs_chunk <= 0) rhs_chunk = 8;
    auto h = std::make_unique<bf_batch>();
    BatchState& b = h->s;
    b.ctx = &ctx->c;
    b.rhs_chunk = rhs_chunk;
    int maxr = 0;
    for (int i = 0; i < n_ops; ++i) {
      if (!ops[i] || nrhs[i] < 1) {
        set_error("bf_batch_create: operator %d missing or nrhs < 1", i);
        return BF_EINVAL;
      }
      Operator& op = ops[i]->op;
      const bool f32 = op.d_A2 != nullptr;
      if (i == 0) b.f32 = f32;
      if (f32 != b.f32) {
        set_error("bf_batch_create: operators mix complex FP32 and float-float factors");
        return BF_ENOTSUP;
      }
      b.ops.push_back(&op);
      b.nrhs.push_back(nrhs[i]);
      b.n_levels = std::max<int>(b.n_levels, (int)op.plan.n_stages());
      maxr = std::max(maxr, nrhs[i]);
    }
    b.n_chunks = (maxr + rhs_chunk - 1) / rhs_chunk;
    BF_TRY_CUDA(cudaSetDevice(b.ctx->device));
    BF_TRY_CUDA(cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking));
    // per-operator buffers
    for (int i = 0; i < n_ops; ++i) {
      Operator& op = *b.ops[i];
      const Plan& p = op.plan;
      BatchOpDev o{};
      o.tasks = op.d_tasks;
      o.A = b.f32 ? (const void*)op.d_A2 : (const void*)op.d_A;
      o.maps = op.d_maps;
      o.xperm = op.d_xperm;
      o.yperm = op.d_yperm;
      o.ws_entries = p.ws_entries;
      o.xg_off = p.xg_off;
      o.yg_off = p.yg_off;
      o.n_rows = p.n_rows;
      o.n_cols = p.n_cols;
      o.nrhs = nrhs[i];
      o.yg_covered = p.yg_covered ? 1 : 0;
      const int nws = std::min(nrhs[i], rhs_chunk);
      void *ws = nullptr, *X = nullptr, *Y = nullptr;
      const size_t wsb = (size_t)std::max<int64_t>(p.ws_entries, 1) * nws * sizeof(float4);
      if (cudaMalloc(&ws, wsb) != cudaSuccess ||
          cudaMalloc(&X, (size_t)std::max<int64_t>(p.n_cols, 1) * nrhs[i] * sizeof(double2)) !=
              cudaSuccess ||
          cudaMalloc(&Y, (size_t)std::max<int64_t>(p.n_rows, 1) * nrhs[i] * sizeof(double2)) !=
              cudaSuccess) {
        cudaGetLastError();
        for (void* q : {ws, X, Y})
          if (q) cudaFree(q);
        set_error("bf_batch_create: out of device memory at operator %d", i);
        return BF_ENOMEM;
      }
      b.allocs.insert(b.allocs.end(), {ws, X, Y});
      b.ws_bytes += (int64_t)wsb;
      BF_TRY_CUDA(cudaMemset(ws, 0, wsb));
      BF_TRY_CUDA(cudaMemset(X, 0, (size_t)std::max<int64_t>(p.n_cols, 1) * nrhs[i] * sizeof(double2)));
      o.ws = (float4*)ws;
      o.X = (const double2*)X;
      o.Y = (double2*)Y;
      b.hops.push_back(o);
      b.max_n = std::max(b.max_n, std::max(p.n_rows, p.n_cols));
    }
    BF_TRY_CUDA(cudaMalloc(&b.d_ops, b.hops.size() * sizeof(BatchOpDev)));
    BF_TRY_CUDA(cudaMemcpy(b.d_ops, b.hops.data(), b.hops.size() * sizeof(BatchOpDev),
                           cudaMemcpyHostToDevice));
    for (int ch = 0; ch < b.n_chunks; ++ch) {
      std::vector<int2> pr;
      for (int i = 0; i < n_ops; ++i)
        for (int r = 0; r < rhs_chunk && ch * rhs_chunk + r < nrhs[i]; ++r)
          pr.push_back(make_int2(i, r));
      if (pr.size() > 65535) {
        set_error("bf_batch_create: %zu (operator, rhs) pairs per chunk exceed 65535", pr.size());
        return BF_EINVAL;
      }
      int2* d = nullptr;
      BF_TRY_CUDA(cudaMalloc(&d, std::max<size_t>(1, pr.size()) * sizeof(int2)));
      BF_TRY_CUDA(cudaMemcpy(d, pr.data(), pr.size() * sizeof(int2), cudaMemcpyHostToDevice));
      b.d_pairs.push_back(d);
      b.n_pairs.push_back((int)pr.size());
    }
    BF_TRY_CUDA(cudaMalloc(&b.d_counters, (size_t)std::max(1, b.n_chunks * b.n_levels) * sizeof(int)));
    BF_TRY(configure(b, b.cfg));
    *out = h.release();
    return BF_OK;
  } catch (const std::exception& e) {
    set_error("bf_batch_create: %s", e.what());
    return BF_ENOMEM;
  }
}

int bf_batch_destroy(bf_batch_t b) {
  delete b;
  return BF_OK;
}

int bf_batch_buffers(bf_batch_t h, int32_t op, double** x_dev, double** y_dev) {
  if (!h || op < 0 || op >= (int32_t)h->s.hops.size()) {
    set_error("bf_batch_buffers: invalid operator index");
    return BF_EINVAL;
  }
  if (x_dev) *x_dev = (double*)h->s.hops[op].X;
  if (y_dev) *y_dev = (double*)h->s.hops[op].Y;
  return BF_OK;
}

int bf_batch_run(bf_batch_t h, void* stream) {
  if (!h || !h->s.exec) {
    set_error("bf_batch_run: batch not configured");
    return BF_EINVAL;
  }
  BF_TRY_CUDA(cudaSetDevice(h->s.ctx->device));
  BF_TRY_CUDA(cudaGraphLaunch(h->s.exec, stream ? (cudaStream_t)stream : h->s.st));
  if (!stream) BF_TRY_CUDA(cudaStreamSynchronize(h->s.st));
  return BF_OK;
}

int bf_batch_matvec(bf_batch_t h, const double* const* x, const int64_t* ldx, double* const* y,
                    const int64_t* ldy, int ptr_mode, void* stream) {
  if (!h || !x || !y) {
    set_error("bf_batch_matvec: NULL argument");
    return BF_EINVAL;
  }
  if (ptr_mode != BF_PTR_HOST && ptr_mode != BF_PTR_DEVICE) {
    set_error("bf_batch_matvec: invalid ptr_mode %d", ptr_mode);
    return BF_EINVAL;
  }
  BatchState& b = h->s;
  BF_TRY_CUDA(cudaSetDevice(b.ctx->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : b.st;
  const cudaMemcpyKind kin = ptr_mode == BF_PTR_HOST ? cudaMemcpyHostToDevice
                                                     : cudaMemcpyDeviceToDevice;
  const cudaMemcpyKind kout = ptr_mode == BF_PTR_HOST ? cudaMemcpyDeviceToHost
                                                      : cudaMemcpyDeviceToDevice;
  for (size_t i = 0; i < b.hops.size(); ++i) {
    const BatchOpDev& o = b.hops[i];
    const int64_t lx = ldx ? ldx[i] : o.n_cols;
    if (!x[i] || lx < o.n_cols) {
      set_error("bf_batch_matvec: operator %zu: bad x or ldx", i);
      return BF_EINVAL;
    }
    BF_TRY_CUDA(cudaMemcpy2DAsync((void*)o.X, o.n_cols * sizeof(double2), x[i],
                                  lx * sizeof(double2), o.n_cols * sizeof(double2), o.nrhs, kin,
                                  st));
  }
  BF_TRY_CUDA(cudaGraphLaunch(b.exec, st));
  for (size_t i = 0; i < b.hops.size(); ++i) {
    const BatchOpDev& o = b.hops[i];
    const int64_t ly = ldy ? ldy[i] : o.n_rows;
    if (!y[i] || ly < o.n_rows) {
      set_error("bf_batch_matvec: operator %zu: bad y or ldy", i);
      return BF_EINVAL;
    }
    BF_TRY_CUDA(cudaMemcpy2DAsync(y[i], ly * sizeof(double2), o.Y, o.n_rows * sizeof(double2),
                                  o.n_rows * sizeof(double2), o.nrhs, kout, st));
  }
  if (ptr_mode == BF_PTR_HOST || !stream) BF_TRY_CUDA(cudaStreamSynchronize(st));
  return BF_OK;
}

int bf_batch_autotune(bf_batch_t h, int32_t nrep, double* best_ms, int32_t* best_cfg) {
  if (!h) {
    set_error("bf_batch_autotune: NULL batch");
    return BF_EINVAL;
  }
  BatchState& b = h->s;
  BF_TRY_CUDA(cudaSetDevice(b.ctx->device));
  if (nrep < 1) nrep = 1;
  cudaEvent_t e0, e1;
  BF_TRY_CUDA(cudaEventCreate(&e0));
  BF_TRY_CUDA(cudaEventCreate(&e1));
  struct EvGuard {
    cudaEvent_t a, b;
    ~EvGuard() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } eg{e0, e1};
  double best = 1e30;
  BatchCfg bc = b.cfg;
  for (int fm : {64, 96, 128})
    for (int bk : {0, 1})
      for (int cps : {2, 4, 6}) {
        BatchCfg c{fm, bk, cps};
        BF_TRY(configure(b, c));
        BF_TRY_CUDA(cudaGraphLaunch(b.exec, b.st));  // warm-up
        BF_TRY_CUDA(cudaEventRecord(e0, b.st));
        for (int r = 0; r < nrep; ++r) BF_TRY_CUDA(cudaGraphLaunch(b.exec, b.st));
        BF_TRY_CUDA(cudaEventRecord(e1, b.st));
        BF_TRY_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        BF_TRY_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms / nrep < best) {
          best = ms / nrep;
          bc = c;
        }
      }
  BF_TRY(configure(b, bc));
  if (best_ms) *best_ms = best;
  if (best_cfg) {
    best_cfg[0] = bc.flat_mmax;
    best_cfg[1] = bc.bucketed;
    best_cfg[2] = bc.ctas_per_sm;
  }
  return BF_OK;
}

int bf_batch_info(bf_batch_t h, int64_t* graph_nodes, int64_t* work_items, int64_t* ws_bytes,
                  int32_t* chunks) {
  if (!h) {
    set_error("bf_batch_info: NULL batch");
    return BF_EINVAL;
  }
  if (graph_nodes) *graph_nodes = h->s.graph_nodes;
  if (work_items) *work_items = h->s.item_begin.empty() ? 0 : h->s.item_begin.back();
  if (ws_bytes) *ws_bytes = h->s.ws_bytes;
  if (chunks) *chunks = h->s.n_chunks;
  return BF_OK;
}

}  // extern "C"
