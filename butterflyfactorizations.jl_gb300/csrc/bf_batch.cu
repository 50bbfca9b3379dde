// Many independent far-field operators, many right-hand sides each, in one
// launch sequence (bf_batch_*).
//
// The reference applies operators one at a time, one column at a time
// (src/Butterflyalgebra/bfmatrix.jl:10-75 inside each mul!), and builds an
// adjoint by copying every block (src/Butterflyalgebra/bfadjtr.jl:43-67).
// Here the level sequences of all operators are merged: merged level s holds
// level s of every forward operator and level L-1-s of every adjoint or
// transpose operator that has one.  Per merged level and task class there is
// ONE persistent launch (batch_level_kernel): warps take work items
// (operator, task, row panel or column-pass group) from an atomic queue and
// run the FP64-accurate warp routines of the single-operator path
// (bf_fwd_warp.cuh, bf_adj_warp.cuh) for the right-hand sides of the current
// chunk.  The forward routines apply every factor entry they load to up to
// four right-hand sides from registers; the adjoint routine walks the
// right-hand sides in turn (the task matrix comes from L2 after the first).
//
// Workspace: one per operator, entry-interleaved: level entry e of the
// chunk's right-hand side q sits at ws[e*S + q] (S = min(nrhs, rhs_chunk)),
// so the gather of one input entry for all right-hand sides is one
// contiguous run.  Chunks of rhs_chunk right-hand sides run one after the
// other.
//
// The whole sequence -- per chunk: one batched split (all operators and
// right-hand sides), the merged level launches, one batched combine -- is
// captured once into a CUDA graph and replayed by bf_batch_run, so a batch
// matvec costs a single graph launch.  The work-queue counters are reset by
// a memset node inside the graph.
//
// Autotuner (bf_batch_autotune): the number of right-hand sides a forward
// routine applies per factor load (1 or 4: registers against occupancy), the
// item order (longest first, or operator/task order for locality) and the
// persistent grid size (CTAs per SM) are chosen by timing graph replays of
// the actual batch for every candidate; the fastest is kept.
#include <algorithm>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>

#include "bf_adj_warp.cuh"
#include "bf_dfloat.cuh"
#include "bf_fwd_warp.cuh"
#include "bf_internal.h"

namespace bfg {
namespace {

// task classes of the batch kernels
enum : int32_t {
  BC_TALL = 0,   // forward, 64-row panel (M > 32)
  BC_SMALL = 1,  // forward, M <= 32
  BC_COPY = 2,   // identity block, forward
  BC_ADJ = 3,    // adjoint (conjugate transpose), a group of column passes
  BC_ADJT = 4,   // transpose, a group of column passes
  BC_COPYR = 5,  // identity block, adjoint / transpose
  BC_N = 6
};

// r0: first row of a tall panel, or the first column pass of an adjoint item;
// aux: pass stride of an adjoint item (its passes are r0, r0 + aux, ...)
struct alignas(16) BatchItem {
  int32_t op, task, r0, aux;
};

struct BatchOpDev {
  const DTask* tasks;
  const void* A;          // float2 or float4 entries (one type per batch)
  const int32_t* maps;
  float4* ws;             // ws_entries x S, entry-interleaved
  const int32_t* in_perm;   // leaf order of the input region
  const int32_t* out_perm;  // leaf order of the output region
  const double2* X;       // n_in x nrhs, column-major
  double2* Y;             // n_out x nrhs
  long long ws_entries, in_off, out_off, n_in, n_out;
  int nrhs, S, out_covered, trans;
};

struct BatchCfg {
  int nr_max;       // right-hand sides per factor load in the forward routines: 1 or 4
  int order;        // 0 = longest item first, 1 = operator / task order
  int ctas_per_sm;  // persistent grid = ctas_per_sm x SMs
};

// NR right-hand sides starting at ws (stride S) for one forward item
template <typename FT, int CLS, int NR>
__device__ __forceinline__ void batch_fwd(const BatchItem& it, const DTask& t, const FT* A,
                                          const BatchOpDev& o, float4* ws, float4* xw) {
  if constexpr (CLS == BC_TALL) {
    warp_tall<FT, NR>(t, it.r0, A, o.maps, ws, xw, o.S);
  } else if constexpr (CLS == BC_SMALL) {
    warp_small<FT, NR>(t, A, o.maps, ws, xw, o.S);
  } else {
    warp_copy<NR>(t, o.maps, ws, CLS == BC_COPYR ? 1 : 0, o.S);
    __syncwarp();
  }
}

template <typename FT, int CLS, int NRMAX>
__global__ void __launch_bounds__(FW_WARPS * 32) batch_level_kernel(
    const BatchItem* __restrict__ items, int n_items, int* __restrict__ counter,
    const BatchOpDev* __restrict__ ops, int rhs_base) {
  __shared__ float4 xs[FW_WARPS][FW_XB];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    int i = 0;
    if (lane == 0) i = atomicAdd(counter, 1);
    i = __shfl_sync(0xffffffffu, i, 0);
    if (i >= n_items) break;
    const BatchItem it = items[i];
    const BatchOpDev& o = ops[it.op];
    const int nr = min(o.S, o.nrhs - rhs_base);
    if (nr <= 0) continue;
    const DTask t = o.tasks[it.task];
    const FT* A = static_cast<const FT*>(o.A);
    if constexpr (CLS == BC_ADJ || CLS == BC_ADJT) {
      constexpr bool CONJ = CLS == BC_ADJ;
      for (int r = 0; r < nr; ++r) {
        float4* ws = o.ws + r;
        switch (rg_of(t.M)) {
          case 2: adj_task_warp<CONJ, 2, FT>(t, A, o.maps, ws, xs[warp], it.r0, it.aux, o.S); break;
          case 4: adj_task_warp<CONJ, 4, FT>(t, A, o.maps, ws, xs[warp], it.r0, it.aux, o.S); break;
          default: adj_task_warp<CONJ, 8, FT>(t, A, o.maps, ws, xs[warp], it.r0, it.aux, o.S); break;
        }
      }
    } else {
      int r = 0;
      if constexpr (NRMAX >= 4)
        for (; r + 4 <= nr; r += 4) batch_fwd<FT, CLS, 4>(it, t, A, o, o.ws + r, xs[warp]);
      if constexpr (NRMAX >= 2)
        for (; r + 2 <= nr; r += 2) batch_fwd<FT, CLS, 2>(it, t, A, o, o.ws + r, xs[warp]);
      for (; r < nr; ++r) batch_fwd<FT, CLS, 1>(it, t, A, o, o.ws + r, xs[warp]);
    }
  }
}

// x of every (operator, right-hand side) pair of the chunk -> the input region
// of its workspace (float-float, leaf order); zeroes output regions that no
// task covers.  blockIdx.y = pair (int2 {op, local rhs}).
__global__ void batch_split_kernel(const int2* __restrict__ pairs, const BatchOpDev* __restrict__ ops,
                                   int rhs_base) {
  const int2 pr = pairs[blockIdx.y];
  const BatchOpDev& o = ops[pr.x];
  const int S = o.S, r = pr.y;
  const double2* x = o.X + (size_t)(rhs_base + r) * o.n_in;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < o.n_in;
       q += (long long)gridDim.x * blockDim.x) {
    const double2 v = x[o.in_perm[q]];
    const float2 re = df_split(v.x), im = df_split(v.y);
    o.ws[(o.in_off + q) * S + r] = make_float4(re.x, re.y, im.x, im.y);
  }
  if (!o.out_covered)
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < o.n_out;
         q += (long long)gridDim.x * blockDim.x)
      o.ws[(o.out_off + q) * S + r] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void batch_combine_kernel(const int2* __restrict__ pairs,
                                     const BatchOpDev* __restrict__ ops, int rhs_base) {
  const int2 pr = pairs[blockIdx.y];
  const BatchOpDev& o = ops[pr.x];
  const int S = o.S, r = pr.y;
  double2* y = o.Y + (size_t)(rhs_base + r) * o.n_out;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < o.n_out;
       q += (long long)gridDim.x * blockDim.x) {
    const float4 a = o.ws[(o.out_off + q) * S + r];
    y[o.out_perm[q]] = make_double2((double)a.x + (double)a.y, (double)a.z + (double)a.w);
  }
}

}  // namespace

struct BatchState {
  Context* ctx = nullptr;
  std::vector<Operator*> ops;
  std::vector<int32_t> nrhs, trans;
  int rhs_chunk = 8;
  bool f32 = true;
  int n_levels = 0, n_chunks = 0;
  std::vector<BatchOpDev> hops;
  BatchOpDev* d_ops = nullptr;
  std::vector<void*> allocs;  // workspaces, X, Y
  std::vector<int2*> d_pairs;  // per chunk
  std::vector<int> n_pairs;
  int64_t max_n = 0;
  // work items per (merged level, class) for the current configuration:
  // item_begin[s * BC_N + c] .. item_begin[s * BC_N + c + 1]
  BatchItem* d_items = nullptr;
  std::vector<int64_t> item_begin;
  int* d_counters = nullptr;  // n_chunks * n_levels * BC_N
  BatchCfg cfg{4, 0, 4};
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

// work items of every merged level for configuration c
int build_items(BatchState& b, const BatchCfg& c) {
  std::vector<std::pair<int64_t, BatchItem>> cls[BC_N];
  std::vector<BatchItem> flat;
  b.item_begin.assign((size_t)b.n_levels * BC_N + 1, 0);
  for (int s = 0; s < b.n_levels; ++s) {
    for (auto& v : cls) v.clear();
    for (size_t oi = 0; oi < b.ops.size(); ++oi) {
      const Plan& p = b.ops[oi]->plan;
      const int64_t ns = p.n_stages();
      if (s >= ns) continue;
      const bool fwd = b.trans[oi] == BF_OP_N;
      const int64_t st = fwd ? s : ns - 1 - s;  // adjoints walk the levels backwards
      const int64_t w = b.nrhs[oi];
      for (int64_t ti = p.stage_begin[st]; ti < p.stage_begin[st + 1]; ++ti) {
        const DTask& t = p.tasks[ti];
        if (t.M <= 0) continue;
        BatchItem it{(int32_t)oi, (int32_t)ti, 0, 0};
        if (t.kind == TASK_COPY) {
          cls[fwd ? BC_COPY : BC_COPYR].push_back({(int64_t)t.M * w, it});
        } else if (!fwd) {
          // column passes split round-robin over up to 8 items per task
          const int passes = adj_passes(t.M, t.n);
          const int k = std::max(1, std::min(passes, 8));
          it.aux = k;
          for (int q = 0; q < k; ++q) {
            it.r0 = q;
            cls[b.trans[oi] == BF_OP_C ? BC_ADJ : BC_ADJT].push_back(
                {(int64_t)t.M * t.n * w / k, it});
          }
        } else if (t.M <= 32) {
          cls[BC_SMALL].push_back({(int64_t)t.M * t.n * w, it});
        } else {
          for (int r0 = 0; r0 < t.M; r0 += TALL_ROWS) {
            it.r0 = r0;
            cls[BC_TALL].push_back({(int64_t)std::min(TALL_ROWS, t.M - r0) * t.n * w, it});
          }
        }
      }
    }
    for (int q = 0; q < BC_N; ++q) {
      auto& v = cls[q];
      if (c.order == 0)
        std::stable_sort(v.begin(), v.end(),
                         [](const auto& a, const auto& x) { return a.first > x.first; });
      b.item_begin[(size_t)s * BC_N + q] = (int64_t)flat.size();
      for (auto& a : v) flat.push_back(a.second);
    }
  }
  b.item_begin[(size_t)b.n_levels * BC_N] = (int64_t)flat.size();
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

template <typename FT>
void launch_class(int c, int nr_max, int grid, cudaStream_t st, const BatchItem* items, int n,
                  int* cnt, const BatchOpDev* ops, int base) {
  const int T = FW_WARPS * 32;
#define BF_BATCH_LAUNCH(CLS, NRM) \
  batch_level_kernel<FT, CLS, NRM><<<grid, T, 0, st>>>(items, n, cnt, ops, base)
  switch (c) {
    case BC_TALL:
      if (nr_max >= 4) BF_BATCH_LAUNCH(BC_TALL, 4); else BF_BATCH_LAUNCH(BC_TALL, 1);
      break;
    case BC_SMALL:
      if (nr_max >= 4) BF_BATCH_LAUNCH(BC_SMALL, 4); else BF_BATCH_LAUNCH(BC_SMALL, 1);
      break;
    case BC_COPY: BF_BATCH_LAUNCH(BC_COPY, 4); break;
    case BC_COPYR: BF_BATCH_LAUNCH(BC_COPYR, 4); break;
    case BC_ADJ: BF_BATCH_LAUNCH(BC_ADJ, 1); break;
    default: BF_BATCH_LAUNCH(BC_ADJT, 1); break;
  }
#undef BF_BATCH_LAUNCH
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
  const size_t ncnt = (size_t)b.n_chunks * b.n_levels * BC_N;
  e = cudaMemsetAsync(b.d_counters, 0, ncnt * sizeof(int), b.st);
  for (int ch = 0; ch < b.n_chunks && e == cudaSuccess; ++ch) {
    const int base = ch * b.rhs_chunk;
    const unsigned gx = (unsigned)std::min<int64_t>((b.max_n + 255) / 256, 4 * sms);
    batch_split_kernel<<<dim3(gx, b.n_pairs[ch]), 256, 0, b.st>>>(b.d_pairs[ch], b.d_ops, base);
    for (int s = 0; s < b.n_levels; ++s)
      for (int q = 0; q < BC_N; ++q) {
        const size_t k = (size_t)s * BC_N + q;
        const int64_t n = b.item_begin[k + 1] - b.item_begin[k];
        if (n == 0) continue;
        const int grid = (int)std::min<int64_t>((n + FW_WARPS - 1) / FW_WARPS,
                                                (int64_t)c.ctas_per_sm * sms);
        int* cnt = b.d_counters + ((size_t)ch * b.n_levels + s) * BC_N + q;
        if (b.f32)
          launch_class<float2>(q, c.nr_max, grid, b.st, b.d_items + b.item_begin[k], (int)n, cnt,
                               b.d_ops, base);
        else
          launch_class<float4>(q, c.nr_max, grid, b.st, b.d_items + b.item_begin[k], (int)n, cnt,
                               b.d_ops, base);
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

namespace bfg {

int batch_create(Context* ctx, Operator* const* ops, const int32_t* trans, const int32_t* nrhs,
                 int32_t n_ops, int32_t rhs_chunk, bf_batch** out) {
  try {
    if (!ctx || !ops || !nrhs || n_ops <= 0 || !out) {
      set_error("bf_batch_create: invalid arguments");
      return BF_EINVAL;
    }
    if (rhs_chunk <= 0) rhs_chunk = 8;
    auto h = std::make_unique<bf_batch>();
    BatchState& b = h->s;
    b.ctx = ctx;
    b.rhs_chunk = rhs_chunk;
    int maxr = 0;
    for (int i = 0; i < n_ops; ++i) {
      if (!ops[i] || nrhs[i] < 1) {
        set_error("bf_batch_create: operator %d missing or nrhs < 1", i);
        return BF_EINVAL;
      }
      const int tr = trans ? trans[i] : BF_OP_N;
      if (tr != BF_OP_N && tr != BF_OP_C && tr != BF_OP_T) {
        set_error("bf_batch_create: operator %d has invalid trans %d", i, tr);
        return BF_EINVAL;
      }
      Operator& op = *ops[i];
      if (op.near) {
        set_error("bf_batch_create: operator %d has a near field; batches apply far fields "
                  "(use bf_matvec for near + far)", i);
        return BF_ENOTSUP;
      }
      const bool f32 = op.d_A2 != nullptr;
      if (i == 0) b.f32 = f32;
      if (f32 != b.f32) {
        set_error("bf_batch_create: operators mix complex FP32 and float-float factors");
        return BF_ENOTSUP;
      }
      b.ops.push_back(&op);
      b.nrhs.push_back(nrhs[i]);
      b.trans.push_back(tr);
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
      const bool fwd = b.trans[i] == BF_OP_N;
      BatchOpDev o{};
      o.tasks = op.d_tasks;
      o.A = b.f32 ? (const void*)op.d_A2 : (const void*)op.d_A;
      o.maps = op.d_maps;
      o.in_perm = fwd ? op.d_xperm : op.d_yperm;
      o.out_perm = fwd ? op.d_yperm : op.d_xperm;
      o.ws_entries = p.ws_entries;
      o.in_off = fwd ? p.xg_off : p.yg_off;
      o.out_off = fwd ? p.yg_off : p.xg_off;
      o.n_in = fwd ? p.n_cols : p.n_rows;
      o.n_out = fwd ? p.n_rows : p.n_cols;
      o.nrhs = nrhs[i];
      o.S = std::min(nrhs[i], rhs_chunk);
      o.out_covered = (fwd ? p.yg_covered : p.xg_covered) ? 1 : 0;
      o.trans = b.trans[i];
      void *ws = nullptr, *X = nullptr, *Y = nullptr;
      const size_t wsb = (size_t)std::max<int64_t>(p.ws_entries, 1) * o.S * sizeof(float4);
      const size_t xb = (size_t)std::max<int64_t>(o.n_in, 1) * nrhs[i] * sizeof(double2);
      const size_t yb = (size_t)std::max<int64_t>(o.n_out, 1) * nrhs[i] * sizeof(double2);
      if (cudaMalloc(&ws, wsb) != cudaSuccess || cudaMalloc(&X, xb) != cudaSuccess ||
          cudaMalloc(&Y, yb) != cudaSuccess) {
        cudaGetLastError();
        for (void* q : {ws, X, Y})
          if (q) cudaFree(q);
        set_error("bf_batch_create: out of device memory at operator %d", i);
        return BF_ENOMEM;
      }
      b.allocs.insert(b.allocs.end(), {ws, X, Y});
      b.ws_bytes += (int64_t)wsb;
      BF_TRY_CUDA(cudaMemset(ws, 0, wsb));
      BF_TRY_CUDA(cudaMemset(X, 0, xb));
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
        for (int r = 0; r < b.hops[i].S && ch * rhs_chunk + r < nrhs[i]; ++r)
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
    BF_TRY_CUDA(cudaMalloc(&b.d_counters,
                           (size_t)std::max(1, b.n_chunks * b.n_levels * BC_N) * sizeof(int)));
    BF_TRY(configure(b, b.cfg));
    *out = h.release();
    return BF_OK;
  } catch (const std::exception& e) {
    set_error("bf_batch_create: %s", e.what());
    return BF_ENOMEM;
  }
}

void batch_destroy(bf_batch* b) { delete b; }

int batch_buffers(bf_batch* b, int op, double2** x, double2** y) {
  if (!b || op < 0 || op >= (int)b->s.hops.size()) {
    set_error("batch: invalid operator index");
    return BF_EINVAL;
  }
  *x = (double2*)b->s.hops[op].X;
  *y = b->s.hops[op].Y;
  return BF_OK;
}

int batch_launch(bf_batch* b, cudaStream_t st) {
  BF_TRY_CUDA(cudaGraphLaunch(b->s.exec, st));
  return BF_OK;
}

}  // namespace bfg

extern "C" {

int bf_batch_create_op(bf_ctx_t ctx, bf_op_t const* ops, const int32_t* trans,
                       const int32_t* nrhs, int32_t n_ops, int32_t rhs_chunk, bf_batch_t* out) {
  if (!ctx || !ops || !nrhs || n_ops <= 0 || !out) {
    set_error("bf_batch_create: invalid arguments");
    return BF_EINVAL;
  }
  std::vector<Operator*> v((size_t)n_ops);
  for (int i = 0; i < n_ops; ++i) v[i] = ops[i] ? &ops[i]->op : nullptr;
  return batch_create(&ctx->c, v.data(), trans, nrhs, n_ops, rhs_chunk, out);
}

int bf_batch_create(bf_ctx_t ctx, bf_op_t const* ops, const int32_t* nrhs, int32_t n_ops,
                    int32_t rhs_chunk, bf_batch_t* out) {
  return bf_batch_create_op(ctx, ops, nullptr, nrhs, n_ops, rhs_chunk, out);
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
    const int64_t lx = ldx ? ldx[i] : o.n_in;
    if (!x[i] || lx < o.n_in) {
      set_error("bf_batch_matvec: operator %zu: bad x or ldx", i);
      return BF_EINVAL;
    }
    BF_TRY_CUDA(cudaMemcpy2DAsync((void*)o.X, o.n_in * sizeof(double2), x[i],
                                  lx * sizeof(double2), o.n_in * sizeof(double2), o.nrhs, kin,
                                  st));
  }
  BF_TRY_CUDA(cudaGraphLaunch(b.exec, st));
  for (size_t i = 0; i < b.hops.size(); ++i) {
    const BatchOpDev& o = b.hops[i];
    const int64_t ly = ldy ? ldy[i] : o.n_out;
    if (!y[i] || ly < o.n_out) {
      set_error("bf_batch_matvec: operator %zu: bad y or ldy", i);
      return BF_EINVAL;
    }
    BF_TRY_CUDA(cudaMemcpy2DAsync(y[i], ly * sizeof(double2), o.Y, o.n_out * sizeof(double2),
                                  o.n_out * sizeof(double2), o.nrhs, kout, st));
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
  for (int nrm : {1, 4})
    for (int ord : {0, 1})
      for (int cps : {2, 4, 6}) {
        BatchCfg c{nrm, ord, cps};
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
    best_cfg[0] = bc.nr_max;
    best_cfg[1] = bc.order;
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
