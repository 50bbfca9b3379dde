// Adjoint / transpose level launches: out = op(A)^T v for every task, with
// op = conj (adjoint, src/Butterflyalgebra/bfadjtr.jl:13-67) or identity
// (transpose), reading the forward factors in place (no copy).  The warp
// routine (row groups x column groups, shuffle reductions) is in
// bf_adj_warp.cuh.  Launch shapes:
//   warp   : one warp per small task (all rows);
//   tall   : one CTA per tall task, warps split the rows, shared-memory sum;
//   wide   : one CTA per short wide task, warps split the column passes.
#include "bf_adj_warp.cuh"
#include "bf_dfloat.cuh"
#include "bf_internal.h"

namespace bfg {
namespace {

// Row walks without per-entry guards (adj_accum) for float-float factors:
// 17.73 -> 15.69 ms for the adjoint of the 262,144-point sphere operator.
// With complex FP32 factors they made the Q-level kernel spill and the whole
// adjoint slower (12.98 -> 13.71 ms), so those keep the guarded walk.  The
// tall kernel's walk takes two row steps per iteration, both steps' loads
// issued first (80 registers, no spills; its level 3.20 -> 3.11 ms).
template <typename FT>
constexpr bool UNGUARDED = sizeof(FT) == sizeof(float4);

// warp per task (small tasks)
template <bool CONJ, typename FT>
__global__ void __launch_bounds__(256) adj_warp_kernel(const int32_t* __restrict__ tlist,
                                                       int n_tasks,
                                                       const DTask* __restrict__ tasks,
                                                       const FT* __restrict__ A,
                                                       const int32_t* __restrict__ maps,
                                                       float4* __restrict__ ws) {
  __shared__ float4 vsm[8][ADJ_VS];
  const int ti = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (ti >= n_tasks) return;
  const DTask t = tasks[tlist[ti]];
  float4* vs = vsm[threadIdx.x >> 5];
  switch (rg_of(t.M)) {
    case 2: adj_task_warp<CONJ, 2, FT, UNGUARDED<FT>>(t, A, maps, ws, vs, 0, 1); break;
    case 4: adj_task_warp<CONJ, 4, FT, UNGUARDED<FT>>(t, A, maps, ws, vs, 0, 1); break;
    default: adj_task_warp<CONJ, 8, FT, UNGUARDED<FT>>(t, A, maps, ws, vs, 0, 1); break;
  }
}

// CTA per wide task: the 8 warps take column passes round-robin
template <bool CONJ, typename FT>
__global__ void __launch_bounds__(256) adj_wide_kernel(const int32_t* __restrict__ tlist,
                                                       const DTask* __restrict__ tasks,
                                                       const FT* __restrict__ A,
                                                       const int32_t* __restrict__ maps,
                                                       float4* __restrict__ ws) {
  __shared__ float4 vsm[8][ADJ_VS];
  const DTask t = tasks[tlist[blockIdx.x]];
  const int w = threadIdx.x >> 5;
  switch (rg_of(t.M)) {
    case 2: adj_task_warp<CONJ, 2, FT, UNGUARDED<FT>>(t, A, maps, ws, vsm[w], w, 8); break;
    case 4: adj_task_warp<CONJ, 4, FT, UNGUARDED<FT>>(t, A, maps, ws, vsm[w], w, 8); break;
    default: adj_task_warp<CONJ, 8, FT, UNGUARDED<FT>>(t, A, maps, ws, vsm[w], w, 8); break;
  }
}

// CTA per tall task (M > 128): the 8 warps split the rows; per column pass the
// warp partials meet in shared memory.
// One CTA per task with more than ADJ_TALL_M rows: the 8 warps split the rows
// (in multiples of RG), each warp walks its rows for RG row groups x CG = 32/RG
// column groups, and the warps' column sums meet in shared memory.  A task of
// more than 16 columns takes RG = 4 (one column pass up to 32 columns) instead
// of RG = 8 (two passes, each staging the rows' inputs again).
template <bool CONJ, typename FT, int RG>
__device__ __forceinline__ void adj_tall_task(const DTask& t, const FT* __restrict__ A,
                                              const int32_t* __restrict__ maps,
                                              float4* __restrict__ ws, float4 (*red)[32],
                                              float4 (*vsm)[ADJ_VS]) {
  constexpr int CG = 32 / RG;
  static_assert(CG * ADJ_CPL <= 32, "reduction buffer");
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rg = lane % RG, cg = lane / RG;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int cpl = adj_cpl(t.n, CG);
  const int per_pass = CG * cpl;
  // row split in multiples of RG so that row groups stay aligned
  const int rows_per_warp = ((t.M + 8 * RG - 1) / (8 * RG)) * RG;
  const int r0 = min(t.M, w * rows_per_warp), r1 = min(t.M, r0 + rows_per_warp);
  // a warp's rows are staged once when they fit
  const bool staged = r1 - r0 <= ADJ_VS;
  if (staged) {
    adj_stage(t, rmap, ws, vsm[w], r0, r1 - r0);
    __syncwarp();
  }
  float4 acc[ADJ_CPL];
  for (int c0 = 0; c0 < t.n; c0 += per_pass) {
    adj_rows<CONJ, RG, FT, UNGUARDED<FT>, 2>(t, A, rmap, ws, vsm[w], staged, r0, r1, c0, cpl, acc);
    if (rg == 0) {
#pragma unroll
      for (int u = 0; u < ADJ_CPL; ++u)
        if (u < cpl) red[w][cg + CG * u] = acc[u];
    }
    __syncthreads();
    if (threadIdx.x < per_pass) {
      const int c = c0 + threadIdx.x;
      if (c < t.n) {
        float4 v = red[0][threadIdx.x];
        for (int q = 1; q < 8; ++q) cdf_add(v, red[q][threadIdx.x]);
        write_out(t, cmap, ws, c, v);
      }
    }
    __syncthreads();
  }
}

// float-float factors: at least 3 CTAs per SM, which lets the walk keep its
// 80 registers (left to itself the compiler chose 64 and spilled, 2.87 against
// 2.26 ms for the Q level's adjoint at 262,144 points); complex FP32 factors
// do better with the compiler's own choice (0: no minimum; 60 registers, 1.99
// against 2.34 ms with the minimum of 3)
template <typename FT>
constexpr int ADJ_TALL_MINB = sizeof(FT) == sizeof(float4) ? 3 : 0;

template <bool CONJ, typename FT>
__global__ void __launch_bounds__(256, ADJ_TALL_MINB<FT>) adj_tall_kernel(const int32_t* __restrict__ tlist,
                                                       const DTask* __restrict__ tasks,
                                                       const FT* __restrict__ A,
                                                       const int32_t* __restrict__ maps,
                                                       float4* __restrict__ ws) {
  __shared__ float4 red[8][32];
  __shared__ float4 vsm[8][ADJ_VS];
  const DTask t = tasks[tlist[blockIdx.x]];
  if (t.n > 16)  // block-uniform
    adj_tall_task<CONJ, FT, 4>(t, A, maps, ws, red, vsm);
  else
    adj_tall_task<CONJ, FT, 8>(t, A, maps, ws, red, vsm);
}

}  // namespace

template <typename FT>
static int launch_adj_stage_t(const Plan& p, int64_t s, bool conj, const int32_t* d_lists,
                              const DTask* d_tasks, const FT* d_A, const int32_t* d_maps,
                              float4* d_ws, cudaStream_t st) {
  auto range = [&](int c, int64_t& b, int64_t& n) {
    b = p.list_begin[c][s];
    n = p.list_begin[c][s + 1] - b;
  };
  int nk = 0;
  int64_t b, n;
  range(Plan::L_AWARP, b, n);
  if (n > 0) {
    unsigned g = (unsigned)((n + 7) / 8);
    if (conj)
      adj_warp_kernel<true, FT><<<g, 256, 0, st>>>(d_lists + b, (int)n, d_tasks, d_A, d_maps, d_ws);
    else
      adj_warp_kernel<false, FT><<<g, 256, 0, st>>>(d_lists + b, (int)n, d_tasks, d_A, d_maps, d_ws);
    ++nk;
  }
  range(Plan::L_WIDE, b, n);
  if (n > 0) {
    if (conj)
      adj_wide_kernel<true, FT><<<(unsigned)n, 256, 0, st>>>(d_lists + b, d_tasks, d_A, d_maps, d_ws);
    else
      adj_wide_kernel<false, FT><<<(unsigned)n, 256, 0, st>>>(d_lists + b, d_tasks, d_A, d_maps, d_ws);
    ++nk;
  }
  range(Plan::L_ATALL, b, n);
  if (n > 0) {
    if (conj)
      adj_tall_kernel<true, FT><<<(unsigned)n, 256, 0, st>>>(d_lists + b, d_tasks, d_A, d_maps, d_ws);
    else
      adj_tall_kernel<false, FT><<<(unsigned)n, 256, 0, st>>>(d_lists + b, d_tasks, d_A, d_maps, d_ws);
    ++nk;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("adjoint launch failed: %s", cudaGetErrorString(e));
    return -1;
  }
  return nk;
}

int launch_adj_stage(const Plan& p, int64_t s, bool conj, const int32_t* d_lists,
                     const DTask* d_tasks, const float4* d_A, const float2* d_A2,
                     const int32_t* d_maps, float4* d_ws, cudaStream_t st) {
  if (d_A2) return launch_adj_stage_t<float2>(p, s, conj, d_lists, d_tasks, d_A2, d_maps, d_ws, st);
  return launch_adj_stage_t<float4>(p, s, conj, d_lists, d_tasks, d_A, d_maps, d_ws, st);
}

}  // namespace bfg
