// Adjoint / transpose level launches: out = op(A)^T v for every task, with
// op = conj (adjoint, src/Butterflyalgebra/bfadjtr.jl:13-67) or identity
// (transpose), reading the forward factors in place (no copy).
//
// A warp splits its lanes into RG row groups x CG = 32/RG column groups.  Lane
// (rg, cg) walks rows rg, rg+RG, ... of CPL columns; for a fixed column the RG
// lanes of a group read RG consecutive entries of the column-major matrix, so
// loads stay coalesced along columns.  After the row walk the RG partial sums
// of each column meet by xor-shuffles (log2 RG steps).  Launch shapes:
//   warp   : one warp per small task (all rows);
//   tall   : one CTA per tall task, warps split the rows, shared-memory sum;
//   wide   : one CTA per short wide task, warps split the column passes.
#include "bf_dfloat.cuh"
#include "bf_internal.h"

namespace bfg {
namespace {

constexpr int ADJ_CPL = 4;  // max columns per lane per pass

__device__ __forceinline__ float4 shfl_xor4(float4 v, int m) {
  v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
  v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
  v.z = __shfl_xor_sync(0xffffffffu, v.z, m);
  v.w = __shfl_xor_sync(0xffffffffu, v.w, m);
  return v;
}

__device__ __forceinline__ float4 vin(const DTask& t, const int32_t* __restrict__ rmap,
                                      const float4* __restrict__ ws, int r) {
  return t.rbase >= 0 ? ws[t.rbase + r] : ws[rmap[r]];
}

__device__ __forceinline__ int rg_of(int M) { return M <= 8 ? 2 : (M <= 32 ? 4 : 8); }

constexpr int ADJ_VS = 128;  // staged input entries per warp

// input entries of rows [r, r + len) into the warp's staging buffer
__device__ __forceinline__ void adj_stage(const DTask& t, const int32_t* __restrict__ rmap,
                                          const float4* __restrict__ ws, float4* __restrict__ vs,
                                          int r, int len) {
  for (int i = threadIdx.x & 31; i < len; i += 32) vs[i] = vin(t, rmap, ws, r + i);
}

// Adds, for this lane, the partial sums of columns c = c0 + cg + CG*u (u < cpl)
// over rows [r_begin, r_end) whose input entries are staged at vs[r - vbase].
// The input entries are gathered once into shared memory (adj_stage), so the
// row walk waits on the factor loads only, not on a routing-map lookup and a
// dependent workspace load per row.
template <bool CONJ, int RG, typename FT>
__device__ __forceinline__ void adj_accum(const DTask& t, const FT* __restrict__ A,
                                          const float4* __restrict__ vs, int vbase, int r_begin,
                                          int r_end, int c0, int cpl, float4 acc[ADJ_CPL]) {
  constexpr int CG = 32 / RG;
  const int lane = threadIdx.x & 31;
  const int rg = lane % RG, cg = lane / RG;
  const int M = t.M, n = t.n;
  const FT* __restrict__ Ab = A + t.a_off;
  // (two row steps per iteration were measured slower: the extra registers
  // cost more occupancy than the extra loads in flight gained)
  for (int r = r_begin + rg; r < r_end; r += RG) {
    const float4 v = vs[r - vbase];
    FT a[ADJ_CPL];
#pragma unroll
    for (int u = 0; u < ADJ_CPL; ++u) {
      const int c = c0 + cg + CG * u;
      a[u] = (u < cpl && c < n) ? __ldg(Ab + (size_t)c * M + r) : fac_zero<FT>();
    }
#pragma unroll
    for (int u = 0; u < ADJ_CPL; ++u) {
      if (u < cpl) {
        if (CONJ)
          cdf_mac_conj(acc[u], a[u], v);
        else
          cdf_mac(acc[u], a[u], v);
      }
    }
  }
}

// the RG partial sums of each column meet (every lane of the group holds the total)
template <int RG>
__device__ __forceinline__ void adj_reduce(float4 acc[ADJ_CPL], int cpl) {
#pragma unroll
  for (int m = 1; m < RG; m <<= 1)
#pragma unroll
    for (int u = 0; u < ADJ_CPL; ++u)
      if (u < cpl) cdf_add(acc[u], shfl_xor4(acc[u], m));
}

// rows [r0, r1) of column pass c0 for this warp: already staged (staged =
// true, at vs[r - r0]) or staged here in chunks of ADJ_VS rows
template <bool CONJ, int RG, typename FT>
__device__ __forceinline__ void adj_rows(const DTask& t, const FT* __restrict__ A,
                                         const int32_t* __restrict__ rmap,
                                         const float4* __restrict__ ws, float4* __restrict__ vs,
                                         bool staged, int r0, int r1, int c0, int cpl,
                                         float4 acc[ADJ_CPL]) {
#pragma unroll
  for (int u = 0; u < ADJ_CPL; ++u) acc[u] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (staged) {
    adj_accum<CONJ, RG, FT>(t, A, vs, r0, r0, r1, c0, cpl, acc);
  } else {
    for (int rc = r0; rc < r1; rc += ADJ_VS) {  // chunk starts stay multiples of RG
      const int len = min(ADJ_VS, r1 - rc);
      __syncwarp();
      adj_stage(t, rmap, ws, vs, rc, len);
      __syncwarp();
      adj_accum<CONJ, RG, FT>(t, A, vs, rc, rc, rc + len, c0, cpl, acc);
    }
  }
  adj_reduce<RG>(acc, cpl);
}

__device__ __forceinline__ void write_out(const DTask& t, const int32_t* __restrict__ cmap,
                                          float4* __restrict__ ws, int c, float4 v) {
  if (t.cbase >= 0)
    ws[t.cbase + c] = cdf_norm(v);
  else
    ws[cmap[c]] = cdf_norm(v);
}

template <bool CONJ, int RG, typename FT>
__device__ void adj_task_warp(const DTask& t, const FT* __restrict__ A,
                              const int32_t* __restrict__ maps, float4* __restrict__ ws,
                              float4* __restrict__ vs, int pass_begin, int pass_step) {
  constexpr int CG = 32 / RG;
  const int lane = threadIdx.x & 31;
  const int rg = lane % RG, cg = lane / RG;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int cpl = min(ADJ_CPL, (t.n + CG - 1) / CG);
  const int per_pass = CG * cpl;
  // the task's input entries are staged once when they fit
  const bool staged = t.M <= ADJ_VS;
  if (staged) {
    adj_stage(t, rmap, ws, vs, 0, t.M);
    __syncwarp();
  }
  float4 acc[ADJ_CPL];
  for (int c0 = pass_begin * per_pass; c0 < t.n; c0 += pass_step * per_pass) {
    adj_rows<CONJ, RG, FT>(t, A, rmap, ws, vs, staged, 0, t.M, c0, cpl, acc);
    if (rg == 0) {
#pragma unroll
      for (int u = 0; u < ADJ_CPL; ++u) {
        const int c = c0 + cg + CG * u;
        if (u < cpl && c < t.n) write_out(t, cmap, ws, c, acc[u]);
      }
    }
  }
  __syncwarp();
}

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
    case 2: adj_task_warp<CONJ, 2, FT>(t, A, maps, ws, vs, 0, 1); break;
    case 4: adj_task_warp<CONJ, 4, FT>(t, A, maps, ws, vs, 0, 1); break;
    default: adj_task_warp<CONJ, 8, FT>(t, A, maps, ws, vs, 0, 1); break;
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
    case 2: adj_task_warp<CONJ, 2, FT>(t, A, maps, ws, vsm[w], w, 8); break;
    case 4: adj_task_warp<CONJ, 4, FT>(t, A, maps, ws, vsm[w], w, 8); break;
    default: adj_task_warp<CONJ, 8, FT>(t, A, maps, ws, vsm[w], w, 8); break;
  }
}

// CTA per tall task (M > 128): the 8 warps split the rows; per column pass the
// warp partials meet in shared memory.
template <bool CONJ, typename FT>
__global__ void __launch_bounds__(256) adj_tall_kernel(const int32_t* __restrict__ tlist,
                                                       const DTask* __restrict__ tasks,
                                                       const FT* __restrict__ A,
                                                       const int32_t* __restrict__ maps,
                                                       float4* __restrict__ ws) {
  constexpr int RG = 8, CG = 4;
  __shared__ float4 red[8][CG * ADJ_CPL];
  __shared__ float4 vsm[8][ADJ_VS];
  const DTask t = tasks[tlist[blockIdx.x]];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rg = lane % RG, cg = lane / RG;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int cpl = min(ADJ_CPL, (t.n + CG - 1) / CG);
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
    adj_rows<CONJ, RG, FT>(t, A, rmap, ws, vsm[w], staged, r0, r1, c0, cpl, acc);
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
