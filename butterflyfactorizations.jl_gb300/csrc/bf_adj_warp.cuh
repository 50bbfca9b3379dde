// Warp-level adjoint / transpose task routine: out = op(A)^T v for one task,
// op = conj (adjoint, src/Butterflyalgebra/bfadjtr.jl:13-67) or identity
// (transpose), reading the forward factors in place (no copy).  Used by the
// adjoint level kernels (bf_adj.cu) and the operator-batch kernels
// (bf_batch.cu); workspace entry e of the right-hand side at hand is ws[e*S]
// (S = 1 on the single-vector path).
//
// A warp splits its lanes into RG row groups x CG = 32/RG column groups.  Lane
// (rg, cg) walks rows rg, rg+RG, ... of CPL columns; for a fixed column the RG
// lanes of a group read RG consecutive entries of the column-major matrix, so
// loads stay coalesced along columns.  After the row walk the RG partial sums
// of each column meet by xor-shuffles (log2 RG steps).
#pragma once

#include "bf_dfloat.cuh"
#include "bf_internal.h"

namespace bfg {

constexpr int ADJ_CPL = 4;  // max columns per lane per pass

__device__ __forceinline__ float4 shfl_xor4(float4 v, int m) {
  v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
  v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
  v.z = __shfl_xor_sync(0xffffffffu, v.z, m);
  v.w = __shfl_xor_sync(0xffffffffu, v.w, m);
  return v;
}

// input entry of row r; workspace entry e of this right-hand side is ws[e*S]
__device__ __forceinline__ float4 vin(const DTask& t, const int32_t* __restrict__ rmap,
                                      const float4* __restrict__ ws, int r, int S = 1) {
  return t.rbase >= 0 ? ws[((long long)t.rbase + r) * S] : ws[(long long)rmap[r] * S];
}

// row groups per column: 4 up to 64 rows (a lane walks up to 16 rows of a column
// and the partial sums meet in 2 shuffle steps; 8 groups for M in 33..64 spent a
// quarter of the arithmetic on the 3-step reduction: 6% slower adjoints with
// complex FP32 factors at 262,144 points)
__host__ __device__ __forceinline__ int rg_of(int M) { return M <= 8 ? 2 : (M <= 64 ? 4 : 8); }

constexpr int ADJ_VS = 128;  // staged input entries per warp

// input entries of rows [r, r + len) into the warp's staging buffer
__device__ __forceinline__ void adj_stage(const DTask& t, const int32_t* __restrict__ rmap,
                                          const float4* __restrict__ ws, float4* __restrict__ vs,
                                          int r, int len, int S = 1) {
  for (int i = threadIdx.x & 31; i < len; i += 32) vs[i] = vin(t, rmap, ws, r + i, S);
}

// Adds, for this lane, the partial sums of columns c = c0 + cg + CG*u (u < cpl)
// over rows [r_begin, r_end) whose input entries are staged at vs[r - vbase],
// every entry under a guard: the form the batch kernels keep (the unguarded
// one below takes registers their work-queue loop needs) and the level
// kernels use with complex FP32 factors.
// The input entries are gathered once into shared memory (adj_stage), so the
// row walk waits on the factor loads only, not on a routing-map lookup and a
// dependent workspace load per row.
template <bool CONJ, int RG, typename FT>
__device__ __forceinline__ void adj_accum_guarded(const DTask& t, const FT* __restrict__ A,
                                                  const float4* __restrict__ vs, int vbase,
                                                  int r_begin, int r_end, int c0, int cpl,
                                                  float4 acc[ADJ_CPL]) {
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

// Adds, for this lane, the partial sums of columns c = c0 + cg + CG*u (u < CPL)
// over rows [r_begin, r_end) whose input entries are staged at vs[r - vbase].
// The input entries are gathered once into shared memory (adj_stage), so the
// row walk waits on the factor loads only, not on a routing-map lookup and a
// dependent workspace load per row.  CPL is a template parameter and a column
// past the task's end reads column n - 1 instead (in bounds; its sum is never
// written), so the row walk carries no per-entry guards.
template <bool CONJ, int RG, int CPL, typename FT, int U = 1>
__device__ __forceinline__ void adj_accum(const DTask& t, const FT* __restrict__ A,
                                          const float4* __restrict__ vs, int vbase, int r_begin,
                                          int r_end, int c0, float4 acc[ADJ_CPL]) {
  constexpr int CG = 32 / RG;
  const int lane = threadIdx.x & 31;
  const int rg = lane % RG, cg = lane / RG;
  const int M = t.M, n = t.n;
  const FT* __restrict__ Ab = A + t.a_off;
  long long coff[CPL];
#pragma unroll
  for (int u = 0; u < CPL; ++u) coff[u] = (long long)min(c0 + cg + CG * u, n - 1) * M;
  // U = 2: two row steps per iteration.  That pays in the tall kernel (long
  // row walks, 80 registers at 3 CTAs per SM); in the warp kernels the extra
  // registers cost more occupancy than the extra loads in flight gained.
  int r = r_begin + rg;
  if constexpr (U == 2) {
    // two row steps per iteration, both steps' loads issued first
    for (; r + RG < r_end; r += 2 * RG) {
      const float4 v0 = vs[r - vbase], v1 = vs[r + RG - vbase];
      FT a0[CPL], a1[CPL];
#pragma unroll
      for (int u = 0; u < CPL; ++u) {
        a0[u] = __ldg(Ab + coff[u] + r);
        a1[u] = __ldg(Ab + coff[u] + r + RG);
      }
#pragma unroll
      for (int u = 0; u < CPL; ++u) {
        if (CONJ)
          cdf_mac_conj(acc[u], a0[u], v0);
        else
          cdf_mac(acc[u], a0[u], v0);
      }
#pragma unroll
      for (int u = 0; u < CPL; ++u) {
        if (CONJ)
          cdf_mac_conj(acc[u], a1[u], v1);
        else
          cdf_mac(acc[u], a1[u], v1);
      }
    }
  }
  for (; r < r_end; r += RG) {
    const float4 v = vs[r - vbase];
    FT a[CPL];
#pragma unroll
    for (int u = 0; u < CPL; ++u) a[u] = __ldg(Ab + coff[u] + r);
#pragma unroll
    for (int u = 0; u < CPL; ++u) {
      if (CONJ)
        cdf_mac_conj(acc[u], a[u], v);
      else
        cdf_mac(acc[u], a[u], v);
    }
  }
}

template <bool CONJ, int RG, typename FT, int U = 1>
__device__ __forceinline__ void adj_accum_n(const DTask& t, const FT* __restrict__ A,
                                            const float4* __restrict__ vs, int vbase,
                                            int r_begin, int r_end, int c0, int cpl,
                                            float4 acc[ADJ_CPL]) {
  static_assert(ADJ_CPL == 4, "one case per column count");
  switch (cpl) {
    case 1: adj_accum<CONJ, RG, 1, FT, U>(t, A, vs, vbase, r_begin, r_end, c0, acc); break;
    case 2: adj_accum<CONJ, RG, 2, FT, U>(t, A, vs, vbase, r_begin, r_end, c0, acc); break;
    case 3: adj_accum<CONJ, RG, 3, FT, U>(t, A, vs, vbase, r_begin, r_end, c0, acc); break;
    default: adj_accum<CONJ, RG, 4, FT, U>(t, A, vs, vbase, r_begin, r_end, c0, acc); break;
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
template <bool CONJ, int RG, typename FT, bool FAST = false, int U = 1>
__device__ __forceinline__ void adj_rows(const DTask& t, const FT* __restrict__ A,
                                         const int32_t* __restrict__ rmap,
                                         const float4* __restrict__ ws, float4* __restrict__ vs,
                                         bool staged, int r0, int r1, int c0, int cpl,
                                         float4 acc[ADJ_CPL], int S = 1) {
#pragma unroll
  for (int u = 0; u < ADJ_CPL; ++u) acc[u] = make_float4(0.f, 0.f, 0.f, 0.f);
  auto walk = [&](int vbase, int rb, int re) {
    if constexpr (FAST)
      adj_accum_n<CONJ, RG, FT, U>(t, A, vs, vbase, rb, re, c0, cpl, acc);
    else
      adj_accum_guarded<CONJ, RG, FT>(t, A, vs, vbase, rb, re, c0, cpl, acc);
  };
  if (staged) {
    walk(r0, r0, r1);
  } else {
    for (int rc = r0; rc < r1; rc += ADJ_VS) {  // chunk starts stay multiples of RG
      const int len = min(ADJ_VS, r1 - rc);
      __syncwarp();
      adj_stage(t, rmap, ws, vs, rc, len, S);
      __syncwarp();
      walk(rc, rc, rc + len);
    }
  }
  adj_reduce<RG>(acc, cpl);
}

__device__ __forceinline__ void write_out(const DTask& t, const int32_t* __restrict__ cmap,
                                          float4* __restrict__ ws, int c, float4 v, int S = 1) {
  if (t.cbase >= 0)
    ws[((long long)t.cbase + c) * S] = cdf_norm(v);
  else
    ws[(long long)cmap[c] * S] = cdf_norm(v);
}

// Columns per lane and pass for a task of n columns over CG column groups:
// the fewest passes of at most ADJ_CPL columns per lane, with the columns
// spread evenly over them.  (Filling every pass but the last would leave most
// lanes of the last pass idle while it walks all rows again: n = 18 over 4
// groups is 12 + 6 columns here instead of 16 + 2.)
__host__ __device__ __forceinline__ int adj_cpl(int n, int CG) {
  int np = (n + CG * ADJ_CPL - 1) / (CG * ADJ_CPL);
  np = np < 1 ? 1 : np;
  const int cpl = (n + CG * np - 1) / (CG * np);
  return cpl < 1 ? 1 : (cpl > ADJ_CPL ? ADJ_CPL : cpl);
}

// Column passes of a task for the warp routine below (per_pass columns
// each): the batch splits wide tasks into work items by pass.
__host__ __device__ __forceinline__ int adj_passes(int M, int n) {
  const int CG = 32 / rg_of(M);
  const int per_pass = CG * adj_cpl(n, CG);
  return (n + per_pass - 1) / per_pass;
}

template <bool CONJ, int RG, typename FT, bool FAST = false>
__device__ void adj_task_warp(const DTask& t, const FT* __restrict__ A,
                              const int32_t* __restrict__ maps, float4* __restrict__ ws,
                              float4* __restrict__ vs, int pass_begin, int pass_step,
                              int S = 1) {
  constexpr int CG = 32 / RG;
  const int lane = threadIdx.x & 31;
  const int rg = lane % RG, cg = lane / RG;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int cpl = adj_cpl(t.n, CG);
  const int per_pass = CG * cpl;
  // the task's input entries are staged once when they fit
  const bool staged = t.M <= ADJ_VS;
  if (staged) {
    adj_stage(t, rmap, ws, vs, 0, t.M, S);
    __syncwarp();
  }
  float4 acc[ADJ_CPL];
  for (int c0 = pass_begin * per_pass; c0 < t.n; c0 += pass_step * per_pass) {
    adj_rows<CONJ, RG, FT, FAST>(t, A, rmap, ws, vs, staged, 0, t.M, c0, cpl, acc, S);
    if (rg == 0) {
#pragma unroll
      for (int u = 0; u < ADJ_CPL; ++u) {
        const int c = c0 + cg + CG * u;
        if (u < cpl && c < t.n) write_out(t, cmap, ws, c, acc[u], S);
      }
    }
  }
  __syncwarp();
}

}  // namespace bfg
