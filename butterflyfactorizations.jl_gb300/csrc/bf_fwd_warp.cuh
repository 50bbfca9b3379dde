// Warp-level forward task routines of the FP64-accurate matvec (float-float
// vectors, factor entries FT = float4 float-float or float2 complex FP32).
//
// Each routine computes, for one dense task t (bf_internal.h DTask),
// ws[rows] = A_t * ws[cols] with the row / column slots addressed through the
// routing maps (or a contiguous base), reading every factor entry once with
// coalesced loads and staging the inputs in warp-private shared memory
// (xw: FW_XB entries, aw: FLAT_MMAX row accumulators).  They are the level
// routines of the per-shape kernels (bf_matvec.cu) and of the operator-batch
// kernels (bf_batch.cu).  The tall, small and copy routines take NR
// right-hand sides at once: workspace entry e of right-hand side q is
// ws[e*S + q] (S >= NR; the single-vector path has NR = S = 1), and every
// factor entry loaded is applied to all NR of them from registers.  Blackwell's paired FP32
// instructions (__ffma2_rn and relatives) were measured slower here: a pair
// costs the FMA pipes as much as two scalar operations, and the operand
// broadcasts they need add instructions.
//   tall  : one 64-row panel of a task with M > 128, 2 rows per lane;
//   flat  : 32 < M <= 128, n <= 256, the warp streams all M*n entries;
//   small : M <= 32, G = 32/M lane groups on interleaved columns;
//   copy  : identity blocks (also used by the batch kernel, bf_batch.cu).
// warp_tall_one / warp_small_one are the single-vector forms of tall and small
// used by the per-shape kernels: their whole column batches run without guards
// (same products in the same order, same bits); the batch kernels keep the
// guarded forms, whose register budget their NR accumulators need.
#pragma once

#include "bf_dfloat.cuh"
#include "bf_internal.h"

namespace bfg {

constexpr int FW_WARPS = 8;
constexpr int FW_XB = 256;                // staged input entries per warp per pass
constexpr int TALL_RPL = TALL_ROWS / 32;  // rows per lane in a tall panel

// floor(n / d) for 0 <= n < 4096 and 1 <= d <= 64 through the fast reciprocal:
// (n + 1/2) / d lies at least 1/(2d) >= 1/128 away from an integer, and
// __fdividef's error (2 ulp, relative 2.4e-7) is below 1e-3 there, so the
// truncation is exact.  Cheaper than the integer division sequence.
__device__ __forceinline__ int small_div(int n, int d) {
  return (int)__fdividef((float)n + 0.5f, (float)d);
}

__device__ __forceinline__ float4 ws_in(const DTask& t, const int32_t* __restrict__ cmap,
                                        const float4* __restrict__ ws, int j) {
  return t.cbase >= 0 ? ws[t.cbase + j] : ws[cmap[j]];
}

// workspace entry of column j (input side of a forward task)
__device__ __forceinline__ long long col_entry(const DTask& t, const int32_t* __restrict__ cmap,
                                               int j) {
  return t.cbase >= 0 ? (long long)t.cbase + j : (long long)cmap[j];
}

// input entries of columns [c0, c0 + nb) for NR right-hand sides (stride S)
// into xw[j*NR + q]
template <int NR>
__device__ __forceinline__ void stage_cols(const DTask& t, const int32_t* __restrict__ cmap,
                                           const float4* __restrict__ ws, int S, int c0, int nb,
                                           float4* __restrict__ xw) {
  const int lane = threadIdx.x & 31;
  if constexpr (NR == 1) {
    if (S == 1)  // the single-vector path (S is the literal 1 there)
      for (int j = lane; j < nb; j += 32) xw[j] = ws_in(t, cmap, ws, c0 + j);
    else
      for (int j = lane; j < nb; j += 32) xw[j] = ws[col_entry(t, cmap, c0 + j) * S];
  } else {
    for (int e = lane; e < nb * NR; e += 32) {
      const int j = e / NR, q = e - j * NR;
      xw[e] = ws[col_entry(t, cmap, c0 + j) * S + q];
    }
  }
}

// In all three routines the first factor batch is issued before the input
// entries are staged (it does not depend on them), and a partial last batch is
// loaded at once under predicates, so a warp waits on few serial latencies.
// (Keeping two batches in flight instead was measured slower: the extra
// registers cost more occupancy than the overlap gained.)
template <typename FT, int NR = 1>
__device__ __forceinline__ void warp_tall(const DTask& t, int r0, const FT* __restrict__ A,
                                          const int32_t* __restrict__ maps,
                                          float4* __restrict__ ws, float4* __restrict__ xw,
                                          int S = 1) {
  const int lane = threadIdx.x & 31;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int M = t.M, n = t.n;
  if (r0 >= M) return;
  constexpr int XB = FW_XB / NR;  // staged columns per pass (xw holds XB * NR entries)
  float4 acc[TALL_RPL][NR];
#pragma unroll
  for (int q = 0; q < TALL_RPL; ++q)
#pragma unroll
    for (int v = 0; v < NR; ++v) acc[q][v] = make_float4(0.f, 0.f, 0.f, 0.f);
  bool act[TALL_RPL];
#pragma unroll
  for (int q = 0; q < TALL_RPL; ++q) act[q] = r0 + lane + 32 * q < M;
  // columns per batch: 128 bytes of factor loads per lane; with complex FP32
  // factors and several right-hand sides, 32 bytes (the NR accumulators need the
  // registers: 80 instead of 128 per thread, three CTAs per SM instead of two;
  // measured 1.16x on 262,144-point operators with 8 right-hand sides)
  constexpr int CPI = (sizeof(FT) == 8 ? (NR > 1 ? 4 : 16) : 8) / TALL_RPL;
  for (int cb = 0; cb < n; cb += XB) {
    const int nb = min(XB, n - cb);  // warp-uniform
    const FT* __restrict__ ap = A + t.a_off + (size_t)cb * M + r0 + lane;
    FT a[CPI][TALL_RPL];
    auto load = [&](FT(&v)[CPI][TALL_RPL], int j) {
#pragma unroll
      for (int c = 0; c < CPI; ++c)
#pragma unroll
        for (int q = 0; q < TALL_RPL; ++q)
          v[c][q] = (act[q] && j + c < nb) ? __ldg(ap + (size_t)(j + c) * M + 32 * q)
                                           : fac_zero<FT>();
    };
    auto mac = [&](const FT(&v)[CPI][TALL_RPL], int j) {
#pragma unroll
      for (int c = 0; c < CPI; ++c)
        if (j + c < nb) {
#pragma unroll
          for (int r = 0; r < NR; ++r) {
            const float4 xc = xw[(j + c) * NR + r];
#pragma unroll
            for (int q = 0; q < TALL_RPL; ++q) cdf_mac(acc[q][r], v[c][q], xc);
          }
        }
    };
    load(a, 0);
    stage_cols<NR>(t, cmap, ws, S, cb, nb, xw);
    __syncwarp();
    for (int j = 0; j < nb; j += CPI) {
      if (j > 0) load(a, j);
      mac(a, j);
    }
    __syncwarp();
  }
#pragma unroll
  for (int q = 0; q < TALL_RPL; ++q)
    if (act[q]) {
      const long long e = rmap[r0 + lane + 32 * q];
#pragma unroll
      for (int r = 0; r < NR; ++r) ws[e * S + r] = cdf_norm(acc[q][r]);
    }
  __syncwarp();
}

// warp_tall for the single-vector path (one right-hand side, S = 1): the
// column batches that are whole run without guards.  Same products in the
// same order, so the same bits as the guarded form.
template <typename FT>
__device__ __forceinline__ void warp_tall_one(const DTask& t, int r0, const FT* __restrict__ A,
                                              const int32_t* __restrict__ maps,
                                              float4* __restrict__ ws, float4* __restrict__ xw) {
  constexpr int NR = 1;
  const int S = 1;
  const int lane = threadIdx.x & 31;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int M = t.M, n = t.n;
  if (r0 >= M) return;
  constexpr int XB = FW_XB / NR;  // staged columns per pass (xw holds XB * NR entries)
  float4 acc[TALL_RPL][NR];
#pragma unroll
  for (int q = 0; q < TALL_RPL; ++q)
#pragma unroll
    for (int v = 0; v < NR; ++v) acc[q][v] = make_float4(0.f, 0.f, 0.f, 0.f);
  bool act[TALL_RPL];
#pragma unroll
  for (int q = 0; q < TALL_RPL; ++q) act[q] = r0 + lane + 32 * q < M;
  // columns per batch: 128 bytes of factor loads per lane
  constexpr int CPI = (sizeof(FT) == 8 ? 16 : 8) / TALL_RPL;
  for (int cb = 0; cb < n; cb += XB) {
    const int nb = min(XB, n - cb);  // warp-uniform
    const FT* __restrict__ ap = A + t.a_off + (size_t)cb * M + r0 + lane;
    FT a[CPI][TALL_RPL];
    auto load = [&](FT(&v)[CPI][TALL_RPL], int j) {
#pragma unroll
      for (int c = 0; c < CPI; ++c)
#pragma unroll
        for (int q = 0; q < TALL_RPL; ++q)
          v[c][q] = (act[q] && j + c < nb) ? __ldg(ap + (size_t)(j + c) * M + 32 * q)
                                           : fac_zero<FT>();
    };
    auto mac = [&](const FT(&v)[CPI][TALL_RPL], int j) {
#pragma unroll
      for (int c = 0; c < CPI; ++c)
        if (j + c < nb) {
#pragma unroll
          for (int r = 0; r < NR; ++r) {
            const float4 xc = xw[(j + c) * NR + r];
#pragma unroll
            for (int q = 0; q < TALL_RPL; ++q) cdf_mac(acc[q][r], v[c][q], xc);
          }
        }
    };
    // whole batches without column guards; a row past the task's end reads
    // row M - 1 instead (in bounds; its sum is never stored)
    int off[TALL_RPL];
#pragma unroll
    for (int q = 0; q < TALL_RPL; ++q) off[q] = act[q] ? 32 * q : M - 1 - r0 - lane;
    auto load_whole = [&](FT(&v)[CPI][TALL_RPL], int j) {
#pragma unroll
      for (int c = 0; c < CPI; ++c)
#pragma unroll
        for (int q = 0; q < TALL_RPL; ++q)
          v[c][q] = __ldg(ap + (long long)(j + c) * M + off[q]);
    };
    auto mac_whole = [&](const FT(&v)[CPI][TALL_RPL], int j) {
#pragma unroll
      for (int c = 0; c < CPI; ++c) {
        const float4 xc = xw[j + c];
#pragma unroll
        for (int q = 0; q < TALL_RPL; ++q) cdf_mac(acc[q][0], v[c][q], xc);
      }
    };
    const int jf = nb / CPI * CPI;  // columns in whole batches (warp-uniform)
    if (jf > 0)
      load_whole(a, 0);
    else
      load(a, 0);
    stage_cols<NR>(t, cmap, ws, S, cb, nb, xw);
    __syncwarp();
    for (int j = 0; j < jf; j += CPI) {
      if (j > 0) load_whole(a, j);
      mac_whole(a, j);
    }
    if (jf < nb) {  // the last, partial batch (nb - jf < CPI)
      if (jf > 0) load(a, jf);
      mac(a, jf);
    }
    __syncwarp();
  }
#pragma unroll
  for (int q = 0; q < TALL_RPL; ++q)
    if (act[q]) {
      const long long e = rmap[r0 + lane + 32 * q];
#pragma unroll
      for (int r = 0; r < NR; ++r) ws[e * S + r] = cdf_norm(acc[q][r]);
    }
  __syncwarp();
}

// One warp streams a whole task flat: lane l reads entry e = l + 32k of the
// column-major M x n matrix.  With M > 32 the 32 entries of one warp load
// belong to 32 distinct rows, so each lane adds its product into a per-row
// accumulator in warp-private shared memory without conflicts.
template <typename FT>
__device__ __forceinline__ void warp_flat(const DTask& t, const FT* __restrict__ A,
                                          const int32_t* __restrict__ maps,
                                          float4* __restrict__ ws, float4* __restrict__ xw,
                                          float4* __restrict__ aw) {
  const int lane = threadIdx.x & 31;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int M = t.M, n = t.n;
  const long long tot = (long long)M * n;
  const FT* __restrict__ ap = A + t.a_off + lane;
  constexpr int LU = sizeof(FT) == 8 ? 8 : 4;  // one warp step: 32*LU entries
  const long long nsteps = tot / (32 * LU);     // whole warp steps (warp-uniform)
  FT a[LU];
  auto load = [&](FT(&v)[LU], long long s) {
#pragma unroll
    for (int u = 0; u < LU; ++u) v[u] = __ldg(ap + s * (32 * LU) + 32 * u);
  };
  int row = lane, col = 0;  // entry lane: row lane of column 0 (M > 32)
  // lane a at step u+1 can hit the row that lane a-(M-32) updates at step u:
  // the warp barrier orders the two read-modify-writes
  auto mac = [&](const FT(&v)[LU]) {
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
  };
  if (nsteps > 0) load(a, 0);  // does not wait for the input staging
  for (int j = lane; j < n; j += 32) xw[j] = ws_in(t, cmap, ws, j);
  for (int i = lane; i < M; i += 32) aw[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  __syncwarp();
  for (long long s = 0; s < nsteps; ++s) {
    if (s > 0) load(a, s);
    mac(a);
  }
  // the last partial warp step (fewer than 32*LU entries), loaded at once
  const long long e0 = nsteps * (32 * LU);  // warp-uniform
#pragma unroll
  for (int u = 0; u < LU; ++u)
    a[u] = e0 + lane + 32 * u < tot ? __ldg(ap + e0 + 32 * u) : fac_zero<FT>();
#pragma unroll
  for (int u = 0; u < LU; ++u) {
    if (e0 + 32 * u >= tot) break;  // warp-uniform
    if (e0 + lane + 32 * u < tot) {
      float4 s = aw[row];
      cdf_mac(s, a[u], xw[col]);
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

// warp_small for one right-hand side (stride S): the column steps that every
// lane group has run in whole batches without guards, and the per-task
// quotients use the fast division.  Same products in the same order, so the
// same bits as the guarded form.
template <typename FT>
__device__ __forceinline__ void warp_small_one(const DTask& t, const FT* __restrict__ A,
                                           const int32_t* __restrict__ maps,
                                           float4* __restrict__ ws, float4* __restrict__ xw,
                                           int S = 1) {
  const int lane = threadIdx.x & 31;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int M = t.M, n = t.n;
  constexpr int NR = 1;
  const int G = small_div(32, M);
  int g = small_div(lane, M), i = lane - g * M;
  const bool active = g < G;
  // lanes past the last whole group mirror a row of group 0 (every other use
  // of g and i is under `active`): their loads stay inside the task and their
  // sums are never read, so whole batches need no guards
  if (!active) {
    g = 0;
    i = lane - G * M;
  }
  constexpr int XB = FW_XB / NR;  // staged columns per pass
  float4 acc[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) acc[r] = make_float4(0.f, 0.f, 0.f, 0.f);
  // lane group g reads columns g, g+G, g+2G, ...; a batch is LU of them (64
  // bytes per lane)
  constexpr int LU = sizeof(FT) == 8 ? 8 : 4;
  const size_t step = (size_t)G * M;
  for (int cb = 0; cb < n; cb += XB) {
    const int nb = min(XB, n - cb);  // warp-uniform
    const int nk = small_div(nb + G - 1, G);  // column steps of group 0 (warp-uniform)
    // steps that every group has, in whole batches (warp-uniform)
    const int kf = small_div(nb, G) / LU * LU;
    const FT* __restrict__ ap = A + t.a_off + (size_t)(cb + g) * M + i;
    FT a[LU];
    auto load = [&](FT(&v)[LU], int k) {
#pragma unroll
      for (int u = 0; u < LU; ++u)
        v[u] = (active && g + (k + u) * G < nb) ? __ldg(ap + (size_t)(k + u) * step)
                                                : fac_zero<FT>();
    };
    auto mac = [&](const FT(&v)[LU], int k) {
#pragma unroll
      for (int u = 0; u < LU; ++u) {
        const int j = g + (k + u) * G;
        if (active && j < nb) {
#pragma unroll
          for (int r = 0; r < NR; ++r) cdf_mac(acc[r], v[u], xw[j * NR + r]);
        }
      }
    };
    auto load_whole = [&](FT(&v)[LU], int k) {
#pragma unroll
      for (int u = 0; u < LU; ++u) v[u] = __ldg(ap + (size_t)(k + u) * step);
    };
    auto mac_whole = [&](const FT(&v)[LU], int k) {
#pragma unroll
      for (int u = 0; u < LU; ++u) {
        const int j = g + (k + u) * G;
#pragma unroll
        for (int r = 0; r < NR; ++r) cdf_mac(acc[r], v[u], xw[j * NR + r]);
      }
    };
    // the first factor batch does not wait for the input staging
    if (kf > 0)
      load_whole(a, 0);
    else
      load(a, 0);
    stage_cols<NR>(t, cmap, ws, S, cb, nb, xw);
    __syncwarp();
    for (int k = 0; k < kf; k += LU) {
      if (k > 0) load_whole(a, k);
      mac_whole(a, k);
    }
    if (kf < nk) {  // the last, partial batch (nk - kf <= LU)
      if (kf > 0) load(a, kf);
      mac(a, kf);
    }
    __syncwarp();
  }
  if (G > 1) {
    // reuse the staging buffer for the group reduction (32 * NR <= FW_XB entries)
#pragma unroll
    for (int r = 0; r < NR; ++r) xw[lane * NR + r] = acc[r];
    __syncwarp();
    if (active && g == 0) {
      for (int q = 1; q < G; ++q)
#pragma unroll
        for (int r = 0; r < NR; ++r) cdf_add(acc[r], xw[(q * M + i) * NR + r]);
      const long long e = rmap[i];
#pragma unroll
      for (int r = 0; r < NR; ++r) ws[e * S + r] = cdf_norm(acc[r]);
    }
  } else if (active) {
    const long long e = rmap[i];
#pragma unroll
    for (int r = 0; r < NR; ++r) ws[e * S + r] = cdf_norm(acc[r]);
  }
  __syncwarp();
}

// M <= 32: G = 32/M lane groups walk interleaved columns (one warp load reads
// G*M contiguous entries); the groups meet in shared memory at the end.
template <typename FT, int NR = 1>
__device__ __forceinline__ void warp_small(const DTask& t, const FT* __restrict__ A,
                                           const int32_t* __restrict__ maps,
                                           float4* __restrict__ ws, float4* __restrict__ xw,
                                           int S = 1) {
  const int lane = threadIdx.x & 31;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int M = t.M, n = t.n;
  const int G = 32 / M;
  const int g = lane / M, i = lane - g * M;
  const bool active = g < G;
  constexpr int XB = FW_XB / NR;  // staged columns per pass
  float4 acc[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) acc[r] = make_float4(0.f, 0.f, 0.f, 0.f);
  // lane group g reads columns g, g+G, g+2G, ...; a batch is LU of them (64
  // bytes per lane)
  constexpr int LU = sizeof(FT) == 8 ? 8 : 4;
  const size_t step = (size_t)G * M;
  for (int cb = 0; cb < n; cb += XB) {
    const int nb = min(XB, n - cb);  // warp-uniform
    const int nk = (nb + G - 1) / G;   // column steps of group 0 (warp-uniform)
    const FT* __restrict__ ap = A + t.a_off + (size_t)(cb + g) * M + i;
    FT a[LU];
    auto load = [&](FT(&v)[LU], int k) {
#pragma unroll
      for (int u = 0; u < LU; ++u)
        v[u] = (active && g + (k + u) * G < nb) ? __ldg(ap + (size_t)(k + u) * step)
                                                : fac_zero<FT>();
    };
    auto mac = [&](const FT(&v)[LU], int k) {
#pragma unroll
      for (int u = 0; u < LU; ++u) {
        const int j = g + (k + u) * G;
        if (active && j < nb) {
#pragma unroll
          for (int r = 0; r < NR; ++r) cdf_mac(acc[r], v[u], xw[j * NR + r]);
        }
      }
    };
    load(a, 0);  // the first factor batch does not wait for the input staging
    stage_cols<NR>(t, cmap, ws, S, cb, nb, xw);
    __syncwarp();
    for (int k = 0; k < nk; k += LU) {
      if (k > 0) load(a, k);
      mac(a, k);
    }
    __syncwarp();
  }
  if (G > 1) {
    // reuse the staging buffer for the group reduction (32 * NR <= FW_XB entries)
#pragma unroll
    for (int r = 0; r < NR; ++r) xw[lane * NR + r] = acc[r];
    __syncwarp();
    if (active && g == 0) {
      for (int q = 1; q < G; ++q)
#pragma unroll
        for (int r = 0; r < NR; ++r) cdf_add(acc[r], xw[(q * M + i) * NR + r]);
      const long long e = rmap[i];
#pragma unroll
      for (int r = 0; r < NR; ++r) ws[e * S + r] = cdf_norm(acc[r]);
    }
  } else if (active) {
    const long long e = rmap[i];
#pragma unroll
    for (int r = 0; r < NR; ++r) ws[e * S + r] = cdf_norm(acc[r]);
  }
  __syncwarp();
}

// identity blocks: copy the input slot to the output slot (reverse: the
// other way), NR right-hand sides at stride S
template <int NR = 1>
__device__ __forceinline__ void warp_copy(const DTask& t, const int32_t* __restrict__ maps,
                                          float4* __restrict__ ws, int reverse, int S = 1) {
  const int lane = threadIdx.x & 31;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  for (int e = lane; e < t.M * NR; e += 32) {
    const int i = e / NR, r = e - i * NR;
    const long long o = (long long)rmap[i] * S + r, c = (long long)cmap[i] * S + r;
    if (reverse)
      ws[c] = ws[o];
    else
      ws[o] = ws[c];
  }
}

}  // namespace bfg
