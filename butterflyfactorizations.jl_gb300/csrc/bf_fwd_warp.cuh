// Warp-level forward task routines of the FP64-accurate matvec (float-float
// vectors, factor entries FT = float4 float-float or float2 complex FP32).
//
// Each routine computes, for one dense task t (bf_internal.h DTask),
// ws[rows] = A_t * ws[cols] with the row / column slots addressed through the
// routing maps (or a contiguous base), reading every factor entry once with
// coalesced loads and staging the inputs in warp-private shared memory
// (xw: FW_XB entries, aw: FLAT_MMAX row accumulators).  They are shared by the
// per-shape level kernels (bf_matvec.cu) and by the persistent batch kernel
// that runs the levels of many operators at once (bf_batch.cu).
//   tall  : one 64-row panel of a task with M > 128, 2 rows per lane;
//   flat  : 32 < M <= 128, n <= 256, the warp streams all M*n entries;
//   small : M <= 32, G = 32/M lane groups on interleaved columns (also used
//           for short wide tasks by the batch kernel);
//   copy  : identity blocks.
#pragma once

#include "bf_dfloat.cuh"
#include "bf_internal.h"

namespace bfg {

constexpr int FW_WARPS = 8;
constexpr int FW_XB = 256;                // staged input entries per warp per pass
constexpr int TALL_RPL = TALL_ROWS / 32;  // rows per lane in a tall panel

__device__ __forceinline__ float4 ws_in(const DTask& t, const int32_t* __restrict__ cmap,
                                        const float4* __restrict__ ws, int j) {
  return t.cbase >= 0 ? ws[t.cbase + j] : ws[cmap[j]];
}

template <typename FT>
__device__ __forceinline__ void warp_tall(const DTask& t, int r0, const FT* __restrict__ A,
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
__device__ __forceinline__ void warp_flat(const DTask& t, const FT* __restrict__ A,
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
__device__ __forceinline__ void warp_small(const DTask& t, const FT* __restrict__ A,
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

// identity blocks: copy the input slot to the output slot (reverse: the other way)
__device__ __forceinline__ void warp_copy(const DTask& t, const int32_t* __restrict__ maps,
                                          float4* __restrict__ ws, int reverse) {
  const int lane = threadIdx.x & 31;
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  for (int i = lane; i < t.M; i += 32) {
    if (reverse)
      ws[cmap[i]] = ws[rmap[i]];
    else
      ws[rmap[i]] = ws[cmap[i]];
  }
}

}  // namespace bfg
