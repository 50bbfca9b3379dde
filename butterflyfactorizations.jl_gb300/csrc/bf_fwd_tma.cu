// Forward level launch as a warp-specialized persistent kernel.
//
// One producer warp streams the column-major task matrices of a level
// (packed back to back, see bf_pack.cpp) and the matching slices of the
// input vector into a ring of shared-memory slots with bulk asynchronous
// copies (cp.async.bulk = TMA without a tensor map; every task input is one
// contiguous workspace range because the x region is stored in leaf order and
// the level slots in reader order).  Eight consumer warps compute from shared
// memory in float-float arithmetic and write each output entry once.  The
// producer keeps up to NSLOT matrix slots in flight per CTA (4 x 16 KB of
// float-float entries, 6 x 8 KB of complex FP32 entries) regardless of task
// boundaries, so the DRAM stream does not stall on per-task set-up.
//
// Chunks: a task with M <= TMA_SLOT rows is cut into groups of whole columns
// (at most TMA_SLOT entries); a taller task into single-column segments of at
// most TMA_SLOT rows, panel by panel.  Consumer mappings by M:
//   S (M <= 32)        : G = 256/M thread groups on interleaved columns;
//   F (32 < M <= 256)  : each warp streams a contiguous run of entries, 32
//                        distinct rows per load, into a per-warp row
//                        accumulator in shared memory;
//   T (256 < M <= SLOT): thread per row, up to 4 rows per thread;
//   P (M > SLOT)       : like T within one row panel.
#include "bf_dfloat.cuh"
#include "bf_internal.h"
#include "bf_tma.cuh"

namespace bfg {
namespace {

constexpr int TMA_CW = 8;                     // consumer warps
constexpr int TMA_CT = TMA_CW * 32;           // consumer threads
constexpr int TMA_THREADS = TMA_CT + 32;      // + one producer warp
constexpr int TMA_SLOT = 1024;                // complex entries per matrix slot (16 KB)
constexpr int TMA_XSLOT = 256;                // input entries per slot (4 KB)
constexpr int TMA_FMAX = 256;                 // rows of the per-warp accumulators (mode F)

// Matrix slot geometry per factor type.  A bulk copy must start on a 16-byte
// boundary and move a multiple of 16 bytes: float4 entries always do; for
// complex FP32 (8-byte) entries a chunk that starts on an odd entry is copied
// from the entry before it, the slot holds that extra entry in front
// (`lead`), and the copy is rounded up to an even entry count (the packed
// factor array has two entries of tail padding for this).
template <typename FT>
struct TmaGeom {
  static constexpr int NSLOT = sizeof(FT) == 8 ? 6 : 4;  // slots in the ring
  static constexpr int SLOT_E = TMA_SLOT + (sizeof(FT) == 8 ? 2 : 0);
  static constexpr size_t SMEM = (size_t)NSLOT * SLOT_E * sizeof(FT) +
                                 (size_t)NSLOT * TMA_XSLOT * 16 +
                                 (size_t)TMA_CW * TMA_FMAX * 16 + 2 * NSLOT * 8;
};

struct Chunking {
  int M, n;
  bool panel;  // M > TMA_SLOT
  int cpc;     // columns per chunk (column mode)
  int np;      // row panels (panel mode)
  __device__ void init(int m, int nn) {
    M = m;
    n = nn;
    panel = M > TMA_SLOT;
    cpc = panel ? 1 : min(TMA_XSLOT, max(1, TMA_SLOT / max(M, 1)));
    np = panel ? (M + TMA_SLOT - 1) / TMA_SLOT : 1;
  }
  __device__ int count() const { return panel ? np * n : (n + cpc - 1) / cpc; }
  // chunk k: columns [c0, c0 + cc), rows [r0, r0 + rr)
  __device__ void get(int k, int& c0, int& cc, int& r0, int& rr) const {
    if (panel) {
      int p = k / n;
      c0 = k - p * n;
      cc = 1;
      r0 = p * TMA_SLOT;
      rr = min(TMA_SLOT, M - r0);
    } else {
      c0 = k * cpc;
      cc = min(cpc, n - c0);
      r0 = 0;
      rr = M;
    }
  }
};

template <typename FT>
__global__ void __launch_bounds__(TMA_THREADS) fwd_tma_kernel(
    const int32_t* __restrict__ tlist, int n_tasks, const DTask* __restrict__ tasks,
    const FT* __restrict__ A, const int32_t* __restrict__ maps, float4* __restrict__ ws,
    int* __restrict__ err, long long wait_limit) {
  constexpr int SLOT_E = TmaGeom<FT>::SLOT_E;
  constexpr int NSLOT = TmaGeom<FT>::NSLOT;
  extern __shared__ __align__(128) unsigned char smem[];
  FT* sA = (FT*)smem;                                          // [NSLOT][SLOT_E]
  float4* sX = (float4*)(sA + NSLOT * SLOT_E);             // [NSLOT][XSLOT]
  float4* sAcc = sX + NSLOT * TMA_XSLOT;                   // [CW][FMAX]
  uint64_t* bars = (uint64_t*)(sAcc + TMA_CW * TMA_FMAX);      // full[NSLOT], empty[NSLOT]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + NSLOT);
  if (threadIdx.x == 0) {
    for (int s = 0; s < NSLOT; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, TMA_CW);
    }
    mbar_fence_init();
  }
  __syncthreads();

  if (warp == TMA_CW) {
    // ---------------- producer ----------------
    if (lane != 0) return;
    int slot = 0;
    uint32_t ph = 0;
    int issued[NSLOT];
    for (int s = 0; s < NSLOT; ++s) issued[s] = -1;
    bool ok = true;
    for (int ti = blockIdx.x; ti < n_tasks && ok; ti += gridDim.x) {
      const DTask t = tasks[tlist[ti]];
      Chunking ch;
      ch.init(t.M, t.n);
      const int nc = ch.count();
      for (int k = 0; k < nc; ++k) {
        if (!mbar_wait(empty0 + 8 * slot, ph ^ 1u, err, wait_limit)) {
          ok = false;
          break;
        }
        int c0, cc, r0, rr;
        ch.get(k, c0, cc, r0, rr);
        const size_t e0 = (size_t)t.a_off + (size_t)c0 * t.M + r0;
        const int lead = sizeof(FT) == 8 ? (int)(e0 & 1) : 0;
        int ne = cc * rr + lead;
        if (sizeof(FT) == 8) ne = (ne + 1) & ~1;
        const uint32_t abytes = (uint32_t)ne * (uint32_t)sizeof(FT), xbytes = (uint32_t)cc * 16u;
        const uint32_t fb = full0 + 8 * slot;
        fence_proxy_async();
        mbar_arrive_expect_tx(fb, abytes + xbytes);
        bulk_g2s(smem_u32(sA + slot * SLOT_E), A + (e0 - lead), abytes, fb);
        bulk_g2s(smem_u32(sX + slot * TMA_XSLOT), ws + t.cbase + c0, xbytes, fb);
        issued[slot] = (int)ph;
        if (++slot == NSLOT) {
          slot = 0;
          ph ^= 1u;
        }
      }
    }
    // no copy may still be in flight when the block exits
    for (int s = 0; s < NSLOT; ++s)
      if (issued[s] >= 0) mbar_wait_drain(full0 + 8 * s, (uint32_t)issued[s], err);
    return;
  }

  // ---------------- consumers ----------------
  const int tid = threadIdx.x;  // < TMA_CT
  float4* accw = sAcc + warp * TMA_FMAX;
  int slot = 0;
  uint32_t ph = 0;
  // after a failed wait a warp keeps walking the same task/chunk sequence
  // (and the same named barriers) without touching data, so no warp can be
  // left waiting at a barrier
  bool dead = false;
  for (int i = lane; i < TMA_FMAX; i += 32) accw[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  __syncwarp();
  for (int ti = blockIdx.x; ti < n_tasks; ti += gridDim.x) {
    const DTask t = tasks[tlist[ti]];
    const int32_t* __restrict__ rmap = maps + t.rmap_off;
    const int M = t.M, n = t.n;
    Chunking ch;
    ch.init(M, n);
    const int nc = ch.count();
    const int mode = M <= 32 ? 0 : (M <= TMA_FMAX ? 1 : 2);  // S, F, T/P
    const int G = mode == 0 ? TMA_CT / M : 1;
    const int g = mode == 0 ? tid / M : 0;
    const int gi = mode == 0 ? tid - g * M : 0;
    float4 acc[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = 0; k < nc; ++k) {
      bool got = dead ? false : mbar_wait(full0 + 8 * slot, ph, err, wait_limit);
      dead = __any_sync(0xffffffffu, !got);
      int c0, cc, r0, rr;
      ch.get(k, c0, cc, r0, rr);
      const int lead =
          sizeof(FT) == 8 ? (int)(((size_t)t.a_off + (size_t)c0 * M + r0) & 1) : 0;
      const FT* __restrict__ a = sA + slot * SLOT_E + lead;
      const float4* __restrict__ xv = sX + slot * TMA_XSLOT;
      if (dead) {
        // skip the data; still release the slot below
      } else if (mode == 0) {
        if (g < G)
          for (int c = g; c < cc; c += G) cdf_mac(acc[0], a[c * M + gi], xv[c]);
      } else if (mode == 1) {
        const int E = cc * M;
        const int per = (E + TMA_CW - 1) / TMA_CW;
        const int e0 = warp * per, e1 = min(E, e0 + per);
        int e = e0 + lane;
        int col = e / M, row = e - col * M;
        // warp-uniform trip count; the warp barrier orders read-modify-writes
        // of one row by different lanes in consecutive steps
        for (; e - lane < e1; e += 32) {
          if (e < e1) {
            float4 s = accw[row];
            cdf_mac(s, a[e], xv[col]);
            accw[row] = s;
          }
          __syncwarp();
          row += 32;
          if (row >= M) {
            row -= M;
            ++col;
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = tid + q * TMA_CT;
          if (i < rr)
            for (int c = 0; c < cc; ++c) cdf_mac(acc[q], a[c * rr + i], xv[c]);
        }
        if (ch.panel && c0 == n - 1) {  // end of a row panel: flush its rows
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int i = tid + q * TMA_CT;
            if (i < rr) ws[rmap[r0 + i]] = cdf_norm(acc[q]);
            acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(empty0 + 8 * slot);
      if (++slot == NSLOT) {
        slot = 0;
        ph ^= 1u;
      }
    }
    // ---- task epilogue: reduce partial sums and write each output once
    if (mode == 0) {
      named_sync(TMA_CT);
      float4* red = sAcc;  // reuse the accumulator area (G*M <= 256 entries)
      if (g < G) red[tid] = acc[0];
      named_sync(TMA_CT);
      if (tid < M) {
        float4 v = red[tid];
        for (int q = 1; q < G; ++q) cdf_add(v, red[q * M + tid]);
        ws[rmap[tid]] = cdf_norm(v);
      }
      named_sync(TMA_CT);
      for (int i = lane; i < TMA_FMAX; i += 32) accw[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      named_sync(TMA_CT);
    } else if (mode == 1) {
      named_sync(TMA_CT);
      if (tid < M) {
        float4 v = sAcc[tid];
        for (int w = 1; w < TMA_CW; ++w) cdf_add(v, sAcc[w * TMA_FMAX + tid]);
        ws[rmap[tid]] = cdf_norm(v);
      }
      named_sync(TMA_CT);
      for (int i = lane; i < M; i += 32) accw[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      __syncwarp();
    } else if (!ch.panel) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = tid + q * TMA_CT;
        if (i < M) ws[rmap[i]] = cdf_norm(acc[q]);
      }
    } else if (n == 0) {
      for (int i = tid; i < M; i += TMA_CT) ws[rmap[i]] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

}  // namespace

template <typename FT>
static int launch_fwd_tma_t(const int32_t* d_tlist, int n_tasks, const DTask* d_tasks,
                            const FT* d_A, const int32_t* d_maps, float4* d_ws, int* d_err,
                            long long wait_limit, int n_sm, cudaStream_t st) {
  constexpr size_t smem = TmaGeom<FT>::SMEM;
  static DeviceOnce attr;
  BF_TRY(attr.run([] {
    return cudaFuncSetAttribute(fwd_tma_kernel<FT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
  }, "fwd_tma_kernel shared memory"));
  if (wait_limit < 0) wait_limit = BF_SPIN_LIMIT;
  int grid = std::min(n_tasks, 2 * n_sm);
  fwd_tma_kernel<FT><<<grid, TMA_THREADS, smem, st>>>(d_tlist, n_tasks, d_tasks, d_A, d_maps,
                                                        d_ws, d_err, wait_limit);
  BF_TRY_CUDA(cudaGetLastError());
  return BF_OK;
}

int launch_fwd_tma(const int32_t* d_tlist, int n_tasks, const DTask* d_tasks, const float4* d_A,
                   const float2* d_A2, const int32_t* d_maps, float4* d_ws, int* d_err,
                   long long wait_limit, int n_sm, cudaStream_t st) {
  if (n_tasks <= 0) return BF_OK;
  if (d_A2)
    return launch_fwd_tma_t<float2>(d_tlist, n_tasks, d_tasks, d_A2, d_maps, d_ws, d_err,
                                    wait_limit, n_sm, st);
  return launch_fwd_tma_t<float4>(d_tlist, n_tasks, d_tasks, d_A, d_maps, d_ws, d_err, wait_limit,
                                  n_sm, st);
}

}  // namespace bfg
