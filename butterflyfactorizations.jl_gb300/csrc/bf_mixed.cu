// Many-right-hand-side matvec on the tensor cores (bf_matvec_mixed).
//
// The level structure is the one of the FP64 path (same tasks, slots and
// routing maps); what changes is the arithmetic and the data layout:
//
//   * right-hand sides are processed in chunks of MX_R = 128.  The workspace
//     holds complex FP32 values, entry-major: slot e of the level sequence is
//     the 1 KB row ws[e * 128 + j], j = right-hand side;
//   * every dense task matrix A (M x n complex) is stored once as the real
//     2M x 2n matrix  Ahat[(m,p),(c,q)]  with  Ahat = [[Ar, -Ai], [Ai, Ar]]  on
//     each complex entry (rows and columns interleave real and imaginary
//     parts), rounded to complex FP32 and split into BF16 hi + lo planes, cut
//     into 8 x 8 complex blocks (16 x 16 reals, 512 B per plane).  The blocks
//     of one column-block are stored top to bottom, all hi planes first, then
//     all lo planes, so that a run of blocks in one column is one contiguous
//     copy and forms a uniform K-major operand tile;
//   * a level is one persistent kernel over work units (task, run of output
//     blocks).  Per unit, tcgen05.mma computes D(128 x 2*outputs) =
//     X(128 x 2*inputs) * Ahat^T in FP32 in tensor memory, X being the
//     unit's input slots for the 128 right-hand sides, split into BF16 hi/lo
//     while staged into shared memory.  Three passes (hi*hi + lo*hi + hi*lo)
//     give about 16 significant bits per operand.  The adjoint reads the same
//     stored blocks as MN-major B operands (Ahat^T is the real form of A^H);
//     the transpose conjugates inputs and outputs on top of that.
//
// Pipeline per CTA (4 warps, 8 CTAs per SM, 64 tensor-memory columns each):
// two stages of shared memory, each one input chunk (8 entries x 128
// right-hand sides, hi and lo) plus the matching factor blocks.  Thread 0
// issues the bulk copies of the factor blocks and the MMAs; all 128 threads
// gather and split the inputs and run the epilogue (thread j owns right-hand
// side j = tensor-memory lane j).  The MMAs of one chunk overlap the gathering
// of the next; the gathers run one chunk and one unit ahead (gathering two
// chunks ahead was measured slower).  Every wait is bounded.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>

#include "bf_dfloat.cuh"
#include "bf_internal.h"
#include "bf_umma.cuh"

namespace bfg {

constexpr int MX_R = 128;                         // right-hand sides per chunk (MMA M)
constexpr int MX_THREADS = 128;
constexpr int MX_IB = 1;                          // input blocks (of 8 entries) per stage
constexpr int MX_IC = MX_IB * 8;                  // input entries per stage
constexpr int MX_OB = 4;                          // output blocks per unit (N <= 64)
constexpr int MX_TCOLS = 64;                      // tensor-memory columns per CTA
constexpr int MX_CTAS_PER_SM = 8;                 // 8 x 24 KB shared memory, 8 x 64 TMEM columns,
                                                  // 8 x 128 threads x 64 registers
constexpr int MX_XPLANE = (MX_IC / 4) * 2048;     // one BF16 plane of the input tile (8 KB)
constexpr int MX_XBYTES = 2 * MX_XPLANE;          // hi + lo
constexpr int MX_FBYTES = MX_OB * MX_IB * 1024;   // factor blocks of one stage (4 KB)
constexpr int MX_STAGE = MX_XBYTES + MX_FBYTES;
constexpr int MX_NST = 2;
constexpr size_t MX_SMEM = (size_t)MX_NST * MX_STAGE + 256;

struct MixedState {
  uint8_t* d_F = nullptr;       // packed BF16 hi/lo blocks
  int64_t F_bytes = 0;
  int64_t* d_moff = nullptr;    // per task: byte offset of its blocks (-1: no blocks)
  int4* d_units = nullptr;      // forward units then adjoint units
  std::vector<int64_t> ufwd, uadj;  // per stage: unit ranges (n_stages + 1 each)
  int* d_counters = nullptr;    // work-queue counters, one per stage
  float2* d_ws = nullptr;       // ws_entries x MX_R complex FP32
  double* d_x = nullptr;        // staging of host right-hand sides
  double* d_y = nullptr;
  int64_t stage_cap = 0;
  std::vector<int64_t> stage_fbytes;  // factor bytes read per level
  std::vector<int64_t> stage_io;      // input + output slots per level
  std::vector<int64_t> stage_mn;      // sum of M*n (useful complex MACs per RHS)
  std::vector<int64_t> stage_mnp;     // sum of padded Mp*np
  int64_t units_total = 0;
  ~MixedState() {
    if (d_F) cudaFree(d_F);
    if (d_moff) cudaFree(d_moff);
    if (d_units) cudaFree(d_units);
    if (d_counters) cudaFree(d_counters);
    if (d_ws) cudaFree(d_ws);
    if (d_x) cudaFree(d_x);
    if (d_y) cudaFree(d_y);
  }
};

void mixed_free(void* p) { delete static_cast<MixedState*>(p); }

namespace {

// ---------------------------------------------------------------- packing
// One CTA per (task, column block): float-float entries -> complex FP32 ->
// real 2x2 form -> BF16 hi/lo, written into the core-matrix layout.
template <typename FT>
__global__ void mx_pack_kernel(const int2* __restrict__ items, const DTask* __restrict__ tasks,
                               const int64_t* __restrict__ moff, const FT* __restrict__ A,
                               uint8_t* __restrict__ F) {
  const int2 it = items[blockIdx.x];
  const DTask t = tasks[it.x];
  const int bj = it.y;
  const int Mb = (t.M + 7) / 8;
  uint8_t* seg = F + moff[it.x] + (size_t)bj * Mb * 1024;
  for (int idx = threadIdx.x; idx < Mb * 64; idx += blockDim.x) {
    const int bi = idx >> 6, r = (idx >> 3) & 7, c = idx & 7;
    const int m = bi * 8 + r, col = bj * 8 + c;
    float ar = 0.f, ai = 0.f;
    if (m < t.M && col < t.n) {
      const float2 a = fac_c32(A[t.a_off + (size_t)col * t.M + m]);
      ar = a.x;
      ai = a.y;
    }
    const float v[2][2] = {{ar, -ai}, {ai, ar}};
    uint8_t* hi = seg + (size_t)bi * 512;
    uint8_t* lo = seg + (size_t)Mb * 512 + (size_t)bi * 512;
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int R = 2 * r + p, C = 2 * c + q;
        const int off = ((R >> 3) * 2 + (C >> 3)) * 128 + (R & 7) * 16 + (C & 7) * 2;
        const __nv_bfloat16 h = __float2bfloat16_rn(v[p][q]);
        const __nv_bfloat16 l = __float2bfloat16_rn(v[p][q] - __bfloat162float(h));
        *(__nv_bfloat16*)(hi + off) = h;
        *(__nv_bfloat16*)(lo + off) = l;
      }
  }
}

// ---------------------------------------------------------------- x / y regions
// x (complex double, column-major, ldx) -> ws rows [off, off + n) in leaf order,
// right-hand sides [0, nr) of the chunk; the rest of each row is zeroed.
// A 32-entry x 128-RHS tile goes through shared memory so that both the reads
// (down the columns of x) and the writes (along the ws rows) are coalesced.
__global__ void __launch_bounds__(256) mx_split_kernel(const double2* __restrict__ x,
                                                       int64_t ldx, int64_t n, int nr,
                                                       float2* __restrict__ ws, int64_t off,
                                                       const int32_t* __restrict__ perm,
                                                       int conj) {
  __shared__ float2 tile[32][MX_R + 1];
  const int64_t q0 = (int64_t)blockIdx.x * 32;
  const int tq = threadIdx.x & 31, tj = threadIdx.x >> 5;  // 8 column groups
  const int64_t q = q0 + tq;
  const int64_t src = q < n ? (perm ? perm[q] : q) : -1;
  for (int j = tj; j < MX_R; j += 8) {
    float2 v = make_float2(0.f, 0.f);
    if (src >= 0 && j < nr) {
      const double2 d = x[(size_t)j * ldx + src];
      v = make_float2((float)d.x, conj ? -(float)d.y : (float)d.y);
    }
    tile[tq][j] = v;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * MX_R; e += 256) {
    const int qq = e / MX_R, j = e % MX_R;
    if (q0 + qq < n) ws[(size_t)(off + q0 + qq) * MX_R + j] = tile[qq][j];
  }
}

// y = beta*y + alpha*ws (conjugated first when conj), same tiling as the split
__global__ void __launch_bounds__(256) mx_combine_kernel(double2* __restrict__ y, int64_t ldy,
                                                         int64_t n, int nr,
                                                         const float2* __restrict__ ws,
                                                         int64_t off,
                                                         const int32_t* __restrict__ perm,
                                                         double2 alpha, double2 beta,
                                                         int beta_zero, int conj) {
  __shared__ float2 tile[32][MX_R + 1];
  const int64_t q0 = (int64_t)blockIdx.x * 32;
  for (int e = threadIdx.x; e < 32 * MX_R; e += 256) {
    const int qq = e / MX_R, j = e % MX_R;
    tile[qq][j] = q0 + qq < n ? ws[(size_t)(off + q0 + qq) * MX_R + j] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int tq = threadIdx.x & 31, tj = threadIdx.x >> 5;
  const int64_t q = q0 + tq;
  if (q >= n) return;
  const int64_t dst = perm ? perm[q] : q;
  for (int j = tj; j < nr; j += 8) {
    const float2 a = tile[tq][j];
    const double vr = a.x, vi = conj ? -(double)a.y : (double)a.y;
    double2 o;
    o.x = alpha.x * vr - alpha.y * vi;
    o.y = alpha.x * vi + alpha.y * vr;
    double2* yp = y + (size_t)j * ldy + dst;
    if (!beta_zero) {
      const double2 yo = *yp;
      o.x += beta.x * yo.x - beta.y * yo.y;
      o.y += beta.x * yo.y + beta.y * yo.x;
    }
    *yp = o;
  }
}

// identity blocks: whole 1 KB rows (forward: rows <- columns; reverse: the other
// way).  An identity block is real, so the transpose needs no conjugation here.
__global__ void __launch_bounds__(MX_R) mx_copy_kernel(const int32_t* __restrict__ tlist,
                                                       const DTask* __restrict__ tasks,
                                                       const int32_t* __restrict__ maps,
                                                       float2* __restrict__ ws, int reverse) {
  const DTask t = tasks[tlist[blockIdx.x]];
  const int32_t* __restrict__ rmap = maps + t.rmap_off;
  const int32_t* __restrict__ cmap = maps + t.cmap_off;
  const int j = threadIdx.x;
  for (int i = 0; i < t.M; ++i) {
    const int64_t src = reverse ? rmap[i] : cmap[i];
    const int64_t dst = reverse ? cmap[i] : rmap[i];
    ws[(size_t)dst * MX_R + j] = ws[(size_t)src * MX_R + j];
  }
}

// ---------------------------------------------------------------- level kernel
__device__ __forceinline__ uint32_t pack_bf2(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// One work unit (a task and a group of output blocks), ADJ = 0: out = rows
// (M), in = columns (n); ADJ = 1: the other way round.
struct MxUnit {
  int64_t fo;  // first byte of the task's BF16 blocks
  const int32_t* in_map;
  const int32_t* out_map;
  int Mb, nb, nin, nout, in_base, out_base, o0, no, nib_total, nchunks;
};

template <int ADJ>
__device__ __forceinline__ MxUnit mx_unit(int u, const int4* __restrict__ units,
                                          const DTask* __restrict__ tasks,
                                          const int64_t* __restrict__ moff,
                                          const int32_t* __restrict__ maps) {
  const int4 un = units[u];
  const DTask t = tasks[un.x];
  MxUnit d;
  d.fo = moff[un.x];
  d.Mb = (t.M + 7) >> 3;
  d.nb = (t.n + 7) >> 3;
  d.nin = ADJ ? t.M : t.n;
  d.nout = ADJ ? t.n : t.M;
  d.in_base = ADJ ? t.rbase : t.cbase;
  d.in_map = maps + (ADJ ? t.rmap_off : t.cmap_off);
  d.out_base = ADJ ? t.cbase : t.rbase;
  d.out_map = maps + (ADJ ? t.cmap_off : t.rmap_off);
  d.o0 = un.y;
  d.no = un.z;
  d.nib_total = ADJ ? d.Mb : d.nb;
  d.nchunks = (d.nib_total + MX_IB - 1) / MX_IB;
  return d;
}

// the input entries of one chunk for right-hand side j
__device__ __forceinline__ void mx_gather(const MxUnit& d, const float2* __restrict__ ws,
                                          float2 (&v)[MX_IC], int chunk, int j) {
  const int kb = chunk * MX_IB, knb = min(MX_IB, d.nib_total - kb);
#pragma unroll
  for (int c = 0; c < MX_IC; ++c) {
    const int e = kb * 8 + c;
    v[c] = make_float2(0.f, 0.f);
    if (c < knb * 8 && e < d.nin) {
      const int64_t slot = d.in_base >= 0 ? (int64_t)d.in_base + e : (int64_t)d.in_map[e];
      v[c] = ws[(size_t)slot * MX_R + j];
    }
  }
}

template <int ADJ>
__global__ void __launch_bounds__(MX_THREADS) mx_level_kernel(
    const int4* __restrict__ units, int n_units, int* __restrict__ counter,
    const DTask* __restrict__ tasks, const int64_t* __restrict__ moff,
    const uint8_t* __restrict__ F, const int32_t* __restrict__ maps, float2* __restrict__ ws,
    int conj, int* err) {
  extern __shared__ __align__(128) uint8_t smem[];
  uint64_t* bars = (uint64_t*)(smem + MX_NST * MX_STAGE);  // fbar[2], mbar[2]
  uint32_t* tslot = (uint32_t*)(bars + 4);
  volatile int* s_unit = (volatile int*)(tslot + 1);  // two slots
  volatile int* s_dead = s_unit + 2;
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t sbase = smem_u32(smem);
  const uint32_t fbar0 = smem_u32(bars), mbar0 = smem_u32(bars + 2);

  if (tid == 0) {
    mbar_init(fbar0, 1);
    mbar_init(fbar0 + 8, 1);
    mbar_init(mbar0, 1);
    mbar_init(mbar0 + 8, 1);
    mbar_fence_init();
    *s_dead = 0;
  }
  if (warp == 0) tmem_alloc(smem_u32(tslot), MX_TCOLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  // per-stage bookkeeping of thread 0 for the final drain
  int last_copy_use[MX_NST] = {-1, -1}, last_commit_use[MX_NST] = {-1, -1};
  int it = 0;  // global chunk counter of this CTA

  // Thread j = right-hand side j gathers the input entries of a chunk.  The
  // next chunk's entries are requested before the current chunk is split and
  // multiplied, and the next unit (claimed when the current one starts) has
  // its descriptor and first chunk requested before the current unit's
  // epilogue waits for its MMAs.  The unit index alternates between two
  // shared slots, so a claim never overwrites an index not yet read.
  if (tid == 0) s_unit[0] = atomicAdd(counter, 1);
  __syncthreads();
  int u = s_unit[0], uslot = 0;
  MxUnit cur{};
  float2 vnext[MX_IC];
  if (u < n_units) {
    cur = mx_unit<ADJ>(u, units, tasks, moff, maps);
    if (cur.nchunks > 0) mx_gather(cur, ws, vnext, 0, tid);
  }
  for (;;) {
    if (u >= n_units || *s_dead) break;
    if (tid == 0) s_unit[uslot ^ 1] = atomicAdd(counter, 1);
    const int64_t fo = cur.fo;
    const int Mb = cur.Mb, nout = cur.nout, out_base = cur.out_base;
    const int32_t* __restrict__ out_map = cur.out_map;
    const int o0 = cur.o0, no = cur.no, nib_total = cur.nib_total, nchunks = cur.nchunks;

    for (int ch = 0; ch < nchunks; ++ch, ++it) {
      const int st = it & 1, use = it >> 1;
      const uint32_t xs = sbase + st * MX_STAGE, fs = xs + MX_XBYTES;
      const int k0 = ch * MX_IB, kn = min(MX_IB, nib_total - k0);
      // stage buffers are free once the MMAs that read them two chunks ago are done
      if (use > 0 && !mbar_wait(mbar0 + 8 * st, (use - 1) & 1, err)) *s_dead = 1;
      if (tid == 0 && !*s_dead) {
        const uint32_t bytes = (uint32_t)(no * kn * 1024);
        mbar_arrive_expect_tx(fbar0 + 8 * st, bytes);
        if (!ADJ) {
          // column blocks bj = k0..k0+kn-1, row blocks o0..o0+no-1
          for (int b = 0; b < kn; ++b) {
            const uint8_t* seg = F + fo + (size_t)(k0 + b) * Mb * 1024;
            const uint32_t d = fs + b * no * 1024;
            bulk_g2s(d, seg + (size_t)o0 * 512, no * 512, fbar0 + 8 * st);
            bulk_g2s(d + no * 512, seg + (size_t)Mb * 512 + (size_t)o0 * 512, no * 512,
                     fbar0 + 8 * st);
          }
        } else {
          // column blocks bj = o0..o0+no-1 (outputs), row blocks k0..k0+kn-1 (inputs)
          for (int b = 0; b < no; ++b) {
            const uint8_t* seg = F + fo + (size_t)(o0 + b) * Mb * 1024;
            const uint32_t d = fs + b * kn * 1024;
            bulk_g2s(d, seg + (size_t)k0 * 512, kn * 512, fbar0 + 8 * st);
            bulk_g2s(d + kn * 512, seg + (size_t)Mb * 512 + (size_t)k0 * 512, kn * 512,
                     fbar0 + 8 * st);
          }
        }
        last_copy_use[st] = use;
      }
      // split the gathered inputs into BF16 hi/lo planes: thread j = right-hand side j
      {
        const int j = tid;
        float2 v[MX_IC];
#pragma unroll
        for (int c = 0; c < MX_IC; ++c) v[c] = vnext[c];
        if (ch + 1 < nchunks) mx_gather(cur, ws, vnext, ch + 1, tid);
        uint8_t* xg = smem + st * MX_STAGE + (j >> 3) * 128 + (j & 7) * 16;
#pragma unroll
        for (int g = 0; g < MX_IC / 4; ++g) {
          if (g * 4 < kn * 8) {
            uint32_t h[4], l[4];
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4) {
              const float re = v[4 * g + c4].x;
              const float im = conj ? -v[4 * g + c4].y : v[4 * g + c4].y;
              const __nv_bfloat16 hr = __float2bfloat16_rn(re), hi_ = __float2bfloat16_rn(im);
              const __nv_bfloat16 lr = __float2bfloat16_rn(re - __bfloat162float(hr));
              const __nv_bfloat16 li = __float2bfloat16_rn(im - __bfloat162float(hi_));
              h[c4] = pack_bf2(hr, hi_);
              l[c4] = pack_bf2(lr, li);
            }
            *(uint4*)(xg + g * 2048) = make_uint4(h[0], h[1], h[2], h[3]);
            *(uint4*)(xg + MX_XPLANE + g * 2048) = make_uint4(l[0], l[1], l[2], l[3]);
          }
        }
      }
      fence_proxy_async();
      __syncthreads();
      if (*s_dead) break;
      if (tid == 0) {
        if (!mbar_wait(fbar0 + 8 * st, use & 1, err)) {
          *s_dead = 1;
        } else {
          tc_fence_after();
          const uint32_t xhi = xs, xlo = xs + MX_XPLANE;
          if (!ADJ) {
            const uint32_t idesc = umma_idesc_bf16(MX_R, 16 * no, 0);
            for (int b = 0; b < kn; ++b) {
              const uint64_t ah = umma_sdesc(xhi + b * 4096, 2048, 128);
              const uint64_t al = umma_sdesc(xlo + b * 4096, 2048, 128);
              const uint32_t fb = fs + b * no * 1024;
              const uint64_t bh = umma_sdesc(fb, 128, 256);
              const uint64_t bl = umma_sdesc(fb + no * 512, 128, 256);
              const uint32_t acc0 = (ch > 0 || b > 0) ? 1u : 0u;
              umma_bf16(tmem, ah, bh, idesc, acc0);
              umma_bf16(tmem, al, bh, idesc, 1u);
              umma_bf16(tmem, ah, bl, idesc, 1u);
            }
          } else {
            const uint32_t idesc = umma_idesc_bf16(MX_R, 16, 1);
            for (int ob = 0; ob < no; ++ob) {
              const uint32_t fb = fs + ob * kn * 1024;
              for (int b = 0; b < kn; ++b) {
                const uint64_t ah = umma_sdesc(xhi + b * 4096, 2048, 128);
                const uint64_t al = umma_sdesc(xlo + b * 4096, 2048, 128);
                const uint64_t bh = umma_sdesc(fb + b * 512, 256, 128);
                const uint64_t bl = umma_sdesc(fb + kn * 512 + b * 512, 256, 128);
                const uint32_t acc0 = (ch > 0 || b > 0) ? 1u : 0u;
                const uint32_t d = tmem + ob * 16;
                umma_bf16(d, ah, bh, idesc, acc0);
                umma_bf16(d, al, bh, idesc, 1u);
                umma_bf16(d, ah, bl, idesc, 1u);
              }
            }
          }
          umma_commit(mbar0 + 8 * st);
          last_commit_use[st] = use;
        }
      }
    }
    __syncthreads();
    if (*s_dead) break;
    // the next unit's descriptor and first chunk are requested before the wait
    // below (inputs and outputs of a level are disjoint slots)
    const int u_next = s_unit[uslot ^ 1];
    MxUnit nxt{};
    if (u_next < n_units) {
      nxt = mx_unit<ADJ>(u_next, units, tasks, moff, maps);
      if (nxt.nchunks > 0) mx_gather(nxt, ws, vnext, 0, tid);
    }
    // epilogue: every MMA of the unit is done once the last commit has landed.
    // A unit without input entries (a task whose input slots are all empty)
    // issued no MMA: its outputs are zero, as in the FP64 path.
    if (nchunks > 0) {
      const int last = it - 1;
      if (!mbar_wait(mbar0 + 8 * (last & 1), (last >> 1) & 1, err)) *s_dead = 1;
    }
    if (!*s_dead) {
      tc_fence_after();
      const int j = tid;
      const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
      for (int ob = 0; ob < no; ++ob) {
        float d[16];
        if (nchunks > 0) {
          tmem_ld16(lane_addr + ob * 16, d);
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i) d[i] = 0.f;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int m = (o0 + ob) * 8 + i;
          if (m < nout) {
            const int64_t slot = out_base >= 0 ? (int64_t)out_base + m : (int64_t)out_map[m];
            ws[(size_t)slot * MX_R + j] = make_float2(d[2 * i], conj ? -d[2 * i + 1] : d[2 * i + 1]);
          }
        }
      }
    }
    tc_fence_before();
    __syncthreads();
    if (*s_dead) break;
    cur = nxt;
    u = u_next;
    uslot ^= 1;
  }

  // drain: let this CTA's own copies and MMAs finish before freeing tensor memory
  __syncthreads();
  if (tid == 0) {
    for (int s = 0; s < MX_NST; ++s) {
      if (last_copy_use[s] >= 0) mbar_wait_drain(fbar0 + 8 * s, last_copy_use[s] & 1, err);
      if (last_commit_use[s] >= 0) mbar_wait_drain(mbar0 + 8 * s, last_commit_use[s] & 1, err);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, MX_TCOLS);
}

inline unsigned grid_rows(int64_t n, int per) { return (unsigned)((n + per - 1) / per); }

}  // namespace

// ---------------------------------------------------------------- host side
static int mixed_setup(Operator& op) {
  if (op.mixed) return BF_OK;
  const Plan& p = op.plan;
  auto ms = std::make_unique<MixedState>();
  const int64_t ns = p.n_stages();
  const int64_t nt = (int64_t)p.tasks.size();
  // block offsets
  std::vector<int64_t> moff(nt, -1);
  std::vector<int2> items;
  int64_t off = 0;
  ms->stage_fbytes.assign(ns, 0);
  ms->stage_io.assign(ns, 0);
  ms->stage_mn.assign(ns, 0);
  ms->stage_mnp.assign(ns, 0);
  for (int64_t s = 0; s < ns; ++s)
    for (int64_t ti = p.stage_begin[s]; ti < p.stage_begin[s + 1]; ++ti) {
      const DTask& t = p.tasks[ti];
      ms->stage_io[s] += (int64_t)t.M + t.n;
      if (t.kind != TASK_DENSE) continue;
      const int64_t Mb = (t.M + 7) / 8, nb = (t.n + 7) / 8;
      moff[ti] = off;
      for (int64_t bj = 0; bj < nb; ++bj) items.push_back(make_int2((int)ti, (int)bj));
      off += Mb * nb * 1024;
      ms->stage_fbytes[s] += Mb * nb * 1024;
      ms->stage_mn[s] += (int64_t)t.M * t.n;
      ms->stage_mnp[s] += Mb * nb * 64;
    }
  ms->F_bytes = off;
  // work units: (task, first output block, output blocks), largest task first per stage
  std::vector<int4> units;
  auto make_units = [&](bool adj, std::vector<int64_t>& beg) {
    beg.assign(ns + 1, 0);
    for (int64_t s = 0; s < ns; ++s) {
      beg[s] = (int64_t)units.size();
      std::vector<std::pair<int64_t, int4>> us;
      for (int64_t ti = p.stage_begin[s]; ti < p.stage_begin[s + 1]; ++ti) {
        const DTask& t = p.tasks[ti];
        if (t.kind != TASK_DENSE) continue;
        const int Mb = (t.M + 7) / 8, nb = (t.n + 7) / 8;
        const int nout_b = adj ? nb : Mb, nin_b = adj ? Mb : nb;
        // the units of one task share its input rows: keyed by the task's work they
        // stay next to each other in the queue, so the second unit's gathers find
        // the rows the first one just brought into L2
        int64_t work = 0;
        for (int o = 0; o < nout_b; o += MX_OB)
          work += (int64_t)((nin_b + MX_IB - 1) / MX_IB) * (4 + std::min(MX_OB, nout_b - o));
        for (int o = 0; o < nout_b; o += MX_OB)
          us.push_back({work, make_int4((int)ti, o, std::min(MX_OB, nout_b - o), 0)});
      }
      std::stable_sort(us.begin(), us.end(),
                       [](const auto& a, const auto& b) { return a.first > b.first; });
      for (auto& x : us) units.push_back(x.second);
    }
    beg[ns] = (int64_t)units.size();
  };
  make_units(false, ms->ufwd);
  make_units(true, ms->uadj);
  ms->units_total = (int64_t)units.size();
  if (units.size() > (size_t)INT32_MAX) {
    set_error("mixed: too many work units");
    return BF_EINVAL;
  }
  BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
  cudaStream_t st = op.stream;
  auto alloc = [&](void** ptr, size_t bytes, const char* what) -> int {
    if (cudaMalloc(ptr, std::max<size_t>(bytes, 16)) != cudaSuccess) {
      cudaGetLastError();
      set_error("mixed: cannot allocate %zu bytes of %s", bytes, what);
      return BF_ENOMEM;
    }
    return BF_OK;
  };
  BF_TRY(alloc((void**)&ms->d_F, (size_t)ms->F_bytes, "BF16 factor blocks"));
  BF_TRY_CUDA(cudaMemsetAsync(ms->d_F, 0, (size_t)ms->F_bytes, st));
  BF_TRY(alloc((void**)&ms->d_moff, nt * sizeof(int64_t), "block offsets"));
  BF_TRY_CUDA(cudaMemcpyAsync(ms->d_moff, moff.data(), nt * sizeof(int64_t),
                              cudaMemcpyHostToDevice, st));
  BF_TRY(alloc((void**)&ms->d_units, units.size() * sizeof(int4), "work units"));
  BF_TRY_CUDA(cudaMemcpyAsync(ms->d_units, units.data(), units.size() * sizeof(int4),
                              cudaMemcpyHostToDevice, st));
  BF_TRY(alloc((void**)&ms->d_counters, (size_t)std::max<int64_t>(ns, 1) * sizeof(int),
               "counters"));
  BF_TRY(alloc((void**)&ms->d_ws, (size_t)std::max<int64_t>(p.ws_entries, 1) * MX_R * sizeof(float2),
               "workspace"));
  BF_TRY_CUDA(cudaMemsetAsync(ms->d_ws, 0,
                              (size_t)std::max<int64_t>(p.ws_entries, 1) * MX_R * sizeof(float2), st));
  if (!items.empty()) {
    int2* d_items = nullptr;
    BF_TRY(alloc((void**)&d_items, items.size() * sizeof(int2), "pack items"));
    BF_TRY_CUDA(cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(int2),
                                cudaMemcpyHostToDevice, st));
    for (size_t b = 0; b < items.size(); b += (1u << 30)) {
      const size_t nb = std::min<size_t>(items.size() - b, 1u << 30);
      if (op.d_A2)
        mx_pack_kernel<float2><<<(unsigned)nb, 128, 0, st>>>(d_items + b, op.d_tasks, ms->d_moff,
                                                             op.d_A2, ms->d_F);
      else
        mx_pack_kernel<float4><<<(unsigned)nb, 128, 0, st>>>(d_items + b, op.d_tasks, ms->d_moff,
                                                             op.d_A, ms->d_F);
    }
    BF_TRY_CUDA(cudaGetLastError());
    BF_TRY_CUDA(cudaStreamSynchronize(st));
    cudaFree(d_items);
  }
  BF_TRY_CUDA(cudaFuncSetAttribute(mx_level_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)MX_SMEM));
  BF_TRY_CUDA(cudaFuncSetAttribute(mx_level_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)MX_SMEM));
  BF_TRY_CUDA(cudaStreamSynchronize(st));
  op.mixed = ms.release();
  return BF_OK;
}

// Launches of level s of the mixed path (counters must be zero); returns the
// number of kernels launched or -1.
static int mixed_stage(Operator& op, int64_t s, int trans, cudaStream_t st) {
  MixedState& ms = *static_cast<MixedState*>(op.mixed);
  const Plan& p = op.plan;
  const bool adj = trans != BF_OP_N;
  const int conj = trans == BF_OP_T ? 1 : 0;
  const std::vector<int64_t>& ub = adj ? ms.uadj : ms.ufwd;
  const int64_t b = ub[s], n = ub[s + 1] - ub[s];
  int nk = 0;
  if (n > 0) {
    const int grid = (int)std::min<int64_t>(
        n, (int64_t)MX_CTAS_PER_SM * op.ctx->prop.multiProcessorCount);
    if (adj)
      mx_level_kernel<1><<<grid, MX_THREADS, MX_SMEM, st>>>(
          ms.d_units + b, (int)n, ms.d_counters + s, op.d_tasks, ms.d_moff, ms.d_F, op.d_maps,
          ms.d_ws, conj, op.d_err);
    else
      mx_level_kernel<0><<<grid, MX_THREADS, MX_SMEM, st>>>(
          ms.d_units + b, (int)n, ms.d_counters + s, op.d_tasks, ms.d_moff, ms.d_F, op.d_maps,
          ms.d_ws, conj, op.d_err);
    ++nk;
  }
  const int64_t cb = p.list_begin[Plan::L_COPY][s], cn = p.list_begin[Plan::L_COPY][s + 1] - cb;
  if (cn > 0) {
    mx_copy_kernel<<<(unsigned)cn, MX_R, 0, st>>>(op.d_lists + cb, op.d_tasks, op.d_maps,
                                                  ms.d_ws, adj ? 1 : 0);
    ++nk;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("mixed level launch failed: %s", cudaGetErrorString(e));
    return -1;
  }
  return nk;
}

// One chunk of at most MX_R right-hand sides, device pointers.
static int mixed_chunk(Operator& op, int trans, int nr, const double2* x, int64_t ldx,
                       double2* y, int64_t ldy, double2 alpha, double2 beta, cudaStream_t st,
                       int64_t* nk_out, std::vector<cudaEvent_t>* ev) {
  MixedState& ms = *static_cast<MixedState*>(op.mixed);
  const Plan& p = op.plan;
  const bool fwd = trans == BF_OP_N;
  const int64_t nin = fwd ? p.n_cols : p.n_rows;
  const int64_t nout = fwd ? p.n_rows : p.n_cols;
  const int64_t in_off = fwd ? p.xg_off : p.yg_off;
  const int64_t out_off = fwd ? p.yg_off : p.xg_off;
  const bool covered = fwd ? p.yg_covered : p.xg_covered;
  const int64_t ns = p.n_stages();
  int64_t nk = 0;
  BF_TRY_CUDA(cudaMemsetAsync(ms.d_counters, 0, (size_t)std::max<int64_t>(ns, 1) * sizeof(int), st));
  if (nin > 0) {
    mx_split_kernel<<<grid_rows(nin, 32), 256, 0, st>>>(x, ldx, nin, nr, ms.d_ws, in_off,
                                                        fwd ? op.d_xperm : op.d_yperm, 0);
    ++nk;
  }
  if (!covered)
    BF_TRY_CUDA(cudaMemsetAsync(ms.d_ws + (size_t)out_off * MX_R, 0,
                                (size_t)nout * MX_R * sizeof(float2), st));
  if (ev) BF_TRY_CUDA(cudaEventRecord((*ev)[0], st));
  for (int64_t k = 0; k < ns; ++k) {
    const int64_t s = fwd ? k : ns - 1 - k;
    const int r = mixed_stage(op, s, trans, st);
    if (r < 0) return BF_ECUDA;
    nk += r;
    if (ev) BF_TRY_CUDA(cudaEventRecord((*ev)[k + 1], st));
  }
  if (nout > 0) {
    mx_combine_kernel<<<grid_rows(nout, 32), 256, 0, st>>>(
        y, ldy, nout, nr, ms.d_ws, out_off, fwd ? op.d_yperm : op.d_xperm, alpha, beta,
        beta.x == 0.0 && beta.y == 0.0, 0);
    ++nk;
  }
  BF_TRY_CUDA(cudaGetLastError());
  if (nk_out) *nk_out = nk;
  return BF_OK;
}

static int check_err(Operator& op, cudaStream_t st) {
  int h = 0;
  BF_TRY_CUDA(cudaMemcpyAsync(&h, op.d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  BF_TRY_CUDA(cudaStreamSynchronize(st));
  if (h != 0) {
    cudaMemsetAsync(op.d_err, 0, sizeof(int), st);
    set_error("mixed matvec: a bounded wait timed out on the device (code %d)", h);
    return BF_ETIMEOUT;
  }
  return BF_OK;
}

int run_matvec_mixed(Operator& op, int trans, int64_t nrhs, const double* x, int64_t ldx,
                     double* y, int64_t ldy, const double* alpha, const double* beta,
                     int ptr_mode, cudaStream_t stream) {
  const Plan& p = op.plan;
  if (trans != BF_OP_N && trans != BF_OP_C && trans != BF_OP_T) {
    set_error("bf_matvec_mixed: invalid trans %d", trans);
    return BF_EINVAL;
  }
  const int64_t nin = trans == BF_OP_N ? p.n_cols : p.n_rows;
  const int64_t nout = trans == BF_OP_N ? p.n_rows : p.n_cols;
  if (nrhs < 0 || (nrhs > 0 && (!x || !y || ldx < nin || ldy < nout))) {
    set_error("bf_matvec_mixed: invalid sizes (nrhs=%lld ldx=%lld ldy=%lld, need %lld/%lld)",
              (long long)nrhs, (long long)ldx, (long long)ldy, (long long)nin, (long long)nout);
    return BF_EINVAL;
  }
  if (ptr_mode != BF_PTR_HOST && ptr_mode != BF_PTR_DEVICE) {
    set_error("bf_matvec_mixed: invalid ptr_mode %d", ptr_mode);
    return BF_EINVAL;
  }
  if (nrhs == 0) return BF_OK;
  BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
  BF_TRY(mixed_setup(op));
  MixedState& ms = *static_cast<MixedState*>(op.mixed);
  const double2 a = make_double2(alpha ? alpha[0] : 1.0, alpha ? alpha[1] : 0.0);
  const double2 b = make_double2(beta ? beta[0] : 0.0, beta ? beta[1] : 0.0);
  const bool bzero = b.x == 0.0 && b.y == 0.0;
  cudaStream_t st = stream ? stream : op.stream;
  const double2* xd = (const double2*)x;
  double2* yd = (double2*)y;
  int64_t lx = ldx, ly = ldy;
  if (ptr_mode == BF_PTR_HOST) {
    const int64_t need = std::max(p.n_rows, p.n_cols) * nrhs;
    if (need > ms.stage_cap) {
      if (ms.d_x) cudaFree(ms.d_x);
      if (ms.d_y) cudaFree(ms.d_y);
      ms.d_x = ms.d_y = nullptr;
      ms.stage_cap = 0;
      BF_TRY_CUDA(cudaMalloc(&ms.d_x, (size_t)need * 2 * sizeof(double)));
      BF_TRY_CUDA(cudaMalloc(&ms.d_y, (size_t)need * 2 * sizeof(double)));
      ms.stage_cap = need;
    }
    BF_TRY_CUDA(cudaMemcpy2DAsync(ms.d_x, nin * 2 * sizeof(double), x, ldx * 2 * sizeof(double),
                                  nin * 2 * sizeof(double), nrhs, cudaMemcpyHostToDevice, st));
    if (!bzero)
      BF_TRY_CUDA(cudaMemcpy2DAsync(ms.d_y, nout * 2 * sizeof(double), y,
                                    ldy * 2 * sizeof(double), nout * 2 * sizeof(double), nrhs,
                                    cudaMemcpyHostToDevice, st));
    xd = (const double2*)ms.d_x;
    yd = (double2*)ms.d_y;
    lx = nin;
    ly = nout;
  }
  for (int64_t c0 = 0; c0 < nrhs; c0 += MX_R) {
    const int nr = (int)std::min<int64_t>(MX_R, nrhs - c0);
    BF_TRY(mixed_chunk(op, trans, nr, xd + c0 * lx, lx, yd + c0 * ly, ly, a, b, st, nullptr,
                       nullptr));
  }
  // the near field, FP64-accurate, column by column on top of the far field
  if (op.near) BF_TRY(near_apply_columns(op, trans, nrhs, xd, lx, yd, ly, a, st));
  if (ptr_mode == BF_PTR_HOST)
    BF_TRY_CUDA(cudaMemcpy2DAsync(y, ldy * 2 * sizeof(double), ms.d_y, nout * 2 * sizeof(double),
                                  nout * 2 * sizeof(double), nrhs, cudaMemcpyDeviceToHost, st));
  return check_err(op, st);
}

// Per-level device time of one 128-RHS chunk (events around every level).
int profile_matvec_mixed(Operator& op, int trans, int nrep, double* ms_out, int64_t* bytes,
                         double* flops, int64_t* kernels) {
  const Plan& p = op.plan;
  BF_TRY_CUDA(cudaSetDevice(op.ctx->device));
  BF_TRY(mixed_setup(op));
  MixedState& ms = *static_cast<MixedState*>(op.mixed);
  const int64_t ns = p.n_stages();
  if (nrep < 1) nrep = 1;
  cudaStream_t st = op.stream;
  const int64_t nin = trans == BF_OP_N ? p.n_cols : p.n_rows;
  const int64_t nout = trans == BF_OP_N ? p.n_rows : p.n_cols;
  double2* x = nullptr;
  double2* y = nullptr;
  BF_TRY_CUDA(cudaMalloc(&x, (size_t)std::max<int64_t>(nin, 1) * MX_R * sizeof(double2)));
  BF_TRY_CUDA(cudaMalloc(&y, (size_t)std::max<int64_t>(nout, 1) * MX_R * sizeof(double2)));
  BF_TRY_CUDA(cudaMemsetAsync(x, 0, (size_t)std::max<int64_t>(nin, 1) * MX_R * sizeof(double2), st));
  std::vector<cudaEvent_t> ev(ns + 1);
  for (auto& e : ev) BF_TRY_CUDA(cudaEventCreate(&e));
  std::vector<double> acc(ns, 0.0);
  int64_t nk = 0;
  int rc = BF_OK;
  for (int r = 0; r < nrep + 1 && rc == BF_OK; ++r) {
    rc = mixed_chunk(op, trans, MX_R, x, nin, y, nout, make_double2(1, 0), make_double2(0, 0),
                     st, &nk, &ev);
    if (rc != BF_OK) break;
    if (cudaEventSynchronize(ev[ns]) != cudaSuccess) {
      rc = BF_ECUDA;
      break;
    }
    if (r == 0) continue;
    for (int64_t k = 0; k < ns; ++k) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      acc[trans == BF_OP_N ? k : ns - 1 - k] += t;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  cudaFree(x);
  cudaFree(y);
  BF_TRY(rc);
  BF_TRY(check_err(op, st));
  for (int64_t s = 0; s < ns; ++s) {
    if (ms_out) ms_out[s] = acc[s] / nrep;
    if (bytes) bytes[s] = ms.stage_fbytes[s] + ms.stage_io[s] * MX_R * (int64_t)sizeof(float2);
    if (flops) flops[s] = 8.0 * MX_R * (double)ms.stage_mn[s];
  }
  if (kernels) *kernels = nk;
  return BF_OK;
}

int mixed_info(Operator& op, int64_t* factor_bytes, int64_t* ws_bytes, int64_t* units) {
  BF_TRY(mixed_setup(op));
  MixedState& ms = *static_cast<MixedState*>(op.mixed);
  if (factor_bytes) *factor_bytes = ms.F_bytes;
  if (ws_bytes) *ws_bytes = op.plan.ws_entries * MX_R * (int64_t)sizeof(float2);
  if (units) *units = ms.units_total;
  return BF_OK;
}

}  // namespace bfg
