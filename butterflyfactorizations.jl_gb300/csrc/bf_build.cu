// Batched construction kernels: observer-row sampling, Helmholtz kernel
// sampling, column-pivoted partial QR and interpolation matrices.
//
// One compression of the reference PartialQR compressor
// (src/ButterflyFactorization/compressors.jl:81-165) is one CTask here; all
// compressions of one butterfly level of all far blocks run in the same
// launches.  Precision follows the design rule of this library: FP64 only for
// the k*r range reduction of the kernel phase and for the QR column norms,
// their downdates and the pivot choice; Householder updates, the triangular
// solve and the factors themselves are complex FP32.
#include <algorithm>
#include <cfloat>

#include "bf_build.h"

namespace bfg {
namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// position pi(j) of the keyed bijection of [0, n) (same definition as the
// host and the oracle: 4-round Feistel on [0, 4^h) with cycle walking)
__device__ long long sample_position(long long j, long long n, unsigned long long key) {
  if (n <= 1) return 0;
  int bits = 64 - __clzll((unsigned long long)(n - 1));
  int h = (bits + 1) / 2;
  unsigned long long mask = (1ull << h) - 1ull;
  unsigned long long x = (unsigned long long)j;
  // cycle walking terminates: pi is a bijection of [0, 4^h) and 4^h < 4n
  for (int guard = 0; guard < 4096; ++guard) {
    unsigned long long L = x >> h, R = x & mask;
#pragma unroll
    for (int rnd = 0; rnd < 4; ++rnd) {
      unsigned long long F = mix64(key ^ ((unsigned long long)(rnd + 1) << 56) ^ R) & mask;
      unsigned long long t = L ^ F;
      L = R;
      R = t;
    }
    x = (L << h) | R;
    if (x < (unsigned long long)n) return (long long)x;
  }
  return j % n;  // unreachable for a bijection; keeps the index in range
}

__global__ void rows_kernel(const CTask* __restrict__ tasks, int ntasks,
                            const int32_t* __restrict__ obs_perm, int32_t* __restrict__ rowpool) {
  int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (w >= ntasks) return;
  const CTask t = tasks[w];
  for (int j = lane; j < t.n_rows; j += 32)
    rowpool[t.rows_off + j] = obs_perm[t.obs_begin + sample_position(j, t.n_obs, t.key)];
}

// G(r) = exp(-i k r) / (4 pi r).  k*r and its reduction modulo 2 pi in FP64
// (Cody-Waite with 2 pi split in two doubles), then FP32 sincos of the reduced
// phase.
__device__ __forceinline__ float2 helmholtz(const double* __restrict__ a,
                                            const double* __restrict__ b, double k) {
  double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  double r = sqrt(fma(dx, dx, fma(dy, dy, dz * dz)));
  const double TWO_PI_HI = 6.283185307179586232;
  const double TWO_PI_LO = 2.449293598294706414e-16;
  const double INV_TWO_PI = 0.15915494309189533577;
  double th = k * r;
  double q = rint(th * INV_TWO_PI);
  double red = fma(-q, TWO_PI_HI, th);
  red = fma(-q, TWO_PI_LO, red);
  float s, c;
  sincosf((float)red, &s, &c);
  float inv = 1.0f / (float)(12.566370614359172954 * r);
  return make_float2(c * inv, -s * inv);
}

// Z[i + j*n] = G(obs[rows[i]], src[cols[j]]) for one task per CTA.
// mode 0: Z batch at z_off (ld = n_rows); mode 1: raw factor store at t_off.
__global__ void eval_kernel(const CTask* __restrict__ tasks, const double* __restrict__ obs,
                            const double* __restrict__ src, const int32_t* __restrict__ rowpool,
                            const int32_t* __restrict__ colpool, float2* __restrict__ out,
                            double k, int mode) {
  const CTask t = tasks[blockIdx.x];
  const int n = t.n_rows, m = t.n_cols;
  float2* __restrict__ o = out + (mode == 0 ? t.z_off : t.t_off);
  const int32_t* __restrict__ rows = rowpool + t.rows_off;
  const int32_t* __restrict__ cols = colpool + t.cols_off;
  const long long tot = (long long)n * m;
  for (long long e = threadIdx.x; e < tot; e += blockDim.x) {
    int j = (int)(e / n), i = (int)(e - (long long)j * n);
    o[e] = helmholtz(obs + 3 * (long long)rows[i], src + 3 * (long long)cols[j], k);
  }
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double cabs2(float2 a) {
  return (double)a.x * a.x + (double)a.y * a.y;
}

// Sum of |c[i]|^2 over i = i0, i0+step, ... < i1, as an FP64 value.  Every
// square of an FP32 value is split exactly into a float pair by the FMA and
// added with TwoSum into a float-float accumulator on the FP32 pipes (relative
// error ~ count * 2^-48); the pair is rounded to FP64 once.  This keeps the
// column norms FP64-accurate without one FP64 operation per entry, which on
// GB300's narrow FP64 pipe bounded the QR kernel.
__device__ __forceinline__ void ff_add(float& sh, float& sl, float b) {
  const float s = __fadd_rn(sh, b);
  const float v = __fsub_rn(s, sh);
  sl = __fadd_rn(sl, __fadd_rn(__fsub_rn(sh, __fsub_rn(s, v)), __fsub_rn(b, v)));
  sh = s;
}
__device__ __forceinline__ double sumsq(const float2* __restrict__ c, int i0, int i1, int step) {
  float sh = 0.f, sl = 0.f;
  for (int i = i0; i < i1; i += step) {
    const float2 a = c[i];
    const float p = __fmul_rn(a.x, a.x), q = __fmul_rn(a.y, a.y);
    ff_add(sh, sl, p);
    ff_add(sh, sl, q);
    sl = __fadd_rn(sl, __fadd_rn(__fmaf_rn(a.x, a.x, -p), __fmaf_rn(a.y, a.y, -q)));
  }
  return (double)sh + (double)sl;
}

// Column-pivoted Householder QR of one sampled block, stopped once the largest
// remaining column norm is <= eps * |R_00| (the truncation of LowRankApprox.pqr
// with rtol = eps, compressors.jl:129).  LAPACK xGEQP3/xLAQP2 conventions:
// H = I - tau v v^H with v(0) = 1, trailing update by H^H, norm downdating with
// recomputation when cancellation exceeds sqrt(eps_fp32).
template <bool SMEM>
__global__ void __launch_bounds__(QR_NT) qr_kernel(CTask* __restrict__ tasks,
                                                   float2* __restrict__ Zg,
                                                   int32_t* __restrict__ permpool) {
  extern __shared__ __align__(16) unsigned char smraw[];
  CTask& task = tasks[blockIdx.x];
  const int n = task.n_rows, m = task.n_cols, tid = threadIdx.x;
  double* nrm = (double*)smraw;
  double* orig = nrm + m;
  double* rv = orig + m;             // 32 doubles
  int* ri = (int*)(rv + 32);         // 32 ints
  float2* sc = (float2*)(ri + 32);   // 4 float2 broadcast scalars
  int* perm = (int*)(sc + 4);
  float2* Z;
  int ld;
  if (SMEM) {
    Z = (float2*)(((uintptr_t)(perm + m) + 15) & ~(uintptr_t)15);
    ld = n | 1;  // odd stride: conflict-free per-column sweeps
    const float2* src = Zg + task.z_off;
    for (long long e = tid; e < (long long)n * m; e += QR_NT) {
      int j = (int)(e / n), i = (int)(e - (long long)j * n);
      Z[i + (long long)j * ld] = src[e];
    }
  } else {
    Z = Zg + task.z_off;
    ld = n;
  }
  __syncthreads();
  for (int j = tid; j < m; j += QR_NT) {
    perm[j] = j;
    const double s = sumsq(Z + (long long)j * ld, 0, n, 1);
    nrm[j] = s;
    orig[j] = s;
  }
  __syncthreads();
  const int kmax = min(n, m);
  const double tol3z = 2.44140625e-4;  // sqrt(FP32 epsilon)
  double r00 = 0.0;
  int rank = kmax;
  for (int k = 0; k < kmax; ++k) {
    // pivot: the largest remaining FP64 column norm, lowest index on ties.
    // Non-negative doubles (and the -1 sentinel) order like their bit
    // patterns read as signed 64-bit integers, so the search runs on the
    // integer pipes; thread 0 alone combines the warps, takes the square root
    // and decides the truncation (r00 lives in thread 0).
    long long bv = __double_as_longlong(-1.0);
    int bi = m;
    for (int j = k + tid; j < m; j += QR_NT) {
      const long long v = __double_as_longlong(nrm[j]);
      if (v > bv) {
        bv = v;
        bi = j;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) {
        bv = ov;
        bi = oi;
      }
    }
    if ((tid & 31) == 0) {
      rv[tid >> 5] = __longlong_as_double(bv);
      ri[tid >> 5] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      for (int w = 1; w < QR_NT / 32; ++w) {
        const long long ov = __double_as_longlong(rv[w]);
        if (ov > bv || (ov == bv && ri[w] < bi)) {
          bv = ov;
          bi = ri[w];
        }
      }
      const double pn = sqrt(fmax(__longlong_as_double(bv), 0.0));
      if (k == 0) r00 = pn;
      ri[QR_NT / 32] = bi;
      ri[QR_NT / 32 + 1] = (r00 == 0.0 || pn <= task.eps * r00) ? 1 : 0;
    }
    __syncthreads();
    if (ri[QR_NT / 32 + 1]) {
      rank = k;
      break;
    }
    bi = ri[QR_NT / 32];
    if (bi != k) {
      for (int i = tid; i < n; i += QR_NT) {
        float2 a = Z[i + (long long)k * ld];
        Z[i + (long long)k * ld] = Z[i + (long long)bi * ld];
        Z[i + (long long)bi * ld] = a;
      }
      if (tid == 0) {
        double t = nrm[k];
        nrm[k] = nrm[bi];
        nrm[bi] = t;
        t = orig[k];
        orig[k] = orig[bi];
        orig[bi] = t;
        int p = perm[k];
        perm[k] = perm[bi];
        perm[bi] = p;
      }
    }
    __syncthreads();
    // Householder reflector of column k: warp 0 sums the squares below the
    // diagonal, its lane 0 forms tau and the scale
    if (tid < 32) {
      double xn2 = sumsq(Z + (long long)k * ld, k + 1 + tid, n, 32);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) xn2 += __shfl_xor_sync(0xffffffffu, xn2, o);
      if (tid == 0) {
        float2 alpha = Z[k + (long long)k * ld];
        if (xn2 == 0.0 && alpha.y == 0.0f) {
          sc[0] = make_float2(0.f, 0.f);  // tau = 0, H = I
          sc[1] = make_float2(0.f, 0.f);
        } else {
          double ar = alpha.x, ai = alpha.y;
          double beta = -copysign(sqrt(ar * ar + ai * ai + xn2), ar);
          float2 tau = make_float2((float)((beta - ar) / beta), (float)(-ai / beta));
          double dr = ar - beta, di = ai;  // scale = 1 / (alpha - beta)
          double den = dr * dr + di * di;
          sc[0] = tau;
          sc[1] = make_float2((float)(dr / den), (float)(-di / den));
          Z[k + (long long)k * ld] = make_float2((float)beta, 0.f);
        }
      }
    }
    __syncthreads();
    const float2 tau = sc[0], scale = sc[1];
    if (tau.x != 0.f || tau.y != 0.f) {
      for (int i = k + 1 + tid; i < n; i += QR_NT)
        Z[i + (long long)k * ld] = cmul(Z[i + (long long)k * ld], scale);
      __syncthreads();
      const float2 ctau = make_float2(tau.x, -tau.y);
      const float2* v = Z + (long long)k * ld;
      for (int j = k + 1 + tid; j < m; j += QR_NT) {
        float2* c = Z + (long long)j * ld;
        float2 w = c[k];
        for (int i = k + 1; i < n; ++i) {
          float2 t = cmulc(v[i], c[i]);
          w.x += t.x;
          w.y += t.y;
        }
        float2 f = cmul(ctau, w);
        c[k].x -= f.x;
        c[k].y -= f.y;
        for (int i = k + 1; i < n; ++i) {
          float2 t = cmul(v[i], f);
          c[i].x -= t.x;
          c[i].y -= t.y;
        }
      }
    }
    __syncthreads();
    // norm downdate (xLAQP2), in FP64.  The norms here are squared, so
    // xLAQP2's nrm*max(1 - |z|^2/nrm, 0) is max(nrm - |z|^2, 0) and its
    // cancellation test max(1 - |z|^2/nrm, 0)*nrm/orig <= tol3z reads
    // max(nrm - |z|^2, 0) <= tol3z*orig: the same quantities without the two
    // FP64 divisions per column and step, which bound this kernel on the FP64
    // pipe.
    for (int j = k + 1 + tid; j < m; j += QR_NT) {
      if (nrm[j] > 0.0) {
        const double t = fmax(nrm[j] - cabs2(Z[k + (long long)j * ld]), 0.0);
        if (t <= tol3z * orig[j]) {
          const double s = sumsq(Z + (long long)j * ld, k + 1, n, 1);
          nrm[j] = s;
          orig[j] = s;
        } else {
          nrm[j] = t;
        }
      }
    }
    __syncthreads();
  }
  if (tid == 0) task.rank = rank;
  for (int j = tid; j < m; j += QR_NT) permpool[task.perm_off + j] = perm[j];
  if (SMEM) {  // R rows back to the batch buffer for the interpolation solve
    float2* dst = Zg + task.z_off;
    for (long long e = tid; e < (long long)rank * m; e += QR_NT) {
      int j = (int)(e / rank), i = (int)(e - (long long)j * rank);
      dst[i + (long long)j * n] = Z[i + (long long)j * ld];
    }
  }
}

// T = R11^-1 [R11 R12] P^T (interpolation matrix, r x m, column-major ld r)
// written at raw[t_off]; skeleton = cols[perm[0..r)] at skelpool[skel_off].
__global__ void __launch_bounds__(128) tsolve_kernel(const CTask* __restrict__ tasks,
                                                     const float2* __restrict__ Zg,
                                                     const int32_t* __restrict__ permpool,
                                                     const int32_t* __restrict__ colpool,
                                                     float2* __restrict__ raw,
                                                     int32_t* __restrict__ skelpool,
                                                     int smem_r) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const CTask t = tasks[blockIdx.x];
  const int r = t.rank, m = t.n_cols, n = t.n_rows;
  if (r <= 0) return;
  const float2* __restrict__ R = Zg + t.z_off;  // ld n
  const int32_t* __restrict__ perm = permpool + t.perm_off;
  float2* __restrict__ T = raw + t.t_off;
  const bool use_smem = r <= smem_r;  // R11 fits the launch's shared memory
  float2* R11 = (float2*)smraw;
  if (use_smem) {
    for (int e = threadIdx.x; e < r * r; e += blockDim.x) {
      int j = e / r, i = e - j * r;
      R11[e] = R[i + (long long)j * n];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < r; i += blockDim.x)
    skelpool[t.skel_off + i] = colpool[t.cols_off + perm[i]];
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    float2* x = T + (long long)r * perm[j];
    if (j < r) {
      for (int i = 0; i < r; ++i) x[i] = make_float2(i == j ? 1.f : 0.f, 0.f);
      continue;
    }
    for (int i = 0; i < r; ++i) x[i] = R[i + (long long)j * n];
    // back substitution, column sweep
    for (int l = r - 1; l >= 0; --l) {
      float2 d = use_smem ? R11[l + l * r] : R[l + (long long)l * n];  // real diagonal
      float2 xl = x[l];
      xl.x /= d.x;
      xl.y /= d.x;
      x[l] = xl;
      for (int i = 0; i < l; ++i) {
        float2 a = use_smem ? R11[i + l * r] : R[i + (long long)l * n];
        float2 p = cmul(a, xl);
        x[i].x -= p.x;
        x[i].y -= p.y;
      }
    }
  }
}

}  // namespace

int launch_rows(const CTask* d_tasks, int ntasks, const int32_t* d_obs_perm, int32_t* d_rowpool,
                cudaStream_t st) {
  if (ntasks <= 0) return BF_OK;
  int threads = 256;
  int blocks = (int)(((long long)ntasks * 32 + threads - 1) / threads);
  rows_kernel<<<blocks, threads, 0, st>>>(d_tasks, ntasks, d_obs_perm, d_rowpool);
  BF_TRY_CUDA(cudaGetLastError());
  return BF_OK;
}

int launch_eval(const CTask* d_tasks, int ntasks, const double* d_obs, const double* d_src,
                const int32_t* d_rowpool, const int32_t* d_colpool, float2* d_out, double k,
                int mode, cudaStream_t st) {
  if (ntasks <= 0) return BF_OK;
  eval_kernel<<<ntasks, 128, 0, st>>>(d_tasks, d_obs, d_src, d_rowpool, d_colpool, d_out, k,
                                      mode);
  BF_TRY_CUDA(cudaGetLastError());
  return BF_OK;
}

size_t qr_smem_bytes(int n, int m, bool with_z) {
  size_t b = (size_t)m * 2 * sizeof(double) + 32 * sizeof(double) + 32 * sizeof(int) +
             4 * sizeof(float2) + (size_t)m * sizeof(int) + 16;
  if (with_z) b += (size_t)(n | 1) * m * sizeof(float2);
  return b;
}

int launch_qr(CTask* d_tasks, int ntasks, float2* d_Z, int32_t* d_permpool, bool smem_z,
              size_t smem, cudaStream_t st) {
  if (ntasks <= 0) return BF_OK;
  static DeviceOnce attr;
  BF_TRY(attr.run([] {
    cudaError_t e = cudaFuncSetAttribute(qr_kernel<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, QR_MAX_SMEM);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(qr_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                QR_MAX_SMEM);
  }, "qr_kernel shared memory"));
  if (smem_z)
    qr_kernel<true><<<ntasks, QR_NT, smem, st>>>(d_tasks, d_Z, d_permpool);
  else
    qr_kernel<false><<<ntasks, QR_NT, smem, st>>>(d_tasks, d_Z, d_permpool);
  BF_TRY_CUDA(cudaGetLastError());
  return BF_OK;
}

namespace {
__global__ void ranks_kernel(const CTask* __restrict__ tasks, int n, int32_t* __restrict__ ranks) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    ranks[i] = tasks[i].rank;
}
__global__ void compact_done_kernel(const CTask* __restrict__ tasks, const CDone* __restrict__ done,
                                    int n, CTask* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const CDone d = done[i];
    CTask c = tasks[d.q];
    c.t_off = d.t_off;
    c.skel_off = d.skel_off;
    out[i] = c;
  }
}
}  // namespace

int launch_ranks(const CTask* d_tasks, int ntasks, int32_t* d_ranks, cudaStream_t st) {
  if (ntasks <= 0) return BF_OK;
  ranks_kernel<<<std::min((ntasks + 255) / 256, 4096), 256, 0, st>>>(d_tasks, ntasks, d_ranks);
  BF_TRY_CUDA(cudaGetLastError());
  return BF_OK;
}

int launch_compact_done(const CTask* d_tasks, const CDone* d_done, int ndone, CTask* d_out,
                        cudaStream_t st) {
  if (ndone <= 0) return BF_OK;
  compact_done_kernel<<<std::min((ndone + 255) / 256, 4096), 256, 0, st>>>(d_tasks, d_done, ndone,
                                                                          d_out);
  BF_TRY_CUDA(cudaGetLastError());
  return BF_OK;
}

int launch_tsolve(const CTask* d_tasks, int ntasks, const float2* d_Z, const int32_t* d_permpool,
                  const int32_t* d_colpool, float2* d_raw, int32_t* d_skel, int max_rank,
                  cudaStream_t st) {
  if (ntasks <= 0) return BF_OK;
  static DeviceOnce attr;
  BF_TRY(attr.run([] {
    return cudaFuncSetAttribute(tsolve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                TS_MAX_SMEM_R * TS_MAX_SMEM_R * (int)sizeof(float2));
  }, "tsolve_kernel shared memory"));
  int rr = max_rank <= TS_MAX_SMEM_R ? max_rank : 0;
  size_t smem = (size_t)rr * rr * sizeof(float2);
  tsolve_kernel<<<ntasks, 128, smem, st>>>(d_tasks, d_Z, d_permpool, d_colpool, d_raw, d_skel,
                                          rr);
  BF_TRY_CUDA(cudaGetLastError());
  return BF_OK;
}

}  // namespace bfg
