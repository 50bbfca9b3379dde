// Learned rank surrogate: GPU inference and training kernels.
//
// Network (bf_surrogate.h): x = (f - mu) / sigma, h1 = gelu(W1 x + b1),
// h2 = gelu(W2 h1 + b2), y = w3 . h2 + b3 with 4 inputs and 64 hidden units,
// y = predicted log skeleton rank.  Weights are kept in FP32 (master copy) and
// rounded to BF16 (nearest even) wherever the network is evaluated; products
// accumulate in FP32.  Gradients pass straight through the rounding.
// gelu is the tanh form (Hendrycks & Gimpel 2016), evaluated with tanhf.
//
// Kernels:
//   sur_predict_kernel   thread per sample, weights in shared memory, the
//                        second layer fused with the output (h2 never stored);
//   sur_grad_kernel      CTA per tile of 64 samples: forward and backward as
//                        small shared-memory matrix products, one partial
//                        gradient (NW floats) and loss per CTA;
//   sur_update_kernel    thread per weight: sums the CTA partials in a fixed
//                        order (deterministic), optionally one Adam step
//                        (Kingma & Ba 2015), the normalisation entries fixed.
// The network is tiny (4.4 k multiply-adds per sample): FP32 FMAs with BF16
// weights keep a million-record epoch well under a millisecond per pass, so
// no tensor-core tiling is used here.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bf_internal.h"
#include "bf_surrogate.h"

namespace bfg {
namespace {

constexpr int H = SUR_H;
constexpr int TILE = 64;      // samples per training CTA
constexpr int GT = 256;       // threads per training CTA
constexpr int LD = H + 1;     // padded row length of the activation tiles
// weight-vector offsets
constexpr int O_MU = 0, O_SG = 4, O_W1 = 8, O_B1 = O_W1 + H * SUR_IN, O_W2 = O_B1 + H,
              O_B2 = O_W2 + H * H, O_W3 = O_B2 + H, O_B3 = O_W3 + H;
static_assert(O_B3 + 1 == SUR_NW, "surrogate layout");

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ float gelu_f(float x) {
  const float c = 0.7978845608028654f, a = 0.044715f;
  return 0.5f * x * (1.0f + tanhf(c * (x + a * x * x * x)));
}

__device__ __forceinline__ float gelu_g(float x) {
  const float c = 0.7978845608028654f, a = 0.044715f;
  const float t = tanhf(c * (x + a * x * x * x));
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * c * (1.0f + 3.0f * a * x * x);
}

// ---------------------------------------------------------------- inference
constexpr int PT = 64;  // threads (samples in flight) per inference CTA

__global__ void __launch_bounds__(PT) sur_predict_kernel(const float* __restrict__ w,
                                                         const float* __restrict__ feat,
                                                         float* __restrict__ out, int64_t n) {
  __shared__ float sW1[H * SUR_IN], sb1[H], sW2[H * H], sb2[H], sW3[H], sx[8];
  __shared__ float sh1[H][PT + 1];  // hidden layer 1, one column per thread
  __shared__ float sb3;
  for (int i = threadIdx.x; i < H * SUR_IN; i += blockDim.x) sW1[i] = bf16r(w[O_W1 + i]);
  for (int i = threadIdx.x; i < H * H; i += blockDim.x) sW2[i] = bf16r(w[O_W2 + i]);
  for (int i = threadIdx.x; i < H; i += blockDim.x) {
    sb1[i] = w[O_B1 + i];
    sb2[i] = w[O_B2 + i];
    sW3[i] = bf16r(w[O_W3 + i]);
  }
  if (threadIdx.x < 8) sx[threadIdx.x] = w[threadIdx.x];
  if (threadIdx.x == 0) sb3 = w[O_B3];
  __syncthreads();
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int c = threadIdx.x;
    float x[SUR_IN];
#pragma unroll
    for (int i = 0; i < SUR_IN; ++i) x[i] = (feat[4 * s + i] - sx[i]) / sx[4 + i];
    for (int o = 0; o < H; ++o) {
      float a = sb1[o];
#pragma unroll
      for (int i = 0; i < SUR_IN; ++i) a = fmaf(sW1[o * SUR_IN + i], x[i], a);
      sh1[o][c] = gelu_f(a);
    }
    float y = sb3;
    for (int o = 0; o < H; ++o) {
      float a = sb2[o];
#pragma unroll 16
      for (int i = 0; i < H; ++i) a = fmaf(sW2[o * H + i], sh1[i][c], a);
      y = fmaf(sW3[o], gelu_f(a), y);
    }
    out[s] = y;
  }
}

// ---------------------------------------------------------------- training
struct GradSmem {
  float W1[H * SUR_IN], b1[H], W2[H * H], W2T[H * H], b2[H], W3[H];
  float X[TILE][SUR_IN], T[TILE], dy[TILE], red[GT];
  float Z1[TILE][LD], H1[TILE][LD], Z2[TILE][LD], H2[TILE][LD], dZ2[TILE][LD], dZ1[TILE][LD];
  float b3;
};

// One tile of samples idx[tile*TILE ...] (idx == nullptr: consecutive); inv_b =
// 1 / (samples of the whole batch).  Writes part[blockIdx.x * NW ...] and
// loss_part[blockIdx.x].
__global__ void __launch_bounds__(GT) sur_grad_kernel(const float* __restrict__ w,
                                                      const float* __restrict__ feat,
                                                      const float* __restrict__ target,
                                                      const int32_t* __restrict__ idx,
                                                      int64_t first, int64_t count, float inv_b,
                                                      float* __restrict__ part,
                                                      float* __restrict__ loss_part) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GradSmem& S = *reinterpret_cast<GradSmem*>(smem_raw);
  const int t = threadIdx.x;
  for (int i = t; i < H * SUR_IN; i += GT) S.W1[i] = bf16r(w[O_W1 + i]);
  for (int i = t; i < H * H; i += GT) {
    const float v = bf16r(w[O_W2 + i]);
    S.W2[i] = v;
    S.W2T[(i % H) * H + i / H] = v;  // W2T[in][out]
  }
  for (int i = t; i < H; i += GT) {
    S.b1[i] = w[O_B1 + i];
    S.b2[i] = w[O_B2 + i];
    S.W3[i] = bf16r(w[O_W3 + i]);
  }
  if (t == 0) S.b3 = w[O_B3];
  const int64_t base = (int64_t)blockIdx.x * TILE;
  if (t < TILE) {
    const int64_t q = base + t;
    const bool ok = q < count;
    const int64_t s = ok ? (idx ? (int64_t)idx[first + q] : first + q) : 0;
#pragma unroll
    for (int i = 0; i < SUR_IN; ++i)
      S.X[t][i] = ok ? (feat[4 * s + i] - w[O_MU + i]) / w[O_SG + i] : 0.f;
    S.T[t] = ok ? target[s] : 0.f;
    S.dy[t] = ok ? 1.f : 0.f;  // validity mask until dy is known
  }
  __syncthreads();
  const int j = t % H;       // unit (column) index
  const int s0 = t / H;      // 0..3: first sample row; rows s0, s0+4, ...
  // layer 1
  for (int s = s0; s < TILE; s += GT / H) {
    float a = S.b1[j];
#pragma unroll
    for (int i = 0; i < SUR_IN; ++i) a = fmaf(S.W1[j * SUR_IN + i], S.X[s][i], a);
    S.Z1[s][j] = a;
    S.H1[s][j] = gelu_f(a);
  }
  __syncthreads();
  // layer 2: Z2[s][j] = b2[j] + sum_i W2[j][i] H1[s][i]  (W2T: consecutive j)
  for (int s = s0; s < TILE; s += GT / H) {
    float a = S.b2[j];
    for (int i = 0; i < H; ++i) a = fmaf(S.W2T[i * H + j], S.H1[s][i], a);
    S.Z2[s][j] = a;
    S.H2[s][j] = gelu_f(a);
  }
  __syncthreads();
  // output, residual, loss
  float lpart = 0.f;
  if (t < TILE) {
    float y = S.b3;
    for (int i = 0; i < H; ++i) y = fmaf(S.W3[i], S.H2[t][i], y);
    const float valid = S.dy[t];
    const float r = (y - S.T[t]) * valid;
    S.dy[t] = r * inv_b;
    lpart = 0.5f * r * r * inv_b;
  }
  S.red[t] = lpart;
  __syncthreads();
  for (int k = GT / 2; k > 0; k >>= 1) {
    if (t < k) S.red[t] += S.red[t + k];
    __syncthreads();
  }
  if (t == 0) loss_part[blockIdx.x] = S.red[0];
  float* g = part + (size_t)blockIdx.x * SUR_NW;
  // output layer gradients and dZ2
  if (t < H) {
    float a = 0.f;
    for (int s = 0; s < TILE; ++s) a = fmaf(S.dy[s], S.H2[s][t], a);
    g[O_W3 + t] = a;
  }
  if (t == H) {
    float a = 0.f;
    for (int s = 0; s < TILE; ++s) a += S.dy[s];
    g[O_B3] = a;
  }
  if (t < 8) g[t] = 0.f;  // normalisation entries are not trained
  for (int s = s0; s < TILE; s += GT / H) S.dZ2[s][j] = S.dy[s] * S.W3[j] * gelu_g(S.Z2[s][j]);
  __syncthreads();
  // dW2[jo][i] = sum_s dZ2[s][jo] H1[s][i]; thread: i = t % H, rows jo = t/H + 4q
  {
    const int i = t % H;
    for (int jo = t / H; jo < H; jo += GT / H) {
      float a = 0.f;
      for (int s = 0; s < TILE; ++s) a = fmaf(S.dZ2[s][jo], S.H1[s][i], a);
      g[O_W2 + jo * H + i] = a;
    }
  }
  if (t < H) {
    float a = 0.f;
    for (int s = 0; s < TILE; ++s) a += S.dZ2[s][t];
    g[O_B2 + t] = a;
  }
  // dH1[s][i] = sum_jo W2[jo][i] dZ2[s][jo]; dZ1 = dH1 * gelu'(Z1)
  for (int s = s0; s < TILE; s += GT / H) {
    const int i = j;
    float a = 0.f;
    for (int jo = 0; jo < H; ++jo) a = fmaf(S.W2[jo * H + i], S.dZ2[s][jo], a);
    S.dZ1[s][i] = a * gelu_g(S.Z1[s][i]);
  }
  __syncthreads();
  // dW1[jo][i] = sum_s dZ1[s][jo] X[s][i]; db1
  for (int e = t; e < H * SUR_IN; e += GT) {
    const int jo = e / SUR_IN, i = e % SUR_IN;
    float a = 0.f;
    for (int s = 0; s < TILE; ++s) a = fmaf(S.dZ1[s][jo], S.X[s][i], a);
    g[O_W1 + e] = a;
  }
  if (t < H) {
    float a = 0.f;
    for (int s = 0; s < TILE; ++s) a += S.dZ1[s][t];
    g[O_B1 + t] = a;
  }
}

// Sum of the nb partial gradients (fixed order) -> grad; with adam != 0 one
// Adam step on w (entries from 8 on).  loss = sum of the loss partials.
__global__ void sur_update_kernel(const float* __restrict__ part, const float* __restrict__ lpart,
                                  int nb, float* __restrict__ w, float* __restrict__ grad,
                                  float* __restrict__ m, float* __restrict__ v,
                                  float* __restrict__ loss_acc, int adam, float lr, float beta1,
                                  float beta2, float eps, float bc1, float bc2) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e == 0 && loss_acc) {
    float L = 0.f;
    for (int b = 0; b < nb; ++b) L += lpart[b];
    *loss_acc += L;
  }
  if (e >= SUR_NW) return;
  float gsum = 0.f;
  for (int b = 0; b < nb; ++b) gsum += part[(size_t)b * SUR_NW + e];
  if (grad) grad[e] = gsum;
  if (!adam || e < 8) return;
  const float mm = beta1 * m[e] + (1.f - beta1) * gsum;
  const float vv = beta2 * v[e] + (1.f - beta2) * gsum * gsum;
  m[e] = mm;
  v[e] = vv;
  w[e] -= lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
}

constexpr size_t GRAD_SMEM = sizeof(GradSmem);

// deterministic 64-bit mixer (SplitMix64 finaliser) for shuffles and init
inline uint64_t smix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  template <typename T>
  T* as() {
    return static_cast<T*>(p);
  }
};

int dalloc(DevBuf& b, size_t bytes) {
  if (cudaMalloc(&b.p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
    cudaGetLastError();
    set_error("surrogate: cannot allocate %zu device bytes", bytes);
    return BF_ENOMEM;
  }
  return BF_OK;
}

// one pass of gradient tiles over count samples starting at first (through
// idx when given) -> sum into grad / Adam step
int grad_pass(const float* d_w, const float* d_f, const float* d_t, const int32_t* d_idx,
              int64_t first, int64_t count, float* d_part, float* d_lpart, float* d_wmut,
              float* d_grad, float* d_m, float* d_v, float* d_loss, int adam, float lr, float b1,
              float b2, float eps, int step, cudaStream_t st) {
  const int nb = (int)((count + TILE - 1) / TILE);
  sur_grad_kernel<<<nb, GT, GRAD_SMEM, st>>>(d_w, d_f, d_t, d_idx, first, count,
                                             1.0f / (float)count, d_part, d_lpart);
  const float bc1 = adam ? 1.f - std::pow(b1, (float)step) : 1.f;
  const float bc2 = adam ? 1.f - std::pow(b2, (float)step) : 1.f;
  sur_update_kernel<<<(SUR_NW + 255) / 256, 256, 0, st>>>(d_part, d_lpart, nb, d_wmut, d_grad,
                                                          d_m, d_v, d_loss, adam, lr, b1, b2, eps,
                                                          bc1, bc2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("surrogate kernels: %s", cudaGetErrorString(e));
    return BF_ECUDA;
  }
  return BF_OK;
}

int set_grad_attr() {
  static DeviceOnce attr;
  return attr.run([] {
    return cudaFuncSetAttribute(sur_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)GRAD_SMEM);
  }, "sur_grad_kernel shared memory");
}

}  // namespace

int surrogate_predict_gpu(const float* d_weights, const float* d_feat, float* d_out, int64_t n,
                          cudaStream_t st) {
  if (n <= 0) return BF_OK;
  const int grid = (int)std::min<int64_t>((n + PT - 1) / PT, 152 * 16);
  sur_predict_kernel<<<grid, PT, 0, st>>>(d_weights, d_feat, d_out, n);
  BF_TRY_CUDA(cudaGetLastError());
  return BF_OK;
}

}  // namespace bfg

using namespace bfg;

extern "C" {

int bf_surrogate_nweights(void) { return SUR_NW; }

int bf_surrogate_init(const float* features, int64_t n, uint64_t seed, float* weights) {
  if (!features || n <= 0 || !weights) {
    set_error("bf_surrogate_init: need features (n > 0) and a weight buffer");
    return BF_EINVAL;
  }
  std::memset(weights, 0, SUR_NW * sizeof(float));
  for (int i = 0; i < SUR_IN; ++i) {
    double s = 0, s2 = 0;
    for (int64_t q = 0; q < n; ++q) {
      const double v = features[4 * q + i];
      s += v;
      s2 += v * v;
    }
    const double mean = s / (double)n;
    const double var = std::max(0.0, s2 / (double)n - mean * mean);
    weights[O_MU + i] = (float)mean;
    weights[O_SG + i] = (float)std::max(std::sqrt(var), 1e-6);
  }
  // Glorot-uniform layers, zero biases
  uint64_t st = seed;
  auto uni = [&](double a) {
    st = smix(st);
    return (float)((((double)(st >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0) * a);
  };
  const double a1 = std::sqrt(6.0 / (SUR_IN + H)), a2 = std::sqrt(6.0 / (H + H)),
               a3 = std::sqrt(6.0 / (H + 1));
  for (int i = 0; i < H * SUR_IN; ++i) weights[O_W1 + i] = uni(a1);
  for (int i = 0; i < H * H; ++i) weights[O_W2 + i] = uni(a2);
  for (int i = 0; i < H; ++i) weights[O_W3 + i] = uni(a3);
  return BF_OK;
}

int bf_surrogate_predict(bf_ctx_t ctx, const float* weights, const float* features, int64_t n,
                         float* out) {
  if (!ctx || !weights || (n > 0 && (!features || !out)) || n < 0) {
    set_error("bf_surrogate_predict: invalid arguments");
    return BF_EINVAL;
  }
  if (n == 0) return BF_OK;
  BF_TRY_CUDA(cudaSetDevice(ctx->c.device));
  DevBuf w, f, o;
  BF_TRY(dalloc(w, SUR_NW * sizeof(float)));
  BF_TRY(dalloc(f, (size_t)n * 4 * sizeof(float)));
  BF_TRY(dalloc(o, (size_t)n * sizeof(float)));
  BF_TRY_CUDA(cudaMemcpy(w.p, weights, SUR_NW * sizeof(float), cudaMemcpyHostToDevice));
  BF_TRY_CUDA(cudaMemcpy(f.p, features, (size_t)n * 4 * sizeof(float), cudaMemcpyHostToDevice));
  BF_TRY(surrogate_predict_gpu(w.as<float>(), f.as<float>(), o.as<float>(), n, 0));
  BF_TRY_CUDA(cudaMemcpy(out, o.p, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost));
  return BF_OK;
}

int bf_surrogate_grad(bf_ctx_t ctx, const float* weights, const float* features,
                      const float* targets, int64_t n, float* grad, float* loss) {
  if (!ctx || !weights || !features || !targets || n <= 0 || !grad) {
    set_error("bf_surrogate_grad: invalid arguments");
    return BF_EINVAL;
  }
  if (n > INT32_MAX) {
    set_error("bf_surrogate_grad: too many samples");
    return BF_EINVAL;
  }
  BF_TRY_CUDA(cudaSetDevice(ctx->c.device));
  BF_TRY(set_grad_attr());
  const int nb = (int)((n + TILE - 1) / TILE);
  DevBuf w, f, t, part, lpart, g, L;
  BF_TRY(dalloc(w, SUR_NW * sizeof(float)));
  BF_TRY(dalloc(f, (size_t)n * 4 * sizeof(float)));
  BF_TRY(dalloc(t, (size_t)n * sizeof(float)));
  BF_TRY(dalloc(part, (size_t)nb * SUR_NW * sizeof(float)));
  BF_TRY(dalloc(lpart, (size_t)nb * sizeof(float)));
  BF_TRY(dalloc(g, SUR_NW * sizeof(float)));
  BF_TRY(dalloc(L, sizeof(float)));
  BF_TRY_CUDA(cudaMemcpy(w.p, weights, SUR_NW * sizeof(float), cudaMemcpyHostToDevice));
  BF_TRY_CUDA(cudaMemcpy(f.p, features, (size_t)n * 4 * sizeof(float), cudaMemcpyHostToDevice));
  BF_TRY_CUDA(cudaMemcpy(t.p, targets, (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
  BF_TRY_CUDA(cudaMemset(L.p, 0, sizeof(float)));
  BF_TRY(grad_pass(w.as<float>(), f.as<float>(), t.as<float>(), nullptr, 0, n, part.as<float>(),
                   lpart.as<float>(), nullptr, g.as<float>(), nullptr, nullptr, L.as<float>(), 0,
                   0.f, 0.f, 0.f, 0.f, 1, 0));
  BF_TRY_CUDA(cudaMemcpy(grad, g.p, SUR_NW * sizeof(float), cudaMemcpyDeviceToHost));
  if (loss) BF_TRY_CUDA(cudaMemcpy(loss, L.p, sizeof(float), cudaMemcpyDeviceToHost));
  return BF_OK;
}

int bf_surrogate_train(bf_ctx_t ctx, const float* features, const float* targets, int64_t n,
                       const bf_train_opts* opts, float* weights, float* loss_per_epoch) {
  if (!ctx || !features || !targets || n <= 0 || !weights || !opts) {
    set_error("bf_surrogate_train: invalid arguments");
    return BF_EINVAL;
  }
  if (opts->epochs < 0 || opts->batch < 1 || !(opts->lr > 0.f) || n > INT32_MAX) {
    set_error("bf_surrogate_train: invalid options (epochs %d batch %d lr %g)", opts->epochs,
              opts->batch, (double)opts->lr);
    return BF_EINVAL;
  }
  BF_TRY_CUDA(cudaSetDevice(ctx->c.device));
  BF_TRY(set_grad_attr());
  const int64_t B = std::min<int64_t>(opts->batch, n);
  const int nbmax = (int)((B + TILE - 1) / TILE);
  cudaStream_t st = nullptr;
  BF_TRY_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{st};
  DevBuf w, f, t, part, lpart, m, v, L, idx;
  BF_TRY(dalloc(w, SUR_NW * sizeof(float)));
  BF_TRY(dalloc(f, (size_t)n * 4 * sizeof(float)));
  BF_TRY(dalloc(t, (size_t)n * sizeof(float)));
  BF_TRY(dalloc(part, (size_t)nbmax * SUR_NW * sizeof(float)));
  BF_TRY(dalloc(lpart, (size_t)nbmax * sizeof(float)));
  BF_TRY(dalloc(m, SUR_NW * sizeof(float)));
  BF_TRY(dalloc(v, SUR_NW * sizeof(float)));
  BF_TRY(dalloc(L, sizeof(float)));
  BF_TRY(dalloc(idx, (size_t)n * sizeof(int32_t)));
  BF_TRY_CUDA(cudaMemcpyAsync(w.p, weights, SUR_NW * sizeof(float), cudaMemcpyHostToDevice, st));
  BF_TRY_CUDA(cudaMemcpyAsync(f.p, features, (size_t)n * 4 * sizeof(float),
                              cudaMemcpyHostToDevice, st));
  BF_TRY_CUDA(cudaMemcpyAsync(t.p, targets, (size_t)n * sizeof(float), cudaMemcpyHostToDevice,
                              st));
  BF_TRY_CUDA(cudaMemsetAsync(m.p, 0, SUR_NW * sizeof(float), st));
  BF_TRY_CUDA(cudaMemsetAsync(v.p, 0, SUR_NW * sizeof(float), st));
  std::vector<int32_t> perm(n);
  for (int64_t q = 0; q < n; ++q) perm[q] = (int32_t)q;
  uint64_t rs = opts->seed ^ 0x5EEDull;
  int step = 0;
  for (int ep = 0; ep < opts->epochs; ++ep) {
    // seeded Fisher-Yates shuffle of the sample order
    for (int64_t q = n - 1; q > 0; --q) {
      rs = smix(rs);
      const int64_t r = (int64_t)(rs % (uint64_t)(q + 1));
      std::swap(perm[q], perm[r]);
    }
    BF_TRY_CUDA(cudaMemcpyAsync(idx.p, perm.data(), (size_t)n * sizeof(int32_t),
                                cudaMemcpyHostToDevice, st));
    BF_TRY_CUDA(cudaMemsetAsync(L.p, 0, sizeof(float), st));
    int nbatch = 0;
    for (int64_t b0 = 0; b0 < n; b0 += B) {
      const int64_t cnt = std::min<int64_t>(B, n - b0);
      ++step;
      ++nbatch;
      BF_TRY(grad_pass(w.as<float>(), f.as<float>(), t.as<float>(), idx.as<int32_t>(), b0, cnt,
                       part.as<float>(), lpart.as<float>(), w.as<float>(), nullptr, m.as<float>(),
                       v.as<float>(), L.as<float>(), 1, opts->lr, opts->beta1, opts->beta2,
                       opts->eps, step, st));
    }
    if (loss_per_epoch) {
      float h = 0.f;
      BF_TRY_CUDA(cudaMemcpyAsync(&h, L.p, sizeof(float), cudaMemcpyDeviceToHost, st));
      BF_TRY_CUDA(cudaStreamSynchronize(st));
      loss_per_epoch[ep] = h / (float)nbatch;
    }
  }
  BF_TRY_CUDA(cudaMemcpyAsync(weights, w.p, SUR_NW * sizeof(float), cudaMemcpyDeviceToHost, st));
  BF_TRY_CUDA(cudaStreamSynchronize(st));
  return BF_OK;
}

}  // extern "C"
