// Host evaluation of the rank surrogate MLP (same arithmetic as the GPU
// inference kernel: BF16-rounded weights, FP32 accumulation, tanh-form GELU).
#include <cstring>

#include "bf_surrogate.h"

namespace bfg {

static inline float bf16_round(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  uint32_t r = ((u >> 16) & 1u) + 0x7FFFu;  // round to nearest even
  u = (u + r) & 0xFFFF0000u;
  float y;
  std::memcpy(&y, &u, 4);
  return y;
}

static inline float gelu(float x) {
  const float c = 0.7978845608028654f;  // sqrt(2/pi)
  return 0.5f * x * (1.0f + std::tanh(c * (x + 0.044715f * x * x * x)));
}

float Surrogate::predict_log_rank(const float f[4]) const {
  const float* mu = w.data();
  const float* sg = mu + 4;
  const float* W1 = sg + 4;
  const float* b1 = W1 + SUR_H * SUR_IN;
  const float* W2 = b1 + SUR_H;
  const float* b2 = W2 + SUR_H * SUR_H;
  const float* W3 = b2 + SUR_H;
  const float* b3 = W3 + SUR_H;
  float x[SUR_IN], h1[SUR_H], h2[SUR_H];
  for (int i = 0; i < SUR_IN; ++i) x[i] = (f[i] - mu[i]) / sg[i];
  for (int o = 0; o < SUR_H; ++o) {
    float a = b1[o];
    for (int i = 0; i < SUR_IN; ++i) a += bf16_round(W1[o * SUR_IN + i]) * x[i];
    h1[o] = gelu(a);
  }
  for (int o = 0; o < SUR_H; ++o) {
    float a = b2[o];
    for (int i = 0; i < SUR_H; ++i) a += bf16_round(W2[o * SUR_H + i]) * h1[i];
    h2[o] = gelu(a);
  }
  float a = b3[0];
  for (int i = 0; i < SUR_H; ++i) a += bf16_round(W3[i]) * h2[i];
  return a;
}

}  // namespace bfg
