// Learned rank surrogate: a 4 -> 64 -> 64 -> 1 GELU MLP predicting the log
// skeleton rank of one compression from (level, k * box diameter,
// separation / diameter, log point count).  No reference counterpart: it
// replaces the fixed ButterflyRankEstimator sample count
// (src/ButterflyFactorization/rankestimation.jl:93-98) so that the batched
// partial QR rarely needs the adaptive re-sampling of compressors.jl:134-151.
//
// Weight vector layout (float32, SUR_NW entries):
//   mu[4] sigma[4]        feature normalisation
//   W1[64][4]  b1[64]     layer 1 (row-major, out x in)
//   W2[64][64] b2[64]     layer 2
//   W3[64]     b3[1]      output
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

#include "bf_internal.h"

namespace bfg {

constexpr int SUR_IN = 4;
constexpr int SUR_H = 64;
constexpr int SUR_NW = 8 + SUR_H * SUR_IN + SUR_H + SUR_H * SUR_H + SUR_H + SUR_H + 1;

// Features of one compression: (level, k * box diameter, centre separation /
// diameter, log point count), the point count being that of the compressed
// problem, min(observer points, columns) -- an upper bound of its rank.
inline void surrogate_features(const Tree& to, const Tree& ts, double k, int stage, int64_t o,
                               int64_t s, int64_t n_obs, int64_t n_cols, float f[4]) {
  double ao = to.radius(o), as = ts.radius(s);
  double D = 2.0 * std::max(ao, as);
  double d2 = 0.0;
  for (int a = 0; a < 3; ++a) {
    double d = to.center[3 * o + a] - ts.center[3 * s + a];
    d2 += d * d;
  }
  f[0] = (float)stage;
  f[1] = (float)(k * D);
  f[2] = (float)(D > 0 ? std::sqrt(d2) / D : 0.0);
  f[3] = (float)std::log(1.0 + (double)std::min(n_obs, n_cols));
}

struct Surrogate {
  std::vector<float> w;
  bool load(const float* p, int64_t n) {
    if (!p || n != SUR_NW) return false;
    w.assign(p, p + n);
    for (float v : w)
      if (!std::isfinite(v)) return false;
    for (int i = 0; i < 4; ++i)
      if (!(w[4 + i] > 0.f)) return false;  // normalisation scales
    return true;
  }
};

// GPU inference of a batch of feature rows (features: n x 4, out: n)
int surrogate_predict_gpu(const float* d_weights, const float* d_feat, float* d_out, int64_t n,
                          cudaStream_t st);

}  // namespace bfg
