// Double-float ("float-float") arithmetic for FP64-accurate complex products on
// the FP32 pipes.  A real value is an unevaluated sum hi + lo of two floats
// (about 48 significant bits); a complex value is a float4
// (re_hi, re_lo, im_hi, im_lo).
//
// Methods: Dekker/Knuth TwoSum for the running sum and an FMA-based TwoProduct
// for the high partial product (Dekker 1971; Knuth TAOCP vol. 2, 4.2.2;
// Ogita-Rump-Oishi 2005 for the compensated dot-product pattern).  The cross
// terms hi*lo are added in plain float, which bounds the per-product relative
// error near 2^-47.  Only __f*_rn intrinsics are used so that the compiler can
// neither contract nor reassociate the error-free transformations.
#pragma once

#include <cuda_runtime.h>

namespace bfg {

// s += a * b, (sh, sl) an unnormalised float-float accumulator.
__device__ __forceinline__ void df_mac(float& sh, float& sl, float ah, float al, float bh,
                                       float bl) {
  float ph = __fmul_rn(ah, bh);
  float pl = __fmaf_rn(ah, bh, -ph);
  pl = __fmaf_rn(ah, bl, pl);
  pl = __fmaf_rn(al, bh, pl);
  float s = __fadd_rn(sh, ph);
  float v = __fsub_rn(s, sh);
  float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, v)), __fsub_rn(ph, v));
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(e, pl));
}

// (ah, al) += (bh, bl)
__device__ __forceinline__ void df_add(float& ah, float& al, float bh, float bl) {
  float s = __fadd_rn(ah, bh);
  float v = __fsub_rn(s, ah);
  float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, v)), __fsub_rn(bh, v));
  ah = s;
  al = __fadd_rn(al, __fadd_rn(e, bl));
}

// canonical form: |lo| <= ulp(hi)/2
__device__ __forceinline__ void df_norm(float& h, float& l) {
  float s = __fadd_rn(h, l);
  l = __fsub_rn(l, __fsub_rn(s, h));
  h = s;
}

// acc += a * x          (forward, transpose)
__device__ __forceinline__ void cdf_mac(float4& acc, const float4 a, const float4 x) {
  df_mac(acc.x, acc.y, a.x, a.y, x.x, x.y);
  df_mac(acc.x, acc.y, -a.z, -a.w, x.z, x.w);
  df_mac(acc.z, acc.w, a.x, a.y, x.z, x.w);
  df_mac(acc.z, acc.w, a.z, a.w, x.x, x.y);
}

// acc += conj(a) * x    (adjoint)
__device__ __forceinline__ void cdf_mac_conj(float4& acc, const float4 a, const float4 x) {
  df_mac(acc.x, acc.y, a.x, a.y, x.x, x.y);
  df_mac(acc.x, acc.y, a.z, a.w, x.z, x.w);
  df_mac(acc.z, acc.w, a.x, a.y, x.z, x.w);
  df_mac(acc.z, acc.w, -a.z, -a.w, x.x, x.y);
}

// s += a * b with a single float a (a factor stored in complex FP32): the
// product a*bh is split exactly by the FMA, a*bl joins the low part.
__device__ __forceinline__ void df_mac1(float& sh, float& sl, float a, float bh, float bl) {
  float ph = __fmul_rn(a, bh);
  float pl = __fmaf_rn(a, bh, -ph);
  pl = __fmaf_rn(a, bl, pl);
  float s = __fadd_rn(sh, ph);
  float v = __fsub_rn(s, sh);
  float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, v)), __fsub_rn(ph, v));
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(e, pl));
}

// acc += a * x, a complex FP32 (re, im)
__device__ __forceinline__ void cdf_mac(float4& acc, const float2 a, const float4 x) {
  df_mac1(acc.x, acc.y, a.x, x.x, x.y);
  df_mac1(acc.x, acc.y, -a.y, x.z, x.w);
  df_mac1(acc.z, acc.w, a.x, x.z, x.w);
  df_mac1(acc.z, acc.w, a.y, x.x, x.y);
}

// acc += conj(a) * x, a complex FP32
__device__ __forceinline__ void cdf_mac_conj(float4& acc, const float2 a, const float4 x) {
  df_mac1(acc.x, acc.y, a.x, x.x, x.y);
  df_mac1(acc.x, acc.y, a.y, x.z, x.w);
  df_mac1(acc.z, acc.w, a.x, x.z, x.w);
  df_mac1(acc.z, acc.w, -a.y, x.x, x.y);
}

// zero factor entry of either storage type
template <typename FT>
__device__ __forceinline__ FT fac_zero();
template <>
__device__ __forceinline__ float4 fac_zero<float4>() {
  return make_float4(0.f, 0.f, 0.f, 0.f);
}
template <>
__device__ __forceinline__ float2 fac_zero<float2>() {
  return make_float2(0.f, 0.f);
}

// complex FP32 value of a factor entry (float-float entries are rounded)
__device__ __forceinline__ float2 fac_c32(const float4 a) {
  return make_float2(a.x + a.y, a.z + a.w);
}
__device__ __forceinline__ float2 fac_c32(const float2 a) { return a; }

__device__ __forceinline__ void cdf_add(float4& a, const float4 b) {
  df_add(a.x, a.y, b.x, b.y);
  df_add(a.z, a.w, b.z, b.w);
}

__device__ __forceinline__ float4 cdf_norm(float4 a) {
  df_norm(a.x, a.y);
  df_norm(a.z, a.w);
  return a;
}

// FP64 value -> float-float (exact for |v| in the normal float range up to the
// 48-bit width of the pair).
__device__ __forceinline__ float2 df_split(double v) {
  float h = __double2float_rn(v);
  float l = __double2float_rn(v - (double)h);
  return make_float2(h, l);
}

}  // namespace bfg
