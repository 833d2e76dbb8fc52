// Double-float ("float-float") helpers: a value is carried as an unevaluated
// sum hi + lo of two floats (Dekker 1971; Knuth's TwoSum).  Products of the
// hi parts are made exact with one fma; the small cross terms are added in
// plain FP32.  On GB300 the FP32 pipes issue ~60x the FP64 rate, so a
// double-float complex multiply-accumulate (~48 FP32 ops) is several times
// faster than four DFMAs while keeping ~2^-48 relative accuracy.
#pragma once
#include "common.cuh"

namespace mgt {

// complex double-float: x = re_hi, y = re_lo, z = im_hi, w = im_lo
__device__ __forceinline__ float4 df_split(double2 v) {
  float rh = (float)v.x, ih = (float)v.y;
  return make_float4(rh, (float)(v.x - (double)rh), ih, (float)(v.y - (double)ih));
}
__device__ __forceinline__ double2 df_join(float4 v) {
  return make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
}

// (h, l) += p + q where p is large and q a small correction.
__device__ __forceinline__ void df_acc(float& h, float& l, float p, float q) {
  float s = h + p;
  float bb = s - h;
  float err = (h - (s - bb)) + (p - bb);
  h = s;
  l += err + q;
}

// acc += (a_h + a_l)(b_h + b_l), one real product
__device__ __forceinline__ void df_mac(float& h, float& l, float ah, float al, float bh, float bl) {
  float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  float t = fmaf(ah, bl, al * bh);
  df_acc(h, l, p, e + t);
}

// complex: acc (re_h, re_l, im_h, im_l) += a * b
__device__ __forceinline__ void df_cmac(float4& acc, float4 a, float4 b) {
  df_mac(acc.x, acc.y, a.x, a.y, b.x, b.y);     // + ar br
  df_mac(acc.x, acc.y, -a.z, -a.w, b.z, b.w);   // - ai bi
  df_mac(acc.z, acc.w, a.x, a.y, b.z, b.w);     // + ar bi
  df_mac(acc.z, acc.w, a.z, a.w, b.x, b.y);     // + ai br
}

}  // namespace mgt
