// Double-float arithmetic on the FP32 pipe (shared by the Lanczos kernels).
//
// A complex128 value x is carried as two complex64 parts, x = hi + lo (hi = x
// rounded to FP32, lo = the rest rounded to FP32: 48 significand bits), stored
// as float4 {re_hi, im_hi, re_lo, im_lo}.  Sums are (hi, lo) FP32 pairs: each
// real product a*b is ah*bh split exactly into p + e by one FMA, plus the
// cross terms ah*bl + al*bh; p goes into the pair by Knuth's two-sum, e and
// the cross terms into its low part.  Relative error of a product ~2^-47
// instead of 2^-53, at FP32-pipe speed (this part's FP64 rate is ~1/60 of its
// FP32 rate).
#pragma once

namespace ed {

struct DF {
  float hi, lo;
};
__device__ __forceinline__ void df_acc(DF& s, float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  const float e = fmaf(ah, bh, -p);
  const float c = fmaf(ah, bl, fmaf(al, bh, e));
  const float t = s.hi + p;
  const float bb = t - s.hi;
  const float err = (s.hi - (t - bb)) + (p - bb);
  s.hi = t;
  s.lo += err + c;
}
// s -= a*b
__device__ __forceinline__ void df_sub(DF& s, float ah, float al, float bh, float bl) { df_acc(s, -ah, -al, bh, bl); }

__device__ __forceinline__ float4 split_c128(double2 v) {
  const float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
  return make_float4(rh, ih, __double2float_rn(v.x - (double)rh), __double2float_rn(v.y - (double)ih));
}

__device__ __forceinline__ double df_value(const DF& s) { return (double)s.hi + (double)s.lo; }

}  // namespace ed
