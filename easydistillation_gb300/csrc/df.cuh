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
// Fold the low part back into the high one (fast two-sum, |lo| <= |hi|): long sums renormalise every few terms so
// that the low part's own rounding stays at 2^-48 of the sum instead of growing with the number of terms.
__device__ __forceinline__ void df_renorm(DF& s) {
  const float t = s.hi + s.lo;
  s.lo -= t - s.hi;
  s.hi = t;
}

__device__ __forceinline__ float4 split_c128(double2 v) {
  const float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
  return make_float4(rh, ih, __double2float_rn(v.x - (double)rh), __double2float_rn(v.y - (double)ih));
}

__device__ __forceinline__ double df_value(const DF& s) { return (double)s.hi + (double)s.lo; }

// The split of df.cuh computed with integer operations on the bits of d (no
// FP64-pipe conversion): hi = d truncated to 24 significant bits, lo = the
// remaining 29 bits rounded to FP32, so hi + lo carries 48 bits of d.  Values
// below 2^-126 in magnitude give hi = 0 (and below about 2^-74 lo = 0 as
// well): absolute errors under 2^-100, far below the data's scale; magnitudes
// of 2^128 and above are out of range (hi = inf).
__device__ __forceinline__ void split_bits(double d, float& hi, float& lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  const unsigned int h32 = (unsigned int)(u >> 32), l32 = (unsigned int)u;
  const unsigned int sign = h32 & 0x80000000u;
  const int e = (int)((h32 >> 20) & 0x7FFu);  // biased FP64 exponent
  const int ef = e - 896;                     // biased FP32 exponent of hi
  unsigned int hb = 0u;
  if (ef >= 255) hb = sign | 0x7F800000u;
  else if (ef > 0) hb = sign | ((unsigned int)ef << 23) | ((h32 & 0xFFFFFu) << 3) | (l32 >> 29);
  hi = __uint_as_float(hb);
  // lo = (the low 29 bits of the significand) * 2^(e - 1075), with d's sign
  const int es = e - 948;  // biased FP32 exponent of 2^(e - 1075)
  float l = 0.f;
  if (ef > 0 && es > 0) l = __uint2float_rn(l32 & 0x1FFFFFFFu) * __uint_as_float((unsigned int)min(es, 254) << 23);
  lo = sign ? -l : l;
}
__device__ __forceinline__ float4 split_c128_bits(double2 v) {
  float4 r;
  split_bits(v.x, r.x, r.z);
  split_bits(v.y, r.y, r.w);
  return r;
}
// an FP32 value as FP64 through its bits (exact; zero and subnormals give 0)
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned int b = __float_as_uint(f);
  const unsigned int ex = (b >> 23) & 0xFFu;
  if (ex == 0u) return 0.0;
  const unsigned long long r = ((unsigned long long)(b & 0x80000000u) << 32) |
                               ((unsigned long long)(ex + 896u) << 52) | ((unsigned long long)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)r);
}

}  // namespace ed
