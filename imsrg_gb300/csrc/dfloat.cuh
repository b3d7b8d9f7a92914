// Double-float arithmetic for sums on the FP32 pipe (FP64 runs at about
// 1/64 of the FP32 rate on this part): (hi, lo) float pairs with Dekker /
// Knuth error-free transformations, about 2^-44 relative per term.  The
// conversions to and from the pairs use integer instructions.
#pragma once

#include <cuda_runtime.h>

namespace imsrg {

// v -> (hi, lo): hi = v truncated to 24 bits, lo = the remaining 29 bits rounded
// to 24; values below the float range give 0 (far below the tolerance).
__device__ __forceinline__ float2 d2ff(double v)
{
  long long b = __double_as_longlong(v);
  unsigned sgn = (unsigned)((unsigned long long)b >> 63) << 31;
  int e = (int)((b >> 52) & 0x7FF);
  int fe = e - 1023 + 127;
  if (e == 0 || fe <= 0) return make_float2(0.f, 0.f);
  if (fe >= 255) return make_float2(__uint_as_float(sgn | 0x7F800000u), 0.f);
  unsigned long long m = (unsigned long long)b & 0xFFFFFFFFFFFFFull;
  float hi = __uint_as_float(sgn | ((unsigned)fe << 23) | (unsigned)(m >> 29));
  unsigned r = (unsigned)(m & 0x1FFFFFFFull);
  float lo = 0.f;
  if (r) {
    int p = 31 - __clz(r);
    int le = fe - 52 + p;
    if (le > 0) {
      unsigned mant = p >= 23 ? (r >> (p - 23)) : (r << (23 - p));
      lo = __uint_as_float(sgn | ((unsigned)le << 23) | (mant & 0x7FFFFFu));
    }
  }
  return make_float2(hi, lo);
}

// exact float -> double by exponent re-bias (zero / subnormal -> 0)
__device__ __forceinline__ double f2d(float f)
{
  unsigned b = __float_as_uint(f);
  unsigned e = (b >> 23) & 0xFFu;
  if (e == 0) return 0.0;
  unsigned long long db = ((unsigned long long)(b >> 31) << 63) | ((unsigned long long)(e - 127 + 1023) << 52) |
                          ((unsigned long long)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)db);
}

// (s, c) += a * b in double-float
__device__ __forceinline__ void df_fma(float2 a, float2 b, float& s, float& c)
{
  float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  float t = __fadd_rn(s, p);
  float z = __fsub_rn(t, s);
  float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
  s = t;
  c = __fadd_rn(c, __fadd_rn(err, e));
}

// (hi, lo) -> double with integer instructions: hi exactly, then lo added as
// a whole number of ulps of hi (|lo| <= ulp_f32(hi) / 2, so hi + lo stays in
// hi's binade except just below a power of two, where the ulps halve)
__device__ __forceinline__ double ff2d(float hi, float lo)
{
  unsigned hb = __float_as_uint(hi), lb = __float_as_uint(lo);
  int eh = (hb >> 23) & 0xFF, el = (lb >> 23) & 0xFF;
  if (eh == 0) return f2d(lo);
  double h = f2d(hi);
  if (el == 0) return h;
  long long bits = __double_as_longlong(h);
  int sh = el - eh + 29;  // lo = m 2^(el-150), ulp(h) = 2^(eh-179)
  long long m = (long long)((lb & 0x7FFFFFu) | 0x800000u);
  long long off = sh >= 0 ? (m << sh) : (sh > -25 ? (m >> -sh) : 0ll);
  if ((hb ^ lb) >> 31) {
    if ((bits & 0xFFFFFFFFFFFFFll) == 0) off <<= 1;
    bits -= off;
  } else {
    bits += off;
  }
  return __longlong_as_double(bits);
}

// (hi, lo) = (s1 + c1) + (s2 + c2), renormalised
__device__ __forceinline__ void df_add(float s1, float c1, float s2, float c2, float& hi, float& lo)
{
  float s = __fadd_rn(s1, s2);
  float bb = __fsub_rn(s, s1);
  float e = __fadd_rn(__fsub_rn(s1, __fsub_rn(s, bb)), __fsub_rn(s2, bb));
  e = __fadd_rn(e, __fadd_rn(c1, c2));
  hi = __fadd_rn(s, e);
  lo = __fsub_rn(e, __fsub_rn(hi, s));
}

}  // namespace imsrg
