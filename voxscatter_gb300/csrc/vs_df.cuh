// Double-float arithmetic: a real number is carried as the unevaluated sum
// hi + lo of two floats (|lo| <= ulp(hi)/2), about 48 significant bits, on
// the FP32 pipes.  GB300 issues FP32 operations at several tens of times its
// FP64 rate, so FP64-accuracy work that is bound by FP64 arithmetic (the
// FFTs of the refinement residual) runs faster in double-float.
//
// Published methods used (no library code): Knuth's TwoSum (TAOCP vol. 2,
// 4.2.2) and Dekker's renormalisation (Numer. Math. 18 (1971) 224-242) for
// the sum; the FMA form of Dekker's exact product (a*b - fl(a*b) is one
// fused multiply-add) for the product; the "sloppy" double-float addition
// of Dekker, whose error is within a few units of 2^-48 (|a| + |b|), the
// accuracy an FFT needs.  The intrinsics __fadd_rn / __fsub_rn / __fmul_rn
// keep the compiler from contracting or reassociating the error terms.
#pragma once
#include "vs_common.cuh"

namespace vs {

struct df {
  float hi, lo;
  __host__ __device__ df() {}
  // the nearest double-float to a double (exact for the double's top 48 bits)
  __host__ __device__ constexpr df(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};

__device__ __forceinline__ df df_make(float hi, float lo) {
  df r;
  r.hi = hi;
  r.lo = lo;
  return r;
}

// hi + lo with |lo| <= ulp(hi)/2 from s + e (|e| small against s)
__device__ __forceinline__ df df_renorm(float s, float e) {
  const float h = __fadd_rn(s, e);
  return df_make(h, __fsub_rn(e, __fsub_rn(h, s)));
}

__device__ __forceinline__ df operator+(df a, df b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float v = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));  // TwoSum error
  return df_renorm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ df operator-(df a) { return df_make(-a.hi, -a.lo); }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }

__device__ __forceinline__ df& operator+=(df& a, df b) { return a = a + b; }
__device__ __forceinline__ df& operator-=(df& a, df b) { return a = a - b; }

__device__ __forceinline__ df operator*(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);  // exact error of the leading product
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_renorm(p, e);
}

// complex double-float
struct dfc {
  df x, y;
};

__device__ __forceinline__ dfc cadd(dfc a, dfc b) { return dfc{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ dfc csub(dfc a, dfc b) { return dfc{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ dfc cmul(dfc a, dfc b) { return dfc{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
// a + b * c
__device__ __forceinline__ dfc cfma(dfc b, dfc c, dfc a) {
  return dfc{a.x + (b.x * c.x - b.y * c.y), a.y + (b.x * c.y + b.y * c.x)};
}
__device__ __forceinline__ dfc cconj(dfc a) { return dfc{a.x, -a.y}; }
template <> __device__ __forceinline__ dfc czero<dfc>() { return dfc{df(0.0), df(0.0)}; }

// Conversions between FP64 storage and double-float from the bits, on the
// integer and FP32 pipes: the FP64 conversions (and the FP64 subtraction
// that forms lo) run on GB300's FP64 pipe, at a small fraction of its FP32
// rate, and bound the double-float passes at loads and stores.
//
// The double-float nearest a double: hi = RN(d), lo = RN(d - hi), the same
// bits as the FP64 conversions (round to nearest, ties to even).  Fast path
// for d = 0 and for 2^-74 <= |d| < 2^126 (biased exponent 949..1149, where
// hi and lo are normal floats); other values take the FP64 conversions.
// From the 53-bit significand S of |d|: hi keeps its top 24 bits, rounded on
// the other 29 (a carry out of the mantissa moves into the exponent field);
// the rounding residual r = S mod 2^29 (less 2^29 if rounded up) is exact,
// |r| <= 2^28, and lo = RN(r) 2^(e-52): r's two halves convert exactly
// through the 1.5 * 2^23 mantissa trick and one FMA rounds their sum.
__device__ __forceinline__ df df_from_double(double d) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(d);
  const unsigned h = (unsigned)(bits >> 32), l = (unsigned)bits;
  const unsigned eb = (h >> 20) & 0x7FFu;
  if (eb - 949u <= 1149u - 949u) {
    const unsigned sign = h & 0x80000000u;
    const unsigned m23 = ((h & 0xFFFFFu) << 3) | (l >> 29);
    const unsigned rem = l & 0x1FFFFFFFu;
    const unsigned up = (rem > 0x10000000u ? 1u : 0u) | ((rem == 0x10000000u ? 1u : 0u) & m23);
    const float hi = __uint_as_float(sign | (((eb - 896u) << 23) + m23 + up));
    int r = (int)rem - (int)(up << 29);
    if (sign) r = -r;
    const float ra = __fsub_rn(__int_as_float(0x4B400000 + (r >> 14)), 12582912.0f);
    const float rb = __fsub_rn(__int_as_float(0x4B400000 + (r & 0x3FFF)), 12582912.0f);
    const float lo = __fmul_rn(__fmaf_rn(ra, 16384.0f, rb), __uint_as_float((eb - 948u) << 23));
    return df_make(hi, lo);
  }
  if ((h & 0x7FFFFFFFu) == 0u && l == 0u) return df_make(__uint_as_float(h), 0.0f);  // +-0
  return df(d);
}
// A float widened to double from its bits (exact; normal floats and zeros,
// others by the FP64 conversion).
__device__ __forceinline__ double double_from_float(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xFFu;
  if (e - 1u < 254u)
    return __hiloint2double((int)((b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7FFFFFu) >> 3)), (int)(b << 29));
  if ((b & 0x7FFFFFFFu) == 0u) return __hiloint2double((int)b, 0);
  return (double)f;
}
// hi + lo rounded to double: one FP64 addition
__device__ __forceinline__ double df_store(df a) { return double_from_float(a.hi) + double_from_float(a.lo); }

// storage (double2) <-> compute (dfc); identity for the native types
template <typename K> __device__ __forceinline__ K to_compute(double2 v);
template <> __device__ __forceinline__ double2 to_compute<double2>(double2 v) { return v; }
template <> __device__ __forceinline__ dfc to_compute<dfc>(double2 v) {
  return dfc{df_from_double(v.x), df_from_double(v.y)};
}
template <typename K> __device__ __forceinline__ K to_compute(float2 v) { return v; }

__device__ __forceinline__ double2 to_storage(double2 v, double2) { return v; }
__device__ __forceinline__ double2 to_storage(dfc v, double2) { return make_double2(df_store(v.x), df_store(v.y)); }
__device__ __forceinline__ float2 to_storage(float2 v, float2) { return v; }

}  // namespace vs
