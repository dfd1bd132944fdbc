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

__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

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

// storage (double2) <-> compute (dfc); identity for the native types
template <typename K> __device__ __forceinline__ K to_compute(double2 v);
template <> __device__ __forceinline__ double2 to_compute<double2>(double2 v) { return v; }
template <> __device__ __forceinline__ dfc to_compute<dfc>(double2 v) { return dfc{df(v.x), df(v.y)}; }
template <typename K> __device__ __forceinline__ K to_compute(float2 v) { return v; }

__device__ __forceinline__ double2 to_storage(double2 v, double2) { return v; }
__device__ __forceinline__ double2 to_storage(dfc v, double2) {
  return make_double2(df_to_double(v.x), df_to_double(v.y));
}
__device__ __forceinline__ float2 to_storage(float2 v, float2) { return v; }

}  // namespace vs
