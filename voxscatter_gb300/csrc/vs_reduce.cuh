// Compensated accumulation and warp / CTA sums shared by the Krylov kernels
// and the pipeline passes that fold BiCGSTAB's vector steps in: float-float
// accumulators for c64 data (every product of two floats formed exactly by an
// FMA and added by TwoSum), double-double for c128, and deterministic warp and
// CTA sums (fixed xor trees, warp 0 adding the warps in order).
#pragma once
#include "vs_common.cuh"

#include <type_traits>

namespace vs {

// FP64 double-double accumulation (TwoSum / TwoProd by fma) for the c128 path.
struct DD {
  double hi, lo;
};
__device__ __forceinline__ DD dd_add(DD a, double b) {
  const double s = a.hi + b;
  const double bb = s - a.hi;
  const double err = (a.hi - (s - bb)) + (b - bb);
  return DD{s, a.lo + err};
}
__device__ __forceinline__ DD dd_add(DD a, DD b) {
  DD r = dd_add(a, b.hi);
  r.lo += b.lo;
  return r;
}
__device__ __forceinline__ DD dd_fma(DD a, double x, double y) {
  const double p = x * y;
  const double e = fma(x, y, -p);
  DD r = dd_add(a, p);
  r.lo += e;
  return r;
}

// Accumulators.  c64 inputs: every product of two floats is formed exactly as
// a float pair (p = a*b rounded, e = fma(a, b, -p)) and added into a
// float-float sum by TwoSum (Knuth), about 48 bits of significand for the
// few elements a thread visits; the CTA and grid sums add the pairs
// float-float as well, and one thread widens the total to double for the
// scalar step.  This keeps compensated inner products without FP64 work per
// element or per thread.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float b) {
  const float s = __fadd_rn(hi, b);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  hi = s;
  lo = __fadd_rn(lo, err);
}
__device__ __forceinline__ void ff_fma(float& hi, float& lo, float a, float b) {
  const float pr = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -pr);
  ff_add(hi, lo, pr);
  lo = __fadd_rn(lo, e);
}
// A float-float value (hi + lo, not necessarily renormalised).
struct FF2 {
  float hi, lo;
};

template <typename T>
struct Acc {
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  // the sums in their own form (float-float here, double for c128), for the
  // CTA and grid sums below
  __device__ __forceinline__ FF2 vre() const { return FF2{rh, rl}; }
  __device__ __forceinline__ FF2 vim() const { return FF2{ih, il}; }
  __device__ __forceinline__ void dot(cplx_t<T> u, cplx_t<T> v) {  // += conj(u) v
    ff_fma(rh, rl, u.x, v.x);
    ff_fma(rh, rl, u.y, v.y);
    ff_fma(ih, il, u.x, v.y);
    ff_fma(ih, il, -u.y, v.x);
  }
  __device__ __forceinline__ void norm2(cplx_t<T> u) {
    ff_fma(rh, rl, u.x, u.x);
    ff_fma(rh, rl, u.y, u.y);
  }
  __device__ __forceinline__ double2 value() const {
    return make_double2((double)rh + (double)rl, (double)ih + (double)il);
  }
};
template <>
struct Acc<double> {
  DD re{0, 0}, im{0, 0};
  __device__ __forceinline__ void dot(double2 u, double2 v) {
    re = dd_fma(re, u.x, v.x);
    re = dd_fma(re, u.y, v.y);
    im = dd_fma(im, u.x, v.y);
    im = dd_fma(im, -u.y, v.x);
  }
  __device__ __forceinline__ void norm2(double2 u) {
    re = dd_fma(re, u.x, u.x);
    re = dd_fma(re, u.y, u.y);
  }
  __device__ __forceinline__ double2 value() const { return make_double2(re.hi + re.lo, im.hi + im.lo); }
  __device__ __forceinline__ double vre() const { return re.hi + re.lo; }
  __device__ __forceinline__ double vim() const { return im.hi + im.lo; }
};

// ff (float-float) sum of two ff values: TwoSum of the leading parts, the
// trailing parts and the error added, renormalised (about 48 bits).
__device__ __forceinline__ void ff_add2(float& hi, float& lo, float bhi, float blo) {
  const float s = __fadd_rn(hi, bhi);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(bhi, bb));
  const float t = __fadd_rn(err, __fadd_rn(lo, blo));
  hi = __fadd_rn(s, t);
  lo = __fsub_rn(t, __fsub_rn(hi, s));
}

// Warp sum (xor tree) of one value per lane: float-float on the FP32 pipes
// (FF, the c64 solver's accumulators, which are float-float already), or
// double (the FP64 path, which keeps double's exponent range).
template <bool FF>
__device__ __forceinline__ double warp_sum(double v) {
  if constexpr (FF) {
    float hi = (float)v;
    float lo = (float)(v - (double)hi);
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, hi, off), ol = __shfl_xor_sync(0xffffffffu, lo, off);
      ff_add2(hi, lo, oh, ol);
    }
    return (double)hi + (double)lo;
  } else {
#pragma unroll
    for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
  }
}


// Warp sum (xor tree) of float-float values, on the FP32 pipes only.
__device__ __forceinline__ FF2 warp_sum(FF2 v) {
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, v.hi, off), ol = __shfl_xor_sync(0xffffffffu, v.lo, off);
    ff_add2(v.hi, v.lo, oh, ol);
  }
  return v;
}

__device__ __forceinline__ FF2 warp_sum_v(FF2 v) { return warp_sum(v); }
__device__ __forceinline__ double warp_sum_v(double v) { return warp_sum<false>(v); }

// A partial sum slot (8 bytes): float-float sums (the c64 solver's) are
// stored there as float2 (hi, lo), doubles as doubles.  GB300 runs FP64 at a
// small fraction of its FP32 rate, so c64 sums stay float-float from the
// per-thread accumulators to the last slot, and only the one thread that
// takes a scalar step widens them to double.
__device__ __forceinline__ void put_slot(double* p, FF2 v) { *reinterpret_cast<float2*>(p) = make_float2(v.hi, v.lo); }
__device__ __forceinline__ void put_slot(double* p, double v) { *p = v; }
// CG: through L2 only (slots written by other CTAs of the same kernel)
template <bool CG>
__device__ __forceinline__ void get_slot(const double* p, FF2& v) {
  const float2 f = CG ? __ldcg(reinterpret_cast<const float2*>(p)) : *reinterpret_cast<const float2*>(p);
  v = FF2{f.x, f.y};
}
template <bool CG>
__device__ __forceinline__ void get_slot(const double* p, double& v) {
  v = CG ? __ldcg(p) : *p;
}
__device__ __forceinline__ void add_slot(FF2& a, FF2 b) { ff_add2(a.hi, a.lo, b.hi, b.lo); }
__device__ __forceinline__ void add_slot(double& a, double b) { a += b; }
__device__ __forceinline__ double widen(FF2 v) { return (double)v.hi + (double)v.lo; }
__device__ __forceinline__ double widen(double v) { return v; }
// The slot form of a precision's sums.
template <typename T>
using SlotV = typename std::conditional<std::is_same<T, float>::value, FF2, double>::type;

// Per-thread sums x[k] of slots b * NV + k for b = t0, t0 + nt, ... < nb, in
// that order; U slots' loads are issued before their adds.
template <int NV, int U, bool CG, typename V>
__device__ __forceinline__ void slot_sums(const double* __restrict__ part, int nb, int t0, int nt, V (&x)[NV]) {
#pragma unroll
  for (int k = 0; k < NV; ++k) x[k] = V{};
  for (int b0 = t0; b0 < nb; b0 += U * nt) {
    V v[U][NV];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int k = 0; k < NV; ++k)
        if (b0 + u * nt < nb) get_slot<CG>(part + (int64_t)(b0 + u * nt) * NV + k, v[u][k]);
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int k = 0; k < NV; ++k)
        if (b0 + u * nt < nb) add_slot(x[k], v[u][k]);
  }
}

// Sums NV per-thread values over the CTA (all threads must call it) and
// writes them to out[0..NV-1] (thread 0; blockDim.x a multiple of 32, at most
// 1024 threads): float-float values by float-float warp trees into float2
// slots, doubles by double trees.
template <int NV>
__device__ __forceinline__ void cta_partials(const FF2 (&v)[NV], double* out) {
  __shared__ float2 sm[NV][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const FF2 x = warp_sum(v[k]);
    if (lane == 0) sm[k][warp] = make_float2(x.hi, x.lo);
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const float2 y = lane < nw ? sm[k][lane] : make_float2(0.f, 0.f);
      const FF2 x = warp_sum(FF2{y.x, y.y});
      if (lane == 0) put_slot(out + k, x);
    }
  }
}
template <int NV>
__device__ __forceinline__ void cta_partials(const double (&v)[NV], double* out) {
  __shared__ double sm[NV][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double x = warp_sum<false>(v[k]);
    if (lane == 0) sm[k][warp] = x;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double x = warp_sum<false>(lane < nw ? sm[k][lane] : 0.0);
      if (lane == 0) out[k] = x;
    }
  }
}

// Complex FP64 scalars of the solver steps (one thread).
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ bool cz(double2 a) { return a.x == 0.0 && a.y == 0.0; }
__device__ __forceinline__ bool cfinite(double2 a) { return isfinite(a.x) && isfinite(a.y); }
// BiCGSTAB's alpha = rho / (rt^H v) (t = rt^H v as re, im) with its breakdown
// test: the flag that ends the iteration (4 breakdown, 5 not finite), or -1
// and alpha in al.
__device__ __forceinline__ int alpha_step(double2 rho, const double (&t)[2], double2& al) {
  const double2 d = make_double2(t[0], t[1]);
  if (cz(d) || !cfinite(d)) return cfinite(d) ? 4 : 5;
  al = cdiv(rho, d);
  return -1;
}

}  // namespace vs
