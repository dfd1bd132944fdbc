// Shared device/host helpers for libvoxscatter: complex arithmetic on
// float2/double2, status codes and launch checks.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <string>
#include <stdexcept>
#include <mutex>
#include <set>
#include <map>
#include <utility>
#include "../../include/voxscatter.h"

namespace vs {

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };
template <typename T> using cplx_t = typename Cplx<T>::type;

template <typename C> __host__ __device__ __forceinline__ C mk(double re, double im) {
  C c; c.x = (decltype(c.x))re; c.y = (decltype(c.y))im; return c;
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a*conj(b)
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__host__ __device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// a + b*c
__host__ __device__ __forceinline__ float2 cfma(float2 b, float2 c, float2 a) {
  return make_float2(fmaf(b.x, c.x, fmaf(-b.y, c.y, a.x)), fmaf(b.x, c.y, fmaf(b.y, c.x, a.y)));
}
__host__ __device__ __forceinline__ double2 cfma(double2 b, double2 c, double2 a) {
  return make_double2(fma(b.x, c.x, fma(-b.y, c.y, a.x)), fma(b.x, c.y, fma(b.y, c.x, a.y)));
}
template <typename C> __host__ __device__ __forceinline__ C czero() { C c; c.x = 0; c.y = 0; return c; }
template <typename C, typename R> __host__ __device__ __forceinline__ C make_c(R re, R im) {
  C c; c.x = re; c.y = im; return c;
}
template <typename D, typename S> __host__ __device__ __forceinline__ D ccast(S s) {
  D d; d.x = (decltype(d.x))s.x; d.y = (decltype(d.y))s.y; return d;
}

// Error carried from a failing CUDA call or argument check to the C ABI.
struct Error : std::runtime_error {
  int status;
  Error(int st, const std::string& m) : std::runtime_error(m), status(st) {}
};

#define VS_CUDA(call)                                                                 \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      throw ::vs::Error(e_ == cudaErrorMemoryAllocation ? VS_ERR_OOM : VS_ERR_CUDA,   \
                        std::string(#call) + ": " + cudaGetErrorString(e_));          \
    }                                                                                 \
  } while (0)

#define VS_LAUNCH_CHECK() VS_CUDA(cudaGetLastError())

#define VS_REQUIRE(cond, msg)                                    \
  do {                                                           \
    if (!(cond)) throw ::vs::Error(VS_ERR_ARG, msg);             \
  } while (0)

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// Raise a kernel's dynamic shared-memory limit once per process and device
// (not per launch, so that launches captured into CUDA graphs issue no
// attribute calls).  The limit is a property of the function shared by every
// host thread, so it is raised straight to the hardware maximum and never
// lowered: launches from concurrent threads with different tile sizes all fit.
inline void set_kernel_smem(const void* kernel, size_t bytes) {
  constexpr size_t kMax = 227 * 1024, kDefault = 48 * 1024;
  if (bytes > kMax)
    throw Error(VS_ERR_UNSUPPORTED, "kernel tile needs " + std::to_string(bytes) + " bytes of shared memory (> 227 KB)");
  int dev = 0;
  VS_CUDA(cudaGetDevice(&dev));
  static std::mutex mu;
  // per kernel and device: its static shared memory, and whether the
  // dynamic limit has been raised to what the static part leaves
  static std::map<std::pair<const void*, int>, std::pair<size_t, bool>> seen;
  std::lock_guard<std::mutex> lock(mu);
  auto it = seen.find({kernel, dev});
  if (it == seen.end()) {
    cudaFuncAttributes fa;
    VS_CUDA(cudaFuncGetAttributes(&fa, kernel));
    it = seen.emplace(std::make_pair(kernel, dev), std::make_pair((size_t)fa.sharedSizeBytes, false)).first;
  }
  const size_t stat = it->second.first;
  // without the attribute, static and dynamic shared memory together must
  // stay within the default 48 KB
  if (bytes + stat <= kDefault || it->second.second) {
    if (bytes + stat > kMax)
      throw Error(VS_ERR_UNSUPPORTED, "kernel tile needs " + std::to_string(bytes) + " bytes of shared memory (> " +
                                          std::to_string(kMax - stat) + " available)");
    return;
  }
  const size_t cap = kMax - stat;
  if (bytes > cap)
    throw Error(VS_ERR_UNSUPPORTED, "kernel tile needs " + std::to_string(bytes) + " bytes of shared memory (> " +
                                        std::to_string(cap) + " available)");
  VS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap));
  it->second.second = true;
}

}  // namespace vs
