// c128 storage with double-float arithmetic: the two-level x and strided (y)
// passes of the FP64 matvec on the FP32 pipes (GB300 issues FP32 at several
// tens of times its FP64 rate).  Built for the embedding lengths 48..256 whose
// longer factor is at most 18, split over four translation units that compile
// in parallel (an unrolled double-float DFT costs seconds of compile time per
// kernel); other lengths keep the FP64 kernels.
#pragma once
#include "vs_xpass.cuh"

#define VS_DF_LIST_A(X) \
  X(6, 8) X(5, 10) X(6, 9) X(6, 10) X(8, 8) X(8, 9) X(5, 15) X(8, 10) X(9, 9) X(9, 10) X(8, 12) X(10, 10) X(9, 12)
#define VS_DF_LIST_B(X) \
  X(10, 12) X(8, 16) X(9, 15) X(12, 12) X(10, 15) X(10, 16) X(9, 18) X(12, 15) X(12, 16) X(12, 18) X(15, 15) X(16, 16)
#define VS_DF_LIST(X) VS_DF_LIST_A(X) VS_DF_LIST_B(X)

namespace vs {
bool x_two_level_df_a(const PipeArgs<double>& a, bool inverse, int mode, int nrhs, cudaStream_t st);
bool x_two_level_df_b(const PipeArgs<double>& a, bool inverse, int mode, int nrhs, cudaStream_t st);
bool strided_two_level_df_a(const StridedArgs<double>& a, bool inverse, int nplanes, int nrhs, cudaStream_t st);
bool strided_two_level_df_b(const StridedArgs<double>& a, bool inverse, int nplanes, int nrhs, cudaStream_t st);
}  // namespace vs

// body of one x-pass unit over LIST
#define VS_DF_X_UNIT(NAME, LIST)                                                                  \
  bool NAME(const PipeArgs<double>& a, bool inverse, int mode, int nrhs, cudaStream_t st) {       \
    switch (a.P) {                                                                                \
      LIST(VS_DF_X_CASE)                                                                          \
      default: return false;                                                                      \
    }                                                                                             \
  }
#define VS_DF_X_CASE(R1, R2)                                              \
  case R1 * R2:                                                           \
    if (inverse) launch_x2<double, R1, R2, true, dfc>(a, mode, nrhs, st); \
    else launch_x2<double, R1, R2, false, dfc>(a, mode, nrhs, st);        \
    return true;

// body of one strided-pass unit over LIST
#define VS_DF_S_UNIT(NAME, LIST)                                                                        \
  bool NAME(const StridedArgs<double>& a, bool inverse, int nplanes, int nrhs, cudaStream_t st) {       \
    switch (a.plan.n) {                                                                                 \
      LIST(VS_DF_S_CASE)                                                                                \
      default: return false;                                                                            \
    }                                                                                                   \
  }
#define VS_DF_S_CASE(R1, R2)                                                 \
  case R1 * R2:                                                              \
    if (inverse) launch_s2<double, R1, R2, true, dfc>(a, nplanes, nrhs, st); \
    else launch_s2<double, R1, R2, false, dfc>(a, nplanes, nrhs, st);        \
    return true;
