// c128 storage with double-float arithmetic: the two-level z pass (the
// FP64-arithmetic-bound piece of the FP64 matvec) on the FP32 pipes.  Built
// for the z lengths up to 64 (the unrolled double-float DFTs of the longer
// lengths cost minutes of compile time); other lengths keep the FP64 kernel.
#include "vs_zpass.cuh"

namespace vs {
bool z_pass_two_level_df(const PipeArgs<double>& a, bool sym, int nrhs, cudaStream_t st) {
  const int s = sym ? 1 : 0;
  switch (a.R) {
#define VS_Z2DF(R1, R2)                                               \
  case R1 * R2: launch_z2<double, R1, R2, dfc>(a, s, true, nrhs, st); \
    return true;
    VS_Z2DF(2, 2) VS_Z2DF(2, 3) VS_Z2DF(2, 4) VS_Z2DF(3, 3) VS_Z2DF(2, 5) VS_Z2DF(3, 4) VS_Z2DF(3, 5)
    VS_Z2DF(4, 4) VS_Z2DF(3, 6) VS_Z2DF(4, 5) VS_Z2DF(4, 6) VS_Z2DF(3, 9) VS_Z2DF(5, 6) VS_Z2DF(4, 8)
    VS_Z2DF(6, 6) VS_Z2DF(5, 8) VS_Z2DF(5, 9) VS_Z2DF(6, 8) VS_Z2DF(6, 9) VS_Z2DF(8, 8)
#undef VS_Z2DF
    default: return false;
  }
}
}  // namespace vs

// ---- double-float x and strided passes (lengths in vs_df_passes.cuh) ----
#include "vs_df_passes.cuh"

namespace vs {
bool x_df_available(int P) {
  switch (P) {
#define VS_DFA(R1, R2) case R1 * R2:
    VS_DF_LIST(VS_DFA)
#undef VS_DFA
    return true;
    default: return false;
  }
}
bool strided_df_available(int n) { return x_df_available(n); }
bool x_two_level_df(const PipeArgs<double>& a, bool inverse, int mode, int nrhs, cudaStream_t st) {
  return x_two_level_df_a(a, inverse, mode, nrhs, st) || x_two_level_df_b(a, inverse, mode, nrhs, st);
}
bool strided_two_level_df(const StridedArgs<double>& a, bool inverse, int nplanes, int nrhs, cudaStream_t st) {
  return strided_two_level_df_a(a, inverse, nplanes, nrhs, st) ||
         strided_two_level_df_b(a, inverse, nplanes, nrhs, st);
}
}  // namespace vs
