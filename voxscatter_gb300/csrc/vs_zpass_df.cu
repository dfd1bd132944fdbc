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
