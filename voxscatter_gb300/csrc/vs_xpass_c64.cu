// c64 instantiations of the two-level x passes.
#include "vs_xpass.cuh"

namespace vs {
template bool x_two_level<float, false>(const PipeArgs<float>&, int, int, cudaStream_t);
template bool x_two_level<float, true>(const PipeArgs<float>&, int, int, cudaStream_t);

int x2_ctas(int P, int nlines) {
  switch (P) {
#define VS_X2_CTAS(R1, R2) \
  case R1 * R2: return (int)ceil_div(nlines, kX2Threads / R2);
    VS_S2_LIST(VS_X2_CTAS)
#undef VS_X2_CTAS
    default: return 0;
  }
}
}  // namespace vs
