// c64 instantiations of the two-level x passes.
#include "vs_xpass.cuh"

namespace vs {
template bool x_two_level<float, false>(const PipeArgs<float>&, int, int, cudaStream_t);
template bool x_two_level<float, true>(const PipeArgs<float>&, int, int, cudaStream_t);
}  // namespace vs
