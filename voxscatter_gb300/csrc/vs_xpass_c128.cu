// c128 instantiations of the two-level x passes.
#include "vs_xpass.cuh"

namespace vs {
template bool x_two_level<double, false>(const PipeArgs<double>&, int, int, cudaStream_t);
template bool x_two_level<double, true>(const PipeArgs<double>&, int, int, cudaStream_t);
}  // namespace vs
