// c64 instantiations of the two-level strided (y) pass.
#include "vs_spass.cuh"

namespace vs {
template bool strided_two_level<float, false>(const StridedArgs<float>&, int, int, cudaStream_t);
template bool strided_two_level<float, true>(const StridedArgs<float>&, int, int, cudaStream_t);
}  // namespace vs
