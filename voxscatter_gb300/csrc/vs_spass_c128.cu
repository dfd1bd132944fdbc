// c128 instantiations of the two-level strided (y) pass.
#include "vs_spass.cuh"

namespace vs {
template bool strided_two_level<double, false>(const StridedArgs<double>&, int, int, cudaStream_t);
template bool strided_two_level<double, true>(const StridedArgs<double>&, int, int, cudaStream_t);
}  // namespace vs
