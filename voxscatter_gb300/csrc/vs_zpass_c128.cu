// c128 instantiations of the two-level z pass.
#include "vs_zpass.cuh"

namespace vs {
template bool z_pass_two_level<double>(const PipeArgs<double>&, bool, bool, int, cudaStream_t);
}  // namespace vs
