// c64 instantiations of the two-level z pass.
#include "vs_zpass.cuh"

namespace vs {
template bool z_pass_two_level<float>(const PipeArgs<float>&, bool, bool, int, cudaStream_t);

int z_pass_length(int min_len) {
  for (const ZSplit& s : kZSplits)
    if (s.R >= min_len) return s.R;
  return smooth_size(min_len);
}
}  // namespace vs
