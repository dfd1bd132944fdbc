// Double-float two-level strided (y) passes on FP64 data, lengths of VS_DF_LIST_A.
#include "vs_df_passes.cuh"

namespace vs {
VS_DF_S_UNIT(strided_two_level_df_a, VS_DF_LIST_A)
}  // namespace vs
