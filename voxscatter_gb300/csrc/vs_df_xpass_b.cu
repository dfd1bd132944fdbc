// Double-float two-level x passes on FP64 data, lengths of VS_DF_LIST_B.
#include "vs_df_passes.cuh"

namespace vs {
VS_DF_X_UNIT(x_two_level_df_b, VS_DF_LIST_B)
}  // namespace vs
