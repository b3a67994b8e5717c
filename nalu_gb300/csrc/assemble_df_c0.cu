// Explicit instantiations of the double-float assembly kernel (see assemble_df.cuh).
#include "assemble_df.cuh"

namespace nalu_gb300 {
template void launch_df_variant<1, 0, false, false>(nalu_ctx*, AsmArgsDF, int);
template void launch_df_variant<1, 0, false, true>(nalu_ctx*, AsmArgsDF, int);
}  // namespace nalu_gb300
