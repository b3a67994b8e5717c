// Explicit instantiations of the ip-per-thread double-float assembly kernel
// (assemble_ip.cuh), 16 elements per block; split so nvcc compiles in parallel.
#include "assemble_ip.cuh"

namespace nalu_gb300 {
template void launch_ip_variant<16, 0, 0, false, false>(nalu_ctx*, AsmArgsDF, int);
template void launch_ip_variant<16, 0, 0, true, false>(nalu_ctx*, AsmArgsDF, int);
}  // namespace nalu_gb300
