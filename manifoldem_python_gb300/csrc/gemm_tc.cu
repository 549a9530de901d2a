// Split-BF16 tcgen05 form of the D contraction (placeholder until the tensor-core kernel lands).
#include "mem_internal.cuh"

namespace mem {
namespace kern {
int gemm_split_bf16(const mem_plan& P, const void* feat_hi, const void* feat_lo,
                    const double* pair_norm, const uint32_t* pd_max, const Tile* tiles,
                    const PdDev* pds, double* D, uint32_t* status, cudaStream_t s) {
    return MEM_ERR_UNSUPPORTED;
}
}  // namespace kern
}  // namespace mem
