// Instantiations of the tensor-core kernel with BF16 operands.
#include "piv_tc_kernel.cuh"

namespace opiv {

cudaError_t launch_piv_tc_bf16(const PivParams& p, int dtype, int mode, int limit, bool split,
                          const void* consts, cudaStream_t s)
{
    return split ? tc::by_mode<false, true>(p, dtype, mode, limit, consts, s)
                 : tc::by_mode<false, false>(p, dtype, mode, limit, consts, s);
}

}  // namespace opiv
