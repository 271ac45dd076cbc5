// Instantiations of the tensor-core kernel with FP16 operands.
#include "piv_tc_kernel.cuh"

namespace opiv {

cudaError_t launch_piv_tc_fp16(const PivParams& p, int dtype, int mode, int limit, bool split,
                          const void* consts, cudaStream_t s)
{
    return split ? tc::by_mode<true, true>(p, dtype, mode, limit, consts, s)
                 : tc::by_mode<true, false>(p, dtype, mode, limit, consts, s);
}

}  // namespace opiv
