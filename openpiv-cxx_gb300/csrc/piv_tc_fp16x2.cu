// Instantiations of the tensor-core kernel with FP16 operands, the data
// split into hi + lo and the constant matrices single (two MMAs per product).
#include "piv_tc_kernel.cuh"

namespace opiv {

cudaError_t launch_piv_tc_fp16x2(const PivParams& p, int dtype, int mode, int limit, const void* consts,
                                 cudaStream_t s)
{
    return tc::by_mode<true, true, false>(p, dtype, mode, limit, consts, s);
}

}  // namespace opiv
