// Instantiations of the 48 px one-window-per-tile tensor-core kernel with
// FP16 operands: 3 MMAs per product (data and constants split), 2 (data
// split) or 1.
#include "piv_tc48_kernel.cuh"

namespace opiv {

cudaError_t launch_piv_tc48_fp16(const PivParams& p, int dtype, int mode, int limit, int passes,
                                 const void* consts, cudaStream_t s)
{
    if (passes == 3) return tc48::by_mode<true, true, true>(p, dtype, mode, limit, consts, s);
    if (passes == 2) return tc48::by_mode<true, true, false>(p, dtype, mode, limit, consts, s);
    return tc48::by_mode<true, false, false>(p, dtype, mode, limit, consts, s);
}

}  // namespace opiv
