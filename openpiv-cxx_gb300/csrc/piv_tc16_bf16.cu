// Instantiations of the 16 px vertical-tile tensor-core kernel with BF16
// operands (split and plain), and the test of its applicability.
#include "piv_tc16_kernel.cuh"

namespace opiv {

bool tc16_takes(const PivParams& p) { return tc16::applicable(p); }

cudaError_t launch_piv_tc16_bf16(const PivParams& p, int dtype, int mode, int limit, bool split,
                                 const void* consts, cudaStream_t s)
{
    return split ? tc16::by_mode<false, true, true>(p, dtype, mode, limit, consts, s)
                 : tc16::by_mode<false, false, false>(p, dtype, mode, limit, consts, s);
}

}  // namespace opiv
