// Instantiations of the 48 px one-window-per-tile tensor-core kernel with
// BF16 operands (split or plain), and the test of its applicability; the
// FP16 instantiations are in piv_tc48_fp16.cu.
#include "piv_tc48_kernel.cuh"

namespace opiv {

bool tc48_takes(const PivParams& p) { return tc48::applicable(p); }

cudaError_t launch_piv_tc48_bf16(const PivParams& p, int dtype, int mode, int limit, bool split,
                                 const void* consts, cudaStream_t s)
{
    return split ? tc48::by_mode<false, true, true>(p, dtype, mode, limit, consts, s)
                 : tc48::by_mode<false, false, false>(p, dtype, mode, limit, consts, s);
}

}  // namespace opiv
