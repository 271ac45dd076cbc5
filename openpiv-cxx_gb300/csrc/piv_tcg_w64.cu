// Instantiations of the generic tensor-core kernel for 64 x 64 windows.
#include "piv_tcg_kernel.cuh"

namespace opiv {

cudaError_t launch_piv_tcg_w64(const PivParams& p, int dtype, int mode, int limit, int passes, bool fp16,
                               const void* consts, cudaStream_t s)
{
    return tcg::launch_w<64>(p, dtype, mode, limit, passes, fp16, consts, s);
}

}  // namespace opiv
