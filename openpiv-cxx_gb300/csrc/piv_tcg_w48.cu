// Instantiations of the generic tensor-core kernel for 48 x 48 windows.
#include "piv_tcg_kernel.cuh"

namespace opiv {

cudaError_t launch_piv_tcg_w48(const PivParams& p, int dtype, int mode, int limit, int passes, bool fp16,
                               const void* consts, cudaStream_t s)
{
    return tcg::launch_w<48>(p, dtype, mode, limit, passes, fp16, consts, s);
}

}  // namespace opiv
