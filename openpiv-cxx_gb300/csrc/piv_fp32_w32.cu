// piv_fp32_w32.cu -- instantiation of the fused FP32 kernel for 32x32 windows.
#include "piv_fp32.cuh"

namespace opiv {

cudaError_t launch_piv_fp32_w32(const PivParams& p, int dtype, int mode, int limit, bool planes,
                                cudaStream_t s)
{
    return fp32::launch_w<32>(p, dtype, mode, limit, planes, s);
}

cudaError_t queue_piv_fp32_w32(const PivQueue& q, int dtype, int mode, int limit, bool vec, int blocks,
                               int* max_ctas, cudaStream_t s)
{
    return fp32::queue_w<32>(q, dtype, mode, limit, vec, blocks, max_ctas, s);
}

}  // namespace opiv
