// piv_fp32_w16.cu -- instantiation of the fused FP32 kernel for 16x16 windows.
#include "piv_fp32.cuh"

namespace opiv {

cudaError_t launch_piv_fp32_w16(const PivParams& p, int dtype, int mode, int limit, bool planes,
                                cudaStream_t s)
{
    return fp32::launch_w<16>(p, dtype, mode, limit, planes, s);
}

cudaError_t queue_piv_fp32_w16(const PivQueue& q, int dtype, int mode, int limit, bool vec, int blocks,
                               int* max_ctas, cudaStream_t s)
{
    return fp32::queue_w<16>(q, dtype, mode, limit, vec, blocks, max_ctas, s);
}

}  // namespace opiv
