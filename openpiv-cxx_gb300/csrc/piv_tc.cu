// Host side of the tensor-core kernel (piv_tc_kernel.cuh): the constant
// matrices in BF16 and FP16 (hi and lo parts, canonical operand layout) and
// the dispatch to the two instantiation units.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "piv_kernels.h"

namespace opiv {

cudaError_t launch_piv_tc_bf16(const PivParams& p, int dtype, int mode, int limit, bool split,
                               const void* consts, cudaStream_t s);
cudaError_t launch_piv_tc_fp16(const PivParams& p, int dtype, int mode, int limit, bool split,
                               const void* consts, cudaStream_t s);

namespace tc {

constexpr int kMat = 2048;   // one 32 x 32 16-bit matrix
constexpr int kSetBytes = kTcNumMat * 2 * kMat;

// byte offset of element (n, k) in a 32 x 32 K-major matrix
constexpr int kmaj32(int n, int k)
{
    return ((n >> 3) * 4 + (k >> 3)) * 128 + (n & 7) * 16 + (k & 7) * 2;
}

// BF16: round to nearest even (finite inputs)
uint16_t bf16_bits(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    const uint32_t r = u + 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(r >> 16);
}

float bf16_value(uint16_t h)
{
    const uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// FP16 (IEEE binary16): round to nearest even, subnormals kept, |f| < 65504
uint16_t fp16_bits(float f)
{
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const int e8 = (int)((x >> 23) & 0xffu);
    uint32_t mant = x & 0x7fffffu;
    if (e8 == 0) return (uint16_t)sign;
    const int e = e8 - 127 + 15;
    if (e >= 31) return (uint16_t)(sign | 0x7c00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        mant |= 0x800000u;
        const int shift = 14 - e;
        uint32_t h = mant >> shift;
        const uint32_t rem = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    uint32_t h = ((uint32_t)e << 10) | (mant >> 13);
    const uint32_t rem = mant & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}

float fp16_value(uint16_t h)
{
    const int e = (h >> 10) & 0x1f;
    const int m = h & 0x3ff;
    const float v = e == 0 ? std::ldexp((float)m, -24) : std::ldexp((float)(1024 + m), e - 25);
    return (h & 0x8000u) ? -v : v;
}

}  // namespace tc

bool tc_supports(int w, int dtype) { return w == 32 && (dtype == kU8 || dtype == kU16); }

size_t tc_constant_bytes() { return 2 * (size_t)tc::kSetBytes; }

// Two sets: BF16, then FP16 (the FP16 stage-1 matrix scaled by 2^-9).
void tc_constants(unsigned char* out)
{
    using namespace tc;
    const double pi = 3.14159265358979323846;
    for (int set = 0; set < 2; ++set) {
        unsigned char* o = out + set * kSetBytes;
        auto put = [&](int m, int n, int k, double v) {
            uint16_t hi, lo;
            if (set == 0) {
                hi = bf16_bits((float)v);
                lo = bf16_bits((float)(v - (double)bf16_value(hi)));
            } else {
                hi = fp16_bits((float)v);
                lo = fp16_bits((float)(v - (double)fp16_value(hi)));
            }
            std::memcpy(o + m * kMat + kmaj32(n, k), &hi, 2);
            std::memcpy(o + (kTcNumMat + m) * kMat + kmaj32(n, k), &lo, 2);
        };
        const double gscale = set == 0 ? 1.0 : 1.0 / 512.0;
        for (int n = 0; n < 32; ++n)
            for (int k = 0; k < 32; ++k) {
                // stage 1, B[k = x][n = coefficient]
                double g;
                if (n < 16) g = std::cos(2 * pi * n * k / 32.0);
                else if (n == 16) g = (k & 1) ? -1.0 : 1.0;
                else g = std::sin(2 * pi * (n - 16) * k / 32.0);
                put(kTcG1, n, k, g * gscale);
                const double c = std::cos(2 * pi * n * k / 32.0), s = std::sin(2 * pi * n * k / 32.0);
                put(kTcC, n, k, c);
                put(kTcS, n, k, s);
                put(kTcNS, n, k, -s);
                // stage 4, B[k = (part, k_x)][n = x'], x = (x' + 16) mod 32
                const int x = (n + 16) & 31;
                const int part = k >> 4, kx = k & 15;
                double v;
                if (part == 0) v = kx == 0 ? 1.0 : 2.0 * std::cos(2 * pi * kx * x / 32.0);
                else v = kx == 0 ? ((x & 1) ? -1.0 : 1.0) : -2.0 * std::sin(2 * pi * kx * x / 32.0);
                put(kTcC4, n, k, v);
            }
    }
}

cudaError_t launch_piv_tc(const PivParams& p, int dtype, int mode, int limit, bool split, bool fp16,
                          const void* consts, cudaStream_t s)
{
    const unsigned char* c = static_cast<const unsigned char*>(consts);
    return fp16 ? launch_piv_tc_fp16(p, dtype, mode, limit, split, c + tc::kSetBytes, s)
                : launch_piv_tc_bf16(p, dtype, mode, limit, split, c, s);
}

}  // namespace opiv
