// Host side of the tensor-core kernels (piv_tc_kernel.cuh for 32 px
// windows, piv_tc16_kernel.cuh, piv_tc48_kernel.cuh and piv_tc64_kernel.cuh
// for 16, 48 and 64 px grids they take, piv_tcg_kernel.cuh for the other
// 16 and 64 px grids): the constant matrices in BF16 and FP16 (hi and lo
// parts, canonical operand layout) and the dispatch to the instantiation
// units.
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
cudaError_t launch_piv_tc_fp16x2(const PivParams& p, int dtype, int mode, int limit, const void* consts,
                                 cudaStream_t s);
bool tc16_takes(const PivParams& p);
bool tc48_takes(const PivParams& p);
bool tc64_takes(const PivParams& p);
cudaError_t launch_piv_tc48_bf16(const PivParams& p, int dtype, int mode, int limit, bool split,
                                 const void* consts, cudaStream_t s);
cudaError_t launch_piv_tc48_fp16(const PivParams& p, int dtype, int mode, int limit, int passes,
                                 const void* consts, cudaStream_t s);
cudaError_t launch_piv_tc64_bf16(const PivParams& p, int dtype, int mode, int limit, bool split,
                                 const void* consts, cudaStream_t s);
cudaError_t launch_piv_tc64_fp16(const PivParams& p, int dtype, int mode, int limit, int passes,
                                 const void* consts, cudaStream_t s);
cudaError_t launch_piv_tc16_bf16(const PivParams& p, int dtype, int mode, int limit, bool split,
                                 const void* consts, cudaStream_t s);
cudaError_t launch_piv_tc16_fp16(const PivParams& p, int dtype, int mode, int limit, int passes,
                                 const void* consts, cudaStream_t s);
cudaError_t launch_piv_tcg_w16(const PivParams& p, int dtype, int mode, int limit, int passes, bool fp16,
                               const void* consts, cudaStream_t s);
cudaError_t launch_piv_tcg_w64(const PivParams& p, int dtype, int mode, int limit, int passes, bool fp16,
                               const void* consts, cudaStream_t s);

namespace tc {

// bytes of the hi and lo parts of the five W x W 16-bit matrices
constexpr int set_bytes(int w) { return kTcNumMat * 2 * w * w * 2; }

// byte offset of element (n, k) in a W x W K-major matrix
constexpr int kmaj(int w, int n, int k)
{
    return ((n >> 3) * (w / 8) + (k >> 3)) * 128 + (n & 7) * 16 + (k & 7) * 2;
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

bool tc_supports(int w, int dtype)
{
    return (w == 16 || w == 32 || w == 48 || w == 64) && (dtype == kU8 || dtype == kU16);
}

size_t tc_constant_bytes(int w) { return 2 * (size_t)tc::set_bytes(w); }

// Two sets: BF16, then FP16 (the FP16 stage-1 matrix scaled by 2^-9).
// Matrix rows n are the products' output index, columns k the summed one:
//   G1  n < W/2: cos(2 pi n x / W); n = W/2: (-1)^x; n > W/2: sin(2 pi (n - W/2) x / W)
//   C, S, -S  cos / sin (2 pi n k / W)
//   C4  n = x' (the swapped column, x = (x' + W/2) mod W), k = (part, k_x):
//       part 0: 1 (k_x = 0) or 2 cos(2 pi k_x x / W); part 1: (-1)^x (k_x = 0)
//       or -2 sin(2 pi k_x x / W)
void tc_constants(int w, unsigned char* out)
{
    using namespace tc;
    const double pi = 3.14159265358979323846;
    const int h = w / 2, mat = w * w * 2, sb = set_bytes(w);
    for (int set = 0; set < 2; ++set) {
        unsigned char* o = out + set * sb;
        auto put = [&](int m, int n, int k, double v) {
            uint16_t hi, lo;
            if (set == 0) {
                hi = bf16_bits((float)v);
                lo = bf16_bits((float)(v - (double)bf16_value(hi)));
            } else {
                hi = fp16_bits((float)v);
                lo = fp16_bits((float)(v - (double)fp16_value(hi)));
            }
            std::memcpy(o + m * mat + kmaj(w, n, k), &hi, 2);
            std::memcpy(o + (kTcNumMat + m) * mat + kmaj(w, n, k), &lo, 2);
        };
        const double gscale = set == 0 ? 1.0 : 1.0 / 512.0;
        for (int n = 0; n < w; ++n)
            for (int k = 0; k < w; ++k) {
                double g;
                if (n < h) g = std::cos(2 * pi * n * k / w);
                else if (n == h) g = (k & 1) ? -1.0 : 1.0;
                else g = std::sin(2 * pi * (n - h) * k / w);
                put(kTcG1, n, k, g * gscale);
                const double c = std::cos(2 * pi * n * k / w), s = std::sin(2 * pi * n * k / w);
                put(kTcC, n, k, c);
                put(kTcS, n, k, s);
                put(kTcNS, n, k, -s);
                const int x = (n + h) % w;
                const int part = k / h, kx = k % h;
                double v;
                if (part == 0) v = kx == 0 ? 1.0 : 2.0 * std::cos(2 * pi * kx * x / w);
                else v = kx == 0 ? ((x & 1) ? -1.0 : 1.0) : -2.0 * std::sin(2 * pi * kx * x / w);
                put(kTcC4, n, k, v);
            }
    }
}

cudaError_t launch_piv_tc(const PivParams& p, int w, int dtype, int mode, int limit, int passes,
                          bool fp16, const void* consts, cudaStream_t s)
{
    const unsigned char* c = static_cast<const unsigned char*>(consts);
    const unsigned char* set = c + (fp16 ? tc::set_bytes(w) : 0);
    if (passes == 2 && !fp16) return cudaErrorInvalidValue;   // data split: FP16 operands
    if (passes == 2 && w == 32) return launch_piv_tc_fp16x2(p, dtype, mode, limit, set, s);
    const bool split = passes == 3;
    switch (w) {
    case 16:   // vertical tiles where the grid allows them, else the generic kernel
        if (tc16_takes(p))
            return fp16 ? launch_piv_tc16_fp16(p, dtype, mode, limit, passes, set, s)
                        : launch_piv_tc16_bf16(p, dtype, mode, limit, split, set, s);
        return launch_piv_tcg_w16(p, dtype, mode, limit, passes, fp16, set, s);
    case 32: return fp16 ? launch_piv_tc_fp16(p, dtype, mode, limit, split, set, s)
                         : launch_piv_tc_bf16(p, dtype, mode, limit, split, set, s);
    case 48:   // every regular grid: one window per tile
        if (!tc48_takes(p)) return cudaErrorNotSupported;
        return fp16 ? launch_piv_tc48_fp16(p, dtype, mode, limit, passes, set, s)
                    : launch_piv_tc48_bf16(p, dtype, mode, limit, split, set, s);
    case 64:   // grids at x multiples of 8: one window per tile
        if (tc64_takes(p))
            return fp16 ? launch_piv_tc64_fp16(p, dtype, mode, limit, passes, set, s)
                        : launch_piv_tc64_bf16(p, dtype, mode, limit, split, set, s);
        return launch_piv_tcg_w64(p, dtype, mode, limit, passes, fp16, set, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace opiv
