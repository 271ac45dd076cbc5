// Adjoint of the window chain extract -> correlate -> find_peaks -> 3-point
// Gaussian fit -> vector (complex mode), d(u, v) / d(pixel) for both frames.
//
// The integer peak (px, py) is piecewise constant in the pixels; u and v
// depend on them only through the sub-pixel fit (image_utils.impl.h:77-101)
//   fx = (ln l - ln r) / (2 (ln l + ln r - 2 ln c)),   u = W/2 - px - fx
// of five plane values c, l, r (row py) and u_, d (column px).  A plane
// value of FFT::cross_correlate (fft.h:188-206) at swapped position (x, y)
// is the circular correlation at lag (dx, dy) = (x - W/2, y - W/2):
//   R(dx, dy) = sum_p a[p] b[p + (dx, dy)],
// so dR/da[p] = b[p + lag], dR/db[q] = a[q - lag].  The kernel recomputes
// the five values as direct sums (no plane is stored), forms the partial
// derivatives of the fit, and either accumulates the vector-Jacobian
// product of per-window cotangents (gu, gv) into image gradients, or the
// propagated standard deviation of u and v for independent pixel noise.
// One warp per window; lanes take the window's columns and walk its rows,
// so every load (and every gradient update) of a warp touches one row
// segment of the frame (coalesced) rather than 32 rows.
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "piv_kernels.h"

namespace opiv {
namespace {

template <typename PixT>
__device__ __forceinline__ float pix(const PixT* f, size_t pitch, int x, int y)
{
    return (float)__ldg(f + (size_t)y * pitch + x);
}

template <typename PixT>
__global__ void __launch_bounds__(128)
piv_adjoint_kernel(const PivParams p, int W, const int32_t* __restrict__ peaks,
                   const float* __restrict__ cot, float* grad_a, float* grad_b, size_t gpitch,
                   float var_a, float var_b, float* sigma)
{
    const int lane = threadIdx.x & 31;
    const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (w >= p.n_win) return;   // warp-uniform
    const int32_t code = peaks[w];
    if (code < 0) {             // fewer than two peaks: the vector is zero, no gradient
        if (sigma && lane == 0) {
            sigma[2 * w] = 0.f;
            sigma[2 * w + 1] = 0.f;
        }
        return;
    }
    const int px = (code & 0xFFFF) % W, py = (code & 0xFFFF) / W;
    const int gy = (int)(w / p.gnx);
    const int bx = p.gx0 + (int)(w - (int64_t)gy * p.gnx) * p.gdx, by = p.gy0 + gy * p.gdy;
    const PixT* fa = reinterpret_cast<const PixT*>(p.fa);
    const PixT* fb = reinterpret_cast<const PixT*>(p.fb);
    const size_t pitch = p.pitch / sizeof(PixT);
    const int m = W - 1;

    // lags of c, l, r, u, d
    const int lx[5] = { px - W / 2, px - 1 - W / 2, px + 1 - W / 2, px - W / 2, px - W / 2 };
    const int ly[5] = { py - W / 2, py - W / 2, py - W / 2, py - 1 - W / 2, py + 1 - W / 2 };

    // the five plane values: columns of the window split over the lanes
    float R[5] = { 0.f, 0.f, 0.f, 0.f, 0.f };
    for (int x = lane; x < W; x += 32)
        for (int y = 0; y < W; ++y) {
            const float av = pix(fa, pitch, bx + x, by + y);
#pragma unroll
            for (int v = 0; v < 5; ++v)
                R[v] = fmaf(av, pix(fb, pitch, bx + ((x + lx[v]) & m), by + ((y + ly[v]) & m)), R[v]);
        }
#pragma unroll
    for (int v = 0; v < 5; ++v)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) R[v] += __shfl_xor_sync(0xffffffffu, R[v], o);

    // partial derivatives of u = W/2 - px - fx and v = W/2 - py - fy
    const float c = R[0], l = R[1], r = R[2], u_ = R[3], d = R[4];
    float gx[5] = { 0.f, 0.f, 0.f, 0.f, 0.f }, gyv[5] = { 0.f, 0.f, 0.f, 0.f, 0.f };
    bool okx = c > 0.f && l > 0.f && r > 0.f, oky = c > 0.f && u_ > 0.f && d > 0.f;
    if (okx) {
        const float N = logf(l) - logf(r), D = 2.f * (logf(l) + logf(r) - 2.f * logf(c));
        okx = D != 0.f;
        if (okx) {
            const float D2 = D * D;
            gx[1] = -(D - 2.f * N) / (l * D2);   // du/dl = -dfx/dl
            gx[2] = (D + 2.f * N) / (r * D2);
            gx[0] = -4.f * N / (c * D2);
        }
    }
    if (oky) {
        const float N = logf(u_) - logf(d), D = 2.f * (logf(u_) + logf(d) - 2.f * logf(c));
        oky = D != 0.f;
        if (oky) {
            const float D2 = D * D;
            gyv[3] = -(D - 2.f * N) / (u_ * D2);
            gyv[4] = (D + 2.f * N) / (d * D2);
            gyv[0] = -4.f * N / (c * D2);
        }
    }
    const float cu = cot ? cot[2 * w] : 0.f, cv = cot ? cot[2 * w + 1] : 0.f;

    // per pixel: du/da[p] = sum_v gx[v] b[p + lag_v], du/db[q] = sum_v gx[v] a[q - lag_v]
    float su = 0.f, sv = 0.f;
    for (int x = lane; x < W; x += 32)
        for (int y = 0; y < W; ++y) {
            float dua = 0.f, dva = 0.f, dub = 0.f, dvb = 0.f;
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                if (gx[v] == 0.f && gyv[v] == 0.f) continue;
                const float bv = pix(fb, pitch, bx + ((x + lx[v]) & m), by + ((y + ly[v]) & m));
                const float av = pix(fa, pitch, bx + ((x - lx[v]) & m), by + ((y - ly[v]) & m));
                dua = fmaf(gx[v], bv, dua);
                dva = fmaf(gyv[v], bv, dva);
                dub = fmaf(gx[v], av, dub);
                dvb = fmaf(gyv[v], av, dvb);
            }
            su = fmaf(var_a * dua, dua, fmaf(var_b * dub, dub, su));
            sv = fmaf(var_a * dva, dva, fmaf(var_b * dvb, dvb, sv));
            if (cot) {
                atomicAdd(grad_a + (size_t)(by + y) * gpitch + bx + x, cu * dua + cv * dva);
                atomicAdd(grad_b + (size_t)(by + y) * gpitch + bx + x, cu * dub + cv * dvb);
            }
        }
    if (sigma) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            su += __shfl_xor_sync(0xffffffffu, su, o);
            sv += __shfl_xor_sync(0xffffffffu, sv, o);
        }
        if (lane == 0) {
            const float nan = __int_as_float(0x7fffffff);
            sigma[2 * w] = okx ? sqrtf(su) : nan;
            sigma[2 * w + 1] = oky ? sqrtf(sv) : nan;
        }
    }
}

}  // namespace

cudaError_t launch_piv_adjoint(const PivParams& p, int w, int dtype, const int32_t* peaks,
                               const float* cot, float* grad_a, float* grad_b, size_t gpitch,
                               float var_a, float var_b, float* sigma, cudaStream_t s)
{
    if (p.n_win <= 0) return cudaSuccess;
    const int warps = 4;
    const unsigned blocks = (unsigned)((p.n_win + warps - 1) / warps);
    switch (dtype) {
    case kU8:
        piv_adjoint_kernel<uint8_t><<<blocks, 32 * warps, 0, s>>>(p, w, peaks, cot, grad_a, grad_b,
                                                                  gpitch, var_a, var_b, sigma);
        break;
    case kU16:
        piv_adjoint_kernel<uint16_t><<<blocks, 32 * warps, 0, s>>>(p, w, peaks, cot, grad_a, grad_b,
                                                                   gpitch, var_a, var_b, sigma);
        break;
    case kF32:
        piv_adjoint_kernel<float><<<blocks, 32 * warps, 0, s>>>(p, w, peaks, cot, grad_a, grad_b,
                                                                gpitch, var_a, var_b, sigma);
        break;
    default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace opiv
