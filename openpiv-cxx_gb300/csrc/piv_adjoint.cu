// Adjoint of the window chain extract -> correlate -> find_peaks -> 3-point
// Gaussian fit -> vector, d(u, v) / d(pixel) for both frames: complex mode
// below, REAL mode further down.
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

// ---- REAL mode (FFT::cross_correlate_real, fft.h:208-227) ----------------
// The reference's two-for-one unpack leaves spectrum column k_x = 0 and rows
// k_y = 0, H/2 at zero (fft.h:163-183), so its plane is IFFT(M B conj A)
// with M the indicator of the other bins.  M is a projection that commutes
// with circular shifts, so M B conj A = (M B) conj (M A) and the plane is the
// plain circular correlation of the projected windows a_c = P a, b_c = P b,
// where P removes each row's mean (k_x = 0) and then, per column, the mean
// and the (-1)^y-weighted mean (k_y = 0, H/2).  Since a shifted b_c already
// lies in P's range, d plane(lag) / da[p] = b_c[p + lag] and
// d plane(lag) / db[q] = a_c[q - lag]: the complex-mode formulas on the
// projected windows.  One warp per window; the projected windows live in
// shared memory (rows padded by one float against bank conflicts).
template <typename PixT>
__device__ void project_window(const PixT* f, size_t pitch, int bx, int by, int W, float* X)
{
    const int lane = threadIdx.x & 31, Wp = W + 1;
    for (int y = 0; y < W; ++y)
        for (int x = lane; x < W; x += 32) X[y * Wp + x] = pix(f, pitch, bx + x, by + y);
    __syncwarp();
    // row means (k_x = 0): lane y sums row y
    for (int y = lane; y < W; y += 32) {
        float m = 0.f;
        for (int x = 0; x < W; ++x) m += X[y * Wp + x];
        X[y * Wp + W] = m / (float)W;   // the pad column holds the row mean
    }
    __syncwarp();
    for (int y = 0; y < W; ++y) {
        const float m = X[y * Wp + W];
        for (int x = lane; x < W; x += 32) X[y * Wp + x] -= m;
    }
    __syncwarp();
    // per column: the mean (k_y = 0) and the alternating mean (k_y = H/2)
    for (int x = lane; x < W; x += 32) {
        float s = 0.f, t = 0.f;
        for (int y = 0; y < W; ++y) {
            const float v = X[y * Wp + x];
            s += v;
            t += (y & 1) ? -v : v;
        }
        s /= (float)W;
        t /= (float)W;
        for (int y = 0; y < W; ++y) X[y * Wp + x] -= (y & 1) ? s - t : s + t;
    }
    __syncwarp();
}

template <typename PixT>
__global__ void __launch_bounds__(128)
piv_adjoint_real_kernel(const PivParams p, int W, const int32_t* __restrict__ peaks,
                        const float* __restrict__ cot, float* grad_a, float* grad_b, size_t gpitch,
                        float var_a, float var_b, float* sigma)
{
    extern __shared__ float adj_sm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    if (w >= p.n_win) return;   // warp-uniform
    const int32_t code = peaks[w];
    if (code < 0) {
        if (sigma && lane == 0) {
            sigma[2 * w] = 0.f;
            sigma[2 * w + 1] = 0.f;
        }
        return;
    }
    const int Wp = W + 1;
    float* A = adj_sm + (size_t)wib * 2 * W * Wp;
    float* B = A + W * Wp;
    const int px = (code & 0xFFFF) % W, py = (code & 0xFFFF) / W;
    const int gy = (int)(w / p.gnx);
    const int bx = p.gx0 + (int)(w - (int64_t)gy * p.gnx) * p.gdx, by = p.gy0 + gy * p.gdy;
    const size_t pitch = p.pitch / sizeof(PixT);
    project_window(reinterpret_cast<const PixT*>(p.fa), pitch, bx, by, W, A);
    project_window(reinterpret_cast<const PixT*>(p.fb), pitch, bx, by, W, B);
    const int m = W - 1;
    const int lx[5] = { px - W / 2, px - 1 - W / 2, px + 1 - W / 2, px - W / 2, px - W / 2 };
    const int ly[5] = { py - W / 2, py - W / 2, py - W / 2, py - 1 - W / 2, py + 1 - W / 2 };

    float R[5] = { 0.f, 0.f, 0.f, 0.f, 0.f };
    for (int x = lane; x < W; x += 32)
        for (int y = 0; y < W; ++y) {
            const float av = A[y * Wp + x];
#pragma unroll
            for (int v = 0; v < 5; ++v)
                R[v] = fmaf(av, B[((y + ly[v]) & m) * Wp + ((x + lx[v]) & m)], R[v]);
        }
#pragma unroll
    for (int v = 0; v < 5; ++v)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) R[v] += __shfl_xor_sync(0xffffffffu, R[v], o);

    const float c = R[0], l = R[1], r = R[2], u_ = R[3], d = R[4];
    float gx[5] = { 0.f, 0.f, 0.f, 0.f, 0.f }, gyv[5] = { 0.f, 0.f, 0.f, 0.f, 0.f };
    bool okx = c > 0.f && l > 0.f && r > 0.f, oky = c > 0.f && u_ > 0.f && d > 0.f;
    if (okx) {
        const float N = logf(l) - logf(r), D = 2.f * (logf(l) + logf(r) - 2.f * logf(c));
        okx = D != 0.f;
        if (okx) {
            const float D2 = D * D;
            gx[1] = -(D - 2.f * N) / (l * D2);
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
    float su = 0.f, sv = 0.f;
    for (int x = lane; x < W; x += 32)
        for (int y = 0; y < W; ++y) {
            float dua = 0.f, dva = 0.f, dub = 0.f, dvb = 0.f;
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                if (gx[v] == 0.f && gyv[v] == 0.f) continue;
                const float bv = B[((y + ly[v]) & m) * Wp + ((x + lx[v]) & m)];
                const float av = A[((y - ly[v]) & m) * Wp + ((x - lx[v]) & m)];
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

template <typename PixT>
cudaError_t launch_real(const PivParams& p, int w, const int32_t* peaks, const float* cot, float* grad_a,
                        float* grad_b, size_t gpitch, float var_a, float var_b, float* sigma, cudaStream_t s)
{
    // warps per CTA so that the projected windows (2 W (W + 1) floats per
    // warp) stay within the default 48 KB of shared memory
    const size_t per_warp = sizeof(float) * 2 * (size_t)w * (w + 1);
    int warps = (int)(49152 / per_warp);
    warps = warps < 1 ? 1 : (warps > 4 ? 4 : warps);
    const unsigned blocks = (unsigned)((p.n_win + warps - 1) / warps);
    piv_adjoint_real_kernel<PixT><<<blocks, 32 * warps, per_warp * warps, s>>>(p, w, peaks, cot, grad_a, grad_b,
                                                                             gpitch, var_a, var_b, sigma);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_piv_adjoint(const PivParams& p, int w, int dtype, int mode, const int32_t* peaks,
                               const float* cot, float* grad_a, float* grad_b, size_t gpitch,
                               float var_a, float var_b, float* sigma, cudaStream_t s)
{
    if (p.n_win <= 0) return cudaSuccess;
    if (mode == kModeReal) {
        if (w > 64) return cudaErrorInvalidValue;
        switch (dtype) {
        case kU8: return launch_real<uint8_t>(p, w, peaks, cot, grad_a, grad_b, gpitch, var_a, var_b, sigma, s);
        case kU16: return launch_real<uint16_t>(p, w, peaks, cot, grad_a, grad_b, gpitch, var_a, var_b, sigma, s);
        case kF32: return launch_real<float>(p, w, peaks, cot, grad_a, grad_b, gpitch, var_a, var_b, sigma, s);
        default: return cudaErrorInvalidValue;
        }
    }
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
