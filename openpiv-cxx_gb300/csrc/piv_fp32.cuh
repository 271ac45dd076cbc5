// piv_fp32.cuh -- fused FP32 PIV window kernel for sm_103a (template; the
// piv_fp32_w*.cu files instantiate it per window size).
//
// One warp processes a task of 2*NG interrogation windows (NG = 32/W lane
// groups of W lanes; W = 32 -> one group, W = 16 -> two groups).  Per window:
//
//   extract (core::extract, image_utils.impl.h:392-419), widen to float and
//   subtract the window mean; z = a + i*b;
//   2-D FFT of z in registers: column FFT (lane = column), transpose through
//   a swizzled shared-memory tile, row FFT;
//   two-for-one unpack A = (Z[k] + conj Z[-k])/2, B = (Z[k] - conj Z[-k])/2i
//   via a lane shuffle, product P = B * conj(A) (fft.h:188-227), with the
//   reference's zeroed spectrum row 0, row W/2 and column 0 in REAL mode;
//   the products of two windows are packed as Q = P1 + i*P2 (both are
//   Hermitian, so one complex inverse gives both real planes);
//   inverse row FFT, transpose, inverse column FFT -> both planes;
//   quadrant swap as an index remap (swap_quadrants, impl:367-386);
//   find_peaks(plane, 2, 1) (impl:42-74) as a warp scan + top-2 reduction
//   (ties to the lowest row-major index, the order the reference's sort
//   keeps among equal values);
//   fit_simple_gaussian (impl:77-101) and the vector of main.cpp:220-236.
//
// Mean subtraction changes only the DC bin; the kernel zeroes that bin and
// adds the exact pedestal (sum a)(sum b) back where values are used, which
// is the reference's raw (unsubtracted) plane.  Planes are computed 4x
// scaled (the 1/2 factors of the unpack are dropped); ratios are unaffected
// and the pedestal is scaled to match.
//
// Every window gets a certification test: decisions (local-max tests, the
// order of the two peaks, signs entering log and sn, the conditioning of
// the Gaussian fit) whose margin is below an error bound of the FP32 plane
// are flagged; flagged windows are re-evaluated by the exact double
// precision kernel (piv_exact.cu), which overwrites their results.

#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "fft_reg.cuh"
#include "piv_kernels.h"

namespace opiv {
namespace fp32 {

constexpr int kWarps = 4;   // warps per CTA
// Certification margins: a window is decided by this kernel only if the
// error bound of its sub-pixel fit stays below kFitTol pixels and the
// relative error bound of its sn below kSnTol * (1 + sn).  The parity
// tolerances are 1e-4 px and 1e-5 * (1 + sn): sn = p0 / p1 is a ratio of
// plane values, and plane values are specified to 1e-5 of the plane peak p0,
// which bounds the relative error of p1 by 1e-5 * p0 / p1 = 1e-5 * sn.
constexpr float kFitTol = 3e-5f;
constexpr float kSnTol = 3e-6f;
#define kNegInf (-__int_as_float(0x7f800000))

// Pixel types: 8/16-bit integers are summed exactly (column sums stay below
// 2^24, window sums in int); float frames are summed in float; double input
// (the per-window batch API) is summed in double.
template <typename PixT> struct px_traits {
    using acc = float;
    static constexpr bool integer = true;
};
template <> struct px_traits<float> {
    using acc = float;
    static constexpr bool integer = false;
};
template <> struct px_traits<double> {
    using acc = double;
    static constexpr bool integer = false;
};

__device__ __forceinline__ void window_origin(const PivParams& p, int64_t w, int& bx, int& by)
{
    if (p.win_xy != nullptr) {
        bx = p.win_xy[2 * w];
        by = p.win_xy[2 * w + 1];
    } else {
        const int64_t gy = w / p.gnx, gx = w - gy * p.gnx;
        bx = p.gx0 + (int)gx * p.gdx;
        by = p.gy0 + (int)gy * p.gdy;
    }
}

// swizzled W x W tile: element (r, c) at r*W + (c ^ r); conflict-free for
// row-wise and column-wise float2 access by W lanes.
template <int W>
__device__ __forceinline__ int swz(int r, int c) { return r * W + (c ^ r); }

// sum over the W lanes of a group
template <int W, typename T = float>
__device__ __forceinline__ T group_sum(T x)
{
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o, W);
    return x;
}
template <int W>
__device__ __forceinline__ int group_sum_int(int x)
{
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o, W);
    return x;
}
template <int W>
__device__ __forceinline__ float group_max(float x)
{
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o, W));
    return x;
}

// One axis of the 3-point Gaussian fit on pedestal-shifted values
// L = l + ped, C = c + ped, R = r + ped (ped added implicitly):
//   (ln L - ln R) / (2 (ln L + ln R - 2 ln C)),  0 if the denominator is 0,
// NaN if any of L, C, R <= 0 (the reference takes log of a non-positive
// number there).  Also returns a bound on the error caused by an absolute
// error `dlt` in each of the plane values.
__device__ __forceinline__ float gauss_axis(float l, float c, float r, float ped, float dlt,
                                            float& err)
{
    const float L = l + ped, C = c + ped, R = r + ped;
    if (!(L > 0.f && C > 0.f && R > 0.f)) {
        err = 0.f;
        return __int_as_float(0x7fffffff);
    }
    const float num = log1pf((l - r) / R);
    const float den = log1pf((l - c) / C) + log1pf((r - c) / C);
    if (den == 0.f) {
        err = 3.4e38f;   // degenerate: leave it to the exact pass
        return 0.f;
    }
    const float f = num / (2.f * den);
    const float m = fminf(fminf(L, R), C);
    err = dlt * (1.f + 4.f * fabsf(f)) / (m * 2.f * fabsf(den));
    return f;
}

template <int W, int MODE, bool LIMIT, typename PixT, bool PLANES>
__global__ void __launch_bounds__(32 * kWarps, (W == 32 ? 3 : 4))
piv_fp32_kernel(const PivParams p)
{
    constexpr int NG = 32 / W;          // lane groups per warp
    constexpr int N = W * W;
    // peak scan range in swapped-plane coordinates (image_utils.impl.h:48,
    // :54; limited search: rect::dilate(0.5), rect.cpp:109-126)
    constexpr int D0 = LIMIT ? W / 4 : 0;
    constexpr int VW = LIMIT ? W / 2 : W;
    constexpr int SY0 = D0 + 1, SY1 = D0 + VW - 2;
    constexpr int SX0 = D0 + 1, SX1 = D0 + VW - 1;

    __shared__ float2 smem[kWarps][NG][N];

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int grp = lane / W;
    const int gl = lane % W;
    const int64_t task = (int64_t)blockIdx.x * kWarps + warp;
    const int64_t first = task * 2 * NG;
    if (first >= p.n_win) return;   // warp-uniform
    float2* S = smem[warp][grp];

    const PixT* fa = reinterpret_cast<const PixT*>(p.fa);
    const PixT* fb = reinterpret_cast<const PixT*>(p.fb);
    const size_t pitch = p.pitch / sizeof(PixT);

    float2 P[W];
    // per-window values of the two windows this group handles (scalars, so
    // that they stay in registers across the runtime loop)
    float ped4_0 = 0.f, ped4_1 = 0.f, en_0 = 0.f, en_1 = 0.f;

#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
        const int64_t w = first + h * NG + grp;
        const bool valid = w < p.n_win;
        int bx = 0, by = 0;
        if (valid) window_origin(p, w, bx, by);

        // ---- extract + widen (lane = column x, register = row y)
        using acc_t = typename px_traits<PixT>::acc;
        float2 v[W];
        acc_t ca = 0, cb = 0;
        if (valid) {
            const PixT* ra = fa + (size_t)by * pitch + bx + gl;
            const PixT* rb = fb + (size_t)by * pitch + bx + gl;
#pragma unroll
            for (int y = 0; y < W; ++y) {
                const acc_t pa = (acc_t)__ldg(ra + (size_t)y * pitch);
                const acc_t pb = (acc_t)__ldg(rb + (size_t)y * pitch);
                v[y].x = (float)pa;
                v[y].y = (float)pb;
                ca += pa;
                cb += pb;
            }
        } else {
#pragma unroll
            for (int y = 0; y < W; ++y) v[y] = make_float2(0.f, 0.f);
        }
        float sa, sb;
        double dped;                    // (sum a)(sum b), exact for integer pixels
        if (px_traits<PixT>::integer) { // column sums are exact integers < 2^24
            const int isa = group_sum_int<W>((int)ca);
            const int isb = group_sum_int<W>((int)cb);
            sa = (float)isa;
            sb = (float)isb;
            dped = PLANES ? (double)isa * (double)isb : 0.0;
        } else {
            const acc_t ta = group_sum<W, acc_t>(ca);
            const acc_t tb = group_sum<W, acc_t>(cb);
            sa = (float)ta;
            sb = (float)tb;
            dped = PLANES ? (double)ta * (double)tb : 0.0;
        }
        const float ma = sa * (1.f / N), mb = sb * (1.f / N);
        float e = 0.f;
#pragma unroll
        for (int y = 0; y < W; ++y) {
            v[y].x -= ma;
            v[y].y -= mb;
            e = fmaf(v[y].x, v[y].x, e);
            e = fmaf(v[y].y, v[y].y, e);
        }
        e = group_sum<W>(e);
        const float pd = (MODE == kModeComplex) ? 4.f * sa * sb : 0.f;
        if (h == 0) { en_0 = e; ped4_0 = pd; } else { en_1 = e; ped4_1 = pd; }
        if (PLANES && valid && gl == 0)
            p.peds[w] = (MODE == kModeComplex) ? dped : 0.0;

        // ---- forward 2-D FFT
        fft_dif<W, false>(v);                       // columns: v[i] = Zc[bitrev(i)][gl]
#pragma unroll
        for (int i = 0; i < W; ++i) S[swz<W>(bitrev<W>(i), gl)] = v[i];
        __syncwarp();
#pragma unroll
        for (int j = 0; j < W; ++j) v[j] = S[swz<W>(gl, j)];
        __syncwarp();
        fft_dif<W, false>(v);                       // rows: v[i] = Z[ky = gl][kx = bitrev(i)]

        // ---- unpack and conjugate product
        const int pl = (W - gl) & (W - 1);
        const bool zero_row = (MODE == kModeReal) && (gl == 0 || gl == W / 2);
#pragma unroll
        for (int i = 0; i < W; ++i) {
            const int kx = bitrev<W>(i);
            const int mi = bitrev<W>((W - kx) & (W - 1));
            float2 zm;
            zm.x = __shfl_sync(0xffffffffu, v[mi].x, pl, W);
            zm.y = __shfl_sync(0xffffffffu, v[mi].y, pl, W);
            const float2 z = v[i];
            const float2 a2 = make_float2(z.x + zm.x, z.y - zm.y);   // 2 A
            const float2 b2 = make_float2(z.y + zm.y, zm.x - z.x);   // 2 B
            float2 q = make_float2(b2.x * a2.x + b2.y * a2.y, b2.y * a2.x - b2.x * a2.y);
            bool zero = zero_row || (MODE == kModeReal && kx == 0) || (kx == 0 && gl == 0);
            if (zero) q = make_float2(0.f, 0.f);
            if (h == 0) {
                P[i] = q;
            } else {
                P[i] = make_float2(P[i].x - q.y, P[i].y + q.x);
            }
        }
    }

    // ---- inverse 2-D FFT of Q = P1 + i P2
    fft_dit<W, true>(P);                            // rows: P[j] = R[ky = gl][x = j]
#pragma unroll
    for (int j = 0; j < W; ++j) S[swz<W>(gl, j)] = P[j];
    __syncwarp();
#pragma unroll
    for (int i = 0; i < W; ++i) P[i] = S[swz<W>(bitrev<W>(i), gl)];
    __syncwarp();
    fft_dit<W, true>(P);                            // columns: P[y] = corr[y][x = gl]

    const float dlt = p.kappa * 5.9604645e-8f * 2.f * (float)N * (en_0 + en_1);
    const int xs = (gl + W / 2) & (W - 1);          // swapped column of this lane
    const bool col_ok = xs >= SX0 && xs < SX1;

#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
        const int64_t w = first + h * NG + grp;
        const bool valid = w < p.n_win;
        float val[W];
#pragma unroll
        for (int y = 0; y < W; ++y) val[y] = h ? P[y].y : P[y].x;

        if (PLANES && valid) {
#pragma unroll
            for (int y = 0; y < W; ++y) {
                const int ys = (y + W / 2) & (W - 1);
                p.planes[(size_t)w * N + ys * W + xs] = 0.25f * val[y];
            }
        }

        // ---- find_peaks: strict 4-neighbour maxima, top two
        float t0 = kNegInf, t1 = kNegInf, umax = kNegInf;
        int t0y = 0;
#pragma unroll
        for (int ys = SY0; ys < SY1; ++ys) {
            const int y = (ys + W / 2) & (W - 1);
            const float c = val[y];
            const float up = val[(y + W - 1) & (W - 1)];
            const float dn = val[(y + 1) & (W - 1)];
            const float lf = __shfl_sync(0xffffffffu, c, (gl + W - 1) & (W - 1), W);
            const float rt = __shfl_sync(0xffffffffu, c, (gl + 1) & (W - 1), W);
            const float m = fmaxf(fmaxf(up, dn), fmaxf(lf, rt));
            const bool strict = col_ok && (m < c);
            const bool unc = col_ok && (fabsf(m - c) <= dlt);
            umax = unc ? fmaxf(umax, c) : umax;
            const float sv = strict ? c : kNegInf;
            const bool gt = sv > t0;
            t1 = gt ? t0 : fmaxf(t1, sv);
            t0y = gt ? ys : t0y;
            t0 = gt ? sv : t0;
        }
        int key = t0y * W + xs;                     // row-major index in the swapped plane
#pragma unroll
        for (int o = W / 2; o > 0; o >>= 1) {
            const float o0 = __shfl_xor_sync(0xffffffffu, t0, o, W);
            const float o1 = __shfl_xor_sync(0xffffffffu, t1, o, W);
            const int ok = __shfl_xor_sync(0xffffffffu, key, o, W);
            const bool take = (o0 > t0) || (o0 == t0 && ok < key);
            const float n1 = take ? fmaxf(t0, o1) : fmaxf(t1, o0);
            t0 = take ? o0 : t0;
            key = take ? ok : key;
            t1 = n1;
        }
        umax = group_max<W>(umax);

        // ---- neighbourhood of the first peak (through shared memory)
#pragma unroll
        for (int y = 0; y < W; ++y) S[y * W + gl] = make_float2(val[y], 0.f);
        __syncwarp();
        const int px = key % W, py = key / W;       // swapped-plane coordinates
        const int ux = (px + W / 2) & (W - 1), uy = (py + W / 2) & (W - 1);
        const float vc = S[uy * W + ux].x;
        const float vl = S[uy * W + ((ux + W - 1) & (W - 1))].x;
        const float vr = S[uy * W + ((ux + 1) & (W - 1))].x;
        const float vu = S[((uy + W - 1) & (W - 1)) * W + ux].x;
        const float vd = S[((uy + 1) & (W - 1)) * W + ux].x;
        __syncwarp();

        if (valid && gl == 0) {
            const bool has2 = t1 > kNegInf;
            const float ped = h ? ped4_1 : ped4_0;
            bool certain;
            opiv_vector out{ 0.f, 0.f, 0.f, 0.f, 0.f };
            int32_t code = -1;
            if (!has2) {
                certain = !(umax > kNegInf);
            } else {
                float ex, ey;
                const float fx = gauss_axis(vl, vc, vr, ped, dlt, ex);
                const float fy = gauss_axis(vu, vc, vd, ped, dlt, ey);
                const float p0 = t0 + ped, p1 = t1 + ped;
                // sn = p0 / p1 when p1 > 0: relative error <= e/|p0| + e/|p1|
                // with e = dlt / 2 the error of one plane value
                const float sn_err = 0.5f * dlt * (1.f / fabsf(p0) + 1.f / fabsf(p1));
                certain = (umax < t1 - 2.f * dlt) && (t0 - t1 > dlt) && (fabsf(p1) > dlt) &&
                          (ex < kFitTol) && (ey < kFitTol) &&
                          (p1 <= 0.f || sn_err < kSnTol * (1.f + p0 / p1));
                int bx, by;
                window_origin(p, w, bx, by);
                out.x = (float)(bx + W / 2);
                out.y = (float)(p.img_h - (by + W / 2));
                out.u = (float)(W / 2 - px) - fx;
                out.v = (float)(W / 2 - py) - fy;
                out.sn = (p1 > 0.f) ? (t0 + ped) / p1 : 0.f;
                code = key;
            }
            p.out_vec[w] = out;
            if (p.out_peak) p.out_peak[w] = code;
            if (!certain && p.flag_list) {
                const unsigned int slot = atomicAdd(p.flag_count, 1u);
                p.flag_list[slot] = (int32_t)w;
            }
        }
    }
}

template <int W, int MODE, bool LIMIT, typename PixT, bool PLANES>
cudaError_t launch_t(const PivParams& p, cudaStream_t s)
{
    constexpr int NG = 32 / W;
    const int64_t tasks = (p.n_win + 2 * NG - 1) / (2 * NG);
    const int64_t blocks = (tasks + kWarps - 1) / kWarps;
    piv_fp32_kernel<W, MODE, LIMIT, PixT, PLANES><<<(unsigned)blocks, 32 * kWarps, 0, s>>>(p);
    return cudaGetLastError();
}

// frames (u8, u16, f32) without plane output; double windows (the per-window
// batch API) with plane output
template <int W, int MODE, bool LIMIT>
cudaError_t launch_dt(const PivParams& p, int dtype, bool planes, cudaStream_t s)
{
    if (planes) return dtype == kF64 ? launch_t<W, MODE, LIMIT, double, true>(p, s)
                                     : cudaErrorInvalidValue;
    switch (dtype) {
    case kU8: return launch_t<W, MODE, LIMIT, uint8_t, false>(p, s);
    case kU16: return launch_t<W, MODE, LIMIT, uint16_t, false>(p, s);
    case kF32: return launch_t<W, MODE, LIMIT, float, false>(p, s);
    default: return cudaErrorInvalidValue;
    }
}

template <int W>
cudaError_t launch_w(const PivParams& p, int dtype, int mode, int limit, bool planes,
                     cudaStream_t s)
{
    if (p.n_win <= 0) return cudaSuccess;
    if (mode == kModeComplex)
        return limit ? launch_dt<W, kModeComplex, true>(p, dtype, planes, s)
                     : launch_dt<W, kModeComplex, false>(p, dtype, planes, s);
    return limit ? launch_dt<W, kModeReal, true>(p, dtype, planes, s)
                 : launch_dt<W, kModeReal, false>(p, dtype, planes, s);
}

}  // namespace fp32
}  // namespace opiv
