// piv_fp32_w64.cu -- fused FP32 PIV kernel for 64 x 64 windows (sm_103a).
//
// A 64-point row does not fit one lane's registers next to everything else,
// so this kernel keeps the pair's spectra in shared memory: one CTA of 256
// threads per pair of windows, two padded 64 x 67 float2 tiles.  The steps
// and the formulas are those of the 16/32 kernel (piv_fp32.cuh):
//   z = a + i b; 2-D FFT (rows, then columns) as two radix-8 decimation-
//   in-frequency passes over the tile (64 = 8^2; outputs in base-8 digit-
//   reversed order, absorbed in the indexing);
//   bank-conflict-free tile layout: column c of a row sits at c + 2 (c/16)
//   and rows are 71 float2 apart, so sixteen threads reading sixteen
//   neighbouring rows, sixteen neighbouring columns, or the sixteen columns
//   of a digit-reversed block all hit distinct banks;
//   4 conj(P) = (2 Im(Z Zm), |Z|^2 - |Zm|^2) with Zm = Z[-k] (P = B conj A,
//   fft.h:188-227), REAL mode's zeroed spectrum row 0, row W/2, column 0
//   (fft.h:166-183), DC product dropped and the pedestal added back;
//   Q = conj(4 P1) + i conj(4 P2), one forward 2-D FFT -> both planes;
//   find_peaks(plane, 2, 1) (image_utils.impl.h:42-74) as a block scan and
//   reduction; fit_simple_gaussian (impl:77-101); vector of main.cpp:220-236;
//   the same certification and hand-off to the exact kernel.

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "fft_reg.cuh"
#include "offsets.cuh"
#include "piv_kernels.h"

namespace opiv {
namespace w64 {

constexpr int W = 64;
constexpr int N = W * W;
constexpr int LD = W + 7;            // row stride (float2), odd: rows fall on distinct banks
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
// certification thresholds: as the 16 / 32 px kernel (piv_fp32.cuh)
constexpr float kFitTol = 6e-5f;
constexpr float kSnTol = 6e-6f;
#define kNegInf64 (-__int_as_float(0x7f800000))

// base-8 digit reversal of a 6-bit index (an involution)
__device__ __forceinline__ int dr(int v) { return ((v & 7) << 3) | (v >> 3); }

__device__ __forceinline__ float2 cmul(float2 a, float2 w)
{
    return make_float2(fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x));
}

// offset of column c inside a row: two pad elements after every 16 columns
__device__ __forceinline__ int pos(int c) { return c + 2 * (c >> 4); }

// In-place forward 8-point DFT, natural order in and out.
__device__ __forceinline__ void dft8(float2* x)
{
    constexpr float r = 0.70710678118654752f;   // cos(pi/4)
    const float2 a0 = make_float2(x[0].x + x[4].x, x[0].y + x[4].y), a1 = make_float2(x[0].x - x[4].x, x[0].y - x[4].y);
    const float2 a2 = make_float2(x[2].x + x[6].x, x[2].y + x[6].y), a3 = make_float2(x[2].x - x[6].x, x[2].y - x[6].y);
    const float2 a4 = make_float2(x[1].x + x[5].x, x[1].y + x[5].y), a5 = make_float2(x[1].x - x[5].x, x[1].y - x[5].y);
    const float2 a6 = make_float2(x[3].x + x[7].x, x[3].y + x[7].y), a7 = make_float2(x[3].x - x[7].x, x[3].y - x[7].y);
    // even outputs: 4-point DFT of (a0, a4, a2, a6)
    const float2 e0 = make_float2(a0.x + a2.x, a0.y + a2.y), e1 = make_float2(a0.x - a2.x, a0.y - a2.y);
    const float2 e2 = make_float2(a4.x + a6.x, a4.y + a6.y), e3 = make_float2(a4.x - a6.x, a4.y - a6.y);
    x[0] = make_float2(e0.x + e2.x, e0.y + e2.y);
    x[4] = make_float2(e0.x - e2.x, e0.y - e2.y);
    x[2] = make_float2(e1.x + e3.y, e1.y - e3.x);   // e1 - i e3
    x[6] = make_float2(e1.x - e3.y, e1.y + e3.x);   // e1 + i e3
    // odd outputs: 4-point DFT of (a1, a5 w, -i a3, a7 w^3), w = exp(-i pi/4)
    const float2 b1 = make_float2((a5.x + a5.y) * r, (a5.y - a5.x) * r);
    const float2 b3 = make_float2((a7.y - a7.x) * r, -(a7.x + a7.y) * r);
    const float2 o0 = make_float2(a1.x + a3.y, a1.y - a3.x), o1 = make_float2(a1.x - a3.y, a1.y + a3.x);
    const float2 o2 = make_float2(b1.x + b3.x, b1.y + b3.y), o3 = make_float2(b1.x - b3.x, b1.y - b3.y);
    x[1] = make_float2(o0.x + o2.x, o0.y + o2.y);
    x[5] = make_float2(o0.x - o2.x, o0.y - o2.y);
    x[3] = make_float2(o1.x + o3.y, o1.y - o3.x);   // o1 - i o3
    x[7] = make_float2(o1.x - o3.y, o1.y + o3.x);   // o1 + i o3
}

// One radix-8 DIF pass over all 64 lines of tile T (rows when ROWS, else
// columns).  FIRST: butterfly j takes elements j + 8 m and scales output m
// by tw[j m] = exp(-2 pi i j m / 64); second pass: butterfly j takes
// elements 8 j + m, no twiddles.  After both passes bin k0 + 8 k1 of a line
// sits at 8 k0 + k1.  Neighbouring threads take neighbouring lines and the
// same butterfly, so a warp's twiddles are one broadcast.
template <bool ROWS, bool FIRST>
__device__ __forceinline__ void dif8_pass(float2* T, const float2* tw)
{
#pragma unroll
    for (int it = 0; it < 64 * 8 / kThreads; ++it) {
        const int k = (int)threadIdx.x + it * kThreads;
        const int line = k & 63, j = k >> 6;
        const int base = FIRST ? j : 8 * j, es = FIRST ? 8 : 1;
        auto el = [&](int e) -> float2& { return ROWS ? T[line * LD + pos(e)] : T[e * LD + pos(line)]; };
        float2 x[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) x[m] = el(base + m * es);
        dft8(x);
        if (FIRST) {
#pragma unroll
            for (int m = 1; m < 8; ++m) x[m] = cmul(x[m], tw[j * m]);
        }
#pragma unroll
        for (int m = 0; m < 8; ++m) el(base + m * es) = x[m];
    }
    __syncthreads();
}

__device__ __forceinline__ void fft2d(float2* T, const float2* tw)
{
    dif8_pass<true, true>(T, tw);
    dif8_pass<true, false>(T, tw);
    dif8_pass<false, true>(T, tw);
    dif8_pass<false, false>(T, tw);
}

// position in a transformed tile of spectrum bin (ky, kx) / plane (y, x)
__device__ __forceinline__ int at(int r, int c) { return dr(r) * LD + pos(dr(c)); }

__device__ __forceinline__ void window_origin(const PivParams& p, int w, int& bx, int& by)
{
    if (p.win_xy != nullptr) {
        bx = p.win_xy[2 * w];
        by = p.win_xy[2 * w + 1];
    } else {
        const int gy = (int)((unsigned)w / (unsigned)p.gnx);
        bx = p.gx0 + (w - gy * p.gnx) * p.gdx;
        by = p.gy0 + gy * p.gdy;
    }
}

// Running top-2 of strict 4-neighbour maxima (find_peaks) plus the largest
// value whose strict-maximum decision is within dlt of flipping.
struct Top2 {
    float t0, t1, umax;
    int key;
    __device__ __forceinline__ void init()
    {
        t0 = t1 = umax = kNegInf64;
        key = 0x7fffffff;
    }
    __device__ __forceinline__ void add(float c, float m, float dlt, int k)
    {
        const float dd = m - c;
        if (fabsf(dd) <= dlt) umax = fmaxf(umax, c);
        if (dd < 0.f) {
            if (c > t0) { t1 = t0; t0 = c; key = k; }
            else t1 = fmaxf(t1, c);
        }
    }
};

__device__ __forceinline__ float block_sum(float v, float* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float s = 0.f;
    for (int i = 0; i < kWarps; ++i) s += red[i];
    __syncthreads();
    return s;
}

extern __shared__ float2 w64_dyn_smem[];

// One task: windows 2 blk and 2 blk + 1 of pair p, run by the whole CTA.
template <int MODE, bool LIMIT, typename PixT, bool PLANES>
__device__ __forceinline__ void w64_task(const PivParams& p, const int blk)
{
    constexpr int D0 = LIMIT ? W / 4 : 0;
    constexpr int VW = LIMIT ? W / 2 : W;
    constexpr int SY0 = D0 + 1, SY1 = D0 + VW - 2;
    constexpr int SX0 = D0 + 1, SX1 = D0 + VW - 1;

    float2* sm = w64_dyn_smem;
    float2* T1 = sm;                  // first window, then Q, then both planes
    float2* T2 = sm + W * LD;         // second window
    __shared__ float2 tw[64];
    __shared__ float red[kWarps * 4];
    __shared__ float rv0[kWarps], rv1[kWarps], ru[kWarps];
    __shared__ int rk[kWarps];
    __shared__ float sped[2];

    const int t = threadIdx.x;
    const int w0 = 2 * blk;
    if (w0 >= (int)p.n_win) return;
    const int w1 = w0 + 1;
    const bool valid1 = w1 < (int)p.n_win;
    if (t < 64) tw[t] = make_float2(c_tw.re[t], c_tw.im[t]);

    const PixT* fa = reinterpret_cast<const PixT*>(p.fa);
    const PixT* fb = reinterpret_cast<const PixT*>(p.fb);
    const size_t pitch = p.pitch / sizeof(PixT);

    // ---- extract, widen, energies (and the exact pedestal for the batch API)
    int bx0, by0, bx1 = 0, by1 = 0, ox0, oy0, ox1 = 0, oy1 = 0;
    window_origin(p, w0, bx0, by0);
    b_offset(p, W, bx0, by0, ox0, oy0);
    if (valid1) {
        window_origin(p, w1, bx1, by1);
        b_offset(p, W, bx1, by1, ox1, oy1);
    }
    float e0 = 0.f, e1 = 0.f;
    double sa0 = 0.0, sb0 = 0.0, sa1 = 0.0, sb1 = 0.0;
    // pixels widen straight to float (exact for 8/16-bit frames); doubles
    // only for the per-window API's exact pedestal (PLANES, double frames)
    for (int i = t; i < N; i += kThreads) {
        const int y = i >> 6, x = i & 63;
        const PixT pa0 = __ldg(fa + (size_t)(by0 + y) * pitch + bx0 + x);
        const PixT pb0 = __ldg(fb + (size_t)(by0 + oy0 + y) * pitch + bx0 + ox0 + x);
        PixT pa1 = PixT(0), pb1 = PixT(0);
        if (valid1) {
            pa1 = __ldg(fa + (size_t)(by1 + y) * pitch + bx1 + x);
            pb1 = __ldg(fb + (size_t)(by1 + oy1 + y) * pitch + bx1 + ox1 + x);
        }
        const float2 z0 = make_float2((float)pa0, (float)pb0), z1 = make_float2((float)pa1, (float)pb1);
        T1[y * LD + pos(x)] = z0;
        T2[y * LD + pos(x)] = z1;
        e0 = fmaf(z0.x, z0.x, fmaf(z0.y, z0.y, e0));
        e1 = fmaf(z1.x, z1.x, fmaf(z1.y, z1.y, e1));
        if (PLANES) {
            sa0 += (double)pa0;
            sb0 += (double)pb0;
            sa1 += (double)pa1;
            sb1 += (double)pb1;
        }
    }
    e0 = block_sum(e0, red);
    e1 = block_sum(e1, red);
    if (PLANES) {
        const double s[4] = { sa0, sb0, sa1, sb1 };
        double tot[4];
        for (int c = 0; c < 4; ++c) {
            double v = s[c];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            __syncthreads();
            if ((t & 31) == 0) reinterpret_cast<double*>(red)[t >> 5] = v;
            __syncthreads();
            double acc = 0.0;
            for (int i = 0; i < kWarps; ++i) acc += reinterpret_cast<double*>(red)[i];
            tot[c] = acc;
            __syncthreads();
        }
        if (t == 0) {
            p.peds[w0] = (MODE == kModeComplex) ? tot[0] * tot[1] : 0.0;
            if (valid1) p.peds[w1] = (MODE == kModeComplex) ? tot[2] * tot[3] : 0.0;
        }
    }
    __syncthreads();

    // ---- forward transforms
    fft2d(T1, tw);
    fft2d(T2, tw);
    if (t == 0) {   // DC bins: (sum a, sum b) of each window
        const float2 d0 = T1[0], d1 = T2[0];
        sped[0] = (MODE == kModeComplex) ? 4.f * d0.x * d0.y : 0.f;
        sped[1] = (MODE == kModeComplex) ? 4.f * d1.x * d1.y : 0.f;
    }
    __syncthreads();
    // zero the DC bin (COMPLEX) or the reference's unpacked-out set (REAL)
    for (int i = t; i < N; i += kThreads) {
        const int ky = i >> 6, kx = i & 63;
        const bool zero = (MODE == kModeReal) ? (ky == 0 || ky == W / 2 || kx == 0)
                                              : (ky == 0 && kx == 0);
        if (zero) {
            T1[at(ky, kx)] = make_float2(0.f, 0.f);
            T2[at(ky, kx)] = make_float2(0.f, 0.f);
        }
    }
    __syncthreads();

    // ---- products, packed: Q[ky][kx] = conj(4 P1) + i conj(4 P2), written
    // in natural order (the next transform is a forward DIF again)
    float2 q[N / kThreads];
#pragma unroll
    for (int n = 0; n < N / kThreads; ++n) {
        const int i = t + n * kThreads;
        const int ky = i >> 6, kx = i & 63;
        const int mky = (W - ky) & (W - 1), mkx = (W - kx) & (W - 1);
        const float2 z1 = T1[at(ky, kx)], m1 = T1[at(mky, mkx)];
        const float2 z2 = T2[at(ky, kx)], m2 = T2[at(mky, mkx)];
        const float im1 = 2.f * fmaf(z1.x, m1.y, z1.y * m1.x);
        const float d1 = fmaf(z1.x, z1.x, fmaf(z1.y, z1.y, -fmaf(m1.x, m1.x, m1.y * m1.y)));
        const float im2 = 2.f * fmaf(z2.x, m2.y, z2.y * m2.x);
        const float d2 = fmaf(z2.x, z2.x, fmaf(z2.y, z2.y, -fmaf(m2.x, m2.x, m2.y * m2.y)));
        q[n] = make_float2(im1 - d2, d1 + im2);
    }
    __syncthreads();
#pragma unroll
    for (int n = 0; n < N / kThreads; ++n) {
        const int i = t + n * kThreads;
        T1[(i >> 6) * LD + pos(i & 63)] = q[n];
    }
    __syncthreads();
    fft2d(T1, tw);   // T1[at(y, x)] = plane1(y, x) + i plane2(y, x), 4x scaled

    const float dlt = p.kappa * 5.9604645e-8f * 2.f * (float)N * (e0 + e1);
    const int lane = t & 31, wp = t >> 5;

    // ---- find_peaks on both planes at once: thread = (column, 16-row
    // block); rows roll through registers, the horizontal neighbours come
    // from the neighbouring lanes (the two edge lanes read theirs)
    Top2 s0, s1;
    s0.init();
    s1.init();
    {
        const int xs = t & 63, yb = (t >> 6) * 16;
        const bool col_ok = xs >= SX0 && xs < SX1;
        auto cell = [&](int ys, int x) -> float2 {   // swapped-plane values of both planes
            return T1[at((ys + W / 2) & (W - 1), (x + W / 2) & (W - 1))];
        };
        float2 up = cell(yb - 1, xs), cc = cell(yb, xs);
        for (int ys = yb; ys < yb + 16; ++ys) {
            const float2 dn = cell(ys + 1, xs);
            float2 lf = make_float2(__shfl_up_sync(0xffffffffu, cc.x, 1), __shfl_up_sync(0xffffffffu, cc.y, 1));
            float2 rt = make_float2(__shfl_down_sync(0xffffffffu, cc.x, 1), __shfl_down_sync(0xffffffffu, cc.y, 1));
            if (lane == 0) lf = cell(ys, xs - 1);
            if (lane == 31) rt = cell(ys, xs + 1);
            if (col_ok && ys >= SY0 && ys < SY1) {
                s0.add(cc.x, fmaxf(fmaxf(up.x, dn.x), fmaxf(lf.x, rt.x)), dlt, ys * W + xs);
                s1.add(cc.y, fmaxf(fmaxf(up.y, dn.y), fmaxf(lf.y, rt.y)), dlt, ys * W + xs);
            }
            up = cc;
            cc = dn;
        }
    }

    for (int h = 0; h < 2; ++h) {
        const int w = h ? w1 : w0;
        const bool valid = h ? valid1 : true;
        const float ped = sped[h];
        auto val = [&](int ys, int xs) -> float {   // swapped-plane value
            const float2 v = T1[at((ys + W / 2) & (W - 1), (xs + W / 2) & (W - 1))];
            return h ? v.y : v.x;
        };
        if (PLANES && valid)
            for (int i = t; i < N; i += kThreads)
                p.planes[(size_t)w * N + i] = 0.25f * val(i >> 6, i & 63);

        float t0 = h ? s1.t0 : s0.t0, t1 = h ? s1.t1 : s0.t1, umax = h ? s1.umax : s0.umax;
        int key = h ? s1.key : s0.key;
        // warp reduction (ties to the lowest row-major index)
        for (int o = 16; o > 0; o >>= 1) {
            const float o0 = __shfl_xor_sync(0xffffffffu, t0, o);
            const float o1 = __shfl_xor_sync(0xffffffffu, t1, o);
            const int ok = __shfl_xor_sync(0xffffffffu, key, o);
            const bool take = (o0 > t0) || (o0 == t0 && ok < key);
            const float n1 = take ? fmaxf(t0, o1) : fmaxf(t1, o0);
            t0 = take ? o0 : t0;
            key = take ? ok : key;
            t1 = n1;
            umax = fmaxf(umax, __shfl_xor_sync(0xffffffffu, umax, o));
        }
        if (lane == 0) { rv0[wp] = t0; rv1[wp] = t1; rk[wp] = key; ru[wp] = umax; }
        __syncthreads();
        if (t == 0) {
            float g0 = kNegInf64, g1 = kNegInf64, gu = kNegInf64;
            int gk = 0x7fffffff;
            for (int i = 0; i < kWarps; ++i) {
                const bool take = (rv0[i] > g0) || (rv0[i] == g0 && rk[i] < gk);
                const float n1 = take ? fmaxf(g0, rv1[i]) : fmaxf(g1, rv0[i]);
                if (take) { g0 = rv0[i]; gk = rk[i]; }
                g1 = n1;
                gu = fmaxf(gu, ru[i]);
            }
            if (valid) {
                opiv_vector out{ 0.f, 0.f, 0.f, 0.f, 0.f };
                int32_t code = -1;
                bool certain;
                if (!(g1 > kNegInf64)) {
                    certain = !(gu > kNegInf64);
                } else {
                    const int px = gk % W, py = gk / W;
                    const float vc = val(py, px), vl = val(py, px - 1), vr = val(py, px + 1);
                    const float vu = val(py - 1, px), vd = val(py + 1, px);
                    const float C = vc + ped, L = vl + ped, R = vr + ped, U = vu + ped, D = vd + ped;
                    const float nan = __int_as_float(0x7fffffff);
                    const bool okx = L > 0.f && C > 0.f && R > 0.f;
                    const bool oky = U > 0.f && C > 0.f && D > 0.f;
                    const float denx = log1pf((vl - vc) / C) + log1pf((vr - vc) / C);
                    const float deny = log1pf((vu - vc) / C) + log1pf((vd - vc) / C);
                    const float fx = okx ? log1pf((vl - vr) / R) / (2.f * denx) : nan;
                    const float fy = oky ? log1pf((vu - vd) / D) / (2.f * deny) : nan;
                    const float mx = fminf(fminf(L, R), C), my = fminf(fminf(U, D), C);
                    const float ex = okx ? (denx == 0.f ? 3.4e38f
                                            : dlt * (1.f + 4.f * fabsf(fx)) / (mx * 2.f * fabsf(denx)))
                                         : (mx < -dlt ? 0.f : 3.4e38f);
                    const float ey = oky ? (deny == 0.f ? 3.4e38f
                                            : dlt * (1.f + 4.f * fabsf(fy)) / (my * 2.f * fabsf(deny)))
                                         : (my < -dlt ? 0.f : 3.4e38f);
                    const float p0 = g0 + ped, p1 = g1 + ped;
                    const float sn_err = 0.5f * dlt * (1.f / fabsf(p0) + 1.f / fabsf(p1));
                    certain = (gu < g1 - 2.f * dlt) && (g0 - g1 > dlt) && (fabsf(p1) > dlt) &&
                              (ex < kFitTol) && (ey < kFitTol) &&
                              (p1 <= 0.f || sn_err < kSnTol * (1.f + p0 / p1));
                    const int bx = h ? bx1 : bx0, by = h ? by1 : by0;
                    out.x = (float)(bx + W / 2);
                    out.y = (float)(p.img_h - (by + W / 2));
                    out.u = (float)(W / 2 - px - (h ? ox1 : ox0)) - fx;
                    out.v = (float)(W / 2 - py - (h ? oy1 : oy0)) - fy;
                    out.sn = (p1 > 0.f) ? p0 / p1 : 0.f;
                    code = gk;
                }
                p.out_vec[w] = out;
                if (p.out_peak) p.out_peak[w] = code;
                if (p.out_disp) {
                    const int ox = h ? ox1 : ox0, oy = h ? oy1 : oy0;
                    p.out_disp[w] = code >= 0 ? pack_disp(gk % W - W / 2 + ox, gk / W - W / 2 + oy)
                                              : pack_disp(ox, oy);
                }
                if (!certain && p.flag_list) {
                    const unsigned int slot = atomicAdd(p.flag_count, 1u);
                    p.flag_list[slot] = (int32_t)w + p.flag_base;
                }
            }
        }
        __syncthreads();
    }
}

template <int MODE, bool LIMIT, typename PixT, bool PLANES>
__global__ void __launch_bounds__(kThreads, 3)
piv_w64_kernel(const PivParams p)
{
    w64_task<MODE, LIMIT, PixT, PLANES>(p, (int)blockIdx.x);
}

// Persistent form over a device work queue: each CTA takes q.chunk tasks
// (window pairs) at a time until the pass's tasks (every image pair's) run
// out, claiming the next chunk while the current one runs (thread 0 keeps
// the atomic's result in a register until the next barrier).  No CTA waits
// for another.
// Copies pair j's descriptor from global memory into `dst` (shared) with
// the CTA's threads; all threads then read it from there.
__device__ __forceinline__ const PivParams& cta_item(const PivQueue& q, int j, PivParams* dst)
{
    constexpr int NQ = (int)(sizeof(PivParams) / 16);
    const uint4* src = reinterpret_cast<const uint4*>(q.items_g + j);
    if ((int)threadIdx.x < NQ) reinterpret_cast<uint4*>(dst)[threadIdx.x] = __ldg(src + threadIdx.x);
    __syncthreads();
    return *dst;
}

template <int MODE, bool LIMIT, typename PixT>
__global__ void __launch_bounds__(kThreads, 3)
piv_w64_queue_kernel(const __grid_constant__ PivQueue q)
{
    __shared__ unsigned int s_t0;
    __shared__ __align__(16) unsigned char s_item[sizeof(PivParams)];
    const int n_tasks = q.first_task[q.n_items];
    unsigned int next = 0;
    if (threadIdx.x == 0) next = atomicAdd(q.head, (unsigned int)q.chunk);
#pragma unroll 1
    for (;;) {
        if (threadIdx.x == 0) s_t0 = next;
        __syncthreads();
        const unsigned int t0 = s_t0;
        __syncthreads();   // every thread has read s_t0 before it is written again
        if (t0 >= (unsigned int)n_tasks) break;
        if (threadIdx.x == 0) next = atomicAdd(q.head, (unsigned int)q.chunk);
        const int t1 = min((int)t0 + q.chunk, n_tasks);
#pragma unroll 1
        for (int t = (int)t0; t < t1; ++t) {
            const int j = __ldg(q.task_item + t);
            // the task ends with a barrier: the previous descriptor is no longer read
            const PivParams& p = cta_item(q, j, reinterpret_cast<PivParams*>(s_item));
            w64_task<MODE, LIMIT, PixT, false>(p, t - q.first_task[j]);
        }
    }
}

template <int MODE, bool LIMIT, typename PixT, bool PLANES>
cudaError_t launch_t(const PivParams& p, cudaStream_t s)
{
    const size_t smem = sizeof(float2) * 2 * W * LD;
    static std::atomic<uint64_t> attr_done{ 0 };   // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(attr_done.load() & bit)) {
        const cudaError_t e = cudaFuncSetAttribute(piv_w64_kernel<MODE, LIMIT, PixT, PLANES>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem);
        if (e != cudaSuccess) return e;
        attr_done.fetch_or(bit);
    }
    const int64_t blocks = (p.n_win + 1) / 2;
    piv_w64_kernel<MODE, LIMIT, PixT, PLANES><<<(unsigned)blocks, kThreads, smem, s>>>(p);
    return cudaGetLastError();
}

template <int MODE, bool LIMIT>
cudaError_t launch_dt(const PivParams& p, int dtype, bool planes, cudaStream_t s)
{
    if (planes) return dtype == kF64 ? launch_t<MODE, LIMIT, double, true>(p, s) : cudaErrorInvalidValue;
    switch (dtype) {
    case kU8: return launch_t<MODE, LIMIT, uint8_t, false>(p, s);
    case kU16: return launch_t<MODE, LIMIT, uint16_t, false>(p, s);
    case kF32: return launch_t<MODE, LIMIT, float, false>(p, s);
    default: return cudaErrorInvalidValue;
    }
}

// The same work list dispatched by the hardware: CTA b runs task b, no
// persistent loop.
template <int MODE, bool LIMIT, typename PixT>
__global__ void __launch_bounds__(kThreads, 3)
piv_w64_list_kernel(const __grid_constant__ PivQueue q)
{
    __shared__ __align__(16) unsigned char s_item[sizeof(PivParams)];
    const int t = (int)blockIdx.x;
    const int j = __ldg(q.task_item + t);
    const PivParams& p = cta_item(q, j, reinterpret_cast<PivParams*>(s_item));
    w64_task<MODE, LIMIT, PixT, false>(p, t - q.first_task[j]);
}

// blocks > 0: the persistent kernel on `blocks` CTAs; blocks == 0: the
// hardware-dispatched list kernel, one CTA per task
template <int MODE, bool LIMIT, typename PixT>
cudaError_t queue_t(const PivQueue& q, int blocks, int* max_ctas, cudaStream_t s)
{
    const size_t smem = sizeof(float2) * 2 * W * LD;
    auto kern = piv_w64_queue_kernel<MODE, LIMIT, PixT>;
    auto list = piv_w64_list_kernel<MODE, LIMIT, PixT>;
    static std::atomic<uint64_t> attr_done{ 0 };   // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(attr_done.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(list, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_done.fetch_or(bit);
    }
    if (max_ctas) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(max_ctas, kern, kThreads, smem);
    if (blocks < 0) return cudaErrorInvalidValue;
    if (blocks == 0) {
        const int n_tasks = q.first_task[q.n_items];
        if (n_tasks <= 0) return cudaSuccess;
        list<<<(unsigned)n_tasks, kThreads, smem, s>>>(q);
    } else {
        kern<<<(unsigned)blocks, kThreads, smem, s>>>(q);
    }
    return cudaGetLastError();
}

template <int MODE, bool LIMIT>
cudaError_t queue_dt(const PivQueue& q, int dtype, int blocks, int* max_ctas, cudaStream_t s)
{
    switch (dtype) {
    case kU8: return queue_t<MODE, LIMIT, uint8_t>(q, blocks, max_ctas, s);
    case kU16: return queue_t<MODE, LIMIT, uint16_t>(q, blocks, max_ctas, s);
    case kF32: return queue_t<MODE, LIMIT, float>(q, blocks, max_ctas, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace w64

// the 64 px kernel loads rows element-wise and needs no alignment flag
cudaError_t queue_piv_fp32_w64(const PivQueue& q, int dtype, int mode, int limit, bool, int blocks,
                               int* max_ctas, cudaStream_t s)
{
    if (mode == kModeComplex)
        return limit ? w64::queue_dt<kModeComplex, true>(q, dtype, blocks, max_ctas, s)
                     : w64::queue_dt<kModeComplex, false>(q, dtype, blocks, max_ctas, s);
    return limit ? w64::queue_dt<kModeReal, true>(q, dtype, blocks, max_ctas, s)
                 : w64::queue_dt<kModeReal, false>(q, dtype, blocks, max_ctas, s);
}

cudaError_t launch_piv_fp32_w64(const PivParams& p, int dtype, int mode, int limit, bool planes,
                                cudaStream_t s)
{
    if (p.n_win <= 0) return cudaSuccess;
    if (mode == kModeComplex)
        return limit ? w64::launch_dt<kModeComplex, true>(p, dtype, planes, s)
                     : w64::launch_dt<kModeComplex, false>(p, dtype, planes, s);
    return limit ? w64::launch_dt<kModeReal, true>(p, dtype, planes, s)
                 : w64::launch_dt<kModeReal, false>(p, dtype, planes, s);
}

}  // namespace opiv
