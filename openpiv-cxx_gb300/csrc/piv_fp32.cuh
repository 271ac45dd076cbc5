// piv_fp32.cuh -- fused FP32 PIV window kernel for sm_103a (template; the
// piv_fp32_w*.cu files instantiate it per window size).
//
// A warp processes a task of 2*NG interrogation windows: NG = 32/W lane
// groups of W lanes, each group a pair of windows.  Per window:
//
//   extract (core::extract, image_utils.impl.h:392-419): lane = window row,
//   128-bit loads where the grid is 16-byte aligned, pixels widened to float
//   exactly (byte-permute into the mantissa of 2^23, then subtract 2^23);
//   z = a + i*b (join_from_channels, image_utils.impl.h:294-315);
//   2-D FFT of z in registers: row FFT (lane = row), transpose through a
//   padded shared-memory tile, column FFT;
//   the two-for-one unpack and the product in one step: with Zm = Z[-k]
//   (fetched from the mirror lane by a shuffle),
//       P = B conj(A) = ( Im(Z Zm) / 2 , (|Zm|^2 - |Z|^2) / 4 ),
//   which is FFT(b) conj(FFT(a)) of fft.h:188-227; REAL mode leaves the
//   reference's unpacked set only (fft.h:166-183: spectrum row 0, row W/2
//   and column 0 stay zero), done by zeroing those Z rows / the Z column;
//   the products of the pair are packed as Q = conj(P1) + i conj(P2): both
//   P are Hermitian, so one *forward* 2-D FFT of Q gives plane1 + i plane2
//   (the reference's unnormalised inverse, fft.h:223, up to the shared
//   conjugation);
//   quadrant swap as an index remap (swap_quadrants, impl:367-386);
//   find_peaks(plane, 2, 1) (impl:42-74): warp scan + top-2 reduction;
//   fit_simple_gaussian (impl:77-101) and the vector of main.cpp:220-236.
//
// Every 1-D transform is the same in-register radix-2 DIT routine (FMA form,
// fft_reg.cuh), run from
// one runtime loop over the six transform stages of a pair, so the kernel's
// code stays small enough for the instruction caches.
//
// The DC product is dropped (P[0][0] = 0) and the pedestal (sum a)(sum b),
// read from the DC bin of Z, is added back where plane values are used:
// the plane then is the reference's raw plane.  Values are 4x scaled; ratios
// are unaffected and the pedestal is scaled to match.
//
// Certification: decisions whose margin is below an error bound of the
// FP32 plane (local-max tests, order of the two peaks, signs entering log
// and sn, conditioning of the fit and of sn) flag the window; flagged
// windows are re-decided by the exact double-precision kernel
// (piv_exact.cu), which overwrites their results.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "fft_reg.cuh"
#include "offsets.cuh"
#include "piv_kernels.h"

namespace opiv {
namespace fp32 {

constexpr int kWarps = 4;   // warps per CTA
// A window is decided by this kernel only if the error bound of its
// sub-pixel fit stays below kFitTol pixels and the relative error bound of
// its sn below kSnTol * (1 + sn).  The parity tolerances are 1e-4 px and
// 1e-5 * (1 + sn): sn = p0 / p1 is a ratio of plane values, and plane values
// are specified to 1e-5 of the plane peak p0, which bounds the relative
// error of p1 by 1e-5 * p0 / p1 = 1e-5 * sn.  The thresholds sit 1.6x inside
// those tolerances (the rounding of the final FP32 logarithms, sums and
// ratio adds ~1e-6 px and ~2e-7 relative on top of the bounds).  At 3e-5 /
// 3e-6 three times as many 16 px windows went to the exact pass, nearly all
// of them for the sn bound.
constexpr float kFitTol = 6e-5f;
constexpr float kSnTol = 6e-6f;
#define kNegInf (-__int_as_float(0x7f800000))
constexpr float kTwo23 = 8388608.0f;

// ---- pixel loading -----------------------------------------------------------
// Exact widening of 8/16-bit pixels: bits 0x4B000000 | u are the float
// 2^23 + u (u < 2^23); subtracting 2^23 is exact.
__device__ __forceinline__ float u16_lo(uint32_t w) { return __int_as_float(__byte_perm(w, 0x4B00, 0x5410)) - kTwo23; }
__device__ __forceinline__ float u16_hi(uint32_t w) { return __int_as_float(__byte_perm(w, 0x4B00, 0x5432)) - kTwo23; }
template <int K>
__device__ __forceinline__ float u8_k(uint32_t w) { return __int_as_float(__byte_perm(w, 0x4B00, 0x5440 | K)) - kTwo23; }

// W consecutive pixels starting at `ptr` into the x (A) or y (B) components
// of v.  VEC: the row start is 16-byte aligned.
template <bool B>
__device__ __forceinline__ void put(float2& z, float f)
{
    if (B) z.y = f;
    else z.x = f;
}

// Pixel x goes to register bitrev(x): the row transform takes bit-reversed
// input.
template <int W, bool B, typename PixT, bool VEC>
__device__ __forceinline__ void load_row(const PixT* ptr, float2 (&v)[W])
{
    if (VEC && sizeof(PixT) == 2) {
        const uint4* q = reinterpret_cast<const uint4*>(ptr);
#pragma unroll
        for (int k = 0; k < W / 8; ++k) {
            const uint4 r = __ldg(q + k);
            put<B>(v[bitrev<W>(8 * k + 0)], u16_lo(r.x)); put<B>(v[bitrev<W>(8 * k + 1)], u16_hi(r.x));
            put<B>(v[bitrev<W>(8 * k + 2)], u16_lo(r.y)); put<B>(v[bitrev<W>(8 * k + 3)], u16_hi(r.y));
            put<B>(v[bitrev<W>(8 * k + 4)], u16_lo(r.z)); put<B>(v[bitrev<W>(8 * k + 5)], u16_hi(r.z));
            put<B>(v[bitrev<W>(8 * k + 6)], u16_lo(r.w)); put<B>(v[bitrev<W>(8 * k + 7)], u16_hi(r.w));
        }
    } else if (VEC && sizeof(PixT) == 1) {
        const uint4* q = reinterpret_cast<const uint4*>(ptr);
#pragma unroll
        for (int k = 0; k < W / 16; ++k) {
            const uint4 r = __ldg(q + k);
            const uint32_t w4[4] = { r.x, r.y, r.z, r.w };
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                put<B>(v[bitrev<W>(16 * k + 4 * j + 0)], u8_k<0>(w4[j]));
                put<B>(v[bitrev<W>(16 * k + 4 * j + 1)], u8_k<1>(w4[j]));
                put<B>(v[bitrev<W>(16 * k + 4 * j + 2)], u8_k<2>(w4[j]));
                put<B>(v[bitrev<W>(16 * k + 4 * j + 3)], u8_k<3>(w4[j]));
            }
        }
    } else if (VEC && sizeof(PixT) == 4) {
        const float4* q = reinterpret_cast<const float4*>(ptr);
#pragma unroll
        for (int k = 0; k < W / 4; ++k) {
            const float4 r = __ldg(q + k);
            put<B>(v[bitrev<W>(4 * k + 0)], r.x); put<B>(v[bitrev<W>(4 * k + 1)], r.y);
            put<B>(v[bitrev<W>(4 * k + 2)], r.z); put<B>(v[bitrev<W>(4 * k + 3)], r.w);
        }
    } else {
#pragma unroll
        for (int x = 0; x < W; ++x) put<B>(v[bitrev<W>(x)], (float)__ldg(ptr + x));
    }
}

// A row that starts anywhere (B windows shifted by a previous pass's
// displacement): the 16-byte blocks covering it are loaded whole and the
// row is shifted out of them by the start's offset inside its block (a
// word select, then a byte permute).  The blocks read hold at least one
// pixel of the row each, so they lie inside the frame's allocation.
template <int W, bool B, typename PixT>
__device__ __forceinline__ void load_row_shifted(const PixT* ptr, float2 (&v)[W])
{
    if constexpr (sizeof(PixT) > 4) {   // double frames: element loads
#pragma unroll
        for (int x = 0; x < W; ++x) put<B>(v[bitrev<W>(x)], (float)__ldg(ptr + x));
    } else {
        constexpr int NW = W * (int)sizeof(PixT) / 4;   // 32-bit words of the row
        constexpr int NC = NW / 4;                      // whole blocks of the row
        const uintptr_t a = reinterpret_cast<uintptr_t>(ptr);
        const uint4* q = reinterpret_cast<const uint4*>(a & ~(uintptr_t)15);
        const int mis = (int)(a & 15);
        uint32_t w[NW + 4];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const uint4 r = __ldg(q + c);
            w[4 * c] = r.x; w[4 * c + 1] = r.y; w[4 * c + 2] = r.z; w[4 * c + 3] = r.w;
        }
        uint4 tail = make_uint4(0u, 0u, 0u, 0u);
        if (mis != 0) tail = __ldg(q + NC);   // only a misaligned row reaches into it
        w[NW] = tail.x; w[NW + 1] = tail.y; w[NW + 2] = tail.z; w[NW + 3] = tail.w;
        const int ws = mis >> 2;
        const uint32_t sel = 0x3210u + 0x1111u * (uint32_t)(mis & 3);
#pragma unroll
        for (int k = 0; k < NW + 2; ++k) w[k] = (ws & 2) ? w[k + 2] : w[k];
#pragma unroll
        for (int k = 0; k < NW + 1; ++k) w[k] = (ws & 1) ? w[k + 1] : w[k];
#pragma unroll
        for (int k = 0; k < NW; ++k) {
            const uint32_t u = __byte_perm(w[k], w[k + 1], sel);
            if constexpr (sizeof(PixT) == 2) {
                put<B>(v[bitrev<W>(2 * k)], u16_lo(u));
                put<B>(v[bitrev<W>(2 * k + 1)], u16_hi(u));
            } else if constexpr (sizeof(PixT) == 1) {
                put<B>(v[bitrev<W>(4 * k + 0)], u8_k<0>(u));
                put<B>(v[bitrev<W>(4 * k + 1)], u8_k<1>(u));
                put<B>(v[bitrev<W>(4 * k + 2)], u8_k<2>(u));
                put<B>(v[bitrev<W>(4 * k + 3)], u8_k<3>(u));
            } else {
                put<B>(v[bitrev<W>(k)], __uint_as_float(u));
            }
        }
    }
}

// Bottom-left corner of window w.  Window indices fit in 32 bits (plans
// hold at most 2^31 - 1 windows), so the grid position is a 32-bit division.
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

template <int W, typename T>
__device__ __forceinline__ T group_sum(T x)
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

// W x W tile with rows padded to W + 1 float2: row-wise and column-wise
// accesses by the W lanes of a group hit distinct banks.
template <int W>
__device__ __forceinline__ int tix(int r, int c) { return r * (W + 1) + c; }
// Hermitian half of a W x W spectrum: columns 0 .. W/2, rows padded.
template <int W>
__device__ __forceinline__ int hix(int r, int c) { return r * (W / 2 + 1) + c; }

// shared memory per lane group: transpose tile + half spectrum
template <int W>
__host__ __device__ constexpr int group_smem_float2() { return W * (W + 1) + W * (W / 2 + 1); }

// Transform stages of a pair, run by one runtime loop around one FFT body.
enum { kStLoad0 = 0, kStCol0 = 1, kStLoad1 = 2, kStCol1 = 3, kStInvA = 4, kStInvB = 5 };

// One task: the 2 * NG windows first = task * 2 * NG ... of pair p, run by
// the calling warp (its lane groups' shared memory at `dyn_smem`).
template <int W, int MODE, bool LIMIT, typename PixT, bool PLANES, bool VEC>
__device__ __forceinline__ void fp32_task(const PivParams& p, const int task, float2* dyn_smem)
{
    constexpr int NG = 32 / W;          // lane groups per warp
    constexpr int N = W * W;
    // peak scan range in swapped-plane coordinates (image_utils.impl.h:48,
    // :54; limited search: rect::dilate(0.5), rect.cpp:109-126)
    constexpr int D0 = LIMIT ? W / 4 : 0;
    constexpr int VW = LIMIT ? W / 2 : W;
    constexpr int SY0 = D0 + 1, SY1 = D0 + VW - 2;
    constexpr int SX0 = D0 + 1, SX1 = D0 + VW - 1;

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int grp = lane / W;
    const int gl = lane % W;
    const int first = task * 2 * NG;
    if (first >= (int)p.n_win) return;   // warp-uniform
    float2* S = dyn_smem + (warp * NG + grp) * group_smem_float2<W>();   // transpose tile
    float2* H = S + W * (W + 1);                                          // first product, half

    const PixT* fa = reinterpret_cast<const PixT*>(p.fa);
    const PixT* fb = reinterpret_cast<const PixT*>(p.fb);
    const size_t pitch = p.pitch / sizeof(PixT);

    float2 v[W];      // the transform being worked on
    float en0 = 0.f, en1 = 0.f, ped0 = 0.f, ped1 = 0.f;

#pragma unroll 1
    for (int st = 0; st < 6; ++st) {
        const int h = (st >= kStLoad1 && st <= kStCol1) ? 1 : 0;
        const int w = first + h * NG + grp;
        const bool valid = w < (int)p.n_win;
        // ---------------- before the transform
        if (st == kStLoad0 || st == kStLoad1) {
            // extract + widen: lane = row y, registers = x
            if (valid) {
                int bx, by, ox, oy;
                window_origin(p, w, bx, by);
                b_offset(p, W, bx, by, ox, oy);
                const size_t off = (size_t)(by + gl) * pitch + bx;
                load_row<W, false, PixT, VEC>(fa + off, v);
                if (p.prev_disp != nullptr)   // shifted B rows need not be aligned
                    load_row_shifted<W, true, PixT>(fb + (size_t)(by + oy + gl) * pitch + bx + ox, v);
                else
                    load_row<W, true, PixT, VEC>(fb + off, v);
                if (PLANES) {   // exact pedestal for the per-window API (double input)
                    double sa = 0.0, sb = 0.0;
#pragma unroll 4
                    for (int x = 0; x < W; ++x) {
                        sa += (double)fa[off + x];
                        sb += (double)fb[off + x];
                    }
                    sa = group_sum<W, double>(sa);
                    sb = group_sum<W, double>(sb);
                    if (gl == 0) p.peds[w] = (MODE == kModeComplex) ? sa * sb : 0.0;
                }
            } else {
#pragma unroll
                for (int x = 0; x < W; ++x) v[x] = make_float2(0.f, 0.f);
            }
            float e = 0.f;
#pragma unroll
            for (int x = 0; x < W; ++x) e = fmaf(v[x].x, v[x].x, fmaf(v[x].y, v[x].y, e));
            e = group_sum<W, float>(e);
            if (h == 0) en0 = e; else en1 = e;
        } else if (st == kStCol0 || st == kStCol1) {
            // v: lane = y, register kx.  Transpose to lane = kx, register
            // bitrev(y).  REAL mode: column kx = 0 of Z is zeroed here, so
            // lane 0's spectrum is zero.
#pragma unroll
            for (int kx = 0; kx < W; ++kx) {
                const float2 z = (MODE == kModeReal && kx == 0) ? make_float2(0.f, 0.f) : v[kx];
                S[tix<W>(kx, gl)] = z;
            }
            __syncwarp();
#pragma unroll
            for (int y = 0; y < W; ++y) v[bitrev<W>(y)] = S[tix<W>(gl, y)];
            __syncwarp();
        } else if (st == kStInvA) {
            // S holds Q at [ky][kx] (written by the second unpack).  To
            // lane = ky, register bitrev(kx).
#pragma unroll
            for (int x = 0; x < W; ++x) v[bitrev<W>(x)] = S[tix<W>(gl, x)];
            __syncwarp();
        } else {   // kStInvB
            // v: lane = ky, register x.  To lane = x, register bitrev(ky).
#pragma unroll
            for (int x = 0; x < W; ++x) S[tix<W>(x, gl)] = v[x];
            __syncwarp();
#pragma unroll
            for (int y = 0; y < W; ++y) v[bitrev<W>(y)] = S[tix<W>(gl, y)];
            __syncwarp();
        }

        fft_dit_fma<W, false>(v);

        // ---------------- after the transform
        if (st == kStCol0 || st == kStCol1) {
            // v: lane = kx, register ky.  DC bin = (sum a, sum b) on lane 0,
            // register 0.
            const float2 dc = make_float2(__shfl_sync(0xffffffffu, v[0].x, 0, W),
                                          __shfl_sync(0xffffffffu, v[0].y, 0, W));
            const float pd = (MODE == kModeComplex) ? 4.f * dc.x * dc.y : 0.f;
            if (h == 0) ped0 = pd; else ped1 = pd;
            if (MODE == kModeComplex && gl == 0) v[0] = make_float2(0.f, 0.f);
            if (MODE == kModeReal) {   // rows ky = 0 and ky = W/2
                v[0] = make_float2(0.f, 0.f);
                v[W / 2] = make_float2(0.f, 0.f);
            }
            const int pl = (W - gl) & (W - 1);
            // first window: its product goes to the half spectrum H (lanes
            // kx <= W/2); second window: lanes kx > W/2 take the first product
            // from the mirror (-ky, W - kx) of H, conjugated, and Q goes to S
            const bool mirror = gl > W / 2;
            const int hc = mirror ? W - gl : gl;
            const float sg = mirror ? -1.f : 1.f;
            const bool store_h = (h == 0) && !mirror;
#pragma unroll
            for (int ky = 0; ky < W; ++ky) {
                const int mky = (W - ky) & (W - 1);
                const float2 z = v[ky];
                const float zmx = __shfl_sync(0xffffffffu, v[mky].x, pl, W);
                const float zmy = __shfl_sync(0xffffffffu, v[mky].y, pl, W);
                // 4 conj(P) = ( 2 Im(Z Zm), |Z|^2 - |Zm|^2 )
                const float im2 = 2.f * fmaf(z.x, zmy, z.y * zmx);
                const float d = fmaf(z.x, z.x, fmaf(z.y, z.y, -fmaf(zmx, zmx, zmy * zmy)));
                if (store_h) H[hix<W>(ky, gl)] = make_float2(im2, d);
                if (h == 1) {
                    // Q = conj(4 P1) + i conj(4 P2), stored at [ky][kx]
                    const float2 c1 = H[hix<W>(mirror ? mky : ky, hc)];
                    S[tix<W>(ky, gl)] = make_float2(c1.x - d, fmaf(sg, c1.y, im2));
                }
            }
            __syncwarp();
        }
    }
    // v: lane = x, register y; v.x = plane of the first window of the pair,
    // v.y of the second (4x scaled, pedestal removed).

    const float dlt = p.kappa * 5.9604645e-8f * 2.f * (float)N * (en0 + en1);
    const int xs = (gl + W / 2) & (W - 1);          // swapped column of this lane
    const bool col_ok = xs >= SX0 && xs < SX1;

#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
        const int w = first + h * NG + grp;
        const bool valid = w < (int)p.n_win;
        if (h == 1) {                                // the second plane into .x
#pragma unroll
            for (int i = 0; i < W; ++i) v[i].x = v[i].y;
        }

        // plane rows y into shared memory (row-major, padded) for the fit
#pragma unroll
        for (int y = 0; y < W; ++y) S[tix<W>(y, gl)].x = v[y].x;
        if (PLANES && valid) {
#pragma unroll
            for (int y = 0; y < W; ++y) {
                const int ys = (y + W / 2) & (W - 1);
                p.planes[(size_t)w * N + ys * W + xs] = 0.25f * v[y].x;
            }
        }

        // ---- find_peaks: strict 4-neighbour maxima, top two
        float t0 = kNegInf, t1 = kNegInf, umax = kNegInf;
        int t0y = 0;
#pragma unroll
        for (int ys = SY0; ys < SY1; ++ys) {
            const int y = (ys + W / 2) & (W - 1);
            const float c = v[y].x;
            const float up = v[(y + W - 1) & (W - 1)].x;
            const float dn = v[(y + 1) & (W - 1)].x;
            const float lf = __shfl_sync(0xffffffffu, c, (gl + W - 1) & (W - 1), W);
            const float rt = __shfl_sync(0xffffffffu, c, (gl + 1) & (W - 1), W);
            float m4;   // max of the four neighbours (a three-source max and a max)
            asm("max.f32 %0, %1, %2, %3;" : "=f"(m4) : "f"(up), "f"(dn), "f"(fmaxf(lf, rt)));
            const float dd = m4 - c;
            const bool strict = col_ok && (dd < 0.f);
            const bool unc = col_ok && (fabsf(dd) <= dlt);
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
        __syncwarp();

        // ---- fit_simple_gaussian: the six logarithms on six lanes
        const int px = key % W, py = key / W;       // swapped-plane coordinates
        const int ux = (px + W / 2) & (W - 1), uy = (py + W / 2) & (W - 1);
        const float ped = h ? ped1 : ped0;
        const float vc = S[tix<W>(uy, ux)].x;
        const float vl = S[tix<W>(uy, (ux + W - 1) & (W - 1))].x;
        const float vr = S[tix<W>(uy, (ux + 1) & (W - 1))].x;
        const float vu = S[tix<W>((uy + W - 1) & (W - 1), ux)].x;
        const float vd = S[tix<W>((uy + 1) & (W - 1), ux)].x;
        __syncwarp();
        // axis x: ln(L/R), ln(L/C), ln(R/C); axis y: ln(U/D), ln(U/C), ln(D/C)
        // with L = vl + ped etc., each as log1p((num - den) / (den + ped))
        const int j = gl < 6 ? gl : 0;
        const float an = j == 0 ? vl : j == 1 ? vl : j == 2 ? vr : j == 3 ? vu : j == 4 ? vu : vd;
        const float ad = j == 0 ? vr : j == 1 ? vc : j == 2 ? vc : j == 3 ? vd : vc;
        const float lg = log1pf((an - ad) / (ad + ped));
        const float lxr = __shfl_sync(0xffffffffu, lg, 0, W);
        const float lxl = __shfl_sync(0xffffffffu, lg, 1, W);
        const float lxrr = __shfl_sync(0xffffffffu, lg, 2, W);
        const float lyd = __shfl_sync(0xffffffffu, lg, 3, W);
        const float lyu = __shfl_sync(0xffffffffu, lg, 4, W);
        const float lydd = __shfl_sync(0xffffffffu, lg, 5, W);

        if (valid && gl == 0) {
            const bool has2 = t1 > kNegInf;
            bool certain;
            opiv_vector out{ 0.f, 0.f, 0.f, 0.f, 0.f };
            int32_t code = -1;
            int bx, by, ox, oy;
            window_origin(p, w, bx, by);
            b_offset(p, W, bx, by, ox, oy);
            if (!has2) {
                certain = !(umax > kNegInf);
            } else {
                const float C = vc + ped, L = vl + ped, R = vr + ped, U = vu + ped, D = vd + ped;
                const float nan = __int_as_float(0x7fffffff);
                // (ln L - ln R) / (2 (ln L + ln R - 2 ln C)), NaN where the
                // reference takes the log of a non-positive value
                const float denx = lxl + lxrr, deny = lyu + lydd;
                const bool okx = L > 0.f && C > 0.f && R > 0.f;
                const bool oky = U > 0.f && C > 0.f && D > 0.f;
                const float fx = okx ? lxr / (2.f * denx) : nan;
                const float fy = oky ? lyd / (2.f * deny) : nan;
                // error bound of each axis for an error dlt/2 per value; a
                // NaN outcome is certain only if a value is clearly negative
                const float mx = fminf(fminf(L, R), C), my = fminf(fminf(U, D), C);
                const float ex = okx ? (denx == 0.f ? 3.4e38f
                                        : dlt * (1.f + 4.f * fabsf(fx)) / (mx * 2.f * fabsf(denx)))
                                     : (mx < -dlt ? 0.f : 3.4e38f);
                const float ey = oky ? (deny == 0.f ? 3.4e38f
                                        : dlt * (1.f + 4.f * fabsf(fy)) / (my * 2.f * fabsf(deny)))
                                     : (my < -dlt ? 0.f : 3.4e38f);
                const float p0 = t0 + ped, p1 = t1 + ped;
                // sn = p0 / p1 when p1 > 0: relative error <= e/|p0| + e/|p1|
                // with e = dlt / 2 the error of one plane value
                const float sn_err = 0.5f * dlt * (1.f / fabsf(p0) + 1.f / fabsf(p1));
                certain = (umax < t1 - 2.f * dlt) && (t0 - t1 > dlt) && (fabsf(p1) > dlt) &&
                          (ex < kFitTol) && (ey < kFitTol) &&
                          (p1 <= 0.f || sn_err < kSnTol * (1.f + p0 / p1));
                out.x = (float)(bx + W / 2);
                out.y = (float)(p.img_h - (by + W / 2));
                out.u = (float)(W / 2 - px - ox) - fx;
                out.v = (float)(W / 2 - py - oy) - fy;
                out.sn = (p1 > 0.f) ? p0 / p1 : 0.f;
                code = key;
            }
            p.out_vec[w] = out;
            if (p.out_peak) p.out_peak[w] = code;
            if (p.out_disp)
                p.out_disp[w] = has2 ? pack_disp(px - W / 2 + ox, py - W / 2 + oy) : pack_disp(ox, oy);
            if (!certain && p.flag_list) {
                const unsigned int slot = atomicAdd(p.flag_count, 1u);
                p.flag_list[slot] = (int32_t)w + p.flag_base;
            }
        }
    }
}

extern __shared__ float2 fp32_dyn_smem[];

// resident CTAs per SM the register budget is set for: a 16 px window's
// transform needs half the registers of a 32 px one
template <int W>
constexpr int min_ctas() { return W == 16 ? 6 : 4; }

template <int W, int MODE, bool LIMIT, typename PixT, bool PLANES, bool VEC>
__global__ void __launch_bounds__(32 * kWarps, min_ctas<W>())
piv_fp32_kernel(const PivParams p)
{
    fp32_task<W, MODE, LIMIT, PixT, PLANES, VEC>(p, (int)blockIdx.x * kWarps + (int)(threadIdx.x >> 5),
                                                 fp32_dyn_smem);
}

// Copies pair j's descriptor from global memory into `dst` (shared) with
// the lanes of one warp; the warp's lanes then read it from there.
__device__ __forceinline__ const PivParams& warp_item(const PivQueue& q, int j, PivParams* dst)
{
    constexpr int NQ = (int)(sizeof(PivParams) / 16);
    const uint4* src = reinterpret_cast<const uint4*>(q.items_g + j);
    uint4* d = reinterpret_cast<uint4*>(dst);
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < NQ; i += 32) d[i] = __ldg(src + i);
    __syncwarp();
    return *dst;
}

// Persistent form over a device work queue: each CTA takes kWarps * q.chunk
// consecutive tasks at a time, its warps interleaved over them (so that, as
// in the single-pair kernel, the warps of a CTA work on neighbouring
// windows, which share image rows in L1), until the pass's tasks (every
// pair's) run out.  The next chunk is claimed while the current one runs
// (thread 0 keeps the atomic's result in a register until the next
// barrier), so no CTA stalls on the counter.  No CTA waits for another.
template <int W, int MODE, bool LIMIT, typename PixT, bool VEC>
__global__ void __launch_bounds__(32 * kWarps, min_ctas<W>())
piv_fp32_queue_kernel(const __grid_constant__ PivQueue q)
{
    __shared__ unsigned int s_t0;
    __shared__ __align__(16) unsigned char s_items[kWarps * sizeof(PivParams)];
    const int warp = threadIdx.x >> 5;
    PivParams* my_item = reinterpret_cast<PivParams*>(s_items) + warp;
    const int n_tasks = q.first_task[q.n_items];
    const int step = kWarps * q.chunk;
    unsigned int next = 0;
    if (threadIdx.x == 0) next = atomicAdd(q.head, (unsigned int)step);
#pragma unroll 1
    for (;;) {
        if (threadIdx.x == 0) s_t0 = next;
        __syncthreads();
        const unsigned int t0 = s_t0;
        __syncthreads();   // every thread has read s_t0 before it is written again
        if (t0 >= (unsigned int)n_tasks) break;
        if (threadIdx.x == 0) next = atomicAdd(q.head, (unsigned int)step);
        const int t1 = min((int)t0 + step, n_tasks);
#pragma unroll 1
        for (int t = (int)t0 + warp; t < t1; t += kWarps) {
            const int j = __ldg(q.task_item + t);
            const PivParams& p = warp_item(q, j, my_item);
            fp32_task<W, MODE, LIMIT, PixT, false, VEC>(p, t - q.first_task[j], fp32_dyn_smem);
            __syncwarp();   // the descriptor is overwritten by the next task
        }
    }
}

template <int W, int MODE, bool LIMIT, typename PixT, bool PLANES>
cudaError_t launch_t(const PivParams& p, cudaStream_t s)
{
    constexpr int NG = 32 / W;
    const int64_t tasks = (p.n_win + 2 * NG - 1) / (2 * NG);
    const int64_t blocks = (tasks + kWarps - 1) / kWarps;
    const size_t px = sizeof(PixT);
    // 128-bit loads when every window row starts on a 16-byte boundary
    const bool vec = p.win_xy == nullptr && ((uintptr_t)p.fa % 16 == 0) &&
                     ((uintptr_t)p.fb % 16 == 0) && (p.pitch % 16 == 0) &&
                     (((size_t)p.gx0 * px) % 16 == 0) && (((size_t)p.gdx * px) % 16 == 0) &&
                     ((W * px) % 16 == 0);
    const size_t smem = sizeof(float2) * kWarps * NG * group_smem_float2<W>();
    auto kern = vec ? piv_fp32_kernel<W, MODE, LIMIT, PixT, PLANES, true>
                    : piv_fp32_kernel<W, MODE, LIMIT, PixT, PLANES, false>;
    // per instantiation, load path and device
    static std::atomic<uint64_t> attr_done[2] = { { 0 }, { 0 } };
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(attr_done[vec].load() & bit)) {
        const cudaError_t e =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_done[vec].fetch_or(bit);
    }
    kern<<<(unsigned)blocks, 32 * kWarps, smem, s>>>(p);
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

// The same work list dispatched by the hardware: CTA b runs tasks
// kWarps * b ... (one per warp), no persistent loop.
template <int W, int MODE, bool LIMIT, typename PixT, bool VEC>
__global__ void __launch_bounds__(32 * kWarps, min_ctas<W>())
piv_fp32_list_kernel(const __grid_constant__ PivQueue q)
{
    __shared__ __align__(16) unsigned char s_items[kWarps * sizeof(PivParams)];
    const int warp = threadIdx.x >> 5;
    const int t = (int)blockIdx.x * kWarps + warp;
    if (t >= q.first_task[q.n_items]) return;   // warp-uniform
    const int j = __ldg(q.task_item + t);
    const PivParams& p = warp_item(q, j, reinterpret_cast<PivParams*>(s_items) + warp);
    fp32_task<W, MODE, LIMIT, PixT, false, VEC>(p, t - q.first_task[j], fp32_dyn_smem);
}

// ---- the persistent queue form ------------------------------------------------
// blocks > 0: the persistent kernel on `blocks` CTAs; blocks == 0: the
// hardware-dispatched list kernel, one CTA per kWarps tasks
template <int W, int MODE, bool LIMIT, typename PixT, bool VEC>
cudaError_t queue_t(const PivQueue& q, int blocks, int* max_ctas, cudaStream_t s)
{
    constexpr int NG = 32 / W;
    const size_t smem = sizeof(float2) * kWarps * NG * group_smem_float2<W>();
    auto kern = piv_fp32_queue_kernel<W, MODE, LIMIT, PixT, VEC>;
    auto list = piv_fp32_list_kernel<W, MODE, LIMIT, PixT, VEC>;
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
    if (max_ctas) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(max_ctas, kern, 32 * kWarps, smem);
    if (blocks < 0) return cudaErrorInvalidValue;
    if (blocks == 0) {
        const int n_tasks = q.first_task[q.n_items];
        if (n_tasks <= 0) return cudaSuccess;
        list<<<(unsigned)((n_tasks + kWarps - 1) / kWarps), 32 * kWarps, smem, s>>>(q);
    } else {
        kern<<<(unsigned)blocks, 32 * kWarps, smem, s>>>(q);
    }
    return cudaGetLastError();
}

template <int W, int MODE, bool LIMIT>
cudaError_t queue_dt(const PivQueue& q, int dtype, bool vec, int blocks, int* max_ctas, cudaStream_t s)
{
    switch (dtype) {
    case kU8: return vec ? queue_t<W, MODE, LIMIT, uint8_t, true>(q, blocks, max_ctas, s)
                         : queue_t<W, MODE, LIMIT, uint8_t, false>(q, blocks, max_ctas, s);
    case kU16: return vec ? queue_t<W, MODE, LIMIT, uint16_t, true>(q, blocks, max_ctas, s)
                          : queue_t<W, MODE, LIMIT, uint16_t, false>(q, blocks, max_ctas, s);
    case kF32: return vec ? queue_t<W, MODE, LIMIT, float, true>(q, blocks, max_ctas, s)
                          : queue_t<W, MODE, LIMIT, float, false>(q, blocks, max_ctas, s);
    default: return cudaErrorInvalidValue;
    }
}

// Launches the queue kernel (max_ctas null) or reports its resident CTAs
// per SM in *max_ctas (nothing launched).
template <int W>
cudaError_t queue_w(const PivQueue& q, int dtype, int mode, int limit, bool vec, int blocks,
                    int* max_ctas, cudaStream_t s)
{
    if (mode == kModeComplex)
        return limit ? queue_dt<W, kModeComplex, true>(q, dtype, vec, blocks, max_ctas, s)
                     : queue_dt<W, kModeComplex, false>(q, dtype, vec, blocks, max_ctas, s);
    return limit ? queue_dt<W, kModeReal, true>(q, dtype, vec, blocks, max_ctas, s)
                 : queue_dt<W, kModeReal, false>(q, dtype, vec, blocks, max_ctas, s);
}

}  // namespace fp32
}  // namespace opiv
