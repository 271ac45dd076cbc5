// Tensor-core (tcgen05) PIV window path for 16 and 64 px windows on the
// grids that the dedicated kernels do not take: the same chain of four DFT
// matrix products as the 32 px kernel (piv_tc_kernel.cuh), written once for
// any window size W that is a multiple of 16 (a DFT matrix needs no power
// of two), without that kernel's 32 px specialisations.  Instantiated per
// size in piv_tcg_w16.cu and piv_tcg_w64.cu.
//
// Mathematics (a, b: the two windows, rows y, columns x, H = W / 2; all
// transforms unnormalised like FFT::cross_correlate, fft.h:188-206):
//   stage 1  row DFT, H1 = X * G1^T with G1 rows: cos(2 pi n x / W) for
//            n < H, (-1)^x for n = H, sin(2 pi (n - H) x / W) for n > H;
//   stage 2  column DFT over y of U_k - i V_k (k < H; the slot k = 0
//            carries U_0 - i U_H), K = (U | V) x y against [C; S] and
//            [-S; C]: columns Re Z and -Im Z;
//   product  P = B conj(A) on k_x = 0..H (the slot k = 0 unpacked by
//            Hermitian symmetry and packed again as P(k_y, 0) + i P(k_y, H)),
//            DC removed (the pedestal sum(a) sum(b) is added back in the
//            fit), (-1)^k_y for the row quadrant swap, REAL mode's zeroed
//            spectrum row 0, row H and column 0 (fft.h:166-183);
//   stage 3  inverse column DFT over k_y, K = (Re | Im) x k_y;
//   stage 4  real inverse row DFT (c2r) over k_x with the weights 1 / 2 / 1
//            and the column quadrant swap folded into the constant matrix.
// Then find_peaks(plane, 2, 1) (image_utils.impl.h:42-74), the 3-point
// Gaussian fit (impl:77-101) and the vector (main.cpp:220-236).
//
// A CTA of 4 warps takes tiles of 128 / W windows of one grid row (eight
// 16 px or two 64 px windows).  Operands: shared memory, no-swizzle canonical layouts, hi and
// lo parts for split precision; accumulators in tensor memory.  Rows of
// the first product's M tiles, the second's and the fourth's follow the
// thread index; the third product has M = 64 (row r in lane
// 32 (r / 16) + r % 16).  Frame a's spectrum rows reach frame b's threads
// through shared memory in FP32.
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "piv_kernels.h"
#include "piv_tc_kernel.cuh"
#include "tc_ptx.cuh"

namespace opiv {
namespace tcg {

using tc::Raw;
using tc::load_raw;
using tc::round8;
using tc::split8;
using tc::widen8;

constexpr int kThreads = 128;

// CSPLIT: the constants' lo parts are used (and held in shared memory)
template <int W, bool SPLIT, bool CSPLIT = SPLIT>
struct Geo {
    static constexpr int H = W / 2;
    static constexpr int WPM = W <= 64 && 64 % W == 0 ? 64 / W : 1;   // windows per stage-1 M tile
    static constexpr int WPT = 2 * WPM;                               // windows per tile
    static constexpr int R1 = WPM * 2 * W;    // used rows of a stage-1 M tile
    static constexpr int R2 = WPT * W;        // used rows of the stage-2 and stage-4 products
    static constexpr int R3 = WPT * H;        // used rows of the stage-3 product (M = 64)
    static constexpr int KS = W / 16;         // 16-deep MMA steps over a W-long K
    static constexpr int kMat = W * W * 2;    // one W x W 16-bit matrix, K-major
    static constexpr int kSet = kTcNumMat * kMat;
    static constexpr int kParts = SPLIT ? 2 : 1;          // data operand parts
    static constexpr int kCParts = CSPLIT ? 2 : 1;        // constant parts
    static constexpr int kOp = 512 * W;       // largest operand (hi part), bytes
    static constexpr int PS = W + 1;          // plane row stride (floats)
    static constexpr int XS = 2 * W + 1;      // exchange row stride (floats), odd
    static constexpr int kXch = 4 * (R3 + WPT) * XS;
    static constexpr int kPlane = 4 * R2 * PS;
    static constexpr int kScratch = ((kXch > kPlane ? kXch : kPlane) + 127) / 128 * 128;
    static constexpr int kTail = 256;
    static constexpr int kSmem = kCParts * kSet + kParts * kOp + kScratch + kTail;
    static constexpr uint32_t kTmemCols = 2 * W <= 32 ? 32 : (2 * W <= 64 ? 64 : 128);
    static_assert(W % 16 == 0 && W >= 16 && W <= 64, "window size");
    static_assert(R1 <= 128 && R2 <= 128 && R3 <= 64, "tile rows");
};

// 8 values into one 16-byte core-matrix row (hi, and lo at +lo)
template <bool F16, bool SPLIT>
__device__ __forceinline__ void put8(unsigned char* base, int off, int lo, const float* v)
{
    if (SPLIT) {
        uint4 h, l;
        split8<F16>(v, h, l);
        *reinterpret_cast<uint4*>(base + off) = h;
        *reinterpret_cast<uint4*>(base + lo + off) = l;
    } else {
        *reinterpret_cast<uint4*>(base + off) = round8<F16>(v);
    }
}

// D (+)= A * B, split: hi*hi, hi*lo (CSPLIT: the constant's lo part),
// lo*hi (a, b: descriptors of the hi parts; the lo parts lie alo / blo
// bytes further)
template <bool SPLIT, bool CSPLIT>
__device__ __forceinline__ void mma3(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, bool acc,
                                     int alo, int blo)
{
    tcx::mma_bf16(d, a, b, idesc, acc);
    if (SPLIT) {
        if (CSPLIT) tcx::mma_bf16(d, a, b + (uint64_t)(blo >> 4), idesc, true);
        tcx::mma_bf16(d, a + (uint64_t)(alo >> 4), b, idesc, true);
    }
}

// 8 pixels starting anywhere: one raw load when the start is aligned to
// their size, else the 16-byte blocks covering them (each holds at least one
// of the pixels) shifted by the start's offset (word select, byte permute)
template <typename PixT>
__device__ __forceinline__ typename Raw<PixT>::type load_any(const PixT* ptr)
{
    constexpr int NB = 8 * (int)sizeof(PixT);   // bytes of the 8 pixels
    const uintptr_t a = reinterpret_cast<uintptr_t>(ptr);
    if ((a & (uintptr_t)(NB - 1)) == 0) return load_raw<PixT>(ptr);
    const uint4* q = reinterpret_cast<const uint4*>(a & ~(uintptr_t)15);
    const int mis = (int)(a & 15);
    const uint4 b0 = __ldg(q);
    uint4 b1 = make_uint4(0u, 0u, 0u, 0u);
    if (mis + NB > 16) b1 = __ldg(q + 1);
    uint32_t w[8] = { b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w };
    const int ws = mis >> 2;
    const uint32_t sel = 0x3210u + 0x1111u * (uint32_t)(mis & 3);
#pragma unroll
    for (int k = 0; k < 6; ++k) w[k] = (ws & 2) ? w[k + 2] : w[k];
#pragma unroll
    for (int k = 0; k < 5; ++k) w[k] = (ws & 1) ? w[k + 1] : w[k];
    typename Raw<PixT>::type r;
    if constexpr (sizeof(PixT) == 2) {
        r = make_uint4(__byte_perm(w[0], w[1], sel), __byte_perm(w[1], w[2], sel), __byte_perm(w[2], w[3], sel),
                       __byte_perm(w[3], w[4], sel));
    } else {
        r = make_uint2(__byte_perm(w[0], w[1], sel), __byte_perm(w[1], w[2], sel));
    }
    return r;
}

// 16 * N consecutive accumulator columns of this thread's lane
template <int N>
__device__ __forceinline__ void tld(uint32_t taddr, float* v)
{
#pragma unroll
    for (int i = 0; i < N; ++i) tcx::tmem_ld16(taddr + 16 * i, v + 16 * i);
}

template <int W, bool F16, bool SPLIT, bool CSPLIT, typename PixT>
__global__ void __launch_bounds__(kThreads)
piv_tcg_kernel(const PivParams p, const uint4* __restrict__ consts, int mode, int limit)
{
    using G = Geo<W, SPLIT, CSPLIT>;
    constexpr int H = G::H, WPM = G::WPM, WPT = G::WPT, KS = G::KS;
    constexpr float kPix = F16 ? 0.0625f : 1.f;
    constexpr float kT = F16 ? 0.015625f : 1.f;
    constexpr float kSumUnscale = F16 ? 8192.f : 1.f;
    constexpr uint32_t kId1 = tcx::idesc_f16kind(128, W, false, F16);
    constexpr uint32_t kId2 = tcx::idesc_f16kind(128, 2 * W, true, F16);
    constexpr uint32_t kId3 = tcx::idesc_f16kind(64, 2 * W, false, F16);
    constexpr uint32_t kId4 = tcx::idesc_f16kind(128, W, true, F16);
    const bool real = mode == kModeReal;
    // peak scan range in swapped-plane coordinates (image_utils.impl.h:48,
    // :54; limited search: rect::dilate(0.5), rect.cpp:109-126)
    const int D0 = limit ? W / 4 : 0, VW = limit ? W / 2 : W;
    const int SY0 = D0 + 1, SY1 = D0 + VW - 2, SX0 = D0 + 1, SX1 = D0 + VW - 1;

    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* cst = smem;
    unsigned char* dat = smem + G::kCParts * G::kSet;
    float* xch = reinterpret_cast<float*>(dat + G::kParts * G::kOp);   // exchange rows, then planes
    // pixel sums [window][frame] as exact integers (row sums are exact FP32
    // accumulator values for integer pixels; window sums reach 2^28)
    int* sums = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(xch) + G::kScratch);
    int2* org = reinterpret_cast<int2*>(sums + 2 * WPT);
    int* gwi = reinterpret_cast<int*>(org + WPT);
    unsigned* wmax = reinterpret_cast<unsigned*>(gwi + WPT);
    int* escale = reinterpret_cast<int*>(wmax + WPT);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(escale + WPT + (WPT & 1));
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
    int* abort_flag = reinterpret_cast<int*>(tslot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t cst_a = tcx::smem_addr(cst), dat_a = tcx::smem_addr(dat);
    const uint64_t dB = tcx::sdesc(cst_a, 128, 16 * W);
    auto mat = [&](int m, int ks) { return dB + (uint64_t)((m * G::kMat + ks * 256) >> 4); };
    const uint64_t dK1 = tcx::sdesc(dat_a, 128, 16 * W);   // K-major, K = W
    const uint64_t dMN = tcx::sdesc(dat_a, 2048, 128);     // MN-major, M = 128
    const uint64_t dK3 = tcx::sdesc(dat_a, 128, 32 * W);   // K-major, K = 2W
    auto off = [](int bytes) { return (uint64_t)(bytes >> 4); };
    const int clo = G::kSet, dlo = G::kOp;

    for (int i = tid; i < G::kCParts * G::kSet / 16; i += kThreads)
        reinterpret_cast<uint4*>(cst)[i] = consts[i];
    if (tid == 0) {
        tcx::mbar_init(mbar, 1);
        *abort_flag = 0;
    }
    if (warp == 0) tcx::tmem_alloc(tslot, G::kTmemCols);
    tcx::fence_before();
    __syncthreads();
    tcx::fence_after();
    const uint32_t tbase = *tslot;
    const uint32_t tlane = tbase + ((uint32_t)(32 * warp) << 16);

    const PixT* fa = reinterpret_cast<const PixT*>(p.fa);
    const PixT* fb = reinterpret_cast<const PixT*>(p.fb);
    const size_t pitch = p.pitch / sizeof(PixT);
    const int gny = (int)(p.n_win / p.gnx);
    const int per_row = (p.gnx + WPT - 1) / WPT;
    const int n_tiles = gny * per_row;
    uint32_t phase = 0;
    auto wait_mma = [&]() {
        if (!tcx::mbar_wait(mbar, phase)) {
            *abort_flag = 1;
            if (p.status) atomicExch(p.status, 1);
        }
        phase ^= 1u;
        tcx::fence_after();
    };

    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        if (tid < WPT) {
            const int row = tile / per_row, col = WPT * (tile - row * per_row) + tid;
            const bool ok = col < p.gnx;
            org[tid] = ok ? make_int2(p.gx0 + col * p.gdx, p.gy0 + row * p.gdy) : make_int2(-1, -1);
            gwi[tid] = row * p.gnx + col;
            sums[2 * tid] = 0;
            sums[2 * tid + 1] = 0;
            wmax[tid] = 0u;
        }
        __syncthreads();

        // ---- stage-1 operand: rows r = m1 * 128 + (wl, f, y), K-major,
        // K = x.  Item i is the 16-byte chunk at byte 16 i: row group i / 8
        // of the chunk column, row i & 7.
#pragma unroll 4
        for (int i = tid; i < 32 * W; i += kThreads) {
            const int r = ((i >> 3) / (W / 8)) * 8 + (i & 7), g = (i >> 3) % (W / 8);
            const int m1 = r >> 7, rl = r & 127;
            const int wl = rl / (2 * W), f = (rl / W) & 1, y = rl % W;
            const int2 o = rl < G::R1 ? org[m1 * WPM + wl] : make_int2(-1, -1);
            typename Raw<PixT>::type raw = Raw<PixT>::zero();
            if (o.x >= 0) raw = load_any<PixT>((f ? fb : fa) + (size_t)(o.y + y) * pitch + o.x + 8 * g);
            float px[8];
            widen8<PixT>(raw, px, kPix);
            put8<F16, SPLIT>(dat, 16 * i, dlo, px);
        }
        tcx::fence_proxy();
        tcx::fence_before();
        __syncthreads();
        if (*abort_flag) break;

        // ---- stage 1: H1 = X * G1^T, two M tiles
        if (tid == 0) {
            tcx::fence_after();
#pragma unroll
            for (int m1 = 0; m1 < 2; ++m1)
#pragma unroll
                for (int ks = 0; ks < KS; ++ks)
                    mma3<SPLIT, CSPLIT>(tbase + m1 * W, dK1 + off(m1 * 256 * W + ks * 256), mat(kTcG1, ks), kId1,
                                ks > 0, dlo, clo);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E1: stage-2 operand, MN-major, rows (window, frame, k) = 128,
        // K = (U | V) x y; window sums from the k = 0 column
#pragma unroll 1
        for (int m1 = 0; m1 < 2; ++m1) {
            float c[W];
            tld<W / 16>(tlane + m1 * W, c);
            const int rl = tid;
            const bool ok = rl < G::R1;
            const int wl = rl / (2 * W), f = (rl / W) & 1, y = rl % W;
            const int wi = m1 * WPM + wl;
            int s = __float2int_rn(c[0] * kSumUnscale);
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (ok && (lane & 15) == 0) atomicAdd(&sums[2 * wi + f], s);
            if (ok) {
#pragma unroll
                for (int g8 = 0; g8 < W / 8; ++g8) {
                    const int part = (8 * g8) / H, j = 8 * g8 - part * H;
                    const int k = part * W + y, m0 = (wi * 2 + f) * H + j;
                    put8<F16, SPLIT>(dat, ((k >> 3) * 16 + (m0 >> 3)) * 128 + (k & 7) * 16, dlo, c + 8 * g8);
                }
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        __syncthreads();

        // ---- stage 2: Re Z = U C - V S, -Im Z = U S + V C
        if (tid == 0) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 2 * KS; ++ks)
                mma3<SPLIT, CSPLIT>(tbase, dMN + off(ks * 4096), ks < KS ? mat(kTcC, ks) : mat(kTcNS, ks - KS), kId2,
                            ks > 0, dlo, clo);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E2: products into the stage-3 operand (K-major, rows
        // (window, k_x) = 64, K = (Re | Im) x k_y)
        {
            const int r = tid;
            const bool ok = r < G::R2;
            const int wi = r / W, f = (r / H) & 1, kx = r % H;
            float* xa = xch + (wi * H + kx) * G::XS;            // frame a's row of this (window, k_x)
            float* xp = xch + (G::R3 + wi) * G::XS;             // frame b's slot-0 row of the window
            // frame a's rows, and frame b's slot-0 rows, into shared memory
#pragma unroll 1
            for (int c0 = 0; c0 < 2 * W; c0 += 16) {
                float v[16];
                tcx::tmem_ld16(tlane + c0, v);
                float* dst = (f == 0) ? xa : xp;
                if (ok && (f == 0 || kx == 0)) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) dst[c0 + i] = v[i];
                }
            }
            __syncthreads();
            const bool prod = ok && f == 1;
            const int m3 = wi * H + kx;
            // the product of (k_y, this k_x), quadrant sign and REAL-mode zeros
            auto product = [&](int ky, float rb, float nb, float& pr, float& pi) {
                const float ra = xa[ky], na = xa[W + ky];
                pr = fmaf(rb, ra, nb * na);
                pi = fmaf(rb, na, -(nb * ra));
                if (real && (ky == 0 || ky == H)) { pr = 0.f; pi = 0.f; }
                if (ky & 1) { pr = -pr; pi = -pi; }
            };
            // the packed slot: P(k_y, 0) + i P(k_y, H) from Z' = U_0 - i U_H
            // of both frames (Z' stored as Re and -Im)
            auto packed = [&](int ky, float& pr, float& pi) {
                const int mk = ky == 0 ? 0 : W - ky;   // -k_y
                const float zar = xa[ky], zai = -xa[W + ky], zanr = xa[mk], zani = -xa[W + mk];
                const float zbr = xp[ky], zbi = -xp[W + ky], zbnr = xp[mk], zbni = -xp[W + mk];
                const float a0r = 0.5f * (zar + zanr), a0i = 0.5f * (zai - zani);
                const float a6r = -0.5f * (zai + zani), a6i = 0.5f * (zar - zanr);
                const float b0r = 0.5f * (zbr + zbnr), b0i = 0.5f * (zbi - zbni);
                const float b6r = -0.5f * (zbi + zbni), b6i = 0.5f * (zbr - zbnr);
                float p0r = b0r * a0r + b0i * a0i, p0i = b0i * a0r - b0r * a0i;
                float p6r = b6r * a6r + b6i * a6i, p6i = b6i * a6r - b6r * a6i;
                if (real) {
                    p0r = 0.f; p0i = 0.f;
                    if (ky == 0 || ky == H) { p6r = 0.f; p6i = 0.f; }
                } else if (ky == 0) {
                    p0r = 0.f; p0i = 0.f;   // pedestal removed
                }
                pr = p0r - p6i;
                pi = p0i + p6r;
                if (ky & 1) { pr = -pr; pi = -pi; }
            };
            // F16: the window's largest product first (scale 2^-e puts it in
            // [2^8, 2^9): the stage-3 sums stay inside FP16 after 2^-6)
            float sc = 1.f;
            if (F16) {
                float m = 0.f;
#pragma unroll 1
                for (int c0 = 0; c0 < W; c0 += 16) {
                    float vr[16], vn[16];
                    tcx::tmem_ld16(tlane + c0, vr);
                    tcx::tmem_ld16(tlane + W + c0, vn);
                    if (prod) {
#pragma unroll
                        for (int i = 0; i < 16; ++i) {
                            float pr, pi;
                            if (kx == 0) packed(c0 + i, pr, pi);
                            else product(c0 + i, vr[i], vn[i], pr, pi);
                            m = fmaxf(m, fmaxf(fabsf(pr), fabsf(pi)));
                        }
                    }
                }
                if (prod) atomicMax(&wmax[wi], __float_as_uint(m));
                __syncthreads();
                if (ok) {
                    const int eb = (int)((wmax[wi] >> 23) & 0xffu);
                    int e = eb == 0 ? 0 : eb - 127 - 8;
                    e = e < -90 ? -90 : (e > 80 ? 80 : e);
                    sc = __uint_as_float((uint32_t)(127 - e) << 23);
                    if (r == wi * W) escale[wi] = e;
                }
            }
#pragma unroll 1
            for (int c0 = 0; c0 < W; c0 += 16) {
                float vr[16], vn[16];
                tcx::tmem_ld16(tlane + c0, vr);
                tcx::tmem_ld16(tlane + W + c0, vn);
                if (prod) {
                    float pr[16], pi[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        if (kx == 0) packed(c0 + i, pr[i], pi[i]);
                        else product(c0 + i, vr[i], vn[i], pr[i], pi[i]);
                        pr[i] *= sc;
                        pi[i] *= sc;
                    }
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int k0 = c0 + 8 * h, k1 = W + c0 + 8 * h;
                        put8<F16, SPLIT>(dat, ((m3 >> 3) * (W / 4) + (k0 >> 3)) * 128 + (m3 & 7) * 16, dlo,
                                         pr + 8 * h);
                        put8<F16, SPLIT>(dat, ((m3 >> 3) * (W / 4) + (k1 >> 3)) * 128 + (m3 & 7) * 16, dlo,
                                         pi + 8 * h);
                    }
                }
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        __syncthreads();

        // ---- stage 3: Re T = Pr C - Pi S, Im T = Pr S + Pi C (M = 64)
        if (tid == 0) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 2 * KS; ++ks)
                mma3<SPLIT, CSPLIT>(tbase, dK3 + off(ks * 256), ks < KS ? mat(kTcC, ks) : mat(kTcNS, ks - KS), kId3,
                            ks > 0, dlo, clo);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E3: T into the stage-4 operand (MN-major, rows (window, y')
        // = 128, K = (Re | Im) x k_x); row r3 = 16 warp + lane (lane < 16)
        {
            const int r3 = 16 * warp + lane;
            const bool ok = lane < 16 && r3 < G::R3;
            const int wi = r3 / H, kx = r3 % H;
#pragma unroll 1
            for (int c0 = 0; c0 < 2 * W; c0 += 16) {
                float v[16];
                tcx::tmem_ld16(tlane + c0, v);
                if (ok) {
                    const int part = c0 / W, y0 = c0 - part * W;
                    const int k = part * H + kx;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        float t8[8];
#pragma unroll
                        for (int i = 0; i < 8; ++i) t8[i] = v[8 * h + i] * kT;
                        const int m0 = wi * W + y0 + 8 * h;
                        put8<F16, SPLIT>(dat, ((k >> 3) * 16 + (m0 >> 3)) * 128 + (k & 7) * 16, dlo, t8);
                    }
                }
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        __syncthreads();

        // ---- stage 4: plane = T * C4^T
        if (tid == 0) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < KS; ++ks)
                mma3<SPLIT, CSPLIT>(tbase, dMN + off(ks * 4096), mat(kTcC4, ks), kId4, ks > 0, dlo, clo);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E4: planes into shared memory (swapped, pedestal removed)
        float* pl = xch;
        {
            const int r = tid;
            const bool ok = r < G::R2;
            const int wi = r / W;
            float us = 1.f;
            if (F16 && ok) us = __uint_as_float((uint32_t)(127 + 32 + escale[wi]) << 23);
#pragma unroll 1
            for (int c0 = 0; c0 < W; c0 += 16) {
                float v[16];
                tcx::tmem_ld16(tlane + c0, v);
                if (ok) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) pl[r * G::PS + c0 + i] = v[i] * us;
                }
            }
        }
        tcx::fence_before();
        __syncthreads();

        // ---- find_peaks, fit, vector: warp w takes windows w, w + 4
        for (int wi = warp; wi < WPT; wi += 4) {
            const int2 o = org[wi];
            if (o.x < 0) continue;   // warp-uniform
            const int gw = gwi[wi];
            const float* P = pl + wi * W * G::PS;
            if (p.planes)
                for (int i = lane; i < W * W; i += 32) p.planes[(size_t)gw * (W * W) + i] = P[(i / W) * G::PS + i % W];
            float t0 = TC_NEG_INF, t1 = TC_NEG_INF;
            int key = 0x7fffffff;
            for (int xs = SX0 + lane; xs < SX1; xs += 32)
                for (int ys = SY0; ys < SY1; ++ys) {
                    const float c = P[ys * G::PS + xs];
                    const float m = fmaxf(fmaxf(P[(ys - 1) * G::PS + xs], P[(ys + 1) * G::PS + xs]),
                                          fmaxf(P[ys * G::PS + xs - 1], P[ys * G::PS + xs + 1]));
                    if (m < c) {
                        const int k = ys * W + xs;
                        if (c > t0 || (c == t0 && k < key)) {
                            t1 = t0;
                            t0 = c;
                            key = k;
                        } else {
                            t1 = fmaxf(t1, c);
                        }
                    }
                }
#pragma unroll
            for (int sh = 16; sh > 0; sh >>= 1) {
                const float o0 = __shfl_xor_sync(0xffffffffu, t0, sh);
                const float o1 = __shfl_xor_sync(0xffffffffu, t1, sh);
                const int ok = __shfl_xor_sync(0xffffffffu, key, sh);
                const bool take = (o0 > t0) || (o0 == t0 && ok < key);
                const float n1 = take ? fmaxf(t0, o1) : fmaxf(t1, o0);
                t0 = take ? o0 : t0;
                key = take ? ok : key;
                t1 = n1;
            }
            if (lane == 0) {
                // the pedestal for the fit in FP32 (the exact integer sums rounded to
                // float: relative error below 2e-7, far inside the fit's tolerance; FP64
                // is slow on this part and only the optional pedestal output needs it)
                const float ped = real ? 0.f : (float)sums[2 * wi] * (float)sums[2 * wi + 1];
                opiv_vector out{ 0.f, 0.f, 0.f, 0.f, 0.f };
                int32_t code = -1;
                const bool has2 = t1 > TC_NEG_INF;
                int px = 0, py = 0;
                if (has2) {
                    px = key % W;
                    py = key / W;
                    const float vc = P[py * G::PS + px];
                    const float vl = P[py * G::PS + px - 1], vr = P[py * G::PS + px + 1];
                    const float vu = P[(py - 1) * G::PS + px], vd = P[(py + 1) * G::PS + px];
                    const float C = vc + ped, L = vl + ped, R = vr + ped, U = vu + ped, D = vd + ped;
                    const float nan = __int_as_float(0x7fffffff);
                    const bool okx = L > 0.f && C > 0.f && R > 0.f;
                    const bool oky = U > 0.f && C > 0.f && D > 0.f;
                    // (ln L - ln R) / (2 (ln L + ln R - 2 ln C)) relative to C
                    const float fx = okx ? log1pf((vl - vr) / R) /
                                               (2.f * (log1pf((vl - vc) / C) + log1pf((vr - vc) / C)))
                                         : nan;
                    const float fy = oky ? log1pf((vu - vd) / D) /
                                               (2.f * (log1pf((vu - vc) / C) + log1pf((vd - vc) / C)))
                                         : nan;
                    const float p0 = t0 + ped, p1 = t1 + ped;
                    out.x = (float)(o.x + W / 2);
                    out.y = (float)(p.img_h - (o.y + W / 2));
                    out.u = (float)(W / 2 - px) - fx;
                    out.v = (float)(W / 2 - py) - fy;
                    out.sn = (p1 > 0.f) ? p0 / p1 : 0.f;
                    code = key;
                }
                p.out_vec[gw] = out;
                if (p.out_peak) p.out_peak[gw] = code;
                if (p.out_disp) p.out_disp[gw] = has2 ? pack_disp(px - W / 2, py - W / 2) : 0;
                if (p.peds) p.peds[gw] = real ? 0.0 : (double)sums[2 * wi] * (double)sums[2 * wi + 1];
            }
        }
        tcx::fence_before();
        __syncthreads();
    }
    tcx::fence_before();
    __syncthreads();
    tcx::fence_after();
    if (warp == 0) tcx::tmem_dealloc(tbase, G::kTmemCols);
}

template <int W, bool F16, bool SPLIT, bool CSPLIT, typename PixT>
cudaError_t launch_t(const PivParams& p, int mode, int limit, const void* consts, cudaStream_t s)
{
    using G = Geo<W, SPLIT, CSPLIT>;
    auto kern = piv_tcg_kernel<W, F16, SPLIT, CSPLIT, PixT>;
    static std::atomic<uint64_t> attr_done{ 0 };   // one bit per device
    static std::atomic<int> cap[64];
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(attr_done.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, G::kSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        // resident CTAs per SM from each limit: shared memory (with the
        // per-block reservation), registers, threads, tensor-memory columns
        int sms = 0, smem_sm = 0, resv = 0, regs_sm = 0, thr_sm = 0;
        cudaFuncAttributes fa{};
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev)) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev)) != cudaSuccess ||
            (e = cudaFuncGetAttributes(&fa, kern)) != cudaSuccess)
            return e;
        int per_sm = smem_sm / (G::kSmem + (int)fa.sharedSizeBytes + resv);
        const int regs = fa.numRegs > 0 ? (fa.numRegs + 7) / 8 * 8 : 1;
        const int by_regs = regs_sm / (regs * kThreads), by_thr = thr_sm / kThreads;
        const int by_tmem = 512 / (int)G::kTmemCols;
        per_sm = per_sm < by_regs ? per_sm : by_regs;
        per_sm = per_sm < by_thr ? per_sm : by_thr;
        per_sm = per_sm < by_tmem ? per_sm : by_tmem;
        cap[dev & 63].store((per_sm > 0 ? per_sm : 1) * sms);
        attr_done.fetch_or(bit);
    }
    const int64_t gny = p.n_win / p.gnx;
    const int64_t tiles = gny * ((p.gnx + G::WPT - 1) / G::WPT);
    const int64_t c = cap[dev & 63].load();
    const int blocks = (int)(tiles < c ? tiles : c);
    if (blocks <= 0) return cudaSuccess;
    kern<<<blocks, kThreads, G::kSmem, s>>>(p, reinterpret_cast<const uint4*>(consts), mode, limit);
    return cudaGetLastError();
}

// one window size: operand type, MMAs per product (3: data and constants
// split, 2: data split, FP16 only, 1: no split) and pixel type
template <int W>
cudaError_t launch_w(const PivParams& p, int dtype, int mode, int limit, int passes, bool fp16,
                     const void* consts, cudaStream_t s)
{
    const bool u8 = dtype == kU8;
    if (fp16) {
        if (passes == 3) return u8 ? launch_t<W, true, true, true, uint8_t>(p, mode, limit, consts, s)
                                   : launch_t<W, true, true, true, uint16_t>(p, mode, limit, consts, s);
        if (passes == 2) return u8 ? launch_t<W, true, true, false, uint8_t>(p, mode, limit, consts, s)
                                   : launch_t<W, true, true, false, uint16_t>(p, mode, limit, consts, s);
        return u8 ? launch_t<W, true, false, false, uint8_t>(p, mode, limit, consts, s)
                  : launch_t<W, true, false, false, uint16_t>(p, mode, limit, consts, s);
    }
    if (passes == 2) return cudaErrorInvalidValue;
    if (passes == 3) return u8 ? launch_t<W, false, true, true, uint8_t>(p, mode, limit, consts, s)
                               : launch_t<W, false, true, true, uint16_t>(p, mode, limit, consts, s);
    return u8 ? launch_t<W, false, false, false, uint8_t>(p, mode, limit, consts, s)
              : launch_t<W, false, false, false, uint16_t>(p, mode, limit, consts, s);
}

}  // namespace tcg
}  // namespace opiv
