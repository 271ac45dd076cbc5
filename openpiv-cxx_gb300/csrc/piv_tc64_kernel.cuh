// Tensor-core (tcgen05) PIV window path for 64 x 64 windows, one window per
// tile, BF16 or FP16 operands, split or plain (kernel templates; instantiated
// in piv_tc64.cu and piv_tc64_fp16.cu): the 2-D cross-correlation of every window
// pair as four chained DFT matrix products (FFT::cross_correlate,
// fft.h:188-206, unnormalised), then find_peaks(plane, 2, 1), the 3-point
// Gaussian fit and the vector (image_utils.impl.h:42-101, main.cpp:214-236).
//
// Mathematics (H = 32; the constant matrices of tc_constants at W = 64):
//   stage 1  row DFT of the window's 64 rows of both frames: U_k
//            (k = 0..31), U_32 in the slot of V_0, V_k (k = 1..31); frame B's
//            rows times (-1)^y, which rotates its column spectrum by 32 in k_y.
//   stage 2  column DFT over y, K = (U | V) x y = 128 against [C; S] and
//            [-S; C]: columns Re Z and -Im Z (N = 128).
//   product  P = B conj(A) on k_x = 0..32, P(k_y, 0) + i P(k_y, 32) packed in
//            the slot k_x = 0, DC removed (the pedestal sum(a) sum(b) is
//            added back in the fit), (-1)^k_y for the row quadrant swap,
//            REAL mode's zeroed spectrum rows 0 and 32 and column 0.
//   stage 3  inverse column DFT over k_y, transposed: the constants as the
//            A operand, the products (rows k_x) as the B operand.
//   stage 4  real inverse row DFT over k_x, the weights and the column
//            quadrant swap folded into the constant matrix C4.
//
// One CTA per SM runs GROUPS independent tile groups of 4 warps sharing one
// copy of the constants; a group takes one window at a time, has 128
// tensor-memory columns (stage 1: accumulator 0..63, pixel operand 64..127;
// later accumulators 0..127) and a 32 KB data buffer.  Rows of the products
// (M = 64 rows sit in lanes 32 (r / 16) + r % 16):
//   stage 1  R = f * 64 + y (thread tid owns lane tid)
//   stage 2  16 j + 8 f + (k_x & 7), j = k_x / 8: warp j, lanes 8 f + k_x % 8
//   stage 3  (Re | Im) x y (thread tid owns lane tid), N = 32 columns k_x
//   stage 4  y' (0..63): warp y' / 16, lanes y' % 16
// The plane goes to shared memory and is scanned by columns (rows rolling
// through registers, neighbouring columns from the neighbouring lanes).
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "piv_kernels.h"
#include "piv_tc_kernel.cuh"
#include "tc_ptx.cuh"

namespace opiv {
namespace tc64 {

using tc::pack2;
using tc::Raw;
using tc::round8;
using tc::split8;
using tc::unpack2;
using tc::widen8;

constexpr int W = 64;
constexpr int H = 32;
constexpr int kThreads = 128;
constexpr int kGroups = 4;
constexpr int kMat = W * W * 2;                 // one 64 x 64 matrix, K-major (8 KB)
constexpr int kSet = kTcNumMat * kMat;
constexpr int kConstBytes = 2 * kSet;           // hi and lo parts (lo unused without the split)
constexpr int kDataBytes = 32768;               // stage-2 and stage-3 operands, hi and lo
constexpr int kLo = 16384;                      // lo-part offset of the operand buffers
constexpr int kPacked = 8192;                   // E2: k_x-slot-0 rows (in stage-3 operand rows 32..63)
constexpr int kPS = W + 1;                      // E4 plane row stride (floats)
constexpr int kTailBytes = 1024;
constexpr int kGroupBytes = kDataBytes + kTailBytes;
constexpr int kSmem = kConstBytes + kGroups * kGroupBytes;
constexpr uint32_t kGroupCols = 128;
constexpr uint32_t kA1 = 64;                    // TMEM column of the stage-1 operand (hi, then lo)
static_assert(kSmem <= 227 * 1024, "shared memory");
static_assert(kGroups * kGroupCols <= 512, "tensor memory");
static_assert(W * kPS * 4 <= kDataBytes, "plane in the data buffer");

// 8 values into one 16-byte core-matrix row (hi, and lo kLo further)
template <bool F16, bool SPLIT>
__device__ __forceinline__ void put8(unsigned char* base, int off, const float* v)
{
    if (SPLIT) {
        uint4 hi, lo;
        split8<F16>(v, hi, lo);
        *reinterpret_cast<uint4*>(base + off) = hi;
        *reinterpret_cast<uint4*>(base + kLo + off) = lo;
    } else {
        *reinterpret_cast<uint4*>(base + off) = round8<F16>(v);
    }
}

template <bool F16, bool SPLIT>
__device__ __forceinline__ void put1(unsigned char* base, int off, float v)
{
    const uint32_t h = pack2<F16>(v, 0.f);
    *reinterpret_cast<uint16_t*>(base + off) = (uint16_t)(h & 0xffffu);
    if (SPLIT) {
        const float hv = unpack2<F16>(h).x;
        *reinterpret_cast<uint16_t*>(base + kLo + off) = (uint16_t)(pack2<F16>(v - hv, 0.f) & 0xffffu);
    }
}

// D (+)= A * B split into hi*hi, hi*lo (CSPLIT: the constant's lo part),
// lo*hi (a, b: descriptors of the hi parts; the data's lo part kLo further,
// the constants' one set further)
template <bool SPLIT, bool CSPLIT>
__device__ __forceinline__ void mma3(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, bool acc)
{
    tcx::mma_bf16(d, a, b, idesc, acc);
    if (SPLIT) {
        if (CSPLIT) tcx::mma_bf16(d, a, b + (uint64_t)(kSet >> 4), idesc, true);
        tcx::mma_bf16(d, a + (uint64_t)(kLo >> 4), b, idesc, true);
    }
}

template <bool SPLIT, bool CSPLIT>
__device__ __forceinline__ void mma3_ta(uint32_t d, uint32_t a_hi, uint32_t a_lo, uint64_t b, uint32_t idesc,
                                        bool acc)
{
    tcx::mma_bf16_ta(d, a_hi, b, idesc, acc);
    if (SPLIT) {
        if (CSPLIT) tcx::mma_bf16_ta(d, a_hi, b + (uint64_t)(kSet >> 4), idesc, true);
        tcx::mma_bf16_ta(d, a_lo, b, idesc, true);
    }
}

// Running top two of strict 4-neighbour maxima (ties: the lower row-major
// index, the reference's scan order)
struct Top2 {
    float t0, t1;
    int key;
};

__device__ __forceinline__ void top2_merge(Top2& s, float o0, float o1, int ok)
{
    const bool take = (o0 > s.t0) || (o0 == s.t0 && ok < s.key);
    const float n1 = take ? fmaxf(s.t0, o1) : fmaxf(s.t1, o0);
    s.t0 = take ? o0 : s.t0;
    s.key = take ? ok : s.key;
    s.t1 = n1;
}

// F16: FP16 operands scaled by powers of two as in the other tensor-core
// kernels (pixels x 2^-4, the stage-1 matrix x 2^-9 in the constants, the
// products x 2^-e with e per window from its largest product, T x 2^-6),
// undone exactly in the peak stage.  CSPLIT: the constants' lo parts enter
// too (three MMAs per product); otherwise only the data is split (two).
template <bool F16, bool SPLIT, bool CSPLIT, int MODE, bool LIMIT, typename PixT>
__global__ void __launch_bounds__(kThreads * kGroups, 1)
piv_tc64_kernel(const PivParams p, const uint4* __restrict__ consts)
{
    constexpr float kPix = F16 ? 0.0625f : 1.f;
    constexpr float kT = F16 ? 0.015625f : 1.f;
    constexpr float kSumUnscale = F16 ? 8192.f : 1.f;
    // peak scan range in swapped-plane coordinates (image_utils.impl.h:48,
    // :54; limited search: rect::dilate(0.5), rect.cpp:109-126)
    constexpr int D0 = LIMIT ? W / 4 : 0;
    constexpr int VW = LIMIT ? W / 2 : W;
    constexpr int SY0 = D0 + 1, SY1 = D0 + VW - 2;
    constexpr int SX0 = D0 + 1, SX1 = D0 + VW - 1;
    constexpr uint32_t kId1 = tcx::idesc_f16kind(128, 64, false, F16);
    constexpr uint32_t kId2 = tcx::idesc_f16kind(64, 128, true, F16);
    constexpr uint32_t kId3 = tcx::idesc_f16kind(128, 32, false, F16);
    constexpr uint32_t kId4 = tcx::idesc_f16kind(64, 64, false, F16);

    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* cst = smem;
    const int grp = (int)(threadIdx.x / kThreads);
    unsigned char* dat = smem + kConstBytes + grp * kGroupBytes;
    // row sums [frame][row] (exact integers: a row sum is an exact FP32
    // accumulator value, at most 2^22 for 64 16-bit pixels)
    float* rs = reinterpret_cast<float*>(dat + kDataBytes);
    float* wt0 = rs + 128;                                  // per-warp top two and keys
    float* wt1 = wt0 + 4;
    int* wkey = reinterpret_cast<int*>(wt1 + 4);
    int* wsum = wkey + 4;                                   // per-warp pixel sums
    float* wmax = reinterpret_cast<float*>(wsum + 4);       // F16: per-warp largest product
    uint64_t* mbar = reinterpret_cast<uint64_t*>(wmax + 4);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
    int* abort_flag = reinterpret_cast<int*>(tslot + 1);
    // the CTA's tensor-memory address lives in group 0's tail
    uint32_t* tslot_cta = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(tslot) - grp * kGroupBytes);

    const int tid = (int)threadIdx.x % kThreads, warp = tid >> 5, lane = tid & 31;
    auto gsync = [&]() { asm volatile("bar.sync %0, %1;" :: "r"(1 + grp), "r"(kThreads) : "memory"); };
    const uint32_t cst_a = tcx::smem_addr(cst), dat_a = tcx::smem_addr(dat);
    // descriptors: constant matrix m (K-major, K groups 128 bytes apart, N
    // groups 16 W); the data buffer as the MN-major stage-2 / stage-4
    // operands (K groups 1 KB apart, 8 M groups of 128 bytes) and the K-major
    // stage-3 operand (16 K groups per row group)
    const uint64_t dB = tcx::sdesc(cst_a, 128, 16 * W);
    auto mat = [&](int m, int ks) { return dB + (uint64_t)((m * kMat + ks * 256) >> 4); };
    const uint64_t dMN = tcx::sdesc(dat_a, 1024, 128);
    const uint64_t dK3 = tcx::sdesc(dat_a, 128, 2048);
    const uint64_t dK4 = tcx::sdesc(dat_a, 128, 1024);   // K-major, K = 64: 8 K groups per row group
    auto off = [](int bytes) { return (uint64_t)(bytes >> 4); };

    for (int i = threadIdx.x; i < (CSPLIT ? 2 : 1) * kSet / 16; i += kThreads * kGroups)
        reinterpret_cast<uint4*>(cst)[i] = consts[i];
    if (tid == 0) {
        tcx::mbar_init(mbar, 1);
        *abort_flag = 0;
    }
    if (threadIdx.x < 32) tcx::tmem_alloc(tslot_cta, kGroups * kGroupCols);
    tcx::fence_before();
    __syncthreads();
    tcx::fence_after();
    const uint32_t tcta = *tslot_cta;
    const uint32_t tbase = tcta + (uint32_t)grp * kGroupCols;
    const uint32_t tlane = tbase + ((uint32_t)(32 * warp) << 16);

    const PixT* fa = reinterpret_cast<const PixT*>(p.fa);
    const PixT* fb = reinterpret_cast<const PixT*>(p.fb);
    const size_t pitch = p.pitch / sizeof(PixT);
    // windows in grid order, each group a contiguous range
    const int64_t n_win = p.n_win;
    const int64_t vb = (int64_t)blockIdx.x * kGroups + grp, vg = (int64_t)gridDim.x * kGroups;
    const int w_begin = (int)(vb * n_win / vg);
    const int w_end = (int)((vb + 1) * n_win / vg);
    uint32_t phase = 0;
    auto wait_mma = [&]() {
        // after a wait has given up, the window finishes without waiting again
        if (!*abort_flag && !tcx::mbar_wait(mbar, phase)) {
            *abort_flag = 1;
            if (p.status) atomicExch(p.status, 1);
        }
        phase ^= 1u;
        tcx::fence_after();
    };
    // grid position of window w_begin, then advanced in registers
    int gcol = w_begin % p.gnx, grow = w_begin / p.gnx;

    for (int win = w_begin; win < w_end; ++win) {
        const int ox = p.gx0 + gcol * p.gdx, oy = p.gy0 + grow * p.gdy;
        // ---- stage-1 operand in tensor memory: thread tid owns lane tid =
        // row R = f * 64 + y.  The row's 64 pixels, widened (frame B rows
        // times (-1)^y), fill 32 columns of the hi part and 32 of the lo
        // part: pixel 2c in the low half of column c.
        {
            const int f = tid >> 6, y = tid & 63;
            const PixT* row = (f ? fb : fa) + (size_t)(oy + y) * pitch + ox;
            const float sg = ((f && (y & 1)) ? -1.f : 1.f) * kPix;
#pragma unroll
            for (int hp = 0; hp < 2; ++hp) {   // pixels 32 hp .. 32 hp + 31: columns 16 hp .. + 15
                uint32_t hw[16], lw[16];
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                    float px[8];
                    widen8<PixT>(tc::load_raw<PixT>(row + 32 * hp + 8 * g), px, sg);
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        hw[4 * g + j] = pack2<F16>(px[2 * j], px[2 * j + 1]);
                        if (SPLIT) {
                            const float2 hf = unpack2<F16>(hw[4 * g + j]);
                            lw[4 * g + j] = pack2<F16>(px[2 * j] - hf.x, px[2 * j + 1] - hf.y);
                        }
                    }
                }
                tcx::tmem_st16(tlane + kA1 + 16 * hp, hw);
                if (SPLIT) tcx::tmem_st16(tlane + kA1 + 32 + 16 * hp, lw);
            }
        }
        tcx::fence_before();
        gsync();
        if (*abort_flag) break;

        // ---- stage 1: H1 = X * G1^T (K = 64 in four steps)
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
                mma3_ta<SPLIT, CSPLIT>(tbase, tbase + kA1 + 8 * ks, tbase + kA1 + 32 + 8 * ks, mat(kTcG1, ks), kId1,
                               ks > 0);
            tcx::commit(mbar);
        }
        // the next window's rows into L2 while this one computes
        if (win + 1 < w_end) {
            const int nc = gcol + 1 < p.gnx ? gcol + 1 : 0;
            const int nr = gcol + 1 < p.gnx ? grow : grow + 1;
            const int f = tid >> 6, y = tid & 63;
            const PixT* q = (f ? fb : fa) + (size_t)(p.gy0 + nr * p.gdy + y) * pitch + p.gx0 + nc * p.gdx;
            asm volatile("prefetch.global.L2 [%0];" :: "l"(q));
        }
        wait_mma();

        // ---- E1: the coefficients into the stage-2 operand: MN-major,
        // M = 16 j + 8 f + k % 8 (j = k / 8), K = (U | V) x y; core matrix
        // (K group, M group) at (K / 8) * 1024 + (M / 8) * 128; row sums
        {
            const int f = tid >> 6, y = tid & 63;
#pragma unroll
            for (int part = 0; part < 2; ++part) {   // U (columns 0..31), then V
                float c[32];
                tcx::tmem_ld32(tlane + 32 * part, c);
                if (part == 0) rs[f * 64 + y] = (f && (y & 1)) ? -c[0] : c[0];   // undo the frame-B row sign
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    put8<F16, SPLIT>(dat, (part * 8 + (y >> 3)) * 1024 + (2 * j + f) * 128 + (y & 7) * 16, c + 8 * j);
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 2: conj of the column DFT: the U part against [C; S],
        // the V part against [-S; C] (M = 64, N = 128, K = 128)
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 8; ++ks)
                mma3<SPLIT, CSPLIT>(tbase, dMN + off(ks * 2048), ks < 4 ? mat(kTcC, ks) : mat(kTcNS, ks - 4), kId2, ks > 0);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E2: products into the stage-3 operand (K-major, rows k_x,
        // K = (Re | Im) x k_y = 128).  Thread: row L = lane % 16 of warp j
        // (frame L / 8, k_x = 8 j + L % 8), column half hh = lane / 16.
        int escale = 0;   // F16: the window's product exponent
        {
            const int L = lane & 15, hh = lane >> 4;
            const int f = L >> 3, kx = 8 * warp + (L & 7);
            float* pk = reinterpret_cast<float*>(dat + kPacked);   // [frame][Re 64 | -Im 64]
            const float sq = f ? -1.f : 1.f;
            // half h: columns 16 hh + 8 h + i of each quarter (i < 8): q[i] Re,
            // q[8 + i] Re 32 further, q[16 + i] -Im, q[24 + i] -Im 32 further
            auto load_half = [&](int h, float* q) {
                if (h == 0) tcx::tmem_ld16x2_8x4<0, 32, 64, 96>(tlane, q);
                else tcx::tmem_ld16x2_8x4<8, 40, 72, 104>(tlane, q);
            };
            auto keep_slot0 = [&](int h, const float* q) {   // the k_x slot-0 rows for the packed bins
                if (kx == 0) {
                    const int b0 = f * 128 + 16 * hh + 8 * h;
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int v4 = 0; v4 < 2; ++v4)
                            *reinterpret_cast<float4*>(pk + b0 + 32 * u + 4 * v4) =
                                make_float4(q[8 * u + 4 * v4], q[8 * u + 4 * v4 + 1], q[8 * u + 4 * v4 + 2],
                                            q[8 * u + 4 * v4 + 3]);
                }
            };
            // frame a's thread computes k_y = 16 hh + 8 h + i, frame b's 32 more;
            // frame b's columns are rotated by 32, so both find their own
            // values in q[i], q[16 + i] and take their partner's (lane ^ 8)
            // q[8 + i], q[24 + i].  With m = own, o = partner values and
            // n = -Im: Re P = m_r o_r + m_n o_n, Im P = +-(o_r m_n - o_n m_r),
            // + for frame a.
            auto products = [&](int h, const float* q, float* pr, float* pi) {
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float mr = q[i], mn = q[16 + i];
                    const float orr = __shfl_xor_sync(0xffffffffu, q[8 + i], 8);
                    const float onn = __shfl_xor_sync(0xffffffffu, q[24 + i], 8);
                    float r = fmaf(mr, orr, mn * onn);
                    float qq = sq * fmaf(orr, mn, -(onn * mr));
                    if (i & 1) { r = -r; qq = -qq; }   // quadrant sign (-1)^k_y
                    if (MODE == kModeReal && i == 0 && hh == 0 && h == 0) { r = 0.f; qq = 0.f; }   // k_y = 0 or 32
                    pr[i] = r;
                    pi[i] = qq;
                }
            };
            auto store_half = [&](int h, const float* pr, const float* pi) {
                if (kx != 0) {
                    const int kr = 32 * f + 16 * hh + 8 * h, ki = 64 + kr;
                    put8<F16, SPLIT>(dat, ((kx >> 3) * 16 + (kr >> 3)) * 128 + (kx & 7) * 16, pr);
                    put8<F16, SPLIT>(dat, ((kx >> 3) * 16 + (ki >> 3)) * 128 + (kx & 7) * 16, pi);
                }
            };
            // the packed row k_x = 0 | 32 (warp 0, k_y = lane + 32 h2)
            auto packed = [&](int h2, float& pkr, float& pkq) {
                const float* sa = pk;          // frame a, k_x slot 0
                const float* sb = pk + 128;    // frame b, columns rotated by 32
                const int ky = lane + 32 * h2, kn = (64 - ky) & 63;
                const int kb = (ky + 32) & 63, kbn = (kn + 32) & 63;
                // Z[k] = Re + i Im with Im = -stored
                const float zar = sa[ky], zai = -sa[64 + ky], zanr = sa[kn], zani = -sa[64 + kn];
                const float zbr = sb[kb], zbi = -sb[64 + kb], zbnr = sb[kbn], zbni = -sb[64 + kbn];
                // X0 = (Z[k] + conj Z[-k]) / 2, X32 = i (Z[k] - conj Z[-k]) / 2
                const float a0r = 0.5f * (zar + zanr), a0i = 0.5f * (zai - zani);
                const float a6r = -0.5f * (zai + zani), a6i = 0.5f * (zar - zanr);
                const float b0r = 0.5f * (zbr + zbnr), b0i = 0.5f * (zbi - zbni);
                const float b6r = -0.5f * (zbi + zbni), b6i = 0.5f * (zbr - zbnr);
                float p0r = b0r * a0r + b0i * a0i, p0i = b0i * a0r - b0r * a0i;
                float p6r = b6r * a6r + b6i * a6i, p6i = b6i * a6r - b6r * a6i;
                if (MODE == kModeReal) {
                    p0r = 0.f; p0i = 0.f;
                    if (ky == 0 || ky == H) { p6r = 0.f; p6i = 0.f; }
                } else if (ky == 0) {
                    p0r = 0.f; p0i = 0.f;         // pedestal removed
                }
                pkr = p0r - p6i;
                pkq = p0i + p6r;
                if (ky & 1) { pkr = -pkr; pkq = -pkq; }
            };
            auto store_packed = [&](int h2, float pkr, float pkq) {
                const int ky = lane + 32 * h2;
                put1<F16, SPLIT>(dat, (ky >> 3) * 128 + (ky & 7) * 2, pkr);
                put1<F16, SPLIT>(dat, ((64 + ky) >> 3) * 128 + (ky & 7) * 2, pkq);
            };
            float sc = 1.f;
            if constexpr (F16) {
                // first the window's largest product over all four warps, so
                // that the products scaled by 2^-e lie below 2^9 (stage 3 sums
                // 128 of them into FP32; T x 2^-6 then fits FP16)
                float m = 0.f;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    float q[32], pr[8], pi[8];
                    load_half(h, q);
                    keep_slot0(h, q);
                    products(h, q, pr, pi);
                    if (kx != 0) {
#pragma unroll
                        for (int i = 0; i < 8; ++i) m = fmaxf(m, fmaxf(fabsf(pr[i]), fabsf(pi[i])));
                    }
                }
                if (warp == 0) {
                    __syncwarp();
#pragma unroll
                    for (int h2 = 0; h2 < 2; ++h2) {
                        float a2, b2;
                        packed(h2, a2, b2);
                        m = fmaxf(m, fmaxf(fabsf(a2), fabsf(b2)));
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
                if (lane == 0) wmax[warp] = m;
                gsync();
                const float mm = fmaxf(fmaxf(wmax[0], wmax[1]), fmaxf(wmax[2], wmax[3]));
                const int eb = (int)((__float_as_uint(mm) >> 23) & 0xffu);
                int e = eb == 0 ? 0 : eb - 127 - 8;
                e = e < -90 ? -90 : (e > 80 ? 80 : e);
                escale = e;
                sc = __uint_as_float((uint32_t)(127 - e) << 23);
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float q[32], pr[8], pi[8];
                load_half(h, q);
                if (!F16) keep_slot0(h, q);
                products(h, q, pr, pi);
                if (F16) {
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        pr[i] *= sc;
                        pi[i] *= sc;
                    }
                }
                store_half(h, pr, pi);
            }
            if (warp == 0) {
                __syncwarp();
#pragma unroll
                for (int h2 = 0; h2 < 2; ++h2) {
                    float a2, b2;
                    packed(h2, a2, b2);
                    store_packed(h2, a2 * sc, b2 * sc);
                }
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 3: inverse column DFT, transposed: T^T = [C; S] x Pr^T +
        // [-S; C] x Pi^T with the constants as the A operand (M = 128 rows:
        // Re T(y) then Im T(y)) and the products as the B operand (N = 32
        // rows k_x, K-major as E2 wrote them, K = (Re | Im) x k_y = 128)
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 8; ++ks) {
                const uint64_t a = ks < 4 ? mat(kTcC, ks) : mat(kTcNS, ks - 4), b = dK3 + off(ks * 256);
                tcx::mma_bf16(tbase, a, b, kId3, ks > 0);
                if (SPLIT) {
                    if (CSPLIT) tcx::mma_bf16(tbase, a + (uint64_t)(kSet >> 4), b, kId3, true);
                    tcx::mma_bf16(tbase, a, b + (uint64_t)(kLo >> 4), kId3, true);
                }
            }
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E3: T into the stage-4 operand (K-major, M = y', K = (Re | Im)
        // x k_x = 64, core matrix (row group, K group) at (y' / 8) * 1024 +
        // (K / 8) * 128).  Thread tid holds accumulator row tid = part * 64 +
        // y: the 32 values T_part(y, k_x).
        {
            const int part = tid >> 6, y = tid & 63;
            float t[32];
            tcx::tmem_ld32(tlane, t);
            if (F16) {
#pragma unroll
                for (int i = 0; i < 32; ++i) t[i] *= kT;
            }
#pragma unroll
            for (int c = 0; c < 4; ++c)
                put8<F16, SPLIT>(dat, ((y >> 3) * 8 + part * 4 + c) * 128 + (y & 7) * 16, t + 8 * c);
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 4: real inverse row DFT, D = T * C4 (M = 64, N = 64,
        // K = 64, the operand K-major)
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
                mma3<SPLIT, CSPLIT>(tbase, dK4 + off(ks * 256), mat(kTcC4, ks), kId4, ks > 0);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E4: the plane into shared memory (row y' of warp y' / 16,
        // lane % 16; lane / 16 the column half), the pixel sums per warp
        float* P = reinterpret_cast<float*>(dat);
        {
            const int L = lane & 15, hh = lane >> 4;
            const int y = 16 * warp + L;
            float v[32];
            tcx::tmem_ld16x2_32(tlane, v);
            if (F16) {   // undo 2^-26 (pixels, stage-1 matrix, twice), 2^-e (products), 2^-6 (T)
                const float us = __uint_as_float((uint32_t)(127 + 32 + escale) << 23);
#pragma unroll
                for (int i = 0; i < 32; ++i) v[i] *= us;
            }
#pragma unroll
            for (int i = 0; i < 32; ++i) P[y * kPS + 32 * hh + i] = v[i];
            if (p.planes) {
                const int gw = grow * p.gnx + gcol;
#pragma unroll
                for (int i = 0; i < 32; i += 4)
                    *reinterpret_cast<float4*>(p.planes + (size_t)gw * (W * W) + y * W + 32 * hh + i) =
                        make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
            }
            // pixel sums: warps 0, 1 frame a, warps 2, 3 frame b (row 64 f + y)
            int s = __float2int_rn(rs[tid] * kSumUnscale);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) wsum[warp] = s;
        }
        tcx::fence_before();
        gsync();

        // ---- find_peaks: thread = (column x, 32-row block); the block's
        // candidate rows roll through registers, neighbouring columns come
        // from the neighbouring lanes (the two edge lanes of a warp read
        // theirs); branch-free top two
        {
            const int xs = tid & 63, yb = (tid >> 6) * 32;
            const bool col_ok = xs >= SX0 && xs < SX1;
            const int y0 = yb > SY0 ? yb : SY0, y1 = yb + 32 < SY1 ? yb + 32 : SY1;   // uniform over the warp
            const int xl = (xs + W - 1) & (W - 1), xr = (xs + 1) & (W - 1);
            Top2 s{ TC_NEG_INF, TC_NEG_INF, 0x7fffffff };
            float up = P[(y0 - 1) * kPS + xs], cc = P[y0 * kPS + xs];
#pragma unroll 4
            for (int ys = y0; ys < y1; ++ys) {
                const float dn = P[(ys + 1) * kPS + xs];
                const float sl = __shfl_up_sync(0xffffffffu, cc, 1);
                const float sr = __shfl_down_sync(0xffffffffu, cc, 1);
                const float lf = lane == 0 ? P[ys * kPS + xl] : sl;
                const float rt = lane == 31 ? P[ys * kPS + xr] : sr;
                const float m = tcx::fmax3(up, dn, fmaxf(lf, rt));
                const float sv = (col_ok && m < cc) ? cc : TC_NEG_INF;
                const bool gt = sv > s.t0;
                s.t1 = gt ? s.t0 : fmaxf(s.t1, sv);
                s.key = gt ? ys * W + xs : s.key;
                s.t0 = gt ? sv : s.t0;
                up = cc;
                cc = dn;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float o0 = __shfl_xor_sync(0xffffffffu, s.t0, o);
                const float o1 = __shfl_xor_sync(0xffffffffu, s.t1, o);
                const int ok = __shfl_xor_sync(0xffffffffu, s.key, o);
                top2_merge(s, o0, o1, ok);
            }
            if (lane == 0) {
                wt0[warp] = s.t0;
                wt1[warp] = s.t1;
                wkey[warp] = s.key;
            }
        }
        gsync();

        // ---- fit_simple_gaussian and the vector: warp 0, the six
        // logarithms on six lanes, relative to the pedestal
        if (warp == 0) {
            Top2 s{ wt0[0], wt1[0], wkey[0] };
#pragma unroll
            for (int i = 1; i < 4; ++i) top2_merge(s, wt0[i], wt1[i], wkey[i]);
            const int sum_a = wsum[0] + wsum[1], sum_b = wsum[2] + wsum[3];
            // the pedestal for the fit in FP32 (the exact integer sums rounded
            // to float); REAL mode's plane has none
            const float ped = MODE == kModeReal ? 0.f : (float)sum_a * (float)sum_b;
            const bool has2 = s.t1 > TC_NEG_INF;
            const int px = s.key & (W - 1), py = (s.key >> 6) & (W - 1);
            // lane j's logarithm: ln(L/R), ln(L/C), ln(R/C), ln(U/D), ln(U/C), ln(D/C)
            const int j = lane < 6 ? lane : 0;
            const int nx = (j == 2) ? px + 1 : (j < 2 ? px - 1 : px);
            const int ny = (j == 3 || j == 4) ? py - 1 : (j == 5 ? py + 1 : py);
            const int qx = (j == 0) ? px + 1 : px;
            const int qy = (j == 3) ? py + 1 : py;
            const float an = P[(ny & (W - 1)) * kPS + (nx & (W - 1))];
            const float ad = P[(qy & (W - 1)) * kPS + (qx & (W - 1))];
            const float lg = log1pf((an - ad) / (ad + ped));
            const float lxr = __shfl_sync(0xffffffffu, lg, 0);
            const float lxl = __shfl_sync(0xffffffffu, lg, 1);
            const float lxrr = __shfl_sync(0xffffffffu, lg, 2);
            const float lyd = __shfl_sync(0xffffffffu, lg, 3);
            const float lyu = __shfl_sync(0xffffffffu, lg, 4);
            const float lydd = __shfl_sync(0xffffffffu, lg, 5);
            if (lane == 0) {
                const int gw = grow * p.gnx + gcol;
                opiv_vector out{ 0.f, 0.f, 0.f, 0.f, 0.f };
                int32_t code = -1;
                if (has2) {
                    const float vc = P[py * kPS + px];
                    const float C = vc + ped;
                    const float Lv = P[py * kPS + px - 1] + ped, R = P[py * kPS + px + 1] + ped;
                    const float U = P[(py - 1) * kPS + px] + ped, D = P[(py + 1) * kPS + px] + ped;
                    const float nan = __int_as_float(0x7fffffff);
                    const bool okx = Lv > 0.f && C > 0.f && R > 0.f;
                    const bool oky = U > 0.f && C > 0.f && D > 0.f;
                    const float fx = okx ? lxr / (2.f * (lxl + lxrr)) : nan;
                    const float fy = oky ? lyd / (2.f * (lyu + lydd)) : nan;
                    const float p0 = s.t0 + ped, p1 = s.t1 + ped;
                    out.x = (float)(ox + W / 2);
                    out.y = (float)(p.img_h - (oy + W / 2));
                    out.u = (float)(W / 2 - px) - fx;
                    out.v = (float)(W / 2 - py) - fy;
                    out.sn = (p1 > 0.f) ? p0 / p1 : 0.f;
                    code = s.key;
                }
                p.out_vec[gw] = out;
                if (p.out_peak) p.out_peak[gw] = code;
                if (p.out_disp) p.out_disp[gw] = has2 ? pack_disp(px - W / 2, py - W / 2) : 0;
                if (p.peds) p.peds[gw] = MODE == kModeReal ? 0.0 : (double)sum_a * (double)sum_b;
            }
        }
        // the next window: the barrier after its pixel stage orders this
        // window's plane and tensor-memory reads before anything overwrites them
        if (++gcol == p.gnx) {
            gcol = 0;
            ++grow;
        }
    }
    tcx::fence_before();
    __syncthreads();
    tcx::fence_after();
    if (threadIdx.x < 32) tcx::tmem_dealloc(tcta, kGroups * kGroupCols);
}

// window x positions and x step on multiples of 8 pixels (16- or 8-byte
// row loads), 16-byte aligned rows
inline bool applicable(const PivParams& p)
{
    return p.gx0 % 8 == 0 && p.gdx % 8 == 0 && p.pitch % 16 == 0 && p.win_xy == nullptr &&
           p.prev_disp == nullptr;
}

template <bool F16, bool SPLIT, bool CSPLIT, int MODE, bool LIMIT, typename PixT>
cudaError_t launch_t(const PivParams& p, const void* consts, cudaStream_t s)
{
    auto kern = piv_tc64_kernel<F16, SPLIT, CSPLIT, MODE, LIMIT, PixT>;
    static std::atomic<uint64_t> attr_done{ 0 };   // one bit per device
    static std::atomic<int> sm_count[64];
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(attr_done.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
        if (e != cudaSuccess) return e;
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        sm_count[dev & 63].store(sms);
        attr_done.fetch_or(bit);
    }
    const int64_t cap = sm_count[dev & 63].load();   // one CTA per SM
    const int64_t want = (p.n_win + kGroups - 1) / kGroups;
    const int blocks = (int)(want < cap ? want : cap);
    if (blocks <= 0) return cudaSuccess;
    kern<<<blocks, kThreads * kGroups, kSmem, s>>>(p, reinterpret_cast<const uint4*>(consts));
    return cudaGetLastError();
}

template <bool F16, bool SPLIT, bool CSPLIT, int MODE, bool LIMIT>
cudaError_t by_dtype(const PivParams& p, int dtype, const void* consts, cudaStream_t s)
{
    return dtype == kU8 ? launch_t<F16, SPLIT, CSPLIT, MODE, LIMIT, uint8_t>(p, consts, s)
                        : launch_t<F16, SPLIT, CSPLIT, MODE, LIMIT, uint16_t>(p, consts, s);
}

template <bool F16, bool SPLIT, bool CSPLIT>
cudaError_t by_mode(const PivParams& p, int dtype, int mode, int limit, const void* consts, cudaStream_t s)
{
    if (mode == kModeReal)
        return limit ? by_dtype<F16, SPLIT, CSPLIT, kModeReal, true>(p, dtype, consts, s)
                     : by_dtype<F16, SPLIT, CSPLIT, kModeReal, false>(p, dtype, consts, s);
    return limit ? by_dtype<F16, SPLIT, CSPLIT, kModeComplex, true>(p, dtype, consts, s)
                 : by_dtype<F16, SPLIT, CSPLIT, kModeComplex, false>(p, dtype, consts, s);
}

}  // namespace tc64
}  // namespace opiv
