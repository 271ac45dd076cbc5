// Tensor-core (tcgen05) PIV window path for 16 x 16 windows on vertical
// tiles (kernel templates; instantiated per operand type in
// piv_tc16_bf16.cu and piv_tc16_fp16.cu): the 32 px kernel's design
// (piv_tc_kernel.cuh) at W = 16 -- the 2-D cross-correlation of every window
// pair as four chained DFT matrix products (FFT::cross_correlate,
// fft.h:188-206, unnormalised), then find_peaks(plane, 2, 1), the 3-point
// Gaussian fit and the vector (image_utils.impl.h:42-101, main.cpp:214-236)
// on the CUDA cores.
//
// Mathematics (H = 8; the constant matrices of tc_constants at W = 16):
//   stage 1  row DFT of each image row: U_k (k = 0..7), U_8 in the slot of
//            V_0, V_k (k = 1..7); frame B's rows are multiplied by (-1)^y,
//            which rotates its column spectrum by 8 in k_y.
//   stage 2  column DFT over the window's 16 rows, K = (U | V) x y = 32
//            against [C; S] and [-S; C]: columns Re Z and -Im Z.
//   product  P = B conj(A) on k_x = 0..8, P(k_y, 0) + i P(k_y, 8) packed in
//            the slot k_x = 0, DC removed (the pedestal sum(a) sum(b) is
//            added back in the fit), (-1)^k_y for the row quadrant swap,
//            REAL mode's zeroed spectrum rows 0 and 8 and column 0.
//   stage 3  inverse column DFT over k_y (M = 64 rows (window, k_x)).
//   stage 4  real inverse row DFT over k_x, the weights and the column
//            quadrant swap folded into the constant matrix C4.
//
// A tile is 8 windows of one grid column (row step <= 6: their 16-row
// windows span at most 58 image rows); one CTA per SM runs GROUPS
// independent tile groups of 4 warps sharing one copy of the constants.
// Thread tid of a group owns tensor-memory lane tid; rows of the products:
//   stage 1  R = f * 64 + y (frame f, image row y below the tile's top)
//   stage 2  16 i + 8 f + k_x (window i, frame f)  -> warp i / 2
//   stage 3  8 i + k_x, M = 64 (lane 32 (r / 16) + r % 16)
//   stage 4  16 i + y'
// so warp w holds windows 2w and 2w + 1 from stage 2 on.  A group has 32
// tensor-memory columns (the stage-1 accumulator in 0..15 and its pixel
// operand in 16..31, later accumulators in 0..31) and a 16 KB data buffer.
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "piv_kernels.h"
#include "piv_tc_kernel.cuh"
#include "tc_ptx.cuh"

namespace opiv {
namespace tc16 {

using tc::pack2;
using tc::Raw;
using tc::round8;
using tc::split8;
using tc::unpack2;
using tc::widen8;

constexpr int W = 16;
constexpr int H = 8;
constexpr int kThreads = 128;
constexpr int kTile = 8;                        // windows per tile
constexpr int kMaxStep = 6;                     // row steps with 8 x 16 rows <= 64
constexpr int kMat = W * W * 2;                 // one 16 x 16 matrix, K-major
constexpr int kSet = kTcNumMat * kMat;
constexpr int kDataBytes = 16384;               // stage-2 operand, hi and lo (its largest user)
constexpr int kLo = 8192;                       // lo-part offset of the operand buffers
constexpr int kPacked = 4096;                   // E2: k_x-slot-0 rows (after the stage-3 operand)
constexpr int kPkWin = 80;                      // E2: floats per window there (the two windows of
                                                // a warp 16 banks apart)
constexpr int kPRow = 20;                       // E4 plane row (floats), padded to 16 bytes
constexpr int kTailBytes = 1024;                // row sums, exponents, mbarrier, slots
constexpr int kGroupBytes = kDataBytes + kTailBytes;
constexpr uint32_t kGroupCols = 32;
constexpr uint32_t kA1 = 16;                    // TMEM column of the stage-1 operand (hi, then lo)

template <int GROUPS>
struct Shape {
    static constexpr int kConstBytes = 2 * kSet;      // hi and lo parts (lo unused without CSPLIT)
    static constexpr int kSmem = kConstBytes + GROUPS * kGroupBytes;
    static constexpr uint32_t kCols = GROUPS * kGroupCols <= 32    ? 32
                                      : GROUPS * kGroupCols <= 64  ? 64
                                      : GROUPS * kGroupCols <= 128 ? 128
                                      : GROUPS * kGroupCols <= 256 ? 256
                                                                   : 512;
    static_assert(kSmem <= 227 * 1024, "shared memory");
    static_assert(GROUPS * kGroupCols <= 512, "tensor memory");
};

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

// D (+)= A * B split into hi*hi, hi*lo (CSPLIT: the constant's lo part) and
// lo*hi; a, b: descriptors of the hi parts (the data's lo part kLo further,
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

// the same with the A operand (hi part a_hi, lo part a_lo) in tensor memory
template <bool SPLIT, bool CSPLIT>
__device__ __forceinline__ void mma3_ta(uint32_t d, uint32_t a_hi, uint32_t a_lo, uint64_t b, uint32_t idesc)
{
    tcx::mma_bf16_ta(d, a_hi, b, idesc, false);
    if (SPLIT) {
        if (CSPLIT) tcx::mma_bf16_ta(d, a_hi, b + (uint64_t)(kSet >> 4), idesc, true);
        tcx::mma_bf16_ta(d, a_lo, b, idesc, true);
    }
}

// 16 pixels of a row whose start is aligned to 4 pixels, as two 8-pixel raw
// words for widen8
template <typename PixT>
__device__ __forceinline__ void load16(const PixT* row, typename Raw<PixT>::type* raw)
{
    if constexpr (sizeof(PixT) == 2) {
        const uint2* q = reinterpret_cast<const uint2*>(row);
        const uint2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3);
        raw[0] = make_uint4(a.x, a.y, b.x, b.y);
        raw[1] = make_uint4(c.x, c.y, d.x, d.y);
    } else {
        const uint32_t* q = reinterpret_cast<const uint32_t*>(row);
        raw[0] = make_uint2(__ldg(q), __ldg(q + 1));
        raw[1] = make_uint2(__ldg(q + 2), __ldg(q + 3));
    }
}

// F16: FP16 operands scaled by powers of two as in the 32 px kernel (pixels
// x 2^-4, the stage-1 matrix x 2^-9 in the constants, the product x 2^-e
// with e per window from its largest value, T x 2^-6), undone exactly in
// the peak stage.  CSPLIT: the constants' lo parts enter too (three MMAs per
// product); otherwise only the data is split (two).
template <bool F16, bool SPLIT, bool CSPLIT, int MODE, bool LIMIT, typename PixT, int GROUPS>
__global__ void __launch_bounds__(kThreads * GROUPS, 1)
piv_tc16_kernel(const PivParams p, const uint4* __restrict__ consts)
{
    using S = Shape<GROUPS>;
    // peak scan range in swapped-plane coordinates (image_utils.impl.h:48,
    // :54; limited search: rect::dilate(0.5), rect.cpp:109-126)
    constexpr int D0 = LIMIT ? W / 4 : 0;
    constexpr int VW = LIMIT ? W / 2 : W;
    constexpr int SY0 = D0 + 1, SY1 = D0 + VW - 2;
    constexpr int SX0 = D0 + 1, SX1 = D0 + VW - 1;
    constexpr float kPix = F16 ? 0.0625f : 1.f;
    constexpr float kT = F16 ? 0.015625f : 1.f;
    constexpr float kSumUnscale = F16 ? 8192.f : 1.f;
    constexpr uint32_t kId1 = tcx::idesc_f16kind(128, 16, false, F16);
    constexpr uint32_t kId2 = tcx::idesc_f16kind(128, 32, true, F16);
    constexpr uint32_t kId3 = tcx::idesc_f16kind(64, 32, false, F16);
    constexpr uint32_t kId4 = tcx::idesc_f16kind(128, 16, true, F16);

    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* cst = smem;
    const int grp = (int)(threadIdx.x / kThreads);
    unsigned char* dat = smem + S::kConstBytes + grp * kGroupBytes;
    // row sums [frame][row] (exact integers: a row sum is an exact FP32
    // accumulator value, at most 2^20 for 16 16-bit pixels)
    float* rs = reinterpret_cast<float*>(dat + kDataBytes);
    int* escale = reinterpret_cast<int*>(rs + 128);                     // F16: product exponent per window
    uint64_t* mbar = reinterpret_cast<uint64_t*>(escale + kTile);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
    int* abort_flag = reinterpret_cast<int*>(tslot + 1);
    // the CTA's tensor-memory address lives in group 0's tail
    uint32_t* tslot_cta = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(tslot) - grp * kGroupBytes);

    const int tid = (int)threadIdx.x % kThreads, warp = tid >> 5, lane = tid & 31;
    auto gsync = [&]() { asm volatile("bar.sync %0, %1;" :: "r"(1 + grp), "r"(kThreads) : "memory"); };
    const uint32_t cst_a = tcx::smem_addr(cst), dat_a = tcx::smem_addr(dat);
    // descriptors: constant matrix m (hi part), the data buffer as the
    // MN-major stage-2 and stage-4 operands (K groups 2 KB apart) and the
    // K-major stage-3 operand (K = 32: 4 K groups per row group)
    const uint64_t dB = tcx::sdesc(cst_a, 128, 16 * W);
    auto mat = [&](int m) { return dB + (uint64_t)((m * kMat) >> 4); };
    const uint64_t dMN = tcx::sdesc(dat_a, 2048, 128);
    const uint64_t dK3 = tcx::sdesc(dat_a, 128, 512);
    auto off = [](int bytes) { return (uint64_t)(bytes >> 4); };

    for (int i = threadIdx.x; i < (CSPLIT ? 2 : 1) * kSet / 16; i += kThreads * GROUPS)
        reinterpret_cast<uint4*>(cst)[i] = consts[i];
    if (tid == 0) {
        tcx::mbar_init(mbar, 1);
        *abort_flag = 0;
    }
    if (threadIdx.x < 32) tcx::tmem_alloc(tslot_cta, S::kCols);
    tcx::fence_before();
    __syncthreads();
    tcx::fence_after();
    const uint32_t tcta = *tslot_cta;
    const uint32_t tbase = tcta + (uint32_t)grp * kGroupCols;
    const uint32_t tlane = tbase + ((uint32_t)(32 * warp) << 16);

    const PixT* fa = reinterpret_cast<const PixT*>(p.fa);
    const PixT* fb = reinterpret_cast<const PixT*>(p.fb);
    const size_t pitch = p.pitch / sizeof(PixT);
    // tiles: kTile consecutive windows of one grid column; each tile group
    // walks a contiguous range of tiles down the columns
    const int gny = (int)(p.n_win / p.gnx);
    const int per_line = (gny + kTile - 1) / kTile;
    const int n_tiles = p.gnx * per_line;
    const int64_t vb = (int64_t)blockIdx.x * GROUPS + grp, vg = (int64_t)gridDim.x * GROUPS;
    const int t_begin = (int)(vb * n_tiles / vg);
    const int t_end = (int)((vb + 1) * n_tiles / vg);
    uint32_t phase = 0;

    auto wait_mma = [&]() {
        // after a wait has given up, the tile finishes without waiting again
        if (!*abort_flag && !tcx::mbar_wait(mbar, phase)) {
            *abort_flag = 1;
            if (p.status) atomicExch(p.status, 1);
        }
        phase ^= 1u;
        tcx::fence_after();
    };

    // the tile's position, kept in registers by every thread: grid column
    // lc, first row lr (tile t: column t / per_line, rows kTile * (t %
    // per_line) + i)
    int lc = t_begin / per_line;
    int lr = kTile * (t_begin - lc * per_line);
    auto advance = [&](int& c, int& r) {
        r += kTile;
        if (r >= per_line * kTile) { r = 0; ++c; }
    };
    // window i of tile t at (c, r): its corner (x < 0: no window) and grid index
    auto window = [&](int t, int c, int r, int i, int& gi) {
        const int row = r + i;
        gi = row * p.gnx + c;
        return (t < t_end && c < p.gnx && row < gny) ? make_int2(p.gx0 + c * p.gdx, p.gy0 + row * p.gdy)
                                                     : make_int2(-1, -1);
    };

    for (int tile = t_begin; tile < t_end; ++tile, advance(lc, lr)) {
        int nc = lc, nr = lr;
        advance(nc, nr);
        auto org = [&](int i) { int gi; return window(tile, lc, lr, i, gi); };

        // image rows of this tile below its top (windows 0 .. nv - 1)
        const int nv = gny - lr < kTile ? gny - lr : kTile;
        const int vrows = (nv - 1) * p.gdy + W;

        // ---- stage-1 operand in tensor memory: thread tid owns lane tid =
        // row R = f * 64 + y.  A row's 16 pixels, widened (frame B rows
        // times (-1)^y), fill 8 columns of the hi part and 8 of the lo part:
        // pixel 2c in the low half of column c.
        {
            const int f = tid >> 6, y = tid & 63;
            const PixT* row = nullptr;
            const int2 o = org(0);
            if (y < vrows) row = (f ? fb : fa) + (size_t)(o.y + y) * pitch + o.x;
            typename Raw<PixT>::type raw[2] = { Raw<PixT>::zero(), Raw<PixT>::zero() };
            if (row) load16<PixT>(row, raw);
            const float sg = ((f && (y & 1)) ? -1.f : 1.f) * kPix;
            uint32_t w[16];
#pragma unroll
            for (int g = 0; g < 2; ++g) {
                float px[8];
                widen8<PixT>(raw[g], px, sg);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    w[4 * g + j] = pack2<F16>(px[2 * j], px[2 * j + 1]);
                    if (SPLIT) {
                        const float2 hf = unpack2<F16>(w[4 * g + j]);
                        w[8 + 4 * g + j] = pack2<F16>(px[2 * j] - hf.x, px[2 * j + 1] - hf.y);
                    } else {
                        w[8 + 4 * g + j] = 0u;
                    }
                }
            }
            tcx::tmem_st16(tlane + kA1, w);
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();
        if (*abort_flag) break;

        // ---- stage 1: H1 = X * G1^T, the operand X in tensor memory
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
            mma3_ta<SPLIT, CSPLIT>(tbase, tbase + kA1, tbase + kA1 + 8, mat(kTcG1), kId1);
            tcx::commit(mbar);
        }
        // the next tile's window rows into L2 while this tile computes
        {
            int gi;
            const int2 o = window(tile + 1, nc, nr, 0, gi);
            const int f = tid >> 6, y = tid & 63;
            if (o.x >= 0 && y < 7 * kMaxStep + W && o.y + y < p.img_h) {
                const PixT* q = (f ? fb : fa) + (size_t)(o.y + y) * pitch + o.x;
                asm volatile("prefetch.global.L2 [%0];" :: "l"(q));
            }
        }
        wait_mma();

        // ---- E1: each image row's coefficients into every window that
        // contains it: stage-2 operand, MN-major, M = 16 i + 8 f + k,
        // K = (U | V) x window row, core matrix (K group, M group) at
        // (K / 8) * 2048 + (M / 8) * 128; row sums into rs
        {
            float c[16];
            tcx::tmem_ld16(tlane, c);
            const int f = tid >> 6, y = tid & 63;
            if (y < vrows) {
                rs[f * 64 + y] = (f && (y & 1)) ? -c[0] : c[0];   // undo the frame-B row sign
                uint4 hi[2], lo[2];
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    if (SPLIT) split8<F16>(c + 8 * q, hi[q], lo[q]);
                    else hi[q] = round8<F16>(c + 8 * q);
                }
#pragma unroll
                for (int i = 0; i < kTile; ++i) {
                    const int yl = y - i * p.gdy;
                    if (i < nv && yl >= 0 && yl < W) {
                        // frame B: (-1)^y of the tile's row is (-1)^yl of the
                        // window's row times (-1)^(i gdy)
                        const uint32_t neg = (f && ((i * p.gdy) & 1)) ? 0x80008000u : 0u;
#pragma unroll
                        for (int part = 0; part < 2; ++part) {
                            const int o = (part * 2 + (yl >> 3)) * 2048 + (2 * i + f) * 128 + (yl & 7) * 16;
                            uint4 q = hi[part];
                            q.x ^= neg; q.y ^= neg; q.z ^= neg; q.w ^= neg;
                            *reinterpret_cast<uint4*>(dat + o) = q;
                            if (SPLIT) {
                                q = lo[part];
                                q.x ^= neg; q.y ^= neg; q.z ^= neg; q.w ^= neg;
                                *reinterpret_cast<uint4*>(dat + kLo + o) = q;
                            }
                        }
                    }
                }
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 2: conj of the column DFT (N = 32): the U part against
        // [C; S], the V part against [-S; C]
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
            mma3<SPLIT, CSPLIT>(tbase, dMN, mat(kTcC), kId2, false);
            mma3<SPLIT, CSPLIT>(tbase, dMN + off(2 * 2048), mat(kTcNS), kId2, true);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E2: products into the stage-3 operand (K-major, rows
        // (window, k_x) = 64, K = (Re | Im) x k_y = 32).  Lane = 16 s + 8 f
        // + k_x: window 2 warp + s, frame f.
        {
            const int s = lane >> 4, f = (lane >> 3) & 1, kxr = lane & 7;
            const int wi = 2 * warp + s;
            float x[32];   // [k_y] = Re X, [16 + k_y] = -Im X of this lane's (frame, k_x)
            tcx::tmem_ld32(tlane, x);
            // k_x slot 0 rows of both frames for the packed bins
            float* pk = reinterpret_cast<float*>(dat + kPacked) + wi * kPkWin;
            if (kxr == 0) {
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    *reinterpret_cast<float4*>(pk + f * 32 + 4 * j) =
                        make_float4(x[4 * j], x[4 * j + 1], x[4 * j + 2], x[4 * j + 3]);
            }
            // frame a's lane computes k_y = j, frame b's k_y = 8 + j (j < 8);
            // frame b's columns are rotated by 8, so both find their own values
            // at [j], [16 + j] and send their partner (lane ^ 8) those at
            // [8 + j], [24 + j].  With m = own, o = partner values and
            // n = -Im: Re P = m_r o_r + m_n o_n, Im P = +-(o_r m_n - o_n m_r),
            // + for frame a (A = m), - for frame b (A = o).
            const float sq = f ? -1.f : 1.f;
            float pr[8], pi[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float mr = x[j], mn = x[16 + j];
                const float orr = __shfl_xor_sync(0xffffffffu, x[8 + j], 8);
                const float onn = __shfl_xor_sync(0xffffffffu, x[24 + j], 8);
                float r = fmaf(mr, orr, mn * onn);
                float q = sq * fmaf(orr, mn, -(onn * mr));
                if (j & 1) { r = -r; q = -q; }   // quadrant sign (-1)^k_y
                if (MODE == kModeReal && j == 0) { r = 0.f; q = 0.f; }   // k_y = 0 or 8
                pr[j] = r;
                pi[j] = q;
            }
            __syncwarp();
            // packed row k_x = 0 | 8, one k_y per lane of the window's half
            float pkr, pkq;
            {
                const int ky = lane & 15, kn = (16 - ky) & 15;
                const float* sa = pk;          // frame a, k_x slot 0
                const float* sb = pk + 32;     // frame b, columns rotated by 8
                const int kb = (ky + 8) & 15, kbn = (kn + 8) & 15;
                // Z[k] = Re + i Im with Im = -stored
                const float zar = sa[ky], zai = -sa[16 + ky], zanr = sa[kn], zani = -sa[16 + kn];
                const float zbr = sb[kb], zbi = -sb[16 + kb], zbnr = sb[kbn], zbni = -sb[16 + kbn];
                // X0 = (Z[k] + conj Z[-k]) / 2, X8 = i (Z[k] - conj Z[-k]) / 2
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
            }
            if (F16) {
                // scale the window's products by 2^-e so that the largest is
                // in [2^8, 2^9): stage 3 sums 32 of them below FP16's 65504
                float m = fmaxf(fabsf(pkr), fabsf(pkq));
                if (kxr != 0) {
#pragma unroll
                    for (int j = 0; j < 8; ++j) m = fmaxf(m, fmaxf(fabsf(pr[j]), fabsf(pi[j])));
                }
#pragma unroll
                for (int o = 8; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
                const int eb = (int)((__float_as_uint(m) >> 23) & 0xffu);
                int e = eb == 0 ? 0 : eb - 127 - 8;
                e = e < -90 ? -90 : (e > 80 ? 80 : e);
                const float sc = __uint_as_float((uint32_t)(127 - e) << 23);
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    pr[j] *= sc;
                    pi[j] *= sc;
                }
                pkr *= sc;
                pkq *= sc;
                if ((lane & 15) == 0) escale[wi] = e;
            }
            if (kxr != 0) {
                const int R3 = wi * 8 + kxr;
#pragma unroll
                for (int part = 0; part < 2; ++part)
                    put8<F16, SPLIT>(dat, ((R3 >> 3) * 4 + part * 2 + f) * 128 + (R3 & 7) * 16, part ? pi : pr);
            }
            {
                const int ky = lane & 15, R0 = wi * 8;
                put1<F16, SPLIT>(dat, ((R0 >> 3) * 4 + (ky >> 3)) * 128 + (ky & 7) * 2, pkr);
                put1<F16, SPLIT>(dat, ((R0 >> 3) * 4 + ((16 + ky) >> 3)) * 128 + (ky & 7) * 2, pkq);
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 3: inverse column DFT (M = 64, N = 32): the Re part
        // against [C; S], the Im part against [-S; C]
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
            mma3<SPLIT, CSPLIT>(tbase, dK3, mat(kTcC), kId3, false);
            mma3<SPLIT, CSPLIT>(tbase, dK3 + off(2 * 128), mat(kTcNS), kId3, true);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E3: T into the stage-4 operand (MN-major, M = 16 i + y',
        // K = (Re | Im) x k_x = 16).  Rows 8 i + k_x of warp w sit in lanes
        // 0..15; lane = part * 16 + 8 s + k_x takes part (Re, Im) of the row.
        {
            const int part = lane >> 4, s = (lane >> 3) & 1, kx = lane & 7;
            const int wi = 2 * warp + s;
            float t1[16];
            tcx::tmem_ld16x2_16(tlane, t1);
            if (F16) {
#pragma unroll
                for (int i = 0; i < 16; ++i) t1[i] *= kT;
            }
            const int k = part * 8 + kx;
#pragma unroll
            for (int h = 0; h < 2; ++h) put8<F16, SPLIT>(dat, (k >> 3) * 2048 + (2 * wi + h) * 128 + (k & 7) * 16, t1 + 8 * h);
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 4: real inverse row DFT, D = T * C4 (N = 16)
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
            mma3<SPLIT, CSPLIT>(tbase, dMN, mat(kTcC4), kId4, false);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E4: find_peaks(plane, 2, 1), fit, vector; lane = 16 s + y'
        // of window 2 warp + s
        {
            const int s = lane >> 4, y = lane & 15;
            const int wi = 2 * warp + s;
            float* pl = reinterpret_cast<float*>(dat) + wi * (W * kPRow);
            int gw;
            const int2 ow = window(tile, lc, lr, wi, gw);
            float v[16];
            tcx::tmem_ld16(tlane, v);
            if (F16) {   // undo 2^-26 (pixels, stage-1 matrix, twice), 2^-e (product), 2^-6 (T)
                const float us = __uint_as_float((uint32_t)(127 + 32 + escale[wi]) << 23);
#pragma unroll
                for (int x = 0; x < W; ++x) v[x] *= us;
            }
            // strict 4-neighbour maxima of this row (rows above and below from
            // the neighbouring lanes of the same half: the scan excludes rows
            // 0 and 15), then the top two by a pairwise tree (ties: the lower
            // column)
            constexpr int NX = SX1 - SX0;
            float T0[NX], T1[NX];
            int I0[NX];
#pragma unroll
            for (int x = SX0; x < SX1; ++x) {
                const float c = v[x];
                const float up = __shfl_up_sync(0xffffffffu, c, 1);
                const float dn = __shfl_down_sync(0xffffffffu, c, 1);
                const float m = tcx::fmax3(up, dn, fmaxf(v[x - 1], v[x + 1]));
                T0[x - SX0] = (m < c) ? c : TC_NEG_INF;
                T1[x - SX0] = TC_NEG_INF;
                I0[x - SX0] = x;
            }
#pragma unroll
            for (int st = 1; st < NX; st *= 2)
#pragma unroll
                for (int i = 0; i + st < NX; i += 2 * st) {
                    const bool gt = T0[i + st] > T0[i];
                    const float lo = fminf(T0[i], T0[i + st]);
                    T1[i] = tcx::fmax3(T1[i], T1[i + st], lo);
                    I0[i] = gt ? I0[i + st] : I0[i];
                    T0[i] = gt ? T0[i + st] : T0[i];
                }
            const bool row_in = y >= SY0 && y < SY1;
            float t0 = row_in ? T0[0] : TC_NEG_INF, t1 = row_in ? T1[0] : TC_NEG_INF;
            const bool valid = ow.x >= 0;
            if (p.planes && valid) {
#pragma unroll
                for (int x = 0; x < W; ++x) p.planes[(size_t)gw * (W * W) + y * W + x] = v[x];
            }
            int key = y * W + I0[0];
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) {
                const float o0 = __shfl_xor_sync(0xffffffffu, t0, o);
                const float o1 = __shfl_xor_sync(0xffffffffu, t1, o);
                const int ok = __shfl_xor_sync(0xffffffffu, key, o);
                const bool take = (o0 > t0) || (o0 == t0 && ok < key);
                const float n1 = take ? fmaxf(t0, o1) : fmaxf(t1, o0);
                t0 = take ? o0 : t0;
                key = take ? ok : key;
                t1 = n1;
            }
            // fit_simple_gaussian: the peak row and its neighbours into shared
            // memory, six logarithms on six lanes of the half, relative to the
            // pedestal sum(a) sum(b) (REAL mode: none)
            const int px = key & (W - 1), py = key >> 4;
            if (y >= py - 1 && y <= py + 1) {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    *reinterpret_cast<float4*>(pl + y * kPRow + 4 * j) =
                        make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            }
            __syncwarp();
            // the window's pixel sums from the row sums (lane y: row y of both
            // frames, added over the 16 lanes of the half)
            int sum_a = __float2int_rn(rs[wi * p.gdy + y] * kSumUnscale);
            int sum_b = __float2int_rn(rs[64 + wi * p.gdy + y] * kSumUnscale);
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) {
                sum_a += __shfl_xor_sync(0xffffffffu, sum_a, o);
                sum_b += __shfl_xor_sync(0xffffffffu, sum_b, o);
            }
            const float ped = MODE == kModeReal ? 0.f : (float)sum_a * (float)sum_b;
            const int j = y < 6 ? y : 0;
            const int nx = (j == 2) ? px + 1 : (j < 2 ? px - 1 : px);
            const int ny = (j == 3 || j == 4) ? py - 1 : (j == 5 ? py + 1 : py);
            const int qx = (j == 0) ? px + 1 : px;
            const int qy = (j == 3) ? py + 1 : py;
            const float an = pl[(ny & 15) * kPRow + (nx & 15)];
            const float ad = pl[(qy & 15) * kPRow + (qx & 15)];
            const float lg = log1pf((an - ad) / (ad + ped));
            const int l0 = lane & 16;
            const float lxr = __shfl_sync(0xffffffffu, lg, l0 + 0);
            const float lxl = __shfl_sync(0xffffffffu, lg, l0 + 1);
            const float lxrr = __shfl_sync(0xffffffffu, lg, l0 + 2);
            const float lyd = __shfl_sync(0xffffffffu, lg, l0 + 3);
            const float lyu = __shfl_sync(0xffffffffu, lg, l0 + 4);
            const float lydd = __shfl_sync(0xffffffffu, lg, l0 + 5);
            if (y == 0 && valid) {
                opiv_vector out{ 0.f, 0.f, 0.f, 0.f, 0.f };
                int32_t code = -1;
                const int2 o = ow;
                const bool has2 = t1 > TC_NEG_INF;
                if (has2) {
                    const float vc = pl[py * kPRow + px];
                    const float C = vc + ped;
                    const float L = pl[py * kPRow + px - 1] + ped, R = pl[py * kPRow + px + 1] + ped;
                    const float U = pl[(py - 1) * kPRow + px] + ped, D = pl[(py + 1) * kPRow + px] + ped;
                    const float nan = __int_as_float(0x7fffffff);
                    const bool okx = L > 0.f && C > 0.f && R > 0.f;
                    const bool oky = U > 0.f && C > 0.f && D > 0.f;
                    const float fx = okx ? lxr / (2.f * (lxl + lxrr)) : nan;
                    const float fy = oky ? lyd / (2.f * (lyu + lydd)) : nan;
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
                if (p.peds) p.peds[gw] = MODE == kModeReal ? 0.0 : (double)sum_a * (double)sum_b;
            }
        }
        // no group barrier here: the next tile's pixel stage writes only the
        // stage-1 operand (tensor-memory columns that E4 does not read) in
        // this warp's own lanes and no shared memory; the barrier after it
        // orders E4 before the stage-1 MMA and the shared-memory writes
        tcx::fence_before();
    }
    tcx::fence_before();
    __syncthreads();
    tcx::fence_after();
    if (threadIdx.x < 32) tcx::tmem_dealloc(tcta, S::kCols);
}

// the vertical-tile form takes row steps 1 .. kMaxStep and window x
// positions on multiples of 4 pixels (16-pixel rows at 4-pixel alignment)
inline bool applicable(const PivParams& p)
{
    return p.gdy >= 1 && p.gdy <= kMaxStep && p.gx0 % 4 == 0 && p.gdx % 4 == 0 && p.pitch % 16 == 0 &&
           p.tc_tile != 2;
}

constexpr int kGroups = 8;

template <bool F16, bool SPLIT, bool CSPLIT, int MODE, bool LIMIT, typename PixT>
cudaError_t launch_t(const PivParams& p, const void* consts, cudaStream_t s)
{
    using S = Shape<kGroups>;
    auto kern = piv_tc16_kernel<F16, SPLIT, CSPLIT, MODE, LIMIT, PixT, kGroups>;
    static std::atomic<uint64_t> attr_done{ 0 };   // one bit per device
    static std::atomic<int> sm_count[64];
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(attr_done.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::kSmem);
        if (e != cudaSuccess) return e;
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        sm_count[dev & 63].store(sms);
        attr_done.fetch_or(bit);
    }
    const int64_t gny = p.n_win / p.gnx;
    const int64_t tiles = (int64_t)p.gnx * ((gny + kTile - 1) / kTile);
    const int64_t cap = sm_count[dev & 63].load();   // one CTA per SM
    const int64_t want = (tiles + kGroups - 1) / kGroups;
    const int blocks = (int)(want < cap ? want : cap);
    if (blocks <= 0) return cudaSuccess;
    kern<<<blocks, kThreads * kGroups, S::kSmem, s>>>(p, reinterpret_cast<const uint4*>(consts));
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

}  // namespace tc16
}  // namespace opiv
