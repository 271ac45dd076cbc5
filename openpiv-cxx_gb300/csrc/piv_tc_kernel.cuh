// Tensor-core (tcgen05) PIV window path for 32 x 32 windows (kernel
// templates; instantiated per operand type in piv_tc_bf16.cu and
// piv_tc_fp16.cu, host side in piv_tc.cu): the 2-D
// cross-correlation of every window pair as four chained DFT matrix
// products, BF16 operands split into hi + lo parts (hi*hi + hi*lo + lo*hi,
// FP32 accumulation in tensor memory), then the reference's peak search,
// 3-point Gaussian fit and vector (image_utils.impl.h:42-101,
// main.cpp:214-236) on the CUDA cores.
//
// Mathematics (a, b: the two windows, rows y, columns x; all transforms
// unnormalised like FFT::cross_correlate, fft.h:188-206):
//   stage 1  row DFT of each window row as a real 32 x 32 product
//            H = X * G: coefficients U_k = sum_x X cos(2 pi k x / 32)
//            (k = 0..15), U_16 (coefficient (-1)^x), V_k = sum_x X sin(..)
//            (k = 1..15); U_16 takes the slot of V_0, which is zero.
//   stage 2  column DFT over y of the complex columns U_k - i V_k, as a
//            real product with K = (U | V) x y; for the slot k = 0 this
//            yields Z = DFT(U_0) - i DFT(U_16), unpacked by Hermitian
//            symmetry.  The stored result is the conjugate spectrum.
//   product  P = B conj(A) on the Hermitian half k_x = 0..16, the DC bin
//            removed (its contribution sum(a) sum(b) is a constant, the
//            pedestal, added back analytically in the fit), the k_y sign
//            (-1)^k_y that swaps the plane's quadrants folded in, P(k_y, 0)
//            and P(k_y, 16) packed as one complex column.
//   stage 3  inverse column DFT over k_y (complex, real product K = (Re |
//            Im) x k_y, N = (Re | Im) x y).
//   stage 4  real inverse row DFT (c2r) over k_x, the weights 1 / 2 / 1 and
//            the column quadrant swap folded into the constant matrix:
//            the result is the swap_quadrants'ed plane minus its pedestal.
//
// One CTA of 4 warps runs tiles of 4 windows; warp w owns tensor-memory
// lanes 32w .. 32w+31.  Every stage: CUDA cores write the operand (hi and
// lo parts) -- stage 1's pixels into tensor memory (tcgen05.st, each thread
// its own lane's image row), the later operands into shared memory
// (canonical no-swizzle layout) -- one thread issues the MMAs and commits
// them to an mbarrier, all threads wait (bounded) and read the accumulator
// back with tcgen05.ld.  Four CTAs (54 KB of shared memory, 128
// tensor-memory columns each: 64 of accumulators, 64 of stage-1 operand)
// share an SM, so the MMAs of some overlap the CUDA-core work of the others.
#pragma once

#include <atomic>
#include <cstdint>
#include <cstring>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "offsets.cuh"
#include "piv_kernels.h"
#include "tc_ptx.cuh"

namespace opiv {
namespace tc {

constexpr int W = 32;
constexpr int kThreads = 128;
constexpr int kTile = 4;                        // windows per tile
constexpr int kMat = 2048;                      // one 32 x 32 BF16 matrix, K-major
constexpr int kConstBytes = kTcNumMat * 2 * kMat;
constexpr int kDataBytes = 32 * 1024;   // stage-2 operand, hi and lo parts (its largest user)
constexpr int kTailBytes = 768;                 // sums, row sums, mbarrier, TMEM slot, flag, exponents
constexpr int kSmemBytes = kConstBytes + kDataBytes + kTailBytes;
constexpr uint32_t kTmemCols = 128;
constexpr uint32_t kA1 = 64;                    // TMEM column of the stage-1 operand (hi, then lo)
// Grouped form (vertical tiles): one CTA per SM runs kGroups independent
// groups of 4 warps, each doing what one CTA of the plain form does, sharing
// one copy of the constant matrices; a group has 64 tensor-memory columns
// (stage-1 accumulator in 0..31, its pixel operand in 32..63, later stages'
// accumulators in 0..63) and its own data buffer, tail, mbarrier and named
// barrier.  Six groups fit the SM's registers (768 threads at 80 each),
// shared memory and tensor memory, against four CTAs of the plain form.
constexpr int kGroups = 6;
constexpr uint32_t kGroupCols = 64;
constexpr uint32_t kA1Grouped = 32;
constexpr int kGroupBytes = (kDataBytes + kTailBytes + 1023) / 1024 * 1024;
constexpr int kSmemGrouped = kConstBytes + kGroups * kGroupBytes;
static_assert(kSmemGrouped <= 227 * 1024, "grouped form: shared memory");
static_assert(kGroups * kGroupCols <= 512, "grouped form: tensor memory");
constexpr int kLo = 16384;                      // lo-part offset of the operand buffers
constexpr int kPacked = 8192;                   // E2: k_x-slot-0 rows (after the stage-3 operand)
constexpr int kPRow = 36;                       // E4 plane row (floats), padded
// Vertical tiles at a row step of 8: window i's rows start at image row 8 i,
// the start of core-matrix row group i, so the stage-2 operand is one copy
// of the tile's 56 image rows that all four windows read.  MN-major, rows
// (frame, k) in M groups g of 8 (128 bytes apart), image rows in K groups of
// 8 (kRowGroup = 4 M groups apart), the U and V parts kRowsPart apart:
// window i's M group 4 i + g at K group j is the image's row group i + j.
constexpr int kRowGroup = 512;
constexpr int kRowsPart = 4096;
// One thread issues every MMA of a stage and commits them to the stage's
// mbarrier.  The MMAs of the other CTAs on the SM overlap a CTA's waits.

#define TC_NEG_INF (-__int_as_float(0x7f800000))

// byte offset of element (n, k) in a 32 x 32 K-major matrix
__host__ __device__ constexpr int kmaj32(int n, int k)
{
    return ((n >> 3) * 4 + (k >> 3)) * 128 + (n & 7) * 16 + (k & 7) * 2;
}

// Operand types of kind::f16: BF16 (F16 = false) or FP16 (F16 = true).
template <bool F16>
__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    uint32_t u;
    if (F16) {
        const __half2 h = __floats2half2_rn(a, b);
        u = *reinterpret_cast<const uint32_t*>(&h);
    } else {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        u = *reinterpret_cast<const uint32_t*>(&h);
    }
    return u;
}

template <bool F16>
__device__ __forceinline__ float2 unpack2(uint32_t u)
{
    if (F16) return __half22float2(*reinterpret_cast<const __half2*>(&u));
    return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u));
}

// hi / lo parts of 8 floats, packed for one 16-byte core-matrix row
template <bool F16>
__device__ __forceinline__ void split8(const float* v, uint4& hi, uint4& lo)
{
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        h[j] = pack2<F16>(v[2 * j], v[2 * j + 1]);
        const float2 hf = unpack2<F16>(h[j]);
        l[j] = pack2<F16>(v[2 * j] - hf.x, v[2 * j + 1] - hf.y);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// 8 floats rounded once (single-pass precision)
template <bool F16>
__device__ __forceinline__ uint4 round8(const float* v)
{
    return make_uint4(pack2<F16>(v[0], v[1]), pack2<F16>(v[2], v[3]), pack2<F16>(v[4], v[5]),
                      pack2<F16>(v[6], v[7]));
}

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

// D (+)= A * B with hi/lo splitting: hi*hi, then hi*lo (CSPLIT: the
// constant's lo part) and lo*hi.  a and b are descriptors of the hi parts;
// the start-address field counts 16-byte units, so a byte offset o is added
// as o >> 4 (no carry: shared addresses are below 2^18).
template <bool SPLIT, bool CSPLIT>
__device__ __forceinline__ void mma3(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, bool acc)
{
    tcx::mma_bf16(d, a, b, idesc, acc);
    if (SPLIT) {
        if (CSPLIT) tcx::mma_bf16(d, a, b + ((kTcNumMat * kMat) >> 4), idesc, true);
        tcx::mma_bf16(d, a + (kLo >> 4), b, idesc, true);
    }
}

// The same with the A operand (hi part a_hi, lo part a_lo) in tensor memory.
template <bool SPLIT, bool CSPLIT>
__device__ __forceinline__ void mma3_ta(uint32_t d, uint32_t a_hi, uint32_t a_lo, uint64_t b, uint32_t idesc,
                                        bool acc)
{
    tcx::mma_bf16_ta(d, a_hi, b, idesc, acc);
    if (SPLIT) {
        if (CSPLIT) tcx::mma_bf16_ta(d, a_hi, b + ((kTcNumMat * kMat) >> 4), idesc, true);
        tcx::mma_bf16_ta(d, a_lo, b, idesc, true);
    }
}

// 8 pixels of one window row: raw load, then exact widening to float (the
// integer in the low mantissa bits of 2^23, minus 2^23)
template <typename PixT> struct Raw;
template <> struct Raw<uint16_t> {
    using type = uint4;
    __device__ static uint4 zero() { return make_uint4(0, 0, 0, 0); }
};
template <> struct Raw<uint8_t> {
    using type = uint2;
    __device__ static uint2 zero() { return make_uint2(0, 0); }
};

template <typename PixT>
__device__ __forceinline__ typename Raw<PixT>::type load_raw(const PixT* ptr)
{
    return __ldg(reinterpret_cast<const typename Raw<PixT>::type*>(ptr));
}

template <typename PixT>
__device__ __forceinline__ void widen8(const typename Raw<PixT>::type& q, float* px, float s);

// s = +1 or -1: the pixels times s (one FMA each, like the subtraction)
template <>
__device__ __forceinline__ void widen8<uint16_t>(const uint4& q, float* px, float s)
{
    const uint32_t w[4] = { q.x, q.y, q.z, q.w };
    const float c = -8388608.f * s;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        // bytes {w.b0, w.b1, 0x00, 0x4b} and {w.b2, w.b3, 0x00, 0x4b}
        px[2 * j] = fmaf(__uint_as_float(__byte_perm(w[j], 0x4b00u, 0x5410u)), s, c);
        px[2 * j + 1] = fmaf(__uint_as_float(__byte_perm(w[j], 0x4b00u, 0x5432u)), s, c);
    }
}

template <>
__device__ __forceinline__ void widen8<uint8_t>(const uint2& q, float* px, float s)
{
    const uint32_t w[2] = { q.x, q.y };
    const float c = -8388608.f * s;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        px[j] = fmaf(__uint_as_float(__byte_perm(w[0], 0x4b00u, 0x5440u + j)), s, c);
        px[4 + j] = fmaf(__uint_as_float(__byte_perm(w[1], 0x4b00u, 0x5440u + j)), s, c);
    }
}

// VT: vertical tiles, four windows of one grid column (row step <= 8): their
// rows overlap, so stage 1 transforms each image row once (56 rows per frame
// instead of 4 x 32) and E1 copies its coefficients into every window that
// contains the row.  Otherwise four windows of one grid row.
// F16: FP16 operands scaled by powers of two to stay inside FP16's range
// (pixels x 2^-4, the stage-1 matrix x 2^-9 in the constants, the
// product x 2^-e with e chosen per window from its largest value, T x
// 2^-6), undone exactly in the peak stage.
// CSPLIT: the constants' lo parts enter too (three MMAs per product);
// otherwise only the data is split (two).
// GROUPS: 1 (one tile group per CTA, four CTAs per SM) or kGroups (the
// grouped form, vertical tiles only).
template <bool F16, bool SPLIT, bool CSPLIT, int MODE, bool LIMIT, typename PixT, bool VT, int GROUPS>
__global__ void __launch_bounds__(kThreads * GROUPS, GROUPS == 1 ? 4 : 1)
piv_tc_kernel(const PivParams p, const uint4* __restrict__ consts)
{
    static_assert(GROUPS == 1 || VT, "the grouped form takes vertical tiles");
    // tensor-memory columns: the stage-1 operand's first column, the CTA's
    // allocation
    constexpr uint32_t A1 = GROUPS == 1 ? kA1 : kA1Grouped;
    constexpr uint32_t kCols = GROUPS == 1 ? kTmemCols : 512;
    // peak scan range in swapped-plane coordinates (image_utils.impl.h:48,
    // :54; limited search: rect::dilate(0.5), rect.cpp:109-126)
    constexpr int D0 = LIMIT ? W / 4 : 0;
    constexpr int VW = LIMIT ? W / 2 : W;
    constexpr int SY0 = D0 + 1, SY1 = D0 + VW - 2;
    constexpr int SX0 = D0 + 1, SX1 = D0 + VW - 1;
    // FP16 scaling (powers of two): pixels, the stage-1 matrix (in the
    // constants), T; sums come out scaled by kPix * 2^-9
    constexpr float kPix = F16 ? 0.0625f : 1.f;
    constexpr float kT = F16 ? 0.015625f : 1.f;
    constexpr float kSumUnscale = F16 ? 8192.f : 1.f;
    constexpr uint32_t kIdK32 = tcx::idesc_f16kind(128, 32, false, F16);
    constexpr uint32_t kIdM32 = tcx::idesc_f16kind(128, 32, true, F16);
    // stage 3 has 64 rows: M = 64 puts row r in lane 32 (r / 16) + r % 16,
    // i.e. window w's 16 rows in the first 16 lanes of warp w
    constexpr uint32_t kIdK64M64 = tcx::idesc_f16kind(64, 64, false, F16);
    constexpr uint32_t kIdM64 = tcx::idesc_f16kind(128, 64, true, F16);

    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* cst = smem;
    // this thread's tile group: its data buffer and tail
    const int grp = GROUPS == 1 ? 0 : (int)(threadIdx.x / kThreads);
    unsigned char* dat = smem + kConstBytes + (GROUPS == 1 ? 0 : grp * kGroupBytes);
    // pixel sums [window][frame], exact integers: a row sum is an exact
    // FP32 accumulator value (integer pixels, at most 2^21 for 32 16-bit
    // pixels); the window sum (up to 2^26) is added in integers
    int* sums = reinterpret_cast<int*>(dat + kDataBytes);
    float* rs = reinterpret_cast<float*>(sums + 2 * kTile);             // VT: row sums [frame][row]
    uint64_t* mbar = reinterpret_cast<uint64_t*>(rs + 128);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
    int* abort_flag = reinterpret_cast<int*>(tslot + 1);
    int* escale = abort_flag + 1;                                       // F16: product exponent per window
    // the CTA's tensor-memory address lives in group 0's tail
    uint32_t* tslot_cta =
        reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(tslot) - (dat - (smem + kConstBytes)));

    // thread, warp and lane within the tile group (warp w of a group reads
    // tensor-memory lanes 32w .. 32w + 31, the quarter of CTA warp 4g + w)
    const int tid = (int)threadIdx.x % kThreads, warp = tid >> 5, lane = tid & 31;
    auto gsync = [&]() {
        if constexpr (GROUPS == 1) __syncthreads();
        else asm volatile("bar.sync %0, %1;" :: "r"(1 + grp), "r"(kThreads) : "memory");
    };
    const uint32_t cst_a = tcx::smem_addr(cst), dat_a = tcx::smem_addr(dat);
    // descriptors: constant matrix m (hi part; the lo parts follow all hi
    // parts), and the data buffer in the layouts of the four stages
    const uint64_t dB = tcx::sdesc(cst_a, 128, 512);
    auto mat = [&](int m, int ks) { return dB + (uint64_t)((m * kMat + ks * 256) >> 4); };
    const uint64_t dA2 = tcx::sdesc(dat_a, 2048, 128);    // MN-major, k-group stride 2 KB
    const uint64_t dA2s = tcx::sdesc(dat_a, kRowGroup, 128);   // shared image rows (row step 8)
    const uint64_t dA3 = tcx::sdesc(dat_a, 128, 1024);    // K-major, 8 k-groups per row group
    auto off = [](int bytes) { return (uint64_t)(bytes >> 4); };

    for (int i = threadIdx.x; i < kConstBytes / 16; i += kThreads * GROUPS)
        reinterpret_cast<uint4*>(cst)[i] = consts[i];
    if (tid == 0) {
        tcx::mbar_init(mbar, 1);
        *abort_flag = 0;
    }
    if (threadIdx.x < 32) tcx::tmem_alloc(tslot_cta, kCols);
    tcx::fence_before();
    __syncthreads();
    tcx::fence_after();
    const uint32_t tcta = *tslot_cta;
    const uint32_t tbase = tcta + (uint32_t)grp * kGroupCols;
    const uint32_t tlane = tbase + ((uint32_t)(32 * warp) << 16);

    const PixT* fa = reinterpret_cast<const PixT*>(p.fa);
    const PixT* fb = reinterpret_cast<const PixT*>(p.fb);
    const size_t pitch = p.pitch / sizeof(PixT);
    // tiles: kTile consecutive windows of one grid column (VT) or row; each
    // CTA walks a contiguous range of tiles down the grid, so consecutive
    // tiles share image rows, which the next tile then finds in L1
    const int gny = (int)(p.n_win / p.gnx);
    // tiles per walked line: a grid column of VT tiles, a grid row otherwise
    const int n_line = VT ? p.gnx : gny;
    const int per_line = VT ? (gny + kTile - 1) / kTile : (p.gnx + kTile - 1) / kTile;
    const int n_tiles = n_line * per_line;
    // each tile group walks its own contiguous range
    const int64_t vb = (int64_t)blockIdx.x * GROUPS + grp, vg = (int64_t)gridDim.x * GROUPS;
    const int t_begin = (int)(vb * n_tiles / vg);
    const int t_end = (int)((vb + 1) * n_tiles / vg);
    uint32_t phase = 0;

    // wait for the committed MMAs; a wait that gives up aborts the CTA
    auto wait_mma = [&]() {
        // after a wait has given up, the tile finishes without waiting again
        if (!*abort_flag && !tcx::mbar_wait(mbar, phase)) {
            *abort_flag = 1;
            if (p.status) atomicExch(p.status, 1);
        }
        phase ^= 1u;
        tcx::fence_after();
    };

    // vertical tiles at row step 8: one shared copy of the image rows
    const bool rows8 = VT && p.gdy == 8;
    // item mapping of the pixel stage: 8 consecutive lanes fill one core
    // matrix (rows R & 7), so the 16-byte stores are conflict-free
    const int it_r7 = tid & 7, it_g = (tid >> 3) & 3, it_rg = tid >> 5;

    // the tile's position, kept in registers by every thread (a group walks
    // a contiguous range of tiles): vertical tiles -- grid column lc, first
    // row lr (tile t: column t / per_line, rows kTile * (t % per_line) + i);
    // row tiles -- grid row lr, first column lc (tile t: row t % gny,
    // columns kTile * (t / gny) + i)
    int lc, lr;
    if (VT) {
        lc = t_begin / per_line;
        lr = kTile * (t_begin - lc * per_line);
    } else {
        const int c = t_begin / gny;
        lr = t_begin - c * gny;
        lc = kTile * c;
    }
    auto advance = [&](int& c, int& r) {
        if (VT) {
            r += kTile;
            if (r >= per_line * kTile) { r = 0; ++c; }
        } else if (++r >= gny) {
            r = 0;
            c += kTile;
        }
    };
    // window i of tile t at (c, r): its corner (x < 0: no window) and grid index
    auto window = [&](int t, int c, int r, int i, int& gi) {
        const int col = VT ? c : c + i, row = VT ? r + i : r;
        gi = row * p.gnx + col;
        return (t < t_end && col < p.gnx && row < gny) ? make_int2(p.gx0 + col * p.gdx, p.gy0 + row * p.gdy)
                                                       : make_int2(-1, -1);
    };

    for (int tile = t_begin; tile < t_end; ++tile, advance(lc, lr)) {
        int nc = lc, nr = lr;
        advance(nc, nr);
        auto org = [&](int i) { int gi; return window(tile, lc, lr, i, gi); };
        auto org_next = [&](int i) { int gi; return window(tile + 1, nc, nr, i, gi); };

        // number of window rows of this tile (VT: image rows below its top)
        const int vrows = VT ? (org(1).x >= 0 ? (org(2).x >= 0 ? (org(3).x >= 0 ? 3 : 2) : 1) : 0) * p.gdy + W
                             : 0;
        // ---- stage-1 operand in tensor memory: thread tid owns lane tid.
        // VT: row R = tid = f * 64 + y of the tile's image rows (y < vrows);
        // otherwise rows R = m1 * 128 + tid = (2 m1 + wl) * 64 + f * 32 + y.
        // A row's 32 pixels, widened (frame B rows times (-1)^y: its column
        // spectrum comes out rotated by 16 in k_y, see E2), fill 16 columns
        // of the hi part (and 16 of the lo part): pixel 2c in the low half
        // of column c.
        {
            constexpr int NM = VT ? 1 : 2;
#pragma unroll
            for (int m1 = 0; m1 < NM; ++m1) {
                const int R = m1 * 128 + tid;
                int f, y;
                const PixT* row = nullptr;
                if constexpr (VT) {
                    f = R >> 6;
                    y = R & 63;
                    const int2 o = org(0);
                    if (o.x >= 0 && y < vrows) row = (f ? fb : fa) + (size_t)(o.y + y) * pitch + o.x;
                } else {
                    f = (R >> 5) & 1;
                    y = R & 31;
                    const int2 o = org(R >> 6);
                    if (o.x >= 0) row = (f ? fb : fa) + (size_t)(o.y + y) * pitch + o.x;
                }
                typename Raw<PixT>::type raw[4];
#pragma unroll
                for (int g = 0; g < 4; ++g) raw[g] = row ? load_raw<PixT>(row + 8 * g) : Raw<PixT>::zero();
                const float sg = ((f && (y & 1)) ? -1.f : 1.f) * kPix;
                uint32_t hw[16], lw[16];
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                    float px[8];
                    widen8<PixT>(raw[g], px, sg);
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        hw[4 * g + j] = pack2<F16>(px[2 * j], px[2 * j + 1]);
                        if (SPLIT) {
                            const float2 hf = unpack2<F16>(hw[4 * g + j]);
                            lw[4 * g + j] = pack2<F16>(px[2 * j] - hf.x, px[2 * j + 1] - hf.y);
                        }
                    }
                }
                tcx::tmem_st16(tlane + A1 + 16 * m1, hw);
                if (SPLIT) tcx::tmem_st16(tlane + A1 + 16 * NM + 16 * m1, lw);
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();
        if (*abort_flag) break;

        // ---- stage 1: H = X * G, one (VT) or two M-tiles of 128 rows, the
        // operand X in tensor memory
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
            constexpr int NM = VT ? 1 : 2;
#pragma unroll
            for (int m1 = 0; m1 < NM; ++m1)
#pragma unroll
                for (int ks = 0; ks < 2; ++ks)
                    mma3_ta<SPLIT, CSPLIT>(tbase + 32 * m1, tbase + A1 + 16 * m1 + 8 * ks,
                                   tbase + A1 + 16 * NM + 16 * m1 + 8 * ks, mat(kTcG1, ks), kIdK32, ks > 0);
            tcx::commit(mbar);
        }
        // the next tile's window rows into L2 while this tile computes
        if constexpr (VT) {
            const int2 o = org_next(0);
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int R = (it_rg + 4 * t) * 8 + it_r7;
                const int f = t >> 1, y = R & 63;
                if (o.x >= 0 && y < 56 && o.y + y < p.img_h) {
                    const PixT* q = (f ? fb : fa) + (size_t)(o.y + y) * pitch + o.x + 8 * it_g;
                    asm volatile("prefetch.global.L2 [%0];" :: "l"(q));
                }
            }
        } else {
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int R = (it_rg + 4 * t) * 8 + it_r7;
                const int w = R >> 6, f = (R >> 5) & 1, y = R & 31;
                const int2 o = org_next(w);
                if (o.x >= 0) {
                    const PixT* q = (f ? fb : fa) + (size_t)(o.y + y) * pitch + o.x + 8 * it_g;
                    asm volatile("prefetch.global.L2 [%0];" :: "l"(q));
                }
            }
        }
        wait_mma();

        if constexpr (VT) {
            // ---- E1: each image row's coefficients into the stage-2 operand
            // (MN-major, rows (window, frame, k) = 128, K = (U | V) x window
            // row = 64): at row step 8 once, in the rows all windows share,
            // otherwise into every window that contains the row; row sums
            // into rs
            float c[32];
            tcx::tmem_ld32(tlane, c);
            const int f = warp >> 1, y = (warp & 1) * 32 + lane;
            if (y < vrows) {
                rs[f * 64 + y] = (f && (y & 1)) ? -c[0] : c[0];   // undo the frame-B row sign
                uint4 hi[4], lo[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (SPLIT) split8<F16>(c + 8 * q, hi[q], lo[q]);
                    else hi[q] = round8<F16>(c + 8 * q);
                }
                if (rows8) {   // once, in M group 2 f + h of row group y / 8
#pragma unroll
                    for (int part = 0; part < 2; ++part)
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const int o = part * kRowsPart + (y >> 3) * kRowGroup + (2 * f + h) * 128 + (y & 7) * 16;
                            *reinterpret_cast<uint4*>(dat + o) = hi[2 * part + h];
                            if (SPLIT) *reinterpret_cast<uint4*>(dat + kLo + o) = lo[2 * part + h];
                        }
                } else {
#pragma unroll
                    for (int i = 0; i < kTile; ++i) {
                        const int yl = y - i * p.gdy;
                        if (org(i).x >= 0 && yl >= 0 && yl < W) {
                            const int g0 = (i * 32 + f * 16) >> 3;
                            // frame B: the row sign (-1)^y of the tile's row
                            // is (-1)^yl of the window's row times
                            // (-1)^(i gdy); flip the sign bits where that is -1
                            const uint32_t neg = (f && ((i * p.gdy) & 1)) ? 0x80008000u : 0u;
#pragma unroll
                            for (int part = 0; part < 2; ++part) {
                                const int k = part * 32 + yl;
                                const int base = (k >> 3) * 2048 + (k & 7) * 16;
#pragma unroll
                                for (int h = 0; h < 2; ++h) {
                                    uint4 q = hi[2 * part + h];
                                    q.x ^= neg; q.y ^= neg; q.z ^= neg; q.w ^= neg;
                                    *reinterpret_cast<uint4*>(dat + base + (g0 + h) * 128) = q;
                                    if (SPLIT) {
                                        q = lo[2 * part + h];
                                        q.x ^= neg; q.y ^= neg; q.z ^= neg; q.w ^= neg;
                                        *reinterpret_cast<uint4*>(dat + kLo + base + (g0 + h) * 128) = q;
                                    }
                                }
                            }
                        }
                    }
                }
            }
        } else {
        // ---- E1: coefficients -> stage-2 operand (MN-major, rows
        // (window, frame, k) = 128, K = (U | V) x y = 64); row sums
        float c2[64];
        tcx::tmem_ld32x2(tlane, tlane + 32, c2, c2 + 32);
#pragma unroll
        for (int m1 = 0; m1 < 2; ++m1) {
            const float* c = c2 + 32 * m1;
            const int w = 2 * m1 + (warp >> 1), f = warp & 1;
            int s = __float2int_rn(((f && (lane & 1)) ? -c[0] : c[0]) * kSumUnscale);   // undo the frame-B row sign
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) sums[2 * w + f] = s;
            const int g0 = (w * 32 + f * 16) >> 3;
#pragma unroll
            for (int part = 0; part < 2; ++part) {
                const int k = part * 32 + lane;
                const int base = (k >> 3) * 2048 + (k & 7) * 16;
#pragma unroll
                for (int h = 0; h < 2; ++h) put8<F16, SPLIT>(dat, base + (g0 + h) * 128, c + part * 16 + h * 8);
            }
        }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 2: conj of the column DFT: Re = U*C + V*(-S),
        // -Im = U*S + V*C
        if (tid == 0 && !p.mma_skip) {   // N = 64: the U part against [C; S], the V part against [-S; C]
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                // K step ks: part ks / 2, window rows 16 (ks % 2) .. + 15
                const uint64_t a = rows8 ? dA2s + off((ks >> 1) * kRowsPart + (ks & 1) * 2 * kRowGroup)
                                         : dA2 + off(ks * 4096);
                mma3<SPLIT, CSPLIT>(tbase, a, mat(ks < 2 ? kTcC : kTcNS, ks & 1), kIdM64, ks > 0);
            }
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E2: products into the stage-3 operand (K-major, rows
        // (window, k_x) = 64, K = (Re | Im) x k_y = 64).  Warp w holds
        // window w: lane = frame * 16 + k_x.
        {
            const int w = warp;
            const int f = lane >> 4, kxr = lane & 15;
            float x[64];   // [k_y] = Re X, [32 + k_y] = -Im X of this lane's (frame, k_x)
            tcx::tmem_ld32x2(tlane, tlane + 32, x, x + 32);
            // k_x slot 0 rows of both frames for the packed bins
            float* pk = reinterpret_cast<float*>(dat + kPacked) + warp * 128;
            if (kxr == 0) {
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    *reinterpret_cast<float4*>(pk + f * 64 + 4 * j) =
                        make_float4(x[4 * j], x[4 * j + 1], x[4 * j + 2], x[4 * j + 3]);
            }
            // frame a's lane computes k_y = j, frame b's k_y = 16 + j (j < 16).
            // Frame b's columns are rotated by 16 (its rows were multiplied by
            // (-1)^y), so both lanes find their own values at [j], [32 + j]
            // and send their partner (lane ^ 16) the values at [16 + j],
            // [48 + j].  With m = own, o = partner values and n = -Im:
            // Re P = m_r o_r + m_n o_n, Im P = +-(o_r m_n - o_n m_r), the
            // sign + for frame a (A = m) and - for frame b (A = o).
            const float sq = f ? -1.f : 1.f;
            float pr[16], pi[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float mr = x[j], mn = x[32 + j];
                const float orr = __shfl_xor_sync(0xffffffffu, x[16 + j], 16);
                const float onn = __shfl_xor_sync(0xffffffffu, x[48 + j], 16);
                float r = fmaf(mr, orr, mn * onn);
                float q = sq * fmaf(orr, mn, -(onn * mr));
                if (j & 1) { r = -r; q = -q; }   // quadrant sign (-1)^k_y
                if (MODE == kModeReal && j == 0) { r = 0.f; q = 0.f; }   // k_y = 0 or 16
                pr[j] = r;
                pi[j] = q;
            }
            __syncwarp();
            // packed row k_x = 0 | 16, one k_y per lane
            float pkr, pkq;
            {
                const int ky = lane, kn = (32 - lane) & 31;
                const float* sa = pk;          // frame a, k_x slot 0
                const float* sb = pk + 64;     // frame b, columns rotated by 16
                const int kb = (ky + 16) & 31, kbn = (kn + 16) & 31;
                // Z[k] = Re + i Im with Im = -stored
                const float zar = sa[ky], zai = -sa[32 + ky], zanr = sa[kn], zani = -sa[32 + kn];
                const float zbr = sb[kb], zbi = -sb[32 + kb], zbnr = sb[kbn], zbni = -sb[32 + kbn];
                // X0 = (Z[k] + conj Z[-k]) / 2, X16 = i (Z[k] - conj Z[-k]) / 2
                const float a0r = 0.5f * (zar + zanr), a0i = 0.5f * (zai - zani);
                const float a6r = -0.5f * (zai + zani), a6i = 0.5f * (zar - zanr);
                const float b0r = 0.5f * (zbr + zbnr), b0i = 0.5f * (zbi - zbni);
                const float b6r = -0.5f * (zbi + zbni), b6i = 0.5f * (zbr - zbnr);
                // P = B conj(A)
                float p0r = b0r * a0r + b0i * a0i, p0i = b0i * a0r - b0r * a0i;
                float p6r = b6r * a6r + b6i * a6i, p6i = b6i * a6r - b6r * a6i;
                if (MODE == kModeReal) {
                    p0r = 0.f; p0i = 0.f;
                    if (ky == 0 || ky == 16) { p6r = 0.f; p6i = 0.f; }
                } else if (ky == 0) {
                    p0r = 0.f; p0i = 0.f;         // pedestal removed
                }
                // packed P(ky, 0) + i P(ky, 16), quadrant sign
                pkr = p0r - p6i;
                pkq = p0i + p6r;
                if (ky & 1) { pkr = -pkr; pkq = -pkq; }
            }
            if (F16) {
                // scale the window's products by 2^-e so that the largest is
                // in [2^8, 2^9): stage 3 sums 64 of them below FP16's 65504
                float m = fmaxf(fabsf(pkr), fabsf(pkq));
                if (kxr != 0) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) m = fmaxf(m, fmaxf(fabsf(pr[j]), fabsf(pi[j])));
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
                const int eb = (int)((__float_as_uint(m) >> 23) & 0xffu);
                int e = eb == 0 ? 0 : eb - 127 - 8;
                e = e < -90 ? -90 : (e > 80 ? 80 : e);
                const float sc = __uint_as_float((uint32_t)(127 - e) << 23);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    pr[j] *= sc;
                    pi[j] *= sc;
                }
                pkr *= sc;
                pkq *= sc;
                if (lane == 0) escale[w] = e;
            }
            if (kxr != 0) {
                const int R3 = w * 16 + kxr;
#pragma unroll
                for (int part = 0; part < 2; ++part)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int k = part * 32 + 16 * f + 8 * h;
                        put8<F16, SPLIT>(dat, ((R3 >> 3) * 8 + (k >> 3)) * 128 + (R3 & 7) * 16,
                                         (part ? pi : pr) + 8 * h);
                    }
            }
            {
                const int ky = lane, R0 = w * 16;
                put1<F16, SPLIT>(dat, ((R0 >> 3) * 8 + (ky >> 3)) * 128 + (ky & 7) * 2, pkr);
                put1<F16, SPLIT>(dat, ((R0 >> 3) * 8 + ((32 + ky) >> 3)) * 128 + (ky & 7) * 2, pkq);
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 3: inverse column DFT, Re T = Pr*C + Pi*(-S),
        // Im T = Pr*S + Pi*C (M = 64)
        if (tid == 0 && !p.mma_skip) {   // N = 64: the Pr part against [C; S], the Pi part against [-S; C]
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
                mma3<SPLIT, CSPLIT>(tbase, dA3 + off(ks * 256), mat(ks < 2 ? kTcC : kTcNS, ks & 1), kIdK64M64,
                            ks > 0);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E3: T into the stage-4 operand (MN-major, rows (window, y') =
        // 128, K = (Re | Im) x k_x = 32); warp w: its window's 16 rows
        // (k_x) sit in lanes 0..15, so lane = part * 16 + k_x takes the Re
        // (part 0) or Im (part 1) half of row k_x
        {
            const int w = warp, part = lane >> 4, kxr = lane & 15;
            float t1[32];
            tcx::tmem_ld16x2_32(tlane, t1);
            if (F16) {
#pragma unroll
                for (int i = 0; i < 32; ++i) t1[i] *= kT;
            }
            const int k = part * 16 + kxr;
            const int base = (k >> 3) * 2048 + (k & 7) * 16;
#pragma unroll
            for (int g = 0; g < 4; ++g) put8<F16, SPLIT>(dat, base + (w * 4 + g) * 128, t1 + 8 * g);
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 4: real inverse row DFT, D = T * C4
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 2; ++ks)
                mma3<SPLIT, CSPLIT>(tbase, dA2 + off(ks * 4096), mat(kTcC4, ks), kIdM32, ks > 0);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E4: find_peaks(plane, 2, 1), fit, vector; warp w, row y' = lane
        {
            float* pl = reinterpret_cast<float*>(dat) + warp * (32 * kPRow);
            const int w = warp;
            int gw;
            const int2 ow = window(tile, lc, lr, w, gw);
            const int y = lane;
            float v[32];
            tcx::tmem_ld32(tlane, v);
            if (F16) {   // undo 2^-26 (pixels, stage-1 matrix, twice), 2^-e (product), 2^-6 (T)
                const float us = __uint_as_float((uint32_t)(127 + 32 + escale[w]) << 23);
#pragma unroll
                for (int x = 0; x < W; ++x) v[x] *= us;
            }
            // strict 4-neighbour maxima of this row (rows above and below
            // from the neighbouring lanes), then the top two by a pairwise
            // tree (ties: the lower column)
            constexpr int NX = SX1 - SX0;
            float T0[NX], T1[NX];
            int I0[NX];
            {
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
            }
            const bool row_in = y >= SY0 && y < SY1;
            float t0 = row_in ? T0[0] : TC_NEG_INF, t1 = row_in ? T1[0] : TC_NEG_INF;
            const int tx = I0[0];
            const bool valid = ow.x >= 0;
            if (p.planes && valid) {
#pragma unroll
                for (int x = 0; x < W; ++x) p.planes[(size_t)gw * (W * W) + y * W + x] = v[x];
            }
            int key = y * W + tx;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float o0 = __shfl_xor_sync(0xffffffffu, t0, o);
                const float o1 = __shfl_xor_sync(0xffffffffu, t1, o);
                const int ok = __shfl_xor_sync(0xffffffffu, key, o);
                const bool take = (o0 > t0) || (o0 == t0 && ok < key);
                const float n1 = take ? fmaxf(t0, o1) : fmaxf(t1, o0);
                t0 = take ? o0 : t0;
                key = take ? ok : key;
                t1 = n1;
            }
            // fit_simple_gaussian: the peak row and its neighbours into
            // shared memory, six logarithms on six lanes, relative to the
            // pedestal sum(a) sum(b)
            const int px = key & (W - 1), py = key >> 5;
            if (y >= py - 1 && y <= py + 1) {
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    *reinterpret_cast<float4*>(pl + y * kPRow + 4 * j) =
                        make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            }
            __syncwarp();
            // the window's pixel sums: vertical tiles add their row sums here
            // (lane y: row y of both frames), row tiles took them in E1
            int sum_a, sum_b;
            if constexpr (VT) {
                sum_a = __float2int_rn(rs[w * p.gdy + y] * kSumUnscale);
                sum_b = __float2int_rn(rs[64 + w * p.gdy + y] * kSumUnscale);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    sum_a += __shfl_xor_sync(0xffffffffu, sum_a, o);
                    sum_b += __shfl_xor_sync(0xffffffffu, sum_b, o);
                }
            } else {
                sum_a = sums[2 * w];
                sum_b = sums[2 * w + 1];
            }
            // REAL mode: the reference's unpack zeroes spectrum row 0, so its
            // plane has no pedestal
            // the pedestal for the fit in FP32 (the exact integer sums rounded to
            // float: relative error below 2e-7, far inside the fit's tolerance; FP64
            // is slow on this part and only the optional pedestal output needs it)
            const float ped = MODE == kModeReal ? 0.f : (float)sum_a * (float)sum_b;
            const int j = lane < 6 ? lane : 0;
            // numerator / denominator positions of lane j's logarithm
            const int nx = (j == 2) ? px + 1 : (j < 2 ? px - 1 : px);
            const int ny = (j == 3 || j == 4) ? py - 1 : (j == 5 ? py + 1 : py);
            const int qx = (j == 0) ? px + 1 : px;
            const int qy = (j == 3) ? py + 1 : py;
            const float an = pl[(ny & 31) * kPRow + (nx & 31)];
            const float ad = pl[(qy & 31) * kPRow + (qx & 31)];
            const float lg = log1pf((an - ad) / (ad + ped));
            const float lxr = __shfl_sync(0xffffffffu, lg, 0);
            const float lxl = __shfl_sync(0xffffffffu, lg, 1);
            const float lxrr = __shfl_sync(0xffffffffu, lg, 2);
            const float lyd = __shfl_sync(0xffffffffu, lg, 3);
            const float lyu = __shfl_sync(0xffffffffu, lg, 4);
            const float lydd = __shfl_sync(0xffffffffu, lg, 5);
            if (lane == 0 && valid) {
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
    if (threadIdx.x < 32) tcx::tmem_dealloc(tcta, kCols);
}

template <bool F16, bool SPLIT, bool CSPLIT, int MODE, bool LIMIT, typename PixT, bool VT>
cudaError_t launch_t(const PivParams& p, const void* consts, cudaStream_t s)
{
    // vertical tiles run the grouped form (one CTA of kGroups tile groups
    // per SM), row tiles the plain form (four CTAs per SM)
    constexpr int G = VT ? kGroups : 1;
    constexpr int kSmem = G == 1 ? kSmemBytes : kSmemGrouped;
    auto kern = piv_tc_kernel<F16, SPLIT, CSPLIT, MODE, LIMIT, PixT, VT, G>;
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
    const int64_t gny = p.n_win / p.gnx;
    const int64_t tiles = VT ? (int64_t)p.gnx * ((gny + kTile - 1) / kTile)
                             : gny * ((p.gnx + kTile - 1) / kTile);
    // four CTAs per SM (plain form) or one (grouped form)
    const int64_t cap = (G == 1 ? 4 : 1) * (int64_t)sm_count[dev & 63].load();
    const int64_t want = (tiles + G - 1) / G;
    const int blocks = (int)(want < cap ? want : cap);
    if (blocks <= 0) return cudaSuccess;
    kern<<<blocks, kThreads * G, kSmem, s>>>(p, reinterpret_cast<const uint4*>(consts));
    return cudaGetLastError();
}

template <bool F16, bool SPLIT, bool CSPLIT, int MODE, bool LIMIT>
cudaError_t by_dtype(const PivParams& p, int dtype, const void* consts, cudaStream_t s)
{
    // four stacked windows span <= 56 rows; the plan may ask for row tiles
    const bool vt = p.tc_tile != 2 && p.gdy > 0 && p.gdy <= 8;
    if (dtype == kU8)
        return vt ? launch_t<F16, SPLIT, CSPLIT, MODE, LIMIT, uint8_t, true>(p, consts, s)
                  : launch_t<F16, SPLIT, CSPLIT, MODE, LIMIT, uint8_t, false>(p, consts, s);
    return vt ? launch_t<F16, SPLIT, CSPLIT, MODE, LIMIT, uint16_t, true>(p, consts, s)
              : launch_t<F16, SPLIT, CSPLIT, MODE, LIMIT, uint16_t, false>(p, consts, s);
}

// SPLIT: hi / lo data (and, with CSPLIT, constant) parts
template <bool F16, bool SPLIT, bool CSPLIT = SPLIT>
cudaError_t by_mode(const PivParams& p, int dtype, int mode, int limit, const void* consts,
                    cudaStream_t s)
{
    if (mode == kModeReal)
        return limit ? by_dtype<F16, SPLIT, CSPLIT, kModeReal, true>(p, dtype, consts, s)
                     : by_dtype<F16, SPLIT, CSPLIT, kModeReal, false>(p, dtype, consts, s);
    return limit ? by_dtype<F16, SPLIT, CSPLIT, kModeComplex, true>(p, dtype, consts, s)
                 : by_dtype<F16, SPLIT, CSPLIT, kModeComplex, false>(p, dtype, consts, s);
}

}  // namespace tc
}  // namespace opiv
