// Tensor-core (tcgen05) PIV window path for 48 x 48 windows, one window per
// tile, BF16 or FP16 operands, split or plain (kernel templates; instantiated
// in piv_tc48.cu and piv_tc48_fp16.cu): the 64 px kernel's design
// (piv_tc64_kernel.cuh) at W = 48, H = 24 -- the 2-D cross-correlation of
// every window pair as four chained DFT matrix products
// (FFT::cross_correlate, fft.h:188-206, without its power-of-two
// restriction: a DFT matrix needs none), then find_peaks(plane, 2, 1), the
// 3-point Gaussian fit and the vector (image_utils.impl.h:42-101,
// main.cpp:214-236).  Any regular grid: a window row loads from the 16-byte
// blocks that cover it (load_row48).
//
// One CTA per SM runs kGroups independent tile groups of 4 warps sharing one
// copy of the constants; a group takes one window at a time, has 128
// tensor-memory columns (stage 1: accumulator 0..47, pixel operand 64..111;
// later accumulators 0..95) and a 25 KB data buffer.  Rows of the products
// (M = 64 rows sit in lanes 32 (r / 16) + r % 16):
//   stage 1  R = f * 64 + y, y < 48 (thread tid owns lane tid; rows 48..63
//            of each frame are zero)
//   stage 2  16 (k_x / 8) + 8 f + k_x % 8: warps 0..2 (rows 48..63 unused)
//   stage 3  transposed: (Re | Im) x y = 96 of 128 rows, N = 32 columns k_x
//            (24 used)
//   stage 4  y' (0..47 of 64 rows): warps 0..2, lanes y' % 16
// A thread of E2 owns twelve k_y of a row (three 4-column loads per quarter
// of the accumulator), so its stores are a full 8-value chunk and a half
// chunk.
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "piv_kernels.h"
#include "piv_tc_kernel.cuh"
#include "tc_ptx.cuh"

namespace opiv {
namespace tc48 {

using tc::pack2;
using tc::Raw;
using tc::round8;
using tc::split8;
using tc::unpack2;
using tc::widen8;

constexpr int W = 48;
constexpr int H = 24;
constexpr int kThreads = 128;
constexpr int kGroups = 4;
constexpr int kMat = W * W * 2;                 // one 48 x 48 matrix, K-major (4,608 bytes)
constexpr int kSet = kTcNumMat * kMat;
constexpr int kConstBytes = 2 * kSet;           // hi and lo parts (lo unused without the constant split)
constexpr int kLo = 12288;                      // lo-part offset of the operand buffers
constexpr int kPacked = 24576;                  // E2: k_x-slot-0 rows, 2 x 96 floats
constexpr int kDataBytes = kPacked + 2 * 96 * 4;
constexpr int kPS = W + 1;                      // E4 plane row stride (floats)
constexpr int kTailBytes = 1024;
constexpr int kGroupBytes = (kDataBytes + kTailBytes + 1023) / 1024 * 1024;
constexpr int kSmem = kConstBytes + kGroups * kGroupBytes;
constexpr uint32_t kGroupCols = 128;
constexpr uint32_t kA1 = 64;                    // TMEM column of the stage-1 operand (hi 24, then lo 24)
static_assert(kSmem <= 227 * 1024, "shared memory");
static_assert(kGroups * kGroupCols <= 512, "tensor memory");
static_assert(W * kPS * 4 <= kPacked, "plane below the packed rows");

// Tensor-memory moves for 24-column rows.  Every access starts on a column
// multiple of its own width (x4 on 4, x8 on 8, x16 on 16).

// 8 consecutive 32-bit columns of this warp's 32 lanes from registers
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t* w)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};\n"
                 "tcgen05.wait::st.sync.aligned;"
                 :: "r"(taddr), "r"(w[0]), "r"(w[1]), "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]),
                    "r"(w[7])
                 : "memory");
}

// Twelve columns from each of four bases under one wait (shape 16x32bx2,
// half-split offset 12, three 4-column loads per base): for base
// c_i = taddr.col + O_i, threads 0-15 get columns c_i .. c_i + 11 of lanes
// taddr.lane + t, threads 16-31 columns c_i + 12 .. c_i + 23 of the same
// lanes; v[12 i + j] holds column j of base i.
template <int O0, int O1, int O2, int O3>
__device__ __forceinline__ void tmem_ld16x2_12x4(uint32_t taddr, float* v)
{
    static_assert(O0 % 4 == 0 && O1 % 4 == 0 && O2 % 4 == 0 && O3 % 4 == 0, "4-column alignment");
    uint32_t r[48];
    asm volatile("tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%0,%1,%2,%3}, [%48], 12;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%4,%5,%6,%7}, [%49], 12;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%8,%9,%10,%11}, [%50], 12;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%12,%13,%14,%15}, [%51], 12;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%16,%17,%18,%19}, [%52], 12;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%20,%21,%22,%23}, [%53], 12;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%24,%25,%26,%27}, [%54], 12;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%28,%29,%30,%31}, [%55], 12;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%32,%33,%34,%35}, [%56], 12;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%36,%37,%38,%39}, [%57], 12;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%40,%41,%42,%43}, [%58], 12;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x4.b32 {%44,%45,%46,%47}, [%59], 12;\n"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
                   "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                   "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]),
                   "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]),
                   "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47])
                 : "r"(taddr + O0), "r"(taddr + O0 + 4), "r"(taddr + O0 + 8), "r"(taddr + O1),
                   "r"(taddr + O1 + 4), "r"(taddr + O1 + 8), "r"(taddr + O2), "r"(taddr + O2 + 4),
                   "r"(taddr + O2 + 8), "r"(taddr + O3), "r"(taddr + O3 + 4), "r"(taddr + O3 + 8)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 48; ++i) v[i] = __uint_as_float(r[i]);
}

// 24 columns per thread (shape 16x32bx2, half-split offset 24, three
// 8-column loads): threads 0-15 columns taddr.col .. +23 of lanes
// taddr.lane + t, threads 16-31 columns taddr.col + 24 .. +47
__device__ __forceinline__ void tmem_ld16x2_24(uint32_t taddr, float* v)
{
    uint32_t r[24];
    asm volatile("tcgen05.ld.sync.aligned.16x32bx2.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%24], 24;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%25], 24;\n"
                 "tcgen05.ld.sync.aligned.16x32bx2.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%26], 24;\n"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
                   "=r"(r[21]), "=r"(r[22]), "=r"(r[23])
                 : "r"(taddr), "r"(taddr + 8), "r"(taddr + 16)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 24; ++i) v[i] = __uint_as_float(r[i]);
}

// The 48 pixels of a window row as six raw 8-pixel words for widen8 (pixel
// 0 in the low bytes), from the aligned 16-byte blocks that cover the row.
// b, the row start's byte offset in its block, is the same for every row of
// a window and both frames (frames 16-byte aligned, pitch a multiple of 16:
// the host refuses other tensor-core passes), so the word select is uniform
// over the group; the last block read is the one holding the row's last
// pixel.
template <typename PixT, int S>
__device__ __forceinline__ void select_row48(const uint32_t* w, int sh, typename Raw<PixT>::type* raw)
{
    constexpr int NW = 12 * (int)sizeof(PixT);   // 32-bit words of a 48-pixel row
    uint32_t o[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j) o[j] = __funnelshift_r(w[S + j], w[S + j + 1], sh);
#pragma unroll
    for (int g = 0; g < 6; ++g) {
        if constexpr (sizeof(PixT) == 2) raw[g] = make_uint4(o[4 * g], o[4 * g + 1], o[4 * g + 2], o[4 * g + 3]);
        else raw[g] = make_uint2(o[2 * g], o[2 * g + 1]);
    }
}

template <typename PixT>
__device__ __forceinline__ void load_row48(const PixT* row, typename Raw<PixT>::type* raw)
{
    constexpr int NB = 3 * (int)sizeof(PixT) + 1;   // blocks covering a row at any offset: 7 or 4
    const uintptr_t a = reinterpret_cast<uintptr_t>(row);
    const int b = (int)(a & 15u);
    const uint4* blk = reinterpret_cast<const uint4*>(a - (uintptr_t)b);
    uint32_t w[4 * NB];
#pragma unroll
    for (int k = 0; k < NB - 1; ++k) {
        const uint4 q = __ldg(blk + k);
        w[4 * k] = q.x;
        w[4 * k + 1] = q.y;
        w[4 * k + 2] = q.z;
        w[4 * k + 3] = q.w;
    }
    // the row reaches into one more block only when it does not start on one
    uint4 q = make_uint4(0u, 0u, 0u, 0u);
    if (b != 0) q = __ldg(blk + NB - 1);
    w[4 * NB - 4] = q.x;
    w[4 * NB - 3] = q.y;
    w[4 * NB - 2] = q.z;
    w[4 * NB - 1] = q.w;
    const int sh = 8 * (b & 3);
    switch (b >> 2) {
    case 0: select_row48<PixT, 0>(w, sh, raw); break;
    case 1: select_row48<PixT, 1>(w, sh, raw); break;
    case 2: select_row48<PixT, 2>(w, sh, raw); break;
    default: select_row48<PixT, 3>(w, sh, raw); break;
    }
}

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

// 4 values into half a core-matrix row (8 bytes; hi, and lo kLo further)
template <bool F16, bool SPLIT>
__device__ __forceinline__ void put4(unsigned char* base, int off, const float* v)
{
    const uint32_t h0 = pack2<F16>(v[0], v[1]), h1 = pack2<F16>(v[2], v[3]);
    *reinterpret_cast<uint2*>(base + off) = make_uint2(h0, h1);
    if (SPLIT) {
        const float2 f0 = unpack2<F16>(h0), f1 = unpack2<F16>(h1);
        *reinterpret_cast<uint2*>(base + kLo + off) =
            make_uint2(pack2<F16>(v[0] - f0.x, v[1] - f0.y), pack2<F16>(v[2] - f1.x, v[3] - f1.y));
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
// lo*hi (a: data, b: constants; the data's lo part kLo further, the
// constants' one set further)
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
piv_tc48_kernel(const PivParams p, const uint4* __restrict__ consts)
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
    constexpr uint32_t kId1 = tcx::idesc_f16kind(128, 48, false, F16);
    constexpr uint32_t kId2 = tcx::idesc_f16kind(64, 96, true, F16);
    constexpr uint32_t kId3 = tcx::idesc_f16kind(128, 32, false, F16);
    constexpr uint32_t kId4 = tcx::idesc_f16kind(64, 48, false, F16);

    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* cst = smem;
    const int grp = (int)(threadIdx.x / kThreads);
    unsigned char* dat = smem + kConstBytes + grp * kGroupBytes;
    // row sums [frame][row] (exact integers: a row sum is an exact FP32
    // accumulator value, below 2^22 for 48 16-bit pixels)
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
    // groups 16 W = 768 bytes); the data buffer as the MN-major stage-2
    // operand (K groups 1 KB apart, 8 M groups of 128 bytes), the K-major
    // stage-3 operand (12 K groups per row group of k_x) and the K-major
    // stage-4 operand (6 K groups per row group of y')
    const uint64_t dB = tcx::sdesc(cst_a, 128, 16 * W);
    auto mat = [&](int m, int ks) { return dB + (uint64_t)((m * kMat + ks * 256) >> 4); };
    const uint64_t dMN = tcx::sdesc(dat_a, 1024, 128);
    const uint64_t dK3 = tcx::sdesc(dat_a, 128, 1536);
    const uint64_t dK4 = tcx::sdesc(dat_a, 128, 768);
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
        // row R = f * 64 + y.  The row's 48 pixels, widened (frame B rows
        // times (-1)^y), fill 24 columns of the hi part and 24 of the lo
        // part (pixel 2c in the low half of column c); rows y >= 48 zero.
        {
            const int f = tid >> 6, y = tid & 63;
            const float sg = ((f && (y & 1)) ? -1.f : 1.f) * kPix;
            uint32_t hw[24], lw[24];
            if (y < W) {
                typename Raw<PixT>::type raw[6];
                load_row48<PixT>((f ? fb : fa) + (size_t)(oy + y) * pitch + ox, raw);
#pragma unroll
                for (int g = 0; g < 6; ++g) {
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
            } else {
#pragma unroll
                for (int i = 0; i < 24; ++i) {
                    hw[i] = 0u;
                    lw[i] = 0u;
                }
            }
            // columns 64..87 (hi) and 88..111 (lo), each store on a multiple
            // of its width
            tcx::tmem_st16(tlane + kA1, hw);
            tmem_st8(tlane + kA1 + 16, hw + 16);
            if (SPLIT) {
                tmem_st8(tlane + kA1 + 24, lw);
                tcx::tmem_st16(tlane + kA1 + 32, lw + 8);
            }
        }
        tcx::fence_before();
        gsync();
        if (*abort_flag) break;

        // ---- stage 1: H1 = X * G1^T (K = 48 in three steps, N = 48)
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 3; ++ks)
                mma3_ta<SPLIT, CSPLIT>(tbase, tbase + kA1 + 8 * ks, tbase + kA1 + 24 + 8 * ks, mat(kTcG1, ks), kId1,
                                       ks > 0);
            tcx::commit(mbar);
        }
        // the next window's rows into L2 while this one computes
        if (win + 1 < w_end) {
            const int nc = gcol + 1 < p.gnx ? gcol + 1 : 0;
            const int nr = gcol + 1 < p.gnx ? grow : grow + 1;
            const int f = tid >> 6, y = tid & 63;
            if (y < W) {
                const PixT* q = (f ? fb : fa) + (size_t)(p.gy0 + nr * p.gdy + y) * pitch + p.gx0 + nc * p.gdx;
                asm volatile("prefetch.global.L2 [%0];" :: "l"(q));
            }
        }
        wait_mma();

        // ---- E1: the coefficients into the stage-2 operand: MN-major,
        // M = 16 j + 8 f + k % 8 (j = k / 8), K = (U | V) x y; core matrix
        // (K group, M group) at (K / 8) * 1024 + (M / 8) * 128; row sums
        {
            const int f = tid >> 6, y = tid & 63;
            float c[48];
            tcx::tmem_ld32(tlane, c);
            tcx::tmem_ld16(tlane + 32, c + 32);
            if (y < W) {
                rs[f * 64 + y] = (f && (y & 1)) ? -c[0] : c[0];   // undo the frame-B row sign
#pragma unroll
                for (int part = 0; part < 2; ++part)
#pragma unroll
                    for (int j = 0; j < 3; ++j)
                        put8<F16, SPLIT>(dat, (part * 6 + (y >> 3)) * 1024 + (2 * j + f) * 128 + (y & 7) * 16,
                                         c + 24 * part + 8 * j);
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 2: conj of the column DFT: the U part against [C; S],
        // the V part against [-S; C] (M = 64, N = 96, K = 96)
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 6; ++ks)
                mma3<SPLIT, CSPLIT>(tbase, dMN + off(ks * 2048), ks < 3 ? mat(kTcC, ks) : mat(kTcNS, ks - 3), kId2,
                                    ks > 0);
            tcx::commit(mbar);
        }
        wait_mma();

        // ---- E2: products into the stage-3 operand (K-major, rows k_x,
        // K = (Re | Im) x k_y = 96).  Warps 0..2; thread: row L = lane % 16
        // (frame L / 8, k_x = 8 warp + L % 8), half hh = lane / 16.
        int escale = 0;   // F16: the window's product exponent
        {
            const int L = lane & 15, hh = lane >> 4;
            const int f = L >> 3, kx = 8 * warp + (L & 7);
            const bool rows = warp < 3;   // warp 3 holds no k_x (rows 48..63 unused)
            float* pk = reinterpret_cast<float*>(dat + kPacked);   // [frame][Re 48 | -Im 48]
            const float sq = f ? -1.f : 1.f;
            // columns 12 hh + i (i < 12) of each quarter: q[i] Re, q[12 + i]
            // Re 24 further, q[24 + i] -Im, q[36 + i] -Im 24 further.  Frame
            // a's thread computes k_y = 12 hh + i, frame b's 24 more; frame b's
            // columns are rotated by 24, so both find their own values in
            // q[i], q[24 + i] and take their partner's (lane ^ 8) q[12 + i],
            // q[36 + i].  With m = own, o = partner values and n = -Im:
            // Re P = m_r o_r + m_n o_n, Im P = +-(o_r m_n - o_n m_r), + for
            // frame a.
            auto products = [&](const float* q, float* pr, float* pi) {
#pragma unroll
                for (int i = 0; i < 12; ++i) {
                    const float mr = q[i], mn = q[24 + i];
                    const float orr = __shfl_xor_sync(0xffffffffu, q[12 + i], 8);
                    const float onn = __shfl_xor_sync(0xffffffffu, q[36 + i], 8);
                    float r = fmaf(mr, orr, mn * onn);
                    float qq = sq * fmaf(orr, mn, -(onn * mr));
                    if (i & 1) { r = -r; qq = -qq; }   // quadrant sign (-1)^k_y
                    if (MODE == kModeReal && i == 0 && hh == 0) { r = 0.f; qq = 0.f; }   // k_y = 0 or 24
                    pr[i] = r;
                    pi[i] = qq;
                }
            };
            // the thread's twelve k_y from k0 = 24 f + 12 hh: hh = 0 a full
            // chunk then the low half of the next, hh = 1 the high half of a
            // chunk then a full one
            auto store = [&](const float* pr, const float* pi) {
                if (rows && kx != 0) {
                    const int rb = ((kx >> 3) * 12) * 128 + (kx & 7) * 16;
#pragma unroll
                    for (int part = 0; part < 2; ++part) {
                        const float* v = part ? pi : pr;
                        const int c0 = part * 6 + 3 * f + hh;   // chunk of k0
                        if (hh == 0) {
                            put8<F16, SPLIT>(dat, rb + c0 * 128, v);
                            put4<F16, SPLIT>(dat, rb + (c0 + 1) * 128, v + 8);
                        } else {
                            put4<F16, SPLIT>(dat, rb + c0 * 128 + 8, v);
                            put8<F16, SPLIT>(dat, rb + (c0 + 1) * 128, v + 4);
                        }
                    }
                }
            };
            // the packed row k_x = 0 | 24 (warp 0, k_y = lane, then lane + 32)
            auto packed = [&](int ky, float& pkr, float& pkq) {
                const float* sa = pk;         // frame a, k_x slot 0
                const float* sb = pk + 96;    // frame b, columns rotated by 24
                const int kn = ky == 0 ? 0 : W - ky;
                const int kb = ky < H ? ky + H : ky - H, kbn = kn < H ? kn + H : kn - H;
                // Z[k] = Re + i Im with Im = -stored
                const float zar = sa[ky], zai = -sa[48 + ky], zanr = sa[kn], zani = -sa[48 + kn];
                const float zbr = sb[kb], zbi = -sb[48 + kb], zbnr = sb[kbn], zbni = -sb[48 + kbn];
                // X0 = (Z[k] + conj Z[-k]) / 2, X24 = i (Z[k] - conj Z[-k]) / 2
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
            auto store_packed = [&](int ky, float pkr, float pkq) {
                put1<F16, SPLIT>(dat, (ky >> 3) * 128 + (ky & 7) * 2, pkr);
                put1<F16, SPLIT>(dat, ((48 + ky) >> 3) * 128 + (ky & 7) * 2, pkq);
            };
            float q[48], pr[12], pi[12];
            tmem_ld16x2_12x4<0, 24, 48, 72>(tlane, q);
            if (rows && kx == 0) {   // the k_x slot-0 rows for the packed bins
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int v4 = 0; v4 < 3; ++v4)
                        *reinterpret_cast<float4*>(pk + f * 96 + 24 * u + 12 * hh + 4 * v4) =
                            make_float4(q[12 * u + 4 * v4], q[12 * u + 4 * v4 + 1], q[12 * u + 4 * v4 + 2],
                                        q[12 * u + 4 * v4 + 3]);
            }
            products(q, pr, pi);
            float sc = 1.f;
            if constexpr (F16) {
                // the window's largest product over the warps, so that the
                // products scaled by 2^-e lie below 2^9
                float m = 0.f;
                if (rows && kx != 0) {
#pragma unroll
                    for (int i = 0; i < 12; ++i) m = fmaxf(m, fmaxf(fabsf(pr[i]), fabsf(pi[i])));
                }
                if (warp == 0) {
                    __syncwarp();
#pragma unroll
                    for (int h2 = 0; h2 < 2; ++h2) {
                        const int ky = lane + 32 * h2;
                        if (ky < W) {
                            float a2, b2;
                            packed(ky, a2, b2);
                            m = fmaxf(m, fmaxf(fabsf(a2), fabsf(b2)));
                        }
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
#pragma unroll
                for (int i = 0; i < 12; ++i) {
                    pr[i] *= sc;
                    pi[i] *= sc;
                }
            }
            store(pr, pi);
            if (warp == 0) {
                __syncwarp();
#pragma unroll
                for (int h2 = 0; h2 < 2; ++h2) {
                    const int ky = lane + 32 * h2;
                    if (ky < W) {
                        float a2, b2;
                        packed(ky, a2, b2);
                        store_packed(ky, a2 * sc, b2 * sc);
                    }
                }
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 3: inverse column DFT, transposed: the constants as the A
        // operand (M = 128 rows: Re T(y), Im T(y), 32 unused), the products as
        // the B operand (N = 32 rows k_x, 24 used; K = (Re | Im) x k_y = 96)
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 6; ++ks) {
                const uint64_t a = ks < 3 ? mat(kTcC, ks) : mat(kTcNS, ks - 3), b = dK3 + off(ks * 256);
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
        // x k_x = 48, core matrix (row group, K group) at (y' / 8) * 768 +
        // (K / 8) * 128).  Thread tid < 96 holds accumulator row tid = 48 part
        // + y: T_part(y, k_x), k_x < 24.
        {
            float t[32];
            tcx::tmem_ld32(tlane, t);
            if (tid < 2 * W) {
                const int part = tid >= W ? 1 : 0, y = tid - W * part;
                if (F16) {
#pragma unroll
                    for (int i = 0; i < 24; ++i) t[i] *= kT;
                }
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    put8<F16, SPLIT>(dat, ((y >> 3) * 6 + part * 3 + c) * 128 + (y & 7) * 16, t + 8 * c);
            }
        }
        tcx::fence_proxy();
        tcx::fence_before();
        gsync();

        // ---- stage 4: real inverse row DFT, D = T * C4 (M = 64, N = 48,
        // K = 48, the operand K-major)
        if (tid == 0 && !p.mma_skip) {
            tcx::fence_after();
#pragma unroll
            for (int ks = 0; ks < 3; ++ks)
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
            float v[24];
            tmem_ld16x2_24(tlane, v);
            if (y < W) {
                if (F16) {   // undo 2^-26 (pixels, stage-1 matrix, twice), 2^-e (products), 2^-6 (T)
                    const float us = __uint_as_float((uint32_t)(127 + 32 + escale) << 23);
#pragma unroll
                    for (int i = 0; i < 24; ++i) v[i] *= us;
                }
#pragma unroll
                for (int i = 0; i < 24; ++i) P[y * kPS + 24 * hh + i] = v[i];
                if (p.planes) {
                    const int gw = grow * p.gnx + gcol;
#pragma unroll
                    for (int i = 0; i < 24; i += 4)
                        *reinterpret_cast<float4*>(p.planes + (size_t)gw * (W * W) + y * W + 24 * hh + i) =
                            make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                }
            }
            // pixel sums: warps 0, 1 frame a, warps 2, 3 frame b (row 64 f + y)
            int s = (tid & 63) < W ? __float2int_rn(rs[tid] * kSumUnscale) : 0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) wsum[warp] = s;
        }
        tcx::fence_before();
        gsync();

        // ---- find_peaks: thread = (column x < 48 of 64, 24-row block); the
        // block's candidate rows roll through registers, neighbouring columns
        // come from the neighbouring lanes (the two edge lanes of a warp read
        // theirs); branch-free top two
        {
            const int xs = tid & 63, yb = (tid >> 6) * 24;
            const bool col_ok = xs >= SX0 && xs < SX1;
            const int y0 = yb > SY0 ? yb : SY0, y1 = yb + 24 < SY1 ? yb + 24 : SY1;   // uniform over the warp
            const int xl = xs == 0 ? W - 1 : xs - 1, xr = xs + 1 < W ? xs + 1 : 0;
            const int xc = xs < W ? xs : 0;   // columns 48..63 read column 0 (never candidates)
            Top2 s{ TC_NEG_INF, TC_NEG_INF, 0x7fffffff };
            float up = P[(y0 - 1) * kPS + xc], cc = P[y0 * kPS + xc];
#pragma unroll 4
            for (int ys = y0; ys < y1; ++ys) {
                const float dn = P[(ys + 1) * kPS + xc];
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
            const int px = has2 ? s.key % W : 1, py = has2 ? s.key / W : 1;
            // lane j's logarithm: ln(L/R), ln(L/C), ln(R/C), ln(U/D), ln(U/C), ln(D/C)
            const int j = lane < 6 ? lane : 0;
            const int nx = (j == 2) ? px + 1 : (j < 2 ? px - 1 : px);
            const int ny = (j == 3 || j == 4) ? py - 1 : (j == 5 ? py + 1 : py);
            const int qx = (j == 0) ? px + 1 : px;
            const int qy = (j == 3) ? py + 1 : py;
            const float an = P[ny * kPS + nx];
            const float ad = P[qy * kPS + qx];
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

// every regular grid; per-window positions and window offsetting are not
// tensor-core features (the exact pass and the FP32 multi-pass chains)
inline bool applicable(const PivParams& p) { return p.win_xy == nullptr && p.prev_disp == nullptr; }

template <bool F16, bool SPLIT, bool CSPLIT, int MODE, bool LIMIT, typename PixT>
cudaError_t launch_t(const PivParams& p, const void* consts, cudaStream_t s)
{
    auto kern = piv_tc48_kernel<F16, SPLIT, CSPLIT, MODE, LIMIT, PixT>;
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

}  // namespace tc48
}  // namespace opiv
