// piv_exact.cu -- exact double-precision window kernel for sm_103a.
//
// Repeats the reference's double arithmetic operation for operation, so its
// correlation planes are bit-identical to OpenPIV-c++ built without fused
// multiply-add contraction:
//   * 2-D FFT = radix-2 DIT on every row, then every column (fft.h:87-119),
//     with the same butterfly graph as the recursive fft_inner
//     (fft.h:245-263): e + o*w, e - o*w, w = table[k * 2n/len], where the
//     table entries exp(-+i*pi*j/n) are computed on the host with the
//     reference's own expression (fft.h:274-294);
//   * complex product (a*c - b*d, b*c + a*d) (pixel_types.h:159-163), every
//     multiply and add rounded separately (__dmul_rn / __dadd_rn, no FMA);
//   * REAL mode: the partial two-for-one unpack of fft.h:163-183;
//   * swap_quadrants (image_utils.impl.h:367-386) as an index remap;
//   * find_peaks (image_utils.impl.h:42-74) with exact comparisons; among
//     equal values the first peak is the one std::sort puts first (its
//     introsort is replayed, sort_order.h);
//   * fit_simple_gaussian (impl:77-101) and the vector of main.cpp:220-236
//     in double.
//
// It serves two purposes: it re-decides the windows the FP32 kernel flagged
// as uncertain, and it is the device FP64 correlation used by the exact
// per-window API.  One CTA of 256 threads handles one window at a time;
// CTAs stride over the work list.  FP64 is slow on this part, so the hot path only sends
// the rare flagged windows here.

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "offsets.cuh"
#include "piv_kernels.h"
#include "sort_order.h"

namespace opiv {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxW = 64;

__device__ __forceinline__ double2 e_add(double2 a, double2 b)
{
    return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y));
}
__device__ __forceinline__ double2 e_sub(double2 a, double2 b)
{
    return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y));
}
// (a + ib)(c + id) = (a*c - b*d, b*c + a*d), pixel_types.h:159-163
__device__ __forceinline__ double2 e_mul(double2 p, double2 q)
{
    return make_double2(__dsub_rn(__dmul_rn(p.x, q.x), __dmul_rn(p.y, q.y)),
                        __dadd_rn(__dmul_rn(p.y, q.x), __dmul_rn(p.x, q.y)));
}
__device__ __forceinline__ double2 e_conj(double2 a) { return make_double2(a.x, -a.y); }

__device__ __forceinline__ double px_d(const uint8_t* p) { return (double)__ldg(p); }
__device__ __forceinline__ double px_d(const uint16_t* p) { return (double)__ldg(p); }
__device__ __forceinline__ double px_d(const float* p) { return (double)__ldg(p); }
__device__ __forceinline__ double px_d(const double* p) { return __ldg(p); }

// Radix-2 DIT transforms of all W lines of a W x W tile, in place, every
// thread of the block cooperating: rows when (s_line, s_elem) = (W, 1),
// columns when (1, W).  Per line this is the butterfly graph of fft_inner
// (bit-reversal, then stages len = 2 .. W combining e + o*w, e - o*w with
// w = tw[k * 2W/len]); spreading butterflies over threads changes no
// operation and no operand.  tw: table of W entries exp(-+i*pi*j/W).
__device__ void dit_lines(double2* X, int W, int lg, int s_line, int s_elem, const double2* tw)
{
    const int t = threadIdx.x, T = blockDim.x;
    for (int q = t; q < W * W; q += T) {
        const int line = q / W, i = q % W;
        const int j = (int)(__brev((unsigned)i) >> (32 - lg));
        if (i < j) {
            double2* x = X + line * s_line;
            const double2 v = x[i * s_elem];
            x[i * s_elem] = x[j * s_elem];
            x[j * s_elem] = v;
        }
    }
    __syncthreads();
    const int nb = W / 2;   // butterflies per line and stage
    for (int len = 2; len <= W; len <<= 1) {
        const int half = len >> 1, tstep = (2 * W) / len;
        for (int q = t; q < W * nb; q += T) {
            const int line = q / nb, b = q % nb;
            const int base = (b / half) * len, k = b % half;
            double2* x = X + line * s_line;
            const double2 e = x[(base + k) * s_elem];
            const double2 o = e_mul(x[(base + k + half) * s_elem], tw[k * tstep]);
            x[(base + k) * s_elem] = e_add(e, o);
            x[(base + k + half) * s_elem] = e_sub(e, o);
        }
        __syncthreads();
    }
}

// 2-D transform: every row, then every column (fft.h:104-116).
__device__ void fft2d(double2* X, int W, const double2* tw)
{
    int lg = 0;
    while ((1 << lg) < W) ++lg;
    dit_lines(X, W, lg, W, 1, tw);
    dit_lines(X, W, lg, 1, W, tw);
}

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

// fit_simple_gaussian's axis function, image_utils.impl.h:86-94
__device__ __forceinline__ double gauss3(double l, double c, double r)
{
    const double num = log(l) - log(r);
    const double den = 2.0 * (log(l) + log(r) - 2.0 * log(c));
    if (den == 0.0) return 0.0;
    return num / den;
}

// One window w of pair p, by the whole CTA (A, B: 2 W^2 double2 of shared
// memory; row_count: W ints; total_cand: one int, both shared).
template <typename PixT>
__device__ __forceinline__ void exact_window(const PivParams& p, const int64_t w, const int W, const int mode,
                                             const int sy0, const int sy1, const int sx0, const int sx1,
                                             double2* A, double2* B, int* row_count, int* total_cand)
{
    const int t = threadIdx.x;
    const int N = W * W;
    const PixT* fa = reinterpret_cast<const PixT*>(p.fa);
    const PixT* fb = reinterpret_cast<const PixT*>(p.fb);
    const size_t pitch = p.pitch / sizeof(PixT);
    int bx, by, ox, oy;
    window_origin(p, w, bx, by);
    b_offset(p, W, bx, by, ox, oy);

    // ---- extract, convert (g_f by value), join / convert to complex
    for (int i = t; i < N; i += blockDim.x) {
        const int y = i / W, x = i % W;
        const double a = px_d(fa + (size_t)(by + y) * pitch + bx + x);
        const double b = px_d(fb + (size_t)(by + oy + y) * pitch + bx + ox + x);
        if (mode == kModeComplex) {
            A[i] = make_double2(a, 0.0);
            B[i] = make_double2(b, 0.0);
        } else {
            A[i] = make_double2(a, b);
        }
    }
    __syncthreads();

    fft2d(A, W, p.tw_fwd);
    if (mode == kModeComplex) {
        fft2d(B, W, p.tw_fwd);
        for (int i = t; i < N; i += blockDim.x) A[i] = e_mul(B[i], e_conj(A[i]));
    } else {
        // transform_real's unpack (fft.h:166-183) fused with the product;
        // each (k, -k) pair is owned by one thread.  Cells outside the
        // unpacked set (row 0, row W/2, column 0) become zero.
        const int npairs = (W / 2 - 1) * (W - 1);
        for (int q = t; q < npairs; q += blockDim.x) {
            const int h = 1 + q / (W - 1), x = 1 + q % (W - 1);
            const int k = h * W + x, m = (W - h) * W + (W - x);
            const double2 t1 = A[k], t2 = A[m];
            const double2 half = make_double2(0.5, 0.0);
            const double2 av = e_mul(half, e_add(t1, e_conj(t2)));
            double2 bv = e_mul(half, e_sub(t1, e_conj(t2)));
            bv = make_double2(bv.y, __dmul_rn(-1.0, bv.x));
            A[k] = e_mul(bv, e_conj(av));
            A[m] = e_mul(e_conj(bv), e_conj(e_conj(av)));
        }
        for (int i = t; i < N; i += blockDim.x) {
            const int y = i / W, x = i % W;
            if (y == 0 || y == W / 2 || x == 0) A[i] = make_double2(0.0, 0.0);
        }
        __syncthreads();
    }
    __syncthreads();
    fft2d(A, W, p.tw_rev);

    // ---- real part, quadrant swap -> plane in B[].x (row-major)
    for (int i = t; i < N; i += blockDim.x) {
        const int y = i / W, x = i % W;
        const int sy = (y + W / 2) % W, sx = (x + W / 2) % W;
        B[i].x = A[sy * W + sx].x;
    }
    __syncthreads();
    if (p.planes64 != nullptr)
        for (int i = t; i < N; i += blockDim.x) p.planes64[(size_t)w * N + i] = B[i].x;

    // ---- find_peaks: strict 4-neighbour maxima of the scanned rows, in
    // row-major scan order (the order the reference pushes them), then
    // std::sort's choice of the first one (sort_order.h) and the second
    // largest value (with multiplicity) for sn.
    peak_cand* cand = reinterpret_cast<peak_cand*>(A);   // A is free now
    int my_count = 0;
    const int y = t;
    const bool row_ok = t < W && y >= sy0 && y < sy1;
    if (row_ok) {
        for (int x = sx0; x < sx1; ++x) {
            const double c = B[y * W + x].x;
            if (B[y * W + x - 1].x < c && B[y * W + x + 1].x < c &&
                B[(y - 1) * W + x].x < c && B[(y + 1) * W + x].x < c)
                ++my_count;
        }
    }
    if (t < W) row_count[t] = my_count;
    __syncthreads();
    if (t == 0) {
        int acc = 0;
        for (int r = 0; r < W; ++r) {
            const int c = row_count[r];
            row_count[r] = acc;
            acc += c;
        }
        (*total_cand) = acc;
    }
    __syncthreads();
    if (row_ok) {
        int o = row_count[t];
        for (int x = sx0; x < sx1; ++x) {
            const double c = B[y * W + x].x;
            if (B[y * W + x - 1].x < c && B[y * W + x + 1].x < c &&
                B[(y - 1) * W + x].x < c && B[(y + 1) * W + x].x < c)
                cand[o++] = peak_cand{ c, y * W + x };
        }
    }
    __syncthreads();
    if (t == 0) {
        const int n = (*total_cand);
        const double ninf = -__longlong_as_double(0x7ff0000000000000ll);
        double g0 = ninf, g1 = ninf;   // two largest values, with multiplicity
        for (int i = 0; i < n; ++i) {
            const double c = cand[i].v;
            if (c > g0) { g1 = g0; g0 = c; }
            else if (c > g1) g1 = c;
        }
        int k = -1;
        if (n >= 2) {
            sort_order_head(cand, n);
            k = cand[0].key;
        }
        const int count = n >= 2 ? 2 : n;
        opiv_vector out{ 0.f, 0.f, 0.f, 0.f, 0.f };
        int32_t code = -1;
        if (count == 2) {
            const int px = k % W, py = k / W;
            const double c = B[py * W + px].x;
            const double lx = (double)px + gauss3(B[py * W + px - 1].x, c, B[py * W + px + 1].x);
            const double ly = (double)py + gauss3(B[(py - 1) * W + px].x, c, B[(py + 1) * W + px].x);
            const int mx = bx + W / 2, my = by + W / 2;
            out.x = (float)mx;
            out.y = (float)((double)p.img_h - (double)my);
            out.u = (float)((double)mx - ((double)bx + lx) - (double)ox);
            out.v = (float)((double)my - ((double)by + ly) - (double)oy);
            out.sn = (g1 > 0) ? (float)(g0 / g1) : 0.f;
            code = k | OPIV_PEAK_EXACT;
        }
        if (p.out_vec) p.out_vec[w] = out;
        if (p.out_peak) p.out_peak[w] = code;
        if (p.out_disp)
            p.out_disp[w] = count == 2 ? pack_disp(k % W - W / 2 + ox, k / W - W / 2 + oy)
                                       : pack_disp(ox, oy);
    }
    __syncthreads();
}

// scan range in plane coordinates (find_peaks on the plane or on its
// centre view rect().dilate(0.5); rect.cpp:109-126)
__device__ __forceinline__ void scan_range(int W, int limit, int& sy0, int& sy1, int& sx0, int& sx1)
{
    int d0 = 0, vw = W;
    if (limit) {
        const int rw = (int)lround(0.5 * W);
        d0 = (W - rw) / 2;
        vw = rw;
    }
    sy0 = d0 + 1;
    sy1 = d0 + vw - 2;
    sx0 = d0 + 1;
    sx1 = d0 + vw - 1;
}

template <typename PixT>
__global__ void __launch_bounds__(kThreads)
piv_exact_kernel(const PivParams p, int W, int mode, int limit, bool use_list)
{
    extern __shared__ double2 sm[];
    __shared__ int row_count[kMaxW];
    __shared__ int total_cand;
    const int64_t nwork = use_list ? (int64_t)(*p.flag_count) : p.n_win;
    int sy0, sy1, sx0, sx1;
    scan_range(W, limit, sy0, sy1, sx0, sx1);
    for (int64_t item = blockIdx.x; item < nwork; item += gridDim.x) {
        const int64_t w = use_list ? (int64_t)p.flag_list[item] : item;
        exact_window<PixT>(p, w, W, mode, sy0, sy1, sx0, sx1, sm, sm + W * W, row_count, &total_cand);
    }
}

// The exact pass of a work queue: every pair's flagged windows, one list
// (combined window numbers), CTAs striding over it.
template <typename PixT>
__global__ void __launch_bounds__(kThreads)
piv_exact_queue_kernel(const __grid_constant__ PivQueue q, int W, int mode, int limit)
{
    extern __shared__ double2 sm[];
    __shared__ int row_count[kMaxW];
    __shared__ int total_cand;
    const int64_t nwork = (int64_t)(*q.flag_count);
    int sy0, sy1, sx0, sx1;
    scan_range(W, limit, sy0, sy1, sx0, sx1);
    for (int64_t item = blockIdx.x; item < nwork; item += gridDim.x) {
        const int g = q.flag_list[item];
        int lo = 0, hi = q.n_items - 1;   // pair of combined window g
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (q.first_win[mid] <= g) lo = mid;
            else hi = mid - 1;
        }
        exact_window<PixT>(q.items[lo], (int64_t)(g - q.first_win[lo]), W, mode, sy0, sy1, sx0, sx1,
                           sm, sm + W * W, row_count, &total_cand);
    }
}

template <typename PixT>
cudaError_t launch_t(const PivParams& p, int w, int mode, int limit, bool use_list, int blocks,
                     cudaStream_t s)
{
    const size_t smem = 2 * sizeof(double2) * (size_t)w * w;
    // the opt-in limit for the largest window, once per device
    static std::atomic<uint64_t> attr_done{ 0 };
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(attr_done.load() & bit)) {
        const cudaError_t e = cudaFuncSetAttribute(piv_exact_kernel<PixT>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)(2 * sizeof(double2) * 64 * 64));
        if (e != cudaSuccess) return e;
        attr_done.fetch_or(bit);
    }
    piv_exact_kernel<PixT><<<blocks, kThreads, smem, s>>>(p, w, mode, limit, use_list);
    return cudaGetLastError();
}

// Threads per CTA of the queue's exact kernel: the kernel needs at least W
// threads (one per plane row in the peak scan).  16 px windows (8 KB of
// shared memory) run one warp each, so that about 28 share an SM instead of
// 8; larger windows are held to a few per SM by shared memory anyway.
inline int exact_queue_threads(int w) { return w <= 16 ? 32 : kThreads; }

template <typename PixT>
cudaError_t queue_t(const PivQueue& q, int w, int mode, int limit, int blocks, cudaStream_t s)
{
    const size_t smem = 2 * sizeof(double2) * (size_t)w * w;
    static std::atomic<uint64_t> attr_done{ 0 };
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(attr_done.load() & bit)) {
        const cudaError_t e = cudaFuncSetAttribute(piv_exact_queue_kernel<PixT>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)(2 * sizeof(double2) * 64 * 64));
        if (e != cudaSuccess) return e;
        attr_done.fetch_or(bit);
    }
    if (blocks <= 0) return cudaSuccess;
    piv_exact_queue_kernel<PixT><<<blocks, exact_queue_threads(w), smem, s>>>(q, w, mode, limit);
    return cudaGetLastError();
}

// ---- the per-window spectral API: FFT::transform, transform_real and
// auto_correlate (fft.h:87-186, :229-242) on a batch of windows, in the
// reference's double arithmetic (the same butterflies, twiddle tables,
// complex products and unpack as the correlation above).  One CTA per
// window (CTAs stride over the batch); X is one W x W double2 tile of
// shared memory.
template <int OP>
__global__ void __launch_bounds__(kThreads)
spectral_exact_kernel(const SpectralParams q)
{
    extern __shared__ double2 X[];
    const int W = q.w, N = W * W, t = threadIdx.x;
    for (int64_t w = blockIdx.x; w < q.n; w += gridDim.x) {
        const size_t o = (size_t)w * N;
        // transform: the input converted to complex (image::operator=,
        // image.h:136-145); transform_real: join_from_channels(a, b)
        // (image_utils.impl.h:288-315); auto_correlate: transform(a)
        for (int i = t; i < N; i += blockDim.x)
            X[i] = OP == kSpectralReal ? make_double2(q.in_ra[o + i], q.in_rb[o + i]) : q.in_c[o + i];
        __syncthreads();
        fft2d(X, W, q.tw);
        if (OP == kSpectralTransform) {
            for (int i = t; i < N; i += blockDim.x) q.out_a[o + i] = X[i];
        } else if (OP == kSpectralReal) {
            // the partial unpack of fft.h:163-183 into two zeroed spectra:
            // rows [1, H/2) x columns [1, W) and their mirrors
            for (int i = t; i < N; i += blockDim.x) {
                q.out_a[o + i] = make_double2(0.0, 0.0);
                q.out_b[o + i] = make_double2(0.0, 0.0);
            }
            __syncthreads();
            const int npairs = (W / 2 - 1) * (W - 1);
            for (int k = t; k < npairs; k += blockDim.x) {
                const int h = 1 + k / (W - 1), x = 1 + k % (W - 1);
                const int i = h * W + x, m = (W - h) * W + (W - x);
                const double2 t1 = X[i], t2 = X[m];
                const double2 half = make_double2(0.5, 0.0);
                const double2 av = e_mul(half, e_add(t1, e_conj(t2)));
                double2 bv = e_mul(half, e_sub(t1, e_conj(t2)));
                bv = make_double2(bv.y, __dmul_rn(-1.0, bv.x));
                q.out_a[o + i] = av;
                q.out_a[o + m] = e_conj(av);
                q.out_b[o + i] = bv;
                q.out_b[o + m] = e_conj(bv);
            }
        } else {
            // |A|^2 = (A * conj A).real (pixel_types.h:198), as a complex
            // image with zero imaginary parts; the unnormalised inverse;
            // its real part, quadrant-swapped (image_utils.impl.h:367-386)
            for (int i = t; i < N; i += blockDim.x) X[i] = make_double2(e_mul(X[i], e_conj(X[i])).x, 0.0);
            __syncthreads();
            fft2d(X, W, q.tw + W);
            for (int i = t; i < N; i += blockDim.x) {
                const int y = i / W, x = i % W;
                const int sy = (y + W / 2) % W, sx = (x + W / 2) % W;
                q.out_a[o + i] = make_double2(X[sy * W + sx].x, 0.0);
            }
        }
        __syncthreads();
    }
}

template <int OP>
cudaError_t spectral_t(const SpectralParams& q, int blocks, cudaStream_t s)
{
    const size_t smem = sizeof(double2) * (size_t)q.w * q.w;
    static std::atomic<uint64_t> attr_done{ 0 };
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(attr_done.load() & bit)) {
        const cudaError_t e = cudaFuncSetAttribute(spectral_exact_kernel<OP>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)(sizeof(double2) * kMaxW * kMaxW));
        if (e != cudaSuccess) return e;
        attr_done.fetch_or(bit);
    }
    spectral_exact_kernel<OP><<<blocks, kThreads, smem, s>>>(q);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_spectral_exact(const SpectralParams& q, int op, int blocks, cudaStream_t s)
{
    if (!exact_supports(q.w) || blocks <= 0 || q.n <= 0) return cudaErrorInvalidValue;
    switch (op) {
    case kSpectralTransform: return spectral_t<kSpectralTransform>(q, blocks, s);
    case kSpectralReal: return spectral_t<kSpectralReal>(q, blocks, s);
    case kSpectralAuto: return spectral_t<kSpectralAuto>(q, blocks, s);
    default: return cudaErrorInvalidValue;
    }
}

int exact_queue_max_ctas_per_sm(int w)
{
    int n = 0;
    const size_t smem = 2 * sizeof(double2) * (size_t)w * w;
    if (queue_t<uint16_t>(PivQueue{}, w, 0, 0, 0, nullptr) != cudaSuccess) return 1;   // attribute set-up only
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, piv_exact_queue_kernel<uint16_t>,
                                                      exact_queue_threads(w), smem) !=
        cudaSuccess)
        return 1;
    return n < 1 ? 1 : n;
}

cudaError_t launch_piv_exact_queue(const PivQueue& q, int w, int dtype, int mode, int limit, int blocks,
                                   cudaStream_t s)
{
    if (!exact_supports(w) || blocks <= 0) return cudaErrorInvalidValue;
    switch (dtype) {
    case kU8: return queue_t<uint8_t>(q, w, mode, limit, blocks, s);
    case kU16: return queue_t<uint16_t>(q, w, mode, limit, blocks, s);
    case kF32: return queue_t<float>(q, w, mode, limit, blocks, s);
    default: return cudaErrorInvalidValue;
    }
}

bool exact_supports(int w) { return w >= 4 && w <= kMaxW && (w & (w - 1)) == 0; }

cudaError_t launch_piv_exact(const PivParams& p, int w, int dtype, int mode, int limit,
                             bool use_list, int blocks, cudaStream_t s)
{
    if (!exact_supports(w) || blocks <= 0) return cudaErrorInvalidValue;
    switch (dtype) {
    case kU8: return launch_t<uint8_t>(p, w, mode, limit, use_list, blocks, s);
    case kU16: return launch_t<uint16_t>(p, w, mode, limit, use_list, blocks, s);
    case kF32: return launch_t<float>(p, w, mode, limit, use_list, blocks, s);
    case kF64: return launch_t<double>(p, w, mode, limit, use_list, blocks, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace opiv
