// opiv_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of OpenPIV-c++'s double-precision PIV window path
// (grid -> extract -> FFT cross-correlate -> find_peaks -> 3-point Gaussian
// fit -> vector assembly).  It is the checker for the GPU path: only tests,
// the smoke check and the CPU-baseline leg of the benchmark may load it.
// Nothing in the product links or calls it.
//
// Every function names the reference lines it restates.  Arithmetic is kept
// operation-for-operation identical to the reference (same radix-2 DIT data
// flow, same twiddle table entries, same complex-multiply formula, same
// unpack expressions), so that built with -ffp-contract=off it reproduces the
// reference's double results bit for bit.  The pin is checked by
// tests/test_oracle.py against the reference compiled from its own sources
// (oracle/Makefile, target "ref") and against the reference tests' golden vectors.
//
// Build: see oracle/Makefile (parity build: -O2 -ffp-contract=off;
// timed build: -O3, default contraction, as a release build of the reference).

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct cplx { double re, im; };

// openpiv/core/pixel_types.h:147-163 (complex +, -, *), :196 (conj)
inline cplx c_add(cplx a, cplx b) { return { a.re + b.re, a.im + b.im }; }
inline cplx c_sub(cplx a, cplx b) { return { a.re - b.re, a.im - b.im }; }
inline cplx c_mul(cplx a, cplx b) { return { a.re * b.re - a.im * b.im, a.im * b.re + a.re * b.im }; }
inline cplx c_conj(cplx a) { return { a.re, -a.im }; }

enum { MODE_REAL = 0, MODE_COMPLEX = 1 };

enum {
    ORC_OK = 0,
    ORC_ERR_OFFSET_RANGE = -1,   // "offsets must be between 0.0 and 1.0"
    ORC_ERR_IMAGE_EMPTY = -2,    // "image size must be non-zero"
    ORC_ERR_IA_EMPTY = -3,       // "interrogation size must be non-zero"
    ORC_ERR_OFFSET_ZERO = -4,    // "offsets must be non-zero"
    ORC_ERR_IA_TOO_BIG = -5,     // "interrogation size is bigger than image"
    ORC_ERR_NOT_POW2 = -6,       // "dimensions must be power of 2"
    ORC_ERR_CAPACITY = -7,
    ORC_ERR_RECT_OUTSIDE = -8,   // "extract: rectangle to extract is too large"
    ORC_ERR_ARG = -9,
};

// openpiv/core/util.h:67-70
inline bool is_pow2(uint64_t v) { return v && (v == (v & (~v + 1))); }

// Twiddle table for one transform length n: entry i = exp(s*i*pi*i/n) with
// s = -1 forward, +1 reverse.  openpiv/algos/fft.h:274-294 (same expression,
// evaluated in the same order, with std::cos / std::sin).
std::vector<cplx> twiddle_table(size_t n, int dir)
{
    std::vector<cplx> t(n);
    const double s = dir < 0 ? -1.0 : 1.0;
    for (size_t i = 0; i < n; ++i) {
        const double theta = (s * M_PI * (double)(int)i) / (double)n;
        t[i] = { std::cos(theta), std::sin(theta) };
    }
    return t;
}

// Radix-2 decimation-in-time DFT of n points src[0], src[stride], ... into
// dst[0..n).  Same butterfly graph and twiddle entries as the recursive
// fft_inner of openpiv/algos/fft.h:245-263: at each level the even and odd
// half-transforms are combined as e + o*w, e - o*w with w = table[k * tws].
void dit(const cplx* src, size_t stride, cplx* dst, size_t n, const cplx* tw, size_t tws)
{
    if (n == 1) { dst[0] = src[0]; return; }
    const size_t h = n / 2;
    dit(src, 2 * stride, dst, h, tw, 2 * tws);
    dit(src + stride, 2 * stride, dst + h, h, tw, 2 * tws);
    for (size_t k = 0; k < h; ++k) {
        const cplx e = dst[k];
        const cplx o = c_mul(dst[k + h], tw[k * tws]);
        dst[k] = c_add(e, o);
        dst[k + h] = c_sub(e, o);
    }
}

// Per-size FFT context (the reference's FFT object: fft.h:76-84).
struct fft_ctx {
    uint32_t w = 0, h = 0;
    std::vector<cplx> fw_w, fw_h, rv_w, rv_h;   // twiddles per axis / direction
    std::vector<cplx> a, b, line_in, line_out;  // scratch
    fft_ctx(uint32_t w_, uint32_t h_) : w(w_), h(h_)
    {
        fw_w = twiddle_table(w, -1); rv_w = twiddle_table(w, +1);
        fw_h = twiddle_table(h, -1); rv_h = twiddle_table(h, +1);
        a.resize((size_t)w * h); b.resize((size_t)w * h);
        line_in.resize(std::max(w, h)); line_out.resize(std::max(w, h));
    }
};

// 2-D transform in place: every row, then every column (the reference does
// rows, transpose, rows, transpose back: fft.h:87-119).  Unnormalised.
void fft2d(fft_ctx& c, cplx* img, int dir)
{
    const cplx* tw_w = (dir < 0 ? c.fw_w : c.rv_w).data();
    const cplx* tw_h = (dir < 0 ? c.fw_h : c.rv_h).data();
    for (uint32_t y = 0; y < c.h; ++y) {
        std::memcpy(c.line_in.data(), img + (size_t)y * c.w, sizeof(cplx) * c.w);
        dit(c.line_in.data(), 1, img + (size_t)y * c.w, c.w, tw_w, 2);
    }
    for (uint32_t x = 0; x < c.w; ++x) {
        for (uint32_t y = 0; y < c.h; ++y) c.line_in[y] = img[(size_t)y * c.w + x];
        dit(c.line_in.data(), 1, c.line_out.data(), c.h, tw_h, 2);
        for (uint32_t y = 0; y < c.h; ++y) img[(size_t)y * c.w + x] = c.line_out[y];
    }
}

// openpiv/core/detail/image_utils.impl.h:367-386 (literal loop, in place).
template <typename T>
void swap_quadrants(T* im, uint32_t w, uint32_t h)
{
    for (uint32_t y = 0; y < h; ++y) {
        T* i = im + (size_t)y * w;
        T* o = im + (size_t)((y + h / 2) % h) * w;
        for (uint32_t x = 0; x < w / 2; ++x) std::swap(i[x], o[(x + w / 2) % w]);
    }
}

// Two-for-one forward transform with the reference's partial unpack:
// openpiv/algos/fft.h:130-186.  Only rows [1, h/2) x columns [1, w) and their
// mirrors are written; row 0, row h/2 and column 0 stay zero.
void transform_real(fft_ctx& c, const double* a, const double* b, cplx* out_a, cplx* out_b)
{
    const size_t n = (size_t)c.w * c.h;
    cplx* z = c.a.data();
    for (size_t i = 0; i < n; ++i) z[i] = { a[i], b[i] };   // join_from_channels
    fft2d(c, z, -1);
    for (size_t i = 0; i < n; ++i) { out_a[i] = { 0.0, 0.0 }; out_b[i] = { 0.0, 0.0 }; }
    const uint32_t W = c.w, H = c.h;
    for (uint32_t y = 1; y < H / 2; ++y) {
        for (uint32_t x = 1; x < W; ++x) {
            const cplx t1 = z[(size_t)y * W + x];
            const cplx t2 = z[(size_t)(H - y) * W + (W - x)];
            // 0.5*(t1 + conj t2), evaluated as complex(0.5, 0) * (...)
            const cplx s = c_add(t1, c_conj(t2));
            const cplx av = c_mul(cplx{ 0.5, 0.0 }, s);
            out_a[(size_t)y * W + x] = av;
            out_a[(size_t)(H - y) * W + (W - x)] = c_conj(av);
            const cplx d = c_sub(t1, c_conj(t2));
            cplx bv = c_mul(cplx{ 0.5, 0.0 }, d);
            bv = cplx{ bv.im, -1.0 * bv.re };
            out_b[(size_t)y * W + x] = bv;
            out_b[(size_t)(H - y) * W + (W - x)] = c_conj(bv);
        }
    }
}

// FFT::cross_correlate (fft.h:188-206, mode COMPLEX) and
// FFT::cross_correlate_real (fft.h:208-227, mode REAL).  plane: w*h doubles,
// quadrant-swapped, zero lag at (w/2, h/2).
void cross_correlate(fft_ctx& c, const double* a, const double* b, int mode, double* plane)
{
    const size_t n = (size_t)c.w * c.h;
    cplx* A = c.a.data();
    cplx* B = c.b.data();
    if (mode == MODE_COMPLEX) {
        for (size_t i = 0; i < n; ++i) A[i] = { a[i], 0.0 };
        fft2d(c, A, -1);
        for (size_t i = 0; i < n; ++i) B[i] = { b[i], 0.0 };
        fft2d(c, B, -1);
    } else {
        std::vector<cplx> ta(n), tb(n);
        transform_real(c, a, b, ta.data(), tb.data());
        std::copy(ta.begin(), ta.end(), A);
        std::copy(tb.begin(), tb.end(), B);
    }
    for (size_t i = 0; i < n; ++i) A[i] = c_mul(B[i], c_conj(A[i]));
    fft2d(c, A, +1);
    for (size_t i = 0; i < n; ++i) plane[i] = A[i].re;
    swap_quadrants(plane, c.w, c.h);
}

struct peak { double v; int32_t x, y; };

// find_peaks over the sub-rectangle (x0, y0, vw, vh) of a w-wide plane:
// openpiv/core/detail/image_utils.impl.h:42-74.  Scan rows [r, vh-2r),
// columns [r, vw-r); strict 4-neighbour test; std::sort descending by the
// centre value (same comparator, hence same order among ties); keep num.
// Returned x, y are plane coordinates of the centre pixel.
std::vector<peak> find_peaks(const double* plane, uint32_t w, uint32_t x0, uint32_t y0,
                             uint32_t vw, uint32_t vh, uint16_t num, uint32_t r)
{
    std::vector<peak> res;
    for (uint32_t hh = r; hh < vh - 2 * r; ++hh) {
        const double* above = plane + (size_t)(y0 + hh - 1) * w + x0;
        const double* line = plane + (size_t)(y0 + hh) * w + x0;
        const double* below = plane + (size_t)(y0 + hh + 1) * w + x0;
        for (uint32_t ww = r; ww < vw - r; ++ww) {
            if (line[ww - 1] < line[ww] && line[ww + 1] < line[ww] &&
                above[ww] < line[ww] && below[ww] < line[ww])
                res.push_back(peak{ line[ww], (int32_t)(x0 + ww), (int32_t)(y0 + hh) });
        }
    }
    std::sort(res.begin(), res.end(), [](const peak& p, const peak& q) { return p.v > q.v; });
    res.resize(std::min(res.size(), (size_t)num));
    return res;
}

// fit_simple_gaussian: openpiv/core/detail/image_utils.impl.h:77-101.
inline double gauss3(double l, double c, double r)
{
    double num = std::log(l) - std::log(r);
    double den = 2.0 * (std::log(l) + std::log(r) - 2.0 * std::log(c));
    if (den == 0.0) return 0.0;
    return num / den;
}

void fit_simple_gaussian(const double* plane, uint32_t w, int32_t px, int32_t py, double* out)
{
    const double* row = plane + (size_t)py * w;
    out[0] = (double)px + gauss3(row[px - 1], row[px], row[px + 1]);
    out[1] = (double)py + gauss3(plane[(size_t)(py - 1) * w + px], row[px],
                                 plane[(size_t)(py + 1) * w + px]);
}

// rect::dilate(double): openpiv/core/rect.cpp:109-126 applied to the plane
// rect {(0,0),(w,h)}.
void dilate_half(uint32_t w, uint32_t h, uint32_t* x0, uint32_t* y0, uint32_t* vw, uint32_t* vh)
{
    const int32_t W = (int32_t)w, H = (int32_t)h;
    const int32_t rw = (int32_t)std::lround(0.5 * W);
    const int32_t rh = (int32_t)std::lround(0.5 * H);
    *x0 = (uint32_t)((W - rw) / 2);
    *y0 = (uint32_t)((H - rh) / 2);
    *vw = (uint32_t)rw;
    *vh = (uint32_t)rh;
}

// One window of examples/process/main.cpp:189-237.  vec = {x, y, u, v, sn};
// pk = {px, py} of the first peak, or {-1, -1} when fewer than two peaks.
// Frame B's window is extracted at (bbx, bby) (equal to (bx, by) in a single
// pass; offset in a multi-pass chain); the vector refers to frame A's rect.
void process_window(fft_ctx& c, const double* img_a, const double* img_b, uint32_t img_w,
                    uint32_t img_h, int32_t bx, int32_t by, int32_t bbx, int32_t bby, int mode,
                    int limit_search, std::vector<double>& wa, std::vector<double>& wb,
                    std::vector<double>& plane, double* vec, int32_t* pk)
{
    const uint32_t W = c.w, H = c.h;
    for (uint32_t y = 0; y < H; ++y) {   // core::extract, image_utils.impl.h:392-419
        std::memcpy(&wa[(size_t)y * W], img_a + (size_t)(by + y) * img_w + bx, sizeof(double) * W);
        std::memcpy(&wb[(size_t)y * W], img_b + (size_t)(bby + y) * img_w + bbx, sizeof(double) * W);
    }
    cross_correlate(c, wa.data(), wb.data(), mode, plane.data());
    uint32_t x0 = 0, y0 = 0, vw = W, vh = H;
    if (limit_search) dilate_half(W, H, &x0, &y0, &vw, &vh);
    const std::vector<peak> pk2 = find_peaks(plane.data(), W, x0, y0, vw, vh, 2, 1);
    for (int i = 0; i < 5; ++i) vec[i] = 0.0;
    pk[0] = -1; pk[1] = -1;
    if (pk2.size() != 2) return;
    double loc[2];
    fit_simple_gaussian(plane.data(), W, pk2[0].x, pk2[0].y, loc);
    const int32_t mx = bx + (int32_t)(W / 2), my = by + (int32_t)(H / 2);
    vec[0] = (double)mx;
    vec[1] = (double)my;
    vec[2] = (double)mx - ((double)bx + loc[0]);
    vec[3] = (double)my - ((double)by + loc[1]);
    vec[1] = (double)img_h - vec[1];
    if (pk2[1].v > 0) vec[4] = pk2[0].v / pk2[1].v;
    pk[0] = pk2[0].x; pk[1] = pk2[0].y;
}

}  // namespace

extern "C" {

int orc_version() { return 1; }

// generate_cartesian_grid(size, size, array<uint32,2>):
// openpiv/core/detail/grid.impl.h:24-61.  Writes (x, y) of each window's
// bottom-left corner, y outer / x inner.  Returns the count or an error.
int64_t orc_grid_offsets(uint32_t img_w, uint32_t img_h, uint32_t ia_w, uint32_t ia_h,
                         uint32_t dx, uint32_t dy, int32_t* out_xy, int64_t cap)
{
    if ((uint64_t)img_w * img_h == 0) return ORC_ERR_IMAGE_EMPTY;
    if ((uint64_t)ia_w * ia_h == 0) return ORC_ERR_IA_EMPTY;
    if (dx == 0 || dy == 0) return ORC_ERR_OFFSET_ZERO;
    if (ia_w > img_w || ia_h > img_h) return ORC_ERR_IA_TOO_BIG;
    const uint32_t xc = 1 + (img_w - ia_w) / dx;
    const uint32_t yc = 1 + (img_h - ia_h) / dy;
    const uint32_t xs = (img_w - ia_w - (dx * (xc - 1))) / 2;
    const uint32_t ys = (img_h - ia_h - (dy * (yc - 1))) / 2;
    const int64_t n = (int64_t)xc * yc;
    if (out_xy == nullptr) return n;
    if (cap < n) return ORC_ERR_CAPACITY;
    int64_t k = 0;
    for (size_t y = 0; y < yc; ++y)
        for (size_t x = 0; x < xc; ++x) {
            out_xy[2 * k] = (int32_t)(xs + x * dx);
            out_xy[2 * k + 1] = (int32_t)(ys + y * dy);
            ++k;
        }
    return n;
}

// generate_cartesian_grid(size, size, double): grid.impl.h:9-22.
int64_t orc_grid(uint32_t img_w, uint32_t img_h, uint32_t ia_w, uint32_t ia_h, double frac,
                 int32_t* out_xy, int64_t cap)
{
    if (frac < 0.0 || frac > 1.0) return ORC_ERR_OFFSET_RANGE;
    return orc_grid_offsets(img_w, img_h, ia_w, ia_h, (uint32_t)(ia_w * frac),
                            (uint32_t)(ia_h * frac), out_xy, cap);
}

// 2-D FFT of an interleaved complex image (re, im pairs), in place.
// FFT::transform: fft.h:87-119.  dir: -1 forward, +1 reverse.
int orc_transform(double* data, uint32_t w, uint32_t h, int dir)
{
    if (!(is_pow2(w) && is_pow2(h))) return ORC_ERR_NOT_POW2;
    fft_ctx c(w, h);
    fft2d(c, reinterpret_cast<cplx*>(data), dir);
    return ORC_OK;
}

// FFT::transform_real: fft.h:130-186.  out_a, out_b interleaved complex.
int orc_transform_real(const double* a, const double* b, uint32_t w, uint32_t h, double* out_a,
                       double* out_b)
{
    if (!(is_pow2(w) && is_pow2(h))) return ORC_ERR_NOT_POW2;
    fft_ctx c(w, h);
    transform_real(c, a, b, reinterpret_cast<cplx*>(out_a), reinterpret_cast<cplx*>(out_b));
    return ORC_OK;
}

// One correlation plane (w*h doubles) of two w x h windows.
int orc_cross_correlate(const double* a, const double* b, uint32_t w, uint32_t h, int mode,
                        double* plane)
{
    if (!(is_pow2(w) && is_pow2(h))) return ORC_ERR_NOT_POW2;
    fft_ctx c(w, h);
    cross_correlate(c, a, b, mode, plane);
    return ORC_OK;
}

int orc_swap_quadrants(double* im, uint32_t w, uint32_t h)
{
    swap_quadrants(im, w, h);
    return ORC_OK;
}

// find_peaks on a whole w x h image: returns the number of peaks written
// (x, y, value per peak, in sorted order).
int orc_find_peaks(const double* im, uint32_t w, uint32_t h, uint16_t num, uint32_t radius,
                   int32_t* out_xy, double* out_v)
{
    const std::vector<peak> p = find_peaks(im, w, 0, 0, w, h, num, radius);
    for (size_t i = 0; i < p.size(); ++i) {
        out_xy[2 * i] = p[i].x; out_xy[2 * i + 1] = p[i].y; out_v[i] = p[i].v;
    }
    return (int)p.size();
}

// fit_simple_gaussian on the 3x3 neighbourhood of (px, py) of a w-wide plane.
int orc_fit_simple_gaussian(const double* plane, uint32_t w, int32_t px, int32_t py, double* out)
{
    fit_simple_gaussian(plane, w, px, py, out);
    return ORC_OK;
}

// Correlation planes of a list of windows of one image pair (row-major
// double images, img_w x img_h).  win_xy: bottom-left corners.  planes: n*w*w.
int orc_correlate_windows(const double* img_a, const double* img_b, uint32_t img_w,
                          uint32_t img_h, const int32_t* win_xy, int64_t n, uint32_t w, int mode,
                          double* planes)
{
    if (!is_pow2(w)) return ORC_ERR_NOT_POW2;
    fft_ctx c(w, w);
    std::vector<double> wa((size_t)w * w), wb((size_t)w * w);
    for (int64_t k = 0; k < n; ++k) {
        const int32_t bx = win_xy[2 * k], by = win_xy[2 * k + 1];
        if (bx < 0 || by < 0 || (uint32_t)bx + w > img_w || (uint32_t)by + w > img_h)
            return ORC_ERR_RECT_OUTSIDE;
        for (uint32_t y = 0; y < w; ++y) {
            std::memcpy(&wa[(size_t)y * w], img_a + (size_t)(by + y) * img_w + bx, sizeof(double) * w);
            std::memcpy(&wb[(size_t)y * w], img_b + (size_t)(by + y) * img_w + bx, sizeof(double) * w);
        }
        cross_correlate(c, wa.data(), wb.data(), mode, planes + (size_t)k * w * w);
    }
    return ORC_OK;
}

// The whole processing loop of examples/process/main.cpp:138-302 for a list
// of windows: out_vec n*5 doubles {x, y, u, v, sn}; out_peak n*2 int32
// (first-peak plane position or -1).  threads <= 1 runs one thread; more runs
// a pool of worker threads that take one window at a time (the reference's
// "pool" execution, main.cpp:265-276).  Returns the processing time in
// seconds (timing covers the loop only, as main.cpp:239/304 does), or a
// negative error code.
static double process_windows_impl(const double* img_a, const double* img_b, uint32_t img_w,
                                   uint32_t img_h, const int32_t* win_xy, const int32_t* win_b,
                                   int64_t n, uint32_t w, int mode, int limit_search, int threads,
                                   double* out_vec, int32_t* out_peak);

double orc_process_windows(const double* img_a, const double* img_b, uint32_t img_w,
                           uint32_t img_h, const int32_t* win_xy, int64_t n, uint32_t w, int mode,
                           int limit_search, int threads, double* out_vec, int32_t* out_peak)
{
    return process_windows_impl(img_a, img_b, img_w, img_h, win_xy, nullptr, n, w, mode,
                                limit_search, threads, out_vec, out_peak);
}

// Same with frame B's windows at their own corners win_b (multi-pass
// window offsetting, composed from the same reference steps).
double orc_process_windows_ab(const double* img_a, const double* img_b, uint32_t img_w,
                              uint32_t img_h, const int32_t* win_xy, const int32_t* win_b,
                              int64_t n, uint32_t w, int mode, int limit_search, int threads,
                              double* out_vec, int32_t* out_peak)
{
    return process_windows_impl(img_a, img_b, img_w, img_h, win_xy, win_b, n, w, mode,
                                limit_search, threads, out_vec, out_peak);
}

static double process_windows_impl(const double* img_a, const double* img_b, uint32_t img_w,
                                   uint32_t img_h, const int32_t* win_xy, const int32_t* win_b,
                                   int64_t n, uint32_t w, int mode, int limit_search, int threads,
                                   double* out_vec, int32_t* out_peak)
{
    if (!is_pow2(w)) return ORC_ERR_NOT_POW2;
    for (int64_t k = 0; k < n; ++k) {
        for (const int32_t* xy : { win_xy, win_b }) {
            if (!xy) continue;
            const int32_t bx = xy[2 * k], by = xy[2 * k + 1];
            if (bx < 0 || by < 0 || (uint32_t)bx + w > img_w || (uint32_t)by + w > img_h)
                return ORC_ERR_RECT_OUTSIDE;
        }
    }
    std::atomic<int64_t> next{ 0 };
    auto worker = [&]() {
        fft_ctx c(w, w);
        std::vector<double> wa((size_t)w * w), wb((size_t)w * w), plane((size_t)w * w);
        for (;;) {
            const int64_t k = next.fetch_add(1, std::memory_order_relaxed);
            if (k >= n) break;
            const int32_t* bxy = win_b ? win_b : win_xy;
            process_window(c, img_a, img_b, img_w, img_h, win_xy[2 * k], win_xy[2 * k + 1],
                           bxy[2 * k], bxy[2 * k + 1], mode, limit_search, wa, wb, plane,
                           out_vec + 5 * k, out_peak + 2 * k);
        }
    };
    const auto t1 = std::chrono::steady_clock::now();
    if (threads <= 1) {
        worker();
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
        for (auto& t : pool) t.join();
    }
    const auto t2 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t2 - t1).count();
}

}  // extern "C"
