// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Exposes the reference OpenPIV-c++ implementation, compiled from its own
// sources (headers under openpiv/, plus core/{size,rect,util}.cpp and the
// example's ThreadPool), through the same extern "C" surface as
// opiv_oracle.cpp, so the restatement can be checked against the real thing.
// Built by oracle/Makefile (target "ref") into oracle/_ref/; never part of
// the product.

#include <chrono>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "algos/fft.h"
#include "core/grid.h"
#include "core/image.h"
#include "core/image_utils.h"
#include "core/image_view.h"
#include "threadpool.hpp"

using namespace openpiv;

namespace {

int map_error(const std::exception& e)
{
    const std::string m = e.what();
    if (m.find("between 0.0 and 1.0") != std::string::npos) return -1;
    if (m.find("image size must be non-zero") != std::string::npos) return -2;
    if (m.find("interrogation size must be non-zero") != std::string::npos) return -3;
    if (m.find("offsets must be non-zero") != std::string::npos) return -4;
    if (m.find("bigger than image") != std::string::npos) return -5;
    if (m.find("power of 2") != std::string::npos) return -6;
    if (m.find("too large for image") != std::string::npos) return -8;
    return -9;
}

int64_t emit_grid(const std::vector<core::rect>& g, int32_t* out_xy, int64_t cap)
{
    const int64_t n = (int64_t)g.size();
    if (out_xy == nullptr) return n;
    if (cap < n) return -7;
    for (int64_t k = 0; k < n; ++k) {
        out_xy[2 * k] = g[k].bottomLeft()[0];
        out_xy[2 * k + 1] = g[k].bottomLeft()[1];
    }
    return n;
}

core::gf_image from_buffer(const double* p, uint32_t w, uint32_t h)
{
    core::gf_image im(w, h);
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) im[{ x, y }] = p[(size_t)y * w + x];
    return im;
}

void to_buffer(const core::gf_image& im, double* p)
{
    for (uint32_t y = 0; y < im.height(); ++y)
        for (uint32_t x = 0; x < im.width(); ++x) p[(size_t)y * im.width() + x] = im[{ x, y }];
}

void to_buffer(const core::cf_image& im, double* p)
{
    for (uint32_t y = 0; y < im.height(); ++y)
        for (uint32_t x = 0; x < im.width(); ++x) {
            const auto v = im[{ x, y }];
            p[2 * ((size_t)y * im.width() + x)] = v.real;
            p[2 * ((size_t)y * im.width() + x) + 1] = v.imag;
        }
}

}  // namespace

extern "C" {

int orc_version() { return 1001; }

int64_t orc_grid_offsets(uint32_t img_w, uint32_t img_h, uint32_t ia_w, uint32_t ia_h,
                         uint32_t dx, uint32_t dy, int32_t* out_xy, int64_t cap)
{
    try {
        return emit_grid(core::generate_cartesian_grid({ img_w, img_h }, { ia_w, ia_h },
                                                       std::array<uint32_t, 2>{ dx, dy }),
                         out_xy, cap);
    } catch (const std::exception& e) { return map_error(e); }
}

int64_t orc_grid(uint32_t img_w, uint32_t img_h, uint32_t ia_w, uint32_t ia_h, double frac,
                 int32_t* out_xy, int64_t cap)
{
    try {
        return emit_grid(core::generate_cartesian_grid({ img_w, img_h }, { ia_w, ia_h }, frac),
                         out_xy, cap);
    } catch (const std::exception& e) { return map_error(e); }
}

int orc_transform(double* data, uint32_t w, uint32_t h, int dir)
{
    try {
        algos::FFT fft({ w, h });
        core::cf_image im(w, h);
        for (uint32_t y = 0; y < h; ++y)
            for (uint32_t x = 0; x < w; ++x)
                im[{ x, y }] = core::c_f{ data[2 * ((size_t)y * w + x)], data[2 * ((size_t)y * w + x) + 1] };
        core::cf_image out{ fft.transform(im, dir < 0 ? algos::direction::FORWARD
                                                      : algos::direction::REVERSE) };
        to_buffer(out, data);
        return 0;
    } catch (const std::exception& e) { return map_error(e); }
}

int orc_transform_real(const double* a, const double* b, uint32_t w, uint32_t h, double* out_a,
                       double* out_b)
{
    try {
        algos::FFT fft({ w, h });
        auto [A, B] = fft.transform_real(from_buffer(a, w, h), from_buffer(b, w, h));
        to_buffer(A, out_a);
        to_buffer(B, out_b);
        return 0;
    } catch (const std::exception& e) { return map_error(e); }
}

int orc_cross_correlate(const double* a, const double* b, uint32_t w, uint32_t h, int mode,
                        double* plane)
{
    try {
        algos::FFT fft({ w, h });
        const auto ia = from_buffer(a, w, h), ib = from_buffer(b, w, h);
        const core::gf_image out{ mode == 1 ? fft.cross_correlate(ia, ib)
                                            : fft.cross_correlate_real(ia, ib) };
        to_buffer(out, plane);
        return 0;
    } catch (const std::exception& e) { return map_error(e); }
}

int orc_swap_quadrants(double* im, uint32_t w, uint32_t h)
{
    auto img = from_buffer(im, w, h);
    core::swap_quadrants(img);
    to_buffer(img, im);
    return 0;
}

int orc_find_peaks(const double* im, uint32_t w, uint32_t h, uint16_t num, uint32_t radius,
                   int32_t* out_xy, double* out_v)
{
    const auto img = from_buffer(im, w, h);
    const auto peaks = core::find_peaks(img, num, radius);
    for (size_t i = 0; i < peaks.size(); ++i) {
        const auto m = peaks[i].rect().midpoint();
        out_xy[2 * i] = m[0];
        out_xy[2 * i + 1] = m[1];
        out_v[i] = peaks[i][{ radius, radius }];
    }
    return (int)peaks.size();
}

int orc_fit_simple_gaussian(const double* plane, uint32_t w, int32_t px, int32_t py, double* out)
{
    const auto img = from_buffer(plane, w, w);
    const auto view = core::create_image_view(img, core::rect{ { px - 1, py - 1 }, { 3, 3 } });
    const auto p = core::fit_simple_gaussian(view);
    out[0] = p[0];
    out[1] = p[1];
    return 0;
}

int orc_correlate_windows(const double* img_a, const double* img_b, uint32_t img_w,
                          uint32_t img_h, const int32_t* win_xy, int64_t n, uint32_t w, int mode,
                          double* planes)
{
    try {
        const auto A = from_buffer(img_a, img_w, img_h), B = from_buffer(img_b, img_w, img_h);
        algos::FFT fft({ w, w });
        for (int64_t k = 0; k < n; ++k) {
            const core::rect ia{ { win_xy[2 * k], win_xy[2 * k + 1] }, { w, w } };
            const auto va{ core::extract(A, ia) };
            const auto vb{ core::extract(B, ia) };
            const core::gf_image out{ mode == 1 ? fft.cross_correlate(va, vb)
                                                : fft.cross_correlate_real(va, vb) };
            to_buffer(out, planes + (size_t)k * w * w);
        }
        return 0;
    } catch (const std::exception& e) { return map_error(e); }
}

// The processing loop of examples/process/main.cpp, driven through the
// reference API in the same order as its processor lambda, executed by the
// example's own ThreadPool in "pool" mode (one task per window) when
// threads > 1.  Returns the loop time in seconds.
static double process_ab(const double* img_a, const double* img_b, uint32_t img_w, uint32_t img_h,
                         const int32_t* win_xy, const int32_t* win_b, int64_t n, uint32_t w,
                         int mode, int limit_search, int threads, double* out_vec,
                         int32_t* out_peak);

double orc_process_windows(const double* img_a, const double* img_b, uint32_t img_w,
                           uint32_t img_h, const int32_t* win_xy, int64_t n, uint32_t w, int mode,
                           int limit_search, int threads, double* out_vec, int32_t* out_peak)
{
    return process_ab(img_a, img_b, img_w, img_h, win_xy, nullptr, n, w, mode, limit_search,
                      threads, out_vec, out_peak);
}

// Frame B's window extracted at its own rect (window offsetting composed
// from the same reference calls: extract, correlator, find_peaks, fit).
double orc_process_windows_ab(const double* img_a, const double* img_b, uint32_t img_w,
                              uint32_t img_h, const int32_t* win_xy, const int32_t* win_b,
                              int64_t n, uint32_t w, int mode, int limit_search, int threads,
                              double* out_vec, int32_t* out_peak)
{
    return process_ab(img_a, img_b, img_w, img_h, win_xy, win_b, n, w, mode, limit_search,
                      threads, out_vec, out_peak);
}

static double process_ab(const double* img_a, const double* img_b, uint32_t img_w, uint32_t img_h,
                         const int32_t* win_xy, const int32_t* win_b, int64_t n, uint32_t w,
                         int mode, int limit_search, int threads, double* out_vec,
                         int32_t* out_peak)
{
    std::vector<core::gf_image> images;
    images.push_back(from_buffer(img_a, img_w, img_h));
    images.push_back(from_buffer(img_b, img_w, img_h));
    const core::size ia_size{ w, w };
    std::vector<core::rect> grid;
    for (int64_t k = 0; k < n; ++k) grid.push_back(core::rect{ { win_xy[2 * k], win_xy[2 * k + 1] }, ia_size });

    // main.cpp:153-178 keeps one function-local static FFT per correlator;
    // here one FFT per call is shared by all workers in the same way (the
    // class is thread-safe through its thread-local scratch, fft.h:45-73).
    const algos::FFT fft{ ia_size };
    using correlator_t = std::function<core::gf_image(const core::gf_image&, const core::gf_image&)>;
    correlator_t correlator;
    if (mode == 1)
        correlator = [&fft](const core::gf_image& a, const core::gf_image& b) -> core::gf_image {
            return fft.cross_correlate(a, b);
        };
    else
        correlator = [&fft](const core::gf_image& a, const core::gf_image& b) -> core::gf_image {
            return fft.cross_correlate_real(a, b);
        };

    auto processor = [&](size_t i, const core::rect& ia) {
        double* vec = out_vec + 5 * i;
        int32_t* pk = out_peak + 2 * i;
        for (int j = 0; j < 5; ++j) vec[j] = 0.0;
        pk[0] = -1; pk[1] = -1;
        const core::rect ib = win_b ? core::rect{ { win_b[2 * i], win_b[2 * i + 1] }, ia.size() } : ia;
        const auto view_a{ core::extract(images[0], ia) };
        const auto view_b{ core::extract(images[1], ib) };
        const core::gf_image output{ correlator(view_a, view_b) };
        core::peaks_t<core::g_f> peaks;
        if (limit_search) {
            auto centre = core::create_image_view(output, output.rect().dilate(0.5));
            peaks = core::find_peaks(centre, 2, 1);
        } else {
            peaks = core::find_peaks(output, 2, 1);
        }
        if (peaks.size() != 2) return;
        const auto bl = ia.bottomLeft();
        const auto midpoint = ia.midpoint();
        const auto loc = core::fit_simple_gaussian(peaks[0]);
        vec[0] = midpoint[0];
        vec[1] = midpoint[1];
        vec[2] = midpoint[0] - (bl[0] + loc[0]);
        vec[3] = midpoint[1] - (bl[1] + loc[1]);
        vec[1] = images[0].height() - vec[1];
        if (peaks[1][{ 1, 1 }] > 0) vec[4] = peaks[0][{ 1, 1 }] / peaks[1][{ 1, 1 }];
        const auto m = peaks[0].rect().midpoint();
        pk[0] = m[0]; pk[1] = m[1];
    };

    const auto t1 = std::chrono::steady_clock::now();
    if (threads <= 1) {
        for (int64_t k = 0; k < n; ++k) processor((size_t)k, grid[k]);
    } else {
        ThreadPool pool((size_t)threads);
        size_t i = 0;
        for (const auto& ia : grid) {
            pool.enqueue([i, ia, &processor]() { processor(i, ia); });
            ++i;
        }
    }
    const auto t2 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t2 - t1).count();
}

}  // extern "C"
