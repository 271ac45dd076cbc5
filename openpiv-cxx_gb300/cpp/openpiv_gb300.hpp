// openpiv_gb300.hpp -- C++17 facade over the C ABI (include/openpiv_gb300.h)
// with the names of the reference's openpiv::core / openpiv::algos interface
// for the window-correlation path, so code written against the reference
// ports by changing the namespace:
//
//   reference (openpiv/...)                         here (openpiv::gb300)
//   core::generate_cartesian_grid (grid.h:88-107)   generate_cartesian_grid
//   algos::FFT(size) (fft.h:76-84)                  FFT(size)
//   FFT::cross_correlate[_real] (fft.h:188-227)     FFT::cross_correlate[_real]
//   core::find_peaks (image_utils.impl.h:42-74)     find_peaks (peaks by value)
//   core::fit_simple_gaussian (impl:77-101)         fit_simple_gaussian
//   the loop of examples/process/main.cpp:189-302   piv_pass::process
//   (no counterpart: multi-pass batches)           piv_batch
//
// Failures throw std::runtime_error whose message starts like the
// reference's exception text (e.g. "dimensions must be power of 2").
// Images are plain row-major containers; peaks are returned by value
// (centre position and value) instead of views into the plane.
#pragma once

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "openpiv_gb300.h"

namespace openpiv::gb300 {

inline void check(int status)
{
    if (status < 0) throw std::runtime_error(opiv_last_error());
}

struct size {
    uint32_t w = 0, h = 0;
    uint32_t width() const { return w; }
    uint32_t height() const { return h; }
    bool operator==(const size& o) const { return w == o.w && h == o.h; }
    bool operator!=(const size& o) const { return !(*this == o); }
};

struct point2i {
    int32_t x = 0, y = 0;
};
struct point2d {
    double x = 0, y = 0;
};

// core::rect: bottom-left corner + size; midpoint = bl + size / 2 (rect.cpp:63-66)
struct rect {
    point2i bl;
    gb300::size sz;
    point2i bottomLeft() const { return bl; }
    gb300::size size() const { return sz; }
    point2i midpoint() const
    {
        return { bl.x + (int32_t)(sz.w / 2), bl.y + (int32_t)(sz.h / 2) };
    }
};

template <typename T>
class image {
public:
    image() = default;
    image(uint32_t w, uint32_t h, T fill = T{}) : size_{ w, h }, data_((size_t)w * h, fill) {}
    uint32_t width() const { return size_.w; }
    uint32_t height() const { return size_.h; }
    gb300::size size() const { return size_; }
    T* line(uint32_t y) { return data_.data() + (size_t)y * size_.w; }
    const T* line(uint32_t y) const { return data_.data() + (size_t)y * size_.w; }
    T& operator()(uint32_t x, uint32_t y) { return data_[(size_t)y * size_.w + x]; }
    const T& operator()(uint32_t x, uint32_t y) const { return data_[(size_t)y * size_.w + x]; }
    T* data() { return data_.data(); }
    const T* data() const { return data_.data(); }

private:
    gb300::size size_;
    std::vector<T> data_;
};

using g8_image = image<uint8_t>;
using g16_image = image<uint16_t>;
using gf_image = image<double>;

// ---- grid ------------------------------------------------------------------
inline std::vector<rect> to_rects(const std::vector<int32_t>& xy, const size& ia)
{
    std::vector<rect> out(xy.size() / 2);
    for (size_t k = 0; k < out.size(); ++k) out[k] = rect{ { xy[2 * k], xy[2 * k + 1] }, ia };
    return out;
}

inline std::vector<rect> generate_cartesian_grid(const size& image_size, const size& ia,
                                                 double step_fraction)
{
    const int64_t n = opiv_grid(image_size.w, image_size.h, ia.w, ia.h, step_fraction, nullptr, 0);
    check((int)(n < 0 ? n : 0));
    std::vector<int32_t> xy(2 * n);
    check((int)opiv_grid(image_size.w, image_size.h, ia.w, ia.h, step_fraction, xy.data(), n));
    return to_rects(xy, ia);
}

inline std::vector<rect> generate_cartesian_grid(const size& image_size, const size& ia,
                                                 std::array<uint32_t, 2> offsets)
{
    const int64_t n = opiv_grid_offsets(image_size.w, image_size.h, ia.w, ia.h, offsets[0],
                                        offsets[1], nullptr, 0);
    check((int)(n < 0 ? n : 0));
    std::vector<int32_t> xy(2 * n);
    check((int)opiv_grid_offsets(image_size.w, image_size.h, ia.w, ia.h, offsets[0], offsets[1],
                                 xy.data(), n));
    return to_rects(xy, ia);
}

// ---- per-window correlation -------------------------------------------------
// FFT of one window size; cross_correlate* run on the GPU (one window or a
// batch per call).  exact = true repeats the reference's double arithmetic
// bit for bit; exact = false uses the FP32 kernels (plane within 1e-5 of its
// peak).
class FFT {
public:
    explicit FFT(const size& s, bool exact = false, int device = 0)
        : size_(s), exact_(exact), device_(device)
    {
        auto pow2 = [](uint32_t v) { return v && (v & (v - 1)) == 0; };
        if (!(pow2(s.w) && pow2(s.h)))
            throw std::runtime_error("dimensions must be power of 2: [" + std::to_string(s.w) + ", " +
                                     std::to_string(s.h) + "]");
    }

    gf_image cross_correlate(const gf_image& a, const gf_image& b) const
    {
        return correlate(a, b, OPIV_CORR_COMPLEX);
    }
    gf_image cross_correlate_real(const gf_image& a, const gf_image& b) const
    {
        return correlate(a, b, OPIV_CORR_REAL);
    }

    // n windows stacked row-wise (n*h rows of w) -> n planes, same layout
    std::vector<double> cross_correlate_batch(const std::vector<double>& a,
                                              const std::vector<double>& b, int mode) const
    {
        const size_t per = (size_t)size_.w * size_.h;
        if (a.size() != b.size() || a.size() % per != 0)
            throw std::runtime_error("image size is different from expected");
        std::vector<double> out(a.size());
        check(opiv_cross_correlate_batch(a.data(), b.data(), size_.w, (int64_t)(a.size() / per), mode,
                                         exact_ ? 1 : 0, out.data(), device_));
        return out;
    }

private:
    gf_image correlate(const gf_image& a, const gf_image& b, int mode) const
    {
        if (a.size() != size_ || b.size() != size_)
            throw std::runtime_error("image size is different from expected: [" +
                                     std::to_string(a.width()) + ", " + std::to_string(a.height()) +
                                     "], [" + std::to_string(size_.w) + ", " +
                                     std::to_string(size_.h) + "]");
        if (size_.w != size_.h) throw std::runtime_error("no kernel for non-square windows");
        gf_image out(size_.w, size_.h);
        check(opiv_cross_correlate_batch(a.data(), b.data(), size_.w, 1, mode, exact_ ? 1 : 0,
                                         out.data(), device_));
        return out;
    }

    size size_;
    bool exact_;
    int device_;
};

// ---- peaks and the Gaussian fit (host) -----------------------------------
struct peak {
    point2i centre;   // plane coordinates of the centre pixel
    double value = 0;
};

inline std::vector<peak> find_peaks(const gf_image& im, uint16_t num_peaks, uint32_t radius)
{
    std::vector<int32_t> xy(2 * (size_t)num_peaks + 2);
    std::vector<double> v((size_t)num_peaks + 1);
    const int n = opiv_find_peaks(im.data(), im.width(), im.height(), num_peaks, radius, xy.data(),
                                  v.data());
    check(n);
    std::vector<peak> out(n);
    for (int k = 0; k < n; ++k) out[k] = peak{ { xy[2 * k], xy[2 * k + 1] }, v[k] };
    return out;
}

inline point2d fit_simple_gaussian(const gf_image& plane, const peak& p)
{
    double xy[2];
    check(opiv_fit_simple_gaussian(plane.data(), plane.width(), plane.height(), p.centre.x,
                                   p.centre.y, xy));
    return { xy[0], xy[1] };
}

// ---- the whole pass -------------------------------------------------------
// One plan: image size, pixel type, window size, step, mode.  process()
// replaces the grid loop of examples/process/main.cpp with one GPU pass.
class piv_pass {
public:
    piv_pass(const size& image_size, int dtype, uint32_t ia, uint32_t step, int mode,
             bool limit_search = false, int device = 0)
    {
        check(opiv_plan_create(&plan_, image_size.w, image_size.h, dtype, ia, step, step, mode,
                               limit_search ? 1 : 0, device));
    }
    piv_pass(const piv_pass&) = delete;
    piv_pass& operator=(const piv_pass&) = delete;
    ~piv_pass() { opiv_plan_destroy(plan_); }

    int64_t window_count() const { return opiv_plan_window_count(plan_); }

    std::vector<rect> grid(const size& ia) const
    {
        std::vector<int32_t> xy(2 * (size_t)window_count());
        check(opiv_plan_grid(plan_, xy.data(), window_count()));
        return to_rects(xy, ia);
    }

    template <typename T>
    std::vector<opiv_vector> process(const image<T>& a, const image<T>& b) const
    {
        std::vector<opiv_vector> out((size_t)window_count());
        check(opiv_process_pair(plan_, a.data(), b.data(), sizeof(T) * a.width(), out.data(), nullptr));
        return out;
    }

    // OPIV_PREC_FP32 (reference-exact peaks), the tensor-core precisions
    // (32 x 32 windows) or OPIV_PREC_FP64 (every window exact)
    void set_precision(int precision) { check(opiv_plan_set_precision(plan_, precision)); }
    // tile shape of the 32 px tensor-core kernel (OPIV_TILE_*), forced or
    // timed on device frames by the autotuner; returns the shape in use
    void set_tile(int tile) { check(opiv_plan_set_tile(plan_, tile)); }
    int autotune(const void* d_frame_a, const void* d_frame_b, size_t pitch_bytes, void* stream = nullptr)
    {
        check(opiv_plan_autotune(plan_, d_frame_a, d_frame_b, pitch_bytes, stream));
        return check_value(opiv_plan_get_tile(plan_));
    }

private:
    static int check_value(int v)
    {
        check(v);
        return v;
    }
    opiv_plan* plan_ = nullptr;
};

// ---- batches ------------------------------------------------------------------
// Many image pairs (sizes may differ) through one multi-pass schedule: pass
// k >= 1 offsets each frame-B window by the previous pass's integer
// displacement.  No counterpart in the reference (multi-pass is a TODO
// there); see opiv_batch_* in the C ABI.  Schedules: OPIV_BATCH_STREAMS
// (per-pair pass chains on fork streams) or OPIV_BATCH_QUEUE (per pass one
// launch over a device work list of all pairs' windows); autotune() picks
// the queue's launch shapes and lanes by timing them on the frames held.
class piv_batch {
public:
    struct pass {
        uint32_t ia = 0, step = 0;
    };
    piv_batch(const std::vector<size>& sizes, int dtype, const std::vector<pass>& passes, int mode,
              bool limit_search = false, int device = 0)
        : n_pairs_((int)sizes.size()), n_passes_((int)passes.size())
    {
        std::vector<uint32_t> w, h, ia, st;
        for (const size& s : sizes) {
            w.push_back(s.w);
            h.push_back(s.h);
        }
        for (const pass& p : passes) {
            ia.push_back(p.ia);
            st.push_back(p.step);
        }
        check(opiv_batch_create(&batch_, n_pairs_, w.data(), h.data(), dtype, n_passes_, ia.data(),
                                st.data(), mode, limit_search ? 1 : 0, device));
    }
    piv_batch(const piv_batch&) = delete;
    piv_batch& operator=(const piv_batch&) = delete;
    ~piv_batch() { opiv_batch_destroy(batch_); }

    int pairs() const { return n_pairs_; }
    int passes() const { return n_passes_; }
    int64_t window_count(int pair, int pass_index) const
    {
        const int64_t n = opiv_batch_window_count(batch_, pair, pass_index);
        check((int)(n < 0 ? n : 0));
        return n;
    }

    template <typename T>
    void upload(int pair, const image<T>& a, const image<T>& b, void* stream = nullptr)
    {
        check(opiv_batch_upload(batch_, pair, a.data(), b.data(), sizeof(T) * a.width(), stream));
    }
    void run(bool use_graph = true, void* stream = nullptr) { check(opiv_batch_run(batch_, use_graph ? 1 : 0, stream)); }
    void set_schedule(int schedule) { check(opiv_batch_set_schedule(batch_, schedule)); }
    void set_lanes(int lanes) { check(opiv_batch_set_lanes(batch_, lanes)); }
    void autotune(void* stream = nullptr) { check(opiv_batch_autotune(batch_, stream)); }

    // vectors of pair `pair`, pass `pass_index` (synchronises the device)
    std::vector<opiv_vector> results(int pair, int pass_index) const
    {
        std::vector<opiv_vector> out((size_t)window_count(pair, pass_index));
        check(opiv_batch_results(batch_, pair, pass_index, out.data(), nullptr, nullptr));
        return out;
    }

private:
    opiv_batch* batch_ = nullptr;
    int n_pairs_ = 0, n_passes_ = 0;
};

// ---- image ingest ----------------------------------------------------------
// PNM / uncompressed TIFF -> 16-bit grey samples (8-bit files widened by value)
inline g16_image load_g16(const std::string& path)
{
    uint32_t w = 0, h = 0;
    int dtype = 0;
    check(opiv_image_info(path.c_str(), &w, &h, &dtype));
    g16_image im(w, h);
    if (dtype == OPIV_U16) {
        check(opiv_image_load(path.c_str(), im.data(), 2 * (size_t)w, w, h, OPIV_U16));
    } else {
        g8_image tmp(w, h);
        check(opiv_image_load(path.c_str(), tmp.data(), w, w, h, OPIV_U8));
        for (size_t k = 0; k < (size_t)w * h; ++k) im.data()[k] = tmp.data()[k];
    }
    return im;
}

}  // namespace openpiv::gb300
