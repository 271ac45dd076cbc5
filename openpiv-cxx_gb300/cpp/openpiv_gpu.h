// openpiv_gpu.h -- OpenPIV-c++'s correlator and peak interface, computed by
// this library's CUDA kernels, as templates over the caller's own openpiv
// image types.
//
// What it replaces (the reference's names and signatures, same arguments,
// same return types, same exceptions):
//
//   reference                                       here
//   algos::FFT(size)             fft.h:76-84        gpu::FFT(size)
//   FFT::transform(im, d)        fft.h:87-119       gpu::FFT::transform
//   FFT::transform_real(a, b, d) fft.h:123-186      gpu::FFT::transform_real
//   FFT::cross_correlate(a, b)   fft.h:188-206      gpu::FFT::cross_correlate
//   FFT::cross_correlate_real    fft.h:208-227      gpu::FFT::cross_correlate_real
//   FFT::auto_correlate(a)       fft.h:229-242      gpu::FFT::auto_correlate
//   core::find_peaks             image_utils.impl.h:42-74   gpu::find_peaks
//   core::fit_simple_gaussian    image_utils.impl.h:77-101  gpu::fit_simple_gaussian
//   core::generate_cartesian_grid grid.impl.h:9-61  gpu::generate_cartesian_grid
//   (no counterpart)                                gpu::FFT::correlate_grid, gpu::process_grid
//
// Swapping it into examples/process/main.cpp: include this header after the
// openpiv headers and write `gpu::FFT` where the correlator map says
// `algos::FFT` (main.cpp:153-178); nothing else changes.  The correlation,
// the transforms and the per-window arithmetic run on the GPU in double
// precision with the reference's own butterflies, twiddle tables and complex
// products, so every plane equals the reference's bit for bit, and the
// caller's core::find_peaks / core::fit_simple_gaussian give the reference's
// vectors.  gpu::process_grid runs the whole per-window loop of
// main.cpp:189-237 as one batched pass (FP32 kernels plus the exact
// re-decision: integer peaks identical to the reference, u, v within
// 1e-4 px).
//
// This header includes no openpiv header and links nothing of OpenPIV-c++:
// it is written against the caller's types, which must be declared first --
// include it after core/image.h, core/image_view.h, core/image_utils.h,
// core/rect.h, core/vector.h and algos/fft_common.h (the headers the
// process example includes anyway).  The types it uses: core::size, rect,
// point2, vector2, g<T>, c_f / cf_image, image<T>, image_view<T>,
// create_image_view, peaks_t and algos::direction.
//
// Per call, the per-window functions copy one window pair to the GPU and the
// result back (the interface hands over one window at a time); for many
// windows use correlate_grid (one batched call) or process_grid (the whole
// pass in one launch pair).  A GPU is required: with no CUDA device every
// GPU-backed call throws std::runtime_error.  Thread-safe like the
// reference's FFT: transform and auto_correlate return references to
// per-thread, per-instance storage.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "openpiv_gb300.h"

namespace openpiv::gpu {

namespace detail {

inline void check(int status)
{
    if (status < 0) throw std::runtime_error(opiv_last_error());
}

inline bool is_pow2(uint32_t v) { return v != 0 && (v & (v - 1)) == 0; }

// complex pixel types (c_f and the like) have real and imag members
template <typename P, typename = void>
struct is_complex_px : std::false_type {};
template <typename P>
struct is_complex_px<P, std::void_t<decltype(std::declval<const P&>().real),
                                    decltype(std::declval<const P&>().imag)>> : std::true_type {};

// window pixels as interleaved (re, im) doubles: the reference's conversion
// to c_f (image::operator=, image.h:136-145, pixel_types.h:432-439)
template <typename ImageT>
void to_complex(const ImageT& im, double* out)
{
    using P = std::remove_cv_t<std::remove_reference_t<decltype(im.line(0)[0])>>;
    for (uint32_t h = 0; h < im.height(); ++h) {
        const auto* line = im.line(h);
        for (uint32_t w = 0; w < im.width(); ++w) {
            if constexpr (is_complex_px<P>::value) {
                out[2 * (h * im.width() + w)] = (double)line[w].real;
                out[2 * (h * im.width() + w) + 1] = (double)line[w].imag;
            } else {
                out[2 * (h * im.width() + w)] = (double)line[w];
                out[2 * (h * im.width() + w) + 1] = 0.0;
            }
        }
    }
}

// window pixels as real doubles (g<T> converts by value)
template <typename ImageT>
void to_real(const ImageT& im, double* out)
{
    for (uint32_t h = 0; h < im.height(); ++h) {
        const auto* line = im.line(h);
        for (uint32_t w = 0; w < im.width(); ++w) out[h * im.width() + w] = (double)line[w];
    }
}

template <typename ImageT>
void from_complex(const double* in, ImageT& im)
{
    using P = std::remove_cv_t<std::remove_reference_t<decltype(im.line(0)[0])>>;
    for (uint32_t h = 0; h < im.height(); ++h) {
        auto* line = im.line(h);
        for (uint32_t w = 0; w < im.width(); ++w)
            line[w] = P{ in[2 * (h * im.width() + w)], in[2 * (h * im.width() + w) + 1] };
    }
}

template <typename ImageT>
void from_real(const double* in, ImageT& im)
{
    for (uint32_t h = 0; h < im.height(); ++h) {
        auto* line = im.line(h);
        for (uint32_t w = 0; w < im.width(); ++w) line[w] = in[h * im.width() + w];
    }
}

template <typename SizeT>
std::string size_text(const SizeT& s)
{
    std::ostringstream os;
    os << s;
    return os.str();
}

// pixel type code of the C ABI for a mono pixel type's value_t
template <typename V>
constexpr int dtype_of()
{
    if constexpr (std::is_same_v<V, uint8_t>) return OPIV_U8;
    else if constexpr (std::is_same_v<V, uint16_t>) return OPIV_U16;
    else return OPIV_F32;   // float, double (converted to float), other integers
}

}  // namespace detail

// ---- algos::FFT on the GPU ---------------------------------------------------
class FFT {
public:
    /// fft.h:76-84: the window size; throws std::runtime_error("dimensions
    /// must be power of 2: ...") for other sizes.  `device`: the CUDA device.
    explicit FFT(const core::size& size, int device = 0) : size_(size), device_(device)
    {
        if (!(detail::is_pow2(size_.width()) && detail::is_pow2(size_.height())))
            throw std::runtime_error("dimensions must be power of 2: " + detail::size_text(size_));
    }

    const core::size& size() const { return size_; }

    /// fft.h:87-119: unnormalised 2-D transform, complex output (a reference
    /// to per-thread, per-instance storage, as the reference returns).
    template <template <typename> class ImageT, typename ContainedT>
    const core::cf_image& transform(const ImageT<ContainedT>& input,
                                    algos::direction d = algos::direction::FORWARD) const
    {
        check_size(input.size());
        std::vector<double> in(2 * area()), out(2 * area());
        detail::to_complex(input, in.data());
        detail::check(opiv_transform_batch(in.data(), size_.width(), 1,
                                           d == algos::direction::FORWARD ? OPIV_FORWARD : OPIV_REVERSE,
                                           out.data(), device_));
        core::cf_image& result = cache();
        detail::from_complex(out.data(), result);
        return result;
    }

    /// fft.h:123-186: two real windows through one complex transform, with
    /// the reference's partial unpack (spectrum row 0, row H/2 and column 0
    /// stay zero).
    template <template <typename> class ImageT, typename ContainedT>
    std::tuple<core::cf_image, core::cf_image>
    transform_real(const ImageT<ContainedT>& a, const ImageT<ContainedT>& b,
                   algos::direction d = algos::direction::FORWARD) const
    {
        check_size(a.size());
        check_size(b.size());
        std::vector<double> ra(area()), rb(area()), oa(2 * area()), ob(2 * area());
        detail::to_real(a, ra.data());
        detail::to_real(b, rb.data());
        detail::check(opiv_transform_real_batch(ra.data(), rb.data(), size_.width(), 1,
                                                d == algos::direction::FORWARD ? OPIV_FORWARD : OPIV_REVERSE,
                                                oa.data(), ob.data(), device_));
        core::cf_image out_a(size_), out_b(size_);
        detail::from_complex(oa.data(), out_a);
        detail::from_complex(ob.data(), out_b);
        return { std::move(out_a), std::move(out_b) };
    }

    /// fft.h:188-206: IFFT(FFT(b) conj FFT(a)), quadrant-swapped; the
    /// reference's return type image<g<value_t>>.
    template <template <typename> class ImageT, typename ContainedT,
              typename ValueT = typename ContainedT::value_t, typename OutT = core::image<core::g<ValueT>>>
    OutT cross_correlate(const ImageT<ContainedT>& a, const ImageT<ContainedT>& b) const
    {
        return correlate<OutT>(a, b, OPIV_CORR_COMPLEX);
    }

    /// fft.h:208-227: the same with transform_real's unpack.
    template <template <typename> class ImageT, typename ContainedT,
              typename ValueT = typename ContainedT::value_t, typename OutT = core::image<core::g<ValueT>>>
    OutT cross_correlate_real(const ImageT<ContainedT>& a, const ImageT<ContainedT>& b) const
    {
        return correlate<OutT>(a, b, OPIV_CORR_REAL);
    }

    /// fft.h:229-242: real(IFFT(|FFT(a)|^2)), quadrant-swapped, as a complex
    /// image (per-thread, per-instance storage).
    template <template <typename> class ImageT, typename ContainedT>
    const core::cf_image& auto_correlate(const ImageT<ContainedT>& a) const
    {
        check_size(a.size());
        std::vector<double> in(2 * area()), out(2 * area());
        detail::to_complex(a, in.data());
        detail::check(opiv_auto_correlate_batch(in.data(), size_.width(), 1, out.data(), device_));
        core::cf_image& result = cache();
        detail::from_complex(out.data(), result);
        return result;
    }

    /// No counterpart in the reference: cross_correlate (complex = true) or
    /// cross_correlate_real of every window of `grid`, extracted from
    /// frames a and b (core::extract, image_utils.impl.h:392-419), in one
    /// batched GPU call.  Planes in grid order, as a per-window loop of
    /// cross_correlate[_real] over extract(a, r), extract(b, r) returns them.
    template <template <typename> class ImageT, typename ContainedT,
              typename ValueT = typename ContainedT::value_t, typename OutT = core::image<core::g<ValueT>>>
    std::vector<OutT> correlate_grid(const ImageT<ContainedT>& a, const ImageT<ContainedT>& b,
                                     const std::vector<core::rect>& grid, bool complex = true) const
    {
        if (a.size() != b.size())
            throw std::runtime_error("image size is different from expected: " + detail::size_text(a.size()) +
                                     ", " + detail::size_text(b.size()));
        const size_t N = area();
        std::vector<double> wa(N * grid.size()), wb(N * grid.size());
        for (size_t k = 0; k < grid.size(); ++k) {
            const core::rect& r = grid[k];
            check_size(r.size());
            if (r.bottomLeft()[0] < 0 || r.bottomLeft()[1] < 0 ||
                (uint64_t)r.bottomLeft()[0] + r.width() > a.width() ||
                (uint64_t)r.bottomLeft()[1] + r.height() > a.height())
                throw std::runtime_error("extract: rectangle to extract is too large for image");
            for (uint32_t h = 0; h < r.height(); ++h) {
                const auto* la = a.line(r.bottomLeft()[1] + h) + r.bottomLeft()[0];
                const auto* lb = b.line(r.bottomLeft()[1] + h) + r.bottomLeft()[0];
                for (uint32_t w = 0; w < r.width(); ++w) {
                    wa[k * N + h * r.width() + w] = (double)la[w];
                    wb[k * N + h * r.width() + w] = (double)lb[w];
                }
            }
        }
        std::vector<double> planes(N * grid.size());
        detail::check(opiv_cross_correlate_batch(wa.data(), wb.data(), size_.width(), (int64_t)grid.size(),
                                                 complex ? OPIV_CORR_COMPLEX : OPIV_CORR_REAL, 1,
                                                 planes.data(), device_));
        std::vector<OutT> out;
        out.reserve(grid.size());
        for (size_t k = 0; k < grid.size(); ++k) {
            OutT plane(size_);
            detail::from_real(planes.data() + k * N, plane);
            out.push_back(std::move(plane));
        }
        return out;
    }

private:
    size_t area() const { return (size_t)size_.width() * size_.height(); }

    template <typename SizeT>
    void check_size(const SizeT& s) const
    {
        if (s.width() != size_.width() || s.height() != size_.height())
            throw std::runtime_error("image size is different from expected: " + detail::size_text(s) + ", " +
                                     detail::size_text(size_));
        // the reference's transpose step rejects non-square windows
        // (image_utils.impl.h:330-333); so do the kernels here
        if (size_.width() != size_.height())
            throw std::runtime_error("input and output must have transposed dimensions: " +
                                     detail::size_text(size_) + ", " + detail::size_text(size_));
    }

    template <typename OutT, typename ImgA>
    OutT correlate(const ImgA& a, const ImgA& b, int mode) const
    {
        check_size(a.size());
        check_size(b.size());
        std::vector<double> wa(area()), wb(area()), plane(area());
        detail::to_real(a, wa.data());
        detail::to_real(b, wb.data());
        detail::check(opiv_cross_correlate_batch(wa.data(), wb.data(), size_.width(), 1, mode, 1, plane.data(),
                                                 device_));
        OutT out(size_);
        detail::from_real(plane.data(), out);
        return out;
    }

    // per-thread, per-instance result storage (the reference's TLS cache,
    // fft.h:37-73)
    core::cf_image& cache() const
    {
        thread_local std::vector<std::pair<const FFT*, core::cf_image>> store;
        for (auto& [owner, im] : store)
            if (owner == this && im.size() == size_) return im;
        store.emplace_back(this, core::cf_image(size_));
        return store.back().second;
    }

    core::size size_;
    int device_ = 0;
};

// ---- core::find_peaks / fit_simple_gaussian ----------------------------------

/// image_utils.impl.h:42-74: strict 4-neighbour maxima of rows
/// [r, H - 2r) and columns [r, W - r), highest first (std::sort with the
/// reference's comparator, so ties come out in the reference's order),
/// cut to num_peaks; each peak is a (2r + 1)^2 view into `im`, which must
/// outlive the views.
template <template <typename> class ImageT, typename ContainedT>
std::vector<core::image_view<ContainedT>> find_peaks(const ImageT<ContainedT>& im, uint16_t num_peaks,
                                                     uint32_t peak_radius)
{
    const uint32_t W = im.width(), H = im.height();
    std::vector<double> plane((size_t)W * H);
    detail::to_real(im, plane.data());
    // the host helper of the C ABI: the peaks of one plane the caller holds
    std::vector<int32_t> xy(2 * (size_t)num_peaks + 2);
    std::vector<double> values((size_t)num_peaks + 1);
    const int n = opiv_find_peaks(plane.data(), W, H, num_peaks, peak_radius, xy.data(), values.data());
    detail::check(n);
    std::vector<core::image_view<ContainedT>> result;
    const uint32_t side = 2 * peak_radius + 1;
    for (int k = 0; k < n; ++k) {
        const core::rect r{ { (int32_t)(xy[2 * k] - (int32_t)peak_radius),
                              (int32_t)(xy[2 * k + 1] - (int32_t)peak_radius) },
                            { side, side } };
        result.push_back(core::create_image_view(im, r));
    }
    return result;
}

/// image_utils.impl.h:77-101: the view's midpoint plus the 3-point Gaussian
/// offsets on each axis; throws std::runtime_error for views other than 3x3.
template <template <typename> class ImageT, typename ContainedT>
core::point2<double> fit_simple_gaussian(const ImageT<ContainedT>& im)
{
    if (im.width() != 3 || im.height() != 3)
        throw std::runtime_error("fit_simple_gaussian: input must be 3x3");
    double v[9];
    detail::to_real(im, v);
    double f[2];
    detail::check(opiv_gaussian_offsets(v, f));
    core::point2<double> result{ im.rect().midpoint() };
    result[0] += f[0];
    result[1] += f[1];
    return result;
}

// ---- core::generate_cartesian_grid ---------------------------------------------

namespace detail {
inline std::vector<core::rect> to_rects(const std::vector<int32_t>& xy, const core::size& ia)
{
    std::vector<core::rect> out;
    out.reserve(xy.size() / 2);
    for (size_t k = 0; k < xy.size() / 2; ++k) out.push_back(core::rect{ { xy[2 * k], xy[2 * k + 1] }, ia });
    return out;
}
}  // namespace detail

/// grid.impl.h:9-22: step = (uint32)(ia * offset) per axis.
inline std::vector<core::rect> generate_cartesian_grid(const core::size& image_size, const core::size& ia,
                                                       double offset)
{
    const int64_t n = opiv_grid(image_size.width(), image_size.height(), ia.width(), ia.height(), offset,
                                nullptr, 0);
    detail::check((int)(n < 0 ? n : 0));
    std::vector<int32_t> xy(2 * (size_t)n);
    detail::check((int)opiv_grid(image_size.width(), image_size.height(), ia.width(), ia.height(), offset,
                                 xy.data(), n));
    return detail::to_rects(xy, ia);
}

/// grid.impl.h:24-61: explicit offsets in pixels, centred, row-major.
inline std::vector<core::rect> generate_cartesian_grid(const core::size& image_size, const core::size& ia,
                                                       std::array<uint32_t, 2> offsets)
{
    const int64_t n = opiv_grid_offsets(image_size.width(), image_size.height(), ia.width(), ia.height(),
                                        offsets[0], offsets[1], nullptr, 0);
    detail::check((int)(n < 0 ? n : 0));
    std::vector<int32_t> xy(2 * (size_t)n);
    detail::check((int)opiv_grid_offsets(image_size.width(), image_size.height(), ia.width(), ia.height(),
                                         offsets[0], offsets[1], xy.data(), n));
    return detail::to_rects(xy, ia);
}

// ---- the whole per-window loop --------------------------------------------------

/// One window's result, as the process example's point_vector
/// (main.cpp:144-149).
struct piv_vector {
    core::point2<double> xy;
    core::vector2<double> vxy;
    double sn = 0.0;
};

/// No counterpart in the reference: the processor of main.cpp:189-237 over
/// every window of `grid` as one GPU pass.  `grid` must be a lattice that
/// generate_cartesian_grid makes (equal square power-of-2 windows, constant
/// steps, centred, row-major); std::invalid_argument otherwise.  fft_type
/// "complex", "real", "pocket" or "pocket_real" as main.cpp:153-178.  8- and
/// 16-bit pixel types go to the GPU as they are; other mono types are
/// converted to float (exact for integer values below 2^24).
template <template <typename> class ImageT, typename ContainedT>
std::vector<piv_vector> process_grid(const ImageT<ContainedT>& a, const ImageT<ContainedT>& b,
                                     const std::vector<core::rect>& grid, const std::string& fft_type,
                                     bool limit_search = false, int device = 0)
{
    using V = typename ContainedT::value_t;
    constexpr int dtype = detail::dtype_of<V>();
    using PixT = std::conditional_t<dtype == OPIV_U8, uint8_t,
                                    std::conditional_t<dtype == OPIV_U16, uint16_t, float>>;
    const int mode = fft_type == "complex" ? OPIV_CORR_COMPLEX
                     : fft_type == "real" ? OPIV_CORR_REAL
                     : fft_type == "pocket" ? OPIV_CORR_POCKET
                     : fft_type == "pocket_real" ? OPIV_CORR_POCKET_REAL : -1;
    if (mode < 0) throw std::invalid_argument("unknown fft type: " + fft_type);
    if (a.size() != b.size())
        throw std::runtime_error("image size is different from expected: " + detail::size_text(a.size()) +
                                 ", " + detail::size_text(b.size()));
    if (grid.empty()) return {};
    // the lattice: first row's x step, the rows' y step
    const uint32_t ia = grid[0].width();
    size_t nx = 1;
    while (nx < grid.size() && grid[nx].bottomLeft()[1] == grid[0].bottomLeft()[1]) ++nx;
    const uint32_t dx = nx > 1 ? (uint32_t)(grid[1].bottomLeft()[0] - grid[0].bottomLeft()[0]) : 1;
    const uint32_t dy = grid.size() > nx ? (uint32_t)(grid[nx].bottomLeft()[1] - grid[0].bottomLeft()[1]) : 1;
    const int64_t n_expect = opiv_grid_offsets(a.width(), a.height(), ia, ia, dx, dy, nullptr, 0);
    std::vector<int32_t> xy(2 * (size_t)std::max<int64_t>(n_expect, 0));
    bool lattice = grid[0].height() == ia && n_expect == (int64_t)grid.size() &&
                   opiv_grid_offsets(a.width(), a.height(), ia, ia, dx, dy, xy.data(), n_expect) == n_expect;
    for (size_t k = 0; lattice && k < grid.size(); ++k)
        lattice = grid[k].width() == ia && grid[k].height() == ia && grid[k].bottomLeft()[0] == xy[2 * k] &&
                  grid[k].bottomLeft()[1] == xy[2 * k + 1];
    if (!lattice)
        throw std::invalid_argument("process_grid: the grid is not a generate_cartesian_grid lattice; "
                                    "use FFT::correlate_grid");
    // frames in the plan's pixel type
    std::vector<PixT> fa((size_t)a.width() * a.height()), fb(fa.size());
    for (uint32_t h = 0; h < a.height(); ++h) {
        const auto* la = a.line(h);
        const auto* lb = b.line(h);
        for (uint32_t w = 0; w < a.width(); ++w) {
            fa[(size_t)h * a.width() + w] = (PixT)(V)la[w];
            fb[(size_t)h * a.width() + w] = (PixT)(V)lb[w];
        }
    }
    opiv_plan* plan = nullptr;
    detail::check(opiv_plan_create(&plan, a.width(), a.height(), dtype, ia, dx, dy, mode, limit_search ? 1 : 0,
                                   device));
    std::vector<opiv_vector> vec(grid.size());
    const int rc = opiv_process_pair(plan, fa.data(), fb.data(), sizeof(PixT) * a.width(), vec.data(), nullptr);
    opiv_plan_destroy(plan);
    detail::check(rc);
    std::vector<piv_vector> out(grid.size());
    for (size_t k = 0; k < grid.size(); ++k) {
        out[k].xy = core::point2<double>{ (double)vec[k].x, (double)vec[k].y };
        out[k].vxy = core::vector2<double>{ (double)vec[k].u, (double)vec[k].v };
        out[k].sn = vec[k].sn;
    }
    return out;
}

}  // namespace openpiv::gpu
