// The per-window loop of OpenPIV-c++'s process example (examples/process/
// main.cpp:137-237: grid, correlator map, processor) with one change: the
// correlators are openpiv::gpu::FFT (openpiv_gpu.h) instead of algos::FFT.
//
// Built two ways:
//   -DOPIV_WITH_REFERENCE  against the reference's own headers (its
//                          core::image, image_view, g_f, rect, ...), with the
//                          reference's find_peaks, fit_simple_gaussian and
//                          generate_cartesian_grid; with -DOPIV_GPU_PEAKS the
//                          gpu:: versions of those three instead;
//   otherwise              against openpiv_standin.h, a test-only set of
//                          container types with the same interface (the GPU
//                          machine has no reference sources), with the gpu::
//                          peak, fit and grid functions.
//
// usage: process_dropin W H frame_a.u8 frame_b.u8 ia overlap fft_type limit [grid]
//   frames: raw 8-bit W x H row-major; overlap: the step fraction
//   (generate_cartesian_grid's third argument); fft_type: complex | real |
//   pocket | pocket_real; limit: 0 | 1 (main.cpp's -l); "grid": process the
//   whole grid with gpu::process_grid instead of the per-window loop.
// Prints "x, y, u, v, sn" per window (main.cpp:312-313) with 17 digits.
#include <cstdint>
#include <cstdio>
#include <cstring>   // the reference's util.impl.h uses memcpy without including it
#include <fstream>
#include <functional>
#include <iostream>
#include <string>
#include <unordered_map>
#include <vector>

#if defined(OPIV_WITH_REFERENCE)
#include "algos/fft_common.h"
#include "core/grid.h"
#include "core/image.h"
#include "core/image_utils.h"
#include "core/vector.h"
#else
#include "openpiv_standin.h"
#endif
#include "openpiv_gpu.h"

using namespace openpiv;

#if defined(OPIV_WITH_REFERENCE) && !defined(OPIV_GPU_PEAKS)
namespace peak_fns = openpiv::core;
#else
namespace peak_fns = openpiv::gpu;
#endif

static core::gf_image load_u8(const char* path, uint32_t w, uint32_t h)
{
    std::vector<uint8_t> raw((size_t)w * h);
    std::ifstream f(path, std::ios::binary);
    f.read(reinterpret_cast<char*>(raw.data()), (std::streamsize)raw.size());
    if (!f) throw std::runtime_error(std::string("cannot read ") + path);
    core::gf_image im(w, h);
    // the loaders convert integer samples to g_f by value
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) im.line(y)[x] = (double)raw[(size_t)y * w + x];
    return im;
}

int main(int argc, char* argv[])
{
    if (argc < 9) {
        std::cerr << "usage: process_dropin W H a.u8 b.u8 ia overlap fft_type limit [grid]\n";
        return 2;
    }
    const uint32_t W = (uint32_t)std::stoul(argv[1]), H = (uint32_t)std::stoul(argv[2]);
    std::vector<core::gf_image> images{ load_u8(argv[3], W, H), load_u8(argv[4], W, H) };
    const uint32_t size = (uint32_t)std::stoul(argv[5]);
    const double overlap = std::stod(argv[6]);
    const std::string fft_type = argv[7];
    const bool limit_search = std::string(argv[8]) == "1";
    const bool whole_grid = argc > 9 && std::string(argv[9]) == "grid";

    // main.cpp:137-138
    core::size ia{ size, size };
    auto grid = peak_fns::generate_cartesian_grid(images[0].size(), ia, overlap);

    struct point_vector
    {
        core::point2<double> xy;
        core::vector2<double> vxy;
        double sn = 0.0;
    };
    std::vector<point_vector> found_peaks(grid.size());

    if (whole_grid) {
        // the whole loop as one GPU pass
        const auto v = gpu::process_grid(images[0], images[1], grid, fft_type, limit_search);
        for (size_t i = 0; i < v.size(); ++i) found_peaks[i] = { v[i].xy, v[i].vxy, v[i].sn };
    } else {
        // main.cpp:153-178, the correlators on the GPU
        using correlator_t = std::function<core::gf_image(const core::gf_image&, const core::gf_image&)>;
        std::unordered_map<std::string, correlator_t> correlators = {
            { "complex",
              [ia](const core::gf_image& im_a, const core::gf_image& im_b) -> core::gf_image {
                  static gpu::FFT fft{ ia };
                  return fft.cross_correlate(im_a, im_b);
              } },
            { "real",
              [ia](const core::gf_image& im_a, const core::gf_image& im_b) -> core::gf_image {
                  static gpu::FFT fft{ ia };
                  return fft.cross_correlate_real(im_a, im_b);
              } },
            // PocketFFT's c2c / r2c-c2r correlation is the true circular
            // correlation, which cross_correlate computes
            { "pocket",
              [ia](const core::gf_image& im_a, const core::gf_image& im_b) -> core::gf_image {
                  static gpu::FFT fft{ ia };
                  return fft.cross_correlate(im_a, im_b);
              } },
            { "pocket_real",
              [ia](const core::gf_image& im_a, const core::gf_image& im_b) -> core::gf_image {
                  static gpu::FFT fft{ ia };
                  return fft.cross_correlate(im_a, im_b);
              } } };
        if (correlators.count(fft_type) == 0) {
            std::cerr << "unknown fft type: " << fft_type << "\n";
            return 1;
        }
        auto correlator = correlators[fft_type];

        // main.cpp:189-237
        auto processor = [&images, &found_peaks, correlator = std::move(correlator),
                          limit_search](size_t i, const core::rect& ia) {
            const auto view_a{ core::extract(images[0], ia) };
            const auto view_b{ core::extract(images[1], ia) };
            const core::gf_image output{ correlator(view_a, view_b) };

            constexpr uint16_t num_peaks = 2;
            constexpr uint16_t radius = 1;
            core::peaks_t<core::g_f> peaks;
            if (limit_search) {
                auto centre = core::create_image_view(output, output.rect().dilate(0.5));
                peaks = peak_fns::find_peaks(centre, num_peaks, radius);
            } else {
                peaks = peak_fns::find_peaks(output, num_peaks, radius);
            }
            if (peaks.size() != num_peaks) return;

            point_vector result;
            auto bl = ia.bottomLeft();
            auto midpoint = ia.midpoint();
            auto peak = peaks[0];
            auto peak_location = peak_fns::fit_simple_gaussian(peak);

            result.xy = midpoint;
            result.vxy = { midpoint[0] - (bl[0] + peak_location[0]), midpoint[1] - (bl[1] + peak_location[1]) };
            result.xy[1] = images[0].height() - result.xy[1];
            if (peaks[1][{ 1, 1 }] > 0) result.sn = peaks[0][{ 1, 1 }] / peaks[1][{ 1, 1 }];
            found_peaks[i] = std::move(result);
        };

        size_t i = 0;
        for (const auto& r : grid) processor(i++, r);
    }

    std::cout.precision(17);
    for (const auto& pv : found_peaks)
        std::cout << pv.xy[0] << ", " << pv.xy[1] << ", " << pv.vxy[0] << ", " << pv.vxy[1] << ", " << pv.sn
                  << "\n";
    return 0;
}
