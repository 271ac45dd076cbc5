// process_gb300 -- the reference's examples/process, with the per-window loop
// (main.cpp:189-302) replaced by one GPU pass through the C ABI.
//
//   process_gb300 [-s size] [-o overlap] [-f complex|real|pocket|pocket_real]
//                 [-l] [-d device]
//                 [-i] frame_a frame_b
//
// Same options and meaning as main.cpp:53-63: -s interrogation size
// (default 32), -o the step fraction (default 0.5: step = size * 0.5),
// -f FFT type (default complex), -l limit the peak search to the central
// 25 % of the correlation plane.  Frames: PNM (P5/P6) or uncompressed TIFF.
// Prints "x, y, u, v, sn" per window to stdout (main.cpp:312-313) and the
// processing time to stderr (main.cpp:304-309).

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "openpiv_gb300.hpp"

namespace gb = openpiv::gb300;

int main(int argc, char** argv)
{
    uint32_t size = 32;
    double overlap = 0.5;
    std::string fft_type = "complex";
    bool limit_search = false;
    int device = 0;
    std::vector<std::string> inputs;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&]() -> std::string {
            if (i + 1 >= argc) {
                std::cerr << "missing value for " << a << "\n";
                std::exit(1);
            }
            return argv[++i];
        };
        if (a == "-s" || a == "--size") size = (uint32_t)std::stoul(next());
        else if (a == "-o" || a == "--overlap") overlap = std::stod(next());
        else if (a == "-f" || a == "--ffttype") fft_type = next();
        else if (a == "-l" || a == "--limit-search") limit_search = true;
        else if (a == "-d" || a == "--device") device = std::stoi(next());
        else if (a == "-i" || a == "--input") inputs.push_back(next());
        else if (a == "-h" || a == "--help") {
            std::cout << "process_gb300 [-s size] [-o overlap] [-f complex|real] [-l] [-d device] a b\n";
            return 0;
        } else inputs.push_back(a);
    }
    if (inputs.size() != 2) {
        std::cerr << "require two input images\n";
        return 1;
    }
    int mode;
    if (fft_type == "complex") mode = OPIV_CORR_COMPLEX;
    else if (fft_type == "real") mode = OPIV_CORR_REAL;
    else if (fft_type == "pocket") mode = OPIV_CORR_POCKET;
    else if (fft_type == "pocket_real") mode = OPIV_CORR_POCKET_REAL;
    else {
        std::cerr << "unknown fft type: " << fft_type << "\n";
        return 1;
    }
    try {
        const gb::g16_image a = gb::load_g16(inputs[0]);
        const gb::g16_image b = gb::load_g16(inputs[1]);
        if (a.size() != b.size()) {
            std::cerr << "image sizes don't match\n";
            return 1;
        }
        // generate_cartesian_grid(size, ia, overlap): step = (uint32_t)(ia * overlap)
        const gb::size ia{ size, size };
        const auto grid = gb::generate_cartesian_grid(a.size(), ia, overlap);
        std::cerr << "size: " << size << " x " << size << "\noverlap: " << overlap
                  << "\ngrid count: " << grid.size() << "\n";
        const uint32_t step = (uint32_t)(size * overlap);
        gb::piv_pass pass(a.size(), OPIV_U16, size, step, mode, limit_search, device);
        const auto t1 = std::chrono::steady_clock::now();
        const std::vector<opiv_vector> out = pass.process(a, b);
        const auto t2 = std::chrono::steady_clock::now();
        const double us = std::chrono::duration<double, std::micro>(t2 - t1).count();
        std::cerr << "processing time: " << us << "us, " << us / (double)out.size()
                  << "us per interrogation area\n";
        gb::check(opiv_vectors_write(nullptr, out.data(), (int64_t)out.size()));
    } catch (const std::exception& e) {
        std::cerr << e.what() << "\n";
        return 1;
    }
    return 0;
}
