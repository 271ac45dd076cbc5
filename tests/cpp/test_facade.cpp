// Host-side checks of the C++17 facade (openpiv_gb300.hpp): the reference's
// names and error messages, no GPU needed.  Prints "ok" on success.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "openpiv_gb300.hpp"

namespace gb = openpiv::gb300;

#define EXPECT(c)                                                   \
    do {                                                            \
        if (!(c)) {                                                 \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); \
            return 1;                                               \
        }                                                           \
    } while (0)

template <typename F>
bool throws_with(F f, const std::string& text)
{
    try {
        f();
    } catch (const std::runtime_error& e) {
        return std::string(e.what()).find(text) != std::string::npos;
    }
    return false;
}

int main()
{
    // tests/grid_test.cpp:57-71: {100, 50}, 32 x 32, 0.5 -> 10 windows, first at (2, 1)
    const auto g = gb::generate_cartesian_grid({ 100, 50 }, { 32, 32 }, 0.5);
    EXPECT(g.size() == 10);
    EXPECT(g[0].bottomLeft().x == 2 && g[0].bottomLeft().y == 1);
    EXPECT(g[9].bottomLeft().x == 66 && g[9].bottomLeft().y == 17);
    EXPECT(g[0].midpoint().x == 18 && g[0].midpoint().y == 17);
    const auto g2 = gb::generate_cartesian_grid({ 64, 64 }, { 32, 16 }, std::array<uint32_t, 2>{ 16, 8 });
    EXPECT(g2.size() == 21);
    EXPECT(throws_with([] { gb::generate_cartesian_grid({ 100, 100 }, { 32, 32 }, 1.5); },
                       "offsets must be between 0.0 and 1.0"));
    EXPECT(throws_with([] { gb::generate_cartesian_grid({ 16, 100 }, { 32, 32 }, 0.5); },
                       "interrogation size is bigger than image"));
    EXPECT(throws_with([] { gb::FFT f({ 512, 400 }); }, "power of 2"));

    // tests/image_utils_test.cpp:246-267: peaks in order 50, 40, 30
    gb::gf_image im(100, 100);
    im(20, 20) = 20.0;
    im(30, 30) = 30.0;
    im(40, 40) = 40.0;
    im(50, 50) = 50.0;
    const auto p = gb::find_peaks(im, 3, 1);
    EXPECT(p.size() == 3);
    EXPECT(p[0].centre.x == 50 && p[0].centre.y == 50 && p[0].value == 50.0);
    EXPECT(p[2].centre.x == 30 && p[2].value == 30.0);
    EXPECT(gb::find_peaks(gb::gf_image(100, 100), 3, 1).empty());

    // fit_simple_gaussian on a sampled Gaussian centred at (10.3, 7.8)
    gb::gf_image pl(32, 32);
    for (uint32_t y = 0; y < 32; ++y)
        for (uint32_t x = 0; x < 32; ++x)
            pl(x, y) = std::exp(-((x - 10.3) * (x - 10.3) + (y - 7.8) * (y - 7.8)) / 4.0);
    const auto q = gb::find_peaks(pl, 1, 1);
    EXPECT(q.size() == 1 && q[0].centre.x == 10 && q[0].centre.y == 8);
    const auto f = gb::fit_simple_gaussian(pl, q[0]);
    EXPECT(std::fabs(f.x - 10.3) < 1e-9 && std::fabs(f.y - 7.8) < 1e-9);

    // batches and passes check their window sizes before touching a device
    EXPECT(throws_with([] { gb::piv_batch b({ { 512, 512 } }, OPIV_U16, { { 24, 12 } }, OPIV_CORR_COMPLEX); },
                       "power of 2"));
    EXPECT(throws_with([] { gb::piv_pass p({ 512, 512 }, OPIV_U16, 24, 12, OPIV_CORR_COMPLEX); }, "power of 2"));
    std::printf("ok\n");
    return 0;
}
