// The C++ facade's piv_batch on the GPU: two synthetic pairs of different
// sizes through a 64/32/16 px multi-pass schedule, the streams schedule
// against the queue schedule after autotune(); every pass's vectors must be
// bit-identical.  Prints "ok".
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "openpiv_gb300.hpp"

namespace gb = openpiv::gb300;

// particles as 3x3 blobs at LCG positions, frame b shifted by (3, -2)
static void make_pair(uint32_t w, uint32_t h, uint32_t seed, gb::image<uint16_t>& a, gb::image<uint16_t>& b)
{
    a = gb::image<uint16_t>(w, h);
    b = gb::image<uint16_t>(w, h);
    uint32_t s = seed;
    auto next = [&s]() { s = s * 1664525u + 1013904223u; return s >> 8; };
    const uint32_t n = w * h / 40;
    for (uint32_t k = 0; k < n; ++k) {
        const int x = (int)(next() % w), y = (int)(next() % h);
        const uint16_t v = (uint16_t)(1500 + next() % 2500);
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const uint16_t q = (dx == 0 && dy == 0) ? v : (uint16_t)(v / 3);
                const int ax = x + dx, ay = y + dy, bx = ax + 3, by = ay - 2;
                if (ax >= 0 && ay >= 0 && ax < (int)w && ay < (int)h) a(ax, ay) = q > a(ax, ay) ? q : a(ax, ay);
                if (bx >= 0 && by >= 0 && bx < (int)w && by < (int)h) b(bx, by) = q > b(bx, by) ? q : b(bx, by);
            }
    }
}

int main()
{
    const std::vector<gb::size> sizes = { { 512, 384 }, { 768, 512 } };
    const std::vector<gb::piv_batch::pass> passes = { { 64, 32 }, { 32, 16 }, { 16, 8 } };
    gb::piv_batch batch(sizes, OPIV_U16, passes, OPIV_CORR_COMPLEX);
    std::vector<gb::image<uint16_t>> fa(2), fb(2);
    for (int i = 0; i < 2; ++i) {
        make_pair(sizes[i].w, sizes[i].h, 7u + 11u * (uint32_t)i, fa[i], fb[i]);
        batch.upload(i, fa[i], fb[i]);
    }
    batch.run(false);
    std::vector<std::vector<opiv_vector>> ref;
    for (int i = 0; i < 2; ++i)
        for (int k = 0; k < 3; ++k) ref.push_back(batch.results(i, k));
    batch.set_schedule(OPIV_BATCH_QUEUE);
    batch.autotune();
    batch.run(true);
    batch.run(true);
    int bad = 0, found = 0;
    for (int i = 0; i < 2; ++i)
        for (int k = 0; k < 3; ++k) {
            const auto got = batch.results(i, k);
            const auto& r = ref[(size_t)(3 * i + k)];
            if (got.size() != r.size() || std::memcmp(got.data(), r.data(), sizeof(opiv_vector) * r.size()) != 0)
                ++bad;
            for (const opiv_vector& v : got) found += v.sn > 0.f;
        }
    if (bad || found == 0) {
        std::printf("mismatch: %d passes differ, %d vectors found\n", bad, found);
        return 1;
    }
    std::printf("ok\n");
    return 0;
}
