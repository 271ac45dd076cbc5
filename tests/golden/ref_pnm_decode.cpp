// Decodes a PNM file through the reference's own loader
// (loaders/pnm_image_loader.cpp, found through image_loader_registry::find
// as examples/process/main.cpp:104-125 does) into 16-bit grey samples.
// Built and run by make_ingest_golden.py on a machine with the reference
// sources; the decoded samples become the committed fixture.
//
// usage: ref_pnm_decode in.pnm out.raw
//   out.raw: uint32 width, uint32 height, then width * height uint16
//   samples, little-endian, row-major
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>

#include "core/image.h"
#include "loaders/image_loader.h"

int main(int argc, char* argv[])
{
    using namespace openpiv;
    if (argc != 3) return 2;
    std::ifstream is(argv[1], std::ios::binary);
    auto loader = core::image_loader_registry::find(is);
    if (!loader) {
        std::cerr << "no loader for " << argv[1] << "\n";
        return 1;
    }
    core::g16_image im;
    if (!loader->load(is, im)) return 1;
    std::ofstream os(argv[2], std::ios::binary);
    const uint32_t wh[2] = { im.width(), im.height() };
    os.write(reinterpret_cast<const char*>(wh), sizeof wh);
    for (uint32_t y = 0; y < im.height(); ++y)
        for (uint32_t x = 0; x < im.width(); ++x) {
            const uint16_t v = im.line(y)[x];
            const unsigned char b[2] = { (unsigned char)(v & 0xff), (unsigned char)(v >> 8) };
            os.write(reinterpret_cast<const char*>(b), 2);
        }
    return os ? 0 : 1;
}
