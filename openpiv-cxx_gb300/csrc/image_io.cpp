// image_io.cpp -- image ingest and vector output for the PIV path (host C++).
//
// Ingest mirrors what the reference's loaders hand to examples/process:
//   * PNM (loaders/pnm_image_loader.cpp): binary P5 grey and P6 RGB, 8-bit
//     samples or 16-bit big-endian samples (maxval > 255, :199-226); RGB is
//     turned into grey with (218 r + 732 g + 74 b) >> 10
//     (core/pixel_types.h:390-400).  Samples are read as unsigned bytes (the
//     reference's 8-bit RGB copy goes through a signed char, which corrupts
//     samples above 127 where char is signed; that is not reproduced).
//   * TIFF (loaders/tiff_image_loader.cpp:41-79, :190-226, via libtiff
//     there): baseline uncompressed TIFF read directly -- little or big
//     endian, strips, chunky samples, 1 or 3 samples of 8 or 16 bits, first
//     image of the file.  Compressed TIFF is refused with a clear error.
// The loaders widen the 8/16-bit samples to double by value; the GPU path
// takes the 8/16-bit samples themselves (same values).
//
// Output mirrors main.cpp:312-313: one "x, y, u, v, sn" line per window,
// default stream formatting (6 significant digits, "%g").

#include <cerrno>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "openpiv_gb300.h"
#include "piv_kernels.h"

namespace {

int io_fail(int status, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return opiv::record_error(status, buf);
}

bool read_file(const char* path, std::vector<uint8_t>& out)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0) { std::fclose(f); return false; }
    out.resize((size_t)n);
    const size_t got = n ? std::fread(out.data(), 1, (size_t)n, f) : 0;
    std::fclose(f);
    return got == (size_t)n;
}

struct decoded {
    uint32_t w = 0, h = 0;
    int bits = 8;                  // 8 or 16 (per output sample)
    std::vector<uint16_t> px;      // grey samples, row-major
};

inline uint16_t grey_from_rgb(uint32_t r, uint32_t g, uint32_t b)
{
    return (uint16_t)((r * 218ULL + g * 732ULL + b * 74ULL) >> 10);
}

// ---- PNM ---------------------------------------------------------------------
bool pnm_token(const std::vector<uint8_t>& d, size_t& i, uint32_t& v)
{
    for (;;) {   // whitespace and comments
        while (i < d.size() && (d[i] == ' ' || d[i] == '\t' || d[i] == '\n' || d[i] == '\r')) ++i;
        if (i < d.size() && d[i] == '#') {
            while (i < d.size() && d[i] != '\n') ++i;
            continue;
        }
        break;
    }
    if (i >= d.size() || d[i] < '0' || d[i] > '9') return false;
    uint64_t x = 0;
    while (i < d.size() && d[i] >= '0' && d[i] <= '9') {
        x = x * 10 + (d[i] - '0');
        if (x > 0xFFFFFFFFull) return false;
        ++i;
    }
    v = (uint32_t)x;
    return true;
}

int decode_pnm(const std::vector<uint8_t>& d, decoded& out)
{
    const int type = d[1] - '0';
    size_t i = 2;
    uint32_t w = 0, h = 0, maxval = 0;
    if (!pnm_token(d, i, w) || !pnm_token(d, i, h) || !pnm_token(d, i, maxval))
        return io_fail(OPIV_ERR_ARG, "PNM: malformed header");
    if (i >= d.size()) return io_fail(OPIV_ERR_ARG, "PNM: no pixel data");
    ++i;   // the single whitespace byte that ends the header
    if (w == 0 || h == 0 || maxval == 0 || maxval > 65535)
        return io_fail(OPIV_ERR_ARG, "PNM: invalid size or maxval");
    const int spp = type == 5 ? 1 : 3;
    const int bps = maxval > 255 ? 2 : 1;
    const size_t need = (size_t)w * h * spp * bps;
    if (d.size() - i < need) return io_fail(OPIV_ERR_ARG, "PNM: truncated pixel data");
    out.w = w;
    out.h = h;
    out.bits = bps * 8;
    out.px.resize((size_t)w * h);
    const uint8_t* p = d.data() + i;
    for (size_t k = 0; k < (size_t)w * h; ++k) {
        uint32_t s[3];
        for (int c = 0; c < spp; ++c) {
            s[c] = bps == 2 ? ((uint32_t)p[0] << 8) | p[1] : p[0];
            p += bps;
        }
        out.px[k] = spp == 1 ? (uint16_t)s[0] : grey_from_rgb(s[0], s[1], s[2]);
    }
    return OPIV_OK;
}

// ---- TIFF --------------------------------------------------------------------
struct tiff_reader {
    const std::vector<uint8_t>& d;
    bool le;
    uint16_t u16(size_t o) const
    {
        return le ? (uint16_t)(d[o] | (d[o + 1] << 8)) : (uint16_t)((d[o] << 8) | d[o + 1]);
    }
    uint32_t u32(size_t o) const
    {
        return le ? (uint32_t)d[o] | ((uint32_t)d[o + 1] << 8) | ((uint32_t)d[o + 2] << 16) |
                        ((uint32_t)d[o + 3] << 24)
                  : ((uint32_t)d[o] << 24) | ((uint32_t)d[o + 1] << 16) |
                        ((uint32_t)d[o + 2] << 8) | (uint32_t)d[o + 3];
    }
};

int decode_tiff(const std::vector<uint8_t>& d, decoded& out)
{
    tiff_reader r{ d, d[0] == 'I' };
    if (d.size() < 8 || r.u16(2) != 42) return io_fail(OPIV_ERR_ARG, "TIFF: not a classic TIFF file");
    const size_t ifd = r.u32(4);
    if (ifd + 2 > d.size()) return io_fail(OPIV_ERR_ARG, "TIFF: bad IFD offset");
    const uint16_t n = r.u16(ifd);
    if (ifd + 2 + 12 * (size_t)n > d.size()) return io_fail(OPIV_ERR_ARG, "TIFF: truncated IFD");
    uint32_t w = 0, h = 0, compression = 1, photometric = 1, planar = 1, rows_per_strip = 0;
    uint32_t spp = 1, bps = 8, sample_format = 1;
    std::vector<uint32_t> offsets, counts;
    auto values = [&](size_t e, std::vector<uint32_t>& dst) -> bool {
        const uint16_t type = r.u16(e + 2);
        const uint32_t count = r.u32(e + 4);
        const size_t size = type == 3 ? 2 : type == 4 ? 4 : 0;
        if (size == 0 || count == 0) return false;
        size_t at = e + 8;
        if (size * count > 4) at = r.u32(e + 8);
        if (at + size * count > d.size()) return false;
        dst.resize(count);
        for (uint32_t k = 0; k < count; ++k) dst[k] = size == 2 ? r.u16(at + 2 * k) : r.u32(at + 4 * k);
        return true;
    };
    for (uint16_t k = 0; k < n; ++k) {
        const size_t e = ifd + 2 + 12 * (size_t)k;
        const uint16_t tag = r.u16(e);
        std::vector<uint32_t> v;
        if (!values(e, v)) continue;
        switch (tag) {
        case 256: w = v[0]; break;
        case 257: h = v[0]; break;
        case 258: bps = v[0]; for (uint32_t b : v) if (b != v[0]) bps = 0; break;
        case 259: compression = v[0]; break;
        case 262: photometric = v[0]; break;
        case 273: offsets = v; break;
        case 277: spp = v[0]; break;
        case 278: rows_per_strip = v[0]; break;
        case 279: counts = v; break;
        case 284: planar = v[0]; break;
        case 339: sample_format = v[0]; break;
        default: break;
        }
    }
    if (compression != 1)
        return io_fail(OPIV_ERR_UNSUPPORTED, "TIFF: compression %u is not supported (uncompressed only)",
                       compression);
    if (w == 0 || h == 0 || offsets.empty()) return io_fail(OPIV_ERR_ARG, "TIFF: missing size or strips");
    if ((spp != 1 && spp != 3) || (bps != 8 && bps != 16) || sample_format != 1 ||
        (spp == 3 && planar != 1))
        return io_fail(OPIV_ERR_UNSUPPORTED,
                       "TIFF: %u samples of %u bits (format %u, planar %u) not supported", spp, bps,
                       sample_format, planar);
    if (rows_per_strip == 0 || rows_per_strip > h) rows_per_strip = h;
    const size_t bpp = spp * (bps / 8);
    const size_t row_bytes = (size_t)w * bpp;
    out.w = w;
    out.h = h;
    out.bits = (int)bps;
    out.px.resize((size_t)w * h);
    for (uint32_t y = 0; y < h; ++y) {
        const uint32_t strip = y / rows_per_strip;
        if (strip >= offsets.size()) return io_fail(OPIV_ERR_ARG, "TIFF: missing strip %u", strip);
        const size_t at = (size_t)offsets[strip] + (size_t)(y % rows_per_strip) * row_bytes;
        if (at + row_bytes > d.size()) return io_fail(OPIV_ERR_ARG, "TIFF: truncated strip %u", strip);
        for (uint32_t x = 0; x < w; ++x) {
            const size_t o = at + x * bpp;
            uint32_t s[3];
            for (uint32_t c = 0; c < spp; ++c)
                s[c] = bps == 16 ? r.u16(o + 2 * c) : d[o + c];
            uint16_t g = spp == 1 ? (uint16_t)s[0] : grey_from_rgb(s[0], s[1], s[2]);
            if (spp == 1 && photometric == 0) g = (uint16_t)((bps == 16 ? 65535u : 255u) - g);
            out.px[(size_t)y * w + x] = g;
        }
    }
    return OPIV_OK;
}

int decode(const char* path, decoded& out)
{
    std::vector<uint8_t> d;
    if (!path || !read_file(path, d)) return io_fail(OPIV_ERR_ARG, "failed to open %s", path ? path : "(null)");
    if (d.size() >= 2 && d[0] == 'P' && (d[1] == '5' || d[1] == '6')) return decode_pnm(d, out);
    if (d.size() >= 4 && ((d[0] == 'I' && d[1] == 'I') || (d[0] == 'M' && d[1] == 'M')))
        return decode_tiff(d, out);
    return io_fail(OPIV_ERR_UNSUPPORTED, "failed to find loader for %s", path);
}

}  // namespace

extern "C" {

int opiv_image_info(const char* path, uint32_t* width, uint32_t* height, int* dtype)
{
    if (!width || !height || !dtype) return io_fail(OPIV_ERR_ARG, "null argument");
    decoded im;
    const int rc = decode(path, im);
    if (rc != OPIV_OK) return rc;
    *width = im.w;
    *height = im.h;
    *dtype = im.bits == 16 ? OPIV_U16 : OPIV_U8;
    return OPIV_OK;
}

int opiv_image_load(const char* path, void* out, size_t pitch_bytes, uint32_t width, uint32_t height,
                    int dtype)
{
    if (!out) return io_fail(OPIV_ERR_ARG, "null argument");
    if (dtype != OPIV_U8 && dtype != OPIV_U16) return io_fail(OPIV_ERR_ARG, "pixel type must be u8 or u16");
    decoded im;
    const int rc = decode(path, im);
    if (rc != OPIV_OK) return rc;
    if (im.w != width || im.h != height)
        return io_fail(OPIV_ERR_SIZE_MISMATCH, "image size is different from expected: [%u, %u], [%u, %u]",
                       im.w, im.h, width, height);
    const size_t px = dtype == OPIV_U16 ? 2 : 1;
    if (pitch_bytes < (size_t)width * px) return io_fail(OPIV_ERR_ARG, "pitch smaller than a row");
    for (uint32_t y = 0; y < height; ++y) {
        uint8_t* row = static_cast<uint8_t*>(out) + (size_t)y * pitch_bytes;
        for (uint32_t x = 0; x < width; ++x) {
            const uint16_t g = im.px[(size_t)y * width + x];
            if (dtype == OPIV_U16) {
                std::memcpy(row + 2 * x, &g, 2);
            } else {
                if (g > 255) return io_fail(OPIV_ERR_ARG, "16-bit samples do not fit u8");
                row[x] = (uint8_t)g;
            }
        }
    }
    return OPIV_OK;
}

int opiv_vectors_write(const char* path, const opiv_vector* v, int64_t n)
{
    if (!v || n < 0) return io_fail(OPIV_ERR_ARG, "null argument");
    FILE* f = (path == nullptr || std::strcmp(path, "-") == 0) ? stdout : std::fopen(path, "w");
    if (!f) return io_fail(OPIV_ERR_ARG, "failed to open %s: %s", path, std::strerror(errno));
    for (int64_t k = 0; k < n; ++k)
        std::fprintf(f, "%g, %g, %g, %g, %g\n", (double)v[k].x, (double)v[k].y, (double)v[k].u,
                     (double)v[k].v, (double)v[k].sn);
    const bool ok = std::ferror(f) == 0;
    if (f != stdout) std::fclose(f);
    else std::fflush(f);
    return ok ? OPIV_OK : io_fail(OPIV_ERR_ARG, "write failed");
}

}  // extern "C"
