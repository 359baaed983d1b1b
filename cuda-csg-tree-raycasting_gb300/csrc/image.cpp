// Headless image export (csg_image_write in include/csgrt.h): an RGBA8 frame as binary
// PPM (RGB, alpha dropped) or PNG (RGBA, 8 bits per channel), the headless stand-in for
// the reference's OpenGL blit of its pixel buffer (RenderManager.cpp:69-84).
//
// The PNG is written without a compression library: its zlib stream holds "stored"
// (uncompressed) deflate blocks, which every decoder reads.  Row 0 of the frame is the
// top row of the picture, as in the reference's ray generation (ny = 1 - 2v).
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "csgrt.h"

namespace {

struct CrcTable {
    uint32_t v[256];
    CrcTable()
    {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            v[i] = c;
        }
    }
};

uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n)
{
    static const CrcTable t;  // initialised once, thread-safely
    const uint32_t* table = t.v;
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return ~crc;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x)
{
    v.push_back(uint8_t(x >> 24));
    v.push_back(uint8_t(x >> 16));
    v.push_back(uint8_t(x >> 8));
    v.push_back(uint8_t(x));
}

void put_chunk(std::vector<uint8_t>& out, const char type[4], const std::vector<uint8_t>& data)
{
    put_be32(out, (uint32_t)data.size());
    const size_t start = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    put_be32(out, crc32_update(0, out.data() + start, out.size() - start));
}

std::vector<uint8_t> encode_png(const uint32_t* rgba8, int32_t w, int32_t h)
{
    // filtered scanlines: a 0 (no filter) byte, then the row's RGBA bytes
    const size_t row = (size_t)w * 4 + 1;
    std::vector<uint8_t> raw(row * (size_t)h);
    for (int32_t y = 0; y < h; ++y) {
        uint8_t* r = raw.data() + row * (size_t)y;
        r[0] = 0;
        for (int32_t x = 0; x < w; ++x) {
            const uint32_t q = rgba8[(size_t)y * w + x];
            r[1 + 4 * x + 0] = uint8_t(q);
            r[1 + 4 * x + 1] = uint8_t(q >> 8);
            r[1 + 4 * x + 2] = uint8_t(q >> 16);
            r[1 + 4 * x + 3] = uint8_t(q >> 24);
        }
    }
    // zlib stream of stored deflate blocks
    std::vector<uint8_t> z;
    z.push_back(0x78);
    z.push_back(0x01);
    size_t pos = 0;
    do {
        const size_t n = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + n == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back(uint8_t(n));
        z.push_back(uint8_t(n >> 8));
        z.push_back(uint8_t(~n));
        z.push_back(uint8_t(~n >> 8));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
        pos += n;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;  // Adler-32 of the uncompressed bytes
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put_be32(z, (b << 16) | a);

    std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, (uint32_t)w);
    put_be32(ihdr, (uint32_t)h);
    ihdr.push_back(8);  // bits per channel
    ihdr.push_back(6);  // RGBA
    ihdr.push_back(0);  // deflate
    ihdr.push_back(0);  // adaptive filtering
    ihdr.push_back(0);  // no interlace
    put_chunk(out, "IHDR", ihdr);
    put_chunk(out, "IDAT", z);
    put_chunk(out, "IEND", {});
    return out;
}

std::vector<uint8_t> encode_ppm(const uint32_t* rgba8, int32_t w, int32_t h)
{
    char head[64];
    const int n = std::snprintf(head, sizeof(head), "P6\n%d %d\n255\n", w, h);
    std::vector<uint8_t> out(head, head + n);
    out.reserve(out.size() + (size_t)w * h * 3);
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        out.push_back(uint8_t(rgba8[i]));
        out.push_back(uint8_t(rgba8[i] >> 8));
        out.push_back(uint8_t(rgba8[i] >> 16));
    }
    return out;
}

}  // namespace

extern "C" int csg_image_write(const char* path, const uint32_t* rgba8, int32_t w, int32_t h, int32_t format)
{
    if (!path || !rgba8 || w <= 0 || h <= 0 || (int64_t)w * h > (1ll << 30)) return CSG_E_ARG;
    if (format != CSG_IMAGE_PPM && format != CSG_IMAGE_PNG) return CSG_E_ARG;
    const std::vector<uint8_t> bytes = format == CSG_IMAGE_PNG ? encode_png(rgba8, w, h) : encode_ppm(rgba8, w, h);
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return CSG_E_ARG;
    const size_t wrote = std::fwrite(bytes.data(), 1, bytes.size(), f);
    const int closed = std::fclose(f);
    return (wrote == bytes.size() && closed == 0) ? CSG_OK : CSG_E_ARG;
}
