// PNG file writer for ffr-img's output (the reference writes PNG through
// Boost.GIL + libpng, writePng, src/utils/image.cpp:9-16; neither library is
// a dependency here).
//
// The file is the PNG signature, IHDR (8/16-bit gray or RGB, no interlace),
// one IDAT and IEND.  IDAT holds a zlib stream of uncompressed ("stored")
// deflate blocks of at most 65535 bytes each, followed by the Adler-32 of
// the raw image data; every scan line starts with filter byte 0 (none), and
// 16-bit samples are written big-endian as PNG requires.  Chunk CRCs are
// the CRC-32 of ISO 3309 (polynomial 0xEDB88320, reflected).
#include "ffr_gpu.h"

#include <cstring>
#include <string>
#include <vector>

namespace {

uint32_t crc_table_entry(uint32_t n)
{
    uint32_t c = n;
    for (int k = 0; k < 8; ++k)
        c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    return c;
}

struct Crc32
{
    uint32_t table[256];
    Crc32()
    {
        for (uint32_t n = 0; n < 256; ++n)
            table[n] = crc_table_entry(n);
    }
    uint32_t update(uint32_t crc, const unsigned char* p, size_t n) const
    {
        uint32_t c = crc ^ 0xFFFFFFFFu;
        for (size_t i = 0; i < n; ++i)
            c = table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
        return c ^ 0xFFFFFFFFu;
    }
};

void put32(std::vector<unsigned char>& o, uint32_t v)
{
    o.push_back((unsigned char)(v >> 24));
    o.push_back((unsigned char)(v >> 16));
    o.push_back((unsigned char)(v >> 8));
    o.push_back((unsigned char)v);
}

void chunk(std::vector<unsigned char>& o, const Crc32& crc, const char* type,
           const std::vector<unsigned char>& data)
{
    put32(o, (uint32_t)data.size());
    const size_t start = o.size();
    o.insert(o.end(), type, type + 4);
    o.insert(o.end(), data.begin(), data.end());
    put32(o, crc.update(0, o.data() + start, o.size() - start));
}

} // namespace

extern "C" ffr_status ffr_encode_png(const void* pixels, uint32_t width, uint32_t height,
                                     uint32_t channels, uint32_t bits, void* out, size_t cap,
                                     size_t* len)
{
    if (!pixels || !len || width == 0 || height == 0 || (channels != 1 && channels != 3)
            || (bits != 8 && bits != 16))
        return FFR_ERR_ARG;
    const size_t bpp = (size_t)channels * (bits / 8);
    const size_t row = (size_t)width * bpp;
    const size_t raw_bytes = (row + 1) * height;
    const size_t nblocks = (raw_bytes + 65534) / 65535;      // raw_bytes > 0
    const size_t idat = 2 + raw_bytes + 5 * nblocks + 4;
    const size_t total = 8 + (12 + 13) + (12 + idat) + 12;
    *len = total;
    if (!out || cap < total)
        return FFR_ERR_IO;

    // scan lines: filter 0, samples big-endian
    std::vector<unsigned char> raw(raw_bytes);
    const unsigned char* src = static_cast<const unsigned char*>(pixels);
    for (uint32_t y = 0; y < height; ++y)
    {
        unsigned char* d = raw.data() + (size_t)y * (row + 1);
        d[0] = 0;
        const unsigned char* s = src + (size_t)y * row;
        if (bits == 8)
            std::memcpy(d + 1, s, row);
        else
            for (size_t k = 0; k < row; k += 2)
            {
                uint16_t v;
                std::memcpy(&v, s + k, 2);
                d[1 + k] = (unsigned char)(v >> 8);
                d[2 + k] = (unsigned char)v;
            }
    }
    // zlib stream: header (deflate, 32K window, check bits), stored blocks
    std::vector<unsigned char> z;
    z.reserve(idat);
    z.push_back(0x78);
    z.push_back(0x01);
    size_t pos = 0;
    do
    {
        const size_t n = raw_bytes - pos < 65535 ? raw_bytes - pos : 65535;
        const bool last = pos + n == raw_bytes;
        z.push_back(last ? 1 : 0);
        z.push_back((unsigned char)n);
        z.push_back((unsigned char)(n >> 8));
        z.push_back((unsigned char)~n);
        z.push_back((unsigned char)(~n >> 8));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
        pos += n;
    } while (pos < raw_bytes);
    uint32_t a = 1, b = 0;          // Adler-32
    for (size_t i = 0; i < raw_bytes; ++i)
    {
        a = (a + raw[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    put32(z, (b << 16) | a);

    static const Crc32 crc;
    std::vector<unsigned char> f;
    f.reserve(total);
    static const unsigned char sig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    f.insert(f.end(), sig, sig + 8);
    std::vector<unsigned char> ihdr;
    put32(ihdr, width);
    put32(ihdr, height);
    ihdr.push_back((unsigned char)bits);
    ihdr.push_back(channels == 3 ? 2 : 0);      // colour type: RGB or gray
    ihdr.push_back(0);                          // deflate
    ihdr.push_back(0);                          // adaptive filtering
    ihdr.push_back(0);                          // no interlace
    chunk(f, crc, "IHDR", ihdr);
    chunk(f, crc, "IDAT", z);
    chunk(f, crc, "IEND", {});
    if (f.size() != total)
        return FFR_ERR_STATE;
    std::memcpy(out, f.data(), total);
    return FFR_OK;
}
