// Image.cpp -- minimal PNG writer: 8-bit RGBA, filter 0 on every row, zlib
// stream of stored (uncompressed) deflate blocks (RFC 1950/1951, PNG spec 1.2).
#include "Image.hpp"

#include <array>
#include <fstream>
#include <stdexcept>

namespace {

uint32_t crc32(const uint8_t *data, size_t n, uint32_t crc = 0xffffffffu)
{
    static const std::array<uint32_t, 256> table = [] {
        std::array<uint32_t, 256> t{};
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xedb88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
        return t;
    }();
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ data[i]) & 0xff] ^ (crc >> 8);
    return crc;
}

void put32(std::vector<uint8_t> &o, uint32_t v)
{
    o.push_back((uint8_t)(v >> 24));
    o.push_back((uint8_t)(v >> 16));
    o.push_back((uint8_t)(v >> 8));
    o.push_back((uint8_t)v);
}

void chunk(std::ofstream &f, const char type[4], const std::vector<uint8_t> &data)
{
    std::vector<uint8_t> buf;
    put32(buf, (uint32_t)data.size());
    buf.insert(buf.end(), type, type + 4);
    buf.insert(buf.end(), data.begin(), data.end());
    const uint32_t crc = crc32(buf.data() + 4, buf.size() - 4) ^ 0xffffffffu;
    put32(buf, crc);
    f.write(reinterpret_cast<const char *>(buf.data()), (std::streamsize)buf.size());
}

}  // namespace

void savePNG(const std::string &path, const std::vector<uint32_t> &pixels, Size2i size)
{
    if (size.width <= 0 || size.height <= 0 || pixels.size() < (size_t)size.area())
        throw std::runtime_error("savePNG: bad image size");
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("savePNG: cannot open " + path);
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    f.write(reinterpret_cast<const char *>(sig), 8);

    std::vector<uint8_t> ihdr;
    put32(ihdr, (uint32_t)size.width);
    put32(ihdr, (uint32_t)size.height);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8 bits, RGBA, deflate, filter 0, no interlace
    chunk(f, "IHDR", ihdr);

    std::vector<uint8_t> raw;
    raw.reserve((size_t)size.height * (1 + 4 * (size_t)size.width));
    for (int y = 0; y < size.height; ++y) {
        raw.push_back(0);
        for (int x = 0; x < size.width; ++x) {
            const uint32_t p = pixels[(size_t)y * size.width + x];
            raw.insert(raw.end(), {(uint8_t)p, (uint8_t)(p >> 8), (uint8_t)(p >> 16), (uint8_t)(p >> 24)});
        }
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    uint32_t a = 1, b = 0;  // Adler-32
    for (uint8_t v : raw) {
        a = (a + v) % 65521u;
        b = (b + a) % 65521u;
    }
    for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
        const size_t len = std::min<size_t>(65535, raw.size() - off);
        const bool last = off + len >= raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)len);
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)~len);
        z.push_back((uint8_t)(~len >> 8));
        z.insert(z.end(), raw.begin() + (std::ptrdiff_t)off, raw.begin() + (std::ptrdiff_t)(off + len));
        if (last) break;
    }
    put32(z, (b << 16) | a);
    chunk(f, "IDAT", z);
    chunk(f, "IEND", {});
}
