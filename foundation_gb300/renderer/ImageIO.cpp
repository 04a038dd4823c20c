// ImageIO.cpp — PFM and PNG writers (see ImageIO.hpp).
//
// PNG layout: signature, IHDR (8-bit RGBA, colour type 6), one IDAT holding a
// zlib stream (RFC 1950) of stored deflate blocks (RFC 1951, BTYPE 00, at
// most 65,535 bytes each) over the scanlines, each prefixed by filter byte 0,
// then IEND. Chunk CRCs are CRC-32 (polynomial 0xEDB88320, reflected); the
// zlib trailer is the Adler-32 of the uncompressed scanlines.
#include "ImageIO.hpp"

#include <array>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "FoundationCore.hpp"

namespace Foundation {
namespace Renderer {
namespace {

const std::array<uint32_t, 256>& CrcTable() {
    static const std::array<uint32_t, 256> table = [] {
        std::array<uint32_t, 256> t{};
        for (uint32_t n = 0; n < 256; ++n) {
            uint32_t c = n;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[n] = c;
        }
        return t;
    }();
    return table;
}

uint32_t Crc32(const uint8_t* p, size_t n, uint32_t crc = 0xFFFFFFFFu) {
    const auto& t = CrcTable();
    for (size_t i = 0; i < n; ++i) crc = t[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return crc;
}

void Put32(std::vector<uint8_t>& v, uint32_t x) {
    for (int s = 24; s >= 0; s -= 8) v.push_back((uint8_t)(x >> s));
}

void Chunk(std::FILE* f, const char type[4], const std::vector<uint8_t>& data) {
    std::vector<uint8_t> head;
    Put32(head, (uint32_t)data.size());
    std::vector<uint8_t> body(type, type + 4);
    body.insert(body.end(), data.begin(), data.end());
    std::vector<uint8_t> tail;
    Put32(tail, Crc32(body.data(), body.size()) ^ 0xFFFFFFFFu);
    std::fwrite(head.data(), 1, head.size(), f);
    std::fwrite(body.data(), 1, body.size(), f);
    std::fwrite(tail.data(), 1, tail.size(), f);
}

}  // namespace

void WritePfm(const char* path, std::span<const float> rgb, uint32_t w, uint32_t h) {
    CHECK(rgb.size() >= 3ull * w * h);
    std::FILE* f = std::fopen(path, "wb");
    if (f == nullptr) throw std::runtime_error(std::string("cannot write ") + path);
    std::fprintf(f, "PF\n%u %u\n-1.0\n", w, h);
    bool ok = true;
    for (uint32_t y = 0; y < h; ++y)  // PFM rows run bottom to top
        ok = ok && std::fwrite(&rgb[3 * (size_t)(h - 1 - y) * w], sizeof(float), 3 * (size_t)w, f) == 3 * (size_t)w;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) throw std::runtime_error(std::string("write to ") + path + " failed");
}

void WritePng(const char* path, std::span<const uint8_t> rgba, uint32_t w, uint32_t h) {
    CHECK(w > 0 && h > 0 && rgba.size() >= 4ull * w * h);
    const size_t row = 1 + 4 * (size_t)w;
    std::vector<uint8_t> raw(row * h);
    for (uint32_t y = 0; y < h; ++y) {
        raw[y * row] = 0;  // filter type 0 (None)
        std::copy(rgba.begin() + 4 * (size_t)y * w, rgba.begin() + 4 * (size_t)(y + 1) * w, raw.begin() + y * row + 1);
    }
    std::vector<uint8_t> z = {0x78, 0x01};  // deflate, 32K window, no dictionary
    for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
        const size_t n = std::min<size_t>(65535, raw.size() - off);
        const bool last = off + n >= raw.size();
        z.push_back(last ? 1 : 0);  // BFINAL, BTYPE 00
        z.push_back((uint8_t)(n & 0xFF));
        z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)(~n & 0xFF));
        z.push_back((uint8_t)((~n >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + n);
        if (last) break;
    }
    uint32_t a = 1, b = 0;  // Adler-32
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    Put32(z, (b << 16) | a);
    std::vector<uint8_t> ihdr;
    Put32(ihdr, w);
    Put32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit, RGBA, deflate, filter method 0, no interlace
    std::FILE* f = std::fopen(path, "wb");
    if (f == nullptr) throw std::runtime_error(std::string("cannot write ") + path);
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::fwrite(sig, 1, 8, f);
    Chunk(f, "IHDR", ihdr);
    Chunk(f, "IDAT", z);
    Chunk(f, "IEND", {});
    if (std::fclose(f) != 0) throw std::runtime_error(std::string("write to ") + path + " failed");
}

}  // namespace Renderer
}  // namespace Foundation
