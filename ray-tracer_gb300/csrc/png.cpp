// Minimal PNG writer (RGBA8, stored deflate blocks, own CRC-32 and Adler-32) for headless frames.
// The reference displayed frames through a GL pixel buffer object (PixelBuffer.cpp:41,67); here a frame
// lands in a device buffer and can be written to disk.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/rsh.h"

namespace {

uint32_t crc_table[256];
bool crc_ready = false;

void crc_init() {
    for (uint32_t n = 0; n < 256; ++n) {
        uint32_t c = n;
        for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
        crc_table[n] = c;
    }
    crc_ready = true;
}

uint32_t crc32(const unsigned char* p, size_t n, uint32_t c = 0xFFFFFFFFu) {
    for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return c;
}

void put32(std::vector<unsigned char>& v, uint32_t x) {
    v.push_back((unsigned char)(x >> 24));
    v.push_back((unsigned char)(x >> 16));
    v.push_back((unsigned char)(x >> 8));
    v.push_back((unsigned char)x);
}

void chunk(std::FILE* f, const char* type, const std::vector<unsigned char>& data) {
    std::vector<unsigned char> buf;
    put32(buf, (uint32_t)data.size());
    buf.insert(buf.end(), type, type + 4);
    buf.insert(buf.end(), data.begin(), data.end());
    const uint32_t c = crc32(buf.data() + 4, buf.size() - 4) ^ 0xFFFFFFFFu;
    put32(buf, c);
    std::fwrite(buf.data(), 1, buf.size(), f);
}

}  // namespace

extern "C" rsh_status rsh_write_png(const char* path, const uint32_t* rgba, uint32_t w, uint32_t h) {
    if (!path || !rgba || w == 0 || h == 0) return RSH_ERR_INVALID;
    if (!crc_ready) crc_init();
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return RSH_ERR_INVALID;
    const unsigned char sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    std::fwrite(sig, 1, 8, f);
    std::vector<unsigned char> ihdr;
    put32(ihdr, w);
    put32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit RGBA
    chunk(f, "IHDR", ihdr);
    // raw scanlines, top row = image row h-1 (the engine's y grows upwards)
    std::vector<unsigned char> raw;
    raw.reserve((size_t)h * (4ull * w + 1));
    for (uint32_t yy = 0; yy < h; ++yy) {
        const uint32_t y = h - 1 - yy;
        raw.push_back(0);
        for (uint32_t x = 0; x < w; ++x) {
            const uint32_t p = rgba[(size_t)y * w + x];
            raw.push_back((unsigned char)(p & 0xFF));
            raw.push_back((unsigned char)((p >> 8) & 0xFF));
            raw.push_back((unsigned char)((p >> 16) & 0xFF));
            raw.push_back((unsigned char)((p >> 24) & 0xFF));
        }
    }
    std::vector<unsigned char> z = {0x78, 0x01};
    uint32_t a = 1, b = 0;
    for (unsigned char c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    size_t pos = 0;
    do {
        const size_t len = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((unsigned char)(len & 0xFF));
        z.push_back((unsigned char)(len >> 8));
        z.push_back((unsigned char)(~len & 0xFF));
        z.push_back((unsigned char)((~len >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
        pos += len;
    } while (pos < raw.size());
    put32(z, (b << 16) | a);
    chunk(f, "IDAT", z);
    chunk(f, "IEND", {});
    std::fclose(f);
    return RSH_OK;
}
