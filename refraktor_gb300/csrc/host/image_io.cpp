// PNG writer for headless artefacts (8-bit RGB / RGBA, no interlace): the
// image rows, each behind a filter byte 0, in a zlib stream of stored
// (uncompressed) DEFLATE blocks (RFC 1950 / 1951), CRC-32 per chunk
// (ISO 3309 polynomial 0xEDB88320) and Adler-32 over the raw data.
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "runtime_internal.h"

using namespace rfk::rt;

namespace {

uint32_t crc_table_entry(uint32_t c) {
    for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    return c;
}

uint32_t crc32(const uint8_t* p, size_t n, uint32_t crc = 0xFFFFFFFFu) {
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; i++) table[i] = crc_table_entry(i);
        init = true;
    }
    for (size_t i = 0; i < n; i++) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return crc;
}

void put32(std::vector<uint8_t>& o, uint32_t v) {
    o.push_back((uint8_t)(v >> 24));
    o.push_back((uint8_t)(v >> 16));
    o.push_back((uint8_t)(v >> 8));
    o.push_back((uint8_t)v);
}

void chunk(std::vector<uint8_t>& file, const char* type, const std::vector<uint8_t>& data) {
    put32(file, (uint32_t)data.size());
    std::vector<uint8_t> body(type, type + 4);
    body.insert(body.end(), data.begin(), data.end());
    file.insert(file.end(), body.begin(), body.end());
    put32(file, crc32(body.data(), body.size()) ^ 0xFFFFFFFFu);
}

}  // namespace

extern "C" rfk_status rfk_write_png(const char* path, const uint8_t* pixels, uint32_t w, uint32_t h, int channels) {
    return guard([&] {
        if (!path || !pixels) fail(RFK_E_INVALID, "null argument");
        if (w == 0 || h == 0 || (channels != 3 && channels != 4)) fail(RFK_E_INVALID, "bad image size or channels");
        const size_t row = (size_t)w * channels;
        std::vector<uint8_t> raw;
        raw.reserve((row + 1) * h);
        for (uint32_t y = 0; y < h; y++) {
            raw.push_back(0);
            raw.insert(raw.end(), pixels + y * row, pixels + (y + 1) * row);
        }
        std::vector<uint8_t> z = {0x78, 0x01};
        for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
            const size_t n = std::min<size_t>(65535, raw.size() - off);
            const bool last = off + n >= raw.size();
            z.push_back(last ? 1 : 0);
            z.push_back((uint8_t)(n & 0xFF));
            z.push_back((uint8_t)(n >> 8));
            z.push_back((uint8_t)(~n & 0xFF));
            z.push_back((uint8_t)((~n >> 8) & 0xFF));
            z.insert(z.end(), raw.begin() + off, raw.begin() + off + n);
            if (last) break;
        }
        uint32_t a = 1, b = 0;
        for (uint8_t v : raw) {
            a = (a + v) % 65521u;
            b = (b + a) % 65521u;
        }
        put32(z, (b << 16) | a);
        std::vector<uint8_t> file = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
        std::vector<uint8_t> ihdr;
        put32(ihdr, w);
        put32(ihdr, h);
        ihdr.push_back(8);
        ihdr.push_back(channels == 4 ? 6 : 2);
        ihdr.push_back(0);
        ihdr.push_back(0);
        ihdr.push_back(0);
        chunk(file, "IHDR", ihdr);
        chunk(file, "IDAT", z);
        chunk(file, "IEND", {});
        FILE* f = std::fopen(path, "wb");
        if (!f) fail(RFK_E_INVALID, std::string("cannot open ") + path);
        const size_t wrote = std::fwrite(file.data(), 1, file.size(), f);
        std::fclose(f);
        if (wrote != file.size()) fail(RFK_E_INVALID, std::string("short write to ") + path);
    });
}
