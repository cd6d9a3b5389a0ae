// Reader of the denoiser's weight files: the `params` array of a NumPy .npz
// archive (a zip file whose members are .npy arrays, stored or DEFLATE-
// compressed), as the Python side writes them, so that C and C++ callers can
// load a trained network without Python. Formats: the zip local file header
// (PKWARE APPNOTE 4.3.7), the .npy header (NumPy format versions 1-3), IEEE
// 754 binary16 / binary32 little-endian values.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../../include/rfk_denoise.h"
#include "inflate.h"
#include "runtime_internal.h"
#include "value.h"

using namespace rfk::rt;

namespace {

std::vector<uint8_t> read_all(const char* path) {
    FILE* f = std::fopen(path, "rb");
    if (!f) throw rfk::format_error(std::string("cannot open ") + path);
    std::vector<uint8_t> d;
    uint8_t buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) d.insert(d.end(), buf, buf + n);
    std::fclose(f);
    return d;
}

uint32_t le16(const std::vector<uint8_t>& d, size_t i) { return d[i] | (d[i + 1] << 8); }
uint32_t le32(const std::vector<uint8_t>& d, size_t i) {
    return d[i] | (d[i + 1] << 8) | (d[i + 2] << 16) | ((uint32_t)d[i + 3] << 24);
}

uint64_t le64(const std::vector<uint8_t>& d, size_t i) { return le32(d, i) | ((uint64_t)le32(d, i + 4) << 32); }

// The bytes of zip member `name` (the first local header with that name).
// Sizes of 0xFFFFFFFF are in the header's ZIP64 extra field (id 1: the
// uncompressed size, then the compressed size, each present only when its
// 32-bit field is 0xFFFFFFFF), as NumPy writes every member.
std::vector<uint8_t> zip_member(const std::vector<uint8_t>& z, const std::string& name) {
    size_t at = 0;
    while (at + 30 <= z.size() && le32(z, at) == 0x04034b50u) {
        const uint32_t flags = le16(z, at + 6), method = le16(z, at + 8);
        uint64_t csize = le32(z, at + 18);
        const uint32_t usize32 = le32(z, at + 22);
        const uint32_t nlen = le16(z, at + 26), xlen = le16(z, at + 28);
        if (at + 30 + nlen + xlen > z.size()) break;
        const std::string n(z.begin() + at + 30, z.begin() + at + 30 + nlen);
        const size_t data = at + 30 + nlen + xlen;
        if (csize == 0xFFFFFFFFu) {
            for (size_t e = at + 30 + nlen; e + 4 <= data;) {
                const uint32_t id = le16(z, e), len = le16(z, e + 2);
                if (e + 4 + len > data) break;
                if (id == 1) {
                    const size_t off = e + 4 + (usize32 == 0xFFFFFFFFu ? 8 : 0);
                    if (off + 8 <= e + 4 + len) csize = le64(z, off);
                    break;
                }
                e += 4 + len;
            }
        }
        const bool sized = csize != 0xFFFFFFFFu && !(flags & 8);
        if (n == name) {
            if (method == 8) return rfk::inflate_raw(z, data);  // self-terminating
            if (method == 0 && sized && csize <= z.size() - data)
                return std::vector<uint8_t>(z.begin() + data, z.begin() + data + (size_t)csize);
            throw rfk::format_error("npz: unsupported compression of " + name);
        }
        if (!sized) break;  // the next header's position is unknown
        at = data + (size_t)csize;
    }
    throw rfk::format_error("npz: no member " + name);
}

float half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h >> 15) << 31;
    const int exp = (h >> 10) & 0x1F;
    uint32_t man = h & 0x3FF;
    uint32_t bits;
    if (exp == 0x1F) {
        bits = sign | 0x7F800000u | (man << 13);  // inf / nan
    } else if (exp != 0) {
        bits = sign | ((uint32_t)(exp - 15 + 127) << 23) | (man << 13);
    } else if (man == 0) {
        bits = sign;
    } else {  // subnormal: normalise
        int e = -14;
        while (!(man & 0x400)) {
            man <<= 1;
            e--;
        }
        bits = sign | ((uint32_t)(e + 127) << 23) | ((man & 0x3FF) << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

// The values of a 1-D little-endian float16 / float32 .npy array as floats.
std::vector<float> npy_values(const std::vector<uint8_t>& a) {
    if (a.size() < 10 || std::memcmp(a.data(), "\x93NUMPY", 6) != 0) throw rfk::format_error("npy: bad magic");
    const int major = a[6];
    size_t hlen, hstart;
    if (major == 1) {
        hlen = le16(a, 8);
        hstart = 10;
    } else if (major == 2 || major == 3) {
        if (a.size() < 12) throw rfk::format_error("npy: truncated header");
        hlen = le32(a, 8);
        hstart = 12;
    } else {
        throw rfk::format_error("npy: unsupported version");
    }
    if (hstart + hlen > a.size()) throw rfk::format_error("npy: truncated header");
    const std::string hdr(a.begin() + hstart, a.begin() + hstart + hlen);
    size_t width = 0;
    if (hdr.find("'<f2'") != std::string::npos) width = 2;
    else if (hdr.find("'<f4'") != std::string::npos) width = 4;
    else throw rfk::format_error("npy: parameters must be little-endian float16 or float32");
    if (hdr.find("'fortran_order': False") == std::string::npos) throw rfk::format_error("npy: fortran order");
    const size_t sp = hdr.find("'shape': (");
    if (sp == std::string::npos) throw rfk::format_error("npy: no shape");
    size_t count = 1, dims = 0;
    for (size_t i = sp + 10; i < hdr.size() && hdr[i] != ')';) {
        if (hdr[i] >= '0' && hdr[i] <= '9') {
            size_t v = 0;
            while (i < hdr.size() && hdr[i] >= '0' && hdr[i] <= '9') v = v * 10 + (size_t)(hdr[i++] - '0');
            count *= v;
            dims++;
        } else {
            i++;
        }
    }
    if (dims != 1) throw rfk::format_error("npy: parameters must be a 1-D array");
    const size_t data = hstart + hlen;
    if (data + count * width > a.size()) throw rfk::format_error("npy: truncated data");
    std::vector<float> out(count);
    for (size_t i = 0; i < count; i++) {
        if (width == 2) {
            out[i] = half_to_float((uint16_t)le16(a, data + 2 * i));
        } else {
            const uint32_t b = le32(a, data + 4 * i);
            std::memcpy(&out[i], &b, 4);
        }
    }
    return out;
}

}  // namespace

rfk_status rfk_denoiser_read_params(const char* path, float* out, size_t cap, size_t* count) {
    return guard([&] {
        if (!path || !count) fail(RFK_E_INVALID, "null argument");
        const std::vector<float> v = npy_values(zip_member(read_all(path), "params.npy"));
        *count = v.size();
        if (!out) return;
        if (cap < v.size()) fail(RFK_E_INVALID, "output holds " + std::to_string(cap) + " of " + std::to_string(v.size()) + " parameters");
        std::memcpy(out, v.data(), v.size() * sizeof(float));
    });
}
