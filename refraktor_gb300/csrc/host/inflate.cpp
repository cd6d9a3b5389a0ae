#include "inflate.h"

#include "value.h"

namespace rfk {

std::vector<uint8_t> base64_decode(const std::string& text) {
    auto val = [](char c) -> int {
        if (c >= 'A' && c <= 'Z') return c - 'A';
        if (c >= 'a' && c <= 'z') return c - 'a' + 26;
        if (c >= '0' && c <= '9') return c - '0' + 52;
        if (c == '+' || c == '-') return 62;
        if (c == '/' || c == '_') return 63;
        return -1;
    };
    std::vector<uint8_t> out;
    uint32_t acc = 0;
    int bits = 0;
    for (char c : text) {
        if (c == '=') break;
        int v = val(c);
        if (v < 0) continue;  // whitespace and line breaks
        acc = (acc << 6) | (uint32_t)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((uint8_t)((acc >> bits) & 0xFF));
        }
    }
    return out;
}

namespace {

struct bit_reader {
    const std::vector<uint8_t>& d;
    size_t pos;
    uint32_t buf = 0;
    int cnt = 0;
    uint32_t bits(int n) {
        while (cnt < n) {
            if (pos >= d.size()) throw format_error("zlib: truncated stream");
            buf |= (uint32_t)d[pos++] << cnt;
            cnt += 8;
        }
        uint32_t v = buf & ((n == 32) ? 0xFFFFFFFFu : ((1u << n) - 1));
        buf >>= n;
        cnt -= n;
        return v;
    }
    void align() {
        buf = 0;
        cnt = 0;
    }
};

// Canonical Huffman decoding table (RFC 1951 section 3.2.2).
struct huffman {
    std::vector<uint16_t> count, symbol;
    void build(const uint8_t* lengths, int n) {
        count.assign(16, 0);
        symbol.assign(n, 0);
        for (int i = 0; i < n; i++) count[lengths[i]]++;
        count[0] = 0;
        std::vector<uint16_t> offs(16, 0);
        for (int i = 1; i < 16; i++) offs[i] = offs[i - 1] + count[i - 1];
        for (int i = 0; i < n; i++)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
    }
    int decode(bit_reader& br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++) {
            code |= (int)br.bits(1);
            int c = count[len];
            if (code - c < first) return symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
        }
        throw format_error("zlib: bad Huffman code");
    }
};

const uint16_t kLenBase[] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint16_t kLenExtra[] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint16_t kDistExtra[] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void inflate_block(bit_reader& br, std::vector<uint8_t>& out, const huffman& lit, const huffman& dist) {
    for (;;) {
        int sym = lit.decode(br);
        if (sym < 256) {
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return;
        } else {
            sym -= 257;
            if (sym >= 29) throw format_error("zlib: bad length symbol");
            size_t len = kLenBase[sym] + br.bits(kLenExtra[sym]);
            int ds = dist.decode(br);
            if (ds >= 30) throw format_error("zlib: bad distance symbol");
            size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
            if (d > out.size()) throw format_error("zlib: distance too far back");
            size_t from = out.size() - d;
            for (size_t i = 0; i < len; i++) out.push_back(out[from + i]);
        }
    }
}

}  // namespace

std::vector<uint8_t> zlib_uncompress(const std::vector<uint8_t>& data) {
    if (data.size() < 2) throw format_error("zlib: stream too short");
    uint8_t cmf = data[0], flg = data[1];
    if ((cmf & 0x0F) != 8 || ((cmf << 8) | flg) % 31 != 0) throw format_error("zlib: bad header");
    if (flg & 0x20) throw format_error("zlib: preset dictionary not supported");
    return inflate_raw(data, 2);
}

std::vector<uint8_t> inflate_raw(const std::vector<uint8_t>& data, size_t start) {
    if (start >= data.size()) throw format_error("deflate: stream too short");
    bit_reader br{data, start};
    std::vector<uint8_t> out;
    int final_block = 0;
    do {
        final_block = (int)br.bits(1);
        int type = (int)br.bits(2);
        if (type == 0) {
            br.align();
            if (br.pos + 4 > data.size()) throw format_error("zlib: truncated stored block");
            uint16_t len = data[br.pos] | (data[br.pos + 1] << 8);
            br.pos += 4;
            if (br.pos + len > data.size()) throw format_error("zlib: truncated stored block");
            out.insert(out.end(), data.begin() + br.pos, data.begin() + br.pos + len);
            br.pos += len;
        } else if (type == 1) {
            uint8_t l[288], d[30];
            for (int i = 0; i < 144; i++) l[i] = 8;
            for (int i = 144; i < 256; i++) l[i] = 9;
            for (int i = 256; i < 280; i++) l[i] = 7;
            for (int i = 280; i < 288; i++) l[i] = 8;
            for (int i = 0; i < 30; i++) d[i] = 5;
            huffman lit, dist;
            lit.build(l, 288);
            dist.build(d, 30);
            inflate_block(br, out, lit, dist);
        } else if (type == 2) {
            int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
            static const int order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; i++) cl[order[i]] = (uint8_t)br.bits(3);
            huffman clh;
            clh.build(cl, 19);
            uint8_t lens[320] = {0};
            int n = 0;
            while (n < hlit + hdist) {
                int sym = clh.decode(br);
                if (sym < 16) {
                    lens[n++] = (uint8_t)sym;
                } else {
                    int rep = 0;
                    uint8_t v = 0;
                    if (sym == 16) {
                        if (n == 0) throw format_error("zlib: repeat with no previous length");
                        v = lens[n - 1];
                        rep = 3 + (int)br.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)br.bits(3);
                    } else {
                        rep = 11 + (int)br.bits(7);
                    }
                    if (n + rep > hlit + hdist) throw format_error("zlib: too many lengths");
                    while (rep--) lens[n++] = v;
                }
            }
            huffman lit, dist;
            lit.build(lens, hlit);
            dist.build(lens + hlit, hdist);
            inflate_block(br, out, lit, dist);
        } else {
            throw format_error("zlib: bad block type");
        }
    } while (!final_block);
    return out;
}

}  // namespace rfk
