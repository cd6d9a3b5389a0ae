// zlib (RFC 1950) / DEFLATE (RFC 1951) decoder and base64 decoder.
//
// The reference stores genome palettes as base64 text of a zlib stream
// (src/librefrakt/src/flame_types.cpp:429-432, 471-482). zlib itself is not
// available to this library, so the decoder is written here from the RFCs.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace rfk {

std::vector<uint8_t> base64_decode(const std::string& text);
std::vector<uint8_t> zlib_uncompress(const std::vector<uint8_t>& data);
// A raw DEFLATE stream starting at data[start] (self-terminating: its last block
// is marked), as stored in zip members.
std::vector<uint8_t> inflate_raw(const std::vector<uint8_t>& data, size_t start);

}  // namespace rfk
