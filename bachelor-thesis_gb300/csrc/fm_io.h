// Host-side particle-file input: gzip / DEFLATE decoding and the classic BGEO
// layout.  Plain C++ (no CUDA types), shared by inflate.cpp and bgeo.cu.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace fm {
namespace io {

// CRC-32 of RFC 1952 (reflected polynomial 0xEDB88320), continuing from `crc`.
uint32_t crc32(const uint8_t* p, size_t n, uint32_t crc = 0);

bool is_gzip(const uint8_t* p, size_t n);

// Raw DEFLATE stream (RFC 1951) from in[0, n): appends to out.  consumed =
// bytes of the stream (through the final block).  stop_after > 0: return as
// soon as out holds at least that many bytes (a partial decode; consumed is
// then not meaningful).  0 on success, -1 with err set.
int inflate_raw(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t* consumed, size_t stop_after,
                std::string& err);

// First gzip member (RFC 1952) of in[0, n) into out; CRC-32 and length are
// checked unless stop_after > 0 (a prefix of the data only).
int gunzip(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t stop_after, std::string& err);

// Classic BGEO (version 5) point layout, as Partio reads it
// (vendor/partio/src/io/BGEO.cpp readBGEO): a big-endian header, point
// attribute definitions, then one record of `words` 32-bit big-endian words
// per point, the first four x y z w.
struct BgeoLayout {
    uint64_t points = 0;
    uint32_t words = 4;       // per point record
    uint32_t attributes = 0;  // point attributes besides position
    size_t data_offset = 0;   // byte offset of the first point record
};

// Parses the header and attribute definitions from the first n bytes of the
// decompressed file.  need_points: also require the whole point block.
// 0 on success, 1 when more bytes are needed for the header, -1 on error.
int bgeo_layout(const uint8_t* d, size_t n, bool need_points, BgeoLayout& L, std::string& err);

// Whole file into `raw`; decompressed (gzip detected by its magic, as
// Partio's reader does) into `data` (which is `raw` itself for a plain file:
// data then aliases raw's storage).  header_only: decompress just enough for
// the header.
struct BgeoFile {
    std::vector<uint8_t> raw, inflated;
    const uint8_t* data = nullptr;
    size_t size = 0;
    bool compressed = false;
    uint64_t file_bytes = 0;
    BgeoLayout layout;
};
int bgeo_load(const char* path, bool header_only, BgeoFile& f, std::string& err);

// Positions (3 floats per point) of the first `count` points, byte-swapped.
void bgeo_positions(const BgeoFile& f, float* xyz, uint64_t count);

}  // namespace io
}  // namespace fm
