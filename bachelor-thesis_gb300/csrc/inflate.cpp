// DEFLATE (RFC 1951) and gzip member (RFC 1952) decoding on the host, for
// the particle-file loader.
//
// The reference reads gzip-compressed BGEO files through Partio, which parses
// the gzip header itself and hands the DEFLATE stream to zlib's raw inflate
// (vendor/partio/src/io/ZIP.cpp: GZipFileHeader::Read, ZipStreambufDecompress).
// zlib is not part of this library: this is an independent decoder written
// from the two RFCs.  Huffman codes are canonical (RFC 1951 3.2.2); a 10-bit
// lookup table decodes short codes in one step and a bit-serial walk over the
// per-length code counts decodes the longer ones.
//
// Differences from Partio's path, all on inputs Partio mis-reads or does not
// check: the gzip flag bits are read as RFC 1952 defines them (FHCRC 2,
// FEXTRA 4, FNAME 8, FCOMMENT 16; Partio tests 2 for the extra field, 4 and 8
// for the two strings and 1 for the header CRC, which agrees for the flag
// values writers use, 0 and FNAME); the member's CRC-32 and length are
// checked; a truncated stream is an error.

#include <algorithm>
#include <cstring>

#include "fm_io.h"

namespace fm {
namespace io {

namespace {

// ---- CRC-32, slicing by 8 -------------------------------------------------

struct CrcTables {
    uint32_t t[8][256];
    CrcTables() {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? (0xEDB88320u ^ (c >> 1)) : (c >> 1);
            t[0][i] = c;
        }
        for (uint32_t i = 0; i < 256; ++i)
            for (int s = 1; s < 8; ++s) t[s][i] = (t[s - 1][i] >> 8) ^ t[0][t[s - 1][i] & 0xff];
    }
};

const CrcTables& crc_tables() {
    static const CrcTables tables;
    return tables;
}

// ---- bit input, least significant bit first ---------------------------------

struct BitIn {
    const uint8_t* start;
    const uint8_t* p;
    const uint8_t* end;
    uint64_t buf = 0;
    int cnt = 0;       // valid bits in buf
    size_t past = 0;   // zero bytes fed past the end

    BitIn(const uint8_t* s, size_t n) : start(s), p(s), end(s + n) {}

    // at least 57 valid bits afterwards
    void fill() {
        if (end - p >= 8) {
            uint64_t w = 0;
            for (int k = 7; k >= 0; --k) w = (w << 8) | p[k];
            buf |= w << cnt;  // bits above the whole bytes taken are loaded again later, unchanged
            const int take = (63 - cnt) >> 3;
            p += take;
            cnt += take * 8;
            return;
        }
        while (cnt <= 56) {
            uint64_t b = 0;
            if (p < end)
                b = *p++;
            else
                ++past;
            buf |= b << cnt;
            cnt += 8;
        }
    }
    uint32_t bits(int n) {  // n <= 32
        if (cnt < n) fill();
        const uint32_t v = (uint32_t)(buf & ((1ull << n) - 1));
        buf >>= n;
        cnt -= n;
        return v;
    }
    void drop(int n) {
        buf >>= n;
        cnt -= n;
    }
    // bits consumed so far
    uint64_t consumed_bits() const { return (uint64_t)(p - start + past) * 8 - (uint64_t)cnt; }
    bool truncated() const { return consumed_bits() > (uint64_t)(end - start) * 8; }
    // move to the next byte boundary and restart reading there
    void align_and_reset() {
        const uint64_t byte = (consumed_bits() + 7) / 8;
        p = start + (byte < (uint64_t)(end - start) ? byte : (uint64_t)(end - start));
        past = byte > (uint64_t)(end - start) ? byte - (uint64_t)(end - start) : 0;
        buf = 0;
        cnt = 0;
    }
};

// ---- canonical Huffman codes ----------------------------------------------

constexpr int kFast = 10;

struct Huff {
    uint16_t fast[1 << kFast];  // (symbol << 4) | length; 0: code longer than kFast bits or unassigned
    uint16_t count[16];         // codes of each length
    uint16_t sym[320];          // symbols in canonical code order

    // 0, or -1 for an over-subscribed set of lengths.  Incomplete sets are
    // accepted: their unassigned codes fail when met.
    int build(const uint8_t* len, int n) {
        std::memset(count, 0, sizeof(count));
        for (int i = 0; i < n; ++i) count[len[i]]++;
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; ++l) {
            left = (left << 1) - count[l];
            if (left < 0) return -1;
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; ++l) offs[l + 1] = (uint16_t)(offs[l] + count[l]);
        for (int i = 0; i < n; ++i)
            if (len[i]) sym[offs[len[i]]++] = (uint16_t)i;
        std::memset(fast, 0, sizeof(fast));
        uint32_t code = 0;
        int idx = 0;
        for (int l = 1; l < 16; ++l) {
            for (int j = 0; j < count[l]; ++j, ++code, ++idx) {
                if (l > kFast) continue;
                uint32_t rev = 0;  // codes are sent most significant bit first
                for (int b = 0; b < l; ++b) rev |= ((code >> b) & 1u) << (l - 1 - b);
                const uint16_t e = (uint16_t)((sym[idx] << 4) | l);
                for (uint32_t r = rev; r < (1u << kFast); r += 1u << l) fast[r] = e;
            }
            code <<= 1;
        }
        return 0;
    }

    int decode(BitIn& b) const {
        if (b.cnt < 15) b.fill();
        const uint16_t e = fast[b.buf & ((1u << kFast) - 1)];
        if (e) {
            b.drop(e & 15);
            return e >> 4;
        }
        // bit-serial: the first code of each length follows the last one of the
        // previous length, shifted left
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; ++l) {
            code |= (int)b.bits(1);
            const int c = count[l];
            if (code - first < c) return sym[index + code - first];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;
    }
};

// RFC 1951 3.2.5: length codes 257..285, distance codes 0..29
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// order of the code-length code lengths (RFC 1951 3.2.7)
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

struct Fixed {
    Huff lit, dist;
    Fixed() {
        uint8_t l[288];
        for (int i = 0; i < 144; ++i) l[i] = 8;
        for (int i = 144; i < 256; ++i) l[i] = 9;
        for (int i = 256; i < 280; ++i) l[i] = 7;
        for (int i = 280; i < 288; ++i) l[i] = 8;
        lit.build(l, 288);
        uint8_t d[30];
        for (int i = 0; i < 30; ++i) d[i] = 5;
        dist.build(d, 30);
    }
};

const Fixed& fixed_codes() {
    static const Fixed f;
    return f;
}

struct Out {
    std::vector<uint8_t>& v;
    size_t pos;
    explicit Out(std::vector<uint8_t>& vec) : v(vec), pos(vec.size()) {}
    void reserve(size_t extra) {
        if (pos + extra > v.size()) v.resize(std::max(pos + extra, v.size() * 2 + 4096));
    }
    void finish() { v.resize(pos); }
};

int fail(std::string& err, const char* msg) {
    err = msg;
    return -1;
}

int codes_block(BitIn& bin, const Huff& lit, const Huff& dist, Out& o, size_t base, std::string& err) {
    // The loop works on local copies of the bit reader and the output cursor:
    // a byte store into the output may alias any object in memory, so state
    // kept only in those structs would be reloaded after every literal.
    BitIn b = bin;
    uint8_t* out = o.v.data();
    size_t pos = o.pos, cap = o.v.size();
    int rc = 0;
    for (;;) {
        if (b.past > 8) {
            rc = fail(err, "deflate stream is truncated");
            break;
        }
        if (b.cnt < 48) b.fill();
        const int s = lit.decode(b);
        if (s < 0) {
            rc = fail(err, "invalid literal/length code");
            break;
        }
        if (s < 256) {
            if (pos == cap) {
                o.pos = pos;
                o.reserve(1);
                out = o.v.data();
                cap = o.v.size();
            }
            out[pos++] = (uint8_t)s;
            continue;
        }
        if (s == 256) break;
        const int li = s - 257;
        if (li >= 29) {
            rc = fail(err, "invalid length symbol");
            break;
        }
        const size_t len = kLenBase[li] + b.bits(kLenExtra[li]);
        const int di = dist.decode(b);
        if (di < 0 || di >= 30) {
            rc = fail(err, "invalid distance code");
            break;
        }
        const size_t d = kDistBase[di] + b.bits(kDistExtra[di]);
        if (d > pos - base) {
            rc = fail(err, "distance reaches before the start of the output");
            break;
        }
        if (pos + len > cap) {
            o.pos = pos;
            o.reserve(len);
            out = o.v.data();
            cap = o.v.size();
        }
        uint8_t* dst = out + pos;
        const uint8_t* src = dst - d;
        if (d >= len) {
            std::memcpy(dst, src, len);
        } else {
            for (size_t k = 0; k < len; ++k) dst[k] = src[k];  // overlapping: a repeated pattern
        }
        pos += len;
    }
    o.pos = pos;
    bin = b;
    return rc;
}

int dynamic_codes(BitIn& b, Huff& lit, Huff& dist, std::string& err) {
    const int nlen = (int)b.bits(5) + 257, ndist = (int)b.bits(5) + 1, ncode = (int)b.bits(4) + 4;
    if (nlen > 286 || ndist > 30) return fail(err, "too many length or distance codes");
    uint8_t cl[19] = {0};
    for (int i = 0; i < ncode; ++i) cl[kClOrder[i]] = (uint8_t)b.bits(3);
    Huff clh;
    if (clh.build(cl, 19) != 0) return fail(err, "over-subscribed code-length code");
    uint8_t lens[286 + 30];
    int i = 0;
    while (i < nlen + ndist) {
        if (b.past > 8) return fail(err, "deflate stream is truncated");
        const int s = clh.decode(b);
        if (s < 0) return fail(err, "invalid code-length code");
        if (s < 16) {
            lens[i++] = (uint8_t)s;
            continue;
        }
        uint8_t v = 0;
        int rep;
        if (s == 16) {
            if (i == 0) return fail(err, "length repeat with no previous length");
            v = lens[i - 1];
            rep = 3 + (int)b.bits(2);
        } else if (s == 17) {
            rep = 3 + (int)b.bits(3);
        } else {
            rep = 11 + (int)b.bits(7);
        }
        if (i + rep > nlen + ndist) return fail(err, "code lengths overrun");
        while (rep--) lens[i++] = v;
    }
    if (lens[256] == 0) return fail(err, "no end-of-block code");
    if (lit.build(lens, nlen) != 0) return fail(err, "over-subscribed literal/length code");
    if (dist.build(lens + nlen, ndist) != 0) return fail(err, "over-subscribed distance code");
    return 0;
}

}  // namespace

uint32_t crc32(const uint8_t* p, size_t n, uint32_t crc) {
    const CrcTables& T = crc_tables();
    uint32_t c = ~crc;
    while (n >= 8) {
        const uint32_t a = c ^ ((uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24);
        c = T.t[7][a & 0xff] ^ T.t[6][(a >> 8) & 0xff] ^ T.t[5][(a >> 16) & 0xff] ^ T.t[4][a >> 24] ^
            T.t[3][p[4]] ^ T.t[2][p[5]] ^ T.t[1][p[6]] ^ T.t[0][p[7]];
        p += 8;
        n -= 8;
    }
    while (n--) c = T.t[0][(c ^ *p++) & 0xff] ^ (c >> 8);
    return ~c;
}

bool is_gzip(const uint8_t* p, size_t n) { return n >= 2 && p[0] == 0x1f && p[1] == 0x8b; }

int inflate_raw(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t* consumed, size_t stop_after,
                std::string& err) {
    BitIn b(in, n);
    Out o(out);
    const size_t base = o.pos;
    Huff lit, dist;
    int last = 0;
    int rc = 0;
    while (!last && rc == 0) {
        if (stop_after && o.pos >= stop_after) break;
        last = (int)b.bits(1);
        const int type = (int)b.bits(2);
        if (type == 0) {
            b.align_and_reset();
            const size_t at = (size_t)(b.p - in);
            if (b.past || n - at < 4) {
                rc = fail(err, "deflate stream is truncated");
                break;
            }
            const uint32_t len = (uint32_t)in[at] | (uint32_t)in[at + 1] << 8;
            const uint32_t nlen = (uint32_t)in[at + 2] | (uint32_t)in[at + 3] << 8;
            if ((len ^ 0xffffu) != nlen) {
                rc = fail(err, "stored block length check failed");
                break;
            }
            if (n - at - 4 < len) {
                rc = fail(err, "deflate stream is truncated");
                break;
            }
            o.reserve(len);
            std::memcpy(o.v.data() + o.pos, in + at + 4, len);
            o.pos += len;
            b.p = in + at + 4 + len;
        } else if (type == 1) {
            rc = codes_block(b, fixed_codes().lit, fixed_codes().dist, o, base, err);
        } else if (type == 2) {
            rc = dynamic_codes(b, lit, dist, err);
            if (rc == 0) rc = codes_block(b, lit, dist, o, base, err);
        } else {
            rc = fail(err, "invalid block type 3");
        }
        if (rc == 0 && b.truncated()) rc = fail(err, "deflate stream is truncated");
    }
    o.finish();
    if (rc) return rc;
    if (consumed) *consumed = (size_t)((b.consumed_bits() + 7) / 8);
    return 0;
}

int gunzip(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t stop_after, std::string& err) {
    if (!is_gzip(in, n)) return fail(err, "not a gzip stream");
    if (n < 18) return fail(err, "gzip stream is truncated");
    if (in[2] != 8) return fail(err, "gzip compression method is not deflate");
    const uint8_t flg = in[3];
    if (flg & 0xe0) return fail(err, "reserved gzip flag bits are set");
    size_t at = 10;
    if (flg & 4) {  // FEXTRA
        if (n - at < 2) return fail(err, "gzip header is truncated");
        const size_t xlen = (size_t)in[at] | (size_t)in[at + 1] << 8;
        at += 2;
        if (n - at < xlen) return fail(err, "gzip header is truncated");
        at += xlen;
    }
    for (int f : {8, 16}) {  // FNAME, FCOMMENT: zero-terminated
        if (!(flg & f)) continue;
        while (at < n && in[at] != 0) ++at;
        if (at >= n) return fail(err, "gzip header is truncated");
        ++at;
    }
    if (flg & 2) at += 2;  // FHCRC
    if (at > n) return fail(err, "gzip header is truncated");
    // the last four bytes give the size of a single-member file: a capacity hint
    const size_t hint = (size_t)in[n - 4] | (size_t)in[n - 3] << 8 | (size_t)in[n - 2] << 16 | (size_t)in[n - 1] << 24;
    out.clear();
    // DEFLATE expands at most ~1032:1, which bounds a corrupt size field
    const size_t bound = (n / 1024 + 1) * 1032 + 65536;
    out.reserve(stop_after ? stop_after + 65536 : std::min(hint, bound));
    size_t used = 0;
    if (inflate_raw(in + at, n - at, out, &used, stop_after, err) != 0) return -1;
    if (stop_after) return 0;
    at += used;
    if (n - at < 8) return fail(err, "gzip trailer is truncated");
    const uint32_t crc = (uint32_t)in[at] | (uint32_t)in[at + 1] << 8 | (uint32_t)in[at + 2] << 16 |
                         (uint32_t)in[at + 3] << 24;
    const uint32_t isize = (uint32_t)in[at + 4] | (uint32_t)in[at + 5] << 8 | (uint32_t)in[at + 6] << 16 |
                           (uint32_t)in[at + 7] << 24;
    if (isize != (uint32_t)out.size()) return fail(err, "gzip length check failed");
    if (crc != crc32(out.data(), out.size())) return fail(err, "gzip CRC-32 check failed");
    return 0;
}

}  // namespace io
}  // namespace fm
