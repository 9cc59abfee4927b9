// Image codecs of the reference's dataset format (include/isti_io.h).
//
// The reference decodes keyframe images with third-party libraries
// (src/util/image_buffer.cu:103-178: fpng / stb_image for PNG, tinyexr's
// LoadEXR for EXR) and encodes client frames with fpng (:180-200).  This file
// implements the formats from their specifications:
//   DEFLATE  RFC 1951, zlib container RFC 1950;
//   PNG      ISO/IEC 15948 (W3C PNG specification), converted to RGBA8 with
//            the rules stb_image applies for 4 requested channels;
//   OpenEXR  scan-line files (OpenEXR file layout document), NONE / RLE /
//            ZIPS / ZIP / PIZ compression, with the channel mapping of LoadEXR.
#include "isti_io.h"
#include "isti_error.hpp"

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace
{
using isti::set_error;

thread_local int t_decode_threads = 0;

// Threads for a decode of `units` independent pieces: one per 4 pieces, at most 8 and
// the hardware's, unless the caller set a budget (isti::set_decode_threads).
int decode_threads(int units)
{
    int n = t_decode_threads;
    if (n <= 0)
        n = std::min<int>(8, std::max(1u, std::thread::hardware_concurrency()));
    return std::max(1, std::min(n, units / 4));
}

// ------------------------------------------------------------------ files

bool read_file(const char *path, std::vector<uint8_t> &out, std::string &err)
{
    if (!path)
        return err = "null path", false;
    FILE *f = std::fopen(path, "rb");
    if (!f)
        return err = std::string("cannot open ") + path, false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0)
    {
        std::fclose(f);
        return err = std::string("cannot read ") + path, false;
    }
    out.resize(size_t(n));
    const size_t got = n ? std::fread(out.data(), 1, size_t(n), f) : 0;
    std::fclose(f);
    if (got != size_t(n))
        return err = std::string("short read of ") + path, false;
    return true;
}

bool write_file(const char *path, const std::vector<uint8_t> &data, std::string &err)
{
    if (!path)
        return err = "null path", false;
    FILE *f = std::fopen(path, "wb");
    if (!f)
        return err = std::string("cannot create ") + path, false;
    const size_t put = data.empty() ? 0 : std::fwrite(data.data(), 1, data.size(), f);
    const bool ok = put == data.size() && std::fclose(f) == 0;
    if (!ok)
        return err = std::string("cannot write ") + path, false;
    return true;
}

uint32_t be32(const uint8_t *p) { return uint32_t(p[0]) << 24 | uint32_t(p[1]) << 16 | uint32_t(p[2]) << 8 | p[3]; }
uint32_t le32(const uint8_t *p) { return uint32_t(p[3]) << 24 | uint32_t(p[2]) << 16 | uint32_t(p[1]) << 8 | p[0]; }
uint64_t le64(const uint8_t *p) { return uint64_t(le32(p + 4)) << 32 | le32(p); }

// ------------------------------------------------------------------ checksums

uint32_t adler32(const uint8_t *p, size_t n)
{
    uint32_t a = 1, b = 0;
    while (n)
    {
        const size_t k = n < 5552 ? n : 5552; // largest run without 32-bit overflow
        for (size_t i = 0; i < k; i++)
        {
            a += p[i];
            b += a;
        }
        a %= 65521;
        b %= 65521;
        p += k;
        n -= k;
    }
    return b << 16 | a;
}

struct Crc32Table
{
    uint32_t t[256];
    Crc32Table()
    {
        for (uint32_t i = 0; i < 256; i++)
        {
            uint32_t c = i;
            for (int k = 0; k < 8; k++)
                c = (c & 1) ? 0xedb88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
    }
};

uint32_t crc32(const uint8_t *p, size_t n, uint32_t crc = 0)
{
    static const Crc32Table table;
    crc = ~crc;
    for (size_t i = 0; i < n; i++)
        crc = table.t[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
    return ~crc;
}

// ------------------------------------------------------------------ inflate (RFC 1951)

constexpr int FAST_BITS = 10;
constexpr uint16_t LEN_BASE[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                   31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr uint8_t LEN_EXTRA[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr uint16_t DIST_BASE[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                    193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr uint8_t DIST_EXTRA[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
constexpr uint8_t CODE_LENGTH_ORDER[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

uint32_t reverse_bits(uint32_t v, int n)
{
    uint32_t r = 0;
    for (int i = 0; i < n; i++, v >>= 1)
        r = r << 1 | (v & 1);
    return r;
}

// Canonical Huffman code: a FAST_BITS-bit lookup for short codes, counts and
// sorted symbols for the bit-by-bit decode of longer ones.
struct Huffman
{
    uint16_t fast[1 << FAST_BITS]; // (length << 9) | symbol; 0 = not in the table
    uint16_t count[16];
    uint16_t symbol[288];

    bool build(const uint8_t *lengths, int n)
    {
        std::memset(fast, 0, sizeof(fast));
        std::memset(count, 0, sizeof(count));
        for (int i = 0; i < n; i++)
            count[lengths[i]]++;
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; len++)
        {
            left = left * 2 - count[len];
            if (left < 0)
                return false; // over-subscribed
        }
        uint16_t offs[16], next[16];
        offs[1] = 0;
        for (int len = 1; len < 15; len++)
            offs[len + 1] = uint16_t(offs[len] + count[len]);
        uint32_t code = 0;
        for (int len = 1; len < 16; len++)
        {
            code = (code + count[len - 1]) << 1;
            next[len] = uint16_t(code);
        }
        for (int s = 0; s < n; s++)
        {
            const int len = lengths[s];
            if (!len)
                continue;
            symbol[offs[len]++] = uint16_t(s);
            const uint32_t c = next[len]++;
            if (len <= FAST_BITS)
                for (uint32_t k = reverse_bits(c, len); k < (1u << FAST_BITS); k += 1u << len)
                    fast[k] = uint16_t(len << 9 | s);
        }
        return true;
    }
};

struct BitReader
{
    const uint8_t *p, *end;
    uint64_t buf = 0;
    int cnt = 0;
    size_t padding = 0; // zero bytes appended past the end

    void refill()
    {
        if (end - p >= 8) // whole bytes up to 56..63 buffered bits, from one 8-byte load
        {
            uint64_t v = 0;
            for (int k = 0; k < 8; k++) // little-endian assembly (the compiler folds it to one load)
                v |= uint64_t(p[k]) << (8 * k);
            const int take = (63 - cnt) >> 3; // 1..7 bytes: the bits above cnt stay zero
            buf |= (v & ((uint64_t(1) << (8 * take)) - 1)) << cnt;
            p += take;
            cnt += take * 8;
            return;
        }
        while (cnt <= 56)
        {
            uint64_t byte = 0;
            if (p < end)
                byte = *p++;
            else
                padding++;
            buf |= byte << cnt;
            cnt += 8;
        }
    }
    uint32_t get(int n)
    {
        if (n == 0)
            return 0;
        if (cnt < n)
            refill();
        const uint32_t v = uint32_t(buf & ((uint64_t(1) << n) - 1));
        buf >>= n;
        cnt -= n;
        return v;
    }
    // true when bits past the end of the input were consumed
    bool overrun() const { return padding * 8 > size_t(cnt); }
    // bytes of the input consumed so far (whole bytes, after byte alignment)
    size_t consumed(const uint8_t *start) const { return size_t(p - start) + padding - size_t(cnt / 8); }
};

int decode_symbol(BitReader &b, const Huffman &h)
{
    if (b.cnt < 16)
        b.refill();
    const uint16_t e = h.fast[b.buf & ((1u << FAST_BITS) - 1)];
    if (e)
    {
        b.buf >>= e >> 9;
        b.cnt -= e >> 9;
        return e & 511;
    }
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; len++)
    {
        code |= int((b.buf >> (len - 1)) & 1);
        const int c = h.count[len];
        if (code - first < c)
        {
            b.buf >>= len;
            b.cnt -= len;
            return h.symbol[index + code - first];
        }
        index += c;
        first = (first + c) << 1;
        code <<= 1;
    }
    return -1;
}

struct FixedTables
{
    Huffman lit, dist;
    FixedTables()
    {
        uint8_t l[288];
        for (int i = 0; i < 288; i++)
            l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
        lit.build(l, 288);
        uint8_t d[30];
        std::memset(d, 5, sizeof(d));
        dist.build(d, 30);
    }
};

// Inflates a raw DEFLATE stream into `out` (appending); `*used` receives the
// input bytes consumed.  Output beyond `max_out` bytes is an error.
bool inflate(const uint8_t *src, size_t n, std::vector<uint8_t> &out, size_t max_out, size_t *used, std::string &err)
{
    static const FixedTables fixed;
    BitReader b{src, src + n};
    size_t pos = out.size();
    auto ensure = [&](size_t extra) {
        if (pos + extra > out.size())
            out.resize(std::max(pos + extra, std::min(max_out, out.size() * 2 + 65536)));
    };
    if (max_out <= (size_t(1) << 31)) // a known output size (PNG, EXR): one allocation up front
        ensure(max_out - pos);
    Huffman lit, dist;
    bool final = false;
    while (!final)
    {
        final = b.get(1);
        const uint32_t type = b.get(2);
        if (type == 0)
        {
            b.get(b.cnt & 7); // to the byte boundary
            const uint32_t len = b.get(16), nlen = b.get(16);
            if ((len ^ 0xffffu) != nlen)
                return err = "deflate: corrupt stored block", false;
            if (pos + len > max_out)
                return err = "deflate: output larger than expected", false;
            ensure(len);
            uint32_t k = 0;
            for (; k < len && b.cnt >= 8; k++)
                out[pos++] = uint8_t(b.get(8));
            if (b.overrun())
                return err = "deflate: truncated stream", false;
            if (k < len)
            {
                if (size_t(b.end - b.p) < len - k)
                    return err = "deflate: truncated stored block", false;
                std::memcpy(out.data() + pos, b.p, len - k);
                pos += len - k;
                b.p += len - k;
            }
            continue;
        }
        const Huffman *hl = &fixed.lit, *hd = &fixed.dist;
        if (type == 2)
        {
            const int hlit = int(b.get(5)) + 257, hdist = int(b.get(5)) + 1, hclen = int(b.get(4)) + 4;
            if (hlit > 286 || hdist > 30)
                return err = "deflate: bad code counts", false;
            uint8_t cl[19] = {};
            for (int i = 0; i < hclen; i++)
                cl[CODE_LENGTH_ORDER[i]] = uint8_t(b.get(3));
            Huffman clh;
            if (!clh.build(cl, 19))
                return err = "deflate: bad code-length code", false;
            uint8_t lens[286 + 30];
            int i = 0;
            while (i < hlit + hdist)
            {
                const int s = decode_symbol(b, clh);
                if (s < 0)
                    return err = "deflate: bad code-length symbol", false;
                if (s < 16)
                {
                    lens[i++] = uint8_t(s);
                    continue;
                }
                int rep;
                uint8_t val = 0;
                if (s == 16)
                {
                    if (i == 0)
                        return err = "deflate: repeat without a previous length", false;
                    val = lens[i - 1];
                    rep = 3 + int(b.get(2));
                }
                else if (s == 17)
                    rep = 3 + int(b.get(3));
                else
                    rep = 11 + int(b.get(7));
                if (i + rep > hlit + hdist)
                    return err = "deflate: code lengths overflow", false;
                while (rep--)
                    lens[i++] = val;
            }
            if (b.overrun())
                return err = "deflate: truncated stream", false;
            if (lens[256] == 0)
                return err = "deflate: no end-of-block code", false;
            if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist))
                return err = "deflate: bad literal/length or distance code", false;
            hl = &lit;
            hd = &dist;
        }
        else if (type != 1)
            return err = "deflate: bad block type", false;

        for (;;)
        {
            const int s = decode_symbol(b, *hl);
            if (s < 256)
            {
                if (s < 0)
                    return err = "deflate: bad literal/length code", false;
                if (pos >= max_out)
                    return err = "deflate: output larger than expected", false;
                ensure(1);
                out[pos++] = uint8_t(s);
                continue;
            }
            if (s == 256)
                break;
            const int li = s - 257;
            if (li >= 29)
                return err = "deflate: bad length symbol", false;
            const uint32_t len = LEN_BASE[li] + b.get(LEN_EXTRA[li]);
            const int ds = decode_symbol(b, *hd);
            if (ds < 0 || ds >= 30)
                return err = "deflate: bad distance symbol", false;
            const uint32_t d = DIST_BASE[ds] + b.get(DIST_EXTRA[ds]);
            if (d > pos)
                return err = "deflate: distance before the start", false;
            if (pos + len > max_out)
                return err = "deflate: output larger than expected", false;
            if (b.overrun())
                return err = "deflate: truncated stream", false;
            ensure(len);
            uint8_t *o = out.data() + pos;
            const uint8_t *from = o - d;
            if (d >= len)
                std::memcpy(o, from, len); // no overlap
            else if (d >= 8)
            {
                uint32_t k = 0; // overlapping, but every 8-byte chunk reads bytes already written
                for (; k + 8 <= len; k += 8)
                    std::memcpy(o + k, from + k, 8);
                for (; k < len; k++)
                    o[k] = from[k];
            }
            else
            {
                // a pattern of period d < 8: copy the first bytes one at a time, then 8-byte
                // chunks from a multiple of d back (>= 8), which repeats the same pattern
                const uint32_t d8 = d * ((8 + d - 1) / d);
                uint32_t k = 0;
                for (; k < len && k < d8; k++)
                    o[k] = from[k];
                for (; k + 8 <= len; k += 8)
                    std::memcpy(o + k, o + k - d8, 8);
                for (; k < len; k++)
                    o[k] = o[k - d];
            }
            pos += len;
        }
        if (b.overrun())
            return err = "deflate: truncated stream", false;
    }
    out.resize(pos);
    if (used)
        *used = b.consumed(src);
    return true;
}

bool zlib_decompress(const uint8_t *src, size_t n, std::vector<uint8_t> &out, size_t max_out, std::string &err)
{
    if (n < 6)
        return err = "zlib: stream too short", false;
    const uint32_t cmf = src[0], flg = src[1];
    if ((cmf * 256 + flg) % 31 != 0 || (cmf & 15) != 8 || (cmf >> 4) > 7)
        return err = "zlib: bad header", false;
    if (flg & 32)
        return err = "zlib: preset dictionary not supported", false;
    const size_t start = out.size();
    size_t used = 0;
    if (!inflate(src + 2, n - 2, out, max_out, &used, err))
        return false;
    if (2 + used + 4 > n)
        return err = "zlib: missing checksum", false;
    if (be32(src + 2 + used) != adler32(out.data() + start, out.size() - start))
        return err = "zlib: checksum mismatch", false;
    return true;
}

// ------------------------------------------------------------------ deflate (fixed codes, greedy LZ77)

struct BitWriter
{
    std::vector<uint8_t> &out;
    uint64_t buf = 0;
    int cnt = 0;
    void put(uint32_t v, int n)
    {
        buf |= uint64_t(v) << cnt;
        cnt += n;
        while (cnt >= 8)
        {
            out.push_back(uint8_t(buf));
            buf >>= 8;
            cnt -= 8;
        }
    }
    void put_code(uint32_t code, int n) { put(reverse_bits(code, n), n); } // Huffman codes go MSB first
    void flush()
    {
        if (cnt)
            out.push_back(uint8_t(buf));
        buf = 0;
        cnt = 0;
    }
};

void put_literal(BitWriter &w, int v)
{
    if (v < 144)
        w.put_code(0x30 + v, 8);
    else if (v < 256)
        w.put_code(0x190 + (v - 144), 9);
    else if (v < 280)
        w.put_code(v - 256, 7);
    else
        w.put_code(0xc0 + (v - 280), 8);
}

void put_match(BitWriter &w, uint32_t len, uint32_t dist)
{
    int li = 28;
    while (LEN_BASE[li] > len)
        li--;
    put_literal(w, 257 + li);
    w.put(len - LEN_BASE[li], LEN_EXTRA[li]);
    int di = 29;
    while (DIST_BASE[di] > dist)
        di--;
    w.put_code(uint32_t(di), 5);
    w.put(dist - DIST_BASE[di], DIST_EXTRA[di]);
}

void zlib_compress(const uint8_t *src, size_t n, std::vector<uint8_t> &out)
{
    out.push_back(0x78);
    out.push_back(0x9c);
    BitWriter w{out};
    w.put(1, 1); // final block
    w.put(1, 2); // fixed Huffman codes
    constexpr int HASH_BITS = 16;
    std::vector<int64_t> head(size_t(1) << HASH_BITS, -1);
    auto hash3 = [&](size_t i) {
        const uint32_t v = uint32_t(src[i]) | uint32_t(src[i + 1]) << 8 | uint32_t(src[i + 2]) << 16;
        return (v * 2654435761u) >> (32 - HASH_BITS);
    };
    size_t i = 0;
    while (i < n)
    {
        uint32_t best = 0, dist = 0;
        if (i + 3 <= n)
        {
            const uint32_t h = hash3(i);
            const int64_t cand = head[h];
            head[h] = int64_t(i);
            if (cand >= 0 && i - size_t(cand) <= 32768)
            {
                const size_t maxlen = std::min<size_t>(258, n - i);
                uint32_t l = 0;
                while (l + 8 <= maxlen) // 8 bytes at a time, then the tail
                {
                    uint64_t p, q;
                    std::memcpy(&p, src + size_t(cand) + l, 8);
                    std::memcpy(&q, src + i + l, 8);
                    if (p != q)
                        break;
                    l += 8;
                }
                while (l < maxlen && src[size_t(cand) + l] == src[i + l])
                    l++;
                if (l >= 3)
                {
                    best = l;
                    dist = uint32_t(i - size_t(cand));
                }
            }
        }
        if (best)
        {
            put_match(w, best, dist);
            for (size_t k = i + 1; k < i + best && k + 3 <= n; k++)
                head[hash3(k)] = int64_t(k);
            i += best;
        }
        else
            put_literal(w, src[i++]);
    }
    put_literal(w, 256);
    w.flush();
    const uint32_t a = adler32(src, n);
    for (int s = 24; s >= 0; s -= 8)
        out.push_back(uint8_t(a >> s));
}

// ------------------------------------------------------------------ PNG

constexpr uint8_t PNG_SIG[8] = {137, 80, 78, 71, 13, 10, 26, 10};

int png_channels(int color) { return color == 2 ? 3 : color == 4 ? 2 : color == 6 ? 4 : 1; }

bool png_depth_ok(int color, int depth)
{
    switch (color)
    {
    case 0: return depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16;
    case 3: return depth == 1 || depth == 2 || depth == 4 || depth == 8;
    case 2:
    case 4:
    case 6: return depth == 8 || depth == 16;
    }
    return false;
}

uint8_t paeth(int a, int b, int c)
{
    const int p = a + b - c;
    const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc)
        return uint8_t(a);
    return uint8_t(pb <= pc ? b : c);
}

// Reverses the per-row filters of one (sub-)image in place; rows are
// [filter byte][row_bytes], `bpp` the filter's byte distance.
bool png_unfilter(uint8_t *data, uint32_t rows, size_t row_bytes, int bpp, std::string &err)
{
    std::vector<uint8_t> zero(row_bytes, 0);
    const uint8_t *prior = zero.data();
    for (uint32_t y = 0; y < rows; y++)
    {
        uint8_t *row = data + size_t(y) * (row_bytes + 1);
        const uint8_t f = row[0];
        uint8_t *r = row + 1;
        switch (f)
        {
        case 0: break;
        case 1:
            for (size_t i = size_t(bpp); i < row_bytes; i++)
                r[i] = uint8_t(r[i] + r[i - bpp]);
            break;
        case 2:
            for (size_t i = 0; i < row_bytes; i++)
                r[i] = uint8_t(r[i] + prior[i]);
            break;
        case 3:
        {
            const size_t first = std::min(size_t(bpp), row_bytes); // no left neighbour
            for (size_t i = 0; i < first; i++)
                r[i] = uint8_t(r[i] + (prior[i] >> 1));
            for (size_t i = first; i < row_bytes; i++)
                r[i] = uint8_t(r[i] + ((int(r[i - bpp]) + prior[i]) >> 1));
            break;
        }
        case 4:
        {
            const size_t first = std::min(size_t(bpp), row_bytes); // paeth(0, up, 0) = up
            for (size_t i = 0; i < first; i++)
                r[i] = uint8_t(r[i] + prior[i]);
            for (size_t i = first; i < row_bytes; i++)
                r[i] = uint8_t(r[i] + paeth(r[i - bpp], prior[i], prior[i - bpp]));
            break;
        }
        default: return err = "png: bad filter type", false;
        }
        prior = r;
    }
    return true;
}

struct PngHeader
{
    uint32_t w = 0, h = 0;
    int depth = 0, color = 0, interlace = 0;
    uint8_t palette[256][4];
    int palette_n = 0;
    bool has_trns = false;
    uint16_t trns_key[3] = {};
};

// Writes the pixels of one unfiltered (sub-)image row into the RGBA8 result at
// x = x0 + i * dx, with stb_image's conversions for 4 requested channels.
void png_emit_row(const PngHeader &hd, const uint8_t *r, uint32_t n, uint8_t *dst, uint32_t dx)
{
    static const uint8_t depth_scale[9] = {0, 0xff, 0x55, 0, 0x11, 0, 0, 0, 0x01};
    const int ch = png_channels(hd.color);
    if (hd.depth == 8 && dx == 1 && (hd.color == 6 || (hd.color == 2 && !hd.has_trns)))
    {
        // the common layouts: RGBA8 as it is, RGB8 with opaque alpha
        if (hd.color == 6)
            std::memcpy(dst, r, size_t(n) * 4);
        else
            for (uint32_t i = 0; i < n; i++, dst += 4, r += 3)
            {
                dst[0] = r[0];
                dst[1] = r[1];
                dst[2] = r[2];
                dst[3] = 255;
            }
        return;
    }
    auto sample = [&](uint32_t i, int c) -> uint32_t {
        const uint32_t idx = i * uint32_t(ch) + uint32_t(c);
        if (hd.depth == 16)
            return uint32_t(r[2 * idx]) << 8 | r[2 * idx + 1];
        if (hd.depth == 8)
            return r[idx];
        const uint32_t bit = idx * uint32_t(hd.depth);
        return (r[bit >> 3] >> (8 - hd.depth - (bit & 7))) & ((1u << hd.depth) - 1);
    };
    auto to8 = [&](uint32_t v) -> uint8_t { return hd.depth == 16 ? uint8_t(v >> 8) : uint8_t(v); };
    for (uint32_t i = 0; i < n; i++, dst += 4 * size_t(dx))
    {
        switch (hd.color)
        {
        case 0:
        {
            const uint32_t g = sample(i, 0);
            uint8_t a = 255;
            if (hd.depth == 16)
            {
                if (hd.has_trns && g == hd.trns_key[0])
                    a = 0;
                dst[0] = dst[1] = dst[2] = uint8_t(g >> 8);
            }
            else
            {
                const uint8_t s = depth_scale[hd.depth];
                const uint8_t gs = uint8_t(g * s);
                if (hd.has_trns && gs == uint8_t((hd.trns_key[0] & 255) * s))
                    a = 0;
                dst[0] = dst[1] = dst[2] = gs;
            }
            dst[3] = a;
            break;
        }
        case 2:
        {
            const uint32_t rr = sample(i, 0), gg = sample(i, 1), bb = sample(i, 2);
            uint8_t a = 255;
            if (hd.has_trns)
            {
                const bool match = hd.depth == 16 ? (rr == hd.trns_key[0] && gg == hd.trns_key[1] && bb == hd.trns_key[2])
                                                  : (rr == (hd.trns_key[0] & 255u) && gg == (hd.trns_key[1] & 255u) &&
                                                     bb == (hd.trns_key[2] & 255u));
                if (match)
                    a = 0;
            }
            dst[0] = to8(rr);
            dst[1] = to8(gg);
            dst[2] = to8(bb);
            dst[3] = a;
            break;
        }
        case 3:
        {
            const uint32_t k = sample(i, 0);
            if (int(k) < hd.palette_n)
                std::memcpy(dst, hd.palette[k], 4);
            else
                dst[0] = dst[1] = dst[2] = 0, dst[3] = 255;
            break;
        }
        case 4:
        {
            const uint8_t g = to8(sample(i, 0));
            dst[0] = dst[1] = dst[2] = g;
            dst[3] = to8(sample(i, 1));
            break;
        }
        default: // 6
            dst[0] = to8(sample(i, 0));
            dst[1] = to8(sample(i, 1));
            dst[2] = to8(sample(i, 2));
            dst[3] = to8(sample(i, 3));
            break;
        }
    }
}

bool png_decode(const uint8_t *d, size_t n, uint32_t &w, uint32_t &h, std::vector<uint8_t> &rgba, std::string &err)
{
    if (n < 8 || std::memcmp(d, PNG_SIG, 8) != 0)
        return err = "png: not a PNG file", false;
    PngHeader hd;
    std::vector<uint8_t> idat;
    size_t pos = 8;
    bool seen_ihdr = false, seen_end = false;
    while (!seen_end)
    {
        if (pos + 12 > n)
            return err = "png: truncated chunk", false;
        const uint32_t len = be32(d + pos);
        const uint8_t *type = d + pos + 4;
        const uint8_t *body = d + pos + 8;
        if (len > n - pos - 12)
            return err = "png: truncated chunk", false;
        const uint32_t t = be32(type);
        if (!seen_ihdr && t != 0x49484452u)
            return err = "png: first chunk is not IHDR", false;
        switch (t)
        {
        case 0x49484452u: // IHDR
            if (seen_ihdr || len != 13)
                return err = "png: bad IHDR", false;
            seen_ihdr = true;
            hd.w = be32(body);
            hd.h = be32(body + 4);
            hd.depth = body[8];
            hd.color = body[9];
            hd.interlace = body[12];
            if (hd.w == 0 || hd.h == 0 || hd.w > (1u << 24) || hd.h > (1u << 24))
                return err = "png: bad image size", false;
            if (!png_depth_ok(hd.color, hd.depth))
                return err = "png: bad colour type / bit depth", false;
            if (body[10] != 0 || body[11] != 0 || hd.interlace > 1)
                return err = "png: bad compression, filter or interlace method", false;
            break;
        case 0x504c5445u: // PLTE
            if (len % 3 != 0 || len / 3 > 256 || len == 0)
                return err = "png: bad PLTE", false;
            hd.palette_n = int(len / 3);
            for (int i = 0; i < hd.palette_n; i++)
            {
                hd.palette[i][0] = body[3 * i];
                hd.palette[i][1] = body[3 * i + 1];
                hd.palette[i][2] = body[3 * i + 2];
                hd.palette[i][3] = 255;
            }
            break;
        case 0x74524e53u: // tRNS
            if (!idat.empty())
                return err = "png: tRNS after IDAT", false;
            if (hd.color == 3)
            {
                if (hd.palette_n == 0)
                    return err = "png: tRNS before PLTE", false;
                if (int(len) > hd.palette_n)
                    return err = "png: bad tRNS length", false;
                for (uint32_t i = 0; i < len; i++)
                    hd.palette[i][3] = body[i];
            }
            else if (hd.color == 0 || hd.color == 2)
            {
                const uint32_t need = hd.color == 0 ? 2 : 6;
                if (len != need)
                    return err = "png: bad tRNS length", false;
                hd.has_trns = true;
                for (uint32_t k = 0; k < need / 2; k++)
                    hd.trns_key[k] = uint16_t(body[2 * k] << 8 | body[2 * k + 1]);
            }
            else
                return err = "png: tRNS with an alpha channel", false;
            break;
        case 0x49444154u: // IDAT
            idat.insert(idat.end(), body, body + len);
            break;
        case 0x49454e44u: // IEND
            seen_end = true;
            break;
        default:
            if (!(type[0] & 0x20))
                return err = "png: unknown critical chunk", false;
            break;
        }
        pos += 12 + size_t(len);
    }
    if (hd.color == 3 && hd.palette_n == 0)
        return err = "png: palette image without PLTE", false;
    if (idat.empty())
        return err = "png: no image data", false;

    const int ch = png_channels(hd.color);
    const size_t bits_pp = size_t(ch) * size_t(hd.depth);
    const int bpp = int(std::max<size_t>(1, bits_pp / 8));
    struct Pass { uint32_t x0, y0, dx, dy; };
    static const Pass ADAM7[7] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4}, {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    const Pass whole{0, 0, 1, 1};
    const Pass *passes = hd.interlace ? ADAM7 : &whole;
    const int n_passes = hd.interlace ? 7 : 1;
    size_t raw_size = 0;
    for (int p = 0; p < n_passes; p++)
    {
        const uint32_t pw = hd.w > passes[p].x0 ? (hd.w - passes[p].x0 + passes[p].dx - 1) / passes[p].dx : 0;
        const uint32_t ph = hd.h > passes[p].y0 ? (hd.h - passes[p].y0 + passes[p].dy - 1) / passes[p].dy : 0;
        if (pw && ph)
            raw_size += size_t(ph) * (1 + (size_t(pw) * bits_pp + 7) / 8);
    }
    std::vector<uint8_t> raw;
    raw.reserve(raw_size);
    if (!zlib_decompress(idat.data(), idat.size(), raw, raw_size, err))
        return err = "png: " + err, false;
    if (raw.size() != raw_size)
        return err = "png: image data has the wrong size", false;

    rgba.assign(size_t(hd.w) * hd.h * 4, 0);
    size_t off = 0;
    for (int p = 0; p < n_passes; p++)
    {
        const Pass &ps = passes[p];
        const uint32_t pw = hd.w > ps.x0 ? (hd.w - ps.x0 + ps.dx - 1) / ps.dx : 0;
        const uint32_t ph = hd.h > ps.y0 ? (hd.h - ps.y0 + ps.dy - 1) / ps.dy : 0;
        if (!pw || !ph)
            continue;
        const size_t row_bytes = (size_t(pw) * bits_pp + 7) / 8;
        if (!png_unfilter(raw.data() + off, ph, row_bytes, bpp, err))
            return false;
        for (uint32_t j = 0; j < ph; j++)
        {
            const uint8_t *r = raw.data() + off + size_t(j) * (row_bytes + 1) + 1;
            const size_t y = size_t(ps.y0) + size_t(j) * ps.dy;
            png_emit_row(hd, r, pw, rgba.data() + (y * hd.w + ps.x0) * 4, ps.dx);
        }
        off += size_t(ph) * (row_bytes + 1);
    }
    w = hd.w;
    h = hd.h;
    return true;
}

void png_chunk(std::vector<uint8_t> &out, const char *type, const uint8_t *data, size_t len)
{
    const size_t at = out.size();
    for (int s = 24; s >= 0; s -= 8)
        out.push_back(uint8_t(len >> s));
    out.insert(out.end(), type, type + 4);
    if (len)
        out.insert(out.end(), data, data + len);
    const uint32_t c = crc32(out.data() + at + 4, 4 + len);
    for (int s = 24; s >= 0; s -= 8)
        out.push_back(uint8_t(c >> s));
}

void png_encode(uint32_t w, uint32_t h, int ch, const uint8_t *px, std::vector<uint8_t> &out)
{
    const size_t row_bytes = size_t(w) * ch;
    std::vector<uint8_t> filtered(size_t(h) * (row_bytes + 1));
    std::vector<uint8_t> zero(row_bytes, 0);
    auto mag = [](uint8_t v) { return uint32_t(v < 128 ? v : 256 - v); };
    for (uint32_t y = 0; y < h; y++)
    {
        const uint8_t *r = px + size_t(y) * row_bytes;
        const uint8_t *up = y ? r - row_bytes : zero.data();
        uint8_t *dst = filtered.data() + size_t(y) * (row_bytes + 1);
        // the filter with the smallest sum of |residual| (signed bytes), all five costs in one pass
        uint64_t cost[5] = {0, 0, 0, 0, 0};
        for (size_t i = 0; i < row_bytes; i++)
        {
            const int a = i >= size_t(ch) ? r[i - ch] : 0;
            const int b = up[i];
            const int c = i >= size_t(ch) ? up[i - ch] : 0;
            const int x = r[i];
            cost[0] += mag(uint8_t(x));
            cost[1] += mag(uint8_t(x - a));
            cost[2] += mag(uint8_t(x - b));
            cost[3] += mag(uint8_t(x - ((a + b) >> 1)));
            cost[4] += mag(uint8_t(x - paeth(a, b, c)));
        }
        int f = 0;
        for (int k = 1; k < 5; k++)
            if (cost[k] < cost[f])
                f = k;
        dst[0] = uint8_t(f);
        for (size_t i = 0; i < row_bytes; i++)
        {
            const int a = i >= size_t(ch) ? r[i - ch] : 0;
            const int b = up[i];
            const int c = i >= size_t(ch) ? up[i - ch] : 0;
            const int pred = f == 0 ? 0 : f == 1 ? a : f == 2 ? b : f == 3 ? (a + b) >> 1 : paeth(a, b, c);
            dst[1 + i] = uint8_t(r[i] - pred);
        }
    }
    std::vector<uint8_t> z;
    zlib_compress(filtered.data(), filtered.size(), z);
    out.assign(PNG_SIG, PNG_SIG + 8);
    uint8_t ihdr[13];
    for (int s = 0; s < 4; s++)
    {
        ihdr[s] = uint8_t(w >> (24 - 8 * s));
        ihdr[4 + s] = uint8_t(h >> (24 - 8 * s));
    }
    ihdr[8] = 8;
    ihdr[9] = ch == 4 ? 6 : 2;
    ihdr[10] = ihdr[11] = ihdr[12] = 0;
    png_chunk(out, "IHDR", ihdr, 13);
    png_chunk(out, "IDAT", z.data(), z.size());
    png_chunk(out, "IEND", nullptr, 0);
}

// ------------------------------------------------------------------ OpenEXR

enum ExrPixel { EXR_UINT = 0, EXR_HALF = 1, EXR_FLOAT = 2 };

struct ExrChannel
{
    std::string name;
    int type;
};

// Exact binary16 -> binary32 (IEEE 754): same value, NaN payload kept.
uint32_t half_bits_to_float_bits(uint16_t hv)
{
    const uint32_t sign = uint32_t(hv & 0x8000u) << 16;
    uint32_t exp = (hv >> 10) & 0x1f;
    uint32_t mant = hv & 0x3ffu;
    if (exp == 0x1f)
        return sign | 0x7f800000u | mant << 13;
    if (exp == 0)
    {
        if (mant == 0)
            return sign;
        // subnormal: normalise
        int e = -1;
        do
        {
            mant <<= 1;
            e++;
        } while (!(mant & 0x400u));
        mant &= 0x3ffu;
        return sign | uint32_t(127 - 15 - e) << 23 | mant << 13;
    }
    return sign | (exp + 112) << 23 | mant << 13;
}

// OpenEXR's RLE: a signed count byte, negative = that many literal bytes,
// otherwise one byte repeated count + 1 times.
bool exr_unrle(const uint8_t *in, size_t n, uint8_t *out, size_t out_n)
{
    size_t o = 0, i = 0;
    while (i < n)
    {
        const int c = int(int8_t(in[i++]));
        if (c < 0)
        {
            const size_t k = size_t(-c);
            if (i + k > n || o + k > out_n)
                return false;
            std::memcpy(out + o, in + i, k);
            i += k;
            o += k;
        }
        else
        {
            const size_t k = size_t(c) + 1;
            if (i >= n || o + k > out_n)
                return false;
            std::memset(out + o, in[i++], k);
            o += k;
        }
    }
    return o == out_n;
}

// The byte predictor and half-split reordering applied by the ZIP and RLE
// compressors of OpenEXR, undone.
void exr_unpredict(std::vector<uint8_t> &t, uint8_t *out)
{
    for (size_t i = 1; i < t.size(); i++)
        t[i] = uint8_t(int(t[i - 1]) + int(t[i]) - 128);
    const size_t half = (t.size() + 1) / 2;
    for (size_t i = 0; i < t.size(); i++)
        out[i] = (i & 1) ? t[half + i / 2] : t[i / 2];
}

// ---- PIZ (OpenEXR compression 4), restated from the published OpenEXR format:
// a block of 32 scan lines is split into 16-bit words (a HALF sample is one
// word, a FLOAT or UINT sample two, per channel plane), the words present are
// remapped to a dense range through a 65536-bit presence bitmap, each plane is
// transformed by a 2-D Haar-like wavelet, and the words are Huffman coded
// with a run-length symbol.  Block layout: u16 first and last non-zero bitmap
// byte, those bitmap bytes, i32 Huffman stream length, the Huffman stream.
namespace piz
{
constexpr int kEncSize = 65537;   // code-length table entries (symbols 0..65535, plus one)
constexpr int kDecBits = 14;      // bits of the direct decoding table
constexpr int kDecSize = 1 << kDecBits;
constexpr int kShortZeroRun = 59; // code lengths 59..62 encode 2..5 zero lengths
constexpr int kLongZeroRun = 63;  // followed by 8 bits: 6..261 zero lengths
constexpr int kShortestLongRun = 2 + kLongZeroRun - kShortZeroRun;

struct Bits
{
    const uint8_t *p, *end;
    uint64_t c = 0;
    int lc = 0;
    bool more() const { return p < end; }
    bool fill(int nb) // at least nb (<= 56) bits buffered
    {
        while (lc < nb)
        {
            if (p >= end)
                return false;
            c = (c << 8) | *p++;
            lc += 8;
        }
        return true;
    }
    bool get(int nb, uint64_t &v)
    {
        if (!fill(nb))
            return false;
        lc -= nb;
        v = (c >> lc) & ((uint64_t(1) << nb) - 1);
        return true;
    }
};

struct DecEntry
{
    int len = 0;               // > 0: a code of at most kDecBits bits for symbol `sym`
    uint32_t sym = 0;
    std::vector<uint32_t> lng; // symbols of the longer codes sharing this kDecBits-bit prefix
};

// Code lengths of symbols lo..hi (6 bits each, with zero-run escapes), then the
// canonical code of every symbol: entry = length | code << 6.  Codes are given
// from the longest length down, each length's codes in symbol order.
bool read_code_table(Bits &in, int lo, int hi, std::vector<uint64_t> &code)
{
    code.assign(kEncSize, 0);
    for (int s = lo; s <= hi; s++)
    {
        uint64_t l;
        if (!in.get(6, l))
            return false;
        int run = 0;
        if (l == uint64_t(kLongZeroRun))
        {
            uint64_t r;
            if (!in.get(8, r))
                return false;
            run = int(r) + kShortestLongRun;
        }
        else if (l >= uint64_t(kShortZeroRun))
            run = int(l) - kShortZeroRun + 2;
        if (run)
        {
            if (s + run > hi + 1)
                return false;
            s += run - 1; // entries are already zero
        }
        else
            code[size_t(s)] = l;
    }
    uint64_t count[59] = {};
    for (int s = 0; s < kEncSize; s++)
        count[code[size_t(s)]]++;
    uint64_t next = 0;
    for (int l = 58; l > 0; l--)
    {
        const uint64_t start = next;
        next = (next + count[l]) >> 1;
        count[l] = start;
    }
    for (int s = 0; s < kEncSize; s++)
    {
        const uint64_t l = code[size_t(s)];
        if (l > 0)
            code[size_t(s)] = l | (count[l]++ << 6);
    }
    return true;
}

bool build_decoder(const std::vector<uint64_t> &code, int lo, int hi, std::vector<DecEntry> &dec)
{
    dec.assign(kDecSize, DecEntry());
    for (int s = lo; s <= hi; s++)
    {
        const uint64_t c = code[size_t(s)] >> 6;
        const int l = int(code[size_t(s)] & 63);
        if (l == 0)
            continue;
        if (c >> l)
            return false; // more code bits than its length
        if (l > kDecBits)
        {
            DecEntry &e = dec[size_t(c >> (l - kDecBits))];
            if (e.len)
                return false;
            e.lng.push_back(uint32_t(s));
        }
        else
        {
            const size_t first = size_t(c << (kDecBits - l)), cnt = size_t(1) << (kDecBits - l);
            for (size_t i = first; i < first + cnt; i++)
            {
                if (dec[i].len || !dec[i].lng.empty())
                    return false;
                dec[i].len = l;
                dec[i].sym = uint32_t(s);
            }
        }
    }
    return true;
}

// One decoded symbol: a literal word, or (the highest symbol) 8 bits of run length
// repeating the previous word.
inline bool emit(uint32_t sym, uint32_t run_sym, Bits &in, uint16_t *out, size_t &o, size_t no)
{
    if (sym == run_sym)
    {
        uint64_t cnt;
        if (!in.get(8, cnt) || o == 0 || o + cnt > no)
            return false;
        const uint16_t prev = out[o - 1];
        for (uint64_t i = 0; i < cnt; i++)
            out[o++] = prev;
        return true;
    }
    if (o >= no)
        return false;
    out[o++] = uint16_t(sym);
    return true;
}

bool huffman_decode(const uint8_t *src, size_t n, uint16_t *out, size_t no)
{
    if (n == 0)
        return no == 0;
    if (n < 20)
        return false;
    const uint32_t lo = le32(src), hi = le32(src + 4), n_bits = le32(src + 12);
    if (lo >= uint32_t(kEncSize) || hi >= uint32_t(kEncSize) || lo > hi)
        return false;
    Bits tab{src + 20, src + n};
    std::vector<uint64_t> code;
    if (!read_code_table(tab, int(lo), int(hi), code))
        return false;
    const size_t avail = size_t(src + n - tab.p);
    if (uint64_t(n_bits) > 8 * uint64_t(avail))
        return false;
    std::vector<DecEntry> dec;
    if (!build_decoder(code, int(lo), int(hi), dec))
        return false;

    Bits in{tab.p, tab.p + (size_t(n_bits) + 7) / 8};
    size_t o = 0;
    while (in.more())
    {
        in.c = (in.c << 8) | *in.p++;
        in.lc += 8;
        while (in.lc >= kDecBits)
        {
            const DecEntry &e = dec[size_t((in.c >> (in.lc - kDecBits)) & (kDecSize - 1))];
            if (e.len)
            {
                in.lc -= e.len;
                if (!emit(e.sym, hi, in, out, o, no))
                    return false;
                continue;
            }
            if (e.lng.empty())
                return false;
            bool found = false;
            for (uint32_t s : e.lng)
            {
                const int l = int(code[s] & 63);
                while (in.lc < l && in.more())
                {
                    in.c = (in.c << 8) | *in.p++;
                    in.lc += 8;
                }
                if (in.lc >= l && (code[s] >> 6) == ((in.c >> (in.lc - l)) & ((uint64_t(1) << l) - 1)))
                {
                    in.lc -= l;
                    if (!emit(s, hi, in, out, o, no))
                        return false;
                    found = true;
                    break;
                }
            }
            if (!found)
                return false;
        }
    }
    // the codes in the last partial byte: drop its padding bits, then decode short codes
    const int pad = int((8 - n_bits) & 7);
    in.c >>= pad;
    in.lc -= pad;
    while (in.lc > 0)
    {
        const DecEntry &e = dec[size_t((in.c << (kDecBits - in.lc)) & (kDecSize - 1))];
        if (!e.len || e.len > in.lc)
            return false;
        in.lc -= e.len;
        if (!emit(e.sym, hi, in, out, o, no))
            return false;
    }
    return o == no;
}

// inverse of the 14-bit wavelet step (values below 1 << 14, signed arithmetic)
inline void wdec14(uint16_t l, uint16_t h, uint16_t &a, uint16_t &b)
{
    const int ls = int16_t(l), hs = int16_t(h);
    const int ai = ls + (hs & 1) + (hs >> 1);
    a = uint16_t(int16_t(ai));
    b = uint16_t(int16_t(ai - hs));
}

// inverse of the 16-bit wavelet step (modulo 2^16)
inline void wdec16(uint16_t l, uint16_t h, uint16_t &a, uint16_t &b)
{
    const int m = l, d = h;
    const int bb = (m - (d >> 1)) & 0xffff;
    const int aa = (d + bb - 0x8000) & 0xffff;
    a = uint16_t(aa);
    b = uint16_t(bb);
}

// Inverse 2-D wavelet of an nx x ny plane of words at stride ox (x) and oy (y),
// from the coarsest level to the finest.
void wavelet_decode(uint16_t *in, int nx, int ox, int ny, int oy, uint16_t max_value)
{
    const bool w14 = max_value < (1 << 14);
    auto dec = [w14](uint16_t l, uint16_t h, uint16_t &a, uint16_t &b) { w14 ? wdec14(l, h, a, b) : wdec16(l, h, a, b); };
    const int n = nx > ny ? ny : nx;
    int p = 1;
    while (p <= n)
        p <<= 1;
    p >>= 1;
    int p2 = p;
    p >>= 1;
    while (p >= 1)
    {
        const ptrdiff_t oy1 = ptrdiff_t(oy) * p, oy2 = ptrdiff_t(oy) * p2, ox1 = ptrdiff_t(ox) * p, ox2 = ptrdiff_t(ox) * p2;
        const ptrdiff_t ey = ptrdiff_t(oy) * (ny - p2);
        ptrdiff_t py = 0;
        for (; py <= ey; py += oy2)
        {
            ptrdiff_t px = py;
            const ptrdiff_t ex = py + ptrdiff_t(ox) * (nx - p2);
            for (; px <= ex; px += ox2)
            {
                uint16_t *q00 = in + px, *q01 = q00 + ox1, *q10 = q00 + oy1, *q11 = q10 + ox1;
                uint16_t i00, i01, i10, i11;
                dec(*q00, *q10, i00, i10);
                dec(*q01, *q11, i01, i11);
                dec(i00, i01, *q00, *q01);
                dec(i10, i11, *q10, *q11);
            }
            if (nx & p) // odd column: 1-D in y
            {
                uint16_t *q00 = in + px, *q10 = q00 + oy1, i00;
                dec(*q00, *q10, i00, *q10);
                *q00 = i00;
            }
        }
        if (ny & p) // odd line: 1-D in x
        {
            ptrdiff_t px = py;
            const ptrdiff_t ex = py + ptrdiff_t(ox) * (nx - p2);
            for (; px <= ex; px += ox2)
            {
                uint16_t *q00 = in + px, *q01 = q00 + ox1, i00;
                dec(*q00, *q01, i00, *q01);
                *q00 = i00;
            }
        }
        p2 = p;
        p >>= 1;
    }
}

// One PIZ block of `lines` scan lines of width w -> the uncompressed block (per
// line, per channel in header order, little-endian samples).
bool decompress(const uint8_t *src, size_t n, const std::vector<int> &words_per_sample, int w, int lines, uint8_t *out)
{
    size_t total = 0;
    for (int s : words_per_sample)
        total += size_t(w) * size_t(lines) * size_t(s);
    if (n < 4)
        return false;
    const uint16_t min_nz = uint16_t(src[0] | src[1] << 8), max_nz = uint16_t(src[2] | src[3] << 8);
    size_t pos = 4;
    if (max_nz >= 8192)
        return false;
    std::vector<uint8_t> bitmap(8192, 0);
    if (min_nz <= max_nz)
    {
        const size_t cnt = size_t(max_nz) - min_nz + 1;
        if (pos + cnt > n)
            return false;
        std::memcpy(bitmap.data() + min_nz, src + pos, cnt);
        pos += cnt;
    }
    // dense index -> word: 0 always, then every word whose bitmap bit is set
    std::vector<uint16_t> lut(65536, 0);
    size_t k = 0;
    for (uint32_t i = 0; i < 65536; i++)
        if (i == 0 || (bitmap[i >> 3] >> (i & 7) & 1))
            lut[k++] = uint16_t(i);
    const uint16_t max_value = uint16_t(k - 1);
    if (pos + 4 > n)
        return false;
    const int32_t length = int32_t(le32(src + pos));
    pos += 4;
    if (length < 0 || size_t(length) > n - pos)
        return false;
    std::vector<uint16_t> words(total);
    if (!huffman_decode(src + pos, size_t(length), words.data(), total))
        return false;
    size_t start = 0;
    std::vector<size_t> plane(words_per_sample.size());
    for (size_t c = 0; c < words_per_sample.size(); c++)
    {
        const int s = words_per_sample[c];
        plane[c] = start;
        for (int j = 0; j < s; j++)
            wavelet_decode(words.data() + start + j, w, s, lines, w * s, max_value);
        start += size_t(w) * size_t(lines) * size_t(s);
    }
    for (uint16_t &v : words)
        v = lut[v];
    uint8_t *o = out;
    for (int y = 0; y < lines; y++)
        for (size_t c = 0; c < words_per_sample.size(); c++)
        {
            const size_t cnt = size_t(w) * size_t(words_per_sample[c]);
            const uint16_t *s = words.data() + plane[c] + size_t(y) * cnt;
            for (size_t i = 0; i < cnt; i++)
            {
                *o++ = uint8_t(s[i]);
                *o++ = uint8_t(s[i] >> 8);
            }
        }
    return true;
}
} // namespace piz

bool exr_decode(const uint8_t *d, size_t n, int &width, int &height, int &channels, std::vector<float> &result,
                isti_status &status, std::string &err)
{
    status = ISTI_ERR_INVALID_ARG;
    if (n < 8 || le32(d) != 20000630u)
        return err = "exr: not an OpenEXR file", false;
    const uint32_t version = le32(d + 4);
    if ((version & 0xff) != 2)
        return err = "exr: unsupported version", false;
    if (version & (0x800u | 0x1000u))
        return status = ISTI_ERR_UNSUPPORTED, err = "exr: multi-part and deep files are not supported", false;
    if (version & 0x200u)
        return status = ISTI_ERR_UNSUPPORTED, err = "exr: tiled files are not supported", false;

    size_t pos = 8;
    auto read_str = [&](std::string &s) {
        const size_t start = pos;
        while (pos < n && d[pos])
            pos++;
        if (pos >= n)
            return false;
        s.assign(reinterpret_cast<const char *>(d + start), pos - start);
        pos++;
        return true;
    };
    std::vector<ExrChannel> chans;
    int compression = -1;
    int32_t box[4] = {0, 0, -1, -1};
    bool have_box = false;
    for (;;)
    {
        std::string name, type;
        if (!read_str(name))
            return err = "exr: truncated header", false;
        if (name.empty())
            break;
        if (!read_str(type) || pos + 4 > n)
            return err = "exr: truncated header", false;
        const uint32_t size = le32(d + pos);
        pos += 4;
        if (size > n - pos)
            return err = "exr: truncated header", false;
        const uint8_t *v = d + pos;
        if (name == "channels" && type == "chlist")
        {
            size_t q = 0;
            while (q < size && v[q])
            {
                const size_t s0 = q;
                while (q < size && v[q])
                    q++;
                if (q + 17 > size)
                    return err = "exr: bad channel list", false;
                ExrChannel c;
                c.name.assign(reinterpret_cast<const char *>(v + s0), q - s0);
                q++;
                c.type = int(le32(v + q));
                const int32_t xs = int32_t(le32(v + q + 8)), ys = int32_t(le32(v + q + 12));
                q += 16;
                if (c.type < 0 || c.type > 2)
                    return err = "exr: bad channel pixel type", false;
                if (xs != 1 || ys != 1)
                    return status = ISTI_ERR_UNSUPPORTED, err = "exr: subsampled channels are not supported", false;
                chans.push_back(c);
            }
        }
        else if (name == "compression" && size >= 1)
            compression = v[0];
        else if (name == "dataWindow" && type == "box2i" && size >= 16)
        {
            for (int k = 0; k < 4; k++)
                box[k] = int32_t(le32(v + 4 * k));
            have_box = true;
        }
        else if (name == "tiles")
            return status = ISTI_ERR_UNSUPPORTED, err = "exr: tiled files are not supported", false;
        pos += size;
    }
    if (chans.empty() || !have_box || compression < 0)
        return err = "exr: header lacks channels, dataWindow or compression", false;
    int lines_per_block;
    switch (compression)
    {
    case 0:
    case 1:
    case 2: lines_per_block = 1; break;
    case 3: lines_per_block = 16; break;
    case 4: lines_per_block = 32; break;
    default: return status = ISTI_ERR_UNSUPPORTED, err = "exr: compression " + std::to_string(compression) + " is not supported", false;
    }
    const int64_t w64 = int64_t(box[2]) - box[0] + 1, h64 = int64_t(box[3]) - box[1] + 1;
    if (w64 <= 0 || h64 <= 0 || w64 > (1 << 24) || h64 > (1 << 24))
        return err = "exr: bad data window", false;
    const int w = int(w64), h = int(h64);

    // LoadEXR's channel selection: names of the default layer (no '.', or a
    // leading '.'); one channel -> grey; otherwise R, G, B (and A) among the
    // first four of them.
    struct LayerCh { int index; std::string name; };
    std::vector<LayerCh> layer;
    for (size_t c = 0; c < chans.size(); c++)
    {
        const std::string &nm = chans[c].name;
        const size_t dot = nm.find_last_of('.');
        if (dot != std::string::npos)
        {
            if (dot != 0)
                continue;
            layer.push_back({int(c), nm.substr(1)});
        }
        else
            layer.push_back({int(c), nm});
    }
    if (layer.empty())
        return err = "exr: no channel in the default layer", false;
    int sel[4] = {-1, -1, -1, -1};
    const size_t look = layer.size() < 4 ? layer.size() : 4;
    for (size_t c = 0; c < look; c++)
    {
        const std::string &nm = layer[c].name;
        if (nm == "R") sel[0] = layer[c].index;
        else if (nm == "G") sel[1] = layer[c].index;
        else if (nm == "B") sel[2] = layer[c].index;
        else if (nm == "A") sel[3] = layer[c].index;
    }
    const bool grey = layer.size() == 1;
    if (grey)
        sel[0] = layer[0].index;
    else if (sel[0] < 0 || sel[1] < 0 || sel[2] < 0)
        return err = std::string("exr: ") + (sel[0] < 0 ? "R" : sel[1] < 0 ? "G" : "B") + " channel not found", false;
    channels = grey ? 1 : 4;

    // bytes of one scan line of every channel, in header order
    std::vector<size_t> ch_off(chans.size());
    size_t line_bytes = 0;
    for (size_t c = 0; c < chans.size(); c++)
    {
        ch_off[c] = line_bytes;
        line_bytes += size_t(w) * (chans[c].type == EXR_HALF ? 2 : 4);
    }
    std::vector<int> piz_words(chans.size()); // 16-bit words per sample, for PIZ
    for (size_t c = 0; c < chans.size(); c++)
        piz_words[c] = chans[c].type == EXR_HALF ? 1 : 2;
    const int n_blocks = (h + lines_per_block - 1) / lines_per_block;
    if (pos + size_t(n_blocks) * 8 > n)
        return err = "exr: truncated offset table", false;
    result.assign(size_t(w) * h * channels, 0.0f);
    if (!grey && sel[3] < 0)
        for (size_t i = 0; i < size_t(w) * h; i++)
            result[4 * i + 3] = 1.0f;

    // chunk table first (in file order, the first bad entry is the error), then the chunks,
    // on several threads when there are many and no two chunks claim the same lines
    struct Chunk
    {
        const uint8_t *src;
        uint32_t size;
        int64_t row0;
        int lines;
    };
    const size_t nb = size_t(n_blocks);
    std::vector<Chunk> chunks(nb);
    std::vector<uint8_t> claimed(nb, 0);
    bool unique = true;
    for (int bi = 0; bi < n_blocks; bi++)
    {
        const uint64_t off = le64(d + pos + 8 * size_t(bi));
        if (off + 8 > n)
            return err = "exr: bad chunk offset", false;
        const int32_t y = int32_t(le32(d + off));
        const uint32_t size = le32(d + off + 4);
        if (size > n - off - 8)
            return err = "exr: truncated chunk", false;
        const int64_t row0 = int64_t(y) - box[1];
        if (row0 < 0 || row0 >= h || row0 % lines_per_block != 0)
            return err = "exr: bad chunk line number", false;
        uint8_t &c = claimed[size_t(row0 / lines_per_block)];
        unique = unique && !c;
        c = 1;
        chunks[size_t(bi)] = Chunk{d + off + 8, size, row0, int(std::min<int64_t>(lines_per_block, h - row0))};
    }
    std::vector<std::string> errors(nb);
    auto decode_chunk = [&](int bi, std::vector<uint8_t> &block, std::vector<uint8_t> &tmp) -> bool {
        const Chunk &ck = chunks[size_t(bi)];
        std::string &e = errors[size_t(bi)];
        const int lines = ck.lines;
        const size_t raw = line_bytes * size_t(lines);
        const uint8_t *src = ck.src;
        const uint32_t size = ck.size;
        block.resize(raw);
        if (size == raw || compression == 0)
        {
            if (size != raw)
                return e = "exr: uncompressed chunk has the wrong size", false;
            std::memcpy(block.data(), src, raw);
        }
        else if (compression == 1)
        {
            tmp.resize(raw);
            if (!exr_unrle(src, size, tmp.data(), raw))
                return e = "exr: corrupt RLE chunk", false;
            exr_unpredict(tmp, block.data());
        }
        else if (compression == 4)
        {
            if (!piz::decompress(src, size, piz_words, w, lines, block.data()))
                return e = "exr: corrupt PIZ chunk", false;
        }
        else
        {
            tmp.clear();
            tmp.reserve(raw);
            if (!zlib_decompress(src, size, tmp, raw, e))
                return e = "exr: " + e, false;
            if (tmp.size() != raw)
                return e = "exr: ZIP chunk has the wrong size", false;
            exr_unpredict(tmp, block.data());
        }
        const int64_t row0 = ck.row0;
        for (int l = 0; l < lines; l++)
        {
            const uint8_t *line = block.data() + size_t(l) * line_bytes;
            float *dst = result.data() + (size_t(row0) + size_t(l)) * size_t(w) * size_t(channels);
            for (int k = 0; k < channels; k++)
            {
                const int c = sel[k];
                if (c < 0)
                    continue;
                const uint8_t *s = line + ch_off[size_t(c)];
                for (int x = 0; x < w; x++)
                {
                    uint32_t bits;
                    if (chans[size_t(c)].type == EXR_HALF)
                        bits = half_bits_to_float_bits(uint16_t(s[2 * x] | s[2 * x + 1] << 8));
                    else
                        bits = le32(s + 4 * size_t(x)); // FLOAT, or UINT whose bits LoadEXR hands over as they are
                    std::memcpy(&dst[size_t(x) * size_t(channels) + size_t(k)], &bits, 4);
                }
            }
        }
        return true;
    };
    const int n_threads = unique ? decode_threads(n_blocks) : 1;
    std::atomic<int> next{0};
    std::atomic<bool> failed{false};
    auto worker = [&]() {
        std::vector<uint8_t> block, tmp;
        for (int bi; !failed.load(std::memory_order_relaxed) && (bi = next.fetch_add(1)) < n_blocks;)
            if (!decode_chunk(bi, block, tmp))
                failed = true;
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < n_threads; t++)
        pool.emplace_back(worker);
    worker();
    for (std::thread &t : pool)
        t.join();
    if (failed)
        for (const std::string &e : errors) // the first failing chunk in file order
            if (!e.empty())
                return err = e, false;
    width = w;
    height = h;
    status = ISTI_OK;
    return true;
}

void put_le32(std::vector<uint8_t> &o, uint32_t v)
{
    for (int s = 0; s < 32; s += 8)
        o.push_back(uint8_t(v >> s));
}

void put_attr(std::vector<uint8_t> &o, const char *name, const char *type, const std::vector<uint8_t> &value)
{
    o.insert(o.end(), name, name + std::strlen(name) + 1);
    o.insert(o.end(), type, type + std::strlen(type) + 1);
    put_le32(o, uint32_t(value.size()));
    o.insert(o.end(), value.begin(), value.end());
}

// Scan-line OpenEXR file of FLOAT channels: one channel named "Y", or RGBA
// stored as the channels A, B, G, R (the format's alphabetical order).
// compression 0 = NONE, 3 = ZIP (16 lines per block, predictor + split).
void exr_encode(int w, int h, int channels, const float *px, int compression, std::vector<uint8_t> &o)
{
    o.clear();
    put_le32(o, 20000630u);
    put_le32(o, 2);
    static const char *const RGBA_NAMES[4] = {"A", "B", "G", "R"};
    static const int RGBA_SRC[4] = {3, 2, 1, 0}; // channel k of the file <- component of the pixel
    std::vector<uint8_t> v;
    for (int k = 0; k < channels; k++)
    {
        const char *name = channels == 1 ? "Y" : RGBA_NAMES[k];
        v.insert(v.end(), name, name + std::strlen(name) + 1);
        put_le32(v, 2); // FLOAT
        for (int z = 0; z < 4; z++)
            v.push_back(0); // pLinear + reserved
        put_le32(v, 1);
        put_le32(v, 1);
    }
    v.push_back(0);
    put_attr(o, "channels", "chlist", v);
    put_attr(o, "compression", "compression", {uint8_t(compression)});
    v.clear();
    for (int32_t x : {0, 0, w - 1, h - 1})
        put_le32(v, uint32_t(x));
    put_attr(o, "dataWindow", "box2i", v);
    put_attr(o, "displayWindow", "box2i", v);
    put_attr(o, "lineOrder", "lineOrder", {0});
    v.clear();
    put_le32(v, 0x3f800000u);
    put_attr(o, "pixelAspectRatio", "float", v);
    v.assign(8, 0);
    put_attr(o, "screenWindowCenter", "v2f", v);
    v.clear();
    put_le32(v, 0x3f800000u);
    put_attr(o, "screenWindowWidth", "float", v);
    o.push_back(0); // end of header

    const int lpb = compression == 3 ? 16 : 1;
    const int n_blocks = (h + lpb - 1) / lpb;
    const size_t table = o.size();
    o.resize(table + 8 * size_t(n_blocks));
    std::vector<uint8_t> raw, tmp, z;
    for (int b = 0; b < n_blocks; b++)
    {
        const int y0 = b * lpb, lines = std::min(lpb, h - y0);
        raw.clear();
        for (int l = 0; l < lines; l++)
            for (int k = 0; k < channels; k++)
                for (int x = 0; x < w; x++)
                {
                    uint32_t bits;
                    const int comp = channels == 1 ? 0 : RGBA_SRC[k];
                    std::memcpy(&bits, &px[(size_t(y0 + l) * size_t(w) + size_t(x)) * size_t(channels) + size_t(comp)], 4);
                    for (int s = 0; s < 32; s += 8)
                        raw.push_back(uint8_t(bits >> s));
                }
        const std::vector<uint8_t> *payload = &raw;
        if (compression == 3)
        {
            // split even/odd bytes, then the byte predictor, then zlib
            tmp.resize(raw.size());
            const size_t half = (raw.size() + 1) / 2;
            for (size_t i = 0; i < raw.size(); i++)
                tmp[(i & 1) ? half + i / 2 : i / 2] = raw[i];
            for (size_t i = tmp.size(); i-- > 1;)
                tmp[i] = uint8_t(int(tmp[i]) - int(tmp[i - 1]) + 128 + 256);
            z.clear();
            zlib_compress(tmp.data(), tmp.size(), z);
            if (z.size() < raw.size())
                payload = &z;
        }
        const uint64_t off = o.size();
        for (int s = 0; s < 64; s += 8)
            o[table + 8 * size_t(b) + size_t(s / 8)] = uint8_t(off >> s);
        put_le32(o, uint32_t(y0));
        put_le32(o, uint32_t(payload->size()));
        o.insert(o.end(), payload->begin(), payload->end());
    }
}

template <class T>
T *to_malloc(const std::vector<T> &v)
{
    T *p = static_cast<T *>(std::malloc(v.size() * sizeof(T) + 1));
    if (p && !v.empty())
        std::memcpy(p, v.data(), v.size() * sizeof(T));
    return p;
}

} // namespace

extern "C" {

isti_status isti_zlib_decompress(const uint8_t *src, size_t src_size, uint8_t **out, size_t *out_size)
{
    if (!src || !out || !out_size)
        return set_error(ISTI_ERR_INVALID_ARG, "isti_zlib_decompress: null argument");
    std::vector<uint8_t> o;
    std::string err;
    if (!zlib_decompress(src, src_size, o, size_t(1) << 40, err))
        return set_error(ISTI_ERR_INVALID_ARG, err);
    if (!(*out = to_malloc(o)))
        return set_error(ISTI_ERR_OOM, "isti_zlib_decompress: out of host memory");
    *out_size = o.size();
    return ISTI_OK;
}

isti_status isti_png_decode_memory(const uint8_t *data, size_t size, int32_t *width, int32_t *height, uint8_t **rgba)
{
    if (!data || !width || !height || !rgba)
        return set_error(ISTI_ERR_INVALID_ARG, "isti_png_decode: null argument");
    uint32_t w = 0, h = 0;
    std::vector<uint8_t> px;
    std::string err;
    if (!png_decode(data, size, w, h, px, err))
        return set_error(ISTI_ERR_INVALID_ARG, err);
    if (!(*rgba = to_malloc(px)))
        return set_error(ISTI_ERR_OOM, "isti_png_decode: out of host memory");
    *width = int32_t(w);
    *height = int32_t(h);
    return ISTI_OK;
}

isti_status isti_png_decode_file(const char *path, int32_t *width, int32_t *height, uint8_t **rgba)
{
    std::vector<uint8_t> bytes;
    std::string err;
    if (!read_file(path, bytes, err))
        return set_error(ISTI_ERR_INVALID_ARG, err);
    const isti_status s = isti_png_decode_memory(bytes.data(), bytes.size(), width, height, rgba);
    if (s != ISTI_OK)
        set_error(s, std::string(isti_last_error()) + " (" + path + ")");
    return s;
}

isti_status isti_png_encode_memory(int32_t width, int32_t height, int32_t channels, const uint8_t *pixels, uint8_t **png,
                                   size_t *png_size)
{
    if (!pixels || !png || !png_size || width <= 0 || height <= 0 || (channels != 3 && channels != 4))
        return set_error(ISTI_ERR_INVALID_ARG, "isti_png_encode: bad argument");
    std::vector<uint8_t> out;
    png_encode(uint32_t(width), uint32_t(height), channels, pixels, out);
    if (!(*png = to_malloc(out)))
        return set_error(ISTI_ERR_OOM, "isti_png_encode: out of host memory");
    *png_size = out.size();
    return ISTI_OK;
}

isti_status isti_png_encode_file(const char *path, int32_t width, int32_t height, int32_t channels, const uint8_t *pixels)
{
    if (!pixels || width <= 0 || height <= 0 || (channels != 3 && channels != 4))
        return set_error(ISTI_ERR_INVALID_ARG, "isti_png_encode: bad argument");
    std::vector<uint8_t> out;
    png_encode(uint32_t(width), uint32_t(height), channels, pixels, out);
    std::string err;
    if (!write_file(path, out, err))
        return set_error(ISTI_ERR_INVALID_ARG, err);
    return ISTI_OK;
}

isti_status isti_exr_decode_memory(const uint8_t *bytes, size_t size, int32_t *width, int32_t *height, int32_t *channels,
                                   float **data)
{
    if (!bytes || !width || !height || !channels || !data)
        return set_error(ISTI_ERR_INVALID_ARG, "isti_exr_decode: null argument");
    int w = 0, h = 0, c = 0;
    std::vector<float> px;
    std::string err;
    isti_status st;
    if (!exr_decode(bytes, size, w, h, c, px, st, err))
        return set_error(st, err);
    if (!(*data = to_malloc(px)))
        return set_error(ISTI_ERR_OOM, "isti_exr_decode: out of host memory");
    *width = w;
    *height = h;
    *channels = c;
    return ISTI_OK;
}

isti_status isti_exr_decode_file(const char *path, int32_t *width, int32_t *height, int32_t *channels, float **data)
{
    std::vector<uint8_t> bytes;
    std::string err;
    if (!read_file(path, bytes, err))
        return set_error(ISTI_ERR_INVALID_ARG, err);
    const isti_status s = isti_exr_decode_memory(bytes.data(), bytes.size(), width, height, channels, data);
    if (s != ISTI_OK)
        set_error(s, std::string(isti_last_error()) + " (" + path + ")");
    return s;
}

isti_status isti_exr_encode_file(const char *path, int32_t width, int32_t height, int32_t channels, const float *data,
                                 int32_t compression)
{
    if (!data || width <= 0 || height <= 0 || (channels != 1 && channels != 4) || (compression != 0 && compression != 3))
        return set_error(ISTI_ERR_INVALID_ARG, "isti_exr_encode: bad argument");
    std::vector<uint8_t> out;
    exr_encode(width, height, channels, data, compression, out);
    std::string err;
    if (!write_file(path, out, err))
        return set_error(ISTI_ERR_INVALID_ARG, err);
    return ISTI_OK;
}

void isti_image_free(void *p) { std::free(p); }

} // extern "C"

void isti::set_decode_threads(int n) { t_decode_threads = n; }
