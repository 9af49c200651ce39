// Image codecs: inflate, zlib, PNG decoding (see image_io.h).
//
// Inflate follows RFC 1951: stored, fixed-Huffman and dynamic-Huffman
// blocks; each canonical Huffman code is decoded through one table indexed by
// the next maxLen input bits (bit-reversed codes), so a symbol costs one
// lookup. Every read is bounds-checked; a stream that runs past its input,
// refers back before the start of the output or over-subscribes a code is an
// error, never undefined behaviour.
#include "image_io.h"

#include <cstring>

namespace optimg {

namespace {

struct CrcTable {
    uint32_t t[256];
    CrcTable()
    {
        for (uint32_t n = 0; n < 256; ++n) {
            uint32_t c = n;
            for (int k = 0; k < 8; ++k)
                c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[n] = c;
        }
    }
};
const CrcTable kCrc;

// RFC 1951 3.2.5: length codes 257..285 and distance codes 0..29.
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// Order of the code-length code lengths in a dynamic block header.
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

struct BitReader {
    const uint8_t *p;
    size_t n, pos = 0;
    uint64_t buf = 0;
    int cnt = 0;
    size_t overrun = 0;  // zero bytes supplied past the end
    BitReader(const uint8_t *d, size_t len) : p(d), n(len) {}
    void refill()
    {
        while (cnt <= 56) {
            uint64_t b = 0;
            if (pos < n)
                b = p[pos];
            else
                ++overrun;
            ++pos;
            buf |= b << cnt;
            cnt += 8;
        }
    }
    uint32_t peek(int k) { return (uint32_t)(buf & ((1ull << k) - 1)); }
    void drop(int k)
    {
        buf >>= k;
        cnt -= k;
    }
    uint32_t bits(int k)
    {
        if (k == 0)
            return 0;
        if (cnt < k)
            refill();
        uint32_t v = peek(k);
        drop(k);
        return v;
    }
    // Bytes consumed past the end of the input, counting only whole bytes
    // whose bits were actually used.
    bool exhausted() const
    {
        const size_t unusedBytes = (size_t)cnt / 8;
        return overrun > unusedBytes;
    }
    void alignByte() { drop(cnt & 7); }
};

// Canonical Huffman decoding table: entry = symbol | length << 9 (0 = no code).
struct Huffman {
    std::vector<uint16_t> table;
    int maxLen = 0;
    bool build(const uint8_t *lens, int num)
    {
        int count[16] = {0};
        maxLen = 0;
        for (int s = 0; s < num; ++s) {
            count[lens[s]]++;
            if (lens[s] > maxLen)
                maxLen = lens[s];
        }
        count[0] = 0;
        int left = 1;
        for (int l = 1; l <= 15; ++l) {
            left = (left << 1) - count[l];
            if (left < 0)
                return false;  // over-subscribed
        }
        int next[16];
        int code = 0;
        for (int l = 1; l <= 15; ++l) {
            code = (code + count[l - 1]) << 1;
            next[l] = code;
        }
        if (maxLen == 0)
            maxLen = 1;
        table.assign((size_t)1 << maxLen, 0);
        for (int s = 0; s < num; ++s) {
            const int l = lens[s];
            if (!l)
                continue;
            const int c = next[l]++;
            int rev = 0;
            for (int k = 0; k < l; ++k)
                rev |= ((c >> k) & 1) << (l - 1 - k);
            for (int f = rev; f < (1 << maxLen); f += 1 << l)
                table[f] = (uint16_t)(s | (l << 9));
        }
        return true;
    }
    // -1 when the bits match no code (incomplete code).
    int decode(BitReader &br) const
    {
        if (br.cnt < maxLen)
            br.refill();
        const uint16_t e = table[br.peek(maxLen)];
        if (!e)
            return -1;
        br.drop(e >> 9);
        return e & 511;
    }
};

bool inflateBlock(BitReader &br, const Huffman &lit, const Huffman &dist, std::vector<uint8_t> &out, size_t maxOut,
                  std::string &err)
{
    while (true) {
        const int sym = lit.decode(br);
        if (sym < 0) {
            err = "invalid literal/length code";
            return false;
        }
        if (sym < 256) {
            if (out.size() >= maxOut) {
                err = "output larger than expected";
                return false;
            }
            out.push_back((uint8_t)sym);
            continue;
        }
        if (sym == 256)
            return true;
        if (sym > 285) {
            err = "invalid length symbol";
            return false;
        }
        const size_t len = kLenBase[sym - 257] + br.bits(kLenExtra[sym - 257]);
        const int ds = dist.decode(br);
        if (ds < 0 || ds > 29) {
            err = "invalid distance code";
            return false;
        }
        const size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
        if (d > out.size()) {
            err = "distance before start of output";
            return false;
        }
        if (out.size() + len > maxOut) {
            err = "output larger than expected";
            return false;
        }
        size_t from = out.size() - d;
        for (size_t k = 0; k < len; ++k)
            out.push_back(out[from + k]);
        if (br.exhausted()) {
            err = "unexpected end of deflate data";
            return false;
        }
    }
}

}  // namespace

uint32_t crc32(const uint8_t *p, size_t n, uint32_t crc)
{
    crc = ~crc;
    for (size_t i = 0; i < n; ++i)
        crc = kCrc.t[(crc ^ p[i]) & 0xFF] ^ (crc >> 8);
    return ~crc;
}

uint32_t adler32(const uint8_t *p, size_t n, uint32_t a)
{
    uint32_t s1 = a & 0xFFFF, s2 = a >> 16;
    while (n) {
        size_t k = n < 5552 ? n : 5552;
        n -= k;
        while (k--) {
            s1 += *p++;
            s2 += s1;
        }
        s1 %= 65521;
        s2 %= 65521;
    }
    return (s2 << 16) | s1;
}

bool inflate(const uint8_t *in, size_t n, std::vector<uint8_t> &out, size_t maxOut, std::string &err)
{
    BitReader br(in, n);
    Huffman fixedLit, fixedDist;
    bool fixedBuilt = false;
    while (true) {
        const uint32_t final = br.bits(1);
        const uint32_t type = br.bits(2);
        if (type == 0) {
            br.alignByte();
            const uint32_t len = br.bits(16), nlen = br.bits(16);
            if ((len ^ 0xFFFF) != nlen) {
                err = "stored block length check failed";
                return false;
            }
            if (out.size() + len > maxOut) {
                err = "output larger than expected";
                return false;
            }
            // Whatever whole bytes remain in the bit buffer come first.
            for (uint32_t k = 0; k < len; ++k)
                out.push_back((uint8_t)br.bits(8));
            if (br.exhausted()) {
                err = "unexpected end of stored block";
                return false;
            }
        } else if (type == 1) {
            if (!fixedBuilt) {
                uint8_t l[288], d[30];
                for (int s = 0; s < 288; ++s)
                    l[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
                for (int s = 0; s < 30; ++s)
                    d[s] = 5;
                fixedLit.build(l, 288);
                fixedDist.build(d, 30);
                fixedBuilt = true;
            }
            if (!inflateBlock(br, fixedLit, fixedDist, out, maxOut, err))
                return false;
        } else if (type == 2) {
            const int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
            if (hlit > 286 || hdist > 30) {
                err = "bad dynamic block header";
                return false;
            }
            uint8_t cl[19] = {0};
            for (int k = 0; k < hclen; ++k)
                cl[kClOrder[k]] = (uint8_t)br.bits(3);
            Huffman clh;
            if (!clh.build(cl, 19)) {
                err = "bad code-length code";
                return false;
            }
            uint8_t lens[286 + 30] = {0};
            int k = 0;
            while (k < hlit + hdist) {
                const int sym = clh.decode(br);
                if (sym < 0) {
                    err = "invalid code-length symbol";
                    return false;
                }
                if (sym < 16) {
                    lens[k++] = (uint8_t)sym;
                    continue;
                }
                int rep;
                uint8_t val = 0;
                if (sym == 16) {
                    if (k == 0) {
                        err = "repeat with no previous length";
                        return false;
                    }
                    val = lens[k - 1];
                    rep = 3 + (int)br.bits(2);
                } else if (sym == 17) {
                    rep = 3 + (int)br.bits(3);
                } else {
                    rep = 11 + (int)br.bits(7);
                }
                if (k + rep > hlit + hdist) {
                    err = "code lengths overflow";
                    return false;
                }
                while (rep--)
                    lens[k++] = val;
            }
            if (lens[256] == 0) {
                err = "no end-of-block code";
                return false;
            }
            Huffman lit, dist;
            if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist)) {
                err = "over-subscribed Huffman code";
                return false;
            }
            if (!inflateBlock(br, lit, dist, out, maxOut, err))
                return false;
        } else {
            err = "invalid block type";
            return false;
        }
        if (br.exhausted()) {
            err = "unexpected end of deflate data";
            return false;
        }
        if (final)
            return true;
    }
}

bool zlibDecompress(const uint8_t *in, size_t n, std::vector<uint8_t> &out, size_t maxOut, std::string &err)
{
    if (n < 6) {
        err = "zlib stream too short";
        return false;
    }
    const uint8_t cmf = in[0], flg = in[1];
    if ((cmf & 0x0F) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0) {
        err = "bad zlib header";
        return false;
    }
    if (flg & 0x20) {
        err = "zlib preset dictionary not supported";
        return false;
    }
    if (!inflate(in + 2, n - 6, out, maxOut, err))
        return false;
    const uint8_t *t = in + n - 4;
    const uint32_t want = ((uint32_t)t[0] << 24) | ((uint32_t)t[1] << 16) | ((uint32_t)t[2] << 8) | t[3];
    if (adler32(out.data(), out.size()) != want) {
        err = "zlib Adler-32 mismatch";
        return false;
    }
    return true;
}

// ------------------------------------------------------------------ PNG

namespace {

uint32_t be32(const uint8_t *p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

uint8_t paeth(int a, int b, int c)
{
    const int p = a + b - c;
    const int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    if (pa <= pb && pa <= pc)
        return (uint8_t)a;
    return (uint8_t)(pb <= pc ? b : c);
}

// Reverses the per-row filters of one (sub-)image in place: `data` holds
// rows of 1 + rowBytes bytes; the unfiltered rows go to `rows`.
bool unfilter(const uint8_t *data, uint32_t h, size_t rowBytes, int bpp, std::vector<uint8_t> &rows, std::string &err)
{
    rows.assign((size_t)h * rowBytes, 0);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t ft = data[(size_t)y * (rowBytes + 1)];
        const uint8_t *src = data + (size_t)y * (rowBytes + 1) + 1;
        uint8_t *cur = rows.data() + (size_t)y * rowBytes;
        const uint8_t *prev = y ? cur - rowBytes : nullptr;
        for (size_t i = 0; i < rowBytes; ++i) {
            const int a = i >= (size_t)bpp ? cur[i - bpp] : 0;
            const int b = prev ? prev[i] : 0;
            const int c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
            int v = src[i];
            switch (ft) {
            case 0: break;
            case 1: v += a; break;
            case 2: v += b; break;
            case 3: v += (a + b) >> 1; break;
            case 4: v += paeth(a, b, c); break;
            default: err = "bad PNG filter type"; return false;
            }
            cur[i] = (uint8_t)v;
        }
    }
    return true;
}

struct PngInfo {
    uint32_t w, h;
    int depth, colour, channels;
    uint8_t palette[256][4];
    int paletteSize = 0;
    bool hasKey = false;
    uint16_t key[3] = {0, 0, 0};
};

// Raw sample k of pixel x in an unfiltered row (any bit depth).
inline uint32_t sample(const uint8_t *row, uint32_t idx, int depth)
{
    switch (depth) {
    case 8: return row[idx];
    case 16: return ((uint32_t)row[2 * idx] << 8) | row[2 * idx + 1];
    default: {
        const uint32_t bit = idx * (uint32_t)depth;
        const uint32_t shift = 8 - depth - (bit & 7);
        return (row[bit >> 3] >> shift) & ((1u << depth) - 1);
    }
    }
}

inline uint8_t to8(uint32_t v, int depth)
{
    if (depth == 16)
        return (uint8_t)(v >> 8);
    if (depth == 8)
        return (uint8_t)v;
    return (uint8_t)(v * (255u / ((1u << depth) - 1)));
}

void emitRow(const PngInfo &pi, const uint8_t *row, uint32_t cols, uint8_t *dst, size_t dstStride)
{
    for (uint32_t x = 0; x < cols; ++x) {
        uint8_t *o = dst + (size_t)x * dstStride;
        const uint32_t base = x * (uint32_t)pi.channels;
        switch (pi.colour) {
        case 0: {
            const uint32_t g = sample(row, base, pi.depth);
            o[0] = o[1] = o[2] = to8(g, pi.depth);
            o[3] = (pi.hasKey && g == pi.key[0]) ? 0 : 255;
            break;
        }
        case 2: {
            const uint32_t r = sample(row, base, pi.depth), g = sample(row, base + 1, pi.depth),
                           b = sample(row, base + 2, pi.depth);
            o[0] = to8(r, pi.depth);
            o[1] = to8(g, pi.depth);
            o[2] = to8(b, pi.depth);
            o[3] = (pi.hasKey && r == pi.key[0] && g == pi.key[1] && b == pi.key[2]) ? 0 : 255;
            break;
        }
        case 3: {
            const uint32_t i = sample(row, base, pi.depth);
            memcpy(o, pi.palette[i], 4);
            break;
        }
        case 4:
            o[0] = o[1] = o[2] = to8(sample(row, base, pi.depth), pi.depth);
            o[3] = to8(sample(row, base + 1, pi.depth), pi.depth);
            break;
        default:
            for (int c = 0; c < 4; ++c)
                o[c] = to8(sample(row, base + c, pi.depth), pi.depth);
            break;
        }
    }
}

}  // namespace

bool isPng(const uint8_t *p, size_t n)
{
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    return n >= 8 && memcmp(p, sig, 8) == 0;
}

bool decodePng(const uint8_t *p, size_t n, Image &img, std::string &err)
{
    if (!isPng(p, n)) {
        err = "not a PNG file";
        return false;
    }
    PngInfo pi{};
    bool haveHeader = false, interlaced = false;
    std::vector<uint8_t> idat;
    size_t pos = 8;
    bool ended = false;
    while (pos + 12 <= n) {
        const uint32_t len = be32(p + pos);
        if (len > n - pos - 12) {
            err = "truncated PNG chunk";
            return false;
        }
        const uint8_t *type = p + pos + 4, *data = p + pos + 8;
        if (crc32(type, (size_t)len + 4) != be32(data + len)) {
            err = "PNG chunk CRC mismatch";
            return false;
        }
        const bool critical = !(type[0] & 0x20);
        if (!memcmp(type, "IHDR", 4)) {
            if (len != 13) {
                err = "bad IHDR";
                return false;
            }
            pi.w = be32(data);
            pi.h = be32(data + 4);
            pi.depth = data[8];
            pi.colour = data[9];
            if (data[10] != 0 || data[11] != 0 || data[12] > 1) {
                err = "unsupported PNG compression, filter or interlace method";
                return false;
            }
            interlaced = data[12] == 1;
            static const int chans[7] = {1, 0, 3, 1, 2, 0, 4};
            const int d = pi.depth;
            bool ok = pi.colour <= 6 && chans[pi.colour] != 0;
            if (ok) {
                pi.channels = chans[pi.colour];
                if (pi.colour == 0)
                    ok = d == 1 || d == 2 || d == 4 || d == 8 || d == 16;
                else if (pi.colour == 3)
                    ok = d == 1 || d == 2 || d == 4 || d == 8;
                else
                    ok = d == 8 || d == 16;
            }
            if (!ok) {
                err = "invalid PNG colour type / bit depth";
                return false;
            }
            if (pi.w == 0 || pi.h == 0 || (uint64_t)pi.w * pi.h > (1ull << 28)) {
                err = "PNG dimensions out of range";
                return false;
            }
            haveHeader = true;
        } else if (!haveHeader) {
            err = "PNG chunk before IHDR";
            return false;
        } else if (!memcmp(type, "PLTE", 4)) {
            if (len % 3 || len / 3 > 256 || len == 0) {
                err = "bad PLTE";
                return false;
            }
            pi.paletteSize = (int)(len / 3);
            for (int i = 0; i < pi.paletteSize; ++i) {
                pi.palette[i][0] = data[3 * i];
                pi.palette[i][1] = data[3 * i + 1];
                pi.palette[i][2] = data[3 * i + 2];
                pi.palette[i][3] = 255;
            }
        } else if (!memcmp(type, "tRNS", 4)) {
            if (pi.colour == 3) {
                if (len > (uint32_t)pi.paletteSize) {
                    err = "bad tRNS";
                    return false;
                }
                for (uint32_t i = 0; i < len; ++i)
                    pi.palette[i][3] = data[i];
            } else if (pi.colour == 0 && len == 2) {
                pi.hasKey = true;
                pi.key[0] = (uint16_t)((data[0] << 8) | data[1]);
            } else if (pi.colour == 2 && len == 6) {
                pi.hasKey = true;
                for (int c = 0; c < 3; ++c)
                    pi.key[c] = (uint16_t)((data[2 * c] << 8) | data[2 * c + 1]);
            } else {
                err = "bad tRNS";
                return false;
            }
        } else if (!memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), data, data + len);
        } else if (!memcmp(type, "IEND", 4)) {
            ended = true;
            break;
        } else if (critical) {
            err = "unknown critical PNG chunk";
            return false;
        }
        pos += 12 + (size_t)len;
    }
    if (!haveHeader || !ended || idat.empty()) {
        err = "incomplete PNG";
        return false;
    }
    if (pi.colour == 3 && pi.paletteSize == 0) {
        err = "palette image without PLTE";
        return false;
    }
    const int bitsPerPixel = pi.depth * pi.channels;
    const int bpp = bitsPerPixel >= 8 ? bitsPerPixel / 8 : 1;
    auto rowBytesOf = [&](uint32_t cols) { return ((size_t)cols * bitsPerPixel + 7) / 8; };
    // Adam7 passes: x0, y0, dx, dy.
    static const int adam[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                   {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    size_t expected = 0;
    if (!interlaced) {
        expected = (size_t)pi.h * (rowBytesOf(pi.w) + 1);
    } else {
        for (auto &a : adam) {
            const uint32_t cw = pi.w > (uint32_t)a[0] ? (pi.w - a[0] + a[2] - 1) / a[2] : 0;
            const uint32_t ch = pi.h > (uint32_t)a[1] ? (pi.h - a[1] + a[3] - 1) / a[3] : 0;
            if (cw && ch)
                expected += (size_t)ch * (rowBytesOf(cw) + 1);
        }
    }
    std::vector<uint8_t> raw;
    raw.reserve(expected);
    if (!zlibDecompress(idat.data(), idat.size(), raw, expected, err))
        return false;
    if (raw.size() != expected) {
        err = "PNG image data size mismatch";
        return false;
    }
    img.width = pi.w;
    img.height = pi.h;
    img.rgba.assign((size_t)pi.w * pi.h * 4, 0);
    std::vector<uint8_t> rows;
    if (!interlaced) {
        const size_t rb = rowBytesOf(pi.w);
        if (!unfilter(raw.data(), pi.h, rb, bpp, rows, err))
            return false;
        for (uint32_t y = 0; y < pi.h; ++y)
            emitRow(pi, rows.data() + (size_t)y * rb, pi.w, img.rgba.data() + (size_t)y * pi.w * 4, 4);
        return true;
    }
    size_t off = 0;
    for (auto &a : adam) {
        const uint32_t cw = pi.w > (uint32_t)a[0] ? (pi.w - a[0] + a[2] - 1) / a[2] : 0;
        const uint32_t ch = pi.h > (uint32_t)a[1] ? (pi.h - a[1] + a[3] - 1) / a[3] : 0;
        if (!cw || !ch)
            continue;
        const size_t rb = rowBytesOf(cw);
        if (!unfilter(raw.data() + off, ch, rb, bpp, rows, err))
            return false;
        off += (size_t)ch * (rb + 1);
        for (uint32_t y = 0; y < ch; ++y) {
            const uint32_t oy = (uint32_t)a[1] + y * (uint32_t)a[3];
            emitRow(pi, rows.data() + (size_t)y * rb, cw,
                    img.rgba.data() + ((size_t)oy * pi.w + (uint32_t)a[0]) * 4, (size_t)a[2] * 4);
        }
    }
    return true;
}

}  // namespace optimg
