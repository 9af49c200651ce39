// Image encoders for frame output: DEFLATE / zlib, PNG, Radiance RGBE and
// OpenEXR (see image_io.h). The reference writes output.png through
// stb_image_write, output.hdr through stbi_write_hdr and output.exr through
// OpenEXR's RgbaOutputFile (cu/kernels.cu:35-76, src/renderer.cpp:1001-1026);
// neither library is available, so the formats are written from their
// published specifications (RFC 1950/1951, PNG 1.2, the Radiance picture
// format, the OpenEXR file layout).
//
// DEFLATE: greedy LZ77 over a 32 KB window with 3-byte hash chains (at most
// 32 candidates per position), blocks of up to 32K tokens coded with
// dynamic Huffman codes (lengths limited to 15 by repeatedly halving the
// frequencies), or stored when that is smaller. Large inputs are split into
// pieces compressed on separate host threads; every piece but the last ends
// with an empty stored block, so the pieces concatenate into one stream.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <queue>
#include <thread>

#include "image_io.h"

namespace optimg {

namespace {

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

struct BitWriter {
    std::vector<uint8_t> &out;
    uint64_t buf = 0;
    int cnt = 0;
    explicit BitWriter(std::vector<uint8_t> &o) : out(o) {}
    void put(uint32_t v, int k)
    {
        buf |= (uint64_t)v << cnt;
        cnt += k;
        while (cnt >= 8) {
            out.push_back((uint8_t)buf);
            buf >>= 8;
            cnt -= 8;
        }
    }
    void align()
    {
        if (cnt > 0)
            put(0, 8 - cnt);
    }
};

// Code lengths of a Huffman code for `freq`, limited to maxLen bits. At
// least two symbols get codes, so every code is complete.
void huffmanLengths(const uint32_t *freqIn, int n, int maxLen, uint8_t *lens)
{
    std::vector<uint32_t> freq(freqIn, freqIn + n);
    int used = 0;
    for (int s = 0; s < n; ++s)
        used += freq[s] != 0;
    for (int s = 0; used < 2 && s < n; ++s)
        if (!freq[s]) {
            freq[s] = 1;
            ++used;
        }
    while (true) {
        struct Node {
            uint64_t f;
            int id;
            bool operator>(const Node &o) const { return f != o.f ? f > o.f : id > o.id; }
        };
        std::priority_queue<Node, std::vector<Node>, std::greater<Node>> pq;
        std::vector<int> parent(2 * n, -1);
        for (int s = 0; s < n; ++s)
            if (freq[s])
                pq.push({freq[s], s});
        int next = n;
        while (pq.size() > 1) {
            Node a = pq.top();
            pq.pop();
            Node b = pq.top();
            pq.pop();
            parent[a.id] = parent[b.id] = next;
            pq.push({a.f + b.f, next++});
        }
        int worst = 0;
        for (int s = 0; s < n; ++s) {
            int d = 0;
            if (freq[s])
                for (int p = s; parent[p] >= 0; p = parent[p])
                    ++d;
            lens[s] = (uint8_t)d;
            worst = std::max(worst, d);
        }
        if (worst <= maxLen)
            return;
        for (int s = 0; s < n; ++s)
            if (freq[s])
                freq[s] = (freq[s] >> 1) | 1;
    }
}

// Bit-reversed canonical codes for lengths.
void canonicalCodes(const uint8_t *lens, int n, uint16_t *codes)
{
    int count[16] = {0}, next[16] = {0};
    for (int s = 0; s < n; ++s)
        count[lens[s]]++;
    count[0] = 0;
    int code = 0;
    for (int l = 1; l <= 15; ++l) {
        code = (code + count[l - 1]) << 1;
        next[l] = code;
    }
    for (int s = 0; s < n; ++s) {
        const int l = lens[s];
        if (!l) {
            codes[s] = 0;
            continue;
        }
        const int c = next[l]++;
        int rev = 0;
        for (int k = 0; k < l; ++k)
            rev |= ((c >> k) & 1) << (l - 1 - k);
        codes[s] = (uint16_t)rev;
    }
}

struct Token {
    uint16_t litlen;  // literal byte, or match length 3..258 (+256 marks a match)
    uint16_t dist;    // 0 for literals
};

int lenSymbol(int len)
{
    int i = 28;
    while (kLenBase[i] > len)
        --i;
    return i;
}
int distSymbol(int d)
{
    int i = 29;
    while (kDistBase[i] > d)
        --i;
    return i;
}

void storedBlock(BitWriter &bw, const uint8_t *p, size_t n, bool final)
{
    do {
        const size_t k = std::min<size_t>(n, 65535);
        bw.put(final && k == n ? 1 : 0, 1);
        bw.put(0, 2);
        bw.align();
        bw.put((uint32_t)k, 16);
        bw.put((uint32_t)k ^ 0xFFFF, 16);
        for (size_t i = 0; i < k; ++i)
            bw.put(p[i], 8);
        p += k;
        n -= k;
    } while (n);
}

void emitBlock(BitWriter &bw, const std::vector<Token> &toks, const uint8_t *raw, size_t rawLen, bool final)
{
    uint32_t lf[286] = {0}, df[30] = {0};
    for (const Token &t : toks) {
        if (t.dist == 0) {
            lf[t.litlen]++;
        } else {
            lf[257 + lenSymbol(t.litlen - 256)]++;
            df[distSymbol(t.dist)]++;
        }
    }
    lf[256] = 1;
    uint8_t ll[286], dl[30];
    huffmanLengths(lf, 286, 15, ll);
    huffmanLengths(df, 30, 15, dl);
    int hlit = 286, hdist = 30;
    while (hlit > 257 && ll[hlit - 1] == 0)
        --hlit;
    while (hdist > 1 && dl[hdist - 1] == 0)
        --hdist;
    // Run-length code the concatenated code lengths (symbols 16, 17, 18).
    std::vector<uint8_t> all(ll, ll + hlit);
    all.insert(all.end(), dl, dl + hdist);
    std::vector<std::pair<uint8_t, uint8_t>> cl;  // symbol, extra value
    for (size_t i = 0; i < all.size();) {
        size_t run = 1;
        while (i + run < all.size() && all[i + run] == all[i])
            ++run;
        if (all[i] == 0 && run >= 3) {
            const size_t r = std::min<size_t>(run, 138);
            cl.push_back(r >= 11 ? std::make_pair((uint8_t)18, (uint8_t)(r - 11)) : std::make_pair((uint8_t)17, (uint8_t)(r - 3)));
            i += r;
        } else if (all[i] != 0 && run >= 4) {
            cl.push_back({all[i], 0});
            const size_t r = std::min<size_t>(run - 1, 6);
            cl.push_back({16, (uint8_t)(r - 3)});
            i += 1 + r;
        } else {
            cl.push_back({all[i], 0});
            ++i;
        }
    }
    uint32_t cf[19] = {0};
    for (auto &c : cl)
        cf[c.first]++;
    uint8_t cll[19];
    huffmanLengths(cf, 19, 7, cll);
    int hclen = 19;
    while (hclen > 4 && cll[kClOrder[hclen - 1]] == 0)
        --hclen;
    // Dynamic block cost against stored.
    uint64_t bits = 3 + 5 + 5 + 4 + 3ull * hclen;
    for (auto &c : cl)
        bits += cll[c.first] + (c.first == 16 ? 2 : c.first == 17 ? 3 : c.first == 18 ? 7 : 0);
    for (int s = 0; s < 286; ++s)
        bits += (uint64_t)lf[s] * ll[s];
    for (int s = 257; s < 286; ++s)
        bits += (uint64_t)lf[s] * kLenExtra[s - 257];
    for (int s = 0; s < 30; ++s)
        bits += (uint64_t)df[s] * (dl[s] + kDistExtra[s]);
    const uint64_t storedBits = (rawLen / 65535 + 1) * 40 + 8ull * rawLen + 7;
    if (storedBits < bits) {
        storedBlock(bw, raw, rawLen, final);
        return;
    }
    uint16_t lc[286], dc[30], cc[19];
    canonicalCodes(ll, 286, lc);
    canonicalCodes(dl, 30, dc);
    canonicalCodes(cll, 19, cc);
    bw.put(final ? 1 : 0, 1);
    bw.put(2, 2);
    bw.put((uint32_t)(hlit - 257), 5);
    bw.put((uint32_t)(hdist - 1), 5);
    bw.put((uint32_t)(hclen - 4), 4);
    for (int k = 0; k < hclen; ++k)
        bw.put(cll[kClOrder[k]], 3);
    for (auto &c : cl) {
        bw.put(cc[c.first], cll[c.first]);
        if (c.first == 16)
            bw.put(c.second, 2);
        else if (c.first == 17)
            bw.put(c.second, 3);
        else if (c.first == 18)
            bw.put(c.second, 7);
    }
    for (const Token &t : toks) {
        if (t.dist == 0) {
            bw.put(lc[t.litlen], ll[t.litlen]);
        } else {
            const int len = t.litlen - 256, ls = lenSymbol(len), ds = distSymbol(t.dist);
            bw.put(lc[257 + ls], ll[257 + ls]);
            bw.put((uint32_t)(len - kLenBase[ls]), kLenExtra[ls]);
            bw.put(dc[ds], dl[ds]);
            bw.put((uint32_t)(t.dist - kDistBase[ds]), kDistExtra[ds]);
        }
    }
    bw.put(lc[256], ll[256]);
}

}  // namespace

void deflate(const uint8_t *in, size_t n, std::vector<uint8_t> &out, bool sync)
{
    BitWriter bw(out);
    const int HBITS = 15, WSIZE = 32768, MAXCHAIN = 32;
    std::vector<int32_t> head((size_t)1 << HBITS, -1), prev(WSIZE, -1);
    auto hash = [&](size_t i) {
        const uint32_t v = (uint32_t)in[i] | ((uint32_t)in[i + 1] << 8) | ((uint32_t)in[i + 2] << 16);
        return (v * 2654435761u) >> (32 - HBITS);
    };
    std::vector<Token> toks;
    toks.reserve(32768);
    size_t blockStart = 0, i = 0;
    auto insert = [&](size_t p) {
        if (p + 2 < n) {
            const uint32_t h = hash(p);
            prev[p & (WSIZE - 1)] = head[h];
            head[h] = (int32_t)p;
        }
    };
    while (i < n) {
        int bestLen = 0, bestDist = 0;
        if (i + 2 < n) {
            const uint32_t h = hash(i);
            int32_t cand = head[h];
            const size_t maxLen = std::min<size_t>(258, n - i);
            for (int chain = 0; cand >= 0 && chain < MAXCHAIN; ++chain) {
                const size_t d = i - (size_t)cand;
                if (d > (size_t)WSIZE - 1)
                    break;
                if (in[cand + bestLen] == in[i + bestLen]) {
                    size_t l = 0;
                    while (l < maxLen && in[cand + l] == in[i + l])
                        ++l;
                    if ((int)l > bestLen) {
                        bestLen = (int)l;
                        bestDist = (int)d;
                        if (l == maxLen)
                            break;
                    }
                }
                const int32_t nx = prev[cand & (WSIZE - 1)];
                if (nx >= cand)
                    break;
                cand = nx;
            }
        }
        if (bestLen >= 3) {
            toks.push_back({(uint16_t)(256 + bestLen), (uint16_t)bestDist});
            for (int k = 0; k < bestLen; ++k)
                insert(i + (size_t)k);
            i += (size_t)bestLen;
        } else {
            toks.push_back({in[i], 0});
            insert(i);
            ++i;
        }
        if (toks.size() >= 32768 || i == n) {
            emitBlock(bw, toks, in + blockStart, i - blockStart, !sync && i == n);
            toks.clear();
            blockStart = i;
        }
    }
    if (n == 0 && !sync) {
        // Empty input: one final fixed block holding only end-of-block.
        bw.put(1, 1);
        bw.put(1, 2);
        bw.put(0, 7);
    }
    if (sync) {
        bw.put(0, 1);
        bw.put(0, 2);
        bw.align();
        bw.put(0, 16);
        bw.put(0xFFFF, 16);
    }
    bw.align();
}

void zlibCompress(const uint8_t *in, size_t n, std::vector<uint8_t> &out, int threads, size_t grain)
{
    out.push_back(0x78);
    out.push_back(0x9C);
    if (grain == 0)
        grain = 1;
    const size_t minPiece = 1 << 20;
    size_t pieces = std::max<size_t>(1, std::min<size_t>((size_t)std::max(threads, 1), n / minPiece));
    std::vector<size_t> cut(pieces + 1, n);
    cut[0] = 0;
    for (size_t k = 1; k < pieces; ++k)
        cut[k] = std::min(n, (n * k / pieces) / grain * grain);
    std::vector<std::vector<uint8_t>> parts(pieces);
    auto work = [&](size_t k) { deflate(in + cut[k], cut[k + 1] - cut[k], parts[k], k + 1 < pieces); };
    if (pieces == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (size_t k = 0; k < pieces; ++k)
            th.emplace_back(work, k);
        for (auto &t : th)
            t.join();
    }
    for (auto &p : parts)
        out.insert(out.end(), p.begin(), p.end());
    const uint32_t a = adler32(in, n);
    for (int s = 24; s >= 0; s -= 8)
        out.push_back((uint8_t)(a >> s));
}

namespace {

void putBe32(std::vector<uint8_t> &o, uint32_t v)
{
    for (int s = 24; s >= 0; s -= 8)
        o.push_back((uint8_t)(v >> s));
}

void pngChunk(std::vector<uint8_t> &o, const char *tag, const uint8_t *data, size_t n)
{
    putBe32(o, (uint32_t)n);
    const size_t at = o.size();
    o.insert(o.end(), tag, tag + 4);
    o.insert(o.end(), data, data + n);
    putBe32(o, crc32(o.data() + at, n + 4));
}

uint8_t paethPredict(int a, int b, int c)
{
    const int p = a + b - c;
    const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc)
        return (uint8_t)a;
    return (uint8_t)(pb <= pc ? b : c);
}

}  // namespace

void encodePng(const uint8_t *rgba, uint32_t w, uint32_t h, size_t stride, std::vector<uint8_t> &out, int threads)
{
    const size_t rb = (size_t)w * 4;
    std::vector<uint8_t> filtered((rb + 1) * h);
    auto filterRows = [&](uint32_t y0, uint32_t y1) {
        std::vector<uint8_t> cand(rb);
        for (uint32_t y = y0; y < y1; ++y) {
            const uint8_t *cur = rgba + (size_t)y * stride, *prv = y ? cur - stride : nullptr;
            uint8_t *dst = filtered.data() + (size_t)y * (rb + 1);
            long best = -1;
            for (int f = 0; f < 5; ++f) {
                long cost = 0;
                for (size_t i = 0; i < rb; ++i) {
                    const int a = i >= 4 ? cur[i - 4] : 0, b = prv ? prv[i] : 0, c = (prv && i >= 4) ? prv[i - 4] : 0;
                    const int pred = f == 0 ? 0 : f == 1 ? a : f == 2 ? b : f == 3 ? (a + b) >> 1 : paethPredict(a, b, c);
                    const uint8_t r = (uint8_t)(cur[i] - pred);
                    cand[i] = r;
                    cost += r < 128 ? r : 256 - r;
                }
                if (best < 0 || cost < best) {
                    best = cost;
                    dst[0] = (uint8_t)f;
                    memcpy(dst + 1, cand.data(), rb);
                }
            }
        }
    };
    const int nt = std::max(1, std::min<int>(threads, (int)(h / 16)));
    if (nt == 1) {
        filterRows(0, h);
    } else {
        std::vector<std::thread> th;
        for (int k = 0; k < nt; ++k)
            th.emplace_back(filterRows, (uint32_t)((uint64_t)h * k / nt), (uint32_t)((uint64_t)h * (k + 1) / nt));
        for (auto &t : th)
            t.join();
    }
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    out.assign(sig, sig + 8);
    uint8_t ihdr[13] = {0};
    for (int s = 0; s < 4; ++s) {
        ihdr[s] = (uint8_t)(w >> (24 - 8 * s));
        ihdr[4 + s] = (uint8_t)(h >> (24 - 8 * s));
    }
    ihdr[8] = 8;
    ihdr[9] = 6;
    pngChunk(out, "IHDR", ihdr, 13);
    std::vector<uint8_t> z;
    zlibCompress(filtered.data(), filtered.size(), z, threads, rb + 1);
    for (size_t off = 0; off < z.size(); off += (1u << 20))
        pngChunk(out, "IDAT", z.data() + off, std::min<size_t>(z.size() - off, 1u << 20));
    pngChunk(out, "IEND", nullptr, 0);
}

void encodeHdr(const uint8_t *rgbe, uint32_t w, uint32_t h, std::vector<uint8_t> &out)
{
    char head[128];
    const int hl = snprintf(head, sizeof(head), "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %u +X %u\n", h, w);
    out.assign(head, head + hl);
    const bool rle = w >= 8 && w < 32768;
    std::vector<uint8_t> comp(w);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t *row = rgbe + (size_t)y * w * 4;
        if (!rle) {
            out.insert(out.end(), row, row + (size_t)w * 4);
            continue;
        }
        out.push_back(2);
        out.push_back(2);
        out.push_back((uint8_t)(w >> 8));
        out.push_back((uint8_t)(w & 255));
        for (int c = 0; c < 4; ++c) {
            for (uint32_t x = 0; x < w; ++x)
                comp[x] = row[4 * x + c];
            uint32_t x = 0;
            while (x < w) {
                // A run of at least 4 equal bytes is coded as (128 + n, v).
                uint32_t run = 1;
                while (x + run < w && run < 127 && comp[x + run] == comp[x])
                    ++run;
                if (run >= 4) {
                    out.push_back((uint8_t)(128 + run));
                    out.push_back(comp[x]);
                    x += run;
                    continue;
                }
                // Literals up to the next run of 4 (at most 128).
                uint32_t lit = 0;
                while (x + lit < w && lit < 128) {
                    uint32_t r = 1;
                    while (x + lit + r < w && r < 4 && comp[x + lit + r] == comp[x + lit])
                        ++r;
                    if (r >= 4)
                        break;
                    ++lit;
                }
                out.push_back((uint8_t)lit);
                out.insert(out.end(), comp.begin() + x, comp.begin() + x + lit);
                x += lit;
            }
        }
    }
}

namespace {

void putLe32(std::vector<uint8_t> &o, uint32_t v)
{
    for (int s = 0; s < 32; s += 8)
        o.push_back((uint8_t)(v >> s));
}
void attr(std::vector<uint8_t> &o, const char *name, const char *type, const std::vector<uint8_t> &val)
{
    o.insert(o.end(), name, name + strlen(name) + 1);
    o.insert(o.end(), type, type + strlen(type) + 1);
    putLe32(o, (uint32_t)val.size());
    o.insert(o.end(), val.begin(), val.end());
}

}  // namespace

bool encodeExr(const uint16_t *rows, uint32_t w, uint32_t h, int compression, std::vector<uint8_t> &out, int threads)
{
    if (compression != 0 && compression != 3)
        return false;
    out.clear();
    putLe32(out, 20000630u);  // magic
    putLe32(out, 2u);         // version 2, single-part scanline
    std::vector<uint8_t> v;
    for (const char *ch : {"A", "B", "G", "R"}) {
        v.push_back((uint8_t)ch[0]);
        v.push_back(0);
        putLe32(v, 1);  // HALF
        v.push_back(0);  // pLinear
        v.push_back(0);
        v.push_back(0);
        v.push_back(0);
        putLe32(v, 1);
        putLe32(v, 1);
    }
    v.push_back(0);
    attr(out, "channels", "chlist", v);
    attr(out, "compression", "compression", {(uint8_t)compression});
    v.clear();
    putLe32(v, 0);
    putLe32(v, 0);
    putLe32(v, w - 1);
    putLe32(v, h - 1);
    attr(out, "dataWindow", "box2i", v);
    attr(out, "displayWindow", "box2i", v);
    attr(out, "lineOrder", "lineOrder", {0});
    v.clear();
    const float one = 1.0f, zero = 0.0f;
    uint32_t bits;
    memcpy(&bits, &one, 4);
    putLe32(v, bits);
    attr(out, "pixelAspectRatio", "float", v);
    v.clear();
    memcpy(&bits, &zero, 4);
    putLe32(v, bits);
    putLe32(v, bits);
    attr(out, "screenWindowCenter", "v2f", v);
    v.clear();
    memcpy(&bits, &one, 4);
    putLe32(v, bits);
    attr(out, "screenWindowWidth", "float", v);
    out.push_back(0);  // end of header
    const uint32_t lines = compression == 3 ? 16 : 1;
    const uint32_t chunks = (h + lines - 1) / lines;
    const size_t tableAt = out.size();
    out.resize(out.size() + 8ull * chunks);
    const size_t lineBytes = (size_t)w * 4 * 2;
    std::vector<std::vector<uint8_t>> packed(chunks);
    auto pack = [&](uint32_t c0, uint32_t c1) {
        std::vector<uint8_t> tmp;
        for (uint32_t c = c0; c < c1; ++c) {
            const uint32_t y0 = c * lines, n = std::min(lines, h - y0);
            const uint8_t *raw = (const uint8_t *)(rows + (size_t)y0 * w * 4);
            const size_t len = lineBytes * n;
            if (compression == 0) {
                packed[c].assign(raw, raw + len);
                continue;
            }
            // ZIP: bytes split into even and odd halves, then differenced.
            tmp.resize(len);
            size_t e = 0, o = (len + 1) / 2;
            for (size_t i = 0; i < len; ++i)
                tmp[(i & 1) ? o++ : e++] = raw[i];
            for (size_t i = len - 1; i > 0; --i)
                tmp[i] = (uint8_t)(tmp[i] - tmp[i - 1] + 128);
            std::vector<uint8_t> z;
            zlibCompress(tmp.data(), len, z, 1, 1);
            if (z.size() < len)
                packed[c].swap(z);
            else
                packed[c].assign(raw, raw + len);
        }
    };
    const int nt = std::max(1, std::min<int>(threads, (int)chunks));
    if (nt == 1) {
        pack(0, chunks);
    } else {
        std::vector<std::thread> th;
        for (int k = 0; k < nt; ++k)
            th.emplace_back(pack, (uint32_t)((uint64_t)chunks * k / nt), (uint32_t)((uint64_t)chunks * (k + 1) / nt));
        for (auto &t : th)
            t.join();
    }
    for (uint32_t c = 0; c < chunks; ++c) {
        const uint64_t at = out.size();
        for (int s = 0; s < 8; ++s)
            out[tableAt + 8ull * c + s] = (uint8_t)(at >> (8 * s));
        putLe32(out, c * lines);
        putLe32(out, (uint32_t)packed[c].size());
        out.insert(out.end(), packed[c].begin(), packed[c].end());
    }
    return true;
}

}  // namespace optimg

// ------------------------------------------------------------------ C ABI
#include <cmath>
#include "../../include/optpt.h"

extern "C" int optpt_internal_set_error(int code, const char *msg);

namespace optimg {

// Float to IEEE half, round to nearest even (the rounding __float2half_rn
// and OpenEXR's half use); NaN stays NaN, overflow goes to infinity.
uint16_t halfFromFloat(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    const uint32_t sign = (u >> 16) & 0x8000u;
    u &= 0x7FFFFFFFu;
    if (u >= 0x7F800000u)
        return (uint16_t)(sign | (u > 0x7F800000u ? 0x7E00u : 0x7C00u));
    const uint32_t e = u >> 23;
    if (e >= 143)  // >= 2^16: infinity
        return (uint16_t)(sign | 0x7C00u);
    uint32_t sig = u & 0x7FFFFFu, shift, base;
    if (e >= 113) {  // normal half
        base = ((e - 112) << 10) | (sig >> 13);
        shift = 13;
        sig &= 0x1FFFu;
    } else {  // subnormal half: value = m * 2^-24, m = significand >> (126 - e)
        if (e < 101)  // below 2^-26: rounds to zero
            return (uint16_t)sign;
        sig |= 0x800000u;
        shift = 126 - e;
        base = sig >> shift;
        sig &= (1u << shift) - 1;
    }
    const uint32_t half = 1u << (shift - 1);
    if (sig > half || (sig == half && (base & 1)))
        ++base;  // may carry into the exponent, or to infinity: both correct
    return (uint16_t)(sign | base);
}

// Ward's RGBE with the same float operations as the GPU kernel.
uint32_t rgbeFromFloat(float r, float g, float b)
{
    const float m = std::fmax(r, std::fmax(g, b));
    if (!(m >= 1e-32f))
        return 0u;
    int e;
    const float f = std::frexp(m, &e);
    const float scale = (f * 256.0f) / m;
    auto q = [&](float c) { return (uint32_t)std::fmin(std::fmax(c * scale, 0.0f), 255.0f); };
    const uint32_t ex = (uint32_t)std::min(e + 128, 255);
    return q(r) | (q(g) << 8) | (q(b) << 16) | (ex << 24);
}

}  // namespace optimg

namespace {

int handOut(const std::vector<uint8_t> &v, void **out, size_t *size)
{
    void *p = malloc(v.empty() ? 1 : v.size());
    if (!p)
        return optpt_internal_set_error(OPTPT_ERR_NOMEM, "encoder output allocation failed");
    memcpy(p, v.data(), v.size());
    *out = p;
    *size = v.size();
    return OPTPT_OK;
}

int hostThreads()
{
    return (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
}

}  // namespace

extern "C" {

int optpt_encode_png(const uint8_t *rgba, uint32_t width, uint32_t height, size_t strideBytes, void **out, size_t *size)
{
    if (!rgba || !out || !size)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    if (width == 0 || height == 0 || (strideBytes && strideBytes < (size_t)width * 4))
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "bad image size or stride");
    std::vector<uint8_t> v;
    optimg::encodePng(rgba, width, height, strideBytes ? strideBytes : (size_t)width * 4, v, hostThreads());
    return handOut(v, out, size);
}

int optpt_encode_hdr(const float *rgba, uint32_t width, uint32_t height, void **out, size_t *size)
{
    if (!rgba || !out || !size)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    if (width == 0 || height == 0)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "bad image size");
    const size_t n = (size_t)width * height;
    std::vector<uint32_t> px(n);
    for (size_t i = 0; i < n; ++i)
        px[i] = optimg::rgbeFromFloat(rgba[4 * i], rgba[4 * i + 1], rgba[4 * i + 2]);
    std::vector<uint8_t> v;
    optimg::encodeHdr((const uint8_t *)px.data(), width, height, v);
    return handOut(v, out, size);
}

int optpt_encode_exr(const float *rgba, uint32_t width, uint32_t height, int compression, void **out, size_t *size)
{
    if (!rgba || !out || !size)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    if (width == 0 || height == 0 || (compression != 0 && compression != 3))
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "bad image size or compression (0 none, 3 ZIP)");
    std::vector<uint16_t> rows((size_t)width * height * 4);
    const uint16_t one = optimg::halfFromFloat(1.0f);
    for (uint32_t y = 0; y < height; ++y)
        for (uint32_t x = 0; x < width; ++x) {
            const float *p = rgba + 4 * ((size_t)y * width + x);
            uint16_t *row = rows.data() + (size_t)y * 4 * width + x;
            row[0] = one;
            row[width] = optimg::halfFromFloat(p[2]);
            row[2 * width] = optimg::halfFromFloat(p[1]);
            row[3 * width] = optimg::halfFromFloat(p[0]);
        }
    std::vector<uint8_t> v;
    optimg::encodeExr(rows.data(), width, height, compression, v, hostThreads());
    return handOut(v, out, size);
}

void optpt_free(void *p) { free(p); }

}  // extern "C"
