// Baseline / extended-sequential JPEG decoding to RGBA8 (ITU-T T.81, 8-bit
// samples, Huffman coding), for glTF textures: the reference reads them with
// stb_image inside tinygltf (src/gltf_loader.cpp:532), which is absent here.
//
// Covered: SOF0 and SOF1 frames with 1 (grey) or 3 (YCbCr, or RGB when an
// Adobe APP14 segment says so) components, any sampling factors 1..4,
// interleaved and non-interleaved scans (several scans per frame), 8- and
// 16-bit quantisation tables, restart intervals. Progressive, lossless,
// arithmetic-coded, 12-bit and CMYK files are reported as unsupported.
// Reconstruction: dequantise, separable floating-point inverse DCT, level
// shift, round and clamp; chroma planes are brought to full resolution by
// centred bilinear interpolation (the "fancy" upsampling of common
// decoders), then YCbCr -> RGB with the JFIF (BT.601 full-range) matrix.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "image_io.h"

namespace optimg {

namespace {

// Zigzag order: position k of the coded sequence -> natural (row-major) index.
const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct HuffTable {
    bool present = false;
    uint8_t vals[256];
    int maxcode[18];  // largest code of each length (-1 if none), [17] sentinel
    int valptr[17];
    int mincode[17];
    void build(const uint8_t *counts, const uint8_t *symbols, int nsym)
    {
        memcpy(vals, symbols, (size_t)nsym);
        int code = 0, k = 0;
        for (int l = 1; l <= 16; ++l) {
            valptr[l] = k;
            mincode[l] = code;
            code += counts[l - 1];
            k += counts[l - 1];
            maxcode[l] = counts[l - 1] ? code - 1 : -1;
            code <<= 1;
        }
        maxcode[17] = 0x7FFFFFFF;
        present = true;
    }
};

struct Component {
    int id, h, v, tq;
    int td = 0, ta = 0;
    int bw = 0, bh = 0;  // blocks across / down in the plane (whole MCUs)
    std::vector<uint8_t> plane;
    int dcPred = 0;
};

struct BitReader {
    const uint8_t *p;
    size_t n, pos;
    uint32_t buf = 0;
    int cnt = 0;
    bool marker = false;  // a marker was reached: only zero bits follow
    BitReader(const uint8_t *d, size_t len, size_t start) : p(d), n(len), pos(start) {}
    void fill()
    {
        while (cnt <= 24) {
            uint32_t b = 0;
            if (!marker && pos < n) {
                b = p[pos];
                if (b == 0xFF) {
                    const uint8_t nx = pos + 1 < n ? p[pos + 1] : 0;
                    if (nx == 0x00) {
                        pos += 2;
                    } else {
                        marker = true;  // leave pos on the marker
                        b = 0;
                    }
                } else {
                    ++pos;
                }
            }
            buf |= b << (24 - cnt);
            cnt += 8;
        }
    }
    int bit()
    {
        if (cnt < 1)
            fill();
        const int r = (int)(buf >> 31);
        buf <<= 1;
        --cnt;
        return r;
    }
    int bits(int k)
    {
        if (k == 0)
            return 0;
        if (cnt < k)
            fill();
        const int r = (int)(buf >> (32 - k));
        buf <<= k;
        cnt -= k;
        return r;
    }
    void reset()
    {
        buf = 0;
        cnt = 0;
    }
};

int decodeHuff(BitReader &br, const HuffTable &t)
{
    int code = br.bit();
    for (int l = 1; l <= 16; ++l) {
        if (t.maxcode[l] >= 0 && code <= t.maxcode[l] && code >= t.mincode[l])
            return t.vals[t.valptr[l] + code - t.mincode[l]];
        code = (code << 1) | br.bit();
    }
    return -1;
}

int extend(int v, int s) { return s == 0 ? 0 : (v < (1 << (s - 1)) ? v - (1 << s) + 1 : v); }

struct Idct {
    float c[8][8];  // c[x][u] = C(u) / 2 * cos((2x + 1) u pi / 16)
    Idct()
    {
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                c[x][u] = (float)((u == 0 ? std::sqrt(0.5) : 1.0) * 0.5 *
                                  std::cos((2.0 * x + 1.0) * u * 3.14159265358979323846 / 16.0));
    }
    void run(const int *coef, uint8_t *out, int stride) const
    {
        float tmp[8][8];
        for (int y = 0; y < 8; ++y)          // rows of the coefficient block: v
            for (int x = 0; x < 8; ++x) {    // spatial x
                float s = 0.0f;
                for (int u = 0; u < 8; ++u)
                    s += c[x][u] * (float)coef[y * 8 + u];
                tmp[y][x] = s;
            }
        for (int x = 0; x < 8; ++x)
            for (int y = 0; y < 8; ++y) {
                float s = 0.0f;
                for (int v = 0; v < 8; ++v)
                    s += c[y][v] * tmp[v][x];
                const float val = std::floor(s + 128.0f + 0.5f);
                out[y * stride + x] = (uint8_t)(val < 0.0f ? 0.0f : val > 255.0f ? 255.0f : val);
            }
    }
};

const Idct kIdct;

uint32_t be16(const uint8_t *p) { return ((uint32_t)p[0] << 8) | p[1]; }

}  // namespace

bool isJpeg(const uint8_t *p, size_t n) { return n >= 3 && p[0] == 0xFF && p[1] == 0xD8 && p[2] == 0xFF; }

bool decodeJpeg(const uint8_t *p, size_t n, Image &img, std::string &err)
{
    if (!isJpeg(p, n)) {
        err = "not a JPEG file";
        return false;
    }
    uint16_t qt[4][64];
    bool qtPresent[4] = {false, false, false, false};
    HuffTable dc[4], ac[4];
    std::vector<Component> comps;
    int width = 0, height = 0, hmax = 1, vmax = 1, restart = 0;
    int adobeTransform = -1;
    bool frame = false, sawScan = false;
    size_t pos = 2;
    while (pos + 4 <= n) {
        if (p[pos] != 0xFF) {
            err = "marker expected";
            return false;
        }
        const uint8_t m = p[pos + 1];
        if (m == 0xFF) {  // fill byte
            ++pos;
            continue;
        }
        if (m == 0xD9)  // EOI
            break;
        if (m >= 0xD0 && m <= 0xD7) {  // stray RSTn
            pos += 2;
            continue;
        }
        const uint32_t len = be16(p + pos + 2);
        if (len < 2 || pos + 2 + len > n) {
            err = "truncated JPEG segment";
            return false;
        }
        const uint8_t *s = p + pos + 4;
        const size_t sl = len - 2;
        if (m == 0xDB) {  // DQT
            size_t k = 0;
            while (k < sl) {
                const int pq = s[k] >> 4, tq = s[k] & 15;
                ++k;
                if (tq > 3 || pq > 1 || k + (pq ? 128u : 64u) > sl) {
                    err = "bad DQT";
                    return false;
                }
                for (int i = 0; i < 64; ++i) {
                    qt[tq][kZigzag[i]] = pq ? (uint16_t)be16(s + k + 2 * i) : s[k + i];
                }
                k += pq ? 128 : 64;
                qtPresent[tq] = true;
            }
        } else if (m == 0xC4) {  // DHT
            size_t k = 0;
            while (k < sl) {
                if (k + 17 > sl) {
                    err = "bad DHT";
                    return false;
                }
                const int tc = s[k] >> 4, th = s[k] & 15;
                const uint8_t *counts = s + k + 1;
                int total = 0;
                for (int i = 0; i < 16; ++i)
                    total += counts[i];
                if (tc > 1 || th > 3 || total > 256 || k + 17 + (size_t)total > sl) {
                    err = "bad DHT";
                    return false;
                }
                (tc ? ac[th] : dc[th]).build(counts, s + k + 17, total);
                k += 17 + (size_t)total;
            }
        } else if (m == 0xDD) {  // DRI
            if (sl < 2) {
                err = "bad DRI";
                return false;
            }
            restart = (int)be16(s);
        } else if (m == 0xEE) {  // APP14 (Adobe): colour transform flag
            if (sl >= 12 && !memcmp(s, "Adobe", 5))
                adobeTransform = s[11];
        } else if (m == 0xC0 || m == 0xC1) {  // SOF0 / SOF1
            if (sl < 6 || s[0] != 8) {
                err = "only 8-bit JPEG samples are supported";
                return false;
            }
            height = (int)be16(s + 1);
            width = (int)be16(s + 3);
            const int nc = s[5];
            if (width <= 0 || height <= 0 || (uint64_t)width * height > (1ull << 28)) {
                err = "JPEG dimensions out of range";
                return false;
            }
            if ((nc != 1 && nc != 3) || sl < 6 + 3u * nc) {
                err = "only grey and three-component JPEG files are supported";
                return false;
            }
            comps.resize(nc);
            for (int c = 0; c < nc; ++c) {
                comps[c].id = s[6 + 3 * c];
                comps[c].h = s[7 + 3 * c] >> 4;
                comps[c].v = s[7 + 3 * c] & 15;
                comps[c].tq = s[8 + 3 * c];
                if (comps[c].h < 1 || comps[c].h > 4 || comps[c].v < 1 || comps[c].v > 4 || comps[c].tq > 3) {
                    err = "bad JPEG component";
                    return false;
                }
                hmax = std::max(hmax, comps[c].h);
                vmax = std::max(vmax, comps[c].v);
            }
            const int mcux = (width + 8 * hmax - 1) / (8 * hmax), mcuy = (height + 8 * vmax - 1) / (8 * vmax);
            for (auto &c : comps) {
                c.bw = mcux * c.h;
                c.bh = mcuy * c.v;
                c.plane.assign((size_t)c.bw * 8 * c.bh * 8, 0);
            }
            frame = true;
        } else if (m >= 0xC2 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) {
            err = m == 0xC2 ? "progressive JPEG is not supported" : "unsupported JPEG coding process";
            return false;
        } else if (m == 0xDA) {  // SOS
            if (!frame) {
                err = "scan before frame header";
                return false;
            }
            const int ns = s[0];
            if (ns < 1 || ns > 4 || sl < 1 + 2u * ns + 3) {
                err = "bad SOS";
                return false;
            }
            std::vector<Component *> sc;
            for (int i = 0; i < ns; ++i) {
                const int cid = s[1 + 2 * i], t = s[2 + 2 * i];
                Component *c = nullptr;
                for (auto &x : comps)
                    if (x.id == cid)
                        c = &x;
                if (!c || (t >> 4) > 3 || (t & 15) > 3) {
                    err = "bad SOS component";
                    return false;
                }
                c->td = t >> 4;
                c->ta = t & 15;
                if (!dc[c->td].present || !ac[c->ta].present || !qtPresent[c->tq]) {
                    err = "JPEG scan refers to a missing table";
                    return false;
                }
                c->dcPred = 0;
                sc.push_back(c);
            }
            BitReader br(p, n, pos + 2 + len);
            // Units of this scan: interleaved MCUs, or the component's blocks.
            int unitsX, unitsY;
            if (ns == 1) {
                const Component &c = *sc[0];
                unitsX = (int)((std::ceil((double)width * c.h / hmax) + 7) / 8);
                unitsY = (int)((std::ceil((double)height * c.v / vmax) + 7) / 8);
            } else {
                unitsX = (width + 8 * hmax - 1) / (8 * hmax);
                unitsY = (height + 8 * vmax - 1) / (8 * vmax);
            }
            const long total = (long)unitsX * unitsY;
            int coef[64];
            auto block = [&](Component &c, int bx, int by) -> bool {
                memset(coef, 0, sizeof(coef));
                const int t = decodeHuff(br, dc[c.td]);
                if (t < 0 || t > 11) {
                    err = "bad JPEG DC code";
                    return false;
                }
                c.dcPred += extend(br.bits(t), t);
                coef[0] = c.dcPred * qt[c.tq][0];
                for (int k = 1; k < 64;) {
                    const int rs = decodeHuff(br, ac[c.ta]);
                    if (rs < 0) {
                        err = "bad JPEG AC code";
                        return false;
                    }
                    const int r = rs >> 4, sz = rs & 15;
                    if (sz == 0) {
                        if (r == 15) {
                            k += 16;
                            continue;
                        }
                        break;  // end of block
                    }
                    k += r;
                    if (k > 63) {
                        err = "JPEG AC run past the block";
                        return false;
                    }
                    coef[kZigzag[k]] = extend(br.bits(sz), sz) * qt[c.tq][kZigzag[k]];
                    ++k;
                }
                if (bx < c.bw && by < c.bh) {
                    const int stride = c.bw * 8;
                    kIdct.run(coef, c.plane.data() + (size_t)by * 8 * stride + (size_t)bx * 8, stride);
                }
                return true;
            };
            for (long u = 0; u < total; ++u) {
                if (restart && u > 0 && u % restart == 0) {
                    // byte-align, expect RSTn, reset predictions
                    br.reset();
                    if (br.marker) {
                        if (br.pos + 1 < n && p[br.pos] == 0xFF && p[br.pos + 1] >= 0xD0 && p[br.pos + 1] <= 0xD7) {
                            br.pos += 2;
                            br.marker = false;
                        }
                    } else {
                        // skip to the marker
                        while (br.pos + 1 < n && !(p[br.pos] == 0xFF && p[br.pos + 1] >= 0xD0 && p[br.pos + 1] <= 0xD7))
                            ++br.pos;
                        if (br.pos + 1 < n)
                            br.pos += 2;
                    }
                    for (auto *c : sc)
                        c->dcPred = 0;
                }
                const int ux = (int)(u % unitsX), uy = (int)(u / unitsX);
                if (ns == 1) {
                    if (!block(*sc[0], ux, uy))
                        return false;
                } else {
                    for (auto *c : sc)
                        for (int by = 0; by < c->v; ++by)
                            for (int bx = 0; bx < c->h; ++bx)
                                if (!block(*c, ux * c->h + bx, uy * c->v + by))
                                    return false;
                }
            }
            // continue after the entropy-coded segment: find the next marker
            size_t q = br.pos;
            while (q + 1 < n && !(p[q] == 0xFF && p[q + 1] != 0x00 && !(p[q + 1] >= 0xD0 && p[q + 1] <= 0xD7)))
                ++q;
            pos = q;
            sawScan = true;
            continue;
        }
        pos += 2 + len;
    }
    if (!frame || !sawScan) {
        err = "incomplete JPEG";
        return false;
    }
    img.width = (uint32_t)width;
    img.height = (uint32_t)height;
    img.rgba.assign((size_t)width * height * 4, 255);
    // Component sample at full-resolution pixel (x, y): centred bilinear.
    auto sample = [&](const Component &c, int x, int y) -> float {
        const int stride = c.bw * 8;
        if (c.h == hmax && c.v == vmax)
            return c.plane[(size_t)y * stride + x];
        const float cx = ((float)x + 0.5f) * (float)c.h / (float)hmax - 0.5f;
        const float cy = ((float)y + 0.5f) * (float)c.v / (float)vmax - 0.5f;
        const int cw = (int)std::ceil((double)width * c.h / hmax), ch = (int)std::ceil((double)height * c.v / vmax);
        const int x0 = (int)std::floor(cx), y0 = (int)std::floor(cy);
        const float fx = cx - (float)x0, fy = cy - (float)y0;
        auto at = [&](int xx, int yy) -> float {
            xx = xx < 0 ? 0 : xx >= cw ? cw - 1 : xx;
            yy = yy < 0 ? 0 : yy >= ch ? ch - 1 : yy;
            return c.plane[(size_t)yy * stride + xx];
        };
        const float top = at(x0, y0) + (at(x0 + 1, y0) - at(x0, y0)) * fx;
        const float bot = at(x0, y0 + 1) + (at(x0 + 1, y0 + 1) - at(x0, y0 + 1)) * fx;
        return top + (bot - top) * fy;
    };
    const bool rgbDirect = comps.size() == 3 && adobeTransform == 0;
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            uint8_t *o = img.rgba.data() + ((size_t)y * width + x) * 4;
            if (comps.size() == 1) {
                const float g = sample(comps[0], x, y);
                o[0] = o[1] = o[2] = (uint8_t)g;
                continue;
            }
            const float Y = sample(comps[0], x, y), cb = sample(comps[1], x, y), cr = sample(comps[2], x, y);
            float rgb[3];
            if (rgbDirect) {
                rgb[0] = Y;
                rgb[1] = cb;
                rgb[2] = cr;
            } else {
                rgb[0] = Y + 1.402f * (cr - 128.0f);
                rgb[1] = Y - 0.344136f * (cb - 128.0f) - 0.714136f * (cr - 128.0f);
                rgb[2] = Y + 1.772f * (cb - 128.0f);
            }
            for (int k = 0; k < 3; ++k) {
                const float v = std::floor(rgb[k] + 0.5f);
                o[k] = (uint8_t)(v < 0.0f ? 0.0f : v > 255.0f ? 255.0f : v);
            }
        }
    return true;
}

}  // namespace optimg
