// ORACLE (test infrastructure only; never linked into the product).
//
// Host restatement of the reference's render path, used as the checker for
// the GPU kernels and as the timed CPU baseline:
//   * LBVH: 30-bit Morton codes of bounding-box centroids, a stable sort, and
//     Karras' radix tree with subtrees of <= leafSize triangles collapsed to
//     leaves; the same construction rules as the GPU build, so sorted codes,
//     leaf order and topology must match it exactly.
//   * closest-hit / occlusion traversal with the watertight ray-triangle test
//     (Woop, Benthin, Wald, JCGT 2013); the closest hit is the smallest
//     (t, primitive index), which makes hit IDs independent of traversal order.
//   * the progressive integrator of cu/device_programs.cu:15-106 and
//     cu/path_tracer.cu:17-582 (camera jitter, any-hit alpha, closest-hit
//     shading, point-light and emissive-triangle next-event estimation, BSDF
//     sampling, Russian roulette, miss), templated on the shading precision.
//   * the counter-based PCG32 stream of the product (a pure function of seed,
//     pixel, sample and path depth), so every sample can be replayed.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include "../include/optpt.h"
#include "oracle_bsdf.hpp"

namespace {

using orc::V3;

// ------------------------------------------------------------------ random numbers
// PCG32 XSH-RR (O'Neill 2014) seeded by SplitMix64 of (seed, pixel) and
// (sample, depth).
uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
struct Pcg {
    uint64_t state = 0, inc = 1;
    uint32_t next()
    {
        uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
        uint32_t rot = (uint32_t)(old >> 59);
        return (xs >> rot) | (xs << ((0u - rot) & 31u));
    }
    float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
};
Pcg pathRng(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t depth)
{
    Pcg r;
    uint64_t initstate = splitmix64(((uint64_t)seed << 32) | pixel);
    uint64_t initseq = splitmix64(((uint64_t)sample << 8) | (depth & 0xFFu));
    r.state = 0;
    r.inc = (initseq << 1u) | 1u;
    r.next();
    r.state += initstate;
    r.next();
    return r;
}
float blendUniform(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t depth, uint32_t prim)
{
    uint64_t k = splitmix64(((uint64_t)seed << 32) | pixel) ^
                 splitmix64(((uint64_t)sample << 40) ^ ((uint64_t)depth << 32) ^ prim);
    return (float)(splitmix64(k) >> 40) * (1.0f / 16777216.0f);
}

// ------------------------------------------------------------------ geometry
struct F3 {
    float x, y, z;
};
F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
float comp(F3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

struct Tri {
    F3 v0, v1, v2;
    int prim;
};

struct RayPre {
    F3 o;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
RayPre rayPrepare(F3 o, F3 d)
{
    RayPre r;
    r.o = o;
    float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    float dz = comp(d, kz);
    if (dz < 0.0f)
        std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = comp(d, kx) / dz;
    r.Sy = comp(d, ky) / dz;
    r.Sz = 1.0f / dz;
    return r;
}
// Watertight test; roundings made explicit with fmaf.
bool intersectTri(const RayPre &r, const Tri &tr, float tmin, float tmax, float &t, float &u, float &v)
{
    F3 A = sub(tr.v0, r.o), B = sub(tr.v1, r.o), C = sub(tr.v2, r.o);
    float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
    float Ax = std::fmaf(-r.Sx, Akz, comp(A, r.kx)), Ay = std::fmaf(-r.Sy, Akz, comp(A, r.ky));
    float Bx = std::fmaf(-r.Sx, Bkz, comp(B, r.kx)), By = std::fmaf(-r.Sy, Bkz, comp(B, r.ky));
    float Cx = std::fmaf(-r.Sx, Ckz, comp(C, r.kx)), Cy = std::fmaf(-r.Sy, Ckz, comp(C, r.ky));
    float U = std::fmaf(Cx, By, -(Cy * Bx));
    float V = std::fmaf(Ax, Cy, -(Ay * Cx));
    float W = std::fmaf(Bx, Ay, -(By * Ax));
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f))
        return false;
    float det = U + V + W;
    if (det == 0.0f)
        return false;
    float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
    float T = std::fmaf(U, Az, std::fmaf(V, Bz, W * Cz));
    float tt = T / det;
    if (!(tt > tmin && tt <= tmax))
        return false;
    t = tt;
    u = V / det;
    v = W / det;
    return true;
}

// ------------------------------------------------------------------ LBVH
unsigned expandBits(unsigned v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
unsigned quantize(float c, float lo, float hi)
{
    float ext = hi - lo;
    float nrm = ext > 0.0f ? (c - lo) / ext : 0.0f;
    float s = std::fmin(std::fmax(nrm * 1024.0f, 0.0f), 1023.0f);
    return (unsigned)s;
}
int clz32(unsigned x) { return x ? __builtin_clz(x) : 32; }

struct Box {
    float lo[3], hi[3];
};

struct HostBvh {
    std::vector<unsigned> codes;     // sorted
    std::vector<int> order;          // sorted position -> primitive
    std::vector<int> nodes4;         // (ref0, ref1, cnt0, cnt1) per internal slot; zeros where unused
    std::vector<Box> nodeBoxL, nodeBoxR;
    std::vector<Tri> tris;           // leaf order
    int usedNodes = 0, leaves = 0;
};

Box primBox(const float *P, const int *I, int t)
{
    Box b;
    for (int k = 0; k < 3; ++k) {
        float a = P[3 * I[3 * t] + k], c = P[3 * I[3 * t + 1] + k], d = P[3 * I[3 * t + 2] + k];
        b.lo[k] = std::fmin(std::fmin(a, c), d);
        b.hi[k] = std::fmax(std::fmax(a, c), d);
    }
    return b;
}

// Builds the LBVH: same rules as the GPU build (see the file comment).
void buildHostBvh(const float *P, const int *I, int n, int leafSize, HostBvh &h)
{
    h = HostBvh{};
    if (n <= 0)
        return;
    std::vector<Box> pb(n);
    float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    std::vector<float> cen(3 * (size_t)n);
    for (int t = 0; t < n; ++t) {
        pb[t] = primBox(P, I, t);
        for (int k = 0; k < 3; ++k) {
            float c = (pb[t].lo[k] + pb[t].hi[k]) * 0.5f;
            cen[3 * t + k] = c;
            cmin[k] = std::fmin(cmin[k], c);
            cmax[k] = std::fmax(cmax[k], c);
        }
    }
    std::vector<unsigned> code(n);
    for (int t = 0; t < n; ++t)
        code[t] = (expandBits(quantize(cen[3 * t], cmin[0], cmax[0])) << 2) |
                  (expandBits(quantize(cen[3 * t + 1], cmin[1], cmax[1])) << 1) |
                  expandBits(quantize(cen[3 * t + 2], cmin[2], cmax[2]));
    h.order.resize(n);
    for (int t = 0; t < n; ++t)
        h.order[t] = t;
    std::stable_sort(h.order.begin(), h.order.end(), [&](int a, int b) { return code[a] < code[b]; });
    h.codes.resize(n);
    for (int i = 0; i < n; ++i)
        h.codes[i] = code[h.order[i]];
    h.tris.resize(n);
    for (int i = 0; i < n; ++i) {
        int p = h.order[i];
        auto v = [&](int k) { return F3{P[3 * I[3 * p + k]], P[3 * I[3 * p + k] + 1], P[3 * I[3 * p + k] + 2]}; };
        h.tris[i] = Tri{v(0), v(1), v(2), p};
    }
    const int nInt = n > 1 ? n - 1 : 1;
    h.nodes4.assign(4 * (size_t)nInt, 0);
    h.nodeBoxL.assign(nInt, Box{});
    h.nodeBoxR.assign(nInt, Box{});
    if (n == 1) {
        h.nodes4[0] = 0;
        h.nodes4[1] = -1;
        h.nodes4[2] = 1;
        h.nodes4[3] = 0;
        h.nodeBoxL[0] = pb[0];
        h.usedNodes = 1;
        h.leaves = 1;
        return;
    }
    const unsigned *C = h.codes.data();
    auto delta = [&](int i, int j) -> int {
        if (j < 0 || j >= n)
            return -1;
        if (C[i] == C[j])
            return 32 + clz32((unsigned)(i ^ j));
        return clz32(C[i] ^ C[j]);
    };
    const unsigned LEAF = 0x80000000u;
    std::vector<int> childL(n - 1), childR(n - 1), first(n - 1), parentI(n - 1, -1), parentL(n, -1);
    for (int i = 0; i < n - 1; ++i) {
        int d = (delta(i, i + 1) - delta(i, i - 1)) >= 0 ? 1 : -1;
        int dmin = delta(i, i - d);
        int lmax = 2;
        while (delta(i, i + lmax * d) > dmin)
            lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (delta(i, i + (l + t) * d) > dmin)
                l += t;
        int j = i + l * d;
        int dnode = delta(i, j);
        int s = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (delta(i, i + (s + t) * d) > dnode)
                s += t;
        } while (t > 1);
        int gamma = i + s * d + std::min(d, 0);
        int f = std::min(i, j), la = std::max(i, j);
        if (f == gamma) {
            childL[i] = (int)((unsigned)gamma | LEAF);
            parentL[gamma] = i;
        } else {
            childL[i] = gamma;
            parentI[gamma] = i;
        }
        if (la == gamma + 1) {
            childR[i] = (int)((unsigned)(gamma + 1) | LEAF);
            parentL[gamma + 1] = i;
        } else {
            childR[i] = gamma + 1;
            parentI[gamma + 1] = i;
        }
        first[i] = f;
    }
    // Subtree boxes and sizes, children before parents (post-order).
    std::vector<Box> nb(n - 1);
    std::vector<int> cnt(n - 1, 0);
    auto childInfo = [&](int c, Box &b, int &k) {
        if ((unsigned)c & LEAF) {
            b = pb[h.order[(int)((unsigned)c & ~LEAF)]];
            k = 1;
        } else {
            b = nb[c];
            k = cnt[c];
        }
    };
    std::vector<int> stack{0}, post;
    while (!stack.empty()) {
        int x = stack.back();
        stack.pop_back();
        post.push_back(x);
        if (!((unsigned)childL[x] & LEAF))
            stack.push_back(childL[x]);
        if (!((unsigned)childR[x] & LEAF))
            stack.push_back(childR[x]);
    }
    for (auto it = post.rbegin(); it != post.rend(); ++it) {
        int x = *it;
        Box a, b;
        int ka, kb;
        childInfo(childL[x], a, ka);
        childInfo(childR[x], b, kb);
        for (int k = 0; k < 3; ++k) {
            nb[x].lo[k] = std::fmin(a.lo[k], b.lo[k]);
            nb[x].hi[k] = std::fmax(a.hi[k], b.hi[k]);
        }
        cnt[x] = ka + kb;
    }
    for (int i = 0; i < n - 1; ++i) {
        if (cnt[i] <= leafSize) {
            if (i == 0) {
                h.nodes4[0] = 0;
                h.nodes4[1] = -1;
                h.nodes4[2] = n;
                h.nodes4[3] = 0;
                h.nodeBoxL[0] = nb[0];
                h.usedNodes = 1;
                h.leaves = 1;
            }
            continue;
        }
        ++h.usedNodes;
        for (int side = 0; side < 2; ++side) {
            int c = side == 0 ? childL[i] : childR[i];
            int ref, k;
            Box b;
            if ((unsigned)c & LEAF) {
                ref = (int)((unsigned)c & ~LEAF);
                k = 1;
                b = pb[h.order[ref]];
                ++h.leaves;
            } else if (cnt[c] <= leafSize) {
                ref = first[c];
                k = cnt[c];
                b = nb[c];
                ++h.leaves;
            } else {
                ref = c;
                k = 0;
                b = nb[c];
            }
            h.nodes4[4 * i + side] = ref;
            h.nodes4[4 * i + 2 + side] = k;
            (side == 0 ? h.nodeBoxL[i] : h.nodeBoxR[i]) = b;
        }
    }
}

// ------------------------------------------------------------------ BVH8 collapse
// The product's collapse rules restated: level by level, each BVH2 node that
// becomes a BVH8 node opens its internal child of largest surface area until
// it has 8 entries or only leaves; children and triangles are placed by
// prefix sums in item order; children take their centroid-octant slot (or the
// nearest free one by Hamming distance); boxes are quantised outwards by one
// step with a per-axis power-of-two scale; FP32 with directed rounding
// (extent up, a child's low offset down and high offset up).
struct Node8 {
    float p[3];
    uint32_t ew;
    uint32_t childBase, triBase, meta0, meta1;
    uint32_t q[3][4];
};
static_assert(sizeof(Node8) == 80, "80-byte node");

struct Entry8 {
    int ref, cnt;
    float lo[3], hi[3];
};

float sa8(const Entry8 &e)
{
    float dx = e.hi[0] - e.lo[0], dy = e.hi[1] - e.lo[1], dz = e.hi[2] - e.lo[2];
    return (dx * dy + dy * dz) + dz * dx;
}

// a - b rounded down / up, from the round-to-nearest difference and its
// exact error (Knuth's TwoSum), as the device's __fsub_rd / __fsub_ru give.
float subDown(float a, float b)
{
    const float s = a - b, bv = s - a, err = (a - (s - bv)) + (-b - bv);
    return err < 0.0f ? std::nextafter(s, -INFINITY) : s;
}
float subUp(float a, float b)
{
    const float s = a - b, bv = s - a, err = (a - (s - bv)) + (-b - bv);
    return err > 0.0f ? std::nextafter(s, INFINITY) : s;
}

int scaleExp(float ext)
{
    if (!(ext > 0.0f))
        return -126;
    int e = std::ilogb(ext) - 7;
    while (std::ldexp(253.0f, e) < ext)
        ++e;
    while (e > -126 && std::ldexp(253.0f, e - 1) >= ext)
        --e;
    return std::max(-126, std::min(127, e));
}

void buildHostBvh8(const HostBvh &B, std::vector<Node8> &out, std::vector<int> &order8)
{
    out.clear();
    order8.clear();
    const int n = (int)B.tris.size();
    if (n == 0)
        return;
    auto child = [&](int node, int side, Entry8 &e) {
        e.ref = B.nodes4[4 * (size_t)node + side];
        e.cnt = B.nodes4[4 * (size_t)node + 2 + side];
        const Box &b = side == 0 ? B.nodeBoxL[node] : B.nodeBoxR[node];
        for (int k = 0; k < 3; ++k) {
            e.lo[k] = b.lo[k];
            e.hi[k] = b.hi[k];
        }
    };
    std::vector<int> items{0};
    order8.assign(n, -1);
    int triStart = 0;
    while (!items.empty()) {
        const int levelStart = (int)out.size();
        std::vector<std::vector<Entry8>> ents(items.size());
        std::vector<int> scanK(items.size() + 1, 0), scanT(items.size() + 1, 0);
        for (size_t i = 0; i < items.size(); ++i) {
            std::vector<Entry8> &e = ents[i];
            for (int side = 0; side < 2; ++side) {
                Entry8 c;
                child(items[i], side, c);
                if (c.ref >= 0)
                    e.push_back(c);
            }
            while (e.size() < 8) {
                int best = -1;
                float bestA = -1.0f;
                for (size_t j = 0; j < e.size(); ++j) {
                    if (e[j].cnt != 0)
                        continue;
                    float A = sa8(e[j]);
                    if (A > bestA) {
                        bestA = A;
                        best = (int)j;
                    }
                }
                if (best < 0)
                    break;
                Entry8 l, r;
                child(e[best].ref, 0, l);
                child(e[best].ref, 1, r);
                e[best] = l;
                e.push_back(r);
            }
            int k = 0, t = 0;
            for (auto &x : e) {
                if (x.cnt == 0)
                    ++k;
                else
                    t += x.cnt;
            }
            scanK[i + 1] = scanK[i] + k;
            scanT[i + 1] = scanT[i] + t;
        }
        const int nextStart = levelStart + (int)items.size();
        std::vector<int> next(scanK.back());
        out.resize(nextStart);
        for (size_t i = 0; i < items.size(); ++i) {
            const std::vector<Entry8> &e = ents[i];
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (auto &x : e)
                for (int k = 0; k < 3; ++k) {
                    lo[k] = std::fmin(lo[k], x.lo[k]);
                    hi[k] = std::fmax(hi[k], x.hi[k]);
                }
            float cen[3];
            for (int k = 0; k < 3; ++k)
                cen[k] = (lo[k] + hi[k]) * 0.5f;
            int refAt[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
            uint32_t used = 0;
            for (size_t j = 0; j < e.size(); ++j) {
                uint32_t code = 0;
                for (int k = 0; k < 3; ++k)
                    if ((e[j].lo[k] + e[j].hi[k]) * 0.5f > cen[k])
                        code |= 1u << k;
                int slot = -1;
                if (!((used >> code) & 1u)) {
                    slot = (int)code;
                } else {
                    int bestD = 99;
                    for (int s = 0; s < 8; ++s) {
                        if ((used >> s) & 1u)
                            continue;
                        int dd = __builtin_popcount((unsigned)s ^ code);
                        if (dd < bestD) {
                            bestD = dd;
                            slot = s;
                        }
                    }
                }
                used |= 1u << slot;
                refAt[slot] = (int)j;
            }
            int ex[3];
            for (int k = 0; k < 3; ++k)
                ex[k] = scaleExp(subUp(hi[k], lo[k]));
            uint32_t meta[8] = {0, 0, 0, 0, 0, 0, 0, 0}, ql[3][8] = {}, qh[3][8] = {};
            uint32_t imask = 0;
            const int childBase = nextStart + scanK[i], triBase = triStart + scanT[i];
            int rank = 0, toff = 0;
            for (int s = 0; s < 8; ++s) {
                const int j = refAt[s];
                if (j < 0)
                    continue;
                for (int k = 0; k < 3; ++k) {
                    const float inv = std::ldexp(1.0f, -ex[k]);
                    float a = std::floor(subDown(e[j].lo[k], lo[k]) * inv);
                    float b = std::ceil(subUp(e[j].hi[k], lo[k]) * inv);
                    a = a > 0.0f ? a - 1.0f : 0.0f;
                    b = std::fmin(b + 1.0f, 255.0f);
                    ql[k][s] = (uint32_t)a;
                    qh[k][s] = (uint32_t)std::fmax(b, 0.0f);
                }
                if (e[j].cnt == 0) {
                    imask |= 1u << s;
                    meta[s] = 1u;
                    next[scanK[i] + rank] = e[j].ref;
                    ++rank;
                } else {
                    meta[s] = ((uint32_t)e[j].cnt << 5) | (uint32_t)toff;
                    for (int c = 0; c < e[j].cnt; ++c)
                        order8[triBase + toff + c] = B.tris[e[j].ref + c].prim;
                    toff += e[j].cnt;
                }
            }
            Node8 &N = out[levelStart + i];
            N.p[0] = lo[0];
            N.p[1] = lo[1];
            N.p[2] = lo[2];
            N.ew = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) | ((uint32_t)(ex[2] + 127) << 16) |
                   (imask << 24);
            N.childBase = (uint32_t)childBase;
            N.triBase = (uint32_t)triBase;
            N.meta0 = meta[0] | meta[1] << 8 | meta[2] << 16 | meta[3] << 24;
            N.meta1 = meta[4] | meta[5] << 8 | meta[6] << 16 | meta[7] << 24;
            for (int k = 0; k < 3; ++k) {
                N.q[k][0] = ql[k][0] | ql[k][1] << 8 | ql[k][2] << 16 | ql[k][3] << 24;
                N.q[k][1] = ql[k][4] | ql[k][5] << 8 | ql[k][6] << 16 | ql[k][7] << 24;
                N.q[k][2] = qh[k][0] | qh[k][1] << 8 | qh[k][2] << 16 | qh[k][3] << 24;
                N.q[k][3] = qh[k][4] | qh[k][5] << 8 | qh[k][6] << 16 | qh[k][7] << 24;
            }
        }
        triStart += scanT.back();
        items.swap(next);
    }
}

// ------------------------------------------------------------------ scene view
struct SceneView {
    const optpt_scene *s;
    HostBvh bvh;
    std::vector<int> emissive;  // triangle ids
    float srgb[256];
};

float boxEntry(const Box &b, F3 o, F3 inv, float tmin, float tmax)
{
    float tn = tmin, tf = INFINITY;
    const float oo[3] = {o.x, o.y, o.z}, iv[3] = {inv.x, inv.y, inv.z};
    for (int k = 0; k < 3; ++k) {
        float a = (b.lo[k] - oo[k]) * iv[k], c = (b.hi[k] - oo[k]) * iv[k];
        tn = std::fmax(tn, std::fmin(a, c));
        tf = std::fmin(tf, std::fmax(a, c));
    }
    // widened by 2^-19 so equal-t candidates reach the index tie-break
    return tn <= std::fmin(tf, tmax) * 1.0000019f ? tn : INFINITY;
}
float safeInv(float d) { return 1.0f / (std::fabs(d) > 1e-20f ? d : std::copysign(1e-20f, d)); }

float texFetch(const optpt_texture &t, const float *lut, int x, int y, int c);

// Alpha of a candidate (cu/device_programs.cu:108-166, 180-219): baseColour.w
// times the base-colour texture alpha at the untransformed coordinate.
struct AlphaCtx {
    const SceneView *sv;
    uint32_t seed, pixel, sample, depth;
    float shadowXi;  // < 0: radiance ray
};
float sampleTex(const SceneView &sv, int tex, float u, float v, float out[4]);
// w t0 + u t1 + v t2 with w = 1 - u - v, as the same fused multiply-adds the
// device uses, so texture lookups agree bit for bit.
template <class R> R baryInterp(R u, R v, R t0, R t1, R t2)
{
    const R w = (R(1) - u) - v;
    return std::fma(v, t2, std::fma(u, t1, w * t0));
}
bool alphaAccept(const AlphaCtx &a, int prim, float u, float v)
{
    const optpt_scene *s = a.sv->s;
    const MaterialData &M = s->materials[s->matIndices[prim]];
    if (M.alphaMode == AM_OPAQUE)
        return true;
    float alpha = M.baseColour[3];
    if (M.hasBaseColourTexture && M.baseColourTexture >= 0 && s->texCoords) {
        const int *I = s->triIndices + 3 * prim;
        float tu = baryInterp(u, v, s->texCoords[2 * I[0]], s->texCoords[2 * I[1]], s->texCoords[2 * I[2]]);
        float tv = baryInterp(u, v, s->texCoords[2 * I[0] + 1], s->texCoords[2 * I[1] + 1], s->texCoords[2 * I[2] + 1]);
        float c[4];
        sampleTex(*a.sv, M.baseColourTexture, tu, tv, c);
        alpha *= c[3];
    }
    if (M.alphaMode == AM_MASK)
        return !(alpha < M.alphaCutoff);
    float xi = a.shadowXi >= 0.0f ? a.shadowXi : blendUniform(a.seed, a.pixel, a.sample, a.depth, (uint32_t)prim);
    return !(xi > alpha);
}

struct HitH {
    float t, u, v;
    int prim;  // -1 = miss
};

// Closest (any = false) or first accepted (any = true) hit.
bool traverse(const SceneView &sv, F3 o, F3 d, float tmin, float tmax, bool any, const AlphaCtx &ac, HitH &hit,
              uint64_t *nodeVisits = nullptr, uint64_t *triTests = nullptr)
{
    hit.prim = -1;
    const HostBvh &B = sv.bvh;
    if (B.tris.empty())
        return false;
    const RayPre pre = rayPrepare(o, d);
    const F3 inv{safeInv(d.x), safeInv(d.y), safeInv(d.z)};
    int stack[64];
    int sp = 0, node = 0;
    float tcur = tmax;
    int bestPrim = INT_MAX;
    while (true) {
        if (nodeVisits)
            ++*nodeVisits;
        const int *N = &B.nodes4[4 * (size_t)node];
        float tl = N[0] >= 0 ? boxEntry(B.nodeBoxL[node], o, inv, tmin, tcur) : INFINITY;
        float tr = N[1] >= 0 ? boxEntry(B.nodeBoxR[node], o, inv, tmin, tcur) : INFINITY;
        bool hl = tl != INFINITY, hr = tr != INFINITY;
        for (int side = 0; side < 2; ++side) {
            bool h = side == 0 ? hl : hr;
            int cnt = N[2 + side];
            if (!h || cnt == 0)
                continue;
            int first = N[side];
            for (int k = first; k < first + cnt; ++k) {
                if (triTests)
                    ++*triTests;
                float t, u, v;
                if (!intersectTri(pre, B.tris[k], tmin, tcur, t, u, v))
                    continue;
                int prim = B.tris[k].prim;
                if (!alphaAccept(ac, prim, u, v))
                    continue;
                if (any) {
                    hit = HitH{t, u, v, prim};
                    return true;
                }
                if (t < tcur || prim < bestPrim) {
                    tcur = t;
                    bestPrim = prim;
                    hit = HitH{t, u, v, prim};
                }
            }
            (side == 0 ? hl : hr) = false;
        }
        if (hl && hr) {
            bool lf = tl <= tr;
            if (sp < 64)
                stack[sp++] = lf ? N[1] : N[0];
            node = lf ? N[0] : N[1];
        } else if (hl) {
            node = N[0];
        } else if (hr) {
            node = N[1];
        } else {
            if (sp == 0)
                break;
            node = stack[--sp];
        }
    }
    return hit.prim >= 0;
}

// ------------------------------------------------------------------ textures
// Bilinear (or point) RGBA8 sampling with wrap modes and sRGB decode; the
// texture-unit behaviour of src/renderer.cpp:1439-1757 with FP32 weights.
int wrapTexel(int i, int n, int mode)
{
    if (mode == 1)
        return std::min(std::max(i, 0), n - 1);
    if (mode == 2) {
        int p = 2 * n, m = ((i % p) + p) % p;
        return m < n ? m : p - 1 - m;
    }
    return ((i % n) + n) % n;
}
float texChan(const SceneView &sv, const optpt_texture &t, int x, int y, int c)
{
    uint8_t b = t.rgba[4 * ((size_t)y * t.width + x) + c];
    if (c < 3 && t.srgb)
        return sv.srgb[b];
    return (float)b * (1.0f / 255.0f);
}
float sampleTex(const SceneView &sv, int tex, float u, float v, float out[4])
{
    const optpt_texture &t = sv.s->textures[tex];
    const int W = (int)t.width, H = (int)t.height;
    if (t.filter == 1) {
        // Nearest texel (cudaFilterModePoint): floor(u * W), floor(v * H).
        const int px = wrapTexel((int)std::floor(u * (float)W), W, t.wrapS);
        const int py = wrapTexel((int)std::floor(v * (float)H), H, t.wrapT);
        for (int c = 0; c < 4; ++c)
            out[c] = texChan(sv, t, px, py, c);
        return out[3];
    }
    const float x = std::fma(u, (float)W, -0.5f), y = std::fma(v, (float)H, -0.5f);
    float fx0 = std::floor(x), fy0 = std::floor(y);
    float ax = x - fx0, ay = y - fy0;
    int x0 = (int)fx0, y0 = (int)fy0;
    int xa = wrapTexel(x0, W, t.wrapS), xb = wrapTexel(x0 + 1, W, t.wrapS);
    int ya = wrapTexel(y0, H, t.wrapT), yb = wrapTexel(y0 + 1, H, t.wrapT);
    for (int c = 0; c < 4; ++c) {
        float c00 = texChan(sv, t, xa, ya, c), c10 = texChan(sv, t, xb, ya, c);
        float c01 = texChan(sv, t, xa, yb, c), c11 = texChan(sv, t, xb, yb, c);
        const float top = std::fma(c10 - c00, ax, c00), bot = std::fma(c11 - c01, ax, c01);
        out[c] = std::fma(bot - top, ay, top);
    }
    return out[3];
}

// ------------------------------------------------------------------ integrator
template <class R> struct PcgU {
    Pcg *p;
    R next() { return R(p->uniform()); }
};

template <class R> V3<R> v3f(const float *p) { return orc::v3<R>(R(p[0]), R(p[1]), R(p[2])); }
template <class R> F3 tof(V3<R> a) { return F3{(float)a.x, (float)a.y, (float)a.z}; }

struct RenderParams {
    uint32_t w, h, seed, sampleBase, spp, maxDepth;
    float eye[3], U[3], V[3], W[3], bg[3];
    int vis;  // LaunchParams::vis: 0 = path tracing, 1-12 = material visualisation
};

struct Counters {
    uint64_t ext = 0, shadow = 0, nodes = 0, tris = 0;
};

// One path sample (cu/device_programs.cu:15-106 with cu/path_tracer.cu:17-582).
template <class R>
V3<R> tracePath(const SceneView &sv, const RenderParams &rp, uint32_t pixel, uint32_t sample, Counters &cnt)
{
    using namespace orc;
    const optpt_scene *s = sv.s;
    const uint32_t x = pixel % rp.w, y = pixel / rp.w;
    Pcg r0 = pathRng(rp.seed, pixel, sample, 0);
    const float jx = r0.uniform(), jy = r0.uniform();
    const R fx = R((float)x + jx), fy = R((float)y + jy);
    const R ndcx = (fx / R(rp.w)) * R(2) + R(-1);
    const R ndcy = (fy / R(rp.h)) * R(-2) + R(1);
    V3<R> dir = normalize(ndcx * v3f<R>(rp.U) + ndcy * v3f<R>(rp.V) + v3f<R>(rp.W));
    V3<R> org = v3f<R>(rp.eye);
    V3<R> T = v3s<R>(R(1)), L = v3s<R>(R(0));
    bool prevSpecular = false;
    for (uint32_t depth = 1; depth <= rp.maxDepth; ++depth) {
        AlphaCtx ac{&sv, rp.seed, pixel, sample, depth, -1.0f};
        HitH hit;
        ++cnt.ext;
        if (!traverse(sv, tof(org), tof(dir), 0.0f, 1e16f, false, ac, hit, &cnt.nodes, &cnt.tris)) {
            L = L + v3f<R>(rp.bg) * T;  // __miss__radiance (cu/device_programs.cu:168-174)
            break;
        }
        Pcg rng = pathRng(rp.seed, pixel, sample, depth);
        PcgU<R> U{&rng};
        const int prim = hit.prim;
        const MaterialData &M = s->materials[s->matIndices[prim]];
        const int *I = s->triIndices + 3 * prim;
        const R u = R(hit.u), v = R(hit.v);
        const V3<R> rayDir = dir;
        V3<R> hitPoint = org + R(hit.t) * rayDir;
        const V3<R> p0 = v3f<R>(s->positions + 3 * I[0]), p1 = v3f<R>(s->positions + 3 * I[1]),
                    p2 = v3f<R>(s->positions + 3 * I[2]);
        const V3<R> Ng = normalize(cross(p1 - p0, p2 - p0));
        V3<R> interpN = Ng;
        bool hasN = false;
        if (s->normals) {
            interpN = normalize((R(1) - u - v) * v3f<R>(s->normals + 3 * I[0]) + u * v3f<R>(s->normals + 3 * I[1]) +
                                v * v3f<R>(s->normals + 3 * I[2]));
            hasN = true;
        }
        R tcu = R(0), tcv = R(0);
        const bool anyTex = M.hasBaseColourTexture || M.hasNormalTexture || M.hasMetallicRoughnessTexture ||
                            M.hasEmissiveTexture || M.hasSheenColourTexture || M.hasSheenRoughnessTexture;
        if (anyTex && s->texCoords) {
            tcu = baryInterp<R>(u, v, R(s->texCoords[2 * I[0]]), R(s->texCoords[2 * I[1]]), R(s->texCoords[2 * I[2]]));
            tcv = baryInterp<R>(u, v, R(s->texCoords[2 * I[0] + 1]), R(s->texCoords[2 * I[1] + 1]),
                                R(s->texCoords[2 * I[2] + 1]));
        }
        auto tex = [&](int id, const TextureTransform &tf, float out[4]) {
            float tu = (float)std::fma(tcu, R(tf.scale[0]), R(tf.offset[0]));
            float tv = (float)std::fma(tcv, R(tf.scale[1]), R(tf.offset[1]));
            sampleTex(sv, id, tu, tv, out);
        };
        V3<R> normal = interpN;
        if (M.hasNormalTexture && s->texCoords) {  // cu/path_tracer.cu:64-144
            float c[4];
            tex(M.normalTexture, M.normalTexTf, c);
            V3<R> sn = normalize(v3<R>(R(c[0]) * R(2) - R(1), R(c[1]) * R(2) - R(1), R(c[2]) * R(2) - R(1)));
            const float *w0 = s->texCoords + 2 * I[0], *w1 = s->texCoords + 2 * I[1], *w2 = s->texCoords + 2 * I[2];
            const V3<R> e1 = p1 - p0, e2 = p2 - p0;
            const R d1x = R(w1[0]) - R(w0[0]), d1y = R(w1[1]) - R(w0[1]);
            const R d2x = R(w2[0]) - R(w0[0]), d2y = R(w2[1]) - R(w0[1]);
            const R f = R(1) / (d1x * d2y - d2x * d1y);
            V3<R> tl = normalize(v3<R>(f * (d2y * e1.x - d1y * e2.x), f * (d2y * e1.y - d1y * e2.y),
                                       f * (d2y * e1.z - d1y * e2.z)));
            const V3<R> N = hasN ? interpN : Ng;
            const V3<R> Tg = normalize(tl - dot(tl, N) * N);
            const V3<R> Bt = cross(N, Tg);
            normal = normalize(v3<R>(Tg.x * sn.x + Bt.x * sn.y + N.x * sn.z, Tg.y * sn.x + Bt.y * sn.y + N.y * sn.z,
                                     Tg.z * sn.x + Bt.z * sn.y + N.z * sn.z));
        }
        // Material inputs after textures (cu/path_tracer.cu:165-229).
        V3<R> albedo = v3f<R>(M.baseColour);
        R alpha = R(M.baseColour[3]);
        if (M.hasBaseColourTexture) {
            float c[4];
            tex(M.baseColourTexture, M.baseColourTexTf, c);
            albedo = albedo * v3<R>(R(c[0]), R(c[1]), R(c[2]));
            alpha *= R(c[3]);
        }
        R roughness = R(M.roughness), metallic = R(M.metallic), occlusion = R(1);
        if (M.hasMetallicRoughnessTexture) {
            float c[4];
            tex(M.metallicRoughnessTexture, M.metallicRoughnessTexTf, c);
            occlusion *= R(c[0]);
            roughness *= R(c[1]);
            metallic = c[2] < 0.04f ? R(0) : metallic * R(c[2]);
        }
        V3<R> emission = v3f<R>(M.emission);
        if (M.hasEmissiveTexture) {
            float c[4];
            tex(M.emissiveTexture, M.emissiveTexTf, c);
            emission = emission * v3<R>(R(c[0]), R(c[1]), R(c[2]));
        }
        V3<R> sheenColour = v3f<R>(M.sheenColour);
        if (M.hasSheenColourTexture) {
            float c[4];
            tex(M.sheenColourTexture, M.sheenColourTexTf, c);
            sheenColour = sheenColour * v3<R>(R(c[0]), R(c[1]), R(c[2]));
        }
        R sheenRoughness = R(M.sheenRoughness);
        if (M.hasSheenRoughnessTexture) {
            float c[4];
            tex(M.sheenRoughnessTexture, M.sheenRoughnessTexTf, c);
            sheenRoughness *= R(c[3]);
        }
        MatCat<R> mc{M.category, R(M.coatWeight), R(M.coatRoughness), R(M.transmissionWeight), R(M.specular),
                     R(M.subsurfaceWeight)};
        R cw;
        const uint32_t cat =
            categorise(mc, -rayDir, normal, roughness, metallic, emission, sheenColour, sheenRoughness, U, cw);
        if (rp.vis != 0) {  // material visualisation: the path ends here (cu/path_tracer.cu:252-315)
            switch (rp.vis) {
            case 1: L = v3s<R>(metallic); break;
            case 2: L = v3s<R>(roughness); break;
            case 3: L = v3s<R>(occlusion); break;
            case 4: L = emission; break;
            case 5: L = normal * R(0.5f) + v3s<R>(R(0.5f)); break;
            case 6: L = Ng * R(0.5f) + v3s<R>(R(0.5f)); break;
            case 7: L = albedo; break;
            case 8: L = metallic * albedo * v3s<R>(R(M.specular)); break;  // "glossy colour"
            case 10: L = sheenColour; break;
            case 11: L = v3s<R>(sheenRoughness); break;
            case 12: L = v3s<R>(alpha); break;
            default: break;  // 9 (specular colour) is unfinished in the reference: radiance unchanged
            }
            break;
        }
        const bool spec = (cat & Specular) != 0;
        if (!spec)
            hitPoint = hitPoint - rayDir * R(0.001f);
        if (cat & Emission) {  // cu/path_tracer.cu:324-339
            if (dot(rayDir, normal) < R(0) && (depth == 1 || prevSpecular))
                L = L + (emission + albedo * T);
            break;
        }
        prevSpecular = spec;
        const MatMR<R> m = makeMatMR(albedo, R(M.ior), metallic, R(M.specular), R(M.transmissionWeight),
                                     R(M.subsurfaceWeight), R(M.coatWeight), sheenColour, cat, normal, roughness,
                                     R(M.coatRoughness), R(M.sheenRoughness));
        const V3<R> wo = -rayDir;
        if (!spec && s->numLights != 0) {  // cu/path_tracer.cu:375-412, cu/light_sampling.cu:6-59
            const R lu = U.next();
            const int li = std::min((int)(float)(lu * R(s->numLights)), (int)s->numLights - 1);
            const R selPdf = R(1) / R(s->numLights);
            const Light &Lt = s->lights[li];
            V3<R> ldir, Li;
            R ldist;
            if (Lt.type == LIGHT_TYPE_DIRECTIONAL) {
                const V3<R> n = v3f<R>(Lt.normal);
                const V3<R> pos = hitPoint + (-n * R(Lt.distance));
                ldir = -n;
                Li = v3f<R>(Lt.radiance);
                ldist = length(pos - hitPoint);
            } else {
                ldir = v3f<R>(Lt.p0) - hitPoint;
                ldist = length(ldir);
                ldir = ldir / ldist;
                R fo = R(1);
                if (Lt.type == LIGHT_TYPE_SPOT) {
                    const R ct = dot(v3f<R>(Lt.normal), -ldir);
                    if (ct < R(Lt.cosWidth))
                        fo = R(0);
                    else if (ct > R(Lt.cosFalloffStart))
                        fo = R(1);
                    else {
                        const R dl = (ct - R(Lt.cosWidth)) / (R(Lt.cosFalloffStart) - R(Lt.cosWidth));
                        fo = (dl * dl) * (dl * dl);
                    }
                    Li = v3f<R>(Lt.radiance) * fo / (ldist * ldist);
                } else {
                    Li = v3f<R>(Lt.radiance) / (ldist * ldist);
                }
            }
            const R cosX = std::fmax(dot(normal, ldir), R(0));
            const float sxi = (float)U.next();
            const V3<R> brdf = mrBrdf(m, ldir, wo, U);
            const V3<R> colour = brdf * Li * cosX / R(1) / selPdf;
            const V3<R> c = colour * T;
            if (c.x != R(0) || c.y != R(0) || c.z != R(0) || !std::isfinite(c.x) || !std::isfinite(c.y) ||
                !std::isfinite(c.z)) {
                AlphaCtx sc{&sv, rp.seed, pixel, sample, depth, sxi};
                HitH sh;
                ++cnt.shadow;
                const bool occ = traverse(sv, tof(hitPoint), tof(ldir), 0.0001f, (float)(ldist - R(0.0001f)), true,
                                          sc, sh, &cnt.nodes, &cnt.tris);
                L = L + (occ ? c * R(0) : c);
            }
        }
        if (!spec && !sv.emissive.empty()) {  // cu/path_tracer.cu:415-515
            const int ne = (int)sv.emissive.size();
            const int ei = std::min((int)(float)(U.next() * R(ne)), ne - 1);
            const R selPdf = R(1) / R(ne);
            R xa = U.next(), xb = U.next();
            if (xa + xb > R(1)) {
                xa = R(1) - xa;
                xb = R(1) - xb;
            }
            const int et = sv.emissive[ei];
            const int *EI = s->triIndices + 3 * et;
            const V3<R> q0 = v3f<R>(s->positions + 3 * EI[0]), q1 = v3f<R>(s->positions + 3 * EI[1]),
                        q2 = v3f<R>(s->positions + 3 * EI[2]);
            const V3<R> e1 = q1 - q0, e2 = q2 - q0;
            const V3<R> lightPos = q0 + e1 * xa + e2 * xb;
            const V3<R> lnv = cross(e1, e2);
            const V3<R> ln = normalize(lnv);
            const R pdfA = R(1) / (length(lnv) * R(0.5));
            const V3<R> lvec = lightPos - hitPoint;
            const R dist = length(lvec);
            const V3<R> ldir = lvec / dist;
            const R cosY = std::fmax(R(0), dot(ln, -ldir));
            const MaterialData &EM = s->materials[s->matIndices[et]];
            V3<R> Le = v3f<R>(EM.emission);
            if (EM.hasEmissiveTexture && s->texCoords) {
                // Barycentrics (include/barycentrics.h:17-44); the HIT material's
                // transform is applied (cu/path_tracer.cu:466-468).
                const V3<R> mm = cross(q1 - q0, q2 - q0);
                const R ax = std::fabs(mm.x), ay = std::fabs(mm.y), az = std::fabs(mm.z);
                auto area2 = [](R x1, R y1, R x2, R y2, R x3, R y3) { return (x1 - x2) * (y2 - y3) - (x2 - x3) * (y1 - y2); };
                R nu, nv, ood;
                const V3<R> &P = lightPos;
                if (ax >= ay && ax >= az) {
                    nu = area2(P.y, P.z, q1.y, q1.z, q2.y, q2.z);
                    nv = area2(P.y, P.z, q2.y, q2.z, q0.y, q0.z);
                    ood = R(1) / mm.x;
                } else if (ay >= ax && ay >= az) {
                    nu = area2(P.x, P.z, q1.x, q1.z, q2.x, q2.z);
                    nv = area2(P.x, P.z, q2.x, q2.z, q0.x, q0.z);
                    ood = R(1) / -mm.y;
                } else {
                    nu = area2(P.x, P.y, q1.x, q1.y, q2.x, q2.y);
                    nv = area2(P.x, P.y, q2.x, q2.y, q0.x, q0.y);
                    ood = R(1) / mm.z;
                }
                const R bu = nu * ood, bv = nv * ood;
                const float *c0 = s->texCoords + 2 * EI[0], *c1 = s->texCoords + 2 * EI[1], *c2 = s->texCoords + 2 * EI[2];
                const R etu = baryInterp<R>(bu, bv, R(c0[0]), R(c1[0]), R(c2[0]));
                const R etv = baryInterp<R>(bu, bv, R(c0[1]), R(c1[1]), R(c2[1]));
                float c[4];
                sampleTex(sv, EM.emissiveTexture, (float)std::fma(etu, R(M.emissiveTexTf.scale[0]), R(M.emissiveTexTf.offset[0])),
                          (float)std::fma(etv, R(M.emissiveTexTf.scale[1]), R(M.emissiveTexTf.offset[1])), c);
                Le = Le * v3<R>(R(c[0]), R(c[1]), R(c[2]));
            }
            const R cosX = std::fmax(R(0), dot(normal, ldir));
            const R G = cosX * cosY / (dist * dist);
            const float sxi = (float)U.next();
            const V3<R> brdf = mrBrdf(m, ldir, wo, U);
            const V3<R> colour = Le * brdf * G / (pdfA * selPdf);
            const V3<R> c = colour * T;
            if (c.x != R(0) || c.y != R(0) || c.z != R(0) || !std::isfinite(c.x) || !std::isfinite(c.y) ||
                !std::isfinite(c.z)) {
                AlphaCtx sc{&sv, rp.seed, pixel, sample, depth, sxi};
                HitH sh;
                ++cnt.shadow;
                const bool occ = traverse(sv, tof(hitPoint), tof(ldir), 0.0001f, (float)(dist - R(0.0001f)), true, sc,
                                          sh, &cnt.nodes, &cnt.tris);
                L = L + (occ ? c * R(0) : c);
            }
        }
        if (depth == rp.maxDepth)
            break;
        V3<R> xi;  // cu/path_tracer.cu:522-581
        xi.x = U.next();
        xi.y = U.next();
        xi.z = U.next();
        Sample<R> smp;
        smp.dir = v3s<R>(R(0));
        smp.bsdf = v3s<R>(R(0));
        smp.pdf = R(0);
        mrSample(m, wo, xi, U, smp);
        smp.pdf = smp.pdf * cw;
        if (smp.pdf < R(0.0001f) || maxc(smp.bsdf) < R(0.0001f))
            break;
        T = T * (smp.bsdf * std::fabs(dot(normal, smp.dir)) / smp.pdf);
        const R maxC = maxc(T);
        if (depth > 3 || maxC < R(0.3f)) {
            const R q = std::fmax(R(0.05f), R(1) - maxC);
            if (U.next() < q)
                break;
            T = T / (R(1) - q);
        }
        if (!spec)
            hitPoint = hitPoint + rayDir * R(0.001f);
        org = hitPoint + smp.dir * R(0.0001f);
        dir = smp.dir;
    }
    return L;
}

SceneView *makeView(const optpt_scene *s, int leafSize)
{
    SceneView *sv = new SceneView();
    sv->s = s;
    buildHostBvh(s->positions, s->triIndices, (int)s->numTriangles, leafSize, sv->bvh);
    for (uint32_t t = 0; t < s->numTriangles; ++t) {
        const MaterialData &m = s->materials[s->matIndices[t]];
        if (m.emission[0] > 0.0f || m.emission[1] > 0.0f || m.emission[2] > 0.0f || m.hasEmissiveTexture)
            sv->emissive.push_back((int)t);
    }
    for (int i = 0; i < 256; ++i) {
        double c = i / 255.0;
        sv->srgb[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
    }
    return sv;
}

}  // namespace

extern "C" {

void *orc_scene_view(const optpt_scene *s, int leafSize) { return makeView(s, leafSize); }
void orc_scene_view_free(void *sv) { delete (SceneView *)sv; }

// LBVH products: sorted codes, leaf order (primitive per sorted position),
// nodes4 (ref0, ref1, cnt0, cnt1 per internal slot), node/leaf counts.
int orc_bvh(void *view, uint32_t *codes, int32_t *order, int32_t *nodes4, uint32_t capacity, uint32_t *counts)
{
    const HostBvh &B = ((SceneView *)view)->bvh;
    const size_t n = B.codes.size();
    if (codes)
        memcpy(codes, B.codes.data(), n * 4);
    if (order)
        memcpy(order, B.order.data(), n * 4);
    counts[0] = (uint32_t)(B.nodes4.size() / 4);
    counts[1] = (uint32_t)B.usedNodes;
    counts[2] = (uint32_t)B.leaves;
    if (nodes4) {
        if (capacity < counts[0])
            return -1;
        memcpy(nodes4, B.nodes4.data(), B.nodes4.size() * 4);
    }
    return 0;
}

// The compressed 8-wide BVH collapsed from this view's BVH2: 80-byte nodes and
// the primitive of every triangle slot. counts[0] = nodes.
int orc_bvh8(void *view, void *nodes, uint32_t capacity, int32_t *order8, uint32_t *counts)
{
    const SceneView &sv = *(SceneView *)view;
    std::vector<Node8> out;
    std::vector<int> ord;
    buildHostBvh8(sv.bvh, out, ord);
    counts[0] = (uint32_t)out.size();
    if (nodes) {
        if (capacity < out.size())
            return -1;
        memcpy(nodes, out.data(), out.size() * sizeof(Node8));
    }
    if (order8)
        memcpy(order8, ord.data(), ord.size() * sizeof(int));
    return 0;
}

// rays: 8 floats per ray (origin, tmin, direction, tmax); hits: (t, u, v, prim bits).
int orc_trace(void *view, const float *rays, float *hits, uint32_t n, int anyHit, int threads)
{
    const SceneView &sv = *(SceneView *)view;
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
        AlphaCtx ac{&sv, 0, 0, 0, 0, anyHit ? 0.5f : -1.0f};
        for (uint32_t i; (i = next.fetch_add(256)) < n;) {
            for (uint32_t k = i; k < std::min(n, i + 256); ++k) {
                const float *r = rays + 8 * (size_t)k;
                HitH h;
                bool hit = traverse(sv, F3{r[0], r[1], r[2]}, F3{r[4], r[5], r[6]}, r[3], r[7], anyHit != 0, ac, h);
                float *o = hits + 4 * (size_t)k;
                o[0] = hit ? h.t : INFINITY;
                o[1] = hit ? h.u : 0.0f;
                o[2] = hit ? h.v : 0.0f;
                int p = hit ? h.prim : -1;
                memcpy(o + 3, &p, 4);
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < std::max(1, threads); ++t)
        pool.emplace_back(work);
    work();
    for (auto &t : pool)
        t.join();
    return 0;
}

// Renders `spp` samples per pixel for rows [y0, y1) into FP64 sum / sum of
// squares (3 doubles per pixel each, for the whole image) using `threads`
// host threads. precision: 32 or 64. counters: ext rays, shadow rays, BVH
// nodes visited, triangle tests.
int orc_render(void *view, const float *camera /* eye U V W bg: 15 floats */, uint32_t w, uint32_t h, uint32_t seed,
               uint32_t sampleBase, uint32_t spp, uint32_t maxDepth, uint32_t y0, uint32_t y1, int precision,
               int threads, double *sum, double *sumSq, uint64_t *counters, int vis)
{
    const SceneView &sv = *(SceneView *)view;
    RenderParams rp{};
    rp.w = w;
    rp.h = h;
    rp.seed = seed;
    rp.sampleBase = sampleBase;
    rp.spp = spp;
    rp.maxDepth = maxDepth;
    rp.vis = vis;
    memcpy(rp.eye, camera, 12);
    memcpy(rp.U, camera + 3, 12);
    memcpy(rp.V, camera + 6, 12);
    memcpy(rp.W, camera + 9, 12);
    memcpy(rp.bg, camera + 12, 12);
    std::atomic<uint32_t> nextRow{y0};
    std::vector<Counters> percnt(std::max(1, threads));
    auto work = [&](int tid) {
        Counters &c = percnt[tid];
        for (uint32_t y; (y = nextRow.fetch_add(1)) < y1;) {
            for (uint32_t x = 0; x < w; ++x) {
                const uint32_t px = y * w + x;
                double S[3] = {0, 0, 0}, Q[3] = {0, 0, 0};
                uint32_t n = 0;
                for (uint32_t s = 0; s < spp; ++s) {
                    double L[3];
                    if (precision == 64) {
                        V3<double> l = tracePath<double>(sv, rp, px, sampleBase + s, c);
                        L[0] = l.x; L[1] = l.y; L[2] = l.z;
                    } else {
                        V3<float> l = tracePath<float>(sv, rp, px, sampleBase + s, c);
                        L[0] = l.x; L[1] = l.y; L[2] = l.z;
                    }
                    if (std::isnan(L[0]) || std::isnan(L[1]) || std::isnan(L[2])) {
                        for (int k = 0; k < 3; ++k)
                            L[k] = n ? S[k] / n : 0.0;
                    }
                    for (int k = 0; k < 3; ++k) {
                        S[k] += L[k];
                        Q[k] += L[k] * L[k];
                    }
                    ++n;
                }
                for (int k = 0; k < 3; ++k) {
                    sum[3 * (size_t)px + k] += S[k];
                    sumSq[3 * (size_t)px + k] += Q[k];
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < std::max(1, threads); ++t)
        pool.emplace_back(work, t);
    work(0);
    for (auto &t : pool)
        t.join();
    if (counters) {
        for (auto &c : percnt) {
            counters[0] += c.ext;
            counters[1] += c.shadow;
            counters[2] += c.nodes;
            counters[3] += c.tris;
        }
    }
    return 0;
}

}  // extern "C"
