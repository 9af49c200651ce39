// Collapse of the LBVH (BVH2) into the compressed 8-wide BVH of bvh8.cuh, on
// the GPU, one tree level per step:
//   1. every BVH2 node that becomes a BVH8 node opens its children greedily,
//      always the internal child of largest surface area, until 8 entries or
//      only leaves remain;
//   2. exclusive prefix sums over the items' internal-child and triangle
//      counts place each node's children and triangles (so the layout is
//      deterministic and reproducible on the host);
//   3. each node is quantised (per-axis power-of-two scale, 8-bit child
//      boxes rounded outwards by one step), its children are put in the slots
//      of their centroid octants, and its leaf triangles are copied next to
//      each other in slot order.
#include <cub/cub.cuh>
#include "bvh8.cuh"
#include "engine.h"

namespace {

struct Entry {
    int ref;  // BVH2 node (cnt == 0) or first sorted triangle (cnt > 0)
    int cnt;
    float lo[3], hi[3];
};

OPT_D float surfaceArea(const Entry &e)
{
    const float dx = e.hi[0] - e.lo[0], dy = e.hi[1] - e.lo[1], dz = e.hi[2] - e.lo[2];
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx));
}

OPT_D void childOf(const BvhNode &N, int side, Entry &e)
{
    e.ref = side == 0 ? N.d.x : N.d.y;
    e.cnt = side == 0 ? N.d.z : N.d.w;
    if (side == 0) {
        e.lo[0] = N.a.x; e.hi[0] = N.a.y; e.lo[1] = N.a.z; e.hi[1] = N.a.w; e.lo[2] = N.c.x; e.hi[2] = N.c.y;
    } else {
        e.lo[0] = N.b.x; e.hi[0] = N.b.y; e.lo[1] = N.b.z; e.hi[1] = N.b.w; e.lo[2] = N.c.z; e.hi[2] = N.c.w;
    }
}

__global__ void kCollapseOpen(const BvhNode *__restrict__ n2, const int *__restrict__ items, int nItems,
                              Entry *__restrict__ ent, int *__restrict__ nEnt, int *__restrict__ kInt,
                              int *__restrict__ nTri)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nItems)
        return;
    Entry e[8];
    int ne = 0;
    const BvhNode N = n2[items[i]];
    for (int side = 0; side < 2; ++side) {
        Entry c;
        childOf(N, side, c);
        if (c.ref >= 0)
            e[ne++] = c;
    }
    while (ne < 8) {
        int best = -1;
        float bestA = -1.0f;
        for (int j = 0; j < ne; ++j) {
            if (e[j].cnt != 0)
                continue;
            const float A = surfaceArea(e[j]);
            if (A > bestA) {
                bestA = A;
                best = j;
            }
        }
        if (best < 0)
            break;
        const BvhNode C = n2[e[best].ref];
        Entry l, r;
        childOf(C, 0, l);
        childOf(C, 1, r);
        e[best] = l;
        e[ne++] = r;
    }
    int k = 0, t = 0;
    for (int j = 0; j < ne; ++j) {
        ent[8 * i + j] = e[j];
        if (e[j].cnt == 0)
            ++k;
        else
            t += e[j].cnt;
    }
    nEnt[i] = ne;
    kInt[i] = k;
    nTri[i] = t;
}

// Box quantisation shared by the collapse and the refit, in FP32 with
// directed rounding so that it is cheap on the GPU and still conservative:
// the extent is rounded up, a child's offset from the node origin rounded
// down (low bound) or up (high bound), then widened by one step.
OPT_D int scaleExponent(float ext)  // smallest e with 253 * 2^e >= ext, in [-126, 127]
{
    if (!(ext > 0.0f))
        return -126;
    int e = ilogbf(ext) - 7;
    while (ldexpf(253.0f, e) < ext)
        ++e;
    while (e > -126 && ldexpf(253.0f, e - 1) >= ext)
        --e;
    return max(-126, min(127, e));
}
OPT_D void quantise(float elo, float ehi, float lo, int ex, uint32_t &ql, uint32_t &qh)
{
    const float inv = ldexpf(1.0f, -ex);
    float a = floorf(__fsub_rd(elo, lo) * inv), b = ceilf(__fsub_ru(ehi, lo) * inv);
    a = a > 0.0f ? a - 1.0f : 0.0f;
    b = fminf(b + 1.0f, 255.0f);
    ql = (uint32_t)a;
    qh = (uint32_t)fmaxf(b, 0.0f);
}

__global__ void kCollapseEmit(const int *__restrict__ items, int nItems, const Entry *__restrict__ ent,
                              const int *__restrict__ nEnt, const int *__restrict__ scanK,
                              const int *__restrict__ scanT, int levelStart, int nextStart, int triStart,
                              const float4 *__restrict__ triV2, Bvh8Node *__restrict__ out,
                              int *__restrict__ nextItems, float4 *__restrict__ triV8, int cap, int numTris)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nItems || levelStart + i >= cap || nextStart + scanK[i + 1] > cap ||
        triStart + scanT[i + 1] > numTris)
        return;  // bounds guard; a valid BVH2 never trips it (checked on the host)
    const int ne = nEnt[i];
    Entry e[8];
    float lo[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
    float hi[3] = {-__int_as_float(0x7f800000), -__int_as_float(0x7f800000), -__int_as_float(0x7f800000)};
    for (int j = 0; j < ne; ++j) {
        e[j] = ent[8 * i + j];
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], e[j].lo[k]);
            hi[k] = fmaxf(hi[k], e[j].hi[k]);
        }
    }
    // Slots: each entry goes to its centroid's octant relative to the node
    // centre, or the free slot nearest to it in Hamming distance.
    float cen[3];
    for (int k = 0; k < 3; ++k)
        cen[k] = __fmul_rn(__fadd_rn(lo[k], hi[k]), 0.5f);
    int slotOf[8];
    uint32_t used = 0;
    for (int j = 0; j < ne; ++j) {
        uint32_t code = 0;
        for (int k = 0; k < 3; ++k)
            if (__fmul_rn(__fadd_rn(e[j].lo[k], e[j].hi[k]), 0.5f) > cen[k])
                code |= 1u << k;
        int slot = -1;
        if (!((used >> code) & 1u)) {
            slot = (int)code;
        } else {
            int bestD = 99;
            for (int s = 0; s < 8; ++s) {
                if ((used >> s) & 1u)
                    continue;
                const int dd = __popc((uint32_t)s ^ code);
                if (dd < bestD) {
                    bestD = dd;
                    slot = s;
                }
            }
        }
        used |= 1u << slot;
        slotOf[j] = slot;
    }
    int ex[3];
    for (int k = 0; k < 3; ++k)
        ex[k] = scaleExponent(__fsub_ru(hi[k], lo[k]));
    uint32_t meta[8] = {0, 0, 0, 0, 0, 0, 0, 0}, qlo[3][8], qhi[3][8];
    int refAt[8];
    for (int s = 0; s < 8; ++s) {
        refAt[s] = -1;
        for (int k = 0; k < 3; ++k)
            qlo[k][s] = qhi[k][s] = 0u;
    }
    for (int j = 0; j < ne; ++j)
        refAt[slotOf[j]] = j;
    uint32_t imask = 0;
    const int childBase = nextStart + scanK[i];
    const int triBase = triStart + scanT[i];
    int rank = 0, toff = 0;
    for (int s = 0; s < 8; ++s) {
        const int j = refAt[s];
        if (j < 0)
            continue;
        for (int k = 0; k < 3; ++k)
            quantise(e[j].lo[k], e[j].hi[k], lo[k], ex[k], qlo[k][s], qhi[k][s]);
        if (e[j].cnt == 0) {
            imask |= 1u << s;
            meta[s] = 1u;
            nextItems[scanK[i] + rank] = e[j].ref;
            ++rank;
        } else {
            meta[s] = ((uint32_t)e[j].cnt << 5) | (uint32_t)toff;
            for (int c = 0; c < e[j].cnt; ++c) {
                const int src = e[j].ref + c, dst = triBase + toff + c;
                triV8[3 * dst] = triV2[3 * src];
                triV8[3 * dst + 1] = triV2[3 * src + 1];
                triV8[3 * dst + 2] = triV2[3 * src + 2];
            }
            toff += e[j].cnt;
        }
    }
    Bvh8Node N;
    const uint32_t ew = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) | ((uint32_t)(ex[2] + 127) << 16) |
                        (imask << 24);
    N.a = make_float4(lo[0], lo[1], lo[2], __uint_as_float(ew));
    N.b = make_uint4((uint32_t)childBase, (uint32_t)triBase, meta[0] | meta[1] << 8 | meta[2] << 16 | meta[3] << 24,
                     meta[4] | meta[5] << 8 | meta[6] << 16 | meta[7] << 24);
    uint4 *q[3] = {&N.qx, &N.qy, &N.qz};
    for (int k = 0; k < 3; ++k) {
        q[k]->x = qlo[k][0] | qlo[k][1] << 8 | qlo[k][2] << 16 | qlo[k][3] << 24;
        q[k]->y = qlo[k][4] | qlo[k][5] << 8 | qlo[k][6] << 16 | qlo[k][7] << 24;
        q[k]->z = qhi[k][0] | qhi[k][1] << 8 | qhi[k][2] << 16 | qhi[k][3] << 24;
        q[k]->w = qhi[k][4] | qhi[k][5] << 8 | qhi[k][6] << 16 | qhi[k][7] << 24;
    }
    out[levelStart + i] = N;
}

// Refit, step 1: the leaf-ordered triangle records take the new vertex
// positions (the record's w fields, prim id, material and flags, are kept).
__global__ void kRefitTris(int n, const float *__restrict__ pos, const int *__restrict__ idx,
                           float4 *__restrict__ triV8)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    float4 *t = triV8 + 3 * (size_t)k;
    const int prim = __float_as_int(t[0].w);
    if (prim < 0 || prim >= n)
        return;
    for (int v = 0; v < 3; ++v) {
        const int vi = __ldg(idx + 3 * prim + v);
        float4 r = t[v];
        r.x = __ldg(pos + 3 * (size_t)vi);
        r.y = __ldg(pos + 3 * (size_t)vi + 1);
        r.z = __ldg(pos + 3 * (size_t)vi + 2);
        t[v] = r;
    }
}

// Refit, step 2 (one launch per level, deepest first): eight lanes per node,
// one per child slot. A lane forms its slot's box (an internal child's refit
// box, or its leaf triangles' bounds); the node box is the union over the
// eight lanes (shuffles); each lane quantises its own slot exactly as the
// collapse does, and the bytes are packed into the node's words by shuffles.
// With unchanged vertices the nodes come out bit-identical.
__global__ void __launch_bounds__(128) kRefitLevel(int begin, int end, Bvh8Node *__restrict__ nodes,
                                                   const float4 *__restrict__ triV8, float *__restrict__ box8,
                                                   int numNodes8, int numTris)
{
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int i = begin + (t >> 3), s = t & 7;
    const bool live = i < end;
    const float inf = __int_as_float(0x7f800000);
    float elo[3] = {inf, inf, inf}, ehi[3] = {-inf, -inf, -inf};
    uint4 b = make_uint4(0u, 0u, 0u, 0u);
    uint32_t imask = 0;
    bool present = false;
    if (live) {
        b = nodes[i].b;
        imask = __float_as_uint(nodes[i].a.w) >> 24;
        const uint32_t meta = byteOf(b, 8 + s);
        present = meta != 0u;
        if (present && ((imask >> s) & 1u)) {
            const int c = (int)b.x + __popc(imask & ((1u << s) - 1u));
            if (c >= 0 && c < numNodes8)
                for (int k = 0; k < 3; ++k) {
                    elo[k] = box8[6 * (size_t)c + k];
                    ehi[k] = box8[6 * (size_t)c + 3 + k];
                }
        } else if (present) {
            const int first = (int)b.y + (int)(meta & 31u), cnt = (int)(meta >> 5);
            for (int tr = first; tr < first + cnt && tr < numTris; ++tr)
                for (int v = 0; v < 3; ++v) {
                    const float4 p = triV8[3 * (size_t)tr + v];
                    elo[0] = fminf(elo[0], p.x);
                    elo[1] = fminf(elo[1], p.y);
                    elo[2] = fminf(elo[2], p.z);
                    ehi[0] = fmaxf(ehi[0], p.x);
                    ehi[1] = fmaxf(ehi[1], p.y);
                    ehi[2] = fmaxf(ehi[2], p.z);
                }
        }
    }
    float lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = elo[k];
        hi[k] = ehi[k];
        for (int off = 1; off < 8; off <<= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], off));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], off));
        }
    }
    int ex[3];
    uint32_t ql[3] = {0u, 0u, 0u}, qh[3] = {0u, 0u, 0u};
    for (int k = 0; k < 3; ++k) {
        ex[k] = scaleExponent(__fsub_ru(hi[k], lo[k]));
        if (present)
            quantise(elo[k], ehi[k], lo[k], ex[k], ql[k], qh[k]);
    }
    // pack: word of slots 0-3 (or 4-7) from the lanes of this quad
    const int sh = 8 * (s & 3);
    uint32_t wl[3], wh[3];
    for (int k = 0; k < 3; ++k) {
        wl[k] = ql[k] << sh;
        wh[k] = qh[k] << sh;
        for (int off = 1; off < 4; off <<= 1) {
            wl[k] |= __shfl_xor_sync(0xffffffffu, wl[k], off);
            wh[k] |= __shfl_xor_sync(0xffffffffu, wh[k], off);
        }
    }
    if (!live)
        return;
    Bvh8Node *N = nodes + i;
    uint32_t *qw[3] = {&N->qx.x, &N->qy.x, &N->qz.x};
    if (s == 0 || s == 4) {
        const int half = s >> 2;  // 0: slots 0-3 (words x, z), 1: slots 4-7 (words y, w)
        for (int k = 0; k < 3; ++k) {
            qw[k][half] = wl[k];
            qw[k][2 + half] = wh[k];
        }
    }
    if (s == 0) {
        const uint32_t ew = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) |
                            ((uint32_t)(ex[2] + 127) << 16) | (imask << 24);
        N->a = make_float4(lo[0], lo[1], lo[2], __uint_as_float(ew));
        for (int k = 0; k < 3; ++k) {
            box8[6 * (size_t)i + k] = lo[k];
            box8[6 * (size_t)i + 3 + k] = hi[k];
        }
    }
}

}  // namespace

int refitBvh8(BvhBuild &b, const float *positions, const int *triIndices, int numTris, cudaStream_t st)
{
    if (numTris <= 0 || b.nodes8 == nullptr)
        return 0;
    if (!b.box8) {
        cudaError_t e = cudaMalloc(&b.box8, sizeof(float) * 6 * (size_t)(b.numNodes8 > 0 ? b.numNodes8 : 1));
        if (e != cudaSuccess)
            return (int)e;
    }
    kRefitTris<<<(numTris + 255) / 256, 256, 0, st>>>(numTris, positions, triIndices, b.triV8);
    for (int l = b.levels8 - 1; l >= 0; --l) {
        const int begin = b.levelOff8[l], end = b.levelOff8[l + 1];
        if (end > begin)
            kRefitLevel<<<(8 * (end - begin) + 127) / 128, 128, 0, st>>>(begin, end, b.nodes8, b.triV8, b.box8,
                                                                        b.numNodes8, numTris);
    }
    return (int)cudaGetLastError();
}

// Collapses a built BVH2 (`in`) into in.nodes8 / in.triV8. Returns 0 or a CUDA
// error code.
int buildBvh8(BvhBuild &in, int numTris, cudaStream_t st)
{
    if (numTris <= 0 || in.nodes == nullptr)
        return 0;
    const int cap = in.numNodes > 0 ? in.numNodes : 1;
    cudaError_t err = cudaSuccess;
    int *items = nullptr, *nextItems = nullptr, *nEnt = nullptr, *kInt = nullptr, *nTri = nullptr;
    int *scanK = nullptr, *scanT = nullptr;
    Entry *ent = nullptr;
    void *temp = nullptr;
    size_t tempBytes = 0;
    int nItems = 1, levelStart = 0, triStart = 0, levels = 0;
    const int zero = 0;
#define CK8(x)                                                                                                         \
    do {                                                                                                               \
        if ((err = (x)) != cudaSuccess)                                                                                \
            goto done;                                                                                                 \
    } while (0)
    CK8(cudaMalloc(&in.nodes8, sizeof(Bvh8Node) * cap));
    CK8(cudaMalloc(&in.triV8, sizeof(float4) * 3 * (size_t)numTris));
    CK8(cudaMalloc(&items, sizeof(int) * cap));
    CK8(cudaMalloc(&nextItems, sizeof(int) * cap));
    CK8(cudaMalloc(&nEnt, sizeof(int) * cap));
    CK8(cudaMalloc(&kInt, sizeof(int) * (cap + 1)));
    CK8(cudaMalloc(&nTri, sizeof(int) * (cap + 1)));
    CK8(cudaMalloc(&scanK, sizeof(int) * (cap + 1)));
    CK8(cudaMalloc(&scanT, sizeof(int) * (cap + 1)));
    CK8(cudaMalloc(&ent, sizeof(Entry) * 8 * (size_t)cap));
    CK8(cub::DeviceScan::ExclusiveSum(nullptr, tempBytes, kInt, scanK, cap + 1, st));
    CK8(cudaMalloc(&temp, tempBytes));
    CK8(cudaMemcpyAsync(items, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
    while (nItems > 0 && levels < 256) {
        in.levelOff8[levels] = levelStart;
        const int G = (nItems + 127) / 128;
        kCollapseOpen<<<G, 128, 0, st>>>(in.nodes, items, nItems, ent, nEnt, kInt, nTri);
        // one extra zero entry so the exclusive scan's last element is the total
        CK8(cudaMemsetAsync(kInt + nItems, 0, sizeof(int), st));
        CK8(cudaMemsetAsync(nTri + nItems, 0, sizeof(int), st));
        size_t tb = tempBytes;
        CK8(cub::DeviceScan::ExclusiveSum(temp, tb, kInt, scanK, nItems + 1, st));
        CK8(cub::DeviceScan::ExclusiveSum(temp, tb, nTri, scanT, nItems + 1, st));
        int totals[2];
        CK8(cudaMemcpyAsync(&totals[0], scanK + nItems, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK8(cudaMemcpyAsync(&totals[1], scanT + nItems, sizeof(int), cudaMemcpyDeviceToHost, st));
        const int nextStart = levelStart + nItems;
        kCollapseEmit<<<G, 128, 0, st>>>(items, nItems, ent, nEnt, scanK, scanT, levelStart, nextStart, triStart,
                                         in.triV, in.nodes8, nextItems, in.triV8, cap, numTris);
        CK8(cudaGetLastError());
        CK8(cudaStreamSynchronize(st));
        if (nextStart + totals[0] > cap) {  // cannot happen for a valid BVH2
            err = cudaErrorInvalidValue;
            goto done;
        }
        levelStart = nextStart;
        triStart += totals[1];
        nItems = totals[0];
        int *t = items;
        items = nextItems;
        nextItems = t;
        ++levels;
    }
    in.numNodes8 = levelStart;
    in.levels8 = levels;
    in.levelOff8[levels] = levelStart;
    if (triStart != numTris)
        err = cudaErrorInvalidValue;
done:
#undef CK8
    cudaFree(items);
    cudaFree(nextItems);
    cudaFree(nEnt);
    cudaFree(kInt);
    cudaFree(nTri);
    cudaFree(scanK);
    cudaFree(scanT);
    cudaFree(ent);
    cudaFree(temp);
    if (err != cudaSuccess) {
        cudaFree(in.nodes8);
        cudaFree(in.triV8);
        in.nodes8 = nullptr;
        in.triV8 = nullptr;
        return (int)err;
    }
    return 0;
}
