// GPU LBVH build: the replacement for optixAccelBuild (reference:
// src/renderer.cpp:441-513). Steps, all on the GPU:
//   1. per-triangle bounds and the centroid bounds of the scene
//   2. 30-bit Morton code of each centroid (10 bits per axis)
//   3. CUB radix sort of (code, primitive) pairs (stable: ties keep index order)
//   4. Karras' parallel radix-tree construction ("Maximizing Parallelism in the
//      Construction of BVHs, Octrees, and k-d Trees", HPG 2012)
//   5. bottom-up bounding boxes and subtree sizes (atomic arrival counters)
//   6. emission of BVH2 nodes, collapsing every subtree of <= leafSize
//      triangles into one leaf (a Karras subtree covers a contiguous range of
//      sorted primitives)
//   7. leaf-ordered triangle records (3 x float4) for traversal and shading
// The arithmetic that decides codes and order uses explicitly rounded
// operations so the host oracle reproduces codes, order and topology exactly.
// Alternatively (an option for the 8-wide BVH) steps 4-6 are replaced by
// PLOC clustering on the sorted triangles (below), which places large
// triangles and sparse regions by surface area instead of by Morton bits.
#include <cub/cub.cuh>
#include "engine.h"

namespace {

#define LEAF_BIT 0x80000000u

OPT_D unsigned floatToOrdered(float f)
{
    unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
OPT_HD float orderedToFloat(unsigned b)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float((b & 0x80000000u) ? (b & 0x7fffffffu) : ~b);
#else
    unsigned r = (b & 0x80000000u) ? (b & 0x7fffffffu) : ~b;
    float f;
    memcpy(&f, &r, 4);
    return f;
#endif
}

OPT_D float3 loadPos(const float *pos, int i) { return mk3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]); }

__global__ void kPrimBounds(const float *pos, const int *idx, int n, float4 *lo, float4 *hi, unsigned *cb)
{
    float3 cmin = mk3s(__int_as_float(0x7f800000)), cmax = mk3s(-__int_as_float(0x7f800000));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float3 a = loadPos(pos, idx[3 * i]), b = loadPos(pos, idx[3 * i + 1]), c = loadPos(pos, idx[3 * i + 2]);
        const float3 l = mk3(fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y), fminf(fminf(a.z, b.z), c.z));
        const float3 h = mk3(fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y), fmaxf(fmaxf(a.z, b.z), c.z));
        lo[i] = make_float4(l.x, l.y, l.z, 0.0f);
        hi[i] = make_float4(h.x, h.y, h.z, 0.0f);
        const float3 cen = mk3(__fmul_rn(__fadd_rn(l.x, h.x), 0.5f), __fmul_rn(__fadd_rn(l.y, h.y), 0.5f),
                               __fmul_rn(__fadd_rn(l.z, h.z), 0.5f));
        cmin = mk3(fminf(cmin.x, cen.x), fminf(cmin.y, cen.y), fminf(cmin.z, cen.z));
        cmax = mk3(fmaxf(cmax.x, cen.x), fmaxf(cmax.y, cen.y), fmaxf(cmax.z, cen.z));
    }
    for (int off = 16; off > 0; off >>= 1) {
        cmin.x = fminf(cmin.x, __shfl_down_sync(0xffffffffu, cmin.x, off));
        cmin.y = fminf(cmin.y, __shfl_down_sync(0xffffffffu, cmin.y, off));
        cmin.z = fminf(cmin.z, __shfl_down_sync(0xffffffffu, cmin.z, off));
        cmax.x = fmaxf(cmax.x, __shfl_down_sync(0xffffffffu, cmax.x, off));
        cmax.y = fmaxf(cmax.y, __shfl_down_sync(0xffffffffu, cmax.y, off));
        cmax.z = fmaxf(cmax.z, __shfl_down_sync(0xffffffffu, cmax.z, off));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(cb + 0, floatToOrdered(cmin.x));
        atomicMin(cb + 1, floatToOrdered(cmin.y));
        atomicMin(cb + 2, floatToOrdered(cmin.z));
        atomicMax(cb + 3, floatToOrdered(cmax.x));
        atomicMax(cb + 4, floatToOrdered(cmax.y));
        atomicMax(cb + 5, floatToOrdered(cmax.z));
    }
}

OPT_D unsigned expandBits(unsigned v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

OPT_D unsigned quantize(float c, float lo, float hi)
{
    const float ext = __fsub_rn(hi, lo);
    const float nrm = ext > 0.0f ? __fdiv_rn(__fsub_rn(c, lo), ext) : 0.0f;
    const float s = fminf(fmaxf(__fmul_rn(nrm, 1024.0f), 0.0f), 1023.0f);
    return (unsigned)s;
}

__global__ void kMorton(const float4 *lo, const float4 *hi, int n, const unsigned *cb, unsigned *codes, int *ids)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float3 cmin = mk3(orderedToFloat(cb[0]), orderedToFloat(cb[1]), orderedToFloat(cb[2]));
    const float3 cmax = mk3(orderedToFloat(cb[3]), orderedToFloat(cb[4]), orderedToFloat(cb[5]));
    const float4 l = lo[i], h = hi[i];
    const float cx = __fmul_rn(__fadd_rn(l.x, h.x), 0.5f), cy = __fmul_rn(__fadd_rn(l.y, h.y), 0.5f),
                cz = __fmul_rn(__fadd_rn(l.z, h.z), 0.5f);
    codes[i] = (expandBits(quantize(cx, cmin.x, cmax.x)) << 2) | (expandBits(quantize(cy, cmin.y, cmax.y)) << 1) |
               expandBits(quantize(cz, cmin.z, cmax.z));
    ids[i] = i;
}

OPT_D int deltaK(const unsigned *codes, int n, int i, int j)
{
    if (j < 0 || j >= n)
        return -1;
    const unsigned a = codes[i], b = codes[j];
    if (a == b)
        return 32 + __clz((unsigned)(i ^ j));
    return __clz(a ^ b);
}

// Internal node i: children (internal index, or sorted leaf index | LEAF_BIT),
// its range of sorted leaves, and parent links.
__global__ void kKarras(const unsigned *codes, int n, int2 *child, int2 *range, int *parentInternal, int *parentLeaf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1)
        return;
    const int d = (deltaK(codes, n, i, i + 1) - deltaK(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = deltaK(codes, n, i, i - d);
    int lmax = 2;
    while (deltaK(codes, n, i, i + lmax * d) > dmin)
        lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (deltaK(codes, n, i, i + (l + t) * d) > dmin)
            l += t;
    const int j = i + l * d;
    const int dnode = deltaK(codes, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (deltaK(codes, n, i, i + (s + t) * d) > dnode)
            s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int first = min(i, j), last = max(i, j);
    int2 c;
    if (first == gamma) {
        c.x = (int)((unsigned)gamma | LEAF_BIT);
        parentLeaf[gamma] = i;
    } else {
        c.x = gamma;
        parentInternal[gamma] = i;
    }
    if (last == gamma + 1) {
        c.y = (int)((unsigned)(gamma + 1) | LEAF_BIT);
        parentLeaf[gamma + 1] = i;
    } else {
        c.y = gamma + 1;
        parentInternal[gamma + 1] = i;
    }
    child[i] = c;
    range[i] = make_int2(first, last);
    if (i == 0)
        parentInternal[0] = -1;
}

OPT_D void childBox(int c, const int *ids, const float4 *plo, const float4 *phi, const float4 *nlo, const float4 *nhi,
                    const int *ncount, float4 &lo, float4 &hi, int &cnt)
{
    if ((unsigned)c & LEAF_BIT) {
        const int leaf = (int)((unsigned)c & ~LEAF_BIT);
        const int p = ids[leaf];
        lo = plo[p];
        hi = phi[p];
        cnt = 1;
    } else {
        lo = __ldcg(nlo + c);
        hi = __ldcg(nhi + c);
        cnt = __ldcg(ncount + c);
    }
}

__global__ void kBottomUp(int n, const int *ids, const float4 *plo, const float4 *phi, const int2 *child,
                          const int *parentInternal, const int *parentLeaf, float4 *nlo, float4 *nhi, int *ncount,
                          unsigned *flags)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    int node = parentLeaf[i];
    for (int level = 0; node >= 0 && level < 4096; ++level) {  // tree depth <= 64 + log2(n)
        __threadfence();
        if (atomicAdd(flags + node, 1u) == 0u)
            return;
        __threadfence();
        const int2 c = child[node];
        float4 l0, h0, l1, h1;
        int c0, c1;
        childBox(c.x, ids, plo, phi, nlo, nhi, ncount, l0, h0, c0);
        childBox(c.y, ids, plo, phi, nlo, nhi, ncount, l1, h1, c1);
        __stcg(nlo + node, make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.0f));
        __stcg(nhi + node, make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.0f));
        __stcg(ncount + node, c0 + c1);
        node = parentInternal[node];
    }
}

__global__ void kEmit(int n, int leafSize, const int *ids, const float4 *plo, const float4 *phi, const int2 *child,
                      const int2 *range, const float4 *nlo, const float4 *nhi, const int *ncount, BvhNode *nodes,
                      unsigned *stats)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1)
        return;
    if (ncount[i] <= leafSize) {
        if (i == 0) {  // the whole scene fits in one leaf
            BvhNode N;
            N.a = make_float4(nlo[0].x, nhi[0].x, nlo[0].y, nhi[0].y);
            N.b = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            N.c = make_float4(nlo[0].z, nhi[0].z, 0.0f, 0.0f);
            N.d = make_int4(0, -1, n, 0);
            nodes[0] = N;
            atomicAdd(stats + 0, 1u);
            atomicAdd(stats + 1, 1u);
        }
        return;
    }
    const int2 c = child[i];
    float4 lo[2], hi[2];
    int ref[2], cnt[2];
    unsigned leaves = 0;
    for (int k = 0; k < 2; ++k) {
        const int ch = k == 0 ? c.x : c.y;
        if ((unsigned)ch & LEAF_BIT) {
            const int leaf = (int)((unsigned)ch & ~LEAF_BIT);
            lo[k] = plo[ids[leaf]];
            hi[k] = phi[ids[leaf]];
            ref[k] = leaf;
            cnt[k] = 1;
            ++leaves;
        } else {
            lo[k] = nlo[ch];
            hi[k] = nhi[ch];
            if (ncount[ch] <= leafSize) {
                ref[k] = range[ch].x;
                cnt[k] = ncount[ch];
                ++leaves;
            } else {
                ref[k] = ch;
                cnt[k] = 0;
            }
        }
    }
    BvhNode N;
    N.a = make_float4(lo[0].x, hi[0].x, lo[0].y, hi[0].y);
    N.b = make_float4(lo[1].x, hi[1].x, lo[1].y, hi[1].y);
    N.c = make_float4(lo[0].z, hi[0].z, lo[1].z, hi[1].z);
    N.d = make_int4(ref[0], ref[1], cnt[0], cnt[1]);
    nodes[i] = N;
    atomicAdd(stats + 0, 1u);
    if (leaves)
        atomicAdd(stats + 1, leaves);
}

__global__ void kSingle(const float4 *plo, const float4 *phi, BvhNode *nodes, unsigned *stats)
{
    BvhNode N;
    N.a = make_float4(plo[0].x, phi[0].x, plo[0].y, phi[0].y);
    N.b = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    N.c = make_float4(plo[0].z, phi[0].z, 0.0f, 0.0f);
    N.d = make_int4(0, -1, 1, 0);
    nodes[0] = N;
    stats[0] = 1u;
    stats[1] = 1u;
}

__global__ void kTriV(int n, const int *ids, const float *pos, const int *idx, const int *mat, const uint32_t *flags,
                      float4 *triV)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int p = ids[i];
    const float3 a = loadPos(pos, idx[3 * p]), b = loadPos(pos, idx[3 * p + 1]), c = loadPos(pos, idx[3 * p + 2]);
    triV[3 * i] = make_float4(a.x, a.y, a.z, __int_as_float(p));
    triV[3 * i + 1] = make_float4(b.x, b.y, b.z, __int_as_float(mat[p]));
    triV[3 * i + 2] = make_float4(c.x, c.y, c.z, __uint_as_float(flags ? flags[p] : 0u));
}

// ------------------------------------------------------------------ PLOC
// Parallel locally-ordered clustering (Meister and Bittner, "Parallel
// Locally-Ordered Clustering for Bounding Volume Hierarchy Construction",
// IEEE TVCG 2018): the clusters (at first one per triangle, in Morton order)
// each find the neighbour within PLOC_RADIUS positions whose merged box has
// the smallest surface area; mutual neighbours merge into a new node, which
// keeps the lower position; the survivors are compacted in order, and the
// steps repeat until one cluster is left. Nodes are numbered downwards from
// n - 2 in merge order, so the last merge (the root) is node 0. Ties are
// broken by the pair's positions, so the smallest pair of every step is
// mutual (progress) and the build is deterministic.
#define PLOC_RADIUS 16
#define PLOC_BLOCK 256

OPT_D float mergedArea(float4 al, float4 ah, float4 bl, float4 bh)
{
    const float dx = fmaxf(ah.x, bh.x) - fminf(al.x, bl.x), dy = fmaxf(ah.y, bh.y) - fminf(al.y, bl.y),
                dz = fmaxf(ah.z, bh.z) - fminf(al.z, bl.z);
    return dx * dy + dy * dz + dz * dx;
}

// Cluster i = (lo.xyz, ref) / (hi.xyz, -); ref: node index, or sorted
// triangle position | LEAF_BIT.
__global__ void kPlocInit(int n, const int *ids, const float4 *plo, const float4 *phi, float4 *clo, float4 *chi)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float4 l = plo[ids[i]], h = phi[ids[i]];
    clo[i] = make_float4(l.x, l.y, l.z, __uint_as_float((unsigned)i | LEAF_BIT));
    chi[i] = make_float4(h.x, h.y, h.z, 0.0f);
}

__global__ void __launch_bounds__(PLOC_BLOCK) kPlocNearest(int m, const float4 *clo, const float4 *chi, int *nn)
{
    __shared__ float4 sl[PLOC_BLOCK + 2 * PLOC_RADIUS], sh[PLOC_BLOCK + 2 * PLOC_RADIUS];
    const int b0 = blockIdx.x * PLOC_BLOCK;
    for (int k = threadIdx.x; k < PLOC_BLOCK + 2 * PLOC_RADIUS; k += PLOC_BLOCK) {
        const int j = b0 - PLOC_RADIUS + k;
        if (j >= 0 && j < m) {
            sl[k] = clo[j];
            sh[k] = chi[j];
        }
    }
    __syncthreads();
    const int i = b0 + threadIdx.x;
    if (i >= m)
        return;
    const int si = threadIdx.x + PLOC_RADIUS;
    const float4 al = sl[si], ah = sh[si];
    float best = __int_as_float(0x7f800000);
    int bj = -1;
    for (int d = -PLOC_RADIUS; d <= PLOC_RADIUS; ++d) {
        const int j = i + d;
        if (d == 0 || j < 0 || j >= m)
            continue;
        const float a = mergedArea(al, ah, sl[si + d], sh[si + d]);
        // ties: the pair with the lower (min, max) positions; for a fixed i
        // that is the lower j
        if (a < best || (a == best && j < bj)) {
            best = a;
            bj = j;
        }
    }
    nn[i] = bj;
}

// keep[i] = cluster i survives this step (not the upper half of a merge);
// merge[i] = cluster i merges with its upper neighbour.
__global__ void kPlocFlags(int m, const int *nn, int *keep, int *merge)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    const int j = nn[i];
    const bool mutual = j >= 0 && nn[j] == i;
    keep[i] = (mutual && j < i) ? 0 : 1;
    merge[i] = (mutual && i < j) ? 1 : 0;
}

__global__ void kPlocEmit(int m, const float4 *clo, const float4 *chi, const int *nn, const int *keep,
                          const int *keepPos, const int *merge, const int *mergePos, int nodeBase, BvhNode *nodes,
                          float4 *olo, float4 *ohi)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || !keep[i])
        return;
    const float4 al = clo[i], ah = chi[i];
    const int pos = keepPos[i];
    if (!merge[i]) {
        olo[pos] = al;
        ohi[pos] = ah;
        return;
    }
    const int j = nn[i];
    const float4 bl = clo[j], bh = chi[j];
    const int node = nodeBase - 1 - mergePos[i];
    int ref[2], cnt[2];
    const unsigned r2[2] = {__float_as_uint(al.w), __float_as_uint(bl.w)};
    for (int k = 0; k < 2; ++k) {
        ref[k] = (int)(r2[k] & ~LEAF_BIT);
        cnt[k] = (r2[k] & LEAF_BIT) ? 1 : 0;
    }
    BvhNode N;
    N.a = make_float4(al.x, ah.x, al.y, ah.y);
    N.b = make_float4(bl.x, bh.x, bl.y, bh.y);
    N.c = make_float4(al.z, ah.z, bl.z, bh.z);
    N.d = make_int4(ref[0], ref[1], cnt[0], cnt[1]);
    nodes[node] = N;
    olo[pos] = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), __int_as_float(node));
    ohi[pos] = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f);
}

template <class T> cudaError_t dalloc(T *&p, size_t count)
{
    return cudaMalloc((void **)&p, sizeof(T) * (count ? count : 1));
}

}  // namespace

#define CK(x)                                                                                                          \
    do {                                                                                                               \
        cudaError_t e_ = (x);                                                                                          \
        if (e_ != cudaSuccess) {                                                                                       \
            err = e_;                                                                                                  \
            goto done;                                                                                                 \
        }                                                                                                              \
    } while (0)

// The PLOC steps on sorted triangles: the BVH2 in out.nodes (n - 1 nodes,
// leaves of one triangle). Synchronises `st` once per step for the counts.
#define PLOC_MAX_STEPS 1024
#define PLOC_GAVE_UP (-1)  // more steps than PLOC_MAX_STEPS: the caller builds the LBVH instead

static int buildPloc(int n, const int *ids, const float4 *plo, const float4 *phi, BvhBuild &out, cudaStream_t st)
{
    cudaError_t err = cudaSuccess;
    float4 *clo[2] = {nullptr, nullptr}, *chi[2] = {nullptr, nullptr};
    int *nn = nullptr, *keep = nullptr, *merge = nullptr, *keepPos = nullptr, *mergePos = nullptr;
    void *temp = nullptr;
    size_t tempBytes = 0;
    int m = n, nodeBase = n - 1, cur = 0, steps = 0;
    const int B = 256;
    CK(dalloc(clo[0], n));
    CK(dalloc(clo[1], n));
    CK(dalloc(chi[0], n));
    CK(dalloc(chi[1], n));
    CK(dalloc(nn, n));
    CK(dalloc(keep, n));
    CK(dalloc(merge, n));
    CK(dalloc(keepPos, n));
    CK(dalloc(mergePos, n));
    CK(cub::DeviceScan::ExclusiveSum(nullptr, tempBytes, keep, keepPos, n, st));
    CK(cudaMalloc(&temp, tempBytes));
    kPlocInit<<<(n + B - 1) / B, B, 0, st>>>(n, ids, plo, phi, clo[0], chi[0]);
    CK(cudaGetLastError());
    while (m > 1) {
        if (++steps > PLOC_MAX_STEPS) {  // (a few dozen steps for ordinary scenes)
            cudaFree(temp);
            temp = nullptr;
            err = cudaSuccess;
            for (int k = 0; k < 2; ++k) {
                cudaFree(clo[k]);
                cudaFree(chi[k]);
            }
            cudaFree(nn);
            cudaFree(keep);
            cudaFree(merge);
            cudaFree(keepPos);
            cudaFree(mergePos);
            return PLOC_GAVE_UP;
        }
        const int G = (m + B - 1) / B;
        kPlocNearest<<<(m + PLOC_BLOCK - 1) / PLOC_BLOCK, PLOC_BLOCK, 0, st>>>(m, clo[cur], chi[cur], nn);
        kPlocFlags<<<G, B, 0, st>>>(m, nn, keep, merge);
        CK(cudaGetLastError());
        CK(cub::DeviceScan::ExclusiveSum(temp, tempBytes, keep, keepPos, m, st));
        CK(cub::DeviceScan::ExclusiveSum(temp, tempBytes, merge, mergePos, m, st));
        kPlocEmit<<<G, B, 0, st>>>(m, clo[cur], chi[cur], nn, keep, keepPos, merge, mergePos, nodeBase, out.nodes,
                                    clo[cur ^ 1], chi[cur ^ 1]);
        CK(cudaGetLastError());
        int last[4];
        CK(cudaMemcpyAsync(last, keepPos + m - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(last + 1, keep + m - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(last + 2, mergePos + m - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(last + 3, merge + m - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        const int merges = last[2] + last[3];
        if (merges <= 0) {  // cannot happen (the smallest pair is mutual); a broken step stops the build
            err = cudaErrorUnknown;
            goto done;
        }
        m = last[0] + last[1];
        nodeBase -= merges;
        cur ^= 1;
    }
done:
    for (int k = 0; k < 2; ++k) {
        cudaFree(clo[k]);
        cudaFree(chi[k]);
    }
    cudaFree(nn);
    cudaFree(keep);
    cudaFree(merge);
    cudaFree(keepPos);
    cudaFree(mergePos);
    cudaFree(temp);
    return (int)err;
}

int buildBvh(const float *positions, const int *triIndices, const int *matIndices, const uint32_t *triFlags,
             int n, int leafSize, BvhBuild &out, cudaStream_t st, bool ploc)
{
    out = BvhBuild{};
    if (n <= 0)
        return 0;
    cudaError_t err = cudaSuccess;
    float4 *plo = nullptr, *phi = nullptr, *nlo = nullptr, *nhi = nullptr;
    unsigned *cb = nullptr, *codes = nullptr, *flags = nullptr, *stats = nullptr;
    int *idsIn = nullptr, *ncount = nullptr, *parentI = nullptr, *parentL = nullptr;
    int2 *child = nullptr, *range = nullptr;
    void *temp = nullptr;
    size_t tempBytes = 0;
    unsigned hstats[2] = {0, 0};
    const unsigned cbInit[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
    const int nInt = n > 1 ? n - 1 : 1;
    const int B = 256, G = (n + B - 1) / B;
    int pe = 0;

    CK(dalloc(plo, n));
    CK(dalloc(phi, n));
    CK(dalloc(cb, 6));
    CK(dalloc(codes, n));
    CK(dalloc(idsIn, n));
    CK(dalloc(out.mortonSorted, n));
    CK(dalloc(out.primOrder, n));
    CK(dalloc(out.nodes, nInt));
    CK(dalloc(out.triV, 3 * (size_t)n));
    CK(dalloc(stats, 2));
    CK(cudaMemcpyAsync(cb, cbInit, sizeof(cbInit), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(stats, 0, 2 * sizeof(unsigned), st));
    CK(cudaMemsetAsync(out.nodes, 0, sizeof(BvhNode) * nInt, st));

    kPrimBounds<<<min(G, 4096), B, 0, st>>>(positions, triIndices, n, plo, phi, cb);
    kMorton<<<G, B, 0, st>>>(plo, phi, n, cb, codes, idsIn);
    CK(cudaGetLastError());
    CK(cub::DeviceRadixSort::SortPairs(nullptr, tempBytes, codes, out.mortonSorted, idsIn, out.primOrder, n, 0, 30, st));
    CK(cudaMalloc(&temp, tempBytes));
    CK(cub::DeviceRadixSort::SortPairs(temp, tempBytes, codes, out.mortonSorted, idsIn, out.primOrder, n, 0, 30, st));

    if (n == 1) {
        kSingle<<<1, 1, 0, st>>>(plo, phi, out.nodes, stats);
    } else if (ploc && (pe = buildPloc(n, out.primOrder, plo, phi, out, st)) != PLOC_GAVE_UP) {
        if (pe) {
            err = (cudaError_t)pe;
            goto done;
        }
    } else {
        ploc = false;
        CK(cudaMemsetAsync(out.nodes, 0, sizeof(BvhNode) * nInt, st));
        CK(dalloc(child, n - 1));
        CK(dalloc(range, n - 1));
        CK(dalloc(parentI, n - 1));
        CK(dalloc(parentL, n));
        CK(dalloc(nlo, n - 1));
        CK(dalloc(nhi, n - 1));
        CK(dalloc(ncount, n - 1));
        CK(dalloc(flags, n - 1));
        CK(cudaMemsetAsync(flags, 0, sizeof(unsigned) * (n - 1), st));
        kKarras<<<(n - 1 + B - 1) / B, B, 0, st>>>(out.mortonSorted, n, child, range, parentI, parentL);
        kBottomUp<<<G, B, 0, st>>>(n, out.primOrder, plo, phi, child, parentI, parentL, nlo, nhi, ncount, flags);
        kEmit<<<(n - 1 + B - 1) / B, B, 0, st>>>(n, leafSize, out.primOrder, plo, phi, child, range, nlo, nhi, ncount,
                                                 out.nodes, stats);
    }
    kTriV<<<G, B, 0, st>>>(n, out.primOrder, positions, triIndices, matIndices, triFlags, out.triV);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(hstats, stats, sizeof(hstats), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    out.numNodes = nInt;
    out.usedNodes = ploc && n > 1 ? n - 1 : (int)hstats[0];  // PLOC: every slot, leaves of one triangle
    out.numLeaves = ploc && n > 1 ? n : (int)hstats[1];

done:
    cudaFree(plo);
    cudaFree(phi);
    cudaFree(cb);
    cudaFree(codes);
    cudaFree(idsIn);
    cudaFree(stats);
    cudaFree(child);
    cudaFree(range);
    cudaFree(parentI);
    cudaFree(parentL);
    cudaFree(nlo);
    cudaFree(nhi);
    cudaFree(ncount);
    cudaFree(flags);
    cudaFree(temp);
    if (err != cudaSuccess) {
        freeBvh(out);
        return (int)err;
    }
    return 0;
}

void freeBvh(BvhBuild &b)
{
    cudaFree(b.nodes);
    cudaFree(b.triV);
    cudaFree(b.mortonSorted);
    cudaFree(b.primOrder);
    cudaFree(b.nodes8);
    cudaFree(b.triV8);
    cudaFree(b.box8);
    b = BvhBuild{};
}
