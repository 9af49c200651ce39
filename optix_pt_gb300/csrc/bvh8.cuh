// Compressed 8-wide BVH (after Ylitie, Karras, Laine, "Efficient Incoherent
// Ray Traversal on GPUs Through Compressed Wide BVHs", HPG 2017), built by
// collapsing the LBVH on the GPU, and its traversal.
//
// Node, 80 B (5 x 16 B):
//   a  : p.xyz (box origin, float) | w = ex | ey << 8 | ez << 16 | imask << 24
//        (e = biased exponents of the per-axis scales 2^(e-127); imask bit s =
//        slot s holds an internal child)
//   b  : childBase, triBase, meta[0..3], meta[4..7]
//        meta 0 = empty slot; 1 = internal child; leaf = count << 5 | offset
//        (count 1..7 triangles at triBase + offset)
//   qx : qlo.x[0..7], qhi.x[0..7] (bytes); qy, qz likewise
// Internal children of a node are contiguous from childBase in slot order;
// child slot s is node childBase + popc(imask & ((1 << s) - 1)). A child sits
// in the slot of its centroid's octant relative to the parent's box centre,
// so a ray with direction-sign octant r visits slots in order of s ^ r,
// approximately near to far.
#pragma once
#include "trace.cuh"

struct Bvh8Node {
    float4 a;
    uint4 b;
    uint4 qx, qy, qz;
};

#ifndef TRAV8_REFILL
#define TRAV8_REFILL 8  // idle lanes that trigger a refill of a persistent warp
#endif

OPT_D uint32_t byteOf(uint4 v, int k)  // k in 0..15
{
    const uint32_t w = k < 4 ? v.x : (k < 8 ? v.y : (k < 12 ? v.z : v.w));
    return (w >> ((k & 3) * 8)) & 0xFFu;
}

// Byte k (0..3) of w as a float, exactly: 0x4B0000qq is 2^23 + q.
OPT_D float byteToFloat(uint32_t w, int k)
{
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | (uint32_t)k)) - 8388608.0f;
}

// Three-input minimum and maximum (PTX `min.f32` / `max.f32` with three
// sources, sm_100 and later). NaN operands are ignored, as by fminf / fmaxf,
// so the result equals the two-input chain bit for bit.
OPT_D float min3f(float a, float b, float c)
{
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
OPT_D float max3f(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Bit s of m moved to bit s ^ oct (8-bit masks): adjacent bits, pairs and
// nibbles swap for oct bits 0, 1 and 2.
OPT_D uint32_t octantOrder(uint32_t m, uint32_t oct)
{
    if (oct & 1u)
        m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (oct & 2u)
        m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (oct & 4u)
        m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
    return m;
}

// Traversal state of one ray: registers, plus the node-group stack in local
// memory. `step` visits one node (and the triangles of the leaf children the
// ray reaches) and reports whether the ray is finished.
struct Trav8 {
    RayPre pre;
    float3 o, inv;
    float tmin, tcur;
    uint32_t oct;
    int node, sp, bestPrim, budget;
    // The group the next node comes from (child base, hits << 8 | imask)
    // stays in registers; a group goes to the stack only when a newer one
    // replaces it with hits left, and comes back when the newer runs out.
    uint2 grp;
    uint2 stack[BVH8_STACK];

    OPT_D void init(float3 ro, float3 d, float rtmin, float rtmax, HitRec &hit, int nodeBudget)
    {
        hit.leaf = -1;
        pre = rayPrepare(ro, d);
        o = ro;
        inv = mk3(safeInv(d.x), safeInv(d.y), safeInv(d.z));
        oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
        tmin = rtmin;
        tcur = rtmax;
        node = 0;
        sp = 0;
        bestPrim = INT_MAX;
        budget = nodeBudget;
        grp = make_uint2(0u, 0u);
    }

    template <bool ANY, class AlphaFn, class Counter>
    OPT_D bool step(const Bvh8Node *__restrict__ nodes, const float4 *__restrict__ triV, HitRec &hit, AlphaFn &alpha,
                    Counter &ctr)
    {
        if (--budget < 0) {
            hit.leaf = HIT_CUT_SHORT;  // a miss that the kernel counts as a fault
            return true;
        }
        ctr.node();
        const Bvh8Node *N = nodes + node;
        const float4 a = __ldg(&N->a);
        const uint4 b = __ldg(&N->b), qx = __ldg(&N->qx), qy = __ldg(&N->qy), qz = __ldg(&N->qz);
        const uint32_t ew = __float_as_uint(a.w);
        const float sx = __uint_as_float((ew & 0xFFu) << 23), sy = __uint_as_float(((ew >> 8) & 0xFFu) << 23),
                    sz = __uint_as_float(((ew >> 16) & 0xFFu) << 23);
        const uint32_t imask = ew >> 24;
        // t = (p + q * s - o) * inv = q * (s * inv) + (p - o) * inv. The ray's
        // direction signs pick the near plane of each axis (lo for a positive
        // direction) once per node.
        const float axs = sx * inv.x, ays = sy * inv.y, azs = sz * inv.z;
        const float bx = (a.x - o.x) * inv.x, by = (a.y - o.y) * inv.y, bz = (a.z - o.z) * inv.z;
        const bool px = inv.x >= 0.0f, py = inv.y >= 0.0f, pz = inv.z >= 0.0f;
        const uint32_t nx0 = px ? qx.x : qx.z, nx1 = px ? qx.y : qx.w, fx0 = px ? qx.z : qx.x, fx1 = px ? qx.w : qx.y;
        const uint32_t ny0 = py ? qy.x : qy.z, ny1 = py ? qy.y : qy.w, fy0 = py ? qy.z : qy.x, fy1 = py ? qy.w : qy.y;
        const uint32_t nz0 = pz ? qz.x : qz.z, nz1 = pz ? qz.y : qz.w, fz0 = pz ? qz.z : qz.x, fz1 = pz ? qz.w : qz.y;
        uint32_t hm = 0;
#pragma unroll
        // Empty slots are not skipped: their boxes are the single point at the
        // node's origin (all-zero quantised bounds), which a ray reaches only
        // by grazing that point, and then the slot counts as a leaf of zero
        // triangles. Testing all eight saves the per-slot branch.
        for (int s = 0; s < 8; ++s) {
            const int k = s & 3;
            const float xn = fmaf(byteToFloat(s < 4 ? nx0 : nx1, k), axs, bx);
            const float xf = fmaf(byteToFloat(s < 4 ? fx0 : fx1, k), axs, bx);
            const float yn = fmaf(byteToFloat(s < 4 ? ny0 : ny1, k), ays, by);
            const float yf = fmaf(byteToFloat(s < 4 ? fy0 : fy1, k), ays, by);
            const float zn = fmaf(byteToFloat(s < 4 ? nz0 : nz1, k), azs, bz);
            const float zf = fmaf(byteToFloat(s < 4 ? fz0 : fz1, k), azs, bz);
            // far plane: min(tf * w, tcur * w) == min(tf, tcur) * w exactly
            // (scaling by w > 0 and rounding are both monotone)
            const float tn = max3f(xn, yn, fmaxf(zn, tmin));
            const float tf = min3f(xf, yf, fminf(zf, tcur)) * BOX_WIDEN;
            hm |= (tn <= tf ? 1u : 0u) << s;
        }
        uint32_t lhits = hm & ~imask;
        const uint32_t ihits = octantOrder(hm & imask, oct);
        // Leaf children: their triangles, now.
        while (lhits) {
            const int s = __ffs(lhits) - 1;
            lhits &= lhits - 1u;
            const uint32_t meta = byteOf(b, 8 + s);
            const int first = (int)b.y + (int)(meta & 31u), cnt = (int)(meta >> 5);
            for (int k = first; k < first + cnt; ++k) {
                ctr.tri();
                const float4 t0 = __ldg(triV + 3 * k), t1 = __ldg(triV + 3 * k + 1), t2 = __ldg(triV + 3 * k + 2);
                float t, u, v;
                if (!intersectTri(pre, f3of4(t0), f3of4(t1), f3of4(t2), tmin, tcur, t, u, v))
                    continue;
                const int prim = __float_as_int(t0.w);
                if ((__float_as_uint(t2.w) & TRI_FLAG_ALPHA) && !alpha(k, prim, u, v))
                    continue;
                if (ANY) {
                    hit.t = t;
                    hit.u = u;
                    hit.v = v;
                    hit.leaf = k;
                    return true;  // occluded: finished
                }
                if (t < tcur || prim < bestPrim) {
                    tcur = t;
                    bestPrim = prim;
                    hit.t = t;
                    hit.u = u;
                    hit.v = v;
                    hit.leaf = k;
                }
            }
        }
        if (ihits) {
            // The stack holds at most one group per tree level below the
            // root, and the build refuses trees deeper than BVH8_STACK
            // levels, so the bound never drops a group.
            if ((grp.y >> 8) && sp < BVH8_STACK)
                stack[sp++] = grp;
            grp = make_uint2(b.x, (ihits << 8) | imask);
        }
        if (!(grp.y >> 8)) {
            if (sp == 0)
                return true;  // nothing left to visit
            grp = stack[--sp];
        }
        // Next internal child: lowest set bit of the current group (octant order).
        uint32_t hits = grp.y >> 8;
        const uint32_t gmask = grp.y & 0xFFu;
        const uint32_t bpos = (uint32_t)(__ffs(hits) - 1);
        const uint32_t s = bpos ^ oct;
        hits &= hits - 1u;
        node = (int)grp.x + __popc(gmask & ((1u << s) - 1u));
        grp.y = (hits << 8) | gmask;
        return false;
    }
};

template <bool ANY, class AlphaFn, class Counter>
OPT_D bool traverse8(const Bvh8Node *__restrict__ nodes, const float4 *__restrict__ triV, float3 o, float3 d,
                     float tmin, float tmax, HitRec &hit, AlphaFn alpha, Counter &ctr, int budget)
{
    hit.leaf = -1;
    if (nodes == nullptr)
        return false;
    Trav8 T;
    T.init(o, d, tmin, tmax, hit, budget);
    while (!T.step<ANY>(nodes, triV, hit, alpha, ctr)) {
    }
    return hit.leaf >= 0;
}

// A queue of rays traversed by persistent warps with lane refill (dynamic
// ray fetch, after Aila and Laine, "Understanding the Efficiency of Ray
// Traversal on GPUs", HPG 2009): a lane whose ray is finished takes the next
// ray of the queue (one atomicAdd per warp for all lanes needing one), so no
// lane idles while the longest ray of its warp finishes. Every lane runs the
// same per-ray traversal as traverse8. All 32 lanes of each warp must call
// it. fetch(i, o, d, tmin, tmax, alpha) loads ray i (and its alpha-test
// parameters); finish(i, hit) stores ray i's result.
template <bool ANY, class Fetch, class Finish, class AlphaFn, class Counter>
OPT_D void traverse8Queue(const Bvh8Node *__restrict__ nodes, const float4 *__restrict__ triV, uint32_t count,
                          uint32_t *next, Fetch fetch, Finish finish, AlphaFn alpha, Counter &ctr, int budget)
{
    const uint32_t lane = threadIdx.x & 31u;
    // The first 32 rays of every warp come in queue order without the
    // counter (warp w takes w * 32 .. w * 32 + 31): no burst of atomics on
    // one address when the grid starts, and none at all when the queue is
    // shorter than the grid. The counter hands out the rest, from there on.
    const uint32_t firstRound = (gridDim.x * blockDim.x) & ~31u;
    bool started = false;
    Trav8 T;
    HitRec hit;
    hit.leaf = -1;
    int ray = -1;
    bool exhausted = false;
    while (true) {
        const bool need = ray < 0 && !exhausted;
        const unsigned nm = __ballot_sync(0xffffffffu, need);
        // Refill in batches: a fetch stalls the whole warp on the atomic, so
        // wait until enough lanes are idle (or none is busy).
        if (nm && (!started || __popc(nm) >= TRAV8_REFILL || __ballot_sync(0xffffffffu, ray >= 0) == 0u)) {
            const int leader = __ffs(nm) - 1;
            uint32_t base;
            if (!started) {
                base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;  // this warp's first 32
                started = true;
            } else {
                base = 0;
                if ((int)lane == leader)
                    base = atomicAdd(next, (uint32_t)__popc(nm));
                base = __shfl_sync(0xffffffffu, base, leader) + firstRound;
            }
            if (need) {
                const uint32_t i = base + (uint32_t)__popc(nm & ((1u << lane) - 1u));
                if (i < count) {
                    float3 o, d;
                    float tmin, tmax;
                    fetch(i, o, d, tmin, tmax, alpha);
                    T.init(o, d, tmin, tmax, hit, budget);
                    ray = (int)i;
                } else {
                    exhausted = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, ray >= 0) == 0u)
            break;
        if (ray >= 0 && (nodes == nullptr || T.step<ANY>(nodes, triV, hit, alpha, ctr))) {
            finish((uint32_t)ray, hit);
            ray = -1;
        }
    }
}
