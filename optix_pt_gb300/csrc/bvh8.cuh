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

#define BVH8_STACK 64

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

template <bool ANY, class AlphaFn, class Counter = NoCount>
OPT_D bool traverse8(const Bvh8Node *__restrict__ nodes, const float4 *__restrict__ triV, float3 o, float3 d,
                     float tmin, float tmax, HitRec &hit, AlphaFn alpha, Counter &&ctr = Counter())
{
    hit.leaf = -1;
    if (nodes == nullptr)
        return false;
    const RayPre pre = rayPrepare(o, d);
    const float3 inv = mk3(safeInv(d.x), safeInv(d.y), safeInv(d.z));
    const uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    uint2 stack[BVH8_STACK];
    int sp = 0;
    int node = 0;
    float tcur = tmax;
    int bestPrim = INT_MAX;
    for (int budget = 1 << 24; budget > 0; --budget) {
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
        const float tlim = tcur * BOX_WIDEN;
        uint32_t ihits = 0, lhits = 0;
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const uint32_t meta = byteOf(b, 8 + s);
            if (meta == 0u)
                continue;
            const int k = s & 3;
            const float xn = fmaf(byteToFloat(s < 4 ? nx0 : nx1, k), axs, bx);
            const float xf = fmaf(byteToFloat(s < 4 ? fx0 : fx1, k), axs, bx);
            const float yn = fmaf(byteToFloat(s < 4 ? ny0 : ny1, k), ays, by);
            const float yf = fmaf(byteToFloat(s < 4 ? fy0 : fy1, k), ays, by);
            const float zn = fmaf(byteToFloat(s < 4 ? nz0 : nz1, k), azs, bz);
            const float zf = fmaf(byteToFloat(s < 4 ? fz0 : fz1, k), azs, bz);
            const float tn = fmaxf(fmaxf(xn, yn), fmaxf(zn, tmin));
            const float tf = fminf(fminf(xf, yf), zf) * BOX_WIDEN;
            if (tn <= fminf(tf, tlim)) {
                if ((imask >> s) & 1u)
                    ihits |= 1u << ((uint32_t)s ^ oct);
                else
                    lhits |= 1u << s;
            }
        }
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
                    return true;
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
        if (ihits && sp < BVH8_STACK)
            stack[sp++] = make_uint2(b.x, (ihits << 8) | imask);
        if (sp == 0)
            break;
        // Next internal child: lowest set bit of the top group (octant order).
        uint2 &g = stack[sp - 1];
        uint32_t hits = g.y >> 8;
        const uint32_t gmask = g.y & 0xFFu;
        const uint32_t bpos = (uint32_t)(__ffs(hits) - 1);
        const uint32_t s = bpos ^ oct;
        hits &= hits - 1u;
        node = (int)g.x + __popc(gmask & ((1u << s) - 1u));
        if (hits)
            g.y = (hits << 8) | gmask;
        else
            --sp;
    }
    return hit.leaf >= 0;
}
