// BVH2 traversal kernels' device routines: closest hit (the radiance ray of
// cu/device_programs.cu:63 with __anyhit__radiance's alpha test, :108-166)
// and occlusion (the shadow ray of cu/path_tracer.cu:396,485 with
// __anyhit__shadow, cu/device_programs.cu:180-219).
#pragma once
#include <climits>
#include "bvh.cuh"

#define BVH_STACK 64  // >= LBVH depth: 30 Morton bits + log2(duplicate run)

struct HitRec {
    float t, u, v;
    int leaf;  // leaf-order triangle index, -1 = miss
};

OPT_D float safeInv(float d) { return 1.0f / (fabsf(d) > 1e-20f ? d : copysignf(1e-20f, d)); }

// Slab tests compare the entry distance with min(exit, current hit) widened
// by 2^-19 relative (cf. Ize, "Robust BVH Ray Traversal", JCGT 2(2), 2013):
// rounding in the box test never culls a box whose triangle the watertight
// test would hit, and boxes holding a triangle at exactly the current hit
// distance are still opened, so equal-t candidates reach the index tie-break
// whatever the tree shape.
#define BOX_WIDEN 1.0000019f

// Slab test of one child box; returns the entry distance or +inf on a miss.
OPT_D float boxEntry(float lox, float hix, float loy, float hiy, float loz, float hiz, float3 o, float3 inv,
                     float tmin, float tmax)
{
    float x0 = (lox - o.x) * inv.x, x1 = (hix - o.x) * inv.x;
    float y0 = (loy - o.y) * inv.y, y1 = (hiy - o.y) * inv.y;
    float z0 = (loz - o.z) * inv.z, z1 = (hiz - o.z) * inv.z;
    float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
    float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fmaxf(z0, z1));
    return tn <= fminf(tf, tmax) * BOX_WIDEN ? tn : __int_as_float(0x7f800000);
}

// Walks the BVH. ANY = true stops at the first accepted hit (occlusion).
// `alpha(leaf, prim, u, v)` decides whether a candidate on a triangle with
// TRI_FLAG_ALPHA is kept (the any-hit programs' optixIgnoreIntersection).
//
// Counters: node() / tri() count BVH work (counting variants only).
struct NoCount {
    OPT_D void node() {}
    OPT_D void tri() {}
};
struct Count {
    uint32_t nodes = 0, tris = 0;
    OPT_D void node() { ++nodes; }
    OPT_D void tri() { ++tris; }
};

// Traversal faults leave a ray's result possibly wrong, so they are never
// silent: the walk returns a miss with one of these leaf values, and the
// kernels count them (renderer totals 8 and 9, optpt_stats).
#define HIT_STACK_OVERFLOW (-3)  // a node group was dropped: the stack was full
#define HIT_CUT_SHORT (-2)       // the walk ran out of its node budget
// Adds a traversal fault of `leaf` (if it is one) to totals[8] / totals[9].
OPT_D void countFault(int leaf, unsigned long long *totals)
{
    if (leaf < -1)
        atomicAdd(totals + (leaf == HIT_STACK_OVERFLOW ? 8 : 9), 1ull);
}

template <bool ANY, class AlphaFn, class Counter>
OPT_D bool traverse(const BvhNode *__restrict__ nodes, const float4 *__restrict__ triV, float3 o, float3 d,
                    float tmin, float tmax, HitRec &hit, AlphaFn alpha, Counter &ctr, int budget)
{
    bool dropped = false;
    hit.leaf = -1;
    if (nodes == nullptr)  // empty scene
        return false;
    const RayPre pre = rayPrepare(o, d);
    const float3 inv = mk3(safeInv(d.x), safeInv(d.y), safeInv(d.z));
    int stack[BVH_STACK];
    int sp = 0;
    int node = 0;
    float tcur = tmax;
    int bestPrim = INT_MAX;
    // The node budget bounds the walk even on a corrupted tree (a valid BVH of
    // n triangles visits at most 2n nodes); running out of it is a fault.
    for (;; --budget) {
        if (budget <= 0) {
            hit.leaf = HIT_CUT_SHORT;
            return false;
        }
        ctr.node();
        const BvhNode *N = nodes + node;
        const float4 a = __ldg(&N->a), b = __ldg(&N->b), c = __ldg(&N->c);
        const int4 r = __ldg(&N->d);
        float tl = r.x >= 0 ? boxEntry(a.x, a.y, a.z, a.w, c.x, c.y, o, inv, tmin, tcur) : __int_as_float(0x7f800000);
        float tr = r.y >= 0 ? boxEntry(b.x, b.y, b.z, b.w, c.z, c.w, o, inv, tmin, tcur) : __int_as_float(0x7f800000);
        bool hl = tl != __int_as_float(0x7f800000), hr = tr != __int_as_float(0x7f800000);
        // Leaf children are intersected on the spot.
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const bool h = side == 0 ? hl : hr;
            const int cnt = side == 0 ? r.z : r.w;
            if (!h || cnt == 0)
                continue;
            const int first = side == 0 ? r.x : r.y;
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
            if (side == 0)
                hl = false;
            else
                hr = false;
        }
        if (hl && hr) {
            const bool leftFirst = tl <= tr;
            if (sp < BVH_STACK)
                stack[sp++] = leftFirst ? r.y : r.x;
            else
                dropped = true;
            node = leftFirst ? r.x : r.y;
        } else if (hl) {
            node = r.x;
        } else if (hr) {
            node = r.y;
        } else {
            if (sp == 0)
                break;
            node = stack[--sp];
        }
    }
    if (dropped) {
        hit.leaf = HIT_STACK_OVERFLOW;
        return false;
    }
    return hit.leaf >= 0;
}

struct NoAlpha {
    OPT_D bool operator()(int, int, float, float) const { return true; }
};
