// BVH layout and traversal: the replacement for OptiX's GAS and optixTrace
// (reference: src/renderer.cpp:441-513 builds the GAS; cu/device_programs.cu:63
// and cu/path_tracer.cu:396,485 trace against it).
//
// Layout in HBM:
//   nodes  : BVH2 node = 4 x 16 B (two child boxes, SoA by axis, plus refs)
//   triV   : 3 x float4 per triangle in leaf order (Morton order); v0.w holds
//            the primitive index, v1.w the material index, v2.w flag bits
//
// Closest hit is decided by (t, primitive index): a candidate replaces the
// current hit if t is smaller, or equal with a smaller primitive index, so the
// result does not depend on traversal order and matches any other traversal
// of the same triangles bit for bit.
#pragma once
#include "common.cuh"

struct BvhNode {
    float4 a;  // (L.lo.x, L.hi.x, L.lo.y, L.hi.y)
    float4 b;  // (R.lo.x, R.hi.x, R.lo.y, R.hi.y)
    float4 c;  // (L.lo.z, L.hi.z, R.lo.z, R.hi.z)
    int4 d;    // (L ref, R ref, L count, R count); count > 0: leaf of `count`
               // triangles starting at ref; count == 0: internal node `ref`;
               // ref < 0: empty child
};

#define TRI_FLAG_ALPHA 1u  // material needs the alpha (any-hit) test

// Nodes one ray may visit before its walk is cut short (and counted as a
// fault): more than 2n, the most a walk of a valid BVH2 of n < 2^25
// triangles visits.
#define TRAV_DEFAULT_BUDGET (1 << 26)
// Entries of a ray's BVH8 node-group stack; the build refuses deeper trees.
#define BVH8_STACK 64

// Per-ray constants of the watertight test (Woop, Benthin, Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013).
struct RayPre {
    float3 o;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

OPT_HD float comp(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

OPT_HD RayPre rayPrepare(float3 o, float3 d)
{
    RayPre r;
    r.o = o;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    float dz = comp(d, kz);
    if (dz < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = comp(d, kx) / dz;
    r.Sy = comp(d, ky) / dz;
    r.Sz = 1.0f / dz;
    return r;
}

// Returns true and (t, u, v) for a hit with tmin < t <= tmax. u, v weight
// vertices 1 and 2 (OptiX's barycentric convention). All roundings are
// explicit (fmaf) so the host oracle reproduces the result exactly.
OPT_HD bool intersectTri(const RayPre &r, float3 v0, float3 v1, float3 v2, float tmin, float tmax, float &t,
                         float &u, float &v)
{
    float3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
    float Ax = fmaf(-r.Sx, Akz, comp(A, r.kx)), Ay = fmaf(-r.Sy, Akz, comp(A, r.ky));
    float Bx = fmaf(-r.Sx, Bkz, comp(B, r.kx)), By = fmaf(-r.Sy, Bkz, comp(B, r.ky));
    float Cx = fmaf(-r.Sx, Ckz, comp(C, r.kx)), Cy = fmaf(-r.Sy, Ckz, comp(C, r.ky));
    float U = fmaf(Cx, By, -(Cy * Bx));
    float V = fmaf(Ax, Cy, -(Ay * Cx));
    float W = fmaf(Bx, Ay, -(By * Ax));
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f))
        return false;
    float det = U + V + W;
    if (det == 0.0f)
        return false;
    float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
    float T = fmaf(U, Az, fmaf(V, Bz, W * Cz));
    float tt = T / det;
    if (!(tt > tmin && tt <= tmax))
        return false;
    t = tt;
    u = V / det;
    v = W / det;
    return true;
}
