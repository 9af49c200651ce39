// Wavefront path-tracing kernels: generate -> (extend -> shade -> shadow) x depth
// -> accumulate. Together they replace the reference's OptiX megakernel
// (cu/device_programs.cu:15-106 raygen loop, cu/path_tracer.cu:17-582
// closest-hit shading with next-event estimation, the any-hit/miss programs
// of cu/device_programs.cu:108-223, and cu/light_sampling.cu:6-81).
//
// Paths live in SoA buffers indexed by path id (= sample-in-batch * npix +
// pixel). Each bounce's rays are a compacted queue: shade appends survivors
// with one atomic per warp (ballot + popc prefix). Kernels are persistent:
// grids of a few blocks per SM loop over the queue length, which they read
// from device memory, so the whole bounce loop can be captured in one graph.
#include <cfloat>
#include "bsdf.cuh"
#include "engine.h"
#include "texture.cuh"
#include "trace.cuh"
#include "bvh8.cuh"
#include "guide.cuh"

// The traversal kernels are compiled for 4 resident 256-thread blocks per SM
// (64 registers per thread): the extra warps hide node-fetch latency better
// than the registers saved spill (3-5 % more rays/s on the 1080p sweep).
#define OPTPT_TRAV_MINB 4

// Closest hit / occlusion through the BVH in use: the compressed 8-wide BVH
// (WIDE) or the BVH2 it was collapsed from.
template <bool ANY, bool WIDE, class A, class C>
OPT_D bool traceScene(const DevScene &s, float3 o, float3 d, float tmin, float tmax, HitRec &h, A alpha, C &ctr)
{
    if constexpr (WIDE)
        return traverse8<ANY>(s.nodes8, s.triV, o, d, tmin, tmax, h, alpha, ctr, s.nodeBudget);
    else
        return traverse<ANY>(s.nodes, s.triV, o, d, tmin, tmax, h, alpha, ctr, s.nodeBudget);
}


namespace {

struct PcgSource {
    Pcg32 *r;
    OPT_D float next() { return r->uniform(); }
};

OPT_D float4 mk4(float3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

// Appends `want` lanes' records to a queue: one atomicAdd per warp, slots
// ordered by lane. Must be reached by all 32 lanes.
template <int N> OPT_D void warpPush(bool want, uint32_t *counter, float4 *const (&dst)[N], const float4 (&val)[N])
{
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (m == 0u)
        return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader)
        base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (want) {
        const uint32_t slot = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
#pragma unroll
        for (int k = 0; k < N; ++k)
            dst[k][slot] = val[k];
    }
}

// Block-granular compaction of the three shading outputs (continuation,
// point-light shadow, emissive shadow): one atomicAdd per block and queue.
// Every thread of the block must call it (trip counts are block-uniform).
struct BlockPushScratch {
    uint32_t count[3][8], base[3][8];
};
OPT_D void blockPush3(const bool (&want)[3], uint32_t *const (&counter)[3], float4 *const (&d0)[2],
                      const float4 (&v0)[2], float4 *const (&d1)[3], const float4 (&v1)[3], float4 *const (&d2)[3],
                      const float4 (&v2)[3], BlockPushScratch &sh)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    unsigned m[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        m[k] = __ballot_sync(0xffffffffu, want[k]);
        if (lane == 0)
            sh.count[k][warp] = (uint32_t)__popc(m[k]);
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        uint32_t tot = 0;
        for (int w = 0; w < nw; ++w) {
            sh.base[k][w] = tot;
            tot += sh.count[k][w];
        }
        const uint32_t b = tot ? atomicAdd(counter[k], tot) : 0u;
        for (int w = 0; w < nw; ++w)
            sh.base[k][w] += b;
    }
    __syncthreads();
    const unsigned below = (1u << lane) - 1u;
    if (want[0]) {
        const uint32_t slot = sh.base[0][warp] + (uint32_t)__popc(m[0] & below);
        d0[0][slot] = v0[0];
        d0[1][slot] = v0[1];
    }
    if (want[1]) {
        const uint32_t slot = sh.base[1][warp] + (uint32_t)__popc(m[1] & below);
#pragma unroll
        for (int k = 0; k < 3; ++k)
            d1[k][slot] = v1[k];
    }
    if (want[2]) {
        const uint32_t slot = sh.base[2][warp] + (uint32_t)__popc(m[2] & below);
#pragma unroll
        for (int k = 0; k < 3; ++k)
            d2[k][slot] = v2[k];
    }
    __syncthreads();  // scratch reused by the next iteration
}

// Alpha test of a candidate (cu/device_programs.cu:108-166 radiance,
// :180-219 shadow). The any-hit programs interpolate the texture coordinate
// without the texture transform (:126-130).
struct AlphaTest {
    const float4 *triV;
    const DevMaterial *materials;
    const int *triIndices;
    const float *texCoords;
    const uint32_t *texels;
    const int4 *texInfo;
    uint32_t seed, pixel, sample, depth;
    float shadowXi;  // < 0: radiance ray (blend uniform hashed per candidate)
    OPT_D bool operator()(int leaf, int prim, float u, float v) const
    {
        const int matIdx = __float_as_int(__ldg(&triV[3 * leaf + 1]).w);
        const DevMaterial &M = materials[matIdx];
        const int4 fl = __ldg(&M.flags);
        const float4 bc = __ldg(&M.baseColour);
        float alpha = bc.w;
        if ((fl.z & TEXBIT_BASE) && texCoords) {
            const int i0 = __ldg(triIndices + 3 * prim), i1 = __ldg(triIndices + 3 * prim + 1),
                      i2 = __ldg(triIndices + 3 * prim + 2);
            const float tu = baryInterp(u, v, __ldg(texCoords + 2 * i0), __ldg(texCoords + 2 * i1),
                                        __ldg(texCoords + 2 * i2));
            const float tv = baryInterp(u, v, __ldg(texCoords + 2 * i0 + 1), __ldg(texCoords + 2 * i1 + 1),
                                        __ldg(texCoords + 2 * i2 + 1));
            alpha *= sampleTexture(texels, __ldg(texInfo + __ldg(&M.tex0).x), tu, tv).w;
        }
        if (fl.y == AM_MASK)
            return !(alpha < __ldg(&M.emissionCutoff).w);
        if (fl.y == AM_BLEND) {
            const float xi = shadowXi >= 0.0f ? shadowXi : blendUniform(seed, pixel, sample, depth, (uint32_t)prim);
            return !(xi > alpha);
        }
        return true;
    }
};

OPT_D AlphaTest makeAlpha(const DevScene &s, uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t depth,
                          float shadowXi)
{
    return AlphaTest{s.triV, s.materials, s.triIndices, s.texCoords, s.texels, s.texInfo,
                     seed, pixel, sample, depth, shadowXi};
}

// ------------------------------------------------------------------ generate
// normalize(ndcx * U + ndcy * V + W) rounded operation by operation, without
// fused multiply-adds, exactly as the host restatement evaluates it: camera
// rays, and therefore first hits, are bit-identical on both sides.
OPT_D float3 cameraDir(float nx, float ny, float3 U, float3 V, float3 W)
{
    const float3 d = mk3(__fadd_rn(__fadd_rn(__fmul_rn(nx, U.x), __fmul_rn(ny, V.x)), W.x),
                         __fadd_rn(__fadd_rn(__fmul_rn(nx, U.y), __fmul_rn(ny, V.y)), W.y),
                         __fadd_rn(__fadd_rn(__fmul_rn(nx, U.z), __fmul_rn(ny, V.z)), W.z));
    const float dd = __fadd_rn(__fadd_rn(__fmul_rn(d.x, d.x), __fmul_rn(d.y, d.y)), __fmul_rn(d.z, d.z));
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dd));
    return mk3(__fmul_rn(d.x, inv), __fmul_rn(d.y, inv), __fmul_rn(d.z, inv));
}

// Camera ray with pixel jitter (cu/device_programs.cu:40-53).
__global__ void __launch_bounds__(256) kGenerate(FrameParams fp, WaveBufs q)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t sampleBase = __ldg(fp.state);
    const float4 e4 = __ldg(&fp.fc->eye), u4 = __ldg(&fp.fc->U), v4 = __ldg(&fp.fc->V), w4 = __ldg(&fp.fc->W);
    const uint32_t seed = __float_as_uint(e4.w);
    float3 eye = f3of4(e4), camU = f3of4(u4), camV = f3of4(v4), camW = f3of4(w4);
    const uint32_t numPaths = passPaths(fp);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < numPaths; p += stride) {
        uint32_t pixel, sample, x, y, w = fp.w, h = fp.h;
        if (fp.batch.on) {
            // the path's view: its camera and resolution (batched multi-view)
            pathPixelSample(fp, p, pixel, sample);
            const BatchView &V = fp.batch.views[__ldg(fp.batch.pixelView + pixel)];
            const float4 ve = __ldg(&V.eye), vu = __ldg(&V.U), vv = __ldg(&V.V), vw = __ldg(&V.W);
            eye = f3of4(ve);
            camU = f3of4(vu);
            camV = f3of4(vv);
            camW = f3of4(vw);
            w = __float_as_uint(ve.w);
            h = __float_as_uint(vu.w);
            const uint32_t local = pixel - __float_as_uint(vv.w);
            x = local % w;
            y = local / w;
        } else {
            pixel = p % fp.npix;
            sample = sampleBase + p / fp.npix;
            x = pixel % fp.w;
            y = pixel / fp.w;
        }
        Pcg32 rng = pathRng(seed, pixel, sample, 0u);
        const float jx = rng.uniform(), jy = rng.uniform();
        const float fx = (float)x + jx, fy = (float)y + jy;
        // (multiplying by +-2 is exact, so a fused multiply-add rounds the
        // same as the separate operations here)
        const float ndcx = (fx / (float)w) * 2.0f + -1.0f;
        const float ndcy = (fy / (float)h) * -2.0f + 1.0f;
        const float3 dir = cameraDir(ndcx, ndcy, camU, camV, camW);
        q.rayO[1][p] = mk4(eye, __int_as_float((int)p));
        q.rayD[1][p] = mk4(dir, 0.0f);
        q.pathT[p] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(0u));
        q.pathL[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        q.counters[CNT_EXT + 1] = numPaths;
}

// ------------------------------------------------------------------ extend
// Closest hit of each queued ray: tmin 0, tmax 1e16 (cu/device_programs.cu:63).
// Adds per-thread traversal counts to totals[slot], [slot + 1] (counting mode).
OPT_D void flushCounts(const Count &c, unsigned long long *totals, int slot)
{
    unsigned long long n = c.nodes, t = c.tris;
    for (int off = 16; off > 0; off >>= 1) {
        n += __shfl_down_sync(0xffffffffu, n, off);
        t += __shfl_down_sync(0xffffffffu, t, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(totals + slot, n);
        atomicAdd(totals + slot + 1, t);
    }
}

template <bool COUNT, bool WIDE>
__global__ void __launch_bounds__(256, OPTPT_TRAV_MINB) kExtend(DevScene s, FrameParams fp, WaveBufs q, int depth)
{
    const uint32_t count = q.counters[CNT_EXT + depth];
    const int cur = depth & 1;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t sampleBase = __ldg(fp.state);
    const uint32_t seed = __float_as_uint(__ldg(&fp.fc->eye).w);
    typename std::conditional<COUNT, Count, NoCount>::type ctr;
    if constexpr (WIDE) {
        // persistent warps over the queue, lanes refilled as their rays finish
        auto fetch = [&](uint32_t i, float3 &o, float3 &d, float &tmin, float &tmax, AlphaTest &at) {
            const float4 ro = q.rayO[cur][i], rd = q.rayD[cur][i];
            pathPixelSample(fp, (uint32_t)__float_as_int(ro.w), at.pixel, at.sample);
            o = f3of4(ro);
            d = f3of4(rd);
            tmin = 0.0f;
            tmax = 1e16f;
        };
        auto finish = [&](uint32_t i, const HitRec &h) {
            q.hit[i] = h.leaf >= 0 ? make_float4(h.t, h.u, h.v, __int_as_float(h.leaf))
                                   : make_float4(__int_as_float(0x7f800000), 0.0f, 0.0f, __int_as_float(-1));
            countFault(h.leaf, q.totals);
        };
        traverse8Queue<false>(s.nodes8, s.triV, count, q.counters + CNT_FETCH_EXT + depth, fetch, finish,
                              makeAlpha(s, seed, 0u, 0u, (uint32_t)depth, -1.0f), ctr, s.nodeBudget);
    } else {
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
            const float4 ro = q.rayO[cur][i], rd = q.rayD[cur][i];
            const uint32_t path = (uint32_t)__float_as_int(ro.w);
            uint32_t pixel, sample;
            pathPixelSample(fp, path, pixel, sample);
            const AlphaTest at = makeAlpha(s, seed, pixel, sample, (uint32_t)depth, -1.0f);
            HitRec h;
            const bool hit = traceScene<false, WIDE>(s, f3of4(ro), f3of4(rd), 0.0f, 1e16f, h, at, ctr);
            q.hit[i] = hit ? make_float4(h.t, h.u, h.v, __int_as_float(h.leaf))
                           : make_float4(__int_as_float(0x7f800000), 0.0f, 0.0f, __int_as_float(-1));
            countFault(h.leaf, q.totals);
        }
    }
    if constexpr (COUNT)
        flushCounts(ctr, q.totals, 4);
}

// ------------------------------------------------------------------ shade
struct LightSampleD {
    float3 dir, Li;
    float pdf, dist;
};

// point_sample / directional_sample / spot_sample (cu/light_sampling.cu:6-59)
OPT_D LightSampleD sampleLight(const DevLight &L, float3 p)
{
    LightSampleD r;
    const float4 a = __ldg(&L.p0Type), b = __ldg(&L.radianceDist), c = __ldg(&L.normalCosW);
    const int type = __float_as_int(a.w);
    const float3 rad = f3of4(b);
    r.pdf = 1.0f;
    if (type == 1) {
        const float3 n = f3of4(c);
        const float3 pos = p + (-n * b.w);
        r.dir = -n;
        r.Li = rad;
        r.dist = length3(pos - p);
    } else {
        float3 dir = f3of4(a) - p;
        const float dist = length3(dir);
        dir = dir / dist;
        r.dir = dir;
        r.dist = dist;
        if (type == 2) {  // falloff (include/sampling.h:64-77)
            const float cw = c.w, cfs = __ldg(&L.cosFalloff).x;
            const float ct = dot3(f3of4(c), -dir);
            float fo;
            if (ct < cw)
                fo = 0.0f;
            else if (ct > cfs)
                fo = 1.0f;
            else {
                const float dl = (ct - cw) / (cfs - cw);
                fo = (dl * dl) * (dl * dl);
            }
            r.Li = rad * fo / (dist * dist);
        } else {
            r.Li = rad / (dist * dist);
        }
    }
    return r;
}

OPT_D bool nonzeroOrNonfinite(float3 c)
{
    return c.x != 0.0f || c.y != 0.0f || c.z != 0.0f || !isfinite(c.x) || !isfinite(c.y) || !isfinite(c.z);
}

OPT_D float2 interpTc(const DevScene &s, int prim, float u, float v)
{
    const int i0 = __ldg(s.triIndices + 3 * prim), i1 = __ldg(s.triIndices + 3 * prim + 1),
              i2 = __ldg(s.triIndices + 3 * prim + 2);
    const float2 t0 = __ldg(reinterpret_cast<const float2 *>(s.texCoords) + i0);
    const float2 t1 = __ldg(reinterpret_cast<const float2 *>(s.texCoords) + i1);
    const float2 t2 = __ldg(reinterpret_cast<const float2 *>(s.texCoords) + i2);
    return make_float2(baryInterp(u, v, t0.x, t1.x, t2.x), baryInterp(u, v, t0.y, t1.y, t2.y));
}

OPT_D float4 texAt(const DevScene &s, int tex, float4 tf, float2 tc)
{
    const float x = fmaf(tc.x, tf.z, tf.x), y = fmaf(tc.y, tf.w, tf.y);  // uv * scale + offset
    return sampleTexture(s.texels, __ldg(s.texInfo + tex), x, y);
}

// Constants of a shading launch.
struct ShadeConsts {
    uint32_t seed;  // frame seed
    int vis;        // material visualisation mode (0: path tracing)
    float3 bg;      // background colour
    float ramp;     // guided variant: phase-in of the mixture's selection probability
};

OPT_D ShadeConsts shadeConsts(const FrameParams &fp, bool guided)
{
    ShadeConsts k;
    k.seed = __float_as_uint(__ldg(&fp.fc->eye).w);
    k.vis = __float_as_int(__ldg(&fp.fc->U).w);
    k.bg = f3of4(__ldg(&fp.fc->bg));
    // guide selection probability: ramps in with training (any value keeps
    // the estimator unbiased; an untrained proposal should be used sparingly)
    k.ramp = guided ? fminf(1.0f, (float)__ldg(fp.guide.step) / fp.guide.alphaRamp) : 0.0f;
    return k;
}

// Closest-hit shading of one ray at bounce `depth` (queue slot i; ray ro/rd
// with the path id in ro.w; its hit record hrec: t, u, v, leaf): attributes,
// textures, categorisation, emitter hit, point-light and emissive-triangle
// NEE set-up, BSDF (or guided) sampling and Russian roulette
// (cu/path_tracer.cu:17-582), or the miss (cu/device_programs.cu:168-174).
// Reads and writes the path's throughput, flags and radiance; returns the
// continuation ray (cont) and the shadow rays to trace (wantP, wantE).
// GUIDED: the learned-guiding variant (mixture sampling and training
// records); the plain variant carries none of that code.
template <bool GUIDED>
OPT_D void shadeRay(const DevScene &s, const FrameParams &fp, const WaveBufs &q, int depth, uint32_t i,
                    const ShadeConsts &k, float4 ro, float4 rd, float4 hrec, bool &cont, float4 (&nxtRay)[2],
                    bool &wantP, float4 (&shP)[3], bool &wantE, float4 (&shE)[3])
{
    const uint32_t seed = k.seed;
    const int vis = k.vis;
    const float3 bg = k.bg;
    const float ramp = k.ramp;

    const uint32_t path = (uint32_t)__float_as_int(ro.w);
    float4 T4 = q.pathT[path];
    float3 T = f3of4(T4);
    float3 L = f3of4(q.pathL[path]);
    uint32_t flags = __float_as_uint(T4.w);
    const float3 rayDir = f3of4(rd), rayOrig = f3of4(ro);
    const int leaf = __float_as_int(hrec.w);
    // Guiding: a training path's previous vertex learns the radiance
    // and throughput on arrival here (everything added from now on
    // arrived along its sampled direction).
    const GuidePass &gp = fp.guide;
    const uint32_t stamp = __ldg(fp.state + 1) + 1u;
    float4 *rec = nullptr;
    if (GUIDED && gp.train &&
        path % gp.trainStride == guideTrainOffset(path / gp.trainStride, stamp, gp.trainStride))
        rec = gp.rec + (size_t)(path / gp.trainStride) * fp.maxDepth * GUIDE_REC;
    if (rec && depth > 1) {
        float4 *r = rec + (size_t)(depth - 2) * GUIDE_REC;
        r[5] = mk4(L, __uint_as_float(stamp));
        r[6] = mk4(T, 0.0f);
    }
    if (leaf < 0) {
        L = L + bg * T;
    } else {
        uint32_t pixel, sample;
        pathPixelSample(fp, path, pixel, sample);
        Pcg32 rng = pathRng(seed, pixel, sample, (uint32_t)depth);
        PcgSource U{&rng};
        const float4 t0 = __ldg(&s.triV[3 * leaf]), t1 = __ldg(&s.triV[3 * leaf + 1]),
                     t2 = __ldg(&s.triV[3 * leaf + 2]);
        const int prim = __float_as_int(t0.w), matIdx = __float_as_int(t1.w);
        const DevMaterial &M = s.materials[matIdx];
        const float4 mbc = __ldg(&M.baseColour), mem = __ldg(&M.emissionCutoff), msh = __ldg(&M.sheen);
        const float4 mp0 = __ldg(&M.p0), mp1 = __ldg(&M.p1);
        const int4 mfl = __ldg(&M.flags);
        const float u = hrec.y, v = hrec.z;

        float2 tc = make_float2(0.0f, 0.0f);
        if (mfl.z != 0 && s.texCoords)
            tc = interpTc(s, prim, u, v);

        float3 hitPoint = rayOrig + hrec.x * rayDir;
        const float3 v0 = f3of4(t0), v1 = f3of4(t1), v2 = f3of4(t2);
        const float3 Ng = normalize3(cross3(v1 - v0, v2 - v0));
        float3 interpN = Ng;
        bool hasN = false;
        if (s.normals) {
            const int i0 = __ldg(s.triIndices + 3 * prim), i1 = __ldg(s.triIndices + 3 * prim + 1),
                      i2 = __ldg(s.triIndices + 3 * prim + 2);
            const float3 n0 = mk3(__ldg(s.normals + 3 * i0), __ldg(s.normals + 3 * i0 + 1),
                                  __ldg(s.normals + 3 * i0 + 2));
            const float3 n1 = mk3(__ldg(s.normals + 3 * i1), __ldg(s.normals + 3 * i1 + 1),
                                  __ldg(s.normals + 3 * i1 + 2));
            const float3 n2 = mk3(__ldg(s.normals + 3 * i2), __ldg(s.normals + 3 * i2 + 1),
                                  __ldg(s.normals + 3 * i2 + 2));
            interpN = normalize3((1.0f - u - v) * n0 + u * n1 + v * n2);
            hasN = true;
        }
        float3 normal = interpN;
        if ((mfl.z & TEXBIT_NORMAL) && s.texCoords) {
            // Tangent-space normal map (cu/path_tracer.cu:64-144).
            float3 sn = f3of4(texAt(s, __ldg(&M.tex0).y, __ldg(&M.tf[1]), tc));
            sn = normalize3(sn * 2.0f - mk3s(1.0f));
            const int i0 = __ldg(s.triIndices + 3 * prim), i1 = __ldg(s.triIndices + 3 * prim + 1),
                      i2 = __ldg(s.triIndices + 3 * prim + 2);
            const float2 w0 = __ldg(reinterpret_cast<const float2 *>(s.texCoords) + i0);
            const float2 w1 = __ldg(reinterpret_cast<const float2 *>(s.texCoords) + i1);
            const float2 w2 = __ldg(reinterpret_cast<const float2 *>(s.texCoords) + i2);
            const float3 e1 = v1 - v0, e2 = v2 - v0;
            const float2 d1 = make_float2(w1.x - w0.x, w1.y - w0.y), d2 = make_float2(w2.x - w0.x, w2.y - w0.y);
            const float f = 1.0f / (d1.x * d2.y - d2.x * d1.y);
            float3 tl = mk3(f * (d2.y * e1.x - d1.y * e2.x), f * (d2.y * e1.y - d1.y * e2.y),
                            f * (d2.y * e1.z - d1.y * e2.z));
            tl = normalize3(tl);
            const float3 N = hasN ? interpN : Ng;
            const float3 Tg = normalize3(tl - dot3(tl, N) * N);
            const float3 B = cross3(N, Tg);
            normal = normalize3(mk3(Tg.x * sn.x + B.x * sn.y + N.x * sn.z, Tg.y * sn.x + B.y * sn.y + N.y * sn.z,
                                    Tg.z * sn.x + B.z * sn.y + N.z * sn.z));
        }

        // Material inputs after textures (cu/path_tracer.cu:165-229).
        float3 albedo = f3of4(mbc);
        float alpha = mbc.w;
        if (mfl.z & TEXBIT_BASE) {
            const float4 bt = texAt(s, __ldg(&M.tex0).x, __ldg(&M.tf[0]), tc);
            albedo = albedo * f3of4(bt);
            alpha *= bt.w;
        }
        float occlusion = 1.0f, roughness = mp0.y, metallic = mp0.z;
        if (mfl.z & TEXBIT_MR) {
            const float4 mr = texAt(s, __ldg(&M.tex0).z, __ldg(&M.tf[2]), tc);
            occlusion *= mr.x;
            roughness *= mr.y;
            metallic = mr.z < 0.04f ? 0.0f : metallic * mr.z;
        }
        float3 emission = f3of4(mem);
        if (mfl.z & TEXBIT_EMISSIVE)
            emission = emission * f3of4(texAt(s, __ldg(&M.tex0).w, __ldg(&M.tf[3]), tc));
        float3 sheenColour = f3of4(msh);
        if (mfl.z & TEXBIT_SHEENC)
            sheenColour = sheenColour * f3of4(texAt(s, __ldg(&M.tex1).x, __ldg(&M.tf[4]), tc));
        float sheenRoughness = msh.w;
        if (mfl.z & TEXBIT_SHEENR)
            sheenRoughness *= texAt(s, __ldg(&M.tex1).y, __ldg(&M.tf[5]), tc).w;

        const bsdf::CatIn ci{(uint32_t)mfl.x, mp1.z, mp1.w, mp1.x, mp0.w, mp1.y};
        float cw;
        const uint32_t cat = bsdf::categorise(ci, -rayDir, normal, roughness, metallic, emission, sheenColour,
                                              sheenRoughness, U, cw);
        const bool spec = (cat & MF_SPECULAR) != 0;

        if (vis != 0) {
            // Material visualisation AOVs (cu/path_tracer.cu:252-315).
            switch (vis) {
            case 1: L = mk3s(metallic); break;
            case 2: L = mk3s(roughness); break;
            case 3: L = mk3s(occlusion); break;
            case 4: L = emission; break;
            case 5: L = normal * 0.5f + mk3s(0.5f); break;
            case 6: L = Ng * 0.5f + mk3s(0.5f); break;
            case 7: L = albedo; break;
            case 8: L = metallic * albedo * mk3s(mp0.w); break;
            case 10: L = sheenColour; break;
            case 11: L = mk3s(sheenRoughness); break;
            case 12: L = mk3s(alpha); break;
            default: break;
            }
        } else {
            if (!spec)
                hitPoint = hitPoint - rayDir * OPT_SHADOW_BIAS;
            if (cat & MF_EMISSION) {
                if (dot3(rayDir, normal) < 0.0f && (depth == 1 || (flags & 1u)))
                    L = L + (emission + albedo * T);
            } else {
                flags = spec ? 1u : 0u;
                const bsdf::MatMR m = bsdf::makeMatMR(albedo, mp0.x, metallic, sheenColour, cat, normal,
                                                      roughness, mp1.w, msh.w);
                const float3 wo = -rayDir;
                if (!spec && s.numLights != 0) {
                    // Point / directional / spot NEE (cu/path_tracer.cu:375-412).
                    const float lu = U.next();
                    const int li = min((int)(lu * (float)s.numLights), s.numLights - 1);
                    const float selPdf = 1.0f / (float)s.numLights;
                    const LightSampleD ls = sampleLight(s.lights[li], hitPoint);
                    const float cosX = fmaxf(dot3(normal, ls.dir), 0.0f);
                    const float sxi = U.next();
                    const float3 brdf = bsdf::evalBrdf(m, ls.dir, wo, U);
                    const float3 colour = brdf * ls.Li * cosX / ls.pdf / selPdf;
                    const float3 c = colour * T;
                    if (nonzeroOrNonfinite(c)) {
                        wantP = true;
                        shP[0] = mk4(hitPoint, __int_as_float((int)path));
                        shP[1] = mk4(ls.dir, ls.dist - OPT_SCENE_EPSILON);
                        shP[2] = mk4(c, sxi);
                    }
                }
                if (!spec && s.numEmissive != 0) {
                    // Emissive-triangle NEE (cu/path_tracer.cu:415-515).
                    const int ei = min((int)(U.next() * (float)s.numEmissive), s.numEmissive - 1);
                    const float selPdf = 1.0f / (float)s.numEmissive;
                    float xa = U.next(), xb = U.next();
                    if (xa + xb > 1.0f) {
                        xa = 1.0f - xa;
                        xb = 1.0f - xb;
                    }
                    const float3 p0 = f3of4(__ldg(&s.emisV[3 * ei])), p1 = f3of4(__ldg(&s.emisV[3 * ei + 1])),
                                 p2 = f3of4(__ldg(&s.emisV[3 * ei + 2]));
                    const float3 e1 = p1 - p0, e2 = p2 - p0;
                    const float3 lightPos = p0 + e1 * xa + e2 * xb;
                    const float3 lnv = cross3(e1, e2);
                    const float3 ln = normalize3(lnv);
                    const float pdfA = 1.0f / (length3(lnv) * 0.5f);
                    const float3 lvec = lightPos - hitPoint;
                    const float dist = length3(lvec);
                    const float3 ldir = lvec / dist;
                    const float cosY = fmaxf(0.0f, dot3(ln, -ldir));
                    const float4 er = __ldg(&s.emisRad[ei]);
                    float3 Le = f3of4(er);
                    const DevMaterial &EM = s.materials[__float_as_int(er.w)];
                    if ((__ldg(&EM.flags).z & TEXBIT_EMISSIVE) && s.texCoords) {
                        // Barycentrics of the light point (include/barycentrics.h:17-44); the
                        // hit material's transform is applied, as in the reference (:466-468).
                        const float3 mm = cross3(p1 - p0, p2 - p0);
                        const float ax = fabsf(mm.x), ay = fabsf(mm.y), az = fabsf(mm.z);
                        float nu, nv, ood;
                        auto area2 = [](float x1, float y1, float x2, float y2, float x3, float y3) {
                            return (x1 - x2) * (y2 - y3) - (x2 - x3) * (y1 - y2);
                        };
                        if (ax >= ay && ax >= az) {
                            nu = area2(lightPos.y, lightPos.z, p1.y, p1.z, p2.y, p2.z);
                            nv = area2(lightPos.y, lightPos.z, p2.y, p2.z, p0.y, p0.z);
                            ood = 1.0f / mm.x;
                        } else if (ay >= ax && ay >= az) {
                            nu = area2(lightPos.x, lightPos.z, p1.x, p1.z, p2.x, p2.z);
                            nv = area2(lightPos.x, lightPos.z, p2.x, p2.z, p0.x, p0.z);
                            ood = 1.0f / -mm.y;
                        } else {
                            nu = area2(lightPos.x, lightPos.y, p1.x, p1.y, p2.x, p2.y);
                            nv = area2(lightPos.x, lightPos.y, p2.x, p2.y, p0.x, p0.y);
                            ood = 1.0f / mm.z;
                        }
                        const float bu = nu * ood, bv = nv * ood;
                        const float2 c0 = __ldg(&s.emisTc[3 * ei]), c1 = __ldg(&s.emisTc[3 * ei + 1]),
                                     c2 = __ldg(&s.emisTc[3 * ei + 2]);
                        const float4 tf = __ldg(&M.tf[3]);
                        const float ex = fmaf(baryInterp(bu, bv, c0.x, c1.x, c2.x), tf.z, tf.x);
                        const float ey = fmaf(baryInterp(bu, bv, c0.y, c1.y, c2.y), tf.w, tf.y);
                        Le = Le * f3of4(sampleTexture(s.texels, __ldg(s.texInfo + __ldg(&EM.tex0).w), ex, ey));
                    }
                    const float cosX = fmaxf(0.0f, dot3(normal, ldir));
                    const float G = cosX * cosY / (dist * dist);
                    const float sxi = U.next();
                    const float3 brdf = bsdf::evalBrdf(m, ldir, wo, U);
                    const float3 colour = Le * brdf * G / (pdfA * selPdf);
                    const float3 c = colour * T;
                    if (nonzeroOrNonfinite(c)) {
                        wantE = true;
                        shE[0] = mk4(hitPoint, __int_as_float((int)path));
                        shE[1] = mk4(ldir, dist - OPT_SCENE_EPSILON);
                        shE[2] = mk4(c, sxi);
                    }
                }
                if ((uint32_t)depth < fp.maxDepth) {
                    // BSDF sampling, throughput, Russian roulette (cu/path_tracer.cu:522-581).
                    float3 xi;
                    xi.x = U.next();
                    xi.y = U.next();
                    xi.z = U.next();
                    bsdf::Sample smp;
                    smp.dir = mk3s(0.0f);
                    smp.bsdf = mk3s(0.0f);
                    smp.pdf = 0.0f;
                    const bool guided =
                        GUIDED && (uint32_t)depth <= fp.guide.maxDepth && bsdf::guidable(cat);
                    float pSample;  // density wi was drawn from (category chosen)
                    float pcLobe = 0.0f;  // the lobe's own density at wi (guided vertices)
                    bool live;
                    if (guided) {
                        // One-sample MIS of the learned mixture and the lobe's own
                        // sampler. The lobe's density decides the kill test, as in
                        // the plain estimator, so both integrate over the same set.
                        // primary hits of one pixel share its first sample's mixture
                        const uint32_t mi =
                            depth == 1 && gp.sharePrimary
                                ? i % (fp.batch.on ? __ldg(fp.batch.dyn) : fp.npix)
                                : i;
                        const guide::Packed gm = reinterpret_cast<const guide::Packed *>(gp.mix)[mi];
                        // selection probability: the network's, phased in with training
                        const float alpha = ramp * fminf(fp.guide.alphaMax,
                                                         fmaxf(fp.guide.alphaMin, guide::packedSelect(gm)));
                        const float uSel = U.next();
                        // the lobe's own sampler: its direction only (value and
                        // density follow for either strategy's direction)
                        smp.dir = uSel < alpha ? guide::mixtureSample(gm, xi.x, 1.0f - xi.y, xi.z)
                                               : bsdf::lobeDir(m, wo, xi);
                        const float pc = bsdf::lobePdf(m, smp.dir, wo);
                        pcLobe = pc;
                        smp.bsdf = bsdf::lobeValue(m, smp.dir, wo);
                        pSample = alpha * guide::mixturePdf(gm, smp.dir) + (1.0f - alpha) * fmaxf(pc, 0.0f);
                        smp.pdf = pSample * cw;
                        live = !(pc * cw < OPT_SCENE_EPSILON || maxc3(smp.bsdf) < OPT_SCENE_EPSILON) &&
                               pSample > 0.0f;
                    } else {
                        bsdf::sampleBrdf(m, wo, xi, U, smp);
                        pSample = smp.pdf;
                        smp.pdf *= cw;
                        live = !(smp.pdf < OPT_SCENE_EPSILON || maxc3(smp.bsdf) < OPT_SCENE_EPSILON);
                    }
                    if (live) {
                        const float3 fcos = smp.bsdf * fabsf(dot3(normal, smp.dir));
                        // Russian roulette reads the plain estimator's throughput for
                        // this direction at guided vertices: a well-guided sample has a
                        // small throughput because its density is high, and must not be
                        // rouletted for it (any survival probability is unbiased).
                        const float maxC = guided ? maxc3(T * (fcos / (cw * fmaxf(pcLobe, 1e-30f))))
                                                  : maxc3(T * (fcos / smp.pdf));
                        T = T * (fcos / smp.pdf);
                        bool alive = true;
                        if (depth > 3 || maxC < 0.3f) {
                            const float qq = fmaxf(0.05f, 1.0f - maxC);
                            if (U.next() < qq)
                                alive = false;
                            else
                                T = T / (1.0f - qq);
                        }
                        if (alive) {
                            if (!spec)
                                hitPoint = hitPoint + rayDir * OPT_SHADOW_BIAS;
                            const float3 origin = hitPoint + smp.dir * OPT_SCENE_EPSILON;
                            cont = true;
                            nxtRay[0] = mk4(origin, __int_as_float((int)path));
                            nxtRay[1] = mk4(smp.dir, 0.0f);
                            if (rec && guided) {
                                // the inference kernel's inputs: hit point, face-forwarded
                                // geometric normal, outgoing direction
                                float4 *r = rec + (size_t)(depth - 1) * GUIDE_REC;
                                const float3 nIn = dot3(Ng, rayDir) < 0.0f ? Ng : -Ng;
                                r[0] = mk4(rayOrig + hrec.x * rayDir, pSample);
                                r[1] = mk4(nIn, __uint_as_float(stamp));
                                r[2] = mk4(wo, fmaxf(pcLobe, 0.0f));
                                r[3] = mk4(smp.dir, 0.0f);
                                r[4] = mk4(fcos, 0.0f);
                            }
                        }
                    }
                }
            }
        }
    }
    q.pathT[path] = mk4(T, __uint_as_float(flags));
    q.pathL[path] = mk4(L, 0.0f);
}

// Closest-hit shading of a bounce's queued rays (shadeRay), with the
// continuation and shadow rays appended to the next queues.
// 72 registers (seven 128-thread blocks per SM) with some spilling to L1
// beats the 124 the compiler would take: the kernel waits on scattered
// material, vertex and texture reads, and more resident warps hide them
// (measured on the 1080p sweep: 1.43 -> 1.27 ms per pass at 64 registers,
// 96 and 80 in between; with one copy of each BSDF lobe, 72 is 0.9 % ahead
// of 64 on the sweep and 56 behind).
// The guided variant (mixture reads, sampling and densities) has its own cap.
#ifndef OPTPT_SHADE_GUIDED_REGS
#define OPTPT_SHADE_GUIDED_REGS 72
#endif
template <bool GUIDED, bool BLOCKPUSH>
__global__ void __maxnreg__(GUIDED ? OPTPT_SHADE_GUIDED_REGS : 72) kShade(DevScene s, FrameParams fp, WaveBufs q,
                                                                         int depth)
{
    const uint32_t count = q.counters[CNT_EXT + depth];
    const int lane = threadIdx.x & 31;
    const uint32_t warpId = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nWarps = (gridDim.x * blockDim.x) >> 5;
    const int cur = depth & 1, nxt = cur ^ 1;
    const ShadeConsts k = shadeConsts(fp, GUIDED);
    float4 *const nextQ[2] = {q.rayO[nxt], q.rayD[nxt]};
    float4 *const shPQ[3] = {q.shO[0], q.shD[0], q.shC[0]};
    float4 *const shEQ[3] = {q.shO[1], q.shD[1], q.shC[1]};

    __shared__ BlockPushScratch pushScratch;
    // warp-granular compaction walks the queue by warps; block-granular by
    // blocks, so that every thread of a block makes the same number of trips
    const uint32_t first = BLOCKPUSH ? blockIdx.x * blockDim.x : warpId * 32u;
    const uint32_t step = BLOCKPUSH ? gridDim.x * blockDim.x : nWarps * 32u;
    for (uint32_t base = first; base < count; base += step) {
        const uint32_t i = base + (BLOCKPUSH ? threadIdx.x : (uint32_t)lane);
        bool cont = false, wantP = false, wantE = false;
        float4 nxtRay[2], shP[3], shE[3];
        if (i < count)
            shadeRay<GUIDED>(s, fp, q, depth, i, k, q.rayO[cur][i], q.rayD[cur][i], q.hit[i], cont, nxtRay, wantP,
                             shP, wantE, shE);
        if (BLOCKPUSH) {
            const bool want[3] = {cont, wantP, wantE};
            uint32_t *const ctrs[3] = {q.counters + CNT_EXT + depth + 1, q.counters + CNT_SHADOW_P + depth,
                                       q.counters + CNT_SHADOW_E + depth};
            blockPush3(want, ctrs, nextQ, nxtRay, shPQ, shP, shEQ, shE, pushScratch);
        } else {
            warpPush<2>(cont, q.counters + CNT_EXT + depth + 1, nextQ, nxtRay);
            warpPush<3>(wantP, q.counters + CNT_SHADOW_P + depth, shPQ, shP);
            warpPush<3>(wantE, q.counters + CNT_SHADOW_E + depth, shEQ, shE);
        }
    }
}

// ------------------------------------------------------------------ shadow
// A shadow ray's outcome: an unoccluded ray adds its contribution to the
// path's radiance; an occluded one adds c * 0, which only matters (as NaN)
// when the contribution was not finite.
OPT_D void resolveShadow(const WaveBufs &q, uint32_t path, float4 c, bool occluded)
{
    const float3 cc = f3of4(c);
    const bool finite = isfinite(cc.x) && isfinite(cc.y) && isfinite(cc.z);
    if (!occluded || !finite) {
        float4 L = q.pathL[path];
        const float3 add = occluded ? cc * 0.0f : cc;
        q.pathL[path] = make_float4(L.x + add.x, L.y + add.y, L.z + add.z, L.w);
    }
}

// Occlusion test of queued NEE rays, tmin = SCENE_EPSILON
// (cu/path_tracer.cu:396,485, cu/device_programs.cu:180-219). An unoccluded
// ray adds its contribution; an occluded one adds contribution * 0, which
// only matters (as NaN) when the contribution was not finite, exactly as the
// reference's lightVisibility product.
template <bool COUNT, bool WIDE>
__global__ void __launch_bounds__(256, OPTPT_TRAV_MINB)
    kShadow(DevScene s, FrameParams fp, WaveBufs q, int depth, int which)
{
    const uint32_t count = q.counters[(which == 0 ? CNT_SHADOW_P : CNT_SHADOW_E) + depth];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t sampleBase = __ldg(fp.state);
    const uint32_t seed = __float_as_uint(__ldg(&fp.fc->eye).w);
    typename std::conditional<COUNT, Count, NoCount>::type ctr;
    // Shadow rays are short: a lane-refilling persistent warp (as the
    // extension kernel uses) spends more on refills than it saves here
    // (measured), so each thread walks the queue with a fixed stride.
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += stride) {
        const float4 o = q.shO[which][j], d = q.shD[which][j], c = q.shC[which][j];
        const uint32_t path = (uint32_t)__float_as_int(o.w);
        uint32_t pixel, sample;
        pathPixelSample(fp, path, pixel, sample);
        const AlphaTest at = makeAlpha(s, seed, pixel, sample, (uint32_t)depth, c.w);
        HitRec h;
        const bool occluded =
            traceScene<true, WIDE>(s, f3of4(o), f3of4(d), OPT_SCENE_EPSILON, d.w, h, at, ctr);
        countFault(h.leaf, q.totals);
        resolveShadow(q, path, c, occluded);
    }
    if constexpr (COUNT)
        flushCounts(ctr, q.totals, 6);
}

// ------------------------------------------------------------------ finish: the tail of a pass
// Past the first bounces most paths have left the scene: the queues are
// short, and each per-bounce launch lasts as long as its slowest rays' chain
// of dependent node fetches while most of the GPU idles. From bounce depth0
// on, kFinish takes each remaining path and runs all its further bounces
// itself -- closest hit, shading (shadeRay), the point-light and emissive
// shadow rays, continuation -- with the same functions, in the same order,
// as the per-bounce kernels, so the image is bit-identical to the all-
// wavefront pass. Persistent warps take their first 32 paths in queue order
// and then refill idle lanes from the queue in batches (one atomic per
// refill). The rays traced are added to the per-bounce queue counters, so
// ray totals and per-bounce counts stay exact. Plain sampling only (guided
// shading needs the batched inference between extension and shading).
template <bool COUNT, bool WIDE>
__global__ void __launch_bounds__(128, 4) kFinish(DevScene s, FrameParams fp, WaveBufs q, int depth0)
{
    const uint32_t count = q.counters[CNT_EXT + depth0];
    const int cur = depth0 & 1;
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned below = (1u << lane) - 1u;
    const uint32_t firstRound = (gridDim.x * blockDim.x) & ~31u;
    const ShadeConsts k = shadeConsts(fp, false);
    typename std::conditional<COUNT, Count, NoCount>::type cExt, cSh;
    bool started = false, exhausted = false;
    int depth = 0;  // this lane's bounce; 0 = idle
    float4 ro = make_float4(0.0f, 0.0f, 0.0f, 0.0f), rd = ro;
    while (true) {
        const bool need = depth == 0 && !exhausted;
        const unsigned nm = __ballot_sync(0xffffffffu, need);
        if (nm && (!started || __popc(nm) >= TRAV8_REFILL || __ballot_sync(0xffffffffu, depth != 0) == 0u)) {
            uint32_t base;
            if (!started) {
                base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;  // this warp's first 32
                started = true;
            } else {
                const int leader = __ffs(nm) - 1;
                base = 0;
                if ((int)lane == leader)
                    base = atomicAdd(q.counters + CNT_FETCH_EXT + depth0, (uint32_t)__popc(nm));
                base = __shfl_sync(0xffffffffu, base, leader) + firstRound;
            }
            if (need) {
                const uint32_t i = base + (uint32_t)__popc(nm & below);
                if (i < count) {
                    ro = q.rayO[cur][i];
                    rd = q.rayD[cur][i];
                    depth = depth0;
                } else {
                    exhausted = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, depth != 0) == 0u)
            break;
        const int d = depth;
        bool wantP = false, wantE = false;
        if (depth != 0) {
            // closest hit (tmin 0, tmax 1e16, cu/device_programs.cu:63)
            const uint32_t path = (uint32_t)__float_as_int(ro.w);
            uint32_t pixel, sample;
            pathPixelSample(fp, path, pixel, sample);
            HitRec h;
            traceScene<false, WIDE>(s, f3of4(ro), f3of4(rd), 0.0f, 1e16f, h,
                                    makeAlpha(s, k.seed, pixel, sample, (uint32_t)depth, -1.0f), cExt);
            countFault(h.leaf, q.totals);
            const float4 hrec = h.leaf >= 0 ? make_float4(h.t, h.u, h.v, __int_as_float(h.leaf))
                                            : make_float4(__int_as_float(0x7f800000), 0.0f, 0.0f,
                                                          __int_as_float(-1));
            bool cont = false;
            float4 nxt[2], shP[3], shE[3];
            shadeRay<false>(s, fp, q, depth, 0u, k, ro, rd, hrec, cont, nxt, wantP, shP, wantE, shE);
            // the shadow rays, point light first (the per-bounce kernels'
            // launch order), each adding to the path's radiance
            for (int which = 0; which < 2; ++which) {
                if (!(which == 0 ? wantP : wantE))
                    continue;
                const float4 so = which == 0 ? shP[0] : shE[0], sd = which == 0 ? shP[1] : shE[1],
                             sc = which == 0 ? shP[2] : shE[2];
                HitRec hs;
                const bool occluded = traceScene<true, WIDE>(
                    s, f3of4(so), f3of4(sd), OPT_SCENE_EPSILON, sd.w, hs,
                    makeAlpha(s, k.seed, pixel, sample, (uint32_t)depth, sc.w), cSh);
                countFault(hs.leaf, q.totals);
                resolveShadow(q, path, sc, occluded);
            }
            if (cont) {
                ro = nxt[0];
                rd = nxt[1];
                ++depth;
            } else {
                depth = 0;
            }
        }
        // Per-bounce ray counts, one atomic per bounce present in the warp
        // (bounce depth0's extension rays are already counted by its queue).
        const int keys[3] = {d > depth0 ? d : 0, wantP ? d : 0, wantE ? d : 0};
        const int bases[3] = {CNT_EXT, CNT_SHADOW_P, CNT_SHADOW_E};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const unsigned peers = __match_any_sync(0xffffffffu, keys[c]);
            if (keys[c] != 0 && (peers & below) == 0u)
                atomicAdd(q.counters + bases[c] + keys[c], (uint32_t)__popc(peers));
        }
    }
    if constexpr (COUNT) {
        flushCounts(cExt, q.totals, 4);
        flushCounts(cSh, q.totals, 6);
    }
}

// ------------------------------------------------------------------ accumulate
// FP64 progressive accumulation, then tone mapping and gamma
// (cu/device_programs.cu:67-101, include/tone_mapping.h:5-29,
// include/gamma_correction.h:3-7). A NaN sample contributes the running mean,
// which is what the reference's lerp does when it skips the write.
__global__ void __launch_bounds__(256) kAccumulate(FrameParams fp, WaveBufs q, AccumBufs a)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t samplesBefore = __ldg(fp.state);
    const int toneFlags = __float_as_int(__ldg(&fp.fc->V).w);
    const float gammaTerm = __ldg(&fp.fc->W).w;
    uint32_t nanLocal = 0;
    const uint32_t active = fp.batch.on ? __ldg(fp.batch.dyn) : fp.npix;
    const uint32_t perPixel = fp.batch.on ? __ldg(fp.batch.dyn + 1) : fp.sppBatch;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < active; i += stride) {
        uint32_t px = i, n = samplesBefore;
        if (fp.batch.on) {  // active pixel i of the batch: its global pixel and view's sample count
            px = __ldg(fp.batch.pixelList + i);
            n = __float_as_uint(__ldg(&fp.batch.views[__ldg(fp.batch.pixelView + px)].W).w);
        }
        Acc4 S = a.sum[px], Q = a.sumSq[px];
        for (uint32_t b = 0; b < perPixel; ++b) {
            const float4 Lf = q.pathL[b * active + i];
            double lx, ly, lz;
            if (isnan(Lf.x) || isnan(Lf.y) || isnan(Lf.z)) {
                ++nanLocal;
                lx = n ? S.x / n : 0.0;
                ly = n ? S.y / n : 0.0;
                lz = n ? S.z / n : 0.0;
            } else {
                lx = Lf.x;
                ly = Lf.y;
                lz = Lf.z;
            }
            S.x += lx; S.y += ly; S.z += lz;
            Q.x += lx * lx; Q.y += ly * ly; Q.z += lz * lz;
            ++n;
        }
        a.sum[px] = S;
        a.sumSq[px] = Q;
        const double inv = 1.0 / (double)n;
        float4 c = make_float4((float)(S.x * inv), (float)(S.y * inv), (float)(S.z * inv), 0.0f);
        a.accumFrameBuffer[px] = c;
        if (toneFlags & 1) {
            if (!(toneFlags & 2)) {
                c = make_float4(c.x / (c.x + 1.0f), c.y / (c.y + 1.0f), c.z / (c.z + 1.0f), c.w / (c.w + 1.0f));
            } else {
                auto aces = [](float x) {
                    const float t = (x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f);
                    return fmaxf(0.0f, fminf(t, 1.0f));
                };
                c = make_float4(aces(c.x), aces(c.y), aces(c.z), aces(c.w));
            }
        }
        if (toneFlags & 4) {
            const float ig = 1.0f / gammaTerm;
            c = make_float4(powf(c.x, ig), powf(c.y, ig), powf(c.z, ig), c.w);
        }
        a.frameBuffer[px] = c;
    }
    // Per-frame statistics: NaN samples, and the ray counts of every queue.
    for (int off = 16; off > 0; off >>= 1)
        nanLocal += __shfl_down_sync(0xffffffffu, nanLocal, off);
    if ((threadIdx.x & 31) == 0 && nanLocal)
        atomicAdd(q.totals + 3, (unsigned long long)nanLocal);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        unsigned long long ext = 0, sh = 0;
        for (uint32_t d = 1; d <= fp.maxDepth; ++d) {
            ext += q.counters[CNT_EXT + d];
            sh += q.counters[CNT_SHADOW_P + d] + q.counters[CNT_SHADOW_E + d];
        }
        q.totals[0] += ext;
        q.totals[1] += sh;
        q.totals[2] += (unsigned long long)active * perPixel;
    }
}

// Advances the sample counter after a pass (one thread).
// state[0]: samples accumulated (reset with the accumulator); state[1]: passes
// run by this renderer (never reset; stamps guiding records).
// The pipelined frame loop's device snapshot of the frame buffer, by the
// SMs at HBM speed (it sits between two frames' passes on the stream).
__global__ void kCopyFrame(const float4 *__restrict__ src, float4 *__restrict__ dst, size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = __ldcs(src + i);
}

__global__ void kAdvance(uint32_t *state, uint32_t by)
{
    state[0] += by;
    state[1] += 1u;
}

// ------------------------------------------------------------------ parity entry points
__global__ void kTrace(DevScene s, const float4 *rays, float4 *hits, uint32_t n, int anyHit,
                       unsigned long long *totals)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float4 o = rays[2 * i], d = rays[2 * i + 1];
    const AlphaTest at = makeAlpha(s, 0u, 0u, 0u, 0u, anyHit ? 0.5f : -1.0f);
    HitRec h;
    NoCount ctr;
    bool hit;
    if (s.nodes8)
        hit = anyHit ? traceScene<true, true>(s, f3of4(o), f3of4(d), o.w, d.w, h, at, ctr)
                     : traceScene<false, true>(s, f3of4(o), f3of4(d), o.w, d.w, h, at, ctr);
    else
        hit = anyHit ? traceScene<true, false>(s, f3of4(o), f3of4(d), o.w, d.w, h, at, ctr)
                     : traceScene<false, false>(s, f3of4(o), f3of4(d), o.w, d.w, h, at, ctr);
    countFault(h.leaf, totals);
    const int prim = hit ? __float_as_int(__ldg(&s.triV[3 * h.leaf]).w) : -1;
    hits[i] = hit ? make_float4(h.t, h.u, h.v, __int_as_float(prim))
                  : make_float4(__int_as_float(0x7f800000), 0.0f, 0.0f, __int_as_float(-1));
}

// Layouts of optpt_bsdf_query / optpt_bsdf_result (include/optpt.h).
struct BsdfQueryD {
    float baseColour[3], emission[3], sheenColour[3];
    float metallic, roughness, specular, transmissionWeight, subsurfaceWeight, coatWeight, coatRoughness,
        sheenRoughnessMat, sheenRoughness, ior;
    uint32_t category;
    float n[3], wo[3], wi[3], xs[12];
};
struct BsdfResultD {
    uint32_t category;
    int32_t ret, used;
    float categoryWeight;
    float f[3], dir[3], bsdf[3];
    float pdf;
};
struct XsSource {
    const float *xs;
    int used;
    OPT_D float next()
    {
        const float x = used < 12 ? xs[used] : 0.5f;
        ++used;
        return x;
    }
};

__global__ void kBsdfBatch(const BsdfQueryD *qs, BsdfResultD *rs, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const BsdfQueryD &Q = qs[i];
    XsSource U{Q.xs, 0};
    const float3 nn = mk3(Q.n[0], Q.n[1], Q.n[2]), wo = mk3(Q.wo[0], Q.wo[1], Q.wo[2]),
                 wi = mk3(Q.wi[0], Q.wi[1], Q.wi[2]);
    const float3 albedo = mk3(Q.baseColour[0], Q.baseColour[1], Q.baseColour[2]);
    const float3 sheen = mk3(Q.sheenColour[0], Q.sheenColour[1], Q.sheenColour[2]);
    const bsdf::CatIn ci{Q.category, Q.coatWeight, Q.coatRoughness, Q.transmissionWeight, Q.specular,
                         Q.subsurfaceWeight};
    float cw;
    const uint32_t cat = bsdf::categorise(ci, wo, nn, Q.roughness, Q.metallic,
                                          mk3(Q.emission[0], Q.emission[1], Q.emission[2]), sheen, Q.sheenRoughness,
                                          U, cw);
    BsdfResultD R;
    R.category = cat;
    R.categoryWeight = cw;
    if (cat & MF_EMISSION) {
        for (int k = 0; k < 3; ++k)
            R.f[k] = R.dir[k] = R.bsdf[k] = 0.0f;
        R.pdf = 0.0f;
        R.ret = 0;
        R.used = U.used;
        rs[i] = R;
        return;
    }
    const bsdf::MatMR m = bsdf::makeMatMR(albedo, Q.ior, Q.metallic, sheen, cat, nn, Q.roughness, Q.coatRoughness,
                                          Q.sheenRoughnessMat);
    const float3 f = bsdf::evalBrdf(m, wi, wo, U);
    float3 xi;
    xi.x = U.next();
    xi.y = U.next();
    xi.z = U.next();
    bsdf::Sample smp;
    smp.dir = mk3s(0.0f);
    smp.bsdf = mk3s(0.0f);
    smp.pdf = 0.0f;
    const bool ok = bsdf::sampleBrdf(m, wo, xi, U, smp);
    smp.pdf *= cw;
    R.f[0] = f.x; R.f[1] = f.y; R.f[2] = f.z;
    R.dir[0] = smp.dir.x; R.dir[1] = smp.dir.y; R.dir[2] = smp.dir.z;
    R.bsdf[0] = smp.bsdf.x; R.bsdf[1] = smp.bsdf.y; R.bsdf[2] = smp.bsdf.z;
    R.pdf = smp.pdf;
    R.ret = ok ? 1 : 0;
    R.used = U.used;
    rs[i] = R;
}

}  // namespace

// ------------------------------------------------------------------ launchers
void launchGenerate(const LaunchShape &ls, const FrameParams &fp, const WaveBufs &q, cudaStream_t st)
{
    kGenerate<<<ls.gridGenerate, ls.block, 0, st>>>(fp, q);
}
void launchExtend(const LaunchShape &ls, const DevScene &s, const FrameParams &fp, const WaveBufs &q, int depth,
                  cudaStream_t st, bool count)
{
    const bool wide = s.nodes8 != nullptr;
    if (count)
        (wide ? kExtend<true, true> : kExtend<true, false>)<<<ls.gridExtend, ls.block, 0, st>>>(s, fp, q, depth);
    else
        (wide ? kExtend<false, true> : kExtend<false, false>)<<<ls.gridExtend, ls.block, 0, st>>>(s, fp, q, depth);
}
void launchShade(const LaunchShape &ls, const DevScene &s, const FrameParams &fp, const WaveBufs &q, int depth,
                 cudaStream_t st)
{
    const bool blockPush = ls.compaction == 1;
    if (fp.guide.on && blockPush)
        kShade<true, true><<<ls.gridShade, ls.block, 0, st>>>(s, fp, q, depth);
    else if (fp.guide.on)
        kShade<true, false><<<ls.gridShade, ls.block, 0, st>>>(s, fp, q, depth);
    else if (blockPush)
        kShade<false, true><<<ls.gridShade, ls.block, 0, st>>>(s, fp, q, depth);
    else
        kShade<false, false><<<ls.gridShade, ls.block, 0, st>>>(s, fp, q, depth);
}
void launchShadow(const LaunchShape &ls, const DevScene &s, const FrameParams &fp, const WaveBufs &q, int depth,
                  int which, cudaStream_t st, bool count)
{
    const bool wide = s.nodes8 != nullptr;
    if (count)
        (wide ? kShadow<true, true> : kShadow<true, false>)<<<ls.gridShadow, ls.block, 0, st>>>(s, fp, q, depth,
                                                                                               which);
    else
        (wide ? kShadow<false, true> : kShadow<false, false>)<<<ls.gridShadow, ls.block, 0, st>>>(s, fp, q, depth,
                                                                                                 which);
}
void launchFinish(const LaunchShape &ls, const DevScene &s, const FrameParams &fp, const WaveBufs &q, int depth0,
                  cudaStream_t st, bool count)
{
    const bool wide = s.nodes8 != nullptr;
    if (count)
        (wide ? kFinish<true, true> : kFinish<true, false>)<<<ls.gridFinish, 128, 0, st>>>(s, fp, q, depth0);
    else
        (wide ? kFinish<false, true> : kFinish<false, false>)<<<ls.gridFinish, 128, 0, st>>>(s, fp, q, depth0);
}
void launchAccumulate(const LaunchShape &ls, const FrameParams &fp, const WaveBufs &q, const AccumBufs &a,
                      cudaStream_t st)
{
    kAccumulate<<<ls.gridAccum, ls.block, 0, st>>>(fp, q, a);
}
void launchCopyFrame(const float4 *src, float4 *dst, size_t n, cudaStream_t st)
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t blocks = (n + 255) / 256, cap = (size_t)sms * 8;
    kCopyFrame<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, st>>>(src, dst, n);
}
void launchAdvance(const FrameParams &fp, uint32_t *state, cudaStream_t st)
{
    kAdvance<<<1, 1, 0, st>>>(state, fp.sppBatch);
}
void launchTrace(const DevScene &s, const float4 *rays, float4 *hits, uint32_t n, int anyHit,
                 unsigned long long *totals, cudaStream_t st)
{
    if (n == 0)
        return;
    kTrace<<<(n + 127) / 128, 128, 0, st>>>(s, rays, hits, n, anyHit, totals);
}
void launchBsdfBatch(const void *queries, void *results, uint32_t n, cudaStream_t st)
{
    if (n == 0)
        return;
    kBsdfBatch<<<(n + 127) / 128, 128, 0, st>>>(static_cast<const BsdfQueryD *>(queries),
                                                 static_cast<BsdfResultD *>(results), n);
}

int occupancyGrid(int kernelId, int block)
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const void *fn = nullptr;
    switch (kernelId) {
    case 0: fn = (const void *)kGenerate; break;
    case 1: fn = (const void *)kExtend<false, true>; break;
    case 2: fn = (const void *)kShade<false, false>; break;
    case 3: fn = (const void *)kShadow<false, true>; break;
    case 11: fn = (const void *)kExtend<false, false>; break;
    case 13: fn = (const void *)kShadow<false, false>; break;
    case 5: fn = (const void *)kFinish<false, true>; break;
    case 15: fn = (const void *)kFinish<false, false>; break;
    default: fn = (const void *)kAccumulate; break;
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, 0);
    if (per < 1)
        per = 1;
    return sms * per;
}

// sRGB decode table, IEC 61966-2-1.
int uploadSrgbTable()
{
    float t[256];
    for (int i = 0; i < 256; ++i) {
        double c = i / 255.0;
        t[i] = (float)(c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4));
    }
    return (int)cudaMemcpyToSymbol(c_srgbToLinear, t, sizeof(t));
}
