// Learned path guiding: the hash-grid encoded MLP on the fifth-generation
// tensor cores (tcgen05 MMAs from shared memory into TMEM), its fused
// training kernel (forward, loss gradient, backward, weight gradients) and
// the Adam optimiser. Device math shared with shading is in guide.cuh.
//
// Network: inputs (64) = 16 levels x 2 hash-grid features, shading normal,
// outgoing direction, a constant 1 (bias), zero padding; four hidden layers
// of 64 ReLU units; 40 outputs = 8 vMF lobes (mu xyz, log kappa, weight
// logit). No biases besides the constant input. BF16 operands, FP32
// accumulation; FP32 master weights.
//
// A CTA is 4 warps, one sample per thread, 128 samples per tile. Weight
// tiles reach shared memory by bulk TMA copies (cp.async.bulk); one thread
// issues the MMAs; everybody waits on an mbarrier (bounded) and reads its
// row of the accumulator with tcgen05.ld.
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>
#include "optpt.h"
#include "tc.cuh"
#include "guide_net.h"
#include "engine.h"

extern "C" int optpt_internal_set_error(int code, const char *msg);

using namespace guide;

namespace {

constexpr int TILE_ROWS = 128;
constexpr uint32_t TILE_BYTES = TILE_ROWS * WIDTH * 2;  // 16 KB activations
constexpr uint32_t W_BYTES = WIDTH * WIDTH * 2;         // 8 KB weights
constexpr uint32_t IDESC_FWD = tc::idescBf16(128, 64, false, false);
constexpr uint32_t IDESC_DW = tc::idescBf16(64, 64, true, true);

__device__ __forceinline__ void bulkLoad(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     tc::smemAddr(dst)),
                 "l"(src), "r"(bytes), "r"(tc::smemAddr(bar))
                 : "memory");
}
__device__ __forceinline__ void expectTx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smemAddr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ float loadBf16(const uint8_t *tile, uint32_t row, uint32_t col)
{
    return __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(tile + tc::tileOffset(row, col)));
}
// 8 consecutive columns (one 16-byte core-matrix row) at once.
__device__ __forceinline__ void storeRow8(uint8_t *tile, uint32_t row, uint32_t col8, const float *v)
{
    __align__(16) __nv_bfloat16 h[8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        h[k] = __float2bfloat16_rn(v[k]);
    *reinterpret_cast<uint4 *>(tile + tc::tileOffset(row, col8)) = *reinterpret_cast<const uint4 *>(h);
}

__device__ __forceinline__ float3 unitPos(const GuideGeom &g, float3 p)
{
    const float one = 0.99999994f;
    return mk3(fminf(fmaxf((p.x - g.lo.x) * g.invExt.x, 0.0f), one),
               fminf(fmaxf((p.y - g.lo.y) * g.invExt.y, 0.0f), one),
               fminf(fmaxf((p.z - g.lo.z) * g.invExt.z, 0.0f), one));
}

// Input row: hash features (FP32 table for training; for inference the FP16
// pair copy, whose slot e holds entry e's features followed by entry e + 1's).
// Each level's two features go straight to shared memory (one 32-bit store),
// so the level loop stays rolled: a fully unrolled 16 x 8 gather loop costs
// more in instruction fetch than it saves.
template <bool HALF>
__device__ void encodeRow(const GuideGeom &g, const float *hash, const __half *hashH, float3 pos, float3 n, float3 wo,
                          bool valid, uint8_t *tile, uint32_t row)
{
    if (valid) {
        const float3 p = unitPos(g, pos);
        // four levels at a time: their 32 gathers are issued before any is
        // used; only the raw features and each level's fractions live across
        // the gathers (the corner weights are formed as they are consumed)
        using Raw = typename std::conditional<HALF, __half2, float2>::type;
#pragma unroll 1
        for (int l0 = 0; l0 < LEVELS; l0 += 4) {
            float t[4][3];
            Raw v[4][8];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                uint32_t e[8];
                levelCell(g.levels, l0 + j, p.x, p.y, p.z, e, t[j][0], t[j][1], t[j][2]);
                if constexpr (HALF) {
                    // pair copy: entry e's features, then entry e + 1's
                    // (corner c + 1 is corner c's x-neighbour)
#pragma unroll
                    for (int c = 0; c < 8; c += 2) {
                        const uint2 pr =
                            __ldg(reinterpret_cast<const uint2 *>(hashH) + ((size_t)(l0 + j) * TABLE + e[c]));
                        v[j][c] = *reinterpret_cast<const __half2 *>(&pr.x);
                        v[j][c + 1] = *reinterpret_cast<const __half2 *>(&pr.y);
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 8; ++c)
                        v[j][c] = __ldg(reinterpret_cast<const float2 *>(hash + ((size_t)(l0 + j) * TABLE + e[c]) * FEATS));
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const float w = cornerWeight(c, t[j][0], t[j][1], t[j][2]);
                    float2 f;
                    if constexpr (HALF)
                        f = __half22float2(v[j][c]);
                    else
                        f = v[j][c];
                    f0 += w * f.x;
                    f1 += w * f.y;
                }
                *reinterpret_cast<__nv_bfloat162 *>(tile + tc::tileOffset(row, 2 * (l0 + j))) =
                    __floats2bfloat162_rn(f0, f1);
            }
        }
    } else {
#pragma unroll
        for (int c8 = 0; c8 < IN_NORMAL; c8 += 8)
            *reinterpret_cast<uint4 *>(tile + tc::tileOffset(row, c8)) = make_uint4(0, 0, 0, 0);
    }
    float in[WIDTH - IN_NORMAL];
#pragma unroll
    for (int c = 0; c < WIDTH - IN_NORMAL; ++c)
        in[c] = 0.0f;
    if (valid) {
        in[0] = n.x;
        in[1] = n.y;
        in[2] = n.z;
        in[IN_WO - IN_NORMAL] = wo.x;
        in[IN_WO - IN_NORMAL + 1] = wo.y;
        in[IN_WO - IN_NORMAL + 2] = wo.z;
        in[IN_ONE - IN_NORMAL] = 1.0f;
    }
#pragma unroll
    for (int c8 = IN_NORMAL; c8 < WIDTH; c8 += 8)
        storeRow8(tile, row, c8, in + c8 - IN_NORMAL);
}

struct Sync {
    uint64_t *bar;
    uint32_t phase;
    // all threads: shared-memory writes -> visible to the tensor core, and
    // previous TMEM reads finished before the next MMA overwrites them
    __device__ void toTensor()
    {
        tc::fenceProxyAsync();
        tc::fenceBeforeSync();
        __syncthreads();
        tc::fenceAfterSync();
    }
    // all threads: wait for the MMAs committed last; false on expiry (agreed)
    __device__ bool wait()
    {
        const bool ok = tc::mbarWait(bar, phase);
        phase ^= 1u;
        tc::fenceAfterSync();
        return __syncthreads_and(ok ? 1 : 0) != 0;
    }
};

// The same for one 128-thread group of a larger CTA, on named barrier `id`.
struct GroupSync {
    uint64_t *bar;
    uint32_t phase;
    int id;
    __device__ void toTensor()
    {
        tc::fenceProxyAsync();
        tc::fenceBeforeSync();
        asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory");
        tc::fenceAfterSync();
    }
    __device__ bool wait()
    {
        const bool ok = tc::mbarWait(bar, phase);
        phase ^= 1u;
        tc::fenceAfterSync();
        uint32_t all;
        asm volatile(
            "{\n\t.reg .pred q, o;\n\t"
            "setp.ne.u32 q, %1, 0;\n\t"
            "bar.red.and.pred o, %2, 128, q;\n\t"
            "selp.u32 %0, 1, 0, o;\n\t}"
            : "=r"(all)
            : "r"(ok ? 1u : 0u), "r"(id)
            : "memory");
        return all != 0;
    }
};

// This thread's row (64 FP32 columns from col0) of a 128-lane accumulator.
__device__ __forceinline__ void loadRow(uint32_t tmem, uint32_t col0, float (&v)[WIDTH])
{
    const uint32_t lane = (uint32_t)(32 * ((threadIdx.x >> 5) & 3)) << 16;  // the warp's lane quarter
    tc::ld64(tmem + lane + col0, v);
}

// Issues D = X W^T for one 128 x 64 x 64 layer (thread 0 only).
__device__ __forceinline__ void issueLayer(uint32_t dTmem, const uint8_t *x, const uint8_t *w)
{
    const uint32_t xa = tc::smemAddr(x), wa = tc::smemAddr(w);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        tc::mma(dTmem, tc::smemDesc(xa + 256 * k, 128, 1024), tc::smemDesc(wa + 256 * k, 128, 1024), IDESC_FWD,
                k > 0);
}

// ------------------------------------------------------------------ inference
struct QueryInput {
    const GuideQuery *q;
    uint32_t n;
    __device__ bool fetch(uint32_t i, float3 &p, float3 &nrm, float3 &wo) const
    {
        if (i >= n)
            return false;
        const GuideQuery r = q[i];
        p = f3of4(r.pos);
        nrm = f3of4(r.n);
        wo = f3of4(r.wo);
        return true;
    }
    __device__ uint32_t count() const { return n; }
    __device__ void resolve() {}
};

// Hits of the extension queue at one depth: position, face-forwarded
// geometric normal and outgoing direction (the same inputs the shading
// kernel records for training).
struct HitInput {
    const float4 *rayO, *rayD, *hit, *triV;
    const uint32_t *countPtr;
    uint32_t n;
    const uint32_t *limitPtr;  // if set, at most *limitPtr queries (else `limit`, if non-zero)
    uint32_t limit;
    __device__ bool fetch(uint32_t i, float3 &p, float3 &nrm, float3 &wo) const
    {
        if (i >= n)
            return false;
        const float4 h = hit[i];
        const int leaf = __float_as_int(h.w);
        if (leaf < 0)
            return false;
        const float3 o = f3of4(rayO[i]), d = f3of4(rayD[i]);
        p = o + h.x * d;
        const float3 v0 = f3of4(__ldg(&triV[3 * leaf])), v1 = f3of4(__ldg(&triV[3 * leaf + 1])),
                     v2 = f3of4(__ldg(&triV[3 * leaf + 2]));
        const float3 Ng = normalize3(cross3(v1 - v0, v2 - v0));
        nrm = dot3(Ng, d) < 0.0f ? Ng : -Ng;
        wo = -d;
        return true;
    }
    __device__ uint32_t count() const { return n; }
    __device__ void resolve()
    {
        n = *countPtr;
        const uint32_t cap = limitPtr ? *limitPtr : limit;
        if (cap && cap < n)
            n = cap;
    }
};

// Inference CTA shape: INFER_GROUPS groups of 128 threads, each with its own
// 128-row activation tile, mbarrier, 64 TMEM columns and named barrier, all
// sharing one copy of the weights; INFER_MINB CTAs resident per SM. While
// one group waits on its MMA the others gather or convert.
#ifndef OPTPT_INFER_GROUPS
#define OPTPT_INFER_GROUPS 2
#endif
#ifndef OPTPT_INFER_MINB
#define OPTPT_INFER_MINB 2
#endif
constexpr int INFER_GROUPS = OPTPT_INFER_GROUPS;
constexpr int INFER_THREADS = 128 * INFER_GROUPS;
constexpr uint32_t INFER_SMEM = LAYERS * W_BYTES + INFER_GROUPS * TILE_BYTES + 1024;
// TMEM columns per CTA: a power of two of at least 32
constexpr uint32_t INFER_TMEM = INFER_GROUPS <= 2 ? 128u : INFER_GROUPS <= 4 ? 256u : 512u;
static_assert(INFER_GROUPS >= 1 && INFER_GROUPS <= 8, "inference groups");
static_assert(INFER_TMEM * OPTPT_INFER_MINB <= 512, "TMEM columns of the resident CTAs");

template <class In>
__global__ void __launch_bounds__(INFER_THREADS, OPTPT_INFER_MINB)
    kGuideInfer(GuideGeom g, const __half *hashH, const uint8_t *tiles, In in, Packed *out, int *status)
{
    extern __shared__ uint8_t smRaw[];
    uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smRaw) + 1023) & ~uintptr_t(1023));
    const int t = threadIdx.x, grp = t >> 7, row = t & 127;
    uint8_t *sW = sm, *sX = sm + LAYERS * W_BYTES + grp * TILE_BYTES;
    __shared__ uint64_t barLoad, barMma[INFER_GROUPS];
    __shared__ uint32_t tmemBase;
    if (t == 0) {
        tc::mbarInit(&barLoad, 1);
        for (int k = 0; k < INFER_GROUPS; ++k)
            tc::mbarInit(&barMma[k], 1);
    }
    if (t < 32)
        tc::tmemAlloc(&tmemBase, INFER_TMEM);
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    if (t == 0) {
        expectTx(&barLoad, LAYERS * W_BYTES);
        for (int l = 0; l < LAYERS; ++l)
            bulkLoad(sW + l * W_BYTES, tiles + (size_t)l * W_BYTES, W_BYTES, &barLoad);
    }
    const uint32_t tm = tmemBase + 64u * (uint32_t)grp;
    bool ok = __syncthreads_and(tc::mbarWait(&barLoad, 0) ? 1 : 0) != 0;
    GroupSync sync{&barMma[grp], 0, 1 + grp};
    in.resolve();
    const uint32_t n = in.count();
    const uint32_t lane = (uint32_t)(32 * ((t >> 5) & 3)) << 16;  // the warp's TMEM lane quarter
    for (uint32_t base = (blockIdx.x * INFER_GROUPS + grp) * TILE_ROWS; ok && base < n;
         base += gridDim.x * INFER_GROUPS * TILE_ROWS) {
        float3 p, nrm, wo;
        const bool valid = in.fetch(base + row, p, nrm, wo);
        encodeRow<true>(g, nullptr, hashH, p, nrm, wo, valid, sX, row);
        for (int l = 0; l < LAYERS - 1 && ok; ++l) {
            sync.toTensor();
            if (row == 0) {
                issueLayer(tm, sX, sW + l * W_BYTES);
                tc::commit(&barMma[grp]);
            }
            ok = sync.wait();
            if (!ok)
                break;
            // hidden layer: ReLU, back to the activation tile in two
            // 32-column halves (the MMA reading sX has completed)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float v[32];
                tc::ld32(tm + lane + 32u * h, v);
#pragma unroll
                for (int c8 = 0; c8 < 32; c8 += 8) {
                    float r[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        r[k] = fmaxf(v[c8 + k], 0.0f);
                    storeRow8(sX, row, 32 * h + c8, r);
                }
            }
        }
        if (ok) {
            sync.toTensor();
            if (row == 0) {
                issueLayer(tm, sX, sW + (LAYERS - 1) * W_BYTES);
                tc::commit(&barMma[grp]);
            }
            ok = sync.wait();
        }
        // the 41 outputs: columns 0-31, then 32-47. tcgen05.ld is a
        // warp-collective (.sync.aligned) instruction: every lane of the warp
        // loads, valid row or not, and only the decoding depends on the row.
        float o[48];
        if (ok) {
            float lo[32], hi[16];
            tc::ld32(tm + lane, lo);
            tc::ld16(tm + lane + 32u, hi);
#pragma unroll
            for (int k = 0; k < 48; ++k)
                o[k] = k < 32 ? lo[k] : hi[k - 32];
        }
        if (ok && valid) {
            Mixture m;
            decodeOutputs(o, m);
            Packed pk;
            pack(m, pk);
            out[base + row] = pk;
        } else if (ok && base + row < n) {
            // no hit: a null mixture (zero weights, zero selection), so a
            // vertex that reads this row (a shared primary mixture) samples
            // the BSDF alone
            out[base + row] = Packed{};
        }
    }
    if (!ok && row == 0)
        atomicExch(status, 1);
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    if (t < 32)
        tc::tmemFree(tmemBase, INFER_TMEM);
}

// The shading kernel's mixture sampler and density on given rows.
__global__ void kMixtureEval(const Packed *mix, uint32_t n, const float *xi, float4 *dirPdf)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Packed p = mix[i];
        const float3 d = xi ? mixtureSample(p, xi[3 * i], 1.0f - xi[3 * i + 1], xi[3 * i + 2]) : f3of4(dirPdf[i]);
        dirPdf[i] = make_float4(d.x, d.y, d.z, mixturePdf(p, d));
    }
}

// ------------------------------------------------------------------ training
// Gradient w.r.t. the 41 raw outputs of -c log(a q(wi) + (1 - a) pb), the
// density of the one-sample MIS proposal the renderer samples from (a = the
// selection probability, pb = the BSDF lobe's density at wi); c pre-normalised.
// Lobe gradients are those of -c log q scaled by beta = a q / (a q + (1-a) pb)
// (or unscaled, wholeTarget: the lobes then fit the whole target).
__device__ void lossGradient(const float *o, float3 wi, float pb, float c, bool wholeTarget, float *d, float &loss)
{
    Mixture m;
    decodeOutputs(o, m);
    float v[LOBES], q = 0.0f;
#pragma unroll
    for (int k = 0; k < LOBES; ++k) {
        v[k] = vmfPdf(m.lobe[k], wi);
        q += m.lobe[k].weight * v[k];
    }
    q = fmaxf(q, 1e-30f);
    const float a = m.select;
    const float mix = fmaxf(a * q + (1.0f - a) * pb, 1e-30f);
    loss = -c * logf(mix);
    const float sg = (a - SELECT_MIN) / SELECT_SPAN;  // sigmoid(logit)
    d[OUT_SELECT] = -c * (q - pb) / mix * SELECT_SPAN * sg * (1.0f - sg);
    if (!wholeTarget)
        c *= a * q / mix;  // else the lobes fit the whole target (-c log q)
#pragma unroll
    for (int k = 0; k < LOBES; ++k) {
        const Lobe &L = m.lobe[k];
        const float r = L.weight * v[k] / q;  // responsibility
        d[5 * k + 4] = c * (L.weight - r);
        const float lk = o[5 * k + 3];
        const float kap = L.kappa;
        const float tdot = dot3(L.mu, wi);
        // d log v / d kappa = 1/kappa - 2/(exp(2 kappa) - 1) + (t - 1)
        const float dlogC = kap < 1e-3f ? (2.0f / 3.0f) * kap : 1.0f / kap - 2.0f / expm1f(2.0f * kap);
        const float dk = -c * r * (dlogC + tdot - 1.0f);
        d[5 * k + 3] = (lk > LOG_KAPPA_MIN && lk < LOG_KAPPA_MAX) ? dk * kap : 0.0f;
        const float3 raw = mk3(o[5 * k], o[5 * k + 1], o[5 * k + 2]);
        const float len = sqrtf(dot3(raw, raw));
        float3 dm = mk3(0.0f, 0.0f, 0.0f);
        if (len > 1e-12f) {
            const float3 dmu = (-c * r * kap) * wi;
            dm = (dmu - dot3(dmu, L.mu) * L.mu) * (1.0f / len);
        }
        d[5 * k] = dm.x;
        d[5 * k + 1] = dm.y;
        d[5 * k + 2] = dm.z;
    }
}

constexpr double WEIGHT_CAP = 16.0;
constexpr uint32_t TRAIN_SMEM = 2 * LAYERS * W_BYTES + LAYERS * TILE_BYTES + TILE_BYTES + 1024;
constexpr uint32_t TRAIN_TMEM = 512;  // [0, 64) layer results; [64 + 64 l, 128 + 64 l) dW_l

__global__ void __launch_bounds__(128, 1)
    kGuideTrain(GuideGeom g, const float *hash, const uint8_t *tiles, const GuideSample *smp, const uint32_t *countPtr,
                uint32_t capacity, uint32_t slice, uint32_t slices, const double *stats, float *gMlp, float *gHash,
                double *lossOut, int *status)
{
    extern __shared__ uint8_t smRaw[];
    uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smRaw) + 1023) & ~uintptr_t(1023));
    uint8_t *sW = sm;                              // W_0..W_4, then W_0^T..W_4^T
    uint8_t *sX = sm + 2 * LAYERS * W_BYTES;       // X_0..X_4
    uint8_t *sD = sX + LAYERS * TILE_BYTES;        // dZ of the current layer
    __shared__ uint64_t barLoad, barMma;
    __shared__ uint32_t tmemBase;
    const int t = threadIdx.x;
    if (t == 0) {
        tc::mbarInit(&barLoad, 1);
        tc::mbarInit(&barMma, 1);
    }
    if (t < 32)
        tc::tmemAlloc(&tmemBase, TRAIN_TMEM);
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    if (t == 0) {
        expectTx(&barLoad, 2 * LAYERS * W_BYTES);
        for (int l = 0; l < 2 * LAYERS; ++l)
            bulkLoad(sW + l * W_BYTES, tiles + (size_t)l * W_BYTES, W_BYTES, &barLoad);
    }
    const uint32_t tm = tmemBase;
    bool ok = __syncthreads_and(tc::mbarWait(&barLoad, 0) ? 1 : 0) != 0;
    Sync sync{&barMma, 0};
    const uint32_t total = min(*countPtr, capacity);
    const uint32_t b0 = (uint32_t)((uint64_t)total * slice / slices);
    const uint32_t n = (uint32_t)((uint64_t)total * (slice + 1) / slices);
    // weights are normalised by the batch sum and capped at WEIGHT_CAP times
    // the mean positive weight: single-path radiance estimates are heavy
    // tailed, and a handful of samples would otherwise steer a whole step
    const double wsum = stats[0];
    const float scale = wsum > 0.0 ? (float)(1.0 / wsum) : 0.0f;
    const float cap = stats[3] > 0.0 ? (float)(WEIGHT_CAP * wsum / stats[3]) : 0.0f;
    bool firstTile = true;
    float lossAcc = 0.0f;
    for (uint32_t base = b0 + blockIdx.x * TILE_ROWS; ok && base < n; base += gridDim.x * TILE_ROWS) {
        const uint32_t i = base + t;
        const bool valid = i < n;
        GuideSample s{};
        if (valid)
            s = smp[i];
        const float c = valid && isfinite(s.pos.w) && s.pos.w > 0.0f ? fminf(s.pos.w, cap) * scale : 0.0f;
        encodeRow<false>(g, hash, nullptr, f3of4(s.pos), f3of4(s.n), f3of4(s.wo), valid, sX, t);
        float v[WIDTH];
        // forward
        for (int l = 0; l < LAYERS && ok; ++l) {
            sync.toTensor();
            if (t == 0) {
                issueLayer(tm, sX + l * TILE_BYTES, sW + l * W_BYTES);
                tc::commit(&barMma);
            }
            ok = sync.wait();
            if (!ok)
                break;
            loadRow(tm, 0, v);
            if (l < LAYERS - 1) {
#pragma unroll
                for (int c8 = 0; c8 < WIDTH; c8 += 8) {
                    float r[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        r[k] = fmaxf(v[c8 + k], 0.0f);
                    storeRow8(sX + (l + 1) * TILE_BYTES, t, c8, r);
                }
            }
        }
        if (!ok)
            break;
        // loss gradient w.r.t. the outputs -> dZ_4
        {
            float d[WIDTH];
#pragma unroll
            for (int k = 0; k < WIDTH; ++k)
                d[k] = 0.0f;
            if (c > 0.0f) {
                float loss;
                lossGradient(v, f3of4(s.wi), fmaxf(s.wo.w, 0.0f), c, g.lobeLoss != 0, d, loss);
                lossAcc += loss;
            }
#pragma unroll
            for (int c8 = 0; c8 < WIDTH; c8 += 8)
                storeRow8(sD, t, c8, d + c8);
        }
        // backward: dW_l += dZ_l^T X_l ; dX_l = dZ_l W_l ; dZ_{l-1} = dX_l * [X_l > 0]
        for (int l = LAYERS - 1; l >= 0 && ok; --l) {
            sync.toTensor();
            if (t == 0) {
                const uint32_t da = tc::smemAddr(sD), xa = tc::smemAddr(sX + l * TILE_BYTES);
                const uint32_t dw = tm + 64u + 64u * (uint32_t)l;
#pragma unroll
                for (int k = 0; k < 8; ++k)  // K = 128 samples, 16 per MMA
                    tc::mma(dw, tc::smemDesc(da + 2048 * k, 1024, 128), tc::smemDesc(xa + 2048 * k, 1024, 128),
                            IDESC_DW, !firstTile || k > 0);
                issueLayer(tm, sD, sW + (LAYERS + l) * W_BYTES);  // dX_l = dZ_l (W_l^T)^T
                tc::commit(&barMma);
            }
            ok = sync.wait();
            if (!ok)
                break;
            loadRow(tm, 0, v);  // dX_l
            if (l > 0) {
                const uint8_t *xl = sX + l * TILE_BYTES;
#pragma unroll
                for (int c8 = 0; c8 < WIDTH; c8 += 8) {
                    float r[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        r[k] = loadBf16(xl, t, c8 + k) > 0.0f ? v[c8 + k] : 0.0f;
                    storeRow8(sD, t, c8, r);  // the MMAs reading sD have completed
                }
            } else if (c > 0.0f) {
                // hash-grid features: scatter d input into the table gradients
                // (d input parked in this thread's row of sD, which the MMAs no
                // longer read, so the level loop can stay rolled)
                float2 *dIn = reinterpret_cast<float2 *>(sD) + t * LEVELS;
#pragma unroll
                for (int lv = 0; lv < LEVELS; ++lv)
                    dIn[lv] = make_float2(v[2 * lv], v[2 * lv + 1]);
                const float3 p = unitPos(g, f3of4(s.pos));
#pragma unroll 1
                for (int lv = 0; lv < LEVELS; ++lv) {
                    const float2 dd = dIn[lv];
                    if (dd.x == 0.0f && dd.y == 0.0f)
                        continue;
#pragma unroll
                    for (int cn = 0; cn < 8; ++cn) {
                        uint32_t e;
                        float w;
                        corner(g.levels, lv, p.x, p.y, p.z, cn, e, w);
                        float2 *dst = reinterpret_cast<float2 *>(gHash + ((size_t)lv * TABLE + e) * FEATS);
                        atomicAdd(dst, make_float2(w * dd.x, w * dd.y));
                    }
                }
            }
        }
        firstTile = false;
    }
    // weight gradients: TMEM (M = 64 layout: row r in lane (r/16)*32 + r%16) -> global
    if (ok && !firstTile) {
        sync.toTensor();
        const int warp = t >> 5, lane = t & 31;
        for (int l = 0; l < LAYERS; ++l) {
            float v[WIDTH];
            loadRow(tm, 64u + 64u * (uint32_t)l, v);
            if (lane < 16) {
                const int row = warp * 16 + lane;
                float *dst = gMlp + (size_t)l * WIDTH * WIDTH + row * WIDTH;
#pragma unroll 8
                for (int k = 0; k < WIDTH; ++k)
                    atomicAdd(dst + k, v[k]);
            }
        }
    }
    // loss
    for (int off = 16; off > 0; off >>= 1)
        lossAcc += __shfl_down_sync(0xffffffffu, lossAcc, off);
    if ((t & 31) == 0 && lossAcc != 0.0f)
        atomicAdd(lossOut, (double)lossAcc);
    if (!ok && t == 0)
        atomicExch(status, 1);
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    if (t < 32)
        tc::tmemFree(tm, TRAIN_TMEM);
}

// Sum of finite positive sample weights and the sample count of the batch.
__global__ void kBatchStats(const GuideSample *smp, const uint32_t *countPtr, uint32_t capacity, uint32_t slice,
                            uint32_t slices, double *stats)
{
    const uint32_t total = min(*countPtr, capacity);
    const uint32_t b0 = (uint32_t)((uint64_t)total * slice / slices);
    const uint32_t n = (uint32_t)((uint64_t)total * (slice + 1) / slices);
    double acc = 0.0, pos = 0.0;
    for (uint32_t i = b0 + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float w = smp[i].pos.w;
        if (isfinite(w) && w > 0.0f) {
            acc += (double)w;
            pos += 1.0;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        acc += __shfl_down_sync(0xffffffffu, acc, off);
        pos += __shfl_down_sync(0xffffffffu, pos, off);
    }
    if ((threadIdx.x & 31) == 0 && acc != 0.0) {
        atomicAdd(stats, acc);
        atomicAdd(stats + 3, pos);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(stats + 2, (double)(n - b0));
}

// ------------------------------------------------------------------ training samples of a pass
// For every complete record (vertex written at depth d, arrival snapshot at
// d + 1, both in this pass): incident radiance Li = (L_final - L_arrival) /
// T_arrival; target F = luminance(f cos * Li); weight = F / density of wi.
__global__ void kGuideGather(FrameParams fp, WaveBufs q)
{
    const GuidePass gp = fp.guide;
    const uint32_t stamp = __ldg(fp.state + 1) + 1u;
    const uint32_t numPaths = passPaths(fp);
    const uint32_t numTrain = (numPaths + gp.trainStride - 1u) / gp.trainStride;
    const uint32_t total = numTrain * fp.maxDepth;
    GuideSample *batch = reinterpret_cast<GuideSample *>(gp.batch);
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const float4 *r = gp.rec + (size_t)idx * GUIDE_REC;
        const float4 r1 = r[1], r5 = r[5];
        if (__float_as_uint(r1.w) != stamp || __float_as_uint(r5.w) != stamp)
            continue;
        const uint32_t group = idx / fp.maxDepth;
        const uint32_t path = group * gp.trainStride + guideTrainOffset(group, stamp, gp.trainStride);
        if (path >= numPaths)
            continue;
        const float3 Lf = f3of4(q.pathL[path]), Ls = f3of4(r5), Ta = f3of4(r[6]), fc = f3of4(r[4]);
        const float3 dL = Lf - Ls;
        const float3 Li = mk3(Ta.x > 0.0f ? dL.x / Ta.x : 0.0f, Ta.y > 0.0f ? dL.y / Ta.y : 0.0f,
                              Ta.z > 0.0f ? dL.z / Ta.z : 0.0f);
        const float F = 0.2126f * fc.x * Li.x + 0.7152f * fc.y * Li.y + 0.0722f * fc.z * Li.z;
        const float4 r0 = r[0];
        const float w = F / r0.w;
        if (!(w > 0.0f) || !isfinite(w))
            continue;
        const uint32_t slot = atomicAdd(gp.batchCount, 1u);
        if (slot >= gp.batchCapacity)
            continue;
        GuideSample smp;
        smp.pos = make_float4(r0.x, r0.y, r0.z, w);
        smp.n = r1;
        smp.wo = r[2];
        smp.wi = r[3];
        batch[slot] = smp;
    }
}

// ------------------------------------------------------------------ Adam
constexpr float BETA1 = 0.9f, BETA2 = 0.99f, ADAM_EPS = 1e-15f;

__global__ void kAdamStep(uint32_t *step) { *step += 1u; }

__device__ __forceinline__ void biasCorrection(const uint32_t *step, float &c1, float &c2)
{
    const float t = (float)*step;
    c1 = 1.0f / (1.0f - powf(BETA1, t));
    c2 = 1.0f / (1.0f - powf(BETA2, t));
}

// Parameter i of the FP32 table into the FP16 pair copy: slot e holds
// (entry e, entry e + 1) of its level, so entry e's feature f goes to slot e
// (first half) and slot e - 1 (second half), modulo the table.
__device__ __forceinline__ void writePair(__half *ph, size_t i, __half h)
{
    const size_t f = i % FEATS, e = (i / FEATS) % TABLE, l = i / ((size_t)FEATS * TABLE);
    ph[((l * TABLE + e) * 2) * FEATS + f] = h;
    ph[((l * TABLE + ((e + TABLE - 1) & (TABLE - 1))) * 2 + 1) * FEATS + f] = h;
}

__global__ void kAdamHash(float *p, __half *ph, float *gr, float *m, float *v, size_t n, float lr, const uint32_t *step)
{
    float c1, c2;
    biasCorrection(step, c1, c2);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float g = gr[i];
        float mi = m[i], vi = v[i];
        if (g == 0.0f && mi == 0.0f)
            continue;  // never touched: nothing to move
        mi = BETA1 * mi + (1.0f - BETA1) * g;
        vi = BETA2 * vi + (1.0f - BETA2) * g * g;
        const float x = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + ADAM_EPS);
        p[i] = x;
        writePair(ph, i, __float2half_rn(x));
        m[i] = mi;
        v[i] = vi;
        gr[i] = 0.0f;
    }
}

// MLP weights: Adam, then both BF16 tile layouts.
__global__ void kAdamMlp(float *p, uint8_t *tiles, float *gr, float *m, float *v, float lr, const uint32_t *step)
{
    float c1, c2;
    biasCorrection(step, c1, c2);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MLP_PARAMS; i += gridDim.x * blockDim.x) {
        const float g = gr[i];
        const float mi = BETA1 * m[i] + (1.0f - BETA1) * g;
        const float vi = BETA2 * v[i] + (1.0f - BETA2) * g * g;
        const float x = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
        p[i] = x;
        m[i] = mi;
        v[i] = vi;
        gr[i] = 0.0f;
        const int l = i / (WIDTH * WIDTH), out = (i / WIDTH) % WIDTH, in = i % WIDTH;
        const __nv_bfloat16 b = __float2bfloat16_rn(x);
        *reinterpret_cast<__nv_bfloat16 *>(tiles + (size_t)l * W_BYTES + tc::tileOffset(out, in)) = b;
        *reinterpret_cast<__nv_bfloat16 *>(tiles + (size_t)(LAYERS + l) * W_BYTES + tc::tileOffset(in, out)) = b;
    }
}

__global__ void kBuildTiles(const float *p, uint8_t *tiles)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MLP_PARAMS; i += gridDim.x * blockDim.x) {
        const int l = i / (WIDTH * WIDTH), out = (i / WIDTH) % WIDTH, in = i % WIDTH;
        const __nv_bfloat16 b = __float2bfloat16_rn(p[i]);
        *reinterpret_cast<__nv_bfloat16 *>(tiles + (size_t)l * W_BYTES + tc::tileOffset(out, in)) = b;
        *reinterpret_cast<__nv_bfloat16 *>(tiles + (size_t)(LAYERS + l) * W_BYTES + tc::tileOffset(in, out)) = b;
    }
}

__global__ void kHashToHalf(const float *p, __half *ph, size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        writePair(ph, i, __float2half_rn(p[i]));
}

// splitmix64 for parameter initialisation (host)
uint64_t splitmix(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
float unit(uint64_t &s) { return (float)((splitmix(s) >> 40) * (1.0 / 16777216.0)); }

cudaError_t setSmem()
{
    static bool done = false;
    if (done)
        return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kGuideTrain, cudaFuncAttributeMaxDynamicSharedMemorySize, TRAIN_SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kGuideInfer<QueryInput>, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kGuideInfer<HitInput>, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM);
    done = e == cudaSuccess;
    return e;
}

}  // namespace

// ------------------------------------------------------------------ host side
GuideGeom guideGeom(const optpt_guide *g)
{
    GuideGeom r;
    r.levels = g->levels;
    r.lo = make_float3(g->lo[0], g->lo[1], g->lo[2]);
    r.invExt = make_float3(g->invExt[0], g->invExt[1], g->invExt[2]);
    r.lobeLoss = g->lobeLoss;
    return r;
}

void guideFree(optpt_guide *g)
{
    void *ptrs[] = {g->mlp, g->tiles, g->hash, g->hashH, g->gMlp, g->gHash, g->mMlp,
                    g->vMlp, g->mHash, g->vHash, g->stats, g->status, g->dStep};
    for (void *p : ptrs)
        if (p)
            cudaFree(p);
    *g = optpt_guide{};
}

int guideCreate(optpt_guide *g, const float lo[3], const float hi[3], uint32_t seed)
{
    const double b = std::exp(std::log((double)RES_MAX / RES_MIN) / (LEVELS - 1));
    for (int l = 0; l < LEVELS; ++l) {
        const double r = std::floor(RES_MIN * std::pow(b, l));
        g->levels.res[l] = (float)r;
        g->levels.dense[l] = (r + 1) * (r + 1) * (r + 1) <= (double)TABLE ? 1u : 0u;
    }
    for (int a = 0; a < 3; ++a) {
        const float ext = std::max(hi[a] - lo[a], 1e-6f);
        g->lo[a] = lo[a] - 0.01f * ext;
        g->invExt[a] = 1.0f / (1.02f * ext);
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g->numSMs, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void **p, size_t bytes) {
        if (e == cudaSuccess)
            e = cudaMalloc(p, bytes);
        if (e == cudaSuccess)
            e = cudaMemset(*p, 0, bytes);
    };
    alloc((void **)&g->mlp, sizeof(float) * MLP_PARAMS);
    alloc((void **)&g->tiles, 2 * LAYERS * W_BYTES);
    alloc((void **)&g->hash, sizeof(float) * HASH_PARAMS);
    alloc((void **)&g->hashH, sizeof(__half) * 2 * HASH_PARAMS);  // pair copy
    alloc((void **)&g->gMlp, sizeof(float) * MLP_PARAMS);
    alloc((void **)&g->gHash, sizeof(float) * HASH_PARAMS);
    alloc((void **)&g->mMlp, sizeof(float) * MLP_PARAMS);
    alloc((void **)&g->vMlp, sizeof(float) * MLP_PARAMS);
    alloc((void **)&g->mHash, sizeof(float) * HASH_PARAMS);
    alloc((void **)&g->vHash, sizeof(float) * HASH_PARAMS);
    alloc((void **)&g->stats, sizeof(double) * 4);
    alloc((void **)&g->status, sizeof(int));
    alloc((void **)&g->dStep, sizeof(uint32_t));
    if (e != cudaSuccess) {
        guideFree(g);
        return optpt_internal_set_error(OPTPT_ERR_NOMEM, cudaGetErrorString(e));
    }
    // initial parameters: Xavier-uniform weights, hash features U(-1e-4, 1e-4)
    uint64_t s = 0x6a09e667f3bcc909ull ^ ((uint64_t)seed << 17);
    std::vector<float> w(MLP_PARAMS);
    for (int l = 0; l < LAYERS; ++l) {
        const float fanIn = l == 0 ? (float)(IN_ONE + 1) : (float)WIDTH;
        const float a = std::sqrt(6.0f / (fanIn + WIDTH)) * (l == LAYERS - 1 ? 0.5f : 1.0f);
        for (int o = 0; o < WIDTH; ++o)
            for (int i = 0; i < WIDTH; ++i)
                w[(size_t)l * WIDTH * WIDTH + o * WIDTH + i] =
                    (l == 0 && i > IN_ONE) ? 0.0f : (2.0f * unit(s) - 1.0f) * a;
    }
    std::vector<float> hsh(HASH_PARAMS);
    for (size_t i = 0; i < HASH_PARAMS; ++i)
        hsh[i] = (2.0f * unit(s) - 1.0f) * 1e-4f;
    e = cudaMemcpy(g->mlp, w.data(), sizeof(float) * MLP_PARAMS, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(g->hash, hsh.data(), sizeof(float) * HASH_PARAMS, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        kBuildTiles<<<20, 256>>>(g->mlp, g->tiles);
        kHashToHalf<<<1024, 256>>>(g->hash, g->hashH, HASH_PARAMS);
        e = cudaDeviceSynchronize();
    }
    if (e == cudaSuccess)
        e = setSmem();
    if (e != cudaSuccess) {
        guideFree(g);
        return optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString(e));
    }
    return OPTPT_OK;
}

cudaError_t guideInferQueries(const optpt_guide *g, const GuideQuery *q, uint32_t n, Packed *out, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    const int tiles = (int)((n + TILE_ROWS - 1) / TILE_ROWS);
    const int grid = std::min((tiles + INFER_GROUPS - 1) / INFER_GROUPS, g->numSMs * OPTPT_INFER_MINB);
    kGuideInfer<QueryInput><<<grid, INFER_THREADS, INFER_SMEM, s>>>(guideGeom(g), g->hashH, g->tiles, QueryInput{q, n}, out,
                                                          g->status);
    return cudaGetLastError();
}

cudaError_t guideGradients(optpt_guide *g, const GuideSample *smp, const uint32_t *count, uint32_t capacity,
                           cudaStream_t s, uint32_t slice, uint32_t slices)
{
    cudaError_t e = cudaMemsetAsync(g->stats, 0, sizeof(double) * 4, s);
    if (e != cudaSuccess)
        return e;
    kBatchStats<<<g->numSMs, 256, 0, s>>>(smp, count, capacity, slice, slices, g->stats);
    const uint32_t perSlice = (capacity + slices - 1) / slices;
    const int grid = std::min(g->numSMs, (int)((perSlice + TILE_ROWS - 1) / TILE_ROWS));
    if (grid > 0)
        kGuideTrain<<<grid, 128, TRAIN_SMEM, s>>>(guideGeom(g), g->hash, g->tiles, smp, count, capacity, slice, slices,
                                                   g->stats, g->gMlp, g->gHash, g->stats + 1, g->status);
    return cudaGetLastError();
}

cudaError_t guideAdam(optpt_guide *g, cudaStream_t s)
{
    kAdamStep<<<1, 1, 0, s>>>(g->dStep);
    kAdamMlp<<<20, 256, 0, s>>>(g->mlp, g->tiles, g->gMlp, g->mMlp, g->vMlp, g->lr, g->dStep);
    kAdamHash<<<g->numSMs * 8, 256, 0, s>>>(g->hash, g->hashH, g->gHash, g->mHash, g->vHash, HASH_PARAMS, g->lr,
                                            g->dStep);
    return cudaGetLastError();
}

void launchGuideInfer(const optpt_guide *g, const DevScene &sc, const FrameParams &fp, const WaveBufs &q, int depth,
                      cudaStream_t st)
{
    const int cur = depth & 1;
    HitInput in{q.rayO[cur], q.rayD[cur], q.hit, sc.triV, q.counters + CNT_EXT + depth, 0u, nullptr, 0u};
    if (depth == 1 && fp.guide.sharePrimary) {
        // one query per pixel: the first sample of each pixel heads the queue
        if (fp.batch.on)
            in.limitPtr = fp.batch.dyn;
        else
            in.limit = fp.npix;
    }
    kGuideInfer<HitInput><<<g->numSMs * OPTPT_INFER_MINB, INFER_THREADS, INFER_SMEM, st>>>(
        guideGeom(g), g->hashH, g->tiles, in, reinterpret_cast<Packed *>(const_cast<void *>(fp.guide.mix)),
        g->status);
}

void launchGuideGather(const FrameParams &fp, const WaveBufs &q, cudaStream_t st)
{
    kGuideGather<<<1024, 256, 0, st>>>(fp, q);
}

// ------------------------------------------------------------------ C ABI
extern "C" {

int optpt_guide_create(const float lo[3], const float hi[3], uint32_t seed, optpt_guide **out)
{
    if (!lo || !hi || !out)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    optpt_guide *g = new optpt_guide();
    int rc = guideCreate(g, lo, hi, seed);
    if (rc != OPTPT_OK) {
        delete g;
        return rc;
    }
    *out = g;
    return OPTPT_OK;
}

int optpt_guide_mixture_eval(const void *mixtures, uint32_t n, const float *xi, float *dirPdf, void *stream)
{
    if (n == 0)
        return OPTPT_OK;
    if (!mixtures || !dirPdf)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    const int grid = (int)std::min<uint32_t>((n + 255) / 256, 4096u);
    kMixtureEval<<<grid, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const Packed *>(mixtures), n, xi,
                                                         reinterpret_cast<float4 *>(dirPdf));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? OPTPT_OK : optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString(e));
}

int optpt_guide_destroy(optpt_guide *g)
{
    if (!g)
        return OPTPT_OK;
    guideFree(g);
    delete g;
    return OPTPT_OK;
}

int optpt_guide_params(optpt_guide *g, float *mlp, float *hash, int write)
{
    if (!g)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL guide");
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess && mlp)
        e = write ? cudaMemcpy(g->mlp, mlp, sizeof(float) * MLP_PARAMS, cudaMemcpyHostToDevice)
                  : cudaMemcpy(mlp, g->mlp, sizeof(float) * MLP_PARAMS, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && hash)
        e = write ? cudaMemcpy(g->hash, hash, sizeof(float) * HASH_PARAMS, cudaMemcpyHostToDevice)
                  : cudaMemcpy(hash, g->hash, sizeof(float) * HASH_PARAMS, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && write) {
        kBuildTiles<<<20, 256>>>(g->mlp, g->tiles);
        kHashToHalf<<<1024, 256>>>(g->hash, g->hashH, HASH_PARAMS);
        e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString(e));
    return OPTPT_OK;
}

int optpt_guide_levels(optpt_guide *g, float *res, uint32_t *dense, float *lo, float *invExt)
{
    if (!g)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL guide");
    for (int l = 0; l < LEVELS; ++l) {
        if (res)
            res[l] = g->levels.res[l];
        if (dense)
            dense[l] = g->levels.dense[l];
    }
    for (int a = 0; a < 3; ++a) {
        if (lo)
            lo[a] = g->lo[a];
        if (invExt)
            invExt[a] = g->invExt[a];
    }
    return OPTPT_OK;
}

int optpt_guide_infer(optpt_guide *g, const float *queries, uint32_t n, void *mixtures, void *stream)
{
    if (!g || (n && (!queries || !mixtures)))
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    cudaError_t e = guideInferQueries(g, reinterpret_cast<const GuideQuery *>(queries), n,
                                      reinterpret_cast<Packed *>(mixtures), (cudaStream_t)stream);
    if (e != cudaSuccess)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString(e));
    return OPTPT_OK;
}

int optpt_guide_gradients(optpt_guide *g, const float *samples, const uint32_t *count, uint32_t capacity,
                          float *dMlp, float *dHash, double *loss, void *stream)
{
    if (!g || !samples || !count)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(g->gMlp, 0, sizeof(float) * MLP_PARAMS, s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(g->gHash, 0, sizeof(float) * HASH_PARAMS, s);
    if (e == cudaSuccess)
        e = guideGradients(g, reinterpret_cast<const GuideSample *>(samples), count, capacity, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    int st = 0;
    if (e == cudaSuccess)
        e = cudaMemcpy(&st, g->status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && dMlp)
        e = cudaMemcpy(dMlp, g->gMlp, sizeof(float) * MLP_PARAMS, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && dHash)
        e = cudaMemcpy(dHash, g->gHash, sizeof(float) * HASH_PARAMS, cudaMemcpyDeviceToHost);
    double stats[4] = {0, 0, 0, 0};
    if (e == cudaSuccess)
        e = cudaMemcpy(stats, g->stats, sizeof(stats), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString(e));
    if (st != 0)
        return optpt_internal_set_error(OPTPT_ERR_TIMEOUT, "tensor-core completion wait expired");
    if (loss)
        *loss = stats[1];
    return OPTPT_OK;
}

int optpt_guide_train_step(optpt_guide *g, const float *samples, const uint32_t *count, uint32_t capacity,
                           void *stream)
{
    if (!g || !samples || !count)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = guideGradients(g, reinterpret_cast<const GuideSample *>(samples), count, capacity, s);
    if (e == cudaSuccess)
        e = guideAdam(g, s);
    if (e != cudaSuccess)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString(e));
    return OPTPT_OK;
}

int optpt_guide_status(optpt_guide *g, int *status, double *lastLoss, double *lastSamples)
{
    if (!g || !status)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    double stats[4];
    cudaError_t e = cudaMemcpy(status, g->status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(stats, g->stats, sizeof(stats), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString(e));
    if (lastLoss)
        *lastLoss = stats[1];
    if (lastSamples)
        *lastSamples = stats[2];
    return OPTPT_OK;
}

// ------------------------------------------------------------------ tensor-core self-test
}  // extern "C"

namespace {

constexpr int ST_TILE = 16384;  // 128 x 64 BF16
constexpr int ST_SMEM = 3 * ST_TILE + 8192 + 16384;  // A, G, X, B (64 x 64) + headroom

// One CTA of 128 threads: C = A B^T (M 128, N 64, K 64, K-major operands)
// and dW = G^T X (M 64, N 64, K 128, MN-major operands read from the same
// row-major tiles), then every TMEM lane and column of both results is
// copied out: C to rows 0..127 of `c` (64 columns), the M = 64 result to
// `dwRaw` as 128 lanes x 64 columns.
__global__ void __launch_bounds__(128, 1)
    kTcSelftest(const uint16_t *A, const uint16_t *B, const uint16_t *G, const uint16_t *X, float *c, float *dwRaw,
                int *status)
{
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tmemBase;
    uint8_t *sA = sm, *sG = sm + ST_TILE, *sX = sm + 2 * ST_TILE, *sB = sm + 3 * ST_TILE;
    const int t = threadIdx.x, warp = t >> 5;
    for (int col = 0; col < 64; ++col) {
        *reinterpret_cast<uint16_t *>(sA + tc::tileOffset(t, col)) = A[t * 64 + col];
        *reinterpret_cast<uint16_t *>(sG + tc::tileOffset(t, col)) = G[t * 64 + col];
        *reinterpret_cast<uint16_t *>(sX + tc::tileOffset(t, col)) = X[t * 64 + col];
        if (t < 64)
            *reinterpret_cast<uint16_t *>(sB + tc::tileOffset(t, col)) = B[t * 64 + col];
    }
    if (t == 0)
        tc::mbarInit(&bar, 1);
    if (warp == 0)
        tc::tmemAlloc(&tmemBase, 128);
    tc::fenceProxyAsync();
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tm = tmemBase;
    if (t == 0) {
        const uint32_t a = tc::smemAddr(sA), b = tc::smemAddr(sB), g = tc::smemAddr(sG), x = tc::smemAddr(sX);
        for (int k = 0; k < 4; ++k)  // K = 16 per instruction: 2 core matrices along the columns
            tc::mma(tm, tc::smemDesc(a + 256 * k, 128, 1024), tc::smemDesc(b + 256 * k, 128, 1024),
                    tc::idescBf16(128, 64, false, false), k > 0);
        for (int k = 0; k < 8; ++k)  // K = 16 rows per instruction: 2 row groups
            tc::mma(tm + 64, tc::smemDesc(g + 2048 * k, 1024, 128), tc::smemDesc(x + 2048 * k, 1024, 128),
                    tc::idescBf16(64, 64, true, true), k > 0);
        tc::commit(&bar);
    }
    const bool ok = tc::mbarWait(&bar, 0);
    tc::fenceAfterSync();
    if (ok) {
        const uint32_t lane = (uint32_t)(32 * warp) << 16;
        for (int j = 0; j < 8; ++j) {
            float v[16];
            tc::ld16(tm + lane + 16 * j, v);
            float *dst = j < 4 ? c + t * 64 + 16 * j : dwRaw + t * 64 + 16 * (j - 4);
            for (int k = 0; k < 16; ++k)
                dst[k] = v[k];
        }
    } else if (t == 0) {
        *status = 1;
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    if (warp == 0)
        tc::tmemFree(tm, 128);
}

}  // namespace

extern "C" int optpt_tc_selftest(const uint16_t *A, const uint16_t *B, const uint16_t *G, const uint16_t *X, float *c,
                                 float *dwRaw, int *status, void *stream)
{
    if (!A || !B || !G || !X || !c || !dwRaw || !status)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    cudaError_t e = cudaFuncSetAttribute(kTcSelftest, cudaFuncAttributeMaxDynamicSharedMemorySize, ST_SMEM);
    if (e != cudaSuccess)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString(e));
    kTcSelftest<<<1, 128, ST_SMEM, (cudaStream_t)stream>>>(A, B, G, X, c, dwRaw, status);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString(e));
    return OPTPT_OK;
}
