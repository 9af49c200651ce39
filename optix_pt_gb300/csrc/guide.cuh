// Learned path guiding, device side shared by the network kernels and the
// shading kernel: the multiresolution hash-grid position encoding (after
// Mueller et al., "Instant Neural Graphics Primitives", SIGGRAPH 2022), the
// network's input/output layout, and the von Mises-Fisher mixture the network
// emits (evaluation, sampling and decoding; mixture parameterisation after
// Dong et al., "Neural Parametric Mixtures for Path Guiding", SIGGRAPH 2023).
#pragma once
#include <cuda_fp16.h>
#include <cstdint>
#include "common.cuh"

namespace guide {

constexpr int LEVELS = 16;            // hash-grid levels
constexpr int FEATS = 2;              // features per level
constexpr uint32_t TABLE = 1u << 19;  // entries per level
constexpr float RES_MIN = 16.0f, RES_MAX = 256.0f;
constexpr int WIDTH = 64;             // network width (inputs padded to 64)
constexpr int LAYERS = 5;             // 64x64 weight matrices: in -> h1 -> h2 -> h3 -> h4 -> out
constexpr int LOBES = 8;              // vMF lobes; outputs 5k..5k+4 = (mu raw xyz, log kappa, weight logit)
constexpr int OUT_SELECT = 5 * LOBES; // output 40: logit of the probability of sampling the mixture
constexpr float SELECT_MIN = 0.02f, SELECT_SPAN = 0.96f;  // that probability = MIN + SPAN * sigmoid(logit)
constexpr int IN_NORMAL = 2 * LEVELS, IN_WO = IN_NORMAL + 3, IN_ONE = IN_WO + 3;
constexpr float LOG_KAPPA_MIN = -3.0f, LOG_KAPPA_MAX = 5.5f;
constexpr size_t HASH_PARAMS = (size_t)LEVELS * TABLE * FEATS;
constexpr int MLP_PARAMS = LAYERS * WIDTH * WIDTH;

// Grid resolution of level l: floor(RES_MIN * b^l), b = (RES_MAX/RES_MIN)^(1/(LEVELS-1)).
// The host computes the table once (levelRes) so device and oracle agree.
struct Levels {
    float res[LEVELS];
    uint32_t dense[LEVELS];  // 1: (res+1)^3 <= TABLE, direct indexing
};

// Table entry of grid vertex (x, y, z): direct indexing on dense levels, else
// a spatial hash. x enters both by addition, so the vertex at x + 1 is the
// next entry (modulo the table): the inference copy of the table stores each
// entry beside its successor and fetches both x-corners of a cell edge with
// one 8-byte load.
OPT_HD uint32_t cornerIndex(uint32_t x, uint32_t y, uint32_t z, uint32_t res1, bool dense)
{
    if (dense)
        return x + res1 * (y + res1 * z);
    return (x + (y * 2654435761u ^ z * 805459861u)) & (TABLE - 1u);
}

// Trilinear corner c (bit 0 = x, 1 = y, 2 = z) of level `l` for a position
// in the unit cube: the table entry and the weight.
OPT_HD void corner(const Levels &L, int l, float px, float py, float pz, int c, uint32_t &entry, float &w)
{
    const float r = L.res[l];
    const float gx = px * r, gy = py * r, gz = pz * r;
    const float fx = floorf(gx), fy = floorf(gy), fz = floorf(gz);
    const float tx = gx - fx, ty = gy - fy, tz = gz - fz;
    const uint32_t x = (uint32_t)fx + (c & 1), y = (uint32_t)fy + ((c >> 1) & 1), z = (uint32_t)fz + ((c >> 2) & 1);
    w = ((c & 1) ? tx : 1.0f - tx) * (((c >> 1) & 1) ? ty : 1.0f - ty) * (((c >> 2) & 1) ? tz : 1.0f - tz);
    entry = cornerIndex(x, y, z, (uint32_t)r + 1u, L.dense[l] != 0);
}

// All 8 trilinear corners of level `l` (the same arithmetic as `corner`,
// with the cell computed once).
OPT_HD void levelCorners(const Levels &L, int l, float px, float py, float pz, uint32_t (&entry)[8], float (&w)[8])
{
    const float r = L.res[l];
    const float gx = px * r, gy = py * r, gz = pz * r;
    const float fx = floorf(gx), fy = floorf(gy), fz = floorf(gz);
    const float tx = gx - fx, ty = gy - fy, tz = gz - fz;
    const uint32_t x0 = (uint32_t)fx, y0 = (uint32_t)fy, z0 = (uint32_t)fz, res1 = (uint32_t)r + 1u;
    const bool dense = L.dense[l] != 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        w[c] = ((c & 1) ? tx : 1.0f - tx) * (((c >> 1) & 1) ? ty : 1.0f - ty) * (((c >> 2) & 1) ? tz : 1.0f - tz);
        entry[c] = cornerIndex(x0 + (c & 1), y0 + ((c >> 1) & 1), z0 + ((c >> 2) & 1), res1, dense);
    }
}

// The same cell without the weights: the 8 corner entries and the fractions
// (tx, ty, tz), from which cornerWeight forms corner c's weight with
// levelCorners' arithmetic, at the point of use.
OPT_HD void levelCell(const Levels &L, int l, float px, float py, float pz, uint32_t (&entry)[8], float &tx,
                      float &ty, float &tz)
{
    const float r = L.res[l];
    const float gx = px * r, gy = py * r, gz = pz * r;
    const float fx = floorf(gx), fy = floorf(gy), fz = floorf(gz);
    tx = gx - fx;
    ty = gy - fy;
    tz = gz - fz;
    const uint32_t x0 = (uint32_t)fx, y0 = (uint32_t)fy, z0 = (uint32_t)fz, res1 = (uint32_t)r + 1u;
    const bool dense = L.dense[l] != 0;
#pragma unroll
    for (int c = 0; c < 8; ++c)
        entry[c] = cornerIndex(x0 + (c & 1), y0 + ((c >> 1) & 1), z0 + ((c >> 2) & 1), res1, dense);
}
OPT_HD float cornerWeight(int c, float tx, float ty, float tz)
{
    return ((c & 1) ? tx : 1.0f - tx) * (((c >> 1) & 1) ? ty : 1.0f - ty) * (((c >> 2) & 1) ? tz : 1.0f - tz);
}

// ------------------------------------------------------------------ vMF mixture
struct Lobe {
    float3 mu;
    float kappa, weight;
};
struct Mixture {
    Lobe lobe[LOBES];
    float select;  // probability of sampling the mixture rather than the BSDF
};

// Normalisation kappa / (2 pi (1 - exp(-2 kappa))), the isotropic 1/(4 pi) as kappa -> 0.
OPT_D float vmfNorm(float kappa)
{
    if (kappa < 1e-4f)
        return 0.25f * OPT_INV_PI;
    return kappa * (0.5f * OPT_INV_PI) / -expm1f(-2.0f * kappa);
}
OPT_D float vmfPdf(const Lobe &L, float3 w)
{
    return vmfNorm(L.kappa) * expf(L.kappa * (dot3(L.mu, w) - 1.0f));
}
// Direction from a vMF lobe by Jakob's stable inversion ("Numerically
// stable sampling of the von Mises-Fisher distribution on S^2").
OPT_D float3 vmfSample(float3 mu, float kappa, float xi1, float xi2)
{
    float w;
    if (kappa < 1e-4f)
        w = 1.0f - 2.0f * xi1;
    else
        w = 1.0f + logf(xi1 + (1.0f - xi1) * expf(-2.0f * kappa)) / kappa;
    w = fminf(fmaxf(w, -1.0f), 1.0f);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - w * w));
    float sp, cp;
    sincosf(2.0f * OPT_PI * xi2, &sp, &cp);
    // frame around mu (Duff et al. 2017 branchless ONB)
    const float3 n = mu;
    const float sign = copysignf(1.0f, n.z);
    const float a = -1.0f / (sign + n.z), b = n.x * n.y * a;
    const float3 t = mk3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    const float3 bt = mk3(b, sign + n.y * n.y * a, -n.y);
    return normalize3(w * n + (s * cp) * t + (s * sp) * bt);
}

// Network outputs o[0..40] -> mixture (softmax weights, exp kappa, unit mu)
// and the selection probability.
OPT_D void decodeOutputs(const float *o, Mixture &m)
{
    m.select = SELECT_MIN + SELECT_SPAN / (1.0f + expf(-o[OUT_SELECT]));
    float mx = -1e30f;
#pragma unroll
    for (int k = 0; k < LOBES; ++k)
        mx = fmaxf(mx, o[5 * k + 4]);
    float sum = 0.0f;
#pragma unroll
    for (int k = 0; k < LOBES; ++k) {
        const float e = expf(o[5 * k + 4] - mx);
        m.lobe[k].weight = e;
        sum += e;
        const float3 r = mk3(o[5 * k], o[5 * k + 1], o[5 * k + 2]);
        const float len = sqrtf(dot3(r, r));
        m.lobe[k].mu = len > 1e-12f ? r * (1.0f / len) : mk3(0.0f, 0.0f, 1.0f);
        m.lobe[k].kappa = expf(fminf(fmaxf(o[5 * k + 3], LOG_KAPPA_MIN), LOG_KAPPA_MAX));
    }
    const float inv = 1.0f / sum;
#pragma unroll
    for (int k = 0; k < LOBES; ++k)
        m.lobe[k].weight *= inv;
}

// Packed mixture as stored per ray between the inference and shading kernels:
// per lobe (mu.xyz, kappa) as 4 halves, the 8 weights, then the selection
// probability, as halves: 96 B.
struct alignas(16) Packed {
    uint4 q[6];
};
OPT_D void pack(const Mixture &m, Packed &p)
{
    __half h[48];
#pragma unroll
    for (int k = 40; k < 48; ++k)
        h[k] = __float2half_rn(0.0f);
    h[40] = __float2half_rn(m.select);
#pragma unroll
    for (int k = 0; k < LOBES; ++k) {
        h[4 * k] = __float2half_rn(m.lobe[k].mu.x);
        h[4 * k + 1] = __float2half_rn(m.lobe[k].mu.y);
        h[4 * k + 2] = __float2half_rn(m.lobe[k].mu.z);
        h[4 * k + 3] = __float2half_rn(fminf(m.lobe[k].kappa, 60000.0f));
        h[32 + k] = __float2half_rn(m.lobe[k].weight);
    }
    memcpy(&p, h, sizeof(p));
}
// The shading kernel reads the packed mixture directly (no unpacked copy, so
// nothing is indexed at run time and it all stays in registers). Sampling
// and evaluation use the same decoded values, so the density evaluated is
// exactly the one sampled from: mu renormalised from its halves, kappa,
// weights normalised to sum 1 (uniform if they are all zero).
OPT_D float packedHalf(const Packed &p, int i)  // i: a constant after unrolling
{
    const uint4 q = p.q[i >> 3];
    const int wi = (i >> 1) & 3;
    const uint32_t w = wi == 0 ? q.x : wi == 1 ? q.y : wi == 2 ? q.z : q.w;
    return __half2float(__ushort_as_half((unsigned short)((i & 1) ? (w >> 16) : (w & 0xFFFFu))));
}
// Unit mean direction from a lobe's halves: r / |r| by one reciprocal square
// root ((0, 0, 1) for a null lobe). Sampling and evaluation both use it, so
// the density evaluated is the one sampled from.
OPT_D float3 unitMu(float rx, float ry, float rz)
{
    const float d2 = rx * rx + ry * ry + rz * rz;
    if (!(d2 > 1e-12f))
        return mk3(0.0f, 0.0f, 1.0f);
    const float il = rsqrtf(d2);
    return mk3(rx * il, ry * il, rz * il);
}
OPT_D float3 packedMu(const Packed &p, int k)
{
    return unitMu(packedHalf(p, 4 * k), packedHalf(p, 4 * k + 1), packedHalf(p, 4 * k + 2));
}
OPT_D float packedSelect(const Packed &p) { return packedHalf(p, 40); }
OPT_D float packedWeightSum(const Packed &p)
{
    float sum = 0.0f;
#pragma unroll
    for (int k = 0; k < LOBES; ++k)
        sum += packedHalf(p, 32 + k);
    return sum;
}
OPT_D float packedWeight(const Packed &p, int k, float sum, float inv)
{
    return sum > 0.0f ? packedHalf(p, 32 + k) * inv : 1.0f / LOBES;
}
// vMF density of a packed lobe with the hardware exponential: a packed kappa
// is 0 (null mixture: isotropic) or exp(log kappa) >= exp(LOG_KAPPA_MIN)
// ~ 0.05, where 1 - exp(-2 kappa) >= 0.095, so the subtraction keeps a
// relative error near 1e-6 without expm1.
OPT_D float vmfPdfPacked(float3 mu, float kappa, float3 w)
{
    if (kappa < 1e-4f)
        return 0.25f * OPT_INV_PI;
    const float norm = __fdividef(kappa * (0.5f * OPT_INV_PI), 1.0f - __expf(-2.0f * kappa));
    return norm * __expf(kappa * (dot3(mu, w) - 1.0f));
}
OPT_D float mixturePdf(const Packed &p, float3 w)
{
    const float sum = packedWeightSum(p), inv = sum > 0.0f ? 1.0f / sum : 0.0f;
    float pdf = 0.0f;
#pragma unroll
    for (int k = 0; k < LOBES; ++k)
        pdf += packedWeight(p, k, sum, inv) * vmfPdfPacked(packedMu(p, k), packedHalf(p, 4 * k + 3), w);
    return pdf;
}
// Lobe by xi0 over the weights, then a direction from it.
OPT_D float3 mixtureSample(const Packed &p, float xi0, float xi1, float xi2)
{
    const float sum = packedWeightSum(p), inv = sum > 0.0f ? 1.0f / sum : 0.0f;
    float acc = 0.0f;
    int k = LOBES - 1;
    bool found = false;
#pragma unroll
    for (int j = 0; j < LOBES; ++j) {
        acc += packedWeight(p, j, sum, inv);
        if (!found && xi0 < acc) {
            k = j;
            found = true;
        }
    }
    // the chosen lobe's halves first, then one normalisation (packedMu's)
    float rx = packedHalf(p, 4 * (LOBES - 1)), ry = packedHalf(p, 4 * (LOBES - 1) + 1),
          rz = packedHalf(p, 4 * (LOBES - 1) + 2), kappa = packedHalf(p, 4 * (LOBES - 1) + 3);
#pragma unroll
    for (int j = 0; j < LOBES - 1; ++j)
        if (j == k) {
            rx = packedHalf(p, 4 * j);
            ry = packedHalf(p, 4 * j + 1);
            rz = packedHalf(p, 4 * j + 2);
            kappa = packedHalf(p, 4 * j + 3);
        }
    return vmfSample(unitMu(rx, ry, rz), kappa, xi1, xi2);
}

}  // namespace guide
