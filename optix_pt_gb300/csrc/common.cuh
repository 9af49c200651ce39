// Shared device/host helpers: float3 algebra, the counter-based PCG32 random
// stream, and the constants of the reference integrator.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define OPT_HD __host__ __device__ __forceinline__
#define OPT_D __device__ __forceinline__

// cu/... cuda_utils.h:5-7 of the reference: MAX_DEPTH is a runtime value here.
#define OPT_SCENE_EPSILON 0.0001f
#define OPT_SHADOW_BIAS 0.001f
#define OPT_PI 3.14159265358979323846f
#define OPT_INV_PI 0.318309886183790671538f

OPT_HD float3 mk3(float x, float y, float z) { return make_float3(x, y, z); }
OPT_HD float3 mk3s(float s) { return make_float3(s, s, s); }
OPT_HD float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
OPT_HD float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
OPT_HD float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
OPT_HD float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
OPT_HD float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
OPT_HD float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
OPT_HD float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
OPT_HD float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
OPT_HD float3 cross3(float3 a, float3 b)
{
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
OPT_HD float length3(float3 a) { return sqrtf(dot3(a, a)); }
OPT_HD float3 normalize3(float3 a)
{
    float inv = 1.0f / sqrtf(dot3(a, a));
    return a * inv;
}
OPT_HD float maxc3(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
OPT_HD float3 f3of4(float4 a) { return make_float3(a.x, a.y, a.z); }

// ---------------------------------------------------------------- random numbers
// Counter-based PCG32 (O'Neill, "PCG: A Family of Simple Fast Space-Efficient
// Statistically Good Algorithms for Random Number Generation", 2014): the
// XSH-RR output of a 64-bit LCG. The reference keeps a cuRAND XORWOW state per
// pixel across frames (random_number_generators.h:64-93, cu/kernels.cu:78-86);
// here a stream is a pure function of (seed, pixel, sample, depth), so no
// state is stored and any sample can be replayed exactly.

OPT_HD uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

struct Pcg32 {
    uint64_t state;
    uint64_t inc;

    OPT_HD uint32_t next()
    {
        uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18) ^ old) >> 27);
        uint32_t rot = (uint32_t)(old >> 59);
        return (xorshifted >> rot) | (xorshifted << ((0u - rot) & 31u));
    }
    // Uniform in [0, 1) with 24 random bits.
    OPT_HD float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }

    OPT_HD void seed(uint64_t initstate, uint64_t initseq)
    {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
};

// The stream of pixel `pixel`, sample `sample`, path vertex `depth` (0 = camera
// jitter, d >= 1 = shading of the d-th hit).
OPT_HD Pcg32 pathRng(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t depth)
{
    Pcg32 r;
    r.seed(splitmix64(((uint64_t)seed << 32) | pixel), splitmix64(((uint64_t)sample << 8) | (depth & 0xFFu)));
    return r;
}

// One uniform for an alpha-blended candidate hit (the reference draws it from
// the path stream inside any-hit, cu/device_programs.cu:159, in traversal
// order; here it is a hash of the candidate so the result does not depend on
// the order in which the BVH is walked).
OPT_HD float blendUniform(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t depth, uint32_t prim)
{
    uint64_t k = splitmix64(((uint64_t)seed << 32) | pixel) ^ splitmix64(((uint64_t)sample << 40) ^
                                                                        ((uint64_t)depth << 32) ^ prim);
    return (float)(splitmix64(k) >> 40) * (1.0f / 16777216.0f);
}
