// Software texture sampling of RGBA8 images stored as packed texels in HBM.
// Stands in for the reference's hardware texture objects (src/renderer.cpp:
// 1439-1757: normalized coordinates, linear or point filter, wrap/clamp/mirror
// per axis, sRGB decode for colour textures). Filter weights are FP32 rather
// than the texture unit's 8-bit fixed point, so the host oracle reproduces the
// result exactly.
#pragma once
#include "common.cuh"

#define TEX_WRAP_REPEAT 0
#define TEX_WRAP_CLAMP 1
#define TEX_WRAP_MIRROR 2

// sRGB -> linear for the 256 byte values (IEC 61966-2-1), filled by the host.
__constant__ float c_srgbToLinear[256];

OPT_D int wrapTexel(int i, int n, int mode)
{
    if (mode == TEX_WRAP_CLAMP)
        return min(max(i, 0), n - 1);
    if (mode == TEX_WRAP_MIRROR) {
        int p = 2 * n;
        int m = ((i % p) + p) % p;
        return m < n ? m : p - 1 - m;
    }
    return ((i % n) + n) % n;
}

// Byte -> [0, 1] as one rounded multiply; __fmul_rn keeps the compiler from
// fusing it into the filter's differences (a fused multiply-subtract rounds
// differently from the host's separate operations).
OPT_D float4 texelToFloat(uint32_t t, bool srgb)
{
    float4 c;
    if (srgb) {
        c.x = c_srgbToLinear[t & 0xFFu];
        c.y = c_srgbToLinear[(t >> 8) & 0xFFu];
        c.z = c_srgbToLinear[(t >> 16) & 0xFFu];
    } else {
        c.x = __fmul_rn((float)(t & 0xFFu), 1.0f / 255.0f);
        c.y = __fmul_rn((float)((t >> 8) & 0xFFu), 1.0f / 255.0f);
        c.z = __fmul_rn((float)((t >> 16) & 0xFFu), 1.0f / 255.0f);
    }
    c.w = __fmul_rn((float)(t >> 24), 1.0f / 255.0f);
    return c;
}

// info = (first texel, width, height, wrapS | wrapT << 4 | srgb << 8 | point << 9)
OPT_D float4 sampleTexture(const uint32_t *__restrict__ texels, int4 info, float u, float v)
{
    const int W = info.y, H = info.z;
    const int ws = info.w & 0xF, wt = (info.w >> 4) & 0xF;
    const bool srgb = (info.w >> 8) & 1, point = (info.w >> 9) & 1;
    const uint32_t *img = texels + info.x;
    if (point) {
        const float x = __fmul_rn(u, (float)W), y = __fmul_rn(v, (float)H);
        int ix = wrapTexel((int)floorf(x), W, ws), iy = wrapTexel((int)floorf(y), H, wt);
        return texelToFloat(__ldg(img + iy * W + ix), srgb);
    }
    // Every multiply-add is an explicit fmaf, in the order the host oracle uses.
    const float x = fmaf(u, (float)W, -0.5f), y = fmaf(v, (float)H, -0.5f);
    float fx0 = floorf(x), fy0 = floorf(y);
    float ax = x - fx0, ay = y - fy0;
    int x0 = (int)fx0, y0 = (int)fy0;
    int xa = wrapTexel(x0, W, ws), xb = wrapTexel(x0 + 1, W, ws);
    int ya = wrapTexel(y0, H, wt), yb = wrapTexel(y0 + 1, H, wt);
    float4 c00 = texelToFloat(__ldg(img + ya * W + xa), srgb), c10 = texelToFloat(__ldg(img + ya * W + xb), srgb);
    float4 c01 = texelToFloat(__ldg(img + yb * W + xa), srgb), c11 = texelToFloat(__ldg(img + yb * W + xb), srgb);
    auto bl = [&](float a00, float a10, float a01, float a11) {
        const float top = fmaf(a10 - a00, ax, a00), bot = fmaf(a11 - a01, ax, a01);
        return fmaf(bot - top, ay, top);
    };
    return make_float4(bl(c00.x, c10.x, c01.x, c11.x), bl(c00.y, c10.y, c01.y, c11.y), bl(c00.z, c10.z, c01.z, c11.z),
                       bl(c00.w, c10.w, c01.w, c11.w));
}

// Barycentric interpolation of a texture coordinate: w t0 + u t1 + v t2 with
// w = 1 - u - v, as explicit fmaf (identical on the host).
OPT_D float baryInterp(float u, float v, float t0, float t1, float t2)
{
    const float w = (1.0f - u) - v;
    return fmaf(v, t2, fmaf(u, t1, __fmul_rn(w, t0)));
}
