// Frame output on the GPU: one pass over the frame buffers produces every
// payload the image writers need, so the host only entropy-codes.
//
// * RGBA8 of the tone-mapped frame buffer: the reference's processImage
//   (cu/kernels.cu:22-33), r = int(clamp(255.99 x, 0, 255)), packed
//   0xff000000 | r | g << 8 | b << 16;
// * RGBE of the accumulated mean radiance for the Radiance .hdr writer
//   (stbi_write_hdr in src/renderer.cpp:1009-1017): Ward's shared-exponent
//   encoding, mantissa m of frexp(max(r, g, b)), channel = c * 256 m / max;
// * HALF RGBA of the accumulated mean (A = 1) for OpenEXR
//   (dumpAccumFbToOpenExr, cu/kernels.cu:57-76), rounded to nearest even and
//   written channel-planar per scanline (A[w], B[w], G[w], R[w]), the byte
//   order an EXR scanline block stores.
// Each pixel is read once (32 B) and writes at most 16 B: the kernel is HBM
// bound; a grid-stride loop over pixels keeps every load and store coalesced.
#include <cuda_fp16.h>

#include "engine.h"

namespace {

__device__ __forceinline__ uint32_t quantise(float v)
{
    return (uint32_t)(int)fmaxf(0.0f, fminf(__fmul_rn(255.99f, v), 255.0f));
}

__device__ __forceinline__ uint32_t rgbe(float r, float g, float b)
{
    const float m = fmaxf(r, fmaxf(g, b));
    if (!(m >= 1e-32f))
        return 0u;
    int e;
    const float f = frexpf(m, &e);
    const float scale = __fdiv_rn(__fmul_rn(f, 256.0f), m);
    auto q = [&](float c) { return (uint32_t)fminf(fmaxf(__fmul_rn(c, scale), 0.0f), 255.0f); };
    const uint32_t ex = (uint32_t)min(e + 128, 255);
    return q(r) | (q(g) << 8) | (q(b) << 16) | (ex << 24);
}

// Four pixels per thread and iteration, all loads issued before any store,
// so each thread keeps up to eight 16-byte loads in flight.
__global__ void __launch_bounds__(256) kImageOut(const float4 *__restrict__ fb, const float4 *__restrict__ mean,
                                                 uint32_t w, uint32_t n, uint32_t *__restrict__ rgba8,
                                                 uint32_t *__restrict__ rgbeOut, __half *__restrict__ rows)
{
    constexpr int U = 4;
    const uint32_t stride = gridDim.x * blockDim.x;
    const bool wantMean = rgbeOut || rows;
    for (uint32_t base = blockIdx.x * blockDim.x + threadIdx.x; base < n; base += U * stride) {
        float4 c[U], m[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t i = base + (uint32_t)u * stride;
            if (i < n) {
                if (rgba8)
                    c[u] = __ldcs(fb + i);
                if (wantMean)
                    m[u] = __ldcs(mean + i);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t i = base + (uint32_t)u * stride;
            if (i >= n)
                break;
            if (rgba8)
                __stcs(rgba8 + i, 0xff000000u | quantise(c[u].x) | (quantise(c[u].y) << 8) | (quantise(c[u].z) << 16));
            if (rgbeOut)
                __stcs(rgbeOut + i, rgbe(m[u].x, m[u].y, m[u].z));
            if (rows) {
                const uint32_t y = i / w, x = i - y * w;
                __half *row = rows + (size_t)y * 4 * w + x;
                row[0] = __float2half_rn(1.0f);
                row[w] = __float2half_rn(m[u].z);
                row[2 * w] = __float2half_rn(m[u].y);
                row[3 * w] = __float2half_rn(m[u].x);
            }
        }
    }
}

}  // namespace

void launchImageOut(const float4 *fb, const float4 *mean, uint32_t w, uint32_t h, uint32_t *rgba8, uint32_t *rgbeOut,
                    void *rows, cudaStream_t st)
{
    const uint32_t n = w * h;
    if (n == 0)
        return;
    // One resident wave: SMs x the blocks per SM the kernel's registers allow.
    static int perSm = 0, sms = 0;
    if (!perSm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kImageOut, 256, 0);
        if (perSm < 1)
            perSm = 1;
    }
    const uint32_t want = (n + 1023) / 1024, cap = (uint32_t)(sms > 0 ? sms : 1) * (uint32_t)perSm;
    kImageOut<<<want < cap ? want : cap, 256, 0, st>>>(fb, mean, w, n, rgba8, rgbeOut, static_cast<__half *>(rows));
}
