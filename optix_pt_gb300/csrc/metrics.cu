// Error reductions on the GPU, in FP64: the relative MSE of a progressive
// image against a reference image, the error measure of the equal-time
// comparisons (relMSE = mean over pixels of sum over rgb of
// (I - R)^2 / (R^2 + 1e-2)).
//
// Two kernels: each block reduces one tile of RELMSE_TILE pixels to a partial
// sum (scratch, one double per tile), then one block adds the partials in a
// fixed order, so the result is deterministic for a given image size.
#include <cuda_runtime.h>
#include <mutex>
#include <string>
#include "../../include/optpt.h"
#include "engine.h"

extern "C" int optpt_internal_set_error(int code, const char *msg);

namespace {

constexpr int RELMSE_BLOCK = 256;
constexpr int RELMSE_PER_THREAD = 8;
constexpr uint32_t RELMSE_TILE = RELMSE_BLOCK * RELMSE_PER_THREAD;

__device__ __forceinline__ double blockSum(double v)
{
    __shared__ double warpSums[RELMSE_BLOCK / 32];
    for (int off = 16; off > 0; off >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0)
        warpSums[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < RELMSE_BLOCK / 32 ? warpSums[threadIdx.x] : 0.0;
        for (int off = 16; off > 0; off >>= 1)
            t += __shfl_down_sync(0xffffffffu, t, off);
    }
    return t;
}

__global__ void __launch_bounds__(RELMSE_BLOCK)
    kRelMseTiles(const Acc4 *__restrict__ sum, double invN, const Acc4 *__restrict__ ref, uint32_t n,
                 double *__restrict__ partial)
{
    const uint32_t base = blockIdx.x * RELMSE_TILE;
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < RELMSE_PER_THREAD; ++k) {
        const uint32_t i = base + (uint32_t)k * RELMSE_BLOCK + threadIdx.x;
        if (i < n) {
            const Acc4 s = sum[i], r = ref[i];
            const double dx = s.x * invN - r.x, dy = s.y * invN - r.y, dz = s.z * invN - r.z;
            acc += dx * dx / (r.x * r.x + 1e-2) + dy * dy / (r.y * r.y + 1e-2) + dz * dz / (r.z * r.z + 1e-2);
        }
    }
    const double t = blockSum(acc);
    if (threadIdx.x == 0)
        partial[blockIdx.x] = t;
}

__global__ void __launch_bounds__(RELMSE_BLOCK)
    kRelMseFinal(const double *__restrict__ partial, uint32_t tiles, uint32_t n, double *__restrict__ out)
{
    double acc = 0.0;
    for (uint32_t i = threadIdx.x; i < tiles; i += RELMSE_BLOCK)
        acc += partial[i];
    const double t = blockSum(acc);
    if (threadIdx.x == 0)
        out[0] = t / (double)n;
}

}  // namespace

// Launches both kernels with caller-chosen scratch (tiles doubles).
int relmseLaunch(const double *sum, uint32_t nSamples, const double *ref, uint32_t numPixels, double *out,
                 double *scratch, cudaStream_t st)
{
    const uint32_t tiles = (numPixels + RELMSE_TILE - 1) / RELMSE_TILE;
    kRelMseTiles<<<tiles, RELMSE_BLOCK, 0, st>>>(reinterpret_cast<const Acc4 *>(sum), 1.0 / (double)nSamples,
                                                 reinterpret_cast<const Acc4 *>(ref), numPixels, scratch);
    kRelMseFinal<<<1, RELMSE_BLOCK, 0, st>>>(scratch, tiles, numPixels, out);
    return (int)cudaGetLastError();
}

uint32_t relmseTiles(uint32_t numPixels) { return (numPixels + RELMSE_TILE - 1) / RELMSE_TILE; }

// ------------------------------------------------------------------ allocation-free variant
//
// For callers that must not allocate device memory at the point of the call:
// code inside a CUDA stream capture (cudaMalloc is not allowed there, and a
// stream-ordered allocation would become part of the graph), real-time frame
// loops that forbid allocator calls, and hosts whose memory pool owns all
// device memory. The partial sums live in a fixed array in the library's own
// device memory instead. It holds RELMSE_NOALLOC_TILES tiles, so images of up
// to RELMSE_NOALLOC_TILES * 2048 = 8,388,608 pixels (a 3840x2160 frame fits);
// larger images are rejected. Every GPU that loads the library keeps these
// 32 KiB until the process exits.
constexpr uint32_t RELMSE_NOALLOC_TILES = 4096;
static __device__ __align__(256) double g_relmseScratch[RELMSE_NOALLOC_TILES];

namespace {
constexpr int MAX_DEVICES = 64;
std::mutex g_scratchMutex;
double *g_scratchAddr[MAX_DEVICES] = {};  // device address of g_relmseScratch, per device

// Looks up (once per device, with that device current) the device address of
// the scratch array; host code cannot use the symbol itself as a pointer.
int scratchAddress(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_scratchMutex);
    if (!g_scratchAddr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_relmseScratch);
        if (e != cudaSuccess)
            return optpt_internal_set_error(OPTPT_ERR_CUDA,
                                            (std::string("scratch address: ") + cudaGetErrorString(e)).c_str());
        g_scratchAddr[dev] = static_cast<double *>(p);
    }
    *out = g_scratchAddr[dev];
    return OPTPT_OK;
}
}  // namespace

extern "C" int optpt_relmse_noalloc(const double *sum, uint32_t nSamples, const double *ref, uint32_t numPixels,
                                    double *out, void *stream)
{
    if (!sum || !ref || !out || numPixels == 0 || nSamples == 0)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "optpt_relmse_noalloc: NULL buffer or empty image");
    if (relmseTiles(numPixels) > RELMSE_NOALLOC_TILES)
        return optpt_internal_set_error(
            OPTPT_ERR_INVALID,
            ("optpt_relmse_noalloc: " + std::to_string(numPixels) + " pixels exceed the maximum of " +
             std::to_string((unsigned long long)RELMSE_NOALLOC_TILES * RELMSE_TILE) + "; use optpt_relmse")
                .c_str());
    double *scratch = nullptr;
    int rc = scratchAddress(&scratch);
    if (rc)
        return rc;
    // Every tile the final kernel reads is written by the first kernel of the
    // same call, so no clearing is needed; calls that overlap on the GPU
    // share the array and race.
    rc = relmseLaunch(sum, nSamples, ref, numPixels, out, scratch, (cudaStream_t)stream);
    if (rc)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString((cudaError_t)rc));
    return OPTPT_OK;
}

extern "C" int optpt_relmse(const double *sum, uint32_t nSamples, const double *ref, uint32_t numPixels, double *out,
                            void *stream)
{
    if (!sum || !ref || !out || numPixels == 0 || nSamples == 0)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "optpt_relmse: NULL buffer or empty image");
    cudaStream_t st = (cudaStream_t)stream;
    double *scratch = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&scratch, sizeof(double) * relmseTiles(numPixels), st);
    if (e != cudaSuccess)
        return optpt_internal_set_error(OPTPT_ERR_NOMEM, (std::string("optpt_relmse scratch: ") + cudaGetErrorString(e)).c_str());
    int rc = relmseLaunch(sum, nSamples, ref, numPixels, out, scratch, st);
    cudaFreeAsync(scratch, st);
    if (rc)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, cudaGetErrorString((cudaError_t)rc));
    return OPTPT_OK;
}
