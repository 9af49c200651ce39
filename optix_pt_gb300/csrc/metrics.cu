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

// Tiles of an image, in 64 bits: no pixel count can wrap it.
uint64_t relmseTiles(uint32_t numPixels) { return ((uint64_t)numPixels + RELMSE_TILE - 1) / RELMSE_TILE; }

// Launches both kernels with caller-chosen scratch (relmseTiles doubles).
// Returns 0 or the CUDA error of these two launches. An error left pending by
// earlier, unrelated work on this thread is reported as such, without
// launching and without clearing it, so it is not blamed on this call.
int relmseLaunch(const double *sum, uint32_t nSamples, const double *ref, uint32_t numPixels, double *out,
                 double *scratch, cudaStream_t st)
{
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, (std::string("relMSE not launched: an earlier CUDA error is "
                                                                     "pending: ") + cudaGetErrorString(pending)).c_str());
    // at most 2^21 tiles for a 32-bit pixel count, within the grid limit
    const uint32_t tiles = (uint32_t)relmseTiles(numPixels);
    kRelMseTiles<<<tiles, RELMSE_BLOCK, 0, st>>>(reinterpret_cast<const Acc4 *>(sum), 1.0 / (double)nSamples,
                                                 reinterpret_cast<const Acc4 *>(ref), numPixels, scratch);
    kRelMseFinal<<<1, RELMSE_BLOCK, 0, st>>>(scratch, tiles, numPixels, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return optpt_internal_set_error(OPTPT_ERR_CUDA, (std::string("relMSE launch: ") + cudaGetErrorString(e)).c_str());
    return OPTPT_OK;
}

// ------------------------------------------------------------------ allocation-free variant
//
// For callers that must not allocate device memory at the point of the call:
// a progressive viewer's per-frame loop that promises no allocator call per
// frame (cudaMalloc and cudaFree can synchronise the device and stall the
// frame), and host applications whose own memory pool owns all device memory
// and does not let a library allocate behind its back. The partial sums live
// in a fixed array in the library's own device memory instead. It holds
// RELMSE_NOALLOC_TILES tiles, so images of up to RELMSE_NOALLOC_TILES * 2048 =
// 8,388,608 pixels (a 3840x2160 frame fits); larger images are rejected.
// Every GPU that loads the library keeps these 32 KiB until the process exits.
constexpr uint32_t RELMSE_NOALLOC_TILES = 4096;
static __device__ __align__(256) double g_relmseScratch[RELMSE_NOALLOC_TILES];

namespace {
constexpr int MAX_DEVICES = 64;
std::mutex g_scratchMutex;
double *g_scratchAddr[MAX_DEVICES] = {};  // device address of g_relmseScratch, per device

// Looks up (once per device, with that device current) the device address of
// the scratch array; host code cannot use the symbol itself as a pointer. The
// address is cached for the life of the process: a cudaDeviceReset (or any
// reset of the primary context) unloads the module and makes it stale, so a
// process that resets a device must not call optpt_relmse_noalloc on it
// afterwards.
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
    if ((uint64_t)numPixels > (uint64_t)RELMSE_NOALLOC_TILES * RELMSE_TILE)
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
    return relmseLaunch(sum, nSamples, ref, numPixels, out, scratch, (cudaStream_t)stream);
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
    const int rc = relmseLaunch(sum, nSamples, ref, numPixels, out, scratch, st);
    cudaFreeAsync(scratch, st);
    return rc;
}
