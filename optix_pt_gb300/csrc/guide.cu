// Learned path guiding: a hash-grid encoded MLP on the fifth-generation
// tensor cores. This file holds the tensor-core operand self-test; the
// network kernels build on the same helpers (tc.cuh).
#include <cuda_runtime.h>
#include <cstdint>
#include "optpt.h"
#include "tc.cuh"

extern "C" int optpt_internal_set_error(int code, const char *msg);

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

// Tensor-core operand self-test (no counterpart in the reference; it checks
// this library's tcgen05 descriptors and TMEM layouts). Device pointers:
// A[128][64], B[64][64], G[128][64], X[128][64] BF16 bits; c[128][64],
// dwRaw[128][64] FP32; status: one int, set to 1 if the MMA wait expired.
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
