// The guiding network's device state and the launchers the renderer calls.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cstdint>
#include "guide.cuh"

struct optpt_guide {
    guide::Levels levels{};
    float lo[3] = {0, 0, 0}, invExt[3] = {1, 1, 1};  // world -> unit cube
    // parameters: FP32 masters, the FP16 hash copy and the BF16 weight tiles
    float *mlp = nullptr;     // [LAYERS][64 out][64 in]
    uint8_t *tiles = nullptr; // 2 * LAYERS tiles of 8 KB: W_l (rows out) then W_l^T (rows in)
    float *hash = nullptr;    // [LEVELS][TABLE][FEATS]
    __half *hashH = nullptr;  // FP16 pair copy: slot e = (entry e, entry e + 1) of its level
    // gradients and Adam moments
    float *gMlp = nullptr, *gHash = nullptr;
    float *mMlp = nullptr, *vMlp = nullptr, *mHash = nullptr, *vHash = nullptr;
    double *stats = nullptr;  // [0] sum of normalised weights, [1] loss sum, [2] samples
    int *status = nullptr;    // device: non-zero if a tensor-core wait expired
    uint32_t *dStep = nullptr;  // device: Adam step count
    float lr = 1e-2f;
    int numSMs = 0;
    int lobeLoss = 1;  // 1: lobes fit the whole target (-c log q); 0: what the BSDF leaves (mixture loss)
};

// Unit-cube mapping and level table as passed to kernels.
struct GuideGeom {
    guide::Levels levels;
    float3 lo, invExt;
    int lobeLoss;
};

// One training sample: (pos.xyz, weight), (n.xyz, -), (wo.xyz, BSDF lobe
// density at wi), (wi.xyz, -).
// Weight = target radiance estimate / sampling pdf of wi (the batch is
// normalised by the sum of weights before the gradient).
struct GuideSample {
    float4 pos, n, wo, wi;
};

// Shading-point queries for inference: (pos, -), (n, -), (wo, -).
struct GuideQuery {
    float4 pos, n, wo;
};

int guideCreate(optpt_guide *g, const float lo[3], const float hi[3], uint32_t seed);
void guideFree(optpt_guide *g);
GuideGeom guideGeom(const optpt_guide *g);
// Packed mixtures (80 B each) for n queries.
cudaError_t guideInferQueries(const optpt_guide *g, const GuideQuery *q, uint32_t n, guide::Packed *out,
                              cudaStream_t s);
// Gradients of the batch into gMlp / gHash (accumulated; zeroed by Adam).
// Slice `slice` of `slices` equal parts of the batch (one minibatch).
cudaError_t guideGradients(optpt_guide *g, const GuideSample *smp, const uint32_t *count, uint32_t capacity,
                           cudaStream_t s, uint32_t slice = 0, uint32_t slices = 1);
cudaError_t guideAdam(optpt_guide *g, cudaStream_t s);
