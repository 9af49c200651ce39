// Internal engine types shared by the build, wavefront and API translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "bvh.cuh"

struct Bvh8Node;  // bvh8.cuh

// Material record used by the shading kernels (derived from MaterialData at
// upload): 10 x 16 B, read with vector loads.
struct DevMaterial {
    float4 baseColour;      // rgb, alpha
    float4 emissionCutoff;  // emission rgb, alphaCutoff
    float4 sheen;           // sheenColour rgb, sheenRoughness
    float4 p0;              // ior, roughness, metallic, specular
    float4 p1;              // transmissionWeight, subsurfaceWeight, coatWeight, coatRoughness
    int4 flags;             // category, alphaMode, texture mask bits, 0
    int4 tex0;              // baseColour, normal, metallicRoughness, emissive texture ids
    int4 tex1;              // sheenColour, sheenRoughness texture ids, 0, 0
    float4 tf[6];           // (offset.xy, scale.xy) per texture slot
};
enum { TEXBIT_BASE = 1, TEXBIT_NORMAL = 2, TEXBIT_MR = 4, TEXBIT_EMISSIVE = 8, TEXBIT_SHEENC = 16, TEXBIT_SHEENR = 32 };

// Light record used by next-event estimation.
struct DevLight {
    float4 p0Type;       // p0.xyz, type (int bits)
    float4 radianceDist; // radiance.xyz, distance
    float4 normalCosW;   // normal.xyz, cosWidth
    float4 cosFalloff;   // cosFalloffStart, 0, 0, 0
};

struct DevScene {
    const BvhNode *nodes;   // BVH2 (used when nodes8 is null)
    const Bvh8Node *nodes8; // compressed BVH8
    const float4 *triV;  // 3 per triangle, leaf order of the BVH in use
    const int *triIndices;  // int3 per primitive (original order)
    const float *normals;   // float3 per vertex or null
    const float *texCoords; // float2 per vertex or null
    const DevMaterial *materials;
    const DevLight *lights;
    const float4 *emisV;    // 3 per emissive triangle
    const float2 *emisTc;   // 3 per emissive triangle
    const float4 *emisRad;  // radiance.xyz, material index bits
    const uint32_t *texels; // RGBA8 texels of all textures
    const int4 *texInfo;    // (first texel, width, height, wrapS | wrapT << 4 | srgb << 8)
    int numNodes;
    int numTris;
    int numLights;
    int numEmissive;
    int nodeBudget;  // BVH nodes one ray may visit; a walk cut short there is counted as a fault
};

// Per-frame constants, device resident and uploaded before every render (the
// reference uploads LaunchParams every frame, src/renderer.cpp:937), so camera
// or tone-mapping changes need no graph re-capture.
struct FrameConst {
    float4 eye;  // xyz; w = seed (uint bits)
    float4 U;    // xyz; w = vis (int bits)
    float4 V;    // xyz; w = toneMapping | toneMappingImpl << 1 | gammaCorrection << 2
    float4 W;    // xyz; w = gammaTerm
    float4 bg;   // xyz
};

// Learned guiding inside a pass (all null / 0 when guiding is off).
//   mix      : packed vMF mixture per queued extension ray (80 B), written by
//              the inference kernel after each extend
//   rec      : training records, GUIDE_REC float4 per (training path, depth)
//   batch    : training samples gathered at the end of the pass
struct GuidePass {
    const void *mix;
    float4 *rec;
    void *batch;
    uint32_t *batchCount;    // device
    uint32_t on;             // 1: guided sampling at guidable vertices
    uint32_t train;          // 1: record training vertices
    uint32_t trainStride;    // every trainStride-th path is a training path
    uint32_t batchCapacity;
    const uint32_t *step;    // device: training steps taken so far
    float alphaMin;          // floor on the probability of sampling the learned mixture
    float alphaMax;          // cap on the probability of sampling the learned mixture
    float alphaRamp;         // that probability is min(alphaMax, min(1, steps / alphaRamp) * network's)
    uint32_t maxDepth;       // vertices deeper than this sample the BSDF only
    uint32_t sharePrimary;   // 1: a pass's first hits of one pixel share one mixture (its first sample's)
};
#define GUIDE_REC 7

// Training paths: one per group of `stride` consecutive paths, at an offset
// drawn per group and per pass, so every pixel contributes over passes.
__host__ __device__ inline uint32_t guideTrainOffset(uint32_t group, uint32_t stamp, uint32_t stride)
{
    uint32_t h = group * 0x9E3779B1u ^ stamp * 0x85EBCA77u;
    h ^= h >> 16;
    h *= 0x7FEB352Du;
    h ^= h >> 15;
    h *= 0x846CA68Bu;
    h ^= h >> 16;
    return h % stride;
}

// Batched multi-view rendering: the pixels of all views are concatenated
// (view v owns global pixels first .. first + width * height - 1). A pass
// renders `dyn[1]` samples for each of the `dyn[0]` active global pixels in
// `pixelList`; path p is sample p / dyn[0] of pixel pixelList[p % dyn[0]].
struct BatchView {
    float4 eye;  // xyz; w = width (uint bits)
    float4 U;    // xyz; w = height (uint bits)
    float4 V;    // xyz; w = first global pixel (uint bits)
    float4 W;    // xyz; w = samples accumulated before this pass (uint bits)
};
struct BatchPass {
    const BatchView *views;
    const uint32_t *pixelList;  // active global pixels of this pass
    const uint16_t *pixelView;  // view of every global pixel
    const uint32_t *dyn;        // [0] active pixels, [1] samples per active pixel
    uint32_t on;
};

// Launch-shape parameters baked into a captured pass.
struct FrameParams {
    uint32_t w, h, npix, sppBatch, numPaths;
    uint32_t maxDepth;
    const uint32_t *state;   // device: [0] = samples accumulated before this pass, [1] = passes run
    const FrameConst *fc;    // device
    GuidePass guide;
    BatchPass batch;
};

// Global pixel (the RNG's pixel key) and sample index of a path.
__device__ __forceinline__ void pathPixelSample(const FrameParams &fp, uint32_t path, uint32_t &pixel,
                                                uint32_t &sample)
{
    if (fp.batch.on) {
        const uint32_t n = __ldg(fp.batch.dyn);
        pixel = __ldg(fp.batch.pixelList + path % n);
        const uint32_t v = __ldg(fp.batch.pixelView + pixel);
        sample = __float_as_uint(__ldg(&fp.batch.views[v].W).w) + path / n;
    } else {
        pixel = path % fp.npix;
        sample = __ldg(fp.state) + path / fp.npix;
    }
}
// Paths of this pass (device-resident in batch mode).
__device__ __forceinline__ uint32_t passPaths(const FrameParams &fp)
{
    return fp.batch.on ? __ldg(fp.batch.dyn) * __ldg(fp.batch.dyn + 1) : fp.numPaths;
}

// Device counters: per-depth queue lengths. Depth d uses index d.
#define CNT_EXT 0
#define CNT_SHADOW_P 64
#define CNT_SHADOW_E 128
// next unclaimed ray of each extension queue (persistent warps with lane refill)
#define CNT_FETCH_EXT 192
#define CNT_TOTAL 256
#define OPT_MAX_DEPTH 62
#define TOTALS_COUNT 10  // entries of WaveBufs::totals

// Wavefront buffers (SoA; P = numPaths):
//   pathT/pathL : float4 per path (throughput + flags, radiance)
//   rayO/rayD   : two ping-pong ray queues, float4 (origin, path id) and (dir, -)
//   hit         : float4 (t, u, v, leaf) per queued ray
//   shO/shD/shC : two shadow queues (point lights, emissive triangles):
//                 (origin, path id), (dir, tmax), (contribution, blend xi)
struct WaveBufs {
    float4 *pathT, *pathL;
    float4 *rayO[2], *rayD[2];
    float4 *hit;
    float4 *shO[2], *shD[2], *shC[2];
    uint32_t *counters;              // CNT_TOTAL entries
    unsigned long long *totals;      // 0 ext rays, 1 shadow rays, 2 samples, 3 NaN samples,
                                     // 4-5 ext nodes/tris, 6-7 shadow nodes/tris (counting mode),
                                     // 8 traversal stack overflows, 9 walks cut short by the node budget
};

// FP64 per-pixel accumulator (xyz used), 32-byte aligned for vector access.
struct alignas(32) Acc4 {
    double x, y, z, w;
};

struct AccumBufs {
    Acc4 *sum, *sumSq;
    float4 *frameBuffer, *accumFrameBuffer;
};

struct LaunchShape {
    int gridGenerate, gridExtend, gridShade, gridShadow, gridAccum, gridFinish;
    int block;
    int compaction;  // shading-queue appends: 0 one atomic per warp, 1 one per block
};

// wavefront.cu
void launchGenerate(const LaunchShape &ls, const FrameParams &fp, const WaveBufs &q, cudaStream_t st);
// count = true runs the counting variant (BVH nodes and triangles visited
// added to totals[4..5] for extension rays, totals[6..7] for shadow rays).
void launchExtend(const LaunchShape &ls, const DevScene &s, const FrameParams &fp, const WaveBufs &q, int depth,
                  cudaStream_t st, bool count = false);
void launchShade(const LaunchShape &ls, const DevScene &s, const FrameParams &fp, const WaveBufs &q, int depth,
                 cudaStream_t st);
void launchShadow(const LaunchShape &ls, const DevScene &s, const FrameParams &fp, const WaveBufs &q, int depth,
                  int which, cudaStream_t st, bool count = false);
// The rest of every path from bounce depth0 on, in one launch (plain
// sampling; 128-thread blocks): closest hit, shading and shadow rays per
// bounce, bit-identical to the per-bounce kernels.
void launchFinish(const LaunchShape &ls, const DevScene &s, const FrameParams &fp, const WaveBufs &q, int depth0,
                  cudaStream_t st, bool count = false);
void launchAccumulate(const LaunchShape &ls, const FrameParams &fp, const WaveBufs &q, const AccumBufs &a,
                      cudaStream_t st);
void launchAdvance(const FrameParams &fp, uint32_t *state, cudaStream_t st);
void launchCopyFrame(const float4 *src, float4 *dst, size_t n, cudaStream_t st);
// Traversal faults of the traced rays are added to totals[8], totals[9].
void launchTrace(const DevScene &s, const float4 *rays, float4 *hits, uint32_t n, int anyHit,
                 unsigned long long *totals, cudaStream_t st);
void launchBsdfBatch(const void *queries, void *results, uint32_t n, cudaStream_t st);
// guide.cu: inference over the extension queue of `depth` (after extend), and
// the end-of-pass gather of training samples from the records.
struct optpt_guide;
void launchGuideInfer(const optpt_guide *g, const DevScene &s, const FrameParams &fp, const WaveBufs &q, int depth,
                      cudaStream_t st);
void launchGuideGather(const FrameParams &fp, const WaveBufs &q, cudaStream_t st);
int occupancyGrid(int kernelId, int block);  // persistent grid for a kernel class
// Vertex deformation and emissive-vertex regather (deform.cu).
void launchDeform(uint32_t nv, const float *restP, const float *restN, const uint32_t *vShape, const void *joints,
                  const void *weights, const float *shapeM, const float *shapeN, const float *jointM,
                  uint32_t numShapes, uint32_t numJoints, float *outP, float *outN, cudaStream_t st);
void launchEmissiveVerts(int numEmis, const int *emisPrim, const float *pos, const int *idx, int numTris,
                         float4 *emisV, cudaStream_t st);
// Frame output payloads (image_out.cu): any output pointer may be null.
void launchImageOut(const float4 *fb, const float4 *mean, uint32_t w, uint32_t h, uint32_t *rgba8, uint32_t *rgbe,
                    void *halfRows, cudaStream_t st);

// bvh_build.cu, bvh8_build.cu
struct Bvh8Node;
struct BvhBuild {
    BvhNode *nodes;        // n - 1 slots (holes where subtrees collapsed to leaves)
    float4 *triV;          // 3 * n, BVH2 leaf (Morton) order
    uint32_t *mortonSorted;
    int *primOrder;
    int numNodes;          // slots allocated
    int usedNodes;         // internal nodes emitted
    int numLeaves;
    Bvh8Node *nodes8;      // compressed 8-wide BVH (null until collapsed)
    float4 *triV8;         // 3 * n, BVH8 leaf order
    int numNodes8;
    int levels8;
    int levelOff8[258];    // first node of each BVH8 level; [levels8] = numNodes8
    float *box8;           // refit: full-precision box (lo xyz, hi xyz) per BVH8 node (lazy)
};
// Collapses the BVH2 of `b` into b.nodes8 / b.triV8 (leaf sizes <= 4).
int buildBvh8(BvhBuild &b, int numTris, cudaStream_t st);
// Builds the BVH2 on `st`: the LBVH, or with `ploc` the PLOC tree on the same
// Morton order (leaves of one triangle; leafSize ignored). positions /
// triIndices / matIndices are device arrays; triFlags (device, per primitive)
// go to triV[3i+2].w. Returns 0 or a CUDA error.
int buildBvh(const float *positions, const int *triIndices, const int *matIndices, const uint32_t *triFlags,
             int numTris, int leafSize, BvhBuild &out, cudaStream_t st, bool ploc = false);
void freeBvh(BvhBuild &b);
// Refits the BVH8 in place after the vertex positions changed: triangle
// records regathered, then every level's quantised child boxes recomputed
// from the deepest level up; topology, slots and leaf layout kept. Enqueued
// on `st` without host synchronisation (capturable). 0 or a CUDA error.
int refitBvh8(BvhBuild &b, const float *positions, const int *triIndices, int numTris, cudaStream_t st);
