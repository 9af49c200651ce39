// Project-written autotuner for the wavefront tracer. It picks the launch
// and build parameters the reference leaves to OptiX (src/renderer.cpp:
// 441-513 builds the acceleration structure with OptiX's own choices): the
// BVH8 tree (PLOC, or the LBVH with its leaf size), the wavefront block size and the shading-queue compaction
// granularity, by timing each candidate on the caller's scene, then (plain
// sampling) the bounce from which the path-completion kernel takes over,
// with the chosen parameters. It is a client of the public C ABI (one
// renderer per candidate) plus CUDA events.
#include <cuda_runtime.h>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/optpt.h"

extern "C" int optpt_internal_set_error(int code, const char *msg);

namespace {

struct Timed {
    double samplesPerS = 0.0, mraysPerS = 0.0;
};

// Renders `warm` samples untimed, then times `spp` samples with CUDA events.
int timeCandidate(const optpt_scene *scene, const optpt_options &o, uint32_t w, uint32_t h, uint32_t warm,
                  uint32_t spp, int guiding, Timed &out)
{
    optpt_renderer *r = nullptr;
    int rc = optpt_create(scene, &o, &r);
    if (rc)
        return rc;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    do {
        if ((rc = optpt_setup_output_buffer(r, w, h)))
            break;
        if (guiding && (rc = optpt_set_guiding(r, guiding)))
            break;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
            rc = optpt_internal_set_error(OPTPT_ERR_CUDA, "autotune: stream/event creation failed");
            break;
        }
        if ((rc = optpt_render(r, warm, st)))
            break;
        optpt_stats s0{}, s1{};
        cudaStreamSynchronize(st);
        optpt_get_stats(r, &s0);
        cudaEventRecord(e0, st);
        if ((rc = optpt_render(r, spp, st)))
            break;
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            rc = optpt_internal_set_error(OPTPT_ERR_CUDA, "autotune: render failed");
            break;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        optpt_get_stats(r, &s1);
        const double sec = ms > 0.0f ? ms * 1e-3 : 1e-9;
        out.samplesPerS = (double)(s1.pathSamples - s0.pathSamples) / sec;
        out.mraysPerS =
            (double)((s1.extensionRays - s0.extensionRays) + (s1.shadowRays - s0.shadowRays)) / sec * 1e-6;
    } while (false);
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    if (st)
        cudaStreamDestroy(st);
    optpt_destroy(r);
    return rc;
}

}  // namespace

extern "C" int optpt_autotune(const optpt_scene *scene, const optpt_autotune_request *req, optpt_options *best,
                              optpt_autotune_trial *trials, uint32_t maxTrials, uint32_t *numTrials)
{
    if (!scene || !req || !best)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    if (req->width == 0 || req->height == 0 || req->spp == 0)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "autotune: width, height and spp must be positive");
    // the tree: the LBVH with leaves of up to one or two triangles, or PLOC
    // (its leaves hold one triangle)
    static const uint32_t trees[][2] = {{0, 1}, {0, 2}, {1, 1}};  // (bvhBuilder, leafSize)
    static const uint32_t blocks[] = {64, 128, 256};
    static const uint32_t compactions[] = {32, 1};
    double bestRate = -1.0;
    uint32_t n = 0;
    optpt_options chosen{};
    for (const auto &tree : trees)
        for (uint32_t blk : blocks)
            for (uint32_t comp : compactions) {
                optpt_options o{};
                o.bvhBuilder = tree[0];
                o.leafSize = tree[1];
                o.blockSize = blk;
                o.compaction = comp;
                o.useGraph = 1;
                o.bvhWidth = 8;
                Timed t;
                int rc = timeCandidate(scene, o, req->width, req->height, req->warmupSpp ? req->warmupSpp : 2,
                                       req->spp, (int)req->guiding, t);
                if (rc)
                    return rc;
                if (trials && n < maxTrials) {
                    trials[n].options = o;
                    trials[n].samplesPerS = t.samplesPerS;
                    trials[n].mraysPerS = t.mraysPerS;
                }
                ++n;
                if (t.samplesPerS > bestRate) {
                    bestRate = t.samplesPerS;
                    chosen = o;
                }
            }
    if (!req->guiding) {
        // the path-completion switch: never, or from one of these bounces
        static const uint32_t tails[] = {0xFFFFFFFFu, 3, 4, 5, 6, 8};
        const optpt_options base = chosen;
        for (uint32_t tb : tails) {
            optpt_options o = base;
            o.tailBounce = tb;
            Timed t;
            int rc = timeCandidate(scene, o, req->width, req->height, req->warmupSpp ? req->warmupSpp : 2, req->spp,
                                   0, t);
            if (rc)
                return rc;
            if (trials && n < maxTrials) {
                trials[n].options = o;
                trials[n].samplesPerS = t.samplesPerS;
                trials[n].mraysPerS = t.mraysPerS;
            }
            ++n;
            if (t.samplesPerS > bestRate) {
                bestRate = t.samplesPerS;
                chosen = o;
            }
        }
    }
    *best = chosen;
    if (numTrials)
        *numTrials = n;
    return OPTPT_OK;
}
