/* Frame contract: the reference's LaunchParams (include/launch_params.h:16-48)
 * with the same field names and meaning. `traversable` is the renderer's BVH
 * handle instead of an OptiX handle; `randState` is kept for layout only
 * (random numbers are counter-based and need no per-pixel state). The fields
 * after `gammaTerm` are additions: the reference compiles the path depth in
 * (MAX_DEPTH, cuda_utils.h:5) and stores the background colour in its miss
 * record (sbt_record.h:12-15). */
#pragma once
#include <stdint.h>
#include "light.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct LaunchParams {
    float *frameBuffer;      /* device float4 w*h: tone-mapped, gamma-encoded */
    float *accumFrameBuffer; /* device float4 w*h: running mean radiance      */
    uint32_t w;
    uint32_t h;

    uint32_t sample; /* samples accumulated so far */
    uint32_t seed;

    float eye[3];
    float U[3];
    float V[3];
    float W[3];

    uint64_t traversable;

    Light *lights;
    uint32_t numLights;

    uint32_t numEmissiveTriangles;

    void *randState;

    int32_t vis;

    int32_t toneMapping;     /* bool in the reference */
    int32_t toneMappingImpl; /* 0 = Reinhard, 1 = ACES (Narkowicz) */

    int32_t gammaCorrection; /* bool in the reference */
    float gammaTerm;

    uint32_t maxDepth;    /* reference: MAX_DEPTH = 8 */
    float bgColour[3];    /* reference: MissData.colour */
} LaunchParams;

#ifdef __cplusplus
}
#endif
