/* Punctual lights: the reference's Light record (include/light.h:11-46 of
 * markcmagro/optix_pt) with the same field names, order and meaning, float3
 * fields spelled as float[3] so the header is plain C. For a point light,
 * `radiance` holds the intensity (W/sr), as the reference's createPointLight
 * stores it (src/light.cpp:5-12). */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { LIGHT_TYPE_POINT = 0, LIGHT_TYPE_DIRECTIONAL = 1, LIGHT_TYPE_SPOT = 2 };

typedef struct Light {
    int32_t type;       /* LightType                                    */
    float radiance[3];  /* all; intensity for point and spot lights     */
    float colour[3];
    float power[3];     /* watts x colour                               */
    float p0[3];        /* all: position (point, spot)                  */
    float p1[3];
    float p2[3];
    float normal[3];    /* directional: direction of travel; spot: axis */
    float v1[3];
    float v2[3];
    float area;
    float radius;
    float distance;     /* directional                                  */
    float widthRad;     /* spot                                         */
    float cosWidth;     /* spot                                         */
    float cosFalloffStart; /* spot                                      */
} Light;

#ifdef __cplusplus
}
#endif
