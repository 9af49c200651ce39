/* Flat record layouts shared by the oracle restatement (oracle_capi.cpp) and
 * the reference host build (ref_driver.cpp). Tests fill these from numpy
 * structured arrays of the same layout. Plain C, 4-byte fields only. */
#pragma once
#include <stdint.h>

#define ORC_NXS 12

/* One BSDF query: the hit-point material state that the reference's
 * closest-hit program hands to categoriseMaterial / metallicRoughnessBrdf /
 * metallicRoughnessSample (path_tracer.cu:165-370), plus the uniforms those
 * functions draw, in the order they draw them. */
typedef struct {
    float baseColour[3];       /* albedo after the base-colour texture       */
    float emission[3];         /* emission after the emissive texture        */
    float sheenColour[3];      /* sheen colour after its texture             */
    float metallic;            /* after the metallic-roughness texture       */
    float roughness;           /* after the metallic-roughness texture       */
    float specular;            /* MaterialData.specular                      */
    float transmissionWeight;  /* MaterialData.transmissionWeight            */
    float subsurfaceWeight;    /* MaterialData.subsurfaceWeight              */
    float coatWeight;          /* MaterialData.coatWeight                    */
    float coatRoughness;       /* MaterialData.coatRoughness                 */
    float sheenRoughnessMat;   /* MaterialData.sheenRoughness                */
    float sheenRoughness;      /* sheen roughness after its texture          */
    float ior;                 /* MaterialData.ior                           */
    uint32_t category;         /* MaterialData.category (0 = Uncategorised)  */
    float n[3];                /* shading normal                             */
    float wo[3];               /* v = -rayDir                                */
    float wi[3];               /* l, the direction evaluated by the BRDF     */
    float xs[ORC_NXS];         /* uniforms, consumed front to back           */
} orc_bsdf_query;

/* Result of one query, in the precision of the implementation. */
typedef struct {
    uint32_t category;
    int32_t ret;               /* metallicRoughnessSample's return value     */
    int32_t used;              /* uniforms consumed by the whole query       */
    int32_t pad;
    double categoryWeight;
    double f[3];               /* metallicRoughnessBrdf(l = wi, v = wo)      */
    double dir[3];             /* sampled direction                          */
    double bsdf[3];            /* sampled BSDF value                         */
    double pdf;                /* sample pdf times categoryWeight            */
} orc_bsdf_result;

/* A punctual light in the reference's Light layout subset used by sampling. */
typedef struct {
    int32_t type;              /* LightType: 0 point, 1 directional, 2 spot  */
    float radiance[3];
    float p0[3];
    float normal[3];
    float distance;
    float cosWidth;
    float cosFalloffStart;
} orc_light;

typedef struct {
    float lightDir[3];
    float radiance[3];
    float pdf;
    float lightDist;
} orc_light_sample;
