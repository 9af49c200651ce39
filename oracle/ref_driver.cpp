// Host build of the reference's own device headers, UNMODIFIED, behind a flat
// extern "C" surface. Compiled by oracle/build.py against the reference tree
// with the project-written stand-ins in oracle/ref_shim (OptiX typedef,
// float-vector operators, glm types, and a cuRAND replay generator).
//
// The query procedure mirrors the reference closest-hit program
// (cu/path_tracer.cu:231-370 for categorisation and the MaterialMetallicRoughness
// set-up, :400 for the BRDF evaluation used by next-event estimation, and
// :524-526 for BSDF sampling), in the same random-number order.
//
// This file is test infrastructure: it produces golden vectors that pin the
// oracle restatement; nothing in the product links it.
#include "principled_bsdf.h"
#include "tone_mapping.h"
#include "gamma_correction.h"
#include "barycentrics.h"
#include "light_sampling.cu"
#include "query_abi.h"

static inline float3 f3(const float *p) { return ::make_float3(p[0], p[1], p[2]); }
static inline void put3(double *d, float3 v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; }

extern "C" int ref_bsdf_query(const orc_bsdf_query *q, orc_bsdf_result *r, int n)
{
    for (int i = 0; i < n; ++i) {
        const orc_bsdf_query &Q = q[i];
        PRD prd{};
        curandState st{Q.xs, ORC_NXS, 0};
        prd.random.init(&st);
        prd.debug = false;

        MaterialData mat{};
        mat.ior = Q.ior;
        mat.roughness = Q.roughness;
        mat.metallic = Q.metallic;
        mat.specular = Q.specular;
        mat.transmissionWeight = Q.transmissionWeight;
        mat.subsurfaceWeight = Q.subsurfaceWeight;
        mat.coatWeight = Q.coatWeight;
        mat.coatRoughness = Q.coatRoughness;
        mat.sheenRoughness = Q.sheenRoughnessMat;
        mat.category = Q.category;

        const float3 n3 = f3(Q.n), wo = f3(Q.wo), wi = f3(Q.wi);
        const float3 albedo = f3(Q.baseColour), emission = f3(Q.emission), sheen = f3(Q.sheenColour);

        float categoryWeight = 1.0f;
        unsigned int category = categoriseMaterial(prd, mat, wo, n3, albedo, Q.roughness, Q.metallic, emission,
                                                   sheen, Q.sheenRoughness, categoryWeight);

        MaterialMetallicRoughness m;
        m.baseColour = albedo;
        m.ior = mat.ior;
        m.metallic = Q.metallic;
        m.specular = mat.specular;
        m.transmissionWeight = mat.transmissionWeight;
        m.subsurfaceWeight = mat.subsurfaceWeight;
        m.coatWeight = mat.coatWeight;
        m.sheenColour = sheen;
        m.type = 0;
        m.category = category;
        m.shadingNormal = n3;
        m.geometricNormal = n3;
        m.faceForwardNormal = n3;
        if (category & MaterialFlags::Coat) {
            m.roughness = mat.coatRoughness;
            m.alpha = mat.coatRoughness * mat.coatRoughness;
        } else if (category & MaterialFlags::Sheen) {
            m.roughness = mat.sheenRoughness;
            m.alpha = mat.sheenRoughness * mat.sheenRoughness;
        } else {
            m.roughness = Q.roughness;
            m.alpha = Q.roughness * Q.roughness;
        }
        m.alpha2 = m.alpha * m.alpha;

        orc_bsdf_result &R = r[i];
        R.category = category;
        R.categoryWeight = categoryWeight;
        if (category & MaterialFlags::Emission) {
            // The reference stops at an emitter before any BSDF work.
            R.f[0] = R.f[1] = R.f[2] = 0.0;
            R.dir[0] = R.dir[1] = R.dir[2] = 0.0;
            R.bsdf[0] = R.bsdf[1] = R.bsdf[2] = 0.0;
            R.pdf = 0.0;
            R.ret = 0;
            R.used = prd.random.state.used;
            continue;
        }
        float3 f = metallicRoughnessBrdf(prd, m, wi, wo);
        put3(R.f, f);

        BsdfSample s;
        s.newRayDir = ::make_float3(0.f, 0.f, 0.f);
        s.bsdf = ::make_float3(0.f, 0.f, 0.f);
        s.pdf = 0.f;
        float3 xi = prd.random.rng3();
        bool ok = metallicRoughnessSample(prd, m, wo, xi, s);
        s.pdf *= categoryWeight;
        put3(R.dir, s.newRayDir);
        put3(R.bsdf, s.bsdf);
        R.pdf = s.pdf;
        R.ret = ok ? 1 : 0;
        R.used = prd.random.state.used;
    }
    return 0;
}

// Tone mapping + gamma as the reference's raygen applies them
// (cu/device_programs.cu:84-96): impl 0 = Reinhard, 1 = ACES (Narkowicz).
extern "C" int ref_tonemap(const float *rgba_in, float *rgba_out, int n, int toneMapping, int impl,
                           int gammaCorrection, float gammaTerm)
{
    for (int i = 0; i < n; ++i) {
        float4 c = ::make_float4(rgba_in[4 * i], rgba_in[4 * i + 1], rgba_in[4 * i + 2], rgba_in[4 * i + 3]);
        float4 p;
        if (toneMapping)
            p = impl == 0 ? toneMapReinhard(c, 1.5f) : toneMapAcesNarkowicz(c);
        else
            p = c;
        if (gammaCorrection)
            p = linearToSrgb(p, gammaTerm);
        rgba_out[4 * i] = p.x; rgba_out[4 * i + 1] = p.y; rgba_out[4 * i + 2] = p.z; rgba_out[4 * i + 3] = p.w;
    }
    return 0;
}

// Punctual-light sampling via the reference's direct callable
// (cu/light_sampling.cu:61-81).
extern "C" int ref_light_sample(const orc_light *lights, const float *points, orc_light_sample *out, int n)
{
    for (int i = 0; i < n; ++i) {
        Light L{};
        L.type = (LightType)lights[i].type;
        L.radiance = f3(lights[i].radiance);
        L.p0 = f3(lights[i].p0);
        L.normal = f3(lights[i].normal);
        L.distance = lights[i].distance;
        L.cosWidth = lights[i].cosWidth;
        L.cosFalloffStart = lights[i].cosFalloffStart;
        LCG<8> unused;
        unused.state = 0;
        LightSample s{};
        __direct_callable__sampleLight(L, unused, f3(points + 3 * i), s);
        out[i].lightDir[0] = s.lightDir.x; out[i].lightDir[1] = s.lightDir.y; out[i].lightDir[2] = s.lightDir.z;
        out[i].radiance[0] = s.radiance.x; out[i].radiance[1] = s.radiance.y; out[i].radiance[2] = s.radiance.z;
        out[i].pdf = s.pdf;
        out[i].lightDist = s.lightDist;
    }
    return 0;
}

// Point / spot light construction (src/light.cpp:5-73) -> radiance field.
extern "C" int ref_create_light(int type, const float *a, const float *b, float w0, float w1, float wattage,
                                const float *colour, float *radiance_out, float *extra_out)
{
    Light L{};
    if (type == 0)
        L.createPointLight(f3(a), wattage, f3(colour));
    else if (type == 2)
        L.createSpotLight(f3(a), f3(b), w0, w1, wattage, f3(colour));
    else
        return -1;
    radiance_out[0] = L.radiance.x; radiance_out[1] = L.radiance.y; radiance_out[2] = L.radiance.z;
    extra_out[0] = L.cosWidth; extra_out[1] = L.cosFalloffStart;
    extra_out[2] = L.normal.x; extra_out[3] = L.normal.y; extra_out[4] = L.normal.z;
    return 0;
}

// Barycentrics of a point on a triangle (barycentrics.h:17-44).
extern "C" int ref_barycentric(const float *tri, const float *p, float *uvw, int n)
{
    for (int i = 0; i < n; ++i) {
        const float *t = tri + 9 * i;
        float u, v, w;
        calcBarycentric(f3(t), f3(t + 3), f3(t + 6), f3(p + 3 * i), u, v, w);
        uvw[3 * i] = u; uvw[3 * i + 1] = v; uvw[3 * i + 2] = w;
    }
    return 0;
}
