// Device (FP32) glTF metallic-roughness BSDF: categorisation, evaluation and
// sampling, following the reference's formulas and their evaluation order
// (include/principled_bsdf.h:25-961 and the helpers it includes). Each routine
// cites the reference function it reproduces. Uniforms come from a source `U`
// with `float next()`: the path's PCG stream in the integrator, or an explicit
// list in the parity entry point.
#pragma once
#include "common.cuh"
#include "../../include/optix_pt/material_data.h"

namespace bsdf {

// MaterialMetallicRoughness (include/material_metallic_roughness.h:3-23),
// reduced to the fields the BSDF reads.
struct MatMR {
    float3 baseColour;
    float3 sheenColour;
    float3 n;  // shading normal
    float ior, metallic, alpha, alpha2;
    uint32_t category;
};

struct Sample {
    float3 dir;
    float3 bsdf;
    float pdf;
};

// calcF0 (principled_bsdf_helpers.h:7-11)
OPT_D float calcF0(float ior)
{
    float t = (1.0f - ior) / (1.0f + ior);
    return t * t;
}
// fresnelPowerTerm / fresnelSchlick (schlick.h:6-23)
OPT_D float schlickPow(float vDotH) { return powf(1.0f - fabsf(vDotH), 5.0f); }
OPT_D float schlick(float f0, float vDotH) { return f0 + (1.0f - f0) * schlickPow(vDotH); }

// reflectRay / refractRay (reflection_and_refraction.h:5-48)
OPT_D float3 reflectRay(float3 n, float3 i) { return -i + (2.0f * dot3(n, i)) * n; }
OPT_D float3 refractRay(float3 n, float3 i, float eta)
{
    float c = dot3(n, i);
    if (c < 0.0f) {
        eta = 1.0f / eta;
        c = -c;
        n = -n;
    }
    float sin2i = fmaxf(0.0f, 1.0f - c * c);
    float sin2t = sin2i / (eta * eta);
    if (sin2t >= 1.0f)
        return reflectRay(n, i);
    float cosT = sqrtf(fmaxf(0.0f, 1.0f - sin2t));
    return -i / eta + (c / eta - cosT) * n;
}
// transmissionHalfVectorVolumetric (reflection_and_refraction.h:69-97)
OPT_D float3 halfVolumetric(float3 n, float3 l, float3 v, float etaI, float etaV)
{
    if (dot3(n, v) < 0.0f) {
        float t = etaI;
        etaI = etaV;
        etaV = t;
    }
    return normalize3(-(etaI * v + etaV * l));
}

// OrthonormalBasis::localToWorld (orthonormal_basis.h:11-41)
OPT_D float3 onbToWorld(float3 n, float3 p)
{
    float3 b = fabsf(n.x) > fabsf(n.z) ? mk3(-n.y, n.x, 0.0f) : mk3(0.0f, -n.z, n.y);
    b = normalize3(b);
    float3 t = cross3(b, n);
    return p.x * t + p.y * b + p.z * n;
}

// ---------------------------------------------------------------- microfacet
// trowbridgeReitzD (trowbridge_reitz.h:12-26)
OPT_D float ggxD(float nDotH, float alpha)
{
    if (nDotH <= 0.0f)
        return 0.0f;
    float a2 = fmaxf(0.00001f, alpha * alpha);
    float t = nDotH * nDotH * (a2 - 1.0f) + 1.0f;
    return a2 / (OPT_PI * t * t);
}
// trowbridgeReitzGetHalfVector (trowbridge_reitz.h:28-47)
OPT_D float3 ggxHalf(float alpha2, float3 n, float x, float y)
{
    float theta = acosf(sqrtf((1.0f - x) / ((alpha2 - 1.0f) * x + 1.0f)));
    float phi = 2.0f * OPT_PI * y;
    float st, ct, sp, cp;
    sincosf(theta, &st, &ct);
    sincosf(phi, &sp, &cp);
    return onbToWorld(n, mk3(st * cp, st * sp, ct));
}
// trowbridgeReitzPdf (trowbridge_reitz.h:49-63)
OPT_D float ggxPdf(float3 n, float3 h, float3 v, float alpha)
{
    float nDotH = dot3(n, h);
    float D = ggxD(nDotH, alpha);
    return (D * nDotH) / (4.0f * fabsf(dot3(h, v)));
}
// smithV (smith.h:35-52)
OPT_D float smithV(float hDotL, float nl, float hDotV, float nv, float alpha)
{
    if (hDotL <= 0.0f || hDotV <= 0.0f)
        return 0.0f;
    float a2 = alpha * alpha;
    float t1 = nl + sqrtf(a2 + (1.0f - a2) * nl * nl);
    float t2 = nv + sqrtf(a2 + (1.0f - a2) * nv * nv);
    return 1.0f / (t1 * t2);
}

// ---------------------------------------------------------------- sheen (sheen.h:16-46)
OPT_D float charlieD(float nDotH, float a)
{
    float invR = 1.0f / a;
    float sin2 = 1.0f - nDotH * nDotH;
    return (2.0f + invR) * powf(sin2, invR * 0.5f) * (0.5f * OPT_INV_PI);
}
OPT_D float lerpS(float a, float b, float t) { return a + t * (b - a); }
OPT_D float sheenL(float x, float a)
{
    float t = (1.0f - a) * (1.0f - a);
    float A = lerpS(21.5473f, 25.3245f, t);
    float B = lerpS(3.82987f, 3.32435f, t);
    float C = lerpS(0.19823f, 0.16801f, t);
    float D = lerpS(-1.97760f, -1.27393f, t);
    float E = lerpS(-4.32054f, -4.85967f, t);
    return A / (1.0f + B * powf(x, C)) + D * x + E;
}
OPT_D float sheenLambda(float c, float a)
{
    if (fabsf(c) < 0.5f)
        return expf(sheenL(c, a));
    return expf(2.0f * sheenL(0.5f, a) - sheenL(1.0f - c, a));
}
OPT_D float charlieV(float nv, float nl, float a)
{
    return 1.0f / ((1.0f + sheenLambda(nv, a) + sheenLambda(nl, a)) * (4.0f * nv * nl));
}

// ---------------------------------------------------------------- lobes
// evalOrenNayar (oren_nayar.h:15-59)
OPT_D float3 orenNayar(const MatMR &m, float3 l, float3 v)
{
    float sigma = 0.7071067f * atanf(m.alpha);
    float nDotV = fminf(fmaxf(0.00001f, dot3(m.n, v)), 1.0f);
    float nDotL = fminf(fmaxf(0.00001f, dot3(m.n, l)), 1.0f);
    float thetaV = acosf(nDotV), thetaL = acosf(nDotL);
    float a = fmaxf(thetaV, thetaL), b = fminf(thetaV, thetaL);
    float3 lp = l - nDotL * m.n, vp = v - nDotV * m.n;
    float cosPhi = dot3(normalize3(vp), normalize3(lp));
    float s2 = sigma * sigma;
    float A = 1.0f - 0.5f * (s2 / (s2 + 0.33f));
    float B = 0.45f * (s2 / (s2 + 0.09f));
    float on = A + B * fmaxf(0.0f, cosPhi) * sinf(a) * tanf(b);
    float3 refl = m.baseColour * (1.0f - m.metallic);
    return refl * (on * OPT_INV_PI * dot3(m.n, l));
}
// diffuseBrdf (principled_bsdf.h:253-264)
OPT_D float3 diffuseBrdf(const MatMR &m, float3 l, float3 v)
{
    if (m.category & MF_LAMBERTIAN)
        return m.baseColour * OPT_INV_PI;
    return orenNayar(m, l, v);
}
// cosineSampleHemisphere (sampling.h:27-42) around n
OPT_D float3 cosineDir(float3 n, float x, float y)
{
    float r = sqrtf(x);
    float phi = y * 2.0f * OPT_PI;
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float px = r * cp, py = r * sp;
    float z = sqrtf(fmaxf(0.0f, 1.0f - px * px - py * py));
    return onbToWorld(n, mk3(px, py, z));
}
// diffuseSample (principled_bsdf.h:245-279)
OPT_D bool diffuseSample(const MatMR &m, float3 v, float x, float y, Sample &s)
{
    s.dir = cosineDir(m.n, x, y);
    s.bsdf = diffuseBrdf(m, s.dir, v);
    s.pdf = dot3(m.n, s.dir) * OPT_INV_PI;
    return true;
}
// reflectionGetNewRayDir (principled_bsdf.h:384-406)
OPT_D float3 reflectionDir(const MatMR &m, float3 v, float x, float y)
{
    if (m.category & MF_SPECULAR)
        return reflectRay(m.n, v);
    return reflectRay(ggxHalf(m.alpha2, m.n, x, y), v);
}
// reflectionBrdf (principled_bsdf.h:408-458)
OPT_D float3 reflectionBrdf(const MatMR &m, float3 l, float3 v)
{
    if (m.category & MF_SPECULAR)
        return m.baseColour / fabsf(dot3(l, m.n));
    float3 h = normalize3(l + v);
    float nl = fmaxf(fabsf(dot3(m.n, l)), 0.00001f);
    float nv = fmaxf(fabsf(dot3(m.n, v)), 0.00001f);
    float V = smithV(dot3(h, l), nl, dot3(h, v), nv, m.alpha);
    float D = ggxD(dot3(m.n, h), m.alpha);
    return mk3s(V * D);
}
// reflectionPdf (principled_bsdf.h:462-481)
OPT_D float reflectionPdf(const MatMR &m, float3 l, float3 v)
{
    if (m.category & MF_SPECULAR)
        return 1.0f;
    return ggxPdf(m.n, normalize3(l + v), v, m.alpha);
}
// specularReflectionSample (principled_bsdf.h:285-292)
OPT_D bool specReflSample(const MatMR &m, float3 wo, Sample &s)
{
    s.dir = reflectRay(m.n, wo);
    s.bsdf = m.baseColour / fabsf(dot3(s.dir, m.n));
    s.pdf = 1.0f;
    return true;
}
// reflectionSample (principled_bsdf.h:483-520)
OPT_D bool reflectionSample(const MatMR &m, float3 v, float x, float y, Sample &s)
{
    if (m.category & MF_SPECULAR)
        return specReflSample(m, v, s);
    s.dir = reflectionDir(m, v, x, y);
    float3 h = normalize3(s.dir + v);
    if (dot3(s.dir, h) > 0.0f && dot3(s.dir, m.n) > 0.0f) {
        s.pdf = reflectionPdf(m, s.dir, v);
        s.bsdf = reflectionBrdf(m, s.dir, v);
        return true;
    }
    s.bsdf = mk3s(0.0f);
    s.pdf = 0.0f;
    return false;
}
// transmissionBrdf (principled_bsdf.h:560-597)
OPT_D float3 transmissionBrdf(const MatMR &m, float3 l, float3 v)
{
    if (m.category & MF_SPECULAR)
        return m.baseColour / fabsf(dot3(m.n, l));
    float3 h = halfVolumetric(m.n, l, v, 1.0f, 1.5f);
    float hl = dot3(h, l) / dot3(m.n, l);
    float hv = dot3(h, v) / dot3(m.n, v);
    float nl = fmaxf(fabsf(dot3(m.n, l)), 0.00001f);
    float nv = fmaxf(fabsf(dot3(m.n, v)), 0.00001f);
    float V = smithV(hl, nl, hv, nv, m.alpha);
    float D = ggxD(dot3(m.n, h), m.alpha);
    return mk3s(V * D);
}
// transmissionPdf (principled_bsdf.h:599-619)
OPT_D float transmissionPdf(const MatMR &m, float3 l, float3 v)
{
    if (m.category & MF_SPECULAR)
        return 1.0f;
    return ggxPdf(m.n, halfVolumetric(m.n, l, v, 1.0f, 1.5f), v, m.alpha);
}
// transmissionSample (principled_bsdf.h:621-632), specular branch
// specularTransmissionSample (:298-339)
OPT_D bool transmissionSample(const MatMR &m, float3 v, float x, float y, Sample &s)
{
    if (m.category & MF_SPECULAR) {
        s.dir = refractRay(m.n, v, m.ior);
        s.bsdf = m.baseColour / fabsf(dot3(m.n, s.dir));
        s.pdf = 1.0f;
        return true;
    }
    s.dir = refractRay(ggxHalf(m.alpha2, m.n, x, y), v, m.ior);
    s.bsdf = transmissionBrdf(m, s.dir, v);
    s.pdf = transmissionPdf(m, s.dir, v);
    return true;
}
// metalBrdf (principled_bsdf.h:748-762) + conductorFresnel (principled_bsdf_helpers.h:24-31)
OPT_D float3 metalBrdf(const MatMR &m, float3 l, float3 v)
{
    float3 fs = reflectionBrdf(m, l, v);
    float3 h = normalize3(l + v);
    float p = schlickPow(dot3(v, h));
    return fs * (m.baseColour + (mk3s(1.0f) - m.baseColour) * p);
}
// sheenBrdf (principled_bsdf.h:797-826)
OPT_D float3 sheenBrdf(const MatMR &m, float3 l, float3 v)
{
    if (m.category & MF_SPECULAR)
        return m.sheenColour / fabsf(dot3(l, m.n));
    float3 h = normalize3(l + v);
    float V = charlieV(dot3(h, v), dot3(h, l), m.alpha);
    float D = charlieD(dot3(m.n, h), m.alpha);
    return m.sheenColour * (V * D) / fabsf(dot3(m.n, v));
}

// metallicRoughnessBrdf (principled_bsdf.h:866-898) with dielectricBrdf
// (:638-681), which draws one uniform for transmissive materials (:649).
// The reference's branches pick a lobe first; each lobe is then evaluated at
// one place in the code (the shading kernel's speed is bound by instruction
// fetch, and every inlined copy of a lobe adds to what it fetches).
template <class U> OPT_D float3 evalBrdf(const MatMR &m, float3 l, float3 v, U &u)
{
    const uint32_t c = m.category;
    int lobe = 4;  // 0 GGX / mirror reflection, 1 transmission, 2 diffuse, 3 sheen, 4 none
    if (c & MF_METAL) {
        lobe = 0;
    } else if (c & MF_DIELECTRIC) {
        if (c & MF_TRANSMISSION) {
            float F = schlick(calcF0(m.ior), dot3(v, m.n));
            float xi = u.next();
            lobe = xi < F ? 0 : 1;
        } else {
            lobe = (c & MF_REFLECTION) ? 0 : 2;
        }
    } else if (c & MF_COAT) {
        lobe = 0;
    } else if (c & MF_SHEEN) {
        lobe = 3;
    }
    if (lobe == 0) {
        const float3 fs = reflectionBrdf(m, l, v);
        if (!(c & MF_METAL))
            return fs;
        // metalBrdf (principled_bsdf.h:748-762): conductor Fresnel on top
        const float3 h = normalize3(l + v);
        const float p = schlickPow(dot3(v, h));
        return fs * (m.baseColour + (mk3s(1.0f) - m.baseColour) * p);
    }
    if (lobe == 1)
        return transmissionBrdf(m, l, v);
    if (lobe == 2)
        return diffuseBrdf(m, l, v);
    if (lobe == 3)
        return sheenBrdf(m, l, v);
    return mk3(1.0f, 0.0f, 1.0f);
}

// metallicRoughnessSample (principled_bsdf.h:902-961) with metalSample
// (:769-785), dielectricSample (:683-735), sheenSample (:852-859); lobe first,
// as in evalBrdf. Metal and sheen take reflectionDir's direction without
// reflectionSample's validity test, as the reference does.
template <class U> OPT_D bool sampleBrdf(const MatMR &m, float3 wo, float3 xi, U &u, Sample &s)
{
    const uint32_t c = m.category;
    // 0 metal, 1 GGX / mirror reflection, 2 transmission, 3 diffuse, 4 sheen, 5 none
    int lobe = 5;
    bool fresnelSplit = false;  // transmissive dielectric: reflection F, transmission 1 - F
    float F = 0.0f;
    if (c & MF_METAL) {
        lobe = 0;
    } else if (c & MF_DIELECTRIC) {
        if (c & MF_TRANSMISSION) {
            F = schlick(fminf(calcF0(m.ior), 1.0f), dot3(wo, m.n));
            float r1 = u.next();
            fresnelSplit = true;
            lobe = r1 < F ? 1 : 2;
        } else {
            lobe = (c & MF_REFLECTION) ? 1 : 3;
        }
    } else if (c & MF_COAT) {
        lobe = 1;
    } else if (c & MF_SHEEN) {
        lobe = 4;
    }
    bool ret = true;
    if (lobe == 1 && (c & MF_SPECULAR)) {
        ret = specReflSample(m, wo, s);
    } else if (lobe == 0 || lobe == 1 || lobe == 4) {
        s.dir = reflectionDir(m, wo, xi.x, xi.y);
        if (lobe == 4) {
            s.bsdf = sheenBrdf(m, s.dir, wo);
            s.pdf = 1.0f;
        } else {
            // reflectionSample (principled_bsdf.h:483-520) rejects directions
            // below the surface or against the half vector; metal does not
            const float3 h = normalize3(s.dir + wo);
            if (lobe == 0 || (dot3(s.dir, h) > 0.0f && dot3(s.dir, m.n) > 0.0f)) {
                s.pdf = reflectionPdf(m, s.dir, wo);
                const float3 fs = reflectionBrdf(m, s.dir, wo);
                if (lobe == 0) {
                    // metalBrdf: conductor Fresnel on top
                    const float p = schlickPow(dot3(wo, h));
                    s.bsdf = fs * (m.baseColour + (mk3s(1.0f) - m.baseColour) * p);
                } else {
                    s.bsdf = fs;
                }
            } else {
                s.bsdf = mk3s(0.0f);
                s.pdf = 0.0f;
                ret = false;
            }
        }
    } else if (lobe == 2) {
        ret = transmissionSample(m, wo, xi.x, xi.y, s);
    } else if (lobe == 3) {
        ret = diffuseSample(m, wo, xi.x, xi.y, s);
    } else {
        s.dir = mk3(0.0f, 1.0f, 0.0f);
        s.bsdf = mk3(1.0f, 0.0f, 1.0f);
        s.pdf = 1.0f;
    }
    if (fresnelSplit) {
        const float k = lobe == 1 ? F : 1.0f - F;
        s.bsdf = s.bsdf * k;
        s.pdf = s.pdf * k;
    }
    return ret;
}

// Lobes a learned proposal may be mixed with (one-sample MIS): those whose
// sampler above has a closed-form density over all directions and whose
// value does not depend on extra random draws. Excluded: specular (delta),
// transmission (pdf without the refraction Jacobian, stochastic value) and
// sheen (pdf 1).
OPT_D bool guidable(uint32_t c)
{
    if (c & MF_SPECULAR)
        return false;
    if (c & MF_METAL)
        return true;
    if (c & MF_DIELECTRIC)
        return !(c & MF_TRANSMISSION);
    return (c & MF_COAT) != 0;
}
OPT_D bool reflectionLobe(uint32_t c) { return !(c & MF_METAL) && ((c & MF_REFLECTION) || !(c & MF_DIELECTRIC)); }
// Density of sampleBrdf's direction for a guidable lobe, evaluated at l,
// including the directions its sampler rejects (density 0 there, as a
// rejected sample is a killed path).
OPT_D float lobePdf(const MatMR &m, float3 l, float3 v)
{
    const uint32_t c = m.category;
    if (c & MF_METAL)
        return reflectionPdf(m, l, v);
    if (reflectionLobe(c)) {
        const float3 h = normalize3(l + v);
        return (dot3(l, h) > 0.0f && dot3(l, m.n) > 0.0f) ? reflectionPdf(m, l, v) : 0.0f;
    }
    return dot3(m.n, l) * OPT_INV_PI;  // cosine-weighted diffuse
}
// Direction sampleBrdf draws for a guidable lobe, by the same arithmetic
// (these lobes draw no extra uniforms); its value and density at that
// direction are lobeValue's and lobePdf's.
OPT_D float3 lobeDir(const MatMR &m, float3 wo, float3 xi)
{
    const uint32_t c = m.category;
    if ((c & MF_METAL) || reflectionLobe(c))
        return reflectionDir(m, wo, xi.x, xi.y);
    return cosineDir(m.n, xi.x, xi.y);
}
// Value sampleBrdf reports for direction l of a guidable lobe.
OPT_D float3 lobeValue(const MatMR &m, float3 l, float3 v)
{
    const uint32_t c = m.category;
    if (c & MF_METAL)
        return metalBrdf(m, l, v);
    if (reflectionLobe(c)) {
        const float3 h = normalize3(l + v);
        return (dot3(l, h) > 0.0f && dot3(l, m.n) > 0.0f) ? reflectionBrdf(m, l, v) : mk3s(0.0f);
    }
    return diffuseBrdf(m, l, v);
}

// The MaterialData fields that categorisation reads.
struct CatIn {
    uint32_t category;
    float coatWeight, coatRoughness, transmissionWeight, specular, subsurfaceWeight;
};

// categoriseMaterial (principled_bsdf.h:25-239): stochastic lobe choice. The
// layer weight is the cumulative selection value, as in the reference.
template <class U>
OPT_D uint32_t categorise(const CatIn &mat, float3 v, float3 n, float roughness, float metallic, float3 emission,
                          float3 sheenColour, float sheenRoughness, U &u, float &cw)
{
    uint32_t c = mat.category;
    cw = 1.0f;
    if (c != MF_UNCATEGORISED)
        return c;
    const uint32_t reflective = MF_METAL | MF_REFLECTION | MF_TRANSMISSION | MF_COAT | MF_SHEEN;
    float F = schlick(calcF0(1.5f), dot3(v, n));
    float coatW = mat.coatWeight * F;
    float baseW = 1.0f - coatW;
    float sheenW = maxc3(sheenColour);
    float sum = baseW + coatW + sheenW;
    float sx = baseW / sum, sy = coatW / sum, sz = sheenW / sum;
    sy += sx;
    sz += sy;
    float xi = u.next();
    if (xi < sx) {
        cw *= sx;
    } else if (xi < sy) {
        cw *= sy;
        c |= MF_COAT;
    } else {
        cw *= sz;
        c |= MF_SHEEN;
    }
    if (c & MF_COAT) {
        if (mat.coatRoughness == 0.0f)
            c |= MF_SPECULAR;
        return c;
    }
    if (c & MF_SHEEN) {
        if (sheenRoughness == 0.0f)
            c |= MF_SPECULAR;
        return c;
    }
    if (maxc3(emission) > 0.0f) {
        c |= MF_EMISSION;
    } else if (metallic == 1.0f) {
        c |= MF_METAL;
    } else if (metallic == 0.0f) {
        c |= MF_DIELECTRIC;
    } else {
        if (u.next() < metallic) {
            c |= MF_METAL;
            cw *= metallic;
        } else {
            c |= MF_DIELECTRIC;
            cw *= 1.0f - metallic;
        }
    }
    if (c & MF_DIELECTRIC) {
        if (mat.transmissionWeight == 1.0f) {
            c |= MF_TRANSMISSION;
        } else if (mat.transmissionWeight == 0.0f) {
            c |= MF_OPAQUE;
        } else if (u.next() < mat.transmissionWeight) {
            c |= MF_TRANSMISSION;
            cw *= mat.transmissionWeight;
        } else {
            c |= MF_OPAQUE;
            cw *= 1.0f - mat.transmissionWeight;
        }
    }
    if (c & MF_OPAQUE) {
        if (mat.specular > 0.0f) {
            if (u.next() < F) {
                c |= MF_REFLECTION;
                if (roughness == 0.0f)
                    cw *= F;
            } else if (roughness == 0.0f) {
                cw *= 1.0f - F;
            }
        }
        if (!(c & MF_REFLECTION)) {
            if (mat.subsurfaceWeight == 1.0f) {
                c |= MF_SUBSURFACE;
            } else if (mat.subsurfaceWeight == 0.0f) {
                c |= MF_DIFFUSE;
            } else if (u.next() < mat.subsurfaceWeight) {
                c |= MF_SUBSURFACE;
                cw *= mat.subsurfaceWeight;
            } else {
                c |= MF_DIFFUSE;
                cw *= 1.0f - mat.subsurfaceWeight;
            }
            if ((c & MF_DIFFUSE) && roughness == 0.0f)
                c |= MF_LAMBERTIAN;
        }
    }
    if ((c & reflective) && roughness == 0.0f)
        c |= MF_SPECULAR;
    return c;
}

// Material set-up of the closest-hit program (cu/path_tracer.cu:343-370).
OPT_D MatMR makeMatMR(float3 albedo, float ior, float metallic, float3 sheenColour, uint32_t category, float3 n,
                      float roughness, float coatRoughness, float sheenRoughnessMat)
{
    MatMR m;
    m.baseColour = albedo;
    m.sheenColour = sheenColour;
    m.n = n;
    m.ior = ior;
    m.metallic = metallic;
    m.category = category;
    float r = (category & MF_COAT) ? coatRoughness : ((category & MF_SHEEN) ? sheenRoughnessMat : roughness);
    m.alpha = r * r;
    m.alpha2 = m.alpha * m.alpha;
    return m;
}

}  // namespace bsdf
