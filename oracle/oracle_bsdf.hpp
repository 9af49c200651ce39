// ORACLE (test infrastructure only; never linked into the product).
//
// A precision-templated CPU restatement of the reference's glTF
// metallic-roughness BSDF and its sampling helpers. Real = double is the FP64
// oracle; Real = float restates the same formulas at the reference's own
// precision and is checked against the reference headers compiled for the host
// (oracle/ref_driver.cpp). Every function cites the reference file:line that it
// follows; the reference's quirks are kept on purpose (they define parity).
//
// Random numbers: the reference draws uniforms inside categorisation,
// evaluation and sampling. Here every draw goes through Uniforms::next(), which
// replays a caller-supplied list in draw order.
#pragma once
#include <cmath>
#include <cstdint>

namespace orc {

enum Flags : uint32_t {  // include/material_flags.h:3-18
    Uncategorised = 0,
    Metal = 1u << 0,
    Dielectric = 1u << 1,
    Emission = 1u << 2,
    Opaque = 1u << 3,
    Transmission = 1u << 4,
    Reflection = 1u << 5,
    Diffuse = 1u << 6,
    Subsurface = 1u << 7,
    Coat = 1u << 8,
    Sheen = 1u << 9,
    Lambertian = 1u << 10,
    Specular = 1u << 11,
};

template <class R> struct V3 {
    R x, y, z;
};
template <class R> inline V3<R> v3(R a, R b, R c) { return V3<R>{a, b, c}; }
template <class R> inline V3<R> v3s(R s) { return V3<R>{s, s, s}; }
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
template <class R> inline V3<R> normalize(V3<R> a)
{
    R inv = R(1) / std::sqrt(dot(a, a));
    return a * inv;
}
template <class R> inline R maxc(V3<R> a) { return std::fmax(a.x, std::fmax(a.y, a.z)); }

template <class R> struct Consts {
    static constexpr R pi = R(3.14159265358979323846);
    static constexpr R inv_pi = R(0.318309886183790671538);
};

// Replays uniforms in draw order (the reference draws through
// PRD::random.rng(), random_number_generators.h:73-92).
template <class R> struct Uniforms {
    const float *xs;
    int n;
    int used;
    R next()
    {
        R x = used < n ? R(xs[used]) : R(0.5);
        ++used;
        return x;
    }
};

// MaterialMetallicRoughness (include/material_metallic_roughness.h:3-23).
template <class R> struct MatMR {
    V3<R> baseColour;
    R ior, roughness, metallic, specular, transmissionWeight, subsurfaceWeight, coatWeight;
    V3<R> sheenColour;
    uint32_t category;
    V3<R> n;  // shading normal
    R alpha, alpha2;
};

template <class R> struct Sample {
    V3<R> dir;
    V3<R> bsdf;
    R pdf;
};

// ---------------------------------------------------------------- helpers

// calcF0 (include/principled_bsdf_helpers.h:7-11)
template <class R> inline R calcF0(R ior)
{
    R t = (R(1) - ior) / (R(1) + ior);
    return t * t;
}
// fresnelPowerTerm / fresnelSchlick (include/schlick.h:6-23); |v.h| per :8
template <class R> inline R schlickPow(R vDotH) { return std::pow(R(1) - std::fabs(vDotH), R(5)); }
template <class R> inline R schlick(R f0, R vDotH) { return f0 + (R(1) - f0) * schlickPow(vDotH); }
template <class R> inline V3<R> schlick3(V3<R> f0, R vDotH)
{
    R p = schlickPow(vDotH);
    return f0 + (v3s<R>(R(1)) - f0) * p;
}

// reflectRay (include/reflection_and_refraction.h:5-14)
template <class R> inline V3<R> reflectRay(V3<R> n, V3<R> i) { return -i + (R(2) * dot(n, i)) * n; }

// refractRay (include/reflection_and_refraction.h:16-48); TIR returns the
// reflection about the flipped normal.
template <class R> inline V3<R> refractRay(V3<R> n, V3<R> i, R eta)
{
    R c = dot(n, i);
    if (c < R(0)) {
        eta = R(1) / eta;
        c = -c;
        n = -n;
    }
    R sin2i = std::fmax(R(0), R(1) - c * c);
    R sin2t = sin2i / (eta * eta);
    if (sin2t >= R(1))
        return reflectRay(n, i);
    R cosT = std::sqrt(std::fmax(R(0), R(1) - sin2t));
    return -i / eta + (c / eta - cosT) * n;
}

// transmissionHalfVectorVolumetric (include/reflection_and_refraction.h:69-97):
// only the IOR pair swaps when v is inside; the flipped normal is unused.
template <class R> inline V3<R> halfVolumetric(V3<R> n, V3<R> l, V3<R> v, R etaI, R etaV)
{
    if (dot(n, v) < R(0)) {
        R t = etaI;
        etaI = etaV;
        etaV = t;
    }
    return normalize(-(etaI * v + etaV * l));
}

// OrthonormalBasis (include/orthonormal_basis.h:11-41)
template <class R> struct Onb {
    V3<R> t, b, n;
    explicit Onb(V3<R> nn)
    {
        n = nn;
        if (std::fabs(n.x) > std::fabs(n.z))
            b = v3<R>(-n.y, n.x, R(0));
        else
            b = v3<R>(R(0), -n.z, n.y);
        b = normalize(b);
        t = cross(b, n);
    }
    V3<R> toWorld(V3<R> p) const { return p.x * t + p.y * b + p.z * n; }
};

// sphericalToCartesian (include/cuda_utils.h:24-30)
template <class R> inline V3<R> sphericalToCartesian(R theta, R phi)
{
    return v3<R>(std::sin(theta) * std::cos(phi), std::sin(theta) * std::sin(phi), std::cos(theta));
}

// cosineSampleHemisphere via sampleDisk (include/sampling.h:27-42)
template <class R> inline V3<R> cosineSampleHemisphere(R x, R y)
{
    R r = std::sqrt(x);
    R phi = y * R(2) * Consts<R>::pi;
    R px = r * std::cos(phi), py = r * std::sin(phi);
    R z = std::sqrt(std::fmax(R(0), R(1) - px * px - py * py));
    return v3<R>(px, py, z);
}

// ---------------------------------------------------------------- microfacet

// trowbridgeReitzD (include/trowbridge_reitz.h:12-26), alpha^2 clamped >= 1e-5
template <class R> inline R ggxD(R nDotH, R alpha)
{
    if (nDotH <= R(0))
        return R(0);
    R a2 = std::fmax(R(0.00001f), alpha * alpha);
    R t = nDotH * nDotH * (a2 - R(1)) + R(1);
    return a2 / (Consts<R>::pi * t * t);
}

// trowbridgeReitzGetHalfVector (include/trowbridge_reitz.h:28-47); uses
// mat.alpha2 (= roughness^4)
template <class R> inline V3<R> ggxHalf(const MatMR<R> &m, V3<R> n, R x, R y)
{
    R theta = std::acos(std::sqrt((R(1) - x) / ((m.alpha2 - R(1)) * x + R(1))));
    R phi = R(2) * Consts<R>::pi * y;
    V3<R> h = sphericalToCartesian(theta, phi);
    return Onb<R>(n).toWorld(h);
}

// trowbridgeReitzPdf (include/trowbridge_reitz.h:49-63)
template <class R> inline R ggxPdf(V3<R> n, V3<R> h, V3<R> v, R alpha)
{
    R nDotH = dot(n, h);
    R D = ggxD(nDotH, alpha);
    return (D * nDotH) / (R(4) * std::fabs(dot(h, v)));
}

// smithV (include/smith.h:35-52), separable, heaviside on h.l and h.v
template <class R> inline R smithV(R hDotL, R nl, R hDotV, R nv, R alpha)
{
    if (hDotL <= R(0) || hDotV <= R(0))
        return R(0);
    R a2 = alpha * alpha;
    R t1 = nl + std::sqrt(a2 + (R(1) - a2) * nl * nl);
    R t2 = nv + std::sqrt(a2 + (R(1) - a2) * nv * nv);
    return R(1) / (t1 * t2);
}

// ---------------------------------------------------------------- sheen
// charlieSheenD / l / lambdaSheen / charlieSheenV (include/sheen.h:16-46)
template <class R> inline R charlieD(R nDotH, R a)
{
    R invR = R(1) / a;
    R sin2 = R(1) - nDotH * nDotH;
    return (R(2) + invR) * std::pow(sin2, invR * R(0.5)) * (R(0.5) * Consts<R>::inv_pi);
}
template <class R> inline R lerpS(R a, R b, R t) { return a + t * (b - a); }  // cuda_utils.h:19-22
template <class R> inline R sheenL(R x, R a)
{
    R t = (R(1) - a) * (R(1) - a);
    R A = lerpS(R(21.5473f), R(25.3245f), t);
    R B = lerpS(R(3.82987f), R(3.32435f), t);
    R C = lerpS(R(0.19823f), R(0.16801f), t);
    R D = lerpS(R(-1.97760f), R(-1.27393f), t);
    R E = lerpS(R(-4.32054f), R(-4.85967f), t);
    return A / (R(1) + B * std::pow(x, C)) + D * x + E;
}
template <class R> inline R sheenLambda(R c, R a)
{
    if (std::fabs(c) < R(0.5))
        return std::exp(sheenL(c, a));
    return std::exp(R(2) * sheenL(R(0.5), a) - sheenL(R(1) - c, a));
}
template <class R> inline R charlieV(R nv, R nl, R a)
{
    return R(1) / ((R(1) + sheenLambda(nv, a) + sheenLambda(nl, a)) * (R(4) * nv * nl));
}

// ---------------------------------------------------------------- lobes

// Oren-Nayar (include/oren_nayar.h:15-59); the n.l factor is applied inside and
// the projected vectors use the clamped cosines.
template <class R> inline V3<R> orenNayar(const MatMR<R> &m, V3<R> l, V3<R> v)
{
    R sigma = R(0.7071067f) * std::atan(m.alpha);
    R nDotV = std::fmin(std::fmax(R(0.00001f), dot(m.n, v)), R(1));
    R nDotL = std::fmin(std::fmax(R(0.00001f), dot(m.n, l)), R(1));
    R thetaV = std::acos(nDotV), thetaL = std::acos(nDotL);
    R a = std::fmax(thetaV, thetaL), b = std::fmin(thetaV, thetaL);
    V3<R> lp = l - nDotL * m.n, vp = v - nDotV * m.n;
    R cosPhi = dot(normalize(vp), normalize(lp));
    R s2 = sigma * sigma;
    R A = R(1) - R(0.5) * (s2 / (s2 + R(0.33f)));
    R B = R(0.45f) * (s2 / (s2 + R(0.09f)));
    R on = A + B * std::fmax(R(0), cosPhi) * std::sin(a) * std::tan(b);
    V3<R> refl = m.baseColour * (R(1) - m.metallic);
    return refl * (on * Consts<R>::inv_pi * dot(m.n, l));
}

// diffuseBrdf / diffusePdf (include/principled_bsdf.h:253-270)
template <class R> inline V3<R> diffuseBrdf(const MatMR<R> &m, V3<R> l, V3<R> v)
{
    if (m.category & Lambertian)
        return m.baseColour * Consts<R>::inv_pi;
    return orenNayar(m, l, v);
}
template <class R> inline R diffusePdf(V3<R> n, V3<R> l) { return dot(n, l) * Consts<R>::inv_pi; }

// diffuseSample (include/principled_bsdf.h:245-279)
template <class R> inline bool diffuseSample(const MatMR<R> &m, V3<R> v, R x, R y, Sample<R> &s)
{
    s.dir = Onb<R>(m.n).toWorld(cosineSampleHemisphere(x, y));
    s.bsdf = diffuseBrdf(m, s.dir, v);
    s.pdf = diffusePdf(m.n, s.dir);
    return true;
}

// specularReflectionSample (include/principled_bsdf.h:285-292)
template <class R> inline bool specReflSample(const MatMR<R> &m, V3<R> wo, Sample<R> &s)
{
    s.dir = reflectRay(m.n, wo);
    s.bsdf = m.baseColour / std::fabs(dot(s.dir, m.n));
    s.pdf = R(1);
    return true;
}

// specularTransmissionSample (include/principled_bsdf.h:298-339)
template <class R> inline bool specTransSample(const MatMR<R> &m, V3<R> wo, Sample<R> &s)
{
    s.dir = refractRay(m.n, wo, m.ior);
    s.bsdf = m.baseColour / std::fabs(dot(m.n, s.dir));
    s.pdf = R(1);
    return true;
}

// reflectionGetNewRayDir (include/principled_bsdf.h:384-406)
template <class R> inline V3<R> reflectionDir(const MatMR<R> &m, V3<R> n, V3<R> v, R x, R y)
{
    if (m.category & Specular)
        return reflectRay(n, v);
    V3<R> h = ggxHalf(m, n, x, y);
    return reflectRay(h, v);
}

// reflectionBrdf (include/principled_bsdf.h:408-458): V*D, no Fresnel, no tint
template <class R> inline V3<R> reflectionBrdf(const MatMR<R> &m, V3<R> n, V3<R> l, V3<R> v)
{
    if (m.category & Specular)
        return m.baseColour / std::fabs(dot(l, n));
    V3<R> h = normalize(l + v);
    R hl = dot(h, l), hv = dot(h, v);
    R nl = std::fmax(std::fabs(dot(n, l)), R(0.00001f));
    R nv = std::fmax(std::fabs(dot(n, v)), R(0.00001f));
    R V = smithV(hl, nl, hv, nv, m.alpha);
    R D = ggxD(dot(n, h), m.alpha);
    return v3s<R>(V * D);
}

// reflectionPdf (include/principled_bsdf.h:462-481)
template <class R> inline R reflectionPdf(const MatMR<R> &m, V3<R> n, V3<R> l, V3<R> v)
{
    if (m.category & Specular)
        return R(1);
    V3<R> h = normalize(l + v);
    return ggxPdf(n, h, v, m.alpha);
}

// reflectionSample (include/principled_bsdf.h:483-520): rejects l.h <= 0 or
// l.n <= 0
template <class R> inline bool reflectionSample(const MatMR<R> &m, V3<R> v, R x, R y, Sample<R> &s)
{
    if (m.category & Specular)
        return specReflSample(m, v, s);
    s.dir = reflectionDir(m, m.n, v, x, y);
    V3<R> h = normalize(s.dir + v);
    if (dot(s.dir, h) > R(0) && dot(s.dir, m.n) > R(0)) {
        s.pdf = reflectionPdf(m, m.n, s.dir, v);
        s.bsdf = reflectionBrdf(m, m.n, s.dir, v);
        return true;
    }
    s.bsdf = v3s<R>(R(0));
    s.pdf = R(0);
    return false;
}

// transmissionGetNewRayDir (include/principled_bsdf.h:526-558)
template <class R> inline V3<R> transmissionDir(const MatMR<R> &m, V3<R> v, R x, R y)
{
    if (m.category & Specular)
        return refractRay(m.n, v, m.ior);
    V3<R> h = ggxHalf(m, m.n, x, y);
    return refractRay(h, v, m.ior);
}

// transmissionBrdf (include/principled_bsdf.h:560-597): fixed IOR pair 1.0/1.5
template <class R> inline V3<R> transmissionBrdf(const MatMR<R> &m, V3<R> n, V3<R> l, V3<R> v)
{
    if (m.category & Specular)
        return m.baseColour / std::fabs(dot(n, l));
    V3<R> h = halfVolumetric(n, l, v, R(1), R(1.5f));
    R hl = dot(h, l) / dot(n, l);
    R hv = dot(h, v) / dot(n, v);
    R nl = std::fmax(std::fabs(dot(n, l)), R(0.00001f));
    R nv = std::fmax(std::fabs(dot(n, v)), R(0.00001f));
    R V = smithV(hl, nl, hv, nv, m.alpha);
    R D = ggxD(dot(n, h), m.alpha);
    return v3s<R>(V * D);
}

// transmissionPdf (include/principled_bsdf.h:599-619): reflection-style pdf,
// no refraction Jacobian
template <class R> inline R transmissionPdf(const MatMR<R> &m, V3<R> l, V3<R> v)
{
    if (m.category & Specular)
        return R(1);
    V3<R> h = halfVolumetric(m.n, l, v, R(1), R(1.5f));
    return ggxPdf(m.n, h, v, m.alpha);
}

// transmissionSample (include/principled_bsdf.h:621-632)
template <class R> inline bool transmissionSample(const MatMR<R> &m, V3<R> v, R x, R y, Sample<R> &s)
{
    if (m.category & Specular)
        return specTransSample(m, v, s);
    s.dir = transmissionDir(m, v, x, y);
    s.bsdf = transmissionBrdf(m, m.n, s.dir, v);
    s.pdf = transmissionPdf(m, s.dir, v);
    return true;
}

// dielectricBrdf (include/principled_bsdf.h:638-681): the transmission branch
// draws a uniform inside the evaluation (:649)
template <class R, class U> inline V3<R> dielectricBrdf(const MatMR<R> &m, V3<R> l, V3<R> v, U &u)
{
    if (m.category & Transmission) {
        R f0 = calcF0(m.ior);
        R F = schlick(f0, dot(v, m.n));
        R xi = u.next();
        if (xi < F)
            return reflectionBrdf(m, m.n, l, v);
        return transmissionBrdf(m, m.n, l, v);
    }
    if (m.category & Reflection)
        return reflectionBrdf(m, m.n, l, v);
    return diffuseBrdf(m, l, v);
}

// dielectricSample (include/principled_bsdf.h:683-735): f0 clamped to 1 here
template <class R, class U>
inline bool dielectricSample(const MatMR<R> &m, V3<R> v, R x, R y, U &u, Sample<R> &s)
{
    if (m.category & Transmission) {
        R f0 = std::fmin(calcF0(m.ior), R(1));
        R F = schlick(f0, dot(v, m.n));
        R r1 = u.next();
        bool ret;
        if (r1 < F) {
            ret = reflectionSample(m, v, x, y, s);
            s.bsdf = s.bsdf * F;
            s.pdf = s.pdf * F;
        } else {
            ret = transmissionSample(m, v, x, y, s);
            s.bsdf = s.bsdf * (R(1) - F);
            s.pdf = s.pdf * (R(1) - F);
        }
        return ret;
    }
    if (m.category & Reflection)
        return reflectionSample(m, v, x, y, s);
    return diffuseSample(m, v, x, y, s);
}

// metalBrdf (include/principled_bsdf.h:748-762) with conductorFresnel
// (include/principled_bsdf_helpers.h:24-31): Schlick with f0 = base colour
template <class R> inline V3<R> metalBrdf(const MatMR<R> &m, V3<R> l, V3<R> v)
{
    V3<R> fs = reflectionBrdf(m, m.n, l, v);
    V3<R> h = normalize(l + v);
    return fs * schlick3(m.baseColour, dot(v, h));
}

// metalSample (include/principled_bsdf.h:769-785): no rejection test
template <class R> inline bool metalSample(const MatMR<R> &m, V3<R> v, R x, R y, Sample<R> &s)
{
    s.dir = reflectionDir(m, m.n, v, x, y);
    s.pdf = reflectionPdf(m, m.n, s.dir, v);
    s.bsdf = metalBrdf(m, s.dir, v);
    return true;
}

// sheenBrdf (include/principled_bsdf.h:797-826)
template <class R> inline V3<R> sheenBrdf(const MatMR<R> &m, V3<R> l, V3<R> v)
{
    if (m.category & Specular)
        return m.sheenColour / std::fabs(dot(l, m.n));
    V3<R> h = normalize(l + v);
    R V = charlieV(dot(h, v), dot(h, l), m.alpha);
    R D = charlieD(dot(m.n, h), m.alpha);
    return m.sheenColour * (V * D) / std::fabs(dot(m.n, v));
}

// sheenSample (include/principled_bsdf.h:852-859): GGX direction, pdf = 1 (:849)
template <class R> inline bool sheenSample(const MatMR<R> &m, V3<R> v, R x, R y, Sample<R> &s)
{
    s.dir = reflectionDir(m, m.n, v, x, y);
    s.bsdf = sheenBrdf(m, s.dir, v);
    s.pdf = R(1);
    return true;
}

// metallicRoughnessBrdf (include/principled_bsdf.h:866-898)
template <class R, class U> inline V3<R> mrBrdf(const MatMR<R> &m, V3<R> l, V3<R> v, U &u)
{
    if (m.category & Metal)
        return metalBrdf(m, l, v);
    if (m.category & Dielectric)
        return dielectricBrdf(m, l, v, u);
    if (m.category & Coat)
        return reflectionBrdf(m, m.n, l, v);
    if (m.category & Sheen)
        return sheenBrdf(m, l, v);
    return v3<R>(R(1), R(0), R(1));
}

// metallicRoughnessSample (include/principled_bsdf.h:902-961)
template <class R, class U> inline bool mrSample(const MatMR<R> &m, V3<R> wo, V3<R> xi, U &u, Sample<R> &s)
{
    if (m.category & Metal)
        return metalSample(m, wo, xi.x, xi.y, s);
    if (m.category & Dielectric)
        return dielectricSample(m, wo, xi.x, xi.y, u, s);
    if (m.category & Coat)
        return reflectionSample(m, wo, xi.x, xi.y, s);
    if (m.category & Sheen)
        return sheenSample(m, wo, xi.x, xi.y, s);
    s.dir = v3<R>(R(0), R(1), R(0));
    s.bsdf = v3<R>(R(1), R(0), R(1));
    s.pdf = R(1);
    return true;
}

// Inputs of categoriseMaterial that come from MaterialData.
template <class R> struct MatCat {
    uint32_t category;
    R coatWeight, coatRoughness, transmissionWeight, specular, subsurfaceWeight;
};

// categoriseMaterial (include/principled_bsdf.h:25-239). The layer weight is
// the CUMULATIVE selection value (:108-124), kept as in the reference.
template <class R, class U>
inline uint32_t categorise(const MatCat<R> &mat, V3<R> v, V3<R> n, R roughness, R metallic, V3<R> emission,
                           V3<R> sheenColour, R sheenRoughness, U &u, R &cw)
{
    uint32_t c = mat.category;
    cw = R(1);
    if (c != Uncategorised)
        return c;
    const uint32_t reflective = Metal | Reflection | Transmission | Coat | Sheen;
    R f0 = calcF0(R(1.5f));
    R F = schlick(f0, dot(v, n));
    R coatW = mat.coatWeight * F;
    R baseW = R(1) - coatW;
    R sheenW = maxc(sheenColour);
    R sum = baseW + coatW + sheenW;
    R sx = baseW / sum, sy = coatW / sum, sz = sheenW / sum;
    sy += sx;
    sz += sy;
    R layerWeight;
    R xi = u.next();
    if (xi < sx) {
        layerWeight = sx;
    } else if (xi < sy) {
        layerWeight = sy;
        c |= Coat;
    } else {
        layerWeight = sz;
        c |= Sheen;
    }
    cw *= layerWeight;
    if (c & Coat) {
        if (mat.coatRoughness == R(0))
            c |= Specular;
        return c;
    }
    if (c & Sheen) {
        if (sheenRoughness == R(0))
            c |= Specular;
        return c;
    }
    if (maxc(emission) > R(0)) {
        c |= Emission;
    } else if (metallic == R(1)) {
        c |= Metal;
    } else if (metallic == R(0)) {
        c |= Dielectric;
    } else {
        R x = u.next();
        if (x < metallic) {
            c |= Metal;
            cw *= metallic;
        } else {
            c |= Dielectric;
            cw *= R(1) - metallic;
        }
    }
    if (c & Dielectric) {
        if (mat.transmissionWeight == R(1)) {
            c |= Transmission;
        } else if (mat.transmissionWeight == R(0)) {
            c |= Opaque;
        } else {
            R x = u.next();
            if (x < mat.transmissionWeight) {
                c |= Transmission;
                cw *= mat.transmissionWeight;
            } else {
                c |= Opaque;
                cw *= R(1) - mat.transmissionWeight;
            }
        }
    }
    if (c & Opaque) {
        if (mat.specular > R(0)) {
            R x = u.next();
            if (x < F) {
                c |= Reflection;
                if (roughness == R(0))
                    cw *= F;
            } else {
                if (roughness == R(0))
                    cw *= R(1) - F;
            }
        }
        if (!(c & Reflection)) {
            if (mat.subsurfaceWeight == R(1)) {
                c |= Subsurface;
            } else if (mat.subsurfaceWeight == R(0)) {
                c |= Diffuse;
            } else {
                R x = u.next();
                if (x < mat.subsurfaceWeight) {
                    c |= Subsurface;
                    cw *= mat.subsurfaceWeight;
                } else {
                    c |= Diffuse;
                    cw *= R(1) - mat.subsurfaceWeight;
                }
            }
            if ((c & Diffuse) && roughness == R(0))
                c |= Lambertian;
        }
    }
    if ((c & reflective) && roughness == R(0))
        c |= Specular;
    return c;
}

// The MaterialMetallicRoughness set-up of the closest-hit program
// (cu/path_tracer.cu:343-370): coat and sheen layers use their own roughness
// (the sheen one from MaterialData, before its texture).
template <class R>
inline MatMR<R> makeMatMR(V3<R> albedo, R ior, R metallic, R specular, R tw, R sw, R coatW, V3<R> sheenColour,
                          uint32_t category, V3<R> n, R roughness, R coatRoughness, R sheenRoughnessMat)
{
    MatMR<R> m;
    m.baseColour = albedo;
    m.ior = ior;
    m.metallic = metallic;
    m.specular = specular;
    m.transmissionWeight = tw;
    m.subsurfaceWeight = sw;
    m.coatWeight = coatW;
    m.sheenColour = sheenColour;
    m.category = category;
    m.n = n;
    if (category & Coat) {
        m.roughness = coatRoughness;
        m.alpha = coatRoughness * coatRoughness;
    } else if (category & Sheen) {
        m.roughness = sheenRoughnessMat;
        m.alpha = sheenRoughnessMat * sheenRoughnessMat;
    } else {
        m.roughness = roughness;
        m.alpha = roughness * roughness;
    }
    m.alpha2 = m.alpha * m.alpha;
    return m;
}

// ---------------------------------------------------------------- tone map
// toneMapReinhard / toneMapAcesNarkowicz (include/tone_mapping.h:5-29),
// linearToSrgb (include/gamma_correction.h:3-7)
template <class R> inline R reinhard(R c) { return c / (c + R(1)); }
template <class R> inline R aces(R c)
{
    const R a = R(2.51f), b = R(0.03f), cc = R(2.43f), d = R(0.59f), e = R(0.14f);
    R t = (c * (a * c + b)) / (c * (cc * c + d) + e);
    return std::fmax(R(0), std::fmin(t, R(1)));
}
template <class R> inline R gammaEncode(R c, R gammaTerm) { return std::pow(c, R(1) / gammaTerm); }

}  // namespace orc
