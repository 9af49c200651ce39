// ORACLE (test infrastructure only; never linked into the product).
//
// extern "C" surface of the oracle restatement: BSDF queries in FP32 and FP64,
// tone mapping, punctual-light sampling and barycentrics, with the same record
// layouts as the reference host build (query_abi.h) so the two can be compared
// query by query.
#include <cmath>
#include <cstdint>
#include "oracle_bsdf.hpp"
#include "query_abi.h"

namespace {

template <class R> orc::V3<R> v3f(const float *p) { return orc::v3<R>(R(p[0]), R(p[1]), R(p[2])); }
template <class R> void put3(double *d, orc::V3<R> v)
{
    d[0] = double(v.x);
    d[1] = double(v.y);
    d[2] = double(v.z);
}

// The query procedure of cu/path_tracer.cu:231-370 (categorise + material set-up),
// :400 (BRDF evaluation for next-event estimation) and :524-526 (sampling).
template <class R> void bsdfQuery(const orc_bsdf_query &Q, orc_bsdf_result &Rz)
{
    using namespace orc;
    Uniforms<R> u{Q.xs, ORC_NXS, 0};
    MatCat<R> mc{Q.category, R(Q.coatWeight), R(Q.coatRoughness), R(Q.transmissionWeight), R(Q.specular),
                 R(Q.subsurfaceWeight)};
    V3<R> n = v3f<R>(Q.n), wo = v3f<R>(Q.wo), wi = v3f<R>(Q.wi);
    R cw;
    uint32_t cat = categorise(mc, wo, n, R(Q.roughness), R(Q.metallic), v3f<R>(Q.emission), v3f<R>(Q.sheenColour),
                              R(Q.sheenRoughness), u, cw);
    Rz.category = cat;
    Rz.categoryWeight = double(cw);
    if (cat & Emission) {
        for (int k = 0; k < 3; ++k)
            Rz.f[k] = Rz.dir[k] = Rz.bsdf[k] = 0.0;
        Rz.pdf = 0.0;
        Rz.ret = 0;
        Rz.used = u.used;
        return;
    }
    MatMR<R> m = makeMatMR(v3f<R>(Q.baseColour), R(Q.ior), R(Q.metallic), R(Q.specular), R(Q.transmissionWeight),
                           R(Q.subsurfaceWeight), R(Q.coatWeight), v3f<R>(Q.sheenColour), cat, n, R(Q.roughness),
                           R(Q.coatRoughness), R(Q.sheenRoughnessMat));
    put3(Rz.f, mrBrdf(m, wi, wo, u));
    V3<R> xi;
    xi.x = u.next();
    xi.y = u.next();
    xi.z = u.next();
    Sample<R> s;
    s.dir = v3s<R>(R(0));
    s.bsdf = v3s<R>(R(0));
    s.pdf = R(0);
    bool ok = mrSample(m, wo, xi, u, s);
    s.pdf = s.pdf * cw;
    put3(Rz.dir, s.dir);
    put3(Rz.bsdf, s.bsdf);
    Rz.pdf = double(s.pdf);
    Rz.ret = ok ? 1 : 0;
    Rz.used = u.used;
}

}  // namespace

extern "C" int orc_bsdf_query_f32(const orc_bsdf_query *q, orc_bsdf_result *r, int n)
{
    for (int i = 0; i < n; ++i)
        bsdfQuery<float>(q[i], r[i]);
    return 0;
}

extern "C" int orc_bsdf_query_f64(const orc_bsdf_query *q, orc_bsdf_result *r, int n)
{
    for (int i = 0; i < n; ++i)
        bsdfQuery<double>(q[i], r[i]);
    return 0;
}

// Tone mapping then gamma, per channel; alpha passes through the tone map
// (cu/device_programs.cu:84-96, tone_mapping.h:5-29, gamma_correction.h:3-7).
extern "C" int orc_tonemap_f64(const double *rgba_in, double *rgba_out, int n, int toneMapping, int impl,
                               int gammaCorrection, double gammaTerm)
{
    for (int i = 0; i < n; ++i) {
        for (int c = 0; c < 4; ++c) {
            double x = rgba_in[4 * i + c];
            if (toneMapping)
                x = impl == 0 ? orc::reinhard(x) : orc::aces(x);
            if (gammaCorrection && c < 3)
                x = orc::gammaEncode(x, gammaTerm);
            rgba_out[4 * i + c] = x;
        }
    }
    return 0;
}

// Punctual-light sampling (cu/light_sampling.cu:6-81, include/sampling.h:64-77).
extern "C" int orc_light_sample_f64(const orc_light *lights, const float *points, double *out, int n)
{
    using namespace orc;
    for (int i = 0; i < n; ++i) {
        const orc_light &L = lights[i];
        V3<double> p = v3f<double>(points + 3 * i), p0 = v3f<double>(L.p0), ln = v3f<double>(L.normal);
        V3<double> rad = v3f<double>(L.radiance), dir;
        double dist, pdf = 1.0;
        V3<double> Li;
        if (L.type == 1) {  // directional (:26-44)
            V3<double> pos = p + (-ln * double(L.distance));
            dir = -ln;
            Li = rad;
            dist = length(pos - p);
        } else {
            dir = p0 - p;
            dist = length(dir);
            dir = dir / dist;
            Li = rad / (dist * dist);
            if (L.type == 2) {  // spot (:46-59) with falloff (sampling.h:64-77)
                double c = dot(ln, -dir), fo;
                if (c < L.cosWidth)
                    fo = 0.0;
                else if (c > L.cosFalloffStart)
                    fo = 1.0;
                else {
                    double d = (c - L.cosWidth) / (double(L.cosFalloffStart) - L.cosWidth);
                    fo = (d * d) * (d * d);
                }
                Li = rad * fo / (dist * dist);
            }
        }
        double *o = out + 8 * i;
        o[0] = dir.x; o[1] = dir.y; o[2] = dir.z;
        o[3] = Li.x; o[4] = Li.y; o[5] = Li.z;
        o[6] = pdf; o[7] = dist;
    }
    return 0;
}

// calcBarycentric (include/barycentrics.h:12-44), dominant-axis projection.
extern "C" int orc_barycentric_f64(const float *tri, const float *p, double *uvw, int n)
{
    using namespace orc;
    auto area2 = [](double x1, double y1, double x2, double y2, double x3, double y3) {
        return (x1 - x2) * (y2 - y3) - (x2 - x3) * (y1 - y2);
    };
    for (int i = 0; i < n; ++i) {
        V3<double> a = v3f<double>(tri + 9 * i), b = v3f<double>(tri + 9 * i + 3), c = v3f<double>(tri + 9 * i + 6);
        V3<double> q = v3f<double>(p + 3 * i);
        V3<double> m = cross(b - a, c - a);
        double x = std::fabs(m.x), y = std::fabs(m.y), z = std::fabs(m.z), nu, nv, ood;
        if (x >= y && x >= z) {
            nu = area2(q.y, q.z, b.y, b.z, c.y, c.z);
            nv = area2(q.y, q.z, c.y, c.z, a.y, a.z);
            ood = 1.0 / m.x;
        } else if (y >= x && y >= z) {
            nu = area2(q.x, q.z, b.x, b.z, c.x, c.z);
            nv = area2(q.x, q.z, c.x, c.z, a.x, a.z);
            ood = 1.0 / -m.y;
        } else {
            nu = area2(q.x, q.y, b.x, b.y, c.x, c.y);
            nv = area2(q.x, q.y, c.x, c.y, a.x, a.y);
            ood = 1.0 / m.z;
        }
        uvw[3 * i] = nu * ood;
        uvw[3 * i + 1] = nv * ood;
        uvw[3 * i + 2] = 1.0 - nu * ood - nv * ood;
    }
    return 0;
}
