// Host side of scene input: seeded procedural scenes, the host material
// categorisation, and the configs/*.json scene-selection format.
//
// The reference imports glTF 2.0 (src/gltf_loader.cpp) from a scenes
// repository that is not available here; the procedural scenes below stand in
// for it with the shapes, sizes and material distributions of the benchmark
// workloads. Arithmetic is in double and only rounded to float at the end,
// and the file is compiled without floating-point contraction, so x86 and Arm
// hosts produce identical scenes.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>
#include "../../include/optpt.h"
#include "host_scene.h"
#include "json.h"

extern "C" int optpt_internal_set_error(int code, const char *msg);

using namespace optjson;

namespace {

struct Vec {
    double x, y, z;
};
Vec operator+(Vec a, Vec b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
Vec operator-(Vec a, Vec b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
Vec operator*(Vec a, double s) { return {a.x * s, a.y * s, a.z * s}; }
double dotv(Vec a, Vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
Vec crossv(Vec a, Vec b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
Vec normv(Vec a)
{
    double l = std::sqrt(dotv(a, a));
    return a * (1.0 / l);
}

// Small deterministic generator for scene parameters (SplitMix64).
struct SceneRng {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double range(double a, double b) { return a + (b - a) * uniform(); }
};

}  // namespace

namespace opthost {

// MaterialParams::isDeterministic / categorise (include/material_params.h:
// 116-223 of the reference): materials without any per-hit choice get their
// category on the host; the others stay Uncategorised (0).
uint32_t hostCategory(const MaterialData &m)
{
    const bool emissive = m.emission[0] > 0.0f || m.emission[1] > 0.0f || m.emission[2] > 0.0f;
    const float sheenMax = std::fmax(std::fmax(m.sheenColour[0], m.sheenColour[1]), m.sheenColour[2]);
    bool det;
    if (m.coatWeight != 0.0f || sheenMax != 0.0f)
        det = false;
    else if (emissive)
        det = !m.hasEmissiveTexture;
    else if (m.metallic != 0.0f && m.metallic != 1.0f)
        det = false;
    else if (m.hasMetallicRoughnessTexture)
        det = false;
    else if (m.metallic == 1.0f)
        det = true;
    else if (m.transmissionWeight != 0.0f && m.transmissionWeight != 1.0f)
        det = false;
    else if (m.transmissionWeight == 1.0f)
        det = true;
    else if (m.specular != 0.0f)
        det = false;
    else if (m.subsurfaceWeight != 0.0f && m.subsurfaceWeight != 1.0f)
        det = false;
    else
        det = true;
    if (!det)
        return MF_UNCATEGORISED;
    if (emissive)
        return MF_EMISSION;
    uint32_t c = 0;
    if (m.metallic == 1.0f) {
        c |= MF_METAL;
    } else {
        c |= MF_DIELECTRIC;
        if (m.transmissionWeight == 1.0f) {
            c |= MF_TRANSMISSION;
        } else {
            c |= MF_OPAQUE;
            if (m.subsurfaceWeight == 1.0f) {
                c |= MF_SUBSURFACE;
            } else {
                c |= MF_DIFFUSE;
                if (m.roughness == 0.0f)
                    c |= MF_LAMBERTIAN;
            }
        }
    }
    if ((c & MF_METAL) || (c & MF_TRANSMISSION)) {
        if (m.roughness == 0.0f)
            c |= MF_SPECULAR;
    }
    return c;
}

MaterialData baseMaterial(double r, double g, double b)
{
    MaterialData m;
    memset(&m, 0, sizeof(m));
    m.baseColourTexture = m.normalTexture = m.metallicRoughnessTexture = -1;
    m.emissiveTexture = m.sheenColourTexture = m.sheenRoughnessTexture = -1;
    m.baseColour[0] = (float)r;
    m.baseColour[1] = (float)g;
    m.baseColour[2] = (float)b;
    m.baseColour[3] = 1.0f;
    m.alphaMode = AM_OPAQUE;
    m.alphaCutoff = 0.5f;
    TextureTransform *tf[6] = {&m.baseColourTexTf, &m.normalTexTf, &m.metallicRoughnessTexTf,
                               &m.emissiveTexTf, &m.sheenColourTexTf, &m.sheenRoughnessTexTf};
    for (auto *t : tf) {
        t->scale[0] = 1.0f;
        t->scale[1] = 1.0f;
    }
    m.ior = 1.5f;
    m.roughness = 1.0f;
    m.metallic = 0.0f;
    m.specular = 0.0f;
    return m;
}

}  // namespace opthost

using namespace opthost;

namespace {

struct Builder {
    std::vector<float> pos, nrm, tc;
    std::vector<int32_t> idx, mat;
    std::vector<MaterialData> materials;
    std::vector<Light> lights;
    bool withNormals = false;

    int addVertex(Vec p, Vec n = {0, 0, 0})
    {
        pos.push_back((float)p.x);
        pos.push_back((float)p.y);
        pos.push_back((float)p.z);
        nrm.push_back((float)n.x);
        nrm.push_back((float)n.y);
        nrm.push_back((float)n.z);
        tc.push_back(0.0f);
        tc.push_back(0.0f);
        return (int)(pos.size() / 3 - 1);
    }
    void tri(int a, int b, int c, int m)
    {
        idx.push_back(a);
        idx.push_back(b);
        idx.push_back(c);
        mat.push_back(m);
    }
    // Triangle whose geometric normal cross(b - a, c - a) faces `facing`.
    void triFacing(Vec a, Vec b, Vec c, Vec facing, int m, Vec n)
    {
        if (dotv(crossv(b - a, c - a), facing) < 0.0)
            std::swap(b, c);
        int i0 = addVertex(a, n), i1 = addVertex(b, n), i2 = addVertex(c, n);
        tri(i0, i1, i2, m);
    }
    void quad(Vec a, Vec b, Vec c, Vec d, Vec facing, int m)
    {
        Vec n = normv(facing);
        triFacing(a, b, c, facing, m, n);
        triFacing(a, c, d, facing, m, n);
    }
    // Axis-aligned box of half size h around the origin, rotated by `deg`
    // about +y, moved to `centre`; 12 triangles with outward normals.
    void box(Vec centre, Vec h, double deg, int m)
    {
        const double a = deg * 3.14159265358979323846 / 180.0, ca = std::cos(a), sa = std::sin(a);
        auto xf = [&](Vec p) { return Vec{ca * p.x + sa * p.z + centre.x, p.y + centre.y, -sa * p.x + ca * p.z + centre.z}; };
        auto rot = [&](Vec p) { return Vec{ca * p.x + sa * p.z, p.y, -sa * p.x + ca * p.z}; };
        for (int axis = 0; axis < 3; ++axis) {
            for (int sgn = -1; sgn <= 1; sgn += 2) {
                Vec n{0, 0, 0}, u{0, 0, 0}, v{0, 0, 0};
                if (axis == 0) {
                    n = {(double)sgn, 0, 0};
                    u = {0, h.y, 0};
                    v = {0, 0, h.z};
                } else if (axis == 1) {
                    n = {0, (double)sgn, 0};
                    u = {h.x, 0, 0};
                    v = {0, 0, h.z};
                } else {
                    n = {0, 0, (double)sgn};
                    u = {h.x, 0, 0};
                    v = {0, h.y, 0};
                }
                Vec c0{n.x * h.x, n.y * h.y, n.z * h.z};
                Vec p0 = xf(c0 - u - v), p1 = xf(c0 + u - v), p2 = xf(c0 + u + v), p3 = xf(c0 - u + v);
                quad(p0, p1, p2, p3, rot(n), m);
            }
        }
    }
    // Icosphere: icosahedron subdivided `levels` times (20 * 4^levels faces),
    // projected to the sphere, with per-vertex normals.
    void icosphere(Vec centre, double radius, int levels, int m, Vec scale = {1, 1, 1}, double yawDeg = 0.0)
    {
        const double t = (1.0 + std::sqrt(5.0)) / 2.0;
        std::vector<Vec> v = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                              {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
        for (auto &p : v)
            p = normv(p);
        std::vector<int> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                              11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                              3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
        for (int l = 0; l < levels; ++l) {
            std::map<std::pair<int, int>, int> mid;
            auto midpoint = [&](int a, int b) {
                std::pair<int, int> k(std::min(a, b), std::max(a, b));
                auto it = mid.find(k);
                if (it != mid.end())
                    return it->second;
                v.push_back(normv((v[a] + v[b]) * 0.5));
                int id = (int)v.size() - 1;
                mid[k] = id;
                return id;
            };
            std::vector<int> nf;
            nf.reserve(f.size() * 4);
            for (size_t i = 0; i < f.size(); i += 3) {
                int a = f[i], b = f[i + 1], c = f[i + 2];
                int ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
                int q[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
                nf.insert(nf.end(), q, q + 12);
            }
            f.swap(nf);
        }
        const double ya = yawDeg * 3.14159265358979323846 / 180.0, cy = std::cos(ya), sy = std::sin(ya);
        const int base = (int)(pos.size() / 3);
        for (const Vec &p : v) {
            Vec s{p.x * scale.x, p.y * scale.y, p.z * scale.z};
            Vec r{cy * s.x + sy * s.z, s.y, -sy * s.x + cy * s.z};
            Vec n = normv(Vec{p.x / scale.x, p.y / scale.y, p.z / scale.z});
            Vec rn{cy * n.x + sy * n.z, n.y, -sy * n.x + cy * n.z};
            addVertex(centre + r * radius, rn);
        }
        for (size_t i = 0; i < f.size(); i += 3) {
            int a = f[i], b = f[i + 1], c = f[i + 2];
            if (dotv(crossv(v[b] - v[a], v[c] - v[a]), v[a] + v[b] + v[c]) < 0.0)
                std::swap(b, c);
            tri(base + a, base + b, base + c, m);
        }
    }
    int addMaterial(MaterialData m)
    {
        m.category = hostCategory(m);
        materials.push_back(m);
        return (int)materials.size() - 1;
    }
};

template <class T> T *dup(const std::vector<T> &v)
{
    if (v.empty())
        return nullptr;
    T *p = (T *)malloc(sizeof(T) * v.size());
    if (p)
        memcpy(p, v.data(), sizeof(T) * v.size());
    return p;
}

void setv(float *d, double x, double y, double z)
{
    d[0] = (float)x;
    d[1] = (float)y;
    d[2] = (float)z;
}

int finish(Builder &b, optpt_scene *out)
{
    out->positions = dup(b.pos);
    out->numVertices = (uint32_t)(b.pos.size() / 3);
    out->normals = b.withNormals ? dup(b.nrm) : nullptr;
    out->texCoords = nullptr;
    out->triIndices = dup(b.idx);
    out->numTriangles = (uint32_t)b.mat.size();
    out->matIndices = dup(b.mat);
    out->materials = dup(b.materials);
    out->numMaterials = (uint32_t)b.materials.size();
    out->lights = dup(b.lights);
    out->numLights = (uint32_t)b.lights.size();
    out->textures = nullptr;
    out->numTextures = 0;
    return OPTPT_OK;
}

// Procedural Cornell box: room [-1,1]x[0,2]x[-1,1] of 10 wall triangles
// (open front), a 0.5 x 0.5 quad light at y = 1.99 with radiance (17,12,4),
// and two boxes of 12 triangles rotated -18 and +18 degrees about y. All
// surfaces are rough (roughness 1, Oren-Nayar) diffuse with specular 0.
int buildCornell(uint32_t, optpt_scene *out)
{
    Builder b;
    const int white = b.addMaterial(baseMaterial(0.73, 0.73, 0.73));
    const int red = b.addMaterial(baseMaterial(0.65, 0.05, 0.05));
    const int green = b.addMaterial(baseMaterial(0.12, 0.45, 0.15));
    MaterialData lm = baseMaterial(0.0, 0.0, 0.0);
    setv(lm.emission, 17.0, 12.0, 4.0);
    const int light = b.addMaterial(lm);
    b.quad({-1, 0, -1}, {1, 0, -1}, {1, 0, 1}, {-1, 0, 1}, {0, 1, 0}, white);    // floor
    b.quad({-1, 2, -1}, {1, 2, -1}, {1, 2, 1}, {-1, 2, 1}, {0, -1, 0}, white);   // ceiling
    b.quad({-1, 0, -1}, {1, 0, -1}, {1, 2, -1}, {-1, 2, -1}, {0, 0, 1}, white);  // back
    b.quad({-1, 0, -1}, {-1, 0, 1}, {-1, 2, 1}, {-1, 2, -1}, {1, 0, 0}, red);    // left
    b.quad({1, 0, -1}, {1, 0, 1}, {1, 2, 1}, {1, 2, -1}, {-1, 0, 0}, green);     // right
    b.quad({-0.25, 1.99, -0.25}, {0.25, 1.99, -0.25}, {0.25, 1.99, 0.25}, {-0.25, 1.99, 0.25}, {0, -1, 0}, light);
    b.box({0.35, 0.3, 0.3}, {0.3, 0.3, 0.3}, -18.0, white);
    b.box({-0.35, 0.6, -0.3}, {0.3, 0.6, 0.3}, 18.0, white);
    finish(b, out);
    setv(out->camEye, 0.0, 1.0, 3.4);
    setv(out->camTarget, 0.0, 1.0, 0.0);
    setv(out->camUp, 0.0, 1.0, 0.0);
    out->camFovYDeg = 40.0f;
    out->resX = 512;
    out->resY = 512;
    setv(out->bgColour, 0.0, 0.0, 0.0);
    out->spp = 64;
    out->maxDepth = 8;
    return OPTPT_OK;
}

// Material sweep: 8 x 8 icospheres (subdivision 4, 5,120 triangles each) on a
// ground plane; metallic 0 -> 1 by row, roughness 0.05 -> 1.0 by column, base
// colour U(0.2, 0.9)^3 from the seed, glTF default specular 1 and ior 1.5;
// one quad emitter and one point light of intensity 50.
int buildSpheres(uint32_t seed, optpt_scene *out)
{
    Builder b;
    b.withNormals = true;
    SceneRng rng{0x5eed0000ull + seed};
    MaterialData ground = baseMaterial(0.5, 0.5, 0.5);
    ground.roughness = 0.8f;
    const int groundM = b.addMaterial(ground);
    MaterialData lm = baseMaterial(0.0, 0.0, 0.0);
    setv(lm.emission, 6.0, 6.0, 6.0);
    const int lightM = b.addMaterial(lm);
    b.quad({-10, 0, -10}, {10, 0, -10}, {10, 0, 10}, {-10, 0, 10}, {0, 1, 0}, groundM);
    b.quad({-1.5, 6, -1.5}, {1.5, 6, -1.5}, {1.5, 6, 1.5}, {-1.5, 6, 1.5}, {0, -1, 0}, lightM);
    for (int row = 0; row < 8; ++row) {
        for (int col = 0; col < 8; ++col) {
            const double r = rng.range(0.2, 0.9), g = rng.range(0.2, 0.9), bl = rng.range(0.2, 0.9);
            MaterialData m = baseMaterial(r, g, bl);
            m.metallic = (float)(row / 7.0);
            m.roughness = (float)(0.05 + col * (0.95 / 7.0));
            m.specular = 1.0f;
            const int mi = b.addMaterial(m);
            b.icosphere({(col - 3.5) * 1.0, 0.4, (row - 3.5) * 1.0}, 0.4, 4, mi);
        }
    }
    Light pl;
    memset(&pl, 0, sizeof(pl));
    pl.type = LIGHT_TYPE_POINT;
    setv(pl.p0, -4.0, 5.0, 4.0);
    setv(pl.radiance, 50.0, 50.0, 50.0);
    setv(pl.colour, 1.0, 1.0, 1.0);
    b.lights.push_back(pl);
    finish(b, out);
    setv(out->camEye, 0.0, 5.5, 8.5);
    setv(out->camTarget, 0.0, 0.0, 0.3);
    setv(out->camUp, 0.0, 1.0, 0.0);
    out->camFovYDeg = 40.0f;
    out->resX = 1920;
    out->resY = 1080;
    setv(out->bgColour, 0.051, 0.051, 0.051);
    out->spp = 256;
    out->maxDepth = 12;
    return OPTPT_OK;
}

// ------------------------------------------------------------------ terrain
// Lattice value noise with smooth interpolation and fractal sums, all in
// double from integer hashes (identical on every host).
double hashUnit(int64_t x, int64_t y, uint64_t seed)
{
    uint64_t h = (uint64_t)x * 0x9E3779B97F4A7C15ull ^ (uint64_t)y * 0xC2B2AE3D27D4EB4Full ^ seed * 0x165667B19E3779F9ull;
    h ^= h >> 29;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 32;
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}
double valueNoise(double x, double y, uint64_t seed)
{
    const double fx = std::floor(x), fy = std::floor(y);
    const int64_t ix = (int64_t)fx, iy = (int64_t)fy;
    double tx = x - fx, ty = y - fy;
    tx = tx * tx * (3.0 - 2.0 * tx);
    ty = ty * ty * (3.0 - 2.0 * ty);
    const double a = hashUnit(ix, iy, seed), b = hashUnit(ix + 1, iy, seed);
    const double c = hashUnit(ix, iy + 1, seed), d = hashUnit(ix + 1, iy + 1, seed);
    return (a + (b - a) * tx) + ((c + (d - c) * tx) - (a + (b - a) * tx)) * ty;
}
double fbm(double x, double y, uint64_t seed, int octaves)
{
    double s = 0.0, amp = 0.5, f = 1.0;
    for (int o = 0; o < octaves; ++o) {
        s += amp * valueNoise(x * f, y * f, seed + (uint64_t)o * 1013u);
        amp *= 0.5;
        f *= 2.0;
    }
    return s;  // in [0, 1)
}

// 1024^2 RGBA8 textures of the alpha-masked quads: colour noise with an fBm
// alpha (about half below the 0.5 cutoff), and the tangent-space normal map
// of an fBm height field. Both tile.
void makeFoliageTextures(int res, uint64_t seed, std::vector<uint8_t> &albedo, std::vector<uint8_t> &normal)
{
    albedo.resize((size_t)res * res * 4);
    normal.resize((size_t)res * res * 4);
    const double period = 16.0;
    auto tiled = [&](double u, double v, uint64_t sd) {
        // bilinear blend of four offsets makes the pattern tile with the texture
        const double a = fbm(u, v, sd, 5), b = fbm(u - period, v, sd, 5);
        const double c = fbm(u, v - period, sd, 5), d = fbm(u - period, v - period, sd, 5);
        const double wu = u / period, wv = v / period;
        return (a * (1 - wu) + b * wu) * (1 - wv) + (c * (1 - wu) + d * wu) * wv;
    };
    std::vector<double> h((size_t)res * res);
    for (int y = 0; y < res; ++y)
        for (int x = 0; x < res; ++x) {
            const double u = period * x / res, v = period * y / res;
            const double n = tiled(u, v, seed), m = tiled(u * 2.0, v * 2.0, seed + 7);
            uint8_t *p = &albedo[4 * ((size_t)y * res + x)];
            p[0] = (uint8_t)std::lround(255.0 * (0.20 + 0.25 * m));
            p[1] = (uint8_t)std::lround(255.0 * (0.35 + 0.45 * n));
            p[2] = (uint8_t)std::lround(255.0 * (0.10 + 0.15 * m));
            p[3] = (uint8_t)std::lround(255.0 * std::fmin(1.0, std::fmax(0.0, (n - 0.5) * 6.0 + 0.5)));
            h[(size_t)y * res + x] = tiled(u * 3.0, v * 3.0, seed + 13);
        }
    for (int y = 0; y < res; ++y)
        for (int x = 0; x < res; ++x) {
            auto H = [&](int xx, int yy) { return h[(size_t)((yy + res) % res) * res + (size_t)((xx + res) % res)]; };
            const double dx = (H(x + 1, y) - H(x - 1, y)) * 0.5 * res * 0.02, dy = (H(x, y + 1) - H(x, y - 1)) * 0.5 * res * 0.02;
            Vec n = normv(Vec{-dx, -dy, 1.0});
            uint8_t *p = &normal[4 * ((size_t)y * res + x)];
            p[0] = (uint8_t)std::lround(255.0 * (n.x * 0.5 + 0.5));
            p[1] = (uint8_t)std::lround(255.0 * (n.y * 0.5 + 0.5));
            p[2] = (uint8_t)std::lround(255.0 * (n.z * 0.5 + 0.5));
            p[3] = 255;
        }
}

// Traversal-bound landscape: a grid x grid quad fBm terrain (seed 7), rocks
// (flattened, randomly scaled and rotated subdivision-1 icospheres; 30% rough
// glass: ior 1.5, transmission 1, roughness U(0, 0.3)), alpha-masked quads
// (20% of the rock count) with an RGBA8 noise texture (cutoff 0.5) and a
// tangent-space normal map, and a sun-like quad emitter. grid = 2048,
// rocks = 20000, texture 1024^2 gives the 10-million-triangle workload.
int buildTerrain(uint32_t seed, int grid, int rocks, int texRes, optpt_scene *out)
{
    Builder b;
    b.withNormals = true;
    SceneRng rng{0x7e44a100ull + seed};
    const double extent = 200.0, amp = 18.0;
    auto height = [&](double x, double z) { return amp * fbm(x / 25.0 + 100.0, z / 25.0 + 100.0, 7, 6); };

    MaterialData ground = baseMaterial(0.35, 0.30, 0.22);
    ground.roughness = 0.9f;
    const int groundM = b.addMaterial(ground);
    MaterialData sun = baseMaterial(0.0, 0.0, 0.0);
    setv(sun.emission, 40.0, 37.0, 32.0);
    const int sunM = b.addMaterial(sun);
    std::vector<int> rockM, glassM;
    for (int k = 0; k < 12; ++k) {
        MaterialData m = baseMaterial(rng.range(0.25, 0.6), rng.range(0.22, 0.5), rng.range(0.2, 0.45));
        m.roughness = (float)rng.range(0.4, 1.0);
        m.metallic = k % 4 == 0 ? 1.0f : 0.0f;
        m.specular = k % 3 == 0 ? 0.5f : 0.0f;
        rockM.push_back(b.addMaterial(m));
    }
    for (int k = 0; k < 16; ++k) {
        MaterialData m = baseMaterial(rng.range(0.8, 1.0), rng.range(0.85, 1.0), rng.range(0.85, 1.0));
        m.transmissionWeight = 1.0f;
        m.ior = 1.5f;
        m.roughness = (float)rng.range(0.0, 0.3);
        m.specular = 1.0f;
        glassM.push_back(b.addMaterial(m));
    }
    MaterialData leaf = baseMaterial(1.0, 1.0, 1.0);
    leaf.roughness = 0.7f;
    leaf.alphaMode = AM_MASK;
    leaf.alphaCutoff = 0.5f;
    leaf.baseColourTexture = 0;
    leaf.hasBaseColourTexture = 1;
    leaf.normalTexture = 1;
    leaf.hasNormalTexture = 1;
    leaf.baseColourTexTf.scale[0] = leaf.baseColourTexTf.scale[1] = 2.0f;
    leaf.normalTexTf.scale[0] = leaf.normalTexTf.scale[1] = 2.0f;
    const int leafM = b.addMaterial(leaf);

    // terrain: (grid + 1)^2 vertices with finite-difference normals
    const int nv = grid + 1;
    const double cell = extent / grid;
    const int base = (int)(b.pos.size() / 3);
    std::vector<double> hs((size_t)nv * nv);
    for (int j = 0; j < nv; ++j)
        for (int i = 0; i < nv; ++i)
            hs[(size_t)j * nv + i] = height(-extent / 2 + i * cell, -extent / 2 + j * cell);
    for (int j = 0; j < nv; ++j)
        for (int i = 0; i < nv; ++i) {
            auto H = [&](int ii, int jj) {
                ii = std::min(std::max(ii, 0), nv - 1);
                jj = std::min(std::max(jj, 0), nv - 1);
                return hs[(size_t)jj * nv + ii];
            };
            Vec n = normv(Vec{-(H(i + 1, j) - H(i - 1, j)) / (2 * cell), 1.0, -(H(i, j + 1) - H(i, j - 1)) / (2 * cell)});
            const int v = b.addVertex(Vec{-extent / 2 + i * cell, hs[(size_t)j * nv + i], -extent / 2 + j * cell}, n);
            b.tc[2 * v] = (float)(i * 0.25);
            b.tc[2 * v + 1] = (float)(j * 0.25);
        }
    for (int j = 0; j < grid; ++j)
        for (int i = 0; i < grid; ++i) {
            const int a = base + j * nv + i, c = a + 1, d = a + nv, e = d + 1;
            b.tri(a, d, c, groundM);  // normals face +y: cross(d - a, c - a) has +y
            b.tri(c, d, e, groundM);
        }
    // rocks
    for (int k = 0; k < rocks; ++k) {
        const double x = rng.range(-extent * 0.45, extent * 0.45), z = rng.range(-extent * 0.45, extent * 0.45);
        const double s = rng.range(0.3, 1.5), flat = rng.range(0.3, 0.6), yaw = rng.range(0.0, 360.0);
        const bool glass = rng.uniform() < 0.3;
        const int m = glass ? glassM[(size_t)(rng.uniform() * glassM.size()) % glassM.size()]
                            : rockM[(size_t)(rng.uniform() * rockM.size()) % rockM.size()];
        b.icosphere(Vec{x, height(x, z) + s * flat * 0.6, z}, s, 1, m, Vec{1.0, flat, rng.range(0.6, 1.0)}, yaw);
    }
    // alpha-masked quads (vertical, textured)
    const int quads = rocks / 5;
    for (int k = 0; k < quads; ++k) {
        const double x = rng.range(-extent * 0.45, extent * 0.45), z = rng.range(-extent * 0.45, extent * 0.45);
        const double w = rng.range(1.0, 3.0), hgt = rng.range(1.0, 3.0), yaw = rng.range(0.0, 3.14159265358979);
        const double y0 = height(x, z) - 0.1;
        const Vec ax{std::cos(yaw) * w * 0.5, 0.0, std::sin(yaw) * w * 0.5};
        const Vec c{x, y0, z};
        const Vec n = normv(Vec{-std::sin(yaw), 0.0, std::cos(yaw)});
        const Vec p[4] = {c - ax, c + ax, c + ax + Vec{0, hgt, 0}, c - ax + Vec{0, hgt, 0}};
        const double uv[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
        int id[4];
        for (int q = 0; q < 4; ++q) {
            id[q] = b.addVertex(p[q], n);
            b.tc[2 * id[q]] = (float)uv[q][0];
            b.tc[2 * id[q] + 1] = (float)uv[q][1];
        }
        b.tri(id[0], id[1], id[2], leafM);
        b.tri(id[0], id[2], id[3], leafM);
    }
    // sun: a 40 x 40 quad high above, facing down towards the terrain centre
    b.quad({60, 250, -20}, {100, 250, -20}, {100, 250, 20}, {60, 250, 20}, {0, -1, 0}, sunM);
    finish(b, out);
    out->texCoords = dup(b.tc);
    std::vector<uint8_t> alb, nrm;
    makeFoliageTextures(texRes, seed, alb, nrm);
    optpt_texture *tex = (optpt_texture *)calloc(2, sizeof(optpt_texture));
    tex[0].width = tex[0].height = (uint32_t)texRes;
    tex[0].rgba = dup(alb);
    tex[0].srgb = 1;
    tex[1].width = tex[1].height = (uint32_t)texRes;
    tex[1].rgba = dup(nrm);
    tex[1].srgb = 0;
    out->textures = tex;
    out->numTextures = 2;
    const double ex = -70.0, ez = -75.0;
    setv(out->camEye, ex, height(ex, ez) + 14.0, ez);
    setv(out->camTarget, 10.0, height(10.0, 10.0), 10.0);
    setv(out->camUp, 0.0, 1.0, 0.0);
    out->camFovYDeg = 45.0f;
    out->resX = 1920;
    out->resY = 1080;
    setv(out->bgColour, 0.30, 0.45, 0.70);
    out->spp = 64;
    out->maxDepth = 16;
    return OPTPT_OK;
}

// Indirect-lit interior: a closed 10 x 4 x 6 room (x in [-5, 5], y in [0, 4],
// z in [-3, 3]) whose only opening is a 1 x 2 doorway (z in [-0.5, 0.5],
// y in [0, 2]) through a 0.1-thick wall at x = 5. Outside, a 2 x 2 quad
// emitter of radiance 50 hangs on the outer face of that wall beside the
// doorway, facing away from the house, onto an outside ground and a bounce
// wall at x = 9. No point inside sees the emitter's front: everything inside
// is lit indirectly, through the doorway (next-event estimation finds no
// light from inside). The background is black. Furniture: tables and chairs
// of boxes, shelves, and `balls` icospheres of `subdiv` levels on the floor,
// table tops and shelves; materials are diffuse (roughness 1, no specular
// lobe) or GGX metal (roughness U(0.1, 0.6)).
int buildInterior(uint32_t seed, int balls, int subdiv, optpt_scene *out)
{
    Builder b;
    b.withNormals = true;
    SceneRng rng{0x1d00a7ull + seed};
    MaterialData wall = baseMaterial(0.72, 0.70, 0.66);
    wall.specular = 0.0f;
    const int wallM = b.addMaterial(wall);
    MaterialData floorMat = baseMaterial(0.45, 0.32, 0.20);
    floorMat.specular = 0.0f;
    const int floorM = b.addMaterial(floorMat);
    MaterialData light = baseMaterial(0.0, 0.0, 0.0);
    setv(light.emission, 50.0, 50.0, 50.0);
    const int lightM = b.addMaterial(light);
    MaterialData outside = baseMaterial(0.8, 0.78, 0.74);
    outside.specular = 0.0f;
    const int outM = b.addMaterial(outside);
    std::vector<int> furnM;
    for (int k = 0; k < 16; ++k) {
        MaterialData m = baseMaterial(rng.range(0.2, 0.9), rng.range(0.2, 0.9), rng.range(0.2, 0.9));
        if (k % 2 == 0) {
            m.metallic = 1.0f;
            m.roughness = (float)rng.range(0.1, 0.6);
        } else {
            m.specular = 0.0f;
        }
        furnM.push_back(b.addMaterial(m));
    }
    auto pick = [&]() { return furnM[(size_t)(rng.uniform() * furnM.size()) % furnM.size()]; };

    const double X = 5.0, Y = 4.0, Z = 3.0, dz = 0.5, dy = 2.0, T = 0.1, XO = X + T;
    b.quad({-X, 0, -Z}, {X, 0, -Z}, {X, 0, Z}, {-X, 0, Z}, {0, 1, 0}, floorM);      // floor
    b.quad({-X, Y, -Z}, {X, Y, -Z}, {X, Y, Z}, {-X, Y, Z}, {0, -1, 0}, wallM);      // ceiling
    b.quad({-X, 0, -Z}, {X, 0, -Z}, {X, Y, -Z}, {-X, Y, -Z}, {0, 0, 1}, wallM);     // back (z = -3)
    b.quad({-X, 0, Z}, {X, 0, Z}, {X, Y, Z}, {-X, Y, Z}, {0, 0, -1}, wallM);        // front (z = +3)
    b.quad({-X, 0, -Z}, {-X, 0, Z}, {-X, Y, Z}, {-X, Y, -Z}, {1, 0, 0}, wallM);     // x = -5
    // the door wall, inner face (x = 5) and outer face (x = 5.1) around the
    // doorway, and the doorway's jambs and lintel
    for (double x : {X, XO}) {
        const Vec f{x == X ? -1.0 : 1.0, 0, 0};
        b.quad({x, 0, -Z}, {x, 0, -dz}, {x, Y, -dz}, {x, Y, -Z}, f, wallM);
        b.quad({x, 0, dz}, {x, 0, Z}, {x, Y, Z}, {x, Y, dz}, f, wallM);
        b.quad({x, dy, -dz}, {x, dy, dz}, {x, Y, dz}, {x, Y, -dz}, f, wallM);
    }
    b.quad({X, 0, -dz}, {XO, 0, -dz}, {XO, dy, -dz}, {X, dy, -dz}, {0, 0, 1}, wallM);
    b.quad({X, 0, dz}, {XO, 0, dz}, {XO, dy, dz}, {X, dy, dz}, {0, 0, -1}, wallM);
    b.quad({X, dy, -dz}, {XO, dy, -dz}, {XO, dy, dz}, {X, dy, dz}, {0, -1, 0}, wallM);
    // outside: ground, bounce wall, and the emitter on the outer wall beside the door
    b.quad({XO, 0, -Z}, {9.0, 0, -Z}, {9.0, 0, Z}, {XO, 0, Z}, {0, 1, 0}, outM);
    b.quad({9.0, 0, -Z}, {9.0, 0, Z}, {9.0, Y, Z}, {9.0, Y, -Z}, {-1, 0, 0}, outM);
    b.quad({XO + 0.02, 0.3, 0.8}, {XO + 0.02, 0.3, 2.8}, {XO + 0.02, 2.3, 2.8}, {XO + 0.02, 2.3, 0.8}, {1, 0, 0},
           lightM);

    // tables (top + 4 legs) with chairs, keeping a lane from the doorway clear
    std::vector<Vec> tops;
    for (int t = 0; t < 6; ++t) {
        const double cx = -3.6 + 1.4 * t, cz = (t % 2 == 0) ? -1.7 : 1.7;
        const int m = pick();
        b.box({cx, 0.74, cz}, {0.5, 0.03, 0.4}, 0.0, m);
        for (int l = 0; l < 4; ++l)
            b.box({cx + (l & 1 ? 0.44 : -0.44), 0.36, cz + (l & 2 ? 0.34 : -0.34)}, {0.03, 0.36, 0.03}, 0.0, m);
        tops.push_back({cx, 0.77, cz});
        for (int c = 0; c < 2; ++c) {
            const double ox = c == 0 ? -0.75 : 0.75;
            const int cm = pick();
            b.box({cx + ox, 0.45, cz}, {0.2, 0.03, 0.2}, 0.0, cm);
            b.box({cx + ox + (c == 0 ? -0.18 : 0.18), 0.75, cz}, {0.02, 0.3, 0.2}, 0.0, cm);
            for (int l = 0; l < 4; ++l)
                b.box({cx + ox + (l & 1 ? 0.17 : -0.17), 0.21, cz + (l & 2 ? 0.17 : -0.17)}, {0.02, 0.21, 0.02}, 0.0, cm);
        }
    }
    // shelves along the back and front walls
    std::vector<Vec> shelves;
    for (int s = 0; s < 4; ++s) {
        const double cx = -3.0 + 2.0 * s, cz = (s % 2 == 0) ? -2.75 : 2.75;
        const int m = pick();
        for (int level = 0; level < 4; ++level) {
            b.box({cx, 0.3 + 0.6 * level, cz}, {0.7, 0.02, 0.2}, 0.0, m);
            shelves.push_back({cx, 0.32 + 0.6 * level, cz});
        }
        b.box({cx - 0.7, 1.1, cz}, {0.02, 1.1, 0.2}, 0.0, m);
        b.box({cx + 0.7, 1.1, cz}, {0.02, 1.1, 0.2}, 0.0, m);
    }
    // icospheres: on table tops, shelves and the floor
    for (int k = 0; k < balls; ++k) {
        const double u = rng.uniform();
        const int m = pick();
        if (u < 0.3) {
            const Vec &t = tops[(size_t)(rng.uniform() * tops.size()) % tops.size()];
            const double r = rng.range(0.05, 0.12);
            b.icosphere({t.x + rng.range(-0.38, 0.38), t.y + r, t.z + rng.range(-0.28, 0.28)}, r, subdiv, m);
        } else if (u < 0.6) {
            const Vec &s = shelves[(size_t)(rng.uniform() * shelves.size()) % shelves.size()];
            const double r = rng.range(0.04, 0.1);
            b.icosphere({s.x + rng.range(-0.6, 0.6), s.y + r, s.z + rng.range(-0.1, 0.1)}, r, subdiv, m);
        } else {
            const double r = rng.range(0.1, 0.35);
            double x = rng.range(-X + 0.4, X - 0.6), z = rng.range(-Z + 0.4, Z - 0.4);
            if (x > 2.5 && std::fabs(z) < 0.9)  // keep the doorway lane clear
                z = z < 0 ? z - 0.9 : z + 0.9;
            b.icosphere({x, r, z}, r, subdiv, m);
        }
    }
    finish(b, out);
    setv(out->camEye, -4.6, 1.6, -2.2);
    setv(out->camTarget, 1.5, 0.9, 1.2);
    setv(out->camUp, 0.0, 1.0, 0.0);
    out->camFovYDeg = 60.0f;
    out->resX = 1280;
    out->resY = 720;
    setv(out->bgColour, 0.0, 0.0, 0.0);
    out->spp = 64;
    out->maxDepth = 12;
    return OPTPT_OK;
}

}  // namespace

extern "C" {

int optpt_scene_procedural(const char *name, uint32_t seed, optpt_scene *out)
{
    if (!name || !out)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    memset(out, 0, sizeof(*out));
    if (strcmp(name, "cornell") == 0)
        return buildCornell(seed, out);
    if (strcmp(name, "spheres") == 0)
        return buildSpheres(seed, out);
    if (strcmp(name, "terrain") == 0)
        return buildTerrain(seed, 2048, 20000, 1024, out);
    if (strcmp(name, "terrain_small") == 0)
        return buildTerrain(seed, 96, 400, 128, out);
    if (strcmp(name, "interior") == 0)
        return buildInterior(seed, 380, 4, out);
    if (strcmp(name, "interior_small") == 0)
        return buildInterior(seed, 60, 2, out);
    return optpt_internal_set_error(OPTPT_ERR_INVALID, (std::string("unknown procedural scene '") + name + "'").c_str());
}

void optpt_scene_release(optpt_scene *s)
{
    if (!s)
        return;
    free((void *)s->positions);
    free((void *)s->normals);
    free((void *)s->texCoords);
    free((void *)s->triIndices);
    free((void *)s->matIndices);
    free((void *)s->materials);
    free((void *)s->lights);
    if (s->textures) {
        for (uint32_t t = 0; t < s->numTextures; ++t)
            free((void *)s->textures[t].rgba);
        free((void *)s->textures);
    }
    memset(s, 0, sizeof(*s));
}

// getSceneFilename + SceneDesc::parse (src/scene_desc.cpp:50-153 of the
// reference): {"scene": id, id: name} names <dir>/<name>.json, whose "scene"
// object holds the scene source and a "renderer" object.
int optpt_scene_from_config(const char *sceneListPath, optpt_scene *out)
{
    if (!sceneListPath || !out)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    memset(out, 0, sizeof(*out));
    std::string listText, sceneText;
    const std::string listPath(sceneListPath);
    if (!readFile(listPath, listText))
        return optpt_internal_set_error(OPTPT_ERR_IO, ("cannot read scene list " + listPath).c_str());
    Json list;
    int rc = parseJson(listText, list, "scene list");
    if (rc)
        return rc;
    const Json *id = list.type == Json::Obj ? list.get("scene") : nullptr;
    if (!id || id->type != Json::Str)
        return optpt_internal_set_error(OPTPT_ERR_PARSE, "invalid scene list file format");
    const Json *name = list.get(id->str);
    if (!name || name->type != Json::Str)
        return optpt_internal_set_error(OPTPT_ERR_PARSE, ("scene with ID " + id->str + " not found").c_str());
    const size_t slash = listPath.find_last_of("/\\");
    const std::string dir = slash == std::string::npos ? std::string() : listPath.substr(0, slash + 1);
    const std::string scenePath = dir + name->str + ".json";
    if (!readFile(scenePath, sceneText))
        return optpt_internal_set_error(OPTPT_ERR_IO, ("cannot read scene file " + scenePath).c_str());
    Json doc;
    if ((rc = parseJson(sceneText, doc, "scene file")))
        return rc;
    const Json *scene = doc.type == Json::Obj ? doc.get("scene") : nullptr;
    if (!scene || scene->type != Json::Obj)
        return optpt_internal_set_error(OPTPT_ERR_PARSE, "object \"scene\" not found");
    const Json *proc = scene->get("procedural scene");
    const Json *gltf = scene->get("gltf scene file");
    if (proc && proc->type == Json::Str) {
        uint32_t seed = 1;
        if (const Json *sd = scene->get("seed"))
            if (sd->type == Json::Num)
                seed = (uint32_t)sd->num;
        if ((rc = optpt_scene_procedural(proc->str.c_str(), seed, out)))
            return rc;
    } else if (gltf && gltf->type == Json::Str) {
        // SceneDesc::parseGltfScene (src/scene_desc.cpp:78-93): the file as
        // given (the reference opens it relative to the working directory),
        // else relative to this scene file; up hint default (0, 1, 0).
        float up[3] = {0.0f, 1.0f, 0.0f};
        if (const Json *uh = scene->get("gltf up hint"))
            if (!vec3(uh, up))
                return optpt_internal_set_error(OPTPT_ERR_PARSE, "\"gltf up hint\" must be [x, y, z]");
        std::string path = gltf->str, probe;
        const bool absolute = !path.empty() && (path[0] == '/' || path[0] == '\\');
        if (!absolute && !readFile(path, probe) && readFile(dir + path, probe))
            path = dir + path;
        if ((rc = optpt_scene_from_gltf(path.c_str(), up, out)))
            return rc;
    } else {
        return optpt_internal_set_error(OPTPT_ERR_PARSE, "no scene source in \"scene\"");
    }
    const Json *ren = scene->get("renderer");
    if (!ren || ren->type != Json::Obj) {
        optpt_scene_release(out);
        return optpt_internal_set_error(OPTPT_ERR_PARSE, "object \"renderer\" not found");
    }
    const Json *dims = ren->get("dimensions");
    if (!dims || dims->type != Json::Arr || dims->arr.size() != 2 || dims->arr[0].type != Json::Num ||
        dims->arr[1].type != Json::Num || dims->arr[0].num < 1 || dims->arr[1].num < 1) {
        optpt_scene_release(out);
        return optpt_internal_set_error(OPTPT_ERR_PARSE, "renderer.dimensions must be [width, height]");
    }
    out->resX = (uint32_t)dims->arr[0].num;
    out->resY = (uint32_t)dims->arr[1].num;
    if (const Json *bg = ren->get("background colour"))
        if (!vec3(bg, out->bgColour)) {
            optpt_scene_release(out);
            return optpt_internal_set_error(OPTPT_ERR_PARSE, "renderer.background colour must be [r, g, b]");
        }
    if (const Json *spp = ren->get("spp"))
        if (spp->type == Json::Num)
            out->spp = (uint32_t)spp->num;
    if (const Json *md = ren->get("max depth"))
        if (md->type == Json::Num)
            out->maxDepth = (uint32_t)md->num;
    return OPTPT_OK;
}

}  // extern "C"
