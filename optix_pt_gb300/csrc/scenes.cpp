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

extern "C" int optpt_internal_set_error(int code, const char *msg);

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

// ------------------------------------------------------------------ JSON
// A small recursive-descent JSON reader for the scene-selection files (the
// reference uses rapidjson, src/scene_desc.cpp:50-153).
struct Json {
    enum Type { Null, Bool, Num, Str, Arr, Obj } type = Null;
    double num = 0;
    bool b = false;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;
    const Json *get(const std::string &k) const
    {
        for (auto &kv : obj)
            if (kv.first == k)
                return &kv.second;
        return nullptr;
    }
};

struct JsonParser {
    const std::string &s;
    size_t i = 0;
    std::string err;
    explicit JsonParser(const std::string &src) : s(src) {}
    void ws()
    {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r'))
            ++i;
    }
    bool fail(const char *m)
    {
        if (err.empty())
            err = std::string(m) + " at offset " + std::to_string(i);
        return false;
    }
    bool value(Json &v, int depth)
    {
        if (depth > 64)
            return fail("nesting too deep");
        ws();
        if (i >= s.size())
            return fail("unexpected end");
        char c = s[i];
        if (c == '{') {
            v.type = Json::Obj;
            ++i;
            ws();
            if (i < s.size() && s[i] == '}') {
                ++i;
                return true;
            }
            while (true) {
                ws();
                Json k;
                if (i >= s.size() || s[i] != '"' || !string(k.str))
                    return fail("expected member name");
                ws();
                if (i >= s.size() || s[i] != ':')
                    return fail("expected ':'");
                ++i;
                Json val;
                if (!value(val, depth + 1))
                    return false;
                v.obj.emplace_back(k.str, std::move(val));
                ws();
                if (i < s.size() && s[i] == ',') {
                    ++i;
                    continue;
                }
                if (i < s.size() && s[i] == '}') {
                    ++i;
                    return true;
                }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.type = Json::Arr;
            ++i;
            ws();
            if (i < s.size() && s[i] == ']') {
                ++i;
                return true;
            }
            while (true) {
                Json val;
                if (!value(val, depth + 1))
                    return false;
                v.arr.push_back(std::move(val));
                ws();
                if (i < s.size() && s[i] == ',') {
                    ++i;
                    continue;
                }
                if (i < s.size() && s[i] == ']') {
                    ++i;
                    return true;
                }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.type = Json::Str;
            return string(v.str);
        }
        if (s.compare(i, 4, "true") == 0) {
            v.type = Json::Bool;
            v.b = true;
            i += 4;
            return true;
        }
        if (s.compare(i, 5, "false") == 0) {
            v.type = Json::Bool;
            i += 5;
            return true;
        }
        if (s.compare(i, 4, "null") == 0) {
            i += 4;
            return true;
        }
        if (c == '-' || (c >= '0' && c <= '9')) {
            const char *b0 = s.c_str() + i;
            char *e = nullptr;
            v.num = std::strtod(b0, &e);
            if (e == b0)
                return fail("bad number");
            v.type = Json::Num;
            i += (size_t)(e - b0);
            return true;
        }
        return fail("unexpected character");
    }
    bool string(std::string &out)
    {
        ++i;  // opening quote
        while (i < s.size() && s[i] != '"') {
            if (s[i] == '\\') {
                if (i + 1 >= s.size())
                    return fail("bad escape");
                char e = s[i + 1];
                out.push_back(e == 'n' ? '\n' : e == 't' ? '\t' : e);
                i += 2;
            } else {
                out.push_back(s[i++]);
            }
        }
        if (i >= s.size())
            return fail("missing closing quote");
        ++i;
        return true;
    }
};

bool readFile(const std::string &path, std::string &out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f)
        return false;
    std::stringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return !out.empty();
}

int parseJson(const std::string &text, Json &out, const std::string &what)
{
    JsonParser p(text);
    if (!p.value(out, 0))
        return optpt_internal_set_error(OPTPT_ERR_PARSE, ("error parsing " + what + ": " + p.err).c_str());
    p.ws();
    if (p.i != text.size())
        return optpt_internal_set_error(OPTPT_ERR_PARSE, ("error parsing " + what + ": trailing characters").c_str());
    return OPTPT_OK;
}

bool vec3(const Json *j, float *d)
{
    if (!j || j->type != Json::Arr || j->arr.size() != 3)
        return false;
    for (int k = 0; k < 3; ++k) {
        if (j->arr[k].type != Json::Num)
            return false;
        d[k] = (float)j->arr[k].num;
    }
    return true;
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
    if (!proc || proc->type != Json::Str) {
        if (scene->get("gltf scene file"))
            return optpt_internal_set_error(OPTPT_ERR_INVALID, "glTF scene files are not supported; use \"procedural scene\"");
        return optpt_internal_set_error(OPTPT_ERR_PARSE, "no scene source in \"scene\"");
    }
    uint32_t seed = 1;
    if (const Json *sd = scene->get("seed"))
        if (sd->type == Json::Num)
            seed = (uint32_t)sd->num;
    if ((rc = optpt_scene_procedural(proc->str.c_str(), seed, out)))
        return rc;
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
