// glTF 2.0 import: the reference's GltfLoader (src/gltf_loader.cpp:19-1388)
// plus the scene set-up of Renderer::loadScene / updateScene
// (src/renderer.cpp:191-265, 1060-1303), producing the flattened world-space
// optpt_scene the renderer consumes.
//
// What is read, and how it maps (reference line numbers in brackets):
// * the default scene's node tree; local transforms from "matrix" or T*R*S
//   (updateGlobalTransform :1228-1278), world = parent * local, in float;
// * every mesh node's triangle primitives (:908-1220): POSITION, NORMAL,
//   TEXCOORD_0, indices; positions go through the node's world matrix and
//   normals through its inverse transpose (src/renderer.cpp:1265-1275), not
//   renormalised; skinned meshes in their rest pose (joint matrices
//   inverse(world) * jointWorld * inverseBind, src/renderer.cpp:1163-1182);
// * materials (initMaterialParams :445-906) with the reference's defaults and
//   quirks: specular 1 unless KHR_materials_specular says otherwise; the
//   emissive texture only when emissiveFactor is non-zero; sheen only when
//   sheenColorFactor is present and sheen roughness only when
//   sheenRoughnessFactor is; texture transforms carry offset, rotation and
//   scale and every texture reads TEXCOORD_0;
// * textures (PNG, baseline JPEG) as RGBA8 (stb's four-component decode): the base-colour
//   texture takes its sampler's wrap modes and magnification filter, the
//   others repeat and filter linearly (src/renderer.cpp:1439-1757); base
//   colour, emissive and both sheen textures decode sRGB;
// * KHR_lights_punctual (loadLight :1280-1360): wattage = intensity / 683 *
//   4 pi, then src/light.cpp's point / directional (distance 1000) / spot
//   records; the first perspective camera (loadCamera :1362-1388): eye =
//   world * (0,0,0,1), target = world * (0,0,-1,1), up from the scene
//   description's "gltf up hint".
// Differences, each because the reference's behaviour is undefined or a
// crash: primitives without a material (-1) get the glTF default material
// appended at the end; primitives without normals in a scene that has some
// are unindexed and given their face normal (the reference's normal array
// falls out of step); TEXCOORD_0 missing on one primitive gives that
// primitive zero coordinates; triangle strips and fans are converted;
// points and lines are skipped; .glb containers, data: URIs, unsigned byte
// indices, normalised integer attributes and sparse accessors are read.
// The file is compiled without floating-point contraction.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <vector>
#include "../../include/optpt.h"
#include "host_scene.h"
#include "image_io.h"
#include "json.h"

extern "C" int optpt_internal_set_error(int code, const char *msg);

using optjson::Json;

namespace {

// Column-major 4x4 float matrix, m[c][r] as glm stores it.
struct Mat4 {
    float m[4][4];
    static Mat4 identity()
    {
        Mat4 a{};
        for (int i = 0; i < 4; ++i)
            a.m[i][i] = 1.0f;
        return a;
    }
};

Mat4 mul(const Mat4 &a, const Mat4 &b)
{
    Mat4 r{};
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) {
            float s = a.m[0][row] * b.m[c][0];
            s = s + a.m[1][row] * b.m[c][1];
            s = s + a.m[2][row] * b.m[c][2];
            s = s + a.m[3][row] * b.m[c][3];
            r.m[c][row] = s;
        }
    return r;
}

void xform(const Mat4 &a, const float v[4], float out[3])
{
    for (int row = 0; row < 3; ++row) {
        float s = a.m[0][row] * v[0];
        s = s + a.m[1][row] * v[1];
        s = s + a.m[2][row] * v[2];
        s = s + a.m[3][row] * v[3];
        out[row] = s;
    }
}

// Rotation matrix of a unit quaternion (x, y, z, w).
Mat4 fromQuat(float x, float y, float z, float w)
{
    Mat4 r = Mat4::identity();
    const float xx = x * x, yy = y * y, zz = z * z, xz = x * z, xy = x * y, yz = y * z, wx = w * x, wy = w * y,
                wz = w * z;
    r.m[0][0] = 1.0f - 2.0f * (yy + zz);
    r.m[0][1] = 2.0f * (xy + wz);
    r.m[0][2] = 2.0f * (xz - wy);
    r.m[1][0] = 2.0f * (xy - wz);
    r.m[1][1] = 1.0f - 2.0f * (xx + zz);
    r.m[1][2] = 2.0f * (yz + wx);
    r.m[2][0] = 2.0f * (xz + wy);
    r.m[2][1] = 2.0f * (yz - wx);
    r.m[2][2] = 1.0f - 2.0f * (xx + yy);
    return r;
}

// Inverse transpose of the upper 3x3 (in double, rounded once).
void normalMatrix(const Mat4 &a, float n[3][3])
{
    double m[3][3];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r)
            m[r][c] = a.m[c][r];
    const double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1], c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2],
                 c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    const double det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
    const double inv = det != 0.0 ? 1.0 / det : 0.0;
    // (M^-1)^T = cofactor matrix / det; n[r][c] multiplies normal component c.
    n[0][0] = (float)(c00 * inv);
    n[0][1] = (float)(c01 * inv);
    n[0][2] = (float)(c02 * inv);
    n[1][0] = (float)((m[0][2] * m[2][1] - m[0][1] * m[2][2]) * inv);
    n[1][1] = (float)((m[0][0] * m[2][2] - m[0][2] * m[2][0]) * inv);
    n[1][2] = (float)((m[0][1] * m[2][0] - m[0][0] * m[2][1]) * inv);
    n[2][0] = (float)((m[0][1] * m[1][2] - m[0][2] * m[1][1]) * inv);
    n[2][1] = (float)((m[0][2] * m[1][0] - m[0][0] * m[1][2]) * inv);
    n[2][2] = (float)((m[0][0] * m[1][1] - m[0][1] * m[1][0]) * inv);
}

double num(const Json *j, double dflt)
{
    return j && j->isNum() ? j->num : dflt;
}
int inum(const Json *j, int dflt)
{
    return j && j->isNum() ? (int)j->num : dflt;
}
const Json *child(const Json *j, const char *k)
{
    return j && j->isObj() ? j->get(k) : nullptr;
}
const Json *elem(const Json *arr, int i)
{
    if (!arr || !arr->isArr() || i < 0 || (size_t)i >= arr->arr.size())
        return nullptr;
    return &arr->arr[(size_t)i];
}

struct Err {
    int code = 0;
    std::string msg;
    bool set(int c, const std::string &m)
    {
        if (!code) {
            code = c;
            msg = m;
        }
        return false;
    }
};

bool base64(const std::string &s, size_t from, std::vector<uint8_t> &out)
{
    auto val = [](char c) -> int {
        if (c >= 'A' && c <= 'Z')
            return c - 'A';
        if (c >= 'a' && c <= 'z')
            return c - 'a' + 26;
        if (c >= '0' && c <= '9')
            return c - '0' + 52;
        if (c == '+' || c == '-')
            return 62;
        if (c == '/' || c == '_')
            return 63;
        return -1;
    };
    uint32_t acc = 0;
    int bits = 0;
    for (size_t i = from; i < s.size(); ++i) {
        const char c = s[i];
        if (c == '=')
            break;
        const int v = val(c);
        if (v < 0)
            return false;
        acc = (acc << 6) | (uint32_t)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((uint8_t)(acc >> bits));
        }
    }
    return true;
}

std::string percentDecode(const std::string &u)
{
    std::string o;
    for (size_t i = 0; i < u.size(); ++i) {
        if (u[i] == '%' && i + 2 < u.size()) {
            char h[3] = {u[i + 1], u[i + 2], 0};
            char *e = nullptr;
            long v = strtol(h, &e, 16);
            if (e == h + 2) {
                o.push_back((char)v);
                i += 2;
                continue;
            }
        }
        o.push_back(u[i]);
    }
    return o;
}

// A parsed glTF document with its buffers.
struct Doc {
    Json j;
    std::string dir;
    std::vector<std::vector<uint8_t>> buffers;
    std::vector<uint8_t> glbBin;
    bool hasGlbBin = false;
    Err err;

    const Json *arr(const char *k) const { return j.get(k); }
    const Json *at(const char *k, int i) const { return elem(j.get(k), i); }

    bool loadUri(const std::string &uri, std::vector<uint8_t> &out, const char *what)
    {
        if (uri.compare(0, 5, "data:") == 0) {
            const size_t comma = uri.find(',');
            if (comma == std::string::npos || uri.rfind(";base64", comma) == std::string::npos ||
                !base64(uri, comma + 1, out))
                return err.set(OPTPT_ERR_PARSE, std::string("unsupported data URI in ") + what);
            return true;
        }
        std::string data;
        const std::string path = dir + percentDecode(uri);
        if (!optjson::readFile(path, data))
            return err.set(OPTPT_ERR_IO, "cannot read " + path);
        out.assign(data.begin(), data.end());
        return true;
    }

    bool loadBuffers()
    {
        const Json *bs = arr("buffers");
        if (!bs)
            return true;
        buffers.resize(bs->arr.size());
        for (size_t b = 0; b < bs->arr.size(); ++b) {
            const Json &bj = bs->arr[b];
            const Json *uri = child(&bj, "uri");
            const size_t len = (size_t)num(child(&bj, "byteLength"), 0);
            if (!uri || !uri->isStr()) {
                if (b == 0 && hasGlbBin) {
                    buffers[b] = glbBin;
                } else {
                    return err.set(OPTPT_ERR_PARSE, "buffer " + std::to_string(b) + " has no data");
                }
            } else if (!loadUri(uri->str, buffers[b], "buffer")) {
                return false;
            }
            if (buffers[b].size() < len)
                return err.set(OPTPT_ERR_PARSE, "buffer " + std::to_string(b) + " shorter than byteLength");
        }
        return true;
    }

    // Byte range of a buffer view: pointer, length, stride (0 = packed).
    bool view(int v, const uint8_t *&p, size_t &len, size_t &stride)
    {
        const Json *bv = at("bufferViews", v);
        if (!bv)
            return err.set(OPTPT_ERR_PARSE, "bufferView " + std::to_string(v) + " missing");
        const int b = inum(child(bv, "buffer"), -1);
        if (b < 0 || (size_t)b >= buffers.size())
            return err.set(OPTPT_ERR_PARSE, "bufferView " + std::to_string(v) + ": bad buffer");
        const size_t off = (size_t)num(child(bv, "byteOffset"), 0);
        len = (size_t)num(child(bv, "byteLength"), 0);
        stride = (size_t)num(child(bv, "byteStride"), 0);
        if (off > buffers[b].size() || len > buffers[b].size() - off)
            return err.set(OPTPT_ERR_PARSE, "bufferView " + std::to_string(v) + " out of range");
        p = buffers[b].data() + off;
        return true;
    }

    // Reads an accessor as `count` rows of `comps` floats (integer types
    // converted; normalised integers scaled as the glTF spec defines).
    bool readFloats(int a, int wantComps, std::vector<float> &out, size_t &count)
    {
        const Json *ac = at("accessors", a);
        if (!ac)
            return err.set(OPTPT_ERR_PARSE, "accessor " + std::to_string(a) + " missing");
        const int ct = inum(child(ac, "componentType"), 0);
        const Json *tj = child(ac, "type");
        const std::string type = tj && tj->isStr() ? tj->str : "";
        const int comps = type == "SCALAR" ? 1 : type == "VEC2" ? 2 : type == "VEC3" ? 3 : type == "VEC4" ? 4
                        : type == "MAT4" ? 16 : 0;
        if (comps == 0 || comps < wantComps)
            return err.set(OPTPT_ERR_PARSE, "accessor " + std::to_string(a) + ": unexpected type " + type);
        const bool normalized = child(ac, "normalized") && child(ac, "normalized")->b;
        const size_t csize = ct == 5120 || ct == 5121 ? 1 : ct == 5122 || ct == 5123 ? 2 : ct == 5125 || ct == 5126 ? 4 : 0;
        if (!csize)
            return err.set(OPTPT_ERR_PARSE, "accessor " + std::to_string(a) + ": bad componentType");
        count = (size_t)num(child(ac, "count"), 0);
        out.assign(count * (size_t)wantComps, 0.0f);
        auto conv = [&](const uint8_t *q) -> float {
            switch (ct) {
            case 5126: {
                float f;
                memcpy(&f, q, 4);
                return f;
            }
            case 5120: {
                const float v = (float)(int8_t)q[0];
                return normalized ? std::fmax(v / 127.0f, -1.0f) : v;
            }
            case 5121: return normalized ? (float)q[0] / 255.0f : (float)q[0];
            case 5122: {
                int16_t s;
                memcpy(&s, q, 2);
                return normalized ? std::fmax((float)s / 32767.0f, -1.0f) : (float)s;
            }
            case 5123: {
                uint16_t s;
                memcpy(&s, q, 2);
                return normalized ? (float)s / 65535.0f : (float)s;
            }
            default: {
                uint32_t s;
                memcpy(&s, q, 4);
                return (float)s;
            }
            }
        };
        const Json *bvj = child(ac, "bufferView");
        if (bvj && bvj->isNum()) {
            const uint8_t *p;
            size_t len, stride;
            if (!view((int)bvj->num, p, len, stride))
                return false;
            const size_t off = (size_t)num(child(ac, "byteOffset"), 0);
            const size_t elem = csize * (size_t)comps;
            if (!stride)
                stride = elem;
            if (count && (off > len || (count - 1) * stride + elem > len - off))
                return err.set(OPTPT_ERR_PARSE, "accessor " + std::to_string(a) + " runs past its bufferView");
            for (size_t i = 0; i < count; ++i)
                for (int c = 0; c < wantComps; ++c)
                    out[i * wantComps + c] = conv(p + off + i * stride + (size_t)c * csize);
        }
        if (const Json *sp = child(ac, "sparse")) {
            const size_t n = (size_t)num(child(sp, "count"), 0);
            const Json *ij = child(sp, "indices"), *vj = child(sp, "values");
            const uint8_t *ip, *vp;
            size_t il, is, vl, vs;
            if (!ij || !vj || !view(inum(child(ij, "bufferView"), -1), ip, il, is) ||
                !view(inum(child(vj, "bufferView"), -1), vp, vl, vs))
                return err.code ? false : err.set(OPTPT_ERR_PARSE, "bad sparse accessor");
            const int ict = inum(child(ij, "componentType"), 5125);
            const size_t isz = ict == 5121 ? 1 : ict == 5123 ? 2 : 4;
            const size_t ioff = (size_t)num(child(ij, "byteOffset"), 0), voff = (size_t)num(child(vj, "byteOffset"), 0);
            const size_t elem = csize * (size_t)comps;
            if (ioff + n * isz > il || voff + n * elem > vl)
                return err.set(OPTPT_ERR_PARSE, "sparse accessor out of range");
            for (size_t k = 0; k < n; ++k) {
                uint32_t idx = 0;
                memcpy(&idx, ip + ioff + k * isz, isz);
                if (idx >= count)
                    return err.set(OPTPT_ERR_PARSE, "sparse index out of range");
                for (int c = 0; c < wantComps; ++c)
                    out[idx * wantComps + c] = conv(vp + voff + k * elem + (size_t)c * csize);
            }
        }
        return true;
    }

    bool readIndices(int a, std::vector<uint32_t> &out)
    {
        const Json *ac = at("accessors", a);
        const int ct = inum(child(ac, "componentType"), 0);
        if (ct != 5121 && ct != 5123 && ct != 5125)
            return err.set(OPTPT_ERR_PARSE, "index accessor " + std::to_string(a) + ": bad componentType");
        std::vector<float> f;
        size_t n;
        // Unsigned 32-bit indices above 2^24 would not survive float: read
        // them directly.
        if (ct == 5125 && child(ac, "bufferView") && !child(ac, "sparse")) {
            const uint8_t *p;
            size_t len, stride;
            if (!view(inum(child(ac, "bufferView"), -1), p, len, stride))
                return false;
            n = (size_t)num(child(ac, "count"), 0);
            const size_t off = (size_t)num(child(ac, "byteOffset"), 0);
            if (!stride)
                stride = 4;
            if (n && (off > len || (n - 1) * stride + 4 > len - off))
                return err.set(OPTPT_ERR_PARSE, "index accessor runs past its bufferView");
            out.resize(n);
            for (size_t i = 0; i < n; ++i)
                memcpy(&out[i], p + off + i * stride, 4);
            return true;
        }
        if (!readFloats(a, 1, f, n))
            return false;
        out.resize(n);
        for (size_t i = 0; i < n; ++i)
            out[i] = (uint32_t)f[i];
        return true;
    }
};

struct Loader {
    Doc &d;
    const float *up;
    std::vector<float> pos, nrm, tc;
    std::vector<int32_t> idx, mat;
    std::vector<MaterialData> materials;
    std::vector<Light> lights;
    std::vector<optpt_texture> textures;
    std::map<std::tuple<int, int, int, int, int>, int> texKey;  // image, wrapS, wrapT, srgb, filter
    std::map<int, optimg::Image> images;
    bool anyNormals = false, anyTexCoords = false;
    int defaultMaterial = -1;
    bool camera = false;
    float camEye[3] = {0, 0, 0}, camTarget[3] = {0, 0, -1}, fovYDeg = 45.0f;
    std::vector<Mat4> world;  // per glTF node, rest pose

    // Deformation data: every emitted vertex in its shape's (mesh node's)
    // space, the shape it belongs to and, for skinned shapes, four joint
    // slots and weights. A shape's joint slots are its own (the joint
    // matrices depend on the mesh node's world matrix).
    std::vector<uint32_t> vShape;
    std::vector<uint16_t> vJoints;
    std::vector<float> vWeights;
    bool anySkin = false;
    struct Shape {
        int node, skin, jointBase;
    };
    std::vector<Shape> shapes;
    struct Skin {
        std::vector<int> joints;
        std::vector<Mat4> ibm;
    };
    std::map<int, Skin> skins;
    int jointSlots = 0;

    Loader(Doc &doc, const float *upHint) : d(doc), up(upHint) {}

    Mat4 local(const Json &node)
    {
        const Json *m = child(&node, "matrix");
        if (m && m->isArr() && m->arr.size() == 16) {
            Mat4 r;
            for (int i = 0; i < 16; ++i)
                r.m[i / 4][i % 4] = (float)num(&m->arr[(size_t)i], 0);
            return r;
        }
        Mat4 t = Mat4::identity(), r = Mat4::identity(), s = Mat4::identity();
        if (const Json *tj = child(&node, "translation"))
            if (tj->isArr() && tj->arr.size() == 3)
                for (int k = 0; k < 3; ++k)
                    t.m[3][k] = (float)num(&tj->arr[(size_t)k], 0);
        if (const Json *rj = child(&node, "rotation"))
            if (rj->isArr() && rj->arr.size() == 4)
                r = fromQuat((float)num(&rj->arr[0], 0), (float)num(&rj->arr[1], 0), (float)num(&rj->arr[2], 0),
                             (float)num(&rj->arr[3], 1));
        if (const Json *sj = child(&node, "scale"))
            if (sj->isArr() && sj->arr.size() == 3)
                for (int k = 0; k < 3; ++k)
                    s.m[k][k] = (float)num(&sj->arr[(size_t)k], 1);
        return mul(mul(t, r), s);
    }

    // Computes world matrices of the whole tree under `n` (all nodes, so that
    // skin joints outside the mesh's subtree are known).
    bool worlds(int n, const Mat4 &parent, int depth)
    {
        const Json *node = d.at("nodes", n);
        if (!node || depth > 256)
            return d.err.set(OPTPT_ERR_PARSE, "bad node " + std::to_string(n));
        world[(size_t)n] = mul(parent, local(*node));
        if (const Json *ch = child(node, "children"))
            for (auto &c : ch->arr)
                if (!worlds(inum(&c, -1), world[(size_t)n], depth + 1))
                    return false;
        return true;
    }

    int texture(int texIndex, bool srgb, bool useSampler)
    {
        const Json *t = d.at("textures", texIndex);
        if (!t) {
            d.err.set(OPTPT_ERR_PARSE, "texture " + std::to_string(texIndex) + " missing");
            return -2;
        }
        const int img = inum(child(t, "source"), -1);
        int wrapS = 0, wrapT = 0, filter = 0;
        if (useSampler) {
            if (const Json *s = d.at("samplers", inum(child(t, "sampler"), -1))) {
                auto wrap = [](int w) { return w == 33071 ? 1 : w == 33648 ? 2 : 0; };
                wrapS = wrap(inum(child(s, "wrapS"), 10497));
                wrapT = wrap(inum(child(s, "wrapT"), 10497));
                filter = inum(child(s, "magFilter"), 9729) == 9728 ? 1 : 0;
            }
        }
        auto key = std::make_tuple(img, wrapS, wrapT, srgb ? 1 : 0, filter);
        auto it = texKey.find(key);
        if (it != texKey.end())
            return it->second;
        auto im = images.find(img);
        if (im == images.end()) {
            const Json *ij = d.at("images", img);
            if (!ij) {
                d.err.set(OPTPT_ERR_PARSE, "image " + std::to_string(img) + " missing");
                return -2;
            }
            std::vector<uint8_t> bytes;
            if (const Json *uri = child(ij, "uri")) {
                if (!uri->isStr() || !d.loadUri(uri->str, bytes, "image"))
                    return -2;
            } else {
                const uint8_t *p;
                size_t len, stride;
                if (!d.view(inum(child(ij, "bufferView"), -1), p, len, stride))
                    return -2;
                bytes.assign(p, p + len);
            }
            optimg::Image decoded;
            std::string e;
            const bool png = optimg::isPng(bytes.data(), bytes.size());
            const bool jpeg = !png && optimg::isJpeg(bytes.data(), bytes.size());
            if (!png && !jpeg) {
                d.err.set(OPTPT_ERR_PARSE, "image " + std::to_string(img) + ": only PNG and JPEG images are supported");
                return -2;
            }
            if (!(png ? optimg::decodePng(bytes.data(), bytes.size(), decoded, e)
                      : optimg::decodeJpeg(bytes.data(), bytes.size(), decoded, e))) {
                d.err.set(OPTPT_ERR_PARSE, "image " + std::to_string(img) + ": " + e);
                return -2;
            }
            im = images.emplace(img, std::move(decoded)).first;
        }
        optpt_texture tx{};
        tx.width = im->second.width;
        tx.height = im->second.height;
        uint8_t *px = (uint8_t *)malloc(im->second.rgba.size());
        if (!px) {
            d.err.set(OPTPT_ERR_NOMEM, "texture allocation failed");
            return -2;
        }
        memcpy(px, im->second.rgba.data(), im->second.rgba.size());
        tx.rgba = px;
        tx.wrapS = wrapS;
        tx.wrapT = wrapT;
        tx.srgb = srgb ? 1 : 0;
        tx.filter = filter;
        textures.push_back(tx);
        const int id = (int)textures.size() - 1;
        texKey[key] = id;
        return id;
    }

    static void transformOf(const Json *texInfo, TextureTransform &tf)
    {
        const Json *tt = child(child(texInfo, "extensions"), "KHR_texture_transform");
        if (!tt)
            return;
        if (const Json *o = child(tt, "offset"))
            if (o->isArr() && o->arr.size() == 2) {
                tf.offset[0] = (float)num(&o->arr[0], 0);
                tf.offset[1] = (float)num(&o->arr[1], 0);
            }
        if (const Json *r = child(tt, "rotation"))
            if (r->isNum())
                tf.rotation = (float)r->num;
        if (const Json *s = child(tt, "scale"))
            if (s->isArr() && s->arr.size() == 2) {
                tf.scale[0] = (float)num(&s->arr[0], 1);
                tf.scale[1] = (float)num(&s->arr[1], 1);
            }
    }

    // Binds texture info `ti` (an object with "index") into slot (index,
    // has flag, transform); false on error.
    bool bind(const Json *ti, bool srgb, bool useSampler, int32_t &slot, uint8_t &has, TextureTransform &tf)
    {
        if (!ti || !child(ti, "index"))
            return true;
        const int t = texture(inum(child(ti, "index"), -1), srgb, useSampler);
        if (t < 0)
            return false;
        slot = t;
        has = 1;
        transformOf(ti, tf);
        return true;
    }

    bool loadMaterials()
    {
        const Json *ms = d.arr("materials");
        const size_t n = ms ? ms->arr.size() : 0;
        for (size_t i = 0; i < n; ++i) {
            const Json *mj = &ms->arr[i];
            MaterialData m = opthost::baseMaterial(1, 1, 1);
            const Json *pbr = child(mj, "pbrMetallicRoughness");
            const Json *ext = child(mj, "extensions");
            if (const Json *bc = child(pbr, "baseColorFactor"))
                if (bc->isArr() && bc->arr.size() == 4)
                    for (int k = 0; k < 4; ++k)
                        m.baseColour[k] = (float)num(&bc->arr[(size_t)k], 1);
            if (!bind(child(pbr, "baseColorTexture"), true, true, m.baseColourTexture, m.hasBaseColourTexture,
                      m.baseColourTexTf))
                return false;
            const Json *am = child(mj, "alphaMode");
            m.alphaMode = am && am->isStr() ? (am->str == "BLEND" ? AM_BLEND : am->str == "MASK" ? AM_MASK : AM_OPAQUE)
                                            : AM_OPAQUE;
            m.alphaCutoff = (float)num(child(mj, "alphaCutoff"), 0.5);
            if (!bind(child(mj, "normalTexture"), false, false, m.normalTexture, m.hasNormalTexture, m.normalTexTf))
                return false;
            m.metallic = (float)num(child(pbr, "metallicFactor"), 1.0);
            if (!bind(child(pbr, "metallicRoughnessTexture"), false, false, m.metallicRoughnessTexture,
                      m.hasMetallicRoughnessTexture, m.metallicRoughnessTexTf))
                return false;
            m.roughness = (float)num(child(pbr, "roughnessFactor"), 1.0);
            m.specular = (float)num(child(child(ext, "KHR_materials_specular"), "specularFactor"), 1.0);
            m.transmissionWeight =
                (float)num(child(child(ext, "KHR_materials_transmission"), "transmissionFactor"), 0.0);
            m.ior = (float)num(child(child(ext, "KHR_materials_ior"), "ior"), 1.5);
            double ef[3] = {0, 0, 0};
            if (const Json *e = child(mj, "emissiveFactor"))
                if (e->isArr() && e->arr.size() == 3)
                    for (int k = 0; k < 3; ++k)
                        ef[k] = num(&e->arr[(size_t)k], 0);
            float strength = 1.0f;
            if (std::fmax(std::fmax(ef[0], ef[1]), ef[2]) > 0.0) {
                strength = (float)num(child(child(ext, "KHR_materials_emissive_strength"), "emissiveStrength"), 1.0);
                if (!bind(child(mj, "emissiveTexture"), true, false, m.emissiveTexture, m.hasEmissiveTexture,
                          m.emissiveTexTf))
                    return false;
            }
            for (int k = 0; k < 3; ++k)
                m.emission[k] = (float)ef[k] * strength;
            const Json *cc = child(ext, "KHR_materials_clearcoat");
            m.coatWeight = (float)num(child(cc, "clearcoatFactor"), 0.0);
            m.coatRoughness = (float)num(child(cc, "clearcoatRoughnessFactor"), 0.0);
            if (const Json *sh = child(ext, "KHR_materials_sheen")) {
                const Json *scf = child(sh, "sheenColorFactor");
                if (scf && scf->isArr() && scf->arr.size() == 3) {
                    for (int k = 0; k < 3; ++k)
                        m.sheenColour[k] = (float)num(&scf->arr[(size_t)k], 0);
                    if (!bind(child(sh, "sheenColorTexture"), true, false, m.sheenColourTexture,
                              m.hasSheenColourTexture, m.sheenColourTexTf))
                        return false;
                }
                const Json *srf = child(sh, "sheenRoughnessFactor");
                if (srf && srf->isNum()) {
                    m.sheenRoughness = (float)srf->num;
                    if (!bind(child(sh, "sheenRoughnessTexture"), true, false, m.sheenRoughnessTexture,
                              m.hasSheenRoughnessTexture, m.sheenRoughnessTexTf))
                        return false;
                }
            }
            m.category = opthost::hostCategory(m);
            materials.push_back(m);
        }
        return true;
    }

    int materialOf(int mi)
    {
        if (mi >= 0 && (size_t)mi < materials.size())
            return mi;
        if (defaultMaterial < 0) {
            // glTF's default material: white, metallic 1, roughness 1.
            MaterialData m = opthost::baseMaterial(1, 1, 1);
            m.metallic = 1.0f;
            m.specular = 1.0f;
            m.category = opthost::hostCategory(m);
            materials.push_back(m);
            defaultMaterial = (int)materials.size() - 1;
        }
        return defaultMaterial;
    }

    void light(const Json *ext, const Mat4 &w)
    {
        const int li = inum(child(ext, "light"), -1);
        const Json *lj = elem(child(child(d.j.get("extensions"), "KHR_lights_punctual"), "lights"), li);
        if (!lj)
            return;
        const Json *tj = child(lj, "type");
        const std::string type = tj && tj->isStr() ? tj->str : "";
        const float intensity = (float)num(child(lj, "intensity"), 1.0);
        const float pi = 3.14159265358979323846f;
        const float wattage = intensity / 683.0f * 4.0f * pi;
        float colour[3] = {1, 1, 1};
        if (const Json *c = child(lj, "color"))
            if (c->isArr() && c->arr.size() == 3)
                for (int k = 0; k < 3; ++k)
                    colour[k] = (float)num(&c->arr[(size_t)k], 1);
        Light L;
        memset(&L, 0, sizeof(L));
        const float origin[4] = {0, 0, 0, 1}, axis[4] = {0, 0, -1, 0};
        float p[3], dir[3];
        xform(w, origin, p);
        xform(w, axis, dir);
        const float dl = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        for (int k = 0; k < 3; ++k) {
            dir[k] = dl > 0 ? dir[k] / dl : 0.0f;
            L.colour[k] = colour[k];
            L.power[k] = wattage * colour[k];
        }
        if (type == "point") {
            L.type = LIGHT_TYPE_POINT;
            for (int k = 0; k < 3; ++k) {
                L.p0[k] = p[k];
                L.radiance[k] = L.power[k] / (4.0f * pi);
            }
        } else if (type == "directional") {
            L.type = LIGHT_TYPE_DIRECTIONAL;
            for (int k = 0; k < 3; ++k) {
                L.p0[k] = L.p1[k] = L.p2[k] = 1000.0f * -dir[k];
                L.normal[k] = dir[k];
                L.radiance[k] = L.power[k] / (4.0f * pi);
            }
            L.distance = 1000.0f;
        } else if (type == "spot") {
            const Json *sp = child(lj, "spot");
            const double outer = num(child(sp, "outerConeAngle"), pi / 4.0), inner = num(child(sp, "innerConeAngle"), 0.0);
            L.type = LIGHT_TYPE_SPOT;
            L.widthRad = (float)outer;
            L.cosWidth = std::cos(L.widthRad);
            L.cosFalloffStart = std::cos((float)inner);
            const float cosTheta = 0.5f * (L.cosWidth + L.cosFalloffStart);
            const float solid = 2.0f * pi * (1.0f - cosTheta);
            for (int k = 0; k < 3; ++k) {
                L.p0[k] = p[k];
                L.normal[k] = dir[k];
                L.radiance[k] = L.power[k] / solid;
            }
        } else {
            return;
        }
        lights.push_back(L);
    }

    bool primitive(const Json &pr, uint32_t shape, bool skinned)
    {
        const int mode = inum(child(&pr, "mode"), 4);
        if (mode < 4)
            return true;  // points and lines are not surfaces
        const Json *at = child(&pr, "attributes");
        const Json *pa = child(at, "POSITION");
        if (!pa)
            return true;
        std::vector<float> P, N, T, J, W;
        size_t nv, nn = 0, nt = 0, nj = 0, nw = 0;
        if (!d.readFloats(inum(pa, -1), 3, P, nv))
            return false;
        const Json *na = child(at, "NORMAL"), *ta = child(at, "TEXCOORD_0");
        if (na && !d.readFloats(inum(na, -1), 3, N, nn))
            return false;
        if (ta && !d.readFloats(inum(ta, -1), 2, T, nt))
            return false;
        if ((na && nn != nv) || (ta && nt != nv))
            return d.err.set(OPTPT_ERR_PARSE, "primitive attributes of different lengths");
        if (skinned) {
            const Json *ja = child(at, "JOINTS_0"), *wa = child(at, "WEIGHTS_0");
            if (ja && wa) {
                if (!d.readFloats(inum(ja, -1), 4, J, nj) || !d.readFloats(inum(wa, -1), 4, W, nw))
                    return false;
                if (nj != nv || nw != nv)
                    return d.err.set(OPTPT_ERR_PARSE, "skin attributes of different lengths");
                const size_t nJoints = skins[shapes[shape].skin].joints.size();
                for (float j : J)
                    if ((size_t)j >= nJoints)
                        return d.err.set(OPTPT_ERR_PARSE, "joint index out of range");
            }
        }
        std::vector<uint32_t> ind;
        if (const Json *ij = child(&pr, "indices")) {
            if (!d.readIndices(inum(ij, -1), ind))
                return false;
        } else {
            ind.resize(nv);
            for (size_t i = 0; i < nv; ++i)
                ind[i] = (uint32_t)i;
        }
        for (uint32_t i : ind)
            if (i >= nv)
                return d.err.set(OPTPT_ERR_PARSE, "index out of range");
        std::vector<uint32_t> tri;
        if (mode == 4) {
            tri.assign(ind.begin(), ind.begin() + (ind.size() / 3) * 3);
        } else if (mode == 5) {
            for (size_t i = 2; i < ind.size(); ++i) {
                const bool odd = (i & 1) != 0;
                tri.push_back(ind[i - 2]);
                tri.push_back(odd ? ind[i] : ind[i - 1]);
                tri.push_back(odd ? ind[i - 1] : ind[i]);
            }
        } else {
            for (size_t i = 2; i < ind.size(); ++i) {
                tri.push_back(ind[0]);
                tri.push_back(ind[i - 1]);
                tri.push_back(ind[i]);
            }
        }
        const int m = materialOf(inum(child(&pr, "material"), -1));
        const int jb = shapes[shape].jointBase;
        auto vertex = [&](uint32_t vi, const float *normal) {
            for (int q = 0; q < 3; ++q)
                pos.push_back(P[3 * vi + q]);
            if (anyNormals)
                for (int q = 0; q < 3; ++q)
                    nrm.push_back(normal ? normal[q] : N[3 * vi + q]);
            if (anyTexCoords) {
                tc.push_back(T.empty() ? 0.0f : T[2 * vi]);
                tc.push_back(T.empty() ? 0.0f : T[2 * vi + 1]);
            }
            vShape.push_back(shape);
            for (int k = 0; k < 4; ++k) {
                vJoints.push_back(J.empty() ? (uint16_t)0 : (uint16_t)(jb + (int)J[4 * vi + k]));
                vWeights.push_back(J.empty() ? 0.0f : W[4 * vi + k]);
            }
            anySkin |= !J.empty();
        };
        if (anyNormals && N.empty()) {
            // Unindexed, each corner carrying the face normal (in the
            // shape's space; it follows the shape's normal matrix).
            for (size_t t = 0; t + 2 < tri.size(); t += 3) {
                const float *a = &P[3 * tri[t]], *b = &P[3 * tri[t + 1]], *c = &P[3 * tri[t + 2]];
                const double e1[3] = {(double)b[0] - a[0], (double)b[1] - a[1], (double)b[2] - a[2]};
                const double e2[3] = {(double)c[0] - a[0], (double)c[1] - a[1], (double)c[2] - a[2]};
                const double fn[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                      e1[0] * e2[1] - e1[1] * e2[0]};
                const double l = std::sqrt(fn[0] * fn[0] + fn[1] * fn[1] + fn[2] * fn[2]);
                const float f[3] = {l > 0 ? (float)(fn[0] / l) : 0.0f, l > 0 ? (float)(fn[1] / l) : 0.0f,
                                    l > 0 ? (float)(fn[2] / l) : 0.0f};
                const int32_t base = (int32_t)(vShape.size());
                for (int k = 0; k < 3; ++k) {
                    vertex(tri[t + (size_t)k], f);
                    idx.push_back(base + k);
                }
                mat.push_back(m);
            }
            return true;
        }
        const int32_t base = (int32_t)(vShape.size());
        for (size_t v = 0; v < nv; ++v)
            vertex((uint32_t)v, nullptr);
        for (size_t t = 0; t + 2 < tri.size(); t += 3) {
            for (int k = 0; k < 3; ++k)
                idx.push_back(base + (int32_t)tri[t + (size_t)k]);
            mat.push_back(m);
        }
        return true;
    }

    bool loadSkin(int skinIndex)
    {
        if (skins.count(skinIndex))
            return true;
        const Json *sk = d.at("skins", skinIndex);
        const Json *joints = child(sk, "joints");
        if (!sk || !joints || !joints->isArr())
            return d.err.set(OPTPT_ERR_PARSE, "bad skin " + std::to_string(skinIndex));
        Skin S;
        for (auto &j : joints->arr) {
            const int jn = inum(&j, -1);
            if (jn < 0 || (size_t)jn >= world.size())
                return d.err.set(OPTPT_ERR_PARSE, "bad joint node");
            S.joints.push_back(jn);
        }
        const size_t nj = S.joints.size();
        S.ibm.assign(nj, Mat4::identity());
        if (const Json *ib = child(sk, "inverseBindMatrices")) {
            std::vector<float> ibm;
            size_t cnt = 0;
            if (!d.readFloats(inum(ib, -1), 16, ibm, cnt))
                return false;
            if (cnt < nj)
                return d.err.set(OPTPT_ERR_PARSE, "skin has fewer inverse bind matrices than joints");
            for (size_t j = 0; j < nj; ++j)
                for (int k = 0; k < 16; ++k)
                    S.ibm[j].m[k / 4][k % 4] = ibm[j * 16 + (size_t)k];
        }
        skins[skinIndex] = std::move(S);
        return true;
    }

    static bool invert4(const double m[16], double out[16])
    {
        // Gauss-Jordan with partial pivoting on [m | I] (m column-major).
        double a[4][8];
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) {
                a[r][c] = m[c * 4 + r];
                a[r][c + 4] = r == c ? 1.0 : 0.0;
            }
        for (int c = 0; c < 4; ++c) {
            int p = c;
            for (int r = c + 1; r < 4; ++r)
                if (std::fabs(a[r][c]) > std::fabs(a[p][c]))
                    p = r;
            if (a[p][c] == 0.0)
                return false;
            for (int k = 0; k < 8; ++k)
                std::swap(a[c][k], a[p][k]);
            const double iv = 1.0 / a[c][c];
            for (int k = 0; k < 8; ++k)
                a[c][k] *= iv;
            for (int r = 0; r < 4; ++r)
                if (r != c) {
                    const double f = a[r][c];
                    for (int k = 0; k < 8; ++k)
                        a[r][k] -= f * a[c][k];
                }
        }
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c)
                out[c * 4 + r] = a[r][c + 4];
        return true;
    }

    // Depth-first over the default scene (loadNode :908-1226).
    bool visit(int n, int depth)
    {
        const Json *node = d.at("nodes", n);
        if (!node || depth > 256)
            return d.err.set(OPTPT_ERR_PARSE, "bad node " + std::to_string(n));
        const Mat4 &w = world[(size_t)n];
        if (const Json *lp = child(child(node, "extensions"), "KHR_lights_punctual"))
            light(lp, w);
        const int cam = inum(child(node, "camera"), -1);
        if (cam >= 0 && !camera) {
            const Json *cj = d.at("cameras", cam);
            const Json *ct = child(cj, "type");
            if (ct && ct->isStr() && ct->str == "perspective") {
                camera = true;
                const double yfov = num(child(child(cj, "perspective"), "yfov"), 0.7853981633974483);
                fovYDeg = (float)(yfov * 57.295779513082320876798154814105);
                const float o[4] = {0, 0, 0, 1}, t[4] = {0, 0, -1, 1};
                xform(w, o, camEye);
                xform(w, t, camTarget);
            }
        }
        const int mesh = inum(child(node, "mesh"), -1);
        if (mesh >= 0) {
            const Json *mj = d.at("meshes", mesh);
            if (!mj)
                return d.err.set(OPTPT_ERR_PARSE, "mesh " + std::to_string(mesh) + " missing");
            const int skin = inum(child(node, "skin"), -1);
            if (skin >= 0 && !loadSkin(skin))
                return false;
            shapes.push_back({n, skin, jointSlots});
            if (skin >= 0)
                jointSlots += (int)skins[skin].joints.size();
            if (jointSlots > 65535)
                return d.err.set(OPTPT_ERR_PARSE, "more than 65535 joint slots");
            const uint32_t shape = (uint32_t)shapes.size() - 1;
            if (const Json *prims = child(mj, "primitives"))
                for (auto &pr : prims->arr)
                    if (!primitive(pr, shape, skin >= 0))
                        return false;
        }
        if (const Json *ch = child(node, "children"))
            for (auto &c : ch->arr)
                if (!visit(inum(&c, -1), depth + 1))
                    return false;
        return true;
    }

    // Whether any primitive under the scene's nodes has NORMAL / TEXCOORD_0.
    void scan(int n, int depth)
    {
        const Json *node = d.at("nodes", n);
        if (!node || depth > 256)
            return;
        if (const Json *mj = d.at("meshes", inum(child(node, "mesh"), -1)))
            if (const Json *prims = child(mj, "primitives"))
                for (auto &pr : prims->arr) {
                    if (inum(child(&pr, "mode"), 4) < 4)
                        continue;
                    const Json *at = child(&pr, "attributes");
                    anyNormals |= child(at, "NORMAL") != nullptr;
                    anyTexCoords |= child(at, "TEXCOORD_0") != nullptr;
                }
        if (const Json *ch = child(node, "children"))
            for (auto &c : ch->arr)
                scan(inum(&c, -1), depth + 1);
    }
};

// ------------------------------------------------------------------ animation
// Node transforms and one animation (the reference's loadAnimations,
// src/gltf_loader.cpp:1390-1509: animation 2 when the file has three or
// more, else animation 0), evaluated as Renderer::updateScene does
// (src/renderer.cpp:1060-1182): channels set a node's translation, rotation
// or scale (STEP holds the previous key, LINEAR mixes, rotations slerp);
// time wraps modulo each channel's last key time; world matrices are
// recomputed down the tree (nodes with a "matrix" keep it); a shape's
// vertices go through world * skin, with skin = sum of weight * joint matrix
// and joint matrix = inverse(world(mesh node)) * world(joint) *
// inverseBind; normals go through the inverse transpose of the mesh node's
// world matrix only. Differences: CUBICSPLINE channels use the glTF cubic
// Hermite spline (the reference's string test never matches them and reads
// tangents as values); before the first key and at the last key the first
// / last value is held (the reference divides by zero before the first key
// and jumps to the first value at the last).
struct Channel {
    int node = -1, path = 0, interp = 1;  // path 0 T, 1 R, 2 S; interp 0 STEP, 1 LINEAR, 2 CUBICSPLINE
    std::vector<float> t, v;              // v: comps per key (x3 for CUBICSPLINE: in-tangent, value, out-tangent)
};

struct NodeTRS {
    bool hasMatrix = false;
    Mat4 matrix = Mat4::identity();
    float t[3] = {0, 0, 0}, r[4] = {0, 0, 0, 1}, s[3] = {1, 1, 1};
    std::vector<int> children;
};

float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }

void slerp(const float *x, const float *y, float a, float *out)
{
    float z[4] = {y[0], y[1], y[2], y[3]};
    float c = x[0] * y[0] + x[1] * y[1] + x[2] * y[2] + x[3] * y[3];
    if (c < 0.0f) {
        for (int k = 0; k < 4; ++k)
            z[k] = -z[k];
        c = -c;
    }
    if (c > 1.0f - 1.1920929e-07f) {  // nearly parallel: linear
        for (int k = 0; k < 4; ++k)
            out[k] = mixf(x[k], z[k], a);
        return;
    }
    const float angle = std::acos(c), sa = std::sin(angle);
    const float wa = std::sin((1.0f - a) * angle), wb = std::sin(a * angle);
    for (int k = 0; k < 4; ++k)
        out[k] = (wa * x[k] + wb * z[k]) / sa;
}

void sampleChannel(const Channel &ch, float time, float *out)
{
    const int comps = ch.path == 1 ? 4 : 3;
    const size_t n = ch.t.size();
    const int stride = ch.interp == 2 ? 3 * comps : comps, off = ch.interp == 2 ? comps : 0;
    auto key = [&](size_t i) { return &ch.v[i * (size_t)stride + (size_t)off]; };
    float t = time;
    const float tmax = ch.t[n - 1];
    if (tmax > 0.0f && t > tmax) {
        float ip;
        t = std::modf(t / tmax, &ip) * tmax;
    }
    size_t next = n;
    for (size_t i = 0; i < n; ++i)
        if (ch.t[i] > t) {
            next = i;
            break;
        }
    if (next == 0 || next == n || ch.interp == 0) {
        const size_t i = next == 0 ? 0 : next == n ? n - 1 : next - 1;
        memcpy(out, key(i), sizeof(float) * (size_t)comps);
        return;
    }
    const size_t prev = next - 1;
    const float td = ch.t[next] - ch.t[prev];
    const float a = (t - ch.t[prev]) / td;
    if (ch.interp == 2) {
        const float a2 = a * a, a3 = a2 * a;
        const float h00 = 2 * a3 - 3 * a2 + 1, h10 = a3 - 2 * a2 + a, h01 = -2 * a3 + 3 * a2, h11 = a3 - a2;
        const float *v0 = key(prev), *v1 = key(next);
        const float *b0 = v0 + comps, *a1 = v1 - comps;  // out-tangent of prev, in-tangent of next
        for (int k = 0; k < comps; ++k)
            out[k] = h00 * v0[k] + h10 * td * b0[k] + h01 * v1[k] + h11 * td * a1[k];
        if (comps == 4) {
            const float l = std::sqrt(out[0] * out[0] + out[1] * out[1] + out[2] * out[2] + out[3] * out[3]);
            for (int k = 0; k < 4 && l > 0; ++k)
                out[k] /= l;
        }
        return;
    }
    if (comps == 4) {
        slerp(key(prev), key(next), a, out);
        return;
    }
    for (int k = 0; k < 3; ++k)
        out[k] = mixf(key(prev)[k], key(next)[k], a);
}

template <class T> T *dupv(const std::vector<T> &v)
{
    if (v.empty())
        return nullptr;
    T *p = (T *)malloc(sizeof(T) * v.size());
    if (p)
        memcpy(p, v.data(), sizeof(T) * v.size());
    return p;
}

int parseDocument(const std::string &path, Doc &d)
{
    std::string text;
    if (!optjson::readFile(path, text))
        return optpt_internal_set_error(OPTPT_ERR_IO, ("cannot read glTF file " + path).c_str());
    const size_t slash = path.find_last_of("/\\");
    d.dir = slash == std::string::npos ? std::string() : path.substr(0, slash + 1);
    std::string json = text;
    if (text.size() >= 12 && memcmp(text.data(), "glTF", 4) == 0) {
        // Binary container: 12-byte header, JSON chunk, optional BIN chunk.
        auto u32 = [&](size_t o) {
            uint32_t v;
            memcpy(&v, text.data() + o, 4);
            return v;
        };
        if (u32(4) != 2)
            return optpt_internal_set_error(OPTPT_ERR_PARSE, "unsupported .glb version");
        size_t o = 12;
        bool haveJson = false;
        while (o + 8 <= text.size()) {
            const uint32_t len = u32(o), type = u32(o + 4);
            if (len > text.size() - o - 8)
                return optpt_internal_set_error(OPTPT_ERR_PARSE, "truncated .glb chunk");
            if (type == 0x4E4F534Au && !haveJson) {
                json.assign(text.data() + o + 8, len);
                haveJson = true;
            } else if (type == 0x004E4942u && !d.hasGlbBin) {
                d.glbBin.assign((const uint8_t *)text.data() + o + 8, (const uint8_t *)text.data() + o + 8 + len);
                d.hasGlbBin = true;
            }
            o += 8 + ((size_t)len + 3) / 4 * 4;
        }
        if (!haveJson)
            return optpt_internal_set_error(OPTPT_ERR_PARSE, ".glb without a JSON chunk");
    }
    int rc = optjson::parseJson(json, d.j, "glTF file " + path);
    if (rc)
        return rc;
    if (!d.j.isObj())
        return optpt_internal_set_error(OPTPT_ERR_PARSE, "glTF root is not an object");
    const Json *ver = child(child(&d.j, "asset"), "version");
    if (!ver || !ver->isStr() || ver->str.compare(0, 2, "2.") != 0)
        return optpt_internal_set_error(OPTPT_ERR_PARSE, "unsupported glTF version");
    if (!d.loadBuffers())
        return optpt_internal_set_error(d.err.code, d.err.msg.c_str());
    return OPTPT_OK;
}

}  // namespace

// A loaded glTF scene: the flattened static data plus what is needed to pose
// it at any time (node tree, skins, one animation, per-vertex bindings).
struct optpt_gltf {
    std::vector<float> restPos, restNrm, tc;
    std::vector<int32_t> idx, mat;
    std::vector<MaterialData> materials;
    std::vector<Light> lights;
    std::vector<optpt_texture> textures;  // pixels owned here until handed to a scene
    float camEye[3], camTarget[3], camUp[3], fovYDeg;
    bool anyNormals = false, anyTexCoords = false, anySkin = false;
    std::vector<uint32_t> vShape;
    std::vector<uint16_t> vJoints;
    std::vector<float> vWeights;
    struct Shape {
        int node, skin, jointBase;
    };
    std::vector<Shape> shapes;
    std::map<int, std::pair<std::vector<int>, std::vector<Mat4>>> skins;  // joints, inverse binds
    int jointSlots = 0;
    std::vector<NodeTRS> nodes;
    std::vector<int> roots;
    std::vector<Channel> channels;
    float duration = 0.0f;

    ~optpt_gltf()
    {
        for (auto &t : textures)
            free((void *)t.rgba);
    }

    void worlds(int n, const Mat4 &parent, const std::vector<NodeTRS> &cur, std::vector<Mat4> &w, int depth) const
    {
        if (n < 0 || (size_t)n >= cur.size() || depth > 256)
            return;
        const NodeTRS &N = cur[(size_t)n];
        Mat4 local = N.matrix;
        if (!N.hasMatrix) {
            Mat4 t = Mat4::identity(), s = Mat4::identity();
            for (int k = 0; k < 3; ++k) {
                t.m[3][k] = N.t[k];
                s.m[k][k] = N.s[k];
            }
            local = mul(mul(t, fromQuat(N.r[0], N.r[1], N.r[2], N.r[3])), s);
        }
        w[(size_t)n] = mul(parent, local);
        for (int c : N.children)
            worlds(c, w[(size_t)n], cur, w, depth + 1);
    }

    // Shape matrices (16 per shape), shape normal matrices (9 per shape, row
    // r multiplies the normal), joint matrices (16 per slot), at `time`
    // (animation applied when animate).
    bool pose(float time, bool animate, float *shapeM, float *shapeN, float *jointM) const
    {
        std::vector<NodeTRS> cur = nodes;
        if (animate)
            for (const Channel &ch : channels) {
                float v[4];
                sampleChannel(ch, time, v);
                NodeTRS &N = cur[(size_t)ch.node];
                if (ch.path == 0)
                    memcpy(N.t, v, 12);
                else if (ch.path == 1)
                    memcpy(N.r, v, 16);
                else
                    memcpy(N.s, v, 12);
            }
        std::vector<Mat4> w(cur.size(), Mat4::identity());
        for (int r : roots)
            worlds(r, Mat4::identity(), cur, w, 0);
        for (size_t s = 0; s < shapes.size(); ++s) {
            const Mat4 &G = w[(size_t)shapes[s].node];
            if (shapeM)
                memcpy(shapeM + 16 * s, G.m, 64);
            if (shapeN) {
                float nm[3][3];
                normalMatrix(G, nm);
                memcpy(shapeN + 9 * s, nm, 36);
            }
            if (jointM && shapes[s].skin >= 0) {
                const auto &sk = skins.at(shapes[s].skin);
                double a[16], inv[16];
                for (int c = 0; c < 4; ++c)
                    for (int r = 0; r < 4; ++r)
                        a[c * 4 + r] = G.m[c][r];
                if (!Loader::invert4(a, inv))
                    return false;
                Mat4 iw;
                for (int c = 0; c < 4; ++c)
                    for (int r = 0; r < 4; ++r)
                        iw.m[c][r] = (float)inv[c * 4 + r];
                for (size_t j = 0; j < sk.first.size(); ++j) {
                    const Mat4 J = mul(mul(iw, w[(size_t)sk.first[j]]), sk.second[j]);
                    memcpy(jointM + 16 * ((size_t)shapes[s].jointBase + j), J.m, 64);
                }
            }
        }
        return true;
    }
};

// The vertex transform the GPU deformation kernel applies, in the same
// float operations (this file is compiled without contraction).
static void deformVertex(const float *p, const float *n, uint32_t shape, const uint16_t *joints, const float *weights,
                  const float *shapeM, const float *shapeN, const float *jointM, float *outP, float *outN)
{
    const float *G = shapeM + 16 * (size_t)shape;
    float P[16];
    if (joints) {
        float S[16];
        for (int e = 0; e < 16; ++e) {
            float acc = weights[0] * jointM[16 * (size_t)joints[0] + e];
            acc = acc + weights[1] * jointM[16 * (size_t)joints[1] + e];
            acc = acc + weights[2] * jointM[16 * (size_t)joints[2] + e];
            acc = acc + weights[3] * jointM[16 * (size_t)joints[3] + e];
            S[e] = acc;
        }
        for (int c = 0; c < 4; ++c)
            for (int r = 0; r < 4; ++r) {
                float acc = G[0 * 4 + r] * S[c * 4 + 0];
                acc = acc + G[1 * 4 + r] * S[c * 4 + 1];
                acc = acc + G[2 * 4 + r] * S[c * 4 + 2];
                acc = acc + G[3 * 4 + r] * S[c * 4 + 3];
                P[c * 4 + r] = acc;
            }
    } else {
        memcpy(P, G, 64);
    }
    for (int r = 0; r < 3; ++r) {
        float acc = P[0 * 4 + r] * p[0];
        acc = acc + P[1 * 4 + r] * p[1];
        acc = acc + P[2 * 4 + r] * p[2];
        acc = acc + P[3 * 4 + r];
        outP[r] = acc;
    }
    if (n && outN) {
        const float *N = shapeN + 9 * (size_t)shape;
        for (int r = 0; r < 3; ++r) {
            float acc = N[3 * r] * n[0];
            acc = acc + N[3 * r + 1] * n[1];
            acc = acc + N[3 * r + 2] * n[2];
            outN[r] = acc;
        }
    }
}

namespace {

int loadModel(const char *path, const float upHint[3], optpt_gltf *&out)
{
    out = nullptr;
    Doc d;
    int rc = parseDocument(path, d);
    if (rc)
        return rc;
    const Json *sceneIdx = d.j.get("scene");
    if (!sceneIdx || !sceneIdx->isNum())
        return optpt_internal_set_error(OPTPT_ERR_PARSE, "no scene specified");
    const Json *scene = d.at("scenes", (int)sceneIdx->num);
    if (!scene)
        return optpt_internal_set_error(OPTPT_ERR_PARSE, "default scene not found");
    const float defaultUp[3] = {0, 1, 0};
    Loader L(d, upHint ? upHint : defaultUp);
    const Json *nodes = d.j.get("nodes");
    const size_t numNodes = nodes && nodes->isArr() ? nodes->arr.size() : 0;
    L.world.assign(numNodes, Mat4::identity());
    bool ok = L.loadMaterials();
    const Json *roots = child(scene, "nodes");
    if (ok && roots) {
        for (auto &r : roots->arr)
            if (!(ok = L.worlds(inum(&r, -1), Mat4::identity(), 0)))
                break;
        if (ok)
            for (auto &r : roots->arr)
                L.scan(inum(&r, -1), 0);
        if (ok)
            for (auto &r : roots->arr)
                if (!(ok = L.visit(inum(&r, -1), 0)))
                    break;
    }
    optpt_gltf *g = new (std::nothrow) optpt_gltf();
    if (!g) {
        for (auto &t : L.textures)
            free((void *)t.rgba);
        return optpt_internal_set_error(OPTPT_ERR_NOMEM, "glTF model allocation failed");
    }
    g->textures.swap(L.textures);  // owned (and freed) by g from here on
    // Node tree with rest transforms, and the animation's channels.
    g->nodes.resize(numNodes);
    for (size_t n = 0; ok && n < numNodes; ++n) {
        const Json &nj = nodes->arr[n];
        NodeTRS &N = g->nodes[n];
        const Json *m = child(&nj, "matrix");
        if (m && m->isArr() && m->arr.size() == 16) {
            N.hasMatrix = true;
            for (int i = 0; i < 16; ++i)
                N.matrix.m[i / 4][i % 4] = (float)num(&m->arr[(size_t)i], 0);
        }
        auto vec = [&](const char *k, float *dst, size_t len, float dflt) {
            const Json *v = child(&nj, k);
            if (v && v->isArr() && v->arr.size() == len)
                for (size_t i = 0; i < len; ++i)
                    dst[i] = (float)num(&v->arr[i], dflt);
        };
        vec("translation", N.t, 3, 0.0f);
        vec("rotation", N.r, 4, 0.0f);
        vec("scale", N.s, 3, 1.0f);
        if (const Json *ch = child(&nj, "children"))
            for (auto &c : ch->arr) {
                const int ci = inum(&c, -1);
                if (ci < 0 || (size_t)ci >= numNodes) {
                    ok = d.err.set(OPTPT_ERR_PARSE, "bad child node");
                    break;
                }
                N.children.push_back(ci);
            }
    }
    if (ok && roots)
        for (auto &r : roots->arr)
            g->roots.push_back(inum(&r, -1));
    const Json *anims = d.j.get("animations");
    if (ok && anims && anims->isArr() && !anims->arr.empty()) {
        const Json &an = anims->arr[anims->arr.size() >= 3 ? 2 : 0];
        const Json *samplers = child(&an, "samplers"), *chans = child(&an, "channels");
        if (chans && chans->isArr())
            for (auto &cj : chans->arr) {
                const Json *tgt = child(&cj, "target");
                const Json *pathJ = child(tgt, "path");
                const int node = inum(child(tgt, "node"), -1);
                const std::string path = pathJ && pathJ->isStr() ? pathJ->str : "";
                const int p = path == "translation" ? 0 : path == "rotation" ? 1 : path == "scale" ? 2 : -1;
                if (p < 0 || node < 0 || (size_t)node >= numNodes)
                    continue;  // morph-target weights and the like are not animated
                const Json *sj = elem(samplers, inum(child(&cj, "sampler"), -1));
                if (!sj) {
                    ok = d.err.set(OPTPT_ERR_PARSE, "animation channel without sampler");
                    break;
                }
                Channel ch;
                ch.node = node;
                ch.path = p;
                const Json *ij = child(sj, "interpolation");
                const std::string interp = ij && ij->isStr() ? ij->str : "LINEAR";
                ch.interp = interp == "STEP" ? 0 : interp == "CUBICSPLINE" ? 2 : 1;
                size_t nt = 0, nv = 0;
                if (!d.readFloats(inum(child(sj, "input"), -1), 1, ch.t, nt) ||
                    !d.readFloats(inum(child(sj, "output"), -1), p == 1 ? 4 : 3, ch.v, nv)) {
                    ok = false;
                    break;
                }
                if (nt == 0 || nv != nt * (ch.interp == 2 ? 3u : 1u)) {
                    ok = d.err.set(OPTPT_ERR_PARSE, "animation sampler input/output counts differ");
                    break;
                }
                for (size_t i = 1; i < nt; ++i)
                    if (!(ch.t[i] > ch.t[i - 1])) {
                        ok = d.err.set(OPTPT_ERR_PARSE, "animation key times must increase");
                        break;
                    }
                if (!ok)
                    break;
                g->duration = std::max(g->duration, ch.t.back());
                g->channels.push_back(std::move(ch));
            }
    }
    if (!ok) {
        delete g;
        return optpt_internal_set_error(d.err.code ? d.err.code : OPTPT_ERR_PARSE, d.err.msg.c_str());
    }
    g->restPos.swap(L.pos);
    g->restNrm.swap(L.nrm);
    g->tc.swap(L.tc);
    g->idx.swap(L.idx);
    g->mat.swap(L.mat);
    g->materials.swap(L.materials);
    g->lights.swap(L.lights);
    for (int k = 0; k < 3; ++k) {
        g->camEye[k] = L.camEye[k];
        g->camTarget[k] = L.camTarget[k];
        g->camUp[k] = L.up[k];
    }
    g->fovYDeg = L.fovYDeg;
    g->anyNormals = L.anyNormals;
    g->anyTexCoords = L.anyTexCoords;
    g->anySkin = L.anySkin;
    g->vShape.swap(L.vShape);
    g->vJoints.swap(L.vJoints);
    g->vWeights.swap(L.vWeights);
    for (auto &s : L.shapes)
        g->shapes.push_back({s.node, s.skin, s.jointBase});
    for (auto &kv : L.skins)
        g->skins[kv.first] = {kv.second.joints, kv.second.ibm};
    g->jointSlots = L.jointSlots;
    out = g;
    return OPTPT_OK;
}

// Positions and normals of every vertex at `time` on the host.
int applyPose(const optpt_gltf *g, float time, bool animate, float *positions, float *normals)
{
    std::vector<float> M(16 * g->shapes.size()), N(9 * g->shapes.size()), J(16 * (size_t)g->jointSlots);
    if (!g->pose(time, animate, M.data(), N.data(), J.data()))
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "singular node transform on a skinned mesh");
    const size_t nv = g->vShape.size();
    for (size_t v = 0; v < nv; ++v) {
        // A vertex follows its skin when it has a non-zero weight (a skinned
        // primitive without JOINTS_0 / WEIGHTS_0 stays rigid with its node).
        const float *w = &g->vWeights[4 * v];
        const bool skinned = g->anySkin && g->shapes[g->vShape[v]].skin >= 0 &&
                             (w[0] != 0.0f || w[1] != 0.0f || w[2] != 0.0f || w[3] != 0.0f);
        deformVertex(&g->restPos[3 * v], g->anyNormals ? &g->restNrm[3 * v] : nullptr, g->vShape[v],
                     skinned ? &g->vJoints[4 * v] : nullptr, skinned ? &g->vWeights[4 * v] : nullptr, M.data(),
                     N.data(), J.data(), positions + 3 * v, normals ? normals + 3 * v : nullptr);
    }
    return OPTPT_OK;
}

// The model's scene at `time`; textures are copied (the model keeps its own).
int sceneOf(const optpt_gltf *g, float time, bool animate, optpt_scene *out)
{
    memset(out, 0, sizeof(*out));
    const size_t nv = g->vShape.size();
    std::vector<float> P(3 * nv), Nn(g->anyNormals ? 3 * nv : 0);
    int rc = applyPose(g, time, animate, P.data(), g->anyNormals ? Nn.data() : nullptr);
    if (rc)
        return rc;
    std::vector<optpt_texture> tex = g->textures;
    for (auto &t : tex) {
        const size_t bytes = (size_t)t.width * t.height * 4;
        uint8_t *px = (uint8_t *)malloc(bytes ? bytes : 1);
        if (!px) {
            for (auto &u : tex)
                if (&u != &t && u.rgba != nullptr && (&u < &t))
                    free((void *)u.rgba);
            return optpt_internal_set_error(OPTPT_ERR_NOMEM, "texture allocation failed");
        }
        memcpy(px, t.rgba, bytes);
        t.rgba = px;
    }
    out->positions = dupv(P);
    out->numVertices = (uint32_t)nv;
    out->normals = g->anyNormals ? dupv(Nn) : nullptr;
    out->texCoords = g->anyTexCoords ? dupv(g->tc) : nullptr;
    out->triIndices = dupv(g->idx);
    out->numTriangles = (uint32_t)g->mat.size();
    out->matIndices = dupv(g->mat);
    out->materials = dupv(g->materials);
    out->numMaterials = (uint32_t)g->materials.size();
    out->lights = dupv(g->lights);
    out->numLights = (uint32_t)g->lights.size();
    out->textures = dupv(tex);
    out->numTextures = (uint32_t)tex.size();
    for (int k = 0; k < 3; ++k) {
        out->camEye[k] = g->camEye[k];
        out->camTarget[k] = g->camTarget[k];
        out->camUp[k] = g->camUp[k];
    }
    out->camFovYDeg = g->fovYDeg;
    out->resX = 1280;
    out->resY = 720;
    out->spp = 64;
    out->maxDepth = 8;
    return OPTPT_OK;
}

}  // namespace

extern "C" {

int optpt_scene_from_gltf(const char *path, const float upHint[3], optpt_scene *out)
{
    if (!path || !out)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    memset(out, 0, sizeof(*out));
    optpt_gltf *g = nullptr;
    int rc = loadModel(path, upHint, g);
    if (rc)
        return rc;
    rc = sceneOf(g, 0.0f, false, out);
    delete g;
    return rc;
}

int optpt_gltf_open(const char *path, const float upHint[3], optpt_gltf **out)
{
    if (!path || !out)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    *out = nullptr;
    return loadModel(path, upHint, *out);
}

void optpt_gltf_close(optpt_gltf *g) { delete g; }

int optpt_gltf_scene(const optpt_gltf *g, float time, int animate, optpt_scene *out)
{
    if (!g || !out)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    return sceneOf(g, time, animate != 0, out);
}

int optpt_gltf_info(const optpt_gltf *g, optpt_gltf_info_t *info)
{
    if (!g || !info)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    info->numVertices = (uint32_t)g->vShape.size();
    info->numShapes = (uint32_t)g->shapes.size();
    info->numJointSlots = (uint32_t)g->jointSlots;
    info->numChannels = (uint32_t)g->channels.size();
    info->duration = g->duration;
    info->skinned = g->anySkin ? 1 : 0;
    return OPTPT_OK;
}

int optpt_gltf_deformation(const optpt_gltf *g, optpt_deformation *out)
{
    if (!g || !out)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    memset(out, 0, sizeof(*out));
    out->restPositions = g->restPos.data();
    out->restNormals = g->anyNormals ? g->restNrm.data() : nullptr;
    out->vertexShape = g->vShape.data();
    out->joints = g->anySkin ? g->vJoints.data() : nullptr;
    out->weights = g->anySkin ? g->vWeights.data() : nullptr;
    out->numVertices = (uint32_t)g->vShape.size();
    out->numShapes = (uint32_t)g->shapes.size();
    out->numJoints = (uint32_t)g->jointSlots;
    return OPTPT_OK;
}

int optpt_gltf_pose(const optpt_gltf *g, float time, float *shapeMatrices, float *shapeNormalMatrices,
                    float *jointMatrices)
{
    if (!g)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    if (!g->pose(time, true, shapeMatrices, shapeNormalMatrices, jointMatrices))
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "singular node transform on a skinned mesh");
    return OPTPT_OK;
}

int optpt_gltf_apply(const optpt_gltf *g, float time, float *positions, float *normals)
{
    if (!g || !positions)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    return applyPose(g, time, true, positions, normals);
}

int optpt_image_decode_png(const void *data, size_t size, optpt_image *out)
{
    if (!data || !out)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    memset(out, 0, sizeof(*out));
    optimg::Image img;
    std::string e;
    if (!optimg::decodePng((const uint8_t *)data, size, img, e))
        return optpt_internal_set_error(OPTPT_ERR_PARSE, ("PNG: " + e).c_str());
    uint8_t *px = (uint8_t *)malloc(img.rgba.size());
    if (!px)
        return optpt_internal_set_error(OPTPT_ERR_NOMEM, "image allocation failed");
    memcpy(px, img.rgba.data(), img.rgba.size());
    out->width = img.width;
    out->height = img.height;
    out->rgba = px;
    return OPTPT_OK;
}

int optpt_image_decode_jpeg(const void *data, size_t size, optpt_image *out)
{
    if (!data || !out)
        return optpt_internal_set_error(OPTPT_ERR_INVALID, "NULL argument");
    memset(out, 0, sizeof(*out));
    optimg::Image img;
    std::string e;
    if (!optimg::decodeJpeg((const uint8_t *)data, size, img, e))
        return optpt_internal_set_error(OPTPT_ERR_PARSE, ("JPEG: " + e).c_str());
    uint8_t *px = (uint8_t *)malloc(img.rgba.size());
    if (!px)
        return optpt_internal_set_error(OPTPT_ERR_NOMEM, "image allocation failed");
    memcpy(px, img.rgba.data(), img.rgba.size());
    out->width = img.width;
    out->height = img.height;
    out->rgba = px;
    return OPTPT_OK;
}

void optpt_image_release(optpt_image *img)
{
    if (!img)
        return;
    free(img->rgba);
    memset(img, 0, sizeof(*img));
}

}  // extern "C"
