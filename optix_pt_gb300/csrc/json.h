// A small recursive-descent JSON reader shared by the scene-selection files
// (the reference parses them with rapidjson, src/scene_desc.cpp:50-153) and
// the glTF 2.0 importer (the reference uses tinygltf, src/gltf_loader.cpp:19).
// Values are a plain tree; objects keep member order. Errors carry the byte
// offset of the first problem.
#pragma once
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

extern "C" int optpt_internal_set_error(int code, const char *msg);

namespace optjson {

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
    bool isNum() const { return type == Num; }
    bool isObj() const { return type == Obj; }
    bool isArr() const { return type == Arr; }
    bool isStr() const { return type == Str; }
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
        if (depth > 256)
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
                v.obj.emplace_back(std::move(k.str), std::move(val));
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
    static void utf8(std::string &out, uint32_t cp)
    {
        if (cp < 0x80) {
            out.push_back((char)cp);
        } else if (cp < 0x800) {
            out.push_back((char)(0xC0 | (cp >> 6)));
            out.push_back((char)(0x80 | (cp & 0x3F)));
        } else if (cp < 0x10000) {
            out.push_back((char)(0xE0 | (cp >> 12)));
            out.push_back((char)(0x80 | ((cp >> 6) & 0x3F)));
            out.push_back((char)(0x80 | (cp & 0x3F)));
        } else {
            out.push_back((char)(0xF0 | (cp >> 18)));
            out.push_back((char)(0x80 | ((cp >> 12) & 0x3F)));
            out.push_back((char)(0x80 | ((cp >> 6) & 0x3F)));
            out.push_back((char)(0x80 | (cp & 0x3F)));
        }
    }
    bool hex4(uint32_t &cp)
    {
        if (i + 4 > s.size())
            return false;
        cp = 0;
        for (int k = 0; k < 4; ++k) {
            const char h = s[i + k];
            const int d = h >= '0' && h <= '9' ? h - '0' : h >= 'a' && h <= 'f' ? h - 'a' + 10
                        : h >= 'A' && h <= 'F' ? h - 'A' + 10 : -1;
            if (d < 0)
                return false;
            cp = cp * 16 + (uint32_t)d;
        }
        i += 4;
        return true;
    }
    bool string(std::string &out)
    {
        ++i;  // opening quote
        while (i < s.size() && s[i] != '"') {
            if (s[i] != '\\') {
                out.push_back(s[i++]);
                continue;
            }
            if (i + 1 >= s.size())
                return fail("bad escape");
            const char e = s[i + 1];
            i += 2;
            switch (e) {
            case 'n': out.push_back('\n'); break;
            case 't': out.push_back('\t'); break;
            case 'r': out.push_back('\r'); break;
            case 'b': out.push_back('\b'); break;
            case 'f': out.push_back('\f'); break;
            case 'u': {
                uint32_t cp;
                if (!hex4(cp))
                    return fail("bad \\u escape");
                if (cp >= 0xD800 && cp < 0xDC00 && i + 1 < s.size() && s[i] == '\\' && s[i + 1] == 'u') {
                    i += 2;
                    uint32_t lo;
                    if (!hex4(lo) || lo < 0xDC00 || lo >= 0xE000)
                        return fail("bad surrogate pair");
                    cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                }
                utf8(out, cp);
                break;
            }
            default: out.push_back(e); break;  // '"', '\\', '/'
            }
        }
        if (i >= s.size())
            return fail("missing closing quote");
        ++i;
        return true;
    }
};

inline bool readFile(const std::string &path, std::string &out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f)
        return false;
    std::stringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return !out.empty();
}

// OPTPT_ERR_PARSE (-4) with the parser's message on failure.
inline int parseJson(const std::string &text, Json &out, const std::string &what)
{
    JsonParser p(text);
    if (!p.value(out, 0))
        return optpt_internal_set_error(-4, ("error parsing " + what + ": " + p.err).c_str());
    p.ws();
    if (p.i != text.size())
        return optpt_internal_set_error(-4, ("error parsing " + what + ": trailing characters").c_str());
    return 0;
}

inline bool vec3(const Json *j, float *d)
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

}  // namespace optjson
