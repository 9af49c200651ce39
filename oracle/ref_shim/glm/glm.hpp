#pragma once
// Minimal host stand-in for the glm types that the reference's shared structs
// (MaterialData, TextureTransform) and src/light.cpp name. Only what those
// files use is provided.
#include <cmath>
namespace glm {
struct vec2 { float x, y; vec2(float s = 0.0f) : x(s), y(s) {} vec2(float a, float b) : x(a), y(b) {} };
struct vec3 { float x, y, z; vec3(float s = 0.0f) : x(s), y(s), z(s) {} vec3(float a, float b, float c) : x(a), y(b), z(c) {} };
struct vec4 { float x, y, z, w; vec4(float s = 0.0f) : x(s), y(s), z(s), w(s) {} };
inline float radians(float deg) { return deg * 0.01745329251994329577f; }
}
