#pragma once
// Host stand-in for the OptiX SDK's sutil/vec_math.h: the float2/float3/float4
// component-wise operators and helpers that the reference's BSDF headers call,
// written from plain vector algebra. Scalar lerp and maxValue are NOT defined
// here because the reference defines them itself (cuda_utils.h:14-22).
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#ifndef M_PIf
#define M_PIf 3.14159265358979323846f
#endif
#ifndef M_1_PIf
#define M_1_PIf 0.318309886183790671538f
#endif
#define VM_INL inline

VM_INL float2 make_float2(float s) { return ::make_float2(s, s); }
VM_INL float3 make_float3(float s) { return ::make_float3(s, s, s); }
VM_INL float3 make_float3(const float4 &a) { return ::make_float3(a.x, a.y, a.z); }
VM_INL float4 make_float4(float s) { return ::make_float4(s, s, s, s); }
VM_INL float4 make_float4(const float3 &a, float w) { return ::make_float4(a.x, a.y, a.z, w); }

// float2
VM_INL float2 operator+(float2 a, float2 b) { return ::make_float2(a.x + b.x, a.y + b.y); }
VM_INL float2 operator+(float2 a, float b) { return ::make_float2(a.x + b, a.y + b); }
VM_INL float2 operator+(float a, float2 b) { return ::make_float2(a + b.x, a + b.y); }
VM_INL float2 operator-(float2 a, float2 b) { return ::make_float2(a.x - b.x, a.y - b.y); }
VM_INL float2 operator-(float a, float2 b) { return ::make_float2(a - b.x, a - b.y); }
VM_INL float2 operator*(float2 a, float2 b) { return ::make_float2(a.x * b.x, a.y * b.y); }
VM_INL float2 operator*(float2 a, float s) { return ::make_float2(a.x * s, a.y * s); }
VM_INL float2 operator*(float s, float2 a) { return ::make_float2(s * a.x, s * a.y); }
VM_INL float2 operator/(float2 a, float2 b) { return ::make_float2(a.x / b.x, a.y / b.y); }
VM_INL float2 operator/(float2 a, float s) { return ::make_float2(a.x / s, a.y / s); }
VM_INL float2 operator/(float s, float2 a) { return ::make_float2(s / a.x, s / a.y); }
VM_INL void operator*=(float2 &a, float2 b) { a = a * b; }
VM_INL void operator+=(float2 &a, float2 b) { a = a + b; }
VM_INL float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }

// float3
VM_INL float3 operator+(float3 a, float3 b) { return ::make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
VM_INL float3 operator+(float3 a, float b) { return ::make_float3(a.x + b, a.y + b, a.z + b); }
VM_INL float3 operator+(float a, float3 b) { return ::make_float3(a + b.x, a + b.y, a + b.z); }
VM_INL float3 operator-(float3 a) { return ::make_float3(-a.x, -a.y, -a.z); }
VM_INL float3 operator-(float3 a, float3 b) { return ::make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
VM_INL float3 operator-(float3 a, float b) { return ::make_float3(a.x - b, a.y - b, a.z - b); }
VM_INL float3 operator-(float a, float3 b) { return ::make_float3(a - b.x, a - b.y, a - b.z); }
VM_INL float3 operator*(float3 a, float3 b) { return ::make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
VM_INL float3 operator*(float3 a, float s) { return ::make_float3(a.x * s, a.y * s, a.z * s); }
VM_INL float3 operator*(float s, float3 a) { return ::make_float3(s * a.x, s * a.y, s * a.z); }
VM_INL float3 operator/(float3 a, float3 b) { return ::make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
VM_INL float3 operator/(float3 a, float s) { return ::make_float3(a.x / s, a.y / s, a.z / s); }
VM_INL float3 operator/(float s, float3 a) { return ::make_float3(s / a.x, s / a.y, s / a.z); }
VM_INL void operator+=(float3 &a, float3 b) { a = a + b; }
VM_INL void operator-=(float3 &a, float3 b) { a = a - b; }
VM_INL void operator*=(float3 &a, float3 b) { a = a * b; }
VM_INL void operator*=(float3 &a, float s) { a = a * s; }
VM_INL void operator/=(float3 &a, float s) { a = a / s; }
VM_INL float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
VM_INL float3 cross(float3 a, float3 b)
{
    return ::make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
VM_INL float length(float3 a) { return sqrtf(dot(a, a)); }
VM_INL float3 normalize(float3 a) { float inv = 1.0f / sqrtf(dot(a, a)); return a * inv; }
VM_INL float3 faceforward(float3 n, float3 i, float3 nref) { return n * copysignf(1.0f, dot(i, nref)); }
VM_INL float fmaxf(float3 a) { return ::fmaxf(::fmaxf(a.x, a.y), a.z); }
VM_INL float3 fminf(float3 a, float3 b) { return ::make_float3(::fminf(a.x, b.x), ::fminf(a.y, b.y), ::fminf(a.z, b.z)); }
VM_INL float3 lerp(float3 a, float3 b, float t) { return a + t * (b - a); }

// float4
VM_INL float4 operator+(float4 a, float4 b) { return ::make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
VM_INL float4 operator+(float4 a, float b) { return ::make_float4(a.x + b, a.y + b, a.z + b, a.w + b); }
VM_INL float4 operator-(float4 a, float4 b) { return ::make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
VM_INL float4 operator*(float4 a, float4 b) { return ::make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
VM_INL float4 operator*(float s, float4 a) { return ::make_float4(s * a.x, s * a.y, s * a.z, s * a.w); }
VM_INL float4 operator*(float4 a, float s) { return ::make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
VM_INL float4 operator/(float4 a, float4 b) { return ::make_float4(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w); }
VM_INL float4 operator/(float4 a, float s) { return ::make_float4(a.x / s, a.y / s, a.z / s, a.w / s); }
VM_INL float4 lerp(float4 a, float4 b, float t) { return a + t * (b - a); }
VM_INL float clamp(float f, float a, float b) { return ::fmaxf(a, ::fminf(f, b)); }
VM_INL float4 clamp(float4 v, float a, float b)
{
    return ::make_float4(clamp(v.x, a, b), clamp(v.y, a, b), clamp(v.z, a, b), clamp(v.w, a, b));
}
