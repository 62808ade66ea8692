/*
 * helper_math.h stand-in: the float3/int3/uint3 arithmetic the reference
 * kernels rely on, written out for the CPU emulation (test infrastructure).
 * Semantics follow the usual CUDA-samples conventions: component-wise
 * operators, dot as x*x'+y*y'+z*z' (left to right), length = sqrt(dot),
 * normalize = v * rsqrt(dot(v, v)), lerp(a, b, t) = a + t*(b - a),
 * clamp(v, lo, hi) = max(lo, min(v, hi)).
 */
#pragma once
#include <cmath>
#include <algorithm>
#include "vector_types.h"
#include "vector_functions.h"

inline float fminf_(float a, float b) { return a < b ? a : b; }
inline float fmaxf_(float a, float b) { return a > b ? a : b; }

/* conversions */
inline float3 make_float3(float s) { return make_float3(s, s, s); }
inline float3 make_float3(int3 a) { return make_float3((float)a.x, (float)a.y, (float)a.z); }
inline float3 make_float3(uint3 a) { return make_float3((float)a.x, (float)a.y, (float)a.z); }
inline float3 make_float3(float4 a) { return make_float3(a.x, a.y, a.z); }
inline int3 make_int3(int s) { return make_int3(s, s, s); }
inline int3 make_int3(float3 a) { return make_int3((int)a.x, (int)a.y, (int)a.z); }
inline int3 make_int3(uint3 a) { return make_int3((int)a.x, (int)a.y, (int)a.z); }
inline uint3 make_uint3(unsigned int s) { return make_uint3(s, s, s); }
inline uint3 make_uint3(int3 a) { return make_uint3((unsigned int)a.x, (unsigned int)a.y, (unsigned int)a.z); }

/* float3 */
inline float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
inline float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator+(float3 a, float b) { return make_float3(a.x + b, a.y + b, a.z + b); }
inline float3 operator+(float b, float3 a) { return make_float3(a.x + b, a.y + b, a.z + b); }
inline void operator+=(float3& a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
inline void operator+=(float3& a, float b) { a.x += b; a.y += b; a.z += b; }
inline float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator-(float3 a, float b) { return make_float3(a.x - b, a.y - b, a.z - b); }
inline float3 operator-(float b, float3 a) { return make_float3(b - a.x, b - a.y, b - a.z); }
inline void operator-=(float3& a, float3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
inline void operator-=(float3& a, float b) { a.x -= b; a.y -= b; a.z -= b; }
inline float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator*(float3 a, float b) { return make_float3(a.x * b, a.y * b, a.z * b); }
inline float3 operator*(float b, float3 a) { return make_float3(b * a.x, b * a.y, b * a.z); }
inline void operator*=(float3& a, float3 b) { a.x *= b.x; a.y *= b.y; a.z *= b.z; }
inline void operator*=(float3& a, float b) { a.x *= b; a.y *= b; a.z *= b; }
inline float3 operator/(float3 a, float3 b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator/(float3 a, float b) { return make_float3(a.x / b, a.y / b, a.z / b); }
inline float3 operator/(float b, float3 a) { return make_float3(b / a.x, b / a.y, b / a.z); }
inline void operator/=(float3& a, float3 b) { a.x /= b.x; a.y /= b.y; a.z /= b.z; }
inline void operator/=(float3& a, float b) { a.x /= b; a.y /= b; a.z /= b; }

/* int3 */
inline int3 operator-(int3 a) { return make_int3(-a.x, -a.y, -a.z); }
inline int3 operator+(int3 a, int3 b) { return make_int3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline int3 operator+(int3 a, int b) { return make_int3(a.x + b, a.y + b, a.z + b); }
inline int3 operator-(int3 a, int3 b) { return make_int3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline int3 operator-(int3 a, int b) { return make_int3(a.x - b, a.y - b, a.z - b); }
inline int3 operator*(int3 a, int b) { return make_int3(a.x * b, a.y * b, a.z * b); }

/* uint3 */
inline uint3 operator+(uint3 a, uint3 b) { return make_uint3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline uint3 operator+(uint3 a, unsigned int b) { return make_uint3(a.x + b, a.y + b, a.z + b); }
inline uint3 operator-(uint3 a, uint3 b) { return make_uint3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline uint3 operator-(uint3 a, unsigned int b) { return make_uint3(a.x - b, a.y - b, a.z - b); }
inline uint3 operator*(uint3 a, unsigned int b) { return make_uint3(a.x * b, a.y * b, a.z * b); }

/* reductions and shaping */
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(float3 v) { return std::sqrt(dot(v, v)); }
inline float3 normalize(float3 v) { float inv = 1.0f / std::sqrt(dot(v, v)); return v * inv; }
inline float lerp(float a, float b, float t) { return a + t * (b - a); }
inline float3 lerp(float3 a, float3 b, float t) { return a + t * (b - a); }
inline float clamp(float f, float a, float b) { return fmaxf_(a, fminf_(f, b)); }
inline int clamp(int f, int a, int b) { return std::max(a, std::min(f, b)); }
inline unsigned int clamp(unsigned int f, unsigned int a, unsigned int b) { return std::max(a, std::min(f, b)); }
inline float3 clamp(float3 v, float3 a, float3 b) { return make_float3(clamp(v.x, a.x, b.x), clamp(v.y, a.y, b.y), clamp(v.z, a.z, b.z)); }
inline int3 clamp(int3 v, int3 a, int3 b) { return make_int3(clamp(v.x, a.x, b.x), clamp(v.y, a.y, b.y), clamp(v.z, a.z, b.z)); }
inline uint3 clamp(uint3 v, uint3 a, uint3 b) { return make_uint3(clamp(v.x, a.x, b.x), clamp(v.y, a.y, b.y), clamp(v.z, a.z, b.z)); }
inline float3 cross(float3 a, float3 b) { return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
