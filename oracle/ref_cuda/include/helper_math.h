/*
 * helper_math.h stand-in for the reference's CUDA build (baseline timing only):
 * the float3/int3/uint3 arithmetic the reference relies on, for host and
 * device.  Conventions of the CUDA samples' header: component-wise operators,
 * dot as x*x'+y*y'+z*z' (left to right), length = sqrt(dot), normalize =
 * v * rsqrt(dot(v, v)), lerp(a, b, t) = a + t*(b - a), clamp(v, lo, hi) =
 * max(lo, min(v, hi)).
 */
#pragma once
#include <cuda_runtime.h>
#include <vector_types.h>
#include <vector_functions.h>
#include <math.h>

#ifndef __CUDACC__
inline float rsqrtf(float x) { return 1.0f / sqrtf(x); }
#endif

/* conversions */
__host__ __device__ inline float3 make_float3(float s) { return make_float3(s, s, s); }
__host__ __device__ inline float3 make_float3(int3 a) { return make_float3((float)a.x, (float)a.y, (float)a.z); }
__host__ __device__ inline float3 make_float3(uint3 a) { return make_float3((float)a.x, (float)a.y, (float)a.z); }
__host__ __device__ inline float3 make_float3(float4 a) { return make_float3(a.x, a.y, a.z); }
__host__ __device__ inline int3 make_int3(int s) { return make_int3(s, s, s); }
__host__ __device__ inline int3 make_int3(float3 a) { return make_int3((int)a.x, (int)a.y, (int)a.z); }
__host__ __device__ inline int3 make_int3(uint3 a) { return make_int3((int)a.x, (int)a.y, (int)a.z); }
__host__ __device__ inline uint3 make_uint3(unsigned int s) { return make_uint3(s, s, s); }
__host__ __device__ inline uint3 make_uint3(int3 a) { return make_uint3((unsigned int)a.x, (unsigned int)a.y, (unsigned int)a.z); }

/* float3 */
__host__ __device__ inline float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
__host__ __device__ inline float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline float3 operator+(float3 a, float b) { return make_float3(a.x + b, a.y + b, a.z + b); }
__host__ __device__ inline float3 operator+(float b, float3 a) { return make_float3(a.x + b, a.y + b, a.z + b); }
__host__ __device__ inline void operator+=(float3& a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
__host__ __device__ inline void operator+=(float3& a, float b) { a.x += b; a.y += b; a.z += b; }
__host__ __device__ inline float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline float3 operator-(float3 a, float b) { return make_float3(a.x - b, a.y - b, a.z - b); }
__host__ __device__ inline float3 operator-(float b, float3 a) { return make_float3(b - a.x, b - a.y, b - a.z); }
__host__ __device__ inline void operator-=(float3& a, float3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
__host__ __device__ inline void operator-=(float3& a, float b) { a.x -= b; a.y -= b; a.z -= b; }
__host__ __device__ inline float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ inline float3 operator*(float3 a, float b) { return make_float3(a.x * b, a.y * b, a.z * b); }
__host__ __device__ inline float3 operator*(float b, float3 a) { return make_float3(b * a.x, b * a.y, b * a.z); }
__host__ __device__ inline void operator*=(float3& a, float3 b) { a.x *= b.x; a.y *= b.y; a.z *= b.z; }
__host__ __device__ inline void operator*=(float3& a, float b) { a.x *= b; a.y *= b; a.z *= b; }
__host__ __device__ inline float3 operator/(float3 a, float3 b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
__host__ __device__ inline float3 operator/(float3 a, float b) { return make_float3(a.x / b, a.y / b, a.z / b); }
__host__ __device__ inline float3 operator/(float b, float3 a) { return make_float3(b / a.x, b / a.y, b / a.z); }
__host__ __device__ inline void operator/=(float3& a, float3 b) { a.x /= b.x; a.y /= b.y; a.z /= b.z; }
__host__ __device__ inline void operator/=(float3& a, float b) { a.x /= b; a.y /= b; a.z /= b; }

/* int3 */
__host__ __device__ inline int3 operator-(int3 a) { return make_int3(-a.x, -a.y, -a.z); }
__host__ __device__ inline int3 operator+(int3 a, int3 b) { return make_int3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline int3 operator+(int3 a, int b) { return make_int3(a.x + b, a.y + b, a.z + b); }
__host__ __device__ inline int3 operator-(int3 a, int3 b) { return make_int3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline int3 operator-(int3 a, int b) { return make_int3(a.x - b, a.y - b, a.z - b); }
__host__ __device__ inline int3 operator*(int3 a, int b) { return make_int3(a.x * b, a.y * b, a.z * b); }

/* uint3 */
__host__ __device__ inline uint3 operator+(uint3 a, uint3 b) { return make_uint3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline uint3 operator+(uint3 a, unsigned int b) { return make_uint3(a.x + b, a.y + b, a.z + b); }
__host__ __device__ inline uint3 operator-(uint3 a, uint3 b) { return make_uint3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline uint3 operator-(uint3 a, unsigned int b) { return make_uint3(a.x - b, a.y - b, a.z - b); }
__host__ __device__ inline uint3 operator*(uint3 a, unsigned int b) { return make_uint3(a.x * b, a.y * b, a.z * b); }

/* reductions and shaping */
__host__ __device__ inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline float length(float3 v) { return sqrtf(dot(v, v)); }
__host__ __device__ inline float3 normalize(float3 v) { float inv = rsqrtf(dot(v, v)); return v * inv; }
__host__ __device__ inline float lerp(float a, float b, float t) { return a + t * (b - a); }
__host__ __device__ inline float3 lerp(float3 a, float3 b, float t) { return a + t * (b - a); }
__host__ __device__ inline float clamp(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
__host__ __device__ inline int clamp(int f, int a, int b) { return f < a ? a : (f > b ? b : f); }
__host__ __device__ inline unsigned int clamp(unsigned int f, unsigned int a, unsigned int b) { return f < a ? a : (f > b ? b : f); }
__host__ __device__ inline float3 clamp(float3 v, float3 a, float3 b) { return make_float3(clamp(v.x, a.x, b.x), clamp(v.y, a.y, b.y), clamp(v.z, a.z, b.z)); }
__host__ __device__ inline int3 clamp(int3 v, int3 a, int3 b) { return make_int3(clamp(v.x, a.x, b.x), clamp(v.y, a.y, b.y), clamp(v.z, a.z, b.z)); }
__host__ __device__ inline uint3 clamp(uint3 v, uint3 a, uint3 b) { return make_uint3(clamp(v.x, a.x, b.x), clamp(v.y, a.y, b.y), clamp(v.z, a.z, b.z)); }
__host__ __device__ inline float3 cross(float3 a, float3 b) { return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
