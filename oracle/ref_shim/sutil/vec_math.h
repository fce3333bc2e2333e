/* TEST INFRASTRUCTURE (oracle/_ref only): host restatement, from the vector algebra, of the
 * float2/float3/float4 helpers the reference takes from the OptiX SDK's sutil/vec_math.h.
 * Operation order (it fixes float rounding) is the one the C oracle uses:
 *   dot = x*x' + y*y' + z*z' (left to right), normalize(v) = v * (1 / sqrt(dot(v, v))),
 *   reflect(i, n) = i - 2 n dot(n, i), faceforward(n, i, nref) = dot(i, nref) >= 0 ? n : -n. */
#ifndef ORC_SHIM_VEC_MATH_H
#define ORC_SHIM_VEC_MATH_H
#include "../cuda_runtime.h"
#ifndef M_PIf
#define M_PIf 3.14159265358979323846f
#endif
static inline float3 make_float3(const float4& a) { return make_float3(a.x, a.y, a.z); }
static inline float4 make_float4(const float3& a, float w) { return make_float4(a.x, a.y, a.z, w); }
static inline float4 make_float4(float x, const float3& a) { return make_float4(x, a.x, a.y, a.z); }
static inline float3 operator+(const float3& a, const float3& b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline float3 operator-(const float3& a, const float3& b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline float3 operator-(const float3& a) { return make_float3(-a.x, -a.y, -a.z); }
static inline float3 operator*(const float3& a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
static inline float3 operator*(float s, const float3& a) { return make_float3(s * a.x, s * a.y, s * a.z); }
static inline float3 operator/(const float3& a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
static inline void operator*=(float3& a, float s) { a.x *= s; a.y *= s; a.z *= s; }
static inline void operator+=(float3& a, const float3& b) { a.x += b.x; a.y += b.y; a.z += b.z; }
static inline float dot(const float3& a, const float3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float dot(const float2& a, const float2& b) { return a.x * b.x + a.y * b.y; }
static inline float3 cross(const float3& a, const float3& b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float length(const float3& v) { return sqrtf(dot(v, v)); }
static inline float3 normalize(const float3& v) { float inv = 1.0f / sqrtf(dot(v, v)); return v * inv; }
static inline float3 reflect(const float3& i, const float3& n) { return i - 2.0f * n * dot(n, i); }
static inline float3 faceforward(const float3& n, const float3& i, const float3& nref) {
    return dot(i, nref) >= 0.0f ? n : -n;
}
#endif
