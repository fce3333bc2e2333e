/* TEST INFRASTRUCTURE: host stand-in for make_float2/3/4 (oracle/_ref only). */
#ifndef ORC_SHIM_VECTOR_FUNCTIONS_H
#define ORC_SHIM_VECTOR_FUNCTIONS_H
#include "vector_types.h"
static inline float2 make_float2(float x, float y) { float2 r = {x, y}; return r; }
static inline float3 make_float3(float x, float y, float z) { float3 r = {x, y, z}; return r; }
static inline float4 make_float4(float x, float y, float z, float w) { float4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }
static inline uint3 make_uint3(unsigned int x, unsigned int y, unsigned int z) { uint3 r = {x, y, z}; return r; }
#endif
