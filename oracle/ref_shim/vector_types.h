/* TEST INFRASTRUCTURE: host stand-in for the CUDA vector types, used only to compile the
 * reference's device programs on the host (oracle/_ref).  Names and member layout follow the CUDA
 * headers; nothing else is taken from them. */
#ifndef ORC_SHIM_VECTOR_TYPES_H
#define ORC_SHIM_VECTOR_TYPES_H
struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct alignas(16) float4 { float x, y, z, w; };
struct uint3 { unsigned int x, y, z; };
struct int2 { int x, y; };
#endif
