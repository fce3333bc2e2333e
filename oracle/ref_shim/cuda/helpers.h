/* TEST INFRASTRUCTURE (oracle/_ref only): the one helper the reference uses from the SDK's
 * cuda/helpers.h, restated: pass a float3 as three 32-bit attribute words. */
#ifndef ORC_SHIM_CUDA_HELPERS_H
#define ORC_SHIM_CUDA_HELPERS_H
#define float3_as_args(u) __float_as_uint((u).x), __float_as_uint((u).y), __float_as_uint((u).z)
#endif
