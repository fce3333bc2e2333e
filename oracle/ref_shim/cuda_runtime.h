/* TEST INFRASTRUCTURE: minimal host stand-in for <cuda_runtime.h> so the reference's device
 * programs and scene code compile as plain C++ (oracle/_ref only). */
#ifndef ORC_SHIM_CUDA_RUNTIME_H
#define ORC_SHIM_CUDA_RUNTIME_H
#include <cstring>
#include <cmath>
#include <math.h>
#include "vector_types.h"
#include "vector_functions.h"
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __global__
#define __global__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
#ifndef __inline__
#define __inline__ inline
#endif
/* Each reference .cu file defines its own `params`; compiled as separate host translation units
 * they each keep a private copy that the driver fills. */
#ifndef __constant__
#define __constant__ static
#endif
static inline unsigned int __float_as_uint(float f) { unsigned int u; std::memcpy(&u, &f, 4); return u; }
static inline float __uint_as_float(unsigned int u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline int __float_as_int(float f) { int u; std::memcpy(&u, &f, 4); return u; }
static inline float __int_as_float(int u) { float f; std::memcpy(&f, &u, 4); return f; }
#endif
