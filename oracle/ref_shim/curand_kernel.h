/* TEST INFRASTRUCTURE (oracle/_ref only).  The reference seeds a cuRAND XORWOW state per ray
 * (cuda/sun.cu:72-84).  That generator is replaced by Philox-4x32-10 keyed on
 * (seed, instance) with counter (ray, bounce 0): curand_init's `seed` argument is the ray number;
 * successive curand_uniform calls return successive Philox words mapped to (0, 1]. */
#ifndef ORC_SHIM_CURAND_KERNEL_H
#define ORC_SHIM_CURAND_KERNEL_H
#include "../orc_detmath.h"
struct curandState { orc_u32x4 block; int used; };
extern thread_local unsigned long long orc_ref_seed;
extern thread_local unsigned int orc_ref_instance;
static inline void curand_init(unsigned long long seed, unsigned long long subsequence, unsigned long long offset,
                               curandState* st) {
    (void)subsequence; (void)offset;
    st->block = orc_draw(seed, 0, 0, orc_ref_instance, orc_ref_seed);
    st->used = 0;
}
static inline float curand_uniform(curandState* st) { return orc_u01(st->block.v[(st->used++) & 3]); }
#endif
