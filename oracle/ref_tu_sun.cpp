/* TEST INFRASTRUCTURE (oracle/_ref only): compiles the reference's cuda/sun.cu on the host.
 * cosf/sinf of the cone-sampling angle are routed to the project's deterministic sin/cos so the
 * host build, the C oracle and the CUDA kernels draw identical directions. */
#include "ref_shim/ref_prelude.h"
#include "orc_detmath.h"
static inline float orc_ref_cosf(float x) { float s, c; orc_sincosf(x, &s, &c); return c; }
static inline float orc_ref_sinf(float x) { float s, c; orc_sincosf(x, &s, &c); return s; }
#define cosf(x) orc_ref_cosf(x)
#define sinf(x) orc_ref_sinf(x)
#include "cuda/sun.cu"
#undef cosf
#undef sinf
extern "C" void orc_ref_set_params_sun(const soltrace::LaunchParams* p) { params = *p; }
