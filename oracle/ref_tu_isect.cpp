/* TEST INFRASTRUCTURE (oracle/_ref only): compiles the reference's cuda/intersection.cu on the host. */
#include "ref_shim/ref_prelude.h"
#include "cuda/intersection.cu"
extern "C" void orc_ref_set_params_isect(const soltrace::LaunchParams* p) { params = *p; }
