/* TEST INFRASTRUCTURE (oracle/_ref only): compiles the reference's cuda/materials.cu on the host. */
#include "ref_shim/ref_prelude.h"
#include "cuda/materials.cu"
extern "C" void orc_ref_set_params_mat(const soltrace::LaunchParams* p) { params = *p; }
