// csp_kernels.cuh -- launch interface of the CUDA kernels (host side).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "csp_types.cuh"

namespace csp {

struct TraceArgs {
    const Node* nodes;
    const Prim* prims;
    const Optics* optics;
    const SunFrame* sun;
    float4* hits;        // [count * kMaxDepth] for rays ray_begin .. ray_begin + count - 1
    uint32_t* ids;       // [count * kMaxDepth] or nullptr
    uint64_t ray_begin;  // global index of the first ray of this launch
    uint64_t count;      // rays in this launch
    uint64_t seed;
    uint32_t instance;
    int pad;
};

// Sun-plane distance and parallelogram (lib/geometry_manager.cpp:97-148 with the reductions of
// lib/sun_utils.cu:53-179) plus the per-launch cone frame (cuda/sun.cu:76-79), one block.
cudaError_t launch_prepare_sun(const Aabb* aabbs, int n, float sx, float sy, float sz, float tan_pad, int shape,
                               float param, SunFrame* out, cudaStream_t stream);

// Trace rays [ray_begin, ray_begin + count): generation, closest-hit search, shading, the dense
// hit-record write.  Scenes of up to 8 elements (n_prims) take the shared-memory element list path.
cudaError_t launch_trace(const TraceArgs& args, int n_prims, cudaStream_t stream);

}  // namespace csp
