// csp_system.h -- state behind one csp_handle.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "csp_c_api.h"
#include "csp_kernels.cuh"
#include "csp_scene.h"

namespace csp {

int set_error(int status, const std::string& msg);

// A named range on the NVTX timeline (Nsight Systems, Nsight Compute's range filters) for the
// lifetime of the object: the host stages of the library (setup, update, trace, copies, batch runs,
// server steps).  Without a tool attached the calls do nothing.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
int cuda_status(cudaError_t e, const char* what);

// Sun shapes the ABI accepts: pillbox or Gaussian, with or without CSP_SUN_ACCURATE.
inline bool valid_sun_shape(int shape) { return shape >= 0 && shape <= (CSP_SUN_GAUSSIAN | CSP_SUN_ACCURATE); }

// Angle the sun plane is padded by: the pillbox half angle (lib/geometry_manager.cpp:129), or 5
// sigma for the Gaussian sun.
inline double sun_pad_angle(int shape, double param) { return (shape & CSP_SUN_GAUSSIAN) ? 5.0 * param : param; }

// A ray window [first, first + count) whose indices all stay below kRayIndexLimit (checked without
// overflow).
inline bool valid_ray_window(uint64_t first, uint64_t count) {
    return first <= kRayIndexLimit && count <= kRayIndexLimit - first;
}

struct System {
    int device = -1;
    uint64_t num_rays = 0;
    std::vector<csp_element> elements;
    double sun_dir[3] = {0.0, 0.0, 1.0};
    int sun_shape = CSP_SUN_PILLBOX;
    double sun_param = 0.0;
    uint64_t seed = 0;
    uint32_t instance = 0;
    bool record_ids = false;
    bool initialized = false;

    HostScene scene;
    HostGrid grid;
    int accel = CSP_ACCEL_AUTO;

    Node* d_nodes = nullptr;
    Prim* d_prims = nullptr;
    Optics* d_optics = nullptr;
    Aabb* d_aabbs = nullptr;
    SunFrame* d_sun = nullptr;
    float4* d_hits = nullptr;
    uint32_t* d_ids = nullptr;
    GridDesc* d_grid = nullptr;
    const float* h3t12 = nullptr;  // Halton table of the device (halton3_table)
    GridDesc grid_host{};  // host copy of the descriptor (source of the async upload)
    uint32_t* d_cells = nullptr;
    Aabb* d_items = nullptr;
    Aabb* d_global = nullptr;
    size_t cap_cells = 0, cap_items = 0, cap_global = 0;
    // sun-ray candidate grid (scenes of more than kFlatListMax elements): its arrays, and the build
    // job (host copy = source of the async upload)
    unsigned char* d_sgrid = nullptr;
    size_t cap_sgrid = 0;
    SunGridJob* d_sgjob = nullptr;
    unsigned long long* d_tile_counter = nullptr;  // guided tile grabs of the launches on `stream`
    SunGridJob sgjob_host{};
    // compact records (csp_run_to_host_compact): points, counts, block offsets, records
    float* d_cpoints = nullptr;
    uint8_t* d_ccounts = nullptr;
    unsigned long long* d_csums = nullptr;
    float4* d_crecords = nullptr;
    uint64_t cap_compact_rays = 0, cap_crecords = 0;
    uint32_t* d_flux = nullptr;              // csp_flux_map counts
    unsigned long long* d_fstats = nullptr;  // [4]
    size_t cap_flux = 0;
    size_t cap_nodes = 0, cap_prims = 0, cap_optics = 0, cap_aabbs = 0;
    uint64_t cap_rays = 0;
    bool ids_allocated = false;

    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    double time_setup = 0.0;
    double time_trace = 0.0;

    ~System();
    void release();
    int ensure_streams();
    int upload_scene();
    int upload_grid(bool arrays);
    int prepare_sun();
    int build_sungrid();
    float pad_angle() const;
    int ensure_hit_buffers();
    int initialize();
    int update();
    TraceArgs args(uint64_t begin, uint64_t count) const;
    int trace_async(cudaStream_t st);
    int run();
    int run_to_host(float* dst, uint32_t* ids);
    int run_to_host_compact(float* points, uint8_t* counts, float* records, uint64_t capacity, uint64_t* n_records);
    int flux_map(uint32_t nx, uint32_t ny, uint32_t* counts, double dni, double* flux, bool staged = false);
};

// |(v1 - v0) x (v3 - v0)| of a sun frame, in double
double sun_plane_area(const SunFrame& f);

// flux = counts * dni * sun area / rays / bin area
void counts_to_flux(const uint32_t* counts, size_t n, double dni, double sun_area, uint64_t rays, double bin_area,
                    double* flux);

}  // namespace csp
