// csp_c_api.cpp -- the C ABI (include/csp_c_api.h): handle lifecycle, device buffers, launches.
#include "csp_c_api.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "csp_kernels.cuh"
#include "csp_math.cuh"
#include "csp_scene.h"
#include "csp_system.h"

namespace {

thread_local std::string t_last_error;

int fail(int status, const std::string& msg) {
    t_last_error = msg;
    return status;
}

}  // namespace

namespace csp {

int set_error(int status, const std::string& msg) { return fail(status, msg); }

namespace {

// Allocations left before the injected failure (csp_debug_fail_allocation); -1: none pending.
std::atomic<long long> g_fail_after{-1};

bool injected_failure() {
    long long v = g_fail_after.load();
    while (v >= 0) {
        if (g_fail_after.compare_exchange_weak(v, v == 0 ? -1 : v - 1)) return v == 0;
    }
    return false;
}

}  // namespace

cudaError_t dev_alloc(void** p, size_t bytes) {
    if (injected_failure()) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

cudaError_t host_alloc(void** p, size_t bytes) {
    if (injected_failure()) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaHostAlloc(p, bytes, cudaHostAllocDefault);
}

int cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return CSP_OK;
    const int st = (e == cudaErrorMemoryAllocation) ? CSP_ERR_OUT_OF_MEMORY : CSP_ERR_CUDA;
    cudaGetLastError();  // clear the sticky-free error state of the runtime API
    return fail(st, std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
static int upload(T*& dptr, size_t& cap, const std::vector<T>& host, cudaStream_t st, const char* what) {
    const size_t n = host.size();
    if (n > cap) {
        if (dptr) cudaFree(dptr);
        dptr = nullptr;
        cap = 0;
        int rc = cuda_status(dev_alloc((void**)&dptr, std::max<size_t>(n, 1) * sizeof(T)), what);
        if (rc) return rc;
        cap = n;
    }
    if (n) return cuda_status(cudaMemcpyAsync(dptr, host.data(), n * sizeof(T), cudaMemcpyHostToDevice, st), what);
    return CSP_OK;
}

System::~System() { release(); }

void System::release() {
    if (device >= 0) cudaSetDevice(device);
    cudaFree(d_nodes);
    cudaFree(d_prims);
    cudaFree(d_optics);
    cudaFree(d_aabbs);
    cudaFree(d_sun);
    cudaFree(d_hits);
    cudaFree(d_ids);
    cudaFree(d_grid);
    cudaFree(d_cells);
    cudaFree(d_items);
    cudaFree(d_global);
    d_grid = nullptr;
    d_cells = nullptr;
    d_items = d_global = nullptr;
    cap_cells = cap_items = cap_global = 0;
    cudaFree(d_sgrid);
    cudaFree(d_sgjob);
    cudaFree(d_tile_counter);
    d_sgrid = nullptr;
    d_sgjob = nullptr;
    d_tile_counter = nullptr;
    cap_sgrid = 0;
    cudaFree(d_cpoints);
    cudaFree(d_ccounts);
    cudaFree(d_csums);
    cudaFree(d_crecords);
    d_cpoints = nullptr;
    d_ccounts = nullptr;
    d_csums = nullptr;
    d_crecords = nullptr;
    cap_compact_rays = cap_crecords = 0;
    cudaFree(d_flux);
    cudaFree(d_fstats);
    d_flux = nullptr;
    d_fstats = nullptr;
    cap_flux = 0;
    d_nodes = nullptr;
    d_prims = nullptr;
    d_optics = nullptr;
    d_aabbs = nullptr;
    d_sun = nullptr;
    d_hits = nullptr;
    d_ids = nullptr;
    cap_nodes = cap_prims = cap_optics = cap_aabbs = 0;
    cap_rays = 0;
    ids_allocated = false;
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    if (stream) cudaStreamDestroy(stream);
    ev0 = ev1 = nullptr;
    stream = copy_stream = nullptr;
    initialized = false;
}

int System::ensure_streams() {
    if (stream) return CSP_OK;
    int rc = cuda_status(cudaSetDevice(device), "cudaSetDevice");
    if (rc) return rc;
    if ((rc = cuda_status(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate"))) return rc;
    if ((rc = cuda_status(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking), "cudaStreamCreate")))
        return rc;
    if ((rc = cuda_status(cudaEventCreate(&ev0), "cudaEventCreate"))) return rc;
    return cuda_status(cudaEventCreate(&ev1), "cudaEventCreate");
}

int System::upload_scene() {
    int rc;
    if ((rc = upload(d_prims, cap_prims, scene.prims, stream, "upload prims"))) return rc;
    if ((rc = upload(d_optics, cap_optics, scene.optics, stream, "upload optics"))) return rc;
    if ((rc = upload(d_aabbs, cap_aabbs, scene.aabbs, stream, "upload aabbs"))) return rc;
    if ((rc = upload(d_nodes, cap_nodes, scene.nodes, stream, "upload bvh"))) return rc;
    if (!d_sun) {
        if ((rc = cuda_status(dev_alloc((void**)&d_sun, sizeof(SunFrame)), "cudaMalloc sun"))) return rc;
    }
    return CSP_OK;
}

// Field grid on the device: the cell arrays (when `arrays`) and the descriptor.
int System::upload_grid(bool arrays) {
    if (!grid.valid) return CSP_OK;
    int rc;
    if (arrays) {
        if ((rc = upload(d_cells, cap_cells, grid.cell_start, stream, "upload grid cells"))) return rc;
        if ((rc = upload(d_items, cap_items, grid.items, stream, "upload grid items"))) return rc;
        if ((rc = upload(d_global, cap_global, grid.global, stream, "upload grid globals"))) return rc;
    }
    if (!d_grid && (rc = cuda_status(dev_alloc((void**)&d_grid, sizeof(GridDesc)), "cudaMalloc grid"))) return rc;
    grid_host = csp::grid_desc(grid, d_cells, d_items, d_global);
    return cuda_status(cudaMemcpyAsync(d_grid, &grid_host, sizeof(GridDesc), cudaMemcpyHostToDevice, stream),
                       "upload grid");
}

float System::pad_angle() const {
    return (float)sun_pad_angle(sun_shape, sun_param);
}

int System::prepare_sun() {
    float s[3];
    sun_vector_f(sun_dir, s);
    scene.sun[0] = s[0];
    scene.sun[1] = s[1];
    scene.sun[2] = s[2];
    const float tan_pad = tanf(pad_angle());
    return cuda_status(launch_prepare_sun(d_aabbs, (int)scene.prims.size(), s[0], s[1], s[2], tan_pad, sun_shape,
                                          (float)sun_param, d_sun, stream),
                       "prepare_sun_kernel");
}

// Sun-ray candidate grid of the current poses and sun frame, built on the device behind the sun
// plane (scenes of more than kFlatListMax elements; the element list needs none).
int System::build_sungrid() {
    const uint32_t n = (uint32_t)scene.prims.size();
    if (n <= kFlatListMax) return CSP_OK;
    int rc;
    const size_t bytes = sungrid_bytes(n);
    if (bytes > cap_sgrid) {
        cudaFree(d_sgrid);
        d_sgrid = nullptr;
        cap_sgrid = 0;
        if ((rc = cuda_status(dev_alloc((void**)&d_sgrid, bytes), "cudaMalloc sun grid"))) return rc;
        cap_sgrid = bytes;
    }
    if (!d_sgjob && (rc = cuda_status(dev_alloc((void**)&d_sgjob, sizeof(SunGridJob)), "cudaMalloc sun grid job")))
        return rc;
    sungrid_place(d_sgrid, n, sgjob_host);
    sgjob_host.sun = d_sun;
    sgjob_host.aabbs = d_aabbs;
    if ((rc = cuda_status(cudaMemcpyAsync(d_sgjob, &sgjob_host, sizeof(SunGridJob), cudaMemcpyHostToDevice, stream),
                          "upload sun grid job")))
        return rc;
    return cuda_status(launch_sungrid_build(d_sgjob, 1, (int)n, stream), "sun grid build");
}

int System::ensure_hit_buffers() {
    if (num_rays > cap_rays || (record_ids && !ids_allocated)) {
        cudaFree(d_hits);
        cudaFree(d_ids);
        d_hits = nullptr;
        d_ids = nullptr;
        cap_rays = 0;
        ids_allocated = false;
        const size_t n = std::max<uint64_t>(num_rays, 1);
        int rc = cuda_status(dev_alloc((void**)&d_hits, n * kMaxDepth * sizeof(float4)), "cudaMalloc hit buffer");
        if (rc) return rc;
        if (record_ids) {
            rc = cuda_status(dev_alloc((void**)&d_ids, n * kMaxDepth * sizeof(uint32_t)), "cudaMalloc id buffer");
            if (rc) return rc;
            ids_allocated = true;
        }
        cap_rays = num_rays;
    }
    return CSP_OK;
}

int System::initialize() {
    NvtxRange nvtx("csp initialize");
    const auto t0 = std::chrono::steady_clock::now();
    int rc = ensure_streams();
    if (rc) return rc;
    if (!d_tile_counter &&
        (rc = cuda_status(dev_alloc((void**)&d_tile_counter, sizeof(unsigned long long)), "cudaMalloc tile counter")))
        return rc;
    h3t12 = halton3_table();
    std::string err;
    if ((rc = build_elements(elements.data(), (uint32_t)elements.size(), scene, err))) return fail(rc, err);
    build_bvh(scene);
    grid = HostGrid{};
    if (accel != CSP_ACCEL_BVH) build_grid(scene, grid);
    if (accel == CSP_ACCEL_GRID && !grid.valid && elements.size() > kFlatListMax)
        return fail(CSP_ERR_BAD_SCENE, "the scene is not a planar field: no grid (use CSP_ACCEL_AUTO or _BVH)");
    if ((rc = upload_scene())) return rc;
    if ((rc = upload_grid(true))) return rc;
    if ((rc = prepare_sun())) return rc;
    if ((rc = build_sungrid())) return rc;
    if ((rc = ensure_hit_buffers())) return rc;
    if ((rc = cuda_status(cudaStreamSynchronize(stream), "initialize"))) return rc;
    initialized = true;
    time_setup = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return CSP_OK;
}

int System::update() {
    NvtxRange nvtx("csp update");
    if (!initialized) return fail(CSP_ERR_STATE, "update() before initialize()");
    if (elements.size() != scene.prims.size())
        return fail(CSP_ERR_STATE, "update() needs the element count of initialize(); call initialize() again");
    std::string err;
    int rc = build_elements(elements.data(), (uint32_t)elements.size(), scene, err);
    if (rc) return fail(rc, err);
    refit_bvh(scene);
    // the grid holds one set of poses: rebuilt for the new ones
    grid = HostGrid{};
    if (accel != CSP_ACCEL_BVH) build_grid(scene, grid);
    if (accel == CSP_ACCEL_GRID && !grid.valid && elements.size() > kFlatListMax)
        return fail(CSP_ERR_BAD_SCENE, "the new poses are not a planar field: no grid (use CSP_ACCEL_AUTO or _BVH)");
    if ((rc = upload_scene())) return rc;
    if ((rc = upload_grid(true))) return rc;
    if ((rc = prepare_sun())) return rc;
    if ((rc = build_sungrid())) return rc;
    if ((rc = ensure_hit_buffers())) return rc;
    return cuda_status(cudaStreamSynchronize(stream), "update");
}

TraceArgs System::args(uint64_t begin, uint64_t count) const {
    TraceArgs a;
    a.nodes = d_nodes;
    a.prims = d_prims;
    a.optics = d_optics;
    a.sun = d_sun;
    a.hits = d_hits + begin * kMaxDepth;
    a.ids = (record_ids && d_ids) ? d_ids + begin * kMaxDepth : nullptr;
    a.ray_begin = begin;
    a.count = count;
    a.seed = seed;
    a.instance = instance;
    a.pad = 0;
    a.grid = grid.valid ? d_grid : nullptr;
    a.h3t12 = h3t12;
    a.sgrid = scene.prims.size() > kFlatListMax && d_sgrid ? sgjob_host.desc : nullptr;
    a.tile_counter = d_tile_counter;
    return a;
}

int System::trace_async(cudaStream_t st) {
    if (!initialized) return fail(CSP_ERR_STATE, "trace before initialize()");
    int rc = ensure_hit_buffers();
    if (rc) return rc;
    // it writes the hit buffer: it never overlaps the handle's other launches, so the tile counter
    // serves it on any stream
    return cuda_status(launch_trace(args(0, num_rays), (int)scene.prims.size(), st ? st : stream), "trace_kernel");
}

int System::run() {
    NvtxRange nvtx("csp run");
    if (!initialized) return fail(CSP_ERR_STATE, "run() before initialize()");
    int rc = ensure_hit_buffers();
    if (rc) return rc;
    if ((rc = cuda_status(cudaEventRecord(ev0, stream), "cudaEventRecord"))) return rc;
    if ((rc = cuda_status(launch_trace(args(0, num_rays), (int)scene.prims.size(), stream), "trace_kernel"))) return rc;
    if ((rc = cuda_status(cudaEventRecord(ev1, stream), "cudaEventRecord"))) return rc;
    if ((rc = cuda_status(cudaEventSynchronize(ev1), "trace"))) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    time_trace = ms * 1e-3;
    return CSP_OK;
}

int System::run_to_host(float* dst, uint32_t* ids_dst) {
    NvtxRange nvtx("csp run_to_host");
    if (!initialized) return fail(CSP_ERR_STATE, "run() before initialize()");
    int rc = ensure_hit_buffers();
    if (rc) return rc;
    const uint64_t chunk = std::max<uint64_t>(1u << 20, (num_rays + 15) / 16);
    std::vector<cudaEvent_t> done;
    const auto t0 = std::chrono::steady_clock::now();
    for (uint64_t b = 0; b < num_rays; b += chunk) {
        const uint64_t c = std::min(chunk, num_rays - b);
        if ((rc = cuda_status(launch_trace(args(b, c), (int)scene.prims.size(), stream), "trace_kernel"))) break;
        cudaEvent_t ev;
        if ((rc = cuda_status(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate"))) break;
        done.push_back(ev);
        if ((rc = cuda_status(cudaEventRecord(ev, stream), "cudaEventRecord"))) break;
        if ((rc = cuda_status(cudaStreamWaitEvent(copy_stream, ev, 0), "cudaStreamWaitEvent"))) break;
        rc = cuda_status(cudaMemcpyAsync(dst + b * kMaxDepth * 4, d_hits + b * kMaxDepth, c * kMaxDepth * sizeof(float4),
                                         cudaMemcpyDeviceToHost, copy_stream),
                         "D2H hit records");
        if (rc) break;
        if (ids_dst && record_ids && d_ids) {
            rc = cuda_status(cudaMemcpyAsync(ids_dst + b * kMaxDepth, d_ids + b * kMaxDepth,
                                             c * kMaxDepth * sizeof(uint32_t), cudaMemcpyDeviceToHost, copy_stream),
                             "D2H ids");
            if (rc) break;
        }
    }
    const int sync_rc = cuda_status(cudaStreamSynchronize(copy_stream), "D2H sync");
    const int sync_rc2 = cuda_status(cudaStreamSynchronize(stream), "trace sync");
    for (cudaEvent_t ev : done) cudaEventDestroy(ev);
    if (rc) return rc;
    if (sync_rc) return sync_rc;
    if (sync_rc2) return sync_rc2;
    time_trace = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return CSP_OK;
}

// Trace, then move the records in compact form: per ray its sun-plane point and the number of its
// further records, and those records in ray order (kernels in csp_kernels.cu).  Nothing is copied
// when the records exceed `capacity`; *n_records then tells how many there are.
int System::run_to_host_compact(float* points, uint8_t* counts, float* records, uint64_t capacity,
                                uint64_t* n_records) {
    NvtxRange nvtx("csp run_to_host_compact");
    if (!initialized) return fail(CSP_ERR_STATE, "run() before initialize()");
    int rc = ensure_hit_buffers();
    if (rc) return rc;
    const uint64_t n = num_rays;
    if (n > cap_compact_rays) {
        cudaFree(d_cpoints);
        cudaFree(d_ccounts);
        cudaFree(d_csums);
        d_cpoints = nullptr;
        d_ccounts = nullptr;
        d_csums = nullptr;
        cap_compact_rays = 0;
        if ((rc = cuda_status(dev_alloc((void**)&d_cpoints, std::max<uint64_t>(n, 1) * 3 * sizeof(float)), "cudaMalloc")))
            return rc;
        if ((rc = cuda_status(dev_alloc((void**)&d_ccounts, std::max<uint64_t>(n, 1)), "cudaMalloc"))) return rc;
        if ((rc = cuda_status(dev_alloc((void**)&d_csums, (compact_blocks(n) + 1) * sizeof(unsigned long long)),
                              "cudaMalloc")))
            return rc;
        cap_compact_rays = n;
    }
    const auto t0 = std::chrono::steady_clock::now();
    if ((rc = cuda_status(launch_trace(args(0, n), (int)scene.prims.size(), stream), "trace_kernel"))) return rc;
    if ((rc = cuda_status(launch_compact_count(d_hits, n, d_ccounts, d_csums, stream), "compact_count_kernel")))
        return rc;
    unsigned long long total = 0;
    if ((rc = cuda_status(cudaMemcpyAsync(&total, d_csums + compact_blocks(n), sizeof total, cudaMemcpyDeviceToHost,
                                          stream),
                          "D2H record count")))
        return rc;
    if ((rc = cuda_status(cudaStreamSynchronize(stream), "compact count"))) return rc;
    if (n_records) *n_records = total;
    if (total > capacity) return fail(CSP_ERR_INVALID_ARGUMENT, "the run's records exceed the capacity");
    if (total > cap_crecords) {
        cudaFree(d_crecords);
        d_crecords = nullptr;
        cap_crecords = 0;
        if ((rc = cuda_status(dev_alloc((void**)&d_crecords, total * sizeof(float4)), "cudaMalloc compact records")))
            return rc;
        cap_crecords = total;
    }
    if ((rc = cuda_status(launch_compact_write(d_hits, n, d_csums, d_cpoints, d_crecords, stream), "compact_write_kernel")))
        return rc;
    if (n && (rc = cuda_status(cudaMemcpyAsync(points, d_cpoints, n * 3 * sizeof(float), cudaMemcpyDeviceToHost, stream),
                               "D2H points")))
        return rc;
    if (n && (rc = cuda_status(cudaMemcpyAsync(counts, d_ccounts, n, cudaMemcpyDeviceToHost, stream), "D2H counts")))
        return rc;
    if (total && (rc = cuda_status(cudaMemcpyAsync(records, d_crecords, total * sizeof(float4), cudaMemcpyDeviceToHost,
                                                   stream),
                                   "D2H records")))
        return rc;
    if ((rc = cuda_status(cudaStreamSynchronize(stream), "compact copy"))) return rc;
    time_trace = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return CSP_OK;
}

double sun_plane_area(const SunFrame& f) {
    const double a[3] = {(double)f.v1.x - f.v0.x, (double)f.v1.y - f.v0.y, (double)f.v1.z - f.v0.z};
    const double b[3] = {(double)f.v3.x - f.v0.x, (double)f.v3.y - f.v0.y, (double)f.v3.z - f.v0.z};
    const double c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    return std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
}

void counts_to_flux(const uint32_t* counts, size_t n, double dni, double sun_area, uint64_t rays, double bin_area,
                    double* flux) {
    const double per = (rays > 0 && bin_area > 0) ? dni * sun_area / (double)rays / bin_area : 0.0;
    for (size_t i = 0; i < n; ++i) flux[i] = counts[i] * per;
}

int System::flux_map(uint32_t nx, uint32_t ny, uint32_t* counts, double dni, double* flux, bool staged) {
    NvtxRange nvtx("csp flux_map");
    if (!initialized || !d_hits) return fail(CSP_ERR_STATE, "flux map before initialize()/run()");
    if (nx == 0 || ny == 0 || (uint64_t)nx * ny > (1u << 26)) return fail(CSP_ERR_INVALID_ARGUMENT, "bad flux grid");
    const size_t nb = (size_t)nx * ny;
    int rc;
    if (nb > cap_flux) {
        cudaFree(d_flux);
        d_flux = nullptr;
        cap_flux = 0;
        if ((rc = cuda_status(dev_alloc((void**)&d_flux, nb * sizeof(uint32_t)), "cudaMalloc flux map"))) return rc;
        cap_flux = nb;
    }
    if (!d_fstats && (rc = cuda_status(dev_alloc((void**)&d_fstats, 4 * sizeof(unsigned long long)), "cudaMalloc")))
        return rc;
    FluxTarget F;
    flux_target(elements.back(), nx, ny, F);
    F.counts = d_flux;
    F.stats = d_fstats;
    F.staged = staged ? 1 : 0;
    if ((rc = cuda_status(cudaMemsetAsync(d_flux, 0, nb * sizeof(uint32_t), stream), "memset flux"))) return rc;
    if ((rc = cuda_status(cudaMemsetAsync(d_fstats, 0, 4 * sizeof(unsigned long long), stream), "memset"))) return rc;
    if ((rc = cuda_status(launch_flux_records(d_hits, num_rays * kMaxDepth, F, stream), "flux_records_kernel")))
        return rc;
    std::vector<uint32_t> host(nb);
    if ((rc = cuda_status(cudaMemcpyAsync(host.data(), d_flux, nb * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream),
                          "D2H flux map")))
        return rc;
    SunFrame f;
    if ((rc = cuda_status(cudaMemcpyAsync(&f, d_sun, sizeof(f), cudaMemcpyDeviceToHost, stream), "D2H sun frame")))
        return rc;
    if ((rc = cuda_status(cudaStreamSynchronize(stream), "flux map"))) return rc;
    if (counts) std::copy(host.begin(), host.end(), counts);
    if (flux)
        counts_to_flux(host.data(), nb, dni, sun_plane_area(f), num_rays, flux_bin_area(elements.back(), nx, ny), flux);
    return CSP_OK;
}

}  // namespace csp

using csp::System;

#define CSP_GUARD(h)                                                              \
    do {                                                                          \
        if (!(h)) return fail(CSP_ERR_INVALID_ARGUMENT, "null handle");           \
    } while (0)

extern "C" {

const char* csp_last_error(void) { return t_last_error.c_str(); }
int csp_abi_version(void) { return CSP_ABI_VERSION; }

int csp_bounds_check_status(int device, uint32_t* sites) {
    if (!sites) return fail(CSP_ERR_INVALID_ARGUMENT, "null output");
    *sites = 0;
    if (!csp::kBoundsCheckBuild) return fail(CSP_ERR_STATE, "not a bounds-check build (-DCSP_BOUNDS_CHECK)");
    int prev = -1;
    cudaGetDevice(&prev);
    int rc = csp::cuda_status(cudaSetDevice(device), "cudaSetDevice");
    if (rc) return rc;
    if ((rc = csp::cuda_status(cudaDeviceSynchronize(), "cudaDeviceSynchronize"))) return rc;
    *sites = csp::bounds_sites_trace() | csp::bounds_sites_batch() | csp::bounds_sites_sungrid();
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    return CSP_OK;
}

int csp_debug_fail_allocation(int64_t after) {
    if (after < -1) return fail(CSP_ERR_INVALID_ARGUMENT, "after must be >= -1");
    csp::g_fail_after.store((long long)after);
    return CSP_OK;
}

int csp_create(csp_handle* out, int device, uint64_t num_rays) {
    if (!out) return fail(CSP_ERR_INVALID_ARGUMENT, "null output handle");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return csp::cuda_status(e, "cudaGetDeviceCount");
    if (device < 0 || device >= count) return fail(CSP_ERR_INVALID_ARGUMENT, "no such CUDA device");
    if (!csp::valid_ray_window(0, num_rays)) return fail(CSP_ERR_INVALID_ARGUMENT, "num_rays must stay below 2^56");
    System* s = new (std::nothrow) System();
    if (!s) return fail(CSP_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->device = device;
    s->num_rays = num_rays;
    *out = reinterpret_cast<csp_handle>(s);
    return CSP_OK;
}

int csp_destroy(csp_handle h) {
    CSP_GUARD(h);
    delete reinterpret_cast<System*>(h);
    return CSP_OK;
}

int csp_set_num_rays(csp_handle h, uint64_t num_rays) {
    CSP_GUARD(h);
    if (!csp::valid_ray_window(0, num_rays)) return fail(CSP_ERR_INVALID_ARGUMENT, "num_rays must stay below 2^56");
    reinterpret_cast<System*>(h)->num_rays = num_rays;
    return CSP_OK;
}

int csp_add_element(csp_handle h, const csp_element* e) {
    CSP_GUARD(h);
    if (!e) return fail(CSP_ERR_INVALID_ARGUMENT, "null element");
    reinterpret_cast<System*>(h)->elements.push_back(*e);
    return CSP_OK;
}

int csp_set_elements(csp_handle h, const csp_element* e, uint32_t n) {
    CSP_GUARD(h);
    if (!e && n) return fail(CSP_ERR_INVALID_ARGUMENT, "null elements");
    System* s = reinterpret_cast<System*>(h);
    s->elements.assign(e, e + n);
    return CSP_OK;
}

int csp_get_num_elements(csp_handle h, uint32_t* n) {
    CSP_GUARD(h);
    if (!n) return fail(CSP_ERR_INVALID_ARGUMENT, "null output");
    *n = (uint32_t)reinterpret_cast<System*>(h)->elements.size();
    return CSP_OK;
}

int csp_get_elements(csp_handle h, csp_element* out, uint32_t cap) {
    CSP_GUARD(h);
    System* s = reinterpret_cast<System*>(h);
    if (!out || cap < s->elements.size()) return fail(CSP_ERR_INVALID_ARGUMENT, "output too small");
    std::copy(s->elements.begin(), s->elements.end(), out);
    return CSP_OK;
}

int csp_set_sun_vector(csp_handle h, double x, double y, double z) {
    CSP_GUARD(h);
    System* s = reinterpret_cast<System*>(h);
    s->sun_dir[0] = x;
    s->sun_dir[1] = y;
    s->sun_dir[2] = z;
    return CSP_OK;
}

int csp_set_sun_shape(csp_handle h, int shape, double param) {
    CSP_GUARD(h);
    if (!csp::valid_sun_shape(shape)) return fail(CSP_ERR_INVALID_ARGUMENT, "unknown sun shape");
    if (!(param >= 0.0) || param > 0.5) return fail(CSP_ERR_INVALID_ARGUMENT, "sun shape parameter out of range");
    System* s = reinterpret_cast<System*>(h);
    s->sun_shape = shape;
    s->sun_param = param;
    return CSP_OK;
}

int csp_set_seed(csp_handle h, uint64_t seed, uint32_t instance) {
    CSP_GUARD(h);
    System* s = reinterpret_cast<System*>(h);
    s->seed = seed;
    s->instance = instance;
    return CSP_OK;
}

int csp_set_accel(csp_handle h, int mode) {
    CSP_GUARD(h);
    if (mode != CSP_ACCEL_AUTO && mode != CSP_ACCEL_BVH && mode != CSP_ACCEL_GRID)
        return fail(CSP_ERR_INVALID_ARGUMENT, "unknown acceleration mode");
    System* s = reinterpret_cast<System*>(h);
    s->accel = mode;
    s->initialized = false;  // takes effect at the next initialize()
    return CSP_OK;
}

int csp_get_accel(csp_handle h, int* mode) {
    CSP_GUARD(h);
    if (!mode) return fail(CSP_ERR_INVALID_ARGUMENT, "null output");
    const System* s = reinterpret_cast<System*>(h);
    *mode = (s->elements.size() <= csp::kFlatListMax) ? CSP_ACCEL_LIST : (s->grid.valid ? CSP_ACCEL_GRID : CSP_ACCEL_BVH);
    return CSP_OK;
}

int csp_set_record_ids(csp_handle h, int enable) {
    CSP_GUARD(h);
    reinterpret_cast<System*>(h)->record_ids = enable != 0;
    return CSP_OK;
}

int csp_initialize(csp_handle h) {
    CSP_GUARD(h);
    return reinterpret_cast<System*>(h)->initialize();
}

int csp_run(csp_handle h) {
    CSP_GUARD(h);
    return reinterpret_cast<System*>(h)->run();
}

int csp_trace_async(csp_handle h, void* stream) {
    CSP_GUARD(h);
    return reinterpret_cast<System*>(h)->trace_async(reinterpret_cast<cudaStream_t>(stream));
}

int csp_update(csp_handle h) {
    CSP_GUARD(h);
    return reinterpret_cast<System*>(h)->update();
}

int csp_copy_hits(csp_handle h, float* dst, uint32_t* ids, uint64_t first, uint64_t count) {
    CSP_GUARD(h);
    System* s = reinterpret_cast<System*>(h);
    if (!s->initialized || !s->d_hits) return fail(CSP_ERR_STATE, "no hit buffer (initialize first)");
    if (first > s->num_rays || count > s->num_rays - first) return fail(CSP_ERR_INVALID_ARGUMENT, "ray range out of bounds");
    if (!dst && count) return fail(CSP_ERR_INVALID_ARGUMENT, "null destination");
    int rc = csp::cuda_status(cudaStreamSynchronize(s->stream), "sync");
    if (rc) return rc;
    if (count) {
        rc = csp::cuda_status(cudaMemcpy(dst, s->d_hits + first * csp::kMaxDepth, count * csp::kMaxDepth * sizeof(float4),
                                         cudaMemcpyDeviceToHost),
                              "D2H hit records");
        if (rc) return rc;
    }
    if (ids) {
        if (!s->record_ids || !s->d_ids) return fail(CSP_ERR_STATE, "element ids are not being recorded");
        if (count)
            return csp::cuda_status(cudaMemcpy(ids, s->d_ids + first * csp::kMaxDepth,
                                               count * csp::kMaxDepth * sizeof(uint32_t), cudaMemcpyDeviceToHost),
                                    "D2H ids");
    }
    return CSP_OK;
}

int csp_trace_into(csp_handle h, void* hits, void* ids, uint64_t first, uint64_t count, void* stream) {
    CSP_GUARD(h);
    System* s = reinterpret_cast<System*>(h);
    if (!s->initialized) return fail(CSP_ERR_STATE, "trace before initialize()");
    if (!hits && count) return fail(CSP_ERR_INVALID_ARGUMENT, "null hit buffer");
    if (!csp::valid_ray_window(first, count))
        return fail(CSP_ERR_INVALID_ARGUMENT, "ray window [first_ray, first_ray + count) must stay below 2^56");
    csp::TraceArgs a = s->args(0, 0);
    a.hits = reinterpret_cast<float4*>(hits);
    a.ids = reinterpret_cast<uint32_t*>(ids);
    a.ray_begin = first;
    a.count = count;
    cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : s->stream;
    if (st != s->stream) a.tile_counter = nullptr;  // may overlap the launches on the handle's stream
    return csp::cuda_status(csp::launch_trace(a, (int)s->scene.prims.size(), st), "trace_kernel");
}

int csp_run_to_host_compact(csp_handle h, float* points, uint8_t* counts, float* records, uint64_t capacity,
                            uint64_t* n_records) {
    CSP_GUARD(h);
    System* s = reinterpret_cast<System*>(h);
    if (s->num_rays && (!points || !counts)) return fail(CSP_ERR_INVALID_ARGUMENT, "null output");
    if (capacity && !records) return fail(CSP_ERR_INVALID_ARGUMENT, "null records with a capacity");
    return s->run_to_host_compact(points, counts, records, capacity, n_records);
}

int csp_run_to_host(csp_handle h, float* dst, uint32_t* ids) {
    CSP_GUARD(h);
    if (!dst) return fail(CSP_ERR_INVALID_ARGUMENT, "null destination");
    return reinterpret_cast<System*>(h)->run_to_host(dst, ids);
}

int csp_get_device_buffers(csp_handle h, void** hits, void** ids) {
    CSP_GUARD(h);
    System* s = reinterpret_cast<System*>(h);
    if (hits) *hits = s->d_hits;
    if (ids) *ids = s->record_ids ? s->d_ids : nullptr;
    return CSP_OK;
}

int csp_get_timing(csp_handle h, double* setup_s, double* trace_s) {
    CSP_GUARD(h);
    System* s = reinterpret_cast<System*>(h);
    if (setup_s) *setup_s = s->time_setup;
    if (trace_s) *trace_s = s->time_trace;
    return CSP_OK;
}

int csp_element_frame(const csp_element* e, double* euler, double* g2l, double* aabb_lo, double* aabb_hi) {
    if (!e) return fail(CSP_ERR_INVALID_ARGUMENT, "null element");
    double eu[3], G[9], lo[3], hi[3];
    csp::element_frame(*e, eu, G, lo, hi);
    if (euler) std::memcpy(euler, eu, sizeof eu);
    if (g2l) std::memcpy(g2l, G, sizeof G);
    if (aabb_lo) std::memcpy(aabb_lo, lo, sizeof lo);
    if (aabb_hi) std::memcpy(aabb_hi, hi, sizeof hi);
    return CSP_OK;
}

int csp_flux_map(csp_handle h, uint32_t nx, uint32_t ny, uint32_t* counts, double dni, double* flux) {
    CSP_GUARD(h);
    return reinterpret_cast<System*>(h)->flux_map(nx, ny, counts, dni, flux);
}

int csp_flux_map_ex(csp_handle h, uint32_t nx, uint32_t ny, int flags, uint32_t* counts, double dni, double* flux) {
    CSP_GUARD(h);
    if (flags & ~CSP_OUT_STAGED) return fail(CSP_ERR_INVALID_ARGUMENT, "unknown output flags");
    return reinterpret_cast<System*>(h)->flux_map(nx, ny, counts, dni, flux, (flags & CSP_OUT_STAGED) != 0);
}

int csp_flux_target(const csp_element* rcv, uint32_t nx, uint32_t ny, float* out) {
    if (!rcv || !out) return fail(CSP_ERR_INVALID_ARGUMENT, "null argument");
    if (nx == 0 || ny == 0) return fail(CSP_ERR_INVALID_ARGUMENT, "bad flux grid");
    csp::FluxTarget F;
    csp::flux_target(*rcv, nx, ny, F);
    const float v[20] = {F.o.x, F.o.y, F.o.z, F.x.x, F.x.y, F.x.z, F.y.x, F.y.y, F.y.z, F.z.x,
                         F.z.y, F.z.z, F.hx,  F.hy,  F.kx,  F.ky,  F.keep, (float)F.kind,
                         (float)csp::flux_bin_area(*rcv, nx, ny), 0.f};
    std::memcpy(out, v, sizeof(v));
    return CSP_OK;
}

int csp_get_sun_plane(csp_handle h, float* out) {
    CSP_GUARD(h);
    System* s = reinterpret_cast<System*>(h);
    if (!out) return fail(CSP_ERR_INVALID_ARGUMENT, "null output");
    if (!s->initialized) return fail(CSP_ERR_STATE, "initialize first");
    csp::SunFrame f;
    int rc = csp::cuda_status(cudaMemcpy(&f, s->d_sun, sizeof(f), cudaMemcpyDeviceToHost), "D2H sun frame");
    if (rc) return rc;
    const float v[16] = {f.s_d.x, f.s_d.y, f.s_d.z, f.v0.x, f.v0.y, f.v0.z, f.v1.x, f.v1.y,
                         f.v1.z,  f.v2.x,  f.v2.y,  f.v2.z, f.v3.x, f.v3.y, f.v3.z, f.s_d.w};
    std::memcpy(out, v, sizeof(v));
    return CSP_OK;
}

}  // extern "C"
