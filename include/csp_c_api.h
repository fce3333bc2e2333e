/*
 * csp_c_api.h -- C ABI of the GB300 concentrated-solar ray tracer (libcsp_gb300.so).
 *
 * Plain C types only (pointers, sizes, integers, doubles); no CUDA or PyTorch types cross it.  Every
 * call returns a csp_status (0 = OK); on failure csp_last_error() returns a thread-local message.
 * The C++ drop-in classes (SolTraceSystem, Element, ...) sit on top of this ABI and turn a non-zero
 * status into std::runtime_error, as the reference's CUDA_CHECK/OPTIX_CHECK do
 * (lib/util_check.hpp:54-63,93-104 of the reference).
 *
 * Reference interface each entry point replaces (paths inside uwsbel/optixSoltraceDemos):
 *   csp_create / csp_destroy      SolTraceSystem::SolTraceSystem(int)   lib/soltrace_system.cpp:49-70
 *                                 SolTraceSystem::clean_up()            lib/soltrace_system.cpp:267-297
 *   csp_set_num_rays              SolTraceSystem::set_sun_points(int)   lib/soltrace_system.h:49
 *   csp_add_element /
 *   csp_set_elements              SolTraceSystem::add_element(...)      lib/soltrace_system.cpp:427-433
 *                                 (+ Element setters, lib/element.h:41-102)
 *   csp_set_sun_vector            SolTraceSystem::set_sun_vector(...)   lib/soltrace_system.cpp:443-447
 *   csp_set_sun_shape             SolTraceSystem::set_sun_angle(double) lib/soltrace_system.h:57
 *   csp_initialize                SolTraceSystem::initialize()          lib/soltrace_system.cpp:76-143
 *   csp_run                       SolTraceSystem::run()                 lib/soltrace_system.cpp:145-170
 *   csp_update                    SolTraceSystem::update()              lib/soltrace_system.cpp:172-184
 *   csp_read_stinput              SolTraceSystem::read_st_input(...)    lib/soltrace_system.cpp:186-206
 *   csp_write_output              SolTraceSystem::write_output(...)     lib/soltrace_system.cpp:208-264
 *   csp_get_timing                get_time_trace / get_time_setup       lib/soltrace_system.cpp:435-441
 *   csp_get_sun_plane             print_launch_params                   lib/soltrace_system.cpp:24-47
 *   csp_copy_hits                 the hit_point_buffer D2H copy         lib/soltrace_system.cpp:209-211
 *   csp_flux_map                  FluxMapCalculator.calculate_flux_map  scripts/post_processing/
 *                                                                        flux_map_calculator.py:135-179
 * Additions with no single reference counterpart: csp_trace_async (enqueue on a caller stream),
 * csp_get_device_buffers (zero-copy consumers), csp_set_seed, csp_set_record_ids, csp_set_accel,
 * the flux map target, and the batch (csp_batch_*) and server (csp_server_*) interfaces.
 */
#ifndef CSP_C_API_H
#define CSP_C_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CSP_API __attribute__((visibility("default")))

/* Slots per ray in the hit buffer: MAX_TRACE_DEPTH of the reference (cuda/Soltrace.h:11). */
#define CSP_MAX_TRACE_DEPTH 5
#define CSP_ABI_VERSION 1
/* element id recorded for the sun-plane slot and for unused slots */
#define CSP_NO_ELEMENT 0xFFFFFFFFu

typedef struct csp_system* csp_handle;

typedef enum csp_status {
    CSP_OK = 0,
    CSP_ERR_INVALID_ARGUMENT = -1,
    CSP_ERR_CUDA = -2,
    CSP_ERR_OUT_OF_MEMORY = -3,
    CSP_ERR_BAD_SCENE = -4,
    CSP_ERR_TIMEOUT = -5,
    CSP_ERR_STATE = -6,
    CSP_ERR_IO = -7,
    CSP_ERR_PARSE = -8
} csp_status;

/* SurfaceType / ApertureType values of lib/soltrace_type.h:4-15 */
enum { CSP_SURFACE_FLAT = 0, CSP_SURFACE_PARABOLIC = 1, CSP_SURFACE_CYLINDER = 3 };
enum { CSP_APERTURE_RECTANGLE = 0, CSP_APERTURE_CIRCLE = 1 };
/* Sun shape of a trace: CSP_SUN_PILLBOX or CSP_SUN_GAUSSIAN, optionally OR-ed with the
 * CSP_SUN_ACCURATE flag (see csp_set_sun_shape). */
enum {
    CSP_SUN_PILLBOX = 0,
    CSP_SUN_GAUSSIAN = 1,
    CSP_SUN_ACCURATE = 2,
    CSP_SUN_PILLBOX_ACCURATE = CSP_SUN_PILLBOX | CSP_SUN_ACCURATE,
    CSP_SUN_GAUSSIAN_ACCURATE = CSP_SUN_GAUSSIAN | CSP_SUN_ACCURATE
};

/* One optical element, as the reference's Element holds it (lib/element.h:41-102): origin, aim
 * point, z rotation in degrees, rectangular aperture (for a cylinder: width = 2 * radius, height =
 * full height, axis along the element's local y, lib/element.cpp:146-160), parabolic curvatures.
 * reflectivity / slope_error / specularity_error (radians, Gaussian sigma) are optical properties the
 * reference parses but never applies; 1 / 0 / 0 reproduces the reference's trace exactly.
 * The last element of a scene is the receiver (lib/geometry_manager.cpp:78-90). */
typedef struct csp_element {
    double origin[3];
    double aim_point[3];
    double zrot_deg;
    double width;
    double height;
    double curv_x;
    double curv_y;
    double reflectivity;
    double slope_error;
    double specularity_error;
    int32_t surface;
    int32_t aperture;
} csp_element;

CSP_API const char* csp_last_error(void);
CSP_API int csp_abi_version(void);

/* Create a tracer bound to CUDA device `device`.  num_rays = number of sun points (rays). */
CSP_API int csp_create(csp_handle* out, int device, uint64_t num_rays);
/* Free every device buffer and the handle (clean_up + destructor). */
CSP_API int csp_destroy(csp_handle h);

CSP_API int csp_set_num_rays(csp_handle h, uint64_t num_rays);
CSP_API int csp_add_element(csp_handle h, const csp_element* element);
CSP_API int csp_set_elements(csp_handle h, const csp_element* elements, uint32_t count);
CSP_API int csp_get_num_elements(csp_handle h, uint32_t* count);
CSP_API int csp_get_elements(csp_handle h, csp_element* out, uint32_t capacity);
CSP_API int csp_set_sun_vector(csp_handle h, double x, double y, double z);
/* shape CSP_SUN_PILLBOX: param = half angle (rad), the reference's max_sun_angle, sampled with the
 *   reference's float formula z = cos(angle) + (1 - cos(angle)) r (cuda/sun.cu:82-86);
 * shape CSP_SUN_GAUSSIAN: param = sigma (rad) per tangent-plane axis (extension).
 * Flag CSP_SUN_ACCURATE (extension): the same scene, sun and random draws traced with two float
 * formulas of the reference replaced by cancellation-free ones -- the pillbox cone carries
 * 1 - z = (1 - cos(angle)) (1 - r) with 1 - cos(angle) = 2 sin^2(angle / 2) (the reference's float z
 * quantizes 1 - z in steps of 2^-24, ~2e-4 rad of direction error at 4.65 mrad), and the cylinder
 * receiver's side roots come from the ray's closest approach to its axis (the reference's
 * B^2 - 4AC cancels for rays that start hundreds of metres away, ~1 mm on the hit point).  Records
 * then differ from the reference's float trace by the rounding removed; flux maps agree with the
 * FP64 oracle to well under 1 %.  Without the flag the trace is the reference's, bit for bit. */
CSP_API int csp_set_sun_shape(csp_handle h, int shape, double param_rad);
/* Philox key of the random draws (seed) and the instance word of their counter. */
CSP_API int csp_set_seed(csp_handle h, uint64_t seed, uint32_t instance);
/* Also record the element index of every slot (uint32 per slot, CSP_NO_ELEMENT when empty). */
CSP_API int csp_set_record_ids(csp_handle h, int enable);
/* Closest-hit search structure for scenes of more than 8 elements (the reference leaves this to
 * OptiX's GAS): AUTO = a uniform grid over the heliostat layer when the mirrors lie in a thin
 * layer, else a BVH; BVH or GRID force one (GRID fails at initialize() for non-planar scenes).
 * Scenes of up to 8 elements always use the element list (CSP_ACCEL_LIST).  Results are the same
 * whichever structure is used.  Takes effect at the next csp_initialize. */
#define CSP_ACCEL_AUTO 0
#define CSP_ACCEL_BVH 1
#define CSP_ACCEL_GRID 2
#define CSP_ACCEL_LIST 3
CSP_API int csp_set_accel(csp_handle h, int mode);
/* The structure the last csp_initialize / csp_update chose. */
CSP_API int csp_get_accel(csp_handle h, int* mode);

/* Build device geometry, acceleration structure and sun plane; allocate the hit buffer. */
CSP_API int csp_initialize(csp_handle h);
/* Trace num_rays rays and wait for them (run()).  Fully rewrites the num_rays x 5 hit buffer. */
CSP_API int csp_run(csp_handle h);
/* Enqueue the trace on `stream` (a cudaStream_t, NULL = the handle's own stream); no host sync.
 * It writes the handle's hit buffer, so it must not overlap another run or trace of the handle on
 * the GPU (it also shares the handle's work counter with them). */
CSP_API int csp_trace_async(csp_handle h, void* stream);
/* Re-read the element poses given since initialize (same count), refit the acceleration structure
 * in place and recompute the sun plane (update()). */
CSP_API int csp_update(csp_handle h);

/* Copy hit records of rays [first_ray, first_ray + count) to host memory: dst holds count * 5 * 4
 * floats {stage, x, y, z}; ids (may be NULL) count * 5 uint32. */
CSP_API int csp_copy_hits(csp_handle h, float* dst, uint32_t* ids, uint64_t first_ray, uint64_t count);
/* Trace and copy every hit record to host memory in one call (run() + the D2H copy of
 * write_output), pipelining the copy of finished chunks behind the trace of later ones.  dst (and
 * ids when not NULL) should be page-locked for full speed. */
CSP_API int csp_run_to_host(csp_handle h, float* dst, uint32_t* ids);
/* Enqueue the trace of rays [first_ray, first_ray + count) on `stream` (NULL = the handle's own)
 * into caller-provided buffers of count * 5 records: device memory, or page-locked host memory
 * the device can address (the kernel then stores the records across the host link directly).
 * ids may be NULL.  No host synchronisation; the handle's own hit buffer is not touched, so windows
 * may be traced on several streams at once (off the handle's own stream the CTAs take tiles in a
 * fixed order instead of from the handle's work counter). */
CSP_API int csp_trace_into(csp_handle h, void* hits, void* ids, uint64_t first_ray, uint64_t count, void* stream);
/* Trace all rays, then move the records in compact form for consumers of the reference's
 * write_output (lib/soltrace_system.cpp:208-264), which need every record but not the empty slots:
 * points[3 num_rays] = each ray's sun-plane point (its stage-0 record), counts[num_rays] = the
 * number of its further records (0..4), records[4 capacity] = those records {stage, x, y, z} in ray
 * order -- instead of 80 bytes per ray.  *n_records = their number; when it exceeds `capacity`
 * (4 num_rays always suffices) nothing is copied and CSP_ERR_INVALID_ARGUMENT is returned.
 * csp_write_compact_csv writes the same CSV from them as csp_write_hits_csv from the dense
 * records. */
CSP_API int csp_run_to_host_compact(csp_handle h, float* points, uint8_t* counts, float* records, uint64_t capacity,
                                    uint64_t* n_records);
CSP_API int csp_write_compact_csv(const float* points, const uint8_t* counts, const float* records, uint64_t num_rays,
                                  const char* path, int flags);
/* One trace that allocates no memory (no counterpart in the reference).  For callers that cannot
 * call cudaMalloc -- a framework whose allocator already holds the device memory, a real-time
 * tracking loop that cannot take cudaMalloc's device-wide synchronisation: the caller passes the
 * elements (at most 8), the sun, and its own output buffers (hits: num_rays * 5 float4, ids: NULL
 * or num_rays * 5 uint32, device-addressable); rays [first_ray, first_ray + num_rays) are traced on
 * `stream` of `device`, bit-identical to csp_trace_into on a handle with the same scene.  The only
 * intermediate data live in a fixed 4 KB device array inside the library (held on every device that
 * uses it until the library is unloaded); every call overwrites it fully, and calls whose work
 * overlaps on the GPU (different streams or host threads) race on it.  The first call on a device
 * looks up that array's address; make it before any stream capture, and do not reset the device
 * after it (the address is kept for the life of the process).  More than 8 elements is
 * rejected with CSP_ERR_INVALID_ARGUMENT.  No host synchronisation. */
CSP_API int csp_trace_noalloc(int device, const csp_element* elements, uint32_t count, const double* sun_dir,
                              int sun_shape, double sun_param, uint64_t seed, uint32_t instance, uint64_t first_ray,
                              uint64_t num_rays, void* hits, void* ids, void* stream);
/* Device pointers of the hit buffer ([num_rays*5] float4) and id buffer (NULL unless recorded). */
CSP_API int csp_get_device_buffers(csp_handle h, void** hits, void** ids);

CSP_API int csp_get_timing(csp_handle h, double* setup_s, double* trace_s);

/* Host-only element geometry (no GPU): Euler angles (yaw, pitch, roll; rad), global-to-local
 * matrix (row-major, rows = the element's local x, y, z axes in world space) and exact double AABB,
 * as Element::update_euler_angles / get_rotation_matrix / compute_bounding_box compute them
 * (lib/element.cpp:77-93,97-103,172-275, lib/math_util.h:21-59).  Any output may be NULL. */
CSP_API int csp_element_frame(const csp_element* e, double* euler, double* g2l, double* aabb_lo, double* aabb_hi);

/* ---- SolTrace .stinput input and hit-record CSV output ---- */
/* Also apply each element's front optical surface (reflectivity, RMS slope / specularity error in
 * mrad) -- the reference parses and discards these values; without the flag so does this reader. */
#define CSP_STINPUT_APPLY_OPTICS 1
/* Parse a .stinput file on the host (no GPU).  With out == NULL only *count is set. */
CSP_API int csp_parse_stinput(const char* path, csp_element* out, uint32_t capacity, uint32_t* count,
                              double* sun_dir, double* sun_angle, int flags);
/* Append the file's elements to the handle and take its sun vector and angle (pillbox). */
CSP_API int csp_read_stinput(csp_handle h, const char* path, int flags);
/* Write num_rays x 5 hit records (host memory) as the reference's CSV (no GPU). */
CSP_API int csp_write_hits_csv(const float* hits, uint64_t num_rays, const char* path);
/* Copy the hit buffer to the host and write it as CSV (write_output). */
CSP_API int csp_write_output(csp_handle h, const char* path);
/* Staged results (SolTrace's stage order: the receiver sees only light from the mirrors): rays
 * whose first interaction is the receiver -- straight from the sun -- are left out.  The CSV then
 * equals the reference's file after scripts/post_processing/clean_direct_sun.py:6-18 (rows of
 * those rays dropped, the other rays keep their numbers); flux maps and batch flux maps do not
 * count their receiver records. */
#define CSP_OUT_STAGED 1
CSP_API int csp_write_hits_csv_ex(const float* hits, uint64_t num_rays, const char* path, int flags);
CSP_API int csp_write_output_ex(csp_handle h, const char* path, int flags);
/* out[16]: sun vector (3), v0 (3), v1 (3), v2 (3), v3 (3), plane distance (1). */
CSP_API int csp_get_sun_plane(csp_handle h, float* out);

/* ---- Receiver flux maps ---- */
/* Flux map of the last run on the receiver (last element), computed on the device from the hit
 * buffer: stage-2 records binned nx x ny as scripts/post_processing/flux_map_calculator.py:135-179
 * does (flat receiver: local x, y over the aperture; cylinder: angle about the axis in [0, 2 pi)
 * from the local x axis, and the axial coordinate; cylinder cap hits are dropped), bin (i, j) at
 * [i * ny + j].  counts (may be NULL) receives hit counts; flux (may be NULL) receives W/m^2 =
 * counts * dni * sun-plane area / rays / bin area. */
CSP_API int csp_flux_map(csp_handle h, uint32_t nx, uint32_t ny, uint32_t* counts, double dni, double* flux);
/* The same with flags (CSP_OUT_STAGED). */
CSP_API int csp_flux_map_ex(csp_handle h, uint32_t nx, uint32_t ny, int flags, uint32_t* counts, double dni,
                            double* flux);
/* Host-only (no GPU): the float binning parameters the device uses for a receiver element.
 * out[20]: origin (3), local x, y, z axes (9), hx, hy, kx, ky, keep, kind (0 flat, 1 cylinder),
 * bin area (m^2), 0.  A record at p lands in bx = floor((lx + hx) kx) (flat) or
 * floor(atan2(lz, lx) mod 2 pi * kx) (cylinder, |ly| < keep only), by = floor((ly + hy) ky). */
CSP_API int csp_flux_target(const csp_element* receiver, uint32_t nx, uint32_t ny, float* out);

/* ---- Batched tracing: many scene instances in one persistent launch ----
 * A batch holds scenes (element lists; a scene's BVH topology is built once) and instances (a
 * scene with optional per-instance element poses -- same count and surfaces, new origins, aim
 * points or rotations -- a sun vector and shape, a ray count, a seed and a Philox instance id).
 * csp_batch_run uploads the instances, refits each instance's BVH on the device, computes every
 * instance's sun plane and traces all instances in one persistent launch per scene class
 * (<= 8 elements / larger), binning receiver records into per-instance flux maps on the fly; no
 * per-ray records are kept.  The device work of a run is one CUDA graph, re-launched while the
 * batch layout (instances, element and ray counts) is unchanged.  Instance i's flux map equals
 * csp_flux_map of a plain run of the same scene, sun, rays, seed and instance id.
 * Replaces the reference's per-scene loop of set_sun_vector / update / run
 * (lib/soltrace_system.cpp:145-184, demos/demo_dynamic_scene.cpp:18-78) with one launch. */
typedef struct csp_batch_s* csp_batch;
CSP_API int csp_batch_create(csp_batch* out, int device);
CSP_API int csp_batch_destroy(csp_batch b);
/* Flux map grid of every instance (default 100 x 100), from the next run on. */
CSP_API int csp_batch_set_flux_grid(csp_batch b, uint32_t nx, uint32_t ny);
/* Output flags of the instances' flux maps (CSP_OUT_STAGED or 0, default 0), from the next run on. */
CSP_API int csp_batch_set_output(csp_batch b, int flags);
CSP_API int csp_batch_add_scene(csp_batch b, const csp_element* elements, uint32_t count, uint32_t* scene_id);
/* poses: NULL (the scene's own elements) or count elements matching the scene's surfaces. */
CSP_API int csp_batch_add_instance(csp_batch b, uint32_t scene_id, const csp_element* poses, const double* sun_dir,
                                   int sun_shape, double sun_param, uint64_t num_rays, uint64_t seed,
                                   uint32_t instance, uint32_t* index);
CSP_API int csp_batch_clear_instances(csp_batch b);
CSP_API int csp_batch_num_instances(csp_batch b, uint32_t* count);
/* Launch parameters: CTA/tile size (128 or 256 rays), resident CTAs per SM (0 = occupancy limit),
 * the most tiles one work grab takes (grabs shrink towards single tiles as the work runs out).
 * block = 0 selects the autotuner (default), which times tile sizes and CTAs per SM on a sample of
 * the batch at the first run of each scene class (grabs of at most 256 tiles) and keeps the fastest
 * per device. */
CSP_API int csp_batch_set_tuning(csp_batch b, int block, int ctas_per_sm, int chunk);
/* The parameters the last run used for one kernel group: CSP_ACCEL_LIST (<= 8 elements),
 * CSP_ACCEL_BVH or CSP_ACCEL_GRID instances (an instance whose poses move an origin or change a
 * size leaves its scene's grid for the BVH). */
CSP_API int csp_batch_get_tuning(csp_batch b, int group, int* block, int* ctas_per_sm, int* chunk);
CSP_API int csp_batch_run(csp_batch b);
/* Pipelined runs.  csp_batch_run_async builds the current instances on the host and queues their
 * device work behind the run in flight (at most two runs in flight, else CSP_ERR_STATE), so the
 * host work of one run overlaps the device work of the previous one; csp_batch_wait completes the
 * oldest run in flight and makes its results the current ones (CSP_ERR_STATE when none is in
 * flight).  csp_batch_run waits for every run in flight, then runs and waits.  Instances and the
 * flux grid may change while runs are in flight: each run keeps what its results need.  The
 * current results stay valid until the next csp_batch_run or csp_batch_run_async. */
CSP_API int csp_batch_run_async(csp_batch b);
CSP_API int csp_batch_wait(csp_batch b);
/* Results of the last completed run: counts / flux as csp_flux_map; stats[4] = rays, mirror
 * records, receiver records, binned receiver records. */
CSP_API int csp_batch_get_flux(csp_batch b, uint32_t index, uint32_t* counts, double dni, double* flux);
CSP_API int csp_batch_get_stats(csp_batch b, uint32_t index, uint64_t* stats);
/* out[16] as csp_get_sun_plane, for one instance. */
CSP_API int csp_batch_get_sun_plane(csp_batch b, uint32_t index, float* out);
/* setup_s: host element builds and upload; trace_s: device time of refit + sun planes + trace. */
CSP_API int csp_batch_get_timing(csp_batch b, double* setup_s, double* trace_s);
/* Bytes the last completed run copied host to device (the staging image: element records, grids,
 * launch descriptors) and device to host (flux maps, counters, sun frames). */
CSP_API int csp_batch_get_transfer(csp_batch b, uint64_t* h2d_bytes, uint64_t* d2h_bytes);

/* ---- Serving: a request loop with continuous batching ----
 * A server owns one worker thread, one CUDA stream and a device-memory arena of memory_budget
 * bytes (0 = half the free device memory, at most 8 GiB).  Scenes are added once and stay resident
 * (element records, BVH topology, field grid).  csp_server_submit (any thread, non-blocking)
 * queues a trace request: a scene, optional per-request poses (same count and surfaces: heliostat
 * tracking, refitted in place on the device), a sun, a ray count, seed and Philox instance id.
 * The worker admits requests as slots (max_active) and arena memory free up and traces every active
 * request's next slice of rays (step_rays across all active requests per step, 0 = 64M, but at
 * least 2^24 rays per request, or its remaining rays) in one persistent launch per kernel group,
 * so requests that arrive while others run share the GPU.
 * Each request's flux map is accumulated on the device and equals the batch / plain result for the
 * same inputs, alone or in any mix.  Replaces the reference's one-scene run() loop
 * (lib/soltrace_system.cpp:145-184) for many concurrent callers. */
typedef struct csp_server_s* csp_server;
CSP_API int csp_server_create(csp_server* out, int device, uint64_t memory_budget, uint32_t max_active,
                              uint64_t step_rays);
/* Finishes the admitted and queued requests, then stops the worker and frees everything. */
CSP_API int csp_server_destroy(csp_server s);
CSP_API int csp_server_add_scene(csp_server s, const csp_element* elements, uint32_t count, uint32_t* scene_id);
CSP_API int csp_server_submit(csp_server s, uint32_t scene_id, const csp_element* poses, const double* sun_dir,
                              int sun_shape, double sun_param, uint64_t num_rays, uint64_t seed, uint32_t instance,
                              uint64_t* request_id);
/* Output flags (CSP_OUT_STAGED or 0, default 0) of the requests submitted from now on. */
CSP_API int csp_server_set_output(csp_server s, int flags);
/* hold != 0: admit no further requests (they stay queued; active ones run to completion);
 * hold == 0: resume admission, admitting the queued requests together.  Destroying a held server
 * drops its queued requests. */
CSP_API int csp_server_hold(csp_server s, int hold);
/* Block until the request is done (timeout_s < 0: no limit; CSP_ERR_TIMEOUT otherwise), then hand
 * out its results and forget it: counts[100 * 100] (bin (i, j) at i * 100 + j, as csp_flux_map),
 * stats[4] (rays, mirror records, receiver records, binned records), latency_s[2] (submission to
 * completion, submission to admission); any output may be NULL. */
CSP_API int csp_server_wait(csp_server s, uint64_t request_id, double timeout_s, uint32_t* counts, uint64_t* stats,
                            double* latency_s);
/* out[8]: completed requests, rays traced, p50 and p99 latency (s) of the completed requests,
 * rays/s from the first submission to the last completion, peak active requests, peak arena bytes,
 * steps. */
CSP_API int csp_server_stats(csp_server s, double* out);

/* ---- Diagnostics and tuning (no counterpart in the reference, which stops the process on any
 * CUDA error, lib/util_check.hpp:54-63, and has no tunable launches) ----
 * Allocation-failure injection, for tests of the error paths: the device or pinned-host
 * allocation of this library that follows `after` further successful ones fails as if the device
 * were out of memory, once (the call that made it returns CSP_ERR_OUT_OF_MEMORY, or a served
 * request fails with it); -1 cancels.  Handles stay usable after such a failure. */
CSP_API int csp_debug_fail_allocation(int64_t after);
/* Persistent cache of the batched mode's autotuner: a JSON file of tuned launch parameters per
 * (device, kernel build, kernel group, ray-count class), read now (a missing file is an empty
 * cache) and rewritten after every autotuning.  NULL or "" keeps tunings in this process only, the
 * default unless the environment variable CSP_TUNE_CACHE names a file.  csp_tune_cache_entries: the
 * tunings known now. */
CSP_API int csp_set_tune_cache(const char* path);
CSP_API int csp_tune_cache_entries(uint32_t* entries);
/* Builds with -DCSP_BOUNDS_CHECK check the queue, record-row, flux-bin and grid indices of every
 * launch against their buffers and skip the access that fails: `sites` receives the mask of the
 * checks that failed on the device since the last call (0 = none) and clears it.  CSP_ERR_STATE in
 * a build without the checks. */
CSP_API int csp_bounds_check_status(int device, uint32_t* sites);

#ifdef __cplusplus
}
#endif
#endif /* CSP_C_API_H */
