// csp_kernels.cuh -- launch interface of the CUDA kernels (host side).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "csp_types.cuh"

namespace csp {

// Bounds-check builds (-DCSP_BOUNDS_CHECK): the failed-check sites recorded on the current device by
// the kernels of each translation unit, read and cleared (0 in other builds).
#ifdef CSP_BOUNDS_CHECK
constexpr bool kBoundsCheckBuild = true;
#else
constexpr bool kBoundsCheckBuild = false;
#endif
uint32_t bounds_sites_trace();
uint32_t bounds_sites_batch();
uint32_t bounds_sites_sungrid();

// Every device and pinned-host allocation of the library goes through these (csp_c_api.cpp): the
// allocation-failure injection of csp_debug_fail_allocation lives there.
cudaError_t dev_alloc(void** p, size_t bytes);
cudaError_t host_alloc(void** p, size_t bytes);

// Closest-hit search of a launch: the element list in shared memory (<= 8 elements), the BVH, or
// the field grid (GridDesc).
enum Accel : int { kAccelFlat = 0, kAccelBvh = 1, kAccelGrid = 2 };

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
    const GridDesc* grid;  // field grid of the scene, nullptr: BVH (or element list) traversal
    const float* h3t12;    // Halton base-3 partial sums after 12 digits (halton3_table), or nullptr
    const SunGrid* sgrid;  // candidate grid of the sun rays (scenes of more than 8 elements)
    // single-scene launches: tiles handed out by this device counter (zeroed by launch_trace before
    // the kernel) in guided grabs; nullptr: static round robin (launches that may overlap on the
    // GPU with another of the same counter use that)
    unsigned long long* tile_counter;
};

// Arguments of the single-scene element-list kernel: TraceArgs plus the Philox key schedule of
// `seed` (philox_keys), read as kernel parameters.
struct TraceArgsK : TraceArgs {
    uint32_t keys[20];
};

// Device table of the base-3 Halton fold after its first 12 digits, t[m] = the reference loop's
// sum for m < 3^12 (2.1 MB, filled once per device by the same loop), or nullptr if it could not be
// made.  Thread-safe; the calling thread's current device.
const float* halton3_table();

// Sun-plane distance and parallelogram (lib/geometry_manager.cpp:97-148 with the reductions of
// lib/sun_utils.cu:53-179) plus the per-launch cone frame (cuda/sun.cu:76-79), one block.
cudaError_t launch_prepare_sun(const Aabb* aabbs, int n, float sx, float sy, float sz, float tan_pad, int shape,
                               float param, SunFrame* out, cudaStream_t stream);

// Sun-ray candidate grid of one scene state (SunGrid): device arrays of its build and where its
// descriptor goes.  All of it is written by launch_sungrid_build (nothing needs zeroing).
struct SunGridJob {
    SunGrid* desc;            // the descriptor the trace reads (TraceArgs::sgrid)
    const SunFrame* sun;      // sun frame of the state (prepare_sun output)
    const Aabb* aabbs;        // [n] exact boxes, lo.w = element | type << kTypeShift
    int n;
    int cap_cells;            // cell_start holds cap_cells + 1 entries, cursor cap_cells
    uint32_t cap_items;
    int pad;
    uint32_t* cell_start;
    uint32_t* cursor;
    float4* rect;             // [n]
    float4* item_rect;        // [cap_items]
    Aabb* item_box;           // [cap_items]
    uint32_t* global_id;      // [n]
};

// Capacities of the sun grid of an n-element scene and the device bytes of its arrays (each array
// 256-byte aligned, in the order of sungrid_place), descriptor included.
struct SunGridCaps {
    int cap_cells;
    uint32_t cap_items;
};
SunGridCaps sungrid_caps(uint32_t n);
size_t sungrid_bytes(uint32_t n);
// Carve the arrays of an n-element scene's sun grid out of `base` (sungrid_bytes(n) bytes, 256-byte
// aligned); fills every SunGridJob field except sun and aabbs.
void sungrid_place(unsigned char* base, uint32_t n, SunGridJob& job);

// Build the sun grids of n_jobs scene states (jobs: device array) on `stream`: reach rectangles and
// grid size, counts, prefix sums, fill.  max_n = the largest element count among the jobs.
cudaError_t launch_sungrid_build(const SunGridJob* jobs, int n_jobs, int max_n, cudaStream_t stream);

// Trace rays [ray_begin, ray_begin + count): generation, closest-hit search, shading, the dense
// hit-record write.  Scenes of up to 8 elements (n_prims) take the shared-memory element list path;
// larger ones need args.sgrid.
cudaError_t launch_trace(const TraceArgs& args, int n_prims, cudaStream_t stream);

// Compact form of a dense hit buffer of n rays (csp_run_to_host_compact): count pass -- per ray the
// number of records after slot 0 (uint8) and, in block_sums[compact_blocks(n) + 1], the exclusive
// offsets of the 256-ray blocks with the total at the end -- then the write pass: the sun-plane
// point of every ray (3 floats) and the records after slot 0, in ray order.
uint64_t compact_blocks(uint64_t n);
cudaError_t launch_compact_count(const float4* hits, uint64_t n, uint8_t* counts, unsigned long long* block_sums,
                                 cudaStream_t stream);
cudaError_t launch_compact_write(const float4* hits, uint64_t n, const unsigned long long* block_offsets, float* points,
                                 float4* records, cudaStream_t stream);

// Bin the stage-2 records of a dense hit buffer into F.counts and count records into F.stats[1..3]
// (both zeroed by the caller).
cudaError_t launch_flux_records(const float4* hits, uint64_t n_records, const FluxTarget& F, cudaStream_t stream);

// ---------------------------------------------------------------------- multi-instance launches --
// One instance = one scene state (its own prims, optics, node boxes, sun frame) traced for
// rays [args.ray_begin, args.ray_begin + args.count) with (args.seed, args.instance), its receiver
// records binned into flux.counts.  Instances of one launch are laid out as consecutive tile
// ranges; CTAs take chunks of tiles from a global counter.
struct alignas(16) InstanceDesc {
    TraceArgs args;       // hits = ids = nullptr; args.grid -> grid (grid instances)
    FluxTarget flux;
    GridDesc grid;
    uint64_t tile_begin;  // first tile of this instance in the launch
    int n_prims;
    int pad[3];
};

struct BatchLaunch {
    const InstanceDesc* inst;        // device
    const uint64_t* tile_begin;      // device, [n_inst + 1]; last entry = total_tiles
    int n_inst;
    int chunk;                       // tiles per grab
    uint64_t total_tiles;
    unsigned long long* next_tile;   // device work counter, zero before the launch
};

struct BatchTuning {
    int block;        // CTA size = tile size: 128 or 256
    int ctas_per_sm;  // resident CTAs per SM of the persistent grid (<= occupancy limit)
    int chunk;        // tiles taken per grab
};

// Bottom-up refit of one BVH topology into per-instance node arrays: leaves get the exact element
// AABB, internal nodes the union of the pruning boxes of the leaves below them.
struct RefitJob {
    const Node* topo;   // node links of the topology (boxes ignored)
    const Aabb* aabbs;  // exact element AABBs of the instance
    const Aabb* prune;  // pruning boxes of the instance
    Node* out;          // [n_nodes]
    int n_nodes;
    int pad;
};

struct SunJob {
    const Aabb* aabbs;
    int n;
    float sx, sy, sz, tan_pad;
    int shape;
    float param;
    SunFrame* out;
};

cudaError_t launch_refit(const RefitJob* jobs, int n_jobs, int max_nodes, cudaStream_t stream);
cudaError_t launch_prepare_sun_batch(const SunJob* jobs, int n_jobs, cudaStream_t stream);
// Closest-hit search of a batch group: 0 element list (<= 8 elements), 1 BVH, 2 field grid.
constexpr int kBatchGroups = 3;
// Occupancy limit of the multi-instance kernel for (accel, block); 0 if unsupported.
int batch_occupancy(int accel, int block);
// Fingerprint of the multi-instance kernels of a group as built (registers, shared and local memory
// of both block sizes): part of the autotuner cache key.
uint32_t batch_kernel_build(int accel);
cudaError_t launch_trace_batch(const BatchLaunch& L, int accel, const BatchTuning& t, cudaStream_t stream);

}  // namespace csp
