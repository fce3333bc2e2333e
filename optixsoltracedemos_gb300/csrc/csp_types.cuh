// csp_types.cuh -- device data layout shared by the host scene builder and the CUDA kernels.
//
// Layout in HBM (all arrays 16-byte aligned, read through the read-only path):
//   Prim   [n]      64 B  geometry of one element in the form its intersection test consumes
//   Optics [n]      16 B  reflectivity, slope error, specularity error (extension)
//   Aabb   [n]      32 B  element AABB exactly as the reference hands it to OptiX (float)
//   Node   [m]      32 B  stackless BVH node: box + hit link + miss link
//   SunFrame        sun-plane parallelogram and cone frame, written on device by the prepare kernel
//   hits   [N*5]    80 B/ray  float4 {stage, x, y, z}, the reference's hit_point_buffer
//   ids    [N*5]    20 B/ray  uint32 element index per slot (optional)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace csp {

// OpticalEntityType of the reference (cuda/Soltrace.h:24-30).
enum EntityType : uint32_t { kFlatMirror = 0, kParabolicMirror = 1, kFlatReceiver = 2, kCylReceiver = 3 };

constexpr int kMaxDepth = 5;               // MAX_TRACE_DEPTH (cuda/Soltrace.h:11)
constexpr float kTminSun = 0.001f;         // cuda/sun.cu:123
constexpr float kTminBounce = 0.01f;       // cuda/materials.cu:76
constexpr float kTmax = 1e16f;             // cuda/sun.cu:124
constexpr uint32_t kLeafFlag = 0x80000000u;
constexpr uint32_t kTypeShift = 28;
constexpr uint32_t kPrimMask = 0x0FFFFFFFu;
constexpr uint32_t kNoElement = 0xFFFFFFFFu;
// Every ray index of a trace lies below 2^56: the BVH and grid kernels queue a ray with the bounce
// depth of its pending hit in the top 8 bits of its 64-bit index.  The host entry points reject
// ray windows that reach past it before any launch.
constexpr uint64_t kRayIndexLimit = 1ull << 56;

// Prim field layout by entity type (all values float, computed on the host with the same float
// operations the reference's intersection programs perform per call, so hoisting them is exact):
//  flat mirror / flat receiver (Rectangle_Flat, cuda/GeometryDataST.h:41-58):
//    a = (plane normal n, plane w)   b = (center, width/2)   c = (x axis, height/2)   d = (y axis, 0)
//  parabolic mirror (Rectangle_Parabolic, cuda/GeometryDataST.h:79-103, cuda/intersection.cu:335-352):
//    a = (e1, L1/2)   b = (e2, L2/2)   c = (n = normalize(e2 x e1), curv_x)   d = (rect center, curv_y)
//  cylinder receiver (Cylinder_Y, cuda/GeometryDataST.h:60-77, cuda/intersection.cu:188-194):
//    a = (center, radius)   b = (local x, half height)   c = (local y = z x x, radius^2)   d = (local z, 0)
struct alignas(16) Prim {
    float4 a, b, c, d;
};

struct alignas(16) Optics {
    float reflectivity, slope, spec, pad;
};

struct alignas(16) Aabb {
    float4 lo;  // xyz, w unused
    float4 hi;
};

// Stackless BVH node.  lo.w / hi.w carry int32 links (bit patterns):
//   internal: hit = index of the first child, visited when the box is entered; miss = next node
//             in traversal order once this subtree is done (-1 = end).
//   leaf:     hit = kLeafFlag | type << kTypeShift | element index; miss as above.
// Internal boxes bound every surface below them (sag-inflated for paraboloids); a leaf box is the
// element's exact AABB, the box whose overlap decides whether the element is tested at all.
struct alignas(16) Node {
    float4 lo;
    float4 hi;
};

struct alignas(16) SunFrame {
    float4 s_d;    // normalized sun vector, plane distance d
    float4 v0;     // parallelogram corner
    float4 e1;     // v1 - v0
    float4 e2;     // v3 - v0
    float4 v1, v2, v3;
    float4 w;      // cone axis = -sun
    float4 u, v;   // cone frame
    float cos_theta, sigma, tan_pad;
    float omc;     // 1 - cos_theta as 2 sin^2(half angle / 2) (shape 2, the accurate cone sampler)
    int shape, n_prims, pad1, pad2;
};

// Uniform 2D grid over a planar heliostat field (the alternative to the BVH for field-like
// scenes), built for one set of poses.  Cells of size `cell` cover [x0, x1] x [y0, y1]; the items of
// cell (ix, iy) are items[cell_start[iy * nx + ix] .. cell_start[iy * nx + ix + 1]), one per element
// whose pruning box (widened by a margin) overlaps the cell in xy: the element's exact AABB with
// lo.w = element | type << 28 (bits).  Rays walk the cells their xy path crosses inside the layer
// [zlo, zhi], which holds every gridded surface; the global items (the receiver, oversized
// elements) are tested by every ray.  Every candidate passes the exact AABB test before its
// intersection program runs.
struct alignas(16) GridDesc {
    float x0, y0, x1, y1;
    float cell, inv_cell, zlo, zhi;
    int nx, ny, n_global, pad;
    const uint32_t* cell_start;
    const Aabb* items;
    const Aabb* global;
    const void* reserved;
};

// Candidate grid of the sun rays of one scene state and sun frame (scenes of more than 8
// elements), built on the device after the sun plane.  Every element has a reach rectangle in the
// Halton coordinates (u, v) of the sun plane, outside which no sun ray can meet its AABB (rect[e],
// see reach_rect in csp_trace.cuh).  [0, 1]^2 is cut into nu x nv cells; cell (iu, iv) lists
// (items[cell_start[iv nu + iu] .. cell_start[iv nu + iu + 1])) every element whose rectangle overlaps
// it, with the rectangle (item_rect) and the element's exact box (item_box, lo.w = element | type
// << kTypeShift) inline, so that a candidate's box test does not wait for an index.  Elements whose
// rectangle covers more than kSunGridMaxCells cells are in the global list instead, tested by every
// ray.  A sun ray at (u, v) can only meet the elements of its cell and the global list whose
// rectangles hold (u, v); a ray that lies in none meets no element box at all.
constexpr int kSunGridMaxCells = 64;     // cells of one element's rectangle before it goes global
constexpr int kSunGridItemsPerElem = 12;  // item capacity per element (the sizing keeps the total below)
struct alignas(16) SunGrid {
    int nu, nv, n_global, n;
    float fnu, fnv, pad0, pad1;
    const uint32_t* cell_start;  // [nu nv + 1]
    const float4* item_rect;
    const Aabb* item_box;
    const uint32_t* global_id;   // [n_global]
    const float4* rect;          // [n], every element's reach rectangle
    const Aabb* aabbs;           // exact element boxes, lo.w = element | type << kTypeShift (bits)
};

// Receiver flux map target (scripts/post_processing/flux_map_calculator.py:135-179 binning, in
// float).  A receiver (stage-2) record at world point p has local coordinates t = p - o,
// (lx, ly, lz) = (t.x_axis, t.y_axis, t.z_axis) and lands in bin (bx, by), counts[bx * ny + by]:
//   flat      bx = floor((lx + hx) kx), by = floor((ly + hy) ky), kx = nx / w, ky = ny / h
//   cylinder  a = atan2(lz, lx) in [0, 2 pi), bx = floor(a kx), kx = nx / (2 pi); by as above;
//             only side hits (|ly| < keep) are binned, cap hits are dropped
// both indices clamped to the grid.
enum FluxKind : int { kFluxFlat = 0, kFluxCylinder = 1 };

struct alignas(16) FluxTarget {
    float4 o, x, y, z;          // receiver origin and local axes (xyz; w unused)
    float hx, hy, kx, ky;
    float keep;
    int kind, nx, ny;
    uint32_t* counts;           // [nx * ny]
    unsigned long long* stats;  // [4]: rays, mirror records, receiver records, binned records
    // staged results (SolTrace's stage order: the receiver only sees light from the mirrors): a
    // receiver record in slot 1, i.e. straight from the sun, is dropped with its ray
    // (scripts/post_processing/clean_direct_sun.py:6-18)
    int staged;
};

// Halton base-3 digit weights: f_k = fl(f_{k-1} / 3), f_0 = 1 (the float sequence cuda/sun.cu:19
// produces), k = 1..41 enough for 64-bit indices.
#ifdef __CUDACC__
__constant__ const float c_halton3_f[41] = {
    0x1.5555560000000p-2f,
    0x1.c71c720000000p-4f,
    0x1.2f684c0000000p-5f,
    0x1.948b100000000p-7f,
    0x1.0db20a0000000p-8f,
    0x1.67980e0000000p-10f,
    0x1.df75680000000p-12f,
    0x1.3fa39a0000000p-13f,
    0x1.aa2f780000000p-15f,
    0x1.1c1fa60000000p-16f,
    0x1.7ad4de0000000p-18f,
    0x1.f91bd20000000p-20f,
    0x1.50bd360000000p-21f,
    0x1.c0fc480000000p-23f,
    0x1.2b52da0000000p-24f,
    0x1.8f19220000000p-26f,
    0x1.0a10c20000000p-27f,
    0x1.62c1020000000p-29f,
    0x1.d901580000000p-31f,
    0x1.3b563a0000000p-32f,
    0x1.a472f80000000p-34f,
    0x1.184ca60000000p-35f,
    0x1.75bb880000000p-37f,
    0x1.f24f600000000p-39f,
    0x1.4c34ea0000000p-40f,
    0x1.baf1380000000p-42f,
    0x1.274b7a0000000p-43f,
    0x1.89b9f80000000p-45f,
    0x1.067bfa0000000p-46f,
    0x1.5dfaa20000000p-48f,
    0x1.d2a3820000000p-50f,
    0x1.3717ac0000000p-51f,
    0x1.9eca3a0000000p-53f,
    0x1.1486d20000000p-54f,
    0x1.70b3c20000000p-56f,
    0x1.eb9a580000000p-58f,
    0x1.47bc3a0000000p-59f,
    0x1.b4faf80000000p-61f,
    0x1.2351fa0000000p-62f,
    0x1.846d4e0000000p-64f,
    0x1.02f38a0000000p-65f
};
#endif

}  // namespace csp
