// csp_trace.cuh -- device side of the trace path, shared by the single-scene kernel
// (csp_kernels.cu) and the multi-instance kernel (csp_batch.cu).
//
// Everything here is compiled with -fmad=false and IEEE division/sqrt: expressions round exactly as
// written, which keeps records bit-identical to the host restatement of the reference.
//
// Reference counterparts (paths inside the reference project):
//   generate            ray generation, cuda/sun.cu:16-38 (Halton point), :72-91,106 (cone)
//   hit_flat/parab/cyl  intersection programs, cuda/intersection.cu:47-85, 318-448, 177-296
//   traverse            OptiX traversal: closest hit among the elements whose AABB the ray overlaps
//   classify/shade      closest-hit programs, cuda/materials.cu:26-231; miss program :236-253
//
// Wavefront inside each CTA (kB threads, one tile = kB consecutive rays of one instance):
//   phase A (one ray per thread, every ray): sun sample and the cheap, branch-free part of the first
//     segment.  Rays with more to do are pushed into a shared-memory queue (warp ballot + one shared
//     atomic per warp):
//       small scenes (kFlat, <= kFlatMax elements, all in shared memory): phase A only runs the AABB
//         slab tests; rays whose segment overlaps some element box are queued with that mask;
//       BVH and grid scenes: phase A finds and records the first hit; mirror hits are queued
//         unshaded.
//   phase B (only on full batches of kB queued rays, and on the remainder at the end): the rest of
//     each queued path -- intersection programs, shading, further segments.
// In the heliostat workloads ~10% of rays meet an element; running their intersection programs and
// shading on full warps instead of inside warps where ~90% of lanes have finished is the point.
//
// Output sinks (compile-time):
//   kDense  the reference's hit_point_buffer: 5 float4 records per ray (+ optional element ids).
//           Phase A stages the warp's records in shared memory and writes them as coalesced rows;
//           phase B writes its records straight to global memory (their rows were written by phase A
//           of an earlier tile of this CTA, ordered by the barriers in between).
//   kFlux   receiver records are binned into the instance's flux map in the shading stage (global
//           reductions), with per-instance record counters; nothing per ray leaves the SM.
#pragma once

#include <cfloat>
#include <type_traits>

#include "csp_kernels.cuh"
#include "csp_math.cuh"

namespace csp {
namespace {

// Index checks of the bounds-check build (-DCSP_BOUNDS_CHECK): CSP_BOUNDS(site, cond) is cond, and a
// false cond sets bit `site` of this translation unit's device word (the caller skips the access);
// read and cleared by the host through csp_bounds_check_status.  Sites: 0 bounce-queue append,
// 1 generation-queue append, 2 record row, 3 flux bin, 4 field-grid cell, 5 sun-grid cell and item
// range, 6 sun-grid build, 7 Halton table.  In other builds CSP_BOUNDS(site, cond) is true and cond is
// not evaluated.
#ifdef CSP_BOUNDS_CHECK
__device__ unsigned int g_bounds_sites;
__device__ __forceinline__ bool bounds_ok(int site, bool ok) {
    if (!ok) atomicOr(&g_bounds_sites, 1u << site);
    return ok;
}
#define CSP_BOUNDS(site, cond) bounds_ok((site), (cond))
// Host: the sites this translation unit's kernels recorded on the current device, cleared.
inline uint32_t take_bounds_sites() {
    unsigned int v = 0, z = 0;
    if (cudaMemcpyFromSymbol(&v, g_bounds_sites, sizeof v) != cudaSuccess ||
        cudaMemcpyToSymbol(g_bounds_sites, &z, sizeof z) != cudaSuccess) {
        cudaGetLastError();
        return 0x80000000u;  // unreadable: reported as a failed check
    }
    return v;
}
#else
#define CSP_BOUNDS(site, cond) true
inline uint32_t take_bounds_sites() { return 0; }
#endif

constexpr float kTwoPi = 2.0f * 3.14159265358979323846f;  // 2.0f * M_PIf, cuda/sun.cu:85
constexpr float kTwoPiF = 0x1.921fb6p+2f;                  // fl32(2 pi), flux angle wrap
constexpr int kFlatMax = 8;
constexpr uint32_t kH3TabDigits = 6, kH3Tab = 729;

template <int kB, bool kFlat>
struct CoreSmem;
template <int kB>
struct FlatStageSmem;

template <int kB_, int kAccel_, bool kDense_, bool kFlux_>
struct Cfg {
    static constexpr int kB = kB_;        // CTA size = tile size (rays)
    static constexpr int kAccel = kAccel_;
    static constexpr bool kFlat = kAccel_ == kAccelFlat;
    static constexpr bool kDense = kDense_;
    static constexpr bool kFlux = kFlux_;
    // grid and BVH launches give each warp 32 rays whose sun-plane points are close together
    static constexpr bool kCoherent = kAccel_ != kAccelFlat;
    // Philox from the precomputed key schedule: the single-scene element-list kernel only (the field
    // kernels would lose a resident CTA to the extra registers, the batch kernel reads its
    // arguments from shared memory)
    static constexpr bool kSched = kAccel_ == kAccelFlat && kDense_;
    using Args = std::conditional_t<kSched, TraceArgsK, TraceArgs>;
    // every launch defers the direction of the sun rays whose sun-plane point may reach an element
    // box to full batches (the generation queue); the other rays provably miss.  Element-list
    // launches test the reach rectangles of their elements, the others the sun grid (SunGrid).
    using Core = CoreSmem<kB_, kFlat>;
    // phase A record staging of dense element-list launches
    using Stage = FlatStageSmem<kB_>;
};

// Coherent ray order: position kk of a launch of `count` rays -> ray offset.  Rays come in blocks
// of 32 S; in a block, the warp at position m takes offsets m + j S (lane j).  The Halton
// coordinates of offsets that differ by a multiple of S = 2^a 3^b differ by less than 2^-a in u
// (base 2) and 3^-b in v (base 3), so a warp's rays start within a small patch of the sun plane and
// walk the same grid cells.  Whole blocks of S = 2^8 3^5 first, then of S = 2^7 3^4 over the rest,
// then the identity order for the tail: a bijection on [0, count).  kFine puts whole blocks of
// S = 2^9 3^6 (11,943,936 rays) before them: launches without dense records gain from the smaller
// patches, while in dense launches a warp's 32 rows would then span ~1 GB of the hit buffer, which
// measured slower.  With G > 1 groups of G consecutive warps (of one tile, i.e. CTA) take
// neighbouring patches: warp k of group t in a block gets m = k S / G + t, and offsets that differ
// by S / G = 2^(a-log2 G) 3^b have u coordinates 2^-a apart -- a strip of G adjacent patches whose
// grid cells the group's warps share in L1.
constexpr uint64_t kCoherentS0 = 512u * 729u, kCoherentB0 = 32u * kCoherentS0;
constexpr uint64_t kCoherentS1 = 256u * 243u, kCoherentB1 = 32u * kCoherentS1;
constexpr uint64_t kCoherentS2 = 128u * 81u, kCoherentB2 = 32u * kCoherentS2;

// warp position m in a block of S warps for the warp at index r >> 5 of the block (G | S)
template <int G, class U>
__device__ __forceinline__ U coherent_warp(U r, U S) {
    const U w = r >> 5;
    if constexpr (G == 1) return w;
    else return (w % G) * (S / G) + w / G;
}

template <bool kFine, int G, class U>
__device__ __forceinline__ U coherent_order_t(U kk, U count) {
    static_assert(G == 1 || G == 2 || G == 4 || G == 8 || G == 16, "warp groups must divide every S");
    constexpr U B0 = (U)kCoherentB0, S0 = (U)kCoherentS0, B1 = (U)kCoherentB1, S1 = (U)kCoherentS1;
    constexpr U B2 = (U)kCoherentB2, S2 = (U)kCoherentS2;
    U full0 = 0;
    if constexpr (kFine) {
        full0 = (count / B0) * B0;
        if (kk < full0) {
            const U blk = kk / B0, r = kk - blk * B0;
            return blk * B0 + (U)coherent_warp<G>(r, S0) + (r & 31u) * S0;
        }
    }
    const U k1 = kk - full0, c1 = count - full0;
    const U full1 = (c1 / B1) * B1;
    if (k1 < full1) {
        const U blk = k1 / B1, r = k1 - blk * B1;
        return full0 + blk * B1 + (U)coherent_warp<G>(r, S1) + (r & 31u) * S1;
    }
    const U k2 = k1 - full1;
    const U full2 = ((c1 - full1) / B2) * B2;
    if (k2 < full2) {
        const U blk = k2 / B2, r = k2 - blk * B2;
        return full0 + full1 + blk * B2 + (U)coherent_warp<G>(r, S2) + (r & 31u) * S2;
    }
    return kk;
}

// Launches of fewer than 2^32 rays (all but the largest) take the 32-bit form: the same
// arithmetic, without the cost of 64-bit division by the block sizes.
template <bool kFine, int G>
__device__ __forceinline__ uint64_t coherent_order(uint64_t kk, uint64_t count) {
    if (count <= 0xFFFFFFFFull) return coherent_order_t<kFine, G, uint32_t>((uint32_t)kk, (uint32_t)count);
    return coherent_order_t<kFine, G, uint64_t>(kk, count);
}

// ------------------------------------------------------------------------------ sun plane -----
__device__ __forceinline__ float3 corner(const Aabb& b, int k) {
    return make_float3((k & 1) ? b.hi.x : b.lo.x, (k & 2) ? b.hi.y : b.lo.y, (k & 4) ? b.hi.z : b.lo.z);
}

template <bool kMax>
__device__ float block_reduce(float v, float* scratch) {
    for (int o = 16; o > 0; o >>= 1) {
        const float w = __shfl_xor_sync(0xffffffffu, v, o);
        v = kMax ? fmaxf(v, w) : fminf(v, w);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    v = scratch[0];
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) v = kMax ? fmaxf(v, scratch[i]) : fminf(v, scratch[i]);
    return v;
}

// One block computes the sun frame of one scene: plane distance, u/v bounds, parallelogram
// (lib/sun_utils.cu:53-179, lib/geometry_manager.cpp:97-148) and cone frame (cuda/sun.cu:76-79).
// `scratch` holds blockDim.x / 32 floats.
__device__ void sun_frame_block(const Aabb* __restrict__ aabbs, int n, float3 s, float tan_pad, int shape,
                                float param, SunFrame* __restrict__ out, float* scratch) {
    // plane distance: max over every AABB corner of |c . s| (and 0), lib/sun_utils.cu:53-104
    float md = 0.0f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const Aabb b = aabbs[i];
        for (int k = 0; k < 8; ++k) md = fmaxf(md, fabsf(dot(corner(b, k), s)));
    }
    const float d = block_reduce<true>(md, scratch);

    const float3 axis = (fabsf(s.x) < 0.9f) ? f3(1.0f, 0.0f, 0.0f) : f3(0.0f, 1.0f, 0.0f);
    const float3 su = normalize(cross(axis, s));
    const float3 sv = normalize(cross(s, su));
    const float3 pc = scale(d, s);
    // u/v bounds padded by |c . s| tan(angle), lib/sun_utils.cu:106-179
    float umin = FLT_MAX, umax = -FLT_MAX, vmin = FLT_MAX, vmax = -FLT_MAX;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const Aabb b = aabbs[i];
        for (int k = 0; k < 8; ++k) {
            const float3 pt = corner(b, k);
            const float buf = fabsf(dot(pt, s)) * tan_pad;
            const float3 proj = sub(pt, scale(dot(sub(pt, pc), s), s));
            const float u = dot(proj, su), v = dot(proj, sv);
            umin = fminf(umin, u - buf);
            umax = fmaxf(umax, u + buf);
            vmin = fminf(vmin, v - buf);
            vmax = fmaxf(vmax, v + buf);
        }
    }
    umin = block_reduce<false>(umin, scratch);
    umax = block_reduce<true>(umax, scratch);
    vmin = block_reduce<false>(vmin, scratch);
    vmax = block_reduce<true>(vmax, scratch);
    if (threadIdx.x != 0) return;
    const float3 ds = scale(d, s);
    const float3 v0 = add(add(scale(umin, su), scale(vmin, sv)), ds);
    const float3 v1 = add(add(scale(umax, su), scale(vmin, sv)), ds);
    const float3 v2 = add(add(scale(umax, su), scale(vmax, sv)), ds);
    const float3 v3 = add(add(scale(umin, su), scale(vmax, sv)), ds);
    // cone frame, cuda/sun.cu:76-79 with dir = -normalize(sun_vector) (cuda/sun.cu:106)
    const float3 w = normalize(neg(normalize(s)));
    const float3 cu = normalize(cross(fabsf(w.x) > 0.99f ? f3(0.0f, 1.0f, 0.0f) : f3(1.0f, 0.0f, 0.0f), w));
    const float3 cv = cross(w, cu);
    SunFrame f;
    f.s_d = make_float4(s.x, s.y, s.z, d);
    f.v0 = make_float4(v0.x, v0.y, v0.z, 0.f);
    const float3 e1 = sub(v1, v0), e2 = sub(v3, v0);
    f.e1 = make_float4(e1.x, e1.y, e1.z, 0.f);
    f.e2 = make_float4(e2.x, e2.y, e2.z, 0.f);
    f.v1 = make_float4(v1.x, v1.y, v1.z, 0.f);
    f.v2 = make_float4(v2.x, v2.y, v2.z, 0.f);
    f.v3 = make_float4(v3.x, v3.y, v3.z, 0.f);
    f.w = make_float4(w.x, w.y, w.z, 0.f);
    f.u = make_float4(cu.x, cu.y, cu.z, 0.f);
    f.v = make_float4(cv.x, cv.y, cv.z, 0.f);
    f.omc = 0.0f;
    if (shape & 1) {
        f.cos_theta = 1.0f;
        f.sigma = param;
    } else if (shape & 2) {
        // accurate cone sampler: 1 - cos(half_angle) = 2 sin^2(half_angle / 2), free of the
        // cancellation of 1 - cosf(half_angle)
        float sn, cs;
        det_sincos(param * 0.5f, sn, cs);
        f.omc = (sn + sn) * sn;
        f.cos_theta = 1.0f - f.omc;
        f.sigma = 0.0f;
    } else {
        float sn, cs;
        det_sincos(param, sn, cs);  // cosf(half_angle), cuda/sun.cu:82
        f.cos_theta = cs;
        f.sigma = 0.0f;
    }
    f.tan_pad = tan_pad;
    f.shape = shape;
    f.n_prims = n;
    f.pad1 = f.pad2 = 0;
    *out = f;
}

// ------------------------------------------------------------------------------ sampling ------
// Halton radical inverse, cuda/sun.cu:16-24: f /= b; r += f * (i mod b); i /= b, in float.
// The loop's partial sum after its first 24 digits (the low 24 bits of i) is a dyadic fraction of
// at most 24 bits, so every step so far was exact and the sum equals the bit-reversed low bits
// scaled by 2^-32; the loop then goes on from that state (f = 2^-24) over the remaining digits.
__device__ __forceinline__ float halton2(uint64_t i) {
    float r = (float)__brev((uint32_t)i & 0xFFFFFFu) * 0x1p-32f;
    i >>= 24;
    float f = 0x1p-24f;
    while (i > 0) {
        f = f * 0.5f;  // f / 2 is exact
        r = r + f * (float)(uint32_t)(i & 1u);
        i >>= 1;
    }
    return r;
}

__device__ __forceinline__ float halton3(uint64_t i) {
    float r = 0.0f;
    int k = 0;
    while (i >= (1ull << 32)) {
        const uint64_t q = i / 3u;
        r = r + c_halton3_f[k++] * (float)(uint32_t)(i - 3u * q);
        i = q;
    }
    uint32_t j = (uint32_t)i;
    while (j > 0) {
        const uint32_t q = j / 3u;
        r = r + c_halton3_f[k++] * (float)(j - 3u * q);
        j = q;
    }
    return r;
}

// Same fold with its first steps looked up: t6[m] = halton3(m) for m < 3^6 (shared memory) or
// t12[m] = halton3(m) for m < 3^12 (global table, when present).  The partial sum of the reference
// loop after k digits depends only on i mod 3^k and equals halton3(i mod 3^k) (a zero digit adds +0,
// which leaves the sum unchanged); for larger i the loop continues from exactly that sum with digit
// k + 1, so the result is identical bit for bit.
constexpr uint32_t kH3T12Digits = 12, kH3T12 = 531441;
__device__ __forceinline__ float halton3_tab(uint64_t i, const float* __restrict__ t6, const float* __restrict__ t12) {
    if (i >= (1ull << 32)) return halton3(i);
    uint32_t j = (uint32_t)i;
    float r;
    int k;
    if (t12) {
        const uint32_t q = j / kH3T12;
        if (!CSP_BOUNDS(7, j - kH3T12 * q < kH3T12)) return 0.0f;
        r = __ldg(t12 + (j - kH3T12 * q));
        k = kH3T12Digits;
        j = q;
    } else {
        const uint32_t q = j / kH3Tab;
        r = t6[j - kH3Tab * q];
        k = kH3TabDigits;
        j = q;
    }
    while (j > 0) {
        const uint32_t q = j / 3u;
        r = r + c_halton3_f[k++] * (float)(j - 3u * q);
        j = q;
    }
    return r;
}

__device__ __forceinline__ float3 perturb(float3 n, float sigma, float g1, float g2) {
    const float3 t1 = normalize(cross(fabsf(n.x) > 0.9f ? f3(0.0f, 1.0f, 0.0f) : f3(1.0f, 0.0f, 0.0f), n));
    const float3 t2 = cross(n, t1);
    return normalize(add(add(n, scale(sigma * g1, t1)), scale(sigma * g2, t2)));
}

// ------------------------------------------------------------------------------ intersection --
// Rectangle_Flat, cuda/intersection.cu:47-85.
__device__ __forceinline__ bool hit_flat(const Prim& p, float3 o, float3 d, float tmin, float& tout) {
    const float3 n = xyz(p.a);
    const float dt = dot(d, n);
    const float t = (p.a.w - dot(n, o)) / dt;
    if (!(t > tmin && t < kTmax)) return false;
    const float3 v = sub(add(o, scale(t, d)), xyz(p.b));
    const float x = dot(xyz(p.c), v), y = dot(xyz(p.d), v);
    const float hw = p.b.w, hh = p.c.w;
    if (x >= -hw && x <= hw && y >= -hh && y <= hh) {
        tout = t;
        return true;
    }
    return false;
}

// Rectangle_Parabolic, cuda/intersection.cu:318-419.  The reference's bounds test
// a = x_hit / (L/2.) evaluated in double then rounded to float, |a| <= 1, is decided here as
// |x_hit| <= L/2 in float: for floats x, h > 0, fl32(fl64(x/h)) > 1 exactly when x > h (if x > h
// then x >= succ(h), so x/h >= 1 + 2^-24 + 2^-48 and both roundings stay above 1; if x <= h the
// quotient is <= 1), and symmetrically for -1; NaN passes both forms.
__device__ __forceinline__ bool hit_parab(const Prim& p, float3 o, float3 d, float tmin, float& tout) {
    const float3 e1 = xyz(p.a), e2 = xyz(p.b), n = xyz(p.c), c = xyz(p.d);
    const float cx = p.c.w, cy = p.d.w;
    const float3 dd = sub(o, c);
    const float ox = dot(dd, e1), oy = dot(dd, e2), oz = dot(dd, n);
    const float dx = dot(d, e1), dy = dot(d, e2), dz = dot(d, n);
    const float A = (cx * 0.5f) * (dx * dx) + (cy * 0.5f) * (dy * dy);
    const float B = cx * (ox * dx) + cy * (oy * dy) - dz;
    const float C = (cx * 0.5f) * (ox * ox) + (cy * 0.5f) * (oy * oy) - oz;
    float t = 0.0f;
    bool valid = false;
    if (fabsf(A) < 1e-12f) {
        t = -C / B;
        valid = (t > 0.0f);
    } else {
        const float disc = B * B - 4.0f * A * C;
        if (disc >= 0.0f) {
            const float sq = sqrtf(disc);
            const float t1 = (-B - sq) / (2.0f * A);
            const float t2 = (-B + sq) / (2.0f * A);
            if (t1 > 0.0f && t1 < t2) {
                t = t1;
                valid = true;
            } else if (t2 > 0.0f) {
                t = t2;
                valid = true;
            }
        }
    }
    if (!valid || t < tmin || t > kTmax) return false;
    const float xh = ox + t * dx, yh = oy + t * dy;
    const float h1 = p.a.w, h2 = p.b.w;
    if (xh > h1 || xh < -h1 || yh > h2 || yh < -h2) return false;
    tout = t;
    return true;
}

// World normal the parabolic intersection program reports for a hit at t (cuda/intersection.cu:
// 354-361 local coordinates again, then :430-436).
__device__ __forceinline__ float3 parab_normal(const Prim& p, float3 o, float3 d, float t) {
    const float3 e1 = xyz(p.a), e2 = xyz(p.b), n = xyz(p.c);
    const float3 dd = sub(o, xyz(p.d));
    const float ox = dot(dd, e1), oy = dot(dd, e2);
    const float dx = dot(d, e1), dy = dot(d, e2);
    const float xh = ox + t * dx, yh = oy + t * dy;
    const float3 nl = normalize(f3(-p.c.w * xh, -p.d.w * yh, 1.0f));
    return normalize(add(add(scale(nl.x, e1), scale(nl.y, e2)), scale(nl.z, n)));
}

// Cylinder_Y with caps, cuda/intersection.cu:177-296.  `accurate` (extension, the CSP_SUN_ACCURATE
// trace flag): the side roots from the ray's closest approach to the axis, tm = -(Ox Dx + Oz Dz) / A,
// and the half chord sqrt((r^2 - |Q|^2) / A) with Q = O + tm D in the (x, z) plane, instead of
// B^2 - 4AC, which cancels to ~1e-4 relative when the ray starts hundreds of metres from the
// receiver (about 1 mm on the hit point in float).
__device__ __forceinline__ bool hit_cyl(const Prim& p, float3 o, float3 draw, float tmin, bool accurate, float& tout) {
    const float3 d = normalize(draw);
    const float3 lo = sub(o, xyz(p.a));
    const float3 lx = xyz(p.b), ly = xyz(p.c), lz = xyz(p.d);
    const float Ox = dot(lo, lx), Oy = dot(lo, ly), Oz = dot(lo, lz);
    const float Dx = dot(d, lx), Dy = dot(d, ly), Dz = dot(d, lz);
    const float half = p.b.w, r2 = p.c.w;
    const float A = Dx * Dx + Dz * Dz;
    const float inval = kTmax + 1.0f;
    float tc = inval;
    float t1 = 0.0f, t2 = 0.0f;
    bool side = false;
    if (accurate) {
        if (A > 0.0f) {
            const float tm = -(Ox * Dx + Oz * Dz) / A;
            const float qx = Ox + tm * Dx, qz = Oz + tm * Dz;
            const float h2 = r2 - (qx * qx + qz * qz);
            if (h2 >= 0.0f) {
                const float hh = sqrtf(h2 / A);
                t1 = tm - hh;
                t2 = tm + hh;
                side = true;
            }
        }
    } else {
        const float B = 2.0f * (Ox * Dx + Oz * Dz);
        const float C = Ox * Ox + Oz * Oz - r2;
        const float det = B * B - 4.0f * A * C;
        if (det >= 0.0f) {
            const float sq = sqrtf(det);
            t1 = (-B - sq) / (2.0f * A);
            t2 = (-B + sq) / (2.0f * A);
            side = true;
        }
    }
    if (side) {
        if (t1 > tmin && t1 < kTmax && fabsf(Oy + t1 * Dy) <= half) tc = t1;
        else if (t2 > tmin && t2 < kTmax && fabsf(Oy + t2 * Dy) <= half) tc = t2;
    }
    float tcap = inval;
    if (fabsf(Dy) > 1e-6f) {
        const float tb = (-half - Oy) / Dy;
        const float bx = Ox + tb * Dx, bz = Oz + tb * Dz;
        if (tb > tmin && tb < kTmax && bx * bx + bz * bz <= r2) tcap = tb;
        const float tt = (half - Oy) / Dy;
        const float tx = Ox + tt * Dx, tz = Oz + tt * Dz;
        if (tt > tmin && tt < kTmax && tx * tx + tz * tz <= r2) tcap = fminf(tcap, tt);
    }
    const float t = fminf(tc, tcap);
    if (t >= kTmax || t <= tmin) return false;
    tout = t;
    return true;
}

// `acc`: the accurate arithmetic trace flag (bit 1 of the sun shape).
__device__ __forceinline__ bool hit_prim(uint32_t type, const Prim& p, float3 o, float3 d, float tmin, bool acc,
                                         float& t) {
    if (type == kParabolicMirror) return hit_parab(p, o, d, tmin, t);
    if (type == kCylReceiver) return hit_cyl(p, o, d, tmin, acc, t);
    return hit_flat(p, o, d, tmin, t);
}

__device__ __forceinline__ Prim load_prim(const Prim* prims, uint32_t i) {
    const float4* q = reinterpret_cast<const float4*>(prims + i);
    Prim p;
    p.a = __ldg(q);
    p.b = __ldg(q + 1);
    p.c = __ldg(q + 2);
    p.d = __ldg(q + 3);
    return p;
}

// Closest hit among the elements whose AABB the segment [tmin, kTmax] overlaps; equal t keeps the
// lower element index.  Internal nodes are pruned against the closest hit so far with slack
// (their boxes bound every surface below them with a margin); leaves test the exact AABB.
__device__ __forceinline__ int traverse(const Node* __restrict__ nodes, const Prim* __restrict__ prims, float3 o,
                                        float3 d, float tmin, bool acc, float& best_t, uint32_t& best_type) {
    const float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    int best = -1;
    best_t = __int_as_float(0x7f800000);
    float prune = kTmax;
    int node = 0;
    while (node >= 0) {
        const float4* q = reinterpret_cast<const float4*>(nodes + node);
        const float4 lo = __ldg(q), hi = __ldg(q + 1);
        const float t0x = (lo.x - o.x) * inv.x, t1x = (hi.x - o.x) * inv.x;
        const float t0y = (lo.y - o.y) * inv.y, t1y = (hi.y - o.y) * inv.y;
        const float t0z = (lo.z - o.z) * inv.z, t1z = (hi.z - o.z) * inv.z;
        const float tn = fmaxf(tmin, fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z)));
        const float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
        const uint32_t hitw = __float_as_uint(lo.w);
        const int miss = __float_as_int(hi.w);
        if (hitw & kLeafFlag) {
            if (tn <= fminf(kTmax, tf)) {
                const uint32_t prim = hitw & kPrimMask;
                const uint32_t type = (hitw >> kTypeShift) & 7u;
                float t;
                if (hit_prim(type, load_prim(prims, prim), o, d, tmin, acc, t) &&
                    (t < best_t || (t == best_t && (int)prim < best))) {
                    best = (int)prim;
                    best_t = t;
                    best_type = type;
                    prune = fminf(kTmax, best_t + best_t * 1e-3f + 1e-3f);
                }
            }
            node = miss;
        } else {
            node = (tn <= fminf(prune, tf)) ? (int)hitw : miss;
        }
    }
    return best;
}

__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// Exact-AABB culling and intersection program of one grid candidate (a BVH leaf's work): the
// element's exact AABB lo, hi with lo.w = element | type << 28.
__device__ __forceinline__ void test_box(float4 lo, float4 hi, const Prim* __restrict__ prims, float3 o, float3 d,
                                         float3 inv, float tmin, bool acc, int& best, float& best_t,
                                         uint32_t& best_type, float& prune) {
    const float t0x = (lo.x - o.x) * inv.x, t1x = (hi.x - o.x) * inv.x;
    const float t0y = (lo.y - o.y) * inv.y, t1y = (hi.y - o.y) * inv.y;
    const float t0z = (lo.z - o.z) * inv.z, t1z = (hi.z - o.z) * inv.z;
    const float tn = fmaxf(tmin, fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z)));
    const float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    if (!(tn <= fminf(kTmax, tf))) return;
    const uint32_t w = __float_as_uint(lo.w);
    const uint32_t prim = w & kPrimMask;
    const uint32_t type = (w >> kTypeShift) & 7u;
    float t;
    if (hit_prim(type, load_prim(prims, prim), o, d, tmin, acc, t) &&
        (t < best_t || (t == best_t && (int)prim < best))) {
        best = (int)prim;
        best_t = t;
        best_type = type;
        prune = fminf(kTmax, best_t + best_t * 1e-3f + 1e-3f);
    }
}

// Restrict [ta, tb] to the parameters where coordinate o + t d lies in [lo, hi] (an empty range
// stays empty).
__device__ __forceinline__ void clip_axis(float o, float d, float inv, float lo, float hi, float& ta, float& tb) {
    if (d == 0.0f) {
        if (!(o >= lo && o <= hi)) {
            ta = 1.0f;
            tb = 0.0f;
        }
        return;
    }
    const float t0 = (lo - o) * inv, t1 = (hi - o) * inv;
    ta = fmaxf(ta, fminf(t0, t1));
    tb = fminf(tb, fmaxf(t0, t1));
}

// Closest hit through the field grid: the global elements, then the cells of the xy path inside
// the layer in ray order (2D DDA), each cell's candidates through test_box, until a cell is
// entered beyond the pruning distance.  The result equals traverse()'s: every element whose
// surface holds a hit point at t is registered in the cell the walk assigns to that point (the
// registered boxes exceed the surfaces by a margin far above the walk's rounding), that cell is
// entered at or before t, and the walk only stops beyond best_t + best_t 1e-3 + 1e-3.
__device__ __forceinline__ int traverse_grid(const GridDesc& G, const Prim* __restrict__ prims, float3 o, float3 d,
                                             float tmin, bool acc, float& best_t, uint32_t& best_type) {
    const float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    int best = -1;
    best_t = __int_as_float(0x7f800000);
    float prune = kTmax;
    float ta = tmin, tb = kTmax;
    clip_axis(o.z, d.z, inv.z, G.zlo, G.zhi, ta, tb);
    clip_axis(o.x, d.x, inv.x, G.x0, G.x1, ta, tb);
    clip_axis(o.y, d.y, inv.y, G.y0, G.y1, ta, tb);
    const bool walk = ta <= tb;
    const float px = o.x + ta * d.x, py = o.y + ta * d.y;
    int ix = (int)fminf(fmaxf(floorf((px - G.x0) * G.inv_cell), 0.0f), (float)(G.nx - 1));
    int iy = (int)fminf(fmaxf(floorf((py - G.y0) * G.inv_cell), 0.0f), (float)(G.ny - 1));
    const int sx = d.x > 0.0f ? 1 : -1, sy = d.y > 0.0f ? 1 : -1;
    const float inf = __int_as_float(0x7f800000);
    // candidate lists in order: the global elements, then the cells of the walk (one test site).
    // (ix, iy) is the next cell of the walk, entered at ctc: it does not depend on the tests, so its
    // item range is prefetched into L1 before the current list is tested; it is entered only if
    // ctc lies within the segment and the pruning distance the tests leave.
    const Aabb* list = G.global;
    uint32_t j = 0, e = (uint32_t)G.n_global;
    bool next = walk;
    float ctc = ta;
    if (next) prefetch_l1(G.cell_start + (iy * G.nx + ix));
    int step = 0;
    for (;;) {
        for (; j < e; ++j) {
            const float4* q = reinterpret_cast<const float4*>(list + j);
            test_box(__ldg(q), __ldg(q + 1), prims, o, d, inv, tmin, acc, best, best_t, best_type, prune);
        }
        if (!next || ctc > tb || ctc > prune || step > G.nx + G.ny) break;
        const int c = iy * G.nx + ix;
        if (!CSP_BOUNDS(4, c >= 0 && c < G.nx * G.ny)) break;
        list = G.items;
        j = __ldg(G.cell_start + c);
        e = __ldg(G.cell_start + c + 1);
        ++step;
        // the cell after it: parameters of the next x and y cell boundaries, from the cell index
        const float tnx = (d.x != 0.0f) ? (G.x0 + (float)(ix + (sx > 0)) * G.cell - o.x) * inv.x : inf;
        const float tny = (d.y != 0.0f) ? (G.y0 + (float)(iy + (sy > 0)) * G.cell - o.y) * inv.y : inf;
        if (tnx < tny) {
            ctc = fmaxf(ctc, tnx);
            ix += sx;
            next = ix >= 0 && ix < G.nx;
        } else {
            ctc = fmaxf(ctc, tny);
            iy += sy;
            next = iy >= 0 && iy < G.ny;
        }
        if (next) prefetch_l1(G.cell_start + (iy * G.nx + ix));
    }
    return best;
}

// ------------------------------------------------------------------------------ sun grid ------
// Cell index of a Halton coordinate x in [0, 1] along an axis of n cells (f = n as a float).  The
// build registers a rectangle [lo, hi] in cells sg_cell(max(lo, 0)) .. sg_cell(min(hi, 1)); float
// multiplication and truncation are monotonic, so a point x with lo <= x <= hi lies in one of them.
__device__ __forceinline__ int sg_cell(float x, float f, int n) { return min((int)(x * f), n - 1); }

__device__ __forceinline__ bool in_rect(float4 r, float u, float v) {
    return (u >= r.x) & (u <= r.y) & (v >= r.z) & (v <= r.w);
}

// Whether some element's reach rectangle holds the sun-plane point (u, v): only then can the ray
// meet an element box (otherwise its record is the sun-plane point alone).
__device__ __forceinline__ bool sun_reach_any(const SunGrid& G, float u, float v) {
    const int c = sg_cell(v, G.fnv, G.nv) * G.nu + sg_cell(u, G.fnu, G.nu);
    if (!CSP_BOUNDS(5, c >= 0 && c < G.nu * G.nv)) return true;
    uint32_t j = __ldg(G.cell_start + c);
    const uint32_t e = __ldg(G.cell_start + c + 1);
    if (!CSP_BOUNDS(5, j <= e && e <= __ldg(G.cell_start + G.nu * G.nv))) return true;
    for (; j < e; ++j)
        if (in_rect(__ldg(G.item_rect + j), u, v)) return true;
    for (int k = 0; k < G.n_global; ++k)
        if (in_rect(__ldg(G.rect + __ldg(G.global_id + k)), u, v)) return true;
    return false;
}

// Closest hit of the sun ray leaving the plane at (u, v) = o with direction d: the elements of its
// cell and of the global list whose reach rectangles hold (u, v), each through the exact AABB test
// and its intersection program (test_box).  Every element whose box the ray meets is among them,
// so this is the closest hit over all elements (equal t keeps the lower element index).
__device__ __forceinline__ int sun_closest(const SunGrid& G, const Prim* __restrict__ prims, float u, float v,
                                           float3 o, float3 d, bool acc, float& best_t, uint32_t& best_type) {
    const float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    int best = -1;
    best_t = __int_as_float(0x7f800000);
    float prune = kTmax;
    const int c = sg_cell(v, G.fnv, G.nv) * G.nu + sg_cell(u, G.fnu, G.nu);
    if (!CSP_BOUNDS(5, c >= 0 && c < G.nu * G.nv)) return best;
    uint32_t j = __ldg(G.cell_start + c);
    const uint32_t e = __ldg(G.cell_start + c + 1);
    if (!CSP_BOUNDS(5, j <= e && e <= __ldg(G.cell_start + G.nu * G.nv))) return best;
    for (; j < e; ++j) {
        if (!in_rect(__ldg(G.item_rect + j), u, v)) continue;
        const float4* q = reinterpret_cast<const float4*>(G.item_box + j);
        test_box(__ldg(q), __ldg(q + 1), prims, o, d, inv, kTminSun, acc, best, best_t, best_type, prune);
    }
    for (int k = 0; k < G.n_global; ++k) {
        const uint32_t id = __ldg(G.global_id + k);
        if (!in_rect(__ldg(G.rect + id), u, v)) continue;
        const float4* q = reinterpret_cast<const float4*>(G.aabbs + id);
        test_box(__ldg(q), __ldg(q + 1), prims, o, d, inv, kTminSun, acc, best, best_t, best_type, prune);
    }
    return best;
}

// ------------------------------------------------------------------------------ flux bins -----
// Bin of a receiver record at world point p, or -1 for a cylinder cap hit (see FluxTarget).
__device__ __forceinline__ int flux_bin(const FluxTarget& F, float3 p) {
    const float3 t = sub(p, xyz(F.o));
    const float lx = dot(t, xyz(F.x)), ly = dot(t, xyz(F.y));
    float u;
    if (F.kind == kFluxCylinder) {
        if (!(fabsf(ly) < F.keep)) return -1;
        const float lz = dot(t, xyz(F.z));
        float a = det_atan2(lz, lx);
        if (a < 0.0f) a = a + kTwoPiF;
        u = a * F.kx;
    } else {
        u = (lx + F.hx) * F.kx;
    }
    const float v = (ly + F.hy) * F.ky;
    const int bx = (int)fminf(fmaxf(floorf(u), 0.0f), (float)(F.nx - 1));
    const int by = (int)fminf(fmaxf(floorf(v), 0.0f), (float)(F.ny - 1));
    return bx * F.ny + by;
}

// ------------------------------------------------------------------------------ trace ---------
struct Segment {
    float3 o, d;
    float tmin;
    int depth;
};

// Scene copy in shared memory for kFlat launches.
struct FlatScene {
    Prim prim[kFlatMax];
    Aabb box[kFlatMax];
    Optics optics[kFlatMax];
    uint32_t type[kFlatMax];
    int n;
};

// AABB culling of the intersection programs (segment [tmin, kTmax] against each element box) for a
// kFlat scene: bit k set when element k's program has to run.
__device__ __forceinline__ uint32_t candidates(const FlatScene& fs, float3 o, float3 d, float tmin) {
    const float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    uint32_t mask = 0;
    const int nb = fs.n;
#pragma unroll
    for (int k = 0; k < kFlatMax; ++k) {
        if (k >= nb) break;
        const float4 lo = fs.box[k].lo, hi = fs.box[k].hi;
        const float t0x = (lo.x - o.x) * inv.x, t1x = (hi.x - o.x) * inv.x;
        const float t0y = (lo.y - o.y) * inv.y, t1y = (hi.y - o.y) * inv.y;
        const float t0z = (lo.z - o.z) * inv.z, t1z = (hi.z - o.z) * inv.z;
        const float tn = fmaxf(tmin, fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z)));
        const float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
        if (tn <= fminf(kTmax, tf)) mask |= 1u << k;
    }
    return mask;
}

// Closest hit among the candidate elements, in ascending index (equal t keeps the lower index).
__device__ __forceinline__ int closest_in(const FlatScene& fs, uint32_t mask, float3 o, float3 d, float tmin,
                                          bool acc, float& best_t, uint32_t& best_type) {
    int best = -1;
    best_t = __int_as_float(0x7f800000);
    while (mask) {
        const int k = __ffs(mask) - 1;
        mask &= mask - 1u;
        float t;
        if (hit_prim(fs.type[k], fs.prim[k], o, d, tmin, acc, t) && t < best_t) {
            best = k;
            best_t = t;
            best_type = fs.type[k];
        }
    }
    return best;
}

struct Hit {
    int best;  // element index, -1 on a miss
    float t;
    uint32_t type;
};

// What the closest-hit program of a hit records: slot depth+1 (mirrors and the cylinder always,
// below max depth; the flat receiver only from the front, cuda/materials.cu:86-163), and whether a
// mirror has to be shaded next (cuda/materials.cu:44-60,180-197: only below max depth).
__device__ __forceinline__ bool classify(const Prim& p, const Segment& g, const Hit& h, float4& rec, int& slot) {
    slot = -1;
    const int nd = g.depth + 1;
    if (nd >= kMaxDepth) return false;
    const float3 hit = add(g.o, scale(h.t, g.d));
    if (h.type == kFlatMirror || h.type == kParabolicMirror) {
        rec = make_float4(1.0f, hit.x, hit.y, hit.z);
        slot = nd;
        return true;
    }
    if (h.type == kFlatReceiver) {
        const float3 rn = cross(xyz(p.c), xyz(p.d));
        if (!(dot(g.d, rn) < 0.0f)) return false;
    }
    rec = make_float4(2.0f, hit.x, hit.y, hit.z);
    slot = nd;
    return false;
}

// __closesthit__mirror / __closesthit__mirror__parabolic (cuda/materials.cu:26-84,170-231): normal
// as the intersection program reports it, faced against the ray, ideal reflection; plus the
// extensions (Gaussian slope and specularity error, absorption with probability 1 - reflectivity).
// Returns false when the ray is absorbed.
// C::kSched: draws use the precomputed key schedule A.keys (kernel parameters, free operands in the
// single-scene element-list kernel); otherwise the schedule is derived from A.seed per draw.
template <class C>
__device__ __forceinline__ u32x4 draw(const typename C::Args& A, uint64_t ray, uint32_t bounce,
                                      uint32_t draw_index) {
    if constexpr (C::kSched) return draw_block_sched(ray, bounce, draw_index, A.instance, A.keys);
    else return draw_block(ray, bounce, draw_index, A.instance, A.seed);
}

template <class C>
__device__ __forceinline__ bool shade_mirror(const typename C::Args& A, uint64_t ray, const Prim& p, const Optics& op,
                                             const Segment& g, const Hit& h, Segment& next) {
    const int nd = g.depth + 1;
    const float3 hit = add(g.o, scale(h.t, g.d));
    const float3 wn = (h.type == kFlatMirror) ? normalize(xyz(p.a)) : normalize(parab_normal(p, g.o, g.d, h.t));
    float3 ffn = (dot(neg(g.d), wn) >= 0.0f) ? wn : neg(wn);
    const bool need_rng = (op.slope > 0.0f) || (op.spec > 0.0f) || !(op.reflectivity >= 1.0f);
    u32x4 ra = {0u, 0u, 0u, 0u};
    if (need_rng) ra = draw<C>(A, ray, (uint32_t)nd, 0);
    if (op.slope > 0.0f) {
        float g1, g2;
        box_muller(u01(ra.y), u01(ra.z), g1, g2);
        ffn = perturb(ffn, op.slope, g1, g2);
    }
    float3 rd = reflect(g.d, ffn);
    if (op.spec > 0.0f) {
        const u32x4 rb = draw<C>(A, ray, (uint32_t)nd, 1);
        float g1, g2;
        box_muller(u01(rb.x), u01(rb.y), g1, g2);
        rd = perturb(normalize(rd), op.spec, g1, g2);
    }
    if (need_rng && u01(ra.x) > op.reflectivity) return false;  // absorbed at the mirror
    next = Segment{hit, rd, kTminBounce, nd};
    return true;
}

// Ray generation: cuda/sun.cu:28-38 (Halton point on the sun parallelogram) and :72-91, :106
// (direction in the sun cone; Gaussian sun as an extension).
__device__ __forceinline__ float3 sun_point(const SunFrame& S, float hu, float hv) {
    return add(add(xyz(S.v0), scale(hu, xyz(S.e1))), scale(hv, xyz(S.e2)));
}

template <class C>
__device__ __forceinline__ float3 sun_direction(const typename C::Args& A, const SunFrame& S, uint64_t ray) {
    const u32x4 r0 = draw<C>(A, ray, 0, 0);
    const float3 w = xyz(S.w), cu = xyz(S.u), cv = xyz(S.v);
    float3 dir;
    if (S.shape & 1) {
        float g1, g2;
        box_muller(u01(r0.x), u01(r0.y), g1, g2);
        dir = normalize(add(add(w, scale(S.sigma * g1, cu)), scale(S.sigma * g2, cv)));
    } else if (S.shape & 2) {
        // the reference's uniform z in [cos(half_angle), 1] (cuda/sun.cu:82-86) carried as
        // 1 - z = (1 - cos(half_angle)) (1 - rand2), so that the cone radius
        // sqrt(1 - z^2) = sqrt((1 - z)(2 - (1 - z))) keeps full relative precision (the float z of
        // the reference formula quantizes 1 - z in steps of 2^-24)
        const float rand1 = u01(r0.x), rand2 = u01(r0.y);
        const float phi = kTwoPi * rand1;
        const float omz = S.omc * (1.0f - rand2);
        const float z = 1.0f - omz;
        const float r = sqrtf(omz * (2.0f - omz));
        float sp, cp;
        det_sincos(phi, sp, cp);
        dir = normalize(add(scale(r, add(scale(cp, cu), scale(sp, cv))), scale(z, w)));
    } else {
        const float rand1 = u01(r0.x), rand2 = u01(r0.y);
        const float phi = kTwoPi * rand1;
        const float z = S.cos_theta + (1.0f - S.cos_theta) * rand2;
        const float r = sqrtf(1.0f - z * z);
        float sp, cp;
        det_sincos(phi, sp, cp);
        dir = normalize(add(scale(r, add(scale(cp, cu), scale(sp, cv))), scale(z, w)));
    }
    return dir;
}

// Reach rectangle of one element box: Halton coordinates (u in [x, y], v in [z, w]) outside which
// no sun ray can meet the box.  A ray leaves the sun plane at o = v0 + u e1 + v e2 with a direction
// at most a from the cone axis w; at depth h below the plane it has moved at most h tan a across
// it, and every point of the box lies at depth <= H (its deepest corner).  So o projects within
// H tan a of the box's projection; in Halton units that is the corners' range of
// ((c - v0).e1 / |e1|^2, (c - v0).e2 / |e2|^2) widened by H tan a / |e1|, H tan a / |e2|.
// tan a: pillbox tan(half angle) (the accurate sampler: from 1 - cos directly); Gaussian sigma |(g1, g2)| with |(g1, g2)| <= sqrt(-2 ln 2^-24)
// = 5.77 (the smallest uniform is 2^-24).  Margins: 1 % on tan a, 1e-4 of the scene's extent plus
// 1 mm on the distance, 1e-5 in Halton units, far above the float rounding of the ray's origin,
// direction and box test, so a ray outside every rectangle fails the exact box test of every
// element.  Degenerate frames give the whole plane.
__device__ __forceinline__ float4 reach_rect(const SunFrame& S, float4 lo, float4 hi) {
    const float3 v0 = xyz(S.v0), e1 = xyz(S.e1), e2 = xyz(S.e2), w = xyz(S.w);
    const float l1 = dot(e1, e1), l2 = dot(e2, e2);
    float tan_a;
    if (S.shape & 1) {
        tan_a = 5.8f * S.sigma;
    } else if (S.shape & 2) {
        const float c = S.cos_theta;
        tan_a = c > 0.2f ? sqrtf(S.omc * (2.0f - S.omc)) / c : __int_as_float(0x7f800000);
    } else {
        const float c = S.cos_theta;
        tan_a = c > 0.2f ? sqrtf(fmaxf(0.0f, 1.0f - c * c)) / c : __int_as_float(0x7f800000);
    }
    tan_a = tan_a * 1.01f + 1e-6f;
    float umin = __int_as_float(0x7f800000), umax = -umin, vmin = umin, vmax = -umin, hmax = 0.0f;
    const Aabb b{lo, hi};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float3 r = sub(corner(b, k), v0);
        const float du = dot(r, e1) / l1, dv = dot(r, e2) / l2;
        umin = fminf(umin, du);
        umax = fmaxf(umax, du);
        vmin = fminf(vmin, dv);
        vmax = fmaxf(vmax, dv);
        hmax = fmaxf(hmax, dot(r, w));
    }
    const float n1 = sqrtf(l1), n2 = sqrtf(l2);
    const float rad = hmax * tan_a + 1e-4f * (length(v0) + n1 + n2 + hmax) + 1e-3f;
    const float ru = rad / n1 + 1e-5f, rv = rad / n2 + 1e-5f;
    float4 r = make_float4(umin - ru, umax + ru, vmin - rv, vmax + rv);
    if (!(l1 > 0.0f && l2 > 0.0f && r.x <= r.y && r.z <= r.w)) {
        const float inf = __int_as_float(0x7f800000);
        r = make_float4(-inf, inf, -inf, inf);
    }
    return r;
}

// Queue entries of BVH/grid launches carry the depth of their pending mirror hit in the top bits of
// the ray index (ray indices stay below 2^56, kRayIndexLimit, which every host entry point checks).
constexpr int kDepthShift = 56;
constexpr uint64_t kRayMask = (1ull << kDepthShift) - 1u;
static_assert((1ull << kDepthShift) == kRayIndexLimit, "the host ray-window check must match the packing");

// Shared memory of one CTA: the bounce queue, the generation queue (sun rays waiting for their
// direction: kFlat launches keep the sun-plane point, the others its Halton coordinates), the
// Halton table, the sun frame, and the kFlat scene with its elements' reach rectangles or the
// descriptors of the grids of the other launches.
template <int kB, bool kFlat>
struct CoreSmem {
    float qo[3][2 * kB], qd[3][2 * kB], qt[2 * kB];
    uint32_t qw[2 * kB];  // kFlat: candidate mask; BVH: element | type << 28 of the pending mirror hit
    uint64_t qray[2 * kB];
    float go[3][2 * kB];
    uint64_t gray[2 * kB];
    float4 reach[kFlat ? kFlatMax : 1];
    float t6[kH3Tab];
    FlatScene flat;
    SunFrame sun;
    GridDesc grid;
    SunGrid sg;
    // next free queue positions (shared atomics hand them out); every thread also carries the
    // sizes in registers, updated at the barriers that close each append
    int qsize;
    int gsize;
};

// Closest hit of a segment in a BVH or grid launch.
template <class C>
__device__ __forceinline__ int find_closest(const typename C::Args& A, const typename C::Core& sm, float3 o, float3 d,
                                            float tmin, float& t, uint32_t& type) {
    const bool acc = (sm.sun.shape & 2) != 0;
    if constexpr (C::kAccel == kAccelGrid) return traverse_grid(sm.grid, A.prims, o, d, tmin, acc, t, type);
    else return traverse(A.nodes, A.prims, o, d, tmin, acc, t, type);
}

// Dense element-list launches: phase A produces slot 0 of each row only (the sun-plane record);
// the other slots are empty until phase B writes them straight to global memory.
template <int kB>
struct FlatStageSmem {
    float4 rec0[kB];
};

// Where kFlux records go: the instance's flux target and the CTA's record counters.
struct Sink {
    const FluxTarget* F;
    unsigned long long* stat;  // shared memory, [4]
};

// warp-aggregated increment by the lanes that execute it together
__device__ __forceinline__ void warp_count(unsigned long long* s) {
    const unsigned m = __activemask();
    if ((int)(threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(s, (unsigned long long)__popc(m));
}

// Out of line: one copy serves every emit site (the phase A and phase B paths), which keeps the
// flux kernels' instruction footprint close to the dense ones'.
__device__ __noinline__ void flux_record(const Sink& k, float4 rec, int slot) {
    if (rec.x == 1.0f) {
        warp_count(k.stat + 1);
        return;
    }
    if (slot == 1 && k.F->staged) return;  // direct sun on the receiver: not a staged result
    warp_count(k.stat + 2);
    const int b = flux_bin(*k.F, make_float3(rec.y, rec.z, rec.w));
    if (b >= 0 && CSP_BOUNDS(3, b < k.F->nx * k.F->ny)) {
        atomicAdd(k.F->counts + b, 1u);
        warp_count(k.stat + 3);
    }
}

__device__ __forceinline__ void store_record(const TraceArgs& A, uint64_t ray, int slot, float4 rec, uint32_t id) {
    const uint64_t row = (ray - A.ray_begin) * kMaxDepth + (uint64_t)slot;
    if (!CSP_BOUNDS(2, ray >= A.ray_begin && row < A.count * kMaxDepth)) return;
    A.hits[row] = rec;
    if (A.ids) A.ids[row] = id;
}

template <class C>
__device__ __forceinline__ void emit(const typename C::Args& A, const Sink& k, uint64_t ray, int slot, float4 rec,
                                     uint32_t id) {
    if constexpr (C::kDense) store_record(A, ray, slot, rec, id);
    if constexpr (C::kFlux) flux_record(k, rec, slot);
}

// warp-aggregated append of the lanes with `want` set to the generation queue; every lane of the
// warp must call it
template <class Core>
__device__ __forceinline__ void push_gen(Core& sm, bool want, uint64_t ray, float3 o) {
    const unsigned mask = __ballot_sync(0xffffffffu, want);
    if (mask == 0u) return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == __ffs(mask) - 1) base = atomicAdd(&sm.gsize, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
    if (want && CSP_BOUNDS(1, base + __popc(mask & ((1u << lane) - 1u)) < (int)(sizeof(sm.gray) / sizeof(sm.gray[0])))) {
        const int k = base + __popc(mask & ((1u << lane) - 1u));
        sm.go[0][k] = o.x;
        sm.go[1][k] = o.y;
        sm.go[2][k] = o.z;
        sm.gray[k] = ray;
    }
}

// warp-aggregated append of the lanes with `want` set; every lane of the warp must call it
template <class Core>
__device__ __forceinline__ void push(Core& sm, bool want, uint64_t ray, float3 o, float3 d, float t,
                                     uint32_t w) {
    const unsigned mask = __ballot_sync(0xffffffffu, want);
    if (mask == 0u) return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == __ffs(mask) - 1) base = atomicAdd(&sm.qsize, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
    if (want && CSP_BOUNDS(0, base + __popc(mask & ((1u << lane) - 1u)) < (int)(sizeof(sm.qray) / sizeof(sm.qray[0])))) {
        const int k = base + __popc(mask & ((1u << lane) - 1u));
        sm.qo[0][k] = o.x;
        sm.qo[1][k] = o.y;
        sm.qo[2][k] = o.z;
        sm.qd[0][k] = d.x;
        sm.qd[1][k] = d.y;
        sm.qd[2][k] = d.z;
        sm.qt[k] = t;
        sm.qw[k] = w;
        sm.qray[k] = ray;
    }
}

// Remainder of a path in phase B, from the closest hit `h` of segment `g`: record, shade, next
// segment, until the ray misses, is absorbed, ends on the receiver or reaches the depth limit.
// pending: `h` is a mirror hit whose record was already emitted (phase A), shading comes next.
template <class C>
__device__ void finish_path(const typename C::Args& A, const Sink& k, const typename C::Core& sm, uint64_t ray, Segment g,
                            Hit h, bool pending) {
    for (;;) {
        if (h.best < 0) return;  // __miss__ms, cuda/materials.cu:236-253
        const Prim p = C::kFlat ? sm.flat.prim[h.best] : load_prim(A.prims, (uint32_t)h.best);
        if (!pending) {
            float4 rec;
            int slot;
            const bool mirror = classify(p, g, h, rec, slot);
            if (slot >= 0) emit<C>(A, k, ray, slot, rec, (uint32_t)h.best);
            if (!mirror) return;
        }
        pending = false;
        const Optics op = C::kFlat ? sm.flat.optics[h.best] : A.optics[h.best];
        Segment next;
        if (!shade_mirror<C>(A, ray, p, op, g, h, next)) return;
        g = next;
        if (C::kFlat) {
            const uint32_t m = candidates(sm.flat, g.o, g.d, g.tmin);
            h.best = closest_in(sm.flat, m, g.o, g.d, g.tmin, (sm.sun.shape & 2) != 0, h.t, h.type);
        } else {
            h.best = find_closest<C>(A, sm, g.o, g.d, g.tmin, h.t, h.type);
        }
    }
}

// One batch of up to kB rays from the top of the bounce queue (qs entries): kFlat launches finish
// their paths, BVH/grid launches advance them by one bounce.  Returns the queue size after it, the
// same in every thread (the barrier that ends the batch counts the rays queued again), so that no
// thread reads the shared counter after the batch: a warp that has gone on to the next tile may
// already be appending to it.
template <class C>
__device__ __forceinline__ int bounce_batch(const typename C::Args& A, const Sink& k, typename C::Core& sm, int qs) {
    {
        const int n = min(qs, C::kB);
        const int base = qs - n;
        const bool have = (int)threadIdx.x < n;
        float3 o = f3(0.f, 0.f, 0.f), d = f3(0.f, 0.f, 1.f);
        float t = 0.f;
        uint32_t w = 0;
        uint64_t ray = 0;
        if (have) {
            const int q = base + threadIdx.x;
            o = f3(sm.qo[0][q], sm.qo[1][q], sm.qo[2][q]);
            d = f3(sm.qd[0][q], sm.qd[1][q], sm.qd[2][q]);
            t = sm.qt[q];
            w = sm.qw[q];
            ray = sm.qray[q];
        }
        // the barrier both ends the reads of the popped entries and publishes the new size: no
        // thread appends (atomicAdd on qsize, then writes from `base` on) before it, and none read
        // qsize since the barrier that closed the last append
        if (threadIdx.x == 0) sm.qsize = base;
        __syncthreads();
        if (have) {
            if (C::kFlat) {
                // first segment from the sun: intersection programs of the candidate elements
                const Segment g{o, d, kTminSun, 0};
                Hit h;
                h.best = closest_in(sm.flat, w, o, d, kTminSun, (sm.sun.shape & 2) != 0, h.t, h.type);
                finish_path<C>(A, k, sm, ray, g, h, false);
            }
        }
        if (!C::kFlat) {
            // one bounce per batch: shade the pending mirror hit (its record is out), find the next
            // hit, record it, and queue it again when it is another mirror below the depth limit
            bool again = false;
            Segment next{f3(0.f, 0.f, 0.f), f3(0.f, 0.f, 1.f), 0.f, 0};
            Hit h2{-1, 0.f, 0u};
            const uint64_t r = ray & kRayMask;
            if (have) {
                const int depth = (int)(ray >> kDepthShift);
                const Segment g{o, d, depth == 0 ? kTminSun : kTminBounce, depth};
                const Hit h{(int)(w & kPrimMask), t, w >> kTypeShift};
                const Prim p = load_prim(A.prims, (uint32_t)h.best);
                if (shade_mirror<C>(A, r, p, A.optics[h.best], g, h, next)) {
                    h2.best = find_closest<C>(A, sm, next.o, next.d, next.tmin, h2.t, h2.type);
                    if (h2.best >= 0) {
                        const Prim p2 = load_prim(A.prims, (uint32_t)h2.best);
                        float4 rec;
                        int slot;
                        again = classify(p2, next, h2, rec, slot);
                        if (slot >= 0) emit<C>(A, k, r, slot, rec, (uint32_t)h2.best);
                    }
                }
            }
            push(sm, again, r | ((uint64_t)next.depth << kDepthShift), next.o, next.d, h2.t,
                 (uint32_t)h2.best | (h2.type << kTypeShift));
            return base + __syncthreads_count(again);
        }
        __syncthreads();
        return base;
    }
}

// One batch of up to kB rays from the top of the generation queue (gs entries): sun direction and
// the closest-hit search of the first segment, on full warps.  Element-list launches run the box
// tests and queue the rays that meet a box with their candidate mask; the others find the closest
// hit among the sun-grid candidates, emit its record and queue mirror hits for shading.  Both append
// to the bounce queue (qs entries, fewer than kB on entry).  Updates gs and qs, the same in every
// thread (the closing barrier counts the rays queued).
template <class C>
__device__ __forceinline__ void gen_batch(const typename C::Args& A, const Sink& k, typename C::Core& sm, int& gs,
                                          int& qs) {
    const int n = min(gs, C::kB);
    const int base = gs - n;
    const bool have = (int)threadIdx.x < n;
    float a = 0.f, b = 0.f, c = 0.f;
    uint64_t ray = 0;
    if (have) {
        const int q = base + threadIdx.x;
        a = sm.go[0][q];
        b = sm.go[1][q];
        c = sm.go[2][q];
        ray = sm.gray[q];
    }
    __syncthreads();
    if (threadIdx.x == 0) sm.gsize = base;
    if constexpr (C::kFlat) {
        const float3 o = f3(a, b, c);
        float3 d = f3(0.f, 0.f, 1.f);
        uint32_t m = 0;
        if (have) {
            d = sun_direction<C>(A, sm.sun, ray);
            m = candidates(sm.flat, o, d, kTminSun);
        }
        push(sm, m != 0u, ray, o, d, 0.0f, m);
        qs += __syncthreads_count(m != 0u);
    } else {
        // (a, b) = the Halton coordinates of the ray's sun-plane point
        bool again = false;
        Segment g{f3(0.f, 0.f, 0.f), f3(0.f, 0.f, 1.f), kTminSun, 0};
        Hit h{-1, 0.f, 0u};
        if (have) {
            g.o = sun_point(sm.sun, a, b);
            g.d = sun_direction<C>(A, sm.sun, ray);
            h.best = sun_closest(sm.sg, A.prims, a, b, g.o, g.d, (sm.sun.shape & 2) != 0, h.t, h.type);
            if (h.best >= 0) {
                const Prim p = load_prim(A.prims, (uint32_t)h.best);
                float4 rec;
                int s;
                again = classify(p, g, h, rec, s);
                if (s >= 0) emit<C>(A, k, ray, s, rec, (uint32_t)h.best);
            }
        }
        push(sm, again, ray, g.o, g.d, h.t, (uint32_t)h.best | (h.type << kTypeShift));
        qs += __syncthreads_count(again);
    }
    gs = base;
}

// Phase B: run full batches of queued rays (all = also the remainders).  The bounce queue is below
// kB before each generation batch (a bounce batch never grows it), so neither queue exceeds 2 kB.  qs and gs
// are the sizes of the bounce and generation queues, carried in registers by every thread of the
// CTA (equal in all of them); the caller has passed a barrier since the last append.
template <class C>
__device__ void drain(const typename C::Args& A, const Sink& k, typename C::Core& sm, bool all, int& qs, int& gs) {
    for (;;) {
        if (qs >= C::kB || (all && qs > 0 && gs == 0)) qs = bounce_batch<C>(A, k, sm, qs);
        else if (gs >= C::kB || (all && gs > 0)) gen_batch<C>(A, k, sm, gs, qs);
        else break;
    }
}

// Per-CTA setup of an instance: sun frame and the kFlat element list or the grid descriptors into
// shared memory.
// Callers synchronise before the first use.
template <class C>
__device__ __forceinline__ void load_instance_smem(const typename C::Args& A, typename C::Core& sm) {
    if (threadIdx.x < sizeof(SunFrame) / 4)
        reinterpret_cast<uint32_t*>(&sm.sun)[threadIdx.x] = reinterpret_cast<const uint32_t*>(A.sun)[threadIdx.x];
    if (C::kFlat && threadIdx.x < kFlatMax) {
        const int nprim = A.sun->n_prims;
        const int k = threadIdx.x;
        if (k < nprim) {
            // a kFlat scene's nodes are its leaves in element order
            const Node nd = A.nodes[k];
            sm.flat.prim[k] = A.prims[k];
            sm.flat.optics[k] = A.optics[k];
            sm.flat.box[k].lo = nd.lo;
            sm.flat.box[k].hi = nd.hi;
            sm.flat.type[k] = (__float_as_uint(nd.lo.w) >> kTypeShift) & 7u;
            sm.reach[k] = reach_rect(*A.sun, nd.lo, nd.hi);
        }
        if (k == 0) sm.flat.n = min(nprim, kFlatMax);
    }
    if (C::kAccel == kAccelGrid && threadIdx.x < sizeof(GridDesc) / 4)
        reinterpret_cast<uint32_t*>(&sm.grid)[threadIdx.x] = reinterpret_cast<const uint32_t*>(A.grid)[threadIdx.x];
    if (!C::kFlat && threadIdx.x >= 64 && threadIdx.x < 64 + sizeof(SunGrid) / 4)
        reinterpret_cast<uint32_t*>(&sm.sg)[threadIdx.x - 64] =
            reinterpret_cast<const uint32_t*>(A.sgrid)[threadIdx.x - 64];
}

// Phase A of one tile (rays A.ray_begin + tile * kB ...) followed by phase B on full batches.
// `stage` is the kDense staging area of element-list launches (unused otherwise); qs, gs: the queue
// sizes (see drain).
template <class C>
__device__ __forceinline__ void trace_tile(const typename C::Args& A, const Sink& k, typename C::Core& sm,
                                           typename C::Stage* stage, uint64_t tile, int& qs, int& gs) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t kk = tile * C::kB + threadIdx.x;
    uint64_t pos = kk;
    // dense launches group warps in pairs: larger groups scatter their record rows more than the
    // shared cells save
    if constexpr (C::kCoherent) pos = coherent_order<!C::kDense, C::kDense ? 2 : C::kB / 32>(kk, A.count);
    const uint64_t ray = A.ray_begin + pos;
    // sun-plane point; the direction waits in the generation queue unless the point lies outside
    // every reach rectangle (then the ray meets no element box and its record is the point alone)
    bool want = false;
    float hu = 0.f, hv = 0.f;
    float3 o = f3(0.f, 0.f, 0.f);
    if (kk < A.count) {
        hu = halton2(ray);
        hv = halton3_tab(ray, sm.t6, A.h3t12);
        o = sun_point(sm.sun, hu, hv);
        if constexpr (C::kFlat) {
            const int nr = sm.flat.n;
#pragma unroll
            for (int e = 0; e < kFlatMax; ++e) {
                if (e >= nr) break;
                want |= in_rect(sm.reach[e], hu, hv);
            }
        } else {
            want = sun_reach_any(sm.sg, hu, hv);
        }
    }
    __syncwarp();
    // element-list launches queue the point, the others its Halton coordinates (their batch looks
    // up the cell again)
    if constexpr (C::kFlat) push_gen(sm, want, ray, o);
    else push_gen(sm, want, ray, f3(hu, hv, 0.f));
    if constexpr (C::kDense && C::kCoherent) {
        // each lane writes its own ray's 80 B row: the sun-plane record, then empty slots (the
        // generation and bounce batches overwrite the slots they fill, after the barriers between)
        if (kk < A.count && CSP_BOUNDS(2, pos < A.count)) {
            float4* gh = A.hits + pos * kMaxDepth;
            gh[0] = make_float4(0.0f, o.x, o.y, o.z);
#pragma unroll
            for (int s = 1; s < kMaxDepth; ++s) gh[s] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (A.ids) {
                uint32_t* gi = A.ids + pos * kMaxDepth;
#pragma unroll
                for (int s = 0; s < kMaxDepth; ++s) gi[s] = kNoElement;
            }
        }
    } else if constexpr (C::kDense) {
        // the warp's 32 x 80 B of records leave as 5 fully coalesced 512-byte rows: record e of the
        // warp is slot e mod 5 of ray e / 5, the staged sun-plane record for slot 0, else empty
        float4* wh = stage->rec0 + warp * 32;
        wh[lane] = make_float4(0.0f, o.x, o.y, o.z);
        __syncwarp();
        const uint64_t warp_first = tile * C::kB + (uint64_t)warp * 32;
        if (warp_first < A.count) {
            const uint32_t n_rec = (uint32_t)min((uint64_t)32, A.count - warp_first) * kMaxDepth;
            float4* gh = A.hits + warp_first * kMaxDepth;
#pragma unroll
            for (int s = 0; s < kMaxDepth; ++s) {
                const uint32_t e = (uint32_t)(s * 32 + lane);
                const uint32_t r = e / kMaxDepth;
                if (e < n_rec) gh[e] = (e == r * kMaxDepth) ? wh[r] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            if (A.ids) {
                uint32_t* gi = A.ids + warp_first * kMaxDepth;
#pragma unroll
                for (int s = 0; s < kMaxDepth; ++s) {
                    const uint32_t e = (uint32_t)(s * 32 + lane);
                    if (e < n_rec) gi[e] = kNoElement;
                }
            }
        }
    }
    // the barrier before phase B counts this tile's appends to the generation queue
    gs += __syncthreads_count(want);
    drain<C>(A, k, sm, false, qs, gs);
}

}  // namespace
}  // namespace csp
