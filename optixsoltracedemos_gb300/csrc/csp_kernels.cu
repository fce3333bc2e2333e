// csp_kernels.cu -- sm_103a kernels of the single-scene trace path.
//
// Built with -fmad=false (plus IEEE division and square root): every expression rounds exactly as
// written, which is what makes the hit records bit-identical to the host restatement of the
// reference.  Fused multiply-adds appear only as explicit fmaf() calls in csp_math.cuh.
//
// Kernel map (reference counterpart in parentheses, paths inside the reference project):
//   prepare_sun_kernel   sun-plane distance, u/v bounds, parallelogram, cone frame
//                        (lib/sun_utils.cu:53-179, lib/geometry_manager.cpp:97-148, cuda/sun.cu:76-79)
//   trace_kernel         ray generation (cuda/sun.cu:16-38,72-134), closest-hit search over the
//                        elements whose AABB the ray overlaps (OptiX traversal + the intersection
//                        programs of cuda/intersection.cu:47-85,177-296,318-448), shading
//                        (cuda/materials.cu:26-231) and the hit_point_buffer write.
//   flux_records_kernel  receiver flux map from a dense hit buffer
//                        (scripts/post_processing/flux_map_calculator.py:135-179)
// The device functions of the path live in csp_trace.cuh.
#include <algorithm>
#include <atomic>
#include <mutex>

#include "csp_kernels.cuh"
#include "csp_trace.cuh"

namespace csp {
namespace {

constexpr int kTraceBlock = 256;
constexpr int kPrepBlock = 512;
constexpr int kFluxBlock = 256;

__global__ void __launch_bounds__(kPrepBlock) prepare_sun_kernel(const Aabb* __restrict__ aabbs, int n, float3 s,
                                                                   float tan_pad, int shape, float param,
                                                                   SunFrame* __restrict__ out) {
    __shared__ float scratch[kPrepBlock / 32];
    sun_frame_block(aabbs, n, s, tan_pad, shape, param, out, scratch);
}

template <int kAccel>
using PlainCfg = Cfg<kTraceBlock, kAccel, true, false>;

template <int kAccel>
struct TraceSmem {
    typename PlainCfg<kAccel>::Stage stage;
    typename PlainCfg<kAccel>::Core core;
};

// Resident 256-thread CTAs per SM the register budget is cut for: four (64 registers, 1,024
// threads) -- more warps to cover the record stream of the element-list kernel and the dependent
// loads of the candidate and cell lists of the others (64 registers measured faster than 72 or 77
// for every kernel); 256-thread CTAs instead of eight of 128: the 10,000-heliostat field 32.05 ->
// 30.23 ms per 268M rays, the single parabolic heliostat 0.3305 -> 0.3283 ms per 16M (two of 512:
// 30.4 and 0.347 ms).
template <int kAccel>
constexpr int trace_min_blocks() {
    return 4;
}

// Persistent kernel over the tiles of one launch; dense records out.  With a tile counter the CTAs
// take guided grabs (a quarter of an even share of the tiles left, at most kTraceGrab, shrinking to
// single tiles at the end), else static round robin.  The records do not depend on which CTA traces
// a tile.  Guided grabs measured 27.5 ms per 268M rays of the 10,000-heliostat field against
// 30.3 ms round robin (a CTA's tiles differ much in work, so round robin ends in a long tail), and
// 0.325 against 0.328 ms per 16M rays of the single parabolic heliostat.
constexpr unsigned long long kTraceGrab = 64;

template <int kAccel>
__global__ void __launch_bounds__(kTraceBlock, trace_min_blocks<kAccel>()) trace_kernel(
    const typename PlainCfg<kAccel>::Args A) {
    using C = PlainCfg<kAccel>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TraceSmem<kAccel>& sm = *reinterpret_cast<TraceSmem<kAccel>*>(smem_raw);
    load_instance_smem<C>(A, sm.core);
    // the shared-memory Halton table serves only launches without the device-wide 3^12 table
    if (!A.h3t12)
        for (uint32_t m = threadIdx.x; m < kH3Tab; m += kTraceBlock) sm.core.t6[m] = halton3(m);
    if (threadIdx.x == 0) {
        sm.core.qsize = 0;
        sm.core.gsize = 0;
    }
    __syncthreads();
    const Sink none{nullptr, nullptr};
    const uint64_t tiles = (A.count + kTraceBlock - 1) / kTraceBlock;
    int qs = 0, gs = 0;
    if (A.tile_counter) {
        __shared__ unsigned long long s_grab, s_want;
        unsigned long long seen = 0;  // end of this CTA's last grab (thread 0's estimate of the rest)
        for (;;) {
            if (threadIdx.x == 0) {
                const unsigned long long left = tiles > seen ? tiles - seen : 0;
                const unsigned long long want =
                    max(1ull, min(kTraceGrab, left / ((unsigned long long)gridDim.x * 4)));
                s_grab = atomicAdd(A.tile_counter, want);
                s_want = want;
            }
            __syncthreads();
            // every thread reads the grab before thread 0 can write the next one: trace_tile has
            // CTA barriers, and a grab past the end ends the loop in every thread
            const uint64_t g0 = s_grab, g1 = min((uint64_t)(g0 + s_want), tiles);
            if (g0 >= tiles) break;
            seen = g1;
            for (uint64_t tile = g0; tile < g1; ++tile) trace_tile<C>(A, none, sm.core, &sm.stage, tile, qs, gs);
        }
    } else {
        for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x)
            trace_tile<C>(A, none, sm.core, &sm.stage, tile, qs, gs);
    }
    drain<C>(A, none, sm.core, true, qs, gs);
}

template <int kAccel>
cudaError_t launch_trace_t(const TraceArgs& args, cudaStream_t stream) {
    // persistent grid: every resident CTA slot of the device, never more CTAs than tiles
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // the attribute is set once per device (bit `dev` of the mask; devices past 63 set it every time)
    static std::atomic<unsigned long long> attr_set{0};
    const unsigned long long bit = (dev >= 0 && dev < 64) ? 1ull << dev : 0ull;
    if (e == cudaSuccess && !(bit && (attr_set.load(std::memory_order_acquire) & bit))) {
        e = cudaFuncSetAttribute(trace_kernel<kAccel>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(TraceSmem<kAccel>));
        if (e == cudaSuccess) attr_set.fetch_or(bit, std::memory_order_acq_rel);
    }
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_kernel<kAccel>, kTraceBlock,
                                                          sizeof(TraceSmem<kAccel>));
    if (e != cudaSuccess) return e;
    const uint64_t tiles = (args.count + kTraceBlock - 1) / kTraceBlock;  // CTAs that have work
    const uint64_t grid = std::min<uint64_t>(tiles, (uint64_t)std::max(1, sms * std::max(1, per_sm)));
    typename PlainCfg<kAccel>::Args a;
    static_cast<TraceArgs&>(a) = args;
    if constexpr (PlainCfg<kAccel>::kSched) philox_keys(args.seed, a.keys);
    if (args.tile_counter) {
        e = cudaMemsetAsync(args.tile_counter, 0, sizeof(unsigned long long), stream);
        if (e != cudaSuccess) return e;
    }
    trace_kernel<kAccel><<<(unsigned)grid, kTraceBlock, sizeof(TraceSmem<kAccel>), stream>>>(a);
    return cudaGetLastError();
}

// Grid-stride pass over n_records float4 records {stage, x, y, z}: stage-1 records are counted,
// stage-2 records are counted and binned.
__global__ void __launch_bounds__(kFluxBlock) flux_records_kernel(const float4* __restrict__ hits,
                                                                    uint64_t n_records, const FluxTarget F) {
    __shared__ unsigned long long stat[4];
    if (threadIdx.x < 4) stat[threadIdx.x] = 0;
    __syncthreads();
    const Sink k{&F, stat};
    for (uint64_t i = blockIdx.x * (uint64_t)kFluxBlock + threadIdx.x; i < n_records;
         i += (uint64_t)gridDim.x * kFluxBlock) {
        const float4 r = __ldg(hits + i);
        if (r.x == 1.0f || r.x == 2.0f) flux_record(k, r, (int)(i % kMaxDepth));
    }
    __syncthreads();
    if (threadIdx.x < 4 && threadIdx.x > 0 && stat[threadIdx.x]) atomicAdd(F.stats + threadIdx.x, stat[threadIdx.x]);
}

// Compact records (csp_run_to_host_compact): a row of the dense buffer is the sun-plane record in
// slot 0, then the ray's further records in slots 1.. (stage 1 or 2, so x != 0), then empty slots.
constexpr int kCompactBlock = 256;

__device__ __forceinline__ uint32_t row_records(const float4* __restrict__ hits, uint64_t r) {
    uint32_t c = 0;
#pragma unroll
    for (int s = 1; s < kMaxDepth; ++s) c += __ldg(&hits[r * kMaxDepth + s].x) != 0.0f ? 1u : 0u;
    return c;
}

// Block-wide exclusive prefix of v (kCompactBlock threads); `total` receives the block's sum.
__device__ uint32_t block_exclusive(uint32_t v, uint32_t* scratch, uint32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) scratch[warp] = x;
    __syncthreads();
    uint32_t before = 0;
    total = 0;
    for (int w = 0; w < kCompactBlock / 32; ++w) {
        if (w < warp) before += scratch[w];
        total += scratch[w];
    }
    return before + x - v;
}

// Records beyond slot 0 of every ray, and their sum per block.
__global__ void __launch_bounds__(kCompactBlock) compact_count_kernel(const float4* __restrict__ hits, uint64_t n,
                                                                      uint8_t* __restrict__ counts,
                                                                      unsigned long long* __restrict__ block_sums) {
    __shared__ uint32_t scratch[kCompactBlock / 32];
    const uint64_t r = (uint64_t)blockIdx.x * kCompactBlock + threadIdx.x;
    uint32_t c = 0;
    if (r < n) {
        c = row_records(hits, r);
        counts[r] = (uint8_t)c;
    }
    uint32_t total;
    block_exclusive(c, scratch, total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// In place: block sums -> exclusive block offsets, the grand total after the last block.
__global__ void __launch_bounds__(1024) compact_scan_kernel(unsigned long long* __restrict__ sums, uint64_t nb) {
    __shared__ unsigned long long part[1024];
    const uint64_t chunk = (nb + 1023) / 1024;
    const uint64_t c0 = min(nb, (uint64_t)threadIdx.x * chunk), c1 = min(nb, c0 + chunk);
    unsigned long long s = 0;
    for (uint64_t c = c0; c < c1; ++c) s += sums[c];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned long long v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0ull;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long run = part[threadIdx.x] - s;
    for (uint64_t c = c0; c < c1; ++c) {
        const unsigned long long k = sums[c];
        sums[c] = run;
        run += k;
    }
    if (threadIdx.x == 1023) sums[nb] = part[1023];
}

// Sun-plane points (3 floats per ray) and the records beyond slot 0, in ray order.
__global__ void __launch_bounds__(kCompactBlock) compact_write_kernel(const float4* __restrict__ hits, uint64_t n,
                                                                      const unsigned long long* __restrict__ offsets,
                                                                      float* __restrict__ points,
                                                                      float4* __restrict__ records) {
    __shared__ uint32_t scratch[kCompactBlock / 32];
    const uint64_t r = (uint64_t)blockIdx.x * kCompactBlock + threadIdx.x;
    uint32_t c = 0;
    if (r < n) c = row_records(hits, r);
    uint32_t total;
    const uint32_t ex = block_exclusive(c, scratch, total);
    if (r >= n) return;
    const float4 p = __ldg(&hits[r * kMaxDepth]);
    points[3 * r] = p.y;
    points[3 * r + 1] = p.z;
    points[3 * r + 2] = p.w;
    const uint64_t o = offsets[blockIdx.x] + ex;
    for (uint32_t s = 0; s < c; ++s) records[o + s] = __ldg(&hits[r * kMaxDepth + 1 + s]);
}

__global__ void __launch_bounds__(256) halton3_table_kernel(float* __restrict__ t) {
    const uint32_t m = blockIdx.x * 256u + threadIdx.x;
    if (m < kH3T12) t[m] = halton3(m);
}

}  // namespace

const float* halton3_table() {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static float* tables[kMaxDevices] = {};
    static bool tried[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(mu);
    if (!tried[dev]) {
        tried[dev] = true;
        float* t = nullptr;
        if (dev_alloc((void**)&t, kH3T12 * sizeof(float)) == cudaSuccess) {
            halton3_table_kernel<<<(kH3T12 + 255) / 256, 256>>>(t);
            if (cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess) tables[dev] = t;
            else cudaFree(t);
        }
        cudaGetLastError();  // a failed table only means the loop path
    }
    return tables[dev];
}

cudaError_t launch_prepare_sun(const Aabb* aabbs, int n, float sx, float sy, float sz, float tan_pad, int shape,
                               float param, SunFrame* out, cudaStream_t stream) {
    prepare_sun_kernel<<<1, kPrepBlock, 0, stream>>>(aabbs, n, make_float3(sx, sy, sz), tan_pad, shape, param, out);
    return cudaGetLastError();
}

cudaError_t launch_trace(const TraceArgs& args, int n_prims, cudaStream_t stream) {
    if (args.count == 0) return cudaSuccess;
    if (n_prims <= kFlatMax) return launch_trace_t<kAccelFlat>(args, stream);
    if (!args.sgrid) return cudaErrorInvalidValue;  // scenes above the element list need their sun grid
    if (args.grid) return launch_trace_t<kAccelGrid>(args, stream);
    return launch_trace_t<kAccelBvh>(args, stream);
}

uint64_t compact_blocks(uint64_t n) { return (n + kCompactBlock - 1) / kCompactBlock; }

cudaError_t launch_compact_count(const float4* hits, uint64_t n, uint8_t* counts, unsigned long long* block_sums,
                                 cudaStream_t stream) {
    const uint64_t nb = compact_blocks(n);
    if (nb == 0) return cudaSuccess;
    if (nb > 0x7FFFFFFFull) return cudaErrorInvalidValue;
    compact_count_kernel<<<(unsigned)nb, kCompactBlock, 0, stream>>>(hits, n, counts, block_sums);
    compact_scan_kernel<<<1, 1024, 0, stream>>>(block_sums, nb);
    return cudaGetLastError();
}

cudaError_t launch_compact_write(const float4* hits, uint64_t n, const unsigned long long* block_offsets, float* points,
                                 float4* records, cudaStream_t stream) {
    const uint64_t nb = compact_blocks(n);
    if (nb == 0) return cudaSuccess;
    compact_write_kernel<<<(unsigned)nb, kCompactBlock, 0, stream>>>(hits, n, block_offsets, points, records);
    return cudaGetLastError();
}

cudaError_t launch_flux_records(const float4* hits, uint64_t n_records, const FluxTarget& F, cudaStream_t stream) {
    if (n_records == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const uint64_t blocks = std::min<uint64_t>((n_records + kFluxBlock - 1) / kFluxBlock, (uint64_t)sms * 8);
    flux_records_kernel<<<(unsigned)blocks, kFluxBlock, 0, stream>>>(hits, n_records, F);
    return cudaGetLastError();
}

uint32_t bounds_sites_trace() { return take_bounds_sites(); }

}  // namespace csp
