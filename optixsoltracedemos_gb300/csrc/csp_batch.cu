// csp_batch.cu -- multi-instance kernels: BVH refit, per-instance sun frames, and the persistent
// trace kernel that runs many scene instances (sun positions, heliostat aim states, ray counts)
// in one launch with the receiver flux map accumulated in the shading stage.
//
// Reference counterparts (paths inside the reference project): the refit replaces the OptiX GAS
// update of lib/geometry_manager.cpp:150-266 (OPERATION_UPDATE); the sun frames are the
// per-launch setup of lib/geometry_manager.cpp:97-148 and lib/sun_utils.cu:53-179; the trace is the
// optixLaunch of lib/soltrace_system.cpp:145-170 with the flux binning of
// scripts/post_processing/flux_map_calculator.py:135-179 moved into the closest-hit stage.
#include <algorithm>
#include <atomic>

#include "csp_kernels.cuh"
#include "csp_trace.cuh"

namespace csp {
namespace {

constexpr int kRefitBlock = 256;  // 8 warps, one node per warp
constexpr int kPrepBlock = 512;

__global__ void __launch_bounds__(kRefitBlock) refit_kernel(const RefitJob* __restrict__ jobs) {
    const RefitJob J = jobs[blockIdx.y];
    const int node = blockIdx.x * (kRefitBlock / 32) + (threadIdx.x >> 5);
    if (node >= J.n_nodes) return;
    const int lane = threadIdx.x & 31;
    const float4 tlo = __ldg(reinterpret_cast<const float4*>(J.topo + node));
    const float4 thi = __ldg(reinterpret_cast<const float4*>(J.topo + node) + 1);
    const uint32_t hitw = __float_as_uint(tlo.w);
    if (hitw & kLeafFlag) {
        if (lane == 0) {
            const Aabb a = J.aabbs[hitw & kPrimMask];
            Node o;
            o.lo = make_float4(a.lo.x, a.lo.y, a.lo.z, tlo.w);
            o.hi = make_float4(a.hi.x, a.hi.y, a.hi.z, thi.w);
            J.out[node] = o;
        }
        return;
    }
    // the subtree of an internal node is the index range [node, miss) of the depth-first layout
    const int miss = __float_as_int(thi.w);
    const int end = miss >= 0 ? miss : J.n_nodes;
    float lx = FLT_MAX, ly = FLT_MAX, lz = FLT_MAX, hx = -FLT_MAX, hy = -FLT_MAX, hz = -FLT_MAX;
#pragma unroll 4
    for (int j = node + 1 + lane; j < end; j += 32) {
        const uint32_t w = __float_as_uint(__ldg(reinterpret_cast<const float*>(J.topo + j) + 3));
        if (w & kLeafFlag) {
            const Aabb b = J.prune[w & kPrimMask];
            lx = fminf(lx, b.lo.x);
            ly = fminf(ly, b.lo.y);
            lz = fminf(lz, b.lo.z);
            hx = fmaxf(hx, b.hi.x);
            hy = fmaxf(hy, b.hi.y);
            hz = fmaxf(hz, b.hi.z);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
        ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
        lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
        hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
        hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
        hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
    }
    if (lane == 0) {
        Node o;
        o.lo = make_float4(lx, ly, lz, tlo.w);
        o.hi = make_float4(hx, hy, hz, thi.w);
        J.out[node] = o;
    }
}

__global__ void __launch_bounds__(kPrepBlock) prepare_sun_batch_kernel(const SunJob* __restrict__ jobs) {
    __shared__ float scratch[kPrepBlock / 32];
    const SunJob J = jobs[blockIdx.x];
    sun_frame_block(J.aabbs, J.n, make_float3(J.sx, J.sy, J.sz), J.tan_pad, J.shape, J.param, J.out, scratch);
}

template <int kB, int kAccel>
struct BatchSmem {
    typename Cfg<kB, kAccel, false, true>::Core core;
    TraceArgs A;
    FluxTarget F;
    unsigned long long stat[4];
    unsigned long long grab;
    unsigned long long want;
};

// Drain the queues of the current instance and add its record counters to the instance's totals.
template <class C>
__device__ __forceinline__ void finish_instance(BatchSmem<C::kB, C::kAccel>& sm, const Sink& k, int& qs, int& gs) {
    drain<C>(sm.A, k, sm.core, true, qs, gs);
    __syncthreads();
    if (threadIdx.x > 0 && threadIdx.x < 4) {
        const unsigned long long v = sm.stat[threadIdx.x];
        if (v) atomicAdd(sm.F.stats + threadIdx.x, v);
        sm.stat[threadIdx.x] = 0;
    }
    __syncthreads();
}

// Resident threads per SM the register budget is cut for: 1024 for the field kernels (64
// registers: more warps to hide the grid walk's load latency), 1152 for the element-list kernel
// (nine 128-thread CTAs, 56 registers: its phases are short latency chains, and it measured 3.5 %
// faster than at 64 registers despite a few spilled bytes).
template <int kAccel>
constexpr int batch_threads_per_sm() {
    return kAccel == kAccelFlat ? 1152 : 1024;
}

template <int kB, int kAccel>
__global__ void __launch_bounds__(kB, batch_threads_per_sm<kAccel>() / kB) batch_kernel(const BatchLaunch L) {
    using C = Cfg<kB, kAccel, false, true>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BatchSmem<kB, kAccel>& sm = *reinterpret_cast<BatchSmem<kB, kAccel>*>(smem_raw);
    for (uint32_t m = threadIdx.x; m < kH3Tab; m += kB) sm.core.t6[m] = halton3(m);
    if (threadIdx.x < 4) sm.stat[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        sm.core.qsize = 0;
        sm.core.gsize = 0;
        sm.grab = 0;
    }
    const Sink k{&sm.F, sm.stat};
    bool have = false;
    uint64_t t0 = 0, t1 = 0;  // tile range of the current instance
    int qs = 0, gs = 0;       // queue sizes (see drain)
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            // guided grabs: a quarter of an even share of the tiles left (as this CTA last saw
            // them), at most L.chunk and at least one, so grabs shrink towards single tiles at the
            // end (a large grab taken last would otherwise run alone).  Large grabs early keep a CTA
            // on one instance across consecutive grabs: each switch drains its queues in partial
            // batches.
            const unsigned long long left = L.total_tiles > sm.grab ? L.total_tiles - sm.grab : 0;
            const unsigned long long want =
                max(1ull, min((unsigned long long)L.chunk, left / ((unsigned long long)gridDim.x * 4)));
            sm.grab = atomicAdd(L.next_tile, want);
            sm.want = want;
        }
        __syncthreads();
        const uint64_t g0 = sm.grab;
        if (g0 >= L.total_tiles) break;
        const uint64_t g1 = min(g0 + (uint64_t)sm.want, L.total_tiles);
        for (uint64_t g = g0; g < g1; ++g) {
            if (!have || g < t0 || g >= t1) {
                // instance of tile g: the last i with tile_begin[i] <= g (empty instances skipped)
                int lo = 0, hi = L.n_inst - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (__ldg(L.tile_begin + mid) <= g) lo = mid;
                    else hi = mid - 1;
                }
                if (have) finish_instance<C>(sm, k, qs, gs);
                const uint32_t* src = reinterpret_cast<const uint32_t*>(L.inst + lo);
                constexpr int kWordsA = sizeof(TraceArgs) / 4, kWordsF = sizeof(FluxTarget) / 4;
                for (int w = threadIdx.x; w < kWordsA + kWordsF; w += kB) {
                    if (w < kWordsA) reinterpret_cast<uint32_t*>(&sm.A)[w] = __ldg(src + w);
                    else reinterpret_cast<uint32_t*>(&sm.F)[w - kWordsA] =
                        __ldg(src + offsetof(InstanceDesc, flux) / 4 + (w - kWordsA));
                }
                __syncthreads();
                load_instance_smem<C>(sm.A, sm.core);
                __syncthreads();
                have = true;
                t0 = __ldg(L.tile_begin + lo);
                t1 = __ldg(L.tile_begin + lo + 1);
            }
            trace_tile<C>(sm.A, k, sm.core, nullptr, g - t0, qs, gs);
        }
    }
    if (have) finish_instance<C>(sm, k, qs, gs);
}

template <int kB, int kAccel>
constexpr size_t batch_smem() {
    return sizeof(BatchSmem<kB, kAccel>);
}

// Occupancy limit on the current device; the shared-memory attribute is set (and the limit
// computed) once per device.
template <int kB, int kAccel>
int occupancy_t() {
    constexpr int kMaxDevices = 64;
    static std::atomic<int> cached[kMaxDevices];  // 0 = not yet known (a kernel that fits has >= 1)
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (dev >= 0 && dev < kMaxDevices) {
        const int c = cached[dev].load(std::memory_order_acquire);
        if (c > 0) return c;
    }
    if (cudaFuncSetAttribute(batch_kernel<kB, kAccel>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)batch_smem<kB, kAccel>()) != cudaSuccess)
        return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel<kB, kAccel>, kB, batch_smem<kB, kAccel>()) !=
        cudaSuccess)
        return 0;
    if (dev >= 0 && dev < kMaxDevices && per_sm > 0) cached[dev].store(per_sm, std::memory_order_release);
    return per_sm;
}

template <int kB, int kAccel>
cudaError_t launch_t(const BatchLaunch& L, const BatchTuning& t, cudaStream_t stream) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int occ = occupancy_t<kB, kAccel>();
    if (occ <= 0) return cudaErrorInvalidConfiguration;
    const int per_sm = std::max(1, std::min(occ, t.ctas_per_sm > 0 ? t.ctas_per_sm : occ));
    const uint64_t grid = std::min<uint64_t>(std::max<uint64_t>(L.total_tiles, 1), (uint64_t)sms * per_sm);
    batch_kernel<kB, kAccel><<<(unsigned)grid, kB, batch_smem<kB, kAccel>(), stream>>>(L);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_refit(const RefitJob* jobs, int n_jobs, int max_nodes, cudaStream_t stream) {
    if (n_jobs <= 0 || max_nodes <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((max_nodes + kRefitBlock / 32 - 1) / (kRefitBlock / 32)), (unsigned)n_jobs);
    refit_kernel<<<grid, kRefitBlock, 0, stream>>>(jobs);
    return cudaGetLastError();
}

cudaError_t launch_prepare_sun_batch(const SunJob* jobs, int n_jobs, cudaStream_t stream) {
    if (n_jobs <= 0) return cudaSuccess;
    prepare_sun_batch_kernel<<<(unsigned)n_jobs, kPrepBlock, 0, stream>>>(jobs);
    return cudaGetLastError();
}

int batch_occupancy(int accel, int block) {
    switch (accel * 1000 + block) {
        case kAccelFlat * 1000 + 128: return occupancy_t<128, kAccelFlat>();
        case kAccelFlat * 1000 + 256: return occupancy_t<256, kAccelFlat>();
        case kAccelBvh * 1000 + 128: return occupancy_t<128, kAccelBvh>();
        case kAccelBvh * 1000 + 256: return occupancy_t<256, kAccelBvh>();
        case kAccelGrid * 1000 + 128: return occupancy_t<128, kAccelGrid>();
        case kAccelGrid * 1000 + 256: return occupancy_t<256, kAccelGrid>();
        default: return 0;
    }
}

namespace {

template <int kB, int kAccel>
uint32_t build_of() {
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, batch_kernel<kB, kAccel>) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    // FNV-1a over the numbers that change when the kernel's code generation changes
    uint32_t h = 2166136261u;
    for (uint64_t v : {(uint64_t)a.numRegs, (uint64_t)a.sharedSizeBytes, (uint64_t)a.localSizeBytes,
                       (uint64_t)a.maxThreadsPerBlock, (uint64_t)a.constSizeBytes, (uint64_t)batch_smem<kB, kAccel>()})
        for (int b = 0; b < 8; ++b) h = (h ^ (uint32_t)((v >> (8 * b)) & 0xffu)) * 16777619u;
    return h;
}

}  // namespace

uint32_t batch_kernel_build(int accel) {
    switch (accel) {
        case kAccelFlat: return build_of<128, kAccelFlat>() ^ (build_of<256, kAccelFlat>() * 3u);
        case kAccelBvh: return build_of<128, kAccelBvh>() ^ (build_of<256, kAccelBvh>() * 3u);
        case kAccelGrid: return build_of<128, kAccelGrid>() ^ (build_of<256, kAccelGrid>() * 3u);
        default: return 0;
    }
}

cudaError_t launch_trace_batch(const BatchLaunch& L, int accel, const BatchTuning& t, cudaStream_t stream) {
    if (L.total_tiles == 0 || L.n_inst <= 0) return cudaSuccess;
    if (t.chunk <= 0) return cudaErrorInvalidValue;
    switch (accel * 1000 + t.block) {
        case kAccelFlat * 1000 + 128: return launch_t<128, kAccelFlat>(L, t, stream);
        case kAccelFlat * 1000 + 256: return launch_t<256, kAccelFlat>(L, t, stream);
        case kAccelBvh * 1000 + 128: return launch_t<128, kAccelBvh>(L, t, stream);
        case kAccelBvh * 1000 + 256: return launch_t<256, kAccelBvh>(L, t, stream);
        case kAccelGrid * 1000 + 128: return launch_t<128, kAccelGrid>(L, t, stream);
        case kAccelGrid * 1000 + 256: return launch_t<256, kAccelGrid>(L, t, stream);
        default: return cudaErrorInvalidValue;
    }
}

uint32_t bounds_sites_batch() { return take_bounds_sites(); }

}  // namespace csp
