// csp_sungrid.cu -- device build of the sun-ray candidate grid (SunGrid, csp_types.cuh) of each
// scene state, after its sun frame.
//
// The reference has no counterpart: OptiX traverses its GAS from the sun plane for every ray
// (cuda/sun.cu:119-133).  Here the sun rays of scenes above 8 elements find their candidates in one
// cell of a grid over the sun plane's Halton coordinates, binned from the elements' reach
// rectangles (reach_rect, csp_trace.cuh), and rays outside every rectangle skip the direction and
// the search altogether.  Which elements a ray tests changes, never which hit it finds: the reach
// rectangles bound every ray that can meet an element's AABB, and the closest hit keeps the lower
// element index on equal t whatever the order of the candidates.
//
// Four launches per set of states (blockIdx.y or blockIdx.x = the state):
//   size   one block per state: every element's rectangle, the grid size from their mean extent
//          (shrunk until the registered items fit the capacity), the descriptor, zeroed counts
//   count  one thread per element: per-cell counts, or a place in the global list for rectangles of
//          more than kSunGridMaxCells cells
//   scan   one block per state: exclusive prefix sums of the counts (cell_start) and fill cursors
//   fill   one thread per element: rectangles and exact boxes into their cells
// The order of the items within a cell and of the global list follows the atomics; nothing that a
// ray records depends on it.
#include <algorithm>

#include "csp_kernels.cuh"
#include "csp_trace.cuh"

namespace csp {
namespace {

constexpr int kSizeBlock = 512;
constexpr int kElemBlock = 256;
constexpr int kScanBlock = 1024;
constexpr int kMaxAxisCells = 4096;
constexpr float kCellScale = 0.5f;  // cell width / mean rectangle width
constexpr int kMaxJobsPerLaunch = 65535;  // gridDim.y limit

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

// Cells covered by rectangle r in an nu x nv grid; false when r holds no point of [0, 1]^2.
__device__ __forceinline__ bool sg_range(float4 r, float fnu, float fnv, int nu, int nv, int& iu0, int& iu1, int& iv0,
                                         int& iv1) {
    if (!(r.y >= 0.0f && r.x <= 1.0f && r.w >= 0.0f && r.z <= 1.0f)) return false;
    iu0 = sg_cell(fmaxf(r.x, 0.0f), fnu, nu);
    iu1 = sg_cell(fminf(r.y, 1.0f), fnu, nu);
    iv0 = sg_cell(fmaxf(r.z, 0.0f), fnv, nv);
    iv1 = sg_cell(fminf(r.w, 1.0f), fnv, nv);
    return true;
}

// Block-wide sum in a fixed order (the same result on every run).
template <class T>
__device__ T block_sum(T v, T* scratch) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    T s = scratch[0];
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) s += scratch[i];
    return s;
}

__global__ void __launch_bounds__(kSizeBlock) sungrid_size_kernel(const SunGridJob* __restrict__ jobs) {
    const SunGridJob J = jobs[blockIdx.x];
    __shared__ SunFrame S;
    __shared__ float fs[kSizeBlock / 32];
    __shared__ unsigned long long us[kSizeBlock / 32];
    __shared__ int s_nu, s_nv;
    if (threadIdx.x < sizeof(SunFrame) / 4)
        reinterpret_cast<uint32_t*>(&S)[threadIdx.x] = reinterpret_cast<const uint32_t*>(J.sun)[threadIdx.x];
    __syncthreads();
    // reach rectangles; mean extent of the ordinary ones (not the whole-plane or oversized ones)
    float su = 0.0f, sv = 0.0f;
    unsigned long long cnt = 0;
    for (int e = threadIdx.x; e < J.n; e += kSizeBlock) {
        const Aabb b = J.aabbs[e];
        const float4 r = reach_rect(S, b.lo, b.hi);
        J.rect[e] = r;
        if (r.y >= 0.0f && r.x <= 1.0f && r.w >= 0.0f && r.z <= 1.0f) {
            const float wu = fminf(r.y, 1.0f) - fmaxf(r.x, 0.0f), wv = fminf(r.w, 1.0f) - fmaxf(r.z, 0.0f);
            if (wu < 0.25f && wv < 0.25f) {
                su += wu;
                sv += wv;
                ++cnt;
            }
        }
    }
    su = block_sum(su, fs);
    sv = block_sum(sv, fs);
    cnt = block_sum(cnt, us);
    if (threadIdx.x == 0) {
        // cells half as wide as the mean rectangle: a rectangle covers about 3 x 3 cells, and a ray
        // scans the items of its cell -- on the 256-instance field batch 13 per generated ray with
        // cells as wide as the mean rectangle (3.5 of them holding the ray), and 5 % less batch time
        // with half-width cells than with those (no gain from a third)
        int nu = 1, nv = 1;
        if (cnt > 0) {
            const float mu = fmaxf(su / (float)cnt, 1.0f / kMaxAxisCells), mv = fmaxf(sv / (float)cnt, 1.0f / kMaxAxisCells);
            nu = min(kMaxAxisCells, max(1, (int)ceilf(1.0f / (mu * kCellScale))));
            nv = min(kMaxAxisCells, max(1, (int)ceilf(1.0f / (mv * kCellScale))));
        }
        while ((long long)nu * nv > (long long)J.cap_cells) {
            nu = max(1, nu * 3 / 4);
            nv = max(1, nv * 3 / 4);
        }
        s_nu = nu;
        s_nv = nv;
    }
    __syncthreads();
    // shrink until the registered items fit (at 1 x 1 every element holds at most one item)
    for (;;) {
        const int nu = s_nu, nv = s_nv;
        const float fnu = (float)nu, fnv = (float)nv;
        unsigned long long items = 0;
        for (int e = threadIdx.x; e < J.n; e += kSizeBlock) {
            int iu0, iu1, iv0, iv1;
            if (!sg_range(J.rect[e], fnu, fnv, nu, nv, iu0, iu1, iv0, iv1)) continue;
            const long long cells = (long long)(iu1 - iu0 + 1) * (iv1 - iv0 + 1);
            if (cells <= kSunGridMaxCells) items += (unsigned long long)cells;
        }
        items = block_sum(items, us);
        if (items <= J.cap_items || (nu == 1 && nv == 1)) break;
        __syncthreads();
        if (threadIdx.x == 0) {
            s_nu = max(1, nu * 3 / 4);
            s_nv = max(1, nv * 3 / 4);
        }
        __syncthreads();
    }
    const int nu = s_nu, nv = s_nv;
    for (int c = threadIdx.x; c <= nu * nv; c += kSizeBlock) J.cell_start[c] = 0;
    if (threadIdx.x == 0) {
        SunGrid d;
        d.nu = nu;
        d.nv = nv;
        d.n_global = 0;
        d.n = J.n;
        d.fnu = (float)nu;
        d.fnv = (float)nv;
        d.pad0 = d.pad1 = 0.0f;
        d.cell_start = J.cell_start;
        d.item_rect = J.item_rect;
        d.item_box = J.item_box;
        d.global_id = J.global_id;
        d.rect = J.rect;
        d.aabbs = J.aabbs;
        *J.desc = d;
    }
}

__global__ void __launch_bounds__(kElemBlock) sungrid_count_kernel(const SunGridJob* __restrict__ jobs) {
    const SunGridJob& J = jobs[blockIdx.y];
    const int e = blockIdx.x * kElemBlock + threadIdx.x;
    if (e >= J.n) return;
    const int nu = J.desc->nu, nv = J.desc->nv;
    int iu0, iu1, iv0, iv1;
    if (!sg_range(J.rect[e], (float)nu, (float)nv, nu, nv, iu0, iu1, iv0, iv1)) return;
    if ((long long)(iu1 - iu0 + 1) * (iv1 - iv0 + 1) > kSunGridMaxCells) {
        const int k = atomicAdd(&J.desc->n_global, 1);
        if (CSP_BOUNDS(6, k < J.n)) J.global_id[k] = (uint32_t)e;
        return;
    }
    for (int iv = iv0; iv <= iv1; ++iv)
        for (int iu = iu0; iu <= iu1; ++iu)
            if (CSP_BOUNDS(6, iv * nu + iu < J.cap_cells)) atomicAdd(J.cell_start + iv * nu + iu, 1u);
}

__global__ void __launch_bounds__(kScanBlock) sungrid_scan_kernel(const SunGridJob* __restrict__ jobs) {
    const SunGridJob& J = jobs[blockIdx.x];
    __shared__ uint32_t part[kScanBlock];
    const int nc = J.desc->nu * J.desc->nv;
    const int chunk = (nc + kScanBlock - 1) / kScanBlock;
    const int c0 = min(nc, (int)threadIdx.x * chunk), c1 = min(nc, c0 + chunk);
    uint32_t s = 0;
    for (int c = c0; c < c1; ++c) s += J.cell_start[c];
    part[threadIdx.x] = s;
    __syncthreads();
    // inclusive scan of the per-thread sums (Hillis-Steele)
    for (int o = 1; o < kScanBlock; o <<= 1) {
        const uint32_t v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
    for (int c = c0; c < c1; ++c) {
        const uint32_t k = J.cell_start[c];
        J.cell_start[c] = run;
        J.cursor[c] = run;
        run += k;
    }
    if (threadIdx.x == kScanBlock - 1) J.cell_start[nc] = part[kScanBlock - 1];
}

__global__ void __launch_bounds__(kElemBlock) sungrid_fill_kernel(const SunGridJob* __restrict__ jobs) {
    const SunGridJob& J = jobs[blockIdx.y];
    const int e = blockIdx.x * kElemBlock + threadIdx.x;
    if (e >= J.n) return;
    const int nu = J.desc->nu, nv = J.desc->nv;
    const float4 r = J.rect[e];
    int iu0, iu1, iv0, iv1;
    if (!sg_range(r, (float)nu, (float)nv, nu, nv, iu0, iu1, iv0, iv1)) return;
    if ((long long)(iu1 - iu0 + 1) * (iv1 - iv0 + 1) > kSunGridMaxCells) return;
    for (int iv = iv0; iv <= iv1; ++iv)
        for (int iu = iu0; iu <= iu1; ++iu) {
            if (!CSP_BOUNDS(6, iv * nu + iu < J.cap_cells)) continue;
            const uint32_t k = atomicAdd(J.cursor + iv * nu + iu, 1u);
            if (!CSP_BOUNDS(6, k < J.cap_items)) continue;
            J.item_rect[k] = r;
            J.item_box[k] = J.aabbs[e];
        }
}

}  // namespace

uint32_t bounds_sites_sungrid() { return take_bounds_sites(); }

SunGridCaps sungrid_caps(uint32_t n) {
    SunGridCaps c;
    c.cap_cells = (int)std::min<uint64_t>(262144, std::max<uint64_t>(64, 8ull * n));
    c.cap_items = (uint32_t)std::min<uint64_t>(0xFFFFFFF0u, (uint64_t)kSunGridItemsPerElem * n + 64);
    return c;
}

size_t sungrid_bytes(uint32_t n) {
    const SunGridCaps c = sungrid_caps(n);
    return a256(sizeof(SunGrid)) + a256(((size_t)c.cap_cells + 1) * sizeof(uint32_t)) +
           a256((size_t)c.cap_cells * sizeof(uint32_t)) + a256((size_t)n * sizeof(float4)) +
           a256((size_t)c.cap_items * sizeof(float4)) + a256((size_t)c.cap_items * sizeof(Aabb)) +
           a256((size_t)std::max<uint32_t>(n, 1) * sizeof(uint32_t));
}

void sungrid_place(unsigned char* base, uint32_t n, SunGridJob& job) {
    const SunGridCaps c = sungrid_caps(n);
    size_t o = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = base + o;
        o += a256(bytes);
        return p;
    };
    job.desc = reinterpret_cast<SunGrid*>(take(sizeof(SunGrid)));
    job.cell_start = reinterpret_cast<uint32_t*>(take(((size_t)c.cap_cells + 1) * sizeof(uint32_t)));
    job.cursor = reinterpret_cast<uint32_t*>(take((size_t)c.cap_cells * sizeof(uint32_t)));
    job.rect = reinterpret_cast<float4*>(take((size_t)n * sizeof(float4)));
    job.item_rect = reinterpret_cast<float4*>(take((size_t)c.cap_items * sizeof(float4)));
    job.item_box = reinterpret_cast<Aabb*>(take((size_t)c.cap_items * sizeof(Aabb)));
    job.global_id = reinterpret_cast<uint32_t*>(take((size_t)std::max<uint32_t>(n, 1) * sizeof(uint32_t)));
    job.n = (int)n;
    job.cap_cells = c.cap_cells;
    job.cap_items = c.cap_items;
    job.pad = 0;
}

cudaError_t launch_sungrid_build(const SunGridJob* jobs, int n_jobs, int max_n, cudaStream_t stream) {
    if (n_jobs <= 0 || max_n <= 0) return cudaSuccess;
    for (int j0 = 0; j0 < n_jobs; j0 += kMaxJobsPerLaunch) {
        const int nj = std::min(kMaxJobsPerLaunch, n_jobs - j0);
        const SunGridJob* J = jobs + j0;
        const dim3 eg((unsigned)((max_n + kElemBlock - 1) / kElemBlock), (unsigned)nj);
        sungrid_size_kernel<<<nj, kSizeBlock, 0, stream>>>(J);
        sungrid_count_kernel<<<eg, kElemBlock, 0, stream>>>(J);
        sungrid_scan_kernel<<<nj, kScanBlock, 0, stream>>>(J);
        sungrid_fill_kernel<<<eg, kElemBlock, 0, stream>>>(J);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace csp
