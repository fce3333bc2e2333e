// csp_noalloc.cu -- csp_trace_noalloc: a trace that allocates no device or host memory (only an
// error return records its message through the library's usual error channel).
//
// Who needs it: callers that cannot call cudaMalloc.  A host framework whose own allocator has
// already reserved the device memory (a caching allocator holding HBM for a whole process) would see
// a library cudaMalloc fail or fragment its pool; a real-time heliostat-tracking loop cannot afford
// the device-wide synchronisation that cudaMalloc/cudaFree may imply.  Such a caller passes its own
// input (the element list and sun) and output buffers, and this entry point keeps its only
// intermediate data -- the packed element records and the sun-plane frame -- in one file-scope
// device array of fixed size instead of library-allocated device memory.
//
// Limits and sharing: at most kNoAllocMaxElements elements (the shared-memory element-list path of
// the trace kernel); the array lives for as long as the library stays loaded, on every device that
// uses it (kNoAllocScratchBytes each).  Every call on a device reuses the same array and overwrites
// it completely before the kernels read it, so nothing carries over from one call to the next; two
// calls whose work overlaps on the GPU (different streams, or different host threads) race on it.
// The first call on a device looks up the array's device address (cudaGetSymbolAddress) with that
// device current; make that first call before any stream capture.  The address is kept for the
// life of the process, so resetting a device (cudaDeviceReset, or anything else that destroys its
// primary context) after that first call is not supported: later calls would use a stale address.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "csp_c_api.h"
#include "csp_kernels.cuh"
#include "csp_math.cuh"
#include "csp_scene.h"
#include "csp_system.h"

namespace csp {
namespace {

constexpr uint32_t kNoAllocMaxElements = 8;
constexpr size_t kOffNodes = 0;
constexpr size_t kOffPrims = kOffNodes + kNoAllocMaxElements * sizeof(Node);
constexpr size_t kOffOptics = kOffPrims + kNoAllocMaxElements * sizeof(Prim);
constexpr size_t kOffAabbs = kOffOptics + kNoAllocMaxElements * sizeof(Optics);
constexpr size_t kOffSun = kOffAabbs + kNoAllocMaxElements * sizeof(Aabb);
constexpr size_t kNoAllocScratchBytes = 4096;
static_assert(kOffSun + sizeof(SunFrame) <= kNoAllocScratchBytes, "scratch layout exceeds the array");
static_assert(kOffSun % 16 == 0, "records must stay 16-byte aligned");

// The only intermediate storage of csp_trace_noalloc (see the file comment).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The packed records travel to the device as a kernel parameter (no staging copy) and this kernel,
// which names the array directly, stores them.
struct alignas(16) RecordBlock {
    unsigned char bytes[kOffSun];
};
static_assert(sizeof(RecordBlock) % 16 == 0 && sizeof(RecordBlock) <= 4096, "record block must fit a parameter");

__global__ void noalloc_upload_kernel(const RecordBlock blk) {
    const int i = threadIdx.x;
    if (i < (int)(sizeof(RecordBlock) / 16))
        reinterpret_cast<uint4*>(g_noalloc_scratch)[i] = reinterpret_cast<const uint4*>(blk.bytes)[i];
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// Device address of the array on `device` (which must be current), looked up once per device.
int scratch_address(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress of the no-allocation scratch array");
        g_scratch_addr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_addr[device];
    return CSP_OK;
}

// Element records of a scene of at most kNoAllocMaxElements elements, packed in the scratch layout
// by the scene builder's own per-element packing (pack_element, the one csp_initialize uses); the
// nodes are the element list itself, one leaf per element in element order.
int pack_records(const csp_element* el, uint32_t n, unsigned char* block) {
    Node* nodes = reinterpret_cast<Node*>(block + kOffNodes);
    Prim* prims = reinterpret_cast<Prim*>(block + kOffPrims);
    Optics* optics = reinterpret_cast<Optics*>(block + kOffOptics);
    Aabb* aabbs = reinterpret_cast<Aabb*>(block + kOffAabbs);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t type = 0;
        const char* why = "";
        if (pack_element(el[i], i + 1 == n, type, aabbs[i], prims[i], optics[i], nullptr, why))
            return set_error(CSP_ERR_BAD_SCENE, std::string("csp_trace_noalloc: element ") + std::to_string(i) + ": " + why);
        const uint32_t hitw = kLeafFlag | (type << kTypeShift) | i;
        const int32_t miss = (i + 1 < n) ? (int32_t)(i + 1) : -1;
        nodes[i].lo = make_float4(aabbs[i].lo.x, aabbs[i].lo.y, aabbs[i].lo.z, u2f(hitw));
        nodes[i].hi = make_float4(aabbs[i].hi.x, aabbs[i].hi.y, aabbs[i].hi.z, u2f((uint32_t)miss));
    }
    return CSP_OK;
}

}  // namespace
}  // namespace csp

extern "C" int csp_trace_noalloc(int device, const csp_element* elements, uint32_t count, const double* sun_dir,
                                 int sun_shape, double sun_param, uint64_t seed, uint32_t instance, uint64_t first_ray,
                                 uint64_t num_rays, void* hits, void* ids, void* stream) {
    using namespace csp;
    if (!elements || !sun_dir) return set_error(CSP_ERR_INVALID_ARGUMENT, "csp_trace_noalloc: null elements or sun");
    if (count == 0 || count > kNoAllocMaxElements)
        return set_error(CSP_ERR_INVALID_ARGUMENT,
                         "csp_trace_noalloc: 1 to 8 elements (its fixed scratch array holds no more); "
                         "use csp_create/csp_initialize for larger scenes");
    if (!hits && num_rays) return set_error(CSP_ERR_INVALID_ARGUMENT, "csp_trace_noalloc: null hit buffer");
    if (!valid_ray_window(first_ray, num_rays))
        return set_error(CSP_ERR_INVALID_ARGUMENT, "csp_trace_noalloc: ray window must stay below 2^56");
    if (!valid_sun_shape(sun_shape))
        return set_error(CSP_ERR_INVALID_ARGUMENT, "csp_trace_noalloc: unknown sun shape");
    if (!(sun_param >= 0.0) || sun_param > 0.5)
        return set_error(CSP_ERR_INVALID_ARGUMENT, "csp_trace_noalloc: sun shape parameter out of range");
    if (device < 0 || device >= kMaxDevices) return set_error(CSP_ERR_INVALID_ARGUMENT, "csp_trace_noalloc: bad device");

    int prev = -1;
    int rc = cuda_status(cudaGetDevice(&prev), "cudaGetDevice");
    if (rc) return rc;
    if (prev != device && (rc = cuda_status(cudaSetDevice(device), "cudaSetDevice"))) return rc;

    unsigned char* scratch = nullptr;
    RecordBlock block;
    std::memset(&block, 0, sizeof block);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (!(rc = scratch_address(device, &scratch)) && !(rc = pack_records(elements, count, block.bytes))) {
        noalloc_upload_kernel<<<1, 128, 0, st>>>(block);
        rc = cuda_status(cudaGetLastError(), "csp_trace_noalloc: record upload");
    }
    if (!rc) {
        float s[3];
        sun_vector_f(sun_dir, s);
        const float pad = (float)sun_pad_angle(sun_shape, sun_param);
        SunFrame* sun = reinterpret_cast<SunFrame*>(scratch + kOffSun);
        rc = cuda_status(launch_prepare_sun(reinterpret_cast<const Aabb*>(scratch + kOffAabbs), (int)count, s[0], s[1],
                                            s[2], tanf(pad), sun_shape, (float)sun_param, sun, st),
                         "csp_trace_noalloc: prepare_sun_kernel");
        if (!rc && num_rays) {
            TraceArgs a;
            a.tile_counter = nullptr;  // static round robin: nothing to allocate
            a.nodes = reinterpret_cast<const Node*>(scratch + kOffNodes);
            a.prims = reinterpret_cast<const Prim*>(scratch + kOffPrims);
            a.optics = reinterpret_cast<const Optics*>(scratch + kOffOptics);
            a.sun = sun;
            a.hits = reinterpret_cast<float4*>(hits);
            a.ids = reinterpret_cast<uint32_t*>(ids);
            a.ray_begin = first_ray;
            a.count = num_rays;
            a.seed = seed;
            a.instance = instance;
            a.pad = 0;
            a.grid = nullptr;
            a.h3t12 = nullptr;
            a.sgrid = nullptr;
            rc = cuda_status(launch_trace(a, (int)count, st), "csp_trace_noalloc: trace_kernel");
        }
    }
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    return rc;
}
