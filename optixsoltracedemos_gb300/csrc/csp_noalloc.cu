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
// device current; make that first call before any stream capture.
#include <cmath>
#include <cstring>
#include <mutex>

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

inline float3 f3d(double x, double y, double z) { return make_float3((float)x, (float)y, (float)z); }

// Element records of a scene of at most kNoAllocMaxElements elements, packed in the scratch layout,
// with the same arithmetic as the scene builder used by csp_initialize (entity types of
// lib/geometry_manager.cpp:50-90, geometry of lib/element.cpp:114-164 and the GeometryDataST
// constructors); the nodes are the element list itself, one leaf per element in element order.
int pack_records(const csp_element* el, uint32_t n, unsigned char* block) {
    Node* nodes = reinterpret_cast<Node*>(block + kOffNodes);
    Prim* prims = reinterpret_cast<Prim*>(block + kOffPrims);
    Optics* optics = reinterpret_cast<Optics*>(block + kOffOptics);
    Aabb* aabbs = reinterpret_cast<Aabb*>(block + kOffAabbs);
    for (uint32_t i = 0; i < n; ++i) {
        const csp_element& e = el[i];
        const bool last = (i + 1 == n);
        if (e.aperture != CSP_APERTURE_RECTANGLE || !(e.width > 0) || !(e.height > 0))
            return set_error(CSP_ERR_BAD_SCENE, "csp_trace_noalloc: elements need a rectangular aperture of positive size");
        uint32_t type;
        if (e.surface == CSP_SURFACE_FLAT) type = last ? kFlatReceiver : kFlatMirror;
        else if (e.surface == CSP_SURFACE_PARABOLIC) type = kParabolicMirror;
        else if (e.surface == CSP_SURFACE_CYLINDER && last) type = kCylReceiver;
        else return set_error(CSP_ERR_BAD_SCENE, "csp_trace_noalloc: unsupported surface, or a cylinder that is not last");
        double G[9], euler[3], lo[3], hi[3];
        element_frame(e, euler, G, lo, hi);
        const double w = e.width, h = e.height;
        Aabb& box = aabbs[i];
        box.lo = make_float4((float)lo[0], (float)lo[1], (float)lo[2], 0.f);
        box.hi = make_float4((float)hi[0], (float)hi[1], (float)hi[2], 0.f);
        Prim& p = prims[i];
        if (e.surface == CSP_SURFACE_FLAT) {
            const float3 center = f3d(e.origin[0], e.origin[1], e.origin[2]);
            const float3 x = f3d(G[0], G[1], G[2]), y = f3d(G[3], G[4], G[5]);
            const float fw = (float)w, fh = (float)h;
            const float3 nrm = normalize(cross(x, y));
            const float pw = dot(nrm, center);
            p.a = make_float4(nrm.x, nrm.y, nrm.z, pw);
            p.b = make_float4(center.x, center.y, center.z, fw / 2);
            p.c = make_float4(x.x, x.y, x.z, fh / 2);
            p.d = make_float4(y.x, y.y, y.z, 0.f);
        } else if (e.surface == CSP_SURFACE_PARABOLIC) {
            const double sw = (double)(float)(-w), sh = (double)(float)h;
            const double v1[3] = {G[0] * sw, G[1] * sw, G[2] * sw}, v2[3] = {G[3] * sh, G[4] * sh, G[5] * sh};
            float3 fv1 = f3d(v1[0], v1[1], v1[2]), fv2 = f3d(v2[0], v2[1], v2[2]);
            const float3 anchor = f3d(e.origin[0] - v1[0] * 0.5 - v2[0] * 0.5, e.origin[1] - v1[1] * 0.5 - v2[1] * 0.5,
                                      e.origin[2] - v1[2] * 0.5 - v2[2] * 0.5);
            const float i1 = 1.0f / dot(fv1, fv1), i2 = 1.0f / dot(fv2, fv2);
            fv1 = make_float3(fv1.x * i1, fv1.y * i1, fv1.z * i1);
            fv2 = make_float3(fv2.x * i2, fv2.y * i2, fv2.z * i2);
            const float L1 = 1.0f / length(fv1), L2 = 1.0f / length(fv2);
            const float3 e1 = scale(L1, fv1), e2 = scale(L2, fv2);
            const float3 nn = normalize(cross(e2, e1));
            const float3 rc = add(add(anchor, scale(L1 / 2.0f, e1)), scale(L2 / 2.0f, e2));
            p.a = make_float4(e1.x, e1.y, e1.z, L1 / 2.0f);
            p.b = make_float4(e2.x, e2.y, e2.z, L2 / 2.0f);
            p.c = make_float4(nn.x, nn.y, nn.z, (float)e.curv_x);
            p.d = make_float4(rc.x, rc.y, rc.z, (float)e.curv_y);
        } else {
            const float radius = (float)w / 2.0f, half = (float)h / 2.0f;
            const float3 center = f3d(e.origin[0], e.origin[1], e.origin[2]);
            const float3 bx = f3d(G[0], G[1], G[2]), bz = f3d(G[6], G[7], G[8]);
            const float3 ly = cross(bz, bx);
            p.a = make_float4(center.x, center.y, center.z, radius);
            p.b = make_float4(bx.x, bx.y, bx.z, half);
            p.c = make_float4(ly.x, ly.y, ly.z, radius * radius);
            p.d = make_float4(bz.x, bz.y, bz.z, 0.f);
        }
        Optics& o = optics[i];
        o.reflectivity = (float)e.reflectivity;
        o.slope = (float)e.slope_error;
        o.spec = (float)e.specularity_error;
        o.pad = 0.f;
        const uint32_t hitw = kLeafFlag | (type << kTypeShift) | i;
        const int32_t miss = (i + 1 < n) ? (int32_t)(i + 1) : -1;
        nodes[i].lo = make_float4(box.lo.x, box.lo.y, box.lo.z, u2f(hitw));
        nodes[i].hi = make_float4(box.hi.x, box.hi.y, box.hi.z, u2f((uint32_t)miss));
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
    if (sun_shape != CSP_SUN_PILLBOX && sun_shape != CSP_SUN_GAUSSIAN)
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
        const float pad = (float)(sun_shape == CSP_SUN_GAUSSIAN ? 5.0 * sun_param : sun_param);
        SunFrame* sun = reinterpret_cast<SunFrame*>(scratch + kOffSun);
        rc = cuda_status(launch_prepare_sun(reinterpret_cast<const Aabb*>(scratch + kOffAabbs), (int)count, s[0], s[1],
                                            s[2], tanf(pad), sun_shape, (float)sun_param, sun, st),
                         "csp_trace_noalloc: prepare_sun_kernel");
        if (!rc && num_rays) {
            TraceArgs a;
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
            rc = cuda_status(launch_trace(a, (int)count, st), "csp_trace_noalloc: trace_kernel");
        }
    }
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    return rc;
}
