/*
 * ref_driver.cpp -- TEST INFRASTRUCTURE (builds oracle/_ref/libref_host.so).
 *
 * Runs the reference's own device programs (cuda/sun.cu, cuda/intersection.cu, cuda/materials.cu)
 * and its host scene model (lib/element.cpp, lib/Aperture.cpp), compiled on the host from the
 * reference sources in place, under project-written stand-ins for the OptiX SDK (ref_shim/).
 * What this file supplies, each restated from the reference and from OptiX's documented semantics:
 *
 *  - scene collection: lib/geometry_manager.cpp:10-94 (AABB per element, entity type by surface,
 *    last element re-tagged as the receiver) using the reference's Element class itself;
 *  - sun plane: lib/geometry_manager.cpp:97-148 and the two reduction kernels of
 *    lib/sun_utils.cu:53-179, restated as loops (max/min reductions are order independent);
 *  - the OptiX device API: optixTrace visits every primitive whose AABB the ray segment
 *    [tmin, tmax] overlaps (brute force, ascending primitive index), runs the entity type's
 *    intersection program with optixGetRayTmax() = closest hit so far, keeps a report only when
 *    t < that value (so equal-t ties keep the lower index), then runs the closest-hit program, or
 *    the miss program when nothing was reported.  Program table: lib/pipeline_manager.cpp:20-28,
 *    252-268 and lib/soltrace_system.cpp:302-425.
 *
 * Random draws come from the curand_kernel.h stand-in (Philox keyed on seed and instance).
 */
#include "ref_shim/ref_prelude.h"
#include "cuda/Soltrace.h"
#include "lib/element.h"

#include <cfloat>
#include <cstdint>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "orc_detmath.h"

thread_local unsigned long long orc_ref_seed = 0;
thread_local unsigned int orc_ref_instance = 0;

extern "C" {
void __raygen__sun_source();
void __intersection__rectangle_flat();
void __intersection__rectangle_parabolic();
void __intersection__cylinder_y_capped();
void __closesthit__mirror();
void __closesthit__mirror__parabolic();
void __closesthit__receiver();
void __closesthit__receiver__cylinder__y();
void __miss__ms();
void orc_ref_set_params_sun(const soltrace::LaunchParams* p);
void orc_ref_set_params_isect(const soltrace::LaunchParams* p);
void orc_ref_set_params_mat(const soltrace::LaunchParams* p);
}

/* same layout as csp_element / orc_element */
struct ref_element {
    double origin[3];
    double aim_point[3];
    double zrot_deg;
    double width, height;
    double curv_x, curv_y;
    double reflectivity, slope_error, specularity_error;
    int32_t surface, aperture;
};

namespace {

struct Scene {
    std::vector<OptixAabb> aabb;
    std::vector<uint32_t> sbt;
    std::vector<GeometryDataST> geom;
    soltrace::LaunchParams params;
};

Scene g_scene;

struct Frame {
    float3 o, d;
    float tmin, tmax_launch, tmax;
    unsigned int prim;
    unsigned int payload[2];
    unsigned int cand_attr[5], attr[5];
    bool have_hit;
    unsigned int best_prim;
};

thread_local Frame t_frames[16];
thread_local int t_depth = -1;
thread_local uint3 t_launch;
thread_local uint32_t* t_ids = nullptr; /* per-ray element-id slots, 5 entries */

inline Frame& top() { return t_frames[t_depth]; }

/* NaN-robust slab test, identical to the C oracle's aabb_hit. */
bool aabb_overlap(const OptixAabb& b, float3 o, float3 inv, float tmin, float tmax) {
    const float lo[3] = {b.minX, b.minY, b.minZ}, hi[3] = {b.maxX, b.maxY, b.maxZ};
    const float oo[3] = {o.x, o.y, o.z}, ii[3] = {inv.x, inv.y, inv.z};
    float tn = tmin, tf = tmax;
    for (int a = 0; a < 3; ++a) {
        float t0 = (lo[a] - oo[a]) * ii[a];
        float t1 = (hi[a] - oo[a]) * ii[a];
        tn = fmaxf(tn, fminf(t0, t1));
        tf = fminf(tf, fmaxf(t0, t1));
    }
    return tn <= tf;
}

int build_scene(const ref_element* el, uint32_t n, const double sun_dir[3], double sun_angle, char* err) {
    Scene& S = g_scene;
    S.aabb.assign(n, OptixAabb{});
    S.sbt.assign(n, 0);
    S.geom.assign(n, GeometryDataST());
    std::vector<std::shared_ptr<Element>> elements;
    for (uint32_t i = 0; i < n; ++i) {
        const ref_element& r = el[i];
        if (r.aperture != 0) { std::snprintf(err, 256, "only rectangle apertures"); return -1; }
        auto e = std::make_shared<Element>();
        e->set_origin(Vector3d(r.origin[0], r.origin[1], r.origin[2]));
        e->set_aim_point(Vector3d(r.aim_point[0], r.aim_point[1], r.aim_point[2]));
        e->set_zrot(r.zrot_deg);
        e->set_aperture(std::make_shared<ApertureRectangle>(r.width, r.height));
        if (r.surface == 0) e->set_surface(std::make_shared<SurfaceFlat>());
        else if (r.surface == 1) {
            auto s = std::make_shared<SurfaceParabolic>();
            s->set_curvature(r.curv_x, r.curv_y);
            e->set_surface(s);
        } else if (r.surface == 3) {
            auto s = std::make_shared<SurfaceCylinder>();
            s->set_radius(r.width / 2);
            s->set_half_height(r.height / 2);
            e->set_surface(s);
        } else { std::snprintf(err, 256, "unknown surface"); return -1; }
        e->update_euler_angles(); /* SolTraceSystem::add_element, lib/soltrace_system.cpp:427-433 */
        elements.push_back(e);
    }
    for (uint32_t i = 0; i < n; ++i) {
        auto& e = elements[i];
        e->compute_bounding_box();
        OptixAabb b;
        b.minX = (float)(e->get_lower_bounding_box()[0]);
        b.minY = (float)(e->get_lower_bounding_box()[1]);
        b.minZ = (float)(e->get_lower_bounding_box()[2]);
        b.maxX = (float)(e->get_upper_bounding_box()[0]);
        b.maxY = (float)(e->get_upper_bounding_box()[1]);
        b.maxZ = (float)(e->get_upper_bounding_box()[2]);
        S.aabb[i] = b;
        uint32_t sbt = 0;
        if (e->get_surface_type() == SurfaceType::PARABOLIC) sbt = soltrace::RECTANGLE_PARABOLIC_MIRROR;
        else if (e->get_surface_type() == SurfaceType::FLAT) sbt = soltrace::RECTANGLE_FLAT_MIRROR;
        else if (i + 1 != n) { std::snprintf(err, 256, "cylinder only as receiver"); return -1; }
        S.sbt[i] = sbt;
        S.geom[i] = e->toDeviceGeometryData();
    }
    auto recv = elements[n - 1];
    if (recv->get_surface_type() == SurfaceType::FLAT) S.sbt[n - 1] = soltrace::RECTANGLE_FLAT_RECEIVER;
    else if (recv->get_surface_type() == SurfaceType::CYLINDER) S.sbt[n - 1] = soltrace::CYLINDRICAL_RECEIVER;

    /* SolTraceSystem::initialize, lib/soltrace_system.cpp:81-85 */
    Vector3d sv = Vector3d(sun_dir[0], sun_dir[1], sun_dir[2]).normalized();
    soltrace::LaunchParams& P = S.params;
    std::memset(&P, 0, sizeof(P));
    P.sun_vector = mathUtil::toFloat3(sv);
    P.max_sun_angle = (float)sun_angle;

    /* compute_sun_plane_H + kernels */
    const float3 s = P.sun_vector;
    float d = 0.0f;
    for (const OptixAabb& b : S.aabb) {
        const float3 c[8] = {make_float3(b.minX, b.minY, b.minZ), make_float3(b.maxX, b.minY, b.minZ),
                             make_float3(b.minX, b.maxY, b.minZ), make_float3(b.maxX, b.maxY, b.minZ),
                             make_float3(b.minX, b.minY, b.maxZ), make_float3(b.maxX, b.minY, b.maxZ),
                             make_float3(b.minX, b.maxY, b.maxZ), make_float3(b.maxX, b.maxY, b.maxZ)};
        float md = 0.0f;
        for (int k = 0; k < 8; ++k) md = fmaxf(md, fabsf(dot(c[k], s)));
        d = fmaxf(d, md);
    }
    float3 axis = (fabsf(s.x) < 0.9f) ? make_float3(1.0f, 0.0f, 0.0f) : make_float3(0.0f, 1.0f, 0.0f);
    float3 su = normalize(cross(axis, s));
    float3 sv3 = normalize(cross(s, su));
    const float tan_a = tanf(P.max_sun_angle);
    float umin = FLT_MAX, umax = -FLT_MAX, vmin = FLT_MAX, vmax = -FLT_MAX;
    for (const OptixAabb& b : S.aabb) {
        const float3 c[8] = {make_float3(b.minX, b.minY, b.minZ), make_float3(b.maxX, b.minY, b.minZ),
                             make_float3(b.minX, b.maxY, b.minZ), make_float3(b.maxX, b.maxY, b.minZ),
                             make_float3(b.minX, b.minY, b.maxZ), make_float3(b.maxX, b.minY, b.maxZ),
                             make_float3(b.minX, b.maxY, b.maxZ), make_float3(b.maxX, b.maxY, b.maxZ)};
        float3 pc = d * s;
        for (int k = 0; k < 8; ++k) {
            float3 pt = c[k];
            float dist = fabsf(dot(pt, s));
            float buf = dist * tan_a;
            float3 proj = pt - dot(pt - pc, s) * s;
            float u = dot(proj, su), v = dot(proj, sv3);
            umin = fminf(umin, u - buf);
            umax = fmaxf(umax, u + buf);
            vmin = fminf(vmin, v - buf);
            vmax = fmaxf(vmax, v + buf);
        }
    }
    P.sun_v0 = umin * su + vmin * sv3 + d * s;
    P.sun_v1 = umax * su + vmin * sv3 + d * s;
    P.sun_v2 = umax * su + vmax * sv3 + d * s;
    P.sun_v3 = umin * su + vmax * sv3 + d * s;
    P.height = 1;
    P.max_depth = soltrace::MAX_TRACE_DEPTH;
    P.handle = 1;
    P.geometry_data_array = S.geom.data();
    return 0;
}

void call_is(uint32_t type) {
    if (type == soltrace::RECTANGLE_PARABOLIC_MIRROR) __intersection__rectangle_parabolic();
    else if (type == soltrace::CYLINDRICAL_RECEIVER) __intersection__cylinder_y_capped();
    else __intersection__rectangle_flat();
}

void call_ch(uint32_t type) {
    switch (type) {
        case soltrace::RECTANGLE_FLAT_MIRROR: __closesthit__mirror(); break;
        case soltrace::RECTANGLE_PARABOLIC_MIRROR: __closesthit__mirror__parabolic(); break;
        case soltrace::RECTANGLE_FLAT_RECEIVER: __closesthit__receiver(); break;
        default: __closesthit__receiver__cylinder__y(); break;
    }
}

} // namespace

/* ------------------------------------------------------------ OptiX device API stand-ins ---- */
uint3 optixGetLaunchIndex() { return t_launch; }
uint3 optixGetLaunchDimensions() { return make_uint3(g_scene.params.width, 1, 1); }
float3 optixGetWorldRayOrigin() { return top().o; }
float3 optixGetWorldRayDirection() { return top().d; }
float optixGetRayTmin() { return top().tmin; }
float optixGetRayTmax() { return top().tmax; }
unsigned int optixGetPrimitiveIndex() { return top().prim; }
unsigned int optixGetPayload_0() { return top().payload[0]; }
unsigned int optixGetPayload_1() { return top().payload[1]; }
void optixSetPayload_0(unsigned int p) { top().payload[0] = p; }
void optixSetPayload_1(unsigned int p) { top().payload[1] = p; }
unsigned int optixGetAttribute_0() { return top().attr[0]; }
unsigned int optixGetAttribute_1() { return top().attr[1]; }
unsigned int optixGetAttribute_2() { return top().attr[2]; }
unsigned int optixGetAttribute_3() { return top().attr[3]; }
unsigned int optixGetAttribute_4() { return top().attr[4]; }
float3 optixTransformNormalFromObjectToWorldSpace(float3 n) { return n; } /* GAS traced directly */

bool optixReportIntersection(float t, unsigned int, unsigned int a0, unsigned int a1, unsigned int a2,
                             unsigned int a3, unsigned int a4) {
    Frame& f = top();
    if (!(t >= f.tmin && t < f.tmax)) return false;
    f.tmax = t;
    f.have_hit = true;
    f.best_prim = f.prim;
    f.cand_attr[0] = a0; f.cand_attr[1] = a1; f.cand_attr[2] = a2; f.cand_attr[3] = a3; f.cand_attr[4] = a4;
    return true;
}

void optixTrace(OptixTraversableHandle, float3 o, float3 d, float tmin, float tmax, float, OptixVisibilityMask,
                unsigned int, unsigned int, unsigned int, unsigned int, unsigned int& p0, unsigned int& p1) {
    ++t_depth;
    Frame& f = top();
    f.o = o;
    f.d = d;
    f.tmin = tmin;
    f.tmax_launch = tmax;
    f.tmax = tmax;
    f.payload[0] = p0;
    f.payload[1] = p1;
    f.have_hit = false;
    const float3 inv = make_float3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    const uint32_t n = (uint32_t)g_scene.aabb.size();
    for (uint32_t k = 0; k < n; ++k) {
        if (!aabb_overlap(g_scene.aabb[k], o, inv, tmin, tmax)) continue;
        f.prim = k;
        call_is(g_scene.sbt[k]);
    }
    if (f.have_hit) {
        f.prim = f.best_prim;
        for (int a = 0; a < 5; ++a) f.attr[a] = f.cand_attr[a];
        const unsigned int slot = f.payload[1] + 1;
        call_ch(g_scene.sbt[f.best_prim]);
        if (t_ids && slot < (unsigned)soltrace::MAX_TRACE_DEPTH) {
            const float4& h = g_scene.params.hit_point_buffer[g_scene.params.max_depth * t_launch.x + slot];
            if (h.x != 0.0f && t_ids[slot] == 0xFFFFFFFFu) t_ids[slot] = f.best_prim;
        }
    } else {
        __miss__ms();
    }
    p0 = f.payload[0];
    p1 = f.payload[1];
    --t_depth;
}

/* ------------------------------------------------------------ exported driver --------------- */
static char g_err[256];
extern "C" __attribute__((visibility("default"))) const char* ref_last_error(void) { return g_err; }

/* Trace rays [first, first + count) with the reference's programs.  Pillbox sun only (the only
 * shape the reference implements); no slope error, no reflectivity.  Output layout as orc_trace. */
extern "C" __attribute__((visibility("default"))) int ref_trace(const ref_element* el, uint32_t n,
                                                                const double sun_dir[3], double sun_angle,
                                                                uint64_t first, uint64_t count, uint64_t seed,
                                                                uint32_t instance, double* hits, uint32_t* ids,
                                                                int nthreads) {
    if (n == 0) { std::snprintf(g_err, sizeof g_err, "no elements"); return -1; }
    if (first + count > (1ull << 31) / soltrace::MAX_TRACE_DEPTH) {
        std::snprintf(g_err, sizeof g_err, "ray index beyond the reference's 32-bit hit-buffer index");
        return -1;
    }
    if (build_scene(el, n, sun_dir, sun_angle, g_err)) return -1;
    const int D = soltrace::MAX_TRACE_DEPTH;
    std::vector<float4> buf((size_t)count * D);
    std::memset(buf.data(), 0, buf.size() * sizeof(float4));
    soltrace::LaunchParams P = g_scene.params;
    P.width = (unsigned)(first + count);
    /* the programs index hit_point_buffer[max_depth * ray + slot]; shift the base so ray `first`
     * lands on element 0 of the local buffer */
    P.hit_point_buffer = reinterpret_cast<float4*>(reinterpret_cast<uintptr_t>(buf.data()) -
                                                   (uintptr_t)(first * D * sizeof(float4)));
    g_scene.params = P;
    orc_ref_set_params_sun(&P);
    orc_ref_set_params_isect(&P);
    orc_ref_set_params_mat(&P);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 512)
#endif
    for (int64_t k = 0; k < (int64_t)count; ++k) {
        orc_ref_seed = seed;
        orc_ref_instance = instance;
        uint32_t local_ids[16];
        for (int s = 0; s < D; ++s) local_ids[s] = 0xFFFFFFFFu;
        t_ids = local_ids;
        t_depth = -1;
        t_launch = make_uint3((unsigned)(first + (uint64_t)k), 0, 0);
        __raygen__sun_source();
        t_ids = nullptr;
        for (int s = 0; s < D; ++s) {
            const float4& h = buf[(size_t)k * D + s];
            double* o = hits + ((size_t)k * D + s) * 4;
            o[0] = h.x; o[1] = h.y; o[2] = h.z; o[3] = h.w;
            if (ids) ids[(size_t)k * D + s] = local_ids[s];
        }
    }
    return 0;
}

/* Scene introspection, same layout as orc_scene_info. */
extern "C" __attribute__((visibility("default"))) int ref_scene_info(const ref_element* el, uint32_t n,
                                                                     const double sun_dir[3], double sun_angle,
                                                                     double* prim_out, double* sun_out) {
    if (n == 0) return -1;
    if (build_scene(el, n, sun_dir, sun_angle, g_err)) return -1;
    for (uint32_t i = 0; i < n; ++i) {
        double* o = prim_out + 32 * i;
        std::memset(o, 0, 32 * sizeof(double));
        const uint32_t t = g_scene.sbt[i];
        o[0] = t;
        const OptixAabb& b = g_scene.aabb[i];
        o[1] = b.minX; o[2] = b.minY; o[3] = b.minZ; o[4] = b.maxX; o[5] = b.maxY; o[6] = b.maxZ;
        double* g = o + 7;
        const GeometryDataST& G = g_scene.geom[i];
        if (t == soltrace::RECTANGLE_FLAT_MIRROR || t == soltrace::RECTANGLE_FLAT_RECEIVER) {
            const auto& r = G.getRectangle_Flat();
            const float v[16] = {r.plane.x, r.plane.y, r.plane.z, r.plane.w, r.center.x, r.center.y, r.center.z,
                                 r.x.x, r.x.y, r.x.z, r.y.x, r.y.y, r.y.z, r.width, r.height, 0};
            for (int k = 0; k < 16; ++k) g[k] = v[k];
        } else if (t == soltrace::RECTANGLE_PARABOLIC_MIRROR) {
            const auto& r = G.getRectangleParabolic();
            const float v[16] = {r.v1.x, r.v1.y, r.v1.z, r.v2.x, r.v2.y, r.v2.z, r.anchor.x, r.anchor.y,
                                 r.anchor.z, r.curv_x, r.curv_y, 0, 0, 0, 0, 0};
            for (int k = 0; k < 16; ++k) g[k] = v[k];
        } else {
            const auto& r = G.getCylinder_Y();
            const float v[16] = {r.center.x, r.center.y, r.center.z, r.radius, r.half_height, r.base_x.x,
                                 r.base_x.y, r.base_x.z, r.base_z.x, r.base_z.y, r.base_z.z, 0, 0, 0, 0, 0};
            for (int k = 0; k < 16; ++k) g[k] = v[k];
        }
    }
    const soltrace::LaunchParams& P = g_scene.params;
    const float sv[16] = {P.sun_vector.x, P.sun_vector.y, P.sun_vector.z, P.sun_v0.x, P.sun_v0.y, P.sun_v0.z,
                          P.sun_v1.x, P.sun_v1.y, P.sun_v1.z, P.sun_v2.x, P.sun_v2.y, P.sun_v2.z,
                          P.sun_v3.x, P.sun_v3.y, P.sun_v3.z, 0};
    for (int k = 0; k < 15; ++k) sun_out[k] = sv[k];
    return 0;
}
