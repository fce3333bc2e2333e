// csp_scene.cpp -- host scene model.  Compiled with -ffp-contract=off: the double and float
// arithmetic below must round exactly as written to reproduce the reference's device geometry.
#include "csp_scene.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <numeric>

#include "csp_math.cuh"

namespace csp {
namespace {

struct D3 {
    double x, y, z;
};

inline float3 tof3(const D3& v) { return make_float3((float)v.x, (float)v.y, (float)v.z); }

// Element orientation: lib/element.cpp:77-93 (normal = aim - origin), lib/math_util.h:21-32
// (yaw = atan2(nx, nz), pitch = asin(ny), roll = zrot in radians) and lib/math_util.h:41-59
// (global-to-local matrix, Spencer & Murty).  Returns G2L row-major; the local x, y, z axes in
// world space are its rows (the columns of L2G = G2L^T, lib/vector3d.h:151-159).
void global_to_local(const csp_element& e, double G[9], double* euler = nullptr) {
    double n[3] = {e.aim_point[0] - e.origin[0], e.aim_point[1] - e.origin[1], e.aim_point[2] - e.origin[2]};
    const double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (len > 0) {
        n[0] = n[0] / len;
        n[1] = n[1] / len;
        n[2] = n[2] / len;
    } else {
        n[0] = n[1] = n[2] = 0.0;
    }
    const double alpha = std::atan2(n[0], n[2]);
    const double beta = std::asin(n[1]);
    const double gamma = e.zrot_deg * M_PI / 180.0;
    if (euler) {
        euler[0] = alpha;
        euler[1] = beta;
        euler[2] = gamma;
    }
    const double ca = std::cos(alpha), sa = std::sin(alpha);
    const double cb = std::cos(beta), sb = std::sin(beta);
    const double cg = std::cos(gamma), sg = std::sin(gamma);
    G[0] = ca * cg + sa * sb * sg;
    G[1] = -cb * sg;
    G[2] = -sa * cg + ca * sb * sg;
    G[3] = ca * sg - sa * sb * cg;
    G[4] = cb * cg;
    G[5] = -sa * sg - ca * sb * cg;
    G[6] = sa * cb;
    G[7] = sb;
    G[8] = ca * cb;
}

// L2G * v + origin (Matrix33d * Vector3d, lib/vector3d.h:113-119, then + origin)
D3 to_world(const double G[9], const double v[3], const double o[3]) {
    return D3{G[0] * v[0] + G[3] * v[1] + G[6] * v[2] + o[0], G[1] * v[0] + G[4] * v[1] + G[7] * v[2] + o[1],
              G[2] * v[0] + G[5] * v[1] + G[8] * v[2] + o[2]};
}

void box_init(Aabb& b) {
    b.lo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f);
    b.hi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
}
void box_grow(Aabb& b, const Aabb& o) {
    b.lo.x = std::min(b.lo.x, o.lo.x);
    b.lo.y = std::min(b.lo.y, o.lo.y);
    b.lo.z = std::min(b.lo.z, o.lo.z);
    b.hi.x = std::max(b.hi.x, o.hi.x);
    b.hi.y = std::max(b.hi.y, o.hi.y);
    b.hi.z = std::max(b.hi.z, o.hi.z);
}

// Round a double box outwards to float and widen it by a margin that covers float rounding of
// the intersection arithmetic (1e-5 relative to the coordinate magnitude, plus 1 mm).
Aabb outward(const double lo[3], const double hi[3]) {
    double m = 0;
    for (int a = 0; a < 3; ++a) m = std::max(m, std::max(std::fabs(lo[a]), std::fabs(hi[a])));
    const double pad = 1e-5 * m + 1e-3;
    Aabb b;
    b.lo = make_float4(std::nextafter((float)(lo[0] - pad), -FLT_MAX), std::nextafter((float)(lo[1] - pad), -FLT_MAX),
                       std::nextafter((float)(lo[2] - pad), -FLT_MAX), 0.f);
    b.hi = make_float4(std::nextafter((float)(hi[0] + pad), FLT_MAX), std::nextafter((float)(hi[1] + pad), FLT_MAX),
                       std::nextafter((float)(hi[2] + pad), FLT_MAX), 0.f);
    return b;
}

}  // namespace

void element_frame(const csp_element& e, double euler[3], double G[9], double lo[3], double hi[3]) {
    global_to_local(e, G, euler);
    const double w = e.width, h = e.height;
    if (e.surface != CSP_SURFACE_CYLINDER) {
        const double c[4][3] = {{-w / 2, -h / 2, 0.0}, {w / 2, -h / 2, 0.0}, {w / 2, h / 2, 0.0}, {-w / 2, h / 2, 0.0}};
        D3 g[4];
        for (int k = 0; k < 4; ++k) g[k] = to_world(G, c[k], e.origin);
        lo[0] = std::fmin(std::fmin(g[0].x, g[1].x), std::fmin(g[2].x, g[3].x));
        lo[1] = std::fmin(std::fmin(g[0].y, g[1].y), std::fmin(g[2].y, g[3].y));
        lo[2] = std::fmin(std::fmin(g[0].z, g[1].z), std::fmin(g[2].z, g[3].z));
        hi[0] = std::fmax(std::fmax(g[0].x, g[1].x), std::fmax(g[2].x, g[3].x));
        hi[1] = std::fmax(std::fmax(g[0].y, g[1].y), std::fmax(g[2].y, g[3].y));
        hi[2] = std::fmax(std::fmax(g[0].z, g[1].z), std::fmax(g[2].z, g[3].z));
    } else {
        lo[0] = lo[1] = lo[2] = DBL_MAX;
        hi[0] = hi[1] = hi[2] = -DBL_MAX;
        for (int k = 0; k < 8; ++k) {
            const double c[3] = {(k & 1) ? w / 2 : -w / 2, (k & 2) ? h / 2 : -h / 2, (k & 4) ? w / 2 : -w / 2};
            const D3 g = to_world(G, c, e.origin);
            lo[0] = std::fmin(lo[0], g.x);
            lo[1] = std::fmin(lo[1], g.y);
            lo[2] = std::fmin(lo[2], g.z);
            hi[0] = std::fmax(hi[0], g.x);
            hi[1] = std::fmax(hi[1], g.y);
            hi[2] = std::fmax(hi[2], g.z);
        }
    }
}

void flux_target(const csp_element& rcv, uint32_t nx, uint32_t ny, FluxTarget& F) {
    double euler[3], G[9], lo[3], hi[3];
    element_frame(rcv, euler, G, lo, hi);
    F = FluxTarget{};
    F.o = make_float4((float)rcv.origin[0], (float)rcv.origin[1], (float)rcv.origin[2], 0.f);
    F.x = make_float4((float)G[0], (float)G[1], (float)G[2], 0.f);
    F.y = make_float4((float)G[3], (float)G[4], (float)G[5], 0.f);
    F.z = make_float4((float)G[6], (float)G[7], (float)G[8], 0.f);
    F.nx = (int)nx;
    F.ny = (int)ny;
    const double w = rcv.width, h = rcv.height;
    F.hy = (float)(h / 2.0);
    F.ky = (float)((double)ny / h);
    if (rcv.surface == CSP_SURFACE_CYLINDER) {
        const double r = w / 2.0, half = h / 2.0;
        F.kind = kFluxCylinder;
        F.hx = 0.f;
        F.kx = (float)((double)nx / (2.0 * M_PI));
        F.keep = (float)(half - 1e-4 * std::max(half, r));
    } else {
        F.kind = kFluxFlat;
        F.hx = (float)(w / 2.0);
        F.kx = (float)((double)nx / w);
        F.keep = FLT_MAX;
    }
}

double flux_bin_area(const csp_element& rcv, uint32_t nx, uint32_t ny) {
    const double w = rcv.width, h = rcv.height;
    if (rcv.surface == CSP_SURFACE_CYLINDER) return (2.0 * M_PI * (w / 2.0) / nx) * (h / ny);
    return (w / nx) * (h / ny);
}

void sun_vector_f(const double d[3], float out[3]) {
    const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double n[3] = {0, 0, 0};
    if (len > 0) {
        n[0] = d[0] / len;
        n[1] = d[1] / len;
        n[2] = d[2] / len;
    }
    out[0] = (float)n[0];
    out[1] = (float)n[1];
    out[2] = (float)n[2];
}

int pack_element(const csp_element& e, bool last, uint32_t& type, Aabb& box, Prim& p, Optics& o, Aabb* prune,
                 const char*& why) {
    if (e.aperture != CSP_APERTURE_RECTANGLE) {
        why = "only rectangular apertures are supported";
        return CSP_ERR_BAD_SCENE;
    }
    if (!(e.width > 0) || !(e.height > 0)) {
        why = "aperture dimensions must be positive";
        return CSP_ERR_BAD_SCENE;
    }
    // entity type: lib/geometry_manager.cpp:50-59 (mirrors), :78-90 (last element = receiver)
    if (e.surface == CSP_SURFACE_FLAT) type = last ? kFlatReceiver : kFlatMirror;
    else if (e.surface == CSP_SURFACE_PARABOLIC) type = kParabolicMirror;  // a parabolic last element stays a mirror
    else if (e.surface == CSP_SURFACE_CYLINDER) {
        if (!last) {
            why = "a cylinder is only supported as the receiver (last element)";
            return CSP_ERR_BAD_SCENE;
        }
        type = kCylReceiver;
    } else {
        why = "unknown surface type";
        return CSP_ERR_BAD_SCENE;
    }

    double G[9], euler[3], lo[3], hi[3];
    element_frame(e, euler, G, lo, hi);
    const double w = e.width, h = e.height;
    box.lo = make_float4((float)lo[0], (float)lo[1], (float)lo[2], 0.f);
    box.hi = make_float4((float)hi[0], (float)hi[1], (float)hi[2], 0.f);

    // device geometry: lib/element.cpp:114-164 and the GeometryDataST constructors
    const D3 xb{G[0], G[1], G[2]}, yb{G[3], G[4], G[5]}, zb{G[6], G[7], G[8]};
    double plo[3] = {lo[0], lo[1], lo[2]}, phi[3] = {hi[0], hi[1], hi[2]};
    if (e.surface == CSP_SURFACE_FLAT) {
        const float3 center = tof3(D3{e.origin[0], e.origin[1], e.origin[2]});
        const float3 x = tof3(xb), y = tof3(yb);
        const float fw = (float)w, fh = (float)h;
        const float3 nrm = normalize(cross(x, y));
        const float pw = dot(nrm, center);
        p.a = make_float4(nrm.x, nrm.y, nrm.z, pw);
        p.b = make_float4(center.x, center.y, center.z, fw / 2);
        p.c = make_float4(x.x, x.y, x.z, fh / 2);
        p.d = make_float4(y.x, y.y, y.z, 0.f);
    } else if (e.surface == CSP_SURFACE_PARABOLIC) {
        const double sw = (double)(float)(-w), sh = (double)(float)h;
        const D3 v1{xb.x * sw, xb.y * sw, xb.z * sw}, v2{yb.x * sh, yb.y * sh, yb.z * sh};
        const D3 an{e.origin[0] - v1.x * 0.5 - v2.x * 0.5, e.origin[1] - v1.y * 0.5 - v2.y * 0.5,
                    e.origin[2] - v1.z * 0.5 - v2.z * 0.5};
        float3 fv1 = tof3(v1), fv2 = tof3(v2);
        const float3 anchor = tof3(an);
        const float i1 = 1.0f / dot(fv1, fv1), i2 = 1.0f / dot(fv2, fv2);
        fv1 = make_float3(fv1.x * i1, fv1.y * i1, fv1.z * i1);
        fv2 = make_float3(fv2.x * i2, fv2.y * i2, fv2.z * i2);
        // per-call values of cuda/intersection.cu:335-352
        const float L1 = 1.0f / length(fv1), L2 = 1.0f / length(fv2);
        const float3 e1 = scale(L1, fv1), e2 = scale(L2, fv2);
        const float3 nn = normalize(cross(e2, e1));
        const float3 rc = add(add(anchor, scale(L1 / 2.0f, e1)), scale(L2 / 2.0f, e2));
        const float cx = (float)e.curv_x, cy = (float)e.curv_y;
        p.a = make_float4(e1.x, e1.y, e1.z, L1 / 2.0f);
        p.b = make_float4(e2.x, e2.y, e2.z, L2 / 2.0f);
        p.c = make_float4(nn.x, nn.y, nn.z, cx);
        p.d = make_float4(rc.x, rc.y, rc.z, cy);
        // surface bounds: z = cx/2 x^2 + cy/2 y^2 over |x| <= L1/2, |y| <= L2/2
        const double h1 = L1 / 2.0, h2 = L2 / 2.0;
        const double zx = 0.5 * cx * h1 * h1, zy = 0.5 * cy * h2 * h2;
        const double zmin = std::min(0.0, zx) + std::min(0.0, zy), zmax = std::max(0.0, zx) + std::max(0.0, zy);
        for (int k = 0; k < 8; ++k) {
            const double lx = (k & 1) ? h1 : -h1, ly = (k & 2) ? h2 : -h2, lz = (k & 4) ? zmax : zmin;
            const double P[3] = {rc.x + lx * e1.x + ly * e2.x + lz * nn.x, rc.y + lx * e1.y + ly * e2.y + lz * nn.y,
                                 rc.z + lx * e1.z + ly * e2.z + lz * nn.z};
            for (int a = 0; a < 3; ++a) {
                plo[a] = std::min(plo[a], P[a]);
                phi[a] = std::max(phi[a], P[a]);
            }
        }
    } else {
        const float radius = (float)w / 2.0f, half = (float)h / 2.0f;
        const float3 center = tof3(D3{e.origin[0], e.origin[1], e.origin[2]});
        const float3 bx = tof3(xb), bz = tof3(zb);
        const float3 ly = cross(bz, bx);
        p.a = make_float4(center.x, center.y, center.z, radius);
        p.b = make_float4(bx.x, bx.y, bx.z, half);
        p.c = make_float4(ly.x, ly.y, ly.z, radius * radius);
        p.d = make_float4(bz.x, bz.y, bz.z, 0.f);
    }
    if (prune) *prune = outward(plo, phi);
    o.reflectivity = (float)e.reflectivity;
    o.slope = (float)e.slope_error;
    o.spec = (float)e.specularity_error;
    o.pad = 0.f;
    return CSP_OK;
}

namespace {

int check_count(uint32_t n, std::string& err) {
    if (n == 0) {
        err = "scene has no elements";
        return CSP_ERR_BAD_SCENE;
    }
    if (n > kPrimMask) {
        err = "too many elements";
        return CSP_ERR_BAD_SCENE;
    }
    return CSP_OK;
}

void size_scene(uint32_t n, HostScene& s) {
    s.prims.assign(n, Prim{});
    s.optics.assign(n, Optics{});
    s.aabbs.assign(n, Aabb{});
    s.prune.assign(n, Aabb{});
    s.types.assign(n, 0);
}

// Packs elements [begin, end); returns the index of the first that fails (and its status and
// message), or end.
uint32_t pack_range(const csp_element* el, uint32_t n, uint32_t begin, uint32_t end, HostScene& s, int& rc,
                    const char*& why) {
    for (uint32_t i = begin; i < end; ++i) {
        rc = pack_element(el[i], i + 1 == n, s.types[i], s.aabbs[i], s.prims[i], s.optics[i], &s.prune[i], why);
        // the exact box carries its element and entity type (the sun grid's candidate tests)
        s.aabbs[i].lo.w = u2f((s.types[i] << kTypeShift) | i);
        if (rc) return i;
    }
    return end;
}

int pack_error(const csp_element* el, uint32_t i, int rc, const char* why, std::string& err) {
    err = "element " + std::to_string(i) + ": " + why;
    if (el[i].surface != CSP_SURFACE_FLAT && el[i].surface != CSP_SURFACE_PARABOLIC &&
        el[i].surface != CSP_SURFACE_CYLINDER)
        err += " " + std::to_string(el[i].surface);
    return rc;
}

}  // namespace

int build_elements(const csp_element* el, uint32_t n, HostScene& s, std::string& err) {
    int rc = check_count(n, err);
    if (rc) return rc;
    size_scene(n, s);
    const char* why = "";
    const uint32_t bad = pack_range(el, n, 0, n, s, rc, why);
    return bad < n ? pack_error(el, bad, rc, why, err) : CSP_OK;
}

int build_elements(const csp_element* el, uint32_t n, HostScene& s, std::string& err, const ParallelFor& pf) {
    int rc = check_count(n, err);
    if (rc) return rc;
    size_scene(n, s);
    const size_t chunks = (n + kBuildChunk - 1) / kBuildChunk;
    std::vector<uint32_t> bad(chunks);
    std::vector<int> status(chunks, CSP_OK);
    std::vector<const char*> whys(chunks, "");
    pf(chunks, [&](size_t c) {
        const uint32_t b = (uint32_t)(c * kBuildChunk), e = std::min<uint32_t>(n, b + kBuildChunk);
        bad[c] = pack_range(el, n, b, e, s, status[c], whys[c]);
        if (bad[c] == e) bad[c] = n;
    });
    for (size_t c = 0; c < chunks; ++c)
        if (bad[c] < n) return pack_error(el, bad[c], status[c], whys[c], err);
    return CSP_OK;
}

namespace {

struct BuildNode {
    Aabb box;
    int left = -1, right = -1, prim = -1, size = 1;
};

float area(const Aabb& b) {
    const float dx = b.hi.x - b.lo.x, dy = b.hi.y - b.lo.y, dz = b.hi.z - b.lo.z;
    if (dx < 0 || dy < 0 || dz < 0) return 0.f;
    return 2.f * (dx * dy + dy * dz + dz * dx);
}

struct Builder {
    const std::vector<Aabb>& prune;
    std::vector<BuildNode> nodes;
    std::vector<uint32_t> idx;
    std::vector<float3> cent;

    explicit Builder(const std::vector<Aabb>& p) : prune(p) {
        idx.resize(p.size());
        std::iota(idx.begin(), idx.end(), 0u);
        cent.resize(p.size());
        for (size_t i = 0; i < p.size(); ++i)
            cent[i] = make_float3(0.5f * (p[i].lo.x + p[i].hi.x), 0.5f * (p[i].lo.y + p[i].hi.y),
                                  0.5f * (p[i].lo.z + p[i].hi.z));
    }

    static float comp(const float3& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

    int build(uint32_t begin, uint32_t end) {
        const int me = (int)nodes.size();
        nodes.emplace_back();
        Aabb box;
        box_init(box);
        for (uint32_t i = begin; i < end; ++i) box_grow(box, prune[idx[i]]);
        nodes[me].box = box;
        const uint32_t count = end - begin;
        if (count == 1) {
            nodes[me].prim = (int)idx[begin];
            return me;
        }
        // binned SAH over centroids, all three axes
        float cmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, cmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (uint32_t i = begin; i < end; ++i)
            for (int a = 0; a < 3; ++a) {
                cmin[a] = std::min(cmin[a], comp(cent[idx[i]], a));
                cmax[a] = std::max(cmax[a], comp(cent[idx[i]], a));
            }
        constexpr int B = 16;
        float best_cost = FLT_MAX;
        int best_axis = -1, best_split = -1;
        for (int a = 0; a < 3; ++a) {
            const float ext = cmax[a] - cmin[a];
            if (!(ext > 0)) continue;
            Aabb bb[B];
            int bc[B] = {0};
            for (int k = 0; k < B; ++k) box_init(bb[k]);
            for (uint32_t i = begin; i < end; ++i) {
                int k = (int)((comp(cent[idx[i]], a) - cmin[a]) / ext * B);
                k = std::min(std::max(k, 0), B - 1);
                bc[k]++;
                box_grow(bb[k], prune[idx[i]]);
            }
            float la[B], ra[B];
            int lc[B], rc[B];
            Aabb acc;
            box_init(acc);
            int cnt = 0;
            for (int k = 0; k < B; ++k) {
                box_grow(acc, bb[k]);
                cnt += bc[k];
                la[k] = area(acc);
                lc[k] = cnt;
            }
            box_init(acc);
            cnt = 0;
            for (int k = B - 1; k >= 0; --k) {
                box_grow(acc, bb[k]);
                cnt += bc[k];
                ra[k] = area(acc);
                rc[k] = cnt;
            }
            for (int k = 0; k < B - 1; ++k) {
                if (lc[k] == 0 || rc[k + 1] == 0) continue;
                const float cost = la[k] * lc[k] + ra[k + 1] * rc[k + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = a;
                    best_split = k;
                }
            }
        }
        uint32_t mid;
        if (best_axis < 0) {
            mid = begin + count / 2;  // coincident centroids: split the range in half
        } else {
            const int a = best_axis;
            const float ext = cmax[a] - cmin[a];
            auto it = std::partition(idx.begin() + begin, idx.begin() + end, [&](uint32_t p) {
                int k = (int)((comp(cent[p], a) - cmin[a]) / ext * B);
                k = std::min(std::max(k, 0), B - 1);
                return k <= best_split;
            });
            mid = (uint32_t)(it - idx.begin());
            if (mid == begin || mid == end) mid = begin + count / 2;
        }
        const int l = build(begin, mid);
        const int r = build(mid, end);
        nodes[me].left = l;
        nodes[me].right = r;
        nodes[me].size = 1 + nodes[l].size + nodes[r].size;
        return me;
    }
};

inline int32_t as_i(float f) { return (int32_t)f2u(f); }
inline float as_f(int32_t i) { return u2f((uint32_t)i); }

void emit(const Builder& B, const HostScene& s, int bn, int32_t at, int32_t miss, int32_t par,
          std::vector<Node>& out, std::vector<int32_t>& parent, std::vector<int32_t>& leaf_of) {
    const BuildNode& n = B.nodes[bn];
    parent[at] = par;
    if (n.prim >= 0) {
        const Aabb& a = s.aabbs[n.prim];
        const uint32_t hit = kLeafFlag | (s.types[n.prim] << kTypeShift) | (uint32_t)n.prim;
        out[at].lo = make_float4(a.lo.x, a.lo.y, a.lo.z, as_f((int32_t)hit));
        out[at].hi = make_float4(a.hi.x, a.hi.y, a.hi.z, as_f(miss));
        leaf_of[n.prim] = at;
        return;
    }
    const int32_t left_at = at + 1;
    const int32_t right_at = left_at + B.nodes[n.left].size;
    out[at].lo = make_float4(n.box.lo.x, n.box.lo.y, n.box.lo.z, as_f(left_at));
    out[at].hi = make_float4(n.box.hi.x, n.box.hi.y, n.box.hi.z, as_f(miss));
    emit(B, s, n.left, left_at, right_at, at, out, parent, leaf_of);
    emit(B, s, n.right, right_at, miss, at, out, parent, leaf_of);
}

}  // namespace

void build_bvh(HostScene& s) {
    const uint32_t n = (uint32_t)s.prims.size();
    s.leaf_of.assign(n, -1);
    if (n <= kFlatListMax) {
        s.nodes.assign(n, Node{});
        s.parent.assign(n, -1);
        for (uint32_t i = 0; i < n; ++i) {
            const Aabb& a = s.aabbs[i];
            const uint32_t hit = kLeafFlag | (s.types[i] << kTypeShift) | i;
            const int32_t miss = (i + 1 < n) ? (int32_t)(i + 1) : -1;
            s.nodes[i].lo = make_float4(a.lo.x, a.lo.y, a.lo.z, as_f((int32_t)hit));
            s.nodes[i].hi = make_float4(a.hi.x, a.hi.y, a.hi.z, as_f(miss));
            s.leaf_of[i] = (int32_t)i;
        }
        return;
    }
    Builder B(s.prune);
    const int root = B.build(0, n);
    s.nodes.assign(B.nodes[root].size, Node{});
    s.parent.assign(B.nodes[root].size, -1);
    emit(B, s, root, 0, -1, -1, s.nodes, s.parent, s.leaf_of);
}

void refit_bvh(HostScene& s) {
    const int32_t m = (int32_t)s.nodes.size();
    std::vector<Aabb> box(m);
    for (int32_t i = 0; i < m; ++i) box_init(box[i]);
    for (uint32_t p = 0; p < s.leaf_of.size(); ++p) box[s.leaf_of[p]] = s.prune[p];
    for (int32_t i = m - 1; i >= 0; --i) {
        const uint32_t hit = f2u(s.nodes[i].lo.w);
        if (hit & kLeafFlag) {
            const uint32_t prim = hit & kPrimMask;
            const Aabb& a = s.aabbs[prim];
            s.nodes[i].lo = make_float4(a.lo.x, a.lo.y, a.lo.z, s.nodes[i].lo.w);
            s.nodes[i].hi = make_float4(a.hi.x, a.hi.y, a.hi.z, s.nodes[i].hi.w);
        } else {
            s.nodes[i].lo = make_float4(box[i].lo.x, box[i].lo.y, box[i].lo.z, s.nodes[i].lo.w);
            s.nodes[i].hi = make_float4(box[i].hi.x, box[i].hi.y, box[i].hi.z, s.nodes[i].hi.w);
        }
        if (s.parent[i] >= 0) box_grow(box[s.parent[i]], box[i]);
    }
}

}  // namespace csp

namespace csp {

namespace {

constexpr int kGridMaxCellsPerItem = 64;
constexpr size_t kGridMaxCells = 1u << 22;

}  // namespace

void build_grid(const HostScene& s, HostGrid& g) {
    g = HostGrid{};
    const uint32_t n = (uint32_t)s.prims.size();
    if (n <= kFlatListMax) return;
    // registered xy boxes: pruning box + margin; gridded = every element but the last (receiver)
    std::vector<double> lo(2 * n), hi(2 * n), size(n, 0.0);
    std::vector<uint8_t> gridded(n, 0);
    std::vector<double> sizes;
    for (uint32_t i = 0; i + 1 < n; ++i) {
        const Aabb& b = s.prune[i];
        const double m = 2e-5 * std::max(std::max(std::fabs((double)b.lo.x), std::fabs((double)b.hi.x)),
                                          std::max(std::fabs((double)b.lo.y), std::fabs((double)b.hi.y))) +
                         0.05;
        lo[2 * i] = (double)b.lo.x - m;
        lo[2 * i + 1] = (double)b.lo.y - m;
        hi[2 * i] = (double)b.hi.x + m;
        hi[2 * i + 1] = (double)b.hi.y + m;
        size[i] = std::max(hi[2 * i] - lo[2 * i], hi[2 * i + 1] - lo[2 * i + 1]);
        sizes.push_back(size[i]);
    }
    std::nth_element(sizes.begin(), sizes.begin() + sizes.size() / 2, sizes.end());
    double cell = (double)(float)(1.4 * sizes[sizes.size() / 2]);
    if (!(cell > 0)) return;
    double X0 = DBL_MAX, Y0 = DBL_MAX, X1 = -DBL_MAX, Y1 = -DBL_MAX;
    float zmin = FLT_MAX, zmax = -FLT_MAX;
    for (uint32_t i = 0; i + 1 < n; ++i) {
        if (size[i] > 8.0 * cell) continue;  // oversized: global list
        gridded[i] = 1;
        X0 = std::min(X0, lo[2 * i]);
        Y0 = std::min(Y0, lo[2 * i + 1]);
        X1 = std::max(X1, hi[2 * i]);
        Y1 = std::max(Y1, hi[2 * i + 1]);
        zmin = std::min(zmin, s.prune[i].lo.z);
        zmax = std::max(zmax, s.prune[i].hi.z);
    }
    if (!(X1 > X0) || !(Y1 > Y0)) return;
    if ((double)zmax - (double)zmin > 0.25 * std::max(X1 - X0, Y1 - Y0)) return;  // not a thin layer
    double nxd = std::ceil((X1 - X0) / cell), nyd = std::ceil((Y1 - Y0) / cell);
    while (nxd * nyd > (double)kGridMaxCells) {
        cell = (double)(float)(cell * 1.5);
        nxd = std::ceil((X1 - X0) / cell);
        nyd = std::ceil((Y1 - Y0) / cell);
    }
    g.nx = std::max(1, (int)nxd);
    g.ny = std::max(1, (int)nyd);
    g.x0 = (float)X0;
    g.y0 = (float)Y0;
    g.cell = (float)cell;
    g.inv_cell = 1.0f / g.cell;
    g.x1 = g.x0 + (float)g.nx * g.cell;
    g.y1 = g.y0 + (float)g.ny * g.cell;
    // the float bounds must still cover every registered box
    while ((double)g.x1 < X1 || (double)g.y1 < Y1 || (double)g.x0 > X0 || (double)g.y0 > Y0) {
        g.x0 = std::nextafter(g.x0, -FLT_MAX);
        g.y0 = std::nextafter(g.y0, -FLT_MAX);
        g.x1 = std::nextafter(g.x1, FLT_MAX);
        g.y1 = std::nextafter(g.y1, FLT_MAX);
    }
    // the layer: every gridded surface lies in its pruning box
    const float mz = 1e-5f * std::max(std::fabs(zmin), std::fabs(zmax)) + 0.01f;
    g.zlo = std::nextafter(zmin - mz, -FLT_MAX);
    g.zhi = std::nextafter(zmax + mz, FLT_MAX);
    auto cell_range = [&](uint32_t i, int& ax, int& ay, int& bx, int& by) {
        ax = std::max(0, std::min(g.nx - 1, (int)std::floor((lo[2 * i] - g.x0) / cell)));
        ay = std::max(0, std::min(g.ny - 1, (int)std::floor((lo[2 * i + 1] - g.y0) / cell)));
        bx = std::max(0, std::min(g.nx - 1, (int)std::floor((hi[2 * i] - g.x0) / cell)));
        by = std::max(0, std::min(g.ny - 1, (int)std::floor((hi[2 * i + 1] - g.y0) / cell)));
    };
    std::vector<uint32_t> count((size_t)g.nx * g.ny, 0);
    for (uint32_t i = 0; i + 1 < n; ++i) {
        if (!gridded[i]) continue;
        int ax, ay, bx, by;
        cell_range(i, ax, ay, bx, by);
        if ((bx - ax + 1) * (by - ay + 1) > kGridMaxCellsPerItem) {
            gridded[i] = 0;
            continue;
        }
        for (int y = ay; y <= by; ++y)
            for (int x = ax; x <= bx; ++x) count[(size_t)y * g.nx + x]++;
    }
    g.cell_start.assign((size_t)g.nx * g.ny + 1, 0);
    for (size_t c = 0; c < (size_t)g.nx * g.ny; ++c) g.cell_start[c + 1] = g.cell_start[c] + count[c];
    g.items.assign(g.cell_start.back(), Aabb{});
    std::vector<uint32_t> fill(g.cell_start.begin(), g.cell_start.end() - 1);
    auto item = [&](uint32_t i) {
        Aabb a = s.aabbs[i];
        a.lo.w = u2f((s.types[i] << kTypeShift) | i);
        a.hi.w = 0.f;
        return a;
    };
    for (uint32_t i = 0; i + 1 < n; ++i) {
        if (!gridded[i]) continue;
        int ax, ay, bx, by;
        cell_range(i, ax, ay, bx, by);
        const Aabb a = item(i);
        for (int y = ay; y <= by; ++y)
            for (int x = ax; x <= bx; ++x) g.items[fill[(size_t)y * g.nx + x]++] = a;
    }
    for (uint32_t i = 0; i < n; ++i)
        if (!gridded[i]) g.global.push_back(item(i));
    g.valid = true;
}

GridDesc grid_desc(const HostGrid& g, const uint32_t* cell_start, const Aabb* items, const Aabb* global) {
    GridDesc d{};
    d.x0 = g.x0;
    d.y0 = g.y0;
    d.x1 = g.x1;
    d.y1 = g.y1;
    d.cell = g.cell;
    d.inv_cell = g.inv_cell;
    d.zlo = g.zlo;
    d.zhi = g.zhi;
    d.nx = g.nx;
    d.ny = g.ny;
    d.n_global = (int)g.global.size();
    d.pad = 0;
    d.cell_start = cell_start;
    d.items = items;
    d.global = global;
    d.reserved = nullptr;
    return d;
}

}  // namespace csp
