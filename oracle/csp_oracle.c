/*
 * csp_oracle.c -- TEST INFRASTRUCTURE.  CPU restatement of the reference's hot path, used only as
 * the checker by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.  The product
 * never links, loads or calls it.
 *
 * Compiled twice from this one source:
 *   liboracle_f32.so  (-DORC_REAL=float)  follows the reference's float arithmetic operation by
 *                     operation (no contraction: -ffp-contract=off), so it is bit-comparable with the
 *                     reference's own device programs built on the host (oracle/_ref) and with the
 *                     product's CUDA kernels.
 *   liboracle_f64.so  (-DORC_REAL=double) the FP64 oracle: the same physics in double, used for the
 *                     flux-map L2 accuracy figure.
 *
 * Parity pinning: the reference ships no tests or golden vectors.  This restatement is pinned by
 * comparing it bit-for-bit with the reference's own cuda/sun.cu, cuda/intersection.cu,
 * cuda/materials.cu, lib/element.cpp and lib/Aperture.cpp compiled on the host against project
 * shims for the absent OptiX SDK (oracle/Makefile, target _ref), and by analytic known-answer tests.
 *
 * Reference files followed (paths inside the reference project):
 *   scene setup      lib/element.cpp:77-93 (update_euler_angles), :114-164 (toDeviceGeometryData),
 *                    :172-275 (compute_bounding_box); lib/math_util.h:21-59; lib/vector3d.h:151-159;
 *                    cuda/GeometryDataST.h:41-103 (constructors); lib/geometry_manager.cpp:10-94
 *                    (entity types, receiver = last element)
 *   sun plane        lib/geometry_manager.cpp:97-148; lib/sun_utils.cu:53-179
 *   ray generation   cuda/sun.cu:16-38 (Halton), :72-91 (cone), :94-134 (raygen)
 *   intersection     cuda/intersection.cu:47-85 (flat), :177-296 (capped cylinder),
 *                    :318-448 (parabolic)
 *   closest hit      cuda/materials.cu:26-84 (mirror), :86-121 (flat receiver),
 *                    :123-163 (cylinder receiver), :170-231 (parabolic mirror), :236-253 (miss)
 * Extensions not in the reference (defined here and by the product identically): Gaussian sun,
 * Gaussian slope/specularity error and mirror reflectivity, all drawn from Philox keyed on
 * (instance, ray, bounce).  With sigma = 0 and reflectivity = 1 the trace is the reference's.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "orc_detmath.h"

#ifndef ORC_REAL
#define ORC_REAL float
#endif
typedef ORC_REAL real;
#define IS_F32 (sizeof(real) == sizeof(float))

#define EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------ element input (ABI) ----- */
/* Same memory layout as csp_element in include/csp_c_api.h. */
typedef struct orc_element {
    double origin[3];
    double aim_point[3];
    double zrot_deg;
    double width, height;
    double curv_x, curv_y;
    double reflectivity;
    double slope_error;
    double specularity_error;
    int32_t surface;  /* 0 flat, 1 parabolic, 3 cylinder (lib/soltrace_type.h:10-15) */
    int32_t aperture; /* 0 rectangle, 1 circle */
} orc_element;

enum { SURF_FLAT = 0, SURF_PARABOLIC = 1, SURF_CYLINDER = 3 };
/* OpticalEntityType (cuda/Soltrace.h:24-30) */
enum { ENT_FLAT_MIRROR = 0, ENT_PARABOLIC_MIRROR = 1, ENT_FLAT_RECEIVER = 2, ENT_CYL_RECEIVER = 3 };

/* ------------------------------------------------------------------ vector helpers ---------- */
typedef struct { real x, y, z; } v3;

static inline real rsqrt_(real x) { return IS_F32 ? (real)sqrtf((float)x) : (real)sqrt((double)x); }
static inline real rabs_(real x) { return IS_F32 ? (real)fabsf((float)x) : (real)fabs((double)x); }
static inline real rmin_(real a, real b) { return IS_F32 ? (real)fminf((float)a, (float)b) : (real)fmin(a, b); }
static inline real rmax_(real a, real b) { return IS_F32 ? (real)fmaxf((float)a, (float)b) : (real)fmax(a, b); }

static inline v3 mk(real x, real y, real z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 scl(real s, v3 a) { return mk(s * a.x, s * a.y, s * a.z); }
static inline v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
static inline real dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* sutil-style normalize restated from the math: v * (1 / |v|). */
static inline v3 normalize(v3 v) { real inv = (real)1 / rsqrt_(dot(v, v)); return scl(inv, v); }
static inline real length(v3 v) { return rsqrt_(dot(v, v)); }
static inline v3 reflect(v3 i, v3 n) { return sub(i, scl(dot(n, i), scl((real)2, n))); }
static inline v3 faceforward(v3 n, v3 i, v3 nref) {
    real s = dot(i, nref) >= 0 ? (real)1 : (real)-1;
    return scl(s, n);
}

/* ------------------------------------------------------------------ scene ------------------ */
typedef struct {
    int type;
    real lo[3], hi[3];                   /* AABB as OptiX receives it (float in the f32 build) */
    /* Rectangle_Flat */
    v3 f_n; real f_w; v3 f_center, f_x, f_y; real f_width, f_height;
    /* Rectangle_Parabolic (v1, v2 already scaled by 1/|v|^2) */
    v3 p_v1, p_v2, p_anchor; real p_cx, p_cy;
    /* Cylinder_Y */
    v3 c_center, c_bx, c_bz; real c_radius, c_half;
    /* optics (extension) */
    real rho, slope, spec;
} prim_t;

typedef struct {
    v3 s;                 /* normalized sun vector */
    v3 v0, v1, v2, v3_;   /* sun plane parallelogram */
    real d;               /* sun plane distance */
    v3 w, u, v;           /* cone frame */
    real cos_theta;       /* cos(max_sun_angle) */
    real omc;             /* 1 - cos(max_sun_angle) = 2 sin^2(max_sun_angle / 2) (accurate pillbox) */
    int shape;            /* bit 0: gaussian (else pillbox); bit 1: accurate arithmetic (extension) */
    real sigma;           /* gaussian sun sigma */
} sun_t;

static double dnorm3(const double v[3]) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

/* lib/math_util.h:21-59 and lib/element.cpp:77-93: normal = aim - origin, Euler angles,
 * global-to-local matrix (Spencer & Murty).  Returns G2L row-major; L2G = transpose. */
static void element_g2l(const orc_element* e, double G[9]) {
    double n[3] = {e->aim_point[0] - e->origin[0], e->aim_point[1] - e->origin[1],
                   e->aim_point[2] - e->origin[2]};
    double len = dnorm3(n);
    if (len > 0) { n[0] = n[0] / len; n[1] = n[1] / len; n[2] = n[2] / len; }
    else { n[0] = n[1] = n[2] = 0.0; }
    double alpha = atan2(n[0], n[2]);
    double beta = asin(n[1]);
    double gamma = e->zrot_deg * M_PI / 180.0;
    double ca = cos(alpha), sa = sin(alpha);
    double cb = cos(beta), sb = sin(beta);
    double cg = cos(gamma), sg = sin(gamma);
    G[0] = ca * cg + sa * sb * sg; G[1] = -cb * sg; G[2] = -sa * cg + ca * sb * sg;
    G[3] = ca * sg - sa * sb * cg; G[4] = cb * cg;  G[5] = -sa * sg - ca * sb * cg;
    G[6] = sa * cb;                G[7] = sb;       G[8] = ca * cb;
}

/* L2G * v + origin, L2G = G2L^T (lib/vector3d.h:113-119). */
static void l2g_point(const double G[9], const double v[3], const double o[3], double out[3]) {
    out[0] = G[0] * v[0] + G[3] * v[1] + G[6] * v[2] + o[0];
    out[1] = G[1] * v[0] + G[4] * v[1] + G[7] * v[2] + o[1];
    out[2] = G[2] * v[0] + G[5] * v[1] + G[8] * v[2] + o[2];
}

static inline real tor(double x) { return (real)x; }
static inline v3 tov(const double a[3]) { return mk(tor(a[0]), tor(a[1]), tor(a[2])); }

static int build_prim(const orc_element* e, int is_last, prim_t* p, char* err) {
    memset(p, 0, sizeof(*p));
    if (e->aperture != 0) { sprintf(err, "only rectangle apertures are supported"); return -1; }
    if (e->surface != SURF_FLAT && e->surface != SURF_PARABOLIC && e->surface != SURF_CYLINDER) {
        sprintf(err, "unknown surface type %d", e->surface); return -1;
    }
    double G[9];
    element_g2l(e, G);
    const double xb[3] = {G[0], G[1], G[2]}, yb[3] = {G[3], G[4], G[5]}, zb[3] = {G[6], G[7], G[8]};
    const double w = e->width, h = e->height;

    /* bounding box: lib/element.cpp:172-275 */
    if (e->surface != SURF_CYLINDER) {
        const double c[4][3] = {{-w / 2, -h / 2, 0.0}, {w / 2, -h / 2, 0.0}, {w / 2, h / 2, 0.0}, {-w / 2, h / 2, 0.0}};
        double g[4][3];
        for (int k = 0; k < 4; ++k) l2g_point(G, c[k], e->origin, g[k]);
        for (int a = 0; a < 3; ++a) {
            p->lo[a] = tor(fmin(fmin(g[0][a], g[1][a]), fmin(g[2][a], g[3][a])));
            p->hi[a] = tor(fmax(fmax(g[0][a], g[1][a]), fmax(g[2][a], g[3][a])));
        }
    } else {
        const double c[8][3] = {{-w / 2, -h / 2, -w / 2}, {w / 2, -h / 2, -w / 2}, {-w / 2, h / 2, -w / 2},
                                {w / 2, h / 2, -w / 2},   {-w / 2, -h / 2, w / 2}, {w / 2, -h / 2, w / 2},
                                {-w / 2, h / 2, w / 2},   {w / 2, h / 2, w / 2}};
        double mn[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, mx[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
        for (int k = 0; k < 8; ++k) {
            double g[3];
            l2g_point(G, c[k], e->origin, g);
            for (int a = 0; a < 3; ++a) { mn[a] = fmin(mn[a], g[a]); mx[a] = fmax(mx[a], g[a]); }
        }
        for (int a = 0; a < 3; ++a) { p->lo[a] = tor(mn[a]); p->hi[a] = tor(mx[a]); }
    }

    /* entity type: lib/geometry_manager.cpp:50-59,78-90 */
    if (!is_last) {
        if (e->surface == SURF_PARABOLIC) p->type = ENT_PARABOLIC_MIRROR;
        else if (e->surface == SURF_FLAT) p->type = ENT_FLAT_MIRROR;
        else { sprintf(err, "cylinder surfaces are only supported as the receiver (last element)"); return -1; }
    } else {
        if (e->surface == SURF_FLAT) p->type = ENT_FLAT_RECEIVER;
        else if (e->surface == SURF_CYLINDER) p->type = ENT_CYL_RECEIVER;
        else p->type = ENT_PARABOLIC_MIRROR; /* reference prints an error and keeps the mirror */
    }

    /* device geometry: lib/element.cpp:114-164, cuda/GeometryDataST.h constructors */
    if (e->surface == SURF_FLAT) {
        p->f_center = tov(e->origin);
        p->f_x = tov(xb);
        p->f_y = tov(yb);
        p->f_width = (real)(float)w;
        p->f_height = (real)(float)h;
        if (!IS_F32) { p->f_width = (real)w; p->f_height = (real)h; }
        p->f_n = normalize(cross(p->f_x, p->f_y));
        p->f_w = dot(p->f_n, p->f_center);
    } else if (e->surface == SURF_PARABOLIC) {
        double sw = IS_F32 ? (double)(float)(-w) : -w;
        double sh = IS_F32 ? (double)(float)h : h;
        double v1[3] = {xb[0] * sw, xb[1] * sw, xb[2] * sw};
        double v2[3] = {yb[0] * sh, yb[1] * sh, yb[2] * sh};
        double an[3];
        for (int a = 0; a < 3; ++a) an[a] = e->origin[a] - v1[a] * 0.5 - v2[a] * 0.5;
        v3 fv1 = tov(v1), fv2 = tov(v2);
        p->p_anchor = tov(an);
        p->p_cx = tor(e->curv_x);
        p->p_cy = tor(e->curv_y);
        real i1 = (real)1 / dot(fv1, fv1);
        real i2 = (real)1 / dot(fv2, fv2);
        p->p_v1 = mk(fv1.x * i1, fv1.y * i1, fv1.z * i1);
        p->p_v2 = mk(fv2.x * i2, fv2.y * i2, fv2.z * i2);
    } else {
        p->c_radius = IS_F32 ? (real)((float)w / 2.0f) : (real)(w / 2.0);
        p->c_half = IS_F32 ? (real)((float)h / 2.0f) : (real)(h / 2.0);
        p->c_center = tov(e->origin);
        p->c_bx = tov(xb);
        p->c_bz = tov(zb);
    }
    p->rho = tor(e->reflectivity);
    p->slope = tor(e->slope_error);
    p->spec = tor(e->specularity_error);
    return 0;
}

/* lib/sun_utils.cu:41-50 corner order */
static void aabb_corner(const prim_t* p, int k, real out[3]) {
    out[0] = (k & 1) ? p->hi[0] : p->lo[0];
    out[1] = (k & 2) ? p->hi[1] : p->lo[1];
    out[2] = (k & 4) ? p->hi[2] : p->lo[2];
}

/* lib/geometry_manager.cpp:97-148 with lib/sun_utils.cu:53-179 restated as loops. */
static void build_sun(const prim_t* prims, uint32_t n, const double sun_dir[3], int shape, double param, sun_t* S) {
    double len = dnorm3(sun_dir);
    double sd[3] = {0, 0, 0};
    if (len > 0) { sd[0] = sun_dir[0] / len; sd[1] = sun_dir[1] / len; sd[2] = sun_dir[2] / len; }
    S->s = tov(sd);
    S->shape = shape;
    /* The reference pads the plane by the pillbox half angle; the Gaussian extension pads by 5 sigma. */
    const double pad_angle = (shape & 1) ? 5.0 * param : param;
    const real angle = tor(pad_angle);
    real d = 0;
    for (uint32_t i = 0; i < n; ++i)
        for (int k = 0; k < 8; ++k) {
            real c[3];
            aabb_corner(&prims[i], k, c);
            d = rmax_(d, rabs_(dot(mk(c[0], c[1], c[2]), S->s)));
        }
    S->d = d;
    v3 axis = (rabs_(S->s.x) < (real)0.9f) ? mk(1, 0, 0) : mk(0, 1, 0);
    v3 su = normalize(cross(axis, S->s));
    v3 sv = normalize(cross(S->s, su));
    const real tan_a = IS_F32 ? (real)tanf((float)angle) : (real)tan((double)angle);
    real umin = IS_F32 ? (real)FLT_MAX : (real)DBL_MAX, umax = -umin, vmin = umin, vmax = -umin;
    v3 pc = scl(d, S->s);
    for (uint32_t i = 0; i < n; ++i)
        for (int k = 0; k < 8; ++k) {
            real c[3];
            aabb_corner(&prims[i], k, c);
            v3 pt = mk(c[0], c[1], c[2]);
            real dist = rabs_(dot(pt, S->s));
            real buf = dist * tan_a;
            v3 proj = sub(pt, scl(dot(sub(pt, pc), S->s), S->s));
            real u = dot(proj, su), v = dot(proj, sv);
            umin = rmin_(umin, u - buf);
            umax = rmax_(umax, u + buf);
            vmin = rmin_(vmin, v - buf);
            vmax = rmax_(vmax, v + buf);
        }
    v3 ds = scl(d, S->s);
    S->v0 = add(add(scl(umin, su), scl(vmin, sv)), ds);
    S->v1 = add(add(scl(umax, su), scl(vmin, sv)), ds);
    S->v2 = add(add(scl(umax, su), scl(vmax, sv)), ds);
    S->v3_ = add(add(scl(umin, su), scl(vmax, sv)), ds);
    /* cone frame: cuda/sun.cu:72-79, dir = -normalize(sun_vector) (cuda/sun.cu:106) */
    v3 dir = neg(normalize(S->s));
    S->w = normalize(dir);
    S->u = normalize(cross(rabs_(S->w.x) > (real)0.99f ? mk(0, 1, 0) : mk(1, 0, 0), S->w));
    S->v = cross(S->w, S->u);
    S->omc = 0;
    if (shape & 1) { S->cos_theta = 1; S->sigma = tor(param); }
    else if (shape & 2) {
        /* accurate cone sampler (extension): 1 - cos(angle) as 2 sin^2(angle / 2), no cancellation */
        if (IS_F32) {
            float sn, cs;
            orc_sincosf((float)param * 0.5f, &sn, &cs);
            S->omc = (sn + sn) * sn;
        } else {
            const double sn = sin(param * 0.5);
            S->omc = (real)(2.0 * sn * sn);
        }
        S->cos_theta = (real)1 - S->omc;
        S->sigma = 0;
    } else {
        /* cosf(half_angle) of cuda/sun.cu:82, with the project's deterministic cos */
        if (IS_F32) { float sn, cs; orc_sincosf((float)param, &sn, &cs); S->cos_theta = cs; }
        else S->cos_theta = (real)cos(param);
        S->sigma = 0;
    }
}

/* ------------------------------------------------------------------ sampling --------------- */
/* cuda/sun.cu:16-24 */
static real halton(uint64_t index, uint32_t base) {
    real f = 1, r = 0;
    const real b = (real)base;
    while (index > 0) {
        f = f / b;
        r = r + f * (real)(index % base);
        index = index / base;
    }
    return r;
}

static void sincos_r(real x, real* s, real* c) {
    if (IS_F32) { float fs, fc; orc_sincosf((float)x, &fs, &fc); *s = fs; *c = fc; }
    else { *s = (real)sin((double)x); *c = (real)cos((double)x); }
}

static void box_muller_r(float u1, float u2, real* g1, real* g2) {
    if (IS_F32) { float a, b; orc_box_muller(u1, u2, &a, &b); *g1 = a; *g2 = b; }
    else {
        double rad = sqrt(-2.0 * log((double)u1));
        double ang = 2.0 * M_PI * (double)u2;
        *g1 = (real)(rad * cos(ang));
        *g2 = (real)(rad * sin(ang));
    }
}

/* ------------------------------------------------------------------ intersection ----------- */
/* Slab test deciding whether the "intersection program" of a primitive runs (the reference runs it
 * for every primitive whose AABB the ray segment [tmin, tmax] overlaps).  NaN-robust min/max. */
static int aabb_hit(const prim_t* p, v3 o, v3 inv, real tmin, real tmax) {
    const real oo[3] = {o.x, o.y, o.z}, ii[3] = {inv.x, inv.y, inv.z};
    real tn = tmin, tf = tmax;
    for (int a = 0; a < 3; ++a) {
        real t0 = (p->lo[a] - oo[a]) * ii[a];
        real t1 = (p->hi[a] - oo[a]) * ii[a];
        tn = rmax_(tn, rmin_(t0, t1));
        tf = rmin_(tf, rmax_(t0, t1));
    }
    return tn <= tf;
}

/* cuda/intersection.cu:47-85 */
static int is_flat(const prim_t* p, v3 o, v3 d, real tmin, real tmax, real* tout) {
    v3 n = p->f_n;
    real dt = dot(d, n);
    real t = (p->f_w - dot(n, o)) / dt;
    if (t > tmin && t < tmax) {
        v3 pt = add(o, scl(t, d));
        v3 v = sub(pt, p->f_center);
        real x = dot(p->f_x, v), y = dot(p->f_y, v);
        if (x >= -p->f_width / 2 && x <= p->f_width / 2 && y >= -p->f_height / 2 && y <= p->f_height / 2) {
            *tout = t;
            return 1;
        }
    }
    return 0;
}

/* cuda/intersection.cu:177-296.  accurate (extension): the side roots from the ray's closest
 * approach to the axis, tm = -(Ox Dx + Oz Dz) / A, and the half chord sqrt((r^2 - |Q|^2) / A) with
 * Q = O + tm D in the (x, z) plane, instead of B^2 - 4AC, which cancels to ~1e-4 relative when the
 * ray starts hundreds of metres from the receiver (about 1 mm on the hit point in float). */
static int is_cyl(const prim_t* p, v3 o, v3 draw, real tmin, real tmax, int accurate, real* tout) {
    v3 d = normalize(draw);
    v3 lo = sub(o, p->c_center);
    v3 lx = p->c_bx, lz = p->c_bz, ly = cross(lz, lx);
    v3 O = mk(dot(lo, lx), dot(lo, ly), dot(lo, lz));
    v3 D = mk(dot(d, lx), dot(d, ly), dot(d, lz));
    real A = D.x * D.x + D.z * D.z;
    real tc = tmax + (real)1;
    if (accurate) {
        if (A > 0) {
            real tm = -(O.x * D.x + O.z * D.z) / A;
            real qx = O.x + tm * D.x, qz = O.z + tm * D.z;
            real h2 = p->c_radius * p->c_radius - (qx * qx + qz * qz);
            if (h2 >= 0) {
                real hh = rsqrt_(h2 / A);
                real t1 = tm - hh, t2 = tm + hh;
                if (t1 > tmin && t1 < tmax && rabs_(O.y + t1 * D.y) <= p->c_half) tc = t1;
                else if (t2 > tmin && t2 < tmax && rabs_(O.y + t2 * D.y) <= p->c_half) tc = t2;
            }
        }
    }
    real B = (real)2 * (O.x * D.x + O.z * D.z);
    real C = O.x * O.x + O.z * O.z - p->c_radius * p->c_radius;
    real det = B * B - (real)4 * A * C;
    if (!accurate && det >= 0) {
        real sq = rsqrt_(det);
        real t1 = (-B - sq) / ((real)2 * A);
        real t2 = (-B + sq) / ((real)2 * A);
        if (t1 > tmin && t1 < tmax && rabs_(O.y + t1 * D.y) <= p->c_half) tc = t1;
        else if (t2 > tmin && t2 < tmax && rabs_(O.y + t2 * D.y) <= p->c_half) tc = t2;
    }
    real tcap = tmax + (real)1;
    if (rabs_(D.y) > (real)1e-6f) {
        real t = (-p->c_half - O.y) / D.y;
        real hx = O.x + t * D.x, hz = O.z + t * D.z;
        if (t > tmin && t < tmax && hx * hx + hz * hz <= p->c_radius * p->c_radius) tcap = t;
    }
    if (rabs_(D.y) > (real)1e-6f) {
        real t = (p->c_half - O.y) / D.y;
        real hx = O.x + t * D.x, hz = O.z + t * D.z;
        if (t > tmin && t < tmax && hx * hx + hz * hz <= p->c_radius * p->c_radius) tcap = rmin_(tcap, t);
    }
    real t = rmin_(tc, tcap);
    if (t >= tmax || t <= tmin) return 0;
    *tout = t;
    return 1;
}

/* cuda/intersection.cu:318-448.  Returns t and the world normal. */
static int is_parab(const prim_t* p, v3 o, v3 d, real tmin, real tmax, real* tout, v3* nout) {
    real L1 = (real)1 / length(p->p_v1);
    real L2 = (real)1 / length(p->p_v2);
    v3 e1 = scl(L1, p->p_v1);
    v3 e2 = scl(L2, p->p_v2);
    v3 n = normalize(cross(e2, e1));
    v3 c = add(add(p->p_anchor, scl(L1 / (real)2, e1)), scl(L2 / (real)2, e2));
    v3 dd = sub(o, c);
    real ox = dot(dd, e1), oy = dot(dd, e2), oz = dot(dd, n);
    real dx = dot(d, e1), dy = dot(d, e2), dz = dot(d, n);
    real cx = p->p_cx, cy = p->p_cy;
    real A = (cx * (real)0.5) * (dx * dx) + (cy * (real)0.5) * (dy * dy);
    real B = cx * (ox * dx) + cy * (oy * dy) - dz;
    real C = (cx * (real)0.5) * (ox * ox) + (cy * (real)0.5) * (oy * oy) - oz;
    real t = 0;
    int valid = 0;
    if (rabs_(A) < (real)1e-12f) {
        t = -C / B;
        valid = (t > 0);
    } else {
        real disc = B * B - (real)4 * A * C;
        if (disc >= 0) {
            real sq = rsqrt_(disc);
            real t1 = (-B - sq) / ((real)2 * A);
            real t2 = (-B + sq) / ((real)2 * A);
            if (t1 > 0 && t1 < t2) { t = t1; valid = 1; }
            else if (t2 > 0) { t = t2; valid = 1; }
        }
    }
    if (!valid || t < tmin || t > tmax) return 0;
    real xh = ox + t * dx, yh = oy + t * dy;
    /* a1 = x_hit / (L1/2.) is evaluated in double by the reference (literal 2.). */
    real a1 = (real)((double)xh / ((double)L1 / 2.));
    real a2 = (real)((double)yh / ((double)L2 / 2.));
    if (a1 < (real)-1 || a1 > (real)1 || a2 < (real)-1 || a2 > (real)1) return 0;
    v3 nl = normalize(mk(-cx * xh, -cy * yh, (real)1));
    v3 wn = normalize(add(add(scl(nl.x, e1), scl(nl.y, e2)), scl(nl.z, n)));
    *tout = t;
    *nout = wn;
    return 1;
}

/* ------------------------------------------------------------------ trace ------------------ */
static void perturb(v3 n, real sigma, real g1, real g2, v3* out) {
    v3 t1 = normalize(cross(rabs_(n.x) > (real)0.9f ? mk(0, 1, 0) : mk(1, 0, 0), n));
    v3 t2 = cross(n, t1);
    *out = normalize(add(add(n, scl(sigma * g1, t1)), scl(sigma * g2, t2)));
}

static void trace_ray(const prim_t* prims, uint32_t n, const sun_t* S, uint64_t ray, uint64_t seed,
                      uint32_t instance, int max_depth, double* hout, uint32_t* iout) {
    for (int k = 0; k < max_depth; ++k) {
        hout[4 * k] = hout[4 * k + 1] = hout[4 * k + 2] = hout[4 * k + 3] = 0.0;
        if (iout) iout[k] = 0xFFFFFFFFu;
    }
    /* ray generation: cuda/sun.cu:28-38,94-115 */
    real hu = halton(ray, 2), hv = halton(ray, 3);
    v3 e1 = sub(S->v1, S->v0), e2 = sub(S->v3_, S->v0);
    v3 pos = add(add(S->v0, scl(hu, e1)), scl(hv, e2));
    orc_u32x4 r0 = orc_draw(ray, 0, 0, instance, seed);
    v3 dir;
    if (S->shape & 1) {
        real g1, g2;
        box_muller_r(orc_u01(r0.v[0]), orc_u01(r0.v[1]), &g1, &g2);
        dir = normalize(add(add(S->w, scl(S->sigma * g1, S->u)), scl(S->sigma * g2, S->v)));
    } else if (S->shape & 2) {
        /* the same uniform z in [cos(angle), 1] as cuda/sun.cu:82-86, carried as 1 - z =
         * (1 - cos(angle)) (1 - rand2) so the cone radius sqrt(1 - z^2) = sqrt((1 - z)(2 - (1 - z)))
         * keeps full relative precision (the reference's float z quantizes 1 - z in steps of 2^-24) */
        real rand1 = (real)orc_u01(r0.v[0]), rand2 = (real)orc_u01(r0.v[1]);
        real phi = (IS_F32 ? (real)(2.0f * 3.14159265358979323846f) : (real)(2.0 * M_PI)) * rand1;
        real omz = S->omc * ((real)1 - rand2);
        real z = (real)1 - omz;
        real r = rsqrt_(omz * ((real)2 - omz));
        real sp, cp;
        sincos_r(phi, &sp, &cp);
        dir = normalize(add(scl(r, add(scl(cp, S->u), scl(sp, S->v))), scl(z, S->w)));
    } else {
        real rand1 = (real)orc_u01(r0.v[0]), rand2 = (real)orc_u01(r0.v[1]);
        real phi = (IS_F32 ? (real)(2.0f * 3.14159265358979323846f) : (real)(2.0 * M_PI)) * rand1;
        real z = S->cos_theta + ((real)1 - S->cos_theta) * rand2;
        real r = rsqrt_((real)1 - z * z);
        real sp, cp;
        sincos_r(phi, &sp, &cp);
        dir = normalize(add(scl(r, add(scl(cp, S->u), scl(sp, S->v))), scl(z, S->w)));
    }
    hout[1] = pos.x; hout[2] = pos.y; hout[3] = pos.z;

    v3 o = pos, d = dir;
    real tmin = (real)0.001f;
    const real tmax = (real)1e16f;
    int depth = 0;
    for (;;) {
        v3 inv = mk((real)1 / d.x, (real)1 / d.y, (real)1 / d.z);
        real best_t = (real)INFINITY;
        int best = -1;
        v3 best_n = mk(0, 0, 0);
        for (uint32_t k = 0; k < n; ++k) {
            const prim_t* p = &prims[k];
            if (!aabb_hit(p, o, inv, tmin, tmax)) continue;
            real t;
            v3 nn;
            int ok;
            switch (p->type) {
                case ENT_FLAT_MIRROR:
                case ENT_FLAT_RECEIVER: ok = is_flat(p, o, d, tmin, tmax, &t); nn = p->f_n; break;
                case ENT_PARABOLIC_MIRROR: ok = is_parab(p, o, d, tmin, tmax, &t, &nn); break;
                default: ok = is_cyl(p, o, d, tmin, tmax, (S->shape & 2) != 0, &t); nn = mk(0, 0, 0); break;
            }
            /* closest hit; equal t keeps the lower element index */
            if (ok && t < best_t) { best_t = t; best = (int)k; best_n = nn; }
        }
        if (best < 0) break; /* __miss__ms: nothing recorded */
        const prim_t* p = &prims[best];
        const int nd = depth + 1;
        v3 hit = add(o, scl(best_t, d));
        if (p->type == ENT_FLAT_MIRROR || p->type == ENT_PARABOLIC_MIRROR) {
            /* cuda/materials.cu:26-84 / :170-231 */
            v3 wn = normalize(best_n);
            v3 ffn = faceforward(wn, neg(d), wn);
            if (!(nd < max_depth)) break;
            hout[4 * nd] = 1.0; hout[4 * nd + 1] = hit.x; hout[4 * nd + 2] = hit.y; hout[4 * nd + 3] = hit.z;
            if (iout) iout[nd] = (uint32_t)best;
            orc_u32x4 ra = orc_draw(ray, (uint32_t)nd, 0, instance, seed);
            if (p->slope > 0) {
                real g1, g2;
                box_muller_r(orc_u01(ra.v[1]), orc_u01(ra.v[2]), &g1, &g2);
                perturb(ffn, p->slope, g1, g2, &ffn);
            }
            v3 rd = reflect(d, ffn);
            if (p->spec > 0) {
                orc_u32x4 rb = orc_draw(ray, (uint32_t)nd, 1, instance, seed);
                real g1, g2;
                box_muller_r(orc_u01(rb.v[0]), orc_u01(rb.v[1]), &g1, &g2);
                perturb(normalize(rd), p->spec, g1, g2, &rd);
            }
            if ((real)orc_u01(ra.v[0]) > p->rho) break; /* absorbed at the mirror (extension) */
            depth = nd;
            o = hit;
            d = rd;
            tmin = (real)0.01f;
            continue;
        }
        if (p->type == ENT_FLAT_RECEIVER) {
            /* cuda/materials.cu:86-121: one-sided */
            v3 rn = cross(p->f_x, p->f_y);
            if (dot(d, rn) < 0 && nd < max_depth) {
                hout[4 * nd] = 2.0; hout[4 * nd + 1] = hit.x; hout[4 * nd + 2] = hit.y; hout[4 * nd + 3] = hit.z;
                if (iout) iout[nd] = (uint32_t)best;
            }
            break;
        }
        /* cuda/materials.cu:123-163: cylinder records every hit */
        if (nd < max_depth) {
            hout[4 * nd] = 2.0; hout[4 * nd + 1] = hit.x; hout[4 * nd + 2] = hit.y; hout[4 * nd + 3] = hit.z;
            if (iout) iout[nd] = (uint32_t)best;
        }
        break;
    }
}

static int prepare(const orc_element* el, uint32_t n, const double sun_dir[3], int shape, double param,
                   prim_t** prims_out, sun_t* S, char* err) {
    if (n == 0) { sprintf(err, "no elements"); return -1; }
    prim_t* prims = (prim_t*)calloc(n, sizeof(prim_t));
    for (uint32_t i = 0; i < n; ++i)
        if (build_prim(&el[i], i + 1 == n, &prims[i], err)) { free(prims); return -1; }
    build_sun(prims, n, sun_dir, shape, param, S);
    *prims_out = prims;
    return 0;
}

static char g_err[256];
EXPORT const char* orc_last_error(void) { return g_err; }
EXPORT const char* orc_precision(void) { return IS_F32 ? "f32" : "f64"; }

/* Trace rays [first_ray, first_ray + count).  hits: count * max_depth * 4 doubles (stage, x, y, z);
 * ids: count * max_depth (element index, 0xFFFFFFFF for the sun slot and unused slots), may be NULL. */
EXPORT int orc_trace(const orc_element* el, uint32_t n, const double sun_dir[3], int sun_shape, double sun_param,
                     uint64_t first_ray, uint64_t count, uint64_t seed, uint32_t instance, int max_depth,
                     double* hits, uint32_t* ids, int nthreads) {
    prim_t* prims;
    sun_t S;
    if (max_depth < 1 || max_depth > 16) { sprintf(g_err, "max_depth out of range"); return -1; }
    if (prepare(el, n, sun_dir, sun_shape, sun_param, &prims, &S, g_err)) return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1024)
#endif
    for (int64_t k = 0; k < (int64_t)count; ++k)
        trace_ray(prims, n, &S, first_ray + (uint64_t)k, seed, instance, max_depth, hits + (size_t)k * max_depth * 4,
                  ids ? ids + (size_t)k * max_depth : NULL);
    free(prims);
    return 0;
}

/* Scene introspection for tests: per element 32 doubles, the sun frame in 32 doubles.
 * prim layout: [type, lo3, hi3, geometry 16 (type dependent), rho, slope, spec, pad...]
 * sun layout:  [s3, v0 3, v1 3, v2 3, v3 3, d, w3, u3, v3, cos_theta, sigma, shape, 1 - cos_theta (shape 2)] */
EXPORT int orc_scene_info(const orc_element* el, uint32_t n, const double sun_dir[3], int sun_shape,
                          double sun_param, double* prim_out, double* sun_out) {
    prim_t* prims;
    sun_t S;
    if (prepare(el, n, sun_dir, sun_shape, sun_param, &prims, &S, g_err)) return -1;
    for (uint32_t i = 0; i < n; ++i) {
        double* o = prim_out + 32 * i;
        const prim_t* p = &prims[i];
        memset(o, 0, 32 * sizeof(double));
        o[0] = p->type;
        for (int a = 0; a < 3; ++a) { o[1 + a] = p->lo[a]; o[4 + a] = p->hi[a]; }
        double* g = o + 7;
        if (p->type == ENT_FLAT_MIRROR || p->type == ENT_FLAT_RECEIVER) {
            const real v[16] = {p->f_n.x, p->f_n.y, p->f_n.z, p->f_w, p->f_center.x, p->f_center.y, p->f_center.z,
                                p->f_x.x, p->f_x.y, p->f_x.z, p->f_y.x, p->f_y.y, p->f_y.z, p->f_width, p->f_height, 0};
            for (int k = 0; k < 16; ++k) g[k] = v[k];
        } else if (p->type == ENT_PARABOLIC_MIRROR) {
            const real v[16] = {p->p_v1.x, p->p_v1.y, p->p_v1.z, p->p_v2.x, p->p_v2.y, p->p_v2.z, p->p_anchor.x,
                                p->p_anchor.y, p->p_anchor.z, p->p_cx, p->p_cy, 0, 0, 0, 0, 0};
            for (int k = 0; k < 16; ++k) g[k] = v[k];
        } else {
            const real v[16] = {p->c_center.x, p->c_center.y, p->c_center.z, p->c_radius, p->c_half, p->c_bx.x,
                                p->c_bx.y, p->c_bx.z, p->c_bz.x, p->c_bz.y, p->c_bz.z, 0, 0, 0, 0, 0};
            for (int k = 0; k < 16; ++k) g[k] = v[k];
        }
        o[23] = p->rho; o[24] = p->slope; o[25] = p->spec;
    }
    const real sv[31] = {S.s.x, S.s.y, S.s.z, S.v0.x, S.v0.y, S.v0.z, S.v1.x, S.v1.y, S.v1.z, S.v2.x, S.v2.y,
                         S.v2.z, S.v3_.x, S.v3_.y, S.v3_.z, S.d, S.w.x, S.w.y, S.w.z, S.u.x, S.u.y, S.u.z,
                         S.v.x, S.v.y, S.v.z, S.cos_theta, S.sigma, (real)S.shape, S.omc, 0, 0};
    for (int k = 0; k < 31; ++k) sun_out[k] = sv[k];
    free(prims);
    return 0;
}

/* Deterministic-math probes for tests (f32 build semantics regardless of ORC_REAL). */
EXPORT void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    orc_u32x4 c = {{ctr[0], ctr[1], ctr[2], ctr[3]}};
    orc_u32x4 r = orc_philox4x32_10(c, key[0], key[1]);
    memcpy(out, r.v, 16);
}
EXPORT void orc_sincos_batch(const float* x, int64_t n, float* s, float* c) {
    for (int64_t i = 0; i < n; ++i) orc_sincosf(x[i], &s[i], &c[i]);
}
EXPORT void orc_sincos2pi_batch(const float* u, int64_t n, float* s, float* c) {
    for (int64_t i = 0; i < n; ++i) orc_sincos2pi(u[i], &s[i], &c[i]);
}
EXPORT void orc_log_batch(const float* x, int64_t n, float* y) {
    for (int64_t i = 0; i < n; ++i) y[i] = orc_logf(x[i]);
}
EXPORT void orc_atan2_batch(const float* y, const float* x, int64_t n, float* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = orc_atan2f(y[i], x[i]);
}

/* Receiver flux map, scripts/post_processing/flux_map_calculator.py:135-179 (stage-2 records binned
 * over the receiver) with the cylinder convention of plot_flux_map_gpu.py:174-210 (angle about the
 * axis, axial coordinate, caps dropped), evaluated in float from the receiver parameters t[20] of
 * csp_flux_target: origin (3), local x, y, z axes (9), hx, hy, kx, ky, keep, kind.
 * rec: n float records {stage, x, y, z}.  counts[nx * ny] and stats[4] (rays unused, mirror
 * records, receiver records, binned) are accumulated into. */
EXPORT void orc_flux_counts(const float* rec, int64_t n, const float* t, int nx, int ny, uint32_t* counts,
                            uint64_t* stats) {
    for (int64_t i = 0; i < n; ++i) {
        const float* r = rec + 4 * i;
        if (r[0] == 1.0f) { stats[1] += 1; continue; }
        if (r[0] != 2.0f) continue;
        stats[2] += 1;
        const float px = r[1] - t[0], py = r[2] - t[1], pz = r[3] - t[2];
        const float lx = px * t[3] + py * t[4] + pz * t[5];
        const float ly = px * t[6] + py * t[7] + pz * t[8];
        float u;
        if (t[17] == 1.0f) {
            if (!(fabsf(ly) < t[16])) continue;
            const float lz = px * t[9] + py * t[10] + pz * t[11];
            float a = orc_atan2f(lz, lx);
            if (a < 0.0f) a = a + 0x1.921fb6p+2f;
            u = a * t[14];
        } else {
            u = (lx + t[12]) * t[14];
        }
        const float v = (ly + t[13]) * t[15];
        const int bx = (int)fminf(fmaxf(floorf(u), 0.0f), (float)(nx - 1));
        const int by = (int)fminf(fmaxf(floorf(v), 0.0f), (float)(ny - 1));
        counts[(size_t)bx * ny + by] += 1;
        stats[3] += 1;
    }
}
