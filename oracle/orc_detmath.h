/*
 * orc_detmath.h -- TEST INFRASTRUCTURE (oracle side). Never linked into the product.
 *
 * Deterministic scalar math shared by the C oracle (csp_oracle.c) and the host build of the
 * reference's own device programs (ref_driver.cpp + ref_shim/).  Every function here gives the
 * same bits on any IEEE-754 machine when compiled with -ffp-contract=off: only +,-,*,/, sqrt,
 * rint and explicit fmaf (all correctly rounded) are used.
 *
 *  - Philox-4x32-10 counter-based generator: Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
 *    as easy as 1, 2, 3", SC'11.  Round constants are the paper's (Weyl key bumps 0x9E3779B9 /
 *    0xBB67AE85, multipliers 0xD2511F53 / 0xCD9E8D57).  It stands in for the reference's cuRAND
 *    XORWOW draws (cuda/sun.cu:72-84), which cannot be reproduced here.
 *  - sin/cos: Cody-Waite reduction by pi/2 (two-term split, exact first step through fmaf), then the
 *    Taylor series of sin and cos on [-pi/4, pi/4] evaluated by Horner's rule.
 *  - log: x = m * 2^e with m in [sqrt(1/2), sqrt(2)], log m = 2 atanh(s), s = (m-1)/(m+1), odd
 *    series of atanh to s^9, plus e*ln2 with ln2 split in two floats.
 *
 * The product's CUDA kernels carry their own implementation of the same published methods; the
 * parity tests check the two agree bit-for-bit through whole traces.
 */
#ifndef ORC_DETMATH_H
#define ORC_DETMATH_H

#include <stdint.h>
#include <math.h>
#include <string.h>

#ifdef __cplusplus
#define ORC_INLINE static inline
#else
#define ORC_INLINE static inline
#endif

/* ---------------------------------------------------------------- Philox-4x32-10 ------------ */
typedef struct { uint32_t v[4]; } orc_u32x4;

ORC_INLINE void orc_mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

ORC_INLINE orc_u32x4 orc_philox4x32_10(orc_u32x4 ctr, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        orc_mulhilo32(0xD2511F53u, ctr.v[0], &hi0, &lo0);
        orc_mulhilo32(0xCD9E8D57u, ctr.v[2], &hi1, &lo1);
        orc_u32x4 n;
        n.v[0] = hi1 ^ ctr.v[1] ^ k0;
        n.v[1] = lo1;
        n.v[2] = hi0 ^ ctr.v[3] ^ k1;
        n.v[3] = lo0;
        ctr = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return ctr;
}

/* Counter layout used across the project: (ray_lo, ray_hi, bounce<<4 | draw, instance),
 * key = (seed_lo, seed_hi).  bounce 0 = sun sample, bounce k>=1 = k-th surface interaction. */
ORC_INLINE orc_u32x4 orc_draw(uint64_t ray, uint32_t bounce, uint32_t draw, uint32_t instance,
                              uint64_t seed) {
    orc_u32x4 c;
    c.v[0] = (uint32_t)ray;
    c.v[1] = (uint32_t)(ray >> 32);
    c.v[2] = (bounce << 4) | (draw & 15u);
    c.v[3] = instance;
    return orc_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

/* 24-bit uniform in (0, 1], exact in float (same convention as curand_uniform's range). */
ORC_INLINE float orc_u01(uint32_t x) { return (float)((x >> 8) + 1u) * 0x1p-24f; }

/* ---------------------------------------------------------------- sin / cos ----------------- */
#define ORC_PIO2_HI 0x1.921fb6p+0f      /* fl32(pi/2) */
#define ORC_PIO2_LO (-0x1.777a5cp-25f)  /* fl32(pi/2 - ORC_PIO2_HI) */
#define ORC_TWO_OVER_PI 0x1.45f306p-1f

ORC_INLINE void orc_sincos_poly(float x, float* s, float* c) {
    const float x2 = x * x;
    float ps = fmaf(x2, (float)(1.0 / 362880.0), (float)(-1.0 / 5040.0));
    ps = fmaf(x2, ps, (float)(1.0 / 120.0));
    ps = fmaf(x2, ps, (float)(-1.0 / 6.0));
    *s = fmaf(x * x2, ps, x);
    float pc = fmaf(x2, (float)(-1.0 / 3628800.0), (float)(1.0 / 40320.0));
    pc = fmaf(x2, pc, (float)(-1.0 / 720.0));
    pc = fmaf(x2, pc, (float)(1.0 / 24.0));
    pc = fmaf(x2, pc, -0.5f);
    *c = fmaf(x2, pc, 1.0f);
}

ORC_INLINE void orc_quadrant(int q, float s, float c, float* so, float* co) {
    switch (q & 3) {
        case 0: *so = s;  *co = c;  break;
        case 1: *so = c;  *co = -s; break;
        case 2: *so = -s; *co = -c; break;
        default: *so = -c; *co = s; break;
    }
}

/* sin/cos of a float argument, |x| <= 64. */
ORC_INLINE void orc_sincosf(float x, float* s, float* c) {
    const float k = rintf(x * ORC_TWO_OVER_PI);
    float r = fmaf(-k, ORC_PIO2_HI, x);
    r = fmaf(-k, ORC_PIO2_LO, r);
    float ps, pc;
    orc_sincos_poly(r, &ps, &pc);
    orc_quadrant((int)k, ps, pc, s, c);
}

/* sin/cos of 2*pi*u for u in [0, 1] (Box-Muller angle). q = 4u is exact, f = q - rint(q) exact. */
ORC_INLINE void orc_sincos2pi(float u, float* s, float* c) {
    const float q = u * 4.0f;
    const float k = rintf(q);
    const float f = q - k;
    float ps, pc;
    orc_sincos_poly(f * ORC_PIO2_HI, &ps, &pc);
    orc_quadrant((int)k, ps, pc, s, c);
}

/* ---------------------------------------------------------------- log ----------------------- */
#define ORC_LN2_HI 0x1.62e43p-1f
#define ORC_LN2_LO (-0x1.05c61p-29f)

/* natural log for normal positive x. */
ORC_INLINE float orc_logf(float x) {
    uint32_t b;
    memcpy(&b, &x, 4);
    int e = (int)((b >> 23) & 0xffu) - 127;
    uint32_t mb = (b & 0x7fffffu) | 0x3f800000u;
    float m;
    memcpy(&m, &mb, 4);
    if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = fmaf(s2, (float)(1.0 / 9.0), (float)(1.0 / 7.0));
    p = fmaf(s2, p, (float)(1.0 / 5.0));
    p = fmaf(s2, p, (float)(1.0 / 3.0));
    p = s2 * p;
    const float two_s = 2.0f * s;
    const float lm = fmaf(two_s, p, two_s);
    const float fe = (float)e;
    return fmaf(fe, ORC_LN2_HI, fmaf(fe, ORC_LN2_LO, lm));
}

/* Box-Muller pair of standard normals from two (0,1] uniforms. */
ORC_INLINE void orc_box_muller(float u1, float u2, float* g1, float* g2) {
    const float rad = sqrtf(-2.0f * orc_logf(u1));
    float s, c;
    orc_sincos2pi(u2, &s, &c);
    *g1 = rad * c;
    *g2 = rad * s;
}

/* atan2 by quadrant reduction to t = min/max in [0, 1], the tangent subtraction formula
 * atan t = pi/6 + atan((t sqrt3 - 1)/(t + sqrt3)) for t > tan(pi/12), and the odd Taylor series of
 * atan to t^13 on |t| <= tan(pi/12) (Horner, fused steps as written).  Used to bin receiver angles. */
#define ORC_TAN_PI12 0x1.126146p-2f
#define ORC_SQRT3 0x1.bb67aep+0f
#define ORC_PI6 0x1.0c1524p-1f
#define ORC_PIO2_F 0x1.921fb6p+0f
#define ORC_PI_F 0x1.921fb6p+1f

ORC_INLINE float orc_atan2f(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    if (!(mx > 0.0f)) return 0.0f;
    float t = mn / mx;
    float base = 0.0f;
    if (t > ORC_TAN_PI12) {
        t = (t * ORC_SQRT3 - 1.0f) / (t + ORC_SQRT3);
        base = ORC_PI6;
    }
    const float t2 = t * t;
    float p = fmaf(t2, (float)(1.0 / 13.0), (float)(-1.0 / 11.0));
    p = fmaf(t2, p, (float)(1.0 / 9.0));
    p = fmaf(t2, p, (float)(-1.0 / 7.0));
    p = fmaf(t2, p, (float)(1.0 / 5.0));
    p = fmaf(t2, p, (float)(-1.0 / 3.0));
    float r = fmaf(t * t2, p, t) + base;
    if (ay > ax) r = ORC_PIO2_F - r;
    if (x < 0.0f) r = ORC_PI_F - r;
    return (y < 0.0f) ? -r : r;
}

#endif /* ORC_DETMATH_H */
