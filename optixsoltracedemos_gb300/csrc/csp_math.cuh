// csp_math.cuh -- float3 algebra, Philox-4x32-10 and deterministic sin/cos/log, usable from host
// and device code.
//
// Bit-reproducibility contract: the library is compiled with -fmad=false (device) and
// -ffp-contract=off (host), so every a*b+c written below rounds twice exactly as written, and the
// only fused operations are the explicit fmaf() calls.  Division and sqrt are IEEE (no fast math).
// With that, a host evaluation and a device evaluation of any function here give identical bits.
//
// Operation order follows the reference's vector helpers (used by cuda/*.cu of the reference):
//   dot = x*x' + y*y' + z*z' left to right; normalize(v) = v * (1 / sqrt(dot(v, v)));
//   reflect(i, n) = i - (2 n) dot(n, i).
//
// Philox-4x32-10: Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11 (multipliers 0xD2511F53 / 0xCD9E8D57, Weyl key increments 0x9E3779B9 / 0xBB67AE85).
// sin/cos: Cody-Waite reduction by pi/2 (two-float split, first step exact via fmaf), Taylor series
// of sin (to x^9) and cos (to x^10) on [-pi/4, pi/4] by Horner's rule.
// log: x = m 2^e, m in [sqrt(1/2), sqrt(2)], log m = 2 atanh((m-1)/(m+1)) by its odd series to s^9,
// plus e ln2 with ln2 split into two floats.
#pragma once

#include <cstdint>
#include <cstring>
#include <cmath>
#include <cuda_runtime.h>

#if defined(__CUDACC__)
#define CSP_HD __host__ __device__ __forceinline__
#else
#define CSP_HD inline
#endif

namespace csp {

// ------------------------------------------------------------------------------------ float3 ---
CSP_HD float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
CSP_HD float3 add(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
CSP_HD float3 sub(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
CSP_HD float3 scale(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
CSP_HD float3 neg(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
CSP_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
CSP_HD float3 cross(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
CSP_HD float length(float3 v) { return sqrtf(dot(v, v)); }
CSP_HD float3 normalize(float3 v) {
    const float inv = 1.0f / sqrtf(dot(v, v));
    return scale(inv, v);
}
CSP_HD float3 reflect(float3 i, float3 n) { return sub(i, scale(dot(n, i), scale(2.0f, n))); }
CSP_HD float3 xyz(float4 a) { return make_float3(a.x, a.y, a.z); }

CSP_HD uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}
CSP_HD float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}

// ------------------------------------------------------------------------------------ Philox ---
struct u32x4 {
    uint32_t x, y, z, w;
};

CSP_HD u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        // one 32x32->64 multiply per product gives both halves
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c = u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// The same rounds with the key schedule precomputed: keys[2r], keys[2r + 1] = the key of round r.
CSP_HD u32x4 philox4x32_10_sched(u32x4 c, const uint32_t* keys) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c = u32x4{hi1 ^ c.y ^ keys[2 * r], lo1, hi0 ^ c.w ^ keys[2 * r + 1], lo0};
    }
    return c;
}

// Key schedule of a seed for philox4x32_10_sched.
CSP_HD void philox_keys(uint64_t seed, uint32_t* keys) {
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        keys[2 * r] = k0;
        keys[2 * r + 1] = k1;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// Draw block for (ray, bounce, draw, instance) under the key schedule of the seed.
CSP_HD u32x4 draw_block_sched(uint64_t ray, uint32_t bounce, uint32_t draw, uint32_t instance, const uint32_t* keys) {
    return philox4x32_10_sched(u32x4{(uint32_t)ray, (uint32_t)(ray >> 32), (bounce << 4) | (draw & 15u), instance},
                               keys);
}

// Draw block for (ray, bounce, draw, instance) under key = seed.  bounce 0 = sun sample,
// bounce k >= 1 = k-th surface interaction; draw selects one of up to 16 blocks per bounce.
CSP_HD u32x4 draw_block(uint64_t ray, uint32_t bounce, uint32_t draw, uint32_t instance, uint64_t seed) {
    return philox4x32_10(u32x4{(uint32_t)ray, (uint32_t)(ray >> 32), (bounce << 4) | (draw & 15u), instance},
                         (uint32_t)seed, (uint32_t)(seed >> 32));
}

// 24-bit uniform in (0, 1], exact in float.
CSP_HD float u01(uint32_t x) { return (float)((x >> 8) + 1u) * 0x1p-24f; }

// ------------------------------------------------------------------------------- sin / cos ----
constexpr float kPio2Hi = 0x1.921fb6p+0f;      // fl32(pi/2)
constexpr float kPio2Lo = -0x1.777a5cp-25f;    // fl32(pi/2 - kPio2Hi)
constexpr float kTwoOverPi = 0x1.45f306p-1f;   // fl32(2/pi)

CSP_HD void sincos_kernel(float x, float& s, float& c) {
    const float x2 = x * x;
    float ps = fmaf(x2, (float)(1.0 / 362880.0), (float)(-1.0 / 5040.0));
    ps = fmaf(x2, ps, (float)(1.0 / 120.0));
    ps = fmaf(x2, ps, (float)(-1.0 / 6.0));
    s = fmaf(x * x2, ps, x);
    float pc = fmaf(x2, (float)(-1.0 / 3628800.0), (float)(1.0 / 40320.0));
    pc = fmaf(x2, pc, (float)(-1.0 / 720.0));
    pc = fmaf(x2, pc, (float)(1.0 / 24.0));
    pc = fmaf(x2, pc, -0.5f);
    c = fmaf(x2, pc, 1.0f);
}

CSP_HD void quadrant(int q, float s, float c, float& so, float& co) {
    const int qq = q & 3;
    so = (qq == 0) ? s : (qq == 1) ? c : (qq == 2) ? -s : -c;
    co = (qq == 0) ? c : (qq == 1) ? -s : (qq == 2) ? -c : s;
}

// sin and cos of x, |x| <= 64.
CSP_HD void det_sincos(float x, float& s, float& c) {
    const float k = rintf(x * kTwoOverPi);
    float r = fmaf(-k, kPio2Hi, x);
    r = fmaf(-k, kPio2Lo, r);
    float ps, pc;
    sincos_kernel(r, ps, pc);
    quadrant((int)k, ps, pc, s, c);
}

// sin and cos of 2 pi u, u in [0, 1].  4u and 4u - rint(4u) are exact.
CSP_HD void det_sincos2pi(float u, float& s, float& c) {
    const float q = u * 4.0f;
    const float k = rintf(q);
    const float f = q - k;
    float ps, pc;
    sincos_kernel(f * kPio2Hi, ps, pc);
    quadrant((int)k, ps, pc, s, c);
}

constexpr float kLn2Hi = 0x1.62e43p-1f;
constexpr float kLn2Lo = -0x1.05c61p-29f;

// natural log of a normal positive float.
CSP_HD float det_log(float x) {
    const uint32_t b = f2u(x);
    int e = (int)((b >> 23) & 0xffu) - 127;
    float m = u2f((b & 0x7fffffu) | 0x3f800000u);
    if (m > 0x1.6a09e6p+0f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = fmaf(s2, (float)(1.0 / 9.0), (float)(1.0 / 7.0));
    p = fmaf(s2, p, (float)(1.0 / 5.0));
    p = fmaf(s2, p, (float)(1.0 / 3.0));
    p = s2 * p;
    const float two_s = 2.0f * s;
    const float lm = fmaf(two_s, p, two_s);
    const float fe = (float)e;
    return fmaf(fe, kLn2Hi, fmaf(fe, kLn2Lo, lm));
}

// Box-Muller: two standard normals from two (0, 1] uniforms.
CSP_HD void box_muller(float u1, float u2, float& g1, float& g2) {
    const float rad = sqrtf(-2.0f * det_log(u1));
    float s, c;
    det_sincos2pi(u2, s, c);
    g1 = rad * c;
    g2 = rad * s;
}

// --------------------------------------------------------------------------------- atan2 -----
// Quadrant reduction to t = min/max in [0, 1], then atan t = pi/6 + atan((t sqrt3 - 1)/(t + sqrt3))
// for t > tan(pi/12) (the tangent subtraction formula), leaving |t| <= tan(pi/12) = 0.268 where
// the odd Taylor series of atan to t^13 has a truncation error below 2e-10.  Absolute error about
// 3e-7 rad; used for binning receiver angles, where the same bits on host and device matter more.
constexpr float kTanPi12 = 0x1.126146p-2f;   // fl32(2 - sqrt(3))
constexpr float kSqrt3 = 0x1.bb67aep+0f;     // fl32(sqrt(3))
constexpr float kPi6 = 0x1.0c1524p-1f;       // fl32(pi/6)
constexpr float kPio2 = 0x1.921fb6p+0f;      // fl32(pi/2)
constexpr float kPiF = 0x1.921fb6p+1f;       // fl32(pi)

CSP_HD float det_atan2(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    if (!(mx > 0.0f)) return 0.0f;
    float t = mn / mx;
    float base = 0.0f;
    if (t > kTanPi12) {
        t = (t * kSqrt3 - 1.0f) / (t + kSqrt3);
        base = kPi6;
    }
    const float t2 = t * t;
    float p = fmaf(t2, (float)(1.0 / 13.0), (float)(-1.0 / 11.0));
    p = fmaf(t2, p, (float)(1.0 / 9.0));
    p = fmaf(t2, p, (float)(-1.0 / 7.0));
    p = fmaf(t2, p, (float)(1.0 / 5.0));
    p = fmaf(t2, p, (float)(-1.0 / 3.0));
    float r = fmaf(t * t2, p, t) + base;
    if (ay > ax) r = kPio2 - r;
    if (x < 0.0f) r = kPiF - r;
    return (y < 0.0f) ? -r : r;
}

}  // namespace csp
