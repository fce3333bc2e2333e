// csp_format.h -- text of a float as the C++ stream prints it by default (printf "%g", six
// significant digits): the CSV writer's number format (lib/soltrace_system.cpp:208-264 writes the
// records through an std::ofstream with default precision).
//
// format_g6 gives the characters std::to_chars(first, last, v, std::chars_format::general, 6)
// gives, for every float (checked against it over all 2^32 bit patterns).  Fast path: the decimal
// exponent e from the binary one, then |v| as a double times (or divided by) the exact power of ten
// 10^(5 - e) puts the six digits in [1e5, 1e6) with one rounding, so the computed value is within
// 1.1e-10 of the exact one; unless that lies within 1e-9 of a rounding boundary (a half-integer, or
// 1e5 / 1e6 for the exponent), rounding it to the nearest integer gives the digits of the exact
// value.  Everything else (zero handled directly,
// non-finite values, |v| outside [1e-17, 1e27), values near a boundary) goes to std::to_chars.
#pragma once

#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace csp {

namespace fmt_detail {

// 10^k for k in [0, 22], exact in double
inline double pow10_exact(int k) {
    static const double t[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                 1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    return t[k];
}

inline char* slow(float v, char* p, char* end) { return std::to_chars(p, end, v, std::chars_format::general, 6).ptr; }

}  // namespace fmt_detail

// Writes the text of v at p (at most 16 characters; `end` bounds the fallback) and returns the end.
inline char* format_g6(float v, char* p, char* end) {
    using namespace fmt_detail;
    if (v == 0.0f) {
        if (std::signbit(v)) *p++ = '-';
        *p++ = '0';
        return p;
    }
    if (!std::isfinite(v)) return slow(v, p, end);
    const double a = std::fabs((double)v);
    if (!(a >= 1e-17 && a < 1e27)) return slow(v, p, end);
    // t = a 10^(5 - e), one rounding (the power of ten is exact); -1 outside the exact table
    auto scaled = [a](int e) {
        if (e <= 5) return 5 - e <= 22 ? a * pow10_exact(5 - e) : -1.0;
        return e - 5 <= 22 ? a / pow10_exact(e - 5) : -1.0;
    };
    // decimal exponent from the binary one: floor(b log10 2) or one less (1233 / 4096 < log10 2),
    // and the true exponent is at most one more than floor(b log10 2)
    uint32_t bits;
    std::memcpy(&bits, &v, 4);
    const int b = (int)((bits >> 23) & 0xffu) - 127;
    int e = (b * 1233) >> 12;
    double t = scaled(e);
    for (int k = 0; k < 2 && t >= 1e6 + 1e-9; ++k) t = scaled(++e);
    if (!(t >= 1e5 + 1e-9 && t < 1e6 - 1e-9)) return slow(v, p, end);
    const uint32_t ti = (uint32_t)t;  // floor: t is positive
    const double fl = (double)ti;
    const double fr = t - fl;  // exact (Sterbenz)
    if (fr > 0.5 - 1e-9 && fr < 0.5 + 1e-9) return slow(v, p, end);
    uint32_t d = ti + (fr > 0.5 ? 1u : 0u);
    if (d == 1000000u) {  // rounded up to the next power of ten
        d = 100000u;
        ++e;
    }
    char dig[6];
    const uint32_t hi = d / 10000u, mid = (d / 100u) % 100u, lo = d % 100u;
    dig[0] = (char)('0' + hi / 10u);
    dig[1] = (char)('0' + hi % 10u);
    dig[2] = (char)('0' + mid / 10u);
    dig[3] = (char)('0' + mid % 10u);
    dig[4] = (char)('0' + lo / 10u);
    dig[5] = (char)('0' + lo % 10u);
    int nd = 6;  // significant digits without trailing zeros
    while (nd > 1 && dig[nd - 1] == '0') --nd;
    if (v < 0.0f) *p++ = '-';
    if (e >= -4 && e < 6) {
        if (e >= 0) {
            for (int i = 0; i <= e; ++i) *p++ = dig[i];
            if (nd > e + 1) {
                *p++ = '.';
                for (int i = e + 1; i < nd; ++i) *p++ = dig[i];
            }
        } else {
            *p++ = '0';
            *p++ = '.';
            for (int i = 0; i < -e - 1; ++i) *p++ = '0';
            for (int i = 0; i < nd; ++i) *p++ = dig[i];
        }
    } else {
        *p++ = dig[0];
        if (nd > 1) {
            *p++ = '.';
            for (int i = 1; i < nd; ++i) *p++ = dig[i];
        }
        *p++ = 'e';
        int x = e;
        if (x < 0) {
            *p++ = '-';
            x = -x;
        } else {
            *p++ = '+';
        }
        if (x >= 10) {
            *p++ = (char)('0' + x / 10);
            *p++ = (char)('0' + x % 10);
        } else {
            *p++ = '0';
            *p++ = (char)('0' + x);
        }
    }
    return p;
}

}  // namespace csp
