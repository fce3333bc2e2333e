// The CSV writer's float text (format_g6) equals std::to_chars(general, 6), the C++ stream's
// default format of the reference's writer, on every stride-th float bit pattern and on values
// next to the fast path's boundaries.  Usage: format_g6_check <stride>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "csp_format.h"

static bool same(float v) {
    char a[64], b[64];
    char* pa = csp::format_g6(v, a, a + sizeof a);
    char* pb = std::to_chars(b, b + sizeof b, v, std::chars_format::general, 6).ptr;
    if (pa - a == pb - b && std::memcmp(a, b, (size_t)(pa - a)) == 0) return true;
    std::printf("MISMATCH %a: '%.*s' vs '%.*s'\n", (double)v, (int)(pa - a), a, (int)(pb - b), b);
    return false;
}

int main(int argc, char** argv) {
    const uint64_t stride = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 97;
    std::atomic<uint64_t> bad{0}, checked{0};
    const unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            uint64_t nb = 0, nc = 0;
            for (uint64_t u = (uint64_t)t * stride; u < (1ull << 32); u += (uint64_t)nt * stride) {
                const uint32_t bits = (uint32_t)u;
                float v;
                std::memcpy(&v, &bits, 4);
                nb += same(v) ? 0 : 1;
                ++nc;
            }
            bad += nb;
            checked += nc;
        });
    for (auto& x : th) x.join();
    // around every power of ten and every rounding tie of six digits near them, both signs
    uint64_t nb = 0, nc = 0;
    for (int k = -45; k <= 39; ++k) {
        const double p = std::pow(10.0, k);
        for (double m : {1.0, 9.999995, 9.999994999, 9.9999950001, 1.000005, 1.0000049999, 5.000005, 2.5}) {
            float v = (float)(m * p);
            for (int s = 0; s < 64; ++s) {
                nb += same(v) ? 0 : 1;
                nb += same(-v) ? 0 : 1;
                nc += 2;
                v = std::nextafter(v, INFINITY);
            }
        }
    }
    for (float v : {0.0f, -0.0f, INFINITY, -INFINITY, NAN, 1e-45f, 3.4028235e38f, 1e-17f, 1e27f, 999999.5f, 99999.95f})
        nb += same(v) ? 0 : 1, ++nc;
    std::printf("checked %llu values, %llu mismatches\n", (unsigned long long)(checked.load() + nc),
                (unsigned long long)(bad.load() + nb));
    return bad.load() + nb ? 1 : 0;
}
