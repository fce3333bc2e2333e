// Element records built in ranges on several threads (build_elements with a ParallelFor, as the
// server does for large submissions) equal the serial build byte for byte, and a failing element
// gives the same error (the lowest failing index).  Usage: scene_build_ranges <elements.bin>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "csp_scene.h"

using namespace csp;

template <class T>
static bool same(const std::vector<T>& a, const std::vector<T>& b) {
    return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0);
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    std::vector<csp_element> el(1 << 16);
    const size_t n = std::fread(el.data(), sizeof(csp_element), el.size(), f);
    std::fclose(f);
    el.resize(n);
    const ParallelFor pf = [](size_t tasks, const std::function<void(size_t)>& body) {
        std::vector<std::thread> th;
        const size_t workers = 5;
        for (size_t w = 0; w < workers; ++w)
            th.emplace_back([&, w] {
                for (size_t k = w; k < tasks; k += workers) body(k);
            });
        for (auto& t : th) t.join();
    };
    HostScene a, b;
    std::string ea, eb;
    const int ra = build_elements(el.data(), (uint32_t)n, a, ea);
    const int rb = build_elements(el.data(), (uint32_t)n, b, eb, pf);
    if (ra != CSP_OK || rb != CSP_OK) {
        std::printf("FAIL build %d %d\n", ra, rb);
        return 1;
    }
    if (!same(a.prims, b.prims) || !same(a.optics, b.optics) || !same(a.aabbs, b.aabbs) || !same(a.prune, b.prune) ||
        !same(a.types, b.types)) {
        std::printf("FAIL records differ\n");
        return 1;
    }
    // two bad elements in different ranges: both forms name the lower one
    el[n - 2 * kBuildChunk - 3].surface = 99;
    el[kBuildChunk + 7].surface = 98;
    const int rc = build_elements(el.data(), (uint32_t)n, a, ea);
    const int rd = build_elements(el.data(), (uint32_t)n, b, eb, pf);
    if (rc != rd || rc == CSP_OK || ea != eb) {
        std::printf("FAIL errors: %d '%s' / %d '%s'\n", rc, ea.c_str(), rd, eb.c_str());
        return 1;
    }
    std::printf("OK %zu elements, error '%s'\n", n, ea.c_str());
    return 0;
}
