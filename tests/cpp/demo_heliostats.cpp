// Demo against the drop-in C++ API: three flat heliostats and a flat receiver (or a .stinput
// file), traced through SolTraceSystem; writes the reference's CSV and a raw dump of the hit
// records.  Usage: demo_heliostats <out.csv> <out.raw> <num_rays> [file.stinput]
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "lib/element.h"
#include "soltrace_optix_interface.hpp"
#include "soltrace_system.h"
#include "timer.h"

static std::shared_ptr<Element> heliostat(const Vector3d& origin, const Vector3d& aim) {
    auto e = std::make_shared<Element>();
    e->set_origin(origin);
    e->set_aim_point(aim);
    e->set_zrot(0.0);
    e->set_surface(std::make_shared<SurfaceFlat>());
    e->set_aperture(std::make_shared<ApertureRectangle>(1.0, 1.95));
    return e;
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::cerr << "usage: " << argv[0] << " <out.csv> <out.raw> <num_rays> [file.stinput]" << std::endl;
        return 2;
    }
    const int num_rays = std::atoi(argv[3]);
    SolTraceSystem system(num_rays);
    if (argc > 4) {
        if (!system.read_st_input(argv[4])) {
            std::cerr << "could not read " << argv[4] << std::endl;
            return 1;
        }
    } else {
        // aim points on the bisector of the sun vector and the receiver direction
        const Vector3d sun(0.0, -1.0, 1.0), recv(0.0, 0.0, 10.0);
        const Vector3d origins[3] = {Vector3d(-5, 5, 0), Vector3d(0, 5, 0), Vector3d(5, 5, 0)};
        for (const Vector3d& o : origins) {
            const Vector3d n = (sun.normalized() + (recv - o).normalized()).normalized();
            system.add_element(heliostat(o, o + n * 100.0));
        }
        auto receiver = std::make_shared<Element>();
        receiver->set_origin(recv);
        receiver->set_aim_point(Vector3d(0.0, 1.0, 10.0));
        receiver->set_zrot(0.0);
        receiver->set_surface(std::make_shared<SurfaceFlat>());
        receiver->set_aperture(std::make_shared<ApertureRectangle>(2.0, 2.0));
        system.add_element(receiver);
        system.set_sun_vector(sun);
        system.set_sun_angle(0.00465);
    }
    system.initialize();
    system.run();
    std::cout << "heliostats " << system.get_num_heliostats() << ", receivers " << system.get_num_receivers()
              << ", setup " << system.get_time_setup() << " s, trace " << system.get_time_trace() << " s" << std::endl;
    system.write_output(argv[1]);
    std::vector<float> hits((size_t)num_rays * CSP_MAX_TRACE_DEPTH * 4);
    system.copy_hits(hits.data(), nullptr, 0, (uint64_t)num_rays);
    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 1;
    std::fwrite(hits.data(), sizeof(float), hits.size(), f);
    std::fclose(f);
    // the element records actually traced, for an exact comparison
    f = std::fopen((std::string(argv[2]) + ".elements").c_str(), "wb");
    if (!f) return 1;
    for (const auto& e : system.get_elements()) {
        const csp_element c = e->to_csp_element();
        std::fwrite(&c, sizeof c, 1, f);
    }
    std::fclose(f);
    system.clean_up();

    // the facade, once, on the same scene description when a file is given
    if (argc > 4) {
        soltrace_optix_interface facade(1000);
        facade.read_st_input(argv[4]);
        facade.initialize();
        facade.run();
        facade.write_output((std::string(argv[1]) + ".facade.csv").c_str());
    }
    return 0;
}
