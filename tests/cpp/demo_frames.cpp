// Frame loop against the drop-in C++ API, the pattern of a dynamic scene: trace, write the CSV,
// move the sun, update -- repeated for a number of frames.  The scene is a parabolic mirror
// (curvatures 0.0170679 / 0.0370679, 1.0 x 1.95 m at (0, 5, 0)) facing a flat 2 x 4 m receiver at
// (0, 0, 10), sun vector (0, -20, 100) with a collimated sun; after every frame the sun vector's y
// component grows by 1.
// Usage: demo_frames <out_prefix> <num_rays> <frames>
// Writes <out_prefix>_<frame>.csv per frame and <out_prefix>.elements (the traced element records).
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <memory>
#include <string>

#include "lib/element.h"
#include "soltrace_system.h"

int main(int argc, char** argv) {
    if (argc < 4) {
        std::cerr << "usage: " << argv[0] << " <out_prefix> <num_rays> <frames>" << std::endl;
        return 2;
    }
    const std::string prefix = argv[1];
    const int num_rays = std::atoi(argv[2]);
    const int frames = std::atoi(argv[3]);
    SolTraceSystem system(num_rays);

    auto mirror = std::make_shared<Element>();
    mirror->set_origin(Vector3d(0.0, 5.0, 0.0));
    mirror->set_aim_point(Vector3d(0.0, -17.360680, 94.721360));
    mirror->set_zrot(0.0);
    auto para = std::make_shared<SurfaceParabolic>();
    para->set_curvature(0.0170679, 0.0370679);
    mirror->set_surface(para);
    mirror->set_aperture(std::make_shared<ApertureRectangle>(1.0, 1.95));
    system.add_element(mirror);

    auto receiver = std::make_shared<Element>();
    receiver->set_origin(Vector3d(0.0, 0.0, 10.0));
    receiver->set_aim_point(Vector3d(0.0, 5.0, 0.0));
    receiver->set_zrot(0.0);
    receiver->set_surface(std::make_shared<SurfaceFlat>());
    receiver->set_aperture(std::make_shared<ApertureRectangle>(2.0, 4.0));
    system.add_element(receiver);

    Vector3d sun(0.0, -20.0, 100.0);
    system.set_sun_vector(sun);
    system.set_sun_angle(0.0);
    system.initialize();

    FILE* f = std::fopen((prefix + ".elements").c_str(), "wb");
    if (!f) return 1;
    for (const auto& e : system.get_elements()) {
        const csp_element c = e->to_csp_element();
        std::fwrite(&c, sizeof c, 1, f);
    }
    std::fclose(f);

    for (int frame = 0; frame < frames; ++frame) {
        system.run();
        system.write_output(prefix + "_" + std::to_string(frame) + ".csv");
        sun[1] += 1.0;
        system.set_sun_vector(sun);
        system.update();
    }
    system.clean_up();
    std::cout << frames << " frames of " << num_rays << " rays" << std::endl;
    return 0;
}
