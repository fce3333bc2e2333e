// soltrace_optix_interface.hpp -- facade with the interface of the reference's
// interface/soltrace_optix_interface.hpp (pimpl over SolTraceSystem).
#pragma once
#include <memory>

#include "soltrace_type.h"

class CSP_CXX_API soltrace_optix_interface {
public:
    explicit soltrace_optix_interface(int num_rays = 10000);
    ~soltrace_optix_interface();

    void set_sun_vector(double x, double y, double z);
    void set_sun_angle(double angle);
    void set_sun_points(int n);

    void read_st_input(const char* stinputPath);
    void initialize();
    void run();
    void write_output(const char* outPath);

private:
    struct Impl;
    std::unique_ptr<Impl> impl;
};
