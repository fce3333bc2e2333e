// soltrace_system.h -- SolTraceSystem with the public interface of the reference's
// lib/soltrace_system.h, running on the GB300 trace path through the C ABI (csp_c_api.h).
// Errors from the device path throw std::runtime_error, as the reference's CUDA/OptiX checks do.
#ifndef CSP_DROPIN_SOLTRACE_SYSTEM_H
#define CSP_DROPIN_SOLTRACE_SYSTEM_H

#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "csp_c_api.h"
#include "element.h"
#include "timer.h"
#include "vector3d.h"

class CSP_CXX_API SolTraceSystem {
public:
    explicit SolTraceSystem(int numSunPoints);
    ~SolTraceSystem();

    void initialize();
    void run();
    // run with a new ray count (reallocates the hit buffer when it grows)
    void run(uint64_t num_rays);
    void update();
    bool read_st_input(const char* filename);
    void write_output(const std::string& filename);
    void clean_up();

    void set_verbose(bool verbose) { m_verbose = verbose; }
    void set_sun_points(int num) { m_num_sunpoints = (uint64_t)num; }
    void set_sun_vector(Vector3d vect) { m_sun_vector = vect; }
    void set_sun_angle(double angle) { m_sun_angle = angle; }

    size_t get_num_heliostats() const { return m_element_list.size() - 1; }
    int get_num_receivers() const { return 1; }

    void add_element(std::shared_ptr<Element> element);

    double get_time_trace();
    double get_time_setup();
    void print_launch_params();

    // ---- extensions
    void set_seed(uint64_t seed, uint32_t instance = 0);
    // Gaussian sun of per-axis sigma (rad) instead of the pillbox of set_sun_angle
    void set_sun_shape_gaussian(double sigma_rad);
    // trace in the cancellation-free float formulas (CSP_SUN_ACCURATE: cone sampler, cylinder
    // roots) instead of the reference's; false (the default) traces the reference's arithmetic
    void set_accurate_arithmetic(bool enable);
    void set_record_element_ids(bool enable);
    const std::vector<std::shared_ptr<Element>>& get_elements() const { return m_element_list; }
    uint64_t get_num_rays() const { return m_num_sunpoints; }
    // copy hit records [first, first + count) ({stage, x, y, z} float4 per slot, 5 slots per ray)
    void copy_hits(float* dst, uint32_t* ids, uint64_t first, uint64_t count);
    csp_handle handle() const { return m_handle; }

private:
    void check(int status, const char* what) const;
    void push_scene();

    csp_handle m_handle = nullptr;
    uint64_t m_num_sunpoints;
    bool m_verbose = false;
    Vector3d m_sun_vector{0.0, 0.0, 1.0};
    double m_sun_angle = 0.0;
    int m_sun_shape = CSP_SUN_PILLBOX;
    bool m_accurate = false;
    double m_sun_sigma = 0.0;
    std::vector<std::shared_ptr<Element>> m_element_list;
    Timer m_timer_setup, m_timer_trace;
};

#endif
