// dropin.cpp -- the reference's C++ API (SolTraceSystem, Element, soltrace_optix_interface) over
// the C ABI.  Behaviour follows lib/soltrace_system.cpp, lib/element.cpp and
// interface/soltrace_optix_interface.cpp of the reference; device work happens in libcsp_gb300.
#include <cstdio>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "element.h"
#include "soltrace_optix_interface.hpp"
#include "soltrace_system.h"

// ------------------------------------------------------------------------------ Element -------
Element::Element()
    : m_origin(0.0, 0.0, 0.0),
      m_aim_point(0.0, 0.0, 1.0),
      m_euler_angles(0.0, 0.0, 0.0),
      m_zrot(0.0),
      m_pose_zrot(0.0),
      m_has_pose(false) {}

void Element::update_euler_angles(const Vector3d& aim_point, double zrot) {
    m_pose_origin = m_origin;
    m_pose_aim = aim_point;
    m_pose_zrot = zrot;
    m_has_pose = true;
    const csp_element e = to_csp_element();
    double eu[3];
    csp_element_frame(&e, eu, nullptr, nullptr, nullptr);
    m_euler_angles = Vector3d(eu[0], eu[1], eu[2]);
}

void Element::update_euler_angles() { update_euler_angles(m_aim_point, m_zrot); }

void Element::update_element(const Vector3d& aim_point, double zrot) {
    m_aim_point = aim_point;
    m_zrot = zrot;
    update_euler_angles();
}

Matrix33d Element::get_rotation_matrix() const {
    const csp_element e = to_csp_element();
    double g[9];
    csp_element_frame(&e, nullptr, g, nullptr, nullptr);
    return Matrix33d(g).transpose();
}

void Element::compute_bounding_box() {
    const csp_element e = to_csp_element();
    double lo[3], hi[3];
    csp_element_frame(&e, nullptr, nullptr, lo, hi);
    m_lower_box_bound = Vector3d(lo[0], lo[1], lo[2]);
    m_upper_box_bound = Vector3d(hi[0], hi[1], hi[2]);
}

csp_element Element::to_csp_element() const {
    csp_element e;
    std::memset(&e, 0, sizeof e);
    for (int a = 0; a < 3; ++a) e.origin[a] = m_origin[a];
    if (m_has_pose) {
        // orientation frozen at the last update: same aim direction from the current origin
        bool moved = false;
        for (int a = 0; a < 3; ++a) moved |= (m_origin[a] != m_pose_origin[a]);
        for (int a = 0; a < 3; ++a)
            e.aim_point[a] = moved ? m_origin[a] + (m_pose_aim[a] - m_pose_origin[a]) : m_pose_aim[a];
        e.zrot_deg = m_pose_zrot;
    } else {
        for (int a = 0; a < 3; ++a) e.aim_point[a] = m_aim_point[a];
        e.zrot_deg = m_zrot;
    }
    if (m_aperture) {
        e.aperture = m_aperture->get_aperture_type() == ApertureType::RECTANGLE ? CSP_APERTURE_RECTANGLE
                                                                                 : CSP_APERTURE_CIRCLE;
        e.width = m_aperture->get_width();
        e.height = m_aperture->get_height();
    }
    if (m_surface) {
        switch (m_surface->get_surface_type()) {
            case SurfaceType::FLAT: e.surface = CSP_SURFACE_FLAT; break;
            case SurfaceType::PARABOLIC: e.surface = CSP_SURFACE_PARABOLIC; break;
            case SurfaceType::CYLINDER: e.surface = CSP_SURFACE_CYLINDER; break;
            default: e.surface = -1; break;
        }
        e.curv_x = m_surface->get_curvature_1();
        e.curv_y = m_surface->get_curvature_2();
    }
    e.reflectivity = m_reflectivity;
    e.slope_error = m_slope_error;
    e.specularity_error = m_specularity_error;
    return e;
}

// ------------------------------------------------------------------------------ SolTraceSystem -
SolTraceSystem::SolTraceSystem(int numSunPoints) : m_num_sunpoints((uint64_t)numSunPoints) {
    check(csp_create(&m_handle, 0, m_num_sunpoints), "csp_create");
}

SolTraceSystem::~SolTraceSystem() {
    // like the reference, device resources are released by clean_up(); a handle that is still
    // open here is released so that nothing leaks
    if (m_handle) csp_destroy(m_handle);
}

void SolTraceSystem::check(int status, const char* what) const {
    if (status != CSP_OK) throw std::runtime_error(std::string(what) + " failed: " + csp_last_error());
}

void SolTraceSystem::add_element(std::shared_ptr<Element> e) {
    e->update_euler_angles();
    m_element_list.push_back(e);
}

void SolTraceSystem::push_scene() {
    if (!m_handle) throw std::runtime_error("SolTraceSystem used after clean_up()");
    std::vector<csp_element> el;
    el.reserve(m_element_list.size());
    for (const auto& e : m_element_list) el.push_back(e->to_csp_element());
    check(csp_set_elements(m_handle, el.data(), (uint32_t)el.size()), "csp_set_elements");
    check(csp_set_sun_vector(m_handle, m_sun_vector[0], m_sun_vector[1], m_sun_vector[2]), "csp_set_sun_vector");
    const int flags = m_accurate ? CSP_SUN_ACCURATE : 0;
    if (m_sun_shape == CSP_SUN_GAUSSIAN)
        check(csp_set_sun_shape(m_handle, CSP_SUN_GAUSSIAN | flags, m_sun_sigma), "sun shape");
    else check(csp_set_sun_shape(m_handle, CSP_SUN_PILLBOX | flags, m_sun_angle), "sun shape");
}

void SolTraceSystem::initialize() {
    m_timer_setup.start();
    push_scene();
    check(csp_set_num_rays(m_handle, m_num_sunpoints), "csp_set_num_rays");
    check(csp_initialize(m_handle), "csp_initialize");
    m_timer_setup.stop();
    if (m_verbose) print_launch_params();
}

void SolTraceSystem::run() {
    if (!m_handle) throw std::runtime_error("SolTraceSystem used after clean_up()");
    m_timer_trace.start();
    check(csp_run(m_handle), "csp_run");
    m_timer_trace.stop();
}

void SolTraceSystem::run(uint64_t num_rays) {
    if (!m_handle) throw std::runtime_error("SolTraceSystem used after clean_up()");
    m_num_sunpoints = num_rays;
    check(csp_set_num_rays(m_handle, num_rays), "csp_set_num_rays");
    run();
}

void SolTraceSystem::update() {
    push_scene();
    check(csp_update(m_handle), "csp_update");
}

bool SolTraceSystem::read_st_input(const char* filename) {
    uint32_t n = 0;
    double sun[3], angle = 0.0;
    if (csp_parse_stinput(filename, nullptr, 0, &n, sun, &angle, 0) != CSP_OK) {
        if (m_verbose) std::printf("error in system input file: %s\n", csp_last_error());
        return false;
    }
    std::vector<csp_element> el(n);
    if (csp_parse_stinput(filename, el.data(), n, &n, sun, &angle, 0) != CSP_OK) return false;
    for (const csp_element& c : el) {
        auto e = std::make_shared<Element>();
        e->set_origin(Vector3d(c.origin[0], c.origin[1], c.origin[2]));
        e->set_aim_point(Vector3d(c.aim_point[0], c.aim_point[1], c.aim_point[2]));
        e->set_zrot(c.zrot_deg);
        e->set_aperture(std::make_shared<ApertureRectangle>(c.width, c.height));
        if (c.surface == CSP_SURFACE_PARABOLIC) e->set_surface(std::make_shared<SurfaceParabolic>(c.curv_x, c.curv_y));
        else if (c.surface == CSP_SURFACE_CYLINDER) {
            auto s = std::make_shared<SurfaceCylinder>();
            s->set_radius(c.width / 2);
            s->set_half_height(c.height / 2);
            e->set_surface(s);
        } else e->set_surface(std::make_shared<SurfaceFlat>());
        add_element(e);
    }
    set_sun_angle(angle);
    set_sun_vector(Vector3d(sun[0], sun[1], sun[2]));
    return true;
}

void SolTraceSystem::write_output(const std::string& filename) {
    if (!m_handle) throw std::runtime_error("SolTraceSystem used after clean_up()");
    const int rc = csp_write_output(m_handle, filename.c_str());
    if (rc == CSP_ERR_IO) {
        // the reference reports an unwritable file on stderr and returns
        std::cerr << "Error: Could not open the file " << filename << " for writing." << std::endl;
        return;
    }
    check(rc, "csp_write_output");
}

void SolTraceSystem::clean_up() {
    if (m_handle) {
        check(csp_destroy(m_handle), "csp_destroy");
        m_handle = nullptr;
    }
}

double SolTraceSystem::get_time_trace() { return m_timer_trace.get_time_sec(); }
double SolTraceSystem::get_time_setup() { return m_timer_setup.get_time_sec(); }

void SolTraceSystem::print_launch_params() {
    float p[16];
    check(csp_get_sun_plane(m_handle, p), "csp_get_sun_plane");
    auto edge = [&](int a, int b) {
        const float dx = p[a] - p[b], dy = p[a + 1] - p[b + 1], dz = p[a + 2] - p[b + 2];
        return std::sqrt(dx * dx + dy * dy + dz * dz);
    };
    std::cout << "print launch params: " << std::endl;
    std::cout << "width: " << m_num_sunpoints << std::endl;
    std::cout << "height: 1" << std::endl;
    std::cout << "max_depth: " << CSP_MAX_TRACE_DEPTH << std::endl;
    std::cout << "sun_vector: " << p[0] << " " << p[1] << " " << p[2] << std::endl;
    std::cout << "max_sun_angle: " << (float)m_sun_angle << std::endl;
    for (int k = 0; k < 4; ++k)
        std::cout << "sun_v" << k << ": " << p[3 + 3 * k] << " " << p[4 + 3 * k] << " " << p[5 + 3 * k] << std::endl;
    std::cout << "sun_box_edge_a: " << edge(3, 6) << std::endl;
    std::cout << "sun_box_edge_b: " << edge(6, 9) << std::endl;
}

void SolTraceSystem::set_seed(uint64_t seed, uint32_t instance) {
    if (!m_handle) throw std::runtime_error("SolTraceSystem used after clean_up()");
    check(csp_set_seed(m_handle, seed, instance), "csp_set_seed");
}

void SolTraceSystem::set_sun_shape_gaussian(double sigma_rad) {
    m_sun_shape = CSP_SUN_GAUSSIAN;
    m_sun_sigma = sigma_rad;
}

void SolTraceSystem::set_accurate_arithmetic(bool enable) { m_accurate = enable; }

void SolTraceSystem::set_record_element_ids(bool enable) {
    if (!m_handle) throw std::runtime_error("SolTraceSystem used after clean_up()");
    check(csp_set_record_ids(m_handle, enable ? 1 : 0), "csp_set_record_ids");
}

void SolTraceSystem::copy_hits(float* dst, uint32_t* ids, uint64_t first, uint64_t count) {
    if (!m_handle) throw std::runtime_error("SolTraceSystem used after clean_up()");
    check(csp_copy_hits(m_handle, dst, ids, first, count), "csp_copy_hits");
}

// ------------------------------------------------------------------------------ facade --------
struct soltrace_optix_interface::Impl {
    SolTraceSystem sys;
    explicit Impl(int n) : sys(n) {}
};

soltrace_optix_interface::soltrace_optix_interface(int num_rays) : impl(new Impl(num_rays)) {}
soltrace_optix_interface::~soltrace_optix_interface() = default;
void soltrace_optix_interface::set_sun_vector(double x, double y, double z) { impl->sys.set_sun_vector(Vector3d(x, y, z)); }
void soltrace_optix_interface::set_sun_angle(double angle) { impl->sys.set_sun_angle(angle); }
void soltrace_optix_interface::set_sun_points(int n) { impl->sys.set_sun_points(n); }
void soltrace_optix_interface::read_st_input(const char* path) { impl->sys.read_st_input(path); }
void soltrace_optix_interface::initialize() { impl->sys.initialize(); }
void soltrace_optix_interface::run() { impl->sys.run(); }
void soltrace_optix_interface::write_output(const char* path) { impl->sys.write_output(path); }
