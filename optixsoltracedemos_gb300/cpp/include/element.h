// element.h -- optical element with the interface of the reference's lib/element.h.
//
// Orientation follows the reference: update_euler_angles() (called by SolTraceSystem::add_element
// and by update_element) freezes the orientation from the aim point and z rotation at that moment;
// later set_aim_point / set_zrot calls change nothing until the next update.  The reference's
// toDeviceGeometryData() (an OptiX record) is replaced by to_csp_element() (the C ABI record).
#ifndef CSP_DROPIN_ELEMENT_H
#define CSP_DROPIN_ELEMENT_H

#include <cstdint>
#include <memory>
#include <string>

#include "Aperture.h"
#include "Surface.h"
#include "csp_c_api.h"
#include "math_util.h"
#include "soltrace_type.h"
#include "vector3d.h"

class CSP_CXX_API ElementBase {
public:
    ElementBase() = default;
    virtual ~ElementBase() = default;
    virtual const Vector3d& get_origin() const = 0;
    virtual void set_origin(const Vector3d&) = 0;
    virtual const Vector3d& get_aim_point() const = 0;
    virtual void set_aim_point(const Vector3d&) = 0;
    virtual csp_element to_csp_element() const = 0;
};

class CSP_CXX_API Element : public ElementBase {
public:
    Element();
    ~Element() override = default;

    const Vector3d& get_origin() const override { return m_origin; }
    void set_origin(const Vector3d& o) override { m_origin = o; }
    void set_aim_point(const Vector3d& a) override { m_aim_point = a; }
    const Vector3d& get_aim_point() const override { return m_aim_point; }
    void set_zrot(double zrot) { m_zrot = zrot; }
    double get_zrot() const { return m_zrot; }
    std::shared_ptr<Aperture> get_aperture() const { return m_aperture; }
    std::shared_ptr<Surface> get_surface() const { return m_surface; }
    ApertureType get_aperture_type() const { return m_aperture->get_aperture_type(); }
    SurfaceType get_surface_type() const { return m_surface->get_surface_type(); }
    void set_aperture(const std::shared_ptr<Aperture>& a) { m_aperture = a; }
    void set_surface(const std::shared_ptr<Surface>& s) { m_surface = s; }

    // orientation from (aim_point, zrot), or from the element's own aim point and zrot
    void update_euler_angles(const Vector3d& aim_point, double zrot);
    void update_euler_angles();
    // set aim point and zrot and update the orientation
    void update_element(const Vector3d& aim_point, double zrot);

    const Vector3d& get_euler_angles() const { return m_euler_angles; }
    // local-to-global rotation (columns = local x, y, z axes)
    Matrix33d get_rotation_matrix() const;
    Vector3d get_upper_bounding_box() const { return m_upper_box_bound; }
    Vector3d get_lower_bounding_box() const { return m_lower_box_bound; }
    void compute_bounding_box();

    // the C ABI record of this element (orientation as of the last update); optical properties
    // default to the reference's behaviour (reflectivity 1, no errors)
    csp_element to_csp_element() const override;

    // optical properties (extension; the reference parses but never applies them)
    void set_optics(double reflectivity, double slope_error_rad, double specularity_error_rad) {
        m_reflectivity = reflectivity;
        m_slope_error = slope_error_rad;
        m_specularity_error = specularity_error_rad;
    }

private:
    Vector3d m_origin;
    Vector3d m_aim_point;
    Vector3d m_euler_angles;
    double m_zrot;
    Vector3d m_upper_box_bound, m_lower_box_bound;
    std::shared_ptr<Surface> m_surface;
    std::shared_ptr<Aperture> m_aperture;
    // pose used by the last orientation update
    Vector3d m_pose_origin, m_pose_aim;
    double m_pose_zrot;
    bool m_has_pose;
    double m_reflectivity = 1.0, m_slope_error = 0.0, m_specularity_error = 0.0;
};

#endif
