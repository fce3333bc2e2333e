// Surface.h -- surface classes with the interface of the reference's lib/Surface.h.
#ifndef CSP_DROPIN_SURFACE_H
#define CSP_DROPIN_SURFACE_H

#include "soltrace_type.h"

class Surface {
public:
    Surface() = default;
    virtual ~Surface() = default;
    virtual SurfaceType get_surface_type() const = 0;
    virtual double get_curvature_1() const { return 0.0; }
    virtual double get_curvature_2() const { return 0.0; }
};

// z = c1/2 x^2 + c2/2 y^2 in the element frame
class SurfaceParabolic : public Surface {
public:
    SurfaceParabolic() : c1_(0.0), c2_(0.0) {}
    SurfaceParabolic(double c1, double c2) : c1_(c1), c2_(c2) {}
    SurfaceType get_surface_type() const override { return SurfaceType::PARABOLIC; }
    void set_curvature(double c1, double c2) {
        c1_ = c1;
        c2_ = c2;
    }
    double get_curvature_1() const override { return c1_; }
    double get_curvature_2() const override { return c2_; }

private:
    double c1_, c2_;
};

class SurfaceFlat : public Surface {
public:
    SurfaceType get_surface_type() const override { return SurfaceType::FLAT; }
};

// Cylinder with end caps.  As in the reference, the traced radius and height come from the
// element's rectangular aperture (width = 2 r, height = full height); these fields are descriptive.
class SurfaceCylinder : public Surface {
public:
    SurfaceType get_surface_type() const override { return SurfaceType::CYLINDER; }
    void set_radius(double r) { radius_ = r; }
    double get_radius() const { return radius_; }
    void set_half_height(double h) { half_height_ = h; }
    double get_half_height() const { return half_height_; }

private:
    double radius_ = 1.0;
    double half_height_ = 1.0;
};

#endif
