// Aperture.h -- aperture classes with the interface of the reference's lib/Aperture.h.
#ifndef CSP_DROPIN_APERTURE_H
#define CSP_DROPIN_APERTURE_H

#include "soltrace_type.h"

class Aperture {
public:
    Aperture() = default;
    virtual ~Aperture() = default;
    virtual ApertureType get_aperture_type() const = 0;
    virtual double get_width() const { return 0.0; }
    virtual double get_height() const { return 0.0; }
    virtual double get_radius() const { return 0.0; }
};

class ApertureCircle : public Aperture {
public:
    ApertureCircle() : radius_(1.0) {}
    explicit ApertureCircle(double r) : radius_(r) {}
    ApertureType get_aperture_type() const override { return ApertureType::CIRCLE; }
    void set_size(double r) { radius_ = r; }
    double get_radius() const override { return radius_; }
    double get_width() const override { return 2.0 * radius_; }
    double get_height() const override { return 2.0 * radius_; }

private:
    double radius_;
};

class ApertureRectangle : public Aperture {
public:
    ApertureRectangle() : x_(1.0), y_(1.0) {}
    ApertureRectangle(double x_dim, double y_dim) : x_(x_dim), y_(y_dim) {}
    ApertureType get_aperture_type() const override { return ApertureType::RECTANGLE; }
    double get_width() const override { return x_; }
    double get_height() const override { return y_; }

private:
    double x_, y_;
};

#endif
