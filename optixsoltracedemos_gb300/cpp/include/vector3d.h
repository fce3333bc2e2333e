// vector3d.h -- Vector3d / Matrix33d with the public interface of the reference's lib/vector3d.h
// (3-vector and row-major 3x3 matrix of doubles used by the scene model).
#ifndef CSP_DROPIN_VECTOR3D_H
#define CSP_DROPIN_VECTOR3D_H

#include <cmath>
#include <initializer_list>
#include <ostream>
#include <stdexcept>

class Vector3d {
public:
    Vector3d() : v_{0.0, 0.0, 0.0} {}
    Vector3d(double x, double y, double z) : v_{x, y, z} {}

    double operator[](int i) const { return v_[i]; }
    double& operator[](int i) { return v_[i]; }

    Vector3d operator+(const Vector3d& o) const { return {v_[0] + o.v_[0], v_[1] + o.v_[1], v_[2] + o.v_[2]}; }
    Vector3d operator-(const Vector3d& o) const { return {v_[0] - o.v_[0], v_[1] - o.v_[1], v_[2] - o.v_[2]}; }
    Vector3d operator*(double s) const { return {v_[0] * s, v_[1] * s, v_[2] * s}; }
    Vector3d operator/(double s) const { return {v_[0] / s, v_[1] / s, v_[2] / s}; }

    double dot(const Vector3d& o) const { return v_[0] * o.v_[0] + v_[1] * o.v_[1] + v_[2] * o.v_[2]; }
    Vector3d cross(const Vector3d& o) const {
        return {v_[1] * o.v_[2] - v_[2] * o.v_[1], v_[2] * o.v_[0] - v_[0] * o.v_[2], v_[0] * o.v_[1] - v_[1] * o.v_[0]};
    }
    double norm() const { return std::sqrt(dot(*this)); }
    // unit vector, or the zero vector for a zero-length input
    Vector3d normalized() const {
        const double n = norm();
        return n > 0 ? (*this) / n : Vector3d();
    }

    friend std::ostream& operator<<(std::ostream& os, const Vector3d& v) {
        return os << "(" << v.v_[0] << ", " << v.v_[1] << ", " << v.v_[2] << ")";
    }

private:
    double v_[3];
};

// Row-major 3x3 matrix; for a rotation, the basis getters return its columns.
class Matrix33d {
public:
    Matrix33d() : m_{1, 0, 0, 0, 1, 0, 0, 0, 1} {}
    explicit Matrix33d(const double a[9]) {
        for (int i = 0; i < 9; ++i) m_[i] = a[i];
    }
    Matrix33d(double a11, double a12, double a13, double a21, double a22, double a23, double a31, double a32,
              double a33)
        : m_{a11, a12, a13, a21, a22, a23, a31, a32, a33} {}
    Matrix33d(std::initializer_list<double> init) {
        if (init.size() != 9) throw std::runtime_error("must have exactly 9 elements.");
        int i = 0;
        for (double x : init) m_[i++] = x;
    }

    Matrix33d operator*(const Matrix33d& o) const {
        Matrix33d r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double acc = 0;
                for (int k = 0; k < 3; ++k) acc += m_[3 * i + k] * o.m_[3 * k + j];
                r.m_[3 * i + j] = acc;
            }
        return r;
    }
    Vector3d operator*(const Vector3d& v) const {
        return {m_[0] * v[0] + m_[1] * v[1] + m_[2] * v[2], m_[3] * v[0] + m_[4] * v[1] + m_[5] * v[2],
                m_[6] * v[0] + m_[7] * v[1] + m_[8] * v[2]};
    }
    double operator()(int i, int j) const { return m_[3 * i + j]; }
    Matrix33d transpose() const { return {m_[0], m_[3], m_[6], m_[1], m_[4], m_[7], m_[2], m_[5], m_[8]}; }

    Vector3d get_x_basis() const { return {m_[0], m_[3], m_[6]}; }
    Vector3d get_y_basis() const { return {m_[1], m_[4], m_[7]}; }
    Vector3d get_z_basis() const { return {m_[2], m_[5], m_[8]}; }

private:
    double m_[9];
};

#endif
