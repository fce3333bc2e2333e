// math_util.h -- orientation helpers with the interface of the reference's lib/math_util.h
// (double precision; the float conversion helper of the reference is not part of this API).
#ifndef CSP_DROPIN_MATH_UTIL_H
#define CSP_DROPIN_MATH_UTIL_H

#include <cmath>

#include "vector3d.h"

namespace mathUtil {

// Euler angles (yaw = atan2(nx, nz), pitch = asin(ny), roll = zrot in radians) of a normal and a
// z rotation given in degrees.
inline Vector3d normal_to_euler(const Vector3d& normal, double zrot_deg) {
    const Vector3d n = normal.normalized();
    return Vector3d(std::atan2(n[0], n[2]), std::asin(n[1]), zrot_deg * M_PI / 180.0);
}

// Global-to-local rotation (Spencer & Murty convention) of Euler angles (yaw, pitch, roll).
inline Matrix33d get_rotation_matrix_G2L(const Vector3d& e) {
    const double ca = std::cos(e[0]), sa = std::sin(e[0]);
    const double cb = std::cos(e[1]), sb = std::sin(e[1]);
    const double cg = std::cos(e[2]), sg = std::sin(e[2]);
    return Matrix33d{ca * cg + sa * sb * sg, -cb * sg, -sa * cg + ca * sb * sg,
                     ca * sg - sa * sb * cg, cb * cg,  -sa * sg - ca * sb * cg,
                     sa * cb,                sb,       ca * cb};
}

// local -> global with a global-to-local matrix (applies its transpose) and an origin
inline Vector3d local_to_global(const Vector3d& p, const Matrix33d& g2l, const Vector3d& origin) {
    return Vector3d(g2l(0, 0) * p[0] + g2l(1, 0) * p[1] + g2l(2, 0) * p[2],
                    g2l(0, 1) * p[0] + g2l(1, 1) * p[1] + g2l(2, 1) * p[2],
                    g2l(0, 2) * p[0] + g2l(1, 2) * p[1] + g2l(2, 2) * p[2]) + origin;
}

inline Vector3d global_to_local(const Vector3d& p, const Matrix33d& g2l, const Vector3d& origin) {
    const Vector3d t = p - origin;
    return Vector3d(g2l(0, 0) * t[0] + g2l(0, 1) * t[1] + g2l(0, 2) * t[2],
                    g2l(1, 0) * t[0] + g2l(1, 1) * t[1] + g2l(1, 2) * t[2],
                    g2l(2, 0) * t[0] + g2l(2, 1) * t[1] + g2l(2, 2) * t[2]);
}

}  // namespace mathUtil

#endif
