// soltrace_type.h -- aperture / surface kinds (values of the reference's lib/soltrace_type.h).
#ifndef CSP_DROPIN_SOLTRACE_TYPE_H
#define CSP_DROPIN_SOLTRACE_TYPE_H

// exported C++ classes of libcsp_gb300.so
#define CSP_CXX_API __attribute__((visibility("default")))

enum class ApertureType { RECTANGLE, CIRCLE };
enum class SurfaceType { FLAT, PARABOLIC, MESH, CYLINDER };

struct SurfaceApertureMap {
    SurfaceType surfaceType;
    ApertureType apertureType;
    bool operator==(const SurfaceApertureMap& o) const {
        return surfaceType == o.surfaceType && apertureType == o.apertureType;
    }
};

#endif
