/* TEST INFRASTRUCTURE: host stand-in for the parts of the OptiX 8 device/host API that the
 * reference's device programs use (oracle/_ref only).  The OptiX SDK is not present; the
 * declared functions are implemented by oracle/ref_driver.cpp with OptiX's documented result
 * semantics (closest reported hit among primitives whose AABB the ray overlaps). */
#ifndef ORC_SHIM_OPTIX_H
#define ORC_SHIM_OPTIX_H
#include "cuda_runtime.h"
typedef unsigned long long OptixTraversableHandle;
typedef unsigned int OptixVisibilityMask;
enum OptixRayFlags { OPTIX_RAY_FLAG_NONE = 0 };
struct OptixAabb { float minX, minY, minZ, maxX, maxY, maxZ; };

uint3 optixGetLaunchIndex();
uint3 optixGetLaunchDimensions();
float3 optixGetWorldRayOrigin();
float3 optixGetWorldRayDirection();
float optixGetRayTmin();
float optixGetRayTmax();
unsigned int optixGetPrimitiveIndex();
unsigned int optixGetPayload_0();
unsigned int optixGetPayload_1();
void optixSetPayload_0(unsigned int p);
void optixSetPayload_1(unsigned int p);
unsigned int optixGetAttribute_0();
unsigned int optixGetAttribute_1();
unsigned int optixGetAttribute_2();
unsigned int optixGetAttribute_3();
unsigned int optixGetAttribute_4();
bool optixReportIntersection(float hitT, unsigned int hitKind, unsigned int a0, unsigned int a1, unsigned int a2,
                             unsigned int a3, unsigned int a4);
float3 optixTransformNormalFromObjectToWorldSpace(float3 n);
void optixTrace(OptixTraversableHandle handle, float3 rayOrigin, float3 rayDirection, float tmin, float tmax,
                float rayTime, OptixVisibilityMask visibilityMask, unsigned int rayFlags, unsigned int SBToffset,
                unsigned int SBTstride, unsigned int missSBTIndex, unsigned int& p0, unsigned int& p1);
#endif
