// Declarations of the Embree 3 names that XDG's public headers mention
// (primitive_ref.h, embree3.h, ray.h), so that the CUDA backend compiles
// against the unmodified XDG headers on a machine without Embree.  Nothing
// here is defined or called: the CUDA backend uses no Embree code.  Inside a
// real XDG build the genuine <embree3/rtcore.h> takes this file's place.
#pragma once

#include <cstdint>

#define RTC_INVALID_GEOMETRY_ID ((unsigned int)-1)

struct RTCSceneTy;
typedef RTCSceneTy* RTCScene;
struct RTCDeviceTy;
typedef RTCDeviceTy* RTCDevice;
struct RTCGeometryTy;
typedef RTCGeometryTy* RTCGeometry;

struct RTCRay {
  float org_x, org_y, org_z, tnear;
  float dir_x, dir_y, dir_z, time;
  float tfar;
  unsigned int mask, id, flags;
};
struct RTCHit {
  float Ng_x, Ng_y, Ng_z, u, v;
  unsigned int primID, geomID, instID[1];
};
struct RTCRayHit {
  RTCRay ray;
  RTCHit hit;
};
struct RTCPointQuery {
  float x, y, z, time, radius;
};
struct RTCIntersectContext {
  unsigned int flags;
  void* filter;
  unsigned int instID[1];
};
struct RTCIntersectFunctionNArguments;
struct RTCOccludedFunctionNArguments;
struct RTCBoundsFunctionArguments;
struct RTCPointQueryFunctionArguments;

void rtcInitIntersectContext(RTCIntersectContext* context);
void rtcIntersect1(RTCScene scene, RTCIntersectContext* context, RTCRayHit* rayhit);
void rtcOccluded1(RTCScene scene, RTCIntersectContext* context, RTCRay* ray);
