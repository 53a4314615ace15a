/*
 * Stand-in for Embree 3's public header (the library is absent), for the reference-renderer builds in
 * oracle/_ref only.  TEST INFRASTRUCTURE ONLY.  It declares the types and the calls the reference
 * makes (src/core/Ray.h, Scene.h/.cpp, TriangleMesh.cpp, Instance.cpp); oracle/ref_shim/rtcore_bvh.cpp
 * implements them for the integrator library, and the golden-vector library links none of them.
 */
#pragma once
#include <cstddef>
#include <cmath>

typedef struct RTCDeviceTy *RTCDevice;
typedef struct RTCSceneTy *RTCScene;
typedef struct RTCGeometryTy *RTCGeometry;
#define RTC_INVALID_GEOMETRY_ID ((unsigned)-1)
#define RTC_MAX_INSTANCE_LEVEL_COUNT 1
enum RTCSceneFlags { RTC_SCENE_FLAG_NONE = 0 };
enum RTCBuildQuality { RTC_BUILD_QUALITY_LOW, RTC_BUILD_QUALITY_MEDIUM, RTC_BUILD_QUALITY_HIGH };
enum RTCIntersectContextFlags { RTC_INTERSECT_CONTEXT_FLAG_INCOHERENT = 0, RTC_INTERSECT_CONTEXT_FLAG_COHERENT = 1 };
enum RTCGeometryType { RTC_GEOMETRY_TYPE_TRIANGLE, RTC_GEOMETRY_TYPE_INSTANCE };
enum RTCFormat { RTC_FORMAT_UINT3, RTC_FORMAT_FLOAT3, RTC_FORMAT_FLOAT3X4_COLUMN_MAJOR };
enum RTCBufferType { RTC_BUFFER_TYPE_INDEX, RTC_BUFFER_TYPE_VERTEX };
struct RTCBounds { float lower_x, lower_y, lower_z, align0, upper_x, upper_y, upper_z, align1; };
struct RTCRay { float org_x, org_y, org_z, tnear, dir_x, dir_y, dir_z, time, tfar; unsigned mask, id, flags; };
struct RTCHit { float Ng_x, Ng_y, Ng_z, u, v; unsigned primID, geomID, instID[RTC_MAX_INSTANCE_LEVEL_COUNT]; };
struct RTCRayHit { RTCRay ray; RTCHit hit; };
struct RTCIntersectContext { RTCIntersectContextFlags flags; void *filter; unsigned instID[RTC_MAX_INSTANCE_LEVEL_COUNT]; };
struct RTCCollision { unsigned geomID0, primID0, geomID1, primID1; };
typedef void (*RTCCollideFunc)(void *, RTCCollision *, unsigned);
inline void rtcInitIntersectContext(RTCIntersectContext *c) { c->flags = RTC_INTERSECT_CONTEXT_FLAG_INCOHERENT; c->filter = nullptr; }
/* implemented in rtcore_bvh.cpp (integrator library only) */
RTCDevice rtcNewDevice(const char *);
RTCScene rtcNewScene(RTCDevice);
void rtcSetSceneFlags(RTCScene, RTCSceneFlags);
void rtcSetSceneBuildQuality(RTCScene, RTCBuildQuality);
void rtcCommitScene(RTCScene);
void rtcGetSceneBounds(RTCScene, RTCBounds *);
void rtcIntersect1(RTCScene, RTCIntersectContext *, RTCRayHit *);
void rtcOccluded1(RTCScene, RTCIntersectContext *, RTCRay *);
unsigned rtcAttachGeometry(RTCScene, RTCGeometry);
void rtcAttachGeometryByID(RTCScene, RTCGeometry, unsigned);
void rtcDetachGeometry(RTCScene, unsigned);
RTCGeometry rtcNewGeometry(RTCDevice, RTCGeometryType);
void rtcSetSharedGeometryBuffer(RTCGeometry, RTCBufferType, unsigned, RTCFormat, const void *, size_t, size_t, size_t);
void rtcRetainGeometry(RTCGeometry);
void rtcCommitGeometry(RTCGeometry);
void rtcSetGeometryInstancedScene(RTCGeometry, RTCScene);
void rtcSetGeometryTransform(RTCGeometry, unsigned, RTCFormat, const void *);
void rtcCollide(RTCScene, RTCScene, RTCCollideFunc, void *);
