// Harness around the reference's geometry code -- TEST INFRASTRUCTURE.
//
// oracle/Makefile (target `geo`) compiles this file with the reference's
// GeoTools/GeoTools.cpp, GeoTools/BoundingBoxes.cpp and
// MathTools/polynomial_equations.cpp (unmodified, read where they lie) into
// oracle/_ref/libgeo_ref.so.  The tests use it to pin the lattice set-up
// (a2c_lattice_build) against the reference's own signed distances and
// bounding boxes, with the calculators built from the geometry parameters
// the way SpaceInitializer::SortUserSpecifiedGeometries builds them
// (SpaceInitializer.cpp:326-600) and the boxes taken the way
// FindLatticeDomainBoundingBox takes them (:726-880).  Never shipped.
#include <cmath>
#include <cstdint>

#include "BoundingBoxes.h"
#include "DistancePointToCylinderCone.h"
#include "DistancePointToCylinderSphere.h"
#include "DistancePointToParallelepiped.h"
#include "DistancePointToPlane.h"
#include "DistancePointToSphere.h"
#include "DistancePointToSpheroid.h"
#include "Vector3D.h"

using namespace GeoTools;

namespace {

// parameter layout of a2c_geometry.p, per type (include/a2c_gpp.h)
enum { PLANE = 0, CYL_CONE = 1, CYL_SPHERE = 2, SPHERE = 3, PARALLELEPIPED = 4, SPHEROID = 5 };

}  // namespace

extern "C" {

// Signed distance (> 0 outside) of n points q (3 each) to geometry `type`.
int geo_ref_distance(int type, const double *p, const double *q, int64_t n, double *out) {
  Vec3D x0(p[0], p[1], p[2]);
  if (type == PLANE) {
    Vec3D dir(p[3], p[4], p[5]);
    DistanceFromPointToPlane c(x0, dir);
    for (int64_t i = 0; i < n; ++i) out[i] = c.Calculate((double *)(q + 3 * i));
  } else if (type == SPHERE) {
    DistanceFromPointToSphere c(x0, p[3]);
    for (int64_t i = 0; i < n; ++i) out[i] = c.Calculate((double *)(q + 3 * i));
  } else if (type == PARALLELEPIPED) {
    Vec3D oa(p[3], p[4], p[5]);
    oa -= x0;
    Vec3D ob(p[6], p[7], p[8]);
    ob -= x0;
    Vec3D oc(p[9], p[10], p[11]);
    oc -= x0;
    DistanceFromPointToParallelepiped c(x0, oa, ob, oc);
    for (int64_t i = 0; i < n; ++i) out[i] = c.Calculate((double *)(q + 3 * i));
  } else if (type == SPHEROID) {
    Vec3D axis(p[3], p[4], p[5]);
    DistanceFromPointToSpheroid c(x0, axis, p[6], p[7]);
    for (int64_t i = 0; i < n; ++i) out[i] = c.Calculate((double *)(q + 3 * i));
  } else if (type == CYL_CONE) {
    Vec3D dir(p[3], p[4], p[5]);
    double L = p[7], R = p[6];
    double tan_alpha = tan(p[8] / 180.0 * acos(-1.0));
    double Hmax = R / tan_alpha;
    double H = std::min(p[9], Hmax);
    DistanceFromPointToCylinderCone c(x0, dir, L, R, tan_alpha, H);
    for (int64_t i = 0; i < n; ++i) out[i] = c.Calculate((double *)(q + 3 * i));
  } else if (type == CYL_SPHERE) {
    Vec3D dir(p[3], p[4], p[5]);
    DistanceFromPointToCylinderSphere c(x0, dir, p[7], p[6], p[8] != 0.0, p[9] != 0.0);
    for (int64_t i = 0; i < n; ++i) out[i] = c.Calculate((double *)(q + 3 * i));
  } else {
    return 1;
  }
  return 0;
}

// Bounding box of an interior geometry in the reference's lattice
// coordinates (origin O, lattice vectors abc[9]).
int geo_ref_bbox(int type, const double *p, const double *O_, const double *abc, double *lmin_, double *lmax_) {
  Vec3D O(O_[0], O_[1], O_[2]);
  Vec3D a(abc[0], abc[1], abc[2]), b(abc[3], abc[4], abc[5]), c(abc[6], abc[7], abc[8]);
  Vec3D lmin, lmax;
  Vec3D x0(p[0], p[1], p[2]);
  if (type == SPHERE) {
    GetBoundingBoxOfSphere(x0, p[3], O, a, b, c, lmin, lmax);
  } else if (type == PARALLELEPIPED) {
    Vec3D oa(p[3], p[4], p[5]);
    oa -= x0;
    Vec3D ob(p[6], p[7], p[8]);
    ob -= x0;
    Vec3D oc(p[9], p[10], p[11]);
    oc -= x0;
    GetBoundingBoxOfParallelepiped(x0, oa, ob, oc, O, a, b, c, lmin, lmax);
  } else if (type == SPHEROID) {
    Vec3D axis(p[3], p[4], p[5]);
    GetBoundingBoxOfSpheroid(x0, axis, p[6], p[7], O, a, b, c, lmin, lmax);
  } else if (type == CYL_CONE) {
    Vec3D dir(p[3], p[4], p[5]);
    dir /= dir.norm();
    double L = p[7], R = p[6];
    double tan_alpha = tan(p[8] / 180.0 * acos(-1.0));
    double Hmax = R / tan_alpha;
    double H = std::min(p[9], Hmax);
    GetBoundingBoxOfCylinderCone(x0, dir, R, L, tan_alpha, H, O, a, b, c, lmin, lmax);
  } else if (type == CYL_SPHERE) {
    Vec3D dir(p[3], p[4], p[5]);
    dir /= dir.norm();
    GetBoundingBoxOfCylinderSphere(x0, dir, p[6], p[7], p[8] != 0.0, p[9] != 0.0, O, a, b, c, lmin, lmax);
  } else {
    return 1;
  }
  for (int i = 0; i < 3; ++i) {
    lmin_[i] = lmin[i];
    lmax_[i] = lmax[i];
  }
  return 0;
}

}  // extern "C"
