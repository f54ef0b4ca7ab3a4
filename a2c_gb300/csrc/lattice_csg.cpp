// Lattice set-up from a lattice description (the reference's
// SpaceInitializer::CreateOneLattice, SpaceInitializer.cpp:119-320, with
// CheckAndAddSitesInCell :603-724 and FindLatticeDomainBoundingBox
// :726-880), on the host.
//
// Which cells are visited follows the reference exactly: the bounding box
// of every interior finite geometry is taken in GeoTools' way
// (BoundingBoxes.cpp: the vertices of an enclosing parallelepiped projected
// on each lattice direction and divided by its length, which is the
// lattice coordinate only for orthogonal lattice vectors), its union is
// floored/ceiled to cells, and cells are visited c, b, a.  The arithmetic
// of those steps is the reference's, so the same cells are visited.
//
// Which sites are kept: geometries are applied in their operation order,
// starting from "inside" (all of space); an Intersection geometry is tested
// only while the site is inside, a Union geometry only while it is outside.
// Planes keep the positive side (distance > 0); the other geometries
// (Side = Interior / Exterior) call a point on their boundary outside, as
// the reference's signed distance >= 0 does.  Plane, sphere and
// parallelepiped decisions use the same expressions as the reference's
// signed distances and agree with them bit for bit; spheroid and the two
// cylinder shapes use exact closed-form inside tests, which agree with the
// reference's computed distances except within rounding of their surfaces.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "a2c_gpp.h"

namespace {

struct V {
  double v[3];
  double &operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};
V mk(double x, double y, double z) { return V{{x, y, z}}; }
V operator+(const V &a, const V &b) { return mk(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
V operator-(const V &a, const V &b) { return mk(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
V operator*(double c, const V &a) { return mk(c * a[0], c * a[1], c * a[2]); }
double dot(const V &a, const V &b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
V cross(const V &a, const V &b) {
  return mk(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
double norm(const V &a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
V scale_by_inverse(V a, double c) {  // a times 1/c (in-place division of the reference's vectors)
  c = 1.0 / c;
  return mk(a[0] * c, a[1] * c, a[2] * c);
}
V divide(const V &a, double c) { return mk(a[0] / c, a[1] / c, a[2] / c); }
V vec(const double *p) { return mk(p[0], p[1], p[2]); }

struct Fail {
  std::string msg;
};

// Two unit vectors completing the unit vector U0 to a right-handed
// orthonormal basis, chosen as GeoTools::GetOrthonormalVectors chooses them
// (GeoTools.cpp:473-520): a coordinate axis where U0 has a zero component.
void orthonormal(const V &U0, V &U1, V &U2) {
  U1 = mk(0.0, 0.0, 0.0);
  U2 = mk(0.0, 0.0, 0.0);
  bool done = false;
  for (int i = 0; i < 3 && !done; ++i) {
    if (U0[i] == 0) {
      U1[i] = 1.0;
      bool got2 = false;
      for (int j = i + 1; j < 3; ++j)
        if (U0[j] == 0) {
          U2[j] = 1.0;
          got2 = true;
          break;
        }
      if (!got2) {
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
        U2[i1] = -U0[i2];
        U2[i2] = U0[i1];
        U2 = scale_by_inverse(U2, norm(U2));
      }
      done = true;
    }
  }
  if (!done) {
    U1 = mk(1.0, 0.0, -U0[0] / U0[2]);
    U1 = scale_by_inverse(U1, norm(U1));
    U2 = mk(1.0, -(U0[2] * U0[2] / U0[0] + U0[0]) / U0[1], U0[2] / U0[0]);
    U2 = scale_by_inverse(U2, norm(U2));
  }
  if (dot(cross(U0, U1), U2) < 0.0) std::swap(U1, U2);
}

struct Frame {  // the lattice: origin and the three lattice vectors
  V O, d[3];
};

// Bounding box in the reference's lattice "coordinates" of the
// parallelepiped P + [0,1]^3 (PA, PB, PC) (BoundingBoxes.cpp:111-184).
void bbox_parallelepiped(const V &P, const V &PA, const V &PB, const V &PC, const Frame &F, V &lmin, V &lmax) {
  V v[8];
  v[0] = P;
  v[1] = P + PA;
  v[2] = P + PB;
  v[3] = P + PC;
  v[4] = v[1] + PB;
  v[5] = v[1] + PC;
  v[6] = v[2] + PC;
  v[7] = v[4] + PC;
  V dir[3];
  double dn[3];
  for (int i = 0; i < 3; ++i) {
    dn[i] = norm(F.d[i]);
    dir[i] = scale_by_inverse(F.d[i], dn[i]);
  }
  lmin = mk(DBL_MAX, DBL_MAX, DBL_MAX);
  lmax = mk(-DBL_MAX, -DBL_MAX, -DBL_MAX);
  for (int i = 0; i < 8; ++i) {
    const V Ov = v[i] - F.O;
    for (int j = 0; j < 3; ++j) {
      const double c = dot(Ov, dir[j]);
      if (c < lmin[j]) lmin[j] = c;
      if (c > lmax[j]) lmax[j] = c;
    }
  }
  for (int i = 0; i < 3; ++i) {
    lmin[i] /= dn[i];
    lmax[i] /= dn[i];
  }
}

// (BoundingBoxes.cpp:85-108)
void bbox_sphere(const V &c, double r, const Frame &F, V &lmin, V &lmax) {
  const V Oc = c - F.O;
  for (int i = 0; i < 3; ++i) {
    const double dn = norm(F.d[i]);
    const V dir = scale_by_inverse(F.d[i], dn);
    const double proj = dot(Oc, dir);
    lmin[i] = (proj - r) / dn;
    lmax[i] = (proj + r) / dn;
  }
}

struct Geom {
  a2c_geometry g;
  // derived
  V x0, n;                  // plane point and unit normal; cylinder base and unit axis; spheroid centre, axis
  double R = 0, L = 0, tan_a = 0, H = 0, A = 0;
  bool front = false, back = false;
  V face_o[6], face_n[6];   // parallelepiped faces
};

Geom prepare(const a2c_geometry &g) {
  Geom G;
  G.g = g;
  const double *p = g.p;
  switch (g.type) {
    case A2C_GEOM_PLANE: {  // DistanceFromPointToPlane
      G.x0 = vec(p);
      const V dir = vec(p + 3);
      const double nn = norm(dir);
      if (!(nn > 0)) throw Fail{"plane with a zero normal"};
      G.n = scale_by_inverse(dir, nn);
      break;
    }
    case A2C_GEOM_SPHERE:
      G.x0 = vec(p);
      G.R = p[3];
      break;
    case A2C_GEOM_PARALLELEPIPED: {  // vertices P, A, B, C (DistanceFromPointToParallelepiped)
      const V O = vec(p), OA = vec(p + 3) - O, OB = vec(p + 6) - O, OC = vec(p + 9) - O;
      if (norm(OA) == 0 || norm(OB) == 0 || norm(OC) == 0 || dot(cross(OA, OB), OC) <= 0.0)
        throw Fail{"parallelepiped with overlapping vertices or violating the right-hand rule"};
      const V A = O + OA, B = O + OB, C = O + OC, D = A + OB, E = A + OC, Fv = B + OC;
      const V o[6] = {O, O, A, B, O, C};
      const V e1[6] = {OB, OA, D - A, Fv - B, OC, E - C};
      const V e2[6] = {OA, OC, E - A, D - B, OB, Fv - C};
      for (int f = 0; f < 6; ++f) {
        const V nrm = cross(e1[f], e2[f]);
        G.face_o[f] = o[f];
        G.face_n[f] = scale_by_inverse(nrm, norm(nrm));
      }
      G.x0 = O;
      break;
    }
    case A2C_GEOM_SPHEROID: {
      G.x0 = vec(p);
      G.n = vec(p + 3);
      const double nn = norm(G.n);
      if (!(nn > 0) || !(p[6] > 0) || !(p[7] > 0)) throw Fail{"spheroid with a zero axis, length or radius"};
      G.n = divide(G.n, nn);
      G.A = p[6];
      G.R = p[7];
      break;
    }
    case A2C_GEOM_CYLINDER_CONE:
    case A2C_GEOM_CYLINDER_SPHERE: {
      G.x0 = vec(p);
      const V dir = vec(p + 3);
      const double nn = norm(dir);
      if (!(nn > 0)) throw Fail{"cylinder with a zero axis"};
      G.n = scale_by_inverse(dir, nn);
      G.R = p[6];
      G.L = p[7];
      if (g.type == A2C_GEOM_CYLINDER_CONE) {
        G.tan_a = std::tan(p[8] / 180.0 * std::acos(-1.0));
        const double Hmax = G.R / G.tan_a;
        G.H = std::min(p[9], Hmax);
      } else {
        G.front = p[8] != 0.0;
        G.back = p[9] != 0.0;
      }
      break;
    }
    default:
      throw Fail{"unknown geometry type " + std::to_string(g.type)};
  }
  return G;
}

// True when q is outside the geometry or on its boundary (the reference's
// signed distance >= 0).
bool outside(const Geom &G, const V &q) {
  switch (G.g.type) {
    case A2C_GEOM_SPHERE:
      return norm(q - G.x0) - G.R >= 0.0;
    case A2C_GEOM_PARALLELEPIPED:
      // the reference's distance is >= 0 exactly when some face plane has
      // the point on or beyond it (its own construction: face normals out)
      for (int f = 0; f < 6; ++f)
        if (dot(q - G.face_o[f], G.face_n[f]) >= 0.0) return true;
      return false;
    case A2C_GEOM_SPHEROID: {
      const V x = q - G.x0;
      const double a = dot(x, G.n);
      const V perp = x - a * G.n;
      return (a / G.A) * (a / G.A) + dot(perp, perp) / (G.R * G.R) >= 1.0;
    }
    case A2C_GEOM_CYLINDER_SPHERE: {
      const V x = q - G.x0;
      const double h = dot(x, G.n);
      const V perp = x - h * G.n;
      const double rho = norm(perp);
      if (h > 0.0 && h < G.L && rho < G.R) return false;
      if (G.back && norm(x) < G.R) return false;
      if (G.front && norm(q - (G.x0 + G.L * G.n)) < G.R) return false;
      return true;
    }
    case A2C_GEOM_CYLINDER_CONE: {
      const V x = q - G.x0;
      const double h = dot(x, G.n);
      const double rho = norm(x - h * G.n);
      if (h > 0.0 && h < G.L && rho < G.R) return false;
      if (h >= G.L && h < G.L + G.H && rho < G.R - (h - G.L) * G.tan_a) return false;
      return true;
    }
    default:
      return true;
  }
}

bool contains(const Geom &G, const V &q) {
  if (G.g.type == A2C_GEOM_PLANE) return dot(q - G.x0, G.n) > 0.0;  // ProjectPointToPlane, normalized
  const bool out = outside(G, q);
  return G.g.exterior ? out : !out;
}

// FindLatticeDomainBoundingBox: the union of the interior geometries' boxes
void lattice_box(const std::vector<Geom> &geoms, const Frame &F, V &lmin, V &lmax) {
  lmin = mk(DBL_MAX, DBL_MAX, DBL_MAX);
  lmax = mk(-DBL_MAX, -DBL_MAX, -DBL_MAX);
  auto merge = [&](const V &a, const V &b) {
    for (int i = 0; i < 3; ++i) {
      if (a[i] < lmin[i]) lmin[i] = a[i];
      if (b[i] > lmax[i]) lmax[i] = b[i];
    }
  };
  // the reference walks cylinder-cones, cylinder-spheres, spheres,
  // parallelepipeds, spheroids in turn; the union does not depend on it
  for (const Geom &G : geoms) {
    if (G.g.type == A2C_GEOM_PLANE || G.g.exterior) continue;
    V a, b;
    const double *p = G.g.p;
    if (G.g.type == A2C_GEOM_SPHERE) {
      bbox_sphere(G.x0, G.R, F, a, b);
    } else if (G.g.type == A2C_GEOM_PARALLELEPIPED) {
      const V P = vec(p);
      bbox_parallelepiped(P, vec(p + 3) - P, vec(p + 6) - P, vec(p + 9) - P, F, a, b);
    } else {
      // cylinder shapes: the axis normalized by the caller, then again;
      // spheroid: the raw axis (SpaceInitializer.cpp:744-747, 770-771, 840)
      V n = vec(p + 3);
      if (G.g.type != A2C_GEOM_SPHEROID) n = scale_by_inverse(n, norm(n));
      const V U0 = divide(n, norm(n));
      V U1, U2;
      orthonormal(U0, U1, U2);
      const V x0 = vec(p);
      if (G.g.type == A2C_GEOM_SPHEROID) {
        const double sl = p[6], r = p[7];
        const V P = x0 - sl * U0 - r * U1 - r * U2;
        bbox_parallelepiped(P, 2.0 * r * U1, 2.0 * r * U2, 2.0 * sl * U0, F, a, b);
      } else if (G.g.type == A2C_GEOM_CYLINDER_CONE) {
        const double r = G.R, L = G.L, H = G.H;
        const V P = x0 - r * U1 - r * U2;
        bbox_parallelepiped(P, 2.0 * r * U1, 2.0 * r * U2, (L + H) * U0, F, a, b);
      } else {
        const double r = G.R, L = G.L;
        V P = x0 - r * U1 - r * U2;
        if (G.back) P = P - r * U0;
        bbox_parallelepiped(P, 2.0 * r * U1, 2.0 * r * U2, (L + (G.back ? r : 0.0) + (G.front ? r : 0.0)) * U0, F,
                            a, b);
      }
    }
    merge(a, b);
  }
  for (int i = 0; i < 3; ++i)
    if (!std::isfinite(lmin[i]) || !std::isfinite(lmax[i]) || lmin[i] >= lmax[i])
      throw Fail{"unable to find a bounding box for the lattice domain: it is unbounded"};
}

// Geometries prepared, and their indices in operation order
// (SortUserSpecifiedGeometries, SpaceInitializer.cpp:326-600).
void prepare_ordered(const a2c_geometry *g, int ng, std::vector<Geom> &geoms, std::vector<int> &order) {
  order.assign(ng, -1);
  geoms.clear();
  geoms.reserve(ng);
  for (int k = 0; k < ng; ++k) {
    if (g[k].order < 0 || g[k].order >= ng || order[g[k].order] != -1)
      throw Fail{"geometry " + std::to_string(k) + " has an invalid or conflicting order (" +
                 std::to_string(g[k].order) + ")"};
    if (g[k].inclusion != A2C_INCLUSION_INTERSECTION && g[k].inclusion != A2C_INCLUSION_UNION)
      throw Fail{"unsupported geometry inclusion operator (must be Intersection or Union)"};
    order[g[k].order] = k;
    geoms.push_back(prepare(g[k]));
  }
}

// Whether the geometries, applied in order from "everything", contain q
// (CheckAndAddSitesInCell, SpaceInitializer.cpp:622-698).
bool inside_all(const std::vector<Geom> &geoms, const std::vector<int> &order, const V &q) {
  bool in = true;
  for (int k : order) {
    const Geom &G = geoms[k];
    const bool intersect = G.g.inclusion == A2C_INCLUSION_INTERSECTION;
    if ((in && intersect) || (!in && !intersect)) in = contains(G, q);
  }
  return in;
}

a2c_status fail(char *errmsg, int errlen, const std::string &m) {
  if (errmsg && errlen > 0) std::snprintf(errmsg, (size_t)errlen, "%s", m.c_str());
  return A2C_ERR_INVALID;
}

}  // namespace

extern "C" a2c_status a2c_lattice_build(const a2c_lattice_desc *d, a2c_lattice_sites *out, char *errmsg, int errlen) {
  if (!d || !out || d->nsites < 0 || d->ngeom < 0 || (d->nsites > 0 && !d->sites) || (d->ngeom > 0 && !d->geoms) ||
      out->capacity < 0)
    return fail(errmsg, errlen, "invalid arguments");
  if (out->capacity > 0 && (!out->q || !out->q0 || !out->l || !out->siteid || !out->matid || !out->tag ||
                            !out->sigma || !out->x))
    return fail(errmsg, errlen, "output arrays missing");
  try {
    Frame F;
    F.O = vec(d->origin);
    for (int i = 0; i < 3; ++i) {
      F.d[i] = vec(d->abc + 3 * i);
      if (!(norm(F.d[i]) > 0)) throw Fail{"zero lattice vector"};
    }
    // LatticeStructure::Setup's checks (LatticeStructure.cpp:64-102)
    if (d->nsites == 0) throw Fail{"no lattice sites specified"};
    for (int s = 0; s < d->nsites; ++s) {
      for (int i = 0; i < 3; ++i)
        if (!(d->sites[s].l[i] >= 0.0 && d->sites[s].l[i] < 1.0))
          throw Fail{"site coordinates must be in [0, 1) (site " + std::to_string(s) + ")"};
      if (d->sites[s].materialid < 0) throw Fail{"site " + std::to_string(s) + " has no material id"};
    }
    std::vector<int> order;
    std::vector<Geom> geoms;
    prepare_ordered(d->geoms, d->ngeom, geoms, order);
    V lmin, lmax;
    lattice_box(geoms, F, lmin, lmax);
    int lo[3], hi[3];
    double cells = 1.0;
    for (int i = 0; i < 3; ++i) {
      // the reference's guard (a long long that is never infinite) cannot
      // fire; here the cell range must fit int and the scan a few 1e10 sites
      if (std::fabs(lmin[i]) > 1.0e9 || std::fabs(lmax[i]) > 1.0e9)
        throw Fail{"the bounding box of the lattice domain is too large"};
      lo[i] = (int)std::floor(lmin[i]);
      hi[i] = (int)std::ceil(lmax[i]) + 1;  // one past the last cell
      cells *= (double)(hi[i] - lo[i]);
    }
    if (cells * (double)d->nsites > 4.0e10) throw Fail{"the bounding box of the lattice domain is too large"};
    int64_t n = 0;
    for (int lk = lo[2]; lk < hi[2]; ++lk)
      for (int lj = lo[1]; lj < hi[1]; ++lj)
        for (int li = lo[0]; li < hi[0]; ++li)
          for (int s = 0; s < d->nsites; ++s) {
            const a2c_site_group &sg = d->sites[s];
            const V l = mk(sg.l[0] + li, sg.l[1] + lj, sg.l[2] + lk);
            const V q = F.O + l[0] * F.d[0] + l[1] * F.d[1] + l[2] * F.d[2];  // LatticeStructure::GetXYZ
            if (!inside_all(geoms, order, q)) continue;
            if (n < out->capacity) {
              for (int k = 0; k < 3; ++k) {
                out->l[3 * n + k] = l[k];
                out->q0[3 * n + k] = q[k];
                out->q[3 * n + k] = q[k] + sg.mean_displacement[k];
              }
              out->siteid[n] = s;
              out->matid[n] = sg.materialid;
              out->tag[n] = sg.tag;
              out->sigma[n] = sg.atomic_frequency;
              out->x[n] = sg.x;
            }
            ++n;
          }
    out->count = n;
  } catch (const Fail &e) {
    return fail(errmsg, errlen, e.msg);
  }
  if (errmsg && errlen > 0) errmsg[0] = 0;
  return A2C_OK;
}

extern "C" a2c_status a2c_lattice_apply_region(const a2c_region *r, a2c_lattice_sites *out, char *errmsg,
                                               int errlen) {
  if (!r || !out || r->ngeom < 0 || (r->ngeom > 0 && !r->geoms) || out->count < 0)
    return fail(errmsg, errlen, "invalid arguments");
  if (out->count > 0 && (!out->q || !out->siteid || !out->matid || !out->tag || !out->sigma || !out->x))
    return fail(errmsg, errlen, "site arrays missing");
  try {
    std::vector<int> order;
    std::vector<Geom> geoms;
    prepare_ordered(r->geoms, r->ngeom, geoms, order);
    for (int64_t i = 0; i < out->count; ++i) {
      if (out->matid[i] != r->materialid || out->siteid[i] != r->siteid) continue;
      double *q = out->q + 3 * i;
      if (!inside_all(geoms, order, mk(q[0], q[1], q[2]))) continue;
      for (int k = 0; k < 3; ++k) q[k] += r->mean_displacement[k];
      out->sigma[i] = r->atomic_frequency;
      out->tag[i] = r->tag;
      if (r->x >= 0.0) out->x[i] = r->x;
    }
  } catch (const Fail &e) {
    return fail(errmsg, errlen, e.msg);
  }
  if (errmsg && errlen > 0) errmsg[0] = 0;
  return A2C_OK;
}

// Sites of q with a site of q_other inside the cube of half-width dmin
// around them (KDTree::findCandidatesWithin's box test: every coordinate
// within dmin), found through a grid of dmin-sized cells over q_other.
extern "C" a2c_status a2c_lattice_conflicts(const double *q, int64_t n, const double *q_other, int64_t n_other,
                                            double dmin, unsigned char *keep, int64_t *n_removed) {
  if (n < 0 || n_other < 0 || (n > 0 && (!q || !keep)) || (n_other > 0 && !q_other) || !(dmin > 0))
    return A2C_ERR_INVALID;
  int64_t removed = 0;
  if (n_other == 0) {
    for (int64_t i = 0; i < n; ++i) keep[i] = 1;
    if (n_removed) *n_removed = 0;
    return A2C_OK;
  }
  double lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = DBL_MAX;
    hi[k] = -DBL_MAX;
  }
  for (int64_t j = 0; j < n_other; ++j)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], q_other[3 * j + k]);
      hi[k] = std::max(hi[k], q_other[3 * j + k]);
    }
  // cells of about dmin, at most ~2 per point of q_other (any grid gives
  // the same answer: every cell meeting the query cube is searched)
  const double budget = std::max(1.0, std::min(2.0 * (double)n_other, 16.0 * 1024 * 1024));
  const double per_axis = std::cbrt(budget);
  int64_t dim[3];
  for (int k = 0; k < 3; ++k) {
    const double want = std::floor((hi[k] - lo[k]) / dmin) + 1.0;
    dim[k] = (int64_t)std::max(1.0, std::min(want, per_axis));
  }
  auto cell_of = [&](double x, int k) {
    int64_t c = (int64_t)std::floor((x - lo[k]) / (hi[k] - lo[k] > 0 ? (hi[k] - lo[k]) / dim[k] : 1.0));
    return std::max<int64_t>(0, std::min<int64_t>(c, dim[k] - 1));
  };
  const int64_t ncell = dim[0] * dim[1] * dim[2];
  std::vector<int64_t> start(ncell + 1, 0), item(n_other);
  std::vector<int64_t> cell(n_other);
  for (int64_t j = 0; j < n_other; ++j) {
    const double *p = q_other + 3 * j;
    cell[j] = cell_of(p[0], 0) + dim[0] * (cell_of(p[1], 1) + dim[1] * cell_of(p[2], 2));
    ++start[cell[j] + 1];
  }
  for (int64_t c = 0; c < ncell; ++c) start[c + 1] += start[c];
  std::vector<int64_t> fill(start.begin(), start.end() - 1);
  for (int64_t j = 0; j < n_other; ++j) item[fill[cell[j]]++] = j;
  for (int64_t i = 0; i < n; ++i) {
    const double *p = q + 3 * i;
    int64_t c0[3], c1[3];
    for (int k = 0; k < 3; ++k) {
      c0[k] = cell_of(p[k] - dmin, k);
      c1[k] = cell_of(p[k] + dmin, k);
    }
    bool hit = false;
    for (int64_t cz = c0[2]; cz <= c1[2] && !hit; ++cz)
      for (int64_t cy = c0[1]; cy <= c1[1] && !hit; ++cy)
        for (int64_t cx = c0[0]; cx <= c1[0] && !hit; ++cx) {
          const int64_t c = cx + dim[0] * (cy + dim[1] * cz);
          for (int64_t t = start[c]; t < start[c + 1]; ++t) {
            const double *r = q_other + 3 * item[t];
            double m = 0.0;
            for (int k = 0; k < 3; ++k) m = std::max(m, std::max(r[k] - p[k], p[k] - r[k]));
            if (m <= dmin) {
              hit = true;
              break;
            }
          }
        }
    keep[i] = hit ? 0 : 1;
    removed += hit ? 1 : 0;
  }
  if (n_removed) *n_removed = removed;
  return A2C_OK;
}
