// Seeded synthetic fcc Pd lattice with octahedral H sites, the input
// generator for tests and benchmarks.  It stands in for the reference's
// lattice setup (SpaceInitializer.cpp:119-320, 603-640: cells scanned z, y,
// x with the basis inside each cell), producing the minimizer's AoS state
// directly.  Draws come from std::mt19937_64 in a fixed order: three
// Box-Muller normals per site for the positions (Pd sites then H sites),
// then one uniform per site for sigma when a range is given, then one
// uniform per H site for the occupancy jitter.
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "a2c_gpp.h"

namespace {

struct Normal {
  std::mt19937_64 &g;
  bool have = false;
  double spare = 0.0;
  static double unit(std::mt19937_64 &g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }
  double next() {
    if (have) {
      have = false;
      return spare;
    }
    const double u1 = 1.0 - unit(g);  // (0, 1]
    const double u2 = unit(g);
    const double r = std::sqrt(-2.0 * std::log(u1));
    const double t = 6.283185307179586 * u2;
    spare = r * std::sin(t);
    have = true;
    return r * std::cos(t);
  }
};

const double kPdBasis[4][3] = {{0.0, 0.0, 0.0}, {0.0, 0.5, 0.5}, {0.5, 0.0, 0.5}, {0.5, 0.5, 0.0}};
const double kHBasis[4][3] = {{0.5, 0.0, 0.0}, {0.0, 0.5, 0.0}, {0.0, 0.0, 0.5}, {0.5, 0.5, 0.5}};

}  // namespace

extern "C" a2c_status a2c_lattice_fcc(const a2c_lattice_spec *sp, double *X, double *xH, int *surface) {
  if (!sp || !X) return A2C_ERR_INVALID;
  for (int d = 0; d < 3; ++d)
    if (sp->ncell[d] < 1) return A2C_ERR_INVALID;
  if (!(sp->a > 0.0) || sp->pos_std < 0.0) return A2C_ERR_INVALID;
  const int64_t nc = (int64_t)sp->ncell[0] * sp->ncell[1] * sp->ncell[2];
  const int64_t nPd = 4 * nc, nH = 4 * nc, N = nPd + nH;
  if (N >= (int64_t(1) << 27)) return A2C_ERR_INVALID;
  std::mt19937_64 g(sp->seed);
  Normal nrm{g};
  const double a = sp->a;
  const double L[3] = {sp->ncell[0] * a, sp->ncell[1] * a, sp->ncell[2] * a};
  const double ctr[3] = {0.5 * L[0], 0.5 * L[1], 0.5 * L[2]};
  std::vector<double> lat(3 * (size_t)N);
  int64_t s = 0;
  for (int species = 0; species < 2; ++species) {
    const double(*basis)[3] = species == 0 ? kPdBasis : kHBasis;
    for (int cz = 0; cz < sp->ncell[2]; ++cz)
      for (int cy = 0; cy < sp->ncell[1]; ++cy)
        for (int cx = 0; cx < sp->ncell[0]; ++cx)
          for (int b = 0; b < 4; ++b, ++s) {
            lat[3 * s] = a * (cx + basis[b][0]);
            lat[3 * s + 1] = a * (cy + basis[b][1]);
            lat[3 * s + 2] = a * (cz + basis[b][2]);
          }
  }
  for (s = 0; s < N; ++s)
    for (int d = 0; d < 3; ++d) X[4 * s + d] = lat[3 * s + d] + sp->pos_std * nrm.next();
  for (s = 0; s < N; ++s)
    X[4 * s + 3] = (sp->sigma_hi > sp->sigma_lo) ? sp->sigma_lo + (sp->sigma_hi - sp->sigma_lo) * Normal::unit(g)
                                                 : sp->sigma_lo;
  if (xH) {
    for (int64_t h = 0; h < nH; ++h) {
      const double *q = &lat[3 * (size_t)(nPd + h)];
      double x;
      if (sp->x_mode == 1) {
        const double dx = q[0] - ctr[0], dy = q[1] - ctr[1], dz = q[2] - ctr[2];
        const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
        x = sp->x_matrix +
            (sp->x_nucleus - sp->x_matrix) * 0.5 * (1.0 - std::tanh((r - sp->nucleus_radius) / sp->interface_width));
        x += sp->x_half * (2.0 * Normal::unit(g) - 1.0);
      } else {
        x = sp->x_center + sp->x_half * (2.0 * Normal::unit(g) - 1.0);
      }
      if (x < sp->xLb) x = sp->xLb;
      if (x > sp->xUb) x = sp->xUb;
      xH[h] = x;
    }
  }
  if (surface)
    for (int64_t h = 0; h < nH; ++h) surface[h] = lat[3 * (size_t)(nPd + h) + 2] < 1e-6 ? 1 : 0;
  (void)L;
  return A2C_OK;
}
