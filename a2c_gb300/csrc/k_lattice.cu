// Seeded synthetic lattice generated on the device: the lattice of
// a2c_lattice_fcc (fcc Pd basis + octahedral H basis, cells z, y, x, all Pd
// then all H -- the order of SpaceInitializer.cpp:266-268, 622) with the
// same distributions, one thread per site.  The host generator draws from
// one sequential std::mt19937_64 stream; here draw k of site s is output
// number 8 s + k of a SplitMix64 stream (Steele, Lea and Flood, 2014), which
// can be computed directly from its index, so every site draws
// independently.  The lattice positions, the fixed widths and the
// deterministic occupancy profile are bit-identical to the host generator's
// (compiled without FMA contraction); the random parts have the same
// distributions but other values.
#include <cmath>

#include "internal.cuh"

namespace a2c {
namespace {

__device__ __forceinline__ uint64_t splitmix(uint64_t seed, uint64_t i) {
  uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double unit(uint64_t seed, uint64_t i) {
  return (double)(splitmix(seed, i) >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
}

struct LatArgs {
  int ncell[3];
  double a, pos_std, sigma_lo, sigma_hi;
  int x_mode;
  double x_center, x_half, x_matrix, x_nucleus, nucleus_radius, interface_width, xLb, xUb;
  uint64_t seed;
  int64_t nPd, N;
};

__global__ void k_lattice(LatArgs p, double *X, double *xH, int *surface) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= p.N) return;
  const bool H = s >= p.nPd;
  const int64_t loc = H ? s - p.nPd : s;
  const int b = (int)(loc % 4);
  const int64_t c = loc / 4;
  const int cx = (int)(c % p.ncell[0]), cy = (int)((c / p.ncell[0]) % p.ncell[1]);
  const int cz = (int)(c / ((int64_t)p.ncell[0] * p.ncell[1]));
  // the basis of the host generator, in its order
  double bx, by, bz;
  if (!H) {
    bx = (b == 2 || b == 3) ? 0.5 : 0.0;
    by = (b == 1 || b == 3) ? 0.5 : 0.0;
    bz = (b == 1 || b == 2) ? 0.5 : 0.0;
  } else {
    bx = (b == 0 || b == 3) ? 0.5 : 0.0;
    by = (b == 1 || b == 3) ? 0.5 : 0.0;
    bz = (b == 2 || b == 3) ? 0.5 : 0.0;
  }
  const double q0 = p.a * (cx + bx), q1 = p.a * (cy + by), q2 = p.a * (cz + bz);
  // three normals by Box-Muller from draws 0-3
  const uint64_t i0 = 8 * (uint64_t)s;
  double n[4];
  for (int k = 0; k < 2; ++k) {
    const double u1 = 1.0 - unit(p.seed, i0 + 2 * k), u2 = unit(p.seed, i0 + 2 * k + 1);
    const double r = sqrt(-2.0 * log(u1)), t = 6.283185307179586 * u2;
    n[2 * k] = r * cos(t);
    n[2 * k + 1] = r * sin(t);
  }
  X[4 * s] = q0 + p.pos_std * n[0];
  X[4 * s + 1] = q1 + p.pos_std * n[1];
  X[4 * s + 2] = q2 + p.pos_std * n[2];
  X[4 * s + 3] =
      (p.sigma_hi > p.sigma_lo) ? p.sigma_lo + (p.sigma_hi - p.sigma_lo) * unit(p.seed, i0 + 4) : p.sigma_lo;
  if (!H) return;
  if (xH) {
    double x;
    if (p.x_mode == 1) {
      const double L0 = p.ncell[0] * p.a, L1 = p.ncell[1] * p.a, L2 = p.ncell[2] * p.a;
      const double dx = q0 - 0.5 * L0, dy = q1 - 0.5 * L1, dz = q2 - 0.5 * L2;
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      x = p.x_matrix + (p.x_nucleus - p.x_matrix) * 0.5 * (1.0 - tanh((r - p.nucleus_radius) / p.interface_width));
      x += p.x_half * (2.0 * unit(p.seed, i0 + 5) - 1.0);
    } else {
      x = p.x_center + p.x_half * (2.0 * unit(p.seed, i0 + 5) - 1.0);
    }
    if (x < p.xLb) x = p.xLb;
    if (x > p.xUb) x = p.xUb;
    xH[loc] = x;
  }
  if (surface) surface[loc] = q2 < 1e-6 ? 1 : 0;
}

}  // namespace
}  // namespace a2c

using namespace a2c;

// Device pointers X (4N), xH (nH), surface (nH; each of the last two may be
// NULL); stream-ordered on `stream` (a cudaStream_t; NULL = the default
// stream).
extern "C" a2c_status a2c_lattice_fcc_device(const a2c_lattice_spec *sp, double *dX, double *dxH, int *dsurface,
                                             void *stream) {
  if (!sp || !dX) return A2C_ERR_INVALID;
  for (int d = 0; d < 3; ++d)
    if (sp->ncell[d] < 1) return A2C_ERR_INVALID;
  if (!(sp->a > 0.0) || sp->pos_std < 0.0) return A2C_ERR_INVALID;
  const int64_t nc = (int64_t)sp->ncell[0] * sp->ncell[1] * sp->ncell[2];
  const int64_t N = 8 * nc;
  if (N >= (int64_t(1) << 27)) return A2C_ERR_INVALID;
  LatArgs p;
  for (int d = 0; d < 3; ++d) p.ncell[d] = sp->ncell[d];
  p.a = sp->a;
  p.pos_std = sp->pos_std;
  p.sigma_lo = sp->sigma_lo;
  p.sigma_hi = sp->sigma_hi;
  p.x_mode = sp->x_mode;
  p.x_center = sp->x_center;
  p.x_half = sp->x_half;
  p.x_matrix = sp->x_matrix;
  p.x_nucleus = sp->x_nucleus;
  p.nucleus_radius = sp->nucleus_radius;
  p.interface_width = sp->interface_width;
  p.xLb = sp->xLb;
  p.xUb = sp->xUb;
  p.seed = sp->seed;
  p.nPd = 4 * nc;
  p.N = N;
  k_lattice<<<grid_for(N, 256), 256, 0, (cudaStream_t)stream>>>(p, dX, dxH, dsurface);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}
