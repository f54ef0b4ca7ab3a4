// Cell-list neighbor build.  Replaces findNeighbors (neighbors.cpp:8-115,
// KD-tree + inclusive d^2 <= rc^2 test, self excluded) followed by
// Minimizer::findLocalNeighbors (minimizer.cpp:833-1144: refilter at rc, Pd
// shell counts PdPdnum, first H shell HH1).  Compiled with -fmad=false so
// the distance test reproduces the reference's arithmetic exactly: the
// neighbor SETS are bit-exact; each list is sorted by global id (the
// reference's order is a KD-tree traversal artefact).
//
// Periodic dimensions use the minimum image, which the reference lacks: the
// image multiplier m = -rint((q_j - q_i)/L) is fixed at build time and
// stored in the entry's top bits, as the reference holds its lists fixed
// through a solve.
//
// Skin (Verlet) lists: with a skin s > 0 the cell-list build makes extended
// candidate lists at rc + s (findNeighbors' _ext lists) and the lists at rc
// are re-filtered from them on the device with the same acceptance test
// (findLocalNeighbors, minimizer.cpp:833-1144).  While no site has moved
// more than s/2 since the extended build, every pair now within rc was
// within rc + s then, and filtering each sorted extended list in order gives
// exactly the lists a full build would.
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace a2c {
namespace {

constexpr int kBlock = 128;
constexpr int kMaxPerSite = 1000;  // neighbors.cpp:42 (maxNei)

struct GridArgs {
  int n[3];
  int scan_all[3];  // periodic with fewer than 3 cells: visit every cell once
  int periodic[3];
  double lo[3], cs[3], box[3];
  double rc, rc2, A75, A125;
  int nPd;
  int64_t N;
  const double *X;
  // FP32 prefilter (see prefilter below): positions as float, the largest
  // |coordinate| (as float bits, set by k_positions_f32), the box as float
  const float4 *Xf = nullptr;
  const unsigned *qmax_bits = nullptr;
  float boxf[3] = {0.f, 0.f, 0.f}, invboxf[3] = {0.f, 0.f, 0.f}, Lmaxf = 0.f, rcf = 0.f;
  float rc2f = 0.f, A75f = 0.f, A125f = 0.f;  // the FP64 thresholds rounded to float
};

__device__ __forceinline__ int cell_coord(const GridArgs &g, double x, int d) {
  double t;
  if (g.periodic[d]) t = x - g.box[d] * floor(x / g.box[d]);
  else t = x - g.lo[d];
  int c = (int)floor(t / g.cs[d]);
  return c < 0 ? 0 : (c >= g.n[d] ? g.n[d] - 1 : c);
}

__device__ __forceinline__ int64_t cell_of(const GridArgs &g, int64_t s) {
  const int c0 = cell_coord(g, g.X[4 * s], 0), c1 = cell_coord(g, g.X[4 * s + 1], 1),
            c2 = cell_coord(g, g.X[4 * s + 2], 2);
  return ((int64_t)c2 * g.n[1] + c1) * g.n[0] + c0;
}

// The reference's acceptance test (KDTree.h:250-254 Chebyshev prefilter,
// neighbors.cpp:77-82 self and squared distance) in FP64, with the image
// shift m (fixed by the FP32 prefilter, or decoded from an entry).
__device__ __forceinline__ bool exact_test(const GridArgs &g, int64_t i, int64_t j, const int m[3], uint32_t &entry,
                                           double &d2) {
  if (i == j) return false;
  double dd[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double qi = g.X[4 * i + d];
    double qj = g.X[4 * j + d];
    if (m[d] != 0) qj = qj + m[d] * g.box[d];
    dd[d] = qj - qi;
    if (fabs(dd[d]) > g.rc) return false;
  }
  d2 = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2];
  if (d2 > g.rc2) return false;
  if (m[0] < -1 || m[0] > 1 || m[1] < -1 || m[1] > 1 || m[2] < -1 || m[2] > 1) return false;
  entry = (uint32_t)j | ((uint32_t)((m[0] + 1) + 3 * (m[1] + 1) + 9 * (m[2] + 1)) << kIdBits);
  return true;
}

// FP32 prefilter: rejects candidates farther than rc + guard in any
// coordinate or in distance, and picks the image m of the rest.  guard
// bounds the FP32 error of a coordinate difference (coordinates rounded to
// float, one subtraction, the image shift) four times over, so a pair the
// FP64 test accepts is never rejected here; a pair within rc + guard has a
// unique nearest image because the box exceeds 2 (rc + guard) (checked on
// the host before the prefilter is used), so m is the image the FP64
// division rint((qj - qi) / L) would pick.
__device__ __forceinline__ float prefilter_guard(const GridArgs &g) {
  const float qmax = __uint_as_float(*g.qmax_bits);
  return 1e-4f + 1.9073486328125e-6f * (qmax + g.Lmaxf + g.rcf);  // 2^-19 (qmax + L + rc)
}
// The FP32 pass over one candidate: coordinate differences with the image
// m, and their squared length.  false: farther than rc + guard (rejected).
__device__ __forceinline__ bool prefilter(const GridArgs &g, float4 fi, int64_t j, float lim, int m[3], float dd[3],
                                          float &d2f) {
  const float4 fj = g.Xf[j];
  dd[0] = fj.x - fi.x;
  dd[1] = fj.y - fi.y;
  dd[2] = fj.z - fi.z;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    m[d] = 0;
    if (g.periodic[d]) {
      const float n = rintf(dd[d] * g.invboxf[d]);
      dd[d] = dd[d] - n * g.boxf[d];
      m[d] = -(int)n;
    }
    if (fabsf(dd[d]) > lim) return false;
  }
  d2f = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2];
  return d2f <= lim * lim;
}

// Whether the FP32 values decide every comparison the FP64 test and the
// shell counts make: each |coordinate difference| at least guard inside rc,
// and d^2 at least `band` away from rc^2, 0.75 a^2 and 1.25 a^2.  A
// coordinate difference is off by at most guard/4 (see prefilter_guard), so
// d^2 is off by at most 2 sqrt(3) |d| guard/4 + 3 (guard/4)^2 plus three
// FP32 roundings of d^2, which band = 2 guard (rc + 1) + 1e-5 bounds for
// every d up to rc + guard.
__device__ __forceinline__ bool fp32_decides(const GridArgs &g, const float dd[3], float d2f, float guard) {
  const float band = 2.0f * guard * (g.rcf + 1.0f) + 1e-5f, inner = g.rcf - guard;
  return fabsf(dd[0]) < inner && fabsf(dd[1]) < inner && fabsf(dd[2]) < inner && d2f < g.rc2f - band &&
         fabsf(d2f - g.A75f) > band && fabsf(d2f - g.A125f) > band;
}

__device__ __forceinline__ uint32_t encode(int64_t j, const int m[3]) {
  return (uint32_t)j | ((uint32_t)((m[0] + 1) + 3 * (m[1] + 1) + 9 * (m[2] + 1)) << kIdBits);
}

// The shell class of a pair for the Pd shell counts and the first H shell
// (minimizer.cpp:935-947, 999-1004): 0 below 0.75 a^2, 1 strictly between
// 0.75 a^2 and 1.25 a^2, 2 otherwise.
template <class T>
__device__ __forceinline__ int shell_class(T d2, T A75, T A125) {
  return d2 < A75 ? 0 : (d2 > A75 && d2 < A125 ? 1 : 2);
}

// Candidate j of site i.  The FP32 pass rejects everything farther than
// rc + guard and accepts every pair whose decisions it settles
// (fp32_decides: nearly all), its shell class from the FP32 values too (d^2
// lies at least the guard band away from both thresholds, so the FP32
// comparisons give the FP64 answers; GB300's FP64 pipe made the widened
// comparisons the refilter's bound); the rest take the FP64 test.  lim <= 0
// (the prefilter cannot be used: a periodic box of at most 2 (rc + guard))
// takes the image from the FP64 division and the FP64 test.
__device__ __forceinline__ bool pair_test(const GridArgs &g, int64_t i, float4 fi, float lim, int64_t j,
                                          uint32_t &entry, int &cls) {
  int m[3];
  if (i == j) return false;
  if (lim > 0.0f) {
    float dd[3], d2f;
    if (!prefilter(g, fi, j, lim, m, dd, d2f)) return false;
    if (fp32_decides(g, dd, d2f, lim - g.rcf) && m[0] >= -1 && m[0] <= 1 && m[1] >= -1 && m[1] <= 1 && m[2] >= -1 &&
        m[2] <= 1) {
      entry = encode(j, m);
      cls = shell_class(d2f, g.A75f, g.A125f);
      return true;
    }
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d)
      m[d] = g.periodic[d] ? -(int)rint((g.X[4 * j + d] - g.X[4 * i + d]) / g.box[d]) : 0;
  }
  double d2;
  if (!exact_test(g, i, j, m, entry, d2)) return false;
  cls = shell_class(d2, g.A75, g.A125);
  return true;
}

// The prefilter's cutoff for this build, or 0 when it cannot be used.
__device__ __forceinline__ float prefilter_lim(const GridArgs &g) {
  const float lim = g.rcf + prefilter_guard(g);
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (g.periodic[d] && !(0.5f * g.boxf[d] > lim * 1.0001f)) return 0.0f;
  return lim;
}

// Positions as float for the prefilter and the largest |coordinate|.
__global__ void k_positions_f32(const double *X, int64_t N, float4 *Xf, unsigned *qmax_bits) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N) return;
  const float4 f = make_float4((float)X[4 * s], (float)X[4 * s + 1], (float)X[4 * s + 2], 0.0f);
  Xf[s] = f;
  const float q = fmaxf(fabsf(f.x), fmaxf(fabsf(f.y), fabsf(f.z)));
  atomicMax(qmax_bits, __float_as_uint(q) + 1u);  // one ulp up: the float rounding of |q| may round down
}

template <class Fn>
__device__ __forceinline__ void for_candidates(const GridArgs &g, const int64_t *cstart, const int *items,
                                               int64_t i, Fn fn) {
  int c[3], lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    c[d] = cell_coord(g, g.X[4 * i + d], d);
    if (g.scan_all[d]) {
      lo[d] = 0;
      hi[d] = g.n[d] - 1;
    } else {
      lo[d] = c[d] - 1;
      hi[d] = c[d] + 1;
    }
  }
  for (int a = lo[2]; a <= hi[2]; ++a) {
    int ca = a;
    if (!g.scan_all[2]) {
      if (g.periodic[2]) ca = (a + g.n[2]) % g.n[2];
      else if (a < 0 || a >= g.n[2]) continue;
    }
    for (int b = lo[1]; b <= hi[1]; ++b) {
      int cb = b;
      if (!g.scan_all[1]) {
        if (g.periodic[1]) cb = (b + g.n[1]) % g.n[1];
        else if (b < 0 || b >= g.n[1]) continue;
      }
      for (int e = lo[0]; e <= hi[0]; ++e) {
        int ce = e;
        if (!g.scan_all[0]) {
          if (g.periodic[0]) ce = (e + g.n[0]) % g.n[0];
          else if (e < 0 || e >= g.n[0]) continue;
        }
        const int64_t cell = ((int64_t)ca * g.n[1] + cb) * g.n[0] + ce;
        for (int64_t t = cstart[cell]; t < cstart[cell + 1]; ++t) fn((int64_t)items[t]);
      }
    }
  }
}

// Candidate sources: the 27 cells around the site, or its extended list.
struct CellSrc {
  const int64_t *cstart;
  const int *items;
  template <class Fn>
  __device__ __forceinline__ void each(const GridArgs &g, int64_t i, Fn fn) const {
    for_candidates(g, cstart, items, i, fn);
  }
};
struct ExtSrc {
  const int64_t *off;
  const uint32_t *nbr;
  template <class Fn>
  __device__ __forceinline__ void each(const GridArgs &, int64_t i, Fn fn) const {
    for (int64_t t = off[i]; t < off[i + 1]; ++t) fn((int64_t)(nbr[t] & kIdMask));
  }
};

__global__ void k_cell_count(GridArgs g, int *cell, int *ccount) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= g.N) return;
  const int64_t c = cell_of(g, s);
  cell[s] = (int)c;
  atomicAdd(&ccount[c], 1);
}

__global__ void k_cell_fill(GridArgs g, const int *cell, const int64_t *cstart, int *cfill, int *items) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= g.N) return;
  const int c = cell[s];
  const int slot = atomicAdd(&cfill[c], 1);
  items[cstart[c] + slot] = (int)s;
}

// Each cell's sites in increasing id (the fill above leaves them in the
// order its atomics ran).
__global__ void k_cell_sort(int64_t ncell, const int64_t *cstart, int *items) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int64_t b = cstart[c], e = cstart[c + 1];
  for (int64_t t = b + 1; t < e; ++t) {
    const int v = items[t];
    int64_t u = t - 1;
    while (u >= b && items[u] > v) {
      items[u + 1] = items[u];
      --u;
    }
    items[u + 1] = v;
  }
}

// Counts per site; npd, shell and hh1count may be null (extended lists).
template <class Src>
__global__ void __launch_bounds__(kBlock) k_nbr_count(GridArgs g, Src src, int64_t *count, int *npd,
                                                      int64_t *hh1count, int *shell, int *status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.N) return;
  int64_t n = 0, nP = 0, n1 = 0;
  int sh[3] = {0, 0, 0};
  const bool iPd = i < g.nPd;
  const float4 fi = g.Xf[i];
  const float lim = prefilter_lim(g);
  src.each(g, i, [&](int64_t j) {
    uint32_t e;
    int cls;
    if (!pair_test(g, i, fi, lim, j, e, cls)) return;
    ++n;
    const bool jPd = j < g.nPd;
    if (jPd) {
      ++nP;
      if (iPd) {  // minimizer.cpp:935-947
        ++sh[cls];
      }
    } else if (!iPd && cls == 0) {  // minimizer.cpp:999-1004
      ++n1;
    }
  });
  count[i] = n;
  if (npd) npd[i] = (int)nP;
  if (iPd) {
    if (shell) {
      shell[3 * i] = sh[0];
      shell[3 * i + 1] = sh[1];
      shell[3 * i + 2] = sh[2];
    }
  } else if (hh1count) {
    hh1count[i - g.nPd] = n1;
  }
  if (n > kMaxPerSite) atomicOr(status, kStatusOverflow);
}

// Insertion sort of nbr[b, e) by global id; cheap when the entries arrive
// nearly sorted, as they do here (see k_nbr_fill).
__device__ __forceinline__ void sort_by_id(uint32_t *nbr, int64_t b, int64_t e) {
  for (int64_t t = b + 1; t < e; ++t) {
    const uint32_t v = nbr[t];
    const uint32_t key = v & kIdMask;
    int64_t u = t - 1;
    while (u >= b && (nbr[u] & kIdMask) > key) {
      nbr[u + 1] = nbr[u];
      --u;
    }
    nbr[u + 1] = v;
  }
}

// Fills the lists (sorted by id); hh1 may be null (extended lists).  The Pd
// neighbors go to the head of the list (npd of them, from the count pass)
// and the H neighbors after them, so each part is sorted on its own: the
// candidates arrive as runs sorted by id (cells' site lists are sorted,
// cells are visited in the order site ids follow on lattice inputs, an
// extended list is sorted), which leaves the insertion sort little to move.
template <class Src>
__global__ void __launch_bounds__(kBlock) k_nbr_fill(GridArgs g, Src src, const int64_t *off, const int *npd,
                                                     uint32_t *nbr, const int64_t *hh1_off, int *hh1, int *status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.N) return;
  const int64_t b = off[i], e = off[i + 1], m = b + npd[i];
  int64_t wP = b, wH = m;
  const float4 fi = g.Xf[i];
  const float lim = prefilter_lim(g);
  src.each(g, i, [&](int64_t j) {
    uint32_t en;
    int cls;
    if (!pair_test(g, i, fi, lim, j, en, cls)) return;
    if (j < g.nPd) {
      if (wP < m) nbr[wP] = en;
      ++wP;
    } else {
      if (wH < e) nbr[wH] = en;
      ++wH;
    }
  });
  if (wP != m || wH != e) {
    atomicOr(status, kStatusBadIndex);
    return;
  }
  sort_by_id(nbr, b, m);
  sort_by_id(nbr, m, e);
  if (hh1 && i >= g.nPd) {
    const int64_t h = i - g.nPd;
    int64_t w1 = hh1_off[h];
    for (int64_t t = b; t < e; ++t) {
      const uint32_t ent = nbr[t];
      const int64_t j = ent & kIdMask;
      if (j < g.nPd) continue;
      uint32_t en;
      int cls;
      if (pair_test(g, i, fi, lim, j, en, cls) && cls == 0) {
        if (w1 < hh1_off[h + 1]) hh1[w1] = (int)(j - g.nPd);
        ++w1;
      }
    }
    if (w1 != hh1_off[h + 1]) atomicOr(status, kStatusBadIndex);
  }
}

__global__ void k_max_count(const int64_t *count, int64_t n, int *out) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) atomicMax(out, (int)count[s]);
}

// The skin path's position checks, one pass: kPosMoved when a site moved
// more than sqrt(lim2) from its reference position (Xref, may be null),
// kPosNonfinite for a coordinate or width that is not finite, kPosOutside
// for a periodic coordinate outside [-L/2, 3L/2] (the host entry points'
// checks).  X may be the caller's host memory (pinned: read through the
// coherent link), copied then to Xout; Xout null checks X in place.
constexpr int kPosMoved = 1, kPosNonfinite = 2, kPosOutside = 4;
__global__ void k_check_positions(const double *X, double *Xout, const double *Xref, int64_t n, double lim2,
                                  double L0, double L1, double L2, int per, int *flags) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const double x = X[4 * s], y = X[4 * s + 1], z = X[4 * s + 2], w = X[4 * s + 3];
  if (Xout) {
    Xout[4 * s] = x;
    Xout[4 * s + 1] = y;
    Xout[4 * s + 2] = z;
    Xout[4 * s + 3] = w;
  }
  int f = 0;
  if (!isfinite(x) || !isfinite(y) || !isfinite(z) || !isfinite(w)) f |= kPosNonfinite;
  if (((per & 1) && (x < -0.5 * L0 || x > 1.5 * L0)) || ((per & 2) && (y < -0.5 * L1 || y > 1.5 * L1)) ||
      ((per & 4) && (z < -0.5 * L2 || z > 1.5 * L2)))
    f |= kPosOutside;
  if (Xref) {
    const double dx = x - Xref[4 * s], dy = y - Xref[4 * s + 1], dz = z - Xref[4 * s + 2];
    if (dx * dx + dy * dy + dz * dz > lim2) f |= kPosMoved;
  }
  if (f) atomicOr(flags, f);
}

// Skin refilter, one exact pass over the extended lists: site i's
// neighbors at rc go to tmp[ext_off[i] ...] in the extended list's order --
// its Pd part, then its H part, each sorted by id, the order k_nbr_fill
// gives -- with the counts of k_nbr_count.
__global__ void __launch_bounds__(kBlock) k_refilter(GridArgs g, ExtSrc src, uint32_t *tmp, int64_t *count, int *npd,
                                                     int64_t *hh1count, int *shell) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.N) return;
  const int64_t w = src.off[i];
  int64_t n = 0, nP = 0, n1 = 0;
  int sh[3] = {0, 0, 0};
  const bool iPd = i < g.nPd;
  const float4 fi = g.Xf[i];
  const float lim = prefilter_lim(g);
  src.each(g, i, [&](int64_t j) {
    uint32_t e;
    int cls;
    if (!pair_test(g, i, fi, lim, j, e, cls)) return;
    tmp[w + n] = e;
    ++n;
    if (j < g.nPd) {
      ++nP;
      if (iPd) {  // minimizer.cpp:935-947
        ++sh[cls];
      }
    } else if (!iPd && cls == 0) {  // minimizer.cpp:999-1004
      ++n1;
    }
  });
  count[i] = n;
  npd[i] = (int)nP;
  if (iPd) {
    shell[3 * i] = sh[0];
    shell[3 * i + 1] = sh[1];
    shell[3 * i + 2] = sh[2];
  } else {
    hh1count[i - g.nPd] = n1;
  }
}

// The re-filtered lists packed at their offsets, and each H site's first H
// shell (k_nbr_fill's second part).
__global__ void __launch_bounds__(kBlock) k_refilter_pack(GridArgs g, const int64_t *ext_off, const uint32_t *tmp,
                                                          const int64_t *off, uint32_t *nbr, const int64_t *hh1_off,
                                                          int *hh1, int *status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.N) return;
  const int64_t b = off[i], n = off[i + 1] - b;
  const uint32_t *src = tmp + ext_off[i];
  for (int64_t t = 0; t < n; ++t) nbr[b + t] = src[t];
  if (i < g.nPd) return;
  const int64_t h = i - g.nPd;
  const float4 fi = g.Xf[i];
  const float lim = prefilter_lim(g);
  int64_t w1 = hh1_off[h];
  for (int64_t t = 0; t < n; ++t) {
    const int64_t j = src[t] & kIdMask;
    if (j < g.nPd) continue;
    uint32_t en;
    int cls;
    if (pair_test(g, i, fi, lim, j, en, cls) && cls == 0) {
      if (w1 < hh1_off[h + 1]) hh1[w1] = (int)(j - g.nPd);
      ++w1;
    }
  }
  if (w1 != hh1_off[h + 1]) atomicOr(status, kStatusBadIndex);
}

template <class T>
a2c_status scan_exclusive(const T *in, int64_t *out, int64_t n, cudaStream_t st) {
  size_t bytes = 0;
  A2C_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, n, st));
  void *tmp = nullptr;
  A2C_CUDA(cudaMallocAsync(&tmp, bytes, st));
  cudaError_t e = cub::DeviceScan::ExclusiveSum(tmp, bytes, in, out, n, st);
  cudaFreeAsync(tmp, st);
  A2C_CUDA(e);
  return A2C_OK;
}

struct DevBuf {
  void *p = nullptr;
  cudaStream_t st;
  explicit DevBuf(cudaStream_t s) : st(s) {}
  ~DevBuf() {
    if (p) cudaFreeAsync(p, st);
  }
};

// Cell grid for cutoff `cut` (cells at least `cut` wide).  h_X (host
// positions) gives the extents of free directions; with h_X null (a list
// re-filter, which uses no cells) they are left nominal.
int64_t make_grid(const a2c_gpp_ctx *c, const double *h_X, double cut, GridArgs &g) {
  const int64_t N = c->N;
  const a2c_gpp_params &p = c->p;
  g = GridArgs{};
  g.N = N;
  g.nPd = p.nPd;
  g.X = c->d_X;
  g.rc = cut;
  g.rc2 = cut * cut;
  g.A75 = p.a_Pd * p.a_Pd * 0.75;
  g.A125 = p.a_Pd * p.a_Pd * 1.25;
  g.rcf = (float)cut;
  g.rc2f = (float)g.rc2;
  g.A75f = (float)g.A75;
  g.A125f = (float)g.A125;
  for (int d = 0; d < 3; ++d)
    if (p.periodic[d]) {
      g.boxf[d] = (float)p.box[d];
      g.invboxf[d] = (float)(1.0 / p.box[d]);
      g.Lmaxf = std::max(g.Lmaxf, (float)p.box[d]);
    }
  int64_t ncell = 1;
  for (int d = 0; d < 3; ++d) {
    g.periodic[d] = p.periodic[d] ? 1 : 0;
    g.box[d] = p.box[d];
    double ext;
    if (g.periodic[d]) {
      g.lo[d] = 0.0;
      ext = p.box[d];
    } else if (!h_X) {
      g.lo[d] = 0.0;
      ext = cut;
    } else {
      double lo = HUGE_VAL, hi = -HUGE_VAL;
      for (int64_t s = 0; s < N; ++s) {
        lo = std::min(lo, h_X[4 * s + d]);
        hi = std::max(hi, h_X[4 * s + d]);
      }
      if (N == 0) lo = hi = 0.0;
      g.lo[d] = lo;
      ext = hi - lo;
    }
    int n = (int)std::floor(ext / (cut + 1e-6));
    if (n < 1) n = 1;
    if (n > 512) n = 512;
    g.n[d] = n;
    g.cs[d] = (ext > 0.0) ? ext / n : 1.0;
    g.scan_all[d] = (g.periodic[d] && n < 3) || n < 3 ? 1 : 0;
    ncell *= n;
  }
  return ncell;
}

a2c_status grow(uint32_t **p, int64_t *cap, int64_t need) {
  if (need <= *cap) return A2C_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  if (cudaMalloc(p, sizeof(uint32_t) * std::max<int64_t>(need, 1)) != cudaSuccess) return A2C_ERR_NOMEM;
  *cap = need;
  return A2C_OK;
}
a2c_status grow(int **p, int64_t *cap, int64_t need) {
  if (need <= *cap) return A2C_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  if (cudaMalloc(p, sizeof(int) * std::max<int64_t>(need, 1)) != cudaSuccess) return A2C_ERR_NOMEM;
  *cap = need;
  return A2C_OK;
}

// Count, scan, allocate and fill from one candidate source.  ext = true:
// the extended lists (no Pd head counts, shells or HH1).
template <class Src>
a2c_status make_lists(a2c_gpp_ctx *c, const GridArgs &g0, Src src, bool ext) {
  const int64_t N = c->N;
  const a2c_gpp_params &p = c->p;
  cudaStream_t st = c->stream;
  DevBuf counts(st), hh1c(st), maxc(st), xf(st), qmax(st), npd_ext(st);
  GridArgs g = g0;  // with the prefilter's positions
  A2C_CUDA(cudaMallocAsync(&xf.p, sizeof(float4) * std::max<int64_t>(N, 1), st));
  A2C_CUDA(cudaMallocAsync(&qmax.p, sizeof(unsigned), st));
  A2C_CUDA(cudaMemsetAsync(qmax.p, 0, sizeof(unsigned), st));
  if (N > 0) {
    k_positions_f32<<<grid_for(N, 256), 256, 0, st>>>(c->d_X, N, (float4 *)xf.p, (unsigned *)qmax.p);
    A2C_CUDA(cudaGetLastError());
  }
  g.Xf = (const float4 *)xf.p;
  g.qmax_bits = (const unsigned *)qmax.p;
  A2C_CUDA(cudaMallocAsync(&counts.p, sizeof(int64_t) * (N + 1), st));
  A2C_CUDA(cudaMallocAsync(&hh1c.p, sizeof(int64_t) * (p.nH + 1), st));
  A2C_CUDA(cudaMallocAsync(&maxc.p, sizeof(int), st));
  A2C_CUDA(cudaMemsetAsync(counts.p, 0, sizeof(int64_t) * (N + 1), st));
  A2C_CUDA(cudaMemsetAsync(hh1c.p, 0, sizeof(int64_t) * (p.nH + 1), st));
  A2C_CUDA(cudaMemsetAsync(maxc.p, 0, sizeof(int), st));
  int64_t *off = ext ? c->d_ext_off : c->d_off;
  // the Pd head of each list (the extended lists keep theirs only for the fill)
  if (ext) A2C_CUDA(cudaMallocAsync(&npd_ext.p, sizeof(int) * std::max<int64_t>(N, 1), st));
  int *npd = ext ? (int *)npd_ext.p : c->d_npd;
  if (N > 0) {
    k_nbr_count<Src><<<grid_for(N, kBlock), kBlock, 0, st>>>(g, src, (int64_t *)counts.p, npd,
                                                             ext ? nullptr : (int64_t *)hh1c.p,
                                                             ext ? nullptr : c->d_shell, c->d_status);
    A2C_CUDA(cudaGetLastError());
    k_max_count<<<grid_for(N, 256), 256, 0, st>>>((const int64_t *)counts.p, N, (int *)maxc.p);
    A2C_CUDA(cudaGetLastError());
  }
  A2C_TRY(scan_exclusive((const int64_t *)counts.p, off, N + 1, st));
  if (!ext) A2C_TRY(scan_exclusive((const int64_t *)hh1c.p, c->d_hh1_off, (int64_t)p.nH + 1, st));
  int64_t total = 0, total1 = 0;
  int maxn = 0, stat = 0;
  A2C_CUDA(cudaMemcpyAsync(&total, off + N, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  if (!ext) A2C_CUDA(cudaMemcpyAsync(&total1, c->d_hh1_off + p.nH, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  A2C_CUDA(cudaMemcpyAsync(&maxn, maxc.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  A2C_CUDA(cudaMemcpyAsync(&stat, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  A2C_CUDA(cudaStreamSynchronize(st));
  if (stat & kStatusOverflow) return A2C_ERR_NEIGHBOR_OVERFLOW;
  if (ext) {
    A2C_TRY(grow(&c->d_ext_nbr, &c->ext_cap, total));
    c->ext_total = total;
  } else {
    A2C_TRY(grow(&c->d_nbr, &c->nbr_cap, total));
    A2C_TRY(grow(&c->d_hh1, &c->hh1_cap, total1));
    c->nbr_total = total;
    c->hh1_total = total1;
    c->max_neighbors = maxn;
  }
  if (N > 0) {
    k_nbr_fill<Src><<<grid_for(N, kBlock), kBlock, 0, st>>>(g, src, off, npd, ext ? c->d_ext_nbr : c->d_nbr,
                                                            c->d_hh1_off, ext ? nullptr : c->d_hh1, c->d_status);
    A2C_CUDA(cudaGetLastError());
  }
  A2C_CUDA(cudaMemcpyAsync(&stat, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  A2C_CUDA(cudaStreamSynchronize(st));
  if (stat & kStatusBadIndex) return A2C_ERR_STATE;
  if (!ext) {
    ++c->nbr_version;
    // span guard: lists at the cutoff, built from the positions in d_X
    for (int d = 0; d < 3; ++d) c->list_reach[d] = p.periodic[d] ? 0.0 : g.rc;
    if (c->d_xlist && N > 0)
      A2C_CUDA(cudaMemcpyAsync(c->d_xlist, c->d_X, sizeof(double) * 4 * N, cudaMemcpyDeviceToDevice, st));
  }
  return A2C_OK;
}

// Lists (rc, or rc + skin for the extended lists) from a cell list.
a2c_status lists_from_cells(a2c_gpp_ctx *c, const double *h_X, double cut, bool ext) {
  const int64_t N = c->N;
  cudaStream_t st = c->stream;
  GridArgs g;
  const int64_t ncell = make_grid(c, h_X, cut, g);
  A2C_CUDA(cudaMemsetAsync(c->d_status, 0, sizeof(int), st));
  DevBuf cell(st), ccount(st), cstart(st), cfill(st), items(st);
  A2C_CUDA(cudaMallocAsync(&cell.p, sizeof(int) * std::max<int64_t>(N, 1), st));
  A2C_CUDA(cudaMallocAsync(&ccount.p, sizeof(int) * (ncell + 1), st));
  A2C_CUDA(cudaMallocAsync(&cstart.p, sizeof(int64_t) * (ncell + 1), st));
  A2C_CUDA(cudaMallocAsync(&cfill.p, sizeof(int) * (ncell + 1), st));
  A2C_CUDA(cudaMallocAsync(&items.p, sizeof(int) * std::max<int64_t>(N, 1), st));
  A2C_CUDA(cudaMemsetAsync(ccount.p, 0, sizeof(int) * (ncell + 1), st));
  A2C_CUDA(cudaMemsetAsync(cfill.p, 0, sizeof(int) * (ncell + 1), st));
  if (N > 0) {
    k_cell_count<<<grid_for(N, 256), 256, 0, st>>>(g, (int *)cell.p, (int *)ccount.p);
    A2C_CUDA(cudaGetLastError());
  }
  A2C_TRY(scan_exclusive((const int *)ccount.p, (int64_t *)cstart.p, ncell + 1, st));
  if (N > 0) {
    k_cell_fill<<<grid_for(N, 256), 256, 0, st>>>(g, (const int *)cell.p, (const int64_t *)cstart.p,
                                                   (int *)cfill.p, (int *)items.p);
    k_cell_sort<<<grid_for(ncell, 256), 256, 0, st>>>(ncell, (const int64_t *)cstart.p, (int *)items.p);
    A2C_CUDA(cudaGetLastError());
  }
  return make_lists(c, g, CellSrc{(const int64_t *)cstart.p, (const int *)items.p}, ext);
}

// The lists at rc from the extended lists (the skin path): the same lists,
// shells and first H shells as make_lists over ExtSrc, with one exact test
// per candidate (k_refilter keeps the survivors) where make_lists tests
// each twice (count, then fill).
a2c_status refilter_lists(a2c_gpp_ctx *c, const GridArgs &g0) {
  const int64_t N = c->N;
  const a2c_gpp_params &p = c->p;
  cudaStream_t st = c->stream;
  DevBuf counts(st), hh1c(st), maxc(st), xf(st), qmax(st), tmp(st);
  GridArgs g = g0;
  A2C_CUDA(cudaMallocAsync(&xf.p, sizeof(float4) * std::max<int64_t>(N, 1), st));
  A2C_CUDA(cudaMallocAsync(&qmax.p, sizeof(unsigned), st));
  A2C_CUDA(cudaMemsetAsync(qmax.p, 0, sizeof(unsigned), st));
  A2C_CUDA(cudaMallocAsync(&tmp.p, sizeof(uint32_t) * std::max<int64_t>(c->ext_total, 1), st));
  A2C_CUDA(cudaMallocAsync(&counts.p, sizeof(int64_t) * (N + 1), st));
  A2C_CUDA(cudaMallocAsync(&hh1c.p, sizeof(int64_t) * (p.nH + 1), st));
  A2C_CUDA(cudaMallocAsync(&maxc.p, sizeof(int), st));
  A2C_CUDA(cudaMemsetAsync(counts.p, 0, sizeof(int64_t) * (N + 1), st));
  A2C_CUDA(cudaMemsetAsync(hh1c.p, 0, sizeof(int64_t) * (p.nH + 1), st));
  A2C_CUDA(cudaMemsetAsync(maxc.p, 0, sizeof(int), st));
  g.Xf = (const float4 *)xf.p;
  g.qmax_bits = (const unsigned *)qmax.p;
  if (N > 0) {
    k_positions_f32<<<grid_for(N, 256), 256, 0, st>>>(c->d_X, N, (float4 *)xf.p, (unsigned *)qmax.p);
    k_refilter<<<grid_for(N, kBlock), kBlock, 0, st>>>(g, ExtSrc{c->d_ext_off, c->d_ext_nbr}, (uint32_t *)tmp.p,
                                                       (int64_t *)counts.p, c->d_npd, (int64_t *)hh1c.p, c->d_shell);
    k_max_count<<<grid_for(N, 256), 256, 0, st>>>((const int64_t *)counts.p, N, (int *)maxc.p);
    A2C_CUDA(cudaGetLastError());
  }
  A2C_TRY(scan_exclusive((const int64_t *)counts.p, c->d_off, N + 1, st));
  A2C_TRY(scan_exclusive((const int64_t *)hh1c.p, c->d_hh1_off, (int64_t)p.nH + 1, st));
  int64_t total = 0, total1 = 0;
  int maxn = 0, stat = 0;
  A2C_CUDA(cudaMemcpyAsync(&total, c->d_off + N, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  A2C_CUDA(cudaMemcpyAsync(&total1, c->d_hh1_off + p.nH, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  A2C_CUDA(cudaMemcpyAsync(&maxn, maxc.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  A2C_CUDA(cudaStreamSynchronize(st));
  A2C_TRY(grow(&c->d_nbr, &c->nbr_cap, total));
  A2C_TRY(grow(&c->d_hh1, &c->hh1_cap, total1));
  c->nbr_total = total;
  c->hh1_total = total1;
  c->max_neighbors = maxn;
  if (N > 0) {
    k_refilter_pack<<<grid_for(N, kBlock), kBlock, 0, st>>>(g, c->d_ext_off, (const uint32_t *)tmp.p, c->d_off,
                                                            c->d_nbr, c->d_hh1_off, c->d_hh1, c->d_status);
    A2C_CUDA(cudaGetLastError());
  }
  A2C_CUDA(cudaMemcpyAsync(&stat, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  A2C_CUDA(cudaStreamSynchronize(st));
  if (stat & kStatusBadIndex) return A2C_ERR_STATE;
  ++c->nbr_version;
  for (int d = 0; d < 3; ++d) c->list_reach[d] = p.periodic[d] ? 0.0 : g.rc;
  if (c->d_xlist && N > 0)
    A2C_CUDA(cudaMemcpyAsync(c->d_xlist, c->d_X, sizeof(double) * 4 * N, cudaMemcpyDeviceToDevice, st));
  return A2C_OK;
}

// The k_check_positions flags for X (device memory, or a device-visible
// view of host memory when Xout is the device copy to fill).
a2c_status check_positions(a2c_gpp_ctx *c, const double *X, double *Xout, const double *Xref, int *flags) {
  const int64_t N = c->N;
  cudaStream_t st = c->stream;
  *flags = 0;
  if (N <= 0) return A2C_OK;
  int per = 0;
  for (int d = 0; d < 3; ++d) per |= c->p.periodic[d] ? 1 << d : 0;
  const double half = 0.5 * c->skin;
  DevBuf flag(st);
  A2C_CUDA(cudaMallocAsync(&flag.p, sizeof(int), st));
  A2C_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), st));
  k_check_positions<<<grid_for(N, 256), 256, 0, st>>>(X, Xout, Xref, N, half * half, c->p.box[0], c->p.box[1],
                                                      c->p.box[2], per, (int *)flag.p);
  A2C_CUDA(cudaGetLastError());
  A2C_CUDA(cudaMemcpyAsync(flags, flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  A2C_CUDA(cudaStreamSynchronize(st));
  return A2C_OK;
}

}  // namespace

a2c_status stage_positions(a2c_gpp_ctx *c, const double *X, const double *mX, int *moved) {
  const int64_t N = c->N;
  cudaStream_t st = c->stream;
  *moved = 0;
  if (N <= 0) return A2C_OK;
  DevBuf stage(st);
  A2C_CUDA(cudaMallocAsync(&stage.p, sizeof(double) * 4 * N, st));
  double *S = (double *)stage.p;
  if (!mX) A2C_CUDA(cudaMemcpyAsync(S, X, sizeof(double) * 4 * N, cudaMemcpyHostToDevice, st));
  int f = 0;
  A2C_TRY(check_positions(c, mX ? mX : S, mX ? S : nullptr, c->has_ext ? c->d_xref : nullptr, &f));
  if (f & kPosNonfinite) return A2C_ERR_NONFINITE;
  if (f & kPosOutside) return A2C_ERR_INVALID;
  A2C_CUDA(cudaMemcpyAsync(c->d_X, S, sizeof(double) * 4 * N, cudaMemcpyDeviceToDevice, st));
  *moved = (f & kPosMoved) ? 1 : 0;
  return A2C_OK;
}

a2c_status build_neighbors_device(a2c_gpp_ctx *c, const double *h_X) {
  c->has_ext = false;  // a full build invalidates the extended lists
  return lists_from_cells(c, h_X, c->p.rc, false);
}

// Skin path: rebuild the extended lists when a site has moved more than
// skin/2 since they were built (or none exist), then re-filter at rc.
// Positions are in c->d_X; h_X (may be null) serves the extended build's
// free-direction extents, else it is copied from the device.  moved: 0 or 1
// when stage_positions has already checked the positions, -1 to check here.
a2c_status update_neighbors_device(a2c_gpp_ctx *c, const double *h_X, int *rebuilt, int moved) {
  const int64_t N = c->N;
  cudaStream_t st = c->stream;
  bool need = !c->has_ext;
  if (!need && N > 0) {
    if (moved < 0) {
      int f = 0;
      A2C_TRY(check_positions(c, c->d_X, nullptr, c->d_xref, &f));
      moved = f & kPosMoved;
    }
    need = moved != 0;
  }
  if (need) {
    std::vector<double> hx;
    bool free_dim = false;
    for (int d = 0; d < 3; ++d) free_dim = free_dim || !c->p.periodic[d];
    if (!h_X && free_dim && N > 0) {
      hx.resize((size_t)(4 * N));
      A2C_CUDA(cudaMemcpyAsync(hx.data(), c->d_X, sizeof(double) * 4 * N, cudaMemcpyDeviceToHost, st));
      A2C_CUDA(cudaStreamSynchronize(st));
      h_X = hx.data();
    }
    A2C_TRY(lists_from_cells(c, h_X, c->p.rc + c->skin, true));
    if (N > 0) A2C_CUDA(cudaMemcpyAsync(c->d_xref, c->d_X, sizeof(double) * 4 * N, cudaMemcpyDeviceToDevice, st));
    c->has_ext = true;
  }
  if (rebuilt) *rebuilt = need ? 1 : 0;
  GridArgs g;
  make_grid(c, nullptr, c->p.rc, g);  // only the cutoff and box are read on this path
  A2C_CUDA(cudaMemsetAsync(c->d_status, 0, sizeof(int), st));
  return refilter_lists(c, g);
}

}  // namespace a2c
