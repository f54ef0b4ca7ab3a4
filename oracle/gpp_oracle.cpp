// CPU oracle for the GPP-EAM hot path -- TEST INFRASTRUCTURE ONLY (see
// gpp_oracle.h).  Compile with -O2 -ffp-contract=off and without
// -ffast-math: every floating-point expression below is written in the
// reference's evaluation order, and contraction into FMA would change bits.
#include "gpp_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../a2c_gb300/csrc/ddmath.cuh"

namespace {

const double kB = 8.6173324e-5;  // minimizer.cpp:92

// Arithmetic mode.  0 (default): the reference's arithmetic -- the C
// library's exp/pow/log and sequential sums; this mode is pinned bit for bit
// to the reference's own sources.  1: the device's arithmetic -- the
// portable exp/pow/log of ddmath.cuh (dd::fexp in the EAM functions,
// dd::cr_pow, dd::cr_log, dd::cr_exp in the diffusion step) and the GPU's
// fixed reduction tree for global sums and L-BFGS dot products; in this mode
// the GPU plain form reproduces the oracle bit for bit.
int g_arith = 0;
inline double e_exp(double x) { return g_arith ? a2c::dd::fexp(x) : std::exp(x); }
inline double e_pow(double u, double y) { return g_arith ? a2c::dd::cr_pow(u, y) : std::pow(u, y); }
inline double x_log(double u) { return g_arith ? a2c::dd::cr_log(u) : std::log(u); }
inline double d_exp(double x) { return g_arith ? a2c::dd::cr_exp(x) : std::exp(x); }

// The GPU's deterministic reduction: `grid` blocks of 256 threads, thread t
// of block b sums terms b*256+t, +grid*256, ... from 0.0; each warp then
// combines lanes pairwise at strides 16, 8, 4, 2, 1 (lane 0's value is
// kept); warp results 0..7 are combined the same way (zero-padded); a final
// block of 256 threads sums the block partials strided by 256 and combines
// them by the same tree.
double warp_tree(double v[32]) {
  for (int o = 16; o > 0; o >>= 1)
    for (int i = 0; i < o; ++i) v[i] = v[i] + v[i + o];
  return v[0];
}
double block_tree(const double lane[256]) {
  double w[32] = {0.0};
  for (int k = 0; k < 8; ++k) {
    double v[32];
    for (int i = 0; i < 32; ++i) v[i] = lane[32 * k + i];
    w[k] = warp_tree(v);
  }
  return warp_tree(w);
}
template <class Term>
double gpu_tree_sum(int64_t n, int maxgrid, Term term) {
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(maxgrid, (n + 255) / 256));
  std::vector<double> part((size_t)grid);
  double lane[256];
  for (int64_t b = 0; b < grid; ++b) {
    for (int t = 0; t < 256; ++t) {
      double s = 0.0;
      for (int64_t i = b * 256 + t; i < n; i += grid * 256) s += term(i);
      lane[t] = s;
    }
    part[(size_t)b] = block_tree(lane);
  }
  for (int t = 0; t < 256; ++t) {
    double s = 0.0;
    for (int64_t i = t; i < grid; i += 256) s += part[(size_t)i];
    lane[t] = s;
  }
  return block_tree(lane);
}

// The batched-instance reduction (one instance's terms): the n terms are
// cut into chunks of g_chunk consecutive terms; one block of 256 threads
// reduces each chunk (thread t sums its terms t, t+256, ... from 0.0, then
// the block tree above), and one block sums the chunk partials strided by
// 256 and combines them by the same tree.  g_chunk = 0 selects the
// single-system reduction (gpu_tree_sum).
int g_chunk = 0;
template <class Term>
double chunk_sum(int64_t n, Term term) {
  std::vector<double> part;
  double lane[256];
  for (int64_t c0 = 0; c0 < n; c0 += g_chunk) {
    const int64_t len = std::min<int64_t>(g_chunk, n - c0);
    for (int t = 0; t < 256; ++t) {
      double s = 0.0;
      for (int64_t i = t; i < len; i += 256) s += term(c0 + i);
      lane[t] = s;
    }
    part.push_back(block_tree(lane));
  }
  for (int t = 0; t < 256; ++t) {
    double s = 0.0;
    for (size_t i = (size_t)t; i < part.size(); i += 256) s += part[i];
    lane[t] = s;
  }
  return block_tree(lane);
}
template <class Term>
double dev_sum(int64_t n, int maxgrid, Term term) {
  return g_chunk > 0 ? chunk_sum(n, term) : gpu_tree_sum(n, maxgrid, term);
}

// --------------------------------------------------------------------------
// Vec3D arithmetic, in the order of Vector3D.h:83 (norm), 281-286 (dot),
// 291-302 (scalar * vector), and the component-wise +/- operators.
// --------------------------------------------------------------------------
struct V3 {
  double v[3];
};
inline V3 add(const V3 &a, const V3 &b) { return {{a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]}}; }
inline V3 sub(const V3 &a, const V3 &b) { return {{a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]}}; }
inline V3 scl(double c, const V3 &a) { return {{c * a.v[0], c * a.v[1], c * a.v[2]}}; }
inline double dot(const V3 &a, const V3 &b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]; }
inline double norm(const V3 &a) { return std::sqrt(a.v[0] * a.v[0] + a.v[1] * a.v[1] + a.v[2] * a.v[2]); }
inline void addto(V3 &a, const V3 &b) { a.v[0] += b.v[0]; a.v[1] += b.v[1]; a.v[2] += b.v[2]; }

// --------------------------------------------------------------------------
// EAM Pd-H potential, potential.cpp:16-205 (Zhou et al. 2007 fit).  The
// numeric constants are the reference's; they define the potential.
// --------------------------------------------------------------------------
struct Eam {
  double eps;

  // potential.cpp:16-38
  double F_Pd(double rho) const {
    const double a1 = 295878.9003038662, a2 = 0.20581955357385892,
                 a3 = 0.081228755904399, a4 = 0.05298811034615951;
    const double b[5][2] = {{2.4242616904962846, 1.4791899886249564},
                            {2.1376274623740064, 1.2169215689822592},
                            {1.6486007989726832, 0.8159825255339774},
                            {1.0749204110338482, 0.42007491336688396},
                            {0.5128056047933808, 0.12468685331167456}};
    rho /= 50.0;
    double y = a1 * (rho - a2);
    y = y * (rho - a3);
    y = y * rho;
    y = y * (rho + a4);
    for (int m = 0; m < 5; ++m) y = y * (rho * (rho - b[m][0]) + b[m][1]);
    const double Fprime = 0.251546;
    y -= 50.0 * Fprime * rho;
    return y;
  }
  double F_Pd_deriv(double rho) const { return (F_Pd(rho + eps) - F_Pd(rho - eps)) / (2.0 * eps); }

  // potential.cpp:45-57
  double F_H(double rho) const {
    const double c = 0.000197047, d = 1.18860, a = 9.99780, b = 60.0155, eps1 = 0.0540638;
    double y = -c * (1.0 / (2.0 + d) * e_pow(rho + eps1, 2.0 + d) -
                     (a + b) / (1.0 + d) * e_pow(rho + eps1, 1.0 + d) +
                     a * b / d * e_pow(rho + eps1, d));
    const double Fprime = -0.0296604;
    y -= Fprime * rho;
    return y;
  }
  double F_H_deriv(double rho) const { return (F_H(rho + eps) - F_H(rho - eps)) / (2.0 * eps); }

  // potential.cpp:64-98
  double f_Pd(double r) const {
    const double funRc = 0.001510569378297, funDerivRc = -0.077976566126292;
    const double a[7][2] = {{2.7267629107325706, 1.8716766113599643},
                            {2.50290548851635, 1.668549182690922},
                            {2.0924467509943674, 1.3150372774478005},
                            {1.564328475106985, 0.8987511149780485},
                            {1.009780903403673, 0.5124363774128722},
                            {0.5304054524800665, 0.2169886022464641},
                            {0.1356566408715063, 0.035852347523891395}};
    const double b1 = -0.02972698211669922, b2 = 0.6676807403564453,
                 b3 = -255.8965835571289, b4 = 14673.409149169922,
                 b5 = -2.597301181336601e7;
    r /= 5.0;
    double rho_a = r;
    for (int m = 0; m < 7; ++m) rho_a = rho_a * (r * (r - a[m][0]) + a[m][1]);
    double y = b1 + r * (b2 + r * (b3 + r * (b4 + b5 * rho_a)));
    if (r * 5.0 <= 0.0)
      y = 0.0;
    else if (r * 5.0 > 5.0)
      y = funRc * e_exp(funDerivRc / funRc * (r * 5.0 - 5.0));
    return y;
  }
  double f_Pd_deriv(double r) const { return (f_Pd(r + eps) - f_Pd(r - eps)) / (2.0 * eps); }

  // potential.cpp:105-119
  double f_H(double r) const {
    const double funRc = 0.009986990526578, funDerivRc = -0.013075667086408;
    const double C = 11.0025, delta = 1.30927;
    if (r <= 0.0) return 0.0;
    if (r > 5.35) return funRc * e_exp(funDerivRc / funRc * (r - 5.35));
    return C * e_exp(-delta * r);
  }
  double f_H_deriv(double r) const { return (f_H(r + eps) - f_H(r - eps)) / (2.0 * eps); }

  // potential.cpp:126-155
  double phi_Pd(double r) const {
    const double funRc = -0.016958780164980, funDerivRc = 0.089019679316328;
    const double a1 = -79415.24035137112, a2 = 1.0699996145674568,
                 a3 = 1.06015072612581, a4 = 0.42433991011376526,
                 a5 = 0.06169160085238687;
    const double b[4][2] = {{2.0586473420376348, 1.0683922574015199},
                            {1.6696359816422877, 0.7337878627470482},
                            {1.1690370066230809, 0.3909805777737639},
                            {0.2635598721249787, 0.033551116514910245}};
    r /= 5.0;
    double y = a1 * (r - a2);
    y = y * (r - a3);
    y = y * (r - a4);
    y = y * (r + a5);
    for (int m = 0; m < 4; ++m) y = y * (r * (r - b[m][0]) + b[m][1]);
    r *= 5.0;
    const double Fprime = 0.251546;
    y += 2 * Fprime * f_Pd(r);
    if (r <= 0.0)
      y = 0.0;
    else if (r > 5.05)
      y = funRc * e_exp(funDerivRc / funRc * (r - 5.05));
    return y;
  }
  double phi_Pd_deriv(double r) const { return (phi_Pd(r + eps) - phi_Pd(r - eps)) / (2.0 * eps); }

  // potential.cpp:162-177
  double phi_PdH(double r) const {
    const double funRc = -3.353001113951400e-04, funDerivRc = 7.147062196813336e-04;
    const double D = 0.2494540, alpha = 4.82613, beta = 2.13158, r0 = 1.50964;
    if (r <= 0.0) return 0.0;
    if (r > 5.35) return funRc * e_exp(funDerivRc / funRc * (r - 5.35));
    return D * (beta * e_exp(-alpha * (r - r0)) - alpha * e_exp(-beta * (r - r0)));
  }
  double phi_PdH_deriv(double r) const { return (phi_PdH(r + eps) - phi_PdH(r - eps)) / (2.0 * eps); }

  // potential.cpp:185-200
  double phi_H(double r) const {
    const double funRc = -0.003702722457147, funDerivRc = 0.005465945471933;
    const double D = 0.0661496, alpha = 3.67263, beta = 1.47797, r0 = 2.51980;
    if (r <= 0.0) return 0.0;
    if (r > 5.35) return funRc * e_exp(funDerivRc / funRc * (r - 5.35));
    return D * (beta * e_exp(-alpha * (r - r0)) - alpha * e_exp(-beta * (r - r0)));
  }
  double phi_H_deriv(double r) const { return (phi_H(r + eps) - phi_H(r - eps)) / (2.0 * eps); }
};

// --------------------------------------------------------------------------
// Quadrature rule, quadrature.cpp:101-133 with dim = 6: point 2m (2m+1) has
// +sqrt(3) (-sqrt(3)) in coordinate m of R^6, split into atom i (0-2) and
// atom j (3-5) blocks.
// --------------------------------------------------------------------------
struct Quad {
  V3 P[12][2];
  Quad() {
    const int dim = 6;
    for (int i = 0; i < dim; ++i) {
      double t1[6], t2[6];
      for (int j = 0; j < dim; ++j) {
        t1[j] = (i == j) ? std::sqrt(dim / 2.0) : 0.0;
        t2[j] = (i == j) ? -std::sqrt(dim / 2.0) : 0.0;
      }
      for (int b = 0; b < 2; ++b) {
        P[2 * i][b] = {{t1[3 * b], t1[3 * b + 1], t1[3 * b + 2]}};
        P[2 * i + 1][b] = {{t2[3 * b], t2[3 * b + 1], t2[3 * b + 2]}};
      }
    }
  }
};
const Quad &quad() {
  static Quad q;
  return q;
}

// --------------------------------------------------------------------------
// Site access helpers.  Entries carry the global id in the low 27 bits and
// the periodic image code (mx+1)+3(my+1)+9(mz+1) in the top 5 bits; the
// image position is q_j + m*L per periodic dimension (m = 0 adds nothing).
// --------------------------------------------------------------------------
const uint32_t ID_MASK = (1u << 27) - 1u;
const uint32_t NO_SHIFT = 13u;

inline V3 site_q(const double *X, int64_t s) { return {{X[4 * s], X[4 * s + 1], X[4 * s + 2]}}; }

inline V3 image_q(const orc_params *p, const double *X, uint32_t e) {
  const int64_t j = e & ID_MASK;
  V3 q = site_q(X, j);
  const uint32_t c = e >> 27;
  if (c != NO_SHIFT) {
    int m[3] = {int(c % 3) - 1, int((c / 3) % 3) - 1, int(c / 9) - 1};
    for (int d = 0; d < 3; ++d)
      if (m[d] != 0) q.v[d] = q.v[d] + m[d] * p->box[d];
  }
  return q;
}

// r = q_i + sqrt(2)*sigma_i*xi0 - q_j - sqrt(2)*sigma_j*xi1
// (electrondensity.cpp:23; minimizer.cpp:179), left to right.
inline V3 quad_r(const V3 &qi, double si, const V3 &qj, double sj, int k) {
  const Quad &Q = quad();
  V3 a = add(qi, scl(std::sqrt(2.0) * si, Q.P[k][0]));
  a = sub(a, qj);
  return sub(a, scl(std::sqrt(2.0) * sj, Q.P[k][1]));
}

struct Lists {
  const orc_params *p;
  const int64_t *off;
  const uint32_t *nbr;
  int64_t N() const { return (int64_t)p->nPd + p->nH; }
  // first H entry of site s (lists are sorted by global id)
  int64_t split(int64_t s) const {
    int64_t e = off[s];
    while (e < off[s + 1] && (int64_t)(nbr[e] & ID_MASK) < p->nPd) ++e;
    return e;
  }
};

// --------------------------------------------------------------------------
// Pass 1: electronDensity, electrondensity.cpp:12-56.
// --------------------------------------------------------------------------
double density_site(const Eam &eam, const Lists &L, const double *X, const double *xall, int64_t n) {
  const orc_params *p = L.p;
  const double QWp = p->QWp;
  const V3 qn = site_q(X, n);
  const double sn = X[4 * n + 3];
  const int64_t b = L.off[n], m = L.split(n), e = L.off[n + 1];
  double rho = 0.0;
  for (int64_t t = b; t < m; ++t) {  // Pd neighbors: f_Pd
    const int64_t j = L.nbr[t] & ID_MASK;
    const V3 qj = image_q(p, X, L.nbr[t]);
    for (int k = 0; k < 12; ++k) {
      V3 r = quad_r(qn, sn, qj, X[4 * j + 3], k);
      rho += eam.f_Pd(norm(r)) * QWp;
    }
  }
  for (int64_t t = m; t < e; ++t) {  // H neighbors: x_j * f_H
    const int64_t j = L.nbr[t] & ID_MASK;
    const V3 qj = image_q(p, X, L.nbr[t]);
    for (int k = 0; k < 12; ++k) {
      V3 r = quad_r(qn, sn, qj, X[4 * j + 3], k);
      rho += xall[j] * eam.f_H(norm(r)) * QWp;
    }
  }
  return rho;
}

std::vector<double> occupancy_all(const orc_params *p, const double *xH) {
  std::vector<double> x((size_t)p->nPd + p->nH, 1.0);
  for (int h = 0; h < p->nH; ++h) x[(size_t)p->nPd + h] = xH[h];
  return x;
}

void all_density(const Eam &eam, const Lists &L, const double *X, const double *xall, int nthreads,
                 std::vector<double> &rho) {
  const int64_t N = L.N();
  rho.assign((size_t)N, 0.0);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
  for (int64_t s = 0; s < N; ++s) rho[(size_t)s] = density_site(eam, L, X, xall, s);
}

// --------------------------------------------------------------------------
// Pass 2: minimizer.cpp:162-351 for one site.  Returns the site's energy
// contributions through *V (either added to the running sum in reference
// order, or accumulated from 0 as a per-site partial) and *S (sigma term).
// The embedding derivatives are re-evaluated per pair-point exactly as the
// reference does (its cost is part of the CPU baseline).
// --------------------------------------------------------------------------
void gradient_site(const Eam &eam, const Lists &L, const double *X, const double *xall,
                   const std::vector<double> &rho, int64_t s, double *V, double *S, double *G) {
  const orc_params *p = L.p;
  const double QWp = p->QWp, T = p->T;
  const Quad &Q = quad();
  const bool isPd = s < p->nPd;
  const V3 qi = site_q(X, s);
  const double sigmai = X[4 * s + 3];
  const double xi = xall[(size_t)s];
  const double rhoi = rho[(size_t)s];
  V3 Fq = {{0.0, 0.0, 0.0}};
  double Fs = 0.0;
  const int64_t b = L.off[s], m = L.split(s), e = L.off[s + 1];

  if (isPd) {
    *V += eam.F_Pd(rhoi);
    for (int64_t t = b; t < m; ++t) {  // Pd-Pd, minimizer.cpp:172-194
      const int64_t jj = L.nbr[t] & ID_MASK;
      const V3 qj = image_q(p, X, L.nbr[t]);
      const double sigmaj = X[4 * jj + 3];
      for (int k = 0; k < 12; ++k) {
        V3 r = quad_r(qi, sigmai, qj, sigmaj, k);
        V3 v;
        v = scl(QWp * eam.F_Pd_deriv(rhoi) * eam.f_Pd_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
        v = scl(QWp * eam.F_Pd_deriv(rho[jj]) * eam.f_Pd_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
        *V += 0.5 * QWp * eam.phi_Pd(norm(r));
        v = scl(QWp * eam.phi_Pd_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
      }
    }
    for (int64_t t = m; t < e; ++t) {  // Pd-H, minimizer.cpp:197-219
      const int64_t jj = L.nbr[t] & ID_MASK;
      const V3 qj = image_q(p, X, L.nbr[t]);
      const double sigmaj = X[4 * jj + 3];
      const double xj = xall[jj];
      for (int k = 0; k < 12; ++k) {
        V3 r = quad_r(qi, sigmai, qj, sigmaj, k);
        V3 v;
        v = scl(xj * QWp * eam.F_Pd_deriv(rhoi) * eam.f_H_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
        v = scl(xj * QWp * eam.F_H_deriv(rho[jj]) * eam.f_Pd_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
        *V += 0.5 * xj * QWp * eam.phi_PdH(norm(r));
        v = scl(xj * QWp * eam.phi_PdH_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
      }
    }
    for (int c = 0; c < 3; ++c) Fq.v[c] *= 1.0 / T;   // minimizer.cpp:220-223
    Fs *= 1.0 / T * std::sqrt(2.0);
    Fs -= 3.0 * kB / sigmai;
    *S += x_log(sigmai);
  } else {
    *V += xi * eam.F_H(rhoi);
    for (int64_t t = b; t < m; ++t) {  // H-Pd, minimizer.cpp:234-256
      const int64_t jj = L.nbr[t] & ID_MASK;
      const V3 qj = image_q(p, X, L.nbr[t]);
      const double sigmaj = X[4 * jj + 3];
      for (int k = 0; k < 12; ++k) {
        V3 r = quad_r(qi, sigmai, qj, sigmaj, k);
        V3 v;
        v = scl(QWp * eam.F_H_deriv(rhoi) * eam.f_Pd_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
        v = scl(QWp * eam.F_Pd_deriv(rho[jj]) * eam.f_H_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
        *V += 0.5 * xi * QWp * eam.phi_PdH(norm(r));
        v = scl(QWp * eam.phi_PdH_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
      }
    }
    for (int64_t t = m; t < e; ++t) {  // H-H, minimizer.cpp:259-281
      const int64_t jj = L.nbr[t] & ID_MASK;
      const V3 qj = image_q(p, X, L.nbr[t]);
      const double sigmaj = X[4 * jj + 3];
      const double xj = xall[jj];
      for (int k = 0; k < 12; ++k) {
        V3 r = quad_r(qi, sigmai, qj, sigmaj, k);
        V3 v;
        v = scl(xj * QWp * eam.F_H_deriv(rhoi) * eam.f_H_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
        v = scl(xj * QWp * eam.F_H_deriv(rho[jj]) * eam.f_H_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
        *V += 0.5 * xi * xj * QWp * eam.phi_H(norm(r));
        v = scl(xj * QWp * eam.phi_H_deriv(norm(r)) / norm(r), r);
        addto(Fq, v); Fs += dot(v, Q.P[k][0]);
      }
    }
    for (int c = 0; c < 3; ++c) Fq.v[c] *= 1.0 / T * xi;   // minimizer.cpp:282-285
    Fs *= 1.0 / T * std::sqrt(2.0) * xi;
    Fs -= 3.0 * kB / sigmai * xi;
    *S += x_log(sigmai) * xi;
  }
  G[4 * s] = Fq.v[0];
  G[4 * s + 1] = Fq.v[1];
  G[4 * s + 2] = Fq.v[2];
  G[4 * s + 3] = Fs;
}

bool check_params(const orc_params *p) {
  if (!p || p->nPd < 0 || p->nH < 0) return false;
  if ((int64_t)p->nPd + p->nH >= (int64_t(1) << 27)) return false;
  for (int d = 0; d < 3; ++d)
    if (p->periodic[d] && !(p->box[d] > 2.0 * p->rc)) return false;
  return true;
}

int eval_impl(const orc_params *p, const double *X, const double *xH, const int64_t *off,
              const uint32_t *nbr, int mode, int nthreads, double *f, double *G, double *rho_out,
              double *Vsite) {
  if (!check_params(p)) return 1;
  Eam eam{p->eps};
  Lists L{p, off, nbr};
  const int64_t N = L.N();
  std::vector<double> xall = occupancy_all(p, xH);
  std::vector<double> rho;
  all_density(eam, L, X, xall.data(), nthreads, rho);
  if (rho_out) std::memcpy(rho_out, rho.data(), sizeof(double) * (size_t)N);
  double sum_V = 0.0, sum_sigma = 0.0;
  if (mode == 0) {
    // one running accumulator in the reference's site order
    for (int64_t s = 0; s < N; ++s) {
      double before = sum_V;
      gradient_site(eam, L, X, xall.data(), rho, s, &sum_V, &sum_sigma, G);
      if (Vsite) Vsite[s] = sum_V - before;
    }
  } else {
    std::vector<double> Vs((size_t)N), Ss((size_t)N);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int64_t s = 0; s < N; ++s) {
      double v = 0.0, sg = 0.0;
      gradient_site(eam, L, X, xall.data(), rho, s, &v, &sg, G);
      Vs[(size_t)s] = v;
      Ss[(size_t)s] = sg;
    }
    if (g_arith) {
      sum_V = dev_sum(N, 1024, [&](int64_t i) { return Vs[(size_t)i]; });
      sum_sigma = dev_sum(N, 1024, [&](int64_t i) { return Ss[(size_t)i]; });
    } else {
      for (int64_t s = 0; s < N; ++s) {
        sum_V += Vs[(size_t)s];
        sum_sigma += Ss[(size_t)s];
      }
    }
    if (Vsite) std::memcpy(Vsite, Vs.data(), sizeof(double) * (size_t)N);
  }
  *f = 1.0 / p->T * sum_V - 3.0 * kB * sum_sigma;  // minimizer.cpp:353
  return 0;
}

// --------------------------------------------------------------------------
// Neighbor predicate: neighbors.cpp:74-82 and KDTree.h:241-262 (a candidate
// is dropped when any |coordinate difference| exceeds rc, or when the
// squared distance, summed x,y,z left to right, exceeds rc*rc; self is
// dropped), with the minimum-image extension for periodic dimensions.
// --------------------------------------------------------------------------
struct Grid {
  int n[3];
  double lo[3], cs[3];
  std::vector<int64_t> start;  // cell -> first slot
  std::vector<int64_t> items;  // site ids sorted by cell
};

int cell_coord(const orc_params *p, const Grid &g, double x, int d) {
  double t;
  if (p->periodic[d]) {
    double L = p->box[d];
    t = x - L * std::floor(x / L);
  } else {
    t = x - g.lo[d];
  }
  int c = (int)std::floor(t / g.cs[d]);
  if (c < 0) c = 0;
  if (c >= g.n[d]) c = g.n[d] - 1;
  return c;
}

void build_grid(const orc_params *p, const double *X, Grid &g) {
  const int64_t N = (int64_t)p->nPd + p->nH;
  for (int d = 0; d < 3; ++d) {
    double ext;
    if (p->periodic[d]) {
      g.lo[d] = 0.0;
      ext = p->box[d];
    } else {
      double lo = 1e300, hi = -1e300;
      for (int64_t s = 0; s < N; ++s) {
        lo = std::min(lo, X[4 * s + d]);
        hi = std::max(hi, X[4 * s + d]);
      }
      if (N == 0) lo = hi = 0.0;
      g.lo[d] = lo;
      ext = hi - lo;
    }
    int n = (int)std::floor(ext / p->rc);
    if (n < 1) n = 1;
    if (n > 1024) n = 1024;
    g.n[d] = n;
    g.cs[d] = (ext > 0.0) ? ext / n : 1.0;
  }
  const int64_t nc = (int64_t)g.n[0] * g.n[1] * g.n[2];
  std::vector<int64_t> cell((size_t)N);
  g.start.assign((size_t)nc + 1, 0);
  for (int64_t s = 0; s < N; ++s) {
    int c0 = cell_coord(p, g, X[4 * s], 0), c1 = cell_coord(p, g, X[4 * s + 1], 1),
        c2 = cell_coord(p, g, X[4 * s + 2], 2);
    cell[(size_t)s] = ((int64_t)c2 * g.n[1] + c1) * g.n[0] + c0;
    g.start[(size_t)cell[(size_t)s] + 1]++;
  }
  for (int64_t c = 0; c < nc; ++c) g.start[(size_t)c + 1] += g.start[(size_t)c];
  g.items.assign((size_t)N, 0);
  std::vector<int64_t> fill(g.start.begin(), g.start.end() - 1);
  for (int64_t s = 0; s < N; ++s) g.items[(size_t)fill[(size_t)cell[(size_t)s]]++] = s;
}

// Returns true and sets *entry / *d2 when j is a neighbor of i.
bool neighbor_test(const orc_params *p, const double *X, int64_t i, int64_t j, uint32_t *entry,
                   double *d2out) {
  if (i == j) return false;
  double dd[3];
  int m[3] = {0, 0, 0};
  for (int d = 0; d < 3; ++d) {
    const double qi = X[4 * i + d];
    double qj = X[4 * j + d];
    if (p->periodic[d]) {
      const double L = p->box[d];
      const double n = std::nearbyint((qj - qi) / L);
      m[d] = -(int)n;
      if (m[d] != 0) qj = qj + m[d] * L;
    }
    dd[d] = qj - qi;
    if (std::fabs(dd[d]) > p->rc) return false;
  }
  const double d2 = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2];
  if (d2 > p->rc * p->rc) return false;
  for (int d = 0; d < 3; ++d)
    if (m[d] < -1 || m[d] > 1) return false;
  *entry = (uint32_t)j | ((uint32_t)((m[0] + 1) + 3 * (m[1] + 1) + 9 * (m[2] + 1)) << 27);
  *d2out = d2;
  return true;
}

template <class Fn>
void for_candidates(const orc_params *p, const Grid &g, const double *X, int64_t i, Fn fn) {
  int c[3];
  for (int d = 0; d < 3; ++d) c[d] = cell_coord(p, g, X[4 * i + d], d);
  int lst[3][3], cnt[3];
  for (int d = 0; d < 3; ++d) {
    cnt[d] = 0;
    if (p->periodic[d] && g.n[d] < 3) {
      for (int t = 0; t < g.n[d]; ++t) lst[d][cnt[d]++] = t;
    } else {
      for (int o = -1; o <= 1; ++o) {
        int t = c[d] + o;
        if (p->periodic[d]) t = (t + g.n[d]) % g.n[d];
        else if (t < 0 || t >= g.n[d]) continue;
        lst[d][cnt[d]++] = t;
      }
    }
  }
  for (int a = 0; a < cnt[2]; ++a)
    for (int b = 0; b < cnt[1]; ++b)
      for (int e = 0; e < cnt[0]; ++e) {
        int64_t cell = ((int64_t)lst[2][a] * g.n[1] + lst[1][b]) * g.n[0] + lst[0][e];
        for (int64_t t = g.start[(size_t)cell]; t < g.start[(size_t)cell + 1]; ++t) fn(g.items[(size_t)t]);
      }
}

void site_neighbors(const orc_params *p, const Grid &g, const double *X, int64_t i,
                    std::vector<std::pair<uint32_t, double>> &out) {
  out.clear();
  for_candidates(p, g, X, i, [&](int64_t j) {
    uint32_t e;
    double d2;
    if (neighbor_test(p, X, i, j, &e, &d2)) out.push_back({e, d2});
  });
  std::sort(out.begin(), out.end(), [](const std::pair<uint32_t, double> &a, const std::pair<uint32_t, double> &b) {
    return (a.first & ID_MASK) < (b.first & ID_MASK);
  });
}

}  // namespace

extern "C" {

void orc_set_arith(int mode) { g_arith = mode ? 1 : 0; }
int orc_get_arith(void) { return g_arith; }
void orc_set_reduction(int chunk) { g_chunk = chunk > 0 ? chunk : 0; }
int orc_get_reduction(void) { return g_chunk; }

void orc_eam(int which, const double *in, int64_t n, double eps, double *out) {
  Eam e{eps};
  for (int64_t t = 0; t < n; ++t) {
    double v = in[t], r = 0.0;
    switch (which) {
      case 0: r = e.F_Pd(v); break;
      case 1: r = e.F_Pd_deriv(v); break;
      case 2: r = e.F_H(v); break;
      case 3: r = e.F_H_deriv(v); break;
      case 4: r = e.f_Pd(v); break;
      case 5: r = e.f_Pd_deriv(v); break;
      case 6: r = e.f_H(v); break;
      case 7: r = e.f_H_deriv(v); break;
      case 8: r = e.phi_Pd(v); break;
      case 9: r = e.phi_Pd_deriv(v); break;
      case 10: r = e.phi_PdH(v); break;
      case 11: r = e.phi_PdH_deriv(v); break;
      case 12: r = e.phi_H(v); break;
      case 13: r = e.phi_H_deriv(v); break;
      default: r = NAN;
    }
    out[t] = r;
  }
}

int orc_neighbor_counts(const orc_params *p, const double *X, int64_t *counts, int64_t *hh1_counts) {
  if (!check_params(p)) return 1;
  Grid g;
  build_grid(p, X, g);
  const int64_t N = (int64_t)p->nPd + p->nH;
  const double A75 = p->a_Pd * p->a_Pd * 0.75;
#pragma omp parallel
  {
    std::vector<std::pair<uint32_t, double>> out;
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < N; ++i) {
      site_neighbors(p, g, X, i, out);
      counts[i] = (int64_t)out.size();
      if (i >= p->nPd) {
        int64_t c = 0;
        for (auto &pr : out)
          if ((int64_t)(pr.first & ID_MASK) >= p->nPd && pr.second < A75) ++c;
        hh1_counts[i - p->nPd] = c;
      }
    }
  }
  return 0;
}

int orc_neighbor_fill(const orc_params *p, const double *X, const int64_t *off, uint32_t *nbr, int *PdPdnum,
                      const int64_t *hh1_off, int *hh1) {
  if (!check_params(p)) return 1;
  Grid g;
  build_grid(p, X, g);
  const int64_t N = (int64_t)p->nPd + p->nH;
  const double A75 = p->a_Pd * p->a_Pd * 0.75, A125 = p->a_Pd * p->a_Pd * 1.25;
  int bad = 0;
#pragma omp parallel reduction(| : bad)
  {
    std::vector<std::pair<uint32_t, double>> out;
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < N; ++i) {
      site_neighbors(p, g, X, i, out);
      if ((int64_t)out.size() != off[i + 1] - off[i]) {
        bad |= 1;
        continue;
      }
      int64_t w = off[i];
      for (auto &pr : out) nbr[w++] = pr.first;
      if (i < p->nPd) {  // minimizer.cpp:932-947
        int c0 = 0, c1 = 0, c2 = 0;
        for (auto &pr : out) {
          if ((int64_t)(pr.first & ID_MASK) >= p->nPd) continue;
          const double d2 = pr.second;
          if (d2 < A75) ++c0;
          else if (d2 > A75 && d2 < A125) ++c1;
          else ++c2;
        }
        PdPdnum[3 * i] = c0;
        PdPdnum[3 * i + 1] = c1;
        PdPdnum[3 * i + 2] = c2;
      } else {  // minimizer.cpp:996-1004
        int64_t h = i - p->nPd, w1 = hh1_off[h];
        for (auto &pr : out) {
          const int64_t j = pr.first & ID_MASK;
          if (j >= p->nPd && pr.second < A75) {
            if (w1 >= hh1_off[h + 1]) { bad |= 1; break; }
            hh1[w1++] = (int)(j - p->nPd);
          }
        }
      }
    }
  }
  return bad ? 2 : 0;
}

int orc_density(const orc_params *p, const double *X, const double *xH, const int64_t *off, const uint32_t *nbr,
                int nthreads, double *rho) {
  if (!check_params(p)) return 1;
  Eam eam{p->eps};
  Lists L{p, off, nbr};
  std::vector<double> xall = occupancy_all(p, xH), r;
  all_density(eam, L, X, xall.data(), nthreads, r);
  std::memcpy(rho, r.data(), sizeof(double) * r.size());
  return 0;
}

int orc_eval(const orc_params *p, const double *X, const double *xH, const int64_t *off, const uint32_t *nbr,
             int mode, int nthreads, double *f, double *G, double *rho, double *Vsite) {
  return eval_impl(p, X, xH, off, nbr, mode, nthreads > 0 ? nthreads : 1, f, G, rho, Vsite);
}

// minimizer.cpp:588-802 (one rank: the site partition is the identity).
int orc_chem_potential(const orc_params *p, const double *X, const double *xH, const int64_t *off,
                       const uint32_t *nbr, double gammabd, int nthreads, double *gamma, int *full_H) {
  if (!check_params(p)) return 1;
  Eam eam{p->eps};
  Lists L{p, off, nbr};
  const int nPd = p->nPd, nH = p->nH;
  const double T = p->T, QWp = p->QWp;
  const double *coe_Pd = p->coe_Pd, *coe_H = p->coe_H;
  std::vector<double> xall = occupancy_all(p, xH), rho;
  all_density(eam, L, X, xall.data(), nthreads > 0 ? nthreads : 1, rho);
  std::vector<double> send((size_t)nH, 0.0);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : 1)
  for (int i = 0; i < nH; ++i) {
    if (full_H[i] == 1) continue;
    const int64_t s = (int64_t)nPd + i;
    const V3 qi = site_q(X, s);
    const double sigmai = X[4 * s + 3];
    const int64_t b = off[s], m = L.split(s), e = off[s + 1];
    const double nHPd_i = (double)(m - b);
    double sum_Vx = 0.0;
    sum_Vx += eam.F_H(rho[(size_t)s]);
    double tmp = coe_H[1] * nHPd_i * nHPd_i;
    for (int64_t t = m; t < e; ++t) {
      const double xj = xall[nbr[t] & ID_MASK];
      tmp += 2.0 * coe_H[2] * nHPd_i * xj;
      for (int64_t u = m; u < e; ++u) tmp += coe_H[3] * xj * xall[nbr[u] & ID_MASK];
    }
    sum_Vx += 0.5 * T * coe_H[0] * tmp;
    for (int64_t t = b; t < m; ++t) {  // H-Pd pairs
      const int64_t jj = nbr[t] & ID_MASK;
      const V3 qj = image_q(p, X, nbr[t]);
      const double sigmaj = X[4 * jj + 3];
      for (int k = 0; k < 12; ++k) {
        V3 r = quad_r(qi, sigmai, qj, sigmaj, k);
        sum_Vx += QWp * eam.F_Pd_deriv(rho[jj]) * eam.f_H(norm(r));
        sum_Vx += QWp * eam.phi_PdH(norm(r));
      }
      const int64_t mj = L.split(jj);
      sum_Vx += T * coe_Pd[0] * coe_Pd[2] * (double)(mj - off[jj]);
      for (int64_t u = mj; u < off[jj + 1]; ++u) sum_Vx += T * coe_Pd[0] * coe_Pd[3] * xall[nbr[u] & ID_MASK];
    }
    for (int64_t t = m; t < e; ++t) {  // H-H pairs
      const int64_t jj = nbr[t] & ID_MASK;
      const V3 qj = image_q(p, X, nbr[t]);
      const double sigmaj = X[4 * jj + 3];
      const double xj = xall[jj];
      for (int k = 0; k < 12; ++k) {
        V3 r = quad_r(qi, sigmai, qj, sigmaj, k);
        sum_Vx += xj * QWp * eam.F_H_deriv(rho[jj]) * eam.f_H(norm(r));
        sum_Vx += xj * QWp * eam.phi_H(norm(r));
      }
      const int64_t mj = L.split(jj);
      sum_Vx += xj * T * coe_H[0] * coe_H[2] * (double)(mj - off[jj]);
      for (int64_t u = mj; u < off[jj + 1]; ++u) sum_Vx += xj * T * coe_H[0] * coe_H[3] * xall[nbr[u] & ID_MASK];
    }
    const double x0 = xH[i];
    if (x0 > 0.0 && x0 < 1.0) send[(size_t)i] = x_log(x0 / (1.0 - x0)) + sum_Vx / (kB * T);
  }
  for (int i = 0; i < nH; ++i) {  // minimizer.cpp:793-800
    if (full_H[i] == 1) continue;
    gamma[i] = send[(size_t)i] + 1.5;
    if (gamma[i] > gammabd) {
      gamma[i] = gammabd;
      if (xH[i] > 0.9999) full_H[i] = 1;
    }
  }
  return 0;
}

// integrate.cpp:9-87 (one rank).
int orc_diffuse(int nH, const double *x0, const int64_t *hh1_off, const int *hh1, const double *gamma,
                const int *full_H, double T, double dt, double v, double Qm, double xLb, double xUb, double *x) {
  const double prefactor = v * std::exp(-Qm / (kB * T));
  std::vector<double> send((size_t)nH, 0.0);
  for (int i = 0; i < nH; ++i) {
    if (full_H[i] == 1) continue;
    double x_deriv = 0.0;
    const double fi = gamma[i] - x_log(x0[i] / (1.0 - x0[i]));
    for (int64_t t = hh1_off[i]; t < hh1_off[i + 1]; ++t) {
      const int j = hh1[t];
      const double fj = gamma[j] - x_log(x0[j] / (1.0 - x0[j]));
      x_deriv += x0[j] * (1.0 - x0[i]) * d_exp(-(fi - fj) / 2.0) -
                 x0[i] * (1.0 - x0[j]) * d_exp((fi - fj) / 2.0);
    }
    send[(size_t)i] = x0[i] + prefactor * x_deriv * dt;
  }
  for (int i = 0; i < nH; ++i) {
    if (full_H[i] == 1) continue;
    x[i] = send[(size_t)i];
    if (x[i] < xLb) x[i] = xLb;
    else if (x[i] > xUb) x[i] = xUb;
  }
  return 0;
}

// boundaryconditions.cpp:30-55
void orc_dirichlet(const int *sites, int n, double gammabd, double xUb, double *x0, double *gamma, int *full_H) {
  for (int t = 0; t < n; ++t) {
    gamma[sites[t]] = gammabd;
    full_H[sites[t]] = 1;
    x0[sites[t]] = xUb;
  }
}

// calculateresults.cpp:8-78 (one rank; membership test instead of std::find)
void orc_macro_results(int nH, const double *x, const int *HSurf, int nSurf, double *xH, double *xHinterior) {
  std::vector<char> surf((size_t)nH, 0);
  for (int t = 0; t < nSurf; ++t)
    if (HSurf[t] >= 0 && HSurf[t] < nH) surf[(size_t)HSurf[t]] = 1;
  double s = 0.0, s3 = 0.0;
  for (int i = 0; i < nH; ++i) {
    s += x[i];
    if (!surf[(size_t)i]) s3 += x[i];
  }
  *xH = s / nH;
  *xHinterior = s3 / (nH - nSurf);
}

// Projected L-BFGS standing in for TAO BLMVM (minimizer.cpp:534-586, bounds
// at 804-830).  The same algorithm, step for step, drives the GPU evaluator.
int orc_minimize(const orc_params *p, double *X, const double *xH, const int64_t *off, const uint32_t *nbr,
                 const orc_lbfgs *lp, int nthreads, double *fmin, int *iters, int *nfev_out, double *gnorm_out,
                 int *reason) {
  if (!check_params(p) || !lp || lp->m < 1) return 1;
  const int64_t n = 4 * ((int64_t)p->nPd + p->nH);
  const double lb = lp->sigma_lb;
  const double f_noise = lp->f_noise > 0.0 ? lp->f_noise : 1.0e-14;
  const double stall_rtol = lp->stall_rtol > 0.0 ? lp->stall_rtol : 1.0e-14;
  std::vector<double> fhist;  // f after each accepted iteration
  auto is_sig = [](int64_t t) { return (t & 3) == 3; };
  auto project = [&](std::vector<double> &v) {
    for (int64_t t = 3; t < n; t += 4)
      if (v[(size_t)t] < lb) v[(size_t)t] = lb;
  };
  auto dotv = [&](const std::vector<double> &a, const std::vector<double> &b) {
    if (g_arith) return dev_sum(n, 512, [&](int64_t t) { return a[(size_t)t] * b[(size_t)t]; });
    double s = 0.0;
    for (int64_t t = 0; t < n; ++t) s += a[(size_t)t] * b[(size_t)t];
    return s;
  };
  std::vector<double> x(X, X + n), g((size_t)n), pg((size_t)n), d((size_t)n), xn((size_t)n), gn((size_t)n);
  project(x);
  double f;
  int nfev = 0;
  auto F = [&](const std::vector<double> &xx, double *ff, std::vector<double> &gg) {
    ++nfev;
    return eval_impl(p, xx.data(), xH, off, nbr, 1, nthreads > 0 ? nthreads : 1, ff, gg.data(), nullptr, nullptr);
  };
  if (F(x, &f, g)) return 1;
  const int m = lp->m;
  std::vector<std::vector<double>> S((size_t)m), Y((size_t)m);
  std::vector<double> rhoS((size_t)m), alph((size_t)m);
  int npairs = 0, head = 0;  // head = slot of the next insert
  int it = 0, why = 0;
  double gnorm = 0.0;
  while (true) {
    for (int64_t t = 0; t < n; ++t)
      pg[(size_t)t] = (is_sig(t) && x[(size_t)t] <= lb && g[(size_t)t] > 0.0) ? 0.0 : g[(size_t)t];
    gnorm = std::sqrt(dotv(pg, pg));
    if (!std::isfinite(f) || !std::isfinite(gnorm)) { why = -4; break; }
    if (gnorm <= lp->gatol) { why = 3; break; }
    if (it >= lp->max_it) { why = -2; break; }
    if (nfev >= lp->max_fev) { why = -5; break; }
    auto steepest = [&]() {
      double amax = 0.0;
      for (int64_t t = 0; t < n; ++t) amax = std::max(amax, std::fabs(pg[(size_t)t]));
      const double sc = lp->init_step / amax;
      for (int64_t t = 0; t < n; ++t) d[(size_t)t] = -pg[(size_t)t] * sc;
    };
    if (npairs == 0) {
      steepest();
    } else {
      std::vector<double> &q = d;
      q = pg;
      for (int c = 0; c < npairs; ++c) {  // newest to oldest
        int sl = ((head - 1 - c) % m + m) % m;
        alph[(size_t)sl] = rhoS[(size_t)sl] * dotv(S[(size_t)sl], q);
        for (int64_t t = 0; t < n; ++t) q[(size_t)t] -= alph[(size_t)sl] * Y[(size_t)sl][(size_t)t];
      }
      const int nw = ((head - 1) % m + m) % m;
      const double gam = dotv(S[(size_t)nw], Y[(size_t)nw]) / dotv(Y[(size_t)nw], Y[(size_t)nw]);
      for (int64_t t = 0; t < n; ++t) q[(size_t)t] *= gam;
      for (int c = npairs - 1; c >= 0; --c) {  // oldest to newest
        int sl = ((head - 1 - c) % m + m) % m;
        const double beta = rhoS[(size_t)sl] * dotv(Y[(size_t)sl], q);
        for (int64_t t = 0; t < n; ++t) q[(size_t)t] += (alph[(size_t)sl] - beta) * S[(size_t)sl][(size_t)t];
      }
      for (int64_t t = 0; t < n; ++t) {
        d[(size_t)t] = -q[(size_t)t];
        if (is_sig(t) && x[(size_t)t] <= lb && g[(size_t)t] > 0.0) d[(size_t)t] = 0.0;
      }
    }
    double gd = dotv(g, d);
    if (!(gd < 0.0)) {
      npairs = 0;
      head = 0;
      steepest();
    }
    double dmax = 0.0;
    for (int64_t t = 0; t < n; ++t) dmax = std::max(dmax, std::fabs(d[(size_t)t]));
    double alpha = (lp->max_step > 0.0 && dmax > lp->max_step) ? lp->max_step / dmax : 1.0, fn = 0.0;
    bool ok = false;
    for (int ls = 0; ls < lp->max_ls; ++ls) {
      for (int64_t t = 0; t < n; ++t) xn[(size_t)t] = x[(size_t)t] + alpha * d[(size_t)t];
      project(xn);
      if (F(xn, &fn, gn)) return 1;
      double dec = 0.0;
      if (g_arith)
        dec = dev_sum(n, 512, [&](int64_t t) { return g[(size_t)t] * (xn[(size_t)t] - x[(size_t)t]); });
      else
        for (int64_t t = 0; t < n; ++t) dec += g[(size_t)t] * (xn[(size_t)t] - x[(size_t)t]);
      if (std::isfinite(fn) && fn <= f + lp->c1 * dec) { ok = true; break; }
      // objective change within its noise: the derivative form of the
      // Armijo test, g_new.s <= (2 c1 - 1) g.s (exact for a quadratic)
      if (std::isfinite(fn) && std::fabs(fn - f) <= f_noise * std::fabs(f)) {
        double dn = 0.0;
        if (g_arith)
          dn = dev_sum(n, 512, [&](int64_t t) { return gn[(size_t)t] * (xn[(size_t)t] - x[(size_t)t]); });
        else
          for (int64_t t = 0; t < n; ++t) dn += gn[(size_t)t] * (xn[(size_t)t] - x[(size_t)t]);
        if (dn <= (2.0 * lp->c1 - 1.0) * dec) { ok = true; break; }
      }
      alpha *= 0.5;
      if (nfev >= lp->max_fev) break;
    }
    if (!ok) {
      if (npairs > 0 && nfev < lp->max_fev) {
        npairs = 0;
        head = 0;
        continue;
      }
      why = (nfev >= lp->max_fev) ? -5 : -6;
      break;
    }
    std::vector<double> s((size_t)n), y((size_t)n);
    for (int64_t t = 0; t < n; ++t) {
      s[(size_t)t] = xn[(size_t)t] - x[(size_t)t];
      y[(size_t)t] = gn[(size_t)t] - g[(size_t)t];
    }
    const double sy = dotv(s, y), yy = dotv(y, y);
    if (sy > 2.220446049250313e-16 * yy) {
      S[(size_t)head] = std::move(s);
      Y[(size_t)head] = std::move(y);
      rhoS[(size_t)head] = 1.0 / sy;
      head = (head + 1) % m;
      if (npairs < m) ++npairs;
    }
    x.swap(xn);
    g.swap(gn);
    f = fn;
    ++it;
    fhist.push_back(f);
    const int W = lp->stall_window;
    if (W > 0 && (int)fhist.size() > W && fhist[fhist.size() - 1 - W] - f <= stall_rtol * std::fabs(f)) {
      why = 6;
      break;
    }
  }
  std::memcpy(X, x.data(), sizeof(double) * (size_t)n);
  *fmin = f;
  *iters = it;
  *nfev_out = nfev;
  *gnorm_out = gnorm;
  *reason = why;
  return 0;
}

int orc_lattice_fcc(const int ncell[3], double a, double pos_std, double sigma_lo, double sigma_hi, int x_mode,
                    double x_center, double x_half, double x_matrix, double x_nucleus, double nucleus_radius,
                    double interface_width, double xLb, double xUb, uint64_t seed, double *X, double *xH,
                    int *surface) {
  if (!ncell || !X || ncell[0] < 1 || ncell[1] < 1 || ncell[2] < 1 || !(a > 0.0) || pos_std < 0.0) return -1;
  const int64_t nx = ncell[0], ny = ncell[1], nz = ncell[2];
  const int64_t half = 4 * nx * ny * nz, N = 2 * half;
  // lattice point of site s: species s / half, cell (s % half) / 4 in
  // z-major order, basis vector (s % half) % 4
  static const double basis[2][4][3] = {{{0.0, 0.0, 0.0}, {0.0, 0.5, 0.5}, {0.5, 0.0, 0.5}, {0.5, 0.5, 0.0}},
                                        {{0.5, 0.0, 0.0}, {0.0, 0.5, 0.0}, {0.0, 0.0, 0.5}, {0.5, 0.5, 0.5}}};
  auto lattice_point = [&](int64_t s, double q[3]) {
    const int sp = s >= half ? 1 : 0;
    const int64_t r = s - sp * half, cell = r / 4;
    const int b = (int)(r % 4);
    const int64_t cx = cell % nx, cy = (cell / nx) % ny, cz = cell / (nx * ny);
    q[0] = a * ((double)cx + basis[sp][b][0]);
    q[1] = a * ((double)cy + basis[sp][b][1]);
    q[2] = a * ((double)cz + basis[sp][b][2]);
  };
  std::mt19937_64 rng(seed);
  auto uniform = [&]() { return (double)(rng() >> 11) * (1.0 / 9007199254740992.0); };
  double pending = 0.0;
  bool have_pending = false;
  auto normal = [&]() {
    if (have_pending) {
      have_pending = false;
      return pending;
    }
    const double u1 = 1.0 - uniform(), u2 = uniform();
    const double rad = std::sqrt(-2.0 * std::log(u1)), ang = 6.283185307179586 * u2;
    pending = rad * std::sin(ang);
    have_pending = true;
    return rad * std::cos(ang);
  };
  for (int64_t s = 0; s < N; ++s) {
    double q[3];
    lattice_point(s, q);
    for (int d = 0; d < 3; ++d) X[4 * s + d] = q[d] + pos_std * normal();
  }
  for (int64_t s = 0; s < N; ++s)
    X[4 * s + 3] = sigma_hi > sigma_lo ? sigma_lo + (sigma_hi - sigma_lo) * uniform() : sigma_lo;
  const double centre[3] = {0.5 * a * (double)nx, 0.5 * a * (double)ny, 0.5 * a * (double)nz};
  for (int64_t h = 0; h < half; ++h) {
    double q[3];
    lattice_point(half + h, q);
    if (xH) {
      double x;
      if (x_mode == 1) {
        const double dx = q[0] - centre[0], dy = q[1] - centre[1], dz = q[2] - centre[2];
        const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
        x = x_matrix + (x_nucleus - x_matrix) * 0.5 * (1.0 - std::tanh((r - nucleus_radius) / interface_width));
        x += x_half * (2.0 * uniform() - 1.0);
      } else {
        x = x_center + x_half * (2.0 * uniform() - 1.0);
      }
      xH[h] = std::min(std::max(x, xLb), xUb);
    }
    if (surface) surface[h] = q[2] < 1e-6 ? 1 : 0;
  }
  return 0;
}

}  // extern "C"
