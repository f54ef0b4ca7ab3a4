// FP64 plain-form kernels: pass 1 (site electron density), pass 2 (energy
// and gradient gather) and the occupancy gradient.  Compiled with
// -fmad=false.  One thread owns one site and walks its neighbor list in
// order, so every per-site sum is formed in the reference's order
// (electrondensity.cpp:20-49, minimizer.cpp:162-351, 658-789); the only
// difference from the CPU arithmetic is the device exp/pow/log.
//
// Geometry: for quadrature point k = 2m (+sqrt(3)) or 2m+1 (-sqrt(3)) only
// coordinate m of R^6 is non-zero, so r_k differs from the pair's base
// vector q_i - q_j in one component.  The reference forms
// r = ((q_i + u_i*xi0) - q_j) - u_j*xi1 with u = sqrt(2)*sigma; adding or
// subtracting an exact zero leaves a value unchanged, so the component-wise
// forms used below are bit-identical to it.
#include <algorithm>
#include <mutex>

#include "eam64.cuh"

#include "internal.cuh"

namespace a2c {
namespace {

constexpr int kBlock = 128;

struct PairGeo {
  double D[3];      // q_i - q_j (image applied)
  double Pi[3][2];  // (q_i[m] + u_i) - q_j[m], (q_i[m] - u_i) - q_j[m]
  double Pj[3][2];  // D[c] - u_j, D[c] + u_j
  double D2[3];     // D[c]^2
};

__device__ __forceinline__ void image_pos(const SiteArgs &a, const double *box, uint32_t e, double q[3]) {
  const int64_t j = e & kIdMask;
  q[0] = a.X[4 * j];
  q[1] = a.X[4 * j + 1];
  q[2] = a.X[4 * j + 2];
  const uint32_t c = e >> kIdBits;
  if (c != kNoShift) {
    const int m0 = (int)(c % 3u) - 1, m1 = (int)((c / 3u) % 3u) - 1, m2 = (int)(c / 9u) - 1;
    if (m0) q[0] = q[0] + m0 * box[0];
    if (m1) q[1] = q[1] + m1 * box[1];
    if (m2) q[2] = q[2] + m2 * box[2];
  }
}

__device__ __forceinline__ void make_geo(const double qi[3], double ui, const double qj[3], double uj, PairGeo &g) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    g.D[c] = qi[c] - qj[c];
    g.Pi[c][0] = (qi[c] + ui) - qj[c];
    g.Pi[c][1] = (qi[c] + (-ui)) - qj[c];
    g.Pj[c][0] = g.D[c] - uj;
    g.Pj[c][1] = g.D[c] - (-uj);
    g.D2[c] = g.D[c] * g.D[c];
  }
}

// r_k and |r_k| for quadrature point k (quadrature.cpp:111-132 ordering).
__device__ __forceinline__ double point(const PairGeo &g, int k, double r[3], int &comp, double &xi0) {
  const int m = k >> 1, sgn = k & 1;
  r[0] = g.D[0];
  r[1] = g.D[1];
  r[2] = g.D[2];
  double s2;
  if (m < 3) {
    comp = m;
    r[m] = g.Pi[m][sgn];
    xi0 = sgn ? -1.7320508075688772 : 1.7320508075688772;
  } else {
    comp = m - 3;
    r[m - 3] = g.Pj[m - 3][sgn];
    xi0 = 0.0;
  }
  const double a0 = (comp == 0) ? r[0] * r[0] : g.D2[0];
  const double a1 = (comp == 1) ? r[1] * r[1] : g.D2[1];
  const double a2 = (comp == 2) ? r[2] * r[2] : g.D2[2];
  s2 = a0 + a1 + a2;
  return sqrt(s2);
}

// Fsigma += dot(v, xi0): xi0 has one non-zero component, +-sqrt(3) at
// index comp (k < 6), or is all zero (k >= 6), and x + (+-0) == x.
__device__ __forceinline__ void accum(double Fq[3], double &Fs, double c, const double r[3], int k, int comp,
                                      double xi0) {
  const double v0 = c * r[0], v1 = c * r[1], v2 = c * r[2];
  Fq[0] = Fq[0] + v0;
  Fq[1] = Fq[1] + v1;
  Fq[2] = Fq[2] + v2;
  if (k < 6) {
    const double vc = (comp == 0) ? v0 : (comp == 1) ? v1 : v2;
    Fs = Fs + vc * xi0;
  }
}

// Pass 1 for site s (electrondensity.cpp:20-49).
__device__ __forceinline__ void density_site(const SiteArgs &a, int64_t s, bool iPd, const double *box) {
  const double qi[3] = {a.X[4 * s], a.X[4 * s + 1], a.X[4 * s + 2]};
  const double ui = (1.4142135623730951 * a.X[4 * s + 3]) * 1.7320508075688772;
  const int64_t b = a.off[s], m = b + a.npd[s], e = a.off[s + 1];
  const double W = a.W;
  double rho = 0.0;
  for (int64_t t = b; t < m; ++t) {
    const uint32_t en = a.nbr[t];
    const int64_t j = en & kIdMask;
    double qj[3];
    image_pos(a, box, en, qj);
    const double uj = (1.4142135623730951 * a.X[4 * j + 3]) * 1.7320508075688772;
    PairGeo g;
    make_geo(qi, ui, qj, uj, g);
#pragma unroll 1
    for (int k = 0; k < 12; ++k) {
      double r[3], xi0;
      int comp;
      const double sk = point(g, k, r, comp, xi0);
      rho = rho + eam64::f_Pd(sk) * W;
    }
  }
  for (int64_t t = m; t < e; ++t) {
    const uint32_t en = a.nbr[t];
    const int64_t j = en & kIdMask;
    double qj[3];
    image_pos(a, box, en, qj);
    const double uj = (1.4142135623730951 * a.X[4 * j + 3]) * 1.7320508075688772;
    const double xj = a.occ[j];
    PairGeo g;
    make_geo(qi, ui, qj, uj, g);
#pragma unroll 1
    for (int k = 0; k < 12; ++k) {
      double r[3], xi0;
      int comp;
      const double sk = point(g, k, r, comp, xi0);
      rho = rho + (xj * eam64::f_H(sk)) * W;
    }
  }
  a.rho[s] = rho;
  a.Fp[s] = iPd ? eam64::F_Pd_d(rho, a.eps) : eam64::F_H_d(rho, a.eps);
  if (!isfinite(rho)) atomicOr(a.status, kStatusNonfinite);
}

__global__ void __launch_bounds__(kBlock) k_density64(SiteArgs a) {
  const int64_t N = (int64_t)a.nPd + a.nH;
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N) return;
  density_site(a, s, s < a.nPd, a.box);
}

// Pass 2.  Per pair-point the three gradient terms of minimizer.cpp:180-190
// (and their Pd-H / H-Pd / H-H forms) are, with x_j = 1 for a Pd neighbor:
//   c1 = (((x_j*W)*F'_A(rho_i))*f'_B(s))/s
//   c2 = (((x_j*W)*F'_B(rho_j))*f'_A(s))/s
//   c3 = ((x_j*W)*phi'_AB(s))/s
// and the energy term ((0.5*x_i)*x_j)*W*phi_AB(s); the factors equal to 1
// for Pd sites multiply exactly, so one form serves all four pair types.
__device__ __forceinline__ void gradient_site(const SiteArgs &a, int64_t s, bool iPd, const double *box, double T) {
  const double qi[3] = {a.X[4 * s], a.X[4 * s + 1], a.X[4 * s + 2]};
  const double sigmai = a.X[4 * s + 3];
  const double ui = (1.4142135623730951 * sigmai) * 1.7320508075688772;
  const double xi = a.occ[s];
  const double rhoi = a.rho[s];
  const double Fpi = a.Fp[s];
  const double W = a.W, eps = a.eps;
  const int64_t b = a.off[s], m = b + a.npd[s], e = a.off[s + 1];
  double V = 0.0;
  V = V + (iPd ? eam64::F_Pd(rhoi) : xi * eam64::F_H(rhoi));
  double Fq[3] = {0.0, 0.0, 0.0}, Fs = 0.0;
  const double half_xi = 0.5 * xi;

  // Pd neighbors (PdPd for a Pd site, HPd for an H site)
  for (int64_t t = b; t < m; ++t) {
    const uint32_t en = a.nbr[t];
    const int64_t j = en & kIdMask;
    double qj[3];
    image_pos(a, box, en, qj);
    const double uj = (1.4142135623730951 * a.X[4 * j + 3]) * 1.7320508075688772;
    const double Fpj = a.Fp[j];
    PairGeo g;
    make_geo(qi, ui, qj, uj, g);
#pragma unroll 1
    for (int k = 0; k < 12; ++k) {
      double r[3], xi0;
      int comp;
      const double sk = point(g, k, r, comp, xi0);
      if (iPd) {
        const double fd = eam64::f_Pd_d(sk, eps);
        accum(Fq, Fs, ((W * Fpi) * fd) / sk, r, k, comp, xi0);
        accum(Fq, Fs, ((W * Fpj) * fd) / sk, r, k, comp, xi0);
        V = V + (0.5 * W) * eam64::phi_Pd(sk);
        accum(Fq, Fs, (W * eam64::phi_Pd_d(sk, eps)) / sk, r, k, comp, xi0);
      } else {
        accum(Fq, Fs, ((W * Fpi) * eam64::f_Pd_d(sk, eps)) / sk, r, k, comp, xi0);
        accum(Fq, Fs, ((W * Fpj) * eam64::f_H_d(sk, eps)) / sk, r, k, comp, xi0);
        V = V + (half_xi * W) * eam64::phi_PdH(sk);
        accum(Fq, Fs, (W * eam64::phi_PdH_d(sk, eps)) / sk, r, k, comp, xi0);
      }
    }
  }
  // H neighbors (PdH for a Pd site, HH for an H site)
  for (int64_t t = m; t < e; ++t) {
    const uint32_t en = a.nbr[t];
    const int64_t j = en & kIdMask;
    double qj[3];
    image_pos(a, box, en, qj);
    const double uj = (1.4142135623730951 * a.X[4 * j + 3]) * 1.7320508075688772;
    const double Fpj = a.Fp[j];
    const double xj = a.occ[j];
    const double xW = xj * W;
    PairGeo g;
    make_geo(qi, ui, qj, uj, g);
#pragma unroll 1
    for (int k = 0; k < 12; ++k) {
      double r[3], xi0;
      int comp;
      const double sk = point(g, k, r, comp, xi0);
      if (iPd) {
        accum(Fq, Fs, ((xW * Fpi) * eam64::f_H_d(sk, eps)) / sk, r, k, comp, xi0);
        accum(Fq, Fs, ((xW * Fpj) * eam64::f_Pd_d(sk, eps)) / sk, r, k, comp, xi0);
        V = V + ((0.5 * xj) * W) * eam64::phi_PdH(sk);
        accum(Fq, Fs, (xW * eam64::phi_PdH_d(sk, eps)) / sk, r, k, comp, xi0);
      } else {
        const double fd = eam64::f_H_d(sk, eps);
        accum(Fq, Fs, ((xW * Fpi) * fd) / sk, r, k, comp, xi0);
        accum(Fq, Fs, ((xW * Fpj) * fd) / sk, r, k, comp, xi0);
        V = V + ((half_xi * xj) * W) * eam64::phi_H(sk);
        accum(Fq, Fs, (xW * eam64::phi_H_d(sk, eps)) / sk, r, k, comp, xi0);
      }
    }
  }
  // minimizer.cpp:220-223 and 282-285
  const double cq = (1.0 / T) * xi;
  const double cs = ((1.0 / T) * 1.4142135623730951) * xi;
  const double ce = ((3.0 * kB) / sigmai) * xi;
  a.G[4 * s] = Fq[0] * cq;
  a.G[4 * s + 1] = Fq[1] * cq;
  a.G[4 * s + 2] = Fq[2] * cq;
  a.G[4 * s + 3] = Fs * cs - ce;
  a.Vs[s] = V;
  a.Ss[s] = dd::cr_log(sigmai) * xi;
  if (!isfinite(V) || !isfinite(Fs) || !isfinite(Fq[0] + Fq[1] + Fq[2])) atomicOr(a.status, kStatusNonfinite);
}

__global__ void __launch_bounds__(kBlock) k_gradient64(SiteArgs a) {
  const int64_t N = (int64_t)a.nPd + a.nH;
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N) return;
  gradient_site(a, s, s < a.nPd, a.box, a.T);
}

// Batched: the listed sites, each with its instance's box, T and species.
// Persistent grids (a fixed launch serves any list length, so the launch
// can live in a CUDA graph while the list shrinks).
__global__ void __launch_bounds__(kBlock) k_density64_list(SiteArgs a) {
  const int n = *a.bv.count;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int64_t s = a.bv.list[k];
    const InstGeo &g = a.bv.geo[a.bv.inst[s]];
    density_site(a, s, s - g.start < g.nPd, g.S);
  }
}

__global__ void __launch_bounds__(kBlock) k_gradient64_list(SiteArgs a) {
  const int n = *a.bv.count;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int64_t s = a.bv.list[k];
    const InstGeo &g = a.bv.geo[a.bv.inst[s]];
    gradient_site(a, s, s - g.start < g.nPd, g.S, g.T);
  }
}

// Occupancy gradient, minimizer.cpp:658-789, one thread per H site.  d_send
// receives log(x/(1-x)) + sum_Vx/(kB*T) (or stays 0, as send_H does).
__global__ void __launch_bounds__(kBlock) k_chem64(SiteArgs a, const double coePd0, const double coePd2,
                                                 const double coePd3, const double coeH0, const double coeH1,
                                                 const double coeH2, const double coeH3, const int *full,
                                                 double *send) {
  const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= a.nH) return;
  send[h] = 0.0;
  if (full[h] == 1) return;
  const int64_t s = (int64_t)a.nPd + h;
  const double qi[3] = {a.X[4 * s], a.X[4 * s + 1], a.X[4 * s + 2]};
  const double ui = (1.4142135623730951 * a.X[4 * s + 3]) * 1.7320508075688772;
  const double W = a.W, T = a.T, eps = a.eps;
  const double *box = a.box;
  const int64_t b = a.off[s], m = b + a.npd[s], e = a.off[s + 1];
  const double nHPd = (double)(m - b);
  double sum = 0.0;
  sum = sum + eam64::F_H(a.rho[s]);
  double tmp = (coeH1 * nHPd) * nHPd;
  for (int64_t t = m; t < e; ++t) {
    const double xj = a.occ[a.nbr[t] & kIdMask];
    tmp = tmp + ((2.0 * coeH2) * nHPd) * xj;
    for (int64_t u = m; u < e; ++u) tmp = tmp + (coeH3 * xj) * a.occ[a.nbr[u] & kIdMask];
  }
  sum = sum + ((0.5 * T) * coeH0) * tmp;
  for (int64_t t = b; t < m; ++t) {  // H-Pd pairs
    const uint32_t en = a.nbr[t];
    const int64_t j = en & kIdMask;
    double qj[3];
    image_pos(a, box, en, qj);
    const double uj = (1.4142135623730951 * a.X[4 * j + 3]) * 1.7320508075688772;
    const double WF = W * a.Fp[j];
    PairGeo g;
    make_geo(qi, ui, qj, uj, g);
#pragma unroll 1
    for (int k = 0; k < 12; ++k) {
      double r[3], xi0;
      int comp;
      const double sk = point(g, k, r, comp, xi0);
      sum = sum + WF * eam64::f_H(sk);
      sum = sum + W * eam64::phi_PdH(sk);
    }
    const int64_t bj = a.off[j], mj = bj + a.npd[j], ej = a.off[j + 1];
    sum = sum + ((T * coePd0) * coePd2) * (double)(mj - bj);
    for (int64_t u = mj; u < ej; ++u) sum = sum + ((T * coePd0) * coePd3) * a.occ[a.nbr[u] & kIdMask];
  }
  for (int64_t t = m; t < e; ++t) {  // H-H pairs
    const uint32_t en = a.nbr[t];
    const int64_t j = en & kIdMask;
    double qj[3];
    image_pos(a, box, en, qj);
    const double uj = (1.4142135623730951 * a.X[4 * j + 3]) * 1.7320508075688772;
    const double xj = a.occ[j];
    const double xWF = (xj * W) * a.Fp[j];
    const double xW = xj * W;
    PairGeo g;
    make_geo(qi, ui, qj, uj, g);
#pragma unroll 1
    for (int k = 0; k < 12; ++k) {
      double r[3], xi0;
      int comp;
      const double sk = point(g, k, r, comp, xi0);
      sum = sum + xWF * eam64::f_H(sk);
      sum = sum + xW * eam64::phi_H(sk);
    }
    const int64_t bj = a.off[j], mj = bj + a.npd[j], ej = a.off[j + 1];
    sum = sum + (((xj * T) * coeH0) * coeH2) * (double)(mj - bj);
    for (int64_t u = mj; u < ej; ++u) sum = sum + (((xj * T) * coeH0) * coeH3) * a.occ[a.nbr[u] & kIdMask];
  }
  const double x0 = a.occ[s];
  if (x0 > 0.0 && x0 < 1.0) send[h] = dd::cr_log(x0 / (1.0 - x0)) + sum / (kB * T);
}

__global__ void k_eam64(int which, const double *in, int64_t n, double eps, double *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = in[i];
  double r;
  switch (which) {
    case 0: r = eam64::F_Pd(v); break;
    case 1: r = eam64::F_Pd_d(v, eps); break;
    case 2: r = eam64::F_H(v); break;
    case 3: r = eam64::F_H_d(v, eps); break;
    case 4: r = eam64::f_Pd(v); break;
    case 5: r = eam64::f_Pd_d(v, eps); break;
    case 6: r = eam64::f_H(v); break;
    case 7: r = eam64::f_H_d(v, eps); break;
    case 8: r = eam64::phi_Pd(v); break;
    case 9: r = eam64::phi_Pd_d(v, eps); break;
    case 10: r = eam64::phi_PdH(v); break;
    case 11: r = eam64::phi_PdH_d(v, eps); break;
    case 12: r = eam64::phi_H(v); break;
    default: r = eam64::phi_H_d(v, eps); break;
  }
  out[i] = r;
}

SiteArgs site_args(a2c_gpp_ctx *c, const double *dX) {
  SiteArgs a;
  a.nPd = c->p.nPd;
  a.nH = c->p.nH;
  a.T = c->p.T;
  a.W = c->p.QWp;
  a.eps = c->p.eps;
  for (int d = 0; d < 3; ++d) a.box[d] = c->p.box[d];
  a.X = dX;
  a.occ = c->d_occ;
  a.off = c->d_off;
  a.nbr = c->d_nbr;
  a.npd = c->d_npd;
  a.rho = c->d_rho;
  a.Fp = c->d_Fp;
  a.G = c->d_G;
  a.Vs = c->d_Vs;
  a.Ss = c->d_Ss;
  a.status = c->d_status;
  return a;
}

}  // namespace

// Block size of the thread-per-site FP64 kernels.  A site's thread runs a
// long serial FP64 chain, and the warps of one SM share its narrow FP64
// pipe: a small system finishes sooner when its warps are spread over as
// many SMs as possible (one-warp blocks); a large one fills the device
// either way.  Results do not depend on the block size.
unsigned block64(int64_t n) { return n < (int64_t)current_device_sms() * kBlock * 4 ? 32u : (unsigned)kBlock; }

a2c_status launch_density64(a2c_gpp_ctx *c, const double *dX) {
  if (c->N == 0) return A2C_OK;
  SiteArgs a = site_args(c, dX);
  const unsigned bs = block64(c->N);
  k_density64<<<grid_for(c->N, (int)bs), bs, 0, c->stream>>>(a);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

a2c_status launch_gradient64(a2c_gpp_ctx *c, const double *dX, double *dG) {
  if (c->N == 0) return A2C_OK;
  SiteArgs a = site_args(c, dX);
  a.G = dG;
  const unsigned bs = block64(c->N);
  k_gradient64<<<grid_for(c->N, (int)bs), bs, 0, c->stream>>>(a);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

// One-warp blocks (see block64): the list length is only known on the
// device, and a short list must still spread over all SMs.
a2c_status launch_eval64_list(a2c_gpp_ctx *c, const double *dX, double *dG, const BatchView &bv) {
  constexpr int kLB = 32;
  // persistent grid sizes per device, computed once under a lock
  static std::mutex m;
  static int caps[kMaxDevices][2] = {};
  int cap[2];
  {
    const int dev = (c->device >= 0 && c->device < kMaxDevices) ? c->device : 0;
    std::lock_guard<std::mutex> lock(m);
    if (!caps[dev][0]) {
      const int sms = device_sms(c->device);
      int b0 = 0, b1 = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b0, k_density64_list, kLB, 0);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_gradient64_list, kLB, 0);
      (void)cudaGetLastError();
      if (b0 > 0 && b1 > 0) {
        caps[dev][0] = sms * b0;
        caps[dev][1] = sms * b1;
      }
    }
    cap[0] = std::max(1, caps[dev][0]);
    cap[1] = std::max(1, caps[dev][1]);
  }
  if (c->N == 0) return A2C_OK;
  SiteArgs a = site_args(c, dX);
  a.G = dG;
  a.bv = bv;
  const int64_t need = (c->N + kLB - 1) / kLB;
  k_density64_list<<<(unsigned)std::min<int64_t>(need, cap[0]), kLB, 0, c->stream>>>(a);
  k_gradient64_list<<<(unsigned)std::min<int64_t>(need, cap[1]), kLB, 0, c->stream>>>(a);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

a2c_status launch_eam64(a2c_gpp_ctx *c, int which, const double *d_in, int64_t n, double *d_out) {
  if (n <= 0) return A2C_OK;
  k_eam64<<<grid_for(n, 256), 256, 0, c->stream>>>(which, d_in, n, c->p.eps, d_out);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

a2c_status launch_chem64(a2c_gpp_ctx *c, const double *dX, double /*gamma_bd*/, double *d_send, const int *d_full) {
  if (c->p.nH == 0) return A2C_OK;
  SiteArgs a = site_args(c, dX);
  const double *cp = c->p.coe_Pd, *ch = c->p.coe_H;
  k_chem64<<<grid_for(c->p.nH, kBlock), kBlock, 0, c->stream>>>(a, cp[0], cp[2], cp[3], ch[0], ch[1], ch[2], ch[3],
                                                                 d_full, d_send);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

}  // namespace a2c
