// a2c_host.hpp -- the reference's host entry points, GB300 edition.
//
// Header-only C++ over the C ABI in a2c_gpp.h, with the reference's names
// and argument lists so that a2c's own driver code compiles against it:
//   Minimizer::Minimizer / initialize / minimizeFreeEntropy /
//     calculateChemicalPotential / findLocalNeighbors   (minimizer.h:52-99)
//   findNeighbors                                        (neighbors.cpp:8)
//   integrateDiffusion                                   (integrate.cpp:9)
//   enforceBoundaryConditions                            (boundaryconditions.cpp:30)
//   calculateMacroResults                                (calculateresults.cpp:8)
//   readResults (+ writeResults, which the reference tree lacks)
//                                                        (readresults.cpp:10)
//   SetupLatticeVariables (the lattices of an input file) (SpaceInitializer.cpp:41)
// The vector type V3 is the caller's (anything with operator[](int) over
// three doubles, such as a2c's Vec3D) and the input type is anything with the
// reference's `input.file.*` fields (T0, eps, rc, a_Pd, xLb, xUb, v, Qm,
// foldername, filename_base, restart_file_num), so no a2c header is needed
// here.  Errors: every function returns the a2c_status of the first failing
// C-ABI call (0 = success, like the reference's PetscErrorCode); nothing
// throws.  No PETSc or MPI: one process drives one GPU.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "a2c_gpp.h"

namespace a2c_gb300 {

using std::vector;

namespace detail {
template <class V3>
inline void pack(const vector<V3> &qPd, const vector<V3> &qH, const vector<double> &sPd, const vector<double> &sH,
                 vector<double> &X) {
  X.resize(4 * (qPd.size() + qH.size()));
  size_t k = 0;
  for (size_t i = 0; i < qPd.size(); ++i) {
    X[k++] = qPd[i][0];
    X[k++] = qPd[i][1];
    X[k++] = qPd[i][2];
    X[k++] = sPd[i];
  }
  for (size_t i = 0; i < qH.size(); ++i) {
    X[k++] = qH[i][0];
    X[k++] = qH[i][1];
    X[k++] = qH[i][2];
    X[k++] = sH[i];
  }
}
template <class V3>
inline void unpack(const vector<double> &X, vector<V3> &qPd, vector<V3> &qH, vector<double> &sPd,
                   vector<double> &sH) {
  size_t k = 0;
  for (size_t i = 0; i < qPd.size(); ++i) {
    qPd[i][0] = X[k++];
    qPd[i][1] = X[k++];
    qPd[i][2] = X[k++];
    sPd[i] = X[k++];
  }
  for (size_t i = 0; i < qH.size(); ++i) {
    qH[i][0] = X[k++];
    qH[i][1] = X[k++];
    qH[i][2] = X[k++];
    sH[i] = X[k++];
  }
}
inline void to_csr(const vector<vector<int> > &L, vector<int64_t> &off, vector<int> &idx) {
  off.assign(L.size() + 1, 0);
  idx.clear();
  for (size_t i = 0; i < L.size(); ++i) {
    idx.insert(idx.end(), L[i].begin(), L[i].end());
    off[i + 1] = (int64_t)idx.size();
  }
}
inline a2c_status from_ctx(a2c_gpp_ctx *ctx, int list, size_t n, vector<vector<int> > &L) {
  int64_t tot = 0;
  a2c_status s = a2c_gpp_neighbor_total(ctx, list, &tot);
  if (s) return s;
  vector<int64_t> off(n + 1);
  vector<int> idx((size_t)(tot > 0 ? tot : 1));
  s = a2c_gpp_get_neighbors(ctx, list, off.data(), idx.data());
  if (s) return s;
  L.assign(n, vector<int>());
  for (size_t i = 0; i < n; ++i) L[i].assign(idx.begin() + off[i], idx.begin() + off[i + 1]);
  return A2C_OK;
}
template <class Input>
inline a2c_gpp_params params(const Input &input, int nPd, int nH) {
  a2c_gpp_params p;
  a2c_gpp_default_params(&p);
  p.nPd = nPd;
  p.nH = nH;
  p.T = input.file.T0;
  p.eps = input.file.eps;
  p.rc = input.file.rc;
  p.a_Pd = input.file.a_Pd;
  return p;
}
}  // namespace detail

// The reference's solver wrapper (minimizer.h:52-99).  The TAO BLMVM solve is
// the device L-BFGS of a2c_gpp_minimize; `lbfgs` and `params` may be tuned
// before initialize (precision, periodic box, correction coefficients).
class Minimizer {
 public:
  a2c_gpp_params params;
  a2c_lbfgs_params lbfgs;
  a2c_status last_status = A2C_OK;
  int last_reason = 0, last_iters = 0;

  Minimizer(int * = nullptr, char *** = nullptr) {  // PetscInitialize had nothing to do here
    a2c_gpp_default_params(&params);
    a2c_lbfgs_default_params(&lbfgs);
  }
  ~Minimizer() { a2c_gpp_destroy(ctx_); }
  Minimizer(const Minimizer &) = delete;
  Minimizer &operator=(const Minimizer &) = delete;

  a2c_gpp_ctx *context() const { return ctx_; }

  // minimizer.cpp:484-546: creates the device context and loads the caller's
  // neighbor lists (in their order) and state.  QPp is the reference's
  // 12-point rule (only its size is checked); QWp and coe_* are used.
  template <class Input, class V3, class QP>
  a2c_status initialize(Input *input, vector<vector<int> > *PdPd, vector<vector<int> > *PdH,
                        vector<vector<int> > *HPd, vector<vector<int> > *HH, vector<V3> &q_Pd0, vector<V3> &q_H0,
                        vector<double> &sigma_Pd0, vector<double> &sigma_H0, vector<double> &x0, QP *QPp,
                        double &QWp, vector<double> *coe_Pd, vector<double> *coe_H,
                        vector<vector<int> > *HH1 = nullptr) {
    if (QPp && QPp->size() != 12) return A2C_ERR_INVALID;
    const int nPd = (int)q_Pd0.size(), nH = (int)q_H0.size();
    if (!PdPd || !PdH || !HPd || !HH || PdPd->size() != (size_t)nPd || PdH->size() != (size_t)nPd ||
        HPd->size() != (size_t)nH || HH->size() != (size_t)nH || (HH1 && HH1->size() != (size_t)nH) ||
        sigma_Pd0.size() != (size_t)nPd || sigma_H0.size() != (size_t)nH || x0.size() != (size_t)nH)
      return last_status = A2C_ERR_INVALID;
    a2c_gpp_params p = params;
    const a2c_gpp_params q = detail::params(*input, nPd, nH);
    p.nPd = nPd;
    p.nH = nH;
    p.T = q.T;
    p.eps = q.eps;
    p.rc = q.rc;
    p.a_Pd = q.a_Pd;
    p.QWp = QWp;
    for (int k = 0; k < 4; ++k) {
      p.coe_Pd[k] = coe_Pd && coe_Pd->size() > (size_t)k ? (*coe_Pd)[k] : 0.0;
      p.coe_H[k] = coe_H && coe_H->size() > (size_t)k ? (*coe_H)[k] : 0.0;
    }
    params = p;
    a2c_gpp_destroy(ctx_);
    ctx_ = nullptr;
    nPd_ = nPd;
    nH_ = nH;
    a2c_status s = a2c_gpp_create(&params, &ctx_);
    if (s) return last_status = s;
    vector<double> X;
    detail::pack(q_Pd0, q_H0, sigma_Pd0, sigma_H0, X);
    if ((s = a2c_gpp_set_occupancy(ctx_, x0.data()))) return last_status = s;
    vector<int64_t> o[5];
    vector<int> ix[5];
    detail::to_csr(*PdPd, o[0], ix[0]);
    detail::to_csr(*PdH, o[1], ix[1]);
    detail::to_csr(*HPd, o[2], ix[2]);
    detail::to_csr(*HH, o[3], ix[3]);
    if (HH1) detail::to_csr(*HH1, o[4], ix[4]);
    else o[4].assign((size_t)nH + 1, 0);
    s = a2c_gpp_set_neighbor_lists(ctx_, X.data(), o[0].data(), ix[0].data(), o[1].data(), ix[1].data(),
                                   o[2].data(), ix[2].data(), o[3].data(), ix[3].data(), o[4].data(),
                                   ix[4].data(), nullptr);
    return last_status = s;
  }

  // minimizer.cpp:548-586; free_entropy receives the minimum.
  template <class V3>
  a2c_status minimizeFreeEntropy(double /*dt*/, vector<V3> &q_Pd0, vector<V3> &q_H0, vector<double> &sigma_Pd0,
                                 vector<double> &sigma_H0, vector<double> &x0, vector<V3> &q_Pd, vector<V3> &q_H,
                                 vector<double> &sigma_Pd, vector<double> &sigma_H, double &free_entropy) {
    if (!ctx_) return A2C_ERR_STATE;
    a2c_status s = a2c_gpp_set_occupancy(ctx_, x0.data());
    if (s) return last_status = s;
    vector<double> X;
    detail::pack(q_Pd0, q_H0, sigma_Pd0, sigma_H0, X);
    int nfev = 0;
    double gnorm = 0.0;
    s = a2c_gpp_minimize(ctx_, X.data(), &lbfgs, &free_entropy, &last_iters, &nfev, &gnorm, &last_reason);
    if (s) return last_status = s;
    if (last_reason <= 0) std::fprintf(stdout, "  WARNING: the minimizer did not converge!\n");  // minimizer.cpp:578-580
    q_Pd.resize(q_Pd0.size());
    q_H.resize(q_H0.size());
    sigma_Pd.resize(sigma_Pd0.size());
    sigma_H.resize(sigma_H0.size());
    detail::unpack(X, q_Pd, q_H, sigma_Pd, sigma_H);
    return last_status = A2C_OK;
  }

  // minimizer.cpp:588-802, at the context's current state.
  a2c_status calculateChemicalPotential(vector<double> &x0, double gammabd, vector<double> &gamma,
                                        vector<int> &full_H) {
    if (!ctx_) return A2C_ERR_STATE;
    a2c_status s = a2c_gpp_set_occupancy(ctx_, x0.data());
    if (!s) s = a2c_gpp_chem_potential(ctx_, gammabd, gamma.data(), full_H.data());
    return last_status = s;
  }

  // minimizer.cpp:833-1144: the lists at rc from the current state (the
  // _ext superset lists are not needed by the cell-list build).
  a2c_status findLocalNeighbors(vector<vector<int> > &, vector<vector<int> > &, vector<vector<int> > &,
                                vector<vector<int> > &, vector<vector<int> > &PdPd, vector<vector<int> > &PdH,
                                vector<vector<int> > &HPd, vector<vector<int> > &HH, vector<vector<int> > &PdPdnum,
                                vector<vector<int> > &HH1, int &maxNeib) {
    if (!ctx_) return A2C_ERR_STATE;
    vector<double> X(4 * (size_t)(nPd_ + nH_));
    a2c_status s = a2c_gpp_get_state(ctx_, X.data());
    if (!s) s = a2c_gpp_build_neighbors(ctx_, X.data(), &maxNeib);
    if (!s) s = detail::from_ctx(ctx_, A2C_LIST_PDPD, nPd_, PdPd);
    if (!s) s = detail::from_ctx(ctx_, A2C_LIST_PDH, nPd_, PdH);
    if (!s) s = detail::from_ctx(ctx_, A2C_LIST_HPD, nH_, HPd);
    if (!s) s = detail::from_ctx(ctx_, A2C_LIST_HH, nH_, HH);
    if (!s) s = detail::from_ctx(ctx_, A2C_LIST_HH1, nH_, HH1);
    if (!s) {
      vector<int> sh(3 * (size_t)(nPd_ > 0 ? nPd_ : 1));
      s = a2c_gpp_get_shell_counts(ctx_, sh.data());
      PdPdnum.assign(nPd_, vector<int>(3, 0));
      for (int i = 0; i < nPd_ && !s; ++i)
        for (int k = 0; k < 3; ++k) PdPdnum[i][k] = sh[3 * i + k];
    }
    return last_status = s;
  }

 private:
  a2c_gpp_ctx *ctx_ = nullptr;
  int nPd_ = 0, nH_ = 0;
};

// neighbors.cpp:8-115: all pairs within rc, self excluded, built on the GPU
// (device 0); returns maxNeib, or -status on failure.
template <class V3>
inline int findNeighbors(double a_Pd, double rc, vector<V3> &q_Pd0, vector<V3> &q_H0, vector<vector<int> > &PdPd,
                         vector<vector<int> > &PdH, vector<vector<int> > &HPd, vector<vector<int> > &HH) {
  a2c_gpp_params p;
  a2c_gpp_default_params(&p);
  p.nPd = (int)q_Pd0.size();
  p.nH = (int)q_H0.size();
  p.rc = rc;
  p.a_Pd = a_Pd;
  a2c_gpp_ctx *ctx = nullptr;
  a2c_status s = a2c_gpp_create(&p, &ctx);
  if (s) return -(int)s;
  vector<double> X;
  vector<double> sPd(q_Pd0.size(), 1.0), sH(q_H0.size(), 1.0);
  detail::pack(q_Pd0, q_H0, sPd, sH, X);
  int maxNeib = 0;
  s = a2c_gpp_build_neighbors(ctx, X.data(), &maxNeib);
  if (!s) s = detail::from_ctx(ctx, A2C_LIST_PDPD, q_Pd0.size(), PdPd);
  if (!s) s = detail::from_ctx(ctx, A2C_LIST_PDH, q_Pd0.size(), PdH);
  if (!s) s = detail::from_ctx(ctx, A2C_LIST_HPD, q_H0.size(), HPd);
  if (!s) s = detail::from_ctx(ctx, A2C_LIST_HH, q_H0.size(), HH);
  a2c_gpp_destroy(ctx);
  return s ? -(int)s : maxNeib;
}

// integrate.cpp:9-87 on the GPU (device 0).
template <class Input>
inline int integrateDiffusion(Input &input, double dt, vector<vector<int> > &HH1, vector<double> &gamma,
                              vector<double> &x0, vector<double> &x, vector<int> &full_H) {
  vector<int64_t> off;
  vector<int> idx;
  detail::to_csr(HH1, off, idx);
  if (idx.empty()) idx.push_back(0);
  return (int)a2c_diffuse_lists(0, (int)x0.size(), off.data(), idx.data(), x0.data(), gamma.data(), full_H.data(),
                                input.file.T0, dt, input.file.v, input.file.Qm, input.file.xLb, input.file.xUb,
                                x.data());
}

// boundaryconditions.cpp:30-55: bookkeeping on the caller's arrays (the
// device-resident loop applies the same condition with a2c_gpp_apply_dirichlet).
template <class Input, class V3>
inline int enforceBoundaryConditions(Input &input, double, vector<V3> &, vector<V3> &, vector<double> &,
                                     vector<double> &, vector<double> &x0, vector<double> &gamma,
                                     vector<int> &HSubsurf, double &gammabd, vector<int> &full_H) {
  for (size_t t = 0; t < HSubsurf.size(); ++t) {
    const int i = HSubsurf[t];
    if (i < 0 || (size_t)i >= x0.size()) return (int)A2C_ERR_INVALID;
    gamma[i] = gammabd;
    full_H[i] = 1;
    x0[i] = input.file.xUb;
  }
  return 0;
}

// calculateresults.cpp:8-78 on the GPU (a context of the right size).
template <class V3>
inline int calculateMacroResults(a2c_gpp_ctx *ctx, vector<vector<int> > &, vector<vector<int> > &, vector<V3> &,
                                 vector<double> &x, vector<int> &, vector<int> &HSurf, double &xH,
                                 double &xHinterior) {
  return (int)a2c_gpp_macro_results(ctx, x.data(), HSurf.empty() ? nullptr : HSurf.data(), (int)HSurf.size(), &xH,
                                    &xHinterior);
}

// readresults.cpp:10-55 (reads <foldername>/<filename_base>.<restart_file_num>.dat).
template <class Input, class V3>
inline int readResults(Input &input, vector<V3> &q_Pd0, vector<V3> &q_H0, vector<double> &sigma_Pd0,
                       vector<double> &sigma_H0, vector<double> &x0, vector<double> &gamma, vector<int> &full_H) {
  char path[1024];
  std::snprintf(path, sizeof(path), "%s/%s.%d.dat", input.file.foldername, input.file.filename_base,
                input.file.restart_file_num);
  const int nPd = (int)q_Pd0.size(), nH = (int)q_H0.size();
  vector<double> X(4 * (size_t)(nPd + nH));
  const a2c_status s = a2c_restart_read(path, nPd, nH, input.file.xLb, input.file.xUb, X.data(), x0.data(),
                                        gamma.data(), full_H.data());
  if (s) return (int)s;
  detail::unpack(X, q_Pd0, q_H0, sigma_Pd0, sigma_H0);
  return 0;
}

// The writer of that format (not in the reference tree).
template <class Input, class V3>
inline int writeResults(Input &input, int file_num, vector<V3> &q_Pd, vector<V3> &q_H, vector<double> &sigma_Pd,
                        vector<double> &sigma_H, vector<double> &x, vector<double> &gamma, vector<int> &full_H,
                        double time = 0.0) {
  char path[1024];
  std::snprintf(path, sizeof(path), "%s/%s.%d.dat", input.file.foldername, input.file.filename_base, file_num);
  vector<double> X;
  detail::pack(q_Pd, q_H, sigma_Pd, sigma_H, X);
  return (int)a2c_restart_write(path, (int)q_Pd.size(), (int)q_H.size(), X.data(), x.data(), gamma.data(),
                                full_H.data(), file_num, time);
}

// The sites of one lattice (the LatticeVariables fields the set-up fills).
struct LatticeSites {
  vector<double> q, q0, l;  // 3 per site
  vector<int> siteid, matid, tag;
  vector<double> sigma, x;
  int64_t size() const { return (int64_t)siteid.size(); }
};

namespace detail {
inline a2c_lattice_sites view(LatticeSites &s, int64_t n) {
  a2c_lattice_sites v{};
  v.capacity = v.count = n;
  v.q = s.q.data();
  v.q0 = s.q0.data();
  v.l = s.l.data();
  v.siteid = s.siteid.data();
  v.matid = s.matid.data();
  v.tag = s.tag.data();
  v.sigma = s.sigma.data();
  v.x = s.x.data();
  return v;
}
inline void keep_only(LatticeSites &s, const vector<unsigned char> &keep) {
  int64_t w = 0;
  for (int64_t i = 0; i < s.size(); ++i) {
    if (!keep[(size_t)i]) continue;
    for (int k = 0; k < 3; ++k) {
      s.q[3 * w + k] = s.q[3 * i + k];
      s.q0[3 * w + k] = s.q0[3 * i + k];
      s.l[3 * w + k] = s.l[3 * i + k];
    }
    s.siteid[w] = s.siteid[i];
    s.matid[w] = s.matid[i];
    s.tag[w] = s.tag[i];
    s.sigma[w] = s.sigma[i];
    s.x[w] = s.x[i];
    ++w;
  }
  s.q.resize(3 * w);
  s.q0.resize(3 * w);
  s.l.resize(3 * w);
  s.siteid.resize(w);
  s.matid.resize(w);
  s.tag.resize(w);
  s.sigma.resize(w);
  s.x.resize(w);
}
}  // namespace detail

// SpaceInitializer::SetupLatticeVariables (SpaceInitializer.cpp:41-116) for
// Lattice[0 .. n_lattices-1] and the RegionalInitialCondition blocks of an
// input file: every lattice built, the regions applied in index order,
// then the MinDistance removals in the reference's order.  errmsg (may be
// null) receives the reader's or builder's message.
inline int SetupLatticeVariables(const char *input_file, int n_lattices, vector<LatticeSites> &LVS,
                                 char *errmsg = nullptr, int errlen = 0) {
  const int kMax = 1024;
  LVS.assign((size_t)std::max(n_lattices, 0), LatticeSites());
  vector<double> dmin((size_t)std::max(n_lattices, 0));
  for (int k = 0; k < n_lattices; ++k) {
    a2c_lattice_desc d;
    vector<a2c_site_group> sg(kMax);
    vector<a2c_geometry> geo(kMax);
    a2c_status s = a2c_input_lattice(input_file, k, &d, sg.data(), kMax, geo.data(), kMax, errmsg, errlen);
    if (s) return (int)s;
    a2c_lattice_sites cnt{};
    if ((s = a2c_lattice_build(&d, &cnt, errmsg, errlen))) return (int)s;
    LatticeSites &L = LVS[(size_t)k];
    const int64_t n = cnt.count;
    L.q.resize(3 * n);
    L.q0.resize(3 * n);
    L.l.resize(3 * n);
    L.siteid.resize(n);
    L.matid.resize(n);
    L.tag.resize(n);
    L.sigma.resize(n);
    L.x.resize(n);
    a2c_lattice_sites v = detail::view(L, n);
    if (n > 0 && (s = a2c_lattice_build(&d, &v, errmsg, errlen))) return (int)s;
    double m = d.dmin;
    if (m <= 0.0) {  // LatticeStructure.cpp:56-58: the shortest lattice vector
      m = -1.0;
      for (int i = 0; i < 3; ++i) {
        const double *a = d.abc + 3 * i;
        const double len = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        m = (m < 0.0 || len < m) ? len : m;
      }
    }
    dmin[(size_t)k] = m;
  }
  vector<a2c_region> reg(kMax);
  vector<a2c_geometry> rgeo(kMax);
  int nreg = 0;
  a2c_status s = a2c_input_regions(input_file, reg.data(), kMax, rgeo.data(), kMax, &nreg, errmsg, errlen);
  if (s) return (int)s;
  for (int r = 0; r < nreg; ++r) {
    if (reg[(size_t)r].lattice_id >= n_lattices) return (int)A2C_ERR_INVALID;
    for (int k = 0; k < n_lattices; ++k) {
      if (reg[(size_t)r].lattice_id >= 0 && reg[(size_t)r].lattice_id != k) continue;
      a2c_lattice_sites v = detail::view(LVS[(size_t)k], LVS[(size_t)k].size());
      if ((s = a2c_lattice_apply_region(&reg[(size_t)r], &v, errmsg, errlen))) return (int)s;
    }
  }
  for (int i = 0; i < n_lattices; ++i)
    for (int j = 0; j < n_lattices; ++j) {
      if (j == i || (j < i && dmin[(size_t)j] <= dmin[(size_t)i])) continue;  // already resolved
      LatticeSites &A = LVS[(size_t)i];
      const LatticeSites &B = LVS[(size_t)j];
      vector<unsigned char> keep((size_t)std::max<int64_t>(A.size(), 1));
      int64_t removed = 0;
      if ((s = a2c_lattice_conflicts(A.q.data(), A.size(), B.q.data(), B.size(), dmin[(size_t)i], keep.data(),
                                     &removed)))
        return (int)s;
      if (removed) detail::keep_only(A, keep);
    }
  return 0;
}

}  // namespace a2c_gb300
