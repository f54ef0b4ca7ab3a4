// Harness around the reference's own hot-path sources -- TEST INFRASTRUCTURE.
//
// oracle/Makefile (target `ref`) compiles this file together with the
// reference's potential.cpp, electrondensity.cpp, quadrature.cpp,
// neighbors.cpp, minimizer.cpp, integrate.cpp, boundaryconditions.cpp,
// calculateresults.cpp and readresults.cpp (unmodified, read where they lie)
// against the
// single-rank shims in oracle/ref_shim, producing oracle/_ref/liba2c_ref.so.
// The tests use it to pin the oracle restatement bit for bit.  It is built
// only where the reference tree is present and is never shipped.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "Vector3D.h"
#include "input.h"
#include "minimizer.h"
#include "potential.h"

using std::vector;

Tao shim_last_tao = nullptr;

extern double eps;  // potential.cpp:13
int findNeighbors(double a_Pd, double rc, vector<Vec3D> &q_Pd0, vector<Vec3D> &q_H0, vector<vector<int> > &PdPd,
                  vector<vector<int> > &PdH, vector<vector<int> > &HPd, vector<vector<int> > &HH);
void gaussianQuadrature(int dim, vector<vector<Vec3D> > &QP);
double electronDensity(char atype, int n, double rc, vector<vector<int> > &PdPd, vector<vector<int> > &PdH,
                       vector<vector<int> > &HPd, vector<vector<int> > &HH, vector<Vec3D> &q_Pd,
                       vector<Vec3D> &q_H, vector<double> &sigma_Pd, vector<double> &sigma_H, vector<double> &x,
                       vector<vector<Vec3D> > &QPp, double &QWp);
int integrateDiffusion(Input &input, double dt, vector<vector<int> > &HH1, vector<double> &gamma,
                       vector<double> &x0, vector<double> &x, vector<int> &full_H);
int enforceBoundaryConditions(Input &input, double dt, vector<Vec3D> &q_Pd0, vector<Vec3D> &q_H0,
                              vector<double> &sigma_Pd0, vector<double> &sigma_H0, vector<double> &x0,
                              vector<double> &gamma, vector<int> &HSubsurf, double &gammabd, vector<int> &full_H);
int calculateMacroResults(vector<vector<int> > &PdPd, vector<vector<int> > &PdPdnum, vector<Vec3D> &q_Pd,
                          vector<double> &x, vector<int> &PdSurf, vector<int> &HSurf, double &xH,
                          double &xHinterior);
void readResults(Input &input, vector<Vec3D> &q_Pd0, vector<Vec3D> &q_H0, vector<double> &sigma_Pd0,
                 vector<double> &sigma_H0, vector<double> &x0, vector<double> &gamma, vector<int> &full_H);

namespace {

const uint32_t ID_MASK = (1u << 27) - 1u;

struct State {
  vector<Vec3D> qPd, qH;
  vector<double> sPd, sH, x0;
};

State unpack(int nPd, int nH, const double *X, const double *xH) {
  State s;
  for (int i = 0; i < nPd; ++i) {
    s.qPd.push_back(Vec3D(X[4 * i], X[4 * i + 1], X[4 * i + 2]));
    s.sPd.push_back(X[4 * i + 3]);
  }
  for (int i = 0; i < nH; ++i) {
    const int64_t t = (int64_t)nPd + i;
    s.qH.push_back(Vec3D(X[4 * t], X[4 * t + 1], X[4 * t + 2]));
    s.sH.push_back(X[4 * t + 3]);
    s.x0.push_back(xH ? xH[i] : 0.0);
  }
  return s;
}

// combined per-site list (global ids, Pd first) -> the reference's four lists
void split_lists(int nPd, int nH, const int64_t *off, const uint32_t *nbr, vector<vector<int> > &PdPd,
                 vector<vector<int> > &PdH, vector<vector<int> > &HPd, vector<vector<int> > &HH) {
  PdPd.assign(nPd, {});
  PdH.assign(nPd, {});
  HPd.assign(nH, {});
  HH.assign(nH, {});
  for (int64_t s = 0; s < (int64_t)nPd + nH; ++s)
    for (int64_t t = off[s]; t < off[s + 1]; ++t) {
      const int64_t j = nbr[t] & ID_MASK;
      const bool jPd = j < nPd;
      if (s < nPd) (jPd ? PdPd[s] : PdH[s]).push_back(jPd ? (int)j : (int)(j - nPd));
      else (jPd ? HPd[s - nPd] : HH[s - nPd]).push_back(jPd ? (int)j : (int)(j - nPd));
    }
}

struct Setup {
  Input input;
  vector<vector<int> > PdPd, PdH, HPd, HH;
  vector<vector<Vec3D> > QPp;
  double QWp;
  vector<double> coe_Pd, coe_H;
  State st;
  Minimizer *mz = nullptr;
  int argc = 1;
  char *argv0 = (char *)"ref";
  char **argv = &argv0;
};

Setup *make_setup(int nPd, int nH, double T, double QWp, double eps_, double rc, double a_Pd, const double *coe,
                  const double *X, const double *xH, const int64_t *off, const uint32_t *nbr) {
  Setup *S = new Setup;
  eps = eps_;
  S->input.file.T0 = T;
  S->input.file.rc = rc;
  S->input.file.a_Pd = a_Pd;
  S->input.file.eps = eps_;
  S->QWp = QWp;
  S->coe_Pd.assign(coe, coe + 4);
  S->coe_H.assign(coe + 4, coe + 8);
  gaussianQuadrature(6, S->QPp);
  S->st = unpack(nPd, nH, X, xH);
  if (off) split_lists(nPd, nH, off, nbr, S->PdPd, S->PdH, S->HPd, S->HH);
  S->mz = new Minimizer(&S->argc, &S->argv);
  S->mz->initialize(&S->input, &S->PdPd, &S->PdH, &S->HPd, &S->HH, S->st.qPd, S->st.qH, S->st.sPd, S->st.sH,
                    S->st.x0, &S->QPp, S->QWp, &S->coe_Pd, &S->coe_H);
  return S;
}

void free_setup(Setup *S) {
  delete S->mz;
  delete S;
}

// neighbor results kept between the run and the getters
vector<vector<int> > g_lists[7];  // PdPd, PdH, HPd, HH, HH1 (refiltered), PdPdnum, ext sizes
int g_maxneib[2];

}  // namespace

extern "C" {

void ref_eam(int which, const double *in, int64_t n, double eps_, double *out) {
  eps = eps_;
  EAM e;
  for (int64_t t = 0; t < n; ++t) {
    const double v = in[t];
    double r = 0.0;
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
    }
    out[t] = r;
  }
}

// Reference objective and gradient: Minimizer::formFunctionAndGradient.
int ref_eval(int nPd, int nH, double T, double QWp, double eps_, double rc, double a_Pd, const double *coe,
             const double *X, const double *xH, const int64_t *off, const uint32_t *nbr, double *f, double *G,
             double *rho) {
  Setup *S = make_setup(nPd, nH, T, QWp, eps_, rc, a_Pd, coe, X, xH, off, nbr);
  const int64_t n = 4 * ((int64_t)nPd + nH);
  Vec Xv, Gv;
  VecCreateMPI(0, (PetscInt)n, (PetscInt)n, &Xv);
  VecCreateMPI(0, (PetscInt)n, (PetscInt)n, &Gv);
  std::memcpy(Xv->a.data(), X, sizeof(double) * (size_t)n);
  PetscReal fv = 0.0;
  int e = shim_last_tao->objgrad(shim_last_tao, Xv, &fv, Gv, shim_last_tao->objctx);
  *f = fv;
  std::memcpy(G, Gv->a.data(), sizeof(double) * (size_t)n);
  if (rho) {
    AppCtx *app = (AppCtx *)shim_last_tao->objctx;
    for (int i = 0; i < nPd; ++i) rho[i] = app->recv_Pd[i];
    for (int i = 0; i < nH; ++i) rho[nPd + i] = app->recv_H[i];
  }
  VecDestroy(&Xv);
  VecDestroy(&Gv);
  free_setup(S);
  return e;
}

// Reference pass 1 for every site: electronDensity.
void ref_density(int nPd, int nH, double QWp, double eps_, double rc, const double *X, const double *xH,
                 const int64_t *off, const uint32_t *nbr, double *rho) {
  eps = eps_;
  vector<vector<int> > PdPd, PdH, HPd, HH;
  split_lists(nPd, nH, off, nbr, PdPd, PdH, HPd, HH);
  State st = unpack(nPd, nH, X, xH);
  vector<vector<Vec3D> > QPp;
  gaussianQuadrature(6, QPp);
  double W = QWp;
  for (int i = 0; i < nPd; ++i)
    rho[i] = electronDensity('P', i, rc, PdPd, PdH, HPd, HH, st.qPd, st.qH, st.sPd, st.sH, st.x0, QPp, W);
  for (int i = 0; i < nH; ++i)
    rho[nPd + i] = electronDensity('H', i, rc, PdPd, PdH, HPd, HH, st.qPd, st.qH, st.sPd, st.sH, st.x0, QPp, W);
}

// Reference chemical potential: Minimizer::calculateChemicalPotential.
int ref_chem_potential(int nPd, int nH, double T, double QWp, double eps_, double rc, double a_Pd,
                       const double *coe, const double *X, const double *xH, const int64_t *off,
                       const uint32_t *nbr, double gammabd, double *gamma, int *full_H) {
  Setup *S = make_setup(nPd, nH, T, QWp, eps_, rc, a_Pd, coe, X, xH, off, nbr);
  vector<double> x0(xH, xH + nH), g(gamma, gamma + nH);
  vector<int> fh(full_H, full_H + nH);
  int e = S->mz->calculateChemicalPotential(x0, gammabd, g, fh);
  for (int i = 0; i < nH; ++i) {
    gamma[i] = g[i];
    full_H[i] = fh[i];
  }
  free_setup(S);
  return e;
}

// Reference neighbor build: findNeighbors (global KD-tree) followed by
// Minimizer::findLocalNeighbors (refilter, Pd shells, first H shell).
int ref_neighbors_run(int nPd, int nH, double rc, double a_Pd, const double *X) {
  double coe[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  Setup *S = make_setup(nPd, nH, 300.0, 1.0 / 12, 1e-5, rc, a_Pd, coe, X, nullptr, nullptr, nullptr);
  vector<vector<int> > ePdPd, ePdH, eHPd, eHH;
  g_maxneib[0] = findNeighbors(a_Pd, rc, S->st.qPd, S->st.qH, ePdPd, ePdH, eHPd, eHH);
  for (int l = 0; l < 7; ++l) g_lists[l].clear();
  int e = S->mz->findLocalNeighbors(ePdPd, ePdH, eHPd, eHH, g_lists[0], g_lists[1], g_lists[2], g_lists[3],
                                    g_lists[5], g_lists[4], g_maxneib[1]);
  g_lists[6].assign(4, {});
  g_lists[6][0].push_back(0);
  free_setup(S);
  return e;
}

int64_t ref_neighbors_total(int list) {
  int64_t t = 0;
  for (auto &v : g_lists[list]) t += (int64_t)v.size();
  return t;
}

void ref_neighbors_get(int list, int64_t *off, int *idx) {
  int64_t w = 0;
  off[0] = 0;
  for (size_t i = 0; i < g_lists[list].size(); ++i) {
    for (int v : g_lists[list][i]) idx[w++] = v;
    off[i + 1] = w;
  }
}

int ref_neighbors_maxneib(int which) { return g_maxneib[which]; }

// Reference diffusion: integrateDiffusion.
int ref_diffuse(int nH, const double *x0, const int64_t *hh1_off, const int *hh1, const double *gamma,
                const int *full_H, double T, double dt, double v, double Qm, double xLb, double xUb, double *x) {
  Input in;
  in.file.T0 = T;
  in.file.v = v;
  in.file.Qm = Qm;
  in.file.xLb = xLb;
  in.file.xUb = xUb;
  vector<vector<int> > HH1((size_t)nH);
  for (int i = 0; i < nH; ++i)
    for (int64_t t = hh1_off[i]; t < hh1_off[i + 1]; ++t) HH1[(size_t)i].push_back(hh1[t]);
  vector<double> g(gamma, gamma + nH), xx0(x0, x0 + nH), xx(x, x + nH);
  vector<int> fh(full_H, full_H + nH);
  int e = integrateDiffusion(in, dt, HH1, g, xx0, xx, fh);
  for (int i = 0; i < nH; ++i) x[i] = xx[(size_t)i];
  return e;
}

// Reference Dirichlet condition: enforceBoundaryConditions.
int ref_dirichlet(int nH, const int *sites, int n, double gammabd, double xUb, double *x0, double *gamma,
                  int *full_H) {
  Input in;
  in.file.xUb = xUb;
  vector<Vec3D> q;
  vector<double> s;
  vector<double> xx0(x0, x0 + nH), g(gamma, gamma + nH);
  vector<int> fh(full_H, full_H + nH), sub(sites, sites + n);
  double gb = gammabd;
  int e = enforceBoundaryConditions(in, 0.0, q, q, s, s, xx0, g, sub, gb, fh);
  for (int i = 0; i < nH; ++i) {
    x0[i] = xx0[(size_t)i];
    gamma[i] = g[(size_t)i];
    full_H[i] = fh[(size_t)i];
  }
  return e;
}

// Reference macro results: calculateMacroResults.
int ref_macro_results(int nH, const double *x, const int *HSurf, int nSurf, double *xH, double *xHinterior) {
  vector<vector<int> > a, b;
  vector<Vec3D> q;
  vector<double> xx(x, x + nH);
  vector<int> ps, hs(HSurf, HSurf + nSurf);
  return calculateMacroResults(a, b, q, xx, ps, hs, *xH, *xHinterior);
}

// Reference restart reader: readResults (reads <folder>/<base>.<num>.dat).
int ref_read_results(const char *folder, const char *base, int num, int nPd, int nH, double xLb, double xUb,
                     double *X, double *xH, double *gamma, int *full_H) {
  Input in;
  std::snprintf(in.file.foldername, sizeof(in.file.foldername), "%s", folder);
  std::snprintf(in.file.filename_base, sizeof(in.file.filename_base), "%s", base);
  in.file.restart_file_num = num;
  in.file.xLb = xLb;
  in.file.xUb = xUb;
  vector<Vec3D> qPd(nPd), qH(nH);
  vector<double> sPd(nPd), sH(nH), x0(nH), g(nH);
  vector<int> fh(nH);
  readResults(in, qPd, qH, sPd, sH, x0, g, fh);
  for (int i = 0; i < nPd; ++i) {
    for (int d = 0; d < 3; ++d) X[4 * i + d] = qPd[i][d];
    X[4 * i + 3] = sPd[i];
  }
  for (int h = 0; h < nH; ++h) {
    for (int d = 0; d < 3; ++d) X[4 * (nPd + h) + d] = qH[h][d];
    X[4 * (nPd + h) + 3] = sH[h];
    xH[h] = x0[h];
    gamma[h] = g[h];
    full_H[h] = fh[h];
  }
  return 0;
}

}  // extern "C"
