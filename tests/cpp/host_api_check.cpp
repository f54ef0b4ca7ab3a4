// Drives the reference-named C++ host API (include/a2c_host.hpp) through one
// DMD outer step on a small periodic lattice and prints the results as JSON,
// for tests/test_host_api.py.  The Vec3D and Input types here are minimal
// stand-ins with the reference's member names.
#include <cmath>
#include <cstdio>
#include <vector>

#include "a2c_host.hpp"

struct Vec3 {
  double v[3] = {0.0, 0.0, 0.0};
  double &operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};
struct InputFile {
  double eps = 1.0e-5, rc = 5.35, T0 = 300.0, dt = 1e-12, a_Pd = 3.89, xUb = 1.0 - 1.0e-16, xLb = 1.0e-3;
  double v = 1.0e13, Qm = 0.23;
  char foldername[256] = ".";
  char filename_base[256] = "host_api_check";
  int restart_file_num = 0;
};
struct Input {
  InputFile file;
};

int main(int argc, char **argv) {
  using namespace a2c_gb300;
  const int cells = 4;
  a2c_lattice_spec sp = {};
  sp.ncell[0] = sp.ncell[1] = sp.ncell[2] = cells;
  sp.a = 3.89;
  sp.periodic[0] = sp.periodic[1] = 1;
  sp.pos_std = 0.02;
  sp.sigma_lo = sp.sigma_hi = 0.1;
  sp.x_center = 0.05;
  sp.x_half = 0.01;
  sp.xLb = 1e-3;
  sp.xUb = 1.0 - 1e-16;
  sp.seed = 11;
  const int nPd = 4 * cells * cells * cells, nH = nPd, N = nPd + nH;
  std::vector<double> X(4 * (size_t)N), xH(nH);
  std::vector<int> surf(nH);
  if (a2c_lattice_fcc(&sp, X.data(), xH.data(), surf.data())) return 2;
  std::vector<Vec3> qPd(nPd), qH(nH), qPd1, qH1;
  std::vector<double> sPd(nPd), sH(nH), sPd1, sH1;
  for (int i = 0; i < N; ++i) {
    Vec3 &q = i < nPd ? qPd[i] : qH[i - nPd];
    for (int d = 0; d < 3; ++d) q[d] = X[4 * i + d];
    (i < nPd ? sPd[i] : sH[i - nPd]) = X[4 * i + 3];
  }
  Input input;
  if (argc > 1) std::snprintf(input.file.foldername, sizeof(input.file.foldername), "%s", argv[1]);
  std::vector<std::vector<int> > PdPd, PdH, HPd, HH, PdPdnum, HH1;
  // the box is periodic in x and y: the context needs it before the lists
  Minimizer mz;
  mz.params.periodic[0] = mz.params.periodic[1] = 1;
  mz.params.box[0] = mz.params.box[1] = cells * 3.89;
  mz.lbfgs.gatol = 1e-6;
  // the reference's neighbor routine would see no images; build the lists
  // through the context (minimum image), then hand them to initialize
  std::vector<std::vector<int> > e0(nPd), e1(nPd), e2(nH), e3(nH);  // empty lists to start the context
  std::vector<std::vector<Vec3> > QPp(12, std::vector<Vec3>(2));
  double QWp = 1.0 / 12.0;
  std::vector<double> coe(4, 0.0);
  int st = mz.initialize(&input, &e0, &e1, &e2, &e3, qPd, qH, sPd, sH, xH, &QPp, QWp, &coe, &coe);
  if (!st) {
    int maxNeib = 0;
    st = mz.findLocalNeighbors(e0, e1, e2, e3, PdPd, PdH, HPd, HH, PdPdnum, HH1, maxNeib);
  }
  if (!st) st = mz.initialize(&input, &PdPd, &PdH, &HPd, &HH, qPd, qH, sPd, sH, xH, &QPp, QWp, &coe, &coe, &HH1);
  double f0 = 0.0, fmin = 0.0;
  std::vector<double> G(4 * (size_t)N);
  if (!st) st = a2c_gpp_eval(mz.context(), X.data(), &f0, G.data());
  if (!st) st = mz.minimizeFreeEntropy(1e-12, qPd, qH, sPd, sH, xH, qPd1, qH1, sPd1, sH1, fmin);
  std::vector<double> gamma(nH, 0.0), x(xH);
  std::vector<int> full(nH, 0), bd;
  for (int h = 0; h < nH; ++h)
    if (surf[h]) bd.push_back(h);
  double gbd = 2.0, xm = 0.0, xi = 0.0;
  if (!st) st = mz.calculateChemicalPotential(xH, gbd, gamma, full);
  if (!st) st = enforceBoundaryConditions(input, 1e-12, qPd1, qH1, sPd1, sH1, xH, gamma, bd, gbd, full);
  if (!st) st = integrateDiffusion(input, 1e-12, HH1, gamma, xH, x, full);
  if (!st) st = calculateMacroResults(mz.context(), PdPd, PdPdnum, qPd1, x, bd, bd, xm, xi);
  std::vector<Vec3> qPd2(nPd), qH2(nH);
  std::vector<double> sPd2(nPd), sH2(nH), x2(nH), g2(nH);
  std::vector<int> full2(nH);
  if (!st) st = writeResults(input, 7, qPd1, qH1, sPd1, sH1, x, gamma, full);
  input.file.restart_file_num = 7;
  if (!st) st = readResults(input, qPd2, qH2, sPd2, sH2, x2, g2, full2);
  bool same = !st;
  for (int i = 0; i < nPd && same; ++i) same = qPd2[i][0] == qPd1[i][0] && sPd2[i] == sPd1[i];
  for (int h = 0; h < nH && same; ++h) same = x2[h] == std::fmax(x[h], 1e-3) && g2[h] == gamma[h];
  std::printf("{\"status\": %d, \"f0\": %.17g, \"fmin\": %.17g, \"iters\": %d, \"reason\": %d, \"xH_mean\": %.17g, "
              "\"xH_interior\": %.17g, \"n_pdpd\": %zu, \"restart_round_trip\": %s, \"gamma0\": %.17g}\n",
              st, f0, fmin, mz.last_iters, mz.last_reason, xm, xi, PdPd.empty() ? 0 : PdPd[0].size(),
              same ? "true" : "false", gamma.empty() ? 0.0 : gamma[0]);
  return st ? 1 : 0;
}
