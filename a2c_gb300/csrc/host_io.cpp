// Restart I/O in the format the reference's readResults reads
// (readresults.cpp:10-55): nine header lines, then per site nine
// whitespace-separated columns, all Pd sites first.  The reference tree has
// no writer; the column meaning follows its reader (qx qy qz sigma in
// columns 3-6; x gamma full_H in 7-9 for H sites).
#include <cmath>
#include <cstdio>
#include <fstream>
#include <limits>
#include <string>

#include "a2c_gpp.h"

extern "C" a2c_status a2c_restart_write(const char *path, int nPd, int nH, const double *X, const double *xH,
                                        const double *gamma, const int *full_H, int step, double time) {
  if (!path || nPd < 0 || nH < 0 || (nPd + nH > 0 && !X) || (nH > 0 && (!xH || !gamma || !full_H)))
    return A2C_ERR_INVALID;
  FILE *f = std::fopen(path, "w");
  if (!f) return A2C_ERR_INVALID;
  std::fprintf(f, "# a2c_gb300 restart\n# step %d\n# time %.17g\n# nPd %d\n# nH %d\n", step, time, nPd, nH);
  std::fprintf(f, "# columns: id species(0 Pd, 1 H) qx qy qz sigma x gamma full_H\n");
  std::fprintf(f, "# Pd rows first, then H rows\n# values printed with 17 significant digits\n# ----\n");
  for (int i = 0; i < nPd; ++i)
    std::fprintf(f, "%d 0 %.17g %.17g %.17g %.17g 1 0 0\n", i, X[4 * i], X[4 * i + 1], X[4 * i + 2], X[4 * i + 3]);
  for (int h = 0; h < nH; ++h) {
    const long s = (long)nPd + h;
    std::fprintf(f, "%d 1 %.17g %.17g %.17g %.17g %.17g %.17g %d\n", h, X[4 * s], X[4 * s + 1], X[4 * s + 2],
                 X[4 * s + 3], xH[h], gamma[h], full_H[h]);
  }
  const bool ok = std::ferror(f) == 0;
  std::fclose(f);
  return ok ? A2C_OK : A2C_ERR_INVALID;
}

extern "C" a2c_status a2c_restart_read(const char *path, int nPd, int nH, double xLb, double xUb, double *X,
                                       double *xH, double *gamma, int *full_H) {
  if (!path || nPd < 0 || nH < 0 || (nPd + nH > 0 && !X) || (nH > 0 && (!xH || !gamma || !full_H)))
    return A2C_ERR_INVALID;
  std::ifstream in(path);
  if (!in) return A2C_ERR_INVALID;
  for (int k = 0; k < 9; ++k) in.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
  double skip;
  for (int i = 0; i < nPd; ++i)
    in >> skip >> skip >> X[4 * i] >> X[4 * i + 1] >> X[4 * i + 2] >> X[4 * i + 3] >> skip >> skip >> skip;
  for (int h = 0; h < nH; ++h) {
    const long s = (long)nPd + h;
    in >> skip >> skip >> X[4 * s] >> X[4 * s + 1] >> X[4 * s + 2] >> X[4 * s + 3] >> xH[h] >> gamma[h] >> full_H[h];
  }
  if (!in) return A2C_ERR_INVALID;
  for (int h = 0; h < nH; ++h) {  // readresults.cpp:48-51
    if (xH[h] < xLb) xH[h] = xLb;
    else if (xH[h] > xUb) xH[h] = xUb;
  }
  return A2C_OK;
}
