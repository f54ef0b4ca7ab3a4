// Host construction of the FP32 tables of the mixed-precision form.
//
// f_Pd and phi_Pd are degree-17 / degree-8 polynomials in r/5 whose terms
// cancel by up to four orders of magnitude (potential.cpp:84-91, 145), so
// they cannot be evaluated in FP32 directly (errors reach 1e-3..1e+1
// relative).  They are tabulated here as piecewise cubic Hermite
// interpolants on a uniform grid: values and exact first derivatives are
// computed in FP64 by forward-mode differentiation (dual numbers) of the
// reference's formulas, and the cubic's coefficients are rounded to FP32.
// The caller picks the grid; the mixed kernels use r in [1, 7) A with
// h = 1/160 A, so the branch points 5.0 (f_Pd tail) and 5.05 (phi_Pd tail)
// are knots and each interval lies in one branch.
// The embedding functions F_Pd(rho), F_H(rho) (per site) are tabulated the
// same way on rho in [0, 64), h = 1/64.
#include <cmath>
#include <cstdint>
#include <vector>

namespace a2c {
namespace tables {

struct Dual {
  double v, d;
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
inline Dual operator-(Dual a, double b) { return {a.v - b, a.d}; }
inline Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
inline Dual operator*(double b, Dual a) { return {a.v * b, a.d * b}; }
inline Dual dexp(Dual a) {
  const double e = std::exp(a.v);
  return {e, e * a.d};
}
inline Dual dpow(Dual u, double y) { return {std::pow(u.v, y), y * std::pow(u.v, y - 1.0) * u.d}; }

// potential.cpp:64-98; `branch` is the radius that selects the branch
Dual f_Pd(Dual r, double branch) {
  const double a[7][2] = {{2.7267629107325706, 1.8716766113599643}, {2.50290548851635, 1.668549182690922},
                          {2.0924467509943674, 1.3150372774478005}, {1.564328475106985, 0.8987511149780485},
                          {1.009780903403673, 0.5124363774128722},  {0.5304054524800665, 0.2169886022464641},
                          {0.1356566408715063, 0.035852347523891395}};
  if (branch > 5.0) return 0.001510569378297 * dexp((-0.077976566126292 / 0.001510569378297) * (r - 5.0));
  const Dual z = r * 0.2;
  Dual ra = z;
  for (int m = 0; m < 7; ++m) ra = ra * (z * (z - a[m][0]) + a[m][1]);
  return z * (z * (z * (ra * -2.597301181336601e7 + 14673.409149169922) + -255.8965835571289) + 0.6676807403564453) +
         -0.02972698211669922;
}

// potential.cpp:126-155
Dual phi_Pd(Dual r, double branch) {
  if (branch > 5.05) return -0.016958780164980 * dexp((0.089019679316328 / -0.016958780164980) * (r - 5.05));
  const double b[4][2] = {{2.0586473420376348, 1.0683922574015199}, {1.6696359816422877, 0.7337878627470482},
                          {1.1690370066230809, 0.3909805777737639}, {0.2635598721249787, 0.033551116514910245}};
  const Dual z = r * 0.2;
  Dual y = (z - 1.0699996145674568) * -79415.24035137112;
  y = y * (z - 1.06015072612581);
  y = y * (z - 0.42433991011376526);
  y = y * (z + 0.06169160085238687);
  for (int m = 0; m < 4; ++m) y = y * (z * (z - b[m][0]) + b[m][1]);
  return y + (2 * 0.251546) * f_Pd(r, branch);
}

// potential.cpp:16-38
Dual F_Pd(Dual rho) {
  const double b[5][2] = {{2.4242616904962846, 1.4791899886249564}, {2.1376274623740064, 1.2169215689822592},
                          {1.6486007989726832, 0.8159825255339774}, {1.0749204110338482, 0.42007491336688396},
                          {0.5128056047933808, 0.12468685331167456}};
  const Dual z = rho * 0.02;
  Dual y = (z - 0.20581955357385892) * 295878.9003038662;
  y = y * (z - 0.081228755904399);
  y = y * z;
  y = y * (z + 0.05298811034615951);
  for (int m = 0; m < 5; ++m) y = y * (z * (z - b[m][0]) + b[m][1]);
  return y - (50.0 * 0.251546) * z;
}

// potential.cpp:45-57
Dual F_H(Dual rho) {
  const double c = 0.000197047, d = 1.18860, a = 9.99780, b = 60.0155, eps1 = 0.0540638;
  const Dual u = rho + eps1;
  Dual y = dpow(u, 2.0 + d) * (1.0 / (2.0 + d)) - dpow(u, 1.0 + d) * ((a + b) / (1.0 + d)) + dpow(u, d) * (a * b / d);
  return y * -c - rho * -0.0296604;
}

// cubic Hermite coefficients of [x0, x0+h] in t = (x - x0)/h
void hermite(Dual p0, Dual p1, double h, float *c) {
  const double c0 = p0.v, c1 = h * p0.d;
  const double c2 = 3.0 * (p1.v - p0.v) - h * (2.0 * p0.d + p1.d);
  const double c3 = 2.0 * (p0.v - p1.v) + h * (p0.d + p1.d);
  c[0] = (float)c0;
  c[1] = (float)c1;
  c[2] = (float)c2;
  c[3] = (float)c3;
}

}  // namespace tables

// Pair table: per interval 8 floats, f_Pd's cubic then phi_Pd's cubic.
void build_pair_table(double r0, double h, int n, std::vector<float> &out) {
  out.assign((size_t)n * 8, 0.0f);
  for (int i = 0; i < n; ++i) {
    const double xa = r0 + h * i, xb = r0 + h * (i + 1), mid = r0 + h * (i + 0.5);
    tables::hermite(tables::f_Pd({xa, 1.0}, mid), tables::f_Pd({xb, 1.0}, mid), h, &out[(size_t)8 * i]);
    tables::hermite(tables::phi_Pd({xa, 1.0}, mid), tables::phi_Pd({xb, 1.0}, mid), h, &out[(size_t)8 * i + 4]);
  }
}

// Embedding tables: per interval 4 floats; species 0 = Pd, 1 = H.
void build_embed_table(int species, double h, int n, std::vector<float> &out) {
  out.assign((size_t)n * 4, 0.0f);
  for (int i = 0; i < n; ++i) {
    const tables::Dual a = {h * i, 1.0}, b = {h * (i + 1), 1.0};
    if (species == 0)
      tables::hermite(tables::F_Pd(a), tables::F_Pd(b), h, &out[(size_t)4 * i]);
    else
      tables::hermite(tables::F_H(a), tables::F_H(b), h, &out[(size_t)4 * i]);
  }
}

}  // namespace a2c

namespace a2c {

// The same tables written into caller-provided arrays (8n and 4n floats),
// with no heap allocation.
void build_pair_table_raw(double r0, double h, int n, float *out) {
  for (int i = 0; i < n; ++i) {
    const double xa = r0 + h * i, xb = r0 + h * (i + 1), mid = r0 + h * (i + 0.5);
    tables::hermite(tables::f_Pd({xa, 1.0}, mid), tables::f_Pd({xb, 1.0}, mid), h, &out[(size_t)8 * i]);
    tables::hermite(tables::phi_Pd({xa, 1.0}, mid), tables::phi_Pd({xb, 1.0}, mid), h, &out[(size_t)8 * i + 4]);
  }
}

void build_embed_table_raw(int species, double h, int n, float *out) {
  for (int i = 0; i < n; ++i) {
    const tables::Dual a = {h * i, 1.0}, b = {h * (i + 1), 1.0};
    if (species == 0)
      tables::hermite(tables::F_Pd(a), tables::F_Pd(b), h, &out[(size_t)4 * i]);
    else
      tables::hermite(tables::F_H(a), tables::F_H(b), h, &out[(size_t)4 * i]);
  }
}

}  // namespace a2c
