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
#include <cstring>
#include <vector>

#include "tables.h"

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

// potential.cpp:105-119 (the tail beyond 5.35 A continues the exponential)
Dual f_H(Dual r) {
  if (r.v > 5.35) return 0.009986990526578 * dexp((-0.013075667086408 / 0.009986990526578) * (r - 5.35));
  return 11.0025 * dexp(-1.30927 * r);
}

// potential.cpp:162-177 and 185-200: D (b e^{-a (r - r0)} - a e^{-b (r - r0)}),
// exponential tail beyond 5.35 A
Dual morse(Dual r, double D, double a, double b, double r0, double fc, double fdc) {
  if (r.v > 5.35) return fc * dexp((fdc / fc) * (r - 5.35));
  return D * (b * dexp(-a * (r - r0)) - a * dexp(-b * (r - r0)));
}
Dual phi_PdH(Dual r) {
  return morse(r, 0.2494540, 4.82613, 2.13158, 1.50964, -3.353001113951400e-04, 7.147062196813336e-04);
}
Dual phi_H(Dual r) { return morse(r, 0.0661496, 3.67263, 1.47797, 2.51980, -0.003702722457147, 0.005465945471933); }

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

// The same cubic in the offset from the interval's midpoint, t' = t - 1/2
// in [-1/2, 1/2] (the form the pair kernels index without a float-to-int
// conversion).
void hermite_mid(Dual p0, Dual p1, double h, float *c) {
  const double c0 = p0.v, c1 = h * p0.d;
  const double c2 = 3.0 * (p1.v - p0.v) - h * (2.0 * p0.d + p1.d);
  const double c3 = 2.0 * (p0.v - p1.v) + h * (p0.d + p1.d);
  c[0] = (float)(c0 + 0.5 * c1 + 0.25 * c2 + 0.125 * c3);
  c[1] = (float)(c1 + c2 + 0.75 * c3);
  c[2] = (float)(c2 + 1.5 * c3);
  c[3] = (float)c3;
}

}  // namespace tables

// Pair table: per interval 8 floats, f_Pd's cubic then phi_Pd's cubic.
void build_pair_table(double r0, double h, int n, std::vector<float> &out) {
  out.assign((size_t)n * 8, 0.0f);
  for (int i = 0; i < n; ++i) {
    const double xa = r0 + h * i, xb = r0 + h * (i + 1), mid = r0 + h * (i + 0.5);
    tables::hermite_mid(tables::f_Pd({xa, 1.0}, mid), tables::f_Pd({xb, 1.0}, mid), h, &out[(size_t)8 * i]);
    tables::hermite_mid(tables::phi_Pd({xa, 1.0}, mid), tables::phi_Pd({xb, 1.0}, mid), h, &out[(size_t)8 * i + 4]);
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
    tables::hermite_mid(tables::f_Pd({xa, 1.0}, mid), tables::f_Pd({xb, 1.0}, mid), h, &out[(size_t)8 * i]);
    tables::hermite_mid(tables::phi_Pd({xa, 1.0}, mid), tables::phi_Pd({xb, 1.0}, mid), h, &out[(size_t)8 * i + 4]);
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

#include "a2c_gpp.h"

// Value and analytic (forward-mode) derivative of an EAM function in FP64,
// numbered like a2c_gpp_eam_eval's functions: 0 F_Pd, 2 F_H, 4 f_Pd, 6 f_H,
// 8 phi_Pd, 10 phi_PdH, 12 phi_H.  The reference differentiates by central
// differences (potential.cpp:40-205); these are the exact derivatives the
// mixed form's tables are built from.
extern "C" a2c_status a2c_eam_analytic(int which, const double *x, int64_t n, double *value, double *deriv) {
  if (!x || !value || !deriv || n < 0 || which < 0 || which > 12 || (which & 1)) return A2C_ERR_INVALID;
  using a2c::tables::Dual;
  for (int64_t k = 0; k < n; ++k) {
    const Dual d{x[k], 1.0};
    Dual y{0.0, 0.0};
    switch (which) {
      case 0: y = a2c::tables::F_Pd(d); break;
      case 2: y = a2c::tables::F_H(d); break;
      case 4: y = a2c::tables::f_Pd(d, x[k]); break;
      case 6: y = a2c::tables::f_H(d); break;
      case 8: y = a2c::tables::phi_Pd(d, x[k]); break;
      case 10: y = a2c::tables::phi_PdH(d); break;
      default: y = a2c::tables::phi_H(d); break;
    }
    value[k] = y.v;
    deriv[k] = y.d;
  }
  return A2C_OK;
}

namespace {
float hv(const float *c, float t) { return std::fma(std::fma(std::fma(c[3], t, c[2]), t, c[1]), t, c[0]); }
float hd(const float *c, float t) { return std::fma(std::fma(3.0f * c[3], t, 2.0f * c[2]), t, c[1]); }
}  // namespace

// The mixed form's FP32 table interpolants evaluated on the host with the
// kernels' arithmetic (index clamp, cubic Hermite in FP32): which = 0 F_Pd,
// 2 F_H (embedding tables), 4 f_Pd, 8 phi_Pd (pair tables).  For checking
// the tables against a2c_eam_analytic.
extern "C" a2c_status a2c_mixed_table_eval(int which, const double *x, int64_t n, double *value, double *deriv) {
  if (!x || !value || !deriv || n < 0 || (which != 0 && which != 2 && which != 4 && which != 8)) return A2C_ERR_INVALID;
  static std::vector<float> pair, embPd, embH;
  static bool ready = false;
  if (!ready) {
    a2c::build_pair_table(a2c::kTabR0, 1.0 / a2c::kTabInvH, a2c::kTabN, pair);
    a2c::build_embed_table(0, 1.0 / a2c::kEmbInvH, a2c::kEmbN, embPd);
    a2c::build_embed_table(1, 1.0 / a2c::kEmbInvH, a2c::kEmbN, embH);
    ready = true;
  }
  for (int64_t k = 0; k < n; ++k) {
    const float s = (float)x[k];
    if (which == 0 || which == 2) {
      float u = std::fmin(std::fmax(s * (float)a2c::kEmbInvH, 0.0f), (float)a2c::kEmbN - 0.5f);
      const int i = (int)u;
      const float t = u - (float)i;
      const float *c = (which == 0 ? embPd : embH).data() + 4 * i;
      value[k] = hv(c, t);
      deriv[k] = hd(c, t) * (float)a2c::kEmbInvH;
    } else {
      // the pair kernels' indexing (k_mixed.cu tab_index): interval and
      // midpoint offset by the 1.5 * 2^23 rounding of an FMA result
      float xm = std::fma(s, (float)a2c::kTabInvH, (float)(-a2c::kTabR0 * a2c::kTabInvH - 0.5));
      xm = std::fmin(std::fmax(xm, -0.5f), (float)a2c::kTabN - 1.0f);
      const float y = xm + 12582912.0f;
      const float t = xm - (y - 12582912.0f);
      int32_t bits;
      std::memcpy(&bits, &y, 4);
      const int i = bits - 0x4B400000;
      const float *c = pair.data() + 8 * i + (which == 4 ? 0 : 4);
      value[k] = hv(c, t);
      deriv[k] = hd(c, t) * (float)a2c::kTabInvH;
    }
  }
  return A2C_OK;
}
