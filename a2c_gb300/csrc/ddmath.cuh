// Near-correctly-rounded exp, log and pow for the FP64 plain form, built on
// double-double ("dd") arithmetic: Dekker's and Knuth's error-free
// transformations (two-sum, two-product via FMA), as used in Bailey's QD
// library.  Why: the reference differentiates F_H (three pow calls) by a
// central difference with step 1e-5, which multiplies a one-ulp difference
// between two libm implementations by ~1e5.  Rounding the exact value
// correctly makes the device result agree with any accurate C library
// (glibc's pow/exp/log are within ~0.52 ulp) except in rare near-midpoint
// cases, instead of in a sizeable fraction of calls.
//
// Method (published, textbook):
//   exp(a):  k = rint(a/ln2), r = (a - k ln2)/2^10 in dd, e^r - 1 by its
//            Taylor series to r^11 in dd, then (1+s)^(2^10) by ten
//            squarings of the expm1 form s <- 2s + s^2, times 2^k.
//   log(u):  y0 = log(u) in double, one Newton step y = y0 + t - t^2/2
//            with t = u*exp(-y0) - 1 evaluated in dd.
//   pow(u,y) = exp(y * log(u)) with the product and exp in dd.
// The Taylor coefficients 1/n! and ln 2 are mathematical constants split
// into hi + lo doubles.  All functions are __host__ __device__ so the host
// build can be tested against the C library directly.
//
// fexp is the fast exp of the per-pair-point EAM terms: Tang's table-driven
// method with 64 subintervals, x = (64k + j) ln2/64 + r, |r| <= ln2/128,
// e^x = 2^k 2^(j/64) (1 + p(r)), p the degree-6 Taylor polynomial of
// e^r - 1 (truncation < 4e-20), 2^(j/64) held as hi + lo, reduction and
// reconstruction with FMA.  Its error is ~0.5 ulp and, being plain IEEE
// arithmetic, it gives the same bits on the host and on the device, which
// lets the CPU oracle reproduce the GPU plain form exactly.
#pragma once

#include <cmath>

namespace a2c {
namespace dd {

#if defined(__CUDACC__)
#define A2C_HD __host__ __device__ __forceinline__
#else
#define A2C_HD inline
#endif

struct D2 {
  double hi, lo;
};

A2C_HD D2 two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  const double e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
A2C_HD D2 quick_two_sum(double a, double b) {
  const double s = a + b;
  return {s, b - (s - a)};
}
A2C_HD D2 two_prod(double a, double b) {
  const double p = a * b;
  return {p, fma(a, b, -p)};
}
A2C_HD D2 add(D2 a, D2 b) {
  D2 s = two_sum(a.hi, b.hi);
  const D2 t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
A2C_HD D2 mul(D2 a, D2 b) {
  D2 p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return quick_two_sum(p.hi, p.lo);
}
A2C_HD D2 mul_d(D2 a, double b) {
  D2 p = two_prod(a.hi, b);
  p.lo += a.lo * b;
  return quick_two_sum(p.hi, p.lo);
}

// e^a for a double-double argument; |a| < 700.
A2C_HD D2 exp_dd(D2 a) {
  const D2 LN2 = {0.6931471805599453, 2.3190468138462996e-17};
  const double k = rint(a.hi / LN2.hi);
  D2 r = add(a, mul_d(LN2, -k));
  r.hi *= 0.0009765625;  // 2^-10, exact
  r.lo *= 0.0009765625;
  // Taylor coefficients 1/n!, n = 2..11
  const D2 C[10] = {{0.5, 0.0},
                    {0.16666666666666666, 9.25185853854297e-18},
                    {0.041666666666666664, 2.3129646346357427e-18},
                    {0.008333333333333333, 1.1564823173178714e-19},
                    {0.001388888888888889, -5.300543954373577e-20},
                    {0.0001984126984126984, 1.7209558293420705e-22},
                    {2.48015873015873e-05, 2.1511947866775882e-23},
                    {2.7557319223985893e-06, -1.858393274046472e-22},
                    {2.755731922398589e-07, 2.3767714622250297e-23},
                    {2.505210838544172e-08, -1.448814070935912e-24}};
  // s = r + r^2/2! + ... + r^11/11!  (Horner on the coefficients)
  D2 p = C[9];
  for (int n = 8; n >= 0; --n) p = add(mul(p, r), C[n]);
  D2 s = add(mul(p, mul(r, r)), r);
  for (int i = 0; i < 10; ++i) s = add(mul_d(s, 2.0), mul(s, s));  // (1+s)^2 - 1
  D2 e = add({1.0, 0.0}, s);
  const int ki = (int)k;
  return {ldexp(e.hi, ki), ldexp(e.lo, ki)};
}

// log(u) as double-double, u > 0 finite.
A2C_HD D2 log_dd(double u) {
  const double y0 = log(u);
  const D2 e = exp_dd({-y0, 0.0});
  const D2 t = add(mul_d(e, u), {-1.0, 0.0});  // u e^{-y0} - 1, |t| ~ 1e-16
  const double t2 = 0.5 * t.hi * t.hi;
  return add({y0, 0.0}, add(t, {-t2, 0.0}));
}

A2C_HD double round_dd(D2 a) { return a.hi + a.lo; }

// 2^(j/64), j = 0..63, split into hi + lo
#define A2C_EXP2_TABLE \
    {1.0, 0.0}, \
    {1.0108892860517005, -1.5234778603368577e-17}, \
    {1.0218971486541166, 5.109225028973444e-17}, \
    {1.0330248790212284, 7.600838874027088e-18}, \
    {1.0442737824274138, 8.551889705537965e-17}, \
    {1.0556451783605572, 1.759325738772092e-18}, \
    {1.0671404006768237, -7.899853966841582e-17}, \
    {1.0787607977571199, -6.656660436056593e-17}, \
    {1.0905077326652577, -3.046782079812471e-17}, \
    {1.102382583307841, 5.2660368715706944e-17}, \
    {1.1143867425958924, 1.0410278456845571e-16}, \
    {1.1265216186082418, 5.165856758795457e-17}, \
    {1.1387886347566916, 8.912812676025408e-17}, \
    {1.1511892299529827, 3.250710218863827e-17}, \
    {1.1637248587775775, 3.8292048369240935e-17}, \
    {1.1763969916502812, 5.554203254218079e-17}, \
    {1.189207115002721, 3.982015231465646e-17}, \
    {1.202156731452703, 6.644981499252301e-17}, \
    {1.215247359980469, -7.712630692681488e-17}, \
    {1.22848053610687, -1.89878163130253e-17}, \
    {1.241857812073484, 4.658027591836937e-17}, \
    {1.255380757024691, -6.7113898212968784e-18}, \
    {1.2690509571917332, 2.667932131342186e-18}, \
    {1.2828700160787783, 1.713594918243561e-17}, \
    {1.2968395546510096, 2.5382502794888315e-17}, \
    {1.3109612115247644, -7.181536135519454e-17}, \
    {1.3252366431597413, -2.8587312100388614e-17}, \
    {1.339667524053303, 8.927282594831732e-17}, \
    {1.3542555469368927, 7.70094837980299e-17}, \
    {1.3690024229745905, 9.593797919118849e-17}, \
    {1.383909881963832, -6.770511658794786e-17}, \
    {1.3989796725383112, -9.614213209051323e-17}, \
    {1.4142135623730951, -9.667293313452913e-17}, \
    {1.42961333839197, -1.2031642489053655e-17}, \
    {1.4451808069770467, -3.0237581349939873e-17}, \
    {1.460917794180647, -5.600377186075216e-17}, \
    {1.4768261459394993, -3.483994556892796e-17}, \
    {1.4929077282912648, 1.4192920154284036e-17}, \
    {1.5091644275934228, -1.016455327754295e-16}, \
    {1.5255981507445384, -1.1024941712342561e-16}, \
    {1.5422108254079407, 7.949834809697621e-17}, \
    {1.559004400237837, 3.7812070533575275e-17}, \
    {1.5759808451078865, -1.0136916471278304e-17}, \
    {1.593142151342267, -1.0094406542311964e-16}, \
    {1.6104903319492543, 2.4707192569797888e-17}, \
    {1.6280274218573478, -6.712955084707084e-17}, \
    {1.645755478153965, -1.0125679913674773e-16}, \
    {1.6636765803267364, 5.8909926967131e-17}, \
    {1.681792830507429, 8.199010020581497e-17}, \
    {1.7001063537185235, -8.0237193703977e-18}, \
    {1.718619298122478, -1.851380418263111e-17}, \
    {1.7373338352737062, 3.164389299292957e-17}, \
    {1.7562521603732995, 2.960140695448873e-17}, \
    {1.7753764925265212, 6.429731796556572e-17}, \
    {1.7947090750031072, 1.8227458427912087e-17}, \
    {1.8142521755003989, -9.969531538920349e-17}, \
    {1.8340080864093424, 3.283107224245627e-17}, \
    {1.8539791250833855, 9.761887490727594e-17}, \
    {1.8741676341103, -6.122763413004143e-17}, \
    {1.8945759815869656, 3.4034035352165297e-17}, \
    {1.9152065613971474, -1.0619946056195963e-16}, \
    {1.9360617934922943, 1.0332385960676326e-16}, \
    {1.9571441241754002, 8.960767791036668e-17}, \
    {1.978456026387951, 4.0388753109278167e-17}
#if defined(__CUDACC__)
__device__ const double kExp2TabDev[64][2] = {A2C_EXP2_TABLE};
#endif
static const double kExp2TabHost[64][2] = {A2C_EXP2_TABLE};
#undef A2C_EXP2_TABLE

// Results below 2^-1021 are flushed to zero (no argument of the potential
// comes near), above 709.78 overflow to +inf; NaN propagates.
A2C_HD double fexp(double x) {
  if (!(x > -708.0)) return (x != x) ? x : 0.0;
  if (x > 709.78) return HUGE_VAL;
  const double n = rint(x * 92.33248261689366);  // x * 64/ln2
  const int ni = (int)n;
  const int j = ni & 63;
  const int k = (ni - j) / 64;
  double r = fma(-n, 0.010830424696249145, x);    // ln2/64, hi
  r = fma(-n, 3.623510646634843e-19, r);           // ln2/64, lo
  double p = fma(r, 0.001388888888888889, 0.008333333333333333);
  p = fma(r, p, 0.041666666666666664);
  p = fma(r, p, 0.16666666666666666);
  p = fma(r, p, 0.5);
  p = fma(r * r, p, r);
#if defined(__CUDA_ARCH__)
  const double th = kExp2TabDev[j][0], tl = kExp2TabDev[j][1];
#else
  const double th = kExp2TabHost[j][0], tl = kExp2TabHost[j][1];
#endif
  return ldexp(th + fma(th, p, tl), k);
}

// Correctly rounded except in rare near-midpoint cases.
A2C_HD double cr_exp(double x) {
  if (!(x > -700.0 && x < 700.0)) return exp(x);
  return round_dd(exp_dd({x, 0.0}));
}
A2C_HD double cr_log(double u) {
  if (!(u > 0.0) || !(u < 1.0e300) || u < 1.0e-300) return log(u);
  return round_dd(log_dd(u));
}
A2C_HD double cr_pow(double u, double y) {
  if (!(u > 0.0) || !(u < 1.0e300) || u < 1.0e-300 || !(fabs(y) < 1.0e6)) return pow(u, y);
  const D2 l = mul_d(log_dd(u), y);
  if (!(l.hi > -700.0 && l.hi < 700.0)) return pow(u, y);
  return round_dd(exp_dd(l));
}

#undef A2C_HD

}  // namespace dd
}  // namespace a2c
