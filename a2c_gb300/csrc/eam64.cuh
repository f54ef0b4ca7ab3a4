// FP64 device restatement of the EAM Pd-H potential (potential.cpp:16-205,
// Zhou et al. 2007), written in the reference's evaluation order so that the
// plain form reproduces its bits.  exp is dd::fexp (0.5-ulp, the same bits
// on host and device) and pow is dd::cr_pow (ddmath.cuh).  Translation units including this header
// are compiled with -fmad=false: no multiply-add may be contracted into an
// FMA, exactly as the reference's x86-64 build performs them.  The numeric
// constants are the reference's; they define the potential.
#pragma once

#include "ddmath.cuh"

namespace a2c {
namespace eam64 {

// potential.cpp:16-38
__device__ __forceinline__ double F_Pd(double rho) {
  rho = rho / 50.0;
  double y = 295878.9003038662 * (rho - 0.20581955357385892);
  y = y * (rho - 0.081228755904399);
  y = y * rho;
  y = y * (rho + 0.05298811034615951);
  y = y * (rho * (rho - 2.4242616904962846) + 1.4791899886249564);
  y = y * (rho * (rho - 2.1376274623740064) + 1.2169215689822592);
  y = y * (rho * (rho - 1.6486007989726832) + 0.8159825255339774);
  y = y * (rho * (rho - 1.0749204110338482) + 0.42007491336688396);
  y = y * (rho * (rho - 0.5128056047933808) + 0.12468685331167456);
  y = y - (50.0 * 0.251546) * rho;
  return y;
}

// potential.cpp:45-57.  F_H is differentiated by a central difference, so
// its three pow calls use the correctly rounded dd::cr_pow (a one-ulp pow
// difference would otherwise become a ~1e-11 relative gradient error).
__device__ __forceinline__ double F_H(double rho) {
  const double c = 0.000197047, d = 1.18860, a = 9.99780, b = 60.0155, eps1 = 0.0540638;
  const double u = rho + eps1;
  double y = -c * (1.0 / (2.0 + d) * dd::cr_pow(u, 2.0 + d) - (a + b) / (1.0 + d) * dd::cr_pow(u, 1.0 + d) +
                   a * b / d * dd::cr_pow(u, d));
  y = y - (-0.0296604) * rho;
  return y;
}

// potential.cpp:64-98
__device__ __forceinline__ double f_Pd(double r) {
  r = r / 5.0;
  double ra = r;
  ra = ra * (r * (r - 2.7267629107325706) + 1.8716766113599643);
  ra = ra * (r * (r - 2.50290548851635) + 1.668549182690922);
  ra = ra * (r * (r - 2.0924467509943674) + 1.3150372774478005);
  ra = ra * (r * (r - 1.564328475106985) + 0.8987511149780485);
  ra = ra * (r * (r - 1.009780903403673) + 0.5124363774128722);
  ra = ra * (r * (r - 0.5304054524800665) + 0.2169886022464641);
  ra = ra * (r * (r - 0.1356566408715063) + 0.035852347523891395);
  double y = -0.02972698211669922 +
             r * (0.6676807403564453 + r * (-255.8965835571289 + r * (14673.409149169922 + -2.597301181336601e7 * ra)));
  const double r5 = r * 5.0;
  if (r5 <= 0.0) y = 0.0;
  else if (r5 > 5.0) y = 0.001510569378297 * dd::fexp(-0.077976566126292 / 0.001510569378297 * (r5 - 5.0));
  return y;
}

// potential.cpp:105-119
__device__ __forceinline__ double f_H(double r) {
  if (r <= 0.0) return 0.0;
  if (r > 5.35) return 0.009986990526578 * dd::fexp(-0.013075667086408 / 0.009986990526578 * (r - 5.35));
  return 11.0025 * dd::fexp(-1.30927 * r);
}

// potential.cpp:126-155
__device__ __forceinline__ double phi_Pd(double r) {
  r = r / 5.0;
  double y = -79415.24035137112 * (r - 1.0699996145674568);
  y = y * (r - 1.06015072612581);
  y = y * (r - 0.42433991011376526);
  y = y * (r + 0.06169160085238687);
  y = y * (r * (r - 2.0586473420376348) + 1.0683922574015199);
  y = y * (r * (r - 1.6696359816422877) + 0.7337878627470482);
  y = y * (r * (r - 1.1690370066230809) + 0.3909805777737639);
  y = y * (r * (r - 0.2635598721249787) + 0.033551116514910245);
  r = r * 5.0;
  y = y + (2 * 0.251546) * f_Pd(r);
  if (r <= 0.0) y = 0.0;
  else if (r > 5.05) y = -0.016958780164980 * dd::fexp(0.089019679316328 / -0.016958780164980 * (r - 5.05));
  return y;
}

// potential.cpp:162-177
__device__ __forceinline__ double phi_PdH(double r) {
  if (r <= 0.0) return 0.0;
  if (r > 5.35) return -3.353001113951400e-04 * dd::fexp(7.147062196813336e-04 / -3.353001113951400e-04 * (r - 5.35));
  const double D = 0.2494540, alpha = 4.82613, beta = 2.13158, r0 = 1.50964;
  return D * (beta * dd::fexp(-alpha * (r - r0)) - alpha * dd::fexp(-beta * (r - r0)));
}

// potential.cpp:185-200
__device__ __forceinline__ double phi_H(double r) {
  if (r <= 0.0) return 0.0;
  if (r > 5.35) return -0.003702722457147 * dd::fexp(0.005465945471933 / -0.003702722457147 * (r - 5.35));
  const double D = 0.0661496, alpha = 3.67263, beta = 1.47797, r0 = 2.51980;
  return D * (beta * dd::fexp(-alpha * (r - r0)) - alpha * dd::fexp(-beta * (r - r0)));
}

// Central finite differences with step eps (potential.cpp:40, 59, 100, 121,
// 157, 179, 202).
__device__ __forceinline__ double F_Pd_d(double x, double e) { return (F_Pd(x + e) - F_Pd(x - e)) / (2.0 * e); }
__device__ __forceinline__ double F_H_d(double x, double e) { return (F_H(x + e) - F_H(x - e)) / (2.0 * e); }
__device__ __forceinline__ double f_Pd_d(double x, double e) { return (f_Pd(x + e) - f_Pd(x - e)) / (2.0 * e); }
__device__ __forceinline__ double f_H_d(double x, double e) { return (f_H(x + e) - f_H(x - e)) / (2.0 * e); }
__device__ __forceinline__ double phi_Pd_d(double x, double e) { return (phi_Pd(x + e) - phi_Pd(x - e)) / (2.0 * e); }
__device__ __forceinline__ double phi_PdH_d(double x, double e) { return (phi_PdH(x + e) - phi_PdH(x - e)) / (2.0 * e); }
__device__ __forceinline__ double phi_H_d(double x, double e) { return (phi_H(x + e) - phi_H(x - e)) / (2.0 * e); }

}  // namespace eam64
}  // namespace a2c
