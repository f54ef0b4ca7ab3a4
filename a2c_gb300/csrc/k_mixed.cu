// Mixed-precision evaluator: FP32 pair quadrature with compensated per-site
// sums; FP64 for the per-site finish, the global free-entropy reduction and
// everything the L-BFGS touches.  Same mathematics as minimizer.cpp:83-369
// (pass 1: electrondensity.cpp:20-49) with analytic derivatives in place of
// the reference's central differences.
//
// Layout per evaluation (k_prep): every site becomes one int4 -- its
// position as three 32-bit fixed-point coordinates (unit S/2^32 with S the
// periodic box length, or kFreeSpan = 64 A in a free direction) and sigma
// as FP32 bits.  The integer difference of two coordinates, taken modulo
// 2^32, is the minimum-image difference exactly, so no FP64 arithmetic and
// no image decoding happen per neighbor; converting it to FP32 costs one
// rounding.  In a free direction it is exact while the pair is less than
// 32 A apart: the prep kernels flag any site that moved far enough from
// its position at the list build for a listed pair to get there
// (span_check), and the call returns A2C_ERR_LISTS_STALE.
//
// Quadrature in closed form: point k moves coordinate m = k/2 mod 3 of atom i
// (k < 6) or of atom j (k >= 6) by u = sqrt(6) sigma, so with the pair
// vector D, |r_k|^2 = (|D|^2 + u^2) +- 2 D_m u: one FMA per point.  The
// gradient sums reduce to per-pair scalars (sum of c_k, per-coordinate
// u-weighted differences), multiplied by D once per neighbor.
//
// Functions: f_Pd and phi_Pd from the FP32 cubic Hermite tables of
// tables.cpp (their polynomial forms cancel catastrophically in FP32), held
// in shared memory: the kernels are persistent, each block loads the 30 KB
// of tables once and then walks many sites -- from global memory the
// data-dependent table gathers (28 sectors per request) saturated the L1;
// f_H, phi_PdH, phi_H analytically with ex2.approx (their exponential tails
// beyond 5.35 A are C1 continuations, selected branch-free); F and F' per
// site from FP32 Hermite tables in rho.
//
// Mapping: TPS threads per site (1, 2, 4 or 8), each taking every TPS-th
// neighbor, first among the Pd then among the H neighbors (so the lanes of a
// warp evaluate the same pair type together), combined by shuffles.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "ddmath.cuh"
#include "internal.cuh"
#include "tables.h"

namespace a2c {

void build_pair_table(double r0, double h, int n, std::vector<float> &out);
void build_pair_table_raw(double r0, double h, int n, float *out);
void build_embed_table(int species, double h, int n, std::vector<float> &out);

struct Mixed {
  int64_t N = 0;
  int4 *P = nullptr;        // per site: fixed-point x, y, z; sigma (FP32 bits)
  float *occ = nullptr;     // per site occupancy (1 for Pd)
  float2 *FF = nullptr;     // per site (F'(rho), F(rho))
  float4 *tabPair = nullptr;  // f_Pd cubics, phi_Pd cubics, f_Pd' quadratics (kTabN each)
  int grid_cap[9] = {};       // persistent grid size per threads-per-site
  float4 *tabEmb = nullptr;   // per rho interval: F_Pd cubics, then F_H cubics
  int tps = 0;                // threads per site (0 = choose)
  int rho_block = 0, grad_block = 0;  // threads per block of pass 1 and pass 2 (0 = 256)
  // Pass 2 with every pair evaluated once (sorted, symmetric lists): per
  // list entry of a pair the site owns (neighbor id below its own) the slot
  // of the reverse entry; per site the count of such entries, with the
  // validation flag after the last site; per entry the contribution the
  // neighbor's side receives from the owner.
  int pair_mode = A2C_PAIRS_ONCE;
  uint32_t *rev = nullptr;
  int *npre = nullptr;
  float4 *recv = nullptr;
  double *Gown = nullptr;  // 4 per site: the owner's share of the gradient (k_grad_once)
  void *fpart = nullptr;     // the objective's block sums: one ObjSum per block of k_objective
  unsigned *fcount = nullptr;
  int64_t sym_entries = 0, sym_sites = 0;  // capacities
  uint64_t sym_version = ~0ull;            // list version the index was built for
  bool sym_ok = false;
};

namespace {

constexpr int kBlock = 256;  // threads per block of the other kernels (and the tiles' default)
// Pass 2 resident threads per SM the register allocation must allow: 1024
// (64 registers per thread), whatever the block size.
#ifndef A2C_GRAD_MIN_BLOCKS
#define A2C_GRAD_MIN_BLOCKS 4
#endif
// Pass 1 at 256 threads per block: 5 blocks = 48 registers per thread.
// Its 98 KB of table copies allow two blocks per SM, so larger blocks are
// how it gets more warps: 512 threads (2 blocks, 64 registers) or 768
// (2 blocks, 42 registers).
#ifndef A2C_RHO_MIN_BLOCKS
#define A2C_RHO_MIN_BLOCKS 5
#endif
template <int BLOCK>
constexpr int grad_min_blocks() {
  return A2C_GRAD_MIN_BLOCKS * 256 / BLOCK;
}
template <int BLOCK>
constexpr int rho_min_blocks() {
  return BLOCK == 256 ? A2C_RHO_MIN_BLOCKS : 2;
}

// Folded exponential constants of f_H, phi_PdH, phi_H (see fH, morse below).
struct MorseExp {
  float K1, C1, L1, K2, C2, L2, Kt, Ct, Lt;
};
struct ExpTerms {
  float fK, fC, fdC;
  MorseExp pdh, hh;
};
struct ObjSum;
struct MixArgs {
  int64_t N;
  int nPd;
  float W;
  float sc[3];  // metres of one fixed-point unit per dimension [A]
  const int4 *P;
  const float *occ;
  const int64_t *off;
  const uint32_t *nbr;
  const int *npd;
  ExpTerms ex;
  const float4 *tabPair;
  const float4 *tabEmb;
  float2 *FF;
  double *G, *Vs, *Ss;
  double T;
  BatchView bv;  // batched list launch (LIST kernels)
  const uint32_t *rev;  // pairs evaluated once (k_grad_once, k_grad_recv)
  const int *npre;
  float4 *recv;
  double *Gown;
  // A single system's objective (k_objective): per block its sums, the
  // count of blocks done, f and its two sums.
  ObjSum *fpart;
  unsigned *fcount;
  double *f, *fsums;
  // host-pointer calls: pinned memory that receives f and the status word
  // (then cleared), null otherwise
  double *hout;
  int *status;
};

__device__ __forceinline__ float ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rsq(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ void kahan(float &s, float &c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

__device__ __forceinline__ float3 pair_vec(float3 sc, int4 pi, int4 pj) {  // q_i - q_j
  return make_float3((float)(int)((unsigned)pi.x - (unsigned)pj.x) * sc.x,
                     (float)(int)((unsigned)pi.y - (unsigned)pj.y) * sc.y,
                     (float)(int)((unsigned)pi.z - (unsigned)pj.z) * sc.z);
}

// The site handled by work item k and what it needs from its instance.
template <bool LIST>
struct SiteRef {
  int64_t s;
  bool iPd;
  float3 sc;
  double T;
};
template <bool LIST>
__device__ __forceinline__ SiteRef<LIST> site_ref(const MixArgs &a, int64_t k) {
  SiteRef<LIST> r;
  if (LIST) {
    r.s = a.bv.list[k];
    const InstGeo &g = a.bv.geo[a.bv.inst[r.s]];
    r.iPd = r.s - g.start < g.nPd;
    r.sc = make_float3(g.sc[0], g.sc[1], g.sc[2]);
    r.T = g.T;
  } else {
    r.s = k;
    r.iPd = k < a.nPd;
    r.sc = make_float3(a.sc[0], a.sc[1], a.sc[2]);
    r.T = a.T;
  }
  return r;
}

__device__ __forceinline__ float hv(float4 c, float t) { return fmaf(fmaf(fmaf(c.w, t, c.z), t, c.y), t, c.x); }
__device__ __forceinline__ float hd(float4 c, float t) { return fmaf(fmaf(3.0f * c.w, t, 2.0f * c.z), t, c.y); }
// h times the derivative from its own coefficients (c1, 2 c2, 3 c3)
__device__ __forceinline__ float dq(float4 d, float t) { return fmaf(fmaf(d.z, t, d.y), t, d.x); }

// Interval of the pair tables and the offset t in [-1/2, 1/2] from its
// midpoint (the tables hold midpoint-centred cubics), without a float-to-int
// conversion: xm = (s - r0)/h - 1/2, clamped to [-1/2, NTAB - 1], plus
// 1.5 * 2^23 rounds to 1.5 * 2^23 + rint(xm), whose low bits are the
// interval (a tie at a knot picks the even neighbor; both cubics agree
// there).
template <int NTAB = kTabN>
__device__ __forceinline__ int tab_index(float s, float &t) {
  float xm = fmaf(s, (float)kTabInvH, (float)(-kTabR0 * kTabInvH - 0.5));
  xm = fminf(fmaxf(xm, -0.5f), (float)NTAB - 1.0f);
  const float y = xm + 12582912.0f;
  t = xm - (y - 12582912.0f);
  return __float_as_int(y) - 0x4B400000;
}

// f_H, phi_PdH and phi_H as exponentials 2^(K s + C): the prefactor, the
// shift and the log2(e) scale are folded into K and C on the host, in
// double (exp_terms), so each term costs one FMA and one ex2.
//   f_H(r) = C e^{-delta r} (potential.cpp:105-119; its tail beyond 5.35 A
//     is the same exponential): f_H = 2^(fK s + fC), -f_H' = 2^(fK s + fdC).
//   phi_PdH, phi_H (potential.cpp:162-200) = D (b e^{-a(r-r0)} - a
//     e^{-b(r-r0)}) for r <= 5.35 A, funRc e^{k(r-5.35)} beyond:
//     phi = E1 - E2, phi' = L1 E1 + L2 E2 with E1 = 2^(K1 s + C1) and
//     E2 = 2^(K2 s + C2) inside; phi = -Et, phi' = Lt Et with
//     Et = 2^(Kt s + Ct) beyond.  (MorseExp, ExpTerms are declared above.)
__device__ __forceinline__ float fH(const ExpTerms &x, float s) { return ex2(fmaf(s, x.fK, x.fC)); }
__device__ __forceinline__ float fHd_neg(const ExpTerms &x, float s) { return ex2(fmaf(s, x.fK, x.fdC)); }
// Inside the switch radius only (the caller has checked s <= 5.35 A).
__device__ __forceinline__ void morse_in(const MorseExp &m, float s, float &v, float &d) {
  const float e1 = ex2(fmaf(s, m.K1, m.C1)), e2 = ex2(fmaf(s, m.K2, m.C2));
  v = e1 - e2;
  d = fmaf(m.L1, e1, m.L2 * e2);
}
__device__ __forceinline__ void morse(const MorseExp &m, float s, float &v, float &d) {
  const bool tail = s > 5.35f;
  const float e1 = tail ? 0.0f : ex2(fmaf(s, m.K1, m.C1));
  const float e2 = ex2(fmaf(s, tail ? m.Kt : m.K2, tail ? m.Ct : m.C2));
  v = e1 - e2;
  d = fmaf(m.L1, e1, (tail ? m.Lt : m.L2) * e2);
}

constexpr float kSqrt6 = 2.449489742783178f;

// The four squared radii of coordinate c for the pair (D, ui, uj):
// atom i moved by +ui, -ui; atom j moved by -uj, +uj (r = q_i - q_j).
#define A2C_RADII(c, Dc)                                  \
  const float bi = 2.0f * (Dc) * ui, bj = 2.0f * (Dc) * uj; \
  const float s2[4] = {Ai + bi, Ai - bi, Aj - bj, Aj + bj};


// Walks neighbor entries begin, begin+step, ... < end with the loads of the
// next neighbor (its entry one step further ahead) issued before the current
// one is computed: the entry -> state -> arithmetic chain is otherwise a
// dependent global-load latency per neighbor (the dominant stall).
template <bool OCC, bool FP, class Body>
__device__ __forceinline__ void walk_neighbors(const MixArgs &a, int64_t begin, int64_t end, int step, Body body) {
  int64_t t = begin;
  if (t >= end) return;
  int64_t j0 = __ldg(&a.nbr[t]) & kIdMask;
  int4 p0 = __ldg(&a.P[j0]);
  float x0 = OCC ? __ldg(&a.occ[j0]) : 1.0f;
  float f0 = FP ? __ldg(&a.FF[j0].x) : 0.0f;
  int64_t t1 = t + step;
  uint32_t e1 = (t1 < end) ? __ldg(&a.nbr[t1]) : 0u;
  for (; t < end; t += step) {
    const int64_t t2 = t1 + step;
    int4 p1 = p0;
    float x1 = x0, f1 = f0;
    uint32_t e2 = 0u;
    if (t1 < end) {
      const int64_t j1 = e1 & kIdMask;
      p1 = __ldg(&a.P[j1]);
      if (OCC) x1 = __ldg(&a.occ[j1]);
      if (FP) f1 = __ldg(&a.FF[j1].x);
    }
    if (t2 < end) e2 = __ldg(&a.nbr[t2]);
    body(t, p0, x0, f0);
    p0 = p1;
    x0 = x1;
    f0 = f1;
    e1 = e2;
    t1 = t2;
  }
}

// The per-site finish of pass 1: rho = W * (sum of the density terms), then
// F'(rho) and F(rho) from the embedding table of the site's species.
__device__ __forceinline__ void rho_finish(const MixArgs &a, int64_t s, bool iPd, float tot) {
  const float rho = tot * a.W;
  float x = fminf(fmaxf(rho * (float)kEmbInvH, 0.0f), (float)kEmbN - 0.5f);
  const int i = (int)x;
  const float tt = x - (float)i;
  const float4 c = __ldg(&a.tabEmb[(iPd ? 0 : kEmbN) + i]);
  a.FF[s] = make_float2(hd(c, tt) * (float)kEmbInvH, hv(c, tt));
}

// ---------------------------------------------------------------- pass 1
// The f_Pd table in shared memory as 8 interleaved copies: interval i of
// copy c is float4 number 8 i + c, in bank group c.  A 128-bit shared load
// serves a warp in four phases of 8 consecutive lanes; lane l reads copy
// l mod 8, so the 8 lanes of a phase always hit 8 different bank groups
// and a lookup takes the minimum 4 wavefronts, where random intervals in
// one copy took about 10.  Pass 1 keeps the intervals below 5.8 A (f_Pd <
// 1e-19 A beyond; the last interval's value stands in there).
constexpr int kRhoTabN = 768;
constexpr int kRhoCopies = 8;
constexpr size_t kRhoSmem = sizeof(float4) * kRhoTabN * kRhoCopies;  // 98,304 B: two blocks per SM

// Pass 2 reads two tables (f_Pd' and phi_Pd).  Interleaved copies cost it
// occupancy (8 copies of both: one 256-thread block per SM; 4: two), and
// pass 2 needs the resident warps more than conflict-free lookups: on a
// GB300 at 262,144 sites pass 2 took 0.329 ms with one copy (four blocks
// per SM), 0.375 ms with 4 copies and 0.530 ms with 8.  So one copy.
#ifndef A2C_GRAD_COPIES
#define A2C_GRAD_COPIES 1
#endif
constexpr int kGradCopies = A2C_GRAD_COPIES;
constexpr int kGradTabN = kTabN;  // phi_Pd is -3e-4 eV at 5.8 A: every interval
constexpr size_t kGradSmem = 2 * sizeof(float4) * kGradTabN * kGradCopies;

template <int TPS, bool LIST, int BLOCK>
__global__ void __launch_bounds__(BLOCK, rho_min_blocks<BLOCK>()) k_rho_mixed(MixArgs a) {
  constexpr int kSitesPerBlock = BLOCK / TPS;
  const int64_t n = LIST ? (int64_t)*a.bv.count : a.N;
  if ((int64_t)blockIdx.x * kSitesPerBlock >= n) return;
  extern __shared__ float4 sF8[];
  for (int i = threadIdx.x; i < kRhoTabN * kRhoCopies; i += blockDim.x) sF8[i] = __ldg(&a.tabPair[i / kRhoCopies]);
  __syncthreads();
  const float4 *sF = sF8 + (threadIdx.x % kRhoCopies);  // this lane's copy: interval i at sF[8 i]
  for (int64_t base = (int64_t)blockIdx.x * kSitesPerBlock; base < n;
       base += (int64_t)gridDim.x * kSitesPerBlock) {
  const int64_t k = base + threadIdx.x / TPS;
  const int lane = (int)(threadIdx.x % TPS);
  const bool live = k < n;
  SiteRef<LIST> R{};
  if (live) R = site_ref<LIST>(a, k);
  const int64_t s = R.s;
  float acc = 0.0f, cmp = 0.0f;
  if (live) {
    const int4 pi = a.P[s];
    const float ui = kSqrt6 * __int_as_float(pi.w), ui2 = ui * ui;
    const int64_t b = a.off[s], m = b + a.npd[s], e = a.off[s + 1];
    walk_neighbors<false, false>(a, b + lane, m, TPS, [&](int64_t, int4 pj, float, float) {  // Pd neighbors: f_Pd
      const float3 D = pair_vec(R.sc, pi, pj);
      const float uj = kSqrt6 * __int_as_float(pj.w);
      const float D2 = fmaf(D.x, D.x, fmaf(D.y, D.y, D.z * D.z));
      const float Ai = D2 + ui2, Aj = fmaf(uj, uj, D2);
      float part = 0.0f;
      const float Dv[3] = {D.x, D.y, D.z};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        A2C_RADII(c, Dv[c])
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float r = s2[q] * rsq(s2[q]);
          float tt;
          const int i = tab_index<kRhoTabN>(r, tt);
          part += hv(sF[kRhoCopies * i], tt);
        }
      }
      kahan(acc, cmp, part);
    });
    walk_neighbors<true, false>(a, m + lane, e, TPS, [&](int64_t, int4 pj, float xj, float) {  // H neighbors: x_j f_H
      const float3 D = pair_vec(R.sc, pi, pj);
      const float uj = kSqrt6 * __int_as_float(pj.w);
      const float D2 = fmaf(D.x, D.x, fmaf(D.y, D.y, D.z * D.z));
      const float Ai = D2 + ui2, Aj = fmaf(uj, uj, D2);
      float part = 0.0f;
      const float Dv[3] = {D.x, D.y, D.z};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        A2C_RADII(c, Dv[c])
#pragma unroll
        for (int q = 0; q < 4; ++q) part += fH(a.ex, s2[q] * rsq(s2[q]));
      }
      kahan(acc, cmp, part * xj);
    });
  }
  float tot = acc;
#pragma unroll
  for (int o = TPS / 2; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if (live && lane == 0) rho_finish(a, s, R.iPd, tot);
  }
}

// ---------------------------------------------------------------- pass 2
// Per pair: c_k = g(s_k)/s_k with g = F'_A(rho_i) f'_B + F'_B(rho_j) f'_A +
// phi'_AB; the pair's gradient contributions are
//   sum_k c_k r_k = D * sum_k c_k + e_m * sum over the points moving m of c_k delta_k
//   sigma part    = sqrt(3) sum_m [ D_m (c_{+i} - c_{-i}) + ui (c_{+i} + c_{-i}) ]
// scaled by W x_j; the energy is 0.5 W x_i x_j sum_k phi(s_k).  c_k is
// symmetric in the two sites, so the neighbor's side of the same pair is
// -(D sum_k c_k + e) for its position and, for its width,
//   sigj = sqrt(3) sum_m [ D_m (c_{+j} - c_{-j}) + uj (c_{+j} + c_{-j}) ]
// in the notation below (c_{+j}: r = D + uj e_m, c_{-j}: r = D - uj e_m).
struct PairAcc {
  float csum, e[3], sig, v, sigj;
};

// True when all 12 quadrature points of the pair lie within the 5.35 A
// switch radius of phi_PdH / phi_H: the largest squared radius is
// |D|^2 + u^2 + 2 u max|D_c| with u the larger displacement.
__device__ __forceinline__ bool pair_inside(float3 D, float ui, float uj) {
  const float u = fmaxf(ui, uj);
  const float m = fmaxf(fabsf(D.x), fmaxf(fabsf(D.y), fabsf(D.z)));
  const float D2 = fmaf(D.x, D.x, fmaf(D.y, D.y, D.z * D.z));
  return fmaf(2.0f * u, m, fmaf(u, u, D2)) <= 5.35f * 5.35f;
}

// TAIL = false: every point is inside the switch radius (pair_inside), so
// the Morse terms skip the per-point branch selection.
template <int TYPE, bool TAIL = true>  // 0 Pd-Pd, 1 Pd i / H j, 2 H i / Pd j, 3 H-H
__device__ __forceinline__ void pair_terms(const ExpTerms &x, const float4 *sF, const float4 *sP, float Fa, float Fb,
                                           float3 D, float ui, float uj, PairAcc &p) {
  const float D2 = fmaf(D.x, D.x, fmaf(D.y, D.y, D.z * D.z));
  const float Ai = fmaf(ui, ui, D2), Aj = fmaf(uj, uj, D2);
  const float Dv[3] = {D.x, D.y, D.z};
  p.csum = 0.0f;
  p.sig = 0.0f;
  p.v = 0.0f;
  p.sigj = 0.0f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    A2C_RADII(c, Dv[c])
    float ck[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float is = rsq(s2[q]);
      const float r = s2[q] * is;
      float g, phi;
      if (TYPE == 0) {
        float tt;
        const int i = kGradCopies * tab_index<kGradTabN>(r, tt);
        const float4 cf = sF[i], cp = sP[i];
        // phi and h phi' share one Horner chain
        const float hp = fmaf(cp.w, tt, cp.z), hq = fmaf(hp, tt, cp.y);
        phi = fmaf(hq, tt, cp.x);
        g = fmaf(Fa + Fb, dq(cf, tt), fmaf(fmaf(cp.w, tt, hp), tt, hq)) * (float)kTabInvH;
      } else if (TYPE == 3) {
        const float nfhd = fHd_neg(x, r);  // -f_H'
        float dphi;
        if (TAIL) morse(x.hh, r, phi, dphi);
        else morse_in(x.hh, r, phi, dphi);
        g = fmaf(-(Fa + Fb), nfhd, dphi);
      } else {
        float tt;
        const int i = kGradCopies * tab_index<kGradTabN>(r, tt);
        const float fpd = dq(sF[i], tt) * (float)kTabInvH;
        const float nfhd = fHd_neg(x, r);
        float dphi;
        if (TAIL) morse(x.pdh, r, phi, dphi);
        else morse_in(x.pdh, r, phi, dphi);
        g = (TYPE == 1) ? fmaf(-Fa, nfhd, fmaf(Fb, fpd, dphi)) : fmaf(Fa, fpd, fmaf(-Fb, nfhd, dphi));
      }
      ck[q] = g * is;
      p.v += phi;
    }
    const float cpi = ck[0], cmi = ck[1], cmj = ck[2], cpj = ck[3];
    p.csum += (cpi + cmi) + (cmj + cpj);
    p.e[c] = fmaf(ui, cpi - cmi, uj * (cpj - cmj));
    p.sig = fmaf(Dv[c], cpi - cmi, fmaf(ui, cpi + cmi, p.sig));
    p.sigj = fmaf(Dv[c], cpj - cmj, fmaf(uj, cpj + cmj, p.sigj));
  }
}

struct SiteAcc {
  float s[5], c[5];  // Fq x, y, z, Fsigma, V  with Kahan compensations
};

// The gradient components are plain FP32 sums: compensating them measured
// no change in the gradient's error (1.28e-5 relative to the FP64 form
// either way at 262,144 sites -- it is set by the FP32 rounding of the pair
// terms, not by their summation) and cost pass 2 3%.  The energy, whose
// terms do not cancel, keeps its compensation.
__device__ __forceinline__ void add_pair(SiteAcc &A, const PairAcc &p, float3 D, float wx, float vx) {
  A.s[0] = fmaf(wx, fmaf(D.x, p.csum, p.e[0]), A.s[0]);
  A.s[1] = fmaf(wx, fmaf(D.y, p.csum, p.e[1]), A.s[1]);
  A.s[2] = fmaf(wx, fmaf(D.z, p.csum, p.e[2]), A.s[2]);
  A.s[3] = fmaf(wx, p.sig, A.s[3]);
  kahan(A.s[4], A.c[4], vx * p.v);
}

// The objective of a single system, f = (1/T) sum_i V_i - 3 kB sum_i x_i
// ln sigma_i (minimizer.cpp:353), in one launch: every block sums a
// stride of the per-site terms and the last block to finish adds the block
// sums (15 us at 262,144 sites on a GB300, where the two-kernel FP64
// reduction the plain form keeps took 18 us; appended to k_grad_once the
// same tail cost its main loop 8%, to k_grad_recv 25 us).  The sums do not
// depend on the order of their terms, so neither the tile, the grid nor
// the order in which blocks finish changes a bit: every term is added as a
// 64.64 fixed-point number (a signed 128-bit integer in units of 2^-64,
// exact integer adds; a term's bits below 2^-64 are dropped, some 1e-19
// eV); terms of magnitude 2^40 or more or not finite go to plain double
// sums that then decide f (a state no minimization reaches; their order
// follows the blocks').  The last block resets the counter for the next
// launch and, for a host-pointer call, writes f and the status word to
// pinned memory.
struct Fix {
  unsigned long long lo;
  long long hi;
};
__device__ __forceinline__ Fix fix_add(Fix a, Fix b) {
  Fix r;
  r.lo = a.lo + b.lo;
  r.hi = a.hi + b.hi + (r.lo < a.lo ? 1 : 0);
  return r;
}
// A double of magnitude below 2^40 (biased exponent e < 1063) as 64.64
// fixed point, its magnitude truncated to a multiple of 2^-64, from its bits
// with integer operations only (GB300's FP64 pipe is narrow): v = m
// 2^(e - 1075) with the 53-bit significand m, i.e. m 2^(e - 1011) units.
__device__ __forceinline__ Fix fix_of_bits(unsigned long long b, int e) {
  if (e == 0) return Fix{0ull, 0ll};  // zero or subnormal: below one unit
  const unsigned long long m = (b & 0xfffffffffffffull) | 0x10000000000000ull;
  const int sh = e - 1011;  // below 52 for e < 1063
  unsigned long long lo, hi;
  if (sh >= 0) {
    lo = m << sh;
    hi = sh ? m >> (64 - sh) : 0ull;
  } else {
    lo = sh > -64 ? m >> -sh : 0ull;
    hi = 0ull;
  }
  if (b >> 63) {  // two's complement of the 128-bit magnitude
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0ull ? 1ull : 0ull);
  }
  return Fix{lo, (long long)hi};
}
__device__ __forceinline__ double fix_value(Fix a) { return (double)a.hi + (double)a.lo * 5.421010862427522e-20; }
struct ObjSum {
  Fix v, s;       // sum V, sum x ln sigma
  double bv, bs;  // their terms left out of the fixed-point sums
};
__device__ __forceinline__ void obj_term(ObjSum &o, double v, bool second) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ffu);
  if (e < 1063) {  // |v| < 2^40 (2^23 such terms still fit); not NaN or infinite
    const Fix f = fix_of_bits(b, e);
    if (second) o.s = fix_add(o.s, f);
    else o.v = fix_add(o.v, f);
  } else if (second) {
    o.bs += v;
  } else {
    o.bv += v;
  }
}
__device__ __forceinline__ ObjSum obj_add(ObjSum a, const ObjSum &b) {
  a.v = fix_add(a.v, b.v);
  a.s = fix_add(a.s, b.s);
  a.bv += b.bv;
  a.bs += b.bs;
  return a;
}
__device__ __forceinline__ ObjSum obj_shfl(const ObjSum &a, int o) {
  ObjSum r;
  r.v.lo = __shfl_xor_sync(0xffffffffu, a.v.lo, o);
  r.v.hi = __shfl_xor_sync(0xffffffffu, a.v.hi, o);
  r.s.lo = __shfl_xor_sync(0xffffffffu, a.s.lo, o);
  r.s.hi = __shfl_xor_sync(0xffffffffu, a.s.hi, o);
  r.bv = __shfl_xor_sync(0xffffffffu, a.bv, o);
  r.bs = __shfl_xor_sync(0xffffffffu, a.bs, o);
  return r;
}
// the block's sum, in thread 0
__device__ __forceinline__ ObjSum obj_block(ObjSum a, ObjSum *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = obj_add(a, obj_shfl(a, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = a;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) a = obj_add(a, sh[k]);
  __syncthreads();
  return a;
}

__global__ void __launch_bounds__(kBlock) k_objective(MixArgs a) {
  __shared__ ObjSum sh[32];
  __shared__ bool last;
  ObjSum o{};
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < a.N; s += (int64_t)gridDim.x * blockDim.x) {
    obj_term(o, a.Vs[s], false);
    obj_term(o, a.Ss[s], true);
  }
  o = obj_block(o, sh);
  if (threadIdx.x == 0) {
    a.fpart[blockIdx.x] = o;
    __threadfence();
    last = atomicAdd(a.fcount, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  ObjSum t{};
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
    const volatile ObjSum *q = a.fpart + i;
    ObjSum b;
    b.v.lo = q->v.lo;
    b.v.hi = q->v.hi;
    b.s.lo = q->s.lo;
    b.s.hi = q->s.hi;
    b.bv = q->bv;
    b.bs = q->bs;
    t = obj_add(t, b);
  }
  t = obj_block(t, sh);
  if (threadIdx.x == 0) {
    const double sa = fix_value(t.v) + t.bv, sb = fix_value(t.s) + t.bs;
    const double f = 1.0 / a.T * sa - 3.0 * kB * sb;
    *a.f = f;
    a.fsums[0] = sa;
    a.fsums[1] = sb;
    *a.fcount = 0u;
    if (a.hout) {  // every other kernel of the evaluation has finished: its status bits are in
      a.hout[0] = f;
      *reinterpret_cast<int *>(a.hout + 1) = atomicExch(a.status, 0);
    }
  }
}

template <int TPS, bool LIST, int BLOCK>
__global__ void __launch_bounds__(BLOCK, grad_min_blocks<BLOCK>()) k_grad_mixed(MixArgs a) {
  constexpr int kSitesPerBlock = BLOCK / TPS;
  const int64_t n = LIST ? (int64_t)*a.bv.count : a.N;
  if ((int64_t)blockIdx.x * kSitesPerBlock >= n) return;
  extern __shared__ float4 sTab[];  // f_Pd' quadratics, then phi_Pd cubics, kGradCopies-way interleaved
  for (int i = threadIdx.x; i < kGradTabN * kGradCopies; i += blockDim.x) {
    sTab[i] = __ldg(&a.tabPair[2 * kTabN + i / kGradCopies]);
    sTab[kGradTabN * kGradCopies + i] = __ldg(&a.tabPair[kTabN + i / kGradCopies]);
  }
  __syncthreads();
  const float4 *sF = sTab + threadIdx.x % kGradCopies, *sP = sF + kGradTabN * kGradCopies;
  for (int64_t base = (int64_t)blockIdx.x * kSitesPerBlock; base < n;
       base += (int64_t)gridDim.x * kSitesPerBlock) {
  const int64_t k = base + threadIdx.x / TPS;
  const int lane = (int)(threadIdx.x % TPS);
  const bool live = k < n;
  SiteRef<LIST> R{};
  if (live) R = site_ref<LIST>(a, k);
  const int64_t s = R.s;
  SiteAcc A;
#pragma unroll
  for (int k = 0; k < 5; ++k) A.s[k] = A.c[k] = 0.0f;
  float xi = 0.0f, sigi = 1.0f;
  float2 ffi = make_float2(0.0f, 0.0f);
  if (live) {
    const int4 pi = a.P[s];
    sigi = __int_as_float(pi.w);
    const float ui = kSqrt6 * sigi;
    xi = a.occ[s];
    ffi = a.FF[s];
    const bool iPd = R.iPd;
    const int64_t b = a.off[s], m = b + a.npd[s], e = a.off[s + 1];
    const float hw = 0.5f * a.W * xi;
    walk_neighbors<false, true>(a, b + lane, m, TPS, [&](int64_t, int4 pj, float, float Fb) {  // Pd neighbors
      const float3 D = pair_vec(R.sc, pi, pj);
      const float uj = kSqrt6 * __int_as_float(pj.w);
      PairAcc p;
      if (iPd) {
        pair_terms<0>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, p);
      } else if (pair_inside(D, ui, uj)) {
        pair_terms<2, false>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, p);
      } else {
        pair_terms<2, true>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, p);
      }
      add_pair(A, p, D, a.W, hw);
    });
    walk_neighbors<true, true>(a, m + lane, e, TPS, [&](int64_t, int4 pj, float xj, float Fb) {  // H neighbors
      const float3 D = pair_vec(R.sc, pi, pj);
      const float uj = kSqrt6 * __int_as_float(pj.w);
      PairAcc p;
      const bool in = pair_inside(D, ui, uj);
      if (iPd) {
        if (in) pair_terms<1, false>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, p);
        else pair_terms<1, true>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, p);
      } else {
        if (in) pair_terms<3, false>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, p);
        else pair_terms<3, true>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, p);
      }
      add_pair(A, p, D, a.W * xj, hw * xj);
    });
  }
  double tot[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    float v = A.s[k] - A.c[k];
#pragma unroll
    for (int o = TPS / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    tot[k] = (double)v;
  }
  if (live && lane == 0) {
    const double x = xi, sg = sigi, invT = 1.0 / R.T;
    a.G[4 * s] = tot[0] * (invT * x);
    a.G[4 * s + 1] = tot[1] * (invT * x);
    a.G[4 * s + 2] = tot[2] * (invT * x);
    a.G[4 * s + 3] = tot[3] * (1.7320508075688772 * 1.4142135623730951 * invT * x) - 3.0 * kB / sg * x;
    a.Vs[s] = x * (double)ffi.y + tot[4];
    a.Ss[s] = (double)logf(sigi) * x;
  }
  }
}

// ------------------------------------------------- pass 2, pairs once
// The pair (i, j) with j < i is evaluated by site i alone: i keeps its share
// (with the pair's whole energy, W x_i x_j sum_k phi) and stores j's share
// -- W x_i (-(D sum_k c_k + e), sigj), the same c_k seen from j -- in the
// slot of j's list that holds i (rev).  k_grad_recv then adds to every site
// the shares stored in its own list, in list order.  Lists are sorted by
// id, so a site's owned entries are the first npre of its list; Pd ids
// precede H ids, so a Pd site owns Pd neighbors only and the pair types are
// Pd-Pd (a Pd site), H-Pd and H-H (an H site).
// slot: the reverse entry, loaded when the pair starts so its latency
// overlaps the pair's arithmetic (measured 1% on pass 2)
__device__ __forceinline__ void send_share(const MixArgs &a, uint32_t slot, const PairAcc &p, float3 D, float w) {
  a.recv[slot] = make_float4(-w * fmaf(D.x, p.csum, p.e[0]), -w * fmaf(D.y, p.csum, p.e[1]),
                             -w * fmaf(D.z, p.csum, p.e[2]), w * p.sigj);
}

template <int TPS, bool LIST, int BLOCK>
__global__ void __launch_bounds__(BLOCK, grad_min_blocks<BLOCK>()) k_grad_once(MixArgs a) {
  constexpr int kSitesPerBlock = BLOCK / TPS;
  const int64_t n = LIST ? (int64_t)*a.bv.count : a.N;
  if ((int64_t)blockIdx.x * kSitesPerBlock >= n) return;
  extern __shared__ float4 sTab[];  // f_Pd' quadratics, then phi_Pd cubics, kGradCopies-way interleaved
  for (int i = threadIdx.x; i < kGradTabN * kGradCopies; i += blockDim.x) {
    sTab[i] = __ldg(&a.tabPair[2 * kTabN + i / kGradCopies]);
    sTab[kGradTabN * kGradCopies + i] = __ldg(&a.tabPair[kTabN + i / kGradCopies]);
  }
  __syncthreads();
  const float4 *sF = sTab + threadIdx.x % kGradCopies, *sP = sF + kGradTabN * kGradCopies;
  for (int64_t base = (int64_t)blockIdx.x * kSitesPerBlock; base < n;
       base += (int64_t)gridDim.x * kSitesPerBlock) {
  const int64_t k = base + threadIdx.x / TPS;
  const int lane = (int)(threadIdx.x % TPS);
  const bool live = k < n;
  SiteRef<LIST> R{};
  if (live) R = site_ref<LIST>(a, k);
  const int64_t s = R.s;
  SiteAcc A;
#pragma unroll
  for (int k = 0; k < 5; ++k) A.s[k] = A.c[k] = 0.0f;
  float xi = 0.0f, sigi = 1.0f;
  float2 ffi = make_float2(0.0f, 0.0f);
  if (live) {
    const int4 pi = a.P[s];
    sigi = __int_as_float(pi.w);
    const float ui = kSqrt6 * sigi;
    xi = a.occ[s];
    ffi = a.FF[s];
    const bool iPd = R.iPd;
    const int64_t b = a.off[s], m = b + a.npd[s], p = b + a.npre[s];
    const float w = a.W * xi;  // the neighbor's share and the pair energy carry W x_i
    walk_neighbors<false, true>(a, b + lane, m < p ? m : p, TPS, [&](int64_t t, int4 pj, float, float Fb) {
      const uint32_t slot = __ldg(&a.rev[t]);
      const float3 D = pair_vec(R.sc, pi, pj);
      const float uj = kSqrt6 * __int_as_float(pj.w);
      PairAcc q;
      if (iPd) {
        pair_terms<0>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, q);
      } else if (pair_inside(D, ui, uj)) {
        pair_terms<2, false>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, q);
      } else {
        pair_terms<2, true>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, q);
      }
      add_pair(A, q, D, a.W, w);
      send_share(a, slot, q, D, w);
    });
    walk_neighbors<true, true>(a, m + lane, p, TPS, [&](int64_t t, int4 pj, float xj, float Fb) {  // H site, H j < i
      const uint32_t slot = __ldg(&a.rev[t]);
      const float3 D = pair_vec(R.sc, pi, pj);
      const float uj = kSqrt6 * __int_as_float(pj.w);
      PairAcc q;
      if (pair_inside(D, ui, uj)) pair_terms<3, false>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, q);
      else pair_terms<3, true>(a.ex, sF, sP, ffi.x, Fb, D, ui, uj, q);
      add_pair(A, q, D, a.W * xj, w * xj);
      send_share(a, slot, q, D, w);
    });
  }
  double tot[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    float v = A.s[k] - A.c[k];
#pragma unroll
    for (int o = TPS / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    tot[k] = (double)v;
  }
  if (live && lane == 0) {  // the site's own share (16-byte stores: Gown is the library's); k_grad_recv completes G
    const double x = xi, sg = sigi, invT = 1.0 / R.T;
    double2 *own = reinterpret_cast<double2 *>(a.Gown + 4 * s);
    own[0] = make_double2(tot[0] * (invT * x), tot[1] * (invT * x));
    own[1] = make_double2(tot[2] * (invT * x),
                          tot[3] * (1.7320508075688772 * 1.4142135623730951 * invT * x) - 3.0 * kB / sg * x);
    a.Vs[s] = x * (double)ffi.y + tot[4];
    a.Ss[s] = (double)logf(sigi) * x;
  }
  }
}

// The shares a site received (its list entries after the first npre),
// summed in list order with compensation and added to its own share: G is
// written once (it may be the caller's host-mapped memory).
template <int TPS, bool LIST>
__global__ void __launch_bounds__(kBlock) k_grad_recv(MixArgs a) {
  constexpr int kSitesPerBlock = kBlock / TPS;
  const int64_t n = LIST ? (int64_t)*a.bv.count : a.N;
  for (int64_t base = (int64_t)blockIdx.x * kSitesPerBlock; base < n;
       base += (int64_t)gridDim.x * kSitesPerBlock) {
    const int64_t k = base + threadIdx.x / TPS;
    const int lane = (int)(threadIdx.x % TPS);
    const bool live = k < n;
    SiteRef<LIST> R{};
    if (live) R = site_ref<LIST>(a, k);
    const int64_t s = R.s;
    float sum[4] = {0.0f, 0.0f, 0.0f, 0.0f}, cmp[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (live) {
      const int64_t e = a.off[s + 1];
      for (int64_t t = a.off[s] + a.npre[s] + lane; t < e; t += TPS) {
        const float4 v = __ldcs(&a.recv[t]);
        kahan(sum[0], cmp[0], v.x);
        kahan(sum[1], cmp[1], v.y);
        kahan(sum[2], cmp[2], v.z);
        kahan(sum[3], cmp[3], v.w);
      }
    }
    double tot[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float v = sum[c] - cmp[c];
#pragma unroll
      for (int o = TPS / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      tot[c] = (double)v;
    }
    // lanes 0-3 of the site write one component each: the sites of a warp
    // store one contiguous run of G (the caller's memory may be host-mapped,
    // where scattered 8-byte stores are slow)
    static_assert(TPS >= 4, "one lane per gradient component");
    if (live && lane < 4) {
      const double x = a.occ[s], invT = 1.0 / R.T;
      const double v = lane == 0 ? tot[0] : lane == 1 ? tot[1] : lane == 2 ? tot[2] : tot[3];
      const double scale = lane == 3 ? 1.7320508075688772 * 1.4142135623730951 * invT * x : invT * x;
      a.G[4 * s + lane] = a.Gown[4 * s + lane] + v * scale;
    }
  }
}

// Chemical potential of the H sites in the mixed form (the DMD loop's
// step after each minimization; minimizer.cpp:658-789): per H site the
// quadrature sums  sum_{j in HPd} sum_k W [F'_Pd(rho_j) f_H(s) + phi_PdH(s)]
// and  sum_{j in HH} x_j sum_k W [F'_H(rho_j) f_H(s) + phi_H(s)]  in FP32 with
// compensated sums over neighbors (F' and F from pass 1 of the same state),
// then F_H(rho_i), the correction terms (FP64; zero unless coe_* are set)
// and log(x/(1-x)) + chi/(kB T) in FP64.  One thread per H site; send as in
// k_chem64.
__global__ void __launch_bounds__(kBlock) k_chem_mixed(MixArgs a, int nH, double coePd0, double coePd2, double coePd3,
                                                       double coeH0, double coeH1, double coeH2, double coeH3,
                                                       const double *occ64, const int *full, double *send) {
  const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= nH) return;
  send[h] = 0.0;
  if (full[h] == 1) return;
  const int64_t s = (int64_t)a.nPd + h;
  const int4 pi = a.P[s];
  const float ui = kSqrt6 * __int_as_float(pi.w), ui2 = ui * ui;
  const float3 sc = make_float3(a.sc[0], a.sc[1], a.sc[2]);
  const int64_t b = a.off[s], m = b + a.npd[s], e = a.off[s + 1];
  float acc = 0.0f, cmp = 0.0f;
  for (int64_t t = b; t < e; ++t) {
    const int64_t j = __ldg(&a.nbr[t]) & kIdMask;
    const int4 pj = __ldg(&a.P[j]);
    const float3 D = pair_vec(sc, pi, pj);
    const float uj = kSqrt6 * __int_as_float(pj.w);
    const float D2 = fmaf(D.x, D.x, fmaf(D.y, D.y, D.z * D.z));
    const float Ai = D2 + ui2, Aj = fmaf(uj, uj, D2);
    const float Fj = __ldg(&a.FF[j].x);
    const bool jPd = t < m;
    const MorseExp &mo = jPd ? a.ex.pdh : a.ex.hh;
    float part = 0.0f;
    const float Dv[3] = {D.x, D.y, D.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      A2C_RADII(c, Dv[c])
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float r = s2[q] * rsq(s2[q]);
        float phi, dphi;
        morse(mo, r, phi, dphi);
        part += fmaf(Fj, fH(a.ex, r), phi);
      }
    }
    kahan(acc, cmp, part * (jPd ? a.W : a.W * __ldg(&a.occ[j])));
  }
  const double T = a.T;
  double sum = (double)a.FF[s].y + (double)(acc - cmp);
  if (coeH0 != 0.0 || coeH1 != 0.0 || coeH2 != 0.0 || coeH3 != 0.0 || coePd0 != 0.0) {
    // the correction terms (minimizer.cpp:667-719), in FP64
    const double nHPd = (double)(m - b);
    double xs = 0.0;
    for (int64_t t = m; t < e; ++t) xs += occ64[a.nbr[t] & kIdMask];
    const double tmp = (coeH1 * nHPd) * nHPd + (2.0 * coeH2) * nHPd * xs + coeH3 * xs * xs;
    sum += ((0.5 * T) * coeH0) * tmp;
    for (int64_t t = b; t < e; ++t) {
      const int64_t j = a.nbr[t] & kIdMask;
      const int64_t bj = a.off[j], mj = bj + a.npd[j], ej = a.off[j + 1];
      double xl = 0.0;
      for (int64_t u = mj; u < ej; ++u) xl += occ64[a.nbr[u] & kIdMask];
      if (t < m) sum += ((T * coePd0) * coePd2) * (double)(mj - bj) + ((T * coePd0) * coePd3) * xl;
      else sum += occ64[j] * T * coeH0 * (coeH2 * (double)(mj - bj) + coeH3 * xl);
    }
  }
  const double x0 = occ64[s];
  if (x0 > 0.0 && x0 < 1.0) send[h] = dd::cr_log(x0 / (1.0 - x0)) + sum / (kB * T);
}

// The index of the pairs-once scheme for lists off/nbr over sites [0, N):
// per site the count of neighbors with a smaller id (npre), per owned entry
// the slot of the reverse entry (rev).  Sets *bad when a list is not
// strictly increasing, holds the site itself or an id out of range, or
// lacks the reverse of an entry (asymmetric lists).  kSymLanes lanes per
// site share its entries, so the reverse searches (a chain of dependent
// loads each) of one site run side by side.
constexpr int kSymLanes = 8;
__global__ void k_sym_index(int64_t N, const int64_t *off, const uint32_t *nbr, uint32_t *rev, int *npre, int *bad) {
  const int lane = (int)(threadIdx.x % kSymLanes);
  const unsigned group = 0xffu << ((threadIdx.x % 32) & ~(kSymLanes - 1));  // this site's lanes in the warp
  const int64_t stride = (int64_t)gridDim.x * (blockDim.x / kSymLanes);
  for (int64_t s = (int64_t)blockIdx.x * (blockDim.x / kSymLanes) + threadIdx.x / kSymLanes; s < N; s += stride) {
    const int64_t b = off[s], e = off[s + 1];
    int below = 0;  // entries with an id below s: the owned head of a sorted list
    bool ok = true;
    for (int64_t t = b + lane; t < e; t += kSymLanes) {
      const uint32_t id = nbr[t] & kIdMask;
      if ((t > b && id <= (nbr[t - 1] & kIdMask)) || (int64_t)id == s || (int64_t)id >= N) ok = false;
      below += (int64_t)id < s;
    }
#pragma unroll
    for (int o = kSymLanes / 2; o > 0; o >>= 1) below += __shfl_xor_sync(group, below, o);
    ok = __all_sync(group, ok);
    const int64_t p = b + below;
    if (lane == 0) npre[s] = below;
    if (!ok) {
      if (lane == 0) atomicOr(bad, 1);
      continue;
    }
    for (int64_t t = b + lane; t < p; t += kSymLanes) {
      const int64_t j = nbr[t] & kIdMask;
      int64_t lo = off[j], hi = off[j + 1];
      while (lo < hi) {  // first entry of j's list with id >= s
        const int64_t mid = lo + ((hi - lo) >> 1);
        if ((int64_t)(nbr[mid] & kIdMask) < s) lo = mid + 1;
        else hi = mid;
      }
      if (lo >= off[j + 1] || (int64_t)(nbr[lo] & kIdMask) != s) {
        atomicOr(bad, 1);
        break;
      }
      rev[t] = (uint32_t)lo;
    }
  }
}

// Span guard (free directions only; xl null when every direction is
// periodic): a site more than lim from the position its lists were built at
// could make a listed pair leave the fixed-point span, where the encoded
// difference would wrap.  Flag it; the caller gets A2C_ERR_LISTS_STALE.
__device__ __forceinline__ void span_check(const double4 &x, const double *xl, int64_t s, double l0, double l1,
                                           double l2, int *status) {
  if (!xl) return;
  const double4 r = *reinterpret_cast<const double4 *>(xl + 4 * s);
  if (fabs(x.x - r.x) > l0 || fabs(x.y - r.y) > l1 || fabs(x.z - r.z) > l2) atomicOr(status, kStatusSpan);
}

struct SpanArgs {
  const double *xl;  // list positions (4N), null when all directions are periodic
  double lim[3];
  int *status;
};

__global__ void k_prep(const double *X, const double *occ, int64_t N, double k0, double k1, double k2, int4 *P,
                       float *occf, SpanArgs sg) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N) return;
  const double4 x = make_double4(X[4 * s], X[4 * s + 1], X[4 * s + 2], X[4 * s + 3]);
  span_check(x, sg.xl, s, sg.lim[0], sg.lim[1], sg.lim[2], sg.status);
  const long long u0 = __double2ll_rn(x.x * k0);
  const long long u1 = __double2ll_rn(x.y * k1);
  const long long u2 = __double2ll_rn(x.z * k2);
  P[s] = make_int4((int)(unsigned)u0, (int)(unsigned)u1, (int)(unsigned)u2, __float_as_int((float)x.w));
  occf[s] = (float)occ[s];
}

// The same, reading X from the caller's pinned host memory over the
// coherent host link: also keeps the context's device copy of the state and
// flags non-finite inputs (what a separate copy and check would do).
__global__ void k_prep_copy(const double *X, const double *occ, int64_t N, double k0, double k1, double k2, int4 *P,
                            float *occf, double *Xcopy, SpanArgs sg) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N) return;
  const double4 x = *reinterpret_cast<const double4 *>(X + 4 * s);
  *reinterpret_cast<double4 *>(Xcopy + 4 * s) = x;
  if (!isfinite(x.x) || !isfinite(x.y) || !isfinite(x.z) || !isfinite(x.w)) atomicOr(sg.status, kStatusNonfinite);
  span_check(x, sg.xl, s, sg.lim[0], sg.lim[1], sg.lim[2], sg.status);
  const long long u0 = __double2ll_rn(x.x * k0);
  const long long u1 = __double2ll_rn(x.y * k1);
  const long long u2 = __double2ll_rn(x.z * k2);
  P[s] = make_int4((int)(unsigned)u0, (int)(unsigned)u1, (int)(unsigned)u2, __float_as_int((float)x.w));
  occf[s] = (float)occ[s];
}

// Batched: positions of the listed sites with their instance's scale (and
// its span-guard limits; xl null when no instance has a free direction).
__global__ void k_prep_list(const double *X, const double *occ, BatchView bv, int4 *P, float *occf, const double *xl,
                            int *status) {
  const int n = *bv.count;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int64_t s = bv.list[k];
    const InstGeo &g = bv.geo[bv.inst[s]];
    const double4 x = make_double4(X[4 * s], X[4 * s + 1], X[4 * s + 2], X[4 * s + 3]);
    span_check(x, xl, s, g.lim[0], g.lim[1], g.lim[2], status);
    const long long u0 = __double2ll_rn(x.x * (4294967296.0 / g.S[0]));
    const long long u1 = __double2ll_rn(x.y * (4294967296.0 / g.S[1]));
    const long long u2 = __double2ll_rn(x.z * (4294967296.0 / g.S[2]));
    P[s] = make_int4((int)(unsigned)u0, (int)(unsigned)u1, (int)(unsigned)u2, __float_as_int((float)x.w));
    occf[s] = (float)occ[s];
  }
}

SpanArgs span_args(const a2c_gpp_ctx *c) {
  SpanArgs sg;
  span_limits(c, sg.lim, &sg.xl);
  sg.status = c->d_status;
  return sg;
}

// Persistent grids: as many blocks as fit on the device at once (occupancy
// query, cached per kernel), capped by the work (for a list launch, by the
// largest list the system can have).
// The folded exponential constants (see ExpTerms) from the reference's
// parameters: f_H C = 11.0025, delta = 1.30927 (potential.cpp:105-119);
// phi_PdH and phi_H D, a, b, r0 and the tail funRc, funRc' at 5.35 A
// (potential.cpp:162-200).
MorseExp morse_exp(double D, double a, double b, double r0, double funRc, double dfunRc) {
  constexpr double kL2E = 1.4426950408889634, kRc = 5.35;
  const double K1 = -a * kL2E, K2 = -b * kL2E, k = dfunRc / funRc, Kt = k * kL2E;
  MorseExp m;
  m.K1 = (float)K1;
  m.C1 = (float)(std::log2(D * b) - K1 * r0);
  m.L1 = (float)(-a);
  m.K2 = (float)K2;
  m.C2 = (float)(std::log2(D * a) - K2 * r0);
  m.L2 = (float)b;
  m.Kt = (float)Kt;
  m.Ct = (float)(std::log2(-funRc) - Kt * kRc);
  m.Lt = (float)(-k);
  return m;
}
ExpTerms exp_terms() {
  constexpr double kL2E = 1.4426950408889634, kC = 11.0025, kDelta = 1.30927;
  ExpTerms x;
  x.fK = (float)(-kDelta * kL2E);
  x.fC = (float)std::log2(kC);
  x.fdC = (float)std::log2(kC * kDelta);
  x.pdh = morse_exp(0.2494540, 4.82613, 2.13158, 1.50964, -3.353001113951400e-04, 7.147062196813336e-04);
  x.hh = morse_exp(0.0661496, 3.67263, 1.47797, 2.51980, -0.003702722457147, 0.005465945471933);
  return x;
}
const ExpTerms &exp_consts() {
  static const ExpTerms x = exp_terms();
  return x;
}

// once = true: pass 2 evaluates every pair once (k_grad_once + k_grad_recv;
// a.rev, a.npre, a.recv set), else from both sides (k_grad_mixed).  Pass 1
// evaluates its pairs from both sides: a pairs-once pass 1 (a 4-byte
// density share per pair, scattered to the neighbor's slot, and a receive
// kernel) measured slower on a GB300 at 262,144 sites (0.184 against 0.139
// ms at 2 threads per site) -- its share traffic costs more than the
// arithmetic it saves.
constexpr int kRecvTps = 8;  // lanes per site summing the received shares
// k_objective's grid: blocks per SM at most (at 262,144 sites 2 per SM took
// 12.3 us, 8 per SM 17.9 us: the last-block count is one contended atomic)
constexpr int kObjBlocksPerSm = 2;
// Persistent grid size of a kernel at a block size on the current device
// (resident blocks x SMs), computed once per (kernel, block, device) under
// a lock, with the dynamic shared-memory limit raised on that device first.
int grid_cap(const void *fn, int block, size_t smem) {
  struct Entry {
    const void *fn;
    int dev, block, cap;
  };
  static std::mutex m;
  static std::vector<Entry> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  std::lock_guard<std::mutex> lock(m);
  for (const Entry &e : cache)
    if (e.fn == fn && e.dev == dev && e.block == block) return e.cap;
  int nb = 0;
  if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, block, smem);
  (void)cudaGetLastError();
  if (nb < 1) return 1;  // not cached: asked again next time
  cache.push_back({fn, dev, block, nb * device_sms(dev)});
  return cache.back().cap;
}

inline unsigned persistent_grid(int64_t n_items, int per_block, int cap) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n_items + per_block - 1) / per_block, cap));
}

template <int TPS, bool LIST, int B>
void launch_rho(const MixArgs &a, cudaStream_t st) {
  const void *fn = (const void *)k_rho_mixed<TPS, LIST, B>;
  k_rho_mixed<TPS, LIST, B><<<persistent_grid(a.N, B / TPS, grid_cap(fn, B, kRhoSmem)), B, kRhoSmem, st>>>(a);
}
template <int TPS, bool LIST, int B>
void launch_grad(const MixArgs &a, cudaStream_t st, bool once) {
  if (once) {
    const void *fn = (const void *)k_grad_once<TPS, LIST, B>;
    k_grad_once<TPS, LIST, B><<<persistent_grid(a.N, B / TPS, grid_cap(fn, B, kGradSmem)), B, kGradSmem, st>>>(a);
  } else {
    const void *fn = (const void *)k_grad_mixed<TPS, LIST, B>;
    k_grad_mixed<TPS, LIST, B><<<persistent_grid(a.N, B / TPS, grid_cap(fn, B, kGradSmem)), B, kGradSmem, st>>>(a);
  }
}

template <int TPS, bool LIST>
void launch_pair_kernels(const MixArgs &a, cudaStream_t st, cudaEvent_t *ev, bool once, const Tile &t) {
  switch (t.rho_block) {
    case 512: launch_rho<TPS, LIST, 512>(a, st); break;
    case 768: launch_rho<TPS, LIST, 768>(a, st); break;
    default: launch_rho<TPS, LIST, 256>(a, st); break;
  }
  if (ev) cudaEventRecord(ev[2], st);
  switch (t.grad_block) {
    case 128: launch_grad<TPS, LIST, 128>(a, st, once); break;
    case 512: launch_grad<TPS, LIST, 512>(a, st, once); break;
    default: launch_grad<TPS, LIST, 256>(a, st, once); break;
  }
  if (once) {
    const void *fn = (const void *)k_grad_recv<kRecvTps, LIST>;
    k_grad_recv<kRecvTps, LIST><<<persistent_grid(a.N, kBlock / kRecvTps, grid_cap(fn, kBlock, 0)), kBlock, 0, st>>>(a);
  }
  if (ev) cudaEventRecord(ev[3], st);
}

// Dispatch on threads per site.
void launch_tile(const MixArgs &a, cudaStream_t st, cudaEvent_t *ev, bool once, const Tile &t, bool list) {
  if (list) {
    switch (t.tps) {
      case 1: launch_pair_kernels<1, true>(a, st, ev, once, t); break;
      case 2: launch_pair_kernels<2, true>(a, st, ev, once, t); break;
      case 4: launch_pair_kernels<4, true>(a, st, ev, once, t); break;
      default: launch_pair_kernels<8, true>(a, st, ev, once, t); break;
    }
  } else {
    switch (t.tps) {
      case 1: launch_pair_kernels<1, false>(a, st, ev, once, t); break;
      case 2: launch_pair_kernels<2, false>(a, st, ev, once, t); break;
      case 4: launch_pair_kernels<4, false>(a, st, ev, once, t); break;
      default: launch_pair_kernels<8, false>(a, st, ev, once, t); break;
    }
  }
}

// The pair tables as the kernels read them (3 kTabN float4): the f_Pd
// cubics (pass 1), the phi_Pd cubics, and the f_Pd' quadratics
// (c1, 2 c2, 3 c3) of pass 2, which needs only the derivative.
void pair_tables(float *out) {
  static std::mutex m;  // guards the static scratch below
  std::lock_guard<std::mutex> lock(m);
  static float inter[8 * kTabN];
  build_pair_table_raw(kTabR0, 1.0 / kTabInvH, kTabN, inter);
  for (int i = 0; i < kTabN; ++i) {
    const float *f = inter + 8 * i, *p = inter + 8 * i + 4;
    for (int k = 0; k < 4; ++k) {
      out[4 * i + k] = f[k];
      out[4 * (kTabN + i) + k] = p[k];
    }
    float *d = out + 4 * (2 * kTabN + i);
    d[0] = f[1];
    d[1] = 2.0f * f[2];
    d[2] = 3.0f * f[3];
    d[3] = 0.0f;
  }
}

a2c_status ensure_mixed(a2c_gpp_ctx *c) {
  if (c->mixed && c->mixed->N == c->N) return A2C_OK;
  mixed_free(c);
  Mixed *M = new Mixed;
  c->mixed = M;
  M->N = c->N;
  const int64_t n = std::max<int64_t>(c->N, 1);
  if (cudaMalloc(&M->P, sizeof(int4) * n) != cudaSuccess || cudaMalloc(&M->occ, sizeof(float) * n) != cudaSuccess ||
      cudaMalloc(&M->FF, sizeof(float2) * n) != cudaSuccess ||
      cudaMalloc(&M->tabPair, sizeof(float4) * 3 * kTabN) != cudaSuccess ||
      cudaMalloc(&M->tabEmb, sizeof(float4) * 2 * kEmbN) != cudaSuccess)
    return A2C_ERR_NOMEM;
  if (cudaMalloc(&M->fpart, sizeof(ObjSum) * kObjBlocksPerSm * device_sms(c->device)) != cudaSuccess ||
      cudaMalloc(&M->fcount, sizeof(unsigned)) != cudaSuccess)
    return A2C_ERR_NOMEM;
  A2C_CUDA(cudaMemsetAsync(M->fcount, 0, sizeof(unsigned), c->stream));
  std::vector<float> pair((size_t)12 * kTabN), embPd, embH;
  pair_tables(pair.data());
  build_embed_table(0, 1.0 / kEmbInvH, kEmbN, embPd);
  build_embed_table(1, 1.0 / kEmbInvH, kEmbN, embH);
  A2C_CUDA(cudaMemcpyAsync(M->tabPair, pair.data(), sizeof(float) * pair.size(), cudaMemcpyHostToDevice, c->stream));
  A2C_CUDA(cudaMemcpyAsync(M->tabEmb, embPd.data(), sizeof(float) * embPd.size(), cudaMemcpyHostToDevice, c->stream));
  A2C_CUDA(cudaMemcpyAsync(M->tabEmb + kEmbN, embH.data(), sizeof(float) * embH.size(), cudaMemcpyHostToDevice,
                           c->stream));
  A2C_CUDA(cudaStreamSynchronize(c->stream));  // host vectors go out of scope
  return A2C_OK;
}

// The pairs-once index for the context's current lists (k_sym_index),
// rebuilt when the lists changed.  Lists it cannot serve (unsorted,
// asymmetric, or 2^32 entries and more) and a failed allocation leave
// sym_ok false: pass 2 then visits pairs from both sides.
a2c_status ensure_sym(a2c_gpp_ctx *c) {
  Mixed *M = c->mixed;
  if (M->sym_version == c->nbr_version) return A2C_OK;
  M->sym_ok = false;
  const int64_t N = c->N, E = c->nbr_total;
  cudaStream_t st = c->stream;
  if (N == 0 || E >= (int64_t)0xffffffffLL) {
    M->sym_version = c->nbr_version;
    return A2C_OK;
  }
  if (E > M->sym_entries) {
    if (M->rev) cudaFree(M->rev);
    if (M->recv) cudaFree(M->recv);
    M->rev = nullptr;
    M->recv = nullptr;
    M->sym_entries = 0;
    if (cudaMalloc(&M->rev, sizeof(uint32_t) * E) != cudaSuccess ||
        cudaMalloc(&M->recv, sizeof(float4) * E) != cudaSuccess) {
      (void)cudaGetLastError();  // out of memory: keep the both-sides pass
      M->sym_version = c->nbr_version;
      return A2C_OK;
    }
    M->sym_entries = E;
  }
  if (N + 1 > M->sym_sites) {
    if (M->npre) cudaFree(M->npre);
    if (M->Gown) cudaFree(M->Gown);
    M->npre = nullptr;
    M->Gown = nullptr;
    M->sym_sites = 0;
    if (cudaMalloc(&M->npre, sizeof(int) * (N + 1)) != cudaSuccess ||
        cudaMalloc(&M->Gown, sizeof(double) * 4 * (N + 1)) != cudaSuccess) {
      (void)cudaGetLastError();
      M->sym_version = c->nbr_version;
      return A2C_OK;
    }
    M->sym_sites = N + 1;
  }
  A2C_CUDA(cudaMemsetAsync(M->npre + N, 0, sizeof(int), st));
  const int sms = device_sms(c->device);
  k_sym_index<<<(unsigned)std::min<int64_t>(grid_for(N * kSymLanes, 256), 8 * (int64_t)sms), 256, 0, st>>>(
      N, c->d_off, c->d_nbr, M->rev, M->npre, M->npre + N);
  A2C_CUDA(cudaGetLastError());
  int bad = 1;
  A2C_CUDA(cudaMemcpyAsync(&bad, M->npre + N, sizeof(int), cudaMemcpyDeviceToHost, st));
  A2C_CUDA(cudaStreamSynchronize(st));
  M->sym_ok = bad == 0;
  M->sym_version = c->nbr_version;
  return A2C_OK;
}

// Outside a stream capture: bring the pairs-once index up to date.  Under
// capture the index is used only if it is already current.
a2c_status refresh_sym(a2c_gpp_ctx *c) {
  Mixed *M = c->mixed;
  if (M->pair_mode != A2C_PAIRS_ONCE || M->sym_version == c->nbr_version) return A2C_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  A2C_CUDA(cudaStreamIsCapturing(c->stream, &cs));
  return cs == cudaStreamCaptureStatusNone ? ensure_sym(c) : A2C_OK;
}

bool use_once(const a2c_gpp_ctx *c) {
  const Mixed *M = c->mixed;
  return M->pair_mode == A2C_PAIRS_ONCE && M->sym_ok && M->sym_version == c->nbr_version;
}

}  // namespace

a2c_status mixed_lists_changed(a2c_gpp_ctx *c) {
  if (c->p.precision != A2C_MIXED && !c->mixed) return A2C_OK;
  A2C_TRY(ensure_mixed(c));
  return refresh_sym(c);
}

a2c_status mixed_set_pair_mode(a2c_gpp_ctx *c, int mode) {
  if (mode != A2C_PAIRS_BOTH_SIDES && mode != A2C_PAIRS_ONCE) return A2C_ERR_INVALID;
  A2C_TRY(ensure_mixed(c));
  c->mixed->pair_mode = mode;
  return A2C_OK;
}

a2c_status mixed_get_pair_mode(a2c_gpp_ctx *c, int *mode) {
  A2C_TRY(ensure_mixed(c));
  if (c->has_neighbors) A2C_TRY(refresh_sym(c));
  *mode = (c->has_neighbors && use_once(c)) ? A2C_PAIRS_ONCE : A2C_PAIRS_BOTH_SIDES;
  return A2C_OK;
}

void mixed_free(a2c_gpp_ctx *c) {
  Mixed *M = c->mixed;
  if (!M) return;
  for (void *p : {(void *)M->P, (void *)M->occ, (void *)M->FF, (void *)M->tabPair, (void *)M->tabEmb,
                  (void *)M->rev, (void *)M->npre, (void *)M->recv, (void *)M->Gown, (void *)M->fpart, (void *)M->fcount})
    if (p) cudaFree(p);
  delete M;
  c->mixed = nullptr;
}

int mixed_threads_per_site(a2c_gpp_ctx *c) { return (c->mixed && c->mixed->tps) ? c->mixed->tps : 0; }

Tile effective_tile(const Tile &t, int64_t n_sites, int sms) {
  Tile e;
  e.tps = t.tps ? t.tps : default_threads_per_site(n_sites, sms);
  e.rho_block = t.rho_block ? t.rho_block : kBlock;
  e.grad_block = t.grad_block ? t.grad_block : kBlock;
  return e;
}

Tile mixed_tile(a2c_gpp_ctx *c) {
  Tile t;
  if (c->mixed) {
    t.tps = c->mixed->tps;
    t.rho_block = c->mixed->rho_block;
    t.grad_block = c->mixed->grad_block;
  }
  return t;
}

a2c_status mixed_set_tile(a2c_gpp_ctx *c, const Tile &t) {
  if (!valid_tile(t.tps, t.rho_block, t.grad_block)) return A2C_ERR_INVALID;
  A2C_TRY(ensure_mixed(c));
  c->mixed->tps = t.tps;
  c->mixed->rho_block = t.rho_block;
  c->mixed->grad_block = t.grad_block;
  return A2C_OK;
}

a2c_status mixed_set_threads_per_site(a2c_gpp_ctx *c, int tps) {
  if (tps != 0 && tps != 1 && tps != 2 && tps != 4 && tps != 8) return A2C_ERR_INVALID;
  A2C_TRY(ensure_mixed(c));
  c->mixed->tps = tps;
  return A2C_OK;
}

a2c_status mixed_eval(a2c_gpp_ctx *c, const double *dX, double *d_f, double *dG, cudaEvent_t *ev, double *Xcopy,
                      double *h_out) {
  A2C_TRY(ensure_mixed(c));
  Mixed *M = c->mixed;
  const int64_t N = c->N;
  MixArgs a{};
  a.N = N;
  a.nPd = c->p.nPd;
  a.W = (float)c->p.QWp;
  double k[3];
  for (int d = 0; d < 3; ++d) {
    const double S = c->p.periodic[d] ? c->p.box[d] : kFreeSpan;  // free direction: guarded span (span_check)
    k[d] = 4294967296.0 / S;
    a.sc[d] = (float)(S / 4294967296.0);
  }
  a.P = M->P;
  a.occ = M->occ;
  a.off = c->d_off;
  a.nbr = c->d_nbr;
  a.npd = c->d_npd;
  a.ex = exp_consts();
  a.tabPair = M->tabPair;
  a.tabEmb = M->tabEmb;
  a.FF = M->FF;
  a.G = dG;
  a.Vs = c->d_Vs;
  a.Ss = c->d_Ss;
  a.T = c->p.T;
  if (N > 0) A2C_TRY(refresh_sym(c));
  const bool once = N > 0 && use_once(c);
  a.rev = M->rev;
  a.npre = M->npre;
  a.recv = M->recv;
  a.Gown = M->Gown;
  a.fpart = (ObjSum *)M->fpart;  // k_objective
  a.fcount = M->fcount;
  a.f = d_f;
  a.fsums = c->d_red + 2 * 1024;
  a.hout = h_out;
  a.status = c->d_status;
  if (ev) cudaEventRecord(ev[0], c->stream);
  if (N > 0) {
    const SpanArgs sg = span_args(c);
    if (Xcopy)
      k_prep_copy<<<grid_for(N, 256), 256, 0, c->stream>>>(dX, c->d_occ, N, k[0], k[1], k[2], M->P, M->occ, Xcopy,
                                                           sg);
    else
      k_prep<<<grid_for(N, 256), 256, 0, c->stream>>>(dX, c->d_occ, N, k[0], k[1], k[2], M->P, M->occ, sg);
    A2C_CUDA(cudaGetLastError());
    if (ev) cudaEventRecord(ev[1], c->stream);
    launch_tile(a, c->stream, ev, once, effective_tile(mixed_tile(c), N, device_sms(c->device)), false);
    A2C_CUDA(cudaGetLastError());
  } else if (ev) {
    for (int k2 = 1; k2 < 4; ++k2) cudaEventRecord(ev[k2], c->stream);
  }
  k_objective<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(grid_for(N, kBlock),
                                                                  kObjBlocksPerSm * (int64_t)device_sms(c->device))),
                kBlock, 0, c->stream>>>(a);
  A2C_CUDA(cudaGetLastError());
  if (ev) cudaEventRecord(ev[4], c->stream);
  return A2C_OK;
}

a2c_status mixed_prepare(a2c_gpp_ctx *c) {
  A2C_TRY(ensure_mixed(c));
  return refresh_sym(c);
}

void mixed_graph_key(a2c_gpp_ctx *c, const void *key[5]) {
  const Mixed *M = c->mixed;
  const bool once = M && use_once(c);
  key[0] = once ? (const void *)c : nullptr;
  key[1] = M ? (const void *)M->rev : nullptr;
  key[2] = M ? (const void *)M->npre : nullptr;
  key[3] = M ? (const void *)M->recv : nullptr;
  key[4] = M ? (const void *)M->Gown : nullptr;
}

a2c_status mixed_eval_list(a2c_gpp_ctx *c, const double *dX, double *dG, const BatchView &bv, const Tile &tile) {
  A2C_TRY(ensure_mixed(c));
  Mixed *M = c->mixed;
  const int64_t N = c->N;
  if (N == 0) return A2C_OK;
  MixArgs a{};
  a.N = N;  // upper bound of the list length (sizes the persistent grids)
  a.W = (float)c->p.QWp;
  a.P = M->P;
  a.occ = M->occ;
  a.off = c->d_off;
  a.nbr = c->d_nbr;
  a.npd = c->d_npd;
  a.ex = exp_consts();
  a.tabPair = M->tabPair;
  a.tabEmb = M->tabEmb;
  a.FF = M->FF;
  a.G = dG;
  a.Vs = c->d_Vs;
  a.Ss = c->d_Ss;
  a.bv = bv;
  A2C_TRY(refresh_sym(c));
  const bool once = use_once(c);
  a.rev = M->rev;
  a.npre = M->npre;
  a.recv = M->recv;
  a.Gown = M->Gown;
  const int prep_cap = 8 * device_sms(c->device);
  k_prep_list<<<(unsigned)std::min<int64_t>(grid_for(N, 256), prep_cap), 256, 0, c->stream>>>(
      dX, c->d_occ, bv, M->P, M->occ, c->d_xlist, c->d_status);
  launch_tile(a, c->stream, nullptr, once, effective_tile(tile, N, device_sms(c->device)), true);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

}  // namespace a2c

namespace a2c {

a2c_status mixed_chem(a2c_gpp_ctx *c, const double *dX, double *d_send, const int *d_full) {
  const int nH = c->p.nH;
  if (nH == 0) return A2C_OK;
  A2C_TRY(ensure_mixed(c));
  Mixed *M = c->mixed;
  const int64_t N = c->N;
  MixArgs a{};
  a.N = N;
  a.nPd = c->p.nPd;
  a.W = (float)c->p.QWp;
  double k[3];
  for (int d = 0; d < 3; ++d) {
    const double S = c->p.periodic[d] ? c->p.box[d] : kFreeSpan;
    k[d] = 4294967296.0 / S;
    a.sc[d] = (float)(S / 4294967296.0);
  }
  a.P = M->P;
  a.occ = M->occ;
  a.off = c->d_off;
  a.nbr = c->d_nbr;
  a.npd = c->d_npd;
  a.ex = exp_consts();
  a.tabPair = M->tabPair;
  a.tabEmb = M->tabEmb;
  a.FF = M->FF;
  a.T = c->p.T;
  // the state's fixed-point form and pass 1 (F and F' of every site)
  k_prep<<<grid_for(N, 256), 256, 0, c->stream>>>(dX, c->d_occ, N, k[0], k[1], k[2], M->P, M->occ, span_args(c));
  const Tile t = effective_tile(mixed_tile(c), N, device_sms(c->device));
  switch (t.rho_block) {
    case 512: launch_rho<1, false, 512>(a, c->stream); break;
    case 768: launch_rho<1, false, 768>(a, c->stream); break;
    default: launch_rho<1, false, 256>(a, c->stream); break;
  }
  const double *cp = c->p.coe_Pd, *ch = c->p.coe_H;
  k_chem_mixed<<<grid_for(nH, kBlock), kBlock, 0, c->stream>>>(a, nH, cp[0], cp[2], cp[3], ch[0], ch[1], ch[2], ch[3],
                                                               c->d_occ, d_full, d_send);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

}  // namespace a2c

// ---------------------------------------------------------------------------
// Allocation-free evaluation: a2c_gpp_eval_mixed_noalloc.
//
// For callers that cannot allocate device memory at evaluation time -- a
// host code whose device memory is owned by another allocator (a PETSc or
// solver-framework callback running under its own memory pool), or work
// recorded into a CUDA graph by a driver that forbids allocation while it
// records -- this entry point evaluates the mixed-precision form with all of
// its scratch in one file-scope device array of fixed size instead of
// memory from cudaMalloc.  Every GPU that loads the library holds the array
// (about 5.8 MB) until the process exits.
// ---------------------------------------------------------------------------
namespace a2c {

void build_pair_table_raw(double r0, double h, int n, float *out);
void build_embed_table_raw(int species, double h, int n, float *out);

namespace {

constexpr int64_t kNaMaxSites = 131072;  // the largest problem the fixed scratch holds
constexpr int kNaRedGrid = 1024, kNaRedBlock = 256;
// byte offsets of the scratch regions, each a multiple of 256
constexpr size_t kNaP = 0;
constexpr size_t kNaOcc = kNaP + 16 * (size_t)kNaMaxSites;
constexpr size_t kNaFF = kNaOcc + 4 * (size_t)kNaMaxSites;
constexpr size_t kNaVs = kNaFF + 8 * (size_t)kNaMaxSites;
constexpr size_t kNaSs = kNaVs + 8 * (size_t)kNaMaxSites;
constexpr size_t kNaPart = kNaSs + 8 * (size_t)kNaMaxSites;
constexpr size_t kNaTabPair = kNaPart + 8 * 2 * (size_t)kNaRedGrid;
constexpr size_t kNaTabEmb = kNaTabPair + 16 * 3 * (size_t)kTabN;
constexpr size_t kNaBytes = kNaTabEmb + 16 * 2 * (size_t)kEmbN;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

// Host side, per device: the array's device address and the id of the
// CUDA context it was resolved in.  A context id is never reused, so a
// device reset (a new primary context, with the array's contents lost) is
// seen on the next call, which then resolves the address and loads the
// tables again.
unsigned char *g_na_base[kMaxDevices] = {};
unsigned long long g_na_ctx[kMaxDevices] = {};
std::mutex g_na_mutex;
float g_na_pair_host[12 * kTabN];
float g_na_emb_host[2 * 4 * kEmbN];
bool g_na_host_ready = false;

// The current context's id through the driver entry point (no link-time
// dependency on the driver library); 0 when it cannot be had.
unsigned long long na_context_id() {
  using CtxGetId = int (*)(void *, unsigned long long *);
  static CtxGetId fn = nullptr;
  static bool looked = false;
  if (!looked) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (CtxGetId)p;
    (void)cudaGetLastError();
    looked = true;
  }
  unsigned long long id = 0;
  if (!fn || fn(nullptr, &id) != 0) return 0;
  return id;
}

// Set-up on the current device: resolve the array's device address and
// load the constant function tables into it.  Runs on a device's first
// call, and again after the device's context was replaced.
a2c_status na_setup(int dev, unsigned char **base) {
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (dev < 0 || dev >= kMaxDevices) return A2C_ERR_INVALID;
  const unsigned long long ctx = na_context_id();
  if (g_na_base[dev] && ctx != 0 && ctx == g_na_ctx[dev]) {
    *base = g_na_base[dev];
    return A2C_OK;
  }
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_status(e);
  if (!g_na_host_ready) {
    pair_tables(g_na_pair_host);
    build_embed_table_raw(0, 1.0 / kEmbInvH, kEmbN, g_na_emb_host);
    build_embed_table_raw(1, 1.0 / kEmbInvH, kEmbN, g_na_emb_host + 4 * kEmbN);
    g_na_host_ready = true;
  }
  unsigned char *b = (unsigned char *)ptr;
  e = cudaMemcpy(b + kNaTabPair, g_na_pair_host, sizeof(g_na_pair_host), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b + kNaTabEmb, g_na_emb_host, sizeof(g_na_emb_host), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_status(e);
  g_na_base[dev] = b;
  g_na_ctx[dev] = ctx;  // 0 (no context id available): set up again on every call
  *base = b;
  return A2C_OK;
}

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double na_block_sum(double v, double *sh) {
  v = na_warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
  if (w == 0) v = na_warp_sum(v);
  __syncthreads();
  return v;
}
// The objective reduction (the same fixed-partition tree as the context path)
__global__ void __launch_bounds__(kNaRedBlock) k_na_partial(const double *a, const double *b, int64_t n, double *pa,
                                                             double *pb) {
  __shared__ double sh[kNaRedBlock / 32];
  double sa = 0.0, sb = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    sa += a[i];
    sb += b[i];
  }
  sa = na_block_sum(sa, sh);
  sb = na_block_sum(sb, sh);
  if (threadIdx.x == 0) {
    pa[blockIdx.x] = sa;
    pb[blockIdx.x] = sb;
  }
}
__global__ void __launch_bounds__(kNaRedBlock) k_na_final(const double *pa, const double *pb, int np, double T,
                                                           double *f) {
  __shared__ double sh[kNaRedBlock / 32];
  double sa = 0.0, sb = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    sa += pa[i];
    sb += pb[i];
  }
  sa = na_block_sum(sa, sh);
  sb = na_block_sum(sb, sh);
  if (threadIdx.x == 0) *f = 1.0 / T * sa - 3.0 * kB * sb;
}

}  // namespace
}  // namespace a2c

extern "C" a2c_status a2c_gpp_eval_mixed_noalloc(a2c_gpp_ctx *c, const double *dX, double *df, double *dG) {
  using namespace a2c;
  if (!c || !df || (c->N > 0 && (!dX || !dG))) return A2C_ERR_INVALID;
  if (c->N > kNaMaxSites) return A2C_ERR_INVALID;  // larger than the fixed scratch array
  if (!c->has_neighbors) return A2C_ERR_STATE;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_status(e);
  unsigned char *base = nullptr;
  A2C_TRY(na_setup(c->device, &base));
  const int64_t N = c->N;
  MixArgs a{};
  a.N = N;
  a.nPd = c->p.nPd;
  a.W = (float)c->p.QWp;
  double k[3];
  for (int d = 0; d < 3; ++d) {
    const double S = c->p.periodic[d] ? c->p.box[d] : kFreeSpan;
    k[d] = 4294967296.0 / S;
    a.sc[d] = (float)(S / 4294967296.0);
  }
  a.P = (const int4 *)(base + kNaP);
  a.occ = (const float *)(base + kNaOcc);
  a.off = c->d_off;
  a.nbr = c->d_nbr;
  a.npd = c->d_npd;
  a.ex = exp_consts();
  a.tabPair = (const float4 *)(base + kNaTabPair);
  a.tabEmb = (const float4 *)(base + kNaTabEmb);
  a.FF = (float2 *)(base + kNaFF);
  a.G = dG;
  a.Vs = (double *)(base + kNaVs);
  a.Ss = (double *)(base + kNaSs);
  a.T = c->p.T;
  double *pa = (double *)(base + kNaPart), *pb = pa + kNaRedGrid;
  // No region needs clearing: every word a kernel reads was written earlier
  // in this call (P, occupancy, F/F', energy partials, block partials).
  // Pass 2 evaluates each pair once when the context holds a current
  // pairs-once index (a mixed-precision context builds it, with its share
  // buffers, when its lists change); nothing is allocated here.
  const bool once = N > 0 && c->mixed && use_once(c);
  if (once) {
    const Mixed *M = c->mixed;
    a.rev = M->rev;
    a.npre = M->npre;
    a.recv = M->recv;
    a.Gown = M->Gown;
  }
  if (N > 0) {
    k_prep<<<grid_for(N, 256), 256, 0, c->stream>>>(dX, c->d_occ, N, k[0], k[1], k[2], (int4 *)(base + kNaP),
                                                     (float *)(base + kNaOcc), span_args(c));
    launch_tile(a, c->stream, nullptr, once, effective_tile(mixed_tile(c), N, device_sms(c->device)), false);
  }
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(kNaRedGrid, (N + kNaRedBlock - 1) / kNaRedBlock));
  k_na_partial<<<grid, kNaRedBlock, 0, c->stream>>>(a.Vs, a.Ss, N, pa, pb);
  k_na_final<<<1, kNaRedBlock, 0, c->stream>>>(pa, pb, grid, c->p.T, df);
  e = cudaGetLastError();
  return e == cudaSuccess ? A2C_OK : cuda_status(e);
}
