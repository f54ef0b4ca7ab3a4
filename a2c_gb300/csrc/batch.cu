// Batched independent instances: many Pd-H lattices of uneven size,
// temperature and loading minimized together in one system.
//
// Layout.  The instances' sites are concatenated in the caller's order
// (instance-major; within an instance Pd then H, the reference's layout of
// minimizer.cpp:398-418), so the state vector of the batch is the
// concatenation of the instances' 4N-double TAO vectors.  Each site carries
// its instance index; the per-instance box, temperature and species split
// come from a small table.  Neighbor lists are built per instance (the same
// cell-list build as one system) and stored with batch-global ids, so one
// launch of each evaluator kernel walks every instance at once.
//
// Minimization.  Each instance runs the projected L-BFGS of lbfgs.cu (the
// stand-in for TAO BLMVM, minimizer.cpp:534-586) with its own iterate,
// memory, step length and stopping state.  The control flow lives on the
// device: one "tick" is a fixed sequence of launches that (A) computes a new
// direction for every instance that needs one, (B) compacts the lists of
// live sites and reduction chunks, (C) evaluates every live instance at its
// trial point and (D) applies each instance's line-search decision.  Every
// live instance receives exactly one evaluation per tick, so the tick can be
// captured once in a CUDA graph and replayed; converged instances drop out
// of the lists (they retire) and cost nothing afterwards.
//
// Reductions.  Per instance, its terms are cut into chunks of kChunk
// consecutive terms; a block reduces each chunk and one block per instance
// sums the chunk partials in order.  The order depends only on the
// instance's own size, so an instance's results do not depend on the rest of
// the batch, and the oracle reproduces them (its "batch" reduction order).
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <new>
#include <vector>

#include "internal.cuh"

namespace a2c {
namespace {

constexpr int kChunk = 2048;  // terms per reduction chunk
constexpr int kBlk = 256;
constexpr int kMaxM = 48;

enum : int { kNeedEval = 0, kNeedDir = 1, kLineSearch = 2, kDone = 3 };
enum : int { kPhaseMixed = 0, kPhaseFp64 = 1 };

// Per-instance L-BFGS state.
struct Inst {
  double f, fn, alpha, amax, gnorm, coef, gam_num, gam_den, f_noise, stall_rtol, mixed_gnorm;
  int state, phase, npairs, head, it, fev, ls, why, copy, steep, nhist, it0, mixed_iters, fp64_iters;
  int fresh;  // a new direction awaits its first trial step length
};

struct Chunk {
  int64_t start;  // first term (element or site index)
  int len;
  int inst;
};

// Constants of one minimization.
struct Cfg {
  int B, m, ring, max_it, max_fev, max_ls, polish, W;
  int64_t nec, nsc, n;  // element chunks, site chunks, vector length
  double gatol, c1, init_step, lb, max_step;
  double fn_mixed, fn_fp64, st_mixed, st_fp64;
};

// Device pointers of the batch state (kernel parameter).
struct Dev {
  Inst *st;
  const InstGeo *geo;
  const Chunk *ech, *sch;  // element / site chunks
  const int *ecb, *scb;    // per instance: first chunk (B + 1)
  const int *le, *ls;      // live element / site chunks
  int *cnt;                // list lengths, see kCnt*
  double *x, *g, *pg, *d, *xn, *gn, *S, *Y;
  double *part;            // 8 x nec element partials, then 2 x nsc site partials
  double *rho, *alph;      // B x ring
  double *fh;              // B x (W + 1): objective history of the phase
  const double *Vs, *Ss;
};

enum : int { kCntMixed = 0, kCntFp64 = 1, kCntEch = 2, kCntSch = 3, kCntLive = 4, kCntChanged = 5, kCntLeft = 6 };

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double wmax(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// block of kBlk threads: the warp tree, then warp 0 over the 8 warp sums
template <bool MAX>
__device__ __forceinline__ double bred(double v, double *sh) {
  v = MAX ? wmax(v) : wsum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
  if (w == 0) v = MAX ? wmax(v) : wsum(v);
  __syncthreads();
  return v;
}

__device__ __forceinline__ bool on_bound(int64_t t, const double *x, const double *g, double lb) {
  return (t & 3) == 3 && x[t] <= lb && g[t] > 0.0;
}

// sum over the instance's chunk partials part[c], c in [c0, c1), in order
__device__ __forceinline__ double chunk_total(const double *part, int c0, int c1, double *sh) {
  double s = 0.0;
  for (int i = c0 + threadIdx.x; i < c1; i += blockDim.x) s += part[i];
  return bred<false>(s, sh);
}
__device__ __forceinline__ double chunk_max(const double *part, int c0, int c1, double *sh) {
  double s = 0.0;
  for (int i = c0 + threadIdx.x; i < c1; i += blockDim.x) s = fmax(s, part[i]);
  return bred<true>(s, sh);
}

__device__ __forceinline__ int slot(int head, int k, int ring) { return ((head - 1 - k) % ring + ring) % ring; }

// End of a phase: hand over to the FP64 polish, or retire.
__device__ void end_phase(Inst &I, const Cfg &cf, int why) {
  if (I.phase == kPhaseMixed) {
    I.mixed_iters = I.it;
    I.mixed_gnorm = I.gnorm;
  } else {
    I.fp64_iters = I.it - I.it0;
  }
  I.why = why;
  if (I.phase == kPhaseMixed && cf.polish && (why == A2C_CONVERGED_GATOL || why == A2C_DIVERGED_LS_FAILURE ||
                                               why == A2C_CONVERGED_STALLED)) {
    I.phase = kPhaseFp64;
    I.state = kNeedEval;
    I.nhist = 0;
    I.it0 = I.it;
    I.f_noise = cf.fn_fp64;
    I.stall_rtol = cf.st_fp64;
  } else {
    I.state = kDone;
  }
}

// ------------------------------------------------------------ set-up
__global__ void k_init_state(Dev D, Cfg cf, int phase0) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= cf.B) return;
  Inst I;
  memset(&I, 0, sizeof(I));
  I.state = kNeedEval;
  I.phase = phase0;
  I.f_noise = phase0 == kPhaseMixed ? cf.fn_mixed : cf.fn_fp64;
  I.stall_rtol = phase0 == kPhaseMixed ? cf.st_mixed : cf.st_fp64;
  D.st[b] = I;
}

__global__ void k_project_all(double *x, int64_t n, double lb) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    if ((t & 3) == 3 && x[t] < lb) x[t] = lb;
}

// ------------------------------------------------------------ list plan
// One block: per instance its listing code (-1 retired, 0 mixed, 1 FP64),
// exclusive prefix sums of the site and chunk counts, and whether anything
// changed since the last plan (only then does k_fill rewrite the lists).
constexpr int kPlanThreads = 1024;
__global__ void __launch_bounds__(kPlanThreads) k_plan(Dev D, int B, int *listed, int *loff) {
  __shared__ int sh[7][kPlanThreads];
  __shared__ int changed;
  if (threadIdx.x == 0) changed = 0;
  const int per = (B + kPlanThreads - 1) / kPlanThreads;
  const int b0 = min(B, (int)threadIdx.x * per), b1 = min(B, b0 + per);
  int q[7] = {0, 0, 0, 0, 0, 0, 0};
  bool ch = false;
  for (int b = b0; b < b1; ++b) {
    const Inst &I = D.st[b];
    const int code = I.state == kDone ? -1 : I.phase;
    if (code != listed[b]) ch = true;
    const InstGeo &g = D.geo[b];
    if (code == 0) { q[0] += g.nPd; q[1] += g.nH; }
    if (code == 1) { q[2] += g.nPd; q[3] += g.nH; }
    if (code >= 0) {
      q[4] += D.ecb[b + 1] - D.ecb[b];
      q[5] += D.scb[b + 1] - D.scb[b];
      q[6] += 1;
    }
  }
  __syncthreads();
  if (ch) atomicOr(&changed, 1);
  for (int k = 0; k < 7; ++k) sh[k][threadIdx.x] = q[k];
  __syncthreads();
  // inclusive Hillis-Steele scan of the per-thread sums
  for (int o = 1; o < kPlanThreads; o <<= 1) {
    int v[7];
    for (int k = 0; k < 7; ++k) v[k] = threadIdx.x >= (unsigned)o ? sh[k][threadIdx.x - o] : 0;
    __syncthreads();
    for (int k = 0; k < 7; ++k) sh[k][threadIdx.x] += v[k];
    __syncthreads();
  }
  int run[7];
  for (int k = 0; k < 7; ++k) run[k] = sh[k][threadIdx.x] - q[k];
  const int totPdM = sh[0][kPlanThreads - 1], totPdF = sh[2][kPlanThreads - 1];
  if (changed) {
    for (int b = b0; b < b1; ++b) {
      const Inst &I = D.st[b];
      const int code = I.state == kDone ? -1 : I.phase;
      const InstGeo &g = D.geo[b];
      int *o = loff + 6 * b;
      o[0] = code == 0 ? run[0] : (code == 1 ? run[2] : -1);               // Pd sites
      o[1] = code == 0 ? totPdM + run[1] : (code == 1 ? totPdF + run[3] : -1);  // H sites
      o[2] = code >= 0 ? run[4] : -1;
      o[3] = code >= 0 ? run[5] : -1;
      o[4] = code;
      if (code == 0) { run[0] += g.nPd; run[1] += g.nH; }
      if (code == 1) { run[2] += g.nPd; run[3] += g.nH; }
      if (code >= 0) {
        run[4] += D.ecb[b + 1] - D.ecb[b];
        run[5] += D.scb[b + 1] - D.scb[b];
      }
      listed[b] = code;
    }
  }
  if (threadIdx.x == kPlanThreads - 1) {
    D.cnt[kCntMixed] = sh[0][threadIdx.x] + sh[1][threadIdx.x];
    D.cnt[kCntFp64] = sh[2][threadIdx.x] + sh[3][threadIdx.x];
    D.cnt[kCntEch] = sh[4][threadIdx.x];
    D.cnt[kCntSch] = sh[5][threadIdx.x];
    D.cnt[kCntLive] = sh[6][threadIdx.x];
    D.cnt[kCntChanged] = changed;
  }
}

// One block per instance: its sites into the mixed or FP64 list (Pd sites
// of all listed instances first, so warps stay species-uniform) and its
// chunks into the live chunk lists.
__global__ void k_fill(Dev D, int B, const int *loff, int *lm, int *lf, int *le, int *ls) {
  if (!D.cnt[kCntChanged]) return;
  const int b = blockIdx.x;
  if (b >= B) return;
  const int *o = loff + 6 * b;
  const int code = o[4];
  if (code < 0) return;
  const InstGeo &g = D.geo[b];
  int *L = code == 0 ? lm : lf;
  for (int i = threadIdx.x; i < g.nPd; i += blockDim.x) L[o[0] + i] = g.start + i;
  for (int i = threadIdx.x; i < g.nH; i += blockDim.x) L[o[1] + i] = g.start + g.nPd + i;
  const int e0 = D.ecb[b], ne = D.ecb[b + 1] - e0, s0 = D.scb[b], ns = D.scb[b + 1] - s0;
  for (int i = threadIdx.x; i < ne; i += blockDim.x) le[o[2] + i] = e0 + i;
  for (int i = threadIdx.x; i < ns; i += blockDim.x) ls[o[3] + i] = s0 + i;
}

__global__ void k_count_left(Dev D, int B) {
  __shared__ double sh[kBlk / 32];
  double v = 0.0;
  for (int b = threadIdx.x; b < B; b += blockDim.x) v += D.st[b].state != kDone ? 1.0 : 0.0;
  v = bred<false>(v, sh);
  if (threadIdx.x == 0) D.cnt[kCntLeft] = (int)v;
}

// ------------------------------------------------------------ direction
// Element-chunk kernels walk the live element chunks; a whole block takes
// one chunk, so the per-instance tests below are block-uniform.
#define A2C_ECHUNKS(D)                                                     \
  for (int kk = blockIdx.x; kk < (D).cnt[kCntEch]; kk += gridDim.x) {       \
    const int c = (D).le[kk];                                             \
    const Chunk ch = (D).ech[c];                                          \
    Inst &I = (D).st[ch.inst];
#define A2C_ECHUNKS_END }

// pg = projected gradient; partials of |pg|^2 and max |pg|
__global__ void __launch_bounds__(kBlk) k_projgrad(Dev D, Cfg cf) {
  __shared__ double sh[kBlk / 32];
  A2C_ECHUNKS(D)
  if (I.state != kNeedDir) continue;
  double s = 0.0, mx = 0.0;
  for (int i = threadIdx.x; i < ch.len; i += kBlk) {
    const int64_t t = ch.start + i;
    const double v = on_bound(t, D.x, D.g, cf.lb) ? 0.0 : D.g[t];
    D.pg[t] = v;
    s += v * v;
    mx = fmax(mx, fabs(v));
  }
  s = bred<false>(s, sh);
  mx = bred<true>(mx, sh);
  if (threadIdx.x == 0) {
    D.part[c] = s;
    D.part[cf.nec + c] = mx;
  }
  A2C_ECHUNKS_END
}

// gnorm and the stopping tests (TAO's gatol test and the caps)
__global__ void __launch_bounds__(kBlk) k_dir_begin(Dev D, Cfg cf) {
  __shared__ double sh[kBlk / 32];
  const int b = blockIdx.x;
  Inst &I = D.st[b];
  if (threadIdx.x == 0) I.copy = 0;
  if (I.state != kNeedDir) return;
  const double s = chunk_total(D.part, D.ecb[b], D.ecb[b + 1], sh);
  const double mx = chunk_max(D.part + cf.nec, D.ecb[b], D.ecb[b + 1], sh);
  if (threadIdx.x != 0) return;
  I.gnorm = sqrt(s);
  I.amax = mx;
  I.steep = 0;
  if (!isfinite(I.f) || !isfinite(I.gnorm)) end_phase(I, cf, A2C_DIVERGED_NAN);
  else if (I.gnorm <= cf.gatol) end_phase(I, cf, A2C_CONVERGED_GATOL);
  else if (I.it >= cf.max_it) end_phase(I, cf, A2C_DIVERGED_MAXITS);
  else if (I.fev >= cf.max_fev) end_phase(I, cf, A2C_DIVERGED_MAXFCN);
  else I.steep = I.npairs == 0 ? 1 : 0;
}

// Two-loop recursion, first loop, step j (newest pair first): apply the
// update of step j-1, then the partial dot S_j . q.
__global__ void __launch_bounds__(kBlk) k_loop1(Dev D, Cfg cf, int j) {
  __shared__ double sh[kBlk / 32];
  A2C_ECHUNKS(D)
  if (I.state != kNeedDir || I.steep) continue;
  const int b = ch.inst, np = I.npairs;
  const bool upd = j > 0 && j - 1 < np, dot = j < np;
  if (j > 0 && !upd && !dot) continue;
  const int slp = slot(I.head, j - 1, cf.ring), sl = slot(I.head, j, cf.ring);
  const double a = upd ? D.alph[b * cf.ring + slp] : 0.0;
  const double *Yp = D.Y + (size_t)slp * cf.n, *Sj = D.S + (size_t)sl * cf.n;
  double s = 0.0;
  for (int i = threadIdx.x; i < ch.len; i += kBlk) {
    const int64_t t = ch.start + i;
    double q = j == 0 ? D.pg[t] : D.d[t];
    if (upd) q -= a * Yp[t];
    D.d[t] = q;
    if (dot) s += Sj[t] * q;
  }
  s = bred<false>(s, sh);
  if (threadIdx.x == 0) D.part[2 * cf.nec + c] = s;
  A2C_ECHUNKS_END
}

__global__ void __launch_bounds__(kBlk) k_loop1_fin(Dev D, Cfg cf, int j) {
  __shared__ double sh[kBlk / 32];
  const int b = blockIdx.x;
  Inst &I = D.st[b];
  if (I.state != kNeedDir || I.steep || j >= I.npairs) return;
  const double s = chunk_total(D.part + 2 * cf.nec, D.ecb[b], D.ecb[b + 1], sh);
  if (threadIdx.x == 0) {
    const int sl = slot(I.head, j, cf.ring);
    D.alph[b * cf.ring + sl] = s * D.rho[b * cf.ring + sl];
  }
}

// the pending update of the last first-loop step, then q *= s.y / y.y
__global__ void __launch_bounds__(kBlk) k_scale(Dev D, Cfg cf) {
  A2C_ECHUNKS(D)
  if (I.state != kNeedDir || I.steep) continue;
  const int b = ch.inst;
  const bool upd = I.npairs == cf.m;
  const int slp = slot(I.head, cf.m - 1, cf.ring);
  const double a = upd ? D.alph[b * cf.ring + slp] : 0.0;
  const double gam = I.gam_num / I.gam_den;
  const double *Yp = D.Y + (size_t)slp * cf.n;
  for (int i = threadIdx.x; i < ch.len; i += kBlk) {
    const int64_t t = ch.start + i;
    double q = D.d[t];
    if (upd) q -= a * Yp[t];
    D.d[t] = q * gam;
  }
  A2C_ECHUNKS_END
}

// Second loop, step j (oldest pair first): apply the update of step j-1,
// then the partial dot Y_j . q.
__global__ void __launch_bounds__(kBlk) k_loop2(Dev D, Cfg cf, int j) {
  __shared__ double sh[kBlk / 32];
  A2C_ECHUNKS(D)
  if (I.state != kNeedDir || I.steep) continue;
  const int np = I.npairs;
  const bool upd = j > 0 && j - 1 < np, dot = j < np;
  if (!upd && !dot) continue;
  const int slp = slot(I.head, np - j, cf.ring), sl = slot(I.head, np - 1 - j, cf.ring);
  const double cp = I.coef;
  const double *Sp = D.S + (size_t)slp * cf.n, *Yj = D.Y + (size_t)sl * cf.n;
  double s = 0.0;
  for (int i = threadIdx.x; i < ch.len; i += kBlk) {
    const int64_t t = ch.start + i;
    double q = D.d[t];
    if (upd) q += cp * Sp[t];
    D.d[t] = q;
    if (dot) s += Yj[t] * q;
  }
  s = bred<false>(s, sh);
  if (threadIdx.x == 0) D.part[2 * cf.nec + c] = s;
  A2C_ECHUNKS_END
}

__global__ void __launch_bounds__(kBlk) k_loop2_fin(Dev D, Cfg cf, int j) {
  __shared__ double sh[kBlk / 32];
  const int b = blockIdx.x;
  Inst &I = D.st[b];
  if (I.state != kNeedDir || I.steep || j >= I.npairs) return;
  const double s = chunk_total(D.part + 2 * cf.nec, D.ecb[b], D.ecb[b + 1], sh);
  if (threadIdx.x == 0) {
    const int sl = slot(I.head, I.npairs - 1 - j, cf.ring);
    I.coef = D.alph[b * cf.ring + sl] - D.rho[b * cf.ring + sl] * s;
  }
}

// d = -q off the active set (or the scaled steepest descent); partial g.d
__global__ void __launch_bounds__(kBlk) k_finish(Dev D, Cfg cf) {
  __shared__ double sh[kBlk / 32];
  A2C_ECHUNKS(D)
  if (I.state != kNeedDir) continue;
  const bool steep = I.steep != 0;
  const bool upd = !steep && I.npairs == cf.m;
  const int slp = slot(I.head, 0, cf.ring);
  const double cp = I.coef, sc = -cf.init_step / I.amax;
  const double *Sp = D.S + (size_t)slp * cf.n;
  double s = 0.0, mx = 0.0;
  for (int i = threadIdx.x; i < ch.len; i += kBlk) {
    const int64_t t = ch.start + i;
    double v;
    if (steep) {
      v = D.pg[t] * sc;
    } else {
      double q = D.d[t];
      if (upd) q += cp * Sp[t];
      v = on_bound(t, D.x, D.g, cf.lb) ? 0.0 : -q;
    }
    D.d[t] = v;
    s += D.g[t] * v;
    mx = fmax(mx, fabs(v));
  }
  s = bred<false>(s, sh);
  mx = bred<true>(mx, sh);
  if (threadIdx.x == 0) {
    D.part[3 * cf.nec + c] = s;
    D.part[cf.nec + c] = mx;  // the slot of max |pg|, read before this kernel
  }
  A2C_ECHUNKS_END
}

// not a descent direction: drop the memory, fall back to steepest descent
__global__ void __launch_bounds__(kBlk) k_dir_end(Dev D, Cfg cf) {
  __shared__ double sh[kBlk / 32];
  const int b = blockIdx.x;
  Inst &I = D.st[b];
  if (I.state != kNeedDir) return;
  const double gd = chunk_total(D.part + 3 * cf.nec, D.ecb[b], D.ecb[b + 1], sh);
  if (threadIdx.x != 0) return;
  if (!(gd < 0.0)) {
    I.npairs = 0;
    I.head = 0;
    I.steep = 2;
  } else {
    I.steep = 0;
  }
  I.alpha = 1.0;
  I.ls = 0;
  I.fresh = 1;
  I.state = kLineSearch;
}

__global__ void __launch_bounds__(kBlk) k_steep(Dev D, Cfg cf) {
  __shared__ double sh[kBlk / 32];
  A2C_ECHUNKS(D)
  if (I.steep != 2) continue;
  const double sc = -cf.init_step / I.amax;
  double mx = 0.0;
  for (int i = threadIdx.x; i < ch.len; i += kBlk) {
    const int64_t t = ch.start + i;
    const double v = D.pg[t] * sc;
    D.d[t] = v;
    mx = fmax(mx, fabs(v));
  }
  mx = bred<true>(mx, sh);
  if (threadIdx.x == 0) D.part[cf.nec + c] = mx;
  A2C_ECHUNKS_END
}

// first trial step length: min(1, max_step / max|d|)
__global__ void __launch_bounds__(kBlk) k_alpha0(Dev D, Cfg cf) {
  __shared__ double sh[kBlk / 32];
  const int b = blockIdx.x;
  Inst &I = D.st[b];
  if (I.state != kLineSearch || !I.fresh) return;
  const double dmax = chunk_max(D.part + cf.nec, D.ecb[b], D.ecb[b + 1], sh);
  if (threadIdx.x != 0) return;
  I.fresh = 0;
  if (cf.max_step > 0.0 && dmax > cf.max_step) I.alpha = cf.max_step / dmax;
}

// ------------------------------------------------------------ trial / decide
// xn = P(x + alpha d) (line search) or xn = x (first evaluation of a
// phase); partial g.(xn - x)
__global__ void __launch_bounds__(kBlk) k_trial(Dev D, Cfg cf) {
  __shared__ double sh[kBlk / 32];
  A2C_ECHUNKS(D)
  if (I.state != kLineSearch && I.state != kNeedEval) continue;
  const bool ls = I.state == kLineSearch;
  const double al = I.alpha;
  double s = 0.0;
  for (int i = threadIdx.x; i < ch.len; i += kBlk) {
    const int64_t t = ch.start + i;
    double v = D.x[t];
    if (ls) {
      v = D.x[t] + al * D.d[t];
      if ((t & 3) == 3 && v < cf.lb) v = cf.lb;
      s += D.g[t] * (v - D.x[t]);
    }
    D.xn[t] = v;
  }
  s = bred<false>(s, sh);
  if (threadIdx.x == 0) D.part[4 * cf.nec + c] = s;
  A2C_ECHUNKS_END
}

// candidate pair into the free ring slot; partials gn.s, s.y, y.y
__global__ void __launch_bounds__(kBlk) k_post(Dev D, Cfg cf) {
  __shared__ double sh[kBlk / 32];
  A2C_ECHUNKS(D)
  if (I.state != kLineSearch) continue;
  double *Sh = D.S + (size_t)I.head * cf.n, *Yh = D.Y + (size_t)I.head * cf.n;
  double dn = 0.0, sy = 0.0, yy = 0.0;
  for (int i = threadIdx.x; i < ch.len; i += kBlk) {
    const int64_t t = ch.start + i;
    const double s = D.xn[t] - D.x[t], y = D.gn[t] - D.g[t];
    Sh[t] = s;
    Yh[t] = y;
    dn += D.gn[t] * s;
    sy += s * y;
    yy += y * y;
  }
  dn = bred<false>(dn, sh);
  sy = bred<false>(sy, sh);
  yy = bred<false>(yy, sh);
  if (threadIdx.x == 0) {
    D.part[5 * cf.nec + c] = dn;
    D.part[6 * cf.nec + c] = sy;
    D.part[7 * cf.nec + c] = yy;
  }
  A2C_ECHUNKS_END
}

// site-chunk partials of the energy and sigma-entropy sums
__global__ void __launch_bounds__(kBlk) k_objpart(Dev D, Cfg cf, int all) {
  __shared__ double sh[kBlk / 32];
  for (int kk = blockIdx.x; kk < D.cnt[kCntSch]; kk += gridDim.x) {
    const int c = D.ls[kk];
    const Chunk ch = D.sch[c];
    const Inst &I = D.st[ch.inst];
    if (!all && I.state != kLineSearch && I.state != kNeedEval) continue;
    double v = 0.0, s = 0.0;
    for (int i = threadIdx.x; i < ch.len; i += kBlk) {
      v += D.Vs[ch.start + i];
      s += D.Ss[ch.start + i];
    }
    v = bred<false>(v, sh);
    s = bred<false>(s, sh);
    if (threadIdx.x == 0) {
      D.part[8 * cf.nec + c] = v;
      D.part[8 * cf.nec + cf.nsc + c] = s;
    }
  }
}

// f = (1/T) sum V - 3 kB sum sigma  (minimizer.cpp:353)
__device__ __forceinline__ double objective(const Dev &D, const Cfg &cf, int b, double *sh) {
  const double sv = chunk_total(D.part + 8 * cf.nec, D.scb[b], D.scb[b + 1], sh);
  const double ss = chunk_total(D.part + 8 * cf.nec + cf.nsc, D.scb[b], D.scb[b + 1], sh);
  return 1.0 / D.geo[b].T * sv - 3.0 * kB * ss;
}

__global__ void __launch_bounds__(kBlk) k_objective(Dev D, Cfg cf, double *f) {
  __shared__ double sh[kBlk / 32];
  const int b = blockIdx.x;
  const double v = objective(D, cf, b, sh);
  if (threadIdx.x == 0) f[b] = v;
}

// The line-search decision (lbfgs.cu, one instance per block).
__global__ void __launch_bounds__(kBlk) k_decide(Dev D, Cfg cf) {
  __shared__ double sh[kBlk / 32];
  const int b = blockIdx.x;
  Inst &I = D.st[b];
  if (I.state != kLineSearch && I.state != kNeedEval) return;
  const double fn = objective(D, cf, b, sh);
  const int e0 = D.ecb[b], e1 = D.ecb[b + 1];
  const double dec = chunk_total(D.part + 4 * cf.nec, e0, e1, sh);
  const double dn = chunk_total(D.part + 5 * cf.nec, e0, e1, sh);
  const double sy = chunk_total(D.part + 6 * cf.nec, e0, e1, sh);
  const double yy = chunk_total(D.part + 7 * cf.nec, e0, e1, sh);
  if (threadIdx.x != 0) return;
  I.fev += 1;
  I.fn = fn;
  if (I.state == kNeedEval) {
    I.f = fn;
    I.copy = 2;
    I.nhist = 0;
    I.state = kNeedDir;
    return;
  }
  bool ok = isfinite(fn) && fn <= I.f + cf.c1 * dec;
  if (!ok && isfinite(fn) && fabs(fn - I.f) <= I.f_noise * fabs(I.f)) ok = dn <= (2.0 * cf.c1 - 1.0) * dec;
  if (ok) {
    if (sy > 2.220446049250313e-16 * yy) {
      D.rho[b * cf.ring + I.head] = 1.0 / sy;
      I.gam_num = sy;
      I.gam_den = yy;
      I.head = (I.head + 1) % cf.ring;
      if (I.npairs < cf.m) ++I.npairs;
    }
    I.copy = 1;
    I.f = fn;
    I.it += 1;
    const int W = cf.W;
    if (W > 0) {
      double *h = D.fh + (size_t)b * (W + 1);
      h[I.nhist % (W + 1)] = fn;
      I.nhist += 1;
      if (I.nhist > W && h[(I.nhist - 1 - W) % (W + 1)] - fn <= I.stall_rtol * fabs(fn)) {
        end_phase(I, cf, A2C_CONVERGED_STALLED);
        return;
      }
    }
    I.state = kNeedDir;
    return;
  }
  I.copy = 0;
  I.alpha *= 0.5;
  I.ls += 1;
  if (I.fev >= cf.max_fev || I.ls >= cf.max_ls) {
    if (I.npairs > 0 && I.fev < cf.max_fev) {
      I.npairs = 0;
      I.head = 0;
      I.state = kNeedDir;
    } else {
      end_phase(I, cf, I.fev >= cf.max_fev ? A2C_DIVERGED_MAXFCN : A2C_DIVERGED_LS_FAILURE);
    }
  }
}

// accepted step: x <- xn, g <- gn; first evaluation of a phase: g <- gn
__global__ void __launch_bounds__(kBlk) k_copy(Dev D, Cfg cf) {
  A2C_ECHUNKS(D)
  if (!I.copy) continue;
  const bool both = I.copy == 1;
  for (int i = threadIdx.x; i < ch.len; i += kBlk) {
    const int64_t t = ch.start + i;
    if (both) D.x[t] = D.xn[t];
    D.g[t] = D.gn[t];
  }
  A2C_ECHUNKS_END
}

// ------------------------------------------------------------ CSR assembly
__global__ void k_copy_csr(const int64_t *off, const uint32_t *nbr, const int *npd, int64_t n, int64_t total,
                           int64_t start, int64_t base, int64_t *boff, uint32_t *bnbr, int *bnpd) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    boff[start + s] = base + off[s];
    bnpd[start + s] = npd[s];
  }
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t e = nbr[t];
    bnbr[base + t] = (uint32_t)((e & kIdMask) + (uint32_t)start) | (e & ~kIdMask);
  }
}

__global__ void k_set_i64(int64_t *p, int64_t v) { *p = v; }

}  // namespace
}  // namespace a2c

using namespace a2c;

struct a2c_gpp_batch {
  int B = 0;
  int device = 0;
  int precision = A2C_FP64;
  Tile tile;  // the mixed pair kernels' tile (zeros: the library's choice)
  bool graphs = true;
  a2c_gpp_ctx *c = nullptr;  // the union system (evaluator buffers, lists, stream)
  std::vector<a2c_gpp_params> P;
  std::vector<int64_t> start;  // B + 1
  std::vector<int> ecb, scb;   // B + 1
  int64_t nec = 0, nsc = 0;
  // device tables
  InstGeo *geo = nullptr;
  uint16_t *inst = nullptr;
  Chunk *ech = nullptr, *sch = nullptr;
  int *d_ecb = nullptr, *d_scb = nullptr;
  int *lm = nullptr, *lf = nullptr, *le = nullptr, *ls = nullptr;
  int *cnt = nullptr, *listed = nullptr, *loff = nullptr;
  Inst *st = nullptr;
  double *part = nullptr;
  // L-BFGS buffers (allocated at the first minimization)
  int m = 0, W = -1;
  double *x = nullptr, *g = nullptr, *pg = nullptr, *d = nullptr, *xn = nullptr, *gn = nullptr;
  double *S = nullptr, *Y = nullptr, *rho = nullptr, *alph = nullptr, *fh = nullptr;
  int *h_cnt = nullptr;  // pinned
  // the captured tick (and the neighbor array it was captured with: a list
  // rebuild may reallocate it)
  cudaGraphExec_t exec = nullptr;
  Cfg exec_cfg{};
  Tile exec_tile{-1, -1, -1};
  const void *exec_nbr = nullptr;
  const void *exec_pass2[5] = {};  // the captured pass 2: mode and its index buffers
  bool borrowed = false;  // c belongs to a context (the one-instance engine)
  // statistics of the last minimization
  int ticks = 0;
  double seconds = 0.0;
};

namespace {

template <class T>
a2c_status dmalloc(T **p, int64_t n) {
  *p = nullptr;
  if (cudaMalloc((void **)p, sizeof(T) * (size_t)std::max<int64_t>(n, 1)) != cudaSuccess) return A2C_ERR_NOMEM;
  return A2C_OK;
}

void free_lbfgs(a2c_gpp_batch *b) {
  for (double *p : {b->x, b->g, b->pg, b->d, b->xn, b->gn, b->S, b->Y, b->rho, b->alph, b->fh})
    if (p) cudaFree(p);
  b->x = b->g = b->pg = b->d = b->xn = b->gn = b->S = b->Y = b->rho = b->alph = b->fh = nullptr;
  b->m = 0;
  b->W = -1;
}

Dev dev_view(a2c_gpp_batch *b) {
  Dev D{};
  D.st = b->st;
  D.geo = b->geo;
  D.ech = b->ech;
  D.sch = b->sch;
  D.ecb = b->d_ecb;
  D.scb = b->d_scb;
  D.le = b->le;
  D.ls = b->ls;
  D.cnt = b->cnt;
  D.x = b->x;
  D.g = b->g;
  D.pg = b->pg;
  D.d = b->d;
  D.xn = b->xn;
  D.gn = b->gn;
  D.S = b->S;
  D.Y = b->Y;
  D.part = b->part;
  D.rho = b->rho;
  D.alph = b->alph;
  D.fh = b->fh;
  D.Vs = b->c->d_Vs;
  D.Ss = b->c->d_Ss;
  return D;
}

BatchView view(a2c_gpp_batch *b, int which) {
  BatchView v;
  v.inst = b->inst;
  v.geo = b->geo;
  v.list = which == 0 ? b->lm : b->lf;
  v.count = b->cnt + (which == 0 ? kCntMixed : kCntFp64);
  return v;
}

// The chunk kernels stride over chunks; each chunk's sum has a fixed
// order, so results do not depend on this grid.
int chunk_grid(int64_t nchunks) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(nchunks, 8 * (int64_t)current_device_sms()));
}

a2c_status plan(a2c_gpp_batch *b, const Dev &D) {
  cudaStream_t s = b->c->stream;
  k_plan<<<1, kPlanThreads, 0, s>>>(D, b->B, b->listed, b->loff);
  k_fill<<<b->B, kBlk, 0, s>>>(D, b->B, b->loff, b->lm, b->lf, b->le, b->ls);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

Tile batch_tile(a2c_gpp_batch *b) { return effective_tile(b->tile, b->c->N, device_sms(b->c->device)); }

// Evaluation of every listed site at xn into gn (both forms; a form with
// an empty list costs an empty launch).
a2c_status eval_lists(a2c_gpp_batch *b, const double *X, double *G, const Tile &tile) {
  A2C_TRY(mixed_eval_list(b->c, X, G, view(b, 0), tile));
  A2C_TRY(launch_eval64_list(b->c, X, G, view(b, 1)));
  return A2C_OK;
}

// One tick (see the file comment); the same launches whether captured or not.
a2c_status tick(a2c_gpp_batch *b, const Dev &D, const Cfg &cf, const Tile &tps) {
  cudaStream_t s = b->c->stream;
  const int ge = chunk_grid(cf.nec), gs = chunk_grid(cf.nsc), B = cf.B;
  k_projgrad<<<ge, kBlk, 0, s>>>(D, cf);
  k_dir_begin<<<B, kBlk, 0, s>>>(D, cf);
  for (int j = 0; j < cf.m; ++j) {
    k_loop1<<<ge, kBlk, 0, s>>>(D, cf, j);
    k_loop1_fin<<<B, kBlk, 0, s>>>(D, cf, j);
  }
  k_scale<<<ge, kBlk, 0, s>>>(D, cf);
  for (int j = 0; j < cf.m; ++j) {
    k_loop2<<<ge, kBlk, 0, s>>>(D, cf, j);
    k_loop2_fin<<<B, kBlk, 0, s>>>(D, cf, j);
  }
  k_finish<<<ge, kBlk, 0, s>>>(D, cf);
  k_dir_end<<<B, kBlk, 0, s>>>(D, cf);
  k_steep<<<ge, kBlk, 0, s>>>(D, cf);
  k_alpha0<<<B, kBlk, 0, s>>>(D, cf);
  A2C_TRY(plan(b, D));
  k_trial<<<ge, kBlk, 0, s>>>(D, cf);
  A2C_TRY(eval_lists(b, b->xn, b->gn, tps));
  k_post<<<ge, kBlk, 0, s>>>(D, cf);
  k_objpart<<<gs, kBlk, 0, s>>>(D, cf, 0);
  k_decide<<<B, kBlk, 0, s>>>(D, cf);
  k_copy<<<ge, kBlk, 0, s>>>(D, cf);
  k_count_left<<<1, kBlk, 0, s>>>(D, B);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

a2c_status ensure_lbfgs(a2c_gpp_batch *b, int m, int W) {
  if (b->x && b->m == m && b->W == W) return A2C_OK;
  free_lbfgs(b);
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  const int64_t n = 4 * b->c->N;
  for (double **p : {&b->x, &b->g, &b->pg, &b->d, &b->xn, &b->gn}) A2C_TRY(dmalloc(p, n));
  A2C_TRY(dmalloc(&b->S, n * (m + 1)));
  A2C_TRY(dmalloc(&b->Y, n * (m + 1)));
  A2C_TRY(dmalloc(&b->rho, (int64_t)b->B * (m + 1)));
  A2C_TRY(dmalloc(&b->alph, (int64_t)b->B * (m + 1)));
  A2C_TRY(dmalloc(&b->fh, (int64_t)b->B * (W + 1)));
  A2C_CUDA(cudaMemset(b->rho, 0, sizeof(double) * b->B * (m + 1)));
  A2C_CUDA(cudaMemset(b->alph, 0, sizeof(double) * b->B * (m + 1)));
  b->m = m;
  b->W = W;
  return A2C_OK;
}

struct DeviceGuard {
  explicit DeviceGuard(int d) { cudaSetDevice(d); }
};

bool same_common(const a2c_gpp_params &a, const a2c_gpp_params &b) {
  if (a.QWp != b.QWp || a.eps != b.eps || a.rc != b.rc || a.a_Pd != b.a_Pd || a.precision != b.precision ||
      a.device != b.device)
    return false;
  for (int k = 0; k < 4; ++k)
    if (a.coe_Pd[k] != b.coe_Pd[k] || a.coe_H[k] != b.coe_H[k]) return false;
  return true;
}

struct DeviceGuard2 {
  explicit DeviceGuard2(int d) { cudaSetDevice(d); }
};

// The span-guard limits of instance k (InstGeo::lim): a batch builds its
// lists at each instance's cutoff; a context's one-instance engine takes
// the reach of the context's lists (which the caller may have supplied).
void set_limits(const a2c_gpp_batch *b, int k, InstGeo &G) {
  const a2c_gpp_params &p = b->P[(size_t)k];
  for (int d = 0; d < 3; ++d) {
    const double reach = b->borrowed ? b->c->list_reach[d] : p.rc;
    G.lim[d] = p.periodic[d] ? HUGE_VALF
                             : (std::isfinite(reach) ? (float)(0.5 * (0.5 * kFreeSpan - reach)) : -HUGE_VALF);
  }
}

// Instance, chunk and list tables of a batch whose system b->c exists;
// set_occ: Pd occupancy 1, H 0 (a fresh union system).
a2c_status init_tables(a2c_gpp_batch *b, const a2c_gpp_params *params, int n, bool set_occ) {
  DeviceGuard2 dg(b->device);
  const int64_t N = b->c->N;
  // instance table and chunk tables
  b->start.assign(n + 1, 0);
  b->ecb.assign(n + 1, 0);
  b->scb.assign(n + 1, 0);
  std::vector<InstGeo> geo(n);
  std::vector<Chunk> ech, sch;
  std::vector<uint16_t> inst((size_t)N);
  std::vector<double> occ((size_t)N, 0.0);
  for (int k = 0; k < n; ++k) {
    const a2c_gpp_params &p = params[k];
    const int64_t s0 = b->start[k], nk = (int64_t)p.nPd + p.nH;
    b->start[k + 1] = s0 + nk;
    InstGeo &G = geo[k];
    for (int d = 0; d < 3; ++d) {
      G.S[d] = p.periodic[d] ? p.box[d] : kFreeSpan;
      G.sc[d] = (float)(G.S[d] / 4294967296.0);
    }
    set_limits(b, k, G);
    G.T = p.T;
    G.start = (int)s0;
    G.nPd = p.nPd;
    G.nH = p.nH;
    for (int64_t i = 0; i < nk; ++i) inst[(size_t)(s0 + i)] = (uint16_t)k;
    for (int64_t i = 0; i < p.nPd; ++i) occ[(size_t)(s0 + i)] = 1.0;
    b->ecb[k] = (int)ech.size();
    for (int64_t c0 = 0; c0 < 4 * nk; c0 += kChunk)
      ech.push_back({4 * s0 + c0, (int)std::min<int64_t>(kChunk, 4 * nk - c0), k});
    b->scb[k] = (int)sch.size();
    for (int64_t c0 = 0; c0 < nk; c0 += kChunk) sch.push_back({s0 + c0, (int)std::min<int64_t>(kChunk, nk - c0), k});
  }
  b->ecb[n] = (int)ech.size();
  b->scb[n] = (int)sch.size();
  b->nec = (int64_t)ech.size();
  b->nsc = (int64_t)sch.size();
  a2c_status s = A2C_OK;
  if (!s) s = dmalloc(&b->geo, n);
  if (!s) s = dmalloc(&b->inst, N);
  if (!s) s = dmalloc(&b->ech, b->nec);
  if (!s) s = dmalloc(&b->sch, b->nsc);
  if (!s) s = dmalloc(&b->d_ecb, n + 1);
  if (!s) s = dmalloc(&b->d_scb, n + 1);
  if (!s) s = dmalloc(&b->lm, N);
  if (!s) s = dmalloc(&b->lf, N);
  if (!s) s = dmalloc(&b->le, b->nec);
  if (!s) s = dmalloc(&b->ls, b->nsc);
  if (!s) s = dmalloc(&b->cnt, 8);
  if (!s) s = dmalloc(&b->listed, n);
  if (!s) s = dmalloc(&b->loff, 6 * (int64_t)n);
  if (!s) s = dmalloc(&b->st, n);
  if (!s) s = dmalloc(&b->part, 8 * b->nec + 2 * b->nsc);
  if (!s && cudaMallocHost((void **)&b->h_cnt, 8 * sizeof(int)) != cudaSuccess) s = A2C_ERR_NOMEM;
  auto up = [&](void *dst, const void *src, size_t bytes) {
    if (!s && bytes && cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) s = A2C_ERR_CUDA;
  };
  up(b->geo, geo.data(), sizeof(InstGeo) * n);
  up(b->inst, inst.data(), sizeof(uint16_t) * N);
  up(b->ech, ech.data(), sizeof(Chunk) * ech.size());
  up(b->sch, sch.data(), sizeof(Chunk) * sch.size());
  up(b->d_ecb, b->ecb.data(), sizeof(int) * (n + 1));
  up(b->d_scb, b->scb.data(), sizeof(int) * (n + 1));
  if (set_occ) up(b->c->d_occ, occ.data(), sizeof(double) * N);
  if (!s && cudaMemset(b->cnt, 0, 8 * sizeof(int)) != cudaSuccess) s = A2C_ERR_CUDA;
  return s;
}

// Set-up of a minimization: argument checks, L-BFGS buffers, constants,
// threads per site and the mixed form's tables (all outside any capture).
a2c_status setup_min(a2c_gpp_batch *b, const a2c_lbfgs_params *lp, Cfg &cf, Tile &tps) {
  if (lp->m < 1 || lp->m > kMaxM || lp->max_ls < 1 || !(lp->sigma_lb > 0.0) || !(lp->init_step > 0.0) ||
      lp->stall_window < 0 || lp->stall_window > 4096 || lp->max_fev < 1)
    return A2C_ERR_INVALID;
  a2c_gpp_ctx *c = b->c;
  if (!c->has_neighbors) return A2C_ERR_STATE;
  A2C_TRY(ensure_lbfgs(b, lp->m, lp->stall_window));
  const int64_t N = c->N;
  cf = Cfg{};
  cf.B = b->B;
  cf.m = lp->m;
  cf.ring = lp->m + 1;
  cf.max_it = lp->max_it;
  cf.max_fev = lp->max_fev;
  cf.max_ls = lp->max_ls;
  cf.polish = b->precision == A2C_MIXED ? lp->polish : 0;
  cf.W = lp->stall_window;
  cf.nec = b->nec;
  cf.nsc = b->nsc;
  cf.n = 4 * N;
  cf.gatol = lp->gatol;
  cf.c1 = lp->c1;
  cf.init_step = lp->init_step;
  cf.lb = lp->sigma_lb;
  cf.max_step = lp->max_step;
  cf.fn_mixed = lp->f_noise > 0.0 ? lp->f_noise : 1.0e-7;
  cf.fn_fp64 = lp->f_noise > 0.0 ? lp->f_noise : 1.0e-14;
  cf.st_mixed = lp->stall_rtol > 0.0 ? lp->stall_rtol : 1.0e-10;
  cf.st_fp64 = lp->stall_rtol > 0.0 ? lp->stall_rtol : 1.0e-14;
  tps = batch_tile(b);
  if (b->precision == A2C_MIXED) A2C_TRY(mixed_prepare(c));
  return A2C_OK;
}

// The launches that start a minimization from X (device or host memory):
// iterate, projection onto the bounds, per-instance records, site lists.
a2c_status start_min(a2c_gpp_batch *b, const Dev &D, const Cfg &cf, const double *X, bool dev) {
  cudaStream_t s = b->c->stream;
  A2C_CUDA(cudaMemcpyAsync(b->x, X, sizeof(double) * cf.n, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  k_project_all<<<chunk_grid((cf.n + 255) / 256), 256, 0, s>>>(b->x, cf.n, cf.lb);
  k_init_state<<<(b->B + 127) / 128, 128, 0, s>>>(D, cf, b->precision == A2C_MIXED ? kPhaseMixed : kPhaseFp64);
  A2C_CUDA(cudaMemsetAsync(b->listed, 0xff, sizeof(int) * b->B, s));  // -1: force a plan
  return plan(b, D);
}

// Ticks a minimization may take at most (each tick is at least one
// evaluation of every live instance; line searches and the polish add some).
int64_t max_ticks_for(const a2c_lbfgs_params *lp) { return 2 * ((int64_t)lp->max_fev + 2) + 16; }

// The minimization of every instance; X in/out on the host or (dev) on
// the device.  Per-instance results into the host arrays (any may be null)
// and, when `last` is given, the per-instance records.
a2c_status minimize_core(a2c_gpp_batch *b, double *X, bool dev, const a2c_lbfgs_params *lp, double *fmin, int *iters,
                         int *nfev, double *gnorm, int *reason, int *mixed_iters, int *fp64_iters,
                         std::vector<Inst> *last) {
  if (!b || !X || !lp) return A2C_ERR_INVALID;
  a2c_gpp_ctx *c = b->c;
  DeviceGuard2 dg(b->device);
  const int64_t N = c->N;
  if (!dev)
    for (int64_t t = 0; t < 4 * N; ++t)
      if (!std::isfinite(X[t])) return A2C_ERR_NONFINITE;
  Cfg cf{};
  Tile tps;
  A2C_TRY(setup_min(b, lp, cf, tps));
  cudaStream_t s = c->stream;
  Dev D = dev_view(b);
  cudaEvent_t e0, e1;
  A2C_CUDA(cudaEventCreate(&e0));
  A2C_CUDA(cudaEventCreate(&e1));
  a2c_status st = A2C_OK;
  auto fail = [&](a2c_status v) {
    if (!st) st = v;
  };
  cudaEventRecord(e0, s);
  fail(start_min(b, D, cf, X, dev));
  // the first tick (every instance's first evaluation) runs eagerly: it also
  // performs the launchers' one-time occupancy queries outside any capture
  if (!st) fail(tick(b, D, cf, tps));
  // the captured tick, reused while the configuration is unchanged
  const void *pass2[5];
  mixed_graph_key(c, pass2);
  const bool same = b->exec && b->exec_tile == tps && b->exec_nbr == (const void *)c->d_nbr &&
                    !std::memcmp(b->exec_pass2, pass2, sizeof(pass2)) && !std::memcmp(&b->exec_cfg, &cf, sizeof(Cfg));
  if (!st && b->graphs && !same) {
    if (b->exec) {
      cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    }
    cudaGraph_t gr = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) fail(A2C_ERR_CUDA);
    const a2c_status ts = st ? st : tick(b, D, cf, tps);
    if (cudaStreamEndCapture(s, &gr) != cudaSuccess) fail(A2C_ERR_CUDA);
    fail(ts);
    if (!st && cudaGraphInstantiate(&b->exec, gr, 0) != cudaSuccess) fail(A2C_ERR_CUDA);
    if (gr) cudaGraphDestroy(gr);
    b->exec_cfg = cf;
    b->exec_tile = tps;
    b->exec_nbr = c->d_nbr;
    std::memcpy(b->exec_pass2, pass2, sizeof(pass2));
  }
  // replay: K ticks, then read how many instances are left
  const int K = 8;
  const int64_t max_ticks = max_ticks_for(lp);
  int64_t ticks = 1;
  while (!st) {
    for (int k = 0; k < K; ++k) {
      if (b->graphs) {
        if (cudaGraphLaunch(b->exec, s) != cudaSuccess) fail(A2C_ERR_CUDA);
      } else {
        fail(tick(b, D, cf, tps));
      }
    }
    ticks += K;
    if (cudaMemcpyAsync(b->h_cnt, b->cnt, 7 * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(b->h_cnt + 7, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      fail(A2C_ERR_CUDA);
    // a span-guard flag ends the minimization: its gradients could be wrong
    if (!st && (b->h_cnt[7] & kStatusSpan)) fail(A2C_ERR_LISTS_STALE);
    if (st || b->h_cnt[kCntLeft] == 0) break;
    if (ticks >= max_ticks) {
      fail(A2C_ERR_STATE);
      break;
    }
  }
  cudaEventRecord(e1, s);
  if (!st && cudaMemcpyAsync(X, b->x, sizeof(double) * 4 * N, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             s) != cudaSuccess)
    fail(A2C_ERR_CUDA);
  std::vector<Inst> hs((size_t)b->B);
  if (!st && cudaMemcpyAsync(hs.data(), b->st, sizeof(Inst) * b->B, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    fail(A2C_ERR_CUDA);
  if (cudaMemcpyAsync(b->h_cnt + 7, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    fail(A2C_ERR_CUDA);
  if (cudaStreamSynchronize(s) != cudaSuccess) fail(A2C_ERR_CUDA);
  if (!st && (b->h_cnt[7] & kStatusSpan)) fail(A2C_ERR_LISTS_STALE);
  float ms = 0.0f;
  if (!st && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) b->seconds = 1e-3 * ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->ticks = (int)ticks;
  // a trial point with a non-finite objective is rejected by the line
  // search; it is not an error of the minimization
  cudaMemsetAsync(c->d_status, 0, sizeof(int), s);
  if (st) return st;
  for (int k = 0; k < b->B; ++k) {
    if (fmin) fmin[k] = hs[k].f;
    if (iters) iters[k] = hs[k].it;
    if (nfev) nfev[k] = hs[k].fev;
    if (gnorm) gnorm[k] = hs[k].gnorm;
    if (reason) reason[k] = hs[k].why;
    if (mixed_iters) mixed_iters[k] = hs[k].mixed_iters;
    if (fp64_iters) fp64_iters[k] = hs[k].phase == kPhaseFp64 ? hs[k].fp64_iters : 0;
  }
  if (last) last->swap(hs);
  c->has_state = true;
  return A2C_OK;
}


}  // namespace

extern "C" {

a2c_status a2c_gpp_batch_create(const a2c_gpp_params *params, int n, a2c_gpp_batch **out) {
  if (!out) return A2C_ERR_INVALID;
  *out = nullptr;
  if (!params || n < 1 || n > 65535) return A2C_ERR_INVALID;
  int64_t N = 0, nPd = 0, nH = 0;
  for (int b = 0; b < n; ++b) {
    const a2c_gpp_params &p = params[b];
    if (!same_common(p, params[0]) || p.nPd < 0 || p.nH < 0 || (int64_t)p.nPd + p.nH < 1 || !(p.T > 0.0))
      return A2C_ERR_INVALID;
    for (int d = 0; d < 3; ++d)
      if (p.periodic[d] && !(p.box[d] > 2.0 * p.rc)) return A2C_ERR_INVALID;
    N += (int64_t)p.nPd + p.nH;
    nPd += p.nPd;
    nH += p.nH;
  }
  if (N >= (int64_t(1) << kIdBits) || N > INT32_MAX / 4) return A2C_ERR_INVALID;
  a2c_gpp_params u = params[0];
  u.nPd = (int)nPd;
  u.nH = (int)nH;
  a2c_gpp_batch *b = new (std::nothrow) a2c_gpp_batch();
  if (!b) return A2C_ERR_NOMEM;
  b->B = n;
  b->device = u.device;
  b->precision = u.precision;
  b->P.assign(params, params + n);
  a2c_status s = a2c_gpp_create(&u, &b->c);
  if (s) {
    delete b;
    return s;
  }
  s = init_tables(b, params, n, true);
  bool any_free = false;
  for (int k = 0; k < n; ++k)
    for (int d = 0; d < 3; ++d) any_free = any_free || !params[k].periodic[d];
  if (!s && any_free && !b->c->d_xlist &&
      cudaMalloc(&b->c->d_xlist, sizeof(double) * 4 * (size_t)std::max<int64_t>(N, 1)) != cudaSuccess)
    s = A2C_ERR_NOMEM;
  if (s) {
    a2c_gpp_batch_destroy(b);
    return s;
  }
  *out = b;
  return A2C_OK;
}

a2c_status a2c_gpp_batch_destroy(a2c_gpp_batch *b) {
  if (!b) return A2C_OK;
  DeviceGuard dg(b->device);
  if (b->c && b->c->stream) cudaStreamSynchronize(b->c->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  free_lbfgs(b);
  for (void *p : {(void *)b->geo, (void *)b->inst, (void *)b->ech, (void *)b->sch, (void *)b->d_ecb, (void *)b->d_scb,
                  (void *)b->lm, (void *)b->lf, (void *)b->le, (void *)b->ls, (void *)b->cnt, (void *)b->listed,
                  (void *)b->loff, (void *)b->st, (void *)b->part})
    if (p) cudaFree(p);
  if (b->h_cnt) cudaFreeHost(b->h_cnt);
  if (!b->borrowed) a2c_gpp_destroy(b->c);
  delete b;
  return A2C_OK;
}

a2c_status a2c_gpp_batch_info(a2c_gpp_batch *b, int *n_instances, int64_t *n_sites) {
  if (!b) return A2C_ERR_INVALID;
  if (n_instances) *n_instances = b->B;
  if (n_sites) *n_sites = b->c->N;
  return A2C_OK;
}

a2c_status a2c_gpp_batch_set_occupancy(a2c_gpp_batch *b, const double *xH) {
  if (!b || (!xH && b->c->p.nH > 0)) return A2C_ERR_INVALID;
  DeviceGuard dg(b->device);
  std::vector<double> occ((size_t)b->c->N, 1.0);
  int64_t h = 0;
  for (int k = 0; k < b->B; ++k)
    for (int i = 0; i < b->P[k].nH; ++i) {
      const double v = xH[h++];
      if (!std::isfinite(v) || v < 0.0 || v > 1.0) return A2C_ERR_INVALID;
      occ[(size_t)(b->start[k] + b->P[k].nPd + i)] = v;
    }
  A2C_CUDA(cudaMemcpy(b->c->d_occ, occ.data(), sizeof(double) * occ.size(), cudaMemcpyHostToDevice));
  return A2C_OK;
}

a2c_status a2c_gpp_batch_build_neighbors(a2c_gpp_batch *b, const double *X, int *max_neighbors) {
  if (!b || !X) return A2C_ERR_INVALID;
  DeviceGuard dg(b->device);
  a2c_gpp_ctx *c = b->c;
  const int64_t N = c->N;
  for (int64_t t = 0; t < 4 * N; ++t)
    if (!std::isfinite(X[t])) return A2C_ERR_NONFINITE;
  if (b->exec) {  // the captured tick holds the list arrays' addresses
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  int64_t base = 0;
  int maxn = 0;
  for (int k = 0; k < b->B; ++k) {
    a2c_gpp_params p = b->P[k];
    p.precision = A2C_FP64;
    a2c_gpp_ctx *t = nullptr;
    A2C_TRY(a2c_gpp_create(&p, &t));
    int mk = 0;
    a2c_status s = a2c_gpp_build_neighbors(t, X + 4 * b->start[k], &mk);
    const int64_t nk = t->N, tot = t->nbr_total;
    if (!s && base + tot > c->nbr_cap) {  // grow, keeping what is there
      const int64_t cap = std::max<int64_t>(base + tot, 2 * c->nbr_cap);
      uint32_t *nn = nullptr;
      if (cudaMalloc(&nn, sizeof(uint32_t) * (size_t)cap) != cudaSuccess) s = A2C_ERR_NOMEM;
      if (!s && base > 0 && cudaMemcpy(nn, c->d_nbr, sizeof(uint32_t) * base, cudaMemcpyDeviceToDevice) != cudaSuccess)
        s = A2C_ERR_CUDA;
      if (!s) {
        if (c->d_nbr) cudaFree(c->d_nbr);
        c->d_nbr = nn;
        c->nbr_cap = cap;
      } else if (nn) {
        cudaFree(nn);
      }
    }
    if (!s) {
      const int64_t w = std::max(nk, tot);
      k_copy_csr<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((w + 255) / 256, 4096)), 256, 0, c->stream>>>(
          t->d_off, t->d_nbr, t->d_npd, nk, tot, b->start[k], base, c->d_off, c->d_nbr, c->d_npd);
      if (cudaStreamSynchronize(c->stream) != cudaSuccess) s = A2C_ERR_CUDA;
    }
    a2c_gpp_destroy(t);
    A2C_TRY(s);
    base += tot;
    maxn = std::max(maxn, mk);
  }
  k_set_i64<<<1, 1, 0, c->stream>>>(c->d_off + N, base);
  if (c->d_xlist && N > 0)  // span guard: the positions the lists were built at
    A2C_CUDA(cudaMemcpyAsync(c->d_xlist, X, sizeof(double) * 4 * N, cudaMemcpyHostToDevice, c->stream));
  A2C_CUDA(cudaStreamSynchronize(c->stream));
  c->nbr_total = base;
  c->max_neighbors = maxn;
  ++c->nbr_version;
  c->has_neighbors = true;
  if (max_neighbors) *max_neighbors = maxn;
  return A2C_OK;
}

a2c_status a2c_gpp_batch_set_threads_per_site(a2c_gpp_batch *b, int tps) {
  if (!b || (tps != 0 && tps != 1 && tps != 2 && tps != 4 && tps != 8)) return A2C_ERR_INVALID;
  b->tile.tps = tps;
  return A2C_OK;
}

a2c_status a2c_gpp_batch_set_graphs(a2c_gpp_batch *b, int on) {
  if (!b) return A2C_ERR_INVALID;
  b->graphs = on != 0;
  return A2C_OK;
}

// Per-instance objective (f[B]) and gradient (G[4N]) at X (4N), every
// instance in the batch's precision.
a2c_status a2c_gpp_batch_eval(a2c_gpp_batch *b, const double *X, double *f, double *G) {
  if (!b || !X || !f || !G) return A2C_ERR_INVALID;
  a2c_gpp_ctx *c = b->c;
  if (!c->has_neighbors) return A2C_ERR_STATE;
  DeviceGuard dg(b->device);
  const int64_t N = c->N;
  cudaStream_t s = c->stream;
  double *df = nullptr;
  A2C_TRY(dmalloc(&df, b->B));
  Dev D = dev_view(b);
  Cfg cf{};
  cf.B = b->B;
  cf.nec = b->nec;
  cf.nsc = b->nsc;
  cf.n = 4 * N;
  cf.fn_mixed = cf.fn_fp64 = 0.0;
  a2c_status st = A2C_OK;
  const int phase = b->precision == A2C_MIXED ? kPhaseMixed : kPhaseFp64;
  k_init_state<<<(b->B + 127) / 128, 128, 0, s>>>(D, cf, phase);
  if (cudaMemsetAsync(b->listed, 0xff, sizeof(int) * b->B, s) != cudaSuccess) st = A2C_ERR_CUDA;  // -1: force a plan
  if (!st && cudaMemsetAsync(c->d_status, 0, sizeof(int), s) != cudaSuccess) st = A2C_ERR_CUDA;
  if (!st) st = plan(b, D);
  if (!st && cudaMemcpyAsync(c->d_X, X, sizeof(double) * 4 * N, cudaMemcpyHostToDevice, s) != cudaSuccess)
    st = A2C_ERR_CUDA;
  if (!st) st = eval_lists(b, c->d_X, c->d_G, batch_tile(b));
  if (!st) {
    k_objpart<<<chunk_grid(b->nsc), kBlk, 0, s>>>(D, cf, 1);
    k_objective<<<b->B, kBlk, 0, s>>>(D, cf, df);
    if (cudaGetLastError() != cudaSuccess) st = A2C_ERR_CUDA;
  }
  if (!st && cudaMemcpyAsync(G, c->d_G, sizeof(double) * 4 * N, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    st = A2C_ERR_CUDA;
  if (!st && cudaMemcpyAsync(f, df, sizeof(double) * b->B, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    st = A2C_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess && !st) st = A2C_ERR_CUDA;
  cudaFree(df);
  if (!st) {
    c->has_state = true;
    st = check_status_word(c);
  }
  return st;
}

// Minimizes every instance from X (4N, in/out).  Per instance: fmin, iters,
// nfev, gnorm, reason (a2c_reason numbering), and, where not NULL,
// mixed_iters / fp64_iters (the mixed phase and the FP64 polish).
a2c_status a2c_gpp_batch_minimize(a2c_gpp_batch *b, double *X, const a2c_lbfgs_params *lp, double *fmin, int *iters,
                                  int *nfev, double *gnorm, int *reason, int *mixed_iters, int *fp64_iters) {
  if (!b || !X || !lp || !fmin || !iters || !nfev || !gnorm || !reason) return A2C_ERR_INVALID;
  return minimize_core(b, X, false, lp, fmin, iters, nfev, gnorm, reason, mixed_iters, fp64_iters, nullptr);
}

// Autotuner of the mixed form's threads per site over the whole batch at X
// (every instance listed): each choice evaluates once untimed, then `reps`
// times between two events; the fastest choice is kept for the batch.
namespace {
// Mean milliseconds of `reps` mixed evaluations of every instance at tile t
// (the state in c->d_X, every instance listed; one untimed evaluation first).
a2c_status time_batch_tile(a2c_gpp_batch *b, int reps, const Tile &t, float *ms) {
  a2c_gpp_ctx *c = b->c;
  cudaStream_t s = c->stream;
  A2C_TRY(mixed_eval_list(c, c->d_X, c->d_G, view(b, 0), t));
  cudaEvent_t e0, e1;
  A2C_CUDA(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return A2C_ERR_CUDA;
  }
  a2c_status st = cudaEventRecord(e0, s) == cudaSuccess ? A2C_OK : A2C_ERR_CUDA;
  for (int r = 0; r < reps && !st; ++r) st = mixed_eval_list(c, c->d_X, c->d_G, view(b, 0), t);
  if (!st && cudaEventRecord(e1, s) != cudaSuccess) st = A2C_ERR_CUDA;
  float v = 0.0f;
  if (!st && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&v, e0, e1) != cudaSuccess))
    st = A2C_ERR_CUDA;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = v / (float)reps;
  return st;
}

// Every instance listed, X on the device: the state the tuners time.
a2c_status tune_setup(a2c_gpp_batch *b, const double *X) {
  a2c_gpp_ctx *c = b->c;
  if (!c->has_neighbors) return A2C_ERR_STATE;
  cudaStream_t s = c->stream;
  A2C_TRY(mixed_prepare(c));
  Dev D = dev_view(b);
  Cfg cf{};
  cf.B = b->B;
  k_init_state<<<(b->B + 127) / 128, 128, 0, s>>>(D, cf, kPhaseMixed);
  A2C_CUDA(cudaMemsetAsync(b->listed, 0xff, sizeof(int) * b->B, s));
  A2C_TRY(plan(b, D));
  A2C_CUDA(cudaMemcpyAsync(c->d_X, X, sizeof(double) * 4 * c->N, cudaMemcpyHostToDevice, s));
  return A2C_OK;
}
}  // namespace

a2c_status a2c_gpp_batch_autotune(a2c_gpp_batch *b, const double *X, int reps, int *tps_out, float *ms) {
  if (!b || !X || reps < 1 || reps > 1000) return A2C_ERR_INVALID;
  DeviceGuard dg(b->device);
  A2C_TRY(tune_setup(b, X));
  const int choice[4] = {1, 2, 4, 8};
  float best_ms = 0.0f;
  int best = 0;
  for (int k = 0; k < 4; ++k) {
    float t = 0.0f;
    A2C_TRY(time_batch_tile(b, reps, Tile{choice[k], b->tile.rho_block, b->tile.grad_block}, &t));
    if (ms) ms[k] = t;
    if (best == 0 || t < best_ms) {
      best_ms = t;
      best = choice[k];
    }
  }
  b->tile.tps = best;
  if (tps_out) *tps_out = best;
  return check_status_word(b->c);
}

a2c_status a2c_gpp_batch_autotune_tile(a2c_gpp_batch *b, const double *X, int reps, int *tile, float *ms) {
  if (!b || !X || reps < 1 || reps > 1000) return A2C_ERR_INVALID;
  DeviceGuard dg(b->device);
  A2C_TRY(tune_setup(b, X));
  Tile best;
  A2C_TRY(tune_tile([&](const Tile &t, float *v) { return time_batch_tile(b, reps, t, v); }, &best, ms));
  b->tile = best;
  if (tile) {
    tile[0] = best.tps;
    tile[1] = best.rho_block;
    tile[2] = best.grad_block;
  }
  return check_status_word(b->c);
}

a2c_status a2c_gpp_batch_set_tile(a2c_gpp_batch *b, int tps, int rho_block, int grad_block) {
  if (!b || !valid_tile(tps, rho_block, grad_block)) return A2C_ERR_INVALID;
  b->tile = Tile{tps, rho_block, grad_block};
  return A2C_OK;
}

a2c_status a2c_gpp_batch_get_tile(a2c_gpp_batch *b, int *tile) {
  if (!b || !tile) return A2C_ERR_INVALID;
  const Tile t = batch_tile(b);
  tile[0] = t.tps;
  tile[1] = t.rho_block;
  tile[2] = t.grad_block;
  return A2C_OK;
}

// Ticks replayed and device seconds of the last a2c_gpp_batch_minimize.
a2c_status a2c_gpp_batch_stats(a2c_gpp_batch *b, int *ticks, double *seconds) {
  if (!b) return A2C_ERR_INVALID;
  if (ticks) *ticks = b->ticks;
  if (seconds) *seconds = b->seconds;
  return A2C_OK;
}

}  // extern "C"

namespace a2c {

// The device-driven minimizer for one context: the context wrapped as a
// one-instance batch (its buffers and lists borrowed), so an L-BFGS
// iteration is a captured tick replayed on the device instead of a host
// loop with a synchronization per scalar.  Created at the first call.
a2c_status engine_minimize(a2c_gpp_ctx *c, double *dX, const a2c_lbfgs_params *lp, double *fmin, int *iters,
                           int *nfev, double *gnorm, int *reason) {
  a2c_gpp_batch *b = (a2c_gpp_batch *)c->engine;
  if (!b) {
    b = new (std::nothrow) a2c_gpp_batch();
    if (!b) return A2C_ERR_NOMEM;
    b->B = 1;
    b->device = c->device;
    b->c = c;
    b->borrowed = true;
    b->P.assign(1, c->p);
    const a2c_status s = init_tables(b, &c->p, 1, false);
    if (s) {
      a2c_gpp_batch_destroy(b);
      return s;
    }
    c->engine = b;
  }
  b->precision = c->p.precision;
  b->tile = mixed_tile(c);
  {  // the context's lists may have changed since the tables were made
    InstGeo G{};
    set_limits(b, 0, G);
    A2C_CUDA(cudaMemcpy((char *)b->geo + offsetof(InstGeo, lim), G.lim, sizeof(G.lim), cudaMemcpyHostToDevice));
  }
  std::vector<Inst> last;
  int it = 0, fev = 0, why = 0;
  double f = 0.0, gn = 0.0;
  A2C_TRY(minimize_core(b, dX, true, lp, &f, &it, &fev, &gn, &why, nullptr, nullptr, &last));
  *fmin = f;
  *iters = it;
  *nfev = fev;
  *gnorm = gn;
  *reason = why;
  const Inst &I = last[0];
  c->last_mixed_iters = b->precision == A2C_MIXED ? I.mixed_iters : 0;
  c->last_fp64_iters = I.phase == kPhaseFp64 ? I.fp64_iters : 0;
  c->last_mixed_gnorm = b->precision == A2C_MIXED ? I.mixed_gnorm : 0.0;
  return A2C_OK;
}

void engine_free(a2c_gpp_ctx *c) {
  if (c->engine) a2c_gpp_batch_destroy((a2c_gpp_batch *)c->engine);
  c->engine = nullptr;
}

// ------------------------------------------------- DMD run as one graph
namespace {

// The L-BFGS tick loop's condition: continue while an instance is live,
// for at most max_ticks ticks (counters[1]); running out sets the timeout
// bit instead of looping on.
__global__ void k_tick_cond(cudaGraphConditionalHandle h, const int *cnt, int *counters, int max_ticks, int *status) {
  const int t = counters[1] + 1;
  counters[1] = t;
  const bool more = cnt[kCntLeft] > 0;
  if (more && t >= max_ticks) atomicOr(status, kStatusTimeout);
  cudaGraphSetConditional(h, (more && t < max_ticks) ? 1u : 0u);
}

__global__ void k_set_cond(cudaGraphConditionalHandle h, unsigned v) { cudaGraphSetConditional(h, v); }

// After a minimization: a trial point the line search rejected for a
// non-finite objective is not an error (the eager engine clears the word
// likewise); every other bit stays.
__global__ void k_status_keep(int *status, int keep) { *status &= keep; }

// End of an outer step: its records, the next step index, and the outer
// loop's condition (more steps, and no error bit set).
__global__ void k_dmd_record(const Inst *st, const double *macro, int *counters, double *rec, int nsteps,
                             const int *status, int fatal, cudaGraphConditionalHandle h) {
  const int k = counters[0];
  rec[4 * k] = macro[0];
  rec[4 * k + 1] = macro[1];
  rec[4 * k + 2] = st[0].f;
  rec[4 * k + 3] = (double)st[0].it;
  counters[0] = k + 1;
  counters[1] = 0;
  cudaGraphSetConditional(h, (k + 1 < nsteps && !(*status & fatal)) ? 1u : 0u);
}

// The launches of one outer step after its minimization (minimizer.cpp:588
// -> boundaryconditions.cpp:30 -> integrate.cpp:9 -> calculateresults.cpp:8),
// as the host-sequenced loop issues them (the chemical potential's pair
// quadrature in FP32 for the mixed form).
a2c_status dmd_post(a2c_gpp_ctx *c, const a2c_dmd_params *dp, const DmdDev &dd) {
  cudaStream_t s = c->stream;
  const int nH = c->p.nH;
  if (c->p.precision == A2C_MIXED) {
    A2C_TRY(mixed_chem(c, c->d_X, dd.send, dd.full));
  } else {
    A2C_TRY(launch_density64(c, c->d_X));
    A2C_TRY(launch_chem64(c, c->d_X, dp->gamma_bd, dd.send, dd.full));
  }
  A2C_TRY(launch_gamma_update(c, dd.send, dp->gamma_bd, dd.gamma, dd.full));
  A2C_TRY(launch_dirichlet(c, dd.bd, dd.n_bd, dp->gamma_bd, dp->x_bd, dd.gamma, dd.full));
  A2C_CUDA(cudaMemcpyAsync(dd.x, c->d_occ + c->p.nPd, sizeof(double) * nH, cudaMemcpyDeviceToDevice, s));
  A2C_TRY(launch_diffuse(c, dd.gamma, dd.full, dp->dt, dp->nu, dp->Qm, dp->xLb, dp->xUb, dd.x));
  A2C_CUDA(cudaMemcpyAsync(c->d_occ + c->p.nPd, dd.x, sizeof(double) * nH, cudaMemcpyDeviceToDevice, s));
  return launch_macro_device(c, dd.x, dd.surf, dd.n_surf, dd.macro);
}

}  // namespace

bool engine_dmd_graph_usable(const a2c_gpp_ctx *c, const a2c_dmd_params *dp) {
  if (!c->engine || dp->neighbor_update) return false;
  return (c->p.precision == A2C_MIXED && c->host_loop == A2C_MINIMIZER_DEFAULT) ||
         c->host_loop == A2C_MINIMIZER_DEVICE;
}

a2c_status engine_dmd_graph(a2c_gpp_ctx *c, const a2c_dmd_params *dp, const DmdDev &dd, int first, int nsteps) {
  a2c_gpp_batch *b = (a2c_gpp_batch *)c->engine;
  if (!b || first >= nsteps) return b ? A2C_OK : A2C_ERR_STATE;
  const a2c_lbfgs_params *lp = &dp->lbfgs;
  b->precision = c->p.precision;
  b->tile = mixed_tile(c);
  {
    InstGeo G{};
    set_limits(b, 0, G);
    A2C_CUDA(cudaMemcpy((char *)b->geo + offsetof(InstGeo, lim), G.lim, sizeof(G.lim), cudaMemcpyHostToDevice));
  }
  Cfg cf{};
  Tile tps;
  A2C_TRY(setup_min(b, lp, cf, tps));
  const Dev D = dev_view(b);
  cudaStream_t s = c->stream;
  const int init[2] = {first, 0};
  A2C_CUDA(cudaMemcpyAsync(dd.counters, init, sizeof(init), cudaMemcpyHostToDevice, s));
  A2C_CUDA(cudaStreamSynchronize(s));
  const int max_ticks = (int)std::min<int64_t>(max_ticks_for(lp), 1 << 30);
  const int fatal = kStatusBadIndex | kStatusOverflow | kStatusTimeout | kStatusNonfinite | kStatusSpan;

  a2c_status st = A2C_OK;
  auto fail = [&](a2c_status v) {
    if (!st) st = v;
  };
  auto cuda = [&](cudaError_t e) {
    if (e != cudaSuccess) fail(cuda_status(e));
  };
  cudaGraph_t G = nullptr;
  cudaGraphExec_t E = nullptr;
  cuda(cudaGraphCreate(&G, 0));
  // the loop over outer steps
  cudaGraphConditionalHandle hStep = 0, hTick = 0;
  cudaGraph_t bodyStep = nullptr, bodyTick = nullptr;
  if (!st) cuda(cudaGraphConditionalHandleCreate(&hStep, G, 1, cudaGraphCondAssignDefault));
  if (!st) {
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = hStep;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t n = nullptr;
    cuda(cudaGraphAddNode(&n, G, nullptr, nullptr, 0, &np));
    if (!st) bodyStep = np.conditional.phGraph_out[0];
  }
  if (!st) cuda(cudaGraphConditionalHandleCreate(&hTick, bodyStep, 1, cudaGraphCondAssignDefault));
  // one outer step: start the minimization, the tick loop, the rest
  if (!st && cudaStreamBeginCaptureToGraph(s, bodyStep, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
                 cudaSuccess) {
    fail(start_min(b, D, cf, c->d_X, true));
    k_set_cond<<<1, 1, 0, s>>>(hTick, 1u);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    if (!st) cuda(cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &nd));
    if (!st) {
      cudaGraphNodeParams tp{};
      tp.type = cudaGraphNodeTypeConditional;
      tp.conditional.handle = hTick;
      tp.conditional.type = cudaGraphCondTypeWhile;
      tp.conditional.size = 1;
      cudaGraphNode_t n = nullptr;
      cuda(cudaGraphAddNode(&n, cg, deps, nullptr, nd, &tp));
      if (!st) {
        bodyTick = tp.conditional.phGraph_out[0];
        cuda(cudaStreamUpdateCaptureDependencies(s, &n, nullptr, 1, cudaStreamSetCaptureDependencies));
      }
    }
    if (!st) {
      k_status_keep<<<1, 1, 0, s>>>(c->d_status, ~(int)kStatusNonfinite);
      cuda(cudaMemcpyAsync(c->d_X, b->x, sizeof(double) * cf.n, cudaMemcpyDeviceToDevice, s));
      fail(dmd_post(c, dp, dd));
      k_dmd_record<<<1, 1, 0, s>>>(D.st, dd.macro, dd.counters, dd.rec, nsteps, c->d_status, fatal, hStep);
      cuda(cudaGetLastError());
    }
    cudaGraph_t out = nullptr;
    cuda(cudaStreamEndCapture(s, &out));
  } else if (!st) {
    fail(A2C_ERR_CUDA);
  }
  // the tick loop's body: one L-BFGS tick and the loop condition
  if (!st && cudaStreamBeginCaptureToGraph(s, bodyTick, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
                 cudaSuccess) {
    fail(tick(b, D, cf, tps));
    k_tick_cond<<<1, 1, 0, s>>>(hTick, b->cnt, dd.counters, max_ticks, c->d_status);
    cuda(cudaGetLastError());
    cudaGraph_t out = nullptr;
    cuda(cudaStreamEndCapture(s, &out));
  } else if (!st) {
    fail(A2C_ERR_CUDA);
  }
  if (!st) cuda(cudaGraphInstantiate(&E, G, 0));
  if (!st) cuda(cudaGraphLaunch(E, s));
  cuda(cudaStreamSynchronize(s));
  if (E) cudaGraphExecDestroy(E);
  if (G) cudaGraphDestroy(G);
  (void)cudaGetLastError();
  return st;
}

}  // namespace a2c
