// Bound-constrained (projected) L-BFGS on the device, standing in for PETSc
// TAO BLMVM (minimizer.cpp:534-586; bounds sigma >= 1e-6 at 804-830).  TAO
// is not available to this build, so the algorithm is written out here and,
// step for step, in the CPU oracle:
//   pg = projected gradient (zero where sigma sits on its bound with g > 0)
//   stop when ||pg||_2 <= gatol (TAO's gatol test), or at the caps
//   d  = -H pg by the two-loop recursion over the last m pairs, H0 =
//        (s.y / y.y) I; zero on the active set; with no pairs (or if d is
//        not a descent direction) d = -pg * init_step / max|pg|
//   backtracking projected Armijo search from alpha = min(1, max_step /
//   max|d|) (no coordinate or width moves more than max_step in the first
//   trial), halving; when the
//   objective change is below its noise level (|f_new - f| <= f_noise |f|)
//   the step is accepted by the derivative form of the Armijo test,
//   g_new.s <= (2 c1 - 1) g.s, exact for a quadratic (the approximate-Wolfe
//   idea of Hager and Zhang, 2005) -- this keeps the mixed-precision form,
//   whose objective carries FP32 rounding noise, converging on its gradient
//   pair (s, y) kept when s.y > 2^-52 y.y
// Mixed precision with `polish`: when the mixed phase stops (gatol reached
// on the mixed gradient, or a failed line search), the iteration continues
// from the same point and memory with FP64 evaluations until gatol.
// All vector algebra is FP64 with fixed-partition (deterministic) block
// reductions; the objective is whichever form the context evaluates.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace a2c {

struct Lbfgs {
  int64_t n = 0;
  int m = 0;
  double *x = nullptr, *g = nullptr, *pg = nullptr, *d = nullptr, *xn = nullptr, *gn = nullptr;
  double *S = nullptr, *Y = nullptr;  // (m+1) x n each: a ring with one free slot
  double *red = nullptr;              // partials (kGrid x 4) + scalars
  double *f = nullptr, *fn = nullptr;
};

namespace {

constexpr int kBlock = 256;
constexpr int kGrid = 512;

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

__device__ __forceinline__ bool active(int64_t t, const double *x, const double *g, double lb) {
  return (t & 3) == 3 && x[t] <= lb && g[t] > 0.0;
}

// pg = projected g; partial[0] = sum pg^2, partial[1] = max |pg|
__global__ void __launch_bounds__(kBlock) k_projgrad(const double *x, const double *g, double *pg, int64_t n, double lb,
                                                      double *part) {
  __shared__ double sh[kBlock / 32];
  double s = 0.0, mx = 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const double v = active(t, x, g, lb) ? 0.0 : g[t];
    pg[t] = v;
    s += v * v;
    mx = fmax(mx, fabs(v));
  }
  s = bred<false>(s, sh);
  mx = bred<true>(mx, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s;
    part[2 * blockIdx.x + 1] = mx;
  }
}

// out[0] = sum of column 0, out[1] = max of column 1
__global__ void __launch_bounds__(kBlock) k_final_sum_max(const double *part, int np, double *out) {
  __shared__ double sh[kBlock / 32];
  double s = 0.0, mx = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    s += part[2 * i];
    mx = fmax(mx, part[2 * i + 1]);
  }
  s = bred<false>(s, sh);
  mx = bred<true>(mx, sh);
  if (threadIdx.x == 0) {
    out[0] = s;
    out[1] = mx;
  }
}

// generic dot products: part[k*np + b] for k < nd
__global__ void __launch_bounds__(kBlock) k_dot2(const double *a0, const double *b0, const double *a1,
                                                  const double *b1, int64_t n, double *part) {
  __shared__ double sh[kBlock / 32];
  double s0 = 0.0, s1 = 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    s0 += a0[t] * b0[t];
    if (a1) s1 += a1[t] * b1[t];
  }
  s0 = bred<false>(s0, sh);
  s1 = bred<false>(s1, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s0;
    part[2 * blockIdx.x + 1] = s1;
  }
}

__global__ void __launch_bounds__(kBlock) k_final_sum2(const double *part, int np, double *out) {
  __shared__ double sh[kBlock / 32];
  double s0 = 0.0, s1 = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    s0 += part[2 * i];
    s1 += part[2 * i + 1];
  }
  s0 = bred<false>(s0, sh);
  s1 = bred<false>(s1, sh);
  if (threadIdx.x == 0) {
    out[0] = s0;
    out[1] = s1;
  }
}

__global__ void k_scale(const double *a, double c, double *out, int64_t n) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    out[t] = a[t] * c;
}

// q -= alpha * y   (alpha read from device memory)
__global__ void k_axpy_dev(double *q, const double *y, const double *alpha, double sgn, int64_t n) {
  const double a = *alpha * sgn;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    q[t] -= a * y[t];
}

// q += (alpha - beta) * s
__global__ void k_axpy_ab(double *q, const double *s, const double *alpha, const double *beta_dot, double rho,
                          int64_t n) {
  const double c = *alpha - rho * *beta_dot;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    q[t] += c * s[t];
}

__global__ void k_neg_mask(double *d, const double *x, const double *g, int64_t n, double lb) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    d[t] = active(t, x, g, lb) ? 0.0 : -d[t];
}

// xn = P(x + alpha d); part = g . (xn - x)
__global__ void __launch_bounds__(kBlock) k_trial(const double *x, const double *d, const double *g, double alpha,
                                                   double lb, double *xn, int64_t n, double *part) {
  __shared__ double sh[kBlock / 32];
  double s = 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    double v = x[t] + alpha * d[t];
    if ((t & 3) == 3 && v < lb) v = lb;
    xn[t] = v;
    s += g[t] * (v - x[t]);
  }
  s = bred<false>(s, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s;
    part[2 * blockIdx.x + 1] = 0.0;
  }
}

// part = (0, max |d|)
__global__ void __launch_bounds__(kBlock) k_absmax(const double *d, int64_t n, double *part) {
  __shared__ double sh[kBlock / 32];
  double mx = 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    mx = fmax(mx, fabs(d[t]));
  mx = bred<true>(mx, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = 0.0;
    part[2 * blockIdx.x + 1] = mx;
  }
}

// S = xn - x, Y = gn - g; part = (s.y, y.y)
__global__ void __launch_bounds__(kBlock) k_pair(const double *x, const double *xn, const double *g, const double *gn,
                                                  double *S, double *Y, int64_t n, double *part) {
  __shared__ double sh[kBlock / 32];
  double sy = 0.0, yy = 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const double s = xn[t] - x[t], y = gn[t] - g[t];
    S[t] = s;
    Y[t] = y;
    sy += s * y;
    yy += y * y;
  }
  sy = bred<false>(sy, sh);
  yy = bred<false>(yy, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sy;
    part[2 * blockIdx.x + 1] = yy;
  }
}

// part = g_new . (xn - x)
__global__ void __launch_bounds__(kBlock) k_dot_step(const double *gn, const double *xn, const double *x, int64_t n,
                                                      double *part) {
  __shared__ double sh[kBlock / 32];
  double s = 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    s += gn[t] * (xn[t] - x[t]);
  s = bred<false>(s, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s;
    part[2 * blockIdx.x + 1] = 0.0;
  }
}

__global__ void k_project(double *x, int64_t n, double lb) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    if ((t & 3) == 3 && x[t] < lb) x[t] = lb;
}

int grid_n(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(kGrid, (n + kBlock - 1) / kBlock)); }

}  // namespace

void lbfgs_free(a2c_gpp_ctx *c) {
  Lbfgs *L = c->lbfgs;
  if (!L) return;
  for (double *p : {L->x, L->g, L->pg, L->d, L->xn, L->gn, L->S, L->Y, L->red}) cudaFree(p);
  delete L;
  c->lbfgs = nullptr;
}

static a2c_status lbfgs_alloc(a2c_gpp_ctx *c, int m) {
  const int64_t n = 4 * c->N;
  if (c->lbfgs && c->lbfgs->n == n && c->lbfgs->m == m) return A2C_OK;
  lbfgs_free(c);
  Lbfgs *L = new Lbfgs;
  c->lbfgs = L;
  L->n = n;
  L->m = m;
  const size_t b = sizeof(double) * (size_t)std::max<int64_t>(n, 1);
  for (double **p : {&L->x, &L->g, &L->pg, &L->d, &L->xn, &L->gn})
    if (cudaMalloc(p, b) != cudaSuccess) return A2C_ERR_NOMEM;
  if (cudaMalloc(&L->S, b * (m + 1)) != cudaSuccess || cudaMalloc(&L->Y, b * (m + 1)) != cudaSuccess)
    return A2C_ERR_NOMEM;
  if (cudaMalloc(&L->red, sizeof(double) * (2 * kGrid + 64)) != cudaSuccess) return A2C_ERR_NOMEM;
  L->f = L->red + 2 * kGrid;
  L->fn = L->f + 1;
  return A2C_OK;
}

a2c_status lbfgs_minimize(a2c_gpp_ctx *c, double *dX, const a2c_lbfgs_params *lp, double *fmin, int *iters, int *nfev,
                          double *gnorm_out, int *reason) {
  if (!lp || lp->m < 1 || lp->m > 48 || lp->max_ls < 1 || !(lp->sigma_lb > 0.0) || !(lp->init_step > 0.0))
    return A2C_ERR_INVALID;
  // Mixed precision: the same algorithm driven on the device (batch.cu, one
  // instance; its global sums in the per-instance chunk order) unless the
  // host loop below is asked for.  The FP64 plain form keeps the host loop,
  // whose reductions the oracle replays bit for bit, unless the device
  // engine is asked for.
  if ((c->p.precision == A2C_MIXED && c->host_loop == A2C_MINIMIZER_DEFAULT) || c->host_loop == A2C_MINIMIZER_DEVICE)
    return engine_minimize(c, dX, lp, fmin, iters, nfev, gnorm_out, reason);
  A2C_TRY(lbfgs_alloc(c, lp->m));
  Lbfgs *L = c->lbfgs;
  cudaStream_t st = c->stream;
  const int64_t n = L->n;
  const int gr = grid_n(n), m = lp->m, ring = m + 1;
  const double lb = lp->sigma_lb;
  double *part = L->red, *scal = L->red + 2 * kGrid + 2;  // scal[0..61]: sums, alphas
  auto fetch = [&](const double *src, double *dst, int k) -> a2c_status {
    A2C_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * k, cudaMemcpyDeviceToHost, st));
    A2C_CUDA(cudaStreamSynchronize(st));
    return A2C_OK;
  };
  auto dot2 = [&](const double *a0, const double *b0, const double *a1, const double *b1, double *out) {
    k_dot2<<<gr, kBlock, 0, st>>>(a0, b0, a1, b1, n, part);
    k_final_sum2<<<1, kBlock, 0, st>>>(part, gr, out);
  };

  A2C_CUDA(cudaMemcpyAsync(L->x, dX, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  k_project<<<gr, kBlock, 0, st>>>(L->x, n, lb);
  const int saved_precision = c->p.precision;
  int fev = 0;
  double f = 0.0;
  // pairs occupy slots head-1, ..., head-npairs (mod m+1); slot head is free,
  // so a rejected pair never overwrites a live one
  std::vector<double> rhoS(ring, 0.0);
  int npairs = 0, head = 0, it = 0, why = 0;
  double gnorm = 0.0;
  c->last_mixed_iters = c->last_fp64_iters = 0;
  c->last_mixed_gnorm = 0.0;

  std::vector<double> fhist;  // f after each accepted iteration of the phase
  auto phase = [&](double f_noise, double stall_rtol) -> a2c_status {
    fhist.clear();
    A2C_TRY(eval_device_impl(c, L->x, L->f, L->g));
    ++fev;
    A2C_TRY(fetch(L->f, &f, 1));
    while (true) {
      k_projgrad<<<gr, kBlock, 0, st>>>(L->x, L->g, L->pg, n, lb, part);
      k_final_sum_max<<<1, kBlock, 0, st>>>(part, gr, scal);
      double sm[2];
      A2C_TRY(fetch(scal, sm, 2));
      gnorm = std::sqrt(sm[0]);
      const double amax = sm[1];
      if (!std::isfinite(f) || !std::isfinite(gnorm)) { why = A2C_DIVERGED_NAN; break; }
      if (gnorm <= lp->gatol) { why = A2C_CONVERGED_GATOL; break; }
      if (it >= lp->max_it) { why = A2C_DIVERGED_MAXITS; break; }
      if (fev >= lp->max_fev) { why = A2C_DIVERGED_MAXFCN; break; }
      auto steepest = [&]() { k_scale<<<gr, kBlock, 0, st>>>(L->pg, -lp->init_step / amax, L->d, n); };
      if (npairs == 0) {
        steepest();
      } else {
        // two-loop recursion; alpha_j kept in scal[4 + j]
        A2C_CUDA(cudaMemcpyAsync(L->d, L->pg, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        for (int k = 0; k < npairs; ++k) {
          const int sl = ((head - 1 - k) % ring + ring) % ring;
          dot2(L->S + (size_t)sl * n, L->d, nullptr, nullptr, scal + 2);
          k_scale<<<1, 1, 0, st>>>(scal + 2, rhoS[sl], scal + 4 + sl, 1);  // alpha = rho (s . q)
          k_axpy_dev<<<gr, kBlock, 0, st>>>(L->d, L->Y + (size_t)sl * n, scal + 4 + sl, 1.0, n);
        }
        const int nw = ((head - 1) % ring + ring) % ring;
        double sy_yy[2];
        dot2(L->S + (size_t)nw * n, L->Y + (size_t)nw * n, L->Y + (size_t)nw * n, L->Y + (size_t)nw * n, scal + 2);
        A2C_TRY(fetch(scal + 2, sy_yy, 2));
        k_scale<<<gr, kBlock, 0, st>>>(L->d, sy_yy[0] / sy_yy[1], L->d, n);
        for (int k = npairs - 1; k >= 0; --k) {
          const int sl = ((head - 1 - k) % ring + ring) % ring;
          dot2(L->Y + (size_t)sl * n, L->d, nullptr, nullptr, scal + 2);
          k_axpy_ab<<<gr, kBlock, 0, st>>>(L->d, L->S + (size_t)sl * n, scal + 4 + sl, scal + 2, rhoS[sl], n);
        }
        k_neg_mask<<<gr, kBlock, 0, st>>>(L->d, L->x, L->g, n, lb);
      }
      double gd[2];
      dot2(L->g, L->d, nullptr, nullptr, scal + 2);
      A2C_TRY(fetch(scal + 2, gd, 1));
      if (!(gd[0] < 0.0)) {
        npairs = 0;
        head = 0;
        steepest();
      }
      double alpha = 1.0, fn = 0.0;
      if (lp->max_step > 0.0) {
        double dm[2];
        k_absmax<<<gr, kBlock, 0, st>>>(L->d, n, part);
        k_final_sum_max<<<1, kBlock, 0, st>>>(part, gr, scal + 2);
        A2C_TRY(fetch(scal + 2, dm, 2));
        if (dm[1] > lp->max_step) alpha = lp->max_step / dm[1];
      }
      bool ok = false;
      for (int ls = 0; ls < lp->max_ls; ++ls) {
        k_trial<<<gr, kBlock, 0, st>>>(L->x, L->d, L->g, alpha, lb, L->xn, n, part);
        k_final_sum2<<<1, kBlock, 0, st>>>(part, gr, scal + 2);
        A2C_TRY(eval_device_impl(c, L->xn, L->fn, L->gn));
        ++fev;
        double v[2];
        A2C_TRY(fetch(scal + 2, v, 1));
        A2C_TRY(fetch(L->fn, &fn, 1));
        if (std::isfinite(fn) && fn <= f + lp->c1 * v[0]) { ok = true; break; }
        if (std::isfinite(fn) && std::fabs(fn - f) <= f_noise * std::fabs(f)) {
          double dn[2];
          k_dot_step<<<gr, kBlock, 0, st>>>(L->gn, L->xn, L->x, n, part);
          k_final_sum2<<<1, kBlock, 0, st>>>(part, gr, scal + 2);
          A2C_TRY(fetch(scal + 2, dn, 1));
          if (dn[0] <= (2.0 * lp->c1 - 1.0) * v[0]) { ok = true; break; }
        }
        alpha *= 0.5;
        if (fev >= lp->max_fev) break;
      }
      if (!ok) {
        if (npairs > 0 && fev < lp->max_fev) {
          npairs = 0;
          head = 0;
          continue;
        }
        why = (fev >= lp->max_fev) ? A2C_DIVERGED_MAXFCN : A2C_DIVERGED_LS_FAILURE;
        break;
      }
      k_pair<<<gr, kBlock, 0, st>>>(L->x, L->xn, L->g, L->gn, L->S + (size_t)head * n, L->Y + (size_t)head * n, n,
                                    part);
      k_final_sum2<<<1, kBlock, 0, st>>>(part, gr, scal + 2);
      double sy[2];
      A2C_TRY(fetch(scal + 2, sy, 2));
      if (sy[0] > 2.220446049250313e-16 * sy[1]) {
        rhoS[head] = 1.0 / sy[0];
        head = (head + 1) % ring;
        if (npairs < m) ++npairs;
      }
      std::swap(L->x, L->xn);
      std::swap(L->g, L->gn);
      f = fn;
      ++it;
      fhist.push_back(f);
      const int W = lp->stall_window;
      if (W > 0 && (int)fhist.size() > W && fhist[fhist.size() - 1 - W] - f <= stall_rtol * std::fabs(f)) {
        why = A2C_CONVERGED_STALLED;
        break;
      }
    }
    return A2C_OK;
  };

  a2c_status st_run;
  if (saved_precision == A2C_MIXED) {
    st_run = phase(lp->f_noise > 0.0 ? lp->f_noise : 1.0e-7, lp->stall_rtol > 0.0 ? lp->stall_rtol : 1.0e-10);
    c->last_mixed_iters = it;
    c->last_mixed_gnorm = gnorm;
    if (st_run == A2C_OK && lp->polish &&
        (why == A2C_CONVERGED_GATOL || why == A2C_DIVERGED_LS_FAILURE || why == A2C_CONVERGED_STALLED)) {
      c->p.precision = A2C_FP64;
      const int it0 = it;
      st_run = phase(lp->f_noise > 0.0 ? lp->f_noise : 1.0e-14, lp->stall_rtol > 0.0 ? lp->stall_rtol : 1.0e-14);
      c->last_fp64_iters = it - it0;
      c->p.precision = saved_precision;
    }
  } else {
    st_run = phase(lp->f_noise > 0.0 ? lp->f_noise : 1.0e-14, lp->stall_rtol > 0.0 ? lp->stall_rtol : 1.0e-14);
    c->last_fp64_iters = it;
  }
  c->p.precision = saved_precision;
  A2C_TRY(st_run);
  A2C_CUDA(cudaMemcpyAsync(dX, L->x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  int word = 0;  // the mixed form's span guard (a rejected non-finite trial is not an error here)
  A2C_CUDA(cudaMemcpyAsync(&word, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  A2C_CUDA(cudaStreamSynchronize(st));
  if (word & kStatusSpan) {
    A2C_CUDA(cudaMemsetAsync(c->d_status, 0, sizeof(int), st));
    return A2C_ERR_LISTS_STALE;
  }
  *fmin = f;
  *iters = it;
  *nfev = fev;
  *gnorm_out = gnorm;
  *reason = why;
  return A2C_OK;
}

}  // namespace a2c
