// FP64 kernels around the evaluator: the objective reduction, the
// chemical-potential update, the Dirichlet condition, the mean-field
// diffusion step and the macro results.  Compiled with -fmad=false.
#include <algorithm>
#include <cmath>

#include "ddmath.cuh"
#include "internal.cuh"

namespace a2c {
namespace {

constexpr int kRedBlock = 256;
constexpr int kRedGrid = 1024;  // fixed partition: the reduction order depends only on n

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
  if (w == 0) v = warp_sum(v);
  __syncthreads();
  return v;
}

// partial[b] = sum over a fixed strided slice of a and b arrays
__global__ void __launch_bounds__(kRedBlock) k_partial2(const double *a, const double *b, int64_t n, double *pa,
                                                         double *pb) {
  __shared__ double sh[kRedBlock / 32];
  double sa = 0.0, sb = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    sa += a[i];
    sb += b[i];
  }
  sa = block_sum(sa, sh);
  sb = block_sum(sb, sh);
  if (threadIdx.x == 0) {
    pa[blockIdx.x] = sa;
    pb[blockIdx.x] = sb;
  }
}

// f = (1/T)*sum_V - (3*kB)*sum_sigma  (minimizer.cpp:353)
__global__ void __launch_bounds__(kRedBlock) k_final_objective(const double *pa, const double *pb, int np, double T,
                                                                double *f, double *sums) {
  __shared__ double sh[kRedBlock / 32];
  double sa = 0.0, sb = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    sa += pa[i];
    sb += pb[i];
  }
  sa = block_sum(sa, sh);
  sb = block_sum(sb, sh);
  if (threadIdx.x == 0) {
    *f = 1.0 / T * sa - 3.0 * kB * sb;
    sums[0] = sa;
    sums[1] = sb;
  }
}

__global__ void k_finite(const double *d, int64_t n, int *status) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!isfinite(d[i])) {
      atomicOr(status, kStatusNonfinite);
      return;
    }
}

// minimizer.cpp:793-800
__global__ void k_gamma_update(const double *send, const double *xH, int nH, double gamma_bd, double *gamma,
                               int *full) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nH || full[i] == 1) return;
  double g = send[i] + 1.5;
  if (g > gamma_bd) {
    g = gamma_bd;
    if (xH[i] > 0.9999) full[i] = 1;
  }
  gamma[i] = g;
}

// boundaryconditions.cpp:47-51
__global__ void k_dirichlet(const int *sites, int n, double gamma_bd, double xUb, double *xH, double *gamma,
                            int *full, int nH, int *status) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = sites[t];
  if (i < 0 || i >= nH) {
    atomicOr(status, kStatusBadIndex);
    return;
  }
  gamma[i] = gamma_bd;
  full[i] = 1;
  xH[i] = xUb;
}

// integrate.cpp:26-81: explicit Euler step of the hop-rate master equation
// over the first H shell; sites with full_H == 1 keep their value.
__global__ void k_diffuse(const double *x0, const int64_t *hh1_off, const int *hh1, const double *gamma,
                          const int *full, int nH, double prefactor, double dt, double xLb, double xUb, double *x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nH || full[i] == 1) return;
  const double xi = x0[i];
  double x_deriv = 0.0;
  // per-site logs and exps use the correctly rounded dd:: forms (cheap here)
  const double fi = gamma[i] - dd::cr_log(xi / (1.0 - xi));
  for (int64_t t = hh1_off[i]; t < hh1_off[i + 1]; ++t) {
    const int j = hh1[t];
    const double xj = x0[j];
    const double fj = gamma[j] - dd::cr_log(xj / (1.0 - xj));
    x_deriv = x_deriv + (xj * (1.0 - xi) * dd::cr_exp(-(fi - fj) / 2.0) - xi * (1.0 - xj) * dd::cr_exp((fi - fj) / 2.0));
  }
  double v = xi + prefactor * x_deriv * dt;
  if (v < xLb) v = xLb;
  else if (v > xUb) v = xUb;
  x[i] = v;
}

__global__ void __launch_bounds__(kRedBlock) k_macro_partial(const double *x, const int *surf, int nH, double *pa,
                                                              double *pb) {
  __shared__ double sh[kRedBlock / 32];
  double sa = 0.0, sb = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nH; i += gridDim.x * blockDim.x) {
    sa += x[i];
    if (!surf[i]) sb += x[i];
  }
  sa = block_sum(sa, sh);
  sb = block_sum(sb, sh);
  if (threadIdx.x == 0) {
    pa[blockIdx.x] = sa;
    pb[blockIdx.x] = sb;
  }
}

__global__ void __launch_bounds__(kRedBlock) k_macro_final(const double *pa, const double *pb, int np, int nH,
                                                            int nSurf, double *out) {
  __shared__ double sh[kRedBlock / 32];
  double sa = 0.0, sb = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    sa += pa[i];
    sb += pb[i];
  }
  sa = block_sum(sa, sh);
  sb = block_sum(sb, sh);
  if (threadIdx.x == 0) {
    out[0] = sa / nH;
    out[1] = sb / (nH - nSurf);
  }
}

}  // namespace

// d_red layout: [0, kRedGrid) partial A, [kRedGrid, 2 kRedGrid) partial B,
// then scalars.
a2c_status reduce_objective(a2c_gpp_ctx *c, double *d_f) {
  double *pa = c->d_red, *pb = c->d_red + kRedGrid;
  const int64_t N = c->N;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(kRedGrid, (N + kRedBlock - 1) / kRedBlock));
  k_partial2<<<grid, kRedBlock, 0, c->stream>>>(c->d_Vs, c->d_Ss, N, pa, pb);
  A2C_CUDA(cudaGetLastError());
  k_final_objective<<<1, kRedBlock, 0, c->stream>>>(pa, pb, grid, c->p.T, d_f, c->d_red + 2 * kRedGrid);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

a2c_status launch_finite_check(a2c_gpp_ctx *c, const double *d, int64_t n) {
  if (n <= 0) return A2C_OK;
  const int grid = (int)std::min<int64_t>(1024, (n + 255) / 256);
  k_finite<<<grid, 256, 0, c->stream>>>(d, n, c->d_status);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

a2c_status launch_gamma_update(a2c_gpp_ctx *c, const double *d_send, double gamma_bd, double *d_gamma, int *d_full) {
  if (c->p.nH == 0) return A2C_OK;
  k_gamma_update<<<grid_for(c->p.nH, 256), 256, 0, c->stream>>>(d_send, c->d_occ + c->p.nPd, c->p.nH, gamma_bd,
                                                                d_gamma, d_full);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

a2c_status launch_dirichlet(a2c_gpp_ctx *c, const int *d_sites, int n, double gamma_bd, double xUb, double *d_gamma,
                            int *d_full) {
  if (n <= 0) return A2C_OK;
  k_dirichlet<<<grid_for(n, 256), 256, 0, c->stream>>>(d_sites, n, gamma_bd, xUb, c->d_occ + c->p.nPd, d_gamma,
                                                       d_full, c->p.nH, c->d_status);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

a2c_status launch_diffuse(a2c_gpp_ctx *c, const double *d_gamma, const int *d_full, double dt, double nu, double Qm,
                          double xLb, double xUb, double *d_x) {
  if (c->p.nH == 0) return A2C_OK;
  // integrate.cpp:26 (evaluated on the host, as the reference does)
  const double prefactor = nu * std::exp(-Qm / (kB * c->p.T));
  k_diffuse<<<grid_for(c->p.nH, 256), 256, 0, c->stream>>>(c->d_occ + c->p.nPd, c->d_hh1_off, c->d_hh1, d_gamma,
                                                           d_full, c->p.nH, prefactor, dt, xLb, xUb, d_x);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

a2c_status launch_macro_device(a2c_gpp_ctx *c, const double *d_x, const int *d_surf_flags, int nSurf, double *d_out) {
  const int nH = c->p.nH;
  double *pa = c->d_red, *pb = c->d_red + kRedGrid;
  const int grid = std::max(1, std::min(kRedGrid, (nH + kRedBlock - 1) / kRedBlock));
  k_macro_partial<<<grid, kRedBlock, 0, c->stream>>>(d_x, d_surf_flags, nH, pa, pb);
  A2C_CUDA(cudaGetLastError());
  k_macro_final<<<1, kRedBlock, 0, c->stream>>>(pa, pb, grid, nH, nSurf, d_out);
  A2C_CUDA(cudaGetLastError());
  return A2C_OK;
}

a2c_status launch_macro(a2c_gpp_ctx *c, const double *d_x, const int *d_surf_flags, int nSurf, double *h_xH,
                        double *h_xHint) {
  double *out = c->d_red + 2 * kRedGrid + 4;
  A2C_TRY(launch_macro_device(c, d_x, d_surf_flags, nSurf, out));
  double h[2];
  A2C_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  A2C_CUDA(cudaStreamSynchronize(c->stream));
  *h_xH = h[0];
  *h_xHint = h[1];
  return A2C_OK;
}

a2c_status check_status_word(a2c_gpp_ctx *c) {
  int st = 0;
  A2C_CUDA(cudaMemcpyAsync(&st, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  A2C_CUDA(cudaStreamSynchronize(c->stream));
  A2C_CUDA(cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream));
  if (st & kStatusBadIndex) return A2C_ERR_INVALID;
  if (st & kStatusOverflow) return A2C_ERR_NEIGHBOR_OVERFLOW;
  if (st & kStatusTimeout) return A2C_ERR_TIMEOUT;
  if (st & kStatusNonfinite) return A2C_ERR_NONFINITE;
  if (st & kStatusSpan) return A2C_ERR_LISTS_STALE;
  return A2C_OK;
}

}  // namespace a2c
