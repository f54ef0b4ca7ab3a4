// The C ABI (include/a2c_gpp.h): context lifecycle, host<->device staging,
// validation and the order of kernel launches.  No function here aborts,
// traps or lets a C++ exception cross the boundary; every failure returns
// an a2c_status.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "internal.cuh"

namespace a2c {

a2c_status cuda_status(cudaError_t e) {
  switch (e) {
    case cudaSuccess: return A2C_OK;
    case cudaErrorMemoryAllocation: return A2C_ERR_NOMEM;
    case cudaErrorNoDevice:
    case cudaErrorInsufficientDriver:
    case cudaErrorInvalidDevice: return A2C_ERR_NO_DEVICE;
    default: return A2C_ERR_CUDA;
  }
}

int device_sms(int dev) {
  static std::mutex m;
  static int cache[kMaxDevices] = {};
  if (dev < 0 || dev >= kMaxDevices) return 1;
  std::lock_guard<std::mutex> lock(m);
  if (!cache[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
      (void)cudaGetLastError();
      return 1;  // not cached: asked again next time
    }
    cache[dev] = n;
  }
  return cache[dev];
}

void span_limits(const a2c_gpp_ctx *c, double lim[3], const double **xlist) {
  bool any = false;
  for (int d = 0; d < 3; ++d) {
    if (c->p.periodic[d]) {
      lim[d] = HUGE_VAL;
    } else {
      any = true;
      lim[d] = std::isfinite(c->list_reach[d]) ? 0.5 * (0.5 * kFreeSpan - c->list_reach[d]) : -HUGE_VAL;
    }
  }
  *xlist = any ? c->d_xlist : nullptr;
}

int current_device_sms() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return 1;
  }
  return device_sms(dev);
}

a2c_status eval_device_impl(a2c_gpp_ctx *c, const double *dX, double *d_f, double *dG, cudaEvent_t *ev) {
  if (!c->has_neighbors) return A2C_ERR_STATE;
  if (c->p.precision == A2C_MIXED) {
    A2C_TRY(mixed_eval(c, dX, d_f, dG, ev));
  } else {
    if (ev) cudaEventRecord(ev[0], c->stream);
    if (ev) cudaEventRecord(ev[1], c->stream);
    A2C_TRY(launch_density64(c, dX));
    if (ev) cudaEventRecord(ev[2], c->stream);
    A2C_TRY(launch_gradient64(c, dX, dG));
    if (ev) cudaEventRecord(ev[3], c->stream);
    A2C_TRY(reduce_objective(c, d_f));
    if (ev) cudaEventRecord(ev[4], c->stream);
  }
  c->has_density = (c->p.precision != A2C_MIXED);
  return A2C_OK;
}

// Mean milliseconds of `reps` mixed evaluations of the context's current
// state at tile t (after one untimed evaluation).
a2c_status time_context_tile(a2c_gpp_ctx *c, int reps, const Tile &t, float *ms) {
  double *d_f = c->d_red + 2 * 1024 + 8;
  A2C_TRY(mixed_set_tile(c, t));
  A2C_TRY(eval_device_impl(c, c->d_X, d_f, c->d_G));
  cudaEvent_t e0, e1;
  A2C_CUDA(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return A2C_ERR_CUDA;
  }
  a2c_status s = cudaEventRecord(e0, c->stream) == cudaSuccess ? A2C_OK : A2C_ERR_CUDA;
  for (int r = 0; r < reps && !s; ++r) s = eval_device_impl(c, c->d_X, d_f, c->d_G);
  if (!s && cudaEventRecord(e1, c->stream) != cudaSuccess) s = A2C_ERR_CUDA;
  float t_ms = 0.0f;
  if (!s && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&t_ms, e0, e1) != cudaSuccess))
    s = A2C_ERR_CUDA;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t_ms / (float)reps;
  return s;
}

a2c_status tune_tile(const std::function<a2c_status(const Tile &, float *)> &time_tile, Tile *best, float *ms) {
  static const int tps_c[4] = {1, 2, 4, 8}, rho_c[3] = {256, 512, 768}, grad_c[3] = {128, 256, 512};
  Tile b;
  b.rho_block = 256;
  b.grad_block = 256;
  float best_ms = 0.0f;
  int k = 0;
  auto trial = [&](const Tile &t) -> a2c_status {
    float v = 0.0f;
    A2C_TRY(time_tile(t, &v));
    if (ms) ms[k] = v;
    ++k;
    if (b.tps == 0 || v < best_ms) {
      best_ms = v;
      b = t;
    }
    return A2C_OK;
  };
  for (int q : tps_c) A2C_TRY(trial(Tile{q, 256, 256}));
  const Tile after_tps = b;
  for (int q : rho_c) A2C_TRY(trial(Tile{after_tps.tps, q, after_tps.grad_block}));
  const Tile after_rho = b;
  for (int q : grad_c) A2C_TRY(trial(Tile{after_rho.tps, after_rho.rho_block, q}));
  *best = b;
  return A2C_OK;
}

}  // namespace a2c

using namespace a2c;

namespace {

bool valid_params(const a2c_gpp_params *p) {
  if (!p) return false;
  if (p->nPd < 0 || p->nH < 0) return false;
  if ((int64_t)p->nPd + p->nH >= (int64_t(1) << kIdBits)) return false;
  if (!(p->T > 0.0) || !(p->eps > 0.0) || !(p->rc > 0.0) || !std::isfinite(p->QWp)) return false;
  if (!std::isfinite(p->a_Pd)) return false;
  for (int d = 0; d < 3; ++d)
    if (p->periodic[d] && !(p->box[d] > 2.0 * p->rc)) return false;
  if (p->precision != A2C_FP64 && p->precision != A2C_MIXED) return false;
  return true;
}

struct DeviceGuard {
  explicit DeviceGuard(int d) { cudaSetDevice(d); }
};

// Host memory the device can address directly (pinned or registered): its
// device-side address, else null.
const void *mapped(const void *p) {
  cudaPointerAttributes a;
  if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

a2c_status copy_in(a2c_gpp_ctx *c, double *dst, const double *src, int64_t n) {
  if (n <= 0) return A2C_OK;
  A2C_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  return A2C_OK;
}

a2c_status finish(a2c_gpp_ctx *c) {
  A2C_CUDA(cudaStreamSynchronize(c->stream));
  return check_status_word(c);
}

template <class T>
a2c_status dalloc(T **p, int64_t n) {
  if (cudaMalloc((void **)p, sizeof(T) * (size_t)std::max<int64_t>(n, 1)) != cudaSuccess) return A2C_ERR_NOMEM;
  return A2C_OK;
}

// per-call scratch on H sites (stream-ordered allocations)
a2c_status ensure_hscratch(a2c_gpp_ctx *c, double **gamma, double **send, double **x, int **full) {
  const int64_t nH = std::max(c->p.nH, 1);
  A2C_CUDA(cudaMallocAsync((void **)gamma, sizeof(double) * nH, c->stream));
  A2C_CUDA(cudaMallocAsync((void **)send, sizeof(double) * nH, c->stream));
  A2C_CUDA(cudaMallocAsync((void **)x, sizeof(double) * nH, c->stream));
  A2C_CUDA(cudaMallocAsync((void **)full, sizeof(int) * nH, c->stream));
  return A2C_OK;
}

void free_hscratch(a2c_gpp_ctx *c, double *gamma, double *send, double *x, int *full) {
  cudaFreeAsync(gamma, c->stream);
  cudaFreeAsync(send, c->stream);
  cudaFreeAsync(x, c->stream);
  cudaFreeAsync(full, c->stream);
}

// The snapshot in flight: pinned copies of the state, the host-side
// arrays, and the writer thread.
struct SnapJob {
  std::thread th;
  double *pinned = nullptr;
  size_t cap = 0;
  cudaEvent_t ev = nullptr;
  a2c_status result = A2C_OK;
  std::string prefix;
  a2c_snapshot_desc desc{};
  std::vector<double> X0, gamma;
  std::vector<signed char> siteid, tag;
};

a2c_status snapshot_join(a2c_gpp_ctx *c) {
  SnapJob *j = (SnapJob *)c->snap;
  if (!j) return A2C_OK;
  if (j->th.joinable()) j->th.join();
  const a2c_status r = j->result;
  j->result = A2C_OK;
  return r;
}

void snapshot_release(a2c_gpp_ctx *c) {
  SnapJob *j = (SnapJob *)c->snap;
  if (!j) return;
  snapshot_join(c);
  if (j->pinned) cudaFreeHost(j->pinned);
  if (j->ev) cudaEventDestroy(j->ev);
  delete j;
  c->snap = nullptr;
}

__global__ void k_fill(double *p, int64_t n, double v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

}  // namespace

extern "C" {

void a2c_gpp_default_params(a2c_gpp_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->T = 300.0;           // DiffusionData::T0 default (IoData.cpp:626)
  p->QWp = 1.0 / 12.0;    // 0.5/dim for dim = 6 (quadrature.cpp:96-97)
  p->eps = 1.0e-5;        // InteratomicPotentialData::eps (IoData.cpp:517)
  p->rc = 5.35;           // InteratomicPotentialData::rc (IoData.cpp:518)
  p->a_Pd = 3.89;
  p->precision = A2C_FP64;
  p->device = 0;
}

void a2c_lbfgs_default_params(a2c_lbfgs_params *p) {
  if (!p) return;
  p->m = 5;
  p->max_it = 10000;
  p->max_fev = 20000;
  p->max_ls = 30;
  p->gatol = 1.0e-6;
  p->c1 = 1.0e-4;
  p->init_step = 1.0e-2;
  p->sigma_lb = 1.0e-6;
  p->f_noise = 0.0;
  p->polish = 1;
  p->stall_window = 50;
  p->stall_rtol = 0.0;
  p->max_step = 0.25;
}

const char *a2c_status_string(a2c_status s) {
  switch (s) {
    case A2C_OK: return "ok";
    case A2C_ERR_INVALID: return "invalid argument";
    case A2C_ERR_CUDA: return "CUDA runtime error";
    case A2C_ERR_NOMEM: return "device allocation failed";
    case A2C_ERR_NEIGHBOR_OVERFLOW: return "neighbor capacity exceeded (more than 1000 neighbors at a site)";
    case A2C_ERR_NONFINITE: return "non-finite value in an input or result";
    case A2C_ERR_STATE: return "call order violated (build neighbors / set state first)";
    case A2C_ERR_TIMEOUT: return "bounded device wait gave up";
    case A2C_ERR_NO_DEVICE: return "no usable CUDA device";
    case A2C_ERR_LISTS_STALE:
      return "mixed form: a site moved too far in a free direction since the neighbor lists were built; rebuild them";
    default: return "unknown status";
  }
}

a2c_status a2c_gpp_create(const a2c_gpp_params *p, a2c_gpp_ctx **out) {
  if (!out) return A2C_ERR_INVALID;
  *out = nullptr;
  if (!valid_params(p)) return A2C_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return A2C_ERR_NO_DEVICE;
  if (p->device < 0 || p->device >= ndev) return A2C_ERR_NO_DEVICE;
  A2C_CUDA(cudaSetDevice(p->device));
  a2c_gpp_ctx *c = new (std::nothrow) a2c_gpp_ctx();
  if (!c) return A2C_ERR_NOMEM;
  c->p = *p;
  c->device = p->device;
  c->N = (int64_t)p->nPd + p->nH;
  const int64_t N = c->N;
  a2c_status s = A2C_OK;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) s = A2C_ERR_CUDA;
  if (!s) s = dalloc(&c->d_X, 4 * N);
  if (!s) s = dalloc(&c->d_G, 4 * N);
  if (!s) s = dalloc(&c->d_occ, N);
  if (!s) s = dalloc(&c->d_rho, N);
  if (!s) s = dalloc(&c->d_Fp, N);
  if (!s) s = dalloc(&c->d_Vs, N);
  if (!s) s = dalloc(&c->d_Ss, N);
  if (!s) s = dalloc(&c->d_red, 2 * 1024 + 64);
  if (!s) s = dalloc(&c->d_status, 1);
  if (!s) s = dalloc(&c->d_off, N + 1);
  if (!s) s = dalloc(&c->d_npd, N);
  if (!s) s = dalloc(&c->d_shell, 3 * (int64_t)p->nPd);
  if (!s) s = dalloc(&c->d_hh1_off, (int64_t)p->nH + 1);
  for (int d = 0; d < 3; ++d) c->list_reach[d] = HUGE_VAL;  // no lists yet
  if (!s && (!p->periodic[0] || !p->periodic[1] || !p->periodic[2])) s = dalloc(&c->d_xlist, 4 * N);
  if (!s && cudaMallocHost((void **)&c->h_small, 64) != cudaSuccess) s = A2C_ERR_NOMEM;
  if (!s) {
    if (N > 0) {
      k_fill<<<grid_for(N, 256), 256, 0, c->stream>>>(c->d_occ, N, 0.0);
      if (p->nPd > 0) k_fill<<<grid_for(p->nPd, 256), 256, 0, c->stream>>>(c->d_occ, p->nPd, 1.0);
    }
    if (cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream) != cudaSuccess) s = A2C_ERR_CUDA;
    if (cudaMemsetAsync(c->d_X, 0, sizeof(double) * std::max<int64_t>(4 * N, 1), c->stream) != cudaSuccess)
      s = A2C_ERR_CUDA;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) s = A2C_ERR_CUDA;
  }
  if (s) {
    a2c_gpp_destroy(c);
    return s;
  }
  *out = c;
  return A2C_OK;
}

a2c_status a2c_gpp_destroy(a2c_gpp_ctx *c) {
  if (!c) return A2C_OK;
  DeviceGuard g(c->device);
  snapshot_release(c);
  engine_free(c);
  if (c->stream) cudaStreamSynchronize(c->stream);
  mixed_free(c);
  lbfgs_free(c);
  for (void *p : {(void *)c->d_X, (void *)c->d_G, (void *)c->d_occ, (void *)c->d_rho, (void *)c->d_Fp,
                  (void *)c->d_Vs, (void *)c->d_Ss, (void *)c->d_red, (void *)c->d_status, (void *)c->d_off,
                  (void *)c->d_nbr, (void *)c->d_npd, (void *)c->d_shell, (void *)c->d_hh1_off, (void *)c->d_hh1,
                  (void *)c->d_ext_off, (void *)c->d_ext_nbr, (void *)c->d_xref, (void *)c->d_xlist})
    if (p) cudaFree(p);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->h_small) cudaFreeHost(c->h_small);
  delete c;
  return A2C_OK;
}

void *a2c_gpp_stream(a2c_gpp_ctx *c) { return c ? (void *)c->stream : nullptr; }

a2c_status a2c_gpp_set_threads_per_site(a2c_gpp_ctx *c, int tps) {
  if (!c) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  return mixed_set_threads_per_site(c, tps);
}

a2c_status a2c_gpp_set_pair_mode(a2c_gpp_ctx *c, int mode) {
  if (!c) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  return mixed_set_pair_mode(c, mode);
}

a2c_status a2c_gpp_get_pair_mode(a2c_gpp_ctx *c, int *mode) {
  if (!c || !mode) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  return mixed_get_pair_mode(c, mode);
}

// Autotuner of the mixed form's work mapping: each threads-per-site choice
// (1, 2, 4, 8) evaluates the context's current state once untimed and then
// `reps` times between two events on the context's stream; the fastest
// choice is kept.
a2c_status a2c_gpp_autotune(a2c_gpp_ctx *c, int reps, int *tps_out, float *ms) {
  if (!c || reps < 1 || reps > 1000) return A2C_ERR_INVALID;
  if (!c->has_neighbors || !c->has_state) return A2C_ERR_STATE;
  DeviceGuard g(c->device);
  const int saved = c->p.precision;
  c->p.precision = A2C_MIXED;
  const Tile keep = mixed_tile(c);
  const int choice[4] = {1, 2, 4, 8};
  float best_ms = 0.0f;
  int best = 0;
  a2c_status s = A2C_OK;
  for (int k = 0; k < 4 && !s; ++k) {
    float t = 0.0f;
    s = time_context_tile(c, reps, Tile{choice[k], keep.rho_block, keep.grad_block}, &t);
    if (ms) ms[k] = t;
    if (!s && (best == 0 || t < best_ms)) {
      best_ms = t;
      best = choice[k];
    }
  }
  c->p.precision = saved;
  c->has_density = false;
  if (!s) s = mixed_set_tile(c, Tile{best, keep.rho_block, keep.grad_block});
  if (!s && tps_out) *tps_out = best;
  if (!s) s = check_status_word(c);
  return s;
}

a2c_status a2c_gpp_autotune_tile(a2c_gpp_ctx *c, int reps, int *tile, float *ms) {
  if (!c || reps < 1 || reps > 1000) return A2C_ERR_INVALID;
  if (!c->has_neighbors || !c->has_state) return A2C_ERR_STATE;
  DeviceGuard g(c->device);
  const int saved = c->p.precision;
  c->p.precision = A2C_MIXED;
  Tile best;
  a2c_status s = tune_tile([&](const Tile &t, float *v) { return time_context_tile(c, reps, t, v); }, &best, ms);
  c->p.precision = saved;
  c->has_density = false;
  if (!s) s = mixed_set_tile(c, best);
  if (!s && tile) {
    tile[0] = best.tps;
    tile[1] = best.rho_block;
    tile[2] = best.grad_block;
  }
  if (!s) s = check_status_word(c);
  return s;
}

a2c_status a2c_gpp_set_tile(a2c_gpp_ctx *c, int tps, int rho_block, int grad_block) {
  if (!c || !valid_tile(tps, rho_block, grad_block)) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  return mixed_set_tile(c, Tile{tps, rho_block, grad_block});
}

a2c_status a2c_gpp_get_tile(a2c_gpp_ctx *c, int *tile) {
  if (!c || !tile) return A2C_ERR_INVALID;
  const Tile t = effective_tile(mixed_tile(c), c->N, device_sms(c->device));
  tile[0] = t.tps;
  tile[1] = t.rho_block;
  tile[2] = t.grad_block;
  return A2C_OK;
}

a2c_status a2c_gpp_set_minimizer(a2c_gpp_ctx *c, int mode) {
  if (!c || mode < A2C_MINIMIZER_DEFAULT || mode > A2C_MINIMIZER_DEVICE) return A2C_ERR_INVALID;
  c->host_loop = mode;
  return A2C_OK;
}

a2c_status a2c_gpp_synchronize(a2c_gpp_ctx *c) {
  if (!c) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  return finish(c);
}

a2c_status a2c_gpp_set_precision(a2c_gpp_ctx *c, int precision) {
  if (!c || (precision != A2C_FP64 && precision != A2C_MIXED)) return A2C_ERR_INVALID;
  c->p.precision = precision;
  c->has_density = false;
  return A2C_OK;
}

a2c_status a2c_gpp_set_occupancy(a2c_gpp_ctx *c, const double *xH) {
  if (!c || (!xH && c->p.nH > 0)) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  for (int i = 0; i < c->p.nH; ++i)
    if (!std::isfinite(xH[i])) return A2C_ERR_NONFINITE;
  A2C_TRY(copy_in(c, c->d_occ + c->p.nPd, xH, c->p.nH));
  c->has_density = false;
  return finish(c);
}

a2c_status a2c_gpp_get_occupancy(a2c_gpp_ctx *c, double *xH) {
  if (!c || (!xH && c->p.nH > 0)) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  if (c->p.nH > 0)
    A2C_CUDA(cudaMemcpyAsync(xH, c->d_occ + c->p.nPd, sizeof(double) * c->p.nH, cudaMemcpyDeviceToHost, c->stream));
  return finish(c);
}

a2c_status a2c_gpp_set_state(a2c_gpp_ctx *c, const double *X) {
  if (!c || (!X && c->N > 0)) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  A2C_TRY(copy_in(c, c->d_X, X, 4 * c->N));
  c->has_state = true;
  c->has_density = false;
  return finish(c);
}

a2c_status a2c_gpp_get_state(a2c_gpp_ctx *c, double *X) {
  if (!c || (!X && c->N > 0)) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  if (c->N > 0) A2C_CUDA(cudaMemcpyAsync(X, c->d_X, sizeof(double) * 4 * c->N, cudaMemcpyDeviceToHost, c->stream));
  return finish(c);
}

a2c_status a2c_gpp_build_neighbors(a2c_gpp_ctx *c, const double *X, int *max_neighbors) {
  if (!c || (!X && c->N > 0)) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  // finite, and periodic coordinates within [-L/2, 3L/2] (images are limited
  // to one box length either way): checked on the device
  int moved = 0;
  A2C_TRY(stage_positions(c, X, (uintptr_t)X % 8 == 0 ? (const double *)mapped(X) : nullptr, &moved));
  c->has_state = true;
  c->has_neighbors = false;
  c->has_density = false;
  A2C_TRY(build_neighbors_device(c, X));
  c->has_neighbors = true;
  A2C_TRY(mixed_lists_changed(c));
  if (max_neighbors) *max_neighbors = c->max_neighbors;
  return finish(c);
}

// Skin lists (findLocalNeighbors' refilter of the extended lists,
// minimizer.cpp:833-1144, on the device).
a2c_status a2c_gpp_snapshot_async(a2c_gpp_ctx *c, const a2c_snapshot_desc *d, int frame, double time,
                                  const double *X0, const double *gamma, const signed char *siteid,
                                  const signed char *tag) {
  if (!c || !d || !d->prefix || frame < 0 || d->format < 1 || d->format > 3 || d->precision < 0 || d->precision > 2)
    return A2C_ERR_INVALID;
  if (!c->has_state) return A2C_ERR_STATE;
  DeviceGuard g(c->device);
  if (!c->snap) c->snap = new (std::nothrow) SnapJob();
  SnapJob *j = (SnapJob *)c->snap;
  if (!j) return A2C_ERR_NOMEM;
  const a2c_status prev = snapshot_join(c);
  const int64_t N = c->N, nPd = c->p.nPd, nH = c->p.nH;
  const size_t need = (size_t)(4 * N + nH);
  if (need > j->cap) {
    if (j->pinned) cudaFreeHost(j->pinned);
    j->pinned = nullptr;
    j->cap = 0;
    if (cudaMallocHost((void **)&j->pinned, sizeof(double) * std::max<size_t>(need, 1)) != cudaSuccess)
      return A2C_ERR_NOMEM;
    j->cap = need;
  }
  if (!j->ev) A2C_CUDA(cudaEventCreateWithFlags(&j->ev, cudaEventDisableTiming));
  if (N > 0) A2C_CUDA(cudaMemcpyAsync(j->pinned, c->d_X, sizeof(double) * 4 * N, cudaMemcpyDeviceToHost, c->stream));
  if (nH > 0)
    A2C_CUDA(cudaMemcpyAsync(j->pinned + 4 * N, c->d_occ + nPd, sizeof(double) * nH, cudaMemcpyDeviceToHost,
                             c->stream));
  A2C_CUDA(cudaEventRecord(j->ev, c->stream));
  j->prefix = d->prefix;
  j->desc = *d;
  j->desc.prefix = j->prefix.c_str();
  j->X0.assign(X0 ? X0 : nullptr, X0 ? X0 + 4 * N : nullptr);
  j->gamma.assign(gamma ? gamma : nullptr, gamma ? gamma + nH : nullptr);
  j->siteid.assign(siteid ? siteid : nullptr, siteid ? siteid + N : nullptr);
  j->tag.assign(tag ? tag : nullptr, tag ? tag + N : nullptr);
  const int dev = c->device;
  j->th = std::thread([j, dev, frame, time, nPd, nH, N]() {
    cudaSetDevice(dev);
    if (cudaEventSynchronize(j->ev) != cudaSuccess) {
      j->result = A2C_ERR_CUDA;
      return;
    }
    j->result = a2c_snapshot_write(&j->desc, frame, time, (int)nPd, (int)nH, j->pinned,
                                   j->X0.empty() ? nullptr : j->X0.data(), j->pinned + 4 * N,
                                   j->gamma.empty() ? nullptr : j->gamma.data(),
                                   j->siteid.empty() ? nullptr : j->siteid.data(),
                                   j->tag.empty() ? nullptr : j->tag.data());
  });
  return prev;
}

a2c_status a2c_gpp_snapshot_wait(a2c_gpp_ctx *c) {
  if (!c) return A2C_ERR_INVALID;
  return snapshot_join(c);
}

a2c_status a2c_gpp_set_neighbor_skin(a2c_gpp_ctx *c, double skin) {
  if (!c || !(skin >= 0.0) || !std::isfinite(skin)) return A2C_ERR_INVALID;
  for (int d = 0; d < 3; ++d)  // the minimum image must stay unique at rc + skin
    if (c->p.periodic[d] && !(c->p.box[d] > 2.0 * (c->p.rc + skin))) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  if (skin > 0.0 && !c->d_ext_off) {
    A2C_TRY(dalloc(&c->d_ext_off, c->N + 1));
    A2C_TRY(dalloc(&c->d_xref, 4 * c->N));
  }
  c->skin = skin;
  c->has_ext = false;
  return A2C_OK;
}

a2c_status a2c_gpp_update_neighbors(a2c_gpp_ctx *c, const double *X, int *max_neighbors, int *rebuilt) {
  if (!c || (!X && c->N > 0)) return A2C_ERR_INVALID;
  if (!(c->skin > 0.0)) {
    if (rebuilt) *rebuilt = 1;
    return a2c_gpp_build_neighbors(c, X, max_neighbors);
  }
  DeviceGuard g(c->device);
  // checked on the device: pinned X is read there directly, other memory
  // is copied first
  int moved = 0;
  A2C_TRY(stage_positions(c, X, (uintptr_t)X % 8 == 0 ? (const double *)mapped(X) : nullptr, &moved));
  c->has_state = true;
  c->has_neighbors = false;
  c->has_density = false;
  A2C_TRY(update_neighbors_device(c, X, rebuilt, moved));
  c->has_neighbors = true;
  A2C_TRY(mixed_lists_changed(c));
  if (max_neighbors) *max_neighbors = c->max_neighbors;
  return finish(c);
}

namespace {
// host copies of off / npd for list export
a2c_status host_lists(a2c_gpp_ctx *c, std::vector<int64_t> &off, std::vector<int> &npd) {
  off.resize(c->N + 1);
  npd.resize(std::max<int64_t>(c->N, 1));
  A2C_CUDA(cudaMemcpyAsync(off.data(), c->d_off, sizeof(int64_t) * (c->N + 1), cudaMemcpyDeviceToHost, c->stream));
  if (c->N > 0)
    A2C_CUDA(cudaMemcpyAsync(npd.data(), c->d_npd, sizeof(int) * c->N, cudaMemcpyDeviceToHost, c->stream));
  A2C_CUDA(cudaStreamSynchronize(c->stream));
  return A2C_OK;
}
}  // namespace

a2c_status a2c_gpp_set_neighbor_lists(a2c_gpp_ctx *c, const double *X, const int64_t *pdpd_off,
                                      const int *pdpd_idx, const int64_t *pdh_off, const int *pdh_idx,
                                      const int64_t *hpd_off, const int *hpd_idx, const int64_t *hh_off,
                                      const int *hh_idx, const int64_t *hh1_off, const int *hh1_idx,
                                      const int *PdPdnum) {
  if (!c) return A2C_ERR_INVALID;
  const int nPd = c->p.nPd, nH = c->p.nH;
  const int64_t N = c->N;
  const bool per = c->p.periodic[0] || c->p.periodic[1] || c->p.periodic[2];
  if ((per && N > 0 && !X) || (nPd > 0 && (!pdpd_off || !pdh_off)) || (nH > 0 && (!hpd_off || !hh_off || !hh1_off)))
    return A2C_ERR_INVALID;
  std::vector<int64_t> off((size_t)N + 1, 0);
  std::vector<uint32_t> nbr;
  std::vector<int> npd((size_t)std::max<int64_t>(N, 1), 0);
  auto code = [&](int64_t i, int64_t j) -> uint32_t {
    if (!per) return kNoShift;
    int m[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d)
      if (c->p.periodic[d]) m[d] = -(int)std::nearbyint((X[4 * j + d] - X[4 * i + d]) / c->p.box[d]);
    for (int d = 0; d < 3; ++d)
      if (m[d] < -1 || m[d] > 1) return 0xffffffffu;
    return (uint32_t)((m[0] + 1) + 3 * (m[1] + 1) + 9 * (m[2] + 1));
  };
  auto append = [&](int64_t s, const int64_t *o, const int *idx, int64_t row, int64_t base, int64_t lim) -> bool {
    for (int64_t t = o[row]; t < o[row + 1]; ++t) {
      const int64_t j = idx[t];
      if (j < 0 || j >= lim) return false;
      const uint32_t cd = code(s, base + j);
      if (cd == 0xffffffffu) return false;
      nbr.push_back((uint32_t)(base + j) | (cd << kIdBits));
    }
    return true;
  };
  int maxn = 0;
  for (int64_t s = 0; s < N; ++s) {
    const bool iPd = s < nPd;
    const int64_t row = iPd ? s : s - nPd;
    if (!append(s, iPd ? pdpd_off : hpd_off, iPd ? pdpd_idx : hpd_idx, row, 0, nPd)) return A2C_ERR_INVALID;
    npd[(size_t)s] = (int)(nbr.size() - (size_t)off[(size_t)s]);
    if (!append(s, iPd ? pdh_off : hh_off, iPd ? pdh_idx : hh_idx, row, nPd, nH)) return A2C_ERR_INVALID;
    off[(size_t)s + 1] = (int64_t)nbr.size();
    const int cnt = (int)(off[(size_t)s + 1] - off[(size_t)s]);
    if (cnt > 1000) return A2C_ERR_NEIGHBOR_OVERFLOW;
    maxn = std::max(maxn, cnt);
  }
  const int64_t total = (int64_t)nbr.size(), total1 = nH > 0 ? hh1_off[nH] : 0;
  for (int64_t t = 0; t < total1; ++t)
    if (hh1_idx[t] < 0 || hh1_idx[t] >= nH) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  if (total > c->nbr_cap) {
    if (c->d_nbr) cudaFree(c->d_nbr);
    c->d_nbr = nullptr;
    c->nbr_cap = 0;
    if (cudaMalloc(&c->d_nbr, sizeof(uint32_t) * std::max<int64_t>(total, 1)) != cudaSuccess) return A2C_ERR_NOMEM;
    c->nbr_cap = total;
  }
  if (total1 > c->hh1_cap) {
    if (c->d_hh1) cudaFree(c->d_hh1);
    c->d_hh1 = nullptr;
    c->hh1_cap = 0;
    if (cudaMalloc(&c->d_hh1, sizeof(int) * std::max<int64_t>(total1, 1)) != cudaSuccess) return A2C_ERR_NOMEM;
    c->hh1_cap = total1;
  }
  cudaStream_t st = c->stream;
  A2C_CUDA(cudaMemcpyAsync(c->d_off, off.data(), sizeof(int64_t) * (N + 1), cudaMemcpyHostToDevice, st));
  if (N > 0) A2C_CUDA(cudaMemcpyAsync(c->d_npd, npd.data(), sizeof(int) * N, cudaMemcpyHostToDevice, st));
  if (total > 0) A2C_CUDA(cudaMemcpyAsync(c->d_nbr, nbr.data(), sizeof(uint32_t) * total, cudaMemcpyHostToDevice, st));
  if (nH > 0) A2C_CUDA(cudaMemcpyAsync(c->d_hh1_off, hh1_off, sizeof(int64_t) * (nH + 1), cudaMemcpyHostToDevice, st));
  if (total1 > 0) A2C_CUDA(cudaMemcpyAsync(c->d_hh1, hh1_idx, sizeof(int) * total1, cudaMemcpyHostToDevice, st));
  if (PdPdnum && nPd > 0)
    A2C_CUDA(cudaMemcpyAsync(c->d_shell, PdPdnum, sizeof(int) * 3 * nPd, cudaMemcpyHostToDevice, st));
  else if (nPd > 0)
    A2C_CUDA(cudaMemsetAsync(c->d_shell, 0, sizeof(int) * 3 * nPd, st));
  A2C_CUDA(cudaStreamSynchronize(st));  // host vectors go out of scope
  c->nbr_total = total;
  c->hh1_total = total1;
  c->max_neighbors = maxn;
  ++c->nbr_version;
  c->has_neighbors = true;
  // the span guard: how far apart a listed pair is in each free direction
  // (unknown without positions)
  for (int d = 0; d < 3; ++d) {
    c->list_reach[d] = (c->p.periodic[d] || (X && N > 0)) ? 0.0 : HUGE_VAL;
    if (c->p.periodic[d] || !X) continue;
    double r = 0.0;
    for (int64_t i = 0; i < N; ++i)
      for (int64_t t = off[(size_t)i]; t < off[(size_t)i + 1]; ++t)
        r = std::max(r, std::fabs(X[4 * i + d] - X[4 * (int64_t)(nbr[(size_t)t] & kIdMask) + d]));
    c->list_reach[d] = r;
  }
  A2C_TRY(mixed_lists_changed(c));
  c->has_density = false;
  if (X && N > 0) {
    A2C_TRY(copy_in(c, c->d_X, X, 4 * N));
    if (c->d_xlist) A2C_TRY(copy_in(c, c->d_xlist, X, 4 * N));
    c->has_state = true;
  }
  return finish(c);
}

a2c_status a2c_gpp_neighbor_total(a2c_gpp_ctx *c, int list, int64_t *total) {
  if (!c || !total || list < 0 || list > 4) return A2C_ERR_INVALID;
  if (!c->has_neighbors) return A2C_ERR_STATE;
  DeviceGuard g(c->device);
  if (list == A2C_LIST_HH1) {
    *total = c->hh1_total;
    return A2C_OK;
  }
  std::vector<int64_t> off;
  std::vector<int> npd;
  A2C_TRY(host_lists(c, off, npd));
  const bool pdsite = (list == A2C_LIST_PDPD || list == A2C_LIST_PDH);
  const bool pdnbr = (list == A2C_LIST_PDPD || list == A2C_LIST_HPD);
  const int64_t lo = pdsite ? 0 : c->p.nPd, hi = pdsite ? c->p.nPd : c->N;
  int64_t t = 0;
  for (int64_t s = lo; s < hi; ++s) t += pdnbr ? npd[s] : (off[s + 1] - off[s] - npd[s]);
  *total = t;
  return A2C_OK;
}

a2c_status a2c_gpp_get_neighbors(a2c_gpp_ctx *c, int list, int64_t *offsets, int *idx) {
  if (!c || !offsets || list < 0 || list > 4) return A2C_ERR_INVALID;
  if (!c->has_neighbors) return A2C_ERR_STATE;
  DeviceGuard g(c->device);
  const int nPd = c->p.nPd, nH = c->p.nH;
  if (list == A2C_LIST_HH1) {
    A2C_CUDA(cudaMemcpyAsync(offsets, c->d_hh1_off, sizeof(int64_t) * (nH + 1), cudaMemcpyDeviceToHost, c->stream));
    if (c->hh1_total > 0)
      A2C_CUDA(cudaMemcpyAsync(idx, c->d_hh1, sizeof(int) * c->hh1_total, cudaMemcpyDeviceToHost, c->stream));
    A2C_CUDA(cudaStreamSynchronize(c->stream));
    return A2C_OK;
  }
  std::vector<int64_t> off;
  std::vector<int> npd;
  A2C_TRY(host_lists(c, off, npd));
  std::vector<uint32_t> nbr((size_t)std::max<int64_t>(c->nbr_total, 1));
  if (c->nbr_total > 0)
    A2C_CUDA(cudaMemcpy(nbr.data(), c->d_nbr, sizeof(uint32_t) * c->nbr_total, cudaMemcpyDeviceToHost));
  const bool pdsite = (list == A2C_LIST_PDPD || list == A2C_LIST_PDH);
  const bool pdnbr = (list == A2C_LIST_PDPD || list == A2C_LIST_HPD);
  const int64_t lo = pdsite ? 0 : nPd, hi = pdsite ? nPd : c->N;
  int64_t w = 0;
  offsets[0] = 0;
  for (int64_t s = lo; s < hi; ++s) {
    const int64_t b = pdnbr ? off[s] : off[s] + npd[s];
    const int64_t e = pdnbr ? off[s] + npd[s] : off[s + 1];
    for (int64_t t = b; t < e; ++t) {
      const int64_t j = nbr[t] & kIdMask;
      idx[w++] = (int)(pdnbr ? j : j - nPd);
    }
    offsets[s - lo + 1] = w;
  }
  return A2C_OK;
}

a2c_status a2c_gpp_get_shell_counts(a2c_gpp_ctx *c, int *PdPdnum) {
  if (!c || (!PdPdnum && c->p.nPd > 0)) return A2C_ERR_INVALID;
  if (!c->has_neighbors) return A2C_ERR_STATE;
  DeviceGuard g(c->device);
  if (c->p.nPd > 0)
    A2C_CUDA(cudaMemcpyAsync(PdPdnum, c->d_shell, sizeof(int) * 3 * c->p.nPd, cudaMemcpyDeviceToHost, c->stream));
  return finish(c);
}

a2c_status a2c_gpp_eval_device(a2c_gpp_ctx *c, const double *dX, double *df, double *dG) {
  if (!c || (!dX && c->N > 0) || !df || (!dG && c->N > 0)) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  A2C_TRY(eval_device_impl(c, dX, df, dG));
  if (dX != c->d_X && c->N > 0)
    A2C_CUDA(cudaMemcpyAsync(c->d_X, dX, sizeof(double) * 4 * c->N, cudaMemcpyDeviceToDevice, c->stream));
  c->has_state = true;
  return A2C_OK;
}

a2c_status a2c_gpp_profile_eval(a2c_gpp_ctx *c, const double *dX, double *df, double *dG, float *stage_ms) {
  if (!c || (!dX && c->N > 0) || !df || (!dG && c->N > 0) || !stage_ms) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  cudaEvent_t ev[5];
  for (auto &e : ev) A2C_CUDA(cudaEventCreate(&e));
  a2c_status s = eval_device_impl(c, dX, df, dG, ev);
  if (!s && cudaEventSynchronize(ev[4]) != cudaSuccess) s = A2C_ERR_CUDA;
  for (int k = 0; k < 4 && !s; ++k)
    if (cudaEventElapsedTime(&stage_ms[k], ev[k], ev[k + 1]) != cudaSuccess) s = A2C_ERR_CUDA;
  for (auto &e : ev) cudaEventDestroy(e);
  if (s) return s;
  return check_status_word(c);
}

a2c_status a2c_gpp_eval(a2c_gpp_ctx *c, const double *X, double *f, double *G) {
  if (!c || (!X && c->N > 0) || !f || (!G && c->N > 0)) return A2C_ERR_INVALID;
  if (!c->has_neighbors) return A2C_ERR_STATE;
  DeviceGuard g(c->device);
  // Mixed form with pinned caller buffers: the prep kernel reads X and pass 2
  // writes G through the coherent host link while they compute, instead of
  // bulk copies before and after; f and the status word come back through
  // pinned memory the last kernel writes.
  const double *mX = (c->p.precision == A2C_MIXED && c->N > 0 && (uintptr_t)X % 32 == 0)
                         ? (const double *)mapped(X) : nullptr;  // read as double4
  double *mG = (mX && (uintptr_t)G % 8 == 0) ? (double *)mapped(G) : nullptr;
  if (mX && (uintptr_t)mX % 32 != 0) mX = nullptr;
  if (mX && mG && c->h_small) {
    c->has_state = true;
    double *d_f = c->d_red + 2 * 1024 + 8;
    double *hs = (double *)mapped(c->h_small);
    A2C_TRY(mixed_eval(c, mX, d_f, mG, nullptr, c->d_X, hs));
    c->has_density = false;
    if (!hs) {
      A2C_CUDA(cudaMemcpyAsync(c->h_small, d_f, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      A2C_CUDA(cudaMemcpyAsync(c->h_small + 1, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      A2C_CUDA(cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream));
    }
    A2C_CUDA(cudaStreamSynchronize(c->stream));
    *f = c->h_small[0];
    int st = 0;
    std::memcpy(&st, c->h_small + 1, sizeof(int));
    if (st & kStatusBadIndex) return A2C_ERR_INVALID;
    if (st & kStatusOverflow) return A2C_ERR_NEIGHBOR_OVERFLOW;
    if (st & kStatusTimeout) return A2C_ERR_TIMEOUT;
    if (st & kStatusNonfinite) return A2C_ERR_NONFINITE;
    if (st & kStatusSpan) return A2C_ERR_LISTS_STALE;
    return A2C_OK;
  }
  A2C_TRY(copy_in(c, c->d_X, X, 4 * c->N));
  c->has_state = true;
  double *d_f = c->d_red + 2 * 1024 + 8;
  A2C_TRY(launch_finite_check(c, c->d_X, 4 * c->N));
  A2C_TRY(eval_device_impl(c, c->d_X, d_f, c->d_G));
  A2C_CUDA(cudaMemcpyAsync(f, d_f, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (c->N > 0) A2C_CUDA(cudaMemcpyAsync(G, c->d_G, sizeof(double) * 4 * c->N, cudaMemcpyDeviceToHost, c->stream));
  return finish(c);
}

a2c_status a2c_gpp_get_density(a2c_gpp_ctx *c, double *rho) {
  if (!c || (!rho && c->N > 0)) return A2C_ERR_INVALID;
  if (!c->has_density) return A2C_ERR_STATE;
  DeviceGuard g(c->device);
  if (c->N > 0) A2C_CUDA(cudaMemcpyAsync(rho, c->d_rho, sizeof(double) * c->N, cudaMemcpyDeviceToHost, c->stream));
  return finish(c);
}

a2c_status a2c_gpp_eam_eval(a2c_gpp_ctx *c, int which, const double *in, int64_t n, double *out) {
  if (!c || which < 0 || which > 13 || n < 0 || (n > 0 && (!in || !out))) return A2C_ERR_INVALID;
  if (n == 0) return A2C_OK;
  DeviceGuard g(c->device);
  double *d = nullptr;
  A2C_CUDA(cudaMallocAsync((void **)&d, sizeof(double) * 2 * n, c->stream));
  a2c_status s = A2C_OK;
  if (cudaMemcpyAsync(d, in, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream)) s = A2C_ERR_CUDA;
  if (!s) s = launch_eam64(c, which, d, n, d + n);
  if (!s && cudaMemcpyAsync(out, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream)) s = A2C_ERR_CUDA;
  cudaFreeAsync(d, c->stream);
  if (s) return s;
  return finish(c);
}

a2c_status a2c_gpp_bounds(a2c_gpp_ctx *c, double *lb, double *ub) {
  if (!c || (!lb && c->N > 0) || (!ub && c->N > 0)) return A2C_ERR_INVALID;
  for (int64_t s = 0; s < c->N; ++s) {
    for (int d = 0; d < 3; ++d) {
      lb[4 * s + d] = -HUGE_VAL;
      ub[4 * s + d] = HUGE_VAL;
    }
    lb[4 * s + 3] = 1.0e-6;
    ub[4 * s + 3] = HUGE_VAL;
  }
  return A2C_OK;
}

a2c_status a2c_gpp_minimize(a2c_gpp_ctx *c, double *X, const a2c_lbfgs_params *lp, double *fmin, int *iters,
                            int *nfev, double *gnorm, int *reason) {
  if (!c || (!X && c->N > 0) || !lp || !fmin || !iters || !nfev || !gnorm || !reason) return A2C_ERR_INVALID;
  if (!c->has_neighbors) return A2C_ERR_STATE;
  DeviceGuard g(c->device);
  for (int64_t t = 0; t < 4 * c->N; ++t)
    if (!std::isfinite(X[t])) return A2C_ERR_NONFINITE;
  A2C_TRY(copy_in(c, c->d_X, X, 4 * c->N));
  A2C_TRY(lbfgs_minimize(c, c->d_X, lp, fmin, iters, nfev, gnorm, reason));
  c->has_state = true;
  c->has_density = false;
  if (c->N > 0) A2C_CUDA(cudaMemcpyAsync(X, c->d_X, sizeof(double) * 4 * c->N, cudaMemcpyDeviceToHost, c->stream));
  return finish(c);
}

a2c_status a2c_gpp_minimize_stats(a2c_gpp_ctx *c, int *mixed_iters, int *fp64_iters, double *mixed_gnorm) {
  if (!c) return A2C_ERR_INVALID;
  if (mixed_iters) *mixed_iters = c->last_mixed_iters;
  if (fp64_iters) *fp64_iters = c->last_fp64_iters;
  if (mixed_gnorm) *mixed_gnorm = c->last_mixed_gnorm;
  return A2C_OK;
}

a2c_status a2c_gpp_chem_potential(a2c_gpp_ctx *c, double gamma_bd, double *gamma, int *full_H) {
  if (!c || ((!gamma || !full_H) && c->p.nH > 0)) return A2C_ERR_INVALID;
  if (!c->has_neighbors || !c->has_state) return A2C_ERR_STATE;
  DeviceGuard g(c->device);
  const int nH = c->p.nH;
  if (nH == 0) return A2C_OK;
  double *dg, *dsend, *dx;
  int *dfull;
  A2C_TRY(ensure_hscratch(c, &dg, &dsend, &dx, &dfull));
  a2c_status s = A2C_OK;
  if (cudaMemcpyAsync(dg, gamma, sizeof(double) * nH, cudaMemcpyHostToDevice, c->stream) ||
      cudaMemcpyAsync(dfull, full_H, sizeof(int) * nH, cudaMemcpyHostToDevice, c->stream))
    s = A2C_ERR_CUDA;
  // minimizer.cpp:607-789: densities at the current state and the pair
  // sums, FP64 (the reference's arithmetic) or, in the mixed form, with
  // the pair quadrature in FP32
  const bool mixed = c->p.precision == A2C_MIXED;
  if (!s) s = mixed ? mixed_chem(c, c->d_X, dsend, dfull) : launch_density64(c, c->d_X);
  if (!s && !mixed) s = launch_chem64(c, c->d_X, gamma_bd, dsend, dfull);
  if (!s) s = launch_gamma_update(c, dsend, gamma_bd, dg, dfull);
  if (!s && (cudaMemcpyAsync(gamma, dg, sizeof(double) * nH, cudaMemcpyDeviceToHost, c->stream) ||
             cudaMemcpyAsync(full_H, dfull, sizeof(int) * nH, cudaMemcpyDeviceToHost, c->stream)))
    s = A2C_ERR_CUDA;
  free_hscratch(c, dg, dsend, dx, dfull);
  if (s) return s;
  c->has_density = !mixed;
  return finish(c);
}

a2c_status a2c_gpp_apply_dirichlet(a2c_gpp_ctx *c, const int *sites, int n, double gamma_bd, double xUb,
                                   double *gamma, int *full_H) {
  if (!c || n < 0 || (n > 0 && (!sites || !gamma || !full_H))) return A2C_ERR_INVALID;
  const int nH = c->p.nH;
  for (int t = 0; t < n; ++t)
    if (sites[t] < 0 || sites[t] >= nH) return A2C_ERR_INVALID;
  if (n == 0) return A2C_OK;
  DeviceGuard g(c->device);
  int *dsites = nullptr;
  double *dg = nullptr;
  int *dfull = nullptr;
  A2C_CUDA(cudaMallocAsync((void **)&dsites, sizeof(int) * n, c->stream));
  A2C_CUDA(cudaMallocAsync((void **)&dg, sizeof(double) * nH, c->stream));
  A2C_CUDA(cudaMallocAsync((void **)&dfull, sizeof(int) * nH, c->stream));
  a2c_status s = A2C_OK;
  if (cudaMemcpyAsync(dsites, sites, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream) ||
      cudaMemcpyAsync(dg, gamma, sizeof(double) * nH, cudaMemcpyHostToDevice, c->stream) ||
      cudaMemcpyAsync(dfull, full_H, sizeof(int) * nH, cudaMemcpyHostToDevice, c->stream))
    s = A2C_ERR_CUDA;
  if (!s) s = launch_dirichlet(c, dsites, n, gamma_bd, xUb, dg, dfull);
  if (!s && (cudaMemcpyAsync(gamma, dg, sizeof(double) * nH, cudaMemcpyDeviceToHost, c->stream) ||
             cudaMemcpyAsync(full_H, dfull, sizeof(int) * nH, cudaMemcpyDeviceToHost, c->stream)))
    s = A2C_ERR_CUDA;
  cudaFreeAsync(dsites, c->stream);
  cudaFreeAsync(dg, c->stream);
  cudaFreeAsync(dfull, c->stream);
  if (s) return s;
  c->has_density = false;
  return finish(c);
}

a2c_status a2c_gpp_diffuse(a2c_gpp_ctx *c, double dt, double nu, double Qm, double xLb, double xUb,
                           const double *gamma, const int *full_H, double *x) {
  if (!c || ((!gamma || !full_H || !x) && c->p.nH > 0)) return A2C_ERR_INVALID;
  if (!c->has_neighbors) return A2C_ERR_STATE;
  const int nH = c->p.nH;
  if (nH == 0) return A2C_OK;
  DeviceGuard g(c->device);
  double *dg, *dsend, *dx;
  int *dfull;
  A2C_TRY(ensure_hscratch(c, &dg, &dsend, &dx, &dfull));
  a2c_status s = A2C_OK;
  if (cudaMemcpyAsync(dg, gamma, sizeof(double) * nH, cudaMemcpyHostToDevice, c->stream) ||
      cudaMemcpyAsync(dfull, full_H, sizeof(int) * nH, cudaMemcpyHostToDevice, c->stream) ||
      cudaMemcpyAsync(dx, x, sizeof(double) * nH, cudaMemcpyHostToDevice, c->stream))
    s = A2C_ERR_CUDA;
  if (!s) s = launch_diffuse(c, dg, dfull, dt, nu, Qm, xLb, xUb, dx);
  if (!s && cudaMemcpyAsync(x, dx, sizeof(double) * nH, cudaMemcpyDeviceToHost, c->stream)) s = A2C_ERR_CUDA;
  free_hscratch(c, dg, dsend, dx, dfull);
  if (s) return s;
  return finish(c);
}

a2c_status a2c_diffuse_lists(int device, int nH, const int64_t *hh1_off, const int *hh1_idx, const double *x0,
                             const double *gamma, const int *full_H, double T, double dt, double nu, double Qm,
                             double xLb, double xUb, double *x) {
  if (nH < 0 || (nH > 0 && (!hh1_off || !x0 || !gamma || !full_H || !x)) || !(T > 0.0)) return A2C_ERR_INVALID;
  if (nH == 0) return A2C_OK;
  const int64_t total = hh1_off[nH];
  if (total > 0 && !hh1_idx) return A2C_ERR_INVALID;
  for (int64_t t = 0; t < total; ++t)
    if (hh1_idx[t] < 0 || hh1_idx[t] >= nH) return A2C_ERR_INVALID;
  a2c_gpp_params p;
  a2c_gpp_default_params(&p);
  p.nPd = 0;
  p.nH = nH;
  p.T = T;
  p.device = device;
  a2c_gpp_ctx *c = nullptr;
  A2C_TRY(a2c_gpp_create(&p, &c));
  DeviceGuard g(c->device);
  a2c_status s = A2C_OK;
  double *dg = nullptr, *dsend = nullptr, *dx = nullptr;
  int *dfull = nullptr;
  if (cudaMalloc(&c->d_hh1, sizeof(int) * std::max<int64_t>(total, 1)) != cudaSuccess) s = A2C_ERR_NOMEM;
  if (!s) s = ensure_hscratch(c, &dg, &dsend, &dx, &dfull);
  if (!s && (cudaMemcpyAsync(c->d_hh1_off, hh1_off, sizeof(int64_t) * (nH + 1), cudaMemcpyHostToDevice, c->stream) ||
             (total > 0 && cudaMemcpyAsync(c->d_hh1, hh1_idx, sizeof(int) * total, cudaMemcpyHostToDevice, c->stream)) ||
             cudaMemcpyAsync(c->d_occ, x0, sizeof(double) * nH, cudaMemcpyHostToDevice, c->stream) ||
             cudaMemcpyAsync(dg, gamma, sizeof(double) * nH, cudaMemcpyHostToDevice, c->stream) ||
             cudaMemcpyAsync(dfull, full_H, sizeof(int) * nH, cudaMemcpyHostToDevice, c->stream) ||
             cudaMemcpyAsync(dx, x, sizeof(double) * nH, cudaMemcpyHostToDevice, c->stream)))
    s = A2C_ERR_CUDA;
  if (!s) s = launch_diffuse(c, dg, dfull, dt, nu, Qm, xLb, xUb, dx);
  if (!s && cudaMemcpyAsync(x, dx, sizeof(double) * nH, cudaMemcpyDeviceToHost, c->stream)) s = A2C_ERR_CUDA;
  if (dg) free_hscratch(c, dg, dsend, dx, dfull);
  if (!s) s = finish(c);
  a2c_gpp_destroy(c);
  return s;
}

a2c_status a2c_gpp_macro_results(a2c_gpp_ctx *c, const double *x, const int *HSurf, int nSurf, double *xH,
                                 double *xHinterior) {
  if (!c || !xH || !xHinterior || nSurf < 0 || (c->p.nH > 0 && !x) || (nSurf > 0 && !HSurf)) return A2C_ERR_INVALID;
  const int nH = c->p.nH;
  if (nH == 0) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  std::vector<int> flags((size_t)nH, 0);
  for (int t = 0; t < nSurf; ++t)
    if (HSurf[t] >= 0 && HSurf[t] < nH) flags[(size_t)HSurf[t]] = 1;
  double *dx = nullptr;
  int *df = nullptr;
  A2C_CUDA(cudaMallocAsync((void **)&dx, sizeof(double) * nH, c->stream));
  A2C_CUDA(cudaMallocAsync((void **)&df, sizeof(int) * nH, c->stream));
  a2c_status s = A2C_OK;
  if (cudaMemcpyAsync(dx, x, sizeof(double) * nH, cudaMemcpyHostToDevice, c->stream) ||
      cudaMemcpyAsync(df, flags.data(), sizeof(int) * nH, cudaMemcpyHostToDevice, c->stream))
    s = A2C_ERR_CUDA;
  if (!s) s = launch_macro(c, dx, df, nSurf, xH, xHinterior);
  cudaFreeAsync(dx, c->stream);
  cudaFreeAsync(df, c->stream);
  if (s) return s;
  return finish(c);
}

a2c_status a2c_gpp_dmd_run(a2c_gpp_ctx *c, double *X, double *xH, double *gamma, int *full_H, const int *bd_sites,
                           int n_bd, const int *surf_sites, int n_surf, const a2c_dmd_params *dp, int nsteps,
                           double *xH_mean, double *xH_interior, double *fmin, int *iters) {
  if (!c || !dp || nsteps < 0 || n_bd < 0 || n_surf < 0 || (c->N > 0 && !X) ||
      (c->p.nH > 0 && (!xH || !gamma || !full_H)) || (n_bd > 0 && !bd_sites) || (n_surf > 0 && !surf_sites))
    return A2C_ERR_INVALID;
  if (!c->has_neighbors) return A2C_ERR_STATE;
  const int nH = c->p.nH;
  for (int t = 0; t < n_bd; ++t)
    if (bd_sites[t] < 0 || bd_sites[t] >= nH) return A2C_ERR_INVALID;
  if (nH == 0) return A2C_ERR_INVALID;
  DeviceGuard g(c->device);
  cudaStream_t st = c->stream;
  std::vector<int> flags((size_t)nH, 0);
  for (int t = 0; t < n_surf; ++t)
    if (surf_sites[t] >= 0 && surf_sites[t] < nH) flags[(size_t)surf_sites[t]] = 1;
  double *dg = nullptr, *dsend = nullptr, *dx = nullptr, *drec = nullptr;
  int *dfull = nullptr, *dbd = nullptr, *dsurf = nullptr, *dcnt = nullptr;
  A2C_TRY(ensure_hscratch(c, &dg, &dsend, &dx, &dfull));
  a2c_status s = A2C_OK;
  if (cudaMallocAsync((void **)&dbd, sizeof(int) * std::max(n_bd, 1), st) ||
      cudaMallocAsync((void **)&dsurf, sizeof(int) * nH, st) ||
      cudaMallocAsync((void **)&drec, sizeof(double) * (4 * (size_t)std::max(nsteps, 1) + 2), st) ||
      cudaMallocAsync((void **)&dcnt, sizeof(int) * 2, st))
    s = A2C_ERR_NOMEM;
  if (!s && (cudaMemcpyAsync(c->d_X, X, sizeof(double) * 4 * c->N, cudaMemcpyHostToDevice, st) ||
             cudaMemcpyAsync(c->d_occ + c->p.nPd, xH, sizeof(double) * nH, cudaMemcpyHostToDevice, st) ||
             cudaMemcpyAsync(dg, gamma, sizeof(double) * nH, cudaMemcpyHostToDevice, st) ||
             cudaMemcpyAsync(dfull, full_H, sizeof(int) * nH, cudaMemcpyHostToDevice, st) ||
             (n_bd > 0 && cudaMemcpyAsync(dbd, bd_sites, sizeof(int) * n_bd, cudaMemcpyHostToDevice, st)) ||
             cudaMemcpyAsync(dsurf, flags.data(), sizeof(int) * nH, cudaMemcpyHostToDevice, st)))
    s = A2C_ERR_CUDA;
  c->has_state = true;
  std::vector<double> hX;
  // After an eager first step (one-time set-up, the engine), the remaining
  // steps can run as one CUDA graph (engine_dmd_graph).
  const bool graph = !dp->host_steps && nsteps >= 2 && !dp->neighbor_update &&
                     ((c->p.precision == A2C_MIXED && c->host_loop == A2C_MINIMIZER_DEFAULT) ||
                      c->host_loop == A2C_MINIMIZER_DEVICE);
  const int eager_steps = graph ? 1 : nsteps;
  for (int k = 0; k < eager_steps && !s; ++k) {
    double f = 0.0, gn = 0.0;
    int it = 0, fev = 0, why = 0;
    if (k > 0 && dp->neighbor_update) {  // findNeighbors + findLocalNeighbors at the current positions
      if (c->skin > 0.0) {
        s = update_neighbors_device(c, nullptr, nullptr, -1);
      } else {
        hX.resize((size_t)(4 * c->N));
        if (cudaMemcpyAsync(hX.data(), c->d_X, sizeof(double) * 4 * c->N, cudaMemcpyDeviceToHost, st) ||
            cudaStreamSynchronize(st))
          s = A2C_ERR_CUDA;
        if (!s) s = build_neighbors_device(c, hX.data());
      }
      if (s) break;
    }
    s = lbfgs_minimize(c, c->d_X, &dp->lbfgs, &f, &it, &fev, &gn, &why);  // minimizer.cpp:548
    // minimizer.cpp:607-789: densities and chemical potential at the
    // minimum (pair quadrature in FP32 for the mixed form)
    if (!s) s = c->p.precision == A2C_MIXED ? mixed_chem(c, c->d_X, dsend, dfull) : launch_density64(c, c->d_X);
    if (!s && c->p.precision != A2C_MIXED) s = launch_chem64(c, c->d_X, dp->gamma_bd, dsend, dfull);
    if (!s) s = launch_gamma_update(c, dsend, dp->gamma_bd, dg, dfull);   // minimizer.cpp:793-800
    if (!s) s = launch_dirichlet(c, dbd, n_bd, dp->gamma_bd, dp->x_bd, dg, dfull);  // boundaryconditions.cpp:47-51
    if (!s && cudaMemcpyAsync(dx, c->d_occ + c->p.nPd, sizeof(double) * nH, cudaMemcpyDeviceToDevice, st))
      s = A2C_ERR_CUDA;
    if (!s) s = launch_diffuse(c, dg, dfull, dp->dt, dp->nu, dp->Qm, dp->xLb, dp->xUb, dx);  // integrate.cpp:26-81
    if (!s && cudaMemcpyAsync(c->d_occ + c->p.nPd, dx, sizeof(double) * nH, cudaMemcpyDeviceToDevice, st))
      s = A2C_ERR_CUDA;
    double a = 0.0, b = 0.0;
    if (!s) s = launch_macro(c, dx, dsurf, n_surf, &a, &b);  // calculateresults.cpp:8-78
    if (!s) s = check_status_word(c);
    if (xH_mean) xH_mean[k] = a;
    if (xH_interior) xH_interior[k] = b;
    if (fmin) fmin[k] = f;
    if (iters) iters[k] = it;
  }
  if (!s && graph && engine_dmd_graph_usable(c, dp)) {
    DmdDev dd{dg, dsend, dx, drec, drec + 4 * (size_t)nsteps, dfull, dbd, dsurf, dcnt, n_bd, n_surf};
    s = engine_dmd_graph(c, dp, dd, eager_steps, nsteps);
    std::vector<double> rec(4 * (size_t)nsteps);
    int done[2] = {0, 0};
    if (!s && (cudaMemcpyAsync(rec.data(), drec, sizeof(double) * rec.size(), cudaMemcpyDeviceToHost, st) ||
               cudaMemcpyAsync(done, dcnt, sizeof(done), cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st)))
      s = A2C_ERR_CUDA;
    if (!s) s = check_status_word(c);
    if (!s && done[0] != nsteps) s = A2C_ERR_STATE;
    for (int k = eager_steps; k < nsteps && !s; ++k) {
      if (xH_mean) xH_mean[k] = rec[4 * (size_t)k];
      if (xH_interior) xH_interior[k] = rec[4 * (size_t)k + 1];
      if (fmin) fmin[k] = rec[4 * (size_t)k + 2];
      if (iters) iters[k] = (int)rec[4 * (size_t)k + 3];
    }
  } else if (!s && graph) {
    s = A2C_ERR_STATE;
  }
  if (!s && (cudaMemcpyAsync(X, c->d_X, sizeof(double) * 4 * c->N, cudaMemcpyDeviceToHost, st) ||
             cudaMemcpyAsync(xH, c->d_occ + c->p.nPd, sizeof(double) * nH, cudaMemcpyDeviceToHost, st) ||
             cudaMemcpyAsync(gamma, dg, sizeof(double) * nH, cudaMemcpyDeviceToHost, st) ||
             cudaMemcpyAsync(full_H, dfull, sizeof(int) * nH, cudaMemcpyDeviceToHost, st)))
    s = A2C_ERR_CUDA;
  free_hscratch(c, dg, dsend, dx, dfull);
  if (dbd) cudaFreeAsync(dbd, st);
  if (dsurf) cudaFreeAsync(dsurf, st);
  if (drec) cudaFreeAsync(drec, st);
  if (dcnt) cudaFreeAsync(dcnt, st);
  c->has_density = false;
  if (s) return s;
  return finish(c);
}

}  // extern "C"
