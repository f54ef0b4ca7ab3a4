// Internal declarations shared by the CUDA translation units of liba2c_gpp.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>

#include "a2c_gpp.h"

namespace a2c {

// Neighbor entry: global site id in the low 27 bits, periodic image code
// (mx+1) + 3(my+1) + 9(mz+1) in the top 5 bits; code 13 means no shift.
constexpr uint32_t kIdBits = 27;
constexpr uint32_t kIdMask = (1u << kIdBits) - 1u;
constexpr uint32_t kNoShift = 13u;
constexpr double kB = 8.6173324e-5;  // minimizer.cpp:92

// Batched instances (many independent lattices in one system): the sites
// of instance b are [start, start + nPd + nH), Pd first, in the caller's
// concatenated layout; neighbor lists never cross instances.
struct InstGeo {
  double S[3];   // periodic box length, or kFreeSpan in a free direction
  double T;      // temperature [K]
  float sc[3];   // S / 2^32 (one fixed-point unit of the mixed form)
  int start;     // first site
  int nPd, nH;
  float lim[3];  // free direction: how far a site may move from its list position (span guard); else +inf
};

// What a list-driven evaluator launch reads: the instance of every site,
// the per-instance geometry, and the sites to evaluate (count on device).
struct BatchView {
  const uint16_t *inst = nullptr;
  const InstGeo *geo = nullptr;
  const int *list = nullptr;
  const int *count = nullptr;
};

// Device pointers and scalars one FP64 kernel launch needs.
struct SiteArgs {
  int nPd, nH;
  double T, W, eps;
  double box[3];
  const double *X;      // 4N AoS [qx,qy,qz,sigma]
  const double *occ;    // N: 1 for Pd, x for H
  const int64_t *off;   // N+1
  const uint32_t *nbr;  // entries
  const int *npd;       // N: number of Pd entries at the head of each list
  double *rho;          // N
  double *Fp;           // N: F'(rho) of the site's species (FD form)
  double *G;            // 4N
  double *Vs;           // N: per-site energy partial
  double *Ss;           // N: per-site sigma-entropy partial
  int *status;          // device status word (0 = ok)
  BatchView bv;         // list-driven batched launch when bv.list != nullptr
};

// Device status bits (a2c never traps; kernels record and return).
// kStatusSpan: the mixed form's fixed-point span cannot represent a listed
// pair any more (a site moved too far in a free direction since the lists
// were built).
enum : int { kStatusNonfinite = 1, kStatusOverflow = 2, kStatusTimeout = 4, kStatusBadIndex = 8, kStatusSpan = 16 };

// The mixed form encodes free-direction coordinates modulo this span [A]:
// the difference of two encoded coordinates is exact while the pair is
// less than half of it apart.
constexpr double kFreeSpan = 64.0;

struct Mixed;   // mixed-precision buffers (k_mixed.cu)
struct Lbfgs;   // L-BFGS buffers (lbfgs.cu)

}  // namespace a2c

struct a2c_gpp_ctx {
  a2c_gpp_params p;
  int64_t N;
  int device;
  cudaStream_t stream;
  bool has_state, has_neighbors, has_density;
  // state and results
  double *d_X, *d_G, *d_occ, *d_rho, *d_Fp, *d_Vs, *d_Ss;
  double *d_red;   // reduction scratch (partials + scalars)
  int *d_status;
  // neighbors
  int64_t *d_off;
  uint32_t *d_nbr;
  int64_t nbr_cap, nbr_total;
  uint64_t nbr_version;  // bumped whenever the lists above change
  int *d_npd;
  int *d_shell;        // nPd x 3
  int64_t *d_hh1_off;  // nH+1
  int *d_hh1;
  int64_t hh1_cap, hh1_total;
  int max_neighbors;
  // skin lists: candidates at rc + skin and the positions they were built at
  double skin;
  bool has_ext;
  int64_t *d_ext_off;  // N+1
  uint32_t *d_ext_nbr;
  int64_t ext_cap, ext_total;
  double *d_xref;      // 4N
  // The mixed form's free-direction guard: positions the current lists were
  // built from (4N, allocated when a direction is free) and, per direction,
  // how far apart a listed pair was at most then (infinite when unknown).
  double *d_xlist;
  double list_reach[3];
  // host staging
  double *h_pinned;
  int64_t h_pinned_n;
  a2c::Mixed *mixed;
  a2c::Lbfgs *lbfgs;
  void *snap;  // the snapshot in flight (api.cu)
  void *engine;     // the device-driven minimizer (batch.cu), created on first use
  int host_loop;    // L-BFGS driver, A2C_MINIMIZER_* (a2c_gpp_set_minimizer)
  double *h_small;  // pinned: f and the status word of a host-pointer call
  int last_mixed_iters, last_fp64_iters;
  double last_mixed_gnorm;
};

namespace a2c {

// error helpers
a2c_status cuda_status(cudaError_t e);
#define A2C_CUDA(call)                               \
  do {                                               \
    cudaError_t e__ = (call);                        \
    if (e__ != cudaSuccess) return a2c::cuda_status(e__); \
  } while (0)
#define A2C_TRY(call)                \
  do {                               \
    a2c_status s__ = (call);         \
    if (s__ != A2C_OK) return s__;   \
  } while (0)

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

// Streaming multiprocessors of a device, queried once per device (api.cu).
constexpr int kMaxDevices = 64;
int device_sms(int dev);
int current_device_sms();
// Tile shape of the mixed pair kernels: threads per site (1, 2, 4, 8) and
// threads per block of pass 1 (256, 512, 768) and pass 2 (128, 256, 512);
// 0 = the library's choice.
struct Tile {
  int tps = 0, rho_block = 0, grad_block = 0;
  bool operator==(const Tile &o) const { return tps == o.tps && rho_block == o.rho_block && grad_block == o.grad_block; }
};
inline bool valid_tile(int tps, int rho_block, int grad_block) {
  return (tps == 0 || tps == 1 || tps == 2 || tps == 4 || tps == 8) &&
         (rho_block == 0 || rho_block == 256 || rho_block == 512 || rho_block == 768) &&
         (grad_block == 0 || grad_block == 128 || grad_block == 256 || grad_block == 512);
}
// The tile tuner (api.cu): threads per site at the default block sizes,
// then the pass-1 block size, then the pass-2 block size, each stage keeping
// the fastest; time_tile(tile, &ms) measures one candidate.  ms[10]
// receives the candidates' times in that order (may be null).
constexpr int kTileCandidates = 10;
a2c_status tune_tile(const std::function<a2c_status(const Tile &, float *)> &time_tile, Tile *best, float *ms);
// Threads per site of the mixed pair kernels when none was chosen: a
// system with fewer than 2048 sites per SM spreads each site over 4 lanes
// so that every SM gets work; a larger one runs one lane per site.
inline int default_threads_per_site(int64_t n_sites, int sms) { return n_sites < (int64_t)sms * 2048 ? 4 : 1; }

// k_fp64.cu
a2c_status launch_density64(a2c_gpp_ctx *c, const double *dX);
a2c_status launch_gradient64(a2c_gpp_ctx *c, const double *dX, double *dG);
a2c_status launch_eam64(a2c_gpp_ctx *c, int which, const double *d_in, int64_t n, double *d_out);
a2c_status launch_chem64(a2c_gpp_ctx *c, const double *dX, double gamma_bd, double *d_send, const int *d_full);
// batched: both passes over the listed sites (persistent grids; G, Vs, Ss)
a2c_status launch_eval64_list(a2c_gpp_ctx *c, const double *dX, double *dG, const BatchView &bv);

// k_misc.cu
a2c_status reduce_objective(a2c_gpp_ctx *c, double *d_f);        // f from Vs, Ss
a2c_status launch_finite_check(a2c_gpp_ctx *c, const double *d, int64_t n);
a2c_status launch_gamma_update(a2c_gpp_ctx *c, const double *d_send, double gamma_bd, double *d_gamma, int *d_full);
a2c_status launch_diffuse(a2c_gpp_ctx *c, const double *d_gamma, const int *d_full, double dt, double nu,
                          double Qm, double xLb, double xUb, double *d_x);
a2c_status launch_dirichlet(a2c_gpp_ctx *c, const int *d_sites, int n, double gamma_bd, double xUb, double *d_gamma,
                            int *d_full);
a2c_status launch_macro(a2c_gpp_ctx *c, const double *d_x, const int *d_surf_flags, int nSurf, double *h_xH,
                        double *h_xHint);
// the same reduction into d_out[2] on the device (stream-ordered, capturable)
a2c_status launch_macro_device(a2c_gpp_ctx *c, const double *d_x, const int *d_surf_flags, int nSurf, double *d_out);
a2c_status check_status_word(a2c_gpp_ctx *c);

// k_neighbors.cu
a2c_status build_neighbors_device(a2c_gpp_ctx *c, const double *h_X);
// skin path (positions in c->d_X; h_X may be null): rebuild the extended
// lists if needed, then re-filter at rc
a2c_status update_neighbors_device(a2c_gpp_ctx *c, const double *h_X, int *rebuilt, int moved);
// The skin path's new positions X (host memory; mX its device-visible view
// when pinned, else null), checked on the device -- A2C_ERR_NONFINITE,
// A2C_ERR_INVALID for a periodic coordinate outside [-L/2, 3L/2], d_X then
// unchanged -- and moved into d_X; moved = 1 when a site moved more than
// half the skin since the extended lists were built.
a2c_status stage_positions(a2c_gpp_ctx *c, const double *X, const double *mX, int *moved);

// The span guard of the mixed form: per direction, how far a site may move
// from the position the lists were built at before a listed pair could
// reach half the free span (+inf where periodic; negative when the lists'
// reach is unknown or too long), and the list positions to compare with
// (null when every direction is periodic).
void span_limits(const a2c_gpp_ctx *c, double lim[3], const double **xlist);

// k_mixed.cu
// ev: optional 5 events recorded before the first launch and after each
// stage (prep, pass 1, pass 2, reduction) on the context's stream
// Xcopy: X is the caller's pinned host memory (device-mapped); the prep
// kernel also copies it to Xcopy and flags non-finite values
// h_out: pinned host memory (2 doubles) that receives f and the status word
// (an int in the second; the device word is cleared), written by the last
// kernel where it finishes the objective, else copied
a2c_status mixed_eval(a2c_gpp_ctx *c, const double *dX, double *d_f, double *dG, cudaEvent_t *ev = nullptr,
                      double *Xcopy = nullptr, double *h_out = nullptr);
void mixed_free(a2c_gpp_ctx *c);
a2c_status mixed_set_threads_per_site(a2c_gpp_ctx *c, int tps);
int mixed_threads_per_site(a2c_gpp_ctx *c);
// the context's tile as chosen (zeros: the library's choice) and as used
a2c_status mixed_set_tile(a2c_gpp_ctx *c, const Tile &t);
Tile mixed_tile(a2c_gpp_ctx *c);
Tile effective_tile(const Tile &t, int64_t n_sites, int sms);
// batched: prep + both passes over the listed sites (G, Vs, Ss; no objective)
a2c_status mixed_eval_list(a2c_gpp_ctx *c, const double *dX, double *dG, const BatchView &bv, const Tile &tile);
a2c_status mixed_prepare(a2c_gpp_ctx *c);  // tables and buffers, before any graph capture
// the H sites' chemical potential (k_chem64's d_send) with the pair
// quadrature in FP32: pass 1 at dX, then the per-site sums; stream-ordered
a2c_status mixed_chem(a2c_gpp_ctx *c, const double *dX, double *d_send, const int *d_full);
// pass 2 pair visiting (A2C_PAIRS_*); the pairs-once index is rebuilt when
// the lists change (mixed_lists_changed, called after every list build)
a2c_status mixed_set_pair_mode(a2c_gpp_ctx *c, int mode);
a2c_status mixed_get_pair_mode(a2c_gpp_ctx *c, int *mode);
a2c_status mixed_lists_changed(a2c_gpp_ctx *c);
// what a captured batch tick bakes in of pass 2: the mode in use and the
// pairs-once index buffers (a graph is re-captured when any of them changes)
void mixed_graph_key(a2c_gpp_ctx *c, const void *key[5]);

// batch.cu: the one-instance device-driven minimizer of a context
a2c_status engine_minimize(a2c_gpp_ctx *c, double *dX, const a2c_lbfgs_params *lp, double *fmin, int *iters,
                           int *nfev, double *gnorm, int *reason);
// Device buffers of a DMD run (a2c_gpp_dmd_run): chemical potential, its
// pair sums, the diffused occupancy, full flags, boundary sites, surface
// flags; per step 4 records (xH mean, xH interior, f, iterations); two ints
// of loop counters.
struct DmdDev {
  double *gamma, *send, *x, *rec, *macro;
  int *full, *bd, *surf, *counters;
  int n_bd, n_surf;
};
// Outer steps first..nsteps-1 of a DMD run as one CUDA graph: a loop over
// steps, each the device-driven minimization (a loop over L-BFGS ticks)
// followed by the chemical potential, the Dirichlet condition, the
// diffusion step and the macro results.  Needs the context's engine (a
// step run eagerly before).  Waits for completion.
a2c_status engine_dmd_graph(a2c_gpp_ctx *c, const a2c_dmd_params *dp, const DmdDev &dd, int first, int nsteps);
bool engine_dmd_graph_usable(const a2c_gpp_ctx *c, const a2c_dmd_params *dp);
void engine_free(a2c_gpp_ctx *c);

// lbfgs.cu
a2c_status lbfgs_minimize(a2c_gpp_ctx *c, double *dX, const a2c_lbfgs_params *lp, double *fmin, int *iters,
                          int *nfev, double *gnorm, int *reason);
void lbfgs_free(a2c_gpp_ctx *c);

// api.cu
a2c_status eval_device_impl(a2c_gpp_ctx *c, const double *dX, double *d_f, double *dG, cudaEvent_t *ev = nullptr);

}  // namespace a2c
