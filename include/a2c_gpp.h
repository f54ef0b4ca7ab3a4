/*
 * a2c_gpp.h -- C ABI of the GB300-native GPP-EAM evaluator for a2c's
 * diffusive-molecular-dynamics hot path.
 *
 * Everything crosses this boundary as plain pointers, sizes and status codes;
 * no C++ exception, CUDA type or torch type appears in a signature.  A
 * context owns all device memory; host pointers are borrowed for the call.
 * Calls on one context are single-host-thread; all device work runs on the
 * context's stream.  Functions without the _device suffix take host
 * pointers and return after the results are in host memory; the _device
 * variants take device pointers and are stream-ordered.
 *
 * Layouts follow the reference:
 *   X, G   4*(nPd+nH) doubles, AoS per site [qx, qy, qz, sigma], all Pd sites
 *          then all H sites (minimizer.cpp:398-418, 464-473)
 *   xH     nH doubles, H site occupancy (Pd sites carry an implicit 1)
 *   lists  per-site neighbor indices local to the neighbor's species, as in
 *          the reference's PdPd / PdH / HPd / HH / HH1 vectors
 */
#ifndef A2C_GPP_H
#define A2C_GPP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  0 is success, as PetscErrorCode (minimizer.cpp:110). */
typedef int a2c_status;
enum {
  A2C_OK = 0,
  A2C_ERR_INVALID = 1,            /* bad argument or parameter */
  A2C_ERR_CUDA = 2,               /* a CUDA runtime call failed */
  A2C_ERR_NOMEM = 3,              /* device allocation failed */
  A2C_ERR_NEIGHBOR_OVERFLOW = 4,  /* a site exceeded the neighbor capacity */
  A2C_ERR_NONFINITE = 5,          /* NaN/Inf in an input or a result */
  A2C_ERR_STATE = 6,              /* call order violated (e.g. no neighbors) */
  A2C_ERR_TIMEOUT = 7,            /* a bounded device wait gave up */
  A2C_ERR_NO_DEVICE = 8,          /* no usable CUDA device */
  A2C_ERR_LISTS_STALE = 9         /* mixed form: since the neighbor lists were
                                     built a site moved so far in a free
                                     (non-periodic) direction that a listed
                                     pair could leave the form's fixed-point
                                     span (more than (32 A - reach) / 2, reach
                                     = the lists' cutoff); rebuild the lists */
};

/* Arithmetic forms of the evaluator. */
enum {
  A2C_FP64 = 0,  /* plain form: the reference's FP64 arithmetic and order */
  A2C_MIXED = 1  /* FP32 pair quadrature; FP64 per-site finish and entropy terms; the
                    objective summed exactly (fixed point), a batch's by an FP64 tree */
};

/* Neighbor list ids for a2c_gpp_get_neighbors. */
enum { A2C_LIST_PDPD = 0, A2C_LIST_PDH = 1, A2C_LIST_HPD = 2, A2C_LIST_HH = 3, A2C_LIST_HH1 = 4 };

/* L-BFGS termination reasons, numbered like TaoConvergedReason. */
enum {
  A2C_CONVERGED_GATOL = 3,
  A2C_CONVERGED_STALLED = 6, /* no objective progress (like TAO's steptol) */
  A2C_CONTINUE = 0,
  A2C_DIVERGED_MAXITS = -2,
  A2C_DIVERGED_NAN = -4,
  A2C_DIVERGED_MAXFCN = -5,
  A2C_DIVERGED_LS_FAILURE = -6
};

/* Problem parameters.  The reference reads these from its input object
 * (input.file.T0, eps, rc, a_Pd; QWp, coe_Pd, coe_H from the missing
 * driver).  periodic[] and box[] enable the minimum-image extension, which
 * the reference does not have. */
typedef struct a2c_gpp_params {
  int nPd, nH;
  double T;          /* temperature [K] */
  double QWp;        /* quadrature weight, 1/12 for the 12-point rule */
  double eps;        /* finite-difference step of the EAM derivatives */
  double rc;         /* neighbor cutoff [A] */
  double a_Pd;       /* lattice constant for shell classification [A] */
  double box[3];     /* periodic lengths [A] */
  int periodic[3];
  double coe_Pd[4];  /* correction coefficients of the chemical potential */
  double coe_H[4];
  int precision;     /* A2C_FP64 or A2C_MIXED */
  int device;        /* CUDA device ordinal */
} a2c_gpp_params;

typedef struct a2c_lbfgs_params {
  int m;            /* stored correction pairs */
  int max_it;       /* iteration cap */
  int max_fev;      /* objective-evaluation cap */
  int max_ls;       /* backtracking steps per line search */
  double gatol;     /* ||projected gradient||_2 tolerance (TAO gatol) */
  double c1;        /* Armijo constant */
  double init_step; /* max |component| of a steepest-descent step */
  double sigma_lb;  /* lower bound on widths (minimizer.cpp:815, 822) */
  double f_noise;   /* relative objective noise: a step whose |f change| is
                       below f_noise*|f| is accepted by the derivative form of
                       the Armijo test; 0 = 1e-14 (FP64) or 1e-7 (mixed) */
  int polish;       /* mixed precision: after the mixed phase stops, continue
                       with FP64 evaluations to gatol (1) or not (0) */
  int stall_window; /* stop (A2C_CONVERGED_STALLED) when f fell by no more
                       than stall_rtol*|f| over this many iterations */
  double stall_rtol;/* 0 = 1e-14 (FP64) or 1e-10 (mixed phase) */
  double max_step;  /* largest change of any coordinate or width in a first
                       trial step [A]: the line search starts from
                       min(1, max_step / max|d|); 0 = no cap.  Keeps widths
                       from being carried over the binding barrier into the
                       region where -3 kB x ln(sigma) falls without bound */
} a2c_lbfgs_params;

typedef struct a2c_gpp_ctx a2c_gpp_ctx;

/* Fills defaults: T=300, QWp=1/12, eps=1e-5, rc=5.35, a_Pd=3.89,
 * coefficients 0, FP64, device 0, non-periodic. */
void a2c_gpp_default_params(a2c_gpp_params *p);
void a2c_lbfgs_default_params(a2c_lbfgs_params *p);
const char *a2c_status_string(a2c_status s);

/* Lifecycle.  Replaces Minimizer::Minimizer + Minimizer::initialize
 * (minimizer.cpp:60-69, 484-546) and ~Minimizer (72-80). */
a2c_status a2c_gpp_create(const a2c_gpp_params *p, a2c_gpp_ctx **out);
a2c_status a2c_gpp_destroy(a2c_gpp_ctx *ctx);
/* The context's CUDA stream, as a cudaStream_t cast to void*. */
void *a2c_gpp_stream(a2c_gpp_ctx *ctx);
a2c_status a2c_gpp_set_precision(a2c_gpp_ctx *ctx, int precision);
/* Threads per site of the mixed-precision kernels: 1, 2, 4 or 8, or 0 to
 * let the library choose (a2c_gpp_autotune measures the candidates and sets
 * the fastest). */
a2c_status a2c_gpp_set_threads_per_site(a2c_gpp_ctx *ctx, int tps);
/* How the mixed-precision pass 2 visits pairs.  A2C_PAIRS_ONCE (default):
 * each pair is evaluated once, by the site with the larger id, which keeps
 * its own share and stores the neighbor's share in the neighbor's list slot
 * of the pair; a second kernel sums each site's received shares in list
 * order, so results are deterministic.  It needs every list sorted by id
 * and the lists symmetric, as the library's builds make them; other lists
 * (a2c_gpp_set_neighbor_lists input that is not) use A2C_PAIRS_BOTH_SIDES: each
 * site evaluates all of its pairs, the gather of minimizer.cpp:162-351.
 * a2c_gpp_get_pair_mode reports the mode the current lists run with. */
enum { A2C_PAIRS_BOTH_SIDES = 0, A2C_PAIRS_ONCE = 1 };
a2c_status a2c_gpp_set_pair_mode(a2c_gpp_ctx *ctx, int mode);
a2c_status a2c_gpp_get_pair_mode(a2c_gpp_ctx *ctx, int *mode);

/* Waits for all work queued on the context's stream (for _device calls). */
a2c_status a2c_gpp_synchronize(a2c_gpp_ctx *ctx);

/* H occupancy x0 used by every later call; replaces the x0 pointer swap of
 * Minimizer::updateApplicationContext (minimizer.cpp:372-378). */
a2c_status a2c_gpp_set_occupancy(a2c_gpp_ctx *ctx, const double *xH);
a2c_status a2c_gpp_get_occupancy(a2c_gpp_ctx *ctx, double *xH);
/* Stores X as the context's current state (used by chem_potential). */
a2c_status a2c_gpp_set_state(a2c_gpp_ctx *ctx, const double *X);
a2c_status a2c_gpp_get_state(a2c_gpp_ctx *ctx, double *X);

/* Neighbor build from positions X: cell list, d^2 <= rc^2, self excluded,
 * minimum image where periodic.  Replaces findNeighbors
 * (neighbors.cpp:8-115) followed by Minimizer::findLocalNeighbors
 * (minimizer.cpp:833-1144); the lists are held fixed until the next build,
 * as in the reference.  max_neighbors receives the largest per-site count
 * (the reference's maxNeib). */
a2c_status a2c_gpp_build_neighbors(a2c_gpp_ctx *ctx, const double *X, int *max_neighbors);
/* Neighbor lists supplied by the caller in the reference's form (the
 * PdPd/PdH/HPd/HH/HH1 vectors of findNeighbors / findLocalNeighbors, as
 * offsets[n+1] + local indices; PdPdnum may be NULL), e.g. the reference's
 * own KD-tree lists.  Each site's sums then run in the given order, as the
 * reference's loops do.  X gives the positions used to fix periodic images
 * (the reference has none: with no periodic dimension X may be NULL). */
a2c_status a2c_gpp_set_neighbor_lists(a2c_gpp_ctx *ctx, const double *X, const int64_t *pdpd_off,
                                      const int *pdpd_idx, const int64_t *pdh_off, const int *pdh_idx,
                                      const int64_t *hpd_off, const int *hpd_idx, const int64_t *hh_off,
                                      const int *hh_idx, const int64_t *hh1_off, const int *hh1_idx,
                                      const int *PdPdnum);
/* Sizes for a2c_gpp_get_neighbors: total entries of a list. */
/* Skin (Verlet) lists, replacing the refilter of findNeighbors' extended
 * lists in Minimizer::findLocalNeighbors (minimizer.cpp:833-1144).  With
 * skin > 0, a2c_gpp_update_neighbors keeps candidate lists at rc + skin and
 * re-filters them at rc on the device; it rebuilds the candidates (cell
 * list) only when a site has moved more than skin/2 since they were built
 * (*rebuilt = 1).  The lists it produces are those a2c_gpp_build_neighbors
 * would build at X.  Periodic boxes must exceed 2 (rc + skin).  skin = 0
 * (default): every update is a full build. */
a2c_status a2c_gpp_set_neighbor_skin(a2c_gpp_ctx *ctx, double skin);
a2c_status a2c_gpp_update_neighbors(a2c_gpp_ctx *ctx, const double *X, int *max_neighbors, int *rebuilt);

a2c_status a2c_gpp_neighbor_total(a2c_gpp_ctx *ctx, int list_id, int64_t *total);
/* Export a list in the reference's form: offsets[n+1], idx[total] local to
 * the neighbor species, each site's list sorted ascending. */
a2c_status a2c_gpp_get_neighbors(a2c_gpp_ctx *ctx, int list_id, int64_t *offsets, int *idx);
/* PdPdnum (minimizer.cpp:935-947): nPd x 3 shell counts. */
a2c_status a2c_gpp_get_shell_counts(a2c_gpp_ctx *ctx, int *PdPdnum);

/* Objective (free entropy) and gradient at X.  Replaces the TAO callback
 * Minimizer::formFunctionAndGradient (minimizer.cpp:83-369); X also becomes
 * the current state. */
a2c_status a2c_gpp_eval(a2c_gpp_ctx *ctx, const double *X, double *f, double *G);
a2c_status a2c_gpp_eval_device(a2c_gpp_ctx *ctx, const double *dX, double *df, double *dG);
/* Mixed-precision objective and gradient that allocates no device memory,
 * for callers that cannot call cudaMalloc while they evaluate: a host code
 * whose device memory belongs to another allocator (a solver framework's
 * callback running inside its own memory pool) or work being recorded by a
 * driver that forbids allocation during recording.  It has no counterpart
 * in the reference.  Inputs dX (4N doubles) and outputs df (1 double), dG
 * (4N doubles) are device pointers; the context supplies the neighbor lists
 * (build them first) and the occupancy; pass 2 evaluates each pair once
 * when the context holds a current pairs-once index (a mixed-precision
 * context builds it, and its share buffers, with its lists), else from
 * both sides.  All scratch lives in one fixed device array of about 5.8 MB that
 * every GPU loading the library keeps until the process exits, so problems
 * above 131,072 sites are rejected with A2C_ERR_INVALID.  The first call on
 * a device finds the array's address and loads constant tables into it
 * (synchronous copies): make that first call before any stream capture.  A
 * device reset (a new context) is noticed on the next call, which loads
 * them again.  Calls share the array and it keeps the last call's contents;
 * nothing in it needs clearing, but calls that overlap on the GPU (two
 * streams, two contexts on one device) race.  Stream-ordered on the
 * context's stream, like a2c_gpp_eval_device. */
a2c_status a2c_gpp_eval_mixed_noalloc(a2c_gpp_ctx *ctx, const double *dX, double *df, double *dG);
/* Host-only checks of the mixed form's functions (no GPU needed).
 * a2c_eam_analytic: value and exact derivative (forward mode, FP64) of the
 * EAM function numbered as in a2c_gpp_eam_eval (0 F_Pd, 2 F_H, 4 f_Pd,
 * 6 f_H, 8 phi_Pd, 10 phi_PdH, 12 phi_H), against which the reference's
 * central differences (potential.cpp:40-205) converge at second order.
 * a2c_mixed_table_eval: the FP32 table interpolants (0 F_Pd, 2 F_H, 4 f_Pd,
 * 8 phi_Pd) with the kernels' arithmetic. */
a2c_status a2c_eam_analytic(int which, const double *x, int64_t n, double *value, double *deriv);
a2c_status a2c_mixed_table_eval(int which, const double *x, int64_t n, double *value, double *deriv);

/* Autotuner (no reference counterpart): times the mixed-precision
 * evaluation at the context's current state (set by a2c_gpp_eval /
 * a2c_gpp_set_state) for 1, 2, 4 and 8 threads per site, `reps` timed
 * evaluations each after one untimed, and keeps the fastest for the
 * context.  tps receives the choice, ms[4] (may be NULL) the mean time per
 * evaluation of each candidate in milliseconds. */
a2c_status a2c_gpp_autotune(a2c_gpp_ctx *ctx, int reps, int *tps, float *ms);
/* Tile shape of the mixed-precision pair kernels: threads per site (1, 2,
 * 4, 8) and threads per block of pass 1 (256, 512, 768 -- its 98 KB of
 * table copies allow two blocks per SM, so larger blocks mean more resident
 * warps) and of pass 2 (128, 256, 512); 0 = the library's choice.
 * a2c_gpp_get_tile reports the tile in use, tile[3] = {tps, pass-1 block,
 * pass-2 block}.  a2c_gpp_autotune_tile measures candidates by coordinate
 * descent -- threads per site at 256-thread blocks, then the pass-1 block,
 * then the pass-2 block, each stage keeping the fastest -- on the context's
 * current state, sets the fastest and returns it; ms[10] (may be NULL)
 * receives the mean milliseconds per evaluation of the ten candidates in
 * that order. */
a2c_status a2c_gpp_set_tile(a2c_gpp_ctx *ctx, int tps, int rho_block, int grad_block);
a2c_status a2c_gpp_get_tile(a2c_gpp_ctx *ctx, int *tile);
a2c_status a2c_gpp_autotune_tile(a2c_gpp_ctx *ctx, int reps, int *tile, float *ms);

/* Which L-BFGS driver a2c_gpp_minimize and a2c_gpp_dmd_run use.
 * A2C_MINIMIZER_DEFAULT: mixed precision device-driven -- each L-BFGS
 * iteration is one CUDA-graph replay of the batched engine with this
 * context as its only instance (global sums in the per-instance chunk
 * order) -- and the FP64 plain form host-driven (its reductions replayed
 * bit for bit by the oracle).  A2C_MINIMIZER_HOST: the host-driven loop for
 * both forms.  A2C_MINIMIZER_DEVICE: the device-driven engine for both
 * forms (for FP64, the same minimization in the engine's summation order).
 * The value 1 keeps its earlier meaning (host_loop = 1). */
enum { A2C_MINIMIZER_DEFAULT = 0, A2C_MINIMIZER_HOST = 1, A2C_MINIMIZER_DEVICE = 2 };
a2c_status a2c_gpp_set_minimizer(a2c_gpp_ctx *ctx, int mode);

/* Profiling aid: one stream-ordered evaluation on device pointers with CUDA
 * events between its launches; stage_ms[4] receives the durations of the
 * state preparation, pass 1 (densities), pass 2 (energy and gradient) and
 * the objective reduction.  Waits for completion. */
a2c_status a2c_gpp_profile_eval(a2c_gpp_ctx *ctx, const double *dX, double *df, double *dG, float *stage_ms);
/* Site electron densities of the last evaluation, all Pd then all H
 * (electrondensity.cpp:12-56, the reference's recv_Pd / recv_H). */
a2c_status a2c_gpp_get_density(a2c_gpp_ctx *ctx, double *rho);

/* Known-answer access to the device EAM functions (potential.cpp:16-205):
 * evaluates function `which` (0 F_Pd, 1 F_Pd_deriv, 2 F_H, 3 F_H_deriv,
 * 4 f_Pd, 5 f_Pd_deriv, 6 f_H, 7 f_H_deriv, 8 phi_Pd, 9 phi_Pd_deriv,
 * 10 phi_PdH, 11 phi_PdH_deriv, 12 phi_H, 13 phi_H_deriv) of the FP64 plain
 * form on the context's device, host arrays in and out, step = params eps. */
a2c_status a2c_gpp_eam_eval(a2c_gpp_ctx *ctx, int which, const double *in, int64_t n, double *out);

/* Variable bounds: q free, sigma >= 1e-6 (minimizer.cpp:804-830). */
a2c_status a2c_gpp_bounds(a2c_gpp_ctx *ctx, double *lb, double *ub);

/* Iterations of the last a2c_gpp_minimize spent in each precision. */
a2c_status a2c_gpp_minimize_stats(a2c_gpp_ctx *ctx, int *mixed_iters, int *fp64_iters, double *mixed_gnorm);

/* Bound-constrained L-BFGS from X (in/out) on the device; replaces
 * Minimizer::minimizeFreeEntropy + TaoSolve (minimizer.cpp:548-586).
 * X becomes the current state.  reason follows TaoConvergedReason. */
a2c_status a2c_gpp_minimize(a2c_gpp_ctx *ctx, double *X, const a2c_lbfgs_params *lp, double *fmin, int *iters,
                            int *nfev, double *gnorm, int *reason);

/* Occupancy gradient / chemical potential at the current state.  Replaces
 * Minimizer::calculateChemicalPotential (minimizer.cpp:588-802); gamma and
 * full_H are nH arrays, read and updated in place.  A mixed-precision
 * context evaluates the pair quadrature in FP32 (compensated per-site sums,
 * F and F' from its pass 1) and the rest in FP64; an FP64 context follows
 * the reference's arithmetic. */
a2c_status a2c_gpp_chem_potential(a2c_gpp_ctx *ctx, double gamma_bd, double *gamma, int *full_H);

/* Dirichlet condition on the listed H sites: gamma = gamma_bd, full_H = 1,
 * x0 = xUb, applied to the context occupancy and to the caller's arrays.
 * Replaces enforceBoundaryConditions (boundaryconditions.cpp:30-55). */
a2c_status a2c_gpp_apply_dirichlet(a2c_gpp_ctx *ctx, const int *sites, int n, double gamma_bd, double xUb,
                                   double *gamma, int *full_H);

/* One explicit mean-field diffusion step over the first H shell from the
 * context occupancy x0 into x (nH, in/out: sites with full_H == 1 keep the
 * caller's value).  Replaces integrateDiffusion (integrate.cpp:9-87). */
a2c_status a2c_gpp_diffuse(a2c_gpp_ctx *ctx, double dt, double nu, double Qm, double xLb, double xUb,
                           const double *gamma, const int *full_H, double *x);

/* The same step with caller-supplied first-shell lists and occupancy, no
 * context: integrateDiffusion's own signature (integrate.cpp:9-87), on
 * `device`.  x0, gamma, full_H, x are host arrays of nH. */
a2c_status a2c_diffuse_lists(int device, int nH, const int64_t *hh1_off, const int *hh1_idx, const double *x0,
                             const double *gamma, const int *full_H, double T, double dt, double nu, double Qm,
                             double xLb, double xUb, double *x);

/* Mean H fraction over all H sites and over sites not in HSurf.  Replaces
 * calculateMacroResults (calculateresults.cpp:8-78). */
a2c_status a2c_gpp_macro_results(a2c_gpp_ctx *ctx, const double *x, const int *HSurf, int nSurf, double *xH,
                                 double *xHinterior);

/* Measured peak of the FP64 (precision A2C_FP64) or FP32 (A2C_MIXED) FMA
 * pipe of a device, in flop/s: the roofline denominator for the evaluator's
 * compute-bound kernels (no reference counterpart; a measurement aid). */
a2c_status a2c_gpp_peak_flops(int device, int precision, double *flops_per_s);

/* One DMD outer step, as the reference's (missing) driver sequences it
 * (minimizer.cpp:548, 588; boundaryconditions.cpp:30; integrate.cpp:9;
 * calculateresults.cpp:8): minimize the free entropy at fixed occupancy,
 * chemical potential at the minimum, Dirichlet condition on the boundary
 * sites, one explicit diffusion step, occupancy <- diffused occupancy, macro
 * results. */
typedef struct a2c_dmd_params {
  double dt, nu, Qm;       /* time step [s], attempt frequency [1/s], activation energy [eV] */
  double xLb, xUb;         /* clamp of the diffusion step */
  double x_bd, gamma_bd;   /* occupancy and chemical potential held on the boundary sites */
  a2c_lbfgs_params lbfgs;  /* the minimization of every step */
  int neighbor_update;     /* 1: re-derive the neighbor lists (incl. HH1) at the start of every step after the
                              first, through the skin refilter when a skin is set; 0: keep them fixed */
  int host_steps;          /* 0 (default): with fixed lists and the device-driven minimizer, the first step runs
                              eagerly and steps 2..nsteps as ONE CUDA graph -- a device loop over outer steps,
                              each a device loop over L-BFGS ticks followed by the chemical potential, the
                              Dirichlet condition, the diffusion step and the macro results, with no host
                              round trip; 1: every step sequenced from the host (same results, bit for bit) */
} a2c_dmd_params;

/* Runs nsteps outer steps with all state on the device; X (4N), xH, gamma,
 * full_H (nH) are read at the start and written back at the end.
 * Per step k: xH_mean[k], xH_interior[k] (macro results over all H sites /
 * those not in surf_sites), fmin[k] and iters[k] of the minimization (any of
 * the four output arrays may be NULL).  Neighbor lists are held fixed, as
 * the reference holds them through a solve; build them before the call. */
a2c_status a2c_gpp_dmd_run(a2c_gpp_ctx *ctx, double *X, double *xH, double *gamma, int *full_H, const int *bd_sites,
                           int n_bd, const int *surf_sites, int n_surf, const a2c_dmd_params *dp, int nsteps,
                           double *xH_mean, double *xH_interior, double *fmin, int *iters);

/* Restart file in the format readResults reads (readresults.cpp:10-55):
 * 9 header lines, then one row of 9 columns per site, Pd rows first:
 *   id species qx qy qz sigma x gamma full_H
 * (the reader ignores the first two columns and, for Pd rows, the last
 * three).  The writer has no counterpart in the reference tree.  The reader
 * clamps x to [xLb, xUb] as readresults.cpp:48-51 does. */
a2c_status a2c_restart_write(const char *path, int nPd, int nH, const double *X, const double *xH,
                             const double *gamma, const int *full_H, int step, double time);
a2c_status a2c_restart_read(const char *path, int nPd, int nH, double xLb, double xUb, double *X, double *xH,
                            double *gamma, int *full_H);

/* ------------------------------------------------------------------------
 * Batched independent instances (the reference runs one lattice per
 * process; these entry points have no reference counterpart and replace a
 * loop of Minimizer::initialize + minimizeFreeEntropy, minimizer.cpp:484-586,
 * over many lattices).  Instance b is described by params[b] (its nPd, nH,
 * T, box, periodic flags); QWp, eps, rc, a_Pd, the correction coefficients,
 * the precision and the device must agree across instances.  Arrays are the
 * instances' reference-layout arrays concatenated in instance order: X and
 * G are sum(4 (nPd_b + nH_b)) doubles, xH is sum(nH_b).  All instances are
 * evaluated by one launch of each kernel; their reductions are per instance
 * and do not depend on the other instances.
 * ------------------------------------------------------------------------ */
typedef struct a2c_gpp_batch a2c_gpp_batch;

a2c_status a2c_gpp_batch_create(const a2c_gpp_params *params, int n_instances, a2c_gpp_batch **out);
a2c_status a2c_gpp_batch_destroy(a2c_gpp_batch *batch);
a2c_status a2c_gpp_batch_info(a2c_gpp_batch *batch, int *n_instances, int64_t *n_sites);
a2c_status a2c_gpp_batch_set_occupancy(a2c_gpp_batch *batch, const double *xH);
/* per-instance neighbor build (findNeighbors + findLocalNeighbors, as
 * a2c_gpp_build_neighbors) from host X; max_neighbors may be NULL */
a2c_status a2c_gpp_batch_build_neighbors(a2c_gpp_batch *batch, const double *X, int *max_neighbors);
/* mixed-precision threads per site (0 = library choice), as
 * a2c_gpp_set_threads_per_site */
a2c_status a2c_gpp_batch_set_threads_per_site(a2c_gpp_batch *batch, int tps);
/* 1 (default): one L-BFGS tick of all instances is captured once in a CUDA
 * graph and replayed; 0: the same launches issued one by one */
a2c_status a2c_gpp_batch_set_graphs(a2c_gpp_batch *batch, int on);
/* host X (4N) -> f[n_instances], G (4N) */
a2c_status a2c_gpp_batch_eval(a2c_gpp_batch *batch, const double *X, double *f, double *G);
/* Minimizes every instance (the algorithm of a2c_gpp_minimize, per
 * instance) from X, which receives the minima.  Per instance: fmin, iters,
 * nfev, gnorm, reason; mixed_iters / fp64_iters (may be NULL) split the
 * iterations between the mixed phase and the FP64 polish.  Instances retire
 * when they stop; the call returns when all have. */
a2c_status a2c_gpp_batch_minimize(a2c_gpp_batch *batch, double *X, const a2c_lbfgs_params *lbfgs, double *fmin,
                                  int *iters, int *nfev, double *gnorm, int *reason, int *mixed_iters,
                                  int *fp64_iters);
/* ticks (one evaluation of every live instance each) and device seconds of
 * the last a2c_gpp_batch_minimize */
a2c_status a2c_gpp_batch_stats(a2c_gpp_batch *batch, int *ticks, double *seconds);
/* the autotuner (see a2c_gpp_autotune) over the whole batch at host X */
a2c_status a2c_gpp_batch_autotune(a2c_gpp_batch *batch, const double *X, int reps, int *tps, float *ms);
/* The tile of the batch's mixed pair kernels (see a2c_gpp_set_tile):
 * set, read back, and tuned on the whole batch at X (every instance
 * evaluated per candidate). */
a2c_status a2c_gpp_batch_set_tile(a2c_gpp_batch *batch, int tps, int rho_block, int grad_block);
a2c_status a2c_gpp_batch_get_tile(a2c_gpp_batch *batch, int *tile);
a2c_status a2c_gpp_batch_autotune_tile(a2c_gpp_batch *batch, const double *X, int reps, int *tile, float *ms);

/* Solution snapshots in the formats of the reference's Output class
 * (Output.cpp:60-90, 133-480): per frame a VTK PolyData file
 * <prefix>_L<k>_<frame>.vtp (points q; SiteID, MaterialID, Tag,
 * AtomicFrequency = sigma, MolarFraction = occupancy, ChemicalPotential =
 * gamma) with an entry in the collection <prefix>_L<k>.pvd, and/or an
 * extended-XYZ file <prefix>_L<k>_<frame>.xyz (species, q, q - q0, site id,
 * sigma, tag, occupancy, gamma).  One lattice, one species column pair:
 * Pd sites carry occupancy 1 and gamma 0. */
typedef struct a2c_snapshot_desc {
  const char *prefix;   /* path prefix including the file base name */
  int format;           /* 1 VTP, 2 XYZ, 3 both (OutputData::VTP, XYZ, VTP_and_XYZ) */
  int precision;        /* 0 %7.4e, 1 %10.6e, 2 %16.10e (OutputData precision LOW, MEDIUM, HIGH) */
  double axes[9];       /* lattice axes a, b, c for the XYZ header */
  double origin[3];
  int periodic[3];
  int lattice_id;       /* the k of _L<k> in the file names (Output.cpp:74, 143); 0 for the evaluator's lattice */
} a2c_snapshot_desc;
/* the collection header (Output's constructor); call once before the frames */
a2c_status a2c_snapshot_begin(const a2c_snapshot_desc *desc);
/* host arrays: X (4N), X0 (4N, may be NULL: zero displacement), xH (nH),
 * gamma (nH, may be NULL), siteid / tag (N, may be NULL: species / 0) */
a2c_status a2c_snapshot_write(const a2c_snapshot_desc *desc, int frame, double time, int nPd, int nH, const double *X,
                              const double *X0, const double *xH, const double *gamma, const signed char *siteid,
                              const signed char *tag);
/* The context's current state (positions, widths, occupancy) written
 * without stalling the GPU: copied on the context's stream into pinned host
 * memory, then formatted and written by a host thread while later work
 * runs.  The host arrays (X0, gamma, siteid, tag; each may be NULL) are
 * copied before the call returns.  One snapshot is in flight per context;
 * a new one (or a2c_gpp_snapshot_wait, or destroy) waits for the previous
 * one, and a2c_gpp_snapshot_wait returns its status. */
a2c_status a2c_gpp_snapshot_async(a2c_gpp_ctx *ctx, const a2c_snapshot_desc *desc, int frame, double time,
                                  const double *X0, const double *gamma, const signed char *siteid,
                                  const signed char *tag);
a2c_status a2c_gpp_snapshot_wait(a2c_gpp_ctx *ctx);

/* Input files in the reference's syntax (parser/Parser.y, parser/Lexer.l:
 * assignments, "under X { ... }" groups, dotted and indexed names,
 * integer/double expressions, strings, keywords, comments, "end"), read by a
 * hand-written parser.  The fields below are filled from the reference's
 * keys with its defaults (IoData.cpp); other objects of a full input file
 * (geometry, species, initial conditions, ...) are parsed and counted. */
typedef struct a2c_input {
  double T, nu, Qm, t_subsurf, mubd; /* Diffusion.Temperature, AttemptFrequency, ActivationEnergy,
                                        SubsurfaceThickness, SoluteChemicalPotential */
  double eps, rc;                    /* Material[0].InteratomicPotential.Tolerance, CutOffDistance */
  char potential_file[256];          /* Material[0].InteratomicPotential.File */
  double dt, max_time, cfl;          /* Time.TimeStep, MaxTime, CFL */
  int max_its;                       /* Time.MaxIts */
  int output_format;                 /* Output.Format: 1 VTP, 2 XYZ, 3 both (a2c_snapshot_desc.format) */
  int output_precision;              /* Output.Precision: 0 Low, 1 Medium, 2 High */
  int output_frequency;              /* Output.Frequency */
  double output_interval;            /* Output.TimeInterval */
  char output_prefix[256], output_solution[256]; /* Output.Prefix, Output.Solution */
  double lattice_axes[9];            /* Lattice[0].OAx ... OCz */
  double lattice_origin[3];          /* Lattice[0].Ox, Oy, Oz */
  int lattice_periodic[3];           /* Lattice[0].PeriodicOA/OB/OC */
  int n_assignments;                 /* assignments in the file */
  int n_used;                        /* of which filled a field above */
} a2c_input;
/* errmsg (may be NULL) receives "syntax error near line N" and the like */
a2c_status a2c_input_read(const char *path, a2c_input *input, char *errmsg, int errlen);
/* T, eps, rc of an input into evaluator parameters */
a2c_status a2c_input_apply(const a2c_input *input, a2c_gpp_params *params);

/* Seeded synthetic fcc Pd lattice with octahedral H sites (stand-in for the
 * reference's SpaceInitializer lattice setup).  Site order: cells z, y, x,
 * then basis; all Pd then all H.  Writes X (4N), xH (nH) and surface flags
 * (nH; 1 where the unperturbed z is below 1e-6). */
typedef struct a2c_lattice_spec {
  int ncell[3];
  double a;
  int periodic[3];
  double pos_std;          /* N(0, pos_std) per position component */
  double sigma_lo, sigma_hi; /* sigma ~ U(lo, hi), or lo when hi <= lo */
  int x_mode;              /* 0: x = x_center + U(-x_half, x_half); 1: nucleus */
  double x_center, x_half;
  double x_matrix, x_nucleus, nucleus_radius, interface_width;
  double xLb, xUb;         /* clamp of the drawn occupancy */
  uint64_t seed;
} a2c_lattice_spec;
a2c_status a2c_lattice_fcc(const a2c_lattice_spec *spec, double *X, double *xH, int *surface);
/* The same lattice generated on the device, one thread per site: device
 * pointers X (4N), xH and surface (nH; may be NULL), stream-ordered on
 * `stream` (a cudaStream_t, NULL = default stream).  Lattice positions,
 * fixed widths and the deterministic occupancy profile are those of
 * a2c_lattice_fcc; the random draws come from a counter-based SplitMix64
 * stream (draw k of site s = output 8 s + k), so they follow the same
 * distributions with other values. */
a2c_status a2c_lattice_fcc_device(const a2c_lattice_spec *spec, double *X, double *xH, int *surface, void *stream);

/* Lattice set-up from an input file's lattice description: replaces
 * SpaceInitializer::CreateOneLattice (SpaceInitializer.cpp:119-320) and
 * CheckAndAddSitesInCell (:603-724).  The lattice cells inside the
 * bounding box of the interior geometries (FindLatticeDomainBoundingBox,
 * :726-880, with GeoTools' bounding boxes) are visited c, b, a (slowest to
 * fastest); each site group of a cell is kept when the geometries, applied
 * in their operation order as Intersection or Union, contain it.  Sites are
 * in that order.  Not built: the custom-geometry plug-in (dlopen) and the
 * regional initial conditions (ApplyRegionalICOnOneLattice). */
enum {
  A2C_GEOM_PLANE = 0,            /* p: point[3], normal[3]; contains q where (q-point).n/|n| > 0 */
  A2C_GEOM_CYLINDER_CONE = 1,    /* p: base centre[3], axis[3], radius, height, opening angle (deg), cone height */
  A2C_GEOM_CYLINDER_SPHERE = 2,  /* p: base centre[3], axis[3], radius, height, front cap (0/1), back cap (0/1) */
  A2C_GEOM_SPHERE = 3,           /* p: centre[3], radius */
  A2C_GEOM_PARALLELEPIPED = 4,   /* p: P[3], A[3], B[3], C[3] (vertices: edges PA, PB, PC, right-handed) */
  A2C_GEOM_SPHEROID = 5          /* p: centre[3], axis[3], semi-length (along the axis), radius */
};
enum { A2C_INCLUSION_INTERSECTION = 1, A2C_INCLUSION_UNION = 2 };
typedef struct a2c_geometry {
  int type;       /* A2C_GEOM_* */
  int order;      /* OperationOrder: 0 .. ngeom-1, each once */
  int inclusion;  /* A2C_INCLUSION_* */
  int exterior;   /* Side: 0 Interior, 1 Exterior (not read for planes) */
  double p[12];
} a2c_geometry;
typedef struct a2c_site_group {
  double l[3];               /* La, Lb, Lc: lattice coordinates in the cell */
  int materialid, tag;
  double atomic_frequency;   /* the initial width sigma */
  double mean_displacement[3];
  double x;                  /* LocalSpecies[0].MolarFraction (-1e-3: not given, the reference's default) */
} a2c_site_group;
typedef struct a2c_lattice_desc {
  double abc[9];        /* lattice vectors OA, OB, OC */
  double origin[3];
  int periodic[3];
  double dmin;          /* MinDistance (<= 0: the shortest lattice vector, as the reference) */
  int nsites;
  const a2c_site_group *sites;
  int ngeom;
  const a2c_geometry *geoms;
} a2c_lattice_desc;
typedef struct a2c_lattice_sites {
  int64_t capacity;     /* sites the arrays hold; 0 with NULL arrays counts only */
  int64_t count;        /* set: sites of the lattice (all of them, also when above capacity) */
  double *q, *q0, *l;   /* 3 per site: position (q0 + mean displacement), lattice position, lattice coordinates */
  int *siteid, *matid, *tag;
  double *sigma, *x;
} a2c_lattice_sites;
a2c_status a2c_lattice_build(const a2c_lattice_desc *desc, a2c_lattice_sites *out, char *errmsg, int errlen);
/* Snapshot of a set-up lattice's sites (a2c_lattice_sites with count
 * sites): the files of a2c_snapshot_write with each site's own site group,
 * material id, tag, width and occupancy, and in the XYZ species column its
 * material's name (material_names[matid], else "M<matid>"), as Output.cpp
 * writes a lattice (:133-480).  gamma (count, may be NULL: 0). */
a2c_status a2c_snapshot_write_lattice(const a2c_snapshot_desc *desc, int frame, double time,
                                      const a2c_lattice_sites *sites, const double *gamma,
                                      const char *const *material_names, int n_materials);
/* SetupLatticeVariables' removal of sites closer than dmin to another
 * lattice's sites (SpaceInitializer.cpp:94-112, LatticeVariables.cpp:78-140):
 * keep[i] = 0 for every site i of q (n sites) with a site of q_other
 * within dmin in every coordinate (the KD-tree box test of
 * KDTree.h:244-262), else 1.  Returns the number removed in *n_removed. */
a2c_status a2c_lattice_conflicts(const double *q, int64_t n, const double *q_other, int64_t n_other, double dmin,
                                 unsigned char *keep, int64_t *n_removed);
/* A regional initial condition (RegionalIcData; applied by
 * SpaceInitializer::ApplyRegionalICOnOneLattice, SpaceInitializer.cpp:
 * 883-1040): on the sites of material materialid and site group siteid
 * whose current position q the geometries contain (the rule of
 * a2c_lattice_build), q moves by mean_displacement, sigma becomes
 * atomic_frequency (as given: the reference sets it also when left at its
 * -1 default), tag becomes tag, and x becomes x when x >= 0 (the first
 * LocalSpecies' MolarFraction; one species per site here).  lattice_id < 0:
 * every lattice. */
typedef struct a2c_region {
  int lattice_id, materialid, siteid, tag;
  double atomic_frequency;
  double mean_displacement[3];
  double x;
  int ngeom;
  const a2c_geometry *geoms;
} a2c_region;
/* Applies one region to out->count sites (arrays as a2c_lattice_build
 * filled them), in place. */
a2c_status a2c_lattice_apply_region(const a2c_region *region, a2c_lattice_sites *sites, char *errmsg, int errlen);
/* The RegionalInitialCondition[k] blocks of an input file, k = 0 .. n-1,
 * into regions[] (max_regions) with their geometries stored in geoms[]
 * (max_geoms in all); *n_regions receives n. */
a2c_status a2c_input_regions(const char *path, a2c_region *regions, int max_regions, a2c_geometry *geoms,
                             int max_geoms, int *n_regions, char *errmsg, int errlen);
/* Material[0 .. n-1].MaterialName of an input file (IoData.cpp:538-560;
 * default ""): names[m] receives up to name_len bytes each (names holds
 * max_materials * name_len); *n_materials receives n. */
a2c_status a2c_input_material_names(const char *path, char *names, int max_materials, int name_len,
                                    int *n_materials, char *errmsg, int errlen);
/* Lattice[id] of an input file as a description: sites (capacity
 * max_sites) and geometries (max_geoms) are filled from the file's
 * Site[k] and Plane/Sphere/Parallelepiped/Spheroid/CylinderAndCone/
 * CylinderWithSphericalCaps[k] blocks with the reference's defaults
 * (IoData.cpp:9-470); desc->sites / geoms point at the arrays given. */
a2c_status a2c_input_lattice(const char *path, int lattice_id, a2c_lattice_desc *desc, a2c_site_group *sites,
                             int max_sites, a2c_geometry *geoms, int max_geoms, char *errmsg, int errlen);

#ifdef __cplusplus
}
#endif
#endif
