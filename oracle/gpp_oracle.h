/*
 * CPU oracle for the GPP-EAM hot path of a2c -- TEST INFRASTRUCTURE ONLY.
 *
 * This library is a plain C++ restatement of the reference's CPU algorithm,
 * kept in the reference's operation order (finite-difference derivatives,
 * left-to-right products, per-pair-point redundant embedding-derivative calls)
 * so that its FP64 results are bit-comparable with the reference.  It is used
 * by the tests (as the checker), by __graft_entry__.smoke(), and by bench.py's
 * CPU-baseline leg.  No product code path links, loads or calls it.
 *
 * Reference files restated (paths inside the a2c project):
 *   potential.cpp:16-205        EAM functions and their FD derivatives
 *   quadrature.cpp:101-133      12-point Gaussian rule for dim = 6
 *   electrondensity.cpp:12-56   pass 1 (site electron density)
 *   minimizer.cpp:83-369        objective + gradient (TAO callback)
 *   minimizer.cpp:588-802       chemical potential / occupancy gradient
 *   minimizer.cpp:804-830       variable bounds (sigma >= 1e-6)
 *   minimizer.cpp:833-1144      local neighbor refilter, Pd shells, HH1
 *   neighbors.cpp:8-115         neighbor predicate (d^2 <= rc^2, self excluded)
 *   integrate.cpp:9-87          mean-field H diffusion
 *   boundaryconditions.cpp:30-55 Dirichlet boundary condition
 *   calculateresults.cpp:8-78   macro results (H fraction)
 *   Vector3D.h:83,281-316       Vec3D norm / dot / scalar product order
 *
 * Parity pin: oracle/Makefile (target `ref`) compiles the reference's own
 * hot-path sources against single-rank shims (oracle/ref_shim) into
 * oracle/_ref, and tests/test_oracle_pin.py checks this restatement against
 * it bit for bit.
 */
#ifndef A2C_GPP_ORACLE_H
#define A2C_GPP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
  int nPd, nH;
  double T;        /* temperature, input.file.T0 */
  double QWp;      /* quadrature weight */
  double eps;      /* finite-difference step, input.file.eps */
  double rc;       /* neighbor cutoff, input.file.rc */
  double a_Pd;     /* lattice constant used for the shell tests */
  double box[3];   /* periodic lengths (used only where periodic[d] != 0) */
  int periodic[3]; /* minimum-image extension; the reference has none */
  double coe_Pd[4], coe_H[4];
} orc_params;

typedef struct orc_lbfgs {
  int m;            /* memory pairs */
  int max_it;       /* iteration cap */
  int max_fev;      /* evaluation cap */
  int max_ls;       /* backtracking steps per line search */
  double gatol;     /* ||projected gradient||_2 tolerance */
  double c1;        /* Armijo constant */
  double init_step; /* max |displacement| of the first (steepest) step */
  double sigma_lb;  /* lower bound on widths */
  double f_noise;   /* relative objective noise for the derivative Armijo form; 0 = 1e-14 */
  int stall_window; /* stop (6) when f fell by <= stall_rtol*|f| over this many iterations */
  double stall_rtol;/* 0 = 1e-14 */
  double max_step;  /* first trial step length min(1, max_step / max|d|); 0 = no cap */
} orc_lbfgs;

/* Arithmetic mode: 0 = the reference's (C library exp/pow/log, sequential
 * sums; the default, pinned to the reference); 1 = the device's (portable
 * exp/pow/log of a2c_gb300/csrc/ddmath.cuh and the GPU reduction tree). */
void orc_set_arith(int mode);
int orc_get_arith(void);
/* Reduction order of the device arithmetic: 0 = the single-system trees
 * (grid-strided partials); chunk > 0 = the batched-instance order (per
 * instance, partials of `chunk` consecutive terms, then one block). */
void orc_set_reduction(int chunk);
int orc_get_reduction(void);

/* EAM function by id (see gpp_oracle.cpp: 0..13), applied elementwise. */
void orc_eam(int which, const double *in, int64_t n, double eps, double *out);

/* Neighbor build.  Entries are global site ids (Pd 0..nPd-1, H nPd..N-1) in
 * the low 27 bits and the periodic image code in the top 5 bits; each site's
 * list is sorted by global id (so Pd neighbors precede H neighbors). */
int orc_neighbor_counts(const orc_params *p, const double *X, int64_t *counts,
                        int64_t *hh1_counts);
int orc_neighbor_fill(const orc_params *p, const double *X, const int64_t *off,
                      uint32_t *nbr, int *PdPdnum, const int64_t *hh1_off,
                      int *hh1);

/* Objective/gradient.  X and G are 4N AoS [qx,qy,qz,sigma] per site, Pd block
 * then H block (minimizer.cpp:398-418).  mode 0 accumulates the energy into a
 * single running sum in the reference's loop order (single thread); mode 1
 * sums per-site partials (OpenMP over sites).  rho and Vsite may be NULL. */
int orc_eval(const orc_params *p, const double *X, const double *xH,
             const int64_t *off, const uint32_t *nbr, int mode, int nthreads,
             double *f, double *G, double *rho, double *Vsite);

int orc_density(const orc_params *p, const double *X, const double *xH,
                const int64_t *off, const uint32_t *nbr, int nthreads,
                double *rho);

int orc_chem_potential(const orc_params *p, const double *X, const double *xH,
                       const int64_t *off, const uint32_t *nbr, double gamma_bd,
                       int nthreads, double *gamma, int *full_H);

int orc_diffuse(int nH, const double *x0, const int64_t *hh1_off,
                const int *hh1, const double *gamma, const int *full_H,
                double T, double dt, double nu, double Qm, double xLb,
                double xUb, double *x);

void orc_dirichlet(const int *sites, int n, double gamma_bd, double xUb,
                   double *x0, double *gamma, int *full_H);

void orc_macro_results(int nH, const double *x, const int *HSurf, int nSurf,
                       double *xH, double *xHinterior);

int orc_minimize(const orc_params *p, double *X, const double *xH,
                 const int64_t *off, const uint32_t *nbr, const orc_lbfgs *lp,
                 int nthreads, double *fmin, int *iters, int *nfev,
                 double *gnorm, int *reason);

/* The seeded synthetic lattices of the benchmark configurations, written
 * independently of the library's generator so that CPU baselines need not
 * load the library: fcc cells of edge a visited z, y, x (slowest to
 * fastest), Pd basis (0,0,0) (0,1/2,1/2) (1/2,0,1/2) (1/2,1/2,0) then the
 * octahedral H basis (1/2,0,0) (0,1/2,0) (0,0,1/2) (1/2,1/2,1/2), all Pd
 * sites first; one std::mt19937_64(seed) stream drawn in this order: three
 * Box-Muller normals per site for the positions (pairs from u1 = 1 - U,
 * u2 = U with U = (draw >> 11) / 2^53, cosine first), then one uniform per
 * site for sigma when sigma_hi > sigma_lo, then one uniform per H site for
 * the occupancy jitter.  x_mode 0: x = x_center + x_half (2U - 1);
 * x_mode 1: a tanh nucleus profile about the box centre plus the jitter;
 * clamped to [xLb, xUb].  surface[h] = 1 for H sites of the z = 0 layer.
 * Returns 0, or -1 for invalid arguments. */
int orc_lattice_fcc(const int ncell[3], double a, double pos_std, double sigma_lo, double sigma_hi, int x_mode,
                    double x_center, double x_half, double x_matrix, double x_nucleus, double nucleus_radius,
                    double interface_width, double xLb, double xUb, uint64_t seed, double *X, double *xH,
                    int *surface);

#ifdef __cplusplus
}
#endif
#endif
