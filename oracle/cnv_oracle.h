/*
 * cnv_oracle.h -- CPU restatement of cnavier's explicit vorticity-streamfunction time step.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA path: only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it. The product
 * library (libcnv) never links, loads or calls it, and has no CPU fallback.
 *
 * What it restates (file:line in SorinBetisor/fluid-dynamics1):
 *   - the time-step body of src/main.c:283-395 (BCs, wall vorticity, derivatives, Euler,
 *     Poisson solve for psi with f = -w, velocity recovery, continuity diagnostic);
 *   - the 1-D finite-difference operators of src/finitediff.c:51-153 (Diff1) and
 *     src/finitediff.c:178-292 (Diff2), kept as 7-wide bands per row instead of dense
 *     n x n matrices. The reference applies them as dense Kronecker products
 *     (src/linearalg.c:353-371, src/linearalg.c:236-285); a banded sum over the same nonzero
 *     products in ascending column order, starting from 0.0, is bitwise identical for
 *     finite inputs, because every skipped product is +-0 and x + (+-0) == x;
 *   - euler() of src/fluiddyn.c:71-102 (expression order of src/fluiddyn.c:98);
 *   - poisson_SOR()/poisson_SOR_log() of src/poisson.c:111-173 / :224-285, both the
 *     red-black ordering (:239-261, the OPENMP_ENABLED build) and the lexicographic one
 *     (:264-270), and poisson()/poisson_log() (:62-109, :176-222, in-place Gauss-Seidel);
 *   - the stop norm error() of src/poisson.c:34-60;
 *   - maxel/minel of src/linearalg.c:475-545 for the continuity diagnostic.
 * Jacobi (ping-pong, interior only) follows src/cuda_kernels.cu:229-246, which the
 * reference never builds; it has no CPU counterpart in the reference.
 *
 * Layout: every field is n x n doubles, row-major, index i*n + j; i is the reference's first
 * index (the "y" direction, lid at i = n-1), j the second.
 */
#ifndef CNV_ORACLE_H
#define CNV_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_OK = 0,
    ORC_NOT_CONVERGED = 1,
    ORC_BAD_ARG = 3
};

/* Poisson solver kinds (config key poisson_type of src/main.c:349-361, plus Jacobi). */
enum {
    ORC_POISSON_GS = 1,      /* "no relaxation": Gauss-Seidel, src/poisson.c:62-109 */
    ORC_POISSON_SOR = 2,     /* successive over-relaxation, src/poisson.c:111-173 */
    ORC_POISSON_JACOBI = 3   /* true Jacobi, src/cuda_kernels.cu:229-246 */
};

/* Sweep orderings. */
enum {
    ORC_ORDER_LEX = 0,       /* i-outer, j-inner in-place sweep (sequential build) */
    ORC_ORDER_REDBLACK = 1   /* red (i+j even) pass then black pass (OPENMP_ENABLED build) */
};

typedef struct {
    int n;              /* grid points per side; the reference requires nx == ny */
    int order;          /* finite-difference order: 2, 4 or 6 */
    double dx, dy;      /* Lx/nx and Ly/ny (src/main.c:138-139) */
    double re, dt;
    double u_bc[4];     /* u1..u4 of include/config.h:27-30 */
    double v_bc[4];     /* v1..v4 */
    int poisson_type;   /* ORC_POISSON_* */
    int ordering;       /* ORC_ORDER_* (GS and SOR) */
    double beta;        /* SOR factor */
    int itmax;
    double tol;
    int threads;        /* OpenMP threads for the sweeps, 0 = runtime default */
    int exact_norm;     /* 1: single accumulator in row-major order with sqrt(pow(d,2)) exactly
                           as error() does sequentially; 0: per-row partial sums added in row
                           order (deterministic for any thread count) */
} orc_params;

typedef struct {
    int iters;          /* k of the converged sweep, as logged by src/poisson.c:275 */
    double err;         /* stop norm of that sweep */
    double cont_max;    /* maxel(continuity), src/main.c:407 */
    double cont_min;    /* minel(continuity), src/main.c:408 */
    int status;         /* ORC_OK or ORC_NOT_CONVERGED */
} orc_step_info;

/* Band coefficients of the 1-D operator: band[r*7 + (o+3)] multiplies column r+o.
 * deriv = 1 (Diff1) or 2 (Diff2); h = the grid spacing passed to Diff1/Diff2. */
int orc_fd_band(int n, int order, int deriv, double h, double *band);

/* d = A x along the second index (j, the reference's DX = kron(I, d)) or along the first
 * index (i, DY = kron(d, I)) using a band from orc_fd_band. */
void orc_apply_j(int n, const double *band, const double *x, double *d);
void orc_apply_i(int n, const double *band, const double *x, double *d);

/* Poisson solve for psi with Dirichlet psi = 0 on the edge; rhs f as passed to poisson*()
 * (the caller passes f = -w). psi is overwritten, starting from zero as the reference does. */
int orc_poisson(const orc_params *p, const double *f, double *psi, int *iters, double *err);

/* euler() of src/fluiddyn.c:71-102 over all n*n points, in place on w. */
void orc_euler(int n, double *w, const double *wx, const double *wy, const double *wxx,
               const double *wyy, const double *u, const double *v, double re, double dt);

/* Run nsteps time steps on the state (w, u, v, psi: n*n each, updated in place). info may
 * be NULL or hold nsteps entries. Returns ORC_OK, or ORC_NOT_CONVERGED after the step whose
 * Poisson solve hit itmax (the reference exits there). */
int orc_run(const orc_params *p, int nsteps, double *w, double *u, double *v, double *psi,
            orc_step_info *info);

/* Reference SOR factor of src/main.c:134. */
double orc_sor_beta(int nx, int ny);

/* One smoothing pass of the seeded initial-field rule used for the mixed-precision and
 * adjoint workloads: interior w <- (w[i-1][j] + w[i+1][j] + w[i][j-1] + w[i][j+1]) / 4,
 * edges kept (Jacobi averaging, out of place). */
void orc_smooth_pass(int n, const double *src, double *dst);

#ifdef __cplusplus
}
#endif
#endif
