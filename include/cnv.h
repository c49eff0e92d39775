/*
 * cnv.h -- C ABI of libcnv, the GB300 (sm_103a) implementation of cnavier's explicit
 * vorticity-streamfunction time step (SorinBetisor/fluid-dynamics1).
 *
 * The library replaces the body of cnavier's time loop, src/main.c:283-395:
 *   velocity BCs (:283-296) -> wall vorticity (:298-320) -> vorticity derivatives and the
 *   Euler update (:323-344, src/fluiddyn.c:71-102) -> Poisson solve for psi with f = -w
 *   (:347-363, src/poisson.c) -> u = DY psi, v = -DX psi (:366-383) -> continuity
 *   diagnostic (:387-408).
 * All state stays on the GPU between steps. Every entry point returns a cnv_status and never
 * exits the process (the reference calls exit(1) on the failures listed below).
 *
 * Conventions: fields are n x n doubles, row-major (index i*n + j), i is the reference's first
 * index (the lid is row i = n-1), exactly the flattening of src/linearalg.c:373-408. Host
 * pointers are plain host memory; *_device entry points take device pointers. One state is
 * used by one host thread at a time; each state owns one CUDA stream.
 */
#ifndef CNV_H
#define CNV_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CNV_ABI_VERSION 1

typedef enum cnv_status {
    CNV_OK = 0,
    CNV_NOT_CONVERGED = 1, /* Poisson solve reached poisson_max_it; src/poisson.c:168-172 exits */
    CNV_NONFINITE = 2,     /* NaN or Inf in an input field or in the stop norm */
    CNV_BAD_ARG = 3,       /* invalid size, order, solver type or pointer */
    CNV_CUDA_ERROR = 4,    /* a CUDA runtime call failed; see cnv_last_error() */
    CNV_TIMEOUT = 5,       /* a bounded on-device wait gave up */
    CNV_NO_DEVICE = 6,     /* no usable sm_103 device */
    CNV_IO_ERROR = 7       /* config or output file could not be read or written */
} cnv_status;

/* Poisson solver selection (config key poisson_type, src/main.c:349-361). */
enum {
    CNV_POISSON_GS = 1,     /* "no relaxation" (src/poisson.c:62-109), run as red-black GS */
    CNV_POISSON_SOR = 2,    /* SOR (src/poisson.c:111-173), red-black ordering */
    CNV_POISSON_JACOBI = 3, /* true Jacobi sweeps (extension; src/cuda_kernels.cu:229-246) */
    CNV_POISSON_DIRECT = 4  /* extension: exact solve of the same discrete equation by FP64 sine
                               transforms (the answer SOR converges to, to rounding); iters and
                               err of the step records are 0; FP64 precisions only */
};

/* Arithmetic of the Poisson sweeps (extension key "precision"). */
enum {
    CNV_PREC_FP64 = 0,      /* FP64, the reference's operation order and rounding (default) */
    CNV_PREC_FP64_FMA = 1,  /* FP64, fused multiply-add form of the same update */
    CNV_PREC_MIXED = 2      /* FP32 sweeps inside FP64 defect correction */
};

/* Initial vorticity (extension key "init_field"). */
enum {
    CNV_INIT_REFERENCE = 0, /* w = psi = 0, interior u = ui, v = vi (src/main.c:178-221) */
    CNV_INIT_NOISE = 1      /* seeded Gaussian noise smoothed by Jacobi averaging passes */
};

/*
 * Configuration: the reference's Config (include/config.h:4-36), same names, types and
 * meaning, followed by optional extension keys whose defaults reproduce the reference.
 */
typedef struct cnv_config {
    /* --- include/config.h:4-36 --- */
    double Re;
    int Lx;
    int Ly;
    int nx;
    int ny;
    double dt;
    double tf;
    double max_co;
    int order;
    int poisson_max_it;
    double poisson_tol;
    int output_interval;
    int poisson_type;
    int openmp_enabled;  /* kept for file compatibility; the GPU always sweeps red-black */
    double ui, vi;
    double u1, u2, u3, u4;
    double v1, v2, v3, v4;
    /* --- extensions --- */
    double sor_omega;        /* SOR factor; <= 0 selects the reference formula, src/main.c:134 */
    int nsteps;              /* steps to run; <= 0 selects (int)(tf/dt - 1) + 1, src/main.c:162 */
    int precision;           /* CNV_PREC_* */
    double mixed_rtol;       /* CNV_PREC_MIXED: stop when ||f - A psi||_2 / ||f||_2 <= mixed_rtol
                                (relative residual of the FP64 iterate); <= 0 selects 1e-10 */
    int init_field;          /* CNV_INIT_* */
    unsigned long long seed; /* CNV_INIT_NOISE generator seed (splitmix64) */
    double init_sigma;       /* CNV_INIT_NOISE standard deviation */
    int init_smooth_passes;  /* CNV_INIT_NOISE Jacobi averaging passes */
    int device;              /* CUDA device ordinal */
    int solver_blocks;       /* Poisson solver blocks (tiles); <= 0 picks them from the grid size */
    int mixed_inner_sweeps;  /* CNV_PREC_MIXED: FP32 sweeps per correction; <= 0 picks n */
    int mixed_max_outer;     /* CNV_PREC_MIXED: correction limit (CNV_NOT_CONVERGED past it); <= 0: 100 */
    int sor_blocking;        /* FP64 SOR/GS kernel, by sweeps per border exchange: 0 auto, 1 exchange
                                every half-sweep, 2 or 4 sweeps per exchange on shared-memory tiles
                                (the same bits either way) */
    int mixed_warm_start;    /* CNV_PREC_MIXED (and batches): start each step's solve from the previous
                                step's psi instead of zero (same stop rule: FP64 relative residual) */
    int solver_timeout_ms;   /* bound on every on-device wait for another block; <= 0: 2000 */
    int test_stall_block;    /* testing only: 1 + the index of a block of the FP64 SOR/GS exchange
                                kernel that never raises its progress flags, so that its neighbours'
                                bounded waits run out (the solve returns CNV_TIMEOUT); 0: off */
    int test_guard_cells;    /* testing only: 1 puts 4 KB of 0xFF bytes (NaN in every lane width)
                                before and after every field and work buffer and checks them after
                                each step and Poisson call (CNV_CUDA_ERROR naming the buffer if a
                                kernel wrote there); 2 also changes one guard byte after u at
                                creation, so the first check must report it; 0: off. Batches
                                (cnv_batch_create's base) put a guard after every buffer of every
                                cavity in their arena and check after each cnv_batch_step; adjoint
                                handles check after each forward and backward run */
} cnv_config;

/* Per-step record: the values the reference logs (src/poisson.c:275, src/main.c:407-408). */
typedef struct cnv_step_info {
    int iters;        /* k of the sweep that met the tolerance (0-based), as logged */
    int status;       /* cnv_status of this step */
    double err;       /* stop norm of that sweep */
    double cont_max;  /* maxel(DX u + DY v) */
    double cont_min;  /* minel(DX u + DY v) */
} cnv_step_info;

typedef struct cnv_state cnv_state;

/* load_default_config(), src/config.c:47-87, plus extension defaults. */
int cnv_config_default(cnv_config *cfg);
/* load_config_from_file(), src/config.c:106-214: same key = value format, comments, trimming
 * and warnings; a missing file keeps the defaults and returns CNV_IO_ERROR (the reference
 * prints a message and continues with the defaults). */
int cnv_config_load(const char *path, cnv_config *cfg);
/* Apply one key/value pair as the parser would (returns CNV_BAD_ARG for an unknown key). */
int cnv_config_set(cnv_config *cfg, const char *key, const char *value);
/* Steps the reference would run: it_max + 1 with it_max = (int)(tf/dt - 1) (src/main.c:162),
 * or cfg->nsteps when positive. */
int cnv_config_steps(const cnv_config *cfg);

/* Create the device state for cfg (nx == ny required, as the reference's Kronecker operators
 * are; src/linearalg.c:367). The fields start as src/main.c:178-221 sets them (or as
 * init_field selects). */
int cnv_create(const cnv_config *cfg, cnv_state **out);
void cnv_destroy(cnv_state *s);
/* Back to the initial condition. */
int cnv_reset(cnv_state *s);
int cnv_grid_size(const cnv_state *s);

/* Copy fields in or out (n*n doubles each, row-major). NULL pointers are skipped.
 * cnv_set_fields returns CNV_NONFINITE (and changes nothing) if an input holds NaN or Inf. */
int cnv_set_fields(cnv_state *s, const double *w, const double *u, const double *v);
int cnv_get_fields(cnv_state *s, double *w, double *u, double *v, double *psi);
int cnv_set_fields_device(cnv_state *s, const double *w, const double *u, const double *v);
int cnv_get_fields_device(cnv_state *s, double *w, double *u, double *v, double *psi);

/* Advance nsteps time steps (src/main.c:283-395 each). info may be NULL or hold nsteps
 * records. Stops at the first step whose solve does not converge or goes non-finite and
 * returns that step's status. Synchronises the state's stream before returning. */
int cnv_step(cnv_state *s, int nsteps, cnv_step_info *info);
/* Same, but only enqueues the work on the state's stream; cnv_sync() waits and fills info. */
int cnv_step_async(cnv_state *s, int nsteps);
int cnv_sync(cnv_state *s, cnv_step_info *info, int ninfo);

/* Drop-in replacement of the whole loop body for a caller that keeps its fields in the
 * reference's row-pointer layout (mtrx.M, src/linearalg.c:53-82): uploads w, u, v, runs one
 * step and writes w, u, v and psi back, as src/main.c:283-395 leaves them. */
int cnv_step_rows(cnv_state *s, double **w, double **u, double **v, double **psi,
                  cnv_step_info *info);

/* Poisson solve alone, poisson_SOR() / poisson() semantics (src/poisson.c:111-173, :62-109):
 * psi = 0 start, Dirichlet psi = 0 on the edge, stop at sum |psi_k+1 - psi_k| < tol.
 * f and psi are host arrays of n*n doubles; uses the state's grid, spacing and solver
 * settings. iters/err may be NULL. */
int cnv_poisson(cnv_state *s, const double *f, double *psi, int *iters, double *err);
int cnv_poisson_device(cnv_state *s, const double *f, double *psi, int *iters, double *err);

/* Poisson solve that allocates no device memory. No counterpart in the reference: it exists
 * for callers that may not allocate GPU memory while they run, such as an application whose
 * memory pool owns the whole device, or a real-time loop that forbids cudaMalloc/cudaFree
 * (cudaFree synchronises the device and both calls take unbounded time).
 * Same solve as cnv_poisson_device (psi = 0 start, psi = 0 on the edge, stop at
 * sum |psi_k+1 - psi_k| < tol) on the CURRENT device, on stream (a cudaStream_t, NULL for the
 * default stream), which is synchronised before return. f and psi are device arrays of n*n
 * doubles, row-major; f is the right-hand side as poisson_SOR() takes it. poisson_type is
 * CNV_POISSON_GS, CNV_POISSON_SOR or CNV_POISSON_JACOBI; precision CNV_PREC_FP64 or
 * CNV_PREC_FP64_FMA; beta <= 0 selects the reference SOR factor for n. iters/err may be NULL.
 * Working arrays live in one fixed array in device memory (about 6.3 MB, held by every GPU
 * that has loaded it until the process exits), so n is limited to 512: larger n returns
 * CNV_BAD_ARG with a message on stderr. All calls on a device share that array: calls whose
 * GPU work overlaps (other streams or host threads at the same time) race and must be
 * serialised by the caller.
 * First call on a device: with CUDA's default lazy module loading (CUDA_MODULE_LOADING=LAZY)
 * the array and the solver's kernels are placed on a device when this entry point first runs
 * there, so that first call DOES take device memory (the 6.3 MB array plus the kernels' code).
 * Make one warm-up call on each device at start-up, before the caller's memory pool takes the
 * device and outside any stream capture; every later call allocates nothing. Setting
 * CUDA_MODULE_LOADING=EAGER in the environment places everything when the library loads.
 * Each call looks up the array's device address again (cudaGetSymbolAddress), so the entry
 * point keeps working after the caller resets the device's context (cudaDeviceReset); the
 * next call after such a reset is a first call again. */
int cnv_poisson_noalloc(const double *f, double *psi, int n, double dx, double dy,
                        int poisson_type, int precision, double beta, int itmax, double tol,
                        int *iters, double *err, void *stream);

/* ---------------------------------------------------------------------------------------
 * Batched form: many independent cavities (uneven grid size, Re and lid speed) advanced by one
 * persistent cooperative launch (captured in a CUDA graph). Each cavity runs the step of cnv_step
 * with the mixed-precision Poisson solve (FP32 red-black SOR inside FP64 defect correction to
 * relative residual base->mixed_rtol, default 1e-10). A cavity whose FP32 correction does not
 * fit one block's shared memory is split into row strips run by a group of blocks; the host
 * schedules the cavities (largest first) onto the blocks. No counterpart in the reference, which
 * runs one cavity per process.
 * ------------------------------------------------------------------------------------- */
typedef struct cnv_cavity_spec {
    int n;       /* grid points per side */
    double Re;   /* Reynolds number */
    double lid;  /* lid speed (u4) */
    double dt;   /* time step; <= 0 selects 0.2*min(h^2 Re/4, h/|lid|) */
} cnv_cavity_spec;

typedef struct cnv_batch cnv_batch;

/* count cavities drawn from a splitmix64 stream: n uniform over {64,96,128,192,256,384},
 * Re uniform in [100, 2000], lid uniform in [0.5, 1.5], dt by the stability rule. */
int cnv_batch_specs(int count, unsigned long long seed, cnv_cavity_spec *out);
/* Fields start as cnv_create's; base supplies order, Lx/Ly, the other wall velocities and the
 * mixed-form settings. Cavities whose FP32 correction does not fit one block's shared memory run
 * as row strips on a group of blocks, with the strip counts per cavity size that minimise a cost
 * model of the schedule's makespan (cnv_batch_split(b, 1, n) asks for the smallest counts). */
int cnv_batch_create(const cnv_config *base, int count, const cnv_cavity_spec *specs, cnv_batch **out);
void cnv_batch_destroy(cnv_batch *b);
int cnv_batch_reset(cnv_batch *b);
/* Time one step of each candidate decomposition (row strips only where shared memory needs
 * them, 2x / 4x as many for the largest cavities, or the strip counts per cavity size that a
 * cost model of the schedule picks) from the initial state, keep the fastest, and reset the
 * fields. Reports the launch shape (threads per block, blocks per SM); either
 * pointer may be NULL. */
int cnv_batch_tune(cnv_batch *b, int *threads, int *blocks_per_sm);
/* Use factor times more row strips than shared memory needs for cavities of at least min_n
 * points per side (factor 1: only as needed), rebuild the schedule and reset the fields. */
int cnv_batch_split(cnv_batch *b, int factor, int min_n);
/* Blocks (row strips) of each cavity under the current decomposition (count entries). */
int cnv_batch_groups(cnv_batch *b, int *groups);
/* Host only, no device needed: the row strips per cavity (groups, count entries) that
 * cnv_batch_create picks on a device that runs `blocks` batch blocks of `smem_bytes` bytes of
 * shared memory each (a GB300: 152 and 231424), and the schedule's estimated step time in
 * microseconds (makespan_us, may be NULL). */
int cnv_batch_plan(int count, const cnv_cavity_spec *specs, int blocks, int smem_bytes, int *groups,
                   double *makespan_us);
/* Advance every cavity nsteps steps in one launch; last (count records or NULL) receives each
 * cavity's last step. */
int cnv_batch_step(cnv_batch *b, int nsteps, cnv_step_info *last);
int cnv_batch_get_fields(cnv_batch *b, int index, double *w, double *u, double *v, double *psi);
/* Total cells, FP32 sweeps of the last call (all cavities) and its device time (ms). */
int cnv_batch_stats(cnv_batch *b, long long *cells, long long *sweeps, double *ms);

/* ---------------------------------------------------------------------------------------
 * Differentiable form: the discrete adjoint of the time step. A cnv_adjoint advances one
 * cavity with the step of cnv_step (the same wall, transport and velocity passes) and the
 * exact Poisson solve of CNV_POISSON_DIRECT, and returns the gradient of a scalar of the final
 * vorticity with respect to the initial vorticity and the lid speed (u4) by hand-written adjoint
 * kernels. The forward run keeps a checkpoint of the state every checkpoint_every steps; the
 * backward run recomputes one segment at a time from its checkpoint. The initial velocities
 * are cfg's ui, vi on the interior (src/main.c:213-221); cfg's poisson_* and precision fields
 * are not used. No counterpart in the reference.
 * ------------------------------------------------------------------------------------- */
typedef struct cnv_adjoint cnv_adjoint;

int cnv_adjoint_create(const cnv_config *cfg, int checkpoint_every, cnv_adjoint **out);
void cnv_adjoint_destroy(cnv_adjoint *a);
/* nsteps steps from the initial vorticity w0 (n*n, row-major) with lid speed lid; the final
 * vorticity goes to w_final (may be NULL). Keeps the checkpoints for cnv_adjoint_backward. */
int cnv_adjoint_forward(cnv_adjoint *a, const double *w0, double lid, int nsteps, double *w_final);
/* Given g_final = dJ/dw(T) (n*n) for the last forward run, writes dJ/dw0 (n*n; zero on the
 * edges, which the first wall pass overwrites) and dJ/dlid (may be NULL). */
int cnv_adjoint_backward(cnv_adjoint *a, const double *g_final, double *g_w0, double *g_lid);
/* The same two calls on device pointers (the handle's stream; both return after it is idle). */
int cnv_adjoint_forward_device(cnv_adjoint *a, const double *w0, double lid, int nsteps, double *w_final);
int cnv_adjoint_backward_device(cnv_adjoint *a, const double *g_final, double *g_w0, double *g_lid);
/* J = 1/2 sum over all cells of w(T)^2 dx dy (the final enstrophy) and its gradient. */
int cnv_adjoint_enstrophy_gradient(cnv_adjoint *a, const double *w0, double lid, int nsteps, double *J,
                                   double *g_w0, double *g_lid);
/* Device time (ms) of the last forward and backward runs, and bytes of checkpoint and segment
 * state held. Any pointer may be NULL. */
int cnv_adjoint_stats(cnv_adjoint *a, double *forward_ms, double *backward_ms, long long *state_bytes);

/* Statistics of the last cnv_step/cnv_poisson call: total Poisson sweeps, device time of the
 * whole call (ms, CUDA events on the state's stream) and device time of the Poisson kernel of
 * the last step or solve it ran (ms). Any pointer may be NULL. */
int cnv_last_stats(cnv_state *s, long long *sweeps, double *ms, double *poisson_ms);

/* Device time of the step's two passes around the Poisson solve, for measurement: the
 * pre-solve pass (wall vorticity, derivatives, Euler update, right-hand side) and the
 * post-solve pass (velocity, continuity) are each replayed reps times on the state's current
 * fields, and the mean ms per launch of each is returned (CUDA events on the state's stream).
 * Both passes are idempotent on the fields they read: afterwards the edge cells of w hold the
 * wall vorticity the next step's first pass gives them anyway, every other field is unchanged,
 * and the next cnv_step gives the same results as without this call. No counterpart in the
 * reference. */
int cnv_time_passes(cnv_state *s, int reps, double *pre_ms, double *post_ms);

/* One line naming the Poisson solver this state runs and its geometry, e.g.
 * "sor-exchange grid=152 tiles=8x19" (FP64 SOR/GS exchanging every half-sweep),
 * "sor-tiled sweeps=4 grid=150 tiles=5x30", "mixed grid=152 tiles=8x19" or
 * "direct-sine-transform". Returns CNV_BAD_ARG if it does not fit in len bytes. */
int cnv_solver_info(cnv_state *s, char *buf, size_t len);

/* ---------------------------------------------------------------------------------------
 * Pieces of the step for callers that keep the reference's loop: the Euler update of
 * src/fluiddyn.c:71-102 from caller-supplied derivative fields (count points, in place on w,
 * bit-identical to the reference), on host arrays (staged through per-thread device buffers)
 * or device arrays (enqueued on stream).
 * ------------------------------------------------------------------------------------- */
int cnv_euler(double *w, const double *dwdx, const double *dwdy, const double *d2wdx2, const double *d2wdy2,
              const double *u, const double *v, long long count, double Re, double dt);
int cnv_euler_device(double *w, const double *dwdx, const double *dwdy, const double *d2wdx2,
                     const double *d2wdy2, const double *u, const double *v, long long count, double Re,
                     double dt, void *stream);

/* ---------------------------------------------------------------------------------------
 * Run outputs in the reference's formats.
 * cnv_format_step_log: the lines the reference logs for time step t (src/poisson.c:275 and
 * src/main.c:401-414) from its step record: the Poisson line, then "Iteration: ... | Time: ...
 * | Progress: ... | Iter time: ..." and "Continuity max: ... | Continuity min: ... | Elapsed:
 * ... | Est. remaining: ..." (timings from the caller; it_max as src/main.c:162 computes it).
 * For a step that did not converge, the reference's error line alone. NUL-terminated into buf.
 * cnv_write_vtk: src/utils.c:38-99 -- "<output_dir>/<title>-1-<count>.vtk", ASCII
 * STRUCTURED_POINTS, "%.6lf" values, one line per row, appended; creates output_dir.
 * ------------------------------------------------------------------------------------- */
int cnv_format_step_log(const cnv_step_info *info, int t, double dt, int it_max, double iter_seconds,
                        double elapsed_seconds, char *buf, size_t len);
int cnv_write_vtk(const char *output_dir, const char *title, int count, const double *field, int m, int n);

/* The CNV_INIT_NOISE initial vorticity as a host array (n*n): sigma * N(0,1) per cell from a
 * splitmix64 stream seeded with seed, then `passes` Jacobi averaging passes over the interior. */
int cnv_noise_field(int n, unsigned long long seed, double sigma, int passes, double *out);

/* FP64 arithmetic throughput of a device, measured in place: lane-operations per second of
 * independent round-to-nearest multiply-then-add chains (the exact Poisson update's instruction
 * mix) and of fused multiply-adds (each FMA one operation). Either pointer may be NULL (not
 * both). Runs about 0.3 s of probe kernels on the device's default stream. */
int cnv_probe_fp64(int device, double *add_mul_ops_per_s, double *fma_ops_per_s);
/* out[i] = c * x[i] computed on the device exactly as the exact Poisson update multiplies by its
 * constants (integer arithmetic where it applies, the FP64 pipe otherwise): every result must
 * equal the correctly rounded IEEE product. Host arrays of count doubles. */
int cnv_check_mul_rn(int device, const double *x, int count, double c, double *out);
/* out[i] = x[i] / b computed on the device exactly as the exact Poisson update and the transport
 * pass divide by a constant that is not a power of two: every result must equal the correctly
 * rounded IEEE quotient. *fast (may be NULL) receives how many quotients the three-operation
 * path proved correctly rounded (the rest took the IEEE division). Host arrays of count doubles. */
int cnv_check_div_rn(int device, const double *x, int count, double b, double *out, long long *fast);

/* Human-readable text for the last failing call on this thread. */
const char *cnv_last_error(void);
/* Library version and the device it was built for. */
const char *cnv_version(void);

#ifdef __cplusplus
}
#endif
#endif /* CNV_H */
