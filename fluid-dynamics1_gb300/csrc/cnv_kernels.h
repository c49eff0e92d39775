// cnv_kernels.h -- launchers of libcnv's CUDA kernels (internal).
#pragma once

#include <cuda_runtime.h>

#include "cnv_internal.h"

namespace cnv {

// Buffers and scalars of one time step. Pointers are device pointers.
struct StepArgs {
    int n;
    int pitch;                 // split-layout row pitch in doubles
    const double* w_in;        // vorticity at step start (wall values written in place)
    double* w_wall;            // == w_in, writable view for the wall pass
    double* w_out;             // vorticity after the Euler update
    double* u;                 // velocities, row-major
    double* v;
    double* psi;               // streamfunction, row-major (output copy)
    double* sor[2];            // psi, red/black split layout
    double* rhs[2];            // Poisson right-hand side, split layout (null: not written)
    const FdBands* bands;      // device copy of the operator bands
    BoundaryValues bc;
    double inv_re;             // 1. / Re as src/fluiddyn.c:98 evaluates it
    double dt;
    double c4;                 // dx*dx*dy*dy (src/poisson.c:247 evaluates it left to right)
    int rhs_mode;              // 0: rhs = c4*f; 1: rhs = (c4*f) / den (FMA form);
                               // 2: rhs = (c4*f) * (1/dx^2), an exact power-of-two scaling (folded form)
    DivConst rhs_div;          // division by den (rhs_mode 1, den not a power of two)
    double rhs_rden;
    int rhs_den_pow2;
    double rhs_inv_h2;
    Ctrl* ctrl;
    double* cont_partials;     // 4 * cont_blocks doubles
    int cont_blocks;           // blocks of the post pass's cooperative launch (post_grid)
    long long timeout_ns;      // bound on the post pass's grid barrier
    int tile_rows;             // rows of the passes' 32-column tiles: 32, or 8 on small grids (step_tile_rows)
};

// Pre-solve pass: wall vorticity, derivatives, Euler update (w_in -> w_out, wall values into
// w_in) and the Poisson right-hand side (when rhs[0] is set).
cudaError_t launch_pre(const StepArgs& a, cudaStream_t s);
// Post-solve pass: u, v and row-major psi from the split-layout psi in sor[]; with continuity,
// also the continuity max/min and the step record (a cooperative launch of cont_blocks blocks).
cudaError_t launch_post(const StepArgs& a, bool continuity, cudaStream_t s);
// Rows of the passes' tiles for an n x n grid on `device`: 32, or 8 where 32-row tiles would give
// fewer blocks than twice the SM count.
int step_tile_rows(int n, int device);
// Blocks of the post pass's cooperative launch for an n x n grid on `device` (0 on failure).
int post_grid(int n, int device, int tile_rows);
// Copy a row-major field into the split layout and back (parity tests of the solver alone).
// to_split applies the same right-hand-side scaling as the transport pass (a.c4, a.rhs_mode).
cudaError_t launch_to_split(const double* f, double* r, double* b, const StepArgs& a, cudaStream_t s);
cudaError_t launch_from_split(const double* r, const double* b, double* f, int n, int pitch,
                              cudaStream_t s);
// Scan n*n doubles for NaN/Inf; *flag (device int) is set to 1 when one is found.
cudaError_t launch_nonfinite_scan(const double* x, long long count, int* flag, cudaStream_t s);

// Persistent Poisson solver (cooperative launch, one block per tile). sor/alt are the two
// split-layout copies of psi (the answer ends in sor), rhs the split-layout right-hand side,
// sync a buffer of poisson_sync_bytes() (zeroed by launch_poisson). grid = gx * gy blocks,
// all co-resident.
constexpr int kMaxSolverBlocks = 1024;
struct PoissonLaunch {
    PoissonParams p;
    double* sor[2];
    double* alt[2];
    const double* rhs[2];
    Ctrl* ctrl;
    void* sync;
    int grid, gx, gy;
};
cudaError_t launch_poisson(const PoissonLaunch& L, cudaStream_t s);
int poisson_threads();
size_t poisson_sync_bytes();
const void* poisson_kernel_ptr(Arith a, int kind, bool fold);
// Mixed-precision solve (cnv_mixed.cu): FP32 red-black SOR sweeps inside FP64 defect
// correction. Every array is in the red/black split layout (pitch doubles or floats per row):
// g = c4*f (input), psi = the FP64 iterate and the answer (zeroed by the caller for a zero
// start), rq / eg = FP32 work arrays (correction right-hand side; border-exchange copies by
// epoch parity). sync = mixed_sync_bytes() (zeroed by launch_mixed). gx*gy blocks, one per tile.
struct MixedLaunch {
    int n, pitch, gx, gy;
    double dx2, dy2, den, rden, beta, rtol;
    int max_outer, epochs;
    int rq_in_smem;   // keep the correction right-hand side tile in shared memory
    long long timeout_ns;
    const double* g[2];
    double* psi[2];
    float* rq[2];
    float* eg[2][2];  // [parity][colour]
    Ctrl* ctrl;
    void* sync;
};
cudaError_t launch_mixed(const MixedLaunch& L, cudaStream_t s);
size_t mixed_sync_bytes();
size_t mixed_smem_bytes(int n, int gx, int gy, bool rq_in_smem);
int mixed_threads();
int mixed_sweeps_per_exchange();

// Persistent red-black SOR / GS with 2 or 4 sweeps per border exchange (cnv_poisson_tb.cu):
// the same bits as launch_poisson, with each tile (plus a halo) in shared memory. out = the
// answer (split layout, zeroed edges), snap = tb_snapshot_doubles() of scratch, sync =
// tb_sync_bytes() (zeroed by the launch). One block of tb_threads() per tile, all co-resident.
struct TbLaunch {
    PoissonParams p;
    int sweeps;     // sweeps per exchange: 2 or 4 (halo 2 * sweeps)
    int gx, gy;
    int g_in_smem;  // keep the right-hand side tile in shared memory too
    double* out[2];
    const double* rhs[2];
    double* snap;
    Ctrl* ctrl;
    void* sync;
};
cudaError_t launch_poisson_tb(const TbLaunch& L, cudaStream_t s);
int tb_threads();
size_t tb_sync_bytes();
size_t tb_snapshot_doubles(int n, int pitch);
size_t tb_smem_bytes(int n, int gx, int gy, int sweeps, bool g_smem);
bool tb_tiles_ok(int n, int gx, int gy, int sweeps);

// Tile factorisation grid = gx * gy for an n x n grid (tiles near-square, at least 64 wide when
// possible).
void poisson_tiles(int n, int grid, int* gx, int* gy);
// Number of solver blocks for an n x n grid on a device with `sms` SMs that can hold `per_sm`
// blocks per SM.
int poisson_grid_for(int n, int sms, int per_sm);

}  // namespace cnv
