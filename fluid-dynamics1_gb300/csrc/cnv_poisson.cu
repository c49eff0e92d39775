// cnv_poisson.cu -- persistent Poisson solver for the streamfunction (red-black SOR, red-black
// Gauss-Seidel, Jacobi), one cooperative launch per solve.
//
// Restates poisson_SOR() / poisson() of src/poisson.c (:111-173, :62-109) with the red-black
// ordering of the OPENMP_ENABLED build (:239-261), and a true Jacobi sweep
// (src/cuda_kernels.cu:229-246). psi starts at zero, keeps psi = 0 on the edge, and the solve
// stops at the first sweep k with  e_k = sum over all cells |psi_k+1 - psi_k| < tol
// (src/poisson.c:34-60, :272-278); the iterate of that sweep is the answer and k is reported.
//
// Decomposition. The interior is cut into GX x GY tiles, one block per tile and at most one
// block per SM, so every SM gets the same work. psi is kept in two copies ("sets") of
// the red/black split layout: sweep k reads set (k-1)&1 and writes set k&1, so the state of
// sweep k stays intact while sweep k+1 runs. A tile's interior cells depend only on the tile's
// own data; its frame (first/last row/column next to another tile) reads the neighbours'.
//
// Warp roles. Thirty-one warps update cells; the last (the signal warp) does all inter-block
// work: it polls the four neighbours' progress flags, raises this block's flag once the frame
// is written (fence + release store), adds the block's share of the stop norm to the global
// accumulator and runs the stop test. The two sides meet only at named barriers that the
// cell-update warps pass through without waiting for any fence or poll (bar.arrive where they
// hand something over, bar.sync only where they need the signal warp's answer, which it
// prepares ahead). In each half-sweep the first twelve warps wait for the neighbours' frames
// (barrier GO), update this colour's frame and hand it to the signal warp (PUB); every
// cell-update warp then takes 32-cell chunks of the interior from a shared counter, so the
// frame's latency is covered by the other warps' interior work and the FP64 pipe never idles
// on a block-wide barrier. There is no grid-wide barrier.
//
// Stop test. Each block adds its partial sum of |dpsi| to a fixed-point accumulator (units of
// 2^-80, kept as four 32-bit chunks in 64-bit counters: exact integer adds with no carry, so the
// total is independent of arrival order; cells with |psi| >= 2^46 go to an FP64 side sum) in a
// ring of 8 slots, and counts itself in. The
// signal warp checks e_{k-2} while the other warps finish sweep k-1 and posts the verdict at
// barrier DEC before sweep k; if e_{k-2} < tol every block stops before overwriting set
// (k-2)&1, which holds the answer. The extra sweep k-1 is discarded. Every wait of the signal
// warp is bounded by a timeout and by the abort flag, and records CNV_TIMEOUT instead of
// hanging; it then still passes every barrier, so the block always reaches its end.
//
// Arithmetic. Arith::kExact reproduces the reference's point update bit for bit: in general with
// the full operation sequence of src/poisson.c:247 (division by 2*(dx^2+dy^2) exact when that is
// a power of two, otherwise the correctly rounded division by a constant of cnv_sor.cuh); when dx = dy and dx^2 and 2*(dx^2+dy^2) are powers of
// two (every n = 2^k with L = 1), with the folded form
//     new = RN(RN(beta/4 * RN(RN(RN(up+dn) + RN(rt+lt)) - g')) + RN((1-beta)*old))
// with g' = c4*f / dx^2, which equals the reference's value whenever no intermediate
// (up+dn, rt+lt, their sum, sum - g') lies below 2^-960 in magnitude (then every power-of-two
// scaling is exact); cells that fail that test use the full sequence. 7 FP64 operations instead
// of 10 (c4*f comes precomputed from the transport pass in both). Arith::kFma uses the FMA form
// new = old + beta*(wy*(up+dn) + wx*(rt+lt) - q - old) with q = c4*f/den: 7 FP64 operations.
#include <algorithm>
#include <cfloat>

#include "cnv_kernels.h"
#include "cnv_sor.cuh"

namespace cnv {
namespace {

// One block of 1024 threads per SM. Against two blocks of 512 (15 cell warps and 4 frame warps
// each) it gave the same bits and 10.19 vs 12.14 us per sweep at 384^2, 8.66 vs 9.96 at 512^2,
// 20.50 vs 21.16 at 768^2, 17.08 vs 17.14 at 1024^2, 61.16 vs 60.63 at 1536^2 and 53.95 vs 56.24
// at 2048^2: no block shares its SM's FP64 pipe with another block's (in the two-block layout
// the second block on each SM ran its sweeps about 0.5 us slower, and the slowest blocks pace
// the grid), and the larger tiles have half the frame per cell. Eight frame warps gave 17.12 and
// 54.21, four 18.18 and 54.20 us at 1024^2 and 2048^2.
constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr int kCellWarps = kWarps - 1;          // warps 0..30 update cells
constexpr int kCellThreads = kCellWarps * 32;
constexpr int kSignalWarp = kWarps - 1;         // warp 31: flags, norm, stop test
constexpr int kFrameWarps = 12;                 // warps 0..11 also update the frame
constexpr int kFrameThreads = kFrameWarps * 32;
constexpr int kRing = 8;

// Named barriers (0 is __syncthreads). DEC: the stop verdict for the next sweep (signal warp
// arrives, cell warps wait). GO: the neighbours' frames are ready (signal warp arrives, frame
// warps wait). PUB: this block's frame is written (frame warps arrive, signal warp waits). END:
// the half-sweep is complete (cell warps only). NORM: the warps' norm partials are in shared
// memory (cell warps arrive, signal warp waits).
enum : int { kBarDec = 1, kBarGo = 2, kBarPub = 3, kBarEnd = 4, kBarNorm = 5 };
constexpr int kGoThreads = kFrameThreads + 32;

__device__ __forceinline__ void bar_sync(int id, int count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_arrive(int id, int count) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

struct Geometry {
    int n, pitch;
    int GX, GY;
};

// Per-launch synchronisation state (zeroed before every launch).
struct SyncState {
    // e_k * 2^80 as a 128-bit integer, accumulated in four 32-bit chunks of 64-bit counters so
    // that every contribution is a fire-and-forget add with no carry between words
    unsigned long long acc[kRing][4];
    unsigned int count[kRing];
    double fsum[kRing];         // FP64 part of e_k (cells with |psi| >= 2^46), usually 0
    unsigned int flag[2][kMaxSolverBlocks];  // [colour][block]: last sweep whose frame is written
};

// Block-shared state of the two warp roles.
struct Shared {
    unsigned long long part[2][kCellWarps][4];  // [sweep parity][warp] norm chunk sums
    double side[2];                             // [sweep parity] FP64 side sum of the norm
    unsigned int ctr[2];                        // interior chunk counters, by half-sweep parity
    int stop[2];                                // verdict before sweep k, at [k & 1]
    int status, conv_k;
    double e_last;
};

struct Tile {
    int r0, r1, c0, c1;  // tile rows [r0, r1), columns [c0, c1) (absolute indices)
    int ri0, ri1, ci0, ci1;  // interior region (no neighbour-tile dependency)
    int nb[4];  // neighbour blocks: up (r0-1), down, left, right; -1 if none
};

__device__ __forceinline__ Tile make_tile(const Geometry& g, int b) {
    Tile t;
    const int ni = g.n - 2;
    const int tx = b % g.GX, ty = b / g.GX;
    t.c0 = 1 + (int)((long long)ni * tx / g.GX);
    t.c1 = 1 + (int)((long long)ni * (tx + 1) / g.GX);
    t.r0 = 1 + (int)((long long)ni * ty / g.GY);
    t.r1 = 1 + (int)((long long)ni * (ty + 1) / g.GY);
    t.nb[0] = ty > 0 ? b - g.GX : -1;
    t.nb[1] = ty < g.GY - 1 ? b + g.GX : -1;
    t.nb[2] = tx > 0 ? b - 1 : -1;
    t.nb[3] = tx < g.GX - 1 ? b + 1 : -1;
    t.ri0 = t.r0 + (t.nb[0] >= 0);
    t.ri1 = t.r1 - (t.nb[1] >= 0);
    t.ci0 = t.c0 + (t.nb[2] >= 0);
    t.ci1 = t.c1 - (t.nb[3] >= 0);
    if (t.ri1 < t.ri0) t.ri1 = t.ri0;
    if (t.ci1 < t.ci0) t.ci1 = t.ci0;
    return t;
}

// Loads: interior cells read only this block's own data (written by this block, so L1 is
// coherent for them); frame cells read neighbour tiles, through L2 (ld.cg).
template <bool FRAME>
__device__ __forceinline__ double ld(const double* p) {
    if (FRAME) return __ldcg(p);
    return *p;
}

// Pointers of one sweep: colour c of the previous iterate (prev), of the new one (next), the
// other-colour array each colour's update reads (oth: for SOR/GS red reads black of the previous
// iterate and black reads red of the new one; Jacobi reads the previous iterate for both), and
// the right-hand side.
struct SweepPtrs {
    const double* prev[2];
    double* next[2];
    const double* oth[2];
    const double* rhs[2];
};

// Update one cell (i, j) of colour C.
template <Arith A, int KIND, bool FOLD, bool FRAME>
__device__ __forceinline__ void update_cell(const PoissonParams& p, int i, int j, const double* __restrict__ S_prev,
                                            double* __restrict__ S_new, const double* __restrict__ O,
                                            const double* __restrict__ rhs, NormAcc& acc, double* side) {
    const size_t row = (size_t)i * p.pitch;
    const int m = j >> 1;
    const double old = ld<FRAME>(S_prev + row + m);
    const double up = ld<FRAME>(O + row + p.pitch + m);
    const double dn = ld<FRAME>(O + row - p.pitch + m);
    const double lt = ld<FRAME>(O + row + ((j - 1) >> 1));
    const double rt = ld<FRAME>(O + row + ((j + 1) >> 1));
    S_new[row + m] = point_update<A, KIND, FOLD>(p, up, dn, rt, lt, __ldg(rhs + row + m), old, acc, side);
}

// x / d for 0 <= x < 2^31 and 1 <= d, with m = 0xffffffff / d: the multiply-high estimate is
// x/d or one less, and one correction step makes it exact.
__device__ __forceinline__ int div_magic(int x, int d, unsigned m) {
    int q = (int)__umulhi((unsigned)x, m);
    if (x - q * d >= d) ++q;
    return q;
}

// Interior cells of colour C (C = 2: both colours, Jacobi), in chunks taken from the block's
// counter *ctr by whole warps until none is left. For one colour a chunk is 64 cells, two per
// lane (x and x + 32, consecutive in a row: coalesced), loaded and updated together so that each
// warp keeps two independent FP64 chains in flight; lanes past the region's end recompute the
// region's first cell and store nothing.
template <Arith A, int KIND, bool FOLD, int C>
__device__ __forceinline__ void interior_chunks(const PoissonParams& p, const Tile& t, const SweepPtrs& q,
                                                NormAcc& acc, unsigned* ctr, double* side) {
    const int w = t.ci1 - t.ci0;
    const int h = t.ri1 - t.ri0;
    if (w <= 0 || h <= 0) return;
    const int wq = (w + 1) >> 1;
    const unsigned mq = 0xffffffffu / (unsigned)wq;
    const int per_colour = h * wq;
    const int lane = threadIdx.x & 31;
    if (C == 2) {
        const int total = 2 * per_colour;
        const unsigned nchunks = (unsigned)((total + 31) >> 5);
        for (;;) {
            unsigned c = 0;
            if (lane == 0) c = atomicAdd(ctr, 1u);
            c = __shfl_sync(0xffffffffu, c, 0);
            if (c >= nchunks) break;
            const int x = (int)c * 32 + lane;
            if (x < total) {
                const int cc = x >= per_colour;
                const int xx = cc ? x - per_colour : x;
                const int r = div_magic(xx, wq, mq);
                const int i = t.ri0 + r;
                const int j = t.ci0 + 2 * (xx - r * wq) + ((i + t.ci0 + cc) & 1);
                if (j < t.ci1) {
                    if (cc)
                        update_cell<A, KIND, FOLD, false>(p, i, j, q.prev[1], q.next[1], q.oth[1], q.rhs[1], acc,
                                                          side);
                    else
                        update_cell<A, KIND, FOLD, false>(p, i, j, q.prev[0], q.next[0], q.oth[0], q.rhs[0], acc,
                                                          side);
                }
            }
        }
        return;
    }
    const double* __restrict__ Sp = q.prev[C];
    double* __restrict__ Sn = q.next[C];
    const double* __restrict__ O = q.oth[C];
    const double* __restrict__ G = q.rhs[C];
    const int pitch = p.pitch;
    if (FOLD && wq >= 48) {
        // Row-aligned chunks: chunk c is cells [64 b, 64 b + 64) of row r (b = c % per_row) of
        // this colour, so the row, its parity and the neighbour offsets are the same for the whole
        // chunk and a cell's address is the row's base plus its index (no division per cell).
        // Taken where a row holds at least 48 cells of a colour, so that few lanes idle (1024^2:
        // 16.73 vs 16.84 us per sweep, 2048^2: 52.5 vs 53.2, the same bits); the general form keeps
        // the flat chunks, with which its kernel ran faster.
        const int per_row = (wq + 63) >> 6;
        const unsigned nrc = (unsigned)(h * per_row);
        for (;;) {
            unsigned c = 0;
            if (lane == 0) c = atomicAdd(ctr, 1u);
            c = __shfl_sync(0xffffffffu, c, 0);
            if (c >= nrc) break;
            const int r = (int)c / per_row;
            const int b = (int)c - r * per_row;
            const int i = t.ri0 + r;
            const int j0 = t.ci0 + ((i + t.ci0 + C) & 1);  // the row's first cell of colour C
            const int jl = ((j0 - 1) >> 1) - (j0 >> 1);     // -1 or 0: the left neighbour's offset
            const int jr = ((j0 + 1) >> 1) - (j0 >> 1);     // 0 or +1
            const size_t base = (size_t)i * pitch + (j0 >> 1);
            size_t at[2];
            bool ok[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int tt = b * 64 + u * 32 + lane;  // cell j0 + 2 tt of the row
                ok[u] = tt < wq && j0 + 2 * tt < t.ci1;
                at[u] = base + (ok[u] ? tt : 0);
            }
            double old[2], up[2], dn[2], lt[2], rt[2], g[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                old[u] = Sp[at[u]];
                up[u] = O[at[u] + pitch];
                dn[u] = O[at[u] - pitch];
                lt[u] = O[at[u] + jl];
                rt[u] = O[at[u] + jr];
                g[u] = __ldg(G + at[u]);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const double nw = point_value<A, KIND, FOLD>(p, up[u], dn[u], rt[u], lt[u], g[u], old[u]);
                if (ok[u]) {
                    Sn[at[u]] = nw;
                    if (!norm_add(acc, nw, old[u])) norm_side_add(side, nw, old[u]);
                }
            }
        }
        return;
    }
    const unsigned nchunks = (unsigned)((per_colour + 63) >> 6);
    for (;;) {
        unsigned c = 0;
        if (lane == 0) c = atomicAdd(ctr, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= nchunks) break;
        size_t at[2];
        int jl[2], jr[2];
        bool ok[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int x = (int)c * 64 + u * 32 + lane;
            const int xx = x < per_colour ? x : 0;
            const int r = div_magic(xx, wq, mq);
            const int i = t.ri0 + r;
            const int j = t.ci0 + 2 * (xx - r * wq) + ((i + t.ci0 + C) & 1);
            ok[u] = x < per_colour && j < t.ci1;
            const int jj = ok[u] ? j : t.ci0;
            const int ii = ok[u] ? i : t.ri0;
            at[u] = (size_t)ii * pitch + (jj >> 1);
            jl[u] = ((jj - 1) >> 1) - (jj >> 1);  // -1 or 0: the left neighbour's offset
            jr[u] = ((jj + 1) >> 1) - (jj >> 1);  // 0 or +1
        }
        double old[2], up[2], dn[2], lt[2], rt[2], g[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            old[u] = Sp[at[u]];
            up[u] = O[at[u] + pitch];
            dn[u] = O[at[u] - pitch];
            lt[u] = O[at[u] + jl[u]];
            rt[u] = O[at[u] + jr[u]];
            g[u] = __ldg(G + at[u]);
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const double nw = point_value<A, KIND, FOLD>(p, up[u], dn[u], rt[u], lt[u], g[u], old[u]);
            if (ok[u]) {
                Sn[at[u]] = nw;
                if (!norm_add(acc, nw, old[u])) norm_side_add(side, nw, old[u]);
            }
        }
    }
}

// Frame cells of colour C (C = 2: both colours): tile cells outside the interior region, shared
// out over the kFrameThreads threads of the frame warps.
template <Arith A, int KIND, bool FOLD, int C>
__device__ __forceinline__ void frame_pass(const PoissonParams& p, const Tile& t, const SweepPtrs& q,
                                           NormAcc& acc, double* side) {
    const int W = t.c1 - t.c0;
    const int top = t.ri0 - t.r0, bot = t.r1 - t.ri1;
    const int left = t.ci0 - t.c0, right = t.c1 - t.ci1;
    const int mid = t.ri1 - t.ri0;
    const int n_rows = (top + bot) * W;
    const int total = n_rows + mid * (left + right);
    for (int x = threadIdx.x; x < total; x += kFrameThreads) {
        int i, j;
        if (x < n_rows) {
            const int rr = x / W;
            i = rr < top ? t.r0 + rr : t.ri1 + (rr - top);
            j = t.c0 + (x - rr * W);
        } else {
            const int x2 = x - n_rows;
            const int lr = left + right;
            const int rr = x2 / lr;
            const int side = x2 - rr * lr;
            i = t.ri0 + rr;
            j = side < left ? t.c0 : t.c1 - 1;
        }
        const int cc = (i + j) & 1;
        if (C != 2) {
            if (cc != C) continue;
            update_cell<A, KIND, FOLD, true>(p, i, j, q.prev[C], q.next[C], q.oth[C], q.rhs[C], acc, side);
        } else if (cc) {
            update_cell<A, KIND, FOLD, true>(p, i, j, q.prev[1], q.next[1], q.oth[1], q.rhs[1], acc, side);
        } else {
            update_cell<A, KIND, FOLD, true>(p, i, j, q.prev[0], q.next[0], q.oth[0], q.rhs[0], acc, side);
        }
    }
}

// Signal warp, lane 0: adds this block's share of e_k (the cell warps' chunk sums of sweep k,
// in sh.part[k & 1], and the FP64 side sum sh.side[k & 1], which it clears for sweep k + 2) to
// ring slot k % kRing and counts the block in.
__device__ __forceinline__ void contribute(SyncState* sy, int k, Shared& sh) {
    unsigned long long s[4] = {0, 0, 0, 0};
    for (int w = 0; w < kCellWarps; ++w) {
#pragma unroll
        for (int c = 0; c < 4; ++c) s[c] += sh.part[k & 1][w][c];
    }
    const int slot = k % kRing;
    const double fs = sh.side[k & 1];
    sh.side[k & 1] = 0.0;
    if (fs != 0.0 || fs != fs) atomicAdd(&sy->fsum[slot], fs);  // only where a cell reached 2^46
#pragma unroll
    for (int c = 0; c < 4; ++c) atomicAdd(&sy->acc[slot][c], s[c]);
    __threadfence();
    atomicAdd(&sy->count[slot], 1u);
}

// Signal warp, lane 0: waits until every block has added e_j and evaluates the stop test.
// Returns 0 run on, 1 e_j < tol, 2 wait given up, 3 non-finite; e_j in *e.
__device__ int check_norm(SyncState* sy, int j, const PoissonParams& p, Ctrl* ctl, double* e) {
    const int slot = j % kRing;
    if (!wait_geq(&sy->count[slot], (unsigned)gridDim.x, ctl, p.timeout_ns)) return 2;
    unsigned long long c[4];
#pragma unroll
    for (int w = 0; w < 4; ++w) c[w] = __ldcg(&sy->acc[slot][w]);
    *e = __dadd_rn(norm_total(c), __ldcg(&sy->fsum[slot]));
    if (!isfinite(*e)) return 3;
    return *e < p.tol ? 1 : 0;
}

// The signal warp's whole run: per sweep one DEC arrival, one NORM wait (the previous sweep's
// partials) and per half-sweep one GO arrival and one PUB wait; it ends with the verdict in
// sh.status, sh.conv_k, sh.e_last. Every barrier instance is complete before the next instance
// of the same barrier can be entered: each next arrival of the signal warp follows a PUB wait
// that needs the frame warps past the previous instance, and each next arrival of the cell
// warps follows a GO or END that needs the signal warp past it.
template <int KIND>
__device__ void signal_warp(const PoissonParams& p, const Tile& t, SyncState* sy, Ctrl* ctl, Shared& sh) {
    const int lane = threadIdx.x & 31;
    const int me = blockIdx.x;
    const int kmax = p.itmax;
    constexpr int kHalves = KIND == CNV_POISSON_JACOBI ? 1 : 2;
    int status = CNV_NOT_CONVERGED, conv_k = -1;
    double e_last = 0.0;
    bool gave_up = false;
    bool stopped = false;
    for (int k = 1; k <= kmax; ++k) {
        // verdict before sweep k: e_{k-2} (its shares were added during sweep k-1)
        int v = gave_up ? 2 : 0;
        if (lane == 0 && !gave_up && k >= 3) {
            double e = 0.0;
            v = check_norm(sy, k - 2, p, ctl, &e);
            if (v != 2) e_last = e;
            if (v == 0 && me == 0 && k >= 5) {
                // everyone has read e_{k-4} (they all added e_{k-2}); reuse its slot
                const int slot = (k - 4) % kRing;
#pragma unroll
                for (int w = 0; w < 4; ++w) sy->acc[slot][w] = 0;
                sy->fsum[slot] = 0.0;
                __threadfence();
                atomicExch(&sy->count[slot], 0u);
            }
        }
        v = __shfl_sync(0xffffffffu, v, 0);
        if (lane == 0) sh.stop[k & 1] = v;
        __syncwarp();
        bar_arrive(kBarDec, kThreads);
        if (v) {
            if (v == 1) { status = CNV_OK; conv_k = k - 2; }
            else if (v == 2) status = CNV_TIMEOUT;
            else status = CNV_NONFINITE;
            if (k >= 2) bar_sync(kBarNorm, kThreads);  // sweep k-1's partials, left unused
            stopped = true;
            break;
        }
#pragma unroll
        for (int h = 0; h < kHalves; ++h) {
            // red (and Jacobi) needs the neighbours' black frames of sweep k-1; black their red of k
            const unsigned* fl = h == 0 ? sy->flag[1] : sy->flag[0];
            const unsigned want = h == 0 ? (unsigned)(k - 1) : (unsigned)k;
            bool ok = true;
            if (lane < 4 && !gave_up) {
                const int nb = t.nb[lane];
                if (nb >= 0) ok = wait_geq(fl + nb, want, ctl, p.timeout_ns);
            }
            if (!__all_sync(0xffffffffu, ok)) gave_up = true;
            // Sweep k-1's norm partials. Taken before this sweep's first GO: the cell warps
            // cannot reach sweep k's NORM before every frame warp has passed that GO, so the
            // two NORM instances never overlap (with one half-sweep per sweep, Jacobi, there
            // is no later GO to order them).
            if (h == 0 && k >= 2) bar_sync(kBarNorm, kThreads);
            bar_arrive(kBarGo, kGoThreads);
            bar_sync(kBarPub, kGoThreads);
            if (lane == 0 && me != p.stall_block) {  // a stalled block (tests only) never publishes
                __threadfence();
                st_release(&sy->flag[KIND == CNV_POISSON_JACOBI ? 1 : h][me], (unsigned)k);
            }
            __syncwarp();
            // sh.part[(k-1) & 1] is next written at the end of sweep k+1, after sweep k+1's GO
            if (h == 0 && k >= 2) {
                if (lane == 0) contribute(sy, k - 1, sh);
                __syncwarp();
            }
        }
    }
    if (!stopped && kmax >= 1) {
        // the last sweep's share, then the tests of sweeps kmax-1 and kmax (not checked yet)
        bar_sync(kBarNorm, kThreads);
        if (gave_up) {
            status = CNV_TIMEOUT;
        } else if (lane == 0) {
            contribute(sy, kmax, sh);
            for (int j = (kmax >= 2 ? kmax - 1 : 1); j <= kmax; ++j) {
                double e = 0.0;
                const int v = check_norm(sy, j, p, ctl, &e);
                if (v != 2) e_last = e;
                if (v == 1) { conv_k = j; status = CNV_OK; break; }
                if (v == 2) { status = CNV_TIMEOUT; break; }
                if (v == 3) { status = CNV_NONFINITE; break; }
            }
        }
    }
    if (lane == 0) {
        sh.status = status;
        sh.conv_k = conv_k;
        sh.e_last = e_last;
    }
}

// The cell warps' whole run: the mirror image of signal_warp's barrier sequence.
template <Arith A, int KIND, bool FOLD>
__device__ void cell_warps(const PoissonLaunch& L, const Tile& t, Shared& sh) {
    const PoissonParams& p = L.p;
    const int warp = threadIdx.x >> 5;
    const bool frame_warp = warp < kFrameWarps;
    // two copies of psi: set 0 = L.sor (the caller's output), set 1 = L.alt
    double* const s0r = L.sor[0];
    double* const s0b = L.sor[1];
    double* const s1r = L.alt[0];
    double* const s1b = L.alt[1];
    int half = 0;
    for (int k = 1; k <= p.itmax; ++k) {
        bar_sync(kBarDec, kThreads);
        if (sh.stop[k & 1]) break;
        // sweep k reads set (k-1)&1 and writes set k&1
        const bool odd = k & 1;
        SweepPtrs q;
        q.prev[0] = odd ? s0r : s1r;
        q.prev[1] = odd ? s0b : s1b;
        q.next[0] = odd ? s1r : s0r;
        q.next[1] = odd ? s1b : s0b;
        q.rhs[0] = L.rhs[0];
        q.rhs[1] = L.rhs[1];
        NormAcc acc{{0, 0, 0, 0}};
        double* const side = &sh.side[k & 1];
        if (KIND == CNV_POISSON_JACOBI) {
            q.oth[0] = q.prev[1];
            q.oth[1] = q.prev[0];
            if (frame_warp) {
                bar_sync(kBarGo, kGoThreads);
                frame_pass<A, KIND, FOLD, 2>(p, t, q, acc, side);
                __syncwarp();
                bar_arrive(kBarPub, kGoThreads);
            }
            interior_chunks<A, KIND, FOLD, 2>(p, t, q, acc, &sh.ctr[half & 1], side);
            bar_sync(kBarEnd, kCellThreads);
            if (threadIdx.x == 0) sh.ctr[half & 1] = 0;
            ++half;
        } else {
            // red: black neighbours of sweep k-1, own red of sweep k-1
            q.oth[0] = q.prev[1];
            q.oth[1] = q.next[0];  // black: red of sweep k (new), own black of sweep k-1
            if (frame_warp) {
                bar_sync(kBarGo, kGoThreads);
                frame_pass<A, KIND, FOLD, 0>(p, t, q, acc, side);
                __syncwarp();
                bar_arrive(kBarPub, kGoThreads);
            }
            interior_chunks<A, KIND, FOLD, 0>(p, t, q, acc, &sh.ctr[half & 1], side);
            bar_sync(kBarEnd, kCellThreads);
            if (threadIdx.x == 0) sh.ctr[half & 1] = 0;
            ++half;
            if (frame_warp) {
                bar_sync(kBarGo, kGoThreads);
                frame_pass<A, KIND, FOLD, 1>(p, t, q, acc, side);
                __syncwarp();
                bar_arrive(kBarPub, kGoThreads);
            }
            interior_chunks<A, KIND, FOLD, 1>(p, t, q, acc, &sh.ctr[half & 1], side);
            bar_sync(kBarEnd, kCellThreads);
            if (threadIdx.x == 0) sh.ctr[half & 1] = 0;
            ++half;
        }
        // this warp's share of e_k: integer chunk sums (exact, order-free), handed to the
        // signal warp, which adds the block's total during the next sweep
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            unsigned long long x = acc.c[w];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
            acc.c[w] = x;
        }
        if ((threadIdx.x & 31) == 0) {
#pragma unroll
            for (int w = 0; w < 4; ++w) sh.part[k & 1][warp][w] = acc.c[w];
        }
        __syncwarp();
        bar_arrive(kBarNorm, kThreads);
    }
}

template <Arith A, int KIND, bool FOLD>
__global__ void __launch_bounds__(kThreads, 1) k_poisson(PoissonLaunch L) {
    Ctrl* ctl = L.ctrl;
    const PoissonParams& p = L.p;
    SyncState* sy = reinterpret_cast<SyncState*>(L.sync);
    const Geometry geo{p.n, p.pitch, L.gx, L.gy};
    const Tile t = make_tile(geo, blockIdx.x);
    __shared__ Shared sh;
    __shared__ int s_abort;
    if (threadIdx.x < 2) {
        sh.ctr[threadIdx.x] = 0;
        sh.stop[threadIdx.x] = 0;
        sh.side[threadIdx.x] = 0.0;
    }
    if (threadIdx.x == 0) s_abort = ld_volatile_int(&ctl->abort);
    __syncthreads();
    if (s_abort) return;  // one read for the whole block: the warp roles must all run or none

    if ((threadIdx.x >> 5) == kSignalWarp)
        signal_warp<KIND>(p, t, sy, ctl, sh);
    else
        cell_warps<A, KIND, FOLD>(L, t, sh);
    __syncthreads();

    const int status = sh.status;
    const int conv_k = sh.conv_k;
    if (status == CNV_TIMEOUT) return;
    // the answer is the iterate of sweep conv_k (or of the last sweep): copy it into set 0
    const int ans = conv_k > 0 ? conv_k : p.itmax;
    if (ans & 1) {
        double* const s0r = L.sor[0];
        double* const s0b = L.sor[1];
        const double* const s1r = L.alt[0];
        const double* const s1b = L.alt[1];
        const int h = t.r1 - t.r0, w = t.c1 - t.c0;
        for (int x = threadIdx.x; x < h * w; x += kThreads) {
            const int i = t.r0 + x / w, j = t.c0 + x % w;
            const size_t idx = (size_t)i * p.pitch + (j >> 1);
            if ((i + j) & 1) s0b[idx] = s1b[idx];
            else s0r[idx] = s1r[idx];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const double e_last = sh.e_last;
        const int iters = status == CNV_OK ? conv_k - 1 : p.itmax;
        ctl->iters = iters;
        ctl->err = e_last;
        ctl->status = status;
        ctl->sweeps += (status == CNV_OK ? conv_k : p.itmax);
        const int step = ctl->step;
        if (step < ctl->max_records) {
            StepRecord& r = ctl->records[step];
            r.iters = iters;
            r.status = status;
            r.err = e_last;
            r.cont_max = 0.0;
            r.cont_min = 0.0;
        }
        if (status != CNV_OK) ctl->abort = 1;
    }
}

template <Arith A, int KIND, bool FOLD>
const void* kernel_ptr() {
    return reinterpret_cast<const void*>(&k_poisson<A, KIND, FOLD>);
}

}  // namespace

int poisson_threads() { return kThreads; }
size_t poisson_sync_bytes() { return sizeof(SyncState); }

const void* poisson_kernel_ptr(Arith a, int kind, bool fold) {
    if (a == Arith::kExact) {
        if (fold) {
            if (kind == CNV_POISSON_SOR) return kernel_ptr<Arith::kExact, CNV_POISSON_SOR, true>();
            if (kind == CNV_POISSON_GS) return kernel_ptr<Arith::kExact, CNV_POISSON_GS, true>();
            return kernel_ptr<Arith::kExact, CNV_POISSON_JACOBI, true>();
        }
        if (kind == CNV_POISSON_SOR) return kernel_ptr<Arith::kExact, CNV_POISSON_SOR, false>();
        if (kind == CNV_POISSON_GS) return kernel_ptr<Arith::kExact, CNV_POISSON_GS, false>();
        return kernel_ptr<Arith::kExact, CNV_POISSON_JACOBI, false>();
    }
    if (kind == CNV_POISSON_SOR) return kernel_ptr<Arith::kFma, CNV_POISSON_SOR, false>();
    if (kind == CNV_POISSON_GS) return kernel_ptr<Arith::kFma, CNV_POISSON_GS, false>();
    return kernel_ptr<Arith::kFma, CNV_POISSON_JACOBI, false>();
}

void poisson_tiles(int n, int grid, int* gx, int* gy) {
    // factor grid = GX * GY so that tiles are as close to square as possible, preferring wide ones
    const int ni = n - 2;
    int best_gx = grid, best_gy = 1;
    double best = 1e300;
    for (int a = 1; a <= grid; ++a) {
        if (grid % a) continue;
        const int b = grid / a;  // GX = a columns of tiles, GY = b rows of tiles
        if (a > ni || b > ni) continue;
        const double tw = (double)ni / a, th = (double)ni / b;
        const double cost = 2 * (tw + th) + (tw < 64 ? 64 - tw : 0) * 4;  // frame size, narrow penalty
        if (cost < best) {
            best = cost;
            best_gx = a;
            best_gy = b;
        }
    }
    *gx = best_gx;
    *gy = best_gy;
}

int poisson_grid_for(int n, int sms, int per_sm) {
    // One block per SM from about 700 interior cells per block; below that one block per about
    // 700 cells, picking among the nearby counts the one whose tiles have the smallest frames (a
    // prime count would only tile as strips).
    const long long cells = (long long)(n - 2) * (n - 2);
    const int cap = std::min(std::min(per_sm, 1) * sms, kMaxSolverBlocks);
    if (cells >= 700LL * sms) return std::min(sms, cap);
    const int want = (int)std::max(1LL, std::min<long long>(cells / 700, cap));
    const double ni = n - 2;
    int best = want;
    double best_score = 1e300;
    for (int g = std::max(1, want - want / 4); g <= want; ++g) {
        int gx = 1, gy = 1;
        poisson_tiles(n, g, &gx, &gy);
        const double score = (double)cells / g + 3.0 * (ni / gx + ni / gy);  // cells + frame per block
        if (score < best_score) {
            best_score = score;
            best = g;
        }
    }
    return best;
}

cudaError_t launch_poisson(const PoissonLaunch& L, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(L.sync, 0, sizeof(SyncState), s);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L.grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {const_cast<PoissonLaunch*>(&L)};
    return cudaLaunchKernelExC(&cfg, poisson_kernel_ptr(L.p.arith, L.p.kind, L.p.fold != 0), args);
}

}  // namespace cnv
