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
// block per SM (or two), so every SM gets the same work. psi is kept in two copies ("sets") of
// the red/black split layout: sweep k reads set (k-1)&1 and writes set k&1, so the state of
// sweep k stays intact while sweep k+1 runs. A tile's interior cells depend only on the tile's
// own data; its frame (first/last row/column next to another tile) reads the neighbours'. Each
// half-sweep waits for the four neighbours' progress flags (one thread per neighbour, in
// parallel), updates the frame, publishes its own flag at once, and then updates the interior
// while the neighbours catch up. There is no grid-wide barrier.
//
// Stop test. Each block adds its partial sum of |dpsi| to a 128-bit fixed-point accumulator
// (scale 2^80, kept as four 32-bit chunks in 64-bit counters: exact integer adds with no carry,
// so the total is independent of arrival order) in a ring of 8 slots, and counts itself in. A block checks e_{k-2} at the start of sweep k, when it is
// long complete; if e_{k-2} < tol every block stops before overwriting set (k-2)&1, which holds
// the answer. The extra sweep k-1 is discarded. Every wait is bounded by a timeout and by the
// abort flag, and records CNV_TIMEOUT instead of hanging.
//
// Arithmetic. Arith::kExact reproduces the reference's point update bit for bit: in general with
// the full operation sequence of src/poisson.c:247 (division by 2*(dx^2+dy^2) exact when that is
// a power of two, IEEE division otherwise); when dx = dy and dx^2 and 2*(dx^2+dy^2) are powers of
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

constexpr int kThreads = 512;
constexpr int kRing = 8;

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
    unsigned int nonfinite[kRing];
    unsigned int flag[2][kMaxSolverBlocks];  // [colour][block]: last sweep whose frame is written
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
                                            const double* __restrict__ rhs, NormAcc& acc) {
    const size_t row = (size_t)i * p.pitch;
    const int m = j >> 1;
    const double old = ld<FRAME>(S_prev + row + m);
    const double up = ld<FRAME>(O + row + p.pitch + m);
    const double dn = ld<FRAME>(O + row - p.pitch + m);
    const double lt = ld<FRAME>(O + row + ((j - 1) >> 1));
    const double rt = ld<FRAME>(O + row + ((j + 1) >> 1));
    S_new[row + m] = point_update<A, KIND, FOLD>(p, up, dn, rt, lt, __ldg(rhs + row + m), old, acc);
}

// Interior cells of colour C (C = 2: both colours, Jacobi).
template <Arith A, int KIND, bool FOLD, int C>
__device__ __forceinline__ void interior_pass(const PoissonParams& p, const Tile& t, const SweepPtrs& q,
                                              NormAcc& acc) {
    const int w = t.ci1 - t.ci0;
    const int h = t.ri1 - t.ri0;
    if (w <= 0 || h <= 0) return;
    const int wq = (w + 1) >> 1;
    const int per_colour = h * wq;
    const int total = (C == 2 ? 2 : 1) * per_colour;
#pragma unroll 2
    for (int x = threadIdx.x; x < total; x += kThreads) {
        const int cc = C == 2 ? (x >= per_colour) : C;
        const int xx = (C == 2 && cc) ? x - per_colour : x;
        const int r = xx / wq;
        const int i = t.ri0 + r;
        const int j = t.ci0 + 2 * (xx - r * wq) + ((i + t.ci0 + cc) & 1);
        if (j >= t.ci1) continue;
        if (C == 2) {
            if (cc)
                update_cell<A, KIND, FOLD, false>(p, i, j, q.prev[1], q.next[1], q.oth[1], q.rhs[1], acc);
            else
                update_cell<A, KIND, FOLD, false>(p, i, j, q.prev[0], q.next[0], q.oth[0], q.rhs[0], acc);
        } else {
            update_cell<A, KIND, FOLD, false>(p, i, j, q.prev[C], q.next[C], q.oth[C], q.rhs[C], acc);
        }
    }
}

// Frame cells of colour C (C = 2: both colours): tile cells outside the interior region.
template <Arith A, int KIND, bool FOLD, int C>
__device__ __forceinline__ void frame_pass(const PoissonParams& p, const Tile& t, const SweepPtrs& q,
                                           NormAcc& acc) {
    const int W = t.c1 - t.c0;
    const int top = t.ri0 - t.r0, bot = t.r1 - t.ri1;
    const int left = t.ci0 - t.c0, right = t.c1 - t.ci1;
    const int mid = t.ri1 - t.ri0;
    const int n_rows = (top + bot) * W;
    const int total = n_rows + mid * (left + right);
    for (int x = threadIdx.x; x < total; x += kThreads) {
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
            update_cell<A, KIND, FOLD, true>(p, i, j, q.prev[C], q.next[C], q.oth[C], q.rhs[C], acc);
        } else if (cc) {
            update_cell<A, KIND, FOLD, true>(p, i, j, q.prev[1], q.next[1], q.oth[1], q.rhs[1], acc);
        } else {
            update_cell<A, KIND, FOLD, true>(p, i, j, q.prev[0], q.next[0], q.oth[0], q.rhs[0], acc);
        }
    }
}

// Adds this block's share of e_k (chunk sums of the block in s_chunk[4], overflow flag in
// s_big) to ring slot k % kRing. Called by one thread at a point where no block barrier waits
// for it: the fence before the count stalls only that thread.
__device__ __forceinline__ void contribute(SyncState* sy, int k, const unsigned long long* s_chunk,
                                           unsigned int s_big) {
    const int slot = k % kRing;
    if (s_big) atomicOr(&sy->nonfinite[slot], 1u);
#pragma unroll
    for (int w = 0; w < 4; ++w) atomicAdd(&sy->acc[slot][w], s_chunk[w]);
    __threadfence();
    atomicAdd(&sy->count[slot], 1u);
}

// Threads 0..3 each wait for one neighbour's flag to reach `want` (in parallel); the block then
// goes on together. Returns false if a wait gave up (timeout or abort).
__device__ __forceinline__ bool neighbours_at(const unsigned* flags, const Tile& t, unsigned want, Ctrl* ctl,
                                              long long timeout_ns, int* s_ok) {
    if (threadIdx.x < 4) {
        const int nb = t.nb[threadIdx.x];
        s_ok[threadIdx.x] = nb < 0 ? 1 : (wait_geq(flags + nb, want, ctl, timeout_ns) ? 1 : 0);
    }
    __syncthreads();
    const bool ok = s_ok[0] & s_ok[1] & s_ok[2] & s_ok[3];
    return ok;
}

// After the frame pass: make this block's frame writes visible, then raise its flag. Only thread
// 0 waits for the fence; the others go straight on to the interior pass.
__device__ __forceinline__ void publish(unsigned* flag, unsigned value) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        st_release(flag, value);
    }
}

template <Arith A, int KIND, bool FOLD>
__global__ void __launch_bounds__(kThreads, 2) k_poisson(PoissonLaunch L) {
    Ctrl* ctl = L.ctrl;
    if (ctl->abort) return;
    const PoissonParams p = L.p;
    SyncState* sy = reinterpret_cast<SyncState*>(L.sync);
    const Geometry geo{p.n, p.pitch, L.gx, L.gy};
    const Tile t = make_tile(geo, blockIdx.x);
    const int me = blockIdx.x;
    __shared__ unsigned long long s_wchunk[kThreads / 32][4];
    __shared__ unsigned long long s_chunk[4];
    __shared__ unsigned int s_wbig[kThreads / 32];
    __shared__ unsigned int s_big;
    __shared__ int s_stop;    // 0 run on, 1 converged, 2 failure
    __shared__ double s_e;
    __shared__ int s_ok[4];

    // two copies of psi: set 0 = L.sor (the caller's output), set 1 = L.alt
    double* const s0r = L.sor[0];
    double* const s0b = L.sor[1];
    double* const s1r = L.alt[0];
    double* const s1b = L.alt[1];

    int k = 1, conv_k = -1, status = CNV_NOT_CONVERGED;
    double e_last = 0.0;
    const int kmax = p.itmax;  // sweeps 1..itmax correspond to the reference's k = 0..itmax-1

    // Check e_j (1 <= j); returns 0 run on, 1 converged at j, 2 failure.
    auto check = [&](int j) -> int {
        if (threadIdx.x == 0) {
            int res = 0;
            const int slot = j % kRing;
            if (!wait_geq(&sy->count[slot], (unsigned)gridDim.x, ctl, p.timeout_ns)) {
                res = 2;
            } else {
                unsigned long long c[4];
#pragma unroll
                for (int w = 0; w < 4; ++w) c[w] = __ldcg(&sy->acc[slot][w]);
                // carry-propagate the 32-bit chunks into a 128-bit value
                unsigned long long t = c[0];
                unsigned long long lo = t & 0xffffffffull;
                t = c[1] + (t >> 32);
                lo |= (t & 0xffffffffull) << 32;
                t = c[2] + (t >> 32);
                unsigned long long hi = t & 0xffffffffull;
                t = c[3] + (t >> 32);
                hi |= t << 32;
                const double e = from_fixed96(lo, hi);
                s_e = e;
                if (__ldcg(&sy->nonfinite[slot]) || !isfinite(e)) res = 3;
                else if (e < p.tol) res = 1;
            }
            s_stop = res;
        }
        __syncthreads();
        const int r = s_stop;
        __syncthreads();
        return r;
    };

    for (k = 1; k <= kmax; ++k) {
        if (k >= 3) {
            const int r = check(k - 2);
            if (r == 1) { conv_k = k - 2; status = CNV_OK; e_last = s_e; break; }
            if (r == 2) { status = CNV_TIMEOUT; break; }
            if (r == 3) { status = CNV_NONFINITE; e_last = s_e; break; }
            e_last = s_e;
            if (me == 0 && threadIdx.x == 0 && k >= 5) {
                // everyone has read e_{k-4} (they all finished sweep k-2); reuse its slot
                const int slot = (k - 4) % kRing;
#pragma unroll
                for (int w = 0; w < 4; ++w) sy->acc[slot][w] = 0;
                sy->nonfinite[slot] = 0;
                __threadfence();
                atomicExch(&sy->count[slot], 0u);
            }
        }
        // sweep k reads set (k-1)&1 and writes set k&1
        const bool odd = k & 1;
        SweepPtrs q;
        q.prev[0] = odd ? s0r : s1r;
        q.prev[1] = odd ? s0b : s1b;
        q.next[0] = odd ? s1r : s0r;
        q.next[1] = odd ? s1b : s0b;
        q.rhs[0] = L.rhs[0];
        q.rhs[1] = L.rhs[1];
        NormAcc acc{{0, 0, 0, 0}, 0};
        if (KIND == CNV_POISSON_JACOBI) {
            q.oth[0] = q.prev[1];
            q.oth[1] = q.prev[0];
            if (!neighbours_at(sy->flag[1], t, (unsigned)(k - 1), ctl, p.timeout_ns, s_ok)) { status = CNV_TIMEOUT; break; }
            frame_pass<A, KIND, FOLD, 2>(p, t, q, acc);
            publish(&sy->flag[1][me], (unsigned)k);
            if (threadIdx.x == 32 && k > 1) contribute(sy, k - 1, s_chunk, s_big);
            interior_pass<A, KIND, FOLD, 2>(p, t, q, acc);
            __syncthreads();
        } else {
            // red: black neighbours of sweep k-1, own red of sweep k-1
            q.oth[0] = q.prev[1];
            q.oth[1] = q.next[0];  // black: red of sweep k (new), own black of sweep k-1
            if (!neighbours_at(sy->flag[1], t, (unsigned)(k - 1), ctl, p.timeout_ns, s_ok)) { status = CNV_TIMEOUT; break; }
            frame_pass<A, KIND, FOLD, 0>(p, t, q, acc);
            publish(&sy->flag[0][me], (unsigned)k);
            if (threadIdx.x == 32 && k > 1) contribute(sy, k - 1, s_chunk, s_big);
            interior_pass<A, KIND, FOLD, 0>(p, t, q, acc);
            __syncthreads();
            if (!neighbours_at(sy->flag[0], t, (unsigned)k, ctl, p.timeout_ns, s_ok)) { status = CNV_TIMEOUT; break; }
            frame_pass<A, KIND, FOLD, 1>(p, t, q, acc);
            publish(&sy->flag[1][me], (unsigned)k);
            interior_pass<A, KIND, FOLD, 1>(p, t, q, acc);
            __syncthreads();
        }
        // this block's share of e_k: integer chunk sums (exact, order-free); thread 32 adds them
        // to the ring during the next sweep's interior pass, where no barrier waits for its fence
        {
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                unsigned long long x = acc.c[w];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
                acc.c[w] = x;
            }
            const unsigned big = __any_sync(0xffffffffu, acc.big) ? 1u : 0u;
            if ((threadIdx.x & 31) == 0) {
#pragma unroll
                for (int w = 0; w < 4; ++w) s_wchunk[threadIdx.x >> 5][w] = acc.c[w];
                s_wbig[threadIdx.x >> 5] = big;
            }
            __syncthreads();
            if (threadIdx.x < 4) {
                unsigned long long x = 0;
                for (int w = 0; w < kThreads / 32; ++w) x += s_wchunk[w][threadIdx.x];
                s_chunk[threadIdx.x] = x;
            } else if (threadIdx.x == 4) {
                unsigned b2 = 0;
                for (int w = 0; w < kThreads / 32; ++w) b2 |= s_wbig[w];
                s_big = b2;
            }
            __syncthreads();
        }
    }
    // the last sweep's share is still pending when the loop runs out of sweeps
    if (status == CNV_NOT_CONVERGED && k > kmax && threadIdx.x == 32) contribute(sy, kmax, s_chunk, s_big);
    if (status == CNV_NOT_CONVERGED && k > kmax) {
        // sweeps kmax-1 and kmax are not checked yet
        for (int j = (kmax >= 2 ? kmax - 1 : 1); j <= kmax; ++j) {
            const int r = check(j);
            if (r == 1) { conv_k = j; status = CNV_OK; e_last = s_e; break; }
            if (r == 2) { status = CNV_TIMEOUT; break; }
            if (r == 3) { status = CNV_NONFINITE; e_last = s_e; break; }
            e_last = s_e;
        }
    }
    if (status == CNV_TIMEOUT) return;
    // the answer is the iterate of sweep conv_k (or of the last sweep): copy it into set 0
    const int ans = conv_k > 0 ? conv_k : kmax;
    if (ans & 1) {
        const int h = t.r1 - t.r0, w = t.c1 - t.c0;
        for (int x = threadIdx.x; x < h * w; x += kThreads) {
            const int i = t.r0 + x / w, j = t.c0 + x % w;
            const size_t idx = (size_t)i * p.pitch + (j >> 1);
            if ((i + j) & 1) s0b[idx] = s1b[idx];
            else s0r[idx] = s1r[idx];
        }
    }
    if (me == 0 && threadIdx.x == 0) {
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
    // one block (512 threads) per about 2048 interior cells, at most 2 per SM, and a multiple
    // of the SM count once the grid covers the GPU so that every SM gets the same work
    const long long cells = (long long)(n - 2) * (n - 2);
    const int cap = std::min(std::min(per_sm, 2) * sms, kMaxSolverBlocks);
    long long want = cells / 2048;
    if (want >= 2LL * sms && cap >= 2 * sms) return 2 * sms;
    if (want >= sms) return std::min(sms, cap);
    return (int)std::max(1LL, std::min<long long>(want, cap));
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
