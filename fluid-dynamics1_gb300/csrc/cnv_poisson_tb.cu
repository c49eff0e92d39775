// cnv_poisson_tb.cu -- persistent red-black SOR / Gauss-Seidel with several sweeps per border
// exchange, bit-identical to k_poisson (cnv_poisson.cu).
//
// The same solve as k_poisson (src/poisson.c:111-173 and :62-109 with the red-black ordering
// of :239-261, zero start, stop at the first sweep k with sum|psi_k+1 - psi_k| < tol), with the
// same point update and the same exact stop norm (cnv_sor.cuh), so every iterate, the stop
// sweep and the answer are the same bits. What changes is how blocks cooperate.
//
// Tiles in shared memory. Each block owns one tile of the interior and keeps psi (and the
// right-hand side when it fits) on the tile plus a halo of width H = 2S in shared memory (S = 2
// or 4 sweeps per exchange), in the red/black split layout. An epoch is S sweeps done entirely in
// shared memory: half-sweep h (1 .. 2S) updates its colour on the tile grown by H - h cells on
// every side (clipped to the interior), so after the epoch the tile holds exactly what global
// red-black sweeps would hold; the halo cells are recomputed redundantly. At the end of an epoch
// every block writes its own cells into snapshot slot E % kTbSnap (a full split-layout copy of
// psi in global memory) and raises its flag; the next epoch waits for the eight neighbours'
// flags and loads its halo from that slot. One exchange per S sweeps instead of two per sweep.
//
// Stop test and rollback. Each block adds its share of e_k for every sweep of the epoch to a
// ring of 128-bit fixed-point sums (exact, order-free) and counts itself in per epoch. At the
// start of epoch E a block checks the sweeps of epoch E-2 (long complete). Cells with |psi| >= 2^46
// add to an FP64 side sum instead, as in k_poisson. If sweep k of epoch
// X = E-2 met the tolerance (and no earlier sweep did), every block stops there, reloads its
// tile and halo from the snapshot of the end of epoch X-1 (slot (X-1) % kTbSnap; psi = 0 when
// X = 0), replays the sweeps of epoch X up to k, and writes its own cells of that iterate as the
// answer. Neighbours are at most one epoch ahead of a block and stop at the same check, so the
// slot read by the replay is never overwritten while it is needed (4 slots).
//
// Every wait is bounded (timeout + abort flag) and records CNV_TIMEOUT instead of hanging.
#include <algorithm>
#include <cfloat>

#include "cnv_kernels.h"
#include "cnv_sor.cuh"

namespace cnv {
namespace {

constexpr int kTbThreads = 1024;
constexpr int kTbMaxSweeps = 4;          // sweeps per exchange (one epoch): S = 2 or 4, halo 2S
constexpr int kTbRing = 8;               // epochs of stop-norm sums in flight
constexpr int kTbSnap = 4;               // snapshots of psi kept in global memory

struct TbSync {
    unsigned long long acc[kTbRing][kTbMaxSweeps][4];  // e_k * 2^80 as 32-bit chunks in 64-bit counters
    double fsum[kTbRing][kTbMaxSweeps];             // FP64 part of e_k (cells with |psi| >= 2^46), usually 0
    unsigned int count[kTbRing];                    // blocks that added their share of an epoch
    unsigned int flag[kMaxSolverBlocks];            // epochs a block has completed (snapshot written)
};

struct TbTile {
    int r0, r1, c0, c1;  // owned rows/cols (absolute, interior)
    int nb[8];           // the eight adjacent tiles' blocks, -1 where there is none
};

__device__ __forceinline__ TbTile make_tb_tile(int n, int gx, int gy, int b) {
    TbTile t;
    const int ni = n - 2;
    const int tx = b % gx, ty = b / gx;
    t.c0 = 1 + (int)((long long)ni * tx / gx);
    t.c1 = 1 + (int)((long long)ni * (tx + 1) / gx);
    t.r0 = 1 + (int)((long long)ni * ty / gy);
    t.r1 = 1 + (int)((long long)ni * (ty + 1) / gy);
    int k = 0;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            if (!dx && !dy) continue;
            const int x = tx + dx, y = ty + dy;
            t.nb[k++] = (x >= 0 && x < gx && y >= 0 && y < gy) ? y * gx + x : -1;
        }
    return t;
}

__host__ __device__ __forceinline__ int fhalf(int j) { return j >= 0 ? j / 2 : -((1 - j) / 2); }

// Shared-memory geometry: rows sr0 .. sr0+sh-1, split columns m0 .. m0+swm-1, per colour.
struct TbGeom {
    int sr0, sh, m0, swm;
};

template <int S>
__device__ __forceinline__ TbGeom tb_geom(const TbTile& t) {
    constexpr int H = 2 * S;
    TbGeom g;
    g.sr0 = t.r0 - H;
    g.sh = t.r1 - t.r0 + 2 * H;
    g.m0 = fhalf(t.c0 - H);
    g.swm = fhalf(t.c1 + H - 1) - g.m0 + 1;
    return g;
}

// One colour c of a red-black half-sweep on rows [lo_r, hi_r), columns [lo_c, hi_c) of the
// shared-memory tile. psi of colour c at sc, of the other colour at so; the right-hand side of
// colour c at gs (shared, same geometry) or gg (global split layout, pitch P). With NORM, cells
// of the owned box add |new - old| to this thread's accumulator, which is reduced per warp and
// added to s_sum (4 chunks) at the end; owned cells with |psi| >= 2^46 add to s_fsum in FP64.
extern __shared__ double tb_smem[];

template <Arith A, int KIND, bool FOLD, bool G_SMEM, bool NORM>
__device__ __forceinline__ void tb_half_sweep(const PoissonParams& p, int sc_off, int so_off,
                                              const double* __restrict__ gglob, int g_off, TbGeom G, int lo_r,
                                              int hi_r, int lo_c, int hi_c, int c, int own_r0, int own_r1,
                                              int own_c0, int own_c1, unsigned long long* s_sum,
                                              double* s_fsum) {
    // split columns of a row of parity q = (i + c) & 1 (cell j = 2m + q)
    const int mlo0 = fhalf(lo_c + 1), mhi0 = fhalf(hi_c - 1);       // q = 0
    const int mlo1 = fhalf(lo_c), mhi1 = fhalf(hi_c - 2);           // q = 1
    const int w = max(mhi0 - mlo0, mhi1 - mlo1) + 1;
    const int rows = hi_r - lo_r;
    NormAcc acc{{0, 0, 0, 0}};
    if (w > 0 && rows > 0) {
        const int total = rows * w;
        const int swm = G.swm;
        // shared-memory arrays are addressed through tb_smem with integer offsets, so every
        // access compiles to a shared-memory load or store
        for (int x = threadIdx.x; x < total; x += kTbThreads) {
            const int r = x / w;
            const int i = lo_r + r;
            const int q = (i + c) & 1;
            const int m = (q ? mlo1 : mlo0) + (x - r * w);
            if (m > (q ? mhi1 : mhi0)) continue;
            const int k = (i - G.sr0) * swm - G.m0 + m;
            const double old = tb_smem[sc_off + k];
            const double up = tb_smem[so_off + k + swm];
            const double dn = tb_smem[so_off + k - swm];
            const double lt = tb_smem[so_off + k - 1 + q];
            const double rt = tb_smem[so_off + k + q];
            const double g = G_SMEM ? tb_smem[g_off + k] : __ldg(gglob + (size_t)i * p.pitch + m);
            // one update for every cell (no divergence on the FP64 path); only owned cells count
            const double nw = point_value<A, KIND, FOLD>(p, up, dn, rt, lt, g, old);
            tb_smem[sc_off + k] = nw;
            if (NORM) {
                const int j = 2 * m + q;
                if (i >= own_r0 && i < own_r1 && j >= own_c0 && j < own_c1) {
                    if (!norm_add(acc, nw, old)) norm_side_add(s_fsum, nw, old);
                }
            }
        }
    }
    if (NORM) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            unsigned long long v = acc.c[k];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            acc.c[k] = v;
        }
        if ((threadIdx.x & 31) == 0) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (acc.c[k]) atomicAdd(s_sum + k, acc.c[k]);
        }
    }
}

struct TbLaunchDev {
    PoissonParams p;
    int gx, gy, g_in_smem;
    double* out[2];
    const double* rhs[2];
    double* snap;  // kTbSnap slots x 2 colours x n x pitch doubles
    Ctrl* ctrl;
    void* sync;
};

__device__ __forceinline__ double* snap_at(const TbLaunchDev& L, int slot, int c) {
    return L.snap + ((size_t)(slot * 2 + c) * L.p.n) * L.p.pitch;
}

// Fill the shared tile (both colours) from snapshot `slot`, or with zeros (slot < 0). With
// halo_only, cells of the owned box are kept.
__device__ void tb_load(const TbLaunchDev& L, const TbTile& t, const TbGeom& G, double* const* sp, int slot,
                        bool halo_only) {
    const int n = L.p.n;
    const int total = G.sh * G.swm;
    for (int x = threadIdx.x; x < total; x += kTbThreads) {
        const int r = x / G.swm;
        const int mm = x - r * G.swm;
        const int i = G.sr0 + r;
        const int m = G.m0 + mm;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const int j = 2 * m + ((i + c) & 1);
            const bool inside = i >= 1 && i <= n - 2 && j >= 1 && j <= n - 2;
            const bool own = i >= t.r0 && i < t.r1 && j >= t.c0 && j < t.c1;
            if (halo_only && own) continue;
            sp[c][x] = (inside && slot >= 0) ? __ldcg(snap_at(L, slot, c) + (size_t)i * L.p.pitch + m) : 0.0;
        }
    }
}

// Own cells of the shared tile -> dst[c] (split layout, pitch P).
__device__ void tb_store_own(const TbTile& t, const TbGeom& G, double* const* sp, double* d0, double* d1, int P) {
    const int W = t.c1 - t.c0, H = t.r1 - t.r0;
    const int total = W * H;
    for (int x = threadIdx.x; x < total; x += kTbThreads) {
        const int r = x / W;
        const int i = t.r0 + r;
        const int j = t.c0 + (x - r * W);
        const int c = (i + j) & 1;
        const int m = j >> 1;
        (c ? d1 : d0)[(size_t)i * P + m] = sp[c][(i - G.sr0) * G.swm + (m - G.m0)];
    }
}

// nsweeps red-black sweeps on the shared tile: psi colour c at tb_smem[c * plane ...], the
// right-hand side colour c at tb_smem[(2 + c) * plane ...] (G_SMEM) or rhs[c] (global).
template <int S, Arith A, int KIND, bool FOLD, bool G_SMEM>
__device__ __forceinline__ void tb_sweeps(const TbLaunchDev& L, const TbTile& t, const TbGeom& G, int plane,
                                          int nsweeps, bool norm, unsigned long long (*s_sum)[4],
                                          double* s_fsum) {
    const int n = L.p.n;
    for (int sw = 0; sw < nsweeps; ++sw) {
        for (int c = 0; c < 2; ++c) {
            const int h = 2 * sw + c + 1;
            const int grow = 2 * S - h;
            const int lo_r = max(1, t.r0 - grow), hi_r = min(n - 1, t.r1 + grow);
            const int lo_c = max(1, t.c0 - grow), hi_c = min(n - 1, t.c1 + grow);
            const int sc = c * plane, so = (c ^ 1) * plane, go = (2 + c) * plane;
            const double* gg = c ? L.rhs[1] : L.rhs[0];
            if (norm)
                tb_half_sweep<A, KIND, FOLD, G_SMEM, true>(L.p, sc, so, gg, go, G, lo_r, hi_r, lo_c, hi_c, c, t.r0,
                                                           t.r1, t.c0, t.c1, s_sum[sw], s_fsum + sw);
            else
                tb_half_sweep<A, KIND, FOLD, G_SMEM, false>(L.p, sc, so, gg, go, G, lo_r, hi_r, lo_c, hi_c, c,
                                                            t.r0, t.r1, t.c0, t.c1, nullptr, nullptr);
            __syncthreads();
        }
    }
}

template <int S, Arith A, int KIND, bool FOLD, bool G_SMEM>
__global__ void __launch_bounds__(kTbThreads, 1) k_poisson_tb(TbLaunchDev L) {
    Ctrl* ctl = L.ctrl;
    if (ctl->abort) return;
    double* const s_dyn = tb_smem;
    __shared__ unsigned long long s_sum[kTbMaxSweeps][4];
    __shared__ double s_fsum[kTbMaxSweeps];
    __shared__ int s_ok[8];
    __shared__ int s_res, s_k;
    __shared__ double s_e;
    const PoissonParams& p = L.p;
    TbSync* sy = reinterpret_cast<TbSync*>(L.sync);
    const int n = p.n, P = p.pitch, me = blockIdx.x;
    const TbTile t = make_tb_tile(n, L.gx, L.gy, me);
    const TbGeom G = tb_geom<S>(t);
    const int plane = G.sh * G.swm;
    double* const sp[2] = {s_dyn, s_dyn + plane};
    if (G_SMEM) {
        double* sg0 = s_dyn + 2 * plane;
        double* sg1 = s_dyn + 3 * plane;
        for (int x = threadIdx.x; x < plane; x += kTbThreads) {
            const int r = x / G.swm;
            const int i = G.sr0 + r;
            const int m = G.m0 + (x - r * G.swm);
            const bool row_in = i >= 1 && i <= n - 2;
            const int j0 = 2 * m + (i & 1), j1 = 2 * m + ((i + 1) & 1);
            sg0[x] = (row_in && j0 >= 1 && j0 <= n - 2) ? __ldg(L.rhs[0] + (size_t)i * P + m) : 0.0;
            sg1[x] = (row_in && j1 >= 1 && j1 <= n - 2) ? __ldg(L.rhs[1] + (size_t)i * P + m) : 0.0;
        }
    }
    for (int x = threadIdx.x; x < 2 * plane; x += kTbThreads) s_dyn[x] = 0.0;  // psi = 0 start
    __syncthreads();

    const int kmax = p.itmax;
    const int nepochs = (kmax + S - 1) / S;
    int status = CNV_NOT_CONVERGED, conv_k = -1, checked = -1, E = 0;
    double e_last = 0.0;

    // Check the sweeps of epoch X in order: 0 none met the tolerance, 1 sweep s_k did,
    // 2 timeout, 3 non-finite. Thread 0 decides; the block reads the result.
    auto check = [&](int X) -> int {
        if (threadIdx.x == 0) {
            const int slot = X % kTbRing;
            const int ns = min(S, kmax - X * S);
            int res = 0;
            if (!wait_geq(&sy->count[slot], (unsigned)gridDim.x, ctl, p.timeout_ns)) {
                res = 2;
            } else {
                for (int s = 0; s < ns && res == 0; ++s) {
                    unsigned long long c[4];
#pragma unroll
                    for (int w = 0; w < 4; ++w) c[w] = __ldcg(&sy->acc[slot][s][w]);
                    const double e = __dadd_rn(norm_total(c), __ldcg(&sy->fsum[slot][s]));
                    s_e = e;
                    s_k = X * S + s + 1;
                    if (!isfinite(e)) res = 3;
                    else if (e < p.tol) res = 1;
                }
            }
            s_res = res;
        }
        __syncthreads();
        const int r = s_res;
        __syncthreads();
        return r;
    };

    for (E = 0; E < nepochs; ++E) {
        if (E >= 2) {
            const int r = check(E - 2);
            checked = E - 2;
            e_last = s_e;
            if (r == 1) { conv_k = s_k; status = CNV_OK; break; }
            if (r == 2) { status = CNV_TIMEOUT; break; }
            if (r == 3) { status = CNV_NONFINITE; break; }
            if (me == 0 && threadIdx.x == 0 && E >= 4) {
                // every block has finished epoch E-2, so every block has checked epoch E-4
                const int slot = (E - 4) % kTbRing;
                for (int s = 0; s < kTbMaxSweeps; ++s) {
#pragma unroll
                    for (int w = 0; w < 4; ++w) sy->acc[slot][s][w] = 0;
                    sy->fsum[slot][s] = 0.0;
                }
                __threadfence();
                atomicExch(&sy->count[slot], 0u);
            }
        }
        if (E >= 1) {
            // neighbours' cells after epoch E-1 -> halo
            if (threadIdx.x < 8) {
                const int nb = t.nb[threadIdx.x];
                s_ok[threadIdx.x] = nb < 0 ? 1 : (wait_geq(&sy->flag[nb], (unsigned)E, ctl, p.timeout_ns) ? 1 : 0);
            }
            __syncthreads();
            bool ok = true;
            for (int q = 0; q < 8; ++q) ok = ok && s_ok[q];
            if (!ok) { status = CNV_TIMEOUT; break; }
            tb_load(L, t, G, sp, (E - 1) % kTbSnap, true);
        }
        if (threadIdx.x < kTbMaxSweeps * 4) s_sum[threadIdx.x / 4][threadIdx.x % 4] = 0;
        if (threadIdx.x < kTbMaxSweeps) s_fsum[threadIdx.x] = 0.0;
        __syncthreads();
        const int ns = min(S, kmax - E * S);
        tb_sweeps<S, A, KIND, FOLD, G_SMEM>(L, t, G, plane, ns, true, s_sum, s_fsum);
        // this block's shares of e for the epoch's sweeps, then the epoch count
        const int slot = E % kTbRing;
        if (threadIdx.x < ns * 4) {
            const unsigned long long v = s_sum[threadIdx.x / 4][threadIdx.x % 4];
            if (v) atomicAdd(&sy->acc[slot][threadIdx.x / 4][threadIdx.x % 4], v);
        } else if (threadIdx.x >= 32 && threadIdx.x < 32 + ns) {
            const double fs = s_fsum[threadIdx.x - 32];
            if (fs != 0.0 || fs != fs) atomicAdd(&sy->fsum[slot][threadIdx.x - 32], fs);
        }
        // own cells -> snapshot slot E % kTbSnap
        tb_store_own(t, G, sp, snap_at(L, E % kTbSnap, 0), snap_at(L, E % kTbSnap, 1), P);
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(&sy->count[slot], 1u);
            st_release(&sy->flag[me], (unsigned)(E + 1));
        }
    }
    // epochs not checked yet (the loop ran out of sweeps)
    if (status == CNV_NOT_CONVERGED) {
        for (int X = checked + 1; X < nepochs; ++X) {
            const int r = check(X);
            e_last = s_e;
            if (r == 1) { conv_k = s_k; status = CNV_OK; break; }
            if (r == 2) { status = CNV_TIMEOUT; break; }
            if (r == 3) { status = CNV_NONFINITE; break; }
        }
    }
    if (status == CNV_TIMEOUT) return;
    if (status == CNV_OK) {
        // replay epoch X from the snapshot of its start up to the converged sweep
        const int X = (conv_k - 1) / S;
        __syncthreads();
        tb_load(L, t, G, sp, X > 0 ? (X - 1) % kTbSnap : -1, false);
        __syncthreads();
        tb_sweeps<S, A, KIND, FOLD, G_SMEM>(L, t, G, plane, conv_k - X * S, false, nullptr, nullptr);
    }
    tb_store_own(t, G, sp, L.out[0], L.out[1], P);
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

template <int S, Arith A, int KIND, bool FOLD>
const void* tb_kernel(bool g_smem) {
    return g_smem ? reinterpret_cast<const void*>(&k_poisson_tb<S, A, KIND, FOLD, true>)
                  : reinterpret_cast<const void*>(&k_poisson_tb<S, A, KIND, FOLD, false>);
}

template <int S>
const void* tb_kernel_s(Arith a, int kind, bool fold, bool g_smem) {
    if (a == Arith::kExact) {
        if (fold)
            return kind == CNV_POISSON_SOR ? tb_kernel<S, Arith::kExact, CNV_POISSON_SOR, true>(g_smem)
                                           : tb_kernel<S, Arith::kExact, CNV_POISSON_GS, true>(g_smem);
        return kind == CNV_POISSON_SOR ? tb_kernel<S, Arith::kExact, CNV_POISSON_SOR, false>(g_smem)
                                       : tb_kernel<S, Arith::kExact, CNV_POISSON_GS, false>(g_smem);
    }
    return kind == CNV_POISSON_SOR ? tb_kernel<S, Arith::kFma, CNV_POISSON_SOR, false>(g_smem)
                                   : tb_kernel<S, Arith::kFma, CNV_POISSON_GS, false>(g_smem);
}

const void* tb_kernel_ptr(int sweeps, Arith a, int kind, bool fold, bool g_smem) {
    return sweeps == 2 ? tb_kernel_s<2>(a, kind, fold, g_smem) : tb_kernel_s<4>(a, kind, fold, g_smem);
}

}  // namespace

int tb_threads() { return kTbThreads; }
size_t tb_sync_bytes() { return sizeof(TbSync); }
size_t tb_snapshot_doubles(int n, int pitch) { return (size_t)kTbSnap * 2 * n * pitch; }

// Shared-memory bytes of the largest tile of a gx x gy tiling with `sweeps` sweeps per exchange
// (halo 2 * sweeps): psi (both colours) on the tile plus halo, and the same again for the
// right-hand side when g_smem.
size_t tb_smem_bytes(int n, int gx, int gy, int sweeps, bool g_smem) {
    const int ni = n - 2, H = 2 * sweeps;
    const int tw = (ni + gx - 1) / gx + 2 * H + 1;
    const int th = (ni + gy - 1) / gy + 2 * H;
    const int swm = tw / 2 + 2;
    return (g_smem ? 4 : 2) * (size_t)th * swm * sizeof(double);
}

bool tb_tiles_ok(int n, int gx, int gy, int sweeps) {
    const int ni = n - 2;
    return ni / gx >= 2 * sweeps && ni / gy >= 2 * sweeps;
}

cudaError_t launch_poisson_tb(const TbLaunch& T, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(T.sync, 0, sizeof(TbSync), s);
    if (e != cudaSuccess) return e;
    if (T.sweeps != 2 && T.sweeps != 4) return cudaErrorInvalidValue;
    const size_t smem = tb_smem_bytes(T.p.n, T.gx, T.gy, T.sweeps, T.g_in_smem != 0);
    const void* k = tb_kernel_ptr(T.sweeps, T.p.arith, T.p.kind, T.p.fold != 0, T.g_in_smem != 0);
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    TbLaunchDev L{};
    L.p = T.p;
    L.gx = T.gx;
    L.gy = T.gy;
    L.g_in_smem = T.g_in_smem;
    L.out[0] = T.out[0];
    L.out[1] = T.out[1];
    L.rhs[0] = T.rhs[0];
    L.rhs[1] = T.rhs[1];
    L.snap = T.snap;
    L.ctrl = T.ctrl;
    L.sync = T.sync;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(T.gx * T.gy);
    cfg.blockDim = dim3(kTbThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {&L};
    return cudaLaunchKernelExC(&cfg, k, args);
}

}  // namespace cnv
