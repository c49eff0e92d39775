// cnv_mixed.cu -- mixed-precision Poisson solve: FP32 red-black SOR sweeps inside FP64 defect
// correction, one persistent cooperative launch per solve.
//
// The equation is the reference's discrete Poisson problem (src/poisson.c:247 at its fixed
// point), written with the scaled right-hand side g = dx^2 dy^2 f that the transport pass
// produces:
//     dy^2 (psi[i+1][j] + psi[i-1][j]) + dx^2 (psi[i][j+1] + psi[i][j-1]) - den psi[i][j] = g[i][j]
// on the interior, psi = 0 on the edge, den = 2 (dx^2 + dy^2). Defect correction:
//     psi = 0 (FP64)
//     loop: R = g - A psi (FP64); stop when ||R||_2 <= rtol ||g||_2
//           solve A e = R approximately with `epochs * kSweepsPerExchange` FP32 red-black SOR
//           sweeps from e = 0
//           psi += e (FP64)
// Only the residual, the norm and the correction accumulation are FP64; every sweep is FP32.
//
// Layout. g, psi, the FP32 correction right-hand side R/den and the FP32 border-exchange copies
// of e all use the red/black split layout of the rest of the library (colour c = (i+j)&1 of cell
// (i, j) at A_c[i*pitch + (j>>1)]), and so does the shared-memory tile: every access in a sweep
// is unit-stride, and warps walk whole rows, so no integer division is needed per cell.
//
// Inner sweeps. Each block owns one tile and keeps e on the tile plus a halo of width
// H = 2*kSweepsPerExchange in shared memory. An "epoch" is kSweepsPerExchange red-black sweeps
// done entirely in shared memory: half-sweep s updates its colour on the tile grown by H - s
// cells on every side (clipped to the interior), so after 2*kSweepsPerExchange half-sweeps the
// tile holds exactly what global red-black SOR would hold. The redundant halo work buys one
// neighbour exchange per epoch instead of one per half-sweep. At an epoch's end every block
// writes its border strips (width H) into a global FP32 copy of e (double-buffered by epoch
// parity) and raises its flag; the next epoch waits for the eight neighbours' flags and loads
// their strips into the halo. Tiles are at least H cells wide and tall, so a halo only ever
// comes from the eight adjacent tiles.
//
// All waits are bounded (timeout + abort flag) and report CNV_TIMEOUT instead of hanging.
#include <algorithm>
#include <cfloat>

#include "cnv_kernels.h"
#include "cnv_stencil.cuh"
#include "cnv_sync.cuh"

namespace cnv {
namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr int kSweepsPerExchange = 8;  // 4: 4.05 us per sweep at 1024^2, 8: 3.45, 12: 3.40, 16: 3.47
constexpr int kHalo = 2 * kSweepsPerExchange;

struct MixedSync {
    unsigned int bar_count;     // grid barrier (outer iterations)
    unsigned int pad;
    double partial[2][kMaxSolverBlocks];  // per-block ||R||^2 and ||g||^2
    unsigned int flag[kMaxSolverBlocks];  // last epoch whose border strips a block has written
};

// Grid-wide barrier (counter of arrivals); false if it timed out or another block aborted.
__device__ bool grid_sync(MixedSync* sy, unsigned& epoch, Ctrl* ctl, long long timeout_ns, int* s_ok) {
    __syncthreads();
    ++epoch;
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&sy->bar_count, 1u);
        *s_ok = wait_geq(&sy->bar_count, epoch * gridDim.x, ctl, timeout_ns) ? 1 : 0;
        __threadfence();
    }
    __syncthreads();
    return *s_ok != 0;
}

struct MTile {
    int r0, r1, c0, c1;  // owned rows/cols (absolute)
    int nb[8];           // the eight adjacent tiles' blocks, -1 where there is none
};

__device__ __forceinline__ MTile make_mtile(int n, int gx, int gy, int b) {
    MTile t;
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

// Shared-memory tile in split layout: rows sr0 .. sr0+sh-1, global split columns m0 .. m0+swm-1.
struct SmemTile {
    int sr0, sh, m0, swm;
    float* c[2];
    __device__ __forceinline__ float& at(int col, int i, int m) const { return c[col][(i - sr0) * swm + (m - m0)]; }
};

}  // namespace

size_t mixed_sync_bytes() { return sizeof(MixedSync); }

// Shared-memory bytes the mixed kernel needs for the largest tile of a gx x gy tiling of n:
// e (both colours) on the tile plus halo, and the same again when the correction right-hand side
// is also kept there (rq_in_smem).
size_t mixed_smem_bytes(int n, int gx, int gy, bool rq_in_smem) {
    const int ni = n - 2;
    const int tw = (ni + gx - 1) / gx + 2 * kHalo;
    const int th = (ni + gy - 1) / gy + 2 * kHalo;
    const int swm = tw / 2 + 2;
    return (rq_in_smem ? 4 : 2) * (size_t)th * swm * sizeof(float);
}

namespace {

// The dynamic shared memory of k_mixed. The hot loop addresses it through this array with
// integer offsets, so every access compiles to a shared-memory load or store.
extern __shared__ float mx_smem[];

// One colour c of an FP32 red-black SOR half-sweep on rows [lo_r, hi_r), columns [lo_c, hi_c) of
// the shared-memory tile (split layout: row i of colour k at mx_smem[k_off + (i - sr0) * swm + (m -
// m0)]): e of colour c at sc_off, of the other colour at so_off; the correction right-hand side
// R/den at rq_off in shared memory (RQ_SMEM) or in the global split array rq (pitch P). Kept out
// of line so that it gets its own register allocation: it is the hot loop of the solve.
template <bool RQ_SMEM>
__device__ __noinline__ void mixed_half_sweep(int sc_off, int so_off, int rq_off, const float* __restrict__ rq,
                                              int sr0, int swm, int m0, int lo_r, int hi_r, int lo_c, int hi_c,
                                              int c, int P, float wx, float wy, float beta) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = lo_r + warp; i < hi_r; i += kWarps) {
        const int q = (i + c) & 1;
        const int mlo = floor_half(lo_c - q + 1), mhi = floor_half(hi_c - 1 - q);
        const int row = (i - sr0) * swm - m0;
        const float* rqrow = rq + (size_t)i * P;
        // unrolled 4 deep where R/den comes from L2 (the large grids): 2048^2 8.87 vs 9.18 us per
        // sweep; with R/den in shared memory (1024^2) unrolling ran slower (3.50 vs 3.46), and the
        // batch kernel's strip sweep, the same loop, ran its step 24 % slower unrolled
#pragma unroll(RQ_SMEM ? 1 : 4)
        for (int m = mlo + lane; m <= mhi; m += 32) {
            const int k = row + m;
            const float up = mx_smem[so_off + k + swm], dn = mx_smem[so_off + k - swm];
            const float lt = mx_smem[so_off + k - 1 + q], rt = mx_smem[so_off + k + q];
            // R/den: shared-memory copy, or L2 (rewritten every outer iteration)
            const float r = RQ_SMEM ? mx_smem[rq_off + k] : __ldcg(rqrow + m);
            const float me = mx_smem[sc_off + k];
            const float gs = fmaf(wy, up + dn, fmaf(wx, lt + rt, -r));
            mx_smem[sc_off + k] = fmaf(beta, gs - me, me);
        }
    }
}

__global__ void __launch_bounds__(kThreads, 1) k_mixed(MixedLaunch L) {
    Ctrl* ctl = L.ctrl;
    if (ctl->abort) return;
    float* const s_mem = mx_smem;
    __shared__ int s_ok;
    __shared__ int s_flag[8];
    __shared__ double s_red[kWarps][2];
    __shared__ double s_tot[2];
    MixedSync* sy = reinterpret_cast<MixedSync*>(L.sync);
    const int n = L.n, P = L.pitch;
    const MTile t = make_mtile(n, L.gx, L.gy, blockIdx.x);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    SmemTile S;
    S.sr0 = t.r0 - kHalo;
    S.sh = t.r1 - t.r0 + 2 * kHalo;
    S.m0 = floor_half(t.c0 - kHalo);
    S.swm = floor_half(t.c1 + kHalo - 1) - S.m0 + 1;
    S.c[0] = s_mem;
    S.c[1] = s_mem + S.sh * S.swm;
    const int ssz = 2 * S.sh * S.swm;
    // correction right-hand side tile (both colours) after e, when it fits in shared memory
    float* const srq = L.rq_in_smem ? s_mem + ssz : nullptr;

    const double dx2 = L.dx2, dy2 = L.dy2, den = L.den;
    const float wx = (float)(dx2 / den), wy = (float)(dy2 / den), beta = (float)L.beta;
    unsigned bar = 0, ep = 0;
    int outer = 0, status = CNV_NOT_CONVERGED;
    long long sweeps = 0;
    double rel = 0.0;

    for (outer = 0;; ++outer) {
        // ---- FP64 residual R = g - A psi on own cells, its norm, and the FP32 rhs R/den
        double rr = 0.0, gg = 0.0;
        for (int i = t.r0 + warp; i < t.r1; i += kWarps) {
            for (int c = 0; c < 2; ++c) {
                const int q = (i + c) & 1;  // cell (i, j) of colour c has j = 2m + q
                const int mlo = floor_half(t.c0 - q + 1), mhi = floor_half(t.c1 - 1 - q);
                const double* pc = L.psi[c];
                const double* po = L.psi[c ^ 1];
                for (int m = mlo + lane; m <= mhi; m += 32) {
                    const size_t k = (size_t)i * P + m;
                    const double g = L.g[c][k];
                    const double R = poisson_defect(dy2, dx2, den, __ldcg(po + k + P), __ldcg(po + k - P),
                                                    __ldcg(po + k - 1 + q), __ldcg(po + k + q), __ldcg(pc + k), g);
                    rr = fma(R, R, rr);
                    if (outer == 0) gg = fma(g, g, gg);
                    L.rq[c][k] = (float)(R * L.rden);
                }
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            rr += __shfl_xor_sync(0xffffffffu, rr, off);
            gg += __shfl_xor_sync(0xffffffffu, gg, off);
        }
        if (lane == 0) {
            s_red[warp][0] = rr;
            s_red[warp][1] = gg;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double a = 0.0, b = 0.0;
            for (int w = 0; w < kWarps; ++w) {
                a += s_red[w][0];
                b += s_red[w][1];
            }
            sy->partial[0][blockIdx.x] = a;
            if (outer == 0) sy->partial[1][blockIdx.x] = b;
        }
        if (!grid_sync(sy, bar, ctl, L.timeout_ns, &s_ok)) { status = CNV_TIMEOUT; break; }
        if (threadIdx.x < 32) {
            double a = 0.0, b = 0.0;
            for (int q = threadIdx.x; q < (int)gridDim.x; q += 32) {
                a += __ldcg(&sy->partial[0][q]);
                b += __ldcg(&sy->partial[1][q]);
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                a += __shfl_xor_sync(0xffffffffu, a, off);
                b += __shfl_xor_sync(0xffffffffu, b, off);
            }
            if (threadIdx.x == 0) {
                s_tot[0] = a;
                s_tot[1] = b;
            }
        }
        __syncthreads();
        const double rnorm = sqrt(s_tot[0]), gnorm = sqrt(s_tot[1]);
        rel = gnorm > 0 ? rnorm / gnorm : rnorm;
        __syncthreads();
        if (!isfinite(rel)) { status = CNV_NONFINITE; break; }
        if (rel <= L.rtol) { status = CNV_OK; break; }
        if (outer >= L.max_outer) break;
        if (srq) {
            // R/den on the tile plus halo (every block wrote its own cells before the barrier)
            for (int r = warp; r < S.sh; r += kWarps) {
                const int i = S.sr0 + r;
                for (int c = 0; c < 2; ++c) {
                    const int q = (i + c) & 1;
                    float* dst = srq + c * (S.sh * S.swm) + r * S.swm;
                    for (int mm = lane; mm < S.swm; mm += 32) {
                        const int j = 2 * (S.m0 + mm) + q;
                        dst[mm] = (i >= 1 && i <= n - 2 && j >= 1 && j <= n - 2)
                                      ? __ldcg(L.rq[c] + (size_t)i * P + S.m0 + mm)
                                      : 0.0f;
                    }
                }
            }
            __syncthreads();
        }

        // ---- FP32 inner solve: e = 0, then `epochs` epochs of kSweepsPerExchange sweeps
        for (int x = threadIdx.x; x < ssz; x += kThreads) s_mem[x] = 0.0f;
        __syncthreads();
        bool ok = true;
        for (int e = 0; e < L.epochs && ok; ++e) {
            ++ep;
            if (e > 0) {
                // neighbours' border strips of the previous epoch -> halo
                if (threadIdx.x < 8) {
                    const int nb = t.nb[threadIdx.x];
                    s_flag[threadIdx.x] = nb < 0 ? 1 : (wait_geq(&sy->flag[nb], ep - 1, ctl, L.timeout_ns) ? 1 : 0);
                }
                __syncthreads();
                for (int q = 0; q < 8; ++q) ok = ok && s_flag[q];
                if (!ok) break;
                // one flat loop over the tile-plus-halo box: every thread issues its few
                // independent L2 loads at once (a warp walking rows would wait for each in turn)
                const int par = (ep - 1) & 1;
                const int box = S.sh * S.swm;
                for (int x = threadIdx.x; x < box; x += kThreads) {
                    const int r = x / S.swm;
                    const int i = S.sr0 + r;
                    if (i < 1 || i > n - 2) continue;
                    const int m = S.m0 + (x - r * S.swm);
                    const bool own_row = i >= t.r0 && i < t.r1;
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const int j = 2 * m + ((i + c) & 1);
                        if (j < max(1, t.c0 - kHalo) || j >= min(n - 1, t.c1 + kHalo)) continue;
                        if (own_row && j >= t.c0 && j < t.c1) continue;  // own cell: already current
                        S.at(c, i, m) = __ldcg(L.eg[par][c] + (size_t)i * P + m);
                    }
                }
                __syncthreads();
            }
            for (int s = 1; s <= 2 * kSweepsPerExchange; ++s) {
                const int c = (s - 1) & 1;  // red first
                const int lo_r = max(1, t.r0 - kHalo + s), hi_r = min(n - 1, t.r1 + kHalo - s);
                const int lo_c = max(1, t.c0 - kHalo + s), hi_c = min(n - 1, t.c1 + kHalo - s);
                const int plane = S.sh * S.swm;  // e colour k at k * plane, R/den colour k at (2 + k) * plane
                if (srq)
                    mixed_half_sweep<true>(c * plane, (c ^ 1) * plane, (2 + c) * plane, L.rq[c], S.sr0, S.swm,
                                           S.m0, lo_r, hi_r, lo_c, hi_c, c, P, wx, wy, beta);
                else
                    mixed_half_sweep<false>(c * plane, (c ^ 1) * plane, 0, L.rq[c], S.sr0, S.swm, S.m0, lo_r,
                                            hi_r, lo_c, hi_c, c, P, wx, wy, beta);
                __syncthreads();
            }
            sweeps += kSweepsPerExchange;
            if (e + 1 < L.epochs) {
                // own border strips (width H) -> global copy of this epoch; raise the flag
                const int par = ep & 1;
                const int tw = t.c1 - t.c0, th = t.r1 - t.r0;
                for (int x = threadIdx.x; x < tw * th; x += kThreads) {
                    const int r = x / tw;
                    const int i = t.r0 + r;
                    const int j = t.c0 + (x - r * tw);
                    if (i >= t.r0 + kHalo && i < t.r1 - kHalo && j >= t.c0 + kHalo && j < t.c1 - kHalo) continue;
                    const int c = (i + j) & 1;
                    L.eg[par][c][(size_t)i * P + (j >> 1)] = S.at(c, i, j >> 1);
                }
                __syncthreads();
                if (threadIdx.x == 0) st_release(&sy->flag[blockIdx.x], ep);
            }
        }
        if (!ok) { status = CNV_TIMEOUT; break; }
        // ---- FP64 correction psi += e on own cells
        for (int i = t.r0 + warp; i < t.r1; i += kWarps) {
            for (int c = 0; c < 2; ++c) {
                const int q = (i + c) & 1;
                const int mlo = floor_half(t.c0 - q + 1), mhi = floor_half(t.c1 - 1 - q);
                double* pc = L.psi[c];
                for (int m = mlo + lane; m <= mhi; m += 32) pc[(size_t)i * P + m] += (double)S.at(c, i, m);
            }
        }
        if (!grid_sync(sy, bar, ctl, L.timeout_ns, &s_ok)) { status = CNV_TIMEOUT; break; }
    }
    if (status == CNV_TIMEOUT) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->iters = outer;
        ctl->err = rel;
        ctl->status = status;
        ctl->sweeps += sweeps;
        const int step = ctl->step;
        if (step < ctl->max_records) {
            StepRecord& r = ctl->records[step];
            r.iters = outer;
            r.status = status;
            r.err = rel;
            r.cont_max = 0.0;
            r.cont_min = 0.0;
        }
        if (status != CNV_OK) ctl->abort = 1;
    }
}

}  // namespace

cudaError_t launch_mixed(const MixedLaunch& L, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(L.sync, 0, sizeof(MixedSync), s);
    if (e != cudaSuccess) return e;
    const size_t smem = mixed_smem_bytes(L.n, L.gx, L.gy, L.rq_in_smem != 0);
    e = cudaFuncSetAttribute(k_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L.gx * L.gy);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {const_cast<MixedLaunch*>(&L)};
    return cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(&k_mixed), args);
}

int mixed_threads() { return kThreads; }
int mixed_sweeps_per_exchange() { return kSweepsPerExchange; }

}  // namespace cnv
