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
//           solve A e = R approximately with `inner` FP32 red-black SOR sweeps from e = 0
//           psi += e (FP64)
// Only the residual, the norm and the correction accumulation are FP64; every sweep is FP32.
//
// Inner sweeps. Each block owns one tile and keeps its correction e for the tile plus a halo of
// width H = 2*kSweepsPerExchange in shared memory. An "epoch" is kSweepsPerExchange red-black
// sweeps done entirely in shared memory: half-sweep s updates its colour on the tile grown by
// H - s cells on every side (clipped to the interior), so after 2*kSweepsPerExchange half-sweeps
// the tile itself holds exactly what global red-black SOR would hold. The redundant halo work is
// the price of talking to neighbours once per epoch instead of once per half-sweep. At an epoch's
// end every block writes its border strips (width H) into a global FP32 copy of e
// (double-buffered by epoch parity) and raises its flag; the next epoch starts by waiting for the
// eight neighbours' flags and loading their strips into the halo. The right-hand side of the
// correction (R / den, FP32) is read from global memory (L2) on every update.
//
// All waits are bounded (timeout + abort flag) and report CNV_TIMEOUT instead of hanging.
#include <algorithm>
#include <cfloat>

#include "cnv_kernels.h"

namespace cnv {
namespace {

constexpr int kThreads = 512;
constexpr int kSweepsPerExchange = 4;
constexpr int kHalo = 2 * kSweepsPerExchange;

struct MixedSync {
    unsigned int bar_count;     // grid barrier (outer iterations)
    unsigned int pad;
    double partial[2][kMaxSolverBlocks];  // per-block ||R||^2 and ||g||^2
    unsigned int flag[kMaxSolverBlocks];  // last epoch whose border strips a block has written
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ long long globaltimer_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ bool wait_geq(const unsigned* p, unsigned want, Ctrl* ctl, long long timeout_ns) {
    long long t0 = 0;
    int polls = 0;
    while ((int)(ld_acquire(p) - want) < 0) {
        if (*(const volatile int*)&ctl->abort) return false;
        if (++polls == 64) t0 = globaltimer_ns();
        if (polls > 64 && globaltimer_ns() - t0 > timeout_ns) {
            atomicExch(&ctl->status, CNV_TIMEOUT);
            atomicExch(&ctl->abort, 1);
            return false;
        }
    }
    return true;
}

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
    int nb[8];           // neighbour blocks (ty-1..ty+1, tx-1..tx+1 without self), -1 if none
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

}  // namespace

size_t mixed_sync_bytes() { return sizeof(MixedSync); }

// Shared-memory bytes the mixed kernel needs for the largest tile of a gx x gy tiling of n.
size_t mixed_smem_bytes(int n, int gx, int gy) {
    const int ni = n - 2;
    const int tw = (ni + gx - 1) / gx + 2 * kHalo;
    const int th = (ni + gy - 1) / gy + 2 * kHalo;
    return (size_t)tw * th * sizeof(float);
}

namespace {

__global__ void __launch_bounds__(kThreads, 1) k_mixed(MixedLaunch L) {
    Ctrl* ctl = L.ctrl;
    if (ctl->abort) return;
    extern __shared__ float s_e[];
    __shared__ int s_ok;
    __shared__ int s_flag[8];
    __shared__ double s_red[kThreads / 32][2];
    __shared__ double s_tot[2];
    MixedSync* sy = reinterpret_cast<MixedSync*>(L.sync);
    const int n = L.n;
    const MTile t = make_mtile(n, L.gx, L.gy, blockIdx.x);
    // shared tile geometry: rows r0-H .. r1+H-1, cols c0-H .. c1+H-1
    const int sr0 = t.r0 - kHalo, sc0 = t.c0 - kHalo;
    const int sh = t.r1 - t.r0 + 2 * kHalo, sw = t.c1 - t.c0 + 2 * kHalo;
    const int ssz = sh * sw;
    auto S = [&](int i, int j) -> float& { return s_e[(i - sr0) * sw + (j - sc0)]; };

    const double dx2 = L.dx2, dy2 = L.dy2, den = L.den;
    const float wx = (float)(dx2 / den), wy = (float)(dy2 / den), beta = (float)L.beta;
    unsigned bar = 0, ep = 0;
    int outer = 0, status = CNV_NOT_CONVERGED;
    long long sweeps = 0;
    double rel = 0.0;

    for (outer = 0;; ++outer) {
        // ---- FP64 residual R = g - A psi on own cells, its norm, and the FP32 rhs R/den
        double rr = 0.0, gg = 0.0;
        const int ow = t.c1 - t.c0, oh = t.r1 - t.r0;
        for (int x = threadIdx.x; x < ow * oh; x += kThreads) {
            const int i = t.r0 + x / ow, j = t.c0 + x % ow;
            const size_t k = (size_t)i * n + j;
            const double* P = L.psi;
            const double ap = dy2 * (__ldcg(P + k + n) + __ldcg(P + k - n)) +
                              dx2 * (__ldcg(P + k + 1) + __ldcg(P + k - 1)) - den * __ldcg(P + k);
            const double g = L.g[k];
            const double R = g - ap;
            rr = fma(R, R, rr);
            if (outer == 0) gg = fma(g, g, gg);
            L.rq[k] = (float)(R * L.rden);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            rr += __shfl_xor_sync(0xffffffffu, rr, off);
            gg += __shfl_xor_sync(0xffffffffu, gg, off);
        }
        if ((threadIdx.x & 31) == 0) {
            s_red[threadIdx.x >> 5][0] = rr;
            s_red[threadIdx.x >> 5][1] = gg;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double a = 0.0, b = 0.0;
            for (int w = 0; w < kThreads / 32; ++w) {
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

        // ---- FP32 inner solve: e = 0, then `epochs` epochs of kSweepsPerExchange sweeps
        for (int x = threadIdx.x; x < ssz; x += kThreads) s_e[x] = 0.0f;
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
                const float* eg = L.eg[(ep - 1) & 1];
                for (int x = threadIdx.x; x < ssz; x += kThreads) {
                    const int i = sr0 + x / sw, j = sc0 + x % sw;
                    const bool own = i >= t.r0 && i < t.r1 && j >= t.c0 && j < t.c1;
                    if (own || i < 1 || i > n - 2 || j < 1 || j > n - 2) continue;
                    s_e[x] = __ldcg(eg + (size_t)i * n + j);
                }
                __syncthreads();
            }
            for (int s = 1; s <= 2 * kSweepsPerExchange; ++s) {
                const int c = (s - 1) & 1;  // red first
                const int lo_r = max(1, t.r0 - kHalo + s), hi_r = min(n - 1, t.r1 + kHalo - s);
                const int lo_c = max(1, t.c0 - kHalo + s), hi_c = min(n - 1, t.c1 + kHalo - s);
                const int rw = hi_c - lo_c, rh = hi_r - lo_r;
                const int rq_w = (rw + 1) >> 1;
                for (int x = threadIdx.x; x < rh * rq_w; x += kThreads) {
                    const int r = x / rq_w;
                    const int i = lo_r + r;
                    const int j = lo_c + 2 * (x - r * rq_w) + ((i + lo_c + c) & 1);
                    if (j >= hi_c) continue;
                    float& me = S(i, j);
                    const float up = S(i + 1, j), dn = S(i - 1, j), lt = S(i, j - 1), rt = S(i, j + 1);
                    const float rq = __ldcg(L.rq + (size_t)i * n + j);  // rewritten every outer iteration
                    const float gs = fmaf(wy, up + dn, fmaf(wx, lt + rt, -rq));
                    me = fmaf(beta, gs - me, me);
                }
                __syncthreads();
            }
            sweeps += kSweepsPerExchange;
            if (e + 1 < L.epochs) {
                // own border strips (width H) -> global copy of this epoch; raise the flag
                float* eg = L.eg[ep & 1];
                for (int x = threadIdx.x; x < ow * oh; x += kThreads) {
                    const int i = t.r0 + x / ow, j = t.c0 + x % ow;
                    if (i >= t.r0 + kHalo && i < t.r1 - kHalo && j >= t.c0 + kHalo && j < t.c1 - kHalo) continue;
                    eg[(size_t)i * n + j] = S(i, j);
                }
                __syncthreads();
                if (threadIdx.x == 0) st_release(&sy->flag[blockIdx.x], ep);
            }
        }
        if (!ok) { status = CNV_TIMEOUT; break; }
        // ---- FP64 correction psi += e on own cells
        for (int x = threadIdx.x; x < ow * oh; x += kThreads) {
            const int i = t.r0 + x / ow, j = t.c0 + x % ow;
            L.psi[(size_t)i * n + j] += (double)S(i, j);
        }
        if (!grid_sync(sy, bar, ctl, L.timeout_ns, &s_ok)) { status = CNV_TIMEOUT; break; }
    }
    if (status == CNV_TIMEOUT) return;
    // answer -> red/black split layout for the velocity pass
    {
        const int ow = t.c1 - t.c0, oh = t.r1 - t.r0;
        for (int x = threadIdx.x; x < ow * oh; x += kThreads) {
            const int i = t.r0 + x / ow, j = t.c0 + x % ow;
            L.sor[(i + j) & 1][(size_t)i * L.pitch + (j >> 1)] = L.psi[(size_t)i * n + j];
        }
    }
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
    const size_t smem = mixed_smem_bytes(L.n, L.gx, L.gy);
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
