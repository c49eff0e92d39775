// cnv_poisson.cu -- persistent red-black Poisson solver for the streamfunction.
//
// Restates poisson_SOR() / poisson() of src/poisson.c (:111-173, :62-109) with the red-black
// ordering of the OPENMP_ENABLED build (:239-261), and a true Jacobi sweep
// (src/cuda_kernels.cu:229-246), as ONE cooperative kernel that runs every sweep of a solve:
//
//   for k in 0 .. itmax-1:
//       red half-sweep  (cells with (i+j) even; reads black neighbours)
//       grid barrier
//       black half-sweep (reads the new red values), |psi_new - psi_old| summed per block
//       grid barrier
//       e = sum of the block partials in a fixed order (every block computes the same value)
//       stop when e < tol                                       (src/poisson.c:272-278)
//
// psi lives in the red/black split layout, so each half-sweep streams unit-stride rows: a red
// cell (i, j) at R[i][j>>1] has its black neighbours at B[i+-1][j>>1], B[i][(j-1)>>1] and
// B[i][(j+1)>>1]. Boundary cells are never written (psi = 0 Dirichlet, the reference's zero
// initial matrix). Each block owns a contiguous range of the interior, the same range for both
// colours, so the per-block partial sums, and with them the stop decision, are reproducible.
//
// Arithmetic: Arith::kExact evaluates the reference's point update in its order with
// round-to-nearest intrinsics (no FMA contraction), so psi is bitwise the reference's; the
// division by 2*(dx^2+dy^2) is a multiplication when that constant is a power of two (exact)
// and __ddiv_rn otherwise. Arith::kFma uses the algebraically equal form
//   psi_new = psi_old + beta * (wy*(up+dn) + wx*(rt+lt) - q - psi_old)
// with q = c4*f/den precomputed, in 7 FP64 operations per point instead of 12.
//
// The grid barrier is a counter that every block increments once per barrier; a block waits
// until the counter reaches (barrier index) x (grid size). Waits are bounded by
// PoissonParams::timeout_ns (globaltimer); a block that gives up records CNV_TIMEOUT and
// leaves, so no launch can hang.
#include <cfloat>

#include "cnv_kernels.h"

namespace cnv {
namespace {

constexpr int kThreads = 512;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ long long globaltimer_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Returns false if the wait timed out (the caller must then leave the kernel).
__device__ __forceinline__ bool grid_barrier(unsigned* count, unsigned& epoch, long long timeout_ns,
                                             int* s_ok) {
    __syncthreads();
    ++epoch;
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(count, 1u);
        const unsigned target = epoch * gridDim.x;
        const long long t0 = globaltimer_ns();
        int ok = 1;
        while ((int)(ld_acquire_u32(count) - target) < 0) {
            if (globaltimer_ns() - t0 > timeout_ns) {
                ok = 0;
                break;
            }
        }
        __threadfence();
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// Deterministic block sum: xor-butterfly within each warp (all lanes end with the same value),
// then warp 0 adds the per-warp values in warp order.
__device__ __forceinline__ double block_sum(double x, double* s_warp) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) s_warp[warp] = x;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_warp[w];
    return t;  // valid in thread 0
}

// Fixed-order sum of the grid's partials; the result is broadcast to the whole block.
__device__ __forceinline__ double grid_sum(const double* partials, double* s_bcast) {
    if (threadIdx.x < 32) {
        double x = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) x += __ldcg(partials + b);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
        if (threadIdx.x == 0) *s_bcast = x;
    }
    __syncthreads();
    const double r = *s_bcast;
    __syncthreads();
    return r;
}

template <Arith A, int KIND>
__device__ __forceinline__ double point_update(const PoissonParams& p, double up, double dn, double rt,
                                               double lt, double g, double old, double& acc) {
    if (A == Arith::kExact) {
        // beta*(dy*dy*(up+dn) + dx*dx*(rt+lt) - dx*dx*dy*dy*f) / (2*(dx*dx+dy*dy)) + (1-beta)*u0
        // (src/poisson.c:247); g = dx*dx*dy*dy*f was formed by the transport pass.
        const double num = __dsub_rn(__dadd_rn(__dmul_rn(p.dy2, __dadd_rn(up, dn)),
                                               __dmul_rn(p.dx2, __dadd_rn(rt, lt))), g);
        double nw;
        if (KIND == CNV_POISSON_SOR) {
            const double bn = __dmul_rn(p.beta, num);
            const double q = p.den_pow2 ? __dmul_rn(bn, p.rden) : __ddiv_rn(bn, p.den);
            nw = __dadd_rn(q, __dmul_rn(p.omb, old));
        } else {  // Gauss-Seidel and Jacobi: (num) / den, src/poisson.c:84
            nw = p.den_pow2 ? __dmul_rn(num, p.rden) : __ddiv_rn(num, p.den);
        }
        acc += fabs(__dsub_rn(nw, old));
        return nw;
    } else {
        // g = c4*f/den here; t = GS value - old; new = old + beta*t; |new - old| = beta*|t|
        const double gs = fma(p.wy, up + dn, fma(p.wx, rt + lt, -g));
        const double t = gs - old;
        acc += fabs(t);
        return KIND == CNV_POISSON_SOR ? fma(p.beta, t, old) : gs;
    }
}

// One colour of a red-black sweep over this block's range [beg, end) of the flattened interior
// index (i-1)*W + m. S = array of the colour being updated, O = the other colour.
template <Arith A, int KIND, int C>
__device__ __forceinline__ void half_sweep(const PoissonParams& p, double* __restrict__ S,
                                           const double* __restrict__ O, const double* __restrict__ rhs,
                                           int beg, int end, double& acc) {
    const int n = p.n, W = (n + 1) >> 1, P = p.pitch;
    for (int idx = beg + (int)threadIdx.x; idx < end; idx += kThreads) {
        const int i = 1 + idx / W;
        const int m = idx - (i - 1) * W;
        const int j = 2 * m + ((i + C) & 1);
        if (j < 1 || j > n - 2) continue;
        const size_t row = (size_t)i * P;
        const double old = S[row + m];
        const double up = __ldcg(O + row + P + m);
        const double dn = __ldcg(O + row - P + m);
        const double lt = __ldcg(O + row + ((j - 1) >> 1));
        const double rt = __ldcg(O + row + ((j + 1) >> 1));
        S[row + m] = point_update<A, KIND>(p, up, dn, rt, lt, rhs[row + m], old, acc);
    }
}

// Jacobi: both colours from the old values, written to the other buffer pair.
template <Arith A>
__device__ __forceinline__ void jacobi_sweep(const PoissonParams& p, const double* __restrict__ R,
                                             const double* __restrict__ B, double* __restrict__ Rn,
                                             double* __restrict__ Bn, const double* __restrict__ rhsR,
                                             const double* __restrict__ rhsB, int beg, int end,
                                             double& acc) {
    const int n = p.n, W = (n + 1) >> 1, P = p.pitch;
    for (int idx = beg + (int)threadIdx.x; idx < end; idx += kThreads) {
        const int i = 1 + idx / W;
        const int m = idx - (i - 1) * W;
        const size_t row = (size_t)i * P;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const int j = 2 * m + ((i + c) & 1);
            if (j < 1 || j > n - 2) continue;
            const double* S = c ? B : R;
            const double* O = c ? R : B;
            double* D = c ? Bn : Rn;
            const double* rhs = c ? rhsB : rhsR;
            const double old = __ldcg(S + row + m);
            const double up = __ldcg(O + row + P + m);
            const double dn = __ldcg(O + row - P + m);
            const double lt = __ldcg(O + row + ((j - 1) >> 1));
            const double rt = __ldcg(O + row + ((j + 1) >> 1));
            D[row + m] = point_update<A, CNV_POISSON_JACOBI>(p, up, dn, rt, lt, rhs[row + m], old, acc);
        }
    }
}

template <Arith A, int KIND>
__global__ void __launch_bounds__(kThreads) k_poisson(PoissonLaunch L) {
    Ctrl* ctl = L.ctrl;
    if (ctl->abort) return;  // read once per block before any write: uniform across the grid
    const PoissonParams p = L.p;
    __shared__ double s_warp[kThreads / 32];
    __shared__ double s_bcast;
    __shared__ int s_ok;
    const int W = (p.n + 1) >> 1;
    const int total = (p.n - 2) * W;
    const int beg = (int)((long long)total * blockIdx.x / gridDim.x);
    const int end = (int)((long long)total * (blockIdx.x + 1) / gridDim.x);
    double* R = L.sor[0];
    double* B = L.sor[1];
    double* Ra = L.alt[0];
    double* Ba = L.alt[1];
    unsigned epoch = 0;
    int status = CNV_NOT_CONVERGED, k = 0;
    double etot = 0.0;
    const double escale = (A == Arith::kFma && KIND == CNV_POISSON_SOR) ? p.beta : 1.0;
    for (k = 0; k < p.itmax; ++k) {
        double acc = 0.0;
        if (KIND == CNV_POISSON_JACOBI) {
            jacobi_sweep<A>(p, R, B, Ra, Ba, L.rhs[0], L.rhs[1], beg, end, acc);
        } else {
            half_sweep<A, KIND, 0>(p, R, B, L.rhs[0], beg, end, acc);
            if (!grid_barrier(&ctl->bar_count, epoch, p.timeout_ns, &s_ok)) { status = CNV_TIMEOUT; break; }
            half_sweep<A, KIND, 1>(p, B, R, L.rhs[1], beg, end, acc);
        }
        const double bsum = block_sum(acc, s_warp);
        if (threadIdx.x == 0) L.partials[(k & 1) * gridDim.x + blockIdx.x] = bsum;
        if (!grid_barrier(&ctl->bar_count, epoch, p.timeout_ns, &s_ok)) { status = CNV_TIMEOUT; break; }
        etot = grid_sum(L.partials + (k & 1) * gridDim.x, &s_bcast) * escale;
        if (KIND == CNV_POISSON_JACOBI) {  // the new iterate becomes the current one
            double* t0 = R; R = Ra; Ra = t0;
            double* t1 = B; B = Ba; Ba = t1;
        }
        if (!isfinite(etot)) { status = CNV_NONFINITE; break; }
        if (etot < p.tol) { status = CNV_OK; break; }
    }
    if (KIND == CNV_POISSON_JACOBI && R != L.sor[0] && status != CNV_TIMEOUT) {
        // the answer sits in the alt pair: copy this block's range back (own cells only)
        const int n = p.n, P = p.pitch;
        for (int idx = beg + (int)threadIdx.x; idx < end; idx += kThreads) {
            const int i = 1 + idx / W;
            const int m = idx - (i - 1) * W;
            const size_t q = (size_t)i * P + m;
            L.sor[0][q] = R[q];
            L.sor[1][q] = B[q];
        }
        (void)n;
    }
    if (status == CNV_TIMEOUT) {
        if (threadIdx.x == 0) {
            atomicExch(&ctl->status, CNV_TIMEOUT);
            atomicExch(&ctl->abort, 1);
        }
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const int iters = status == CNV_NOT_CONVERGED ? p.itmax : k;
        ctl->iters = iters;
        ctl->err = etot;
        ctl->status = status;
        ctl->sweeps += (status == CNV_NOT_CONVERGED ? p.itmax : k + 1);
        const int step = ctl->step;
        if (step < ctl->max_records) {
            StepRecord& r = ctl->records[step];
            r.iters = iters;
            r.status = status;
            r.err = etot;
            r.cont_max = 0.0;
            r.cont_min = 0.0;
        }
        if (status != CNV_OK) ctl->abort = 1;
    }
}

template <Arith A, int KIND>
const void* kernel_ptr() {
    return reinterpret_cast<const void*>(&k_poisson<A, KIND>);
}

}  // namespace

int poisson_threads() { return kThreads; }

const void* poisson_kernel_ptr(Arith a, int kind) {
    if (a == Arith::kExact) {
        if (kind == CNV_POISSON_SOR) return kernel_ptr<Arith::kExact, CNV_POISSON_SOR>();
        if (kind == CNV_POISSON_GS) return kernel_ptr<Arith::kExact, CNV_POISSON_GS>();
        return kernel_ptr<Arith::kExact, CNV_POISSON_JACOBI>();
    }
    if (kind == CNV_POISSON_SOR) return kernel_ptr<Arith::kFma, CNV_POISSON_SOR>();
    if (kind == CNV_POISSON_GS) return kernel_ptr<Arith::kFma, CNV_POISSON_GS>();
    return kernel_ptr<Arith::kFma, CNV_POISSON_JACOBI>();
}

cudaError_t launch_poisson(const PoissonLaunch& L, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(&L.ctrl->bar_count, 0, sizeof(unsigned), s);
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
    return cudaLaunchKernelExC(&cfg, poisson_kernel_ptr(L.p.arith, L.p.kind), args);
}

}  // namespace cnv
