// cnv_step_kernels.cu -- the non-Poisson part of cnavier's time step on the GPU.
//
//   wall pass       wall vorticity on the four edges          src/main.c:298-320
//   transport pass  DX/DY/DX2/DY2 of w + Euler update          src/main.c:323-344,
//                   + Poisson right-hand side (f = -w)        src/fluiddyn.c:71-102, :347-348
//   velocity pass   u = DY psi, v = -(DX psi)                  src/main.c:366-383
//   continuity pass DX u + DY v, max and min                   src/main.c:387-408
//
// Every arithmetic operation uses the round-to-nearest intrinsics (__dadd_rn, __dmul_rn, ...),
// which the compiler never contracts into FMAs, in the reference's evaluation order, so these
// passes give the reference's values bit for bit. The dense Kronecker products of the
// reference become 7-tap bands summed from 0.0 in ascending column order (the skipped
// products are exact zeros). Velocity Dirichlet values (src/main.c:283-296) are applied on
// read: u and v keep the values the velocity pass wrote, as in the reference between steps.
#include <cfloat>

#include "cnv_kernels.h"
#include "cnv_stencil.cuh"

namespace cnv {
namespace {

__device__ __forceinline__ double make_rhs(double f_ref, const StepArgs& a) {
    // src/poisson.c:247 multiplies dx*dx*dy*dy*f left to right: (((dx*dx)*dy)*dy)*f = c4*f
    double g = dmul(a.c4, f_ref);
    if (a.rhs_mode == 1) g = a.rhs_den_pow2 ? dmul(g, a.rhs_rden) : __ddiv_rn(g, a.rhs_den);
    else if (a.rhs_mode == 2) g = dmul(g, a.rhs_inv_h2);  // exact: 1/dx^2 is a power of two
    return g;
}

// ---------------------------------------------------------------------------- wall pass
__global__ void k_wall(StepArgs a) {
    if (a.ctrl->abort) return;
    const int n = a.n;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= 4 * n) return;
    const int side = s / n, t = s - side * n;
    const int i = side == 0 ? 0 : side == 1 ? n - 1 : t;
    const int j = side == 2 ? 0 : side == 3 ? n - 1 : t;
    const BoundaryValues bc = a.bc;
    const double* u = a.u;
    const double* v = a.v;
    auto U = [&](int r, int c) { return vel_bc(u, n, r, c, bc.u1, bc.u2, bc.u3, bc.u4); };
    auto V = [&](int r, int c) { return vel_bc(v, n, r, c, bc.v1, bc.v2, bc.v3, bc.v4); };
    const double dvdx = along_j(a.bands->d1x, n, i, j, V);  // DX v
    const double dudy = along_i(a.bands->d1y, n, i, j, U);  // DY u
    a.w_wall[(size_t)i * n + j] = dsub(dvdx, dudy);
}

// ----------------------------------------------------------------------- transport pass
__global__ void k_transport(StepArgs a) {
    if (a.ctrl->abort) return;
    const int n = a.n;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n || j >= n) return;
    const double* w = a.w_in;
    auto W = [&](int r, int c) { return w[(size_t)r * n + c]; };
    const double wx = along_j(a.bands->d1x, n, i, j, W);   // dwdx   = DX  w
    const double wy = along_i(a.bands->d1y, n, i, j, W);   // dwdy   = DY  w
    const double wxx = along_j(a.bands->d2x, n, i, j, W);  // d2wdx2 = DX2 w
    const double wyy = along_i(a.bands->d2y, n, i, j, W);  // d2wdy2 = DY2 w
    const BoundaryValues bc = a.bc;
    const double ue = vel_bc(a.u, n, i, j, bc.u1, bc.u2, bc.u3, bc.u4);
    const double ve = vel_bc(a.v, n, i, j, bc.v1, bc.v2, bc.v3, bc.v4);
    const double w0 = w[(size_t)i * n + j];
    // (-u*dwdx - v*dwdy + (1./Re)*(d2wdx2 + d2wdy2))*dt + w   (src/fluiddyn.c:98)
    const double conv = dsub(dmul(-ue, wx), dmul(ve, wy));
    const double diff = dmul(a.inv_re, dadd(wxx, wyy));
    const double wn = dadd(dmul(dadd(conv, diff), a.dt), w0);
    a.w_out[(size_t)i * n + j] = wn;
    if (a.rhs[0] && i > 0 && i < n - 1 && j > 0 && j < n - 1) {  // no rhs: direct solve reads w_out
        const int c = (i + j) & 1;
        a.rhs[c][(size_t)i * a.pitch + (j >> 1)] = make_rhs(-wn, a);  // f = -w (invsig)
    }
}

// ------------------------------------------------------------------------ velocity pass
__global__ void k_velocity(StepArgs a) {
    if (a.ctrl->abort) return;
    const int n = a.n;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n || j >= n) return;
    const double* r = a.sor[0];
    const double* b = a.sor[1];
    const int pitch = a.pitch;
    auto P = [&](int y, int x) { return ((y + x) & 1 ? b : r)[(size_t)y * pitch + (x >> 1)]; };
    const double uu = along_i(a.bands->d1y, n, i, j, P);   // DY psi
    const double vv = -along_j(a.bands->d1x, n, i, j, P);  // -(DX psi)
    const size_t k = (size_t)i * n + j;
    a.u[k] = uu;
    a.v[k] = vv;
    a.psi[k] = P(i, j);
}

// ---------------------------------------------------------------------- continuity pass
constexpr int kContThreads = 256;

__device__ __forceinline__ double gmax(double a, double b) { return b > a ? b : a; }
__device__ __forceinline__ double gmin(double a, double b) { return b < a ? b : a; }

__global__ void __launch_bounds__(kContThreads) k_continuity(StepArgs a) {
    if (a.ctrl->abort) return;
    const int n = a.n;
    const long long total = (long long)n * n;
    double mx = -DBL_MAX, mn = DBL_MAX;  // maxel/minel start values, src/linearalg.c:478, :514
    const double* u = a.u;
    const double* v = a.v;
    auto U = [&](int r, int c) { return u[(size_t)r * n + c]; };
    auto V = [&](int r, int c) { return v[(size_t)r * n + c]; };
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / n), j = (int)(k - (long long)i * n);
        const double dudx = along_j(a.bands->d1x, n, i, j, U);
        const double dvdy = along_i(a.bands->d1y, n, i, j, V);
        const double c = dadd(dudx, dvdy);
        mx = gmax(mx, c);
        mn = gmin(mn, c);
    }
    __shared__ double smx[kContThreads / 32], smn[kContThreads / 32];
    __shared__ bool last;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        mx = gmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        mn = gmin(mn, __shfl_xor_sync(0xffffffffu, mn, off));
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        smx[warp] = mx;
        smn[warp] = mn;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kContThreads / 32; ++w) {
            mx = gmax(mx, smx[w]);
            mn = gmin(mn, smn[w]);
        }
        a.cont_partials[2 * blockIdx.x] = mx;
        a.cont_partials[2 * blockIdx.x + 1] = mn;
        __threadfence();
        const unsigned t = atomicAdd(&a.ctrl->cont_ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    // last block: fold the partials, write this step's record
    __threadfence();
    const volatile double* cp = a.cont_partials;
    mx = -DBL_MAX;
    mn = DBL_MAX;
    for (int b = 0; b < (int)gridDim.x; ++b) {
        mx = gmax(mx, cp[2 * b]);
        mn = gmin(mn, cp[2 * b + 1]);
    }
    Ctrl* ctl = a.ctrl;
    ctl->cont_ticket = 0;
    const int step = ctl->step;
    if (step < ctl->max_records) {
        StepRecord& r = ctl->records[step];
        r.iters = ctl->iters;
        r.status = ctl->status;
        r.err = ctl->err;
        r.cont_max = mx;
        r.cont_min = mn;
    }
    ctl->step = step + 1;
}

// --------------------------------------------------------------------------- utilities
__global__ void k_to_split(const double* f, double* r, double* b, StepArgs a) {
    const int n = a.n;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n || j >= n) return;
    const double g = (i > 0 && i < n - 1 && j > 0 && j < n - 1) ? make_rhs(f[(size_t)i * n + j], a) : 0.0;
    ((i + j) & 1 ? b : r)[(size_t)i * a.pitch + (j >> 1)] = g;
}

__global__ void k_from_split(const double* r, const double* b, double* f, int n, int pitch) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n || j >= n) return;
    f[(size_t)i * n + j] = ((i + j) & 1 ? b : r)[(size_t)i * pitch + (j >> 1)];
}

__global__ void k_nonfinite(const double* x, long long count, int* flag) {
    int bad = 0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
         k += (long long)gridDim.x * blockDim.x)
        bad |= !isfinite(x[k]);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

dim3 grid2d(int n, dim3 blk) { return dim3((n + blk.x - 1) / blk.x, (n + blk.y - 1) / blk.y); }

}  // namespace

cudaError_t launch_wall(const StepArgs& a, cudaStream_t s) {
    const int threads = 128;
    k_wall<<<(4 * a.n + threads - 1) / threads, threads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_transport(const StepArgs& a, cudaStream_t s) {
    const dim3 blk(32, 8);
    k_transport<<<grid2d(a.n, blk), blk, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_velocity(const StepArgs& a, cudaStream_t s) {
    const dim3 blk(32, 8);
    k_velocity<<<grid2d(a.n, blk), blk, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_continuity(const StepArgs& a, cudaStream_t s) {
    k_continuity<<<a.cont_blocks, kContThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_to_split(const double* f, double* r, double* b, const StepArgs& a, cudaStream_t s) {
    const dim3 blk(32, 8);
    k_to_split<<<grid2d(a.n, blk), blk, 0, s>>>(f, r, b, a);
    return cudaGetLastError();
}

cudaError_t launch_from_split(const double* r, const double* b, double* f, int n, int pitch, cudaStream_t s) {
    const dim3 blk(32, 8);
    k_from_split<<<grid2d(n, blk), blk, 0, s>>>(r, b, f, n, pitch);
    return cudaGetLastError();
}

cudaError_t launch_nonfinite_scan(const double* x, long long count, int* flag, cudaStream_t s) {
    k_nonfinite<<<304, 256, 0, s>>>(x, count, flag);
    return cudaGetLastError();
}

}  // namespace cnv
