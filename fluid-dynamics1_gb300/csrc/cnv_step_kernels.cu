// cnv_step_kernels.cu -- the non-Poisson part of cnavier's time step on the GPU, as two fused
// passes around the Poisson solve.
//
//   k_pre   wall vorticity on the four edges                    src/main.c:298-320
//           + DX/DY/DX2/DY2 of w and the Euler update           src/main.c:323-344, src/fluiddyn.c:71-102
//           + the Poisson right-hand side (f = -w)              src/main.c:347-348
//   k_post  u = DY psi, v = -(DX psi)                           src/main.c:366-383
//           + continuity DX u + DY v, its max and min           src/main.c:387-408
//
// Every arithmetic operation uses the round-to-nearest intrinsics (__dadd_rn, __dmul_rn, ...),
// which the compiler never contracts into FMAs, in the reference's evaluation order, so these
// passes give the reference's values bit for bit. The dense Kronecker products of the
// reference become 7-tap bands summed from 0.0 in ascending column order (the skipped
// products are exact zeros). Velocity Dirichlet values (src/main.c:283-296) are applied on
// read: u and v keep the values the velocity pass wrote, as in the reference between steps.
//
// k_pre. One block per 32 x 32 tile. The block stages w on its tile plus the radius-3 halo of
// the order-6 stencils in shared memory; cells on the grid's edge hold the new wall vorticity
// there, which the block computes itself from u and v wherever its tile or halo touches an edge
// (so no block reads another block's wall values). Each thread then takes four cells of one
// column: the four derivatives from shared memory, u and v at the cell (coalesced global
// loads), the Euler update, and the writes: w_out, the right-hand side in the solver's split
// layout, and on edge cells the wall value into w_in (the reference's w after the wall loop,
// which the adjoint form keeps).
//
// k_post. Persistent and cooperative: every block loops over 32 x 32 tiles. Phase 1 stages psi
// on the tile plus halo (from the solver's split layout) and writes u, v and the row-major psi
// of the tile. A bounded grid barrier follows (continuity reads u and v of neighbouring tiles);
// phase 2 stages u and v on the tile plus halo and reduces DX u + DY v to max and min. The
// reduction keeps, among equal values, the one with the smallest row-major index, which is
// what the reference's sequential maxel/minel keep (so the sign of a zero extremum matches
// too). The last block to finish folds the blocks' partials and writes the step record.
#include <cfloat>
#include <climits>

#include "cnv_kernels.h"
#include "cnv_sor.cuh"
#include "cnv_stencil.cuh"
#include "cnv_sync.cuh"

namespace cnv {

template <>
__device__ __forceinline__ double band_mul<kMulInt>(double c, double x) {
    return mul_rn(c, x);
}

namespace {

// Which pipe multiplies the band coefficients in the passes' derivative products: the passes are
// bound by the FP64 pipe, and the exact integer multiply moves those multiplications to the
// integer pipes (the same bits). Measured on a GB300 (cnv_time_passes on a developed, smoothed-
// noise field; ms at 1024^2 / 2048^2): k_pre 0.162 / 0.544 with FP64 multiplies, 0.116 / 0.388
// with all 28 on the integer pipes; k_post 0.168 / 0.643 and 0.166 / 0.446. With the multiply's
// cheaper rounding step, all on the integer pipes: k_pre 0.112 / 0.372, k_post 0.137 / 0.439;
// half on each pipe (first derivatives on one, second derivatives or continuity on the other)
// ran 0.132-0.134 / 0.437-0.454 and 0.153-0.159 / 0.509-0.521.
constexpr int kPreD1 = kMulInt;      // k_pre: DX w, DY w
constexpr int kPreD2 = kMulInt;      // k_pre: DX2 w, DY2 w
constexpr int kPostVel = kMulInt;    // k_post: DY psi, DX psi
constexpr int kPostCont = kMulInt;   // k_post: DX u, DY v

constexpr int kTX = 32;                 // tile columns (one warp across)
// tile rows TY: 32 (each thread takes 4 cells of one column), or 8 on grids with fewer 32 x 32
// tiles than twice the SM count (one cell per thread, four times the blocks: a 256^2 grid has
// only 64 tiles of 32 x 32 for 152 SMs)
constexpr int kR = 3;                   // stencil radius (order 6; orders 2 and 4 use less)
constexpr int kSW = kTX + 2 * kR;       // staged row width
constexpr int kStepThreads = 256;       // 32 x 8: each thread takes 4 cells of one column
constexpr int kThreadRows = kStepThreads / kTX;  // 8 rows of threads
constexpr int kBandDoubles = (int)(sizeof(FdBands) / sizeof(double));

__device__ __forceinline__ double make_rhs(double f_ref, const StepArgs& a) {
    // src/poisson.c:247 multiplies dx*dx*dy*dy*f left to right: (((dx*dx)*dy)*dy)*f = c4*f
    double g = dmul(a.c4, f_ref);
    if (a.rhs_mode == 1) g = a.rhs_den_pow2 ? dmul(g, a.rhs_rden) : div_rn_const(g, a.rhs_div);
    else if (a.rhs_mode == 2) g = dmul(g, a.rhs_inv_h2);  // exact: 1/dx^2 is a power of two
    return g;
}

// the operator bands, staged in shared memory by the whole block
__device__ __forceinline__ void stage_bands(FdBands& sb, const FdBands* gb) {
    double* d = reinterpret_cast<double*>(&sb);
    const double* s = reinterpret_cast<const double*>(gb);
    for (int x = threadIdx.x; x < kBandDoubles; x += blockDim.x) d[x] = __ldg(s + x);
}

// w at edge cell (i, j) after the wall loops of src/main.c:311-320: DX v - DY u with the
// velocities' Dirichlet values (the corners get the same formula from both loops)
__device__ __forceinline__ double wall_value(const StepArgs& a, const FdBands& b, int i, int j) {
    const int n = a.n;
    const BoundaryValues bc = a.bc;
    const double* u = a.u;
    const double* v = a.v;
    auto U = [&](int r, int c) { return vel_bc(u, n, r, c, bc.u1, bc.u2, bc.u3, bc.u4); };
    auto V = [&](int r, int c) { return vel_bc(v, n, r, c, bc.v1, bc.v2, bc.v3, bc.v4); };
    const double dvdx = along_j(b.d1x, n, i, j, V);  // DX v
    const double dudy = along_i(b.d1y, n, i, j, U);  // DY u
    return dsub(dvdx, dudy);
}

__device__ __forceinline__ bool on_edge(int i, int j, int n) { return i == 0 || i == n - 1 || j == 0 || j == n - 1; }

// ----------------------------------------------------------------------------------- k_pre
template <int TY>
__global__ void __launch_bounds__(kStepThreads) k_pre(StepArgs a) {
    constexpr int kSH = TY + 2 * kR;  // staged rows
    if (a.ctrl->abort) return;
    __shared__ double sw[kSH * kSW];
    __shared__ FdBands sb;
    const int n = a.n;
    const int j0 = blockIdx.x * kTX, i0 = blockIdx.y * TY;
    stage_bands(sb, a.bands);
    __syncthreads();
    // w on the tile and halo; edge cells take the wall value
    const double* __restrict__ w = a.w_in;
    for (int x = threadIdx.x; x < kSH * kSW; x += kStepThreads) {
        const int r = x / kSW, c = x - r * kSW;
        const int i = i0 - kR + r, j = j0 - kR + c;
        double val = 0.0;
        if (i >= 0 && i < n && j >= 0 && j < n) val = on_edge(i, j, n) ? wall_value(a, sb, i, j) : w[(size_t)i * n + j];
        sw[x] = val;
    }
    __syncthreads();
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    const int j = j0 + tx;
    if (j >= n) return;
    auto W = [&](int r, int c) { return sw[(r - i0 + kR) * kSW + (c - j0 + kR)]; };
    const BoundaryValues bc = a.bc;
#pragma unroll 1
    for (int k = 0; k < TY / kThreadRows; ++k) {
        const int i = i0 + ty + k * kThreadRows;
        if (i >= n) break;
        const double wx = along_j<kPreD1>(sb.d1x, n, i, j, W);   // dwdx   = DX  w
        const double wy = along_i<kPreD1>(sb.d1y, n, i, j, W);   // dwdy   = DY  w
        const double wxx = along_j<kPreD2>(sb.d2x, n, i, j, W);  // d2wdx2 = DX2 w
        const double wyy = along_i<kPreD2>(sb.d2y, n, i, j, W);  // d2wdy2 = DY2 w
        const double ue = vel_bc(a.u, n, i, j, bc.u1, bc.u2, bc.u3, bc.u4);
        const double ve = vel_bc(a.v, n, i, j, bc.v1, bc.v2, bc.v3, bc.v4);
        const double w0 = W(i, j);
        // (-u*dwdx - v*dwdy + (1./Re)*(d2wdx2 + d2wdy2))*dt + w   (src/fluiddyn.c:98)
        const double conv = dsub(dmul(-ue, wx), dmul(ve, wy));
        const double diff = dmul(a.inv_re, dadd(wxx, wyy));
        const double wn = dadd(dmul(dadd(conv, diff), a.dt), w0);
        const size_t at = (size_t)i * n + j;
        a.w_out[at] = wn;
        if (on_edge(i, j, n)) {
            a.w_wall[at] = w0;  // the wall value, in place (src/main.c:311-320)
        } else if (a.rhs[0]) {  // no rhs: the direct solve reads w_out itself
            a.rhs[(i + j) & 1][(size_t)i * a.pitch + (j >> 1)] = make_rhs(-wn, a);  // f = -w (invsig)
        }
    }
}

// ---------------------------------------------------------------------------------- k_post
// Extremum with the reference's tie rule: among equal values the earliest (row-major) index.
struct Ext {
    double v;
    int at;  // row-major index; -1 for the start value (which every tie keeps)
};

__device__ __forceinline__ void take_max(Ext& a, double v, int at) {
    if (v > a.v || (v == a.v && at < a.at)) a = Ext{v, at};
}
__device__ __forceinline__ void take_min(Ext& a, double v, int at) {
    if (v < a.v || (v == a.v && at < a.at)) a = Ext{v, at};
}

__device__ __forceinline__ void warp_ext(Ext& mx, Ext& mn) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double xv = __shfl_xor_sync(0xffffffffu, mx.v, off);
        const int xa = __shfl_xor_sync(0xffffffffu, mx.at, off);
        const double nv = __shfl_xor_sync(0xffffffffu, mn.v, off);
        const int na = __shfl_xor_sync(0xffffffffu, mn.at, off);
        take_max(mx, xv, xa);
        take_min(mn, nv, na);
    }
}

template <int TY>
__global__ void __launch_bounds__(kStepThreads) k_post(StepArgs a, int continuity) {
    constexpr int kSH = TY + 2 * kR;  // staged rows
    if (a.ctrl->abort) return;  // stable for the whole launch: every block returns, or none
    __shared__ double sm[2 * kSH * kSW];  // phase 1: psi; phase 2: u and v
    __shared__ FdBands sb;
    __shared__ int s_ok;
    const int n = a.n;
    const int tiles_x = (n + kTX - 1) / kTX;
    const int tiles = tiles_x * ((n + TY - 1) / TY);
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    stage_bands(sb, a.bands);
    __syncthreads();

    // phase 1: u = DY psi, v = -(DX psi), psi row-major
    const double* r = a.sor[0];
    const double* b = a.sor[1];
    const int pitch = a.pitch;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int j0 = (tile % tiles_x) * kTX, i0 = (tile / tiles_x) * TY;
        for (int x = threadIdx.x; x < kSH * kSW; x += kStepThreads) {
            const int rr = x / kSW, c = x - rr * kSW;
            const int i = i0 - kR + rr, j = j0 - kR + c;
            sm[x] = (i >= 0 && i < n && j >= 0 && j < n) ? ((i + j) & 1 ? b : r)[(size_t)i * pitch + (j >> 1)] : 0.0;
        }
        __syncthreads();
        auto P = [&](int y, int c) { return sm[(y - i0 + kR) * kSW + (c - j0 + kR)]; };
        const int j = j0 + tx;
        if (j < n) {
#pragma unroll 1
            for (int k = 0; k < TY / kThreadRows; ++k) {
                const int i = i0 + ty + k * kThreadRows;
                if (i >= n) break;
                const double uu = along_i<kPostVel>(sb.d1y, n, i, j, P);   // DY psi
                const double vv = -along_j<kPostVel>(sb.d1x, n, i, j, P);  // -(DX psi)
                const size_t at = (size_t)i * n + j;
                a.u[at] = uu;
                a.v[at] = vv;
                a.psi[at] = P(i, j);
            }
        }
        __syncthreads();
    }
    if (!continuity) return;

    // bounded grid barrier: continuity reads the neighbouring tiles' u and v
    Ctrl* ctl = a.ctrl;
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&ctl->bar_count, 1u);
        s_ok = wait_geq(&ctl->bar_count, gridDim.x, ctl, a.timeout_ns) ? 1 : 0;
    }
    __syncthreads();
    if (!s_ok) return;  // timeout (status recorded) or another block's abort

    // phase 2: continuity DX u + DY v (the raw velocities the reference's continuity() reads)
    Ext mx{-DBL_MAX, -1}, mn{DBL_MAX, -1};  // maxel/minel start values, src/linearalg.c:478, :514
    double* su = sm;
    double* sv = sm + kSH * kSW;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int j0 = (tile % tiles_x) * kTX, i0 = (tile / tiles_x) * TY;
        for (int x = threadIdx.x; x < kSH * kSW; x += kStepThreads) {
            const int rr = x / kSW, c = x - rr * kSW;
            const int i = i0 - kR + rr, j = j0 - kR + c;
            const bool in = i >= 0 && i < n && j >= 0 && j < n;
            su[x] = in ? __ldcg(a.u + (size_t)i * n + j) : 0.0;  // written by other blocks: via L2
            sv[x] = in ? __ldcg(a.v + (size_t)i * n + j) : 0.0;
        }
        __syncthreads();
        auto U = [&](int y, int c) { return su[(y - i0 + kR) * kSW + (c - j0 + kR)]; };
        auto V = [&](int y, int c) { return sv[(y - i0 + kR) * kSW + (c - j0 + kR)]; };
        const int j = j0 + tx;
        if (j < n) {
#pragma unroll 1
            for (int k = 0; k < TY / kThreadRows; ++k) {
                const int i = i0 + ty + k * kThreadRows;
                if (i >= n) break;
                const double dudx = along_j<kPostCont>(sb.d1x, n, i, j, U);
                const double dvdy = along_i<kPostCont>(sb.d1y, n, i, j, V);
                const double c = dadd(dudx, dvdy);
                take_max(mx, c, i * n + j);
                take_min(mn, c, i * n + j);
            }
        }
        __syncthreads();
    }
    __shared__ Ext smx[kStepThreads / 32], smn[kStepThreads / 32];
    __shared__ bool last;
    warp_ext(mx, mn);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        smx[warp] = mx;
        smn[warp] = mn;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kStepThreads / 32; ++w) {
            take_max(mx, smx[w].v, smx[w].at);
            take_min(mn, smn[w].v, smn[w].at);
        }
        double* part = a.cont_partials + 4 * blockIdx.x;
        part[0] = mx.v;
        part[1] = (double)mx.at;
        part[2] = mn.v;
        part[3] = (double)mn.at;
        __threadfence();
        const unsigned t = atomicAdd(&ctl->cont_ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || warp != 0) return;
    // last block, first warp: fold the partials (each lane a stride of blocks, L2 loads issued
    // together), write this step's record, re-arm the barrier and ticket
    __threadfence();
    const double* cp = a.cont_partials;
    mx = Ext{-DBL_MAX, -1};
    mn = Ext{DBL_MAX, -1};
    for (int q = lane; q < (int)gridDim.x; q += 32) {
        const double2 hi = __ldcg(reinterpret_cast<const double2*>(cp + 4 * q));
        const double2 lo = __ldcg(reinterpret_cast<const double2*>(cp + 4 * q + 2));
        take_max(mx, hi.x, (int)hi.y);
        take_min(mn, lo.x, (int)lo.y);
    }
    warp_ext(mx, mn);
    if (lane != 0) return;
    ctl->cont_ticket = 0;
    ctl->bar_count = 0;  // every block passed the barrier before taking its ticket
    const int step = ctl->step;
    if (step < ctl->max_records) {
        StepRecord& rec = ctl->records[step];
        rec.iters = ctl->iters;
        rec.status = ctl->status;
        rec.err = ctl->err;
        rec.cont_max = mx.v;
        rec.cont_min = mn.v;
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

int tile_count(int n, int ty) { return ((n + kTX - 1) / kTX) * ((n + ty - 1) / ty); }

template <int TY>
cudaError_t launch_post_t(const StepArgs& a, bool continuity, cudaStream_t s) {
    int c = continuity ? 1 : 0;
    if (!continuity) {  // no barrier: one block per tile
        k_post<TY><<<tile_count(a.n, TY), kStepThreads, 0, s>>>(a, c);
        return cudaGetLastError();
    }
    // the grid barrier needs every block resident: a cooperative launch of at most post_grid blocks
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(a.cont_blocks);
    cfg.blockDim = dim3(kStepThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    StepArgs args = a;
    void* kargs[] = {&args, &c};
    return cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(&k_post<TY>), kargs);
}

}  // namespace

int step_tile_rows(int n, int device) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1) return 32;
    return tile_count(n, 32) < 2 * sms ? 8 : 32;
}

cudaError_t launch_pre(const StepArgs& a, cudaStream_t s) {
    if (a.tile_rows == 8)
        k_pre<8><<<dim3((a.n + kTX - 1) / kTX, (a.n + 7) / 8), kStepThreads, 0, s>>>(a);
    else
        k_pre<32><<<dim3((a.n + kTX - 1) / kTX, (a.n + 31) / 32), kStepThreads, 0, s>>>(a);
    return cudaGetLastError();
}

int post_grid(int n, int device, int tile_rows) {
    int sms = 0, per_sm = 0;
    const void* kern =
        tile_rows == 8 ? reinterpret_cast<const void*>(&k_post<8>) : reinterpret_cast<const void*>(&k_post<32>);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kStepThreads, 0) != cudaSuccess || per_sm < 1)
        return 0;
    // every block the same number of tiles: with more tiles than resident blocks, a grid of all
    // resident blocks would leave some with one tile more than others in both phases
    const int tiles = tile_count(n, tile_rows == 8 ? 8 : 32), resident = sms * per_sm;
    const int per_block = (tiles + resident - 1) / resident;
    return (tiles + per_block - 1) / per_block;
}

cudaError_t launch_post(const StepArgs& a, bool continuity, cudaStream_t s) {
    return a.tile_rows == 8 ? launch_post_t<8>(a, continuity, s) : launch_post_t<32>(a, continuity, s);
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
