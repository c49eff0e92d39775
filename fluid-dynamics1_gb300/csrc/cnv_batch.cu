// cnv_batch.cu -- many independent cavities (uneven grid size, Re and lid speed) advanced by one
// persistent launch.
//
// Work unit: one cavity for `nsteps` time steps. Cavities are independent, so a block takes a
// cavity from a queue (largest estimated cost first), integrates it for all the steps of the
// call with no synchronisation beyond its own __syncthreads(), and takes the next. Each step is
// the reference's loop body (src/main.c:283-395) with the same device arithmetic as the
// single-cavity path (reference rounding for the wall, transport, velocity and continuity
// passes) and the mixed-precision Poisson solve of cnv_mixed.cu: FP32 red-black SOR sweeps inside
// FP64 defect correction to a relative FP64 residual. The FP32 correction lives in shared memory
// when the cavity fits (together with its right-hand side when both fit), in the cavity's
// global arrays otherwise.
//
// Launch shape (threads per block, blocks per SM) is picked by an autotuner that times one step
// of each candidate from the initial state (cnv_batch_tune). The launch, with its queue reset, is
// captured in a CUDA graph; the step count is read from device memory so one graph serves every
// call.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "cnv_kernels.h"
#include "cnv_stencil.cuh"

namespace cnv {

struct CavityDesc {
    int n, pitch;       // grid size; split-layout pitch (doubles/floats per row)
    int spitch;         // split-layout pitch of the shared-memory tile (floats per row)
    int smem_mode;      // 0: e and R/den in global memory, 1: e in shared, 2: both in shared
    int inner;          // FP32 sweeps per correction
    int cur;            // current vorticity buffer
    double inv_re, dt, beta, c4, dx2, dy2, den, rden;
    BoundaryValues bc;
    const FdBands* bands;
    double* w[2];
    double* u;
    double* v;
    double* psi_rm;     // row-major psi (output)
    double* psi[2];     // split layout, FP64 iterate
    double* g[2];       // split layout, c4*f
    float* e[2];        // split layout, FP32 correction (global mode)
    float* rq[2];       // split layout, FP32 R/den (global mode)
    StepRecord last;    // record of the cavity's last step
    long long sweeps;   // FP32 sweeps done in the last call
    int steps_done;     // steps completed in the last call
    int pad;
};

struct BatchLaunch {
    CavityDesc* cav;
    const int* order;   // processing order (largest cost first)
    int* queue;         // next index into order (zeroed before each launch)
    const int* nsteps;  // steps per cavity for this call (device memory)
    int count;
    int max_outer;
    double rtol;
    int warm;           // start each step's solve from the previous psi (mixed_warm_start)
    int smem_floats;    // dynamic shared memory available to a block (floats)
};

namespace {

constexpr int kMaxBatchThreads = 1024;

__device__ __forceinline__ int floor_half(int j) { return j >= 0 ? j / 2 : -((1 - j) / 2); }

// Block-wide sum of a double (deterministic: xor butterfly, then warps in order).
__device__ double block_sum(double x, double* s_red) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) s_red[warp] = x;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_red[w];
    __syncthreads();
    return t;
}

__device__ void block_minmax(double& mx, double& mn, double* s_red) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double a = __shfl_xor_sync(0xffffffffu, mx, off);
        const double b = __shfl_xor_sync(0xffffffffu, mn, off);
        mx = a > mx ? a : mx;
        mn = b < mn ? b : mn;
    }
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_red[warp] = mx;
        s_red[32 + warp] = mn;
    }
    __syncthreads();
    mx = -DBL_MAX;
    mn = DBL_MAX;
    for (int w = 0; w < nw; ++w) {
        mx = s_red[w] > mx ? s_red[w] : mx;
        mn = s_red[32 + w] < mn ? s_red[32 + w] : mn;
    }
    __syncthreads();
}

// FP32 red-black SOR half-sweep of colour c over the interior, split layout with row pitch ep
// for e and rp for R/den.
__device__ void batch_half_sweep(float* __restrict__ ec, const float* __restrict__ eo, const float* __restrict__ rq,
                                 int n, int ep, int rp, int c, float wx, float wy, float beta) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int i = 1 + warp; i < n - 1; i += nw) {
        const int q = (i + c) & 1;
        const int mlo = floor_half(1 - q + 1), mhi = floor_half(n - 2 - q);
        const int row = i * ep;
        const float* rrow = rq + (size_t)i * rp;
        for (int m = mlo + lane; m <= mhi; m += 32) {
            const float up = eo[row + ep + m], dn = eo[row - ep + m];
            const float lt = eo[row + m - 1 + q], rt = eo[row + m + q];
            const float me = ec[row + m];
            const float gs = fmaf(wy, up + dn, fmaf(wx, lt + rt, -rrow[m]));
            ec[row + m] = fmaf(beta, gs - me, me);
        }
    }
}

// One time step of one cavity by the whole block. Returns the step's status.
__device__ int batch_step(CavityDesc& C, float* smem, int max_outer, double rtol, bool warm, double* s_red) {
    const int n = C.n, P = C.pitch;
    const int tid = threadIdx.x, nt = blockDim.x;
    double* w_in = C.w[C.cur];
    double* w_out = C.w[C.cur ^ 1];
    const BoundaryValues bc = C.bc;
    const FdBands* B = C.bands;

    // wall vorticity on the four edges (src/main.c:298-320), in place on w_in
    for (int s = tid; s < 4 * n; s += nt) {
        const int side = s / n, t = s - side * n;
        const int i = side == 0 ? 0 : side == 1 ? n - 1 : t;
        const int j = side == 2 ? 0 : side == 3 ? n - 1 : t;
        auto U = [&](int r, int cc) { return vel_bc(C.u, n, r, cc, bc.u1, bc.u2, bc.u3, bc.u4); };
        auto V = [&](int r, int cc) { return vel_bc(C.v, n, r, cc, bc.v1, bc.v2, bc.v3, bc.v4); };
        w_in[(size_t)i * n + j] = dsub(along_j(B->d1x, n, i, j, V), along_i(B->d1y, n, i, j, U));
    }
    __syncthreads();
    // transport: derivatives of w and the Euler update (src/fluiddyn.c:98); g = c4 * (-w)
    for (int k = tid; k < n * n; k += nt) {
        const int i = k / n, j = k - (k / n) * n;
        auto W = [&](int r, int cc) { return w_in[(size_t)r * n + cc]; };
        const double wx = along_j(B->d1x, n, i, j, W), wy = along_i(B->d1y, n, i, j, W);
        const double wxx = along_j(B->d2x, n, i, j, W), wyy = along_i(B->d2y, n, i, j, W);
        const double ue = vel_bc(C.u, n, i, j, bc.u1, bc.u2, bc.u3, bc.u4);
        const double ve = vel_bc(C.v, n, i, j, bc.v1, bc.v2, bc.v3, bc.v4);
        const double conv = dsub(dmul(-ue, wx), dmul(ve, wy));
        const double wn = dadd(dmul(dadd(conv, dmul(C.inv_re, dadd(wxx, wyy))), C.dt), w_in[k]);
        w_out[k] = wn;
        if (i > 0 && i < n - 1 && j > 0 && j < n - 1)
            C.g[(i + j) & 1][(size_t)i * P + (j >> 1)] = dmul(C.c4, -wn);
    }
    // psi = 0 (zero start; zero Dirichlet edge), or the previous step's psi (warm start)
    if (!warm)
        for (int k = tid; k < 2 * n * P; k += nt) (k < n * P ? C.psi[0] : C.psi[1])[k < n * P ? k : k - n * P] = 0.0;
    __syncthreads();

    // mixed-precision Poisson solve (cnv_mixed.cu's scheme, whole cavity in one block)
    const int sp = C.spitch;
    const int eplane = C.smem_mode >= 1 ? n * sp : 0;
    float* e_s[2] = {smem, smem + eplane};
    float* rq_s[2] = {smem + 2 * eplane, smem + 3 * eplane};
    float* ec[2] = {C.smem_mode >= 1 ? e_s[0] : C.e[0], C.smem_mode >= 1 ? e_s[1] : C.e[1]};
    const int ep = C.smem_mode >= 1 ? sp : P;
    float* rqc[2] = {C.smem_mode == 2 ? rq_s[0] : C.rq[0], C.smem_mode == 2 ? rq_s[1] : C.rq[1]};
    const int rp = C.smem_mode == 2 ? sp : P;
    const float wxf = (float)(C.dx2 / C.den), wyf = (float)(C.dy2 / C.den), betaf = (float)C.beta;
    double rel = 0.0, gnorm = 0.0;
    int outer = 0, status = CNV_NOT_CONVERGED;
    long long sweeps = 0;
    for (outer = 0;; ++outer) {
        double rr = 0.0, gg = 0.0;
        for (int k = tid; k < n * n; k += nt) {
            const int i = k / n, j = k - (k / n) * n;
            if (i == 0 || i == n - 1 || j == 0 || j == n - 1) continue;
            const int c = (i + j) & 1, q = (i + c) & 1, m = j >> 1;
            const double* pc = C.psi[c];
            const double* po = C.psi[c ^ 1];
            const size_t kk = (size_t)i * P + m;
            const double g = C.g[c][kk];
            const double R = poisson_defect(C.dy2, C.dx2, C.den, po[kk + P], po[kk - P], po[kk - 1 + q], po[kk + q],
                                            pc[kk], g);
            rr = fma(R, R, rr);
            if (outer == 0) gg = fma(g, g, gg);
            rqc[c][(size_t)i * rp + m] = (float)(R * C.rden);
        }
        rr = block_sum(rr, s_red);
        if (outer == 0) gnorm = sqrt(block_sum(gg, s_red));
        rel = gnorm > 0 ? sqrt(rr) / gnorm : sqrt(rr);
        if (!isfinite(rel)) { status = CNV_NONFINITE; break; }
        if (rel <= rtol) { status = CNV_OK; break; }
        if (outer >= max_outer) break;
        // e = 0 on the whole split plane (edges included), then the FP32 sweeps
        for (int k = tid; k < 2 * n * ep; k += nt) (k < n * ep ? ec[0] : ec[1])[k < n * ep ? k : k - n * ep] = 0.0f;
        __syncthreads();
        for (int s = 0; s < 2 * C.inner; ++s) {
            const int c = s & 1;
            batch_half_sweep(ec[c], ec[c ^ 1], rqc[c], n, ep, rp, c, wxf, wyf, betaf);
            __syncthreads();
        }
        sweeps += C.inner;
        // psi += e (FP64)
        for (int k = tid; k < n * n; k += nt) {
            const int i = k / n, j = k - (k / n) * n;
            if (i == 0 || i == n - 1 || j == 0 || j == n - 1) continue;
            const int c = (i + j) & 1;
            C.psi[c][(size_t)i * P + (j >> 1)] += (double)ec[c][(size_t)i * ep + (j >> 1)];
        }
        __syncthreads();
    }

    // velocity u = DY psi, v = -(DX psi) (src/main.c:366-383), row-major psi for output
    auto PS = [&](int y, int x) { return C.psi[(y + x) & 1][(size_t)y * P + (x >> 1)]; };
    for (int k = tid; k < n * n; k += nt) {
        const int i = k / n, j = k - (k / n) * n;
        C.u[k] = along_i(B->d1y, n, i, j, PS);
        C.v[k] = -along_j(B->d1x, n, i, j, PS);
        C.psi_rm[k] = PS(i, j);
    }
    __syncthreads();
    // continuity DX u + DY v, max and min (src/main.c:387-408)
    double mx = -DBL_MAX, mn = DBL_MAX;
    auto Uf = [&](int r, int cc) { return C.u[(size_t)r * n + cc]; };
    auto Vf = [&](int r, int cc) { return C.v[(size_t)r * n + cc]; };
    for (int k = tid; k < n * n; k += nt) {
        const int i = k / n, j = k - (k / n) * n;
        const double cv = dadd(along_j(B->d1x, n, i, j, Uf), along_i(B->d1y, n, i, j, Vf));
        mx = cv > mx ? cv : mx;
        mn = cv < mn ? cv : mn;
    }
    block_minmax(mx, mn, s_red);
    if (tid == 0) {
        C.last.iters = outer;
        C.last.status = status;
        C.last.err = rel;
        C.last.cont_max = mx;
        C.last.cont_min = mn;
        C.sweeps += sweeps;
        C.cur ^= 1;
    }
    __syncthreads();
    return status;
}

__global__ void __launch_bounds__(kMaxBatchThreads) k_batch(BatchLaunch L) {
    extern __shared__ float smem[];
    __shared__ double s_red[64];
    __shared__ int s_job;
    const int nsteps = *L.nsteps;
    for (;;) {
        if (threadIdx.x == 0) s_job = atomicAdd(L.queue, 1);
        __syncthreads();
        const int job = s_job;
        __syncthreads();
        if (job >= L.count) break;
        CavityDesc& C = L.cav[L.order[job]];
        if (threadIdx.x == 0) {
            C.sweeps = 0;
            C.steps_done = 0;
        }
        __syncthreads();
        for (int t = 0; t < nsteps; ++t) {
            const int st = batch_step(C, smem, L.max_outer, L.rtol, L.warm != 0, s_red);
            if (threadIdx.x == 0) C.steps_done = t + 1;
            if (st != CNV_OK) break;
        }
        __syncthreads();
    }
}

}  // namespace
}  // namespace cnv

using namespace cnv;

struct cnv_batch {
    int count = 0;
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    std::vector<cnv_cavity_spec> specs;
    std::vector<CavityDesc> host_desc;
    CavityDesc* desc = nullptr;
    FdBands* bands = nullptr;
    void* arena = nullptr;
    size_t arena_bytes = 0;
    int* order = nullptr;
    int* queue = nullptr;
    int* nsteps = nullptr;
    int threads = 1024;
    int blocks = 0;
    int smem_bytes = 0;
    int max_outer = 100;
    double rtol = 1e-10;
    int warm = 0;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0;
    long long cells = 0;
    std::string err;
};

namespace {

int bfail(int status, const std::string& msg) {
    set_last_error(msg.c_str());
    return status;
}

#define BCUDA(call)                                                                                   \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return bfail(CNV_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

inline unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double cost_of(int n) { return (double)n * n * n; }  // ~ sweeps (n) x cells (n^2)

int build_graph(cnv_batch* b) {
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    BatchLaunch L{};
    L.cav = b->desc;
    L.order = b->order;
    L.queue = b->queue;
    L.nsteps = b->nsteps;
    L.count = b->count;
    L.max_outer = b->max_outer;
    L.rtol = b->rtol;
    L.warm = b->warm;
    L.smem_floats = b->smem_bytes / 4;
    BCUDA(cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, b->smem_bytes));
    cudaGraph_t g = nullptr;
    BCUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(b->queue, 0, sizeof(int), b->stream);
    k_batch<<<b->blocks, b->threads, b->smem_bytes, b->stream>>>(L);
    const cudaError_t le = cudaGetLastError();
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (le != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bfail(CNV_CUDA_ERROR, std::string("batch launch: ") + cudaGetErrorString(le));
    }
    if (e != cudaSuccess) return bfail(CNV_CUDA_ERROR, std::string("batch capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(CNV_CUDA_ERROR, std::string("batch instantiate: ") + cudaGetErrorString(e));
    return CNV_OK;
}

// Launch shape: threads per block and blocks per SM; shared memory as the SM allows.
int set_shape(cnv_batch* b, int threads, int per_sm) {
    int dev_smem = 0;
    BCUDA(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, b->device));
    int optin = 0;
    BCUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device));
    b->threads = threads;
    b->smem_bytes = std::min(optin, dev_smem / per_sm - 2048) & ~255;
    int occ = 0;
    BCUDA(cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, b->smem_bytes));
    BCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch, threads, b->smem_bytes));
    if (occ < 1) return bfail(CNV_CUDA_ERROR, "batched kernel does not fit on an SM");
    b->blocks = std::min(occ, per_sm) * b->sms;
    // per-cavity placement of the FP32 correction for this shared-memory size
    for (auto& d : b->host_desc) {
        const size_t plane = (size_t)d.n * d.spitch * 4;
        d.smem_mode = 4 * plane <= (size_t)b->smem_bytes ? 2 : 2 * plane <= (size_t)b->smem_bytes ? 1 : 0;
    }
    BCUDA(cudaMemcpy(b->desc, b->host_desc.data(), sizeof(CavityDesc) * b->count, cudaMemcpyHostToDevice));
    return build_graph(b);
}

int reset_fields(cnv_batch* b) {
    BCUDA(cudaMemsetAsync(b->arena, 0, b->arena_bytes, b->stream));
    for (auto& d : b->host_desc) d.cur = 0;
    BCUDA(cudaMemcpyAsync(b->desc, b->host_desc.data(), sizeof(CavityDesc) * b->count, cudaMemcpyHostToDevice,
                          b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    return CNV_OK;
}

int run(cnv_batch* b, int nsteps) {
    BCUDA(cudaMemcpyAsync(b->nsteps, &nsteps, sizeof(int), cudaMemcpyHostToDevice, b->stream));
    BCUDA(cudaEventRecord(b->ev0, b->stream));
    BCUDA(cudaGraphLaunch(b->graph, b->stream));
    BCUDA(cudaEventRecord(b->ev1, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    b->last_ms = ms;
    return CNV_OK;
}

}  // namespace

extern "C" {

int cnv_batch_specs(int count, unsigned long long seed, cnv_cavity_spec* out) {
    if (count < 0 || (count > 0 && !out)) return bfail(CNV_BAD_ARG, "bad count or null output");
    static const int kSizes[6] = {64, 96, 128, 192, 256, 384};
    for (int k = 0; k < count; ++k) {
        const unsigned long long base = seed + 3ull * (unsigned long long)k * 0x9E3779B97F4A7C15ull;
        const double u1 = (double)(mix64(base) >> 11) * 0x1.0p-53;
        const double u2 = (double)(mix64(base + 0x9E3779B97F4A7C15ull) >> 11) * 0x1.0p-53;
        const double u3 = (double)(mix64(base + 2 * 0x9E3779B97F4A7C15ull) >> 11) * 0x1.0p-53;
        out[k].n = kSizes[std::min(5, (int)(u1 * 6))];
        out[k].Re = 100.0 + 1900.0 * u2;
        out[k].lid = 0.5 + u3;
        out[k].dt = 0.0;
    }
    return CNV_OK;
}

int cnv_batch_create(const cnv_config* base, int count, const cnv_cavity_spec* specs, cnv_batch** out) {
    if (!base || !specs || !out || count < 1) return bfail(CNV_BAD_ARG, "null argument or empty batch");
    *out = nullptr;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, base->device) != cudaSuccess || prop.major != 10 || prop.minor != 3)
        return bfail(CNV_NO_DEVICE, "no sm_103 device");
    BCUDA(cudaSetDevice(base->device));
    for (int k = 0; k < count; ++k) {
        const int n = specs[k].n;
        if (n < (base->order == 6 ? 5 : 4) || n > 4096 || !(specs[k].Re > 0) || !(specs[k].lid == specs[k].lid))
            return bfail(CNV_BAD_ARG, "cavity " + std::to_string(k) + ": bad size, Re or lid speed");
    }
    cnv_batch* b = new cnv_batch();
    b->count = count;
    b->device = base->device;
    b->sms = prop.multiProcessorCount;
    b->specs.assign(specs, specs + count);
    b->max_outer = base->mixed_max_outer > 0 ? base->mixed_max_outer : 100;
    b->rtol = base->mixed_rtol > 0 ? base->mixed_rtol : 1e-10;
    b->warm = base->mixed_warm_start ? 1 : 0;
    auto cleanup = [&](int rc, const std::string& m) {
        cnv_batch_destroy(b);
        return bfail(rc, m);
    };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess)
        return cleanup(CNV_CUDA_ERROR, "stream/event creation failed");

    // arena: per cavity w[2], u, v, psi_rm (n*n doubles each), psi/g split (2 x n*pitch doubles
    // each), e/rq split (2 x n*pitch floats each)
    std::vector<size_t> offs(count);
    size_t total = 0;
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    b->host_desc.resize(count);
    for (int k = 0; k < count; ++k) {
        const int n = specs[k].n;
        const int pitch = ((n + 1) / 2 + 31) / 32 * 32;
        offs[k] = total;
        total += align(5 * (size_t)n * n * 8) + align(4 * (size_t)n * pitch * 8) + align(4 * (size_t)n * pitch * 4);
        b->cells += (long long)n * n;
    }
    b->arena_bytes = total;
    if (cudaMalloc(&b->arena, total) != cudaSuccess) return cleanup(CNV_CUDA_ERROR, "arena allocation failed");
    if (cudaMalloc(&b->desc, sizeof(CavityDesc) * count) != cudaSuccess ||
        cudaMalloc(&b->bands, sizeof(FdBands) * count) != cudaSuccess ||
        cudaMalloc(&b->order, sizeof(int) * count) != cudaSuccess ||
        cudaMalloc(&b->queue, sizeof(int)) != cudaSuccess || cudaMalloc(&b->nsteps, sizeof(int)) != cudaSuccess)
        return cleanup(CNV_CUDA_ERROR, "descriptor allocation failed");

    std::vector<FdBands> hb(count);
    const double pi = 3.14159265359;  // include/poisson.h:8
    for (int k = 0; k < count; ++k) {
        const int n = specs[k].n;
        const int pitch = ((n + 1) / 2 + 31) / 32 * 32;
        CavityDesc& d = b->host_desc[k];
        std::memset(&d, 0, sizeof d);
        d.n = n;
        d.pitch = pitch;
        d.spitch = (n + 1) / 2 + 1;
        const double dx = (double)base->Lx / n, dy = (double)base->Ly / n;
        const double h = dx;
        const double dt = specs[k].dt > 0 ? specs[k].dt
                                          : 0.2 * std::min(h * h * specs[k].Re / 4.0, h / std::fabs(specs[k].lid));
        if (build_fd_bands(n, base->order, dx, dy, &hb[k]) != CNV_OK)
            return cleanup(CNV_BAD_ARG, "finite-difference bands for cavity " + std::to_string(k));
        d.inv_re = 1. / specs[k].Re;
        d.dt = dt;
        const double beta_ref = 0.5 * (2 / (1 + sin(pi / (n + 1))) + 2 / (1 + sin(pi / (n + 1))));
        d.beta = base->sor_omega > 0 ? base->sor_omega : beta_ref;
        d.c4 = dx * dx * dy * dy;
        d.dx2 = dx * dx;
        d.dy2 = dy * dy;
        d.den = 2 * (dx * dx + dy * dy);
        d.rden = 1.0 / d.den;
        d.bc = BoundaryValues{base->u1, base->u2, base->u3, specs[k].lid, base->v1, base->v2, base->v3, base->v4};
        // FP32 sweeps per correction, rounded up to whole epochs exactly as the single-cavity
        // mixed solve does, so that both give the same iterates
        const int want = base->mixed_inner_sweeps > 0 ? base->mixed_inner_sweeps : n;
        const int per_epoch = mixed_sweeps_per_exchange();
        d.inner = std::max(1, (want + per_epoch - 1) / per_epoch) * per_epoch;
        d.bands = b->bands + k;
        char* p = static_cast<char*>(b->arena) + offs[k];
        double* f64 = reinterpret_cast<double*>(p);
        d.w[0] = f64;
        d.w[1] = f64 + (size_t)n * n;
        d.u = f64 + 2 * (size_t)n * n;
        d.v = f64 + 3 * (size_t)n * n;
        d.psi_rm = f64 + 4 * (size_t)n * n;
        double* split = reinterpret_cast<double*>(p + align(5 * (size_t)n * n * 8));
        d.psi[0] = split;
        d.psi[1] = split + (size_t)n * pitch;
        d.g[0] = split + 2 * (size_t)n * pitch;
        d.g[1] = split + 3 * (size_t)n * pitch;
        float* f32 = reinterpret_cast<float*>(p + align(5 * (size_t)n * n * 8) + align(4 * (size_t)n * pitch * 8));
        d.e[0] = f32;
        d.e[1] = f32 + (size_t)n * pitch;
        d.rq[0] = f32 + 2 * (size_t)n * pitch;
        d.rq[1] = f32 + 3 * (size_t)n * pitch;
    }
    // largest estimated cost first
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return cost_of(specs[a].n) > cost_of(specs[c].n); });
    if (cudaMemcpy(b->bands, hb.data(), sizeof(FdBands) * count, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b->order, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice) != cudaSuccess)
        return cleanup(CNV_CUDA_ERROR, "descriptor upload failed");
    int rc = reset_fields(b);
    if (rc == CNV_OK) rc = set_shape(b, 1024, 1);
    if (rc != CNV_OK) {
        cnv_batch_destroy(b);
        return rc;
    }
    *out = b;
    return CNV_OK;
}

void cnv_batch_destroy(cnv_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (void* p : {(void*)b->arena, (void*)b->desc, (void*)b->bands, (void*)b->order, (void*)b->queue, (void*)b->nsteps})
        if (p) cudaFree(p);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int cnv_batch_reset(cnv_batch* b) {
    if (!b) return bfail(CNV_BAD_ARG, "null batch");
    BCUDA(cudaSetDevice(b->device));
    return reset_fields(b);
}

int cnv_batch_tune(cnv_batch* b, int* threads_out, int* blocks_per_sm_out) {
    if (!b) return bfail(CNV_BAD_ARG, "null batch");
    BCUDA(cudaSetDevice(b->device));
    // candidates: (threads, blocks per SM); each timed for one step from the initial state
    const int cand[][2] = {{1024, 1}, {512, 1}, {512, 2}, {256, 2}};
    double best = 1e300;
    int bt = 1024, bp = 1;
    for (const auto& c : cand) {
        int rc = set_shape(b, c[0], c[1]);
        if (rc != CNV_OK) continue;
        rc = reset_fields(b);
        if (rc == CNV_OK) rc = run(b, 1);
        if (rc != CNV_OK) return rc;
        if (b->last_ms < best) {
            best = b->last_ms;
            bt = c[0];
            bp = c[1];
        }
    }
    int rc = set_shape(b, bt, bp);
    if (rc == CNV_OK) rc = reset_fields(b);
    if (threads_out) *threads_out = bt;
    if (blocks_per_sm_out) *blocks_per_sm_out = bp;
    return rc;
}

int cnv_batch_step(cnv_batch* b, int nsteps, cnv_step_info* last) {
    if (!b || nsteps < 0) return bfail(CNV_BAD_ARG, "bad batch or step count");
    BCUDA(cudaSetDevice(b->device));
    int rc = run(b, nsteps);
    if (rc != CNV_OK) return rc;
    BCUDA(cudaMemcpy(b->host_desc.data(), b->desc, sizeof(CavityDesc) * b->count, cudaMemcpyDeviceToHost));
    int status = CNV_OK;
    for (int k = 0; k < b->count; ++k) {
        const CavityDesc& d = b->host_desc[k];
        if (last) std::memcpy(&last[k], &d.last, sizeof(StepRecord));
        if (status == CNV_OK && (d.last.status != CNV_OK || d.steps_done != nsteps)) status = d.last.status ? d.last.status : CNV_CUDA_ERROR;
    }
    if (status != CNV_OK) return bfail(status, "a cavity's step did not converge");
    return CNV_OK;
}

int cnv_batch_get_fields(cnv_batch* b, int index, double* w, double* u, double* v, double* psi) {
    if (!b || index < 0 || index >= b->count) return bfail(CNV_BAD_ARG, "bad batch or index");
    BCUDA(cudaSetDevice(b->device));
    BCUDA(cudaMemcpy(&b->host_desc[index], b->desc + index, sizeof(CavityDesc), cudaMemcpyDeviceToHost));
    const CavityDesc& d = b->host_desc[index];
    const size_t bytes = (size_t)d.n * d.n * 8;
    if (w) BCUDA(cudaMemcpy(w, d.w[d.cur], bytes, cudaMemcpyDeviceToHost));
    if (u) BCUDA(cudaMemcpy(u, d.u, bytes, cudaMemcpyDeviceToHost));
    if (v) BCUDA(cudaMemcpy(v, d.v, bytes, cudaMemcpyDeviceToHost));
    if (psi) BCUDA(cudaMemcpy(psi, d.psi_rm, bytes, cudaMemcpyDeviceToHost));
    return CNV_OK;
}

int cnv_batch_stats(cnv_batch* b, long long* cells, long long* sweeps, double* ms) {
    if (!b) return bfail(CNV_BAD_ARG, "null batch");
    long long sw = 0;
    for (const auto& d : b->host_desc) sw += d.sweeps;
    if (cells) *cells = b->cells;
    if (sweeps) *sweeps = sw;
    if (ms) *ms = b->last_ms;
    return CNV_OK;
}

}  // extern "C"
