// cnv_adjoint.cu -- the differentiable form: discrete adjoint of cnavier's time step.
//
// Forward. One step k maps the state (w^k, u^k, v^k) to (w^{k+1}, u^{k+1}, v^{k+1}) with the
// kernels of cnv_step (src/main.c:283-383): the wall pass overwrites the edge values of w with
// DX v_b - DY u_b (u_b, v_b = u, v with the Dirichlet values; the lid speed is u_b on row
// n-1), the transport pass gives w' = w_b + dt (-u_b DX w_b - v_b DY w_b + (DX2 + DY2) w_b / Re),
// the Poisson solve gives psi = c4 M^-1 w' on the interior (M the reference's five-point
// operator; here the exact sine-transform solve, so the map is the converged one and the
// adjoint solve is the same operator), and u = DY psi, v = -(DX psi).
//
// Backward. With adjoints (lw, lu, lv) of the state after step k:
//   lpsi  = DY^T lu - DX^T lv                                  (interior)      k_adj_psi
//   mu    = c4 M^-1 lpsi                                       (M symmetric)   dst_solve
//   l'    = lw + mu
//   lwb   = l' + dt (-DX^T(u_b l') - DY^T(v_b l') + (DX2^T + DY2^T) l' / Re)
//   lub   = -dt (DX w_b) l',  lvb = -dt (DY w_b) l'                            k_adj_transport
//   lub  -= DY^T(E lwb),      lvb += DX^T(E lwb)      (E: the edge cells, the wall pass)
//   lw^k  = lwb, lu^k = lub, lv^k = lvb on the interior, 0 on the edges      k_adj_wall
//   dJ/dlid += sum of lub over row n-1, columns 1 .. n-2 (the cells the lid value sets)
// The transposed 7-tap products read the band of each neighbouring row: (D^T x)(c) =
// sum over r = c-3 .. c+3 of D[r][c] x(r), D[r][c] the tap c - r of row r's class.
//
// Memory. The forward run keeps the state every `checkpoint_every` steps; the backward run
// recomputes one segment at a time from its checkpoint, keeping the segment's states, then
// runs the segment's adjoint steps in reverse. Device memory: (steps / C + C + 1) states of
// 3 n^2 doubles instead of steps states.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cnv_dst.h"
#include "cnv_guard.h"
#include "cnv_kernels.h"
#include "cnv_stencil.cuh"

namespace cnv {
namespace {

struct AdjArgs {
    int n;
    const FdBands* bands;
    BoundaryValues bc;
    double inv_re, dt;
    const double* wb;   // w_b^k (w^k after the wall pass)
    const double* u;    // u^k, v^k as stored (Dirichlet values applied on read)
    const double* v;
    const double* lw;   // adjoint of w^{k+1}
    const double* lu;   // adjoint of u^{k+1}, v^{k+1}
    const double* lv;
    double* lpsi;       // adjoint of psi (interior)
    const double* mu;   // c4 M^-1 lpsi (edges zero)
    double* lwb;        // adjoint of w_b
    double* lub;        // adjoint of u_b, v_b (transport part)
    double* lvb;
    double* lw_out;     // adjoints of w^k, u^k, v^k
    double* lu_out;
    double* lv_out;
    double* lid_row;    // running sum of the lid row of lub (n entries)
};

// (D^T x) at (i, j) along j: sum over rows r = j + o of band[class(r)][-o] x(i, r)
template <class Load>
__device__ __forceinline__ double along_j_t(const double (*band)[kTaps], int n, int i, int j, Load x) {
    double acc = 0.0;
#pragma unroll
    for (int o = -3; o <= 3; ++o) {
        const int r = j + o;
        if (r >= 0 && r < n) acc = fma(band[row_class(r, n)][3 - o], x(i, r), acc);
    }
    return acc;
}

template <class Load>
__device__ __forceinline__ double along_i_t(const double (*band)[kTaps], int n, int i, int j, Load x) {
    double acc = 0.0;
#pragma unroll
    for (int o = -3; o <= 3; ++o) {
        const int r = i + o;
        if (r >= 0 && r < n) acc = fma(band[row_class(r, n)][3 - o], x(r, j), acc);
    }
    return acc;
}

__device__ __forceinline__ bool edge(int i, int j, int n) { return i == 0 || j == 0 || i == n - 1 || j == n - 1; }

__global__ void k_adj_psi(AdjArgs a) {
    const int n = a.n;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i <= 0 || j <= 0 || i >= n - 1 || j >= n - 1) return;
    const double* lu = a.lu;
    const double* lv = a.lv;
    auto LU = [&](int r, int c) { return lu[(size_t)r * n + c]; };
    auto LV = [&](int r, int c) { return lv[(size_t)r * n + c]; };
    a.lpsi[(size_t)i * n + j] = along_i_t(a.bands->d1y, n, i, j, LU) - along_j_t(a.bands->d1x, n, i, j, LV);
}

__global__ void k_adj_transport(AdjArgs a) {
    const int n = a.n;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n || j >= n) return;
    const double* lw = a.lw;
    const double* mu = a.mu;
    const double* u = a.u;
    const double* v = a.v;
    const double* wb = a.wb;
    const BoundaryValues bc = a.bc;
    auto L = [&](int r, int c) { return lw[(size_t)r * n + c] + mu[(size_t)r * n + c]; };
    auto UL = [&](int r, int c) { return vel_bc(u, n, r, c, bc.u1, bc.u2, bc.u3, bc.u4) * L(r, c); };
    auto VL = [&](int r, int c) { return vel_bc(v, n, r, c, bc.v1, bc.v2, bc.v3, bc.v4) * L(r, c); };
    auto W = [&](int r, int c) { return wb[(size_t)r * n + c]; };
    const FdBands* b = a.bands;
    const double adv = along_j_t(b->d1x, n, i, j, UL) + along_i_t(b->d1y, n, i, j, VL);
    const double dif = along_j_t(b->d2x, n, i, j, L) + along_i_t(b->d2y, n, i, j, L);
    const double l = L(i, j);
    const size_t k = (size_t)i * n + j;
    a.lwb[k] = l + a.dt * (a.inv_re * dif - adv);
    a.lub[k] = -a.dt * along_j(b->d1x, n, i, j, W) * l;
    a.lvb[k] = -a.dt * along_i(b->d1y, n, i, j, W) * l;
}

__global__ void k_adj_wall(AdjArgs a) {
    const int n = a.n;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n || j >= n) return;
    const double* lwb = a.lwb;
    auto EL = [&](int r, int c) { return edge(r, c, n) ? lwb[(size_t)r * n + c] : 0.0; };
    const size_t k = (size_t)i * n + j;
    const double lub = a.lub[k] - along_i_t(a.bands->d1y, n, i, j, EL);
    const double lvb = a.lvb[k] + along_j_t(a.bands->d1x, n, i, j, EL);
    const bool e = edge(i, j, n);
    a.lw_out[k] = e ? 0.0 : lwb[k];
    a.lu_out[k] = e ? 0.0 : lub;
    a.lv_out[k] = e ? 0.0 : lvb;
    if (i == n - 1 && j > 0 && j < n - 1) a.lid_row[j] += lub;
}

dim3 grid_for(int n, dim3 blk) { return dim3((n + blk.x - 1) / blk.x, (n + blk.y - 1) / blk.y); }

}  // namespace
}  // namespace cnv

using namespace cnv;

struct cnv_adjoint {
    cnv_config cfg;
    int n = 0, pitch = 0, device = 0;
    int every = 100;
    double dx = 0, dy = 0, c4 = 0;
    cudaStream_t stream = nullptr;
    FdBands* bands = nullptr;
    Ctrl* ctrl = nullptr;
    DstPlan dst{};
    double* sor[2] = {nullptr, nullptr};  // psi, split layout (solve output, velocity input)
    double* psi = nullptr;                // psi, row-major (velocity pass output)
    double* u0 = nullptr;                 // initial u, v (config ui, vi on the interior)
    double* v0 = nullptr;
    // forward state
    double* w[2] = {nullptr, nullptr};
    double* u = nullptr;
    double* v = nullptr;
    // checkpoints and segment states: [slot][3][n*n] (w, u, v)
    double* ck = nullptr;
    size_t ck_slots = 0;
    double* seg = nullptr;
    size_t seg_slots = 0;
    // adjoint buffers
    double* lw = nullptr;
    double* lu = nullptr;
    double* lv = nullptr;
    double* lpsi = nullptr;
    double* mu = nullptr;
    double* lwb = nullptr;
    double* lub = nullptr;
    double* lvb = nullptr;
    double* lid_row = nullptr;
    double* stage = nullptr;              // host transfers of the *_forward / *_backward calls
    // the last forward run
    int steps = -1;
    int cur = 0;
    double lid = 0;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    double fwd_ms = 0, bwd_ms = 0;
    GuardSet guards;  // guard regions around the field buffers (test_guard_cells)
};

namespace {

int afail(int status, const std::string& msg) {
    set_last_error(msg.c_str());
    return status;
}

#define ACUDA(call)                                                                                      \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return afail(CNV_CUDA_ERROR, std::string(#call) + " failed: " + cudaGetErrorString(e_));   \
    } while (0)

// CNV_OK, or CNV_CUDA_ERROR naming the first buffer whose guard bytes changed (test_guard_cells).
int check_guards(cnv_adjoint* a) {
    std::string what;
    return a->guards.check(&what) ? CNV_OK : afail(CNV_CUDA_ERROR, what);
}

void free_adjoint(cnv_adjoint* a) {
    if (!a) return;
    cudaSetDevice(a->device);
    dst_plan_destroy(&a->dst);
    double* bufs[] = {a->sor[0], a->sor[1], a->psi, a->u0, a->v0, a->w[0], a->w[1], a->u, a->v, a->ck, a->seg,
                      a->lw, a->lu, a->lv, a->lpsi, a->mu, a->lwb, a->lub, a->lvb, a->lid_row, a->stage};
    for (double* b : bufs) a->guards.release(b);
    if (a->bands) cudaFree(a->bands);
    if (a->ctrl) cudaFree(a->ctrl);
    for (cudaEvent_t e : a->ev)
        if (e) cudaEventDestroy(e);
    if (a->stream) cudaStreamDestroy(a->stream);
    delete a;
}

size_t nn_of(const cnv_adjoint* a) { return (size_t)a->n * a->n; }

double* slot_w(double* base, size_t nn, size_t k) { return base + 3 * nn * k; }
double* slot_u(double* base, size_t nn, size_t k) { return base + 3 * nn * k + nn; }
double* slot_v(double* base, size_t nn, size_t k) { return base + 3 * nn * k + 2 * nn; }

int ensure_slots(GuardSet& guards, double** buf, size_t* have, size_t want, size_t nn, const char* name) {
    if (want <= *have) return CNV_OK;
    guards.release(*buf);
    *buf = nullptr;
    *have = 0;
    ACUDA(guards.alloc(reinterpret_cast<void**>(buf), want * 3 * nn * sizeof(double), name));
    *have = want;
    return CNV_OK;
}

StepArgs base_args(const cnv_adjoint* a) {
    StepArgs s{};
    s.n = a->n;
    s.pitch = a->pitch;
    s.bands = a->bands;
    const cnv_config& c = a->cfg;
    s.bc = BoundaryValues{c.u1, c.u2, c.u3, a->lid, c.v1, c.v2, c.v3, c.v4};
    s.inv_re = 1. / c.Re;
    s.dt = c.dt;
    s.c4 = a->c4;
    s.psi = a->psi;
    s.sor[0] = a->sor[0];
    s.sor[1] = a->sor[1];
    s.ctrl = a->ctrl;
    s.timeout_ns = 2000000000LL;
    s.tile_rows = step_tile_rows(a->n, a->device);
    return s;
}

// One forward step: (w_in, u_in, v_in) -> (w_out, u_out, v_out). w_in takes the wall values in
// place (it becomes w_b); u_out/v_out may alias u_in/v_in.
int forward_step(cnv_adjoint* a, double* w_in, const double* u_in, const double* v_in, double* w_out, double* u_out,
                 double* v_out) {
    StepArgs s = base_args(a);
    s.w_in = w_in;
    s.w_wall = w_in;
    s.w_out = w_out;
    s.u = const_cast<double*>(u_in);
    s.v = const_cast<double*>(v_in);
    ACUDA(launch_pre(s, a->stream));
    ACUDA(dst_solve_split(a->dst, w_out, a->c4, a->sor[0], a->sor[1], a->pitch, a->stream));
    s.u = u_out;
    s.v = v_out;
    ACUDA(launch_post(s, false, a->stream));
    return CNV_OK;
}

int run_forward(cnv_adjoint* a, const double* w0_dev, double lid, int nsteps, bool checkpoints) {
    const size_t nn = nn_of(a);
    a->lid = lid;
    a->steps = -1;
    if (checkpoints) {
        const size_t want = (size_t)(nsteps + a->every - 1) / a->every;
        int rc = ensure_slots(a->guards, &a->ck, &a->ck_slots, std::max<size_t>(want, 1), nn, "checkpoints");
        if (rc != CNV_OK) return rc;
    }
    ACUDA(cudaMemcpyAsync(a->w[0], w0_dev, nn * 8, cudaMemcpyDeviceToDevice, a->stream));
    ACUDA(cudaMemcpyAsync(a->u, a->u0, nn * 8, cudaMemcpyDeviceToDevice, a->stream));
    ACUDA(cudaMemcpyAsync(a->v, a->v0, nn * 8, cudaMemcpyDeviceToDevice, a->stream));
    ACUDA(cudaEventRecord(a->ev[0], a->stream));
    int cur = 0;
    for (int k = 0; k < nsteps; ++k) {
        if (checkpoints && k % a->every == 0) {
            const size_t sl = (size_t)(k / a->every);
            ACUDA(cudaMemcpyAsync(slot_w(a->ck, nn, sl), a->w[cur], nn * 8, cudaMemcpyDeviceToDevice, a->stream));
            ACUDA(cudaMemcpyAsync(slot_u(a->ck, nn, sl), a->u, nn * 8, cudaMemcpyDeviceToDevice, a->stream));
            ACUDA(cudaMemcpyAsync(slot_v(a->ck, nn, sl), a->v, nn * 8, cudaMemcpyDeviceToDevice, a->stream));
        }
        int rc = forward_step(a, a->w[cur], a->u, a->v, a->w[1 - cur], a->u, a->v);
        if (rc != CNV_OK) return rc;
        cur = 1 - cur;
    }
    ACUDA(cudaEventRecord(a->ev[1], a->stream));
    a->cur = cur;
    a->steps = nsteps;
    return CNV_OK;
}

int run_backward(cnv_adjoint* a, const double* gT_dev, double* gw0_dev, double* g_lid) {
    const int T = a->steps;
    const size_t nn = nn_of(a);
    const int n = a->n;
    int rc = ensure_slots(a->guards, &a->seg, &a->seg_slots, (size_t)a->every + 1, nn, "segment states");
    if (rc != CNV_OK) return rc;
    ACUDA(cudaEventRecord(a->ev[2], a->stream));
    ACUDA(cudaMemcpyAsync(a->lw, gT_dev, nn * 8, cudaMemcpyDeviceToDevice, a->stream));
    ACUDA(cudaMemsetAsync(a->lu, 0, nn * 8, a->stream));
    ACUDA(cudaMemsetAsync(a->lv, 0, nn * 8, a->stream));
    ACUDA(cudaMemsetAsync(a->lid_row, 0, n * 8, a->stream));
    ACUDA(cudaMemsetAsync(a->mu, 0, nn * 8, a->stream));  // edges stay zero: the solve writes the interior
    const dim3 blk(32, 8);
    const dim3 grid = grid_for(n, blk);
    AdjArgs g{};
    g.n = n;
    g.bands = a->bands;
    const cnv_config& c = a->cfg;
    g.bc = BoundaryValues{c.u1, c.u2, c.u3, a->lid, c.v1, c.v2, c.v3, c.v4};
    g.inv_re = 1. / c.Re;
    g.dt = c.dt;
    g.lw = a->lw;
    g.lu = a->lu;
    g.lv = a->lv;
    g.lpsi = a->lpsi;
    g.mu = a->mu;
    g.lwb = a->lwb;
    g.lub = a->lub;
    g.lvb = a->lvb;
    g.lw_out = a->lw;  // k_adj_wall runs after every reader of lw, lu, lv in the step
    g.lu_out = a->lu;
    g.lv_out = a->lv;
    g.lid_row = a->lid_row;
    const int nseg = (T + a->every - 1) / a->every;
    for (int sgi = nseg - 1; sgi >= 0; --sgi) {
        const int k0 = sgi * a->every, k1 = std::min(T, k0 + a->every);
        // recompute the segment's states from its checkpoint
        ACUDA(cudaMemcpyAsync(a->seg, slot_w(a->ck, nn, sgi), 3 * nn * 8, cudaMemcpyDeviceToDevice, a->stream));
        for (int k = k0; k < k1; ++k) {
            const size_t sl = (size_t)(k - k0);
            rc = forward_step(a, slot_w(a->seg, nn, sl), slot_u(a->seg, nn, sl), slot_v(a->seg, nn, sl),
                              slot_w(a->seg, nn, sl + 1), slot_u(a->seg, nn, sl + 1), slot_v(a->seg, nn, sl + 1));
            if (rc != CNV_OK) return rc;
        }
        for (int k = k1 - 1; k >= k0; --k) {
            const size_t sl = (size_t)(k - k0);
            g.wb = slot_w(a->seg, nn, sl);
            g.u = slot_u(a->seg, nn, sl);
            g.v = slot_v(a->seg, nn, sl);
            k_adj_psi<<<grid, blk, 0, a->stream>>>(g);
            ACUDA(cudaGetLastError());
            ACUDA(dst_solve(a->dst, a->lpsi, a->c4, a->mu, a->stream));
            k_adj_transport<<<grid, blk, 0, a->stream>>>(g);
            ACUDA(cudaGetLastError());
            k_adj_wall<<<grid, blk, 0, a->stream>>>(g);
            ACUDA(cudaGetLastError());
        }
    }
    ACUDA(cudaEventRecord(a->ev[3], a->stream));
    if (gw0_dev) ACUDA(cudaMemcpyAsync(gw0_dev, a->lw, nn * 8, cudaMemcpyDeviceToDevice, a->stream));
    std::vector<double> row(n);
    ACUDA(cudaMemcpyAsync(row.data(), a->lid_row, n * 8, cudaMemcpyDeviceToHost, a->stream));
    ACUDA(cudaStreamSynchronize(a->stream));
    double s = 0;
    for (int j = 1; j < n - 1; ++j) s += row[j];
    if (g_lid) *g_lid = s;
    float ms = 0;
    cudaEventElapsedTime(&ms, a->ev[2], a->ev[3]);
    a->bwd_ms = ms;
    return CNV_OK;
}

bool finite_all(const std::vector<double>& x) {
    for (double d : x)
        if (!std::isfinite(d)) return false;
    return true;
}

}  // namespace

extern "C" {

int cnv_adjoint_create(const cnv_config* cfg, int checkpoint_every, cnv_adjoint** out) {
    if (!cfg || !out) return afail(CNV_BAD_ARG, "null argument");
    *out = nullptr;
    if (cfg->nx != cfg->ny) return afail(CNV_BAD_ARG, "nx != ny: the reference's operators need a square grid");
    if (cfg->order != 2 && cfg->order != 4 && cfg->order != 6)
        return afail(CNV_BAD_ARG, "** Error: valid orders are 2, 4 or 6 **");
    if (cfg->nx < (cfg->order == 6 ? 5 : 4) || cfg->nx > 8192) return afail(CNV_BAD_ARG, "grid size outside [5, 8192]");
    if (!(cfg->Re > 0) || !(cfg->dt > 0) || cfg->Lx <= 0 || cfg->Ly <= 0)
        return afail(CNV_BAD_ARG, "invalid Re/dt/Lx/Ly");
    if (checkpoint_every < 1) return afail(CNV_BAD_ARG, "checkpoint_every must be >= 1");
    if (cfg->test_guard_cells < 0 || cfg->test_guard_cells > 2)
        return afail(CNV_BAD_ARG, "test_guard_cells must be 0, 1 or 2");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= cfg->device)
        return afail(CNV_NO_DEVICE, "no CUDA device " + std::to_string(cfg->device));
    ACUDA(cudaSetDevice(cfg->device));
    cnv_adjoint* a = new cnv_adjoint();
    a->cfg = *cfg;
    a->guards.on = cfg->test_guard_cells != 0;
    a->device = cfg->device;
    a->n = cfg->nx;
    a->every = checkpoint_every;
    a->dx = (double)cfg->Lx / cfg->nx;
    a->dy = (double)cfg->Ly / cfg->ny;
    a->c4 = a->dx * a->dx * a->dy * a->dy;
    a->lid = cfg->u4;
    const int n = a->n;
    a->pitch = ((n + 1) / 2 + 31) / 32 * 32;
    const size_t nn = (size_t)n * n, split = (size_t)n * a->pitch;
    auto bad = [&](const std::string& m) {
        free_adjoint(a);
        return afail(CNV_CUDA_ERROR, m);
    };
    if (cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking) != cudaSuccess) return bad("stream");
    for (auto& e : a->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return bad("event");
    double** fields[] = {&a->psi, &a->u0, &a->v0, &a->w[0], &a->w[1], &a->u, &a->v, &a->lw, &a->lu,
                         &a->lv, &a->lpsi, &a->mu, &a->lwb, &a->lub, &a->lvb, &a->stage};
    const char* names[] = {"psi", "u0", "v0", "w[0]", "w[1]", "u", "v", "lw", "lu",
                           "lv", "lpsi", "mu", "lwb", "lub", "lvb", "stage"};
    for (int k = 0; k < 16; ++k) {
        if (a->guards.alloc(reinterpret_cast<void**>(fields[k]), nn * 8, names[k]) != cudaSuccess)
            return bad("cudaMalloc");
        if (cudaMemset(*fields[k], 0, nn * 8) != cudaSuccess) return bad("cudaMemset");
    }
    const char* sor_names[] = {"split psi[0]", "split psi[1]"};
    for (int c = 0; c < 2; ++c) {
        if (a->guards.alloc(reinterpret_cast<void**>(&a->sor[c]), split * 8, sor_names[c]) != cudaSuccess)
            return bad("cudaMalloc");
        if (cudaMemset(a->sor[c], 0, split * 8) != cudaSuccess) return bad("cudaMemset");
    }
    if (a->guards.alloc(reinterpret_cast<void**>(&a->lid_row), n * 8, "lid_row") != cudaSuccess)
        return bad("cudaMalloc");
    if (cudaMalloc(&a->bands, sizeof(FdBands)) != cudaSuccess || cudaMalloc(&a->ctrl, sizeof(Ctrl)) != cudaSuccess)
        return bad("cudaMalloc");
    if (cudaMemset(a->ctrl, 0, sizeof(Ctrl)) != cudaSuccess) return bad("cudaMemset");
    FdBands hb;
    if (build_fd_bands(n, cfg->order, a->dx, a->dy, &hb) != CNV_OK) {
        free_adjoint(a);
        return afail(CNV_BAD_ARG, "finite-difference bands");
    }
    if (cudaMemcpy(a->bands, &hb, sizeof hb, cudaMemcpyHostToDevice) != cudaSuccess) return bad("band upload");
    if (dst_plan_create(n, a->dx, a->dy, &a->dst) != CNV_OK) return bad("sine-transform plan");
    // initial velocities of src/main.c:213-221: ui, vi on the interior, zero on the edges
    std::vector<double> hu(nn, 0.0), hv(nn, 0.0);
    for (int i = 1; i < n - 1; ++i)
        for (int j = 1; j < n - 1; ++j) {
            hu[(size_t)i * n + j] = cfg->ui;
            hv[(size_t)i * n + j] = cfg->vi;
        }
    if (cudaMemcpy(a->u0, hu.data(), nn * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(a->v0, hv.data(), nn * 8, cudaMemcpyHostToDevice) != cudaSuccess)
        return bad("initial velocity upload");
    if (cfg->test_guard_cells == 2 && a->guards.plant("u") != cudaSuccess) return bad("guard setup");
    *out = a;
    return CNV_OK;
}

void cnv_adjoint_destroy(cnv_adjoint* a) { free_adjoint(a); }

int cnv_adjoint_forward_device(cnv_adjoint* a, const double* w0, double lid, int nsteps, double* w_final) {
    if (!a || !w0 || nsteps < 1) return afail(CNV_BAD_ARG, "bad adjoint handle, initial field or step count");
    ACUDA(cudaSetDevice(a->device));
    int rc = run_forward(a, w0, lid, nsteps, true);
    if (rc != CNV_OK) return rc;
    if (w_final)
        ACUDA(cudaMemcpyAsync(w_final, a->w[a->cur], nn_of(a) * 8, cudaMemcpyDeviceToDevice, a->stream));
    ACUDA(cudaStreamSynchronize(a->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, a->ev[0], a->ev[1]);
    a->fwd_ms = ms;
    return check_guards(a);
}

int cnv_adjoint_backward_device(cnv_adjoint* a, const double* g_final, double* g_w0, double* g_lid) {
    if (!a || !g_final || !g_w0) return afail(CNV_BAD_ARG, "null argument");
    if (a->steps < 1) return afail(CNV_BAD_ARG, "no forward run to differentiate");
    ACUDA(cudaSetDevice(a->device));
    const int rc = run_backward(a, g_final, g_w0, g_lid);
    return rc == CNV_OK ? check_guards(a) : rc;
}

int cnv_adjoint_forward(cnv_adjoint* a, const double* w0, double lid, int nsteps, double* w_final) {
    if (!a || !w0 || nsteps < 1) return afail(CNV_BAD_ARG, "bad adjoint handle, initial field or step count");
    ACUDA(cudaSetDevice(a->device));
    const size_t nn = nn_of(a);
    ACUDA(cudaMemcpyAsync(a->stage, w0, nn * 8, cudaMemcpyHostToDevice, a->stream));
    int rc = run_forward(a, a->stage, lid, nsteps, true);
    if (rc != CNV_OK) return rc;
    std::vector<double> h(nn);
    ACUDA(cudaMemcpyAsync(h.data(), a->w[a->cur], nn * 8, cudaMemcpyDeviceToHost, a->stream));
    ACUDA(cudaStreamSynchronize(a->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, a->ev[0], a->ev[1]);
    a->fwd_ms = ms;
    if (w_final) std::memcpy(w_final, h.data(), nn * 8);
    if (!finite_all(h)) return afail(CNV_NONFINITE, "final vorticity holds NaN or Inf");
    return check_guards(a);
}

int cnv_adjoint_backward(cnv_adjoint* a, const double* g_final, double* g_w0, double* g_lid) {
    if (!a || !g_final || !g_w0) return afail(CNV_BAD_ARG, "null argument");
    if (a->steps < 1) return afail(CNV_BAD_ARG, "no forward run to differentiate");
    ACUDA(cudaSetDevice(a->device));
    const size_t nn = nn_of(a);
    ACUDA(cudaMemcpyAsync(a->stage, g_final, nn * 8, cudaMemcpyHostToDevice, a->stream));
    int rc = run_backward(a, a->stage, nullptr, g_lid);
    if (rc != CNV_OK) return rc;
    ACUDA(cudaMemcpyAsync(g_w0, a->lw, nn * 8, cudaMemcpyDeviceToHost, a->stream));
    ACUDA(cudaStreamSynchronize(a->stream));
    return check_guards(a);
}

int cnv_adjoint_enstrophy_gradient(cnv_adjoint* a, const double* w0, double lid, int nsteps, double* J,
                                   double* g_w0, double* g_lid) {
    if (!a || !w0 || !g_w0 || nsteps < 1) return afail(CNV_BAD_ARG, "null argument or bad step count");
    const size_t nn = nn_of(a);
    std::vector<double> wT(nn), seed(nn);
    int rc = cnv_adjoint_forward(a, w0, lid, nsteps, wT.data());
    if (rc != CNV_OK) return rc;
    const double h2 = a->dx * a->dy;
    double s = 0;
    for (size_t k = 0; k < nn; ++k) {
        s += wT[k] * wT[k];
        seed[k] = h2 * wT[k];
    }
    if (J) *J = 0.5 * h2 * s;
    return cnv_adjoint_backward(a, seed.data(), g_w0, g_lid);
}

int cnv_adjoint_stats(cnv_adjoint* a, double* forward_ms, double* backward_ms, long long* state_bytes) {
    if (!a) return afail(CNV_BAD_ARG, "null handle");
    if (forward_ms) *forward_ms = a->fwd_ms;
    if (backward_ms) *backward_ms = a->bwd_ms;
    if (state_bytes) *state_bytes = (long long)((a->ck_slots + a->seg_slots) * 3 * nn_of(a) * 8);
    return CNV_OK;
}

}  // extern "C"
