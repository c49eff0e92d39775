// cnv_api.cu -- state, buffers, CUDA-graph capture of the time step, and the C ABI of cnv.h.
//
// One cnv_state owns one cavity on one GPU: every field stays in device memory between steps,
// one CUDA stream orders all work, and the whole step (wall pass, transport pass, the
// persistent Poisson solve, velocity and continuity passes) is captured once into a CUDA graph
// per vorticity buffer parity, so a call to cnv_step(s, K) enqueues K graph launches and waits
// once. Per-step records (iteration count, stop norm, continuity max/min, status) are written
// by the kernels into a device array and copied back after the last step.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cnv_dst.h"
#include "cnv_guard.h"
#include "cnv_kernels.h"

using namespace cnv;

#define CNV_XSTR(x) #x
#define CNV_STR(x) CNV_XSTR(x)

namespace {

thread_local std::string g_last_error;

int fail(int status, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int status, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

#define CNV_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(CNV_CUDA_ERROR, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                                  \
    } while (0)

// Sweeps per border exchange the FP64 SOR/GS solve uses by default for an n x n grid (1: the
// kernel that exchanges every half-sweep; measured per sweep: 256^2 6.7 us tiled vs 8.6, 320^2
// 12.3 vs 11.3, 512^2 11.4 vs 9.1, 768^2 31.5 vs 26.0).
// Sweeps per border exchange by grid size, from timings of both kernels on the cavity workload
// (us per sweep, exchange kernel vs 2 / 4 sweeps per exchange): 256^2 7.38 vs 6.57 / 6.17,
// 288^2 9.30 vs 8.90 / 8.85, 320^2 9.70 vs 9.42 / 10.12, 352^2 9.67 vs 10.11 / 10.99.
int auto_sor_sweeps(int n) { return n < 300 ? 4 : n < 336 ? 2 : 1; }

bool is_pow2(double x) {
    int e;
    return x > 0 && std::frexp(x, &e) == 0.5;
}

// splitmix64 output function (Steele, Lea, Flood 2014) applied to a counter.
inline unsigned long long splitmix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// w = sigma * N(0,1) per cell (splitmix64 counter stream + Box-Muller), then `passes` Jacobi
// averaging passes over the interior, edges kept.
void noise_field(int n, unsigned long long seed, double sigma, int passes, double* w) {
    const size_t nn = (size_t)n * n;
    const double two_pi = 6.283185307179586476925286766559;
    for (size_t k = 0; k < nn; ++k) {
        const unsigned long long z1 = splitmix64(seed + (2 * k) * 0x9E3779B97F4A7C15ull);
        const unsigned long long z2 = splitmix64(seed + (2 * k + 1) * 0x9E3779B97F4A7C15ull);
        const double u1 = ((double)(z1 >> 11) + 0.5) * 0x1.0p-53;
        const double u2 = (double)(z2 >> 11) * 0x1.0p-53;
        w[k] = sigma * (std::sqrt(-2.0 * std::log(u1)) * std::cos(two_pi * u2));
    }
    std::vector<double> t(nn);
    for (int pass = 0; pass < passes; ++pass) {
        t.assign(w, w + nn);
        for (int i = 1; i < n - 1; ++i)
            for (int j = 1; j < n - 1; ++j) {
                const size_t k = (size_t)i * n + j;
                w[k] = (t[k - n] + t[k + n] + t[k - 1] + t[k + 1]) / 4;
            }
    }
}

}  // namespace

void cnv::set_last_error(const char* msg) { g_last_error = msg; }

struct cnv_state {
    cnv_config cfg;
    int n = 0;
    int pitch = 0;       // split-layout row pitch (doubles)
    double dx = 0, dy = 0;
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;

    double* w[2] = {nullptr, nullptr};
    double* u = nullptr;
    double* v = nullptr;
    double* psi = nullptr;
    double* sor[2] = {nullptr, nullptr};
    double* alt[2] = {nullptr, nullptr};
    double* rhs[2] = {nullptr, nullptr};
    double* scratch = nullptr;   // 2*n*n: right-hand side and result of standalone Poisson solves
    double* stage = nullptr;     // 3*n*n: host fields uploaded by cnv_set_fields, checked on the device
    GuardSet guards;             // guard regions around the buffers (test_guard_cells)
    void* sync = nullptr;        // Poisson solver synchronisation state
    // mixed-precision form (CNV_PREC_MIXED)
    bool mixed = false;
    float* rq = nullptr;         // FP32 correction right-hand side (split layout, both colours)
    float* eg = nullptr;         // FP32 correction border exchange (split layout, 2 parities x 2 colours)
    void* msync = nullptr;
    int mixed_gx = 1, mixed_gy = 1, mixed_epochs = 1, mixed_max_outer = 100;
    bool mixed_rq_smem = false;
    double mixed_rtol = 1e-10;
    // several sweeps per border exchange (FP64 SOR/GS in shared-memory tiles)
    bool tb = false;
    int tb_sweeps = 4;
    int tb_gx = 1, tb_gy = 1;
    bool tb_g_smem = false;
    double* tb_snap = nullptr;
    void* tb_sync = nullptr;
    // exact solve by sine transforms (CNV_POISSON_DIRECT)
    bool direct = false;
    DstPlan dst{};
    double* cont_partials = nullptr;
    int* flag = nullptr;         // non-finite scan result
    FdBands* bands = nullptr;
    Ctrl* ctrl = nullptr;
    StepRecord* records = nullptr;
    int max_records = 0;

    int cur = 0;                 // index of the current vorticity buffer
    int poisson_grid = 0, poisson_gx = 1, poisson_gy = 1;
    int cont_blocks = 0;
    int tile_rows = 32;          // rows of the step passes' tiles
    PoissonParams pp{};
    StepArgs sa{};

    cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [pre/post][parity]
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t evp0 = nullptr, evp1 = nullptr;  // around the Poisson kernel of the last step
    long long last_sweeps = 0;
    double last_ms = 0;
    int last_steps_enqueued = 0;
    int parity_at_start = 0;
};

namespace {

// cudaMalloc for a field or work buffer, with guard regions when test_guard_cells is on.
cudaError_t buf_alloc(cnv_state* s, void** p, size_t bytes, const char* name) { return s->guards.alloc(p, bytes, name); }

void buf_free(cnv_state* s, void* p) { s->guards.release(p); }

// CNV_OK, or CNV_CUDA_ERROR naming the first buffer whose guard bytes changed (test_guard_cells).
int check_guards(cnv_state* s) {
    std::string what;
    if (s->guards.check(&what)) return CNV_OK;
    return fail(CNV_CUDA_ERROR, "%s", what.c_str());
}

void free_state(cnv_state* s) {
    if (!s) return;
    if (s->device >= 0) cudaSetDevice(s->device);
    for (auto& row : s->graph)
        for (auto& g : row)
            if (g) cudaGraphExecDestroy(g);
    double* bufs[] = {s->w[0], s->w[1], s->u, s->v, s->psi, s->sor[0], s->sor[1], s->alt[0],
                      s->alt[1], s->rhs[0], s->rhs[1], s->scratch, s->stage, s->cont_partials};
    for (double* b : bufs) buf_free(s, b);
    for (float* b : {s->rq, s->eg}) buf_free(s, b);
    if (s->msync) cudaFree(s->msync);
    buf_free(s, s->tb_snap);
    if (s->tb_sync) cudaFree(s->tb_sync);
    if (s->direct) dst_plan_destroy(&s->dst);
    buf_free(s, s->flag);
    if (s->sync) cudaFree(s->sync);
    buf_free(s, s->bands);
    buf_free(s, s->ctrl);
    if (s->records) cudaFree(s->records);
    for (cudaEvent_t ev : {s->ev0, s->ev1, s->evp0, s->evp1})
        if (ev) cudaEventDestroy(ev);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

int validate(const cnv_config* c) {
    if (c->nx != c->ny)
        return fail(CNV_BAD_ARG, "nx (%d) != ny (%d): the reference's operators need a square grid", c->nx, c->ny);
    if (c->order != 2 && c->order != 4 && c->order != 6)
        return fail(CNV_BAD_ARG, "** Error: valid orders are 2, 4 or 6 ** (got %d)", c->order);
    if (c->nx < (c->order == 6 ? 5 : 4) || c->nx > 16384)
        return fail(CNV_BAD_ARG, "grid size %d outside [%d, 16384]", c->nx, c->order == 6 ? 5 : 4);
    if (c->poisson_type < 1 || c->poisson_type > 4)
        return fail(CNV_BAD_ARG, "Error - invalid option for Poisson solver (%d)", c->poisson_type);
    if (c->test_stall_block < 0) return fail(CNV_BAD_ARG, "test_stall_block must be >= 0");
    if (c->test_guard_cells < 0 || c->test_guard_cells > 2)
        return fail(CNV_BAD_ARG, "test_guard_cells must be 0, 1 or 2, got %d", c->test_guard_cells);
    if (c->sor_blocking != 0 && c->sor_blocking != 1 && c->sor_blocking != 2 && c->sor_blocking != 4)
        return fail(CNV_BAD_ARG, "sor_blocking must be 0 (auto), 1, 2 or 4 sweeps per exchange, got %d",
                    c->sor_blocking);
    if (c->poisson_type == CNV_POISSON_DIRECT && c->precision == CNV_PREC_MIXED)
        return fail(CNV_BAD_ARG, "the direct Poisson solve is FP64 only (precision %d)", c->precision);
    if (c->precision != CNV_PREC_FP64 && c->precision != CNV_PREC_FP64_FMA && c->precision != CNV_PREC_MIXED)
        return fail(CNV_BAD_ARG, "unknown precision %d", c->precision);
    if (c->Lx <= 0 || c->Ly <= 0 || !(c->Re > 0) || !(c->dt > 0) || c->poisson_max_it < 1 ||
        !(c->poisson_tol >= 0))
        return fail(CNV_BAD_ARG, "invalid Lx/Ly/Re/dt/poisson_max_it/poisson_tol");
    // Courant check of src/main.c:165-174 (it uses u1, as the reference does)
    const double dx = (double)c->Lx / c->nx, dy = (double)c->Ly / c->ny;
    const double r1 = c->u1 * c->dt / dx, r2 = c->u1 * c->dt / dy;
    if (r1 > c->max_co || r2 > c->max_co)
        return fail(CNV_BAD_ARG, "Unstable Solution! r1: %f r2: %f", r1, r2);
    return CNV_OK;
}

int upload_initial(cnv_state* s) {
    const int n = s->n;
    const size_t nn = (size_t)n * n;
    std::vector<double> w(nn, 0.0), u(nn, 0.0), v(nn, 0.0);
    // src/main.c:213-221: interior u = ui, v = vi; everything else zero
    for (int i = 1; i < n - 1; ++i)
        for (int j = 1; j < n - 1; ++j) {
            u[(size_t)i * n + j] = s->cfg.ui;
            v[(size_t)i * n + j] = s->cfg.vi;
        }
    if (s->cfg.init_field == CNV_INIT_NOISE)
        noise_field(n, s->cfg.seed, s->cfg.init_sigma, s->cfg.init_smooth_passes, w.data());
    s->cur = 0;
    CNV_CUDA(cudaMemcpyAsync(s->w[0], w.data(), nn * 8, cudaMemcpyHostToDevice, s->stream));
    CNV_CUDA(cudaMemcpyAsync(s->u, u.data(), nn * 8, cudaMemcpyHostToDevice, s->stream));
    CNV_CUDA(cudaMemcpyAsync(s->v, v.data(), nn * 8, cudaMemcpyHostToDevice, s->stream));
    CNV_CUDA(cudaMemsetAsync(s->psi, 0, nn * 8, s->stream));
    CNV_CUDA(cudaMemsetAsync(s->w[1], 0, nn * 8, s->stream));
    for (double* a : s->sor) CNV_CUDA(cudaMemsetAsync(a, 0, (size_t)n * s->pitch * 8, s->stream));
    CNV_CUDA(cudaStreamSynchronize(s->stream));
    return CNV_OK;
}

int ensure_records(cnv_state* s, int count) {
    if (count <= s->max_records) return CNV_OK;
    int cap = s->max_records ? s->max_records : 64;
    while (cap < count) cap *= 2;
    if (s->records) CNV_CUDA(cudaFree(s->records));
    s->records = nullptr;
    CNV_CUDA(cudaMalloc(&s->records, sizeof(StepRecord) * cap));
    s->max_records = cap;
    return CNV_OK;
}

// Reset the control block for a new call: zero counters, flags, step index; set records.
int reset_ctrl(cnv_state* s) {
    Ctrl h{};
    h.records = s->records;
    h.max_records = s->max_records;
    CNV_CUDA(cudaMemcpyAsync(s->ctrl, &h, sizeof(Ctrl), cudaMemcpyHostToDevice, s->stream));
    return CNV_OK;
}

StepArgs step_args(cnv_state* s, int parity) {
    StepArgs a = s->sa;
    a.w_in = s->w[parity];
    a.w_wall = s->w[parity];
    a.w_out = s->w[1 - parity];
    return a;
}

PoissonLaunch poisson_launch(cnv_state* s) {
    PoissonLaunch L{};
    L.p = s->pp;
    for (int c = 0; c < 2; ++c) {
        L.sor[c] = s->sor[c];
        L.alt[c] = s->alt[c];
        L.rhs[c] = s->rhs[c];
    }
    L.ctrl = s->ctrl;
    L.sync = s->sync;
    L.grid = s->poisson_grid;
    L.gx = s->poisson_gx;
    L.gy = s->poisson_gy;
    return L;
}

MixedLaunch mixed_launch(cnv_state* s) {
    MixedLaunch L{};
    L.n = s->n;
    L.pitch = s->pitch;
    L.gx = s->mixed_gx;
    L.gy = s->mixed_gy;
    L.dx2 = s->pp.dx2;
    L.dy2 = s->pp.dy2;
    L.den = s->pp.den;
    L.rden = 1.0 / s->pp.den;
    L.beta = s->pp.beta;
    L.rtol = s->mixed_rtol;
    L.max_outer = s->mixed_max_outer;
    L.epochs = s->mixed_epochs;
    L.rq_in_smem = s->mixed_rq_smem ? 1 : 0;
    L.timeout_ns = s->pp.timeout_ns;
    const size_t split = (size_t)s->n * s->pitch;
    for (int c = 0; c < 2; ++c) {
        L.g[c] = s->rhs[c];
        L.psi[c] = s->sor[c];
        L.rq[c] = s->rq + c * split;
        for (int par = 0; par < 2; ++par) L.eg[par][c] = s->eg + (2 * par + c) * split;
    }
    L.ctrl = s->ctrl;
    L.sync = s->msync;
    return L;
}

// Enqueue the Poisson solve on the split-layout rhs, or on g for the mixed form (psi starts
// from zero). The direct solve reads the row-major field `in` scaled by `scale` instead
// (w with c4 in a step, f with -c4 for a standalone solve) and reports 0 iterations.
int enqueue_poisson(cnv_state* s, const double* in, double scale, bool in_step) {
    const size_t split_bytes = (size_t)s->n * s->pitch * 8;
    if (s->direct) {
        CNV_CUDA(cudaMemsetAsync(s->sor[0], 0, split_bytes, s->stream));
        CNV_CUDA(cudaMemsetAsync(s->sor[1], 0, split_bytes, s->stream));
        CNV_CUDA(dst_solve_split(s->dst, in, scale, s->sor[0], s->sor[1], s->pitch, s->stream));
        // iters, status (int) and err (double) of the control block: 0, CNV_OK, 0.0
        static_assert(offsetof(Ctrl, status) == offsetof(Ctrl, iters) + 4 && offsetof(Ctrl, err) == offsetof(Ctrl, iters) + 8,
                      "Ctrl layout");
        CNV_CUDA(cudaMemsetAsync(reinterpret_cast<char*>(s->ctrl) + offsetof(Ctrl, iters), 0, 16, s->stream));
        return CNV_OK;
    }
    if (s->tb) {
        CNV_CUDA(cudaMemsetAsync(s->sor[0], 0, split_bytes, s->stream));
        CNV_CUDA(cudaMemsetAsync(s->sor[1], 0, split_bytes, s->stream));
        TbLaunch T{};
        T.p = s->pp;
        T.sweeps = s->tb_sweeps;
        T.gx = s->tb_gx;
        T.gy = s->tb_gy;
        T.g_in_smem = s->tb_g_smem ? 1 : 0;
        T.out[0] = s->sor[0];
        T.out[1] = s->sor[1];
        T.rhs[0] = s->rhs[0];
        T.rhs[1] = s->rhs[1];
        T.snap = s->tb_snap;
        T.ctrl = s->ctrl;
        T.sync = s->tb_sync;
        CNV_CUDA(launch_poisson_tb(T, s->stream));
        return CNV_OK;
    }
    if (s->mixed) {
        // zero start, or (mixed_warm_start, within a time step) the previous step's psi
        if (!(in_step && s->cfg.mixed_warm_start)) {
            CNV_CUDA(cudaMemsetAsync(s->sor[0], 0, split_bytes, s->stream));
            CNV_CUDA(cudaMemsetAsync(s->sor[1], 0, split_bytes, s->stream));
        }
        CNV_CUDA(launch_mixed(mixed_launch(s), s->stream));
        return CNV_OK;
    }
    // both copies of psi start at zero (zero start, zero Dirichlet edge)
    CNV_CUDA(cudaMemsetAsync(s->sor[0], 0, split_bytes, s->stream));
    CNV_CUDA(cudaMemsetAsync(s->sor[1], 0, split_bytes, s->stream));
    CNV_CUDA(cudaMemsetAsync(s->alt[0], 0, split_bytes, s->stream));
    CNV_CUDA(cudaMemsetAsync(s->alt[1], 0, split_bytes, s->stream));
    CNV_CUDA(launch_poisson(poisson_launch(s), s->stream));
    return CNV_OK;
}

// The step is three stream segments: graph[0][parity] (the pre-solve pass: wall, transport,
// right-hand side), the Poisson solve (memsets + one cooperative launch, bracketed by timing
// events), and graph[1][parity] (the post-solve pass: velocity and continuity).
int enqueue_pre(cnv_state* s, int parity) {
    CNV_CUDA(launch_pre(step_args(s, parity), s->stream));
    return CNV_OK;
}

int enqueue_post(cnv_state* s, int parity) {
    CNV_CUDA(launch_post(step_args(s, parity), true, s->stream));
    return CNV_OK;
}

int capture(cnv_state* s, int (*fn)(cnv_state*, int), int parity, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    CNV_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int rc = fn(s, parity);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (rc != CNV_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return fail(CNV_CUDA_ERROR, "graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(CNV_CUDA_ERROR, "graph instantiate: %s", cudaGetErrorString(e));
    return CNV_OK;
}

int build_graphs(cnv_state* s) {
    for (int parity = 0; parity < 2; ++parity) {
        if (!s->graph[0][parity]) {
            int rc = capture(s, enqueue_pre, parity, &s->graph[0][parity]);
            if (rc != CNV_OK) return rc;
        }
        if (!s->graph[1][parity]) {
            int rc = capture(s, enqueue_post, parity, &s->graph[1][parity]);
            if (rc != CNV_OK) return rc;
        }
    }
    return CNV_OK;
}

int enqueue_step(cnv_state* s, int parity) {
    CNV_CUDA(cudaGraphLaunch(s->graph[0][parity], s->stream));
    CNV_CUDA(cudaEventRecord(s->evp0, s->stream));
    int rc = enqueue_poisson(s, s->w[1 - parity], s->sa.c4, true);
    if (rc != CNV_OK) return rc;
    CNV_CUDA(cudaEventRecord(s->evp1, s->stream));
    CNV_CUDA(cudaGraphLaunch(s->graph[1][parity], s->stream));
    return CNV_OK;
}

}  // namespace

extern "C" {

const char* cnv_last_error(void) { return g_last_error.c_str(); }

int cnv_noise_field(int n, unsigned long long seed, double sigma, int passes, double* out) {
    if (n < 1 || passes < 0 || !out) return fail(CNV_BAD_ARG, "bad noise-field arguments");
    noise_field(n, seed, sigma, passes, out);
    return CNV_OK;
}

const char* cnv_version(void) { return "libcnv 1 (sm_103a, CUDA " CNV_STR(CUDART_VERSION) ")"; }

int cnv_create(const cnv_config* cfg, cnv_state** out) {
    if (!cfg || !out) return fail(CNV_BAD_ARG, "null argument");
    *out = nullptr;
    int rc = validate(cfg);
    if (rc != CNV_OK) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= cfg->device)
        return fail(CNV_NO_DEVICE, "no CUDA device %d", cfg->device);
    cudaDeviceProp prop;
    CNV_CUDA(cudaGetDeviceProperties(&prop, cfg->device));
    if (prop.major != 10 || prop.minor != 3)
        return fail(CNV_NO_DEVICE, "device %d is sm_%d%d; libcnv is built for sm_103a", cfg->device,
                    prop.major, prop.minor);
    CNV_CUDA(cudaSetDevice(cfg->device));

    cnv_state* s = new cnv_state();
    s->cfg = *cfg;
    s->guards.on = cfg->test_guard_cells != 0;
    s->device = cfg->device;
    s->n = cfg->nx;
    s->sms = prop.multiProcessorCount;
    const int n = s->n;
    const int W = (n + 1) / 2;
    s->pitch = (W + 31) / 32 * 32;  // 256-byte aligned rows
    s->dx = (double)cfg->Lx / cfg->nx;  // src/main.c:138-139
    s->dy = (double)cfg->Ly / cfg->ny;
    const size_t nn = (size_t)n * n;
    const size_t split = (size_t)n * s->pitch;
#define ALLOC(ptr, count)                                                     \
    do {                                                                      \
        cudaError_t e_ = buf_alloc(s, reinterpret_cast<void**>(&(ptr)), sizeof(*(ptr)) * (count), #ptr); \
        if (e_ != cudaSuccess) {                                              \
            free_state(s);                                                    \
            return fail(CNV_CUDA_ERROR, "cudaMalloc: %s", cudaGetErrorString(e_)); \
        }                                                                     \
    } while (0)
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        free_state(s);
        return fail(CNV_CUDA_ERROR, "cudaStreamCreate failed");
    }
    ALLOC(s->w[0], nn);
    ALLOC(s->w[1], nn);
    ALLOC(s->u, nn);
    ALLOC(s->v, nn);
    ALLOC(s->psi, nn);
    ALLOC(s->scratch, 2 * nn);
    for (int c = 0; c < 2; ++c) {
        ALLOC(s->sor[c], split);
        ALLOC(s->alt[c], split);
        ALLOC(s->rhs[c], split);
    }
    ALLOC(s->bands, 1);
    ALLOC(s->ctrl, 1);
    ALLOC(s->flag, 1);

    // Poisson arithmetic: the folded exact form needs dx = dy with dx^2 and 2*(dx^2+dy^2)
    // powers of two (every n = 2^k on a unit cavity)
    const double dx2 = s->dx * s->dx, dy2 = s->dy * s->dy;
    const Arith arith = cfg->precision == CNV_PREC_FP64_FMA ? Arith::kFma : Arith::kExact;
    const bool fold = arith == Arith::kExact && s->dx == s->dy && is_pow2(dx2) && is_pow2(2 * (dx2 + dy2));
    // Poisson solver geometry: co-resident blocks (one tile each), a multiple of the SM count
    const void* kern =
        poisson_kernel_ptr(arith, cfg->poisson_type == CNV_POISSON_DIRECT ? CNV_POISSON_SOR : cfg->poisson_type, fold);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, poisson_threads(), 0) != cudaSuccess ||
        per_sm < 1) {
        free_state(s);
        return fail(CNV_CUDA_ERROR, "occupancy query failed for the Poisson kernel");
    }
    s->poisson_grid = poisson_grid_for(n, s->sms, per_sm);
    if (cfg->solver_blocks > 0)
        s->poisson_grid = std::min(cfg->solver_blocks, std::min(per_sm * s->sms, kMaxSolverBlocks));
    poisson_tiles(n, s->poisson_grid, &s->poisson_gx, &s->poisson_gy);
    s->poisson_grid = s->poisson_gx * s->poisson_gy;
    s->tile_rows = step_tile_rows(n, s->device);
    s->cont_blocks = post_grid(n, s->device, s->tile_rows);
    if (s->cont_blocks < 1) {
        free_state(s);
        return fail(CNV_CUDA_ERROR, "occupancy query failed for the post-solve pass");
    }
    {
        cudaError_t e_ = cudaMalloc(&s->sync, poisson_sync_bytes());
        if (e_ != cudaSuccess) {
            free_state(s);
            return fail(CNV_CUDA_ERROR, "cudaMalloc: %s", cudaGetErrorString(e_));
        }
    }
    ALLOC(s->cont_partials, 4 * (size_t)s->cont_blocks);
    if (cfg->precision == CNV_PREC_MIXED) {
        // one block per SM; the tile plus its halo must fit in shared memory
        s->mixed = true;
        // every tile at least as wide and tall as the halo, so a halo comes from the eight
        // adjacent tiles only
        const int halo = 2 * mixed_sweeps_per_exchange();
        for (int g = std::min(s->sms, kMaxSolverBlocks); g >= 1; --g) {
            poisson_tiles(n, g, &s->mixed_gx, &s->mixed_gy);
            if ((n - 2) / s->mixed_gx >= halo && (n - 2) / s->mixed_gy >= halo) break;
            s->mixed_gx = s->mixed_gy = 1;
        }
        s->mixed_rq_smem = mixed_smem_bytes(n, s->mixed_gx, s->mixed_gy, true) + 2048 <= prop.sharedMemPerBlockOptin;
        const size_t smem = mixed_smem_bytes(n, s->mixed_gx, s->mixed_gy, s->mixed_rq_smem);
        if (smem + 2048 > prop.sharedMemPerBlockOptin) {
            free_state(s);
            return fail(CNV_BAD_ARG, "grid %d too large for the mixed form (tile needs %zu B of shared memory)", n,
                        smem);
        }
        const int inner = cfg->mixed_inner_sweeps > 0 ? cfg->mixed_inner_sweeps : n;
        s->mixed_epochs = std::max(1, (inner + mixed_sweeps_per_exchange() - 1) / mixed_sweeps_per_exchange());
        s->mixed_max_outer = cfg->mixed_max_outer > 0 ? cfg->mixed_max_outer : 100;
        s->mixed_rtol = cfg->mixed_rtol > 0 ? cfg->mixed_rtol : 1e-10;
        ALLOC(s->rq, 2 * split);
        ALLOC(s->eg, 4 * split);
        cudaError_t e_ = cudaMalloc(&s->msync, mixed_sync_bytes());
        if (e_ != cudaSuccess) {
            free_state(s);
            return fail(CNV_CUDA_ERROR, "cudaMalloc: %s", cudaGetErrorString(e_));
        }
        if (cudaMemsetAsync(s->rq, 0, 2 * split * 4, s->stream) != cudaSuccess ||
            cudaMemsetAsync(s->eg, 0, 4 * split * 4, s->stream) != cudaSuccess) {
            free_state(s);
            return fail(CNV_CUDA_ERROR, "initial memset failed");
        }
    }
#undef ALLOC
    // several sweeps per exchange: one block per SM, tiles at least as wide as the halo, the
    // psi tile (and the right-hand side when it also fits) in shared memory
    const int want_sweeps = cfg->sor_blocking == 0 ? auto_sor_sweeps(n) : cfg->sor_blocking;
    if (!s->mixed && cfg->poisson_type != CNV_POISSON_DIRECT && cfg->poisson_type != CNV_POISSON_JACOBI &&
        want_sweeps > 1) {
        s->tb_sweeps = want_sweeps;
        int g = cfg->solver_blocks > 0 ? std::min(cfg->solver_blocks, s->sms) : s->sms;
        for (; g >= 1; --g) {
            poisson_tiles(n, g, &s->tb_gx, &s->tb_gy);
            if (tb_tiles_ok(n, s->tb_gx, s->tb_gy, want_sweeps)) break;
        }
        const size_t optin = prop.sharedMemPerBlockOptin;
        const bool fits = g >= 1 && tb_smem_bytes(n, s->tb_gx, s->tb_gy, want_sweeps, false) + 2048 <= optin;
        if (fits) {
            s->tb = true;
            s->tb_g_smem = tb_smem_bytes(n, s->tb_gx, s->tb_gy, want_sweeps, true) + 2048 <= optin;
            const size_t snap = tb_snapshot_doubles(n, s->pitch);
            if (buf_alloc(s, reinterpret_cast<void**>(&s->tb_snap), snap * sizeof(double), "s->tb_snap") != cudaSuccess ||
                cudaMalloc(&s->tb_sync, tb_sync_bytes()) != cudaSuccess) {
                free_state(s);
                return fail(CNV_CUDA_ERROR, "cudaMalloc failed (tiled solver buffers)");
            }
        } else if (cfg->sor_blocking > 1) {
            free_state(s);
            return fail(CNV_BAD_ARG, "grid %d too large or too small for shared-memory SOR tiles", n);
        }
    } else if (cfg->sor_blocking > 1) {
        free_state(s);
        return fail(CNV_BAD_ARG, "sor_blocking > 1 needs the FP64 SOR or Gauss-Seidel solver");
    }
    if (cfg->poisson_type == CNV_POISSON_DIRECT) {
        s->direct = true;
        if (dst_plan_create(n, s->dx, s->dy, &s->dst) != CNV_OK) {
            free_state(s);
            return fail(CNV_CUDA_ERROR, "sine-transform plan for n = %d", n);
        }
    }
    if (cudaMemsetAsync(s->ctrl, 0, sizeof(Ctrl), s->stream) != cudaSuccess ||
        cudaMemsetAsync(s->rhs[0], 0, split * 8, s->stream) != cudaSuccess ||
        cudaMemsetAsync(s->rhs[1], 0, split * 8, s->stream) != cudaSuccess) {
        free_state(s);
        return fail(CNV_CUDA_ERROR, "initial memset failed");
    }

    FdBands hb;
    rc = build_fd_bands(n, cfg->order, s->dx, s->dy, &hb);
    if (rc != CNV_OK) {
        free_state(s);
        return fail(rc, "finite-difference bands: order %d, n %d", cfg->order, n);
    }
    if (cudaMemcpy(s->bands, &hb, sizeof hb, cudaMemcpyHostToDevice) != cudaSuccess) {
        free_state(s);
        return fail(CNV_CUDA_ERROR, "band upload failed");
    }

    // Poisson parameters (src/poisson.c:247 evaluates every constant the same way)
    PoissonParams& p = s->pp;
    p.n = n;
    p.pitch = s->pitch;
    p.kind = cfg->poisson_type;
    p.arith = arith;
    p.fold = fold ? 1 : 0;
    p.itmax = cfg->poisson_max_it;
    p.tol = cfg->poisson_tol;
    // src/main.c:134 (PI of include/poisson.h:8); sor_omega > 0 overrides it
    const double pi = 3.14159265359;
    const double beta_ref = 0.5 * (2 / (1 + sin(pi / (cfg->nx + 1))) + 2 / (1 + sin(pi / (cfg->ny + 1))));
    p.beta = cfg->poisson_type == CNV_POISSON_SOR ? (cfg->sor_omega > 0 ? cfg->sor_omega : beta_ref) : 1.0;
    p.omb = 1 - p.beta;
    p.dx2 = s->dx * s->dx;
    p.dy2 = s->dy * s->dy;
    p.den = 2 * (s->dx * s->dx + s->dy * s->dy);
    p.den_pow2 = is_pow2(p.den) ? 1 : 0;
    p.rden = 1.0 / p.den;
    p.dden = div_const(p.den);
    p.wx = p.dx2 / p.den;
    p.wy = p.dy2 / p.den;
    p.b4 = p.beta / 4;
    p.kb4 = mul_const(p.b4);
    p.komb = mul_const(p.omb);
    p.timeout_ns = (cfg->solver_timeout_ms > 0 ? cfg->solver_timeout_ms : 2000) * 1000000LL;  // per wait
    p.stall_block = cfg->test_stall_block - 1;

    StepArgs& a = s->sa;
    a.n = n;
    a.pitch = s->pitch;
    a.u = s->u;
    a.v = s->v;
    a.psi = s->psi;
    for (int c = 0; c < 2; ++c) {
        a.sor[c] = s->sor[c];
        a.rhs[c] = s->direct ? nullptr : s->rhs[c];  // the direct solve reads w_out itself
    }
    a.bands = s->bands;
    a.bc = BoundaryValues{cfg->u1, cfg->u2, cfg->u3, cfg->u4, cfg->v1, cfg->v2, cfg->v3, cfg->v4};
    a.inv_re = 1. / cfg->Re;
    a.dt = cfg->dt;
    a.c4 = s->dx * s->dx * s->dy * s->dy;
    // the mixed form takes g = c4*f as it is; the FP64 forms take their scaled variants
    a.rhs_mode = s->mixed ? 0 : (p.arith == Arith::kFma ? 1 : (p.fold ? 2 : 0));
    a.rhs_div = p.dden;
    a.rhs_rden = p.rden;
    a.rhs_den_pow2 = p.den_pow2;
    a.rhs_inv_h2 = 1.0 / p.dx2;
    a.ctrl = s->ctrl;
    a.cont_partials = s->cont_partials;
    a.cont_blocks = s->cont_blocks;
    a.tile_rows = s->tile_rows;
    a.timeout_ns = p.timeout_ns;

    if (cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess ||
        cudaEventCreate(&s->evp0) != cudaSuccess || cudaEventCreate(&s->evp1) != cudaSuccess) {
        free_state(s);
        return fail(CNV_CUDA_ERROR, "cudaEventCreate failed");
    }
    rc = ensure_records(s, 64);
    if (rc == CNV_OK) rc = upload_initial(s);
    if (rc == CNV_OK && cfg->test_guard_cells == 2 && s->guards.plant("s->u") != cudaSuccess)
        rc = fail(CNV_CUDA_ERROR, "guard setup failed");  // the checker's own test: a byte after u
    if (rc != CNV_OK) {
        free_state(s);
        return rc;
    }
    *out = s;
    return CNV_OK;
}

void cnv_destroy(cnv_state* s) { free_state(s); }

int cnv_reset(cnv_state* s) {
    if (!s) return fail(CNV_BAD_ARG, "null state");
    CNV_CUDA(cudaSetDevice(s->device));
    return upload_initial(s);
}

int cnv_grid_size(const cnv_state* s) { return s ? s->n : -1; }

int cnv_set_fields(cnv_state* s, const double* w, const double* u, const double* v) {
    if (!s) return fail(CNV_BAD_ARG, "null state");
    const size_t nn = (size_t)s->n * s->n;
    CNV_CUDA(cudaSetDevice(s->device));
    // upload into a staging area and check there (a device scan costs microseconds where a host
    // scan of 3 n^2 doubles costs about a millisecond at 1024^2); the state changes only if
    // every field is finite
    if (!s->stage) CNV_CUDA(cudaMalloc(&s->stage, 3 * nn * sizeof(double)));
    const double* src[3] = {w, u, v};
    const double* dev[3] = {nullptr, nullptr, nullptr};
    for (int k = 0; k < 3; ++k) {
        if (!src[k]) continue;
        CNV_CUDA(cudaMemcpyAsync(s->stage + k * nn, src[k], nn * 8, cudaMemcpyHostToDevice, s->stream));
        dev[k] = s->stage + k * nn;
    }
    return cnv_set_fields_device(s, dev[0], dev[1], dev[2]);
}

int cnv_get_fields(cnv_state* s, double* w, double* u, double* v, double* psi) {
    if (!s) return fail(CNV_BAD_ARG, "null state");
    const size_t nn = (size_t)s->n * s->n;
    CNV_CUDA(cudaSetDevice(s->device));
    if (w) CNV_CUDA(cudaMemcpyAsync(w, s->w[s->cur], nn * 8, cudaMemcpyDeviceToHost, s->stream));
    if (u) CNV_CUDA(cudaMemcpyAsync(u, s->u, nn * 8, cudaMemcpyDeviceToHost, s->stream));
    if (v) CNV_CUDA(cudaMemcpyAsync(v, s->v, nn * 8, cudaMemcpyDeviceToHost, s->stream));
    if (psi) CNV_CUDA(cudaMemcpyAsync(psi, s->psi, nn * 8, cudaMemcpyDeviceToHost, s->stream));
    CNV_CUDA(cudaStreamSynchronize(s->stream));
    return CNV_OK;
}

int cnv_set_fields_device(cnv_state* s, const double* w, const double* u, const double* v) {
    if (!s) return fail(CNV_BAD_ARG, "null state");
    const size_t nn = (size_t)s->n * s->n;
    CNV_CUDA(cudaSetDevice(s->device));
    CNV_CUDA(cudaMemsetAsync(s->flag, 0, sizeof(int), s->stream));
    for (const double* x : {w, u, v})
        if (x) CNV_CUDA(launch_nonfinite_scan(x, (long long)nn, s->flag, s->stream));
    int bad = 0;
    CNV_CUDA(cudaMemcpyAsync(&bad, s->flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CNV_CUDA(cudaStreamSynchronize(s->stream));
    if (bad) return fail(CNV_NONFINITE, "input field holds NaN or Inf");
    if (w) CNV_CUDA(cudaMemcpyAsync(s->w[s->cur], w, nn * 8, cudaMemcpyDeviceToDevice, s->stream));
    if (u) CNV_CUDA(cudaMemcpyAsync(s->u, u, nn * 8, cudaMemcpyDeviceToDevice, s->stream));
    if (v) CNV_CUDA(cudaMemcpyAsync(s->v, v, nn * 8, cudaMemcpyDeviceToDevice, s->stream));
    CNV_CUDA(cudaStreamSynchronize(s->stream));
    return CNV_OK;
}

int cnv_get_fields_device(cnv_state* s, double* w, double* u, double* v, double* psi) {
    if (!s) return fail(CNV_BAD_ARG, "null state");
    const size_t nn = (size_t)s->n * s->n;
    CNV_CUDA(cudaSetDevice(s->device));
    if (w) CNV_CUDA(cudaMemcpyAsync(w, s->w[s->cur], nn * 8, cudaMemcpyDeviceToDevice, s->stream));
    if (u) CNV_CUDA(cudaMemcpyAsync(u, s->u, nn * 8, cudaMemcpyDeviceToDevice, s->stream));
    if (v) CNV_CUDA(cudaMemcpyAsync(v, s->v, nn * 8, cudaMemcpyDeviceToDevice, s->stream));
    if (psi) CNV_CUDA(cudaMemcpyAsync(psi, s->psi, nn * 8, cudaMemcpyDeviceToDevice, s->stream));
    CNV_CUDA(cudaStreamSynchronize(s->stream));
    return CNV_OK;
}

int cnv_step_async(cnv_state* s, int nsteps) {
    if (!s || nsteps < 0) return fail(CNV_BAD_ARG, "bad state or step count");
    CNV_CUDA(cudaSetDevice(s->device));
    int rc = ensure_records(s, std::max(nsteps, 1));
    if (rc == CNV_OK) rc = build_graphs(s);
    if (rc == CNV_OK) rc = reset_ctrl(s);
    if (rc != CNV_OK) return rc;
    s->last_steps_enqueued = nsteps;
    s->parity_at_start = s->cur;
    CNV_CUDA(cudaEventRecord(s->ev0, s->stream));
    for (int t = 0; t < nsteps; ++t) {
        rc = enqueue_step(s, s->cur);
        if (rc != CNV_OK) return rc;
        s->cur ^= 1;
    }
    CNV_CUDA(cudaEventRecord(s->ev1, s->stream));
    return CNV_OK;
}

int cnv_sync(cnv_state* s, cnv_step_info* info, int ninfo) {
    if (!s) return fail(CNV_BAD_ARG, "null state");
    CNV_CUDA(cudaSetDevice(s->device));
    Ctrl h{};
    CNV_CUDA(cudaMemcpyAsync(&h, s->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s->stream));
    const int nsteps = s->last_steps_enqueued;
    std::vector<StepRecord> rec(std::max(nsteps, 1));
    if (nsteps > 0)
        CNV_CUDA(cudaMemcpyAsync(rec.data(), s->records, sizeof(StepRecord) * nsteps, cudaMemcpyDeviceToHost,
                                 s->stream));
    CNV_CUDA(cudaStreamSynchronize(s->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->last_ms = ms;
    s->last_sweeps = h.sweeps;
    int rc = CNV_OK;
    int done = nsteps;
    if (h.abort) {
        // step h.step failed; later launches returned at once
        done = h.step;  // index of the failing step
        rc = h.status != CNV_OK ? h.status : CNV_CUDA_ERROR;
        if (done < nsteps) rec[done].status = rc;
        // the failing step ran its transport pass, so the vorticity buffer flipped once for it
        s->cur = (s->parity_at_start + done + 1) & 1;
        fail(rc, "step %d: %s", done,
             rc == CNV_NOT_CONVERGED ? "Error: maximum number of iterations achieved for Poisson equation."
             : rc == CNV_NONFINITE   ? "non-finite stop norm"
             : rc == CNV_TIMEOUT     ? "grid barrier wait timed out"
                                     : "failed");
        for (int t = done + 1; t < nsteps; ++t) rec[t] = StepRecord{0, rc, 0.0, 0.0, 0.0};
    }
    if (info)
        for (int t = 0; t < std::min(ninfo, nsteps); ++t) std::memcpy(&info[t], &rec[t], sizeof(StepRecord));
    if (rc == CNV_OK) rc = check_guards(s);
    return rc;
}

int cnv_step(cnv_state* s, int nsteps, cnv_step_info* info) {
    int rc = cnv_step_async(s, nsteps);
    if (rc != CNV_OK) return rc;
    return cnv_sync(s, info, info ? nsteps : 0);
}

int cnv_step_rows(cnv_state* s, double** w, double** u, double** v, double** psi, cnv_step_info* info) {
    if (!s || !w || !u || !v) return fail(CNV_BAD_ARG, "null argument");
    const int n = s->n;
    std::vector<double> hw((size_t)n * n), hu((size_t)n * n), hv((size_t)n * n), hp((size_t)n * n);
    for (int i = 0; i < n; ++i) {
        std::memcpy(&hw[(size_t)i * n], w[i], n * 8);
        std::memcpy(&hu[(size_t)i * n], u[i], n * 8);
        std::memcpy(&hv[(size_t)i * n], v[i], n * 8);
    }
    int rc = cnv_set_fields(s, hw.data(), hu.data(), hv.data());
    if (rc != CNV_OK) return rc;
    rc = cnv_step(s, 1, info);
    const int rc2 = cnv_get_fields(s, hw.data(), hu.data(), hv.data(), hp.data());
    if (rc2 != CNV_OK) return rc2;
    for (int i = 0; i < n; ++i) {
        std::memcpy(w[i], &hw[(size_t)i * n], n * 8);
        std::memcpy(u[i], &hu[(size_t)i * n], n * 8);
        std::memcpy(v[i], &hv[(size_t)i * n], n * 8);
        if (psi) std::memcpy(psi[i], &hp[(size_t)i * n], n * 8);
    }
    return rc;
}

int cnv_poisson_device(cnv_state* s, const double* f, double* psi_out, int* iters, double* err) {
    if (!s || !f || !psi_out) return fail(CNV_BAD_ARG, "null argument");
    CNV_CUDA(cudaSetDevice(s->device));
    int rc = ensure_records(s, 1);
    if (rc == CNV_OK) rc = reset_ctrl(s);
    if (rc != CNV_OK) return rc;
    CNV_CUDA(launch_to_split(f, s->rhs[0], s->rhs[1], s->sa, s->stream));
    CNV_CUDA(cudaEventRecord(s->ev0, s->stream));
    CNV_CUDA(cudaEventRecord(s->evp0, s->stream));
    rc = enqueue_poisson(s, f, -s->sa.c4, false);
    if (rc != CNV_OK) return rc;
    CNV_CUDA(cudaEventRecord(s->evp1, s->stream));
    CNV_CUDA(cudaEventRecord(s->ev1, s->stream));
    CNV_CUDA(launch_from_split(s->sor[0], s->sor[1], psi_out, s->n, s->pitch, s->stream));
    Ctrl h{};
    CNV_CUDA(cudaMemcpyAsync(&h, s->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s->stream));
    CNV_CUDA(cudaStreamSynchronize(s->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->last_ms = ms;
    s->last_sweeps = h.sweeps;
    if (iters) *iters = h.iters;
    if (err) *err = h.err;
    if (h.status != CNV_OK) return fail(h.status, "Poisson solve status %d", h.status);
    return check_guards(s);
}

int cnv_poisson(cnv_state* s, const double* f, double* psi, int* iters, double* err) {
    if (!s || !f || !psi) return fail(CNV_BAD_ARG, "null argument");
    const size_t nn = (size_t)s->n * s->n;
    CNV_CUDA(cudaSetDevice(s->device));
    CNV_CUDA(cudaMemcpyAsync(s->scratch, f, nn * 8, cudaMemcpyHostToDevice, s->stream));
    // reject a non-finite right-hand side before solving (scanned on the device)
    CNV_CUDA(cudaMemsetAsync(s->flag, 0, sizeof(int), s->stream));
    CNV_CUDA(launch_nonfinite_scan(s->scratch, (long long)nn, s->flag, s->stream));
    int bad = 0;
    CNV_CUDA(cudaMemcpyAsync(&bad, s->flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CNV_CUDA(cudaStreamSynchronize(s->stream));
    if (bad) return fail(CNV_NONFINITE, "right-hand side holds NaN or Inf");
    int rc = cnv_poisson_device(s, s->scratch, s->scratch + nn, iters, err);
    CNV_CUDA(cudaMemcpyAsync(psi, s->scratch + nn, nn * 8, cudaMemcpyDeviceToHost, s->stream));
    CNV_CUDA(cudaStreamSynchronize(s->stream));
    return rc;
}

int cnv_solver_info(cnv_state* s, char* buf, size_t len) {
    if (!s || !buf) return fail(CNV_BAD_ARG, "null argument");
    int w;
    if (s->direct)
        w = snprintf(buf, len, "direct-sine-transform");
    else if (s->mixed)
        w = snprintf(buf, len, "mixed grid=%d tiles=%dx%d", s->mixed_gx * s->mixed_gy, s->mixed_gx, s->mixed_gy);
    else if (s->tb)
        w = snprintf(buf, len, "sor-tiled sweeps=%d grid=%d tiles=%dx%d", s->tb_sweeps, s->tb_gx * s->tb_gy,
                     s->tb_gx, s->tb_gy);
    else
        w = snprintf(buf, len, "sor-exchange grid=%d tiles=%dx%d", s->poisson_grid, s->poisson_gx, s->poisson_gy);
    if (w < 0 || (size_t)w >= len) return fail(CNV_BAD_ARG, "buffer of %zu bytes too small", len);
    return CNV_OK;
}

int cnv_time_passes(cnv_state* s, int reps, double* pre_ms, double* post_ms) {
    if (!s || reps < 1) return fail(CNV_BAD_ARG, "null state or reps < 1");
    CNV_CUDA(cudaSetDevice(s->device));
    int rc = build_graphs(s);
    if (rc != CNV_OK) return rc;
    rc = reset_ctrl(s);
    if (rc != CNV_OK) return rc;
    const int parity = s->cur;
    float ms[2] = {0, 0};
    for (int pass = 0; pass < 2; ++pass) {
        CNV_CUDA(cudaGraphLaunch(s->graph[pass][parity], s->stream));  // warm-up
        CNV_CUDA(cudaEventRecord(s->ev0, s->stream));
        for (int r = 0; r < reps; ++r) CNV_CUDA(cudaGraphLaunch(s->graph[pass][parity], s->stream));
        CNV_CUDA(cudaEventRecord(s->ev1, s->stream));
        CNV_CUDA(cudaEventSynchronize(s->ev1));
        CNV_CUDA(cudaEventElapsedTime(&ms[pass], s->ev0, s->ev1));
    }
    if (pre_ms) *pre_ms = ms[0] / reps;
    if (post_ms) *post_ms = ms[1] / reps;
    return reset_ctrl(s) == CNV_OK ? check_guards(s) : CNV_CUDA_ERROR;
}

int cnv_last_stats(cnv_state* s, long long* sweeps, double* ms, double* poisson_ms) {
    if (!s) return fail(CNV_BAD_ARG, "null state");
    if (sweeps) *sweeps = s->last_sweeps;
    if (ms) *ms = s->last_ms;
    if (poisson_ms) {
        float pm = 0;
        CNV_CUDA(cudaEventElapsedTime(&pm, s->evp0, s->evp1));
        *poisson_ms = pm;
    }
    return CNV_OK;
}

}  // extern "C"
