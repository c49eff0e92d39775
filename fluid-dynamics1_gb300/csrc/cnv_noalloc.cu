// cnv_noalloc.cu -- a Poisson solve that allocates no device memory.
//
// Who needs this: some callers may not allocate GPU memory once they are running. Examples are
// a host application whose memory pool already owns the whole device, and a real-time loop
// that forbids cudaMalloc/cudaFree after start-up. cudaFree synchronises the whole device and
// both calls take unbounded time. Such a caller cannot create a cnv_state, because
// cnv_create allocates the working buffers. cnv_poisson_noalloc takes only the caller's input
// and output arrays and keeps every intermediate array (the two red/black copies of psi, the
// red/black right-hand side, the solver's synchronisation block, the control block) in the
// file-scope array g_scratch below.
//
// When the array is placed: the library's device code is compiled without relocatable device
// code, so g_scratch sits in a module of its own. With CUDA's default lazy module loading, that
// module (and the solver kernels' modules) are loaded onto a device when this entry point
// first runs there: the FIRST call on each device takes device memory for the array (about
// 6.3 MB) and the kernels' code. Callers make one warm-up call per device at start-up, before
// their memory pool owns the device and outside any stream capture; later calls allocate
// nothing. With CUDA_MODULE_LOADING=EAGER everything is placed when the library loads. Every
// device that has loaded the array keeps it until the process exits.
//
// Limits and sharing rules:
//   - grids up to kMaxN x kMaxN (512 x 512); larger n is rejected with CNV_BAD_ARG;
//   - all calls on a device share g_scratch, which keeps the previous call's contents. Each
//     call clears what must start at zero (psi, the control block and the solver's
//     synchronisation block), so back-to-back calls
//     are independent, but two calls whose GPU work overlaps (different streams or host
//     threads at the same time) race on the same memory and give wrong results.
//   - in host code g_scratch names a host-side stand-in, not device memory. Every call looks
//     up the array's device address on the current device with cudaGetSymbolAddress and
//     passes that to the kernels. The lookup is cheap once the module is loaded, and not
//     caching it keeps the entry point valid after the caller resets the device's context
//     (cudaDeviceReset), which frees the old array.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "cnv_kernels.h"

namespace cnv {
namespace {

constexpr int kMaxN = 512;
constexpr int kMaxPitch = ((kMaxN + 1) / 2 + 31) / 32 * 32;  // 256 doubles per split row
constexpr size_t kSplitBytes = (size_t)kMaxN * kMaxPitch * sizeof(double);
constexpr size_t kCtrlBytes = 256;
constexpr size_t kSyncBytes = 16384;                         // >= poisson_sync_bytes()
// control block | solver sync | psi set 0 (red, black) | psi set 1 (red, black) | rhs (red, black)
constexpr size_t kScratchBytes = kCtrlBytes + kSyncBytes + 6 * kSplitBytes;
static_assert(sizeof(Ctrl) <= kCtrlBytes, "control block does not fit its slot");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// This entry point has no state to hold an error string, so it reports why it failed on stderr
// and returns the status code.
int error(int status, const char* msg) {
    std::fprintf(stderr, "cnv_poisson_noalloc: %s\n", msg);
    return status;
}

}  // namespace
}  // namespace cnv

using namespace cnv;

extern "C" int cnv_poisson_noalloc(const double* f, double* psi, int n, double dx, double dy,
                                   int poisson_type, int precision, double beta, int itmax,
                                   double tol, int* iters, double* err, void* stream_handle) {
    if (!f || !psi) return error(CNV_BAD_ARG, "null input or output pointer");
    if (n < 3 || n > kMaxN)
        return error(CNV_BAD_ARG, "grid size n must be between 3 and 512 (the size of the built-in scratch array)");
    if (poisson_type < CNV_POISSON_GS || poisson_type > CNV_POISSON_JACOBI)
        return error(CNV_BAD_ARG, "poisson_type must be 1 (Gauss-Seidel), 2 (SOR) or 3 (Jacobi)");
    if (poisson_sync_bytes() > kSyncBytes) return error(CNV_CUDA_ERROR, "solver sync block too large");
    if (precision != CNV_PREC_FP64 && precision != CNV_PREC_FP64_FMA)
        return error(CNV_BAD_ARG, "precision must be fp64 (0) or fp64_fma (1)");
    if (!(dx > 0) || !(dy > 0) || itmax < 1 || !(tol >= 0))
        return error(CNV_BAD_ARG, "invalid dx, dy, itmax or tol");
    cudaStream_t stream = static_cast<cudaStream_t>(stream_handle);

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return error(CNV_NO_DEVICE, "no current CUDA device");
    // the device address of g_scratch on the current device (loads its module on the first call)
    unsigned char* base = nullptr;
    {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) return error(CNV_CUDA_ERROR, cudaGetErrorString(e));
        base = static_cast<unsigned char*>(p);
    }
    Ctrl* ctrl = reinterpret_cast<Ctrl*>(base);
    void* sync = base + kCtrlBytes;
    double* split = reinterpret_cast<double*>(base + kCtrlBytes + kSyncBytes);
    const int pitch = ((n + 1) / 2 + 31) / 32 * 32;
    const size_t split_elems = (size_t)n * pitch;  // <= kSplitBytes / 8
    const size_t slot = kSplitBytes / sizeof(double);
    double* sor0 = split;
    double* sor1 = split + slot;
    double* alt0 = split + 2 * slot;
    double* alt1 = split + 3 * slot;
    double* rhs0 = split + 4 * slot;
    double* rhs1 = split + 5 * slot;

    // Same constants, evaluated the same way, as a cnv_state built for this grid.
    PoissonParams p{};
    p.n = n;
    p.pitch = pitch;
    p.kind = poisson_type;
    p.arith = precision == CNV_PREC_FP64_FMA ? Arith::kFma : Arith::kExact;
    auto pow2 = [](double x) {
        int e;
        return x > 0 && std::frexp(x, &e) == 0.5;
    };
    p.fold = (p.arith == Arith::kExact && dx == dy && pow2(dx * dx) && pow2(2 * (dx * dx + dy * dy))) ? 1 : 0;
    p.itmax = itmax;
    p.tol = tol;
    const double pi = 3.14159265359;  // include/poisson.h:8
    const double beta_ref = 0.5 * (2 / (1 + sin(pi / (n + 1))) + 2 / (1 + sin(pi / (n + 1))));
    p.beta = poisson_type == CNV_POISSON_SOR ? (beta > 0 ? beta : beta_ref) : 1.0;
    p.omb = 1 - p.beta;
    p.dx2 = dx * dx;
    p.dy2 = dy * dy;
    p.den = 2 * (dx * dx + dy * dy);
    int e2 = 0;
    p.den_pow2 = std::frexp(p.den, &e2) == 0.5 ? 1 : 0;
    p.rden = 1.0 / p.den;
    p.dden = div_const(p.den);
    p.wx = p.dx2 / p.den;
    p.wy = p.dy2 / p.den;
    p.b4 = p.beta / 4;
    p.kb4 = mul_const(p.b4);
    p.komb = mul_const(p.omb);
    p.timeout_ns = 2000000000LL;
    p.stall_block = -1;

    StepArgs a{};
    a.n = n;
    a.pitch = pitch;
    a.c4 = dx * dx * dy * dy;
    a.rhs_mode = p.arith == Arith::kFma ? 1 : (p.fold ? 2 : 0);
    a.rhs_div = p.dden;
    a.rhs_rden = p.rden;
    a.rhs_den_pow2 = p.den_pow2;
    a.rhs_inv_h2 = 1.0 / p.dx2;

    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, poisson_kernel_ptr(p.arith, p.kind, p.fold != 0),
                                                      poisson_threads(), 0) != cudaSuccess ||
        per_sm < 1)
        return error(CNV_CUDA_ERROR, "device query failed");
    int gx = 1, gy = 1;
    poisson_tiles(n, poisson_grid_for(n, sms, per_sm), &gx, &gy);

    // Clear what must start at zero: both copies of psi (zero start, zero Dirichlet edge) and
    // the control block (status, abort flag; no step records in this mode). launch_poisson
    // clears the solver's sync block itself.
    if (cudaMemsetAsync(ctrl, 0, sizeof(Ctrl), stream) != cudaSuccess ||
        cudaMemsetAsync(sor0, 0, split_elems * sizeof(double), stream) != cudaSuccess ||
        cudaMemsetAsync(sor1, 0, split_elems * sizeof(double), stream) != cudaSuccess ||
        cudaMemsetAsync(alt0, 0, split_elems * sizeof(double), stream) != cudaSuccess ||
        cudaMemsetAsync(alt1, 0, split_elems * sizeof(double), stream) != cudaSuccess)
        return error(CNV_CUDA_ERROR, "cudaMemsetAsync failed");
    if (launch_to_split(f, rhs0, rhs1, a, stream) != cudaSuccess)
        return error(CNV_CUDA_ERROR, "right-hand-side pass failed to launch");
    PoissonLaunch L{};
    L.p = p;
    L.sor[0] = sor0;
    L.sor[1] = sor1;
    L.alt[0] = alt0;
    L.alt[1] = alt1;
    L.rhs[0] = rhs0;
    L.rhs[1] = rhs1;
    L.ctrl = ctrl;
    L.sync = sync;
    L.grid = gx * gy;
    L.gx = gx;
    L.gy = gy;
    const cudaError_t le = launch_poisson(L, stream);
    if (le != cudaSuccess) return error(CNV_CUDA_ERROR, cudaGetErrorString(le));
    if (launch_from_split(sor0, sor1, psi, n, pitch, stream) != cudaSuccess)
        return error(CNV_CUDA_ERROR, "output pass failed to launch");
    Ctrl h;
    std::memset(&h, 0, sizeof h);
    if (cudaMemcpyAsync(&h, ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess)
        return error(CNV_CUDA_ERROR, "status read-back failed");
    if (iters) *iters = h.iters;
    if (err) *err = h.err;
    if (h.status != CNV_OK) {
        return error(h.status, h.status == CNV_NOT_CONVERGED ? "maximum number of iterations reached"
                               : h.status == CNV_NONFINITE   ? "non-finite stop norm"
                                                             : "solver status not OK");
    }
    return CNV_OK;
}
