// cnv_euler.cu -- the reference's euler() on the GPU for callers that hold the derivative fields.
//
// src/fluiddyn.c:71-102 updates every point of w in place from the four vorticity derivatives
// and the velocities: w = (-u*dwdx - v*dwdy + (1./Re)*(d2wdx2 + d2wdy2))*dt + w (:98). The
// time step of cnv_step fuses this update into its transport pass; this entry point serves
// callers that compute the derivatives themselves (the reference-signature euler() of the
// compatibility library). Same operation order and round-to-nearest intrinsics as the
// transport pass, so the result equals the reference's bit for bit.
#include <algorithm>
#include <string>

#include "cnv_internal.h"

namespace cnv {
namespace {

__global__ void k_euler(double* w, const double* wx, const double* wy, const double* wxx, const double* wyy,
                        const double* u, const double* v, long long count, double inv_re, double dt) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
         k += (long long)gridDim.x * blockDim.x) {
        const double conv = __dsub_rn(__dmul_rn(-u[k], wx[k]), __dmul_rn(v[k], wy[k]));
        const double diff = __dmul_rn(inv_re, __dadd_rn(wxx[k], wyy[k]));
        w[k] = __dadd_rn(__dmul_rn(__dadd_rn(conv, diff), dt), w[k]);
    }
}

// Per-thread device staging for the host-pointer entry point: 7 arrays, grown on demand and
// kept until the process exits (no CUDA call from a destructor that may run after the runtime
// has shut down).
struct Staging {
    int device = -1;
    cudaStream_t stream = nullptr;
    double* buf = nullptr;
    long long cap = 0;  // elements per array
};
thread_local Staging t_stage;

int efail(int status, const std::string& m) {
    set_last_error(m.c_str());
    return status;
}

}  // namespace
}  // namespace cnv

using namespace cnv;

extern "C" int cnv_euler_device(double* w, const double* dwdx, const double* dwdy, const double* d2wdx2,
                                const double* d2wdy2, const double* u, const double* v, long long count, double Re,
                                double dt, void* stream) {
    if (!w || !dwdx || !dwdy || !d2wdx2 || !d2wdy2 || !u || !v || count < 0 || !(Re != 0))
        return efail(CNV_BAD_ARG, "cnv_euler: null field, negative count or Re = 0");
    if (count == 0) return CNV_OK;
    const int threads = 256;
    const long long blocks = std::min<long long>((count + threads - 1) / threads, 4096);
    k_euler<<<(unsigned)blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(w, dwdx, dwdy, d2wdx2, d2wdy2, u, v,
                                                                                count, 1. / Re, dt);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return efail(CNV_CUDA_ERROR, std::string("cnv_euler: ") + cudaGetErrorString(e));
    return CNV_OK;
}

extern "C" int cnv_euler(double* w, const double* dwdx, const double* dwdy, const double* d2wdx2,
                         const double* d2wdy2, const double* u, const double* v, long long count, double Re,
                         double dt) {
    if (!w || !dwdx || !dwdy || !d2wdx2 || !d2wdy2 || !u || !v || count < 0 || !(Re != 0))
        return efail(CNV_BAD_ARG, "cnv_euler: null field, negative count or Re = 0");
    if (count == 0) return CNV_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return efail(CNV_NO_DEVICE, "cnv_euler: no CUDA device");
    Staging& S = t_stage;
    if (S.device != dev) {
        if (S.buf) cudaFree(S.buf);
        if (S.stream) cudaStreamDestroy(S.stream);
        S.buf = nullptr;
        S.stream = nullptr;
        S.cap = 0;
        S.device = dev;
        if (cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking) != cudaSuccess)
            return efail(CNV_CUDA_ERROR, "cnv_euler: stream creation failed");
    }
    if (S.cap < count) {
        if (S.buf) cudaFree(S.buf);
        S.buf = nullptr;
        S.cap = 0;
        if (cudaMalloc(&S.buf, 7 * count * sizeof(double)) != cudaSuccess)
            return efail(CNV_CUDA_ERROR, "cnv_euler: cudaMalloc failed");
        S.cap = count;
    }
    const double* src[7] = {w, dwdx, dwdy, d2wdx2, d2wdy2, u, v};
    double* dst[7];
    const size_t bytes = count * sizeof(double);
    for (int k = 0; k < 7; ++k) {
        dst[k] = S.buf + k * S.cap;
        if (cudaMemcpyAsync(dst[k], src[k], bytes, cudaMemcpyHostToDevice, S.stream) != cudaSuccess)
            return efail(CNV_CUDA_ERROR, "cnv_euler: upload failed");
    }
    int rc = cnv_euler_device(dst[0], dst[1], dst[2], dst[3], dst[4], dst[5], dst[6], count, Re, dt, S.stream);
    if (rc != CNV_OK) return rc;
    if (cudaMemcpyAsync(w, dst[0], bytes, cudaMemcpyDeviceToHost, S.stream) != cudaSuccess ||
        cudaStreamSynchronize(S.stream) != cudaSuccess)
        return efail(CNV_CUDA_ERROR, "cnv_euler: download failed");
    return CNV_OK;
}
