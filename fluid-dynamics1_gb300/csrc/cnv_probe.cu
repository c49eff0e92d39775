// cnv_probe.cu -- FP64 arithmetic throughput of the device, measured in place.
//
// The exact Poisson update is 7 FP64 additions and multiplications per cell (no fused
// multiply-add), and on this part the FP64 pipe, not memory, bounds it. This probe gives the
// ceiling to compare against, measured on the same device in the same process: every thread
// runs kChains independent chains of a round-to-nearest multiply followed by an add (the same
// instruction mix as the update) or of fused multiply-adds, long enough that launch costs vanish.
#include <cstdio>

#include "cnv_internal.h"
#include "cnv_sor.cuh"

namespace cnv {
namespace {

constexpr int kChains = 8;
constexpr int kProbeThreads = 256;

template <bool FMA>
__global__ void __launch_bounds__(kProbeThreads) k_fp64_probe(double* out, int iters, double x, double y) {
    double a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = 1.0 + 1e-3 * (threadIdx.x + c);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) a[c] = FMA ? fma(a[c], x, y) : __dadd_rn(__dmul_rn(a[c], x), y);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += a[c];
    if (s == 12345.678) out[0] = s;  // never true for these inputs; keeps the chains live
}

// Lane-operations per second of one probe variant (an FMA counts as one operation).
template <bool FMA>
int time_probe(int sms, double* out, double* ops_per_s) {
    const int blocks = sms * 8;
    const int iters = 4096;
    const double ops = (double)blocks * kProbeThreads * iters * kChains * (FMA ? 1 : 2);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return CNV_CUDA_ERROR;
    }
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {  // the first run warms up
        cudaEventRecord(e0);
        k_fp64_probe<FMA><<<blocks, kProbeThreads>>>(out, iters, 0.9999999, 1e-7);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (cudaGetLastError() != cudaSuccess || best >= 1e30f) return CNV_CUDA_ERROR;
    *ops_per_s = ops / (best * 1e-3);
    return CNV_OK;
}

}  // namespace
}  // namespace cnv

namespace cnv {
namespace {

__global__ void k_mul_rn(const double* x, int count, double c, double* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) out[i] = mul_rn(c, x[i]);
}

__global__ void k_div_rn(const double* x, int count, DivConst d, double* out, unsigned long long* fast) {
    unsigned long long mine = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        double q;
        if (div_rn_const_fast(x[i], d, q)) ++mine;
        out[i] = div_rn_const(x[i], d);
    }
    if (mine) atomicAdd(fast, mine);
}

}  // namespace
}  // namespace cnv

extern "C" int cnv_check_mul_rn(int device, const double* x, int count, double c, double* out) {
    using namespace cnv;
    if (!x || !out || count < 0) {
        set_last_error("cnv_check_mul_rn: bad argument");
        return CNV_BAD_ARG;
    }
    if (count == 0) return CNV_OK;
    double* d = nullptr;
    const size_t bytes = (size_t)count * sizeof(double);
    int rc = CNV_OK;
    if (cudaSetDevice(device) != cudaSuccess || cudaMalloc(&d, 2 * bytes) != cudaSuccess) {
        set_last_error("cnv_check_mul_rn: device setup failed");
        return CNV_CUDA_ERROR;
    }
    if (cudaMemcpy(d, x, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = CNV_CUDA_ERROR;
    if (rc == CNV_OK) {
        k_mul_rn<<<(count + 255) / 256 < 4096 ? (count + 255) / 256 : 4096, 256>>>(d, count, c, d + count);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(out, d + count, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = CNV_CUDA_ERROR;
    }
    cudaFree(d);
    if (rc != CNV_OK) set_last_error("cnv_check_mul_rn: kernel or copy failed");
    return rc;
}

extern "C" int cnv_check_div_rn(int device, const double* x, int count, double b, double* out, long long* fast) {
    using namespace cnv;
    if (!x || !out || count < 0) {
        set_last_error("cnv_check_div_rn: bad argument");
        return CNV_BAD_ARG;
    }
    if (fast) *fast = 0;
    if (count == 0) return CNV_OK;
    double* d = nullptr;
    const size_t bytes = (size_t)count * sizeof(double);
    int rc = CNV_OK;
    if (cudaSetDevice(device) != cudaSuccess || cudaMalloc(&d, 2 * bytes + sizeof(unsigned long long)) != cudaSuccess) {
        set_last_error("cnv_check_div_rn: device setup failed");
        return CNV_CUDA_ERROR;
    }
    unsigned long long* nf = reinterpret_cast<unsigned long long*>(d + 2 * (size_t)count);
    if (cudaMemcpy(d, x, bytes, cudaMemcpyHostToDevice) != cudaSuccess || cudaMemset(nf, 0, sizeof *nf) != cudaSuccess)
        rc = CNV_CUDA_ERROR;
    if (rc == CNV_OK) {
        k_div_rn<<<(count + 255) / 256 < 4096 ? (count + 255) / 256 : 4096, 256>>>(d, count, div_const(b), d + count, nf);
        unsigned long long h = 0;
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(out, d + count, bytes, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(&h, nf, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = CNV_CUDA_ERROR;
        if (fast) *fast = (long long)h;
    }
    cudaFree(d);
    if (rc != CNV_OK) set_last_error("cnv_check_div_rn: kernel or copy failed");
    return rc;
}

extern "C" int cnv_probe_fp64(int device, double* add_mul_ops_per_s, double* fma_ops_per_s) {
    using namespace cnv;
    if (!add_mul_ops_per_s && !fma_ops_per_s) {
        set_last_error("cnv_probe_fp64: no output requested");
        return CNV_BAD_ARG;
    }
    int sms = 0;
    double* out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaMalloc(&out, sizeof(double)) != cudaSuccess) {
        set_last_error("cnv_probe_fp64: device setup failed");
        return CNV_CUDA_ERROR;
    }
    int rc = CNV_OK;
    if (add_mul_ops_per_s) rc = time_probe<false>(sms, out, add_mul_ops_per_s);
    if (rc == CNV_OK && fma_ops_per_s) rc = time_probe<true>(sms, out, fma_ops_per_s);
    cudaFree(out);
    if (rc != CNV_OK) set_last_error("cnv_probe_fp64: probe kernel failed");
    return rc;
}
