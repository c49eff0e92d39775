// cnv_dst.h -- exact Poisson solve by discrete sine transforms (internal; cnv_dst.cu).
#pragma once

#include <cuda_runtime.h>

#include "cnv_internal.h"

namespace cnv {

constexpr int kMaxFftStages = 24;  // prime factors of the FFT length
constexpr int kMaxRadix = 251;     // largest prime factor of n - 1 the FFT row transform takes

struct DstPlan {
    int n = 0, m = 0;          // grid size and interior size m = n - 2
    double den = 0;            // 2 (dx^2 + dy^2)
    double dx2 = 0, dy2 = 0;
    // FFT row transforms (len = N = m + 1 > 0), else dense products with S
    int len = 0;
    int nstages = 0;
    int radix[kMaxFftStages] = {};
    int csoff[kMaxFftStages] = {};
    int ncs = 0;
    int fft_smem = 0;          // dynamic shared memory of the FFT kernel
    double2* tw = nullptr;     // exp(-2 pi i t / N)
    double2* cs = nullptr;     // per stage: (cos, sin)(2 pi t / p)
    double* sn = nullptr;      // sin(pi j / N)
    int rows = 4;              // rows per block of the dense product kernel
    double* S = nullptr;       // m x m orthonormal DST-I matrix (symmetric), dense path only
    double* lam_i = nullptr;   // 4 dy^2 sin^2(pi (a+1) / (2 (m+1))): the eigenvalue part along i
    double* lam_j = nullptr;   // 4 dx^2 sin^2(pi (b+1) / (2 (m+1))): along j
    double* t1 = nullptr;      // m x m scratch between the passes
    double* t2 = nullptr;
};

int dst_plan_create(int n, double dx, double dy, DstPlan* plan);
void dst_plan_destroy(DstPlan* plan);

// out(interior) = M^-1 (scale * in(interior)): in and out are n x n row-major; the edges of
// `in` are not read and the edges of `out` are not written. With scale = c4 and in = w this
// is the converged streamfunction of the reference's solver for f = -w.
cudaError_t dst_solve(const DstPlan& plan, const double* in, double scale, double* out, cudaStream_t s);
// The same solve with the result written into the red/black split layout (the layout the
// velocity pass reads); edge cells are not written.
cudaError_t dst_solve_split(const DstPlan& plan, const double* in, double scale, double* red, double* black,
                            int pitch, cudaStream_t s);

}  // namespace cnv
