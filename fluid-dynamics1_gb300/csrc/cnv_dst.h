// cnv_dst.h -- exact Poisson solve by discrete sine transforms (internal; cnv_dst.cu).
#pragma once

#include <cuda_runtime.h>

#include "cnv_internal.h"

namespace cnv {

struct DstPlan {
    int n = 0, m = 0;          // grid size and interior size m = n - 2
    int rows = 4;              // folded rows per block of the product kernels
    double den = 0;            // 2 (dx^2 + dy^2)
    double* S = nullptr;       // m x m orthonormal DST-I matrix (symmetric)
    double* li = nullptr;      // 2 dy^2 cos(pi (a+1)/(m+1)), a = 0 .. m-1
    double* lj = nullptr;      // 2 dx^2 cos(pi (b+1)/(m+1))
    double* t1 = nullptr;      // m x m scratch
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
