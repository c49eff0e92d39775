// cnv_stencil.cuh -- device helpers shared by the step kernels and the batched kernel:
// the reference's derivative products as 7-tap bands, evaluated with round-to-nearest
// intrinsics in the reference's order (sum from 0.0 in ascending column, src/linearalg.c:258-263),
// and the velocity Dirichlet values of src/main.c:283-296.
#pragma once

#include "cnv_internal.h"

namespace cnv {

__device__ __forceinline__ int row_class(int r, int n) { return r < 3 ? r : (r >= n - 3 ? r - n + 7 : 3); }

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// Velocity with the Dirichlet values of src/main.c:283-296: the second loop there (columns
// j = 0 and j = n-1) runs last, so corners take u1/u2 (v1/v2).
__device__ __forceinline__ double vel_bc(const double* f, int n, int i, int j, double b1, double b2,
                                         double b3, double b4) {
    if (j == 0) return b1;
    if (j == n - 1) return b2;
    if (i == 0) return b3;
    if (i == n - 1) return b4;
    return f[(size_t)i * n + j];
}

// c * x rounded to nearest: on the FP64 pipe, or (MUL == kMulInt) by the exact integer multiply
// of cnv_sor.cuh where it applies (the same bits either way). A translation unit that uses kMulInt
// specialises band_mul<kMulInt> after including cnv_sor.cuh.
enum MulPipe { kMulFp64 = 0, kMulInt = 1 };
template <int MUL>
__device__ __forceinline__ double band_mul(double c, double x);
template <>
__device__ __forceinline__ double band_mul<kMulFp64>(double c, double x) {
    return dmul(c, x);
}

// sum over offsets o of band[class(j)][o] * x(i, j+o), ascending column (DX-type product)
template <int MUL = kMulFp64, class Load>
__device__ __forceinline__ double along_j(const double (*band)[kTaps], int n, int i, int j, Load x) {
    const double* c = band[row_class(j, n)];
    double acc = 0.0;
#pragma unroll
    for (int o = -3; o <= 3; ++o) {
        const int col = j + o;
        if (col >= 0 && col < n) acc = dadd(acc, band_mul<MUL>(c[o + 3], x(i, col)));
    }
    return acc;
}

// sum over offsets o of band[class(i)][o] * x(i+o, j), ascending row (DY-type product)
template <int MUL = kMulFp64, class Load>
__device__ __forceinline__ double along_i(const double (*band)[kTaps], int n, int i, int j, Load x) {
    const double* c = band[row_class(i, n)];
    double acc = 0.0;
#pragma unroll
    for (int o = -3; o <= 3; ++o) {
        const int row = i + o;
        if (row >= 0 && row < n) acc = dadd(acc, band_mul<MUL>(c[o + 3], x(row, j)));
    }
    return acc;
}

// Defect of the reference's discrete Poisson equation at one cell, in FP64 with an explicit
// operation order (shared by the mixed-precision kernels so they agree bit for bit):
//     R = g - (dy^2 (up + dn) + dx^2 (lt + rt) - den * p)
__device__ __forceinline__ double poisson_defect(double dy2, double dx2, double den, double up, double dn, double lt,
                                                 double rt, double p, double g) {
    const double ap = __fma_rn(dy2, __dadd_rn(up, dn), __fma_rn(dx2, __dadd_rn(lt, rt), __dmul_rn(-den, p)));
    return __dsub_rn(g, ap);
}

}  // namespace cnv
