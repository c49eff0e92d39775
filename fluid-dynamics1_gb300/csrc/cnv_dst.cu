// cnv_dst.cu -- exact solve of the reference's discrete Poisson equation by sine transforms.
//
// The equation that every SOR sweep of src/poisson.c:241-272 moves towards is, on the interior
// cells (i, j) = 1 .. n-2 with psi = 0 on the edges,
//
//     den psi(i,j) - dy^2 (psi(i+1,j) + psi(i-1,j)) - dx^2 (psi(i,j+1) + psi(i,j-1)) = c4 w(i,j)
//
// (den = 2 (dx^2 + dy^2), c4 = dx^2 dy^2, f = -w). Its matrix M is the Kronecker sum of two
// tridiagonal Toeplitz matrices, diagonalised by the orthonormal DST-I basis
//     S[a][b] = sqrt(2 / (m+1)) sin(pi (a+1)(b+1) / (m+1)),  m = n - 2,  S = S^T = S^-1,
// with eigenvalues den - 2 dy^2 cos(pi (a+1)/(m+1)) - 2 dx^2 cos(pi (b+1)/(m+1)). So
//     psi = S ((S (c4 w) S) ./ Lambda) S,
// four m x m products in FP64 and one division per cell: the converged answer of the
// reference's solver to rounding, at a fixed cost, and an exactly linear, symmetric map (the
// adjoint solve is the same call). This is what the differentiable form uses: a finite-
// difference check of the gradient needs a solve far tighter than an iterative stop rule gives.
//
// Each product uses the mirror symmetry S[m-1-a][b] = (-1)^b S[a][b]: for a < ceil(m/2) the
// kernels accumulate the even-b and odd-b halves of the dot product separately (E, O) and write
// E + O to row a and E - O to row m-1-a, halving the FP64 work (m^3 / 2 fused multiply-adds per
// product). FP64 arithmetic bounds these kernels (GB300's FP64 rate is low); operands are
// staged in shared memory tiles.
#include <cmath>
#include <vector>

#include "cnv_dst.h"

namespace cnv {
namespace {

constexpr int kCols = 64;     // output columns per block (one per thread column)
constexpr int kRowsT = 4;     // thread rows per block
constexpr int kBk = 32;       // reduction chunk (even, so chunk-local parity = global parity)
constexpr int kThreads = kCols * kRowsT;

// out = S * X (left product). X(b, c) = xs * x[(b + xo) * xld + c + xo]. Row a < half of the
// block's folded rows gets E + O, row m-1-a gets E - O. RA folded rows per block (multiple of 4).
template <int RA>
__global__ void __launch_bounds__(kThreads) k_dst_left(const double* __restrict__ S, int m,
                                                       const double* __restrict__ x, int xld, int xo, double xs,
                                                       double* __restrict__ out, int old, int oo) {
    __shared__ double s_s[RA][kBk + 1];
    __shared__ double s_x[kBk][kCols];
    const int half = (m + 1) / 2;
    const int tx = threadIdx.x % kCols, ty = threadIdx.x / kCols;
    const int a0 = blockIdx.y * RA, c = blockIdx.x * kCols + tx;
    constexpr int Q = RA / kRowsT;
    double e[Q], o[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) e[q] = o[q] = 0.0;
    for (int b0 = 0; b0 < m; b0 += kBk) {
        for (int t = threadIdx.x; t < RA * kBk; t += kThreads) {
            const int r = t / kBk, bb = t % kBk;
            const int a = a0 + r, b = b0 + bb;
            s_s[r][bb] = (a < half && b < m) ? S[(size_t)a * m + b] : 0.0;
        }
        for (int t = threadIdx.x; t < kBk * kCols; t += kThreads) {
            const int bb = t / kCols, cc = t % kCols;
            const int b = b0 + bb, col = blockIdx.x * kCols + cc;
            s_x[bb][cc] = (b < m && col < m) ? xs * x[(size_t)(b + xo) * xld + col + xo] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int bb = 0; bb < kBk; bb += 2) {
            const double xe = s_x[bb][tx], xodd = s_x[bb + 1][tx];
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                e[q] = __fma_rn(s_s[ty + kRowsT * q][bb], xe, e[q]);
                o[q] = __fma_rn(s_s[ty + kRowsT * q][bb + 1], xodd, o[q]);
            }
        }
        __syncthreads();
    }
    if (c >= m) return;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int a = a0 + ty + kRowsT * q;
        if (a >= half) continue;
        out[(size_t)(a + oo) * old + c + oo] = e[q] + o[q];
        if (m - 1 - a != a) out[(size_t)(m - 1 - a + oo) * old + c + oo] = e[q] - o[q];
    }
}

// Destination of a right product: row-major out[(r + off) * ld + c + off], or, when red is
// set, the red/black split layout of an n x n field (cell (i, j) = (r + off, c + off) at
// (i + j odd ? black : red)[i * pitch + j / 2]).
struct DstDest {
    double* out;
    int ld, off;
    double* red;
    double* black;
    int pitch;
    __device__ __forceinline__ void put(int r, int c, double val) const {
        const int i = r + off, j = c + off;
        if (red) ((i + j) & 1 ? black : red)[(size_t)i * pitch + (j >> 1)] = val;
        else out[(size_t)i * ld + j] = val;
    }
};

// out = X * S (right product), optionally divided by the eigenvalues. X(r, b) = x[r * xld + b]
// (m x m scratch). Column c < half gets E + O, column m-1-c gets E - O. RR rows per block.
template <int RR>
__global__ void __launch_bounds__(kThreads) k_dst_right(const double* __restrict__ S, int m,
                                                        const double* __restrict__ x, int xld, DstDest dst,
                                                        const double* __restrict__ li,
                                                        const double* __restrict__ lj, double den) {
    __shared__ double s_x[RR][kBk + 1];
    __shared__ double s_s[kBk][kCols];
    const int half = (m + 1) / 2;
    const int tx = threadIdx.x % kCols, ty = threadIdx.x / kCols;
    const int r0 = blockIdx.y * RR, c = blockIdx.x * kCols + tx;  // folded column
    constexpr int Q = RR / kRowsT;
    double e[Q], o[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) e[q] = o[q] = 0.0;
    for (int b0 = 0; b0 < m; b0 += kBk) {
        for (int t = threadIdx.x; t < RR * kBk; t += kThreads) {
            const int r = t / kBk, bb = t % kBk;
            const int row = r0 + r, b = b0 + bb;
            s_x[r][bb] = (row < m && b < m) ? x[(size_t)row * xld + b] : 0.0;
        }
        for (int t = threadIdx.x; t < kBk * kCols; t += kThreads) {
            const int bb = t / kCols, cc = t % kCols;
            const int b = b0 + bb, col = blockIdx.x * kCols + cc;
            s_s[bb][cc] = (b < m && col < half) ? S[(size_t)b * m + col] : 0.0;  // S symmetric
        }
        __syncthreads();
#pragma unroll 8
        for (int bb = 0; bb < kBk; bb += 2) {
            const double se = s_s[bb][tx], so = s_s[bb + 1][tx];
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                e[q] = __fma_rn(s_x[ty + kRowsT * q][bb], se, e[q]);
                o[q] = __fma_rn(s_x[ty + kRowsT * q][bb + 1], so, o[q]);
            }
        }
        __syncthreads();
    }
    if (c >= half) return;
    const int c2 = m - 1 - c;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int r = r0 + ty + kRowsT * q;
        if (r >= m) continue;
        double p = e[q] + o[q], n2 = e[q] - o[q];
        if (li) {
            p = p / (den - li[r] - lj[c]);
            n2 = n2 / (den - li[r] - lj[c2]);
        }
        dst.put(r, c, p);
        if (c2 != c) dst.put(r, c2, n2);
    }
}

int ceil_div(int a, int b) { return (a + b - 1) / b; }

template <int R>
cudaError_t left(const DstPlan& P, const double* x, int xld, int xo, double xs, double* out, int old, int oo,
                 cudaStream_t s) {
    const dim3 grid(ceil_div(P.m, kCols), ceil_div((P.m + 1) / 2, R));
    k_dst_left<R><<<grid, kThreads, 0, s>>>(P.S, P.m, x, xld, xo, xs, out, old, oo);
    return cudaGetLastError();
}

template <int R>
cudaError_t right(const DstPlan& P, const double* x, const DstDest& d, bool divide, cudaStream_t s) {
    const dim3 grid(ceil_div((P.m + 1) / 2, kCols), ceil_div(P.m, R));
    k_dst_right<R><<<grid, kThreads, 0, s>>>(P.S, P.m, x, P.m, d, divide ? P.li : nullptr, divide ? P.lj : nullptr,
                                            P.den);
    return cudaGetLastError();
}

template <int R>
cudaError_t solve(const DstPlan& P, const double* in, double scale, const DstDest& d, cudaStream_t s) {
    // t1 = S (scale * in), t2 = (t1 S) ./ Lambda, t1 = S t2, out = t1 S
    const int n = P.n, m = P.m;
    const DstDest t2{P.t2, m, 0, nullptr, nullptr, 0};
    cudaError_t e;
    if ((e = left<R>(P, in, n, 1, scale, P.t1, m, 0, s)) != cudaSuccess) return e;
    if ((e = right<R>(P, P.t1, t2, true, s)) != cudaSuccess) return e;
    if ((e = left<R>(P, P.t2, m, 0, 1.0, P.t1, m, 0, s)) != cudaSuccess) return e;
    return right<R>(P, P.t1, d, false, s);
}

cudaError_t solve_any(const DstPlan& P, const double* in, double scale, const DstDest& d, cudaStream_t s) {
    switch (P.rows) {
        case 16: return solve<16>(P, in, scale, d, s);
        case 8: return solve<8>(P, in, scale, d, s);
        default: return solve<4>(P, in, scale, d, s);
    }
}

}  // namespace

int dst_plan_create(int n, double dx, double dy, DstPlan* P) {
    *P = DstPlan{};
    if (n < 3) return CNV_BAD_ARG;
    const int m = n - 2;
    P->n = n;
    P->m = m;
    P->den = 2 * (dx * dx + dy * dy);
    std::vector<double> S((size_t)m * m), li(m), lj(m);
    const double pi = std::acos(-1.0);
    const double scale = std::sqrt(2.0 / (m + 1));
    const long long period = 2LL * (m + 1);
    for (int a = 0; a < m; ++a)
        for (int b = 0; b < m; ++b) {
            const long long k = ((long long)(a + 1) * (b + 1)) % period;  // exact argument reduction
            S[(size_t)a * m + b] = scale * std::sin(pi * (double)k / (m + 1));
        }
    for (int a = 0; a < m; ++a) {
        li[a] = 2 * dy * dy * std::cos(pi * (a + 1) / (m + 1));
        lj[a] = 2 * dx * dx * std::cos(pi * (a + 1) / (m + 1));
    }
    const size_t mm = (size_t)m * m;
    if (cudaMalloc(&P->S, mm * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&P->t1, mm * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&P->t2, mm * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&P->li, m * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&P->lj, m * sizeof(double)) != cudaSuccess) {
        dst_plan_destroy(P);
        return CNV_CUDA_ERROR;
    }
    if (cudaMemcpy(P->S, S.data(), mm * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(P->li, li.data(), m * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(P->lj, lj.data(), m * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        dst_plan_destroy(P);
        return CNV_CUDA_ERROR;
    }
    // more, smaller blocks when the grid is small, so that every SM gets work
    int sms = 148;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    P->rows = (ceil_div(m, kCols) * ceil_div((m + 1) / 2, 16) >= 2 * sms) ? 16 : (ceil_div(m, kCols) * ceil_div((m + 1) / 2, 8) >= 2 * sms) ? 8 : 4;
    return CNV_OK;
}

void dst_plan_destroy(DstPlan* P) {
    cudaFree(P->S);
    cudaFree(P->t1);
    cudaFree(P->t2);
    cudaFree(P->li);
    cudaFree(P->lj);
    *P = DstPlan{};
}

cudaError_t dst_solve(const DstPlan& P, const double* in, double scale, double* out, cudaStream_t s) {
    return solve_any(P, in, scale, DstDest{out, P.n, 1, nullptr, nullptr, 0}, s);
}

cudaError_t dst_solve_split(const DstPlan& P, const double* in, double scale, double* red, double* black, int pitch,
                            cudaStream_t s) {
    return solve_any(P, in, scale, DstDest{nullptr, 0, 1, red, black, pitch}, s);
}

}  // namespace cnv
