// cnv_dst.cu -- exact solve of the reference's discrete Poisson equation by sine transforms.
//
// The equation that every SOR sweep of src/poisson.c:241-272 moves towards is, on the interior
// cells (i, j) = 1 .. n-2 with psi = 0 on the edges,
//
//     den psi(i,j) - dy^2 (psi(i+1,j) + psi(i-1,j)) - dx^2 (psi(i,j+1) + psi(i,j-1)) = c4 w(i,j)
//
// (den = 2 (dx^2 + dy^2), c4 = dx^2 dy^2, f = -w). Its matrix is the Kronecker sum of two
// tridiagonal Toeplitz matrices, diagonalised by the orthonormal DST-I basis
//     S[a][b] = sqrt(2 / (m+1)) sin(pi (a+1)(b+1) / (m+1)),  m = n - 2,  S = S^T = S^-1,
// with eigenvalues lambda(a, b) = 4 dy^2 sin^2(t_a / 2) + 4 dx^2 sin^2(t_b / 2), t_k = pi (k+1)/(m+1).
// With X the interior of psi as an m x m matrix (rows i) and R = c4 w:  X = S ((S R S) ./ lambda) S,
// done as four row transforms (each pass transforms every row of its input):
//     1. along j, written transposed      (rows: j-modes b, over i)
//     2. along i, divided by lambda        (rows: b, over i-modes a)
//     3. along a (inverse), written transposed (rows: i, over b)
//     4. along b (inverse), into psi
// On the FFT path passes 2 and 3 run as one kernel (k_dst_fft_divide): they transform the same
// rows, so each block keeps its two rows in shared memory between them.
// The eigenvalues are formed as sums of squared sines, not as den - 2 dy^2 cos - 2 dx^2 cos: that
// difference cancels in the lowest modes (at n = 1024 it loses about four digits), while the
// transforms themselves are orthogonal, so the solve is accurate to a few units of rounding
// (measured against an extended-precision solve). The answer is what the reference's solver
// converges to, to rounding, at a fixed cost; the map is linear and symmetric, so the adjoint
// solve is the same call. The differentiable form uses it: a finite-difference check of the
// gradient needs a solve far tighter than an iterative stop rule gives.
//
// The row transforms. The DST-I F_k = sum_j y_j sin(pi j k / N) of a row y_1 .. y_{N-1} (N = m+1)
// comes from the real DFT of length N of w_j = sin(pi j / N)(y_j + y_{N-j}) + (y_j - y_{N-j})/2: with
// C_k + i S_k = sum_j w_j exp(2 pi i j k / N), the even outputs are F_2k = S_k and the odd ones
// follow from F_2k+1 = F_2k-1 + C_k, F_1 = C_0 / 2, a prefix sum (the method of Numerical Recipes'
// sinft, which works for any N). Two rows go into one complex sequence (real and imaginary parts)
// and are separated after the FFT by the conjugate symmetry of real transforms. The FFT is a
// mixed-radix Stockham transform (self-sorting, two shared-memory buffers, one block per row pair)
// over the prime factors p of N: each stage applies the twiddles, then a p-point DFT in its
// symmetric form (for odd p, outputs q and p-q share the sums over u_q + u_{p-q} and u_q - u_{p-q}:
// 2(p-1) multiply-adds per output pair). Per row that is about N/2 * (sum of the radices + 9)
// FP64 operations, against m^2 / 2 for a dense product: at n = 1024 (N = 1023 = 3 * 11 * 31)
// about a twentieth. Grids whose N has a prime factor above kMaxRadix, or that do not fit shared
// memory, take the dense products with S instead (each folded by the mirror symmetry
// S[b][m-1-c] = (-1)^b S[b][c]).
#include <cmath>
#include <vector>

#include "cnv_dst.h"

namespace cnv {
namespace {

// ---------------------------------------------------------------- FFT row transforms
constexpr int kFftThreads = 256;

struct FftArgs {
    int m, len, nstages;       // len = N = m + 1
    int radix[kMaxFftStages];
    int csoff[kMaxFftStages];  // offset of each stage's p-point table in cs
    int ncs;
    const double2* tw;         // exp(-2 pi i t / N), t = 0 .. N-1
    const double2* cs;         // per stage: (cos 2 pi t / p, sin 2 pi t / p), t = 0 .. p-1
    const double* sn;          // sin(pi j / N), j = 0 .. N-1
    double norm;               // sqrt(2 / N): the orthonormal DST
};

// Destination of a transform's value for row r, column c: row-major out[(r + off) * ld + c + off],
// or out[c * ld + r] when transposed, or, when red is set, the red/black split layout of an n x n
// field (cell (i, j) = (r + off, c + off) at (i + j odd ? black : red)[i * pitch + j / 2]). With
// lam_r set, the value is first divided by lam_r[r] + lam_c[c].
struct DstDest {
    double* out;
    int ld, off;
    double* red;
    double* black;
    int pitch;
    int transposed;
    const double* lam_r;
    const double* lam_c;
    __device__ __forceinline__ void put(int r, int c, double val) const {
        if (lam_r) val = val / (__ldg(lam_r + r) + __ldg(lam_c + c));
        if (transposed) {
            out[(size_t)c * ld + r] = val;
            return;
        }
        const int i = r + off, j = c + off;
        if (red) ((i + j) & 1 ? black : red)[(size_t)i * pitch + (j >> 1)] = val;
        else out[(size_t)i * ld + j] = val;
    }
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(__fma_rn(a.x, b.x, -a.y * b.y), __fma_rn(a.x, b.y, a.y * b.x));
}

// Orthonormal DST-I of two rows (a and b; b absent when two is false), read through
// load(row, c) (row 0 = a, 1 = b; c = 0 .. m-1) and written through store(row, c, value). X and T
// are the two N-long complex buffers, CS the stages' tables in shared memory. T's first 2(K+1)
// doubles hold the C_k after the FFT. Ends with a block barrier.
template <class Load, class Store>
__device__ __forceinline__ void dst_row_pair(const FftArgs& F, double2* X, double2* T, const double2* CS, bool two,
                                             Load load, Store store) {
    const int m = F.m, len = F.len;
    for (int j = threadIdx.x; j < len; j += kFftThreads) {
        // w_j = sin(pi j / N)(y_j + y_{N-j}) + (y_j - y_{N-j})/2 with y_j = X(row, j - 1); for
        // j = 0 both y_0 and y_N lie outside 1 .. m and are 0, for j >= 1 both lie inside
        const int jn = len - j;
        const bool in = j >= 1;
        const double s = __ldg(F.sn + j);
        const double a1 = in ? load(0, j - 1) : 0.0, a2 = in ? load(0, jn - 1) : 0.0;
        const double b1 = (two && in) ? load(1, j - 1) : 0.0, b2 = (two && in) ? load(1, jn - 1) : 0.0;
        X[j] = make_double2(__fma_rn(s, a1 + a2, 0.5 * (a1 - a2)), __fma_rn(s, b1 + b2, 0.5 * (b1 - b2)));
    }
    __syncthreads();
    int L = 1;  // length of the sub-transforms done so far
    for (int s = 0; s < F.nstages; ++s) {
        const int p = F.radix[s];
        const int Lp = L * p, r2 = len / Lp, nb = len / p;  // nb butterflies of p points
        const int stride = r2 * L;                           // between a butterfly's inputs
        const double2* cs = CS + F.csoff[s];
        if (p == 2) {
            for (int b = threadIdx.x; b < nb; b += kFftThreads) {
                const int k = b / L, j1 = b - k * L;
                const double2 u0 = X[k * L + j1];
                const double2 u1 = cmul(X[k * L + j1 + stride], __ldg(F.tw + j1 * r2));
                T[2 * b] = make_double2(u0.x + u1.x, u0.y + u1.y);
                T[2 * b + 1] = make_double2(u0.x - u1.x, u0.y - u1.y);
            }
            __syncthreads();
            for (int e = threadIdx.x; e < len; e += kFftThreads) {
                const int b = e >> 1, q2 = e & 1;
                const int k = b / L, j1 = b - k * L;
                X[k * Lp + j1 + L * q2] = T[e];
            }
            __syncthreads();
        } else {
            const int h = (p - 1) / 2;
            const int per = h + 1;
            // twiddled inputs: u_0, and A_q = u_q + u_{p-q}, B_q = u_q - u_{p-q} (q = 1 .. h)
            for (int e = threadIdx.x; e < nb * per; e += kFftThreads) {
                const int b = e / per, q = e - b * per;
                const int k = b / L, j1 = b - k * L;
                const int base = k * L + j1;
                if (q == 0) {
                    T[b * p] = X[base];
                } else {
                    const double2 uq = cmul(X[base + q * stride], __ldg(F.tw + q * j1 * r2));
                    const double2 up = cmul(X[base + (p - q) * stride], __ldg(F.tw + (p - q) * j1 * r2));
                    T[b * p + q] = make_double2(uq.x + up.x, uq.y + up.y);
                    T[b * p + h + q] = make_double2(uq.x - up.x, uq.y - up.y);
                }
            }
            __syncthreads();
            // outputs q2 and p - q2 of each butterfly: u_0 + C -+ i D with
            // C = sum_q A_q cos(2 pi q q2 / p), D = sum_q B_q sin(2 pi q q2 / p)
            for (int e = threadIdx.x; e < nb * per; e += kFftThreads) {
                const int b = e / per, q2 = e - b * per;
                const int k = b / L, j1 = b - k * L;
                const int ob = k * Lp + j1;
                const double2* tb = T + b * p;
                const double2 u0 = tb[0];
                if (q2 == 0) {
                    double2 acc = u0;
                    for (int q = 1; q <= h; ++q) {
                        acc.x += tb[q].x;
                        acc.y += tb[q].y;
                    }
                    X[ob] = acc;
                } else {
                    double2 C = make_double2(0.0, 0.0), D = make_double2(0.0, 0.0);
                    int t = 0;
                    for (int q = 1; q <= h; ++q) {
                        t += q2;
                        if (t >= p) t -= p;
                        const double2 w = cs[t];
                        const double2 A = tb[q], B = tb[h + q];
                        C.x = __fma_rn(A.x, w.x, C.x);
                        C.y = __fma_rn(A.y, w.x, C.y);
                        D.x = __fma_rn(B.x, w.y, D.x);
                        D.y = __fma_rn(B.y, w.y, D.y);
                    }
                    X[ob + L * q2] = make_double2(u0.x + C.x + D.y, u0.y + C.y - D.x);
                    X[ob + L * (p - q2)] = make_double2(u0.x + C.x - D.y, u0.y + C.y + D.x);
                }
            }
            __syncthreads();
        }
        L = Lp;
    }
    // separate the two real transforms: X_a(k) = (Z_k + conj Z_{N-k}) / 2, X_b(k) = (Z_k - conj Z_{N-k}) / 2i,
    // and with X(k) = C_k - i S_k (forward FFT): the even outputs F_2k = S_k; C_k kept for the odd ones
    const int K = len / 2;
    double* const Cs = reinterpret_cast<double*>(T);  // C of row a at Cs[k], of row b at Cs[K + 1 + k]
    for (int k = threadIdx.x; k <= K; k += kFftThreads) {
        const double2 zk = X[k], zc = X[k ? len - k : 0];
        Cs[k] = 0.5 * (zk.x + zc.x);
        Cs[K + 1 + k] = 0.5 * (zk.y + zc.y);
        if (k >= 1 && 2 * k <= m) {
            store(0, 2 * k - 1, -0.5 * (zk.y - zc.y) * F.norm);
            if (two) store(1, 2 * k - 1, 0.5 * (zk.x - zc.x) * F.norm);
        }
    }
    __syncthreads();
    // odd outputs F_2k+1 = C_0/2 + C_1 + ... + C_k: a prefix sum, row a by warp 0, row b by warp 1
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0 || (warp == 1 && two)) {
        const double* C = Cs + warp * (K + 1);
        const int count = (m + 1) / 2;  // odd outputs 1, 3, .. <= m
        const int chunk = (count + 31) / 32;
        const int k0 = min(count, lane * chunk), k1 = min(count, k0 + chunk);
        double own = 0.0;
        for (int k = k0; k < k1; ++k) own += C[k];
        double incl = own;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const double v = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += v;
        }
        double acc = incl - own;  // the sum over the lanes before this one
        const double half0 = 0.5 * C[0];
        for (int k = k0; k < k1; ++k) {
            acc += C[k];
            store(warp, 2 * k, (acc - half0) * F.norm);
        }
    }
    __syncthreads();
}

// Orthonormal DST-I of rows 2*blockIdx.x and 2*blockIdx.x + 1 of X(r, c) = xs * x[(r + xo) * xld
// + c + xo] (r, c < m), written to dst.
__global__ void __launch_bounds__(kFftThreads) k_dst_fft(FftArgs F, const double* __restrict__ x, int xld, int xo,
                                                          double xs, DstDest dst) {
    extern __shared__ double2 fsm[];
    double2* X = fsm;               // the sequence between stages
    double2* T = fsm + F.len;       // a stage's twiddled (and for odd p, paired) inputs
    double2* CS = fsm + 2 * F.len;  // the stages' p-point tables
    const int ra = 2 * blockIdx.x, rb = ra + 1;  // rb == m: no second row
    for (int t = threadIdx.x; t < F.ncs; t += kFftThreads) CS[t] = F.cs[t];
    const double* xr[2] = {x + (size_t)(ra + xo) * xld + xo, x + (size_t)(rb + xo) * xld + xo};
    dst_row_pair(
        F, X, T, CS, rb < F.m, [&](int row, int c) { return xs * __ldg(xr[row] + c); },
        [&](int row, int c, double v) { dst.put(row ? rb : ra, c, v); });
}

// The middle of a solve in one kernel: for rows 2*blockIdx.x, +1 of x (m x m, the j-modes b, over
// i), the DST along i, division by lam_r[b] + lam_c[a], and the DST back along a, written to dst.
// The intermediate rows stay in shared memory (Y, 2m doubles after the tables).
__global__ void __launch_bounds__(kFftThreads) k_dst_fft_divide(FftArgs F, const double* __restrict__ x,
                                                                 const double* __restrict__ lam_r,
                                                                 const double* __restrict__ lam_c, DstDest dst) {
    extern __shared__ double2 fsm[];
    double2* X = fsm;
    double2* T = fsm + F.len;
    double2* CS = fsm + 2 * F.len;
    double* Y = reinterpret_cast<double*>(CS + F.ncs);  // the two rows between the transforms
    const int m = F.m;
    const int ra = 2 * blockIdx.x, rb = ra + 1;
    const bool two = rb < m;
    for (int t = threadIdx.x; t < F.ncs; t += kFftThreads) CS[t] = F.cs[t];
    const double* xr[2] = {x + (size_t)ra * m, x + (size_t)rb * m};
    const double lr[2] = {__ldg(lam_r + ra), two ? __ldg(lam_r + rb) : 1.0};
    dst_row_pair(
        F, X, T, CS, two, [&](int row, int c) { return __ldg(xr[row] + c); },
        [&](int row, int c, double v) { Y[row * m + c] = v / (lr[row] + __ldg(lam_c + c)); });
    dst_row_pair(
        F, X, T, CS, two, [&](int row, int c) { return Y[row * m + c]; },
        [&](int row, int c, double v) { dst.put(row ? rb : ra, c, v); });
}

// ------------------------------------------------------- dense fallback: out = X * S
constexpr int kCols = 64;     // output columns per block (one per thread column)
constexpr int kRowsT = 4;     // thread rows per block
constexpr int kBk = 32;       // reduction chunk (even, so chunk-local parity = global parity)
constexpr int kThreads = kCols * kRowsT;

// X(r, b) = xs * x[(r + xo) * xld + b + xo]. Column c < half gets E + O, column m-1-c gets E - O
// (E, O: the even-b and odd-b halves of the dot product). RR rows per block.
template <int RR>
__global__ void __launch_bounds__(kThreads) k_dst_right(const double* __restrict__ S, int m,
                                                        const double* __restrict__ x, int xld, int xo, double xs,
                                                        DstDest dst) {
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
            s_x[r][bb] = (row < m && b < m) ? xs * x[(size_t)(row + xo) * xld + b + xo] : 0.0;
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
        dst.put(r, c, e[q] + o[q]);
        if (c2 != c) dst.put(r, c2, e[q] - o[q]);
    }
}

int ceil_div(int a, int b) { return (a + b - 1) / b; }

FftArgs fft_args(const DstPlan& P) {
    FftArgs F{};
    F.m = P.m;
    F.len = P.len;
    F.nstages = P.nstages;
    for (int s = 0; s < P.nstages; ++s) {
        F.radix[s] = P.radix[s];
        F.csoff[s] = P.csoff[s];
    }
    F.ncs = P.ncs;
    F.tw = P.tw;
    F.cs = P.cs;
    F.sn = P.sn;
    F.norm = std::sqrt(2.0 / (P.m + 1));
    return F;
}

// One transform along j of every row: dst(r, c) = sum_b X(r, b) S[b][c], X(r, b) = xs *
// x[(r + xo) * xld + b + xo].
cudaError_t transform_rows(const DstPlan& P, const double* x, int xld, int xo, double xs, const DstDest& d,
                           cudaStream_t s) {
    if (P.len) {
        k_dst_fft<<<ceil_div(P.m, 2), kFftThreads, P.fft_smem, s>>>(fft_args(P), x, xld, xo, xs, d);
        return cudaGetLastError();
    }
    const dim3 grid(ceil_div((P.m + 1) / 2, kCols), ceil_div(P.m, P.rows));
    switch (P.rows) {
        case 16: k_dst_right<16><<<grid, kThreads, 0, s>>>(P.S, P.m, x, xld, xo, xs, d); break;
        case 8: k_dst_right<8><<<grid, kThreads, 0, s>>>(P.S, P.m, x, xld, xo, xs, d); break;
        default: k_dst_right<4><<<grid, kThreads, 0, s>>>(P.S, P.m, x, xld, xo, xs, d); break;
    }
    return cudaGetLastError();
}

cudaError_t solve(const DstPlan& P, const double* in, double scale, const DstDest& d, cudaStream_t s) {
    const int m = P.m;
    const DstDest t1_tr{P.t1, m, 0, nullptr, nullptr, 0, 1, nullptr, nullptr};
    cudaError_t e;
    if ((e = transform_rows(P, in, P.n, 1, scale, t1_tr, s)) != cudaSuccess) return e;  // along j
    if (P.len) {
        // along i, / lambda, back along a: one kernel, the rows staying in shared memory
        const size_t smem = P.fft_smem + 2 * (size_t)m * sizeof(double);
        k_dst_fft_divide<<<ceil_div(m, 2), kFftThreads, smem, s>>>(fft_args(P), P.t1, P.lam_j, P.lam_i,
                                                                   DstDest{P.t2, m, 0, nullptr, nullptr, 0, 1,
                                                                           nullptr, nullptr});
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        return transform_rows(P, P.t2, m, 0, 1.0, d, s);  // back along b
    }
    const DstDest t2_div{P.t2, m, 0, nullptr, nullptr, 0, 0, P.lam_j, P.lam_i};  // rows b, columns a
    if ((e = transform_rows(P, P.t1, m, 0, 1.0, t2_div, s)) != cudaSuccess) return e;  // along i, / lambda
    if ((e = transform_rows(P, P.t2, m, 0, 1.0, t1_tr, s)) != cudaSuccess) return e;   // back along a
    return transform_rows(P, P.t1, m, 0, 1.0, d, s);                                     // back along b
}

// Prime factors of len (ascending), or false when one exceeds kMaxRadix or there are too many.
bool factor(int len, int* radix, int* count) {
    int c = 0;
    for (int p = 2; len > 1; ++p) {
        while (len % p == 0) {
            if (p > kMaxRadix || c == kMaxFftStages) return false;
            radix[c++] = p;
            len /= p;
        }
        if (p * p > len && len > 1) {
            if (len > kMaxRadix || c == kMaxFftStages) return false;
            radix[c++] = len;
            len = 1;
        }
    }
    *count = c;
    return true;
}

}  // namespace

int dst_plan_create(int n, double dx, double dy, DstPlan* P) {
    *P = DstPlan{};
    if (n < 3) return CNV_BAD_ARG;
    const int m = n - 2;
    P->n = n;
    P->m = m;
    P->den = 2 * (dx * dx + dy * dy);
    P->dx2 = dx * dx;
    P->dy2 = dy * dy;
    const double pi = std::acos(-1.0);
    int dev = 0, smem_max = 0, sms = 148;
    if (cudaGetDevice(&dev) != cudaSuccess) return CNV_CUDA_ERROR;
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);

    // the FFT row transforms where N = m+1 factors into small primes and fits shared memory
    const int len = m + 1;
    int radix[kMaxFftStages], ns = 0;
    if (factor(len, radix, &ns)) {
        int ncs = 0;
        for (int s = 0; s < ns; ++s) ncs += radix[s];
        const size_t smem = (2 * (size_t)len + ncs) * sizeof(double2);
        if (smem + 2 * (size_t)m * sizeof(double) <= (size_t)smem_max) {  // the fused middle pass's rows too
            P->len = len;
            P->nstages = ns;
            P->ncs = ncs;
            P->fft_smem = (int)smem;
            // tables in long double, rounded once to double
            const long double lpi = 3.141592653589793238462643383279502884L;
            std::vector<double2> tw(len), cs(ncs);
            std::vector<double> sn(len);
            for (int t = 0; t < len; ++t) {
                const long double a = 2 * lpi * t / len;  // exp(-2 pi i t / N)
                tw[t] = make_double2((double)std::cos(a), (double)-std::sin(a));
                sn[t] = (double)std::sin(lpi * t / len);
            }
            for (int s = 0, off = 0; s < ns; ++s) {
                P->radix[s] = radix[s];
                P->csoff[s] = off;
                for (int t = 0; t < radix[s]; ++t) {
                    const long double a = 2 * lpi * t / radix[s];
                    cs[off + t] = make_double2((double)std::cos(a), (double)std::sin(a));
                }
                off += radix[s];
            }
            if (cudaMalloc(&P->tw, len * sizeof(double2)) != cudaSuccess ||
                cudaMalloc(&P->cs, ncs * sizeof(double2)) != cudaSuccess ||
                cudaMalloc(&P->sn, len * sizeof(double)) != cudaSuccess ||
                cudaMemcpy(P->tw, tw.data(), len * sizeof(double2), cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(P->cs, cs.data(), ncs * sizeof(double2), cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(P->sn, sn.data(), len * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaFuncSetAttribute(k_dst_fft, cudaFuncAttributeMaxDynamicSharedMemorySize, P->fft_smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_dst_fft_divide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     P->fft_smem + 2 * m * (int)sizeof(double)) != cudaSuccess) {
                dst_plan_destroy(P);
                return CNV_CUDA_ERROR;
            }
        }
    }
    if (!P->len) {
        // dense products with the DST matrix
        std::vector<double> S((size_t)m * m);
        const double scale = std::sqrt(2.0 / (m + 1));
        const long long period = 2LL * (m + 1);
        for (int a = 0; a < m; ++a)
            for (int b = 0; b < m; ++b) {
                const long long k = ((long long)(a + 1) * (b + 1)) % period;  // exact argument reduction
                S[(size_t)a * m + b] = scale * std::sin(pi * (double)k / (m + 1));
            }
        if (cudaMalloc(&P->S, (size_t)m * m * sizeof(double)) != cudaSuccess ||
            cudaMemcpy(P->S, S.data(), (size_t)m * m * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
            dst_plan_destroy(P);
            return CNV_CUDA_ERROR;
        }
        // more, smaller blocks when the grid is small, so that every SM gets work
        const int cols = ceil_div((m + 1) / 2, kCols);
        P->rows = (cols * ceil_div(m, 16) >= 2 * sms) ? 16 : (cols * ceil_div(m, 8) >= 2 * sms) ? 8 : 4;
    }
    // eigenvalue parts 4 h^2 sin^2(pi (k+1) / (2 (m+1))), in long double, rounded once
    std::vector<double> li(m), lj(m);
    for (int k = 0; k < m; ++k) {
        const long double sk = std::sin(3.141592653589793238462643383279502884L * (k + 1) / (2.0L * (m + 1)));
        li[k] = (double)(4.0L * (long double)P->dy2 * sk * sk);
        lj[k] = (double)(4.0L * (long double)P->dx2 * sk * sk);
    }
    const size_t mm = (size_t)m * m;
    if (cudaMalloc(&P->t1, mm * sizeof(double)) != cudaSuccess || cudaMalloc(&P->t2, mm * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&P->lam_i, m * sizeof(double)) != cudaSuccess || cudaMalloc(&P->lam_j, m * sizeof(double)) != cudaSuccess ||
        cudaMemcpy(P->lam_i, li.data(), m * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(P->lam_j, lj.data(), m * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        dst_plan_destroy(P);
        return CNV_CUDA_ERROR;
    }
    return CNV_OK;
}

void dst_plan_destroy(DstPlan* P) {
    cudaFree(P->S);
    cudaFree(P->t1);
    cudaFree(P->t2);
    cudaFree(P->lam_i);
    cudaFree(P->lam_j);
    cudaFree(P->tw);
    cudaFree(P->cs);
    cudaFree(P->sn);
    *P = DstPlan{};
}

cudaError_t dst_solve(const DstPlan& P, const double* in, double scale, double* out, cudaStream_t s) {
    return solve(P, in, scale, DstDest{out, P.n, 1, nullptr, nullptr, 0, 0, nullptr, nullptr}, s);
}

cudaError_t dst_solve_split(const DstPlan& P, const double* in, double scale, double* red, double* black, int pitch,
                            cudaStream_t s) {
    return solve(P, in, scale, DstDest{nullptr, 0, 1, red, black, pitch, 0, nullptr, nullptr}, s);
}

}  // namespace cnv
