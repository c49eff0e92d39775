// cnv_internal.h -- shared definitions of libcnv (not part of the C ABI).
//
// Device layout of one cavity (n x n grid, FP64 unless stated):
//   w[2]          vorticity, row-major n*n, ping-pong between steps (the transport pass reads
//                 one and writes the other: its 7-point stencils need the old neighbours)
//   u, v          velocities, row-major n*n, as src/main.c:381-383 leaves them (derivatives of
//                 psi on every cell; the Dirichlet values are applied on read, never stored)
//   psi           streamfunction, row-major n*n (written by the velocity pass, for output)
//   sor[2],alt[2] psi in red/black split layout, two copies (sweeps alternate between them):
//                 colour c = (i + j) & 1 of cell (i, j) lives at sor[c][i * pitch + (j >> 1)];
//                 a red cell's four neighbours are black and vice versa, so every sweep reads and
//                 writes unit-stride rows
//   rhs[2]        the Poisson right-hand side in the same split layout, precomputed once per
//                 step by the transport pass (c4 * f with f = -w, or its FMA-form scaling)
//   coef          finite-difference bands: 7 row classes x 7 taps per operator
//   ctrl          control block (barrier counter, status, abort flag, per-step records)
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>

#include "../../include/cnv.h"

namespace cnv {

// Row classes of the banded 1-D operators: rows 0, 1, 2, the interior, rows n-3, n-2, n-1.
// Class of row r: r < 3 ? r : r >= n - 3 ? r - n + 7 : 3. For n < 7 a row can be both a leading
// and a trailing row; the reference's operators give it the same coefficients either way.
constexpr int kClasses = 7;
constexpr int kTaps = 7;  // offsets -3 .. +3

struct FdBands {
    double d1x[kClasses][kTaps];  // first derivative along j (DX), spacing dx
    double d1y[kClasses][kTaps];  // first derivative along i (DY), spacing dy
    double d2x[kClasses][kTaps];  // second derivative along j (DX2)
    double d2y[kClasses][kTaps];  // second derivative along i (DY2)
};

// Host construction of the bands, restating src/finitediff.c:51-292 (cnv_fd.cpp).
// Returns CNV_OK or CNV_BAD_ARG (unsupported order, n too small).
int build_band(int n, int order, int deriv, double h, double* band /* n * 7 */);
int build_fd_bands(int n, int order, double dx, double dy, FdBands* out);

struct BoundaryValues {
    double u1, u2, u3, u4;  // j = 0, j = n-1, i = 0, i = n-1 (src/main.c:283-296)
    double v1, v2, v3, v4;
};

// Per-step record on the device; same layout as cnv_step_info.
struct StepRecord {
    int iters;
    int status;
    double err;
    double cont_max;
    double cont_min;
};
static_assert(sizeof(StepRecord) == sizeof(cnv_step_info), "StepRecord must mirror cnv_step_info");

struct Ctrl {
    unsigned int bar_count;   // grid barrier arrivals of the post-solve pass (re-armed by its last block)
    unsigned int cont_ticket; // last-block ticket of the continuity reduction
    int abort;                // non-zero after a failed step: later kernels return at once
    int step;                 // index of the current step within the cnv_step call
    int iters;                // result of the last Poisson solve
    int status;
    double err;
    long long sweeps;         // Poisson sweeps done since the counters were cleared
    StepRecord* records;      // device array, one record per step of the current call
    int max_records;
    int pad;
};

// Division by one constant b with the correctly rounded result (div_rn_const, cnv_sor.cuh):
// the exact update's x / den when den is not a power of two. Built on the host by div_const.
struct DivConst {
    double b;                 // the divisor
    double zh, zl;            // a two-term reciprocal: zh = RN(1/b), zl = RN(1/b - zh)
    unsigned long long babs;  // bit pattern of |b|
    int fast;                 // 1: 2^-100 <= |b| < 2^101, the range the fast path takes
};

// 1 - b*zh is a double (zh lies within half an ulp of 1/b), so one FMA gives it exactly and
// zl = RN((1 - b*zh) / b) = RN(1/b - zh).
inline DivConst div_const(double b) {
    DivConst d{};
    d.b = b;
    d.zh = 1.0 / b;
    d.zl = std::fma(-b, d.zh, 1.0) / b;
    std::memcpy(&d.babs, &b, sizeof b);
    d.babs &= 0x7fffffffffffffffull;
    const int e = (int)(d.babs >> 52);
    d.fast = e >= 1023 - 100 && e <= 1023 + 100 && std::isfinite(d.zl) ? 1 : 0;
    return d;
}

// A constant of the exact update's integer multiply (mul_rn_k, cnv_sor.cuh), prepared on the host
// so that the kernel reads its significand, exponent and sign from the launch parameters.
struct MulConst {
    double c;
    unsigned long long m;     // significand with its leading bit, 2^52 <= m < 2^53
    unsigned long long sign;  // sign bit of c, in place
    int e;                    // biased exponent of c
    int ok;                   // c is a normal number (else the FP64 multiply is used)
};

inline MulConst mul_const(double c) {
    MulConst k{};
    k.c = c;
    unsigned long long b;
    std::memcpy(&b, &c, sizeof b);
    k.sign = b & 0x8000000000000000ull;
    k.e = (int)((b >> 52) & 0x7ff);
    k.m = (b & ((1ull << 52) - 1)) | (1ull << 52);
    k.ok = k.e != 0 && k.e != 0x7ff ? 1 : 0;
    return k;
}

// Arithmetic of the SOR point update.
enum class Arith : int { kExact = 0, kFma = 1 };

struct PoissonParams {
    int n;
    int pitch;          // doubles per split-layout row
    int kind;           // CNV_POISSON_SOR / _GS / _JACOBI
    Arith arith;
    int itmax;
    double tol;
    double beta, omb;   // SOR factor and 1 - beta (beta = 1 for Gauss-Seidel)
    double dx2, dy2;    // dx*dx, dy*dy
    double den;         // 2*(dx*dx + dy*dy)
    double rden;        // 1/den when den is a power of two (then x/den == x*rden exactly)
    int den_pow2;
    DivConst dden;      // x/den otherwise (div_const(den))
    double wx, wy;      // FMA form: dx2/den, dy2/den
    double b4;          // beta / 4 (exact), folded exact form
    MulConst kb4, komb;  // b4 and omb for the folded form's integer multiply
    int fold;           // 1: exact form with power-of-two scalings folded (dx = dy, dx^2 and den powers of 2)
    long long timeout_ns;  // bound on every wait for another block
    int stall_block;       // testing only: block of the exchange kernel that never raises its flags (-1: none)
};

// Set the text cnv_last_error() returns on this thread.
void set_last_error(const char* msg);

}  // namespace cnv
