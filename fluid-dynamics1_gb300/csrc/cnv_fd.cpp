// cnv_fd.cpp -- finite-difference bands of cnavier's Diff1/Diff2 operators.
//
// src/finitediff.c:51-153 (Diff1) and :178-292 (Diff2) build dense n x n matrices: leading
// rows at the top, a constant interior stencil, then trailing rows copied from the leading rows
// (first derivative: D[n-1-a][n-1-b] = D[a][w-1-b]; second: D[n-1-a][n-1-b] = D[a][b], for a
// leading row a of width w). Every coefficient is ((double)p / q) / h for the first derivative
// and ((double)p / q) / (h*h) for the second. All nonzeros lie within 3 columns of the
// diagonal, so a row is stored as 7 taps (offsets -3..+3); the three construction stages are
// replayed in the reference's order so that overlapping stages (small n) end with the same
// values. The 2-D operators DX = kron(I, d_x) and DY = kron(d_y, I) (src/main.c:149-152) then
// act along j and i with these taps.
#include <cstring>

#include "cnv_internal.h"

namespace cnv {
namespace {

struct Frac {
    double p, q;
};

struct Stencil {
    int lead_rows;           // rows 0 .. lead_rows-1 are written first
    int lead_width[3];       // leading row a covers columns 0 .. lead_width[a]-1
    Frac lead[3][5];
    int radius;              // interior rows r use columns r-radius .. r+radius
    Frac inner[7];
};

// Diff1, order 2 / 4 / 6 (src/finitediff.c:57-147).
const Stencil kD1[3] = {
    {1, {2, 0, 0}, {{{-1, 1}, {1, 1}}}, 1, {{-0.5, 1}, {0, 1}, {0.5, 1}}},
    {2, {2, 3, 0}, {{{-1, 1}, {1, 1}}, {{-0.5, 1}, {0, 1}, {0.5, 1}}},
     2, {{1, 12}, {-2, 3}, {0, 1}, {2, 3}, {-1, 12}}},
    {3, {2, 3, 5},
     {{{-1, 1}, {1, 1}}, {{-0.5, 1}, {0, 1}, {0.5, 1}}, {{1, 12}, {-2, 3}, {0, 1}, {2, 3}, {-1, 12}}},
     3, {{-1, 60}, {3, 20}, {-3, 4}, {0, 1}, {3, 4}, {-3, 20}, {1, 60}}},
};

// Diff2, order 2 / 4 / 6 (src/finitediff.c:183-285).
const Stencil kD2[3] = {
    {1, {4, 0, 0}, {{{2, 1}, {-5, 1}, {4, 1}, {-1, 1}}}, 1, {{1, 1}, {-2, 1}, {1, 1}}},
    {2, {4, 3, 0}, {{{2, 1}, {-5, 1}, {4, 1}, {-1, 1}}, {{1, 1}, {-2, 1}, {1, 1}}},
     2, {{-1, 12}, {4, 3}, {-5, 2}, {4, 3}, {-1, 12}}},
    {3, {4, 3, 5},
     {{{2, 1}, {-5, 1}, {4, 1}, {-1, 1}}, {{1, 1}, {-2, 1}, {1, 1}}, {{-1, 12}, {4, 3}, {-5, 2}, {4, 3}, {-1, 12}}},
     3, {{1, 90}, {-3, 20}, {3, 2}, {-49, 18}, {3, 2}, {-3, 20}, {1, 90}}},
};

inline bool put(double* band, int n, int r, int c, double val) {
    int o = c - r;
    if (r < 0 || r >= n || c < 0 || c >= n || o < -3 || o > 3) return false;
    band[r * 7 + o + 3] = val;
    return true;
}

}  // namespace

int build_band(int n, int order, int deriv, double h, double* band) {
    if ((order != 2 && order != 4 && order != 6) || (deriv != 1 && deriv != 2)) return CNV_BAD_ARG;
    if (n < (order == 6 ? 5 : 4)) return CNV_BAD_ARG;
    const Stencil& st = (deriv == 1 ? kD1 : kD2)[order / 2 - 1];
    const double scale = deriv == 1 ? h : h * h;
    std::memset(band, 0, sizeof(double) * 7 * static_cast<size_t>(n));
    for (int a = 0; a < st.lead_rows; ++a)
        for (int b = 0; b < st.lead_width[a]; ++b)
            if (!put(band, n, a, b, (double)st.lead[a][b].p / st.lead[a][b].q / scale)) return CNV_BAD_ARG;
    for (int r = st.lead_rows; r < n - st.lead_rows; ++r)
        for (int o = -st.radius; o <= st.radius; ++o) {
            const Frac& f = st.inner[o + st.radius];
            if (!put(band, n, r, r + o, (double)f.p / f.q / scale)) return CNV_BAD_ARG;
        }
    for (int a = 0; a < st.lead_rows; ++a) {
        const int w = st.lead_width[a];
        for (int b = 0; b < w; ++b) {
            const int src_col = deriv == 1 ? w - 1 - b : b;
            const double val = band[a * 7 + (src_col - a) + 3];
            if (!put(band, n, n - 1 - a, n - 1 - b, val)) return CNV_BAD_ARG;
        }
    }
    return CNV_OK;
}

namespace {
int class_rows(int n, double* band, double (*cls)[kTaps]) {
    // class c -> representative row; class 3 (interior) only exists for n >= 7
    const int rows[kClasses] = {0, 1, 2, n >= 7 ? 3 : 0, n - 3, n - 2, n - 1};
    for (int c = 0; c < kClasses; ++c)
        for (int t = 0; t < kTaps; ++t) cls[c][t] = band[rows[c] * 7 + t];
    return CNV_OK;
}
}  // namespace

int build_fd_bands(int n, int order, double dx, double dy, FdBands* out) {
    double* band = new double[7 * static_cast<size_t>(n)];
    int rc = CNV_OK;
    struct { int deriv; double h; double (*dst)[kTaps]; } jobs[4] = {
        {1, dx, out->d1x}, {1, dy, out->d1y}, {2, dx, out->d2x}, {2, dy, out->d2y}};
    for (auto& j : jobs) {
        rc = build_band(n, order, j.deriv, j.h, band);
        if (rc != CNV_OK) break;
        class_rows(n, band, j.dst);
    }
    delete[] band;
    return rc;
}

}  // namespace cnv
