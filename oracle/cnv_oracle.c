/*
 * cnv_oracle.c -- CPU restatement of cnavier's vorticity-streamfunction time step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker for the CUDA path; see cnv_oracle.h). Build with
 * -ffp-contract=off: every expression below must round exactly as the reference's does, and
 * aarch64 gcc contracts a*b+c into an FMA by default.
 *
 * Each function names the reference lines it follows (SorinBetisor/fluid-dynamics1).
 */
#include "cnv_oracle.h"

#include <math.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define BAND(b, r, o) ((b)[(size_t)(r) * 7 + ((o) + 3)])

/* ---------------------------------------------------------------------------------------
 * Finite-difference bands (src/finitediff.c:51-153 and :178-292).
 *
 * The reference fills a dense n x n matrix in three stages: the leading rows (0, 1, 2 as the
 * order needs), the interior rows, then trailing rows copied from the leading rows. Every
 * coefficient is written as ((double)num / den) / s with s = dx (first derivative) or
 * s = dx*dx (second derivative). The trailing copy for leading row a of width w writes
 *     D[n-1-a][n-1-b] = D[a][w-1-b]   (first derivative, b = 0..w-1)
 *     D[n-1-a][n-1-b] = D[a][b]       (second derivative)
 * in ascending a, then b. The stages are replayed here in the same order so that small n,
 * where the stages overlap, gives the same final values.
 * ------------------------------------------------------------------------------------- */
typedef struct {
    int width;               /* leading row occupies columns 0 .. width-1 */
    double num[5], den[5];
} lead_row;

typedef struct {
    int n_lead;              /* leading rows 0 .. n_lead-1 */
    lead_row lead[3];
    int radius;              /* interior stencil half-width */
    double num[7], den[7];   /* interior stencil, offsets -radius .. +radius */
} fd_rule;

/* first derivative, src/finitediff.c:57-147 */
static const fd_rule D1_O2 = {1, {{2, {-1., 1.}, {1, 1}}}, 1, {-0.5, 0., 0.5}, {1, 1, 1}};
static const fd_rule D1_O4 = {2,
                              {{2, {-1, 1}, {1, 1}}, {3, {-0.5, 0, 0.5}, {1, 1, 1}}},
                              2, {1, -2, 0, 2, -1}, {12, 3, 1, 3, 12}};
static const fd_rule D1_O6 = {3,
                              {{2, {-1, 1}, {1, 1}},
                               {3, {-0.5, 0, 0.5}, {1, 1, 1}},
                               {5, {1, -2, 0, 2, -1}, {12, 3, 1, 3, 12}}},
                              3, {-1, 3, -3, 0, 3, -3, 1}, {60, 20, 4, 1, 4, 20, 60}};
/* second derivative, src/finitediff.c:183-285 */
static const fd_rule D2_O2 = {1, {{4, {2., -5., 4., -1.}, {1, 1, 1, 1}}}, 1, {1., -2., 1.}, {1, 1, 1}};
static const fd_rule D2_O4 = {2,
                              {{4, {2, -5, 4, -1}, {1, 1, 1, 1}}, {3, {1, -2, 1}, {1, 1, 1}}},
                              2, {-1, 4, -5, 4, -1}, {12, 3, 2, 3, 12}};
static const fd_rule D2_O6 = {3,
                              {{4, {2, -5, 4, -1}, {1, 1, 1, 1}},
                               {3, {1, -2, 1}, {1, 1, 1}},
                               {5, {-1, 4, -5, 4, -1}, {12, 3, 2, 3, 12}}},
                              3, {1, -3, 3, -49, 3, -3, 1}, {90, 20, 2, 18, 2, 20, 90}};

static int band_put(double *band, int n, int r, int c, double val)
{
    if (r < 0 || r >= n || c < 0 || c >= n || c - r < -3 || c - r > 3) return -1;
    BAND(band, r, c - r) = val;
    return 0;
}

int orc_fd_band(int n, int order, int deriv, double h, double *band)
{
    const fd_rule *rule;
    double s;
    int a, b, r, o;

    if (deriv == 1) rule = order == 2 ? &D1_O2 : order == 4 ? &D1_O4 : order == 6 ? &D1_O6 : NULL;
    else if (deriv == 2) rule = order == 2 ? &D2_O2 : order == 4 ? &D2_O4 : order == 6 ? &D2_O6 : NULL;
    else rule = NULL;
    if (rule == NULL || n < (order == 6 ? 5 : 4)) return ORC_BAD_ARG;

    s = deriv == 1 ? h : h * h;
    memset(band, 0, sizeof(double) * (size_t)n * 7);

    for (a = 0; a < rule->n_lead; ++a)
        for (b = 0; b < rule->lead[a].width; ++b)
            if (band_put(band, n, a, b, (double)rule->lead[a].num[b] / rule->lead[a].den[b] / s))
                return ORC_BAD_ARG;
    for (r = rule->n_lead; r < n - rule->n_lead; ++r)
        for (o = -rule->radius; o <= rule->radius; ++o)
            if (band_put(band, n, r, r + o,
                         (double)rule->num[o + rule->radius] / rule->den[o + rule->radius] / s))
                return ORC_BAD_ARG;
    for (a = 0; a < rule->n_lead; ++a) {
        int w = rule->lead[a].width;
        for (b = 0; b < w; ++b) {
            int src_c = deriv == 1 ? w - 1 - b : b;
            double val = BAND(band, a, src_c - a);
            if (band_put(band, n, n - 1 - a, n - 1 - b, val)) return ORC_BAD_ARG;
        }
    }
    return ORC_OK;
}

/* DX x: the reference forms DX = kron(I, d_x) (src/main.c:149) and multiplies it into the
 * row-major flattening of x (src/main.c:298-341). Row i*n+j of that product is
 * sum_c d_x[j][c] * x[i][c], accumulated from 0.0 in ascending c (src/linearalg.c:258-263). */
void orc_apply_j(int n, const double *band, const double *x, double *d)
{
    int i;
#pragma omp parallel for schedule(static) if (n >= 256)
    for (i = 0; i < n; ++i) {
        int j, o;
        for (j = 0; j < n; ++j) {
            double acc = 0.0;
            for (o = -3; o <= 3; ++o) {
                int c = j + o;
                if (c >= 0 && c < n) acc += BAND(band, j, o) * x[(size_t)i * n + c];
            }
            d[(size_t)i * n + j] = acc;
        }
    }
}

/* DY x with DY = kron(d_y, I) (src/main.c:150): sum_c d_y[i][c] * x[c][j], ascending c. */
void orc_apply_i(int n, const double *band, const double *x, double *d)
{
    int i;
#pragma omp parallel for schedule(static) if (n >= 256)
    for (i = 0; i < n; ++i) {
        int j, o;
        for (j = 0; j < n; ++j) {
            double acc = 0.0;
            for (o = -3; o <= 3; ++o) {
                int c = i + o;
                if (c >= 0 && c < n) acc += BAND(band, i, o) * x[(size_t)c * n + j];
            }
            d[(size_t)i * n + j] = acc;
        }
    }
}

/* euler(), src/fluiddyn.c:71-102; the update expression is the one of src/fluiddyn.c:98. */
void orc_euler(int n, double *w, const double *wx, const double *wy, const double *wxx,
               const double *wyy, const double *u, const double *v, double re, double dt)
{
    long k, nn = (long)n * n;
#pragma omp parallel for schedule(static) if (n >= 256)
    for (k = 0; k < nn; ++k)
        w[k] = (-u[k] * wx[k] - v[k] * wy[k] + (1. / re) * (wxx[k] + wyy[k])) * dt + w[k];
}

/* ---------------------------------------------------------------------------------------
 * Poisson solvers, src/poisson.c.
 * ------------------------------------------------------------------------------------- */
typedef struct {
    double dx2, dy2, c4, den, beta, omb;
} sor_coef;

static sor_coef make_coef(const orc_params *p, double beta)
{
    sor_coef c;
    c.dx2 = p->dx * p->dx;
    c.dy2 = p->dy * p->dy;
    c.c4 = p->dx * p->dx * p->dy * p->dy;
    c.den = 2 * (p->dx * p->dx + p->dy * p->dy);
    c.beta = beta;
    c.omb = 1 - beta;
    return c;
}

/* SOR point update of src/poisson.c:247 / :268. old is u0[i][j], the value at sweep start. */
static inline double sor_point(const sor_coef *c, double up, double dn, double rt, double lt,
                               double f, double old)
{
    return c->beta * (c->dy2 * (up + dn) + c->dx2 * (rt + lt) - c->c4 * f) / c->den + c->omb * old;
}

/* Gauss-Seidel / Jacobi point update of src/poisson.c:84 (no relaxation). */
static inline double gs_point(const sor_coef *c, double up, double dn, double rt, double lt, double f)
{
    return (c->dy2 * (up + dn) + c->dx2 * (rt + lt) - c->c4 * f) / c->den;
}

/* Stop norm of src/poisson.c:34-60: sum over all cells of |u - u0|. */
static double stop_norm(const orc_params *p, const double *u, const double *u0)
{
    int n = p->n;
    if (p->exact_norm) {
        double e = 0;
        long k, nn = (long)n * n;
        for (k = 0; k < nn; ++k) e += sqrt(pow(u[k] - u0[k], 2));
        return e;
    } else {
        double e = 0;
        double *row = (double *)malloc(sizeof(double) * n);
        int i;
#pragma omp parallel for schedule(static) if (n >= 256)
        for (i = 0; i < n; ++i) {
            double s = 0;
            int j;
            for (j = 0; j < n; ++j) s += fabs(u[(size_t)i * n + j] - u0[(size_t)i * n + j]);
            row[i] = s;
        }
        for (i = 0; i < n; ++i) e += row[i];
        free(row);
        return e;
    }
}

/* One red or black half-sweep (src/poisson.c:241-261): cells with (i + j) % 2 == color. */
static void sor_color(const orc_params *p, const sor_coef *c, double *u, const double *u0,
                      const double *f, int color, int relax)
{
    int n = p->n, i;
#pragma omp parallel for schedule(static) if (n >= 128)
    for (i = 1; i < n - 1; ++i) {
        int j0 = ((i + 1) % 2 == color) ? 1 : 2, j;
        for (j = j0; j < n - 1; j += 2) {
            size_t k = (size_t)i * n + j;
            u[k] = relax ? sor_point(c, u[k + n], u[k - n], u[k + 1], u[k - 1], f[k], u0[k])
                         : gs_point(c, u[k + n], u[k - n], u[k + 1], u[k - 1], f[k]);
        }
    }
}

int orc_poisson(const orc_params *p, const double *f, double *psi, int *iters, double *err)
{
    int n = p->n, k;
    size_t nn = (size_t)n * n;
    double *u0, *tmp = NULL;
    double e = 0;
    int relax = p->poisson_type == ORC_POISSON_SOR;
    sor_coef c = make_coef(p, relax ? p->beta : 1.0);

    if (n < 3 || p->itmax < 0) return ORC_BAD_ARG;
#ifdef _OPENMP
    if (p->threads > 0) omp_set_num_threads(p->threads);
#endif
    u0 = (double *)calloc(nn, sizeof(double));
    if (p->poisson_type == ORC_POISSON_JACOBI) tmp = (double *)calloc(nn, sizeof(double));
    memset(psi, 0, sizeof(double) * nn); /* fresh zero start, src/poisson.c:117 / :229 */

    for (k = 0; k < p->itmax; ++k) {
        memcpy(u0, psi, sizeof(double) * nn); /* mtrxcpy(u0, u), src/poisson.c:236 */
        if (p->poisson_type == ORC_POISSON_JACOBI) {
            int i;
#pragma omp parallel for schedule(static) if (n >= 128)
            for (i = 1; i < n - 1; ++i) {
                int j;
                for (j = 1; j < n - 1; ++j) {
                    size_t q = (size_t)i * n + j;
                    tmp[q] = gs_point(&c, u0[q + n], u0[q - n], u0[q + 1], u0[q - 1], f[q]);
                }
            }
            {
                int i2;
                for (i2 = 1; i2 < n - 1; ++i2)
                    memcpy(psi + (size_t)i2 * n + 1, tmp + (size_t)i2 * n + 1, sizeof(double) * (n - 2));
            }
        } else if (p->ordering == ORC_ORDER_REDBLACK) {
            sor_color(p, &c, psi, u0, f, 0, relax);
            sor_color(p, &c, psi, u0, f, 1, relax);
        } else {
            int i, j;
            for (i = 1; i < n - 1; ++i)
                for (j = 1; j < n - 1; ++j) {
                    size_t q = (size_t)i * n + j;
                    psi[q] = relax ? sor_point(&c, psi[q + n], psi[q - n], psi[q + 1], psi[q - 1], f[q], u0[q])
                                   : gs_point(&c, psi[q + n], psi[q - n], psi[q + 1], psi[q - 1], f[q]);
                }
        }
        e = stop_norm(p, psi, u0); /* src/poisson.c:272 */
        if (e < p->tol) {
            if (iters) *iters = k;
            if (err) *err = e;
            free(u0);
            free(tmp);
            return ORC_OK;
        }
    }
    if (iters) *iters = p->itmax;
    if (err) *err = e;
    free(u0);
    free(tmp);
    return ORC_NOT_CONVERGED;
}

double orc_sor_beta(int nx, int ny)
{
    /* src/main.c:134 with PI as defined in include/poisson.h:8 */
    const double pi = 3.14159265359;
    return 0.5 * (2 / (1 + sin(pi / (nx + 1))) + 2 / (1 + sin(pi / (ny + 1))));
}

void orc_smooth_pass(int n, const double *src, double *dst)
{
    int i, j;
    memcpy(dst, src, sizeof(double) * (size_t)n * n);
    for (i = 1; i < n - 1; ++i)
        for (j = 1; j < n - 1; ++j) {
            size_t k = (size_t)i * n + j;
            dst[k] = (src[k - n] + src[k + n] + src[k - 1] + src[k + 1]) / 4;
        }
}

/* ---------------------------------------------------------------------------------------
 * The time step, src/main.c:283-395.
 * ------------------------------------------------------------------------------------- */
int orc_run(const orc_params *p, int nsteps, double *w, double *u, double *v, double *psi,
            orc_step_info *info)
{
    int n = p->n, t, i, j, rc = ORC_OK;
    size_t nn = (size_t)n * n;
    double *d1x, *d1y, *d2x, *d2y;
    double *a, *b, *c, *d, *f;

    if (n < 4 || nsteps < 0) return ORC_BAD_ARG;
#ifdef _OPENMP
    if (p->threads > 0) omp_set_num_threads(p->threads);
#endif
    d1x = (double *)malloc(sizeof(double) * nn / n * 7);
    d1y = (double *)malloc(sizeof(double) * nn / n * 7);
    d2x = (double *)malloc(sizeof(double) * nn / n * 7);
    d2y = (double *)malloc(sizeof(double) * nn / n * 7);
    /* src/main.c:142-145: d_x uses dx, d_y uses dy */
    if (orc_fd_band(n, p->order, 1, p->dx, d1x) || orc_fd_band(n, p->order, 1, p->dy, d1y) ||
        orc_fd_band(n, p->order, 2, p->dx, d2x) || orc_fd_band(n, p->order, 2, p->dy, d2y)) {
        free(d1x); free(d1y); free(d2x); free(d2y);
        return ORC_BAD_ARG;
    }
    a = (double *)malloc(sizeof(double) * nn);
    b = (double *)malloc(sizeof(double) * nn);
    c = (double *)malloc(sizeof(double) * nn);
    d = (double *)malloc(sizeof(double) * nn);
    f = (double *)malloc(sizeof(double) * nn);

    for (t = 0; t < nsteps; ++t) {
        int it = 0;
        double e = 0, cmax, cmin;
        long k;

        /* Dirichlet velocities, src/main.c:283-296 (the second loop sets the corners) */
        for (j = 0; j < n; ++j) {
            v[j] = p->v_bc[2];
            v[(size_t)(n - 1) * n + j] = p->v_bc[3];
            u[j] = p->u_bc[2];
            u[(size_t)(n - 1) * n + j] = p->u_bc[3];
        }
        for (i = 0; i < n; ++i) {
            v[(size_t)i * n] = p->v_bc[0];
            v[(size_t)i * n + n - 1] = p->v_bc[1];
            u[(size_t)i * n] = p->u_bc[0];
            u[(size_t)i * n + n - 1] = p->u_bc[1];
        }

        /* wall vorticity w = dv/dx - du/dy on the four edges, src/main.c:298-320 */
        orc_apply_i(n, d1y, u, a); /* dudy = DY u */
        orc_apply_j(n, d1x, v, b); /* dvdx = DX v */
        for (j = 0; j < n; ++j) {
            w[j] = b[j] - a[j];
            w[(size_t)(n - 1) * n + j] = b[(size_t)(n - 1) * n + j] - a[(size_t)(n - 1) * n + j];
        }
        for (i = 0; i < n; ++i) {
            w[(size_t)i * n] = b[(size_t)i * n] - a[(size_t)i * n];
            w[(size_t)i * n + n - 1] = b[(size_t)i * n + n - 1] - a[(size_t)i * n + n - 1];
        }

        /* vorticity derivatives and the Euler update, src/main.c:323-344 */
        orc_apply_j(n, d1x, w, a); /* dwdx   = DX  w */
        orc_apply_i(n, d1y, w, b); /* dwdy   = DY  w */
        orc_apply_j(n, d2x, w, c); /* d2wdx2 = DX2 w */
        orc_apply_i(n, d2y, w, d); /* d2wdy2 = DY2 w */
        orc_euler(n, w, a, b, c, d, u, v, p->re, p->dt);

        /* streamfunction, src/main.c:347-363: f = -w (invsig) */
        for (k = 0; k < (long)nn; ++k) f[k] = -w[k];
        if (orc_poisson(p, f, psi, &it, &e) != ORC_OK) rc = ORC_NOT_CONVERGED;

        /* velocities u = DY psi, v = -(DX psi), src/main.c:366-383 */
        orc_apply_i(n, d1y, psi, u);
        orc_apply_j(n, d1x, psi, v);
        for (k = 0; k < (long)nn; ++k) v[k] = -v[k];

        /* continuity diagnostic DX u + DY v, src/main.c:387-408 */
        orc_apply_j(n, d1x, u, a);
        orc_apply_i(n, d1y, v, b);
        cmax = -DBL_MAX;
        cmin = DBL_MAX;
        for (k = 0; k < (long)nn; ++k) {
            double q = a[k] + b[k];
            if (q > cmax) cmax = q;
            if (q < cmin) cmin = q;
        }
        if (info) {
            info[t].iters = it;
            info[t].err = e;
            info[t].cont_max = cmax;
            info[t].cont_min = cmin;
            info[t].status = rc;
        }
        if (rc != ORC_OK) break;
    }
    free(d1x); free(d1y); free(d2x); free(d2y);
    free(a); free(b); free(c); free(d); free(f);
    return rc;
}
