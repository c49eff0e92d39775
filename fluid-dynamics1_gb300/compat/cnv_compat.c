/*
 * cnv_compat.c -- the reference's poisson and euler entry points on top of libcnv (cnv_compat.h).
 *
 * poisson* keep one cnv_state per distinct (n, Lx, Ly, solver, beta, itmax, tol) -- the
 * reference's main calls them with the same arguments every step, so after the first call
 * each solve is an upload of f, the persistent GPU solver, and a download of psi. States live
 * until the process exits.
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cnv.h"
#include "cnv_compat.h"

#define MAX_CACHED 8

typedef struct {
    int n, Lx, Ly, type, itmax;
    double beta, tol;
    cnv_state *s;
} cached_state;

static cached_state g_cache[MAX_CACHED];
static int g_cached = 0;
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

static void die(const char *what) {
    printf("** Error: %s **\n", what);
    exit(1);
}

/* L with (double)L / n == h exactly, or -1 */
static int whole_length(double h, int n) {
    double L = floor(h * n + 0.5);
    if (L < 1 || L > 1e9 || (double)(int)L / n != h) return -1;
    return (int)L;
}

static double **rows_alloc(int m, int n) {
    double **A = (double **)malloc(m * sizeof(double *));
    int i;
    if (!A) die("insufficient memory");
    for (i = 0; i < m; ++i) {
        A[i] = (double *)malloc(n * sizeof(double));
        if (!A[i]) die("insufficient memory");
    }
    return A;
}

static cnv_state *state_for(int n, int Lx, int Ly, int type, double beta, int itmax, double tol) {
    cnv_state *s = NULL;
    int k;
    pthread_mutex_lock(&g_lock);
    for (k = 0; k < g_cached; ++k) {
        cached_state *c = &g_cache[k];
        if (c->n == n && c->Lx == Lx && c->Ly == Ly && c->type == type && c->beta == beta && c->itmax == itmax &&
            c->tol == tol) {
            s = c->s;
            break;
        }
    }
    if (!s) {
        cnv_config cfg;
        cnv_config_default(&cfg);
        cfg.nx = cfg.ny = n;
        cfg.Lx = Lx;
        cfg.Ly = Ly;
        cfg.poisson_type = type;
        cfg.sor_omega = beta;
        cfg.poisson_max_it = itmax;
        cfg.poisson_tol = tol;
        cfg.order = n >= 5 ? 6 : 2; /* the operators are not used by a Poisson solve */
        if (cnv_create(&cfg, &s) != CNV_OK) {
            pthread_mutex_unlock(&g_lock);
            printf("** Error: %s **\n", cnv_last_error());
            exit(1);
        }
        if (g_cached == MAX_CACHED) { /* evict the oldest */
            cnv_destroy(g_cache[0].s);
            memmove(g_cache, g_cache + 1, sizeof(cached_state) * (MAX_CACHED - 1));
            --g_cached;
        }
        g_cache[g_cached].n = n;
        g_cache[g_cached].Lx = Lx;
        g_cache[g_cached].Ly = Ly;
        g_cache[g_cached].type = type;
        g_cache[g_cached].beta = beta;
        g_cache[g_cached].itmax = itmax;
        g_cache[g_cached].tol = tol;
        g_cache[g_cached].s = s;
        ++g_cached;
    }
    pthread_mutex_unlock(&g_lock);
    return s;
}

static void say(FILE *log_file, int to_stdout, const char *line) {
    if (to_stdout) {
        fputs(line, stdout);
    } else if (log_file) {
        fputs(line, log_file);
        fflush(log_file);
    }
}

/* One solve with the reference's behaviour: new psi, message, exit(1) on non-convergence. */
static mtrx solve(mtrx f, double dx, double dy, int itmax, double tol, int type, double beta, FILE *log_file,
                  int to_stdout) {
    const int n = f.m;
    int Lx, Ly, it = 0, i, rc;
    double err = 0;
    double *flat, *out;
    mtrx psi;
    char line[160];
    cnv_state *s;

    if (f.M == NULL || f.m < 1 || f.n < 1) die("invalid parameter");
    if (f.m != f.n) die("the GPU Poisson solve needs a square field");
    Lx = whole_length(dx, n);
    Ly = whole_length(dy, n);
    if (Lx < 0 || Ly < 0) die("dx * n and dy * n must be whole numbers");
    s = state_for(n, Lx, Ly, type, type == CNV_POISSON_SOR ? beta : 0.0, itmax, tol);
    flat = (double *)malloc(sizeof(double) * (size_t)n * n * 2);
    if (!flat) die("insufficient memory");
    out = flat + (size_t)n * n;
    for (i = 0; i < n; ++i) memcpy(flat + (size_t)i * n, f.M[i], sizeof(double) * n);
    rc = cnv_poisson(s, flat, out, &it, &err);
    if (rc == CNV_NOT_CONVERGED) {
        free(flat);
        say(log_file, to_stdout, "Error: maximum number of iterations achieved for Poisson equation.\n");
        exit(1);
    }
    if (rc != CNV_OK) {
        free(flat);
        printf("** Error: %s **\n", cnv_last_error());
        exit(1);
    }
    snprintf(line, sizeof line, "Poisson equation solved with %d iterations - root-sum-of-squares error: %E\n", it,
             err);
    say(log_file, to_stdout, line);
    psi.m = n;
    psi.n = n;
    psi.M = rows_alloc(n, n);
    for (i = 0; i < n; ++i) memcpy(psi.M[i], out + (size_t)i * n, sizeof(double) * n);
    free(flat);
    return psi;
}

mtrx poisson(mtrx f, double dx, double dy, int itmax, double tol) {
    return solve(f, dx, dy, itmax, tol, CNV_POISSON_GS, 1.0, NULL, 1);
}

mtrx poisson_SOR(mtrx f, double dx, double dy, int itmax, double tol, double beta) {
    return solve(f, dx, dy, itmax, tol, CNV_POISSON_SOR, beta, NULL, 1);
}

mtrx poisson_log(mtrx f, double dx, double dy, int itmax, double tol, FILE *log_file) {
    return solve(f, dx, dy, itmax, tol, CNV_POISSON_GS, 1.0, log_file, 0);
}

mtrx poisson_SOR_log(mtrx f, double dx, double dy, int itmax, double tol, double beta, FILE *log_file) {
    return solve(f, dx, dy, itmax, tol, CNV_POISSON_SOR, beta, log_file, 0);
}

void set_poisson_openmp_config(int enabled) { (void)enabled; /* the GPU always sweeps red-black */ }

void set_fluiddyn_openmp_config(int enabled) { (void)enabled; }

/* sum over all points of sqrt(pow(u2 - u1, 2)), rows in order (src/poisson.c:34-60) */
double error(mtrx u1, mtrx u2) {
    double e = 0;
    int i, j;
    for (i = 0; i < u1.m; i++)
        for (j = 0; j < u1.n; j++) e += sqrt(pow(u2.M[i][j] - u1.M[i][j], 2));
    return e;
}

void euler(mtrx w, mtrx dwdx, mtrx dwdy, mtrx d2wdx2, mtrx d2wdy2, mtrx u, mtrx v, double Re, double dt) {
    const int m = w.m, n = w.n;
    const size_t nn = (size_t)m * n;
    double *buf;
    int i, k, rc;
    mtrx src[7];
    if (w.M == NULL || m < 1 || n < 1) die("invalid parameter");
    buf = (double *)malloc(sizeof(double) * nn * 7);
    if (!buf) die("insufficient memory");
    src[0] = w;
    src[1] = dwdx;
    src[2] = dwdy;
    src[3] = d2wdx2;
    src[4] = d2wdy2;
    src[5] = u;
    src[6] = v;
    for (k = 0; k < 7; ++k)
        for (i = 0; i < m; ++i) memcpy(buf + k * nn + (size_t)i * n, src[k].M[i], sizeof(double) * n);
    rc = cnv_euler(buf, buf + nn, buf + 2 * nn, buf + 3 * nn, buf + 4 * nn, buf + 5 * nn, buf + 6 * nn,
                   (long long)nn, Re, dt);
    if (rc != CNV_OK) {
        free(buf);
        printf("** Error: %s **\n", cnv_last_error());
        exit(1);
    }
    for (i = 0; i < m; ++i) memcpy(w.M[i], buf + (size_t)i * n, sizeof(double) * n);
    free(buf);
}

mtrx continuity(mtrx dudx, mtrx dvdy) {
    mtrx t;
    int i, j;
    t.m = dudx.m;
    t.n = dudx.n;
    t.M = rows_alloc(t.m, t.n);
    for (i = 0; i < t.m; i++)
        for (j = 0; j < t.n; j++) t.M[i][j] = dudx.M[i][j] + dvdy.M[i][j];
    return t;
}

mtrx vorticity(mtrx dudy, mtrx dvdx) {
    mtrx t;
    int i, j;
    t.m = dudy.m;
    t.n = dudy.n;
    t.M = rows_alloc(t.m, t.n);
    for (i = 0; i < t.m; i++)
        for (j = 0; j < t.n; j++) t.M[i][j] = dvdx.M[i][j] - dudy.M[i][j];
    return t;
}
