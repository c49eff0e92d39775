/*
 * ref_harness.c -- drives the UNMODIFIED reference code of SorinBetisor/fluid-dynamics1
 * (src/finitediff.c, src/linearalg.c, src/fluiddyn.c, src/poisson.c, compiled from the
 * reference tree by oracle/Makefile into oracle/_ref/libcnv_ref.so) through the step body
 * of src/main.c:283-395, with its dense Kronecker operators, so that the banded
 * restatement in cnv_oracle.c can be checked against it bit for bit.
 *
 * TEST INFRASTRUCTURE ONLY. It is built only where the reference tree exists and is used
 * only by tests that skip themselves when oracle/_ref is absent.
 *
 * The reference's Poisson solvers report the iteration count and stop norm only through
 * their log line (src/poisson.c:275), so the harness passes a temporary log file and parses
 * that line back ("%d" and "%E": the count exactly, the norm to 7 significant digits).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include "linearalg.h"
#include "finitediff.h"
#include "fluiddyn.h"
#include "poisson.h"

static mtrx from_flat(const double *x, int n)
{
    mtrx A = initm(n, n);
    int i, j;
    for (i = 0; i < n; ++i)
        for (j = 0; j < n; ++j) A.M[i][j] = x[(size_t)i * n + j];
    return A;
}

static void to_flat(mtrx A, double *x)
{
    int i, j;
    for (i = 0; i < A.m; ++i)
        for (j = 0; j < A.n; ++j) x[(size_t)i * A.n + j] = A.M[i][j];
}

/* apply a dense 2-D operator to a field the way src/main.c:298-304 does */
static mtrx apply2d(mtrx D, mtrx x, int n)
{
    mtrx x0 = reshape(x, n * n, 1);
    mtrx y0 = mtrxmul(D, x0);
    mtrx y = reshape(y0, n, n);
    x0.M = freem(x0);
    y0.M = freem(y0);
    return y;
}

/* Dense 1-D operator as the reference builds it (for the band self-test). */
int ref_fd_dense(int n, int order, int deriv, double h, double *out)
{
    mtrx D = deriv == 1 ? Diff1(n, order, h) : Diff2(n, order, h);
    to_flat(D, out);
    D.M = freem(D);
    return 0;
}

/* Run nsteps of the step body. bc = {u1,u2,u3,u4,v1,v2,v3,v4}. poisson_type 1 or 2.
 * openmp != 0 selects the red-black ordering of the OPENMP_ENABLED build.
 * Outputs per step: iters[t], err[t] (parsed log value), cmax[t], cmin[t]. */
int ref_run(int n, int order, int Lx, int Ly, double Re, double dt, const double *bc,
            int poisson_type, double beta, int itmax, double tol, int openmp, int nsteps,
            double *w_io, double *u_io, double *v_io, double *psi_out,
            int *iters, double *err, double *cmax, double *cmin)
{
    int i, j, t;
    double dx = (double)Lx / n, dy = (double)Ly / n;
    double u1 = bc[0], u2 = bc[1], u3 = bc[2], u4 = bc[3];
    double v1 = bc[4], v2 = bc[5], v3 = bc[6], v4 = bc[7];
    mtrx d_x, d_y, d_x2, d_y2, Ix, Iy, DX, DY, DX2, DY2;
    mtrx u, v, w, psi;

    set_openmp_config(openmp);
    set_poisson_openmp_config(openmp);
    set_fluiddyn_openmp_config(openmp);

    d_x = Diff1(n, order, dx);
    d_y = Diff1(n, order, dy);
    d_x2 = Diff2(n, order, dx);
    d_y2 = Diff2(n, order, dy);
    Ix = eye(n);
    Iy = eye(n);
    DX = kronecker(Ix, d_x);
    DY = kronecker(d_y, Iy);
    DX2 = kronecker(Ix, d_x2);
    DY2 = kronecker(d_y2, Iy);
    d_x.M = freem(d_x); d_y.M = freem(d_y); d_x2.M = freem(d_x2); d_y2.M = freem(d_y2);
    Ix.M = freem(Ix); Iy.M = freem(Iy);

    u = from_flat(u_io, n);
    v = from_flat(v_io, n);
    w = from_flat(w_io, n);
    psi = initm(n, n);

    for (t = 0; t < nsteps; ++t) {
        mtrx dudy, dvdx, dwdx, dwdy, d2wdx2, d2wdy2, dpsidx, dpsidy, dudx, dvdy, cc;
        FILE *lf = tmpfile();
        char line[512];
        int k = -1;
        double e = 0;

        for (j = 0; j < n; ++j) {
            v.M[0][j] = v3; v.M[n - 1][j] = v4; u.M[0][j] = u3; u.M[n - 1][j] = u4;
        }
        for (i = 0; i < n; ++i) {
            v.M[i][0] = v1; v.M[i][n - 1] = v2; u.M[i][0] = u1; u.M[i][n - 1] = u2;
        }
        dudy = apply2d(DY, u, n);
        dvdx = apply2d(DX, v, n);
        for (j = 0; j < n; ++j) {
            w.M[0][j] = dvdx.M[0][j] - dudy.M[0][j];
            w.M[n - 1][j] = dvdx.M[n - 1][j] - dudy.M[n - 1][j];
        }
        for (i = 0; i < n; ++i) {
            w.M[i][0] = dvdx.M[i][0] - dudy.M[i][0];
            w.M[i][n - 1] = dvdx.M[i][n - 1] - dudy.M[i][n - 1];
        }
        dwdx = apply2d(DX, w, n);
        dwdy = apply2d(DY, w, n);
        d2wdx2 = apply2d(DX2, w, n);
        d2wdy2 = apply2d(DY2, w, n);
        euler(w, dwdx, dwdy, d2wdx2, d2wdy2, u, v, Re, dt);

        psi.M = freem(psi);
        invsig(w);
        if (poisson_type == 1) psi = poisson_log(w, dx, dy, itmax, tol, lf);
        else psi = poisson_SOR_log(w, dx, dy, itmax, tol, beta, lf);
        invsig(w);
        rewind(lf);
        while (fgets(line, sizeof line, lf))
            if (sscanf(line, "Poisson equation solved with %d iterations - root-sum-of-squares error: %lE", &k, &e) == 2) break;
        fclose(lf);

        dpsidx = apply2d(DX, psi, n);
        dpsidy = apply2d(DY, psi, n);
        u.M = freem(u);
        v.M = freem(v);
        u = initm(n, n);
        v = initm(n, n);
        mtrxcpy(u, dpsidy);
        invsig(dpsidx);
        mtrxcpy(v, dpsidx);

        dudx = apply2d(DX, u, n);
        dvdy = apply2d(DY, v, n);
        cc = continuity(dudx, dvdy);
        iters[t] = k;
        err[t] = e;
        cmax[t] = maxel(cc);
        cmin[t] = minel(cc);

        dudy.M = freem(dudy); dvdx.M = freem(dvdx);
        dwdx.M = freem(dwdx); dwdy.M = freem(dwdy);
        d2wdx2.M = freem(d2wdx2); d2wdy2.M = freem(d2wdy2);
        dpsidx.M = freem(dpsidx); dpsidy.M = freem(dpsidy);
        dudx.M = freem(dudx); dvdy.M = freem(dvdy); cc.M = freem(cc);
    }
    to_flat(w, w_io);
    to_flat(u, u_io);
    to_flat(v, v_io);
    to_flat(psi, psi_out);
    u.M = freem(u); v.M = freem(v); w.M = freem(w); psi.M = freem(psi);
    DX.M = freem(DX); DY.M = freem(DY); DX2.M = freem(DX2); DY2.M = freem(DY2);
    return 0;
}
