/*
 * cnv_compat.h -- the reference's own solver entry points, served by libcnv (libcnv_compat.so).
 *
 * A build of the reference program that links libcnv_compat.so in place of its
 * src/poisson.c and src/fluiddyn.c calls these functions exactly as before: the same names,
 * argument lists, ownership and messages, with the work done on the GPU. Each replaces:
 *
 *   poisson, poisson_log            include/poisson.h:11, :14   (src/poisson.c:62-109, :176-222)
 *   poisson_SOR, poisson_SOR_log    include/poisson.h:12, :15   (src/poisson.c:111-173, :224-285)
 *   error                           include/poisson.h:10        (src/poisson.c:34-60)
 *   set_poisson_openmp_config       include/poisson.h:17        (src/poisson.c:15-21)
 *   euler                           include/fluiddyn.h:5        (src/fluiddyn.c:71-102)
 *   continuity, vorticity           include/fluiddyn.h:6-7      (src/fluiddyn.c:126-201)
 *   set_fluiddyn_openmp_config      include/fluiddyn.h:10       (src/fluiddyn.c:35-41)
 *
 * Semantics kept: poisson* allocate and return a new psi (rows malloc'ed one by one, as
 * allocm does, so the caller's freem() releases it), start from psi = 0, stop when
 * sum|psi - psi0| < tol, print (or log) "Poisson equation solved with %d iterations - ..." and
 * on non-convergence print the reference's error line and exit(1). euler updates w in place.
 * Differences: the GPU sweeps red-black whatever the OpenMP setting (the reference's OpenMP
 * ordering); f must be square (n x n) with dx*n and dy*n whole numbers, which every call from
 * the reference's main satisfies (dx = (double)Lx / nx with integer Lx); error(), continuity()
 * and vorticity() are elementwise host loops (they are not on the time-step path: the GPU step
 * computes its own stop norm and continuity diagnostic).
 */
#ifndef CNV_COMPAT_H
#define CNV_COMPAT_H

#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef LINEARALG_H_INCLUDED
/* include/linearalg.h:6-11: same members in the same order */
typedef struct matrix {
    double **M; /* row pointers */
    int m;      /* rows */
    int n;      /* columns */
} mtrx;
#endif

double error(mtrx u1, mtrx u2);
mtrx poisson(mtrx f, double dx, double dy, int itmax, double tol);
mtrx poisson_SOR(mtrx f, double dx, double dy, int itmax, double tol, double beta);
mtrx poisson_log(mtrx f, double dx, double dy, int itmax, double tol, FILE *log_file);
mtrx poisson_SOR_log(mtrx f, double dx, double dy, int itmax, double tol, double beta, FILE *log_file);
void set_poisson_openmp_config(int enabled);

void euler(mtrx w, mtrx dwdx, mtrx dwdy, mtrx d2wdx2, mtrx d2wdy2, mtrx u, mtrx v, double Re, double dt);
mtrx continuity(mtrx dudx, mtrx dvdy);
mtrx vorticity(mtrx dudy, mtrx dvdx);
void set_fluiddyn_openmp_config(int enabled);

#ifdef __cplusplus
}
#endif
#endif /* CNV_COMPAT_H */
