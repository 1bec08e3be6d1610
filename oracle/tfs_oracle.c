/*
 * tfs_oracle.c -- CPU restatement of the T-FlowS linear-solver path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it as the checker.
 * The GPU library never links, loads or calls it.
 *
 * It restates, routine by routine, the sequential (n_proc = 0) build of
 *   Sources/Process/Solvers_Mod/Cg.f90          (tfo_cg)
 *   Sources/Process/Solvers_Mod/Bicg.f90        (tfo_bicg)
 *   Sources/Process/Solvers_Mod/Cgs.f90         (tfo_cgs)
 *   Sources/Process/Solvers_Mod/Prec_Form.f90   (tfo_prec_form)
 *   Sources/Process/Solvers_Mod/Prec_Solve.f90  (tfo_prec_solve)
 *   Sources/Process/Solvers_Mod/Residual.f90    (tfo_residual)
 *   Sources/Process/Matrix_Mod/Topology.f90     (tfo_topology_*)
 * with the reference's numeric conventions:
 *   - `real` is IEEE binary64 (Sources/first:112 passes -fdefault-real-8);
 *     `integer` is int32;
 *   - every array index is 1-based.  A C pointer `a` to a Fortran array a(1:n)
 *     is read through the macro A1(a,i) == a[i-1];
 *   - sums run sequentially i = 1..N, products and sums are rounded
 *     separately (build with -ffp-contract=off, no fast-math), as gfortran
 *     -O3 does on a target without FMA;
 *   - glosum/Exchange are the no-op sequential stubs
 *     (Sources/Process/Communication/Sequential/GloSum.f90, Exchange.f90), and
 *     the n_proc buffer loops never execute (Sequential/StaPar.f90:12-13).
 *
 * Deviations, each forced by undefined behaviour in the reference:
 *   - On the first early exit (||b|| < tol, Cg.f90:55-58) the reference
 *     returns an uninitialised local as fin_res.  The oracle returns ||b||,
 *     as the GPU library does; ini_res is left untouched, as in the reference.
 *   - Cgs.f90:142 adds r2*v2 into an uninitialised `alfa` that Cgs.f90:157
 *     overwrites before use; the statement has no effect and is not restated.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define A1(a, i) ((a)[(i) - 1])

/* Sources/Shared/allp_mod.f90:40 */
static const double TINY = 1.e-30;

/* ------------------------------------------------------------------------ */
/* Matrix_Mod_Topology (Sources/Process/Matrix_Mod/Topology.f90:2-127)       */
/* faces_c(1:2, 1:n_faces) is passed as a flat array f[2*(s-1)+0/1].          */
/* ------------------------------------------------------------------------ */

/* Number of stored entries (Topology.f90:33-47): 1 per cell plus 2 per
 * interior face.  The reference allocates one extra padding slot
 * (nonzeros = n + 1); callers size col/val/mir with that extra slot. */
int tfo_topology_count(int n_cells, int n_faces, const int *faces_c)
{
    int n = n_cells;
    for (int s = 1; s <= n_faces; s++) {
        int c2 = faces_c[2 * (s - 1) + 1];
        if (c2 > 0) n += 2;
    }
    return n;
}

/* Insertion sort of one row's column indices.  Topology.f90:76-78 calls the
 * CMLIB quicksort ISORT with kflag = 1 (ascending, nothing carried); the keys
 * of one row are distinct cell numbers, so every correct ascending sort gives
 * the same row. */
static void sort_ascending(int *x, int n)
{
    for (int a = 1; a < n; a++) {
        int v = x[a], b = a - 1;
        while (b >= 0 && x[b] > v) { x[b + 1] = x[b]; b--; }
        x[b + 1] = v;
    }
}

/* row(1:n+1), col(1:nnz+1), dia(1:n), mir(1:nnz+1), pos(1:2,1:n_faces). */
void tfo_topology_fill(int n_cells, int n_faces, const int *faces_c,
                       int *row, int *col, int *dia, int *mir, int *pos)
{
    int *stencw = (int *)malloc(sizeof(int) * (size_t)(n_cells + 1));
    for (int c = 1; c <= n_cells; c++) A1(stencw, c) = 1;

    /* Topology.f90:33-41 stencil widths */
    for (int s = 1; s <= n_faces; s++) {
        int c1 = faces_c[2 * (s - 1)], c2 = faces_c[2 * (s - 1) + 1];
        if (c2 > 0) { A1(stencw, c1)++; A1(stencw, c2)++; }
    }
    int n = 0;
    for (int c = 1; c <= n_cells; c++) n += A1(stencw, c);
    for (int j = 1; j <= n + 1; j++) { A1(col, j) = 0; A1(mir, j) = 0; }

    /* Topology.f90:54-59 row starts and the diagonal as first entry */
    A1(row, 1) = 1;
    for (int c = 1; c <= n_cells; c++) {
        A1(row, c + 1) = A1(row, c) + A1(stencw, c);
        A1(col, A1(row, c)) = c;
        A1(stencw, c) = 1;
    }
    /* Topology.f90:62-71 off-diagonal columns in face order */
    for (int s = 1; s <= n_faces; s++) {
        int c1 = faces_c[2 * (s - 1)], c2 = faces_c[2 * (s - 1) + 1];
        if (c2 > 0) {
            A1(col, A1(row, c1) + A1(stencw, c1)) = c2;
            A1(col, A1(row, c2) + A1(stencw, c2)) = c1;
            A1(stencw, c1)++;
            A1(stencw, c2)++;
        }
    }
    /* Topology.f90:75-82 sort each row, locate the diagonal */
    for (int c = 1; c <= n_cells; c++) {
        sort_ascending(&A1(col, A1(row, c)), A1(stencw, c));
        for (int p = A1(row, c); p <= A1(row, c + 1) - 1; p++)
            if (A1(col, p) == c) A1(dia, c) = p;
    }
    /* Topology.f90:85-103 mirror positions */
    for (int c1 = 1; c1 <= n_cells; c1++) {
        for (int p1 = A1(row, c1); p1 <= A1(row, c1 + 1) - 1; p1++) {
            int c2 = A1(col, p1);
            for (int p2 = A1(row, c2); p2 <= A1(row, c2 + 1) - 1; p2++) {
                if (A1(col, p2) == c1) {
                    A1(mir, p1) = p2;
                    A1(mir, p2) = p1;
                    break;
                }
            }
        }
    }
    /* Topology.f90:106-121 face -> entry positions */
    for (int s = 1; s <= n_faces; s++) {
        int c1 = faces_c[2 * (s - 1)], c2 = faces_c[2 * (s - 1) + 1];
        if (c2 > 0) {
            for (int c = A1(row, c1); c <= A1(row, c1 + 1) - 1; c++)
                if (A1(col, c) == c2) pos[2 * (s - 1)] = c;
            for (int c = A1(row, c2); c <= A1(row, c2 + 1) - 1; c++)
                if (A1(col, c) == c1) pos[2 * (s - 1) + 1] = c;
        }
    }
    free(stencw);
}

/* ------------------------------------------------------------------------ */
/* Prec_Form (Sources/Process/Solvers_Mod/Prec_Form.f90:2-51).               */
/* d(1:n) holds D % val(D % dia(i)).                                         */
/* ------------------------------------------------------------------------ */
void tfo_prec_form(int n, const int *row, const int *col, const int *dia,
                   const double *val, int prec, double *d)
{
    if (prec == 1) {                               /* Prec_Form.f90:24-27 */
        for (int i = 1; i <= n; i++) A1(d, i) = A1(val, A1(dia, i));
    } else if (prec == 2) {                        /* Prec_Form.f90:32-40 */
        for (int i = 1; i <= n; i++) {
            double sum1 = A1(val, A1(dia, i));
            for (int j = A1(row, i); j <= A1(dia, i) - 1; j++) {
                int k = A1(col, j);
                sum1 = sum1 - A1(d, k) * A1(val, j) * A1(val, j);
            }
            A1(d, i) = 1.0 / sum1;
        }
    } else {                                       /* Prec_Form.f90:45-49 */
        for (int i = 1; i <= n; i++) A1(d, i) = 1.0;
    }
}

/* ------------------------------------------------------------------------ */
/* Prec_Solve (Sources/Process/Solvers_Mod/Prec_Solve.f90:2-78): x = M^-1 b. */
/* ------------------------------------------------------------------------ */
void tfo_prec_solve(int n, const int *row, const int *col, const int *dia,
                    const double *val, const double *d, double *x,
                    const double *b, int prec)
{
    if (prec == 1) {                               /* Prec_Solve.f90:35-38 */
        for (int i = 1; i <= n; i++) A1(x, i) = A1(b, i) / A1(d, i);
    } else if (prec == 2) {
        for (int i = 1; i <= n; i++) {             /* Prec_Solve.f90:46-53 */
            double sum1 = A1(b, i);
            for (int j = A1(row, i); j <= A1(dia, i) - 1; j++) {
                int k = A1(col, j);
                sum1 = sum1 - A1(val, j) * A1(x, k);
            }
            A1(x, i) = sum1 * A1(d, i);
        }
        for (int i = 1; i <= n; i++)               /* Prec_Solve.f90:55-57 */
            A1(x, i) = A1(x, i) / (A1(d, i) + TINY);
        for (int i = n; i >= 1; i--) {             /* Prec_Solve.f90:60-67 */
            double sum1 = A1(x, i);
            for (int j = A1(dia, i) + 1; j <= A1(row, i + 1) - 1; j++) {
                int k = A1(col, j);
                sum1 = sum1 - A1(val, j) * A1(x, k);
            }
            A1(x, i) = sum1 * A1(d, i);
        }
    } else {                                       /* Prec_Solve.f90:71-74 */
        for (int i = 1; i <= n; i++) A1(x, i) = A1(b, i);
    }
}

/* Residual (Sources/Process/Solvers_Mod/Residual.f90:22-27): r1 <- r1 - A x,
 * subtracting the products of row i one at a time, in column order. */
void tfo_residual(int n, const int *row, const int *col, const double *val,
                  const double *x, double *r1)
{
    for (int i = 1; i <= n; i++)
        for (int j = A1(row, i); j <= A1(row, i + 1) - 1; j++) {
            int k = A1(col, j);
            A1(r1, i) = A1(r1, i) - A1(val, j) * A1(x, k);
        }
}

/* q = A p, the product loop of Cg.f90:128-134 (q starts at 0.0). */
void tfo_spmv(int n, const int *row, const int *col, const double *val,
              const double *p, double *q)
{
    for (int i = 1; i <= n; i++) {
        A1(q, i) = 0.0;
        for (int j = A1(row, i); j <= A1(row, i + 1) - 1; j++) {
            int k = A1(col, j);
            A1(q, i) = A1(q, i) + A1(val, j) * A1(p, k);
        }
    }
}

static double dot_seq(int n, const double *a, const double *b)
{
    double s = 0.0;
    for (int i = 1; i <= n; i++) s = s + A1(a, i) * A1(b, i);
    return s;
}

static double *vec(int n) { return (double *)calloc((size_t)n + 1, sizeof(double)); }

/* ------------------------------------------------------------------------ */
/* Cg (Sources/Process/Solvers_Mod/Cg.f90:2-183)                             */
/* ------------------------------------------------------------------------ */
void tfo_cg(int n, const int *row, const int *col, const int *dia,
            const double *val, double *x, double *r1, int prec, int *niter,
            double tol, double *ini_res, double *fin_res)
{
    double *d = vec(n), *p1 = vec(n), *q1 = vec(n);
    double alfa, beta, rho, rhoold = 0.0, bnrm2, error;
    int iter;

    tfo_prec_form(n, row, col, dia, val, prec, d);          /* Cg.f90:42 */

    bnrm2 = sqrt(dot_seq(n, r1, r1));                       /* Cg.f90:48-53 */
    if (bnrm2 < tol) { iter = 0; error = bnrm2; goto done; } /* :55-58 */

    tfo_residual(n, row, col, val, x, r1);                  /* Cg.f90:63 */
    for (int i = 1; i <= n; i++) A1(p1, i) = A1(r1, i);     /* Cg.f90:68-70 */

    error = sqrt(dot_seq(n, r1, r1));                       /* Cg.f90:75-80 */
    *ini_res = error;                                       /* Cg.f90:85 */
    if (error < tol) { iter = 0; goto done; }               /* Cg.f90:87-90 */

    for (iter = 1; iter <= *niter; iter++) {                /* Cg.f90:97 */
        tfo_prec_solve(n, row, col, dia, val, d, q1, r1, prec); /* :103 */
        rho = dot_seq(n, r1, q1);                           /* Cg.f90:108-112 */
        if (iter == 1) {                                    /* Cg.f90:114-123 */
            for (int i = 1; i <= n; i++) A1(p1, i) = A1(q1, i);
        } else {
            beta = rho / rhoold;
            for (int i = 1; i <= n; i++) A1(p1, i) = A1(q1, i) + beta * A1(p1, i);
        }
        tfo_spmv(n, row, col, val, p1, q1);                 /* Cg.f90:128-134 */
        alfa = dot_seq(n, p1, q1);                          /* Cg.f90:148-153 */
        alfa = rho / alfa;
        for (int i = 1; i <= n; i++) {                      /* Cg.f90:159-162 */
            A1(x, i) = A1(x, i) + alfa * A1(p1, i);
            A1(r1, i) = A1(r1, i) - alfa * A1(q1, i);
        }
        error = sqrt(dot_seq(n, r1, r1));                   /* Cg.f90:167-172 */
        if (error < tol) goto done;                         /* Cg.f90:174 */
        rhoold = rho;                                       /* Cg.f90:176 */
    }
    /* falling out of `do iter=1,niter` leaves iter = max(niter,0)+1 (F4) */
    if (*niter < 0) iter = 1;
done:
    *fin_res = error;                                       /* Cg.f90:180 */
    *niter = iter;                                          /* Cg.f90:181 */
    free(d); free(p1); free(q1);
}

/* ------------------------------------------------------------------------ */
/* Bicg (Sources/Process/Solvers_Mod/Bicg.f90:2-196).  The shadow system is  */
/* driven with A itself, not A^T (Bicg.f90:136-144).                          */
/* ------------------------------------------------------------------------ */
void tfo_bicg(int n, const int *row, const int *col, const int *dia,
              const double *val, double *x, double *r1, int prec, int *niter,
              double tol, double *ini_res, double *fin_res)
{
    double *d = vec(n), *p1 = vec(n), *p2 = vec(n), *q1 = vec(n), *q2 = vec(n),
           *r2 = vec(n);
    double alfa, beta, rho, rhoold = 0.0, bnrm2, error;
    int iter;

    tfo_prec_form(n, row, col, dia, val, prec, d);          /* Bicg.f90:45 */
    bnrm2 = sqrt(dot_seq(n, r1, r1));                       /* Bicg.f90:51-56 */
    if (bnrm2 < tol) { iter = 0; error = bnrm2; goto done; }

    tfo_residual(n, row, col, val, x, r1);                  /* Bicg.f90:66 */
    error = sqrt(dot_seq(n, r1, r1));                       /* Bicg.f90:71-76 */
    *ini_res = error;
    if (error < tol) { iter = 0; goto done; }

    for (int i = 1; i <= n; i++) A1(r2, i) = A1(r1, i);     /* Bicg.f90:91-93 */

    for (iter = 1; iter <= *niter; iter++) {                /* Bicg.f90:100 */
        tfo_prec_solve(n, row, col, dia, val, d, q1, r1, prec); /* :107 */
        tfo_prec_solve(n, row, col, dia, val, d, q2, r2, prec); /* :108 */
        rho = dot_seq(n, q1, r2);                           /* Bicg.f90:113-117 */
        if (iter == 1) {
            for (int i = 1; i <= n; i++) { A1(p1, i) = A1(q1, i); A1(p2, i) = A1(q2, i); }
        } else {
            beta = rho / rhoold;                            /* Bicg.f90:125-129 */
            for (int i = 1; i <= n; i++) {
                A1(p1, i) = A1(q1, i) + beta * A1(p1, i);
                A1(p2, i) = A1(q2, i) + beta * A1(p2, i);
            }
        }
        for (int i = 1; i <= n; i++) {                      /* Bicg.f90:136-144 */
            A1(q1, i) = 0.0;
            A1(q2, i) = 0.0;
            for (int j = A1(row, i); j <= A1(row, i + 1) - 1; j++) {
                int k = A1(col, j);
                A1(q1, i) = A1(q1, i) + A1(val, j) * A1(p1, k);
                A1(q2, i) = A1(q2, i) + A1(val, j) * A1(p2, k);
            }
        }
        alfa = dot_seq(n, p2, q1);                          /* Bicg.f90:160-165 */
        alfa = rho / alfa;
        for (int i = 1; i <= n; i++) {                      /* Bicg.f90:171-175 */
            A1(x, i) = A1(x, i) + alfa * A1(p1, i);
            A1(r1, i) = A1(r1, i) - alfa * A1(q1, i);
            A1(r2, i) = A1(r2, i) - alfa * A1(q2, i);
        }
        error = sqrt(dot_seq(n, r1, r1));                   /* Bicg.f90:180-185 */
        if (error < tol) goto done;                         /* Bicg.f90:187 */
        rhoold = rho;
    }
    if (*niter < 0) iter = 1;
done:
    *fin_res = error;
    *niter = iter;
    free(d); free(p1); free(p2); free(q1); free(q2); free(r2);
}

/* ------------------------------------------------------------------------ */
/* Cgs (Sources/Process/Solvers_Mod/Cgs.f90:2-232)                           */
/* ------------------------------------------------------------------------ */
void tfo_cgs(int n, const int *row, const int *col, const int *dia,
             const double *val, double *x, double *r1, int prec, int *niter,
             double tol, double *ini_res, double *fin_res)
{
    double *d = vec(n), *p1 = vec(n), *p2 = vec(n), *q1 = vec(n), *q2 = vec(n),
           *r2 = vec(n), *u1 = vec(n), *u2 = vec(n), *v2 = vec(n), *w = vec(n);
    double alfa, beta, rho, rhoold = 0.0, bnrm2, error;
    int iter;

    tfo_prec_form(n, row, col, dia, val, prec, d);          /* Cgs.f90:45 */
    bnrm2 = sqrt(dot_seq(n, r1, r1));                       /* Cgs.f90:51-56 */
    if (bnrm2 < tol) { iter = 0; error = bnrm2; goto done; }

    tfo_residual(n, row, col, val, x, r1);                  /* Cgs.f90:66 */
    for (int i = 1; i <= n; i++) A1(r2, i) = A1(r1, i);     /* Cgs.f90:71-73 */
    error = sqrt(dot_seq(n, r1, r1));                       /* Cgs.f90:78-83 */
    *ini_res = error;
    if (error < tol) { iter = 0; goto done; }

    for (iter = 1; iter <= *niter; iter++) {                /* Cgs.f90:100 */
        rho = dot_seq(n, r1, r2);                           /* Cgs.f90:105-109 */
        if (iter == 1) {
            for (int i = 1; i <= n; i++) { A1(u1, i) = A1(r1, i); A1(u2, i) = A1(u1, i); }
        } else {
            beta = rho / rhoold;                            /* Cgs.f90:117-121 */
            for (int i = 1; i <= n; i++) {
                A1(u1, i) = A1(r1, i) + beta * A1(q1, i);
                A1(u2, i) = A1(u1, i) + beta * (A1(q1, i) + beta * A1(u2, i));
            }
        }
        tfo_prec_solve(n, row, col, dia, val, d, p2, u2, prec); /* :127 */
        tfo_spmv(n, row, col, val, p2, v2);                 /* Cgs.f90:132-139 */
        alfa = dot_seq(n, r2, v2);                          /* Cgs.f90:153-158 */
        alfa = rho / alfa;
        for (int i = 1; i <= n; i++)                        /* Cgs.f90:163-165 */
            A1(q1, i) = A1(u1, i) - alfa * A1(v2, i);
        for (int i = 1; i <= n; i++)                        /* Cgs.f90:170-172 */
            A1(w, i) = A1(u1, i) + A1(q1, i);
        tfo_prec_solve(n, row, col, dia, val, d, p1, w, prec); /* :173 */
        for (int i = 1; i <= n; i++)                        /* Cgs.f90:178-180 */
            A1(x, i) = A1(x, i) + alfa * A1(p1, i);
        tfo_spmv(n, row, col, val, p1, q2);                 /* Cgs.f90:185-191 */
        for (int i = 1; i <= n; i++)                        /* Cgs.f90:205-207 */
            A1(r1, i) = A1(r1, i) - alfa * A1(q2, i);
        error = sqrt(dot_seq(n, r1, r1));                   /* Cgs.f90:212-217 */
        if (error < tol) goto done;                         /* Cgs.f90:219 */
        rhoold = rho;
    }
    if (*niter < 0) iter = 1;
done:
    *fin_res = error;
    *niter = iter;
    free(d); free(p1); free(p2); free(q1); free(q2); free(r2);
    free(u1); free(u2); free(v2); free(w);
}

/* Dispatch by method number (0 = Cg, 1 = Bicg, 2 = Cgs), as the GPU ABI does. */
void tfo_solve(int method, int n, const int *row, const int *col, const int *dia,
               const double *val, double *x, double *r1, int prec, int *niter,
               double tol, double *ini_res, double *fin_res)
{
    if (method == 1)
        tfo_bicg(n, row, col, dia, val, x, r1, prec, niter, tol, ini_res, fin_res);
    else if (method == 2)
        tfo_cgs(n, row, col, dia, val, x, r1, prec, niter, tol, ini_res, fin_res);
    else
        tfo_cg(n, row, col, dia, val, x, r1, prec, niter, tol, ini_res, fin_res);
}

/* Matrix values from per-face coefficients through the face -> entry map,
 * as the face loops of the reference assemble them: NewUVW.f90:366-384 (the
 * interior face updates the two off-diagonal entries through pos(1,s) and
 * pos(2,s) and the two diagonals through dia; a boundary face of a
 * contributing type adds to the diagonal of c1) followed by the cell loop
 * NewUVW.f90:500-505 (the inertial term on every diagonal).  Compute_Pressure_
 * Simple.f90:100-113 is the same loop with off12 = off21 = dia12 = dia21 =
 * A12 (its "= -A12" equals "0 - A12" on a zeroed matrix).  A boundary face
 * whose dia12 is exactly zero stands for a type that adds nothing.
 * faces_c(1:2, 1:n_faces), pos(1:2, 1:n_faces), dia(1:n_cells), val(1:nnz);
 * cell may be NULL. */
void tfo_assemble_faces(int n_cells, int n_faces, const int *faces_c, const int *pos,
                        const int *dia, const double *off12, const double *off21,
                        const double *dia12, const double *dia21, const double *cell,
                        double *val)
{
    for (int s = 1; s <= n_faces; s++) {
        const int c1 = faces_c[2 * (s - 1)], c2 = faces_c[2 * (s - 1) + 1];
        if (c2 > 0) {
            A1(val, pos[2 * (s - 1)]) = A1(val, pos[2 * (s - 1)]) - A1(off12, s);
            A1(val, A1(dia, c1)) = A1(val, A1(dia, c1)) + A1(dia12, s);
            A1(val, pos[2 * (s - 1) + 1]) = A1(val, pos[2 * (s - 1) + 1]) - A1(off21, s);
            A1(val, A1(dia, c2)) = A1(val, A1(dia, c2)) + A1(dia21, s);
        } else if (A1(dia12, s) != 0.0) {
            A1(val, A1(dia, c1)) = A1(val, A1(dia, c1)) + A1(dia12, s);
        }
    }
    if (cell)
        for (int c = 1; c <= n_cells; c++) A1(val, A1(dia, c)) = A1(val, A1(dia, c)) + A1(cell, c);
}
