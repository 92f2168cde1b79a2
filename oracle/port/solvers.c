/*
 * solvers.c -- dense solvers of the reference
 * (oracle restatement of src/gaussBksb.c and src/gmres_el.c; test
 * infrastructure).
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

/* In-place elimination without pivoting; rows are swapped only while the
 * pivot is within 1e-9 of zero, and the first later row whose entry in the
 * pivot column is also that small ends the solve (src/gaussBksb.c:39-108). */
int orc_gauss(unsigned n, double *A, double *B)
{
    const double TOL = 1.0E-9;
    unsigned n1 = n - 1;
#define AA(r, c) A[(size_t)(r) * n + (c)]
    for (unsigned i = 0; i < n1; i++) {
        unsigned i1 = i + 1;
        if (fabs(AA(i, i)) - TOL <= 0) {
            for (unsigned j = i1; j < n; j++) {
                if (fabs(AA(j, i)) - TOL > 0) {
                    for (unsigned k = i; k < n; k++) {
                        double c = AA(i, k);
                        AA(i, k) = AA(j, k);
                        AA(j, k) = c;
                    }
                    double c = B[i];
                    B[i] = B[j];
                    B[j] = c;
                } else {
                    return 1;
                }
            }
        }
        double C = AA(i, i);
        for (unsigned j = i1; j < n; j++) AA(i, j) = AA(i, j) / C;
        B[i] = B[i] / C;
        for (unsigned j = i1; j < n; j++) {
            double c = AA(j, i);
            double *rj = &AA(j, 0), *ri = &AA(i, 0);
            for (unsigned k = i1; k < n; k++) rj[k] = rj[k] - c * ri[k];
            B[j] = B[j] - c * B[i];
        }
    }
    if (!(fabs(AA(n1, n1)) > TOL)) return 1;
    B[n1] = B[n1] / AA(n1, n1);
    for (unsigned i = 0; i < n1; i++) {
        unsigned k = n1 - i - 1;
        for (unsigned j = k + 1; j < n; j++) B[k] = B[k] - AA(k, j) * B[j];
    }
#undef AA
    return 0;
}

struct mv_job {
    unsigned N, r0, r1;
    const double *A, *x;
    double *y;
    unsigned aoff;  /* first row held in A */
};

/* y = (A1 - i A2) x on the compact N x 2N form, rows [r0, r1)
 * (matVectProd_el src/gmres_el.c:323-337). */
static void matvec_rows(const struct mv_job *j)
{
    const unsigned N = j->N;
    for (unsigned i = j->r0; i < j->r1; i++) {
        const double *a = j->A + (size_t)(i - j->aoff) * 2 * N;
        double yr = 0.0, yi = 0.0;
        for (unsigned c = 0; c < N; c++) {
            yr += a[c] * j->x[c] + a[c + N] * j->x[c + N];
            yi += a[c] * j->x[c + N] - a[c + N] * j->x[c];
        }
        j->y[i] = yr;
        j->y[i + N] = yi;
    }
}

static void *mv_thread(void *p)
{
    matvec_rows((const struct mv_job *)p);
    return NULL;
}

static void matvec(unsigned N, const double *A, const double *x, double *y, int nthreads)
{
    if (nthreads <= 1) {
        struct mv_job j = {N, 0, N, A, x, y};
        matvec_rows(&j);
        return;
    }
    struct mv_job jobs[256];
    pthread_t th[256];
    if (nthreads > 256) nthreads = 256;
    unsigned per = (N + (unsigned)nthreads - 1) / (unsigned)nthreads;
    for (int t = 0; t < nthreads; t++) {
        unsigned r0 = (unsigned)t * per, r1 = r0 + per < N ? r0 + per : N;
        if (r0 > N) r0 = N;
        jobs[t] = (struct mv_job){N, r0, r1, A, x, y};
        pthread_create(&th[t], NULL, mv_thread, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

/* Rows [r0, r1) of the compact-form product (used to time a sample of the
 * GMRES matrix-vector product). */
void orc_matvec_rows(unsigned N, const double *A, const double *x, double *y, unsigned r0,
                     unsigned r1, int nthreads)
{
    if (nthreads <= 1) {
        struct mv_job j = {N, r0, r1, A, x, y, r0};
        matvec_rows(&j);
        return;
    }
    struct mv_job jobs[256];
    pthread_t th[256];
    if (nthreads > 256) nthreads = 256;
    unsigned n = r1 - r0, per = (n + (unsigned)nthreads - 1) / (unsigned)nthreads;
    for (int t = 0; t < nthreads; t++) {
        unsigned a = r0 + (unsigned)t * per, b = a + per < r1 ? a + per : r1;
        if (a > r1) a = r1;
        jobs[t] = (struct mv_job){N, a, b, A, x, y, r0};
        pthread_create(&th[t], NULL, mv_thread, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

static double dot(unsigned n, const double *x, const double *y)
{
    double s = 0.0;
    for (unsigned i = 0; i < n; i++) s += x[i] * y[i];
    return s;
}

static double nrm2(unsigned n, const double *x)
{
    return sqrt(dot(n, x, x));
}

/* Un-restarted GMRES (solverGMRES_el src/gmres_el.c:66-128 and
 * iterGMRES_el :149-260):
 *   - optional Jacobi scaling of row i of A and of B[i] (the imaginary
 *     right-hand side B[i + N] is not scaled, as in the reference, :87-93);
 *   - absolute tolerance |B| * tol_rel;
 *   - Arnoldi with modified Gram-Schmidt, Givens rotations as written in
 *     the reference (:202-220), stagnation test |e1 - e0| / e0 < 1e-6 tol;
 *   - upper-triangular solve and x += sum y_j v_j. */
int orc_gmres(unsigned N, unsigned preCond, double tol_rel, unsigned max_iters,
              double *A, double *B, const double *x0, FILE *log, int nthreads,
              unsigned *iters)
{
    const unsigned size = 2 * N;
    const unsigned M = max_iters;
    double *x = (double *)calloc(size, sizeof(double));
    if (x0) memcpy(x, x0, size * sizeof(double));
    if (preCond == 1) {
        for (unsigned i = 0; i < N; i++) {
            double *a = A + (size_t)i * size;
            double diag = 1.0 / a[i];
            B[i] = B[i] * diag;
            for (unsigned j = 0; j < size; j++) a[j] = diag * a[j];
        }
    }
    double tolerance = nrm2(size, B) * tol_rel;
    if (log) {
        fprintf(log, "\n\nRELATIVE TOLERANCE = %10.4e\n", tolerance);
        fprintf(log, "\n%10s%21s\n", "ITER #    ", "RELATIVE RESIDUAL");
        fprintf(log, "%10s%21s\n", "***************", "*******************");
    }
    double *s = (double *)calloc(M + 1, sizeof(double));
    double *c = (double *)calloc(M + 1, sizeof(double));
    double *res = (double *)calloc(M + 2, sizeof(double));
    double *h = (double *)calloc((size_t)(M + 2) * (M + 2), sizeof(double));
    double *V = (double *)malloc((size_t)(M + 1) * size * sizeof(double));
#define H(r, q) h[(size_t)(r) * (M + 2) + (q)]
    /* Initial residual (initRes_el :272-294). */
    double *v0 = V;
    if (nrm2(size, x) != 0.0) {
        double *y = (double *)malloc(size * sizeof(double));
        matvec(N, A, x, y, nthreads);
        for (unsigned i = 0; i < size; i++) v0[i] = B[i] - y[i];
        free(y);
    } else {
        memcpy(v0, B, size * sizeof(double));
    }
    double norm = nrm2(size, v0);
    for (unsigned i = 0; i < size; i++) v0[i] /= norm;
    res[0] = norm;
    double err0 = norm, err1 = norm;
    int status = 1;
    unsigned it = 0;
    if (err0 < tolerance) {
        status = 0;
    } else {
        for (unsigned i = 0; i < M; i++) {
            it++;
            double *vi = V + (size_t)i * size, *w = V + (size_t)(i + 1) * size;
            matvec(N, A, vi, w, nthreads);
            norm = nrm2(size, w);
            for (unsigned j = 0; j <= i; j++) {
                const double *vj = V + (size_t)j * size;
                double hj = dot(size, vj, w);
                H(j, i) = hj;
                for (unsigned k = 0; k < size; k++) w[k] = w[k] - hj * vj[k];
            }
            H(i + 1, i) = nrm2(size, w);
            if (H(i + 1, i) != 0.0)
                for (unsigned k = 0; k < size; k++) w[k] = w[k] / H(i + 1, i);
            for (unsigned j = 0; j + 1 <= i; j++) {
                double h1 = c[j] * H(j, i) + s[j] * H(j + 1, i);
                double h2 = -s[j] * H(j, i) + c[j] * H(j + 1, i);
                H(j, i) = h1;
                H(j + 1, i) = h2;
            }
            double htmp = H(i + 1, i) / H(i, i);
            if (norm != 0.0) {
                c[i] = 1.0 / sqrt(1.0 + htmp * htmp);
                s[i] = c[i] * htmp;
                H(i, i) = c[i] * H(i, i) + s[i] * H(i + 1, i);
                H(i + 1, i) = 0.0;
                res[i + 1] = -s[i] * res[i];
                res[i] = c[i] * res[i];
            }
            err1 = fabs(res[i + 1]);
            if (log) fprintf(log, "%8d%25.4e\n", (int)it, err1);
            if (err1 < tolerance) { status = 0; break; }
            if (fabs((err1 - err0) / err0) < 1.0e-6 * tolerance) { status = 2; break; }
            err0 = err1;
        }
        if (status != 2) {
            /* Back substitution; the column `it` of H is zero. */
            for (int i = (int)it - 1; i >= 0; i--) {
                for (unsigned j = (unsigned)i + 1; j <= it; j++) res[i] -= H(i, j) * res[j];
                res[i] = res[i] / H(i, i);
            }
            for (unsigned k = 0; k < size; k++) {
                double acc = x[k];
                for (unsigned j = 0; j < it; j++) acc += res[j] * V[(size_t)j * size + k];
                x[k] = acc;
            }
        }
    }
#undef H
    if (status == 0) {
        if (log) fprintf(log, "\n\n***PROBLEM CONVERGES IN %d ITERATIONS***\n\n", (int)it);
        memcpy(B, x, size * sizeof(double));
    } else if (status == 1 && log) {
        fprintf(log, "Problem fails to vonverge to given tolerance in %d iterations\n\n", (int)M);
    }
    if (iters) *iters = it;
    free(s); free(c); free(res); free(h); free(V); free(x);
    return status;
}
