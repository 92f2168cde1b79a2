/*
 * assembly.c -- node normals and dense collocation assembly
 * (oracle restatement of src/normals.c and src/assembly_el.c; test
 * infrastructure).
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include "oracle.h"

/* Local coordinates of node position p of a tria6 (src/normals.c:240-264). */
static const double TRIA6_NODE_L[6][2] = {
    {1.0, 0.0}, {0.5, 0.5}, {0.0, 1.0}, {0.0, 0.5}, {0.0, 0.0}, {0.5, 0.0}};

/* Average of the unit element normals at the node over every element that
 * contains it, in element order, re-normalised (getNormal_tria3
 * src/normals.c:120-199, getNormal_tria6 :207-319).  Only the first
 * occurrence of the node within an element counts. */
void orc_node_normal(int nen, unsigned E, const double *nodes, const unsigned *elems,
                     unsigned node1, double n[3])
{
    double acc[3] = {0.0, 0.0, 0.0}, X[18], ln[3];
    for (unsigned e = 0; e < E; e++) {
        int pos = -1;
        for (int k = 0; k < nen; k++)
            if (elems[(size_t)e * nen + k] == node1) { pos = k; break; }
        if (pos < 0) continue;
        for (int k = 0; k < nen; k++) {
            const double *x = nodes + 3 * (size_t)(elems[(size_t)e * nen + k] - 1);
            X[k * 3 + 0] = x[0];
            X[k * 3 + 1] = x[1];
            X[k * 3 + 2] = x[2];
        }
        const double L0[2] = {0.0, 0.0};
        orc_local_normal(nen, X, nen == 6 ? TRIA6_NODE_L[pos] : L0, ln);
        acc[0] += ln[0];
        acc[1] += ln[1];
        acc[2] += ln[2];
    }
    double inv = 1.0 / sqrt(acc[0] * acc[0] + acc[1] * acc[1] + acc[2] * acc[2]);
    n[0] = acc[0] * inv;
    n[1] = acc[1] * inv;
    n[2] = acc[2] * inv;
}

/* A_k, B_k of the interface equation: A_k - i B_k = C (s1 - s2) / (s1 + s2)
 * with s = sigma + i omega eps0 eps_r and C = 1 / (4 pi eps0)
 * (src/assembly_el.c:223-239). */
void orc_interface_coeffs(unsigned nIf, const unsigned *ifaces, const double *mat,
                          double freq, double *Ak, double *Bk)
{
    double C = 1.0 / (ORC_PI4 * ORC_EPS0);
    double W = freq * ORC_PI2 * ORC_EPS0;
    for (unsigned i = 0; i < nIf; i++) {
        unsigned m1 = ifaces[2 * i] - 1, m2 = ifaces[2 * i + 1] - 1;
        double sigTot = mat[2 * m1] + mat[2 * m2];
        double sigDif = mat[2 * m1] - mat[2 * m2];
        double epsTot = W * (mat[2 * m1 + 1] + mat[2 * m2 + 1]);
        double epsDif = W * (mat[2 * m1 + 1] - mat[2 * m2 + 1]);
        double D = C / (sigTot * sigTot + epsTot * epsTot);
        Ak[i] = D * (sigTot * sigDif + epsTot * epsDif);
        Bk[i] = D * (sigDif * epsTot - sigTot * epsDif);
    }
}

struct asm_job {
    int nen, full;
    unsigned N, E;
    const double *nodes;
    const unsigned *elems, *bctype;
    const double *mbc;
    const double *Ak, *Bk;
    unsigned row0, row1;
    double *A;
    size_t lda;
    double *B;
    int bad;
};

/* One collocation row i: conductor rows (type 1) integrate C G N_k, the
 * other rows integrate H N_k with the node normal and take the jump term
 * -1/(2 eps0) on the diagonal (src/assembly_el.c:242-300 compact form,
 * :508-580 full 2x2-block form). */
static void assemble_rows(struct asm_job *jb)
{
    const int nen = jb->nen;
    const unsigned N = jb->N;
    const double C = 1.0 / (ORC_PI4 * ORC_EPS0);
    double X[18], Xe[3], nrm[3] = {0, 0, 0}, Sub[6];
    for (unsigned i = jb->row0; i < jb->row1; i++) {
        unsigned t = jb->bctype[i];
        if (t != 0 && t != 1 && t != 6) { jb->bad = 1; continue; }
        double *Ai = jb->A + (size_t)i * jb->lda;
        double *Aim = jb->full ? jb->A + (size_t)(i + N) * jb->lda : NULL;
        Xe[0] = jb->nodes[3 * (size_t)i];
        Xe[1] = jb->nodes[3 * (size_t)i + 1];
        Xe[2] = jb->nodes[3 * (size_t)i + 2];
        unsigned ifc = 0;
        if (t != 1) {
            ifc = (unsigned)jb->mbc[3 * (size_t)i + 1] - 1;
            orc_node_normal(nen, jb->E, jb->nodes, jb->elems, i + 1, nrm);
            Ai[i] -= 0.5 / ORC_EPS0;
            if (jb->full) Aim[i + N] -= 0.5 / ORC_EPS0;
        }
        for (unsigned e = 0; e < jb->E; e++) {
            const unsigned *el = jb->elems + (size_t)e * nen;
            unsigned sin = 0;
            for (int k = 0; k < nen; k++) {
                const double *x = jb->nodes + 3 * (size_t)(el[k] - 1);
                X[k * 3 + 0] = x[0];
                X[k * 3 + 1] = x[1];
                X[k * 3 + 2] = x[2];
                if (el[k] - 1 == i) sin = (unsigned)k + 1;
            }
            if (t == 1) {
                if (sin == 0) orc_intG(nen, X, Xe, Sub);
                else orc_intSingularG(nen, sin, X, Xe, Sub);
                for (int k = 0; k < nen; k++) {
                    double F = C * Sub[k];
                    unsigned c = el[k] - 1;
                    Ai[c] += F;
                    if (jb->full) Aim[c + N] += F;
                }
            } else {
                if (sin == 0) orc_intH(nen, 0, X, Xe, Sub, nrm);
                else orc_intSingularH(nen, 0, sin, X, Xe, Sub, nrm);
                for (int k = 0; k < nen; k++) {
                    double F = jb->Ak[ifc] * Sub[k];
                    double G = jb->Bk[ifc] * Sub[k];
                    unsigned c = el[k] - 1;
                    Ai[c] += F;
                    Ai[c + N] += G;
                    if (jb->full) {
                        Aim[c] -= G;
                        Aim[c + N] += F;
                    }
                }
            }
        }
        jb->B[i] = jb->mbc[3 * (size_t)i];
        jb->B[i + N] = jb->mbc[3 * (size_t)(i + N)];
    }
}

struct asm_pool {
    struct asm_job proto;
    unsigned next, row1, chunk;
    int bad;
};

/* Worker: takes chunks of `chunk` rows from a shared counter until the
 * range is exhausted; each row is formed exactly as in the serial loop. */
static void *asm_thread(void *p)
{
    struct asm_pool *pool = (struct asm_pool *)p;
    struct asm_job j = pool->proto;
    for (;;) {
        unsigned r0 = __atomic_fetch_add(&pool->next, pool->chunk, __ATOMIC_RELAXED);
        if (r0 >= pool->row1) break;
        j.row0 = r0;
        j.row1 = r0 + pool->chunk < pool->row1 ? r0 + pool->chunk : pool->row1;
        assemble_rows(&j);
    }
    if (j.bad) __atomic_store_n(&pool->bad, 1, __ATOMIC_RELAXED);
    return NULL;
}

int orc_assemble(int nen, int full, unsigned N, unsigned E, unsigned nIf,
                 const double *nodes, const unsigned *elems, const unsigned *bctype,
                 const unsigned *ifaces, const double *mat, double freq,
                 const double *mbc, unsigned row0, unsigned row1,
                 double *A, size_t lda, double *B, int nthreads)
{
    double *Ak = (double *)calloc(nIf ? nIf : 1, sizeof(double));
    double *Bk = (double *)calloc(nIf ? nIf : 1, sizeof(double));
    if (nIf) orc_interface_coeffs(nIf, ifaces, mat, freq, Ak, Bk);
    struct asm_pool pool;
    pool.proto = (struct asm_job){nen, full, N, E, nodes, elems, bctype, mbc, Ak, Bk,
                                  row0, row1, A, lda, B, 0};
    pool.next = row0;
    pool.row1 = row1;
    pool.chunk = 4;
    pool.bad = 0;
    if (nthreads <= 1) {
        assemble_rows(&pool.proto);
        pool.bad = pool.proto.bad;
    } else {
        pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof *th);
        for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, asm_thread, &pool);
        for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
        free(th);
    }
    free(Ak);
    free(Bk);
    return pool.bad;
}
