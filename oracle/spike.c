/*
 * femoracle: truncated SPIKE preconditioner.  TEST INFRASTRUCTURE ONLY (see
 * femoracle.h).
 *
 * Restates the partitioned SPIKE of 00_CommonFiles/Solvers_and_Preconditioners/
 * CSR/SPIKE_precond_setup.c:10-266 and CSR/SPIKE_precond.c:8-158 on one
 * address space, the P MPI ranks becoming P row blocks of the CSR matrix:
 *
 *   set-up   each block's diagonal part A_q is factorised (here: banded LU
 *            without pivoting in place of PARDISO, whose binaries are absent
 *            from the reference tree); the k x k couplings B_q (last k rows of
 *            block q, first k columns of block q+1) and C_q (first k rows of
 *            block q, last k columns of block q-1) give the tips
 *              V_q = bottom k rows of A_q^-1 [0; B_q]   (PARDISO_bottom_tips)
 *              W_q = top k rows of A_q^-1 [C_q; 0]      (PARDISO_top_tips)
 *            and every interface q | q+1 the 2k x 2k reduced system
 *              S_q = [I V_q; W_q+1 I]  (PARALLEL_REDUCED_system, :271-312),
 *            factorised here by dense LU with partial pivoting;
 *   apply    g = A_q^-1 f per block, [xB_q; xT_q+1] = S_q^-1 [g_bottom(q);
 *            g_top(q+1)] per interface, then y_q = A_q^-1 (f_q - B_q xT_q+1
 *            - C_q xB_q-1) per block (SPIKE_precond.c:34-118).
 *
 * Couplings outside the two k x k corners are dropped, as the reference
 * drops them.  Two departures from the reference's arithmetic, both where
 * it is not the textbook method: the reference's tips pass the row-major
 * n x k coupling array to a solver reading it column-major, and it applies
 * B_q xT to the first k rows of the block rather than the last k; here B_q
 * sits in the last k rows in both places.
 *
 * Every loop's operation order is the one the CUDA kernels use (row-wise
 * sums in ascending column order, backward sweeps in descending column
 * order, one division by the pivot), so the GPU set-up and apply are
 * bit-exact against this file when both avoid FMA contraction.
 */
#include "femoracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

struct or_spike {
    int n, k, P;
    int *bs;            /* P+1 block starts */
    int *kl, *ku;       /* per-block lower / upper bandwidth */
    long *boff;         /* P+1 offsets of the band storage */
    double *band;       /* per block column-major band, ld = kl+ku+1 */
    double *B, *C;      /* (P-1) x k x k, row-major; C[q] couples block q+1 */
    double *S;          /* (P-1) x 2k x 2k LU of the reduced systems */
    int *piv;           /* (P-1) x 2k row interchanges */
};

/* element (i, j) of block q (local indices) in band storage */
#define BAND(sp, q, i, j) \
    ((sp)->band[(sp)->boff[q] + (long)((sp)->ku[q] + (i) - (j)) + (long)(j) * ((sp)->kl[q] + (sp)->ku[q] + 1)])

int or_spike_blocks(int n, int k, int parts)
{
    int P = parts;
    if (k > 0 && P > n / (2 * k)) P = n / (2 * k);
    return P < 1 ? 1 : P;
}

/* Banded LU without pivoting of block q (right-looking). */
static int band_lu(or_spike *sp, int q)
{
    const int m = sp->bs[q + 1] - sp->bs[q], kl = sp->kl[q], ku = sp->ku[q];
    int rc = 0;
    for (int j = 0; j < m; ++j) {
        const double piv = BAND(sp, q, j, j);
        if (piv == 0.0) rc = -1;
        const int ie = j + kl < m - 1 ? j + kl : m - 1;
        const int ce = j + ku < m - 1 ? j + ku : m - 1;
        for (int i = j + 1; i <= ie; ++i) BAND(sp, q, i, j) = BAND(sp, q, i, j) / piv;
        for (int i = j + 1; i <= ie; ++i) {
            const double l = BAND(sp, q, i, j);
            for (int c = j + 1; c <= ce; ++c) BAND(sp, q, i, c) = BAND(sp, q, i, c) - l * BAND(sp, q, j, c);
        }
    }
    return rc;
}

/* z <- U^-1 L^-1 z over local rows [r0, m) of block q for nrhs columns of
 * a row-major m x nrhs array (rows below r0 are zero on entry and are left
 * out of the forward sweep; the backward sweep stops at row r0). */
static void band_solve(const or_spike *sp, int q, int r0, double *z, int nrhs)
{
    const int m = sp->bs[q + 1] - sp->bs[q], kl = sp->kl[q], ku = sp->ku[q];
    for (int c = 0; c < nrhs; ++c) {
        for (int i = r0; i < m; ++i) {
            double v = z[(long)i * nrhs + c];
            const int jb = i - kl > r0 ? i - kl : r0;
            for (int j = jb; j < i; ++j) v = v - BAND(sp, q, i, j) * z[(long)j * nrhs + c];
            z[(long)i * nrhs + c] = v;
        }
        for (int i = m - 1; i >= r0; --i) {
            double v = z[(long)i * nrhs + c];
            const int je = i + ku < m - 1 ? i + ku : m - 1;
            for (int j = je; j > i; --j) v = v - BAND(sp, q, i, j) * z[(long)j * nrhs + c];
            z[(long)i * nrhs + c] = v / BAND(sp, q, i, i);
        }
    }
}

/* Dense LU with partial pivoting (first largest |a| wins) of a row-major
 * N x N matrix. */
static int dense_lu(double *a, int *piv, int N)
{
    int rc = 0;
    for (int j = 0; j < N; ++j) {
        int p = j;
        double best = fabs(a[(long)j * N + j]);
        for (int i = j + 1; i < N; ++i)
            if (fabs(a[(long)i * N + j]) > best) { best = fabs(a[(long)i * N + j]); p = i; }
        piv[j] = p;
        if (p != j)
            for (int c = 0; c < N; ++c) {
                double t = a[(long)j * N + c];
                a[(long)j * N + c] = a[(long)p * N + c];
                a[(long)p * N + c] = t;
            }
        const double d = a[(long)j * N + j];
        if (d == 0.0) rc = -1;
        for (int i = j + 1; i < N; ++i) a[(long)i * N + j] = a[(long)i * N + j] / d;
        for (int i = j + 1; i < N; ++i) {
            const double l = a[(long)i * N + j];
            for (int c = j + 1; c < N; ++c) a[(long)i * N + c] = a[(long)i * N + c] - l * a[(long)j * N + c];
        }
    }
    return rc;
}

static void dense_solve(const double *a, const int *piv, int N, double *x)
{
    for (int j = 0; j < N; ++j)
        if (piv[j] != j) { double t = x[j]; x[j] = x[piv[j]]; x[piv[j]] = t; }
    for (int i = 0; i < N; ++i) {
        double v = x[i];
        for (int j = 0; j < i; ++j) v = v - a[(long)i * N + j] * x[j];
        x[i] = v;
    }
    for (int i = N - 1; i >= 0; --i) {
        double v = x[i];
        for (int j = N - 1; j > i; --j) v = v - a[(long)i * N + j] * x[j];
        x[i] = v / a[(long)i * N + i];
    }
}

void or_spike_free(or_spike *sp)
{
    if (!sp) return;
    free(sp->bs); free(sp->kl); free(sp->ku); free(sp->boff); free(sp->band);
    free(sp->B); free(sp->C); free(sp->S); free(sp->piv);
    free(sp);
}

/* Set-up from a CSR matrix (0-based, rows sorted): n rows, coupling size k,
 * at most `parts` blocks (each keeps at least 2k rows).  *err receives 0,
 * -1 (zero pivot in a block or a reduced system) or -2 (bad arguments). */
or_spike *or_spike_setup(int n, const int *IA, const int *JA, const double *AA, int k, int parts, int *err)
{
    *err = 0;
    if (n < 1 || k < 1 || parts < 1) { *err = -2; return NULL; }
    or_spike *sp = (or_spike *)calloc(1, sizeof(or_spike));
    const int P = or_spike_blocks(n, k, parts);
    sp->n = n; sp->k = k; sp->P = P;
    sp->bs = (int *)malloc(sizeof(int) * (P + 1));
    sp->kl = (int *)calloc(P, sizeof(int));
    sp->ku = (int *)calloc(P, sizeof(int));
    sp->boff = (long *)malloc(sizeof(long) * (P + 1));
    for (int q = 0; q <= P; ++q) sp->bs[q] = (int)((long)n * q / P);
    for (int q = 0; q < P; ++q)
        for (int i = sp->bs[q]; i < sp->bs[q + 1]; ++i)
            for (int e = IA[i]; e < IA[i + 1]; ++e) {
                const int j = JA[e];
                if (j < sp->bs[q] || j >= sp->bs[q + 1]) continue;
                if (i - j > sp->kl[q]) sp->kl[q] = i - j;
                if (j - i > sp->ku[q]) sp->ku[q] = j - i;
            }
    sp->boff[0] = 0;
    for (int q = 0; q < P; ++q)
        sp->boff[q + 1] = sp->boff[q] + (long)(sp->bs[q + 1] - sp->bs[q]) * (sp->kl[q] + sp->ku[q] + 1);
    sp->band = (double *)calloc(sp->boff[P] > 0 ? sp->boff[P] : 1, sizeof(double));
    const long kk = (long)k * k, ni = P - 1;
    sp->B = (double *)calloc(ni * kk + 1, sizeof(double));
    sp->C = (double *)calloc(ni * kk + 1, sizeof(double));
    sp->S = (double *)calloc(ni * 4 * kk + 1, sizeof(double));
    sp->piv = (int *)calloc(ni * 2 * k + 1, sizeof(int));
    /* diagonal blocks and the two corner couplings of every interface */
    for (int q = 0; q < P; ++q)
        for (int i = sp->bs[q]; i < sp->bs[q + 1]; ++i)
            for (int e = IA[i]; e < IA[i + 1]; ++e) {
                const int j = JA[e];
                if (j >= sp->bs[q] && j < sp->bs[q + 1]) {
                    BAND(sp, q, i - sp->bs[q], j - sp->bs[q]) = AA[e];
                } else if (q + 1 < P && i >= sp->bs[q + 1] - k && j >= sp->bs[q + 1] && j < sp->bs[q + 1] + k) {
                    sp->B[q * kk + (long)(i - (sp->bs[q + 1] - k)) * k + (j - sp->bs[q + 1])] = AA[e];
                } else if (q > 0 && i < sp->bs[q] + k && j >= sp->bs[q] - k && j < sp->bs[q]) {
                    sp->C[(q - 1) * kk + (long)(i - sp->bs[q]) * k + (j - (sp->bs[q] - k))] = AA[e];
                }
            }
    for (int q = 0; q < P; ++q)
        if (band_lu(sp, q)) *err = -1;
    /* tips and reduced systems */
    const int K2 = 2 * k;
    for (int q = 0; q + 1 < P; ++q) {
        double *S = sp->S + q * 4 * kk;
        const int m0 = sp->bs[q + 1] - sp->bs[q], m1 = sp->bs[q + 2] - sp->bs[q + 1];
        double *z = (double *)calloc((size_t)(m0 > m1 ? m0 : m1) * k, sizeof(double));
        /* V_q: bottom k rows of A_q^-1 [0; B_q] */
        for (long r = 0; r < kk; ++r) z[(long)(m0 - k) * k + r] = sp->B[q * kk + r];
        band_solve(sp, q, m0 - k, z, k);
        for (int r = 0; r < k; ++r) {
            S[(long)r * K2 + r] = 1.0;
            for (int c = 0; c < k; ++c) S[(long)r * K2 + k + c] = z[(long)(m0 - k + r) * k + c];
        }
        /* W_q+1: top k rows of A_q+1^-1 [C_q+1; 0] */
        memset(z, 0, sizeof(double) * (size_t)m1 * k);
        for (long r = 0; r < kk; ++r) z[r] = sp->C[q * kk + r];
        band_solve(sp, q + 1, 0, z, k);
        for (int r = 0; r < k; ++r) {
            for (int c = 0; c < k; ++c) S[(long)(k + r) * K2 + c] = z[(long)r * k + c];
            S[(long)(k + r) * K2 + k + r] = 1.0;
        }
        free(z);
        if (dense_lu(S, sp->piv + (long)q * K2, K2)) *err = -1;
    }
    return sp;
}

/* y = M^-1 f (n entries each; y may be f). */
void or_spike_apply(const or_spike *sp, const double *f, double *y)
{
    const int n = sp->n, k = sp->k, P = sp->P, K2 = 2 * k;
    const long kk = (long)k * k;
    double *g = (double *)malloc(sizeof(double) * n);
    double *x = (double *)calloc((size_t)(P > 1 ? P - 1 : 1) * K2, sizeof(double));
    memcpy(g, f, sizeof(double) * n);
    for (int q = 0; q < P; ++q) band_solve(sp, q, 0, g + sp->bs[q], 1);
    for (int q = 0; q + 1 < P; ++q) {
        double *xq = x + (long)q * K2;
        for (int r = 0; r < k; ++r) {
            xq[r] = g[sp->bs[q + 1] - k + r];
            xq[k + r] = g[sp->bs[q + 1] + r];
        }
        dense_solve(sp->S + q * 4 * kk, sp->piv + (long)q * K2, K2, xq);
    }
    /* corrected right-hand side: rows of block q coupled to xT of the
     * interface below (B_q) and to xB of the interface above (C_q) */
    memcpy(g, f, sizeof(double) * n);
    for (int q = 0; q < P; ++q) {
        if (q + 1 < P)
            for (int r = 0; r < k; ++r) {
                double s = 0.0;
                for (int c = 0; c < k; ++c) s = s + sp->B[q * kk + (long)r * k + c] * x[(long)q * K2 + k + c];
                g[sp->bs[q + 1] - k + r] = g[sp->bs[q + 1] - k + r] - s;
            }
        if (q > 0)
            for (int r = 0; r < k; ++r) {
                double s = 0.0;
                for (int c = 0; c < k; ++c) s = s + sp->C[(q - 1) * kk + (long)r * k + c] * x[(long)(q - 1) * K2 + c];
                g[sp->bs[q] + r] = g[sp->bs[q] + r] - s;
            }
        band_solve(sp, q, 0, g + sp->bs[q], 1);
    }
    memcpy(y, g, sizeof(double) * n);
    free(g);
    free(x);
}

/* Block layout: P, k, block starts (P+1), bandwidths (P each); any NULL. */
int or_spike_info(const or_spike *sp, int *k, int *bs, int *kl, int *ku)
{
    if (k) *k = sp->k;
    for (int q = 0; q <= sp->P; ++q) {
        if (bs) bs[q] = sp->bs[q];
        if (q < sp->P && kl) kl[q] = sp->kl[q];
        if (q < sp->P && ku) ku[q] = sp->ku[q];
    }
    return sp->P;
}
