/*
 * femoracle: assembled CSR path and ILU(0).  TEST INFRASTRUCTURE ONLY (see
 * femoracle.h).
 *
 * Restates 01_SS_Transport_Equation/2D/01_CommonFiles/csr_Initialization.c
 * (pattern of the free dofs, renumbered by the same local RCM as the EBE
 * path, :408-433), csr_assembly.c:3-54 (element blocks summed into CSR
 * slots in element order), 00_CommonFiles/MatrixVector_Operations/CSR/
 * csrmv.c:57-62 (row sums in column order), and ILU(0) of
 * Solvers_and_Preconditioners/CSR/ILUp_precond_setup.c:73-168 (IKJ
 * elimination over the sorted L part, inverse pivots stored) with
 * CSR/ILUp_precond.c:4-47 (forward then backward substitution).
 */
#include "femoracle.h"
#include <stdlib.h>
#include <string.h>

static int find_col(const int *JA, int b, int e, int col)
{
    int lo = b, hi = e - 1;
    while (lo <= hi) {
        int m = (lo + hi) / 2;
        if (JA[m] == col) return m;
        if (JA[m] < col) lo = m + 1; else hi = m - 1;
    }
    return -1;
}

/* CSR pattern of the free dofs with rows and columns renumbered by
 * invPerm (row i of the result is reference dof Perm[i]).  Returns nnz. */
int or_csr_pattern(int nel, const int *ien, const int *type, const int *invp, int NEQ,
                   const int *Perm, const int *invPerm, int *IA, int *JA)
{
    int *IA0 = malloc(sizeof(int) * ((size_t)NEQ + 1));
    int *JA0 = malloc(sizeof(int) * ((size_t)nel * 9 + 1));
    int nnz = or_lm_adjacency(nel, ien, type, invp, NEQ, IA0, JA0);
    int i, k, o = 0;
    IA[0] = 0;
    for (i = 0; i < NEQ; i++) {
        int r = Perm[i], s = o;
        for (k = IA0[r]; k < IA0[r + 1]; k++) JA[o++] = invPerm[JA0[k]];
        /* insertion sort of the (short) row */
        for (int a = s + 1; a < o; a++) {
            int v = JA[a], b = a - 1;
            while (b >= s && JA[b] > v) { JA[b + 1] = JA[b]; b--; }
            JA[b + 1] = v;
        }
        IA[i + 1] = o;
    }
    free(IA0); free(JA0);
    return nnz;
}

/* csr_assembly: AA[slot] += A_e[a][b] for the free (row, column) pairs of
 * each element, elements in order.  lm is in the CSR numbering. */
void or_csr_assemble(int nel, int S, const int *lm, const double *A, int NEQ,
                     const int *IA, const int *JA, double *AA)
{
    memset(AA, 0, sizeof(double) * (size_t)IA[NEQ]);
    for (int e = 0; e < nel; e++)
        for (int a = 0; a < S; a++) {
            int r = lm[(long)S * e + a];
            if (r == NEQ) continue;
            for (int b = 0; b < S; b++) {
                int c = lm[(long)S * e + b];
                if (c == NEQ) continue;
                int k = find_col(JA, IA[r], IA[r + 1], c);
                AA[k] += A[(long)S * S * e + S * a + b];
            }
        }
}

/* csrmv for one rank: Q = A P, rows summed in column order. */
void or_csrmv(int n, const int *IA, const int *JA, const double *AA, const double *P, double *Q)
{
    for (int i = 0; i < n; i++) {
        double q = 0.0;
        for (int k = IA[i]; k < IA[i + 1]; k++) q += AA[k] * P[JA[k]];
        Q[i] = q;
    }
}

/* ILU(0) numeric factorisation on the pattern of A.  LU[k] holds the L
 * multiplier (column < row) or the U entry (column > row) of slot k;
 * D[i] the inverse pivot.  Returns 0, or i+1 on a zero pivot in row i. */
int or_ilu0_factor(int n, const int *IA, const int *JA, const double *AA, double *LU, double *D)
{
    int *jw = malloc(sizeof(int) * ((size_t)n + 1));
    int i, j, k;
    for (j = 0; j < n; j++) jw[j] = -1;
    for (i = 0; i < n; i++) {
        for (k = IA[i]; k < IA[i + 1]; k++) { jw[JA[k]] = k; LU[k] = 0.0; }
        D[i] = 0.0;
        for (k = IA[i]; k < IA[i + 1]; k++) {
            if (JA[k] == i) D[i] = AA[k];
            else LU[k] = AA[k];
        }
        for (k = IA[i]; k < IA[i + 1] && JA[k] < i; k++) {
            int jrow = JA[k];
            LU[k] *= D[jrow];
            for (int m = IA[jrow]; m < IA[jrow + 1]; m++) {
                int col = JA[m];
                if (col <= jrow) continue;            /* U part of jrow */
                int pos = jw[col];
                if (pos < 0) continue;
                if (col == i) D[i] -= LU[k] * LU[m];
                else LU[pos] -= LU[k] * LU[m];
            }
        }
        for (k = IA[i]; k < IA[i + 1]; k++) jw[JA[k]] = -1;
        if (D[i] == 0.0) { free(jw); return i + 1; }
        D[i] = 1.0 / D[i];
    }
    free(jw);
    return 0;
}

/* ILUp_precond: x = U^-1 L^-1 y (x may alias y). */
void or_ilu0_apply(int n, const int *IA, const int *JA, const double *LU, const double *D,
                   const double *y, double *x)
{
    int i, k;
    for (i = 0; i < n; i++) {
        double v = y[i];
        for (k = IA[i]; k < IA[i + 1] && JA[k] < i; k++) v -= x[JA[k]] * LU[k];
        x[i] = v;
    }
    for (i = n - 1; i >= 0; i--) {
        double v = x[i];
        for (k = IA[i]; k < IA[i + 1]; k++)
            if (JA[k] > i) v -= x[JA[k]] * LU[k];
        x[i] = v * D[i];
    }
}
