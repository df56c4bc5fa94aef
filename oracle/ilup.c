/*
 * ILU(p) with level-of-fill dropping: CPU restatement of
 * 00_CommonFiles/Solvers_and_Preconditioners/ilup.c:164-301
 * (LEVEL_OF_FILL_lu, the symbolic factorisation) and of
 * CSR/ILUp_precond_setup.c:73-168 (ILUp, the numeric one) and
 * CSR/ILUp_precond.c:4-47 (the substitutions), on one "factor CSR":
 * row i holds its L columns in ascending order, then the diagonal, then its
 * U columns in the order the symbolic pass let them in (the row's own
 * entries in CSR order, then the fill in discovery order) -- the order the
 * reference's backward substitution sums them in.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of the GPU library).
 */
#include <stdlib.h>
#include <string.h>

#include "femoracle.h"

/* Symbolic ILU(p) of the pattern (IA, JA) (n rows, columns ascending).
 * Returns the factor CSR in freshly allocated *FIA (n+1), *FJA, *FDG (n,
 * position of the diagonal); the caller frees them with free(). */
int or_ilup_symbolic(int n, const int *IA, const int *JA, int p, int **FIA, int **FJA, int **FDG)
{
    int *iw = malloc(sizeof(int) * (size_t)(n ? n : 1));
    int *lc = malloc(sizeof(int) * (size_t)(n ? n : 1)), *ll = malloc(sizeof(int) * (size_t)(n ? n : 1));
    int *uc = malloc(sizeof(int) * (size_t)(n ? n : 1)), *ul = malloc(sizeof(int) * (size_t)(n ? n : 1));
    int **urow = calloc((size_t)(n ? n : 1), sizeof(int *)), **ulev = calloc((size_t)(n ? n : 1), sizeof(int *));
    int **lrow = calloc((size_t)(n ? n : 1), sizeof(int *));
    int *nl = calloc((size_t)(n ? n : 1), sizeof(int)), *nu = calloc((size_t)(n ? n : 1), sizeof(int));
    int i, j, q;
    for (j = 0; j < n; j++) iw[j] = -1;
    for (i = 0; i < n; i++) {
        int incl = 0, incu = 0;
        /* the row's own entries at level 0: L part and U part (iw holds the
           slot, U slots offset by n so the two lists share one map) */
        for (q = IA[i]; q < IA[i + 1]; q++) {
            int c = JA[q];
            if (c < i) { lc[incl] = c; ll[incl] = 0; iw[c] = incl++; }
            else if (c > i) { uc[incu] = c; ul[incu] = 0; iw[c] = n + incu++; }
        }
        /* eliminate the L part leftmost pivot first; fill of level
           lev(i,k) + lev(k,c) + 1 <= p enters the row */
        for (int jp = 0; jp < incl; jp++) {
            int jm = jp;
            for (j = jp + 1; j < incl; j++)
                if (lc[j] < lc[jm]) jm = j;
            if (jm != jp) {
                int tc = lc[jp], tl = ll[jp];
                lc[jp] = lc[jm]; ll[jp] = ll[jm];
                lc[jm] = tc; ll[jm] = tl;
                iw[lc[jp]] = jp;
                iw[lc[jm]] = jm;
            }
            int k = lc[jp];
            for (j = 0; j < nu[k]; j++) {
                int c = urow[k][j], it = ulev[k][j] + ll[jp] + 1;
                if (it > p) continue;
                int slot = iw[c];
                if (slot == -1) {
                    if (c < i) { lc[incl] = c; ll[incl] = it; iw[c] = incl++; }
                    else if (c > i) { uc[incu] = c; ul[incu] = it; iw[c] = n + incu++; }
                } else if (slot < n) {
                    if (it < ll[slot]) ll[slot] = it;
                } else {
                    if (it < ul[slot - n]) ul[slot - n] = it;
                }
            }
        }
        for (j = 0; j < incl; j++) iw[lc[j]] = -1;
        for (j = 0; j < incu; j++) iw[uc[j]] = -1;
        nl[i] = incl;
        nu[i] = incu;
        lrow[i] = malloc(sizeof(int) * (size_t)(incl ? incl : 1));
        memcpy(lrow[i], lc, sizeof(int) * (size_t)incl);
        urow[i] = malloc(sizeof(int) * (size_t)(incu ? incu : 1));
        ulev[i] = malloc(sizeof(int) * (size_t)(incu ? incu : 1));
        memcpy(urow[i], uc, sizeof(int) * (size_t)incu);
        memcpy(ulev[i], ul, sizeof(int) * (size_t)incu);
    }
    int *fia = malloc(sizeof(int) * ((size_t)n + 1)), *fdg = malloc(sizeof(int) * (size_t)(n ? n : 1));
    fia[0] = 0;
    for (i = 0; i < n; i++) fia[i + 1] = fia[i] + nl[i] + 1 + nu[i];
    int *fja = malloc(sizeof(int) * (size_t)(fia[n] ? fia[n] : 1));
    for (i = 0; i < n; i++) {
        int b = fia[i];
        memcpy(fja + b, lrow[i], sizeof(int) * (size_t)nl[i]);
        fdg[i] = b + nl[i];
        fja[fdg[i]] = i;
        memcpy(fja + fdg[i] + 1, urow[i], sizeof(int) * (size_t)nu[i]);
        free(lrow[i]); free(urow[i]); free(ulev[i]);
    }
    free(iw); free(lc); free(ll); free(uc); free(ul); free(urow); free(ulev); free(lrow); free(nl); free(nu);
    *FIA = fia;
    *FJA = fja;
    *FDG = fdg;
    return 0;
}

/* Numeric ILU(p) on the factor CSR: LU receives L (multipliers) and U, D the
 * inverse pivots.  AA holds the matrix on its own pattern (IA, JA).
 * Returns 0, or i + 1 when pivot i is zero. */
int or_ilup_factor(int n, const int *IA, const int *JA, const double *AA, const int *FIA, const int *FJA,
                   const int *FDG, double *LU, double *D)
{
    int *jw = malloc(sizeof(int) * (size_t)(n ? n : 1));
    int i, k;
    for (k = 0; k < n; k++) jw[k] = -1;
    for (i = 0; i < n; i++) {
        for (k = FIA[i]; k < FIA[i + 1]; k++) { jw[FJA[k]] = k; LU[k] = 0.0; }
        D[i] = 0.0;
        for (k = IA[i]; k < IA[i + 1]; k++) {
            if (JA[k] == i) D[i] = AA[k];
            else LU[jw[JA[k]]] = AA[k];
        }
        for (k = FIA[i]; k < FDG[i]; k++) {                  /* L part, ascending */
            int jrow = FJA[k];
            LU[k] *= D[jrow];
            for (int m = FDG[jrow] + 1; m < FIA[jrow + 1]; m++) {
                int pos = jw[FJA[m]];
                if (pos < 0) continue;
                if (FJA[m] == i) D[i] -= LU[k] * LU[m];
                else LU[pos] -= LU[k] * LU[m];
            }
        }
        for (k = FIA[i]; k < FIA[i + 1]; k++) jw[FJA[k]] = -1;
        if (D[i] == 0.0) { free(jw); return i + 1; }
        D[i] = 1.0 / D[i];
    }
    free(jw);
    return 0;
}

/* x = U^-1 L^-1 y on the factor CSR (x may alias y). */
void or_ilup_apply(int n, const int *FIA, const int *FJA, const int *FDG, const double *LU, const double *D,
                   const double *y, double *x)
{
    int i, k;
    for (i = 0; i < n; i++) {
        double v = y[i];
        for (k = FIA[i]; k < FDG[i]; k++) v -= x[FJA[k]] * LU[k];
        x[i] = v;
    }
    for (i = n - 1; i >= 0; i--) {
        double v = x[i];
        for (k = FDG[i] + 1; k < FIA[i + 1]; k++) v -= x[FJA[k]] * LU[k];
        x[i] = v * D[i];
    }
}
