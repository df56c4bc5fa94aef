/*
 * femoracle: structured mesh, Fill_LM, dof adjacency and reverse
 * Cuthill-McKee.  TEST INFRASTRUCTURE ONLY (see femoracle.h).
 */
#include "femoracle.h"
#include <stdlib.h>
#include <string.h>
#include <math.h>

/* Structured rectangle split into triangles, node and triangle order as
 * Mesh_Generator/Structured_Mesh/meshGenerator.c:113-177 produces them:
 * nodes row by row (x fastest); per quad with lower-left node a two
 * triangles, "right" tilt (a, a+1, a+nx+1), (a, a+nx+1, a+nx);
 * "left" tilt (a, a+1, a+nx), (a+1, a+nx+1, a+nx). */
int or_mesh_structured(int M, int N, double x0, double y0, double x1, double y1,
                       int left_tilt, double *x, double *y, int *ien)
{
    int nx = M + 1, ny = N + 1, i, j, e = 0;
    double hx = (x1 - x0) / M, hy = (y1 - y0) / N;
    for (j = 0; j < ny; j++)
        for (i = 0; i < nx; i++) {
            x[j * nx + i] = x0 + i * hx;
            y[j * nx + i] = y0 + j * hy;
        }
    for (j = 0; j < N; j++)
        for (i = 0; i < M; i++) {
            int a = j * nx + i;
            if (!left_tilt) {
                ien[3*e] = a; ien[3*e+1] = a + 1;      ien[3*e+2] = a + nx + 1; e++;
                ien[3*e] = a; ien[3*e+1] = a + nx + 1; ien[3*e+2] = a + nx;     e++;
            } else {
                ien[3*e] = a;     ien[3*e+1] = a + 1;      ien[3*e+2] = a + nx; e++;
                ien[3*e] = a + 1; ien[3*e+1] = a + nx + 1; ien[3*e+2] = a + nx; e++;
            }
        }
    return e;
}

/* Fill_LM (01_SS_Transport_Equation/2D/01_CommonFiles/Fill_LM.c:3-27 for
 * ndof = 1; 03_Euler_Equations/2D/01_CommonFiles/Fill_LM.c:3-31 for ndof > 1):
 * dof k of vertex i of element e goes to slot ndof*i + k; Dirichlet -> NEQ. */
void or_fill_lm(int nel, int ndof, const int *ien, const int *type, const int *invp,
                int NEQ, int *lm)
{
    int S = 3 * ndof;
    for (int e = 0; e < nel; e++)
        for (int i = 0; i < 3; i++) {
            int node = ien[3*e + i];
            for (int k = 0; k < ndof; k++) {
                int d = node * ndof + k;
                lm[e*S + ndof*i + k] = type[d] == 0 ? NEQ : invp[d];
            }
        }
}

static int cmp_int(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* Row-sorted, duplicate-free adjacency of the free dofs
 * (Permutation_of_LM.c:21-49 builds the same sets with sorted linked lists). */
int or_lm_adjacency(int nel, const int *ien, const int *type, const int *invp,
                    int NEQ, int *IA, int *JA)
{
    int *cnt = calloc((size_t)NEQ + 1, sizeof(int));
    int *tmp;
    int e, a, b, r, nnz = 0;
    for (e = 0; e < nel; e++)
        for (a = 0; a < 3; a++)
            if (type[ien[3*e+a]] != 0)
                for (b = 0; b < 3; b++)
                    if (type[ien[3*e+b]] != 0) cnt[invp[ien[3*e+a]]]++;
    IA[0] = 0;
    for (r = 0; r < NEQ; r++) IA[r+1] = IA[r] + cnt[r];
    tmp = malloc(sizeof(int) * ((size_t)IA[NEQ] + 1));
    memset(cnt, 0, sizeof(int) * ((size_t)NEQ + 1));
    for (e = 0; e < nel; e++)
        for (a = 0; a < 3; a++)
            if (type[ien[3*e+a]] != 0) {
                int row = invp[ien[3*e+a]];
                for (b = 0; b < 3; b++)
                    if (type[ien[3*e+b]] != 0)
                        tmp[IA[row] + cnt[row]++] = invp[ien[3*e+b]];
            }
    /* sort and compact each row */
    int out = 0;
    for (r = 0; r < NEQ; r++) {
        int s = IA[r], t = IA[r+1];
        qsort(tmp + s, (size_t)(t - s), sizeof(int), cmp_int);
        IA[r] = out;
        for (int k = s; k < t; k++)
            if (k == s || tmp[k] != tmp[k-1]) JA[out++] = tmp[k];
    }
    IA[NEQ] = out;
    nnz = out;
    free(tmp);
    free(cnt);
    return nnz;
}

/* ---------------------------------------------------------------------
 * Reverse Cuthill-McKee, restating 00_CommonFiles/Reordering/symrcm.c.
 * The permutation must be bit-exact, so the tie-breaking of the
 * reference is kept: neighbours are visited in ascending index order
 * (merge of row i of A and of A^T, :136-199), queued through a binary
 * min-heap keyed by degree alone with strict comparisons (H_insert
 * :508-530, H_remove_min/H_heapify_min :532-567), and the start node of
 * each component comes from the repeated-BFS pseudo-peripheral search
 * (find_starting_node :352-483).
 * ------------------------------------------------------------------- */
typedef struct { int id, deg, dist; } rcm_node;

static void heap_push(rcm_node *h, int *size, rcm_node v)
{
    int i = (*size)++;
    h[i] = v;
    while (i > 0) {
        int p = (i - 1) / 2;
        if (h[i].deg < h[p].deg) { rcm_node t = h[i]; h[i] = h[p]; h[p] = t; i = p; }
        else break;
    }
}

static rcm_node heap_pop(rcm_node *h, int *size)
{
    rcm_node top = h[0];
    int n = --(*size), j = 0;
    h[0] = h[n];
    for (;;) {
        int l = 2*j + 1, r = 2*j + 2, m = j;
        if (l < n && h[l].deg < h[j].deg) m = l;
        if (r < n && h[r].deg < h[m].deg) m = r;
        if (m == j) break;
        rcm_node t = h[j]; h[j] = h[m]; h[m] = t; j = m;
    }
    return top;
}

/* Distinct neighbours of i: the union of row i of (IA,JA) and row i of its
 * transpose (IT,JT), in ascending order.  Returns the count. */
static int neighbours(int i, const int *IA, const int *JA, const int *IT,
                      const int *JT, int *out)
{
    int j1 = IA[i], e1 = IA[i+1], j2 = IT[i], e2 = IT[i+1], n = 0;
    while (j1 < e1 || j2 < e2) {
        if (j1 == e1) out[n++] = JT[j2++];
        else if (j2 == e2) out[n++] = JA[j1++];
        else {
            int a = JA[j1], b = JT[j2];
            if (a <= b) { out[n++] = a; j1++; if (a == b) j2++; }
            else { out[n++] = b; j2++; }
        }
    }
    return n;
}

static int pseudo_peripheral(int n, const int *IA, const int *JA, const int *IT,
                             const int *JT, const int *D, int start,
                             rcm_node *Q, int *seen, int *nb)
{
    rcm_node x = { start, D[start], 0 };
    int max_dist = 0;
    memset(seen, 0, sizeof(int) * (size_t)n);
    int qh = 0, qt = 0;
    Q[qt++] = x;
    seen[start] = 1;
    for (;;) {
        while (qh != qt) {
            rcm_node v = Q[qh++];
            if (v.dist > x.dist || (v.id != x.id && v.deg > x.deg)) x = v;
            int cnt = neighbours(v.id, IA, JA, IT, JT, nb);
            for (int t = 0; t < cnt; t++) {
                int r = nb[t];
                if (!seen[r]) {
                    rcm_node w = { r, D[r], v.dist + 1 };
                    Q[qt++] = w;
                    seen[r] = 1;
                }
            }
        }
        if (max_dist < x.dist) {
            max_dist = x.dist;
            memset(seen, 0, sizeof(int) * (size_t)n);
            seen[x.id] = 1;
            x.dist = 0;
            qh = qt = 0;
            Q[qt++] = x;
        } else break;
    }
    return x.id;
}

void or_symrcm(int n, const int *IA, const int *JA, int *perm)
{
    int nnz = IA[n];
    int *IT = calloc((size_t)n + 1, sizeof(int));
    int *JT = malloc(sizeof(int) * ((size_t)nnz + 1));
    int *D = calloc((size_t)n + 1, sizeof(int));
    int i, k, max_deg = 0;

    /* transpose (symrcm.c:270-305) */
    for (k = 0; k < nnz; k++) IT[JA[k] + 1]++;
    for (i = 0; i < n; i++) IT[i+1] += IT[i];
    {
        int *w = malloc(sizeof(int) * ((size_t)n + 1));
        memcpy(w, IT, sizeof(int) * ((size_t)n + 1));
        for (i = 0; i < n; i++)
            for (k = IA[i]; k < IA[i+1]; k++) JT[w[JA[k]]++] = i;
        free(w);
    }
    /* degrees of the symmetrised pattern (calc_degrees :307-350): every
     * stored entry (i,j) counts for row j of the column-oriented view, and
     * an entry without its mirror also counts for the other end. */
    for (i = 0; i < n; i++)
        for (k = IA[i]; k < IA[i+1]; k++) {
            int r = JA[k];
            D[r]++;
            if (D[r] > max_deg) max_deg = D[r];
            if (r != i) {
                int found = 0;
                for (int l = IA[r]; l < IA[r+1]; l++) {
                    if (JA[l] == i) { found = 1; break; }
                    if (JA[l] > i) break;
                }
                if (!found) { D[i]++; if (D[i] > max_deg) max_deg = D[i]; }
            }
        }
    if (max_deg == 0) {
        for (i = 0; i < n; i++) perm[i] = i;
        free(IT); free(JT); free(D);
        return;
    }
    rcm_node *heap = malloc(sizeof(rcm_node) * ((size_t)max_deg + 1));
    rcm_node *Q = malloc(sizeof(rcm_node) * ((size_t)n + 1));
    rcm_node *Q2 = malloc(sizeof(rcm_node) * ((size_t)n + 1));
    int *seen = malloc(sizeof(int) * ((size_t)n + 1));
    int *visit = calloc((size_t)n + 1, sizeof(int));
    int *nb = malloc(sizeof(int) * (2 * (size_t)max_deg + 2));
    int c = 0, qh = 0, qt = 0;

    while (c < n) {
        for (i = 0; i < n; i++) if (!visit[i]) break;
        rcm_node root = { pseudo_peripheral(n, IA, JA, IT, JT, D, i, Q2, seen, nb), 0, 0 };
        root.deg = D[root.id];
        visit[root.id] = 1;
        Q[qt++] = root;
        while (qh != qt) {
            rcm_node v = Q[qh++];
            int hs = 0;
            perm[c++] = v.id;
            int cnt = neighbours(v.id, IA, JA, IT, JT, nb);
            for (int t = 0; t < cnt; t++) {
                int r = nb[t];
                if (!visit[r]) {
                    rcm_node w = { r, D[r], v.dist + 1 };
                    heap_push(heap, &hs, w);
                    visit[r] = 1;
                }
            }
            while (hs > 0) Q[qt++] = heap_pop(heap, &hs);
        }
    }
    /* reversal (symrcm.c:232-236) */
    for (i = 0; i < n / 2; i++) {
        int t = perm[i]; perm[i] = perm[n - 1 - i]; perm[n - 1 - i] = t;
    }
    free(heap); free(Q); free(Q2); free(seen); free(visit); free(nb);
    free(IT); free(JT); free(D);
}

/* MATRIX_bandwidth (reordering.c:215-236).  The reference's right-band test
 * ends in a stray ';', so the right band is the value of the last row. */
int or_matrix_bandwidth(int n, const int *IA, const int *JA)
{
    int bandl = 0, bandr = 0;
    for (int i = 0; i < n; i++) {
        if (fabs((double)(i - JA[IA[i]])) > bandl) bandl = i - JA[IA[i]];
        bandr = JA[IA[i+1] - 1] - i;
    }
    return bandl > bandr ? bandl : bandr;
}

/* Permutation_of_LM (Permutation_of_LM.c:8-76): adjacency, RCM, bandwidth
 * before and after, and the inverse permutation with the sink fixed. */
int or_permutation_of_lm(int nel, const int *ien, const int *type, const int *invp,
                         int NEQ, int *Perm, int *invPerm, int *bandwidth)
{
    int *IA = malloc(sizeof(int) * ((size_t)NEQ + 1));
    int *JA = malloc(sizeof(int) * ((size_t)nel * 9 + 1));
    int nnz = or_lm_adjacency(nel, ien, type, invp, NEQ, IA, JA);
    int i;
    if (bandwidth) bandwidth[0] = NEQ > 0 ? or_matrix_bandwidth(NEQ, IA, JA) : 0;
    or_symrcm(NEQ, IA, JA, Perm);
    Perm[NEQ] = NEQ;
    for (i = 0; i < NEQ; i++) invPerm[Perm[i]] = i;
    invPerm[NEQ] = NEQ;
    if (bandwidth) {
        /* bandwidth of P A P^T, rows and columns renumbered and sorted */
        int *IB = calloc((size_t)NEQ + 1, sizeof(int));
        int *JB = malloc(sizeof(int) * ((size_t)nnz + 1));
        for (i = 0; i < NEQ; i++) IB[i+1] = IB[i] + (IA[Perm[i]+1] - IA[Perm[i]]);
        for (i = 0; i < NEQ; i++) {
            int o = IB[i];
            for (int k = IA[Perm[i]]; k < IA[Perm[i]+1]; k++) JB[o++] = invPerm[JA[k]];
            qsort(JB + IB[i], (size_t)(IB[i+1] - IB[i]), sizeof(int), cmp_int);
        }
        bandwidth[1] = NEQ > 0 ? or_matrix_bandwidth(NEQ, IB, JB) : 0;
        free(IB); free(JB);
    }
    free(IA); free(JA);
    return nnz;
}
