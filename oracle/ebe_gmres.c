/*
 * femoracle: EBE matvecs, Diag / nodal block-diagonal preconditioners and
 * restarted GMRES.  TEST INFRASTRUCTURE ONLY (see femoracle.h).
 */
#include "femoracle.h"
#include <stdlib.h>
#include <string.h>
#include <math.h>

/* ddot with the reference's 5-way unrolled summation order
 * (00_CommonFiles/BLAS_Operations/ddot.c:4-21; the Allreduce of one rank is
 * the identity). */
double or_ddot(int n, const double *x, const double *y)
{
    long i, m = n - 4;
    double s = 0.0;
    for (i = 0; i < m; i += 5)
        s += x[i]*y[i] + x[i+1]*y[i+1] + x[i+2]*y[i+2] + x[i+3]*y[i+3] + x[i+4]*y[i+4];
    for (; i < n; i++) s += x[i]*y[i];
    return s;
}

/* ebemv (00_CommonFiles/MatrixVector_Operations/EBE/ebemv.c:4-64): the
 * vector is permuted (Pa[I] = P[Perm[I]]), each 3x3 block gathers through
 * invPerm[lm], the products are scattered in element order, and the result
 * is permuted back.  The sink Qa[NEQ] is reset after every element. */
void or_ebemv3_perm(int nel, const int *lm, const double *A, const int *Perm,
                    const int *invPerm, int NEQ, const double *P, double *Q)
{
    double *Pa = calloc((size_t)NEQ + 1, sizeof(double));
    double *Qa = calloc((size_t)NEQ + 1, sizeof(double));
    int I;
    for (I = 0; I < NEQ; I++) Pa[I] = P[Perm[I]];
    for (I = 0; I < nel; I++) {
        const double *a = A + 9L * I;
        int i1 = invPerm[lm[3*I]], i2 = invPerm[lm[3*I+1]], i3 = invPerm[lm[3*I+2]];
        double p1 = Pa[i1], p2 = Pa[i2], p3 = Pa[i3];
        Qa[i1] += a[0]*p1 + a[1]*p2 + a[2]*p3;
        Qa[i2] += a[3]*p1 + a[4]*p2 + a[5]*p3;
        Qa[i3] += a[6]*p1 + a[7]*p2 + a[8]*p3;
        Qa[NEQ] = 0;
    }
    for (I = 0; I < NEQ; I++) Q[Perm[I]] = Qa[I];
    free(Pa);
    free(Qa);
}

/* ebemvNDOF3 / ebemvNDOF4 (EBE/ebemvNDOF3.c:3-92, EBE/ebemvNDOF4.c:4-121):
 * Q = 0, P[NEQ] = 0, then per element row r: Q[lm_r] += sum_c A[r][c] P[lm_c]
 * with the row sum taken left to right, and the sink reset per element. */
void or_ebemv(int nel, int S, const int *lm, const double *A, int NEQ,
              const double *P, double *Q)
{
    double p[12];
    int I, r, c;
    for (I = 0; I <= NEQ; I++) Q[I] = 0;
    for (I = 0; I < nel; I++) {
        const int *l = lm + (long)S * I;
        const double *a = A + (long)S * S * I;
        for (c = 0; c < S; c++) p[c] = l[c] == NEQ ? 0.0 : P[l[c]];
        for (r = 0; r < S; r++) {
            double s = a[r*S] * p[0];
            for (c = 1; c < S; c++) s += a[r*S + c] * p[c];
            Q[l[r]] += s;
        }
        Q[NEQ] = 0.0;
    }
}

/* Diag_precond_EBE_setup (EBE/Diag_precond_EBE_setup.c:3-32).  Diag is
 * never cleared, as in the reference, so a second setup on the same arrays
 * adds the new diagonal to the old one. */
void or_diag_setup(int nel, int S, const int *lm, const double *A, int NEQ,
                   double *Diag, double *invDiag, double *F)
{
    int E, I;
    for (E = 0; E < nel; E++) {
        for (I = 0; I < S; I++) Diag[lm[(long)S*E + I]] += A[(long)S*S*E + I*(S+1)];
        Diag[NEQ] = 0;
    }
    for (I = 0; I < NEQ; I++) invDiag[I] = 1.0 / Diag[I];
    for (I = 0; I < NEQ; I++) F[I] *= invDiag[I];
}

/* Left_scaling_EBE (Solvers_and_Preconditioners/scaling.c:10-42): the
 * accumulating Diag set-up on F, invDiag[NEQ] = invDiag[NEQ-1] (the
 * value the last rank broadcasts for the sink), then every block row
 * times invDiag of its equation.  One rank. */
void or_scale_left(int nel, int S, const int *lm, double *A, int NEQ, double *Diag, double *invDiag, double *F)
{
    int E, I, J;
    or_diag_setup(nel, S, lm, A, NEQ, Diag, invDiag, F);
    invDiag[NEQ] = invDiag[NEQ - 1];
    for (E = 0; E < nel; E++)
        for (I = 0; I < S; I++)
            for (J = 0; J < S; J++) A[(long)S*S*E + S*I + J] *= invDiag[lm[(long)S*E + I]];
}

/* LeftRight_scaling_EBE (scaling.c:92-121): A_IJ *= sqrt(invDiag_I
 * invDiag_J), F = (F / d) * sqrt(d); the solution is unscaled by
 * Left_unscaling (scaling.c:187-196): x *= sqrt(invDiag). */
void or_scale_leftright(int nel, int S, const int *lm, double *A, int NEQ, double *Diag, double *invDiag, double *F)
{
    int E, I, J;
    or_diag_setup(nel, S, lm, A, NEQ, Diag, invDiag, F);
    invDiag[NEQ] = invDiag[NEQ - 1];
    for (E = 0; E < nel; E++)
        for (I = 0; I < S; I++)
            for (J = 0; J < S; J++)
                A[(long)S*S*E + S*I + J] *= sqrt(invDiag[lm[(long)S*E + I]] * invDiag[lm[(long)S*E + J]]);
    for (I = 0; I < NEQ; I++) F[I] *= sqrt(Diag[I]);
}

void or_unscale(int NEQ, const double *invDiag, double *x)
{
    for (int I = 0; I < NEQ; I++) x[I] *= sqrt(invDiag[I]);
}

/* Diag_precond (Solvers_and_Preconditioners/Diag_precond.c:3-15). */
void or_diag_apply(int n, const double *invDiag, const double *p, double *z)
{
    for (int I = 0; I < n; I++) z[I] = p[I] * invDiag[I];
}

/* Closed-form 4x4 inverse by cofactors (EBE/BlockDiag_precond_EBE_setup.c:90-147).
 * The reference's entry 14 multiplies c*j*m where the cofactor has c*f*m;
 * ref_quirks keeps that term so the preconditioner matches the reference. */
static void inv4(const double *B, double *R, int ref_quirks)
{
    double a=B[0],b=B[1],c=B[2],d=B[3],e=B[4],f=B[5],g=B[6],h=B[7];
    double i=B[8],j=B[9],k=B[10],l=B[11],m=B[12],n=B[13],o=B[14],p=B[15];
    double det = (a*f*k*p - a*f*l*o - a*g*j*p + a*g*l*n + a*h*j*o - a*h*k*n
                 -b*e*k*p + b*e*l*o + b*g*i*p - b*g*l*m - b*h*i*o + b*h*k*m +
                 c*(e*j*p - e*l*n - f*i*p + f*l*m + h*i*n - h*j*m) +
                 d*(-e*j*o + e*k*n + f*i*o - f*k*m - g*i*n + g*j*m));
    double q = 1.0 / det;
    R[0]  = q*(-h*k*n + g*l*n + h*j*o - f*l*o - g*j*p + f*k*p);
    R[1]  = q*(d*k*n - c*l*n - d*j*o + b*l*o + c*j*p - b*k*p);
    R[2]  = q*(-d*g*n + c*h*n + d*f*o - b*h*o - c*f*p + b*g*p);
    R[3]  = q*(d*g*j - c*h*j - d*f*k + b*h*k + c*f*l - b*g*l);
    R[4]  = q*(h*k*m - g*l*m - h*i*o + e*l*o + g*i*p - e*k*p);
    R[5]  = q*(-d*k*m + c*l*m + d*i*o - a*l*o - c*i*p + a*k*p);
    R[6]  = q*(d*g*m - c*h*m - d*e*o + a*h*o + c*e*p - a*g*p);
    R[7]  = q*(-d*g*i + c*h*i + d*e*k - a*h*k - c*e*l + a*g*l);
    R[8]  = q*(-h*j*m + f*l*m + h*i*n - e*l*n - f*i*p + e*j*p);
    R[9]  = q*(d*j*m - b*l*m - d*i*n + a*l*n + b*i*p - a*j*p);
    R[10] = q*(-d*f*m + b*h*m + d*e*n - a*h*n - b*e*p + a*f*p);
    R[11] = q*(d*f*i - b*h*i - d*e*j + a*h*j + b*e*l - a*f*l);
    R[12] = q*(g*j*m - f*k*m - g*i*n + e*k*n + f*i*o - e*j*o);
    R[13] = q*(-c*j*m + b*k*m + c*i*n - a*k*n - b*i*o + a*j*o);
    R[14] = q*((ref_quirks ? c*j*m : c*f*m) - b*g*m - c*e*n + a*g*n + b*e*o - a*f*o);
    R[15] = q*(-c*f*i + b*g*i + c*e*j - a*g*j - b*e*k + a*f*k);
}

/* Closed-form 3x3 inverse (EBE/BlockDiagDOF3_precond_EBE_setup.c:84-124). */
static void inv3(const double *B, double *R)
{
    double a=B[0],b=B[1],c=B[2],d=B[3],e=B[4],f=B[5],g=B[6],h=B[7],i=B[8];
    double det = a*e*i - a*f*h - b*d*i + b*f*g + c*d*h - c*e*g;
    double q = 1.0 / det;
    R[0] = q*(e*i - f*h);
    R[1] = q*(c*h - b*i);
    R[2] = q*(b*f - c*e);
    R[3] = q*(f*g - d*i);
    R[4] = q*(a*i - c*g);
    R[5] = q*(c*d - a*f);
    R[6] = q*(d*h - e*g);
    R[7] = q*(b*g - a*h);
    R[8] = q*(a*e - b*d);
}

void or_blockdiag_apply(int nnodes, int B, const int *Id, int NEQ,
                        const double *inv, double *p, double *z)
{
    double v[4];
    int I, r, c;
    p[NEQ] = 0;
    for (I = 0; I < nnodes; I++) {
        const int *id = Id + (long)B * I;
        const double *m = inv + (long)B * B * I;
        for (c = 0; c < B; c++) v[c] = p[id[c]];
        for (r = 0; r < B; r++) {
            double s = m[r*B] * v[0];
            for (c = 1; c < B; c++) s += m[r*B + c] * v[c];
            z[id[r]] = s;
        }
        z[NEQ] = 0.;
    }
}

void or_blockdiag_setup(int nnodes, int nel, int B, const int *ien, const double *A,
                        const int *Id, int NEQ, int ref_quirks,
                        double *BlockDiag, double *invBlockDiag, double *F)
{
    int S = 3 * B, E, v, r, c, I;
    memset(BlockDiag, 0, sizeof(double) * (size_t)B * B * nnodes);
    for (E = 0; E < nel; E++)
        for (v = 0; v < 3; v++) {
            double *bd = BlockDiag + (long)B * B * ien[3*E + v];
            const double *a = A + (long)S * S * E;
            for (r = 0; r < B; r++)
                for (c = 0; c < B; c++)
                    bd[r*B + c] += a[(B*v + r) * S + B*v + c];
        }
    for (I = 0; I < nnodes; I++) {
        if (B == 4) inv4(BlockDiag + 16L*I, invBlockDiag + 16L*I, ref_quirks);
        else inv3(BlockDiag + 9L*I, invBlockDiag + 9L*I);
    }
    or_blockdiag_apply(nnodes, B, Id, NEQ, invBlockDiag, F, F);
}

/* ---------------------------------------------------------------------
 * Restarted left-preconditioned GMRES(kmax), restating
 * 00_CommonFiles/Solvers_and_Preconditioners/pgmres.c:5-200 for one rank:
 * X0 = 0, eps = tol*||B|| (B is already preconditioned by the setup),
 * modified Gram-Schmidt, Givens rotations, at most kmax-1 Arnoldi steps per
 * cycle, restart while rho > eps and fewer than lmax cycles.  precondR is
 * NO_precond in every configuration of the reference's EBE drivers, so it
 * is omitted.  Returns 0; *iterations += Arnoldi steps taken.
 * ------------------------------------------------------------------- */
static int or_pgmres_lr(int NEQ, int kmax, int lmax, double tol, or_mv_fn mv, or_pc_fn precond, or_pc_fn precondR,
                        void *ctx, double *B, double *X, int *iterations);

int or_pgmres(int NEQ, int kmax, int lmax, double tol,
              or_mv_fn mv, or_pc_fn precond, void *ctx,
              double *B, double *X, int *iterations)
{
    return or_pgmres_lr(NEQ, kmax, lmax, tol, mv, precond, NULL, ctx, B, X, iterations);
}

/* pgmres.c:5-200 with the right preconditioner precondR applied in place
 * to v before every matvec (:61, :93) and to X at the end (:186); NULL is
 * NO_precond. */
static int or_pgmres_lr(int NEQ, int kmax, int lmax, double tol, or_mv_fn mv, or_pc_fn precond, or_pc_fn precondR,
                        void *ctx, double *B, double *X, int *iterations)
{
    int n = NEQ, i, j, k, l = 0, cont = 0;
    double *ubuf = calloc((size_t)kmax * (n + 1), sizeof(double));
    double *h = calloc((size_t)kmax * kmax, sizeof(double));
    double *e = calloc((size_t)kmax, sizeof(double));
    double *c = calloc((size_t)kmax, sizeof(double));
    double *s = calloc((size_t)kmax, sizeof(double));
    double *y = calloc((size_t)kmax, sizeof(double));
    double *v = calloc((size_t)n + 1, sizeof(double));
    double normb, eps, rho, r;
#define U(j) (ubuf + (long)(j) * (n + 1))
#define H(a, b) h[(long)(a) * kmax + (b)]
    for (k = 0; k < n; k++) X[k] = 0.0;
    normb = sqrt(or_ddot(n, B, B));
    eps = tol * normb;
    do {
        i = 0;
        for (j = 0; j < kmax; j++) memset(U(j), 0, sizeof(double) * n);
        memcpy(v, X, sizeof(double) * n);
        if (precondR) precondR(ctx, v, v);
        mv(ctx, v, U(0));
        precond(ctx, U(0), U(0));
        for (k = 0; k < n; k++) U(0)[k] += -1.0 * B[k];
        for (k = 0; k < n; k++) U(0)[k] = -1.0 * U(0)[k];
        e[0] = sqrt(or_ddot(n, U(0), U(0)));
        for (k = 0; k < n; k++) U(0)[k] = (1.0 / e[0]) * U(0)[k];
        rho = e[0];
        do {
            cont++;
            memcpy(v, U(i), sizeof(double) * n);
            if (precondR) precondR(ctx, v, v);
            mv(ctx, v, U(i+1));
            precond(ctx, U(i+1), U(i+1));
            for (j = 0; j <= i; j++) {
                H(j, i) = or_ddot(n, U(j), U(i+1));
                double a = -H(j, i);
                for (k = 0; k < n; k++) U(i+1)[k] += a * U(j)[k];
            }
            H(i+1, i) = sqrt(or_ddot(n, U(i+1), U(i+1)));
            {
                double sc = 1.0 / H(i+1, i);
                for (k = 0; k < n; k++) U(i+1)[k] = sc * U(i+1)[k];
            }
            for (j = 0; j <= i - 1; j++) {
                double h1 =  c[j]*H(j, i) + s[j]*H(j+1, i);
                double h2 = -s[j]*H(j, i) + c[j]*H(j+1, i);
                H(j, i) = h1;
                H(j+1, i) = h2;
            }
            r = sqrt(pow(H(i, i), 2) + pow(H(i+1, i), 2));
            c[i] = H(i, i) / r;
            s[i] = H(i+1, i) / r;
            H(i, i) = r;
            H(i+1, i) = 0.0;
            e[i+1] = -s[i]*e[i];
            e[i] = c[i]*e[i];
            rho = fabs(e[i+1]);
            i++;
        } while (rho > eps && i < kmax - 1);
        i--;
        y[i] = e[i] / H(i, i);
        for (j = i - 1; j >= 0; j--) {
            double sum = 0.0;
            for (k = j + 1; k <= i; k++) sum = sum + H(j, k) * y[k];
            y[j] = (e[j] - sum) / H(j, j);
        }
        for (j = 0; j <= i; j++)
            for (k = 0; k < n; k++) X[k] = X[k] + U(j)[k] * y[j];
        l++;
    } while (rho > eps && l < lmax);
#undef U
#undef H
    if (precondR) precondR(ctx, X, X);
    if (iterations) *iterations += cont;
    free(ubuf); free(h); free(e); free(c); free(s); free(y); free(v);
    return 0;
}

/* ---- EBE + Diag solve helper ---- */
typedef struct {
    int nel, S, NEQ;
    const int *lm, *Perm, *invPerm;
    const double *A, *invDiag;
} ebe_ctx;

static int ebe_mv_cb(void *p, double *P, double *Q)
{
    ebe_ctx *c = (ebe_ctx *)p;
    if (c->Perm) or_ebemv3_perm(c->nel, c->lm, c->A, c->Perm, c->invPerm, c->NEQ, P, Q);
    else or_ebemv(c->nel, c->S, c->lm, c->A, c->NEQ, P, Q);
    return 0;
}

static int diag_pc_cb(void *p, double *x, double *z)
{
    ebe_ctx *c = (ebe_ctx *)p;
    or_diag_apply(c->NEQ, c->invDiag, x, z);
    return 0;
}

int or_ebe_diag_solve(int nel, int S, const int *lm, const double *A, int NEQ,
                      const int *Perm, const int *invPerm,
                      double *Diag, double *invDiag, double *F,
                      int kmax, int lmax, double tol, double *X)
{
    ebe_ctx c = { nel, S, NEQ, lm, Perm, invPerm, A, invDiag };
    int it = 0;
    or_diag_setup(nel, S, lm, A, NEQ, Diag, invDiag, F);
    or_pgmres(NEQ, kmax, lmax, tol, ebe_mv_cb, diag_pc_cb, &c, F, X, &it);
    return it;
}

/* ---- EBE + nodal block-diagonal solve helper (NS / Euler drivers) ---- */
typedef struct {
    int nel, S, NEQ, nnodes, B;
    const int *lm, *Id;
    const double *A, *inv;
} blk_ctx;

static int blk_mv_cb(void *p, double *P, double *Q)
{
    blk_ctx *c = (blk_ctx *)p;
    or_ebemv(c->nel, c->S, c->lm, c->A, c->NEQ, P, Q);
    return 0;
}

static int blk_pc_cb(void *p, double *x, double *z)
{
    blk_ctx *c = (blk_ctx *)p;
    or_blockdiag_apply(c->nnodes, c->B, c->Id, c->NEQ, c->inv, x, z);
    return 0;
}

int or_ebe_block_solve(int nnodes, int nel, int B, const int *ien, const int *lm, const double *A,
                       const int *Id, int NEQ, int ref_quirks, double *F, int kmax, int lmax,
                       double tol, double *X)
{
    double *bd = malloc(sizeof(double) * (size_t)B * B * (nnodes ? nnodes : 1));
    double *inv = malloc(sizeof(double) * (size_t)B * B * (nnodes ? nnodes : 1));
    blk_ctx c = { nel, 3 * B, NEQ, nnodes, B, lm, Id, A, inv };
    int it = 0;
    or_blockdiag_setup(nnodes, nel, B, ien, A, Id, NEQ, ref_quirks, bd, inv, F);
    or_pgmres(NEQ, kmax, lmax, tol, blk_mv_cb, blk_pc_cb, &c, F, X, &it);
    free(bd); free(inv);
    return it;
}


/* Block_scaling_EBE (Block_scaling.c:10-118), after the block-diagonal
 * set-up has given inv (B*B per node, row-major): in every element block,
 * the row and the column of each Dirichlet dof are cleared and its diagonal
 * entry set to 1 (matrix_Bondary_Conditions), then every row block of node
 * v is multiplied by inv[v] (matrix_Scaling, sums from 0 in j order). */
void or_block_scale(int nel, int B, const int *ien, const int *Id, int NEQ, const double *inv, double *A)
{
    const int S = 3 * B;
    double *m = malloc(sizeof(double) * (size_t)S * S);
    for (int e = 0; e < nel; e++) {
        double *Ae = A + (size_t)S * S * e;
        memcpy(m, Ae, sizeof(double) * (size_t)S * S);
        for (int I = 0; I < B; I++)
            for (int v = 0; v < 3; v++) {
                if (Id[B * ien[3 * e + v] + I] != NEQ) continue;
                const int d = B * v + I;
                for (int t = 0; t < S; t++) { m[d * S + t] = 0; m[t * S + d] = 0; }
                m[d * S + d] = 1;
            }
        for (int v = 0; v < 3; v++) {
            const double *iv = inv + (size_t)B * B * ien[3 * e + v];
            for (int i = 0; i < B; i++)
                for (int col = 0; col < S; col++) {
                    double a = 0;
                    for (int j = 0; j < B; j++) a += iv[i * B + j] * m[(B * v + j) * S + col];
                    Ae[(B * v + i) * S + col] = a;
                }
        }
    }
    free(m);
}

/* ---- element preconditioners of the EBE scheme (Preconditioner "LUe",
 * "SGSe"; 3x3 blocks).  Both sweep the elements in order, in place on z
 * (z[NEQ] is the sink, kept 0), each element reading the values the
 * earlier ones wrote.  The expressions keep the reference's association:
 * `a += -b*c - d*e` adds ((-(b*c)) - d*e) to a. ---- */

/* LU_precond_EBE_setup.c:20-31: per element, the LU factors of its block
 * with unit diagonal taken as 1 (A row-major, 9 per element). */
void or_lue_setup(int nel, const double *A, double *LUe)
{
    for (int I = 0; I < nel; I++) {
        const double *a = A + 9 * (long)I;
        double *L = LUe + 9 * (long)I;
        L[0] = 1.0;
        L[1] = a[1];
        L[2] = a[2];
        L[3] = a[3];
        L[4] = 1. / (1.0 - a[1] * a[3]);
        L[5] = a[5] - a[2] * a[3];
        L[6] = a[6];
        L[7] = (a[7] - a[1] * a[6]) * L[4];
        L[8] = 1. / (1.0 - a[2] * a[6] - L[7] * L[5]);
    }
}

/* LU_precond_EBE.c:28-60: L then U of each element, in element order. */
void or_lue_apply(int nel, const int *lm, int NEQ, const double *LUe, double *z)
{
    z[NEQ] = 0;
    for (int I = 0; I < nel; I++) {
        const int l0 = lm[3 * I], l1 = lm[3 * I + 1], l2 = lm[3 * I + 2];
        const double *L = LUe + 9 * (long)I;
        double z0 = z[l0], z1 = z[l1], z2 = z[l2];
        z1 += -L[3] * z0;
        z2 += -L[6] * z0 - L[7] * z1;
        z2 *= L[8];
        z1 = (z1 - L[5] * z2) * L[4];
        z0 += -L[1] * z1 - L[2] * z2;
        z[l0] = z0;
        z[l1] = z1;
        z[l2] = z2;
        z[NEQ] = 0;
    }
}

/* SGS_precond_EBE.c:4-40: the forward (lower) sweep, element order. */
void or_sgs_fwd(int nel, const int *lm, int NEQ, const double *A, double *z)
{
    z[NEQ] = 0;
    for (int I = 0; I < nel; I++) {
        const int l0 = lm[3 * I], l1 = lm[3 * I + 1], l2 = lm[3 * I + 2];
        const double *a = A + 9 * (long)I;
        double z0 = z[l0], z1 = z[l1], z2 = z[l2];
        z1 += -a[3] * z0;
        z2 += -a[6] * z0 - a[7] * z1;
        z[l1] = z1;
        z[l2] = z2;
        z[NEQ] = 0.0;
    }
}

/* SGS_precond_EBE.c:42-76 (SGS_precondR_EBE): the backward (upper) sweep,
 * elements in reverse order. */
void or_sgs_bwd(int nel, const int *lm, int NEQ, const double *A, double *z)
{
    z[NEQ] = 0;
    for (int I = nel - 1; I >= 0; I--) {
        const int l0 = lm[3 * I], l1 = lm[3 * I + 1], l2 = lm[3 * I + 2];
        const double *a = A + 9 * (long)I;
        double z0 = z[l0], z1 = z[l1], z2 = z[l2];
        z1 += -a[5] * z2;
        z0 += -a[1] * z1 - a[2] * z2;
        z[l0] = z0;
        z[l1] = z1;
        z[NEQ] = 0.0;
    }
}

typedef struct {
    ebe_ctx e;
    const double *LUe;
} elem_ctx;

static int lue_pc_cb(void *p, double *x, double *z)
{
    elem_ctx *c = (elem_ctx *)p;
    if (z != x) memcpy(z, x, sizeof(double) * (c->e.NEQ + 1));
    or_lue_apply(c->e.nel, c->e.lm, c->e.NEQ, c->LUe, z);
    return 0;
}
static int sgs_fwd_cb(void *p, double *x, double *z)
{
    elem_ctx *c = (elem_ctx *)p;
    if (z != x) memcpy(z, x, sizeof(double) * (c->e.NEQ + 1));
    or_sgs_fwd(c->e.nel, c->e.lm, c->e.NEQ, c->e.A, z);
    return 0;
}
static int sgs_bwd_cb(void *p, double *x, double *z)
{
    elem_ctx *c = (elem_ctx *)p;
    if (z != x) memcpy(z, x, sizeof(double) * (c->e.NEQ + 1));
    or_sgs_bwd(c->e.nel, c->e.lm, c->e.NEQ, c->e.A, z);
    return 0;
}

/* The element preconditioners' set-up (F <- M^-1 F) and pgmres, as
 * Process.c:59-76 sequences them: kind 1 LUe (precond LU_precond_EBE,
 * precondR NO_precond), kind 2 SGSe (precond SGS_precond_EBE, precondR
 * SGS_precondR_EBE).  mv is ebemv (with the local RCM when Perm is given).
 * Returns the GMRES iterations; F is preconditioned in place. */
int or_ebe_elem_solve(int kind, int nel, const int *lm, const double *A, int NEQ, const int *Perm,
                      const int *invPerm, double *F, int kmax, int lmax, double tol, double *X)
{
    double *LUe = kind == 1 ? calloc((size_t)9 * nel, sizeof(double)) : NULL;
    elem_ctx c = { { nel, 3, NEQ, lm, Perm, invPerm, A, NULL }, LUe };
    int it = 0;
    if (kind == 1) {
        or_lue_setup(nel, A, LUe);
        or_lue_apply(nel, lm, NEQ, LUe, F);
        or_pgmres_lr(NEQ, kmax, lmax, tol, ebe_mv_cb, lue_pc_cb, NULL, &c, F, X, &it);
    } else {
        or_sgs_fwd(nel, lm, NEQ, A, F);
        or_pgmres_lr(NEQ, kmax, lmax, tol, ebe_mv_cb, sgs_fwd_cb, sgs_bwd_cb, &c, F, X, &it);
    }
    free(LUe);
    return it;
}
