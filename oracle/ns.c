/*
 * Steady incompressible Navier-Stokes, SUPG/PSPG/LSIC on P1 triangles with
 * equal-order velocity and pressure: CPU restatement of
 * 04_SS_NavierStokes_Equations/2D/01_CommonFiles/Build_K_F_SUPG_PSPG.c:8-669
 * (with eval_U.c:3-35 and ebe_assembly.c) and of the Picard loop of
 * 04_SS_NavierStokes_Equations/2D/01_CommonFiles/Process.c:6-62.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of the GPU library).
 *
 * The element matrix is written per pair of element nodes (i, j) instead of
 * entry by entry; each entry is still the sum of the same terms, added in
 * the same order and with the same association, so the result is
 * bit-identical to the reference compiled without FP contraction.  Rules
 * that keep it so:
 *   - b_i = (y23, y31, y12), c_i = (x32, x13, x21) are the gradient
 *     coefficients of node i;
 *   - the viscous term K and the SUPG/PSPG symmetric terms Ndelta, Gphi
 *     are evaluated with the smaller index first (the reference writes the
 *     upper triangle and reuses it below the diagonal);
 *   - the LSIC term Ks keeps its (row, column) order;
 *   - the density is 1 (Build_K_F_SUPG_PSPG.c:121), so its factors, exact
 *     multiplications by 1, are left out.
 * Only the Picard tangent is built: the Newton branch (:560-648) is taken
 * after 50000 calls of the build (:466) and is never reached.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "femoracle.h"

/* Element geometry, state at the barycentre and stabilisation parameters. */
typedef struct {
    double b[3], c[3];          /* y23 y31 y12 / x32 x13 x21 */
    double Area, invArea, visc;
    double ux, uy, duxdx, duxdy, duydx, duydy, duxduy;
    double p, dpdx, dpdy;
    double C[3];                /* streamline coefficients (u . grad N_i) */
    double tau, tau_l;
} ns_elem;

static void ns_elem_state(ns_elem *g, const double X[3], const double Y[3], const double Ue[9], double Re)
{
    const double third = 1.0 / 3.0;
    double *b = g->b, *c = g->c;
    b[0] = Y[1] - Y[2]; b[1] = Y[2] - Y[0]; b[2] = Y[0] - Y[1];
    c[0] = X[2] - X[1]; c[1] = X[0] - X[2]; c[2] = X[1] - X[0];
    double TwoA = fabs(c[2] * b[1] - c[1] * b[2]);
    g->Area = 0.5 * TwoA;
    g->invArea = 1.0 / g->Area;
    double hi = 0.5 * g->invArea;
    double ux1 = Ue[0], uy1 = Ue[1], p1 = Ue[2];
    double ux2 = Ue[3], uy2 = Ue[4], p2 = Ue[5];
    double ux3 = Ue[6], uy3 = Ue[7], p3 = Ue[8];
    g->ux = third * (ux1 + ux2 + ux3);
    g->uy = third * (uy1 + uy2 + uy3);
    g->duxdx = hi * (ux1 * b[0] + ux2 * b[1] + ux3 * b[2]);
    g->duxdy = hi * (ux1 * c[0] + ux2 * c[1] + ux3 * c[2]);
    g->duydx = hi * (uy1 * b[0] + uy2 * b[1] + uy3 * b[2]);
    g->duydy = hi * (uy1 * c[0] + uy2 * c[1] + uy3 * c[2]);
    g->duxduy = ux1 * b[0] + uy1 * c[0] + ux2 * b[1] + uy2 * c[1] + ux3 * b[2] + uy3 * c[2];
    g->p = third * (p1 + p2 + p3);
    g->dpdx = hi * (p1 * b[0] + p2 * b[1] + p3 * b[2]);
    g->dpdy = hi * (p1 * c[0] + p2 * c[1] + p3 * c[2]);
    for (int i = 0; i < 3; i++) g->C[i] = hi * (g->ux * b[i] + g->uy * c[i]);
    /* tau_SUPG = tau_PSPG (:113-126) and tau_LSIC (:131) */
    double h = sqrt(TwoA);
    g->visc = 1. / Re;
    double nu = g->visc;
    double unorm = sqrt(g->ux * g->ux + g->uy * g->uy);
    double adv = 2.0 * unorm / h, dif = 4.0 * nu / (h * h);
    g->tau = 1.0 / sqrt(adv * adv + 9.0 * dif * dif);
    double lh = 0.5 * h * unorm;
    g->tau_l = sqrt(nu * nu + lh * lh);
}

/* Viscous matrix entry between velocity dofs p <= q (dof 2i+d, d = 0: x). */
static double ns_visc(const ns_elem *g, int p, int q)
{
    int i = p >> 1, j = q >> 1, dp = p & 1, dq = q & 1;
    double s = g->visc * 0.25 * g->invArea;
    const double *b = g->b, *c = g->c;
    if (!dp && !dq) return s * (2 * b[i] * b[j] + c[i] * c[j]);
    if (dp && dq) return s * (b[i] * b[j] + 2 * c[i] * c[j]);
    if (!dp) return s * (c[i] * b[j]);
    return s * (b[i] * c[j]);
}

/* Gradient coefficient of velocity dof p: b for x, c for y. */
static double ns_g(const ns_elem *g, int p) { return (p & 1) ? g->c[p >> 1] : g->b[p >> 1]; }

/* 9x9 Picard tangent (:468-558) and element residual (:412-463). */
static void ns_element(const ns_elem *g, const double fx[3], const double fy[3], double Ke[81], double Res[9])
{
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0;
    const double *b = g->b, *c = g->c, *C = g->C;
    const double A = g->Area, tau = g->tau;
    const double ls = g->tau_l * 0.25 * g->invArea;        /* LSIC scale   */
    const double ps = 0.25 * tau * g->invArea;             /* PSPG Laplace */
    int i, j, di, dj;

    for (i = 0; i < 3; i++)
        for (j = 0; j < 3; j++) {
            int lo = i < j ? i : j, hi = i < j ? j : i;
            double Nj = third * A * C[j];
            double Nd = tau * A * C[lo] * C[hi];
            for (di = 0; di < 2; di++) {
                int p = 2 * i + di, row = 3 * i + di;
                for (dj = 0; dj < 2; dj++) {
                    int q = 2 * j + dj;
                    double k = p <= q ? ns_visc(g, p, q) : ns_visc(g, q, p);
                    double ks = ls * ns_g(g, q) * ns_g(g, p);
                    Ke[row * 9 + 3 * j + dj] = di == dj ? Nj + Nd + k + ks : k + ks;
                }
                /* velocity row, pressure column j: -(G^T + Gdelta) */
                double gd = 0.5 * tau * C[i] * (di ? c[j] : b[j]);
                Ke[row * 9 + 3 * j + 2] = -(sixth * ns_g(g, p) + gd);
            }
            /* pressure row i: G^T + Gdelta against velocity of node j, Gphi */
            for (dj = 0; dj < 2; dj++) {
                int q = 2 * j + dj;
                double gd = 0.5 * tau * C[j] * (dj ? c[i] : b[i]);
                Ke[(3 * i + 2) * 9 + 3 * j + dj] = sixth * ns_g(g, q) + gd;
            }
            Ke[(3 * i + 2) * 9 + 3 * j + 2] = ps * (b[lo] * b[hi] + c[lo] * c[hi]);
        }

    /* source at the barycentre and residual */
    double fxB = third * (fx[0] + fx[1] + fx[2]);
    double fyB = third * (fy[0] + fy[1] + fy[2]);
    double f1 = third * A * fxB, f2 = third * A * fyB;
    double advx = g->duxdx * g->ux + g->duxdy * g->uy;
    double advy = g->duydx * g->ux + g->duydy * g->uy;
    double sym = g->duxdy + g->duydx;
    double GTv = third * A * (g->duxdx + g->duydy);
    for (i = 0; i < 3; i++) {
        double Fx = f1 + tau * A * C[i] * fxB;
        double Fy = f2 + tau * A * C[i] * fyB;
        double Fp = tau * A * (b[i] * fxB + c[i] * fyB);
        double Nvx = third * A * advx, Nvy = third * A * advy;
        double Ndx = tau * A * C[i] * advx, Ndy = tau * A * C[i] * advy;
        double Kvx = 0.5 * g->visc * (2 * b[i] * g->duxdx + c[i] * sym);
        double Kvy = 0.5 * g->visc * (2 * c[i] * g->duydy + b[i] * sym);
        double Ksx = ls * b[i] * g->duxduy, Ksy = ls * c[i] * g->duxduy;
        double Gvx = 0.5 * g->p * b[i], Gvy = 0.5 * g->p * c[i];
        double Gdx = tau * A * C[i] * g->dpdx, Gdy = tau * A * C[i] * g->dpdy;
        double Nphi = 0.5 * tau * (advx * b[i] + advy * c[i]);
        double Gphi = 0.5 * tau * (b[i] * g->dpdx + c[i] * g->dpdy);
        Res[3 * i + 0] = Fx - (Nvx + Ndx + Kvx + Ksx - (Gvx + Gdx));
        Res[3 * i + 1] = Fy - (Nvy + Ndy + Kvy + Ksy - (Gvy + Gdy));
        Res[3 * i + 2] = Fp - (GTv + Nphi + Gphi);
    }
}

void or_build_ns(int nnodes, int nel, const double *x, const double *y, const int *type,
                 const int *invp, const int *ien, int neq, const or_ns_problem *prob,
                 const double *u, double *A, double *F)
{
    int E, v, k, NEQ = neq;
    if (prob->form == 1) {       /* StabilizationForm "VMS-DCDD" (setStabilizationForm.c) */
        or_build_ns_vms(nnodes, nel, x, y, type, invp, ien, neq, prob, u, A, F);
        return;
    }
    double *U = malloc(sizeof(double) * 3 * (size_t)(nnodes ? nnodes : 1));
    /* eval_U.c:3-35: free dofs from u, prescribed ones from the problem */
    for (v = 0; v < nnodes; v++)
        for (k = 0; k < 3; k++) {
            long d = 3L * v + k;
            U[d] = type[d] > 0 ? u[invp[d]] : prob->upresc[d];
        }
    memset(F, 0, sizeof(double) * ((size_t)NEQ + 1));
    for (E = 0; E < nel; E++) {
        double X[3], Y[3], Ue[9], fx[3], fy[3], Res[9];
        int lm[9];
        for (v = 0; v < 3; v++) {
            int J = ien[3 * E + v];
            X[v] = x[J]; Y[v] = y[J];
            fx[v] = prob->f1 ? prob->f1[J] : 0.0;
            fy[v] = prob->f2 ? prob->f2[J] : 0.0;
            for (k = 0; k < 3; k++) {
                long d = 3L * J + k;
                Ue[3 * v + k] = U[d];
                lm[3 * v + k] = type[d] == 0 ? NEQ : invp[d];
            }
        }
        ns_elem g;
        ns_elem_state(&g, X, Y, Ue, prob->reynolds);
        ns_element(&g, fx, fy, A + 81L * E, Res);
        /* F[lm] += Res, sink reset after every element (:652-656) */
        for (k = 0; k < 9; k++) F[lm[k]] += Res[k];
        F[NEQ] = 0;
    }
    free(U);
}

/* ---- Picard loop (Process.c:6-62) with EBE 9x9 and BlockDiagDOF3 ---- */
typedef struct {
    int nel, nnodes, NEQ;
    const int *lm, *Id;
    const double *A, *inv;
} ns_ctx;

static int ns_mv_cb(void *p, double *P, double *Q)
{
    ns_ctx *c = (ns_ctx *)p;
    or_ebemv(c->nel, 9, c->lm, c->A, c->NEQ, P, Q);
    return 0;
}

static int ns_pc_cb(void *p, double *x, double *z)
{
    ns_ctx *c = (ns_ctx *)p;
    or_blockdiag_apply(c->nnodes, 3, c->Id, c->NEQ, c->inv, x, z);
    return 0;
}

int or_ns_process(int nnodes, int nel, const double *x, const double *y, const int *type,
                  const int *invp, const int *ien, int neq, const or_ns_problem *prob,
                  double solver_tol, double nonlinear_tol, int kmax, int lmax, int max_nonlinear,
                  double *u, int *gmres_iterations, double *last_delta)
{
    int NEQ = neq, it = 0, i;
    int *lm = malloc(sizeof(int) * 9 * (size_t)(nel ? nel : 1));
    int *Id = malloc(sizeof(int) * 3 * (size_t)(nnodes ? nnodes : 1));
    double *A = malloc(sizeof(double) * 81 * (size_t)(nel ? nel : 1));
    double *F = calloc((size_t)NEQ + 1, sizeof(double));
    double *s = calloc((size_t)NEQ + 1, sizeof(double));
    double *bd = malloc(sizeof(double) * 9 * (size_t)(nnodes ? nnodes : 1));
    double *inv = malloc(sizeof(double) * 9 * (size_t)(nnodes ? nnodes : 1));
    double delta2 = nonlinear_tol + 1.0;
    or_fill_lm(nel, 3, ien, type, invp, NEQ, lm);
    for (i = 0; i < 3 * nnodes; i++) Id[i] = type[i] == 0 ? NEQ : invp[i];
    ns_ctx c = { nel, nnodes, NEQ, lm, Id, A, inv };
    if (gmres_iterations) *gmres_iterations = 0;
    while (delta2 > nonlinear_tol && it < max_nonlinear) {
        int gi = 0;
        it++;
        or_build_ns(nnodes, nel, x, y, type, invp, ien, neq, prob, u, A, F);
        or_blockdiag_setup(nnodes, nel, 3, ien, A, Id, NEQ, 1, bd, inv, F);
        or_pgmres(NEQ, kmax, lmax, solver_tol, ns_mv_cb, ns_pc_cb, &c, F, s, &gi);
        if (gmres_iterations) *gmres_iterations += gi;
        for (i = 0; i < neq; i++) u[i] += 1 * s[i];
        double norms = sqrt(or_ddot(neq, s, s));
        double normu = sqrt(or_ddot(neq, u, u));
        delta2 = norms / normu;
    }
    if (last_delta) *last_delta = delta2;
    free(lm); free(Id); free(A); free(F); free(s); free(bd); free(inv);
    return it;
}
