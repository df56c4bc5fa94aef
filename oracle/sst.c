/*
 * femoracle: steady SUPG/CAU convection-diffusion-reaction on P1 triangles.
 * TEST INFRASTRUCTURE ONLY (see femoracle.h).
 *
 * Restates 01_SS_Transport_Equation/2D/01_CommonFiles/Build_K_F_SUPG.c with
 * CAU_ShockCapture.c, h_shock_2sqrtArea.c, F_assembly.c, ebe_assembly.c and
 * the Process.c fixed-point loop, and (form 1, StabilizationForm "DD")
 * Build_K_F_DD.c:4-178 with CAU_DD_ShockCapture.c:3-22.  The element
 * formulas are those of the reference, term for term, so that the element
 * blocks agree to the last bit when both are compiled without
 * floating-point contraction.
 */
#include "femoracle.h"
#include <stdlib.h>
#include <string.h>
#include <math.h>

/* CAU_ShockCapture (CAU_ShockCapture.c:3-31). */
static double cau(double kx, double ky, double bx, double by, double gamma,
                  double ue1, double ue2, double ue3, double ueb, double feb,
                  double y23, double y31, double y12, double x32, double x13, double x21,
                  double invArea, double h)
{
    double third = 1. / 3.;
    double bgu = 0.5*invArea*(ue1*(bx*y23 + by*x32) + ue2*(bx*y31 + by*x13) + ue3*(bx*y12 + by*x21));
    double Ru = bgu + gamma*ueb - feb;
    double gx = 0.5*invArea*(y23*ue1 + y31*ue2 + y12*ue3);
    double gy = 0.5*invArea*(x32*ue1 + x13*ue2 + x21*ue3);
    double ng = sqrt(gx*gx + gy*gy);
    double bxp = bgu*gx/(ng*ng);
    double byp = bgu*gy/(ng*ng);
    double kp = bxp*bxp*kx + byp*byp*ky;
    double nbp = sqrt(bxp*bxp + byp*byp);
    double Pe = 0.5*h*nbp*nbp*nbp/kp;
    if (ng > 0) {
        if (third*Pe < 0.7) return 0.5*h*third*Pe*fabs(Ru)/ng;
        return 0.5*h*0.7*fabs(Ru)/ng;
    }
    return 0;
}

/* YZBeta_ShockCapture (YZBeta_ShockCapture.c:3-36): YZ-beta with beta = 1
 * and 2, relaxed against the element's previous value (w = 1/2, or 0 when
 * |R(u)| moved by less than 20%); Re_old / delta_old carry the state. */
static double yzbeta(double *Re_old, double *delta_old, int e, double bx, double by, double gamma,
                     double ue1, double ue2, double ue3, double ueb, double feb, double y23, double y31, double y12,
                     double x32, double x13, double x21, double invArea, double h)
{
    double w = 0.5, Eu;
    double bgu = 0.5*invArea*(ue1*(bx*y23 + by*x32) + ue2*(bx*y31 + by*x13) + ue3*(bx*y12 + by*x21));
    double Ru = bgu + gamma*ueb - feb;
    double nRu = fabs(Ru);
    double gx = 0.5*invArea*(y23*ue1 + y31*ue2 + y12*ue3);
    double gy = 0.5*invArea*(x32*ue1 + x13*ue2 + x21*ue3);
    double ng = sqrt(gx*gx + gy*gy);
    double nu = fabs(ueb);
    if (nu >= 1e-12 && ng >= 1e-12) Eu = 0.25*h*nRu/ng + 0.125*h*h*nRu/nu;
    else Eu = 0;
    if (fabs(nRu - Re_old[e])/nRu < 0.2) w = 0.;
    Eu = w*Eu + (1.0 - w)*delta_old[e];
    Re_old[e] = nRu;
    delta_old[e] = Eu;
    return Eu;
}

/* h_shock_calculation: 2sqrtArea (0, h_shock_2sqrtArea.c), Option1 (1,
 * h_shock_Option1.c:3-19, from grad u) or Option2 (2, h_shock_Option2.c:3-16,
 * from the velocity). */
double or_h_shock(int opt, double bx, double by, double u1, double u2, double u3, double y23, double y31,
                  double y12, double x32, double x13, double x21, double Area)
{
    if (opt == 1) {
        double P1 = fabs(u1*y23*y23 + u2*y31*y23 + u3*y12*y23 + u1*x32*x32 + u2*x13*x32 + u3*x21*x32);
        double P2 = fabs(u1*y23*y31 + u2*y31*y31 + u3*y12*y31 + u1*x32*x13 + u2*x13*x13 + u3*x21*x13);
        double P3 = fabs(u1*y23*y12 + u2*y31*y12 + u3*y12*y12 + u1*x32*x21 + u2*x13*x21 + u3*x21*x21);
        double a1 = y23*u1 + y31*u2 + y12*u3, a2 = x32*u1 + x13*u2 + x21*u3;
        double ng = sqrt(a1*a1 + a2*a2);
        return P1 + P2 + P3 >= 1e-12 ? 4*Area*ng/(P1 + P2 + P3) : 0;
    }
    if (opt == 2) {
        double P1 = fabs(bx*y23 + by*x32), P2 = fabs(bx*y31 + by*x13), P3 = fabs(bx*y12 + by*x21);
        double nb = sqrt(bx*bx + by*by);
        return P1 + P2 + P3 >= 1e-12 ? 4*Area*nb/(P1 + P2 + P3) : 0;
    }
    return sqrt(fabs(2*Area));
}

/* CAU_DD_ShockCapture (CAU_DD_ShockCapture.c:3-22): 0.5 h |R(u)| / |grad u|. */
static double cau_dd(double bx, double by, double gamma, double ue1, double ue2, double ue3, double ueb,
                     double feb, double y23, double y31, double y12, double x32, double x13, double x21,
                     double invArea, double h)
{
    double bgu = 0.5*invArea*(ue1*(bx*y23 + by*x32) + ue2*(bx*y31 + by*x13) + ue3*(bx*y12 + by*x21));
    double Ru = bgu + gamma*ueb - feb;
    double gx = 0.5*invArea*(y23*ue1 + y31*ue2 + y12*ue3);
    double gy = 0.5*invArea*(x32*ue1 + x13*ue2 + x21*ue3);
    double ng = sqrt(gx*gx + gy*gy);
    return ng > 1e-10 ? 0.5*h*fabs(Ru)/ng : 0;
}

/* Build_K_F_DD.c:54-164: Galerkin + dynamic diffusion with the bubble
 * (KBB, KhB, KBh, FB) condensed into the 3x3 block and the load. */
static void dd_element(double kx, double ky, double bx, double by, double gamma, const double fe[3],
                       const double ue[3], int shock, int hopt, double *Re_old, double *delta_old, int e,
                       const double X[3], const double Y[3], double ke[3][3], double Fe[3])
{
    const double third = 1.0/3.0, sixth = 1.0/6.0, seventh = 1.0/7.0, twelfth = 1.0/12.0;
    const double t320 = 3./20.0, n920 = 9./20.0, n940 = 9./40.0;
    double y23 = Y[1] - Y[2], y31 = Y[2] - Y[0], y12 = Y[0] - Y[1];
    double x32 = X[2] - X[1], x13 = X[0] - X[2], x21 = X[1] - X[0];
    double TwoA = x21*y31 - x13*y12;
    double Area = 0.5*TwoA;
    double invArea = 1.0/Area;
    double feb = third*(fe[0] + fe[1] + fe[2]);
    double ueb = third*(ue[0] + ue[1] + ue[2]);
    double a[3] = { bx*y23 + by*x32, bx*y31 + by*x13, bx*y12 + by*x21 };
    double C12 = y23*y31 + x32*x13, C13 = y23*y12 + x32*x21, C23 = y31*y12 + x13*x21;
    double D12 = 0.25*invArea*((kx*y23*y31) + (ky*x32*x13));
    double D13 = 0.25*invArea*((kx*y23*y12) + (ky*x32*x21));
    double D23 = 0.25*invArea*((kx*y31*y12) + (ky*x13*x21));
    double R11 = sixth*gamma*Area, R12 = twelfth*gamma*Area;
    double h = or_h_shock(hopt, bx, by, ue[0], ue[1], ue[2], y23, y31, y12, x32, x13, x21, Area);
    double Eu = 0.0;
    if (shock == 3)
        Eu = yzbeta(Re_old, delta_old, e, bx, by, gamma, ue[0], ue[1], ue[2], ueb, feb, y23, y31, y12, x32, x13,
                    x21, invArea, h);
    else if (shock == 2)
        Eu = cau_dd(bx, by, gamma, ue[0], ue[1], ue[2], ueb, feb, y23, y31, y12, x32, x13, x21, invArea, h);
    else if (shock == 1)
        Eu = cau(kx, ky, bx, by, gamma, ue[0], ue[1], ue[2], ueb, feb, y23, y31, y12, x32, x13, x21, invArea, h);
    double K12 = 0.25*Eu*invArea*C12, K13 = 0.25*Eu*invArea*C13, K23 = 0.25*Eu*invArea*C23;
    double Khh[3][3];
    Khh[0][0] = -(D12 + D13) + sixth*a[0] + R11 -(K12 + K13);
    Khh[0][1] =          D12 + sixth*a[1] + R12 + K12;
    Khh[0][2] =          D13 + sixth*a[2] + R12 + K13;
    Khh[1][0] =          D12 + sixth*a[0] + R12 + K12;
    Khh[1][1] = -(D12 + D23) + sixth*a[1] + R11 -(K12 + K23);
    Khh[1][2] =          D23 + sixth*a[2] + R12 + K23;
    Khh[2][0] =          D13 + sixth*a[0] + R12 + K13;
    Khh[2][1] =          D23 + sixth*a[1] + R12 + K23;
    Khh[2][2] = -(D13 + D23) + sixth*a[2] + R11 -(K13 + K23);
    double KhB[3], KBh[3];
    KhB[0] = n920*(0.5*a[0] + a[1] + a[2]) + t320*gamma*Area;
    KhB[1] = n920*(a[0] + 0.5*a[1] + a[2]) + t320*gamma*Area;
    KhB[2] = n920*(a[0] + a[1] + 0.5*a[2]) + t320*gamma*Area;
    for (int i = 0; i < 3; i++) KBh[i] = n940*a[i] + t320*gamma*Area;
    double KBB = -9*n940*(D12 + D13 + D23) + seventh*t320*(a[0] + a[1] + a[2]) + 9*seventh*n940*Area
               - Eu*invArea*(C12 + C13 + C23)/360.;
    double invKBB = 1.0/KBB;
    double Fh[3] = { twelfth*Area*(2*fe[0] + fe[1] + fe[2]), twelfth*Area*(fe[0] + 2*fe[1] + fe[2]),
                     twelfth*Area*(fe[0] + fe[1] + 2*fe[2]) };
    double FB = t320*Area*(fe[0] + fe[1] + fe[2]);
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) ke[i][j] = Khh[i][j] - invKBB*KhB[i]*KBh[j];
        Fe[i] = Fh[i] - invKBB*KhB[i]*FB;
    }
}

void or_build_k_f_supg(int nnodes, int nel, const double *x, const double *y,
                       const int *type, const int *invp, const int *ien, int neq,
                       const or_transport_problem *prob, const double *u,
                       double *A, double *F)
{
    const double third = 1.0/3.0, sixth = 1.0/6.0, twelfth = 1.0/12.0;
    double kx = prob->k, ky = prob->k, gamma = prob->gamma;
    double *U = malloc(sizeof(double) * (size_t)nnodes);
    int J, E;
    /* the shock-capture state of Process.c:16-17 (fresh zeros when the
       caller keeps none, as for a single build) */
    double *Re_old = prob->Re_old, *delta_old = prob->delta_old, *own = NULL;
    if (!Re_old || !delta_old) {
        own = calloc(2 * (size_t)(nel ? nel : 1), sizeof(double));
        Re_old = own;
        delta_old = own + (nel ? nel : 1);
    }
    memset(A, 0, sizeof(double) * 9 * (size_t)nel);
    for (J = 0; J < neq; J++) F[J] = 0;
    for (J = 0; J < nnodes; J++)
        U[J] = type[J] == 0 ? prob->upresc[J] : u[invp[J]];

    for (E = 0; E < nel; E++) {
        int J1 = ien[3*E], J2 = ien[3*E+1], J3 = ien[3*E+2];
        if (prob->form == 1) {                   /* StabilizationForm "DD" */
            const double Xv[3] = { x[J1], x[J2], x[J3] }, Yv[3] = { y[J1], y[J2], y[J3] };
            const double fv[3] = { prob->f, prob->f, prob->f }, uv[3] = { U[J1], U[J2], U[J3] };
            double ke[3][3], Fe[3];
            dd_element(kx, ky, prob->beta[0], prob->beta[1], gamma, fv, uv, prob->cau, prob->h_shock, Re_old,
                       delta_old, E, Xv, Yv, ke, Fe);
            const int V[3] = { J1, J2, J3 };
            for (int a = 0; a < 3; a++) {        /* F_assembly.c:3-28 */
                if (type[V[a]] != 1) continue;
                F[invp[V[a]]] += Fe[a];
                for (int b = 0; b < 3; b++)
                    if (b != a && type[V[b]] == 0) F[invp[V[a]]] -= ke[a][b] * prob->upresc[V[b]];
            }
            double *Ae = A + 9L * E;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) Ae[3*r + c] = ke[r][c];
            continue;
        }
        double X0 = x[J1], X1 = x[J2], X2 = x[J3];
        double Y0 = y[J1], Y1 = y[J2], Y2 = y[J3];
        double y23 = Y1 - Y2, y31 = Y2 - Y0, y12 = Y0 - Y1;
        double x32 = X2 - X1, x13 = X0 - X2, x21 = X1 - X0;
        double TwoA = x21*y31 - x13*y12;
        double Area = 0.5*TwoA;
        double invArea = 1.0/Area;
        double h = sqrt(fabs(TwoA));
        double bx = prob->beta[0], by = prob->beta[1];
        double norm = sqrt(bx*bx + by*by);
        double tau = norm > 0 ? 0.5*h/norm : 0;
        double fe1 = prob->f, fe2 = prob->f, fe3 = prob->f;
        double feb = third*(fe1 + fe2 + fe3);
        double ue1 = U[J1], ue2 = U[J2], ue3 = U[J3];
        double ueb = third*(ue1 + ue2 + ue3);
        double D12 = 0.25*invArea*((kx*y23*y31) + (ky*x32*x13));
        double D13 = 0.25*invArea*((kx*y23*y12) + (ky*x32*x21));
        double D23 = 0.25*invArea*((kx*y31*y12) + (ky*x13*x21));
        double C11 = sixth*(bx*y23 + by*x32);
        double C12 = sixth*(bx*y31 + by*x13);
        double C13 = sixth*(bx*y12 + by*x21);
        double R11 = sixth*(gamma*Area);
        double R12 = twelfth*(gamma*Area);
        double Cpg12 = 0.25*invArea*tau*(y23*(bx*bx*y31 + bx*by*x13) + x32*(bx*by*y31 + by*by*x13));
        double Cpg13 = 0.25*invArea*tau*(y23*(bx*bx*y12 + bx*by*x21) + x32*(bx*by*y12 + by*by*x21));
        double Cpg23 = 0.25*invArea*tau*(y31*(bx*bx*y12 + bx*by*x21) + x13*(bx*by*y12 + by*by*x21));
        double Rpg11 = sixth*tau*gamma*(bx*y23 + by*x32);
        double Rpg21 = sixth*tau*gamma*(bx*y31 + by*x13);
        double Rpg31 = sixth*tau*gamma*(bx*y12 + by*x21);
        double hs = or_h_shock(prob->h_shock, bx, by, ue1, ue2, ue3, y23, y31, y12, x32, x13, x21, Area);
        double Eu = prob->cau == 3 ? yzbeta(Re_old, delta_old, E, bx, by, gamma, ue1, ue2, ue3, ueb, feb,
                                            y23, y31, y12, x32, x13, x21, invArea, hs)
                  : prob->cau ? cau(kx, ky, bx, by, gamma, ue1, ue2, ue3, ueb, feb,
                                    y23, y31, y12, x32, x13, x21, invArea, hs) : 0.0;
        double Csc12 = Eu*0.25*invArea*(y23*y31 + x32*x13);
        double Csc13 = Eu*0.25*invArea*(y23*y12 + x32*x21);
        double Csc23 = Eu*0.25*invArea*(y31*y12 + x13*x21);
        double ke[3][3];
        ke[0][0] = -(D12 + D13) + C11 - (Cpg12 + Cpg13) + R11 + Rpg11 - (Csc12 + Csc13);
        ke[0][1] = D12 + C12 + Cpg12 + R12 + Rpg11 + Csc12;
        ke[0][2] = D13 + C13 + Cpg13 + R12 + Rpg11 + Csc13;
        ke[1][0] = D12 + C11 + Cpg12 + R12 + Rpg21 + Csc12;
        ke[1][1] = -(D12 + D23) + C12 - (Cpg12 + Cpg23) + R11 + Rpg21 - (Csc12 + Csc23);
        ke[1][2] = D23 + C13 + Cpg23 + R12 + Rpg21 + Csc23;
        ke[2][0] = D13 + C11 + Cpg13 + R12 + Rpg31 + Csc13;
        ke[2][1] = D23 + C12 + Cpg23 + R12 + Rpg31 + Csc23;
        ke[2][2] = -(D13 + D23) + C13 - (Cpg13 + Cpg23) + R11 + Rpg31 - (Csc13 + Csc23);
        double Fe1 = Area*twelfth*(2*fe1 + fe2 + fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y23 + by*x32);
        double Fe2 = Area*twelfth*(fe1 + 2*fe2 + fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y31 + by*x13);
        double Fe3 = Area*twelfth*(fe1 + fe2 + 2*fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y12 + by*x21);
        /* F_assembly (F_assembly.c:3-28): Dirichlet lifting per free vertex */
        const int V[3] = { J1, J2, J3 };
        const double Fe[3] = { Fe1, Fe2, Fe3 };
        for (int a = 0; a < 3; a++) {
            if (type[V[a]] != 1) continue;
            F[invp[V[a]]] += Fe[a];
            for (int b = 0; b < 3; b++)
                if (b != a && type[V[b]] == 0)
                    F[invp[V[a]]] -= ke[a][b] * prob->upresc[V[b]];
        }
        /* ebe_assembly (ebe_assembly.c:3-19) */
        double *Ae = A + 9L * E;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) Ae[3*r + c] = ke[r][c];
    }
    free(U);
    free(own);
}

int or_transport_process(int nnodes, int nel, const double *x, const double *y,
                         const int *type, const int *invp, const int *ien, int neq,
                         const or_transport_problem *prob,
                         double solver_tol, double nonlinear_tol, int kmax, int lmax,
                         int max_nonlinear, double *U, int *gmres_iterations)
{
    int NEQ = neq, it = 0, i;
    int *lm = malloc(sizeof(int) * 3 * (size_t)nel);
    int *Perm = malloc(sizeof(int) * ((size_t)NEQ + 1));
    int *invPerm = malloc(sizeof(int) * ((size_t)NEQ + 1));
    double *A = malloc(sizeof(double) * 9 * (size_t)nel);
    double *F = calloc((size_t)NEQ + 1, sizeof(double));
    double *Diag = calloc((size_t)NEQ + 1, sizeof(double));
    double *invDiag = calloc((size_t)NEQ + 1, sizeof(double));
    double *uold = calloc((size_t)NEQ + 1, sizeof(double));
    double normdiff = nonlinear_tol + 1, normu = 1.0 / nonlinear_tol;

    or_fill_lm(nel, 1, ien, type, invp, NEQ, lm);
    or_permutation_of_lm(nel, ien, type, invp, NEQ, Perm, invPerm, NULL);
    if (gmres_iterations) *gmres_iterations = 0;
    /* Process.c:16-17: the shock-capture state lives for the whole loop */
    or_transport_problem pl = *prob;
    double *state = calloc(2 * (size_t)(nel ? nel : 1), sizeof(double));
    pl.Re_old = state;
    pl.delta_old = state + (nel ? nel : 1);
    prob = &pl;
    /* Process.c:37-86 */
    while (normdiff > nonlinear_tol * normu && it < max_nonlinear) {
        it++;
        memcpy(uold, U, sizeof(double) * neq);
        or_build_k_f_supg(nnodes, nel, x, y, type, invp, ien, neq, prob, U, A, F);
        int gi = or_ebe_diag_solve(nel, 3, lm, A, NEQ, Perm, invPerm, Diag, invDiag, F,
                                   kmax, lmax, solver_tol, U);
        if (gmres_iterations) *gmres_iterations += gi;
        for (i = 0; i < neq; i++) uold[i] += -1 * U[i];
        normdiff = sqrt(or_ddot(neq, uold, uold));
        normu = sqrt(or_ddot(neq, U, U));
    }
    free(lm); free(Perm); free(invPerm); free(A); free(F);
    free(Diag); free(invDiag); free(uold); free(state);
    return it;
}
