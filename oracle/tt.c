/*
 * femoracle: transient SUPG/CAU convection-diffusion-reaction on P1
 * triangles.  TEST INFRASTRUCTURE ONLY (see femoracle.h).
 *
 * Restates 02_Transport_Equation/2D/01_CommonFiles/Build_M_K_R_SUPG.c:6-252
 * (SUPG mass, diffusion, convection, reaction, SUPG and CAU terms; the block
 * Ae = me + alpha dt ke stored per element as ebe_assembly does; the
 * residual R = F - me du - ke u accumulated element by element), with
 * CAU_ShockCapture.c:3-33 (residual including du), h_shock_2sqrtArea.c and
 * eval_U_dU.c, and the Predictor_Old.c:6-134 time loop with Diag
 * preconditioning (accumulating, Diag_precond_EBE_setup.c) and GMRES.  The
 * element formulas are the reference's, term for term, so blocks and
 * residual agree to the last bit when both are compiled without
 * floating-point contraction.
 *
 * StabilizationForm "DD" with TimeIntegration "Predictor1"
 * (setStabilizationForm.c:40-74): Build_M_K_R_DD.c:5-190 with the transient
 * CAU_DD_ShockCapture.c (Ru includes du/dt) relaxed against the element's
 * previous value, cb = (cbtil + cbtil_old) / 2 (the state, delta_old, lives
 * for the whole time loop), the bubble condensed into the mass and
 * stiffness blocks and the load as in the steady DD build.
 *
 * TimeIntegration "Predictor2" with "DD" (setStabilizationForm.c:51-54):
 * Build_M_F_DD.c:6-263 keeps the bubble of each element as an unknown (uB,
 * duB) and condenses it out of the element system (N2 = MBB + alpha dt KBB),
 * calculate_DaB.c:3-30 recovers its increment from Da after the solve, and
 * Predictor_New.c:3-179 predicts and corrects it with u and a.
 */
#include "femoracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* CAU_ShockCapture of the transient driver: Ru includes du/dt. */
static double tt_cau(double kx, double ky, double bx, double by, double gamma, double ue1, double ue2,
                     double ue3, double ueb, double dueb, double feb, double y23, double y31, double y12,
                     double x32, double x13, double x21, double invArea, double h)
{
    double third = 1. / 3.;
    double bgu = 0.5*invArea*(ue1*(bx*y23 + by*x32) + ue2*(bx*y31 + by*x13) + ue3*(bx*y12 + by*x21));
    double Ru = dueb + bgu + gamma*ueb - feb;
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

/* YZBeta_ShockCapture of the transient driver (no state; Ru includes du/dt) */
static double tt_yzbeta(double bx, double by, double gamma, double ue1, double ue2, double ue3, double ueb,
                        double dueb, double feb, double y23, double y31, double y12, double x32, double x13,
                        double x21, double invArea, double h)
{
    double bgu = 0.5*invArea*(ue1*(bx*y23 + by*x32) + ue2*(bx*y31 + by*x13) + ue3*(bx*y12 + by*x21));
    double Ru = dueb + bgu + gamma*ueb - feb;
    double nRu = fabs(Ru);
    double gx = 0.5*invArea*(y23*ue1 + y31*ue2 + y12*ue3);
    double gy = 0.5*invArea*(x32*ue1 + x13*ue2 + x21*ue3);
    double ng = sqrt(gx*gx + gy*gy);
    double nu = fabs(ueb);
    return (nu >= 1e-12 && ng >= 1e-12) ? 0.25*h*nRu/ng + 0.125*h*h*nRu/nu : 0;
}

/* Build_M_K_R_DD.c:61-180 for one element: Ae (row-major), the load term
 * Fr[i] added to R[lm[i]] and the three terms sub[i][j] then subtracted. */
static void tt_dd_element(double kx, double ky, double bx, double by, double gamma, double fv, const double X[3],
                          const double Y[3], const double ue[3], const double due[3], double alpha, double dt,
                          int shock, int hopt, double *cbtilo, int e, double Ae[9], double Fr[3], double sub[3][3])
{
    const double third = 1.0/3.0, sixth = 1.0/6.0, seventh = 1.0/7.0, twelfth = 1.0/12.0;
    const double t320 = 3./20.0, n920 = 9./20.0, n940 = 9./40.0, w = 0.5;
    double y23 = Y[1] - Y[2], y31 = Y[2] - Y[0], y12 = Y[0] - Y[1];
    double x32 = X[2] - X[1], x13 = X[0] - X[2], x21 = X[1] - X[0];
    double TwoA = x21*y31 - x13*y12;
    double Area = 0.5*TwoA;
    double invArea = 1.0/Area;
    double fe1 = fv, fe2 = fv, fe3 = fv;
    double feb = third*(fe1 + fe2 + fe3);
    double ueb = third*(ue[0] + ue[1] + ue[2]);
    double dueb = third*(due[0] + due[1] + due[2]);
    double Mhh = twelfth*Area, MBh = t320*Area;
    double a1 = bx*y23 + by*x32, a2 = bx*y31 + by*x13, a3 = bx*y12 + by*x21;
    double C12 = y23*y31 + x32*x13, C13 = y23*y12 + x32*x21, C23 = y31*y12 + x13*x21;
    double D12 = 0.25*invArea*((kx*y23*y31) + (ky*x32*x13));
    double D13 = 0.25*invArea*((kx*y23*y12) + (ky*x32*x21));
    double D23 = 0.25*invArea*((kx*y31*y12) + (ky*x13*x21));
    double R11 = sixth*gamma*Area, R12 = twelfth*gamma*Area;
    double Eu = 0.0;
    if (shock == 2 || shock == 3) {   /* CAUDD or YZBeta (Ru with du/dt), relaxed */
        double h = or_h_shock(hopt, bx, by, ue[0], ue[1], ue[2], y23, y31, y12, x32, x13, x21, Area);
        double cbtil;
        if (shock == 3) {
            cbtil = tt_yzbeta(bx, by, gamma, ue[0], ue[1], ue[2], ueb, dueb, feb, y23, y31, y12, x32, x13, x21,
                              invArea, h);
        } else {
            double bgu = 0.5*invArea*(ue[0]*(bx*y23 + by*x32) + ue[1]*(bx*y31 + by*x13) + ue[2]*(bx*y12 + by*x21));
            double Ru = dueb + bgu + gamma*ueb - feb;
            double gx = 0.5*invArea*(y23*ue[0] + y31*ue[1] + y12*ue[2]);
            double gy = 0.5*invArea*(x32*ue[0] + x13*ue[1] + x21*ue[2]);
            double ng = sqrt(gx*gx + gy*gy);
            cbtil = ng > 1e-10 ? 0.5*h*fabs(Ru)/ng : 0;
        }
        double cb = w*cbtil + (1 - w)*cbtilo[e];
        cbtilo[e] = cbtil;
        Eu = cb;
    }
    double K12 = 0.25*Eu*invArea*C12, K13 = 0.25*Eu*invArea*C13, K23 = 0.25*Eu*invArea*C23;
    double Khh[3][3];
    Khh[0][0] = -(D12 + D13) + sixth*a1 + R11 -(K12 + K13);
    Khh[0][1] =          D12 + sixth*a2 + R12 + K12;
    Khh[0][2] =          D13 + sixth*a3 + R12 + K13;
    Khh[1][0] =          D12 + sixth*a1 + R12 + K12;
    Khh[1][1] = -(D12 + D23) + sixth*a2 + R11 -(K12 + K23);
    Khh[1][2] =          D23 + sixth*a3 + R12 + K23;
    Khh[2][0] =          D13 + sixth*a1 + R12 + K13;
    Khh[2][1] =          D23 + sixth*a2 + R12 + K23;
    Khh[2][2] = -(D13 + D23) + sixth*a3 + R11 -(K13 + K23);
    double KhB[3] = { n920*(0.5*a1 + a2 + a3) + t320*gamma*Area, n920*(a1 + 0.5*a2 + a3) + t320*gamma*Area,
                      n920*(a1 + a2 + 0.5*a3) + t320*gamma*Area };
    double KBh[3] = { n940*a1 + t320*gamma*Area, n940*a2 + t320*gamma*Area, n940*a3 + t320*gamma*Area };
    double KBB = -9*n940*(D12 + D13 + D23) + seventh*t320*(a1 + a2 + a3) + 9*seventh*n940*Area
               - Eu*invArea*(C12 + C13 + C23)/360.;
    double invKBB = 1.0/KBB;
    double Fh[3] = { twelfth*Area*(2*fe1 + fe2 + fe3), twelfth*Area*(fe1 + 2*fe2 + fe3),
                     twelfth*Area*(fe1 + fe2 + 2*fe3) };
    double FB = t320*Area*(fe1 + fe2 + fe3);
    for (int i = 0; i < 3; i++) {
        double me[3];
        for (int j = 0; j < 3; j++) me[j] = Mhh - invKBB*KhB[i]*MBh;
        me[i] += Mhh;
        Fr[i] = Fh[i] - invKBB*KhB[i]*FB;
        for (int j = 0; j < 3; j++) {
            double ke = Khh[i][j] - invKBB*KhB[i]*KBh[j];
            Ae[3*i + j] = me[j] + alpha*dt*ke;
            sub[i][j] = me[j]*due[j] + ke*ue[j];
        }
    }
}

void or_build_tt(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                 const int *ien, int neq, const or_transport_problem *prob, double alpha, double dt,
                 const double *u, const double *du, double *A, double *R)
{
    const double third = 1.0/3.0, sixth = 1.0/6.0, twelfth = 1.0/12.0;
    const double kx = prob->k, ky = prob->k, gamma = prob->gamma;
    double *U = malloc(sizeof(double) * (size_t)(nnodes ? nnodes : 1));
    double *dU = malloc(sizeof(double) * (size_t)(nnodes ? nnodes : 1));
    int J, E;
    for (J = 0; J <= neq; J++) R[J] = 0;
    for (J = 0; J < nnodes; J++) {          /* eval_U_dU.c:3-22 */
        U[J] = type[J] == 0 ? prob->upresc[J] : u[invp[J]];
        dU[J] = type[J] == 0 ? 0.0 : du[invp[J]];
    }
    double *cbtilo = prob->delta_old, *own = NULL;    /* DD: the time loop's delta_old */
    if (prob->form == 1 && !cbtilo) cbtilo = own = calloc((size_t)(nel ? nel : 1), sizeof(double));
    for (E = 0; E < nel; E++) {
        int J1 = ien[3*E], J2 = ien[3*E+1], J3 = ien[3*E+2];
        if (prob->form == 1) {
            const double Xv[3] = { x[J1], x[J2], x[J3] }, Yv[3] = { y[J1], y[J2], y[J3] };
            const double uv[3] = { U[J1], U[J2], U[J3] }, dv[3] = { dU[J1], dU[J2], dU[J3] };
            double Ae[9], Fr[3], sub[3][3];
            tt_dd_element(kx, ky, prob->beta[0], prob->beta[1], gamma, prob->f, Xv, Yv, uv, dv, alpha, dt,
                          prob->cau, prob->h_shock, cbtilo, E, Ae, Fr, sub);
            const int lm[3] = { type[J1] == 0 ? neq : invp[J1], type[J2] == 0 ? neq : invp[J2],
                                type[J3] == 0 ? neq : invp[J3] };
            for (int i = 0; i < 3; i++) {            /* Build_M_K_R_DD.c:161-176 */
                R[lm[i]] += Fr[i];
                for (int j = 0; j < 3; j++) R[lm[i]] -= sub[i][j];
            }
            R[neq] = 0;
            memcpy(A + 9L * E, Ae, sizeof Ae);
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
        double ue[3] = { U[J1], U[J2], U[J3] }, due[3] = { dU[J1], dU[J2], dU[J3] };
        double ueb = third*(ue[0] + ue[1] + ue[2]);
        double dueb = third*(due[0] + due[1] + due[2]);
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
        double hs = or_h_shock(prob->h_shock, bx, by, ue[0], ue[1], ue[2], y23, y31, y12, x32, x13, x21, Area);
        double Eu = prob->cau == 3 ? tt_yzbeta(bx, by, gamma, ue[0], ue[1], ue[2], ueb, dueb, feb, y23, y31, y12,
                                               x32, x13, x21, invArea, hs)
                  : prob->cau ? tt_cau(kx, ky, bx, by, gamma, ue[0], ue[1], ue[2], ueb, dueb, feb,
                                       y23, y31, y12, x32, x13, x21, invArea, hs) : 0.0;
        double Csc12 = Eu*0.25*invArea*(y23*y31 + x32*x13);
        double Csc13 = Eu*0.25*invArea*(y23*y12 + x32*x21);
        double Csc23 = Eu*0.25*invArea*(y31*y12 + x13*x21);
        double me[3][3], ke[3][3];
        me[0][0] = sixth*Area + tau*C11;
        me[0][1] = twelfth*Area + tau*C11;
        me[0][2] = twelfth*Area + tau*C11;
        me[1][0] = twelfth*Area + tau*C12;
        me[1][1] = sixth*Area + tau*C12;
        me[1][2] = twelfth*Area + tau*C12;
        me[2][0] = twelfth*Area + tau*C13;
        me[2][1] = twelfth*Area + tau*C13;
        me[2][2] = sixth*Area + tau*C13;
        ke[0][0] = -(D12 + D13) + C11 - (Cpg12 + Cpg13) + R11 + Rpg11 - (Csc12 + Csc13);
        ke[0][1] = D12 + C12 + Cpg12 + R12 + Rpg11 + Csc12;
        ke[0][2] = D13 + C13 + Cpg13 + R12 + Rpg11 + Csc13;
        ke[1][0] = D12 + C11 + Cpg12 + R12 + Rpg21 + Csc12;
        ke[1][1] = -(D12 + D23) + C12 - (Cpg12 + Cpg23) + R11 + Rpg21 - (Csc12 + Csc23);
        ke[1][2] = D23 + C13 + Cpg23 + R12 + Rpg21 + Csc23;
        ke[2][0] = D13 + C11 + Cpg13 + R12 + Rpg31 + Csc13;
        ke[2][1] = D23 + C12 + Cpg23 + R12 + Rpg31 + Csc23;
        ke[2][2] = -(D13 + D23) + C13 - (Cpg13 + Cpg23) + R11 + Rpg31 - (Csc13 + Csc23);
        /* lm of the element (Fill_LM.c): equation or the sink neq */
        int lm[3];
        lm[0] = type[J1] == 0 ? neq : invp[J1];
        lm[1] = type[J2] == 0 ? neq : invp[J2];
        lm[2] = type[J3] == 0 ? neq : invp[J3];
        R[lm[0]] += Area*twelfth*(2*fe1 + fe2 + fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y23 + by*x32);
        R[lm[1]] += Area*twelfth*(fe1 + 2*fe2 + fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y31 + by*x13);
        R[lm[2]] += Area*twelfth*(fe1 + fe2 + 2*fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y12 + by*x21);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) R[lm[i]] -= me[i][j]*due[j] + ke[i][j]*ue[j];
        R[neq] = 0;
        double *Ae = A + 9L * E;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) Ae[3*i + j] = me[i][j] + alpha*dt*ke[i][j];
    }
    free(U);
    free(dU);
    free(own);
}

/* Build_M_F_DD.c:52-244 for one element: the bubble kept as an unknown
 * (uB, duB) and condensed out of the element system.  Me (row-major), the
 * load Fe[i] added to F[lm[i]], and cond = (invN2, R2, M2[0..2]), which
 * calculate_DaB reads after the solve. */
static void tt_mfdd_element(double kx, double ky, double bx, double by, double gamma, double fv,
                            const double X[3], const double Y[3], const double ue[3], const double due[3],
                            double uB, double duB, double alpha, double dt, int shock, int hopt, double *cbtilo,
                            int e, double Me[9], double Fe[3], double cond[5])
{
    const double third = 1.0/3.0, sixth = 1.0/6.0, seventh = 1.0/7.0, twelfth = 1.0/12.0;
    const double t320 = 3./20.0, n920 = 9./20.0, n940 = 9./40.0, w = 0.5;
    double y23 = Y[1] - Y[2], y31 = Y[2] - Y[0], y12 = Y[0] - Y[1];
    double x32 = X[2] - X[1], x13 = X[0] - X[2], x21 = X[1] - X[0];
    double TwoA = x21*y31 - x13*y12;
    double Area = 0.5*TwoA;
    double invArea = 1.0/Area;
    double fe1 = fv, fe2 = fv, fe3 = fv;
    double feb = third*(fe1 + fe2 + fe3);
    double ueb = third*(ue[0] + ue[1] + ue[2]);
    double dueb = third*(due[0] + due[1] + due[2]);
    double Mhh = twelfth*Area, MhB = t320*Area, MBh = MhB, MBB = (81.0/280.)*Area;
    double a1 = bx*y23 + by*x32, a2 = bx*y31 + by*x13, a3 = bx*y12 + by*x21;
    double C12 = y23*y31 + x32*x13, C13 = y23*y12 + x32*x21, C23 = y31*y12 + x13*x21;
    double D12 = 0.25*invArea*((kx*y23*y31) + (ky*x32*x13));
    double D13 = 0.25*invArea*((kx*y23*y12) + (ky*x32*x21));
    double D23 = 0.25*invArea*((kx*y31*y12) + (ky*x13*x21));
    double R11 = sixth*gamma*Area, R12 = twelfth*gamma*Area;
    double Eu = 0.0;
    if (shock == 2 || shock == 3) {   /* CAUDD or YZBeta, relaxed against the previous value */
        double h = or_h_shock(hopt, bx, by, ue[0], ue[1], ue[2], y23, y31, y12, x32, x13, x21, Area);
        double cbtil;
        if (shock == 3) {
            cbtil = tt_yzbeta(bx, by, gamma, ue[0], ue[1], ue[2], ueb, dueb, feb, y23, y31, y12, x32, x13, x21,
                              invArea, h);
        } else {
            double bgu = 0.5*invArea*(ue[0]*(bx*y23 + by*x32) + ue[1]*(bx*y31 + by*x13) + ue[2]*(bx*y12 + by*x21));
            double Ru = dueb + bgu + gamma*ueb - feb;
            double gx = 0.5*invArea*(y23*ue[0] + y31*ue[1] + y12*ue[2]);
            double gy = 0.5*invArea*(x32*ue[0] + x13*ue[1] + x21*ue[2]);
            double ng = sqrt(gx*gx + gy*gy);
            cbtil = ng > 1e-10 ? 0.5*h*fabs(Ru)/ng : 0;
        }
        double cb = w*cbtil + (1 - w)*cbtilo[e];
        cbtilo[e] = cbtil;
        Eu = cb;
    }
    double K12 = 0.25*Eu*invArea*C12, K13 = 0.25*Eu*invArea*C13, K23 = 0.25*Eu*invArea*C23;
    double Khh[3][3];
    Khh[0][0] = -(D12 + D13) + sixth*a1 + R11 -(K12 + K13);
    Khh[0][1] =          D12 + sixth*a2 + R12 + K12;
    Khh[0][2] =          D13 + sixth*a3 + R12 + K13;
    Khh[1][0] =          D12 + sixth*a1 + R12 + K12;
    Khh[1][1] = -(D12 + D23) + sixth*a2 + R11 -(K12 + K23);
    Khh[1][2] =          D23 + sixth*a3 + R12 + K23;
    Khh[2][0] =          D13 + sixth*a1 + R12 + K13;
    Khh[2][1] =          D23 + sixth*a2 + R12 + K23;
    Khh[2][2] = -(D13 + D23) + sixth*a3 + R11 -(K13 + K23);
    double KhB[3] = { n920*(0.5*a1 + a2 + a3) + t320*gamma*Area, n920*(a1 + 0.5*a2 + a3) + t320*gamma*Area,
                      n920*(a1 + a2 + 0.5*a3) + t320*gamma*Area };
    double KBh[3] = { n940*a1 + t320*gamma*Area, n940*a2 + t320*gamma*Area, n940*a3 + t320*gamma*Area };
    double KBB = -9*n940*(D12 + D13 + D23) + seventh*t320*(a1 + a2 + a3) + 9*seventh*n940*Area
               - Eu*invArea*(C12 + C13 + C23)/360.;
    double Fh[3] = { twelfth*Area*(2*fe1 + fe2 + fe3), twelfth*Area*(fe1 + 2*fe2 + fe3),
                     twelfth*Area*(fe1 + fe2 + 2*fe3) };
    double FB = t320*Area*(fe1 + fe2 + fe3);
    double N2 = MBB + alpha*dt*KBB;
    double invN2 = 1.0/N2;
    double R2 = FB - MBB*duB - KBB*uB;
    double M1[3][3], M2[3], N1[3], R1[3];
    for (int i = 0; i < 3; i++) {            /* Build_M_F_DD.c:192-206 */
        M1[i][0] = Mhh;
        M1[i][1] = Mhh;
        M1[i][2] = Mhh;
        M1[i][i] += Mhh;
        M2[i] = MBh + alpha*dt*KBh[i];
        N1[i] = MhB + alpha*dt*KhB[i];
        R1[i] = Fh[i] - MhB*duB - KhB[i]*uB;
        R1[i] -= Mhh*due[i];
        for (int j = 0; j < 3; j++) {
            M1[i][j] += alpha*dt*Khh[i][j];
            R1[i] -= Mhh*due[j] + Khh[i][j]*ue[j];
        }
        R2 -= MBh*due[i] + KBh[i]*ue[i];
    }
    for (int i = 0; i < 3; i++) {            /* :208-212 */
        for (int j = 0; j < 3; j++) Me[3*i + j] = M1[i][j] - invN2*N1[i]*M2[j];
        Fe[i] = R1[i] - invN2*N1[i]*R2;
    }
    cond[0] = invN2;
    cond[1] = R2;
    cond[2] = M2[0];
    cond[3] = M2[1];
    cond[4] = M2[2];
}

void or_build_tt_mfdd(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                      const int *ien, int neq, const or_transport_problem *prob, double alpha, double dt,
                      const double *u, const double *du, const double *uB, const double *duB, double *A,
                      double *F, double *cond)
{
    double *U = malloc(sizeof(double) * (size_t)(nnodes ? nnodes : 1));
    double *dU = malloc(sizeof(double) * (size_t)(nnodes ? nnodes : 1));
    int J, E;
    for (J = 0; J <= neq; J++) F[J] = 0;
    for (J = 0; J < nnodes; J++) {          /* eval_U_dU.c:3-22 */
        U[J] = type[J] == 0 ? prob->upresc[J] : u[invp[J]];
        dU[J] = type[J] == 0 ? 0.0 : du[invp[J]];
    }
    double *cbtilo = prob->delta_old, *own = NULL;    /* the time loop's delta_old */
    if (!cbtilo) cbtilo = own = calloc((size_t)(nel ? nel : 1), sizeof(double));
    for (E = 0; E < nel; E++) {
        int J1 = ien[3*E], J2 = ien[3*E+1], J3 = ien[3*E+2];
        const double Xv[3] = { x[J1], x[J2], x[J3] }, Yv[3] = { y[J1], y[J2], y[J3] };
        const double uv[3] = { U[J1], U[J2], U[J3] }, dv[3] = { dU[J1], dU[J2], dU[J3] };
        double Fe[3];
        tt_mfdd_element(prob->k, prob->k, prob->beta[0], prob->beta[1], prob->gamma, prob->f, Xv, Yv, uv, dv,
                        uB[E], duB[E], alpha, dt, prob->cau, prob->h_shock, cbtilo, E, A + 9L * E, Fe,
                        cond + 5L * E);
        const int lm[3] = { type[J1] == 0 ? neq : invp[J1], type[J2] == 0 ? neq : invp[J2],
                            type[J3] == 0 ? neq : invp[J3] };
        for (int i = 0; i < 3; i++) F[lm[i]] += Fe[i];
        F[neq] = 0;
    }
    free(U);
    free(dU);
    free(own);
}

void or_tt_dab(int nel, const int *lm, int NEQ, const double *cond, double *Da, double *DaB)
{
    Da[NEQ] = 0;                             /* calculate_DaB.c:16-27 */
    for (int e = 0; e < nel; e++) {
        const double *c = cond + 5L * e;
        double M2Da = c[2]*Da[lm[3*e]] + c[3]*Da[lm[3*e+1]] + c[4]*Da[lm[3*e+2]];
        DaB[e] = c[0]*(c[1] - M2Da);
    }
}

typedef struct {
    int nel, NEQ;
    const int *lm, *Perm, *invPerm;
    const double *A, *invDiag;
} tt_ctx;

static int tt_mv_cb(void *p, double *P, double *Q)
{
    tt_ctx *c = (tt_ctx *)p;
    or_ebemv3_perm(c->nel, c->lm, c->A, c->Perm, c->invPerm, c->NEQ, P, Q);
    return 0;
}

static int tt_pc_cb(void *p, double *x, double *z)
{
    tt_ctx *c = (tt_ctx *)p;
    or_diag_apply(c->NEQ, c->invDiag, x, z);
    return 0;
}

typedef struct {
    tt_ctx mv;
    int nnodes, nel, neq;
    const double *x, *y;
    const int *type, *invp, *ien;
    const or_transport_problem *prob;
    double *R, *Diag;
    double solver_tol;
    int kmax, lmax;
} tt_loop;

/* one correction: Build_M_K_R_SUPG at Alpha_Build / DeltaT_Build, the
 * accumulating Diag_precond_EBE_setup on R, pgmres for Da */
static int tt_correct(void *p, double alpha_b, double dt_b, const double *u, const double *a, double *Da, int *gi)
{
    tt_loop *c = (tt_loop *)p;
    or_build_tt(c->nnodes, c->nel, c->x, c->y, c->type, c->invp, c->ien, c->neq, c->prob, alpha_b, dt_b, u, a,
                (double *)c->mv.A, c->R);
    or_diag_setup(c->nel, 3, c->mv.lm, c->mv.A, c->neq, c->Diag, (double *)c->mv.invDiag, c->R);
    or_pgmres(c->neq, c->kmax, c->lmax, c->solver_tol, tt_mv_cb, tt_pc_cb, &c->mv, c->R, Da, gi);
    return 0;
}

int or_tt_predictor(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                    const int *ien, int neq, const or_transport_problem *prob, double alpha, double dt,
                    const or_time_opts *to, double solver_tol, int kmax, int lmax, double *u, double *a,
                    or_time_stats *st)
{
    const int NEQ = neq;
    size_t ne = (size_t)(nel ? nel : 1);
    int *lm = malloc(sizeof(int) * 3 * ne);
    int *Perm = malloc(sizeof(int) * ((size_t)NEQ + 1)), *invPerm = malloc(sizeof(int) * ((size_t)NEQ + 1));
    double *A = malloc(sizeof(double) * 9 * ne);
    double *R = calloc((size_t)NEQ + 1, sizeof(double));
    double *Diag = calloc((size_t)NEQ + 1, sizeof(double)), *invDiag = calloc((size_t)NEQ + 1, sizeof(double));
    or_fill_lm(nel, 1, ien, type, invp, NEQ, lm);
    or_permutation_of_lm(nel, ien, type, invp, NEQ, Perm, invPerm, NULL);
    /* the DD shock-capture state lives for the whole loop (Predictor_Old.c:30) */
    or_transport_problem pl = *prob;
    double *state = calloc((size_t)(nel ? nel : 1), sizeof(double));
    pl.delta_old = state;
    tt_loop c = { { nel, NEQ, lm, Perm, invPerm, A, invDiag }, nnodes, nel, neq, x, y, type, invp, ien, &pl, R,
                  Diag, solver_tol, kmax, lmax };
    int steps = or_time_integrate(neq, alpha, dt, to, tt_correct, &c, u, a, st);
    free(lm); free(Perm); free(invPerm); free(A); free(R); free(Diag); free(invDiag); free(state);
    return steps;
}

/* Predictor_New.c:3-179 with Build_M_F_DD and calculate_DaB: the loop of
 * Predictor_Old for (u, a) plus the bubble unknowns (uB, aB) per element,
 * predicted with u and corrected from Da after every solve. */
typedef struct {
    tt_loop base;
    double *uB, *aB, *cond, *DaB;
} tt_loop2;

static void tt_predict2(void *p, int op, double coef, double c2, const double *u)
{
    tt_loop2 *c = (tt_loop2 *)p;
    (void)c2; (void)u;
    if (op != OR_B_PREDICT) return;          /* Predictor_New has no other bubble step */
    for (int e = 0; e < c->base.nel; e++) c->uB[e] += coef * c->aB[e];   /* :82-83 */
    memset(c->aB, 0, sizeof(double) * (size_t)c->base.nel);
}

static int tt_correct2(void *p, double alpha_b, double dt_b, const double *u, const double *a, double *Da, int *gi)
{
    tt_loop2 *c = (tt_loop2 *)p;
    tt_loop *b = &c->base;
    or_build_tt_mfdd(b->nnodes, b->nel, b->x, b->y, b->type, b->invp, b->ien, b->neq, b->prob, alpha_b, dt_b, u,
                     a, c->uB, c->aB, (double *)b->mv.A, b->R, c->cond);
    or_diag_setup(b->nel, 3, b->mv.lm, b->mv.A, b->neq, b->Diag, (double *)b->mv.invDiag, b->R);
    or_pgmres(b->neq, b->kmax, b->lmax, b->solver_tol, tt_mv_cb, tt_pc_cb, &b->mv, b->R, Da, gi);
    or_tt_dab(b->nel, b->mv.lm, b->neq, c->cond, Da, c->DaB);                /* :99 */
    const double coef = alpha_b * dt_b;
    for (int e = 0; e < b->nel; e++) {                                       /* :104-105 */
        c->aB[e] += c->DaB[e];
        c->uB[e] += coef * c->DaB[e];
    }
    return 0;
}

int or_tt_predictor2(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                     const int *ien, int neq, const or_transport_problem *prob, double alpha, double dt,
                     const or_time_opts *to, double solver_tol, int kmax, int lmax, double *u, double *a,
                     double *uB, double *aB, or_time_stats *st)
{
    const int NEQ = neq;
    size_t ne = (size_t)(nel ? nel : 1);
    int *lm = malloc(sizeof(int) * 3 * ne);
    int *Perm = malloc(sizeof(int) * ((size_t)NEQ + 1)), *invPerm = malloc(sizeof(int) * ((size_t)NEQ + 1));
    double *A = malloc(sizeof(double) * 9 * ne);
    double *R = calloc((size_t)NEQ + 1, sizeof(double));
    double *Diag = calloc((size_t)NEQ + 1, sizeof(double)), *invDiag = calloc((size_t)NEQ + 1, sizeof(double));
    double *cond = calloc(5 * ne, sizeof(double)), *DaB = calloc(ne, sizeof(double));
    or_fill_lm(nel, 1, ien, type, invp, NEQ, lm);
    or_permutation_of_lm(nel, ien, type, invp, NEQ, Perm, invPerm, NULL);
    or_transport_problem pl = *prob;
    double *state = calloc(ne, sizeof(double));
    pl.delta_old = state;
    memset(uB, 0, sizeof(double) * ne);      /* Predictor_New.c:24,36 calloc uB and aB */
    memset(aB, 0, sizeof(double) * ne);
    or_time_opts t2 = *to;
    t2.scheme = OR_TIME_PREDICTOR;
    tt_loop2 c = { { { nel, NEQ, lm, Perm, invPerm, A, invDiag }, nnodes, nel, neq, x, y, type, invp, ien, &pl, R,
                     Diag, solver_tol, kmax, lmax }, uB, aB, cond, DaB };
    int steps = or_time_integrate_ex(neq, alpha, dt, &t2, tt_correct2, tt_predict2, &c, u, a, st);
    free(lm); free(Perm); free(invPerm); free(A); free(R); free(Diag); free(invDiag); free(state);
    free(cond); free(DaB);
    return steps;
}
