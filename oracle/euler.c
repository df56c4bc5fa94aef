/*
 * Compressible Euler, SUPG + CAU on P1 triangles with conservative
 * variables (rho, rho u, rho v, rho E): CPU restatement of
 * 03_Euler_Equations/2D/01_CommonFiles/Build_M_K_F_SUPG.c:6-1057 with
 * Ax_Ay_calculations.c:3-98, Delta_CAU.c:4-84, eval_U_dU.c:3-59 and
 * ebe_assembly.c, and of the predictor/multicorrector time loop of
 * 00_CommonFiles/Time_Integration/Predictor_Old.c:6-134 with the stop tests
 * of Criteria.c:3-80.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of the GPU library).
 *
 * The reference writes every product of the Jacobians (AxAx, AxAy, AyAx,
 * AyAy) and the convection blocks (b_i Ax + c_i Ay)/6 term by term, leaving
 * out the terms that multiply a structural zero of Ax and Ay.  Here they are
 * formed as plain 4x4 products and sums over k = 0..3: the extra terms are
 * exact zeros, and adding an exact zero leaves a sum unchanged, so every
 * entry rounds exactly as the reference's.  The one entry the reference
 * never sets, Ay[0][3] (Ax_Ay_calculations.c:33-36 sets Ay[0][0] twice), is
 * a structural zero it never reads; it is set to 0 here.
 * pow(x, 2) is kept where the reference uses it (tau, speed of sound).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "femoracle.h"

/* Jacobians of the Euler fluxes at the barycentric state Ub
 * (Ax_Ay_calculations.c: dimensionless :3-48, dimensional :50-98). */
static void eu_jacobians(double gamma, double mach, int dimensionless, const double Ub[4],
                         double Ax[4][4], double Ay[4][4])
{
    double v1 = Ub[1] / Ub[0], v2 = Ub[2] / Ub[0], E = Ub[3] / Ub[0];
    memset(Ax, 0, 16 * sizeof(double));
    memset(Ay, 0, 16 * sizeof(double));
    Ax[0][1] = 1.0;
    Ay[0][2] = 1.0;
    Ax[1][1] = (3.0 - gamma) * v1;
    Ax[1][2] = -(gamma - 1.0) * v2;
    Ax[2][0] = -v1 * v2;
    Ax[2][1] = v2;
    Ax[2][2] = v1;
    Ax[3][3] = gamma * v1;
    Ay[2][1] = -(gamma - 1.0) * v1;
    Ay[2][2] = (3.0 - gamma) * v2;
    Ay[3][3] = gamma * v2;
    if (dimensionless) {
        double nv = v1 * v1 + v2 * v2, e2 = mach * mach;
        Ax[1][0] = -(v1 * v1) + ((gamma - 1) * nv * 0.5);
        Ax[1][3] = (gamma - 1.0) / e2;
        Ax[3][0] = -v1 * (gamma * E - ((gamma - 1.0) * e2 * nv));
        Ax[3][1] = gamma * E - (gamma - 1.0) * e2 * (0.5 * nv + v1 * v1);
        Ax[3][2] = -(gamma - 1.0) * e2 * v1 * v2;
        Ay[2][0] = -(v2 * v2) + (((gamma - 1.0) * nv * 0.5));
        Ay[3][0] = -v2 * (gamma * E - (gamma - 1.0) * e2 * nv);
        Ay[3][2] = gamma * E - (gamma - 1.0) * e2 * (0.5 * nv + v2 * v2);
    } else {
        double rho = Ub[0], nU = (Ub[1] * Ub[1]) + (Ub[2] * Ub[2]);
        Ax[1][0] = -(v1 * v1) + (((gamma - 1) * nU * 0.5) / (rho * rho));
        Ax[1][3] = gamma - 1.0;
        Ax[3][0] = (-gamma * v1 * E) + ((gamma - 1.0) * v1 * (nU / (rho * rho)));
        Ax[3][1] = (gamma * E) - ((gamma - 1.0) * 0.5 * ((nU / (rho * rho)) + (2.0 * v1 * v1)));
        Ax[3][2] = -((gamma - 1.0) * v1 * v2);
        Ay[2][0] = -(v2 * v2) + (((gamma - 1.0) * nU * 0.5) / (rho * rho));
        Ay[3][0] = (-gamma * v2 * E) + (((gamma - 1.0) * v2 * nU) / (rho * rho));
        Ay[3][2] = (gamma * E) - ((gamma - 1.0) * 0.5 * ((nU / (rho * rho)) + (2.0 * v2 * v2)));
    }
    Ay[1][0] = Ax[2][0];
    Ay[1][1] = v2;
    Ay[1][2] = v1;
    Ay[2][3] = Ax[1][3];
    Ay[3][1] = Ax[3][2];
}

/* P = X Y, sums over k in ascending order */
static void mul4(double X[4][4], double Y[4][4], double P[4][4])
{
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            double s = X[r][0] * Y[0][c];
            for (int k = 1; k < 4; k++) s += X[r][k] * Y[k][c];
            P[r][c] = s;
        }
}

/* w^T A0^-1 w with the symmetric expansion of Delta_CAU.c:37-63 */
static double a0_norm2(double A0[4][4], const double w[4])
{
    return w[0] * (A0[0][0] * w[0] + 2.0 * A0[0][1] * w[1] + 2.0 * A0[0][2] * w[2] + 2.0 * A0[0][3] * w[3]) +
           w[1] * (A0[1][1] * w[1] + 2.0 * A0[1][2] * w[2] + 2.0 * A0[1][3] * w[3]) +
           w[2] * (A0[2][2] * w[2] + 2.0 * A0[2][3] * w[3]) +
           w[3] * A0[3][3] * w[3];
}

/* CAU shock-capturing coefficient (Delta_CAU.c:4-84) */
static double eu_delta_cau(double tolerance, const double gx[4], const double gy[4], double Ax[4][4],
                           double Ay[4][4], double A0[4][4], const double dUb[4], const double b[3],
                           const double c[3], double twoArea)
{
    double Agx[4], Agy[4], kx[4], ky[4], L[4];
    for (int r = 0; r < 4; r++) {
        double sx = Ax[r][0] * gx[0], sy = Ay[r][0] * gy[0];
        for (int k = 1; k < 4; k++) { sx += Ax[r][k] * gx[k]; sy += Ay[r][k] * gy[k]; }
        Agx[r] = sx;
        Agy[r] = sy;
    }
    for (int i = 0; i < 4; i++) {
        kx[i] = (b[0] * gx[i] + c[0] * gy[i]) / twoArea;
        ky[i] = (b[1] * gx[i] + c[1] * gy[i]) / twoArea;
    }
    double nk = sqrt(a0_norm2(A0, kx) + a0_norm2(A0, ky));
    for (int i = 0; i < 4; i++) L[i] = dUb[i] + Agx[i] + Agy[i];
    double nL = sqrt(a0_norm2(A0, L));
    double ng = sqrt(a0_norm2(A0, gx) + a0_norm2(A0, gy));
    return ng >= tolerance ? nL / nk : 0.0;
}

static double eu_delta_yz(const double invY[4], const double gx[4], const double gy[4], double Ax[4][4],
                          double Ay[4][4], const double dUb[4], const double b[3], const double c[3], double twoArea,
                          const double Ub[4], int nmv, double *old);
static const double eu_ones[4] = {1.0, 1.0, 1.0, 1.0};

/* One element: Ae = Me + alpha dt Ke (12x12, row-major) and Re = -Me dUe - Ke Ue. */
static void eu_element(const or_euler_problem *pb, const double X[3], const double Y[3], const double Ue[12],
                       const double dUe[12], double Ae[144], double Re[12])
{
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0;
    const double gamma = pb->gamma, alpha = pb->alpha, dt = pb->dt;
    double b[3] = {Y[1] - Y[2], Y[2] - Y[0], Y[0] - Y[1]};
    double c[3] = {X[2] - X[1], X[0] - X[2], X[1] - X[0]};
    double twoArea = fabs(c[2] * b[1] - c[1] * b[2]);
    double Area = 0.5 * twoArea;
    double Ub[4], dUb[4], gx[4], gy[4];
    int i, j, r, q;
    for (i = 0; i < 4; i++) {
        Ub[i] = (Ue[i] + Ue[i + 4] + Ue[i + 8]) * third;
        dUb[i] = (dUe[i] + dUe[i + 4] + dUe[i + 8]) * third;
    }
    for (i = 0; i < 4; i++) {
        gx[i] = (Ue[i] * b[0] + Ue[i + 4] * b[1] + Ue[i + 8] * b[2]) / twoArea;
        gy[i] = (Ue[i] * c[0] + Ue[i + 4] * c[1] + Ue[i + 8] * c[2]) / twoArea;
    }
    double v1 = Ub[1] / Ub[0], v2 = Ub[2] / Ub[0], E = Ub[3] / Ub[0];
    double nU = (Ub[1] * Ub[1]) + (Ub[2] * Ub[2]);
    double Ax[4][4], Ay[4][4];
    eu_jacobians(gamma, pb->mach, pb->dimensionless, Ub, Ax, Ay);

    /* inverse Riemannian metric A0^-1 in entropy variables (:131-158) */
    double rho_i = Ub[3] - ((nU * 0.5) / Ub[0]);
    double V2 = Ub[1] / rho_i, V3 = Ub[2] / rho_i, V4 = (-Ub[0]) / rho_i;
    double re = -1.0 / (rho_i * V4);
    double k1 = (V2 * V2 + V3 * V3) * 0.5 / V4;
    double A0[4][4];
    A0[0][0] = re * (k1 * k1 + gamma);
    A0[0][1] = re * (k1 * V2);
    A0[0][2] = re * (k1 * V3);
    A0[0][3] = re * ((k1 + 1.0) * V4);
    A0[1][1] = re * (V2 * V2 - V4);
    A0[1][2] = re * (V2 * V3);
    A0[1][3] = re * (V2 * V4);
    A0[2][2] = re * (V3 * V3 - V4);
    A0[2][3] = re * (V3 * V4);
    A0[3][3] = re * V4 * V4;
    A0[1][0] = A0[0][1]; A0[2][0] = A0[0][2]; A0[3][0] = A0[0][3];
    A0[2][1] = A0[1][2]; A0[3][1] = A0[1][3]; A0[3][2] = A0[2][3];

    /* AiAj products (:160-234) */
    double Axx[4][4], Axy[4][4], Ayx[4][4], Ayy[4][4];
    mul4(Ax, Ax, Axx);
    mul4(Ax, Ay, Axy);
    mul4(Ay, Ax, Ayx);
    mul4(Ay, Ay, Ayy);

    /* ShockCapture "CAU" (Delta_CAU) or "YZBeta" (Delta_YZBeta, setStabilizationForm.c:24-26) */
    double delta = pb->shock == 3
                       ? eu_delta_yz(pb->invY ? pb->invY : eu_ones, gx, gy, Ax, Ay, dUb, b, c, twoArea, Ub, 0, NULL)
                       : eu_delta_cau(pb->tolerance, gx, gy, Ax, Ay, A0, dUb, b, c, twoArea);

    /* SUPG tau (:240-269) */
    double betax = 2.0 * (gx[0] * Ub[0] + gx[1] * Ub[1] + gx[2] * Ub[2] + gx[3] * Ub[3]);
    double betay = 2.0 * (gy[0] * Ub[0] + gy[1] * Ub[1] + gy[2] * Ub[2] + gy[3] * Ub[3]);
    double betaxy = sqrt(betax * betax + betay * betay);
    if (betaxy != 0.0) { betax = betax / betaxy; betay = betay / betaxy; }
    double h = sqrt(twoArea);
    double avb = fabs(v1 * betax + v2 * betay);
    double cs = sqrt(gamma * (gamma - 1.0) * (E - 0.5 * (pow(v1, 2) + pow(v2, 2))));
    double CFL = ((cs + avb) * dt) / h;
    double psi = (2.0 * alpha * CFL) * (1.0 / (1.0 + 2.0 * alpha * CFL));
    double tau_d = delta / pow((cs + avb), 2);
    double tau_a = h / (2.0 * (cs + avb));
    double tau_t = (2.0 / (3.0 * (1.0 + 2.0 * alpha * CFL))) * tau_a;
    double tau = tau_t + psi * (tau_a - tau_d);
    if (tau < 0.0) tau = 0.0;

    /* convection blocks C_i = (b_i Ax + c_i Ay)/6 (Galerkin, :277-334) and
     * the SUPG blocks a_i^x = b_i AxAx + c_i AyAx, a_i^y = b_i AxAy + c_i AyAy (:610-733) */
    double C[3][4][4], ax[3][4][4], ay[3][4][4];
    for (i = 0; i < 3; i++)
        for (r = 0; r < 4; r++)
            for (q = 0; q < 4; q++) {
                C[i][r][q] = (b[i] * Ax[r][q] + c[i] * Ay[r][q]) * sixth;
                ax[i][r][q] = b[i] * Axx[r][q] + c[i] * Ayx[r][q];
                ay[i][r][q] = b[i] * Axy[r][q] + c[i] * Ayy[r][q];
            }
    double Mg1 = Area * sixth, Mg2 = Area / 12.0;
    double t4a = tau / (4 * Area);
    double d4a = delta / (4.0 * Area);
    double Kcau[3][3];
    for (i = 0; i < 3; i++)
        for (j = i + 1; j < 3; j++)
            Kcau[i][j] = Kcau[j][i] = d4a * (b[i] * b[j] + c[i] * c[j]);

    /* blocks (row node i, column node j) of Me (:349-561) and Ke (:770-1030) */
    double Me[12][12], Ke[12][12];
    for (i = 0; i < 3; i++) {
        int o1 = i == 0 ? 1 : 0, o2 = i == 2 ? 1 : 2;       /* the other two nodes, ascending */
        for (j = 0; j < 3; j++)
            for (r = 0; r < 4; r++)
                for (q = 0; q < 4; q++) {
                    double mpg = C[i][r][q] * tau;
                    Me[4 * i + r][4 * j + q] = r == q ? (i == j ? Mg1 : Mg2) + mpg : mpg;
                    double kg = C[j][r][q];
                    if (i == j) {
                        double p1 = t4a * (b[o1] * ax[i][r][q] + c[o1] * ay[i][r][q]);
                        double p2 = t4a * (b[o2] * ax[i][r][q] + c[o2] * ay[i][r][q]);
                        double k = kg - (p1 + p2);
                        Ke[4 * i + r][4 * j + q] = r == q ? k - (Kcau[i][o1] + Kcau[i][o2]) : k;
                    } else {
                        double p = t4a * (b[j] * ax[i][r][q] + c[j] * ay[i][r][q]);
                        Ke[4 * i + r][4 * j + q] = r == q ? kg + p + Kcau[i][j] : kg + p;
                    }
                }
    }
    /* local residual and the matrix of the corrector (:1033-1047) */
    double adt = alpha * dt;
    for (r = 0; r < 12; r++) {
        double m = 0, k = 0;
        for (q = 0; q < 12; q++) {
            m += Me[r][q] * dUe[q];
            k += Ke[r][q] * Ue[q];
            Ae[12 * r + q] = Me[r][q] + adt * Ke[r][q];
        }
        Re[r] = -m - k;
    }
}

/* Inverse Riemannian metric A0^-1 in entropy variables at Ub
 * (Build_M_K_F_DD_Transiente.c:132-158, the same as the SUPG build's). */
static void eu_a0inv(double gamma, const double Ub[4], double A0[4][4])
{
    double nU = (Ub[1] * Ub[1]) + (Ub[2] * Ub[2]);
    double rho_i = Ub[3] - ((nU * 0.5) / Ub[0]);
    double V2 = Ub[1] / rho_i, V3 = Ub[2] / rho_i, V4 = (-Ub[0]) / rho_i;
    double re = -1.0 / (rho_i * V4);
    double k1 = (V2 * V2 + V3 * V3) * 0.5 / V4;
    A0[0][0] = re * (k1 * k1 + gamma);
    A0[0][1] = re * (k1 * V2);
    A0[0][2] = re * (k1 * V3);
    A0[0][3] = re * ((k1 + 1.0) * V4);
    A0[1][1] = re * (V2 * V2 - V4);
    A0[1][2] = re * (V2 * V3);
    A0[1][3] = re * (V2 * V4);
    A0[2][2] = re * (V3 * V3 - V4);
    A0[2][3] = re * (V3 * V4);
    A0[3][3] = re * V4 * V4;
    A0[1][0] = A0[0][1]; A0[2][0] = A0[0][2]; A0[3][0] = A0[0][3];
    A0[2][1] = A0[1][2]; A0[3][1] = A0[1][3]; A0[3][2] = A0[2][3];
}

/* Delta_DD.c:4-89: the DD diffusion 0.5 |L U|_A0 / |grad_xi U|_A0 (0 below
 * the tolerance on |grad U|_A0), relaxed against the element's previous
 * value (w = 1/2, the relaxed value is kept), times sqrt(2 Area).  A_x grad
 * and A_y grad use the reference's term lists (rows with a structural zero
 * skip it). */
static double eu_delta_dd(double tolerance, double *delta_old, const double gx[4], const double gy[4],
                          double Ax[4][4], double Ay[4][4], double A0[4][4], const double dUb[4], const double b[3],
                          const double c[3], double twoArea)
{
    double Agx[4], Agy[4], kx[4], ky[4], L[4];
    Agx[0] = gx[1];
    Agx[1] = Ax[1][0] * gx[0] + Ax[1][1] * gx[1] + Ax[1][2] * gx[2] + Ax[1][3] * gx[3];
    Agx[2] = Ax[2][0] * gx[0] + Ax[2][1] * gx[1] + Ax[2][2] * gx[2];
    Agx[3] = Ax[3][0] * gx[0] + Ax[3][1] * gx[1] + Ax[3][2] * gx[2] + Ax[3][3] * gx[3];
    Agy[0] = gy[2];
    Agy[1] = Ay[1][0] * gy[0] + Ay[1][1] * gy[1] + Ay[1][2] * gy[2];
    Agy[2] = Ay[2][0] * gy[0] + Ay[2][1] * gy[1] + Ay[2][2] * gy[2] + Ay[2][3] * gy[3];
    Agy[3] = Ay[3][0] * gy[0] + Ay[3][1] * gy[1] + Ay[3][2] * gy[2] + Ay[3][3] * gy[3];
    for (int i = 0; i < 4; i++) {
        kx[i] = (b[0] * gx[i] + c[0] * gy[i]) / twoArea;
        ky[i] = (b[1] * gx[i] + c[1] * gy[i]) / twoArea;
    }
    double nk = sqrt(a0_norm2(A0, kx) + a0_norm2(A0, ky));
    for (int i = 0; i < 4; i++) L[i] = dUb[i] + Agx[i] + Agy[i];
    double nL = sqrt(a0_norm2(A0, L));
    double ng = sqrt(a0_norm2(A0, gx) + a0_norm2(A0, gy));
    double aux = ng >= tolerance ? 0.5 * nL / nk : 0.0;
    double w = 0.5;
    double delta = w * aux + (1 - w) * (*delta_old);
    *delta_old = delta;
    return delta * sqrt(twoArea);
}

/* Build_M_K_F_DD_Transiente.c:34-896 for one element: the Galerkin
 * convection blocks K_j = b_j Ax + c_j Ay, the DD diffusion, and the bubble
 * (4 unknowns) condensed with T = (MhB + dt KhB) (MBB + dt KBB)^-1:
 * Me = Mhh - T MhB, Ke = Khh - T KBh, Ne = (MhB - T MBB) / dt; Ae = Me +
 * alpha dt Ke, Re = -Me dUe - Ke Ue + Ne uB; the bubble state uB (4) and
 * delta_old are updated. */
static void eu_dd_element(const or_euler_problem *pb, const double X[3], const double Y[3], const double Ue[12],
                          const double dUe[12], double *uB, double *delta_old, double Ae[144], double Re[12])
{
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0, nf = 9.0 / 40.0;
    const double gamma = pb->gamma, alpha = pb->alpha, dt = pb->dt;
    double b[3] = {Y[1] - Y[2], Y[2] - Y[0], Y[0] - Y[1]};
    double c[3] = {X[2] - X[1], X[0] - X[2], X[1] - X[0]};
    double twoArea = fabs(c[2] * b[1] - c[1] * b[2]);
    double Area = 0.5 * twoArea;
    double Ub[4], dUb[4], gx[4], gy[4], uBaux[4];
    int i, j, r, q;
    for (i = 0; i < 4; i++) {
        Ub[i] = (Ue[i] + Ue[i + 4] + Ue[i + 8]) * third;
        dUb[i] = (dUe[i] + dUe[i + 4] + dUe[i + 8]) * third;
        uBaux[i] = uB[i];
    }
    for (i = 0; i < 4; i++) {
        gx[i] = (Ue[i] * b[0] + Ue[i + 4] * b[1] + Ue[i + 8] * b[2]) / twoArea;
        gy[i] = (Ue[i] * c[0] + Ue[i + 4] * c[1] + Ue[i + 8] * c[2]) / twoArea;
    }
    double Ax[4][4], Ay[4][4], A0[4][4];
    eu_jacobians(gamma, pb->mach, pb->dimensionless, Ub, Ax, Ay);
    eu_a0inv(gamma, Ub, A0);
    /* ShockCapture "CAUDD" (Delta_DD) or "YZBeta" (Delta_YZBeta, setStabilizationForm.c:64-66) */
    double delta = pb->shock == 3
                       ? eu_delta_yz(pb->invY ? pb->invY : eu_ones, gx, gy, Ax, Ay, dUb, b, c, twoArea, Ub, 0, NULL)
                       : eu_delta_dd(pb->tolerance, delta_old, gx, gy, Ax, Ay, A0, dUb, b, c, twoArea);

    double K[3][4][4], KhB[12][4], T[12][4];
    for (j = 0; j < 3; j++)
        for (r = 0; r < 4; r++)
            for (q = 0; q < 4; q++) K[j][r][q] = b[j] * Ax[r][q] + c[j] * Ay[r][q];
    double Mhh1 = Area * sixth, Mhh2 = Area / 12.0, MhB = (3.0 * Area) / 20.0, MBB = (81.0 * Area) / 280.0;
    double d4a = delta / (4.0 * Area);
    /* KhB rows of node i: p_i Ax + q_i Ay */
    double p[3] = {nf * (b[0] + 2.0 * b[1] + 2.0 * b[2]), nf * (2.0 * b[0] + b[1] + 2.0 * b[2]),
                   nf * (2.0 * b[0] + 2.0 * b[1] + b[2])};
    double pq[3] = {nf * (c[0] + 2.0 * c[1] + 2.0 * c[2]), nf * (2.0 * c[0] + c[1] + 2.0 * c[2]),
                    nf * (2.0 * c[0] + 2.0 * c[1] + c[2])};
    for (i = 0; i < 3; i++)
        for (r = 0; r < 4; r++)
            for (q = 0; q < 4; q++) KhB[4 * i + r][q] = p[i] * Ax[r][q] + pq[i] * Ay[r][q];
    double S = b[0] * b[0] + b[1] * b[1] + b[2] * b[2] + b[0] * b[1] + b[0] * b[2] + b[1] * b[2] + c[0] * c[0] +
               c[1] * c[1] + c[2] * c[2] + c[0] * c[1] + c[0] * c[2] + c[1] * c[2];
    double KBB = (81.0 * delta * S) / (40.0 * Area);
    double invBB = 1.0 / (MBB + dt * KBB);
    for (r = 0; r < 12; r++)
        for (q = 0; q < 4; q++)
            T[r][q] = (r & 3) == q ? invBB * (MhB + dt * KhB[r][q]) : invBB * dt * KhB[r][q];
    double invdt = 1.0 / dt, adt = alpha * dt;
    for (i = 0; i < 3; i++)
        for (r = 0; r < 4; r++) {
            const int row = 4 * i + r;
            double m = 0, k = 0;
            for (j = 0; j < 3; j++) {
                double dd = d4a * (b[i < j ? i : j] * b[i < j ? j : i] + c[i < j ? i : j] * c[i < j ? j : i]);
                for (q = 0; q < 4; q++) {
                    const int col = 4 * j + q;
                    double me = r == q ? (i == j ? Mhh1 : Mhh2) - T[row][q] * MhB : -T[row][q] * MhB;
                    double ke = K[j][r][q] * sixth;
                    if (r == q) ke = ke + dd;
                    for (int s = 0; s < 4; s++) ke = ke - T[row][s] * (nf * K[j][s][q]);
                    m += me * dUe[col];
                    k += ke * Ue[col];
                    Ae[12 * row + col] = me + adt * ke;
                }
            }
            double N = 0.0;
            for (q = 0; q < 4; q++) {
                double ne = r == q ? (MhB - T[row][q] * MBB) * invdt : (-T[row][q] * MBB) * invdt;
                N = q == 0 ? ne * uBaux[0] : N + ne * uBaux[q];
            }
            Re[row] = N + (-m - k);
        }
    /* the new bubble values (:878-889) */
    for (r = 0; r < 4; r++) {
        double s = (nf * K[0][r][0]) * Ue[0];
        for (int col = 1; col < 12; col++) s += (nf * K[col >> 2][r][col & 3]) * Ue[col];
        uB[r] = invBB * (MBB * uBaux[r] - dt * MhB * (dUe[r] + dUe[r + 4] + dUe[r + 8]) - dt * s);
    }
}

void or_build_euler(int nnodes, int nel, const double *x, const double *y, const int *type,
                    const int *invp, const int *ien, int neq, const or_euler_problem *prob,
                    const double *u, const double *du, double *A, double *R)
{
    int E, v, k, NEQ = neq;
    size_t nn = (size_t)(nnodes ? nnodes : 1);
    double *U = malloc(sizeof(double) * 4 * nn), *dU = malloc(sizeof(double) * 4 * nn);
    /* eval_U_dU.c:3-59 */
    for (v = 0; v < nnodes; v++)
        for (k = 0; k < 4; k++) {
            long d = 4L * v + k;
            if (type[d] > 0) { U[d] = u[invp[d]]; dU[d] = du[invp[d]]; }
            else { U[d] = prob->upresc[d]; dU[d] = 0.0; }
        }
    memset(R, 0, sizeof(double) * ((size_t)NEQ + 1));
    double *uB = prob->uB, *dold = prob->delta_old, *own = NULL;     /* DD state */
    if (prob->form == 1 && (!uB || !dold)) {
        own = calloc(5 * (size_t)(nel ? nel : 1), sizeof(double));
        uB = own;
        dold = own + 4 * (size_t)(nel ? nel : 1);
    }
    for (E = 0; E < nel; E++) {
        double X[3], Y[3], Ue[12], dUe[12], Re[12];
        int lm[12];
        for (v = 0; v < 3; v++) {
            int J = ien[3 * E + v];
            X[v] = x[J]; Y[v] = y[J];
            for (k = 0; k < 4; k++) {
                long d = 4L * J + k;
                Ue[4 * v + k] = U[d];
                dUe[4 * v + k] = dU[d];
                lm[4 * v + k] = type[d] == 0 ? NEQ : invp[d];
            }
        }
        if (prob->form == 1)
            eu_dd_element(prob, X, Y, Ue, dUe, uB + 4L * E, dold + E, A + 144L * E, Re);
        else
            eu_element(prob, X, Y, Ue, dUe, A + 144L * E, Re);
        for (k = 0; k < 12; k++) R[lm[k]] += Re[k];
        R[NEQ] = 0;
    }
    free(U); free(dU); free(own);
}

/* ---- Predictor_Old with EBE 12x12 blocks and BlockDiag (4x4) ---- */
typedef struct {
    int nel, nnodes, NEQ;
    const int *lm, *Id;
    const double *A, *inv;
} eu_ctx;

static int eu_mv_cb(void *p, double *P, double *Q)
{
    eu_ctx *c = (eu_ctx *)p;
    or_ebemv(c->nel, 12, c->lm, c->A, c->NEQ, P, Q);
    return 0;
}

static int eu_pc_cb(void *p, double *x, double *z)
{
    eu_ctx *c = (eu_ctx *)p;
    or_blockdiag_apply(c->nnodes, 4, c->Id, c->NEQ, c->inv, x, z);
    return 0;
}

typedef struct {
    eu_ctx mv;
    int nnodes, nel, neq;
    const double *x, *y;
    const int *type, *invp, *ien;
    const or_euler_problem *prob;
    double *R, *bd;
    double solver_tol;
    int kmax, lmax;
} eu_loop;

/* one correction: Build_M_K_F_SUPG at Alpha_Build / DeltaT_Build,
 * BlockDiag_precond_EBE_setup on R, pgmres for Da */
static int eu_correct(void *p, double alpha_b, double dt_b, const double *u, const double *a, double *Da, int *gi)
{
    eu_loop *c = (eu_loop *)p;
    or_euler_problem pb = *c->prob;
    pb.alpha = alpha_b;
    pb.dt = dt_b;
    or_build_euler(c->nnodes, c->nel, c->x, c->y, c->type, c->invp, c->ien, c->neq, &pb, u, a,
                   (double *)c->mv.A, c->R);
    or_blockdiag_setup(c->nnodes, c->nel, 4, c->ien, c->mv.A, c->mv.Id, c->neq, 1, c->bd, (double *)c->mv.inv, c->R);
    or_pgmres(c->neq, c->kmax, c->lmax, c->solver_tol, eu_mv_cb, eu_pc_cb, &c->mv, c->R, Da, gi);
    return 0;
}

int or_euler_predictor(int nnodes, int nel, const double *x, const double *y, const int *type,
                       const int *invp, const int *ien, int neq, const or_euler_problem *prob,
                       const or_time_opts *to, double solver_tol, int kmax, int lmax,
                       double *u, double *a, or_time_stats *st)
{
    int NEQ = neq, i;
    size_t ne = (size_t)(nel ? nel : 1), nn = (size_t)(nnodes ? nnodes : 1);
    int *lm = malloc(sizeof(int) * 12 * ne), *Id = malloc(sizeof(int) * 4 * nn);
    double *A = malloc(sizeof(double) * 144 * ne);
    double *R = calloc((size_t)NEQ + 1, sizeof(double));
    double *bd = malloc(sizeof(double) * 16 * nn), *inv = malloc(sizeof(double) * 16 * nn);
    or_fill_lm(nel, 4, ien, type, invp, NEQ, lm);
    for (i = 0; i < 4 * nnodes; i++) Id[i] = type[i] == 0 ? NEQ : invp[i];
    /* the DD state (uB, delta_old) lives for the whole loop (Predictor_Old.c:20-30) */
    or_euler_problem pl = *prob;
    double *state = calloc(5 * (size_t)(nel ? nel : 1), sizeof(double));
    pl.uB = state;
    pl.delta_old = state + 4 * (size_t)(nel ? nel : 1);
    eu_loop c = { { nel, nnodes, NEQ, lm, Id, A, inv }, nnodes, nel, neq, x, y, type, invp, ien, &pl, R, bd,
                  solver_tol, kmax, lmax };
    int steps = or_time_integrate(neq, prob->alpha, prob->dt, to, eu_correct, &c, u, a, st);
    free(lm); free(Id); free(A); free(R); free(bd); free(inv); free(state);
    return steps;
}

/* ---- TimeIntegration "Predictor2" with StabilizationForm "DD" and
 * ShockCapture "YZBeta" (setStabilizationForm.c:51-53, 64-66):
 * Build_M_F_DD_Transiente.c:6-821 keeps the four bubble unknowns of each
 * element (uB, duB) and condenses them out of the element system,
 * calculate_DaB.c:3-61 recovers their increments from Da, and
 * Predictor_New.c predicts and corrects them with u and a.  The build
 * passes an A0 it never computes to the shock capture (:137-138): with
 * "CAUDD" (Delta_DD, which reads A0) the result is undefined, so only
 * "YZBeta" (Delta_YZBeta, which does not) is restated.  The
 * no-penetrability adjustment (BC_no_penetrability) is the identity for
 * every problem but CYLINDER and NACA0012 (set_BC_no_penetrability.c). ---- */

/* Delta_YZBeta.c:4-104 (nmv = 0: 0.5 (delta1 + delta2), no state) or
 * Delta_YZBetaNMV.c:4-93 (nmv = 1: 0.5 delta1 relaxed against the element's
 * previous value with w = 1/2, the relaxed value kept; its pow(x, 1) is x) */
static double eu_delta_yz(const double invY[4], const double gx[4], const double gy[4], double Ax[4][4],
                          double Ay[4][4], const double dUb[4], const double b[3], const double c[3], double twoArea,
                          const double Ub[4], int nmv, double *old)
{
    double Agx[4], Agy[4], Z[4];
    Agx[0] = gx[1];
    Agx[1] = Ax[1][0] * gx[0] + Ax[1][1] * gx[1] + Ax[1][2] * gx[2] + Ax[1][3] * gx[3];
    Agx[2] = Ax[2][0] * gx[0] + Ax[2][1] * gx[1] + Ax[2][2] * gx[2];
    Agx[3] = Ax[3][0] * gx[0] + Ax[3][1] * gx[1] + Ax[3][2] * gx[2] + Ax[3][3] * gx[3];
    Agy[0] = gy[2];
    Agy[1] = Ay[1][0] * gy[0] + Ay[1][1] * gy[1] + Ay[1][2] * gy[2];
    Agy[2] = Ay[2][0] * gy[0] + Ay[2][1] * gy[1] + Ay[2][2] * gy[2] + Ay[2][3] * gy[3];
    Agy[3] = Ay[3][0] * gy[0] + Ay[3][1] * gy[1] + Ay[3][2] * gy[2] + Ay[3][3] * gy[3];
    for (int i = 0; i < 4; i++) Z[i] = dUb[i] + Agx[i] + Agy[i];
    double nYZ = sqrt(invY[0] * Z[0] * invY[0] * Z[0] + invY[1] * Z[1] * invY[1] * Z[1] +
                      invY[2] * Z[2] * invY[2] * Z[2] + invY[3] * Z[3] * invY[3] * Z[3]);
    double nx = invY[0] * gx[0] * invY[0] * gx[0] + invY[1] * gx[1] * invY[1] * gx[1] +
                invY[2] * gx[2] * invY[2] * gx[2] + invY[3] * gx[3] * invY[3] * gx[3];
    double ny = invY[0] * gy[0] * invY[0] * gy[0] + invY[1] * gy[1] * invY[1] * gy[1] +
                invY[2] * gy[2] * invY[2] * gy[2] + invY[3] * gy[3] * invY[3] * gy[3];
    double sum = nx + ny;
    double nYU = sqrt(invY[0] * Ub[0] * invY[0] * Ub[0] + invY[1] * Ub[1] * invY[1] * Ub[1] +
                      invY[2] * Ub[2] * invY[2] * Ub[2] + invY[3] * Ub[3] * invY[3] * Ub[3]);
    double ngr = sqrt(gx[0] * gx[0] + gy[0] * gy[0]), J1, J2;
    if (fabs(ngr) >= 1e-12) {
        J1 = gx[0] / ngr;
        J2 = gy[0] / ngr;
    } else {
        J1 = J2 = 0.0;
    }
    double H = (fabs(J1 * b[0] + J2 * c[0]) + fabs(J1 * b[1] + J2 * c[1]) + fabs(J1 * b[2] + J2 * c[2])) / twoArea;
    H = fabs(H) >= 1e-12 ? 2.0 * (1.0 / H) : 0.0;
    double as = fabs(sum) >= 1e-12 ? 1.0 / sqrt(sum) : 0.0;
    double au = fabs(nYU) >= 1e-12 ? 1.0 : 0.0;
    double d1 = nYZ * as * au * (H * 0.5);
    if (nmv) {
        double w = 0.5;
        double d = w * (0.5 * d1) + (1 - w) * (*old);
        *old = d;
        return d;
    }
    double as2 = fabs(sum) >= 1e-12 ? 1.0 : 0.0;
    double au2 = fabs(nYU) >= 1e-12 ? 1.0 / nYU : 0.0;
    double d2 = nYZ * as2 * au2 * (H * 0.5 * H * 0.5);
    return 0.5 * (d1 + d2);
}

/* Build_M_F_DD_Transiente.c:43-810 for one element.  Me is formed from the
 * matrices before the (identity) no-penetrability adjustment, as there. */
static void eu_mfdd_element(const or_euler_problem *pb, const double X[3], const double Y[3], const double Ue[12],
                            const double dUe[12], const double uB[4], const double duB[4], double *old_nmv,
                            double Me[144], double Fe[12], double cond[53])
{
    const double *invY = pb->invY ? pb->invY : eu_ones;
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0, nf = 9.0 / 40.0;
    double b[3] = {Y[1] - Y[2], Y[2] - Y[0], Y[0] - Y[1]};
    double c[3] = {X[2] - X[1], X[0] - X[2], X[1] - X[0]};
    double twoArea = fabs(c[2] * b[1] - c[1] * b[2]);
    double Area = 0.5 * twoArea;
    double Ub[4], dUb[4], gx[4], gy[4];
    int i, j, r, q, k;
    for (i = 0; i < 4; i++) {
        Ub[i] = (Ue[i] + Ue[i + 4] + Ue[i + 8]) * third;
        dUb[i] = (dUe[i] + dUe[i + 4] + dUe[i + 8]) * third;
    }
    for (i = 0; i < 4; i++) {
        gx[i] = (Ue[i] * b[0] + Ue[i + 4] * b[1] + Ue[i + 8] * b[2]) / twoArea;
        gy[i] = (Ue[i] * c[0] + Ue[i + 4] * c[1] + Ue[i + 8] * c[2]) / twoArea;
    }
    double Ax[4][4], Ay[4][4];
    eu_jacobians(pb->gamma, pb->mach, pb->dimensionless, Ub, Ax, Ay);
    double delta = eu_delta_yz(invY, gx, gy, Ax, Ay, dUb, b, c, twoArea, Ub, 0, NULL);
    double K[3][4][4];
    for (j = 0; j < 3; j++)
        for (r = 0; r < 4; r++)
            for (q = 0; q < 4; q++) K[j][r][q] = b[j] * Ax[r][q] + c[j] * Ay[r][q];
    double Mhh1 = Area * sixth, Mhh2 = Area / 12.0, MhB = (3.0 * Area) / 20.0, MBB = (81.0 * Area) / 280.0;
    double d4a = delta / (4.0 * Area);
    double p[3] = {nf * (b[0] + 2.0 * b[1] + 2.0 * b[2]), nf * (2.0 * b[0] + b[1] + 2.0 * b[2]),
                   nf * (2.0 * b[0] + 2.0 * b[1] + b[2])};
    double pq[3] = {nf * (c[0] + 2.0 * c[1] + 2.0 * c[2]), nf * (2.0 * c[0] + c[1] + 2.0 * c[2]),
                    nf * (2.0 * c[0] + 2.0 * c[1] + c[2])};
    double KhB[12][4], KBh[4][12], Khhg[4][12];
    for (i = 0; i < 3; i++)
        for (r = 0; r < 4; r++)
            for (q = 0; q < 4; q++) {
                KhB[4 * i + r][q] = p[i] * Ax[r][q] + pq[i] * Ay[r][q];
                KBh[r][4 * i + q] = nf * K[i][r][q];
                Khhg[r][4 * i + q] = K[i][r][q] * sixth;
            }
    double dnmv = eu_delta_yz(invY, gx, gy, Ax, Ay, dUb, b, c, twoArea, Ub, 1, old_nmv);
    double S = b[0] * b[0] + b[1] * b[1] + b[2] * b[2] + b[0] * b[1] + b[0] * b[2] + b[1] * b[2] + c[0] * c[0] +
               c[1] * c[1] + c[2] * c[2] + c[0] * c[1] + c[0] * c[2] + c[1] * c[2];
    double KBB = (81.0 * dnmv * S) / (40.0 * Area);
    double adt = pb->alpha * pb->dt;
    double M1[12][12], N1[12][4], M2[4][12];
    for (i = 0; i < 3; i++)
        for (j = 0; j < 3; j++) {
            const int lo = i < j ? i : j, hi = i < j ? j : i;
            double dd = d4a * (b[lo] * b[hi] + c[lo] * c[hi]);
            double mhh = i == j ? Mhh1 : Mhh2;
            for (r = 0; r < 4; r++)
                for (q = 0; q < 4; q++) {
                    double kg = Khhg[r][4 * j + q];
                    M1[4 * i + r][4 * j + q] = r == q ? mhh + adt * (kg + dd) : adt * kg;
                }
        }
    for (i = 0; i < 12; i++)
        for (q = 0; q < 4; q++) N1[i][q] = (i & 3) == q ? MhB + adt * KhB[i][q] : adt * KhB[i][q];
    for (r = 0; r < 4; r++)
        for (j = 0; j < 12; j++) M2[r][j] = (j & 3) == r ? MhB + adt * KBh[r][j] : adt * KBh[r][j];
    double invN2 = 1.0 / (MBB + adt * KBB);
    for (i = 0; i < 12; i++)                  /* :692-701 */
        for (j = 0; j < 12; j++) {
            double soma = 0.0;
            for (k = 0; k < 4; k++) soma += N1[i][k] * M2[k][j];
            Me[12 * i + j] = M1[i][j] - invN2 * soma;
        }
    double R1[12], R2[4];
    for (i = 0; i < 3; i++)                   /* :719-760 */
        for (r = 0; r < 4; r++) {
            const int row = 4 * i + r;
            R1[row] = -MhB * duB[r] - (KhB[row][0] * uB[0] + KhB[row][1] * uB[1] + KhB[row][2] * uB[2] +
                                       KhB[row][3] * uB[3]);
            double kh = 0.0;
            for (int col = 0; col < 12; col++) {
                const int jb = col >> 2;
                const int lo = i < jb ? i : jb, hi = i < jb ? jb : i;
                double coef = Khhg[r][col];
                if ((col & 3) == r) coef = d4a * (b[lo] * b[hi] + c[lo] * c[hi]) + coef;
                kh = col == 0 ? coef * Ue[0] : kh + coef * Ue[col];
            }
            double m = (i == 0 ? Mhh1 : Mhh2) * dUe[r] + (i == 1 ? Mhh1 : Mhh2) * dUe[4 + r] +
                       (i == 2 ? Mhh1 : Mhh2) * dUe[8 + r];
            R1[row] += -m - kh;
        }
    for (r = 0; r < 4; r++) {                 /* :764-781 */
        R2[r] = -MBB * duB[r] - KBB * uB[r];
        double kb = KBh[r][0] * Ue[0];
        for (int col = 1; col < 12; col++) kb += KBh[r][col] * Ue[col];
        R2[r] += -(MhB * dUe[r] + MhB * dUe[4 + r] + MhB * dUe[8 + r]) - kb;
    }
    for (i = 0; i < 12; i++)                  /* :789-790 */
        Fe[i] = R1[i] - invN2 * (N1[i][0] * R2[0] + N1[i][1] * R2[1] + N1[i][2] * R2[2] + N1[i][3] * R2[3]);
    cond[0] = invN2;
    for (r = 0; r < 4; r++) cond[1 + r] = R2[r];
    for (r = 0; r < 4; r++)
        for (j = 0; j < 12; j++) cond[5 + 12 * r + j] = M2[r][j];
}

void or_build_euler_mfdd(int nnodes, int nel, const double *x, const double *y, const int *type,
                         const int *invp, const int *ien, int neq, const or_euler_problem *prob,
                         const double *u, const double *du, const double *uB, const double *duB, double *dnmv,
                         double *A, double *F, double *cond)
{
    int E, v, k, NEQ = neq;
    size_t nn = (size_t)(nnodes ? nnodes : 1);
    double *U = malloc(sizeof(double) * 4 * nn), *dU = malloc(sizeof(double) * 4 * nn), *own = NULL;
    for (v = 0; v < nnodes; v++)              /* eval_U_dU.c:3-59 */
        for (k = 0; k < 4; k++) {
            long d = 4L * v + k;
            if (type[d] > 0) { U[d] = u[invp[d]]; dU[d] = du[invp[d]]; }
            else { U[d] = prob->upresc[d]; dU[d] = 0.0; }
        }
    if (!dnmv) dnmv = own = calloc((size_t)(nel ? nel : 1), sizeof(double));
    memset(F, 0, sizeof(double) * ((size_t)NEQ + 1));
    for (E = 0; E < nel; E++) {
        double X[3], Y[3], Ue[12], dUe[12], Fe[12];
        int lm[12];
        for (v = 0; v < 3; v++) {
            int J = ien[3 * E + v];
            X[v] = x[J]; Y[v] = y[J];
            for (k = 0; k < 4; k++) {
                long d = 4L * J + k;
                Ue[4 * v + k] = U[d];
                dUe[4 * v + k] = dU[d];
                lm[4 * v + k] = type[d] == 0 ? NEQ : invp[d];
            }
        }
        eu_mfdd_element(prob, X, Y, Ue, dUe, uB + 4L * E, duB + 4L * E, dnmv + E, A + 144L * E, Fe, cond + 53L * E);
        for (k = 0; k < 12; k++) F[lm[k]] += Fe[k];
        F[NEQ] = 0;
    }
    free(U); free(dU); free(own);
}

void or_euler_dab(int nel, const int *lm, int NEQ, const double *cond, double *Da, double *DaB)
{
    Da[NEQ] = 0.0;                            /* calculate_DaB.c:18-57 */
    for (int e = 0; e < nel; e++) {
        const double *cd = cond + 53L * e;
        const int *l = lm + 12L * e;
        for (int r = 0; r < 4; r++) {
            const double *m = cd + 5 + 12 * r;
            double s = m[0] * Da[l[0]];
            for (int j = 1; j < 12; j++) s += m[j] * Da[l[j]];
            DaB[4L * e + r] = cd[0] * (cd[1 + r] - s);
        }
    }
}

typedef struct {
    eu_loop base;
    double *uB, *aB, *cond, *DaB, *dnmv;
    int *lm12;
    double *uB1, *uB2;         /* uB_old (TR-BDF2) or uB1 (BDF); uB2 (BDF) */
} eu_loop2;

/* uB_InitialSolution.c:3-111: each element's four bubble values are the
 * centroid averages of its nodal state.  The reference tests a prescribed
 * dof by invP_id != NEQ, while Preprocess.c:173 marks them with -1, so it
 * reads u[-1] there; the prescribed value its other branch names is used. */
static void eu_ub_initial(const eu_loop *b, const double *u, double *uB)
{
    const double third = 1.0 / 3.0;
    for (int e = 0; e < b->nel; e++) {
        double Ue[12];
        for (int v = 0; v < 3; v++) {
            const int J = b->ien[3 * e + v];
            for (int k = 0; k < 4; k++) {
                const long d = 4L * J + k;
                Ue[4 * v + k] = b->type[d] > 0 ? u[b->invp[d]] : b->prob->upresc[d];
            }
        }
        for (int i = 0; i < 4; i++) uB[4L * e + i] = (Ue[i] + Ue[i + 4] + Ue[i + 8]) * third;
    }
}

static void eu_bubble2(void *p, int op, double c1, double c2, const double *u)
{
    eu_loop2 *c = (eu_loop2 *)p;
    const size_t m = 4 * (size_t)c->base.nel;
    size_t i;
    switch (op) {
    case OR_B_PREDICT:                        /* Predictor_New.c:82-83, _TRBDF2.c:91-92 */
        for (i = 0; i < m; i++) c->uB[i] += c1 * c->aB[i];
        memset(c->aB, 0, sizeof(double) * m);
        break;
    case OR_B_TRBDF2_START:                   /* Predictor_New_TRBDF2.c:63 */
        eu_ub_initial(&c->base, u, c->uB);
        break;
    case OR_B_TRBDF2_COMBINE:                 /* :151-154 */
        for (i = 0; i < m; i++) {
            c->uB[i] = c1 * c->uB[i] - c2 * c->uB1[i];
            c->aB[i] = 0.0;
        }
        break;
    case OR_B_TRBDF2_SAVE:                    /* :192 */
    case OR_B_BDF_START:                      /* Predictor_New_BDF.c:77-78 */
        memcpy(c->uB1, c->uB, sizeof(double) * m);
        if (op == OR_B_BDF_START) memset(c->aB, 0, sizeof(double) * m);
        break;
    case OR_B_BDF_SAVE2:                      /* :111 */
        memcpy(c->uB2, c->uB, sizeof(double) * m);
        break;
    case OR_B_BDF_COMBINE:                    /* :139-142 */
        for (i = 0; i < m; i++) {
            c->uB[i] = c1 * c->uB2[i] - c2 * c->uB1[i];
            c->aB[i] = 0.0;
        }
        break;
    case OR_B_BDF_SHIFT:                      /* :177-178 */
        memcpy(c->uB1, c->uB2, sizeof(double) * m);
        memcpy(c->uB2, c->uB, sizeof(double) * m);
        break;
    }
}

static int eu_correct2(void *p, double alpha_b, double dt_b, const double *u, const double *a, double *Da, int *gi)
{
    eu_loop2 *c = (eu_loop2 *)p;
    eu_loop *b = &c->base;
    or_euler_problem pb = *b->prob;
    pb.alpha = alpha_b;
    pb.dt = dt_b;
    or_build_euler_mfdd(b->nnodes, b->nel, b->x, b->y, b->type, b->invp, b->ien, b->neq, &pb, u, a, c->uB, c->aB,
                        c->dnmv, (double *)b->mv.A, b->R, c->cond);
    or_blockdiag_setup(b->nnodes, b->nel, 4, b->ien, b->mv.A, b->mv.Id, b->neq, 1, b->bd, (double *)b->mv.inv, b->R);
    or_pgmres(b->neq, b->kmax, b->lmax, b->solver_tol, eu_mv_cb, eu_pc_cb, &b->mv, b->R, Da, gi);
    or_euler_dab(b->nel, c->lm12, b->neq, c->cond, Da, c->DaB);      /* :99 */
    const double coef = alpha_b * dt_b;
    size_t m = 4 * (size_t)b->nel;
    for (size_t i = 0; i < m; i++) {                                  /* :104-105 */
        c->aB[i] += c->DaB[i];
        c->uB[i] += coef * c->DaB[i];
    }
    return 0;
}

int or_euler_predictor2(int nnodes, int nel, const double *x, const double *y, const int *type,
                        const int *invp, const int *ien, int neq, const or_euler_problem *prob,
                        const or_time_opts *to, double solver_tol, int kmax, int lmax,
                        double *u, double *a, double *uB, double *aB, or_time_stats *st)
{
    int NEQ = neq, i;
    size_t ne = (size_t)(nel ? nel : 1), nn = (size_t)(nnodes ? nnodes : 1);
    int *lm = malloc(sizeof(int) * 12 * ne), *Id = malloc(sizeof(int) * 4 * nn);
    double *A = malloc(sizeof(double) * 144 * ne);
    double *R = calloc((size_t)NEQ + 1, sizeof(double));
    double *bd = malloc(sizeof(double) * 16 * nn), *inv = malloc(sizeof(double) * 16 * nn);
    double *cond = calloc(53 * ne, sizeof(double)), *DaB = calloc(4 * ne, sizeof(double));
    double *dnmv = calloc(ne, sizeof(double));
    double *uB1 = calloc(4 * ne, sizeof(double)), *uB2 = calloc(4 * ne, sizeof(double));
    or_fill_lm(nel, 4, ien, type, invp, NEQ, lm);
    for (i = 0; i < 4 * nnodes; i++) Id[i] = type[i] == 0 ? NEQ : invp[i];
    memset(uB, 0, sizeof(double) * 4 * ne);  /* Predictor_New.c:24,36 calloc uB and aB */
    memset(aB, 0, sizeof(double) * 4 * ne);
    or_time_opts t2 = *to;                   /* Predictor_New, _BDF or _TRBDF2 */
    if (t2.scheme != OR_TIME_NEW_BDF && t2.scheme != OR_TIME_TRBDF2) t2.scheme = OR_TIME_PREDICTOR;
    eu_loop2 c = { { { nel, nnodes, NEQ, lm, Id, A, inv }, nnodes, nel, neq, x, y, type, invp, ien, prob, R, bd,
                     solver_tol, kmax, lmax }, uB, aB, cond, DaB, dnmv, lm, uB1, uB2 };
    int steps = or_time_integrate_ex(neq, prob->alpha, prob->dt, &t2, eu_correct2, eu_bubble2, &c, u, a, st);
    free(lm); free(Id); free(A); free(R); free(bd); free(inv); free(cond); free(DaB); free(dnmv);
    free(uB1); free(uB2);
    return steps;
}
