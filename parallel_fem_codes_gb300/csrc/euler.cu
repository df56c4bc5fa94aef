// Compressible Euler on the device: the SUPG + CAU element build of
// 03_Euler_Equations/2D/01_CommonFiles/Build_M_K_F_SUPG.c:6-1057 with
// Ax_Ay_calculations.c, Delta_CAU.c, eval_U_dU.c and ebe_assembly.c.
//
// k_euler_elem is one thread per element (internal element order).  It
// gathers the nodal state (rho, rho u, rho v, rho E) and its time derivative
// (prescribed values and zero for Dirichlet dofs), forms the barycentric
// Jacobians Ax, Ay, the metric A0^-1, the CAU coefficient and the SUPG tau,
// and then writes the 12x12 block Me + alpha dt Ke row by row together with
// the element residual -Me dUe - Ke Ue.  The entries of Me and Ke are formed
// on the fly from Ax and Ay (the rows of the products AxAx, AxAy, AyAx, AyAy
// are recomputed per block row), which keeps about 80 doubles live instead
// of the reference's ~600 named temporaries.
//
// Bit-exactness: the reference writes the Jacobian products and the blocks
// (b_i Ax + c_i Ay)/6 term by term without the terms that multiply a
// structural zero of Ax or Ay; here they are plain 4x4 products and sums over
// k = 0..3, whose extra terms are exact zeros (adding an exact zero leaves a
// sum unchanged).  Ay[0][3], which the reference never sets and never reads,
// is 0.  Every other expression keeps the reference's order and association;
// the unit is compiled with -fmad=false.  pow(x, 2) is evaluated as x * x
// (pow's result for an exponent of 2 is the correctly rounded square).
#include "system.h"

namespace fg {

__device__ __forceinline__ void eu_jacobians(const fg_euler_coeffs &cf, const double Ub[4], double Ax[4][4],
                                             double Ay[4][4])
{
    const double gamma = cf.gamma;
    const double v1 = Ub[1] / Ub[0], v2 = Ub[2] / Ub[0], E = Ub[3] / Ub[0];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) { Ax[r][q] = 0.0; Ay[r][q] = 0.0; }
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
    if (cf.dimensionless) {
        const double nv = v1 * v1 + v2 * v2, e2 = cf.mach * cf.mach;
        Ax[1][0] = -(v1 * v1) + ((gamma - 1) * nv * 0.5);
        Ax[1][3] = (gamma - 1.0) / e2;
        Ax[3][0] = -v1 * (gamma * E - ((gamma - 1.0) * e2 * nv));
        Ax[3][1] = gamma * E - (gamma - 1.0) * e2 * (0.5 * nv + v1 * v1);
        Ax[3][2] = -(gamma - 1.0) * e2 * v1 * v2;
        Ay[2][0] = -(v2 * v2) + (((gamma - 1.0) * nv * 0.5));
        Ay[3][0] = -v2 * (gamma * E - (gamma - 1.0) * e2 * nv);
        Ay[3][2] = gamma * E - (gamma - 1.0) * e2 * (0.5 * nv + v2 * v2);
    } else {
        const double rho = Ub[0], nU = (Ub[1] * Ub[1]) + (Ub[2] * Ub[2]);
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

__device__ double eu_delta_yz(const double invY[4], const double gx[4], const double gy[4], const double Ax[4][4],
                              const double Ay[4][4], const double dUb[4], const double b[3], const double c[3],
                              double twoArea, const double Ub[4], int nmv, double *old);

// w^T A0^-1 w, symmetric expansion of Delta_CAU.c:37-63 (A0 upper triangle)
__device__ __forceinline__ double a0_norm2(const double A0[10], const double w[4])
{
    // A0: 00 01 02 03 11 12 13 22 23 33
    return w[0] * (A0[0] * w[0] + 2.0 * A0[1] * w[1] + 2.0 * A0[2] * w[2] + 2.0 * A0[3] * w[3]) +
           w[1] * (A0[4] * w[1] + 2.0 * A0[5] * w[2] + 2.0 * A0[6] * w[3]) +
           w[2] * (A0[7] * w[2] + 2.0 * A0[8] * w[3]) +
           w[3] * A0[9] * w[3];
}

__global__ void __launch_bounds__(128) k_euler_elem(int nel, int ld, int n, const int *__restrict__ gien,
                                                    const double *__restrict__ gx, const double *__restrict__ gy,
                                                    const int *__restrict__ node_dof, const double *__restrict__ up,
                                                    const double *__restrict__ u, const double *__restrict__ du,
                                                    fg_euler_coeffs cf, double *__restrict__ A64,
                                                    double *__restrict__ Fe)
{
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0;
    const double gamma = cf.gamma;
    double X[3], Y[3], Ue[12], dUe[12];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const int J = gien[(size_t)v * ld + pos];
        X[v] = gx[J];
        Y[v] = gy[J];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int d = node_dof[4 * J + k];
            const bool dir = d == n;
            Ue[4 * v + k] = dir ? up[4 * J + k] : u[d];
            dUe[4 * v + k] = dir ? 0.0 : du[d];
        }
    }
    const double b[3] = {Y[1] - Y[2], Y[2] - Y[0], Y[0] - Y[1]};
    const double c[3] = {X[2] - X[1], X[0] - X[2], X[1] - X[0]};
    const double twoArea = fabs(c[2] * b[1] - c[1] * b[2]);
    const double Area = 0.5 * twoArea;
    double Ub[4], dUb[4], gxu[4], gyu[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        Ub[i] = (Ue[i] + Ue[i + 4] + Ue[i + 8]) * third;
        dUb[i] = (dUe[i] + dUe[i + 4] + dUe[i + 8]) * third;
        gxu[i] = (Ue[i] * b[0] + Ue[i + 4] * b[1] + Ue[i + 8] * b[2]) / twoArea;
        gyu[i] = (Ue[i] * c[0] + Ue[i + 4] * c[1] + Ue[i + 8] * c[2]) / twoArea;
    }
    const double v1 = Ub[1] / Ub[0], v2 = Ub[2] / Ub[0], E = Ub[3] / Ub[0];
    const double nU = (Ub[1] * Ub[1]) + (Ub[2] * Ub[2]);
    double Ax[4][4], Ay[4][4];
    eu_jacobians(cf, Ub, Ax, Ay);

    // A0^-1 (Build_M_K_F_SUPG.c:131-158), upper triangle; ShockCapture "CAU"
    // or "YZBeta" (Delta_YZBeta with invY)
    double delta;
    if (cf.shock == FG_SHOCK_YZBETA) {
        delta = eu_delta_yz(cf.invY, gxu, gyu, Ax, Ay, dUb, b, c, twoArea, Ub, 0, nullptr);
    } else {
        const double rho_i = Ub[3] - ((nU * 0.5) / Ub[0]);
        const double V2 = Ub[1] / rho_i, V3 = Ub[2] / rho_i, V4 = (-Ub[0]) / rho_i;
        const double re = -1.0 / (rho_i * V4);
        const double k1 = (V2 * V2 + V3 * V3) * 0.5 / V4;
        const double A0[10] = {re * (k1 * k1 + gamma), re * (k1 * V2),      re * (k1 * V3), re * ((k1 + 1.0) * V4),
                               re * (V2 * V2 - V4),    re * (V2 * V3),      re * (V2 * V4), re * (V3 * V3 - V4),
                               re * (V3 * V4),         re * V4 * V4};
        // CAU (Delta_CAU.c:4-84)
        double kx[4], ky[4], L[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            double sx = Ax[r][0] * gxu[0], sy = Ay[r][0] * gyu[0];
#pragma unroll
            for (int k = 1; k < 4; ++k) { sx += Ax[r][k] * gxu[k]; sy += Ay[r][k] * gyu[k]; }
            L[r] = dUb[r] + sx + sy;
            kx[r] = (b[0] * gxu[r] + c[0] * gyu[r]) / twoArea;
            ky[r] = (b[1] * gxu[r] + c[1] * gyu[r]) / twoArea;
        }
        const double nk = sqrt(a0_norm2(A0, kx) + a0_norm2(A0, ky));
        const double nL = sqrt(a0_norm2(A0, L));
        const double ng = sqrt(a0_norm2(A0, gxu) + a0_norm2(A0, gyu));
        delta = ng >= cf.tolerance ? nL / nk : 0.0;
    }

    // SUPG tau (:240-269)
    double tau;
    {
        double betax = 2.0 * (gxu[0] * Ub[0] + gxu[1] * Ub[1] + gxu[2] * Ub[2] + gxu[3] * Ub[3]);
        double betay = 2.0 * (gyu[0] * Ub[0] + gyu[1] * Ub[1] + gyu[2] * Ub[2] + gyu[3] * Ub[3]);
        const double betaxy = sqrt(betax * betax + betay * betay);
        if (betaxy != 0.0) { betax = betax / betaxy; betay = betay / betaxy; }
        const double h = sqrt(twoArea);
        const double avb = fabs(v1 * betax + v2 * betay);
        const double cs = sqrt(gamma * (gamma - 1.0) * (E - 0.5 * (v1 * v1 + v2 * v2)));
        const double CFL = ((cs + avb) * cf.dt) / h;
        const double psi = (2.0 * cf.alpha * CFL) * (1.0 / (1.0 + 2.0 * cf.alpha * CFL));
        const double cv = cs + avb;
        const double tau_d = delta / (cv * cv);
        const double tau_a = h / (2.0 * (cs + avb));
        const double tau_t = (2.0 / (3.0 * (1.0 + 2.0 * cf.alpha * CFL))) * tau_a;
        tau = tau_t + psi * (tau_a - tau_d);
        if (tau < 0.0) tau = 0.0;
    }

    const double Mg1 = Area * sixth, Mg2 = Area / 12.0;
    const double t4a = tau / (4 * Area);
    const double d4a = delta / (4.0 * Area);
    const double Kc01 = d4a * (b[0] * b[1] + c[0] * c[1]);
    const double Kc02 = d4a * (b[0] * b[2] + c[0] * c[2]);
    const double Kc12 = d4a * (b[1] * b[2] + c[1] * c[2]);
    const double adt = cf.alpha * cf.dt;
    double *a = A64 + pos;
    double *fe = Fe + pos;
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        const int o1 = i == 0 ? 1 : 0, o2 = i == 2 ? 1 : 2;     // the other two nodes, ascending
        const double kcd = i == 0 ? Kc01 + Kc02 : i == 1 ? Kc01 + Kc12 : Kc02 + Kc12;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            // row r of AxAx, AxAy, AyAx, AyAy (sums over k ascending)
            double pxx[4], pxy[4], pyx[4], pyy[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                double s1 = Ax[r][0] * Ax[0][q], s2 = Ax[r][0] * Ay[0][q];
                double s3 = Ay[r][0] * Ax[0][q], s4 = Ay[r][0] * Ay[0][q];
#pragma unroll
                for (int k = 1; k < 4; ++k) {
                    s1 += Ax[r][k] * Ax[k][q];
                    s2 += Ax[r][k] * Ay[k][q];
                    s3 += Ay[r][k] * Ax[k][q];
                    s4 += Ay[r][k] * Ay[k][q];
                }
                pxx[q] = s1; pxy[q] = s2; pyx[q] = s3; pyy[q] = s4;
            }
            const int R = 4 * i + r;
            double m = 0, k = 0;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const double kij = j == i ? 0.0 : (i + j == 1 ? Kc01 : i + j == 2 ? Kc02 : Kc12);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const double Ci = (b[i] * Ax[r][q] + c[i] * Ay[r][q]) * sixth;
                    const double mpg = Ci * tau;
                    const double Me = r == q ? (i == j ? Mg1 : Mg2) + mpg : mpg;
                    const double kg = (b[j] * Ax[r][q] + c[j] * Ay[r][q]) * sixth;
                    const double ax = b[i] * pxx[q] + c[i] * pyx[q];
                    const double ay = b[i] * pxy[q] + c[i] * pyy[q];
                    double Ke;
                    if (i == j) {
                        const double p1 = t4a * (b[o1] * ax + c[o1] * ay);
                        const double p2 = t4a * (b[o2] * ax + c[o2] * ay);
                        const double kk = kg - (p1 + p2);
                        Ke = r == q ? kk - kcd : kk;
                    } else {
                        const double p = t4a * (b[j] * ax + c[j] * ay);
                        Ke = r == q ? kg + p + kij : kg + p;
                    }
                    const int Q = 4 * j + q;
                    m += Me * dUe[Q];
                    k += Ke * Ue[Q];
                    a[(size_t)(R * 12 + Q) * ld] = Me + adt * Ke;
                }
            }
            fe[(size_t)R * ld] = -m - k;
        }
    }
}

// ---------------------------------------------------------------- DD form
// Build_M_K_F_DD_Transiente.c:34-896 with Delta_DD.c:4-89.  Per element:
// K_j = b_j Ax + c_j Ay (Galerkin convection, K_j / 6 in every row block),
// the DD diffusion delta / (4 Area) (b_i b_j + c_i c_j) on the dof diagonal,
// and the bubble condensed with T = (MhB + dt KhB) / (MBB + dt KBB) (KhB
// rows of node i: p_i Ax + q_i Ay; KBh = 9/40 K_j): Me = Mhh - T MhB,
// Ke = Khh - T KBh, Ne = (MhB - T MBB) / dt; Ae = Me + alpha dt Ke; the
// residual row is Ne uB + (-Me dUe - Ke Ue); the bubble values uB and the
// relaxed delta are element state (internal order) updated here.  K_j, KhB
// and T are recomputed where used (same operands, same rounding) instead of
// held in registers.  Ax_Ay_calculations.c leaves Ay[0][3] unassigned and the
// reference reads it here; eu_jacobians gives it its value, 0.
__device__ __forceinline__ double eu_kj(const double Ax[4][4], const double Ay[4][4], double bj, double cj, int r, int q)
{
    return bj * Ax[r][q] + cj * Ay[r][q];
}

__global__ void __launch_bounds__(128) k_euler_dd_elem(int nel, int ld, int n, const int *__restrict__ gien,
                                                       const double *__restrict__ gx, const double *__restrict__ gy,
                                                       const int *__restrict__ node_dof,
                                                       const double *__restrict__ up, const double *__restrict__ u,
                                                       const double *__restrict__ du, fg_euler_coeffs cf,
                                                       double *delta_old, double *uB, double *__restrict__ A64,
                                                       double *__restrict__ Fe)
{
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0, nf = 9.0 / 40.0;
    const double gamma = cf.gamma, dt = cf.dt;
    double X[3], Y[3], Ue[12], dUe[12];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const int J = gien[(size_t)v * ld + pos];
        X[v] = gx[J];
        Y[v] = gy[J];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int d = node_dof[4 * J + k];
            const bool dir = d == n;
            Ue[4 * v + k] = dir ? up[4 * J + k] : u[d];
            dUe[4 * v + k] = dir ? 0.0 : du[d];
        }
    }
    const double b[3] = {Y[1] - Y[2], Y[2] - Y[0], Y[0] - Y[1]};
    const double c[3] = {X[2] - X[1], X[0] - X[2], X[1] - X[0]};
    const double twoArea = fabs(c[2] * b[1] - c[1] * b[2]);
    const double Area = 0.5 * twoArea;
    double Ub[4], dUb[4], gxu[4], gyu[4], uBaux[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        Ub[i] = (Ue[i] + Ue[i + 4] + Ue[i + 8]) * third;
        dUb[i] = (dUe[i] + dUe[i + 4] + dUe[i + 8]) * third;
        gxu[i] = (Ue[i] * b[0] + Ue[i + 4] * b[1] + Ue[i + 8] * b[2]) / twoArea;
        gyu[i] = (Ue[i] * c[0] + Ue[i + 4] * c[1] + Ue[i + 8] * c[2]) / twoArea;
        uBaux[i] = uB[(size_t)i * ld + pos];
    }
    const double nU = (Ub[1] * Ub[1]) + (Ub[2] * Ub[2]);
    double Ax[4][4], Ay[4][4];
    eu_jacobians(cf, Ub, Ax, Ay);
    double delta;
    if (cf.shock == FG_SHOCK_YZBETA) {   // ShockCapture "YZBeta": Delta_YZBeta, no state
        delta = eu_delta_yz(cf.invY, gxu, gyu, Ax, Ay, dUb, b, c, twoArea, Ub, 0, nullptr);
    } else {   // Delta_DD.c: A0^-1 norms, relaxed (w = 1/2), times sqrt(2 Area)
        const double rho_i = Ub[3] - ((nU * 0.5) / Ub[0]);
        const double V2 = Ub[1] / rho_i, V3 = Ub[2] / rho_i, V4 = (-Ub[0]) / rho_i;
        const double re = -1.0 / (rho_i * V4);
        const double k1 = (V2 * V2 + V3 * V3) * 0.5 / V4;
        const double A0[10] = {re * (k1 * k1 + gamma), re * (k1 * V2),      re * (k1 * V3), re * ((k1 + 1.0) * V4),
                               re * (V2 * V2 - V4),    re * (V2 * V3),      re * (V2 * V4), re * (V3 * V3 - V4),
                               re * (V3 * V4),         re * V4 * V4};
        double Agx[4], Agy[4], kx[4], ky[4], L[4];
        Agx[0] = gxu[1];
        Agx[1] = Ax[1][0] * gxu[0] + Ax[1][1] * gxu[1] + Ax[1][2] * gxu[2] + Ax[1][3] * gxu[3];
        Agx[2] = Ax[2][0] * gxu[0] + Ax[2][1] * gxu[1] + Ax[2][2] * gxu[2];
        Agx[3] = Ax[3][0] * gxu[0] + Ax[3][1] * gxu[1] + Ax[3][2] * gxu[2] + Ax[3][3] * gxu[3];
        Agy[0] = gyu[2];
        Agy[1] = Ay[1][0] * gyu[0] + Ay[1][1] * gyu[1] + Ay[1][2] * gyu[2];
        Agy[2] = Ay[2][0] * gyu[0] + Ay[2][1] * gyu[1] + Ay[2][2] * gyu[2] + Ay[2][3] * gyu[3];
        Agy[3] = Ay[3][0] * gyu[0] + Ay[3][1] * gyu[1] + Ay[3][2] * gyu[2] + Ay[3][3] * gyu[3];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            kx[i] = (b[0] * gxu[i] + c[0] * gyu[i]) / twoArea;
            ky[i] = (b[1] * gxu[i] + c[1] * gyu[i]) / twoArea;
            L[i] = dUb[i] + Agx[i] + Agy[i];
        }
        const double nk = sqrt(a0_norm2(A0, kx) + a0_norm2(A0, ky));
        const double nL = sqrt(a0_norm2(A0, L));
        const double ng = sqrt(a0_norm2(A0, gxu) + a0_norm2(A0, gyu));
        const double aux = ng >= cf.tolerance ? 0.5 * nL / nk : 0.0;
        const double w = 0.5;
        double d = w * aux + (1 - w) * delta_old[pos];
        delta_old[pos] = d;
        delta = d * sqrt(twoArea);
    }
    const double Mhh1 = Area * sixth, Mhh2 = Area / 12.0, MhB = (3.0 * Area) / 20.0, MBB = (81.0 * Area) / 280.0;
    const double d4a = delta / (4.0 * Area);
    const double p[3] = {nf * (b[0] + 2.0 * b[1] + 2.0 * b[2]), nf * (2.0 * b[0] + b[1] + 2.0 * b[2]),
                         nf * (2.0 * b[0] + 2.0 * b[1] + b[2])};
    const double pq[3] = {nf * (c[0] + 2.0 * c[1] + 2.0 * c[2]), nf * (2.0 * c[0] + c[1] + 2.0 * c[2]),
                          nf * (2.0 * c[0] + 2.0 * c[1] + c[2])};
    const double S = b[0] * b[0] + b[1] * b[1] + b[2] * b[2] + b[0] * b[1] + b[0] * b[2] + b[1] * b[2] + c[0] * c[0] +
                     c[1] * c[1] + c[2] * c[2] + c[0] * c[1] + c[0] * c[2] + c[1] * c[2];
    const double KBB = (81.0 * delta * S) / (40.0 * Area);
    const double invBB = 1.0 / (MBB + dt * KBB);
    const double invdt = 1.0 / dt, adt = cf.alpha * dt;
    double *a = A64 + pos;
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
#pragma unroll 1
        for (int r = 0; r < 4; ++r) {
            const int row = 4 * i + r;
            double T[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const double khb = p[i] * Ax[r][q] + pq[i] * Ay[r][q];
                T[q] = r == q ? invBB * (MhB + dt * khb) : invBB * dt * khb;
            }
            double m = 0.0, k = 0.0;
#pragma unroll 1
            for (int j = 0; j < 3; ++j) {
                const int lo = i < j ? i : j, hi = i < j ? j : i;
                const double dd = d4a * (b[lo] * b[hi] + c[lo] * c[hi]);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int col = 4 * j + q;
                    const double me = r == q ? (i == j ? Mhh1 : Mhh2) - T[q] * MhB : -T[q] * MhB;
                    double ke = eu_kj(Ax, Ay, b[j], c[j], r, q) * sixth;
                    if (r == q) ke = ke + dd;
#pragma unroll
                    for (int s2 = 0; s2 < 4; ++s2) ke = ke - T[s2] * (nf * eu_kj(Ax, Ay, b[j], c[j], s2, q));
                    m += me * dUe[col];
                    k += ke * Ue[col];
                    a[(size_t)(12 * row + col) * ld] = me + adt * ke;
                }
            }
            double N = 0.0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const double ne = r == q ? (MhB - T[q] * MBB) * invdt : (-T[q] * MBB) * invdt;
                N = q == 0 ? ne * uBaux[0] : N + ne * uBaux[q];
            }
            Fe[(size_t)row * ld + pos] = N + (-m - k);
        }
    }
    // the new bubble values (:878-889)
#pragma unroll 1
    for (int r = 0; r < 4; ++r) {
        double s = (nf * eu_kj(Ax, Ay, b[0], c[0], r, 0)) * Ue[0];
#pragma unroll
        for (int col = 1; col < 12; ++col) s += (nf * eu_kj(Ax, Ay, b[col >> 2], c[col >> 2], r, col & 3)) * Ue[col];
        uB[(size_t)r * ld + pos] = invBB * (MBB * uBaux[r] - dt * MhB * (dUe[r] + dUe[r + 4] + dUe[r + 8]) - dt * s);
    }
}

// Delta_YZBeta.c:4-104 (nmv = 0: 0.5 (delta1 + delta2), no state) or
// Delta_YZBetaNMV.c:4-93 (nmv = 1: 0.5 delta1 relaxed against *old with
// w = 1/2, the relaxed value kept; its pow(x, 1) is x).  A_x grad and A_y
// grad use the reference's term lists.
__device__ double eu_delta_yz(const double invY[4], const double gx[4], const double gy[4], const double Ax[4][4],
                              const double Ay[4][4], const double dUb[4], const double b[3], const double c[3],
                              double twoArea, const double Ub[4], int nmv, double *old)
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
#pragma unroll
    for (int i = 0; i < 4; ++i) Z[i] = dUb[i] + Agx[i] + Agy[i];
    const double nYZ = sqrt(invY[0] * Z[0] * invY[0] * Z[0] + invY[1] * Z[1] * invY[1] * Z[1] +
                            invY[2] * Z[2] * invY[2] * Z[2] + invY[3] * Z[3] * invY[3] * Z[3]);
    const double nx = invY[0] * gx[0] * invY[0] * gx[0] + invY[1] * gx[1] * invY[1] * gx[1] +
                      invY[2] * gx[2] * invY[2] * gx[2] + invY[3] * gx[3] * invY[3] * gx[3];
    const double ny = invY[0] * gy[0] * invY[0] * gy[0] + invY[1] * gy[1] * invY[1] * gy[1] +
                      invY[2] * gy[2] * invY[2] * gy[2] + invY[3] * gy[3] * invY[3] * gy[3];
    const double sum = nx + ny;
    const double nYU = sqrt(invY[0] * Ub[0] * invY[0] * Ub[0] + invY[1] * Ub[1] * invY[1] * Ub[1] +
                            invY[2] * Ub[2] * invY[2] * Ub[2] + invY[3] * Ub[3] * invY[3] * Ub[3]);
    const double ngr = sqrt(gx[0] * gx[0] + gy[0] * gy[0]);
    double J1 = 0.0, J2 = 0.0;
    if (fabs(ngr) >= 1e-12) {
        J1 = gx[0] / ngr;
        J2 = gy[0] / ngr;
    }
    double H = (fabs(J1 * b[0] + J2 * c[0]) + fabs(J1 * b[1] + J2 * c[1]) + fabs(J1 * b[2] + J2 * c[2])) / twoArea;
    H = fabs(H) >= 1e-12 ? 2.0 * (1.0 / H) : 0.0;
    const double as = fabs(sum) >= 1e-12 ? 1.0 / sqrt(sum) : 0.0;
    const double au = fabs(nYU) >= 1e-12 ? 1.0 : 0.0;
    const double d1 = nYZ * as * au * (H * 0.5);
    if (nmv) {
        const double w = 0.5;
        const double d = w * (0.5 * d1) + (1 - w) * (*old);
        *old = d;
        return d;
    }
    const double as2 = fabs(sum) >= 1e-12 ? 1.0 : 0.0;
    const double au2 = fabs(nYU) >= 1e-12 ? 1.0 / nYU : 0.0;
    const double d2 = nYZ * as2 * au2 * (H * 0.5 * H * 0.5);
    return 0.5 * (d1 + d2);
}

// Build_M_F_DD_Transiente.c:43-810 ("Predictor2", DD, YZBeta), a thread per
// element (internal position pos).  The four bubble unknowns (uB, duB) are
// condensed out of the element system with N2 = MBB + alpha dt KBB: the
// block Me = M1 - N1 M2 / N2 (formed, as there, before the no-penetrability
// adjustment, which is the identity here), the load R1 - N1 R2 / N2 into Fe
// (12 planes), and invN2, R2, M2 into the bubble planes for the correction.
// The entries of M1, N1 and M2 are formed on the fly from Ax, Ay and the
// edge vectors, each with the reference's expression.  Bubble planes (stride
// ld): 0-3 uB, 4-7 aB (duB), 8 invN2, 9-12 R2, 13-60 M2 (4 x 12), 61
// Delta_YZBetaNMV's relaxed state.
__global__ void __launch_bounds__(128) k_euler_mfdd_elem(int nel, int ld, int n, const int *__restrict__ gien,
                                                         const double *__restrict__ gx, const double *__restrict__ gy,
                                                         const int *__restrict__ node_dof,
                                                         const double *__restrict__ up, const double *__restrict__ u,
                                                         const double *__restrict__ du, fg_euler_coeffs cf,
                                                         double *__restrict__ bub, double *__restrict__ A64,
                                                         double *__restrict__ Fe)
{
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0, nf = 9.0 / 40.0;
    double X[3], Y[3], Ue[12], dUe[12];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const int J = gien[(size_t)v * ld + pos];
        X[v] = gx[J];
        Y[v] = gy[J];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int d = node_dof[4 * J + k];
            const bool dir = d == n;
            Ue[4 * v + k] = dir ? up[4 * J + k] : u[d];
            dUe[4 * v + k] = dir ? 0.0 : du[d];
        }
    }
    const double b[3] = {Y[1] - Y[2], Y[2] - Y[0], Y[0] - Y[1]};
    const double c[3] = {X[2] - X[1], X[0] - X[2], X[1] - X[0]};
    const double twoArea = fabs(c[2] * b[1] - c[1] * b[2]);
    const double Area = 0.5 * twoArea;
    double Ub[4], dUb[4], gxu[4], gyu[4], uB[4], duB[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        Ub[i] = (Ue[i] + Ue[i + 4] + Ue[i + 8]) * third;
        dUb[i] = (dUe[i] + dUe[i + 4] + dUe[i + 8]) * third;
        gxu[i] = (Ue[i] * b[0] + Ue[i + 4] * b[1] + Ue[i + 8] * b[2]) / twoArea;
        gyu[i] = (Ue[i] * c[0] + Ue[i + 4] * c[1] + Ue[i + 8] * c[2]) / twoArea;
        uB[i] = bub[(size_t)i * ld + pos];
        duB[i] = bub[(size_t)(4 + i) * ld + pos];
    }
    double Ax[4][4], Ay[4][4];
    eu_jacobians(cf, Ub, Ax, Ay);
    const double delta = eu_delta_yz(cf.invY, gxu, gyu, Ax, Ay, dUb, b, c, twoArea, Ub, 0, nullptr);
    const double Mhh1 = Area * sixth, Mhh2 = Area / 12.0, MhB = (3.0 * Area) / 20.0, MBB = (81.0 * Area) / 280.0;
    const double d4a = delta / (4.0 * Area);
    const double p[3] = {nf * (b[0] + 2.0 * b[1] + 2.0 * b[2]), nf * (2.0 * b[0] + b[1] + 2.0 * b[2]),
                         nf * (2.0 * b[0] + 2.0 * b[1] + b[2])};
    const double pq[3] = {nf * (c[0] + 2.0 * c[1] + 2.0 * c[2]), nf * (2.0 * c[0] + c[1] + 2.0 * c[2]),
                          nf * (2.0 * c[0] + 2.0 * c[1] + c[2])};
    double *old = bub + (size_t)61 * ld + pos;
    double onmv = *old;
    const double dnmv = eu_delta_yz(cf.invY, gxu, gyu, Ax, Ay, dUb, b, c, twoArea, Ub, 1, &onmv);
    *old = onmv;
    const double S = b[0] * b[0] + b[1] * b[1] + b[2] * b[2] + b[0] * b[1] + b[0] * b[2] + b[1] * b[2] + c[0] * c[0] +
                     c[1] * c[1] + c[2] * c[2] + c[0] * c[1] + c[0] * c[2] + c[1] * c[2];
    const double KBB = (81.0 * dnmv * S) / (40.0 * Area);
    const double adt = cf.alpha * cf.dt;
    const double invN2 = 1.0 / (MBB + adt * KBB);
    // M2[r][col] = (MhB +) adt nf (b_j Ax + c_j Ay)[r][q]; N1[row][q] = (MhB +) adt (p_i Ax + pq_i Ay)[r][q]
    auto m2 = [&](int r, int col) {
        const int j = col >> 2, q = col & 3;
        const double kbh = nf * (b[j] * Ax[r][q] + c[j] * Ay[r][q]);
        return q == r ? MhB + adt * kbh : adt * kbh;
    };
    auto khb = [&](int i, int r, int q) { return p[i] * Ax[r][q] + pq[i] * Ay[r][q]; };
    auto n1 = [&](int i, int r, int q) { return r == q ? MhB + adt * khb(i, r, q) : adt * khb(i, r, q); };
    // R2 (:764-781)
    double R2[4];
#pragma unroll 1
    for (int r = 0; r < 4; ++r) {
        R2[r] = -MBB * duB[r] - KBB * uB[r];
        double kb = (nf * (b[0] * Ax[r][0] + c[0] * Ay[r][0])) * Ue[0];
#pragma unroll
        for (int col = 1; col < 12; ++col) {
            const int j = col >> 2, q = col & 3;
            kb += (nf * (b[j] * Ax[r][q] + c[j] * Ay[r][q])) * Ue[col];
        }
        R2[r] += -(MhB * dUe[r] + MhB * dUe[4 + r] + MhB * dUe[8 + r]) - kb;
    }
    double *a = A64 + pos;
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
#pragma unroll 1
        for (int r = 0; r < 4; ++r) {
            const int row = 4 * i + r;
            double N1r[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) N1r[q] = n1(i, r, q);
            double kh = 0.0;
#pragma unroll 1
            for (int j = 0; j < 3; ++j) {
                const int lo = i < j ? i : j, hi = i < j ? j : i;
                const double dd = d4a * (b[lo] * b[hi] + c[lo] * c[hi]);
                const double mhh = i == j ? Mhh1 : Mhh2;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int col = 4 * j + q;
                    const double kg = (b[j] * Ax[r][q] + c[j] * Ay[r][q]) * sixth;
                    const double m1 = r == q ? mhh + adt * (kg + dd) : adt * kg;
                    double soma = 0.0;
#pragma unroll
                    for (int k = 0; k < 4; ++k) soma += N1r[k] * m2(k, col);
                    a[(size_t)(12 * row + col) * ld] = m1 - invN2 * soma;
                    const double coef = r == q ? dd + kg : kg;
                    kh = col == 0 ? coef * Ue[0] : kh + coef * Ue[col];
                }
            }
            const double KhBr0 = khb(i, r, 0), KhBr1 = khb(i, r, 1), KhBr2 = khb(i, r, 2), KhBr3 = khb(i, r, 3);
            double R1 = -MhB * duB[r] - (KhBr0 * uB[0] + KhBr1 * uB[1] + KhBr2 * uB[2] + KhBr3 * uB[3]);
            const double m = (i == 0 ? Mhh1 : Mhh2) * dUe[r] + (i == 1 ? Mhh1 : Mhh2) * dUe[4 + r] +
                             (i == 2 ? Mhh1 : Mhh2) * dUe[8 + r];
            R1 += -m - kh;
            Fe[(size_t)row * ld + pos] =
                R1 - invN2 * (N1r[0] * R2[0] + N1r[1] * R2[1] + N1r[2] * R2[2] + N1r[3] * R2[3]);
        }
    }
    bub[(size_t)8 * ld + pos] = invN2;
#pragma unroll
    for (int r = 0; r < 4; ++r) bub[(size_t)(9 + r) * ld + pos] = R2[r];
#pragma unroll 1
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int col = 0; col < 12; ++col) bub[(size_t)(13 + 12 * r + col) * ld + pos] = m2(r, col);
}

// calculate_DaB.c:18-57 from the solve's Da (internal numbering; Dirichlet
// dofs read 0 as Da[NEQ] = 0 there), then Predictor_New.c:104-105 (update:
// aB += DaB, uB += coef DaB) or DaB into out[r * ld + pos] (!update)
__global__ void k_euler_bubble_correct(int nel, int ld, int n, const int *__restrict__ gien,
                                       const int *__restrict__ node_dof, const double *__restrict__ Da, double coef,
                                       int update, double *__restrict__ bub, double *__restrict__ out)
{
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    double d[12];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const int J = gien[(size_t)v * ld + pos];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int q = node_dof[4 * J + k];
            d[4 * v + k] = q == n ? 0.0 : Da[q];
        }
    }
    const double invN2 = bub[(size_t)8 * ld + pos];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const double *m = bub + (size_t)(13 + 12 * r) * ld + pos;
        double s = m[0] * d[0];
#pragma unroll
        for (int j = 1; j < 12; ++j) s += m[(size_t)j * ld] * d[j];
        const double DaB = invN2 * (bub[(size_t)(9 + r) * ld + pos] - s);
        if (update) {
            bub[(size_t)(4 + r) * ld + pos] += DaB;
            bub[(size_t)r * ld + pos] += coef * DaB;
        } else {
            out[(size_t)r * ld + pos] = DaB;
        }
    }
}

// The bubble steps of Predictor_New.c, Predictor_New_BDF.c and
// Predictor_New_TRBDF2.c on the four unknowns of each element (BubbleOp;
// planes 0-3 uB, 4-7 aB, 62-65 uB_old / uB1, 66-69 uB2).  kBubbleTrStart
// is uB_InitialSolution.c: the element centroids of the state, prescribed
// dofs taking their prescribed values.
__global__ void k_euler_bubble_op(int nel, int ld, int n, int op, double c1, double c2,
                                  const int *__restrict__ gien, const int *__restrict__ node_dof,
                                  const double *__restrict__ up, const double *__restrict__ u,
                                  double *__restrict__ bub)
{
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const double third = 1.0 / 3.0;
    double Ue[12];
    if (op == kBubbleTrStart) {
#pragma unroll
        for (int v = 0; v < 3; ++v) {
            const int J = gien[(size_t)v * ld + pos];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int d = node_dof[4 * J + k];
                Ue[4 * v + k] = d == n ? up[4 * J + k] : u[d];
            }
        }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        double *uB = bub + (size_t)r * ld + pos, *aB = bub + (size_t)(4 + r) * ld + pos;
        double *o1 = bub + (size_t)(62 + r) * ld + pos, *o2 = bub + (size_t)(66 + r) * ld + pos;
        switch (op) {
        case kBubblePredict: *uB += c1 * *aB; *aB = 0.0; break;
        case kBubbleTrStart: *uB = (Ue[r] + Ue[r + 4] + Ue[r + 8]) * third; break;
        case kBubbleTrCombine: *uB = c1 * *uB - c2 * *o1; *aB = 0.0; break;
        case kBubbleTrSave: *o1 = *uB; break;
        case kBubbleBdfStart: *o1 = *uB; *aB = 0.0; break;
        case kBubbleBdfSave2: *o2 = *uB; break;
        case kBubbleBdfCombine: *uB = c1 * *o2 - c2 * *o1; *aB = 0.0; break;
        case kBubbleBdfShift: *o1 = *o2; *o2 = *uB; break;
        default: break;
        }
    }
}

int euler_mfdd_assemble_device(fg_system *s, const fg_euler_coeffs *c, const double *u_dev, const double *du_dev,
                               double *F_dev, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (t.ndof != 4) { set_error("Euler assembly needs ndof == 4"); return FG_ERR_UNSUPPORTED; }
    if (!s->eu_geometry_ok) { set_error("Euler assembly before fg_euler_set_geometry"); return FG_ERR_STATE; }
    if (c->form != FG_EULER_DD) { set_error("Euler Predictor2 builds the DD form (FG_EULER_DD)"); return FG_ERR_ARG; }
    int r = bubble_alloc(s, 4);
    if (r) return r;
    if (t.nel > 0)
        k_euler_mfdd_elem<<<(t.nel + 127) / 128, 128, 0, st>>>(t.nel, s->nel_pad, t.n, s->gien.as<int>(),
                                                              s->gx.as<double>(), s->gy.as<double>(),
                                                              s->node_dof.as<int>(), s->gup.as<double>(), u_dev,
                                                              du_dev, *c, s->bubble.as<double>(), s->A64.as<double>(),
                                                              s->Fe.as<double>());
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    if ((r = gather_residual(s, s->Fe.as<double>(), F_dev, st))) return r;
    s->blocks_ok = true;
    s->csr_dirty = true;
    return convert_blocks(s, st);
}

int euler_bubble_correct_device(fg_system *s, const double *Da_dev, double coef, double *DaB_dev, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (s->bubble_nb != 4) { set_error("no Euler Predictor2 build on this system"); return FG_ERR_STATE; }
    if (t.nel > 0) {
        k_euler_bubble_correct<<<(t.nel + 255) / 256, 256, 0, st>>>(t.nel, s->nel_pad, t.n, s->gien.as<int>(),
                                                                   s->node_dof.as<int>(), Da_dev, coef,
                                                                   DaB_dev ? 0 : 1, s->bubble.as<double>(), DaB_dev);
        FG_CUDA(cudaGetLastError());
        count_launches(1);
    }
    return FG_OK;
}

int euler_bubble_op_device(fg_system *s, int op, double c1, double c2, const double *u_dev, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (s->bubble_nb != 4) { set_error("no Euler Predictor2 build on this system"); return FG_ERR_STATE; }
    if (op < kBubblePredict || op > kBubbleBdfShift) { set_error("unknown bubble step"); return FG_ERR_ARG; }
    if (t.nel > 0) {
        k_euler_bubble_op<<<(t.nel + 255) / 256, 256, 0, st>>>(t.nel, s->nel_pad, t.n, op, c1, c2, s->gien.as<int>(),
                                                              s->node_dof.as<int>(), s->gup.as<double>(), u_dev,
                                                              s->bubble.as<double>());
        FG_CUDA(cudaGetLastError());
        count_launches(1);
    }
    return FG_OK;
}

int euler_assemble_device(fg_system *s, const fg_euler_coeffs *c, const double *u_dev, const double *du_dev,
                          double *R_dev, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (t.ndof != 4) { set_error("Euler assembly needs ndof == 4"); return FG_ERR_UNSUPPORTED; }
    if (!s->eu_geometry_ok) { set_error("Euler assembly before fg_euler_set_geometry"); return FG_ERR_STATE; }
    if (c->form != FG_EULER_SUPG && c->form != FG_EULER_DD) {
        set_error("Euler form must be FG_EULER_SUPG or FG_EULER_DD");
        return FG_ERR_ARG;
    }
    if (c->shock != 0 && c->shock != FG_SHOCK_YZBETA) {
        set_error("Euler shock capture must be 0 (the form's own) or FG_SHOCK_YZBETA");
        return FG_ERR_ARG;
    }
    if (c->form == FG_EULER_DD) {   // element state: delta_old [nel_pad], uB [4][nel_pad]
        int r0;
        if (s->shock_state.bytes < 40 * (size_t)s->nel_pad && (r0 = s->shock_state.alloc(40 * (size_t)s->nel_pad)))
            return r0;
        if (t.nel > 0)
            k_euler_dd_elem<<<(t.nel + 127) / 128, 128, 0, st>>>(t.nel, s->nel_pad, t.n, s->gien.as<int>(),
                                                                s->gx.as<double>(), s->gy.as<double>(),
                                                                s->node_dof.as<int>(), s->gup.as<double>(), u_dev,
                                                                du_dev, *c, s->shock_state.as<double>(),
                                                                s->shock_state.as<double>() + s->nel_pad,
                                                                s->A64.as<double>(), s->Fe.as<double>());
    } else if (t.nel > 0)
        k_euler_elem<<<(t.nel + 127) / 128, 128, 0, st>>>(t.nel, s->nel_pad, t.n, s->gien.as<int>(),
                                                         s->gx.as<double>(), s->gy.as<double>(),
                                                         s->node_dof.as<int>(), s->gup.as<double>(), u_dev, du_dev,
                                                         *c, s->A64.as<double>(), s->Fe.as<double>());
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    int r = gather_residual(s, s->Fe.as<double>(), R_dev, st);
    if (r) return r;
    s->blocks_ok = true;
    s->csr_dirty = true;
    return convert_blocks(s, st);
}

}  // namespace fg
