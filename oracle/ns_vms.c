/*
 * Steady incompressible Navier-Stokes, VMS-DCDD form (variational multiscale
 * with a condensed bubble enrichment, LSIC grad-div term): CPU restatement of
 * 04_SS_NavierStokes_Equations/2D/01_CommonFiles/Build_K_F_VMS_DCDD.c:8-716
 * (the same file serves 05_NavierStokes_Equations), with eval_U.c and
 * ebe_assembly.c.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of the GPU library).
 *
 * Velocity dofs of the element are numbered r = 2 i + d (node i, d = 0: x,
 * 1: y); g_r is the gradient coefficient of dof r (b_i = y23, y31, y12 for
 * x, c_i = x32, x13, x21 for y).  The bubble is condensed through the 2x2
 * inverse W = (K_BB)^-1 (:398-419) with NBh_i = 9/40 (ux b_i + uy c_i),
 * NhB = -NBh and GBh = -9/40 (b; c):
 *   Ndelta(r, s) = (NhB_i W[d][e]) NBh_j                  r = (i,d), s = (j,e)
 *   Gdelta(r, k) = (NhB_i W[d][0]) GBh0_k + (NhB_i W[d][1]) GBh1_k
 *   Gphi(k, m)   = GBh0_m (GBh0_k W00 + GBh1_k W01) + GBh1_m (GBh0_k W01 + GBh1_k W11)
 * Every product and sum is associated as the reference writes it.  What the
 * reference does and this file keeps:
 *   - the tangent holds Ndelta only in the same-direction blocks, from the
 *     upper triangle (Ndelta(min, max)), while the residual uses the full
 *     Ndelta; the (node 2 x, node 1 x) entry adds Ndelta where the others
 *     subtract it (:645);
 *   - the pressure block of the tangent uses the upper triangle of Gphi,
 *     the residual the full Gphi;
 *   - the artificial diffusion delta is 0 (:388-394), and the source is 0
 *     (f1 = f2 = fxB = fyB = 0, :289), so Fe = 0 and the residual is -(...);
 *   - h = sqrt(4 Area / PI) with PI = 3.14159265359 (the header's macro),
 *     tau_LSIC = 0.5 h |u|, density 1 (its factors are exact and left out).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "femoracle.h"

#define VMS_PI 3.14159265359

static void vms_element(const double X[3], const double Y[3], const double Ue[9], double Re, double Ke[81],
                        double Res[9])
{
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0, nf = 9.0 / 40.0;
    double b[3], c[3], g[6];
    int i, j, d, e, k, m;
    b[0] = Y[1] - Y[2]; b[1] = Y[2] - Y[0]; b[2] = Y[0] - Y[1];
    c[0] = X[2] - X[1]; c[1] = X[0] - X[2]; c[2] = X[1] - X[0];
    for (i = 0; i < 3; i++) { g[2 * i] = b[i]; g[2 * i + 1] = c[i]; }
    const double TwoA = fabs(c[2] * b[1] - c[1] * b[2]);
    const double Area = 0.5 * TwoA, invArea = 1.0 / Area, hi = 0.5 * invArea;
    const double ux1 = Ue[0], uy1 = Ue[1], p1 = Ue[2], ux2 = Ue[3], uy2 = Ue[4], p2 = Ue[5];
    const double ux3 = Ue[6], uy3 = Ue[7], p3 = Ue[8];
    const double uvec[6] = { ux1, uy1, ux2, uy2, ux3, uy3 }, pvec[3] = { p1, p2, p3 };
    const double ux = third * (ux1 + ux2 + ux3), uy = third * (uy1 + uy2 + uy3);
    const double duxdx = hi * (ux1 * b[0] + ux2 * b[1] + ux3 * b[2]);
    const double duxdy = hi * (ux1 * c[0] + ux2 * c[1] + ux3 * c[2]);
    const double duydx = hi * (uy1 * b[0] + uy2 * b[1] + uy3 * b[2]);
    const double duydy = hi * (uy1 * c[0] + uy2 * c[1] + uy3 * c[2]);
    const double duxduy = ux1 * b[0] + uy1 * c[0] + ux2 * b[1] + uy2 * c[1] + ux3 * b[2] + uy3 * c[2];
    const double p = third * (p1 + p2 + p3);
    double C[3];
    for (i = 0; i < 3; i++) C[i] = hi * (ux * b[i] + uy * c[i]);
    const double h = sqrt(4 * Area / VMS_PI);
    const double visc = 1. / Re;
    const double unorm = sqrt(ux * ux + uy * uy);
    const double tau_l = 0.5 * h * unorm;
    const double ks = tau_l * 0.25 * invArea;              /* LSIC scale            */
    const double kv = visc * 0.25 * invArea;               /* viscous scale         */

    /* condensed bubble: NBh, NhB, GBh and W = (K_BB + K_BB,delta)^-1 */
    double NBh[3], NhB[3], GB0[3], GB1[3];
    for (i = 0; i < 3; i++) {
        NBh[i] = nf * (ux * b[i] + uy * c[i]);
        NhB[i] = -NBh[i];
        GB0[i] = -nf * b[i];
        GB1[i] = -nf * c[i];
    }
    const double Ab = b[0] * b[0] + b[1] * b[1] + b[2] * b[2] + b[0] * b[1] + b[0] * b[2] + b[1] * b[2];
    const double Bc = c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + c[0] * c[1] + c[0] * c[2] + c[1] * c[2];
    const double Cbc = b[0] * c[0] + b[1] * c[1] + b[2] * c[2];
    const double delta = 0.0;
    const double tv = 2 * visc + delta, vd = visc + delta;
    const double D = (tv * tv + vd * vd) * Ab * Bc + tv * vd * (Ab * Ab + Bc * Bc) - visc * visc * Cbc * Cbc / 4.0;
    double W[2][2];
    W[0][0] = 40.0 * Area / (81.0 * D) * (tv * Bc + vd * Ab);
    W[0][1] = W[1][0] = -40.0 * Area / (81.0 * D) * (visc * Cbc / 2.0);
    W[1][1] = 40.0 * Area / (81.0 * D) * (tv * Ab + vd * Bc);

    double Nd[6][6], Gd[6][3], Gphi[3][3];
    for (i = 0; i < 3; i++)
        for (d = 0; d < 2; d++) {
            for (j = 0; j < 3; j++)
                for (e = 0; e < 2; e++) Nd[2 * i + d][2 * j + e] = NhB[i] * W[d][e] * NBh[j];
            for (k = 0; k < 3; k++) Gd[2 * i + d][k] = NhB[i] * W[d][0] * GB0[k] + NhB[i] * W[d][1] * GB1[k];
        }
    for (k = 0; k < 3; k++)
        for (m = 0; m < 3; m++)
            Gphi[k][m] = GB0[m] * (GB0[k] * W[0][0] + GB1[k] * W[0][1]) + GB1[m] * (GB0[k] * W[0][1] + GB1[k] * W[1][1]);

    /* tangent (:577-665) */
    for (int r = 0; r < 6; r++) {
        const int ni = r >> 1, row = 3 * ni + (r & 1);
        for (int s = 0; s < 6; s++) {
            const int nj = s >> 1, col = 3 * nj + (s & 1);
            const int lo = r < s ? r : s, up = r < s ? s : r;
            const int pl = 2 * (lo >> 1), pu = 2 * (up >> 1);
            double kvis;                                   /* K(lo, up), :165-188 */
            if (!(lo & 1) && !(up & 1)) kvis = kv * (2 * g[pl] * g[pu] + g[pl + 1] * g[pu + 1]);
            else if ((lo & 1) && (up & 1)) kvis = kv * (g[pl] * g[pu] + 2 * g[pl + 1] * g[pu + 1]);
            else if (!(lo & 1)) kvis = kv * (g[pl + 1] * g[pu]);
            else kvis = kv * (g[pl] * g[pu + 1]);
            const double kls = ks * g[s] * g[r];           /* Ks(r, s), :195-230 */
            double v;
            if ((r & 1) == (s & 1)) {
                const double N = third * Area * C[nj];
                if (r == 4 && s == 2) v = N + Nd[lo][up] + kvis + kls;
                else v = N - Nd[lo][up] + kvis + kls;
            } else {
                v = kvis + kls;
            }
            Ke[row * 9 + col] = v;
        }
        for (k = 0; k < 3; k++) Ke[row * 9 + 3 * k + 2] = -(sixth * g[r] - Gd[r][k]);
    }
    for (k = 0; k < 3; k++) {
        const int row = 3 * k + 2;
        for (int s = 0; s < 6; s++) Ke[row * 9 + 3 * (s >> 1) + (s & 1)] = sixth * g[s] - Gd[s][k];
        for (m = 0; m < 3; m++) Ke[row * 9 + 3 * m + 2] = k <= m ? Gphi[k][m] : Gphi[m][k];
    }

    /* residual (:316-342, :532-573) */
    const double advx = duxdx * ux + duxdy * uy, advy = duydx * ux + duydy * uy;
    const double sym = duxdy + duydx;
    const double GTv = third * Area * (duxdx + duydy);
    for (i = 0; i < 3; i++) {
        double Ndv[2], Gdv[2], Nphiv = 0.0, Gphiv;
        for (d = 0; d < 2; d++) {
            const int r = 2 * i + d;
            double sN = Nd[r][0] * uvec[0];
            for (int s = 1; s < 6; s++) sN += Nd[r][s] * uvec[s];
            Ndv[d] = sN;
            Gdv[d] = Gd[r][0] * pvec[0] + Gd[r][1] * pvec[1] + Gd[r][2] * pvec[2];
        }
        Nphiv = -Gd[0][i] * uvec[0];
        for (int s = 1; s < 6; s++) Nphiv += -Gd[s][i] * uvec[s];
        Gphiv = Gphi[i][0] * pvec[0] + Gphi[i][1] * pvec[1] + Gphi[i][2] * pvec[2];
        const double Nvx = third * Area * advx, Nvy = third * Area * advy;
        const double Kvx = 0.5 * visc * (2 * b[i] * duxdx + c[i] * sym);
        const double Kvy = 0.5 * visc * (2 * c[i] * duydy + b[i] * sym);
        const double Ksx = ks * b[i] * duxduy, Ksy = ks * c[i] * duxduy;
        const double Gvx = 0.5 * p * b[i], Gvy = 0.5 * p * c[i];
        Res[3 * i + 0] = 0.0 - (Nvx - Ndv[0] + Kvx + Ksx - (Gvx - Gdv[0]));
        Res[3 * i + 1] = 0.0 - (Nvy - Ndv[1] + Kvy + Ksy - (Gvy - Gdv[1]));
        Res[3 * i + 2] = 0.0 - (GTv - Nphiv + Gphiv);
    }
}

void or_build_ns_vms(int nnodes, int nel, const double *x, const double *y, const int *type,
                     const int *invp, const int *ien, int neq, const or_ns_problem *prob,
                     const double *u, double *A, double *F)
{
    int E, v, k, NEQ = neq;
    double *U = malloc(sizeof(double) * 3 * (size_t)(nnodes ? nnodes : 1));
    for (v = 0; v < nnodes; v++)                          /* eval_U.c:3-35 */
        for (k = 0; k < 3; k++) {
            long q = 3L * v + k;
            U[q] = type[q] > 0 ? u[invp[q]] : prob->upresc[q];
        }
    memset(F, 0, sizeof(double) * ((size_t)NEQ + 1));
    for (E = 0; E < nel; E++) {
        double X[3], Y[3], Ue[9], Res[9];
        int lm[9];
        for (v = 0; v < 3; v++) {
            int J = ien[3 * E + v];
            X[v] = x[J]; Y[v] = y[J];
            for (k = 0; k < 3; k++) {
                long q = 3L * J + k;
                Ue[3 * v + k] = U[q];
                lm[3 * v + k] = type[q] == 0 ? NEQ : invp[q];
            }
        }
        vms_element(X, Y, Ue, prob->reynolds, A + 81L * E, Res);
        for (k = 0; k < 9; k++) F[lm[k]] += Res[k];       /* :705-708 */
        F[NEQ] = 0;
    }
    free(U);
}
