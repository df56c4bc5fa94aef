// Steady incompressible Navier-Stokes on the device: the SUPG/PSPG/LSIC
// element build of 04_SS_NavierStokes_Equations/2D/01_CommonFiles/
// Build_K_F_SUPG_PSPG.c:8-669 (Picard tangent; its Newton branch :560-648
// is only taken after 50000 builds, :466, and is not provided), eval_U.c and
// ebe_assembly.c, and the Picard loop of Process.c:6-62 kept on the device.
//
// k_ns_elem is one thread per element (internal element order): gather the
// three nodes' coordinates and (u, v, p) (free dofs from the state vector,
// Dirichlet dofs from the prescribed values), form the 9x9 tangent straight
// into the SoA block array and the element residual into Fe.
// k_elem_residual (shared with the Euler build) sums the element residuals
// of every free dof in reference element order, as the reference's
// F[lm] += Res loop does, so F is bit-identical.
//
// Every entry is the same sum of the same products, associated the same way,
// as in the reference, written per pair of element nodes (i, j): with
// b = (y23, y31, y12) and c = (x32, x13, x21), the viscous, SUPG and PSPG
// Laplacian terms are evaluated with the lower node or dof index first (the
// reference writes their upper triangle and reuses it below the diagonal),
// the LSIC term keeps its (row, column) order, and the density-1 factors
// (exact multiplications by 1) are left out.  Compiled with -fmad=false.
#include "system.h"

namespace fg {

struct NsElem {
    double b[3], c[3];
    double A, invArea, visc;
    double ux, uy, duxdx, duxdy, duydx, duydy, duxduy;
    double p, dpdx, dpdy;
    double C[3];
    double tau, tau_l;
};

__device__ __forceinline__ void ns_state(NsElem &g, const double X[3], const double Y[3], const double Ue[9],
                                         double Re)
{
    const double third = 1.0 / 3.0;
    g.b[0] = Y[1] - Y[2]; g.b[1] = Y[2] - Y[0]; g.b[2] = Y[0] - Y[1];
    g.c[0] = X[2] - X[1]; g.c[1] = X[0] - X[2]; g.c[2] = X[1] - X[0];
    double TwoA = fabs(g.c[2] * g.b[1] - g.c[1] * g.b[2]);
    g.A = 0.5 * TwoA;
    g.invArea = 1.0 / g.A;
    double hi = 0.5 * g.invArea;
    g.ux = third * (Ue[0] + Ue[3] + Ue[6]);
    g.uy = third * (Ue[1] + Ue[4] + Ue[7]);
    g.duxdx = hi * (Ue[0] * g.b[0] + Ue[3] * g.b[1] + Ue[6] * g.b[2]);
    g.duxdy = hi * (Ue[0] * g.c[0] + Ue[3] * g.c[1] + Ue[6] * g.c[2]);
    g.duydx = hi * (Ue[1] * g.b[0] + Ue[4] * g.b[1] + Ue[7] * g.b[2]);
    g.duydy = hi * (Ue[1] * g.c[0] + Ue[4] * g.c[1] + Ue[7] * g.c[2]);
    g.duxduy = Ue[0] * g.b[0] + Ue[1] * g.c[0] + Ue[3] * g.b[1] + Ue[4] * g.c[1] + Ue[6] * g.b[2] + Ue[7] * g.c[2];
    g.p = third * (Ue[2] + Ue[5] + Ue[8]);
    g.dpdx = hi * (Ue[2] * g.b[0] + Ue[5] * g.b[1] + Ue[8] * g.b[2]);
    g.dpdy = hi * (Ue[2] * g.c[0] + Ue[5] * g.c[1] + Ue[8] * g.c[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) g.C[i] = hi * (g.ux * g.b[i] + g.uy * g.c[i]);
    double h = sqrt(TwoA);
    g.visc = 1. / Re;
    double nu = g.visc;
    double unorm = sqrt(g.ux * g.ux + g.uy * g.uy);
    double adv = 2.0 * unorm / h, dif = 4.0 * nu / (h * h);
    g.tau = 1.0 / sqrt(adv * adv + 9.0 * dif * dif);
    double lh = 0.5 * h * unorm;
    g.tau_l = sqrt(nu * nu + lh * lh);
}

// gradient coefficient of velocity dof p = 2*node + d (d = 0: x, b; 1: y, c)
__device__ __forceinline__ double ns_g(const NsElem &g, int p) { return (p & 1) ? g.c[p >> 1] : g.b[p >> 1]; }

// viscous entry between velocity dofs p <= q
__device__ __forceinline__ double ns_visc(const NsElem &g, int p, int q)
{
    const int i = p >> 1, j = q >> 1, dp = p & 1, dq = q & 1;
    const double s = g.visc * 0.25 * g.invArea;
    if (!dp && !dq) return s * (2 * g.b[i] * g.b[j] + g.c[i] * g.c[j]);
    if (dp && dq) return s * (g.b[i] * g.b[j] + 2 * g.c[i] * g.c[j]);
    if (!dp) return s * (g.c[i] * g.b[j]);
    return s * (g.b[i] * g.c[j]);
}

__global__ void __launch_bounds__(128) k_ns_elem(int nel, int ld, int n, const int *__restrict__ gien,
                                                 const double *__restrict__ gx, const double *__restrict__ gy,
                                                 const int *__restrict__ node_dof, const double *__restrict__ up,
                                                 const double *__restrict__ f1, const double *__restrict__ f2,
                                                 const double *__restrict__ u, double Re,
                                                 double *__restrict__ A64, double *__restrict__ Fe)
{
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0;
    double X[3], Y[3], Ue[9], fx[3], fy[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const int J = gien[(size_t)v * ld + pos];
        X[v] = gx[J];
        Y[v] = gy[J];
        fx[v] = f1 ? f1[J] : 0.0;
        fy[v] = f2 ? f2[J] : 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int d = node_dof[3 * J + k];
            Ue[3 * v + k] = d == n ? up[3 * J + k] : u[d];
        }
    }
    NsElem g;
    ns_state(g, X, Y, Ue, Re);
    const double A = g.A, tau = g.tau;
    const double ls = g.tau_l * 0.25 * g.invArea;
    const double ps = 0.25 * tau * g.invArea;
    double *a = A64 + pos;
    // tangent (Build_K_F_SUPG_PSPG.c:468-558)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int lo = i < j ? i : j, hi = i < j ? j : i;
            const double Nj = third * A * g.C[j];
            const double Nd = tau * A * g.C[lo] * g.C[hi];
#pragma unroll
            for (int di = 0; di < 2; ++di) {
                const int p = 2 * i + di, row = 3 * i + di;
#pragma unroll
                for (int dj = 0; dj < 2; ++dj) {
                    const int q = 2 * j + dj;
                    const double k = p <= q ? ns_visc(g, p, q) : ns_visc(g, q, p);
                    const double ks = ls * ns_g(g, q) * ns_g(g, p);
                    a[(size_t)(row * 9 + 3 * j + dj) * ld] = di == dj ? Nj + Nd + k + ks : k + ks;
                }
                const double gd = 0.5 * tau * g.C[i] * (di ? g.c[j] : g.b[j]);
                a[(size_t)(row * 9 + 3 * j + 2) * ld] = -(sixth * ns_g(g, p) + gd);
            }
#pragma unroll
            for (int dj = 0; dj < 2; ++dj) {
                const int q = 2 * j + dj;
                const double gd = 0.5 * tau * g.C[j] * (dj ? g.c[i] : g.b[i]);
                a[(size_t)((3 * i + 2) * 9 + 3 * j + dj) * ld] = sixth * ns_g(g, q) + gd;
            }
            a[(size_t)((3 * i + 2) * 9 + 3 * j + 2) * ld] = ps * (g.b[lo] * g.b[hi] + g.c[lo] * g.c[hi]);
        }
    }
    // residual (:412-463)
    const double fxB = third * (fx[0] + fx[1] + fx[2]);
    const double fyB = third * (fy[0] + fy[1] + fy[2]);
    const double fa = third * A * fxB, fb = third * A * fyB;
    const double advx = g.duxdx * g.ux + g.duxdy * g.uy;
    const double advy = g.duydx * g.ux + g.duydy * g.uy;
    const double sym = g.duxdy + g.duydx;
    const double GTv = third * A * (g.duxdx + g.duydy);
    double *fe = Fe + pos;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double b = g.b[i], c = g.c[i], Ci = g.C[i];
        const double Fx = fa + tau * A * Ci * fxB;
        const double Fy = fb + tau * A * Ci * fyB;
        const double Fp = tau * A * (b * fxB + c * fyB);
        const double Nvx = third * A * advx, Nvy = third * A * advy;
        const double Ndx = tau * A * Ci * advx, Ndy = tau * A * Ci * advy;
        const double Kvx = 0.5 * g.visc * (2 * b * g.duxdx + c * sym);
        const double Kvy = 0.5 * g.visc * (2 * c * g.duydy + b * sym);
        const double Ksx = ls * b * g.duxduy, Ksy = ls * c * g.duxduy;
        const double Gvx = 0.5 * g.p * b, Gvy = 0.5 * g.p * c;
        const double Gdx = tau * A * Ci * g.dpdx, Gdy = tau * A * Ci * g.dpdy;
        const double Nphi = 0.5 * tau * (advx * b + advy * c);
        const double Gphi = 0.5 * tau * (b * g.dpdx + c * g.dpdy);
        fe[(size_t)(3 * i + 0) * ld] = Fx - (Nvx + Ndx + Kvx + Ksx - (Gvx + Gdx));
        fe[(size_t)(3 * i + 1) * ld] = Fy - (Nvy + Ndy + Kvy + Ksy - (Gvy + Gdy));
        fe[(size_t)(3 * i + 2) * ld] = Fp - (GTv + Nphi + Gphi);
    }
}

// F[d] = sum of the element residual entries of dof d in reference element
// order, as the builds' F[lm] += Res loops add them; F[n] = 0.
__global__ void k_elem_residual(int n, int ld, const int *__restrict__ dptr, const int *__restrict__ dinc,
                                const double *__restrict__ Fe, double *__restrict__ F)
{
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d > n) return;
    if (d == n) { F[n] = 0.0; return; }
    double s = 0.0;
    for (int q = dptr[d]; q < dptr[d + 1]; ++q) {
        const int pos = dinc[q] >> 4, a = dinc[q] & 15;
        s += Fe[(size_t)a * ld + pos];
    }
    F[d] = s;
}

int gather_residual(fg_system *s, const double *Fe, double *F, cudaStream_t st)
{
    const Topology &t = s->topo;
    k_elem_residual<<<(t.n + 256) / 256, 256, 0, st>>>(t.n, s->nel_pad, s->dinc_ptr.as<int>(), s->dinc.as<int>(), Fe,
                                                      F);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

// ---------------------------------------------------------------- VMS-DCDD
// Build_K_F_VMS_DCDD.c:8-716 (StabilizationForm "VMS-DCDD"): Galerkin + LSIC
// with the bubble enrichment condensed through the 2x2 inverse W of K_BB.
// With velocity dofs r = 2 i + d and g_r = b_i (d = 0) or c_i (d = 1):
//   Ndelta(r, s) = (NhB_i W[d][e]) NBh_j,   NBh_i = 9/40 (ux b_i + uy c_i) = -NhB_i
//   Gdelta(r, k) = (NhB_i W[d][0]) GB0_k + (NhB_i W[d][1]) GB1_k,  GB = -9/40 (b; c)
//   Gphi(k, m)   = GB0_m (GB0_k W00 + GB1_k W01) + GB1_m (GB0_k W01 + GB1_k W11)
// evaluated on the fly, each associated as the reference writes it.  The
// reference's own choices are kept: the tangent holds Ndelta only in the
// same-direction blocks and from the upper triangle, with a plus sign at
// (node 2 x, node 1 x) (:645); the pressure block takes the upper triangle
// of Gphi; the residual uses the full matrices; delta = 0 and the source is
// 0 (:289, :388-394), so the residual is 0 - (...).
struct VmsElem {
    double g[6];                  // b0 c0 b1 c1 b2 c2
    double A, invArea, visc, ux, uy, duxdx, duxdy, duydx, duydy, duxduy, p;
    double C[3], NBh[3], W00, W01, W11, ks, kv;
};

__device__ __forceinline__ double vms_gb(const VmsElem &e, int k, int d) { return -(9.0 / 40.0) * e.g[2 * k + d]; }
__device__ __forceinline__ double vms_w(const VmsElem &e, int d, int f)
{
    return d != f ? e.W01 : (d ? e.W11 : e.W00);
}
__device__ __forceinline__ double vms_nd(const VmsElem &e, int r, int s)
{
    return -e.NBh[r >> 1] * vms_w(e, r & 1, s & 1) * e.NBh[s >> 1];
}
__device__ __forceinline__ double vms_gd(const VmsElem &e, int r, int k)
{
    const double nh = -e.NBh[r >> 1];
    return nh * vms_w(e, r & 1, 0) * vms_gb(e, k, 0) + nh * vms_w(e, r & 1, 1) * vms_gb(e, k, 1);
}
__device__ __forceinline__ double vms_gphi(const VmsElem &e, int k, int m)
{
    const double g0k = vms_gb(e, k, 0), g1k = vms_gb(e, k, 1);
    return vms_gb(e, m, 0) * (g0k * e.W00 + g1k * e.W01) + vms_gb(e, m, 1) * (g0k * e.W01 + g1k * e.W11);
}

__global__ void __launch_bounds__(128) k_ns_vms_elem(int nel, int ld, int n, const int *__restrict__ gien,
                                                     const double *__restrict__ gx, const double *__restrict__ gy,
                                                     const int *__restrict__ node_dof, const double *__restrict__ up,
                                                     const double *__restrict__ u, double Re,
                                                     double *__restrict__ A64, double *__restrict__ Fe)
{
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0, nf = 9.0 / 40.0;
    double X[3], Y[3], Ue[9];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const int J = gien[(size_t)v * ld + pos];
        X[v] = gx[J];
        Y[v] = gy[J];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int d = node_dof[3 * J + k];
            Ue[3 * v + k] = d == n ? up[3 * J + k] : u[d];
        }
    }
    VmsElem e;
    double *g = e.g;
    g[0] = Y[1] - Y[2]; g[2] = Y[2] - Y[0]; g[4] = Y[0] - Y[1];
    g[1] = X[2] - X[1]; g[3] = X[0] - X[2]; g[5] = X[1] - X[0];
    const double TwoA = fabs(g[5] * g[2] - g[3] * g[4]);
    e.A = 0.5 * TwoA;
    e.invArea = 1.0 / e.A;
    const double hi = 0.5 * e.invArea;
    e.ux = third * (Ue[0] + Ue[3] + Ue[6]);
    e.uy = third * (Ue[1] + Ue[4] + Ue[7]);
    e.duxdx = hi * (Ue[0] * g[0] + Ue[3] * g[2] + Ue[6] * g[4]);
    e.duxdy = hi * (Ue[0] * g[1] + Ue[3] * g[3] + Ue[6] * g[5]);
    e.duydx = hi * (Ue[1] * g[0] + Ue[4] * g[2] + Ue[7] * g[4]);
    e.duydy = hi * (Ue[1] * g[1] + Ue[4] * g[3] + Ue[7] * g[5]);
    e.duxduy = Ue[0] * g[0] + Ue[1] * g[1] + Ue[3] * g[2] + Ue[4] * g[3] + Ue[6] * g[4] + Ue[7] * g[5];
    e.p = third * (Ue[2] + Ue[5] + Ue[8]);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        e.C[i] = hi * (e.ux * g[2 * i] + e.uy * g[2 * i + 1]);
        e.NBh[i] = nf * (e.ux * g[2 * i] + e.uy * g[2 * i + 1]);
    }
    const double h = sqrt(4 * e.A / 3.14159265359);      // PI of the reference's header
    e.visc = 1. / Re;
    const double unorm = sqrt(e.ux * e.ux + e.uy * e.uy);
    const double tau_l = 0.5 * h * unorm;
    e.ks = tau_l * 0.25 * e.invArea;
    e.kv = e.visc * 0.25 * e.invArea;
    const double Ab = g[0] * g[0] + g[2] * g[2] + g[4] * g[4] + g[0] * g[2] + g[0] * g[4] + g[2] * g[4];
    const double Bc = g[1] * g[1] + g[3] * g[3] + g[5] * g[5] + g[1] * g[3] + g[1] * g[5] + g[3] * g[5];
    const double Cbc = g[0] * g[1] + g[2] * g[3] + g[4] * g[5];
    const double delta = 0.0, visc = e.visc;
    const double tv = 2 * visc + delta, vd = visc + delta;
    const double D = (tv * tv + vd * vd) * Ab * Bc + tv * vd * (Ab * Ab + Bc * Bc) - visc * visc * Cbc * Cbc / 4.0;
    e.W00 = 40.0 * e.A / (81.0 * D) * (tv * Bc + vd * Ab);
    e.W01 = -40.0 * e.A / (81.0 * D) * (visc * Cbc / 2.0);
    e.W11 = 40.0 * e.A / (81.0 * D) * (tv * Ab + vd * Bc);
    double *a = A64 + pos;
    // tangent (:577-665)
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        const int row = 3 * (r >> 1) + (r & 1);
#pragma unroll
        for (int s2 = 0; s2 < 6; ++s2) {
            const int col = 3 * (s2 >> 1) + (s2 & 1);
            const int lo = r < s2 ? r : s2, hi2 = r < s2 ? s2 : r;
            const int pl = lo & ~1, pu = hi2 & ~1;
            double kvis;
            if (!(lo & 1) && !(hi2 & 1)) kvis = e.kv * (2 * g[pl] * g[pu] + g[pl + 1] * g[pu + 1]);
            else if ((lo & 1) && (hi2 & 1)) kvis = e.kv * (g[pl] * g[pu] + 2 * g[pl + 1] * g[pu + 1]);
            else if (!(lo & 1)) kvis = e.kv * (g[pl + 1] * g[pu]);
            else kvis = e.kv * (g[pl] * g[pu + 1]);
            const double kls = e.ks * g[s2] * g[r];
            double v;
            if ((r & 1) == (s2 & 1)) {
                const double N = third * e.A * e.C[s2 >> 1];
                v = (r == 4 && s2 == 2) ? N + vms_nd(e, lo, hi2) + kvis + kls : N - vms_nd(e, lo, hi2) + kvis + kls;
            } else {
                v = kvis + kls;
            }
            a[(size_t)(row * 9 + col) * ld] = v;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) a[(size_t)(row * 9 + 3 * k + 2) * ld] = -(sixth * g[r] - vms_gd(e, r, k));
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int row = 3 * k + 2;
#pragma unroll
        for (int s2 = 0; s2 < 6; ++s2)
            a[(size_t)(row * 9 + 3 * (s2 >> 1) + (s2 & 1)) * ld] = sixth * g[s2] - vms_gd(e, s2, k);
#pragma unroll
        for (int m = 0; m < 3; ++m) a[(size_t)(row * 9 + 3 * m + 2) * ld] = k <= m ? vms_gphi(e, k, m) : vms_gphi(e, m, k);
    }
    // residual (:316-342, :532-573)
    const double uv[6] = {Ue[0], Ue[1], Ue[3], Ue[4], Ue[6], Ue[7]}, pv[3] = {Ue[2], Ue[5], Ue[8]};
    const double advx = e.duxdx * e.ux + e.duxdy * e.uy, advy = e.duydx * e.ux + e.duydy * e.uy;
    const double sym = e.duxdy + e.duydx;
    const double GTv = third * e.A * (e.duxdx + e.duydy);
    double *fe = Fe + pos;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double Ndv[2], Gdv[2];
#pragma unroll
        for (int d = 0; d < 2; ++d) {
            const int r = 2 * i + d;
            double sN = vms_nd(e, r, 0) * uv[0];
#pragma unroll
            for (int s2 = 1; s2 < 6; ++s2) sN += vms_nd(e, r, s2) * uv[s2];
            Ndv[d] = sN;
            Gdv[d] = vms_gd(e, r, 0) * pv[0] + vms_gd(e, r, 1) * pv[1] + vms_gd(e, r, 2) * pv[2];
        }
        double Nphiv = -vms_gd(e, 0, i) * uv[0];
#pragma unroll
        for (int s2 = 1; s2 < 6; ++s2) Nphiv += -vms_gd(e, s2, i) * uv[s2];
        const double Gphiv = vms_gphi(e, i, 0) * pv[0] + vms_gphi(e, i, 1) * pv[1] + vms_gphi(e, i, 2) * pv[2];
        const double b = g[2 * i], c = g[2 * i + 1];
        const double Nvx = third * e.A * advx, Nvy = third * e.A * advy;
        const double Kvx = 0.5 * visc * (2 * b * e.duxdx + c * sym);
        const double Kvy = 0.5 * visc * (2 * c * e.duydy + b * sym);
        const double Ksx = e.ks * b * e.duxduy, Ksy = e.ks * c * e.duxduy;
        const double Gvx = 0.5 * e.p * b, Gvy = 0.5 * e.p * c;
        fe[(size_t)(3 * i + 0) * ld] = 0.0 - (Nvx - Ndv[0] + Kvx + Ksx - (Gvx - Gdv[0]));
        fe[(size_t)(3 * i + 1) * ld] = 0.0 - (Nvy - Ndv[1] + Kvy + Ksy - (Gvy - Gdv[1]));
        fe[(size_t)(3 * i + 2) * ld] = 0.0 - (GTv - Nphiv + Gphiv);
    }
}

int ns_assemble_device(fg_system *s, double reynolds, int form, const double *u_dev, double *F_dev, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (t.ndof != 3) { set_error("Navier-Stokes assembly needs ndof == 3"); return FG_ERR_UNSUPPORTED; }
    if (!s->ns_geometry_ok) { set_error("Navier-Stokes assembly before fg_ns_set_geometry"); return FG_ERR_STATE; }
    if (!(reynolds > 0)) { set_error("Reynolds number must be positive"); return FG_ERR_ARG; }
    if (form != FG_NS_SUPG_PSPG && form != FG_NS_VMS_DCDD) {
        set_error("Navier-Stokes form must be FG_NS_SUPG_PSPG or FG_NS_VMS_DCDD");
        return FG_ERR_ARG;
    }
    if (t.nel > 0 && form == FG_NS_VMS_DCDD)
        k_ns_vms_elem<<<(t.nel + 127) / 128, 128, 0, st>>>(t.nel, s->nel_pad, t.n, s->gien.as<int>(),
                                                          s->gx.as<double>(), s->gy.as<double>(),
                                                          s->node_dof.as<int>(), s->gup.as<double>(), u_dev, reynolds,
                                                          s->A64.as<double>(), s->Fe.as<double>());
    else if (t.nel > 0)
        k_ns_elem<<<(t.nel + 127) / 128, 128, 0, st>>>(t.nel, s->nel_pad, t.n, s->gien.as<int>(), s->gx.as<double>(),
                                                      s->gy.as<double>(), s->node_dof.as<int>(), s->gup.as<double>(),
                                                      s->gf1.as<double>(), s->gf2.as<double>(), u_dev, reynolds,
                                                      s->A64.as<double>(), s->Fe.as<double>());
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    int r = gather_residual(s, s->Fe.as<double>(), F_dev, st);
    if (r) return r;
    s->blocks_ok = true;
    s->csr_dirty = true;
    return convert_blocks(s, st);
}

// ---------------------------------------------------------------- state updates
// The BLAS-1 steps of the nonlinear and time loops (daxpy, and the norms
// their stop tests take), on the device.  Norms are per-CTA partial sums of
// squares added by one CTA in a fixed order: deterministic for a given n.
// Compiled without FMA contraction, like the reference's y += a * x.
constexpr int kNormBlocks = 1024;

static int norm_blocks(int n) { return std::max(1, std::min(kNormBlocks, (n + 255) / 256)); }

__device__ __forceinline__ void block_sums(double a, double b, double *part)
{
    __shared__ double sh[2][8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { sh[0][w] = a; sh[1][w] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { x += sh[0][k]; y += sh[1][k]; }
        part[2 * blockIdx.x] = x;
        part[2 * blockIdx.x + 1] = y;
    }
}

// y += a x; partial sums of x^2 and of the updated y^2
__global__ void __launch_bounds__(256) k_axpy_sq(int n, double a, const double *__restrict__ x,
                                                 double *__restrict__ y, double *__restrict__ part)
{
    double xx = 0.0, yy = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double xi = x[i], v = y[i] + a * xi;
        y[i] = v;
        xx += xi * xi;
        yy += v * v;
    }
    block_sums(xx, yy, part);
}

// partial sums of (u - v)^2 and u^2
__global__ void __launch_bounds__(256) k_diff_sq(int n, const double *__restrict__ u, const double *__restrict__ v,
                                                 double *__restrict__ part)
{
    double dd = 0.0, uu = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double d = u[i] - v[i];
        dd += d * d;
        uu += u[i] * u[i];
    }
    block_sums(dd, uu, part);
}

__global__ void k_axpy(int n, double a, const double *__restrict__ x, double *__restrict__ y)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] += a * x[i];
}

// y = c1 x1 - c2 x2, each product rounded (the BDF2 and TR-BDF2 predictions)
// (y may be x1: each entry is read before it is written by the same thread)
__global__ void k_lincomb(int n, double c1, const double *x1, double c2, const double *__restrict__ x2, double *y)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = c1 * x1[i] - c2 * x2[i];
}

__global__ void k_sum_parts(const double *__restrict__ part, int nb, double *__restrict__ out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    for (int k = 0; k < nb; ++k) { a += part[2 * k]; b += part[2 * k + 1]; }
    out[0] = a;
    out[1] = b;
}

int axpy_norms_device(int n, double a, const double *x, double *y, double *part, double *out, cudaStream_t st)
{
    const int nb = norm_blocks(n);
    k_axpy_sq<<<nb, 256, 0, st>>>(n, a, x, y, part);
    k_sum_parts<<<1, 32, 0, st>>>(part, nb, out);
    FG_CUDA(cudaGetLastError());
    count_launches(2);
    return FG_OK;
}

int diff_norms_device(int n, const double *u, const double *v, double *part, double *out, cudaStream_t st)
{
    const int nb = norm_blocks(n);
    k_diff_sq<<<nb, 256, 0, st>>>(n, u, v, part);
    k_sum_parts<<<1, 32, 0, st>>>(part, nb, out);
    FG_CUDA(cudaGetLastError());
    count_launches(2);
    return FG_OK;
}

int lincomb_device(int n, double c1, const double *x1, double c2, const double *x2, double *y, cudaStream_t st)
{
    k_lincomb<<<norm_blocks(n), 256, 0, st>>>(n, c1, x1, c2, x2, y);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

int axpy_device(int n, double a, const double *x, double *y, cudaStream_t st)
{
    k_axpy<<<norm_blocks(n), 256, 0, st>>>(n, a, x, y);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

size_t norm_scratch_bytes() { return sizeof(double) * (2 * kNormBlocks + 2); }

}  // namespace fg
