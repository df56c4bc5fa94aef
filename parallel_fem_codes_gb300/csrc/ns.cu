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

int ns_assemble_device(fg_system *s, double reynolds, const double *u_dev, double *F_dev, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (t.ndof != 3) { set_error("Navier-Stokes assembly needs ndof == 3"); return FG_ERR_UNSUPPORTED; }
    if (!s->ns_geometry_ok) { set_error("Navier-Stokes assembly before fg_ns_set_geometry"); return FG_ERR_STATE; }
    if (!(reynolds > 0)) { set_error("Reynolds number must be positive"); return FG_ERR_ARG; }
    if (t.nel > 0)
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
