// Set-up kernels: block layout, Diag and nodal block-diagonal
// preconditioner set-up, SUPG/CAU transport assembly, renumbering.
//
// This translation unit is compiled with -fmad=false: every product and sum
// is rounded as written, in the order the reference writes it, so the
// element blocks, right-hand side, diagonal and block inverses agree with
// the reference's C to the last bit (sqrt and division are correctly
// rounded in both).
#include <algorithm>
#include <cmath>

#include "system.h"

namespace fg {

// ---------------------------------------------------------------- renumbering
__global__ void k_permute(const int *__restrict__ map, const double *__restrict__ src, double *__restrict__ dst,
                          int n, int gather)
{
    // gather: dst[i] = src[map[i]]   (map = perm: internal <- reference)
    // scatter: dst[map[i]] = src[i]  (map = perm: reference <- internal)
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        if (gather) dst[i] = src[map[i]];
        else dst[map[i]] = src[i];
    }
    if (i == 0) dst[n] = 0.0;
}

int permute_in(fg_system *s, const double *ref_dev, double *int_dev, cudaStream_t st)
{
    int n = s->topo.n;
    k_permute<<<(n + 255) / 256 + 1, 256, 0, st>>>(s->perm.as<int>(), ref_dev, int_dev, n, 1);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

int permute_out(fg_system *s, const double *int_dev, double *ref_dev, cudaStream_t st)
{
    int n = s->topo.n;
    k_permute<<<(n + 255) / 256 + 1, 256, 0, st>>>(s->perm.as<int>(), int_dev, ref_dev, n, 0);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

// ---------------------------------------------------------------- blocks
// Host layout (reference element order, row-major S x S) -> SoA in the
// internal element order: A64[k][pos] = raw[eorder[pos]][k].
__global__ void k_blocks_in(const double *__restrict__ raw, const int *__restrict__ eorder, double *__restrict__ A64,
                            int nel, int ld, int SS)
{
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const double *src = raw + (size_t)eorder[pos] * SS;
    for (int k = 0; k < SS; ++k) A64[(size_t)k * ld + pos] = src[k];
}

__global__ void k_blocks_out(double *__restrict__ raw, const int *__restrict__ eorder, const double *__restrict__ A64,
                             int nel, int ld, int SS)
{
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    double *dst = raw + (size_t)eorder[pos] * SS;
    for (int k = 0; k < SS; ++k) dst[k] = A64[(size_t)k * ld + pos];
}

__global__ void k_to_f32(const double *__restrict__ a, float *__restrict__ b, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// 3x3 FP32 blocks, blocked per matvec patch: patch p (elements pe0 ..
// pe0 + pne) is one [9][W] block at 9 pe0, W = pne rounded up to 16 (zero
// padded), so the matvec moves a patch's blocks as one contiguous copy.
// Elements without a free dof (after the last patch) have no FP32 copy.
__global__ void k_to_f32_patches(const double *__restrict__ a, float *__restrict__ b, const int *__restrict__ pt_elem,
                                 int npatch, int ld)
{
    for (int p = blockIdx.x; p < npatch; p += gridDim.x) {
        const int pe0 = pt_elem[p], pne = pt_elem[p + 1] - pe0, W = (pne + 15) & ~15;
        float *dst = b + 9 * (size_t)pe0;
        for (int idx = threadIdx.x; idx < 9 * W; idx += blockDim.x) {
            const int m = idx / W, i = idx - m * W;
            dst[idx] = i < pne ? (float)a[(size_t)m * ld + pe0 + i] : 0.0f;
        }
    }
}

int convert_blocks(fg_system *s, cudaStream_t st)
{
    if (s->topo.S == 3) {
        const int np = s->topo.npatch;
        if (np > 0)
            k_to_f32_patches<<<std::max(1, std::min(np, 8 * sm_count())), 256, 0, st>>>(
                s->A64.as<double>(), s->A32.as<float>(), s->pt_elem.as<int>(), np, s->nel_pad);
    } else {
        size_t n = (size_t)s->topo.S * s->topo.S * s->nel_pad;
        k_to_f32<<<std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 8 * sm_count())), 256, 0, st>>>(
            s->A64.as<double>(), s->A32.as<float>(), n);
    }
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

int upload_blocks_raw(fg_system *s, const double *raw_dev, cudaStream_t st)
{
    int nel = s->topo.nel;
    if (nel > 0)
        k_blocks_in<<<(nel + 255) / 256, 256, 0, st>>>(raw_dev, s->eorder.as<int>(), s->A64.as<double>(), nel,
                                                      s->nel_pad, s->topo.S * s->topo.S);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return convert_blocks(s, st);
}

int download_blocks_raw(const fg_system *s, double *raw_dev, cudaStream_t st)
{
    int nel = s->topo.nel;
    if (nel > 0)
        k_blocks_out<<<(nel + 255) / 256, 256, 0, st>>>(raw_dev, s->eorder.as<int>(), s->A64.as<double>(), nel,
                                                       s->nel_pad, s->topo.S * s->topo.S);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

// ---------------------------------------------------------------- Diag
// Diag_precond_EBE_setup (EBE/Diag_precond_EBE_setup.c:3-32), one thread
// per dof, gathering the element diagonals in reference element order so
// the sum is the reference's; accumulate keeps the previous Diag as the
// reference does across nonlinear iterations.
__global__ void k_diag_setup(const int *__restrict__ dptr, const int *__restrict__ dinc, const double *__restrict__ A64,
                             int ld, int S, int n, int accumulate, double *__restrict__ diag,
                             double *__restrict__ invd64, float *__restrict__ invd32, double *__restrict__ F)
{
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    double s = accumulate ? diag[d] : 0.0;
    for (int q = dptr[d]; q < dptr[d + 1]; ++q) {
        int pos = dinc[q] >> 4, r = dinc[q] & 15;
        s += A64[(size_t)(r * S + r) * ld + pos];
    }
    diag[d] = s;
    double inv = 1.0 / s;
    invd64[d] = inv;
    invd32[d] = (float)inv;
    if (F) F[d] *= inv;
}

// ---------------------------------------------------------------- block diagonal
// Nodal B x B diagonal blocks (EBE/BlockDiag_precond_EBE_setup.c:70-80,
// EBE/BlockDiagDOF3_precond_EBE_setup.c:66-76) and their closed-form
// inverses (matrix_Inverse :90-147, DOF3_matrix_Inverse :84-124).
__device__ double inv4(const double *B, double *R, bool quirk)
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
    // the reference writes c*j*m in entry 14 where the cofactor has c*f*m
    R[14] = q*((quirk ? c*j*m : c*f*m) - b*g*m - c*e*n + a*g*n + b*e*o - a*f*o);
    R[15] = q*(-c*f*i + b*g*i + c*e*j - a*g*j - b*e*k + a*f*k);
    return det;
}

__device__ double inv3(const double *B, double *R)
{
    double a=B[0],b=B[1],c=B[2],d=B[3],e=B[4],f=B[5],g=B[6],h=B[7],i=B[8];
    double det = a*e*i - a*f*h - b*d*i + b*f*g + c*d*h - c*e*g;
    double q = 1.0 / det;
    R[0] = q*(e*i - f*h); R[1] = q*(c*h - b*i); R[2] = q*(b*f - c*e);
    R[3] = q*(f*g - d*i); R[4] = q*(a*i - c*g); R[5] = q*(c*d - a*f);
    R[6] = q*(d*h - e*g); R[7] = q*(b*g - a*h); R[8] = q*(a*e - b*d);
    return det;
}

__device__ double inv2(const double *B, double *R)
{
    double det = B[0] * B[3] - B[1] * B[2];
    double q = 1.0 / det;
    R[0] = q * B[3]; R[1] = -q * B[1]; R[2] = -q * B[2]; R[3] = q * B[0];
    return det;
}

// A node with a free dof whose block is singular (zero or non-finite
// determinant) sets *err to FG_ERR_BREAKDOWN; its inverse is still written
// as the reference computes it.
template <int B>
__global__ void k_blockdiag_setup(const int *__restrict__ nptr, const int *__restrict__ ninc, const double *__restrict__ A64,
                                  int ld, int nnodes, int quirk, double *__restrict__ bd, double *__restrict__ ibd64,
                                  float *__restrict__ ibd32, const int *__restrict__ node_dof, int n, int *err)
{
    int nd = blockIdx.x * blockDim.x + threadIdx.x;
    if (nd >= nnodes) return;
    const int S = 3 * B;
    double blk[B * B], inv[B * B];
    for (int q = 0; q < B * B; ++q) blk[q] = 0.0;
    for (int q = nptr[nd]; q < nptr[nd + 1]; ++q) {
        int pos = ninc[q] >> 2, v = ninc[q] & 3;
        for (int r = 0; r < B; ++r)
            for (int c = 0; c < B; ++c) blk[r * B + c] += A64[(size_t)((B * v + r) * S + B * v + c) * ld + pos];
    }
    const double det = B == 4 ? inv4(blk, inv, quirk != 0) : B == 3 ? inv3(blk, inv) : inv2(blk, inv);
    if (!(det != 0.0) || !isfinite(det)) {
        bool free_dof = false;
        for (int a = 0; a < B; ++a) free_dof |= node_dof[nd * B + a] != n;
        if (free_dof) atomicExch(err, FG_ERR_BREAKDOWN);
    }
    for (int q = 0; q < B * B; ++q) {
        bd[(size_t)nd * B * B + q] = blk[q];
        ibd64[(size_t)nd * B * B + q] = inv[q];
        ibd32[(size_t)nd * B * B + q] = (float)inv[q];
    }
}

// F <- B^-1 F per node (BlockDiag_precond.c:12-26), Dirichlet dofs read 0
template <int B>
__global__ void k_blockdiag_apply64(const int *__restrict__ node_dof, const double *__restrict__ ibd, int nnodes, int n,
                                    const double *__restrict__ p, double *__restrict__ z)
{
    int nd = blockIdx.x * blockDim.x + threadIdx.x;
    if (nd >= nnodes) return;
    int id[B];
    double v[B];
    for (int a = 0; a < B; ++a) { id[a] = node_dof[nd * B + a]; v[a] = id[a] == n ? 0.0 : p[id[a]]; }
    const double *m = ibd + (size_t)nd * B * B;
    for (int r = 0; r < B; ++r) {
        double s = m[r * B] * v[0];
        for (int q = 1; q < B; ++q) s += m[r * B + q] * v[q];
        if (id[r] != n) z[id[r]] = s;
    }
}

static int elem_prec_setup(fg_system *s, int kind, cudaStream_t st);

int precond_setup_device(fg_system *s, int kind, int flags, double *F_dev, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (kind == FG_PRECOND_NONE) { s->precond = kind; return FG_OK; }
    if (kind == FG_PRECOND_ILU0) return ilu0_setup_device(s, F_dev, st);
    if (kind == FG_PRECOND_SPIKE) return spike_setup_device(s, F_dev, st);
    if (!s->blocks_ok) { set_error("preconditioner set-up before element blocks were set"); return FG_ERR_STATE; }
    if (kind == FG_PRECOND_DIAG) {
        if (t.n > 0)
            k_diag_setup<<<(t.n + 255) / 256, 256, 0, st>>>(s->dinc_ptr.as<int>(), s->dinc.as<int>(), s->A64.as<double>(),
                                                           s->nel_pad, t.S, t.n, (flags & FG_SETUP_ACCUMULATE) ? 1 : 0,
                                                           s->diag.as<double>(), s->invd64.as<double>(),
                                                           s->invd32.as<float>(), F_dev);
        FG_CUDA(cudaGetLastError());
    count_launches(1);
        s->precond = kind;
        return FG_OK;
    }
    if (kind == FG_PRECOND_LUE || kind == FG_PRECOND_SGSE) {
        int r;
        if ((r = elem_prec_setup(s, kind, st))) return r;
        s->precond = kind;
        if (F_dev && (r = elem_prec_apply_device(s, false, F_dev, F_dev, st))) return r;
        return FG_OK;
    }
    if (kind == FG_PRECOND_BLOCKDIAG) {
        int B = t.ndof;
        if (B < 2) { set_error("block-diagonal preconditioner needs ndof >= 2"); return FG_ERR_UNSUPPORTED; }
        int g = (t.nnodes + 127) / 128;
        int q = (flags & FG_SETUP_REF_QUIRKS) ? 1 : 0;
        const int *np = s->ninc_ptr.as<int>(), *ni = s->ninc.as<int>();
        double *bd = s->bd.as<double>(), *i64 = s->ibd64.as<double>();
        float *i32 = s->ibd32.as<float>();
        const int *nd = s->node_dof.as<int>();
        int *err = s->pc_err.as<int>();
        FG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
        if (B == 4)
            k_blockdiag_setup<4><<<g, 128, 0, st>>>(np, ni, s->A64.as<double>(), s->nel_pad, t.nnodes, q, bd, i64, i32,
                                                    nd, t.n, err);
        else if (B == 3)
            k_blockdiag_setup<3><<<g, 128, 0, st>>>(np, ni, s->A64.as<double>(), s->nel_pad, t.nnodes, q, bd, i64, i32,
                                                    nd, t.n, err);
        else
            k_blockdiag_setup<2><<<g, 128, 0, st>>>(np, ni, s->A64.as<double>(), s->nel_pad, t.nnodes, q, bd, i64, i32,
                                                    nd, t.n, err);
        FG_CUDA(cudaGetLastError());
    count_launches(1);
        s->precond = kind;
        if (F_dev) {
            if (B == 4) k_blockdiag_apply64<4><<<g, 128, 0, st>>>(s->node_dof.as<int>(), i64, t.nnodes, t.n, F_dev, F_dev);
            else if (B == 3) k_blockdiag_apply64<3><<<g, 128, 0, st>>>(s->node_dof.as<int>(), i64, t.nnodes, t.n, F_dev, F_dev);
            else k_blockdiag_apply64<2><<<g, 128, 0, st>>>(s->node_dof.as<int>(), i64, t.nnodes, t.n, F_dev, F_dev);
            FG_CUDA(cudaGetLastError());
    count_launches(1);
        }
        return FG_OK;
    }
    set_error("unknown preconditioner kind");
    return FG_ERR_ARG;
}

// ---------------------------------------------------------------- element preconditioners
// Preconditioner "LUe" (EBE/LU_precond_EBE_setup.c:20-31, LU_precond_EBE.c:
// 28-60) and "SGSe" (EBE/SGS_precond_EBE.c: SGS_precond_EBE forward,
// SGS_precondR_EBE backward).  Each sweeps the elements in order, in place,
// every element reading the values the earlier ones wrote: a dependency
// chain through the whole mesh, so one thread of one warp per system runs
// it, in the reference's element order, while the other lanes stage the
// next 32 element records (internal dofs, 9 coefficients) into shared
// memory.  Expressions keep the reference's association (`a += -b*c -
// d*e` adds ((-(b*c)) - d*e)); compiled without FMA contraction, so the
// sweeps are bit-identical with the reference's.

// per element, in reference element order: the LU factors of its block
// (kind 1) or its entries (kind 2); thread per internal position
__global__ void k_ep_coef(int kind, int nel, int ld, const int *__restrict__ eorder, const double *__restrict__ A64,
                          double *__restrict__ coef)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nel) return;
    double a[9];
    for (int m = 0; m < 9; ++m) a[m] = A64[(size_t)m * ld + p];
    double *L = coef + 9 * (size_t)eorder[p];
    if (kind == 1) {
        L[0] = 1.0;
        L[1] = a[1];
        L[2] = a[2];
        L[3] = a[3];
        L[4] = 1. / (1.0 - a[1] * a[3]);
        L[5] = a[5] - a[2] * a[3];
        L[6] = a[6];
        L[7] = (a[7] - a[1] * a[6]) * L[4];
        L[8] = 1. / (1.0 - a[2] * a[6] - L[7] * L[5]);
    } else {
        for (int m = 0; m < 9; ++m) L[m] = a[m];
    }
}

// out = in (n + 1 entries, the whole CTA), then the sweep on out by warp 0:
// kind 1 LU, 2 SGS forward (elements ascending), 3 SGS backward (elements
// descending).  Must be the CTA's last step (warp 0 alone goes on).
__device__ void elem_sweep(int kind, int nel, int n, const int *__restrict__ lmi, const double *__restrict__ coef,
                           const double *in, double *out)
{
    __shared__ int s_l[2][32][3];
    __shared__ double s_c[2][32][9];
    if (in != out)
        for (int i = threadIdx.x; i <= n; i += blockDim.x) out[i] = in[i];
    __syncthreads();
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x, nch = (nel + 31) / 32;
    int rl[3] = {n, n, n};
    double rc[9];
    for (int m = 0; m < 9; ++m) rc[m] = 0.0;
    auto load = [&](int c) {                          // element record of this lane in chunk c
        const int t = c * 32 + lane;
        if (c < nch && t < nel) {
            const int I = kind == 3 ? nel - 1 - t : t;
            for (int a = 0; a < 3; ++a) rl[a] = lmi[3 * (size_t)I + a];
            for (int m = 0; m < 9; ++m) rc[m] = coef[9 * (size_t)I + m];
        }
    };
    auto store = [&](int b) {
        for (int a = 0; a < 3; ++a) s_l[b][lane][a] = rl[a];
        for (int m = 0; m < 9; ++m) s_c[b][lane][m] = rc[m];
    };
    load(0);
    store(0);
    if (lane == 0) out[n] = 0.0;
    __syncwarp();
    for (int c = 0; c < nch; ++c) {
        load(c + 1);                                  // in flight while lane 0 works
        if (lane == 0) {
            const int cnt = min(32, nel - c * 32), b = c & 1;
            for (int e = 0; e < cnt; ++e) {
                const int l0 = s_l[b][e][0], l1 = s_l[b][e][1], l2 = s_l[b][e][2];
                const double *L = s_c[b][e];
                double z0 = out[l0], z1 = out[l1], z2 = out[l2];
                if (kind == 1) {
                    z1 += -L[3] * z0;
                    z2 += -L[6] * z0 - L[7] * z1;
                    z2 *= L[8];
                    z1 = (z1 - L[5] * z2) * L[4];
                    z0 += -L[1] * z1 - L[2] * z2;
                    out[l0] = z0;
                    out[l1] = z1;
                    out[l2] = z2;
                } else if (kind == 2) {
                    z1 += -L[3] * z0;
                    z2 += -L[6] * z0 - L[7] * z1;
                    out[l1] = z1;
                    out[l2] = z2;
                } else {
                    z1 += -L[5] * z2;
                    z0 += -L[1] * z1 - L[2] * z2;
                    out[l0] = z0;
                    out[l1] = z1;
                }
                out[n] = 0.0;
            }
        }
        __syncwarp();
        store((c + 1) & 1);
        __syncwarp();
    }
}

// one system: in -> out (device vectors, internal numbering)
__global__ void k_elem_prec1(int kind, int nel, int n, const int *lmi, const double *coef, const double *in,
                             double *out)
{
    elem_sweep(kind, nel, n, lmi, coef, in, out);
}

// a batch, a CTA per system (see launch_elem_prec)
__global__ void k_elem_prec(const SysDev *__restrict__ sys, int kind, int sel, int step)
{
    const SysDev &D = sys[blockIdx.x];
    if (sel == 0 ? !D.st->live : sel == 1 ? !D.st->in_cycle : false) return;
    const double *in;
    double *out;
    if (kind == 3) {
        in = sel == 0 || sel == 2 ? D.x : (const double *)D.V + (size_t)step * D.n_pad;
        out = sel == 2 ? D.x : D.r64;
    } else {
        in = sel == 0 ? D.t64 : (const double *)D.t;
        out = sel == 0 ? D.u64 : (double *)D.w;
    }
    elem_sweep(kind, D.nel, D.n, D.ep_lmi, D.ep_coef, in, out);
}

int launch_elem_prec(const SysDev *sys, int nsys, int kind, int sel, int step, cudaStream_t st)
{
    if (nsys > 0) k_elem_prec<<<nsys, 128, 0, st>>>(sys, kind, sel, step);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

// the per-element records of a system (host connectivity, device blocks)
static int elem_prec_setup(fg_system *s, int kind, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (t.S != 3 || s->op != FG_OP_EBE) {
        set_error("the element preconditioners LUe / SGSe need 3x3 blocks on the EBE operator");
        return FG_ERR_UNSUPPORTED;
    }
    int r;
    if (!s->ep_lmi.p) {
        std::vector<int> lmi(3 * (size_t)std::max(t.nel, 1), t.n);
        for (int I = 0; I < t.nel; ++I)
            for (int a = 0; a < 3; ++a) {
                const int q = t.lm[3 * (size_t)I + a];
                lmi[3 * (size_t)I + a] = q == t.n ? t.n : t.iperm[q];
            }
        if ((r = s->ep_lmi.alloc(sizeof(int) * lmi.size()))) return r;
        FG_CUDA(cudaMemcpy(s->ep_lmi.p, lmi.data(), sizeof(int) * lmi.size(), cudaMemcpyHostToDevice));
    }
    if (!s->ep_coef.p && (r = s->ep_coef.alloc(sizeof(double) * 9 * (size_t)std::max(t.nel, 1)))) return r;
    if (t.nel > 0)
        k_ep_coef<<<(t.nel + 127) / 128, 128, 0, st>>>(kind == FG_PRECOND_LUE ? 1 : 2, t.nel, s->nel_pad,
                                                       s->eorder.as<int>(), s->A64.as<double>(),
                                                       s->ep_coef.as<double>());
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

// z = M^-1 p (left) or z = R p (right, SGSe only; the identity otherwise)
int elem_prec_apply_device(fg_system *s, bool right, const double *p, double *z, cudaStream_t st)
{
    const Topology &t = s->topo;
    const bool sgs = s->precond == FG_PRECOND_SGSE;
    if (right && !sgs) {
        if (p != z) FG_CUDA(cudaMemcpyAsync(z, p, 8 * (size_t)(t.n + 1), cudaMemcpyDeviceToDevice, st));
        return FG_OK;
    }
    const int kind = right ? 3 : sgs ? 2 : 1;
    k_elem_prec1<<<1, 128, 0, st>>>(kind, t.nel, t.n, s->ep_lmi.as<int>(), s->ep_coef.as<double>(), p, z);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

// ---------------------------------------------------------------- diagonal scaling
// Left_scaling_EBE / LeftRight_scaling_EBE (scaling.c:10-42, 92-121) on the
// blocks of the internal element order: row I of element e times invDiag of
// its equation (left), or entry (I, J) times sqrt(invDiag_I invDiag_J)
// (left-right); the sink n reads invDiag[n], which the caller set to the
// reference's invDiag[NEQ] = invDiag[NEQ - 1].
__global__ void k_scale_blocks(int nel, int ld, int S, const int *__restrict__ lm, const double *__restrict__ invd,
                               int both, double *__restrict__ A64)
{
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    for (int I = 0; I < S; ++I) {
        const double dI = invd[lm[(size_t)I * ld + pos]];
        for (int J = 0; J < S; ++J) {
            double &a = A64[(size_t)(I * S + J) * ld + pos];
            if (both) a *= sqrt(dI * invd[lm[(size_t)J * ld + pos]]);
            else a *= dI;
        }
    }
}

// x[i] *= sqrt(v[i]) for i < n (F of the left-right scaling with v = Diag;
// Left_unscaling, scaling.c:187-196, with v = invDiag)
__global__ void k_mul_sqrt(int n, const double *__restrict__ v, double *__restrict__ x)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] *= sqrt(v[i]);
}

// Block_scaling_EBE's element part: Dirichlet rows and columns of the block
// cleared with 1 on the diagonal (matrix_Bondary_Conditions), then each row
// block of node v replaced by inv(v) times it (matrix_Scaling: sums from 0
// in j order).  One thread per element; the block is read whole first.
template <int B>
__global__ void k_block_scale(int nel, int ld, int n, const int *__restrict__ gien, const int *__restrict__ node_dof,
                              const double *__restrict__ ibd, double *__restrict__ A64)
{
    constexpr int S = 3 * B;
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    double m[S * S];
    for (int q = 0; q < S * S; ++q) m[q] = A64[(size_t)q * ld + pos];
    int J[3];
    for (int v = 0; v < 3; ++v) J[v] = gien[(size_t)v * ld + pos];
    for (int I = 0; I < B; ++I)
        for (int v = 0; v < 3; ++v) {
            if (node_dof[B * J[v] + I] != n) continue;
            const int d = B * v + I;
            for (int t = 0; t < S; ++t) { m[d * S + t] = 0.0; m[t * S + d] = 0.0; }
            m[d * S + d] = 1.0;
        }
    for (int v = 0; v < 3; ++v) {
        const double *iv = ibd + (size_t)B * B * J[v];
        for (int i = 0; i < B; ++i)
            for (int col = 0; col < S; ++col) {
                double a = 0.0;
                for (int j = 0; j < B; ++j) a += iv[i * B + j] * m[(B * v + j) * S + col];
                A64[(size_t)((B * v + i) * S + col) * ld + pos] = a;
            }
    }
}

int scale_device(fg_system *s, int kind, double *F_dev, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (!s->blocks_ok) { set_error("scaling before element blocks were set"); return FG_ERR_STATE; }
    if (kind != FG_SCALE_LEFT && kind != FG_SCALE_LEFTRIGHT && kind != FG_SCALE_BLOCK) {
        set_error("unknown scaling"); return FG_ERR_ARG;
    }
    int r;
    if (kind == FG_SCALE_BLOCK) {
        const int B = t.ndof;
        if (B < 2 || B > 4) { set_error("block scaling needs ndof 2..4"); return FG_ERR_UNSUPPORTED; }
        if ((r = precond_setup_device(s, FG_PRECOND_BLOCKDIAG, B == 4 ? FG_SETUP_REF_QUIRKS : 0, F_dev, st))) return r;
        if (t.nel > 0) {
            const dim3 g((t.nel + 63) / 64);
            if (B == 2) k_block_scale<2><<<g, 64, 0, st>>>(t.nel, s->nel_pad, t.n, s->gien.as<int>(), s->node_dof.as<int>(), s->ibd64.as<double>(), s->A64.as<double>());
            else if (B == 3) k_block_scale<3><<<g, 64, 0, st>>>(t.nel, s->nel_pad, t.n, s->gien.as<int>(), s->node_dof.as<int>(), s->ibd64.as<double>(), s->A64.as<double>());
            else k_block_scale<4><<<g, 64, 0, st>>>(t.nel, s->nel_pad, t.n, s->gien.as<int>(), s->node_dof.as<int>(), s->ibd64.as<double>(), s->A64.as<double>());
            FG_CUDA(cudaGetLastError());
            count_launches(1);
        }
        s->scale_kind = kind;
        s->precond = FG_PRECOND_NONE;
        s->csr_dirty = true;
        return convert_blocks(s, st);
    }
    if ((r = precond_setup_device(s, FG_PRECOND_DIAG, FG_SETUP_ACCUMULATE, F_dev, st))) return r;
    double *invd = s->invd64.as<double>();
    if (t.n > 0)                                      // invDiag[NEQ] = invDiag[NEQ - 1] (reference numbering)
        FG_CUDA(cudaMemcpyAsync(invd + t.n, invd + t.iperm[t.n - 1], sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (t.nel > 0)
        k_scale_blocks<<<(t.nel + 127) / 128, 128, 0, st>>>(t.nel, s->nel_pad, t.S, s->lm.as<int>(), invd,
                                                           kind == FG_SCALE_LEFTRIGHT, s->A64.as<double>());
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    if (kind == FG_SCALE_LEFTRIGHT && F_dev && t.n > 0) {
        k_mul_sqrt<<<(t.n + 255) / 256, 256, 0, st>>>(t.n, s->diag.as<double>(), F_dev);
        FG_CUDA(cudaGetLastError());
        count_launches(1);
    }
    s->scale_kind = kind;
    s->precond = FG_PRECOND_NONE;                    // the scaled system is solved as it stands
    s->csr_dirty = true;
    return convert_blocks(s, st);
}

int unscale_device(fg_system *s, double *x_dev, cudaStream_t st)
{
    const int n = s->topo.n;
    if (s->scale_kind == FG_SCALE_BLOCK) return FG_OK;   // NO_unscaling
    if (n > 0) k_mul_sqrt<<<(n + 255) / 256, 256, 0, st>>>(n, s->invd64.as<double>(), x_dev);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

__global__ void k_diag_apply(const double *__restrict__ invd, int n, const double *p, double *z)
{
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d < n) z[d] = p[d] * invd[d];
    if (d == n) z[n] = 0.0;
}

int precond_apply_device(fg_system *s, const double *p, double *z, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (s->precond == FG_PRECOND_ILU0) return ilu0_apply_device(s, p, z, st);
    if (s->precond == FG_PRECOND_SPIKE) return spike_apply_device(s, p, z, st);
    if (s->precond == FG_PRECOND_LUE || s->precond == FG_PRECOND_SGSE) return elem_prec_apply_device(s, false, p, z, st);
    if (s->precond == FG_PRECOND_DIAG) {
        k_diag_apply<<<(t.n + 256) / 256, 256, 0, st>>>(s->invd64.as<double>(), t.n, p, z);
    } else if (s->precond == FG_PRECOND_BLOCKDIAG) {
        int g = (t.nnodes + 127) / 128, B = t.ndof;
        if (p != z) FG_CUDA(cudaMemcpyAsync(z, p, 8 * (size_t)(t.n + 1), cudaMemcpyDeviceToDevice, st));
        // in place is safe: each node reads its own dofs before writing them
        if (B == 4) k_blockdiag_apply64<4><<<g, 128, 0, st>>>(s->node_dof.as<int>(), s->ibd64.as<double>(), t.nnodes, t.n, z, z);
        else if (B == 3) k_blockdiag_apply64<3><<<g, 128, 0, st>>>(s->node_dof.as<int>(), s->ibd64.as<double>(), t.nnodes, t.n, z, z);
        else k_blockdiag_apply64<2><<<g, 128, 0, st>>>(s->node_dof.as<int>(), s->ibd64.as<double>(), t.nnodes, t.n, z, z);
    } else if (p != z) {
        FG_CUDA(cudaMemcpyAsync(z, p, 8 * (size_t)(t.n + 1), cudaMemcpyDeviceToDevice, st));
    }
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

// ---------------------------------------------------------------- SUPG/CAU transport
// Build_K_F_SUPG.c:47-177 with CAU_ShockCapture.c:3-31 and
// h_shock_2sqrtArea.c, one thread per element (internal order).  Writes the
// 3x3 block (ebe_assembly.c) into the SoA layout and the element load
// vector Fe; the Dirichlet lifting is applied in k_transport_F.
// YZBeta_ShockCapture.c:3-36: YZ-beta (beta = 1 and 2) relaxed against the
// element's previous value; Re_old / delta_old (per element, internal
// order) carry the state across the builds of one Process run.
__device__ double yzbeta_eu(double *Re_old, double *delta_old, int e, double bx, double by, double gamma,
                            double ue1, double ue2, double ue3, double ueb, double feb, double y23, double y31,
                            double y12, double x32, double x13, double x21, double invArea, double h)
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

// h_shock_calculation: 0 h_shock_2sqrtArea.c, 1 h_shock_Option1.c:3-19
// (from grad u), 2 h_shock_Option2.c:3-16 (from the velocity)
__device__ double h_shock_dev(int opt, double bx, double by, double u1, double u2, double u3, double y23, double y31,
                              double y12, double x32, double x13, double x21, double Area)
{
    if (opt == 1) {
        double P1 = fabs(u1*y23*y23 + u2*y31*y23 + u3*y12*y23 + u1*x32*x32 + u2*x13*x32 + u3*x21*x32);
        double P2 = fabs(u1*y23*y31 + u2*y31*y31 + u3*y12*y31 + u1*x32*x13 + u2*x13*x13 + u3*x21*x13);
        double P3 = fabs(u1*y23*y12 + u2*y31*y12 + u3*y12*y12 + u1*x32*x21 + u2*x13*x21 + u3*x21*x21);
        double a1 = y23*u1 + y31*u2 + y12*u3, a2 = x32*u1 + x13*u2 + x21*u3;
        double ng = sqrt(a1*a1 + a2*a2);
        return P1 + P2 + P3 >= 1e-12 ? 4*Area*ng/(P1 + P2 + P3) : 0.0;
    }
    if (opt == 2) {
        double P1 = fabs(bx*y23 + by*x32), P2 = fabs(bx*y31 + by*x13), P3 = fabs(bx*y12 + by*x21);
        double nb = sqrt(bx*bx + by*by);
        return P1 + P2 + P3 >= 1e-12 ? 4*Area*nb/(P1 + P2 + P3) : 0.0;
    }
    return sqrt(fabs(2*Area));
}

__device__ double cau_eu(double kx, double ky, double bx, double by, double gamma, double ue1, double ue2, double ue3,
                         double ueb, double feb, double y23, double y31, double y12, double x32, double x13,
                         double x21, double invArea, double h)
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

__global__ void k_transport_elem(int nel, int ld, const int *__restrict__ gien, const double *__restrict__ gx,
                                 const double *__restrict__ gy, const int *__restrict__ gtype,
                                 const int *__restrict__ node_dof, const double *__restrict__ up,
                                 const double *__restrict__ u, fg_transport_coeffs cf, double *Re_old,
                                 double *delta_old, double *__restrict__ A64, double *__restrict__ Fe)
{
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const double third = 1.0/3.0, sixth = 1.0/6.0, twelfth = 1.0/12.0;
    const double kx = cf.k, ky = cf.k, gamma = cf.gamma;
    int J1 = gien[pos], J2 = gien[ld + pos], J3 = gien[2 * (size_t)ld + pos];
    double X0 = gx[J1], X1 = gx[J2], X2 = gx[J3];
    double Y0 = gy[J1], Y1 = gy[J2], Y2 = gy[J3];
    double y23 = Y1 - Y2, y31 = Y2 - Y0, y12 = Y0 - Y1;
    double x32 = X2 - X1, x13 = X0 - X2, x21 = X1 - X0;
    double TwoA = x21*y31 - x13*y12;
    double Area = 0.5*TwoA;
    double invArea = 1.0/Area;
    double h = sqrt(fabs(TwoA));
    double bx = cf.beta[0], by = cf.beta[1];
    double norm = sqrt(bx*bx + by*by);
    double tau = norm > 0 ? 0.5*h/norm : 0;
    double fe1 = cf.f, fe2 = cf.f, fe3 = cf.f;
    double feb = third*(fe1 + fe2 + fe3);
    double ue1 = gtype[J1] == 0 ? up[J1] : u[node_dof[J1]];
    double ue2 = gtype[J2] == 0 ? up[J2] : u[node_dof[J2]];
    double ue3 = gtype[J3] == 0 ? up[J3] : u[node_dof[J3]];
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
    double hs = h_shock_dev(cf.h_shock, bx, by, ue1, ue2, ue3, y23, y31, y12, x32, x13, x21, Area);
    double Eu = cf.cau == 3 ? yzbeta_eu(Re_old, delta_old, pos, bx, by, gamma, ue1, ue2, ue3, ueb, feb, y23, y31,
                                        y12, x32, x13, x21, invArea, hs)
              : cf.cau ? cau_eu(kx, ky, bx, by, gamma, ue1, ue2, ue3, ueb, feb, y23, y31, y12, x32, x13, x21,
                                invArea, hs) : 0.0;
    double Csc12 = Eu*0.25*invArea*(y23*y31 + x32*x13);
    double Csc13 = Eu*0.25*invArea*(y23*y12 + x32*x21);
    double Csc23 = Eu*0.25*invArea*(y31*y12 + x13*x21);
    double *a = A64 + pos;
    a[0 * ld] = -(D12 + D13) + C11 - (Cpg12 + Cpg13) + R11 + Rpg11 - (Csc12 + Csc13);
    a[1 * ld] = D12 + C12 + Cpg12 + R12 + Rpg11 + Csc12;
    a[2 * ld] = D13 + C13 + Cpg13 + R12 + Rpg11 + Csc13;
    a[3 * ld] = D12 + C11 + Cpg12 + R12 + Rpg21 + Csc12;
    a[4 * ld] = -(D12 + D23) + C12 - (Cpg12 + Cpg23) + R11 + Rpg21 - (Csc12 + Csc23);
    a[5 * ld] = D23 + C13 + Cpg23 + R12 + Rpg21 + Csc23;
    a[6 * ld] = D13 + C11 + Cpg13 + R12 + Rpg31 + Csc13;
    a[7 * ld] = D23 + C12 + Cpg23 + R12 + Rpg31 + Csc23;
    a[8 * ld] = -(D13 + D23) + C13 - (Cpg13 + Cpg23) + R11 + Rpg31 - (Csc13 + Csc23);
    Fe[pos] = Area*twelfth*(2*fe1 + fe2 + fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y23 + by*x32);
    Fe[ld + pos] = Area*twelfth*(fe1 + 2*fe2 + fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y31 + by*x13);
    Fe[2 * (size_t)ld + pos] = Area*twelfth*(fe1 + fe2 + 2*fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y12 + by*x21);
}

// CAU_DD_ShockCapture.c:3-22: 0.5 h |R(u)| / |grad u| (0 below 1e-10)
__device__ double cau_dd_eu(double bx, double by, double gamma, double ue1, double ue2, double ue3, double ueb,
                            double feb, double y23, double y31, double y12, double x32, double x13, double x21,
                            double invArea, double h)
{
    double bgu = 0.5*invArea*(ue1*(bx*y23 + by*x32) + ue2*(bx*y31 + by*x13) + ue3*(bx*y12 + by*x21));
    double Ru = bgu + gamma*ueb - feb;
    double gx = 0.5*invArea*(y23*ue1 + y31*ue2 + y12*ue3);
    double gy = 0.5*invArea*(x32*ue1 + x13*ue2 + x21*ue3);
    double ng = sqrt(gx*gx + gy*gy);
    return ng > 1e-10 ? 0.5*h*fabs(Ru)/ng : 0.0;
}

// Build_K_F_DD.c:54-164 (StabilizationForm "DD"): Galerkin with dynamic
// diffusion, the element bubble (KBB, KhB, KBh, FB) condensed into the 3x3
// block and the load: ke = Khh - KhB KBh / KBB, Fe = Fh - KhB FB / KBB, each
// term associated as the reference writes it (note R11 = (gamma/6) Area
// here, against gamma Area / 6 in the SUPG build).
__global__ void k_transport_dd_elem(int nel, int ld, const int *__restrict__ gien, const double *__restrict__ gx,
                                    const double *__restrict__ gy, const int *__restrict__ gtype,
                                    const int *__restrict__ node_dof, const double *__restrict__ up,
                                    const double *__restrict__ u, fg_transport_coeffs cf, double *Re_old,
                                    double *delta_old, double *__restrict__ A64, double *__restrict__ Fe)
{
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const double third = 1.0/3.0, sixth = 1.0/6.0, seventh = 1.0/7.0, twelfth = 1.0/12.0;
    const double t320 = 3./20.0, n920 = 9./20.0, n940 = 9./40.0;
    const double kx = cf.k, ky = cf.k, gamma = cf.gamma, bx = cf.beta[0], by = cf.beta[1];
    int J1 = gien[pos], J2 = gien[ld + pos], J3 = gien[2 * (size_t)ld + pos];
    double X0 = gx[J1], X1 = gx[J2], X2 = gx[J3];
    double Y0 = gy[J1], Y1 = gy[J2], Y2 = gy[J3];
    double y23 = Y1 - Y2, y31 = Y2 - Y0, y12 = Y0 - Y1;
    double x32 = X2 - X1, x13 = X0 - X2, x21 = X1 - X0;
    double TwoA = x21*y31 - x13*y12;
    double Area = 0.5*TwoA;
    double invArea = 1.0/Area;
    double fe1 = cf.f, fe2 = cf.f, fe3 = cf.f;
    double feb = third*(fe1 + fe2 + fe3);
    double ue1 = gtype[J1] == 0 ? up[J1] : u[node_dof[J1]];
    double ue2 = gtype[J2] == 0 ? up[J2] : u[node_dof[J2]];
    double ue3 = gtype[J3] == 0 ? up[J3] : u[node_dof[J3]];
    double ueb = third*(ue1 + ue2 + ue3);
    double a1 = bx*y23 + by*x32, a2 = bx*y31 + by*x13, a3 = bx*y12 + by*x21;
    double C12 = y23*y31 + x32*x13, C13 = y23*y12 + x32*x21, C23 = y31*y12 + x13*x21;
    double D12 = 0.25*invArea*((kx*y23*y31) + (ky*x32*x13));
    double D13 = 0.25*invArea*((kx*y23*y12) + (ky*x32*x21));
    double D23 = 0.25*invArea*((kx*y31*y12) + (ky*x13*x21));
    double R11 = sixth*gamma*Area, R12 = twelfth*gamma*Area;
    double h = h_shock_dev(cf.h_shock, bx, by, ue1, ue2, ue3, y23, y31, y12, x32, x13, x21, Area);
    double Eu = 0.0;
    if (cf.cau == 3)
        Eu = yzbeta_eu(Re_old, delta_old, pos, bx, by, gamma, ue1, ue2, ue3, ueb, feb, y23, y31, y12, x32, x13, x21,
                       invArea, h);
    else if (cf.cau == 2)
        Eu = cau_dd_eu(bx, by, gamma, ue1, ue2, ue3, ueb, feb, y23, y31, y12, x32, x13, x21, invArea, h);
    else if (cf.cau == 1)
        Eu = cau_eu(kx, ky, bx, by, gamma, ue1, ue2, ue3, ueb, feb, y23, y31, y12, x32, x13, x21, invArea, h);
    double K12 = 0.25*Eu*invArea*C12, K13 = 0.25*Eu*invArea*C13, K23 = 0.25*Eu*invArea*C23;
    double Khh[9];
    Khh[0] = -(D12 + D13) + sixth*a1 + R11 -(K12 + K13);
    Khh[1] =          D12 + sixth*a2 + R12 + K12;
    Khh[2] =          D13 + sixth*a3 + R12 + K13;
    Khh[3] =          D12 + sixth*a1 + R12 + K12;
    Khh[4] = -(D12 + D23) + sixth*a2 + R11 -(K12 + K23);
    Khh[5] =          D23 + sixth*a3 + R12 + K23;
    Khh[6] =          D13 + sixth*a1 + R12 + K13;
    Khh[7] =          D23 + sixth*a2 + R12 + K23;
    Khh[8] = -(D13 + D23) + sixth*a3 + R11 -(K13 + K23);
    const double KhB[3] = {n920*(0.5*a1 + a2 + a3) + t320*gamma*Area, n920*(a1 + 0.5*a2 + a3) + t320*gamma*Area,
                           n920*(a1 + a2 + 0.5*a3) + t320*gamma*Area};
    const double KBh[3] = {n940*a1 + t320*gamma*Area, n940*a2 + t320*gamma*Area, n940*a3 + t320*gamma*Area};
    double KBB = -9*n940*(D12 + D13 + D23) + seventh*t320*(a1 + a2 + a3) + 9*seventh*n940*Area
               - Eu*invArea*(C12 + C13 + C23)/360.;
    double invKBB = 1.0/KBB;
    const double Fh[3] = {twelfth*Area*(2*fe1 + fe2 + fe3), twelfth*Area*(fe1 + 2*fe2 + fe3),
                          twelfth*Area*(fe1 + fe2 + 2*fe3)};
    double FB = t320*Area*(fe1 + fe2 + fe3);
    double *a = A64 + pos;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) a[(size_t)(3 * i + j) * ld] = Khh[3 * i + j] - invKBB*KhB[i]*KBh[j];
        Fe[(size_t)i * ld + pos] = Fh[i] - invKBB*KhB[i]*FB;
    }
}

// F_assembly (F_assembly.c:3-28) as a gather per free dof, in reference
// element order: F += Fe_a, then F -= ke[a][b] * upresc(b) for the
// Dirichlet vertices b of the element in vertex order.
__global__ void k_transport_F(int n, int ld, const int *__restrict__ dptr, const int *__restrict__ dinc,
                              const int *__restrict__ gien, const int *__restrict__ gtype,
                              const double *__restrict__ up, const double *__restrict__ A64,
                              const double *__restrict__ Fe, double *__restrict__ F)
{
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d > n) return;
    if (d == n) { F[n] = 0.0; return; }
    double s = 0.0;
    for (int q = dptr[d]; q < dptr[d + 1]; ++q) {
        int pos = dinc[q] >> 4, a = dinc[q] & 15;
        s += Fe[(size_t)a * ld + pos];
        for (int b = 0; b < 3; ++b) {
            if (b == a) continue;
            int nb = gien[(size_t)b * ld + pos];
            if (gtype[nb] == 0) s -= A64[(size_t)(a * 3 + b) * ld + pos] * up[nb];
        }
    }
    F[d] = s;
}

// ---------------------------------------------------------------- transient SUPG/CAU transport
// Build_M_K_R_SUPG.c:6-252 (02_Transport_Equation) with its
// CAU_ShockCapture.c:3-33 (the residual includes du/dt), h_shock_2sqrtArea.c
// and eval_U_dU.c, one thread per element (internal order).  Writes the block
// Ae = me + alpha dt ke into the SoA layout and, per element row a, the four
// terms the reference applies to R[lm[a]] in order: + Fe_a, then
// - (me[a][b] du_b + ke[a][b] u_b) for b = 0, 1, 2 (Rt[(4 a + k) ld + pos]).
__device__ double tt_cau_eu(double kx, double ky, double bx, double by, double gamma, double ue1, double ue2,
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

// YZBeta_ShockCapture of the transient driver: no state, Ru includes du/dt
__device__ double tt_yz_eu(double bx, double by, double gamma, double ue1, double ue2, double ue3, double ueb,
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
    return (nu >= 1e-12 && ng >= 1e-12) ? 0.25*h*nRu/ng + 0.125*h*h*nRu/nu : 0.0;
}

__global__ void k_tt_elem(int nel, int ld, const int *__restrict__ gien, const double *__restrict__ gx,
                          const double *__restrict__ gy, const int *__restrict__ gtype,
                          const int *__restrict__ node_dof, const double *__restrict__ up,
                          const double *__restrict__ u, const double *__restrict__ du, fg_tt_coeffs tc,
                          double *__restrict__ A64, double *__restrict__ Rt)
{
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const fg_transport_coeffs &cf = tc.c;
    const double third = 1.0/3.0, sixth = 1.0/6.0, twelfth = 1.0/12.0;
    const double kx = cf.k, ky = cf.k, gamma = cf.gamma;
    int J1 = gien[pos], J2 = gien[ld + pos], J3 = gien[2 * (size_t)ld + pos];
    double X0 = gx[J1], X1 = gx[J2], X2 = gx[J3];
    double Y0 = gy[J1], Y1 = gy[J2], Y2 = gy[J3];
    double y23 = Y1 - Y2, y31 = Y2 - Y0, y12 = Y0 - Y1;
    double x32 = X2 - X1, x13 = X0 - X2, x21 = X1 - X0;
    double TwoA = x21*y31 - x13*y12;
    double Area = 0.5*TwoA;
    double invArea = 1.0/Area;
    double h = sqrt(fabs(TwoA));
    double bx = cf.beta[0], by = cf.beta[1];
    double norm = sqrt(bx*bx + by*by);
    double tau = norm > 0 ? 0.5*h/norm : 0;
    double fe1 = cf.f, fe2 = cf.f, fe3 = cf.f;
    double feb = third*(fe1 + fe2 + fe3);
    const int J[3] = {J1, J2, J3};
    double ue[3], due[3];
    for (int a = 0; a < 3; ++a) {
        const bool fixed = gtype[J[a]] == 0;
        ue[a] = fixed ? up[J[a]] : u[node_dof[J[a]]];
        due[a] = fixed ? 0.0 : du[node_dof[J[a]]];
    }
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
    double hs = h_shock_dev(cf.h_shock, bx, by, ue[0], ue[1], ue[2], y23, y31, y12, x32, x13, x21, Area);
    double Eu = cf.cau == FG_SHOCK_YZBETA ? tt_yz_eu(bx, by, gamma, ue[0], ue[1], ue[2], ueb, dueb, feb, y23, y31, y12,
                                                    x32, x13, x21, invArea, hs)
              : cf.cau ? tt_cau_eu(kx, ky, bx, by, gamma, ue[0], ue[1], ue[2], ueb, dueb, feb, y23, y31, y12, x32,
                                   x13, x21, invArea, hs) : 0.0;
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
    const double adt = tc.alpha*tc.dt;
    double *A = A64 + pos;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) A[(size_t)(3 * a + b) * ld] = me[a][b] + adt*ke[a][b];
    const double Fe[3] = {Area*twelfth*(2*fe1 + fe2 + fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y23 + by*x32),
                          Area*twelfth*(fe1 + 2*fe2 + fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y31 + by*x13),
                          Area*twelfth*(fe1 + fe2 + 2*fe3) + sixth*tau*(fe1+fe2+fe3)*(bx*y12 + by*x21)};
    for (int a = 0; a < 3; ++a) {
        Rt[(size_t)(4 * a) * ld + pos] = Fe[a];
        for (int b = 0; b < 3; ++b) Rt[(size_t)(4 * a + 1 + b) * ld + pos] = me[a][b]*due[b] + ke[a][b]*ue[b];
    }
}

// Build_M_K_R_DD.c:61-180 (StabilizationForm "DD", Predictor1): the steady
// DD element (bubble condensed into the block and the load) with its mass
// block me = Mhh - KhB MBh / KBB (+ Mhh on the diagonal), Ae = me + alpha dt
// ke, and the transient CAUDD (Ru with du/dt) relaxed against the element's
// previous value, cb = (cbtil + cbtil_old) / 2, cbtil_old in cbtilo (per
// element, internal order, kept for the whole time loop).  Same residual
// slots as k_tt_elem.
__global__ void k_tt_dd_elem(int nel, int ld, const int *__restrict__ gien, const double *__restrict__ gx,
                             const double *__restrict__ gy, const int *__restrict__ gtype,
                             const int *__restrict__ node_dof, const double *__restrict__ up,
                             const double *__restrict__ u, const double *__restrict__ du, fg_tt_coeffs tc,
                             double *cbtilo, double *__restrict__ A64, double *__restrict__ Rt)
{
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const fg_transport_coeffs &cf = tc.c;
    const double third = 1.0/3.0, sixth = 1.0/6.0, seventh = 1.0/7.0, twelfth = 1.0/12.0;
    const double t320 = 3./20.0, n920 = 9./20.0, n940 = 9./40.0, w = 0.5;
    const double kx = cf.k, ky = cf.k, gamma = cf.gamma, bx = cf.beta[0], by = cf.beta[1];
    int J1 = gien[pos], J2 = gien[ld + pos], J3 = gien[2 * (size_t)ld + pos];
    double X0 = gx[J1], X1 = gx[J2], X2 = gx[J3];
    double Y0 = gy[J1], Y1 = gy[J2], Y2 = gy[J3];
    double y23 = Y1 - Y2, y31 = Y2 - Y0, y12 = Y0 - Y1;
    double x32 = X2 - X1, x13 = X0 - X2, x21 = X1 - X0;
    double TwoA = x21*y31 - x13*y12;
    double Area = 0.5*TwoA;
    double invArea = 1.0/Area;
    double fe1 = cf.f, fe2 = cf.f, fe3 = cf.f;
    double feb = third*(fe1 + fe2 + fe3);
    const int J[3] = {J1, J2, J3};
    double ue[3], due[3];
    for (int a = 0; a < 3; ++a) {
        const bool fixed = gtype[J[a]] == 0;
        ue[a] = fixed ? up[J[a]] : u[node_dof[J[a]]];
        due[a] = fixed ? 0.0 : du[node_dof[J[a]]];
    }
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
    if (cf.cau == FG_SHOCK_CAUDD || cf.cau == FG_SHOCK_YZBETA) {
        double h = h_shock_dev(cf.h_shock, bx, by, ue[0], ue[1], ue[2], y23, y31, y12, x32, x13, x21, Area);
        double cbtil;
        if (cf.cau == FG_SHOCK_YZBETA) {
            cbtil = tt_yz_eu(bx, by, gamma, ue[0], ue[1], ue[2], ueb, dueb, feb, y23, y31, y12, x32, x13, x21, invArea, h);
        } else {
            double bgu = 0.5*invArea*(ue[0]*(bx*y23 + by*x32) + ue[1]*(bx*y31 + by*x13) + ue[2]*(bx*y12 + by*x21));
            double Ru = dueb + bgu + gamma*ueb - feb;
            double gxu = 0.5*invArea*(y23*ue[0] + y31*ue[1] + y12*ue[2]);
            double gyu = 0.5*invArea*(x32*ue[0] + x13*ue[1] + x21*ue[2]);
            double ng = sqrt(gxu*gxu + gyu*gyu);
            cbtil = ng > 1e-10 ? 0.5*h*fabs(Ru)/ng : 0.0;
        }
        double cb = w*cbtil + (1 - w)*cbtilo[pos];
        cbtilo[pos] = cbtil;
        Eu = cb;
    }
    double K12 = 0.25*Eu*invArea*C12, K13 = 0.25*Eu*invArea*C13, K23 = 0.25*Eu*invArea*C23;
    double Khh[9];
    Khh[0] = -(D12 + D13) + sixth*a1 + R11 -(K12 + K13);
    Khh[1] =          D12 + sixth*a2 + R12 + K12;
    Khh[2] =          D13 + sixth*a3 + R12 + K13;
    Khh[3] =          D12 + sixth*a1 + R12 + K12;
    Khh[4] = -(D12 + D23) + sixth*a2 + R11 -(K12 + K23);
    Khh[5] =          D23 + sixth*a3 + R12 + K23;
    Khh[6] =          D13 + sixth*a1 + R12 + K13;
    Khh[7] =          D23 + sixth*a2 + R12 + K23;
    Khh[8] = -(D13 + D23) + sixth*a3 + R11 -(K13 + K23);
    const double KhB[3] = {n920*(0.5*a1 + a2 + a3) + t320*gamma*Area, n920*(a1 + 0.5*a2 + a3) + t320*gamma*Area,
                           n920*(a1 + a2 + 0.5*a3) + t320*gamma*Area};
    const double KBh[3] = {n940*a1 + t320*gamma*Area, n940*a2 + t320*gamma*Area, n940*a3 + t320*gamma*Area};
    double KBB = -9*n940*(D12 + D13 + D23) + seventh*t320*(a1 + a2 + a3) + 9*seventh*n940*Area
               - Eu*invArea*(C12 + C13 + C23)/360.;
    double invKBB = 1.0/KBB;
    const double Fh[3] = {twelfth*Area*(2*fe1 + fe2 + fe3), twelfth*Area*(fe1 + 2*fe2 + fe3),
                          twelfth*Area*(fe1 + fe2 + 2*fe3)};
    double FB = t320*Area*(fe1 + fe2 + fe3);
    const double adt = tc.alpha*tc.dt;
    double *A = A64 + pos;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double me[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) me[j] = Mhh - invKBB*KhB[i]*MBh;
        me[i] += Mhh;
        Rt[(size_t)(4 * i) * ld + pos] = Fh[i] - invKBB*KhB[i]*FB;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const double ke = Khh[3 * i + j] - invKBB*KhB[i]*KBh[j];
            A[(size_t)(3 * i + j) * ld] = me[j] + adt*ke;
            Rt[(size_t)(4 * i + 1 + j) * ld + pos] = me[j]*due[j] + ke*ue[j];
        }
    }
}

// Build_M_F_DD.c:52-244 (TimeIntegration "Predictor2", form DD), a thread
// per element: the element's bubble kept as an unknown (uB, duB in the
// bubble planes, internal element position) and condensed out with
// N2 = MBB + alpha dt KBB.  Writes Me into the blocks, the load
// R1 - invN2 N1 R2 of vertex i into Rt plane 4 i (one term per incidence),
// and invN2, R2, M2[0..2] into the bubble planes for the correction
// (calculate_DaB).  The shock capture is relaxed against cbtilo as in
// k_tt_dd_elem.
__global__ void k_tt_mfdd_elem(int nel, int ld, const int *__restrict__ gien, const double *__restrict__ gx,
                               const double *__restrict__ gy, const int *__restrict__ gtype,
                               const int *__restrict__ node_dof, const double *__restrict__ up,
                               const double *__restrict__ u, const double *__restrict__ du, fg_tt_coeffs tc,
                               double *cbtilo, double *__restrict__ bub, double *__restrict__ A64,
                               double *__restrict__ Rt)
{
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    const fg_transport_coeffs &cf = tc.c;
    const double third = 1.0/3.0, sixth = 1.0/6.0, seventh = 1.0/7.0, twelfth = 1.0/12.0;
    const double t320 = 3./20.0, n920 = 9./20.0, n940 = 9./40.0, w = 0.5;
    const double kx = cf.k, ky = cf.k, gamma = cf.gamma, bx = cf.beta[0], by = cf.beta[1];
    int J1 = gien[pos], J2 = gien[ld + pos], J3 = gien[2 * (size_t)ld + pos];
    double X0 = gx[J1], X1 = gx[J2], X2 = gx[J3];
    double Y0 = gy[J1], Y1 = gy[J2], Y2 = gy[J3];
    double y23 = Y1 - Y2, y31 = Y2 - Y0, y12 = Y0 - Y1;
    double x32 = X2 - X1, x13 = X0 - X2, x21 = X1 - X0;
    double TwoA = x21*y31 - x13*y12;
    double Area = 0.5*TwoA;
    double invArea = 1.0/Area;
    double fe1 = cf.f, fe2 = cf.f, fe3 = cf.f;
    double feb = third*(fe1 + fe2 + fe3);
    const int J[3] = {J1, J2, J3};
    double ue[3], due[3];
    for (int a = 0; a < 3; ++a) {
        const bool fixed = gtype[J[a]] == 0;
        ue[a] = fixed ? up[J[a]] : u[node_dof[J[a]]];
        due[a] = fixed ? 0.0 : du[node_dof[J[a]]];
    }
    const double uB = bub[pos], duB = bub[(size_t)ld + pos];
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
    if (cf.cau == FG_SHOCK_CAUDD || cf.cau == FG_SHOCK_YZBETA) {
        double h = h_shock_dev(cf.h_shock, bx, by, ue[0], ue[1], ue[2], y23, y31, y12, x32, x13, x21, Area);
        double cbtil;
        if (cf.cau == FG_SHOCK_YZBETA) {
            cbtil = tt_yz_eu(bx, by, gamma, ue[0], ue[1], ue[2], ueb, dueb, feb, y23, y31, y12, x32, x13, x21, invArea, h);
        } else {
            double bgu = 0.5*invArea*(ue[0]*(bx*y23 + by*x32) + ue[1]*(bx*y31 + by*x13) + ue[2]*(bx*y12 + by*x21));
            double Ru = dueb + bgu + gamma*ueb - feb;
            double gxu = 0.5*invArea*(y23*ue[0] + y31*ue[1] + y12*ue[2]);
            double gyu = 0.5*invArea*(x32*ue[0] + x13*ue[1] + x21*ue[2]);
            double ng = sqrt(gxu*gxu + gyu*gyu);
            cbtil = ng > 1e-10 ? 0.5*h*fabs(Ru)/ng : 0.0;
        }
        double cb = w*cbtil + (1 - w)*cbtilo[pos];
        cbtilo[pos] = cbtil;
        Eu = cb;
    }
    double K12 = 0.25*Eu*invArea*C12, K13 = 0.25*Eu*invArea*C13, K23 = 0.25*Eu*invArea*C23;
    double Khh[9];
    Khh[0] = -(D12 + D13) + sixth*a1 + R11 -(K12 + K13);
    Khh[1] =          D12 + sixth*a2 + R12 + K12;
    Khh[2] =          D13 + sixth*a3 + R12 + K13;
    Khh[3] =          D12 + sixth*a1 + R12 + K12;
    Khh[4] = -(D12 + D23) + sixth*a2 + R11 -(K12 + K23);
    Khh[5] =          D23 + sixth*a3 + R12 + K23;
    Khh[6] =          D13 + sixth*a1 + R12 + K13;
    Khh[7] =          D23 + sixth*a2 + R12 + K23;
    Khh[8] = -(D13 + D23) + sixth*a3 + R11 -(K13 + K23);
    const double KhB[3] = {n920*(0.5*a1 + a2 + a3) + t320*gamma*Area, n920*(a1 + 0.5*a2 + a3) + t320*gamma*Area,
                           n920*(a1 + a2 + 0.5*a3) + t320*gamma*Area};
    const double KBh[3] = {n940*a1 + t320*gamma*Area, n940*a2 + t320*gamma*Area, n940*a3 + t320*gamma*Area};
    double KBB = -9*n940*(D12 + D13 + D23) + seventh*t320*(a1 + a2 + a3) + 9*seventh*n940*Area
               - Eu*invArea*(C12 + C13 + C23)/360.;
    const double Fh[3] = {twelfth*Area*(2*fe1 + fe2 + fe3), twelfth*Area*(fe1 + 2*fe2 + fe3),
                          twelfth*Area*(fe1 + fe2 + 2*fe3)};
    double FB = t320*Area*(fe1 + fe2 + fe3);
    const double alpha = tc.alpha, dt = tc.dt;
    double N2 = MBB + alpha*dt*KBB;
    double invN2 = 1.0/N2;
    double R2 = FB - MBB*duB - KBB*uB;
    double M1[9], M2[3], N1[3], R1[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        M1[3 * i] = Mhh;
        M1[3 * i + 1] = Mhh;
        M1[3 * i + 2] = Mhh;
        M1[3 * i + i] += Mhh;
        M2[i] = MBh + alpha*dt*KBh[i];
        N1[i] = MhB + alpha*dt*KhB[i];
        R1[i] = Fh[i] - MhB*duB - KhB[i]*uB;
        R1[i] -= Mhh*due[i];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            M1[3 * i + j] += alpha*dt*Khh[3 * i + j];
            R1[i] -= Mhh*due[j] + Khh[3 * i + j]*ue[j];
        }
        R2 -= MBh*due[i] + KBh[i]*ue[i];
    }
    double *A = A64 + pos;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) A[(size_t)(3 * i + j) * ld] = M1[3 * i + j] - invN2*N1[i]*M2[j];
        Rt[(size_t)(4 * i) * ld + pos] = R1[i] - invN2*N1[i]*R2;
    }
    bub[2 * (size_t)ld + pos] = invN2;
    bub[3 * (size_t)ld + pos] = R2;
    bub[4 * (size_t)ld + pos] = M2[0];
    bub[5 * (size_t)ld + pos] = M2[1];
    bub[6 * (size_t)ld + pos] = M2[2];
}

// calculate_DaB.c:16-27 from the solve's Da (internal numbering; the sink,
// a prescribed vertex, reads 0 as Da[NEQ] = 0 there), then Predictor_New.c:
// 104-105: aB += DaB, uB += coef DaB (update), or DaB into out (!update).
__global__ void k_tt_bubble_correct(int nel, int ld, const int *__restrict__ gien, const int *__restrict__ gtype,
                                    const int *__restrict__ node_dof, const double *__restrict__ Da, double coef,
                                    int update, double *__restrict__ bub, double *__restrict__ out)
{
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    double d[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int J = gien[(size_t)a * ld + pos];
        d[a] = gtype[J] == 0 ? 0.0 : Da[node_dof[J]];
    }
    const double M2Da = bub[4 * (size_t)ld + pos]*d[0] + bub[5 * (size_t)ld + pos]*d[1] + bub[6 * (size_t)ld + pos]*d[2];
    const double DaB = bub[2 * (size_t)ld + pos]*(bub[3 * (size_t)ld + pos] - M2Da);
    if (update) {
        bub[(size_t)ld + pos] += DaB;
        bub[pos] += coef*DaB;
    } else {
        out[pos] = DaB;
    }
}

// Predictor_New.c:82-83: uB += coef aB, aB = 0
__global__ void k_tt_bubble_predict(int nel, int ld, double coef, double *__restrict__ bub)
{
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= nel) return;
    bub[pos] += coef*bub[(size_t)ld + pos];
    bub[(size_t)ld + pos] = 0.0;
}

// R[d]: the element terms of dof d in reference element order, applied as
// the reference applies them (R += Fe, then three subtractions unless the
// build has one term per incidence); R[n] = 0.
template <bool SUB>
__global__ void k_tt_R(int n, int ld, const int *__restrict__ dptr, const int *__restrict__ dinc,
                       const double *__restrict__ Rt, double *__restrict__ R)
{
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d > n) return;
    if (d == n) { R[n] = 0.0; return; }
    double s = 0.0;
    for (int q = dptr[d]; q < dptr[d + 1]; ++q) {
        const int pos = dinc[q] >> 4, a = dinc[q] & 15;
        s += Rt[(size_t)(4 * a) * ld + pos];
        if (SUB) {
            s -= Rt[(size_t)(4 * a + 1) * ld + pos];
            s -= Rt[(size_t)(4 * a + 2) * ld + pos];
            s -= Rt[(size_t)(4 * a + 3) * ld + pos];
        }
    }
    R[d] = s;
}

int tt_assemble_device(fg_system *s, const fg_tt_coeffs *c, const double *u_dev, const double *du_dev, double *R_dev,
                       cudaStream_t st)
{
    const Topology &t = s->topo;
    if (t.ndof != 1) { set_error("transient transport assembly needs ndof == 1"); return FG_ERR_UNSUPPORTED; }
    if (!s->geometry_ok) { set_error("transient transport assembly before fg_set_geometry"); return FG_ERR_STATE; }
    const bool dd = c->c.form == FG_TRANSPORT_DD;
    if (c->c.h_shock < FG_HSHOCK_2SQRTAREA || c->c.h_shock > FG_HSHOCK_OPTION2 ||
        (dd ? (c->c.cau != FG_SHOCK_NONE && c->c.cau != FG_SHOCK_CAUDD && c->c.cau != FG_SHOCK_YZBETA)
            : (c->c.form != FG_TRANSPORT_SUPG || c->c.cau == FG_SHOCK_CAUDD || c->c.cau < FG_SHOCK_NONE ||
               c->c.cau > FG_SHOCK_YZBETA))) {
        set_error("transient transport builds SUPG with CAU, YZBeta or none, or DD with CAUDD, YZBeta or none");
        return FG_ERR_UNSUPPORTED;
    }
    double *cbtilo = nullptr;
    if (dd && (c->c.cau == FG_SHOCK_CAUDD || c->c.cau == FG_SHOCK_YZBETA)) {   // delta_old of the time loop, zero at its start
        int r0;
        if (s->shock_state.bytes < 16 * (size_t)s->nel_pad && (r0 = s->shock_state.alloc(16 * (size_t)s->nel_pad)))
            return r0;
        cbtilo = s->shock_state.as<double>() + s->nel_pad;
    }
    int r;
    if (s->Fe.bytes < 8 * (size_t)12 * s->nel_pad && (r = s->Fe.alloc(8 * (size_t)12 * s->nel_pad))) return r;
    if (t.nel > 0 && dd)
        k_tt_dd_elem<<<(t.nel + 127) / 128, 128, 0, st>>>(t.nel, s->nel_pad, s->gien.as<int>(), s->gx.as<double>(),
                                                         s->gy.as<double>(), s->gtype.as<int>(),
                                                         s->node_dof.as<int>(), s->gup.as<double>(), u_dev, du_dev, *c,
                                                         cbtilo, s->A64.as<double>(), s->Fe.as<double>());
    else if (t.nel > 0)
        k_tt_elem<<<(t.nel + 127) / 128, 128, 0, st>>>(t.nel, s->nel_pad, s->gien.as<int>(), s->gx.as<double>(),
                                                      s->gy.as<double>(), s->gtype.as<int>(), s->node_dof.as<int>(),
                                                      s->gup.as<double>(), u_dev, du_dev, *c, s->A64.as<double>(),
                                                      s->Fe.as<double>());
    FG_CUDA(cudaGetLastError());
    k_tt_R<true><<<(t.n + 256) / 256, 256, 0, st>>>(t.n, s->nel_pad, s->dinc_ptr.as<int>(), s->dinc.as<int>(),
                                                   s->Fe.as<double>(), R_dev);
    FG_CUDA(cudaGetLastError());
    count_launches(2);
    s->blocks_ok = true;
    s->csr_dirty = true;
    return convert_blocks(s, st);
}

// the bubble planes of a Predictor2 build with nb unknowns per element
// (1: transient transport, 4: Euler), zero-filled when (re)allocated
int bubble_alloc(fg_system *s, int nb)
{
    const size_t want = 8 * (size_t)(nb == 4 ? kBubblePlanesEuler : kBubblePlanes) * s->nel_pad;
    if (s->bubble_nb != nb || s->bubble.bytes < want) {
        int r = s->bubble.alloc(want);
        if (r) { s->bubble_nb = 0; return r; }
        s->bubble_nb = nb;
    }
    return FG_OK;
}

int tt_mfdd_assemble_device(fg_system *s, const fg_tt_coeffs *c, const double *u_dev, const double *du_dev,
                            double *F_dev, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (t.ndof != 1) { set_error("transient transport assembly needs ndof == 1"); return FG_ERR_UNSUPPORTED; }
    if (!s->geometry_ok) { set_error("transient transport assembly before fg_set_geometry"); return FG_ERR_STATE; }
    if (c->c.form != FG_TRANSPORT_DD || c->c.h_shock < FG_HSHOCK_2SQRTAREA || c->c.h_shock > FG_HSHOCK_OPTION2 ||
        (c->c.cau != FG_SHOCK_NONE && c->c.cau != FG_SHOCK_CAUDD && c->c.cau != FG_SHOCK_YZBETA)) {
        set_error("Predictor2 builds the DD form with CAUDD, YZBeta or no shock capture");
        return FG_ERR_UNSUPPORTED;
    }
    int r;
    if (s->shock_state.bytes < 16 * (size_t)s->nel_pad && (r = s->shock_state.alloc(16 * (size_t)s->nel_pad)))
        return r;
    if ((r = bubble_alloc(s, 1))) return r;
    if (s->Fe.bytes < 8 * (size_t)12 * s->nel_pad && (r = s->Fe.alloc(8 * (size_t)12 * s->nel_pad))) return r;
    double *cbtilo = s->shock_state.as<double>() + s->nel_pad;
    if (t.nel > 0)
        k_tt_mfdd_elem<<<(t.nel + 127) / 128, 128, 0, st>>>(t.nel, s->nel_pad, s->gien.as<int>(), s->gx.as<double>(),
                                                           s->gy.as<double>(), s->gtype.as<int>(),
                                                           s->node_dof.as<int>(), s->gup.as<double>(), u_dev, du_dev,
                                                           *c, cbtilo, s->bubble.as<double>(), s->A64.as<double>(),
                                                           s->Fe.as<double>());
    FG_CUDA(cudaGetLastError());
    k_tt_R<false><<<(t.n + 256) / 256, 256, 0, st>>>(t.n, s->nel_pad, s->dinc_ptr.as<int>(), s->dinc.as<int>(),
                                                    s->Fe.as<double>(), F_dev);
    FG_CUDA(cudaGetLastError());
    count_launches(2);
    s->blocks_ok = true;
    s->csr_dirty = true;
    return convert_blocks(s, st);
}

int tt_bubble_correct_device(fg_system *s, const double *Da_dev, double coef, double *DaB_dev, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (s->bubble_nb != 1) { set_error("no transient transport Predictor2 build on this system"); return FG_ERR_STATE; }
    if (t.nel > 0) {
        k_tt_bubble_correct<<<(t.nel + 255) / 256, 256, 0, st>>>(t.nel, s->nel_pad, s->gien.as<int>(),
                                                                s->gtype.as<int>(), s->node_dof.as<int>(), Da_dev,
                                                                coef, DaB_dev ? 0 : 1, s->bubble.as<double>(),
                                                                DaB_dev);
        FG_CUDA(cudaGetLastError());
        count_launches(1);
    }
    return FG_OK;
}

int tt_bubble_predict_device(fg_system *s, double coef, cudaStream_t st)
{
    const Topology &t = s->topo;
    if (t.nel > 0) {
        k_tt_bubble_predict<<<(t.nel + 255) / 256, 256, 0, st>>>(t.nel, s->nel_pad, coef, s->bubble.as<double>());
        FG_CUDA(cudaGetLastError());
        count_launches(1);
    }
    return FG_OK;
}

int transport_assemble_device(fg_system *s, const fg_transport_coeffs *c, const double *u_dev, double *F_dev,
                              cudaStream_t st)
{
    const Topology &t = s->topo;
    if (t.ndof != 1) { set_error("transport assembly needs ndof == 1"); return FG_ERR_UNSUPPORTED; }
    if (!s->geometry_ok) { set_error("transport assembly before fg_set_geometry"); return FG_ERR_STATE; }
    if (c->form != FG_TRANSPORT_SUPG && c->form != FG_TRANSPORT_DD) {
        set_error("transport form must be FG_TRANSPORT_SUPG or FG_TRANSPORT_DD");
        return FG_ERR_ARG;
    }
    if (c->cau < FG_SHOCK_NONE || c->cau > FG_SHOCK_YZBETA || (c->cau == FG_SHOCK_CAUDD && c->form != FG_TRANSPORT_DD)) {
        set_error("shock capture must be NONE, CAU or YZBETA, or CAUDD with the DD form");
        return FG_ERR_ARG;
    }
    if (c->h_shock < FG_HSHOCK_2SQRTAREA || c->h_shock > FG_HSHOCK_OPTION2) {
        set_error("h_shock must be FG_HSHOCK_2SQRTAREA, _OPTION1 or _OPTION2");
        return FG_ERR_ARG;
    }
    double *Re_old = nullptr, *delta_old = nullptr;
    if (c->cau == FG_SHOCK_YZBETA) {       // Process.c:16-17: zero state, kept across builds
        int r0;
        if (s->shock_state.bytes < 16 * (size_t)s->nel_pad && (r0 = s->shock_state.alloc(16 * (size_t)s->nel_pad)))
            return r0;
        Re_old = s->shock_state.as<double>();
        delta_old = Re_old + s->nel_pad;
    }
    if (t.nel > 0 && c->form == FG_TRANSPORT_DD)
        k_transport_dd_elem<<<(t.nel + 127) / 128, 128, 0, st>>>(t.nel, s->nel_pad, s->gien.as<int>(),
                                                                s->gx.as<double>(), s->gy.as<double>(),
                                                                s->gtype.as<int>(), s->node_dof.as<int>(),
                                                                s->gup.as<double>(), u_dev, *c, Re_old, delta_old,
                                                                s->A64.as<double>(), s->Fe.as<double>());
    else if (t.nel > 0)
        k_transport_elem<<<(t.nel + 127) / 128, 128, 0, st>>>(t.nel, s->nel_pad, s->gien.as<int>(), s->gx.as<double>(),
                                                             s->gy.as<double>(), s->gtype.as<int>(), s->node_dof.as<int>(),
                                                             s->gup.as<double>(), u_dev, *c, Re_old, delta_old, s->A64.as<double>(),
                                                             s->Fe.as<double>());
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    k_transport_F<<<(t.n + 256) / 256, 256, 0, st>>>(t.n, s->nel_pad, s->dinc_ptr.as<int>(), s->dinc.as<int>(),
                                                    s->gien.as<int>(), s->gtype.as<int>(), s->gup.as<double>(),
                                                    s->A64.as<double>(), s->Fe.as<double>(), F_dev);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    s->blocks_ok = true;
    s->csr_dirty = true;
    return convert_blocks(s, st);
}

}  // namespace fg
