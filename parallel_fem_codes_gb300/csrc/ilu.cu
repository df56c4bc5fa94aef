// Assembled CSR operator and ILU(0) (MatrixVectorProductScheme "CSR",
// Preconditioner "ILU0").
//
// * k_csr_assemble: CSR values from the element blocks, one thread per
//   slot summing its element contributions in reference element order, as
//   csr_assembly.c:3-54 adds them element by element.
// * k_ilu0_factor: ILU(0) of Solvers_and_Preconditioners/CSR/
//   ILUp_precond_setup.c:73-168 (IKJ elimination over the ascending L part
//   of each row, inverse pivots kept).
// * ilu_fwd / ilu_bwd: the forward and backward substitutions of
//   CSR/ILUp_precond.c:4-47.
//
// Rows of a triangular factor depend on earlier (forward) or later
// (backward) rows, so these kernels are "sync-free": each warp claims the
// next chunk of 32 rows from an atomic counter, in solve order, and each
// lane waits on the ready flags of the rows its own row reads.  A row only
// waits on rows claimed before it, by warps already running, so the wait
// always ends; it is still bounded (kSpinLimit polls), and a wait that runs
// out records FG_ERR_TIMEOUT instead of hanging.
//
// Compiled with -fmad=false: the factorisation and the FP64 substitutions
// round exactly as the reference's C.
#include <algorithm>
#include <cuda/atomic>

#include "system.h"

namespace fg {

constexpr long kSpinLimit = 1L << 24;

__device__ __forceinline__ bool wait_ready(const int *flag, int *err)
{
    cuda::atomic_ref<const int, cuda::thread_scope_device> a(*flag);
    for (long it = 0; it < kSpinLimit; ++it) {
        if (a.load(cuda::memory_order_acquire)) return true;
        __nanosleep(32);
    }
    atomicExch(err, FG_ERR_TIMEOUT);
    return false;
}

__device__ __forceinline__ void set_ready(int *flag)
{
    cuda::atomic_ref<int, cuda::thread_scope_device> a(*flag);
    a.store(1, cuda::memory_order_release);
}

// ---------------------------------------------------------------- assembly
__global__ void k_csr_assemble(int nnz, const int *__restrict__ inc_ptr, const int *__restrict__ inc,
                               const double *__restrict__ A64, int ld, int S, double *__restrict__ AA,
                               float *__restrict__ AA32)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnz) return;
    double s = 0.0;
    for (int q = inc_ptr[k]; q < inc_ptr[k + 1]; ++q) {
        int v = inc[q], pos = v >> 8, a = (v >> 4) & 15, b = v & 15;
        s += A64[(size_t)(a * S + b) * ld + pos];
    }
    AA[k] = s;
    AA32[k] = (float)s;
}

// ---------------------------------------------------------------- rows
template <typename T>
__device__ __forceinline__ void fwd_row(int i, const int *ia, const int *ja, const int *dg, const T *LU,
                                        const T *in, T *out, int *flag, int *err)
{
    T v = in[i];
    for (int k = ia[i]; k < dg[i]; ++k) {
        int j = ja[k];
        if (!wait_ready(flag + j, err)) break;
        v -= out[j] * LU[k];
    }
    out[i] = v;
    set_ready(flag + i);
}

template <typename T>
__device__ __forceinline__ void bwd_row(int i, const int *ia, const int *ja, const int *dg, const T *LU,
                                        const T *dinv, T *x, int *flag, int *err)
{
    T v = x[i];
    for (int k = dg[i] + 1; k < ia[i + 1]; ++k) {
        int j = ja[k];
        if (!wait_ready(flag + j, err)) break;
        v -= x[j] * LU[k];
    }
    x[i] = v * dinv[i];
    set_ready(flag + i);
}

__device__ __forceinline__ int claim(int *counter)
{
    int c = 0;
    if ((threadIdx.x & 31) == 0) c = atomicAdd(counter, 1);
    return __shfl_sync(0xffffffffu, c, 0);
}

// ILU(0) factorisation of one system.  chunks: ascending row starts.
__global__ void k_ilu0_factor(int n, const int *__restrict__ ia, const int *__restrict__ ja, const int *__restrict__ dg,
                              const double *__restrict__ AA, double *LU, double *dinv, int *flag, int *counter,
                              int nchunks, int *err)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        int c = claim(counter);
        if (c >= nchunks) break;
        int i = c * 32 + lane;
        if (i >= n) continue;
        const int b = ia[i], e = ia[i + 1];
        for (int k = b; k < e; ++k) LU[k] = k == dg[i] ? 0.0 : AA[k];
        double piv = AA[dg[i]];
        for (int k = b; k < dg[i]; ++k) {
            const int jrow = ja[k];
            if (!wait_ready(flag + jrow, err)) break;
            LU[k] *= dinv[jrow];
            const double lk = LU[k];
            for (int m = dg[jrow] + 1; m < ia[jrow + 1]; ++m) {
                const int col = ja[m];
                // column of row jrow's U part inside row i's pattern?
                int lo = b, hi = e - 1, pos = -1;
                while (lo <= hi) {
                    int mid = (lo + hi) >> 1;
                    if (ja[mid] == col) { pos = mid; break; }
                    if (ja[mid] < col) lo = mid + 1; else hi = mid - 1;
                }
                if (pos < 0) continue;
                if (col == i) piv -= lk * LU[m];
                else LU[pos] -= lk * LU[m];
            }
        }
        if (piv == 0.0) atomicExch(err, FG_ERR_BREAKDOWN);
        dinv[i] = 1.0 / piv;
        set_ready(flag + i);
    }
}

// Substitutions of one system (set-up path: F <- U^-1 L^-1 F, FP64).
__global__ void k_ilu_fwd1(int n, const int *ia, const int *ja, const int *dg, const double *LU, const double *in,
                           double *out, int *flag, int *counter, int nchunks, int *err)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        int c = claim(counter);
        if (c >= nchunks) break;
        int i = c * 32 + lane;
        if (i < n) fwd_row<double>(i, ia, ja, dg, LU, in, out, flag, err);
    }
}

__global__ void k_ilu_bwd1(int n, const int *ia, const int *ja, const int *dg, const double *LU, const double *dinv,
                           double *x, int *flag, int *counter, int nchunks, int *err)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        int c = claim(counter);
        if (c >= nchunks) break;
        int i = (nchunks - 1 - c) * 32 + lane;       // chunks from the last row down
        if (i < n) bwd_row<double>(i, ia, ja, dg, LU, dinv, x, flag, err);
    }
}

// Engine substitutions over a batch.  items: (system, first row) in solve
// order (ascending rows per system for fwd, descending for bwd); sel 0:
// FP64 t64 -> u64 (cycle start, gate live), sel 1: t -> w (Arnoldi, gate
// in cycle).  The flags of every system were cleared before the launch.
template <typename T>
__global__ void k_ilu_solve(const SysDev *__restrict__ sys, const int2 *__restrict__ items, int nitems,
                            int *counter, int sel, int backward, int *err)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        int c = claim(counter);
        if (c >= nitems) break;
        const int2 it = items[c];
        const SysDev &D = sys[it.x];
        if (sel == 0 ? !D.st->live : !D.st->in_cycle) continue;
        const int i = it.y + lane;
        if (i >= D.n) continue;
        const T *LU = sizeof(T) == 8 ? (const T *)D.LU64 : (const T *)D.LU32;
        if (!backward) {
            const T *in = sel == 0 ? (const T *)D.t64 : (const T *)D.t;
            T *out = sel == 0 ? (T *)D.u64 : (T *)D.w;
            fwd_row<T>(i, D.csr_ia, D.csr_ja, D.csr_diag, LU, in, out, D.ilu_flag, err);
        } else {
            T *x = sel == 0 ? (T *)D.u64 : (T *)D.w;
            const T *dinv = sizeof(T) == 8 ? (const T *)D.dinv64 : (const T *)D.dinv32;
            bwd_row<T>(i, D.csr_ia, D.csr_ja, D.csr_diag, LU, dinv, x, D.ilu_flag, err);
        }
    }
}

__global__ void k_f64_to_f32(const double *a, float *b, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// ---------------------------------------------------------------- host side
static int warps_grid()
{
    return 4 * sm_count();   // 256-thread CTAs: 8 warps each
}

int csr_setup(fg_system *s)
{
    if (s->csr_ok) return FG_OK;
    CsrTopology c;
    int r = build_csr(s->topo, c);
    if (r) return r;
    auto up = [](DevMem &m, const std::vector<int> &v) -> int {
        int rr = m.alloc(sizeof(int) * std::max<size_t>(v.size(), 1));
        if (rr) return rr;
        if (!v.empty()) FG_CUDA(cudaMemcpy(m.p, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice));
        return FG_OK;
    };
    size_t nz = (size_t)std::max(c.nnz, 1), n1 = (size_t)c.n + 1;
    if ((r = up(s->csr_ia, c.ia)) || (r = up(s->csr_ja, c.ja)) || (r = up(s->csr_diag, c.diag)) ||
        (r = up(s->csr_inc_ptr, c.inc_ptr)) || (r = up(s->csr_inc, c.inc)) || (r = s->AA64.alloc(8 * nz)) ||
        (r = s->AA32.alloc(4 * nz)) || (r = s->LU64.alloc(8 * nz)) || (r = s->LU32.alloc(4 * nz)) ||
        (r = s->dinv64.alloc(8 * n1)) || (r = s->dinv32.alloc(4 * n1)) || (r = s->ilu_flags.alloc(4 * n1)) ||
        (r = s->ilu_ctr.alloc(64)))
        return r;
    s->csr_nnz = c.nnz;
    double avg = c.n ? (double)c.nnz / c.n : 1.0;
    s->csr_w = avg <= 8 ? 4 : avg <= 16 ? 8 : 32;
    s->csr_ok = true;
    s->csr_dirty = true;
    return FG_OK;
}

int csr_refresh(fg_system *s, cudaStream_t st)
{
    if (!s->csr_ok || !s->csr_dirty) return FG_OK;
    if (!s->blocks_ok) { set_error("CSR values need element blocks"); return FG_ERR_STATE; }
    if (s->csr_nnz > 0)
        k_csr_assemble<<<(s->csr_nnz + 255) / 256, 256, 0, st>>>(s->csr_nnz, s->csr_inc_ptr.as<int>(),
                                                                s->csr_inc.as<int>(), s->A64.as<double>(),
                                                                s->nel_pad, s->topo.S, s->AA64.as<double>(),
                                                                s->AA32.as<float>());
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    s->csr_dirty = false;
    return FG_OK;
}

// ILU(0) set-up of one system and, when F_dev is given, F <- M^-1 F
// (ILUp_precond_setup.c:100-101).
int ilu0_setup_device(fg_system *s, double *F_dev, cudaStream_t st)
{
    int r;
    if (!s->csr_ok) { set_error("ILU(0) needs the CSR operator (fg_set_operator(FG_OP_CSR))"); return FG_ERR_STATE; }
    if ((r = csr_refresh(s, st))) return r;
    const int n = s->topo.n, nch = (n + 31) / 32;
    int *flag = s->ilu_flags.as<int>(), *ctr = s->ilu_ctr.as<int>(), *err = ctr + 4;
    FG_CUDA(cudaMemsetAsync(s->ilu_ctr.p, 0, s->ilu_ctr.bytes, st));
    FG_CUDA(cudaMemsetAsync(flag, 0, 4 * (size_t)(n + 1), st));
    if (n > 0)
        k_ilu0_factor<<<warps_grid(), 256, 0, st>>>(n, s->csr_ia.as<int>(), s->csr_ja.as<int>(), s->csr_diag.as<int>(),
                                                    s->AA64.as<double>(), s->LU64.as<double>(), s->dinv64.as<double>(),
                                                    flag, ctr, nch, err);
    FG_CUDA(cudaGetLastError());
    k_f64_to_f32<<<(std::max(s->csr_nnz, 1) + 255) / 256, 256, 0, st>>>(s->LU64.as<double>(), s->LU32.as<float>(),
                                                                       s->csr_nnz);
    k_f64_to_f32<<<(n + 256) / 256, 256, 0, st>>>(s->dinv64.as<double>(), s->dinv32.as<float>(), n);
    FG_CUDA(cudaGetLastError());
    count_launches(3);
    if (F_dev && n > 0) {
        double *tmp = s->ws.t64.as<double>();   // F_dev is ws.u64 when called from fg_precond_setup
        FG_CUDA(cudaMemsetAsync(flag, 0, 4 * (size_t)(n + 1), st));
        FG_CUDA(cudaMemsetAsync(ctr, 0, 4, st));
        k_ilu_fwd1<<<warps_grid(), 256, 0, st>>>(n, s->csr_ia.as<int>(), s->csr_ja.as<int>(), s->csr_diag.as<int>(),
                                                 s->LU64.as<double>(), F_dev, tmp, flag, ctr, nch, err);
        FG_CUDA(cudaMemsetAsync(flag, 0, 4 * (size_t)(n + 1), st));
        FG_CUDA(cudaMemsetAsync(ctr, 0, 4, st));
        k_ilu_bwd1<<<warps_grid(), 256, 0, st>>>(n, s->csr_ia.as<int>(), s->csr_ja.as<int>(), s->csr_diag.as<int>(),
                                                 s->LU64.as<double>(), s->dinv64.as<double>(), tmp, flag, ctr, nch,
                                                 err);
        FG_CUDA(cudaGetLastError());
        FG_CUDA(cudaMemcpyAsync(F_dev, tmp, 8 * (size_t)n, cudaMemcpyDeviceToDevice, st));
        FG_CUDA(cudaMemsetAsync(tmp, 0, 8 * (size_t)s->n_pad, st));
        count_launches(2);
    }
    int herr = 0;
    FG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    if (herr == FG_ERR_TIMEOUT) { set_error("ILU(0): a row dependency wait ran out"); return FG_ERR_TIMEOUT; }
    if (herr == FG_ERR_BREAKDOWN) { set_error("ILU(0): zero pivot"); return FG_ERR_BREAKDOWN; }
    s->precond = FG_PRECOND_ILU0;
    return FG_OK;
}

// z = U^-1 L^-1 p of one system (FP64, internal numbering; p may be z).
int ilu0_apply_device(fg_system *s, const double *p, double *z, cudaStream_t st)
{
    const int n = s->topo.n, nch = (n + 31) / 32;
    if (s->precond != FG_PRECOND_ILU0) { set_error("ILU(0) not set up"); return FG_ERR_STATE; }
    int *flag = s->ilu_flags.as<int>(), *ctr = s->ilu_ctr.as<int>(), *err = ctr + 4;
    double *tmp = s->ws.t64.as<double>();
    FG_CUDA(cudaMemsetAsync(s->ilu_ctr.p, 0, s->ilu_ctr.bytes, st));
    FG_CUDA(cudaMemsetAsync(flag, 0, 4 * (size_t)(n + 1), st));
    k_ilu_fwd1<<<warps_grid(), 256, 0, st>>>(n, s->csr_ia.as<int>(), s->csr_ja.as<int>(), s->csr_diag.as<int>(),
                                             s->LU64.as<double>(), p, tmp, flag, ctr, nch, err);
    FG_CUDA(cudaMemsetAsync(flag, 0, 4 * (size_t)(n + 1), st));
    FG_CUDA(cudaMemsetAsync(ctr, 0, 4, st));
    k_ilu_bwd1<<<warps_grid(), 256, 0, st>>>(n, s->csr_ia.as<int>(), s->csr_ja.as<int>(), s->csr_diag.as<int>(),
                                             s->LU64.as<double>(), s->dinv64.as<double>(), tmp, flag, ctr, nch, err);
    FG_CUDA(cudaGetLastError());
    count_launches(2);
    FG_CUDA(cudaMemcpyAsync(z, tmp, 8 * (size_t)n, cudaMemcpyDeviceToDevice, st));
    FG_CUDA(cudaMemsetAsync(z + n, 0, 8, st));
    FG_CUDA(cudaMemsetAsync(tmp, 0, 8 * (size_t)s->n_pad, st));
    int herr = 0;
    FG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    if (herr == FG_ERR_TIMEOUT) { set_error("ILU(0): a row dependency wait ran out"); return FG_ERR_TIMEOUT; }
    return FG_OK;
}

// One sync-free substitution over a batch (engine; flags cleared here).
int launch_ilu_solve(const SysDev *sys, const int2 *items, int nitems, int *flags, size_t flag_bytes, int *counter,
                     int *err, int sel, int backward, int fp32, cudaStream_t st)
{
    FG_CUDA(cudaMemsetAsync(flags, 0, flag_bytes, st));
    FG_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
    if (fp32)
        k_ilu_solve<float><<<warps_grid(), 256, 0, st>>>(sys, items, nitems, counter, sel, backward, err);
    else
        k_ilu_solve<double><<<warps_grid(), 256, 0, st>>>(sys, items, nitems, counter, sel, backward, err);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

}  // namespace fg
