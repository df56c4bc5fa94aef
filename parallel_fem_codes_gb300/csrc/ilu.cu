// Assembled CSR operator and ILU(0) (MatrixVectorProductScheme "CSR",
// Preconditioner "ILU0").
//
// * k_csr_assemble: CSR values from the element blocks, one thread per
//   slot summing its element contributions in reference element order, as
//   csr_assembly.c:3-54 adds them element by element.
// * ilu_fill (host): the level-of-fill symbolic pass of ILU(p)
//   (Solvers_and_Preconditioners/ilup.c:164-301, Preconditioner "ILU<p>"),
//   giving the factor pattern: per row the L columns ascending, the
//   diagonal, then the U columns in the order the pass admits them (the
//   row's own, then the fill) -- the order the backward substitution sums
//   them in.  For p = 0 it is the CSR pattern.
// * k_ilu0_factor: ILU(p) of CSR/ILUp_precond_setup.c:73-168 on the factor
//   pattern (IKJ elimination over the ascending L part of each row, inverse
//   pivots kept; the matrix values are scattered into the pattern first).
// * ilu_fwd / ilu_bwd: the forward and backward substitutions of
//   CSR/ILUp_precond.c:4-47.
//
// Rows of a triangular factor depend on earlier (forward) or later
// (backward) rows.  The set-up sorts the rows once by dependency level
// (level of a row = 1 + the largest level of the rows it reads; separately
// for L and for U) and cuts every level into passes of 32/G rows.  The
// kernels are "sync-free" over that order: each warp claims the next pass
// from an atomic counter, G lanes take each row of the pass, and each lane
// waits for the row its entry reads.  The rows of one pass are of one level
// and never read each other, so no lane waits for a row of its own warp,
// and every row waited for belongs to a pass claimed earlier by a running
// warp: the waits always end.  They are still bounded (g_spin_limit polls,
// set by fg_set_wait_limit); a wait that runs out records FG_ERR_TIMEOUT
// and the row goes on with 0 for the missing value, so no later wait
// hangs on it.  Level order keeps the
// critical path at the depth of the dependency graph: in plain row order a
// warp that works through a run of rows turns the chain row i -> row i-1 of
// a CSR matrix into a chain of the whole matrix.
//
// In the substitutions a value is its own ready flag: the output vector is
// filled with a NaN of a payload no arithmetic produces (kPending) before
// the sweep, a row's result is stored with one relaxed atomic store, and a
// reader polls the value itself.  Nothing else passes between rows, so no
// fence is needed, and each dependency costs one round trip through L2.
// The backward sweep therefore writes to a vector other than its input.
// The factorisation, whose rows pass whole row segments, keeps per-row
// flags with release/acquire ordering.
//
// Compiled with -fmad=false: the factorisation and the FP64 substitutions
// round exactly as the reference's C.
#include <algorithm>
#include <map>
#include <mutex>
#include <cuda/atomic>

#include "system.h"

namespace fg {

// Polls of a bounded dependency wait (fg_set_wait_limit; ~0.5 s at the
// default, each poll after the first few sleeping 32 ns).
__device__ long long g_spin_limit = 1LL << 24;

__device__ __forceinline__ bool wait_ready(const int *flag, int *err)
{
    cuda::atomic_ref<const int, cuda::thread_scope_device> a(*flag);
    for (long long it = 0; it < g_spin_limit; ++it) {
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
template <typename T> struct Pending;
template <> struct Pending<double> {
    static __device__ __forceinline__ double value() { return __longlong_as_double(0x7FF4DEAD7FF4DEADll); }
    static __device__ __forceinline__ bool is(double v) { return __double_as_longlong(v) == 0x7FF4DEAD7FF4DEADll; }
};
template <> struct Pending<float> {
    static __device__ __forceinline__ float value() { return __int_as_float(0x7FF4DEAD); }
    static __device__ __forceinline__ bool is(float v) { return __float_as_int(v) == 0x7FF4DEAD; }
};

template <typename T>
__device__ __forceinline__ T wait_value(const T *p, int *err)
{
    cuda::atomic_ref<const T, cuda::thread_scope_device> a(*p);
    for (long long it = 0; it < g_spin_limit; ++it) {
        const T v = a.load(cuda::memory_order_relaxed);
        if (!Pending<T>::is(v)) return v;
        if (it >= 4) __nanosleep(32);
    }
    atomicExch(err, FG_ERR_TIMEOUT);
    return (T)0;
}

template <typename T>
__device__ __forceinline__ void put_value(T *p, T v)
{
    cuda::atomic_ref<T, cuda::thread_scope_device> a(*p);
    a.store(v, cuda::memory_order_relaxed);
}

// A row of a substitution is handled by a group of G lanes (G = 4 ... 32,
// from the longest L or U part of the system): each lane waits for the row
// its entry reads and forms that entry's product, so the waits and loads of
// a row overlap; the products are then subtracted one by one in column
// order (every lane of the group repeats the same subtractions), which
// rounds exactly as the sequential loop of ILUp_precond.c.  The first lane
// of the group stores the row.
template <typename T, int G>
__device__ __forceinline__ void fwd_row(int i, const int *ia, const int *ja, const int *dg, const T *LU,
                                        const T *in, T *out, int *err)
{
    const int gl = threadIdx.x & (G - 1), gb = (threadIdx.x & 31) & ~(G - 1);
    const unsigned gm = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << gb;
    const int b = ia[i], d = dg[i];
    T v = in[i];
    for (int base = b; base < d; base += G) {
        const int k = base + gl;
        T p = (T)0;
        if (k < d) p = wait_value(out + ja[k], err) * LU[k];
        const int cnt = min(G, d - base);
#pragma unroll
        for (int t = 0; t < G; ++t) {
            const T pt = __shfl_sync(gm, p, gb + t);
            if (t < cnt) v = v - pt;
        }
    }
    if (gl == 0) put_value(out + i, v);
}

// x_i = (in_i - sum_{j>i} LU_ij x_j) * dinv_i, x in `out`
template <typename T, int G>
__device__ __forceinline__ void bwd_row(int i, const int *ia, const int *ja, const int *dg, const T *LU,
                                        const T *dinv, const T *in, T *out, int *err)
{
    const int gl = threadIdx.x & (G - 1), gb = (threadIdx.x & 31) & ~(G - 1);
    const unsigned gm = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << gb;
    const int b = dg[i] + 1, e = ia[i + 1];
    T v = in[i];
    for (int base = b; base < e; base += G) {
        const int k = base + gl;
        T p = (T)0;
        if (k < e) p = wait_value(out + ja[k], err) * LU[k];
        const int cnt = min(G, e - base);
#pragma unroll
        for (int t = 0; t < G; ++t) {
            const T pt = __shfl_sync(gm, p, gb + t);
            if (t < cnt) v = v - pt;
        }
    }
    if (gl == 0) put_value(out + i, v * dinv[i]);
}

__device__ __forceinline__ int claim(int *counter)
{
    int c = 0;
    if ((threadIdx.x & 31) == 0) c = atomicAdd(counter, 1);
    return __shfl_sync(0xffffffffu, c, 0);
}

// ILU(0) factorisation of one system: a warp per row, rows claimed one at
// a time in forward level order (the factorisation of a row reads the rows
// of its L part, as the forward substitution does).  The lanes wait for the rows the
// L part reads all at once, then stage the row and the U parts of those
// rows (with each entry's position in the row) in shared memory; the
// elimination then runs over the L entries in column order inside shared
// memory, updating each entry in the same order as the IKJ loop of
// ILUp_precond_setup.c:73-168, so results are bit-identical to it.  Rows
// longer than kFacRow, with more than 32 L entries or more than kFacPairs
// U entries to read take the same loop on one lane, reading global memory.
constexpr int kFacRow = 64, kFacPairs = 448, kFacWarps = 4;

struct FacSm {
    int col[kFacRow];
    double val[kFacRow];
    double dinv[32];
    int u0[32], ustart[33];
    short pos[kFacPairs];
    double uval[kFacPairs];
};

// slot of column c in a factor row (L part and diagonal ascending, ending at
// nL; the U part after it in admission order)
__device__ __forceinline__ int row_pos(const int *col, int len, int nL, int c)
{
    if (c <= col[nL]) {
        int lo = 0, hi = nL;
        while (lo <= hi) {
            int mid = (lo + hi) >> 1;
            if (col[mid] == c) return mid;
            if (col[mid] < c) lo = mid + 1; else hi = mid - 1;
        }
        return -1;
    }
    for (int t = nL + 1; t < len; ++t)
        if (col[t] == c) return t;
    return -1;
}

// One lane, global memory (long rows).
__device__ void fac_row_seq(int i, const int *__restrict__ ia, const int *__restrict__ ja, const int *__restrict__ dg,
                            const double *__restrict__ AA, double *LU, double *dinv, int *flag, int *err)
{
    const int b = ia[i], e = ia[i + 1];
    for (int k = b; k < e; ++k) LU[k] = k == dg[i] ? 0.0 : AA[k];
    double piv = AA[dg[i]];
    for (int k = b; k < dg[i]; ++k) {
        const int jrow = ja[k];
        if (!wait_ready(flag + jrow, err)) break;
        LU[k] = LU[k] * dinv[jrow];
        const double lk = LU[k];
        for (int m = dg[jrow] + 1; m < ia[jrow + 1]; ++m) {
            const int col = ja[m];
            const int rp = row_pos(ja + b, e - b, dg[i] - b, col);
            if (rp < 0) continue;
            const int pos = b + rp;
            if (col == i) piv = piv - lk * LU[m];
            else LU[pos] = LU[pos] - lk * LU[m];
        }
    }
    if (piv == 0.0) atomicExch(err, FG_ERR_BREAKDOWN);
    dinv[i] = 1.0 / piv;
}

__global__ void __launch_bounds__(32 * kFacWarps)
k_ilu0_factor(int n, const int *__restrict__ ord, const int *__restrict__ ia, const int *__restrict__ ja,
              const int *__restrict__ dg, const double *__restrict__ AA, double *LU, double *dinv, int *flag,
              int *counter, int *err)
{
    __shared__ FacSm sm_all[kFacWarps];
    FacSm &S = sm_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    for (;;) {
        const int c = claim(counter);
        if (c >= n) break;
        {
            const int i = ord[c];
            const int b = ia[i], e = ia[i + 1], d = dg[i], len = e - b, nL = d - b;
            int u0 = 0, ulen = 0;
            double dj = 0.0;
            if (nL <= 32 && lane < nL) {
                const int jrow = ja[b + lane];
                wait_ready(flag + jrow, err);
                u0 = dg[jrow] + 1;
                ulen = ia[jrow + 1] - u0;
                dj = dinv[jrow];
            }
            int scan = ulen;                       // inclusive scan of the U lengths
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, scan, o);
                if (lane >= o) scan += t;
            }
            const int total = __shfl_sync(0xffffffffu, scan, 31);
            if (len > kFacRow || nL > 32 || total > kFacPairs) {
                if (lane == 0) fac_row_seq(i, ia, ja, dg, AA, LU, dinv, flag, err);
                __syncwarp();
            } else {
                for (int t = lane; t < len; t += 32) {
                    S.col[t] = ja[b + t];
                    S.val[t] = AA[b + t];          // the diagonal slot carries the pivot
                }
                if (lane < nL) {
                    S.dinv[lane] = dj;
                    S.u0[lane] = u0;
                    S.ustart[lane] = scan - ulen;
                }
                if (lane == 0) S.ustart[nL] = total;
                __syncwarp();
#pragma unroll 2
                for (int q = 0; q < (kFacPairs + 31) / 32; ++q) {
                    const int p = lane + 32 * q;
                    if (p < total) {
                        int lo = 0, hi = nL - 1;       // entry l with ustart[l] <= p < ustart[l+1]
                        while (lo < hi) {
                            const int mid = (lo + hi + 1) >> 1;
                            if (S.ustart[mid] <= p) lo = mid; else hi = mid - 1;
                        }
                        const int m = S.u0[lo] + (p - S.ustart[lo]);
                        S.pos[p] = (short)row_pos(S.col, len, nL, ja[m]);
                        S.uval[p] = __ldcg(LU + m);   // another lane waited for this row: read from L2
                    }
                }
                __syncwarp();
                for (int l = 0; l < nL; ++l) {
                    if (lane == 0) S.val[l] = S.val[l] * S.dinv[l];
                    __syncwarp();
                    const double lk = S.val[l];
                    for (int p = S.ustart[l] + lane; p < S.ustart[l + 1]; p += 32) {
                        const int ps = S.pos[p];
                        if (ps >= 0) S.val[ps] = S.val[ps] - lk * S.uval[p];
                    }
                    __syncwarp();
                }
                for (int t = lane; t < len; t += 32) LU[b + t] = t == nL ? 0.0 : S.val[t];
                if (lane == 0) {
                    const double piv = S.val[nL];
                    if (piv == 0.0) atomicExch(err, FG_ERR_BREAKDOWN);
                    dinv[i] = 1.0 / piv;
                }
                __syncwarp();
            }
            if (lane == 0) {
                __threadfence();
                set_ready(flag + i);
            }
            __syncwarp();
        }
    }
}

// Rows of pass p (start and count in the level order `ord`) for this
// lane's group; a pass longer than 32/G rows (a batch running systems with
// fewer lanes per row) is taken in several rounds, all of one level.
template <int G, typename F>
__device__ __forceinline__ void for_pass_rows(const int *ord, int2 p, F &&row)
{
    const int g = (threadIdx.x & 31) / G;
    for (int r0 = 0; r0 < p.y; r0 += 32 / G)
        if (r0 + g < p.y) row(ord[p.x + r0 + g]);
}

// Substitutions of one system (FP64): fwd in -> out, bwd in -> out.
template <int G>
__global__ void k_ilu_fwd1(const int *ord, const int2 *passes, int npass, const int *ia, const int *ja, const int *dg,
                           const double *LU, const double *in, double *out, int *counter, int *err)
{
    for (;;) {
        const int c = claim(counter);
        if (c >= npass) break;
        for_pass_rows<G>(ord, passes[c], [&](int i) { fwd_row<double, G>(i, ia, ja, dg, LU, in, out, err); });
    }
}

template <int G>
__global__ void k_ilu_bwd1(const int *ord, const int2 *passes, int npass, const int *ia, const int *ja, const int *dg,
                           const double *LU, const double *dinv, const double *in, double *out, int *counter,
                           int *err)
{
    for (;;) {
        const int c = claim(counter);
        if (c >= npass) break;
        for_pass_rows<G>(ord, passes[c], [&](int i) { bwd_row<double, G>(i, ia, ja, dg, LU, dinv, in, out, err); });
    }
}

template <typename T>
__global__ void k_pending1(T *a, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = Pending<T>::value();
}

// Engine substitutions over a batch.  items: (system, pass) in solve order
// (the passes of every system interleaved, each system's in its level
// order).  sel 0 (FP64, cycle start, gate live): fwd t64 -> ilu_tmp, bwd
// ilu_tmp -> u64; sel 1 (T, Arnoldi, gate in cycle): fwd t -> ilu_tmp, bwd
// ilu_tmp -> w.  Outputs were filled with kPending by k_ilu_pending.
template <typename T, int G>
__global__ void k_ilu_solve(const SysDev *__restrict__ sys, const int2 *__restrict__ items, int nitems,
                            int *counter, int sel, int backward, int *err)
{
    for (;;) {
        const int c = claim(counter);
        if (c >= nitems) break;
        const int2 it = items[c];
        const SysDev &D = sys[it.x];
        if (sel == 0 ? !D.st->live : !D.st->in_cycle) continue;
        const T *LU = sizeof(T) == 8 ? (const T *)D.LU64 : (const T *)D.LU32;
        T *tmp = (T *)D.ilu_tmp;
        if (!backward) {
            const T *in = sel == 0 ? (const T *)D.t64 : (const T *)D.t;
            for_pass_rows<G>(D.ilu_ford, D.ilu_fpass[it.y], [&](int i) {
                fwd_row<T, G>(i, D.lu_ia, D.lu_ja, D.lu_dg, LU, in, tmp, err);
            });
        } else {
            T *out = sel == 0 ? (T *)D.u64 : (T *)D.w;
            const T *dinv = sizeof(T) == 8 ? (const T *)D.dinv64 : (const T *)D.dinv32;
            for_pass_rows<G>(D.ilu_bord, D.ilu_bpass[it.y], [&](int i) {
                bwd_row<T, G>(i, D.lu_ia, D.lu_ja, D.lu_dg, LU, dinv, tmp, out, err);
            });
        }
    }
}

// kPending into ilu_tmp and the backward output of every gated system.
template <typename T>
__global__ void k_ilu_pending(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch,
                              const int *__restrict__ nch, int sel)
{
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (sel == 0 ? !D.st->live : !D.st->in_cycle) continue;
        T *tmp = (T *)D.ilu_tmp, *out = sel == 0 ? (T *)D.u64 : (T *)D.w;
        for (int d = k.d0 + threadIdx.x; d < k.d1; d += blockDim.x) {
            tmp[d] = Pending<T>::value();
            out[d] = Pending<T>::value();
        }
    }
}

// b[map[k]] = a[k]: the CSR values onto the ILU(p) factor pattern
__global__ void k_scatter_map(int nnz, const int *__restrict__ map, const double *__restrict__ a, double *__restrict__ b)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz && map[k] >= 0) b[map[k]] = a[k];     // -1: a coupling between ILU blocks
}

__global__ void k_f64_to_f32(const double *a, float *b, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// ---------------------------------------------------------------- block-Jacobi substitutions
// With block-Jacobi ILU(p) every row reads only rows of its own block, and
// the dependency depth inside a block of an RCM-ordered FEM matrix is most
// of its rows (a node's coupled dofs and its RCM neighbours chain): the
// parallelism is across blocks.  So one warp (a CTA of its own) takes one
// block and walks its rows in order (forward ascending, backward
// descending); no row waits on another warp.  Everything a row reads sits
// in shared memory: the block's values (loaded with the inputs, each
// overwritten by its row's result: a row's own input is read only by that
// row), its row pointers and inverse pivots (loaded once per block), and
// the factor entries of the current chunk of kWsChunk rows, copied with
// cp.async one chunk ahead into a double buffer.  Per row the G lanes take
// its entries G at a time and form the products; lane 0 alone subtracts
// them one by one in entry order (GB300's FP64 pipe is narrow and takes a
// whole warp instruction whatever the active lanes: a chain run by every
// lane cost 20-35% more), exactly as fwd_row / bwd_row do, so the result
// is bit-identical to the level-scheduled sweep.  Measured on Euler 513^2,
// 1024 blocks, per correction: the level-scheduled sweep 443 ms (FP64) /
// 346 ms (FP32 in the mixed solver), this kernel 86 / 71 ms; a lane per
// block instead (32 blocks a warp, rows read through L1/L2) 303 / 285 ms.
constexpr int kWsChunk = kIluWsChunk;
constexpr int kWsMaxBytes = 64 * 1024;           // shared memory of one block's warp

// shared-memory layout of one warp: rows = block rows (even), ecap = entry capacity of a chunk
template <typename T> struct WsSmem {
    size_t prod, xs, ia, dg, dinv, ja, lu, total;
    __host__ __device__ WsSmem(int rows, int ecap)
    {
        prod = 0;                                    // one row's products (32)
        xs = prod + sizeof(T) * 32;
        dinv = xs + sizeof(T) * (size_t)rows;
        ia = dinv + sizeof(T) * (size_t)rows;
        dg = ia + 4 * (size_t)(rows + 2);
        lu = (dg + 4 * (size_t)rows + 15) / 16 * 16;
        ja = lu + 2 * sizeof(T) * (size_t)ecap;
        total = (ja + 2 * 4 * (size_t)ecap + 15) / 16 * 16;
    }
};

__device__ __forceinline__ void cp_async4(void *smem, const void *g)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(g)
                 : "memory");
}
__device__ __forceinline__ void cp_async8(void *smem, const void *g)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(g)
                 : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <typename T, int G>
__device__ void ws_block(int r0, int r1, const int *__restrict__ ia, const int *__restrict__ ja,
                         const int *__restrict__ dg, const T *__restrict__ LU, const T *__restrict__ dinv,
                         const T *__restrict__ in, T *__restrict__ out, bool backward, unsigned char *smem, int rows,
                         int ecap)
{
    const int lane = threadIdx.x & 31;
    const int m = r1 - r0, nch = (m + kWsChunk - 1) / kWsChunk;
    const WsSmem<T> L(rows, ecap);
    T *prod = reinterpret_cast<T *>(smem + L.prod);
    T *xs = reinterpret_cast<T *>(smem + L.xs);
    T *dv = reinterpret_cast<T *>(smem + L.dinv);
    int *ias = reinterpret_cast<int *>(smem + L.ia);
    int *dgs = reinterpret_cast<int *>(smem + L.dg);
    T *lus = reinterpret_cast<T *>(smem + L.lu);
    int *jas = reinterpret_cast<int *>(smem + L.ja);
    // the block's inputs, row pointers and pivots
    for (int t = lane; t < m; t += 32) {
        xs[t] = in[r0 + t];
        dgs[t] = dg[r0 + t];
        if (backward) dv[t] = dinv[r0 + t];
    }
    for (int t = lane; t <= m; t += 32) ias[t] = ia[r0 + t];
    __syncwarp();
    auto rows_of = [&](int c, int &lo, int &hi) {     // block-local row range [lo, hi) of chunk c
        const int t0 = c * kWsChunk, t1 = min(m, t0 + kWsChunk);
        lo = backward ? m - t1 : t0;
        hi = backward ? m - t0 : t1;
    };
    auto stage = [&](int c) {                         // the chunk's factor entries into buffer c & 1
        if (c < nch) {
            int lo, hi;
            rows_of(c, lo, hi);
            const int k0 = ias[lo], cnt = ias[hi] - k0;
            T *lb = lus + (size_t)(c & 1) * ecap;
            int *jb = jas + (size_t)(c & 1) * ecap;
            for (int q = lane; q < cnt; q += 32) {
                if (sizeof(T) == 8) cp_async8(lb + q, LU + k0 + q); else cp_async4(lb + q, LU + k0 + q);
                cp_async4(jb + q, ja + k0 + q);
            }
        }
        cp_commit();
    };
    stage(0);
    for (int c = 0; c < nch; ++c) {
        stage(c + 1);
        cp_wait<1>();                                 // chunk c's entries have landed
        __syncwarp();
        int lo, hi;
        rows_of(c, lo, hi);
        const int kb = ias[lo];
        const T *lb = lus + (size_t)(c & 1) * ecap;
        const int *jb = jas + (size_t)(c & 1) * ecap;
        for (int u = 0; u < hi - lo; ++u) {
            const int t = backward ? hi - 1 - u : lo + u;
            const int b = backward ? dgs[t] + 1 : ias[t];
            const int e = backward ? ias[t + 1] : dgs[t];
            T v = xs[t];
            for (int base = b; base < e; base += G) {
                const int k = base + lane;
                if (lane < G && k < e) {
                    const int jx = jb[k - kb] - r0;           // in the block by construction
                    prod[lane] = (unsigned)jx < (unsigned)m ? xs[jx] * lb[k - kb] : (T)0;
                }
                __syncwarp();
                if (lane == 0) {
                    const int cnt = min(G, e - base);
                    for (int q = 0; q < cnt; ++q) v = v - prod[q];
                }
                __syncwarp();
            }
            if (lane == 0) xs[t] = backward ? v * dv[t] : v;
            __syncwarp();
        }
    }
    cp_wait<0>();
    for (int t = lane; t < m; t += 32) out[r0 + t] = xs[t];
}

// rows [r0, r1) of block q of P over n rows (the split of ilu_pattern_setup)
__device__ __forceinline__ void ws_rows(int n, int P, int q, int &r0, int &r1)
{
    r0 = (int)((long long)q * n / P);
    r1 = (int)((long long)(q + 1) * n / P);
}

// one system, FP64: in -> out over its P blocks, a warp (CTA) per block
template <int G>
__global__ void __launch_bounds__(32)
k_ilu_ws1(int n, int P, const int *ia, const int *ja, const int *dg, const double *LU, const double *dinv,
          const double *in, double *out, int backward, int rows, int ecap)
{
    extern __shared__ __align__(16) unsigned char ws_smem[];
    for (int q = blockIdx.x; q < P; q += gridDim.x) {
        int r0, r1;
        ws_rows(n, P, q, r0, r1);
        ws_block<double, G>(r0, r1, ia, ja, dg, LU, dinv, in, out, backward != 0, ws_smem, rows, ecap);
        __syncwarp();
    }
}

// Engine substitutions over a batch, items (system, block), a warp (CTA)
// each: sel 0 (FP64, gate live) fwd t64 -> ilu_tmp, bwd ilu_tmp -> u64;
// sel 1 (T, gate in cycle) fwd t -> ilu_tmp, bwd ilu_tmp -> w.
template <typename T, int G>
__global__ void __launch_bounds__(32)
k_ilu_ws(const SysDev *__restrict__ sys, const int2 *__restrict__ items, int nitems, int sel, int backward, int rows,
         int ecap)
{
    extern __shared__ __align__(16) unsigned char ws_smem[];
    for (int c = blockIdx.x; c < nitems; c += gridDim.x) {
        const int2 it = items[c];
        const SysDev &D = sys[it.x];
        if (sel == 0 ? !D.st->live : !D.st->in_cycle) continue;
        const T *LU = sizeof(T) == 8 ? (const T *)D.LU64 : (const T *)D.LU32;
        const T *dinv = sizeof(T) == 8 ? (const T *)D.dinv64 : (const T *)D.dinv32;
        T *tmp = (T *)D.ilu_tmp;
        const T *in = backward ? tmp : sel == 0 ? (const T *)D.t64 : (const T *)D.t;
        T *out = !backward ? tmp : sel == 0 ? (T *)D.u64 : (T *)D.w;
        int r0, r1;
        ws_rows(D.n, D.ilu_P, it.y, r0, r1);
        ws_block<T, G>(r0, r1, D.lu_ia, D.lu_ja, D.lu_dg, LU, dinv, in, out, backward != 0, ws_smem, rows, ecap);
        __syncwarp();
    }
}

// ---------------------------------------------------------------- host side
// Substitution grid: one 256-thread CTA per SM.  The sweeps are bound by
// the latency along the dependency levels, not by the number of warps in
// flight (19 to 304 CTAs measured within 3% of each other on a 1M-row
// Euler system; 608 CTAs 7% slower from the extra polling).
static int warps_grid()
{
    return sm_count();
}

// Rows of the largest block (rounded up to even) when the warp-per-block
// substitutions apply: block-Jacobi with at least two blocks whose values,
// row pointers, pivots and two chunks of factor entries fit one warp's
// shared memory in FP64; else 0.
int ilu_ws_rows(const fg_system *s)
{
    const int n = s->topo.n;
    if (s->ilu_blocks < 2 || n < 2) return 0;
    const int P = std::min(s->ilu_blocks, n);
    const int rows = (int)((((long long)n + P - 1) / P + 1) & ~1LL);
    return WsSmem<double>(rows, kWsChunk * std::max(1, s->ilu_maxrow)).total <= (size_t)kWsMaxBytes ? rows : 0;
}

// dynamic shared memory above the default: raised per kernel when needed
template <typename K> static void ws_attr(K kern, size_t smem)
{
    static std::mutex mu;
    static std::map<const void *, size_t> set_bytes;
    if (smem <= 48 * 1024) return;
    std::lock_guard<std::mutex> lk(mu);
    size_t &b = set_bytes[reinterpret_cast<const void *>(kern)];
    if (smem > b) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        b = smem;
    }
}

// Level order of the rows for the forward (L) or backward (U) dependency
// graph and its passes of at most `rows` rows, each inside one level.
static void ilu_schedule(int n, const std::vector<int> &ia, const std::vector<int> &ja, const std::vector<int> &dg,
                         bool backward, int rows, std::vector<int> &order, std::vector<int2> &passes)
{
    std::vector<int> lev(n, 0);
    int top = 0;
    for (int t = 0; t < n; ++t) {
        const int i = backward ? n - 1 - t : t;
        const int k0 = backward ? dg[i] + 1 : ia[i], k1 = backward ? ia[i + 1] : dg[i];
        int l = 0;
        for (int k = k0; k < k1; ++k) l = std::max(l, lev[ja[k]] + 1);
        lev[i] = l;
        top = std::max(top, l);
    }
    std::vector<int> start(top + 2, 0);
    for (int i = 0; i < n; ++i) ++start[lev[i] + 1];
    for (int l = 0; l <= top; ++l) start[l + 1] += start[l];
    order.assign(n, 0);
    std::vector<int> pos(start.begin(), start.end() - 1);
    for (int i = 0; i < n; ++i) order[pos[lev[i]]++] = i;
    passes.clear();
    for (int l = 0; l <= top && n > 0; ++l)
        for (int p = start[l]; p < start[l + 1]; p += rows) passes.push_back(make_int2(p, std::min(rows, start[l + 1] - p)));
}

// One substitution of one system, in -> out (out filled with kPending here).
static int sweep1(fg_system *s, bool backward, const double *in, double *out, cudaStream_t st)
{
    const int n = s->topo.n;
    if (ilu_ws_rows(s) > 0) {                         // block-Jacobi: a warp per block
        const int P = std::min(s->ilu_blocks, n), rows = ilu_ws_rows(s), ecap = kWsChunk * s->ilu_maxrow;
        const size_t smem = WsSmem<double>(rows, ecap).total;
        const int g = std::max(1, std::min(P, 32 * sm_count()));
        const int *ia = s->lu_ia.as<int>(), *ja = s->lu_ja.as<int>(), *dg = s->lu_dg.as<int>();
        const double *LU = s->LU64.as<double>(), *dinv = s->dinv64.as<double>();
#define FG_WS1(G)                                                                                        \
    do {                                                                                                 \
        ws_attr(k_ilu_ws1<G>, smem);                                                                     \
        k_ilu_ws1<G><<<g, 32, smem, st>>>(n, P, ia, ja, dg, LU, dinv, in, out, backward, rows, ecap);    \
    } while (0)
        switch (s->ilu_g) {
        case 4: FG_WS1(4); break;
        case 8: FG_WS1(8); break;
        case 16: FG_WS1(16); break;
        default: FG_WS1(32); break;
        }
#undef FG_WS1
        FG_CUDA(cudaGetLastError());
        count_launches(1);
        return FG_OK;
    }
    int *ctr = s->ilu_ctr.as<int>(), *err = ctr + 4;
    const int *ia = s->lu_ia.as<int>(), *ja = s->lu_ja.as<int>(), *dg = s->lu_dg.as<int>();
    const double *LU = s->LU64.as<double>(), *dinv = s->dinv64.as<double>();
    const int *ord = backward ? s->ilu_bord.as<int>() : s->ilu_ford.as<int>();
    const int2 *ps = backward ? s->ilu_bpass.as<int2>() : s->ilu_fpass.as<int2>();
    const int np = backward ? s->ilu_nbpass : s->ilu_nfpass;
    k_pending1<double><<<(n + 255) / 256, 256, 0, st>>>(out, n);
    FG_CUDA(cudaMemsetAsync(ctr, 0, 4, st));
    const int g = warps_grid();
#define FG_SWEEP1(G)                                                                                      \
    (backward ? k_ilu_bwd1<G><<<g, 256, 0, st>>>(ord, ps, np, ia, ja, dg, LU, dinv, in, out, ctr, err)     \
              : k_ilu_fwd1<G><<<g, 256, 0, st>>>(ord, ps, np, ia, ja, dg, LU, in, out, ctr, err))
    switch (s->ilu_g) {
    case 4: FG_SWEEP1(4); break;
    case 8: FG_SWEEP1(8); break;
    case 16: FG_SWEEP1(16); break;
    default: FG_SWEEP1(32); break;
    }
#undef FG_SWEEP1
    FG_CUDA(cudaGetLastError());
    count_launches(2);
    return FG_OK;
}

// Symbolic ILU(p) (ilup.c:164-301): each row starts from its own entries
// at level 0; its L part is eliminated leftmost pivot first, and an entry
// of pivot row k's U part enters the row at level lev(i,k) + lev(k,c) + 1
// when that is <= p (an entry already there keeps the smaller level).
// Output rows: L ascending (the elimination order), diagonal, U in
// admission order.
static void ilu_fill(int n, const std::vector<int> &ia, const std::vector<int> &ja, int p, std::vector<int> &fia,
                     std::vector<int> &fja, std::vector<int> &fdg)
{
    std::vector<int> slot(n, -1), lc, ll, uc, ul;
    std::vector<std::vector<int>> urow(n), ulev(n), lrow(n);
    for (int i = 0; i < n; ++i) {
        lc.clear(); ll.clear(); uc.clear(); ul.clear();
        for (int q = ia[i]; q < ia[i + 1]; ++q) {
            const int c = ja[q];
            if (c < i) { slot[c] = (int)lc.size(); lc.push_back(c); ll.push_back(0); }
            else if (c > i) { slot[c] = n + (int)uc.size(); uc.push_back(c); ul.push_back(0); }
        }
        for (size_t jp = 0; jp < lc.size(); ++jp) {
            size_t jm = jp;
            for (size_t j = jp + 1; j < lc.size(); ++j)
                if (lc[j] < lc[jm]) jm = j;
            if (jm != jp) {
                std::swap(lc[jp], lc[jm]);
                std::swap(ll[jp], ll[jm]);
                slot[lc[jp]] = (int)jp;
                slot[lc[jm]] = (int)jm;
            }
            const int k = lc[jp], lk = ll[jp];
            for (size_t j = 0; j < urow[k].size(); ++j) {
                const int c = urow[k][j], it = ulev[k][j] + lk + 1;
                if (it > p) continue;
                const int sl = slot[c];
                if (sl == -1) {
                    if (c < i) { slot[c] = (int)lc.size(); lc.push_back(c); ll.push_back(it); }
                    else if (c > i) { slot[c] = n + (int)uc.size(); uc.push_back(c); ul.push_back(it); }
                } else if (sl < n) {
                    ll[sl] = std::min(ll[sl], it);
                } else {
                    ul[sl - n] = std::min(ul[sl - n], it);
                }
            }
        }
        for (int c : lc) slot[c] = -1;
        for (int c : uc) slot[c] = -1;
        lrow[i] = lc;
        urow[i] = uc;
        ulev[i] = ul;
    }
    fia.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) fia[i + 1] = fia[i] + (int)(lrow[i].size() + 1 + urow[i].size());
    fja.resize(fia[n]);
    fdg.resize(n);
    for (int i = 0; i < n; ++i) {
        int b = fia[i];
        for (int c : lrow[i]) fja[b++] = c;
        fdg[i] = b;
        fja[b++] = i;
        for (int c : urow[i]) fja[b++] = c;
    }
}

// The factor pattern of the system's fill level, the slot of every CSR
// entry in it, the substitution schedules over it and the factor storage.
int ilu_pattern_setup(fg_system *s)
{
    const int n = s->topo.n;
    std::vector<int> ia(n + 1), ja, dg(n);
    FG_CUDA(cudaMemcpy(ia.data(), s->csr_ia.p, sizeof(int) * (size_t)(n + 1), cudaMemcpyDeviceToHost));
    ja.resize(std::max(ia[n], 0));
    if (!ja.empty()) FG_CUDA(cudaMemcpy(ja.data(), s->csr_ja.p, sizeof(int) * ja.size(), cudaMemcpyDeviceToHost));
    std::vector<int> fia, fja, fdg, map(ja.size());
    // ilu_blocks > 1: block Jacobi, as the reference's ranks each factorise
    // the couplings among their own rows (CSR/ILUp_precond_setup.c:20-29,
    // A->n = neq, the rank's "own" CSR block): entries that couple two row
    // blocks are left out of the factor pattern (their slots map to -1)
    std::vector<int> bia, bja;
    const std::vector<int> *pia = &ia, *pja = &ja;
    if (s->ilu_blocks > 1 && n > 0) {
        const int P = std::min(s->ilu_blocks, n);
        std::vector<int> blk(n);
        for (int q = 0; q < P; ++q)
            for (int i = (int)((long long)q * n / P); i < (int)((long long)(q + 1) * n / P); ++i) blk[i] = q;
        bia.assign(n + 1, 0);
        for (int i = 0; i < n; ++i) {
            for (int q = ia[i]; q < ia[i + 1]; ++q)
                if (blk[ja[q]] == blk[i]) bja.push_back(ja[q]);
            bia[i + 1] = (int)bja.size();
        }
        pia = &bia;
        pja = &bja;
    }
    ilu_fill(n, *pia, *pja, s->ilu_p, fia, fja, fdg);
    {
        std::vector<int> at(n, -1);
        for (int i = 0; i < n; ++i) {
            for (int t = fia[i]; t < fia[i + 1]; ++t) at[fja[t]] = t;
            for (int q = ia[i]; q < ia[i + 1]; ++q) map[q] = at[ja[q]];
            for (int t = fia[i]; t < fia[i + 1]; ++t) at[fja[t]] = -1;
        }
    }
    auto up = [](DevMem &m, const std::vector<int> &v) -> int {
        int rr = m.alloc(sizeof(int) * std::max<size_t>(v.size(), 1));
        if (rr) return rr;
        if (!v.empty()) return h2d(m.p, v.data(), sizeof(int) * v.size());
        return FG_OK;
    };
    const size_t fnz = (size_t)std::max(fia[n], 1);
    int r;
    if ((r = up(s->lu_ia, fia)) || (r = up(s->lu_ja, fja)) || (r = up(s->lu_dg, fdg)) || (r = up(s->lu_map, map)) ||
        (r = s->AAf64.alloc(8 * fnz)) || (r = s->LU64.alloc(8 * fnz)) || (r = s->LU32.alloc(4 * fnz)))
        return r;
    s->lu_nnz = fia[n];
    // substitution schedule: lanes per row from the longest L or U part
    int longest = 1;
    for (int i = 0; i < n; ++i) longest = std::max({longest, fdg[i] - fia[i], fia[i + 1] - fdg[i] - 1});
    s->ilu_g = longest <= 4 ? 4 : longest <= 8 ? 8 : longest <= 16 ? 16 : 32;
    s->ilu_maxrow = 1;
    for (int i = 0; i < n; ++i) s->ilu_maxrow = std::max(s->ilu_maxrow, fia[i + 1] - fia[i]);
    std::vector<int> fo, bo;
    std::vector<int2> fp, bp;
    ilu_schedule(n, fia, fja, fdg, false, 32 / s->ilu_g, fo, fp);
    ilu_schedule(n, fia, fja, fdg, true, 32 / s->ilu_g, bo, bp);
    auto up2 = [](DevMem &m, const std::vector<int2> &v) -> int {
        int rr = m.alloc(sizeof(int2) * std::max<size_t>(v.size(), 1));
        if (rr) return rr;
        if (!v.empty()) return h2d(m.p, v.data(), sizeof(int2) * v.size());
        return FG_OK;
    };
    if ((r = up(s->ilu_ford, fo)) || (r = up(s->ilu_bord, bo)) || (r = up2(s->ilu_fpass, fp)) ||
        (r = up2(s->ilu_bpass, bp)))
        return r;
    s->ilu_nfpass = (int)fp.size();
    s->ilu_nbpass = (int)bp.size();
    return FG_OK;
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
        if (!v.empty()) return h2d(m.p, v.data(), sizeof(int) * v.size());
        return FG_OK;
    };
    size_t nz = (size_t)std::max(c.nnz, 1), n1 = (size_t)c.n + 1;
    if ((r = up(s->csr_ia, c.ia)) || (r = up(s->csr_ja, c.ja)) || (r = up(s->csr_diag, c.diag)) ||
        (r = up(s->csr_inc_ptr, c.inc_ptr)) || (r = up(s->csr_inc, c.inc)) || (r = s->AA64.alloc(8 * nz)) ||
        (r = s->AA32.alloc(4 * nz)) || (r = s->dinv64.alloc(8 * n1)) || (r = s->dinv32.alloc(4 * n1)) || (r = s->ilu_flags.alloc(4 * n1)) ||
        (r = s->ilu_ctr.alloc(64)) || (r = s->ilu_tmp.alloc(8 * (size_t)std::max(s->n_pad, 1))))
        return r;
    s->csr_nnz = c.nnz;
    if ((r = ilu_pattern_setup(s))) return r;
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
    const int n = s->topo.n;
    int *flag = s->ilu_flags.as<int>(), *ctr = s->ilu_ctr.as<int>(), *err = ctr + 4;
    FG_CUDA(cudaMemsetAsync(s->ilu_ctr.p, 0, s->ilu_ctr.bytes, st));
    FG_CUDA(cudaMemsetAsync(flag, 0, 4 * (size_t)(n + 1), st));
    // the matrix values on the factor pattern (fill slots start at 0)
    FG_CUDA(cudaMemsetAsync(s->AAf64.p, 0, s->AAf64.bytes, st));
    if (s->csr_nnz > 0)
        k_scatter_map<<<(s->csr_nnz + 255) / 256, 256, 0, st>>>(s->csr_nnz, s->lu_map.as<int>(), s->AA64.as<double>(),
                                                               s->AAf64.as<double>());
    if (n > 0)
        k_ilu0_factor<<<8 * sm_count(), 32 * kFacWarps, 0, st>>>(n, s->ilu_ford.as<int>(), s->lu_ia.as<int>(),
                                                                 s->lu_ja.as<int>(), s->lu_dg.as<int>(),
                                                                 s->AAf64.as<double>(), s->LU64.as<double>(),
                                                                 s->dinv64.as<double>(), flag, ctr, err);
    FG_CUDA(cudaGetLastError());
    k_f64_to_f32<<<(std::max(s->lu_nnz, 1) + 255) / 256, 256, 0, st>>>(s->LU64.as<double>(), s->LU32.as<float>(),
                                                                      s->lu_nnz);
    k_f64_to_f32<<<(n + 256) / 256, 256, 0, st>>>(s->dinv64.as<double>(), s->dinv32.as<float>(), n);
    FG_CUDA(cudaGetLastError());
    count_launches(4);
    if (F_dev && n > 0) {
        double *tmp = s->ilu_tmp.as<double>();
        int r2;
        if ((r2 = sweep1(s, false, F_dev, tmp, st)) || (r2 = sweep1(s, true, tmp, F_dev, st))) return r2;
    }
    int herr = 0;
    FG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    if (herr == FG_ERR_TIMEOUT) { set_error("ILU(p): a row dependency wait ran out"); return FG_ERR_TIMEOUT; }
    if (herr == FG_ERR_BREAKDOWN) { set_error("ILU(p): zero pivot"); return FG_ERR_BREAKDOWN; }
    s->precond = FG_PRECOND_ILU0;
    return FG_OK;
}

// z = U^-1 L^-1 p of one system (FP64, internal numbering; p may be z).
int ilu0_apply_device(fg_system *s, const double *p, double *z, cudaStream_t st)
{
    const int n = s->topo.n;
    if (s->precond != FG_PRECOND_ILU0) { set_error("ILU(0) not set up"); return FG_ERR_STATE; }
    int *ctr = s->ilu_ctr.as<int>(), *err = ctr + 4;
    double *tmp = s->ilu_tmp.as<double>();
    FG_CUDA(cudaMemsetAsync(s->ilu_ctr.p, 0, s->ilu_ctr.bytes, st));
    int r;
    if ((r = sweep1(s, false, p, tmp, st)) || (r = sweep1(s, true, tmp, z, st))) return r;   // p is read before z is filled
    FG_CUDA(cudaMemsetAsync(z + n, 0, 8, st));
    int herr = 0;
    FG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    if (herr == FG_ERR_TIMEOUT) { set_error("ILU(0): a row dependency wait ran out"); return FG_ERR_TIMEOUT; }
    return FG_OK;
}

// Warp-per-block substitution over a batch (engine): items (system, block),
// rows of the largest block, ecap entries of the longest chunk.
int launch_ilu_ws(const SysDev *sys, const int2 *items, int nitems, int sel, int backward, int fp32, int lanes,
                  int rows, int ecap, cudaStream_t st)
{
    const size_t smem = fp32 ? WsSmem<float>(rows, ecap).total : WsSmem<double>(rows, ecap).total;
    const int g = std::max(1, std::min(nitems, 32 * sm_count()));
#define FG_WS(T, G)                                                                                 \
    do {                                                                                            \
        ws_attr(k_ilu_ws<T, G>, smem);                                                              \
        k_ilu_ws<T, G><<<g, 32, smem, st>>>(sys, items, nitems, sel, backward, rows, ecap);          \
    } while (0)
    if (fp32) {
        switch (lanes) {
        case 4: FG_WS(float, 4); break;
        case 8: FG_WS(float, 8); break;
        case 16: FG_WS(float, 16); break;
        default: FG_WS(float, 32); break;
        }
    } else {
        switch (lanes) {
        case 4: FG_WS(double, 4); break;
        case 8: FG_WS(double, 8); break;
        case 16: FG_WS(double, 16); break;
        default: FG_WS(double, 32); break;
        }
    }
#undef FG_WS
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

// kPending into the outputs of the next substitutions of a batch.
int set_wait_limit(long long polls)
{
    FG_CUDA(cudaMemcpyToSymbol(g_spin_limit, &polls, sizeof(polls)));
    return FG_OK;
}

int launch_ilu_pending(const SysDev *sys, const DChunk *ch, const int *nch, int n_dch, int sel, int fp32,
                       cudaStream_t st)
{
    const int g = std::max(1, std::min(n_dch, 8 * sm_count()));
    if (fp32) k_ilu_pending<float><<<g, 256, 0, st>>>(sys, ch, nch, sel);
    else k_ilu_pending<double><<<g, 256, 0, st>>>(sys, ch, nch, sel);
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

// One sync-free substitution over a batch (engine; counter cleared here).
int launch_ilu_solve(const SysDev *sys, const int2 *items, int nitems, int *counter, int *err, int sel, int backward,
                     int fp32, int lanes, cudaStream_t st)
{
    FG_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
    const int g = warps_grid();
#define FG_SOLVE(T, G) k_ilu_solve<T, G><<<g, 256, 0, st>>>(sys, items, nitems, counter, sel, backward, err)
    if (fp32) {
        switch (lanes) {
        case 4: FG_SOLVE(float, 4); break;
        case 8: FG_SOLVE(float, 8); break;
        case 16: FG_SOLVE(float, 16); break;
        default: FG_SOLVE(float, 32); break;
        }
    } else {
        switch (lanes) {
        case 4: FG_SOLVE(double, 4); break;
        case 8: FG_SOLVE(double, 8); break;
        case 16: FG_SOLVE(double, 16); break;
        default: FG_SOLVE(double, 32); break;
        }
    }
#undef FG_SOLVE
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    return FG_OK;
}

}  // namespace fg
