// EBE matvec and the batched restarted GMRES engine (sm_103a).
//
// Method (00_CommonFiles/Solvers_and_Preconditioners/pgmres.c:5-200):
// restarted, left-preconditioned GMRES(kmax) with X0 = 0, at most kmax-1
// Arnoldi steps per cycle (pgmres.c:159), Givens rotations (:120-155),
// back-substitution (:163-171) and X += V y (:173-175).  The reference's
// modified Gram-Schmidt with one MPI_Allreduce per dot becomes classical
// Gram-Schmidt with reorthogonalisation (CGS2): three streaming passes over
// the basis per step, each ending in a deterministic device-wide reduction
// (fixed part order, "last part reduces"), instead of 2(i+1) dependent
// reductions.
//
// Work decomposition.  A batch holds any number of systems.  Element work
// is cut into patches (grouped by patch colour), dof work into parts per
// system; every
// kernel walks its chunk table with a grid-stride loop and skips systems
// that are not active.  A system's partial sums depend only on its own
// parts, so a result is bit-identical whether the system is solved alone
// or inside a batch.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <type_traits>

#include <cuda_fp16.h>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "system.h"

namespace fg {

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T> __device__ __forceinline__ T ldst(const T *p) { return __ldcs(p); }


// Gate of a kernel: 0 = system live, 1 = inside an Arnoldi cycle, < 0 = always.
__device__ __forceinline__ bool gated(const SysDev &D, int gate)
{
    if (gate < 0) return true;
    return gate == 0 ? D.st->live != 0 : D.st->in_cycle != 0;
}

// Last-part election: returns true in the CTA that completed the final part
// of system D for counter slot `slot` (all threads of the CTA agree).
__device__ __forceinline__ bool last_part(const SysDev &D, int slot)
{
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned prev = atomicAdd(&D.counter[slot], 1u);
        s_last = (prev == (unsigned)D.nparts - 1u);
        if (s_last) D.counter[slot] = 0u;
    }
    __syncthreads();
    if (s_last) __threadfence();
    return s_last != 0;
}

// Deterministic sum over parts of slots [0, nv): warp w reduces slots
// w, w+8, ...; lane l adds parts l, l+32, ... in order, then a fixed
// butterfly.  Results to out[] (shared or global).
__device__ __forceinline__ void reduce_parts(const SysDev &D, int nv, double *out)
{
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int j = warp; j < nv; j += kThreads / 32) {
        double s = 0.0;
        for (int p = lane; p < D.nparts; p += 32) s += __ldcg(&D.part[p * kPartStride + j]);
        s = warp_sum(s);
        if (lane == 0) out[j] = s;
    }
    __syncthreads();
}

// A matvec input entry in the arithmetic type: an FP16 basis vector is
// stored as sigma v, so it is scaled back (exactly: sigma is a power of two).
template <typename TA, typename TX> __device__ __forceinline__ TA in_value(TX v, const SysDev &D)
{
    if constexpr (std::is_same<TX, __half>::value) return (TA)(__half2float(v) * D.vsci);
    else return (TA)v;
}

// ---------------------------------------------------------------- EBE matvec
// y[lm] += A_e x[lm] by patches.  A patch is up to patch_elems(S)
// consecutive elements (internal order: sorted by their smallest dof, so a
// patch covers a compact band of dofs).  The CTAs loop over the patches of
// their launch (one launch per patch colour); per patch:
//  1. x of the patch's dofs is gathered into shared memory;
//  2. the element products A_e x_e are formed and staged in shared memory
//     with the elements' local indices, one thread per element (S = 3: each
//     thread loads its four elements' blocks at once, before step 1, so a
//     whole patch of loads is in flight); A and lm16 are SoA
//     [entry][element], so lane-consecutive elements read consecutive
//     addresses;
//  3. the staged rows are added into a shared-memory y local colour by local
//     colour (elements of one local colour share no dof: no atomics, a fixed
//     summation order), then each dof is written once: a plain store for
//     dofs only this patch touches, a reduction store (red.add) for dofs
//     shared with other patches (patches sharing a dof have different patch
//     colours and run in different launches, so the updates apply in launch
//     order, as read-modify-writes would).
// For 3x3 blocks each thread loads its entries of the patch's dof list
// with the element data, so the x gather costs one dependent round trip and
// the write-back none.
// The patch sizes (patch_elems) and this kernel shape were chosen by a
// measured sweep: an L2 prefetch of the next patch, one thread per block
// row with small patches, and a two-stage bulk-copy pipeline through shared
// memory were all slower.  The sink (index n) is never written.
// in_sel: 0 = x (FP64), 1 = V[step] (T), 2 = aux (TX); out_sel: 0 = t64,
// 1 = t, 2 = aux.
template <int S, typename TA, typename TX, typename TY>
__global__ void __launch_bounds__(kThreads, S == 3 ? (sizeof(TA) == 4 ? 3 : 2) : (sizeof(TA) == 4 ? 4 : 3))
k_ebe_mv(const SysDev *__restrict__ sys, const EChunk *__restrict__ ch, const int *__restrict__ nch,
         int gate, int in_sel, int out_sel, int step, const TX *aux_in, TY *aux_out, int maxdof)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr unsigned short kSink = 0xFFFF;
    constexpr int PE = patch_elems(S);
    constexpr int E = S == 3 ? PE / kThreads : 1;        // S = 3: elements per thread
    constexpr int DMAX = S == 3 ? 1536 / kThreads : 1;  // S = 3: patch dofs per thread (the patch cap)
    const MvSmem L(S, maxdof, (int)sizeof(TA));
    TA *xs = reinterpret_cast<TA *>(smem_raw + L.xs);
    TA *ys = reinterpret_cast<TA *>(smem_raw + L.ys);
    TA *ye = reinterpret_cast<TA *>(smem_raw + L.ye);
    unsigned short *ls = reinterpret_cast<unsigned short *>(smem_raw + L.ls);
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const EChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!gated(D, gate)) continue;
        const TX *X = in_sel == 0 ? (const TX *)D.x
                    : in_sel == 1 ? (const TX *)D.V + (size_t)step * D.n_pad
                    : in_sel == 3 ? (const TX *)D.r64 : aux_in;
        TY *Y = out_sel == 0 ? (TY *)D.t64 : out_sel == 1 ? (TY *)D.t : aux_out;
        const TA *A = sizeof(TA) == 8 ? (const TA *)D.A64 : (const TA *)D.A32;
        const size_t ld = (size_t)D.nel_pad;
        const int p = k.e0;
        const int pe0 = D.pt_elem[p], pne = D.pt_elem[p + 1] - pe0;
        const int pd0 = D.pt_dof[p], pnd = D.pt_dof[p + 1] - pd0;
        const unsigned short *pc = D.pt_col + (size_t)p * kPatchColStride;

        TA av[E][S == 3 ? 9 : 1];
        unsigned short li[E][S == 3 ? 3 : 1];
        int dv[DMAX];                         // S = 3: this thread's entries of the patch's dof list
        if constexpr (S == 3) {
#pragma unroll
            for (int u = 0; u < DMAX; ++u) {
                const int j = threadIdx.x + u * kThreads;
                dv[u] = j < pnd ? __ldg(D.dofs + pd0 + j) : 0;
            }
        }
        if constexpr (S == 3) {
#pragma unroll
            for (int u = 0; u < E; ++u) {
                const int q = min(threadIdx.x + u * kThreads, pne - 1);
#pragma unroll
                for (int a = 0; a < 3; ++a) li[u][a] = __ldcs(D.lm16 + a * ld + pe0 + q);
#pragma unroll
                for (int m = 0; m < 9; ++m) av[u][m] = ldst(A + m * ld + pe0 + q);
            }
        }
        __syncthreads();                      // the previous patch is done with shared memory
        if constexpr (S == 3) {
#pragma unroll
            for (int u = 0; u < DMAX; ++u) {
                const int j = threadIdx.x + u * kThreads;
                if (j < pnd) {
                    xs[j] = in_value<TA>(X[dv[u] & 0x7fffffff], D);
                    ys[j] = (TA)0;
                }
            }
        } else {
            for (int j = threadIdx.x; j < pnd; j += kThreads) {
                xs[j] = in_value<TA>(X[D.dofs[pd0 + j] & 0x7fffffff], D);
                ys[j] = (TA)0;
            }
        }
        __syncthreads();
        if constexpr (S == 3) {
#pragma unroll
            for (int u = 0; u < E; ++u) {
                const int q = threadIdx.x + u * kThreads;
                if (q >= pne) continue;
                TA xv[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) xv[a] = li[u][a] == kSink ? (TA)0 : xs[li[u][a]];
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    TA acc = av[u][3 * r] * xv[0];
                    acc += av[u][3 * r + 1] * xv[1];
                    acc += av[u][3 * r + 2] * xv[2];
                    ye[r * PE + q] = acc;
                    ls[r * PE + q] = li[u][r];
                }
            }
        } else {
            for (int q = threadIdx.x; q < pne; q += kThreads) {
                unsigned short l[S];
                TA xv[S];
#pragma unroll
                for (int a = 0; a < S; ++a) {
                    l[a] = __ldcs(D.lm16 + a * ld + pe0 + q);
                    xv[a] = l[a] == kSink ? (TA)0 : xs[l[a]];
                }
#pragma unroll
                for (int r = 0; r < S; ++r) {
                    TA acc = ldst(A + (size_t)(r * S) * ld + pe0 + q) * xv[0];
#pragma unroll
                    for (int m = 1; m < S; ++m) acc += ldst(A + (size_t)(r * S + m) * ld + pe0 + q) * xv[m];
                    ye[r * PE + q] = acc;
                    ls[r * PE + q] = l[r];
                }
            }
        }
        __syncthreads();
        for (int col = 0; col < kPatchMaxLocalColours; ++col) {
            const int cs = pc[col], ce = pc[col + 1];
            if (cs >= ce) break;
            for (int q = cs + threadIdx.x; q < ce; q += kThreads) {
#pragma unroll
                for (int r = 0; r < S; ++r) {
                    const unsigned short l = ls[r * PE + q];
                    if (l != kSink) ys[l] += ye[r * PE + q];
                }
            }
            __syncthreads();
        }
        // a dof shared with other patches takes a reduction store (no round
        // trip); the patches of one launch share no dof, so each update is
        // Y[d] + v in launch order, as a read-modify-write would be
        auto put = [&](int j, int dd) {
            const int d = dd & 0x7fffffff;
            if (d == D.n) return;                         // dof-list padding
            if (dd < 0) atomicAdd(Y + d, (TY)ys[j]);
            else Y[d] = (TY)ys[j];
        };
        if constexpr (S == 3) {
#pragma unroll
            for (int u = 0; u < DMAX; ++u) {
                const int j = threadIdx.x + u * kThreads;
                if (j < pnd) put(j, dv[u]);
            }
        } else {
            for (int j = threadIdx.x; j < pnd; j += kThreads) put(j, D.dofs[pd0 + j]);
        }
    }
}

// The FP64 S x S matvec (S = 6, 9, 12) with a thread per (element, block
// row) pair of the patch instead of a thread per element, in CTAs of 512
// threads.  A patch colour of a mesh in natural node order holds only a
// few hundred patches (7 colours of 256-element patches on a structured
// mesh), so one launch has that many CTAs: per-element threads left 20% of
// the warp slots filled, the FP64 pipe 40% busy and the loads of A waiting
// on each other (ncu: long-scoreboard stalls); per-pair threads put S
// times more independent rows in flight per CTA (12x12: 1.75 -> 2.07 TB/s
// at 385x385).  In FP32 the S-fold x gathers from shared memory cost more
// than that gains (9x9: 2.70 -> 1.97 TB/s), so FP32 keeps k_ebe_mv.  Per patch: x gathered and the patch's local
// indices staged in shared memory; each pair forms its row product exactly
// as the per-element kernel does (acc = A_r0 x_0, then acc += A_rm x_m in
// m order) and stages it; the staged rows are added into the shared y
// local colour by local colour; each dof is written once (plain store, or
// red.add for a dof shared with patches of other colours).  Same sums in
// the same order as k_ebe_mv, so the results are bit-identical.
constexpr int kMvbThreads = 512;
// rows per thread: FP64 one (every warp slot for the FP64 pipe); FP32 S /
// FG_MVB_GROUPS32 row groups per element, 0 (the default) the per-element
// k_ebe_mv: measured in FP32 (Euler 385^2 12x12 / NS 513^2 9x9, TB/s),
// per element 1.82 / 2.70, one group of 512-thread CTAs 1.87 / 1.92, three
// row groups 1.82 / 2.15.
#ifndef FG_MVB_GROUPS32
#define FG_MVB_GROUPS32 0
#endif
template <int S, typename TA> constexpr int mvb_rows()
{
    constexpr int g = FG_MVB_GROUPS32 > 0 ? FG_MVB_GROUPS32 : 1;
    return sizeof(TA) == 8 ? 1 : (FG_MVB_GROUPS32 > 0 && S > 3 && S % g == 0) ? S / g : 0;
}
template <int S, typename TA, typename TX, typename TY>
__global__ void __launch_bounds__(kMvbThreads, 2)
k_ebe_mvb(const SysDev *__restrict__ sys, const EChunk *__restrict__ ch, const int *__restrict__ nch,
          int gate, int in_sel, int out_sel, int step, const TX *aux_in, TY *aux_out, int maxdof)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr unsigned short kSink = 0xFFFF;
    constexpr int PE = patch_elems(S);
    const MvSmem L(S, maxdof, (int)sizeof(TA));
    TA *xs = reinterpret_cast<TA *>(smem_raw + L.xs);
    TA *ys = reinterpret_cast<TA *>(smem_raw + L.ys);
    TA *ye = reinterpret_cast<TA *>(smem_raw + L.ye);
    unsigned short *ls = reinterpret_cast<unsigned short *>(smem_raw + L.ls);
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const EChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!gated(D, gate)) continue;
        const TX *X = in_sel == 0 ? (const TX *)D.x
                    : in_sel == 1 ? (const TX *)D.V + (size_t)step * D.n_pad
                    : in_sel == 3 ? (const TX *)D.r64 : aux_in;
        TY *Y = out_sel == 0 ? (TY *)D.t64 : out_sel == 1 ? (TY *)D.t : aux_out;
        const TA *A = sizeof(TA) == 8 ? (const TA *)D.A64 : (const TA *)D.A32;
        const size_t ld = (size_t)D.nel_pad;
        const int p = k.e0;
        const int pe0 = D.pt_elem[p], pne = D.pt_elem[p + 1] - pe0;
        const int pd0 = D.pt_dof[p], pnd = D.pt_dof[p + 1] - pd0;
        const unsigned short *pc = D.pt_col + (size_t)p * kPatchColStride;
        __syncthreads();                      // the previous patch is done with shared memory
        for (int j = threadIdx.x; j < pnd; j += kMvbThreads) {
            xs[j] = in_value<TA>(X[D.dofs[pd0 + j] & 0x7fffffff], D);
            ys[j] = (TA)0;
        }
        for (int e = threadIdx.x; e < S * pne; e += kMvbThreads) {
            const int a = e / pne, q = e - a * pne;
            ls[a * PE + q] = __ldcs(D.lm16 + a * ld + pe0 + q);
        }
        __syncthreads();
        constexpr int R = mvb_rows<S, TA>() > 0 ? mvb_rows<S, TA>() : 1, NG = S / R;
        static_assert(S % R == 0, "rows per thread must divide the block");
        for (int e = threadIdx.x; e < NG * pne; e += kMvbThreads) {
            const int g = e / pne, q = e - g * pne;
            TA xv[S];
#pragma unroll
            for (int a = 0; a < S; ++a) {
                const unsigned short l = ls[a * PE + q];
                xv[a] = l == kSink ? (TA)0 : xs[l];
            }
#pragma unroll
            for (int rr = 0; rr < R; ++rr) {
                const int r = g * R + rr;
                const TA *Ar = A + (size_t)(r * S) * ld + pe0 + q;
                TA acc = ldst(Ar) * xv[0];
#pragma unroll
                for (int m = 1; m < S; ++m) acc += ldst(Ar + (size_t)m * ld) * xv[m];
                ye[r * PE + q] = acc;
            }
        }
        __syncthreads();
        for (int col = 0; col < kPatchMaxLocalColours; ++col) {
            const int cs = pc[col], ce = pc[col + 1];
            if (cs >= ce) break;
            for (int q = cs + threadIdx.x; q < ce; q += kMvbThreads) {
#pragma unroll
                for (int r = 0; r < S; ++r) {
                    const unsigned short l = ls[r * PE + q];
                    if (l != kSink) ys[l] += ye[r * PE + q];
                }
            }
            __syncthreads();
        }
        for (int j = threadIdx.x; j < pnd; j += kMvbThreads) {
            const int dd = D.dofs[pd0 + j];
            const int d = dd & 0x7fffffff;
            if (d == D.n) continue;                       // dof-list padding
            if (dd < 0) atomicAdd(Y + d, (TY)ys[j]);
            else Y[d] = (TY)ys[j];
        }
    }
}

// 16-byte asynchronous copy global -> shared (cp.async, L2 only) and its wait.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// The 3x3 matvec: per patch, the dof list, element blocks and local
// indices are loaded into registers (one round trip), x of the patch's dofs
// is gathered into shared memory while the patch's incidence lists arrive
// there by asynchronous copies, the element products are staged in shared
// memory, and then the thread that gathered a dof sums the products that add
// into it, in the fixed order of its incidence list, and writes it: a plain
// store for a dof only this patch touches, a reduction store (red.add) for
// one shared with other patches (those run in other launches, so the updates
// apply in launch order).  Two barriers per patch; every thread sums whole
// dofs, so no shared-memory y and no colour passes.
template <typename TA, typename TX, typename TY>
// FP32: 64 registers, 4 CTAs per SM (56 bytes of spills; measured 3.78 vs
// 3.72 TB/s at 80 registers and 3 CTAs)
__global__ void __launch_bounds__(kThreads, sizeof(TA) == 4 ? 4 : 2)
k_ebe_mv3(const SysDev *__restrict__ sys, const EChunk *__restrict__ ch, const int *__restrict__ nch,
          int gate, int in_sel, int out_sel, int step, const TX *aux_in, TY *aux_out, int maxdof)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr unsigned short kSink = 0xFFFF;
    constexpr int PE = patch_elems(3);
    constexpr int E = PE / kThreads;        // elements per thread
    constexpr int DMAX = 1536 / kThreads;   // patch dofs per thread (the patch cap)
    const MvSmem L(3, maxdof, (int)sizeof(TA));
    TA *xs = reinterpret_cast<TA *>(smem_raw + L.xs);
    TA *ye = reinterpret_cast<TA *>(smem_raw + L.ye);
    unsigned short *ic = reinterpret_cast<unsigned short *>(smem_raw + L.ic);
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const EChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!gated(D, gate)) continue;
        const TX *X = in_sel == 0 ? (const TX *)D.x
                    : in_sel == 1 ? (const TX *)D.V + (size_t)step * D.n_pad
                    : in_sel == 3 ? (const TX *)D.r64 : aux_in;
        TY *Y = out_sel == 0 ? (TY *)D.t64 : out_sel == 1 ? (TY *)D.t : aux_out;
        const TA *A = sizeof(TA) == 8 ? (const TA *)D.A64 : (const TA *)D.A32;
        const size_t ld = (size_t)D.nel_pad;
        const int p = k.e0;
        const int pe0 = D.pt_elem[p], pne = D.pt_elem[p + 1] - pe0;
        const int pd0 = D.pt_dof[p], pnd = D.pt_dof[p + 1] - pd0;
        const int i0 = D.pt_inc[p], ni = D.pt_inc[p + 1] - i0;
        const int head = (pnd + 1 + 7) & ~7;
        const int W = (pne + 15) & ~15;       // staged product row (FP32 blocks: blocked row) length
        // FP64 blocks are [entry][element]; FP32 blocks of a patch are one
        // block [entry][W] at 9 pe0
        const TA *Ap = sizeof(TA) == 8 ? A + pe0 : A + 9 * (size_t)pe0;
        const size_t lda = sizeof(TA) == 8 ? ld : (size_t)W;
        int dv[DMAX];
#pragma unroll
        for (int u = 0; u < DMAX; ++u) {
            const int j = threadIdx.x + u * kThreads;
            dv[u] = j < pnd ? __ldg(D.dofs + pd0 + j) : 0;
        }
        TA av[E][9];
        unsigned short li[E][3];
#pragma unroll
        for (int u = 0; u < E; ++u) {
            const int q = min(threadIdx.x + u * kThreads, pne - 1);
#pragma unroll
            for (int a = 0; a < 3; ++a) li[u][a] = __ldcs(D.lm16 + a * ld + pe0 + q);
#pragma unroll
            for (int m = 0; m < 9; ++m) av[u][m] = ldst(Ap + m * lda + q);
        }
        __syncthreads();                      // the previous patch is done with shared memory
        for (int t = threadIdx.x; t < ni / 8; t += kThreads) cp_async16(ic + 8 * t, D.incl + i0 + 8 * t);
#pragma unroll
        for (int u = 0; u < DMAX; ++u) {
            const int j = threadIdx.x + u * kThreads;
            if (j < pnd) xs[j] = in_value<TA>(X[dv[u] & 0x7fffffff], D);
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < E; ++u) {
            const int q = threadIdx.x + u * kThreads;
            if (q >= pne) continue;
            TA xv[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) xv[a] = li[u][a] == kSink ? (TA)0 : xs[li[u][a]];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                TA acc = av[u][3 * r] * xv[0];
                acc += av[u][3 * r + 1] * xv[1];
                acc += av[u][3 * r + 2] * xv[2];
                ye[r * W + q] = acc;
            }
        }
        cp_async_wait_all();
        __syncthreads();
#pragma unroll
        for (int u = 0; u < DMAX; ++u) {
            const int j = threadIdx.x + u * kThreads;
            const int dd = dv[u];
            const int d = dd & 0x7fffffff;
            if (j >= pnd || d == D.n) continue;           // dof-list padding
            const int e0 = ic[j], e1 = ic[j + 1];
            TA v = (TA)0;
            for (int e = e0; e < e1; ++e) v += ye[ic[head + e]];
            if (dd < 0) atomicAdd(Y + d, (TY)v);          // shared dof: reduction store
            else Y[d] = (TY)v;
        }
    }
}

// ---------------------------------------------------------------- 3x3 matvec, bulk-copy pipeline
// The FP32-block 3x3 matvec of the batched engine as a warp-specialised
// pipeline, one CTA of 1024 threads per SM.  Warp 0 is the producer: for
// each patch of its CTA it waits until a stage of the three-stage
// shared-memory ring is free, then one lane copies into it, with 1-D bulk
// copies (cp.async.bulk, completion counted on the stage's "full"
// mbarrier), everything the patch needs: its nine block rows, the three
// rows of x-segment positions of its elements' vertices, its dof list and
// incidence lists, and x itself -- the dofs of a patch lie in one short
// segment of x (one contiguous band in the RCM numbering), so x arrives
// as one copy instead of a dof-by-dof gather.  Warps 1..31 consume the
// patches in order, with no global loads:
//   products   each thread forms its elements' three row products from the
//              staged blocks and x, and writes them over the first three
//              block rows of its own elements (slots it alone reads);
//   sums       the thread that owns a dof adds the products listed for it,
//              in the fixed order of its incidence list, and writes it once
//              (plain store, or red.add for a dof shared with patches of
//              other colours, which run in other launches);
// so each dof gets the same sum, in the same order, as in k_ebe_mv3.  The
// consumers then release the stage on its "empty" mbarrier.
// Every mbarrier wait is bounded (kMbarWaitCycles, ~2 s).  A consumer wait
// that runs out marks the patch's system FG_ERR_TIMEOUT, stops the
// producer, waits (bounded) for the copies in flight and ends the CTA; the
// producer gives up on a free stage the same way.
constexpr int kMv3pThreads = 1024;
constexpr int kMv3pStages = 3;
constexpr int kMv3pConsumers = kMv3pThreads - 32 * kMv3pStages;
constexpr int kMv3pDofCap = 1536;                       // dofs per patch (the patch cap)
constexpr int kMv3pIncCap = ((kMv3pDofCap + 1 + 7) / 8) * 8 + 3 * patch_elems(3);
constexpr long long kMbarWaitCycles = 4000000000LL;     // ~2 s at 2 GHz
// per-stage facts the producer leaves for the consumers (pne < 0: no patch)
struct Mv3pMeta {
    int pne, pnd, n, sys;
    void *Y;
    float vsci;
    int W;             // block row / staged product row length (pne rounded up to 16)
};
template <typename TX>
struct Mv3pSmem {
    static constexpr int PE = patch_elems(3);
    static constexpr size_t a = 0;                                   // [9][W] float, W <= PE
    static constexpr size_t b = a + 9 * (size_t)PE * 4;              // index blob: [3][W] ushort, dofs, incidence
    static constexpr size_t x = b + 6 * (size_t)PE + 4 * (size_t)kMv3pDofCap + 2 * (size_t)kMv3pIncCap;
    static constexpr size_t meta = (x + (size_t)kPatchXCap * sizeof(TX) + 15) / 16 * 16;
    static constexpr size_t stage = (meta + sizeof(Mv3pMeta) + 127) / 128 * 128;
    static constexpr size_t full = kMv3pStages * stage;             // kMv3pStages mbarriers
    static constexpr size_t empty = full + 8 * kMv3pStages;          // kMv3pStages mbarriers
    static constexpr size_t abort = empty + 8 * kMv3pStages;         // consumers gave up
    static constexpr size_t total = abort + 16;
    static_assert(total <= 227 * 1024, "3x3 pipeline exceeds shared memory");
    static_assert(x % 16 == 0, "x segment must stay 16-byte aligned");
};
static_assert(patch_elems(3) % 16 == 0, "patch rows must stay 16-byte aligned");

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(unsigned dst, const void *src, unsigned bytes, unsigned bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}
// true when the phase with this parity has completed; false after ~2 s
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity)
{
    const long long t0 = clock64();
    for (;;) {
        unsigned ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n" : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
        if (clock64() - t0 > kMbarWaitCycles) return false;
    }
}
// barrier 1 over the consumer warps only; returns true in every consumer
// thread when any of them passed true
__device__ __forceinline__ bool consumers_sync_or(bool v)
{
    unsigned r;
    asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 1, %2, p;\n"
                 " selp.u32 %0, 1, 0, q;\n}\n" : "=r"(r) : "r"((unsigned)v), "n"(kMv3pConsumers) : "memory");
    return r != 0;
}
__device__ __forceinline__ void consumers_sync()
{
    asm volatile("bar.sync 1, %0;\n" ::"n"(kMv3pConsumers) : "memory");
}
// a staged x entry in FP32 (an FP16 basis vector is stored as sigma v)
template <typename TX> __device__ __forceinline__ float staged_x(TX v, float vsci)
{
    if constexpr (std::is_same<TX, __half>::value) return __half2float(v) * vsci;
    else return (float)v;
}

template <typename TX, typename TY>
__global__ void __launch_bounds__(kMv3pThreads, 1)
k_ebe_mv3p(const SysDev *__restrict__ sys, const MvRec *__restrict__ rec, const int *__restrict__ nch,
           int gate, int in_sel, int out_sel, int step, const TX *aux_in, TY *aux_out)
{
    extern __shared__ __align__(128) unsigned char mv3p_smem[];
    using L = Mv3pSmem<TX>;
    using TA = float;
    constexpr int NC = kMv3pConsumers, ST = kMv3pStages;
    constexpr unsigned short kSink = 0xFFFF;
    volatile int *s_abort = reinterpret_cast<volatile int *>(mv3p_smem + L::abort);
    const unsigned full0 = smem_u32(mv3p_smem + L::full), empty0 = smem_u32(mv3p_smem + L::empty);
    const int total = *nch;
    const int tid = threadIdx.x;

    if (tid == 0) {
        for (int s = 0; s < ST; ++s) {
            mbar_init(full0 + 8u * s, 1);
            mbar_init(empty0 + 8u * s, 1);
            reinterpret_cast<Mv3pMeta *>(mv3p_smem + s * L::stage + L::meta)->sys = 0;
        }
        *s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();

    // ------------------------------------------------ producers (warps 0..ST-1)
    // Producer warp w fills stage w with the CTA's patches k = w, w + ST,
    // ...: it waits until the consumers released the stage, then lane 0
    // arms the stage's full barrier and issues the patch's three bulk
    // copies (blocks, index blob, x segment).  The next patch's record and
    // system fields are loaded before the wait, so they overlap it.  A
    // patch whose system is gated off is passed as an empty stage; past the
    // CTA's last patch the producer leaves an end marker and stops.
    if (tid < 32 * ST) {
        if (tid & 31) return;
        const int w = tid >> 5, s = w;
        unsigned char *stg = mv3p_smem + s * L::stage;
        Mv3pMeta *meta = reinterpret_cast<Mv3pMeta *>(stg + L::meta);
        const unsigned full = full0 + 8u * s;
        for (int k = w;; k += ST) {
            const long long c = blockIdx.x + (long long)k * gridDim.x;
            const bool have = c < total;
            MvRec r = have ? rec[c] : MvRec{};
            const SysDev &D = sys[r.sys];
            const bool live = have && gated(D, gate);
            const int pne = r.pn & 0xFFFF, pnd = r.pn >> 16, xlen = r.nx >> 16;
            const int W = (pne + 15) & ~15;
            const TX *X = in_sel == 0 ? (const TX *)D.x
                        : in_sel == 1 ? (const TX *)D.V + (size_t)step * D.n_pad
                    : in_sel == 3 ? (const TX *)D.r64 : aux_in;
            void *Y = out_sel == 0 ? (void *)D.t64 : out_sel == 1 ? (void *)D.t : (void *)aux_out;
            const int n = D.n;
            const float vsci = D.vsci;
            const TA *A = D.A32 + 9 * (size_t)r.pe0;
            const unsigned char *blob = D.blob + 16 * (size_t)r.boff16;
            if (k >= ST && !mbar_wait(empty0 + 8u * s, (unsigned)((k / ST - 1) & 1))) return;
            if (*s_abort) return;
            if (!have) {                                   // end of this CTA's patches
                meta->pne = -1;
                mbar_arrive(full);
                return;
            }
            meta->sys = r.sys;
            if (!live) {                                   // gated off: nothing to do
                meta->pne = 0;
                meta->pnd = 0;
                mbar_arrive(full);
                continue;
            }
            const unsigned ra = 9u * (unsigned)W * 4u, rb = (unsigned)r.bsize;
            const unsigned rx = (unsigned)xlen * (unsigned)sizeof(TX);
            meta->pne = pne;
            meta->pnd = pnd;
            meta->n = n;
            meta->Y = Y;
            meta->vsci = vsci;
            meta->W = W;
            mbar_expect_tx(full, ra + rb + rx);
            bulk_g2s(smem_u32(stg + L::a), A, ra, full);
            bulk_g2s(smem_u32(stg + L::b), blob, rb, full);
            bulk_g2s(smem_u32(stg + L::x), X + r.xlo, rx, full);
        }
    }

    // ------------------------------------------------ consumers (warps ST..31)
    const int ct = tid - 32 * ST;
    for (int j = 0;; ++j) {
        const int s = j % ST;
        unsigned char *stg = mv3p_smem + s * L::stage;
        const Mv3pMeta *meta = reinterpret_cast<const Mv3pMeta *>(stg + L::meta);
        const bool ok = mbar_wait(full0 + 8u * s, (unsigned)((j / ST) & 1));
        const int pne = ok ? meta->pne : 0;
        const int W = meta->W;
        TA *sa = reinterpret_cast<TA *>(stg + L::a);
        const unsigned short *sl = reinterpret_cast<const unsigned short *>(stg + L::b);
        const TX *sx = reinterpret_cast<const TX *>(stg + L::x);
        const float vsci = meta->vsci;
        // products over the block rows 0..2 of the element's own slots
        for (int q = ct; q < pne; q += NC) {
            TA av[9], xv[3];
#pragma unroll
            for (int m = 0; m < 9; ++m) av[m] = sa[m * W + q];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const unsigned short li = sl[a * W + q];
                xv[a] = li == kSink ? (TA)0 : staged_x(sx[li], vsci);
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                TA acc = av[3 * r] * xv[0];
                acc += av[3 * r + 1] * xv[1];
                acc += av[3 * r + 2] * xv[2];
                sa[r * W + q] = acc;
            }
        }
        if (consumers_sync_or(!ok)) {
            // give up: record the timeout, stop the producer, wait (bounded)
            // for the copies that may be in flight into the stages
            if (ct == 0) {
                *s_abort = 1;
                SysState *st = sys[meta->sys].st;         // 0 until the stage was first filled
                st->status = FG_ERR_TIMEOUT;
                st->live = 0;
                for (int q = j; q < j + ST; ++q) mbar_wait(full0 + 8u * (q % ST), (unsigned)((q / ST) & 1));
            }
            return;
        }
        if (pne < 0) break;                               // no more patches
        const int pnd = meta->pnd, n = meta->n;
        TY *Y = reinterpret_cast<TY *>(meta->Y);
        const int head = (pnd + 1 + 7) & ~7;
        const int *dl = reinterpret_cast<const int *>(stg + L::b + 6 * (size_t)W);
        const unsigned short *ic = reinterpret_cast<const unsigned short *>(stg + L::b + 6 * (size_t)W + 4 * (size_t)pnd);
        for (int jj = ct; jj < pnd; jj += NC) {
            const int dd = dl[jj];
            const int d = dd & 0x7fffffff;
            if (d == n) continue;                         // dof-list padding
            const int e0 = ic[jj], e1 = ic[jj + 1];
            TA v = (TA)0;
            for (int e = e0; e < e1; ++e) v += sa[ic[head + e]];
            if (dd < 0) atomicAdd(Y + d, (TY)v);          // shared dof: reduction store
            else Y[d] = (TY)v;
        }
        // this thread's shared-memory writes (the products) before the next
        // bulk copy into the stage
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        consumers_sync();                                 // stage s is free
        if (ct == 0) mbar_arrive(empty0 + 8u * s);
    }
}

// ---------------------------------------------------------------- CSR SpMV
// y = A x for the assembled operator (csrmv.c:57-62), W lanes per row
// (W = 4, 8 or 32 from the mean row length; rows of P1 transport hold ~7
// entries, rows of the 4-dof Euler system ~30): lanes stride the row,
// shuffle-reduce, one lane stores.  Works on dof parts like the Krylov
// kernels; same in/out selection as k_ebe_mv.
template <int W, typename TA, typename TX, typename TY>
__global__ void __launch_bounds__(kThreads)
k_csr_mv(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch, const int *__restrict__ nch,
         int gate, int in_sel, int out_sel, int step, const TX *aux_in, TY *aux_out)
{
    const int total = *nch;
    const int sub = threadIdx.x % W, grp = threadIdx.x / W, ngrp = blockDim.x / W;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!gated(D, gate)) continue;
        const TX *X = in_sel == 0 ? (const TX *)D.x
                    : in_sel == 1 ? (const TX *)D.V + (size_t)step * D.n_pad
                    : in_sel == 3 ? (const TX *)D.r64 : aux_in;
        TY *Y = out_sel == 0 ? (TY *)D.t64 : out_sel == 1 ? (TY *)D.t : aux_out;
        const TA *AA = sizeof(TA) == 8 ? (const TA *)D.AA64 : (const TA *)D.AA32;
        for (int base = k.d0; base < k.d1; base += ngrp) {
            const int row = base + grp;
            TA s = 0;
            if (row < k.d1)
                for (int q = D.csr_ia[row] + sub; q < D.csr_ia[row + 1]; q += W)
                    s += ldst(AA + q) * in_value<TA>(X[__ldcs(D.csr_ja + q)], D);
#pragma unroll
            for (int o = W / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, W);
            if (row < k.d1 && sub == 0) Y[row] = (TY)s;
        }
    }
}

// ---------------------------------------------------------------- block-diagonal apply
// z[dofs of node] = invB(node) * p[dofs of node] (BlockDiag_precond.c:3-29,
// BlockDiagDOF3_precond.c:3-27); dofs that are Dirichlet read 0 and are not
// written.  sel: 0 = t64 -> u64 (FP64), 1 = t -> w (T), 2 = aux.
template <int B, typename T>
__global__ void __launch_bounds__(kThreads)
k_blockdiag(const SysDev *__restrict__ sys, const NChunk *__restrict__ ch, const int *__restrict__ nch,
            int gate, int sel, const T *aux_in, T *aux_out)
{
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const NChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!gated(D, gate)) continue;
        const T *P = sel == 0 ? (const T *)D.t64 : sel == 1 ? (const T *)D.t : aux_in;
        T *Z = sel == 0 ? (T *)D.u64 : sel == 1 ? (T *)D.w : aux_out;
        const T *M = sizeof(T) == 8 ? (const T *)D.ibd64 : (const T *)D.ibd32;
        for (int nd = k.n0 + threadIdx.x; nd < k.n1; nd += blockDim.x) {
            int id[B];
            T v[B];
#pragma unroll
            for (int a = 0; a < B; ++a) {
                id[a] = D.node_dof[nd * B + a];
                v[a] = id[a] == D.n ? (T)0 : P[id[a]];
            }
            const T *m = M + (size_t)nd * B * B;
#pragma unroll
            for (int r = 0; r < B; ++r) {
                T s = m[r * B] * v[0];
#pragma unroll
                for (int q = 1; q < B; ++q) s += m[r * B + q] * v[q];
                if (id[r] != D.n) Z[id[r]] = s;
            }
        }
    }
}

// ---------------------------------------------------------------- cycle start
// FP64: u = M^-1 (A x) (t64 holds A x; for the block-diagonal case u64
// already holds M^-1 t64), r = b - u (pgmres.c:64-75), partial ||r||^2,
// true residual s = F - A x, partial ||s||^2, and on the first cycle ||b||^2
// and ||F||^2.  t64 is cleared for the next use.
__global__ void __launch_bounds__(kThreads)
k_start(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch, const int *__restrict__ nch)
{
    __shared__ double red[4][kThreads / 32];
    __shared__ double tot[4];
    const int total = *nch;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!D.st->live) continue;
        const bool first = D.st->first != 0;
        const bool has_f = D.ftrue != nullptr;
        double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        for (int d = k.d0 + threadIdx.x; d < k.d1; d += blockDim.x) {
            double t = D.t64[d];
            double u = D.precond == FG_PRECOND_DIAG ? t * D.invd64[d]
                     : precond_separate(D.precond) ? D.u64[d] : t;
            double bd = D.b[d];
            double r = -1.0 * (u + -1.0 * bd);
            D.r64[d] = r;
            D.t64[d] = 0.0;
            a0 += r * r;
            if (has_f) {
                double s = D.ftrue[d] - t;
                a1 += s * s;
                if (first) a3 += D.ftrue[d] * D.ftrue[d];
            }
            if (first) a2 += bd * bd;
        }
        a0 = warp_sum(a0); a1 = warp_sum(a1); a2 = warp_sum(a2); a3 = warp_sum(a3);
        if (lane == 0) { red[0][warp] = a0; red[1][warp] = a1; red[2][warp] = a2; red[3][warp] = a3; }
        __syncthreads();
        if (threadIdx.x < 4) {
            double s = 0;
            for (int w = 0; w < kThreads / 32; ++w) s += red[threadIdx.x][w];
            D.part[k.part * kPartStride + threadIdx.x] = s;
        }
        if (last_part(D, 0)) {
            reduce_parts(D, 4, tot);
            if (threadIdx.x == 0) {
                SysState *st = D.st;
                double r0 = sqrt(tot[0]);
                if (st->first) {
                    st->normb = sqrt(tot[2]);
                    st->fnorm = sqrt(tot[3]);
                    st->eps = D.mixed ? D.tol : D.tol * st->normb;
                    st->first = 0;
                }
                double rel_true = has_f ? (st->fnorm > 0 ? sqrt(tot[1]) / st->fnorm : sqrt(tot[1])) : NAN;
                double rel_pre = st->normb > 0 ? r0 / st->normb : r0;
                st->true_res = rel_true;
                st->r0 = r0;
                st->steps = 0;
                bool stop = false;
                if (!(r0 > 0.0)) {                      // exact (or empty) right-hand side
                    stop = true;
                    st->converged = (r0 == 0.0);
                    if (!(r0 == 0.0)) st->status = FG_ERR_BREAKDOWN;
                    st->rho = r0;
                } else if (D.mixed) {
                    double m = has_f ? rel_true : rel_pre;
                    if (m <= D.tol) { stop = true; st->converged = 1; }
                    else if (st->cycles >= D.lmax) { stop = true; st->status = FG_ERR_NOTCONV; }
                    st->target = D.inner_tol * r0;
                }
                if (stop) { st->live = 0; st->in_cycle = 0; }
                else {
                    st->in_cycle = 1;
                    D.g[0] = r0;                        // e[0] = ||r||
                    st->rho = r0;
                }
            }
        }
    }
}

// v0 = r * (1 / ||r||) (pgmres.c:78-81)
template <typename TV>
__device__ __forceinline__ TV to_basis(double v)
{
    if constexpr (std::is_same<TV, __half>::value) return __float2half_rn((float)v);
    else return (TV)v;
}

// v_0 = r / ||r||, stored as sigma v_0 (sigma = 1 unless the basis is FP16)
template <typename T, typename TV = T>
__global__ void __launch_bounds__(kThreads)
k_scale_v0(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch, const int *__restrict__ nch)
{
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!D.st->in_cycle) continue;
        const double sc = 1.0 / D.st->r0;
        TV *V0 = (TV *)D.V;
        for (int d = k.d0 + threadIdx.x; d < k.d1; d += blockDim.x) {
            const T v = (T)(sc * D.r64[d]);
            V0[d] = to_basis<TV>((double)D.vsc * (double)v);
        }
    }
}

#include "arnoldi.cuh"

// final true residual: t64 holds A x
__global__ void __launch_bounds__(kThreads)
k_final(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch, const int *__restrict__ nch)
{
    __shared__ double red[kThreads / 32];
    __shared__ double tot[1];
    const int total = *nch;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        double a = 0;
        for (int d = k.d0 + threadIdx.x; d < k.d1; d += blockDim.x) {
            double t = D.t64[d];
            D.t64[d] = 0.0;
            if (D.ftrue) { double s = D.ftrue[d] - t; a += s * s; }
        }
        a = warp_sum(a);
        if (lane == 0) red[warp] = a;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0;
            for (int w8 = 0; w8 < kThreads / 32; ++w8) s += red[w8];
            D.part[k.part * kPartStride] = s;
        }
        if (last_part(D, 5)) {
            reduce_parts(D, 1, tot);
            if (threadIdx.x == 0) {
                SysState *st = D.st;
                st->true_res = D.ftrue ? (st->fnorm > 0 ? sqrt(tot[0]) / st->fnorm : sqrt(tot[0])) : NAN;
            }
        }
    }
}

__global__ void k_init_state(const SysDev *__restrict__ sys, int nsys)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    SysState *st = sys[s].st;
    memset(st, 0, sizeof(SysState));
    st->live = 1;
    st->first = 1;
    st->status = FG_OK;
    for (int c = 0; c < 8; ++c) sys[s].counter[c] = 0u;
}

// live flags of all systems into one array (one small copy per cycle)
__global__ void k_live(const SysDev *__restrict__ sys, int nsys, int *out)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nsys) out[s] = sys[s].st->live;
}

// ---------------------------------------------------------------- host side
int sm_count()
{
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

namespace {

// FP32 3x3 blocks: the bulk-copy pipeline (k_ebe_mv3p) instead of k_ebe_mv3
#ifndef FG_MV3_PIPELINE
#define FG_MV3_PIPELINE 1
#endif
constexpr bool kMv3Pipeline = FG_MV3_PIPELINE != 0;
// the matvec kernel of an S x S launch: 3x3, the pair kernel, or per element
template <int S, typename TA, typename TX, typename TY, bool PAIRS>
static auto pick_mv()
{
    if constexpr (S == 3) return k_ebe_mv3<TA, TX, TY>;
    else if constexpr (PAIRS && mvb_rows<S, TA>() > 0) return k_ebe_mvb<S, TA, TX, TY>;
    else return k_ebe_mv<S, TA, TX, TY>;
}

struct MvLaunch {
    // Persistent CTAs: as many as fit on the GPU (their dynamic shared memory,
    // mv_smem_bytes, decides how many per SM), at most one per patch.
    template <typename TA, typename TX, typename TY>
    static void go(int S, int nitems, cudaStream_t st, const SysDev *sys, const EChunk *ch, const int *nch,
                   int gate, int in_sel, int out_sel, int step, const TX *ai, TY *ao, int maxdof)
    {
        switch (S) {
        case 3: run<3, TA, TX, TY>(nitems, st, sys, ch, nch, gate, in_sel, out_sel, step, ai, ao, maxdof); break;
        case 6: run<6, TA, TX, TY>(nitems, st, sys, ch, nch, gate, in_sel, out_sel, step, ai, ao, maxdof); break;
        case 9: run<9, TA, TX, TY>(nitems, st, sys, ch, nch, gate, in_sel, out_sel, step, ai, ao, maxdof); break;
        case 12: run<12, TA, TX, TY>(nitems, st, sys, ch, nch, gate, in_sel, out_sel, step, ai, ao, maxdof); break;
        }
    }
    template <int S, typename TA, typename TX, typename TY>
    static void run(int nitems, cudaStream_t st, const SysDev *sys, const EChunk *ch, const int *nch, int gate,
                    int in_sel, int out_sel, int step, const TX *ai, TY *ao, int maxdof)
    {
        const size_t smem = mv_smem_bytes(S, maxdof, sizeof(TA));
        // FP64 S x S blocks: a thread per (element, row) (the FP64 pipe wants
        // every warp slot); FP32: a thread per element (its x values
        // gathered once, not once per row)
        // the pair kernel only for colour launches of up to two waves of the
        // per-element kernel (3 CTAs per SM): FP64 12x12 Euler 513^2 (7
        // launches of ~290-512 patches) 2.02 -> 2.46 TB/s, but NS 1025^2
        // (~1170 a launch) 3.23 -> 2.83 TB/s; both give the same sums
        constexpr bool can_pair = S > 3 && mvb_rows<S, TA>() > 0;
        const bool pairs = can_pair && nitems <= 6 * sm_count();
        auto kern = pairs ? pick_mv<S, TA, TX, TY, true>() : pick_mv<S, TA, TX, TY, false>();
        const int nt = pairs ? kMvbThreads : kThreads;
        // the attribute and the occupancy are cached per kernel (last
        // shared-memory size seen); they are host-side queries only
        static std::mutex mu;
        static size_t set_bytes[2] = {0, 0}, occ_bytes[2] = {0, 0};
        static int occ_cached[2] = {1, 1};
        const int w = pairs ? 1 : 0;
        int occ;
        {
            std::lock_guard<std::mutex> lk(mu);
            if (smem > set_bytes[w]) {
                cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                set_bytes[w] = smem;
            }
            if (smem != occ_bytes[w]) {
                int o = 0;
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, nt, smem);
                occ_cached[w] = std::max(o, 1);
                occ_bytes[w] = smem;
            }
            occ = occ_cached[w];
        }
        const int g = std::max(1, std::min(nitems, occ * sm_count()));
        kern<<<g, nt, smem, st>>>(sys, ch, nch, gate, in_sel, out_sel, step, ai, ao, maxdof);
    }
    // the 3x3 FP32 bulk-copy pipeline: one CTA per SM, at most one per patch
    template <typename TX, typename TY>
    static void pipeline(int nitems, cudaStream_t st, const SysDev *sys, const MvRec *rec, const int *nch, int gate,
                         int in_sel, int out_sel, int step, const TX *ai, TY *ao)
    {
        using L = Mv3pSmem<TX>;
        static std::once_flag once;
        std::call_once(once, [] {
            cudaFuncSetAttribute(k_ebe_mv3p<TX, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::total);
        });
        const int g = std::max(1, std::min(nitems, sm_count()));
        k_ebe_mv3p<TX, TY><<<g, kMv3pThreads, L::total, st>>>(sys, rec, nch, gate, in_sel, out_sel, step, ai, ao);
    }
};

template <typename T>
void launch_blockdiag(int B, dim3 g, cudaStream_t st, const SysDev *sys, const NChunk *ch, const int *nch,
                      int gate, int sel, const T *ai, T *ao)
{
    switch (B) {
    case 2: k_blockdiag<2, T><<<g, kThreads, 0, st>>>(sys, ch, nch, gate, sel, ai, ao); break;
    case 3: k_blockdiag<3, T><<<g, kThreads, 0, st>>>(sys, ch, nch, gate, sel, ai, ao); break;
    case 4: k_blockdiag<4, T><<<g, kThreads, 0, st>>>(sys, ch, nch, gate, sel, ai, ao); break;
    }
}

inline dim3 grid_for(int nchunks)
{
    int cap = 8 * sm_count();
    return dim3((unsigned)std::max(1, std::min(nchunks, cap)));
}

int parts_for(int n, int part_dofs = kPartMax)
{
    int p = (n + part_dofs - 1) / part_dofs;
    return std::max(1, std::min(kMaxParts, p));
}

}  // namespace

// ---------------------------------------------------------------- autotuner
// Measured launch shapes of a batch, chosen by fg_autotune and cached per
// (block size, precision, batch-size class = floor(log2(batch dofs))) for
// the process: the dof-part size of the Krylov kernels and, for 3x3
// blocks in FP32, the matvec kernel (bulk-copy pipeline or the register
// kernel).  A batch with no cached choice uses the built-in rule.
struct TuneKey {
    int S, mixed, vhalf, cls;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(S, mixed, vhalf, cls) < std::tie(o.S, o.mixed, o.vhalf, o.cls);
    }
};
static std::mutex g_tune_mu;
static std::map<TuneKey, fg_tune_choice> g_tune;
// set by the autotuner while it times a candidate (this thread only)
static thread_local const fg_tune_choice *t_tune_force = nullptr;

static long long batch_dofs(const std::vector<BatchMember> &mem)
{
    long long tot = 0;
    for (auto &m : mem) tot += m.s->topo.n;
    return tot;
}
static TuneKey tune_key(int S, const SolveConfig &cfg, long long dofs)
{
    int cls = 0;
    while ((2LL << cls) <= std::max(1LL, dofs)) ++cls;
    return {S, cfg.mixed, cfg.vhalf, cls};
}
// the tuned choice of a batch, or nullptr
static bool tuned_choice(const std::vector<BatchMember> &mem, const SolveConfig &cfg, fg_tune_choice &out)
{
    if (t_tune_force) { out = *t_tune_force; return true; }
    if (mem.empty()) return false;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(mem[0].s->topo.S, cfg, batch_dofs(mem)));
    if (it == g_tune.end()) return false;
    out = it->second;
    return true;
}

namespace {

// part size of a batch (multiple of 8 dofs): the tuned one, else
// 2 sqrt(batch dofs) rounded to the nearest power of two, within
// [kPartMin, kPartMax] (powers of two: a system solved alone and inside a
// batch of similar size get the same parts, hence bit-identical results)
int part_dofs_for(const std::vector<BatchMember> &mem, const SolveConfig &cfg)
{
    fg_tune_choice tc;
    if (tuned_choice(mem, cfg, tc) && tc.part_dofs > 0) return tc.part_dofs & ~7;
    const double tot = (double)std::max(1LL, batch_dofs(mem));
    const long long pd = 1LL << (int)std::lround(std::log2(2.0 * std::sqrt(tot)));
    return (int)std::max<long long>(kPartMin, std::min<long long>(kPartMax, pd));
}

}  // namespace

// Chunk tables of one batch (device copies + host counts).
struct Plan {
    int nsys = 0, ncol = 0, S = 3, B = 1, maxdof = 1;   // ncol: patch colours
    int op = FG_OP_EBE, csr_w = 4, precond = FG_PRECOND_NONE, ilu_g = 4;
    std::vector<int> ech_off;      // ncol+1 offsets into echunks
    int n_dch = 0, n_nch = 0, n_ilu = 0, n_ilub = 0, n_spb = 0, n_spi = 0;
    DevMem sysdev, echunks, ecount, dchunks, dcount, nchunks, ncount, live;
    DevMem mvrec;                                  // 3x3: per matvec work item, for the bulk-copy pipeline
    bool mv3p = true;                              // 3x3 FP32: the bulk-copy pipeline (else the register kernel)
    bool rprec = false;                            // a right preconditioner (SGSe) before every matvec
    DevMem ilu_fwd, ilu_bwd, ilu_ctr;              // sync-free ILU(0) substitutions
    DevMem ilu_ws;                                 // block-Jacobi: (system, block) items, a warp each
    int n_ilw = 0, ilu_wx = 0, ilu_we = 0;         // items, rows of the largest block (0: level-scheduled
                                                   // path), entries of the longest chunk
    DevMem sp_blocks, sp_ifaces;                   // SPIKE (system, block) and (system, interface) items
};

static int build_plan(Plan &P, std::vector<BatchMember> &mem, const SolveConfig &cfg, std::vector<SysDev> &hs,
                      cudaStream_t st)
{
    P.nsys = (int)mem.size();
    P.S = mem[0].s->topo.S;
    P.B = mem[0].s->topo.ndof;
    P.ncol = 0;
    P.maxdof = 1;
    for (auto &m : mem) {
        if (m.s->topo.S != P.S) { set_error("a batch must hold systems of one block size"); return FG_ERR_ARG; }
        P.ncol = std::max(P.ncol, m.s->topo.npcol);
        P.maxdof = std::max(P.maxdof, m.s->topo.maxdof);
    }
    // matvec work items: one per patch, grouped by patch colour
    std::vector<EChunk> ech;
    P.ech_off.assign(P.ncol + 1, 0);
    for (int c = 0; c < P.ncol; ++c) {
        for (int s = 0; s < P.nsys; ++s) {
            const Topology &t = mem[s].s->topo;
            if (c >= t.npcol) continue;
            for (int q = t.pc_ptr[c]; q < t.pc_ptr[c + 1]; ++q) ech.push_back({s, t.pc_list[q], 0});
        }
        P.ech_off[c + 1] = (int)ech.size();
    }
    std::vector<DChunk> dch;
    std::vector<NChunk> nch;
    const int pdofs = part_dofs_for(mem, cfg);
    fg_tune_choice tc;
    const bool tuned = tuned_choice(mem, cfg, tc);
    P.mv3p = !(tuned && tc.mv3_pipeline == 0);
    P.rprec = cfg.precond == FG_PRECOND_SGSE;
    for (int s = 0; s < P.nsys; ++s) {
        int n = mem[s].s->topo.n;
        hs[s].nparts = parts_for(n, pdofs);
        int np = hs[s].nparts;
        // part boundaries on multiples of 8 dofs (16-byte packs in FP16, FP32 and FP64)
        for (int p = 0; p < np; ++p) {
            int d0 = (int)((long long)n * p / np) & ~7;
            int d1 = p + 1 == np ? n : (int)((long long)n * (p + 1) / np) & ~7;
            dch.push_back({s, p, d0, d1});
        }
        int nn = mem[s].s->topo.nnodes;
        for (int a = 0; a < nn; a += 1024) nch.push_back({s, a, std::min(a + 1024, nn)});
    }
    P.n_dch = (int)dch.size();
    P.n_nch = (int)nch.size();
    P.op = mem[0].s->op;
    P.precond = cfg.precond;
    P.csr_w = 4;
    for (auto &m : mem) {
        if (m.s->op != P.op) { set_error("a batch must use one operator kind"); return FG_ERR_ARG; }
        P.csr_w = std::max(P.csr_w, m.s->csr_w);
    }
    // ILU(0) substitutions: one item per pass of a system's level order
    // (forward and backward lists), systems interleaved
    std::vector<int2> fwd, bwd;
    if (cfg.precond == FG_PRECOND_ILU0) {
        int r0;
        if ((r0 = P.ilu_ctr.alloc(64))) return r0;
        int maxp = 0;
        for (int s = 0; s < P.nsys; ++s) {
            maxp = std::max({maxp, mem[s].s->ilu_nfpass, mem[s].s->ilu_nbpass});
            P.ilu_g = std::max(P.ilu_g, mem[s].s->ilu_g);
        }
        for (int q = 0; q < maxp; ++q)
            for (int s = 0; s < P.nsys; ++s) {
                if (q < mem[s].s->ilu_nfpass) fwd.push_back(make_int2(s, q));
                if (q < mem[s].s->ilu_nbpass) bwd.push_back(make_int2(s, q));
            }
        P.n_ilu = (int)fwd.size();
        P.n_ilub = (int)bwd.size();
        // every member block-Jacobi with blocks small enough: a warp per block
        int wx = 0, we = 1;
        bool ws = true;
        for (int s = 0; s < P.nsys && ws; ++s) {
            const int rows = ilu_ws_rows(mem[s].s);
            ws = rows > 0;
            wx = std::max(wx, rows);
            we = std::max(we, mem[s].s->ilu_maxrow);
        }
        we *= kIluWsChunk;
        if (ws && P.nsys > 0) {
            std::vector<int2> wit;
            for (int s = 0; s < P.nsys; ++s) {
                const int np = std::max(1, std::min(mem[s].s->ilu_blocks, mem[s].s->topo.n));
                for (int q = 0; q < np; ++q) wit.push_back(make_int2(s, q));
            }
            if ((r0 = P.ilu_ws.alloc(sizeof(int2) * wit.size()))) return r0;
            FG_CUDA(cudaMemcpyAsync(P.ilu_ws.p, wit.data(), sizeof(int2) * wit.size(), cudaMemcpyHostToDevice, st));
            P.n_ilw = (int)wit.size();
            P.ilu_wx = wx;
            P.ilu_we = we;
        }
    }
    // SPIKE: one CTA per block and per interface of every member
    std::vector<int2> spb, spi;
    if (cfg.precond == FG_PRECOND_SPIKE)
        for (int s = 0; s < P.nsys; ++s) {
            const int np = mem[s].s->sp_P;
            for (int q = 0; q < np; ++q) spb.push_back(make_int2(s, q));
            for (int q = 0; q + 1 < np; ++q) spi.push_back(make_int2(s, q));
        }
    P.n_spb = (int)spb.size();
    P.n_spi = (int)spi.size();
    std::vector<int> ecounts(P.ncol);
    for (int c = 0; c < P.ncol; ++c) ecounts[c] = P.ech_off[c + 1] - P.ech_off[c];
    std::vector<MvRec> recs;
    if (P.S == 3) {
        recs.reserve(ech.size());
        for (const EChunk &k : ech) {
            const Topology &t = mem[k.sys].s->topo;
            const int p = k.e0;
            const int pne = t.pt_elem[p + 1] - t.pt_elem[p], pnd = t.pt_dof[p + 1] - t.pt_dof[p];
            const int ni = t.pt_inc[p + 1] - t.pt_inc[p];
            recs.push_back({k.sys, t.pt_elem[p], (int)(t.pt_boff[p] / 16), (int)(t.pt_boff[p + 1] - t.pt_boff[p]),
                            t.pt_xlo[p], pne | (pnd << 16), ni | (t.pt_xlen[p] << 16), 0});
        }
    }
    int r;
    if ((r = P.sysdev.alloc(sizeof(SysDev) * hs.size())) ||
        (r = P.echunks.alloc(sizeof(EChunk) * std::max<size_t>(1, ech.size()))) ||
        (!recs.empty() && (r = P.mvrec.alloc(sizeof(MvRec) * recs.size()))) ||
        (r = P.ecount.alloc(sizeof(int) * std::max(1, P.ncol))) ||
        (r = P.dchunks.alloc(sizeof(DChunk) * std::max<size_t>(1, dch.size()))) ||
        (r = P.dcount.alloc(sizeof(int))) ||
        (r = P.nchunks.alloc(sizeof(NChunk) * std::max<size_t>(1, nch.size()))) ||
        (r = P.ncount.alloc(sizeof(int))) ||
        (r = P.live.alloc(sizeof(int) * P.nsys)) ||
        (r = P.ilu_fwd.alloc(sizeof(int2) * std::max<size_t>(1, fwd.size()))) ||
        (r = P.ilu_bwd.alloc(sizeof(int2) * std::max<size_t>(1, bwd.size()))) ||
        (r = P.sp_blocks.alloc(sizeof(int2) * std::max<size_t>(1, spb.size()))) ||
        (r = P.sp_ifaces.alloc(sizeof(int2) * std::max<size_t>(1, spi.size()))))
        return r;
    if (!recs.empty())
        FG_CUDA(cudaMemcpyAsync(P.mvrec.p, recs.data(), sizeof(MvRec) * recs.size(), cudaMemcpyHostToDevice, st));
    if (!spb.empty())
        FG_CUDA(cudaMemcpyAsync(P.sp_blocks.p, spb.data(), sizeof(int2) * spb.size(), cudaMemcpyHostToDevice, st));
    if (!spi.empty())
        FG_CUDA(cudaMemcpyAsync(P.sp_ifaces.p, spi.data(), sizeof(int2) * spi.size(), cudaMemcpyHostToDevice, st));
    if (!fwd.empty()) {
        FG_CUDA(cudaMemcpyAsync(P.ilu_fwd.p, fwd.data(), sizeof(int2) * fwd.size(), cudaMemcpyHostToDevice, st));
        FG_CUDA(cudaMemcpyAsync(P.ilu_bwd.p, bwd.data(), sizeof(int2) * bwd.size(), cudaMemcpyHostToDevice, st));
    }
    FG_CUDA(cudaMemcpyAsync(P.sysdev.p, hs.data(), sizeof(SysDev) * hs.size(), cudaMemcpyHostToDevice, st));
    if (!ech.empty())
        FG_CUDA(cudaMemcpyAsync(P.echunks.p, ech.data(), sizeof(EChunk) * ech.size(), cudaMemcpyHostToDevice, st));
    if (P.ncol)
        FG_CUDA(cudaMemcpyAsync(P.ecount.p, ecounts.data(), sizeof(int) * P.ncol, cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(P.dchunks.p, dch.data(), sizeof(DChunk) * dch.size(), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(P.dcount.p, &P.n_dch, sizeof(int), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(P.nchunks.p, nch.data(), sizeof(NChunk) * nch.size(), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(P.ncount.p, &P.n_nch, sizeof(int), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaStreamSynchronize(st));   // host vectors above go out of scope
    return FG_OK;
}

// Enqueue the matvec over all colours: mode 0 (x -> t64, FP64, gate live)
// or mode 1 (V[step] -> t, T, gate in_cycle).
template <typename TA, typename TX, typename TY>
static void launch_csr_mv(const Plan &P, cudaStream_t st, int gate, int in_sel, int out_sel, int step)
{
    const SysDev *sys = P.sysdev.as<SysDev>();
    dim3 g = grid_for(P.n_dch);
    const DChunk *dc = P.dchunks.as<DChunk>();
    const int *nd = P.dcount.as<int>();
    if (P.csr_w == 4)
        k_csr_mv<4, TA, TX, TY><<<g, kThreads, 0, st>>>(sys, dc, nd, gate, in_sel, out_sel, step, nullptr, nullptr);
    else if (P.csr_w == 8)
        k_csr_mv<8, TA, TX, TY><<<g, kThreads, 0, st>>>(sys, dc, nd, gate, in_sel, out_sel, step, nullptr, nullptr);
    else
        k_csr_mv<32, TA, TX, TY><<<g, kThreads, 0, st>>>(sys, dc, nd, gate, in_sel, out_sel, step, nullptr, nullptr);
}

// Enqueue the matvec: mode 0 (x -> t64, FP64, gate live), mode 1 (V[step]
// -> t, T, gate in_cycle), mode 2 (V[0] -> t, T, every member), mode 3
// (x -> t64, FP64, every member).  Returns the number of kernels.
// TV: storage type of the basis vector read in mode 1 (the Arnoldi step)
template <typename T, typename TV = T>
static int enqueue_matvec(const Plan &P, int mode, int step, cudaStream_t st)
{
    const bool f64 = mode == 0 || mode == 3;
    const int gate = mode == 0 ? 0 : mode == 1 ? 1 : -1;
    const int sel = f64 ? 0 : 1;
    // pgmres.c:61,93: v = precondR(x or u_i) before the matvec (SGSe), into r64
    int in0 = 0, in1 = 1, kr = 0;
    if (P.rprec && (mode == 0 || mode == 1)) {
        launch_elem_prec(P.sysdev.as<SysDev>(), P.nsys, 3, mode == 0 ? 0 : 1, step, st);
        in0 = in1 = 3;
        kr = 1;
    }
    if (P.op == FG_OP_CSR) {
        if (f64) launch_csr_mv<double, double, double>(P, st, gate, sel, sel, step);
        else launch_csr_mv<T, TV, T>(P, st, gate, sel, sel, step);
        return 1;
    }
    const SysDev *sys = P.sysdev.as<SysDev>();
    int k = 0;
    for (int c = 0; c < P.ncol; ++c) {
        int cnt = P.ech_off[c + 1] - P.ech_off[c];
        if (!cnt) continue;
        const EChunk *ch = P.echunks.as<EChunk>() + P.ech_off[c];
        const int *nc = P.ecount.as<int>() + c;
        bool done = false;
        if (f64) {
            MvLaunch::go<double, double, double>(P.S, cnt, st, sys, ch, nc, gate, in0, 0, 0, nullptr, nullptr,
                                                 P.maxdof);
            done = true;
        }
        if constexpr (sizeof(T) == 4) {
            if (!done && P.S == 3 && kMv3Pipeline && P.mv3p && P.mvrec.p) {
                MvLaunch::pipeline<TV, T>(cnt, st, sys, P.mvrec.as<MvRec>() + P.ech_off[c], nc, gate, 1, 1, step,
                                          nullptr, nullptr);
                done = true;
            }
        }
        if (!done) MvLaunch::go<T, TV, T>(P.S, cnt, st, sys, ch, nc, gate, in1, 1, step, nullptr, nullptr, P.maxdof);
        ++k;
    }
    return k + kr;
}

// M^-1 applied after a matvec: sel 0 (t64 -> u64, FP64) or 1 (t -> w, T).
template <typename T>
static int enqueue_precond(const Plan &P, int sel, cudaStream_t st)
{
    const SysDev *sys = P.sysdev.as<SysDev>();
    if (P.precond == FG_PRECOND_BLOCKDIAG) {
        if (sel == 0)
            launch_blockdiag<double>(P.B, grid_for(P.n_nch), st, sys, P.nchunks.as<NChunk>(), P.ncount.as<int>(), 0,
                                     0, nullptr, nullptr);
        else
            launch_blockdiag<T>(P.B, grid_for(P.n_nch), st, sys, P.nchunks.as<NChunk>(), P.ncount.as<int>(), 1, 1,
                                nullptr, nullptr);
        return 1;
    }
    if (P.precond == FG_PRECOND_LUE || P.precond == FG_PRECOND_SGSE) {   // FP64 only
        launch_elem_prec(sys, P.nsys, P.precond == FG_PRECOND_LUE ? 1 : 2, sel, 0, st);
        return 1;
    }
    if (P.precond == FG_PRECOND_ILU0 && P.n_ilw > 0) {
        const int fp32 = sel == 1 && sizeof(T) == 4;
        launch_ilu_ws(sys, P.ilu_ws.as<int2>(), P.n_ilw, sel, 0, fp32, P.ilu_g, P.ilu_wx, P.ilu_we, st);
        launch_ilu_ws(sys, P.ilu_ws.as<int2>(), P.n_ilw, sel, 1, fp32, P.ilu_g, P.ilu_wx, P.ilu_we, st);
        return 2;
    }
    if (P.precond == FG_PRECOND_ILU0) {
        int *ctr = P.ilu_ctr.as<int>(), *err = ctr + 4;
        const int fp32 = sel == 1 && sizeof(T) == 4;
        launch_ilu_pending(sys, P.dchunks.as<DChunk>(), P.dcount.as<int>(), P.n_dch, sel, fp32, st);
        launch_ilu_solve(sys, P.ilu_fwd.as<int2>(), P.n_ilu, ctr, err, sel, 0, fp32, P.ilu_g, st);
        launch_ilu_solve(sys, P.ilu_bwd.as<int2>(), P.n_ilub, ctr, err, sel, 1, fp32, P.ilu_g, st);
        return 3;
    }
    if (P.precond == FG_PRECOND_SPIKE) {
        const int fp32 = sel == 1 && sizeof(T) == 4;
        launch_spike_apply(sys, P.sp_blocks.as<int2>(), P.n_spb, P.sp_ifaces.as<int2>(), P.n_spi, sel, fp32, st);
        return P.n_spi > 0 ? 3 : 1;
    }
    return 0;
}

// One restart cycle for every member; returns the number of kernels.  TV
// is the basis' storage type (T, or FP16 under FP32 arithmetic).
template <typename T, typename TV = T>
static int enqueue_cycle(const Plan &P, const SolveConfig &cfg, cudaStream_t st)
{
    const SysDev *sys = P.sysdev.as<SysDev>();
    const DChunk *dc = P.dchunks.as<DChunk>();
    const int *nd = P.dcount.as<int>();
    dim3 gd = grid_for(P.n_dch);
    // mixed precision: one sweep fewer per step (Gram-corrected CGS); the
    // FP64 reference method keeps two full classical passes
    const bool gram = cfg.mixed && cfg.kmax <= 32;   // 2 (i + 1) partial sums fit a part slot
    int k = enqueue_matvec<T>(P, 0, 0, st);
    k += enqueue_precond<T>(P, 0, st);
    k_start<<<gd, kThreads, 0, st>>>(sys, dc, nd);
    k_scale_v0<T, TV><<<gd, kThreads, 0, st>>>(sys, dc, nd);
    k += 2;
    for (int i = 0; i < cfg.kmax - 1; ++i) {
        k += enqueue_matvec<T, TV>(P, 1, i, st);
        k += enqueue_precond<T>(P, 1, st);
        if constexpr (std::is_same<T, TV>::value) {
            if (gram) {
                k_dots1g<T><<<gd, kThreads, 0, st>>>(sys, dc, nd, i);
            } else {
                k_dots1<T><<<gd, kThreads, 0, st>>>(sys, dc, nd, i);
                k_orth1<T><<<gd, kThreads, 0, st>>>(sys, dc, nd, i);
                ++k;
            }
        } else {
            k_dots1g<T, TV><<<gd, kThreads, 0, st>>>(sys, dc, nd, i);   // narrow basis: Gram path only
        }
        k_orth2<T, TV><<<gd, kThreads, 0, st>>>(sys, dc, nd, i);
        k_normalize<T, TV><<<gd, kThreads, 0, st>>>(sys, dc, nd, i);
        k += 3;
    }
    k_update<T, TV><<<gd, kThreads, 0, st>>>(sys, dc, nd);
    k_live<<<(P.nsys + 255) / 256, 256, 0, st>>>(sys, P.nsys, P.live.as<int>());
    return k + 2;
}

// mode: 0 FP64, 1 FP32 basis, 2 FP16 basis (mixed precision in both)
static int ensure_workspace(fg_system *s, int kmax, int mode)
{
    Workspace &w = s->ws;
    if (w.kmax >= kmax && w.mixed == mode) return FG_OK;
    w.kmax = 0;
    w.mixed = -1;
    size_t np = (size_t)s->n_pad;
    size_t ts = mode ? sizeof(float) : sizeof(double);
    size_t vs = mode == 2 ? 2 : ts;
    int r;
    if ((r = w.V.alloc(vs * np * kmax)) || (r = w.w.alloc(ts * np)) || (r = w.t.alloc(ts * np)) ||
        (r = w.x.alloc(8 * np)) || (r = w.b.alloc(8 * np)) || (r = w.ftrue.alloc(8 * np)) ||
        (r = w.r64.alloc(8 * np)) || (r = w.t64.alloc(8 * np)) || (r = w.u64.alloc(8 * np)) ||
        (r = w.small.alloc(8 * ((size_t)(kmax + 1) * kmax + 5 * (kmax + 1) + (size_t)kmax * kmax))) ||
        (r = w.part.alloc(8 * (size_t)kMaxParts * kPartStride)) ||
        (r = w.counter.alloc(sizeof(unsigned) * 8)) || (r = w.state.alloc(sizeof(SysState))))
        return r;
    w.kmax = kmax;
    w.mixed = mode;
    return FG_OK;
}

static SysDev make_desc(fg_system *s, const SolveConfig &cfg, bool has_f)
{
    const Topology &t = s->topo;
    Workspace &w = s->ws;
    SysDev D{};
    D.n = t.n; D.n_pad = s->n_pad; D.nel = t.nel; D.nel_pad = s->nel_pad; D.S = t.S; D.ndof = t.ndof;
    D.ncol = t.ncol; D.nparts = parts_for(t.n); D.nnodes = t.nnodes;
    D.kmax = cfg.kmax; D.lmax = cfg.lmax; D.mixed = cfg.mixed; D.precond = cfg.precond;
    D.tol = cfg.tol; D.inner_tol = cfg.inner_tol;
    D.vhalf = cfg.vhalf;
    D.vsc = D.vsci = 1.0f;
    if (cfg.vhalf) {   // unit vectors times 2^floor(log2 sqrt n): entries of order 1 in FP16
        const int e = (int)std::floor(0.5 * std::log2((double)std::max(t.n, 1)));
        D.vsc = std::ldexp(1.0f, e);
        D.vsci = std::ldexp(1.0f, -e);
    }
    D.lm = s->lm.as<int>(); D.A64 = s->A64.as<double>(); D.A32 = s->A32.as<float>();
    set_patch_fields(D, s);
    D.invd64 = s->invd64.as<double>(); D.invd32 = s->invd32.as<float>();
    D.node_dof = s->node_dof.as<int>(); D.ibd64 = s->ibd64.as<double>(); D.ibd32 = s->ibd32.as<float>();
    D.x = w.x.as<double>(); D.b = w.b.as<double>(); D.ftrue = has_f ? w.ftrue.as<double>() : nullptr;
    D.r64 = w.r64.as<double>(); D.t64 = w.t64.as<double>(); D.u64 = w.u64.as<double>();
    D.V = w.V.p; D.w = w.w.p; D.t = w.t.p;
    double *sm = w.small.as<double>();
    D.H = sm;
    D.g = sm + (size_t)(cfg.kmax + 1) * cfg.kmax;
    D.cs = D.g + (cfg.kmax + 1);
    D.sn = D.cs + (cfg.kmax + 1);
    D.hbuf = D.sn + (cfg.kmax + 1);
    D.y = D.hbuf + (cfg.kmax + 1);
    D.G = D.y + (cfg.kmax + 1);
    D.part = w.part.as<double>();
    D.counter = w.counter.as<unsigned>();
    D.st = w.state.as<SysState>();
    return D;
}

int validate_member(fg_system *s, const SolveConfig &cfg)
{
    if (cfg.kmax < 2 || cfg.kmax > kPartStride - 4) { set_error("kmax must be in [2, 60]"); return FG_ERR_ARG; }
    if (cfg.lmax < 1) { set_error("lmax must be >= 1"); return FG_ERR_ARG; }
    if (!s->blocks_ok) { set_error("solve before element blocks were set"); return FG_ERR_STATE; }
    if (cfg.precond != FG_PRECOND_NONE && s->precond != cfg.precond) {
        set_error("solve with a preconditioner that was not set up"); return FG_ERR_STATE;
    }
    if (cfg.precond == FG_PRECOND_BLOCKDIAG && s->topo.ndof < 2) {
        set_error("block-diagonal preconditioner needs ndof >= 2"); return FG_ERR_UNSUPPORTED;
    }
    if (s->op == FG_OP_CSR && !s->csr_ok) { set_error("CSR operator selected but not set up"); return FG_ERR_STATE; }
    if (cfg.precond == FG_PRECOND_ILU0 && s->op != FG_OP_CSR) {
        set_error("ILU(0) needs the CSR operator (fg_set_operator(FG_OP_CSR))"); return FG_ERR_STATE;
    }
    if ((cfg.precond == FG_PRECOND_LUE || cfg.precond == FG_PRECOND_SGSE) &&
        (cfg.mixed || s->topo.S != 3 || s->op != FG_OP_EBE)) {
        set_error("the element preconditioners LUe / SGSe run in FP64 on 3x3 EBE systems");
        return FG_ERR_UNSUPPORTED;
    }
    if (cfg.precond == FG_PRECOND_SPIKE && (s->op != FG_OP_CSR || !s->sp_ready)) {
        set_error("SPIKE needs the CSR operator and its set-up (fg_precond_setup)"); return FG_ERR_STATE;
    }
    return FG_OK;
}

size_t workspace_bytes(const fg_system *s, int kmax, int mixed)
{
    size_t np = (size_t)s->n_pad, ts = mixed ? 4 : 8;
    return ts * np * (kmax + 2) + 8 * np * 6 +
           8 * ((size_t)(kmax + 1) * kmax + 5 * (kmax + 1) + (size_t)kmax * kmax) +
           8 * (size_t)kMaxParts * kPartStride + 256;
}

int autotune(std::vector<fg_system *> &sys, const SolveConfig &cfg0, bool remeasure, bool lookup_only,
             fg_tune_choice *out)
{
    if (sys.empty()) { set_error("fg_autotune: empty batch"); return FG_ERR_ARG; }
    std::vector<BatchMember> mem;
    for (fg_system *s : sys) {
        if (!s) { set_error("fg_autotune: NULL system"); return FG_ERR_ARG; }
        if (s->topo.S != sys[0]->topo.S) { set_error("fg_autotune: a batch must hold one block size"); return FG_ERR_ARG; }
        if (!s->rhs_ok) { set_error("fg_autotune: system without a resident right-hand side"); return FG_ERR_STATE; }
        mem.push_back({s, s->rhs_b.as<double>(), s->rhs_f.as<double>(), nullptr});
    }
    SolveConfig cfg = cfg0;
    cfg.device_io = 1;
    cfg.use_graph = 0;
    cfg.precond = sys[0]->precond;
    const TuneKey key = tune_key(sys[0]->topo.S, cfg, batch_dofs(mem));
    if (!remeasure || lookup_only) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            *out = it->second;
            out->from_cache = 1;
            return FG_OK;
        }
        if (lookup_only) { set_error("fg_tune_lookup: no cached choice for this batch"); return FG_ERR_STATE; }
    }
    cudaStream_t st = sys[0]->stream;
    for (fg_system *s : sys) FG_CUDA(cudaStreamSynchronize(s->stream));
    std::vector<fg_tune_choice> cand;
    const int pds[] = {256, 512, 1024, 2048, 4096, 8192, 12288, 16384};
    const bool mv3_alt = sys[0]->topo.S == 3 && cfg.mixed && !cfg.vhalf;
    for (int pd : pds)
        for (int mv = 1; mv >= (mv3_alt ? 0 : 1); --mv) cand.push_back({pd, mv, 0.0, 0, 0});
    const char *tlog = getenv("FEMGPU_TUNE_LOG");
    const bool log = tlog && *tlog && *tlog != '0';
    cudaEvent_t e0, e1;
    FG_CUDA(cudaEventCreate(&e0));
    FG_CUDA(cudaEventCreate(&e1));
    fg_tune_choice best{};
    best.ms_per_cycle = 1e300;
    int r = FG_OK;
    std::vector<int> live;
    for (auto &c : cand) {
        t_tune_force = &c;
        {
            BatchRun run(cfg, st);
            for (auto &m : mem)
                if ((r = run.stage(m))) break;
            if (!r) r = run.commit();
            if (!r) r = run.cycle(false, live);                     // warm-up (first launches)
            if (!r) {
                cudaEventRecord(e0, st);
                r = run.cycle(false, live);
                cudaEventRecord(e1, st);
            }
            if (!r) {
                float ms = 0.f;
                cudaError_t ce = cudaEventSynchronize(e1);
                if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
                if (ce != cudaSuccess) r = cuda_fail(ce, "fg_autotune timing");
                c.ms_per_cycle = ms;
            }
        }
        t_tune_force = nullptr;
        if (r) break;
        if (log)
            fprintf(stderr, "fg_autotune: S=%d mixed=%d part_dofs=%d mv3_pipeline=%d: %.3f ms/cycle\n",
                    sys[0]->topo.S, cfg.mixed, c.part_dofs, c.mv3_pipeline, c.ms_per_cycle);
        if (c.ms_per_cycle < best.ms_per_cycle) best = c;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (r) return r;
    best.candidates = (int)cand.size();
    best.from_cache = 0;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[key] = best;
    }
    *out = best;
    return FG_OK;
}

int tune_set(std::vector<fg_system *> &sys, const SolveConfig &cfg0, const fg_tune_choice &c)
{
    if (sys.empty()) { set_error("fg_tune_set: empty batch"); return FG_ERR_ARG; }
    std::vector<BatchMember> mem;
    for (fg_system *s : sys) {
        if (!s) { set_error("fg_tune_set: NULL system"); return FG_ERR_ARG; }
        if (s->topo.S != sys[0]->topo.S) { set_error("fg_tune_set: a batch must hold one block size"); return FG_ERR_ARG; }
        mem.push_back({s, nullptr, nullptr, nullptr});
    }
    if (c.part_dofs < kPartMin || c.part_dofs > kPartMax || c.part_dofs % 8 || (c.mv3_pipeline & ~1)) {
        set_error("fg_tune_set: part_dofs must be a multiple of 8 in [256, 16384], mv3_pipeline 0 or 1");
        return FG_ERR_ARG;
    }
    SolveConfig cfg = cfg0;
    cfg.precond = sys[0]->precond;
    fg_tune_choice k = c;
    k.from_cache = 0;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[tune_key(sys[0]->topo.S, cfg, batch_dofs(mem))] = k;
    return FG_OK;
}

void tune_clear()
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
}

size_t request_bytes(const fg_system *s, int kmax, int mixed, bool time_loop)
{
    const Workspace &w = s->ws;
    const DevMem *held[] = {&w.V, &w.w, &w.t, &w.x, &w.b, &w.ftrue, &w.r64, &w.t64, &w.u64, &w.small, &w.part,
                            &w.counter, &w.state};
    size_t have = 0;
    for (auto *m : held) have += m->bytes;
    size_t b = s->bytes() - std::min(have, s->bytes()) + workspace_bytes(s, kmax, mixed);
    if (time_loop) {
        const DevMem *loop[] = {&s->rhs_f, &s->rhs_b, &s->state_u, &s->state_a, &s->state_old};
        for (auto *m : loop)
            if (!m->p) b += 8 * (size_t)s->n_pad;
    }
    return b;
}

BatchRun::BatchRun(const SolveConfig &c, cudaStream_t s) : cfg(c), st(s) {}

BatchRun::~BatchRun()
{
    if (exec) cudaGraphExecDestroy(exec);
    if (h_live) cudaFreeHost(h_live);
}

// Workspace, cleared vectors and right-hand side of a new member (queued on
// the batch stream); the member joins at the next commit().
int BatchRun::stage(const BatchMember &m)
{
    fg_system *s = m.s;
    int r = validate_member(s, cfg);
    if (r) return r;
    if ((r = ensure_workspace(s, cfg.kmax, cfg.mixed + cfg.vhalf))) return r;
    if (s->op == FG_OP_CSR && (r = csr_refresh(s, st))) return r;
    Workspace &w = s->ws;
    size_t vb = 8 * (size_t)s->n_pad;
    FG_CUDA(cudaMemsetAsync(w.x.p, 0, vb, st));
    FG_CUDA(cudaMemsetAsync(w.t64.p, 0, vb, st));
    FG_CUDA(cudaMemsetAsync(w.t.p, 0, (cfg.mixed ? 4 : 8) * (size_t)s->n_pad, st));
    FG_CUDA(cudaMemsetAsync(w.V.p, 0, (cfg.vhalf ? 2 : cfg.mixed ? 4 : 8) * (size_t)s->n_pad * cfg.kmax, st));
    FG_CUDA(cudaMemsetAsync(w.small.p, 0, w.small.bytes, st));
    if (cfg.device_io) {
        FG_CUDA(cudaMemcpyAsync(w.b.p, m.B, 8 * (size_t)(s->topo.n + 1), cudaMemcpyDeviceToDevice, st));
        if (m.Ftrue) FG_CUDA(cudaMemcpyAsync(w.ftrue.p, m.Ftrue, 8 * (size_t)(s->topo.n + 1), cudaMemcpyDeviceToDevice, st));
    } else {
        // host vectors in reference numbering -> staging -> internal numbering
        size_t hb = 8 * (size_t)(s->topo.n + 1);
        FG_CUDA(cudaMemcpyAsync(w.r64.p, m.B, hb, cudaMemcpyHostToDevice, st));
        if ((r = permute_in(s, w.r64.as<double>(), w.b.as<double>(), st))) return r;
        if (m.Ftrue) {
            FG_CUDA(cudaMemcpyAsync(w.u64.p, m.Ftrue, hb, cudaMemcpyHostToDevice, st));
            if ((r = permute_in(s, w.u64.as<double>(), w.ftrue.as<double>(), st))) return r;
        }
    }
    mem.push_back(m);
    hs.push_back(make_desc(s, cfg, m.Ftrue != nullptr));
    ++pending;
    return FG_OK;
}

// Rebuild the work tables for the current members and initialise the state
// of the members staged since the last commit.
int BatchRun::commit()
{
    if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
    if (mem.empty()) { pending = 0; return FG_OK; }
    P = std::make_unique<Plan>();
    int r = build_plan(*P, mem, cfg, hs, st);
    if (r) return r;
    if (pending > 0) {
        int first = (int)mem.size() - pending;
        k_init_state<<<(pending + 127) / 128, 128, 0, st>>>(P->sysdev.as<SysDev>() + first, pending);
        FG_CUDA(cudaGetLastError());
        count_launches(1);
    }
    pending = 0;
    if ((int)live_cap < (int)mem.size()) {
        if (h_live) cudaFreeHost(h_live);
        live_cap = std::max<size_t>(mem.size(), 2 * live_cap);
        FG_CUDA(cudaMallocHost(&h_live, sizeof(int) * live_cap));
    }
    return FG_OK;
}

// One restart cycle of every member; live[i] tells whether member i goes on.
int BatchRun::cycle(bool use_graph, std::vector<int> &live)
{
    live.assign(mem.size(), 0);
    if (mem.empty()) return FG_OK;
    const Plan &Pl = *P;
    cudaError_t ce = cudaSuccess;
    if (use_graph && !exec) {
        cudaGraph_t graph = nullptr;
        FG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        graph_nodes = cfg.vhalf ? enqueue_cycle<float, __half>(Pl, cfg, st)
                             : cfg.mixed ? enqueue_cycle<float>(Pl, cfg, st) : enqueue_cycle<double>(Pl, cfg, st);
        ce = cudaStreamEndCapture(st, &graph);
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
        ce = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) { exec = nullptr; return cuda_fail(ce, "cudaGraphInstantiate"); }
    }
    if (use_graph) {
        ce = cudaGraphLaunch(exec, st);
        count_launches(graph_nodes);
    } else {
        count_launches(cfg.vhalf ? enqueue_cycle<float, __half>(Pl, cfg, st)
                             : cfg.mixed ? enqueue_cycle<float>(Pl, cfg, st) : enqueue_cycle<double>(Pl, cfg, st));
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(h_live, Pl.live.p, sizeof(int) * mem.size(), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return cuda_fail(ce, "GMRES cycle");
    for (size_t i = 0; i < mem.size(); ++i) live[i] = h_live[i];
    return FG_OK;
}

// True residual of the listed members' current x (FP64), then their state.
int BatchRun::finish(const std::vector<int> &idx, std::vector<SysState> &out)
{
    out.assign(idx.size(), SysState{});
    if (idx.empty()) return FG_OK;
    std::vector<BatchMember> sub;
    std::vector<SysDev> shs;
    for (int i : idx) { sub.push_back(mem[i]); shs.push_back(hs[i]); }
    Plan F;
    int r = build_plan(F, sub, cfg, shs, st);
    if (r) return r;
    const SysDev *sys = F.sysdev.as<SysDev>();
    if (F.rprec) launch_elem_prec(sys, F.nsys, 3, 2, 0, st);   // pgmres.c:186: X = precondR(X)
    count_launches(enqueue_matvec<double>(F, 3, 0, st));
    k_final<<<grid_for(F.n_dch), kThreads, 0, st>>>(sys, F.dchunks.as<DChunk>(), F.dcount.as<int>());
    FG_CUDA(cudaGetLastError());
    count_launches(1);
    for (size_t q = 0; q < idx.size(); ++q)
        FG_CUDA(cudaMemcpyAsync(&out[q], sub[q].s->ws.state.p, sizeof(SysState), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    return FG_OK;
}

// Drop members (indices ascending or not); the tables are rebuilt at the
// next commit().
void BatchRun::remove(std::vector<int> idx)
{
    std::sort(idx.rbegin(), idx.rend());
    for (int i : idx) {
        mem.erase(mem.begin() + i);
        hs.erase(hs.begin() + i);
    }
    if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
    P.reset();
}

void fill_stats(const SysState &s, double secs, fg_solve_stats &o)
{
    o.iterations = s.iterations;
    o.cycles = s.cycles;
    o.converged = s.converged;
    o.status = s.status;
    o.rho = s.rho;
    o.eps = s.eps;
    o.true_rel_residual = s.true_res;
    o.seconds = secs;
}

int solve_batch(std::vector<BatchMember> &mem, const SolveConfig &cfg, fg_solve_stats *stats, cudaStream_t st)
{
    if (mem.empty()) return FG_OK;
    for (auto &m : mem) {
        int r = validate_member(m.s, cfg);
        if (r) return r;
    }
    auto t0 = std::chrono::steady_clock::now();
    BatchRun run(cfg, st);
    int r;
    for (auto &m : mem)
        if ((r = run.stage(m))) return r;
    if ((r = run.commit())) return r;
    std::vector<int> live;
    for (int cyc = 0; cyc < cfg.lmax + 2; ++cyc) {
        if ((r = run.cycle(cfg.use_graph != 0, live))) return r;
        int any = 0;
        for (int v : live) any |= v;
        if (!any) break;
    }
    std::vector<int> all(mem.size());
    for (size_t i = 0; i < all.size(); ++i) all[i] = (int)i;
    std::vector<SysState> sts;
    if ((r = run.finish(all, sts))) return r;
    for (size_t i = 0; i < mem.size(); ++i) {
        BatchMember &m = mem[i];
        fg_system *sy = m.s;
        if (!m.X) continue;
        if (cfg.device_io) {
            FG_CUDA(cudaMemcpyAsync(m.X, sy->ws.x.p, 8 * (size_t)(sy->topo.n + 1), cudaMemcpyDeviceToDevice, st));
        } else {
            if ((r = permute_out(sy, sy->ws.x.as<double>(), sy->ws.r64.as<double>(), st))) return r;
            FG_CUDA(cudaMemcpyAsync(m.X, sy->ws.r64.p, 8 * (size_t)(sy->topo.n + 1), cudaMemcpyDeviceToHost, st));
        }
    }
    FG_CUDA(cudaStreamSynchronize(st));
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats)
        for (size_t i = 0; i < mem.size(); ++i) fill_stats(sts[i], secs, stats[i]);
    return FG_OK;
}

// Single matvec on device vectors (internal numbering, FP64 in/out).
int matvec_device(fg_system *s, const double *x, double *y, int precision, cudaStream_t st)
{
    if (!s->blocks_ok) { set_error("matvec before element blocks were set"); return FG_ERR_STATE; }
    const Topology &t = s->topo;
    SysDev D{};
    D.n = t.n; D.n_pad = s->n_pad; D.nel = t.nel; D.nel_pad = s->nel_pad; D.S = t.S;
    D.lm = s->lm.as<int>(); D.A64 = s->A64.as<double>(); D.A32 = s->A32.as<float>();
    set_patch_fields(D, s);
    DevMem sd, ch, cnt;
    std::vector<EChunk> ech;
    std::vector<int> off(t.npcol + 1, 0), counts(t.npcol);
    for (int c = 0; c < t.npcol; ++c) {
        for (int q = t.pc_ptr[c]; q < t.pc_ptr[c + 1]; ++q) ech.push_back({0, t.pc_list[q], 0});
        off[c + 1] = (int)ech.size();
        counts[c] = off[c + 1] - off[c];
    }
    int r;
    if ((r = sd.alloc(sizeof(SysDev))) || (r = ch.alloc(sizeof(EChunk) * std::max<size_t>(1, ech.size()))) ||
        (r = cnt.alloc(sizeof(int) * std::max(1, t.npcol))))
        return r;
    FG_CUDA(cudaMemcpyAsync(sd.p, &D, sizeof(SysDev), cudaMemcpyHostToDevice, st));
    if (!ech.empty()) FG_CUDA(cudaMemcpyAsync(ch.p, ech.data(), sizeof(EChunk) * ech.size(), cudaMemcpyHostToDevice, st));
    if (t.npcol) FG_CUDA(cudaMemcpyAsync(cnt.p, counts.data(), sizeof(int) * t.npcol, cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemsetAsync(y, 0, 8 * (size_t)(t.n + 1), st));
    if (s->op == FG_OP_CSR) {
        if ((r = csr_refresh(s, st))) return r;
        std::vector<DChunk> dch;
        for (int d = 0; d < t.n; d += 2048) dch.push_back({0, 0, d, std::min(d + 2048, t.n)});
        DevMem dc, dn;
        int nd = (int)dch.size();
        if ((r = dc.alloc(sizeof(DChunk) * std::max<size_t>(1, dch.size()))) || (r = dn.alloc(sizeof(int)))) return r;
        if (nd) FG_CUDA(cudaMemcpyAsync(dc.p, dch.data(), sizeof(DChunk) * nd, cudaMemcpyHostToDevice, st));
        FG_CUDA(cudaMemcpyAsync(dn.p, &nd, sizeof(int), cudaMemcpyHostToDevice, st));
        dim3 g = grid_for(std::max(nd, 1));
        const SysDev *sdp = sd.as<SysDev>();
        const DChunk *dcp = dc.as<DChunk>();
        const int *dnp = dn.as<int>();
        if (precision == 32) {
            if (s->csr_w == 4) k_csr_mv<4, float, double, double><<<g, kThreads, 0, st>>>(sdp, dcp, dnp, -1, 2, 2, 0, x, y);
            else if (s->csr_w == 8) k_csr_mv<8, float, double, double><<<g, kThreads, 0, st>>>(sdp, dcp, dnp, -1, 2, 2, 0, x, y);
            else k_csr_mv<32, float, double, double><<<g, kThreads, 0, st>>>(sdp, dcp, dnp, -1, 2, 2, 0, x, y);
        } else {
            if (s->csr_w == 4) k_csr_mv<4, double, double, double><<<g, kThreads, 0, st>>>(sdp, dcp, dnp, -1, 2, 2, 0, x, y);
            else if (s->csr_w == 8) k_csr_mv<8, double, double, double><<<g, kThreads, 0, st>>>(sdp, dcp, dnp, -1, 2, 2, 0, x, y);
            else k_csr_mv<32, double, double, double><<<g, kThreads, 0, st>>>(sdp, dcp, dnp, -1, 2, 2, 0, x, y);
        }
        FG_CUDA(cudaGetLastError());
        count_launches(1);
        FG_CUDA(cudaStreamSynchronize(st));
        return FG_OK;
    }
    for (int c = 0; c < t.npcol; ++c) {
        if (!counts[c]) continue;
        const EChunk *cp = ch.as<EChunk>() + off[c];
        const int *np = cnt.as<int>() + c;
        if (precision == 32)
            MvLaunch::go<float, double, double>(t.S, counts[c], st, sd.as<SysDev>(), cp, np, -1, 2, 2, 0, x, y, D.maxdof);
        else
            MvLaunch::go<double, double, double>(t.S, counts[c], st, sd.as<SysDev>(), cp, np, -1, 2, 2, 0, x, y, D.maxdof);
    }
    FG_CUDA(cudaGetLastError());
    count_launches(t.npcol);
    FG_CUDA(cudaStreamSynchronize(st));
    return FG_OK;
}

// The batched matvec alone, timed with CUDA events (fg_bench_matvec).
int bench_matvec(std::vector<fg_system *> &systems, int precision, int reps, double *ms, double *bytes)
{
    if (systems.empty() || reps < 1) { set_error("empty batch or reps < 1"); return FG_ERR_ARG; }
    SolveConfig cfg;
    cfg.mixed = precision == 32 ? 1 : 0;
    cfg.kmax = 2;
    std::vector<BatchMember> mem;
    std::vector<SysDev> hs;
    double b = 0;
    const double w = cfg.mixed ? 4.0 : 8.0;
    for (auto *s : systems) {
        if (!s->blocks_ok) { set_error("matvec before element blocks were set"); return FG_ERR_STATE; }
        int kk = std::max(2, s->ws.kmax);
        int r = ensure_workspace(s, kk, cfg.mixed);
        if (r) return r;
        cfg.kmax = kk;
        mem.push_back({s, nullptr, nullptr, nullptr});
        hs.push_back(make_desc(s, cfg, false));
        const Topology &t = s->topo;
        b += (double)t.nel * (t.S * t.S * w + t.S * 4.0) + 2.0 * t.n * w;
    }
    cudaStream_t st = systems[0]->stream;
    Plan P;
    int r = build_plan(P, mem, cfg, hs, st);
    if (r) return r;
    cudaEvent_t e0, e1;
    FG_CUDA(cudaEventCreate(&e0));
    FG_CUDA(cudaEventCreate(&e1));
    auto run = [&](int n) {
        for (int i = 0; i < n; ++i)
            count_launches(cfg.mixed ? enqueue_matvec<float>(P, 2, 0, st) : enqueue_matvec<double>(P, 2, 0, st));
    };
    run(2);  // warm-up
    cudaEventRecord(e0, st);
    run(reps);
    cudaEventRecord(e1, st);
    cudaError_t ce = cudaEventSynchronize(e1);
    float t = 0;
    if (ce == cudaSuccess) ce = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ce != cudaSuccess) return cuda_fail(ce, "bench_matvec");
    for (auto *s : systems)
        FG_CUDA(cudaMemsetAsync(s->ws.t.p, 0, s->ws.t.bytes, st));
    FG_CUDA(cudaStreamSynchronize(st));
    *ms = t / reps;
    *bytes = b;
    return FG_OK;
}

// Colour-by-colour matvec y += A x from a caller-placed descriptor and chunk
// table (device memory the caller owns); used by fg_matvec_noalloc.
int launch_matvec_colours(int S, int precision, const SysDev *sys_dev, const EChunk *ch_dev, const int *counts_dev,
                          const int *off_host, int ncol, int maxdof, const double *x, double *y, cudaStream_t st)
{
    for (int c = 0; c < ncol; ++c) {
        int cnt = off_host[c + 1] - off_host[c];
        if (!cnt) continue;
        const EChunk *cp = ch_dev + off_host[c];
        const int *np = counts_dev + c;
        if (precision == 32)
            MvLaunch::go<float, double, double>(S, cnt, st, sys_dev, cp, np, -1, 2, 2, 0, x, y, maxdof);
        else
            MvLaunch::go<double, double, double>(S, cnt, st, sys_dev, cp, np, -1, 2, 2, 0, x, y, maxdof);
        count_launches(1);
    }
    FG_CUDA(cudaGetLastError());
    return FG_OK;
}

static std::atomic<long long> g_launches{0};
void count_launches(long long n) { g_launches += n; }
long long launch_total() { return g_launches.load(); }

}  // namespace fg
