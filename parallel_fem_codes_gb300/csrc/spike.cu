// Truncated SPIKE preconditioner on the assembled CSR operator (Preconditioner
// "SPIKEk", Solvers_and_Preconditioners/CSR/SPIKE_precond_setup.c:10-312 and
// CSR/SPIKE_precond.c:8-158).
//
// The reference splits the matrix into one row block per MPI rank, factorises
// each diagonal block with PARDISO and couples neighbours through k x k
// corner blocks.  Here the ranks become sp_P row blocks of one system on one
// GPU (at most n / 2k of them, so every block keeps 2k rows):
//
//   set-up   k_spike_fill    band of every diagonal block (RCM keeps the CSR
//                            operator banded) and the corner couplings B_q
//                            (last k rows of q x first k columns of q+1) and
//                            C_q (first k rows of q x last k columns of q-1)
//            k_spike_lu      banded LU without pivoting, one CTA per block
//            k_spike_vtip    V_q = bottom k rows of A_q^-1 [0; B_q]
//            k_spike_wtip    W_q = top k rows of A_q^-1 [C_q; 0]
//            k_spike_reduced LU with partial pivoting of S_q = [I V_q; W_q+1 I]
//   apply    k_spike_block   g = A_q^-1 f, one CTA per block
//            k_spike_iface   [xB_q; xT_q+1] = S_q^-1 [g bottom(q); g top(q+1)]
//            k_spike_block   y_q = A_q^-1 (f_q - B_q xT_q+1 - C_q xB_q-1)
//
// A band solve is sequential over the rows of a block: each CTA sweeps its
// block column by column, the threads updating the rows below (forward) or
// above (backward) the current one, with one barrier per row.  The band
// values of the coming rows do not depend on the data, so each thread keeps
// the next kPrefetch columns' values in registers and the loop waits on
// barriers, not on memory.  The working vector of a block lives in shared
// memory when the block has at most kSpikeSmemRows rows.
//
// Compiled with -fmad=false; every element sees the same operations in the
// same order as the CPU restatement, so set-up and FP64 apply are bit-exact
// against it.
#include <algorithm>

#include "system.h"

namespace fg {

constexpr int kSpikeThreads = 256;
constexpr int kSpikeLuThreads = 1024;   // the trailing update of a step is kl x ku wide
constexpr int kPrefetch = 8;
constexpr size_t kSpikeMaxBandBytes = 8ull << 30;

struct Band {
    const double *a;
    int ld, ku;
    __device__ __forceinline__ double at(int i, int j) const { return a[(long long)(ku + i - j) + (long long)j * ld]; }
};

__device__ __forceinline__ bool spike_gate(const SysDev &D, int sel)
{
    if (sel == 0) return D.st == nullptr || D.st->live;
    return D.st->in_cycle != 0;
}

// ---------------------------------------------------------------- set-up
// One thread per row: scatter the row's entries into its block's band or a
// corner coupling; entries elsewhere are dropped (truncation).
__global__ void k_spike_fill(int n, const int *__restrict__ ia, const int *__restrict__ ja,
                             const double *__restrict__ AA, int P, int k, const int *__restrict__ bs,
                             const int *__restrict__ bl, const int *__restrict__ bu,
                             const long long *__restrict__ boff, double *band, double *B, double *C)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int lo = 0, hi = P - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (bs[mid] <= i) lo = mid; else hi = mid - 1;
    }
    const int q = lo, b0 = bs[q], b1 = bs[q + 1], ld = bl[q] + bu[q] + 1;
    const long long kk = (long long)k * k;
    for (int e = ia[i]; e < ia[i + 1]; ++e) {
        const int j = ja[e];
        if (j >= b0 && j < b1) {
            band[boff[q] + (long long)(bu[q] + (i - b0) - (j - b0)) + (long long)(j - b0) * ld] = AA[e];
        } else if (q + 1 < P && i >= b1 - k && j >= b1 && j < b1 + k) {
            B[q * kk + (long long)(i - (b1 - k)) * k + (j - b1)] = AA[e];
        } else if (q > 0 && i < b0 + k && j >= b0 - k && j < b0) {
            C[(q - 1) * kk + (long long)(i - b0) * k + (j - (b0 - k))] = AA[e];
        }
    }
}

// Banded LU without pivoting, one CTA per block (right-looking: the
// multipliers of column j, then the rank-1 update of the trailing band).
__global__ void __launch_bounds__(kSpikeLuThreads)
k_spike_lu(const int *__restrict__ bs, const int *__restrict__ bl, const int *__restrict__ bu,
           const long long *__restrict__ boff, double *band, int *err)
{
    const int q = blockIdx.x, m = bs[q + 1] - bs[q], kl = bl[q], ku = bu[q], ld = kl + ku + 1;
    double *a = band + boff[q];
    auto A = [&](int i, int j) -> double & { return a[(long long)(ku + i - j) + (long long)j * ld]; };
    for (int j = 0; j < m; ++j) {
        const double piv = A(j, j);
        if (threadIdx.x == 0 && piv == 0.0) atomicExch(err, FG_ERR_BREAKDOWN);
        const int ie = min(kl, m - 1 - j), ce = min(ku, m - 1 - j);
        for (int t = threadIdx.x; t < ie; t += blockDim.x) A(j + 1 + t, j) = A(j + 1 + t, j) / piv;
        __syncthreads();
        const int tot = ie * ce;
        for (int t = threadIdx.x; t < tot; t += blockDim.x) {
            const int i = j + 1 + t % ie, c = j + 1 + t / ie;
            A(i, c) = A(i, c) - A(i, j) * A(j, c);
        }
        __syncthreads();
    }
}

// V_q into rows 0..k-1, columns k..2k-1 of S_q (row-major 2k x 2k, zeroed
// before): thread c solves column c with the trailing k x k of L and U.
__global__ void k_spike_vtip(int k, const int *__restrict__ bs, const int *__restrict__ bl,
                             const int *__restrict__ bu, const long long *__restrict__ boff,
                             const double *__restrict__ band, const double *__restrict__ B, double *S)
{
    const int q = blockIdx.x, c = threadIdx.x;
    if (c >= k) return;
    const int m = bs[q + 1] - bs[q], kl = bl[q], ku = bu[q], K2 = 2 * k, r0 = m - k;
    const Band U{band + boff[q], kl + ku + 1, ku};
    double *Sq = S + (long long)q * K2 * K2;
    const double *Bq = B + (long long)q * k * k;
    for (int r = 0; r < k; ++r) {
        double v = Bq[r * k + c];
        for (int s = max(r - kl, 0); s < r; ++s) v = v - U.at(r0 + r, r0 + s) * Sq[s * K2 + k + c];
        Sq[r * K2 + k + c] = v;
    }
    for (int r = k - 1; r >= 0; --r) {
        double v = Sq[r * K2 + k + c];
        for (int s = min(r + ku, k - 1); s > r; --s) v = v - U.at(r0 + r, r0 + s) * Sq[s * K2 + k + c];
        Sq[r * K2 + k + c] = v / U.at(r0 + r, r0 + r);
    }
    Sq[c * K2 + c] = 1.0;
}

// W_q+1 into rows k..2k-1, columns 0..k-1 of S_q: full band solve of the
// m x k right-hand side [C; 0] of block q+1 in the row-major scratch tw.
__global__ void __launch_bounds__(kSpikeThreads)
k_spike_wtip(int k, const int *__restrict__ bs, const int *__restrict__ bl, const int *__restrict__ bu,
             const long long *__restrict__ boff, const double *__restrict__ band, const double *__restrict__ C,
             double *tw, double *S)
{
    const int q = blockIdx.x + 1, m = bs[q + 1] - bs[q], kl = bl[q], ku = bu[q], K2 = 2 * k;
    const Band U{band + boff[q], kl + ku + 1, ku};
    double *w = tw + (long long)bs[q] * k;
    const double *Cq = C + (long long)(q - 1) * k * k;
    const int kk = k * k;
    for (int t = threadIdx.x; t < m * k; t += blockDim.x) w[t] = t < kk ? Cq[t] : 0.0;
    __syncthreads();
    for (int j = 0; j < m - 1; ++j) {
        const int tot = min(kl, m - 1 - j) * k;
        for (int t = threadIdx.x; t < tot; t += blockDim.x) {
            const int i = j + 1 + t / k, c = t % k;
            w[i * k + c] = w[i * k + c] - U.at(i, j) * w[j * k + c];
        }
        __syncthreads();
    }
    for (int j = m - 1; j >= 0; --j) {
        if (threadIdx.x < k) w[j * k + threadIdx.x] = w[j * k + threadIdx.x] / U.at(j, j);
        __syncthreads();
        const int tot = min(ku, j) * k;
        for (int t = threadIdx.x; t < tot; t += blockDim.x) {
            const int i = j - 1 - t / k, c = t % k;
            w[i * k + c] = w[i * k + c] - U.at(i, j) * w[j * k + c];
        }
        __syncthreads();
    }
    double *Sq = S + (long long)(q - 1) * K2 * K2;
    for (int t = threadIdx.x; t < kk; t += blockDim.x) {
        const int r = t / k, c = t % k;
        Sq[(k + r) * K2 + c] = w[t];
    }
    if (threadIdx.x < k) Sq[(k + threadIdx.x) * K2 + k + threadIdx.x] = 1.0;
}

// LU with partial pivoting (first largest |a| wins) of S_q in place.
__global__ void k_spike_reduced(int k, double *S, int *piv, int *err)
{
    const int q = blockIdx.x, N = 2 * k;
    double *a = S + (long long)q * N * N;
    int *pv = piv + q * N;
    __shared__ int p_sh;
    for (int j = 0; j < N; ++j) {
        if (threadIdx.x == 0) {
            int p = j;
            double best = fabs(a[j * N + j]);
            for (int i = j + 1; i < N; ++i)
                if (fabs(a[i * N + j]) > best) { best = fabs(a[i * N + j]); p = i; }
            pv[j] = p;
            p_sh = p;
        }
        __syncthreads();
        const int p = p_sh;
        if (p != j)
            for (int c = threadIdx.x; c < N; c += blockDim.x) {
                double t = a[j * N + c];
                a[j * N + c] = a[p * N + c];
                a[p * N + c] = t;
            }
        __syncthreads();
        const double d = a[j * N + j];
        if (threadIdx.x == 0 && d == 0.0) atomicExch(err, FG_ERR_BREAKDOWN);
        for (int i = j + 1 + threadIdx.x; i < N; i += blockDim.x) a[i * N + j] = a[i * N + j] / d;
        __syncthreads();
        const int rem = N - 1 - j;
        for (int t = threadIdx.x; t < rem * rem; t += blockDim.x) {
            const int i = j + 1 + t % rem, c = j + 1 + t / rem;
            a[i * N + c] = a[i * N + c] - a[i * N + j] * a[j * N + c];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- apply
// In-place forward (unit L) and backward (U) sweep of one block's working
// vector w (m rows), the backward sweep writing x_j to out(j).  Thread t
// updates row j+1+t (forward) or j-1-t (backward) at row j; rows beyond
// the first blockDim of the band are handled by a plain loop.
template <typename Out>
__device__ __forceinline__ void band_solve_cta(const Band &U, int m, int kl, int ku, double *w, Out out)
{
    const int t = threadIdx.x, nt = blockDim.x;
    double cur[kPrefetch], nxt[kPrefetch];
    // forward: L(j+1+t, j) for rows j = 0 .. m-2
    auto lf = [&](int j) -> double { return (j < m - 1 && t < min(kl, m - 1 - j)) ? U.at(j + 1 + t, j) : 0.0; };
#pragma unroll
    for (int d = 0; d < kPrefetch; ++d) cur[d] = lf(d);
    for (int j0 = 0; j0 < m - 1; j0 += kPrefetch) {
#pragma unroll
        for (int d = 0; d < kPrefetch; ++d) nxt[d] = lf(j0 + kPrefetch + d);
#pragma unroll
        for (int d = 0; d < kPrefetch; ++d) {
            const int j = j0 + d;
            if (j >= m - 1) break;
            const double xj = w[j];
            const int ie = min(kl, m - 1 - j);
            if (t < ie) w[j + 1 + t] = w[j + 1 + t] - cur[d] * xj;
            for (int r = t + nt; r < ie; r += nt) w[j + 1 + r] = w[j + 1 + r] - U.at(j + 1 + r, j) * xj;
            __syncthreads();
        }
#pragma unroll
        for (int d = 0; d < kPrefetch; ++d) cur[d] = nxt[d];
    }
    // backward: U(j-1-t, j) and the pivot U(j, j) for rows j = m-1 .. 0
    double pc[kPrefetch], pn[kPrefetch];
    auto ub = [&](int j) -> double { return (j >= 0 && t < min(ku, j)) ? U.at(j - 1 - t, j) : 0.0; };
    auto pb = [&](int j) -> double { return j >= 0 ? U.at(j, j) : 1.0; };
#pragma unroll
    for (int d = 0; d < kPrefetch; ++d) { cur[d] = ub(m - 1 - d); pc[d] = pb(m - 1 - d); }
    for (int j0 = m - 1; j0 >= 0; j0 -= kPrefetch) {
#pragma unroll
        for (int d = 0; d < kPrefetch; ++d) { nxt[d] = ub(j0 - kPrefetch - d); pn[d] = pb(j0 - kPrefetch - d); }
#pragma unroll
        for (int d = 0; d < kPrefetch; ++d) {
            const int j = j0 - d;
            if (j < 0) break;
            const double xj = w[j] / pc[d];
            if (t == 0) out(j, xj);
            const int ie = min(ku, j);
            if (t < ie) w[j - 1 - t] = w[j - 1 - t] - cur[d] * xj;
            for (int r = t + nt; r < ie; r += nt) w[j - 1 - r] = w[j - 1 - r] - U.at(j - 1 - r, j) * xj;
            __syncthreads();
        }
#pragma unroll
        for (int d = 0; d < kPrefetch; ++d) { cur[d] = nxt[d]; pc[d] = pn[d]; }
    }
}

// One CTA per (system, block) item.  phase 0: g = A_q^-1 f (or the final
// output when the system has a single block); phase 1: corrected solve into
// the final output.  f / out: t64 / u64 (sel 0, FP64) or t / w (sel 1, T).
template <typename T>
__global__ void __launch_bounds__(kSpikeThreads)
k_spike_block(const SysDev *__restrict__ sys, const int2 *__restrict__ items, int phase, int sel)
{
    extern __shared__ double spike_sm[];
    const int2 it = items[blockIdx.x];
    const SysDev &D = sys[it.x];
    if (!spike_gate(D, sel)) return;
    const int P = D.sp_P, q = it.y, k = D.sp_k;
    if (phase == 1 && P == 1) return;
    const int b0 = D.sp_bs[q], m = D.sp_bs[q + 1] - b0, kl = D.sp_bl[q], ku = D.sp_bu[q];
    const Band U{D.sp_band + D.sp_boff[q], kl + ku + 1, ku};
    const T *f = sel == 0 ? (const T *)D.t64 : (const T *)D.t;
    T *y = sel == 0 ? (T *)D.u64 : (T *)D.w;
    double *w = m <= D.sp_smem_rows ? spike_sm : D.sp_h + b0;
    for (int r = threadIdx.x; r < m; r += blockDim.x) w[r] = (double)f[b0 + r];
    __syncthreads();
    if (phase == 1) {
        const int K2 = 2 * k;
        const long long kk = (long long)k * k;
        const int r = threadIdx.x;
        if (r < k && q + 1 < P) {           // B_q xT of the interface below
            const double *Bq = D.sp_B + q * kk + (long long)r * k, *x = D.sp_x + (long long)q * K2 + k;
            double s = 0.0;
            for (int c = 0; c < k; ++c) s = s + Bq[c] * x[c];
            w[m - k + r] = w[m - k + r] - s;
        } else if (r >= k && r < K2 && q > 0) {   // C_q xB of the interface above
            const int rr = r - k;
            const double *Cq = D.sp_C + (q - 1) * kk + (long long)rr * k, *x = D.sp_x + (long long)(q - 1) * K2;
            double s = 0.0;
            for (int c = 0; c < k; ++c) s = s + Cq[c] * x[c];
            w[rr] = w[rr] - s;
        }
        __syncthreads();
    }
    if (phase == 1 || P == 1) {
        T *o = y + b0;
        band_solve_cta(U, m, kl, ku, w, [&](int j, double v) { o[j] = (T)v; });
    } else {
        double *o = D.sp_g + b0;
        band_solve_cta(U, m, kl, ku, w, [&](int j, double v) { o[j] = v; });
    }
}

// One CTA per (system, interface) item: x = S_q^-1 [g bottom(q); g top(q+1)].
__global__ void __launch_bounds__(2 * kSpikeMaxK)
k_spike_iface(const SysDev *__restrict__ sys, const int2 *__restrict__ items, int sel)
{
    __shared__ double x[2 * kSpikeMaxK], xo[2 * kSpikeMaxK];
    const int2 it = items[blockIdx.x];
    const SysDev &D = sys[it.x];
    if (!spike_gate(D, sel)) return;
    const int q = it.y, k = D.sp_k, N = 2 * k, b = D.sp_bs[q + 1], t = threadIdx.x;
    const double *a = D.sp_S + (long long)q * N * N;
    const int *pv = D.sp_piv + q * N;
    if (t < k) { x[t] = D.sp_g[b - k + t]; x[k + t] = D.sp_g[b + t]; }
    __syncthreads();
    if (t == 0)
        for (int j = 0; j < N; ++j)
            if (pv[j] != j) { double v = x[j]; x[j] = x[pv[j]]; x[pv[j]] = v; }
    __syncthreads();
    for (int j = 0; j < N - 1; ++j) {
        const double xj = x[j];
        const int i = j + 1 + t;
        if (i < N) x[i] = x[i] - a[i * N + j] * xj;
        __syncthreads();
    }
    for (int j = N - 1; j >= 0; --j) {
        const double xj = x[j] / a[j * N + j];
        if (t == 0) xo[j] = xj;
        if (t < j) x[t] = x[t] - a[t * N + j] * xj;
        __syncthreads();
    }
    if (t < N) D.sp_x[(long long)q * N + t] = xo[t];
}

// ---------------------------------------------------------------- host side
void set_spike_fields(SysDev &D, const fg_system *s)
{
    D.sp_k = s->sp_k;
    D.sp_P = s->sp_ready ? s->sp_P : 0;
    D.sp_smem_rows = kSpikeSmemRows;
    D.sp_bs = s->sp_bs.as<int>();
    D.sp_bl = s->sp_bl.as<int>();
    D.sp_bu = s->sp_bu.as<int>();
    D.sp_boff = s->sp_boff.as<long long>();
    D.sp_band = s->sp_band.as<double>();
    D.sp_B = s->sp_B.as<double>();
    D.sp_C = s->sp_C.as<double>();
    D.sp_S = s->sp_S.as<double>();
    D.sp_piv = s->sp_piv.as<int>();
    D.sp_g = s->sp_g.as<double>();
    D.sp_h = s->sp_h.as<double>();
    D.sp_x = s->sp_x.as<double>();
}

// Block partition, bandwidths and device storage of a system's SPIKE (from
// the CSR pattern, which depends on the mesh only).
static int spike_structure(fg_system *s, cudaStream_t st)
{
    if (s->sp_ready) return FG_OK;
    const int n = s->topo.n, k = s->sp_k;
    std::vector<int> ia(n + 1), ja(std::max(s->csr_nnz, 1));
    FG_CUDA(cudaMemcpyAsync(ia.data(), s->csr_ia.p, sizeof(int) * (size_t)(n + 1), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaMemcpyAsync(ja.data(), s->csr_ja.p, sizeof(int) * (size_t)s->csr_nnz, cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    int P = s->sp_parts;
    if (P > n / (2 * k)) P = n / (2 * k);
    P = std::max(P, 1);
    std::vector<int> bs(P + 1), bl(P, 0), bu(P, 0);
    std::vector<long long> boff(P + 1, 0);
    for (int q = 0; q <= P; ++q) bs[q] = (int)((long long)n * q / P);
    int maxm = 0;
    for (int q = 0; q < P; ++q) {
        for (int i = bs[q]; i < bs[q + 1]; ++i)
            for (int e = ia[i]; e < ia[i + 1]; ++e) {
                const int j = ja[e];
                if (j < bs[q] || j >= bs[q + 1]) continue;
                bl[q] = std::max(bl[q], i - j);
                bu[q] = std::max(bu[q], j - i);
            }
        boff[q + 1] = boff[q] + (long long)(bs[q + 1] - bs[q]) * (bl[q] + bu[q] + 1);
        maxm = std::max(maxm, bs[q + 1] - bs[q]);
    }
    if ((size_t)boff[P] * 8 > kSpikeMaxBandBytes) {
        set_error("SPIKE: the band factors of this system would take " + std::to_string(boff[P] * 8 >> 20) +
                  " MiB (limit 8192 MiB); use more blocks or another preconditioner");
        return FG_ERR_UNSUPPORTED;
    }
    const size_t ni = (size_t)(P - 1), kk = (size_t)k * k;
    std::vector<int2> items;
    for (int q = 0; q < P; ++q) items.push_back(make_int2(0, q));
    for (int q = 0; q + 1 < P; ++q) items.push_back(make_int2(0, q));
    int r;
    if ((r = s->sp_bs.alloc(4 * (P + 1))) || (r = s->sp_bl.alloc(4 * P)) || (r = s->sp_bu.alloc(4 * P)) ||
        (r = s->sp_boff.alloc(8 * (P + 1))) || (r = s->sp_band.alloc(8 * std::max<size_t>(boff[P], 1))) ||
        (r = s->sp_B.alloc(8 * std::max<size_t>(ni * kk, 1))) || (r = s->sp_C.alloc(8 * std::max<size_t>(ni * kk, 1))) ||
        (r = s->sp_S.alloc(8 * std::max<size_t>(ni * 4 * kk, 1))) ||
        (r = s->sp_piv.alloc(4 * std::max<size_t>(ni * 2 * k, 1))) || (r = s->sp_g.alloc(8 * (size_t)s->n_pad)) ||
        (r = s->sp_h.alloc(8 * (size_t)s->n_pad)) || (r = s->sp_x.alloc(8 * std::max<size_t>(ni * 2 * k, 1))) ||
        (r = s->sp_tw.alloc(8 * std::max<size_t>((size_t)n * k, 1))) || (r = s->sp_err.alloc(64)) ||
        (r = s->sp_items.alloc(sizeof(int2) * items.size())) || (r = s->sp_sysdev.alloc(sizeof(SysDev))))
        return r;
    FG_CUDA(cudaMemcpyAsync(s->sp_bs.p, bs.data(), 4 * (P + 1), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(s->sp_bl.p, bl.data(), 4 * P, cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(s->sp_bu.p, bu.data(), 4 * P, cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(s->sp_boff.p, boff.data(), 8 * (P + 1), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(s->sp_items.p, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaStreamSynchronize(st));
    s->sp_P = P;
    s->sp_maxm = maxm;
    s->sp_bs_host = bs;
    s->sp_ready = true;
    return FG_OK;
}

static int spike_check(fg_system *s, cudaStream_t st, const char *what)
{
    int herr = 0;
    FG_CUDA(cudaMemcpyAsync(&herr, s->sp_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    if (herr == FG_ERR_BREAKDOWN) { set_error(std::string("SPIKE: zero pivot in ") + what); return FG_ERR_BREAKDOWN; }
    return FG_OK;
}

// Factorisation of every block and reduced system from the current CSR
// values and, when F_dev is given, F <- M^-1 F (SPIKE_precond_setup.c:308).
int spike_setup_device(fg_system *s, double *F_dev, cudaStream_t st)
{
    int r;
    if (!s->csr_ok) { set_error("SPIKE needs the CSR operator (fg_set_operator(FG_OP_CSR))"); return FG_ERR_STATE; }
    if ((r = csr_refresh(s, st))) return r;
    if (s->topo.n < 1) { set_error("SPIKE: system without free equations"); return FG_ERR_ARG; }
    if ((r = spike_structure(s, st))) return r;
    const int n = s->topo.n, P = s->sp_P, k = s->sp_k;
    const int *bs = s->sp_bs.as<int>(), *bl = s->sp_bl.as<int>(), *bu = s->sp_bu.as<int>();
    const long long *boff = s->sp_boff.as<long long>();
    int *err = s->sp_err.as<int>();
    FG_CUDA(cudaMemsetAsync(s->sp_err.p, 0, s->sp_err.bytes, st));
    FG_CUDA(cudaMemsetAsync(s->sp_band.p, 0, s->sp_band.bytes, st));
    FG_CUDA(cudaMemsetAsync(s->sp_B.p, 0, s->sp_B.bytes, st));
    FG_CUDA(cudaMemsetAsync(s->sp_C.p, 0, s->sp_C.bytes, st));
    FG_CUDA(cudaMemsetAsync(s->sp_S.p, 0, s->sp_S.bytes, st));
    k_spike_fill<<<(n + 255) / 256, 256, 0, st>>>(n, s->csr_ia.as<int>(), s->csr_ja.as<int>(), s->AA64.as<double>(), P,
                                                  k, bs, bl, bu, boff, s->sp_band.as<double>(), s->sp_B.as<double>(),
                                                  s->sp_C.as<double>());
    k_spike_lu<<<P, kSpikeLuThreads, 0, st>>>(bs, bl, bu, boff, s->sp_band.as<double>(), err);
    int nl = 2;
    if (P > 1) {
        k_spike_vtip<<<P - 1, 64, 0, st>>>(k, bs, bl, bu, boff, s->sp_band.as<double>(), s->sp_B.as<double>(),
                                           s->sp_S.as<double>());
        k_spike_wtip<<<P - 1, kSpikeThreads, 0, st>>>(k, bs, bl, bu, boff, s->sp_band.as<double>(),
                                                      s->sp_C.as<double>(), s->sp_tw.as<double>(),
                                                      s->sp_S.as<double>());
        k_spike_reduced<<<P - 1, 128, 0, st>>>(k, s->sp_S.as<double>(), s->sp_piv.as<int>(), err);
        nl += 3;
    }
    FG_CUDA(cudaGetLastError());
    count_launches(nl);
    if ((r = spike_check(s, st, "a block or reduced system"))) return r;
    s->precond = FG_PRECOND_SPIKE;
    if (F_dev) return spike_apply_device(s, F_dev, F_dev, st);
    return FG_OK;
}

template <typename T>
static void launch_apply(const SysDev *sys, const int2 *blocks, int nblocks, const int2 *ifaces, int nifaces, int sel,
                         size_t smem, cudaStream_t st)
{
    k_spike_block<T><<<nblocks, kSpikeThreads, smem, st>>>(sys, blocks, 0, sel);
    if (nifaces > 0) {
        k_spike_iface<<<nifaces, 2 * kSpikeMaxK, 0, st>>>(sys, ifaces, sel);
        k_spike_block<T><<<nblocks, kSpikeThreads, smem, st>>>(sys, blocks, 1, sel);
    }
}

int launch_spike_apply(const SysDev *sys, const int2 *blocks, int nblocks, const int2 *ifaces, int nifaces, int sel,
                       int fp32, cudaStream_t st)
{
    const size_t smem = 8 * (size_t)kSpikeSmemRows;
    if (nblocks < 1) return FG_OK;
    if (fp32) launch_apply<float>(sys, blocks, nblocks, ifaces, nifaces, sel, smem, st);
    else launch_apply<double>(sys, blocks, nblocks, ifaces, nifaces, sel, smem, st);
    FG_CUDA(cudaGetLastError());
    count_launches(nifaces > 0 ? 3 : 1);
    return FG_OK;
}

// z = M^-1 p of one system (FP64, internal numbering, n+1 entries; p may be z).
int spike_apply_device(fg_system *s, const double *p, double *z, cudaStream_t st)
{
    if (s->precond != FG_PRECOND_SPIKE || !s->sp_ready) { set_error("SPIKE not set up"); return FG_ERR_STATE; }
    SysDev D{};
    D.n = s->topo.n;
    D.n_pad = s->n_pad;
    set_spike_fields(D, s);
    D.t64 = const_cast<double *>(p);
    D.u64 = z;
    D.st = nullptr;
    FG_CUDA(cudaMemcpyAsync(s->sp_sysdev.p, &D, sizeof(SysDev), cudaMemcpyHostToDevice, st));
    const int P = s->sp_P;
    const int2 *items = s->sp_items.as<int2>();
    int r = launch_spike_apply(s->sp_sysdev.as<SysDev>(), items, P, items + P, P - 1, 0, 0, st);
    if (r) return r;
    FG_CUDA(cudaMemsetAsync(z + D.n, 0, 8, st));
    FG_CUDA(cudaStreamSynchronize(st));   // D (host) goes out of scope
    return FG_OK;
}

}  // namespace fg
