// Arnoldi step and cycle-end kernels of the batched GMRES engine
// (included by krylov.cu).
//
// Every dof kernel walks parts of kPartMin..n dofs.  Within a part the work
// is split in two shapes so that loads are never serialised behind
// reductions:
//   * update passes are thread-per-dof: w[d] -= sum_j h_j V[j][d] with the
//     j loop unrolled, so a thread keeps several independent basis loads
//     in flight;
//   * dot passes are warp-per-basis-vector: warp w accumulates
//     <V[j], w> for j = w, w+8, ... over the whole part with four
//     independent accumulators per lane and reduces once at the end.
// Part results are combined by the last part of the system in fixed order.

// 16-byte packs along the dof direction: parts start at multiples of the
// pack width and vectors are zero beyond n up to n_pad, so a pack never
// straddles two parts and reads past n see zeros.
template <typename T> struct Pk {
    static constexpr int N = 16 / sizeof(T);
    struct alignas(16) type { T v[N]; };
};
template <typename T> __device__ __forceinline__ typename Pk<T>::type ld_pk(const T *p)
{
    return *reinterpret_cast<const typename Pk<T>::type *>(p);
}
template <typename T> __device__ __forceinline__ void st_pk(T *p, const typename Pk<T>::type &v)
{
    *reinterpret_cast<typename Pk<T>::type *>(p) = v;
}

// dots of V[0..i] with w over a part: warp-per-j, results to out[j]
template <typename T>
__device__ __forceinline__ void part_dots(const SysDev &D, const DChunk &k, int i, const T *__restrict__ w,
                                          double *out)
{
    constexpr int N = Pk<T>::N;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const T *V = (const T *)D.V;
    for (int j = warp; j <= i; j += kThreads / 32) {
        const T *vj = V + (size_t)j * D.n_pad;
        T a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        int q = k.d0 + lane * N;
        for (; q + 3 * 32 * N < k.d1; q += 4 * 32 * N) {
            auto v0 = ld_pk(vj + q), v1 = ld_pk(vj + q + 32 * N), v2 = ld_pk(vj + q + 64 * N), v3 = ld_pk(vj + q + 96 * N);
            auto w0 = ld_pk(w + q), w1 = ld_pk(w + q + 32 * N), w2 = ld_pk(w + q + 64 * N), w3 = ld_pk(w + q + 96 * N);
#pragma unroll
            for (int c = 0; c < N; ++c) {
                a0 += v0.v[c] * w0.v[c];
                a1 += v1.v[c] * w1.v[c];
                a2 += v2.v[c] * w2.v[c];
                a3 += v3.v[c] * w3.v[c];
            }
        }
        for (; q < k.d1; q += 32 * N) {
            auto v0 = ld_pk(vj + q), w0 = ld_pk(w + q);
#pragma unroll
            for (int c = 0; c < N; ++c) a0 += v0.v[c] * w0.v[c];
        }
        double s = (double)((a0 + a1) + (a2 + a3));
        s = warp_sum(s);
        if (lane == 0) out[j] = s;
    }
}

// dots of V[0..i] with w and with v = V[i] over a part, in one sweep of the
// basis: warp w takes j = w, w+8, w+16, w+24 (i < 32) together, so each pack
// of w and v is loaded once per warp whatever the number of its vectors;
// <V[j], w> to out[j], <V[j], v> to out[i + 1 + j]
template <typename T>
__device__ __forceinline__ void part_dots2(const SysDev &D, const DChunk &k, int i, const T *__restrict__ w,
                                           double *out)
{
    constexpr int N = Pk<T>::N;
    constexpr int NW = kThreads / 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const T *V = (const T *)D.V;
    const T *vi = V + (size_t)i * D.n_pad;
    const int nj = warp <= i ? (i - warp) / NW + 1 : 0;   // vectors of this warp (<= 4)
    if (nj == 0) return;
    const T *vj[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) vj[u] = V + (size_t)min(warp + NW * u, i) * D.n_pad;
    T a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = b[u] = (T)0;
    for (int q = k.d0 + lane * N; q < k.d1; q += 32 * N) {
        const auto w0 = ld_pk(w + q), u0 = ld_pk(vi + q);
        typename Pk<T>::type v0[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (u < nj) v0[u] = ld_pk(vj[u] + q);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (u >= nj) break;
#pragma unroll
            for (int c = 0; c < N; ++c) {
                a[u] += v0[u].v[c] * w0.v[c];
                b[u] += v0[u].v[c] * u0.v[c];
            }
        }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        if (u >= nj) break;
        const double sa = warp_sum((double)a[u]), sb = warp_sum((double)b[u]);
        if (lane == 0) {
            out[warp + NW * u] = sa;
            out[i + 1 + warp + NW * u] = sb;
        }
    }
}

// w[d] -= sum_{j<=i} h[j] V[j][d] for the dofs of the part (a pack per
// thread, four basis vectors in flight); returns this thread's sum of the
// new w^2 when want_norm.  Entries past n stay zero.
template <typename T>
__device__ __forceinline__ double part_update(const SysDev &D, const DChunk &k, int i, const T *h, T *w,
                                              bool want_norm)
{
    constexpr int N = Pk<T>::N;
    using P = typename Pk<T>::type;
    const T *V = (const T *)D.V;
    const size_t ld = (size_t)D.n_pad;
    double nrm = 0.0;
    for (int q = k.d0 + threadIdx.x * N; q < k.d1; q += blockDim.x * N) {
        P s0 = ld_pk(w + q), s1, s2, s3;
#pragma unroll
        for (int c = 0; c < N; ++c) s1.v[c] = s2.v[c] = s3.v[c] = (T)0;
        int j = 0;
        for (; j + 3 <= i; j += 4) {
            P v0 = ld_pk(V + j * ld + q), v1 = ld_pk(V + (j + 1) * ld + q);
            P v2 = ld_pk(V + (j + 2) * ld + q), v3 = ld_pk(V + (j + 3) * ld + q);
            const T h0 = h[j], h1 = h[j + 1], h2 = h[j + 2], h3 = h[j + 3];
#pragma unroll
            for (int c = 0; c < N; ++c) {
                s0.v[c] -= h0 * v0.v[c];
                s1.v[c] -= h1 * v1.v[c];
                s2.v[c] -= h2 * v2.v[c];
                s3.v[c] -= h3 * v3.v[c];
            }
        }
        for (; j <= i; ++j) {
            P v0 = ld_pk(V + j * ld + q);
            const T h0 = h[j];
#pragma unroll
            for (int c = 0; c < N; ++c) s0.v[c] -= h0 * v0.v[c];
        }
#pragma unroll
        for (int c = 0; c < N; ++c) {
            T v = (s0.v[c] + s1.v[c]) + (s2.v[c] + s3.v[c]);
            s0.v[c] = v;
            if (want_norm) nrm += (double)(v * v);
        }
        st_pk(w + q, s0);
    }
    return nrm;
}

// pass 1: w = M^-1 t (t cleared), h1_j = <v_j, w>, j = 0..i
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_dots1(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch, const int *__restrict__ nch, int i)
{
    __shared__ double red[kPartStride];
    __shared__ double tot[kPartStride];
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!D.st->in_cycle) continue;
        T *w = (T *)D.w, *t = (T *)D.t;
        const T *invd = sizeof(T) == 8 ? (const T *)D.invd64 : (const T *)D.invd32;
        constexpr int N = Pk<T>::N;
        typename Pk<T>::type zero;
#pragma unroll
        for (int c = 0; c < N; ++c) zero.v[c] = (T)0;
        for (int q = k.d0 + threadIdx.x * N; q < k.d1; q += blockDim.x * N) {
            if (!precond_separate(D.precond)) {
                auto tv = ld_pk(t + q);
                if (D.precond == FG_PRECOND_DIAG) {
                    auto iv = ld_pk(invd + q);
#pragma unroll
                    for (int c = 0; c < N; ++c) tv.v[c] *= iv.v[c];
                }
                st_pk(w + q, tv);
            }
            st_pk(t + q, zero);
        }
        __syncthreads();
        part_dots<T>(D, k, i, w, red);
        __syncthreads();
        for (int j = threadIdx.x; j <= i; j += blockDim.x) D.part[k.part * kPartStride + j] = red[j];
        if (last_part(D, 1)) {
            reduce_parts(D, i + 1, tot);
            for (int j = threadIdx.x; j <= i; j += blockDim.x) D.H[j * D.kmax + i] = tot[j];
        }
    }
}

// Mixed-precision pass 1 (classical Gram-Schmidt with a Gram correction):
// w = M^-1 t (t cleared), s = V^T w and the new column g = V^T v_i of the
// basis' Gram matrix G = V^T V in one sweep.  The last part forms
// c = s + (s - G s): the coefficients of the two classical passes of CGS2
// (h1 = s, h2 = V^T (w - V s) = s - G s) with the second one taken from G
// instead of a second sweep over the basis; c becomes column i of H and
// the update that k_orth2 applies.  Used when kmax <= 32.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_dots1g(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch, const int *__restrict__ nch, int i)
{
    __shared__ double red[kPartStride];
    __shared__ double tot[kPartStride];
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!D.st->in_cycle) continue;
        T *w = (T *)D.w, *t = (T *)D.t;
        const T *invd = sizeof(T) == 8 ? (const T *)D.invd64 : (const T *)D.invd32;
        constexpr int N = Pk<T>::N;
        typename Pk<T>::type zero;
#pragma unroll
        for (int c = 0; c < N; ++c) zero.v[c] = (T)0;
        for (int q = k.d0 + threadIdx.x * N; q < k.d1; q += blockDim.x * N) {
            if (!precond_separate(D.precond)) {
                auto tv = ld_pk(t + q);
                if (D.precond == FG_PRECOND_DIAG) {
                    auto iv = ld_pk(invd + q);
#pragma unroll
                    for (int c = 0; c < N; ++c) tv.v[c] *= iv.v[c];
                }
                st_pk(w + q, tv);
            }
            st_pk(t + q, zero);
        }
        __syncthreads();
        part_dots2<T>(D, k, i, w, red);
        __syncthreads();
        for (int j = threadIdx.x; j < 2 * (i + 1); j += blockDim.x) D.part[k.part * kPartStride + j] = red[j];
        if (last_part(D, 1)) {
            reduce_parts(D, 2 * (i + 1), tot);
            const int km = D.kmax;
            for (int j = threadIdx.x; j <= i; j += blockDim.x) {
                D.G[j * km + i] = tot[i + 1 + j];
                D.G[i * km + j] = tot[i + 1 + j];
            }
            __syncthreads();
            for (int j = threadIdx.x; j <= i; j += blockDim.x) {
                double gs = 0.0;
                for (int l = 0; l <= i; ++l) gs += D.G[j * km + l] * tot[l];
                const double cj = tot[j] + (tot[j] - gs);
                D.H[j * km + i] = cj;
                D.hbuf[j] = cj;
            }
        }
    }
}

// pass 2: w -= sum_j h1_j v_j ; h2_j = <v_j, w>
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_orth1(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch, const int *__restrict__ nch, int i)
{
    __shared__ double red[kPartStride];
    __shared__ double tot[kPartStride];
    __shared__ T hs[kPartStride];
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!D.st->in_cycle) continue;
        T *w = (T *)D.w;
        for (int j = threadIdx.x; j <= i; j += blockDim.x) hs[j] = (T)D.H[j * D.kmax + i];
        __syncthreads();
        part_update<T>(D, k, i, hs, w, false);
        __syncthreads();
        part_dots<T>(D, k, i, w, red);
        __syncthreads();
        for (int j = threadIdx.x; j <= i; j += blockDim.x) D.part[k.part * kPartStride + j] = red[j];
        if (last_part(D, 2)) {
            reduce_parts(D, i + 1, tot);
            for (int j = threadIdx.x; j <= i; j += blockDim.x) {
                D.hbuf[j] = tot[j];
                D.H[j * D.kmax + i] += tot[j];
            }
        }
    }
}

// Back-substitution of the cycle's least-squares problem (pgmres.c:163-171)
// into D.y; one thread.
__device__ __forceinline__ void solve_y(const SysDev &D, int m)
{
    const int km = D.kmax;
    if (m <= 0) return;
    int i = m - 1;
    D.y[i] = D.g[i] / D.H[i * km + i];
    for (int j = i - 1; j >= 0; --j) {
        double s = 0.0;
        for (int q = j + 1; q <= i; ++q) s = s + D.H[j * km + q] * D.y[q];
        D.y[j] = (D.g[j] - s) / D.H[j * km + j];
    }
}

// pass 3: w -= sum_j h2_j v_j ; ||w||; then, in the last part, the Givens
// rotations of column i and the residual estimate (pgmres.c:111-157), and
// at the end of a cycle the solution of the triangular system.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_orth2(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch, const int *__restrict__ nch, int i)
{
    __shared__ double red[kThreads / 32];
    __shared__ double tot[1];
    __shared__ T hs[kPartStride];
    const int total = *nch;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!D.st->in_cycle) continue;
        T *w = (T *)D.w;
        for (int j = threadIdx.x; j <= i; j += blockDim.x) hs[j] = (T)D.hbuf[j];
        __syncthreads();
        double acc = part_update<T>(D, k, i, hs, w, true);
        acc = warp_sum(acc);
        if (lane == 0) red[warp] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0;
            for (int w8 = 0; w8 < kThreads / 32; ++w8) s += red[w8];
            D.part[k.part * kPartStride] = s;
        }
        if (last_part(D, 3)) {
            reduce_parts(D, 1, tot);
            if (threadIdx.x == 0) {
                SysState *st = D.st;
                const int km = D.kmax;
                double *H = D.H, *cs = D.cs, *sn = D.sn, *g = D.g;
                double hn = sqrt(tot[0]);
                st->hn = hn;
                H[(i + 1) * km + i] = hn;
                for (int j = 0; j <= i - 1; ++j) {
                    double h1 = cs[j] * H[j * km + i] + sn[j] * H[(j + 1) * km + i];
                    double h2 = -sn[j] * H[j * km + i] + cs[j] * H[(j + 1) * km + i];
                    H[j * km + i] = h1;
                    H[(j + 1) * km + i] = h2;
                }
                double r = sqrt(H[i * km + i] * H[i * km + i] + H[(i + 1) * km + i] * H[(i + 1) * km + i]);
                cs[i] = H[i * km + i] / r;
                sn[i] = H[(i + 1) * km + i] / r;
                H[i * km + i] = r;
                H[(i + 1) * km + i] = 0.0;
                g[i + 1] = -sn[i] * g[i];
                g[i] = cs[i] * g[i];
                st->rho = fabs(g[i + 1]);
                st->steps = i + 1;
                st->iterations += 1;
                double target = D.mixed ? st->target : st->eps;
                if (!(r > 0.0) || !isfinite(st->rho)) {
                    st->status = FG_ERR_BREAKDOWN;
                    st->in_cycle = 0;
                    if (!(r > 0.0)) st->steps = i;     // column i unusable
                } else if (!(st->rho > target) || i + 1 >= D.kmax - 1 || !(hn > 0.0)) {
                    st->in_cycle = 0;
                }
                if (!st->in_cycle) solve_y(D, st->steps);
            }
        }
    }
}

// v_{i+1} = w * (1 / h_{i+1,i}) (pgmres.c:117)
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_normalize(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch, const int *__restrict__ nch, int i)
{
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!D.st->in_cycle) continue;
        const T sc = (T)(1.0 / D.st->hn);
        const T *w = (const T *)D.w;
        T *v = (T *)D.V + (size_t)(i + 1) * D.n_pad;
        constexpr int N = Pk<T>::N;
        for (int q = k.d0 + threadIdx.x * N; q < k.d1; q += blockDim.x * N) {
            auto p = ld_pk(w + q);
#pragma unroll
            for (int c = 0; c < N; ++c) p.v[c] = q + c < D.n ? sc * p.v[c] : (T)0;
            st_pk(v + q, p);
        }
    }
}

// ---------------------------------------------------------------- cycle end
// x += V y (pgmres.c:173-175) with y from k_orth2; the last part does the
// restart bookkeeping (:177-179).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_update(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch, const int *__restrict__ nch)
{
    __shared__ double y[kPartStride];
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!D.st->live) continue;
        const int m = D.st->steps;
        __syncthreads();
        for (int j = threadIdx.x; j < m; j += blockDim.x) y[j] = D.y[j];
        __syncthreads();
        const T *V = (const T *)D.V;
        const size_t ld = (size_t)D.n_pad;
        for (int d = k.d0 + threadIdx.x; d < k.d1; d += blockDim.x) {
            double xv = D.x[d];
            int j = 0;
            for (; j + 3 < m; j += 4) {
                const double v0 = (double)V[j * ld + d], v1 = (double)V[(j + 1) * ld + d];
                const double v2 = (double)V[(j + 2) * ld + d], v3 = (double)V[(j + 3) * ld + d];
                xv = xv + v0 * y[j];
                xv = xv + v1 * y[j + 1];
                xv = xv + v2 * y[j + 2];
                xv = xv + v3 * y[j + 3];
            }
            for (; j < m; ++j) xv = xv + (double)V[j * ld + d] * y[j];
            D.x[d] = xv;
        }
        if (last_part(D, 4)) {
            if (threadIdx.x == 0) {
                SysState *st = D.st;
                st->cycles += 1;
                st->in_cycle = 0;
                if (st->status == FG_ERR_BREAKDOWN) { st->live = 0; }
                else if (!D.mixed) {
                    if (!(st->rho > st->eps)) { st->converged = 1; st->live = 0; }
                    else if (st->cycles >= D.lmax) { st->status = FG_ERR_NOTCONV; st->live = 0; }
                }
            }
        }
    }
}
