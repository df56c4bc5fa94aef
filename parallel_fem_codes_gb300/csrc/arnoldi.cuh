// Arnoldi step and cycle-end kernels of the batched GMRES engine
// (included by krylov.cu).
//
// Every dof kernel walks parts of kPartMin..kPartMax dofs (the size is
// chosen per batch from its total dofs).  Within a part the work
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

// The basis may be stored in a narrower type TV than the arithmetic type T
// (FP16 under FP32 arithmetic): a basis pack is 16 bytes of TV, G dofs; the
// work vectors are read and written G dofs at a time as G / Pk<T>::N packs.
template <typename TV> struct VPk { static constexpr int G = 16 / sizeof(TV); };

template <typename T, int G> __device__ __forceinline__ void ld_g(const T *p, T (&o)[G])
{
    constexpr int N = Pk<T>::N;
#pragma unroll
    for (int h = 0; h < G / N; ++h) {
        const auto v = ld_pk(p + h * N);
#pragma unroll
        for (int c = 0; c < N; ++c) o[h * N + c] = v.v[c];
    }
}
template <typename T, int G> __device__ __forceinline__ void st_g(T *p, const T (&o)[G])
{
    constexpr int N = Pk<T>::N;
#pragma unroll
    for (int h = 0; h < G / N; ++h) {
        typename Pk<T>::type v;
#pragma unroll
        for (int c = 0; c < N; ++c) v.v[c] = o[h * N + c];
        st_pk(p + h * N, v);
    }
}
// one basis pack as T
template <typename T, typename TV>
__device__ __forceinline__ void ld_v(const TV *p, T (&o)[VPk<TV>::G])
{
    if constexpr (std::is_same<TV, __half>::value) {
        const uint4 r = *reinterpret_cast<const uint4 *>(p);
        const unsigned u[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            __half2 hv;
            memcpy(&hv, &u[h], 4);
            const float2 f = __half22float2(hv);
            o[2 * h] = (T)f.x;
            o[2 * h + 1] = (T)f.y;
        }
    } else {
        ld_g<T, VPk<TV>::G>(reinterpret_cast<const T *>(p), o);
    }
}
template <typename T, typename TV>
__device__ __forceinline__ void st_v(TV *p, const T (&o)[VPk<TV>::G])
{
    if constexpr (std::is_same<TV, __half>::value) {
        unsigned u[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const __half2 hv = __floats2half2_rn((float)o[2 * h], (float)o[2 * h + 1]);
            memcpy(&u[h], &hv, 4);
        }
        *reinterpret_cast<uint4 *>(p) = make_uint4(u[0], u[1], u[2], u[3]);
    } else {
        st_g<T, VPk<TV>::G>(reinterpret_cast<T *>(p), o);
    }
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
// basis.  With nv = i + 1 >= 8 vectors, warp w takes j = w, w+8, w+16, w+24
// (i < 32) together over the whole part, so each pack of w and v is loaded
// once per warp whatever the number of its vectors.  With fewer vectors
// the idle warps split the dofs instead: S = 8 / nv warps per vector, each
// on every S-th pack, their sums added in slice order (deterministic).
// <V[j], w> to out[j], <V[j], v> to out[i + 1 + j].  Every thread of the
// block must call it (it synchronises when the part is sliced).
template <typename T, typename TV = T>
__device__ __forceinline__ void part_dots2(const SysDev &D, const DChunk &k, int i, const T *__restrict__ w,
                                           double *out)
{
    constexpr int G = VPk<TV>::G;
    constexpr int NW = kThreads / 32;
    __shared__ double sl[2 * NW];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nv = i + 1;
    const int S = nv >= NW ? 1 : NW / nv;                  // warps per vector
    const int j0 = S == 1 ? warp : warp / S, sidx = S == 1 ? 0 : warp % S;
    const int nj = S == 1 ? (warp <= i ? (i - warp) / NW + 1 : 0) : (j0 < nv ? 1 : 0);
    const TV *V = (const TV *)D.V;
    const TV *vi = V + (size_t)i * D.n_pad;
    const TV *vj[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) vj[u] = V + (size_t)min(j0 + NW * u, i) * D.n_pad;
    T a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = b[u] = (T)0;
    if (nj > 0) {
#pragma unroll 1
        for (int q = k.d0 + (lane + 32 * sidx) * G; q < k.d1; q += 32 * G * S) {
            T w0[G], u0[G], v0[4][G];
            ld_g<T, G>(w + q, w0);
            ld_v<T, TV>(vi + q, u0);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (u < nj) ld_v<T, TV>(vj[u] + q, v0[u]);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (u >= nj) break;
#pragma unroll
                for (int c = 0; c < G; ++c) {
                    a[u] += v0[u][c] * w0[c];
                    b[u] += v0[u][c] * u0[c];
                }
            }
        }
    }
    if (S == 1) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (u >= nj) break;
            const double sa = warp_sum((double)a[u]), sb = warp_sum((double)b[u]);
            if (lane == 0) {
                out[j0 + NW * u] = sa;
                out[i + 1 + j0 + NW * u] = sb;
            }
        }
        return;
    }
    const double sa = warp_sum((double)a[0]), sb = warp_sum((double)b[0]);
    if (lane == 0 && nj > 0) {
        sl[2 * warp] = sa;
        sl[2 * warp + 1] = sb;
    }
    __syncthreads();
    if (threadIdx.x < nv) {
        const int j = threadIdx.x;
        double ta = sl[2 * (j * S)], tb = sl[2 * (j * S) + 1];
        for (int q = 1; q < S; ++q) {
            ta += sl[2 * (j * S + q)];
            tb += sl[2 * (j * S + q) + 1];
        }
        out[j] = ta;
        out[i + 1 + j] = tb;
    }
}

// w[d] -= sum_{j<=i} h[j] V[j][d] for the dofs of the part (a pack per
// thread, four basis vectors in flight); returns this thread's sum of the
// new w^2 when want_norm.  Entries past n stay zero.
template <typename T, typename TV = T>
__device__ __forceinline__ double part_update(const SysDev &D, const DChunk &k, int i, const T *h, T *w,
                                              bool want_norm)
{
    constexpr int G = VPk<TV>::G;
    const TV *V = (const TV *)D.V;
    const size_t ld = (size_t)D.n_pad;
    double nrm = 0.0;
    for (int q = k.d0 + threadIdx.x * G; q < k.d1; q += blockDim.x * G) {
        T s0[G], s1[G], s2[G], s3[G];
        ld_g<T, G>(w + q, s0);
#pragma unroll
        for (int c = 0; c < G; ++c) s1[c] = s2[c] = s3[c] = (T)0;
        int j = 0;
        for (; j + 3 <= i; j += 4) {
            T v0[G], v1[G], v2[G], v3[G];
            ld_v<T, TV>(V + j * ld + q, v0);
            ld_v<T, TV>(V + (j + 1) * ld + q, v1);
            ld_v<T, TV>(V + (j + 2) * ld + q, v2);
            ld_v<T, TV>(V + (j + 3) * ld + q, v3);
            const T h0 = h[j], h1 = h[j + 1], h2 = h[j + 2], h3 = h[j + 3];
#pragma unroll
            for (int c = 0; c < G; ++c) {
                s0[c] -= h0 * v0[c];
                s1[c] -= h1 * v1[c];
                s2[c] -= h2 * v2[c];
                s3[c] -= h3 * v3[c];
            }
        }
        for (; j <= i; ++j) {
            T v0[G];
            ld_v<T, TV>(V + j * ld + q, v0);
            const T h0 = h[j];
#pragma unroll
            for (int c = 0; c < G; ++c) s0[c] -= h0 * v0[c];
        }
#pragma unroll
        for (int c = 0; c < G; ++c) {
            T v = (s0[c] + s1[c]) + (s2[c] + s3[c]);
            s0[c] = v;
            if (want_norm) nrm += (double)(v * v);
        }
        st_g<T, G>(w + q, s0);
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
template <typename T, typename TV = T>
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
        part_dots2<T, TV>(D, k, i, w, red);
        __syncthreads();
        for (int j = threadIdx.x; j < 2 * (i + 1); j += blockDim.x) D.part[k.part * kPartStride + j] = red[j];
        if (last_part(D, 1)) {
            reduce_parts(D, 2 * (i + 1), tot);
            const int km = D.kmax;
            // the stored basis is sigma V: dots carry 1 / sigma, Gram entries 1 / sigma^2
            const double s1 = D.vsci, s2 = (double)D.vsci * D.vsci;
            for (int j = threadIdx.x; j <= i; j += blockDim.x) {
                D.G[j * km + i] = tot[i + 1 + j] * s2;
                D.G[i * km + j] = tot[i + 1 + j] * s2;
            }
            __syncthreads();
            for (int j = threadIdx.x; j <= i; j += blockDim.x) {
                double gs = 0.0;
                for (int l = 0; l <= i; ++l) gs += D.G[j * km + l] * (tot[l] * s1);
                const double cj = tot[j] * s1 + (tot[j] * s1 - gs);
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

// The last part's step after pass 3 (pgmres.c:111-157): h(i+1,i) = ||w||
// from the summed squares, the earlier rotations applied to column i, the
// new rotation, the residual estimate and the cycle's stop test; at the
// end of a cycle the solution of the triangular system.  One thread.
__device__ __forceinline__ void givens_step(const SysDev &D, int i, double sumsq)
{
    SysState *st = D.st;
    const int km = D.kmax;
    double *H = D.H, *cs = D.cs, *sn = D.sn, *g = D.g;
    double hn = sqrt(sumsq);
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

// pass 3: w -= sum_j h2_j v_j ; ||w||; then, in the last part, the Givens
// step (givens_step).
template <typename T, typename TV = T>
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
        for (int j = threadIdx.x; j <= i; j += blockDim.x) hs[j] = (T)(D.hbuf[j] * D.vsci);
        __syncthreads();
        double acc = part_update<T, TV>(D, k, i, hs, w, true);
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
            if (threadIdx.x == 0) givens_step(D, i, tot[0]);
        }
    }
}

// v_{i+1} = w * (1 / h_{i+1,i}) (pgmres.c:117)
template <typename T, typename TV = T>
__global__ void __launch_bounds__(kThreads)
k_normalize(const SysDev *__restrict__ sys, const DChunk *__restrict__ ch, const int *__restrict__ nch, int i)
{
    const int total = *nch;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const DChunk k = ch[c];
        const SysDev &D = sys[k.sys];
        if (!D.st->in_cycle) continue;
        const T sc = (T)((double)D.vsc / D.st->hn);     // stored as sigma v
        const T *w = (const T *)D.w;
        TV *v = (TV *)D.V + (size_t)(i + 1) * D.n_pad;
        constexpr int G = VPk<TV>::G;
        for (int q = k.d0 + threadIdx.x * G; q < k.d1; q += blockDim.x * G) {
            T p[G];
            ld_g<T, G>(w + q, p);
#pragma unroll
            for (int c = 0; c < G; ++c) p[c] = q + c < D.n ? sc * p[c] : (T)0;
            st_v<T, TV>(v + q, p);
        }
    }
}

// ---------------------------------------------------------------- cycle end
// x += V y (pgmres.c:173-175) with y from k_orth2; the last part does the
// restart bookkeeping (:177-179).
template <typename T, typename TV = T>
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
        for (int j = threadIdx.x; j < m; j += blockDim.x) y[j] = D.y[j] * D.vsci;
        __syncthreads();
        const TV *V = (const TV *)D.V;
        const size_t ld = (size_t)D.n_pad;
        // a 16-byte pack of the basis per thread and four vectors in flight;
        // each dof still adds v_j y_j in j order (x and V are zero-padded to
        // n_pad, so the pack past n adds zeros)
        constexpr int N = VPk<TV>::G;
        for (int q = k.d0 + threadIdx.x * N; q < k.d1; q += blockDim.x * N) {
            double xv[N];
#pragma unroll
            for (int c = 0; c < N; c += 2) {
                const double2 x2 = *reinterpret_cast<const double2 *>(D.x + q + c);
                xv[c] = x2.x;
                xv[c + 1] = x2.y;
            }
            int j = 0;
            for (; j + 3 < m; j += 4) {
                T v0[N], v1[N], v2[N], v3[N];
                ld_v<T, TV>(V + j * ld + q, v0);
                ld_v<T, TV>(V + (j + 1) * ld + q, v1);
                ld_v<T, TV>(V + (j + 2) * ld + q, v2);
                ld_v<T, TV>(V + (j + 3) * ld + q, v3);
                const double y0 = y[j], y1 = y[j + 1], y2 = y[j + 2], y3 = y[j + 3];
#pragma unroll
                for (int c = 0; c < N; ++c) {
                    xv[c] = xv[c] + (double)v0[c] * y0;
                    xv[c] = xv[c] + (double)v1[c] * y1;
                    xv[c] = xv[c] + (double)v2[c] * y2;
                    xv[c] = xv[c] + (double)v3[c] * y3;
                }
            }
            for (; j < m; ++j) {
                T v0[N];
                ld_v<T, TV>(V + j * ld + q, v0);
                const double y0 = y[j];
#pragma unroll
                for (int c = 0; c < N; ++c) xv[c] = xv[c] + (double)v0[c] * y0;
            }
#pragma unroll
            for (int c = 0; c < N; c += 2)
                *reinterpret_cast<double2 *>(D.x + q + c) = make_double2(xv[c], xv[c + 1]);
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
