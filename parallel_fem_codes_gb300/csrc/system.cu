#include <atomic>
// fg_system lifecycle and the public C ABI (include/femgpu.h).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>

#include "system.h"

namespace fg {

static thread_local std::string g_err = "no error";

void set_error(const std::string &msg) { g_err = msg; }

int cuda_fail(cudaError_t e, const char *what)
{
    g_err = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return FG_ERR_NOMEM;
    return FG_ERR_CUDA;
}

// The zero fill runs on the legacy default stream, which the library's
// non-blocking streams are not ordered after, and cudaMemset returns before
// it is done: wait for it, or a copy queued next on another stream could
// land first and be zeroed.
// Device bytes held by the library's allocations, and the optional cap on
// them (fg_set_memory_limit; 0 = none).
static std::atomic<size_t> g_dev_bytes{0}, g_dev_limit{0};

void DevMem::release()
{
    if (p) {
        cudaFree(p);
        g_dev_bytes -= bytes;
    }
    p = nullptr;
    bytes = 0;
}

int DevMem::alloc(size_t b)
{
    release();
    if (b == 0) b = 16;
    const size_t lim = g_dev_limit.load();
    if (lim && g_dev_bytes.load() + b > lim) {
        set_error("device allocation of " + std::to_string(b) + " bytes would pass the library's memory limit (" +
                  std::to_string(lim) + " bytes)");
        return FG_ERR_NOMEM;
    }
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) { p = nullptr; return cuda_fail(e, "cudaMalloc"); }
    bytes = b;
    g_dev_bytes += b;
    e = cudaMemset(p, 0, b);
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemset");
    return FG_OK;
}

// Host -> device copy that has landed when it returns (cudaMemcpy from
// pageable memory may return before its DMA completes, on the legacy
// stream).
int h2d(void *dst, const void *src, size_t bytes)
{
    cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy");
    return FG_OK;
}

int upload_blocks_raw(fg_system *s, const double *raw_dev, cudaStream_t st);
int download_blocks_raw(const fg_system *s, double *raw_dev, cudaStream_t st);

template <class T>
static int upload(DevMem &m, const std::vector<T> &v)
{
    int r = m.alloc(sizeof(T) * std::max<size_t>(v.size(), 1));
    if (r) return r;
    if (!v.empty()) return h2d(m.p, v.data(), sizeof(T) * v.size());
    return FG_OK;
}

// staging vector on the device for host <-> reference-numbered transfers
static int stage(fg_system *s, DevMem &m, size_t bytes)
{
    if (m.bytes >= bytes) return FG_OK;
    return m.alloc(bytes);
}

}  // namespace fg

using namespace fg;

fg_system::~fg_system()
{
    if (stream) cudaStreamDestroy(stream);
    if (h_vec) cudaFreeHost(h_vec);
}

size_t fg_system::bytes() const
{
    const DevMem *all[] = {&lm, &A64, &A32, &dinc_ptr, &dinc, &ninc_ptr, &ninc, &node_dof, &eorder, &perm,
                           &lm16, &blob, &pt_elem, &pt_dof, &pt_col, &pdofs, &pt_inc, &incl, &rhs_f, &rhs_b,
                           &csr_ia, &csr_ja, &csr_diag, &csr_inc_ptr, &csr_inc, &AA64, &AA32, &LU64, &LU32,
                           &dinv64, &dinv32, &lu_ia, &lu_ja, &lu_dg, &lu_map, &AAf64, &ilu_flags, &ilu_ctr, &ilu_tmp, &ilu_ford, &ilu_bord, &ilu_fpass, &ilu_bpass, &sp_bs, &sp_bl, &sp_bu, &sp_boff, &sp_band,
                           &sp_B, &sp_C, &sp_S, &sp_piv, &sp_g, &sp_h, &sp_x, &sp_tw, &sp_err, &sp_items, &sp_sysdev,
                           &diag, &invd64, &invd32, &bd, &ibd64, &ibd32, &gx, &gy, &gup, &gien, &gtype,
                           &ginvp, &Fe, &F64, &gf1, &gf2, &state_u, &state_a, &state_old, &state_u1, &state_u2, &shock_state, &bubble, &norm_part, &ws.V, &ws.w, &ws.t, &ws.x, &ws.b, &ws.ftrue, &ws.r64,
                           &ws.t64, &ws.u64, &ws.small, &ws.part, &ws.counter, &ws.state, &ep_lmi, &ep_coef};
    size_t b = 0;
    for (auto *m : all) b += m->bytes;
    return b;
}

// dot product in the summation order of BLAS_Operations/ddot.c:10-16
static double ddot5(int n, const double *x, const double *y)
{
    long i, m = n - 4;
    double s = 0.0;
    for (i = 0; i < m; i += 5)
        s += x[i] * y[i] + x[i + 1] * y[i + 1] + x[i + 2] * y[i + 2] + x[i + 3] * y[i + 3] + x[i + 4] * y[i + 4];
    for (; i < n; i++) s += x[i] * y[i];
    return s;
}

extern "C" {

const char *fg_last_error(void) { return g_err.c_str(); }

int fg_version(void) { return 10000; }

int fg_set_device(int device)
{
    FG_CUDA(cudaSetDevice(device));
    return FG_OK;
}

int fg_system_create(fg_system **out, int nnodes, int nel, int ndof, const int *ien, const int *type,
                     const int *invp, int neq, int reorder)
{
    if (!out) { set_error("fg_system_create: out is NULL"); return FG_ERR_ARG; }
    *out = nullptr;
    fg_system *s = new (std::nothrow) fg_system();
    if (!s) { set_error("host allocation failed"); return FG_ERR_NOMEM; }
    int r = build_topology(s->topo, nnodes, nel, ndof, ien, type, invp, neq, reorder);
    if (r) { delete s; return r; }
    const Topology &t = s->topo;
    cudaGetDevice(&s->device);
    cudaError_t ce = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) { delete s; return cuda_fail(ce, "cudaStreamCreate"); }
    s->n_pad = ((t.n + 1) + 31) / 32 * 32;
    s->nel_pad = std::max(32, (t.nel + 31) / 32 * 32);
    const int S = t.S;
    std::vector<int> lm_soa((size_t)S * s->nel_pad, t.n);
    for (int p = 0; p < t.nel; ++p) {
        int e = t.eorder[p];
        for (int a = 0; a < S; ++a) lm_soa[(size_t)a * s->nel_pad + p] = t.iperm[t.lm[(size_t)e * S + a]];
    }
    std::vector<int> gien((size_t)3 * s->nel_pad, 0);
    for (int p = 0; p < t.nel; ++p)
        for (int v = 0; v < 3; ++v) gien[(size_t)v * s->nel_pad + p] = t.ien[3 * (size_t)t.eorder[p] + v];
    std::vector<int> perm(t.perm.begin(), t.perm.end());
    std::vector<unsigned short> lm16((size_t)S * s->nel_pad, (unsigned short)0xFFFF);
    for (int p = 0; p < t.nel; ++p)
        for (int a = 0; a < S; ++a) lm16[(size_t)a * s->nel_pad + p] = t.lm16[(size_t)p * S + a];
    if ((r = upload(s->lm16, lm16)) || (r = upload(s->blob, t.blob)) || (r = upload(s->pt_elem, t.pt_elem)) || (r = upload(s->pt_dof, t.pt_dof)) ||
        (r = upload(s->pt_col, t.pt_col)) || (r = upload(s->pdofs, t.dofs)) || (r = upload(s->pt_inc, t.pt_inc)) ||
        (r = upload(s->incl, t.incl))) {
        delete s;
        return r;
    }
    size_t SS = (size_t)S * S * s->nel_pad;
    if ((r = upload(s->lm, lm_soa)) || (r = upload(s->dinc_ptr, t.dinc_ptr)) || (r = upload(s->dinc, t.dinc)) ||
        (r = upload(s->ninc_ptr, t.ninc_ptr)) || (r = upload(s->ninc, t.ninc)) ||
        (r = upload(s->node_dof, t.node_dof)) || (r = upload(s->eorder, t.eorder)) || (r = upload(s->perm, perm)) ||
        (r = upload(s->gien, gien)) || (r = s->A64.alloc(8 * SS)) || (r = s->A32.alloc(4 * SS)) ||
        (r = s->diag.alloc(8 * (size_t)s->n_pad)) || (r = s->invd64.alloc(8 * (size_t)s->n_pad)) ||
        (r = s->invd32.alloc(4 * (size_t)s->n_pad)) || (r = s->pc_err.alloc(16))) {
        delete s;
        return r;
    }
    if (t.ndof > 1) {
        size_t nb = (size_t)t.nnodes * t.ndof * t.ndof;
        if ((r = s->bd.alloc(8 * nb)) || (r = s->ibd64.alloc(8 * nb)) || (r = s->ibd32.alloc(4 * nb))) {
            delete s;
            return r;
        }
    }
    ce = cudaMallocHost(&s->h_vec, sizeof(double) * 2 * (size_t)(t.n + 1));
    if (ce != cudaSuccess) { delete s; return cuda_fail(ce, "cudaMallocHost"); }
    *out = s;
    return FG_OK;
}

int fg_mesh_analyze(int nnodes, int nel, int ndof, const int *ien, const int *type, const int *invp, int neq,
                    int reorder, int *lm, int *Perm, int *invPerm, int *colour, fg_system_info *info)
{
    Topology t;
    int r = build_topology(t, nnodes, nel, ndof, ien, type, invp, neq, reorder);
    if (r) return r;
    if (lm) std::memcpy(lm, t.lm.data(), sizeof(int) * t.lm.size());
    if (Perm) std::memcpy(Perm, t.perm.data(), sizeof(int) * t.perm.size());
    if (invPerm) std::memcpy(invPerm, t.iperm.data(), sizeof(int) * t.iperm.size());
    if (colour) std::memcpy(colour, t.colour.data(), sizeof(int) * t.colour.size());
    if (info) {
        info->n = t.n; info->nel = t.nel; info->ndof = t.ndof; info->S = t.S; info->nnodes = t.nnodes;
        info->ncolours = t.ncol; info->bandwidth_before = t.band_before; info->bandwidth_after = t.band_after;
        info->nnz = t.nnz; info->device_bytes = 0;
    }
    return FG_OK;
}

int fg_system_destroy(fg_system *s)
{
    if (s) {
        cudaStreamSynchronize(s->stream);
        delete s;
    }
    return FG_OK;
}

int fg_system_get_info(const fg_system *s, fg_system_info *info)
{
    if (!s || !info) { set_error("NULL argument"); return FG_ERR_ARG; }
    const Topology &t = s->topo;
    info->n = t.n; info->nel = t.nel; info->ndof = t.ndof; info->S = t.S; info->nnodes = t.nnodes;
    info->ncolours = t.ncol; info->bandwidth_before = t.band_before; info->bandwidth_after = t.band_after;
    info->nnz = t.nnz; info->device_bytes = s->bytes();
    return FG_OK;
}

int fg_system_get_lm(const fg_system *s, int *lm)
{
    if (!s || !lm) { set_error("NULL argument"); return FG_ERR_ARG; }
    std::memcpy(lm, s->topo.lm.data(), sizeof(int) * s->topo.lm.size());
    return FG_OK;
}

int fg_system_get_perm(const fg_system *s, int *Perm, int *invPerm)
{
    if (!s) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (Perm) std::memcpy(Perm, s->topo.perm.data(), sizeof(int) * s->topo.perm.size());
    if (invPerm) std::memcpy(invPerm, s->topo.iperm.data(), sizeof(int) * s->topo.iperm.size());
    return FG_OK;
}

int fg_system_get_colours(const fg_system *s, int *colour)
{
    if (!s || !colour) { set_error("NULL argument"); return FG_ERR_ARG; }
    std::memcpy(colour, s->topo.colour.data(), sizeof(int) * s->topo.colour.size());
    return FG_OK;
}

int fg_set_blocks(fg_system *s, const double *A)
{
    if (!s || (!A && s->topo.nel)) { set_error("NULL argument"); return FG_ERR_ARG; }
    size_t bytes = sizeof(double) * (size_t)s->topo.nel * s->topo.S * s->topo.S;
    int r = stage(s, s->F64, std::max<size_t>(bytes, 8 * (size_t)s->n_pad));
    if (r) return r;
    if (bytes) FG_CUDA(cudaMemcpyAsync(s->F64.p, A, bytes, cudaMemcpyHostToDevice, s->stream));
    if ((r = upload_blocks_raw(s, s->F64.as<double>(), s->stream))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    s->blocks_ok = true;
    s->csr_dirty = true;
    return FG_OK;
}

int fg_get_blocks(const fg_system *s, double *A)
{
    if (!s || !A) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (!s->blocks_ok) { set_error("no element blocks"); return FG_ERR_STATE; }
    fg_system *m = const_cast<fg_system *>(s);
    size_t bytes = sizeof(double) * (size_t)s->topo.nel * s->topo.S * s->topo.S;
    int r = stage(m, m->F64, std::max<size_t>(bytes, 8 * (size_t)s->n_pad));
    if (r) return r;
    if ((r = download_blocks_raw(s, m->F64.as<double>(), s->stream))) return r;
    if (bytes) FG_CUDA(cudaMemcpyAsync(A, m->F64.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

// host vector (reference numbering, n+1) -> device internal numbering
static int vec_in(fg_system *s, const double *h, double *d_int, double *d_tmp)
{
    FG_CUDA(cudaMemcpyAsync(d_tmp, h, 8 * (size_t)(s->topo.n + 1), cudaMemcpyHostToDevice, s->stream));
    return permute_in(s, d_tmp, d_int, s->stream);
}

static int vec_out(fg_system *s, const double *d_int, double *h, double *d_tmp)
{
    int r = permute_out(s, d_int, d_tmp, s->stream);
    if (r) return r;
    FG_CUDA(cudaMemcpyAsync(h, d_tmp, 8 * (size_t)(s->topo.n + 1), cudaMemcpyDeviceToHost, s->stream));
    return FG_OK;
}

// host state (n entries, reference numbering, NULL = 0) -> device internal numbering
static int state_in(fg_system *s, const double *h, double *d)
{
    if (!h) {
        FG_CUDA(cudaMemsetAsync(d, 0, 8 * (size_t)s->n_pad, s->stream));
        return FG_OK;
    }
    std::memcpy(s->h_vec, h, 8 * (size_t)s->topo.n);
    s->h_vec[s->topo.n] = 0.0;
    int r = vec_in(s, s->h_vec, d, s->ws.r64.as<double>());
    if (r) return r;
    // the pinned staging buffer is reused by the next transfer
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

static int ensure_io(fg_system *s)
{
    int r;
    if ((r = stage(s, s->ws.r64, 8 * (size_t)s->n_pad))) return r;
    if ((r = stage(s, s->ws.t64, 8 * (size_t)s->n_pad))) return r;
    if ((r = stage(s, s->ws.u64, 8 * (size_t)s->n_pad))) return r;
    return FG_OK;
}

int fg_matvec(fg_system *s, const double *P, double *Q, int precision)
{
    if (!s || !P || !Q) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = vec_in(s, P, s->ws.t64.as<double>(), s->ws.r64.as<double>()))) return r;
    if ((r = matvec_device(s, s->ws.t64.as<double>(), s->ws.u64.as<double>(), precision, s->stream))) return r;
    if ((r = vec_out(s, s->ws.u64.as<double>(), Q, s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.t64.p, 0, s->ws.t64.bytes, s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

int fg_precond_setup(fg_system *s, int kind, int flags, double *F)
{
    if (!s) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    double *fd = nullptr;
    if (F) {
        if ((r = vec_in(s, F, s->ws.u64.as<double>(), s->ws.r64.as<double>()))) return r;
        fd = s->ws.u64.as<double>();
    }
    if ((r = precond_setup_device(s, kind, flags, fd, s->stream))) return r;
    if (F) {
        if ((r = vec_out(s, fd, F, s->ws.r64.as<double>()))) return r;
    }
    int perr = 0;
    if (kind == FG_PRECOND_BLOCKDIAG)
        FG_CUDA(cudaMemcpyAsync(&perr, s->pc_err.p, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    if (perr) {
        set_error("block-diagonal set-up: a node with a free dof has a singular diagonal block");
        return FG_ERR_BREAKDOWN;
    }
    return FG_OK;
}

int fg_scale(fg_system *s, int kind, double *F)
{
    if (!s) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    double *fd = nullptr;
    if (F) {
        if ((r = vec_in(s, F, s->ws.u64.as<double>(), s->ws.r64.as<double>()))) return r;
        fd = s->ws.u64.as<double>();
    }
    if ((r = scale_device(s, kind, fd, s->stream))) return r;
    if (F && (r = vec_out(s, fd, F, s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

int fg_unscale(fg_system *s, double *X)
{
    if (!s || !X) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = vec_in(s, X, s->ws.u64.as<double>(), s->ws.r64.as<double>()))) return r;
    if ((r = unscale_device(s, s->ws.u64.as<double>(), s->stream))) return r;
    if ((r = vec_out(s, s->ws.u64.as<double>(), X, s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

int fg_precond_apply(fg_system *s, const double *p, double *z)
{
    if (!s || !p || !z) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = vec_in(s, p, s->ws.u64.as<double>(), s->ws.r64.as<double>()))) return r;
    if ((r = precond_apply_device(s, s->ws.u64.as<double>(), s->ws.u64.as<double>(), s->stream))) return r;
    if ((r = vec_out(s, s->ws.u64.as<double>(), z, s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

int fg_precond_apply_right(fg_system *s, const double *p, double *z)
{
    if (!s || !p || !z) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = vec_in(s, p, s->ws.u64.as<double>(), s->ws.r64.as<double>()))) return r;
    if ((r = elem_prec_apply_device(s, true, s->ws.u64.as<double>(), s->ws.u64.as<double>(), s->stream))) return r;
    if ((r = vec_out(s, s->ws.u64.as<double>(), z, s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

int fg_get_diag(const fg_system *s, double *Diag)
{
    if (!s || !Diag) { set_error("NULL argument"); return FG_ERR_ARG; }
    fg_system *m = const_cast<fg_system *>(s);
    int r = ensure_io(m);
    if (r) return r;
    if ((r = vec_out(m, m->diag.as<double>(), Diag, m->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

int fg_set_diag(fg_system *s, const double *Diag)
{
    if (!s || !Diag) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = vec_in(s, Diag, s->diag.as<double>(), s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

static int batch_config(fg_system *const *systems, int count, const fg_solver_opts *o, SolveConfig &cfg);

int fg_solve(fg_system *s, const fg_solver_opts *o, const double *B, double *X, const double *F_true,
             fg_solve_stats *stats)
{
    if (!s || !o || !B || !X) { set_error("NULL argument"); return FG_ERR_ARG; }
    SolveConfig cfg;
    fg_system *one[1] = {s};
    int r0 = batch_config(one, 1, o, cfg);
    if (r0) return r0;
    std::vector<BatchMember> mem{{s, B, F_true, X}};
    fg_solve_stats st{};
    int r = solve_batch(mem, cfg, &st, s->stream);
    if (stats) *stats = st;
    return r;
}

static int batch_config(fg_system *const *systems, int count, const fg_solver_opts *o, SolveConfig &cfg)
{
    if (!systems || count < 1 || !o) { set_error("NULL argument or empty batch"); return FG_ERR_ARG; }
    if (o->precision != FG_PREC_MIXED && o->precision != FG_PREC_FP64 && o->precision != FG_PREC_MIXED16) {
        set_error("precision must be FG_PREC_FP64, FG_PREC_MIXED or FG_PREC_MIXED16"); return FG_ERR_ARG;
    }
    if (o->precision == FG_PREC_MIXED16 && o->kmax > 32) {
        set_error("FG_PREC_MIXED16 needs kmax <= 32 (Gram-corrected Arnoldi)"); return FG_ERR_ARG;
    }
    cfg.kmax = o->kmax; cfg.lmax = o->lmax; cfg.tol = o->tol;
    cfg.mixed = o->precision == FG_PREC_FP64 ? 0 : 1;
    cfg.vhalf = o->precision == FG_PREC_MIXED16 ? 1 : 0;
    cfg.inner_tol = o->inner_tol > 0 ? o->inner_tol : 1e-5;
    for (int i = 0; i < count; ++i) {
        if (!systems[i]) { set_error("NULL system in batch"); return FG_ERR_ARG; }
        if (systems[i]->device != systems[0]->device) { set_error("batch spans devices"); return FG_ERR_ARG; }
        // the batch runs on the first member's stream: finish each member's own work first
        if (i > 0) FG_CUDA(cudaStreamSynchronize(systems[i]->stream));
    }
    cfg.precond = systems[0]->precond;
    return FG_OK;
}

int fg_solve_batch(fg_system *const *systems, int count, const fg_solver_opts *o, const double *const *B,
                   double *const *X, const double *const *F_true, fg_solve_stats *stats)
{
    SolveConfig cfg;
    int r = batch_config(systems, count, o, cfg);
    if (r) return r;
    if (!B || !X) { set_error("NULL B or X"); return FG_ERR_ARG; }
    std::vector<BatchMember> mem;
    for (int i = 0; i < count; ++i) {
        if (!B[i] || !X[i]) { set_error("NULL B[i] or X[i]"); return FG_ERR_ARG; }
        mem.push_back({systems[i], B[i], F_true ? F_true[i] : nullptr, X[i]});
    }
    std::vector<fg_solve_stats> st(count);
    r = solve_batch(mem, cfg, st.data(), systems[0]->stream);
    if (stats) std::memcpy(stats, st.data(), sizeof(fg_solve_stats) * count);
    return r;
}

int fg_solve_resident(fg_system *const *systems, int count, const fg_solver_opts *o, fg_solve_stats *stats)
{
    SolveConfig cfg;
    int r = batch_config(systems, count, o, cfg);
    if (r) return r;
    cfg.device_io = 1;
    std::vector<BatchMember> mem;
    for (int i = 0; i < count; ++i) {
        if (!systems[i]->rhs_ok) { set_error("fg_solve_resident before fg_transport_prepare"); return FG_ERR_STATE; }
        mem.push_back({systems[i], systems[i]->rhs_b.as<double>(), systems[i]->rhs_f.as<double>(), nullptr});
    }
    std::vector<fg_solve_stats> st(count);
    r = solve_batch(mem, cfg, st.data(), systems[0]->stream);
    if (stats) std::memcpy(stats, st.data(), sizeof(fg_solve_stats) * count);
    return r;
}

int fg_get_solution(const fg_system *s, double *X)
{
    if (!s || !X) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (!s->ws.x.p) { set_error("no solution on the device"); return FG_ERR_STATE; }
    fg_system *m = const_cast<fg_system *>(s);
    int r = vec_out(m, m->ws.x.as<double>(), X, m->ws.r64.as<double>());
    if (r) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

long long fg_launch_count(void) { return launch_total(); }

int fg_set_operator(fg_system *s, int op)
{
    if (!s || (op != FG_OP_EBE && op != FG_OP_CSR)) { set_error("invalid operator"); return FG_ERR_ARG; }
    if (op == FG_OP_CSR) {
        int r = csr_setup(s);
        if (r) return r;
        if (s->blocks_ok && (r = csr_refresh(s, s->stream))) return r;
        FG_CUDA(cudaStreamSynchronize(s->stream));
    }
    s->op = op;
    return FG_OK;
}

int fg_set_spike(fg_system *s, int k, int parts)
{
    if (!s) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (k < 1 || k > kSpikeMaxK) { set_error("SPIKE coupling size k must be in [1, 64]"); return FG_ERR_ARG; }
    if (parts < 1 || parts > 65536) { set_error("SPIKE block count must be in [1, 65536]"); return FG_ERR_ARG; }
    if (k != s->sp_k || parts != s->sp_parts) {
        s->sp_k = k;
        s->sp_parts = parts;
        s->sp_ready = false;
        if (s->precond == FG_PRECOND_SPIKE) s->precond = FG_PRECOND_NONE;   // set up again
    }
    return FG_OK;
}

int fg_set_ilu_fill(fg_system *s, int p)
{
    if (!s) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (p < 0 || p > 16) { set_error("ILU fill level must be in [0, 16]"); return FG_ERR_ARG; }
    if (p == s->ilu_p) return FG_OK;
    s->ilu_p = p;
    if (s->precond == FG_PRECOND_ILU0) s->precond = FG_PRECOND_NONE;   // set up again
    return s->csr_ok ? ilu_pattern_setup(s) : FG_OK;
}

int fg_set_ilu_blocks(fg_system *s, int blocks)
{
    if (!s) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (blocks < 1 || blocks > std::max(1, s->topo.n)) {
        set_error("ILU blocks must be in [1, number of equations]"); return FG_ERR_ARG;
    }
    if (blocks == s->ilu_blocks) return FG_OK;
    s->ilu_blocks = blocks;
    if (s->precond == FG_PRECOND_ILU0) s->precond = FG_PRECOND_NONE;   // set up again
    return s->csr_ok ? ilu_pattern_setup(s) : FG_OK;
}

int fg_set_memory_limit(size_t bytes)
{
    g_dev_limit = bytes;
    return FG_OK;
}

size_t fg_memory_in_use(void) { return g_dev_bytes.load(); }

int fg_set_wait_limit(long long polls)
{
    if (polls < 1) { set_error("wait limit must be >= 1 poll"); return FG_ERR_ARG; }
    return set_wait_limit(polls);
}

int fg_get_csr(const fg_system *s, int *nnz, int *IA, int *JA, double *AA)
{
    if (!s) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (!s->csr_ok) { set_error("no CSR operator (fg_set_operator(FG_OP_CSR))"); return FG_ERR_STATE; }
    fg_system *m = const_cast<fg_system *>(s);
    int r = csr_refresh(m, s->stream);
    if (r) return r;
    if (nnz) *nnz = s->csr_nnz;
    if (IA) FG_CUDA(cudaMemcpyAsync(IA, s->csr_ia.p, sizeof(int) * (size_t)(s->topo.n + 1), cudaMemcpyDeviceToHost, s->stream));
    if (JA) FG_CUDA(cudaMemcpyAsync(JA, s->csr_ja.p, sizeof(int) * (size_t)s->csr_nnz, cudaMemcpyDeviceToHost, s->stream));
    if (AA) FG_CUDA(cudaMemcpyAsync(AA, s->AA64.p, sizeof(double) * (size_t)s->csr_nnz, cudaMemcpyDeviceToHost, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

void *fg_system_stream(const fg_system *s) { return s ? (void *)s->stream : nullptr; }

int fg_bench_matvec(fg_system *const *systems, int count, int precision, int reps, double *ms, double *bytes)
{
    if (!systems || count < 1 || !ms || !bytes) { set_error("NULL argument"); return FG_ERR_ARG; }
    std::vector<fg_system *> v(systems, systems + count);
    for (int i = 1; i < count; ++i) FG_CUDA(cudaStreamSynchronize(systems[i]->stream));
    return bench_matvec(v, precision, reps, ms, bytes);
}

int fg_autotune(fg_system *const *systems, int count, const fg_solver_opts *o, int remeasure, fg_tune_choice *out)
{
    if (!systems || count < 1 || !o || !out) { set_error("NULL argument"); return FG_ERR_ARG; }
    SolveConfig cfg;
    int r = batch_config(systems, count, o, cfg);
    if (r) return r;
    std::vector<fg_system *> v(systems, systems + count);
    return autotune(v, cfg, remeasure != 0, false, out);
}

int fg_tune_lookup(fg_system *const *systems, int count, const fg_solver_opts *o, fg_tune_choice *out)
{
    if (!systems || count < 1 || !o || !out) { set_error("NULL argument"); return FG_ERR_ARG; }
    SolveConfig cfg;
    int r = batch_config(systems, count, o, cfg);
    if (r) return r;
    std::vector<fg_system *> v(systems, systems + count);
    return autotune(v, cfg, false, true, out);
}

int fg_tune_set(fg_system *const *systems, int count, const fg_solver_opts *o, const fg_tune_choice *choice)
{
    if (!systems || count < 1 || !o || !choice) { set_error("NULL argument"); return FG_ERR_ARG; }
    SolveConfig cfg;
    int r = batch_config(systems, count, o, cfg);
    if (r) return r;
    std::vector<fg_system *> v(systems, systems + count);
    return tune_set(v, cfg, *choice);
}

void fg_tune_clear(void) { tune_clear(); }

int fg_transport_prepare(fg_system *s, const fg_transport_coeffs *c, const double *u)
{
    if (!s || !c) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = stage(s, s->rhs_f, 8 * (size_t)s->n_pad)) || (r = stage(s, s->rhs_b, 8 * (size_t)s->n_pad))) return r;
    if ((r = state_in(s, u, s->ws.t64.as<double>()))) return r;
    if ((r = transport_assemble_device(s, c, s->ws.t64.as<double>(), s->rhs_f.as<double>(), s->stream))) return r;
    FG_CUDA(cudaMemsetAsync(s->ws.t64.p, 0, 8 * (size_t)s->n_pad, s->stream));
    FG_CUDA(cudaMemcpyAsync(s->rhs_b.p, s->rhs_f.p, 8 * (size_t)s->n_pad, cudaMemcpyDeviceToDevice, s->stream));
    if ((r = precond_setup_device(s, FG_PRECOND_DIAG, 0, s->rhs_b.as<double>(), s->stream))) return r;
    s->rhs_ok = true;
    return FG_OK;
}

int fg_set_geometry(fg_system *s, const double *x, const double *y, const double *upresc)
{
    if (!s || !x || !y || !upresc) { set_error("NULL argument"); return FG_ERR_ARG; }
    const Topology &t = s->topo;
    std::vector<double> vx(x, x + t.nnodes), vy(y, y + t.nnodes), vu(upresc, upresc + t.nnodes);
    std::vector<int> ty(t.nnodes);
    for (int i = 0; i < t.nnodes; ++i) ty[i] = t.type[(size_t)i * t.ndof];
    int r;
    if ((r = upload(s->gx, vx)) || (r = upload(s->gy, vy)) || (r = upload(s->gup, vu)) || (r = upload(s->gtype, ty)) ||
        (r = s->Fe.alloc(8 * (size_t)3 * s->nel_pad)))
        return r;
    s->geometry_ok = true;
    return FG_OK;
}

int fg_transport_assemble(fg_system *s, const fg_transport_coeffs *c, const double *u, double *F)
{
    if (!s || !c) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = state_in(s, u, s->ws.t64.as<double>()))) return r;
    if ((r = transport_assemble_device(s, c, s->ws.t64.as<double>(), s->ws.u64.as<double>(), s->stream))) return r;
    if (F) {
        if ((r = vec_out(s, s->ws.u64.as<double>(), F, s->ws.r64.as<double>()))) return r;
    }
    FG_CUDA(cudaStreamSynchronize(s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.t64.p, 0, s->ws.t64.bytes, s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

int fg_transport_process(fg_system *s, const fg_transport_coeffs *c, const fg_solver_opts *o, double nonlinear_tol,
                         int max_nonlinear, double *U, fg_process_stats *stats)
{
    if (!s || !c || !o || !U) { set_error("NULL argument"); return FG_ERR_ARG; }
    const int n = s->topo.n;
    auto t0 = std::chrono::steady_clock::now();
    std::vector<double> F(n + 1), Fp(n + 1), X(n + 1, 0.0), uold(n);
    std::memset(U, 0, sizeof(double) * n);
    double normdiff = nonlinear_tol + 1, normu = 1.0 / nonlinear_tol;
    int it = 0, gmres = 0, r;
    double last_res = NAN;
    // a fresh run starts from a zero diagonal (Preprocess.c:292 callocs it)
    // and zero YZBeta state (Process.c:16-17)
    FG_CUDA(cudaMemsetAsync(s->diag.p, 0, s->diag.bytes, s->stream));
    if (s->shock_state.p) FG_CUDA(cudaMemsetAsync(s->shock_state.p, 0, s->shock_state.bytes, s->stream));
    // Process.c:37-86
    while (normdiff > nonlinear_tol * normu && it < max_nonlinear) {
        ++it;
        std::memcpy(uold.data(), U, sizeof(double) * n);
        if ((r = fg_transport_assemble(s, c, U, F.data()))) return r;
        Fp = F;
        if ((r = fg_precond_setup(s, FG_PRECOND_DIAG, FG_SETUP_ACCUMULATE, Fp.data()))) return r;
        fg_solve_stats st{};
        r = fg_solve(s, o, Fp.data(), X.data(), F.data(), &st);
        if (r) return r;
        gmres += st.iterations;
        last_res = st.true_rel_residual;
        for (int i = 0; i < n; ++i) {
            U[i] = X[i];
            uold[i] += -1 * U[i];
        }
        normdiff = std::sqrt(ddot5(n, uold.data(), uold.data()));
        normu = std::sqrt(ddot5(n, U, U));
    }
    if (stats) {
        stats->nonlinear_iterations = it;
        stats->gmres_iterations = gmres;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        stats->true_rel_residual = last_res;
        stats->nonlinear_residual = normdiff / normu;
    }
    return FG_OK;
}

int fg_ns_set_geometry(fg_system *s, const double *x, const double *y, const double *upresc, const double *f1,
                       const double *f2)
{
    if (!s || !x || !y || !upresc) { set_error("NULL argument"); return FG_ERR_ARG; }
    const Topology &t = s->topo;
    if (t.ndof != 3) { set_error("Navier-Stokes geometry needs a system with ndof == 3"); return FG_ERR_UNSUPPORTED; }
    const size_t nn = (size_t)t.nnodes;
    std::vector<double> vx(x, x + nn), vy(y, y + nn), vu(upresc, upresc + 3 * nn);
    std::vector<double> v1 = f1 ? std::vector<double>(f1, f1 + nn) : std::vector<double>(nn, 0.0);
    std::vector<double> v2 = f2 ? std::vector<double>(f2, f2 + nn) : std::vector<double>(nn, 0.0);
    int r;
    if ((r = upload(s->gx, vx)) || (r = upload(s->gy, vy)) || (r = upload(s->gup, vu)) || (r = upload(s->gf1, v1)) ||
        (r = upload(s->gf2, v2)) || (r = s->Fe.alloc(8 * (size_t)9 * s->nel_pad)))
        return r;
    s->ns_geometry_ok = true;
    return FG_OK;
}

int fg_ns_assemble(fg_system *s, const fg_ns_coeffs *c, const double *u, double *F)
{
    if (!s || !c) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = state_in(s, u, s->ws.t64.as<double>()))) return r;
    if ((r = ns_assemble_device(s, c->reynolds, c->form, s->ws.t64.as<double>(), s->ws.u64.as<double>(), s->stream))) return r;
    if (F) {
        if ((r = vec_out(s, s->ws.u64.as<double>(), F, s->ws.r64.as<double>()))) return r;
    }
    FG_CUDA(cudaStreamSynchronize(s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.t64.p, 0, s->ws.t64.bytes, s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

// Process.c:6-62 of the Navier-Stokes driver with the state, the residual and
// the increment kept on the device: per iteration one assembly, one
// preconditioner set-up on the residual, one batched-engine solve and one
// update kernel; only the two norms come back to the host.
int fg_ns_process(fg_system *s, const fg_ns_coeffs *c, const fg_solver_opts *o, double nonlinear_tol,
                  int max_nonlinear, double *u, fg_process_stats *stats)
{
    if (!s || !c || !o || !u) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (c->precond < FG_PRECOND_NONE || c->precond > FG_PRECOND_SPIKE) {
        set_error("Navier-Stokes preconditioner must be NONE, DIAG, BLOCKDIAG, ILU0 or SPIKE");
        return FG_ERR_ARG;
    }
    auto t0 = std::chrono::steady_clock::now();
    const int n = s->topo.n;
    fg_system *one[1] = {s};
    SolveConfig cfg;
    int r = batch_config(one, 1, o, cfg);
    if (r) return r;
    cfg.device_io = 1;
    if ((r = ensure_io(s)) || (r = stage(s, s->rhs_f, 8 * (size_t)s->n_pad)) ||
        (r = stage(s, s->rhs_b, 8 * (size_t)s->n_pad)) || (r = stage(s, s->state_u, 8 * (size_t)s->n_pad)) ||
        (r = stage(s, s->norm_part, norm_scratch_bytes())))
        return r;
    FG_CUDA(cudaMemsetAsync(s->state_u.p, 0, s->state_u.bytes, s->stream));
    if ((r = state_in(s, u, s->state_u.as<double>()))) return r;
    // a fresh run starts from a zero diagonal (Preprocess.c:316 callocs it)
    if (c->precond == FG_PRECOND_DIAG) FG_CUDA(cudaMemsetAsync(s->diag.p, 0, s->diag.bytes, s->stream));
    double *part = s->norm_part.as<double>(), *norms = part + (s->norm_part.bytes / 8 - 2);
    double delta = nonlinear_tol + 1.0, last_res = NAN;
    int it = 0, gmres = 0;
    while (delta > nonlinear_tol && it < max_nonlinear) {
        ++it;
        if ((r = ns_assemble_device(s, c->reynolds, c->form, s->state_u.as<double>(), s->rhs_f.as<double>(), s->stream))) return r;
        FG_CUDA(cudaMemcpyAsync(s->rhs_b.p, s->rhs_f.p, 8 * (size_t)s->n_pad, cudaMemcpyDeviceToDevice, s->stream));
        int flags = c->precond == FG_PRECOND_DIAG ? FG_SETUP_ACCUMULATE : 0;
        if ((r = precond_setup_device(s, c->precond, flags, s->rhs_b.as<double>(), s->stream))) return r;
        s->rhs_ok = true;
        cfg.precond = s->precond;
        std::vector<BatchMember> mem{{s, s->rhs_b.as<double>(), s->rhs_f.as<double>(), nullptr}};
        fg_solve_stats st{};
        if ((r = solve_batch(mem, cfg, &st, s->stream))) return r;
        gmres += st.iterations;
        last_res = st.true_rel_residual;
        if ((r = axpy_norms_device(n, 1, s->ws.x.as<double>(), s->state_u.as<double>(), part, norms, s->stream)))
            return r;
        FG_CUDA(cudaMemcpyAsync(s->h_vec, norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        FG_CUDA(cudaStreamSynchronize(s->stream));
        delta = std::sqrt(s->h_vec[0]) / std::sqrt(s->h_vec[1]);
    }
    if ((r = vec_out(s, s->state_u.as<double>(), s->h_vec, s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    std::memcpy(u, s->h_vec, 8 * (size_t)n);
    if (stats) {
        stats->nonlinear_iterations = it;
        stats->gmres_iterations = gmres;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        stats->true_rel_residual = last_res;
        stats->nonlinear_residual = delta;
    }
    return FG_OK;
}

int fg_euler_set_geometry(fg_system *s, const double *x, const double *y, const double *upresc)
{
    if (!s || !x || !y || !upresc) { set_error("NULL argument"); return FG_ERR_ARG; }
    const Topology &t = s->topo;
    if (t.ndof != 4) { set_error("Euler geometry needs a system with ndof == 4"); return FG_ERR_UNSUPPORTED; }
    const size_t nn = (size_t)t.nnodes;
    std::vector<double> vx(x, x + nn), vy(y, y + nn), vu(upresc, upresc + 4 * nn);
    int r;
    if ((r = upload(s->gx, vx)) || (r = upload(s->gy, vy)) || (r = upload(s->gup, vu)) ||
        (r = s->Fe.alloc(8 * (size_t)12 * s->nel_pad)))
        return r;
    s->eu_geometry_ok = true;
    return FG_OK;
}

int fg_euler_assemble(fg_system *s, const fg_euler_coeffs *c, const double *u, const double *du, double *R)
{
    if (!s || !c) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = stage(s, s->state_a, 8 * (size_t)s->n_pad))) return r;
    if ((r = state_in(s, u, s->ws.t64.as<double>())) || (r = state_in(s, du, s->state_a.as<double>()))) return r;
    if ((r = euler_assemble_device(s, c, s->ws.t64.as<double>(), s->state_a.as<double>(), s->ws.u64.as<double>(),
                                   s->stream)))
        return r;
    if (R && (r = vec_out(s, s->ws.u64.as<double>(), R, s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.t64.p, 0, s->ws.t64.bytes, s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

}  // extern "C"

namespace fg {

// A served request with host buffers: element blocks A (reference element
// order) and right-hand side F (NEQ + 1, reference numbering) uploaded,
// Diag set up afresh and applied: the resident right-hand sides of the
// batch engine (rhs_b = M^-1 F, rhs_f = F for the true residual), as
// fg_set_blocks + fg_precond_setup(FG_PRECOND_DIAG, 0, F) leave them.
int prepare_host_request(fg_system *s, const double *A, const double *F)
{
    int r = fg_set_blocks(s, A);
    if (r) return r;
    if ((r = ensure_io(s))) return r;
    if ((r = stage(s, s->rhs_f, 8 * (size_t)s->n_pad)) || (r = stage(s, s->rhs_b, 8 * (size_t)s->n_pad))) return r;
    FG_CUDA(cudaMemsetAsync(s->rhs_f.p, 0, 8 * (size_t)s->n_pad, s->stream));
    if ((r = vec_in(s, F, s->rhs_f.as<double>(), s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaMemcpyAsync(s->rhs_b.p, s->rhs_f.p, 8 * (size_t)s->n_pad, cudaMemcpyDeviceToDevice, s->stream));
    if ((r = precond_setup_device(s, FG_PRECOND_DIAG, 0, s->rhs_b.as<double>(), s->stream))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    s->rhs_ok = true;
    return FG_OK;
}

// the batch engine's solution of a system (internal numbering) to a host
// vector (reference numbering, NEQ + 1), on stream st
int download_solution(fg_system *s, double *X, cudaStream_t st)
{
    int r;
    if ((r = permute_out(s, s->ws.x.as<double>(), s->ws.r64.as<double>(), st))) return r;
    FG_CUDA(cudaMemcpyAsync(X, s->ws.r64.p, 8 * (size_t)(s->topo.n + 1), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    return FG_OK;
}


// The time loops of 00_CommonFiles/Time_Integration with the state (u, a,
// u_old, and u^{n-1}, u^n for BDF2), the residual and the increment kept on
// the device; per correction one assembly (`assemble(alpha_b, dt_b, u, a,
// R)` on the device, internal numbering, with the Alpha_Build / DeltaT_Build
// of the stage), one preconditioner set-up, one batched-engine solve and two
// update kernels.  Only the norms the stop tests read come back to the host.
// Shared by the Euler and the transient transport drivers (the reference
// shares its predictors between them).
//   FG_TIME_PREDICTOR  Predictor_Old.c:53-126
//   FG_TIME_BDF        Predictor_Old_BDF.c:44-150 (BDF1 start, then BDF2; the
//                      Build keeps Alpha_Build = alpha; u_old stays the
//                      initial state for the steady-state test)
//   FG_TIME_TRBDF2     Predictor_New_TRBDF2.c:55-190 without the bubble
//                      unknowns (TR stage alpha 1/2 over lambda dt, BDF2
//                      stage alpha 1/(2 - lambda) over (1 - lambda) dt)
//   FG_TIME_PREDICTOR2 Predictor_New.c:67-159: the Predictor_Old steps plus
//                      the per-element bubble unknowns (predicted after u
//                      and a, corrected from each Da)
//   FG_TIME_PREDICTOR2_BDF    Predictor_New_BDF.c:54-184 (BDF1 with
//                      Alpha_Build 1 and u += dt Da, then BDF2 with 2/3;
//                      u_old = u before each BDF2 prediction), with bubbles
//   FG_TIME_PREDICTOR2_TRBDF2 Predictor_New_TRBDF2.c: FG_TIME_TRBDF2's stages
//                      with bubbles, uB starting from the element centroids
// The bubble hooks: bubble(op, c1, c2, u) at the points where those loops
// act on uB and aB (BubbleOp), corrected(Da, coef = alpha dt) after
// a += Da and u += coef Da.
struct LoopHooks {
    std::function<int(int, double, double, const double *)> bubble;
    std::function<int(const double *, double)> corrected;
};

template <class Assemble>
static int time_loop(fg_system *s, double dt, double alpha, Assemble &&assemble, const fg_solver_opts *o,
                     const fg_time_opts *to, double *u, double *a, fg_time_stats *stats,
                     const CorrectionSolve *solve = nullptr, const LoopHooks *hooks = nullptr)
{
    if (to->precond < FG_PRECOND_NONE || to->precond > FG_PRECOND_SPIKE) {
        set_error("time-loop preconditioner must be NONE, DIAG, BLOCKDIAG, ILU0 or SPIKE");
        return FG_ERR_ARG;
    }
    if (to->max_corrections < 1 || !(dt > 0)) { set_error("max_corrections >= 1 and dt > 0 required"); return FG_ERR_ARG; }
    if (to->scheme < FG_TIME_PREDICTOR || to->scheme > FG_TIME_PREDICTOR2_TRBDF2) {
        set_error("time scheme must be one of FG_TIME_PREDICTOR .. FG_TIME_PREDICTOR2_TRBDF2");
        return FG_ERR_ARG;
    }
    const bool p2 = to->scheme >= FG_TIME_PREDICTOR2;
    if (p2 && !hooks) {
        set_error("the Predictor2 schemes run the DD bubble builds (fg_tt_predictor, fg_euler_predictor)");
        return FG_ERR_UNSUPPORTED;
    }
    auto bubble = [&](int op, double c1, double c2) -> int {
        return p2 && hooks->bubble ? hooks->bubble(op, c1, c2, s->state_u.as<double>()) : FG_OK;
    };
    auto t0 = std::chrono::steady_clock::now();
    const int n = s->topo.n;
    fg_system *one[1] = {s};
    SolveConfig cfg;
    int r = batch_config(one, 1, o, cfg);
    if (r) return r;
    cfg.device_io = 1;
    const size_t vb = 8 * (size_t)s->n_pad, nb = 8 * (size_t)n;
    if ((r = ensure_io(s)) || (r = stage(s, s->rhs_f, vb)) || (r = stage(s, s->rhs_b, vb)) ||
        (r = stage(s, s->state_u, vb)) || (r = stage(s, s->state_a, vb)) || (r = stage(s, s->state_old, vb)) ||
        (r = stage(s, s->norm_part, norm_scratch_bytes())))
        return r;
    if ((to->scheme == FG_TIME_BDF || to->scheme == FG_TIME_PREDICTOR2_BDF) &&
        ((r = stage(s, s->state_u1, vb)) || (r = stage(s, s->state_u2, vb))))
        return r;
    double *du = s->state_u.as<double>(), *da = s->state_a.as<double>(), *dold = s->state_old.as<double>();
    FG_CUDA(cudaMemsetAsync(s->state_u.p, 0, vb, s->stream));
    if ((r = state_in(s, u, du))) return r;
    FG_CUDA(cudaMemsetAsync(da, 0, vb, s->stream));
    if (to->precond == FG_PRECOND_DIAG) FG_CUDA(cudaMemsetAsync(s->diag.p, 0, s->diag.bytes, s->stream));
    double *part = s->norm_part.as<double>(), *norms = part + (s->norm_part.bytes / 8 - 2);
    double t = 0.0, last_res = NAN;
    int steps = 0, corr = 0, gmres = 0;

    // the multicorrection of every scheme: a += Da, u += coef Da until the
    // correction stop test (Criteria.c:25-41)
    auto multicorrect = [&](double ab, double db, double coef) -> int {
        int it = 0, rr;
        bool stop = false;
        do {
            ++it;
            if ((rr = assemble(ab, db, du, da, s->rhs_f.as<double>()))) return rr;
            FG_CUDA(cudaMemcpyAsync(s->rhs_b.p, s->rhs_f.p, vb, cudaMemcpyDeviceToDevice, s->stream));
            int flags = to->setup_flags | (to->precond == FG_PRECOND_DIAG ? FG_SETUP_ACCUMULATE : 0);
            if ((rr = precond_setup_device(s, to->precond, flags, s->rhs_b.as<double>(), s->stream))) return rr;
            s->rhs_ok = true;
            cfg.precond = s->precond;
            fg_solve_stats st{};
            if (solve) {
                if ((rr = (*solve)(s, cfg, &st))) return rr;
            } else {
                std::vector<BatchMember> mem{{s, s->rhs_b.as<double>(), s->rhs_f.as<double>(), nullptr}};
                if ((rr = solve_batch(mem, cfg, &st, s->stream))) return rr;
            }
            gmres += st.iterations;
            last_res = st.true_rel_residual;
            const double *Da = s->ws.x.as<double>();
            if ((rr = axpy_norms_device(n, 1, Da, da, part, norms, s->stream))) return rr;   // a += Da
            if ((rr = axpy_device(n, coef, Da, du, s->stream))) return rr;                 // u += coef Da
            if (hooks && hooks->corrected && (rr = hooks->corrected(Da, coef))) return rr;
            if (to->stop_by_norm) {
                FG_CUDA(cudaMemcpyAsync(s->h_vec, norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
                FG_CUDA(cudaStreamSynchronize(s->stream));
                const double norm_Da = std::sqrt(s->h_vec[0]), norm_a = std::sqrt(s->h_vec[1]);
                stop = norm_Da < to->correction_tol * norm_a || it >= to->max_corrections;
            } else {
                stop = it >= to->max_corrections;
            }
        } while (!stop);
        corr += it;
        return FG_OK;
    };
    // Criteria.c:44-80 with the DeltaT in force, plus the optional step bound
    auto time_stop = [&](double dt_now, bool &stop_time) -> int {
        if (to->steady_state) {
            int rr = diff_norms_device(n, du, dold, part, norms, s->stream);
            if (rr) return rr;
            FG_CUDA(cudaMemcpyAsync(s->h_vec, norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
            FG_CUDA(cudaStreamSynchronize(s->stream));
            const double nd = std::sqrt(s->h_vec[0]), nu = std::sqrt(s->h_vec[1]);
            stop_time = to->time_tol * nu > nd || std::fabs(to->final_time - t) < dt_now;
        } else {
            stop_time = to->final_time - t < 1e-10;
        }
        if (to->max_steps > 0 && steps >= to->max_steps) stop_time = true;
        return FG_OK;
    };
    auto copy = [&](double *dst, const double *src) -> int {
        FG_CUDA(cudaMemcpyAsync(dst, src, nb, cudaMemcpyDeviceToDevice, s->stream));
        return FG_OK;
    };
    bool stop_time = false;
    if (to->scheme == FG_TIME_PREDICTOR || to->scheme == FG_TIME_PREDICTOR2) {
        do {
            ++steps;
            t += dt;
            if ((r = copy(dold, du))) return r;
            if ((r = axpy_device(n, (1.0 - alpha) * dt, da, du, s->stream))) return r;      // prediction
            FG_CUDA(cudaMemsetAsync(da, 0, nb, s->stream));
            if ((r = bubble(kBubblePredict, (1.0 - alpha) * dt, 0.0))) return r;
            if ((r = multicorrect(alpha, dt, alpha * dt)) || (r = time_stop(dt, stop_time))) return r;
        } while (!stop_time);
    } else if (to->scheme == FG_TIME_PREDICTOR2_BDF) {
        const double four_thirds = 4.0 / 3.0, two_thirds = 2.0 / 3.0, one_third = 1.0 / 3.0;
        double *u1 = s->state_u1.as<double>(), *u2 = s->state_u2.as<double>();
        ++steps;                                                                          // BDF1, Alpha_Build 1
        t += dt;
        if ((r = copy(u1, du))) return r;
        FG_CUDA(cudaMemsetAsync(da, 0, nb, s->stream));
        if ((r = bubble(kBubbleBdfStart, 0.0, 0.0))) return r;
        if ((r = multicorrect(1.0, dt, dt)) || (r = copy(u2, du)) || (r = bubble(kBubbleBdfSave2, 0.0, 0.0))) return r;
        do {                                                                              // BDF2, Alpha_Build 2/3
            ++steps;
            t += dt;
            if ((r = copy(dold, du))) return r;
            if ((r = lincomb_device(n, four_thirds, u2, one_third, u1, du, s->stream))) return r;
            FG_CUDA(cudaMemsetAsync(da, 0, nb, s->stream));
            if ((r = bubble(kBubbleBdfCombine, four_thirds, one_third))) return r;
            if ((r = multicorrect(2.0 / 3.0, dt, two_thirds * dt))) return r;
            if ((r = copy(u1, u2)) || (r = copy(u2, du)) || (r = bubble(kBubbleBdfShift, 0.0, 0.0)) ||
                (r = time_stop(dt, stop_time)))
                return r;
        } while (!stop_time);
    } else if (to->scheme == FG_TIME_BDF) {
        const double four_thirds = 4.0 / 3.0, two_thirds = 2.0 / 3.0, one_third = 1.0 / 3.0;
        double *u1 = s->state_u1.as<double>(), *u2 = s->state_u2.as<double>();
        ++steps;                                                                          // BDF1 start
        t += dt;
        if ((r = copy(dold, du)) || (r = copy(u1, du))) return r;
        FG_CUDA(cudaMemsetAsync(da, 0, nb, s->stream));
        if ((r = multicorrect(alpha, dt, alpha * dt)) || (r = copy(u2, du))) return r;
        do {                                                                              // BDF2 steps
            ++steps;
            t += dt;
            if ((r = lincomb_device(n, four_thirds, u2, one_third, u1, du, s->stream))) return r;
            FG_CUDA(cudaMemsetAsync(da, 0, nb, s->stream));
            if ((r = multicorrect(alpha, dt, two_thirds * dt))) return r;
            if ((r = copy(u1, u2)) || (r = copy(u2, du)) || (r = time_stop(dt, stop_time))) return r;
        } while (!stop_time);
    } else {
        const double lambda = 2.0 - std::sqrt(2.0);
        const double A = 1.0 / (lambda * (2.0 - lambda));
        const double B = (1.0 - lambda) * (1.0 - lambda) / (lambda * (2.0 - lambda));
        const double dtTR = lambda * dt, dtBDF2 = (1.0 - lambda) * dt;
        const double aTR = 0.5, aBDF2 = 1.0 / (2.0 - lambda);
        if ((r = bubble(kBubbleTrStart, 0.0, 0.0)) || (r = copy(dold, du))) return r;
        do {
            ++steps;
            t += dtTR;                                                                    // TR stage
            if ((r = axpy_device(n, aTR * dtTR, da, du, s->stream))) return r;
            FG_CUDA(cudaMemsetAsync(da, 0, nb, s->stream));
            if ((r = bubble(kBubblePredict, aTR * dtTR, 0.0))) return r;
            if ((r = multicorrect(aTR, dtTR, aTR * dtTR))) return r;
            t += dtBDF2;                                                                  // BDF2 stage
            if ((r = lincomb_device(n, A, du, B, dold, du, s->stream))) return r;
            FG_CUDA(cudaMemsetAsync(da, 0, nb, s->stream));
            if ((r = bubble(kBubbleTrCombine, A, B))) return r;
            if ((r = multicorrect(aBDF2, dtBDF2, aBDF2 * dtBDF2))) return r;
            if ((r = copy(dold, du)) || (r = bubble(kBubbleTrSave, 0.0, 0.0)) || (r = time_stop(dtBDF2, stop_time)))
                return r;
        } while (!stop_time);
    }
    if ((r = vec_out(s, du, s->h_vec, s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    std::memcpy(u, s->h_vec, 8 * (size_t)n);
    if (a) {
        if ((r = vec_out(s, da, s->h_vec, s->ws.r64.as<double>()))) return r;
        FG_CUDA(cudaStreamSynchronize(s->stream));
        std::memcpy(a, s->h_vec, 8 * (size_t)n);
    }
    if (stats) {
        stats->steps = steps;
        stats->corrections = corr;
        stats->gmres_iterations = gmres;
        stats->t = t;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        stats->true_rel_residual = last_res;
    }
    return FG_OK;
}


int euler_predictor_hooked(fg_system *s, const fg_euler_coeffs *c, const fg_solver_opts *o, const fg_time_opts *to,
                           double *u, double *a, fg_time_stats *stats, const CorrectionSolve *solve)
{
    if (!s || !c || !o || !to || !u) { set_error("NULL argument"); return FG_ERR_ARG; }
    // the DD element state starts at zero with the loop (Predictor_Old.c callocs uB and delta_old)
    if (s->shock_state.p) FG_CUDA(cudaMemsetAsync(s->shock_state.p, 0, s->shock_state.bytes, s->stream));
    if (c->form == FG_EULER_DD && to->scheme == FG_TIME_TRBDF2) {
        set_error("the DD build with TR-BDF2 is Predictor2_TRBDF2 (FG_TIME_PREDICTOR2_TRBDF2); the reference pairs "
                  "the Predictor1 DD build with Predictor_Old_TRBDF2, which is not restated");
        return FG_ERR_UNSUPPORTED;
    }
    if (to->scheme >= FG_TIME_PREDICTOR2) {
        // "Predictor2", "Predictor2_BDF", "Predictor2_TRBDF2" with "DD" (setStabilizationForm.c:47-58),
        // ShockCapture "YZBeta"
        if (c->form != FG_EULER_DD) {
            set_error("the Predictor2 schemes need the DD form (FG_EULER_DD)");
            return FG_ERR_UNSUPPORTED;
        }
        int r = bubble_alloc(s, 4);
        if (r) return r;
        // uB, aB and Delta_YZBetaNMV's state start at zero (Predictor_New.c calloc)
        FG_CUDA(cudaMemsetAsync(s->bubble.p, 0, s->bubble.bytes, s->stream));
        LoopHooks h;
        h.bubble = [&](int op, double c1, double c2, const double *u_dev) {
            return euler_bubble_op_device(s, op, c1, c2, u_dev, s->stream);
        };
        h.corrected = [&](const double *Da, double coef) {
            return euler_bubble_correct_device(s, Da, coef, nullptr, s->stream);
        };
        return time_loop(s, c->dt, c->alpha,
                         [&](double ab, double db, const double *du, const double *da, double *R) {
                             fg_euler_coeffs cc = *c;
                             cc.alpha = ab;
                             cc.dt = db;
                             return euler_mfdd_assemble_device(s, &cc, du, da, R, s->stream);
                         },
                         o, to, u, a, stats, solve, &h);
    }
    return time_loop(s, c->dt, c->alpha,
                     [&](double ab, double db, const double *du, const double *da, double *R) {
                         fg_euler_coeffs cc = *c;
                         cc.alpha = ab;
                         cc.dt = db;
                         return euler_assemble_device(s, &cc, du, da, R, s->stream);
                     },
                     o, to, u, a, stats, solve);
}

}  // namespace fg

extern "C" {

int fg_euler_predictor(fg_system *s, const fg_euler_coeffs *c, const fg_solver_opts *o, const fg_time_opts *to,
                       double *u, double *a, fg_time_stats *stats)
{
    return euler_predictor_hooked(s, c, o, to, u, a, stats, nullptr);
}

int fg_tt_assemble(fg_system *s, const fg_tt_coeffs *c, const double *u, const double *du, double *R)
{
    if (!s || !c) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = stage(s, s->state_a, 8 * (size_t)s->n_pad))) return r;
    if ((r = state_in(s, u, s->ws.t64.as<double>())) || (r = state_in(s, du, s->state_a.as<double>()))) return r;
    if ((r = tt_assemble_device(s, c, s->ws.t64.as<double>(), s->state_a.as<double>(), s->ws.u64.as<double>(),
                                s->stream)))
        return r;
    if (R && (r = vec_out(s, s->ws.u64.as<double>(), R, s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.t64.p, 0, s->ws.t64.bytes, s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

int fg_tt_predictor(fg_system *s, const fg_tt_coeffs *c, const fg_solver_opts *o, const fg_time_opts *to, double *u,
                    double *a, fg_time_stats *stats)
{
    if (!s || !c || !o || !to || !u) { set_error("NULL argument"); return FG_ERR_ARG; }
    // the DD shock-capture state starts at zero with the loop (Predictor_Old.c:30 callocs delta_old)
    if (s->shock_state.p) FG_CUDA(cudaMemsetAsync(s->shock_state.p, 0, s->shock_state.bytes, s->stream));
    if (to->scheme == FG_TIME_PREDICTOR2_BDF || to->scheme == FG_TIME_PREDICTOR2_TRBDF2) {
        set_error("the transient transport driver offers Predictor2 only (its _BDF and _TRBDF2 options are "
                  "commented out, setStabilizationForm.c:55-62)");
        return FG_ERR_UNSUPPORTED;
    }
    if (to->scheme == FG_TIME_PREDICTOR2) {
        // "Predictor2" exists for the DD form only (setStabilizationForm.c:51-54)
        if (c->c.form != FG_TRANSPORT_DD) {
            set_error("FG_TIME_PREDICTOR2 needs the DD form (FG_TRANSPORT_DD)");
            return FG_ERR_UNSUPPORTED;
        }
        int r = bubble_alloc(s, 1);
        if (r) return r;
        // uB and aB start at zero (Predictor_New.c:24,36 calloc them)
        FG_CUDA(cudaMemsetAsync(s->bubble.p, 0, s->bubble.bytes, s->stream));
        LoopHooks h;
        h.bubble = [&](int op, double c1, double, const double *) {
            return op == kBubblePredict ? tt_bubble_predict_device(s, c1, s->stream) : FG_OK;
        };
        h.corrected = [&](const double *Da, double coef) {
            return tt_bubble_correct_device(s, Da, coef, nullptr, s->stream);
        };
        return time_loop(s, c->dt, c->alpha,
                         [&](double ab, double db, const double *du, const double *da, double *R) {
                             fg_tt_coeffs cc = *c;
                             cc.alpha = ab;
                             cc.dt = db;
                             return tt_mfdd_assemble_device(s, &cc, du, da, R, s->stream);
                         },
                         o, to, u, a, stats, nullptr, &h);
    }
    return time_loop(s, c->dt, c->alpha,
                     [&](double ab, double db, const double *du, const double *da, double *R) {
                         fg_tt_coeffs cc = *c;
                         cc.alpha = ab;
                         cc.dt = db;
                         return tt_assemble_device(s, &cc, du, da, R, s->stream);
                     },
                     o, to, u, a, stats);
}

// host (planes values per element, element-major, reference element order;
// NULL = 0) <-> planes k0.. of a plane array (internal element position)
static int planes_in(fg_system *s, double *dev, int k0, int planes, const double *h)
{
    const Topology &t = s->topo;
    std::vector<double> v((size_t)planes * s->nel_pad, 0.0);
    for (int pos = 0; pos < t.nel; ++pos)
        for (int k = 0; k < planes; ++k)
            v[(size_t)k * s->nel_pad + pos] = h ? h[(size_t)planes * t.eorder[pos] + k] : 0.0;
    FG_CUDA(cudaMemcpyAsync(dev + (size_t)k0 * s->nel_pad, v.data(), 8 * v.size(), cudaMemcpyHostToDevice,
                            s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

static int planes_out(fg_system *s, const double *dev, int k0, int planes, double *h)
{
    const Topology &t = s->topo;
    std::vector<double> v((size_t)planes * s->nel_pad);
    FG_CUDA(cudaMemcpyAsync(v.data(), dev + (size_t)k0 * s->nel_pad, 8 * v.size(), cudaMemcpyDeviceToHost,
                            s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    for (int pos = 0; pos < t.nel; ++pos)
        for (int k = 0; k < planes; ++k) h[(size_t)planes * t.eorder[pos] + k] = v[(size_t)k * s->nel_pad + pos];
    return FG_OK;
}

int fg_tt_bubble_assemble(fg_system *s, const fg_tt_coeffs *c, const double *u, const double *du, const double *uB,
                          const double *duB, double *F, double *cond)
{
    if (!s || !c) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = stage(s, s->state_a, 8 * (size_t)s->n_pad)) || (r = bubble_alloc(s, 1))) return r;
    if ((r = state_in(s, u, s->ws.t64.as<double>())) || (r = state_in(s, du, s->state_a.as<double>()))) return r;
    if ((r = planes_in(s, s->bubble.as<double>(), 0, 1, uB)) || (r = planes_in(s, s->bubble.as<double>(), 1, 1, duB)))
        return r;
    if (s->shock_state.p) FG_CUDA(cudaMemsetAsync(s->shock_state.p, 0, s->shock_state.bytes, s->stream));
    if ((r = tt_mfdd_assemble_device(s, c, s->ws.t64.as<double>(), s->state_a.as<double>(), s->ws.u64.as<double>(),
                                     s->stream)))
        return r;
    if (F && (r = vec_out(s, s->ws.u64.as<double>(), F, s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    if (cond && (r = planes_out(s, s->bubble.as<double>(), 2, 5, cond))) return r;
    FG_CUDA(cudaMemsetAsync(s->ws.t64.p, 0, s->ws.t64.bytes, s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

int fg_euler_bubble_assemble(fg_system *s, const fg_euler_coeffs *c, const double *u, const double *du,
                             const double *uB, const double *duB, double *F, double *cond)
{
    if (!s || !c) { set_error("NULL argument"); return FG_ERR_ARG; }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = stage(s, s->state_a, 8 * (size_t)s->n_pad)) || (r = bubble_alloc(s, 4))) return r;
    if ((r = state_in(s, u, s->ws.t64.as<double>())) || (r = state_in(s, du, s->state_a.as<double>()))) return r;
    // fresh shock-capture state, then uB and duB
    FG_CUDA(cudaMemsetAsync(s->bubble.p, 0, s->bubble.bytes, s->stream));
    if ((r = planes_in(s, s->bubble.as<double>(), 0, 4, uB)) || (r = planes_in(s, s->bubble.as<double>(), 4, 4, duB)))
        return r;
    if ((r = euler_mfdd_assemble_device(s, c, s->ws.t64.as<double>(), s->state_a.as<double>(),
                                        s->ws.u64.as<double>(), s->stream)))
        return r;
    if (F && (r = vec_out(s, s->ws.u64.as<double>(), F, s->ws.r64.as<double>()))) return r;
    FG_CUDA(cudaStreamSynchronize(s->stream));
    if (cond && (r = planes_out(s, s->bubble.as<double>(), 8, 53, cond))) return r;
    FG_CUDA(cudaMemsetAsync(s->ws.t64.p, 0, s->ws.t64.bytes, s->stream));
    FG_CUDA(cudaMemsetAsync(s->ws.u64.p, 0, s->ws.u64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return FG_OK;
}

int fg_bubble_dab(fg_system *s, const double *Da, double *DaB)
{
    if (!s || !Da || !DaB) { set_error("NULL argument"); return FG_ERR_ARG; }
    const int nb = s->bubble_nb;
    // the build's element scratch (Fe, 12 planes of nel_pad) receives DaB
    if (!nb || s->Fe.bytes < 8 * (size_t)nb * s->nel_pad) {
        set_error("no Predictor2 build on this system");
        return FG_ERR_STATE;
    }
    int r = ensure_io(s);
    if (r) return r;
    if ((r = vec_in(s, Da, s->ws.t64.as<double>(), s->ws.r64.as<double>()))) return r;
    r = nb == 4 ? euler_bubble_correct_device(s, s->ws.t64.as<double>(), 0.0, s->Fe.as<double>(), s->stream)
                : tt_bubble_correct_device(s, s->ws.t64.as<double>(), 0.0, s->Fe.as<double>(), s->stream);
    if (r) return r;
    r = planes_out(s, s->Fe.as<double>(), 0, nb, DaB);
    FG_CUDA(cudaMemsetAsync(s->ws.t64.p, 0, s->ws.t64.bytes, s->stream));
    FG_CUDA(cudaStreamSynchronize(s->stream));
    return r;
}

int fg_bubble_state(fg_system *s, double *uB, double *aB)
{
    if (!s) { set_error("NULL argument"); return FG_ERR_ARG; }
    const int nb = s->bubble_nb;
    if (!nb) { set_error("no Predictor2 build on this system"); return FG_ERR_STATE; }
    int r = FG_OK;
    if (uB && (r = planes_out(s, s->bubble.as<double>(), 0, nb, uB))) return r;
    if (aB && (r = planes_out(s, s->bubble.as<double>(), nb, nb, aB))) return r;
    return FG_OK;
}

}  // extern "C"
