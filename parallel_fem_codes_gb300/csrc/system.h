// The fg_system object and the batched Krylov engine (internal).
#pragma once
#include <functional>
#include <memory>
#include <vector>

#include "fg_internal.h"
#include "../../include/femgpu.h"

namespace fg {

// Device allocation owned by a system or a batch.
struct DevMem {
    void *p = nullptr;
    size_t bytes = 0;
    DevMem() = default;
    DevMem(const DevMem &) = delete;
    DevMem &operator=(const DevMem &) = delete;
    ~DevMem() { release(); }
    int alloc(size_t b);     // zero-filled (the fill has completed on return)
    void release();
    template <class T> T *as() const { return static_cast<T *>(p); }
};

// Solver workspace of one system (kept resident between solves).
struct Workspace {
    int kmax = 0, mixed = -1;
    DevMem V, w, t, x, b, ftrue, r64, t64, u64, small, part, counter, state;
};

}  // namespace fg

struct fg_system {
    fg::Topology topo;
    int device = 0;
    cudaStream_t stream = nullptr;
    int n_pad = 0, nel_pad = 0;
    // connectivity and blocks, internal numbering / element order, SoA
    fg::DevMem lm, A64, A32;
    fg::DevMem dinc_ptr, dinc, ninc_ptr, ninc, node_dof, eorder, perm;
    fg::DevMem lm16, pt_elem, pt_dof, pt_col, pdofs, pt_inc, incl;   // matvec patch layout
    fg::DevMem blob;                   // 3x3: per-patch index blobs of the bulk-copy matvec
    // preconditioners
    fg::DevMem diag, invd64, invd32, bd, ibd64, ibd32;
    fg::DevMem pc_err;                 // set-up status word (singular nodal block)
    int precond = FG_PRECOND_NONE;
    bool blocks_ok = false;
    // geometry (device assembly)
    fg::DevMem gx, gy, gup, gien, gtype, ginvp, Fe, F64;
    bool geometry_ok = false;
    // Navier-Stokes / Euler: nodal body force (gup holds ndof values per node),
    // state of the nonlinear and time loops (internal numbering) and norm scratch
    fg::DevMem gf1, gf2, state_u, state_a, state_old, norm_part;
    fg::DevMem state_u1, state_u2;     // u^{n-1}, u^n of the BDF2 steps
    fg::DevMem shock_state;            // YZBeta Re_old, delta_old [2 * nel_pad]
    // Predictor2 bubble planes of nel_pad doubles, nb = 1 (transient
    // transport: uB, aB, invN2, R2, M2[3]) or 4 (Euler: uB[4], aB[4], invN2,
    // R2[4], M2[4][12], Delta_YZBetaNMV's state, uB_old / uB1 [4], uB2 [4])
    fg::DevMem bubble;
    int bubble_nb = 0;
    bool ns_geometry_ok = false, eu_geometry_ok = false;
    // resident right-hand side (internal numbering): F and M^-1 F
    fg::DevMem rhs_f, rhs_b;
    bool rhs_ok = false;
    // assembled CSR operator and ILU(0)
    int op = FG_OP_EBE;
    bool csr_ok = false, csr_dirty = true;
    int csr_nnz = 0, csr_w = 4;
    // ILU(0) schedule: rows in level order (forward / backward) and their
    // passes; ilu_g lanes per row
    int ilu_g = 32, ilu_nfpass = 0, ilu_nbpass = 0;
    fg::DevMem ilu_ford, ilu_bord, ilu_fpass, ilu_bpass;
    // ILU(p) factor pattern (per row: L ascending, diagonal, U in the order
    // the symbolic pass admits it) and the slot of every CSR entry in it
    int ilu_p = 0, lu_nnz = 0;
    int ilu_blocks = 1;                // block-Jacobi ILU over this many row blocks (1: global)
    int ilu_maxrow = 1;                // longest row of the factor pattern
    fg::DevMem ep_lmi, ep_coef;        // element preconditioners: dofs and coefficients per element
    int scale_kind = 0;                // last fg_scale kind (fg_unscale follows it)
    fg::DevMem lu_ia, lu_ja, lu_dg, lu_map, AAf64;
    fg::DevMem csr_ia, csr_ja, csr_diag, csr_inc_ptr, csr_inc, AA64, AA32, LU64, LU32, dinv64, dinv32, ilu_flags,
        ilu_ctr, ilu_tmp;   // ilu_tmp: output of the forward substitution (n_pad doubles)
    // truncated SPIKE over row blocks of the CSR operator
    int sp_k = 16, sp_parts = 16, sp_P = 0, sp_maxm = 0;
    bool sp_ready = false;
    std::vector<int> sp_bs_host;
    fg::DevMem sp_bs, sp_bl, sp_bu, sp_boff, sp_band, sp_B, sp_C, sp_S, sp_piv, sp_g, sp_h, sp_x, sp_tw, sp_err,
        sp_items, sp_sysdev;
    // host staging (pinned)
    double *h_vec = nullptr;   // 2*(n+1) doubles
    fg::Workspace ws;
    size_t bytes() const;
    ~fg_system();
};

namespace fg {

// Host -> device copy, complete on return.
int h2d(void *dst, const void *src, size_t bytes);

// CSR / ILU(0) (ilu.cu)
int csr_setup(fg_system *s);
int ilu_pattern_setup(fg_system *s);   // ILU(p) factor pattern and schedules (after csr_setup)
int csr_refresh(fg_system *s, cudaStream_t st);
int ilu0_setup_device(fg_system *s, double *F_dev, cudaStream_t st);
int ilu0_apply_device(fg_system *s, const double *p, double *z, cudaStream_t st);
int set_wait_limit(long long polls);   // bounded dependency waits of the ILU kernels
int launch_ilu_pending(const SysDev *sys, const DChunk *ch, const int *nch, int n_dch, int sel, int fp32,
                       cudaStream_t st);
int launch_ilu_solve(const SysDev *sys, const int2 *items, int nitems, int *counter, int *err, int sel, int backward,
                     int fp32, int lanes, cudaStream_t st);
int ilu_ws_rows(const fg_system *s);
// element preconditioner sweeps over a batch (setup.cu): kind 1 LU, 2 SGS
// forward (left), 3 SGS backward (right); sel 0: t64 -> u64 (left) or
// x -> r64 (right), gate live; 1: t -> w (left) or V[step] -> r64 (right),
// gate in cycle; 2 (right): x in place, every member
int launch_elem_prec(const SysDev *sys, int nsys, int kind, int sel, int step, cudaStream_t st);
int elem_prec_apply_device(fg_system *s, bool right, const double *p, double *z, cudaStream_t st);   // rows of the largest block-Jacobi block (warp-per-block path), or 0
int launch_ilu_ws(const SysDev *sys, const int2 *items, int nitems, int sel, int backward, int fp32, int lanes,
                  int rows, int ecap, cudaStream_t st);

// Truncated SPIKE (spike.cu)
constexpr int kSpikeMaxK = 64;                 // largest coupling size
constexpr int kSpikeSmemRows = 6144;           // blocks up to this many rows solve in shared memory
int spike_setup_device(fg_system *s, double *F_dev, cudaStream_t st);
int spike_apply_device(fg_system *s, const double *p, double *z, cudaStream_t st);
// One engine apply over a batch: blocks / interfaces are (system, index)
// items; sel 0 (t64 -> u64, FP64, gate live) or 1 (t -> w, T, gate in_cycle).
int launch_spike_apply(const SysDev *sys, const int2 *blocks, int nblocks, const int2 *ifaces, int nifaces, int sel,
                       int fp32, cudaStream_t st);
void set_spike_fields(SysDev &D, const fg_system *s);

// Patch-layout pointers of a system's descriptor (matvec).
inline void set_patch_fields(SysDev &D, const fg_system *s)
{
    D.op = s->op;
    D.csr_w = s->csr_w;
    D.csr_ia = s->csr_ia.as<int>();
    D.csr_ja = s->csr_ja.as<int>();
    D.csr_diag = s->csr_diag.as<int>();
    D.AA64 = s->AA64.as<double>();
    D.AA32 = s->AA32.as<float>();
    D.LU64 = s->LU64.as<double>();
    D.LU32 = s->LU32.as<float>();
    D.lu_ia = s->lu_ia.as<int>();
    D.lu_ja = s->lu_ja.as<int>();
    D.lu_dg = s->lu_dg.as<int>();
    D.dinv64 = s->dinv64.as<double>();
    D.dinv32 = s->dinv32.as<float>();
    D.ilu_tmp = s->ilu_tmp.p;
    D.ilu_ford = s->ilu_ford.as<int>();
    D.ilu_bord = s->ilu_bord.as<int>();
    D.ilu_fpass = s->ilu_fpass.as<int2>();
    D.ilu_bpass = s->ilu_bpass.as<int2>();
    D.ilu_P = std::max(1, std::min(s->ilu_blocks, s->topo.n));
    D.ep_lmi = s->ep_lmi.as<int>();
    D.ep_coef = s->ep_coef.as<double>();
    set_spike_fields(D, s);
    D.lm16 = s->lm16.as<unsigned short>();
    D.pt_elem = s->pt_elem.as<int>();
    D.pt_dof = s->pt_dof.as<int>();
    D.pt_col = s->pt_col.as<unsigned short>();
    D.dofs = s->pdofs.as<int>();
    D.pt_inc = s->pt_inc.as<int>();
    D.incl = s->incl.as<unsigned short>();
    D.blob = s->blob.as<unsigned char>();
    D.maxdof = std::max(1, s->topo.maxdof);
}

// A set of systems solved together: one graph launch per restart cycle
// advances every live member; members stop independently.
struct BatchMember {
    fg_system *s;
    const double *B;       // host or device, see solve_batch
    const double *Ftrue;
    double *X;
};

struct SolveConfig {
    int kmax = 30, lmax = 1000;
    double tol = 1e-10, inner_tol = 1e-5;
    int mixed = 0;         // 0: FP64 reference method; 1: FP32 Arnoldi in FP64 refinement
    int vhalf = 0;         // mixed with the Krylov basis stored in FP16 (Gram path only)
    int precond = FG_PRECOND_DIAG;
    int device_io = 0;     // B/X/Ftrue are device pointers in internal numbering
    int use_graph = 1;
};

struct Plan;

// A steppable batch: members are staged and committed between restart
// cycles, each cycle advances every live member, finished members are
// removed.  solve_batch and the request server are built on it.
class BatchRun {
public:
    BatchRun(const SolveConfig &cfg, cudaStream_t st);
    ~BatchRun();
    int stage(const BatchMember &m);
    int commit();
    int cycle(bool use_graph, std::vector<int> &live);
    int finish(const std::vector<int> &idx, std::vector<SysState> &out);
    void remove(std::vector<int> idx);
    size_t size() const { return mem.size(); }
    const BatchMember &member(size_t i) const { return mem[i]; }
    SolveConfig cfg;
    cudaStream_t st;
private:
    std::vector<BatchMember> mem;
    std::vector<SysDev> hs;
    std::unique_ptr<Plan> P;
    int pending = 0;
    cudaGraphExec_t exec = nullptr;
    int graph_nodes = 0;
    int *h_live = nullptr;
    size_t live_cap = 0;
};

int validate_member(fg_system *s, const SolveConfig &cfg);
size_t workspace_bytes(const fg_system *s, int kmax, int mixed);
void fill_stats(const SysState &s, double secs, fg_solve_stats &o);

// Solve every member; stats[i] receives the result of member i.
int solve_batch(std::vector<BatchMember> &members, const SolveConfig &cfg,
                fg_solve_stats *stats, cudaStream_t stream);

int bench_matvec(std::vector<fg_system *> &systems, int precision, int reps, double *ms, double *bytes);
int autotune(std::vector<fg_system *> &sys, const SolveConfig &cfg, bool remeasure, bool lookup_only,
             fg_tune_choice *out);
void tune_clear();
int tune_set(std::vector<fg_system *> &sys, const SolveConfig &cfg, const fg_tune_choice &c);
int launch_matvec_colours(int S, int precision, const SysDev *sys_dev, const EChunk *ch_dev, const int *counts_dev,
                          const int *off_host, int ncol, int maxdof, const double *x, double *y, cudaStream_t st);

// Matvec on device vectors in internal numbering (precision 64 or 32).
int matvec_device(fg_system *s, const double *x, double *y, int precision, cudaStream_t st);

// Navier-Stokes (ns.cu), residual gather and the loops' BLAS-1 steps
int ns_assemble_device(fg_system *s, double reynolds, int form, const double *u_dev, double *F_dev, cudaStream_t st);
int gather_residual(fg_system *s, const double *Fe, double *F, cudaStream_t st);
// y += a x, out[0] = sum x^2, out[1] = sum y^2 (after the update)
int axpy_norms_device(int n, double a, const double *x, double *y, double *part, double *out, cudaStream_t st);
// out[0] = sum (u - v)^2, out[1] = sum u^2
int diff_norms_device(int n, const double *u, const double *v, double *part, double *out, cudaStream_t st);
int axpy_device(int n, double a, const double *x, double *y, cudaStream_t st);
int lincomb_device(int n, double c1, const double *x1, double c2, const double *x2, double *y, cudaStream_t st);
size_t norm_scratch_bytes();
// Transient transport (setup.cu)
int tt_assemble_device(fg_system *s, const fg_tt_coeffs *c, const double *u_dev, const double *du_dev, double *R_dev,
                       cudaStream_t st);
// TimeIntegration "Predictor2" with the DD form: Build_M_F_DD at (u, du) and
// the bubble planes (uB, aB as duB); F_dev the load.  The correction
// (calculate_DaB from Da, internal numbering) updates aB and uB with coef =
// alpha dt, or writes DaB into DaB_dev (element positions) when given.
constexpr int kBubblePlanes = 7, kBubblePlanesEuler = 70;
// the bubble steps of the Predictor2 loops (Predictor_New*.c)
enum BubbleOp {
    kBubblePredict = 0,     // uB += c1 aB, aB = 0
    kBubbleTrStart,         // uB = element centroids of u (uB_InitialSolution)
    kBubbleTrCombine,       // uB = c1 uB - c2 uB_old, aB = 0
    kBubbleTrSave,          // uB_old = uB
    kBubbleBdfStart,        // uB1 = uB, aB = 0
    kBubbleBdfSave2,        // uB2 = uB
    kBubbleBdfCombine,      // uB = c1 uB2 - c2 uB1, aB = 0
    kBubbleBdfShift         // uB1 = uB2, uB2 = uB
};
int bubble_alloc(fg_system *s, int nb);
int tt_mfdd_assemble_device(fg_system *s, const fg_tt_coeffs *c, const double *u_dev, const double *du_dev,
                            double *F_dev, cudaStream_t st);
int tt_bubble_correct_device(fg_system *s, const double *Da_dev, double coef, double *DaB_dev, cudaStream_t st);
int tt_bubble_predict_device(fg_system *s, double coef, cudaStream_t st);
// Euler "Predictor2" (euler.cu): Build_M_F_DD_Transiente with YZBeta, and
// the same correction / prediction of its four bubble unknowns per element
int euler_mfdd_assemble_device(fg_system *s, const fg_euler_coeffs *c, const double *u_dev, const double *du_dev,
                               double *F_dev, cudaStream_t st);
int euler_bubble_correct_device(fg_system *s, const double *Da_dev, double coef, double *DaB_dev, cudaStream_t st);
int euler_bubble_op_device(fg_system *s, int op, double c1, double c2, const double *u_dev, cudaStream_t st);
// The correction solve of a time loop: the system's resident right-hand
// side (B = rhs_b, Ftrue = rhs_f, device, internal numbering) solved into
// ws.x with cfg; stats receives the result.  The time loops solve alone by
// default; the request server passes one that joins its Euler batch.
using CorrectionSolve = std::function<int(fg_system *, const SolveConfig &, fg_solve_stats *)>;
int euler_predictor_hooked(fg_system *s, const fg_euler_coeffs *c, const fg_solver_opts *o, const fg_time_opts *to,
                           double *u, double *a, fg_time_stats *stats, const CorrectionSolve *solve);
// Device bytes a request will hold once admitted: the system's arrays plus
// the Krylov workspace and, for time loops, the loop's state vectors.
size_t request_bytes(const fg_system *s, int kmax, int mixed, bool time_loop);
// Euler (euler.cu)
int euler_assemble_device(fg_system *s, const fg_euler_coeffs *c, const double *u_dev, const double *du_dev,
                          double *R_dev, cudaStream_t st);

// Set-up kernels (setup.cu)
int precond_setup_device(fg_system *s, int kind, int flags, double *F_dev, cudaStream_t st);
int precond_apply_device(fg_system *s, const double *p, double *z, cudaStream_t st);
int convert_blocks(fg_system *s, cudaStream_t st);
// Left / left-right diagonal scaling of the blocks and F (internal numbering)
int scale_device(fg_system *s, int kind, double *F_dev, cudaStream_t st);
int unscale_device(fg_system *s, double *x_dev, cudaStream_t st);
int transport_assemble_device(fg_system *s, const fg_transport_coeffs *c,
                              const double *u_dev, double *F_dev, cudaStream_t st);
// Gathers / scatters between reference and internal numbering (n+1 vectors)
int permute_in(fg_system *s, const double *ref_dev, double *int_dev, cudaStream_t st);
int permute_out(fg_system *s, const double *int_dev, double *ref_dev, cudaStream_t st);
int prepare_host_request(fg_system *s, const double *A, const double *F);   // server: host blocks and F
int download_solution(fg_system *s, double *X, cudaStream_t st);             // engine x -> host X

int sm_count();

// launch accounting (fg_launch_count)
void count_launches(long long n);
long long launch_total();

}  // namespace fg
