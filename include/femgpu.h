/*
 * femgpu — GB300 (sm_103a) solve path for 2-D stabilised P1 finite elements.
 *
 * Plain C ABI: opaque handles, host pointers and sizes, integer status codes.
 * No function exits the process; every call returns FG_OK or an error code
 * whose text fg_last_error() gives.
 *
 * Numbering.  Host-facing calls use the reference's equation numbering:
 * equations 0..n-1 of the free dofs (Node.invP_id), and every vector has
 * n + 1 slots, slot n being the Dirichlet sink that reads as 0
 * (01_SS_Transport_Equation/2D/01_CommonFiles/Preprocess.c:288-296 with one
 * rank: neq_bef = 0, NEQ = neq).  Element blocks are row-major S x S per
 * element, S = 3 * ndof (ebe_assembly.c:3-19), and lm is Fill_LM's map.
 * Internally the library renumbers the dofs (local reverse Cuthill-McKee,
 * as Permutation_of_LM.c does for ebemv) and colours the elements.
 */
#ifndef FEMGPU_H
#define FEMGPU_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status ---- */
enum {
    FG_OK = 0,
    FG_ERR_ARG = 1,        /* invalid argument or size                         */
    FG_ERR_CUDA = 2,       /* CUDA runtime error (text in fg_last_error)       */
    FG_ERR_NOMEM = 3,      /* device or host allocation failed                 */
    FG_ERR_STATE = 4,      /* call out of order (e.g. solve before blocks)     */
    FG_ERR_BREAKDOWN = 5,  /* zero pivot / non-finite value in the solve       */
    FG_ERR_NOTCONV = 6,    /* iteration limit reached before the tolerance     */
    FG_ERR_UNSUPPORTED = 7, /* option not available for this system            */
    FG_ERR_TIMEOUT = 8     /* a bounded device-side wait ran out               */
};

/* Text of the last error on the calling thread (never NULL). */
const char *fg_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
int fg_version(void);
/* Select the CUDA device for handles created afterwards on this thread. */
int fg_set_device(int device);

/* ---- system: mesh connectivity, element blocks, preconditioner ---- */
typedef struct fg_system fg_system;

enum { FG_REORDER_NONE = 0, FG_REORDER_RCM = 1 };

/* Create a system from the mesh.
 *   ien[nel*3]         element vertices (Element[e].Vertex)
 *   type[nnodes*ndof]  0 = Dirichlet dof, otherwise free (Node.Type)
 *   invp[nnodes*ndof]  equation of each free dof, 0..neq-1 (Node.invP_id)
 * Builds lm (Fill_LM.c), the local RCM numbering of the dof graph
 * (Permutation_of_LM.c, when reorder == FG_REORDER_RCM; the reference's
 * drivers use it for ndof == 1 and node order otherwise), a greedy element
 * colouring and
 * the dof/node incidence lists, and uploads the connectivity.
 * Replaces Preprocess.c:288-340 (lm, Perm, invPerm, A allocation). */
int fg_system_create(fg_system **out, int nnodes, int nel, int ndof,
                     const int *ien, const int *type, const int *invp, int neq,
                     int reorder);

/* ---- mesh files (host only, no device needed) ----
 * fg_mesh_read: a global mesh file as Mesh_Generator/Structured_Mesh/
 * meshGenerator.c:184-209 writes it (per node x, y and one free(1)/
 * prescribed(0) flag per dof; elements v0 v1 v2, with a trailing tag when
 * ndof > 1); equations numbered over the free dofs in node order.
 * fg_mesh_read_rank: a one-rank partition file as SST/Preprocess.c:127-168
 * reads it (per node x, y and per dof Type [Send invP_id]); the file's
 * invP_id numbering is kept.  Call once with NULL arrays for the sizes in
 * *info, then with x, y[nnodes], type, invp[nnodes*ndof], ien[nel*3]; the
 * arrays feed fg_system_create.  Replaces the partitioner's one-rank output
 * (Parallel_Preprocess) for single-GPU runs. */
typedef struct { int nnodes, nel, neq; } fg_mesh_info;
int fg_mesh_read(const char *path, int ndof, fg_mesh_info *info, double *x, double *y, int *type, int *invp,
                 int *ien);
int fg_mesh_read_rank(const char *path, int ndof, fg_mesh_info *info, double *x, double *y, int *type, int *invp,
                      int *ien);

/* Paraview output (the drivers' 01_CommonFiles/Paraview_Output.c): an ASCII
 * VTK UnstructuredGrid of the triangles with the fields as point data, in
 * order.  values are node-major [nnodes*ncomp], ncomp 1..3 (a 2-component
 * field is written with a third component 0).  z lifts the points (the
 * transport drivers write (x, y, u)); NULL writes z = 0.  Host only. */
typedef struct {
    const char *name;
    int ncomp;
    const double *values;
} fg_vtu_field;
int fg_write_vtu(const char *path, int nnodes, int nel, const double *x, const double *y, const int *ien,
                 int nfields, const fg_vtu_field *fields, const double *z);

/* Host-only set-up products of a mesh (no device needed): lm[nel*3*ndof]
 * (Fill_LM), Perm/invPerm[neq+1] (Permutation_of_LM with SYMRCM),
 * colour[nel] (greedy element colouring; -1 for an element without a free
 * dof), and into info: ncolours, bandwidths, nnz.  Any output may be NULL. */
typedef struct fg_system_info fg_system_info;
int fg_mesh_analyze(int nnodes, int nel, int ndof, const int *ien, const int *type,
                    const int *invp, int neq, int reorder, int *lm, int *Perm,
                    int *invPerm, int *colour, fg_system_info *info);
int fg_system_destroy(fg_system *s);

struct fg_system_info {
    int n, nel, ndof, S, nnodes, ncolours;
    int bandwidth_before, bandwidth_after;  /* MATRIX_bandwidth of the dof graph */
    int nnz;                                /* entries of the dof adjacency      */
    size_t device_bytes;                    /* device memory held by the system  */
};
int fg_system_get_info(const fg_system *s, fg_system_info *info);

/* Copies of the set-up products, in the reference's numbering:
 * lm[nel*S]; Perm[n+1], invPerm[n+1] (Permutation_of_LM.c:56-72);
 * colour[nel] (greedy element colouring over the free dofs). */
int fg_system_get_lm(const fg_system *s, int *lm);
int fg_system_get_perm(const fg_system *s, int *Perm, int *invPerm);
int fg_system_get_colours(const fg_system *s, int *colour);

/* Upload element blocks A[nel][S][S] (row-major, ebe_assembly.c) from host
 * memory; keeps an FP64 and an FP32 copy on the device. */
int fg_set_blocks(fg_system *s, const double *A);
/* Download the element blocks (row-major, reference element order). */
int fg_get_blocks(const fg_system *s, double *A);

/* Q = A P (ebemv / ebemvNDOF3 / ebemvNDOF4 on the GPU).  P and Q are host
 * vectors of n+1 entries; Q[n] is returned as 0.  precision: 64 or 32. */
int fg_matvec(fg_system *s, const double *P, double *Q, int precision);

/* Q = A P like fg_matvec, on DEVICE vectors the caller owns (n+1 entries
 * each, reference numbering, Q[n] returned as 0), without allocating any
 * memory.  No counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc after their set-up phase (their device memory
 * belongs to another allocator, or their loop must not pay cudaMalloc's
 * implicit synchronisation).  The scratch it needs comes from one fixed
 * array of about 33 MiB compiled into the library and held on every GPU
 * that loads it; systems with more than 2,097,151 equations, more than
 * 65,536 element patches (a patch holds up to 1024 elements for 3x3
 * blocks, 256 for larger blocks) or more than 64 patch colours are
 * rejected with FG_ERR_ARG.  It always multiplies by the element blocks,
 * also for a system switched to the CSR operator.
 * The first call on a device looks up the array's device address, so make
 * that first call before starting any stream capture.  The work is queued
 * on the system's stream (fg_system_stream) and the call returns without
 * waiting for it.  All calls share the array: calls that overlap on the
 * GPU race and must be serialised by the caller. */
int fg_matvec_noalloc(fg_system *s, const double *P_dev, double *Q_dev, int precision);

/* ---- assembled CSR operator (MatrixVectorProductScheme "CSR") ----
 * FG_OP_CSR builds, once, the CSR pattern of the free dofs in the local RCM
 * numbering (csr_Initialization.c:5-434) and from then on assembles the CSR
 * values from the element blocks on the device (csr_assembly.c:3-54, sums
 * in element order) whenever blocks change; matvecs and solves use the CSR
 * form (csrmv.c:4-65).  FG_OP_EBE (default) uses the element blocks. */
enum { FG_OP_EBE = 0, FG_OP_CSR = 1 };
int fg_set_operator(fg_system *s, int op);
/* CSR values in the reference's CSR layout: IA[n+1], JA[nnz], AA[nnz]
 * (internal numbering = the reference's renumbered equations), any NULL. */
int fg_get_csr(const fg_system *s, int *nnz, int *IA, int *JA, double *AA);

/* ---- preconditioners (Solvers_and_Preconditioners/preconditioners.h) ---- */
enum { FG_PRECOND_NONE = 0, FG_PRECOND_DIAG = 1, FG_PRECOND_BLOCKDIAG = 2,
       FG_PRECOND_ILU0 = 3, /* ILU(0) of the assembled CSR operator (fg_set_operator) */
       FG_PRECOND_SPIKE = 4, /* truncated SPIKE of the CSR operator (fg_set_spike)  */
       FG_PRECOND_LUE = 5,  /* element LU sweep, Preconditioner "LUe" (3x3 EBE, FP64) */
       FG_PRECOND_SGSE = 6  /* element symmetric Gauss-Seidel, "SGSe": forward sweep
                               on the left, backward sweep on the right (3x3 EBE, FP64) */ };
/* Truncated SPIKE ("SPIKEk", CSR/SPIKE_precond_setup.c:10-312 and
 * CSR/SPIKE_precond.c:8-158).  The reference's P MPI ranks become `parts`
 * row blocks of the CSR operator on one GPU (at most n / 2k, so every block
 * keeps 2k rows); each block is factorised by banded LU without pivoting
 * (the reference calls PARDISO) and neighbours are coupled through k x k
 * corner blocks and one 2k x 2k reduced system per interface.  k in
 * [1, 64] (default 16), parts in [1, 65536] (default 16).  Takes effect at
 * the next fg_precond_setup(FG_PRECOND_SPIKE); systems whose band factors
 * would exceed 8 GiB are rejected there with FG_ERR_UNSUPPORTED. */
int fg_set_spike(fg_system *s, int k, int parts);
/* Fill level p of the ILU preconditioner (Preconditioner "ILU<p>",
 * CSR/ILUp_precond_setup.c:16 with the level-of-fill symbolic pass of
 * ilup.c:164-301); 0 (the default) is ILU(0).  FG_PRECOND_ILU0 then sets up
 * and applies ILU(p) on the factor pattern; p in [0, 16]. */
int fg_set_ilu_fill(fg_system *s, int p);
/* Block-Jacobi ILU(p): the CSR operator's rows (RCM numbering) cut into
 * `blocks` equal row blocks, and only the couplings inside a block are
 * factorised -- what `blocks` MPI ranks of the reference compute, each
 * factorising its own rows' block (CSR/ILUp_precond_setup.c:20-29).  The
 * substitutions' dependency depth drops about blocks-fold.  1 (the
 * default) is the global ILU(p). */
int fg_set_ilu_blocks(fg_system *s, int blocks);
/* Polls (>= 1) a device-side dependency wait of the ILU kernels makes
 * before it gives up and the call returns FG_ERR_TIMEOUT (default 2^24,
 * about half a second); applies to the current device. */
int fg_set_wait_limit(long long polls);
/* Cap (bytes) on the device memory the library allocates in this process;
 * an allocation that would pass it fails with FG_ERR_NOMEM and the call
 * that needed it returns that code.  0 (the default) removes the cap.
 * fg_memory_in_use gives the bytes currently allocated. */
int fg_set_memory_limit(size_t bytes);
size_t fg_memory_in_use(void);
enum {
    FG_SETUP_ACCUMULATE = 1, /* Diag += new diagonal, as Diag_precond_EBE_setup
                                does across nonlinear iterations              */
    FG_SETUP_REF_QUIRKS = 2  /* 4x4 block inverse with the reference's entry-14
                                term (BlockDiag_precond_EBE_setup.c:142)      */
};
/* ---- diagonal scaling (Solvers_and_Preconditioners/scaling.c) ----
 * FG_SCALE_LEFT: Left_scaling_EBE (:10-42): the accumulating Diag set-up on
 * F (F /= Diag), then every block row times 1/Diag of its equation.
 * FG_SCALE_LEFTRIGHT: LeftRight_scaling_EBE (:92-121): entries times
 * sqrt(1/Diag_I 1/Diag_J), F = (F / Diag) sqrt(Diag); solve, then
 * fg_unscale (Left_unscaling, :187-196: X *= sqrt(1/Diag)).  F: host n+1,
 * in place, may be NULL.  The system's preconditioner becomes
 * FG_PRECOND_NONE (set another one up afterwards if wanted). */
/* FG_SCALE_BLOCK: Block_scaling_EBE (Block_scaling.c:10-118, Scaling
 * "BlockScaling" of the Euler driver, which installs it but never calls it):
 * the block-diagonal set-up (F <- B^-1 F, the reference's 4x4 inverse), then
 * in every element block the rows and columns of Dirichlet dofs cleared
 * (diagonal 1) and each node's row block multiplied by its inverse block;
 * fg_unscale is then the identity (NO_unscaling).  Systems with ndof 2-4. */
enum { FG_SCALE_LEFT = 1, FG_SCALE_LEFTRIGHT = 2, FG_SCALE_BLOCK = 3 };
int fg_scale(fg_system *s, int kind, double *F);
int fg_unscale(fg_system *s, double *X);

/* Build the preconditioner from the current blocks and, when F is not NULL,
 * precondition F in place (n+1 host entries), as the *_EBE_setup routines
 * do.  The right-hand side the solver receives is then M^-1 F. */
int fg_precond_setup(fg_system *s, int kind, int flags, double *F);
/* z = M^-1 p for host vectors of n+1 entries (p == z allowed). */
int fg_precond_apply(fg_system *s, const double *p, double *z);
/* The right preconditioner of the system's set-up applied to p (host
 * vectors of NEQ + 1, reference numbering): the backward element sweep of
 * FG_PRECOND_SGSE (SGS_precondR_EBE), the identity for every other kind
 * (NO_precond).  p may equal z. */
int fg_precond_apply_right(fg_system *s, const double *p, double *z);
/* Diagonal used by the Diag preconditioner (n+1 entries, host). */
int fg_get_diag(const fg_system *s, double *Diag);
int fg_set_diag(fg_system *s, const double *Diag);

/* ---- GMRES (Solvers_and_Preconditioners/pgmres.c:5-200) ---- */
enum { FG_PREC_FP64 = 64, FG_PREC_MIXED = 32, FG_PREC_MIXED16 = 16 };
typedef struct {
    int kmax;            /* KrylovBasisVectorsQuantity (k-1 Arnoldi steps/cycle) */
    int lmax;            /* LinearMaxIter: restart cycles                         */
    double tol;          /* SolverTolerance                                       */
    int precision;       /* FG_PREC_FP64: the reference's method, all FP64;
                            FG_PREC_MIXED: FP32 Arnoldi (blocks, basis, M^-1)
                            inside FP64 refinement: each cycle restarts from the
                            FP64 residual, stops when the true relative residual
                            ||F - A X|| / ||F|| <= tol;
                            FG_PREC_MIXED16: the same with the Krylov basis
                            stored in FP16 (scaled by a power of two near
                            sqrt n; arithmetic stays FP32, kmax <= 32)            */
    double inner_tol;    /* mixed: relative decrease per FP32 cycle (0 = 1e-5)    */
} fg_solver_opts;

typedef struct {
    int iterations;      /* Arnoldi steps (Parameters->iterations increment)   */
    int cycles;          /* restart cycles                                     */
    int converged;       /* 1 when the stopping test was met                   */
    int status;          /* FG_OK / FG_ERR_NOTCONV / FG_ERR_BREAKDOWN          */
    double rho;          /* last preconditioned residual estimate              */
    double eps;          /* tol * ||M^-1 F|| (FP64) or tol (mixed)             */
    double true_rel_residual; /* ||F - A X||_2 / ||F||_2, FP64 on the device   */
    double seconds;      /* wall time of the solve on the device stream        */
} fg_solve_stats;

/* Solve (M^-1 A) X = B with B = M^-1 F already preconditioned (as the
 * reference's precond_setup leaves F).  X0 = 0.  F_true (optional, n+1,
 * unpreconditioned) is used for the true residual; NULL: B is used with M.
 * B, X, F_true are host vectors of n+1 entries. */
int fg_solve(fg_system *s, const fg_solver_opts *opts, const double *B, double *X,
             const double *F_true, fg_solve_stats *stats);

/* Solve many systems together (same block size and preconditioner kind):
 * one CUDA-graph launch per restart cycle advances every member, members
 * stop independently, and each result is bit-identical to solving that
 * system alone.  B[i], X[i], F_true[i] are host vectors of system i
 * (F_true may be NULL, or F_true[i] NULL).  stats has count entries. */
int fg_solve_batch(fg_system *const *systems, int count, const fg_solver_opts *opts,
                   const double *const *B, double *const *X, const double *const *F_true,
                   fg_solve_stats *stats);

/* Device-resident variant: each system solves with the right-hand side its
 * last fg_transport_prepare left on the device; the solution stays on the
 * device (fg_get_solution copies it out). */
int fg_solve_resident(fg_system *const *systems, int count, const fg_solver_opts *opts,
                      fg_solve_stats *stats);
int fg_get_solution(const fg_system *s, double *X);

/* Kernel launches issued by this library so far (direct launches plus the
 * kernel nodes of every graph launch), for launch accounting. */
long long fg_launch_count(void);

/* The CUDA stream (cudaStream_t) a system's work runs on, for callers that
 * record events or order their own work around it. */
void *fg_system_stream(const fg_system *s);

/* Time the batched EBE matvec of these systems alone: reps back-to-back
 * matvecs (all colours) of V[0] into the Arnoldi work vector, in FP64
 * (precision 64) or FP32 (32), timed with CUDA events on the first
 * system's stream.  *ms_per_matvec receives the mean; *bytes the
 * algorithmic bytes of one matvec: nel*(S*S*w + S*4) + 2*n*w summed over
 * the systems.  Requires a previous solve (workspace) on every system. */
int fg_bench_matvec(fg_system *const *systems, int count, int precision, int reps,
                    double *ms_per_matvec, double *bytes);

/* Autotuner: times candidate launch shapes of a batch on the batch itself
 * (one restart cycle each, CUDA events on the first system's stream) --
 * the dof-part size of the Krylov kernels (256 ... 16384 dofs) and, for
 * 3x3 blocks in FP32, the matvec kernel (bulk-copy pipeline or register
 * kernel) -- and keeps the fastest for the process, keyed by (block size,
 * precision, batch-size class floor(log2(batch dofs))).  Every later batch
 * of that key (fg_solve_batch, fg_solve_resident, the request server) uses
 * it.  The systems need resident right-hand sides (fg_transport_prepare or
 * a time-loop set-up).  remeasure 0 returns a cached choice when there is
 * one (from_cache = 1).  The cycles run on the systems' workspaces, which
 * the next solve reinitialises.  No counterpart in the reference (its
 * launch shapes are fixed). */
typedef struct {
    int part_dofs;        /* dofs per part of the Krylov kernels            */
    int mv3_pipeline;     /* 3x3 FP32 matvec: 1 bulk-copy pipeline, 0 the
                             register kernel (other blocks: 1)              */
    double ms_per_cycle;  /* one restart cycle of the batch with it         */
    int from_cache;       /* taken from the cache, not measured now         */
    int candidates;       /* launch shapes timed                            */
} fg_tune_choice;
int fg_autotune(fg_system *const *systems, int count, const fg_solver_opts *o, int remeasure,
                fg_tune_choice *out);
/* The cached choice for this batch's key; FG_ERR_STATE when none. */
int fg_tune_lookup(fg_system *const *systems, int count, const fg_solver_opts *o, fg_tune_choice *out);
/* Install a choice for this batch's key without timing (a choice kept
 * from an earlier run, or a pinned configuration); later batches of the key
 * use it.  FG_ERR_ARG unless part_dofs is a multiple of 8 in
 * [256, 16384] and mv3_pipeline is 0 or 1. */
int fg_tune_set(fg_system *const *systems, int count, const fg_solver_opts *o, const fg_tune_choice *choice);
/* Forget every cached choice (batches use the built-in rule again). */
void fg_tune_clear(void);

/* ---- steady SUPG/CAU transport assembly on the device ---- */
typedef struct {
    double k;            /* Condutivity(), used for kx and ky         */
    double gamma;        /* Reaction()                                */
    double beta[2];      /* Velocity() (constant field)               */
    double f;            /* Font() (constant source)                  */
    int cau;             /* ShockCapture: 1 "CAU" (CAU_ShockCapture.c),
                            2 "CAUDD" (CAU_DD_ShockCapture.c, DD form
                            only), 3 "YZBeta" (YZBeta_ShockCapture.c:
                            per-element state kept on the device
                            across builds, zeroed when a Process run
                            starts), 0 none                           */
    int form;            /* StabilizationForm: FG_TRANSPORT_SUPG (0)
                            Build_K_F_SUPG.c, or FG_TRANSPORT_DD
                            Build_K_F_DD.c:4-178 (steady builds only) */
    int h_shock;         /* h_Shock: FG_HSHOCK_2SQRTAREA (0), _OPTION1
                            (h_shock_Option1.c), _OPTION2 (steady)    */
} fg_transport_coeffs;
enum { FG_TRANSPORT_SUPG = 0, FG_TRANSPORT_DD = 1 };
enum { FG_SHOCK_NONE = 0, FG_SHOCK_CAU = 1, FG_SHOCK_CAUDD = 2, FG_SHOCK_YZBETA = 3 };
enum { FG_HSHOCK_2SQRTAREA = 0, FG_HSHOCK_OPTION1 = 1, FG_HSHOCK_OPTION2 = 2 };

/* Set node coordinates (x, y) and Dirichlet values upresc[nnodes]. */
int fg_set_geometry(fg_system *s, const double *x, const double *y, const double *upresc);
/* Build_K_F_SUPG on the device at the free-dof state u (host, n entries,
 * NULL = 0): element blocks stay on the device; F (host, n+1) receives the
 * right-hand side when not NULL. */
int fg_transport_assemble(fg_system *s, const fg_transport_coeffs *c, const double *u, double *F);
/* Assemble at u (host, n entries, NULL = 0) and set up a fresh Diag
 * preconditioner, keeping F and M^-1 F on the device as the system's
 * resident right-hand side for fg_solve_resident.  Nothing is copied back. */
int fg_transport_prepare(fg_system *s, const fg_transport_coeffs *c, const double *u);
/* Steady transport Process loop (Process.c:6-93) on the device: assemble,
 * Diag setup (accumulating, as the reference), GMRES, until
 * ||u - u_old|| <= nonlinear_tol * ||u||.  U (host, n entries) holds the
 * solution. */
typedef struct {
    int nonlinear_iterations;
    int gmres_iterations;
    double seconds;
    double true_rel_residual;  /* of the last linear solve */
    double nonlinear_residual; /* the loop's last stopping quantity */
} fg_process_stats;
int fg_transport_process(fg_system *s, const fg_transport_coeffs *c,
                         const fg_solver_opts *opts, double nonlinear_tol,
                         int max_nonlinear, double *U, fg_process_stats *stats);

/* ---- steady incompressible Navier-Stokes, SUPG/PSPG/LSIC (NDOF = 3) ----
 * Replaces Build_K_F_SUPG_PSPG.c:8-669 (with eval_U.c:3-35 and
 * ebe_assembly.c) and the Picard loop of
 * 04_SS_NavierStokes_Equations/2D/01_CommonFiles/Process.c:6-62 for a system
 * created with ndof = 3 (dofs u, v, p per node). */
typedef struct {
    double reynolds;   /* ReynoldsNumber: density 1, viscosity 1/Re          */
    int precond;       /* FG_PRECOND_BLOCKDIAG (BlockDiagDOF3), FG_PRECOND_DIAG
                          (accumulating, as Diag_precond_EBE_setup.c),
                          FG_PRECOND_NONE, or FG_PRECOND_ILU0 / _SPIKE on a
                          system switched to FG_OP_CSR                        */
    int form;          /* StabilizationForm (setStabilizationForm.c):
                          FG_NS_SUPG_PSPG (0) Build_K_F_SUPG_PSPG.c, or
                          FG_NS_VMS_DCDD Build_K_F_VMS_DCDD.c:8-716 (LSIC and
                          the condensed bubble; its source term is 0)         */
} fg_ns_coeffs;
enum { FG_NS_SUPG_PSPG = 0, FG_NS_VMS_DCDD = 1 };

/* Node coordinates, the prescribed (u, v, p) of every node (upresc[3*node+k],
 * read where dof k of the node is Dirichlet: v1presc/v2presc/ppresc at the
 * node) and the body force at the nodes (f1ext/f2ext; NULL = 0). */
int fg_ns_set_geometry(fg_system *s, const double *x, const double *y, const double *upresc,
                       const double *f1, const double *f2);
/* Build_K_F_SUPG_PSPG at the free-dof state u (host, n entries, NULL = 0):
 * the 9x9 Picard tangent stays on the device; F (host, n+1) receives the
 * residual when not NULL. */
int fg_ns_assemble(fg_system *s, const fg_ns_coeffs *c, const double *u, double *F);
/* Picard loop: assemble at u, preconditioner set-up, GMRES for the increment
 * s, u += s, until ||s|| / ||u|| <= nonlinear_tol or max_nonlinear
 * iterations.  u (host, n entries) is the initial state on entry (the
 * reference starts from 0) and the solution on return; the state stays on the
 * device between iterations. */
int fg_ns_process(fg_system *s, const fg_ns_coeffs *c, const fg_solver_opts *opts, double nonlinear_tol,
                  int max_nonlinear, double *u, fg_process_stats *stats);

/* ---- compressible Euler, SUPG + CAU, conservative variables (NDOF = 4) ----
 * Replaces Build_M_K_F_SUPG.c:6-1057 (with Delta_CAU.c, Ax_Ay_calculations.c,
 * eval_U_dU.c and ebe_assembly.c) of 03_Euler_Equations/2D/01_CommonFiles and
 * the predictor/multicorrector loop of
 * 00_CommonFiles/Time_Integration/Predictor_Old.c:6-134 with the stop tests
 * of Criteria.c, for a system created with ndof = 4 (rho, rho u, rho v, rho E
 * per node). */
typedef struct {
    double gamma;      /* FemFunctions->gamma (a constant)                        */
    double mach;       /* Parameters->Mach, used by the dimensionless Jacobians   */
    int dimensionless; /* 1: dimensionless_Ax_Ay_calculations; 0: dimensional    */
    double tolerance;  /* StabilizationTolerance: CAU is off below this |grad U|  */
    double alpha;      /* Alpha (time integration)                                */
    double dt;         /* DeltaT                                                  */
    int form;          /* StabilizationForm: FG_EULER_SUPG (0), or FG_EULER_DD:
                          Build_M_K_F_DD_Transiente.c with Delta_DD.c ("DD",
                          "Predictor1", "CAUDD"); its per-element state (the
                          bubble values and the relaxed delta) stays on the
                          device and is zeroed when fg_euler_predictor starts */
    double invY[4];    /* Parameters->invY: the scaling of the YZBeta shock
                          capture (Delta_YZBeta.c)                             */
    int shock;         /* ShockCapture: 0 = the form's own (Delta_CAU for SUPG,
                          Delta_DD for DD), FG_SHOCK_YZBETA = Delta_YZBeta with
                          invY (setStabilizationForm.c:24-26, 64-66);
                          "Predictor2" always uses YZBeta                      */
} fg_euler_coeffs;
enum { FG_EULER_SUPG = 0, FG_EULER_DD = 1 };

/* Node coordinates and the prescribed (rho, rho u, rho v, rho E) of every node
 * (upresc[4*node+k], read where dof k of the node is Dirichlet). */
int fg_euler_set_geometry(fg_system *s, const double *x, const double *y, const double *upresc);
/* Build_M_K_F_SUPG at the free-dof state u and its time derivative du (host,
 * n entries each; NULL = 0): the 12x12 blocks Me + alpha dt Ke stay on the
 * device; R (host, n+1) receives -Me dU - Ke U when not NULL. */
int fg_euler_assemble(fg_system *s, const fg_euler_coeffs *c, const double *u, const double *du, double *R);

/* Time loop controls (Criteria.c) and the preconditioner of each correction. */
typedef struct {
    int stop_by_norm;      /* 0: StopByIterations; 1: StopByNorm                  */
    int max_corrections;   /* NonLinearMaxIter                                     */
    double correction_tol; /* NonLinearTolerance (StopByNorm)                      */
    int steady_state;      /* 0: StopByTime; 1: StopBySteadyState                  */
    double final_time;     /* FinalTime                                            */
    double time_tol;       /* TimeIntegrationTolerance (StopBySteadyState)         */
    int max_steps;         /* bound on the steps, 0 = none (not in the reference)  */
    int precond;           /* FG_PRECOND_BLOCKDIAG, FG_PRECOND_DIAG or NONE; ILU0 or
                              SPIKE on a system switched to FG_OP_CSR            */
    int setup_flags;       /* FG_SETUP_REF_QUIRKS: the reference's 4x4 inverse     */
    int scheme;            /* FG_TIME_PREDICTOR (0), FG_TIME_BDF, FG_TIME_TRBDF2,
                              FG_TIME_PREDICTOR2 (the DD forms of the transient
                              transport and Euler builds)                     */
} fg_time_opts;

/* TimeIntegration of the drivers (setStabilizationForm.c):
 *   FG_TIME_PREDICTOR  "Predictor1"        Predictor_Old.c
 *   FG_TIME_BDF        "Predictor1_BDF"    Predictor_Old_BDF.c: one BDF1 step
 *                      (no prediction, u += alpha dt Da), then BDF2 steps
 *                      u = 4/3 u^n - 1/3 u^{n-1}, u += 2/3 dt Da; the Build
 *                      keeps Alpha_Build = alpha, and the steady-state test
 *                      compares with the initial state, as the reference does
 *   FG_TIME_TRBDF2     Predictor_New_TRBDF2.c without its bubble unknowns:
 *                      per step a TR stage (alpha 1/2 over lambda dt,
 *                      lambda = 2 - sqrt 2) and a BDF2 stage (alpha
 *                      1/(2 - lambda) over (1 - lambda) dt, prediction
 *                      A u - B u_old).  "Predictor1_TRBDF2"
 *                      (Predictor_Old_TRBDF2.c) solves against a right-hand
 *                      side that nothing fills and is not restated.
 *   FG_TIME_PREDICTOR2 "Predictor2"        Predictor_New.c:3-179 with the
 *                      DD form (fg_tt_predictor: one bubble unknown per
 *                      element; fg_euler_predictor: four, with YZBeta):
 *                      Predictor_Old's steps plus the bubble unknowns,
 *                      predicted with u (uB += (1 - alpha) dt aB, aB = 0)
 *                      and corrected after each solve from Da
 *                      (calculate_DaB: aB += DaB, uB += alpha dt DaB).
 *   FG_TIME_PREDICTOR2_BDF    "Predictor2_BDF"  Predictor_New_BDF.c:54-184
 *                      (fg_euler_predictor, DD): a BDF1 step with
 *                      Alpha_Build = 1 (u += dt Da), then BDF2 steps with
 *                      Alpha_Build = 2/3; u_old = u before each BDF2
 *                      prediction (the steady-state test compares with the
 *                      previous step); the bubble unknowns follow the same
 *                      combinations.
 *   FG_TIME_PREDICTOR2_TRBDF2 "Predictor2_TRBDF2"  Predictor_New_TRBDF2.c
 *                      (fg_euler_predictor, DD): the TR-BDF2 stages of
 *                      FG_TIME_TRBDF2 with the bubble unknowns, uB starting
 *                      from the element centroids of the initial state
 *                      (uB_InitialSolution; prescribed dofs take their
 *                      prescribed value -- the reference reads u[-1] there,
 *                      testing invP_id against NEQ where Preprocess.c:173
 *                      stores -1).  The Predictor1 DD build is not offered
 *                      with FG_TIME_TRBDF2 (the reference pairs it with
 *                      Predictor_Old_TRBDF2, which is not restated). */
enum { FG_TIME_PREDICTOR = 0, FG_TIME_BDF = 1, FG_TIME_TRBDF2 = 2, FG_TIME_PREDICTOR2 = 3,
       FG_TIME_PREDICTOR2_BDF = 4, FG_TIME_PREDICTOR2_TRBDF2 = 5 };

typedef struct {
    int steps;
    int corrections;
    int gmres_iterations;
    double t;                  /* time reached                                    */
    double seconds;
    double true_rel_residual;  /* of the last linear solve                        */
} fg_time_stats;

/* Predictor_Old (t->scheme FG_TIME_PREDICTOR; BDF and TR-BDF2 above): per
 * step t += dt, u += (1 - alpha) dt a, a = 0, then
 * corrections (assemble at (u, a), preconditioner set-up on R, GMRES for Da,
 * a += Da, u += alpha dt Da) until the correction stop test, until the time
 * stop test.  u (host, n) is the initial state on entry (the problem's
 * InitialSolution) and the final state on return; a (host, n, may be NULL)
 * receives du/dt.  The state stays on the device for the whole loop. */
int fg_euler_predictor(fg_system *s, const fg_euler_coeffs *c, const fg_solver_opts *opts,
                       const fg_time_opts *t, double *u, double *a, fg_time_stats *stats);
/* TimeIntegration "Predictor2" of the Euler driver (t->scheme
 * FG_TIME_PREDICTOR2 with c.form FG_EULER_DD; ShockCapture "YZBeta" with
 * c.invY): each correction builds with Build_M_F_DD_Transiente.c:6-821 --
 * four bubble unknowns per element kept and condensed out of the element
 * system, Delta_YZBeta for the DD diffusion and Delta_YZBetaNMV (relaxed,
 * state on the device) for the bubble stiffness -- and recovers the bubble
 * increments from Da (calculate_DaB.c:3-61).  With "CAUDD" the reference
 * passes an A0 it never computes to Delta_DD (:137-138), an undefined
 * result, so that combination is not offered.
 *
 * One build at (u, du, uB, duB) with fresh shock-capture states (u, du:
 * free dofs, reference numbering; uB, duB: 4 per element, reference element
 * order; NULL = 0).  F (host, n+1, may be NULL) receives the load, cond
 * (host, 53 per element, may be NULL) invN2, R2[4], M2[4][12]; the blocks
 * stay on the device (fg_get_blocks). */
int fg_euler_bubble_assemble(fg_system *s, const fg_euler_coeffs *c, const double *u, const double *du,
                             const double *uB, const double *duB, double *F, double *cond);

/* ---- transient SUPG/CAU transport (02_Transport_Equation) ----
 * Replaces Build_M_K_R_SUPG.c:6-252 (with CAU_ShockCapture.c:3-33,
 * h_shock_2sqrtArea.c, eval_U_dU.c and ebe_assembly.c) for a system with
 * ndof = 1 and the geometry of fg_set_geometry: the blocks become
 * Ae = me + alpha dt ke (SUPG mass and the steady operator of
 * fg_transport_assemble), R = F - me du - ke u, accumulated in the
 * reference's element order (bit-identical).  With c.form = FG_TRANSPORT_DD
 * (StabilizationForm "DD", Predictor1) the build is Build_M_K_R_DD.c:5-190:
 * the bubble condensed into me, ke and the load, and c.cau = FG_SHOCK_CAUDD
 * the transient CAUDD relaxed against each element's previous value (state
 * on the device, zeroed when fg_tt_predictor starts). */
typedef struct {
    fg_transport_coeffs c;  /* conductivity, reaction, velocity, source, CAU */
    double alpha;           /* Alpha (Alpha_Build)                          */
    double dt;              /* DeltaT (DeltaT_Build)                         */
} fg_tt_coeffs;
/* One build at (u, du) (free dofs, reference numbering, host; NULL = 0);
 * R (host, n+1, may be NULL) receives the residual. */
int fg_tt_assemble(fg_system *s, const fg_tt_coeffs *c, const double *u, const double *du, double *R);
/* Predictor_Old (Time_Integration/Predictor_Old.c:6-134, Criteria.c) with
 * this build, as fg_euler_predictor runs it: state, residual and increment
 * on the device; t->precond FG_PRECOND_DIAG (accumulating, the reference's
 * Diag_precond_EBE_setup) or any other kind this system supports. */
int fg_tt_predictor(fg_system *s, const fg_tt_coeffs *c, const fg_solver_opts *opts, const fg_time_opts *t,
                    double *u, double *a, fg_time_stats *stats);
/* TimeIntegration "Predictor2" (t->scheme FG_TIME_PREDICTOR2, c.form
 * FG_TRANSPORT_DD): each correction builds with Build_M_F_DD.c:6-263 -- the
 * element's bubble kept as an unknown (uB, duB) and condensed out of the
 * element system, N2 = MBB + alpha dt KBB -- and recovers the bubble
 * increment from Da (calculate_DaB.c:3-30); bubble unknowns and condensation
 * data stay on the device.  Blocks, load and DaB are bit-identical with the
 * reference's functions.
 *
 * One build at (u, du, uB, duB) with a fresh shock-capture state (u, du:
 * free dofs, reference numbering; uB, duB: nel values in reference element
 * order; NULL = 0).  F (host, n+1, may be NULL) receives the load, cond
 * (host, 5 per element, may be NULL) invN2, R2, M2[0..2]; the blocks stay on
 * the device (fg_get_blocks). */
int fg_tt_bubble_assemble(fg_system *s, const fg_tt_coeffs *c, const double *u, const double *du, const double *uB,
                          const double *duB, double *F, double *cond);
/* calculate_DaB after the last Predictor2 build (transient transport or
 * Euler): DaB (host; nb = 1 or 4 values per element, element-major in
 * reference element order) from Da (host, n+1, reference numbering; its
 * sink entry is read as 0). */
int fg_bubble_dab(fg_system *s, const double *Da, double *DaB);
/* The bubble unknowns uB and aB (host, nb per element as above, either may
 * be NULL) after a Predictor2 loop (FG_TIME_PREDICTOR2). */
int fg_bubble_state(fg_system *s, double *uB, double *aB);

/* ---- request server: continuous batching of transport solves ----
 * A worker thread owns one batch.  Requests (a system whose geometry is set,
 * with transport coefficients) wait in a FIFO; between restart cycles the
 * worker admits waiting requests while the Krylov workspace of the admitted
 * ones fits the HBM budget and the active count is below max_active,
 * assembles them on the device (SUPG/CAU at u = 0, fresh Diag), and every
 * cycle advances all admitted solves together; a solve leaves the batch as
 * soon as it converges.  Meshes and Krylov state stay on the device.  A
 * result is bit-identical to solving the same system alone. */
typedef struct fg_server fg_server;
typedef struct {
    int kmax, lmax;
    double tol;
    int precision;            /* FG_PREC_MIXED or FG_PREC_FP64          */
    double inner_tol;
    size_t hbm_budget_bytes;  /* 0: 80% of the free device memory; a
                                 request counts its system's arrays and the
                                 workspace it will allocate; one request
                                 runs alone even when it is larger      */
    int max_active;           /* 0: no limit                            */
} fg_server_opts;
typedef struct {
    unsigned long long tag;
    fg_solve_stats stats;
    double t_submit, t_admit, t_done;  /* seconds on the server's clock */
} fg_server_result;
int fg_server_create(fg_server **out, const fg_server_opts *opts);
/* Queue a request; thread-safe.  The system must not be in use elsewhere
 * until its result has been polled. */
int fg_server_submit(fg_server *sv, fg_system *s, const fg_transport_coeffs *c, unsigned long long tag);
/* Queue a request with host buffers (the C ABI of fg_set_blocks +
 * fg_precond_setup(FG_PRECOND_DIAG, 0, F) + fg_solve, served): A the
 * element blocks (row-major S x S per element, reference element order),
 * F the right-hand side (NEQ + 1); X (NEQ + 1) receives the solution
 * before the result can be polled.  The buffers stay the caller's but must
 * not be touched until then; pinned (page-locked) buffers copy fastest.
 * 3x3 systems. */
int fg_server_submit_host(fg_server *sv, fg_system *s, const double *A, const double *F, double *X,
                          unsigned long long tag);
/* Queue an Euler time loop (fg_euler_predictor with the server's kmax,
 * lmax, tol, precision and inner_tol); thread-safe.  u (host, n) is the
 * initial state and receives the final state; it and the system stay the
 * caller's but must not be touched until the result has been polled.  In
 * the result, stats.iterations counts the GMRES iterations of the loop,
 * stats.cycles its corrections.  Up to 16 loops run at once (each on its
 * system's stream, admitted against the same HBM budget as transport
 * requests); their correction solves with the BlockDiag preconditioner
 * share one continuously batched GMRES run (other preconditioners solve
 * alone), so a loop's result equals its fg_euler_predictor run. */
int fg_server_submit_euler(fg_server *sv, fg_system *s, const fg_euler_coeffs *c, const fg_time_opts *t,
                           double *u, unsigned long long tag);
/* Move up to max finished results into out; *count receives how many. */
int fg_server_poll(fg_server *sv, fg_server_result *out, int max, int *count);
/* Block until at least n results are waiting to be polled, or timeout_s. */
int fg_server_wait(fg_server *sv, int n, double timeout_s);
/* Seconds since the server was created (the clock of the results). */
double fg_server_now(const fg_server *sv);
int fg_server_destroy(fg_server *sv);

#ifdef __cplusplus
}
#endif
#endif
