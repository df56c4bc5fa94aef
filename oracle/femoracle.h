/*
 * femoracle — CPU restatement of the solve path of PARALLEL_FEM_CODES.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * library (libfemgpu): tests, the smoke entry point and the CPU-baseline
 * leg of the benchmark call it; the product path never does.
 *
 * Every function restates one reference routine with single-rank
 * (NPROC = 1) semantics: neq_bef = 0 and NEQ = neq, so every vector has
 * NEQ + 1 slots and slot NEQ is the Dirichlet sink that must read 0.
 * The restatement is pinned against the reference's own C compiled from
 * its sources (oracle/ref_harness) by tests/test_oracle_pin.py.
 *
 * Element blocks are stored as the reference stores them: element e owns
 * S*S doubles, row-major, at A[e*S*S] (ebe_assembly.c:9-17), and the
 * element->equation map lm[e*S + k] (Fill_LM.c).
 */
#ifndef FEMORACLE_H
#define FEMORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- mesh (Mesh_Generator/Structured_Mesh/meshGenerator.c:113-177) ---- */
int  or_mesh_structured(int M, int N, double x0, double y0, double x1, double y1,
                        int left_tilt, double *x, double *y, int *ien);

/* ---- numbering and connectivity ---- */
/* Fill_LM for NDOF dofs per node (01_SS_.../Fill_LM.c:3-27, 03_Euler_.../Fill_LM.c:3-31).
 * type[node*ndof+k] == 0 marks a Dirichlet dof; invp[node*ndof+k] its equation. */
void or_fill_lm(int nel, int ndof, const int *ien, const int *type, const int *invp,
                int NEQ, int *lm);

/* Adjacency of the free dofs of 1-dof meshes, sorted rows without duplicates
 * (Permutation_of_LM.c:21-49 + insertNode/mount_IA_JA :78-143).
 * IA has NEQ+1 entries; JA must hold up to nel*9 entries. Returns nnz. */
int  or_lm_adjacency(int nel, const int *ien, const int *type, const int *invp,
                     int NEQ, int *IA, int *JA);

/* Reverse Cuthill-McKee (00_CommonFiles/Reordering/symrcm.c:4-237). */
void or_symrcm(int n, const int *IA, const int *JA, int *perm);

/* Permutation_of_LM: adjacency + RCM + inverse (Permutation_of_LM.c:8-76).
 * Perm and invPerm have NEQ+1 entries; Perm[NEQ] = invPerm[NEQ] = NEQ.
 * bandwidth[0..1] receives MATRIX_bandwidth before and after (may be NULL). */
int  or_permutation_of_lm(int nel, const int *ien, const int *type, const int *invp,
                          int NEQ, int *Perm, int *invPerm, int *bandwidth);

/* MATRIX_bandwidth with the reference's stray ';' (reordering.c:215-236). */
int  or_matrix_bandwidth(int n, const int *IA, const int *JA);

/* ---- BLAS-1 (00_CommonFiles/BLAS_Operations) ---- */
double or_ddot(int n, const double *x, const double *y);

/* ---- EBE matvec ---- */
/* ebemv: 3x3 blocks through the local RCM permutation (EBE/ebemv.c:4-64). */
void or_ebemv3_perm(int nel, const int *lm, const double *A, const int *Perm,
                    const int *invPerm, int NEQ, const double *P, double *Q);
/* ebemvNDOF3 / ebemvNDOF4 / ebemv without permutation, S = 3, 9 or 12
 * (EBE/ebemvNDOF3.c:3-92, EBE/ebemvNDOF4.c:4-121). Q is zeroed first. */
void or_ebemv(int nel, int S, const int *lm, const double *A, int NEQ,
              const double *P, double *Q);

/* ---- preconditioners ---- */
/* Diag_precond_EBE_setup: Diag accumulates (never zeroed, as in the
 * reference), invDiag = 1/Diag, F *= invDiag (EBE/Diag_precond_EBE_setup.c:3-32). */
void or_diag_setup(int nel, int S, const int *lm, const double *A, int NEQ,
                   double *Diag, double *invDiag, double *F);
void or_diag_apply(int n, const double *invDiag, const double *p, double *z);
/* Left / LeftRight scaling of an EBE system (scaling.c:10-42, 92-121) on
 * the accumulating Diag; or_unscale is Left_unscaling (scaling.c:187-196). */
void or_scale_left(int nel, int S, const int *lm, double *A, int NEQ, double *Diag, double *invDiag, double *F);
void or_scale_leftright(int nel, int S, const int *lm, double *A, int NEQ, double *Diag, double *invDiag, double *F);
void or_unscale(int NEQ, const double *invDiag, double *x);

/* Nodal block-diagonal (B = NDOF = 3 or 4): gather the B x B diagonal blocks
 * of every element node (EBE/BlockDiag_precond_EBE_setup.c:57-80,
 * EBE/BlockDiagDOF3_precond_EBE_setup.c), invert with the reference's
 * closed-form cofactors (matrix_Inverse :90-147, DOF3_matrix_Inverse :84-124),
 * then F <- B^-1 F.  Id[node*B+k] is the equation of dof k (NEQ = sink).
 * ref_quirks != 0 reproduces the reference's 4x4 inverse term for entry 14. */
void or_blockdiag_setup(int nnodes, int nel, int B, const int *ien, const double *A,
                        const int *Id, int NEQ, int ref_quirks,
                        double *BlockDiag, double *invBlockDiag, double *F);
void or_blockdiag_apply(int nnodes, int B, const int *Id, int NEQ,
                        const double *invBlockDiag, double *p, double *z);
/* Block_scaling_EBE: Dirichlet rows/columns of the element blocks cleared
 * (diagonal 1), each node's row block multiplied by its inverse block. */
void or_block_scale(int nel, int B, const int *ien, const int *Id, int NEQ, const double *inv, double *A);

/* ---- GMRES (Solvers_and_Preconditioners/pgmres.c:5-200) ---- */
typedef int (*or_mv_fn)(void *ctx, double *P, double *Q);      /* Q = A P, vectors NEQ+1 */
typedef int (*or_pc_fn)(void *ctx, double *p, double *z);      /* owned slice, may alias */
int or_pgmres(int NEQ, int kmax, int lmax, double tol,
              or_mv_fn mv, or_pc_fn precond, void *ctx,
              double *B, double *X, int *iterations);

/* ---- element preconditioners "LUe" / "SGSe" (EBE/LU_precond_EBE*.c,
 * EBE/SGS_precond_EBE*.c), 3x3 blocks, z (NEQ+1) in place ---- */
void or_lue_setup(int nel, const double *A, double *LUe);
void or_lue_apply(int nel, const int *lm, int NEQ, const double *LUe, double *z);
void or_sgs_fwd(int nel, const int *lm, int NEQ, const double *A, double *z);
void or_sgs_bwd(int nel, const int *lm, int NEQ, const double *A, double *z);
/* set-up (F <- M^-1 F) + pgmres with the left / right pair: kind 1 LUe,
 * kind 2 SGSe.  Returns GMRES iterations. */
int or_ebe_elem_solve(int kind, int nel, const int *lm, const double *A, int NEQ, const int *Perm,
                      const int *invPerm, double *F, int kmax, int lmax, double tol, double *X);

/* One linear solve of an assembled EBE system (S = 3B) with the nodal
 * block-diagonal preconditioner: set-up (F preconditioned in place), then
 * pgmres.  Returns GMRES iterations. */
int or_ebe_block_solve(int nnodes, int nel, int B, const int *ien, const int *lm, const double *A,
                       const int *Id, int NEQ, int ref_quirks, double *F, int kmax, int lmax,
                       double tol, double *X);

/* ---- steady SUPG/CAU transport (01_SS_Transport_Equation) ---- */
typedef struct {
    double k;            /* Condutivity() for kx and ky                      */
    double gamma;        /* Reaction()                                       */
    double beta[2];      /* Velocity(): constant field                       */
    double f;            /* Font(): constant source                          */
    const double *upresc;/* Dirichlet value per node (read where type == 0)  */
    int cau;             /* 1: CAU, 2: CAUDD (DD form only), 3: YZBeta, 0: none */
    int form;            /* 0: SUPG, 1: DD (StabilizationForm)               */
    int h_shock;         /* 0: 2sqrtArea, 1: Option1, 2: Option2             */
    double *Re_old, *delta_old; /* [nel] YZBeta state, NULL: fresh zeros    */
} or_transport_problem;

/* Build_K_F_SUPG + CAU_ShockCapture + h_shock_2sqrtArea + F_assembly +
 * ebe_assembly (Build_K_F_SUPG.c:4-187).  u is the current solution of the
 * free dofs (length neq).  A receives 9 doubles per element, f neq doubles. */
void or_build_k_f_supg(int nnodes, int nel, const double *x, const double *y,
                       const int *type, const int *invp, const int *ien, int neq,
                       const or_transport_problem *prob, const double *u,
                       double *A, double *f);

/* Steady transport Process loop (01_SS_.../Process.c:6-93) with EBE storage,
 * ebemv with local RCM, Diag preconditioner and GMRES.  U has NEQ+1 slots and
 * holds the result.  Returns the number of nonlinear iterations. */
int or_transport_process(int nnodes, int nel, const double *x, const double *y,
                         const int *type, const int *invp, const int *ien, int neq,
                         const or_transport_problem *prob,
                         double solver_tol, double nonlinear_tol, int kmax, int lmax,
                         int max_nonlinear, double *U, int *gmres_iterations);

/* One linear solve of an assembled EBE system with Diag preconditioning:
 * setup (accumulating Diag as the reference does), then pgmres.  With
 * Perm == NULL the unpermuted matvec is used.  Returns GMRES iterations. */
int or_ebe_diag_solve(int nel, int S, const int *lm, const double *A, int NEQ,
                      const int *Perm, const int *invPerm,
                      double *Diag, double *invDiag, double *F,
                      int kmax, int lmax, double tol, double *X);

/* ---- steady Navier-Stokes, SUPG/PSPG/LSIC (04_SS_NavierStokes_Equations) ---- */
typedef struct {
    double reynolds;       /* ReynoldsNumber (density 1, viscosity 1/Re)             */
    const double *upresc;  /* [3*nnodes] prescribed u, v, p (read where type == 0)   */
    const double *f1, *f2; /* [nnodes] body force at the nodes (NULL = 0)            */
    int form;              /* 0: SUPG-PSPG, 1: VMS-DCDD (StabilizationForm)           */
} or_ns_problem;

/* Build_K_F_SUPG_PSPG (Picard tangent) + eval_U + ebe_assembly.  u holds the
 * free dofs (neq); A receives 81 doubles per element (row-major), F the
 * residual (NEQ+1 slots, sink 0). */
void or_build_ns(int nnodes, int nel, const double *x, const double *y, const int *type,
                 const int *invp, const int *ien, int neq, const or_ns_problem *prob,
                 const double *u, double *A, double *F);

/* Build_K_F_VMS_DCDD (oracle/ns_vms.c); or_build_ns calls it for form 1. */
void or_build_ns_vms(int nnodes, int nel, const double *x, const double *y, const int *type,
                     const int *invp, const int *ien, int neq, const or_ns_problem *prob,
                     const double *u, double *A, double *F);

/* Picard loop of 04_SS_NavierStokes_Equations/2D/01_CommonFiles/Process.c:6-62
 * with EBE 9x9 blocks, BlockDiagDOF3 and GMRES: build, set up, solve for the
 * increment s, u += s, until ||s|| / ||u|| <= nonlinear_tol.  Returns the
 * number of nonlinear iterations; *last_delta receives ||s|| / ||u||. */
int or_ns_process(int nnodes, int nel, const double *x, const double *y, const int *type,
                  const int *invp, const int *ien, int neq, const or_ns_problem *prob,
                  double solver_tol, double nonlinear_tol, int kmax, int lmax, int max_nonlinear,
                  double *u, int *gmres_iterations, double *last_delta);

/* ---- compressible Euler, SUPG + CAU (03_Euler_Equations) ---- */
typedef struct {
    double gamma;          /* FemFunctions->gamma (constant)                          */
    double mach;           /* Parameters->Mach (dimensionless Jacobians)               */
    int dimensionless;     /* 1: dimensionless_Ax_Ay_calculations, 0: dimensional      */
    double tolerance;      /* StabilizationTolerance (CAU switch on |grad U|)          */
    double alpha, dt;      /* Alpha_Build, DeltaT_Build                                */
    const double *upresc;  /* [4*nnodes] prescribed rho, rho u, rho v, rho E           */
    int form;              /* 0: SUPG + CAU, 1: DD (Build_M_K_F_DD_Transiente + Delta_DD) */
    double *uB, *delta_old;/* DD state: [4*nel] bubbles, [nel] delta (NULL: fresh zeros) */
    const double *invY;    /* [4] Parameters->invY of YZBeta (NULL: 1, 1, 1, 1)        */
    int shock;             /* 0: the form's own (CAU / CAUDD); 3: YZBeta (Delta_YZBeta) */
} or_euler_problem;

/* Build_M_K_F_SUPG + Delta_CAU + eval_U_dU + ebe_assembly: A receives the
 * 144 entries of Me + alpha dt Ke per element, R the residual -M dU - K U
 * (NEQ+1 slots, sink 0).  u, du: free dofs (neq). */
void or_build_euler(int nnodes, int nel, const double *x, const double *y, const int *type,
                    const int *invp, const int *ien, int neq, const or_euler_problem *prob,
                    const double *u, const double *du, double *A, double *R);

/* TimeIntegration "Predictor2" with StabilizationForm "DD" and ShockCapture
 * "YZBeta": Build_M_F_DD_Transiente (four bubble unknowns per element kept,
 * uB and duB [4*nel], condensed out with N2 = MBB + alpha dt KBB), Me into
 * A (144 per element), the load into F (NEQ + 1, sink 0), cond (invN2, R2[4],
 * M2[4][12]: 53 per element).  dnmv [nel] is Delta_YZBetaNMV's relaxed
 * state (NULL: fresh zeros). */
void or_build_euler_mfdd(int nnodes, int nel, const double *x, const double *y, const int *type,
                         const int *invp, const int *ien, int neq, const or_euler_problem *prob,
                         const double *u, const double *du, const double *uB, const double *duB, double *dnmv,
                         double *A, double *F, double *cond);
/* calculate_DaB of the Euler driver: Da[NEQ] = 0, DaB (4 per element) */
void or_euler_dab(int nel, const int *lm, int NEQ, const double *cond, double *Da, double *DaB);

/* Stop tests of 00_CommonFiles/Time_Integration/Criteria.c */
typedef struct {
    int stop_by_norm;      /* 0: StopByIterations, 1: StopByNorm                      */
    int max_corrections;   /* NonLinearMaxIter                                          */
    double correction_tol; /* NonLinearTolerance                                        */
    int steady_state;      /* 0: StopByTime, 1: StopBySteadyState                      */
    double final_time;     /* FinalTime                                                 */
    double time_tol;       /* TimeIntegrationTolerance                                  */
    int max_steps;         /* bound on the time steps (0: none; not in the reference)   */
    int scheme;            /* OR_TIME_PREDICTOR, OR_TIME_BDF, OR_TIME_TRBDF2 or
                              OR_TIME_NEW_BDF (Predictor_New_BDF's u loop)           */
} or_time_opts;

enum { OR_TIME_PREDICTOR = 0, OR_TIME_BDF = 1, OR_TIME_TRBDF2 = 2, OR_TIME_NEW_BDF = 4 };

typedef struct {
    int steps, corrections, gmres_iterations;
    double t;
} or_time_stats;

/* One correction of a time loop (oracle/time_loop.c): Build at (u, a) with
 * Alpha_Build = alpha_b and DeltaT_Build = dt_b, preconditioner set-up on
 * the residual, GMRES for Da (neq + 1 entries); *gmres receives the
 * iterations.  Non-zero return aborts the loop. */
typedef int (*or_correction_fn)(void *ctx, double alpha_b, double dt_b, const double *u, const double *a,
                                double *Da, int *gmres);
/* Predictor_Old, Predictor_Old_BDF or (bubble-free) Predictor_New_TRBDF2 by
 * to->scheme; u: initial state in, final state out; a: du/dt out.  Returns
 * the steps (a TR-BDF2 step is its TR and BDF2 stages), -1 on failure. */
int or_time_integrate(int neq, double alpha, double dt, const or_time_opts *to, or_correction_fn correct,
                      void *ctx, double *u, double *a, or_time_stats *st);
/* The same with the bubble operations of the Predictor2 loops
 * (Predictor_New.c, Predictor_New_BDF.c, Predictor_New_TRBDF2.c), called
 * where those loops act on their per-element unknowns uB, aB (the
 * correction of uB, aB from Da stays in `correct`):
 *   OR_B_PREDICT        uB += c1 aB, aB = 0
 *   OR_B_TRBDF2_START   uB = the element centroid of u (uB_InitialSolution)
 *   OR_B_TRBDF2_COMBINE uB = c1 uB - c2 uB_old, aB = 0
 *   OR_B_TRBDF2_SAVE    uB_old = uB
 *   OR_B_BDF_START      uB1 = uB, aB = 0
 *   OR_B_BDF_SAVE2      uB2 = uB
 *   OR_B_BDF_COMBINE    uB = c1 uB2 - c2 uB1, aB = 0
 *   OR_B_BDF_SHIFT      uB1 = uB2, uB2 = uB */
enum { OR_B_PREDICT = 0, OR_B_TRBDF2_START, OR_B_TRBDF2_COMBINE, OR_B_TRBDF2_SAVE, OR_B_BDF_START,
       OR_B_BDF_SAVE2, OR_B_BDF_COMBINE, OR_B_BDF_SHIFT };
typedef void (*or_bubble_fn)(void *ctx, int op, double c1, double c2, const double *u);
int or_time_integrate_ex(int neq, double alpha, double dt, const or_time_opts *to, or_correction_fn correct,
                         or_bubble_fn bubble, void *ctx, double *u, double *a, or_time_stats *st);

/* Predictor_Old.c:6-134 with EBE 12x12 blocks, BlockDiag (4x4, the
 * reference's inverse) and GMRES.  u: initial state on entry (the
 * problem's InitialSolution), final state on return; a: du/dt on return. */
int or_euler_predictor(int nnodes, int nel, const double *x, const double *y, const int *type,
                       const int *invp, const int *ien, int neq, const or_euler_problem *prob,
                       const or_time_opts *to, double solver_tol, int kmax, int lmax,
                       double *u, double *a, or_time_stats *st);
/* Predictor_New (to->scheme OR_TIME_PREDICTOR), Predictor_New_BDF
 * (OR_TIME_NEW_BDF) or Predictor_New_TRBDF2 (OR_TIME_TRBDF2) with
 * Build_M_F_DD_Transiente, calculate_DaB, BlockDiag (the reference's 4x4
 * inverse) and GMRES.  u: initial state in, final out; a (neq), uB, aB
 * (4 nel) receive the final du/dt and bubble unknowns. */
int or_euler_predictor2(int nnodes, int nel, const double *x, const double *y, const int *type,
                        const int *invp, const int *ien, int neq, const or_euler_problem *prob,
                        const or_time_opts *to, double solver_tol, int kmax, int lmax,
                        double *u, double *a, double *uB, double *aB, or_time_stats *st);

/* ---- transient SUPG/CAU transport (02_Transport_Equation, oracle/tt.c) ----
 * Build_M_K_R_SUPG: A receives Ae = me + alpha dt ke (9 per element), R the
 * residual F - me du - ke u (NEQ + 1 entries, R[NEQ] = 0); u, du: free dofs. */
void or_build_tt(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                 const int *ien, int neq, const or_transport_problem *prob, double alpha, double dt,
                 const double *u, const double *du, double *A, double *R);
/* Predictor_Old with Build_M_K_R_SUPG, ebemv on the local RCM numbering,
 * accumulating Diag and GMRES.  u: initial state in, final state out; a
 * (neq) receives du/dt. */
int or_tt_predictor(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                    const int *ien, int neq, const or_transport_problem *prob, double alpha, double dt,
                    const or_time_opts *to, double solver_tol, int kmax, int lmax, double *u, double *a,
                    or_time_stats *st);

/* Build_M_F_DD (TimeIntegration "Predictor2" with StabilizationForm "DD"):
 * the bubble unknown of each element kept (uB, duB: nel values) and
 * condensed out; A receives Me (9 per element), F the load (NEQ + 1, F[NEQ]
 * = 0), cond (invN2, R2, M2[0..2]) 5 per element.  prob->delta_old (nel)
 * holds the relaxed shock-capture state (NULL: fresh zeros). */
void or_build_tt_mfdd(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                      const int *ien, int neq, const or_transport_problem *prob, double alpha, double dt,
                      const double *u, const double *du, const double *uB, const double *duB, double *A,
                      double *F, double *cond);
/* calculate_DaB: Da[NEQ] = 0, DaB[e] = invN2 (R2 - M2 . Da[lm[e]]) */
void or_tt_dab(int nel, const int *lm, int NEQ, const double *cond, double *Da, double *DaB);
/* Predictor_New with Build_M_F_DD, calculate_DaB, accumulating Diag and
 * GMRES (the time-step stop tests of to; to->scheme is ignored).  u:
 * initial state in, final out; a (neq), uB, aB (nel) receive the final
 * du/dt and bubble unknowns. */
int or_tt_predictor2(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                     const int *ien, int neq, const or_transport_problem *prob, double alpha, double dt,
                     const or_time_opts *to, double solver_tol, int kmax, int lmax, double *u, double *a,
                     double *uB, double *aB, or_time_stats *st);

/* h_shock_2sqrtArea (opt 0), h_shock_Option1 (1), h_shock_Option2 (2) of the
 * transport drivers (oracle/sst.c). */
double or_h_shock(int opt, double bx, double by, double u1, double u2, double u3, double y23, double y31,
                  double y12, double x32, double x13, double x21, double Area);

/* ---- assembled CSR path and ILU(0) (oracle/csr_ilu.c) ---- */
int  or_csr_pattern(int nel, const int *ien, const int *type, const int *invp, int NEQ,
                    const int *Perm, const int *invPerm, int *IA, int *JA);
void or_csr_assemble(int nel, int S, const int *lm, const double *A, int NEQ,
                     const int *IA, const int *JA, double *AA);
void or_csrmv(int n, const int *IA, const int *JA, const double *AA, const double *P, double *Q);
int  or_ilu0_factor(int n, const int *IA, const int *JA, const double *AA, double *LU, double *D);
/* ILU(p) (oracle/ilup.c): symbolic pass to a factor CSR (per row: L
 * ascending, diagonal, U in the reference's order), numeric factorisation,
 * substitutions. */
int  or_ilup_symbolic(int n, const int *IA, const int *JA, int p, int **FIA, int **FJA, int **FDG);
int  or_ilup_factor(int n, const int *IA, const int *JA, const double *AA, const int *FIA, const int *FJA,
                    const int *FDG, double *LU, double *D);
void or_ilup_apply(int n, const int *FIA, const int *FJA, const int *FDG, const double *LU, const double *D,
                   const double *y, double *x);
void or_ilu0_apply(int n, const int *IA, const int *JA, const double *LU, const double *D,
                   const double *y, double *x);

/* truncated SPIKE over CSR row blocks (spike.c) */
typedef struct or_spike or_spike;
int  or_spike_blocks(int n, int k, int parts);
or_spike *or_spike_setup(int n, const int *IA, const int *JA, const double *AA, int k, int parts, int *err);
void or_spike_apply(const or_spike *sp, const double *f, double *y);
int  or_spike_info(const or_spike *sp, int *k, int *bs, int *kl, int *ku);
void or_spike_free(or_spike *sp);

#ifdef __cplusplus
}
#endif
#endif
