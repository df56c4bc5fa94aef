/*
 * Drop-in shim for the multi-dof drivers, compiled twice by the package
 * build: -DFGC_NS gives libfemgpu_ns.so for the steady Navier-Stokes driver
 * (ebemvNDOF3, BlockDiagDOF3_precond and its EBE set-up), -DFGC_EULER gives
 * libfemgpu_euler.so for the Euler driver (ebemvNDOF4, BlockDiag_precond
 * and its EBE set-up).  Both also export pgmres, Diag_precond,
 * Diag_precond_EBE_setup, NO_precond and NO_precond_setup, with the
 * reference's names and signatures, running on the GPU through libfemgpu,
 * and for MatrixVectorProductScheme "CSR" csr_assembly, csrmv,
 * ILUp_precond(_setup) ("ILU<p>") and SPIKE_precond(_setup) ("SPIKEk").
 * Linking one of them instead of the reference's pgmres.c,
 * MatrixVector_Operations/EBE/ebemvNDOF*.c, CSR/csrmv.c, the driver's
 * csr_assembly.c and the preconditioner files leaves every driver file
 * (Process.c, Predictor_Old.c, the Build functions) unchanged.  The BLAS-1
 * helpers the drivers call on host arrays (ddot.c, daxpy.c, ...) stay the
 * driver's own.
 *
 * One rank only (NPROC = 1): neq_bef = 0, NEQ = neq, vectors of NEQ + 1.
 * The GPU system of a MatrixDataType is created on first use from the
 * driver's Node/Element arrays and cached in a small table keyed by the
 * MatrixDataType pointer: EBE storage keeps the node numbering (as
 * setMatrixVectorProductType.c requires), CSR storage uses the reference's
 * RCM renumbering unless Parameters->reordering is "NOT".  CSR storage:
 * csr_assembly keeps each element's block (the library sums the blocks
 * into its CSR values in element order), so MatrixData->AA is not filled;
 * every consumer of AA on the solve path is in this shim.  SPIKE's
 * row-block count (the reference's rank count) is FEMGPU_SPIKE_BLOCKS
 * (default 16); FEMGPU_ILU_BLOCKS (default 1) gives block-Jacobi ILU over
 * that many row blocks, as that many ranks would factorise.  Errors print
 * the library's message and exit(1) as the reference does, unless
 * FEMGPU_COMPAT_NO_EXIT is set.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#if defined(FGC_NS)
#include "femgpu_ref_ns.h"
#define FGC_MV ebemvNDOF3
#define FGC_BD_APPLY BlockDiagDOF3_precond
#define FGC_BD_SETUP BlockDiagDOF3_precond_EBE_setup
#define FGC_BD_FLAGS 0
#define FGC_LAYOUT fgc_ns_layout
#elif defined(FGC_EULER)
#include "femgpu_ref_euler.h"
#define FGC_MV ebemvNDOF4
#define FGC_BD_APPLY BlockDiag_precond
#define FGC_BD_SETUP BlockDiag_precond_EBE_setup
/* BlockDiag_precond_EBE_setup.c's matrix_Inverse, entry-14 term included */
#define FGC_BD_FLAGS FG_SETUP_REF_QUIRKS
#define FGC_LAYOUT fgc_euler_layout
#else
#error "define FGC_NS or FGC_EULER"
#endif
#include "../../include/femgpu.h"

#define FGC_S (3 * FGC_NDOF)
#define FGC_MAX_SYSTEMS 64

static struct {
    const MatrixDataType *key;
    fg_system *sys;
    int nel, neq;
    double *blocks;     /* CSR storage: element blocks captured by csr_assembly */
    int csr;            /* the system runs on the CSR operator */
} g_tab[FGC_MAX_SYSTEMS];

static int fgc_slot(const MatrixDataType *M)
{
    for (int i = 0; i < FGC_MAX_SYSTEMS; i++)
        if (g_tab[i].key == M) return i;
    return -1;
}

static int fgc_fail(int rc, const char *where)
{
    fprintf(stderr, "femgpu (%s): %s\n", where, fg_last_error());
    if (!getenv("FEMGPU_COMPAT_NO_EXIT")) exit(1);
    return rc;
}

static fg_system *fgc_system(ParametersType *P, MatrixDataType *M, FemStructsType *S)
{
    int i, k, free_slot = -1;
    for (i = 0; i < FGC_MAX_SYSTEMS; i++) {
        if (g_tab[i].key == M && g_tab[i].nel == P->nel && g_tab[i].neq == P->neq) return g_tab[i].sys;
        if (!g_tab[i].key && free_slot < 0) free_slot = i;
    }
    if (P->NPROC > 1 || P->neq_bef != 0) {
        fprintf(stderr, "femgpu: the GPU solve path replaces the MPI decomposition (one rank only)\n");
        if (!getenv("FEMGPU_COMPAT_NO_EXIT")) exit(1);
        return NULL;
    }
    if (free_slot < 0) { fprintf(stderr, "femgpu: too many systems\n"); return NULL; }
    int nn = P->nnodes, ne = P->nel;
    int *type = malloc(sizeof(int) * FGC_NDOF * (size_t)nn), *invp = malloc(sizeof(int) * FGC_NDOF * (size_t)nn);
    int *ien = malloc(sizeof(int) * 3 * (size_t)ne);
    for (i = 0; i < nn; i++)
        for (k = 0; k < FGC_NDOF; k++) {
            int t = S->Node[i].Type[k];
            type[FGC_NDOF * i + k] = t == 0 ? 0 : 1;
            invp[FGC_NDOF * i + k] = t == 0 ? -1 : S->Node[i].invP_id[k];
        }
    for (i = 0; i < ne; i++) {
        ien[3 * i] = S->Element[i].Vertex[0];
        ien[3 * i + 1] = S->Element[i].Vertex[1];
        ien[3 * i + 2] = S->Element[i].Vertex[2];
    }
    fg_system *sys = NULL;
    const int csr = strcasecmp(P->MatrixVectorProductScheme, "CSR") == 0;
    const int reorder = csr && strcasecmp(P->reordering, "NOT") != 0 ? FG_REORDER_RCM : FG_REORDER_NONE;
    int rc = fg_system_create(&sys, nn, ne, FGC_NDOF, ien, type, invp, P->neq, reorder);
    free(type); free(invp); free(ien);
    if (rc) { fgc_fail(rc, "system set-up"); return NULL; }
    g_tab[free_slot].key = M;
    g_tab[free_slot].sys = sys;
    g_tab[free_slot].nel = ne;
    g_tab[free_slot].neq = P->neq;
    g_tab[free_slot].blocks = NULL;
    g_tab[free_slot].csr = 0;
    if (csr) {
        g_tab[free_slot].blocks = calloc((size_t)ne * FGC_S * FGC_S, sizeof(double));
        if (!g_tab[free_slot].blocks) { fgc_fail(FG_ERR_NOMEM, "CSR block buffer"); return NULL; }
    }
    return sys;
}

/* Element blocks as the Build function left them: nel rows of S*S in Aaux
 * (EBE), or as csr_assembly captured them (CSR). */
static int fgc_upload_blocks(fg_system *sys, MatrixDataType *M)
{
    int i = fgc_slot(M);
    const double *blk = i >= 0 && g_tab[i].blocks ? g_tab[i].blocks : M->Aaux;
    int rc = fg_set_blocks(sys, blk);
    if (!rc && i >= 0 && g_tab[i].blocks && !g_tab[i].csr) {
        rc = fg_set_operator(sys, FG_OP_CSR);
        if (!rc) g_tab[i].csr = 1;
    }
    return rc ? fgc_fail(rc, "element blocks") : 0;
}

int NO_precond(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *p, double *z)
{
    (void)P; (void)M; (void)S; (void)p; (void)z;
    return 0;
}

int NO_precond_setup(ParametersType *P, MatrixDataType *M, FemStructsType *S, int tag, double *F)
{
    (void)tag; (void)F;
    fg_system *sys = fgc_system(P, M, S);
    if (!sys || fgc_upload_blocks(sys, M)) return 1;
    int rc = fg_precond_setup(sys, FG_PRECOND_NONE, 0, NULL);
    return rc ? fgc_fail(rc, "NO_precond_setup") : 0;
}

/* Diag_precond_EBE_setup.c:3-32: Diag accumulates in MatrixData->Diag */
int Diag_precond_EBE_setup(ParametersType *P, MatrixDataType *M, FemStructsType *S, int tag, double *F)
{
    (void)tag;
    fg_system *sys = fgc_system(P, M, S);
    if (!sys || fgc_upload_blocks(sys, M)) return 1;
    int rc = fg_set_diag(sys, M->Diag);
    if (!rc) rc = fg_precond_setup(sys, FG_PRECOND_DIAG, FG_SETUP_ACCUMULATE, F);
    if (!rc) rc = fg_get_diag(sys, M->Diag);
    if (rc) return fgc_fail(rc, "Diag_precond_EBE_setup");
    for (int i = 0; i < P->NEQ; i++) M->invDiag[i] = 1.0 / M->Diag[i];
    return 0;
}

/* Nodal block-diagonal set-up: blocks gathered from A, inverted, F <- B^-1 F.
 * The inverses stay on the device (the drivers never read
 * MatrixData->invBlockDiag themselves). */
int FGC_BD_SETUP(ParametersType *P, MatrixDataType *M, FemStructsType *S, int tag, double *F)
{
    (void)tag;
    fg_system *sys = fgc_system(P, M, S);
    if (!sys || fgc_upload_blocks(sys, M)) return 1;
    int rc = fg_precond_setup(sys, FG_PRECOND_BLOCKDIAG, FGC_BD_FLAGS, F);
    return rc ? fgc_fail(rc, "block-diagonal set-up") : 0;
}

static int fgc_apply(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *p, double *z, const char *w)
{
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    double keep = p[P->neq];
    p[P->neq] = 0.0;
    int rc = fg_precond_apply(sys, p, z);
    if (z != p) p[P->neq] = keep;
    return rc ? fgc_fail(rc, w) : 0;
}

int FGC_BD_APPLY(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *p, double *z)
{
    return fgc_apply(P, M, S, p, z, "block-diagonal apply");
}

int Diag_precond(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *p, double *z)
{
    return fgc_apply(P, M, S, p, z, "Diag_precond");
}

/* Q = A P over NEQ + 1 entries (Q[NEQ] = 0), as ebemvNDOF3.c / ebemvNDOF4.c */
int FGC_MV(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *Pv, double *Qv)
{
    fg_system *sys = fgc_system(P, M, S);
    if (!sys || fgc_upload_blocks(sys, M)) return 1;
    Pv[P->NEQ] = 0.0;
    int rc = fg_matvec(sys, Pv, Qv, 64);
    return rc ? fgc_fail(rc, "EBE matvec") : 0;
}

/* csr_assembly (EU and NS csr_assembly.c): the element's S x S block is
 * kept; the library sums the blocks into its CSR values in element order
 * when a CSR consumer below runs. */
void csr_assembly(ParametersType *P, MatrixDataType *M, FemStructsType *S, int E, double (*Me)[FGC_S])
{
    if (!fgc_system(P, M, S)) return;
    int i = fgc_slot(M);
    if (i < 0 || !g_tab[i].blocks || E < 0 || E >= g_tab[i].nel) return;
    double *b = g_tab[i].blocks + (size_t)E * FGC_S * FGC_S;
    for (int a = 0; a < FGC_S; a++)
        for (int c = 0; c < FGC_S; c++) b[FGC_S * a + c] = Me[a][c];
}

/* csrmv (MatrixVector_Operations/CSR/csrmv.c:4-65): Q = A P, Q[NEQ] = 0. */
int csrmv(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *Pv, double *Qv)
{
    fg_system *sys = fgc_system(P, M, S);
    if (!sys || fgc_upload_blocks(sys, M)) return 1;
    Pv[P->NEQ] = 0.0;
    int rc = fg_matvec(sys, Pv, Qv, 64);
    return rc ? fgc_fail(rc, "csrmv") : 0;
}

/* ILUp_precond_setup (CSR/ILUp_precond_setup.c:8-168) for "ILU<p>": ILU(p)
 * of the CSR operator (p = atoi(&Preconditioner[3]), capped at neq as the
 * reference caps it), F preconditioned in place. */
int ILUp_precond_setup(ParametersType *P, MatrixDataType *M, FemStructsType *S, int tag, double *F)
{
    (void)tag;
    int p = atoi(&P->Preconditioner[3]);
    if (p > P->neq) p = P->neq;
    fg_system *sys = fgc_system(P, M, S);
    if (!sys || fgc_upload_blocks(sys, M)) return 1;
    const char *e = getenv("FEMGPU_ILU_BLOCKS");
    int rc = fg_set_ilu_fill(sys, p > 16 ? 16 : p);
    if (!rc) rc = fg_set_ilu_blocks(sys, e && atoi(e) > 0 ? atoi(e) : 1);
    if (!rc) rc = fg_precond_setup(sys, FG_PRECOND_ILU0, 0, F);
    return rc ? fgc_fail(rc, "ILUp_precond_setup") : 0;
}

/* ILUp_precond (CSR/ILUp_precond.c:4-47): z = (LU)^-1 p (p may be z). */
int ILUp_precond(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *p, double *z)
{
    return fgc_apply(P, M, S, p, z, "ILUp_precond");
}

/* SPIKE_precond_setup (CSR/SPIKE_precond_setup.c:10-312): k from the
 * "SPIKEk" string as the reference reads it (:54), the row blocks from
 * FEMGPU_SPIKE_BLOCKS; F preconditioned in place. */
int SPIKE_precond_setup(ParametersType *P, MatrixDataType *M, FemStructsType *S, int tag, double *F)
{
    (void)tag;
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    int k = atoi(&P->Preconditioner[5]);
    const char *e = getenv("FEMGPU_SPIKE_BLOCKS");
    int rc = fg_set_spike(sys, k, e ? atoi(e) : 16);
    if (rc) return fgc_fail(rc, "SPIKE_precond_setup");
    if (fgc_upload_blocks(sys, M)) return 1;
    rc = fg_precond_setup(sys, FG_PRECOND_SPIKE, 0, F);
    if (rc) return fgc_fail(rc, "SPIKE_precond_setup");
    P->k_SPIKE_block_size = k;
    return 0;
}

/* SPIKE_precond (CSR/SPIKE_precond.c:8-158): z = M^-1 p (p may be z). */
int SPIKE_precond(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *p, double *z)
{
    return fgc_apply(P, M, S, p, z, "SPIKE_precond");
}

/* pgmres (pgmres.c:5-200) on the GPU when mv is this shim's matvec (EBE or
 * CSR) and the preconditioner is one of this shim's; the blocks and the
 * preconditioner come from the *_setup call that precedes every solve (NS
 * Process.c:37-38, Predictor_Old.c:95-96).  Parameters->iterations grows by
 * the Arnoldi steps. */
int pgmres(ParametersType *P, MatrixDataType *M, FemStructsType *S, FemFunctionsType *Fn, double *B, double *X)
{
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    const int ebe_ok = Fn->mv == FGC_MV &&
                       (Fn->precond == FGC_BD_APPLY || Fn->precond == Diag_precond || Fn->precond == NO_precond);
    const int csr_ok = Fn->mv == csrmv && (Fn->precond == ILUp_precond || Fn->precond == SPIKE_precond ||
                                           Fn->precond == NO_precond);
    if ((Fn->precondR && Fn->precondR != NO_precond) || !(ebe_ok || csr_ok)) {
        fprintf(stderr, "femgpu: pgmres supports this shim's EBE or CSR matvec and preconditioners on the GPU\n");
        if (!getenv("FEMGPU_COMPAT_NO_EXIT")) exit(1);
        return 1;
    }
    fg_solver_opts o;
    o.kmax = P->KrylovBasisVectorsQuantity;
    o.lmax = P->LinearMaxIter;
    o.tol = P->SolverTolerance;
    o.precision = FG_PREC_FP64;
    o.inner_tol = 0.0;
    fg_solve_stats st;
    memset(&st, 0, sizeof st);
    int rc = fg_solve(sys, &o, B, X, NULL, &st);
    if (rc) return fgc_fail(rc, "pgmres");
    P->iterations += st.iterations;
    return 0;
}

/* Layout pin: sizes and the offsets the shim reads (compared with the
 * reference's own header by the tests). */
#include <stddef.h>
void FGC_LAYOUT(long *out)
{
    int i = 0;
    out[i++] = (long)sizeof(ParametersType);
    out[i++] = (long)offsetof(ParametersType, SolverTolerance);
    out[i++] = (long)offsetof(ParametersType, KrylovBasisVectorsQuantity);
    out[i++] = (long)offsetof(ParametersType, nnodes);
    out[i++] = (long)offsetof(ParametersType, nel);
    out[i++] = (long)offsetof(ParametersType, neq);
    out[i++] = (long)offsetof(ParametersType, neq_bef);
    out[i++] = (long)offsetof(ParametersType, NEQ);
    out[i++] = (long)offsetof(ParametersType, iterations);
    out[i++] = (long)offsetof(ParametersType, RANK);
    out[i++] = (long)offsetof(ParametersType, NPROC);
    out[i++] = (long)offsetof(ParametersType, LinearMaxIter);
    out[i++] = (long)offsetof(ParametersType, PardisoVariables);
    out[i++] = (long)sizeof(MatrixDataType);
    out[i++] = (long)offsetof(MatrixDataType, Aaux);
    out[i++] = (long)offsetof(MatrixDataType, Diag);
    out[i++] = (long)offsetof(MatrixDataType, invDiag);
    out[i++] = (long)offsetof(MatrixDataType, Id);
    out[i++] = (long)offsetof(MatrixDataType, A_SPIKE);
    out[i++] = (long)sizeof(FemStructsType);
    out[i++] = (long)offsetof(FemStructsType, Node);
    out[i++] = (long)offsetof(FemStructsType, Element);
    out[i++] = (long)offsetof(FemStructsType, IdRecv_aft);
    out[i++] = (long)sizeof(FemFunctionsType);
    out[i++] = (long)offsetof(FemFunctionsType, mv);
    out[i++] = (long)offsetof(FemFunctionsType, precond);
    out[i++] = (long)offsetof(FemFunctionsType, precondR);
    out[i++] = (long)offsetof(FemFunctionsType, precond_setup);
    out[i++] = (long)sizeof(NodeType);
    out[i++] = (long)offsetof(NodeType, invP_id);
    out[i++] = (long)sizeof(ElementType);
}
