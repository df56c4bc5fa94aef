/*
 * Drop-in shim for the steady-transport driver: the reference's solve-path
 * entry points, with the reference's names and signatures, running on the
 * GPU through libfemgpu.  Linking this library instead of
 * pgmres.c, ebemv.c, Diag_precond.c, EBE/Diag_precond_EBE_setup.c,
 * EBE/LU_precond_EBE*.c, EBE/SGS_precond_EBE*.c ("LUe", "SGSe"),
 * NO_precond.c and NO_precond_setup.c (EBE storage) or csr_assembly.c,
 * csrmv.c, CSR/ILUp_precond*.c and CSR/SPIKE_precond*.c (MatrixVector-
 * ProductScheme "CSR" with "ILU0" or "SPIKEk") leaves every driver file
 * unchanged.
 *
 * CSR storage: the shim's csr_assembly keeps each element's 3x3 block (the
 * library assembles its CSR values from the blocks, in csr_assembly.c's
 * element order), so MatrixData->AA is not filled; every consumer of AA on
 * the solve path (csrmv, the ILU and SPIKE set-ups and applies, pgmres) is
 * in this shim.  SPIKE's row-block count (the reference's rank count) is
 * FEMGPU_SPIKE_BLOCKS (default 16).
 *
 * One rank only (NPROC = 1): neq_bef = 0, NEQ = neq, vectors of NEQ + 1.
 * The GPU system of a MatrixDataType is created on first use from the
 * driver's Node/Element arrays and cached in a small table keyed by the
 * MatrixDataType pointer (the reference's structs have no room for it).
 *
 * Built with -DFGC_TT the same shim serves the transient-transport driver
 * (02_Transport_Equation: its structs, femgpu_ref_tt.h; its solve path is
 * pgmres, ebemv, Diag and NO; that driver never sets precondR, which the
 * reference's pgmres calls, and the shim reads a NULL precondR as none).
 *
 * Errors: the reference prints and stops (mycalloc.c:10-13,
 * setPreconditioner.c:66-69).  The shim prints the library's message and
 * calls exit(1) the same way, unless FEMGPU_COMPAT_NO_EXIT is set in the
 * environment, in which case it returns the non-zero status instead.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef FGC_TT
#include "femgpu_ref_tt.h"
#define FGC_LAYOUT fgc_tt_layout
#else
#include "femgpu_ref_sst.h"
#define FGC_LAYOUT fgc_sst_layout
#endif
#include "../../include/femgpu.h"

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

/* GPU system of this driver state (created on first use). */
static fg_system *fgc_system(ParametersType *P, MatrixDataType *M, FemStructsType *S)
{
    int i, free_slot = -1;
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
    int *type = malloc(sizeof(int) * (size_t)nn), *invp = malloc(sizeof(int) * (size_t)nn);
    int *ien = malloc(sizeof(int) * 3 * (size_t)ne);
    for (i = 0; i < nn; i++) {
        type[i] = S->Node[i].Type == 0 ? 0 : 1;
        invp[i] = S->Node[i].Type == 0 ? -1 : S->Node[i].invP_id;
    }
    for (i = 0; i < ne; i++) {
        ien[3 * i] = S->Element[i].Vertex[0];
        ien[3 * i + 1] = S->Element[i].Vertex[1];
        ien[3 * i + 2] = S->Element[i].Vertex[2];
    }
    fg_system *sys = NULL;
    int reorder = strcasecmp(P->reordering, "NOT") == 0 ? FG_REORDER_NONE : FG_REORDER_RCM;
    int rc = fg_system_create(&sys, nn, ne, 1, ien, type, invp, P->neq, reorder);
    free(type); free(invp); free(ien);
    if (rc) { fgc_fail(rc, "system set-up"); return NULL; }
    g_tab[free_slot].key = M;
    g_tab[free_slot].sys = sys;
    g_tab[free_slot].nel = ne;
    g_tab[free_slot].neq = P->neq;
    g_tab[free_slot].blocks = NULL;
    g_tab[free_slot].csr = 0;
    if (strcasecmp(P->MatrixVectorProductScheme, "CSR") == 0) {
        g_tab[free_slot].blocks = calloc((size_t)ne * 9, sizeof(double));
        if (!g_tab[free_slot].blocks) { fgc_fail(FG_ERR_NOMEM, "CSR block buffer"); return NULL; }
    }
    return sys;
}

/* Element blocks as Build_K_F_SUPG left them: nel rows of 9 in Aaux
 * (Preprocess.c:331-340 allocates A as row pointers into Aaux). */
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
    if (!sys) return 1;
    if (fgc_upload_blocks(sys, M)) return 1;
    int rc = fg_precond_setup(sys, FG_PRECOND_NONE, 0, NULL);
    return rc ? fgc_fail(rc, "NO_precond_setup") : 0;
}

/* Diag_precond_EBE_setup (EBE/Diag_precond_EBE_setup.c:3-32): Diag keeps
 * accumulating in MatrixData->Diag across calls, as in the reference;
 * invDiag is filled and F is preconditioned in place. */
int Diag_precond_EBE_setup(ParametersType *P, MatrixDataType *M, FemStructsType *S, int tag, double *F)
{
    (void)tag;
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    if (fgc_upload_blocks(sys, M)) return 1;
    int rc = fg_set_diag(sys, M->Diag);
    if (!rc) rc = fg_precond_setup(sys, FG_PRECOND_DIAG, FG_SETUP_ACCUMULATE, F);
    if (!rc) rc = fg_get_diag(sys, M->Diag);
    if (rc) return fgc_fail(rc, "Diag_precond_EBE_setup");
    for (int i = 0; i < P->NEQ; i++) M->invDiag[i] = 1.0 / M->Diag[i];
    return 0;
}

/* Diag_precond (Diag_precond.c:3-15), on the owned slice (p may be z). */
int Diag_precond(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *p, double *z)
{
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    double keep = p[P->neq];
    p[P->neq] = 0.0;
    int rc = fg_precond_apply(sys, p, z);
    if (z != p) p[P->neq] = keep;
    return rc ? fgc_fail(rc, "Diag_precond") : 0;
}

/* The element preconditioners (Preconditioner "LUe", "SGSe"; EBE
 * storage): LU_precond_EBE_setup (EBE/LU_precond_EBE_setup.c:4-35) and
 * SGS_precond_EBE_setup (EBE/SGS_precond_EBE_setup.c:4-12) build them from
 * the current blocks and precondition F in place; LU_precond_EBE,
 * SGS_precond_EBE and SGS_precondR_EBE apply them in place on the owned
 * slice (p is not read, as in the reference: the drivers pass p == z). */
static int fgc_elem_setup(ParametersType *P, MatrixDataType *M, FemStructsType *S, int kind, double *F,
                          const char *where)
{
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    if (fgc_upload_blocks(sys, M)) return 1;
    double keep = F[P->neq];
    F[P->neq] = 0.0;
    int rc = fg_precond_setup(sys, kind, 0, F);
    F[P->neq] = keep;
    return rc ? fgc_fail(rc, where) : 0;
}
static int fgc_elem_apply(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *z, int right,
                          const char *where)
{
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    z[P->neq] = 0.0;
    int rc = right ? fg_precond_apply_right(sys, z, z) : fg_precond_apply(sys, z, z);
    return rc ? fgc_fail(rc, where) : 0;
}
int LU_precond_EBE_setup(ParametersType *P, MatrixDataType *M, FemStructsType *S, int tag, double *F)
{
    (void)tag;
    return fgc_elem_setup(P, M, S, FG_PRECOND_LUE, F, "LU_precond_EBE_setup");
}
int LU_precond_EBE(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *p, double *z)
{
    (void)p;
    return fgc_elem_apply(P, M, S, z, 0, "LU_precond_EBE");
}
int SGS_precond_EBE_setup(ParametersType *P, MatrixDataType *M, FemStructsType *S, int tag, double *F)
{
    (void)tag;
    return fgc_elem_setup(P, M, S, FG_PRECOND_SGSE, F, "SGS_precond_EBE_setup");
}
int SGS_precond_EBE(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *p, double *z)
{
    (void)p;
    return fgc_elem_apply(P, M, S, z, 0, "SGS_precond_EBE");
}
int SGS_precondR_EBE(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *p, double *z)
{
    (void)p;
    return fgc_elem_apply(P, M, S, z, 1, "SGS_precondR_EBE");
}

/* ebemv (EBE/ebemv.c:4-64): Q = A P over NEQ + 1 entries; Q[NEQ] = 0. */
int ebemv(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *Pv, double *Qv)
{
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    if (fgc_upload_blocks(sys, M)) return 1;
    Pv[P->NEQ] = 0.0;
    int rc = fg_matvec(sys, Pv, Qv, 64);
    return rc ? fgc_fail(rc, "ebemv") : 0;
}

/* csr_assembly (csr_assembly.c:3-54): the element's block is kept; the
 * library sums the blocks into its CSR values in element order when a
 * CSR consumer below runs. */
void csr_assembly(ParametersType *P, MatrixDataType *M, FemStructsType *S, int E, double ke[3][3])
{
    if (!fgc_system(P, M, S)) return;
    int i = fgc_slot(M);
    if (i < 0 || !g_tab[i].blocks || E < 0 || E >= g_tab[i].nel) return;
    double *b = g_tab[i].blocks + (size_t)E * 9;
    for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++) b[3 * a + c] = ke[a][c];
}

/* csrmv (MatrixVector_Operations/CSR/csrmv.c:4-65): Q = A P, Q[NEQ] = 0. */
int csrmv(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *Pv, double *Qv)
{
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    if (fgc_upload_blocks(sys, M)) return 1;
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
    if (!sys) return 1;
    if (fgc_upload_blocks(sys, M)) return 1;
    int rc = fg_set_ilu_fill(sys, p > 16 ? 16 : p);
    if (!rc) rc = fg_precond_setup(sys, FG_PRECOND_ILU0, 0, F);
    return rc ? fgc_fail(rc, "ILUp_precond_setup") : 0;
}

/* ILUp_precond (CSR/ILUp_precond.c:4-47): z = (LU)^-1 p (p may be z). */
int ILUp_precond(ParametersType *P, MatrixDataType *M, FemStructsType *S, double *p, double *z)
{
    return Diag_precond(P, M, S, p, z);
}

/* SPIKE_precond_setup (CSR/SPIKE_precond_setup.c:10-312): k from the
 * "SPIKEk" string as the reference reads it (:54), the row blocks from
 * FEMGPU_SPIKE_BLOCKS; F preconditioned in place.  k_SPIKE_block_size
 * receives k, as in the reference. */
int SPIKE_precond_setup(ParametersType *P, MatrixDataType *M, FemStructsType *S, int tag, double *F)
{
    (void)tag;
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    int k = atoi(&P->Preconditioner[5]);
    const char *e = getenv("FEMGPU_SPIKE_BLOCKS");
    int parts = e ? atoi(e) : 16;
    int rc = fg_set_spike(sys, k, parts);
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
    return Diag_precond(P, M, S, p, z);
}

/* pgmres (Solvers_and_Preconditioners/pgmres.c:5-200): the whole restarted
 * GMRES on the GPU when mv is this shim's ebemv with its Diag_precond or
 * NO_precond, or its csrmv with its ILUp_precond, SPIKE_precond or
 * NO_precond (the configurations the steady-transport driver installs,
 * setPreconditioner.c:6-65); the blocks and the
 * preconditioner were set up by the *_setup call that precedes every solve
 * (Process.c:59-76).  Parameters->iterations grows by the Arnoldi steps. */
int pgmres(ParametersType *P, MatrixDataType *M, FemStructsType *S, FemFunctionsType *Fn, double *B, double *X)
{
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    const int right_none = !Fn->precondR || Fn->precondR == NO_precond;
    const int ebe_ok = Fn->mv == ebemv &&
                       (((Fn->precond == Diag_precond || Fn->precond == NO_precond || Fn->precond == LU_precond_EBE) &&
                         right_none) ||
                        (Fn->precond == SGS_precond_EBE && Fn->precondR == SGS_precondR_EBE));
    const int csr_ok = Fn->mv == csrmv && right_none &&
                       (Fn->precond == ILUp_precond || Fn->precond == SPIKE_precond || Fn->precond == NO_precond);
    if (!(ebe_ok || csr_ok)) {
        fprintf(stderr, "femgpu: pgmres supports mv = ebemv with Diag, LUe, SGSe (with its right sweep) or no "
                        "preconditioning, or mv = csrmv with ILU(p), SPIKE or no preconditioning, on the GPU\n");
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

/* Field offsets of the restated structs (layout pin, compared with the
 * reference's own header by the tests). */
#include <stddef.h>
void FGC_LAYOUT(long *out)
{
    out[0] = (long)sizeof(ParametersType);
    out[1] = (long)offsetof(ParametersType, SolverTolerance);
    out[2] = (long)offsetof(ParametersType, KrylovBasisVectorsQuantity);
    out[3] = (long)offsetof(ParametersType, nnodes);
    out[4] = (long)offsetof(ParametersType, nel);
    out[5] = (long)offsetof(ParametersType, neq);
    out[6] = (long)offsetof(ParametersType, neq_bef);
    out[7] = (long)offsetof(ParametersType, NEQ);
    out[8] = (long)offsetof(ParametersType, LinearMaxIter);
    out[9] = (long)offsetof(ParametersType, iterations);
    out[10] = (long)offsetof(ParametersType, RANK);
    out[11] = (long)offsetof(ParametersType, NPROC);
    out[12] = (long)sizeof(MatrixDataType);
    out[13] = (long)offsetof(MatrixDataType, A);
    out[14] = (long)offsetof(MatrixDataType, Aaux);
    out[15] = (long)offsetof(MatrixDataType, Diag);
    out[16] = (long)offsetof(MatrixDataType, invDiag);
    out[17] = (long)offsetof(MatrixDataType, Perm);
    out[18] = (long)offsetof(MatrixDataType, invPerm);
    out[19] = (long)sizeof(FemStructsType);
    out[20] = (long)offsetof(FemStructsType, lm);
    out[21] = (long)offsetof(FemStructsType, lmaux);
    out[22] = (long)offsetof(FemStructsType, Node);
    out[23] = (long)offsetof(FemStructsType, Element);
    out[24] = (long)sizeof(FemFunctionsType);
    out[25] = (long)offsetof(FemFunctionsType, mv);
    out[26] = (long)offsetof(FemFunctionsType, precond);
    out[27] = (long)offsetof(FemFunctionsType, precondR);
    out[28] = (long)offsetof(FemFunctionsType, precond_setup);
    out[29] = (long)sizeof(NodeType);
    out[30] = (long)sizeof(ElementType);
    out[31] = (long)offsetof(MatrixDataType, AA);
    out[32] = (long)offsetof(MatrixDataType, JA);
    out[33] = (long)offsetof(MatrixDataType, IA);
    out[34] = (long)offsetof(ParametersType, MatrixVectorProductScheme);
    out[35] = (long)offsetof(ParametersType, Preconditioner);
    out[36] = (long)offsetof(ParametersType, nnzero);
}
