/*
 * Drop-in shim for the multi-dof drivers, compiled twice by the package
 * build: -DFGC_NS gives libfemgpu_ns.so for the steady Navier-Stokes driver
 * (ebemvNDOF3, BlockDiagDOF3_precond and its EBE set-up), -DFGC_EULER gives
 * libfemgpu_euler.so for the Euler driver (ebemvNDOF4, BlockDiag_precond
 * and its EBE set-up).  Both also export pgmres, Diag_precond,
 * Diag_precond_EBE_setup, NO_precond and NO_precond_setup, with the
 * reference's names and signatures, running on the GPU through libfemgpu.
 * Linking one of them instead of the reference's pgmres.c,
 * MatrixVector_Operations/EBE/ebemvNDOF*.c and the preconditioner files
 * leaves every driver file (Process.c, Predictor_Old.c, the Build
 * functions) unchanged.  The BLAS-1 helpers the drivers call on host arrays
 * (ddot.c, daxpy.c, ...) stay the driver's own.
 *
 * One rank only (NPROC = 1): neq_bef = 0, NEQ = neq, vectors of NEQ + 1.
 * The GPU system of a MatrixDataType is created on first use from the
 * driver's Node/Element arrays (EBE storage: no reordering, as
 * setMatrixVectorProductType.c requires) and cached in a small table keyed
 * by the MatrixDataType pointer.  Errors print the library's message and
 * exit(1) as the reference does, unless FEMGPU_COMPAT_NO_EXIT is set.
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
} g_tab[FGC_MAX_SYSTEMS];

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
    int rc = fg_system_create(&sys, nn, ne, FGC_NDOF, ien, type, invp, P->neq, FG_REORDER_NONE);
    free(type); free(invp); free(ien);
    if (rc) { fgc_fail(rc, "system set-up"); return NULL; }
    g_tab[free_slot].key = M;
    g_tab[free_slot].sys = sys;
    g_tab[free_slot].nel = ne;
    g_tab[free_slot].neq = P->neq;
    return sys;
}

/* Element blocks as the Build function left them: nel rows of S*S in Aaux */
static int fgc_upload_blocks(fg_system *sys, MatrixDataType *M)
{
    int rc = fg_set_blocks(sys, M->Aaux);
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

/* pgmres (pgmres.c:5-200) on the GPU when mv is this shim's matvec and the
 * preconditioner is one of this shim's; the blocks and the preconditioner
 * come from the *_setup call that precedes every solve (NS Process.c:37-38,
 * Predictor_Old.c:95-96).  Parameters->iterations grows by the Arnoldi steps. */
int pgmres(ParametersType *P, MatrixDataType *M, FemStructsType *S, FemFunctionsType *Fn, double *B, double *X)
{
    fg_system *sys = fgc_system(P, M, S);
    if (!sys) return 1;
    if (Fn->mv != FGC_MV || Fn->precondR != NO_precond ||
        (Fn->precond != FGC_BD_APPLY && Fn->precond != Diag_precond && Fn->precond != NO_precond)) {
        fprintf(stderr, "femgpu: pgmres supports this shim's EBE matvec and preconditioners on the GPU\n");
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
