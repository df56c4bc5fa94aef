/*
 * Checker harness around the reference's own steady Navier-Stokes solve
 * path (04_SS_NavierStokes_Equations/2D/01_CommonFiles), compiled from the
 * reference sources by oracle/Makefile (target "ref").
 *
 * As for the transport driver, the reference's Preprocess needs partition
 * files, so this harness fills the structs for one rank (neq_bef = 0,
 * NEQ = neq, EBE storage as Preprocess.c:337-349 allocates it) and calls
 * the reference's own Fill_LM, Build_K_F_SUPG_PSPG, ebemvNDOF3,
 * BlockDiagDOF3_precond_EBE_setup and Process.  setProblem is supplied
 * here: the prescribed velocities and pressure and the body force are
 * the lid-driven-cavity rule of CAVITY/CAVITY_v1presc.c (u = 1 where
 * |y - 1| <= 1e-15) or, per field, the affine function a0 + a1 x + a2 y.
 *
 * Used only by tests.
 */
#include "SSNavierStokesEquations.h"
#include "solvers.h"
#include "preconditioners.h"
#include "matvec.h"

/* ---- synthetic problem (replaces the reference's setProblem.c) ---- */
/* fields: 0 v1, 1 v2, 2 p, 3 f1, 4 f2; g_lid makes v1 the cavity lid */
static double g_c[5][3];
static int g_lid;

static double affine(int k, double X, double Y) { return g_c[k][0] + g_c[k][1] * X + g_c[k][2] * Y; }
static double syn_v1(double X, double Y)
{
    if (g_lid) return fabs(Y - 1.0) <= 1e-15 ? 1.0 : 0.0;
    return affine(0, X, Y);
}
static double syn_v2(double X, double Y) { return affine(1, X, Y); }
static double syn_p(double X, double Y) { return affine(2, X, Y); }
static double syn_f1(double X, double Y) { return affine(3, X, Y); }
static double syn_f2(double X, double Y) { return affine(4, X, Y); }

int setProblem(ParametersType *P, FemFunctionsType *F)
{
    (void)P;
    F->v1presc = syn_v1;
    F->v2presc = syn_v2;
    F->ppresc = syn_p;
    F->f1ext = syn_f1;
    F->f2ext = syn_f2;
    return 0;
}

typedef struct {
    ParametersType P;
    MatrixDataType M;
    FemStructsType S;
    FemFunctionsType F;
    FemOtherFunctionsType O;
} fr_ns;

static int g_form;  /* 0: "SUPG-PSPG", 1: "VMS-DCDD" */

/* StabilizationForm of the following builds and Process runs. */
void fr_ns_set_form(int form) { g_form = form; }

static void fr_ns_setup(fr_ns *c, int nnodes, int nel, const double *x, const double *y,
                        const int *type, const int *invp, const int *ien, int neq, double Re,
                        double solver_tol, double nl_tol, int kmax, int lmax, int max_nl)
{
    int I, k;
    memset(c, 0, sizeof(*c));
    strcpy(c->P.ProblemTitle, "SYNTH");
    strcpy(c->P.Solver, "GMRES");
    strcpy(c->P.Preconditioner, "BlockDiag");
    strcpy(c->P.reordering, "NOT");
    strcpy(c->P.MatrixVectorProductScheme, "EBE");
    strcpy(c->P.StabilizationForm, g_form ? "VMS-DCDD" : "SUPG-PSPG");
    c->P.ReynoldsNumber = Re;
    c->P.SolverTolerance = solver_tol;
    c->P.NonLinearTolerance = nl_tol;
    c->P.NonLinearMaxIter = max_nl;
    c->P.LinearMaxIter = lmax;
    c->P.KrylovBasisVectorsQuantity = kmax;
    c->P.nnodes = c->P.nNodes = nnodes;
    c->P.nel = c->P.nEl = nel;
    c->P.neq = neq;
    c->P.neq_bef = 0;
    c->P.NEQ = neq;
    c->P.RANK = 0;
    c->P.NPROC = 1;

    NodeType *Node = calloc((size_t)nnodes, sizeof(NodeType));
    ElementType *El = calloc((size_t)nel, sizeof(ElementType));
    for (I = 0; I < nnodes; I++) {
        Node[I].x = x[I];
        Node[I].y = y[I];
        for (k = 0; k < NDOF; k++) {
            Node[I].Type[k] = type[NDOF * I + k];
            Node[I].Send[k] = 1;
            Node[I].invP_id[k] = type[NDOF * I + k] == 0 ? -1 : invp[NDOF * I + k];
        }
    }
    for (I = 0; I < nel; I++) {
        El[I].Vertex[0] = ien[3 * I];
        El[I].Vertex[1] = ien[3 * I + 1];
        El[I].Vertex[2] = ien[3 * I + 2];
        El[I].Type = -1;
    }
    double *F = calloc((size_t)neq + 1, sizeof(double));
    double *U = calloc((size_t)neq + 1, sizeof(double));
    int **lm = calloc((size_t)nel, sizeof(int *));
    int *lmaux = calloc((size_t)nel * 9, sizeof(int));
    for (I = 0; I < nel; I++) lm[I] = &lmaux[9 * I];
    c->S.Node = Node;
    c->S.Element = El;
    c->S.lm = lm;
    c->S.lmaux = lmaux;
    c->S.F = F;
    c->S.U = U;
    c->S.f = F;
    c->S.u = U;
    Fill_LM(&c->P, lm, Node, El);
    double **K = calloc((size_t)nel, sizeof(double *));
    double *Kaux = calloc((size_t)nel * 81, sizeof(double));
    for (I = 0; I < nel; I++) K[I] = &Kaux[81 * I];
    c->M.A = K;
    c->M.Aaux = Kaux;
    c->M.Diag = calloc((size_t)neq + 1, sizeof(double));
    c->M.invDiag = calloc((size_t)neq + 1, sizeof(double));
}

static void fr_ns_free(fr_ns *c)
{
    free(c->S.Node); free(c->S.Element); free(c->S.lm); free(c->S.lmaux);
    free(c->S.F); free(c->S.U);
    free(c->M.A); free(c->M.Aaux); free(c->M.Diag); free(c->M.invDiag);
    if (c->M.Id) { free(c->M.IdAux); free(c->M.Id); }
    if (c->M.BlockDiag) { free(c->M.BlockDiagAux); free(c->M.BlockDiag); }
    /* the set-up keeps only row pointers into its inverse array: row 0 is its start */
    if (c->M.invBlockDiag) { free(c->M.invBlockDiag[0]); free(c->M.invBlockDiag); }
}

static void fr_ns_problem(const double *coef, int lid)
{
    memcpy(g_c, coef, sizeof g_c);
    g_lid = lid;
}

/* Connectivity of the NS driver (Fill_LM, NDOF = 3). */
void fr_ns_lm(int nnodes, int nel, const double *x, const double *y, const int *type,
              const int *invp, const int *ien, int neq, int *lm_out)
{
    fr_ns c;
    fr_ns_setup(&c, nnodes, nel, x, y, type, invp, ien, neq, 1.0, 1e-10, 1e-3, 30, 10, 1);
    memcpy(lm_out, c.S.lmaux, sizeof(int) * 9 * (size_t)nel);
    fr_ns_free(&c);
}

/* One build (Build_K_F_SUPG_PSPG or Build_K_F_VMS_DCDD by the form) at the
 * free-dof state u (A: 81 per element). */
void fr_ns_build(int nnodes, int nel, const double *x, const double *y, const int *type,
                 const int *invp, const int *ien, int neq, double Re, const double *coef, int lid,
                 const double *u, double *A_out, double *F_out)
{
    fr_ns c;
    fr_ns_problem(coef, lid);
    fr_ns_setup(&c, nnodes, nel, x, y, type, invp, ien, neq, Re, 1e-10, 1e-3, 30, 10, 1);
    setProblem(&c.P, &c.F);
    setMatrixVectorProductType(&c.P, &c.F);
    setSolver(&c.P, &c.O);
    setPreconditioner(&c.P, &c.F);
    setStabilizationForm(&c.P, &c.F, &c.O);
    memcpy(c.S.u, u, sizeof(double) * (size_t)neq);
    c.O.Build(&c.P, &c.M, &c.S, &c.F);
    memcpy(A_out, c.M.Aaux, sizeof(double) * 81 * (size_t)nel);
    memcpy(F_out, c.S.F, sizeof(double) * ((size_t)neq + 1));
    fr_ns_free(&c);
}

/* BlockDiagDOF3_precond_EBE_setup (first call) on caller blocks; F in place. */
void fr_ns_blockdiag(int nnodes, int nel, const double *x, const double *y, const int *type,
                     const int *invp, const int *ien, int neq, const double *A, double *F,
                     double *inv_out)
{
    fr_ns c;
    int I;
    fr_ns_setup(&c, nnodes, nel, x, y, type, invp, ien, neq, 1.0, 1e-10, 1e-3, 30, 10, 1);
    memcpy(c.M.Aaux, A, sizeof(double) * 81 * (size_t)nel);
    BlockDiagDOF3_precond_EBE_setup(&c.P, &c.M, &c.S, 1, F);
    for (I = 0; I < nnodes; I++) memcpy(inv_out + 9L * I, c.M.invBlockDiag[I], 9 * sizeof(double));
    fr_ns_free(&c);
}

/* ebemvNDOF3 on caller blocks. */
void fr_ns_ebemv(int nnodes, int nel, const double *x, const double *y, const int *type,
                 const int *invp, const int *ien, int neq, const double *A, const double *P, double *Q)
{
    fr_ns c;
    fr_ns_setup(&c, nnodes, nel, x, y, type, invp, ien, neq, 1.0, 1e-10, 1e-3, 30, 10, 1);
    memcpy(c.M.Aaux, A, sizeof(double) * 81 * (size_t)nel);
    double *Pc = calloc((size_t)neq + 1, sizeof(double));
    memcpy(Pc, P, sizeof(double) * ((size_t)neq + 1));
    ebemvNDOF3(&c.P, &c.M, &c.S, Pc, Q);
    free(Pc);
    fr_ns_free(&c);
}

/* The whole Picard Process loop of the reference (BlockDiag, EBE, GMRES). */
int fr_ns_process(int nnodes, int nel, const double *x, const double *y, const int *type,
                  const int *invp, const int *ien, int neq, double Re, const double *coef, int lid,
                  double solver_tol, double nl_tol, int kmax, int lmax, int max_nl,
                  double *u_out, int *gmres_iterations)
{
    fr_ns c;
    fr_ns_problem(coef, lid);
    fr_ns_setup(&c, nnodes, nel, x, y, type, invp, ien, neq, Re, solver_tol, nl_tol, kmax, lmax, max_nl);
    c.P.iterations = 0;
    Process(&c.P, &c.M, &c.S, &c.F, &c.O);
    memcpy(u_out, c.S.u, sizeof(double) * (size_t)neq);
    *gmres_iterations = c.P.iterations;
    fr_ns_free(&c);
    return 0;
}

/* Layout pin: the same sizes and offsets the drop-in shim reports for its
 * restated structs (parallel_fem_codes_gb300/compat/compat_block.c). */
#include <stddef.h>
void fr_ns_layout(long *out)
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
