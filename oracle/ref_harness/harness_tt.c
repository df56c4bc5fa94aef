/*
 * Checker harness around the reference's own transient-transport build
 * (02_Transport_Equation/2D/01_CommonFiles: Build_M_K_R_SUPG.c,
 * Build_M_K_R_DD.c with their shock-capture and h_shock functions and
 * eval_U_dU.c), compiled by oracle/Makefile (target "ref_tt") from a
 * private copy of those sources whose TranspEquation.h includes the MPI
 * stand-in instead of </usr/include/mpi/mpi.h> (its line 8; nothing else
 * is changed).
 *
 * The structs are filled for one rank (neq_bef = 0, NEQ = neq, EBE
 * storage) and the reference's own Fill_LM and Build function are called
 * at the given state (u, du) with Alpha_Build and DeltaT_Build.  The
 * function pointers are installed as setStabilizationForm.c installs them
 * (the file is not linked: it pulls in the time-integration loops);
 * setProblem is supplied here, the same synthetic problem as the steady
 * harness.  Used only by tests.
 *
 * "Predictor2" (fr_tt_mfdd_build, fr_tt_predictor2): Build_M_F_DD.c and
 * calculate_DaB.c, and the reference's own Predictor_New loop with its
 * Criteria, pgmres, ebemv and Diag preconditioner compiled from the same
 * private copy.
 */
#include "TranspEquation.h"

int Build_M_K_R_SUPG(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *);
int Build_M_K_R_DD(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *);
double CAU_ShockCapture(double, double, double, double, double, double, double, double, double, double, double,
                        double, double, double, double, double, double, double, double);
double CAU_DD_ShockCapture(double, double, double, double, double, double, double, double, double, double, double,
                           double, double, double, double, double, double, double, double);
double YZBeta_ShockCapture(double, double, double, double, double, double, double, double, double, double, double,
                           double, double, double, double, double, double, double, double);
double h_shock_2sqrtArea(double, double, double, double, double, double, double, double, double, double, double,
                         double);
double h_shock_Option1(double, double, double, double, double, double, double, double, double, double, double,
                       double);
double h_shock_Option2(double, double, double, double, double, double, double, double, double, double, double,
                       double);
void ebe_assembly(ParametersType *, MatrixDataType *, FemStructsType *, int, double (*)[3]);

/* ---- synthetic problem (constant data, the steady harness's rule for the Dirichlet values) ---- */
static double g_k, g_gamma, g_bx, g_by, g_f, g_upval, g_xmin, g_ymin;
static int g_upmode;

static double syn_k(void) { return g_k; }
static double syn_gamma(void) { return g_gamma; }
static double syn_font(double X, double Y, double k, double gm, double bx, double by)
{ (void)X; (void)Y; (void)k; (void)gm; (void)bx; (void)by; return g_f; }
static void syn_vel(double X, double Y, double B[2]) { (void)X; (void)Y; B[0] = g_bx; B[1] = g_by; }
static double syn_upresc(double X, double Y)
{
    if (g_upmode == 1) return g_upval;
    return (X <= g_xmin + 1e-12 || Y <= g_ymin + 1e-12) ? 1.0 : 0.0;
}

/* form 0 "SUPG" / 1 "DD"; shock 1 "CAU" / 2 "CAUDD" / 3 "YZBeta";
 * h_shock 0 "2sqrtArea" / 1 "Option1" / 2 "Option2" */
static int g_form, g_shock = 1, g_hshock;
void fr_tt_set_form(int form, int shock, int hshock)
{
    g_form = form;
    g_shock = shock;
    g_hshock = hshock;
}

/* One build of the transient transport driver at (u, du): A (9 per
 * element, row-major, Ae = me + alpha dt ke as ebe_assembly stores it) and
 * R (neq).  delta_old (DD's relaxed CAUDD coefficient per element) starts
 * at 0, as the time loop allocates it; `builds` builds run in a row at the
 * same state (the DD state advances), the last one is returned. */
int fr_tt_build(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                const int *ien, int neq, double k, double gamma, double bx, double by, double f, int upmode,
                double upval, double alpha, double dt, const double *u, const double *du, int builds,
                double *A_out, double *R_out)
{
    ParametersType P;
    MatrixDataType M;
    FemStructsType S;
    FemFunctionsType F;
    int I;
    memset(&P, 0, sizeof P);
    memset(&M, 0, sizeof M);
    memset(&S, 0, sizeof S);
    memset(&F, 0, sizeof F);
    g_k = k; g_gamma = gamma; g_bx = bx; g_by = by; g_f = f; g_upmode = upmode; g_upval = upval;
    g_xmin = x[0]; g_ymin = y[0];
    for (I = 1; I < nnodes; I++) {
        if (x[I] < g_xmin) g_xmin = x[I];
        if (y[I] < g_ymin) g_ymin = y[I];
    }
    strcpy(P.MatrixVectorProductScheme, "EBE");
    P.nnodes = P.nNodes = nnodes;
    P.nel = P.nEl = nel;
    P.neq = neq;
    P.NEQ = neq;
    P.NPROC = 1;
    P.Alpha = P.Alpha_Build = alpha;
    P.DeltaT = P.DeltaT_Build = dt;
    F.Condutivity = syn_k;
    F.Reaction = syn_gamma;
    F.Font = syn_font;
    F.Velocity = syn_vel;
    F.upresc = syn_upresc;
    F.assembly = ebe_assembly;
    F.ShockCapture = g_shock == 3 ? YZBeta_ShockCapture : g_shock == 2 ? CAU_DD_ShockCapture : CAU_ShockCapture;
    F.h_shock = g_hshock == 2 ? h_shock_Option2 : g_hshock == 1 ? h_shock_Option1 : h_shock_2sqrtArea;

    NodeType *Node = calloc((size_t)nnodes, sizeof(NodeType));
    ElementType *El = calloc((size_t)nel, sizeof(ElementType));
    for (I = 0; I < nnodes; I++) {
        Node[I].x = x[I];
        Node[I].y = y[I];
        Node[I].Type = type[I];
        Node[I].Send = 1;
        Node[I].invP_id = type[I] == 0 ? -1 : invp[I];
    }
    for (I = 0; I < nel; I++) {
        El[I].Vertex[0] = ien[3 * I];
        El[I].Vertex[1] = ien[3 * I + 1];
        El[I].Vertex[2] = ien[3 * I + 2];
    }
    int **lm = calloc((size_t)nel, sizeof(int *));
    int *lmaux = calloc((size_t)nel * 3, sizeof(int));
    for (I = 0; I < nel; I++) lm[I] = &lmaux[3 * I];
    double **A = calloc((size_t)nel, sizeof(double *));
    double *Aaux = calloc((size_t)nel * 9, sizeof(double));
    for (I = 0; I < nel; I++) A[I] = &Aaux[9 * I];
    S.Node = Node;
    S.Element = El;
    S.lm = lm;
    S.lmaux = lmaux;
    S.F = calloc((size_t)neq + 1, sizeof(double));
    S.u = calloc((size_t)neq + 1, sizeof(double));
    S.du = calloc((size_t)neq + 1, sizeof(double));
    S.delta_old = calloc((size_t)nel + 1, sizeof(double));
    memcpy(S.u, u, sizeof(double) * (size_t)neq);
    memcpy(S.du, du, sizeof(double) * (size_t)neq);
    M.A = A;
    M.Aaux = Aaux;
    Fill_LM(&P, lm, Node, El);
    for (I = 0; I < builds; I++) {
        if (g_form == 1) Build_M_K_R_DD(&P, &M, &S, &F);
        else Build_M_K_R_SUPG(&P, &M, &S, &F);
    }
    memcpy(A_out, Aaux, sizeof(double) * 9 * (size_t)nel);
    memcpy(R_out, S.F, sizeof(double) * (size_t)neq);
    free(Node); free(El); free(lm); free(lmaux); free(A); free(Aaux);
    free(S.F); free(S.u); free(S.du); free(S.delta_old);
    return 0;
}

/* ---- TimeIntegration "Predictor2" with StabilizationForm "DD" ----
 * setStabilizationForm.c:51-54 installs Build_M_F_DD and Predictor_New.
 * fr_tt_mfdd_build: one Build_M_F_DD at (u, du, uB, duB) with a fresh
 * delta_old, then calculate_DaB on the caller's Da (NEQ + 1; its sink is
 * set to 0 there).  A (9 per element), F (NEQ + 1), cond (invN2, R2,
 * M2[0..2] per element) and DaB (nel) are returned. */
int Build_M_F_DD(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *);
int calculate_DaB(ParametersType *, FemStructsType *, double *, double *);
int Predictor_New(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *, FemOtherFunctionsType *);
void setStopCriteria(ParametersType *, FemFunctionsType *);
int pgmres(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *, double *, double *);
int ebemv(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int Diag_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int NO_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
int Diag_precond_EBE_setup(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);

typedef struct {
    ParametersType P;
    MatrixDataType M;
    FemStructsType S;
    FemFunctionsType F;
    FemOtherFunctionsType O;
} fr_tt;

static const double *g_init;
static int syn_init(ParametersType *P, NodeType *Node, double *u)
{
    (void)Node;
    memcpy(u, g_init, sizeof(double) * (size_t)P->neq);
    return 0;
}

static void fr_tt_setup(fr_tt *c, int nnodes, int nel, const double *x, const double *y, const int *type,
                        const int *invp, const int *ien, int neq, double k, double gamma, double bx, double by,
                        double f, int upmode, double upval, double alpha, double dt)
{
    int I;
    memset(c, 0, sizeof(*c));
    g_k = k; g_gamma = gamma; g_bx = bx; g_by = by; g_f = f; g_upmode = upmode; g_upval = upval;
    g_xmin = x[0]; g_ymin = y[0];
    for (I = 1; I < nnodes; I++) {
        if (x[I] < g_xmin) g_xmin = x[I];
        if (y[I] < g_ymin) g_ymin = y[I];
    }
    strcpy(c->P.MatrixVectorProductScheme, "EBE");
    strcpy(c->P.StabilizationForm, "DD");
    strcpy(c->P.TimeIntegration, "Predictor2");
    strcpy(c->P.Preconditioner, "Diag");
    c->P.nnodes = c->P.nNodes = nnodes;
    c->P.nel = c->P.nEl = nel;
    c->P.neq = neq;
    c->P.NEQ = neq;
    c->P.NPROC = 1;
    c->P.Alpha = c->P.Alpha_Build = alpha;
    c->P.DeltaT = c->P.DeltaT_Build = dt;
    c->F.Condutivity = syn_k;
    c->F.Reaction = syn_gamma;
    c->F.Font = syn_font;
    c->F.Velocity = syn_vel;
    c->F.upresc = syn_upresc;
    c->F.InitialSolution = syn_init;
    c->F.assembly = ebe_assembly;
    c->F.ShockCapture = g_shock == 3 ? YZBeta_ShockCapture : CAU_DD_ShockCapture;
    c->F.h_shock = g_hshock == 2 ? h_shock_Option2 : g_hshock == 1 ? h_shock_Option1 : h_shock_2sqrtArea;
    /* setPreconditioner.c:10-15 ("Diag", EBE); the transient driver never
     * sets precondR, which pgmres.c:61,93,186 calls: the identity here, as
     * the other drivers install it (NO_precond) */
    c->F.mv = ebemv;
    c->F.precond = Diag_precond;
    c->F.precondR = NO_precond;
    c->F.precond_setup = Diag_precond_EBE_setup;
    c->O.Build = Build_M_F_DD;
    c->O.solver = pgmres;
    NodeType *Node = calloc((size_t)nnodes, sizeof(NodeType));
    ElementType *El = calloc((size_t)nel, sizeof(ElementType));
    for (I = 0; I < nnodes; I++) {
        Node[I].x = x[I];
        Node[I].y = y[I];
        Node[I].Type = type[I];
        Node[I].Send = 1;
        Node[I].invP_id = type[I] == 0 ? -1 : invp[I];
    }
    for (I = 0; I < nel; I++) {
        El[I].Vertex[0] = ien[3 * I];
        El[I].Vertex[1] = ien[3 * I + 1];
        El[I].Vertex[2] = ien[3 * I + 2];
    }
    c->S.Node = Node;
    c->S.Element = El;
    c->S.lm = calloc((size_t)nel, sizeof(int *));
    c->S.lmaux = calloc((size_t)nel * 3, sizeof(int));
    for (I = 0; I < nel; I++) c->S.lm[I] = &c->S.lmaux[3 * I];
    c->M.A = calloc((size_t)nel, sizeof(double *));
    c->M.Aaux = calloc((size_t)nel * 9, sizeof(double));
    for (I = 0; I < nel; I++) c->M.A[I] = &c->M.Aaux[9 * I];
    c->M.Diag = calloc((size_t)neq + 1, sizeof(double));
    c->M.invDiag = calloc((size_t)neq + 1, sizeof(double));
    c->S.F = calloc((size_t)neq + 1, sizeof(double));
    c->S.u = calloc((size_t)neq + 1, sizeof(double));
    Fill_LM(&c->P, c->S.lm, Node, El);
}

static void fr_tt_free(fr_tt *c)
{
    free(c->S.Node); free(c->S.Element); free(c->S.lm); free(c->S.lmaux); free(c->M.A); free(c->M.Aaux);
    free(c->M.Diag); free(c->M.invDiag); free(c->S.F); free(c->S.u);
}

int fr_tt_mfdd_build(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                     const int *ien, int neq, double k, double gamma, double bx, double by, double f, int upmode,
                     double upval, double alpha, double dt, const double *u, const double *du, const double *uB,
                     const double *duB, const double *Da, double *A_out, double *F_out, double *cond_out,
                     double *DaB_out)
{
    fr_tt c;
    AuxBuildStructuresType Aux;
    int I;
    fr_tt_setup(&c, nnodes, nel, x, y, type, invp, ien, neq, k, gamma, bx, by, f, upmode, upval, alpha, dt);
    memset(&Aux, 0, sizeof Aux);
    double *R2aux = calloc((size_t)nel, sizeof(double)), *M2aux = calloc((size_t)nel * 3, sizeof(double));
    double **R2 = calloc((size_t)nel, sizeof(double *)), **M2 = calloc((size_t)nel, sizeof(double *));
    for (I = 0; I < nel; I++) { R2[I] = &R2aux[I]; M2[I] = &M2aux[3 * I]; }
    Aux.R2 = R2;
    Aux.M2 = M2;
    Aux.invN2 = calloc((size_t)nel, sizeof(double));
    c.S.AuxBuild = &Aux;
    c.S.du = calloc((size_t)neq + 1, sizeof(double));
    c.S.uB = calloc((size_t)nel, sizeof(double));
    c.S.duB = calloc((size_t)nel, sizeof(double));
    c.S.delta_old = calloc((size_t)nel, sizeof(double));
    memcpy(c.S.u, u, sizeof(double) * (size_t)neq);
    memcpy(c.S.du, du, sizeof(double) * (size_t)neq);
    memcpy(c.S.uB, uB, sizeof(double) * (size_t)nel);
    memcpy(c.S.duB, duB, sizeof(double) * (size_t)nel);
    Build_M_F_DD(&c.P, &c.M, &c.S, &c.F);
    double *Dac = calloc((size_t)neq + 1, sizeof(double));
    memcpy(Dac, Da, sizeof(double) * ((size_t)neq + 1));
    calculate_DaB(&c.P, &c.S, Dac, DaB_out);
    memcpy(A_out, c.M.Aaux, sizeof(double) * 9 * (size_t)nel);
    memcpy(F_out, c.S.F, sizeof(double) * ((size_t)neq + 1));
    for (I = 0; I < nel; I++) {
        cond_out[5 * I] = Aux.invN2[I];
        cond_out[5 * I + 1] = R2[I][0];
        cond_out[5 * I + 2] = M2[I][0];
        cond_out[5 * I + 3] = M2[I][1];
        cond_out[5 * I + 4] = M2[I][2];
    }
    free(Dac); free(R2aux); free(M2aux); free(R2); free(M2); free(Aux.invN2);
    free(c.S.du); free(c.S.uB); free(c.S.duB); free(c.S.delta_old);
    fr_tt_free(&c);
    return 0;
}

/* The reference's own Predictor_New loop with Build_M_F_DD, Diag and
 * pgmres (EBE on the caller's local RCM permutation Perm / invPerm, NEQ + 1
 * each).  topt: stop_by_norm, max_corrections, correction_tol,
 * steady_state, final_time, time_tol; solver: kmax, lmax, tol.  u_out
 * (neq) receives the final state; returns the GMRES iterations. */
int fr_tt_predictor2(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                     const int *ien, int neq, double k, double gamma, double bx, double by, double f, int upmode,
                     double upval, double alpha, double dt, const int *Perm, const int *invPerm,
                     const double *init, const double *topt, int kmax, int lmax, double tol, double *u_out)
{
    fr_tt c;
    fr_tt_setup(&c, nnodes, nel, x, y, type, invp, ien, neq, k, gamma, bx, by, f, upmode, upval, alpha, dt);
    c.M.Perm = (int *)Perm;
    c.M.invPerm = (int *)invPerm;
    g_init = init;
    strcpy(c.P.StopMulticorrection, topt[0] != 0.0 ? "NORM" : "ITERATION");
    c.P.NonLinearMaxIter = (int)topt[1];
    c.P.NonLinearTolerance = topt[2];
    strcpy(c.P.StopAtSteadyState, topt[3] != 0.0 ? "YES" : "NO");
    c.P.FinalTime = topt[4];
    c.P.TimeIntegrationTolerance = topt[5];
    c.P.KrylovBasisVectorsQuantity = kmax;
    c.P.LinearMaxIter = lmax;
    c.P.SolverTolerance = tol;
    c.P.iterations = 0;
    setStopCriteria(&c.P, &c.F);
    Predictor_New(&c.P, &c.M, &c.S, &c.F, &c.O);
    memcpy(u_out, c.S.u, sizeof(double) * (size_t)neq);
    int its = c.P.iterations;
    fr_tt_free(&c);
    return its;
}

/* Predictor_Old (TimeIntegration "Predictor1") with the form's build
 * (Build_M_K_R_SUPG or Build_M_K_R_DD, setStabilizationForm.c:8-45), Diag
 * and pgmres; arguments as fr_tt_predictor2. */
int Predictor_Old(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *, FemOtherFunctionsType *);
int fr_tt_predictor1(int nnodes, int nel, const double *x, const double *y, const int *type, const int *invp,
                     const int *ien, int neq, double k, double gamma, double bx, double by, double f, int upmode,
                     double upval, double alpha, double dt, const int *Perm, const int *invPerm,
                     const double *init, const double *topt, int kmax, int lmax, double tol, double *u_out)
{
    fr_tt c;
    fr_tt_setup(&c, nnodes, nel, x, y, type, invp, ien, neq, k, gamma, bx, by, f, upmode, upval, alpha, dt);
    strcpy(c.P.TimeIntegration, "Predictor1");
    strcpy(c.P.StabilizationForm, g_form == 1 ? "DD" : "SUPG");
    c.O.Build = g_form == 1 ? Build_M_K_R_DD : Build_M_K_R_SUPG;
    if (g_form != 1) c.F.ShockCapture = g_shock == 3 ? YZBeta_ShockCapture : CAU_ShockCapture;
    c.M.Perm = (int *)Perm;
    c.M.invPerm = (int *)invPerm;
    g_init = init;
    strcpy(c.P.StopMulticorrection, topt[0] != 0.0 ? "NORM" : "ITERATION");
    c.P.NonLinearMaxIter = (int)topt[1];
    c.P.NonLinearTolerance = topt[2];
    strcpy(c.P.StopAtSteadyState, topt[3] != 0.0 ? "YES" : "NO");
    c.P.FinalTime = topt[4];
    c.P.TimeIntegrationTolerance = topt[5];
    c.P.KrylovBasisVectorsQuantity = kmax;
    c.P.LinearMaxIter = lmax;
    c.P.SolverTolerance = tol;
    c.P.iterations = 0;
    setStopCriteria(&c.P, &c.F);
    Predictor_Old(&c.P, &c.M, &c.S, &c.F, &c.O);
    memcpy(u_out, c.S.u, sizeof(double) * (size_t)neq);
    int its = c.P.iterations;
    fr_tt_free(&c);
    return its;
}

/* Field offsets of the reference's transient-transport structs, the same
 * list the drop-in shim reports (layout pin). */
#include <stddef.h>
void fr_tt_layout(long *out)
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
