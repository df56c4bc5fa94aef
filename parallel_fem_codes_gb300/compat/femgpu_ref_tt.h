/*
 * Memory layout of the transient-transport driver's structs
 * (02_Transport_Equation/2D/01_CommonFiles/TranspEquation.h:16-183),
 * restated so the drop-in shim (compat_sst.c built with -DFGC_TT) compiles
 * without the reference tree.  The shim reads these structs by field
 * offset, so every field keeps the reference's type and order;
 * tests/test_compat_layout.py checks the offsets against the reference's own
 * header compiled by oracle/Makefile (target ref_tt).  The steady driver's
 * names for the same fields differ in ParametersType (no Scaling, and the
 * time-integration controls), MatrixDataType (no element-LU storage) and
 * FemStructsType (the time-loop state).
 */
#ifndef FEMGPU_REF_TT_H
#define FEMGPU_REF_TT_H

#define FGC_NDIM 2
#define FGC_NDOF 1

typedef struct {
    double x, y;
    int Type;
    int Send;
    int invP_id;
} NodeType;

typedef struct {
    int Vertex[FGC_NDIM + 1];
    int Type;
} ElementType;

typedef struct {
    void *A_pt[64];
    int A_iparm[64];
    double A_dparm[64];
    void *S_pt[64];
    int S_iparm[64];
    double S_dparm[64];
} PardisoVariablesType;

typedef struct {
    char ProblemTitle[200];
    char Solver[200];
    char Preconditioner[200];
    char reordering[200];
    char MatrixVectorProductScheme[200];
    char StabilizationForm[200];
    char ShockCapture[200];
    char h_Shock[200];
    char TimeIntegration[200];
    char StopMulticorrection[200];
    char StopAtSteadyState[200];
    double SolverTolerance;
    double NonLinearTolerance;
    double TimeIntegrationTolerance;
    double StabilizationTolerance;
    double FinalTime;
    double Alpha;
    double Alpha_Build;
    double DeltaT;
    double DeltaT_Build;
    double CurrentTime;
    int KrylovBasisVectorsQuantity;
    int nnodes, nNodes;
    int nel, nEl;
    int neq, neq_bef, neqaux_bef, neqaux_aft;
    int nsend_bef, nsend_aft, nrecv_bef, nrecv_aft;
    int NEQ;
    int nedge;
    int nnzero;
    int nnzero_bef;
    int nnzero_aft;
    int NonLinearMaxIter;
    int LinearMaxIter;
    int iterations;
    int k_SPIKE_block_size;
    int bandwidth_bef, bandwidth_aft;
    int RANK;
    int NPROC;
    PardisoVariablesType *PardisoVariables;
} ParametersType;

/* ILU and SPIKE types are held by pointer only */
typedef struct fgc_opaque_ilu SparILU;
typedef struct fgc_opaque_sparmat SparMAT;
typedef struct fgc_opaque_mat MAT;

typedef struct {
    double **A;
    double *Aaux;
    double *AA;
    double *AA_bef;
    double *AA_aft;
    double *Diag;
    double *invDiag;
    int **Scheme_by_Element;
    int **Scheme_by_Element_bef;
    int **Scheme_by_Element_aft;
    int **order;
    int *JA;
    int *IA;
    int *JA_bef;
    int *IA_bef;
    int *JA_aft;
    int *IA_aft;
    int *aux_bef;
    int *aux_aft;
    SparILU *ILUp;
    SparMAT *mat;
    MAT *Ailu;
    int *Perm;
    int *invPerm;
    double **fullC;
    double *fullCaux;
    double **fullB;
    double *fullBaux;
    MAT *A_SPIKE, *B_SPIKE, *C_SPIKE, *S_SPIKE;
} MatrixDataType;

typedef struct {
    double **M2, **R2, *invN2, *delta_old_NMV;
    double tolerance;
} AuxBuildStructuresType;

typedef struct {
    int **lm;
    int *lmaux;
    NodeType *Node;
    ElementType *Element;
    double *F;
    double *U;
    double *u;
    double *du;
    double *f;
    double *uB;
    double *duB;
    double *delta_old;
    AuxBuildStructuresType *AuxBuild;
    double *SendBuffer_bef[2], *SendBuffer_aft[2], *RecvBuffer_bef[2], *RecvBuffer_aft[2];
    int *IdSend_bef, *IdSend_aft, *IdRecv_bef, *IdRecv_aft;
} FemStructsType;

typedef struct {
    double (*Condutivity)(void);
    double (*Font)(double, double, double, double, double, double);
    double (*Reaction)(void);
    void (*Velocity)(double, double, double[]);
    double (*upresc)(double, double);
    int (*InitialSolution)(ParametersType *, NodeType *, double *);
    double (*h_shock)(double, double, double, double, double, double, double, double, double, double, double,
                      double);
    double (*ShockCapture)(double, double, double, double, double, double, double, double, double, double, double,
                           double, double, double, double, double, double, double, double);
    int (*StopCriteria)(ParametersType *, double, double, int);
    int (*StopTimeIntegration)(ParametersType *, double *, double *, double);
    void (*assembly)(ParametersType *, MatrixDataType *, FemStructsType *, int, double[3][3]);
    int (*mv)(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
    int (*precond)(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
    int (*precondR)(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
    int (*precond_setup)(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
    int (*scaling)(ParametersType *, MatrixDataType *, FemStructsType *);
    int (*unscaling)(ParametersType *, MatrixDataType *, FemStructsType *, double *);
} FemFunctionsType;

/* Entry points the shim exports under the reference's names and
 * signatures (Solvers_and_Preconditioners/solvers.h:14, preconditioners.h,
 * MatrixVector_Operations/matvec.h). */
int pgmres(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *, double *B, double *X);
int ebemv(ParametersType *, MatrixDataType *, FemStructsType *, double *P, double *Q);
int Diag_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *p, double *z);
int Diag_precond_EBE_setup(ParametersType *, MatrixDataType *, FemStructsType *, int tag, double *F);
int NO_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *p, double *z);
int NO_precond_setup(ParametersType *, MatrixDataType *, FemStructsType *, int tag, double *F);

#endif
