/*
 * Memory layout of the steady Navier-Stokes driver's structs
 * (04_SS_NavierStokes_Equations/2D/01_CommonFiles/SSNavierStokesEquations.h:16-165),
 * restated so the drop-in shim compiles without the reference tree.  Every
 * field keeps the reference's type and order; tests/test_compat_layout.py
 * checks the offsets against the reference's own header compiled by
 * oracle/Makefile.
 */
#ifndef FEMGPU_REF_NS_H
#define FEMGPU_REF_NS_H

#define FGC_NDOF 3

typedef struct {
    double x, y;
    int Type[FGC_NDOF];
    int Send[FGC_NDOF];
    int invP_id[FGC_NDOF];
} NodeType;

typedef struct {
    int Vertex[3];
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
    char MatrixVectorProductScheme[200];
    char StabilizationForm[200];
    char Preconditioner[200];
    char Experiments[200];
    char reordering[200];
    double SolverTolerance;
    double NonLinearTolerance;
    double ReynoldsNumber;
    int KrylovBasisVectorsQuantity;
    int nnodes, nNodes;
    int nel, nEl;
    int neq, neq_bef, neqaux_bef, neqaux_aft;
    int nsend_bef, nsend_aft, nrecv_bef, nrecv_aft;
    int NEQ;
    int nnzero;
    int nnzero_bef;
    int nnzero_aft;
    int iterations;
    int k_SPIKE_block_size;
    int RANK;
    int NPROC;
    int LinearMaxIter;
    int NonLinearMaxIter;
    int bandwidth_bef, bandwidth_aft;
    PardisoVariablesType *PardisoVariables;
} ParametersType;

#include "femgpu_ref_block_common.h"

typedef struct {
    int **lm;
    int *lmaux;
    NodeType *Node;
    ElementType *Element;
    double *F;
    double *U;
    double *u;
    double *f;
    double *uB;
    double *delta_old;
    AuxBuildStructuresType *AuxBuild;
    double *SendBuffer_bef[2], *SendBuffer_aft[2], *RecvBuffer_bef[2], *RecvBuffer_aft[2];
    int *IdSend_bef, *IdSend_aft, *IdRecv_bef, *IdRecv_aft;
} FemStructsType;

typedef struct {
    double (*v1presc)(double, double);
    double (*v2presc)(double, double);
    double (*ppresc)(double, double);
    double (*f1ext)(double, double);
    double (*f2ext)(double, double);
    void (*assembly)(ParametersType *, MatrixDataType *, FemStructsType *, int, double (*)[9]);
    int (*mv)(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
    int (*precond)(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
    int (*precondR)(ParametersType *, MatrixDataType *, FemStructsType *, double *, double *);
    int (*precond_setup)(ParametersType *, MatrixDataType *, FemStructsType *, int, double *);
} FemFunctionsType;

/* entry points exported under the reference's names and signatures */
int pgmres(ParametersType *, MatrixDataType *, FemStructsType *, FemFunctionsType *, double *B, double *X);
int ebemvNDOF3(ParametersType *, MatrixDataType *, FemStructsType *, double *P, double *Q);
int BlockDiagDOF3_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *p, double *z);
int BlockDiagDOF3_precond_EBE_setup(ParametersType *, MatrixDataType *, FemStructsType *, int tag, double *F);
int Diag_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *p, double *z);
int Diag_precond_EBE_setup(ParametersType *, MatrixDataType *, FemStructsType *, int tag, double *F);
int NO_precond(ParametersType *, MatrixDataType *, FemStructsType *, double *p, double *z);
int NO_precond_setup(ParametersType *, MatrixDataType *, FemStructsType *, int tag, double *F);

#endif
