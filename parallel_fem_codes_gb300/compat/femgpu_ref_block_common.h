/*
 * MatrixDataType and AuxBuildStructuresType, identical in the steady
 * Navier-Stokes (SSNavierStokesEquations.h:93-144) and Euler
 * (EulerEquations.h:95-151) drivers; restated field for field.
 */
#ifndef FEMGPU_REF_BLOCK_COMMON_H
#define FEMGPU_REF_BLOCK_COMMON_H

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
    double **BlockDiag;
    double *BlockDiagAux;
    double **invBlockDiag;
    double *invBlockDiagAux;
    double **invDe;
    double *invDeaux;
    double **LUe;
    double *LUeaux;
    int **Id;
    int *IdAux;
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

#endif
