/*
 * euler2d_compat.h -- the GPUEularSolver2D function surface on top of
 * libeuler2d (static archive libeuler2d_compat.a).
 *
 * These are the entry points the reference's own main() (gpu_fvm.cu:27-68)
 * calls, with the reference's names, argument meaning, C++ signatures and
 * data layouts (gpu_fvm.cuh:14-227), so that gpu_fvm.cu links against this
 * library instead of gpu_init.cu / gpu_solver.cu and runs unchanged:
 *
 *   nvcc gpu_fvm.cu -I<repo>/include -L<lib> -leuler2d_compat -leuler2d
 *
 * The types below must keep exactly the reference's member order and sizes
 * (static_asserts in compat.cpp).  The globals (Ncell, MA, Resd, ...) are the
 * reference's and are defined by the caller's translation unit, as gpu_fvm.cu
 * does (gpu_fvm.cu:5-25).
 *
 * Differences from the reference, all deliberate:
 *   - the mesh / input file names default to the reference's hard-coded
 *     "2822-3k.dat" / "input.dat" and may be overridden with the environment
 *     variables E2D_MESH / E2D_INPUT;
 *   - CalculationMeshGeo is O(N) (same numbering as the O(N^2) original);
 *   - ROE_SOLVER runs the GB300 solver (FP64 by default, E2D_PRECISION=fp32
 *     for the FP32 stencil) and copies the final state back into w, so the
 *     reference's Node_Computing / Output describe the converged field (the
 *     reference leaves w at the initial state, gpu_solver.cu:2448-2468);
 *   - Cuda_Init selects the device given by E2D_DEVICE (default: the current
 *     device) instead of the hard-coded device 2 (gpu_init.cu:253).
 */
#ifndef EULER2D_COMPAT_H
#define EULER2D_COMPAT_H

/* gpu_fvm.cuh:15-33 */
typedef struct Neighbor {
    int celledge;
    int neicell;
} Neighbor;

typedef struct CELL {
    int CLog;
    int Point[3];
    double deltU[2][4];
    double Umax[4], Umin[4];
    double center[2];
    Neighbor neighbor[3];
} CELL;

/* gpu_fvm.cuh:43-54 */
typedef struct NODE {
    int NLog, Nlog1;
    double x;
    double y;
    double ROU, U, V, E;
    double P, T, A;
    double Mach;
    double RoundArea;
} NODE;

/* gpu_fvm.cuh:67-81 */
typedef struct EDGE {
    int ELog, Elog1;
    int left_cell;
    int right_cell;
    int farfieldid;
    int wallid;
    int node1;
    int node2;
    double vectorn;
    double vectorx;
    double vectory;
    double midx, midy;
} EDGE;

/* gpu_fvm.cuh:98-108 */
typedef struct W {
    double density;
    double density_U;
    double density_V;
    double density_E;
    double P;
    double T;
    double A;
    double B;
} W;

/* gpu_fvm.cuh:189-227 (C++ linkage, as in the reference) */
int inputMesh(CELL **cell, NODE **node);
int CalculationPTA(W &WW);
int Initialization(W *w);
double Calc_area(double x1, double y1, double x2, double y2, double x3, double y3);
int CalculationMeshGeo(CELL *cell, NODE *node, EDGE *edge, EDGE *WallEdge);
int ROE_SOLVER(W *w, EDGE *edge, double *CellArea, CELL *cell, NODE *node);
int Cuda_Init();

#endif
