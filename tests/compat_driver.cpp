// compat_driver.cpp -- test driver for libeuler2d_compat.a.  Defines the
// globals a caller of the reference surface provides (as gpu_fvm.cu:5-25
// does), runs inputMesh / Initialization / CalculationMeshGeo in the working
// directory and dumps what they produce, in the same binary layout as the
// reference harness (oracle/ref_harness.cu, mode geo0).
#include <cstdio>
#include <cstdlib>

#include "euler2d_compat.h"

int Ncell, Nnode, Nedge, MAXSTEP, WallNum, step, WallBoundNum, FarBoundNum;
double MA, ALPHA, GAMA, PIN, TIN, CFL, EPSL, UI, VI;
double ROUIN, AIN, VIN, PIS;
double R = 287.06;
double PI = 3.14159265358979;
double RK[4] = {0.0833, 0.2069, 0.4265, 1.0};
double *CellArea;
double *Resd;
CELL *cell;
NODE *node;
EDGE *edge, *WallEdge;
W *w;

static void dump(const char *name, const void *p, size_t bytes) {
    FILE *f = std::fopen(name, "wb");
    if (!f || std::fwrite(p, 1, bytes, f) != bytes) std::exit(3);
    std::fclose(f);
}

int main() {
    inputMesh(&cell, &node);
    w = (W *)std::calloc(Ncell + 1, sizeof(W));
    edge = (EDGE *)std::calloc(Ncell * 3, sizeof(EDGE));
    Resd = (double *)std::calloc(MAXSTEP + 1, sizeof(double));
    CellArea = (double *)std::calloc(Ncell + 1, sizeof(double));
    WallEdge = (EDGE *)std::calloc(Ncell + 1, sizeof(EDGE));
    Initialization(w);
    CalculationMeshGeo(cell, node, edge, WallEdge);
    int counts[5] = {Ncell, Nnode, Nedge, WallBoundNum, FarBoundNum};
    dump("counts.bin", counts, sizeof counts);
    int *ei = new int[7 * Nedge];
    double *ed = new double[5 * Nedge];
    for (int e = 1; e <= Nedge; e++) {
        int *o = ei + 7 * (e - 1);
        o[0] = edge[e].ELog; o[1] = edge[e].left_cell; o[2] = edge[e].right_cell;
        o[3] = edge[e].farfieldid; o[4] = edge[e].wallid; o[5] = edge[e].node1; o[6] = edge[e].node2;
        double *d = ed + 5 * (e - 1);
        d[0] = edge[e].vectorn; d[1] = edge[e].vectorx; d[2] = edge[e].vectory;
        d[3] = edge[e].midx; d[4] = edge[e].midy;
    }
    dump("edge_i.bin", ei, sizeof(int) * 7 * Nedge);
    dump("edge_d.bin", ed, sizeof(double) * 5 * Nedge);
    int *ci = new int[7 * Ncell];
    double *cd = new double[3 * Ncell], *w7 = new double[7 * Ncell];
    for (int i = 1; i <= Ncell; i++) {
        int *o = ci + 7 * (i - 1);
        o[0] = cell[i].CLog;
        for (int f = 0; f < 3; f++) { o[1 + f] = cell[i].neighbor[f].celledge; o[4 + f] = cell[i].neighbor[f].neicell; }
        cd[3 * (i - 1)] = CellArea[i]; cd[3 * (i - 1) + 1] = cell[i].center[0]; cd[3 * (i - 1) + 2] = cell[i].center[1];
        double *q = w7 + 7 * (i - 1);
        q[0] = w[i].density; q[1] = w[i].density_U; q[2] = w[i].density_V; q[3] = w[i].density_E;
        q[4] = w[i].P; q[5] = w[i].T; q[6] = w[i].A;
    }
    dump("cell_i.bin", ci, sizeof(int) * 7 * Ncell);
    dump("cell_d.bin", cd, sizeof(double) * 3 * Ncell);
    dump("w_init.bin", w7, sizeof(double) * 7 * Ncell);
    dump("pis.bin", &PIS, sizeof PIS);
    int *wi = new int[7 * WallBoundNum];
    for (int k = 1; k <= WallBoundNum; k++) {
        int *o = wi + 7 * (k - 1);
        o[0] = WallEdge[k].ELog; o[1] = WallEdge[k].left_cell; o[2] = WallEdge[k].right_cell;
        o[3] = WallEdge[k].farfieldid; o[4] = WallEdge[k].wallid; o[5] = WallEdge[k].node1; o[6] = WallEdge[k].node2;
    }
    dump("wall_i.bin", wi, sizeof(int) * 7 * WallBoundNum);
    int *nl = new int[Nnode];
    for (int n = 1; n <= Nnode; n++) nl[n - 1] = node[n].NLog;
    dump("nlog.bin", nl, sizeof(int) * Nnode);
    return 0;
}
