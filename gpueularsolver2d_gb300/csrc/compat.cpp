// compat.cpp -- the reference's function surface (gpu_fvm.cuh:189-227) over
// libeuler2d, built into libeuler2d_compat.a.  See include/euler2d_compat.h.
#include "../../include/euler2d_compat.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sys/time.h>
#include <vector>

#include <cuda_runtime.h>

#include "internal.h"

static_assert(sizeof(CELL) == 184, "CELL layout must match gpu_fvm.cuh:20-29");
static_assert(sizeof(NODE) == 96, "NODE layout must match gpu_fvm.cuh:43-54");
static_assert(sizeof(EDGE) == 72, "EDGE layout must match gpu_fvm.cuh:67-81");
static_assert(sizeof(W) == 64, "W layout must match gpu_fvm.cuh:98-108");

// The reference's globals (gpu_fvm.cuh:154-169), defined by the caller.
extern int Ncell, Nnode, Nedge, MAXSTEP, WallNum, step, WallBoundNum, FarBoundNum;
extern double MA, ALPHA, GAMA, PIN, TIN, CFL, EPSL, UI, VI;
extern double ROUIN, AIN, VIN, PIS;
extern double R;
extern double PI;
extern double RK[4];
extern double *CellArea;
extern double *Resd;

namespace {

double g_alpha_deg = NAN;  // ALPHA as read, before Initialization turns it into radians

const char *env_or(const char *name, const char *dflt) {
    const char *v = std::getenv(name);
    return v && *v ? v : dflt;
}

// The mesh of the caller's node / cell arrays (1-based, as the reference keeps them).
e2d_mesh *mesh_of(const CELL *cell, const NODE *node) {
    std::vector<double> x(Nnode), y(Nnode);
    std::vector<int32_t> tri(3 * (size_t)Ncell);
    for (int n = 1; n <= Nnode; n++) { x[n - 1] = node[n].x; y[n - 1] = node[n].y; }
    for (int c = 1; c <= Ncell; c++)
        for (int k = 0; k < 3; k++) tri[3 * (size_t)(c - 1) + k] = cell[c].Point[k];
    e2d_mesh *m = nullptr;
    if (e2d_mesh_from_arrays(Nnode, Ncell, x.data(), y.data(), tri.data(), &m) != E2D_OK) return nullptr;
    return m;
}

void fill_edge(EDGE &E, const e2d::MeshTopo &t, int k) {
    std::memset(&E, 0, sizeof E);
    E.ELog = t.elog[k]; E.left_cell = t.eleft[k]; E.right_cell = t.eright[k];
    E.farfieldid = t.efar[k]; E.wallid = t.ewall[k]; E.node1 = t.en1[k]; E.node2 = t.en2[k];
    E.vectorn = t.evn[k]; E.vectorx = t.evx[k]; E.vectory = t.evy[k];
    E.midx = t.emx[k]; E.midy = t.emy[k];
}

}  // namespace

// gpu_init.cu:5-47
int inputMesh(CELL **cell, NODE **node) {
    const char *mp = env_or("E2D_MESH", "2822-3k.dat");
    e2d_mesh *m = nullptr;
    if (e2d_mesh_read(mp, &m) != E2D_OK) {
        std::printf("\nCannot open the mesh data file!\n");
        std::exit(0);
    }
    Nnode = m->nnode;
    Ncell = m->ncell;
    *cell = (CELL *)std::calloc(Ncell + 1, sizeof(CELL));
    *node = (NODE *)std::calloc(Nnode + 1, sizeof(NODE));
    for (int n = 1; n <= Nnode; n++) { (*node)[n].x = m->x[n - 1]; (*node)[n].y = m->y[n - 1]; }
    for (int c = 1; c <= Ncell; c++)
        for (int k = 0; k < 3; k++) (*cell)[c].Point[k] = m->tri[3 * (size_t)(c - 1) + k];
    e2d_mesh_free(m);
    e2d_params p;
    e2d_params_default(&p);
    if (e2d_input_read(env_or("E2D_INPUT", "input.dat"), &p) != E2D_OK) {
        std::printf("\nCannot open input file!\n");
        std::exit(0);
    }
    MA = p.ma; ALPHA = p.alpha_deg; GAMA = p.gamma; PIN = p.pin; TIN = p.tin;
    CFL = p.cfl; EPSL = p.epsl; MAXSTEP = p.maxstep;
    std::printf("inputData finished!\n");
    return 0;
}

// gpu_init.cu:49-61
int CalculationPTA(W &WW) {
    double U = WW.density_U / WW.density;
    double V = WW.density_V / WW.density;
    double E = WW.density_E / WW.density - 0.5 * (U * U + V * V);
    WW.P = (GAMA - 1.0) * WW.density * E;
    WW.A = std::sqrt(GAMA * WW.P / WW.density);
    WW.T = (GAMA - 1.0) * E / R;
    return 0;
}

// gpu_init.cu:63-93
int Initialization(W *w) {
    g_alpha_deg = ALPHA;
    ALPHA = ALPHA * PI / 180.0;
    AIN = std::sqrt(GAMA * R * TIN);
    VIN = MA * AIN;
    ROUIN = PIN / (R * TIN);
    UI = std::cos(ALPHA);
    VI = std::sin(ALPHA);
    double rou_E = R * TIN / (VIN * VIN) / (GAMA - 1.0) + 0.50;
    for (int c = 1; c <= Ncell; c++) {
        w[c].density = 1.0;
        w[c].density_U = std::cos(ALPHA);
        w[c].density_V = std::sin(ALPHA);
        w[c].density_E = rou_E;
        CalculationPTA(w[c]);
    }
    PIS = w[1].P;
    return 0;
}

// gpu_init.cu:95-98
double Calc_area(double x1, double y1, double x2, double y2, double x3, double y3) {
    return (0.5 * ((y3 - y1) * (x2 - x1) - (y2 - y1) * (x3 - x1)));
}

// gpu_init.cu:100-228, in O(N): CellArea, centres, edges in discovery order
// (before the changeEdge partition that ROE_SOLVER applies), neighbours,
// CLog, wall-node flags and the WallEdge list.
int CalculationMeshGeo(CELL *cell, NODE *node, EDGE *edge, EDGE *WallEdge) {
    e2d_mesh *m = mesh_of(cell, node);
    if (!m || e2d::build_topology(m, 2.0) != E2D_OK) {
        std::printf("mesh error: %s\n", e2d_last_error());
        std::exit(1);
    }
    const e2d::MeshTopo &t = m->topo;
    for (int c = 1; c <= Ncell; c++) {
        CellArea[c] = t.area[c - 1];
        cell[c].center[0] = t.cx[c - 1];
        cell[c].center[1] = t.cy[c - 1];
    }
    std::vector<int> post2pre(t.nedge + 1, 0);
    for (int pre = 1; pre <= t.nedge; pre++) post2pre[t.pre2post[pre]] = pre;
    for (int pre = 1; pre <= t.nedge; pre++) fill_edge(edge[pre], t, t.pre2post[pre] - 1);
    for (int c = 1; c <= Ncell; c++) {
        for (int f = 0; f < 3; f++) {
            cell[c].neighbor[f].celledge = post2pre[t.celledge[3 * (size_t)(c - 1) + f]];
            cell[c].neighbor[f].neicell = t.neicell[3 * (size_t)(c - 1) + f];
        }
        cell[c].CLog = t.clog[c - 1];
    }
    for (int k = 0; k < t.nedge; k++)
        if (t.elog[k] == 2) {
            fill_edge(WallEdge[t.ewall[k]], t, k);
            node[t.en1[k]].NLog = 2;
            node[t.en2[k]].NLog = 2;
        }
    Nedge = t.nedge;
    WallBoundNum = t.nwall;
    FarBoundNum = t.nfar;
    e2d_mesh_free(m);
    std::printf("Mesh data Computing's finished!!\n");
    return 0;
}

// gpu_init.cu:249-276: device selection only; the solver owns its memory.
int Cuda_Init() {
    const char *d = std::getenv("E2D_DEVICE");
    if (d && *d) cudaSetDevice(std::atoi(d));
    return 0;
}

// gpu_solver.cu:2171-2473: iterate until Resd <= EPSL or MAXSTEP, printing
// "step,resid" per iteration and filling Resd[] and step; the final state is
// written back into w and the edge / cell numbering gets the changeEdge
// partition the reference applies.
int ROE_SOLVER(W *w, EDGE *edge, double * /*CellArea*/, CELL *cell, NODE *node) {
    struct timeval t0, t1;
    gettimeofday(&t0, nullptr);
    e2d_mesh *m = mesh_of(cell, node);
    if (!m) { std::printf("mesh error: %s\n", e2d_last_error()); std::exit(1); }
    e2d_params p;
    e2d_params_default(&p);
    p.ma = MA; p.gamma = GAMA; p.pin = PIN; p.tin = TIN; p.cfl = CFL; p.epsl = EPSL;
    p.maxstep = MAXSTEP;
    p.alpha_deg = std::isnan(g_alpha_deg) ? ALPHA * 180.0 / PI : g_alpha_deg;
    for (int k = 0; k < 4; k++) p.rk_coef[k] = RK[k];
    p.ordering = E2D_ORDER_MORTON;
    const char *prec = std::getenv("E2D_PRECISION");
    if (prec && !std::strcmp(prec, "fp32")) p.precision = E2D_FP32;
    p.verbose = 1;
    e2d_solver *s = nullptr;
    if (e2d_solver_create(m, &p, &s) != E2D_OK) { std::printf("solver error: %s\n", e2d_last_error()); std::exit(1); }
    std::vector<double> st(4 * (size_t)Ncell);
    for (int c = 1; c <= Ncell; c++) {
        double *q = &st[4 * (size_t)(c - 1)];
        q[0] = w[c].density; q[1] = w[c].density_U; q[2] = w[c].density_V; q[3] = w[c].density_E;
    }
    e2d_set_state(s, st.data());
    step = 0;
    Resd[0] = 100.0;
    std::vector<double> hist(MAXSTEP > 0 ? MAXSTEP : 1);
    int32_t n = 0;
    int rc = e2d_solve(s, MAXSTEP, EPSL, hist.data(), &n);
    std::fflush(stdout);
    for (int k = 0; k < n; k++) Resd[k + 1] = hist[k];
    step = n;
    if (rc != E2D_OK) std::printf("solver stopped: %s\n", e2d_last_error());
    e2d_get_state(s, st.data());
    for (int c = 1; c <= Ncell; c++) {
        const double *q = &st[4 * (size_t)(c - 1)];
        w[c].density = q[0]; w[c].density_U = q[1]; w[c].density_V = q[2]; w[c].density_E = q[3];
        CalculationPTA(w[c]);
    }
    // changeEdge (gpu_solver.cu:1832-1906) on the caller's arrays
    const e2d::MeshTopo &t = m->topo;
    for (int k = 0; k < t.nedge; k++) fill_edge(edge[k + 1], t, k);
    for (int c = 1; c <= Ncell; c++)
        for (int f = 0; f < 3; f++) cell[c].neighbor[f].celledge = t.celledge[3 * (size_t)(c - 1) + f];
    e2d_solver_destroy(s);
    e2d_mesh_free(m);
    gettimeofday(&t1, nullptr);
    std::printf("total time: %g\n", (double)(t1.tv_sec - t0.tv_sec) + 1e-6 * (t1.tv_usec - t0.tv_usec));
    return 0;
}
