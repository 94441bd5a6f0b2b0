// output.cpp -- Tecplot writers of the reference's output interface, fed with
// the solver's current (converged) state: node averages (Node_Computing,
// gpu_fvm.cu:71-131), the field file unresult.plt and the wall pressure file
// unairfoilpress.plt (Output, gpu_fvm.cu:133-195).  The reference writes these
// from its stale host copy of the initial state (its final field is never
// copied back); here they always describe the state the solver holds.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "internal.h"

using namespace e2d;

namespace {

const double kR = 287.06;  // gpu_fvm.cu:8

struct NodeVals {
    std::vector<double> rou, u, v, p, t, a, mach;
};

// gpu_fvm.cu:71-131: area-weighted cell -> node averages; P, T, A of each
// cell from its conserved state as CalculationPTA computes them.
int node_values(e2d_solver *s, e2d_mesh *m, double gamma, NodeVals &nv) {
    const int N = m->ncell, NN = m->nnode;
    std::vector<double> w(4 * (size_t)N);
    int rc = e2d_get_state(s, w.data());
    if (rc) return rc;
    rc = build_topology(m, m->topo.wall_box >= 0 ? m->topo.wall_box : 2.0);
    if (rc) return rc;
    std::vector<double> ra(NN, 0.0), rou(NN, 0.0), ru(NN, 0.0), rv(NN, 0.0), p(NN, 0.0), t(NN, 0.0),
        a(NN, 0.0);
    for (int c = 0; c < N; c++) {
        const double *q = &w[4 * (size_t)c];
        double U = q[1] / q[0], V = q[2] / q[0];
        double E = q[3] / q[0] - 0.5 * (U * U + V * V);
        double P = (gamma - 1.0) * q[0] * E;
        double A = std::sqrt(gamma * P / q[0]);
        double T = (gamma - 1.0) * E / kR;
        const double ar = m->topo.area[c];
        for (int k = 0; k < 3; k++) {
            const int nd = m->tri[3 * (size_t)c + k] - 1;
            rou[nd] += q[0] * ar; ru[nd] += q[1] * ar; rv[nd] += q[2] * ar;
            t[nd] += T * ar; p[nd] += P * ar; a[nd] += A * ar; ra[nd] += ar;
        }
    }
    nv.rou.resize(NN); nv.u.resize(NN); nv.v.resize(NN); nv.p.resize(NN);
    nv.t.resize(NN); nv.a.resize(NN); nv.mach.resize(NN);
    for (int n = 0; n < NN; n++) {
        nv.rou[n] = rou[n] / ra[n];
        nv.u[n] = ru[n] / ra[n] / nv.rou[n];
        nv.v[n] = rv[n] / ra[n] / nv.rou[n];
        nv.p[n] = p[n] / ra[n];
        nv.t[n] = t[n] / ra[n];
        nv.a[n] = a[n] / ra[n];
        nv.mach[n] = std::sqrt(nv.u[n] * nv.u[n] + nv.v[n] * nv.v[n]) / nv.a[n];
    }
    return E2D_OK;
}

}  // namespace

extern "C" {

int e2d_write_field_plt(e2d_solver *s, e2d_mesh *m, const char *path) {
    if (!s || !m || !path) { set_error("null argument"); return E2D_ERR_ARG; }
    e2d_params p;
    int rc = e2d_get_params(s, &p);
    if (rc) return rc;
    NodeVals nv;
    if ((rc = node_values(s, m, p.gamma, nv))) return rc;
    FILE *fp = std::fopen(path, "w");
    if (!fp) { set_error(std::string("cannot write ") + path); return E2D_ERR_IO; }
    // gpu_fvm.cu:145-162
    std::fprintf(fp, "TITLE= \"Data\"\n");
    std::fprintf(fp, "VARIABLES = \"X\" \"Y\" \"Rou\" \"U\" \"V\" \"P\" \"T\" \"MA\" \n");
    std::fprintf(fp, "ZONE T=\"AirfoilMesh\"\n");
    std::fprintf(fp, "N=%d,E=%d, ZONETYPE=FETriangle\n", m->nnode, m->ncell);
    std::fprintf(fp, "DATAPACKING=POINT\n DT=(SINGLE SINGLE SINGLE SINGLE SINGLE SINGLE SINGLE SINGLE)\n");
    for (int n = 0; n < m->nnode; n++)
        std::fprintf(fp, "%20.10f %20.10f %20.10f %20.10f %20.10f %20.10f %20.10f %20.10f \n", m->x[n], m->y[n],
                     nv.rou[n], nv.u[n], nv.v[n], nv.p[n], nv.t[n], nv.mach[n]);
    for (int c = 0; c < m->ncell; c++) {
        for (int k = 0; k < 3; k++) std::fprintf(fp, "%10d", m->tri[3 * (size_t)c + k]);
        std::fprintf(fp, "\n");
    }
    int bad = std::ferror(fp);
    std::fclose(fp);
    if (bad) { set_error("write error"); return E2D_ERR_IO; }
    return E2D_OK;
}

int e2d_write_wall_cp_plt(e2d_solver *s, e2d_mesh *m, const char *path) {
    if (!s || !m || !path) { set_error("null argument"); return E2D_ERR_ARG; }
    e2d_params p;
    int rc = e2d_get_params(s, &p);
    if (rc) return rc;
    NodeVals nv;
    if ((rc = node_values(s, m, p.gamma, nv))) return rc;
    const MeshTopo &t = m->topo;
    std::vector<int> n1(t.nwall + 1), n2(t.nwall + 1);
    for (int e = 0; e < t.nedge; e++)
        if (t.elog[e] == 2) { n1[t.ewall[e]] = t.en1[e]; n2[t.ewall[e]] = t.en2[e]; }
    // gpu_init.cu:66-70: PIN/(ROUIN*VIN*VIN) is the non-dimensional free-stream pressure
    const double ain = std::sqrt(p.gamma * kR * p.tin), vin = p.ma * ain, rouin = p.pin / (kR * p.tin);
    const double pref = p.pin / (rouin * vin * vin);
    FILE *fp = std::fopen(path, "w");
    if (!fp) { set_error(std::string("cannot write ") + path); return E2D_ERR_IO; }
    // gpu_fvm.cu:177-192
    std::fprintf(fp, "TITLE     = \"Dataset\"\nVARIABLES = \"Position\" \"Pressure\" \n");
    std::fprintf(fp, "ZONE N=%d E=%d F=FEPOINT ET=Triangle\n", t.nwall * 2, t.nwall);
    for (int i = 1; i <= t.nwall; i++) {
        std::fprintf(fp, "%20.10lf %20.10lf\n", m->x[n1[i] - 1], -2.0 * (nv.p[n1[i] - 1] - pref));
        std::fprintf(fp, "%20.10lf %20.10lf\n", m->x[n2[i] - 1], -2.0 * (nv.p[n2[i] - 1] - pref));
    }
    for (int i = 1; i <= t.nwall; i++) std::fprintf(fp, "%d %d %d\n", 2 * i - 1, 2 * i, 2 * i - 1);
    int bad = std::ferror(fp);
    std::fclose(fp);
    if (bad) { set_error("write error"); return E2D_ERR_IO; }
    return E2D_OK;
}

}  // extern "C"
