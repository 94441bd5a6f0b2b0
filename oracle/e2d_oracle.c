/*
 * e2d_oracle.c -- CPU FP64 restatement of the GPUEularSolver2D solve path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; see e2d_oracle.h).  Every function
 * names the reference file:line it restates.  Build with -ffp-contract=off:
 * the restatement must not fuse multiply-adds, so that its arithmetic is the
 * same sequence of IEEE operations on x86-64 and on aarch64.
 */
#include "e2d_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* gpu_fvm.cu:8-9: the reference's gas constant and its value of pi. */
#define REF_R 287.06
#define REF_PI 3.14159265358979

static _Thread_local char g_err[256];

static void set_err(const char *m) {
    snprintf(g_err, sizeof g_err, "%s", m);
}

const char *or_last_error(void) { return g_err; }

typedef struct wst { double d, du, dv, de, p, t, a; } wst;

struct or_case {
    or_params p;
    int ncell, nnode, nedge, nwall, nfar;
    double *x, *y;          /* [nnode+1] */
    int *pt;                /* [(ncell+1)*3] Point[0..2] */
    double *area, *cx, *cy; /* [ncell+1] */
    int *clog;              /* [ncell+1] */
    int *celledge, *neicell;/* [(ncell+1)*3] */
    int *elog, *eleft, *eright, *efar, *ewall, *en1, *en2; /* [nedge+1] */
    double *evn, *evx, *evy, *emx, *emy;                     /* [nedge+1] */
    double alpha, ain, vin, rouin, ui, vi, pis;
    double ain_test;        /* sound speed of the supersonic test */
    wst *w, *w0, *farw, *wallw;
    double *du;             /* [(ncell+1)*8] deltU[2][4] */
    double *umax, *umin;    /* [(ncell+1)*4] */
    double *phic;           /* [(ncell+1)*4] cell-wise limiter options      */
    double *rel, *rer;      /* [(nedge+1)*4] Res_e left/right */
    double *dtel, *dter;    /* [nedge+1] deltT_e left/right */
    double *res, *r1, *r2;  /* [(ncell+1)*4] */
    double *dt;             /* [ncell+1] */
    double *phil, *phir;    /* [(nedge+1)*4] limiter values (freeze option) */
    int frozen;
    int step;
    double epsm, last_resd;
};

/* ------------------------------------------------------------------ */
/* parameters                                                          */
/* ------------------------------------------------------------------ */

void or_params_default(or_params *p) {
    memset(p, 0, sizeof *p);
    p->ma = 0.5; p->alpha_deg = 0.0; p->gamma = 1.4; p->pin = 101325.0;
    p->tin = 288.15; p->cfl = 1.0; p->epsl = 1e-6; p->maxstep = 100;
    /* gpu_fvm.cu:10 */
    p->rk_stages = 4;
    p->rk_coef[0] = 0.0833; p->rk_coef[1] = 0.2069;
    p->rk_coef[2] = 0.4265; p->rk_coef[3] = 1.0;
    p->irs_eps = 0.8;      /* gpu_solver.cu:1633 */
    p->irs_sweeps = 2;     /* gpu_solver.cu:1722-1728 */
    p->dt_cap = 0.1;       /* gpu_solver.cu:831 */
    p->entropy_eps = 0.05; /* gpu_solver.cu:603 */
    p->wall_box = 2.0;     /* gpu_init.cu:190 */
    p->limiter_k = 5.0;
}

/* gpu_init.cu:34-42: "%lf %lf %lf %lf %lf %lf %lf %d" */
int or_read_input(const char *path, or_params *p) {
    FILE *f = fopen(path, "r");
    if (!f) { set_err("cannot open input file"); return -1; }
    int n = fscanf(f, "%lf %lf %lf %lf %lf %lf %lf %d", &p->ma, &p->alpha_deg,
                   &p->gamma, &p->pin, &p->tin, &p->cfl, &p->epsl, &p->maxstep);
    fclose(f);
    if (n != 8) { set_err("input file needs 8 values"); return -1; }
    return 0;
}

int or_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------ */
/* point functions                                                     */
/* ------------------------------------------------------------------ */

/* gpu_init.cu:49-61 and gpu_solver.cu:49-60 (kernel_CalculationPTA) */
static void calc_pta(wst *w, double g) {
    double U = w->du / w->d;
    double V = w->dv / w->d;
    double E = w->de / w->d - 0.5 * (U * U + V * V);
    w->p = (g - 1.0) * w->d * E;
    w->a = sqrt(g * w->p / w->d);
    w->t = (g - 1.0) * E / REF_R;
}

/* gpu_solver.cu:62-135 (kernel_Far_Boundary) */
static void far_ghost(const or_case *c, const wst *dw, double vectorx,
                      double vectory, wst *w0) {
    const double g = c->p.gamma;
    double nn = sqrt(vectorx * vectorx + vectory * vectory);
    double nx = vectory / nn;
    double ny = vectorx / nn;
    double UD = dw->du / dw->d;
    double VD = dw->dv / dw->d;
    double Un = fabs(c->ui * nx + c->vi * ny);
    double Uncell = UD * nx + VD * ny;
    if (Un / c->ain_test > 1.0) {
        if (Uncell > 0.0) *w0 = *dw;
        if (Uncell <= 0.0) {
            w0->d = 1.0;
            w0->du = c->ui;
            w0->dv = c->vi;
            w0->de = REF_R * c->p.tin / (c->vin * c->vin) / (g - 1.0) + 0.50;
            calc_pta(w0, g);
        }
    } else {
        double PA = c->pis, PD = dw->p, AD = dw->a, ROUD = dw->d, PB, UB, VB;
        if (Uncell > 0.0) {
            PB = PA;
            w0->p = PB;
            w0->d = ROUD + (PB - PD) / AD / AD;
            UB = UD + nx * (PD - PB) / ROUD / AD;
            VB = VD + ny * (PD - PB) / ROUD / AD;
            w0->du = UB * w0->d;
            w0->dv = VB * w0->d;
            w0->de = PB / (g - 1.0) + 0.5 * (UB * UB + VB * VB) * w0->d;
            calc_pta(w0, g);
        }
        if (Uncell <= 0.0) {
            PB = 0.5 * (PA + PD - ROUD * AD * (nx * (c->ui - UD) + ny * (c->vi - VD)));
            w0->p = PB;
            w0->d = 1.0 + (PB - PA) / AD / AD;
            UB = c->ui - nx * (PA - PB) / ROUD / AD;
            VB = c->vi - ny * (PA - PB) / ROUD / AD;
            w0->du = UB * w0->d;
            w0->dv = VB * w0->d;
            w0->de = PB / (g - 1.0) + 0.5 * (UB * UB + VB * VB) * w0->d;
            calc_pta(w0, g);
        }
    }
}

/* gpu_solver.cu:188-221: slip-wall ghost, velocity mirrored in the face. */
static void wall_ghost(const wst *dw, double vectorx, double vectory,
                       double vectorn, wst *out) {
    double nij0 = vectory / vectorn;
    double nij1 = vectorx / vectorn;
    double UU = dw->du / dw->d;
    double VV = dw->dv / dw->d;
    double UV = UU * nij0 + VV * nij1;
    UU = UU - 2 * UV * nij0;
    VV = VV - 2 * UV * nij1;
    *out = *dw;
    out->du = dw->d * UU;
    out->dv = dw->d * VV;
}

/* gpu_solver.cu:552-566 (kernel_Calc_Function) */
static void calc_function(const wst *w, double g, double *A, double *U,
                          double *V, double *H, double *P) {
    double temp = 1.0 / w->d;
    *U = w->du * temp;
    *V = w->dv * temp;
    *P = (g - 1.0) * w->d * (w->de * temp - 0.5 * (*U * *U + *V * *V));
    *A = sqrt(g * *P * temp);
    *H = w->de * temp + *P * temp;
}

/* gpu_solver.cu:569-647 (kernel_ROE_SCHEME) */
static void roe(const wst *LW, const wst *RW, double nx, double ny, double g,
                double epsilon, double FLUX[4]) {
    double A[2], U[2], V[2], H[2], P[2], M[2], FF[3][4], AD[3], WL[4], WR[4];
    calc_function(LW, g, &A[0], &U[0], &V[0], &H[0], &P[0]);
    calc_function(RW, g, &A[1], &U[1], &V[1], &H[1], &P[1]);
    M[0] = (U[0] * nx + V[0] * ny);
    M[1] = (U[1] * nx + V[1] * ny);
    double DVC = M[1] - M[0];
    double lrou = LW->d, rrou = RW->d;
    double sl = sqrt(lrou), sr = sqrt(rrou);
    double ROUB = sl * sr;
    double UB = (U[0] * sl + U[1] * sr) / (sl + sr);
    double VB = (V[0] * sl + V[1] * sr) / (sl + sr);
    double HB = (H[0] * sl + H[1] * sr) / (sl + sr);
    double QB = UB * UB + VB * VB;
    double AB = sqrt((g - 1.0) * (HB - QB / 2.0));
    double VC = UB * nx + VB * ny;
    if (fabs(VC - AB) < epsilon)
        AD[0] = ((VC - AB) * (VC - AB) + epsilon * epsilon) / (2 * epsilon);
    else
        AD[0] = fabs(VC - AB);
    if (fabs(VC) < epsilon)
        AD[1] = (VC * VC + epsilon * epsilon) / (2 * epsilon);
    else
        AD[1] = fabs(VC);
    if (fabs(VC + AB) < epsilon)
        AD[2] = ((VC + AB) * (VC + AB) + epsilon * epsilon) / (2 * epsilon);
    else
        AD[2] = fabs(VC + AB);
    FF[0][0] = AD[0] * ((P[1] - P[0]) - ROUB * AB * DVC) / (2.0 * AB * AB);
    FF[0][1] = FF[0][0] * (UB - AB * nx);
    FF[0][2] = FF[0][0] * (VB - AB * ny);
    FF[0][3] = FF[0][0] * (HB - AB * VC);
    FF[1][0] = AD[1] * ((rrou - lrou) - (P[1] - P[0]) / (AB * AB));
    FF[1][1] = FF[1][0] * UB + AD[1] * ROUB * (U[1] - U[0] - DVC * nx);
    FF[1][2] = FF[1][0] * VB + AD[1] * ROUB * (V[1] - V[0] - DVC * ny);
    FF[1][3] = FF[1][0] * QB * 0.5 +
               AD[1] * ROUB * (UB * (U[1] - U[0]) + VB * (V[1] - V[0]) - DVC * VC);
    FF[2][0] = AD[2] * ((P[1] - P[0]) + ROUB * AB * DVC) / (2.0 * AB * AB);
    FF[2][1] = FF[2][0] * (UB + AB * nx);
    FF[2][2] = FF[2][0] * (VB + AB * ny);
    FF[2][3] = FF[2][0] * (HB + AB * VC);
    WL[0] = lrou * M[0];
    WL[1] = U[0] * WL[0] + nx * P[0];
    WL[2] = V[0] * WL[0] + ny * P[0];
    WL[3] = WL[0] * H[0];
    WR[0] = rrou * M[1];
    WR[1] = U[1] * WR[0] + nx * P[1];
    WR[2] = V[1] * WR[0] + ny * P[1];
    WR[3] = WR[0] * H[1];
    for (int k = 0; k < 4; k++)
        FLUX[k] = 0.5 * ((WL[k] + WR[k]) - (FF[0][k] + FF[1][k] + FF[2][k]));
}

void or_roe_flux(const double lw[4], const double rw[4], double nx, double ny,
                 double gamma, double entropy_eps, double flux[4]) {
    wst L = {lw[0], lw[1], lw[2], lw[3], 0, 0, 0};
    wst R = {rw[0], rw[1], rw[2], rw[3], 0, 0, 0};
    roe(&L, &R, nx, ny, gamma, entropy_eps, flux);
}

void or_far_ghost(const double dw[4], double vectorx, double vectory,
                  const or_case *c, double out[4]) {
    wst D = {dw[0], dw[1], dw[2], dw[3], 0, 0, 0}, G;
    memset(&G, 0, sizeof G);
    calc_pta(&D, c->p.gamma);
    far_ghost(c, &D, vectorx, vectory, &G);
    out[0] = G.d; out[1] = G.du; out[2] = G.dv; out[3] = G.de;
}

/* ------------------------------------------------------------------ */
/* mesh set-up                                                         */
/* ------------------------------------------------------------------ */

/* gpu_init.cu:95-98 */
static double calc_area(double x1, double y1, double x2, double y2, double x3,
                        double y3) {
    return (0.5 * ((y3 - y1) * (x2 - x1) - (y2 - y1) * (x3 - x1)));
}

typedef struct slot { uint64_t key; int occ1, occ2, count, edge; } slot;

static uint64_t hkey(uint64_t k) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33; return k;
}

static slot *find_slot(slot *tab, uint64_t mask, uint64_t key) {
    uint64_t h = hkey(key) & mask;
    while (tab[h].key != 0 && tab[h].key != key) h = (h + 1) & mask;
    return &tab[h];
}

static void *xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s);
    if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
    return p;
}

/*
 * gpu_init.cu:100-228 (CalculationMeshGeo) followed by gpu_solver.cu:1832-1906
 * (changeEdge).  The reference discovers edges with an O(N^2) search; this
 * restatement uses a hash of the unordered node pair and reproduces the same
 * numbering: an edge gets the next id when it is first met in (cell, face)
 * order, its left cell is that first cell and its right cell is the next cell
 * that has it (-1 if none).  Boundary edges are wall when the midpoint lies
 * inside the |x|,|y| < wall_box box, far field otherwise, and get wall / far
 * ids in order of discovery.  changeEdge then stably partitions the edges into
 * interior, far field, wall and renames every cell's celledge.
 */
static int build_geometry(or_case *c) {
    const int N = c->ncell;
    c->area = xcalloc(N + 1, sizeof(double));
    c->cx = xcalloc(N + 1, sizeof(double));
    c->cy = xcalloc(N + 1, sizeof(double));
    c->clog = xcalloc(N + 1, sizeof(int));
    c->celledge = xcalloc((size_t)(N + 1) * 3, sizeof(int));
    c->neicell = xcalloc((size_t)(N + 1) * 3, sizeof(int));
    for (int i = 1; i <= N; i++) {
        int p0 = c->pt[3 * i], p1 = c->pt[3 * i + 1], p2 = c->pt[3 * i + 2];
        if (p0 < 1 || p0 > c->nnode || p1 < 1 || p1 > c->nnode || p2 < 1 ||
            p2 > c->nnode) { set_err("node id out of range"); return -1; }
        c->area[i] = calc_area(c->x[p0], c->y[p0], c->x[p1], c->y[p1], c->x[p2],
                               c->y[p2]);
        if (!(c->area[i] > 0.0)) { set_err("cell area <= 0 (cells must be CCW)"); return -1; }
        c->cx[i] = (c->x[p0] + c->x[p1] + c->x[p2]) / 3.0;
        c->cy[i] = (c->y[p0] + c->y[p1] + c->y[p2]) / 3.0;
    }
    uint64_t cap = 1;
    while (cap < (uint64_t)N * 6 + 16) cap <<= 1;
    slot *tab = xcalloc(cap, sizeof(slot));
    for (int i = 1; i <= N; i++)
        for (int f = 0; f < 3; f++) {
            int N1 = c->pt[3 * i + (f + 1) % 3], N2 = c->pt[3 * i + (f + 2) % 3];
            if (N1 == N2) { free(tab); set_err("degenerate cell"); return -1; }
            uint64_t lo = N1 < N2 ? N1 : N2, hi = N1 < N2 ? N2 : N1;
            uint64_t key = (lo << 32) | hi;
            slot *s = find_slot(tab, cap - 1, key);
            if (s->key == 0) { s->key = key; s->occ1 = i; s->count = 1; }
            else {
                if (s->occ1 == i) { free(tab); set_err("cell repeats an edge"); return -1; }
                if (s->count >= 2) { free(tab); set_err("non-manifold edge"); return -1; }
                s->occ2 = i; s->count = 2;
            }
        }
    /* discovery pass, numbering as the reference does */
    int cap_e = 3 * N + 1;
    int *elog = xcalloc(cap_e, sizeof(int)), *el = xcalloc(cap_e, sizeof(int));
    int *er = xcalloc(cap_e, sizeof(int)), *ef = xcalloc(cap_e, sizeof(int));
    int *ew = xcalloc(cap_e, sizeof(int)), *n1 = xcalloc(cap_e, sizeof(int));
    int *n2 = xcalloc(cap_e, sizeof(int));
    double *vn = xcalloc(cap_e, sizeof(double)), *vx = xcalloc(cap_e, sizeof(double));
    double *vy = xcalloc(cap_e, sizeof(double)), *mx = xcalloc(cap_e, sizeof(double));
    double *my = xcalloc(cap_e, sizeof(double));
    int ne = 0, nw = 0, nf = 0;
    for (int i = 1; i <= N; i++) {
        for (int f = 0; f < 3; f++) {
            int N1 = c->pt[3 * i + (f + 1) % 3], N2 = c->pt[3 * i + (f + 2) % 3];
            uint64_t lo = N1 < N2 ? N1 : N2, hi = N1 < N2 ? N2 : N1;
            slot *s = find_slot(tab, cap - 1, (lo << 32) | hi);
            if (s->edge == 0) {
                int e = ++ne;
                s->edge = e;
                el[e] = i; n1[e] = N1; n2[e] = N2;
                vx[e] = c->x[N1] - c->x[N2];
                vy[e] = c->y[N2] - c->y[N1];
                mx[e] = 0.5 * (c->x[N1] + c->x[N2]);
                my[e] = 0.5 * (c->y[N1] + c->y[N2]);
                vn[e] = sqrt(vx[e] * vx[e] + vy[e] * vy[e]);
                if (s->count == 2) { er[e] = s->occ2; elog[e] = 0; }
                else {
                    er[e] = -1;
                    if (fabs(mx[e]) < c->p.wall_box && fabs(my[e]) < c->p.wall_box) {
                        elog[e] = 2; ew[e] = ++nw;
                    } else {
                        elog[e] = 1; ef[e] = ++nf;
                    }
                }
            }
            c->celledge[3 * i + f] = s->edge;
        }
        int nn = 3;
        for (int f = 0; f < 3; f++) {
            int e = c->celledge[3 * i + f];
            int nb = el[e] == i ? er[e] : el[e];
            if (nb == -1) { nb *= elog[e]; nn--; }
            c->neicell[3 * i + f] = nb;
        }
        c->clog[i] = nn;
    }
    free(tab);
    /* changeEdge: stable partition by ELog 0, 1, 2 */
    int *newid = xcalloc(ne + 1, sizeof(int));
    int j = 1;
    for (int lg = 0; lg <= 2; lg++)
        for (int e = 1; e <= ne; e++)
            if (elog[e] == lg) newid[e] = j++;
    c->nedge = ne; c->nwall = nw; c->nfar = nf;
    c->elog = xcalloc(ne + 1, sizeof(int)); c->eleft = xcalloc(ne + 1, sizeof(int));
    c->eright = xcalloc(ne + 1, sizeof(int)); c->efar = xcalloc(ne + 1, sizeof(int));
    c->ewall = xcalloc(ne + 1, sizeof(int)); c->en1 = xcalloc(ne + 1, sizeof(int));
    c->en2 = xcalloc(ne + 1, sizeof(int));
    c->evn = xcalloc(ne + 1, sizeof(double)); c->evx = xcalloc(ne + 1, sizeof(double));
    c->evy = xcalloc(ne + 1, sizeof(double)); c->emx = xcalloc(ne + 1, sizeof(double));
    c->emy = xcalloc(ne + 1, sizeof(double));
    for (int e = 1; e <= ne; e++) {
        int k = newid[e];
        c->elog[k] = elog[e]; c->eleft[k] = el[e]; c->eright[k] = er[e];
        c->efar[k] = ef[e]; c->ewall[k] = ew[e]; c->en1[k] = n1[e]; c->en2[k] = n2[e];
        c->evn[k] = vn[e]; c->evx[k] = vx[e]; c->evy[k] = vy[e];
        c->emx[k] = mx[e]; c->emy[k] = my[e];
    }
    for (int i = 1; i <= N; i++)
        for (int f = 0; f < 3; f++) c->celledge[3 * i + f] = newid[c->celledge[3 * i + f]];
    free(newid); free(elog); free(el); free(er); free(ef); free(ew); free(n1); free(n2);
    free(vn); free(vx); free(vy); free(mx); free(my);
    return 0;
}

/* gpu_init.cu:63-93 (Initialization) */
static void initialise(or_case *c) {
    const double g = c->p.gamma;
    c->alpha = c->p.alpha_deg * REF_PI / 180.0;
    c->ain = sqrt(g * REF_R * c->p.tin);
    c->vin = c->p.ma * c->ain;
    /* gpu_solver.cu:79 divides the non-dimensional Un by the dimensional
     * AIN; the far_field_fix option uses the non-dimensional 1/M instead. */
    c->ain_test = c->p.far_field_fix ? 1.0 / c->p.ma : c->ain;
    c->rouin = c->p.pin / (REF_R * c->p.tin);
    c->ui = cos(c->alpha);
    c->vi = sin(c->alpha);
    double rou_U = cos(c->alpha), rou_V = sin(c->alpha);
    double rou_E = REF_R * c->p.tin / (c->vin * c->vin) / (g - 1.0) + 0.50;
    for (int i = 1; i <= c->ncell; i++) {
        c->w[i].d = 1.0; c->w[i].du = rou_U; c->w[i].dv = rou_V; c->w[i].de = rou_E;
        calc_pta(&c->w[i], g);
    }
    c->pis = c->w[1].p;
    c->step = 0;
    c->epsm = 0.0;
    c->last_resd = 100.0; /* gpu_solver.cu:2185 Resd[0]=100 */
}

static or_case *finish_create(or_case *c) {
    if (c->ncell < 1 || c->nnode < 3) { set_err("empty mesh"); or_destroy(c); return NULL; }
    if (build_geometry(c) != 0) { or_destroy(c); return NULL; }
    const int N = c->ncell;
    c->w = xcalloc(N + 1, sizeof(wst)); c->w0 = xcalloc(N + 1, sizeof(wst));
    c->farw = xcalloc(c->nfar + 1, sizeof(wst)); c->wallw = xcalloc(c->nwall + 1, sizeof(wst));
    c->du = xcalloc((size_t)(N + 1) * 8, sizeof(double));
    c->umax = xcalloc((size_t)(N + 1) * 4, sizeof(double));
    c->phic = xcalloc((size_t)(N + 1) * 4, sizeof(double));
    c->umin = xcalloc((size_t)(N + 1) * 4, sizeof(double));
    c->rel = xcalloc((size_t)(c->nedge + 1) * 4, sizeof(double));
    c->rer = xcalloc((size_t)(c->nedge + 1) * 4, sizeof(double));
    c->dtel = xcalloc(c->nedge + 1, sizeof(double));
    c->dter = xcalloc(c->nedge + 1, sizeof(double));
    c->res = xcalloc((size_t)(N + 1) * 4, sizeof(double));
    c->r1 = xcalloc((size_t)(N + 1) * 4, sizeof(double));
    c->r2 = xcalloc((size_t)(N + 1) * 4, sizeof(double));
    c->dt = xcalloc(N + 1, sizeof(double));
    if (c->p.limiter_freeze > 0 || c->p.limiter_freeze_resd > 0.0) {
        c->phil = xcalloc((size_t)(c->nedge + 1) * 4, sizeof(double));
        c->phir = xcalloc((size_t)(c->nedge + 1) * 4, sizeof(double));
    }
    initialise(c);
    return c;
}

or_case *or_create(int nnode, int ncell, const double *x, const double *y,
                   const int *tri, const or_params *p) {
    or_case *c = xcalloc(1, sizeof(or_case));
    c->p = *p;
    c->nnode = nnode; c->ncell = ncell;
    c->x = xcalloc(nnode + 1, sizeof(double)); c->y = xcalloc(nnode + 1, sizeof(double));
    c->pt = xcalloc((size_t)(ncell + 1) * 3, sizeof(int));
    for (int i = 0; i < nnode; i++) { c->x[i + 1] = x[i]; c->y[i + 1] = y[i]; }
    for (int i = 0; i < ncell; i++)
        for (int k = 0; k < 3; k++) c->pt[3 * (i + 1) + k] = tri[3 * i + k];
    return finish_create(c);
}

/* gpu_init.cu:5-33 (inputMesh): "Nnode Ncell", all x, all y, 3 ids per cell */
or_case *or_create_from_file(const char *mesh_path, const or_params *p) {
    FILE *f = fopen(mesh_path, "r");
    if (!f) { set_err("cannot open the mesh data file"); return NULL; }
    int nnode = 0, ncell = 0;
    if (fscanf(f, "%d %d", &nnode, &ncell) != 2 || nnode < 3 || ncell < 1) {
        fclose(f); set_err("bad mesh header"); return NULL;
    }
    or_case *c = xcalloc(1, sizeof(or_case));
    c->p = *p; c->nnode = nnode; c->ncell = ncell;
    c->x = xcalloc(nnode + 1, sizeof(double)); c->y = xcalloc(nnode + 1, sizeof(double));
    c->pt = xcalloc((size_t)(ncell + 1) * 3, sizeof(int));
    int ok = 1;
    for (int i = 1; i <= nnode && ok; i++) ok = fscanf(f, "%lf", &c->x[i]) == 1;
    for (int i = 1; i <= nnode && ok; i++) ok = fscanf(f, "%lf", &c->y[i]) == 1;
    for (int i = 1; i <= ncell && ok; i++)
        for (int k = 0; k < 3 && ok; k++) ok = fscanf(f, "%d", &c->pt[3 * i + k]) == 1;
    fclose(f);
    if (!ok) { set_err("truncated mesh file"); or_destroy(c); return NULL; }
    return finish_create(c);
}

void or_destroy(or_case *c) {
    if (!c) return;
    void *ptrs[] = {c->x, c->y, c->pt, c->area, c->cx, c->cy, c->clog, c->celledge,
                    c->neicell, c->elog, c->eleft, c->eright, c->efar, c->ewall, c->en1,
                    c->en2, c->evn, c->evx, c->evy, c->emx, c->emy, c->w, c->w0,
                    c->farw, c->wallw, c->du, c->umax, c->umin, c->phic, c->rel, c->rer,
                    c->dtel, c->dter, c->res, c->r1, c->r2, c->dt, c->phil, c->phir};
    for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; i++) free(ptrs[i]);
    free(c);
}

void or_counts(const or_case *c, int out[5]) {
    out[0] = c->ncell; out[1] = c->nnode; out[2] = c->nedge;
    out[3] = c->nwall; out[4] = c->nfar;
}

void or_topology(const or_case *c, int *ei, double *ed, int *ci, double *cd) {
    for (int e = 1; e <= c->nedge; e++) {
        size_t k = e - 1;
        if (ei) {
            ei[7 * k + 0] = c->elog[e]; ei[7 * k + 1] = c->eleft[e];
            ei[7 * k + 2] = c->eright[e]; ei[7 * k + 3] = c->efar[e];
            ei[7 * k + 4] = c->ewall[e]; ei[7 * k + 5] = c->en1[e];
            ei[7 * k + 6] = c->en2[e];
        }
        if (ed) {
            ed[5 * k + 0] = c->evn[e]; ed[5 * k + 1] = c->evx[e];
            ed[5 * k + 2] = c->evy[e]; ed[5 * k + 3] = c->emx[e];
            ed[5 * k + 4] = c->emy[e];
        }
    }
    for (int i = 1; i <= c->ncell; i++) {
        size_t k = i - 1;
        if (ci) {
            ci[7 * k] = c->clog[i];
            for (int f = 0; f < 3; f++) {
                ci[7 * k + 1 + f] = c->celledge[3 * i + f];
                ci[7 * k + 4 + f] = c->neicell[3 * i + f];
            }
        }
        if (cd) { cd[3 * k] = c->area[i]; cd[3 * k + 1] = c->cx[i]; cd[3 * k + 2] = c->cy[i]; }
    }
}

void or_get_state(const or_case *c, double *w) {
    for (int i = 1; i <= c->ncell; i++) {
        double *o = w + 4 * (size_t)(i - 1);
        o[0] = c->w[i].d; o[1] = c->w[i].du; o[2] = c->w[i].dv; o[3] = c->w[i].de;
    }
}

int or_set_state(or_case *c, const double *w) {
    for (int i = 1; i <= c->ncell; i++) {
        const double *s = w + 4 * (size_t)(i - 1);
        c->w[i].d = s[0]; c->w[i].du = s[1]; c->w[i].dv = s[2]; c->w[i].de = s[3];
        calc_pta(&c->w[i], c->p.gamma);
    }
    return 0;
}

void or_get_pta(const or_case *c, double *pta) {
    for (int i = 1; i <= c->ncell; i++) {
        double *o = pta + 3 * (size_t)(i - 1);
        o[0] = c->w[i].p; o[1] = c->w[i].t; o[2] = c->w[i].a;
    }
}

double or_pis(const or_case *c) { return c->pis; }
int or_step_count(const or_case *c) { return c->step; }

/* ------------------------------------------------------------------ */
/* one RK stage, kernel by kernel                                      */
/* ------------------------------------------------------------------ */

/* gpu_solver.cu:137-223 (kernel_Boundary) */
static void stage_boundary(or_case *c) {
    #pragma omp parallel for schedule(static)
    for (int e = 1; e <= c->nedge; e++) {
        int lg = c->elog[e];
        if (lg == 1) far_ghost(c, &c->w[c->eleft[e]], c->evx[e], c->evy[e], &c->farw[c->efar[e]]);
        if (lg == 2)
            wall_ghost(&c->w[c->eleft[e]], c->evx[e], c->evy[e], c->evn[e], &c->wallw[c->ewall[e]]);
    }
}

/* gpu_solver.cu:225-383 (kernel_Gradient) */
static void stage_gradient(or_case *c) {
    #pragma omp parallel for schedule(static)
    for (int i = 1; i <= c->ncell; i++) {
        const wst *Ui = &c->w[i];
        double U[4] = {Ui->d, Ui->du, Ui->dv, Ui->de};
        double g[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
        double jmax[4], jmin[4], comp[4] = {0, 0, 0, 0};
        for (int f = 0; f < 3; f++) {
            int N1 = c->pt[3 * i + (f + 1) % 3], N2 = c->pt[3 * i + (f + 2) % 3];
            double vectorx = c->x[N1] - c->x[N2];
            double vectory = c->y[N2] - c->y[N1];
            int e = c->celledge[3 * i + f], nb = c->neicell[3 * i + f];
            const wst *s = NULL;
            if (nb > 0) s = &c->w[nb];
            if (nb == -1) s = &c->farw[c->efar[e]];
            if (nb == -2) s = &c->wallw[c->ewall[e]];
            if (s) { comp[0] = s->d; comp[1] = s->du; comp[2] = s->dv; comp[3] = s->de; }
            if (f == 0) {
                for (int k = 0; k < 4; k++) { jmax[k] = comp[k]; jmin[k] = comp[k]; }
            } else {
                for (int k = 0; k < 4; k++) {
                    if (comp[k] < jmin[k]) jmin[k] = comp[k];
                    if (comp[k] > jmax[k]) jmax[k] = comp[k];
                }
            }
            for (int k = 0; k < 4; k++) {
                g[0][k] += 0.5 * (U[k] + comp[k]) * vectory;
                g[1][k] += 0.5 * (U[k] + comp[k]) * vectorx;
            }
        }
        double area = 1.0 / c->area[i];
        for (int k = 0; k < 4; k++) {
            c->du[8 * (size_t)i + k] = g[0][k] * area;
            c->du[8 * (size_t)i + 4 + k] = g[1][k] * area;
            c->umax[4 * (size_t)i + k] = fmax(U[k], jmax[k]);
            c->umin[4 * (size_t)i + k] = fmin(U[k], jmin[k]);
        }
    }
}

/* Limiter value of one component on one face side (gpu_solver.cu:456-494):
 * kind 0 the reference's min(1, (Umax-U)/delt2) / min(1, (Umin-U)/delt2) /
 * 1, kind 1 the Venkatakrishnan form on the same differences (option).
 * fi_prev: the reference keeps the previous value when delt2 is NaN. */
static double face_phi(const or_case *c, int cell, int k, double u, double delt2, int kind, double fi_prev) {
    double fi = fi_prev;
    if (kind == 1) {
        double K3 = c->p.limiter_k * c->p.limiter_k * c->p.limiter_k;
        double A = c->area[cell];
        double e2 = K3 * A * sqrt(A);
        double d1 = delt2 > 0 ? c->umax[4 * (size_t)cell + k] - u : c->umin[4 * (size_t)cell + k] - u;
        return delt2 == 0 ? 1.0 : (d1 * d1 + e2 + 2 * delt2 * d1) / (d1 * d1 + 2 * delt2 * delt2 + d1 * delt2 + e2);
    }
    if (delt2 > 0) fi = fmin((c->umax[4 * (size_t)cell + k] - u) / delt2, 1.0);
    if (delt2 < 0) fi = fmin((c->umin[4 * (size_t)cell + k] - u) / delt2, 1.0);
    if (delt2 == 0) fi = 1.0;
    return fi;
}

/* Cell-wise limiter options (2: reference form, 3: Venkatakrishnan form; no
 * reference counterpart): per cell and component the smallest per-face value
 * over the cell's interior faces, the faces taken in the cell's face order. */
static void stage_cell_limiter(or_case *c) {
    if (c->p.limiter < 2) return;
    #pragma omp parallel for schedule(static)
    for (int i = 1; i <= c->ncell; i++) {
        const wst *w = &c->w[i];
        double UI[4] = {w->d, w->du, w->dv, w->de};
        const double *du = c->du + 8 * (size_t)i;
        double m[4] = {INFINITY, INFINITY, INFINITY, INFINITY};
        for (int f = 0; f < 3; f++) {
            if (c->neicell[3 * i + f] <= 0) continue;
            int e = c->celledge[3 * i + f];
            double r0 = c->emx[e] - c->cx[i], r1 = c->emy[e] - c->cy[i];
            for (int k = 0; k < 4; k++) {
                double delt2 = du[k] * r0 + du[4 + k] * r1;
                m[k] = fmin(m[k], face_phi(c, i, k, UI[k], delt2, c->p.limiter - 2, 1.0));
            }
        }
        for (int k = 0; k < 4; k++) c->phic[4 * (size_t)i + k] = m[k];
    }
}

/* gpu_solver.cu:456-494 (kernel_Limiter) and 496-549 (kernel_LBJinterpolate):
 * one side of an interior face, limited per face and per component.
 * phi: with the limiter-freeze option, the 4 stored limiter values of this
 * face side (recorded while not frozen, reused once frozen); NULL otherwise. */
static void reconstruct(const or_case *c, int cell, double midx, double midy, wst *out, double *phi) {
    const wst *w = &c->w[cell];
    double UI[4] = {w->d, w->du, w->dv, w->de};
    /* first-order faces option (no reference counterpart): the cell state
       itself during the first first_order_iters iterations, as the
       reference's boundary faces (gpu_solver.cu:689-725) */
    if (c->p.first_order_iters > 0 && c->step <= c->p.first_order_iters) {
        memset(out, 0, sizeof *out);
        out->d = UI[0]; out->du = UI[1]; out->dv = UI[2]; out->de = UI[3];
        return;
    }
    double r0 = midx - c->cx[cell], r1 = midy - c->cy[cell];
    const double *du = c->du + 8 * (size_t)cell;
    double delt2[4], fi = 1.0;
    for (int k = 0; k < 4; k++) delt2[k] = du[k] * r0 + du[4 + k] * r1;
    for (int k = 0; k < 4; k++) {
        if (phi && c->frozen) fi = phi[k];
        else {
            if (c->p.limiter >= 2) fi = c->phic[4 * (size_t)cell + k];  /* cell-wise options */
            else fi = face_phi(c, cell, k, UI[k], delt2[k], c->p.limiter, fi);
            if (phi) phi[k] = fi;
        }
        delt2[k] *= fi;
    }
    memset(out, 0, sizeof *out);
    out->d = UI[0] + delt2[0]; out->du = UI[1] + delt2[1];
    out->dv = UI[2] + delt2[2]; out->de = UI[3] + delt2[3];
    /* positivity fallback option (no reference counterpart): a face side
       whose density or pressure is not positive takes the cell state */
    if (c->p.positivity_fix) {
        double q = 0.5 * (out->du * out->du + out->dv * out->dv) / out->d;
        if (!(out->d > 0) || !((c->p.gamma - 1.0) * (out->de - q) > 0)) {
            out->d = UI[0]; out->du = UI[1]; out->dv = UI[2]; out->de = UI[3];
        }
    }
}

/* gpu_solver.cu:651-764 (kernel_Flux2) and 385-454 (kernel_deltT) */
static void stage_flux(or_case *c) {
    const double g = c->p.gamma;
    #pragma omp parallel for schedule(static)
    for (int e = 1; e <= c->nedge; e++) {
        int lg = c->elog[e], L = c->eleft[e], R = c->eright[e];
        wst LW, RW;
        const wst *G = NULL;
        if (lg == 0) {
            reconstruct(c, L, c->emx[e], c->emy[e], &LW, c->phil ? c->phil + 4 * (size_t)e : NULL);
            reconstruct(c, R, c->emx[e], c->emy[e], &RW, c->phir ? c->phir + 4 * (size_t)e : NULL);
        } else {
            G = lg == 1 ? &c->farw[c->efar[e]] : &c->wallw[c->ewall[e]];
            LW = c->w[L];
            RW = *G;
        }
        double F[4];
        roe(&LW, &RW, c->evy[e] / c->evn[e], c->evx[e] / c->evn[e], g, c->p.entropy_eps, F);
        for (int k = 0; k < 4; k++) {
            F[k] *= c->evn[e];
            c->rel[4 * (size_t)e + k] = F[k];
            c->rer[4 * (size_t)e + k] = R != -1 ? F[k] : 0;
        }
        /* kernel_deltT: mean of the unreconstructed states */
        const wst *Rs = lg == 0 ? &c->w[R] : G;
        const wst *Ls = &c->w[L];
        double vectorx = c->evx[e], vectory = c->evy[e];
        double rou = (Ls->d + Rs->d) * 0.5;
        double u = (Ls->du + Rs->du) / rou * 0.5;
        double v = (Ls->dv + Rs->dv) / rou * 0.5;
        double EE = (Ls->de + Rs->de) * 0.5 / rou - (u * u + v * v) * 0.5;
        double VC = u * vectory + v * vectorx;
        double p = rou * EE * (g - 1.0);
        double CS = sqrt((g * p / rou) * (vectorx * vectorx + vectory * vectory));
        double SR = fabs(VC) + CS;
        c->dtel[e] = SR;
        if (R != -1) c->dter[e] = SR;
    }
}

/* gpu_solver.cu:768-878 (kernel_Flux_e2c) */
static void stage_e2c(or_case *c) {
    #pragma omp parallel for schedule(static)
    for (int i = 1; i <= c->ncell; i++) {
        double T = 0, r[4] = {0.0, 0.0, 0.0, 0.0};
        for (int f = 0; f < 3; f++) {
            int e = c->celledge[3 * i + f];
            if (c->eleft[e] == i) {
                T += c->dtel[e];
                for (int k = 0; k < 4; k++) r[k] += c->rel[4 * (size_t)e + k];
            }
            if (c->eright[e] == i) {
                T += c->dter[e];
                for (int k = 0; k < 4; k++) r[k] -= c->rer[4 * (size_t)e + k];
            }
        }
        for (int k = 0; k < 4; k++) c->res[4 * (size_t)i + k] = r[k];
        c->dt[i] = fmin(c->area[i] * c->p.cfl / T, c->p.dt_cap);
    }
    /* global_dt option: the smallest local step for every cell, the intent
     * of the reference's disabled kernel_TimeStep (gpu_solver.cu:880-936) */
    if (c->p.global_dt) {
        double m = INFINITY;
        for (int i = 1; i <= c->ncell; i++) m = fmin(m, c->dt[i]);
        for (int i = 1; i <= c->ncell; i++) c->dt[i] = m;
    }
}

/* gpu_solver.cu:1635-1720 (kernel_Smooth1 / kernel_Smooth2), generalised to
 * any sweep count: R_0 = Res, R_j = (eps * sum_interior R_{j-1} + Res) /
 * (1 + eps * CLog), and after the last sweep each component of Res takes the
 * smoothed value only where that has the smaller magnitude.  Two sweeps is
 * the reference's fixed choice. */
static void stage_smooth(or_case *c) {
    const int S = c->p.irs_sweeps;
    const double eps = c->p.irs_eps;
    if (S <= 0) return;
    const double *src = c->res;
    for (int s = 0; s < S; s++) {
        double *dst = (s % 2 == 0) ? c->r1 : c->r2;
        #pragma omp parallel for schedule(static)
        for (int i = 1; i <= c->ncell; i++) {
            double data[4] = {0.0, 0.0, 0.0, 0.0};
            const int *nb = c->neicell + 3 * (size_t)i;
            for (int k = 0; k < 4; k++) {
                if (nb[0] > 0) data[k] += src[4 * (size_t)nb[0] + k];
                if (nb[1] > 0) data[k] += src[4 * (size_t)nb[1] + k];
                if (nb[2] > 0) data[k] += src[4 * (size_t)nb[2] + k];
            }
            for (int k = 0; k < 4; k++)
                dst[4 * (size_t)i + k] = (data[k] * (eps) + c->res[4 * (size_t)i + k]) /
                                         (1.0 + (eps) * c->clog[i]);
        }
        src = dst;
    }
    #pragma omp parallel for schedule(static)
    for (int i = 1; i <= c->ncell; i++)
        for (int k = 0; k < 4; k++) {
            double sm = src[4 * (size_t)i + k];
            if (fabs(c->res[4 * (size_t)i + k]) > fabs(sm)) c->res[4 * (size_t)i + k] = sm;
        }
}

/* gpu_solver.cu:938-966 (kernel_RKStep) */
static void stage_rk(or_case *c, double a) {
    const double g = c->p.gamma;
    #pragma omp parallel for schedule(static)
    for (int i = 1; i <= c->ncell; i++) {
        double RK = a;
        RK *= c->dt[i];
        const double *r = c->res + 4 * (size_t)i;
        wst ww;
        memset(&ww, 0, sizeof ww);
        ww.d = c->w0[i].d - RK * r[0] / c->area[i];
        ww.du = c->w0[i].du - RK * r[1] / c->area[i];
        ww.dv = c->w0[i].dv - RK * r[2] / c->area[i];
        ww.de = c->w0[i].de - RK * r[3] / c->area[i];
        calc_pta(&ww, g);
        c->w[i] = ww;
    }
}

/* gpu_solver.cu:968-1020 (kernel_drou) + 2409-2415: sum of (rho-rho0)^2.
 * Summed in fixed blocks of 4096 cells so the value does not depend on the
 * thread count. */
static double stage_drou(const or_case *c) {
    const int B = 4096;
    int nb = (c->ncell + B - 1) / B;
    double *part = xcalloc(nb, sizeof(double));
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; b++) {
        double s = 0.0;
        int lo = 1 + b * B, hi = lo + B - 1 < c->ncell ? lo + B - 1 : c->ncell;
        for (int i = lo; i <= hi; i++) {
            double d = c->w[i].d - c->w0[i].d;
            s += d * d;
        }
        part[b] = s;
    }
    double s = 0.0;
    for (int b = 0; b < nb; b++) s += part[b];
    free(part);
    return s;
}

void or_stage_probe(or_case *c, double *ghost, double *grad, double *umm,
                    double *flux, double *sr, double *res, double *dt) {
    stage_boundary(c);
    stage_gradient(c);
    stage_cell_limiter(c);
    stage_flux(c);
    stage_e2c(c);
    for (int e = 1; e <= c->nedge; e++) {
        size_t k = e - 1;
        if (ghost) {
            const wst *G = NULL;
            if (c->elog[e] == 1) G = &c->farw[c->efar[e]];
            if (c->elog[e] == 2) G = &c->wallw[c->ewall[e]];
            ghost[4 * k] = G ? G->d : 0; ghost[4 * k + 1] = G ? G->du : 0;
            ghost[4 * k + 2] = G ? G->dv : 0; ghost[4 * k + 3] = G ? G->de : 0;
        }
        if (flux) for (int q = 0; q < 4; q++) flux[4 * k + q] = c->rel[4 * (size_t)e + q];
        if (sr) sr[k] = c->dtel[e];
    }
    for (int i = 1; i <= c->ncell; i++) {
        size_t k = i - 1;
        for (int q = 0; q < 8; q++) {
            if (grad) grad[8 * k + q] = c->du[8 * (size_t)i + q];
            if (umm) umm[8 * k + q] = q < 4 ? c->umax[4 * (size_t)i + q] : c->umin[4 * (size_t)i + q - 4];
        }
        if (res) for (int q = 0; q < 4; q++) res[4 * k + q] = c->res[4 * (size_t)i + q];
        if (dt) dt[k] = c->dt[i];
    }
}

/* gpu_solver.cu:2200-2434 (ROE_SOLVER main loop) */
int or_run(or_case *c, int nsteps, double *resid) {
    int done = 0;
    while (done < nsteps && c->last_resd > c->p.epsl) {
        c->step++;
        for (int i = 1; i <= c->ncell; i++) {
            c->w0[i].d = c->w[i].d; c->w0[i].du = c->w[i].du;
            c->w0[i].dv = c->w[i].dv; c->w0[i].de = c->w[i].de;
        }
        double drou = 0.0;
        for (int s = 0; s < c->p.rk_stages; s++) {
            stage_boundary(c);
            stage_gradient(c);
            stage_cell_limiter(c);
            stage_flux(c);
            stage_e2c(c);
            stage_smooth(c);
            stage_rk(c, c->p.rk_coef[s]);
            if (s == c->p.rk_stages - 1) drou = stage_drou(c);
        }
        if (c->step == 1) c->epsm = drou;
        c->last_resd = sqrt((drou + 1.0E-32) / c->epsm);
        if ((c->p.limiter_freeze > 0 && c->step >= c->p.limiter_freeze) ||
            (c->p.limiter_freeze_resd > 0.0 && c->last_resd <= c->p.limiter_freeze_resd))
            c->frozen = 1;
        if (resid) resid[done] = c->last_resd;
        done++;
    }
    return done;
}

/* ------------------------------------------------------------------ */
/* Morton order (no counterpart in the reference)                      */
/* ------------------------------------------------------------------ */

static uint64_t spread21(uint64_t v) {
    v &= 0x1fffffULL;
    v = (v | (v << 32)) & 0x1f00000000ffffULL;
    v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}

typedef struct mk { uint64_t code; int id; } mk;

static int mk_cmp(const void *a, const void *b) {
    const mk *x = a, *y = b;
    if (x->code != y->code) return x->code < y->code ? -1 : 1;
    return x->id < y->id ? -1 : (x->id > y->id);
}

/* Cells sorted by the 2 x 21-bit Morton code of the centroid quantised on its
 * bounding box: q = (unsigned)((c - min) / (max - min) * 2097151.0). */
void or_morton_perm(const or_case *c, int *perm) {
    double x0 = c->cx[1], x1 = c->cx[1], y0 = c->cy[1], y1 = c->cy[1];
    for (int i = 2; i <= c->ncell; i++) {
        if (c->cx[i] < x0) x0 = c->cx[i];
        if (c->cx[i] > x1) x1 = c->cx[i];
        if (c->cy[i] < y0) y0 = c->cy[i];
        if (c->cy[i] > y1) y1 = c->cy[i];
    }
    double sx = x1 > x0 ? x1 - x0 : 1.0, sy = y1 > y0 ? y1 - y0 : 1.0;
    mk *a = xcalloc(c->ncell, sizeof(mk));
    for (int i = 1; i <= c->ncell; i++) {
        uint64_t qx = (uint64_t)((c->cx[i] - x0) / sx * 2097151.0);
        uint64_t qy = (uint64_t)((c->cy[i] - y0) / sy * 2097151.0);
        a[i - 1].code = spread21(qx) | (spread21(qy) << 1);
        a[i - 1].id = i;
    }
    qsort(a, c->ncell, sizeof(mk), mk_cmp);
    for (int k = 0; k < c->ncell; k++) perm[k] = a[k].id;
    free(a);
}

/* ------------------------------------------------------------------ */
/* Reverse Cuthill-McKee order (no counterpart in the reference)       */
/* ------------------------------------------------------------------ */

/* Breadth-first over interior neighbours (neicell > 0).  A component starts
 * at its unvisited cell of smallest degree (CLog), smallest id among equals;
 * the unvisited neighbours of each dequeued cell join the queue by (degree,
 * id); the resulting sequence is reversed.  perm[k] = 1-based file id. */
static const int *rcm_deg;

static int rcm_cmp(const void *a, const void *b) {
    int x = *(const int *)a, y = *(const int *)b;
    if (rcm_deg[x] != rcm_deg[y]) return rcm_deg[x] < rcm_deg[y] ? -1 : 1;
    return x < y ? -1 : (x > y);
}

void or_rcm_perm(const or_case *c, int *perm) {
    const int N = c->ncell;
    int *order = xcalloc(N, sizeof(int));
    char *seen = xcalloc(N + 1, 1);
    int *cand = xcalloc(N, sizeof(int));
    rcm_deg = c->clog;
    for (int i = 0; i < N; i++) cand[i] = i + 1;
    qsort(cand, N, sizeof(int), rcm_cmp); /* start candidates by (degree, id) */
    int n = 0, next = 0;
    while (n < N) {
        while (seen[cand[next]]) next++;
        int head = n;
        order[n++] = cand[next];
        seen[cand[next]] = 1;
        while (head < n) {
            int i = order[head++], nb[3], k = 0;
            for (int f = 0; f < 3; f++) {
                int q = c->neicell[3 * i + f];
                if (q > 0 && !seen[q]) { nb[k++] = q; seen[q] = 1; }
            }
            qsort(nb, k, sizeof(int), rcm_cmp);
            for (int f = 0; f < k; f++) order[n++] = nb[f];
        }
    }
    for (int k = 0; k < N; k++) perm[k] = order[N - 1 - k];
    free(order); free(seen); free(cand);
}

/* ------------------------------------------------------------------ */
/* NACA 0012 O-grid (no reference counterpart: it writes the reference's */
/* mesh format, gpu_init.cu:16-32).  A second statement of the          */
/* library's generator, so that the CPU arm of the benchmark and tests  */
/* can make the same mesh without loading the product library.          */
/* ------------------------------------------------------------------ */

/* splitmix64 finaliser */
static uint64_t og_mix(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

/* uniform [0, 1) with 53 random bits; stream 1/2 jitter x/y, 3 diagonals */
static double og_unit(uint64_t seed, uint64_t stream, uint64_t idx) {
    const uint64_t h = og_mix(seed ^ og_mix(stream * 0x632be59bd9b4e019ULL + idx));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

/* half thickness of NACA 0012 with the closed trailing edge (a4 = -0.1036) */
static double og_thick(double x) {
    if (x < 0.0) x = 0.0;
    if (x > 1.0) x = 1.0;
    return 0.6 * (0.2969 * sqrt(x) - 0.1260 * x - 0.3516 * x * x + 0.2843 * x * x * x -
                  0.1036 * x * x * x * x);
}

/* total of nj geometric steps of first size ds0 and ratio r */
static double og_total(double ds0, double r, int nj) { return ds0 * (pow(r, nj) - 1.0) / (r - 1.0); }

int or_ogrid_naca0012(int ni, int nj, double r_far, double dy_wall, double jitter, uint64_t seed,
                      double *x, double *y, int *tri) {
    if (ni < 8 || nj < 1 || r_far <= 1.0 || dy_wall <= 0 || jitter < 0 || jitter >= 0.25) {
        set_err("ogrid: need ni>=8, nj>=1, r_far>1, dy_wall>0, 0<=jitter<0.25");
        return -1;
    }
    const double pi = 3.14159265358979323846;
    double *wx = xcalloc(ni, sizeof(double)), *wy = xcalloc(ni, sizeof(double));
    double *fx = xcalloc(ni, sizeof(double)), *fy = xcalloc(ni, sizeof(double));
    double *s = xcalloc(nj + 1, sizeof(double));
    /* wall points from the trailing edge around the upper surface, far-field
       circle about mid-chord at the same angles */
    for (int i = 0; i < ni; i++) {
        const double th = 2.0 * pi * i / ni, xw = 0.5 * (1.0 + cos(th));
        wx[i] = xw;
        wy[i] = (i == 0 || 2 * i == ni) ? 0.0 : (2 * i <= ni ? 1.0 : -1.0) * og_thick(xw);
        fx[i] = 0.5 + r_far * cos(th);
        fy[i] = r_far * sin(th);
    }
    /* radial fractions: geometric steps whose first is dy_wall/(r_far-0.5),
       ratio found by 200 bisections */
    double ds0 = dy_wall / (r_far - 0.5), ratio = 1.0;
    if (ds0 * nj < 1.0) {
        double lo = 1.0, hi = 2.0;
        while (og_total(ds0, hi, nj) < 1.0) hi *= 2.0;
        for (int it = 0; it < 200; it++) {
            const double mid = 0.5 * (lo + hi);
            if (og_total(ds0, mid, nj) < 1.0) lo = mid; else hi = mid;
        }
        ratio = 0.5 * (lo + hi);
    } else {
        ds0 = 1.0 / nj;
    }
    s[0] = 0.0;
    for (int j = 1; j <= nj; j++) s[j] = s[j - 1] + ds0 * pow(ratio, j - 1);
    for (int j = 0; j <= nj; j++) s[j] /= s[nj];
    /* nodes: row j = ni points; interior rows jittered by up to `jitter`
       times the distance to the nearest structured neighbour */
    for (int j = 0; j <= nj; j++)
        for (int i = 0; i < ni; i++) {
            double px = wx[i] + s[j] * (fx[i] - wx[i]);
            double py = wy[i] + s[j] * (fy[i] - wy[i]);
            if (j > 0 && j < nj && jitter > 0) {
                const int di[4] = {1, -1, 0, 0}, dj[4] = {0, 0, 1, -1};
                double h = 1e300;
                for (int q = 0; q < 4; q++) {
                    const int ii = (i + di[q] + ni) % ni, jj = j + dj[q];
                    const double qx = wx[ii] + s[jj] * (fx[ii] - wx[ii]);
                    const double qy = wy[ii] + s[jj] * (fy[ii] - wy[ii]);
                    const double d = hypot(qx - px, qy - py);
                    if (d < h) h = d;
                }
                const uint64_t idx = (uint64_t)j * ni + i;
                px += jitter * h * (2.0 * og_unit(seed, 1, idx) - 1.0);
                py += jitter * h * (2.0 * og_unit(seed, 2, idx) - 1.0);
            }
            x[(size_t)j * ni + i] = px;
            y[(size_t)j * ni + i] = py;
        }
    /* two counter-clockwise triangles per quad, split along a seeded diagonal */
    int *t = tri;
    for (int j = 0; j < nj; j++)
        for (int i = 0; i < ni; i++) {
            const int a = j * ni + i + 1, b = j * ni + (i + 1) % ni + 1;
            const int c = (j + 1) * ni + (i + 1) % ni + 1, d = (j + 1) * ni + i + 1;
            const int q[2][6] = {{a, d, c, a, c, b}, {a, d, b, b, d, c}};
            const int pick = og_unit(seed, 3, (uint64_t)j * ni + i) < 0.5 ? 0 : 1;
            memcpy(t, q[pick], sizeof q[pick]);
            t += 6;
        }
    free(wx); free(wy); free(fx); free(fy); free(s);
    for (int cc = 0; cc < 2 * ni * nj; cc++) {
        const int *p = tri + 3 * cc;
        const double ar = calc_area(x[p[0] - 1], y[p[0] - 1], x[p[1] - 1], y[p[1] - 1], x[p[2] - 1], y[p[2] - 1]);
        if (!(ar > 0.0)) { set_err("ogrid: generated a non-positive cell; lower the jitter"); return -2; }
    }
    return 0;
}
