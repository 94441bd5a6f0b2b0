/*
 * e2d_oracle.h -- CPU FP64 restatement of the GPUEularSolver2D solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the GPU library is
 * compared against (tests/, __graft_entry__.smoke() and the cpu_baseline leg
 * of bench.py).  It is never linked into, loaded by or called from the
 * product library.
 *
 * The restatement follows the reference's GPU kernels (gpu_solver.cu) in
 * operation order, because those kernels -- not the loose CPU helpers in the
 * same file -- are what the reference runs.  Arrays are 1-based exactly like
 * the reference (index 0 unused), so cell and edge ids compare directly.
 *
 * Pinning: the mesh set-up (CalculationMeshGeo + changeEdge), the initial
 * state, and the stage-1 boundary ghosts, gradients, limiter bounds and face
 * fluxes are checked against the reference's own host functions compiled in
 * place (oracle/build_ref.py) and against golden vectors generated from them
 * (tests/golden/).
 */
#ifndef E2D_ORACLE_H
#define E2D_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_params {
    /* the eight values of the reference input.dat (gpu_init.cu:41) */
    double ma, alpha_deg, gamma, pin, tin, cfl, epsl;
    int maxstep;
    /* scheme constants that the reference hard-codes */
    int rk_stages;            /* gpu_solver.cu:2211 loops 4 stages        */
    double rk_coef[8];        /* gpu_fvm.cu:10 {0.0833,0.2069,0.4265,1.0} */
    double irs_eps;           /* gpu_solver.cu:1633 (#define eps 0.8)      */
    int irs_sweeps;           /* gpu_solver.cu:1722-1728: two sweeps       */
    double dt_cap;            /* gpu_solver.cu:831 fmin(..., 0.1)          */
    double entropy_eps;       /* gpu_solver.cu:603 epsilon=0.05            */
    double wall_box;          /* gpu_init.cu:190 |mid|<2.0                 */
    int limiter_freeze;       /* option without reference counterpart: > 0
                                 reuses the limiter values of the last stage
                                 of iteration k from iteration k+1 on      */
    int limiter;              /* 0 reference; 1 Venkatakrishnan option     */
    double limiter_k;         /* K of the Venkatakrishnan option           */
    double limiter_freeze_resd; /* option: freeze once Resd <= this        */
    int global_dt;            /* option: every cell uses min_j dt_j         */
    int far_field_fix;        /* option: supersonic test against 1/M        */
    int first_order_iters;    /* option: first-order faces while step <= k  */
    int positivity_fix;       /* option: non-physical face side -> cell state */
} or_params;

typedef struct or_case or_case;

/* Reference defaults for every field; the input.dat fields get M0.5, a0,
 * gamma 1.4, p 101325, T 288.15, CFL 1, EPSL 1e-6, 100 steps. */
void or_params_default(or_params *p);

/* Parse an input.dat file: "MA ALPHA GAMA PIN TIN CFL EPSL MAXSTEP". */
int or_read_input(const char *path, or_params *p);

/* Read a reference .dat mesh (gpu_init.cu:16-32) and build the case. */
or_case *or_create_from_file(const char *mesh_path, const or_params *p);

/* Same from arrays: x,y [nnode], tri [3*ncell] with 1-based node ids. */
or_case *or_create(int nnode, int ncell, const double *x, const double *y,
                   const int *tri, const or_params *p);
void or_destroy(or_case *c);
const char *or_last_error(void);

/* Counts: out[0..4] = ncell, nnode, nedge, nwall, nfar. */
void or_counts(const or_case *c, int out[5]);

/* Set-up outputs in reference numbering (after changeEdge).
 *   ei  [nedge*7]: ELog, left, right, farfieldid, wallid, node1, node2
 *   ed  [nedge*5]: vectorn, vectorx, vectory, midx, midy
 *   ci  [ncell*7]: CLog, celledge[0..2], neicell[0..2]
 *   cd  [ncell*3]: area, centre x, centre y
 * Any pointer may be NULL. */
void or_topology(const or_case *c, int *ei, double *ed, int *ci, double *cd);

/* Conserved state, cell-major [ncell*4] (rho, rho u, rho v, rho E). */
void or_get_state(const or_case *c, double *w);
int or_set_state(or_case *c, const double *w);
/* Primitive copy [ncell*3] (P, T, A) as the reference stores it. */
void or_get_pta(const or_case *c, double *pta);
double or_pis(const or_case *c);

/* Run the reference loop (gpu_solver.cu:2200-2434): at most nsteps more
 * iterations, stopping early when Resd <= epsl.  resid[k] receives Resd of
 * each iteration run by this call.  Returns the number of iterations run. */
int or_run(or_case *c, int nsteps, double *resid);
int or_step_count(const or_case *c);

/* One stage of intermediates for checks against the reference's host
 * functions, evaluated from the current state without advancing it:
 *   ghost [(nedge)*4]    : far/wall ghost state per boundary edge, 0 else
 *   grad  [ncell*8]      : deltU[0][0..3], deltU[1][0..3]
 *   umm   [ncell*8]      : Umax[0..3], Umin[0..3]
 *   flux  [nedge*4]      : face flux times vectorn (Res_e.left)
 *   sr    [nedge]        : spectral radius (deltT_e.left)
 *   res   [ncell*4], dt [ncell] : edge->cell gather and local time step */
void or_stage_probe(or_case *c, double *ghost, double *grad, double *umm,
                    double *flux, double *sr, double *res, double *dt);

/* Morton order of cell centroids: perm[k] = 1-based file id of the cell that
 * sits at position k.  Ties keep file order. */
void or_morton_perm(const or_case *c, int *perm);

/* Reverse Cuthill-McKee order of the interior-face adjacency: breadth-first
 * from the smallest-degree cell (smallest id among equals), neighbours queued
 * by (degree, id), sequence reversed.  perm[k] = 1-based file id. */
void or_rcm_perm(const or_case *c, int *perm);

/* Point kernels, for function-level known-answer checks. */
void or_roe_flux(const double lw[4], const double rw[4], double nx, double ny,
                 double gamma, double entropy_eps, double flux[4]);
void or_far_ghost(const double dw[4], double vectorx, double vectory,
                  const or_case *c, double out[4]);

/* NACA 0012 O-grid of ni (around) x nj (radial) quads, each split into two
 * counter-clockwise triangles along a seeded diagonal; far-field circle of
 * radius r_far about mid-chord, first radial spacing dy_wall, interior nodes
 * jittered by up to `jitter` of their nearest-neighbour distance.  Writes
 * x, y [ni*(nj+1)] and tri [6*ni*nj] (1-based node ids).  Returns 0, or < 0
 * with or_last_error() set.  The same mesh, bit for bit, as the library's
 * e2d_mesh_ogrid_naca0012 with the same arguments. */
int or_ogrid_naca0012(int ni, int nj, double r_far, double dy_wall, double jitter, uint64_t seed,
                      double *x, double *y, int *tri);

/* Threads used by OpenMP loops (1 when built without OpenMP). */
int or_threads(void);
void or_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
