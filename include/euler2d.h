/*
 * euler2d.h -- C ABI of the GB300 cell-centred finite-volume Euler solver
 * for triangle meshes (libeuler2d.so).
 *
 * The library is a drop-in for the solve path of GPUEularSolver2D: it reads
 * the same mesh and input files, builds the same edge numbering, runs the same
 * scheme (far-field Riemann-invariant and slip-wall ghosts, Green-Gauss
 * gradient, per-face Barth-Jespersen-type limited MUSCL reconstruction, Roe
 * flux with Harten entropy fix, local time step, implicit residual smoothing,
 * multistage Runge-Kutta) and reports the same residual history.  Reference
 * functions are cited as file:line of that project.
 *
 * Conventions (new; the reference has no error handling):
 *   - every function returns an int status: 0 success, < 0 error, and
 *     e2d_last_error() describes the last error of the calling thread;
 *   - opaque handles own all their host and device memory;
 *   - a solver is bound to one CUDA stream and must be driven from one thread
 *     at a time;
 *   - cell data crossing this interface is in FILE order (the order of the
 *     cells in the mesh file, 0-based here, 1-based in the reference), whatever
 *     internal renumbering the solver uses;
 *   - conserved variables are (rho, rho u, rho v, rho E), non-dimensional with
 *     rho_inf = 1 and |V_inf| = 1 as in the reference (gpu_init.cu:63-93).
 */
#ifndef EULER2D_H
#define EULER2D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define E2D_OK 0
#define E2D_ERR_ARG -1       /* bad argument                            */
#define E2D_ERR_IO -2        /* file cannot be opened / parsed          */
#define E2D_ERR_MESH -3      /* invalid mesh (area <= 0, non-manifold)  */
#define E2D_ERR_CUDA -4      /* CUDA runtime error / no device          */
#define E2D_ERR_DIVERGED -5  /* non-positive density or pressure, NaN   */
#define E2D_ERR_CAPACITY -6  /* request beyond a fixed capacity         */

#define E2D_FP64 0           /* FP64 stencil (parity variant)          */
#define E2D_FP32 1           /* FP32 stencil, FP64 geometry and norms  */

#define E2D_ORDER_FILE 0     /* cells in file order                    */
#define E2D_ORDER_MORTON 1   /* cells sorted by centroid Morton code   */
#define E2D_ORDER_RCM 2      /* reverse Cuthill-McKee of cell adjacency */

typedef struct e2d_mesh e2d_mesh;
typedef struct e2d_solver e2d_solver;
typedef struct e2d_batch e2d_batch;

/* Solver parameters.  The first eight fields are the reference's input.dat
 * (gpu_init.cu:41); the rest are constants the reference hard-codes, exposed
 * with the reference values as defaults. */
typedef struct e2d_params {
    double ma;           /* free-stream Mach number              (MA)      */
    double alpha_deg;    /* angle of attack, degrees             (ALPHA)   */
    double gamma;        /* ratio of specific heats              (GAMA)    */
    double pin;          /* free-stream pressure, Pa             (PIN)     */
    double tin;          /* free-stream temperature, K           (TIN)     */
    double cfl;          /* CFL number                           (CFL)     */
    double epsl;         /* stop when Resd <= epsl               (EPSL)    */
    int32_t maxstep;     /* iteration limit                      (MAXSTEP) */
    int32_t rk_stages;   /* 1..8; reference 4 (gpu_solver.cu:2211)         */
    double rk_coef[8];   /* reference {0.0833,0.2069,0.4265,1.0} (gpu_fvm.cu:10) */
    double irs_eps;      /* smoothing coefficient; reference 0.8 (gpu_solver.cu:1633) */
    int32_t irs_sweeps;  /* 0 = off; reference 2 (gpu_solver.cu:1722-1728) */
    int32_t precision;   /* E2D_FP64 (default) or E2D_FP32                 */
    double dt_cap;       /* local time step cap; reference 0.1 (gpu_solver.cu:831) */
    double entropy_eps;  /* Harten fix width; reference 0.05 (gpu_solver.cu:603) */
    double wall_box;     /* boundary face is wall if |mid x|,|mid y| < wall_box;
                            reference 2.0 (gpu_init.cu:190)                 */
    int32_t ordering;    /* E2D_ORDER_FILE (default), _MORTON or _RCM        */
    int32_t block_size;  /* threads per CTA, 0 = tuned default              */
    int32_t graph_iters; /* iterations captured per CUDA graph, 0 = default */
    int32_t verbose;     /* e2d_solve prints "step,resid" lines like the
                            reference (gpu_solver.cu:2433) when nonzero     */
    int32_t limiter_freeze; /* option, no reference counterpart: 0 (default,
                            reference) re-evaluates the limiter every stage;
                            k > 0 freezes the per-face limiter values from
                            iteration k on, so the residual can fall below
                            the limiter's chatter floor                     */
    int32_t limiter;     /* E2D_LIMITER_REFERENCE (default): the reference's
                            per-face min((Umax-U)/d, 1) (gpu_solver.cu:456-494);
                            E2D_LIMITER_VENKAT: option, no reference
                            counterpart -- the smooth Venkatakrishnan form on
                            the same per-face differences, eps^2 = (K h)^3,
                            h = sqrt(cell area); E2D_LIMITER_CELL_BARTH /
                            E2D_LIMITER_CELL_VENKAT: options, one value per
                            cell and component, the minimum over the cell's
                            interior faces of the reference / Venkatakrishnan
                            per-face value                                   */
    double limiter_k;    /* K of E2D_LIMITER_VENKAT (default 5)              */
    double limiter_freeze_resd; /* option, no reference counterpart: > 0
                            freezes the limiter values once Resd falls to
                            this level (whichever of this and limiter_freeze
                            comes first)                                     */
    int32_t global_dt;   /* 0 (default): local time step per cell (the
                            reference's loop); 1: every cell advances with
                            the smallest local step of the mesh, as the
                            reference's disabled kernel_TimeStep
                            (gpu_solver.cu:880-936, 2376-2387) intended      */
    int32_t far_field_fix; /* 0 (default): the reference's supersonic test
                            Un / AIN > 1 with the dimensional AIN, which never
                            holds (gpu_solver.cu:79); 1: compares with the
                            non-dimensional free-stream sound speed 1/M     */
    int32_t first_order_iters; /* option, no reference counterpart: 0
                            (default) reconstructs every interior face
                            (gpu_solver.cu:496-549); k > 0 uses the cell
                            states themselves (first order, as the
                            reference's boundary faces, 689-725) during the
                            first k iterations of the solver's history      */
    int32_t positivity_fix; /* option, no reference counterpart: 0 (default)
                            keeps every limited reconstruction; 1 replaces a
                            face side whose reconstructed density or
                            pressure is not positive by the cell state      */
} e2d_params;

#define E2D_LIMITER_REFERENCE 0
#define E2D_LIMITER_VENKAT 1
#define E2D_LIMITER_CELL_BARTH 2  /* option: per cell and component, the smallest
                                     of the reference's per-face values over the
                                     cell's interior faces (Barth-Jespersen)   */
#define E2D_LIMITER_CELL_VENKAT 3 /* option: the same with the Venkatakrishnan
                                     form                                      */

typedef struct e2d_mesh_info {
    int32_t ncell, nnode, nedge, nwall, nfar;
} e2d_mesh_info;

/* ---- errors ----------------------------------------------------------- */
const char *e2d_last_error(void);
const char *e2d_version(void);

/* ---- parameters ------------------------------------------------------- */
/* Reference defaults (input.dat fields: M 0.5, alpha 0, gamma 1.4,
 * p 101325 Pa, T 288.15 K, CFL 1, EPSL 1e-6, MAXSTEP 100). */
int e2d_params_default(e2d_params *p);
/* Reads input.dat: "MA ALPHA GAMA PIN TIN CFL EPSL MAXSTEP" (gpu_init.cu:34-42);
 * fields not in the file are left as they are in *p. */
int e2d_input_read(const char *path, e2d_params *p);

/* ---- meshes ----------------------------------------------------------- */
/* Reads a reference .dat mesh: "Nnode Ncell", Nnode x, Nnode y, then 3
 * 1-based CCW node ids per cell (gpu_init.cu:5-33, replaces inputMesh). */
int e2d_mesh_read(const char *path, e2d_mesh **out);
/* Writes the same format (%.17g, so a read gives back the same doubles). */
int e2d_mesh_write(const char *path, const e2d_mesh *m);
/* Binary cache of the same mesh ("E2DMESH1", int32 nnode, int32 ncell,
 * double x[nnode], double y[nnode], int32 tri[3*ncell]; little-endian), about
 * 10x faster to read than the text format.  e2d_mesh_read recognises it by
 * its first 8 bytes, so either file works wherever a mesh path is taken. */
int e2d_mesh_write_binary(const char *path, const e2d_mesh *m);
/* Builds a mesh from arrays: x,y [nnode]; tri [3*ncell] 1-based node ids. */
int e2d_mesh_from_arrays(int32_t nnode, int32_t ncell, const double *x, const double *y,
                         const int32_t *tri, e2d_mesh **out);
/* O-grid around NACA 0012 (chord 1, closed trailing edge): ni points around,
 * nj cell layers out to a circle of radius r_far chords, first wall spacing
 * dy_wall chords with geometric stretching, each quad split along a seeded
 * random diagonal and interior nodes jittered by +-jitter of the local
 * spacing.  Writes 2*ni*nj cells and ni*(nj+1) nodes.  No reference
 * counterpart. */
int e2d_mesh_ogrid_naca0012(int32_t ni, int32_t nj, double r_far, double dy_wall,
                            double jitter, uint64_t seed, e2d_mesh **out);
void e2d_mesh_free(e2d_mesh *m);
/* Runs the set-up (geometry, edge discovery, boundary tags) if needed. */
int e2d_mesh_info_get(e2d_mesh *m, double wall_box, e2d_mesh_info *info);
/* Set-up in reference numbering, after the interior/far/wall partition of
 * changeEdge (gpu_solver.cu:1832-1906); all ids 1-based as in the reference.
 *   ei [nedge*7]: ELog, left_cell, right_cell, farfieldid, wallid, node1, node2
 *   ed [nedge*5]: vectorn, vectorx, vectory, midx, midy
 *   ci [ncell*7]: CLog, celledge[0..2], neicell[0..2]
 *   cd [ncell*3]: area, centre x, centre y
 * Replaces CalculationMeshGeo (gpu_init.cu:100-228); any pointer may be NULL. */
int e2d_mesh_topology(e2d_mesh *m, double wall_box, int32_t *ei, double *ed, int32_t *ci,
                      double *cd);
/* Mesh nodes and cells: x,y [nnode], tri [3*ncell] (1-based). */
int e2d_mesh_nodes(const e2d_mesh *m, double *x, double *y, int32_t *tri);
/* Cell order used by a given ordering: perm[k] = 0-based file index of the
 * cell at internal position k.  No reference counterpart. */
int e2d_mesh_order(e2d_mesh *m, int32_t ordering, int32_t *perm);

/* ---- solver ----------------------------------------------------------- */
/* Set-up + device upload + free-stream state (gpu_init.cu:63-93,
 * gpu_solver.cu:2187-2194); replaces Initialization, Cuda_Init and the
 * set-up half of ROE_SOLVER.  Uses the current CUDA device.  Parameters out
 * of range (see e2d_params; also gamma <= 1, ma, tin, cfl, dt_cap,
 * entropy_eps or wall_box <= 0, irs_eps < 0, a non-finite coefficient or a
 * NaN epsl) give E2D_ERR_ARG, with the parameter named by e2d_last_error. */
int e2d_solver_create(e2d_mesh *m, const e2d_params *p, e2d_solver **out);
void e2d_solver_destroy(e2d_solver *s);
/* Iterates like ROE_SOLVER (gpu_solver.cu:2200-2434): stops when
 * Resd <= epsl or after max_steps more iterations.  resid_history receives
 * Resd of each iteration run (may be NULL); *nsteps the number run. */
int e2d_solve(e2d_solver *s, int32_t max_steps, double epsl, double *resid_history,
              int32_t *nsteps);
/* Exactly n iterations, no convergence stop (residuals are still recorded). */
int e2d_step(e2d_solver *s, int32_t n);
/* Total iterations so far and the last Resd. */
int e2d_progress(e2d_solver *s, int32_t *step, double *resd);
/* Residual history Resd[1..step] of every iteration so far (cap entries). */
int e2d_residual_history(e2d_solver *s, double *out, int32_t cap, int32_t *n);
/* Residual normalisation: Resd = sqrt((drou + 1e-32) / epsm); by default
 * epsm is drou of iteration 1 (gpu_solver.cu:2428).  Setting it > 0 fixes it. */
int e2d_set_residual_norm(e2d_solver *s, double epsm);
int e2d_get_residual_norm(e2d_solver *s, double *epsm);
/* Conserved state in file order, [ncell*4] FP64. */
int e2d_get_state(e2d_solver *s, double *w);
int e2d_set_state(e2d_solver *s, const double *w);
/* Lift and drag coefficients from the wall pressure of the wall cells
 * (sum over wall faces of (p - p_inf) S, rotated by alpha, divided by
 * 0.5 rho_inf V_inf^2 c = 0.5), accumulated in FP64.  No reference
 * counterpart. */
int e2d_forces(e2d_solver *s, double *cl, double *cd);
/* FP64 integrals of a conserved state.  No reference counterpart.
 *   cl, cd          as e2d_forces;
 *   mass            sum over cells of rho * area;
 *   mass_flux_far   mass leaving through the far-field faces per unit time:
 *                   the scheme's first-order boundary flux (far-field ghost,
 *                   gpu_solver.cu:62-135, and the Roe flux, 569-647) times
 *                   the face length, summed;
 *   mass_flux_wall  the same through the wall faces (slip-wall ghost,
 *                   gpu_solver.cu:188-221).
 * Interior faces cancel in the sum of the cell residuals, so the mass
 * residual summed over the cells is mass_flux_far + mass_flux_wall, which
 * tends to zero as the solution becomes steady. */
typedef struct e2d_integrals {
    double cl, cd, mass, mass_flux_far, mass_flux_wall;
} e2d_integrals;
/* Of the solver's current state. */
int e2d_solver_integrals(e2d_solver *s, e2d_integrals *out);
/* Of a state w [ncell * 4] in the file's cell order on a mesh with the given
 * parameters (free stream, gamma, entropy fix, wall box, far-field option);
 * needs no GPU. */
int e2d_state_integrals(e2d_mesh *m, const e2d_params *p, const double *w, e2d_integrals *out);
/* unresidual.plt as the reference writes it (gpu_fvm.cu:165-175): every
 * 100th step. */
int e2d_write_residual_plt(e2d_solver *s, const char *path);
/* unresult.plt (gpu_fvm.cu:143-163): area-weighted node averages of rho,
 * u, v, P, T and Mach (Node_Computing, gpu_fvm.cu:71-131) of the solver's
 * current state on mesh m (the mesh the solver was created from). */
int e2d_write_field_plt(e2d_solver *s, e2d_mesh *m, const char *path);
/* unairfoilpress.plt (gpu_fvm.cu:177-192): -2 (P - P_inf) at both nodes of
 * every wall face, in wall-face order. */
int e2d_write_wall_cp_plt(e2d_solver *s, e2d_mesh *m, const char *path);
/* Parameters the solver was created with. */
int e2d_get_params(e2d_solver *s, e2d_params *p);
/* Switches the stencil between E2D_FP32 and E2D_FP64 in place: the state is
 * carried over (rounded to FP32 when going down), and the iteration count,
 * residual normalisation and history continue.  The usual use is a fast FP32
 * solve to about 1e-4 followed by FP64 below the FP32 state's rounding floor.
 * Refused while limiter values are frozen (they live in the old precision). */
int e2d_set_precision(e2d_solver *s, int32_t precision);
/* Device time of the kernels of the last e2d_step/e2d_solve call, ms,
 * measured with CUDA events on the solver's stream. */
int e2d_last_device_ms(e2d_solver *s, double *ms);
/* Kernel launches per iteration (all passes of all stages). */
int e2d_launches_per_iteration(e2d_solver *s, int32_t *n);
/* Runs iters iterations launching the kernels one by one (no graph) with a
 * CUDA event pair around every launch, and returns the summed device time per
 * pass kind: ms[0] ghosts+gradient+reconstruction (pass A), ms[1] flux
 * gather (pass B), ms[2] smoothing sweeps (pass C), ms[3] smoothing + RK
 * update (pass D), ms[4] residual; launches[k] (may be NULL) the launch
 * counts.  The iterations advance the solution like e2d_step. */
int e2d_profile_passes(e2d_solver *s, int32_t iters, double *ms, int32_t *launches);
/* Sets the CUDA stream used by the solver (default: a stream it owns). */
int e2d_set_stream(e2d_solver *s, void *cuda_stream);

/* ---- batched cases ------------------------------------------------------
 * Many independent flow cases on meshes of uneven size advanced together on
 * one GPU: every pass is one launch over all cases, one CUDA graph covers
 * several iterations of all of them, and each case keeps its own residual
 * history and convergence test (a converged case stops while the others go
 * on).  Each case gives the same result, bit for bit, as a single-case solver
 * with the same parameters and block size.  No reference counterpart. */

/* params[c] of each case; cases must share precision, RK scheme, smoothing,
 * gamma, entropy fix and dt cap (per case: Mach, alpha, CFL, p, T, mesh).
 * The residual history holds max(params[].maxstep, 1024) iterations. */
int e2d_batch_create(e2d_mesh **meshes, const e2d_params *params, int32_t ncase, e2d_batch **out);
void e2d_batch_destroy(e2d_batch *b);
/* Exactly n iterations for every case that has not stopped. */
int e2d_batch_step(e2d_batch *b, int32_t n);
/* Each case iterates until its Resd <= epsl or max_steps more iterations;
 * nsteps[c] (may be NULL) receives the iterations each case ran. */
int e2d_batch_solve(e2d_batch *b, int32_t max_steps, double epsl, int32_t *nsteps);
int e2d_batch_info(e2d_batch *b, int32_t *ncase, int64_t *ncell_total, int64_t *ncell_padded);
int e2d_batch_get_state(e2d_batch *b, int32_t icase, double *w);
int e2d_batch_set_state(e2d_batch *b, int32_t icase, const double *w);
/* halted: 0 running, 1 stopped (converged / iteration target), 2 diverged. */
int e2d_batch_progress(e2d_batch *b, int32_t icase, int32_t *step, double *resd, int32_t *halted);
int e2d_batch_residual_history(e2d_batch *b, int32_t icase, double *out, int32_t cap, int32_t *n);
int e2d_batch_forces(e2d_batch *b, int32_t icase, double *cl, double *cd);
/* Launch shape: threads per CTA (a divisor of 256, >= 32) and CTAs per launch
 * (0: one per tile; fewer: persistent CTAs walking the tiles). */
int e2d_batch_set_launch(e2d_batch *b, int32_t block, int32_t grid);
int e2d_batch_get_launch(e2d_batch *b, int32_t *block, int32_t *grid);
/* Autotuner: times the candidate launch shapes on `iters` iterations each,
 * keeps the fastest, and restores the state.  cache_path (may be NULL) is a
 * JSON file of earlier results keyed by GPU, cell count, case count and
 * scheme; a hit is applied without timing, a new result is added. */
int e2d_batch_autotune(e2d_batch *b, const char *cache_path, int32_t iters, int32_t *block, int32_t *grid,
                       double *ms_per_iter);
/* e2d_batch_create with the cell order picked by the autotuner too: every
 * case's params.ordering is replaced by each of E2D_ORDER_MORTON,
 * E2D_ORDER_RCM and E2D_ORDER_FILE in turn, each candidate batch is
 * launch-tuned (e2d_batch_autotune, same cache), and the batch of the fastest
 * order and shape is returned; *ordering (may be NULL) receives the order.
 * The order changes only the memory layout: results are the same bits. */
int e2d_batch_create_tuned(e2d_mesh **meshes, const e2d_params *params, int32_t ncase, const char *cache_path,
                           int32_t iters, e2d_batch **out, int32_t *ordering);
int e2d_batch_last_device_ms(e2d_batch *b, double *ms);
int e2d_batch_launches_per_iteration(e2d_batch *b, int32_t *n);

/* ---- learned warm start ------------------------------------------------
 * A coordinate MLP maps per-cell features (x, y, log wall distance, Mach,
 * sin alpha, cos alpha and 16 random Fourier features of (x, y)) to the
 * conserved state; it is trained on steady solutions of this solver and its
 * prediction is an initial state for e2d_set_state.  Training runs on the GPU
 * in hand-written kernels: BF16 tensor-core GEMMs with FP32 accumulation
 * (forward, backward), and Adam on FP32 master weights.  No reference
 * counterpart. */
#define E2D_MLP_FEATURES 22   /* feature count */
#define E2D_MLP_INPUTS 32     /* padded input width (features, then zeros) */

typedef struct e2d_mlp e2d_mlp;
typedef struct e2d_mlp_config {
    int32_t nhidden;  /* hidden layers of width 256 (default 5)         */
    int32_t batch;    /* training batch, a multiple of 2048 (65536)     */
    uint64_t seed;    /* initial weights and batch sampling             */
    double lr, beta1, beta2, eps;  /* Adam (1e-3, 0.9, 0.999, 1e-8)     */
} e2d_mlp_config;

int e2d_mlp_config_default(e2d_mlp_config *c);
int e2d_mlp_create(const e2d_mlp_config *c, e2d_mlp **out);
void e2d_mlp_destroy(e2d_mlp *m);
/* Parameters in order W0, b0, W1, b1, ..., W_out, b_out (row-major W[out][in]). */
int e2d_mlp_param_count(e2d_mlp *m, int64_t *n);
int e2d_mlp_get_params(e2d_mlp *m, float *p);
int e2d_mlp_set_params(e2d_mlp *m, const float *p);
/* Training set: x [n * E2D_MLP_INPUTS] normalised inputs, t [n * 4] targets. */
int e2d_mlp_set_data(e2d_mlp *m, int64_t n, const float *x, const float *t);
/* Adam step size of the following steps (a schedule is a sequence of calls
 * between e2d_mlp_train calls); lr >= 0. */
int e2d_mlp_set_lr(e2d_mlp *m, double lr);
/* steps Adam steps on random batches; loss[k] (may be NULL) = batch MSE. */
int e2d_mlp_train(e2d_mlp *m, int32_t steps, double *loss);
/* y [n * 4] = network(x [n * E2D_MLP_INPUTS]). */
int e2d_mlp_forward(e2d_mlp *m, int64_t n, const float *x, float *y);
/* MSE loss and its gradient (parameter order as e2d_mlp_get_params) on one
 * batch x [batch * E2D_MLP_INPUTS], t [batch * 4]; parameters unchanged. */
int e2d_mlp_gradient(e2d_mlp *m, const float *x, const float *t, double *loss, float *grad);
/* Raw features of every cell of a mesh for one flow condition, [ncell *
 * E2D_MLP_INPUTS] (before normalisation; padding zero).  Fourier
 * frequencies are N(0, sigma^2) per chord, drawn from `seed`. */
int e2d_mlp_features(e2d_mesh *m, double wall_box, double mach, double alpha_deg, uint64_t seed,
                     double sigma, float *out);
/* Distance from every cell centroid to the nearest wall face. */
int e2d_wall_distance(e2d_mesh *m, double wall_box, double *d);

/* ---- iterations without allocation ------------------------------------ */
/* Largest mesh e2d_step_noalloc accepts. */
#define E2D_NOALLOC_MAX_CELLS 32768
/* Runs `iterations` FP64 iterations of the solve path, like e2d_step, for a
 * caller that may not allocate device memory -- for example a plug-in whose
 * host application owns every device allocation and hands it buffers from its
 * own pool.  No counterpart in the reference.
 *
 * It calls no cudaMalloc / cudaFree and no allocating library routine: the
 * per-iteration working arrays live in one fixed device array of the library
 * sized for E2D_NOALLOC_MAX_CELLS cells (about 7.7 MB), which every GPU that
 * loads the library keeps until the process exits.  Meshes with more cells
 * are rejected with E2D_ERR_CAPACITY.
 *
 * The caller passes, all in device memory, the mesh in the solver's cell-local
 * layout for some cell order of its choice (n = ncell, cells 0..n-1):
 *   topo [4n] int32, 16-byte aligned: per cell the three face codes and the
 *        number of interior neighbours; face k joins Point[(k+1)%3] and
 *        Point[(k+2)%3]; its code is (nb << 3) | (right << 2) | slot for an
 *        interior neighbour nb (right = 1 when this cell is the edge's
 *        right_cell in the reference numbering, slot = the face index of the
 *        same edge in nb), -1 for a far-field face, -2 for a wall face;
 *   S    [6n] double, 16-byte aligned: S[2(k n + i) + {0,1}] = (vectory,
 *        vectorx) of face k in cell i's own node order (gpu_init.cu:153-154);
 *   R    [6n] double, 16-byte aligned: face midpoint minus cell centroid;
 *   area [n]  double, 8-byte aligned;
 * every neighbour index nb must lie in [0, ncell) and every slot in 0..2: the
 * call checks the codes on the GPU before any pass reads through them and
 * returns E2D_ERR_ARG, with nothing computed, when one is out of range;
 * the state w [4n] (rho, rho u, rho v, rho E per cell, 32-byte aligned),
 * advanced in place, and resid [iterations] (8-byte aligned) receiving Resd of
 * each iteration.
 *
 * Parameters: the scheme fields of e2d_params act as in e2d_step, except
 * that precision must be E2D_FP64 and limiter_freeze / limiter_freeze_resd
 * must be 0 (E2D_ERR_ARG otherwise: the limiter-freeze buffer is not part of
 * the fixed array).  ordering, block_size and graph_iters are not used: the
 * cells stay in the caller's order and every pass runs 128 threads per block
 * (launch shapes do not change the result).  A CUDA error left pending by earlier work is reported as
 * E2D_ERR_CUDA before anything is launched, and is not cleared.
 * *epsm is the residual normalisation: <= 0 on entry takes drou of this call's
 * first iteration (gpu_solver.cu:2428); the value used is returned in *epsm,
 * so passing it back continues one residual history across calls.
 *
 * The call is synchronous on `stream` (NULL: the legacy default stream).  The
 * first call on each device looks up the array's device address (with that
 * device current) and may load the module; make it before any stream capture.
 * All calls share the one array and it keeps the last call's contents: calls
 * whose work overlaps on a GPU race with each other. */
int e2d_step_noalloc(int32_t ncell, const int32_t *topo, const double *S, const double *R,
                     const double *area, const e2d_params *p, int32_t iterations, double *w,
                     double *resid, double *epsm, void *stream);

#ifdef __cplusplus
}
#endif
#endif
