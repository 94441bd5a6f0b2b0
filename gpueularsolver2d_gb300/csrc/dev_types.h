// dev_types.h -- types shared by the host solver and the kernel translation
// units, and the per-precision launch entry points.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace e2d {

template <typename T> struct alignas(4 * sizeof(T)) V4 { T x, y, z, w; };
template <typename T> struct alignas(2 * sizeof(T)) V2 { T x, y; };

// Device-side iteration control, one per solver (or per batched case).
struct Ctl {
    int step;        // iterations completed
    int halt;        // nonzero: every kernel returns at once (1 done, 2 diverged)
    int target;      // halt when step reaches this
    int check_epsl;  // halt when Resd <= epsl
    int nbad;        // cells with rho <= 0, p <= 0 or NaN after the last iteration
    int fixed_norm;  // epsm given by the caller
    double epsl, epsm, resd;
    int freeze_after;  // > 0: freeze the limiter once step reaches this (option; 0 = reference)
    int frozen;        // limiter values are frozen (set by the residual kernel)
    double freeze_resd;  // > 0: freeze the limiter once Resd falls to this (option)
    // Global time-step option: the smallest local step of RK stage k, as the
    // bits of a non-negative double (whose order is that of the integers), so
    // that blocks fold into it with atomicMin.  kDtNone between iterations.
    unsigned long long dtmin[8];
    unsigned int fold_count;  // blocks of the residual fold done this iteration (0 between iterations)
};

constexpr unsigned long long kDtNone = 0x7FF0000000000000ULL;  // +inf

// Flow constants of one case (gpu_init.cu:63-93).
template <typename T> struct Flow {
    T gamma, ui, vi, ain, tin, vin, R, pis, cfl, dt_cap, eps_entropy, irs_eps;
    T venk_k3;    // K^3 of the Venkatakrishnan option
    int limiter;  // 0 reference, 1 Venkatakrishnan
    int global_dt;  // 1: every cell advances with the smallest local step (option)
    int first_order;  // > 0: first-order faces while fewer iterations are done (option)
    int positivity;   // 1: a non-physical reconstructed face side falls back to the cell state (option)
};

// Cell-local mesh data in internal order (n cells).
//   topo[i] = {f0, f1, f2, clog}; face code f >= 0: (nb << 3) | (right << 2) | slot,
//   -1 far field, -2 wall.  slot = face index of this edge in the neighbour;
//   right = this cell is the edge's right cell in the reference numbering.
//   S[k*n+i] = outward normal of face k in the cell's own node order,
//              (vectory, vectorx) of gpu_init.cu:153-154, so |S| = face length.
//   R[k*n+i] = face midpoint minus cell centroid.
template <typename T> struct MeshDev {
    int n;
    const int4 *__restrict__ topo;
    const V2<T> *__restrict__ S;
    const V2<T> *__restrict__ R;
    const T *__restrict__ area;
};

// Everything one iteration needs.
template <typename T> struct Plan {
    MeshDev<T> m;
    Flow<T> f;
    V4<T> *W[2];   // W[0] holds the iteration's start state and its result
    V4<T> *FS;     // [3n] face-side states
    V4<T> *phi;    // [3n] limiter values (limiter-freeze option), else null
    T *dt;         // [n]
    V4<T> *res;    // [n]
    V4<T> *sm[2];  // [n] smoothing sweeps (ping-pong)
    double *part;  // [blocks] FP64 partials of sum (rho - rho0)^2
    Ctl *ctl;
    double *hist;
    int hist_cap;
    int stages;
    T rk[8];
    int sweeps;
    int block;
};

template <typename T> int launches_per_iteration(const Plan<T> &p) {
    return p.stages * (3 + (p.sweeps > 1 ? p.sweeps - 1 : 0)) + 1;
}

// Batched cases: the cells of all cases in one array, case c in
// [off_c, off_c + n_c) with off_c a multiple of kChunk, so that a tile of B
// cells (B dividing kChunk) lies in one case.  Padding cells are skipped.
constexpr int kChunk = 256;

template <typename T> struct BatchDev {
    const Flow<T> *flows;    // [ncase]
    const int *chunk_case;   // [n / kChunk] case of each chunk
    const int *case_end;     // [ncase] one past the last real cell
    Ctl *ctl;                // [ncase]
};

template <typename T> struct BPlan {
    MeshDev<T> m;            // concatenated mesh (n includes padding)
    Flow<T> f;               // parameters shared by all cases (gamma, irs_eps, ...)
    BatchDev<T> b;
    V4<T> *W[2];
    V4<T> *FS;
    V4<T> *phi;              // [3n] limiter values (limiter-freeze option), else null
    T *dt;
    V4<T> *res;
    V4<T> *sm[2];
    double *part;            // [tiles] one partial per tile
    int ncase;
    const int2 *case_tiles;  // [ncase] {first tile, tile count}
    double *hist;            // [ncase * hist_cap]
    int hist_cap;
    int stages;
    T rk[8];
    int sweeps;
    int block;               // cells per tile = threads per CTA
    bool options = true;     // some case uses a scheme option (pass-A option variant)
    int grid;                // CTAs per launch (persistent when < tiles)
};

template <typename T> int launches_per_iteration(const BPlan<T> &p) {
    return p.stages * (3 + (p.sweeps > 1 ? p.sweeps - 1 : 0)) + 1;
}

template <typename T> void enqueue_batch_iteration(const BPlan<T> &p, cudaStream_t s);

// pairs: the partials are float2 pairs (FP32 stencil) rather than doubles.
void enqueue_batch_resid(double *part, const int2 *case_tiles, int ncase, Ctl *ctl, double *hist,
                         int hist_cap, bool pairs, cudaStream_t s);

// Enqueue one iteration (all RK stages + the residual) on a stream.
// Instantiated for double in kernels_f64.cu and for float in kernels_f32.cu.
template <typename T> void enqueue_iteration(const Plan<T> &p, cudaStream_t s);

// Same, with an event pair around every launch (per-pass timing).
template <typename T> int enqueue_iteration_timed(const Plan<T> &p, cudaStream_t s, cudaEvent_t *ev, int *kind);

// FP64 file-order state <-> T internal-order state (perm[i] = file index).
template <typename T>
void enqueue_import(int n, const int *perm, const double *wfile, V4<T> *W, cudaStream_t s);
template <typename T>
void enqueue_export(int n, const int *perm, const V4<T> *W, double *wfile, cudaStream_t s);

// Residual kernel launcher (resid.cu).
void enqueue_resid(double *part, int nparts, Ctl *ctl, double *hist, int hist_cap, bool pairs,
                   cudaStream_t s);

}  // namespace e2d
