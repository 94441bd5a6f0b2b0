// resid.cu -- residual of one iteration (gpu_solver.cu:2404-2433).
#include "dev_types.h"
#include "pdl.cuh"

namespace e2d {

// drou = sum of the per-block partials in a fixed order, then
// Resd = sqrt((drou + 1e-32) / EPSM) with EPSM = drou of iteration 1 unless
// the caller fixed it.  Sets halt when the loop condition of
// gpu_solver.cu:2200 (step < MAXSTEP && Resd > EPSL) fails or the state went
// unphysical.  One block of 256 threads.
__device__ __forceinline__ void resid_block(const double *__restrict__ part, int nparts, Ctl *ctl,
                                            double *hist, int hist_cap) {
    __shared__ double sh[256];
    double s = 0.0;
    for (int k = threadIdx.x; k < nparts; k += 256) s += part[k];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double drou = sh[0];
    const int step = ctl->step + 1;
    if (step == 1 && !ctl->fixed_norm) ctl->epsm = drou;
    const double resd = sqrt((drou + 1.0E-32) / ctl->epsm);
    if (step - 1 < hist_cap) hist[step - 1] = resd;
    ctl->step = step;
    ctl->resd = resd;
    for (int k = 0; k < 8; k++) ctl->dtmin[k] = kDtNone;  // global time-step slots for the next iteration
    if ((ctl->freeze_after > 0 && step >= ctl->freeze_after) || (ctl->freeze_resd > 0.0 && resd <= ctl->freeze_resd))
        ctl->frozen = 1;
    if (ctl->nbad) ctl->halt = 2;
    else if (ctl->check_epsl && !(resd > ctl->epsl)) ctl->halt = 1;
    else if (step >= ctl->target) ctl->halt = 1;
}

__global__ void __launch_bounds__(256) k_resid(const double *__restrict__ part, int nparts, Ctl *ctl,
                                               double *hist, int hist_cap) {
    wait_prior_grid();
    if (ctl->halt) return;
    resid_block(part, nparts, ctl, hist, hist_cap);
}

// Batched cases: one block per case over that case's tile partials (each
// case's tiles are numbered from a multiple of the chunk, so the grouping of
// its partials is the one a single-case run of the same block size uses).
__global__ void __launch_bounds__(256) kb_resid(const double *__restrict__ part, const int2 *case_tiles,
                                                Ctl *ctl, double *hist, int hist_cap) {
    wait_prior_grid();
    const int c = blockIdx.x;
    if (ctl[c].halt) return;
    const int2 ct = case_tiles[c];
    resid_block(part + ct.x, ct.y, ctl + c, hist + (size_t)c * hist_cap, hist_cap);
}

void enqueue_resid(const double *part, int nparts, Ctl *ctl, double *hist, int hist_cap,
                   cudaStream_t s) {
    launch_chained(k_resid, 1, 256, s, part, nparts, ctl, hist, hist_cap);
}

void enqueue_batch_resid(const double *part, const int2 *case_tiles, int ncase, Ctl *ctl, double *hist,
                         int hist_cap, cudaStream_t s) {
    launch_chained(kb_resid, ncase, 256, s, part, case_tiles, ctl, hist, hist_cap);
}

}  // namespace e2d
