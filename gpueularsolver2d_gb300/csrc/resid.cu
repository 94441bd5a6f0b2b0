// resid.cu -- residual of one iteration (gpu_solver.cu:2404-2433).
#include "dev_types.h"
#include "pdl.cuh"

namespace e2d {

// Partials folded by one block in the first level of the sum.
constexpr int kFoldChunk = 1024;

// One pass-D partial as a double: an FP64 sum, or (pairs) an unevaluated
// float pair, whose two parts add exactly in FP64.
template <bool PAIRS> __device__ __forceinline__ double load_part(const double *part, const int k) {
    if (PAIRS) {
        const float2 v = reinterpret_cast<const float2 *>(part)[k];
        return (double)v.x + (double)v.y;
    }
    return part[k];
}

// Sum of partials [k0, k1) by one 256-thread block in a fixed order (thread t
// adds k0 + t, k0 + t + 256, ... in turn, then a fixed tree); the result is
// returned to every thread.
template <bool PAIRS>
__device__ __forceinline__ double block_fold(const double *part, const int k0, const int k1, double *sh) {
    double s = 0.0;
    for (int k = k0 + (int)threadIdx.x; k < k1; k += 256) s += load_part<PAIRS>(part, k);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// drou -> Resd = sqrt((drou + 1e-32) / EPSM) with EPSM = drou of iteration 1
// unless the caller fixed it.  Sets halt when the loop condition of
// gpu_solver.cu:2200 (step < MAXSTEP && Resd > EPSL) fails or the state went
// unphysical.  One thread.
__device__ __forceinline__ void resid_finish(const double drou, Ctl *ctl, double *hist, int hist_cap) {
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

// drou = sum of the pass-D partials in two levels: block c folds partials
// [c * kFoldChunk, (c + 1) * kFoldChunk) and leaves its sum in the first slot
// of its chunk; the block that finishes last (a counter in the control
// block) adds the chunk sums in chunk order and finishes the residual.  The
// grouping is fixed, so the result does not depend on which block is last.
// (One block folding every partial took ~22 us per iteration at 4.2M cells.)
template <bool PAIRS>
__global__ void __launch_bounds__(256) k_resid(double *__restrict__ part, int nparts, Ctl *ctl, double *hist,
                                               int hist_cap) {
    wait_prior_grid();
    if (ctl->halt) return;
    __shared__ double sh[256];
    const int nch = (nparts + kFoldChunk - 1) / kFoldChunk, c = blockIdx.x;
    const double s = block_fold<PAIRS>(part, c * kFoldChunk, min(nparts, (c + 1) * kFoldChunk), sh);
    if (threadIdx.x != 0) return;
    if (nch == 1) {
        resid_finish(0.0 + s, ctl, hist, hist_cap);
        return;
    }
    part[c * kFoldChunk] = s;  // this chunk's first partial is no longer needed
    __threadfence();
    if (atomicAdd(&ctl->fold_count, 1u) != (unsigned)(nch - 1)) return;  // not the last block
    __threadfence();
    double drou = 0.0;
    for (int k = 0; k < nch; k++) drou += *(volatile double *)&part[k * kFoldChunk];
    ctl->fold_count = 0;
    resid_finish(drou, ctl, hist, hist_cap);
}

// Batched cases: one block per case over that case's tile partials, folded
// in the same two-level grouping as a single-case run of the same block size
// (each case's tiles are numbered from a multiple of the chunk), so every
// case gets the bits of its own single-case run.
template <bool PAIRS>
__global__ void __launch_bounds__(256) kb_resid(const double *__restrict__ part, const int2 *case_tiles,
                                                Ctl *ctl, double *hist, int hist_cap) {
    wait_prior_grid();
    const int c = blockIdx.x;
    if (ctl[c].halt) return;
    __shared__ double sh[256];
    const int2 ct = case_tiles[c];
    const double *p = part + ct.x;
    double drou = 0.0;
    for (int k0 = 0; k0 < ct.y; k0 += kFoldChunk) {
        const double s = block_fold<PAIRS>(p, k0, min(ct.y, k0 + kFoldChunk), sh);
        drou += s;  // every thread keeps the same running sum; thread 0's is used
    }
    if (threadIdx.x == 0) resid_finish(drou, ctl + c, hist + (size_t)c * hist_cap, hist_cap);
}

void enqueue_resid(double *part, int nparts, Ctl *ctl, double *hist, int hist_cap, bool pairs, cudaStream_t s) {
    const int nch = (nparts + kFoldChunk - 1) / kFoldChunk;
    if (pairs) launch_chained(k_resid<true>, nch, 256, s, part, nparts, ctl, hist, hist_cap);
    else launch_chained(k_resid<false>, nch, 256, s, part, nparts, ctl, hist, hist_cap);
}

void enqueue_batch_resid(double *part, const int2 *case_tiles, int ncase, Ctl *ctl, double *hist, int hist_cap,
                         bool pairs, cudaStream_t s) {
    if (pairs) launch_chained(kb_resid<true>, ncase, 256, s, (const double *)part, case_tiles, ctl, hist, hist_cap);
    else launch_chained(kb_resid<false>, ncase, 256, s, (const double *)part, case_tiles, ctl, hist, hist_cap);
}

}  // namespace e2d
