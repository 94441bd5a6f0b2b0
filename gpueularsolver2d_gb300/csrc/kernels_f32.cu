// kernels_f32.cu -- FP32-stencil instantiation of the solve-path kernels
// (geometry is computed in FP64 on the host and stored as float; the
// residual norm is accumulated in FP64).  Built without multiply-add
// contraction (--fmad=false: every inlined copy of a device function rounds
// the same way, so both cells of a face and a batched case and its
// single-case run get the same bits); the FP32 flux and spectral radius fuse
// explicitly with fmaf.  Division and square root are the fast (non-IEEE)
// forms, denormals flush to zero.
#include "kernels.cuh"

namespace e2d {
template void enqueue_iteration<float>(const Plan<float> &p, cudaStream_t s);
template void enqueue_batch_iteration<float>(const BPlan<float> &p, cudaStream_t s);
template int enqueue_iteration_timed<float>(const Plan<float> &p, cudaStream_t s, cudaEvent_t *ev, int *kind);
template void enqueue_import<float>(int n, const int *perm, const double *wfile, V4<float> *W, cudaStream_t s);
template void enqueue_export<float>(int n, const int *perm, const V4<float> *W, double *wfile, cudaStream_t s);
}
