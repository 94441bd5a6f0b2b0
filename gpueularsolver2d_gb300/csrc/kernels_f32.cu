// kernels_f32.cu -- FP32-stencil instantiation of the solve-path kernels
// (geometry is computed in FP64 on the host and stored as float; the
// residual norm is accumulated in FP64).  Built with FMA contraction and
// fast (non-IEEE) division and square root.
#include "kernels.cuh"

namespace e2d {
template void enqueue_iteration<float>(const Plan<float> &p, cudaStream_t s);
template void enqueue_batch_iteration<float>(const BPlan<float> &p, cudaStream_t s);
template int enqueue_iteration_timed<float>(const Plan<float> &p, cudaStream_t s, cudaEvent_t *ev, int *kind);
template void enqueue_import<float>(int n, const int *perm, const double *wfile, V4<float> *W, cudaStream_t s);
template void enqueue_export<float>(int n, const int *perm, const V4<float> *W, double *wfile, cudaStream_t s);
}
