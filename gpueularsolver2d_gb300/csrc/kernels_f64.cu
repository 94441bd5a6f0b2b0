// kernels_f64.cu -- FP64 instantiation of the solve-path kernels.
// Built with --fmad=false: every multiply and add is a separate IEEE
// operation, as in the CPU restatement the parity tests compare against.
#include "kernels.cuh"

namespace e2d {
template void enqueue_iteration<double>(const Plan<double> &p, cudaStream_t s);
template void enqueue_batch_iteration<double>(const BPlan<double> &p, cudaStream_t s);
template int enqueue_iteration_timed<double>(const Plan<double> &p, cudaStream_t s, cudaEvent_t *ev, int *kind);
template void enqueue_import<double>(int n, const int *perm, const double *wfile, V4<double> *W, cudaStream_t s);
template void enqueue_export<double>(int n, const int *perm, const V4<double> *W, double *wfile, cudaStream_t s);
}
