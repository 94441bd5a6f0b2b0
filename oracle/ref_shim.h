/*
 * ref_shim.h -- force-included (-include) when the reference's own sources
 * are compiled by oracle/build_ref.py.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference copies some arrays with sizes that do not match their
 * allocations: gpu_solver.cu:1520-1525 copies Ncell+1 ints into buffers sized
 * Nnode+1 (gpu_solver.cu:2036-2041), and gpu_solver.cu:2464-2468 copies
 * (Ncell+1)*sizeof(CELL) bytes out of buffers sized for NODE, EDGE, W and
 * double.  Those copies run outside their device allocations and, for the
 * host side, past the end of the host arrays.  To run the reference program
 * on a shared GPU without them, every cudaMalloc is recorded and every
 * cudaMemcpy whose device range is not inside one recorded allocation is
 * skipped (with a note on stderr).  None of the skipped arrays is read by the
 * reference's kernels, so the solve itself is unchanged.
 *
 * The header also maps the removed cudaThreadSynchronize to
 * cudaDeviceSynchronize.
 */
#ifndef E2D_REF_SHIM_H
#define E2D_REF_SHIM_H
#include <cuda_runtime.h>
#include <stddef.h>

cudaError_t e2d_ref_malloc(void **ptr, size_t size);
cudaError_t e2d_ref_memcpy(void *dst, const void *src, size_t count, enum cudaMemcpyKind kind);

#define cudaMalloc(p, s) e2d_ref_malloc((void **)(p), (s))
#define cudaMemcpy(d, s, n, k) e2d_ref_memcpy((void *)(d), (const void *)(s), (n), (k))
#define cudaThreadSynchronize cudaDeviceSynchronize

#endif
