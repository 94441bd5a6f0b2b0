// mlp_kernels.cuh -- kernels of the coordinate MLP used for the learned warm
// start: BF16 GEMMs on the tensor cores with FP32 accumulation
// (mma.sync.m16n8k16, operands staged in shared memory and fed by ldmatrix),
// fused bias / GELU epilogues, the small output layer, the MSE loss, and Adam.
// No reference counterpart.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace e2d {
namespace mlp {

typedef __nv_bfloat16 bf16;

constexpr int BM = 128, BN = 128, BK = 32;  // CTA tile
constexpr int PADK = BK + 8;                 // row pitch (bf16) of [rows][BK] tiles
constexpr int PADM = BM + 8;                 // row pitch (bf16) of [BK][rows] tiles

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

__device__ __forceinline__ float gelu_grad(float x) {
    // d/dx [x Phi(x)] = Phi(x) + x phi(x)
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__device__ __forceinline__ void ldsm_x4(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3, const void *p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(a));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3, const void *p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(a));
}

__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Epilogue modes of the GEMM.
enum Epi : int {
    EPI_BIAS_GELU = 0,  // z = acc + bias[n]; out = gelu(z) (bf16), zout = z (bf16)
    EPI_GELU_BWD = 1,   // out = acc * gelu'(zin[m,n])  (bf16): gradient at the previous pre-activation
    EPI_PARTIAL = 2,    // part[split][m][n] = acc (fp32): split-K partial of a weight gradient
};

struct GemmArgs {
    int M, N, K;           // C is M x N, reduction over K (per split: K / gridDim.z)
    const bf16 *A;         // TA=false: [M][lda] ; TA=true: [K][lda]
    int lda;
    const bf16 *B;         // TB=false: [N][ldb] ; TB=true: [K][ldb]
    int ldb;
    const float *bias;     // EPI_BIAS_GELU
    const bf16 *zin;       // EPI_GELU_BWD: [M][ldc]
    bf16 *out;             // EPI_BIAS_GELU / EPI_GELU_BWD: [M][ldc]
    bf16 *zout;            // EPI_BIAS_GELU: [M][ldc]
    float *part;           // EPI_PARTIAL: [splits][M][N]
    int ldc;
};

// C = opA(A) * opB(B): opA(A)[m][k] = TA ? A[k][m] : A[m][k];
//                     opB(B)[k][n] = TB ? B[k][n] : B[n][k].
// 256 threads = 8 warps as 2 (M) x 4 (N); each warp computes 64 x 32.  M and N
// may be ragged (zero-filled tiles, guarded stores); K per split must be a
// multiple of BK.
template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(256) k_gemm(GemmArgs g) {
    __shared__ __align__(16) bf16 As[TA ? BK * PADM : BM * PADK];
    __shared__ __align__(16) bf16 Bs[TB ? BK * PADM : BN * PADK];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int kper = g.K / gridDim.z, kbeg = blockIdx.z * kper, kend = kbeg + kper;
    const int wm = (warp >> 2) * 64, wn = (warp & 3) * 32;
    float acc[4][4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[i][j][q] = 0.f;
    for (int k0 = kbeg; k0 < kend; k0 += BK) {
        // global -> shared, 16-byte chunks; out-of-range rows / columns are zero
#pragma unroll
        for (int it = 0; it < 2; it++) {
            const int c = tid + it * 256;  // 512 chunks of 8 bf16 per operand tile
            uint4 va = make_uint4(0, 0, 0, 0), vb = make_uint4(0, 0, 0, 0);
            if (!TA) {  // A[m][k]: 128 rows x 4 chunks
                const int r = c >> 2, kc = (c & 3) * 8;
                if (m0 + r < g.M) va = *(const uint4 *)(g.A + (size_t)(m0 + r) * g.lda + k0 + kc);
                *(uint4 *)(As + r * PADK + kc) = va;
            } else {    // A[k][m]: 32 rows x 16 chunks
                const int r = c >> 4, mc = (c & 15) * 8;
                if (m0 + mc < g.M) va = *(const uint4 *)(g.A + (size_t)(k0 + r) * g.lda + m0 + mc);
                *(uint4 *)(As + r * PADM + mc) = va;
            }
            if (!TB) {  // B[n][k]
                const int r = c >> 2, kc = (c & 3) * 8;
                if (n0 + r < g.N) vb = *(const uint4 *)(g.B + (size_t)(n0 + r) * g.ldb + k0 + kc);
                *(uint4 *)(Bs + r * PADK + kc) = vb;
            } else {    // B[k][n]
                const int r = c >> 4, nc = (c & 15) * 8;
                if (n0 + nc < g.N) vb = *(const uint4 *)(g.B + (size_t)(k0 + r) * g.ldb + n0 + nc);
                *(uint4 *)(Bs + r * PADM + nc) = vb;
            }
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[4][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int mb = wm + i * 16;
                if (!TA) {
                    const bf16 *p = As + (mb + (lane & 15)) * PADK + kk + (lane >> 4) * 8;
                    ldsm_x4(af[i][0], af[i][1], af[i][2], af[i][3], p);
                } else {
                    // matrices: (m0-7,k0-7) (m8-15,k0-7) (m0-7,k8-15) (m8-15,k8-15), stored [k][m]
                    const int krow = kk + (lane & 7) + ((lane >> 4) << 3);
                    const int mcol = mb + ((lane >> 3) & 1) * 8;
                    ldsm_x4_t(af[i][0], af[i][1], af[i][2], af[i][3], As + krow * PADM + mcol);
                }
            }
#pragma unroll
            for (int j = 0; j < 4; j += 2) {
                const int nb = wn + j * 8;
                uint32_t r0, r1, r2, r3;
                if (!TB) {
                    // matrices: (n0-7,k0-7) (n0-7,k8-15) (n8-15,k0-7) (n8-15,k8-15), stored [n][k]
                    const int nrow = nb + (lane & 7) + ((lane >> 4) << 3);
                    const int kcol = kk + ((lane >> 3) & 1) * 8;
                    ldsm_x4(r0, r1, r2, r3, Bs + nrow * PADK + kcol);
                } else {
                    // same four matrices, stored [k][n]
                    const int krow = kk + (lane & 7) + ((lane >> 3) & 1) * 8;
                    const int ncol = nb + (lane >> 4) * 8;
                    ldsm_x4_t(r0, r1, r2, r3, Bs + krow * PADM + ncol);
                }
                bfr[j][0] = r0; bfr[j][1] = r1; bfr[j + 1][0] = r2; bfr[j + 1][1] = r3;
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bfr[j][0], bfr[j][1]);
        }
        __syncthreads();
    }
    // epilogue: c0,c1 at (row g, cols 2t,2t+1), c2,c3 at row g+8
    const int gr = lane >> 2, tc = (lane & 3) * 2;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int m = m0 + wm + i * 16 + gr + h * 8;
                const int n = n0 + wn + j * 8 + tc;
                if (m >= g.M || n >= g.N) continue;
                const float v0 = acc[i][j][2 * h], v1 = acc[i][j][2 * h + 1];
                if (EPI == EPI_BIAS_GELU) {
                    const float z0 = v0 + g.bias[n], z1 = v1 + g.bias[n + 1];
                    *(__nv_bfloat162 *)(g.zout + (size_t)m * g.ldc + n) = __floats2bfloat162_rn(z0, z1);
                    *(__nv_bfloat162 *)(g.out + (size_t)m * g.ldc + n) = __floats2bfloat162_rn(gelu(z0), gelu(z1));
                } else if (EPI == EPI_GELU_BWD) {
                    const __nv_bfloat162 z = *(const __nv_bfloat162 *)(g.zin + (size_t)m * g.ldc + n);
                    const float d0 = v0 * gelu_grad(__bfloat162float(z.x));
                    const float d1 = v1 * gelu_grad(__bfloat162float(z.y));
                    *(__nv_bfloat162 *)(g.out + (size_t)m * g.ldc + n) = __floats2bfloat162_rn(d0, d1);
                } else {
                    float *p = g.part + ((size_t)blockIdx.z * g.M + m) * g.N + n;
                    p[0] = v0;
                    p[1] = v1;
                }
            }
}

// Output layer (256 -> NOUT) on the CUDA cores: y[b][o] = h[b] . W[o] + bias[o]
// (fp32); loss partial per block of MSE against t, and dY = 2 (y - t) / (B NOUT).
template <int H, int NOUT>
__global__ void __launch_bounds__(256) k_out_fwd_loss(int B, const bf16 *__restrict__ h, const float *__restrict__ W,
                                                      const float *__restrict__ bias, const float *__restrict__ t,
                                                      float *__restrict__ y, float *__restrict__ dy,
                                                      double *__restrict__ loss_part) {
    __shared__ float Ws[NOUT * H];
    for (int k = threadIdx.x; k < NOUT * H; k += blockDim.x) Ws[k] = W[k];
    __syncthreads();
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (b < B) {
        float acc[NOUT];
#pragma unroll
        for (int o = 0; o < NOUT; o++) acc[o] = bias[o];
        const bf16 *hr = h + (size_t)b * H;
        for (int k = 0; k < H; k += 8) {
            const uint4 v = *(const uint4 *)(hr + k);
            const bf16 *e = (const bf16 *)&v;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const float x = __bfloat162float(e[q]);
#pragma unroll
                for (int o = 0; o < NOUT; o++) acc[o] += x * Ws[o * H + k + q];
            }
        }
#pragma unroll
        for (int o = 0; o < NOUT; o++) {
            y[(size_t)b * NOUT + o] = acc[o];
            if (t) {
                const float d = acc[o] - t[(size_t)b * NOUT + o];
                l += (double)d * d;
                dy[(size_t)b * NOUT + o] = 2.0f * d / (float)(B * NOUT);
            }
        }
    }
    if (!loss_part) return;
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    __shared__ double ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += ws[k];
        loss_part[blockIdx.x] = s;
    }
}

// Output layer backward: dz[b][k] = (sum_o dy[b][o] W[o][k]) * gelu'(z[b][k]) (bf16).
template <int H, int NOUT>
__global__ void __launch_bounds__(256) k_out_bwd_data(int B, const float *__restrict__ dy, const float *__restrict__ W,
                                                      const bf16 *__restrict__ z, bf16 *__restrict__ dz) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;  // one (b, pair of k)
    if (idx >= (size_t)B * (H / 2)) return;
    const int b = (int)(idx / (H / 2)), k = (int)(idx % (H / 2)) * 2;
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int o = 0; o < NOUT; o++) {
        const float d = dy[(size_t)b * NOUT + o];
        s0 += d * W[o * H + k];
        s1 += d * W[o * H + k + 1];
    }
    const __nv_bfloat162 zz = *(const __nv_bfloat162 *)(z + (size_t)b * H + k);
    *(__nv_bfloat162 *)(dz + (size_t)b * H + k) =
        __floats2bfloat162_rn(s0 * gelu_grad(__bfloat162float(zz.x)), s1 * gelu_grad(__bfloat162float(zz.y)));
}

// Split partials of the output layer's weight gradient: part[blk][o][k] =
// sum over the block's rows of dy[b][o] h[b][k]; part[blk][NOUT*H + o] = sum dy.
template <int H, int NOUT>
__global__ void __launch_bounds__(256) k_out_bwd_weight(int B, int rows_per_block, const float *__restrict__ dy,
                                                        const bf16 *__restrict__ h, float *__restrict__ part) {
    const int b0 = blockIdx.x * rows_per_block, b1 = min(B, b0 + rows_per_block);
    for (int k = threadIdx.x; k < H; k += blockDim.x) {
        float s[NOUT];
#pragma unroll
        for (int o = 0; o < NOUT; o++) s[o] = 0.f;
        for (int b = b0; b < b1; b++) {
            const float x = __bfloat162float(h[(size_t)b * H + k]);
#pragma unroll
            for (int o = 0; o < NOUT; o++) s[o] += dy[(size_t)b * NOUT + o] * x;
        }
#pragma unroll
        for (int o = 0; o < NOUT; o++) part[(size_t)blockIdx.x * (NOUT * H + NOUT) + o * H + k] = s[o];
    }
    if (threadIdx.x < NOUT) {
        float s = 0.f;
        for (int b = b0; b < b1; b++) s += dy[(size_t)b * NOUT + threadIdx.x];
        part[(size_t)blockIdx.x * (NOUT * H + NOUT) + NOUT * H + threadIdx.x] = s;
    }
}

// Column sums of a bf16 [B][N] gradient over row blocks: part[blk][n].
__global__ void __launch_bounds__(256) k_colsum(int B, int N, int rows_per_block, const bf16 *__restrict__ d,
                                                float *__restrict__ part) {
    const int b0 = blockIdx.x * rows_per_block, b1 = min(B, b0 + rows_per_block);
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        float s = 0.f;
        for (int b = b0; b < b1; b++) s += __bfloat162float(d[(size_t)b * N + n]);
        part[(size_t)blockIdx.x * N + n] = s;
    }
}

// Adam on `count` parameters whose gradient is the sum of `nparts` partials
// (stride `pstride`), summed in a fixed order.  w32 master weights; wbf (may
// be null) receives the bf16 copy used by the GEMMs.
__global__ void __launch_bounds__(256) k_adam(int count, const float *__restrict__ part, int nparts, size_t pstride,
                                              float *__restrict__ w32, bf16 *__restrict__ wbf, float *__restrict__ m,
                                              float *__restrict__ v, float lr, float beta1, float beta2, float eps,
                                              float bc1, float bc2, float *__restrict__ grad_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float g = 0.f;
    for (int p = 0; p < nparts; p++) g += part[(size_t)p * pstride + i];
    if (grad_out) grad_out[i] = g;
    if (lr == 0.f) return;  // gradient only
    const float mi = beta1 * m[i] + (1.f - beta1) * g;
    const float vi = beta2 * v[i] + (1.f - beta2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float w = w32[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w32[i] = w;
    if (wbf) wbf[i] = __float2bfloat16_rn(w);
}

// Random mini-batch gather: rows idx(step, j) of the training set, with the
// step counter read from device memory (the training step is a static graph).
__global__ void __launch_bounds__(256) k_gather(int B, int nin, int nout, unsigned long long seed,
                                                const int *__restrict__ stepp, long long nsamples,
                                                const bf16 *__restrict__ X, const float *__restrict__ T,
                                                bf16 *__restrict__ xb, float *__restrict__ tb) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= B) return;
    const int step = *stepp;
    unsigned long long z = seed + 0x9e3779b97f4a7c15ULL * ((unsigned long long)step * 1315423911ULL + j + 1);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    z ^= z >> 31;
    const long long r = (long long)(z % (unsigned long long)nsamples);
    for (int k = 0; k < nin; k += 8)
        *(uint4 *)(xb + (size_t)j * nin + k) = *(const uint4 *)(X + (size_t)r * nin + k);
    for (int o = 0; o < nout; o++) tb[(size_t)j * nout + o] = T[(size_t)r * nout + o];
}

}  // namespace mlp
}  // namespace e2d
