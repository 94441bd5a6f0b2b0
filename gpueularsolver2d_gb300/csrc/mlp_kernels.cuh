// mlp_kernels.cuh -- kernels of the coordinate MLP used for the learned warm
// start: BF16 GEMMs on the fifth-generation tensor cores with FP32
// accumulation in tensor memory, fused bias / GELU epilogues, the small
// output layer, the MSE loss, and Adam.  No reference counterpart.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace e2d {
namespace mlp {

typedef __nv_bfloat16 bf16;

constexpr int BM = 128, BN = 128;  // CTA tile of every GEMM

// GELU in its tanh form (Hendrycks and Gimpel, "Gaussian Error Linear Units",
// 2016): gelu(x) = x (1 + tanh(u)) / 2 with u = sqrt(2 / pi) (x + 0.044715 x^3),
// and its derivative gelu'(x) = (1 + t) / 2 + x (1 - t^2) u'(x) / 2, t = tanh(u).
// One tanh.approx.f32 (the special-function unit's hyperbolic tangent, relative
// error about 2^-11) serves both; the forward epilogue stores gelu'(z) beside
// gelu(z), so the backward pass multiplies instead of re-evaluating.
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

constexpr float kGeluC0 = 0.7978845608028654f;  // sqrt(2 / pi)
constexpr float kGeluC1 = 0.044715f;

__device__ __forceinline__ void gelu_and_grad(float x, float &h, float &g) {
    const float x2 = x * x;
    const float t = tanh_approx(kGeluC0 * x * fmaf(kGeluC1, x2, 1.0f));
    const float hx = 0.5f * x;
    h = fmaf(hx, t, hx);
    g = fmaf(hx * fmaf(-t, t, 1.0f), kGeluC0 * fmaf(3.0f * kGeluC1, x2, 1.0f), fmaf(0.5f, t, 0.5f));
}

// The same for a pair of values with the packed FP32 arithmetic of this
// architecture (two lanes of fused multiply-add per instruction).
__device__ __forceinline__ void gelu_and_grad2(const float2 x, float2 &h, float2 &g) {
    const float2 one = make_float2(1.0f, 1.0f), half = make_float2(0.5f, 0.5f);
    const float2 x2 = __fmul2_rn(x, x);
    const float2 u = __fmul2_rn(__fmul2_rn(make_float2(kGeluC0, kGeluC0), x),
                                __ffma2_rn(make_float2(kGeluC1, kGeluC1), x2, one));
    const float2 t = make_float2(tanh_approx(u.x), tanh_approx(u.y));
    const float2 hx = __fmul2_rn(half, x);
    h = __ffma2_rn(hx, t, hx);
    const float2 sech2 = __ffma2_rn(make_float2(-t.x, -t.y), t, one);
    const float2 du = __ffma2_rn(make_float2(3.0f * kGeluC1 * kGeluC0, 3.0f * kGeluC1 * kGeluC0), x2,
                                 make_float2(kGeluC0, kGeluC0));
    g = __ffma2_rn(__fmul2_rn(hx, sech2), du, __ffma2_rn(half, t, half));
}

__device__ __forceinline__ float gelu(float x) {
    const float hx = 0.5f * x;
    return fmaf(hx, tanh_approx(kGeluC0 * x * fmaf(kGeluC1, x * x, 1.0f)), hx);
}

// Epilogue modes of the GEMM.
enum Epi : int {
    EPI_BIAS_GELU = 0,  // z = acc + bias[n]; out = gelu(z), zout = gelu'(z) (bf16)
    EPI_GELU_BWD = 1,   // out = acc * zin[m,n] (bf16), zin the forward pass's gelu'(z)
    EPI_PARTIAL = 2,    // part[split][m][n] = acc (fp32): split-K partial of a weight gradient
};

// C = opA(A) * opB(B) with opA(A)[m][k] = TA ? A[k][m] : A[m][k] and
// opB(B)[k][n] = TB ? B[k][n] : B[n][k]: each operand is read in place, K-major
// (reduction index contiguous) or MN-major, and staged in the matching
// tensor-core layout.
struct GemmArgs {
    int M, N, K;           // reduction over K (per split: K / gridDim.z, a multiple of 32)
    const bf16 *A;         // TA ? [K][lda] : [M][lda]
    int lda;
    const bf16 *B;         // TB ? [K][ldb] : [N][ldb]
    int ldb;
    const float *bias;     // EPI_BIAS_GELU
    const bf16 *zin;       // EPI_GELU_BWD: [M][ldc] gelu'(z) of the layer
    bf16 *out;             // EPI_BIAS_GELU / EPI_GELU_BWD: [M][ldc]
    bf16 *zout;            // EPI_BIAS_GELU: [M][ldc] gelu'(z)
    float *part;           // EPI_PARTIAL: [splits][M][N]
    int ldc;
    int *flag;             // set to 1 if a wait timed out
};

// ---------------------------------------------------------------------------
// GEMM on tcgen05: one thread issues tcgen05.mma (kind::f16, M = N = 128,
// K = 16) into a 128-column FP32 accumulator in tensor memory; operands are
// copied global -> shared with cp.async straight into the canonical
// no-swizzle layouts (8 x 8 core matrices of 128 bytes, K-major or MN-major
// as the operand lies in memory), two stages
// ahead of the MMAs through a three-buffer ring; tcgen05.commit on a per-buffer
// mbarrier releases a buffer for refill; the epilogue reads the accumulator
// back with tcgen05.ld.  Every wait is bounded: on a timeout the CTA sets
// *g.flag, skips the epilogue and still frees its tensor memory.
namespace tc {
constexpr int BK = 32;                      // K per stage (two MMAs of K = 16)
constexpr int NST = 3;                      // buffers in the ring
constexpr int TILE = 128 * BK * 2;          // bytes of one 128 x BK operand tile
constexpr int SMEM = 2 * NST * TILE;        // dynamic shared memory per CTA
constexpr uint32_t TMEM_COLS = 128;         // FP32 accumulator columns (N = 128)
constexpr int WAIT_LIMIT = 1 << 22;         // try_wait calls before giving up
// instruction descriptor: FP32 D, BF16 A and B, N = 128, M = 128; bits 15 / 16
// set for an MN-major A / B
template <bool TA, bool TB>
struct Idesc {
    static constexpr uint32_t value = (1u << 4) | (1u << 7) | (1u << 10) | ((TA ? 1u : 0u) << 15) |
                                      ((TB ? 1u : 0u) << 16) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
};

// Tile layouts (128 rows of M or N by BK of K, 8 x 8 core matrices of 128 bytes):
//   K-major : core (r/8, k/8) at ((r/8) * (BK/8) + k/8) * 128, its row r%8 (8 k) at 16 B;
//             descriptor LBO = 128 (next core along K), SBO = 512 (along M / N),
//             a K = 16 step moves the start by 256 B
//   MN-major: core (r/8, k/8) at ((k/8) * 16 + r/8) * 128, its row k%8 (8 r) at 16 B;
//             descriptor LBO = 2048 (next core along K), SBO = 128 (along M / N),
//             a K = 16 step moves the start by 4096 B
template <bool MN> struct Tile;
template <> struct Tile<false> {
    static constexpr uint32_t LBO = 128, SBO = (BK / 8) * 128, KSTEP = 256;
    __device__ static int off(int r, int k) { return ((r >> 3) * (BK / 8) + (k >> 3)) * 128 + (r & 7) * 16; }
};
template <> struct Tile<true> {
    static constexpr uint32_t LBO = 2048, SBO = 128, KSTEP = 4096;
    __device__ static int off(int r, int k) { return ((k >> 3) * 16 + (r >> 3)) * 128 + (k & 7) * 16; }
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, LBO, SBO (16-byte units), version 1, no swizzle
template <bool MN> __device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(Tile<MN>::LBO >> 4) << 16) |
           ((uint64_t)(Tile<MN>::SBO >> 4) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (int it = 0; it < WAIT_LIMIT; it++) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// rows [row0, row0 + 128) x k [k0, k0 + BK) of the operand into tile with
// cp.async, 16 bytes per copy; MN: src is [k][ld] (rows contiguous), else
// [row][ld] (k contiguous).  Rows at or past nrows (a multiple of 8) are
// zero-filled (no bytes read).
template <bool MN>
__device__ __forceinline__ void stage(unsigned char *tile, const bf16 *__restrict__ src, int ld, int row0, int nrows,
                                      int k0) {
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const int c = threadIdx.x + it * 256;
        const int r = MN ? (c & 15) * 8 : c >> 2, k = MN ? c >> 4 : (c & 3) * 8;
        const bool in = row0 + r < nrows;
        const bf16 *g = !in ? src : MN ? src + (size_t)(k0 + k) * ld + row0 + r : src + (size_t)(row0 + r) * ld + k0 + k;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n"
                     :: "r"(smem_u32(tile + Tile<MN>::off(r, k))), "l"(g), "r"(in ? 16 : 0) : "memory");
    }
}

__device__ __forceinline__ void commit_group() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
}  // namespace tc

// resident CTAs per SM the register budget is sized for (the GELU-backward
// epilogue needs more registers than the others)
template <int EPI> struct GemmOcc { static constexpr int value = EPI == EPI_GELU_BWD ? 2 : 3; };

template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(256, GemmOcc<EPI>::value) k_gemm_tc(GemmArgs g) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t bars[tc::NST];
    __shared__ uint32_t tmem_sh;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int kper = g.K / gridDim.z, kbeg = blockIdx.z * kper, nst = kper / tc::BK;
    unsigned char *As = tc_smem, *Bs = tc_smem + tc::NST * tc::TILE;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                     :: "r"(tc::smem_u32(&tmem_sh)), "r"(tc::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0)
        for (int b = 0; b < tc::NST; b++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(tc::smem_u32(&bars[b])));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_sh;
    // prologue: stages 0 .. NST-2 in flight
    for (int s = 0; s < tc::NST - 1; s++) {
        if (s < nst) {
            tc::stage<TA>(As + s * tc::TILE, g.A, g.lda, m0, g.M, kbeg + s * tc::BK);
            tc::stage<TB>(Bs + s * tc::TILE, g.B, g.ldb, n0, g.N, kbeg + s * tc::BK);
        }
        tc::commit_group();
    }
    bool ok = true;
    for (int s = 0; s < nst; s++) {
        const int b = s % tc::NST;
        asm volatile("cp.async.wait_group %0;\n" :: "n"(tc::NST - 2) : "memory");  // stage s has landed
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n");
#pragma unroll
            for (int kk = 0; kk < tc::BK / 16; kk++) {
                const uint64_t ad = tc::sdesc<TA>(tc::smem_u32(As + b * tc::TILE) + kk * tc::Tile<TA>::KSTEP);
                const uint64_t bd = tc::sdesc<TB>(tc::smem_u32(Bs + b * tc::TILE) + kk * tc::Tile<TB>::KSTEP);
                const uint32_t acc = (s > 0 || kk > 0) ? 1u : 0u;
                asm volatile("{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                             " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                             :: "r"(tmem), "l"(ad), "l"(bd), "r"(tc::Idesc<TA, TB>::value), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
                         :: "r"(tc::smem_u32(&bars[b])));
        }
        // refill the buffer of stage s - 1 with stage s + NST - 1 once its MMAs are done
        const int sn = s + tc::NST - 1;
        if (sn < nst) {
            if (s >= 1) {
                const bool w = tc::mbar_wait(tc::smem_u32(&bars[(s - 1) % tc::NST]), ((s - 1) / tc::NST) & 1);
                if (__syncthreads_or(!w)) { ok = false; break; }
            }
            tc::stage<TA>(As + (sn % tc::NST) * tc::TILE, g.A, g.lda, m0, g.M, kbeg + sn * tc::BK);
            tc::stage<TB>(Bs + (sn % tc::NST) * tc::TILE, g.B, g.ldb, n0, g.N, kbeg + sn * tc::BK);
        }
        tc::commit_group();
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    if (ok && nst > 0) {  // the last commit covers every MMA of the CTA
        const int s = nst - 1;
        const bool w = tc::mbar_wait(tc::smem_u32(&bars[s % tc::NST]), (s / tc::NST) & 1);
        if (__syncthreads_or(!w)) ok = false;
    }
    if (!ok && tid == 0) atomicExch(g.flag, 1);
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    if (ok && nst > 0) {
        // warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows), columns 64 (w / 4) .. + 63
        const int lb = (warp & 3) * 32, cb = (warp >> 2) * 64;
        const int m = m0 + lb + lane;
#pragma unroll 1
        for (int ch = 0; ch < 4; ch++) {
            uint32_t v[16];
            const uint32_t taddr = tmem + ((uint32_t)lb << 16) + (uint32_t)(cb + ch * 16);
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                           "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                           "=r"(v[14]), "=r"(v[15])
                         : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            const int n = n0 + cb + ch * 16;
            if (m >= g.M || n >= g.N) continue;
            if (EPI == EPI_PARTIAL) {
                float4 *p = (float4 *)(g.part + ((size_t)blockIdx.z * g.M + m) * g.N + n);
#pragma unroll
                for (int j = 0; j < 4; j++)
                    p[j] = make_float4(__uint_as_float(v[4 * j]), __uint_as_float(v[4 * j + 1]),
                                       __uint_as_float(v[4 * j + 2]), __uint_as_float(v[4 * j + 3]));
                continue;
            }
            __align__(16) __nv_bfloat162 o2[8];
            if (EPI == EPI_BIAS_GELU) {
                __align__(16) __nv_bfloat162 z2[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const float z0 = __uint_as_float(v[2 * j]) + g.bias[n + 2 * j];
                    const float z1 = __uint_as_float(v[2 * j + 1]) + g.bias[n + 2 * j + 1];
                    float h0, g0, h1, g1;
                    gelu_and_grad(z0, h0, g0);
                    gelu_and_grad(z1, h1, g1);
                    z2[j] = __floats2bfloat162_rn(g0, g1);
                    o2[j] = __floats2bfloat162_rn(h0, h1);
                }
                uint4 *zo = (uint4 *)(g.zout + (size_t)m * g.ldc + n);
                zo[0] = ((const uint4 *)z2)[0]; zo[1] = ((const uint4 *)z2)[1];
            } else {
                const uint4 *zi = (const uint4 *)(g.zin + (size_t)m * g.ldc + n);
                __align__(16) uint4 zz[2] = {zi[0], zi[1]};
                const __nv_bfloat162 *z2 = (const __nv_bfloat162 *)zz;
#pragma unroll
                for (int j = 0; j < 8; j++)
                    o2[j] = __floats2bfloat162_rn(__uint_as_float(v[2 * j]) * __bfloat162float(z2[j].x),
                                                  __uint_as_float(v[2 * j + 1]) * __bfloat162float(z2[j].y));
            }
            uint4 *oo = (uint4 *)(g.out + (size_t)m * g.ldc + n);
            oo[0] = ((const uint4 *)o2)[0]; oo[1] = ((const uint4 *)o2)[1];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(tmem), "r"(tc::TMEM_COLS));
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

// Output layer backward: dz[b][k] = (sum_o dy[b][o] W[o][k]) * gd[b][k] (bf16),
// gd = gelu'(z) of the last hidden layer as its forward epilogue stored it.
template <int H, int NOUT>
__global__ void __launch_bounds__(256) k_out_bwd_data(int B, const float *__restrict__ dy, const float *__restrict__ W,
                                                      const bf16 *__restrict__ gd, bf16 *__restrict__ dz) {
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
    const __nv_bfloat162 gg = *(const __nv_bfloat162 *)(gd + (size_t)b * H + k);
    const __nv_bfloat162 d = __floats2bfloat162_rn(s0 * __bfloat162float(gg.x), s1 * __bfloat162float(gg.y));
    *(__nv_bfloat162 *)(dz + (size_t)b * H + k) = d;
}

// Output layer of a training step, forward and backward in one pass over the
// last hidden layer (256 -> NOUT on the CUDA cores), one warp per row: lane l
// holds h[b][8l .. 8l + 7] (one 16-byte load), the NOUT dot products are
// butterfly-reduced over the warp, then y, the squared-error loss, dY = 2 (y - t)
// / (B NOUT), the gradient dz[b][k] = (sum_o dY[b][o] W[o][k]) gd[b][k] (bf16,
// gd = gelu'(z) stored by the forward epilogue) and the lane's share of
// dW = dY^T h, db = sum dY.  Block c (256 rows, 8 warps of 32 rows) writes
// part[c][o * H + k] and part[c][NOUT * H + o] (its warps added in a fixed
// order) and loss_part[c]: deterministic.
template <int H, int NOUT>
__global__ void __launch_bounds__(256, 2) k_out_train(int B, const bf16 *__restrict__ h, const float *__restrict__ W,
                                                   const float *__restrict__ bias, const float *__restrict__ t,
                                                   const bf16 *__restrict__ gd, float *__restrict__ y,
                                                   float *__restrict__ dy, bf16 *__restrict__ dz,
                                                   float *__restrict__ part, double *__restrict__ loss_part) {
    static_assert(H == 256, "one 16-byte load per lane covers a row");
    __shared__ float red[8][NOUT * H + NOUT];
    __shared__ __align__(16) float Ws[NOUT * H];
    __shared__ double lred[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, k0 = lane * 8;
    for (int e = threadIdx.x; e < NOUT * H; e += blockDim.x) Ws[e] = W[e];
    __syncthreads();
    float acc[NOUT][8], dacc[NOUT];
#pragma unroll
    for (int o = 0; o < NOUT; o++) {
        dacc[o] = 0.f;
#pragma unroll
        for (int q = 0; q < 8; q++) acc[o][q] = 0.f;
    }
    double l = 0.0;
    const int r0 = blockIdx.x * 256 + warp * 32;  // B is a multiple of 256
    constexpr int RB = 2;                          // rows whose loads are in flight together
    for (int rb = 0; rb < 32; rb += RB) {
        uint4 hvs[RB], gvs[RB];
#pragma unroll
        for (int j = 0; j < RB; j++) {
            hvs[j] = *(const uint4 *)(h + (size_t)(r0 + rb + j) * H + k0);
            gvs[j] = *(const uint4 *)(gd + (size_t)(r0 + rb + j) * H + k0);
        }
#pragma unroll
    for (int j = 0; j < RB; j++) {
        const int b = r0 + rb + j;
        const uint4 hv = hvs[j], gv = gvs[j];
        const __nv_bfloat162 *h2 = (const __nv_bfloat162 *)&hv;
        float x[8];
#pragma unroll
        for (int q = 0; q < 4; q++) { x[2 * q] = __low2float(h2[q]); x[2 * q + 1] = __high2float(h2[q]); }
        float p[NOUT];
#pragma unroll
        for (int o = 0; o < NOUT; o++) {
            const float4 wa = *(const float4 *)&Ws[o * H + k0], wb = *(const float4 *)&Ws[o * H + k0 + 4];
            p[o] = fmaf(x[0], wa.x, fmaf(x[1], wa.y, fmaf(x[2], wa.z, fmaf(x[3], wa.w,
                   fmaf(x[4], wb.x, fmaf(x[5], wb.y, fmaf(x[6], wb.z, x[7] * wb.w)))))));
        }
#pragma unroll
        for (int o = 0; o < NOUT; o++)
#pragma unroll
            for (int sh = 16; sh > 0; sh >>= 1) p[o] += __shfl_xor_sync(0xffffffffu, p[o], sh);
        float d[NOUT];
#pragma unroll
        for (int o = 0; o < NOUT; o++) {
            const float yo = p[o] + bias[o];
            const float e = yo - t[(size_t)b * NOUT + o];
            if (lane == 0) {
                y[(size_t)b * NOUT + o] = yo;
                l += (double)e * e;
            }
            d[o] = 2.0f * e / (float)(B * NOUT);
            if (lane == o) dy[(size_t)b * NOUT + o] = d[o];
            dacc[o] += d[o];
#pragma unroll
            for (int q = 0; q < 8; q++) acc[o][q] = fmaf(d[o], x[q], acc[o][q]);
        }
        const __nv_bfloat162 *g2 = (const __nv_bfloat162 *)&gv;
        __align__(16) __nv_bfloat162 o2[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            float s0 = 0.f, s1 = 0.f;
#pragma unroll
            for (int o = 0; o < NOUT; o++) {
                const float2 wo = *(const float2 *)&Ws[o * H + k0 + 2 * q];
                s0 = fmaf(d[o], wo.x, s0);
                s1 = fmaf(d[o], wo.y, s1);
            }
            o2[q] = __floats2bfloat162_rn(s0 * __low2float(g2[q]), s1 * __high2float(g2[q]));
        }
        *(uint4 *)(dz + (size_t)b * H + k0) = *(const uint4 *)o2;
    }
    }
#pragma unroll
    for (int o = 0; o < NOUT; o++) {
#pragma unroll
        for (int q = 0; q < 8; q++) red[warp][o * H + k0 + q] = acc[o][q];
        if (lane == 0) red[warp][NOUT * H + o] = dacc[o];
    }
    if (lane == 0) lred[warp] = l;
    __syncthreads();
    float *pc = part + (size_t)blockIdx.x * (NOUT * H + NOUT);
    for (int e = threadIdx.x; e < NOUT * H + NOUT; e += blockDim.x) {
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 8; k++) s += red[k][e];
        pc[e] = s;
    }
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < 8; k++) s += lred[k];
        loss_part[blockIdx.x] = s;
    }
}

// Split partials of the output layer's weight gradient: part[split][o][k] =
// sum over the split's rows of dy[b][o] h[b][k]; part[split][NOUT*H + o] =
// sum dy.  Grid (H / 32, splits): lane = column k, the block's 8 warps take
// every 8th row, then the warps are added in a fixed order (deterministic).
template <int H, int NOUT>
__global__ void __launch_bounds__(256) k_out_bwd_weight(int B, int rows_per_split, const float *__restrict__ dy,
                                                        const bf16 *__restrict__ h, float *__restrict__ part) {
    __shared__ float red[8][NOUT][32];
    __shared__ float dred[8][NOUT];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int k = blockIdx.x * 32 + lane;
    const int b0 = blockIdx.y * rows_per_split, b1 = min(B, b0 + rows_per_split);
    float s[NOUT], ds[NOUT];
#pragma unroll
    for (int o = 0; o < NOUT; o++) s[o] = ds[o] = 0.f;
    for (int b = b0 + warp; b < b1; b += 8) {
        const float x = __bfloat162float(h[(size_t)b * H + k]);
#pragma unroll
        for (int o = 0; o < NOUT; o++) {
            const float d = dy[(size_t)b * NOUT + o];
            s[o] += d * x;
            ds[o] += d;
        }
    }
#pragma unroll
    for (int o = 0; o < NOUT; o++) red[warp][o][lane] = s[o];
    if (lane == 0)
#pragma unroll
        for (int o = 0; o < NOUT; o++) dred[warp][o] = ds[o];
    __syncthreads();
    float *p = part + (size_t)blockIdx.y * (NOUT * H + NOUT);
    if (warp < NOUT) {
        float t = 0.f;
        for (int w = 0; w < 8; w++) t += red[w][warp][lane];
        p[warp * H + k] = t;
    }
    if (blockIdx.x == 0 && threadIdx.x < NOUT) {
        float t = 0.f;
        for (int w = 0; w < 8; w++) t += dred[w][threadIdx.x];
        p[NOUT * H + threadIdx.x] = t;
    }
}

// Column sums of a bf16 [B][N] gradient over row splits: part[split][n].
// Grid (N / 32, splits), same shape as k_out_bwd_weight.
__global__ void __launch_bounds__(256) k_colsum(int B, int N, int rows_per_split, const bf16 *__restrict__ d,
                                                float *__restrict__ part) {
    __shared__ float red[8][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = blockIdx.x * 32 + lane;
    const int b0 = blockIdx.y * rows_per_split, b1 = min(B, b0 + rows_per_split);
    float s = 0.f;
    for (int b = b0 + warp; b < b1; b += 8) s += __bfloat162float(d[(size_t)b * N + n]);
    red[warp][lane] = s;
    __syncthreads();
    if (warp == 0) {
        float t = 0.f;
        for (int w = 0; w < 8; w++) t += red[w][lane];
        part[(size_t)blockIdx.y * N + n] = t;
    }
}

// Random mini-batch gather: rows idx(step, j) of the training set (nin
// columns) into row j of xb (row pitch ldx), with the step counter read from
// device memory (the training step is a static graph).
__global__ void __launch_bounds__(256) k_gather(int B, int nin, int ldx, int nout, unsigned long long seed,
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
        *(uint4 *)(xb + (size_t)j * ldx + k) = *(const uint4 *)(X + (size_t)r * nin + k);
    for (int o = 0; o < nout; o++) tb[(size_t)j * nout + o] = T[(size_t)r * nout + o];
}

}  // namespace mlp
}  // namespace e2d
