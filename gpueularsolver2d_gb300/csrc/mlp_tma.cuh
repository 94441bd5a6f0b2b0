// mlp_tma.cuh -- the hidden-layer GEMMs of the warm-start MLP (the forward
// pass with bias + GELU, the data gradient with GELU', and the weight
// gradient with the bias sums) as persistent, warp-specialised kernels, one
// launch per layer.  No reference counterpart.
//
//   C[B x 256] = A[B x K] . Wt^T,  A and Wt both K-major (row-major, the
//   reduction index contiguous): Wt = W (forward) or W^T (data gradient);
//   K = 256, or 64 for the first layer (its inputs padded to one slice).
//
// One CTA per SM walks 128-row tiles of the batch:
//   warp 0  (one thread) loads the 256 x K weights once and streams each
//           tile's A in 128 x 64 slices by TMA (cp.async.bulk.tensor,
//           128-byte swizzle) into a two-slot ring;
//   warp 1  (one thread) issues tcgen05.mma (kind::f16, M = 128, N = 256,
//           K = 16; BF16 operands from shared memory, FP32 accumulate) into
//           one of two 256-column accumulators in tensor memory; each slice's
//           MMAs release its slot (tcgen05.commit), a finished tile releases
//           its accumulator to the epilogue;
//   warps 2-17 drain the other accumulator with tcgen05.ld (each warp one
//           32-lane quarter of the rows and a quarter of the columns), apply
//           the epilogue into a 32 x 32 bf16 slab of its own in shared memory
//           (64-byte swizzle) and store the slab by TMA, while the next
//           tile's MMAs run; the data gradient's gelu'(z) factors come into
//           the same slabs by TMA before the accumulator is ready.
// Every wait is bounded: a timed-out thread sets *flag and leaves its loop;
// the producer then waits (bounded) for the copies it issued, the MMA thread
// for the MMAs it issued, and the tensor memory is freed on every path.
#pragma once

#include <cuda.h>

#include "mlp_kernels.cuh"

namespace e2d {
namespace mlp {
namespace ws {

constexpr int ND = 256, BM = 128;            // output width, rows per tile
constexpr int KC = 64;                       // K columns per A slice: one 128-byte swizzle row of bf16
constexpr int NSLOT = 2;                     // A slices in flight
constexpr int SLICE_BYTES = BM * KC * 2;     // 16 KB
constexpr int WSLICE_BYTES = ND * KC * 2;    // 32 KB
constexpr int NEPI = 16;                     // epilogue warps: 4 per 32-lane quarter of tensor memory
constexpr int SLAB = 32 * 32 * 2;            // one epilogue slab: 32 rows x 32 columns of bf16
constexpr int SLABS_BYTES = NEPI * 2 * SLAB; // two slabs per epilogue warp
// Shared memory of a layer with NK slices of K (K = 64 NK: 4 for the 256-wide
// layers, 1 for the first layer's inputs padded to 64): weights, A ring,
// slabs, the bias (1 KB), and slack to align the base to 1024 bytes.
template <int NK> struct Gemm {
    static constexpr int W_BYTES = NK * WSLICE_BYTES;
    static constexpr int SMEM = W_BYTES + NSLOT * SLICE_BYTES + SLABS_BYTES + ND * 4 + 1024;
};
constexpr int THREADS = 32 * (2 + NEPI);
constexpr uint32_t TMEM_COLS = 512;          // two 256-column FP32 accumulators
constexpr int WAIT_LIMIT = 1 << 22;          // try_wait calls before giving up

// instruction descriptor: FP32 D, BF16 A and B, both K-major, N = 256, M = 128
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(ND >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

// Shared-memory matrix descriptor of a K-major operand in the 128-byte swizzle
// layout TMA writes: rows of 128 bytes (64 bf16 of K), 8-row groups 1024 bytes
// apart (SBO), version 1, layout type 2 (128-byte swizzle).  A K = 16 step
// inside the 64-column slice advances the start address by 32 bytes.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool wait(uint32_t bar, uint32_t parity) {
    for (int it = 0; it < WAIT_LIMIT; it++) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" :: "r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" :: "r"(bar) : "memory");
}

// 2D tiled TMA load of box (x, y) of the tensor map into shared memory,
// completing on bar.  x is a multiple of 64 elements (128 bytes).
__device__ __forceinline__ void tma_load(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n"
                 :: "r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar) : "memory");
}

// 2D tiled TMA store of a shared-memory box to (x, y) of the tensor map, in
// the calling thread's bulk group.
__device__ __forceinline__ void tma_store(const CUtensorMap *map, uint32_t src, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];\n"
                 :: "l"((uint64_t)map), "r"(x), "r"(y), "r"(src) : "memory");
}

// Byte offset of 16-byte unit u (0..3) of row r in a slab of 64-byte rows
// with the 64-byte swizzle (unit index XOR bits 1-2 of the row), the layout
// of a TMA box of 32 bf16 columns under CU_TENSOR_MAP_SWIZZLE_64B.  A
// quarter-warp (8 consecutive rows, same u) covers all 32 banks.
__device__ __forceinline__ uint32_t slab_off(int r, int u) { return (uint32_t)(r * 64 + ((u ^ ((r >> 1) & 3)) << 4)); }

__device__ __forceinline__ void commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" :: "r"(bar)
                 : "memory");
}

// The row-major [M][256] bf16 outputs (and the data gradient's gelu'(z)
// input) are reached through tensor maps with 32 x 32 boxes and the 64-byte
// swizzle: mapOut = gelu(z) (forward) or the data gradient, mapAux = gelu'(z)
// (written by the forward, read by the data gradient).
struct Args {
    int M;                // rows (batch), a multiple of 128
    const float *bias;    // EPI_BIAS_GELU: [256]
    int *flag;            // set to 1 when a wait gave up
};

template <int EPI, int NK>
__global__ void __launch_bounds__(THREADS, 1)
    k_gemm_ws(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapW,
              const __grid_constant__ CUtensorMap mapOut, const __grid_constant__ CUtensorMap mapAux, Args g) {
    extern __shared__ unsigned char ws_raw[];
    __shared__ __align__(8) uint64_t full[NSLOT], empty[NSLOT], tfull[2], tempty[2], wfull, mdone, aux[NEPI];
    __shared__ uint32_t tmem_sh;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // 1024-byte aligned base: the swizzle pattern is taken from address bits
    const uint32_t base = (smem_u32(ws_raw) + 1023u) & ~1023u;
    constexpr int W_BYTES = Gemm<NK>::W_BYTES, NSLICE = NK;
    const uint32_t Wsm = base, Asm = base + W_BYTES, Ssm = Asm + NSLOT * SLICE_BYTES;
    float *bias_s = (float *)(ws_raw + (Ssm + SLABS_BYTES - smem_u32(ws_raw)));
    const int ntiles = g.M / BM;
    if (EPI == EPI_BIAS_GELU)
        for (int k = tid; k < ND; k += blockDim.x) bias_s[k] = g.bias[k];
    if (tid == 0) {
        for (int e = 0; e < NEPI; e++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&aux[e])));
        for (int s = 0; s < NSLOT; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&empty[s])));
        }
        for (int a = 0; a < 2; a++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&tfull[a])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" :: "r"(smem_u32(&tempty[a])), "n"(NEPI));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&wfull)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&mdone)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                     :: "r"(smem_u32(&tmem_sh)), "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_sh;

    if (warp == 0 && lane == 0) {
        // ---- producer ----
        bool ok = true;
        expect_tx(smem_u32(&wfull), W_BYTES);
        for (int s = 0; s < NSLICE; s++) tma_load(Wsm + s * WSLICE_BYTES, &mapW, s * KC, 0, smem_u32(&wfull));
        int q = 0;
        for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
            for (int s = 0; s < NSLICE; s++, q++) {
                const int slot = q % NSLOT;
                if (!wait(smem_u32(&empty[slot]), ((q / NSLOT) & 1) ^ 1)) { ok = false; break; }
                expect_tx(smem_u32(&full[slot]), SLICE_BYTES);
                tma_load(Asm + slot * SLICE_BYTES, &mapA, s * KC, t * BM, smem_u32(&full[slot]));
            }
        }
        if (!ok) atomicExch(g.flag, 1);
        // every copy issued lands before the CTA can leave: the weights and the
        // last load of each slot
        wait(smem_u32(&wfull), 0);
        for (int k = q - NSLOT > 0 ? q - NSLOT : 0; k < q; k++) wait(smem_u32(&full[k % NSLOT]), (k / NSLOT) & 1);
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        bool ok = wait(smem_u32(&wfull), 0);
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        int q = 0, li = 0;
        for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, li++) {
            const int acc = li & 1;
            if (!wait(smem_u32(&tempty[acc]), ((li >> 1) & 1) ^ 1)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            const uint32_t dt = tmem + (uint32_t)(acc * ND);
            for (int s = 0; s < NSLICE && ok; s++, q++) {
                const int slot = q % NSLOT;
                if (!wait(smem_u32(&full[slot]), (q / NSLOT) & 1)) { ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;\n");
#pragma unroll
                for (int kk = 0; kk < KC / 16; kk++) {
                    const uint64_t ad = desc_sw128(Asm + slot * SLICE_BYTES + kk * 32);
                    const uint64_t bd = desc_sw128(Wsm + s * WSLICE_BYTES + kk * 32);
                    const uint32_t accumulate = (s > 0 || kk > 0) ? 1u : 0u;
                    asm volatile("{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                                 :: "r"(dt), "l"(ad), "l"(bd), "r"(IDESC), "r"(accumulate));
                }
                commit(smem_u32(&empty[slot]));
            }
            if (ok) commit(smem_u32(&tfull[acc]));
        }
        if (!ok) atomicExch(g.flag, 1);
        // every MMA issued completes before the tensor memory is freed
        commit(smem_u32(&mdone));
        wait(smem_u32(&mdone), 0);
    } else if (warp >= 2) {
        // ---- epilogue ----
        // warp: rows 32 quarter .. of the tile (its tensor-memory lane
        // quarter), columns 64 group .. in two 32-column halves, each through
        // one of the warp's two slabs
        const int quarter = warp & 3, ew = warp - 2, group = ew >> 2;
        const uint32_t slab0 = Ssm + (uint32_t)(ew * 2 * SLAB);
        const uint32_t abar = smem_u32(&aux[ew]);
        bool ok = true;
        int li = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, li++) {
            const int acc = li & 1;
            const int row0 = t * BM + quarter * 32, col0 = group * 64;
            if (EPI == EPI_GELU_BWD && lane == 0) {
                // the previous tile's stores have read the slabs; then this
                // tile's gelu'(z) factors into them (they do not depend on
                // the accumulator)
                asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
                expect_tx(abar, 2 * SLAB);
                tma_load(slab0, &mapAux, col0, row0, abar);
                tma_load(slab0 + SLAB, &mapAux, col0 + 32, row0, abar);
            }
            // one lane waits and the warp follows its answer, so that the warp
            // stays converged for the collective tensor-memory loads
            int okw = lane == 0 ? (int)wait(smem_u32(&tfull[acc]), (li >> 1) & 1) : 0;
            okw = __shfl_sync(0xffffffffu, okw, 0);
            if (EPI == EPI_GELU_BWD) {
                // every lane observes the copy's completion before reading the slabs
                okw = __all_sync(0xffffffffu, okw && wait(abar, li & 1));
            }
            if (!okw) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n");
#pragma unroll
            for (int half = 0; half < 2; half++) {
                const uint32_t sl = slab0 + (uint32_t)(half * SLAB);
                if (EPI == EPI_BIAS_GELU) {
                    // the slabs are free once the stores issued from them have read them
                    if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
                    __syncwarp();
                }
#pragma unroll
                for (int c = 0; c < 2; c++) {
                    const int n0 = col0 + half * 32 + c * 16;
                    uint32_t v[16];
                    const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * ND + n0);
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                        "[%16];\n"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                          "=r"(v[14]), "=r"(v[15])
                        : "r"(taddr));
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                    const uint32_t o0 = slab_off(lane, 2 * c), o1 = slab_off(lane, 2 * c + 1);
                    __align__(16) __nv_bfloat162 o2[8];
                    if (EPI == EPI_BIAS_GELU) {
                        // forward: gelu(z) into slab 0's half, gelu'(z) into slab 1's (one half at a time)
                        __align__(16) __nv_bfloat162 z2[8];
#pragma unroll
                        for (int j = 0; j < 8; j++) {
                            const float2 bb = *(const float2 *)&bias_s[n0 + 2 * j];
                            const float2 z = __fadd2_rn(make_float2(__uint_as_float(v[2 * j]),
                                                                    __uint_as_float(v[2 * j + 1])), bb);
                            float2 hh, gg;
                            gelu_and_grad2(z, hh, gg);
                            o2[j] = __floats2bfloat162_rn(hh.x, hh.y);
                            z2[j] = __floats2bfloat162_rn(gg.x, gg.y);
                        }
                        const uint4 *pz = (const uint4 *)z2;
                        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" :: "r"(slab0 + SLAB + o0),
                                     "r"(pz[0].x), "r"(pz[0].y), "r"(pz[0].z), "r"(pz[0].w) : "memory");
                        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" :: "r"(slab0 + SLAB + o1),
                                     "r"(pz[1].x), "r"(pz[1].y), "r"(pz[1].z), "r"(pz[1].w) : "memory");
                        const uint4 *po = (const uint4 *)o2;
                        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" :: "r"(slab0 + o0),
                                     "r"(po[0].x), "r"(po[0].y), "r"(po[0].z), "r"(po[0].w) : "memory");
                        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" :: "r"(slab0 + o1),
                                     "r"(po[1].x), "r"(po[1].y), "r"(po[1].z), "r"(po[1].w) : "memory");
                    } else {
                        // data gradient: acc * gelu'(z), written over the factors it used
                        __align__(16) uint4 zz[2];
                        asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];\n"
                                     : "=r"(zz[0].x), "=r"(zz[0].y), "=r"(zz[0].z), "=r"(zz[0].w) : "r"(sl + o0) : "memory");
                        asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];\n"
                                     : "=r"(zz[1].x), "=r"(zz[1].y), "=r"(zz[1].z), "=r"(zz[1].w) : "r"(sl + o1) : "memory");
                        const __nv_bfloat162 *z2 = (const __nv_bfloat162 *)zz;
#pragma unroll
                        for (int j = 0; j < 8; j++) {
                            const float2 d = __fmul2_rn(make_float2(__uint_as_float(v[2 * j]),
                                                                    __uint_as_float(v[2 * j + 1])),
                                                        __bfloat1622float2(z2[j]));
                            o2[j] = __floats2bfloat162_rn(d.x, d.y);
                        }
                        const uint4 *po = (const uint4 *)o2;
                        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" :: "r"(sl + o0),
                                     "r"(po[0].x), "r"(po[0].y), "r"(po[0].z), "r"(po[0].w) : "memory");
                        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" :: "r"(sl + o1),
                                     "r"(po[1].x), "r"(po[1].y), "r"(po[1].z), "r"(po[1].w) : "memory");
                    }
                }
                if (half == 1) {
                    // the accumulator has been read: the MMAs of a later tile may overwrite it
                    asm volatile("tcgen05.fence::before_thread_sync;\n");
                    __syncwarp();
                    if (lane == 0) arrive(smem_u32(&tempty[acc]));
                }
                // the slab writes become visible to the async proxy, then one
                // lane stores the boxes
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                __syncwarp();
                if (lane == 0) {
                    if (EPI == EPI_BIAS_GELU) {
                        tma_store(&mapOut, slab0, col0 + half * 32, row0);
                        tma_store(&mapAux, slab0 + SLAB, col0 + half * 32, row0);
                    } else {
                        tma_store(&mapOut, sl, col0 + half * 32, row0);
                    }
                    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
                }
            }
        }
        if (!ok && lane == 0) {
            atomicExch(g.flag, 1);
            // a gelu'(z) copy may still be in flight: let it land (bounded)
            if (EPI == EPI_GELU_BWD) wait(abar, li & 1);
        }
        // the stores have completed before the CTA leaves
        if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
        __syncwarp();
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(tmem), "r"(TMEM_COLS));
}

// ---------------------------------------------------------------------------
// Weight gradient of a 256 x 256 hidden layer, split over the batch:
//   part[split][m][n] = sum over the split's rows b of dZ[b][m] H[b][n]
// (the batch, the reduction index, is the slow index of both operands, so
// both are MN-major).  CTA `split` takes WROWS consecutive rows in 64-row
// chunks: warp 0 loads each chunk of dZ and of H as four 64 x 64 boxes apiece
// (TMA, 128-byte swizzle) into a three-stage ring, warp 1 accumulates the two
// 128-row halves of the 256 x 256 product in tensor memory (all 512
// columns), and eight warps write the FP32 partial.  While the MMAs run, the
// same eight warps sum each column of dZ over the split's rows from the
// staged boxes (thread m: column m), the bias gradient's partial
// bpart[split][m]; a stage is released when its MMAs and these reads are
// done.
constexpr int WROWS = 512;                      // batch rows per split (a multiple of WCH)
constexpr int WCH = 64;                         // rows per chunk
constexpr int WBOX = 64 * WCH * 2;              // one 64 (MN) x 64 (K) box: 8 KB
constexpr int WSTAGE = 8 * WBOX;                // dZ and H boxes of one chunk: 64 KB
constexpr int WNST = 3;
constexpr int WSMEM = WNST * WSTAGE + 1024;
constexpr int WEPI = 8;
constexpr int WTHREADS = 32 * (2 + WEPI);

// MN-major operand in the 128-byte swizzle layout: 64-element (128-byte) rows
// along MN, one per K index; 8-row K groups 1024 bytes apart (SBO), the next
// 64 MN elements one box (8 KB) further (LBO); a K = 16 step advances the
// start by two K groups (2048 bytes).
__device__ __forceinline__ uint64_t desc_sw128_mn(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(WBOX >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// The partials are written through mapPart: FP32 [splits * 256][64 NH], boxes
// of 32 x 32 with the 128-byte swizzle.  After the last MMA the ring is free
// and each epilogue warp stages its 32 rows there, up to 128 columns at a time
// (four boxes), for TMA stores.  Instruction descriptor: FP32 D, BF16 A and B,
// both MN-major (bits 15 / 16), N = 64 NH, M = 128.
template <int NH>
__global__ void __launch_bounds__(WTHREADS, 1)
    k_wgrad_ws(const __grid_constant__ CUtensorMap mapDz, const __grid_constant__ CUtensorMap mapH,
               const __grid_constant__ CUtensorMap mapPart, int M, int rows, float *__restrict__ bpart, int *flag) {
    // N = 64 NH columns of H (4 boxes for a 256-wide layer, 1 for the first
    // layer's inputs padded to 64); tensor memory: two M halves of N columns
    constexpr int NCOL = 64 * NH, PASSES = NCOL >= 128 ? NCOL / 128 : 1, PCOLS = NCOL / PASSES;
    constexpr uint32_t TCOLS = 2 * NCOL;
    constexpr uint32_t IDESC_W = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                                 ((uint32_t)(NCOL >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
    constexpr uint32_t STAGE_TX = (4 + NH) * WBOX;
    extern __shared__ unsigned char ws_raw[];
    __shared__ __align__(8) uint64_t full[WNST], empty[WNST], tfull, mdone;
    __shared__ uint32_t tmem_sh;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t base = (smem_u32(ws_raw) + 1023u) & ~1023u;
    const int r0 = blockIdx.x * rows, nch = rows / WCH;
    if (tid == 0) {
        for (int s = 0; s < WNST; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&full[s])));
            // released by the MMAs' commit and by each column-sum warp
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" :: "r"(smem_u32(&empty[s])), "n"(1 + WEPI));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&tfull)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&mdone)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                     :: "r"(smem_u32(&tmem_sh)), "r"(TCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_sh;
    if (warp == 0 && lane == 0) {
        // ---- producer: boxes 0..3 dZ columns 64j.., boxes 4..7 H columns 64j.. ----
        bool ok = true;
        int c = 0;
        for (; c < nch && r0 + c * WCH < M; c++) {
            const int st = c % WNST;
            if (!wait(smem_u32(&empty[st]), ((c / WNST) & 1) ^ 1)) { ok = false; break; }
            expect_tx(smem_u32(&full[st]), STAGE_TX);
            const uint32_t dst = base + st * WSTAGE;
            for (int j = 0; j < 4; j++) tma_load(dst + j * WBOX, &mapDz, 64 * j, r0 + c * WCH, smem_u32(&full[st]));
            for (int j = 0; j < NH; j++)
                tma_load(dst + (4 + j) * WBOX, &mapH, 64 * j, r0 + c * WCH, smem_u32(&full[st]));
        }
        if (!ok) atomicExch(flag, 1);
        for (int k = c - WNST > 0 ? c - WNST : 0; k < c; k++) wait(smem_u32(&full[k % WNST]), (k / WNST) & 1);
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer: D_h (columns 256 h..) += dZ[:, 128 h..]^T H ----
        bool ok = true;
        for (int c = 0; c < nch && r0 + c * WCH < M && ok; c++) {
            const int st = c % WNST;
            if (!wait(smem_u32(&full[st]), (c / WNST) & 1)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            const uint32_t src = base + st * WSTAGE;
#pragma unroll
            for (int kk = 0; kk < WCH / 16; kk++)
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const uint64_t ad = desc_sw128_mn(src + (2 * h) * WBOX + kk * 2048);
                    const uint64_t bd = desc_sw128_mn(src + 4 * WBOX + kk * 2048);
                    const uint32_t accumulate = (c > 0 || kk > 0) ? 1u : 0u;
                    asm volatile("{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                                 :: "r"(tmem + (uint32_t)(h * NCOL)), "l"(ad), "l"(bd), "r"(IDESC_W), "r"(accumulate));
                }
            commit(smem_u32(&empty[st]));
        }
        if (ok) commit(smem_u32(&tfull));
        else atomicExch(flag, 1);
        commit(smem_u32(&mdone));
        wait(smem_u32(&mdone), 0);
    } else if (warp >= 2) {
        // ---- column sums of dZ while the MMAs run (thread e: column e) ----
        const int e = tid - 64;
        const int bj = e >> 6, chunk = (e & 63) >> 3, elem = e & 7;
        float bsum = 0.0f;
        int okw = 1;
        for (int c = 0; c < nch && r0 + c * WCH < M; c++) {
            const int st = c % WNST;
            okw = lane == 0 ? (int)wait(smem_u32(&full[st]), (c / WNST) & 1) : 0;
            okw = __shfl_sync(0xffffffffu, okw, 0);
            if (!okw) break;
            // box bj of dZ: row k at 128 k bytes, its 16-byte chunks swizzled by k % 8
            const unsigned char *box = ws_raw + (base - smem_u32(ws_raw)) + st * WSTAGE + bj * WBOX;
#pragma unroll 8
            for (int k = 0; k < WCH; k++)
                bsum += __bfloat162float(*(const bf16 *)(box + k * 128 + ((chunk ^ (k & 7)) << 4) + elem * 2));
            __syncwarp();
            if (lane == 0) arrive(smem_u32(&empty[st]));
        }
        if (okw) bpart[(size_t)blockIdx.x * ND + e] = bsum;
        // the ring is reused for staging below: every column-sum warp has
        // finished reading it (named barrier 1 over the WEPI epilogue warps)
        asm volatile("bar.sync 1, %0;\n" :: "n"(WEPI * 32) : "memory");
        // ---- epilogue: warp -> (32-lane quarter, half of the rows' M-half) ----
        const int quarter = warp & 3, h = (warp - 2) >> 2;
        if (okw) okw = lane == 0 ? (int)wait(smem_u32(&tfull), 0) : 0;
        okw = __shfl_sync(0xffffffffu, okw, 0);
        if (okw) {
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            // the ring is free: every stage has been consumed by the MMAs and
            // the column sums; 16 KB of it per warp
            const uint32_t stg = base + (uint32_t)((warp - 2) * 4 * 4096);
            const int prow = blockIdx.x * ND + h * BM + quarter * 32;
#pragma unroll 1
            for (int pass = 0; pass < PASSES; pass++) {
                if (pass == 1) {
                    if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
                    __syncwarp();
                }
#pragma unroll 1
                for (int ch = 0; ch < PCOLS / 16; ch++) {
                    uint32_t v[16];
                    const uint32_t taddr =
                        tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(h * NCOL + pass * PCOLS + ch * 16);
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                        "[%16];\n"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                          "=r"(v[14]), "=r"(v[15])
                        : "r"(taddr));
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                    // box ch / 2 (32 columns), 16-byte units 4 (ch % 2) .. of row lane,
                    // swizzled by lane % 8 (conflict-free per quarter-warp)
                    const uint32_t bx = stg + (uint32_t)((ch >> 1) * 4096 + lane * 128);
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int u = (ch & 1) * 4 + j;
                        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n"
                                     :: "r"(bx + (uint32_t)((u ^ (lane & 7)) << 4)), "r"(v[4 * j]), "r"(v[4 * j + 1]),
                                        "r"(v[4 * j + 2]), "r"(v[4 * j + 3]) : "memory");
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                __syncwarp();
                if (lane == 0) {
                    for (int j = 0; j < PCOLS / 32; j++)
                        tma_store(&mapPart, stg + j * 4096, pass * PCOLS + j * 32, prow);
                    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
                }
            }
            if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
            __syncwarp();
        } else if (lane == 0) {
            atomicExch(flag, 1);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(tmem), "r"(TCOLS));
}

}  // namespace ws
}  // namespace mlp
}  // namespace e2d
