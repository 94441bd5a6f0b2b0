// mlp.cu -- the coordinate MLP of the learned warm start, trained on the GPU
// by the kernels of mlp_kernels.cuh.  No reference counterpart.
//
// Network: 32 inputs (22 features, zero padded) -> H -> ... -> H (nhidden
// layers, GELU) -> 4 outputs.  Weights are kept in FP32 (Adam master copy) and
// used in BF16; activations and their gradients are BF16; every product
// accumulates in FP32.  The output layer (H -> 4) runs on the CUDA cores.
// One training step (batch gather, forward, MSE loss, backward, Adam) is one
// CUDA graph; the step counter lives in device memory so the graph is static.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "mlp_kernels.cuh"
#include "mlp_tma.cuh"
#include "solver_internal.h"

using namespace e2d;
using namespace e2d::mlp;

#define CK(call)                                                                       \
    do {                                                                               \
        cudaError_t err_ = (call);                                                     \
        if (err_ != cudaSuccess) {                                                     \
            set_error(std::string("CUDA: ") + #call + ": " + cudaGetErrorString(err_)); \
            return E2D_ERR_CUDA;                                                       \
        }                                                                              \
    } while (0)

namespace {

constexpr int NIN = E2D_MLP_INPUTS;  // padded input width
// Row width of the batch's inputs and of the first layer's BF16 weights on
// the device: the inputs padded with zeros to one 64-column (128-byte) slice,
// the first layer's K on the tensor cores.
constexpr int KX = 64;
constexpr int NOUT = 4;
constexpr int H = 256;
constexpr int kSplits = 64;          // split-K over the batch for weight gradients

__global__ void k_step_update(int *step, float beta1, float beta2, float *bc) {
    const int s = ++*step;
    bc[0] = 1.f - powf(beta1, (float)s);
    bc[1] = 1.f - powf(beta2, (float)s);
}

// One parameter tensor's Adam step: the gradient of element i = (r, c) is the
// sum of nparts partials part[p * pstride + r * pld + c]; wbf (may be null,
// row pitch wld) is the bf16 copy used by
// the GEMMs, wbfT (may be null) its transpose ([cols][rows], the data-gradient
// GEMM's K-major operand); grad_out (may be null) receives the gradient.
struct AdamSeg {
    const float *part;
    size_t pstride;
    int nparts, count, rows, cols;
    int pld, wld;  // row pitch of a partial and of wbf (elements; cols unless padded)
    float *w32, *m, *v;
    bf16 *wbf, *wbfT;
    float *grad_out;
};

// Adam on two tensors (a layer's weights and bias) in one launch: blocks
// [0, nb0) take seg0, the rest seg1, 128 parameters per 256-thread block
// (every count, stride and partial offset a multiple of 4).  Lane l of warp j
// sums parameters 4l .. 4l + 3 of the block over partials j, j + 8, ...
// (16-byte loads, sixteen in flight: one round for up to 128 partials; the
// partials are still in L2, so the kernel is bound by the latency of its
// rounds), the eight warp sums are added in a fixed tree (deterministic), and
// warp 0 applies the step with its moments and weights requested up front.  lr (device, read at run
// time so that the host can schedule it) null: gradient only.
__global__ void __launch_bounds__(256) k_adam_seg(AdamSeg seg0, AdamSeg seg1, int nb0,
                                                  const float *__restrict__ lr_dev, float beta1, float beta2,
                                                  float eps, const float *__restrict__ bc) {
    __shared__ float4 red[8][32];
    const bool first = (int)blockIdx.x < nb0;
    const AdamSeg &S = first ? seg0 : seg1;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int i = (((int)blockIdx.x - (first ? 0 : nb0)) * 32 + lane) * 4;
    const int ri = i / S.cols, ci = i % S.cols;  // cols is 1 or a multiple of 4
    const bool live = i < S.count;
    // the step's other operands are requested first: they do not depend on the sum
    float4 m4 = make_float4(0.f, 0.f, 0.f, 0.f), v4 = m4, w4 = m4;
    float lr = 0.f, bc0 = 1.f, bc1 = 1.f;
    if (wp == 0 && live && lr_dev) {
        m4 = *(const float4 *)(S.m + i);
        v4 = *(const float4 *)(S.v + i);
        w4 = *(const float4 *)(S.w32 + i);
        lr = *lr_dev;
        bc0 = bc[0];
        bc1 = bc[1];
    }
    // partials wp, wp + 8, ..., sixteen 16-byte loads in flight per round
    float4 a[2] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
    if (live) {
        const float *pp = S.part + (size_t)ri * S.pld + ci;
        for (int p0 = wp; p0 < S.nparts; p0 += 128) {
            float4 v[16];
#pragma unroll
            for (int j = 0; j < 16; j++)
                v[j] = p0 + 8 * j < S.nparts ? *(const float4 *)(pp + (size_t)(p0 + 8 * j) * S.pstride)
                                             : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int j = 0; j < 16; j++) {
                float4 &t = a[j & 1];
                t.x += v[j].x; t.y += v[j].y; t.z += v[j].z; t.w += v[j].w;
            }
        }
    }
    red[wp][lane] = make_float4(a[0].x + a[1].x, a[0].y + a[1].y, a[0].z + a[1].z, a[0].w + a[1].w);
    __syncthreads();
    if (wp != 0 || !live) return;
    float g[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float r[8];
#pragma unroll
        for (int k = 0; k < 8; k++) r[k] = ((const float *)&red[k][lane])[q];
        g[q] = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
    }
    if (S.grad_out) *(float4 *)(S.grad_out + i) = make_float4(g[0], g[1], g[2], g[3]);
    if (!lr_dev) return;
    float mo[4], vo[4], wo[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        mo[q] = beta1 * ((const float *)&m4)[q] + (1.f - beta1) * g[q];
        vo[q] = beta2 * ((const float *)&v4)[q] + (1.f - beta2) * g[q] * g[q];
        wo[q] = ((const float *)&w4)[q] - lr * (mo[q] / bc0) / (sqrtf(vo[q] / bc1) + eps);
    }
    *(float4 *)(S.m + i) = make_float4(mo[0], mo[1], mo[2], mo[3]);
    *(float4 *)(S.v + i) = make_float4(vo[0], vo[1], vo[2], vo[3]);
    *(float4 *)(S.w32 + i) = make_float4(wo[0], wo[1], wo[2], wo[3]);
    if (S.wbf) {
        __align__(8) __nv_bfloat162 h2[2] = {__floats2bfloat162_rn(wo[0], wo[1]), __floats2bfloat162_rn(wo[2], wo[3])};
        *(uint2 *)(S.wbf + (size_t)ri * S.wld + ci) = *(const uint2 *)h2;
    }
    if (S.wbfT)
#pragma unroll
        for (int q = 0; q < 4; q++)
            S.wbfT[(size_t)((i + q) % S.cols) * S.rows + (i + q) / S.cols] = __float2bfloat16_rn(wo[q]);
}

// bf16 copy (row pitch ld) of a [rows][cols] matrix, and (bT non-null) of its transpose
__global__ void k_to_bf16(int n, const float *__restrict__ a, bf16 *__restrict__ b, bf16 *__restrict__ bT, int rows,
                          int cols, int ld) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    b[(size_t)(i / cols) * ld + i % cols] = __float2bfloat16_rn(a[i]);
    if (bT) bT[(size_t)(i % cols) * rows + i / cols] = __float2bfloat16_rn(a[i]);
}

// Minimum distance from each point to a set of segments (wall faces).
__global__ void __launch_bounds__(256) k_wall_distance(int n, const double *__restrict__ px,
                                                       const double *__restrict__ py, int nseg,
                                                       const double4 *__restrict__ seg, double *__restrict__ d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    __shared__ double4 s[256];
    double best = 1e300;
    const double x = i < n ? px[i] : 0.0, y = i < n ? py[i] : 0.0;
    for (int base = 0; base < nseg; base += 256) {
        __syncthreads();
        if (base + (int)threadIdx.x < nseg) s[threadIdx.x] = seg[base + threadIdx.x];
        __syncthreads();
        const int cnt = min(256, nseg - base);
        for (int k = 0; k < cnt; k++) {
            const double4 q = s[k];
            const double ex = q.z - q.x, ey = q.w - q.y;
            const double L2 = ex * ex + ey * ey;
            double t = L2 > 0 ? ((x - q.x) * ex + (y - q.y) * ey) / L2 : 0.0;
            t = fmin(1.0, fmax(0.0, t));
            const double dx = x - (q.x + t * ex), dy = y - (q.y + t * ey);
            best = fmin(best, dx * dx + dy * dy);
        }
    }
    if (i < n) d[i] = sqrt(best);
}

struct Tensor {
    int rows, cols;
    float *w32 = nullptr, *m = nullptr, *v = nullptr;
    bf16 *wbf = nullptr;   // hidden layers: [rows][wld()] (the first layer padded to KX columns)
    bf16 *wbfT = nullptr;  // hidden layers after the first: [cols][rows]
    int count() const { return rows * cols; }
    int wld() const { return cols == NIN ? KX : cols; }
};

}  // namespace

struct e2d_mlp {
    e2d_mlp_config cfg;
    int nhidden = 5;
    std::vector<Tensor> W, b;  // hidden layers (W: H x in, b: H x 1) then the output layer
    // batch buffers
    int B = 0;
    bf16 *xb = nullptr;  // [B][KX], the inputs in the first NIN columns
    float *tb = nullptr, *y = nullptr, *dy = nullptr;
    std::vector<bf16 *> Gd, Hh;  // [nhidden] of [B][H]: gelu'(z) and gelu(z) of each hidden layer
    bf16 *dz[2] = {nullptr, nullptr};  // [B][H]
    // weight- and bias-gradient partials, two sets: a layer's Adam step reads
    // one on the side stream while the next layer's gradient fills the other
    float *part[2] = {nullptr, nullptr};
    float *bpart[2] = {nullptr, nullptr};
    double *loss_part = nullptr;
    int *step_dev = nullptr;
    int *flag_dev = nullptr;    // set by a tensor-core GEMM whose wait timed out
    float *bc_dev = nullptr;
    float *lr_dev = nullptr;    // Adam step size, read by every step
    float *grad = nullptr;      // flat gradient of all parameters (gradient probe)
    // training set
    bf16 *X = nullptr;
    float *T = nullptr;
    long long nsamples = 0, cap_samples = 0;
    std::vector<void *> allocs;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;  // Adam steps, overlapping the next layer's gradient
    cudaEvent_t ev_fork = nullptr, ev_done[2] = {nullptr, nullptr};
    cudaGraphExec_t gexec = nullptr;
    // TMA tensor maps of the 256 x 256 GEMMs (ws::k_gemm_ws), per hidden layer
    // l >= 1: forward A = Hh[l-1], W_l; data gradient A = dz[0] / dz[1], W_l^T
    bool use_ws = false;
    int nsm = 0;
    std::vector<CUtensorMap> mapHf, mapW, mapWT, mapHw;
    std::vector<CUtensorMap> mapHo, mapGo;  // Hh[l], Gd[l] in 32 x 32 epilogue slabs
    // dz[0] / dz[1] with 128-row boxes (data gradient), 64-row boxes (weights), 32 x 32 slabs
    CUtensorMap mapDz[2], mapDzw[2], mapDzo[2];
    CUtensorMap mapPart[2], mapPart0[2];  // weight-gradient partials: 256 x 256 layers, the first layer (256 x KX)
    CUtensorMap mapX, mapXw, mapW0;   // the first layer's inputs (128- and 64-row boxes) and BF16 weights
    int wrows = ws::WROWS;  // batch rows per weight-gradient split
    std::vector<double> loss_host;

    ~e2d_mlp() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (stream) cudaStreamDestroy(stream);
        if (side) cudaStreamDestroy(side);
        if (ev_fork) cudaEventDestroy(ev_fork);
        for (cudaEvent_t e : ev_done)
            if (e) cudaEventDestroy(e);
        for (void *p : allocs) cudaFree(p);
        if (X) cudaFree(X);
        if (T) cudaFree(T);
    }
    template <typename P> int alloc(P **p, size_t bytes) {
        CK(cudaMalloc((void **)p, bytes));
        CK(cudaMemset(*p, 0, bytes));
        allocs.push_back(*p);
        return E2D_OK;
    }
};

namespace {

// cuTensorMapEncodeTiled of the driver, found through the runtime (no link
// against the driver library)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return (PFN_cuTensorMapEncodeTiled_v12000)p;
    }();
    return fn;
}

// 2D map of a row-major [rows][cols] bf16 matrix, box 64 columns x box_rows,
// 128-byte swizzle (the layout the ws kernel's descriptors describe)
// Row-major [rows][cols] bf16 tensor, boxes of box_rows x 64 columns with the
// 128-byte swizzle (MMA operands) or, slab = true, 32 x 32 with the 64-byte
// swizzle (the epilogue slabs of ws::k_gemm_ws).
bool map_2d(CUtensorMap *map, const bf16 *ptr, uint64_t rows, uint64_t cols, uint32_t box_rows, bool slab = false) {
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * sizeof(bf16)};
    const cuuint32_t box[2] = {slab ? 32u : (cuuint32_t)ws::KC, slab ? 32u : box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)ptr, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, slab ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The weight-gradient partials, FP32 [rows][cols], as boxes of 32 x 32 with the
// 128-byte swizzle (the staging layout of ws::k_wgrad_ws's epilogue).
bool map_part(CUtensorMap *map, const float *ptr, uint64_t rows, uint64_t cols) {
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * sizeof(float)};
    const cuuint32_t box[2] = {32, 32};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)ptr, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor maps of the warp-specialised GEMMs once the batch buffers exist;
// use_ws stays false (the per-tile kernel runs every layer) when the driver
// entry point, a map or the shared-memory size is not available, or
// E2D_MLP_WS=0.  With E2D_MLP_WS=1 that is an error instead.
int build_ws_maps(e2d_mlp *m) {
    m->use_ws = false;
    const char *env = std::getenv("E2D_MLP_WS");
    const bool required = env && env[0] == '1';
    if (env && env[0] == '0') return E2D_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&m->nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        if (required) { set_error("E2D_MLP_WS=1: no device attributes"); return E2D_ERR_CUDA; }
        return E2D_OK;
    }
    m->mapHf.assign(m->nhidden, CUtensorMap{});
    m->mapW.assign(m->nhidden, CUtensorMap{});
    m->mapWT.assign(m->nhidden, CUtensorMap{});
    m->mapHw.assign(m->nhidden, CUtensorMap{});
    m->mapHo.assign(m->nhidden, CUtensorMap{});
    m->mapGo.assign(m->nhidden, CUtensorMap{});
    bool ok = m->wrows >= ws::WCH && m->wrows % ws::WCH == 0 && m->B % m->wrows == 0;
    for (int l = 0; l < m->nhidden && ok; l++) {
        ok = ok && map_2d(&m->mapHo[l], m->Hh[l], m->B, H, 32, true);
        ok = ok && map_2d(&m->mapGo[l], m->Gd[l], m->B, H, 32, true);
    }
    for (int l = 1; l < m->nhidden && ok; l++) {
        ok = ok && map_2d(&m->mapHf[l], m->Hh[l - 1], m->B, H, ws::BM);
        ok = ok && map_2d(&m->mapW[l], m->W[l].wbf, H, H, ws::ND);
        ok = ok && map_2d(&m->mapWT[l], m->W[l].wbfT, H, H, ws::ND);
        ok = ok && map_2d(&m->mapHw[l], m->Hh[l - 1], m->B, H, ws::WCH);
    }
    for (int k = 0; k < 2 && ok; k++) {
        ok = ok && map_2d(&m->mapDz[k], m->dz[k], m->B, H, ws::BM);
        ok = ok && map_2d(&m->mapDzw[k], m->dz[k], m->B, H, ws::WCH);
        ok = ok && map_2d(&m->mapDzo[k], m->dz[k], m->B, H, 32, true);
    }
    for (int k = 0; k < 2 && ok; k++) {
        ok = ok && map_part(&m->mapPart[k], m->part[k], (uint64_t)(m->B / m->wrows) * H, H);
        ok = ok && map_part(&m->mapPart0[k], m->part[k], (uint64_t)(m->B / m->wrows) * H, KX);
    }
    ok = ok && map_2d(&m->mapX, m->xb, m->B, KX, ws::BM);
    ok = ok && map_2d(&m->mapXw, m->xb, m->B, KX, ws::WCH);
    ok = ok && map_2d(&m->mapW0, m->W[0].wbf, H, KX, ws::ND);
    const auto smem_ok = [](const void *f, int bytes) {
        return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess;
    };
    if (ok && smem_ok((const void *)ws::k_gemm_ws<EPI_BIAS_GELU, 4>, ws::Gemm<4>::SMEM) &&
        smem_ok((const void *)ws::k_gemm_ws<EPI_BIAS_GELU, 1>, ws::Gemm<1>::SMEM) &&
        smem_ok((const void *)ws::k_gemm_ws<EPI_GELU_BWD, 4>, ws::Gemm<4>::SMEM) &&
        smem_ok((const void *)ws::k_wgrad_ws<4>, ws::WSMEM) && smem_ok((const void *)ws::k_wgrad_ws<1>, ws::WSMEM))
        m->use_ws = true;
    cudaGetLastError();
    if (required && !m->use_ws) {
        set_error("E2D_MLP_WS=1: the warp-specialised GEMMs cannot run here (tensor maps or shared memory)");
        return E2D_ERR_CUDA;
    }
    return E2D_OK;
}

template <int EPI, int NK>
void gemm_ws(e2d_mlp *m, const CUtensorMap &a, const CUtensorMap &w, const CUtensorMap &out, const CUtensorMap &aux,
             ws::Args g, cudaStream_t s) {
    g.flag = m->flag_dev;
    const int ntiles = g.M / ws::BM, grid = ntiles < m->nsm ? ntiles : m->nsm;
    ws::k_gemm_ws<EPI, NK><<<grid, ws::THREADS, ws::Gemm<NK>::SMEM, s>>>(a, w, out, aux, g);
}

size_t param_count(const e2d_mlp *m) {
    size_t c = 0;
    for (size_t l = 0; l < m->W.size(); l++) c += m->W[l].count() + m->b[l].count();
    return c;
}

int ensure_batch(e2d_mlp *m, int B) {
    if (m->B == B) return E2D_OK;
    if (m->B != 0) { set_error("batch size is fixed at the first use"); return E2D_ERR_ARG; }
    if (B < 2048 || B % 2048 != 0) {  // split-K slices of the batch are multiples of BK
        set_error("batch must be a positive multiple of 2048");
        return E2D_ERR_ARG;
    }
    m->B = B;
    int rc;
    if ((rc = m->alloc(&m->xb, sizeof(bf16) * (size_t)B * KX))) return rc;  // columns NIN.. stay zero
    if ((rc = m->alloc(&m->tb, sizeof(float) * (size_t)B * NOUT))) return rc;
    if ((rc = m->alloc(&m->y, sizeof(float) * (size_t)B * NOUT))) return rc;
    if ((rc = m->alloc(&m->dy, sizeof(float) * (size_t)B * NOUT))) return rc;
    m->Gd.resize(m->nhidden);
    m->Hh.resize(m->nhidden);
    for (int l = 0; l < m->nhidden; l++) {
        if ((rc = m->alloc(&m->Gd[l], sizeof(bf16) * (size_t)B * H))) return rc;
        if ((rc = m->alloc(&m->Hh[l], sizeof(bf16) * (size_t)B * H))) return rc;
    }
    for (int k = 0; k < 2; k++)
        if ((rc = m->alloc(&m->dz[k], sizeof(bf16) * (size_t)B * H))) return rc;
    // weight-gradient partials: kSplits of the per-tile kernel, or one per
    // wrows rows of the batch for the warp-specialised one (512 rows: 128
    // CTAs at batch 65536, 20.7 us per layer against 26.9 us for 1024 rows,
    // with Adam summing twice the partials)
    const int nparts = std::max(kSplits, B / m->wrows);
    for (int k = 0; k < 2; k++)
        if ((rc = m->alloc(&m->part[k], sizeof(float) * (size_t)nparts * H * H))) return rc;
    // bias / output-layer partials: the same, or one per 256 rows for the output layer
    for (int k = 0; k < 2; k++)
        if ((rc = m->alloc(&m->bpart[k], sizeof(float) * (size_t)std::max(nparts, B / 256) * (NOUT * H + NOUT + H))))
            return rc;
    if ((rc = m->alloc(&m->loss_part, sizeof(double) * (B / 256)))) return rc;
    return build_ws_maps(m);
}

AdamSeg adam_seg(const Tensor &t, const float *part, int nparts, size_t pstride, float *grad_out, int pld = 0) {
    AdamSeg g{};
    g.part = part; g.pstride = pstride; g.nparts = nparts; g.count = t.count();
    g.rows = t.rows; g.cols = t.cols;
    g.pld = pld ? pld : t.cols; g.wld = t.wld();
    g.w32 = t.w32; g.m = t.m; g.v = t.v; g.wbf = t.wbf; g.wbfT = t.wbfT;
    g.grad_out = grad_out;
    return g;
}

// Adam on a weight tensor and its bias in one launch.
void adam2(e2d_mlp *m, cudaStream_t s, const AdamSeg &w, const AdamSeg &b, const float *lr) {
    const auto &c = m->cfg;
    const int nb0 = (w.count + 127) / 128, nb1 = (b.count + 127) / 128;
    k_adam_seg<<<nb0 + nb1, 256, 0, s>>>(w, b, nb0, lr, (float)c.beta1, (float)c.beta2, (float)c.eps, m->bc_dev);
}

template <bool TA, bool TB, int EPI> void gemm(e2d_mlp *m, GemmArgs g, dim3 grid, cudaStream_t s) {
    g.flag = m->flag_dev;
    k_gemm_tc<TA, TB, EPI><<<grid, 256, tc::SMEM, s>>>(g);
}

// Reports (and clears) a timed-out tensor-core wait of the kernels run so far.
int check_flag(e2d_mlp *m) {
    int f = 0;
    CK(cudaMemcpyAsync(&f, m->flag_dev, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    if (f) {
        CK(cudaMemsetAsync(m->flag_dev, 0, sizeof(int), m->stream));
        set_error("a tensor-core GEMM gave up waiting for its MMAs; its results are not valid");
        return E2D_ERR_CUDA;
    }
    return E2D_OK;
}

// Forward on the batch in xb (rows B) through the hidden layers; without
// targets (inference) also the output layer into y.
void forward(e2d_mlp *m, cudaStream_t s, bool with_loss) {
    const int B = m->B;
    for (int l = 0; l < m->nhidden; l++) {
        if (m->use_ws) {
            ws::Args a{};
            a.M = B; a.bias = m->b[l].w32;
            if (l == 0) gemm_ws<EPI_BIAS_GELU, 1>(m, m->mapX, m->mapW0, m->mapHo[0], m->mapGo[0], a, s);
            else gemm_ws<EPI_BIAS_GELU, 4>(m, m->mapHf[l], m->mapW[l], m->mapHo[l], m->mapGo[l], a, s);
            continue;
        }
        GemmArgs g{};
        g.M = B; g.N = H; g.K = l == 0 ? NIN : H;
        g.A = l == 0 ? m->xb : m->Hh[l - 1];
        g.lda = l == 0 ? KX : H;
        g.B = m->W[l].wbf; g.ldb = m->W[l].wld();
        g.bias = m->b[l].w32; g.out = m->Hh[l]; g.zout = m->Gd[l]; g.ldc = H;
        gemm<false, false, EPI_BIAS_GELU>(m, g, dim3(H / BN, (B + BM - 1) / BM, 1), s);
    }
    // with targets the output layer runs at the start of the backward pass
    // (k_out_train), fused with its gradient
    if (with_loss) return;
    const Tensor &Wo = m->W[m->nhidden], &bo = m->b[m->nhidden];
    k_out_fwd_loss<H, NOUT><<<(B + 255) / 256, 256, 0, s>>>(B, m->Hh[m->nhidden - 1], Wo.w32, bo.w32, nullptr,
                                                            m->y, m->dy, nullptr);
}

// Backward + Adam with the step size at lr (null: gradient only, written to
// m->grad in parameter order).
void backward(e2d_mlp *m, cudaStream_t s, const float *lr, bool want_grad) {
    const int B = m->B, L = m->nhidden;
    const int rows = B / kSplits;
    size_t goff = param_count(m);
    auto gslot = [&](const Tensor &t) -> float * {
        if (!want_grad) return nullptr;
        goff -= t.count();
        return m->grad + goff;
    };
    // Each layer's Adam step runs on the side stream, forked after the
    // layer's weight gradient, while the main stream goes on with the next
    // layer (which needs neither the updated weights nor these partials);
    // the partial sets alternate, and a set is only refilled after the Adam
    // step that read it.  Both streams join at the end.
    bool used[2] = {false, false};
    auto claim = [&](int k) {
        if (used[k]) cudaStreamWaitEvent(s, m->ev_done[k], 0);
    };
    auto fork_adam = [&](int k, const AdamSeg &w, const AdamSeg &bias) {
        cudaEventRecord(m->ev_fork, s);
        cudaStreamWaitEvent(m->side, m->ev_fork, 0);
        adam2(m, m->side, w, bias, lr);
        cudaEventRecord(m->ev_done[k], m->side);
        used[k] = true;
    };
    // output layer, forward and backward in one pass (loss, its weight / bias
    // partials, and the gradient at the last pre-activation: the output
    // layer's data gradient times the stored gelu'(z))
    Tensor &Wo = m->W[L], &bo = m->b[L];
    const int oparts = B / 256;
    k_out_train<H, NOUT><<<oparts, 256, 0, s>>>(B, m->Hh[L - 1], Wo.w32, bo.w32, m->tb, m->Gd[L - 1], m->y, m->dy,
                                                m->dz[0], m->bpart[0], m->loss_part);
    const size_t ostride = NOUT * H + NOUT;
    float *gbo = gslot(bo);
    float *gWo = gslot(Wo);
    fork_adam(0, adam_seg(Wo, m->bpart[0], oparts, ostride, gWo),
              adam_seg(bo, m->bpart[0] + NOUT * H, oparts, ostride, gbo));
    int cur = 0;
    for (int l = L - 1; l >= 0; l--) {
        const int kin = l == 0 ? NIN : H, pk = (L - l) & 1;  // partial set of this layer
        // gradient at the previous pre-activation, first (it reads W_l before
        // this layer's Adam step changes it): dz W_l, W_l read MN-major
        // ([out][in] = [K][N]); then the weight gradient, whose partials the
        // Adam step reads straight after, while they are still in L2
        if (l > 0 && m->use_ws) {
            ws::Args a{};
            a.M = B;
            gemm_ws<EPI_GELU_BWD, 4>(m, m->mapDz[cur], m->mapWT[l], m->mapDzo[cur ^ 1], m->mapGo[l - 1], a, s);
        } else if (l > 0) {
            GemmArgs gd{};
            gd.M = B; gd.N = H; gd.K = H;
            gd.A = m->dz[cur]; gd.lda = H;
            gd.B = m->W[l].wbf; gd.ldb = H;
            gd.zin = m->Gd[l - 1]; gd.out = m->dz[cur ^ 1]; gd.ldc = H;
            gemm<false, true, EPI_GELU_BWD>(m, gd, dim3(H / BN, (B + BM - 1) / BM, 1), s);
        }
        claim(pk);
        // dW_l = dz^T hin (split over the batch; both operands are read
        // MN-major, the batch index being their slow one), db_l = column sums
        // of dz
        int wparts = kSplits, pld = kin;
        if (m->use_ws) {
            // the first layer's partials are 256 x KX (its padding columns get zero)
            wparts = B / m->wrows;
            if (l == 0) {
                pld = KX;
                ws::k_wgrad_ws<1><<<wparts, ws::WTHREADS, ws::WSMEM, s>>>(m->mapDzw[cur], m->mapXw, m->mapPart0[pk],
                                                                          B, m->wrows, m->bpart[pk], m->flag_dev);
            } else {
                ws::k_wgrad_ws<4><<<wparts, ws::WTHREADS, ws::WSMEM, s>>>(m->mapDzw[cur], m->mapHw[l], m->mapPart[pk],
                                                                          B, m->wrows, m->bpart[pk], m->flag_dev);
            }
        } else {
            GemmArgs gw{};
            gw.M = H; gw.N = kin; gw.K = B;
            gw.A = m->dz[cur]; gw.lda = H;
            gw.B = l == 0 ? m->xb : m->Hh[l - 1]; gw.ldb = l == 0 ? KX : H;
            gw.part = m->part[pk];
            gemm<true, true, EPI_PARTIAL>(m, gw, dim3((kin + BN - 1) / BN, H / BM, kSplits), s);
            // (the warp-specialised weight-gradient kernel also writes the
            // bias gradient's partials, one per split)
            k_colsum<<<dim3(H / 32, kSplits), 256, 0, s>>>(B, H, rows, m->dz[cur], m->bpart[pk]);
        }
        float *gb = gslot(m->b[l]);
        float *gW = gslot(m->W[l]);
        fork_adam(pk, adam_seg(m->W[l], m->part[pk], wparts, (size_t)H * pld, gW, pld),
                  adam_seg(m->b[l], m->bpart[pk], wparts, H, gb));
        cur ^= 1;
    }
    claim(0);
    claim(1);
}

int build_train_graph(e2d_mlp *m) {
    if (m->gexec) return E2D_OK;
    cudaGraph_t g = nullptr;
    cudaStream_t s = m->stream;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    k_step_update<<<1, 1, 0, s>>>(m->step_dev, (float)m->cfg.beta1, (float)m->cfg.beta2, m->bc_dev);
    // the gather reads the step from device memory through its seed argument
    k_gather<<<(m->B + 255) / 256, 256, 0, s>>>(m->B, NIN, KX, NOUT, m->cfg.seed, m->step_dev, m->nsamples, m->X,
                                                  m->T, m->xb, m->tb);
    forward(m, s, true);
    backward(m, s, m->lr_dev, false);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (e != cudaSuccess) { set_error(std::string("graph capture: ") + cudaGetErrorString(e)); return E2D_ERR_CUDA; }
    e = cudaGraphInstantiate(&m->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { m->gexec = nullptr; set_error(std::string("graph instantiate: ") + cudaGetErrorString(e)); return E2D_ERR_CUDA; }
    return E2D_OK;
}

}  // namespace

extern "C" {

int e2d_mlp_config_default(e2d_mlp_config *c) {
    if (!c) { set_error("null argument"); return E2D_ERR_ARG; }
    std::memset(c, 0, sizeof *c);
    c->nhidden = 5;
    c->lr = 1e-3;
    c->beta1 = 0.9;
    c->beta2 = 0.999;
    c->eps = 1e-8;
    c->batch = 65536;
    c->seed = 3;
    return E2D_OK;
}

int e2d_mlp_create(const e2d_mlp_config *cfg, e2d_mlp **out) {
    if (!cfg || !out) { set_error("null argument"); return E2D_ERR_ARG; }
    *out = nullptr;
    if (cfg->nhidden < 1 || cfg->nhidden > 16) { set_error("nhidden must be 1..16"); return E2D_ERR_ARG; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        set_error("no CUDA device: the MLP trains on the GPU only");
        return E2D_ERR_CUDA;
    }
    auto m = std::make_unique<e2d_mlp>();
    m->cfg = *cfg;
    m->nhidden = cfg->nhidden;
    CK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&m->ev_fork, cudaEventDisableTiming));
    for (cudaEvent_t &e : m->ev_done) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    // He-style initialisation from a fixed-seed generator
    uint64_t st = cfg->seed * 0x9e3779b97f4a7c15ULL + 12345;
    auto rnd = [&]() {
        st ^= st >> 12; st ^= st << 25; st ^= st >> 27;
        return ((st * 0x2545F4914F6CDD1DULL) >> 11) * (1.0 / 9007199254740992.0);
    };
    auto normal = [&]() {
        double u1 = rnd() + 1e-300, u2 = rnd();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    };
    for (int l = 0; l <= m->nhidden; l++) {
        const bool last = l == m->nhidden;
        const int rows = last ? NOUT : H, cols = l == 0 ? NIN : H;
        const int fan_in = l == 0 ? E2D_MLP_FEATURES : H;
        Tensor W{rows, cols}, b{rows, 1};
        std::vector<float> hw((size_t)rows * cols, 0.f), hb(rows, 0.f);
        const double sd = std::sqrt((last ? 1.0 : 2.0) / fan_in);
        for (int r = 0; r < rows; r++)
            for (int c = 0; c < cols; c++)
                hw[(size_t)r * cols + c] = (l == 0 && c >= E2D_MLP_FEATURES) ? 0.f : (float)(sd * normal());
        int rc;
        for (Tensor *t : {&W, &b}) {
            const size_t n = t->count();
            if ((rc = m->alloc(&t->w32, sizeof(float) * n))) return rc;
            if ((rc = m->alloc(&t->m, sizeof(float) * n))) return rc;
            if ((rc = m->alloc(&t->v, sizeof(float) * n))) return rc;
            if (!last && t == &W && (rc = m->alloc(&t->wbf, sizeof(bf16) * (size_t)t->rows * t->wld()))) return rc;
            if (!last && l > 0 && t == &W && (rc = m->alloc(&t->wbfT, sizeof(bf16) * n))) return rc;
        }
        CK(cudaMemcpy(W.w32, hw.data(), sizeof(float) * hw.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(b.w32, hb.data(), sizeof(float) * hb.size(), cudaMemcpyHostToDevice));
        if (W.wbf)
            k_to_bf16<<<(W.count() + 255) / 256, 256, 0, m->stream>>>(W.count(), W.w32, W.wbf, W.wbfT, W.rows,
                                                                       W.cols, W.wld());
        m->W.push_back(W);
        m->b.push_back(b);
    }
    int rc;
    if ((rc = m->alloc(&m->step_dev, sizeof(int)))) return rc;
    if ((rc = m->alloc(&m->flag_dev, sizeof(int)))) return rc;
    CK(cudaFuncSetAttribute(k_gemm_tc<false, false, EPI_BIAS_GELU>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            tc::SMEM));
    CK(cudaFuncSetAttribute(k_gemm_tc<false, true, EPI_GELU_BWD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            tc::SMEM));
    CK(cudaFuncSetAttribute(k_gemm_tc<true, true, EPI_PARTIAL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            tc::SMEM));
    if ((rc = m->alloc(&m->bc_dev, 2 * sizeof(float)))) return rc;
    if ((rc = m->alloc(&m->lr_dev, sizeof(float)))) return rc;
    const float lr0 = (float)cfg->lr;
    CK(cudaMemcpy(m->lr_dev, &lr0, sizeof(float), cudaMemcpyHostToDevice));
    if ((rc = m->alloc(&m->grad, sizeof(float) * param_count(m.get())))) return rc;
    CK(cudaStreamSynchronize(m->stream));
    *out = m.release();
    return E2D_OK;
}

void e2d_mlp_destroy(e2d_mlp *m) { delete m; }

int e2d_mlp_param_count(e2d_mlp *m, int64_t *n) {
    if (!m || !n) { set_error("null argument"); return E2D_ERR_ARG; }
    *n = (int64_t)param_count(m);
    return E2D_OK;
}

int e2d_mlp_get_params(e2d_mlp *m, float *out) {
    if (!m || !out) { set_error("null argument"); return E2D_ERR_ARG; }
    size_t off = 0;
    for (size_t l = 0; l < m->W.size(); l++)
        for (Tensor *t : {&m->W[l], &m->b[l]}) {
            CK(cudaMemcpy(out + off, t->w32, sizeof(float) * t->count(), cudaMemcpyDeviceToHost));
            off += t->count();
        }
    return E2D_OK;
}

int e2d_mlp_set_params(e2d_mlp *m, const float *in) {
    if (!m || !in) { set_error("null argument"); return E2D_ERR_ARG; }
    size_t off = 0;
    for (size_t l = 0; l < m->W.size(); l++)
        for (Tensor *t : {&m->W[l], &m->b[l]}) {
            CK(cudaMemcpy(t->w32, in + off, sizeof(float) * t->count(), cudaMemcpyHostToDevice));
            if (t->wbf)
                k_to_bf16<<<(t->count() + 255) / 256, 256, 0, m->stream>>>(t->count(), t->w32, t->wbf, t->wbfT,
                                                                            t->rows, t->cols, t->wld());
            off += t->count();
        }
    CK(cudaStreamSynchronize(m->stream));
    return E2D_OK;
}

int e2d_mlp_set_lr(e2d_mlp *m, double lr) {
    if (!m) { set_error("null argument"); return E2D_ERR_ARG; }
    if (!(lr >= 0.0 && lr < 1e30)) { set_error("lr must be finite and >= 0"); return E2D_ERR_ARG; }
    const float v = (float)lr;
    // ordered after the steps already queued on the training stream
    CK(cudaMemcpyAsync(m->lr_dev, &v, sizeof(float), cudaMemcpyHostToDevice, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    m->cfg.lr = lr;
    return E2D_OK;
}

int e2d_mlp_set_data(e2d_mlp *m, int64_t nsamples, const float *x, const float *t) {
    if (!m || !x || !t || nsamples < 1) { set_error("bad argument"); return E2D_ERR_ARG; }
    if (m->X) { cudaFree(m->X); m->X = nullptr; }
    if (m->T) { cudaFree(m->T); m->T = nullptr; }
    std::vector<bf16> xb((size_t)nsamples * NIN);
    for (size_t i = 0; i < xb.size(); i++) xb[i] = __float2bfloat16_rn(x[i]);
    CK(cudaMalloc((void **)&m->X, sizeof(bf16) * xb.size()));
    CK(cudaMalloc((void **)&m->T, sizeof(float) * (size_t)nsamples * NOUT));
    CK(cudaMemcpy(m->X, xb.data(), sizeof(bf16) * xb.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(m->T, t, sizeof(float) * (size_t)nsamples * NOUT, cudaMemcpyHostToDevice));
    m->nsamples = nsamples;
    if (m->gexec) { cudaGraphExecDestroy(m->gexec); m->gexec = nullptr; }
    return E2D_OK;
}

int e2d_mlp_train(e2d_mlp *m, int32_t steps, double *loss) {
    if (!m || steps < 1 || !m->X) { set_error("bad argument or no training data"); return E2D_ERR_ARG; }
    int rc = ensure_batch(m, m->cfg.batch);
    if (rc) return rc;
    if ((rc = build_train_graph(m))) return rc;
    const int nlp = m->B / 256;
    std::vector<double> lp(nlp);
    for (int k = 0; k < steps; k++) {
        CK(cudaGraphLaunch(m->gexec, m->stream));
        if (loss) {
            CK(cudaMemcpyAsync(lp.data(), m->loss_part, sizeof(double) * nlp, cudaMemcpyDeviceToHost, m->stream));
            CK(cudaStreamSynchronize(m->stream));
            double s = 0.0;
            for (double v : lp) s += v;
            loss[k] = s / ((double)m->B * NOUT);
        }
    }
    CK(cudaStreamSynchronize(m->stream));
    return check_flag(m);
}

int e2d_mlp_forward(e2d_mlp *m, int64_t n, const float *x, float *y) {
    if (!m || !x || !y || n < 1) { set_error("bad argument"); return E2D_ERR_ARG; }
    int rc = ensure_batch(m, m->cfg.batch);
    if (rc) return rc;
    std::vector<bf16> xb((size_t)m->B * KX, __float2bfloat16_rn(0.f));
    for (int64_t r0 = 0; r0 < n; r0 += m->B) {
        const int64_t cnt = std::min<int64_t>(m->B, n - r0);
        for (size_t r = 0; r < (size_t)m->B; r++)
            for (int c = 0; c < NIN; c++)
                xb[r * KX + c] = __float2bfloat16_rn(r < (size_t)cnt ? x[(size_t)(r0 + r) * NIN + c] : 0.f);
        CK(cudaMemcpyAsync(m->xb, xb.data(), sizeof(bf16) * xb.size(), cudaMemcpyHostToDevice, m->stream));
        forward(m, m->stream, false);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(y + (size_t)r0 * NOUT, m->y, sizeof(float) * cnt * NOUT, cudaMemcpyDeviceToHost, m->stream));
        CK(cudaStreamSynchronize(m->stream));
    }
    return check_flag(m);
}

int e2d_mlp_gradient(e2d_mlp *m, const float *x, const float *t, double *loss, float *grad) {
    if (!m || !x || !t || !grad) { set_error("bad argument"); return E2D_ERR_ARG; }
    int rc = ensure_batch(m, m->cfg.batch);
    if (rc) return rc;
    std::vector<bf16> xb((size_t)m->B * KX, __float2bfloat16_rn(0.f));
    for (size_t r = 0; r < (size_t)m->B; r++)
        for (int c = 0; c < NIN; c++) xb[r * KX + c] = __float2bfloat16_rn(x[r * NIN + c]);
    CK(cudaMemcpy(m->xb, xb.data(), sizeof(bf16) * xb.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(m->tb, t, sizeof(float) * (size_t)m->B * NOUT, cudaMemcpyHostToDevice));
    forward(m, m->stream, true);
    backward(m, m->stream, nullptr, true);
    CK(cudaGetLastError());
    const int nlp = m->B / 256;
    std::vector<double> lp(nlp);
    CK(cudaMemcpyAsync(lp.data(), m->loss_part, sizeof(double) * nlp, cudaMemcpyDeviceToHost, m->stream));
    CK(cudaMemcpyAsync(grad, m->grad, sizeof(float) * param_count(m), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    double s = 0.0;
    for (double v : lp) s += v;
    if (loss) *loss = s / ((double)m->B * NOUT);
    return check_flag(m);
}

int e2d_wall_distance(e2d_mesh *mesh, double wall_box, double *d) {
    if (!mesh || !d) { set_error("null argument"); return E2D_ERR_ARG; }
    int rc = build_topology(mesh, wall_box);
    if (rc) return rc;
    const MeshTopo &t = mesh->topo;
    std::vector<double4> seg;
    for (int e = 0; e < t.nedge; e++)
        if (t.elog[e] == 2)
            seg.push_back(make_double4(mesh->x[t.en1[e] - 1], mesh->y[t.en1[e] - 1], mesh->x[t.en2[e] - 1],
                                       mesh->y[t.en2[e] - 1]));
    const int n = mesh->ncell;
    if (seg.empty()) { for (int i = 0; i < n; i++) d[i] = 1e300; return E2D_OK; }
    struct Bufs {  // freed on every return path
        double *px = nullptr, *py = nullptr, *dd = nullptr;
        double4 *sg = nullptr;
        ~Bufs() { cudaFree(px); cudaFree(py); cudaFree(dd); cudaFree(sg); }
    } b;
    CK(cudaMalloc((void **)&b.px, sizeof(double) * n));
    CK(cudaMalloc((void **)&b.py, sizeof(double) * n));
    CK(cudaMalloc((void **)&b.dd, sizeof(double) * n));
    CK(cudaMalloc((void **)&b.sg, sizeof(double4) * seg.size()));
    CK(cudaMemcpy(b.px, t.cx.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b.py, t.cy.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b.sg, seg.data(), sizeof(double4) * seg.size(), cudaMemcpyHostToDevice));
    k_wall_distance<<<(n + 255) / 256, 256>>>(n, b.px, b.py, (int)seg.size(), b.sg, b.dd);
    CK(cudaGetLastError());
    CK(cudaMemcpy(d, b.dd, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return E2D_OK;
}

// Features per cell: x, y, log(d_wall + 1e-3), Mach, sin a, cos a, then for
// j = 0..7: sin(2 pi f_j . (x, y)), cos(2 pi f_j . (x, y)), f_j ~ N(0, sigma^2).
int e2d_mlp_features(e2d_mesh *mesh, double wall_box, double mach, double alpha_deg, uint64_t seed, double sigma,
                     float *out) {
    if (!mesh || !out) { set_error("null argument"); return E2D_ERR_ARG; }
    const int n = mesh->ncell;
    std::vector<double> d(n);
    int rc = e2d_wall_distance(mesh, wall_box, d.data());
    if (rc) return rc;
    uint64_t st = seed * 0x9e3779b97f4a7c15ULL + 777;
    auto rnd = [&]() {
        st ^= st >> 12; st ^= st << 25; st ^= st >> 27;
        return ((st * 0x2545F4914F6CDD1DULL) >> 11) * (1.0 / 9007199254740992.0);
    };
    double f[8][2];
    for (auto &fj : f)
        for (double &c : fj) {
            double u1 = rnd() + 1e-300, u2 = rnd();
            c = sigma * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
        }
    const double a = alpha_deg * 3.14159265358979 / 180.0, sa = std::sin(a), ca = std::cos(a);
    const MeshTopo &t = mesh->topo;
    for (int i = 0; i < n; i++) {
        float *o = out + (size_t)i * NIN;
        const double x = t.cx[i], y = t.cy[i];
        o[0] = (float)x; o[1] = (float)y; o[2] = (float)std::log(d[i] + 1e-3);
        o[3] = (float)mach; o[4] = (float)sa; o[5] = (float)ca;
        for (int j = 0; j < 8; j++) {
            const double ph = 6.283185307179586 * (f[j][0] * x + f[j][1] * y);
            o[6 + 2 * j] = (float)std::sin(ph);
            o[7 + 2 * j] = (float)std::cos(ph);
        }
        for (int k = E2D_MLP_FEATURES; k < NIN; k++) o[k] = 0.f;
    }
    return E2D_OK;
}

}  // extern "C"
