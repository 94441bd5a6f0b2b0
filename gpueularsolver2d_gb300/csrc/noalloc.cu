// noalloc.cu -- iterations of the FP64 solve path that allocate no memory.
//
// Who needs it: a caller that runs inside a host application which owns all
// device memory -- for example a plug-in whose host hands it pre-allocated
// buffers from its own pool and forbids it to call cudaMalloc / cudaFree, or
// code that runs while the host keeps allocation locked.  Such a caller can
// pass the mesh and the state it already holds, but cannot create a solver
// (e2d_solver_create allocates its own device arena).
//
// The working arrays one iteration needs besides its inputs and outputs (the
// second state buffer, face-side states, time steps, residuals, smoothing
// sweeps, residual partials and the control block) live in one file-scope
// device array of fixed size, E2D_NOALLOC_MAX_CELLS cells.  Every GPU that
// loads the library holds that array until the process exits.
#include <cmath>
#include <cstring>
#include <string>

#include "dev_types.h"
#include "internal.h"
#include "solver_internal.h"

namespace {

using e2d::Ctl;
using e2d::kDtNone;
using e2d::V2;
using e2d::V4;

// Bytes per cell of the FP64 working arrays: W[1] 32, FS 96, dt 8, res 32,
// two smoothing sweeps 64; plus per-block partials and the control block.
constexpr size_t kPerCell = 32 + 96 + 8 + 32 + 64;
constexpr size_t kBlock = 128;
constexpr size_t kScratchBytes =
    kPerCell * E2D_NOALLOC_MAX_CELLS + 256 * (2 + E2D_NOALLOC_MAX_CELLS / kBlock);

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
static unsigned char *g_scratch_addr[kMaxDevices];  // device address of g_scratch per device

// Fresh control block for one call: nothing carries over from the last call.
__global__ void k_noalloc_ctl(Ctl *ctl, int target, double epsm) {
    ctl->step = 0;
    ctl->halt = 0;
    ctl->target = target;
    ctl->check_epsl = 0;
    ctl->nbad = 0;
    ctl->fixed_norm = epsm > 0.0;
    ctl->epsl = 0.0;
    ctl->epsm = epsm > 0.0 ? epsm : 0.0;
    ctl->resd = 100.0;
    ctl->freeze_after = 0;
    ctl->frozen = 0;
    ctl->freeze_resd = 0.0;
    for (int k = 0; k < 8; k++) ctl->dtmin[k] = kDtNone;
    ctl->fold_count = 0;
}

// Every face code of the caller's topology must name a cell of this mesh (or
// be -1 / -2) before any pass gathers through it: a code out of range sets
// halt = 3, which makes every later kernel of the call return at once.
__global__ void k_noalloc_check(int n, const int4 *__restrict__ topo, Ctl *ctl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 t = topo[i];
    bool bad = t.w < 0 || t.w > 3;
    const int code[3] = {t.x, t.y, t.z};
    for (int k = 0; k < 3; k++) {
        const int c = code[k];
        if (c >= 0) bad = bad || (c >> 3) >= n || (c & 3) > 2;
        else bad = bad || (c != -1 && c != -2);
    }
    if (bad) ctl->halt = 3;
}

size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" int e2d_step_noalloc(int32_t ncell, const int32_t *topo, const double *S, const double *R,
                                const double *area, const e2d_params *p, int32_t iterations, double *w,
                                double *resid, double *epsm, void *stream) {
    if (ncell < 1 || !topo || !S || !R || !area || !p || !w || !resid || !epsm || iterations < 1) {
        e2d::set_error("e2d_step_noalloc: bad argument");
        return E2D_ERR_ARG;
    }
    if (ncell > E2D_NOALLOC_MAX_CELLS) {
        e2d::set_error("e2d_step_noalloc: " + std::to_string(ncell) + " cells exceed the fixed scratch of " +
                       std::to_string(E2D_NOALLOC_MAX_CELLS) + " cells");
        return E2D_ERR_CAPACITY;
    }
    if (const char *why = e2d::param_error(p)) {
        e2d::set_error(std::string("e2d_step_noalloc: invalid parameters: ") + why);
        return E2D_ERR_ARG;
    }
    // options this entry point does not carry: refused rather than ignored, so
    // that a call never silently computes something other than e2d_step
    if (p->precision != E2D_FP64) {
        e2d::set_error("e2d_step_noalloc: only precision E2D_FP64 is supported");
        return E2D_ERR_ARG;
    }
    if (p->limiter_freeze > 0 || p->limiter_freeze_resd > 0.0) {
        e2d::set_error("e2d_step_noalloc: limiter_freeze and limiter_freeze_resd are not supported (must be 0)");
        return E2D_ERR_ARG;
    }
    if (((uintptr_t)topo | (uintptr_t)S | (uintptr_t)R) % 16 || (uintptr_t)w % 32 || (uintptr_t)area % 8 ||
        (uintptr_t)resid % 8) {
        e2d::set_error("e2d_step_noalloc: topo, S and R must be 16-byte aligned, w 32-byte aligned, "
                       "area and resid 8-byte aligned");
        return E2D_ERR_ARG;
    }
    // an error left pending by earlier work belongs to its caller: report it
    // without clearing it, and do not take it for one of this call's launches
    if (cudaError_t pending = cudaPeekAtLastError()) {
        e2d::set_error(std::string("e2d_step_noalloc: a CUDA error was pending before the call: ") +
                       cudaGetErrorString(pending));
        return E2D_ERR_CUDA;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        e2d::set_error("e2d_step_noalloc: no usable CUDA device");
        return E2D_ERR_CUDA;
    }
    // set-up once per device, with that device current: the host cannot use
    // g_scratch itself as a device address
    if (!g_scratch_addr[dev]) {
        void *a = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&a, g_scratch);
        if (e != cudaSuccess || !a) {
            e2d::set_error(std::string("e2d_step_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return E2D_ERR_CUDA;
        }
        g_scratch_addr[dev] = (unsigned char *)a;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int n = ncell;
    const int block = (int)kBlock;
    const int G = (n + block - 1) / block;
    unsigned char *base = g_scratch_addr[dev];
    size_t off = 0;
    auto take = [&](size_t b) { unsigned char *q = base + off; off += up256(b); return q; };
    e2d::Plan<double> plan;
    std::memset(&plan, 0, sizeof plan);
    plan.ctl = (Ctl *)take(sizeof(Ctl));
    plan.W[1] = (V4<double> *)take(sizeof(V4<double>) * n);
    plan.FS = (V4<double> *)take(sizeof(V4<double>) * 3 * n);
    plan.dt = (double *)take(sizeof(double) * n);
    plan.res = (V4<double> *)take(sizeof(V4<double>) * n);
    plan.sm[0] = (V4<double> *)take(sizeof(V4<double>) * n);
    plan.sm[1] = (V4<double> *)take(sizeof(V4<double>) * n);
    plan.part = (double *)take(sizeof(double) * G);
    plan.W[0] = (V4<double> *)w;
    plan.m = e2d::MeshDev<double>{n, (const int4 *)topo, (const V2<double> *)S, (const V2<double> *)R, area};
    // free-stream constants exactly as Initialization computes them (gpu_init.cu:63-93)
    const double kR = 287.06, kPi = 3.14159265358979, g = p->gamma;
    const double alpha = p->alpha_deg * kPi / 180.0, ain = std::sqrt(g * kR * p->tin), vin = p->ma * ain;
    const double U = std::cos(alpha) / 1.0, V = std::sin(alpha) / 1.0;
    const double rho_e = kR * p->tin / (vin * vin) / (g - 1.0) + 0.50;
    const double E = rho_e / 1.0 - 0.5 * (U * U + V * V);
    e2d::Flow<double> &f = plan.f;
    f.gamma = g; f.ui = std::cos(alpha); f.vi = std::sin(alpha); f.ain = p->far_field_fix ? 1.0 / p->ma : ain; f.tin = p->tin; f.vin = vin;
    f.R = kR; f.pis = (g - 1.0) * 1.0 * E; f.cfl = p->cfl; f.dt_cap = p->dt_cap;
    f.eps_entropy = p->entropy_eps; f.irs_eps = p->irs_eps;
    f.venk_k3 = p->limiter_k * p->limiter_k * p->limiter_k; f.limiter = p->limiter;
    f.global_dt = p->global_dt;
    f.first_order = p->first_order_iters; f.positivity = p->positivity_fix;
    plan.hist = resid;
    plan.hist_cap = iterations;
    plan.stages = p->rk_stages;
    for (int k = 0; k < 8; k++) plan.rk[k] = p->rk_coef[k];
    plan.sweeps = p->irs_sweeps;
    plan.block = block;
    k_noalloc_ctl<<<1, 1, 0, s>>>(plan.ctl, iterations, *epsm);
    k_noalloc_check<<<G, block, 0, s>>>(n, plan.m.topo, plan.ctl);
    for (int it = 0; it < iterations; it++) e2d::enqueue_iteration<double>(plan, s);
    cudaError_t e = cudaGetLastError();
    Ctl c;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&c, plan.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        e2d::set_error(std::string("e2d_step_noalloc: ") + cudaGetErrorString(e));
        return E2D_ERR_CUDA;
    }
    if (c.halt == 3) {
        e2d::set_error("e2d_step_noalloc: topo holds a face code out of range (a neighbour outside [0, ncell), "
                       "a slot above 2, a negative code other than -1 / -2, or a neighbour count outside 0..3); "
                       "nothing was computed");
        return E2D_ERR_ARG;
    }
    *epsm = c.epsm;
    if (c.halt == 2) {
        e2d::set_error("e2d_step_noalloc: non-positive density or pressure (or NaN)");
        return E2D_ERR_DIVERGED;
    }
    return E2D_OK;
}
