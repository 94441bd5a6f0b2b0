// solver.cu -- the single-case solver behind the C ABI: set-up of the
// cell-local device layout, device arena, CUDA-graph iteration batches and
// the solve / state / residual-history entry points.
//
// Replaces ROE_SOLVER (gpu_solver.cu:2171-2473) and the memory helpers it
// calls (cpuMalloc / gpuMalloc / struct2Array / copyH2D / copyD2H,
// gpu_solver.cu:1505-1630, 1908-2169).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "dev_types.h"
#include "solver_internal.h"

using namespace e2d;

#define CK(call)                                                                       \
    do {                                                                               \
        cudaError_t err_ = (call);                                                     \
        if (err_ != cudaSuccess) {                                                     \
            set_error(std::string("CUDA: ") + #call + ": " + cudaGetErrorString(err_)); \
            return E2D_ERR_CUDA;                                                       \
        }                                                                              \
    } while (0)

namespace e2d {

// gpu_fvm.cu:8-9
static const double kR = 287.06;
static const double kPi = 3.14159265358979;

FreeStream free_stream(const e2d_params &p) {
    FreeStream s;
    const double g = p.gamma;
    s.alpha = p.alpha_deg * kPi / 180.0;
    s.ain = std::sqrt(g * kR * p.tin);
    s.vin = p.ma * s.ain;
    // gpu_solver.cu:79 compares the non-dimensional normal velocity with the
    // dimensional AIN, so its supersonic branch never runs; the fix compares
    // it with the non-dimensional free-stream sound speed 1/M.
    s.ain_test = p.far_field_fix ? 1.0 / p.ma : s.ain;
    s.ui = std::cos(s.alpha);
    s.vi = std::sin(s.alpha);
    s.rho_e = kR * p.tin / (s.vin * s.vin) / (g - 1.0) + 0.50;
    // CalculationPTA of (1, cos a, sin a, rho_e)
    double d = 1.0, du = std::cos(s.alpha), dv = std::sin(s.alpha), de = s.rho_e;
    double U = du / d, V = dv / d;
    double E = de / d - 0.5 * (U * U + V * V);
    s.pis = (g - 1.0) * d * E;
    return s;
}

int build_layout(e2d_mesh *m, const e2d_params &p, HostLayout &L) {
    int rc = build_topology(m, p.wall_box);
    if (rc) return rc;
    const MeshTopo &t = m->topo;
    const int n = m->ncell;
    if ((int64_t)n >= (1 << 28)) { set_error("mesh too large (limit 2^28 cells)"); return E2D_ERR_CAPACITY; }
    L.n = n;
    cell_order(m, p.ordering, L.perm);
    L.iperm.assign(n, 0);
    for (int i = 0; i < n; i++) L.iperm[L.perm[i]] = i;
    L.topo.assign(4 * (size_t)n, 0);
    L.S.assign(6 * (size_t)n, 0.0);
    L.R.assign(6 * (size_t)n, 0.0);
    L.area.assign(n, 0.0);
    const double *X = m->x.data() - 1, *Y = m->y.data() - 1;
    for (int i = 0; i < n; i++) {
        const int c = L.perm[i];
        for (int k = 0; k < 3; k++) {
            const int cf = 3 * c + k;
            const int nb = t.nb[cf];
            L.topo[4 * (size_t)i + k] = nb >= 0 ? (L.iperm[nb] << 3) | (t.is_right[cf] << 2) | t.nb_slot[cf] : nb;
            if (nb == -2) { L.wall_cell.push_back(i); L.wall_k.push_back(k); }
            const int N1 = m->tri[3 * (size_t)c + (k + 1) % 3], N2 = m->tri[3 * (size_t)c + (k + 2) % 3];
            const double vectorx = X[N1] - X[N2], vectory = Y[N2] - Y[N1];
            L.S[2 * ((size_t)k * n + i)] = vectory;
            L.S[2 * ((size_t)k * n + i) + 1] = vectorx;
            const int e = t.celledge[cf] - 1;
            L.R[2 * ((size_t)k * n + i)] = t.emx[e] - t.cx[c];
            L.R[2 * ((size_t)k * n + i) + 1] = t.emy[e] - t.cy[c];
        }
        L.topo[4 * (size_t)i + 3] = t.clog[c];
        L.area[i] = t.area[c];
    }
    return E2D_OK;
}

void forces_from_state(const HostLayout &L, const FreeStream &fs, double gamma, const double *w,
                       double *cl, double *cd) {
    double fx = 0.0, fy = 0.0;
    const int n = L.n;
    for (size_t q = 0; q < L.wall_cell.size(); q++) {
        const int i = L.wall_cell[q], k = L.wall_k[q];
        const double *u = &w[4 * (size_t)L.perm[i]];
        const double p = (gamma - 1.0) * (u[3] - 0.5 * (u[1] * u[1] + u[2] * u[2]) / u[0]);
        fx += (p - fs.pis) * L.S[2 * ((size_t)k * n + i)];
        fy += (p - fs.pis) * L.S[2 * ((size_t)k * n + i) + 1];
    }
    const double ca = std::cos(fs.alpha), sa = std::sin(fs.alpha);
    if (cd) *cd = (fx * ca + fy * sa) / 0.5;
    if (cl) *cl = (-fx * sa + fy * ca) / 0.5;
}

bool freezes(const e2d_params &p) { return p.limiter_freeze > 0 || p.limiter_freeze_resd > 0.0; }

// The topology array (16 bytes per cell) is read by all four passes of every
// stage; keeping it in L2 across them cut an iteration on 4.2M cells from 1.392
// to 1.357 ms.  The persisting carve-out is a limit of this process's context:
// it is raised while a solver or batch that uses it exists, and when the last
// one is destroyed its persisting lines are released and the limit put back
// (otherwise later work in the process runs with less L2).
namespace {
std::mutex l2_mu;
int l2_users = 0;
bool l2_raised = false;
size_t l2_prev = 0;
}  // namespace

void release_l2(bool *held) {
    if (!held || !*held) return;
    *held = false;
    std::lock_guard<std::mutex> lk(l2_mu);
    if (--l2_users > 0) return;
    cudaCtxResetPersistingL2Cache();
    if (l2_raised) cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, l2_prev);
    l2_raised = false;
    cudaGetLastError();
}

void keep_in_l2(cudaGraph_t g, const void *base, size_t bytes, bool *held) {
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess ||
        prop.persistingL2CacheMaxSize <= 0 || prop.accessPolicyMaxWindowSize <= 0) {
        cudaGetLastError();
        return;
    }
    const size_t win = std::min<size_t>(bytes, (size_t)prop.accessPolicyMaxWindowSize);
    const size_t keep = std::min<size_t>(win, (size_t)prop.persistingL2CacheMaxSize);
    {
        std::lock_guard<std::mutex> lk(l2_mu);
        if (!*held) {
            *held = true;
            l2_users++;
        }
        size_t cur = 0;
        if (cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize) == cudaSuccess && cur < keep) {
            if (!l2_raised) {
                l2_prev = cur;
                l2_raised = true;
            }
            cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, keep);
        }
    }
    cudaKernelNodeAttrValue v = {};
    v.accessPolicyWindow.base_ptr = const_cast<void *>(base);
    v.accessPolicyWindow.num_bytes = win;
    v.accessPolicyWindow.hitRatio = win ? (float)keep / (float)win : 0.f;
    v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    size_t nn = 0;
    cudaGraphGetNodes(g, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    cudaGraphGetNodes(g, nodes.data(), &nn);
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
            cudaGraphKernelNodeSetAttribute(nd, cudaKernelNodeAttributeAccessPolicyWindow, &v);
    }
    cudaGetLastError();  // a GPU without the feature keeps the default policy
}

// Null when the parameters are usable, else which one is not.
const char *param_error(const e2d_params *p) {
    if (!(p->gamma > 1.0)) return "gamma must be > 1";
    if (!(p->ma > 0.0)) return "ma must be > 0";
    if (!(p->tin > 0.0)) return "tin must be > 0";
    if (!(p->cfl > 0.0)) return "cfl must be > 0";
    if (std::isnan(p->epsl)) return "epsl must not be NaN";
    if (p->maxstep < 0) return "maxstep must be >= 0";
    if (p->rk_stages < 1 || p->rk_stages > 8) return "rk_stages must be 1..8";
    for (int k = 0; k < p->rk_stages; k++)
        if (!std::isfinite(p->rk_coef[k])) return "rk_coef must be finite";
    if (p->irs_sweeps < 0 || p->irs_sweeps > 16) return "irs_sweeps must be 0..16";
    if (!(p->irs_eps >= 0.0) || !std::isfinite(p->irs_eps)) return "irs_eps must be finite and >= 0";
    if (!(p->dt_cap > 0.0)) return "dt_cap must be > 0";
    if (!(p->entropy_eps > 0.0)) return "entropy_eps must be > 0";
    if (!(p->wall_box > 0.0)) return "wall_box must be > 0";
    if (p->precision != E2D_FP64 && p->precision != E2D_FP32) return "precision must be E2D_FP64 or E2D_FP32";
    if (p->ordering != E2D_ORDER_FILE && p->ordering != E2D_ORDER_MORTON && p->ordering != E2D_ORDER_RCM)
        return "ordering must be E2D_ORDER_FILE, _MORTON or _RCM";
    if (p->block_size != 0 && (p->block_size < 32 || p->block_size > 256 || p->block_size % 32))
        return "block_size must be 0 or a multiple of 32 in 32..256";
    if (p->graph_iters < 0 || p->graph_iters > 256) return "graph_iters must be 0..256";
    if (p->limiter_freeze < 0) return "limiter_freeze must be >= 0";
    if (p->limiter < E2D_LIMITER_REFERENCE || p->limiter > E2D_LIMITER_CELL_VENKAT)
        return "limiter must be E2D_LIMITER_REFERENCE, _VENKAT, _CELL_BARTH or _CELL_VENKAT";
    if ((p->limiter == E2D_LIMITER_VENKAT || p->limiter == E2D_LIMITER_CELL_VENKAT) && !(p->limiter_k > 0.0))
        return "limiter_k must be > 0";
    if (p->global_dt != 0 && p->global_dt != 1) return "global_dt must be 0 or 1";
    if (p->far_field_fix != 0 && p->far_field_fix != 1) return "far_field_fix must be 0 or 1";
    if (p->first_order_iters < 0) return "first_order_iters must be >= 0";
    if (p->positivity_fix != 0 && p->positivity_fix != 1) return "positivity_fix must be 0 or 1";
    return nullptr;
}

struct SolverBase {
    virtual ~SolverBase() {}
    virtual int upload_state(const double *w_file) = 0;
    virtual int download_state(double *w_file) = 0;
    virtual int enqueue(cudaStream_t s) = 0;
    virtual int launches() const = 0;
    virtual int nblocks() const = 0;
    virtual int enqueue_timed(cudaStream_t s, cudaEvent_t *ev, int *kind) = 0;
    virtual const void *topo_ptr() const = 0;
};

template <typename T> struct SolverT : SolverBase {
    HostLayout *L;
    Arena arena;
    Plan<T> plan;
    int *perm_dev = nullptr;       // [n] internal -> file
    double *wfile_dev = nullptr;   // [4n] FP64 state in file order (exchange buffer)
    cudaStream_t *stream = nullptr;

    explicit SolverT(HostLayout *l) : L(l) {}

    int init(const e2d_params &p, const FreeStream &fs, Ctl *ctl, int block) {
        const int n = L->n;
        const int G = (n + block - 1) / block;
        size_t bytes = Arena::up(sizeof(int4) * n) + 2 * Arena::up(sizeof(V2<T>) * 3 * n) +
                       Arena::up(sizeof(T) * n) * 2 + Arena::up(sizeof(V4<T>) * n) * 5 +
                       Arena::up(sizeof(V4<T>) * 3 * n) * (freezes(p) ? 2 : 1) +
                       Arena::up(sizeof(double) * G) +
                       Arena::up(sizeof(int) * n) + Arena::up(sizeof(double) * 4 * n);
        CK(cudaMalloc((void **)&arena.base, bytes));
        arena.cap = bytes;
        int4 *topo = (int4 *)arena.take(sizeof(int4) * n);
        V2<T> *S = (V2<T> *)arena.take(sizeof(V2<T>) * 3 * n);
        V2<T> *R = (V2<T> *)arena.take(sizeof(V2<T>) * 3 * n);
        T *area = (T *)arena.take(sizeof(T) * n);
        plan.W[0] = (V4<T> *)arena.take(sizeof(V4<T>) * n);
        plan.W[1] = (V4<T> *)arena.take(sizeof(V4<T>) * n);
        plan.FS = (V4<T> *)arena.take(sizeof(V4<T>) * 3 * n);
        plan.phi = freezes(p) ? (V4<T> *)arena.take(sizeof(V4<T>) * 3 * n) : nullptr;
        plan.dt = (T *)arena.take(sizeof(T) * n);
        plan.res = (V4<T> *)arena.take(sizeof(V4<T>) * n);
        plan.sm[0] = (V4<T> *)arena.take(sizeof(V4<T>) * n);
        plan.sm[1] = (V4<T> *)arena.take(sizeof(V4<T>) * n);
        plan.part = (double *)arena.take(sizeof(double) * G);
        perm_dev = (int *)arena.take(sizeof(int) * n);
        wfile_dev = (double *)arena.take(sizeof(double) * 4 * n);
        CK(cudaMemcpy(perm_dev, L->perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(topo, L->topo.data(), sizeof(int4) * n, cudaMemcpyHostToDevice));
        std::vector<T> tmp(6 * (size_t)n);
        for (size_t k = 0; k < tmp.size(); k++) tmp[k] = (T)L->S[k];
        CK(cudaMemcpy(S, tmp.data(), sizeof(T) * tmp.size(), cudaMemcpyHostToDevice));
        for (size_t k = 0; k < tmp.size(); k++) tmp[k] = (T)L->R[k];
        CK(cudaMemcpy(R, tmp.data(), sizeof(T) * tmp.size(), cudaMemcpyHostToDevice));
        for (int k = 0; k < n; k++) tmp[k] = (T)L->area[k];
        CK(cudaMemcpy(area, tmp.data(), sizeof(T) * n, cudaMemcpyHostToDevice));
        CK(cudaMemset(plan.W[1], 0, sizeof(V4<T>) * n));
        CK(cudaMemset(plan.part, 0, sizeof(double) * G));
        plan.m = MeshDev<T>{n, topo, S, R, area};
        Flow<T> &f = plan.f;
        f.gamma = (T)p.gamma; f.ui = (T)fs.ui; f.vi = (T)fs.vi; f.ain = (T)fs.ain_test; f.tin = (T)p.tin;
        f.vin = (T)fs.vin; f.R = (T)kR; f.pis = (T)fs.pis; f.cfl = (T)p.cfl; f.dt_cap = (T)p.dt_cap;
        f.eps_entropy = (T)p.entropy_eps; f.irs_eps = (T)p.irs_eps;
        f.venk_k3 = (T)(p.limiter_k * p.limiter_k * p.limiter_k); f.limiter = p.limiter;
        f.global_dt = p.global_dt;
        f.first_order = p.first_order_iters; f.positivity = p.positivity_fix;
        plan.ctl = ctl;
        plan.hist = nullptr;
        plan.hist_cap = 0;
        plan.stages = p.rk_stages;
        for (int k = 0; k < 8; k++) plan.rk[k] = (T)p.rk_coef[k];
        plan.sweeps = p.irs_sweeps;
        plan.block = block;
        return E2D_OK;
    }

    // Caller's FP64 file-order buffer -> device (one copy; from pinned memory
    // it runs at full PCIe/C2C speed), then a permute-and-convert kernel.
    int upload_state(const double *w) override {
        const int n = L->n;
        CK(cudaMemcpyAsync(wfile_dev, w, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, *stream));
        enqueue_import<T>(n, perm_dev, wfile_dev, plan.W[0], *stream);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(*stream));
        return E2D_OK;
    }

    int download_state(double *w) override {
        const int n = L->n;
        enqueue_export<T>(n, perm_dev, plan.W[0], wfile_dev, *stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(w, wfile_dev, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, *stream));
        CK(cudaStreamSynchronize(*stream));
        return E2D_OK;
    }

    int enqueue_timed(cudaStream_t s, cudaEvent_t *ev, int *kind) override {
        return enqueue_iteration_timed<T>(plan, s, ev, kind);
    }

    int enqueue(cudaStream_t s) override {
        enqueue_iteration<T>(plan, s);
        CK(cudaGetLastError());
        return E2D_OK;
    }

    int launches() const override { return launches_per_iteration(plan); }
    const void *topo_ptr() const override { return plan.m.topo; }
    int nblocks() const override { return (L->n + plan.block - 1) / plan.block; }
};

}  // namespace e2d

struct e2d_solver {
    e2d_params prm;
    HostLayout L;
    FreeStream fs;
    std::unique_ptr<SolverBase> impl;
    Ctl *ctl_dev = nullptr;
    Ctl *ctl_host = nullptr;  // pinned mirror
    double *hist_dev = nullptr;
    int hist_cap = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaGraphExec_t gexec = nullptr;   // graph_iters iterations
    cudaGraphExec_t gexec1 = nullptr;  // one iteration (remainders, short runs)
    int graph_iters = 8;
    int block = 128;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0.0;
    std::vector<double> hist;  // host copy of Resd[1..step]
    bool l2_held = false;      // counted among the users of the persisting L2 carve-out

    ~e2d_solver() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (gexec1) cudaGraphExecDestroy(gexec1);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (own_stream && stream) cudaStreamSynchronize(stream);
        release_l2(&l2_held);
        if (own_stream && stream) cudaStreamDestroy(stream);
        if (ctl_dev) cudaFree(ctl_dev);
        if (ctl_host) cudaFreeHost(ctl_host);
        if (hist_dev) cudaFree(hist_dev);
    }
};

namespace {

int push_ctl(e2d_solver *s) {
    CK(cudaMemcpyAsync(s->ctl_dev, s->ctl_host, sizeof(Ctl), cudaMemcpyHostToDevice, s->stream));
    return E2D_OK;
}

int pull_ctl(e2d_solver *s) {
    CK(cudaMemcpyAsync(s->ctl_host, s->ctl_dev, sizeof(Ctl), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return E2D_OK;
}

void drop_graphs(e2d_solver *s) {
    if (s->gexec) { cudaGraphExecDestroy(s->gexec); s->gexec = nullptr; }
    if (s->gexec1) { cudaGraphExecDestroy(s->gexec1); s->gexec1 = nullptr; }
}

// The history buffer lives behind a pointer captured in the graph, so it is
// sized once per growth and the graph is rebuilt when it moves.
int ensure_hist(e2d_solver *s, int need) {
    if (need <= s->hist_cap) return E2D_OK;
    int cap = std::max(need, std::max(1024, 2 * s->hist_cap));
    double *nh = nullptr;
    CK(cudaMalloc((void **)&nh, sizeof(double) * cap));
    if (s->hist_dev) {
        CK(cudaMemcpyAsync(nh, s->hist_dev, sizeof(double) * s->hist_cap, cudaMemcpyDeviceToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        cudaFree(s->hist_dev);
    }
    s->hist_dev = nh;
    s->hist_cap = cap;
    drop_graphs(s);
    return E2D_OK;
}

template <typename T> void set_hist(SolverBase *b, double *h, int cap) {
    auto *t = static_cast<SolverT<T> *>(b);
    t->plan.hist = h;
    t->plan.hist_cap = cap;
}

// One CUDA graph of `iters` iterations on the solver's stream.
int capture(e2d_solver *s, int iters, cudaGraphExec_t *out) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int rc = E2D_OK;
    for (int it = 0; it < iters && rc == E2D_OK; it++) rc = s->impl->enqueue(s->stream);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) { set_error(std::string("graph capture: ") + cudaGetErrorString(e)); return E2D_ERR_CUDA; }
    keep_in_l2(g, s->impl->topo_ptr(), sizeof(int4) * (size_t)s->L.n, &s->l2_held);
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { *out = nullptr; set_error(std::string("graph instantiate: ") + cudaGetErrorString(e)); return E2D_ERR_CUDA; }
    return E2D_OK;
}

int build_graph(e2d_solver *s) {
    if (s->gexec && s->gexec1) return E2D_OK;
    if (s->prm.precision == E2D_FP64) set_hist<double>(s->impl.get(), s->hist_dev, s->hist_cap);
    else set_hist<float>(s->impl.get(), s->hist_dev, s->hist_cap);
    drop_graphs(s);
    int rc = capture(s, s->graph_iters, &s->gexec);
    if (rc == E2D_OK) rc = capture(s, 1, &s->gexec1);
    return rc;
}

// A stencil of the requested precision over the solver's mesh layout, bound
// to the solver's stream and control block (its state is not set).
int make_impl(e2d_solver *s, const e2d_params &p, std::unique_ptr<SolverBase> &out) {
    if (p.precision == E2D_FP64) {
        auto *t = new SolverT<double>(&s->L);
        t->stream = &s->stream;
        out.reset(t);
        return t->init(p, s->fs, s->ctl_dev, s->block);
    }
    auto *t = new SolverT<float>(&s->L);
    t->stream = &s->stream;
    out.reset(t);
    return t->init(p, s->fs, s->ctl_dev, s->block);
}

// Copies the residuals of iterations completed since the last call into the
// host history; with verbose set, prints them as the reference does
// ("%d,%1.20lf", gpu_solver.cu:2433).  The stream must be synchronised.
int sync_hist(e2d_solver *s) {
    const int step = s->ctl_host->step;
    const int have = (int)s->hist.size();
    if (step <= have) return E2D_OK;
    s->hist.resize(step);
    CK(cudaMemcpy(s->hist.data() + have, s->hist_dev + have, sizeof(double) * (step - have),
                  cudaMemcpyDeviceToHost));
    if (s->prm.verbose) {
        for (int k = have; k < step; k++) std::printf("%d,%1.20lf\n", k + 1, s->hist[k]);
        std::fflush(stdout);
    }
    return E2D_OK;
}

// Runs up to n iterations (fewer if the residual test stops the loop).
int run(e2d_solver *s, int n, bool check, double epsl, int poll_every) {
    if (n <= 0) return E2D_OK;
    int rc = ensure_hist(s, s->ctl_host->step + n);
    if (rc) return rc;
    if ((rc = build_graph(s))) return rc;
    Ctl &c = *s->ctl_host;
    c.halt = 0;
    c.nbad = 0;
    c.target = c.step + n;
    c.check_epsl = check ? 1 : 0;
    c.epsl = epsl;
    if ((rc = push_ctl(s))) return rc;
    // whole graphs of graph_iters iterations, then single-iteration graphs for
    // the remainder (no launches of iterations that would only find the halt flag)
    const int full = n / s->graph_iters, rem = n % s->graph_iters;
    CK(cudaEventRecord(s->ev0, s->stream));
    for (int k = 0; k < full; k++) {
        CK(cudaGraphLaunch(s->gexec, s->stream));
        if (check && poll_every > 0 && (k + 1) % poll_every == 0 && (k + 1 < full || rem)) {
            if ((rc = pull_ctl(s))) return rc;
            if ((rc = sync_hist(s))) return rc;
            if (c.halt) break;
        }
    }
    for (int k = 0; k < rem && !c.halt; k++) CK(cudaGraphLaunch(s->gexec1, s->stream));
    CK(cudaEventRecord(s->ev1, s->stream));
    if ((rc = pull_ctl(s))) return rc;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    s->last_ms = ms;
    if ((rc = sync_hist(s))) return rc;
    if (c.halt == 2) {
        set_error("solution diverged: non-positive density or pressure (or NaN) at step " + std::to_string(c.step));
        return E2D_ERR_DIVERGED;
    }
    return E2D_OK;
}

}  // namespace

extern "C" {

int e2d_solver_create(e2d_mesh *m, const e2d_params *p, e2d_solver **out) {
    if (!m || !p || !out) { set_error("null argument"); return E2D_ERR_ARG; }
    *out = nullptr;
    if (const char *why = param_error(p)) { set_error(std::string("invalid parameters: ") + why); return E2D_ERR_ARG; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        set_error("no CUDA device: the solver runs on the GPU only");
        return E2D_ERR_CUDA;
    }
    auto s = std::make_unique<e2d_solver>();
    s->prm = *p;
    int rc = build_layout(m, *p, s->L);
    if (rc) return rc;
    s->fs = free_stream(*p);
    CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    s->own_stream = true;
    CK(cudaEventCreate(&s->ev0));
    CK(cudaEventCreate(&s->ev1));
    CK(cudaMalloc((void **)&s->ctl_dev, sizeof(Ctl)));
    CK(cudaMallocHost((void **)&s->ctl_host, sizeof(Ctl)));
    std::memset(s->ctl_host, 0, sizeof(Ctl));
    s->ctl_host->resd = 100.0;  // gpu_solver.cu:2185 Resd[0]=100
    s->ctl_host->freeze_after = p->limiter_freeze > 0 ? p->limiter_freeze : 0;
    s->ctl_host->freeze_resd = p->limiter_freeze_resd > 0.0 ? p->limiter_freeze_resd : 0.0;
    for (auto &d : s->ctl_host->dtmin) d = kDtNone;
    CK(cudaMemcpy(s->ctl_dev, s->ctl_host, sizeof(Ctl), cudaMemcpyHostToDevice));
    s->graph_iters = p->graph_iters > 0 ? p->graph_iters : 8;
    s->block = p->block_size > 0 ? p->block_size : 128;
    if ((rc = make_impl(s.get(), *p, s->impl))) return rc;
    // free-stream state (gpu_init.cu:79-86)
    std::vector<double> w0(4 * (size_t)s->L.n);
    for (int i = 0; i < s->L.n; i++) {
        w0[4 * (size_t)i] = 1.0; w0[4 * (size_t)i + 1] = std::cos(s->fs.alpha);
        w0[4 * (size_t)i + 2] = std::sin(s->fs.alpha); w0[4 * (size_t)i + 3] = s->fs.rho_e;
    }
    if ((rc = s->impl->upload_state(w0.data()))) return rc;
    if ((rc = ensure_hist(s.get(), std::max(1024, p->maxstep > 0 ? p->maxstep : 0)))) return rc;
    *out = s.release();
    return E2D_OK;
}

void e2d_solver_destroy(e2d_solver *s) { delete s; }

int e2d_step(e2d_solver *s, int32_t n) {
    if (!s || n < 0) { set_error("bad argument"); return E2D_ERR_ARG; }
    return run(s, n, false, 0.0, 0);
}

int e2d_solve(e2d_solver *s, int32_t max_steps, double epsl, double *resid_history, int32_t *nsteps) {
    if (!s || max_steps < 0 || std::isnan(epsl)) { set_error("bad argument"); return E2D_ERR_ARG; }
    const int step0 = s->ctl_host->step;
    int rc = E2D_OK;
    // gpu_solver.cu:2200: while (step < MAXSTEP && Resd[step] > EPSL)
    if (s->ctl_host->resd > epsl) rc = run(s, max_steps, true, epsl, std::max(1, 64 / s->graph_iters));
    const int done = s->ctl_host->step - step0;
    if (nsteps) *nsteps = done;
    if (resid_history) std::memcpy(resid_history, s->hist.data() + step0, sizeof(double) * done);
    return rc;
}

int e2d_progress(e2d_solver *s, int32_t *step, double *resd) {
    if (!s) { set_error("null argument"); return E2D_ERR_ARG; }
    if (step) *step = s->ctl_host->step;
    if (resd) *resd = s->ctl_host->resd;
    return E2D_OK;
}

int e2d_residual_history(e2d_solver *s, double *out, int32_t cap, int32_t *n) {
    if (!s) { set_error("null argument"); return E2D_ERR_ARG; }
    int k = std::min((int)s->hist.size(), std::max(0, (int)cap));
    if (out && k) std::memcpy(out, s->hist.data(), sizeof(double) * k);
    if (n) *n = (int)s->hist.size();
    return E2D_OK;
}

int e2d_set_residual_norm(e2d_solver *s, double epsm) {
    if (!s) { set_error("null argument"); return E2D_ERR_ARG; }
    s->ctl_host->fixed_norm = epsm > 0.0;
    if (epsm > 0.0) s->ctl_host->epsm = epsm;
    return push_ctl(s);
}

int e2d_get_residual_norm(e2d_solver *s, double *epsm) {
    if (!s || !epsm) { set_error("null argument"); return E2D_ERR_ARG; }
    *epsm = s->ctl_host->epsm;
    return E2D_OK;
}

int e2d_get_state(e2d_solver *s, double *w) {
    if (!s || !w) { set_error("null argument"); return E2D_ERR_ARG; }
    return s->impl->download_state(w);
}

int e2d_set_state(e2d_solver *s, const double *w) {
    if (!s || !w) { set_error("null argument"); return E2D_ERR_ARG; }
    return s->impl->upload_state(w);
}

int e2d_profile_passes(e2d_solver *s, int32_t iters, double *ms, int32_t *launches) {
    if (!s || !ms || iters < 1) { set_error("bad argument"); return E2D_ERR_ARG; }
    int rc = ensure_hist(s, s->ctl_host->step + iters);
    if (rc) return rc;
    if ((rc = build_graph(s))) return rc;  // sets the history pointer of the plan
    Ctl &c = *s->ctl_host;
    c.halt = 0; c.nbad = 0; c.target = c.step + iters; c.check_epsl = 0;
    if ((rc = push_ctl(s))) return rc;
    const int per = s->impl->launches();
    std::vector<cudaEvent_t> ev(2 * (size_t)per * iters);
    std::vector<int> kind((size_t)per * iters);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    int j = 0;
    for (int it = 0; it < iters; it++) j += s->impl->enqueue_timed(s->stream, ev.data() + 2 * j, kind.data() + j);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->stream));
    for (int k = 0; k < 5; k++) { ms[k] = 0.0; if (launches) launches[k] = 0; }
    for (int q = 0; q < j; q++) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, ev[2 * q], ev[2 * q + 1]));
        ms[kind[q]] += t;
        if (launches) launches[kind[q]]++;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if ((rc = pull_ctl(s))) return rc;
    if ((rc = sync_hist(s))) return rc;
    return c.halt == 2 ? E2D_ERR_DIVERGED : E2D_OK;
}

int e2d_forces(e2d_solver *s, double *cl, double *cd) {
    if (!s) { set_error("null argument"); return E2D_ERR_ARG; }
    std::vector<double> w(4 * (size_t)s->L.n);
    int rc = e2d_get_state(s, w.data());
    if (rc) return rc;
    forces_from_state(s->L, s->fs, s->prm.gamma, w.data(), cl, cd);
    return E2D_OK;
}

int e2d_solver_integrals(e2d_solver *s, e2d_integrals *out) {
    if (!s || !out) { set_error("null argument"); return E2D_ERR_ARG; }
    std::vector<double> w(4 * (size_t)s->L.n);
    int rc = e2d_get_state(s, w.data());
    if (rc) return rc;
    integrals_from_state(s->L, s->fs, s->prm, w.data(), out);
    return E2D_OK;
}

int e2d_write_residual_plt(e2d_solver *s, const char *path) {
    if (!s || !path) { set_error("null argument"); return E2D_ERR_ARG; }
    FILE *fp = std::fopen(path, "w");
    if (!fp) { set_error(std::string("cannot write ") + path); return E2D_ERR_IO; }
    const int step = (int)s->hist.size();
    // gpu_fvm.cu:165-175
    std::fprintf(fp, "TITLE     = \"Dataset\"\nVARIABLES = \"Time\" \"Resid\" \n");
    std::fprintf(fp, "ZONE I=%d J=%d f=point \n", step, 1);
    for (int i = 1; i <= step; i++)
        if (i % 100 == 0) std::fprintf(fp, "%d %20.10lf\n", i, s->hist[i - 1]);
    std::fclose(fp);
    return E2D_OK;
}

int e2d_set_precision(e2d_solver *s, int32_t precision) {
    if (!s) { set_error("null argument"); return E2D_ERR_ARG; }
    if (precision != E2D_FP64 && precision != E2D_FP32) { set_error("precision must be E2D_FP64 or E2D_FP32"); return E2D_ERR_ARG; }
    if (precision == s->prm.precision) return E2D_OK;
    int rc = pull_ctl(s);
    if (rc) return rc;
    if (s->ctl_host->frozen) {
        set_error("the limiter values are frozen in the current precision and cannot be carried over");
        return E2D_ERR_ARG;
    }
    std::vector<double> w(4 * (size_t)s->L.n);
    if ((rc = s->impl->download_state(w.data()))) return rc;
    e2d_params p = s->prm;
    p.precision = precision;
    std::unique_ptr<SolverBase> next;
    if ((rc = make_impl(s, p, next))) return rc;
    if ((rc = next->upload_state(w.data()))) return rc;
    s->impl = std::move(next);
    s->prm.precision = precision;
    drop_graphs(s);
    return E2D_OK;
}

int e2d_get_params(e2d_solver *s, e2d_params *p) {
    if (!s || !p) { set_error("null argument"); return E2D_ERR_ARG; }
    *p = s->prm;
    return E2D_OK;
}

int e2d_last_device_ms(e2d_solver *s, double *ms) {
    if (!s || !ms) { set_error("null argument"); return E2D_ERR_ARG; }
    *ms = s->last_ms;
    return E2D_OK;
}

int e2d_launches_per_iteration(e2d_solver *s, int32_t *n) {
    if (!s || !n) { set_error("null argument"); return E2D_ERR_ARG; }
    *n = s->impl->launches();
    return E2D_OK;
}

int e2d_set_stream(e2d_solver *s, void *cuda_stream) {
    if (!s) { set_error("null argument"); return E2D_ERR_ARG; }
    CK(cudaStreamSynchronize(s->stream));
    if (s->own_stream) cudaStreamDestroy(s->stream);
    s->own_stream = cuda_stream == nullptr;
    if (s->own_stream) CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    else s->stream = (cudaStream_t)cuda_stream;
    return E2D_OK;
}

}  // extern "C"
