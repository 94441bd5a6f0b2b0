// batch.cu -- many independent flow cases on meshes of uneven size advanced
// together: one launch per pass covers every case, one CUDA graph covers
// graph_iters iterations of all of them, and each case keeps its own residual
// history and convergence test.  A project-written autotuner picks the launch
// shape (threads per CTA, persistent CTA count).  No reference counterpart:
// the reference solves one case per program run.
//
// Layout: the cells of case c (in the case's own internal order) occupy
// [off_c, off_c + n_c) of one concatenated array, off_c a multiple of kChunk =
// 256 cells, so every tile of B | 256 cells belongs to one case and the
// per-tile residual partials of a case group exactly as in a single-case run.
// Each case therefore reproduces its single-case solve bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <sstream>
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

namespace {

struct BatchBase {
    virtual ~BatchBase() {}
    virtual int enqueue(cudaStream_t s) = 0;
    virtual int set_launch(int block, int grid) = 0;
    virtual int launches() const = 0;
    virtual int upload_case(int c, const double *w_file, cudaStream_t s) = 0;
    virtual int download_case(int c, double *w_file, cudaStream_t s) = 0;
    virtual int save_state(cudaStream_t s) = 0;
    virtual int restore_state(cudaStream_t s) = 0;
    virtual const void *topo_ptr() const = 0;
};

template <typename T> struct BatchT : BatchBase {
    const std::vector<HostLayout> *L;
    const std::vector<int> *off;
    int ntot = 0;
    Arena arena;
    BPlan<T> plan;
    int *perm_dev = nullptr;      // [ntot] internal -> file index within the case
    double *wfile_dev = nullptr;  // [4 * max n_c]
    int2 *case_tiles = nullptr;   // [ncase]
    V4<T> *backup = nullptr;      // [ntot] (autotune)
    std::vector<int2> ct_host;

    int init(const std::vector<e2d_params> &P, const std::vector<FreeStream> &FS, int ntot_, Ctl *ctl,
             double *hist, int hist_cap) {
        ntot = ntot_;
        const int n = ntot, ncase = (int)L->size();
        bool freeze = false;
        for (auto &p : P) freeze = freeze || p.limiter_freeze > 0 || p.limiter_freeze_resd > 0.0;
        plan.options = freeze;
        for (auto &p : P)
            plan.options = plan.options || p.limiter != 0 || p.global_dt != 0 || p.first_order_iters > 0 ||
                           p.positivity_fix != 0;
        int nmax = 0;
        for (auto &l : *L) nmax = std::max(nmax, l.n);
        const int maxtiles = (n + 31) / 32;
        size_t bytes = Arena::up(sizeof(int4) * n) + 2 * Arena::up(sizeof(V2<T>) * 3 * n) +
                       2 * Arena::up(sizeof(T) * n) + 6 * Arena::up(sizeof(V4<T>) * n) +
                       Arena::up(sizeof(V4<T>) * 3 * n) * (freeze ? 2 : 1) + Arena::up(sizeof(double) * maxtiles) +
                       Arena::up(sizeof(int) * n) + Arena::up(sizeof(double) * 4 * nmax) +
                       Arena::up(sizeof(Flow<T>) * ncase) + Arena::up(sizeof(int) * (n / kChunk + 1)) +
                       2 * Arena::up(sizeof(int2) * ncase);
        CK(cudaMalloc((void **)&arena.base, bytes));
        arena.cap = bytes;
        int4 *topo = (int4 *)arena.take(sizeof(int4) * n);
        V2<T> *S = (V2<T> *)arena.take(sizeof(V2<T>) * 3 * n);
        V2<T> *R = (V2<T> *)arena.take(sizeof(V2<T>) * 3 * n);
        T *area = (T *)arena.take(sizeof(T) * n);
        plan.W[0] = (V4<T> *)arena.take(sizeof(V4<T>) * n);
        plan.W[1] = (V4<T> *)arena.take(sizeof(V4<T>) * n);
        plan.FS = (V4<T> *)arena.take(sizeof(V4<T>) * 3 * n);
        plan.phi = freeze ? (V4<T> *)arena.take(sizeof(V4<T>) * 3 * n) : nullptr;
        plan.dt = (T *)arena.take(sizeof(T) * n);
        plan.res = (V4<T> *)arena.take(sizeof(V4<T>) * n);
        plan.sm[0] = (V4<T> *)arena.take(sizeof(V4<T>) * n);
        plan.sm[1] = (V4<T> *)arena.take(sizeof(V4<T>) * n);
        backup = (V4<T> *)arena.take(sizeof(V4<T>) * n);
        plan.part = (double *)arena.take(sizeof(double) * maxtiles);
        perm_dev = (int *)arena.take(sizeof(int) * n);
        wfile_dev = (double *)arena.take(sizeof(double) * 4 * nmax);
        Flow<T> *flows = (Flow<T> *)arena.take(sizeof(Flow<T>) * ncase);
        int *chunk_case = (int *)arena.take(sizeof(int) * (n / kChunk + 1));
        int *case_end = (int *)arena.take(sizeof(int) * ncase);
        case_tiles = (int2 *)arena.take(sizeof(int2) * ncase);
        // concatenated mesh (padding cells stay zero and are never touched)
        std::vector<int32_t> ht(4 * (size_t)n, 0);
        std::vector<T> hS(6 * (size_t)n, T(0)), hR(6 * (size_t)n, T(0)), ha(n, T(1));
        std::vector<int> hp(n, 0), hcc(n / kChunk + 1, 0), hce(ncase);
        std::vector<Flow<T>> hf(ncase);
        for (int c = 0; c < ncase; c++) {
            const HostLayout &l = (*L)[c];
            const int o = (*off)[c];
            for (int i = 0; i < l.n; i++) {
                for (int k = 0; k < 3; k++) {
                    int code = l.topo[4 * (size_t)i + k];
                    ht[4 * (size_t)(o + i) + k] = code >= 0 ? code + (o << 3) : code;
                    for (int q = 0; q < 2; q++) {
                        hS[2 * ((size_t)k * n + o + i) + q] = (T)l.S[2 * ((size_t)k * l.n + i) + q];
                        hR[2 * ((size_t)k * n + o + i) + q] = (T)l.R[2 * ((size_t)k * l.n + i) + q];
                    }
                }
                ht[4 * (size_t)(o + i) + 3] = l.topo[4 * (size_t)i + 3];
                ha[o + i] = (T)l.area[i];
                hp[o + i] = l.perm[i];
            }
            const int oend = c + 1 < ncase ? (*off)[c + 1] : n;
            for (int ch = o / kChunk; ch < oend / kChunk; ch++) hcc[ch] = c;
            hce[c] = o + l.n;
            const e2d_params &p = P[c];
            Flow<T> &f = hf[c];
            f.gamma = (T)p.gamma; f.ui = (T)FS[c].ui; f.vi = (T)FS[c].vi; f.ain = (T)FS[c].ain_test;
            f.tin = (T)p.tin; f.vin = (T)FS[c].vin; f.R = (T)287.06; f.pis = (T)FS[c].pis; f.cfl = (T)p.cfl;
            f.dt_cap = (T)p.dt_cap; f.eps_entropy = (T)p.entropy_eps; f.irs_eps = (T)p.irs_eps;
            f.venk_k3 = (T)(p.limiter_k * p.limiter_k * p.limiter_k); f.limiter = p.limiter;
            f.global_dt = p.global_dt;
            f.first_order = p.first_order_iters; f.positivity = p.positivity_fix;
        }
        CK(cudaMemcpy(topo, ht.data(), sizeof(int4) * n, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(S, hS.data(), sizeof(T) * hS.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(R, hR.data(), sizeof(T) * hR.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(area, ha.data(), sizeof(T) * n, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(perm_dev, hp.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(flows, hf.data(), sizeof(Flow<T>) * ncase, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(chunk_case, hcc.data(), sizeof(int) * hcc.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(case_end, hce.data(), sizeof(int) * ncase, cudaMemcpyHostToDevice));
        CK(cudaMemset(plan.W[0], 0, sizeof(V4<T>) * n));
        CK(cudaMemset(plan.W[1], 0, sizeof(V4<T>) * n));
        plan.m = MeshDev<T>{n, topo, S, R, area};
        plan.f = hf[0];
        plan.b = BatchDev<T>{flows, chunk_case, case_end, ctl};
        plan.ncase = ncase;
        plan.case_tiles = case_tiles;
        plan.hist = hist;
        plan.hist_cap = hist_cap;
        plan.stages = P[0].rk_stages;
        for (int k = 0; k < 8; k++) plan.rk[k] = (T)P[0].rk_coef[k];
        plan.sweeps = P[0].irs_sweeps;
        return E2D_OK;
    }

    int set_launch(int block, int grid) override {
        const int ncase = (int)L->size();
        ct_host.resize(ncase);
        for (int c = 0; c < ncase; c++)
            ct_host[c] = make_int2((*off)[c] / block, ((*L)[c].n + block - 1) / block);
        CK(cudaMemcpy(case_tiles, ct_host.data(), sizeof(int2) * ncase, cudaMemcpyHostToDevice));
        plan.block = block;
        plan.grid = grid;
        return E2D_OK;
    }

    int enqueue(cudaStream_t s) override {
        enqueue_batch_iteration<T>(plan, s);
        CK(cudaGetLastError());
        return E2D_OK;
    }

    int launches() const override { return launches_per_iteration(plan); }
    const void *topo_ptr() const override { return plan.m.topo; }

    int upload_case(int c, const double *w, cudaStream_t s) override {
        const int n = (*L)[c].n, o = (*off)[c];
        CK(cudaMemcpyAsync(wfile_dev, w, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, s));
        enqueue_import<T>(n, perm_dev + o, wfile_dev, plan.W[0] + o, s);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(s));
        return E2D_OK;
    }

    int download_case(int c, double *w, cudaStream_t s) override {
        const int n = (*L)[c].n, o = (*off)[c];
        enqueue_export<T>(n, perm_dev + o, plan.W[0] + o, wfile_dev, s);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(w, wfile_dev, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        return E2D_OK;
    }

    int save_state(cudaStream_t s) override {
        CK(cudaMemcpyAsync(backup, plan.W[0], sizeof(V4<T>) * ntot, cudaMemcpyDeviceToDevice, s));
        return E2D_OK;
    }

    int restore_state(cudaStream_t s) override {
        CK(cudaMemcpyAsync(plan.W[0], backup, sizeof(V4<T>) * ntot, cudaMemcpyDeviceToDevice, s));
        return E2D_OK;
    }
};

}  // namespace

struct e2d_batch {
    int ncase = 0;
    std::vector<e2d_params> prm;
    std::vector<HostLayout> L;
    std::vector<FreeStream> fs;
    std::vector<int> off;
    int ntot = 0;
    std::unique_ptr<BatchBase> impl;
    Ctl *ctl_dev = nullptr, *ctl_host = nullptr;  // [ncase]
    double *hist_dev = nullptr;
    int hist_cap = 0;
    std::vector<std::vector<double>> hist;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int graph_iters = 8;
    int block = 128, grid = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0.0;
    bool l2_held = false;  // counted among the users of the persisting L2 carve-out

    ~e2d_batch() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamSynchronize(stream);
        release_l2(&l2_held);
        if (stream) cudaStreamDestroy(stream);
        if (ctl_dev) cudaFree(ctl_dev);
        if (ctl_host) cudaFreeHost(ctl_host);
        if (hist_dev) cudaFree(hist_dev);
    }
};

namespace {

int tiles_of(const e2d_batch *b, int block) { return (b->ntot + block - 1) / block; }

int rebuild_graph(e2d_batch *b) {
    if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int rc = E2D_OK;
    for (int it = 0; it < b->graph_iters && rc == E2D_OK; it++) rc = b->impl->enqueue(b->stream);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) { set_error(std::string("graph capture: ") + cudaGetErrorString(e)); return E2D_ERR_CUDA; }
    keep_in_l2(g, b->impl->topo_ptr(), sizeof(int4) * (size_t)b->ntot, &b->l2_held);
    e = cudaGraphInstantiate(&b->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { b->gexec = nullptr; set_error(std::string("graph instantiate: ") + cudaGetErrorString(e)); return E2D_ERR_CUDA; }
    return E2D_OK;
}

int apply_launch(e2d_batch *b, int block, int grid) {
    if (block < 32 || block > 256 || kChunk % block) { set_error("block must divide 256 (32..256)"); return E2D_ERR_ARG; }
    const int nt = tiles_of(b, block);
    if (grid <= 0 || grid > nt) grid = nt;
    int rc = b->impl->set_launch(block, grid);
    if (rc) return rc;
    b->block = block;
    b->grid = grid;
    return rebuild_graph(b);
}

int pull_all(e2d_batch *b) {
    CK(cudaMemcpyAsync(b->ctl_host, b->ctl_dev, sizeof(Ctl) * b->ncase, cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return E2D_OK;
}

int sync_hist_all(e2d_batch *b) {
    for (int c = 0; c < b->ncase; c++) {
        const int step = b->ctl_host[c].step, have = (int)b->hist[c].size();
        if (step <= have) continue;
        b->hist[c].resize(step);
        CK(cudaMemcpy(b->hist[c].data() + have, b->hist_dev + (size_t)c * b->hist_cap + have,
                      sizeof(double) * (step - have), cudaMemcpyDeviceToHost));
    }
    return E2D_OK;
}

// Runs up to n iterations of every case; with check, a case stops at its own
// Resd <= epsl.  Halted (converged or diverged) cases stay frozen.
int run_batch(e2d_batch *b, int n, bool check, double epsl) {
    if (n <= 0) return E2D_OK;
    for (int c = 0; c < b->ncase; c++) {
        Ctl &C = b->ctl_host[c];
        if (C.halt == 2) continue;  // diverged cases stay stopped
        if (check && C.step > 0 && !(C.resd > epsl)) { C.halt = 1; continue; }
        C.halt = 0;
        C.nbad = 0;
        C.target = C.step + n;
        C.check_epsl = check ? 1 : 0;
        C.epsl = epsl;
    }
    CK(cudaMemcpyAsync(b->ctl_dev, b->ctl_host, sizeof(Ctl) * b->ncase, cudaMemcpyHostToDevice, b->stream));
    const int launches = (n + b->graph_iters - 1) / b->graph_iters;
    const int poll = check ? std::max(1, 64 / b->graph_iters) : 0;
    CK(cudaEventRecord(b->ev0, b->stream));
    for (int k = 0; k < launches; k++) {
        CK(cudaGraphLaunch(b->gexec, b->stream));
        if (poll && (k + 1) % poll == 0 && k + 1 < launches) {
            int rc = pull_all(b);
            if (rc) return rc;
            bool all = true;
            for (int c = 0; c < b->ncase && all; c++) all = b->ctl_host[c].halt != 0;
            if (all) break;
        }
    }
    CK(cudaEventRecord(b->ev1, b->stream));
    int rc = pull_all(b);
    if (rc) return rc;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms;
    if ((rc = sync_hist_all(b))) return rc;
    for (int c = 0; c < b->ncase; c++)
        if (b->ctl_host[c].halt == 2) {
            set_error("case " + std::to_string(c) + " diverged at step " + std::to_string(b->ctl_host[c].step));
            return E2D_ERR_DIVERGED;
        }
    return E2D_OK;
}

std::string gpu_name() {
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "gpu";
    std::string s = prop.name;
    for (auto &ch : s)
        if (ch == ' ' || ch == '"') ch = '_';
    return s;
}

}  // namespace

extern "C" {

int e2d_batch_create(e2d_mesh **meshes, const e2d_params *params, int32_t ncase, e2d_batch **out) {
    if (!meshes || !params || !out || ncase < 1) { set_error("bad argument"); return E2D_ERR_ARG; }
    *out = nullptr;
    const e2d_params &p0 = params[0];
    for (int c = 0; c < ncase; c++) {
        const e2d_params &p = params[c];
        if (!meshes[c]) { set_error("null mesh of case " + std::to_string(c)); return E2D_ERR_ARG; }
        if (const char *why = param_error(&p)) {
            set_error("invalid parameters of case " + std::to_string(c) + ": " + why);
            return E2D_ERR_ARG;
        }
        bool same = p.precision == p0.precision && p.rk_stages == p0.rk_stages && p.irs_sweeps == p0.irs_sweeps &&
                    p.irs_eps == p0.irs_eps && p.gamma == p0.gamma && p.entropy_eps == p0.entropy_eps &&
                    p.dt_cap == p0.dt_cap && std::memcmp(p.rk_coef, p0.rk_coef, sizeof p.rk_coef) == 0;
        if (!same) {
            set_error("cases must share precision, RK scheme, smoothing, gamma, entropy fix and dt cap "
                      "(case " + std::to_string(c) + " differs)");
            return E2D_ERR_ARG;
        }
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        set_error("no CUDA device: the solver runs on the GPU only");
        return E2D_ERR_CUDA;
    }
    auto b = std::make_unique<e2d_batch>();
    b->ncase = ncase;
    b->prm.assign(params, params + ncase);
    b->L.resize(ncase);
    b->fs.resize(ncase);
    b->off.resize(ncase);
    int64_t tot = 0;
    for (int c = 0; c < ncase; c++) {
        int rc = build_layout(meshes[c], params[c], b->L[c]);
        if (rc) return rc;
        b->fs[c] = free_stream(params[c]);
        b->off[c] = (int)tot;
        tot += ((int64_t)b->L[c].n + kChunk - 1) / kChunk * kChunk;
        if (tot >= (1 << 28)) { set_error("batch too large (limit 2^28 cells)"); return E2D_ERR_CAPACITY; }
    }
    b->ntot = (int)tot;
    CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&b->ev0));
    CK(cudaEventCreate(&b->ev1));
    CK(cudaMalloc((void **)&b->ctl_dev, sizeof(Ctl) * ncase));
    CK(cudaMallocHost((void **)&b->ctl_host, sizeof(Ctl) * ncase));
    std::memset(b->ctl_host, 0, sizeof(Ctl) * ncase);
    for (int c = 0; c < ncase; c++) {
        b->ctl_host[c].resd = 100.0;
        b->ctl_host[c].freeze_after = params[c].limiter_freeze > 0 ? params[c].limiter_freeze : 0;
        b->ctl_host[c].freeze_resd = params[c].limiter_freeze_resd > 0.0 ? params[c].limiter_freeze_resd : 0.0;
        for (auto &d : b->ctl_host[c].dtmin) d = kDtNone;
    }
    CK(cudaMemcpy(b->ctl_dev, b->ctl_host, sizeof(Ctl) * ncase, cudaMemcpyHostToDevice));
    // the history buffer is sized once here: its pointer is captured in the graph
    int maxstep = 0;
    for (int c = 0; c < ncase; c++) maxstep = std::max(maxstep, params[c].maxstep);
    b->hist_cap = std::max(1024, maxstep);
    CK(cudaMalloc((void **)&b->hist_dev, sizeof(double) * b->hist_cap * (size_t)ncase));
    b->hist.resize(ncase);
    b->graph_iters = p0.graph_iters > 0 ? p0.graph_iters : 8;
    int rc;
    if (p0.precision == E2D_FP64) {
        auto *t = new BatchT<double>();
        t->L = &b->L; t->off = &b->off;
        b->impl.reset(t);
        rc = t->init(b->prm, b->fs, b->ntot, b->ctl_dev, b->hist_dev, b->hist_cap);
    } else {
        auto *t = new BatchT<float>();
        t->L = &b->L; t->off = &b->off;
        b->impl.reset(t);
        rc = t->init(b->prm, b->fs, b->ntot, b->ctl_dev, b->hist_dev, b->hist_cap);
    }
    if (rc) return rc;
    for (int c = 0; c < ncase; c++) {
        std::vector<double> w0(4 * (size_t)b->L[c].n);
        for (int i = 0; i < b->L[c].n; i++) {
            w0[4 * (size_t)i] = 1.0; w0[4 * (size_t)i + 1] = std::cos(b->fs[c].alpha);
            w0[4 * (size_t)i + 2] = std::sin(b->fs[c].alpha); w0[4 * (size_t)i + 3] = b->fs[c].rho_e;
        }
        if ((rc = b->impl->upload_case(c, w0.data(), b->stream))) return rc;
    }
    const int block = p0.block_size > 0 ? p0.block_size : 128;
    if ((rc = apply_launch(b.get(), block, 0))) return rc;
    *out = b.release();
    return E2D_OK;
}

void e2d_batch_destroy(e2d_batch *b) { delete b; }

int e2d_batch_step(e2d_batch *b, int32_t n) {
    if (!b || n < 0) { set_error("bad argument"); return E2D_ERR_ARG; }
    int maxstep = 0;
    for (int c = 0; c < b->ncase; c++) maxstep = std::max(maxstep, b->ctl_host[c].step);
    if (maxstep + n > b->hist_cap) { set_error("iterations beyond the residual history capacity (maxstep)"); return E2D_ERR_CAPACITY; }
    return run_batch(b, n, false, 0.0);
}

int e2d_batch_solve(e2d_batch *b, int32_t max_steps, double epsl, int32_t *nsteps) {
    if (!b || max_steps < 0 || std::isnan(epsl)) { set_error("bad argument"); return E2D_ERR_ARG; }
    int maxstep = 0;
    for (int c = 0; c < b->ncase; c++) maxstep = std::max(maxstep, b->ctl_host[c].step);
    if (maxstep + max_steps > b->hist_cap) { set_error("iterations beyond the residual history capacity (maxstep)"); return E2D_ERR_CAPACITY; }
    std::vector<int> s0(b->ncase);
    for (int c = 0; c < b->ncase; c++) s0[c] = b->ctl_host[c].step;
    int rc = run_batch(b, max_steps, true, epsl);
    if (nsteps)
        for (int c = 0; c < b->ncase; c++) nsteps[c] = b->ctl_host[c].step - s0[c];
    return rc;
}

int e2d_batch_info(e2d_batch *b, int32_t *ncase, int64_t *ncell_total, int64_t *ncell_padded) {
    if (!b) { set_error("null argument"); return E2D_ERR_ARG; }
    if (ncase) *ncase = b->ncase;
    if (ncell_total) {
        int64_t t = 0;
        for (auto &l : b->L) t += l.n;
        *ncell_total = t;
    }
    if (ncell_padded) *ncell_padded = b->ntot;
    return E2D_OK;
}

int e2d_batch_get_state(e2d_batch *b, int32_t c, double *w) {
    if (!b || !w || c < 0 || c >= b->ncase) { set_error("bad argument"); return E2D_ERR_ARG; }
    return b->impl->download_case(c, w, b->stream);
}

int e2d_batch_set_state(e2d_batch *b, int32_t c, const double *w) {
    if (!b || !w || c < 0 || c >= b->ncase) { set_error("bad argument"); return E2D_ERR_ARG; }
    return b->impl->upload_case(c, w, b->stream);
}

int e2d_batch_progress(e2d_batch *b, int32_t c, int32_t *step, double *resd, int32_t *halted) {
    if (!b || c < 0 || c >= b->ncase) { set_error("bad argument"); return E2D_ERR_ARG; }
    if (step) *step = b->ctl_host[c].step;
    if (resd) *resd = b->ctl_host[c].resd;
    if (halted) *halted = b->ctl_host[c].halt;
    return E2D_OK;
}

int e2d_batch_residual_history(e2d_batch *b, int32_t c, double *out, int32_t cap, int32_t *n) {
    if (!b || c < 0 || c >= b->ncase) { set_error("bad argument"); return E2D_ERR_ARG; }
    const auto &h = b->hist[c];
    int k = std::min((int)h.size(), std::max(0, (int)cap));
    if (out && k) std::memcpy(out, h.data(), sizeof(double) * k);
    if (n) *n = (int)h.size();
    return E2D_OK;
}

int e2d_batch_forces(e2d_batch *b, int32_t c, double *cl, double *cd) {
    if (!b || c < 0 || c >= b->ncase) { set_error("bad argument"); return E2D_ERR_ARG; }
    std::vector<double> w(4 * (size_t)b->L[c].n);
    int rc = b->impl->download_case(c, w.data(), b->stream);
    if (rc) return rc;
    forces_from_state(b->L[c], b->fs[c], b->prm[c].gamma, w.data(), cl, cd);
    return E2D_OK;
}

int e2d_batch_set_launch(e2d_batch *b, int32_t block, int32_t grid) {
    if (!b) { set_error("null argument"); return E2D_ERR_ARG; }
    return apply_launch(b, block, grid);
}

int e2d_batch_get_launch(e2d_batch *b, int32_t *block, int32_t *grid) {
    if (!b) { set_error("null argument"); return E2D_ERR_ARG; }
    if (block) *block = b->block;
    if (grid) *grid = b->grid;
    return E2D_OK;
}

int e2d_batch_create_tuned(e2d_mesh **meshes, const e2d_params *params, int32_t ncase, const char *cache_path,
                           int32_t iters, e2d_batch **out, int32_t *ordering) {
    if (!meshes || !params || !out || ncase < 1 || iters < 1) { set_error("bad argument"); return E2D_ERR_ARG; }
    *out = nullptr;
    std::vector<e2d_params> P(params, params + ncase);
    double best = 1e300;
    int best_ord = E2D_ORDER_MORTON;
    for (int ord : {E2D_ORDER_MORTON, E2D_ORDER_RCM, E2D_ORDER_FILE}) {
        for (auto &p : P) p.ordering = ord;
        e2d_batch *b = nullptr;
        int rc = e2d_batch_create(meshes, P.data(), ncase, &b);
        if (rc) return rc;
        double ms = 0.0;
        rc = e2d_batch_autotune(b, cache_path, iters, nullptr, nullptr, &ms);
        e2d_batch_destroy(b);
        if (rc) return rc;
        if (ms < best) { best = ms; best_ord = ord; }
    }
    for (auto &p : P) p.ordering = best_ord;
    int rc = e2d_batch_create(meshes, P.data(), ncase, out);
    if (rc) return rc;
    // the winner's launch shape is in the cache when there is one, else tune again
    if ((rc = e2d_batch_autotune(*out, cache_path, iters, nullptr, nullptr, nullptr))) {
        e2d_batch_destroy(*out);
        *out = nullptr;
        return rc;
    }
    if (ordering) *ordering = best_ord;
    return E2D_OK;
}

int e2d_batch_last_device_ms(e2d_batch *b, double *ms) {
    if (!b || !ms) { set_error("null argument"); return E2D_ERR_ARG; }
    *ms = b->last_ms;
    return E2D_OK;
}

int e2d_batch_launches_per_iteration(e2d_batch *b, int32_t *n) {
    if (!b || !n) { set_error("null argument"); return E2D_ERR_ARG; }
    *n = b->impl->launches();
    return E2D_OK;
}

// Times candidate launch shapes -- threads per CTA {64, 128, 256} x CTAs
// {one per tile, and persistent grids of 2, 4, 8 and 16 CTAs per SM} -- on
// `iters` iterations each (after one warm-up graph), keeps the fastest and
// leaves the state and residual histories as they were.  With cache_path, a
// result stored for the same GPU, cell count, case count and scheme is reused
// without timing, and new results are added to the file (one JSON object).
int e2d_batch_autotune(e2d_batch *b, const char *cache_path, int32_t iters, int32_t *block, int32_t *grid,
                       double *ms_per_iter) {
    if (!b || iters < 1) { set_error("bad argument"); return E2D_ERR_ARG; }
    std::ostringstream key;
    key << gpu_name() << "|cells=" << b->ntot << "|cases=" << b->ncase << "|prec=" << b->prm[0].precision
        << "|stages=" << b->prm[0].rk_stages << "|sweeps=" << b->prm[0].irs_sweeps
        << "|order=" << b->prm[0].ordering;
    std::string text;
    if (cache_path) {
        if (FILE *f = std::fopen(cache_path, "r")) {
            char buf[4096];
            size_t k;
            while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, k);
            std::fclose(f);
        }
        const std::string pat = "\"" + key.str() + "\": [";
        size_t at = text.find(pat);
        if (at != std::string::npos) {
            int bb = 0, gg = 0;
            double ms = 0;
            if (std::sscanf(text.c_str() + at + pat.size(), "%d, %d, %lf", &bb, &gg, &ms) == 3) {
                int rc = apply_launch(b, bb, gg);
                if (rc) return rc;
                if (block) *block = bb;
                if (grid) *grid = b->grid;
                if (ms_per_iter) *ms_per_iter = ms;
                return E2D_OK;
            }
        }
    }
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // save everything the timing runs change
    std::vector<Ctl> ctl0(b->ctl_host, b->ctl_host + b->ncase);
    auto hist0 = b->hist;
    int rc = b->impl->save_state(b->stream);
    if (rc) return rc;
    std::vector<double> hsave((size_t)b->hist_cap * b->ncase);
    CK(cudaMemcpy(hsave.data(), b->hist_dev, sizeof(double) * hsave.size(), cudaMemcpyDeviceToHost));
    double best = 1e300;
    int bb = 128, bg = 0;
    for (int blk : {64, 128, 256}) {
        const int nt = tiles_of(b, blk);
        for (int per_sm : {0, 2, 4, 8, 16}) {
            int g = per_sm == 0 ? nt : std::min(nt, per_sm * sms);
            if ((rc = apply_launch(b, blk, g))) return rc;
            for (int c = 0; c < b->ncase; c++) {  // timing runs never halt early
                b->ctl_host[c] = ctl0[c];
                b->ctl_host[c].halt = 0;
                b->ctl_host[c].check_epsl = 0;
                b->ctl_host[c].target = 1 << 30;
            }
            CK(cudaMemcpy(b->ctl_dev, b->ctl_host, sizeof(Ctl) * b->ncase, cudaMemcpyHostToDevice));
            CK(cudaGraphLaunch(b->gexec, b->stream));
            const int launches = std::max(1, iters / b->graph_iters);
            CK(cudaEventRecord(b->ev0, b->stream));
            for (int k = 0; k < launches; k++) CK(cudaGraphLaunch(b->gexec, b->stream));
            CK(cudaEventRecord(b->ev1, b->stream));
            CK(cudaStreamSynchronize(b->stream));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
            const double per = ms / (launches * b->graph_iters);
            if (per < best) { best = per; bb = blk; bg = b->grid; }
            if ((rc = b->impl->restore_state(b->stream))) return rc;
        }
    }
    CK(cudaMemcpy(b->hist_dev, hsave.data(), sizeof(double) * hsave.size(), cudaMemcpyHostToDevice));
    std::copy(ctl0.begin(), ctl0.end(), b->ctl_host);
    CK(cudaMemcpy(b->ctl_dev, b->ctl_host, sizeof(Ctl) * b->ncase, cudaMemcpyHostToDevice));
    b->hist = hist0;
    if ((rc = apply_launch(b, bb, bg))) return rc;
    if (block) *block = bb;
    if (grid) *grid = bg;
    if (ms_per_iter) *ms_per_iter = best;
    if (cache_path) {
        std::string body = text;
        size_t close = body.rfind('}');
        std::ostringstream entry;
        entry << "\"" << key.str() << "\": [" << bb << ", " << bg << ", " << best << "]";
        if (close == std::string::npos) body = "{\n  " + entry.str() + "\n}\n";
        else {
            bool empty = body.find('[') == std::string::npos;
            body = body.substr(0, close) + (empty ? "  " : ",\n  ") + entry.str() + "\n}\n";
        }
        if (FILE *f = std::fopen(cache_path, "w")) {
            std::fwrite(body.data(), 1, body.size(), f);
            std::fclose(f);
        }
    }
    return E2D_OK;
}

}  // extern "C"
