// mesh.cpp -- mesh files, the NACA 0012 O-grid generator, the mesh set-up
// (geometry, edge discovery, boundary tags) and cell orderings.
//
// The set-up reproduces the reference numbering of CalculationMeshGeo
// (gpu_init.cu:100-228) and changeEdge (gpu_solver.cu:1832-1906) in O(N)
// instead of the reference's O(N^2) search: faces are bucketed by their lower
// node id, partners are matched inside the (short) buckets, and edges are
// numbered in (cell, face) order of first appearance.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>

#include "internal.h"

namespace e2d {

static thread_local std::string g_error;

void set_error(const std::string &msg) { g_error = msg; }

// gpu_init.cu:95-98 (Calc_area): twice-signed area / 2, positive for CCW
static inline double tri_area(double x1, double y1, double x2, double y2, double x3, double y3) {
    return (0.5 * ((y3 - y1) * (x2 - x1) - (y2 - y1) * (x3 - x1)));
}

// ---- parallel loops of the set-up -----------------------------------------
// The set-up runs on the host cores: a fixed split of [0, n) into one chunk
// per worker (std::thread; the split depends only on n and the worker count,
// so two passes over the same range see the same chunks).  Small ranges run
// on the calling thread.
static int setup_workers() {
    static const int w = [] {
        if (const char *e = std::getenv("E2D_SETUP_THREADS")) {
            const int v = std::atoi(e);
            if (v >= 1) return std::min(v, 256);
        }
        const unsigned h = std::thread::hardware_concurrency();
        return (int)std::min(64u, std::max(1u, h));
    }();
    return w;
}

struct Split {
    int64_t n;
    int T;
    explicit Split(int64_t n_) : n(n_), T(n_ < 32768 ? 1 : (int)std::min<int64_t>(setup_workers(), n_ / 16384)) {}
    int64_t begin(int t) const { return n * t / T; }
    int64_t end(int t) const { return n * (t + 1) / T; }
    // fn(begin, end, chunk) for every chunk
    template <class F> void run(F fn) const {
        if (T == 1) { fn((int64_t)0, n, 0); return; }
        std::vector<std::thread> th;
        th.reserve(T - 1);
        for (int t = 1; t < T; t++) th.emplace_back([&, t] { fn(begin(t), end(t), t); });
        fn(begin(0), end(0), 0);
        for (auto &x : th) x.join();
    }
};

// Set-up of CalculationMeshGeo (gpu_init.cu:100-228) and changeEdge
// (gpu_solver.cu:1832-1906) with the reference's numbering: edges numbered in
// (cell, face) order of first appearance, boundary edges tagged wall or far by
// the box rule and numbered in the same order, then a stable partition
// interior / far / wall.  Each step is a parallel pass over cells or faces
// followed by prefix sums over the chunks, so the result does not depend on
// the number of workers.
int build_topology(e2d_mesh *m, double wall_box) {
    MeshTopo &t = m->topo;
    if (t.wall_box == wall_box && !t.clog.empty()) return E2D_OK;
    t = MeshTopo();
    const int N = m->ncell, NN = m->nnode;
    if (N < 1 || NN < 3) { set_error("empty mesh"); return E2D_ERR_MESH; }
    t.area.resize(N); t.cx.resize(N); t.cy.resize(N);
    const Split cells(N), faces(3 * (int64_t)N);
    // 1. area and centroid; a bad cell is reported by its smallest index
    //    (1 node id out of range, 2 area <= 0)
    std::vector<char> bad(N, 0);
    const double *X = m->x.data() - 1, *Y = m->y.data() - 1;
    cells.run([&](int64_t c0, int64_t c1, int) {
        for (int64_t i = c0; i < c1; i++) {
            const int *p = &m->tri[3 * i];
            if (p[0] < 1 || p[0] > NN || p[1] < 1 || p[1] > NN || p[2] < 1 || p[2] > NN) { bad[i] = 1; continue; }
            t.area[i] = tri_area(X[p[0]], Y[p[0]], X[p[1]], Y[p[1]], X[p[2]], Y[p[2]]);
            if (!(t.area[i] > 0.0)) { bad[i] = 2; continue; }
            t.cx[i] = (X[p[0]] + X[p[1]] + X[p[2]]) / 3.0;
            t.cy[i] = (Y[p[0]] + Y[p[1]] + Y[p[2]]) / 3.0;
        }
    });
    for (int i = 0; i < N; i++) {
        if (bad[i] == 1) { set_error("node id out of range in cell " + std::to_string(i + 1)); return E2D_ERR_MESH; }
        if (bad[i] == 2) {
            set_error("cell " + std::to_string(i + 1) + " has area <= 0 (cells must be counter-clockwise)");
            return E2D_ERR_MESH;
        }
    }
    // face f of a cell joins Point[(f+1)%3] and Point[(f+2)%3]
    auto fnodes = [&](int c, int f, int &a, int &b) {
        a = m->tri[3 * c + (f + 1) % 3];
        b = m->tri[3 * c + (f + 2) % 3];
    };
    // 2. faces bucketed by their lower node id (counting sort; inside a bucket
    //    the faces are put back in (cell, face) order)
    std::vector<std::atomic<int>> cnt(NN + 2);
    for (auto &v : cnt) v.store(0, std::memory_order_relaxed);
    faces.run([&](int64_t f0, int64_t f1, int) {
        for (int64_t cf = f0; cf < f1; cf++) {
            int a, b; fnodes((int)(cf / 3), (int)(cf % 3), a, b);
            cnt[std::min(a, b) + 1].fetch_add(1, std::memory_order_relaxed);
        }
    });
    std::vector<int> start(NN + 2, 0);
    for (int i = 1; i < NN + 2; i++) start[i] = start[i - 1] + cnt[i].load(std::memory_order_relaxed);
    for (int i = 0; i < NN + 2; i++) cnt[i].store(start[i], std::memory_order_relaxed);
    std::vector<int> bucket(3 * (size_t)N);
    faces.run([&](int64_t f0, int64_t f1, int) {
        for (int64_t cf = f0; cf < f1; cf++) {
            int a, b; fnodes((int)(cf / 3), (int)(cf % 3), a, b);
            bucket[cnt[std::min(a, b)].fetch_add(1, std::memory_order_relaxed)] = (int)cf;
        }
    });
    // 3. partner face: the other face of the same node pair (one at most);
    //    err[lo] marks a bucket with a degenerate face, a repeated edge or a
    //    non-manifold edge, reported for the smallest node
    std::vector<int> partner(3 * (size_t)N, -1);
    std::vector<char> err(NN + 2, 0);
    const Split nodes(NN);
    nodes.run([&](int64_t n0, int64_t n1, int) {
        for (int64_t lo = n0 + 1; lo <= n1; lo++) {
            const int s0 = start[lo], e0 = start[lo + 1];
            std::sort(bucket.begin() + s0, bucket.begin() + e0);
            for (int u = s0; u < e0 && !err[lo]; u++) {
                const int cf = bucket[u];
                int a, b; fnodes(cf / 3, cf % 3, a, b);
                if (a == b) { err[lo] = 1; break; }
                const int hi = std::max(a, b);
                int found = 0;
                for (int v = s0; v < e0; v++) {
                    if (v == u) continue;
                    const int cg = bucket[v];
                    int a2, b2; fnodes(cg / 3, cg % 3, a2, b2);
                    if (std::max(a2, b2) != hi) continue;
                    if (cg / 3 == cf / 3) { err[lo] = 2; break; }
                    if (++found > 1) { err[lo] = 3; break; }
                    partner[cf] = cg;
                }
            }
        }
    });
    for (int lo = 1; lo <= NN; lo++) {
        if (!err[lo]) continue;
        const int cf = bucket[start[lo]];
        if (err[lo] == 1) set_error("degenerate cell with node " + std::to_string(lo));
        else if (err[lo] == 2) set_error("cell " + std::to_string(cf / 3 + 1) + " repeats an edge");
        else set_error("non-manifold edge at node " + std::to_string(lo));
        return E2D_ERR_MESH;
    }
    // 4. the face that creates each edge (the first in (cell, face) order) and
    //    its class: 0 interior, 1 far field, 2 wall (the box rule of
    //    gpu_init.cu:190); -1 for a face whose edge an earlier face created
    std::vector<signed char> kind(3 * (size_t)N);
    faces.run([&](int64_t f0, int64_t f1, int) {
        for (int64_t cf = f0; cf < f1; cf++) {
            const int c = (int)(cf / 3), p = partner[cf];
            if (p >= 0) { kind[cf] = p / 3 < c ? -1 : 0; continue; }
            int a, b; fnodes(c, (int)(cf % 3), a, b);
            const double mx = 0.5 * (X[a] + X[b]), my = 0.5 * (Y[a] + Y[b]);
            kind[cf] = (std::fabs(mx) < wall_box && std::fabs(my) < wall_box) ? 2 : 1;
        }
    });
    // prefix sums of the three classes over the chunks
    std::vector<std::array<int, 3>> chunk_cnt(faces.T), chunk_off(faces.T);
    faces.run([&](int64_t f0, int64_t f1, int ch) {
        std::array<int, 3> c3 = {0, 0, 0};
        for (int64_t cf = f0; cf < f1; cf++)
            if (kind[cf] >= 0) c3[kind[cf]]++;
        chunk_cnt[ch] = c3;
    });
    std::array<int, 3> tot = {0, 0, 0};
    for (int ch = 0; ch < faces.T; ch++)
        for (int k = 0; k < 3; k++) { chunk_off[ch][k] = tot[k]; tot[k] += chunk_cnt[ch][k]; }
    const int NI = tot[0], NF = tot[1], NW = tot[2], NE = NI + NF + NW;
    t.nedge = NE; t.nwall = NW; t.nfar = NF;
    for (auto *v : {&t.elog, &t.eleft, &t.eright, &t.efar, &t.ewall, &t.en1, &t.en2}) v->assign(NE, 0);
    for (auto *v : {&t.evn, &t.evx, &t.evy, &t.emx, &t.emy}) v->assign(NE, 0.0);
    t.pre2post.assign(NE + 1, 0);
    // 5. every new edge written at its place after the partition (interior,
    //    then far, then wall; each in discovery order); face_edge = 1-based id
    std::vector<int> face_edge(3 * (size_t)N, 0);
    faces.run([&](int64_t f0, int64_t f1, int ch) {
        std::array<int, 3> r = chunk_off[ch];
        for (int64_t cf = f0; cf < f1; cf++) {
            const int kd = kind[cf];
            if (kd < 0) continue;
            const int c = (int)(cf / 3), p = partner[cf];
            const int pre = r[0] + r[1] + r[2];  // discovery order
            const int k = kd == 0 ? r[0] : kd == 1 ? NI + r[1] : NI + NF + r[2];
            int a, b; fnodes(c, (int)(cf % 3), a, b);
            t.elog[k] = kd; t.eleft[k] = c + 1; t.en1[k] = a; t.en2[k] = b;
            t.eright[k] = p >= 0 ? p / 3 + 1 : -1;
            t.efar[k] = kd == 1 ? r[1] + 1 : 0;
            t.ewall[k] = kd == 2 ? r[2] + 1 : 0;
            const double ex = X[a] - X[b], ey = Y[b] - Y[a];
            t.evx[k] = ex; t.evy[k] = ey;
            t.emx[k] = 0.5 * (X[a] + X[b]); t.emy[k] = 0.5 * (Y[a] + Y[b]);
            t.evn[k] = std::sqrt(ex * ex + ey * ey);
            t.pre2post[pre + 1] = k + 1;
            face_edge[cf] = k + 1;
            r[kd]++;
        }
    });
    faces.run([&](int64_t f0, int64_t f1, int) {
        for (int64_t cf = f0; cf < f1; cf++)
            if (kind[cf] < 0) face_edge[cf] = face_edge[partner[cf]];
    });
    // 6. per-cell tables
    t.celledge.resize(3 * (size_t)N); t.neicell.resize(3 * (size_t)N); t.clog.resize(N);
    t.nb.resize(3 * (size_t)N); t.nb_slot.resize(3 * (size_t)N); t.is_right.resize(3 * (size_t)N);
    cells.run([&](int64_t c0, int64_t c1, int) {
        for (int64_t c = c0; c < c1; c++) {
            int nn = 3;
            for (int f = 0; f < 3; f++) {
                const int64_t cf = 3 * c + f;
                const int e = face_edge[cf] - 1;
                t.celledge[cf] = e + 1;
                int nbr = t.eleft[e] == c + 1 ? t.eright[e] : t.eleft[e];
                if (nbr == -1) { nbr *= t.elog[e]; nn--; }
                t.neicell[cf] = nbr;
                t.nb[cf] = nbr > 0 ? nbr - 1 : nbr;
                t.nb_slot[cf] = partner[cf] >= 0 ? partner[cf] % 3 : 0;
                t.is_right[cf] = (uint8_t)(t.eright[e] == c + 1);
            }
            t.clog[c] = nn;
        }
    });
    t.wall_box = wall_box;
    return E2D_OK;
}

// 21 bits of v spread to the even bit positions of a 64-bit word
static inline uint64_t spread21(uint64_t v) {
    v &= 0x1fffffULL;
    v = (v | (v << 32)) & 0x1f00000000ffffULL;
    v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}

// Reverse Cuthill-McKee order of the cell adjacency graph (interior faces).
// Deterministic: each component starts at its lowest-degree cell (lowest
// index among equals), neighbours join the queue by (degree, index), and the
// whole Cuthill-McKee sequence is reversed at the end.
static void rcm_order(const MeshTopo &t, int N, std::vector<int> &perm) {
    std::vector<int> deg(N, 0), order;
    order.reserve(N);
    for (int c = 0; c < N; c++)
        for (int k = 0; k < 3; k++) deg[c] += t.nb[3 * (size_t)c + k] >= 0;
    std::vector<char> seen(N, 0);
    std::vector<int> byd(N);
    for (int i = 0; i < N; i++) byd[i] = i;
    std::stable_sort(byd.begin(), byd.end(), [&](int a, int b) { return deg[a] < deg[b]; });
    size_t next_start = 0;
    while (order.size() < (size_t)N) {
        while (seen[byd[next_start]]) next_start++;
        const int s0 = byd[next_start];
        seen[s0] = 1;
        size_t head = order.size();
        order.push_back(s0);
        while (head < order.size()) {
            const int c = order[head++];
            int nb[3], cnt = 0;
            for (int k = 0; k < 3; k++) {
                const int q = t.nb[3 * (size_t)c + k];
                if (q >= 0 && !seen[q]) { nb[cnt++] = q; seen[q] = 1; }
            }
            std::sort(nb, nb + cnt, [&](int a, int b) { return deg[a] != deg[b] ? deg[a] < deg[b] : a < b; });
            for (int k = 0; k < cnt; k++) order.push_back(nb[k]);
        }
    }
    for (int i = 0; i < N; i++) perm[i] = order[N - 1 - i];
}

void cell_order(const e2d_mesh *m, int ordering, std::vector<int> &perm) {
    const MeshTopo &t = m->topo;
    const int N = m->ncell;
    perm.resize(N);
    for (int i = 0; i < N; i++) perm[i] = i;
    if (ordering == E2D_ORDER_RCM) { rcm_order(t, N, perm); return; }
    if (ordering != E2D_ORDER_MORTON) return;
    double x0 = t.cx[0], x1 = t.cx[0], y0 = t.cy[0], y1 = t.cy[0];
    for (int i = 1; i < N; i++) {
        x0 = std::min(x0, t.cx[i]); x1 = std::max(x1, t.cx[i]);
        y0 = std::min(y0, t.cy[i]); y1 = std::max(y1, t.cy[i]);
    }
    double sx = x1 > x0 ? x1 - x0 : 1.0, sy = y1 > y0 ? y1 - y0 : 1.0;
    std::vector<uint64_t> code(N);
    for (int i = 0; i < N; i++) {
        uint64_t qx = (uint64_t)((t.cx[i] - x0) / sx * 2097151.0);
        uint64_t qy = (uint64_t)((t.cy[i] - y0) / sy * 2097151.0);
        code[i] = spread21(qx) | (spread21(qy) << 1);
    }
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return code[a] < code[b]; });
}

// ---- NACA 0012 O-grid ------------------------------------------------------

static inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

static inline double unit_rand(uint64_t seed, uint64_t stream, uint64_t idx) {
    uint64_t h = mix64(seed ^ mix64(stream * 0x632be59bd9b4e019ULL + idx));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// NACA 0012 half thickness with the closed trailing edge coefficient -0.1036
static inline double naca0012(double x) {
    x = std::min(std::max(x, 0.0), 1.0);
    return 0.6 * (0.2969 * std::sqrt(x) - 0.1260 * x - 0.3516 * x * x + 0.2843 * x * x * x -
                  0.1036 * x * x * x * x);
}

static int make_ogrid(int ni, int nj, double r_far, double dy_wall, double jitter, uint64_t seed,
                      e2d_mesh *m) {
    if (ni < 8 || nj < 1 || r_far <= 1.0 || dy_wall <= 0 || jitter < 0 || jitter >= 0.25) {
        set_error("ogrid: need ni>=8, nj>=1, r_far>1, dy_wall>0, 0<=jitter<0.25");
        return E2D_ERR_ARG;
    }
    const double pi = 3.14159265358979323846;
    std::vector<double> wx(ni), wy(ni), fx(ni), fy(ni);
    for (int i = 0; i < ni; i++) {
        double th = 2.0 * pi * i / ni;
        double x = 0.5 * (1.0 + std::cos(th));
        wx[i] = x;
        wy[i] = (2 * i <= ni ? 1.0 : -1.0) * naca0012(x);
        if (i == 0 || 2 * i == ni) wy[i] = 0.0;
        fx[i] = 0.5 + r_far * std::cos(th);
        fy[i] = r_far * std::sin(th);
    }
    // geometric stretching s_0=0 .. s_nj=1 with first step ds0
    double ds0 = dy_wall / (r_far - 0.5), ratio = 1.0;
    if (ds0 * nj < 1.0) {
        double lo = 1.0, hi = 2.0;
        auto total = [&](double r) { return ds0 * (std::pow(r, nj) - 1.0) / (r - 1.0); };
        while (total(hi) < 1.0) hi *= 2.0;
        for (int it = 0; it < 200; it++) {
            double mid = 0.5 * (lo + hi);
            (total(mid) < 1.0 ? lo : hi) = mid;
        }
        ratio = 0.5 * (lo + hi);
    } else {
        ds0 = 1.0 / nj;
    }
    std::vector<double> s(nj + 1);
    s[0] = 0.0;
    for (int j = 1; j <= nj; j++) s[j] = s[j - 1] + ds0 * std::pow(ratio, j - 1);
    for (int j = 0; j <= nj; j++) s[j] /= s[nj];
    m->nnode = ni * (nj + 1);
    m->ncell = 2 * ni * nj;
    m->x.assign(m->nnode, 0.0);
    m->y.assign(m->nnode, 0.0);
    auto P = [&](int i, int j, double &x, double &y) {
        x = wx[i] + s[j] * (fx[i] - wx[i]);
        y = wy[i] + s[j] * (fy[i] - wy[i]);
    };
    for (int j = 0; j <= nj; j++)
        for (int i = 0; i < ni; i++) {
            double x, y; P(i, j, x, y);
            if (j > 0 && j < nj && jitter > 0) {
                double h = 1e300, xa, ya;
                const int di[4] = {1, -1, 0, 0}, dj[4] = {0, 0, 1, -1};
                for (int q = 0; q < 4; q++) {
                    P((i + di[q] + ni) % ni, j + dj[q], xa, ya);
                    h = std::min(h, std::hypot(xa - x, ya - y));
                }
                uint64_t idx = (uint64_t)j * ni + i;
                x += jitter * h * (2.0 * unit_rand(seed, 1, idx) - 1.0);
                y += jitter * h * (2.0 * unit_rand(seed, 2, idx) - 1.0);
            }
            m->x[(size_t)j * ni + i] = x;
            m->y[(size_t)j * ni + i] = y;
        }
    m->tri.resize(3 * (size_t)m->ncell);
    int *t = m->tri.data();
    for (int j = 0; j < nj; j++)
        for (int i = 0; i < ni; i++) {
            int a = j * ni + i + 1, b = j * ni + (i + 1) % ni + 1;
            int c = (j + 1) * ni + (i + 1) % ni + 1, d = (j + 1) * ni + i + 1;
            // a->b->c->d runs clockwise; both triangles are written CCW
            if (unit_rand(seed, 3, (uint64_t)j * ni + i) < 0.5) {
                t[0] = a; t[1] = d; t[2] = c; t[3] = a; t[4] = c; t[5] = b;
            } else {
                t[0] = a; t[1] = d; t[2] = b; t[3] = b; t[4] = d; t[5] = c;
            }
            t += 6;
        }
    for (int c = 0; c < m->ncell; c++) {
        const int *p = &m->tri[3 * c];
        const double *x = m->x.data() - 1, *y = m->y.data() - 1;
        if (!(tri_area(x[p[0]], y[p[0]], x[p[1]], y[p[1]], x[p[2]], y[p[2]]) > 0.0)) {
            set_error("ogrid: generated a non-positive cell; lower the jitter");
            return E2D_ERR_MESH;
        }
    }
    return E2D_OK;
}

}  // namespace e2d

using namespace e2d;

extern "C" {

const char *e2d_last_error(void) { return g_error.c_str(); }

const char *e2d_version(void) { return "euler2d-gb300 0.1"; }

// Binary mesh cache: "E2DMESH1", int32 nnode, int32 ncell, double x[nnode],
// double y[nnode], int32 tri[3*ncell] (1-based node ids), little-endian.
static const char kBinMagic[8] = {'E', '2', 'D', 'M', 'E', 'S', 'H', '1'};

static int read_binary(FILE *f, e2d_mesh **out) {
    int32_t hdr[2];
    if (std::fread(hdr, sizeof(int32_t), 2, f) != 2 || hdr[0] < 3 || hdr[1] < 1) {
        set_error("bad binary mesh header"); return E2D_ERR_IO;
    }
    auto *m = new e2d_mesh;
    m->nnode = hdr[0]; m->ncell = hdr[1];
    m->x.resize(m->nnode); m->y.resize(m->nnode); m->tri.resize(3 * (size_t)m->ncell);
    bool ok = std::fread(m->x.data(), sizeof(double), m->nnode, f) == (size_t)m->nnode &&
              std::fread(m->y.data(), sizeof(double), m->nnode, f) == (size_t)m->nnode &&
              std::fread(m->tri.data(), sizeof(int32_t), m->tri.size(), f) == m->tri.size();
    if (!ok) { delete m; set_error("truncated mesh file"); return E2D_ERR_IO; }
    *out = m;
    return E2D_OK;
}

int e2d_mesh_read(const char *path, e2d_mesh **out) {
    if (!path || !out) { set_error("null argument"); return E2D_ERR_ARG; }
    *out = nullptr;
    FILE *f = std::fopen(path, "rb");
    if (!f) { set_error(std::string("cannot open the mesh data file ") + path); return E2D_ERR_IO; }
    char magic[8];
    if (std::fread(magic, 1, 8, f) == 8 && !std::memcmp(magic, kBinMagic, 8)) {
        int rc = read_binary(f, out);
        std::fclose(f);
        return rc;
    }
    std::rewind(f);
    int nnode = 0, ncell = 0;
    if (std::fscanf(f, "%d %d", &nnode, &ncell) != 2 || nnode < 3 || ncell < 1) {
        std::fclose(f); set_error("bad mesh header (need \"Nnode Ncell\")"); return E2D_ERR_IO;
    }
    auto *m = new e2d_mesh;
    m->nnode = nnode; m->ncell = ncell;
    m->x.resize(nnode); m->y.resize(nnode); m->tri.resize(3 * (size_t)ncell);
    bool ok = true;
    for (int i = 0; i < nnode && ok; i++) ok = std::fscanf(f, "%lf", &m->x[i]) == 1;
    for (int i = 0; i < nnode && ok; i++) ok = std::fscanf(f, "%lf", &m->y[i]) == 1;
    for (size_t i = 0; i < 3 * (size_t)ncell && ok; i++) ok = std::fscanf(f, "%d", &m->tri[i]) == 1;
    std::fclose(f);
    if (!ok) { delete m; set_error("truncated mesh file"); return E2D_ERR_IO; }
    *out = m;
    return E2D_OK;
}

int e2d_mesh_write(const char *path, const e2d_mesh *m) {
    if (!path || !m) { set_error("null argument"); return E2D_ERR_ARG; }
    FILE *f = std::fopen(path, "w");
    if (!f) { set_error(std::string("cannot write ") + path); return E2D_ERR_IO; }
    std::fprintf(f, "%d %d\n", m->nnode, m->ncell);
    for (int i = 0; i < m->nnode; i++) std::fprintf(f, "%.17g\n", m->x[i]);
    for (int i = 0; i < m->nnode; i++) std::fprintf(f, "%.17g\n", m->y[i]);
    for (int c = 0; c < m->ncell; c++)
        std::fprintf(f, "%d %d %d\n", m->tri[3 * c], m->tri[3 * c + 1], m->tri[3 * c + 2]);
    int bad = std::ferror(f);
    std::fclose(f);
    if (bad) { set_error("write error"); return E2D_ERR_IO; }
    return E2D_OK;
}

int e2d_mesh_write_binary(const char *path, const e2d_mesh *m) {
    if (!path || !m) { set_error("null argument"); return E2D_ERR_ARG; }
    FILE *f = std::fopen(path, "wb");
    if (!f) { set_error(std::string("cannot write ") + path); return E2D_ERR_IO; }
    const int32_t hdr[2] = {m->nnode, m->ncell};
    bool ok = std::fwrite(kBinMagic, 1, 8, f) == 8 && std::fwrite(hdr, sizeof(int32_t), 2, f) == 2 &&
              std::fwrite(m->x.data(), sizeof(double), m->nnode, f) == (size_t)m->nnode &&
              std::fwrite(m->y.data(), sizeof(double), m->nnode, f) == (size_t)m->nnode &&
              std::fwrite(m->tri.data(), sizeof(int32_t), m->tri.size(), f) == m->tri.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) { set_error("write error"); return E2D_ERR_IO; }
    return E2D_OK;
}

int e2d_mesh_from_arrays(int32_t nnode, int32_t ncell, const double *x, const double *y,
                         const int32_t *tri, e2d_mesh **out) {
    if (!x || !y || !tri || !out || nnode < 3 || ncell < 1) { set_error("bad mesh arrays"); return E2D_ERR_ARG; }
    auto *m = new e2d_mesh;
    m->nnode = nnode; m->ncell = ncell;
    m->x.assign(x, x + nnode); m->y.assign(y, y + nnode);
    m->tri.assign(tri, tri + 3 * (size_t)ncell);
    *out = m;
    return E2D_OK;
}

int e2d_mesh_ogrid_naca0012(int32_t ni, int32_t nj, double r_far, double dy_wall, double jitter,
                            uint64_t seed, e2d_mesh **out) {
    if (!out) { set_error("null argument"); return E2D_ERR_ARG; }
    *out = nullptr;
    auto *m = new e2d_mesh;
    int rc = make_ogrid(ni, nj, r_far, dy_wall, jitter, seed, m);
    if (rc) { delete m; return rc; }
    *out = m;
    return E2D_OK;
}

void e2d_mesh_free(e2d_mesh *m) { delete m; }

int e2d_mesh_info_get(e2d_mesh *m, double wall_box, e2d_mesh_info *info) {
    if (!m || !info) { set_error("null argument"); return E2D_ERR_ARG; }
    int rc = build_topology(m, wall_box);
    if (rc) return rc;
    info->ncell = m->ncell; info->nnode = m->nnode; info->nedge = m->topo.nedge;
    info->nwall = m->topo.nwall; info->nfar = m->topo.nfar;
    return E2D_OK;
}

int e2d_mesh_topology(e2d_mesh *m, double wall_box, int32_t *ei, double *ed, int32_t *ci, double *cd) {
    if (!m) { set_error("null argument"); return E2D_ERR_ARG; }
    int rc = build_topology(m, wall_box);
    if (rc) return rc;
    const MeshTopo &t = m->topo;
    for (int e = 0; e < t.nedge; e++) {
        if (ei) {
            int32_t *o = ei + 7 * (size_t)e;
            o[0] = t.elog[e]; o[1] = t.eleft[e]; o[2] = t.eright[e]; o[3] = t.efar[e];
            o[4] = t.ewall[e]; o[5] = t.en1[e]; o[6] = t.en2[e];
        }
        if (ed) {
            double *o = ed + 5 * (size_t)e;
            o[0] = t.evn[e]; o[1] = t.evx[e]; o[2] = t.evy[e]; o[3] = t.emx[e]; o[4] = t.emy[e];
        }
    }
    for (int c = 0; c < m->ncell; c++) {
        if (ci) {
            int32_t *o = ci + 7 * (size_t)c;
            o[0] = t.clog[c];
            for (int f = 0; f < 3; f++) { o[1 + f] = t.celledge[3 * c + f]; o[4 + f] = t.neicell[3 * c + f]; }
        }
        if (cd) { cd[3 * c] = t.area[c]; cd[3 * c + 1] = t.cx[c]; cd[3 * c + 2] = t.cy[c]; }
    }
    return E2D_OK;
}

int e2d_mesh_nodes(const e2d_mesh *m, double *x, double *y, int32_t *tri) {
    if (!m) { set_error("null argument"); return E2D_ERR_ARG; }
    if (x) std::memcpy(x, m->x.data(), sizeof(double) * m->nnode);
    if (y) std::memcpy(y, m->y.data(), sizeof(double) * m->nnode);
    if (tri) std::memcpy(tri, m->tri.data(), sizeof(int32_t) * 3 * (size_t)m->ncell);
    return E2D_OK;
}

int e2d_mesh_order(e2d_mesh *m, int32_t ordering, int32_t *perm) {
    if (!m || !perm) { set_error("null argument"); return E2D_ERR_ARG; }
    if (ordering != E2D_ORDER_FILE && ordering != E2D_ORDER_MORTON && ordering != E2D_ORDER_RCM) {
        set_error("unknown ordering");
        return E2D_ERR_ARG;
    }
    double wb = m->topo.wall_box >= 0 ? m->topo.wall_box : 2.0;
    int rc = build_topology(m, wb);
    if (rc) return rc;
    std::vector<int> p;
    cell_order(m, ordering, p);
    std::memcpy(perm, p.data(), sizeof(int32_t) * p.size());
    return E2D_OK;
}

int e2d_params_default(e2d_params *p) {
    if (!p) { set_error("null argument"); return E2D_ERR_ARG; }
    std::memset(p, 0, sizeof *p);
    p->ma = 0.5; p->alpha_deg = 0.0; p->gamma = 1.4; p->pin = 101325.0; p->tin = 288.15;
    p->cfl = 1.0; p->epsl = 1e-6; p->maxstep = 100;
    p->rk_stages = 4;
    p->rk_coef[0] = 0.0833; p->rk_coef[1] = 0.2069; p->rk_coef[2] = 0.4265; p->rk_coef[3] = 1.0;
    p->irs_eps = 0.8; p->irs_sweeps = 2; p->precision = E2D_FP64;
    p->dt_cap = 0.1; p->entropy_eps = 0.05; p->wall_box = 2.0;
    p->ordering = E2D_ORDER_FILE; p->block_size = 0; p->graph_iters = 0; p->verbose = 0;
    p->limiter_freeze = 0; p->limiter = E2D_LIMITER_REFERENCE; p->limiter_k = 5.0;
    return E2D_OK;
}

int e2d_input_read(const char *path, e2d_params *p) {
    if (!path || !p) { set_error("null argument"); return E2D_ERR_ARG; }
    FILE *f = std::fopen(path, "r");
    if (!f) { set_error(std::string("cannot open input file ") + path); return E2D_ERR_IO; }
    int n = std::fscanf(f, "%lf %lf %lf %lf %lf %lf %lf %d", &p->ma, &p->alpha_deg, &p->gamma, &p->pin,
                        &p->tin, &p->cfl, &p->epsl, &p->maxstep);
    std::fclose(f);
    if (n != 8) { set_error("input file needs 8 values: MA ALPHA GAMA PIN TIN CFL EPSL MAXSTEP"); return E2D_ERR_IO; }
    return E2D_OK;
}

}  // extern "C"
