// solver_internal.h -- host-side helpers shared by the single-case solver
// (solver.cu) and the batched solver (batch.cu).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "internal.h"

namespace e2d {

// Free-stream constants exactly as Initialization computes them
// (gpu_init.cu:63-93), including PIS = P of the free-stream cell state.
struct FreeStream {
    double alpha, ain, vin, ui, vi, rho_e, pis;
    double ain_test;  // sound speed of the far-field supersonic test (ain, or 1/M with the fix)
};

FreeStream free_stream(const e2d_params &p);

// Cell-local layout in FP64, internal order.
struct HostLayout {
    int n = 0;
    std::vector<int> perm, iperm;        // internal -> file, file -> internal
    std::vector<int32_t> topo;           // [4n]
    std::vector<double> S, R;            // [3n*2] each
    std::vector<double> area;            // [n]
    std::vector<int> wall_cell, wall_k;  // internal cell and face of every wall face
};

int build_layout(e2d_mesh *m, const e2d_params &p, HostLayout &L);

// CL, CD from a file-order state (see e2d_forces).
void forces_from_state(const HostLayout &L, const FreeStream &fs, double gamma, const double *w_file,
                       double *cl, double *cd);

// CL, CD, total mass and boundary mass fluxes of a file-order state (see
// e2d_integrals), all in FP64.
void integrals_from_state(const HostLayout &L, const FreeStream &fs, const e2d_params &p, const double *w_file,
                          e2d_integrals *out);

// Parameter checks shared by the solver constructors.
// Null when the parameters are usable, else which one is not.
const char *param_error(const e2d_params *p);

// Marks [base, base + bytes) as persisting in L2 for every kernel node of a
// captured graph (the cell topology, which all four passes read).
// L2 persistence of a graph's topology reads; *held marks the owner as a user
// of the persisting carve-out until release_l2(held) (at its destruction).
void keep_in_l2(cudaGraph_t g, const void *base, size_t bytes, bool *held);
void release_l2(bool *held);

// Device arena: one cudaMalloc carved into 256-byte aligned pieces.
struct Arena {
    char *base = nullptr;
    size_t cap = 0, used = 0;
    ~Arena() { if (base) cudaFree(base); }
    static size_t up(size_t b) { return (b + 255) & ~(size_t)255; }
    void *take(size_t b) { void *p = base + used; used += up(b); return p; }
};

}  // namespace e2d
