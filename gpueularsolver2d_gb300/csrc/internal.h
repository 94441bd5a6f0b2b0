// internal.h -- host-side structures shared by the translation units of
// libeuler2d.so.  Not part of the public ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/euler2d.h"

namespace e2d {

void set_error(const std::string &msg);

// Mesh as read from a reference .dat file plus its set-up, which is built on
// first use and cached for one wall_box value.
struct MeshTopo {
    double wall_box = -1.0;
    int nedge = 0, nwall = 0, nfar = 0;
    // edges in reference numbering after the changeEdge partition; 0-based
    // arrays, 1-based ids inside (left/right/node ids, far/wall ids)
    std::vector<int> elog, eleft, eright, efar, ewall, en1, en2;
    std::vector<double> evn, evx, evy, emx, emy;
    // cells, 0-based arrays
    std::vector<double> area, cx, cy;
    std::vector<int> clog;
    std::vector<int> celledge, neicell;  // [3*ncell], reference ids
    // edge id before the changeEdge partition (discovery order, as
    // CalculationMeshGeo leaves it) -> id after it; both 1-based
    std::vector<int> pre2post;           // [nedge+1]
    // per cell face: 0-based neighbour cell (-1 far, -2 wall), whether this
    // cell is the edge's right cell, and the face slot of the neighbour
    std::vector<int> nb, nb_slot;
    std::vector<uint8_t> is_right;
};

}  // namespace e2d

struct e2d_mesh {
    int nnode = 0, ncell = 0;
    std::vector<double> x, y;  // [nnode]
    std::vector<int> tri;      // [3*ncell], 1-based node ids (file order)
    e2d::MeshTopo topo;
};

namespace e2d {

// Builds (or reuses) the set-up of m for the given wall box; 0 or error code.
int build_topology(e2d_mesh *m, double wall_box);
// Internal cell order: perm[k] = file index of the cell at position k.
void cell_order(const e2d_mesh *m, int ordering, std::vector<int> &perm);

}  // namespace e2d
