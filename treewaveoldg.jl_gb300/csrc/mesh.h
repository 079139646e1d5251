// The mesh compiler: from a forest's leaves (level, integer corner) to the
// per-block work items and the coarse-fine face list the kernels read.
#pragma once
#include <string>
#include <vector>

#include "../../include/twoldg.h"
#include "kernels_types.h"

namespace twoldg {

struct Mesh {
    int D = 0, P = 0, E = 0, N = 0, nblocks = 0;
    int64_t NN = 0;                    // nodes per block
    std::vector<double> h;             // spacing per block
    std::vector<BlockItem> items;      // one per block, in the caller's order
    std::vector<CfFace> cf;            // coarse-fine faces (both sides)
    double hmin = 0;
    int nwall = 0, nsame = 0;          // face counts, for tests and logs
};

// Validates `d` and builds the mesh. On failure returns false with a
// message in `err` naming the offending block or field.
bool build_mesh(const twoldg_desc& d, Mesh& m, std::string& err);

}  // namespace twoldg
