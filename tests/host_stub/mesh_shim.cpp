// Test infrastructure only: the mesh compiler (csrc/mesh.cpp, host code with
// no device calls) built into a library of its own, with one entry point that
// copies out what it compiled, so that the CPU tests can check its neighbour
// and coarse-fine face tables against a geometric search. The product never
// links it.
#include <cstring>
#include <string>

#include "../../treewaveoldg.jl_gb300/csrc/mesh.h"

extern "C" {

// Builds the mesh of `d`. On success writes per block its six face
// neighbours' slots (nb, nblocks x 6) and flags, the number of coarse-fine
// faces, and per such face (slot, kind, src[0..3], sub, side) into cf (up to
// cap faces); returns 0. On failure writes the message into err and returns 1.
int mesh_tables(const twoldg_desc* d, int32_t* nb, uint32_t* flags, int32_t* ncf, int32_t* cf, int32_t cap,
                char* err, int32_t errlen) {
    twoldg::Mesh m;
    std::string e;
    if (!twoldg::build_mesh(*d, m, e)) {
        std::strncpy(err, e.c_str(), (size_t)errlen - 1);
        err[errlen - 1] = 0;
        return 1;
    }
    for (int b = 0; b < m.nblocks; ++b) {
        for (int f = 0; f < 6; ++f) nb[b * 6 + f] = m.items[b].nb[f];
        flags[b] = m.items[b].flags;
    }
    *ncf = (int32_t)m.cf.size();
    for (int32_t i = 0; i < *ncf && i < cap; ++i) {
        const twoldg::CfFace& c = m.cf[i];
        const int32_t row[8] = {c.slot, c.kind, c.src[0], c.src[1], c.src[2], c.src[3], c.sub, c.side};
        std::memcpy(cf + 8 * i, row, sizeof row);
    }
    return 0;
}

}  // extern "C"
