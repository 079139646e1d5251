// Plain work-item structs shared by the host set-up and the kernels.
#pragma once
#include <stdint.h>

namespace twoldg {

// One mesh block as a work item of the stage and energy kernels.
struct BlockItem {
    int64_t off;        // word offset of the block's u in the state arrays
    int32_t slot;       // face slot of this block's face 0; face f is slot + f
    int32_t nb[6];      // face slot whose exports give face f's ghosts
    uint32_t flags;     // bit f: face f is dense (coarse-fine); bit 8+f: gradient ghost odd
    int32_t problem;    // index into the per-problem time steps
    uint32_t orient;    // 3 bits per face: the face plane's orientation across a glue
    double h;           // the block's spacing
};

// A coarse-fine face: its ghosts are an I or R image of the other side.
struct CfFace {
    int32_t slot;       // the face slot whose ghosts this fills
    int32_t kind;       // 0: fine ghost from coarse (I), 1: coarse ghost from fine (R)
    int32_t src[4];     // kind 0: src[0] the coarse face; kind 1: fine faces by child bits
    int32_t sub;        // kind 0: bit k = which half of the coarse face along tangential dim k
    int32_t side;       // 0 low face, 1 high face
    double h;           // spacing of the block owning `slot`
};

// Dirichlet data a caller supplies for the boundary faces of a full-metric
// problem (boundary kind 2): level k holds, for every boundary face j (the
// faces with no neighbour, in slot order) and its tangential node t, u and
// then the three Cartesian components of its gradient at time t0 + k / inv_half,
// values[((k * nbf + j) * 4 + c) * F + t].
struct BoundaryTable {
    const double* values;
    int32_t nlevels;
    int32_t nbf;
    double t0;
    double inv_half;    // 2 / dt: two levels per step (t_n + dt/2 and t_n + dt)
};

// One block of a regrid transfer: the new block at dst (words), from the old
// leaf src[0] (copy), from its parent src[0] as child `sub` (bit d: the
// upper half along d; refine), or from its 2^D children src[bits] (coarsen).
struct TransferItem {
    int64_t dst;
    int64_t src[8];
    int32_t mode;       // 0 copy, 1 refine, 2 coarsen
    int32_t sub;
};

}  // namespace twoldg
