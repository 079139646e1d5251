// The particle-grid transfer's device passes: what the host plan hands the
// kernels, and the launchers (transfer_kernels.cu) the host plan calls.
//
// The projection (P S)_n = (1/w_n) int_{element(n)} S phi_n runs three
// rules (src/transfer.jl:1-35): the far rule and the graded bands are tensor
// Gauss rules, one CTA per element evaluating S at its q^D points into shared
// memory and contracting them there one dimension at a time (the reference's
// two passes, source_points / contract, fused, so the points never reach
// HBM); the nested rule near a particle runs over the host's point list,
// which comes in innermost lines (the points that share all coordinates but
// the last): a line's points are summed against the last dimension's Lagrange
// polynomials into P+1 numbers, and one outer product with the other
// dimensions' polynomials at the line's fixed coordinates adds them to the
// element's nodes, so that the per-point work is one Lagrange evaluation and
// P+1 multiply-adds instead of D evaluations and (P+1)^D (the reference's
// near_partials_kernel!). Lines are taken in chunks of one element's lines,
// whose per-node sums are added in order by a second kernel.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace twoldg {

constexpr int kNearLines = 64;    // lines per chunk, at most
constexpr int kMaxParticles = 8;

// One particle of the built-in density source rho(x) = Q rho0(|L(v)(x - z)|^2,
// ell) (src/particle.jl:117-127), with the boost's g = gamma^2 / (gamma + 1).
struct TransferParticle {
    double z[3], v[3], ell, charge, g;
};

// A tensor rule element (far or graded): its block, its element index per
// dimension, its rule and where its points' values start.
struct RuleElement {
    int32_t block, e[3], rule, pad;
    int64_t base;
};

// A near element: block, element, its chunks [c0, c1).
struct NearElement {
    int32_t block, e[3], c0, c1;
};

// An innermost line of the nested rule: its points [p0, p1); its fixed
// coordinates and the product of the outer lines' weights sit in line_vals.
struct NearLine {
    int32_t p0, p1;
};

// A chunk of lines [l0, l1) of near element `elem`.
struct NearChunk {
    int32_t l0, l1, elem, pad;
};

enum { SOURCE_VALUES = 0, SOURCE_DENSITY = 1 };

// Everything the kernels read, device pointers in the field type T
// (`prec` 0: double, 1: float).
struct TransferLaunch {
    int prec = 0, D = 3, P = 3, E = 2, N = 8;
    int64_t NN = 0;             // N^D
    const void* origins = nullptr;   // nblocks x D, T
    const void* spacings = nullptr;  // nblocks, T
    // tensor rules: per rule its q, the offset of its nodes (q) and of its
    // contraction ((P+1) x q) in `tables`
    int nrules = 0;
    int rule_q[16] = {0};
    int rule_nodes[16] = {0};
    int rule_contract[16] = {0};
    int max_q = 0;
    const void* tables = nullptr;    // T
    const RuleElement* rule_elems = nullptr;   // grouped by rule
    int64_t n_rule_elems = 0;
    int64_t rule_start[17] = {0};              // rule r's elements: [rule_start[r], rule_start[r+1])
    // nested rule
    const void* near_lx = nullptr;   // per point its last coordinate, T
    const void* near_lw = nullptr;   // per point its last line's weight, T
    const NearLine* lines = nullptr;
    const void* line_vals = nullptr; // per line: its fixed coordinates (2) and outer weight, T
    int64_t n_lines = 0;
    const NearChunk* chunks = nullptr;
    int64_t n_chunks = 0;
    const NearElement* near_elems = nullptr;
    int64_t n_near_elems = 0;
    int64_t near_base = 0;           // index of the first near point among all points
    const void* bary = nullptr;      // P+1, T
    const void* gll = nullptr;       // P+1 Gauss-Lobatto nodes, T
    const void* wn = nullptr;        // (P+1)^D node weights of a finest element, T
    void* partials = nullptr;        // n_chunks x (P+1)^D, T
    // the source
    int source = SOURCE_VALUES;
    const void* values = nullptr;    // all points' values, T (SOURCE_VALUES)
    int nparticles = 0;
    TransferParticle particles[kMaxParticles];
    // the output: du[var] += factor * P S
    void* du = nullptr;
    int var = 1;
    double factor = 1.0;
};

// The averaging over shared nodes (average_shared!, src/transfer.jl:1616-1714):
// the ball's blocks and, per block and dimension, the block across its upper
// face (-1 for none: outside the ball's blocks, on another level, or past
// the domain).
struct AverageLaunch {
    int prec = 0, D = 3, P = 3, E = 2, N = 8;
    int64_t NN = 0;
    const int32_t* blocks = nullptr;
    const int32_t* upper = nullptr;   // nblocks_ball x 3
    int64_t nball = 0;
    void* u = nullptr;
    int var = 2;
};

cudaError_t launch_average(const AverageLaunch& a, cudaStream_t stream);

// The pairing (pairing, src/transfer.jl:1779-1797) of each particle's kernel
// K = (grad rho, rho) (density_kernel, src/dynamic.jl:124-135) with a field:
// int K g_h = sum_m g_m mu_m over the elements that meet the support, where
// mu_m = int K phi_m are the kernel's moments, fixed while the particles do
// not move. They are computed once per set of positions, in FP64 whatever the
// field type, from the nested rule kept to the support (compact), in innermost
// lines as the projection's; each pairing after that is one gather of the
// elements' nodal values (averaged over the elements that share a node, for
// the continuous pairing) and one dot product per particle.
constexpr int kPairComponents = 4;   // d rho / dx_d for d < 3, then rho

// A support element: its box, its particle and its chunks of lines.
struct PairElement {
    double lo[3], hi[3];
    int32_t particle, c0, c1, pad;
};

struct PairingLaunch {
    int prec = 0, P = 3, N = 8;
    int64_t NN = 0;
    int nparticles = 0;
    TransferParticle particles[kMaxParticles];
    int32_t first[kMaxParticles + 1] = {0};   // particle k's elements: [first[k], first[k+1])
    const PairElement* elems = nullptr;
    int64_t n_elems = 0;
    const NearLine* lines = nullptr;
    const double* lx = nullptr;         // per point its last coordinate
    const double* lw = nullptr;         // per point its last line's weight
    const double* line_vals = nullptr;  // per line: fixed coordinates (2), outer weight
    const NearChunk* chunks = nullptr;  // chunk.elem indexes elems
    int64_t n_chunks = 0;
    const double* bary = nullptr;       // P+1
    const double* gll = nullptr;        // P+1
    double* partials = nullptr;         // n_chunks x 4 x (P+1)^3
    double* moments = nullptr;          // n_elems x 4 x (P+1)^3
    // per element and node the state offsets (of variable 1) of the values
    // averaged there, kGather of them, -1 past the last
    const int64_t* gather = nullptr;
    const void* u = nullptr;
    int var = 1;
    double* out = nullptr;              // nparticles x 4
};
constexpr int kGather = 8;

// The moments of every support element, on `stream`.
cudaError_t launch_pairing_moments(const PairingLaunch& a, cudaStream_t stream);
// The pairings with a.u through a.gather into a.out, on `stream`.
cudaError_t launch_pairing_dot(const PairingLaunch& a, cudaStream_t stream);

// The projection's kernels: the far rule on `far`, the graded bands on
// `bands`, the nested rule on `near` (they write disjoint elements, so the
// three may run at once); returns the launch error, if any.
cudaError_t launch_projection(const TransferLaunch& a, cudaStream_t far, cudaStream_t bands, cudaStream_t near);

// Every point of the plan's rules, tensor rules first (element by element,
// dimension 0 fastest), then the near points, as (D, npoints) in T.
cudaError_t launch_points(const TransferLaunch& a, void* xs, int64_t npoints, cudaStream_t stream);

}  // namespace twoldg
