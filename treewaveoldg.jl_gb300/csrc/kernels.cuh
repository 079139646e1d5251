// Device code of the OLDG field step: one mesh block per CTA.
//
// State layout is the reference's (N^D, 2, nblocks), column-major, u then v
// per block (src/stepping.jl:24-25): block b's u starts at b * 2 N^D, its v
// N^D words later. Every kernel is templated on the field type T (float or
// double), the dimension D and the element order P, so that the element
// line contractions unroll with constant coefficients.
//
// Ghosts: the wide derivative (src/evolution.jl:24-35) reads one node past
// its element along the dimension it differentiates, so a block needs its
// neighbours' face nodes of u ("u ghosts") and, for the second application,
// their face values of D_d u ("gradient ghosts"), faces only. Each stage
// kernel exports, per block face, the face node of u (`fu`) and the part of
// the face node's wide derivative that reads the block's own element
// (`fog`, "own gradient"). A neighbour's gradient ghost is then
//     (fog_nb + Wg * (the neighbour's own u ghost)) / h_nb,
// and for a same-level or wall face that u ghost is this block's own face
// node, so a stage needs only the previous stage's face exports and no
// separate exchange pass. Coarse-fine faces are "dense": one small kernel
// (cf_ghost_kernel) fills both their ghost planes through the element-local
// prolongation I and restriction R before the stage kernel runs.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <utility>

#include "kernels_types.h"

namespace twoldg {

constexpr int kMaxD = 3;

enum : int { MODE_RHS = 0, MODE_STAGE1 = 1, MODE_STAGE4 = 4, MODE_ENERGY = 5 };

template <typename T, int P>
struct Tab {
    T W[P + 1][P + 3];   // wide derivative per h, columns are nodes -1 .. P+1
    T tm[P + 1];         // topmode
    T td[P + 1];         // topdual
    T wq[P + 1];         // Gauss-Lobatto weights on [-1, 1]
};

template <typename T, int P>
struct CfTab {
    T I[2 * (P + 1)][P + 1];
    T R[P + 1][2 * (P + 1)];
};

template <typename T>
struct StageArgs {
    const BlockItem* items;
    int nitems;
    int E;
    int mode;
    int truncate;
    T* u;            // u^n (stages) or the rhs input; receives u^{n+1} at stage 4
    T* y;            // stage value
    T* acc;          // increments accumulated over stages 1..3
    T* comp;         // compensation words (compensated float path)
    T* du;           // rhs output
    const T* fu_in;
    const T* fog_in;
    T* fu_out;
    T* fog_out;
    const T* ugd;    // dense u ghosts (coarse-fine faces)
    const T* ggd;    // dense gradient ghosts (coarse-fine faces)
    const T* rk;     // per problem: dt/6, dt/3, dt/2, dt, rounded once to T on the host
    double* partial; // energy: one sum per item
    // diagonal metric (NULL: flat): per item (N^D, 1 + D) node values sqrt(g), A_1..A_D,
    // and the per-line truncation pairs (P+1, E, nitems, D)
    const T* coef;
    const T* trm;
    const T* trd;
    // coarse-fine faces whose ghost planes the 3D register-line kernel
    // writes in its epilogue for the next stage (the faces and, per face
    // slot, the face's index among them; NULL where ugd and ggd are filled
    // by a launch of their own): gsd is this block's own part of the
    // gradient ghost, which adds to ggd, the other side's; the *_out planes
    // are the next stage's
    const CfFace* cf;
    const int* cfidx;
    const T* gsd;
    T* ugd_out;
    T* ggd_out;
    T* gsd_out;
    // under a programmatic dependent launch: 1 where the stage kernel lets
    // the next one launch from its start, 0 where it does so at its end
    int release;
};

__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

// Coordinates helpers. Owned node n = x0 + N x1 + N^2 x2.
template <int D>
struct Geo {
    int N, S, NN, F, SS;
    __device__ Geo(int N_) : N(N_), S(N_ + 2) {
        NN = 1; F = 1; SS = 1;
        for (int k = 0; k < D; ++k) { NN *= N; SS *= S; }
        for (int k = 0; k < D - 1; ++k) F *= N;
    }
    __device__ int sstride(int d) const { int s = 1; for (int k = 0; k < d; ++k) s *= S; return s; }
    __device__ int ostride(int d) const { int s = 1; for (int k = 0; k < d; ++k) s *= N; return s; }
    // owned linear index -> padded smem index
    __device__ int sidx_of_owned(int n) const {
        int r = 0, s = 1;
        for (int k = 0; k < D; ++k) { r += (n % N + 1) * s; n /= N; s *= S; }
        return r;
    }
    // face tangential index t of a face normal to d, with x_d given -> padded smem index
    __device__ int sidx_face(int d, int t, int xd) const {
        int r = 0, s = 1;
        for (int k = 0; k < D; ++k) {
            int x;
            if (k == d) x = xd; else { x = t % N; t /= N; }
            r += (x + 1) * s;
            s *= S;
        }
        return r;
    }
    // owned index of a face node
    __device__ int oidx_face(int d, int t, int xd) const {
        int r = 0, s = 1;
        for (int k = 0; k < D; ++k) {
            int x;
            if (k == d) x = xd; else { x = t % N; t /= N; }
            r += x * s;
            s *= N;
        }
        return r;
    }
};

// ---------------------------------------------------------------------------
// Element-line contractions with the stencil's structural zeros skipped:
// row i reads columns 1..P+1 (its element) except the diagonal i+1, which is
// zero; only row 0 reads column 0 and only row P column P+2 (the faces).
template <typename T, int P>
__device__ __forceinline__ void line_derivative(const Tab<T, P>& tb, const T (&w)[P + 3], T (&out)[P + 1]) {
#pragma unroll
    for (int i = 0; i <= P; ++i) {
        T acc = T(0);
#pragma unroll
        for (int k = 0; k < P + 3; ++k) {
            if (k == i + 1) continue;
            if (k == 0 && i != 0) continue;
            if (k == P + 2 && i != P) continue;
            acc += tb.W[i][k] * w[k];
        }
        out[i] = acc;
    }
}

// Own-element part of the face row: low face row 0 over columns 1..P+1, high
// face row P over columns 1..P+1, applied to the element's P+1 nodes.
template <typename T, int P>
__device__ __forceinline__ T own_face_part(const Tab<T, P>& tb, int side, const T (&e)[P + 1]) {
    T acc = T(0);
    if (side == 0) {
#pragma unroll
        for (int k = 1; k <= P + 1; ++k) if (k != 1) acc += tb.W[0][k] * e[k - 1];
    } else {
#pragma unroll
        for (int k = 1; k <= P + 1; ++k) if (k != P + 1) acc += tb.W[P][k] * e[k - 1];
    }
    return acc;
}

template <typename T, int P>
__device__ __forceinline__ T ghost_coef(const Tab<T, P>& tb, int side) {
    return side == 0 ? tb.W[0][0] : tb.W[P][P + 2];
}

// Programmatic dependent launch (sm_90 and later). A stage or pass kernel
// launched with the programmatic-serialization attribute may become resident
// while the kernel before it on the stream finishes its last CTAs: it waits
// (griddepcontrol.wait: the earlier grid complete, its writes visible) before
// it reads anything that grid wrote, and may let the kernel after it do the
// same from its start (griddepcontrol.launch_dependents, which releases the
// next grid only once every CTA of this one has started or exited, so that
// the next grid never keeps this one's CTAs from their SMs; without it the
// release comes as each CTA exits). Without the attribute both are no-ops.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dependents_launch() { asm volatile("griddepcontrol.launch_dependents;" ::); }

// A launch of `kern`, with the programmatic-serialization attribute when
// `pdl` is set (the kernel then waits on its start as above).
template <typename... KP, typename... A>
inline cudaError_t launch_kernel(void (*kern)(KP...), int grid, int threads, size_t smem, cudaStream_t s, bool pdl,
                                 A&&... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}

// Whether a stage grid under a programmatic dependent launch lets the next
// one launch from its start: when it runs more than one wave (the next
// grid's CTAs then take only the SMs its last wave leaves) or fills at most
// half the SMs. A grid in between keeps the next grid's waiting CTAs beside
// its own all the time it runs, which measured slower than a release at its
// end (the nested reflecting box: 36.2 against 41.9 us a step), while the
// 256^3 box and the 2D quarter-period box run 3 and 11 % faster with the
// early release than with the release at the end.
template <typename K>
inline int release_early(K kern, int grid, int threads, size_t smem) {
    int dev = 0, nsm = 0, r = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kern, threads, smem);
    return grid > r * nsm || 2 * grid <= nsm;
}

// Bulk prefetch of a contiguous range into L2 (cp.async.bulk.prefetch.L2,
// sm_90 and later): one instruction per 64 KiB, no registers or shared memory
// held, nothing to wait for. The instruction wants a 16-byte aligned start
// and a multiple of 16 bytes; other ranges are left to the plain loads.
__device__ __forceinline__ void prefetch_l2(const void* p, size_t bytes) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    if ((a & 15) || (bytes & 15)) return;
    for (size_t o = 0; o < bytes; o += 65536) {
        const uint32_t n = (uint32_t)(bytes - o < 65536 ? bytes - o : 65536);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a + o), "r"(n) : "memory");
    }
}

// The prefetches of one block's stage: its own RK operands (the stage input
// y, u^n, the accumulator and the compensation, as far as the stage reads
// them) and the next block this CTA takes, so that DRAM streams while the
// CTA computes. One thread issues them.
template <typename T>
__device__ __forceinline__ void prefetch_stage(const StageArgs<T>& a, int item, int64_t words) {
    const int mode = a.mode;
    const T* ysrc = (mode == MODE_RHS || mode == MODE_STAGE1) ? a.u : a.y;
    const int64_t off = a.items[item].off;
    const size_t b = (size_t)words * sizeof(T);
    prefetch_l2(ysrc + off, b);
    if (mode != MODE_RHS && mode != MODE_STAGE1) {
        prefetch_l2(a.u + off, b);
        prefetch_l2(a.acc + off, b);
        if (mode == MODE_STAGE4 && a.comp) prefetch_l2(a.comp + off, b);
    }
    const int nxt = item + gridDim.x;
    if (nxt < a.nitems) prefetch_l2(ysrc + a.items[nxt].off, b);
}

// Error-free sum (Knuth's TwoSum).
template <typename T>
__device__ __forceinline__ void two_sum(T a, T b, T& s, T& e) {
    s = a + b;
    T bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// ---------------------------------------------------------------------------
// Face export of an arbitrary state (rk4 start, rhs, energy): per block face
// the face node of u and the own part of its wide derivative.
template <typename T, int D, int P>
__global__ void export_faces_kernel(const BlockItem* items, int nitems, int E, const T* u, T* fu,
                                    T* fog, Tab<T, P> tb) {
    Geo<D> g(E * (P + 1));
    const int perblock = 2 * D * g.F;
    int64_t total = (int64_t)nitems * perblock;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        int b = (int)(i / perblock);
        int r = (int)(i % perblock);
        int f = r / g.F, t = r % g.F;
        int d = f >> 1, side = f & 1;
        const BlockItem& it = items[b];
        const T* ub = u + it.off;
        int sd = g.ostride(d);
        int x0 = side == 0 ? 0 : g.N - 1 - P;
        int base = g.oidx_face(d, t, x0);
        T e[P + 1];
#pragma unroll
        for (int k = 0; k <= P; ++k) e[k] = ub[base + k * sd];
        int slot = it.slot + f;
        fu[(int64_t)slot * g.F + t] = side == 0 ? e[0] : e[P];
        fog[(int64_t)slot * g.F + t] = own_face_part<T, P>(tb, side, e);
    }
}

// ---------------------------------------------------------------------------
// Coarse-fine ghosts. Tangential dims of a face normal to d are the other
// dims in increasing order; a face's tangential index t has the first of
// them fastest.
// The restriction R = M_c^-1 I^T M_f at a coarse face node n (tangential
// coordinates in the coarse face) from the fine face plane `fine` (row
// stride N) that covers it: its coarse element's 2(P+1) fine nodes along
// each tangential dimension.
template <typename T, int DT, int P>
__device__ __forceinline__ T restrict_at(const CfTab<T, P>& ct, const int* n, int N, int halfE, const T* fine) {
    constexpr int P1 = P + 1;
    if constexpr (DT == 0) {
        return fine[0];
    } else if constexpr (DT == 1) {
        const int ec = n[0] / P1, j = n[0] % P1, fb = 2 * (ec % halfE) * P1;
        T acc = T(0);
#pragma unroll
        for (int r = 0; r < 2 * P1; ++r) acc += ct.R[j][r] * fine[fb + r];
        return acc;
    } else {
        const int ec0 = n[0] / P1, j0 = n[0] % P1, fb0 = 2 * (ec0 % halfE) * P1;
        const int ec1 = n[1] / P1, j1 = n[1] % P1, fb1 = 2 * (ec1 % halfE) * P1;
        T acc = T(0);
#pragma unroll
        for (int r1 = 0; r1 < 2 * P1; ++r1) {
            T a = T(0);
#pragma unroll
            for (int r0 = 0; r0 < 2 * P1; ++r0) a += ct.R[j0][r0] * fine[(fb0 + r0) + N * (fb1 + r1)];
            acc += ct.R[j1][r1] * a;
        }
        return acc;
    }
}

// The prolongation I at a fine face node n (tangential coordinates in the
// fine face) from the coarse face plane `coarse` (row stride N): the degree-P
// polynomial of the coarse element over it; q's bit k says which half of the
// coarse face the fine face covers along tangential dimension k, in units of
// halfE coarse elements.
template <typename T, int DT, int P>
__device__ __forceinline__ T prolong_at(const CfTab<T, P>& ct, const int* n, int q, int N, int halfE,
                                        const T* coarse) {
    constexpr int P1 = P + 1;
    if constexpr (DT == 0) {
        return coarse[0];
    } else if constexpr (DT == 1) {
        const int e = n[0] / P1, row = (e & 1) * P1 + n[0] % P1, cb = ((q & 1) * halfE + e / 2) * P1;
        T acc = T(0);
#pragma unroll
        for (int j = 0; j < P1; ++j) acc += ct.I[row][j] * coarse[cb + j];
        return acc;
    } else {
        const int e0 = n[0] / P1, row0 = (e0 & 1) * P1 + n[0] % P1, cb0 = ((q & 1) * halfE + e0 / 2) * P1;
        const int e1 = n[1] / P1, row1 = (e1 & 1) * P1 + n[1] % P1, cb1 = (((q >> 1) & 1) * halfE + e1 / 2) * P1;
        T acc = T(0);
#pragma unroll
        for (int j1 = 0; j1 < P1; ++j1) {
            T a = T(0);
#pragma unroll
            for (int j0 = 0; j0 < P1; ++j0) a += ct.I[row0][j0] * coarse[(cb0 + j0) + N * (cb1 + j1)];
            acc += ct.I[row1][j1] * a;
        }
        return acc;
    }
}

// Coarse-fine ghosts of one face, both planes. u's ghost is the I or R image
// of the other side's face nodes. The gradient's ghost is the image of the
// other side's face gradient, its own part plus its ghost coefficient times
// its u ghost over its spacing, and that u ghost is in turn the image of this
// side's face nodes, so the two images compose and no exchange of the other
// side's gradient is needed. dense_fill forms the other side's face gradient
// over the part of the face that meets this one, in the scratch G (a quarter
// of a coarse face, H^(D-1) words, or the 2^(D-1) fine faces across it,
// 2^(D-1) F words), with the CTA's threads tid = 0 .. nt-1; after a barrier
// dense_point reads this face's two ghosts at its node t. The I and R tables
// `ct` sit in shared memory, which the threads index by their own node.
// The planes are read through accessors, so that they may sit in global
// memory (the face exports) or staged in shared memory: own() is this face's
// u plane, fog(q) and u(q) the other side's q-th face gradient part and u
// plane (q = 0 on a fine side, the fine faces by child bits on a coarse one).
template <typename T, int DT, int P, class Own, class Fog>
__device__ __forceinline__ void dense_fill_at(const CfFace& face, int E, Own own, Fog fog, const Tab<T, P>& tb,
                                              const CfTab<T, P>& ct, T* G, int tid, int nt) {
    constexpr int P1 = P + 1;
    const int N = E * P1, H = N / 2, halfE = E / 2;
    const int F = DT == 0 ? 1 : DT == 1 ? N : N * N;
    const T gco = ghost_coef<T, P>(tb, 1 - face.side);
    if (face.kind == 0) {
        // this block is the fine side: the coarse side's face gradient at the
        // coarse nodes of this block's quarter, its u ghost the R image of
        // this face's nodes
        const T inv_hc = T(1) / T(2.0 * face.h);
        const int nq = DT == 0 ? 1 : DT == 1 ? H : H * H;
        const T* fc = fog(0);
        for (int m = tid; m < nq; m += nt) {
            int n[2] = {0, 0}, mm = m;
            for (int k = 0; k < DT; ++k) { n[k] = ((face.sub >> k) & 1) * H + mm % H; mm /= H; }
            const T ug = restrict_at<T, DT, P>(ct, n, N, halfE, own());
            const int ci = DT == 2 ? n[0] + N * n[1] : n[0];
            G[m] = (fc[ci] + gco * ug) * inv_hc;
        }
    } else {
        // the coarse side: each fine side's face gradient at its nodes, its u
        // ghost the I image of this face's nodes
        const T inv_hf = T(1) / T(0.5 * face.h);
        const int nsub = 1 << DT;
        for (int i = tid; i < nsub * F; i += nt) {
            const int q = i / F, tt = i % F;
            int n[2] = {0, 0};
            if (DT >= 1) n[0] = tt % N;
            if (DT == 2) n[1] = tt / N;
            const T ug = prolong_at<T, DT, P>(ct, n, q, N, halfE, own());
            G[i] = (fog(q)[tt] + gco * ug) * inv_hf;
        }
    }
}

template <typename T, int DT, int P, class U>
__device__ __forceinline__ void dense_point_at(const CfFace& face, int t, int E, U u, const CfTab<T, P>& ct,
                                               const T* G, T& ug, T& gg) {
    constexpr int P1 = P + 1;
    const int N = E * P1, H = N / 2, halfE = E / 2;
    const int F = DT == 0 ? 1 : DT == 1 ? N : N * N;
    int n[2] = {0, 0};
    if (DT >= 1) n[0] = t % N;
    if (DT == 2) n[1] = t / N;
    if (face.kind == 0) {
        ug = prolong_at<T, DT, P>(ct, n, face.sub, N, halfE, u(0));
        gg = prolong_at<T, DT, P>(ct, n, 0, H, halfE, G);
    } else {
        int bits = 0;
        for (int k = 0; k < DT; ++k) bits |= ((n[k] / P1) / halfE) << k;
        ug = restrict_at<T, DT, P>(ct, n, N, halfE, u(bits));
        gg = restrict_at<T, DT, P>(ct, n, N, halfE, G + (int64_t)bits * F);
    }
}

// The two with the planes read from the face exports in global memory.
template <typename T, int DT, int P>
__device__ __forceinline__ void dense_fill(const CfFace& face, int E, const T* fu, const T* fog, const Tab<T, P>& tb,
                                           const CfTab<T, P>& ct, T* G, int tid, int nt) {
    const int N = E * (P + 1);
    const int F = DT == 0 ? 1 : DT == 1 ? N : N * N;
    dense_fill_at<T, DT, P>(
        face, E, [&]() { return fu + (int64_t)face.slot * F; },
        [&](int q) { return fog + (int64_t)face.src[q] * F; }, tb, ct, G, tid, nt);
}

template <typename T, int DT, int P>
__device__ __forceinline__ void dense_point(const CfFace& face, int t, int E, const T* fu, const CfTab<T, P>& ct,
                                            const T* G, T& ug, T& gg) {
    const int N = E * (P + 1);
    const int F = DT == 0 ? 1 : DT == 1 ? N : N * N;
    dense_point_at<T, DT, P>(face, t, E, [&](int q) { return fu + (int64_t)face.src[q] * F; }, ct, G, ug, gg);
}

// A face's planes staged in shared memory for dense_fill_at and
// dense_point_at, in one region of staged_words(kind, F) words: on a coarse
// side the four fine u planes, the four fine face gradient planes (which G
// then overwrites in place) and its own u plane; on a fine side the coarse u
// plane, the coarse face gradient plane, its own u plane and G's quarter.
__host__ __device__ constexpr int staged_words(int kind, int F) { return kind ? 9 * F : 3 * F + (F + 3) / 4; }

template <typename T, int DT, int P>
__device__ __forceinline__ void stage_face_planes(const CfFace& face, int E, const T* fu, const T* fog, T* W, int tid,
                                                  int nt) {
    const int N = E * (P + 1);
    const int F = DT == 0 ? 1 : DT == 1 ? N : N * N;
    const int ns = face.kind ? 1 << DT : 1;
    for (int i = tid; i < ns * F; i += nt) {
        const int q = i / F, tt = i % F;
        const int64_t o = (int64_t)face.src[q] * F + tt;
        W[i] = fu[o];
        W[ns * F + i] = fog[o];
    }
    for (int i = tid; i < F; i += nt) W[2 * ns * F + i] = fu[(int64_t)face.slot * F + i];
}

// The I and R tables into shared memory by the CTA's threads (a barrier
// follows before they are read).
template <typename T, int P>
__device__ __forceinline__ void stage_cftab(const CfTab<T, P>& ct, CfTab<T, P>* dst, int tid, int nt) {
    const T* s = reinterpret_cast<const T*>(&ct);
    T* d = reinterpret_cast<T*>(dst);
    for (int i = tid; i < (int)(sizeof(CfTab<T, P>) / sizeof(T)); i += nt) d[i] = s[i];
}

// Coarse-fine ghosts in their own launch, one face per CTA, both planes (for
// the kernels that do not form them in their prologue).
template <typename T, int D, int P>
__global__ void __launch_bounds__(128) cf_ghost_kernel(const CfFace* cf, int ncf, int E, const T* fu, const T* fog,
                                                       T* ugd, T* ggd, Tab<T, P> tb, CfTab<T, P> ct) {
    constexpr int DT = D - 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ CfTab<T, P> sct;
    T* G = reinterpret_cast<T*>(smem_raw);
    const int N = E * (P + 1);
    const int F = ipow(N, DT);
    stage_cftab<T, P>(ct, &sct, threadIdx.x, blockDim.x);
    for (int c = blockIdx.x; c < ncf; c += gridDim.x) {
        const CfFace& face = cf[c];
        __syncthreads();  // the tables are in place; G is free
        dense_fill<T, DT, P>(face, E, fu, fog, tb, sct, G, threadIdx.x, blockDim.x);
        __syncthreads();
        for (int t = threadIdx.x; t < F; t += blockDim.x) {
            T ug, gg;
            dense_point<T, DT, P>(face, t, E, fu, sct, G, ug, gg);
            ugd[(int64_t)face.slot * F + t] = ug;
            ggd[(int64_t)face.slot * F + t] = gg;
        }
    }
}

// The coarse-fine image of `vars` planes per face slot ((vars, F) per slot):
// the full metric's u ghosts (vars 1, from the face exports) and Cartesian
// gradient ghosts (vars 3, from the V face planes) of a refined brick patch,
// where the map is affine and the flat problem's I and R apply to each. The
// tables are staged in shared memory, which the threads index by their node.
template <typename T, int D, int P>
__global__ void __launch_bounds__(256) cf_plane_kernel(const CfFace* cf, int ncf, int E, int vars, const T* src, T* dst,
                                                       CfTab<T, P> ct) {
    constexpr int P1 = P + 1, DT = D - 1;
    __shared__ CfTab<T, P> sct;
    {
        const T* s = reinterpret_cast<const T*>(&ct);
        T* d = reinterpret_cast<T*>(&sct);
        for (int i = threadIdx.x; i < (int)(sizeof(CfTab<T, P>) / sizeof(T)); i += blockDim.x) d[i] = s[i];
    }
    __syncthreads();
    const int N = E * P1, halfE = E / 2;
    const int F = ipow(N, DT);
    const int64_t total = (int64_t)ncf * vars * F;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int t = (int)(i % F);
        const int comp = (int)((i / F) % vars);
        const CfFace face = cf[i / ((int64_t)F * vars)];
        int n[2] = {0, 0};
        if (DT >= 1) n[0] = t % N;
        if (DT == 2) n[1] = t / N;
        T v;
        if (face.kind == 0) {
            v = prolong_at<T, DT, P>(sct, n, face.sub, N, halfE, src + ((int64_t)face.src[0] * vars + comp) * F);
        } else {
            int bits = 0;
            for (int k = 0; k < DT; ++k) bits |= ((n[k] / P1) / halfE) << k;
            v = restrict_at<T, DT, P>(sct, n, N, halfE, src + ((int64_t)face.src[bits] * vars + comp) * F);
        }
        dst[((int64_t)face.slot * vars + comp) * F + t] = v;
    }
}

// ---------------------------------------------------------------------------
// The stencil gather of the extraction (src/extraction.jl:216-245): out[j] =
// sum_q w[q, j] u[index[q, j] + varoff], one thread per point.
template <typename T>
__global__ void __launch_bounds__(256) gather_kernel(const T* u, int64_t varoff, int64_t npoints, int nper,
                                                     const int64_t* index, const T* w, T* out) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < npoints;
         j += (int64_t)gridDim.x * blockDim.x) {
        T s = T(0);
        for (int q = 0; q < nper; ++q) s += w[j * nper + q] * u[index[j * nper + q] + varoff];
        out[j] = s;
    }
}

// ---------------------------------------------------------------------------
// The regrid transfer (TreeAMR's element-set regrid, which the reference's
// regrid! runs on the host): one CTA per new block, both variables, by
// direct tensor sums of the 1D operators. Refining evaluates the coarse
// element's polynomial at the fine nodes (I along every dimension);
// coarsening is the L2 projection in the Gauss-Lobatto inner product (R =
// M_c^-1 I^T M_f along every dimension). Both keep sum w u.
template <typename T, int D, int P>
__global__ void __launch_bounds__(256) transfer_kernel(const TransferItem* items, int nitems, int E, const T* src,
                                                       T* dst, CfTab<T, P> ct) {
    constexpr int P1 = P + 1;
    const int N = E * P1, halfE = E / 2;
    int NN = 1;
    for (int k = 0; k < D; ++k) NN *= N;
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const TransferItem it = items[item];
        for (int i = threadIdx.x; i < 2 * NN; i += blockDim.x) {
            const int var = i / NN, n = i % NN;
            int x[3] = {0, 0, 0};
            {
                int r = n;
                for (int k = 0; k < D; ++k) { x[k] = r % N; r /= N; }
            }
            T out;
            if (it.mode == 0) {
                out = src[it.src[0] + i];
            } else if (it.mode == 1) {
                // the child's node x: fine element ef = x / P1 of the half `sub` of the
                // parent, row (ef & 1) P1 + x % P1 of I over the parent element's nodes
                int row[3] = {0, 0, 0}, cb[3] = {0, 0, 0};
                for (int k = 0; k < D; ++k) {
                    const int ef = x[k] / P1;
                    row[k] = (ef & 1) * P1 + x[k] % P1;
                    cb[k] = (((it.sub >> k) & 1) * halfE + ef / 2) * P1;
                }
                const T* s = src + it.src[0] + (int64_t)var * NN;
                T acc = T(0);
                const int J1 = D > 1 ? P1 : 1, J2 = D > 2 ? P1 : 1;
                for (int j2 = 0; j2 < J2; ++j2)
                    for (int j1 = 0; j1 < J1; ++j1) {
                        T w12 = T(1);
                        if (D > 1) w12 *= ct.I[row[1]][j1];
                        if (D > 2) w12 *= ct.I[row[2]][j2];
                        const int64_t base = (cb[0]) + (int64_t)N * ((cb[1] + j1) + (int64_t)N * (cb[2] + j2));
                        T a = T(0);
#pragma unroll
                        for (int j0 = 0; j0 < P1; ++j0) a += ct.I[row[0]][j0] * s[base + j0];
                        acc += w12 * a;
                    }
                out = acc;
            } else {
                // the coarse node x: element ec = x / P1 in the half h = ec / (E/2) of
                // the block, covered by the child of those halves, whose fine elements
                // 2 (ec % (E/2)) and the next carry R's 2 P1 columns
                int row[3] = {0, 0, 0}, fb[3] = {0, 0, 0}, child = 0;
                for (int k = 0; k < D; ++k) {
                    const int ec = x[k] / P1;
                    row[k] = x[k] % P1;
                    child |= (ec / halfE) << k;
                    fb[k] = 2 * (ec % halfE) * P1;
                }
                const T* s = src + it.src[child] + (int64_t)var * NN;
                T acc = T(0);
                const int J1 = D > 1 ? 2 * P1 : 1, J2 = D > 2 ? 2 * P1 : 1;
                for (int j2 = 0; j2 < J2; ++j2)
                    for (int j1 = 0; j1 < J1; ++j1) {
                        T w12 = T(1);
                        if (D > 1) w12 *= ct.R[row[1]][j1];
                        if (D > 2) w12 *= ct.R[row[2]][j2];
                        const int64_t base = fb[0] + (int64_t)N * ((fb[1] + j1) + (int64_t)N * (fb[2] + j2));
                        T a = T(0);
#pragma unroll
                        for (int j0 = 0; j0 < 2 * P1; ++j0) a += ct.R[row[0]][j0] * s[base + j0];
                        acc += w12 * a;
                    }
                out = acc;
            }
            dst[it.dst + i] = out;
        }
    }
}

// ---------------------------------------------------------------------------
// Block tiles. A block's u with its face ghosts lives in shared memory in a
// padded layout with an odd x pitch (N+3), so that element lines along x,
// which consecutive threads take at consecutive y, hit distinct banks; the
// gradient along the current d uses the same layout, and the Laplacian
// accumulator / new v a ghost-free layout with x pitch N+1 (odd). A shape
// is either compile-time (ShapeC: N = E(P+1) known, all index arithmetic
// folds to shifts and multiplies) or run-time (ShapeR, for other E).
template <int D, int P, int E_>
struct ShapeC {
    static constexpr int E = E_;
    static constexpr int P1 = P + 1;
    static constexpr int N = E_ * (P + 1);
    static constexpr int F = ipow(N, D - 1);
    static constexpr int NN = ipow(N, D);
    static constexpr int SX = N + 3, SY = N + 2;
    static constexpr int SS = D == 1 ? SX : D == 2 ? SX * SY : SX * SY * SY;
    static constexpr int LX = N + 1;
    static constexpr int LS = LX * ipow(N, D - 1);
    __device__ ShapeC(int) {}
    __device__ static constexpr int sstride(int d) { return d == 0 ? 1 : d == 1 ? SX : SX * SY; }
    __device__ static constexpr int lstride(int d) { return d == 0 ? 1 : d == 1 ? LX : LX * N; }
};

template <int D, int P>
struct ShapeR {
    static constexpr int P1 = P + 1;
    int E, N, F, NN, SX, SY, SS, LX, LS;
    __device__ ShapeR(int E_) : E(E_) {
        N = E_ * P1;
        F = 1;
        for (int k = 0; k < D - 1; ++k) F *= N;
        NN = F * N;
        SX = N + 3;
        SY = N + 2;
        SS = D == 1 ? SX : D == 2 ? SX * SY : SX * SY * SY;
        LX = N + 1;
        LS = LX * F;
    }
    __device__ int sstride(int d) const { return d == 0 ? 1 : d == 1 ? SX : SX * SY; }
    __device__ int lstride(int d) const { return d == 0 ? 1 : d == 1 ? LX : LX * N; }
};

// Coordinates of the node with tangential index t on the plane x_d = xd.
template <int D, class G>
__device__ __forceinline__ void plane_coords(const G& g, int d, int t, int xd, int (&x)[3]) {
    x[0] = x[1] = x[2] = 0;
    if (D == 1) { x[0] = xd; return; }
    if (D == 2) {
        if (d == 0) { x[0] = xd; x[1] = t; } else { x[0] = t; x[1] = xd; }
        return;
    }
    const int a = t % g.N, b = t / g.N;
    if (d == 0) { x[0] = xd; x[1] = a; x[2] = b; }
    else if (d == 1) { x[0] = a; x[1] = xd; x[2] = b; }
    else { x[0] = a; x[1] = b; x[2] = xd; }
}

template <int D, class G>
__device__ __forceinline__ void owned_coords(const G& g, int n, int (&x)[3]) {
    x[0] = n % g.N;
    x[1] = D > 1 ? (n / g.N) % g.N : 0;
    x[2] = D > 2 ? n / (g.N * g.N) : 0;
}

template <int D, class G>
__device__ __forceinline__ int sidx(const G& g, const int (&x)[3]) {
    int r = x[0] + 1;
    if (D > 1) r += g.SX * (x[1] + 1);
    if (D > 2) r += g.SX * g.SY * (x[2] + 1);
    return r;
}

template <int D, class G>
__device__ __forceinline__ int lidx(const G& g, const int (&x)[3]) {
    int r = x[0];
    if (D > 1) r += g.LX * x[1];
    if (D > 2) r += g.LX * g.N * x[2];
    return r;
}

template <int D, class G>
__device__ __forceinline__ int oidx(const G& g, const int (&x)[3]) {
    int r = x[0];
    if (D > 1) r += g.N * x[1];
    if (D > 2) r += g.N * g.N * x[2];
    return r;
}

// 16-byte vectors for the state streams.
template <typename T>
struct V16;
template <>
struct V16<float> { using type = float4; static constexpr int n = 4; };
template <>
struct V16<double> { using type = double2; static constexpr int n = 2; };

template <typename T, int D, class G>
__device__ __forceinline__ constexpr bool vec_ok(const G& g) {
    // 16-byte global loads scatter into shared memory at a stride of their
    // width, which conflicts 4-way; scalar loads are conflict-free and cost
    // less than the replays, so the vector path stays off.
    return false;
}

// The thread count of a block loop: the compile-time NT of a fixed-shape
// kernel (so that trip counts and per-thread coordinates fold), or the
// launch's for NT = 0.
template <int NT>
__device__ __forceinline__ int nthreads() {
    if constexpr (NT > 0) return NT;
    else return (int)blockDim.x;
}

// u of the block (owned layout in global memory) into the padded su, and its
// face ghosts: from the dense coarse-fine planes, or the neighbour's export.
template <typename T, int D, int NT, class G>
__device__ __forceinline__ void load_u_with_ghosts(const G& g, const BlockItem& it, const T* ysrc,
                                                   const StageArgs<T>& a, T* su) {
    const T* yu = ysrc + it.off;
    constexpr int VW = V16<T>::n;
    if (vec_ok<T, D>(g)) {
        using V = typename V16<T>::type;
        const V* src = reinterpret_cast<const V*>(yu);
        #pragma unroll 4
        for (int i = threadIdx.x; i < g.NN / VW; i += nthreads<NT>()) {
            V v = src[i];
            int x[3];
            owned_coords<D>(g, i * VW, x);
            int s0 = sidx<D>(g, x);
            const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
            for (int k = 0; k < VW; ++k) su[s0 + k] = e[k];
        }
    } else {
        #pragma unroll 4
        for (int n = threadIdx.x; n < g.NN; n += nthreads<NT>()) {
            int x[3];
            owned_coords<D>(g, n, x);
            su[sidx<D>(g, x)] = yu[n];
        }
    }
    #pragma unroll 4
    for (int i = threadIdx.x; i < 2 * D * g.F; i += nthreads<NT>()) {
        int f = i / g.F, t = i % g.F;
        int d = f >> 1, side = f & 1;
        T v;
        if (it.flags & (1u << f)) v = a.ugd[(int64_t)(it.slot + f) * g.F + t];
        else v = a.fu_in[(int64_t)it.nb[f] * g.F + t];
        int x[3];
        plane_coords<D>(g, d, t, side == 0 ? -1 : g.N, x);
        su[sidx<D>(g, x)] = v;
    }
}

// Gradient along d at every owned node into sg (padded), scaled by 1/h, and
// the two gradient ghost planes normal to d. With a diagonal metric the
// gradient set holds the flux A_d D_d u / h (src/evolution.jl:67-90), and a
// ghost is the neighbour's flux at its face node, with the neighbour's A_d.
template <typename T, int D, int P, int NT, class G>
__device__ __forceinline__ void gradient_along(const G& g, int d, const BlockItem& it, int item,
                                               const StageArgs<T>& a, const Tab<T, P>& tb, const T* su, T* sg,
                                               T inv_h) {
    constexpr int P1 = P + 1;
    const int sd = g.sstride(d);
    const int od = d == 0 ? 1 : d == 1 ? g.N : g.N * g.N;
    const T* Ad = a.coef ? a.coef + ((int64_t)item * (1 + D) + 1 + d) * g.NN : nullptr;
#pragma unroll 4
    for (int L = threadIdx.x; L < g.E * g.F; L += nthreads<NT>()) {
        int t = L % g.F, e = L / g.F;
        int x[3];
        plane_coords<D>(g, d, t, e * P1, x);
        int base = sidx<D>(g, x);
        T w[P + 3], out[P + 1];
#pragma unroll
        for (int k = 0; k < P + 3; ++k) w[k] = su[base + (k - 1) * sd];
        line_derivative<T, P>(tb, w, out);
        if (Ad) {
            const int ob = oidx<D>(g, x);
#pragma unroll
            for (int i = 0; i <= P; ++i) sg[base + i * sd] = Ad[ob + i * od] * (out[i] * inv_h);
        } else {
#pragma unroll
            for (int i = 0; i <= P; ++i) sg[base + i * sd] = out[i] * inv_h;
        }
    }
#pragma unroll 4
    for (int i = threadIdx.x; i < 2 * g.F; i += nthreads<NT>()) {
        int side = i / g.F, t = i % g.F;
        int f = 2 * d + side;
        int x[3];
        T v;
        if (it.flags & (1u << f)) {
            v = a.ggd[(int64_t)(it.slot + f) * g.F + t];
        } else {
            // the neighbour's face-node derivative: its own part plus its ghost
            // coefficient times its u ghost, which is this block's face node
            int nslot = it.nb[f];
            int nside = nslot & 1;  // slots are b*2D + f, so the parity is the side
            plane_coords<D>(g, d, t, side == 0 ? 0 : g.N - 1, x);
            T own = su[sidx<D>(g, x)];
            T gnb = (a.fog_in[(int64_t)nslot * g.F + t] + ghost_coef<T, P>(tb, nside) * own) * inv_h;
            if (a.coef) {
                int xn[3];
                plane_coords<D>(g, d, t, nside ? g.N - 1 : 0, xn);
                const int nitem = nslot / (2 * D);
                gnb = a.coef[((int64_t)nitem * (1 + D) + 1 + d) * g.NN + oidx<D>(g, xn)] * gnb;
            }
            v = (it.flags & (1u << (8 + f))) ? -gnb : gnb;
        }
        plane_coords<D>(g, d, t, side == 0 ? -1 : g.N, x);
        sg[sidx<D>(g, x)] = v;
    }
}

// Laplacian term along d: sl (+)= D_d(sg) at every owned node (not yet /h).
template <typename T, int D, int P, int NT, class G>
__device__ __forceinline__ void laplacian_along(const G& g, int d, const Tab<T, P>& tb, const T* sg, T* sl,
                                                bool first) {
    constexpr int P1 = P + 1;
    const int sd = g.sstride(d), ld = g.lstride(d);
    #pragma unroll 4
    for (int L = threadIdx.x; L < g.E * g.F; L += nthreads<NT>()) {
        int t = L % g.F, e = L / g.F;
        int x[3];
        plane_coords<D>(g, d, t, e * P1, x);
        int base = sidx<D>(g, x), lb = lidx<D>(g, x);
        T w[P + 3], out[P + 1];
#pragma unroll
        for (int k = 0; k < P + 3; ++k) w[k] = sg[base + (k - 1) * sd];
        line_derivative<T, P>(tb, w, out);
#pragma unroll
        for (int i = 0; i <= P; ++i) {
            if (first) sl[lb + i * ld] = out[i];
            else sl[lb + i * ld] += out[i];
        }
    }
}

// Truncation of v (ghost-free layout sv), per element line along each d in
// turn: c = sum_j topdual_j v_j; v_i -= topmode_i c (src/evolution.jl:222-264).
// With COMP the subtraction is error-free into the compensation words sc.
template <typename T, int D, int P, bool COMP, int NT, class G>
__device__ __forceinline__ void truncate_block(const G& g, const Tab<T, P>& tb, T* sv, T* sc,
                                               const T* trm = nullptr, const T* trd = nullptr, int item = 0,
                                               int nitems = 0) {
    constexpr int P1 = P + 1;
    for (int d = 0; d < D; ++d) {
        const int ld = g.lstride(d);
#pragma unroll 4
        for (int L = threadIdx.x; L < g.E * g.F; L += nthreads<NT>()) {
            int t = L % g.F, e = L / g.F;
            int x[3];
            plane_coords<D>(g, d, t, e * P1, x);
            int lb = lidx<D>(g, x);
            // the line's rank-one pair: the element's, or on a geometry the line's own
            T tm[P1], td[P1];
            if (trm) {
                const int64_t o = (int64_t)P1 * (e + (int64_t)g.E * (item + (int64_t)nitems * d));
#pragma unroll
                for (int j = 0; j < P1; ++j) { tm[j] = trm[o + j]; td[j] = trd[o + j]; }
            } else {
#pragma unroll
                for (int j = 0; j < P1; ++j) { tm[j] = tb.tm[j]; td[j] = tb.td[j]; }
            }
            T v[P1];
            T c = T(0);
#pragma unroll
            for (int j = 0; j < P1; ++j) { v[j] = sv[lb + j * ld]; c += td[j] * v[j]; }
            if (COMP) {
                T cc = T(0);
#pragma unroll
                for (int j = 0; j < P1; ++j) cc += td[j] * sc[lb + j * ld];
                c += cc;
#pragma unroll
                for (int i = 0; i < P1; ++i) {
                    T s, err;
                    two_sum(v[i], -(tm[i] * c), s, err);
                    sv[lb + i * ld] = s;
                    sc[lb + i * ld] += err;
                }
            } else {
#pragma unroll
                for (int i = 0; i < P1; ++i) sv[lb + i * ld] = v[i] - tm[i] * c;
            }
        }
        __syncthreads();
    }
}

// Face export from the padded su of the new stage value.
template <typename T, int D, int P, int NT, class G>
__device__ __forceinline__ void export_from_smem(const G& g, const BlockItem& it, const Tab<T, P>& tb, const T* su,
                                                 T* fu, T* fog) {
    #pragma unroll 4
    for (int i = threadIdx.x; i < 2 * D * g.F; i += nthreads<NT>()) {
        int f = i / g.F, t = i % g.F;
        int d = f >> 1, side = f & 1;
        int sd = g.sstride(d);
        int x[3];
        plane_coords<D>(g, d, t, side == 0 ? 0 : g.N - 1 - P, x);
        int base = sidx<D>(g, x);
        T e[P + 1];
#pragma unroll
        for (int k = 0; k <= P; ++k) e[k] = su[base + k * sd];
        int64_t o = (int64_t)(it.slot + f) * g.F + t;
        fu[o] = side == 0 ? e[0] : e[P];
        fog[o] = own_face_part<T, P>(tb, side, e);
    }
}

// The pointwise stage combination of VW consecutive nodes (along x, in one
// row) starting at owned index n0: k = (Y_v, lap/h), the classic RK4 update
// of stage `mode`, u-part into su, v-part into sl (and its compensation into
// sc at stage 4 with COMP).
// The stage's coefficients: ca multiplies k into the accumulator, cn into
// the next stage value. The host forms dt/6, dt/3, dt/2 and dt in FP64 and
// rounds each once to T.
template <typename T>
struct RkCoef {
    T ca, cn;
    __device__ RkCoef(int mode, const T* rk) {
        ca = mode == 1 || mode == 4 ? rk[0] : rk[1];
        cn = mode == 3 ? rk[3] : rk[2];
    }
};

template <typename T, bool COMP, int VW>
__device__ __forceinline__ void stage_points(int mode, RkCoef<T> rc, const T* yv, const T* un_u, const T* un_v,
                                             T* acc_u, T* acc_v, T* comp_u, const T* comp_v_in, const T* sl_in,
                                             T inv_h, T (&nu)[VW], T (&nv)[VW], T (&cv)[VW]) {
#pragma unroll
    for (int k = 0; k < VW; ++k) {
        T ku = yv[k];
        T kv = sl_in[k] * inv_h;
        T uu = un_u[k], uv = un_v[k];
        if (mode == 1) {
            acc_u[k] = rc.ca * ku;
            acc_v[k] = rc.ca * kv;
            nu[k] = uu + rc.cn * ku;
            nv[k] = uv + rc.cn * kv;
        } else if (mode == 2 || mode == 3) {
            acc_u[k] += rc.ca * ku;
            acc_v[k] += rc.ca * kv;
            nu[k] = uu + rc.cn * ku;
            nv[k] = uv + rc.cn * kv;
        } else {
            T iu = acc_u[k] + rc.ca * ku;
            T iv = acc_v[k] + rc.ca * kv;
            if (COMP) {
                T cu = comp_u[k] + iu, cvv = comp_v_in[k] + iv;
                T eu, ev;
                two_sum(uu, cu, nu[k], eu);
                two_sum(uv, cvv, nv[k], ev);
                comp_u[k] = eu;
                cv[k] = ev;
            } else {
                nu[k] = uu + iu;
                nv[k] = uv + iv;
            }
        }
    }
}

template <typename T, int VW>
struct Pack {
    T v[VW];
};

template <typename T, int VW>
__device__ __forceinline__ Pack<T, VW> ldv(const T* p) {
    Pack<T, VW> r;
    if constexpr (VW == V16<T>::n) {
        using V = typename V16<T>::type;
        V x = *reinterpret_cast<const V*>(p);
        const T* e = reinterpret_cast<const T*>(&x);
#pragma unroll
        for (int k = 0; k < VW; ++k) r.v[k] = e[k];
    } else {
#pragma unroll
        for (int k = 0; k < VW; ++k) r.v[k] = p[k];
    }
    return r;
}

template <typename T, int VW>
__device__ __forceinline__ void stv(T* p, const T (&a)[VW]) {
    if constexpr (VW == V16<T>::n) {
        using V = typename V16<T>::type;
        V x;
        T* e = reinterpret_cast<T*>(&x);
#pragma unroll
        for (int k = 0; k < VW; ++k) e[k] = a[k];
        *reinterpret_cast<V*>(p) = x;
    } else {
#pragma unroll
        for (int k = 0; k < VW; ++k) p[k] = a[k];
    }
}

// One block of the fused stage: k = f(Y) (u' = v, v' = sum_d D_d D_d u), the
// RK4 combination of that stage, the truncation of the new v and the face
// export of the new u. acc holds only increments (dt/6 k1 + dt/3 k2 + dt/3
// k3), added to u^n at stage 4. mode MODE_RHS writes du = f(u) only.
template <typename T, int D, int P, bool COMP, int NT, class G, int VW>
__device__ __forceinline__ void stage_block(const G& g, const StageArgs<T>& a, const Tab<T, P>& tb,
                                            const BlockItem& it, int item, T* su, T* sg, T* sl) {
    const int mode = a.mode;
    const T* ysrc = (mode == MODE_RHS || mode == MODE_STAGE1) ? a.u : a.y;
    const T inv_h = T(1) / T(it.h);
    if (threadIdx.x == 0) prefetch_stage<T>(a, item, 2 * (int64_t)g.NN);
    load_u_with_ghosts<T, D, NT>(g, it, ysrc, a, su);
    __syncthreads();
    for (int d = 0; d < D; ++d) {
        gradient_along<T, D, P, NT>(g, d, it, item, a, tb, su, sg, inv_h);
        __syncthreads();
        laplacian_along<T, D, P, NT>(g, d, tb, sg, sl, d == 0);
        __syncthreads();
    }
    const T* yv = ysrc + it.off + g.NN;
    if (mode == MODE_RHS) {
        T* du = a.du + it.off;
        #pragma unroll 4
        for (int i = threadIdx.x; i < g.NN / VW; i += nthreads<NT>()) {
            const int n0 = i * VW;
            int x[3];
            owned_coords<D>(g, n0, x);
            const int l0 = lidx<D>(g, x);
            Pack<T, VW> v = ldv<T, VW>(yv + n0);
            T lap[VW];
#pragma unroll
            for (int k = 0; k < VW; ++k) {
                lap[k] = sl[l0 + k] * inv_h;
                // a geometry's Laplacian is divided by sqrt(g) (src/evolution.jl:67-110)
                if (a.coef) lap[k] = lap[k] / a.coef[(int64_t)item * (1 + D) * g.NN + n0 + k];
            }
            stv<T, VW>(du + n0, v.v);
            stv<T, VW>(du + g.NN + n0, lap);
        }
        __syncthreads();
        return;
    }
    const RkCoef<T> rc(mode, a.rk + 4 * it.problem);
    const T* __restrict__ un = a.u + it.off;
    T* __restrict__ acc = a.acc + it.off;
    T* __restrict__ comp = COMP ? a.comp + it.off : nullptr;
    const T* __restrict__ yvr = yv;
    T* sc = sg;  // compensation of v during the final truncation (ghost-free layout)
    // Batches of B nodes per thread: every global load of a batch is issued
    // before the first use, so each thread keeps several in flight.
    constexpr int B = 4;
    const int nt = nthreads<NT>();
    for (int j0 = 0; j0 * nt < g.NN; j0 += B) {
        T y[B], uu[B], uv[B], au[B], av[B], cu[B], cvi[B];
#pragma unroll
        for (int q = 0; q < B; ++q) {
            const int n = threadIdx.x + (j0 + q) * nt;
            if (n < g.NN) {
                y[q] = yvr[n];
                uu[q] = un[n];
                uv[q] = un[g.NN + n];
                if (mode != 1) {
                    au[q] = acc[n];
                    av[q] = acc[g.NN + n];
                }
                if (COMP && mode == MODE_STAGE4) {
                    cu[q] = comp[n];
                    cvi[q] = comp[g.NN + n];
                }
            }
        }
#pragma unroll
        for (int q = 0; q < B; ++q) {
            const int n = threadIdx.x + (j0 + q) * nt;
            if (n < g.NN) {
                int x[3];
                owned_coords<D>(g, n, x);
                const int s0 = sidx<D>(g, x), l0 = lidx<D>(g, x);
                T lap[1] = {sl[l0]};
                if (a.coef) lap[0] = lap[0] / a.coef[(int64_t)item * (1 + D) * g.NN + n];
                T nu[1], nv[1], cv[1];
                T yq[1] = {y[q]}, uuq[1] = {uu[q]}, uvq[1] = {uv[q]}, auq[1] = {au[q]}, avq[1] = {av[q]},
                  cuq[1] = {cu[q]}, cviq[1] = {cvi[q]};
                stage_points<T, COMP, 1>(mode, rc, yq, uuq, uvq, auq, avq, cuq, cviq, lap, inv_h, nu, nv, cv);
                if (mode != MODE_STAGE4) {
                    acc[n] = auq[0];
                    acc[g.NN + n] = avq[0];
                }
                if (COMP && mode == MODE_STAGE4) comp[n] = cuq[0];
                su[s0] = nu[0];
                sl[l0] = nv[0];
                if (COMP && mode == MODE_STAGE4) sc[l0] = cv[0];
            }
        }
    }
    __syncthreads();
    const bool final_comp = COMP && mode == MODE_STAGE4;
    if (a.truncate) {
        if (final_comp) truncate_block<T, D, P, true, NT>(g, tb, sl, sc, a.trm, a.trd, item, a.nitems);
        else truncate_block<T, D, P, false, NT>(g, tb, sl, sc, a.trm, a.trd, item, a.nitems);
    }
    T* out = (mode == MODE_STAGE4 ? a.u : a.y) + it.off;
    #pragma unroll 4
    for (int i = threadIdx.x; i < g.NN / VW; i += nthreads<NT>()) {
        const int n0 = i * VW;
        int x[3];
        owned_coords<D>(g, n0, x);
        const int s0 = sidx<D>(g, x), l0 = lidx<D>(g, x);
        T ou[VW], ov[VW], oc[VW];
#pragma unroll
        for (int k = 0; k < VW; ++k) {
            ou[k] = su[s0 + k];
            ov[k] = sl[l0 + k];
            if (final_comp) oc[k] = sc[l0 + k];
        }
        stv<T, VW>(out + n0, ou);
        stv<T, VW>(out + g.NN + n0, ov);
        if (final_comp) stv<T, VW>(comp + g.NN + n0, oc);
    }
    export_from_smem<T, D, P, NT>(g, it, tb, su, a.fu_out, a.fog_out);
    __syncthreads();
}


// Threads per CTA and the CTAs per SM the register budget is sized for, from
// the shape: 64 to 256 threads by block size (512 for large FP64 blocks), and
// as many CTAs as the shared memory allows, at most 65536 / (64 NT) so that a
// thread keeps at least 64 registers.
template <typename T, int D, int P, int E>
struct StageLaunch {
    using G = ShapeC<D, P, E>;
    // the fixed-shape kernel must be launched with exactly NT threads: its
    // block loops stride by this constant
    static constexpr int NT = G::NN >= 2048 ? (sizeof(T) == 8 ? 512 : 256) : G::NN >= 512 ? 128 : 64;
    static constexpr size_t bytes = (2 * (size_t)G::SS + (size_t)G::LS) * sizeof(T) + 1024;
    static constexpr int by_smem = (int)((227 * 1024) / bytes);
    static constexpr int by_regs = 65536 / (NT * 64);
    static constexpr int MINB = by_smem < 1 ? 1 : (by_smem < by_regs ? by_smem : by_regs);
};

// Stage kernel with a compile-time shape (E known). The pointwise phases
// touch shared memory one node per thread (consecutive threads, consecutive
// words: no bank conflicts with the odd pitches), with coalesced scalar
// global accesses.
template <typename T, int D, int P, int E, bool COMP>
__global__ void __launch_bounds__(StageLaunch<T, D, P, E>::NT, StageLaunch<T, D, P, E>::MINB)
    stage_kernel_c(StageArgs<T> a, Tab<T, P> tb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using G = ShapeC<D, P, E>;
    G g(E);
    T* su = reinterpret_cast<T*>(smem_raw);
    T* sg = su + G::SS;
    T* sl = sg + G::SS;
    constexpr int VW = 1;
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        stage_block<T, D, P, COMP, StageLaunch<T, D, P, E>::NT, G, VW>(g, a, tb, it, item, su, sg, sl);
    }
}

// Stage kernel for any E (run-time shape, scalar I/O).
template <typename T, int D, int P, bool COMP>
__global__ void __launch_bounds__(256) stage_kernel(StageArgs<T> a, Tab<T, P> tb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using G = ShapeR<D, P>;
    G g(a.E);
    T* su = reinterpret_cast<T*>(smem_raw);
    T* sg = su + g.SS;
    T* sl = sg + g.SS;
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        stage_block<T, D, P, COMP, 0, G, 1>(g, a, tb, it, item, su, sg, sl);
    }
}

// ---------------------------------------------------------------------------
// Energy (src/evolution.jl:1472-1489, flat): 1/2 sum_nodes w (v^2 + sum_d
// (D_d u)^2), w = prod_d h (P+1)/2 w_hat(i_d). One FP64 partial per block.
template <int D>
__device__ __forceinline__ double block_reduce_sum(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0) {
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) s += red[w];
    }
    __syncthreads();
    return s;
}

template <typename T, int D, int P>
__global__ void __launch_bounds__(256) energy_kernel(StageArgs<T> a, Tab<T, P> tb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using G = ShapeR<D, P>;
    G g(a.E);
    T* su = reinterpret_cast<T*>(smem_raw);
    double* red = reinterpret_cast<double*>(su + g.SS + (g.SS & 1));
    constexpr int P1 = P + 1;
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        const double h = it.h;
        const T inv_h = T(1) / T(h);
        load_u_with_ghosts<T, D, 0>(g, it, a.u, a, su);
        __syncthreads();
        // the quadrature weight of a node is wscale^D times the product of
        // its reference weights: the sum runs over the products, and the
        // block's factor wscale^D multiplies it once, so a node costs few
        // FP64 operations (the accumulation stays FP64)
        double local = 0;
        const double wscale = h * P1 / 2.0;
        double wsD = 1.0;
        for (int k = 0; k < D; ++k) wsD *= wscale;
        double wqd[P1];
#pragma unroll
        for (int i = 0; i < P1; ++i) wqd[i] = (double)tb.wq[i];
        const T* uv = a.u + it.off + g.NN;
        // on a geometry: 1/2 sum w (sqrt(g) v^2 + sum_d F_d^2 / A_d), F_d = A_d D_d u
        const T* cf = a.coef ? a.coef + (int64_t)item * (1 + D) * g.NN : nullptr;
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<D>(g, n, x);
            double w = wqd[x[0] % P1];
            for (int k = 1; k < D; ++k) w *= wqd[x[k] % P1];
            const double v = (double)uv[n];
            local += (cf ? (double)cf[n] * w : w) * v * v;
        }
        for (int d = 0; d < D; ++d) {
            const int sd = g.sstride(d);
            for (int L = threadIdx.x; L < g.E * g.F; L += blockDim.x) {
                int t = L % g.F, e = L / g.F;
                int x[3];
                plane_coords<D>(g, d, t, e * P1, x);
                int base = sidx<D>(g, x);
                double wt = 1.0;
                for (int k = 0; k < D; ++k)
                    if (k != d) wt *= wqd[x[k] % P1];
                T w[P + 3], out[P + 1];
#pragma unroll
                for (int k = 0; k < P + 3; ++k) w[k] = su[base + (k - 1) * sd];
                line_derivative<T, P>(tb, w, out);
                const int ob = oidx<D>(g, x);
                const int od = d == 0 ? 1 : d == 1 ? g.N : g.N * g.N;
                double line = 0;
#pragma unroll
                for (int i = 0; i <= P; ++i) {
                    const double gv = (double)(out[i] * inv_h);
                    const double wi = cf ? (double)cf[(1 + d) * g.NN + ob + i * od] * wqd[i] : wqd[i];
                    line += wi * gv * gv;
                }
                local += wt * line;
            }
        }
        double s = block_reduce_sum<D>(local, red);
        if (threadIdx.x == 0) a.partial[item] = 0.5 * wsD * s;
        __syncthreads();
    }
}

// Quadrature p-norm parts (src/layout.jl:100-122, 223-235): per block
// sum w |x - ref|^p over the selected variables and sum w * nvars; p = 0
// means the largest |x - ref|.
//
// A thread takes columns along the slowest dimension (consecutive threads,
// consecutive columns: coalesced loads), so the weight's factor of the other
// dimensions is one product a column, and the slowest dimension's factor
// wq[q] multiplies P+1 running sums (one per node position q of an element)
// once at the end: a node costs its difference and one FP64 FMA a variable,
// no integer division and no weight product. Every sum stays FP64. A block
// of fewer columns than threads splits each column's elements among
// blockDim / C threads.
template <typename T, int D, int P>
__global__ void norm_kernel(const BlockItem* items, int nitems, int E, const T* u, const T* ref, int p,
                            int vars_mask, Tab<T, P> tb, double* part_num, double* part_vol, const T* coef,
                            int ncoef) {
    __shared__ double red[32];
    constexpr int P1 = P + 1;
    const int N = E * P1;
    const int NN = ipow(N, D);
    const int C = NN / N;   // columns a block: N^(D-1)
    double wqd[P1];
    double wsum = 0;
#pragma unroll
    for (int i = 0; i < P1; ++i) {
        wqd[i] = (double)tb.wq[i];
        wsum += wqd[i];
    }
    const int nvars = (vars_mask & 1) + ((vars_mask >> 1) & 1);
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const BlockItem it = items[item];
        // the weights' block factor wscale^D multiplies the sums once
        const double wscale = it.h * P1 / 2.0;
        double wsD = 1.0;
        for (int k = 0; k < D; ++k) wsD *= wscale;
        const T* cw = coef ? coef + (int64_t)item * ncoef * NN : nullptr;
        double num = 0, vol = 0;
        const bool wide = C >= (int)blockDim.x;
        const int S = wide ? 1 : (int)blockDim.x / C;              // slices of a column's elements
        const int sl = wide ? 0 : (int)threadIdx.x / C;            // this thread's slice
        const int cstep = wide ? (int)blockDim.x : C;
        for (int c = wide ? (int)threadIdx.x : (int)threadIdx.x % C; sl < S && c < C; c += cstep) {
            // the column's weight over the dimensions but the slowest
            double wc = 1.0;
            int m = c;
            for (int k = 1; k < D; ++k) {
                wc *= wqd[(m % N) % P1];
                m /= N;
            }
            double acc[P1], accv[P1];
#pragma unroll
            for (int q = 0; q < P1; ++q) acc[q] = accv[q] = 0.0;
            double mx = 0;
            int ne = 0;
            for (int e = sl; e < E; e += S) {
                ++ne;
#pragma unroll
                for (int q = 0; q < P1; ++q) {
                    const int n = c + C * (e * P1 + q);
                    const double g = cw ? (double)cw[n] : 1.0;
                    if (cw) accv[q] += g;
#pragma unroll
                    for (int var = 0; var < 2; ++var) {
                        if (!(vars_mask & (1 << var))) continue;
                        const int64_t o = it.off + (int64_t)var * NN + n;
                        double x = (double)u[o];
                        if (ref) x -= (double)ref[o];
                        if (p == 0) mx = fmax(mx, fabs(x));
                        else if (p == 2) acc[q] += (cw ? g * x : x) * x;
                        else acc[q] += g * pow(fabs(x), (double)p);
                    }
                }
            }
            if (p == 0) {
                num = fmax(num, mx);
            } else {
                double s = 0;
#pragma unroll
                for (int q = 0; q < P1; ++q) s += wqd[q] * acc[q];
                num += wc * s;
            }
            if (cw) {
                double sv = 0;
#pragma unroll
                for (int q = 0; q < P1; ++q) sv += wqd[q] * accv[q];
                vol += wc * sv * nvars;
            } else {
                vol += wc * wsum * ne * nvars;
            }
        }
        double s;
        if (p == 0) {
            for (int o = 16; o > 0; o >>= 1) num = fmax(num, __shfl_down_sync(0xffffffffu, num, o));
            int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
            if (lane == 0) red[wid] = num;
            __syncthreads();
            s = 0;
            if (threadIdx.x == 0)
                for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) s = fmax(s, red[w]);
            __syncthreads();
        } else {
            s = block_reduce_sum<D>(num, red);
        }
        double v = block_reduce_sum<D>(vol, red);
        if (threadIdx.x == 0) {
            part_num[item] = p == 0 ? s : wsD * s;
            part_vol[item] = wsD * v;
        }
        __syncthreads();
    }
}

// Modal indicator (src/refinement.jl:56-77): per element the largest over
// its lines in every dimension and over the modes q of
// (weights[q] |sum_j duals[q][j] a_j|)^pows[q], times post.
template <typename T, int P>
struct ModeTab {
    T dual[P + 1][P + 1];
    T weight[P + 1];
    T pw[P + 1];
    int nq;
    T post;
};

template <typename T, int D, int P>
__global__ void mode_kernel(const BlockItem* items, int nitems, int E, const T* u, int var, ModeTab<T, P> mt,
                            T* tau) {
    constexpr int P1 = P + 1;
    const int N = E * P1;
    const int NN = ipow(N, D);
    const int EE = ipow(E, D);
    int64_t total = (int64_t)nitems * EE;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        int b = (int)(i / EE), el = (int)(i % EE);
        const T* a = u + items[b].off + (int64_t)var * NN;
        int base = 0, s = 1;
        {
            int m = el;
            for (int k = 0; k < D; ++k) { base += (m % E) * P1 * s; m /= E; s *= N; }
        }
        T best = T(0);
        for (int d = 0; d < D; ++d) {
            int sd = 1;
            for (int k = 0; k < d; ++k) sd *= N;
            const int nl = ipow(P1, D - 1);
            for (int l = 0; l < nl; ++l) {
                int off = 0, ll = l, st = 1;
                for (int k = 0; k < D; ++k) {
                    if (k != d) { off += (ll % P1) * st; ll /= P1; }
                    st *= N;
                }
                T line[P1];
#pragma unroll
                for (int j = 0; j < P1; ++j) line[j] = a[base + off + j * sd];
                for (int q = 0; q < mt.nq; ++q) {
                    T c = T(0);
#pragma unroll
                    for (int j = 0; j < P1; ++j) c += mt.dual[q][j] * line[j];
                    T x = mt.weight[q] * (c < T(0) ? -c : c);
                    T v = mt.pw[q] == T(1) ? x : (T)pow((double)x, (double)mt.pw[q]);
                    best = v > best ? v : best;
                }
            }
        }
        tau[i] = mt.post * best;
    }
}

// The modal indicator with the block staged in shared memory: one CTA a
// block (grid-stride), the variable's N^D values read once with coalesced
// loads, then one thread an (element, dimension) pair (the element index
// fastest), which takes every line of the element along that dimension and
// keeps each mode's largest |c_q| in registers; the weight and power are
// applied once per element and mode: the power is monotone and the weight
// non-negative, so the largest (w |c|)^p over the lines is (w max |c|)^p.
// smem: N^D values and D E^D nq words.
template <typename T, int D, int P>
__global__ void __launch_bounds__(256) mode_staged_kernel(const BlockItem* items, int nitems, int E, const T* u,
                                                         int var, ModeTab<T, P> mt, T* tau) {
    constexpr int P1 = P + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = E * P1;
    const int NN = ipow(N, D);
    const int EE = ipow(E, D);
    const int nl = ipow(P1, D - 1);
    const int nq = mt.nq;
    T* sv = reinterpret_cast<T*>(smem_raw);
    T* best = sv + ((NN + 3) & ~3);
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const T* a = u + items[item].off + (int64_t)var * NN;
        for (int n = threadIdx.x; n < NN; n += blockDim.x) sv[n] = a[n];
        __syncthreads();
        for (int li = threadIdx.x; li < D * EE; li += blockDim.x) {
            const int e = li % EE, d = li / EE;
            int base = 0, s = 1, m = e, sd = 1;
            int st[2] = {0, 0}, nt = 0;   // the strides of the line's two other dimensions
            for (int k = 0; k < D; ++k) {
                base += (m % E) * P1 * s;
                m /= E;
                if (k == d) sd = s;
                else st[nt++] = s;
                s *= N;
            }
            T top[P1];
#pragma unroll
            for (int q = 0; q < P1; ++q) top[q] = T(0);
            for (int l = 0; l < nl; ++l) {
                const int off = base + (l % P1) * st[0] + (D == 3 ? (l / P1) * st[1] : 0);
                T line[P1];
#pragma unroll
                for (int j = 0; j < P1; ++j) line[j] = sv[off + j * sd];
#pragma unroll
                for (int q = 0; q < P1; ++q) {
                    if (q < nq) {
                        T c = T(0);
#pragma unroll
                        for (int j = 0; j < P1; ++j) c += mt.dual[q][j] * line[j];
                        c = c < T(0) ? -c : c;
                        top[q] = c > top[q] ? c : top[q];
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < P1; ++q)
                if (q < nq) best[(d * EE + e) * nq + q] = top[q];
        }
        __syncthreads();
        for (int e = threadIdx.x; e < EE; e += blockDim.x) {
            T out = T(0);
#pragma unroll
            for (int q = 0; q < P1; ++q) {
                if (q < nq) {
                    T c = best[e * nq + q];
                    for (int d = 1; d < D; ++d) {
                        const T cd = best[(d * EE + e) * nq + q];
                        c = cd > c ? cd : c;
                    }
                    const T x = mt.weight[q] * c;
                    const T v = mt.pw[q] == T(1) ? x : (T)pow((double)x, (double)mt.pw[q]);
                    out = v > out ? v : out;
                }
            }
            tau[(int64_t)item * EE + e] = mt.post * out;
        }
        __syncthreads();
    }
}

// The largest |x| is exact in the field's own type, so the comparisons run
// in it and only the block's result is widened to FP64.
template <typename T, int D>
__global__ void maxabs_kernel(const BlockItem* items, int nitems, int NN, const T* u, int var, double* part) {
    __shared__ double red[32];
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const T* a = u + items[item].off + (int64_t)var * NN;
        T mt = T(0);
        for (int n = threadIdx.x; n < NN; n += blockDim.x) {
            const T x = a[n];
            mt = fmax(mt, x < T(0) ? -x : x);
        }
        double m = (double)mt;
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (lane == 0) red[wid] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0;
            for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) s = fmax(s, red[w]);
            part[item] = s;
        }
        __syncthreads();
    }
}

// Standalone truncation of v (twoldg_truncate): one block per CTA, v staged
// in shared memory in the ghost-free layout.
template <typename T, int D, int P>
__global__ void truncate_kernel(const BlockItem* items, int nitems, int E, T* u, Tab<T, P> tb, const T* trm,
                                const T* trd) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sv = reinterpret_cast<T*>(smem_raw);
    using G = ShapeR<D, P>;
    G g(E);
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        T* v = u + items[item].off + g.NN;
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<D>(g, n, x);
            sv[lidx<D>(g, x)] = v[n];
        }
        __syncthreads();
        truncate_block<T, D, P, false, 0>(g, tb, sv, nullptr, trm, trd, item, nitems);
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<D>(g, n, x);
            v[n] = sv[lidx<D>(g, x)];
        }
        __syncthreads();
    }
}

}  // namespace twoldg
