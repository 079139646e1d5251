// The fused RK stage for 3D blocks with a compile-time shape, whole element
// lines in registers. One thread per (a, b) position of the block's N x N
// cross-section; in direction d a thread owns the complete line of N nodes
// at its tangential position (all E elements), so it holds the line of u,
// its gradient D_d u (with the two gradient ghosts, all without the factor
// 1/h, which the Laplacian takes once as 1/h^2) and the Laplacian term
// D_d D_d u in registers: the gradient never goes through shared memory.
// The z direction is the thread's own column, loaded from global memory
// straight into registers, so it touches shared memory only to add its
// Laplacian term; x and y lines read u from the padded shared copy and add
// their terms into the ghost-free accumulator.
//
// The RK combination runs element by element along the column, where the
// truncation along z is applied in registers; along x and y it is applied
// afterwards in shared memory. The dimensions commute, so this is the same
// projector as the generic kernel's (which applies x, y, z in turn) up to
// rounding.
#pragma once

#include "kernels.cuh"

namespace twoldg {

// A pitch of at least `lo` words that keeps 16-byte shared accesses
// conflict-free when consecutive threads step by it: a multiple of the
// vector width whose byte offset, in 4-byte banks modulo 32, is 4, 12, 20 or
// 28 (the eight threads of a 16-byte phase then take disjoint bank quads).
template <typename T>
constexpr int vec_pitch(int lo) {
    constexpr int VW = 16 / sizeof(T);
    for (int x = lo;; ++x) {
        if (x % VW) continue;
        const int b = (int)((x * sizeof(T) / 4) % 32);
        if (b == 4 || b == 12 || b == 20 || b == 28) return x;
    }
}

// A plane stride of at least `lo` words, a multiple of the vector width,
// whose byte offset is 64 modulo 128: the two 16-thread rows of a warp that
// walk along a plane then fall in opposite halves of the banks.
template <typename T>
constexpr int half_bank_stride(int lo) {
    constexpr int VW = 16 / sizeof(T);
    for (int x = lo;; ++x)
        if (x % VW == 0 && (x * sizeof(T)) % 128 == 64) return x;
}

// The L2 prefetch of a block's stage operands (and of the column source of
// the CTA's next block), as the register-line kernel reads them: u^n in
// stages 1 and 2, k1_v in stage 2, the stage input, u^n and the increments in
// stages 3 and 4, the compensation in stage 4.
template <typename T>
__device__ __forceinline__ void prefetch_stage3r(const StageArgs<T>& a, int item, int64_t NN, int stride = 0) {
    const int mode = a.mode;
    const int64_t off = a.items[item].off;
    const size_t w = (size_t)NN * sizeof(T);
    prefetch_l2(a.u + off, 2 * w);
    if (mode == 2) prefetch_l2(a.y + off + NN, w);
    if (mode == 3 || mode == MODE_STAGE4) {
        prefetch_l2(a.y + off, 2 * w);
        prefetch_l2(a.acc + off, 2 * w);
        if (mode == MODE_STAGE4 && a.comp) prefetch_l2(a.comp + off, 2 * w);
    }
    const int nxt = item + (stride ? stride : (int)gridDim.x);
    if (nxt < a.nitems) {
        const T* src = (mode == 3 || mode == MODE_STAGE4) ? a.y : a.u;
        prefetch_l2(src + a.items[nxt].off, 2 * w);
    }
}

template <typename T, int P, int E, bool COMP, bool LEAN = false>
struct Stage3R {
    static constexpr int P1 = P + 1;
    static constexpr int N = E * P1;
    static constexpr int F = N * N;
    static constexpr int NN = N * F;
    static constexpr int VW = 16 / sizeof(T);
    // padded u: x pitch SX (the two x ghosts and 16-byte rows), y pitch SXY
    // over N + 2 rows (the two y ghosts); z planes 0 .. N-1 only, since the
    // z ghosts stay in registers
    static constexpr int SX = vec_pitch<T>(N + 3), SY = N + 2;
    static constexpr int SXY = half_bank_stride<T>(SX * SY);
    static constexpr int SS = SXY * N;
    // ghost-free accumulator / new v: x pitch LX, plane stride LXY
    static constexpr int LX = vec_pitch<T>(N), LXY = half_bank_stride<T>(LX * N);
    static constexpr int LS = LXY * N;
    static constexpr int NT = F;
    // u, the accumulator / new v, and (compensated) the compensation of v
    static constexpr size_t words = (size_t)SS + (size_t)LS + (COMP ? (size_t)LS : 0);
    static constexpr size_t bytes = words * sizeof(T) + 1024;
    static constexpr int by_smem = (int)((227 * 1024) / bytes);
    // registers a thread may use: 80, or 64 in the lean variant that stage 1
    // runs where that lets one more CTA onto an SM (stage 1 moves the least
    // data and waits the longest; the others run best at 80)
    static constexpr int REGS = LEAN ? 64 : 80;
    static constexpr int by_regs = 65536 / (NT * REGS) > 0 ? 65536 / (NT * REGS) : 1;
    static constexpr int MINB = by_smem < 1 ? 1 : (by_smem < by_regs ? by_smem : by_regs);
    static constexpr bool usable = F >= 64 && F <= 1024 && F % 32 == 0;
};

// Derivative of a whole line held in registers: in[0] and in[N+1] are the
// values beyond the two faces (ghosts), in[1..N] the line; out[i] is the wide
// derivative at node i, scaled by s.
template <typename T, int P, int E>
__device__ __forceinline__ void line_full(const Tab<T, P>& tb, const T (&in)[E * (P + 1) + 2],
                                          T (&out)[E * (P + 1)], T s) {
    constexpr int P1 = P + 1;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        T w[P + 3], o[P + 1];
#pragma unroll
        for (int k = 0; k < P + 3; ++k) w[k] = in[e * P1 + k];
        line_derivative<T, P>(tb, w, o);
#pragma unroll
        for (int i = 0; i < P1; ++i) out[e * P1 + i] = o[i] * s;
    }
}

// The gradient ghost of face f at this thread's face point times h, from the
// value prefetched for it: the neighbour's own part `pre` plus its ghost
// coefficient times its u ghost, which is this block's own face node `own`
// (negated across a wall), or a coarse-fine face's plane of gradient values
// times h. The register-line kernels differentiate u and then its gradient
// without the two 1/h factors and scale the Laplacian by 1/h^2 once.
template <typename T, int P>
__device__ __forceinline__ T grad_ghost_raw(const Tab<T, P>& tb, uint32_t flags, int nslot, int f, T pre, T own,
                                            T h) {
    if (flags & (1u << f)) return pre * h;
    const T gnb = pre + ghost_coef<T, P>(tb, nslot & 1) * own;
    return (flags & (1u << (8 + f))) ? -gnb : gnb;
}

// The truncation of the E element lines of a thread's line in shared memory
// (base b, stride ls), with the compensation's two-sum in stage 4; VEC: the
// line is contiguous and each element's P+1 nodes are whole 16-byte words.
template <typename T, int P, int E, bool VEC>
__device__ __forceinline__ void truncate_lines(const Tab<T, P>& tb, T* sl, T* sc, int b, int ls, bool final_comp) {
    constexpr int P1 = P + 1, VW = 16 / sizeof(T);
    using V = typename V16<T>::type;
    auto load = [&](const T* p, int b0, T (&v)[P1]) {
        if constexpr (VEC) {
#pragma unroll
            for (int k = 0; k < P1; k += VW) {
                const V t = *reinterpret_cast<const V*>(p + b0 + k);
                const T* e = reinterpret_cast<const T*>(&t);
#pragma unroll
                for (int q = 0; q < VW; ++q) v[k + q] = e[q];
            }
        } else {
#pragma unroll
            for (int q = 0; q < P1; ++q) v[q] = p[b0 + q * ls];
        }
    };
    auto store = [&](T* p, int b0, const T (&v)[P1]) {
        if constexpr (VEC) {
#pragma unroll
            for (int k = 0; k < P1; k += VW) {
                V t;
                T* e = reinterpret_cast<T*>(&t);
#pragma unroll
                for (int q = 0; q < VW; ++q) e[q] = v[k + q];
                *reinterpret_cast<V*>(p + b0 + k) = t;
            }
        } else {
#pragma unroll
            for (int q = 0; q < P1; ++q) p[b0 + q * ls] = v[q];
        }
    };
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int b0 = b + e * P1 * ls;
        T v[P1];
        load(sl, b0, v);
        T c = T(0);
#pragma unroll
        for (int q = 0; q < P1; ++q) c += tb.td[q] * v[q];
        if (final_comp) {
            T w[P1];
            load(sc, b0, w);
            T cc = T(0);
#pragma unroll
            for (int q = 0; q < P1; ++q) cc += tb.td[q] * w[q];
            c += cc;
#pragma unroll
            for (int q = 0; q < P1; ++q) {
                T s, err;
                two_sum(v[q], -(tb.tm[q] * c), s, err);
                v[q] = s;
                w[q] += err;
            }
            store(sc, b0, w);
        } else {
#pragma unroll
            for (int q = 0; q < P1; ++q) v[q] = v[q] - tb.tm[q] * c;
        }
        store(sl, b0, v);
    }
}

// The coarse-fine epilogue of a block's stage: for each of its coarse-fine
// faces, the images of its new face values that the next stage's ghosts are
// made of, written into the next stage's planes. The gradient ghost of the
// flat problem's coupling is the image of the other side's face gradient, its
// own part plus its ghost coefficient times its u ghost over its spacing,
// and that u ghost is the image of this side's face nodes (dense_fill,
// dense_point); by linearity it splits into the image of the other side's
// own part, which that side writes, and the image of this side's u passed
// there and back, which this side writes:
// - a fine side writes into the coarse side's planes, over its quarter, the
//   R images of its u and of its own gradient part over its spacing, and
//   into its own gsd plane the I image of the R image of its u, times its
//   ghost coefficient over the coarse spacing;
// - a coarse side writes into each fine side's planes the I images of its u
//   and of its own gradient part over its spacing, and into its own gsd
//   plane the R image of the I images of its u, times its ghost coefficient
//   over the fine spacing.
// The block's new u sits in the padded shared copy `su`; the tables, the
// face's planes and the images use the accumulator `sl` as scratch. Every
// thread passes every barrier; the face loop is uniform in the CTA.
template <typename T, int P, int E, class S>
__device__ __forceinline__ void cf_epilogue(const StageArgs<T>& a, const Tab<T, P>& tb, const CfTab<T, P>& ct,
                                            int slot, uint32_t flags, int tid, const T* su, T* sl, int s0, int s1,
                                            int s2) {
    constexpr int N = S::N, F = S::F, H = N / 2, halfE = E / 2, NT = S::NT;
    constexpr int SX = S::SX, SXY = S::SXY;
    constexpr int kTabWords = (int)(sizeof(CfTab<T, P>) / sizeof(T));
    CfTab<T, P>* sct = reinterpret_cast<CfTab<T, P>*>(sl);
    T* U = sl + kTabWords;   // the face's new u
    T* G = U + F;            // its own gradient part
    T* X = G + F;            // R(u) (H^2 words) or I(u) (4 F words)
    stage_cftab<T, P>(ct, sct, tid, NT);
    int n[2] = {tid % N, tid / N};   // this thread's node of a face plane
#pragma unroll 1
    for (int f = 0; f < 6; ++f) {
        if (!(flags & (1u << f))) continue;
        const CfFace& face = a.cf[a.cfidx[slot + f]];
        const int d = f >> 1, side = f & 1;
        const int sd = d == 0 ? 1 : d == 1 ? SX : SXY;
        const int base = (d == 0 ? s0 : d == 1 ? s1 : s2) + (side ? N - 1 - P : 0) * sd;
        T e[P + 1];
#pragma unroll
        for (int k = 0; k <= P; ++k) e[k] = su[base + k * sd];
        U[tid] = side == 0 ? e[0] : e[P];
        G[tid] = own_face_part<T, P>(tb, side, e);
        __syncthreads();
        const T gco = ghost_coef<T, P>(tb, 1 - face.side);
        if (face.kind == 0) {
            // this block is the fine side: the coarse nodes of its quarter
            const T inv_h = T(1) / T(face.h);
            for (int m = tid; m < H * H; m += NT) {
                const int c[2] = {((face.sub & 1) ? H : 0) + m % H, ((face.sub & 2) ? H : 0) + m / H};
                const T ru = restrict_at<T, 2, P>(*sct, c, N, halfE, U);
                const T rg = restrict_at<T, 2, P>(*sct, c, N, halfE, G);
                const int64_t o = (int64_t)face.src[0] * F + c[0] + N * c[1];
                a.ugd_out[o] = ru;
                a.ggd_out[o] = rg * inv_h;
                X[m] = ru;
            }
            __syncthreads();
            const T k = gco * (T(1) / T(2.0 * face.h));
            a.gsd_out[(int64_t)(slot + f) * F + tid] = k * prolong_at<T, 2, P>(*sct, n, 0, H, halfE, X);
        } else {
            // the coarse side: every node of the four fine faces across it
            const T inv_h = T(1) / T(face.h);
            for (int i = tid; i < 4 * F; i += NT) {
                const int q = i / F, tt = i % F;
                const int c[2] = {tt % N, tt / N};
                const T iu = prolong_at<T, 2, P>(*sct, c, q, N, halfE, U);
                const T ig = prolong_at<T, 2, P>(*sct, c, q, N, halfE, G);
                const int64_t o = (int64_t)face.src[q] * F + tt;
                a.ugd_out[o] = iu;
                a.ggd_out[o] = ig * inv_h;
                X[i] = iu;
            }
            __syncthreads();
            int bits = 0;
            for (int kk = 0; kk < 2; ++kk) bits |= ((n[kk] / (P + 1)) / halfE) << kk;
            const T k = gco * (T(1) / T(0.5 * face.h));
            a.gsd_out[(int64_t)(slot + f) * F + tid] = k * restrict_at<T, 2, P>(*sct, n, N, halfE, X + bits * F);
        }
        __syncthreads();
    }
}

// FM: the stage the instantiation runs (1-4), so that each stage's code holds
// only its own data flow, or 0 for the mode in the arguments (the right-hand
// side). CFP (a stage of a forest with refinement): the ghosts of the block's
// coarse-fine faces are read from planes that the previous stage's epilogues
// wrote, u's from ugd and the gradient's as the other side's part ggd plus
// this block's own part gsd, and the block's epilogue writes the next
// stage's (cf_epilogue); without it ugd and ggd are complete, filled by a
// launch of their own, and a uniform forest never reads them.
template <typename T, int P, int E, bool COMP, bool LEAN = false, int FM = 0, bool CFP = false>
__global__ void __launch_bounds__(Stage3R<T, P, E, COMP, LEAN>::NT, Stage3R<T, P, E, COMP, LEAN>::MINB)
    stage3r_kernel(StageArgs<T> a, Tab<T, P> tb, CfTab<T, P> ct) {
    using S = Stage3R<T, P, E, COMP, LEAN>;
    constexpr int P1 = S::P1, N = S::N, F = S::F, NN = S::NN, VW = S::VW;
    // the epilogue's scratch (the tables, a face's new u and own gradient
    // part, and its images, 4 F words at most) lives in the accumulator,
    // free once the block's new v is stored
    constexpr int kTabWords = (int)(sizeof(CfTab<T, P>) / sizeof(T));
    static_assert(!CFP || S::LS >= kTabWords + 6 * F, "the accumulator holds the coarse-fine scratch");
    constexpr int SX = S::SX, SXY = S::SXY, LX = S::LX, LXY = S::LXY;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* su = reinterpret_cast<T*>(smem_raw);
    T* sl = su + S::SS;
    T* sc = sl + S::LS;  // compensated only
    const int tid = threadIdx.x;
    const int ca = tid % N, cb = tid / N;
    // padded index of x_d = 0 on this thread's line along d, and the strides
    // padded index of (x0, x1, x2) is (x0 + 1) + SX (x1 + 1) + SXY x2
    const int s0 = 1 + SX * (ca + 1) + SXY * cb;         // x-line (x1, x2) = (ca, cb)
    const int s1 = (ca + 1) + SX + SXY * cb;             // y-line (x0, x2) = (ca, cb)
    const int s2 = (ca + 1) + SX * (cb + 1);             // z-line (x0, x1) = (ca, cb)
    const int l0 = LX * ca + LXY * cb;
    const int l1 = ca + LXY * cb;
    const int l2 = ca + LX * cb;
    const int mode = FM ? FM : a.mode;
    // The stage's data flow. Stage 1 stores only the stage derivative's v
    // part k1_v, truncated, in the v half of `y` (its u part is u^n's own v):
    // stage 2 forms Y2 = u^n + dt/2 k1 and the first increment dt/6 k1 from
    // u^n, which it reads anyway, and k1_v, so neither Y2 nor the increment
    // goes through HBM (8 words a node instead of 14 over the two stages in
    // FP32). The truncation acts on k1_v instead of on Y2's v, the same by
    // linearity since u^n's v is truncated. Stages 3 and 4 read Y3, Y4 and
    // the increments as stored.
    const T* ysrc = (mode == MODE_RHS || mode == MODE_STAGE1 || mode == 2) ? a.u : a.y;
    const T* vsrc = mode == 2 ? a.y : ysrc;

    // the first block's operands are asked into L2 (a hint: L2 is where the
    // previous stage's writes land, so nothing stale is read) before the
    // wait on the previous stage, so that under a programmatic launch their
    // reads overlap that stage's last CTAs
    if (tid == 0 && (int)blockIdx.x < a.nitems) prefetch_stage3r<T>(a, blockIdx.x, NN);
    grid_dependency_wait();
    if (a.release) grid_dependents_launch();
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        const uint32_t flags = it.flags;
        const int slot = it.slot;
        int nb[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) nb[f] = it.nb[f];
        // the two passes differentiate without 1/h; the Laplacian takes 1/h^2
        const T hb = T(it.h);
        const T inv_h = T(1) / hb;
        const T inv_h2 = inv_h * inv_h;
        const T* yu = ysrc + it.off;
        if (tid == 0 && item != (int)blockIdx.x) prefetch_stage3r<T>(a, item, NN);
        // every global load of the block's prologue at once: the column, the u
        // ghosts and the neighbours' gradient parts at this face point
        T line[N + 2];
        if (mode == 2) {
            // Y2's u, dt/2 k1_u = dt/2 v^n added to u^n
            const T cn1 = a.rk[4 * it.problem + 2];
#pragma unroll
            for (int j = 0; j < N; ++j) line[1 + j] = yu[tid + F * j] + cn1 * yu[NN + tid + F * j];
        } else {
#pragma unroll
            for (int j = 0; j < N; ++j) line[1 + j] = yu[tid + F * j];
        }
        T ug[6], gp[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            if (flags & (1u << f)) {
                const int64_t o = (int64_t)(slot + f) * F + tid;
                ug[f] = a.ugd[o];
                gp[f] = CFP ? a.ggd[o] + a.gsd[o] : a.ggd[o];
            } else {
                ug[f] = a.fu_in[(int64_t)nb[f] * F + tid];
                gp[f] = a.fog_in[(int64_t)nb[f] * F + tid];
            }
        }
        // ---- z: the column in registers (stage 1 keeps a copy: its RK
        // combination reads u^n's u, which is this column, from registers)
        T col[FM == 1 ? N : 1];
        if constexpr (FM == 1) {
#pragma unroll
            for (int j = 0; j < N; ++j) col[j] = line[1 + j];
        }
        {
#pragma unroll
            for (int j = 0; j < N; ++j) su[s2 + SXY * j] = line[1 + j];
            su[s0 - 1] = ug[0];
            su[s0 + N] = ug[1];
            su[s1 - SX] = ug[2];
            su[s1 + N * SX] = ug[3];
            line[0] = ug[4];
            line[N + 1] = ug[5];
            T g[N + 2], gi[N], lap[N];
            line_full<T, P, E>(tb, line, gi, T(1));
#pragma unroll
            for (int j = 0; j < N; ++j) g[1 + j] = gi[j];
            g[0] = grad_ghost_raw<T, P>(tb, flags, nb[4], 4, gp[4], line[1], hb);
            g[N + 1] = grad_ghost_raw<T, P>(tb, flags, nb[5], 5, gp[5], line[N], hb);
            line_full<T, P, E>(tb, g, lap, T(1));
#pragma unroll
            for (int j = 0; j < N; ++j) sl[l2 + LXY * j] = lap[j];
        }
        __syncthreads();
        // ---- x and y lines from the shared copy of u
#pragma unroll
        for (int d = 0; d < 2; ++d) {
            const int sb = d == 0 ? s0 : s1;
            const int ss = d == 0 ? 1 : SX;
            const int lb = d == 0 ? l0 : l1;
            const int ls = d == 0 ? 1 : LX;
            T g[N + 2], gi[N], lap[N];
            if (d == 0) {
                // the x line is contiguous and 16-byte aligned: vector loads
                using V = typename V16<T>::type;
#pragma unroll
                for (int k = 0; k + VW <= N + 2; k += VW) {
                    const V v = *reinterpret_cast<const V*>(su + sb - 1 + k);
                    const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
                    for (int q = 0; q < VW; ++q) line[k + q] = e[q];
                }
#pragma unroll
                for (int k = (N + 2) / VW * VW; k < N + 2; ++k) line[k] = su[sb - 1 + k];
            } else {
#pragma unroll
                for (int k = 0; k < N + 2; ++k) line[k] = su[sb + (k - 1) * ss];
            }
            line_full<T, P, E>(tb, line, gi, T(1));
#pragma unroll
            for (int j = 0; j < N; ++j) g[1 + j] = gi[j];
            g[0] = grad_ghost_raw<T, P>(tb, flags, nb[2 * d], 2 * d, gp[2 * d], line[1], hb);
            g[N + 1] = grad_ghost_raw<T, P>(tb, flags, nb[2 * d + 1], 2 * d + 1, gp[2 * d + 1], line[N], hb);
            line_full<T, P, E>(tb, g, lap, T(1));
            if (d == 0 && N % VW == 0) {
                using V = typename V16<T>::type;
#pragma unroll
                for (int j = 0; j < N; j += VW) {
                    V* pv = reinterpret_cast<V*>(sl + lb + j);
                    V v = *pv;
                    T* e = reinterpret_cast<T*>(&v);
#pragma unroll
                    for (int q = 0; q < VW; ++q) e[q] += lap[j + q];
                    *pv = v;
                }
            } else {
#pragma unroll
                for (int j = 0; j < N; ++j) sl[lb + ls * j] += lap[j];
            }
            __syncthreads();
        }
        const T* yv = vsrc + it.off + NN;
        if (mode == MODE_RHS) {
            T* du = a.du + it.off;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                du[tid + F * j] = yv[tid + F * j];
                du[NN + tid + F * j] = sl[l2 + LXY * j] * inv_h2;
            }
            __syncthreads();
            continue;
        }
        // ---- the RK combination along the column, element by element, with the
        // truncation along z in registers
        const RkCoef<T> rc(mode, a.rk + 4 * it.problem);
        const RkCoef<T> rc1(1, a.rk + 4 * it.problem);   // dt/6 and dt/2
        const T* __restrict__ un = a.u + it.off;
        T* __restrict__ acc = a.acc + it.off;
        T* __restrict__ comp = COMP ? a.comp + it.off : nullptr;
        const bool final_comp = COMP && mode == MODE_STAGE4;
        // the new u is final here (the truncation acts on v only): stages 1-3
        // store it from registers as each element is done; stage 4, which
        // writes u^n in place, stores it with v at the end (measured faster)
        T* out = (mode == MODE_STAGE4 ? a.u : a.y) + it.off;
        const bool early_u = mode == 2 || mode == 3;
#pragma unroll
        for (int ez = 0; ez < E; ++ez) {
            T y[P1], uu[P1], uv[P1], au[P1], av[P1], cu[P1], cvi[P1];
#pragma unroll
            for (int q = 0; q < P1; ++q) {
                const int n = tid + F * (ez * P1 + q);
                y[q] = yv[n];
                if (mode == MODE_STAGE1) {
                    // the stage input is u^n: its u is the column (kept in
                    // registers by the stage-1 instantiation, else in shared
                    // memory), its v the value just loaded
                    if constexpr (FM == 1) uu[q] = col[ez * P1 + q];
                    else uu[q] = su[s2 + SXY * (ez * P1 + q)];
                    uv[q] = y[q];
                } else {
                    uu[q] = un[n];
                    uv[q] = un[NN + n];
                }
                if (mode == 2) {
                    // y[q] holds k1_v: Y2's v and the first increment
                    const T k1v = y[q];
                    y[q] = uv[q] + rc1.cn * k1v;
                    au[q] = rc1.ca * uv[q];
                    av[q] = rc1.ca * k1v;
                } else if (mode != 1) {
                    au[q] = acc[n];
                    av[q] = acc[NN + n];
                }
                if (final_comp) {
                    cu[q] = comp[n];
                    cvi[q] = comp[NN + n];
                }
            }
            T nu[P1], nv[P1], cv[P1];
#pragma unroll
            for (int q = 0; q < P1; ++q) {
                const int j = ez * P1 + q;
                T lap[1] = {sl[l2 + LXY * j]};
                T o_u[1], o_v[1], o_c[1];
                T yq[1] = {y[q]}, uuq[1] = {uu[q]}, uvq[1] = {uv[q]}, auq[1] = {au[q]}, avq[1] = {av[q]},
                  cuq[1] = {cu[q]}, cviq[1] = {cvi[q]};
                if (mode == MODE_STAGE1) {
                    // Y2's u for the face export; the stage derivative's v,
                    // truncated below and stored
                    o_u[0] = uuq[0] + rc.cn * yq[0];
                    o_v[0] = lap[0] * inv_h2;
                    o_c[0] = T(0);
                } else {
                    stage_points<T, COMP, 1>(mode, rc, yq, uuq, uvq, auq, avq, cuq, cviq, lap, inv_h2, o_u, o_v,
                                             o_c);
                }
                au[q] = auq[0];
                av[q] = avq[0];
                cu[q] = cuq[0];
                nu[q] = o_u[0];
                nv[q] = o_v[0];
                cv[q] = o_c[0];
            }
            if (a.truncate) {
                T c = T(0);
#pragma unroll
                for (int q = 0; q < P1; ++q) c += tb.td[q] * nv[q];
                if (final_comp) {
                    T cc = T(0);
#pragma unroll
                    for (int q = 0; q < P1; ++q) cc += tb.td[q] * cv[q];
                    c += cc;
#pragma unroll
                    for (int q = 0; q < P1; ++q) {
                        T s, err;
                        two_sum(nv[q], -(tb.tm[q] * c), s, err);
                        nv[q] = s;
                        cv[q] += err;
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < P1; ++q) nv[q] = nv[q] - tb.tm[q] * c;
                }
            }
#pragma unroll
            for (int q = 0; q < P1; ++q) {
                const int j = ez * P1 + q;
                const int n = tid + F * j;
                if (mode == 2 || mode == 3) {
                    acc[n] = au[q];
                    acc[NN + n] = av[q];
                }
                if (final_comp) comp[n] = cu[q];
                if (early_u) out[n] = nu[q];
                su[s2 + SXY * j] = nu[q];
                sl[l2 + LXY * j] = nv[q];
                if (final_comp) sc[l2 + LXY * j] = cv[q];
            }
            // the column's own z faces from the first and the last element,
            // still in registers
            if (ez == 0 || ez == E - 1) {
                const int side = ez == 0 ? 0 : 1;
                const int64_t o = (int64_t)(slot + 4 + side) * F + tid;
                a.fu_out[o] = side == 0 ? nu[0] : nu[P];
                a.fog_out[o] = own_face_part<T, P>(tb, side, nu);
            }
        }
        __syncthreads();
        // ---- face export of the new u on the x and y faces (reads su only)
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            const int d = f >> 1, side = f & 1;
            const int sd = d == 0 ? 1 : d == 1 ? SX : SXY;
            const int base = (d == 0 ? s0 : d == 1 ? s1 : s2) + (side ? N - 1 - P : 0) * sd;
            T e[P + 1];
#pragma unroll
            for (int k = 0; k <= P; ++k) e[k] = su[base + k * sd];
            const int64_t o = (int64_t)(slot + f) * F + tid;
            a.fu_out[o] = side == 0 ? e[0] : e[P];
            a.fog_out[o] = own_face_part<T, P>(tb, side, e);
        }
        // ---- truncation along x, then y, in shared memory
        if (a.truncate) {
            truncate_lines<T, P, E, (P1 % VW == 0)>(tb, sl, sc, l0, 1, final_comp);
            __syncthreads();
            truncate_lines<T, P, E, false>(tb, sl, sc, l1, LX, final_comp);
            __syncthreads();
        }
        // ---- the new v of the column (and in stage 4 its u)
#pragma unroll
        for (int j = 0; j < N; ++j) {
            if (mode == MODE_STAGE4) out[tid + F * j] = su[s2 + SXY * j];
            out[NN + tid + F * j] = sl[l2 + LXY * j];
            if (final_comp) comp[NN + tid + F * j] = sc[l2 + LXY * j];
        }
        __syncthreads();
        if constexpr (CFP) {
            if (flags & 0x3fu) cf_epilogue<T, P, E, S>(a, tb, ct, slot, flags, tid, su, sl, s0, s1, s2);
        }
    }
}

// The register-line stage of a forest with refinement (CFP), instantiated
// per order in a translation unit of its own (kernels_d3_p<P>_cf.cu): its
// shared-memory attributes, set once per device, and a launch of RK stage
// `mode` (1 to 4), as a programmatic dependent launch when `pdl` is set.
template <typename T, int P, bool COMP>
void stage3r_cf_attrs(int max_smem);
template <typename T, int P, int E, bool COMP>
cudaError_t stage3r_cf_launch(const StageArgs<T>& a, const Tab<T, P>& tb, const CfTab<T, P>& ct, int grid,
                              int mode, cudaStream_t s, bool pdl);

}  // namespace twoldg
