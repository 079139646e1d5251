// The particle-grid transfer's device passes (src/transfer.jl:520-680,
// 1215-1378): the tensor rules (far and graded) fused into one kernel that
// evaluates the source at an element's q^D Gauss points into shared memory
// and contracts them there, and the nested rule over the host's innermost
// lines (per line a reduction against the last dimension's Lagrange
// polynomials and one outer product; per chunk of lines the per-node sums;
// per element the chunks added in order).
//
// On GB300 these passes are bound by the FP64 pipe, not by HBM: the kernels
// are shaped to spend as few double-precision operations per point as the
// rules allow.
#include <algorithm>

#include "transfer.h"

namespace twoldg {

namespace {

constexpr int kRuleThreads = 128;
constexpr int kLineThreads = 128;   // 16 groups of kGroup lanes
constexpr int kGroup = 8;           // lanes per line
constexpr int kFinishThreads = 256;

template <typename T, int D>
__device__ __forceinline__ void element_box(const TransferLaunch& a, int b, const int32_t* e, T (&lo)[D], T (&hi)[D]) {
    const T* org = static_cast<const T*>(a.origins);
    const T h = static_cast<const T*>(a.spacings)[b];
    const int P1 = a.P + 1;
    // both faces as origin + h (multiple of P+1), so neighbouring elements
    // share their faces bit for bit (src/transfer.jl:505-513)
#pragma unroll
    for (int d = 0; d < D; ++d) {
        lo[d] = org[(int64_t)b * D + d] + h * T(e[d] * P1);
        hi[d] = org[(int64_t)b * D + d] + h * T((e[d] + 1) * P1);
    }
}

// The particles' density at x: sum_k Q_k rho0(|L(v_k)(x - z_k)|^2, ell_k),
// rho0(q, l) = l^-3 (3465/512) (1 - q/l^2)^4 / pi inside the support and 0
// outside (src/particle.jl:117-127; src/particle_forms.jl:29-37).
template <typename T>
__device__ __forceinline__ T density(const TransferLaunch& a, T x0, T x1, T x2) {
    T s = T(0);
    for (int k = 0; k < a.nparticles; ++k) {
        const TransferParticle& p = a.particles[k];
        const T r0 = x0 - T(p.z[0]), r1 = x1 - T(p.z[1]), r2 = x2 - T(p.z[2]);
        const T f = T(p.g) * (T(p.v[0]) * r0 + T(p.v[1]) * r1 + T(p.v[2]) * r2);
        const T y0 = r0 + f * T(p.v[0]), y1 = r1 + f * T(p.v[1]), y2 = r2 + f * T(p.v[2]);
        const T q = y0 * y0 + y1 * y1 + y2 * y2;
        const T l = T(p.ell);
        if (q < l * l) {
            const T u = T(1) - q / (l * l);
            const T poly = (((T(3465) / T(512)) * u) * u * u) * u;
            s += T(p.charge) * (poly / (l * l * l) / T(3.141592653589793238462643383279502884));
        }
    }
    return s;
}

// One CTA per far or graded element: S at the rule's q^D points, then the
// contraction with contract[i][k] = w_k phi_i(x_k) / w^_i one dimension at a
// time (the sum over k in order, src/transfer.jl:592-621), and factor times
// the element's P S added to variable `var` of du.
template <typename T, int D, int SRC>
__global__ void __launch_bounds__(kRuleThreads) tensor_rule_kernel(const TransferLaunch a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    const RuleElement el = a.rule_elems[blockIdx.x];
    const int q = a.rule_q[el.rule];
    const int P1 = a.P + 1;
    // the buffers hold q^D values, and P+1 per dimension once contracted
    const int cq = a.max_q > P1 ? a.max_q : P1;
    int cap = 1;
    for (int d = 0; d < D; ++d) cap *= cq;
    T* buf0 = reinterpret_cast<T*>(smem_raw);
    T* buf1 = buf0 + cap;
    T* xg = buf1 + cap;             // D x max_q point coordinates
    T* con = xg + D * a.max_q;
    const T* tables = static_cast<const T*>(a.tables);
    for (int k = tid; k < P1 * q; k += blockDim.x) con[k] = tables[a.rule_contract[el.rule] + k];
    int npts = 1;
    for (int d = 0; d < D; ++d) npts *= q;
    if (SRC == SOURCE_VALUES) {
        const T* vals = static_cast<const T*>(a.values) + el.base;
        for (int j = tid; j < npts; j += blockDim.x) buf0[j] = vals[j];
        __syncthreads();
    } else {
        // the density's elements are those that meet a support (the host's
        // list), so every one is evaluated
        T lo[D], hi[D];
        element_box<T, D>(a, el.block, el.e, lo, hi);
        for (int k = tid; k < D * q; k += blockDim.x) {
            const int d = k / q, j = k % q;
            T l = lo[0], h = hi[0];
#pragma unroll
            for (int dd = 1; dd < D; ++dd)
                if (d == dd) {
                    l = lo[dd];
                    h = hi[dd];
                }
            xg[d * a.max_q + j] = l + (h - l) * (T(1) + tables[a.rule_nodes[el.rule] + j]) / T(2);
        }
        __syncthreads();
        if constexpr (D == 3) {
            for (int j = tid; j < npts; j += blockDim.x) {
                const int j0 = j % q, j1 = (j / q) % q, j2 = j / (q * q);
                buf0[j] = density<T>(a, xg[j0], xg[a.max_q + j1], xg[2 * a.max_q + j2]);
            }
        }
        __syncthreads();
    }
    T* in = buf0;
    T* out = buf1;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        // extents: dimensions below d already contracted (P+1), d itself q in
        // and P+1 out, those above q
        int below = 1, above = 1;
        for (int k = 0; k < d; ++k) below *= P1;
        for (int k = d + 1; k < D; ++k) above *= q;
        const int nout = below * P1 * above;
        for (int o = tid; o < nout; o += blockDim.x) {
            const int lowi = o % below;
            const int i = (o / below) % P1;
            const int upi = o / (below * P1);
            const int base = lowi + below * q * upi;
            const T* c = con + i * q;
            T acc = T(0);
            for (int k = 0; k < q; ++k) acc += c[k] * in[base + below * k];
            out[o] = acc;
        }
        __syncthreads();
        T* t = in;
        in = out;
        out = t;
    }
    int M = 1;
    for (int d = 0; d < D; ++d) M *= P1;
    T* du = static_cast<T*>(a.du) + (int64_t)el.block * 2 * a.NN + (int64_t)(a.var - 1) * a.NN;
    const T factor = T(a.factor);
    for (int m = tid; m < M; m += blockDim.x) {
        int r = m;
        int64_t idx = 0, stride = 1;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int K = r % P1;
            r /= P1;
            idx += (int64_t)(el.e[d] * P1 + K) * stride;
            stride *= a.N;
        }
        du[idx] += factor * in[m];
    }
}

// phi_i(xi) for every node i, bary_i prod_{j != i} (xi - x^_j), by prefix and
// suffix products of the differences.
template <typename T, int P1>
__device__ __forceinline__ void lagrange_all(const T (&nodes)[P1], const T (&bary)[P1], T xi, T (&phi)[P1]) {
    T diff[P1], pre[P1];
#pragma unroll
    for (int j = 0; j < P1; ++j) diff[j] = xi - nodes[j];
    pre[0] = T(1);
#pragma unroll
    for (int j = 1; j < P1; ++j) pre[j] = pre[j - 1] * diff[j - 1];
    T suf = T(1);
#pragma unroll
    for (int i = P1 - 1; i >= 0; --i) {
        phi[i] = bary[i] * (pre[i] * suf);
        suf *= diff[i];
    }
}

template <typename T, int P1>
__device__ __forceinline__ T lagrange_one(const T (&nodes)[P1], const T (&bary)[P1], T xi, int i) {
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < P1; ++k) {
        if (k != i) continue;
        acc = bary[k];
#pragma unroll
        for (int j = 0; j < P1; ++j)
            if (j != k) acc *= xi - nodes[j];
    }
    return acc;
}

template <typename T>
__device__ __forceinline__ T shfl8(unsigned mask, T v, int src) {
    return __shfl_sync(mask, v, src, kGroup);
}

template <typename T>
__device__ __forceinline__ T shfl8_xor(unsigned mask, T v, int off) {
    return __shfl_xor_sync(mask, v, off, kGroup);
}

// The nested rule, one CTA per chunk of an element's innermost lines, a group
// of kGroup lanes per line: the line's points summed against the last
// dimension's Lagrange polynomials, r_i = sum_p w_p S(x_p) phi_i(x_p,last);
// then node (K_0 .. K_D-1) gets w_line prod_{d<D-1} phi_{K_d}(x_d) r_{K_D-1},
// the product of the point's line weights and Lagrange values regrouped
// (src/transfer.jl:1330-1352). The chunk's per-node sums go to partials.
template <typename T, int D, int P1, int SRC>
__global__ void __launch_bounds__(kLineThreads) near_lines_kernel(const TransferLaunch a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int M = D == 1 ? P1 : (D == 2 ? P1 * P1 : P1 * P1 * P1);
    constexpr int MO = M / P1;                       // nodes of the outer dimensions
    constexpr int NPL = (M + kGroup - 1) / kGroup;   // nodes per lane
    constexpr int NOUT = (D - 1) * P1;               // outer Lagrange values per line
    const int tid = threadIdx.x;
    const int group = tid / kGroup, lane = tid % kGroup, ngroups = blockDim.x / kGroup;
    const unsigned mask = 0xffu << ((tid % 32) / kGroup * kGroup);
    const NearChunk ch = a.chunks[blockIdx.x];
    const NearElement ne = a.near_elems[ch.elem];
    T lo[D], hi[D];
    element_box<T, D>(a, ne.block, ne.e, lo, hi);
    T sum[D], inv[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        sum[d] = lo[d] + hi[d];
        inv[d] = T(1) / (hi[d] - lo[d]);
    }
    T nodes[P1], bary[P1];
#pragma unroll
    for (int i = 0; i < P1; ++i) {
        nodes[i] = static_cast<const T*>(a.gll)[i];
        bary[i] = static_cast<const T*>(a.bary)[i];
    }
    const T* lx = static_cast<const T*>(a.near_lx);
    const T* lw = static_cast<const T*>(a.near_lw);
    const T* lv = static_cast<const T*>(a.line_vals);
    const T* vals = static_cast<const T*>(a.values);
    T acc[NPL];
#pragma unroll
    for (int k = 0; k < NPL; ++k) acc[k] = T(0);
    for (int l = ch.l0 + group; l < ch.l1; l += ngroups) {
        const NearLine L = a.lines[l];
        const T pre0 = lv[3 * (int64_t)l], pre1 = lv[3 * (int64_t)l + 1], wl = lv[3 * (int64_t)l + 2];
        T r[P1];
#pragma unroll
        for (int i = 0; i < P1; ++i) r[i] = T(0);
        for (int p = L.p0 + lane; p < L.p1; p += kGroup) {
            const T x = lx[p];
            T phi[P1];
            lagrange_all<T, P1>(nodes, bary, (T(2) * x - sum[D - 1]) * inv[D - 1], phi);
            T S;
            if (SRC == SOURCE_VALUES) {
                S = vals[a.near_base + p];
            } else {
                S = D == 3 ? density<T>(a, pre0, pre1, x) : T(0);
            }
            const T c = lw[p] * S;
#pragma unroll
            for (int i = 0; i < P1; ++i) r[i] += c * phi[i];
        }
#pragma unroll
        for (int off = kGroup / 2; off > 0; off /= 2)
#pragma unroll
            for (int i = 0; i < P1; ++i) r[i] += shfl8_xor(mask, r[i], off);
        // the outer dimensions' Lagrange values at the line's fixed
        // coordinates, value j = d (P+1) + i on lane j % kGroup
        T ov[(NOUT + kGroup - 1) / kGroup + 1];
#pragma unroll
        for (int s = 0; s * kGroup < NOUT; ++s) {
            const int j = s * kGroup + lane;
            T v = T(0);
            if (j < NOUT) {
                const int d = j / P1, i = j % P1;
                // select, not an index: the arrays stay in registers
                const T xc = d == 0 ? pre0 : pre1;
                const T sd = d == 0 ? sum[0] : sum[D > 1 ? 1 : 0];
                const T id = d == 0 ? inv[0] : inv[D > 1 ? 1 : 0];
                v = lagrange_one<T, P1>(nodes, bary, (T(2) * xc - sd) * id, i);
            }
            ov[s] = v;
        }
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
            const int m = lane + kGroup * k;
            const int mm = m < M ? m : 0;
            const int Klast = mm / MO;
            int o = mm % MO;
            T outer = wl;
#pragma unroll
            for (int d = 0; d < D - 1; ++d) {
                const int j = d * P1 + o % P1;
                o /= P1;
                T got = T(0);
#pragma unroll
                for (int s = 0; s * kGroup < NOUT; ++s) {
                    const T t = shfl8(mask, ov[s], j % kGroup);
                    if (j / kGroup == s) got = t;
                }
                outer *= got;
            }
            T rk = T(0);
#pragma unroll
            for (int i = 0; i < P1; ++i)
                if (i == Klast) rk = r[i];
            if (m < M) acc[k] += outer * rk;
        }
    }
    // the groups' sums, added in group order
    T* red = reinterpret_cast<T*>(smem_raw);   // ngroups x M
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
        const int m = lane + kGroup * k;
        if (m < M) red[group * M + m] = acc[k];
    }
    __syncthreads();
    T* partials = static_cast<T*>(a.partials) + (int64_t)blockIdx.x * M;
    for (int m = tid; m < M; m += blockDim.x) {
        T s = T(0);
        for (int g = 0; g < ngroups; ++g) s += red[g * M + m];
        partials[m] = s;
    }
}

// The nested rule's last pass: element i's chunks added in order for node m,
// split over the CTA's threads and added back in thread order, and factor
// times that over w_m added to its node (src/transfer.jl:1354-1369).
template <typename T, int D>
__global__ void __launch_bounds__(kFinishThreads) near_finish_kernel(const TransferLaunch a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* red = reinterpret_cast<T*>(smem_raw);
    const NearElement ne = a.near_elems[blockIdx.x];
    const int P1 = a.P + 1;
    int M = 1;
    for (int d = 0; d < D; ++d) M *= P1;
    const int split = M >= kFinishThreads ? 1 : kFinishThreads / M;
    const T* partials = static_cast<const T*>(a.partials);
    const T* wn = static_cast<const T*>(a.wn);
    T* du = static_cast<T*>(a.du) + (int64_t)ne.block * 2 * a.NN + (int64_t)(a.var - 1) * a.NN;
    const T factor = T(a.factor);
    for (int m0 = 0; m0 < M; m0 += kFinishThreads / split) {
        const int m = m0 + threadIdx.x / split, g = threadIdx.x % split;
        T acc = T(0);
        if (m < M)
            for (int c = ne.c0 + g; c < ne.c1; c += split) acc += partials[(int64_t)c * M + m];
        red[threadIdx.x] = acc;
        __syncthreads();
        if (m < M && g == 0) {
            T s = T(0);
            for (int k = 0; k < split; ++k) s += red[threadIdx.x + k];
            int r = m;
            int64_t idx = 0, stride = 1;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const int K = r % P1;
                r /= P1;
                idx += (int64_t)(ne.e[d] * P1 + K) * stride;
                stride *= a.N;
            }
            du[idx] += factor * s / wn[m];
        }
        __syncthreads();
    }
}

// Every point of the plan: the tensor rules' (one CTA per element), then the
// near points (a warp per line), as (D, npoints).
template <typename T, int D>
__global__ void rule_points_kernel(const TransferLaunch a, T* xs, int64_t npoints) {
    const RuleElement el = a.rule_elems[blockIdx.x];
    const int q = a.rule_q[el.rule];
    const T* nodes = static_cast<const T*>(a.tables) + a.rule_nodes[el.rule];
    T lo[D], hi[D];
    element_box<T, D>(a, el.block, el.e, lo, hi);
    int npts = 1;
    for (int d = 0; d < D; ++d) npts *= q;
    for (int j = threadIdx.x; j < npts; j += blockDim.x) {
        int r = j;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int jd = r % q;
            r /= q;
            xs[(int64_t)d * npoints + el.base + j] = lo[d] + (hi[d] - lo[d]) * (T(1) + nodes[jd]) / T(2);
        }
    }
}

template <typename T, int D>
__global__ void near_points_kernel(const TransferLaunch a, T* xs, int64_t npoints) {
    const int64_t l = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (l >= a.n_lines) return;
    const NearLine L = a.lines[l];
    const T* lv = static_cast<const T*>(a.line_vals);
    const T* lx = static_cast<const T*>(a.near_lx);
    for (int p = L.p0 + threadIdx.x % 32; p < L.p1; p += 32) {
        const int64_t at = a.near_base + p;
#pragma unroll
        for (int d = 0; d < D - 1; ++d) xs[(int64_t)d * npoints + at] = lv[3 * l + d];
        xs[(int64_t)(D - 1) * npoints + at] = lx[p];
    }
}

template <typename T, int D>
size_t rule_smem(const TransferLaunch& a) {
    const size_t cq = (size_t)(a.max_q > a.P + 1 ? a.max_q : a.P + 1);
    size_t cap = 1;
    for (int d = 0; d < D; ++d) cap *= cq;
    return (2 * cap + (size_t)a.max_q * (D + a.P + 1)) * sizeof(T);
}

// One launch per rule of [r0, r1), its shared memory sized for that rule's
// q: the far rule's q = P + 3 needs a fraction of the largest graded band's.
template <typename T, int D, int SRC>
cudaError_t run_rules(const TransferLaunch& a, int r0, int r1, cudaStream_t stream) {
    cudaError_t e = cudaFuncSetAttribute(tensor_rule_kernel<T, D, SRC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)rule_smem<T, D>(a));
    if (e != cudaSuccess) return e;
    for (int r = r0; r < r1; ++r) {
        const int64_t n = a.rule_start[r + 1] - a.rule_start[r];
        if (n <= 0) continue;
        TransferLaunch b = a;
        b.rule_elems = a.rule_elems + a.rule_start[r];
        b.max_q = a.rule_q[r];
        tensor_rule_kernel<T, D, SRC><<<(unsigned)n, kRuleThreads, rule_smem<T, D>(b), stream>>>(b);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename T, int D, int P1, int SRC>
cudaError_t run_lines(const TransferLaunch& a, cudaStream_t stream) {
    constexpr int M = D == 1 ? P1 : (D == 2 ? P1 * P1 : P1 * P1 * P1);
    const size_t smem = (size_t)(kLineThreads / kGroup) * M * sizeof(T);
    cudaError_t e = cudaFuncSetAttribute(near_lines_kernel<T, D, P1, SRC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    near_lines_kernel<T, D, P1, SRC><<<(unsigned)a.n_chunks, kLineThreads, smem, stream>>>(a);
    return cudaGetLastError();
}

template <typename T, int D, int SRC>
cudaError_t run_lines_p(const TransferLaunch& a, cudaStream_t stream) {
    switch (a.P + 1) {
        case 2: return run_lines<T, D, 2, SRC>(a, stream);
        case 3: return run_lines<T, D, 3, SRC>(a, stream);
        case 4: return run_lines<T, D, 4, SRC>(a, stream);
        case 5: return run_lines<T, D, 5, SRC>(a, stream);
        case 6: return run_lines<T, D, 6, SRC>(a, stream);
        case 7: return run_lines<T, D, 7, SRC>(a, stream);
    }
    return cudaErrorInvalidValue;
}

// The nested rule first, on its own stream: its chain (lines, then finish)
// is the longest and its CTAs the fewest; then the graded bands and the far
// rule. The three write disjoint elements' nodes.
template <typename T, int D>
cudaError_t projection(const TransferLaunch& a, cudaStream_t far, cudaStream_t bands, cudaStream_t near) {
    cudaError_t e;
    if (a.n_chunks > 0) {
        e = a.source == SOURCE_VALUES ? run_lines_p<T, D, SOURCE_VALUES>(a, near)
                                      : run_lines_p<T, D, SOURCE_DENSITY>(a, near);
        if (e != cudaSuccess) return e;
        near_finish_kernel<T, D><<<(unsigned)a.n_near_elems, kFinishThreads, kFinishThreads * sizeof(T), near>>>(a);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (a.n_rule_elems > 0) {
        e = a.source == SOURCE_VALUES ? run_rules<T, D, SOURCE_VALUES>(a, 1, a.nrules, bands)
                                      : run_rules<T, D, SOURCE_DENSITY>(a, 1, a.nrules, bands);
        if (e != cudaSuccess) return e;
        e = a.source == SOURCE_VALUES ? run_rules<T, D, SOURCE_VALUES>(a, 0, 1, far)
                                      : run_rules<T, D, SOURCE_DENSITY>(a, 0, 1, far);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename T, int D>
cudaError_t points(const TransferLaunch& a, void* xs, int64_t npoints, cudaStream_t stream) {
    if (a.n_rule_elems > 0) {
        rule_points_kernel<T, D><<<(unsigned)a.n_rule_elems, kRuleThreads, 0, stream>>>(a, static_cast<T*>(xs), npoints);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (a.n_lines > 0) {
        near_points_kernel<T, D><<<(unsigned)((a.n_lines + 7) / 8), 256, 0, stream>>>(a, static_cast<T*>(xs), npoints);
        return cudaGetLastError();
    }
    return cudaSuccess;
}

// One pass of the averaging along dimension d: item (J, k, i) takes, in
// the i-th ball block, the nodes k(P+1) - 1 and k(P+1) along d for k < E (the
// faces between its elements), or for k = E its node N - 1 and node 0 of the
// block across its upper face; J runs over the other dimensions. Both nodes
// get their mean, the lower one's value first. No two items write one node.
template <typename T, int D>
__global__ void average_kernel(const AverageLaunch a, int d) {
    int64_t per = 1;
    for (int m = 0; m < D - 1; ++m) per *= a.N;
    const int64_t total = per * a.E * a.nball;
    const int P1 = a.P + 1;
    for (int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; item < total;
         item += (int64_t)gridDim.x * blockDim.x) {
        const int64_t J = item % per;
        const int k = (int)((item / per) % a.E) + 1;
        const int64_t i = item / (per * a.E);
        // the other dimensions' indices, in order, with d's left out
        int64_t off = 0, stride = 1, rest = J, strd = 1;
        for (int m = 0; m < D; ++m) {
            if (m == d) {
                strd = stride;
            } else {
                off += (rest % a.N) * stride;
                rest /= a.N;
            }
            stride *= a.N;
        }
        T* u = static_cast<T*>(a.u);
        const int64_t b = a.blocks[i];
        const int64_t vb = (int64_t)(a.var - 1) * a.NN;
        if (k < a.E) {
            T* p1 = u + b * 2 * a.NN + vb + off + (int64_t)(k * P1 - 1) * strd;
            T* p2 = u + b * 2 * a.NN + vb + off + (int64_t)(k * P1) * strd;
            const T mean = (*p1 + *p2) / T(2);
            *p1 = mean;
            *p2 = mean;
        } else {
            const int64_t bn = a.upper[i * 3 + d];
            if (bn >= 0) {
                T* p1 = u + b * 2 * a.NN + vb + off + (int64_t)(a.N - 1) * strd;
                T* p2 = u + bn * 2 * a.NN + vb + off;
                const T mean = (*p1 + *p2) / T(2);
                *p1 = mean;
                *p2 = mean;
            }
        }
    }
}

template <typename T, int D>
cudaError_t average(const AverageLaunch& a, cudaStream_t s) {
    int64_t per = 1;
    for (int m = 0; m < D - 1; ++m) per *= a.N;
    const int64_t total = per * a.E * a.nball;
    if (total == 0) return cudaSuccess;
    const unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, 152 * 16);
    for (int d = 0; d < D; ++d) {
        average_kernel<T, D><<<grid, 256, 0, s>>>(a, d);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename T>
cudaError_t projection_d(const TransferLaunch& a, cudaStream_t far, cudaStream_t bands, cudaStream_t near) {
    switch (a.D) {
        case 1: return projection<T, 1>(a, far, bands, near);
        case 2: return projection<T, 2>(a, far, bands, near);
        case 3: return projection<T, 3>(a, far, bands, near);
    }
    return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t points_d(const TransferLaunch& a, void* xs, int64_t n, cudaStream_t s) {
    switch (a.D) {
        case 1: return points<T, 1>(a, xs, n, s);
        case 2: return points<T, 2>(a, xs, n, s);
        case 3: return points<T, 3>(a, xs, n, s);
    }
    return cudaErrorInvalidValue;
}

// Component c of one particle's kernel at x: d rho / dx_c for c < 3, rho for
// c = 3 (density_kernel, src/dynamic.jl:124-135): y = L(v)(x - z), q = y.y,
// rho = Q rho0(q) and grad rho = L(v)(2 Q rho0'(q) y), L being symmetric, with
// rho0(q) = l^-3 (3465/512) (1 - q/l^2)^4 / pi inside the support.
__device__ __forceinline__ double kernel_component(const TransferParticle& p, double x0, double x1, double x2, int c) {
    const double r0 = x0 - p.z[0], r1 = x1 - p.z[1], r2 = x2 - p.z[2];
    const double f = p.g * (p.v[0] * r0 + p.v[1] * r1 + p.v[2] * r2);
    const double y0 = r0 + f * p.v[0], y1 = r1 + f * p.v[1], y2 = r2 + f * p.v[2];
    const double q = y0 * y0 + y1 * y1 + y2 * y2;
    const double l2 = p.ell * p.ell;
    if (!(q < l2)) return 0.0;
    const double u = 1.0 - q / l2;
    const double c0 = p.charge * (3465.0 / 512.0) / (l2 * p.ell) / 3.141592653589793238462643383279502884;
    const double u3 = (u * u) * u;
    if (c == 3) return c0 * (u3 * u);
    const double s = -8.0 * c0 * u3 / l2;            // 2 rho0'(q)
    const double w0 = s * y0, w1 = s * y1, w2 = s * y2;
    const double h = p.g * (p.v[0] * w0 + p.v[1] * w1 + p.v[2] * w2);
    // select, not an index: the values stay in registers
    const double wc = c == 0 ? w0 : (c == 1 ? w1 : w2);
    const double vc = c == 0 ? p.v[0] : (c == 1 ? p.v[1] : p.v[2]);
    return wc + h * vc;
}

// The kernel's moments over one chunk of a support element's compact lines,
// component blockIdx.y: per line r_i = sum_p w_p K_c(x_p) phi_i(x_p,last),
// then node (K_0, K_1, K_2) gets w_line phi_K0(x_0) phi_K1(x_1) r_K2, as the
// nested rule's projection kernel regroups them; the groups' sums in group
// order go to partials[chunk][c].
template <int P1>
__global__ void __launch_bounds__(kLineThreads) pairing_lines_kernel(const PairingLaunch a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int M = P1 * P1 * P1;
    constexpr int MO = P1 * P1;
    constexpr int NPL = (M + kGroup - 1) / kGroup;
    constexpr int NOUT = 2 * P1;
    const int tid = threadIdx.x;
    const int group = tid / kGroup, lane = tid % kGroup, ngroups = blockDim.x / kGroup;
    const unsigned mask = 0xffu << ((tid % 32) / kGroup * kGroup);
    const int comp = blockIdx.y;
    const NearChunk ch = a.chunks[blockIdx.x];
    const PairElement el = a.elems[ch.elem];
    const TransferParticle pt = a.particles[el.particle];
    const double sum0 = el.lo[0] + el.hi[0], sum1 = el.lo[1] + el.hi[1], sum2 = el.lo[2] + el.hi[2];
    const double inv0 = 1.0 / (el.hi[0] - el.lo[0]), inv1 = 1.0 / (el.hi[1] - el.lo[1]);
    const double inv2 = 1.0 / (el.hi[2] - el.lo[2]);
    double nodes[P1], bary[P1];
#pragma unroll
    for (int i = 0; i < P1; ++i) {
        nodes[i] = a.gll[i];
        bary[i] = a.bary[i];
    }
    double acc[NPL];
#pragma unroll
    for (int k = 0; k < NPL; ++k) acc[k] = 0.0;
    for (int l = ch.l0 + group; l < ch.l1; l += ngroups) {
        const NearLine L = a.lines[l];
        const double pre0 = a.line_vals[3 * (int64_t)l], pre1 = a.line_vals[3 * (int64_t)l + 1];
        const double wl = a.line_vals[3 * (int64_t)l + 2];
        double r[P1];
#pragma unroll
        for (int i = 0; i < P1; ++i) r[i] = 0.0;
        for (int p = L.p0 + lane; p < L.p1; p += kGroup) {
            const double x = a.lx[p];
            double phi[P1];
            lagrange_all<double, P1>(nodes, bary, (2.0 * x - sum2) * inv2, phi);
            const double c = a.lw[p] * kernel_component(pt, pre0, pre1, x, comp);
#pragma unroll
            for (int i = 0; i < P1; ++i) r[i] += c * phi[i];
        }
#pragma unroll
        for (int off = kGroup / 2; off > 0; off /= 2)
#pragma unroll
            for (int i = 0; i < P1; ++i) r[i] += shfl8_xor(mask, r[i], off);
        // the two outer dimensions' Lagrange values, value j = d (P+1) + i on
        // lane j % kGroup
        double ov[(NOUT + kGroup - 1) / kGroup + 1];
#pragma unroll
        for (int s = 0; s * kGroup < NOUT; ++s) {
            const int j = s * kGroup + lane;
            double v = 0.0;
            if (j < NOUT) {
                const int d = j / P1, i = j % P1;
                const double xi = d == 0 ? (2.0 * pre0 - sum0) * inv0 : (2.0 * pre1 - sum1) * inv1;
                v = lagrange_one<double, P1>(nodes, bary, xi, i);
            }
            ov[s] = v;
        }
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
            const int m = lane + kGroup * k;
            const int mm = m < M ? m : 0;
            const int Klast = mm / MO;
            int o = mm % MO;
            double outer = wl;
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                const int j = d * P1 + o % P1;
                o /= P1;
                double got = 0.0;
#pragma unroll
                for (int s = 0; s * kGroup < NOUT; ++s) {
                    const double t = shfl8(mask, ov[s], j % kGroup);
                    if (j / kGroup == s) got = t;
                }
                outer *= got;
            }
            double rk = 0.0;
#pragma unroll
            for (int i = 0; i < P1; ++i)
                if (i == Klast) rk = r[i];
            if (m < M) acc[k] += outer * rk;
        }
    }
    double* red = reinterpret_cast<double*>(smem_raw);   // ngroups x M
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
        const int m = lane + kGroup * k;
        if (m < M) red[group * M + m] = acc[k];
    }
    __syncthreads();
    double* out = a.partials + ((int64_t)blockIdx.x * kPairComponents + comp) * M;
    for (int m = tid; m < M; m += blockDim.x) {
        double s = 0.0;
        for (int g = 0; g < ngroups; ++g) s += red[g * M + m];
        out[m] = s;
    }
}

// Each support element's moments: its chunks' sums added in order.
template <int P1>
__global__ void pairing_moments_kernel(const PairingLaunch a) {
    constexpr int CM = kPairComponents * P1 * P1 * P1;
    const PairElement el = a.elems[blockIdx.x];
    for (int j = threadIdx.x; j < CM; j += blockDim.x) {
        double s = 0.0;
        for (int c = el.c0; c < el.c1; ++c) s += a.partials[(int64_t)c * CM + j];
        a.moments[(int64_t)blockIdx.x * CM + j] = s;
    }
}

constexpr int kDotThreads = 256;

// One CTA per particle: over its support elements' nodes, the node's value
// (the mean over the values the gather lists, the element's own first) times
// the node's moments, summed per thread and then over the threads in a fixed
// tree, so that a pairing is the same to the bit on every call.
template <typename T, int P1>
__global__ void __launch_bounds__(kDotThreads) pairing_dot_kernel(const PairingLaunch a) {
    constexpr int M = P1 * P1 * P1;
    __shared__ double red[kPairComponents][kDotThreads];
    const int k = blockIdx.x, tid = threadIdx.x;
    const int64_t e0 = a.first[k], e1 = a.first[k + 1];
    const T* u = static_cast<const T*>(a.u);
    const int64_t vb = (int64_t)(a.var - 1) * a.NN;
    double acc[kPairComponents] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t j = tid; j < (e1 - e0) * M; j += kDotThreads) {
        const int64_t e = e0 + j / M;
        const int m = (int)(j % M);
        const int64_t* gi = a.gather + (e * M + m) * kGather;
        double g = 0.0;
        int n = 0;
        for (int i = 0; i < kGather; ++i) {
            const int64_t o = gi[i];
            if (o < 0) break;
            g += (double)u[o + vb];
            ++n;
        }
        g /= (double)(n > 0 ? n : 1);
        const double* mu = a.moments + e * kPairComponents * M + m;
#pragma unroll
        for (int c = 0; c < kPairComponents; ++c) acc[c] += g * mu[c * M];
    }
#pragma unroll
    for (int c = 0; c < kPairComponents; ++c) red[c][tid] = acc[c];
    __syncthreads();
    for (int s = kDotThreads / 2; s > 0; s /= 2) {
        if (tid < s)
#pragma unroll
            for (int c = 0; c < kPairComponents; ++c) red[c][tid] += red[c][tid + s];
        __syncthreads();
    }
    if (tid < kPairComponents) a.out[k * kPairComponents + tid] = red[tid][0];
}

template <int P1>
cudaError_t pairing_moments(const PairingLaunch& a, cudaStream_t s) {
    constexpr int M = P1 * P1 * P1;
    cudaError_t e;
    if (a.n_chunks > 0) {
        const size_t smem = (size_t)(kLineThreads / kGroup) * M * sizeof(double);
        e = cudaFuncSetAttribute(pairing_lines_kernel<P1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        pairing_lines_kernel<P1><<<dim3((unsigned)a.n_chunks, kPairComponents), kLineThreads, smem, s>>>(a);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (a.n_elems > 0) {
        pairing_moments_kernel<P1><<<(unsigned)a.n_elems, 256, 0, s>>>(a);
        return cudaGetLastError();
    }
    return cudaSuccess;
}

template <typename T, int P1>
cudaError_t pairing_dot(const PairingLaunch& a, cudaStream_t s) {
    if (a.nparticles <= 0) return cudaSuccess;
    pairing_dot_kernel<T, P1><<<(unsigned)a.nparticles, kDotThreads, 0, s>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t pairing_dot_p(const PairingLaunch& a, cudaStream_t s) {
    switch (a.P + 1) {
        case 2: return pairing_dot<T, 2>(a, s);
        case 3: return pairing_dot<T, 3>(a, s);
        case 4: return pairing_dot<T, 4>(a, s);
        case 5: return pairing_dot<T, 5>(a, s);
        case 6: return pairing_dot<T, 6>(a, s);
        case 7: return pairing_dot<T, 7>(a, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_pairing_moments(const PairingLaunch& a, cudaStream_t stream) {
    switch (a.P + 1) {
        case 2: return pairing_moments<2>(a, stream);
        case 3: return pairing_moments<3>(a, stream);
        case 4: return pairing_moments<4>(a, stream);
        case 5: return pairing_moments<5>(a, stream);
        case 6: return pairing_moments<6>(a, stream);
        case 7: return pairing_moments<7>(a, stream);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_pairing_dot(const PairingLaunch& a, cudaStream_t stream) {
    return a.prec == 0 ? pairing_dot_p<double>(a, stream) : pairing_dot_p<float>(a, stream);
}

cudaError_t launch_projection(const TransferLaunch& a, cudaStream_t far, cudaStream_t bands, cudaStream_t near) {
    return a.prec == 0 ? projection_d<double>(a, far, bands, near) : projection_d<float>(a, far, bands, near);
}

cudaError_t launch_points(const TransferLaunch& a, void* xs, int64_t npoints, cudaStream_t stream) {
    return a.prec == 0 ? points_d<double>(a, xs, npoints, stream) : points_d<float>(a, xs, npoints, stream);
}

cudaError_t launch_average(const AverageLaunch& a, cudaStream_t stream) {
    if (a.prec == 0) {
        switch (a.D) {
            case 1: return average<double, 1>(a, stream);
            case 2: return average<double, 2>(a, stream);
            case 3: return average<double, 3>(a, stream);
        }
    } else {
        switch (a.D) {
            case 1: return average<float, 1>(a, stream);
            case 2: return average<float, 2>(a, stream);
            case 3: return average<float, 3>(a, stream);
        }
    }
    return cudaErrorInvalidValue;
}

}  // namespace twoldg
