// The particle-grid transfer's device passes (src/transfer.jl:520-680,
// 1215-1378): the tensor rules (far and graded) fused into one kernel that
// evaluates the source at an element's q^D Gauss points into shared memory
// and contracts them there, and the nested rule's two kernels over the
// host's point list (per-chunk partial sums per node, then each element's
// chunks added in order).
#include "transfer.h"

namespace twoldg {

namespace {

constexpr int kRuleThreads = 128;
constexpr int kNearThreads = 256;

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

// S at x: the caller's value of point `idx`, or the particles' density
// sum_k Q_k rho0(|L(v_k)(x - z_k)|^2, ell_k), rho0(q, l) = l^-3 (3465/512)
// (1 - q/l^2)^4 / pi inside the support (src/particle.jl:117-127;
// src/particle_forms.jl:29-37).
template <typename T, int D>
__device__ __forceinline__ T source_at(const TransferLaunch& a, const T (&x)[D], int64_t idx) {
    if (a.source == SOURCE_VALUES) return static_cast<const T*>(a.values)[idx];
    T s = T(0);
    if constexpr (D == 3) {
        for (int k = 0; k < a.nparticles; ++k) {
            const TransferParticle& p = a.particles[k];
            T r[3], vr = T(0);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                r[d] = x[d] - T(p.z[d]);
                vr += T(p.v[d]) * r[d];
            }
            const T f = T(p.g) * vr;
            T q = T(0);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const T y = r[d] + f * T(p.v[d]);
                q += y * y;
            }
            const T l = T(p.ell);
            if (q < l * l) {
                const T u = T(1) - q / (l * l);
                const T poly = (((T(3465) / T(512)) * u) * u * u) * u;
                s += T(p.charge) * (poly / (l * l * l) / T(3.141592653589793238462643383279502884));
            }
        }
    }
    return s;
}

// One CTA per far or graded element: S at the rule's q^D points, then the
// contraction with contract[i][k] = w_k phi_i(x_k) / w^_i one dimension at a
// time (the sum over k in order, src/transfer.jl:592-621), and factor times
// the element's P S added to variable `var` of du.
template <typename T, int D>
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
    T* nodes = buf1 + cap;
    T* con = nodes + a.max_q;
    const T* tables = static_cast<const T*>(a.tables);
    for (int k = tid; k < q; k += blockDim.x) nodes[k] = tables[a.rule_nodes[el.rule] + k];
    for (int k = tid; k < P1 * q; k += blockDim.x) con[k] = tables[a.rule_contract[el.rule] + k];
    __syncthreads();
    T lo[D], hi[D];
    element_box<T, D>(a, el.block, el.e, lo, hi);
    int npts = 1;
    for (int d = 0; d < D; ++d) npts *= q;
    for (int j = tid; j < npts; j += blockDim.x) {
        T x[D];
        int r = j;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int jd = r % q;
            r /= q;
            x[d] = lo[d] + (hi[d] - lo[d]) * (T(1) + nodes[jd]) / T(2);
        }
        buf0[j] = source_at<T, D>(a, x, el.base + j);
    }
    __syncthreads();
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

// The nested rule, pass 1: chunk c's points summed for every node m of their
// element, sum_p w_p (S(x_p) phi_m(x_p)), with phi_m the product of the
// dimensions' Lagrange polynomials in their product form (src/transfer.jl:
// 171-182, 1330-1352).
template <typename T, int D>
__global__ void __launch_bounds__(kNearThreads) near_partials_kernel(const TransferLaunch a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    const int P1 = a.P + 1;
    const NearChunk ch = a.chunks[blockIdx.x];
    const NearElement ne = a.near_elems[ch.elem];
    const int n = ch.p1 - ch.p0;
    T* sv = reinterpret_cast<T*>(smem_raw);   // S at the points
    T* sw = sv + kNearChunk;                  // their weights
    T* lag = sw + kNearChunk;                 // [p][d][i]
    T lo[D], hi[D];
    element_box<T, D>(a, ne.block, ne.e, lo, hi);
    const T* xs = static_cast<const T*>(a.near_xs);
    const T* bary = static_cast<const T*>(a.bary);
    const T* gll = static_cast<const T*>(a.gll);
    for (int p = tid; p < n; p += blockDim.x) {
        const int64_t g = ch.p0 + p;
        T x[D];
#pragma unroll
        for (int d = 0; d < D; ++d) x[d] = xs[g * D + d];
        sv[p] = source_at<T, D>(a, x, a.near_base + g);
        sw[p] = static_cast<const T*>(a.near_ws)[g];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const T xi = (T(2) * x[d] - lo[d] - hi[d]) / (hi[d] - lo[d]);
            for (int i = 0; i < P1; ++i) {
                T acc = bary[i];
                for (int j = 0; j < P1; ++j)
                    if (j != i) acc *= xi - gll[j];
                lag[(p * D + d) * P1 + i] = acc;
            }
        }
    }
    __syncthreads();
    int M = 1;
    for (int d = 0; d < D; ++d) M *= P1;
    T* partials = static_cast<T*>(a.partials) + (int64_t)blockIdx.x * M;
    for (int m = tid; m < M; m += blockDim.x) {
        int K[D];
        int r = m;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            K[d] = r % P1;
            r /= P1;
        }
        T acc = T(0);
        for (int p = 0; p < n; ++p) {
            T phi = T(1);
#pragma unroll
            for (int d = 0; d < D; ++d) phi = lag[(p * D + d) * P1 + K[d]] * phi;
            acc += sw[p] * (sv[p] * phi);
        }
        partials[m] = acc;
    }
}

// The nested rule, pass 2: element i's chunks added in order for node m, and
// factor times that over w_m added to its node (src/transfer.jl:1354-1369).
template <typename T, int D>
__global__ void near_finish_kernel(const TransferLaunch a) {
    const NearElement ne = a.near_elems[blockIdx.x];
    const int P1 = a.P + 1;
    int M = 1;
    for (int d = 0; d < D; ++d) M *= P1;
    const T* partials = static_cast<const T*>(a.partials);
    const T* wn = static_cast<const T*>(a.wn);
    T* du = static_cast<T*>(a.du) + (int64_t)ne.block * 2 * a.NN + (int64_t)(a.var - 1) * a.NN;
    const T factor = T(a.factor);
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
        T acc = T(0);
        for (int c = ne.c0; c < ne.c1; ++c) acc += partials[(int64_t)c * M + m];
        int r = m;
        int64_t idx = 0, stride = 1;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int K = r % P1;
            r /= P1;
            idx += (int64_t)(ne.e[d] * P1 + K) * stride;
            stride *= a.N;
        }
        du[idx] += factor * acc / wn[m];
    }
}

// Every point of the plan: the tensor rules' (one CTA per element), then the
// near points, as (D, npoints).
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
__global__ void near_points_kernel(const TransferLaunch a, T* xs, int64_t npoints, int64_t nnear) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nnear) return;
    const T* src = static_cast<const T*>(a.near_xs);
#pragma unroll
    for (int d = 0; d < D; ++d) xs[(int64_t)d * npoints + a.near_base + p] = src[p * D + d];
}

template <typename T, int D>
size_t rule_smem(const TransferLaunch& a) {
    const size_t cq = (size_t)(a.max_q > a.P + 1 ? a.max_q : a.P + 1);
    size_t cap = 1;
    for (int d = 0; d < D; ++d) cap *= cq;
    return (2 * cap + (size_t)a.max_q * (a.P + 2)) * sizeof(T);
}

template <typename T, int D>
size_t near_smem(const TransferLaunch& a) {
    return ((size_t)2 * kNearChunk + (size_t)kNearChunk * D * (a.P + 1)) * sizeof(T);
}

template <typename T, int D>
cudaError_t projection(const TransferLaunch& a, cudaStream_t stream) {
    if (a.n_rule_elems > 0) {
        const size_t smem = rule_smem<T, D>(a);
        cudaError_t e = cudaFuncSetAttribute(tensor_rule_kernel<T, D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        tensor_rule_kernel<T, D><<<(unsigned)a.n_rule_elems, kRuleThreads, smem, stream>>>(a);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (a.n_chunks > 0) {
        const size_t smem = near_smem<T, D>(a);
        cudaError_t e = cudaFuncSetAttribute(near_partials_kernel<T, D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        near_partials_kernel<T, D><<<(unsigned)a.n_chunks, kNearThreads, smem, stream>>>(a);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        near_finish_kernel<T, D><<<(unsigned)a.n_near_elems, 128, 0, stream>>>(a);
        e = cudaGetLastError();
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
    const int64_t nnear = npoints - a.near_base;
    if (nnear > 0) {
        near_points_kernel<T, D><<<(unsigned)((nnear + 255) / 256), 256, 0, stream>>>(a, static_cast<T*>(xs), npoints,
                                                                                     nnear);
        return cudaGetLastError();
    }
    return cudaSuccess;
}

template <typename T>
cudaError_t projection_d(const TransferLaunch& a, cudaStream_t s) {
    switch (a.D) {
        case 1: return projection<T, 1>(a, s);
        case 2: return projection<T, 2>(a, s);
        case 3: return projection<T, 3>(a, s);
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

}  // namespace

cudaError_t launch_projection(const TransferLaunch& a, cudaStream_t stream) {
    return a.prec == 0 ? projection_d<double>(a, stream) : projection_d<float>(a, stream);
}

cudaError_t launch_points(const TransferLaunch& a, void* xs, int64_t npoints, cudaStream_t stream) {
    return a.prec == 0 ? points_d<double>(a, xs, npoints, stream) : points_d<float>(a, xs, npoints, stream);
}

}  // namespace twoldg
