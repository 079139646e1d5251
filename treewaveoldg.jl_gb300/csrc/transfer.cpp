// The particle-grid transfer's host side (src/transfer.jl:251-455, 918-1022,
// 1151-1285, 1380-1415): the refusals, the classification of the elements
// of the blocks the source's ball meets into the far rule, the graded bands
// and the nested rule, the nested rule's points (split at each particle's
// support, Gauss inside, Johnston and Elliott's sinh rule outside), and the
// C ABI over the kernels of transfer_kernels.cu. Positions, boxes and the
// nested rule's points are formed in double and rounded once to the field
// type when they are uploaded.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "../../include/twoldg.h"
#include "tables.h"
#include "transfer.h"

namespace twoldg {
int static_rhs_fail(int code, const std::string& msg);
bool problem_shape(twoldg_problem* p, int* D, int* P, int* E, int* prec, int64_t* nblocks, cudaStream_t* stream);
}  // namespace twoldg

using namespace twoldg;

namespace {

int fail(int code, const std::string& msg) { return static_rhs_fail(code, msg); }

std::string fmt(double x) {
    char b[64];
    std::snprintf(b, sizeof b, "%.17g", x);
    return b;
}

struct Support {
    int D;
    double z[3], v[3], ell;
};

struct Rule1D {
    std::vector<double> x, w;
};

// The one-dimensional rules the nested rule transforms, in double.
struct NestedTables {
    Rule1D sinh, mid, inner;
};

Rule1D gauss_rule(int n) {
    RuleTables<double> r64;
    RuleTables<float> r32;
    build_rule(1, n, r64, r32);
    return Rule1D{r64.nodes, r64.weights};
}

// The squared distance from x to the box [lo, hi] over dimensions [d0, d1)
// (src/transfer.jl:292-300).
double box_distance2(const double* x, const double* lo, const double* hi, int d0, int d1) {
    double acc = 0;
    for (int d = d0; d < d1; ++d) {
        const double delta = std::max({lo[d] - x[d], x[d] - hi[d], 0.0});
        acc += delta * delta;
    }
    return acc;
}

// support_breaks (src/transfer.jl:302-366): where the line along dimension
// d = F through the fixed coordinates prefix[0..F) needs a breakpoint inside
// (lo[d], hi[d]), and the extent of the support's section along it. The
// support is r^T M r <= ell^2, M = I + gamma^2 v v^T; with some coordinates
// fixed and the free ones minimised over (Sherman-Morrison), each remaining
// dimension free, at its low face or at its high face gives a quadratic's two
// roots; all free (code 0) is the extent.
void support_breaks(const Support& s, const double* prefix, int F, const double* lo, const double* hi,
                    std::vector<double>& breaks, bool& has_extent, double* extent) {
    const int D = s.D, d = F;
    double vv = 0;
    for (int j = 0; j < D; ++j) vv += s.v[j] * s.v[j];
    const double g2 = 1 / (1 - vv);
    double r2F = 0, vrF = 0;
    for (int j = 0; j < F; ++j) {
        r2F += (prefix[j] - s.z[j]) * (prefix[j] - s.z[j]);
        vrF += s.v[j] * (prefix[j] - s.z[j]);
    }
    breaks.clear();
    has_extent = false;
    int ncodes = 1;
    for (int j = d + 1; j < D; ++j) ncodes *= 3;
    for (int code = 0; code < ncodes; ++code) {
        double r2 = r2F, vr = vrF, vfree = 0;
        int c = code;
        for (int j = d + 1; j < D; ++j) {
            const int k = c % 3;
            c /= 3;
            if (k == 0) {
                vfree += s.v[j] * s.v[j];
            } else {
                const double f = (k == 1 ? lo[j] : hi[j]) - s.z[j];
                r2 += f * f;
                vr += s.v[j] * f;
            }
        }
        const double cc = g2 / (1 + g2 * vfree);
        const double A = 1 + cc * s.v[d] * s.v[d];
        const double B = cc * vr * s.v[d];
        const double C = r2 + cc * vr * vr - s.ell * s.ell;
        const double disc = B * B - A * C;
        if (!(disc > 0)) continue;
        const double q = std::sqrt(disc);
        const double x1 = s.z[d] + (-B - q) / A;
        const double x2 = s.z[d] + (-B + q) / A;
        if (code == 0) {
            has_extent = true;
            extent[0] = x1;
            extent[1] = x2;
        }
        if (lo[d] < x1 && x1 < hi[d]) breaks.push_back(x1);
        if (lo[d] < x2 && x2 < hi[d]) breaks.push_back(x2);
    }
    std::sort(breaks.begin(), breaks.end());
}

// The inner Gauss rule on [a, b] (src/transfer.jl:457-471): plain on the
// innermost line, under x = a + (b - a)(1 - cos theta)/2 on the others.
void inner_points(const Rule1D& r, double a, double b, bool plain, std::vector<double>& xs, std::vector<double>& ws) {
    const double half = (b - a) / 2;
    const double pi = 3.14159265358979323846;
    for (size_t k = 0; k < r.x.size(); ++k) {
        const double th = pi * (1 + r.x[k]) / 2;
        xs.push_back(plain ? a + half * (1 + r.x[k]) : a + half * (1 - std::cos(th)));
        ws.push_back(plain ? r.w[k] * half : r.w[k] * pi / 2 * half * std::sin(th));
    }
}

// The sinh rule on [a, b] toward c at distance beta (src/transfer.jl:233-262,
// 473-486): xi = xi_c + eps sinh(mu u - eta), mu and eta mapping u = +-1 to
// xi = +-1.
void sinh_points(const Rule1D& r, double a, double b, double c, double beta, std::vector<double>& xs,
                 std::vector<double>& ws) {
    const double half = (b - a) / 2, mid = (a + b) / 2;
    const double xc = (c - mid) / half, eps = beta / half;
    const double lo = std::asinh((1 + xc) / eps), hi = std::asinh((1 - xc) / eps);
    const double mu = (hi + lo) / 2, eta = (lo - hi) / 2;
    for (size_t k = 0; k < r.x.size(); ++k) {
        xs.push_back(mid + half * (xc + eps * std::sinh(mu * r.x[k] - eta)));
        ws.push_back(r.w[k] * eps * mu * std::cosh(mu * r.x[k] - eta) * half);
    }
}

// One line of the nested rule along dimension d = prefix.size()
// (LINE_FOLD, src/transfer.jl:368-412): its segments between the support's
// breakpoints, each with the inner rule inside the support's extent, or
// (unless compact) the sinh rule toward the particle's centre projected onto
// the segment, on the scale of its distance from the line; `mid` points
// where that distance is at least half the segment, `sinh` points closer.
template <typename Fn>
void line_fold(const Support& s, const NestedTables& t, const double* lo, const double* hi,
               const std::vector<double>& prefix, bool innermost, bool compact, Fn&& seg) {
    const int D = s.D, F = (int)prefix.size(), d = F;
    std::vector<double> breaks;
    bool has_extent;
    double extent[2] = {0, 0};
    support_breaks(s, prefix.data(), F, lo, hi, breaks, has_extent, extent);
    double off2 = box_distance2(s.z, lo, hi, d + 1, D);
    for (int j = 0; j < F; ++j) off2 += (prefix[j] - s.z[j]) * (prefix[j] - s.z[j]);
    double a = lo[d];
    std::vector<double> xs, ws;
    for (size_t k = 0; k <= breaks.size(); ++k) {
        const double b = k < breaks.size() ? breaks[k] : hi[d];
        if (b > a) {
            const double mid = (a + b) / 2;
            xs.clear();
            ws.clear();
            if (has_extent && extent[0] < mid && mid < extent[1]) {
                inner_points(t.inner, a, b, innermost, xs, ws);
                seg(xs, ws);
            } else if (!compact) {
                const double c = std::min(std::max(s.z[d], a), b);
                const double beta = std::max(std::sqrt(off2 + (s.z[d] - c) * (s.z[d] - c)),
                                             std::numeric_limits<double>::epsilon() * (b - a));
                if (beta >= (b - a) / 2)
                    sinh_points(t.mid, a, b, c, beta, xs, ws);
                else
                    sinh_points(t.sinh, a, b, c, beta, xs, ws);
                seg(xs, ws);
            }
        }
        a = b;
    }
}

// Every point of the nested rule's remaining n dimensions through `prefix`,
// each with w times its lines' weights (collect_points!, src/transfer.jl:
// 1302-1328).
void collect_points(const Support& s, const NestedTables& t, const double* lo, const double* hi,
                    std::vector<double>& prefix, double w, int n, std::vector<double>& xs, std::vector<double>& ws) {
    if (n == 0) {
        xs.insert(xs.end(), prefix.begin(), prefix.end());
        ws.push_back(w);
        return;
    }
    line_fold(s, t, lo, hi, prefix, n == 1, false, [&](const std::vector<double>& lx, const std::vector<double>& lw) {
        for (size_t k = 0; k < lx.size(); ++k) {
            prefix.push_back(lx[k]);
            collect_points(s, t, lo, hi, prefix, w * lw[k], n - 1, xs, ws);
            prefix.pop_back();
        }
    });
}

struct HostElem {
    int block, e[3], particle;
};

}  // namespace

struct twoldg_transfer_plan {
    TransferLaunch L;
    cudaStream_t stream = nullptr;
    int64_t counts[8] = {0};
    int64_t npoints = 0;
    bool density_ok = false;
    std::vector<void*> bufs;
    ~twoldg_transfer_plan() {
        if (stream) cudaStreamSynchronize(stream);
        for (void* b : bufs) cudaFree(b);
    }
    template <typename V>
    cudaError_t upload(const std::vector<V>& v, const void** out) {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(v.size() * sizeof(V), 16));
        if (e != cudaSuccess) return e;
        bufs.push_back(p);
        if (!v.empty()) e = cudaMemcpy(p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice);
        *out = p;
        return e;
    }
};

namespace {

template <typename T>
std::vector<T> rounded(const std::vector<double>& v) {
    return std::vector<T>(v.begin(), v.end());
}

template <typename T>
int upload_all(twoldg_transfer_plan* pl, const std::vector<double>& origins, const std::vector<double>& spacings,
               const std::vector<double>& tabs, const std::vector<double>& nxs, const std::vector<double>& nws,
               const std::vector<double>& bary, const std::vector<double>& gll, const std::vector<double>& wn) {
    TransferLaunch& L = pl->L;
    cudaError_t e;
#define UP(vec, field)                                                                     \
    e = pl->upload(rounded<T>(vec), &L.field);                                             \
    if (e != cudaSuccess) return fail(TWOLDG_ECUDA, std::string("transfer upload: ") + cudaGetErrorString(e));
    UP(origins, origins)
    UP(spacings, spacings)
    UP(tabs, tables)
    UP(nxs, near_xs)
    UP(nws, near_ws)
    UP(bary, bary)
    UP(gll, gll)
    UP(wn, wn)
#undef UP
    int M = 1;
    for (int d = 0; d < L.D; ++d) M *= L.P + 1;
    void* part = nullptr;
    e = cudaMalloc(&part, std::max<size_t>((size_t)L.n_chunks * M * sizeof(T), 16));
    if (e != cudaSuccess) return fail(TWOLDG_ENOMEM, std::string("transfer partials: ") + cudaGetErrorString(e));
    pl->bufs.push_back(part);
    L.partials = part;
    return TWOLDG_OK;
}

}  // namespace

extern "C" {

int twoldg_transfer_table(int32_t order, int32_t precision, const char* name, int32_t q, void* out) {
    if (!name || !out) return fail(TWOLDG_EINVAL, "name and out must not be NULL");
    if (order < 1 || order > kMaxP) return fail(TWOLDG_EINVAL, "order P must be 1.." + std::to_string(kMaxP));
    if (precision != 0 && precision != 1) return fail(TWOLDG_EINVAL, "precision is 0 (float64) or 1 (float32)");
    const std::string n(name);
    auto put = [&](const auto& v64, const auto& v32) {
        if (precision == 0)
            std::memcpy(out, v64.data(), v64.size() * sizeof(double));
        else
            std::memcpy(out, v32.data(), v32.size() * sizeof(float));
    };
    if (n == "bary") {
        std::vector<double> b64;
        std::vector<float> b32;
        build_bary(order, b64, b32);
        put(b64, b32);
        return TWOLDG_OK;
    }
    RuleTables<double> r64;
    RuleTables<float> r32;
    if (!build_rule(order, q, r64, r32))
        return fail(TWOLDG_EINVAL, "a rule has 1.." + std::to_string(kMaxRule) + " points, got q = " + std::to_string(q));
    if (n == "gauss_nodes") put(r64.nodes, r32.nodes);
    else if (n == "gauss_weights") put(r64.weights, r32.weights);
    else if (n == "lagrange") put(r64.lagrange, r32.lagrange);
    else if (n == "contract") put(r64.contract, r32.contract);
    else return fail(TWOLDG_EINVAL, "unknown transfer table " + n);
    return TWOLDG_OK;
}

int twoldg_transfer_plan_create(twoldg_problem* p, const twoldg_transfer_desc* d, twoldg_transfer_plan** out) {
    if (!p || !d || !out) return fail(TWOLDG_EINVAL, "problem, descriptor and out must not be NULL");
    *out = nullptr;
    int D, P, E, prec;
    int64_t nb;
    cudaStream_t stream;
    if (!problem_shape(p, &D, &P, &E, &prec, &nb, &stream)) return fail(TWOLDG_EINVAL, "bad problem");
    if (D < 1 || D > 3) return fail(TWOLDG_EUNSUP, "the transfer runs in 1 to 3 dimensions");
    if (!d->origins || !d->spacings) return fail(TWOLDG_EINVAL, "origins and spacings must not be NULL");
    if (d->nparticles < 0 || d->nparticles > kMaxParticles)
        return fail(TWOLDG_EUNSUP, "at most " + std::to_string(kMaxParticles) + " particles, got " +
                                       std::to_string(d->nparticles));
    if (d->nparticles > 0 && !d->particles) return fail(TWOLDG_EINVAL, "particles must not be NULL");
    if (!(d->h_e > 0)) return fail(TWOLDG_EINVAL, "h_e must be positive");
    const int P1 = P + 1, N = E * P1;
    // the quadrature, with the reference's defaults (src/transfer.jl:139-170)
    const int q = d->q > 0 ? d->q : P + 3;
    const int nsinh = d->nsinh > 0 ? d->nsinh : 48, nmid = d->nmid > 0 ? d->nmid : 16;
    const int ninner = d->ninner > 0 ? d->ninner : 24;
    const double rfar = d->rfar > 0 ? d->rfar : 9.0;
    std::vector<double> band_from = {1, 2, 3, 4};
    std::vector<int> band_points = {14, 10, 8, 7};
    if (d->nbands > 0) {
        if (!d->band_from || !d->band_points) return fail(TWOLDG_EINVAL, "band_from and band_points must not be NULL");
        if (d->nbands > 15) return fail(TWOLDG_EUNSUP, "at most 15 graded bands");
        band_from.assign(d->band_from, d->band_from + d->nbands);
        band_points.assign(d->band_points, d->band_points + d->nbands);
    }
    for (size_t i = 0; i < band_from.size(); ++i) {
        if ((i > 0 && !(band_from[i - 1] < band_from[i])) || !(0 <= band_from[i] && band_from[i] < rfar))
            return fail(TWOLDG_EINVAL, "the graded rule's distances must increase from 0 and stay below rfar = " +
                                           fmt(rfar));
    }
    if (!(0 <= d->rnear && d->rnear <= rfar))
        return fail(TWOLDG_EINVAL, "rnear = " + fmt(d->rnear) + " must lie between 0 and the far rule's distance rfar = " +
                                       fmt(rfar));
    std::vector<int> rule_q = {q};
    for (int b : band_points) rule_q.push_back(b);
    int max_q = 0;
    for (int r : rule_q) {
        if (r < 1) return fail(TWOLDG_EINVAL, "a rule needs at least one point");
        max_q = std::max(max_q, r);
    }
    int64_t cap = 1;
    for (int k = 0; k < D; ++k) cap *= std::max(max_q, P + 1);
    if (cap > 4096) return fail(TWOLDG_EUNSUP, "a tensor rule of " + std::to_string(max_q) + "^" + std::to_string(D) +
                                                  " points exceeds the device's 4096 per element");
    if (nsinh > kMaxRule || nmid > kMaxRule || ninner > kMaxRule)
        return fail(TWOLDG_EINVAL, "the nested rule's lines take at most " + std::to_string(kMaxRule) + " points");

    const double he = d->h_e, rn = d->rnear * he, rf = rfar * he;
    std::vector<Support> parts(d->nparticles);
    for (int k = 0; k < d->nparticles; ++k) {
        const twoldg_particle& tp = d->particles[k];
        Support& s = parts[k];
        s.D = D;
        double vv = 0;
        for (int j = 0; j < 3; ++j) {
            s.z[j] = j < D ? tp.z[j] : 0;
            s.v[j] = j < D ? tp.v[j] : 0;
            vv += s.v[j] * s.v[j];
        }
        s.ell = tp.ell;
        if (!(tp.ell > 0)) return fail(TWOLDG_EINVAL, "particle " + std::to_string(k) + ": ell must be positive");
        if (!(vv < 1)) return fail(TWOLDG_EINVAL, "particle " + std::to_string(k) + ": |v| must be below 1");
    }
    const double* c = d->ball_centre;
    const double R = d->ball_radius;
    auto block_box = [&](int64_t b, double* lo, double* hi) {
        for (int k = 0; k < D; ++k) {
            lo[k] = d->origins[b * D + k];
            hi[k] = lo[k] + d->spacings[b] * N;
        }
    };
    auto in_frame = [&](int64_t b) { return !d->mask || d->mask[b]; };
    // the finest-level checks (check_finest, src/transfer.jl:823-870)
    if (d->levels) {
        int top = 0;
        for (int64_t b = 0; b < nb; ++b) top = std::max(top, (int)d->levels[b]);
        for (int64_t b = 0; b < nb; ++b) {
            if (d->levels[b] == top || !in_frame(b)) continue;
            double lo[3], hi[3];
            block_box(b, lo, hi);
            const double r2 = box_distance2(c, lo, hi, 0, D);
            if (r2 < R * R)
                return fail(TWOLDG_EINVAL,
                            "project_source! needs the finest level, " + std::to_string(top) +
                                ", under the source's ball of radius " + fmt(R) + ", and a block of level " +
                                std::to_string(d->levels[b]) + " reaches to " + fmt(std::sqrt(r2)) +
                                " from the ball's centre: the transfer measures its distances in the finest element "
                                "width h_e, and would integrate a coarser element with a rule chosen for a finer one");
        }
        for (const Support& s : parts) {
            for (int corner = 0; corner < (1 << D); ++corner) {
                double x[3];
                for (int k = 0; k < D; ++k) x[k] = s.z[k] + ((corner >> k) & 1 ? s.ell : -s.ell);
                for (int64_t b = 0; b < nb; ++b) {
                    if (!in_frame(b)) continue;
                    double lo[3], hi[3];
                    block_box(b, lo, hi);
                    bool inside = true;
                    for (int k = 0; k < D; ++k) inside = inside && lo[k] <= x[k] && x[k] < hi[k];
                    if (!inside) continue;
                    if (d->levels[b] != top)
                        return fail(TWOLDG_EINVAL, "project_source! needs the finest level, " + std::to_string(top) +
                                                       ", under every particle's support, and the support of radius " +
                                                       fmt(s.ell) + " reaches a block of level " +
                                                       std::to_string(d->levels[b]));
                    break;
                }
            }
        }
    }
    // the elements by rule (host_elements, element_class, src/transfer.jl:
    // 493-503, 1380-1415)
    std::vector<std::vector<HostElem>> lists(rule_q.size());
    std::vector<HostElem> near;
    int Ed[3] = {1, 1, 1};
    for (int k = 0; k < D; ++k) Ed[k] = E;
    for (int64_t b = 0; b < nb; ++b) {
        if (!in_frame(b)) continue;
        double blo[3], bhi[3];
        block_box(b, blo, bhi);
        if (!(box_distance2(c, blo, bhi, 0, D) < R * R)) continue;
        for (int e2 = 0; e2 < Ed[2]; ++e2)
            for (int e1 = 0; e1 < Ed[1]; ++e1)
                for (int e0 = 0; e0 < Ed[0]; ++e0) {
                    const int e[3] = {e0, e1, e2};
                    double lo[3], hi[3];
                    for (int k = 0; k < D; ++k) {
                        lo[k] = d->origins[b * D + k] + d->spacings[b] * (e[k] * P1);
                        hi[k] = d->origins[b * D + k] + d->spacings[b] * ((e[k] + 1) * P1);
                    }
                    if (box_distance2(c, lo, hi, 0, D) >= R * R) continue;
                    std::vector<double> dist2(parts.size());
                    bool host = false;
                    for (size_t k = 0; k < parts.size(); ++k) {
                        dist2[k] = box_distance2(parts[k].z, lo, hi, 0, D);
                        host = host || dist2[k] < rf * rf;
                    }
                    HostElem he_{(int)b, {e0, e1, e2}, 0};
                    if (!host) {
                        lists[0].push_back(he_);
                        continue;
                    }
                    size_t amin = 0;
                    for (size_t k = 1; k < parts.size(); ++k)
                        if (dist2[k] < dist2[amin]) amin = k;
                    if (dist2[amin] >= rn * rn) {
                        const double delta = std::sqrt(dist2[amin]) / he;
                        int band = 0;
                        for (size_t i = 0; i < band_from.size(); ++i)
                            if (band_from[i] <= delta) band = (int)i;
                        lists[1 + band].push_back(he_);
                        continue;
                    }
                    int inside = 0;
                    for (size_t k = 0; k < parts.size(); ++k) inside += dist2[k] < parts[k].ell * parts[k].ell;
                    if (inside > 1) {
                        std::string at;
                        for (int k = 0; k < D; ++k) at += (k ? ", " : "") + fmt(lo[k]);
                        return fail(TWOLDG_EINVAL, "the supports of two particles meet the element at (" + at +
                                                       "), and the near rule splits at one: the particles are closer "
                                                       "than an element");
                    }
                    he_.particle = (int)amin;
                    near.push_back(he_);
                }
    }
    // the nested rule's points, element by element (nested_points,
    // src/transfer.jl:1257-1285)
    NestedTables nt{gauss_rule(nsinh), gauss_rule(nmid), gauss_rule(ninner)};
    std::vector<double> nxs, nws;
    std::vector<int64_t> first = {0};
    for (const HostElem& h : near) {
        double lo[3], hi[3];
        for (int k = 0; k < D; ++k) {
            lo[k] = d->origins[(int64_t)h.block * D + k] + d->spacings[h.block] * (h.e[k] * P1);
            hi[k] = d->origins[(int64_t)h.block * D + k] + d->spacings[h.block] * ((h.e[k] + 1) * P1);
        }
        std::vector<double> prefix;
        collect_points(parts[h.particle], nt, lo, hi, prefix, 1.0, D, nxs, nws);
        first.push_back((int64_t)nws.size());
        if (nws.size() > (size_t)std::numeric_limits<int32_t>::max())
            return fail(TWOLDG_EUNSUP, "the nested rule's points exceed 2^31");
    }

    std::unique_ptr<twoldg_transfer_plan> pl(new twoldg_transfer_plan());
    pl->stream = stream;
    TransferLaunch& L = pl->L;
    L.prec = prec;
    L.D = D;
    L.P = P;
    L.E = E;
    L.N = N;
    L.NN = 1;
    for (int k = 0; k < D; ++k) L.NN *= N;
    // tensor rules: tables, elements, value offsets
    std::vector<double> tabs;
    L.nrules = (int)rule_q.size();
    L.max_q = max_q;
    for (size_t r = 0; r < rule_q.size(); ++r) {
        RuleTables<double> r64;
        RuleTables<float> r32;
        if (!build_rule(P, rule_q[r], r64, r32)) return fail(TWOLDG_EINVAL, "bad rule");
        L.rule_q[r] = rule_q[r];
        L.rule_nodes[r] = (int)tabs.size();
        tabs.insert(tabs.end(), r64.nodes.begin(), r64.nodes.end());
        L.rule_contract[r] = (int)tabs.size();
        tabs.insert(tabs.end(), r64.contract.begin(), r64.contract.end());
    }
    std::vector<RuleElement> relems;
    int64_t base = 0;
    for (size_t r = 0; r < lists.size(); ++r) {
        int64_t per = 1;
        for (int k = 0; k < D; ++k) per *= rule_q[r];
        for (const HostElem& h : lists[r]) {
            RuleElement re{};
            re.block = h.block;
            for (int k = 0; k < 3; ++k) re.e[k] = h.e[k];
            re.rule = (int)r;
            re.base = base;
            base += per;
            relems.push_back(re);
        }
        if (r == 0) {
            pl->counts[0] = (int64_t)lists[0].size();
            pl->counts[1] = base;
        } else {
            pl->counts[2] += (int64_t)lists[r].size();
        }
    }
    pl->counts[3] = base - pl->counts[1];
    L.near_base = base;
    // near elements and their chunks
    std::vector<NearElement> nelems;
    std::vector<NearChunk> chunks;
    for (size_t i = 0; i < near.size(); ++i) {
        NearElement ne{};
        ne.block = near[i].block;
        for (int k = 0; k < 3; ++k) ne.e[k] = near[i].e[k];
        ne.c0 = (int32_t)chunks.size();
        for (int64_t a = first[i]; a < first[i + 1]; a += kNearChunk)
            chunks.push_back(NearChunk{(int32_t)a, (int32_t)std::min<int64_t>(a + kNearChunk, first[i + 1]), (int32_t)i, 0});
        ne.c1 = (int32_t)chunks.size();
        nelems.push_back(ne);
    }
    pl->counts[4] = (int64_t)near.size();
    pl->counts[5] = (int64_t)nws.size();
    pl->counts[6] = (int64_t)chunks.size();
    pl->npoints = base + (int64_t)nws.size();
    pl->counts[7] = pl->npoints;
    L.n_rule_elems = (int64_t)relems.size();
    L.n_chunks = (int64_t)chunks.size();
    L.n_near_elems = (int64_t)nelems.size();
    // element tables and the finest element's node weights
    std::vector<double> bary64, gll64;
    {
        std::vector<float> b32;
        build_bary(P, bary64, b32);
        ElementTables<double> t64;
        ElementTables<float> t32;
        build_tables(P, t64, t32);
        gll64 = t64.nodes;
        int M = 1;
        for (int k = 0; k < D; ++k) M *= P1;
        std::vector<double> wn(M);
        for (int m = 0; m < M; ++m) {
            double w = 1;
            int r = m;
            for (int k = 0; k < D; ++k) {
                w = t64.weights[r % P1] * (he / 2) * w;
                r /= P1;
            }
            wn[m] = w;
        }
        std::vector<double> origins(d->origins, d->origins + nb * D), spacings(d->spacings, d->spacings + nb);
        int rc = prec == 0 ? upload_all<double>(pl.get(), origins, spacings, tabs, nxs, nws, bary64, gll64, wn)
                           : upload_all<float>(pl.get(), origins, spacings, tabs, nxs, nws, bary64, gll64, wn);
        if (rc) return rc;
    }
    const void* dp = nullptr;
    cudaError_t e = pl->upload(relems, &dp);
    if (e != cudaSuccess) return fail(TWOLDG_ECUDA, std::string("transfer upload: ") + cudaGetErrorString(e));
    L.rule_elems = static_cast<const RuleElement*>(dp);
    e = pl->upload(chunks, &dp);
    if (e != cudaSuccess) return fail(TWOLDG_ECUDA, std::string("transfer upload: ") + cudaGetErrorString(e));
    L.chunks = static_cast<const NearChunk*>(dp);
    e = pl->upload(nelems, &dp);
    if (e != cudaSuccess) return fail(TWOLDG_ECUDA, std::string("transfer upload: ") + cudaGetErrorString(e));
    L.near_elems = static_cast<const NearElement*>(dp);
    // the density source's particles
    L.nparticles = d->nparticles;
    for (int k = 0; k < d->nparticles; ++k) {
        const twoldg_particle& tp = d->particles[k];
        TransferParticle& q_ = L.particles[k];
        double vv = 0;
        for (int j = 0; j < 3; ++j) {
            q_.z[j] = tp.z[j];
            q_.v[j] = tp.v[j];
            vv += tp.v[j] * tp.v[j];
        }
        const double gamma = 1 / std::sqrt(1 - vv);
        q_.g = gamma * gamma / (gamma + 1);
        q_.ell = tp.ell;
        q_.charge = tp.charge;
    }
    pl->density_ok = D == 3;
    *out = pl.release();
    return TWOLDG_OK;
}

int twoldg_transfer_plan_destroy(twoldg_transfer_plan* plan) {
    delete plan;
    return TWOLDG_OK;
}

int twoldg_transfer_plan_counts(const twoldg_transfer_plan* plan, int64_t* counts) {
    if (!plan || !counts) return fail(TWOLDG_EINVAL, "plan and counts must not be NULL");
    std::memcpy(counts, plan->counts, sizeof plan->counts);
    return TWOLDG_OK;
}

int twoldg_transfer_points(twoldg_transfer_plan* plan, void* xs) {
    if (!plan || !xs) return fail(TWOLDG_EINVAL, "plan and xs must not be NULL");
    cudaError_t e = launch_points(plan->L, xs, plan->npoints, plan->stream);
    if (e != cudaSuccess) return fail(TWOLDG_ECUDA, std::string("transfer points: ") + cudaGetErrorString(e));
    return TWOLDG_OK;
}

static int project(twoldg_transfer_plan* plan, int source, const void* values, void* du, double factor, int32_t var) {
    if (!plan || !du) return fail(TWOLDG_EINVAL, "plan and du must not be NULL");
    if (var != 1 && var != 2) return fail(TWOLDG_EINVAL, "var is 1 (u) or 2 (v)");
    TransferLaunch L = plan->L;
    L.source = source;
    L.values = values;
    L.du = du;
    L.var = var;
    L.factor = factor;
    cudaError_t e = launch_projection(L, plan->stream);
    if (e != cudaSuccess) return fail(TWOLDG_ECUDA, std::string("projection: ") + cudaGetErrorString(e));
    return TWOLDG_OK;
}

int twoldg_project_values(twoldg_transfer_plan* plan, const void* values, void* du, double factor, int32_t var) {
    if (plan && plan->npoints > 0 && !values) return fail(TWOLDG_EINVAL, "values must not be NULL");
    return project(plan, SOURCE_VALUES, values, du, factor, var);
}

int twoldg_project_density(twoldg_transfer_plan* plan, void* du, double factor, int32_t var) {
    if (plan && !plan->density_ok) return fail(TWOLDG_EUNSUP, "the particles' density is three-dimensional");
    return project(plan, SOURCE_DENSITY, nullptr, du, factor, var);
}

}  // extern "C"
