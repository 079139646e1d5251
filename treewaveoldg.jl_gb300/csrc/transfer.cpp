// The particle-grid transfer's host side (src/transfer.jl:251-455, 918-1022,
// 1151-1285, 1380-1415): the refusals, the classification of the elements
// of the blocks the source's ball meets into the far rule, the graded bands
// and the nested rule, the nested rule's points (split at each particle's
// support, Gauss inside, Johnston and Elliott's sinh rule outside) in
// innermost lines, the pairing's support elements, compact lines and node
// gathers (:1449-1500, 1726-1797), and the C ABI over the kernels of
// transfer_kernels.cu.
// A plan keeps what does not move with the particles (the frame's geometry,
// the ball's blocks, the tables, on the host and the device) and redoes only
// what the particles' positions decide when they move, into device buffers
// it reuses. Positions, boxes and the nested rule's points are formed in
// double and rounded once to the field type when they are uploaded.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
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
        // sinh and cosh from one exponential
        const double ex = std::exp(mu * r.x[k] - eta), ix = 1 / ex;
        xs.push_back(mid + half * (xc + eps * ((ex - ix) / 2)));
        ws.push_back(r.w[k] * eps * mu * ((ex + ix) / 2) * half);
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
    // scratch per thread and per level of the recursion (an outer line's
    // points are still being visited while its inner lines are folded)
    thread_local std::vector<double> scratch[3][3];
    std::vector<double>& breaks = scratch[F][0];
    std::vector<double>& xs = scratch[F][1];
    std::vector<double>& ws = scratch[F][2];
    bool has_extent;
    double extent[2] = {0, 0};
    support_breaks(s, prefix.data(), F, lo, hi, breaks, has_extent, extent);
    double off2 = box_distance2(s.z, lo, hi, d + 1, D);
    for (int j = 0; j < F; ++j) off2 += (prefix[j] - s.z[j]) * (prefix[j] - s.z[j]);
    double a = lo[d];
    for (size_t k = 0; k <= breaks.size(); ++k) {
        const double b = k < breaks.size() ? breaks[k] : hi[d];
        if (b > a) {
            const double mid = (a + b) / 2;
            xs.clear();
            ws.clear();
            if (has_extent && extent[0] < mid && mid < extent[1]) {
                inner_points(t.inner, a, b, innermost, xs, ws);
                seg(xs, ws, true);
            } else if (!compact) {
                const double c = std::min(std::max(s.z[d], a), b);
                const double beta = std::max(std::sqrt(off2 + (s.z[d] - c) * (s.z[d] - c)),
                                             std::numeric_limits<double>::epsilon() * (b - a));
                if (beta >= (b - a) / 2)
                    sinh_points(t.mid, a, b, c, beta, xs, ws);
                else
                    sinh_points(t.sinh, a, b, c, beta, xs, ws);
                seg(xs, ws, false);
            }
        }
        a = b;
    }
}

// The nested rule's points through `prefix` in innermost lines
// (collect_points!, src/transfer.jl:1302-1328): with n dimensions remaining,
// each point of this line recurses; with one remaining, the line itself is
// emitted, its fixed coordinates (padded to two), the product w of the outer
// lines' weights, and its segments' points and weights in order.
struct NearLines {
    std::vector<double> lx, lw, vals;   // per point (in a line's own, not once laid out); per line: prefix[2], w
    std::vector<int32_t> range;         // per line: p0, p1
    std::vector<int32_t> inner;         // per line: the points inside the support's section
};

// With `compact` (the pairing's rule, whose kernel vanishes outside the
// support) every line keeps only its segments inside the support's section,
// and a line left without points is not emitted.
void collect_lines(const Support& s, const NestedTables& t, const double* lo, const double* hi,
                   std::vector<double>& prefix, double w, int n, bool compact, NearLines& out) {
    if (n == 1) {
        const int32_t p0 = (int32_t)out.lw.size();
        int32_t i0 = -1, i1 = -1;
        line_fold(s, t, lo, hi, prefix, true, compact,
                  [&](const std::vector<double>& lx, const std::vector<double>& lw, bool inside) {
                      // the inside segments are consecutive: the section is an interval
                      if (inside && i0 < 0) i0 = (int32_t)out.lw.size();
                      out.lx.insert(out.lx.end(), lx.begin(), lx.end());
                      out.lw.insert(out.lw.end(), lw.begin(), lw.end());
                      if (inside) i1 = (int32_t)out.lw.size();
                  });
        if (compact && (int32_t)out.lw.size() == p0) return;
        out.range.push_back(p0);
        out.range.push_back((int32_t)out.lw.size());
        out.inner.push_back(i0 < 0 ? 0 : i0);
        out.inner.push_back(i0 < 0 ? 0 : i1);
        out.vals.push_back(prefix.size() > 0 ? prefix[0] : 0.0);
        out.vals.push_back(prefix.size() > 1 ? prefix[1] : 0.0);
        out.vals.push_back(w);
        return;
    }
    line_fold(s, t, lo, hi, prefix, false, compact,
              [&](const std::vector<double>& lx, const std::vector<double>& lw, bool) {
                  for (size_t k = 0; k < lx.size(); ++k) {
                      prefix.push_back(lx[k]);
                      collect_lines(s, t, lo, hi, prefix, w * lw[k], n - 1, compact, out);
                      prefix.pop_back();
                  }
              });
}

struct HostElem {
    int block, e[3], particle;
};

// An element box and the particle whose support splits its nested rule.
struct LineBox {
    double lo[3], hi[3];
    int particle;
};

// fn(i) for i in [0, n) on up to 16 host threads, taken in turn.
template <typename Fn>
void parallel_for(size_t n, Fn&& fn) {
    std::atomic<size_t> next(0);
    auto work = [&]() {
        for (size_t i = next++; i < n; i = next++) fn(i);
    };
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const unsigned nt = (unsigned)std::min<size_t>(hw, n);
    std::vector<std::thread> pool;
    for (unsigned k = 1; k < nt; ++k) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
}

// The nested rule's innermost lines over the boxes, threaded as the reference
// threads its near pass (src/transfer.jl:1160-1213): over the points of each
// box's outermost line (the box's own line in one dimension), each item the
// lines through one point, kept in the serial order. The particle's own
// element holds the most points, and threading over elements left it on one
// thread. Then the layout, threaded too: each item's points at its offset in
// xs and ws (npoints each, of the field type T, which dst(npoints, xs, ws)
// provides), its lines' per-line values, ranges and inner ranges in nl.
// first[i] is box i's first line, first[n] the number of lines. Returns 0,
// 1 if the points exceed what an int32 indexes, 2 if dst failed.
template <typename T, typename Dst>
int nested_lines(const std::vector<Support>& parts, const NestedTables& nt, int D, const std::vector<LineBox>& boxes,
                 bool compact, NearLines& nl, std::vector<int64_t>& first, Dst&& dst) {
    struct Item {
        int box;
        double x, w;
    };
    std::vector<Item> items;
    for (size_t i = 0; i < boxes.size(); ++i) {
        if (D == 1) {
            items.push_back(Item{(int)i, 0.0, 1.0});
            continue;
        }
        line_fold(parts[boxes[i].particle], nt, boxes[i].lo, boxes[i].hi, std::vector<double>(), false, compact,
                  [&](const std::vector<double>& lx, const std::vector<double>& lw, bool) {
                      for (size_t k = 0; k < lx.size(); ++k) items.push_back(Item{(int)i, lx[k], lw[k]});
                  });
    }
    std::vector<NearLines> per(items.size());
    parallel_for(items.size(), [&](size_t n) {
        const Item& it = items[n];
        const LineBox& bx = boxes[it.box];
        std::vector<double> prefix;
        if (D == 1) {
            collect_lines(parts[bx.particle], nt, bx.lo, bx.hi, prefix, 1.0, 1, compact, per[n]);
        } else {
            prefix.push_back(it.x);
            collect_lines(parts[bx.particle], nt, bx.lo, bx.hi, prefix, it.w, D - 1, compact, per[n]);
        }
    });
    std::vector<int64_t> poff(per.size() + 1, 0), loff(per.size() + 1, 0);
    for (size_t n = 0; n < per.size(); ++n) {
        poff[n + 1] = poff[n] + (int64_t)per[n].lw.size();
        loff[n + 1] = loff[n] + (int64_t)per[n].range.size() / 2;
    }
    if (poff.back() > std::numeric_limits<int32_t>::max() / 2) return 1;
    first.assign(boxes.size() + 1, 0);
    for (size_t n = 0; n < per.size(); ++n) first[items[n].box + 1] = loff[n + 1];
    for (size_t i = 0; i < boxes.size(); ++i) first[i + 1] = std::max(first[i + 1], first[i]);
    T* xs = nullptr;
    T* ws = nullptr;
    if (!dst(poff.back(), xs, ws)) return 2;
    const int64_t nlines = loff.back();
    nl.vals.resize(3 * nlines);
    nl.range.resize(2 * nlines);
    nl.inner.resize(2 * nlines);
    parallel_for(per.size(), [&](size_t n) {
        NearLines& x = per[n];
        const int64_t p0 = poff[n], l0 = loff[n];
        const int32_t off = (int32_t)p0;
        for (size_t k = 0; k < x.lw.size(); ++k) {
            xs[p0 + k] = (T)x.lx[k];
            ws[p0 + k] = (T)x.lw[k];
        }
        std::copy(x.vals.begin(), x.vals.end(), nl.vals.begin() + 3 * l0);
        for (size_t k = 0; k < x.range.size(); ++k) nl.range[2 * l0 + k] = x.range[k] + off;
        for (size_t k = 0; k < x.inner.size(); k += 2) {
            const bool any = x.inner[k + 1] > x.inner[k];
            nl.inner[2 * l0 + k] = any ? x.inner[k] + off : 0;
            nl.inner[2 * l0 + k + 1] = any ? x.inner[k + 1] + off : 0;
        }
        x = NearLines();
    });
    return 0;
}

// A page-locked host buffer that grows and is never shrunk: the plan's
// points go there and to the device by an asynchronous copy.
struct PinnedBuf {
    void* p = nullptr;
    size_t cap = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() {
        if (p) cudaFreeHost(p);
    }
    cudaError_t reserve(size_t bytes) {
        bytes = std::max<size_t>(bytes, 16);
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaHostAlloc(&p, bytes, cudaHostAllocDefault);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
};

// At most kNearLines lines a chunk, fewer when the lines are few, so that a
// small set (the density's lines inside the supports) still spreads over the
// GPU's SMs.
int64_t chunk_lines(int64_t nlines) {
    return (int64_t)std::max<int64_t>(4, std::min<int64_t>(kNearLines, (nlines + 607) / 608));
}

// The tables a plan reads, built once per process in double-double and kept
// (the 1D Gauss rules of the nested rule, each tensor rule of an order, the
// element's nodes and weights).
struct TableStore {
    std::mutex m;
    std::map<std::pair<int, int>, RuleTables<double>> rules;
    std::map<int, ElementTables<double>> elements;
    std::map<int, std::vector<double>> bary;

    const RuleTables<double>& rule(int P, int q) {
        std::lock_guard<std::mutex> g(m);
        auto it = rules.find({P, q});
        if (it == rules.end()) {
            RuleTables<double> r64;
            RuleTables<float> r32;
            build_rule(P, q, r64, r32);
            it = rules.emplace(std::make_pair(P, q), std::move(r64)).first;
        }
        return it->second;
    }
    const ElementTables<double>& element(int P) {
        std::lock_guard<std::mutex> g(m);
        auto it = elements.find(P);
        if (it == elements.end()) {
            ElementTables<double> t64;
            ElementTables<float> t32;
            build_tables(P, t64, t32);
            it = elements.emplace(P, std::move(t64)).first;
        }
        return it->second;
    }
    const std::vector<double>& barycentric(int P) {
        std::lock_guard<std::mutex> g(m);
        auto it = bary.find(P);
        if (it == bary.end()) {
            std::vector<double> b64;
            std::vector<float> b32;
            build_bary(P, b64, b32);
            it = bary.emplace(P, std::move(b64)).first;
        }
        return it->second;
    }
};

TableStore& store() {
    static TableStore s;
    return s;
}

Rule1D gauss_line(int n) {
    const RuleTables<double>& r = store().rule(1, n);
    return Rule1D{r.nodes, r.weights};
}

// A device buffer that grows and is never shrunk, so that a plan's updates
// reuse it.
struct DevVec {
    void* p = nullptr;
    size_t cap = 0;
    DevVec() = default;
    DevVec(const DevVec&) = delete;
    DevVec& operator=(const DevVec&) = delete;
    ~DevVec() {
        if (p) cudaFree(p);
    }
    cudaError_t reserve(size_t bytes) {
        bytes = std::max<size_t>(bytes, 16);
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    template <typename V>
    cudaError_t put(const std::vector<V>& v) {
        cudaError_t e = reserve(v.size() * sizeof(V));
        if (e != cudaSuccess || v.empty()) return e;
        return cudaMemcpy(p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice);
    }
    // v rounded to the field type (prec 0: double, 1: float)
    cudaError_t put_field(const std::vector<double>& v, int prec) {
        if (prec == 0) return put(v);
        return put(std::vector<float>(v.begin(), v.end()));
    }
};

}  // namespace

struct twoldg_transfer_plan {
    // what does not move with the particles (SourceBall, src/transfer.jl:946-982)
    int D = 3, P = 3, E = 2, N = 8, P1 = 4, prec = 0;
    int64_t nb = 0;
    cudaStream_t stream = nullptr;
    std::vector<double> origins, spacings;
    std::vector<int32_t> levels;
    std::vector<uint8_t> mask;
    int top = 0;
    double he = 0, centre[3] = {0, 0, 0}, R = 0, rnear = 1, rfar = 9;
    std::vector<double> band_from;
    std::vector<int> rule_q;
    NestedTables nt;
    std::vector<int64_t> ball_blocks;   // the frame's blocks that meet the ball
    DevVec d_origins, d_spacings, d_tables, d_bary, d_gll, d_wn;
    // the averaging's blocks and upper neighbours (SharedNodes)
    DevVec d_avg_blocks, d_avg_upper;
    AverageLaunch A;
    // what the particles decide
    DevVec d_relems, d_lx, d_lw, d_vals, d_lines, d_chunks, d_nelems, d_partials;
    DevVec d_drelems, d_dvals, d_dlines, d_dchunks, d_delems, d_dpartials;
    // L: every element and point; Ld: the built-in density's, which vanishes
    // outside the particles' supports -- the elements that meet a support and,
    // on the near elements, the lines' points inside it
    TransferLaunch L, Ld;
    int64_t counts[8] = {0};
    int64_t npoints = 0;
    bool density_ok = false;
    // the particles as set_particles last took them, and the frame's box
    std::vector<Support> supports;
    double dom_lo[3] = {0, 0, 0}, dom_hi[3] = {0, 0, 0};
    // The pairing, built at the first pairing after the particles move: per
    // particle its support elements, their compact lines and moments, and
    // the gathers of their nodal values, plain and averaged over the elements
    // that share a node (the latter refused, with its reason, where a
    // support element is on the domain's face or next to a coarser block).
    bool pair_ready = false;
    std::string pair_cont_error;
    std::vector<int32_t> pair_list;   // (block, e0, e1, e2) per support element
    DevVec d_pelems, d_plx, d_plw, d_pvals, d_plines, d_pchunks, d_ppartials, d_pmoments;
    DevVec d_pgather, d_pgather_c, d_pbary, d_pgll, d_pout;
    PairingLaunch PL;

    // The projection's three parts run at once: the far rule on the problem's
    // stream, the graded bands on side[0], the nested rule on side[1] (of the
    // highest priority: its chain is the longest), forked from and joined
    // back into the problem's stream by events.
    cudaStream_t side[2] = {nullptr, nullptr};
    cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
    // the nested rule's points staged for the device, two stages in turn,
    // each with the event after its last copy; the per-line values
    PinnedBuf stage[2];
    cudaEvent_t staged[2] = {nullptr, nullptr};
    int stage_next = 0;
    NearLines host_lines;

    // The stream is the problem's, which may be destroyed first (a garbage
    // collector finalises in any order): wait for the device instead.
    ~twoldg_transfer_plan() {
        cudaDeviceSynchronize();
        for (int k = 0; k < 2; ++k) {
            if (side[k]) cudaStreamDestroy(side[k]);
            if (join[k]) cudaEventDestroy(join[k]);
            if (staged[k]) cudaEventDestroy(staged[k]);
        }
        if (fork) cudaEventDestroy(fork);
    }
    int set_particles(const twoldg_particle* tp, int n);
    int build_pairing();
    // the frame's block that holds x (lo <= x < hi), or -1
    int64_t locate(const double* x) const;
};

namespace {

#define TRY_CUDA(call, what)                                                                        \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return fail(TWOLDG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

// The particle-dependent plan (projection_plan, src/transfer.jl:984-1022):
// the supports' finest-level check, the elements of the ball's blocks by rule
// (host_elements, :1380-1415), the nested rule's lines (threaded over the near
// elements, each element's lines in the serial order), the density's subsets,
// and their upload into the plan's reused device buffers.
int twoldg_transfer_plan::set_particles(const twoldg_particle* tps, int np) {
    // the pairing is rebuilt from the supports kept below, the last ones taken
    pair_ready = false;
    if (np < 0 || np > kMaxParticles)
        return fail(TWOLDG_EUNSUP, "at most " + std::to_string(kMaxParticles) + " particles, got " + std::to_string(np));
    if (np > 0 && !tps) return fail(TWOLDG_EINVAL, "particles must not be NULL");
    std::vector<Support> parts(np);
    for (int k = 0; k < np; ++k) {
        Support& s = parts[k];
        s.D = D;
        double vv = 0;
        for (int j = 0; j < 3; ++j) {
            s.z[j] = j < D ? tps[k].z[j] : 0;
            s.v[j] = j < D ? tps[k].v[j] : 0;
            vv += s.v[j] * s.v[j];
        }
        s.ell = tps[k].ell;
        if (!(tps[k].ell > 0)) return fail(TWOLDG_EINVAL, "particle " + std::to_string(k) + ": ell must be positive");
        if (!(vv < 1)) return fail(TWOLDG_EINVAL, "particle " + std::to_string(k) + ": |v| must be below 1");
    }
    auto in_frame = [&](int64_t b) { return mask.empty() || mask[b]; };
    auto block_box = [&](int64_t b, double* lo, double* hi) {
        for (int k = 0; k < D; ++k) {
            lo[k] = origins[b * D + k];
            hi[k] = lo[k] + spacings[b] * N;
        }
    };
    auto elem_box = [&](int64_t b, const int* e, double* lo, double* hi) {
        for (int k = 0; k < D; ++k) {
            lo[k] = origins[b * D + k] + spacings[b] * (e[k] * P1);
            hi[k] = origins[b * D + k] + spacings[b] * ((e[k] + 1) * P1);
        }
    };
    // every support on the finest level (check_finest, src/transfer.jl:847-870)
    if (!levels.empty()) {
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
                    if (levels[b] != top)
                        return fail(TWOLDG_EINVAL, "project_source! needs the finest level, " + std::to_string(top) +
                                                       ", under every particle's support, and the support of radius " +
                                                       fmt(s.ell) + " reaches a block of level " +
                                                       std::to_string(levels[b]));
                    break;
                }
            }
        }
    }
    // the elements by rule
    const double rn = rnear * he, rf = rfar * he;
    std::vector<std::vector<HostElem>> lists(rule_q.size());
    std::vector<HostElem> near;
    int Ed[3] = {1, 1, 1};
    for (int k = 0; k < D; ++k) Ed[k] = E;
    std::vector<double> dist2(parts.size());
    for (int64_t b : ball_blocks) {
        for (int e2 = 0; e2 < Ed[2]; ++e2)
            for (int e1 = 0; e1 < Ed[1]; ++e1)
                for (int e0 = 0; e0 < Ed[0]; ++e0) {
                    const int e[3] = {e0, e1, e2};
                    double lo[3], hi[3];
                    elem_box(b, e, lo, hi);
                    if (box_distance2(centre, lo, hi, 0, D) >= R * R) continue;
                    bool host = false;
                    for (size_t k = 0; k < parts.size(); ++k) {
                        dist2[k] = box_distance2(parts[k].z, lo, hi, 0, D);
                        host = host || dist2[k] < rf * rf;
                    }
                    HostElem h{(int)b, {e0, e1, e2}, 0};
                    if (!host) {
                        lists[0].push_back(h);
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
                        lists[1 + band].push_back(h);
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
                    h.particle = (int)amin;
                    near.push_back(h);
                }
    }
    // the nested rule's lines, per near element its first line
    std::vector<LineBox> boxes(near.size());
    for (size_t i = 0; i < near.size(); ++i) {
        elem_box(near[i].block, near[i].e, boxes[i].lo, boxes[i].hi);
        boxes[i].particle = near[i].particle;
    }
    // The points go straight into a page-locked stage in the field type, two
    // stages taken in turn: the other may still be copying to the device. The
    // per-line values stay on the host, in buffers the plan keeps.
    NearLines& nl = host_lines;
    std::vector<int64_t> first;
    const int sb = stage_next;
    const size_t wsz = prec == 0 ? 8 : 4;
    int64_t npts = 0;
    cudaError_t stage_err = cudaSuccess;
    auto to_stage = [&](int64_t n, auto*& xs, auto*& ws) {
        stage_err = cudaEventSynchronize(staged[sb]);
        if (stage_err == cudaSuccess) stage_err = stage[sb].reserve(2 * (size_t)n * wsz);
        if (stage_err != cudaSuccess) return false;
        using V = std::remove_pointer_t<std::remove_reference_t<decltype(xs)>>;
        xs = static_cast<V*>(stage[sb].p);
        ws = xs + n;
        npts = n;
        return true;
    };
    const int lrc = prec == 0 ? nested_lines<double>(parts, nt, D, boxes, false, nl, first, to_stage)
                              : nested_lines<float>(parts, nt, D, boxes, false, nl, first, to_stage);
    if (lrc == 1) return fail(TWOLDG_EUNSUP, "the nested rule's points exceed 2^30");
    if (lrc == 2) return fail(TWOLDG_ECUDA, std::string("transfer stage: ") + cudaGetErrorString(stage_err));
    stage_next ^= 1;
    // tensor rule elements and the values' offsets
    std::vector<RuleElement> relems;
    int64_t base = 0;
    std::fill(counts, counts + 8, 0);
    for (size_t r = 0; r < lists.size(); ++r) {
        int64_t per_el = 1;
        for (int k = 0; k < D; ++k) per_el *= rule_q[r];
        for (const HostElem& h : lists[r]) {
            RuleElement re{};
            re.block = h.block;
            for (int k = 0; k < 3; ++k) re.e[k] = h.e[k];
            re.rule = (int)r;
            re.base = base;
            base += per_el;
            relems.push_back(re);
        }
        if (r == 0) {
            counts[0] = (int64_t)lists[0].size();
            counts[1] = base;
        } else {
            counts[2] += (int64_t)lists[r].size();
        }
    }
    counts[3] = base - counts[1];
    // near elements and their chunks of lines
    const int64_t cl = chunk_lines(first.back());
    std::vector<NearElement> nelems;
    std::vector<NearChunk> chunks;
    for (size_t i = 0; i < near.size(); ++i) {
        NearElement ne{};
        ne.block = near[i].block;
        for (int k = 0; k < 3; ++k) ne.e[k] = near[i].e[k];
        ne.c0 = (int32_t)chunks.size();
        for (int64_t a = first[i]; a < first[i + 1]; a += cl)
            chunks.push_back(NearChunk{(int32_t)a, (int32_t)std::min<int64_t>(a + cl, first[i + 1]), (int32_t)i, 0});
        ne.c1 = (int32_t)chunks.size();
        nelems.push_back(ne);
    }
    std::vector<NearLine> lines(nl.range.size() / 2);
    for (size_t l = 0; l < lines.size(); ++l) lines[l] = NearLine{nl.range[2 * l], nl.range[2 * l + 1]};
    counts[4] = (int64_t)near.size();
    counts[5] = npts;
    counts[6] = (int64_t)chunks.size();
    npoints = base + npts;
    counts[7] = npoints;
    // The density's elements and lines. Its support |L(v)(x - z)| <= ell lies
    // within |x - z| <= ell; a box farther than that (with a margin of 1e-3
    // for the field type's rounding) from every particle holds no point where
    // it is nonzero, and on a near element that meets no other particle's
    // support, a line's points outside its particle's section are outside too.
    auto meets = [&](int block, const int32_t* e, int k) {
        const int ee[3] = {e[0], e[1], e[2]};
        double lo[3], hi[3];
        elem_box(block, ee, lo, hi);
        return box_distance2(parts[k].z, lo, hi, 0, D) <= parts[k].ell * parts[k].ell * (1 + 1e-3);
    };
    std::vector<RuleElement> drelems;
    for (const RuleElement& re : relems)
        for (size_t k = 0; k < parts.size(); ++k)
            if (meets(re.block, re.e, (int)k)) {
                drelems.push_back(re);
                break;
            }
    // each list's elements by rule (both keep the rules' order)
    auto starts = [&](const std::vector<RuleElement>& v, int64_t* st) {
        for (size_t r = 0; r <= rule_q.size(); ++r) st[r] = 0;
        for (const RuleElement& re : v) ++st[re.rule + 1];
        for (size_t r = 0; r < rule_q.size(); ++r) st[r + 1] += st[r];
    };
    std::vector<NearLine> dlines;
    std::vector<double> dvals;
    std::vector<NearChunk> dchunks;
    std::vector<NearElement> delems;
    std::vector<std::pair<int64_t, int64_t>> dranges(near.size(), {0, 0});
    for (size_t i = 0; i < near.size(); ++i) {
        bool others = false;
        for (size_t k = 0; k < parts.size(); ++k)
            if ((int)k != near[i].particle && meets(near[i].block, nelems[i].e, (int)k)) others = true;
        const int64_t l0 = (int64_t)dlines.size();
        for (int64_t l = first[i]; l < first[i + 1]; ++l) {
            if (others)
                dlines.push_back(lines[l]);
            else if (nl.inner[2 * l + 1] > nl.inner[2 * l])
                dlines.push_back(NearLine{nl.inner[2 * l], nl.inner[2 * l + 1]});
            else
                continue;
            dvals.insert(dvals.end(), nl.vals.begin() + 3 * l, nl.vals.begin() + 3 * l + 3);
        }
        dranges[i] = {l0, (int64_t)dlines.size()};
    }
    const int64_t dcl = chunk_lines((int64_t)dlines.size());
    for (size_t i = 0; i < near.size(); ++i) {
        const int64_t l0 = dranges[i].first, l1 = dranges[i].second;
        if (l1 == l0) continue;
        NearElement ne = nelems[i];
        ne.c0 = (int32_t)dchunks.size();
        for (int64_t a = l0; a < l1; a += dcl)
            dchunks.push_back(NearChunk{(int32_t)a, (int32_t)std::min<int64_t>(a + dcl, l1), (int32_t)delems.size(), 0});
        ne.c1 = (int32_t)dchunks.size();
        delems.push_back(ne);
    }
    // upload: the previous projection may still read the buffers
    TRY_CUDA(cudaStreamSynchronize(stream), "transfer plan");
    int M = 1;
    for (int k = 0; k < D; ++k) M *= P1;
    TRY_CUDA(d_relems.put(relems), "transfer upload");
    TRY_CUDA(d_lx.reserve((size_t)npts * wsz), "transfer upload");
    TRY_CUDA(d_lw.reserve((size_t)npts * wsz), "transfer upload");
    if (npts > 0) {
        const char* st = static_cast<const char*>(stage[sb].p);
        TRY_CUDA(cudaMemcpyAsync(d_lx.p, st, (size_t)npts * wsz, cudaMemcpyHostToDevice, stream), "transfer upload");
        TRY_CUDA(cudaMemcpyAsync(d_lw.p, st + (size_t)npts * wsz, (size_t)npts * wsz, cudaMemcpyHostToDevice, stream),
                 "transfer upload");
        TRY_CUDA(cudaEventRecord(staged[sb], stream), "transfer upload");
    }
    TRY_CUDA(d_vals.put_field(nl.vals, prec), "transfer upload");
    TRY_CUDA(d_lines.put(lines), "transfer upload");
    TRY_CUDA(d_chunks.put(chunks), "transfer upload");
    TRY_CUDA(d_nelems.put(nelems), "transfer upload");
    TRY_CUDA(d_partials.reserve(chunks.size() * M * wsz), "transfer partials");
    TRY_CUDA(d_drelems.put(drelems), "transfer upload");
    TRY_CUDA(d_dvals.put_field(dvals, prec), "transfer upload");
    TRY_CUDA(d_dlines.put(dlines), "transfer upload");
    TRY_CUDA(d_dchunks.put(dchunks), "transfer upload");
    TRY_CUDA(d_delems.put(delems), "transfer upload");
    TRY_CUDA(d_dpartials.reserve(dchunks.size() * M * wsz), "transfer partials");
    L.rule_elems = static_cast<const RuleElement*>(d_relems.p);
    L.n_rule_elems = (int64_t)relems.size();
    starts(relems, L.rule_start);
    L.near_lx = d_lx.p;
    L.near_lw = d_lw.p;
    L.line_vals = d_vals.p;
    L.lines = static_cast<const NearLine*>(d_lines.p);
    L.n_lines = (int64_t)lines.size();
    L.chunks = static_cast<const NearChunk*>(d_chunks.p);
    L.n_chunks = (int64_t)chunks.size();
    L.near_elems = static_cast<const NearElement*>(d_nelems.p);
    L.n_near_elems = (int64_t)nelems.size();
    L.near_base = base;
    L.partials = d_partials.p;
    L.nparticles = np;
    for (int k = 0; k < np; ++k) {
        TransferParticle& q_ = L.particles[k];
        double vv = 0;
        for (int j = 0; j < 3; ++j) {
            q_.z[j] = tps[k].z[j];
            q_.v[j] = tps[k].v[j];
            vv += tps[k].v[j] * tps[k].v[j];
        }
        const double gamma = 1 / std::sqrt(1 - vv);
        q_.g = gamma * gamma / (gamma + 1);
        q_.ell = tps[k].ell;
        q_.charge = tps[k].charge;
    }
    Ld = L;
    Ld.rule_elems = static_cast<const RuleElement*>(d_drelems.p);
    Ld.n_rule_elems = (int64_t)drelems.size();
    starts(drelems, Ld.rule_start);
    Ld.line_vals = d_dvals.p;
    Ld.lines = static_cast<const NearLine*>(d_dlines.p);
    Ld.n_lines = (int64_t)dlines.size();
    Ld.chunks = static_cast<const NearChunk*>(d_dchunks.p);
    Ld.n_chunks = (int64_t)dchunks.size();
    Ld.near_elems = static_cast<const NearElement*>(d_delems.p);
    Ld.n_near_elems = (int64_t)delems.size();
    Ld.partials = d_dpartials.p;
    supports = parts;
    return TWOLDG_OK;
}

int64_t twoldg_transfer_plan::locate(const double* x) const {
    for (int64_t b = 0; b < nb; ++b) {
        if (!mask.empty() && !mask[b]) continue;
        bool in = true;
        for (int k = 0; k < D; ++k) {
            const double lo = origins[b * D + k];
            in = in && lo <= x[k] && x[k] < lo + spacings[b] * N;
        }
        if (in) return b;
    }
    return -1;
}

// The pairing's fixed part for the current particles (support_elements,
// src/transfer.jl:1726-1758; continuous_values, :1449-1500): the elements
// that hold a corner of each support's box, in the corners' order; their
// lines of the nested rule kept to the support and the moments of the
// kernel over them, launched on the plan's stream; and the two gathers.
int twoldg_transfer_plan::build_pairing() {
    if (D != 3) return fail(TWOLDG_EUNSUP, "the particles' density kernel is three-dimensional");
    const int np = (int)supports.size();
    const int M = P1 * P1 * P1;
    const int64_t NNv = (int64_t)N * N * N;
    auto elem_box = [&](int64_t b, const int* e, double* lo, double* hi) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = origins[b * 3 + k] + spacings[b] * (e[k] * P1);
            hi[k] = origins[b * 3 + k] + spacings[b] * ((e[k] + 1) * P1);
        }
    };
    auto element_of = [&](int64_t b, const double* x, int* e) {
        for (int k = 0; k < 3; ++k) {
            const int64_t i = (int64_t)std::floor((x[k] - origins[b * 3 + k]) / (spacings[b] * P1));
            e[k] = (int)std::min<int64_t>(std::max<int64_t>(i, 0), E - 1);
        }
    };
    std::vector<int32_t> list;
    std::vector<LineBox> boxes;
    int32_t firsts[kMaxParticles + 1] = {0};
    for (int k = 0; k < np; ++k) {
        const Support& s = supports[k];
        if (!(2 * s.ell < he))
            return fail(TWOLDG_EINVAL, "the particle's support, 2l = " + fmt(2 * s.ell) +
                                           " across, is not smaller than an element, h_e = " + fmt(he));
        bool inside = true;
        for (int d = 0; d < 3; ++d) inside = inside && dom_lo[d] <= s.z[d] - s.ell && s.z[d] + s.ell < dom_hi[d];
        if (!inside)
            return fail(TWOLDG_EINVAL, "the particle's support around z = (" + fmt(s.z[0]) + ", " + fmt(s.z[1]) + ", " +
                                           fmt(s.z[2]) + ") reaches past the domain's faces; the transfer does not "
                                           "look for periodic images");
        const size_t start = list.size() / 4;
        for (int corner = 0; corner < 8; ++corner) {
            double x[3];
            for (int d = 0; d < 3; ++d) x[d] = s.z[d] + ((corner >> d) & 1 ? s.ell : -s.ell);
            const int64_t b = locate(x);
            if (b < 0) return fail(TWOLDG_EINVAL, "a corner of particle " + std::to_string(k) + "'s support box is "
                                                  "outside the frame's blocks");
            int e[3];
            element_of(b, x, e);
            bool seen = false;
            for (size_t i = start; i < list.size() / 4; ++i)
                seen = seen || (list[4 * i] == b && list[4 * i + 1] == e[0] && list[4 * i + 2] == e[1] &&
                                list[4 * i + 3] == e[2]);
            if (seen) continue;
            list.insert(list.end(), {(int32_t)b, e[0], e[1], e[2]});
            LineBox bx{};
            elem_box(b, e, bx.lo, bx.hi);
            bx.particle = k;
            boxes.push_back(bx);
        }
        firsts[k + 1] = (int32_t)(list.size() / 4);
    }
    const int64_t ne = (int64_t)boxes.size();
    NearLines nl;
    std::vector<int64_t> first;
    auto to_vectors = [&](int64_t n, double*& xs, double*& ws) {
        nl.lx.resize(n);
        nl.lw.resize(n);
        xs = nl.lx.data();
        ws = nl.lw.data();
        return true;
    };
    if (nested_lines<double>(supports, nt, D, boxes, true, nl, first, to_vectors) != 0)
        return fail(TWOLDG_EUNSUP, "the pairing's points exceed 2^30");
    std::vector<NearLine> lines(nl.range.size() / 2);
    for (size_t l = 0; l < lines.size(); ++l) lines[l] = NearLine{nl.range[2 * l], nl.range[2 * l + 1]};
    const int64_t cl = chunk_lines((int64_t)lines.size());
    std::vector<PairElement> pel(ne);
    std::vector<NearChunk> chunks;
    for (int64_t i = 0; i < ne; ++i) {
        for (int k = 0; k < 3; ++k) {
            pel[i].lo[k] = boxes[i].lo[k];
            pel[i].hi[k] = boxes[i].hi[k];
        }
        pel[i].particle = boxes[i].particle;
        pel[i].c0 = (int32_t)chunks.size();
        for (int64_t a = first[i]; a < first[i + 1]; a += cl)
            chunks.push_back(NearChunk{(int32_t)a, (int32_t)std::min<int64_t>(a + cl, first[i + 1]), (int32_t)i, 0});
        pel[i].c1 = (int32_t)chunks.size();
    }
    // the gathers: per element and node (dimension 0 fastest) the state
    // offsets of variable 1; for the continuous one the element's own value
    // first, then the elements across each face, edge and corner the node is
    // on, in the reference's order (the first dimension fastest)
    auto offset = [&](int64_t b, const int* e, const int* K) {
        int64_t o = b * 2 * NNv, st = 1;
        for (int d = 0; d < 3; ++d) {
            o += (int64_t)(e[d] * P1 + K[d]) * st;
            st *= N;
        }
        return o;
    };
    std::vector<int64_t> gplain((size_t)ne * M * kGather, -1), gcont((size_t)ne * M * kGather, -1);
    for (int64_t i = 0; i < ne; ++i) {
        const int e[3] = {list[4 * i + 1], list[4 * i + 2], list[4 * i + 3]};
        for (int m = 0; m < M; ++m) {
            const int K[3] = {m % P1, (m / P1) % P1, m / (P1 * P1)};
            gplain[((size_t)i * M + m) * kGather] = offset(list[4 * i], e, K);
        }
    }
    // the continuous one stops at the first refusal, which it keeps
    pair_cont_error.clear();
    for (int64_t i = 0; i < ne && pair_cont_error.empty(); ++i) {
        const int64_t b = list[4 * i];
        const int e[3] = {list[4 * i + 1], list[4 * i + 2], list[4 * i + 3]};
        const double* lo = boxes[i].lo;
        const double* hi = boxes[i].hi;
        // the element's neighbour in each of the 26 directions, found at its
        // first use (in node order, so that a refusal is the first node's)
        bool nb_found[27] = {false};
        int64_t nb_block[27];
        int nb_e[27][3];
        for (int m = 0; m < M && pair_cont_error.empty(); ++m) {
            const int K[3] = {m % P1, (m / P1) % P1, m / (P1 * P1)};
            int64_t* gc = &gcont[((size_t)i * M + m) * kGather];
            int n = 0;
            gc[n++] = offset(b, e, K);
            int dirs[3], freed[3], nfree = 0;
            for (int d = 0; d < 3; ++d) {
                dirs[d] = K[d] == 0 ? -1 : (K[d] == P ? 1 : 0);
                if (dirs[d] != 0) freed[nfree++] = d;
            }
            for (int code = 1; code < (1 << nfree); ++code) {
                int s[3] = {0, 0, 0};
                for (int j = 0; j < nfree; ++j)
                    if ((code >> j) & 1) s[freed[j]] = dirs[freed[j]];
                int en[3];
                int64_t bn = b;
                bool within = true;
                for (int d = 0; d < 3; ++d) {
                    en[d] = e[d] + s[d];
                    within = within && 0 <= en[d] && en[d] < E;
                }
                if (!within) {
                    const int si = (s[0] + 1) + 3 * (s[1] + 1) + 9 * (s[2] + 1);
                    if (!nb_found[si]) {
                        double x[3];
                        bool in_dom = true;
                        for (int d = 0; d < 3; ++d) {
                            x[d] = (lo[d] + hi[d]) / 2 + s[d] * (hi[d] - lo[d]);
                            in_dom = in_dom && dom_lo[d] < x[d] && x[d] < dom_hi[d];
                        }
                        const int64_t found = in_dom ? locate(x) : -1;
                        const char* why = found < 0 ? " is on the domain's face; the continuous reconstruction, like "
                                                      "the transfer, does not look for periodic images"
                                          : spacings[found] != spacings[b]
                                              ? " has a neighbour on another level; the continuous reconstruction "
                                                "needs the same level across every face"
                                              : nullptr;
                        if (why) {
                            pair_cont_error = "the element at (" + fmt(lo[0]) + ", " + fmt(lo[1]) + ", " +
                                              fmt(lo[2]) + ")" + why;
                            break;
                        }
                        nb_block[si] = found;
                        element_of(found, x, nb_e[si]);
                        nb_found[si] = true;
                    }
                    bn = nb_block[si];
                    for (int d = 0; d < 3; ++d) en[d] = nb_e[si][d];
                }
                int Kn[3];
                for (int d = 0; d < 3; ++d) Kn[d] = s[d] == 0 ? K[d] : (s[d] < 0 ? P : 0);
                gc[n++] = offset(bn, en, Kn);
            }
        }
    }
    // upload (an earlier pairing may still read the buffers), then the moments
    TRY_CUDA(cudaStreamSynchronize(stream), "pairing plan");
    const ElementTables<double>& et = store().element(P);
    TRY_CUDA(d_pbary.put(store().barycentric(P)), "pairing upload");
    TRY_CUDA(d_pgll.put(et.nodes), "pairing upload");
    TRY_CUDA(d_pelems.put(pel), "pairing upload");
    TRY_CUDA(d_plx.put(nl.lx), "pairing upload");
    TRY_CUDA(d_plw.put(nl.lw), "pairing upload");
    TRY_CUDA(d_pvals.put(nl.vals), "pairing upload");
    TRY_CUDA(d_plines.put(lines), "pairing upload");
    TRY_CUDA(d_pchunks.put(chunks), "pairing upload");
    TRY_CUDA(d_pgather.put(gplain), "pairing upload");
    if (pair_cont_error.empty()) TRY_CUDA(d_pgather_c.put(gcont), "pairing upload");
    TRY_CUDA(d_ppartials.reserve(chunks.size() * kPairComponents * M * sizeof(double)), "pairing partials");
    TRY_CUDA(d_pmoments.reserve((size_t)ne * kPairComponents * M * sizeof(double)), "pairing moments");
    TRY_CUDA(d_pout.reserve((size_t)std::max(np, 1) * kPairComponents * sizeof(double)), "pairing output");
    PairingLaunch& a = PL;
    a = PairingLaunch();
    a.prec = prec;
    a.P = P;
    a.N = N;
    a.NN = NNv;
    a.nparticles = np;
    for (int k = 0; k < np; ++k) a.particles[k] = L.particles[k];
    for (int k = 0; k <= np; ++k) a.first[k] = firsts[k];
    a.elems = static_cast<const PairElement*>(d_pelems.p);
    a.n_elems = ne;
    a.lines = static_cast<const NearLine*>(d_plines.p);
    a.lx = static_cast<const double*>(d_plx.p);
    a.lw = static_cast<const double*>(d_plw.p);
    a.line_vals = static_cast<const double*>(d_pvals.p);
    a.chunks = static_cast<const NearChunk*>(d_pchunks.p);
    a.n_chunks = (int64_t)chunks.size();
    a.bary = static_cast<const double*>(d_pbary.p);
    a.gll = static_cast<const double*>(d_pgll.p);
    a.partials = static_cast<double*>(d_ppartials.p);
    a.moments = static_cast<double*>(d_pmoments.p);
    a.out = static_cast<double*>(d_pout.p);
    cudaError_t e = launch_pairing_moments(a, stream);
    if (e != cudaSuccess) return fail(TWOLDG_ECUDA, std::string("pairing moments: ") + cudaGetErrorString(e));
    pair_list = list;
    pair_ready = true;
    return TWOLDG_OK;
}

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
    std::unique_ptr<twoldg_transfer_plan> pl(new twoldg_transfer_plan());
    twoldg_transfer_plan& T = *pl;
    int D, P, E, prec;
    int64_t nb;
    cudaStream_t stream;
    if (!problem_shape(p, &D, &P, &E, &prec, &nb, &stream)) return fail(TWOLDG_EINVAL, "bad problem");
    if (D < 1 || D > 3) return fail(TWOLDG_EUNSUP, "the transfer runs in 1 to 3 dimensions");
    if (!d->origins || !d->spacings) return fail(TWOLDG_EINVAL, "origins and spacings must not be NULL");
    if (!(d->h_e > 0)) return fail(TWOLDG_EINVAL, "h_e must be positive");
    T.D = D;
    T.P = P;
    T.E = E;
    T.P1 = P + 1;
    T.N = E * (P + 1);
    T.prec = prec;
    T.nb = nb;
    T.stream = stream;
    {
        int least = 0, greatest = 0;
        TRY_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest), "transfer streams");
        TRY_CUDA(cudaStreamCreateWithPriority(&T.side[0], cudaStreamNonBlocking, least), "transfer streams");
        TRY_CUDA(cudaStreamCreateWithPriority(&T.side[1], cudaStreamNonBlocking, greatest), "transfer streams");
        TRY_CUDA(cudaEventCreateWithFlags(&T.fork, cudaEventDisableTiming), "transfer events");
        for (int k = 0; k < 2; ++k) {
            TRY_CUDA(cudaEventCreateWithFlags(&T.join[k], cudaEventDisableTiming), "transfer events");
            TRY_CUDA(cudaEventCreateWithFlags(&T.staged[k], cudaEventDisableTiming), "transfer events");
        }
    }
    // the quadrature, with the reference's defaults (src/transfer.jl:139-170)
    const int q = d->q > 0 ? d->q : P + 3;
    const int nsinh = d->nsinh > 0 ? d->nsinh : 48, nmid = d->nmid > 0 ? d->nmid : 16;
    const int ninner = d->ninner > 0 ? d->ninner : 24;
    T.rfar = d->rfar > 0 ? d->rfar : 9.0;
    T.band_from = {1, 2, 3, 4};
    std::vector<int> band_points = {14, 10, 8, 7};
    if (d->nbands > 0) {
        if (!d->band_from || !d->band_points) return fail(TWOLDG_EINVAL, "band_from and band_points must not be NULL");
        if (d->nbands > 15) return fail(TWOLDG_EUNSUP, "at most 15 graded bands");
        T.band_from.assign(d->band_from, d->band_from + d->nbands);
        band_points.assign(d->band_points, d->band_points + d->nbands);
    }
    for (size_t i = 0; i < T.band_from.size(); ++i) {
        if ((i > 0 && !(T.band_from[i - 1] < T.band_from[i])) || !(0 <= T.band_from[i] && T.band_from[i] < T.rfar))
            return fail(TWOLDG_EINVAL, "the graded rule's distances must increase from 0 and stay below rfar = " +
                                           fmt(T.rfar));
    }
    if (!(0 <= d->rnear && d->rnear <= T.rfar))
        return fail(TWOLDG_EINVAL, "rnear = " + fmt(d->rnear) + " must lie between 0 and the far rule's distance rfar = " +
                                       fmt(T.rfar));
    T.rnear = d->rnear;
    T.rule_q = {q};
    for (int b : band_points) T.rule_q.push_back(b);
    int max_q = 0;
    for (int r : T.rule_q) {
        if (r < 1 || r > kMaxRule) return fail(TWOLDG_EINVAL, "a rule needs 1.." + std::to_string(kMaxRule) + " points");
        max_q = std::max(max_q, r);
    }
    int64_t cap = 1;
    for (int k = 0; k < D; ++k) cap *= std::max(max_q, P + 1);
    if (cap > 4096) return fail(TWOLDG_EUNSUP, "a tensor rule of " + std::to_string(max_q) + "^" + std::to_string(D) +
                                                  " points exceeds the device's 4096 per element");
    if (nsinh > kMaxRule || nmid > kMaxRule || ninner > kMaxRule)
        return fail(TWOLDG_EINVAL, "the nested rule's lines take at most " + std::to_string(kMaxRule) + " points");
    T.nt = NestedTables{gauss_line(nsinh), gauss_line(nmid), gauss_line(ninner)};
    T.he = d->h_e;
    for (int k = 0; k < 3; ++k) T.centre[k] = k < D ? d->ball_centre[k] : 0;
    T.R = d->ball_radius;
    T.origins.assign(d->origins, d->origins + nb * D);
    T.spacings.assign(d->spacings, d->spacings + nb);
    if (d->levels) T.levels.assign(d->levels, d->levels + nb);
    if (d->mask) T.mask.assign(d->mask, d->mask + nb);
    // the frame's box: the hull of its blocks
    bool any = false;
    for (int64_t b = 0; b < nb; ++b) {
        if (!T.mask.empty() && !T.mask[b]) continue;
        for (int k = 0; k < D; ++k) {
            const double lo = T.origins[b * D + k], hi = lo + T.spacings[b] * T.N;
            T.dom_lo[k] = any ? std::min(T.dom_lo[k], lo) : lo;
            T.dom_hi[k] = any ? std::max(T.dom_hi[k], hi) : hi;
        }
        any = true;
    }
    // the ball's blocks and the ball's finest-level check (SourceBall,
    // check_finest, src/transfer.jl:823-845, 958-982)
    for (int64_t b = 0; b < nb; ++b)
        if (!T.levels.empty()) T.top = std::max(T.top, (int)T.levels[b]);
    for (int64_t b = 0; b < nb; ++b) {
        if (!T.mask.empty() && !T.mask[b]) continue;
        double lo[3], hi[3];
        for (int k = 0; k < D; ++k) {
            lo[k] = T.origins[b * D + k];
            hi[k] = lo[k] + T.spacings[b] * T.N;
        }
        const double r2 = box_distance2(T.centre, lo, hi, 0, D);
        if (!(r2 < T.R * T.R)) continue;
        if (!T.levels.empty() && T.levels[b] != T.top)
            return fail(TWOLDG_EINVAL,
                        "project_source! needs the finest level, " + std::to_string(T.top) +
                            ", under the source's ball of radius " + fmt(T.R) + ", and a block of level " +
                            std::to_string(T.levels[b]) + " reaches to " + fmt(std::sqrt(r2)) +
                            " from the ball's centre: the transfer measures its distances in the finest element "
                            "width h_e, and would integrate a coarser element with a rule chosen for a finer one");
        T.ball_blocks.push_back(b);
    }
    // The averaging's pairs (SharedNodes, src/transfer.jl:1520-1614): per ball
    // block and dimension the ball block across its upper face on the same
    // level, found by its integer position among the blocks of its spacing
    // (counted from the first such block, in block widths); no periodic images.
    {
        std::map<uint64_t, int64_t> first_of;   // spacing bits -> its first ball block
        std::map<std::tuple<uint64_t, int64_t, int64_t, int64_t>, int32_t> at;
        auto bits = [](double x) {
            uint64_t u;
            std::memcpy(&u, &x, sizeof u);
            return u;
        };
        auto key = [&](int64_t b, int dd) {
            const uint64_t sb = bits(T.spacings[b]);
            const int64_t r = first_of[sb];
            const double w = T.spacings[b] * T.N;
            int64_t c[3] = {0, 0, 0};
            for (int k = 0; k < D; ++k)
                c[k] = std::llround((T.origins[b * D + k] - T.origins[r * D + k]) / w) + (k == dd ? 1 : 0);
            return std::make_tuple(sb, c[0], c[1], c[2]);
        };
        for (int64_t b : T.ball_blocks) first_of.emplace(bits(T.spacings[b]), b);
        for (size_t i = 0; i < T.ball_blocks.size(); ++i) at[key(T.ball_blocks[i], -1)] = (int32_t)T.ball_blocks[i];
        std::vector<int32_t> blocks, upper;
        for (int64_t b : T.ball_blocks) {
            blocks.push_back((int32_t)b);
            for (int k = 0; k < 3; ++k) {
                int32_t u = -1;
                if (k < D) {
                    auto it = at.find(key(b, k));
                    if (it != at.end()) u = it->second;
                }
                upper.push_back(u);
            }
        }
        TRY_CUDA(T.d_avg_blocks.put(blocks), "transfer upload");
        TRY_CUDA(T.d_avg_upper.put(upper), "transfer upload");
        T.A.prec = prec;
        T.A.D = D;
        T.A.P = P;
        T.A.E = E;
        T.A.N = T.N;
        T.A.NN = 1;
        for (int k = 0; k < D; ++k) T.A.NN *= T.N;
        T.A.blocks = static_cast<const int32_t*>(T.d_avg_blocks.p);
        T.A.upper = static_cast<const int32_t*>(T.d_avg_upper.p);
        T.A.nball = (int64_t)blocks.size();
    }
    // tables and geometry on the device, once
    std::vector<double> tabs;
    TransferLaunch& L = T.L;
    L.prec = prec;
    L.D = D;
    L.P = P;
    L.E = E;
    L.N = T.N;
    L.NN = 1;
    for (int k = 0; k < D; ++k) L.NN *= T.N;
    L.nrules = (int)T.rule_q.size();
    L.max_q = max_q;
    for (size_t r = 0; r < T.rule_q.size(); ++r) {
        const RuleTables<double>& rt = store().rule(P, T.rule_q[r]);
        L.rule_q[r] = T.rule_q[r];
        L.rule_nodes[r] = (int)tabs.size();
        tabs.insert(tabs.end(), rt.nodes.begin(), rt.nodes.end());
        L.rule_contract[r] = (int)tabs.size();
        tabs.insert(tabs.end(), rt.contract.begin(), rt.contract.end());
    }
    const ElementTables<double>& et = store().element(P);
    int M = 1;
    for (int k = 0; k < D; ++k) M *= T.P1;
    std::vector<double> wn(M);
    for (int m = 0; m < M; ++m) {
        double w = 1;
        int r = m;
        for (int k = 0; k < D; ++k) {
            w = et.weights[r % T.P1] * (T.he / 2) * w;
            r /= T.P1;
        }
        wn[m] = w;
    }
    TRY_CUDA(T.d_origins.put_field(T.origins, prec), "transfer upload");
    TRY_CUDA(T.d_spacings.put_field(T.spacings, prec), "transfer upload");
    TRY_CUDA(T.d_tables.put_field(tabs, prec), "transfer upload");
    TRY_CUDA(T.d_bary.put_field(store().barycentric(P), prec), "transfer upload");
    TRY_CUDA(T.d_gll.put_field(et.nodes, prec), "transfer upload");
    TRY_CUDA(T.d_wn.put_field(wn, prec), "transfer upload");
    L.origins = T.d_origins.p;
    L.spacings = T.d_spacings.p;
    L.tables = T.d_tables.p;
    L.bary = T.d_bary.p;
    L.gll = T.d_gll.p;
    L.wn = T.d_wn.p;
    T.density_ok = D == 3;
    int rc = T.set_particles(d->particles, d->nparticles);
    if (rc) return rc;
    *out = pl.release();
    return TWOLDG_OK;
}

int twoldg_transfer_plan_update(twoldg_transfer_plan* plan, const twoldg_particle* particles, int32_t nparticles) {
    if (!plan) return fail(TWOLDG_EINVAL, "plan must not be NULL");
    return plan->set_particles(particles, nparticles);
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
    TransferLaunch L = source == SOURCE_DENSITY ? plan->Ld : plan->L;
    L.source = source;
    L.values = values;
    L.du = du;
    L.var = var;
    L.factor = factor;
    TRY_CUDA(cudaEventRecord(plan->fork, plan->stream), "projection fork");
    for (int k = 0; k < 2; ++k) TRY_CUDA(cudaStreamWaitEvent(plan->side[k], plan->fork, 0), "projection fork");
    cudaError_t e = launch_projection(L, plan->stream, plan->side[0], plan->side[1]);
    // the problem's stream waits for both sides, whatever the launches gave
    for (int k = 0; k < 2; ++k) {
        const cudaError_t r = cudaEventRecord(plan->join[k], plan->side[k]);
        const cudaError_t w = r == cudaSuccess ? cudaStreamWaitEvent(plan->stream, plan->join[k], 0) : r;
        if (e == cudaSuccess) e = w;
    }
    if (e != cudaSuccess) return fail(TWOLDG_ECUDA, std::string("projection: ") + cudaGetErrorString(e));
    return TWOLDG_OK;
}

int twoldg_project_values(twoldg_transfer_plan* plan, const void* values, void* du, double factor, int32_t var) {
    if (plan && plan->npoints > 0 && !values) return fail(TWOLDG_EINVAL, "values must not be NULL");
    return project(plan, SOURCE_VALUES, values, du, factor, var);
}

int twoldg_average_shared(twoldg_transfer_plan* plan, void* u, int32_t var) {
    if (!plan || !u) return fail(TWOLDG_EINVAL, "plan and u must not be NULL");
    if (var != 1 && var != 2) return fail(TWOLDG_EINVAL, "var is 1 (u) or 2 (v)");
    AverageLaunch A = plan->A;
    A.u = u;
    A.var = var;
    cudaError_t e = launch_average(A, plan->stream);
    if (e != cudaSuccess) return fail(TWOLDG_ECUDA, std::string("average_shared: ") + cudaGetErrorString(e));
    return TWOLDG_OK;
}

int twoldg_pairing(twoldg_transfer_plan* plan, const void* u, int32_t var, int32_t continuous, double* out) {
    if (!plan || !u || !out) return fail(TWOLDG_EINVAL, "plan, u and out must not be NULL");
    if (var != 1 && var != 2) return fail(TWOLDG_EINVAL, "var is 1 (u) or 2 (v)");
    if (!plan->pair_ready) {
        const int rc = plan->build_pairing();
        if (rc) return rc;
    }
    if (continuous && !plan->pair_cont_error.empty()) return fail(TWOLDG_EINVAL, plan->pair_cont_error);
    const int np = plan->PL.nparticles;
    if (np == 0) return TWOLDG_OK;
    PairingLaunch a = plan->PL;
    a.u = u;
    a.var = var;
    a.gather = static_cast<const int64_t*>(continuous ? plan->d_pgather_c.p : plan->d_pgather.p);
    cudaError_t e = launch_pairing_dot(a, plan->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, a.out, (size_t)np * kPairComponents * sizeof(double), cudaMemcpyDeviceToHost,
                            plan->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(plan->stream);
    if (e != cudaSuccess) return fail(TWOLDG_ECUDA, std::string("pairing: ") + cudaGetErrorString(e));
    return TWOLDG_OK;
}

int twoldg_support_elements(twoldg_transfer_plan* plan, int32_t k, int32_t* out, int32_t* n) {
    if (!plan || !out || !n) return fail(TWOLDG_EINVAL, "plan, out and n must not be NULL");
    if (k < 0 || k >= (int32_t)plan->supports.size())
        return fail(TWOLDG_EINVAL, "particle " + std::to_string(k) + " is not among the plan's " +
                                       std::to_string(plan->supports.size()));
    if (!plan->pair_ready) {
        const int rc = plan->build_pairing();
        if (rc) return rc;
    }
    const int32_t e0 = plan->PL.first[k], e1 = plan->PL.first[k + 1];
    std::memcpy(out, plan->pair_list.data() + 4 * (size_t)e0, 4 * (size_t)(e1 - e0) * sizeof(int32_t));
    *n = e1 - e0;
    return TWOLDG_OK;
}

int twoldg_project_density(twoldg_transfer_plan* plan, void* du, double factor, int32_t var) {
    if (plan && !plan->density_ok) return fail(TWOLDG_EUNSUP, "the particles' density is three-dimensional");
    return project(plan, SOURCE_DENSITY, nullptr, du, factor, var);
}

}  // extern "C"
