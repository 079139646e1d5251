// The C ABI (include/twoldg.h): problem and batch objects over the kernels.
//
// A "runner" holds one or more groups of blocks that share (D, P, E,
// truncate), each group one work list for the templated kernels; a single
// problem is a runner with one group, a batch a runner with one group per
// distinct shape. One RK4 step is 4 x [coarse-fine ghosts (if any) ->
// fused stage] per group, captured once in a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/twoldg.h"
#include "mesh.h"
#include "ops.h"
#include "tables.h"

using namespace twoldg;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(TWOLDG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                         \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

struct TableCache {
    ElementTables<double> t64[kMaxP + 1];
    ElementTables<float> t32[kMaxP + 1];
    bool built[kMaxP + 1] = {};
    bool get(int P) {
        if (P < 1 || P > kMaxP) return false;
        if (!built[P]) built[P] = build_tables(P, t64[P], t32[P]);
        return built[P];
    }
};

TableCache& tables() {
    static TableCache c;
    return c;
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t bytes) {
        if (p) { cudaFree(p); p = nullptr; }
        if (bytes == 0) bytes = 16;
        return cudaMalloc(&p, bytes);
    }
};

struct Group {
    int D = 0, P = 0, E = 0, truncate = 1;
    int64_t NN = 0, F = 1;
    std::vector<BlockItem> items;
    std::vector<CfFace> cf;
    std::vector<int> cfidx;               // per face slot its index in cf (-1: none)
    std::vector<double> h;
    std::unique_ptr<Ops> ops;
    // a flat forest's coarse-fine ghost planes as the 3D register-line
    // kernel's epilogues write them, per stage parity: u's ghost, the other
    // side's part of the gradient's ghost and this side's own part
    DevBuf eu[2], eg[2], es[2];
    DevBuf d_items, d_cf, d_cfidx, fu[2], fog[2], ugd, gfd, ggd, d_part, d_part2;
    bool metric = false;
    int full = 0;                         // 1: the full metric's two-pass stage
    std::vector<double> coef;             // per item (1 + D) N^D (or 1 + D^2: full), then the field type
    std::vector<std::vector<double>> trm, trd;  // per member: (P+1, E, nblocks, D)
    std::vector<int> member_blocks;
    DevBuf d_coef, d_trm, d_trd;
    // full metric
    DevBuf d_V, d_fv, d_bndx, d_eslot, d_ew, d_echol, d_M;
    std::vector<double> bndx, ew, echol;
    std::vector<int> eslot;
    double wave_k[3] = {0, 0, 0}, wave_phi = 0;
    int boundary = 0;
    double kappa = 0, inv_r = 0;
    // the factored truncation: per block slot, per factored block its radial
    // dimension, pair and angular table index, the angular tables
    DevBuf d_fslot, d_fradial, d_frm, d_frd, d_faslot, d_faw, d_fachol;
    // boundary kind 2: per face slot the boundary face's index (-1 inside),
    // the number of boundary faces, and the caller's table as last set (on the
    // host, and on the device where the captured kernels read it)
    std::vector<int> bidx;
    int nbf = 0;
    DevBuf d_bidx, d_btab;
    BoundaryTable h_btab{};
    double btab_dt = 0;
    bool btab_set = false;
    std::vector<int> fslot, fradial, faslot;
    std::vector<double> frm, frd, faw, fachol;
    int nslots() const { return (int)items.size() * 2 * D; }
};

}  // namespace

namespace twoldg {
// Shared with noalloc.cu, which keeps no state of its own besides its scratch.
int static_rhs_fail(int code, const std::string& msg) { return fail(code, msg); }
bool static_rhs_tables(int P, const ElementTables<double>** t64, const ElementTables<float>** t32) {
    if (!tables().get(P)) return false;
    *t64 = &tables().t64[P];
    *t32 = &tables().t32[P];
    return true;
}
}  // namespace twoldg

struct twoldg_runner {
    int prec = 0;
    size_t wsize = 8;
    int nproblems = 0;
    int64_t total_words = 0;
    cudaStream_t stream = nullptr;
    std::vector<std::unique_ptr<Group>> groups;
    std::vector<int64_t> offsets;   // per problem, words
    std::vector<double> hmin;       // per problem
    DevBuf y, acc, comp, d_rk, d_tinfo;
    std::vector<double> h_tinfo;               // per problem: t_n, dt (the full metric's stage times)
    std::vector<double> h_dts;                 // the dt each problem's coefficients were made for
    std::vector<unsigned char> h_rk;           // per problem dt/6, dt/3, dt/2, dt in the field type
    // the captured step graphs, keyed by the state pointer they were captured
    // for (a caller that alternates a few state buffers keeps them all) and
    // the steps one launch takes, most recently used first
    static constexpr int kGraphs = 6;
    struct StepGraph {
        void* u;
        int steps;
        cudaGraphExec_t exec;
    };
    std::vector<StepGraph> graphs;
    // A call takes up to kChunk steps a graph launch (its remainder in a
    // graph of its own): the steps follow one another without a gap between
    // graph launches, and in a batch of several shape groups each group's
    // chain of stages runs through them without waiting for the other groups
    // at every step, so that a group that finishes a step early starts its
    // next one instead of idling until the slowest group is done.
    static constexpr int kChunk = 16;
    void* comp_u = nullptr;
    // Shape groups of a batch never exchange data, so each group's four
    // stages are one independent branch of the step's graph: side[i] carries
    // group i+1's branch, joined back to `stream` by join[i].
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;

    ~twoldg_runner() {
        drop_graphs();
        for (auto e : join) cudaEventDestroy(e);
        for (auto st : side) cudaStreamDestroy(st);
        if (fork) cudaEventDestroy(fork);
        if (stream) cudaStreamDestroy(stream);
    }

    int setup(int n, const twoldg_desc* descs) {
        if (n < 1 || !descs) return fail(TWOLDG_EINVAL, "no problem descriptors");
        prec = descs[0].precision;
        if (prec != TWOLDG_F64 && prec != TWOLDG_F32 && prec != TWOLDG_F32C)
            return fail(TWOLDG_EINVAL, "precision must be TWOLDG_F64, TWOLDG_F32 or TWOLDG_F32C");
        wsize = prec == TWOLDG_F64 ? 8 : 4;
        nproblems = n;
        std::map<std::tuple<int, int, int, int>, int> gidx;
        for (int k = 0; k < n; ++k) {
            const twoldg_desc& d = descs[k];
            if (d.precision != prec) return fail(TWOLDG_EINVAL, "all members of a batch must share one precision");
            Mesh m;
            std::string err;
            if (!build_mesh(d, m, err)) return fail(TWOLDG_EINVAL, err);
            if (!tables().get(m.P))
                return fail(TWOLDG_EUNSUP, "element order P = " + std::to_string(m.P) + " is not built (1..8)");
            const bool metric = d.coef != nullptr;
            const int full = d.metric == 2 ? 1 : 0;
            if (d.metric < 0 || d.metric > 2)
                return fail(TWOLDG_EINVAL, "metric must be 0 (flat), 1 (diagonal) or 2 (full), not " +
                                               std::to_string(d.metric));
            if (d.metric == 1 && !d.coef) return fail(TWOLDG_EINVAL, "a diagonal metric (metric = 1) needs coef");
            // The flat and diagonal kernels read a neighbour's face plane as it
            // lies (no orientation, no boundary face): an explicit face table
            // (glued patches, boundary faces) needs the full metric's kernels.
            if (d.face_nb && !full)
                return fail(TWOLDG_EUNSUP, "an explicit face table (face_nb) is served by the full metric "
                                           "(metric = 2) only: a flat or diagonal forest is a brick of roots");
            if (full) {
                if (m.D != 3) return fail(TWOLDG_EINVAL, "the full metric is three-dimensional");
                if (!d.coef || !d.elem_slot || !d.bnd_x)
                    return fail(TWOLDG_EINVAL, "a full metric needs coef, elem_slot and bnd_x");
                if (n != 1) return fail(TWOLDG_EUNSUP, "a full-metric problem is stepped alone, not in a batch");
                if (d.boundary != 0 && d.boundary != 1 && d.boundary != 2)
                    return fail(TWOLDG_EINVAL, "boundary must be 0 (Dirichlet plane wave), 1 (radiative) or 2 "
                                               "(Dirichlet values the caller supplies)");
                if (d.boundary == 1 && !(d.kappa >= 0))
                    return fail(TWOLDG_EINVAL, "kappa = " + std::to_string(d.kappa) +
                                                   " is negative, and a radiative boundary with kappa < 0 feeds "
                                                   "energy in: take kappa >= 0, 1 for Sommerfeld's condition");
                if (d.boundary == 1 && !(d.inv_r >= 0))
                    return fail(TWOLDG_EINVAL, "inv_r must be 1/R >= 0, or 0 without the u/R term");
            }
            if (metric && !full && (!d.trunc_modes || !d.trunc_duals))
                return fail(TWOLDG_EINVAL, "a metric (coef) needs its truncation pairs (trunc_modes, trunc_duals)");
            if (metric && !full && !m.cf.empty())
                return fail(TWOLDG_EINVAL, "a geometry takes refinement only in an affine patch, which a diagonal "
                                           "metric's coefficients do not describe: no coarse-fine faces with coef");
            auto key = std::make_tuple(m.D, m.P, m.E, (d.truncate ? 1 : 0) + (metric ? 2 : 0) + (full ? 4 : 0));
            auto gi = gidx.find(key);
            Group* g;
            if (gi == gidx.end()) {
                gidx[key] = (int)groups.size();
                groups.emplace_back(new Group());
                g = groups.back().get();
                g->D = m.D; g->P = m.P; g->E = m.E; g->truncate = d.truncate ? 1 : 0;
                g->metric = metric;
                g->full = full;
                g->NN = m.NN;
                for (int q = 0; q < m.D - 1; ++q) g->F *= m.N;
                Ops* ops = nullptr;
                if (m.D == 1) ops = make_ops_d1(prec, m.P, tables().t64[m.P], tables().t32[m.P]);
                if (m.D == 2) ops = make_ops_d2(prec, m.P, tables().t64[m.P], tables().t32[m.P]);
                if (m.D == 3) ops = make_ops_d3(prec, m.P, tables().t64[m.P], tables().t32[m.P]);
                if (!ops) return fail(TWOLDG_EUNSUP, "no kernels for P = " + std::to_string(m.P) + " (built: 1..6)");
                g->ops.reset(ops);
            } else {
                g = groups[gi->second].get();
            }
            const int64_t base = total_words;
            const int slot0 = g->nslots();
            for (auto it : m.items) {
                it.off += base;
                it.slot += slot0;
                for (int f = 0; f < 6; ++f)
                    if (it.nb[f] >= 0) it.nb[f] += slot0;
                it.problem = k;
                g->items.push_back(it);
            }
            for (auto c : m.cf) {
                c.slot += slot0;
                for (int q = 0; q < 4; ++q) c.src[q] += slot0;
                g->cf.push_back(c);
            }
            g->h.insert(g->h.end(), m.h.begin(), m.h.end());
            if (full) {
                const size_t nc = (size_t)(1 + m.D * m.D) * m.NN * m.nblocks;
                g->coef.insert(g->coef.end(), d.coef, d.coef + nc);
                size_t F = 1;
                for (int q = 0; q < m.D - 1; ++q) F *= m.N;
                g->bndx.assign(d.bnd_x, d.bnd_x + (size_t)m.nblocks * 2 * m.D * 3 * F);
                g->eslot.assign(d.elem_slot, d.elem_slot + m.nblocks);
                const size_t P1 = m.P + 1, ne = (size_t)m.E * m.E * m.E;
                const size_t n3 = P1 * P1 * P1, m3 = (size_t)m.P * m.P * m.P;
                if (d.elem_ntab > 0) {
                    g->ew.assign(d.elem_w, d.elem_w + n3 * ne * d.elem_ntab);
                    g->echol.assign(d.elem_chol, d.elem_chol + m3 * m3 * ne * d.elem_ntab);
                }
                for (int q = 0; q < 3; ++q) g->wave_k[q] = d.wave_k[q];
                g->wave_phi = d.wave_phi;
                g->boundary = d.boundary;
                g->bidx.assign((size_t)m.nblocks * 2 * m.D, -1);
                for (size_t q = 0; q < g->bidx.size(); ++q)
                    if (d.face_nb[q] == -1) g->bidx[q] = g->nbf++;
                g->kappa = d.kappa;
                g->inv_r = d.inv_r;
                g->fslot.assign(m.nblocks, 0);
                if (d.fac_slot) {
                    int nf = 0;
                    for (int b = 0; b < m.nblocks; ++b) {
                        const int f = d.fac_slot[b];
                        if (f < 0 || f > m.nblocks) return fail(TWOLDG_EINVAL, "fac_slot out of range");
                        if (f > 0 && d.elem_slot[b] != 0)
                            return fail(TWOLDG_EINVAL, "block " + std::to_string(b) +
                                                           " has both per-element and factored truncation tables");
                        g->fslot[b] = f;
                        nf = std::max(nf, f);
                    }
                    if (nf > 0) {
                        if (!d.fac_radial || !d.fac_rmodes || !d.fac_rduals || !d.fac_aslot || !d.fac_aw ||
                            !d.fac_achol || d.fac_ntab < 1)
                            return fail(TWOLDG_EINVAL, "fac_slot names factored blocks but their tables are missing");
                        g->fradial.assign(d.fac_radial, d.fac_radial + nf);
                        g->faslot.assign(d.fac_aslot, d.fac_aslot + nf);
                        for (int f = 0; f < nf; ++f)
                            if (g->fradial[f] < 0 || g->fradial[f] > 2 || g->faslot[f] < 0 ||
                                g->faslot[f] >= d.fac_ntab)
                                return fail(TWOLDG_EINVAL, "factored block " + std::to_string(f) +
                                                               " has a bad radial dimension or angular table");
                        const size_t nr = P1 * m.E * nf, n2 = P1 * P1, m2 = (size_t)m.P * m.P;
                        const size_t e2 = (size_t)m.E * m.E;
                        g->frm.assign(d.fac_rmodes, d.fac_rmodes + nr);
                        g->frd.assign(d.fac_rduals, d.fac_rduals + nr);
                        g->faw.assign(d.fac_aw, d.fac_aw + n2 * e2 * d.fac_ntab);
                        g->fachol.assign(d.fac_achol, d.fac_achol + m2 * m2 * e2 * d.fac_ntab);
                    }
                }
            } else if (metric) {
                const size_t nc = (size_t)(1 + m.D) * m.NN * m.nblocks;
                g->coef.insert(g->coef.end(), d.coef, d.coef + nc);
                const size_t nt = (size_t)(m.P + 1) * m.E * m.nblocks * m.D;
                g->trm.emplace_back(d.trunc_modes, d.trunc_modes + nt);
                g->trd.emplace_back(d.trunc_duals, d.trunc_duals + nt);
                g->member_blocks.push_back(m.nblocks);
            }
            offsets.push_back(base);
            hmin.push_back(m.hmin);
            total_words += 2 * m.NN * m.nblocks;
        }
        for (auto& gp : groups) {
            Group& g = *gp;
            if (g.ops->stage_smem(g.E) > 227 * 1024)
                return fail(TWOLDG_EUNSUP, "block of N = " + std::to_string(g.E * (g.P + 1)) + " nodes per dim in " +
                                               std::to_string(g.D) + "D does not fit one CTA's shared memory");
        }
        // The smallest shape groups first: their stage launches are few CTAs
        // and bound by latency, so launched first they are all resident at once
        // and the large groups' CTAs fill the GPU around them, where a large
        // launch first would hold every SM until its last wave is dispatched.
        std::stable_sort(groups.begin(), groups.end(), [](const std::unique_ptr<Group>& a,
                                                          const std::unique_ptr<Group>& b) {
            return (int64_t)a->items.size() * a->NN < (int64_t)b->items.size() * b->NN;
        });
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        if (groups.size() > 1) {
            CK(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
            for (size_t i = 1; i < groups.size(); ++i) {
                cudaStream_t st;
                cudaEvent_t ev;
                CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
                side.push_back(st);
                CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
                join.push_back(ev);
            }
        }
        for (auto& gp : groups) {
            Group& g = *gp;
            size_t fbytes = (size_t)g.nslots() * g.F * wsize;
            CK(g.d_items.alloc(g.items.size() * sizeof(BlockItem)));
            CK(cudaMemcpy(g.d_items.p, g.items.data(), g.items.size() * sizeof(BlockItem), cudaMemcpyHostToDevice));
            CK(g.d_cf.alloc(g.cf.size() * sizeof(CfFace)));
            if (!g.cf.empty())
                CK(cudaMemcpy(g.d_cf.p, g.cf.data(), g.cf.size() * sizeof(CfFace), cudaMemcpyHostToDevice));
            if (!g.cf.empty() && !g.full) {
                g.cfidx.assign(g.nslots(), -1);
                for (size_t i = 0; i < g.cf.size(); ++i) g.cfidx[g.cf[i].slot] = (int)i;
                CK(g.d_cfidx.alloc(g.cfidx.size() * sizeof(int)));
                CK(cudaMemcpy(g.d_cfidx.p, g.cfidx.data(), g.cfidx.size() * sizeof(int), cudaMemcpyHostToDevice));
                for (int i = 0; i < 2; ++i) {
                    CK(g.eu[i].alloc(fbytes));
                    CK(g.eg[i].alloc(fbytes));
                    CK(g.es[i].alloc(fbytes));
                }
            }
            for (int i = 0; i < 2; ++i) {
                CK(g.fu[i].alloc(fbytes));
                CK(g.fog[i].alloc(fbytes));
                CK(cudaMemset(g.fu[i].p, 0, fbytes));
                CK(cudaMemset(g.fog[i].p, 0, fbytes));
            }
            size_t dbytes = g.cf.empty() ? 16 : fbytes;
            CK(g.ugd.alloc(dbytes));
            CK(g.gfd.alloc(dbytes));
            // the full metric's dense gradient ghosts are the three Cartesian components
            CK(g.ggd.alloc(g.full && !g.cf.empty() ? 3 * dbytes : dbytes));
            CK(g.d_part.alloc(g.items.size() * sizeof(double)));
            CK(g.d_part2.alloc(g.items.size() * sizeof(double)));
            if (g.full) {
                // sqrt(g) g^de = S[d] . S[e] / sqrt(g) per node, the gradient pass's
                // flux coefficients, formed once in double and rounded once
                std::vector<double> M((size_t)6 * g.NN * g.items.size());
                const int pairs[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
                for (size_t b = 0; b < g.items.size(); ++b)
                    for (int64_t n = 0; n < g.NN; ++n) {
                        const double* cb = g.coef.data() + b * 10 * g.NN;
                        const double J = cb[n];
                        for (int k = 0; k < 6; ++k) {
                            double s = 0;
                            for (int i = 0; i < 3; ++i)
                                s += cb[(1 + 3 * pairs[k][0] + i) * g.NN + n] * cb[(1 + 3 * pairs[k][1] + i) * g.NN + n];
                            M[(b * 6 + k) * g.NN + n] = s / J;
                        }
                    }
                int r = upload_t(g.d_coef, g.coef);
                if (!r) r = upload_t(g.d_M, M);
                if (!r) r = upload_t(g.d_ew, g.ew.empty() ? std::vector<double>(1, 0.0) : g.ew);
                if (!r) r = upload_t(g.d_echol, g.echol.empty() ? std::vector<double>(1, 0.0) : g.echol);
                if (r) return r;
                CK(g.d_V.alloc((size_t)g.items.size() * 3 * g.NN * wsize));
                CK(g.d_fv.alloc((size_t)g.nslots() * 3 * g.F * wsize));
                CK(cudaMemset(g.d_fv.p, 0, (size_t)g.nslots() * 3 * g.F * wsize));
                CK(g.d_bndx.alloc(g.bndx.size() * sizeof(double)));
                CK(cudaMemcpy(g.d_bndx.p, g.bndx.data(), g.bndx.size() * sizeof(double), cudaMemcpyHostToDevice));
                CK(g.d_bidx.alloc(g.bidx.size() * sizeof(int)));
                CK(cudaMemcpy(g.d_bidx.p, g.bidx.data(), g.bidx.size() * sizeof(int), cudaMemcpyHostToDevice));
                CK(g.d_btab.alloc(sizeof(BoundaryTable)));
                CK(cudaMemset(g.d_btab.p, 0, sizeof(BoundaryTable)));
                CK(g.d_eslot.alloc(g.eslot.size() * sizeof(int)));
                CK(cudaMemcpy(g.d_eslot.p, g.eslot.data(), g.eslot.size() * sizeof(int), cudaMemcpyHostToDevice));
                CK(g.d_fslot.alloc(g.fslot.size() * sizeof(int)));
                CK(cudaMemcpy(g.d_fslot.p, g.fslot.data(), g.fslot.size() * sizeof(int), cudaMemcpyHostToDevice));
                if (!g.fradial.empty()) {
                    CK(g.d_fradial.alloc(g.fradial.size() * sizeof(int)));
                    CK(cudaMemcpy(g.d_fradial.p, g.fradial.data(), g.fradial.size() * sizeof(int),
                                  cudaMemcpyHostToDevice));
                    CK(g.d_faslot.alloc(g.faslot.size() * sizeof(int)));
                    CK(cudaMemcpy(g.d_faslot.p, g.faslot.data(), g.faslot.size() * sizeof(int),
                                  cudaMemcpyHostToDevice));
                    int rr = upload_t(g.d_frm, g.frm);
                    if (!rr) rr = upload_t(g.d_frd, g.frd);
                    if (!rr) rr = upload_t(g.d_faw, g.faw);
                    if (!rr) rr = upload_t(g.d_fachol, g.fachol);
                    if (rr) return rr;
                }
            } else if (g.metric) {
                // the per-line tables of every member into the group's (P+1, E, nitems, D) layout
                const int P1 = g.P + 1, nit = (int)g.items.size();
                std::vector<double> tm((size_t)P1 * g.E * nit * g.D), td(tm.size());
                int item0 = 0;
                for (size_t mbr = 0; mbr < g.member_blocks.size(); ++mbr) {
                    const int nb = g.member_blocks[mbr];
                    for (int dd = 0; dd < g.D; ++dd)
                        for (int b = 0; b < nb; ++b)
                            for (int e = 0; e < g.E; ++e)
                                for (int i = 0; i < P1; ++i) {
                                    size_t src = i + (size_t)P1 * (e + (size_t)g.E * (b + (size_t)nb * dd));
                                    size_t dst = i + (size_t)P1 * (e + (size_t)g.E * (item0 + b + (size_t)nit * dd));
                                    tm[dst] = g.trm[mbr][src];
                                    td[dst] = g.trd[mbr][src];
                                }
                    item0 += nb;
                }
                int r = upload_t(g.d_coef, g.coef);
                if (!r) r = upload_t(g.d_trm, tm);
                if (!r) r = upload_t(g.d_trd, td);
                if (r) return r;
            }
        }
        size_t sbytes = (size_t)total_words * wsize;
        if (y.alloc(sbytes) != cudaSuccess || acc.alloc(sbytes) != cudaSuccess)
            return fail(TWOLDG_ENOMEM, "stage scratch allocation failed");
        if (prec == TWOLDG_F32C) {
            if (comp.alloc(sbytes) != cudaSuccess) return fail(TWOLDG_ENOMEM, "compensation allocation failed");
            CK(cudaMemset(comp.p, 0, sbytes));
        }
        CK(d_rk.alloc(n * 4 * wsize));
        CK(d_tinfo.alloc(n * 2 * sizeof(double)));
        h_tinfo.assign(n * 2, 0.0);
        CK(cudaMemcpy(d_tinfo.p, h_tinfo.data(), n * 2 * sizeof(double), cudaMemcpyHostToDevice));
        h_dts.assign(n, 0.0);
        h_rk.assign(n * 4 * wsize, 0);
        CK(cudaMemcpy(d_rk.p, h_rk.data(), h_rk.size(), cudaMemcpyHostToDevice));
        return TWOLDG_OK;
    }

    // doubles -> the field type, rounded once, onto the device
    int upload_t(DevBuf& buf, const std::vector<double>& v) {
        CK(buf.alloc(v.size() * wsize));
        if (wsize == 8) {
            CK(cudaMemcpy(buf.p, v.data(), v.size() * 8, cudaMemcpyHostToDevice));
        } else {
            std::vector<float> f(v.begin(), v.end());
            CK(cudaMemcpy(buf.p, f.data(), f.size() * 4, cudaMemcpyHostToDevice));
        }
        return TWOLDG_OK;
    }

    StagePtrs ptrs(Group& g, void* u, int in) {
        StagePtrs p{};
        p.u = u;
        p.y = y.p;
        p.acc = acc.p;
        p.comp = comp.p;
        p.du = nullptr;
        p.fu_in = g.fu[in].p;
        p.fog_in = g.fog[in].p;
        p.fu_out = g.fu[1 - in].p;
        p.fog_out = g.fog[1 - in].p;
        p.ugd = g.ugd.p;
        p.ggd = g.ggd.p;
        p.rk = d_rk.p;
        p.partial = (double*)g.d_part.p;
        p.coef = g.metric ? g.d_coef.p : nullptr;
        p.trm = g.metric ? g.d_trm.p : nullptr;
        p.trd = g.metric ? g.d_trd.p : nullptr;
        return p;
    }

    // An RK stage's pointers: on a forest with refinement its coarse-fine
    // ghost planes of parity `in` (which the previous stage's epilogues, or
    // prime_cf, wrote) and the next stage's (the other passes read the planes
    // cf_all fills).
    StagePtrs stage_ptrs(Group& g, void* u, int in) {
        StagePtrs p = ptrs(g, u, in);
        // one group's chain of stages: each stage kernel may become resident
        // while the one before finishes. The groups of a batch run their
        // chains side by side, where a stage waiting on its SMs would hold
        // them from another group's running stage.
        p.pdl = groups.size() == 1;
        if (!g.cf.empty()) {
            p.cf = (const CfFace*)g.d_cf.p;
            p.cfidx = (const int*)g.d_cfidx.p;
            p.ncf = (int)g.cf.size();
            p.ugd = g.eu[in].p;
            p.ggd = g.eg[in].p;
            p.gsd = g.es[in].p;
            p.ugd_out = g.eu[1 - in].p;
            p.ggd_out = g.eg[1 - in].p;
            p.gsd_out = g.es[1 - in].p;
        }
        return p;
    }

    // The first stage's coarse-fine ghost planes of every flat group with
    // refinement, from the face exports of u: u's and the whole gradient
    // ghost, with no own part.
    int prime_cf() {
        for (auto& gp : groups) {
            Group& g = *gp;
            if (g.full || g.cf.empty()) continue;
            CK(g.ops->cf_ghosts((const CfFace*)g.d_cf.p, (int)g.cf.size(), g.E, g.fu[0].p, g.fog[0].p, g.eu[0].p,
                                nullptr, g.eg[0].p, stream));
            CK(cudaMemsetAsync(g.es[0].p, 0, (size_t)g.nslots() * g.F * wsize, stream));
        }
        return TWOLDG_OK;
    }

    FmPtrs fptrs(Group& g, void* u, int in) {
        FmPtrs p{};
        // a full-metric problem is one group: its passes as programmatic
        // dependent launches, as the flat stage kernels of a one-group problem
        p.pdl = groups.size() == 1;
        p.u = u;
        p.y = y.p;
        p.acc = acc.p;
        p.comp = comp.p;
        p.fu_in = g.fu[in].p;
        p.fu_out = g.fu[1 - in].p;
        p.V = g.d_V.p;
        p.fv = g.d_fv.p;
        p.coef = g.d_coef.p;
        p.M = g.d_M.p;
        p.rk = d_rk.p;
        p.tinfo = (const double*)d_tinfo.p;
        p.bnd_x = (const double*)g.d_bndx.p;
        for (int q = 0; q < 3; ++q) p.wave_k[q] = g.wave_k[q];
        p.wave_phi = g.wave_phi;
        p.eslot = (const int*)g.d_eslot.p;
        p.boundary = g.boundary;
        p.kappa = g.kappa;
        p.inv_r = g.inv_r;
        p.fslot = (const int*)g.d_fslot.p;
        p.fradial = (const int*)g.d_fradial.p;
        p.frm = g.d_frm.p;
        p.frd = g.d_frd.p;
        p.faslot = (const int*)g.d_faslot.p;
        p.faw = g.d_faw.p;
        p.fachol = g.d_fachol.p;
        p.bidx = (const int*)g.d_bidx.p;
        p.btab = (const BoundaryTable*)g.d_btab.p;
        p.ugd = g.cf.empty() ? nullptr : g.ugd.p;
        p.vgd = g.cf.empty() ? nullptr : g.ggd.p;
        p.ew = g.d_ew.p;
        p.echol = g.d_echol.p;
        p.partial = (double*)g.d_part.p;
        return p;
    }

    // the full metric's stage times: t_n and dt of every problem
    int set_time(double t, const double* dts) {
        for (int k = 0; k < nproblems; ++k) {
            h_tinfo[2 * k] = t;
            h_tinfo[2 * k + 1] = dts ? dts[k] : 0.0;
        }
        CK(cudaMemcpyAsync(d_tinfo.p, h_tinfo.data(), h_tinfo.size() * sizeof(double), cudaMemcpyHostToDevice,
                           stream));
        return TWOLDG_OK;
    }

    // Boundary kind 2: the caller's table must hold every stage time that a
    // call from t of nsteps steps of size dt reaches (t + j dt/2, j = 0 ..
    // 2 nsteps), as levels of its own spacing; nsteps = 0 asks for t alone.
    int boundary_window(double t, double dt, int nsteps) {
        for (auto& gp : groups) {
            Group& g = *gp;
            if (!g.full || g.boundary != 2) continue;
            if (!g.btab_set)
                return fail(TWOLDG_EINVAL, "the problem's Dirichlet data are the caller's (boundary 2) and none "
                                           "were given: call twoldg_set_boundary_values first");
            const double half = 0.5 * g.btab_dt;
            const double kf = (t - g.h_btab.t0) / half;
            const double k0 = std::nearbyint(kf);
            if (!(std::fabs(kf - k0) <= 1e-6))
                return fail(TWOLDG_EINVAL, "t = " + std::to_string(t) + " is not a level of the boundary values "
                                           "(t0 + k dt/2)");
            if (nsteps > 0 && !(std::fabs(dt - g.btab_dt) <= 1e-12 * g.btab_dt))
                return fail(TWOLDG_EINVAL, "the step dt differs from the boundary values' dt");
            if (k0 < 0 || k0 + 2.0 * nsteps > g.h_btab.nlevels - 1)
                return fail(TWOLDG_EINVAL, "the boundary values' " + std::to_string(g.h_btab.nlevels) +
                                               " levels do not cover the call's stage times");
        }
        return TWOLDG_OK;
    }

    bool any_full() const {
        for (auto& g : groups)
            if (g->full) return true;
        return false;
    }

    int export_all(const void* u) {
        for (auto& gp : groups) {
            Group& g = *gp;
            CK(g.ops->export_faces((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, u, g.fu[0].p,
                                   g.fog[0].p, stream));
        }
        return TWOLDG_OK;
    }

    int cf_all(Group& g, int in) {
        if (g.cf.empty()) return TWOLDG_OK;
        CK(g.ops->cf_ghosts((const CfFace*)g.d_cf.p, (int)g.cf.size(), g.E, g.fu[in].p, g.fog[in].p, g.ugd.p,
                            g.gfd.p, g.ggd.p, stream));
        return TWOLDG_OK;
    }

    // Stage s of group g (reading the face planes `in`), enqueued on st.
    // The full metric's coarse-fine ghosts (a refined brick patch): u's from
    // the face exports before the gradient pass (vars 1), V's from its face
    // planes before the stage pass (vars 3).
    int fm_dense(Group& g, const FmPtrs& fp, int vars, cudaStream_t st) {
        if (g.cf.empty()) return TWOLDG_OK;
        const void* src = vars == 1 ? fp.fu_in : (const void*)fp.fv;
        void* dst = vars == 1 ? g.ugd.p : g.ggd.p;
        CK(g.ops->cf_planes((const CfFace*)g.d_cf.p, (int)g.cf.size(), g.E, src, dst, vars, st));
        return TWOLDG_OK;
    }

    int enqueue_stage(Group& g, void* u, int s, int in, cudaStream_t st) {
        if (g.full) {
            FmPtrs fp = fptrs(g, u, in);
            int r = fm_dense(g, fp, 1, st);
            if (r) return r;
            CK(g.ops->fm_gradient((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, s, fp, st));
            r = fm_dense(g, fp, 3, st);
            if (r) return r;
            CK(g.ops->fm_stage((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, s, g.truncate, fp, st));
            return TWOLDG_OK;
        }
        StagePtrs p = stage_ptrs(g, u, in);
        CK(g.ops->stage((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, s, g.truncate, p, 0, st));
        return TWOLDG_OK;
    }

    // One RK4 step of group g, its four stages enqueued on st.
    int enqueue_group(Group& g, void* u, cudaStream_t st) {
        for (int s = 1; s <= 4; ++s) {
            int r = enqueue_stage(g, u, s, (s - 1) & 1, st);
            if (r) return r;
        }
        return TWOLDG_OK;
    }

    // `steps` RK4 steps, enqueued on `stream` (captured into the graph):
    // group 0 on `stream`, every other group on its side stream between a
    // fork and a join, so that the graph runs the groups' chains side by
    // side; groups never exchange data, so each chain takes all its steps
    // before the join. The full metric's boundary reads the problems' time,
    // advanced on the device after every step: its steps each take a fork,
    // the groups' four stages and a join before the advance.
    int enqueue_step(void* u, int steps = 1) {
        const bool full = any_full();
        for (int k0 = 0; k0 < steps; k0 += full ? 1 : steps) {
            const int n = full ? 1 : steps;
            if (groups.size() > 1) CK(cudaEventRecord(fork, stream));
            for (size_t i = 0; i < groups.size(); ++i) {
                cudaStream_t st = i == 0 ? stream : side[i - 1];
                if (i > 0) CK(cudaStreamWaitEvent(st, fork, 0));
                for (int k = 0; k < n; ++k) {
                    int r = enqueue_group(*groups[i], u, st);
                    if (r) return r;
                }
                if (i > 0) CK(cudaEventRecord(join[i - 1], st));
            }
            for (size_t i = 1; i < groups.size(); ++i) CK(cudaStreamWaitEvent(stream, join[i - 1], 0));
            if (full) {
                fm_advance_time(stream);
                CK(cudaGetLastError());
            }
        }
        return TWOLDG_OK;
    }

    void fm_advance_time(cudaStream_t s);

    void drop_graphs() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.exec);
        graphs.clear();
    }

    // The autotuner: for every shape group, time each launch layout the
    // group's kernels offer on stages 1 to 3 of a step from u (which they do
    // not change: they write only the stage scratch and the face planes) and
    // keep the fastest. Layouts found in the cache file (a JSON object, one
    // entry per line, as this function writes it) are taken without timing;
    // new ones are added to it. report receives the chosen layouts in the
    // same form.
    int autotune(void* u, const double* dts, const char* cache, std::string& report) {
        int r = rk4(u, dts, 0);
        if (r) return r;
        r = export_all(u);
        if (!r) r = prime_cf();
        if (r) return r;
        std::map<std::string, std::string> lines;  // key -> the entry's text
        std::map<std::string, Launch> known;
        if (cache) {
            std::ifstream in(cache);
            std::string line;
            while (std::getline(in, line)) {
                const size_t q0 = line.find('"'), q1 = line.find('"', q0 + 1);
                if (q0 == std::string::npos || q1 == std::string::npos) continue;
                Launch l{};
                if (std::sscanf(line.c_str() + q1 + 1, ": {\"kernel\": %d, \"threads\": %d, \"waves\": %d", &l.kernel,
                                &l.threads, &l.waves) != 3)
                    continue;
                const std::string key = line.substr(q0 + 1, q1 - q0 - 1);
                known[key] = l;
                std::string body = line.substr(q0);
                while (!body.empty() && (body.back() == ',' || body.back() == ' ' || body.back() == '\r')) body.pop_back();
                lines[key] = body;
            }
        }
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        const char* pname = prec == TWOLDG_F64 ? "f64" : prec == TWOLDG_F32 ? "f32" : "f32c";
        std::ostringstream rep;
        int rc = TWOLDG_OK;
        for (auto& gp : groups) {
            Group& g = *gp;
            if (g.full) continue;
            const int nit = (int)g.items.size();
            int size_class = 0;
            while ((1 << size_class) <= nit) ++size_class;
            char keyb[128];
            std::snprintf(keyb, sizeof keyb, "%s d%d p%d e%d %s n%d", pname, g.D, g.P, g.E,
                          g.metric ? "diag" : "flat", size_class);
            const std::string key = keyb;
            auto kn = known.find(key);
            if (kn != known.end()) {
                g.ops->set_launch(kn->second, g.E, !g.metric);
                rep << lines[key] << "\n";
                continue;
            }
            Launch cand[32];
            const int nc = g.ops->launch_candidates(g.E, !g.metric, cand, 32);
            float best = INFINITY;
            Launch bl{0, 0, 0};
            auto run3 = [&]() -> cudaError_t {
                int in = 0;
                for (int s = 1; s <= 3; ++s) {
                    StagePtrs sp = stage_ptrs(g, u, in);
                    cudaError_t e = g.ops->stage((const BlockItem*)g.d_items.p, nit, g.E, s, g.truncate, sp, 0, stream);
                    if (e != cudaSuccess) return e;
                    in = 1 - in;
                }
                return cudaSuccess;
            };
            for (int c = 0; c < nc; ++c) {
                g.ops->set_launch(cand[c], g.E, !g.metric);
                if (run3() != cudaSuccess || run3() != cudaSuccess) { cudaGetLastError(); continue; }
                const int reps = 5;
                cudaEventRecord(e0, stream);
                bool ok = true;
                for (int q = 0; q < reps && ok; ++q) ok = run3() == cudaSuccess;
                cudaEventRecord(e1, stream);
                cudaError_t e = cudaEventSynchronize(e1);
                if (e != cudaSuccess) { rc = cuda_fail(e, "autotune"); break; }
                if (!ok) { cudaGetLastError(); continue; }
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                ms /= reps * 3;
                if (ms < best) { best = ms; bl = cand[c]; }
            }
            if (rc) break;
            g.ops->set_launch(bl, g.E, !g.metric);
            char body[256];
            std::snprintf(body, sizeof body, "\"%s\": {\"kernel\": %d, \"threads\": %d, \"waves\": %d, \"us\": %.2f}",
                          key.c_str(), bl.kernel, bl.threads, bl.waves, (double)best * 1e3);
            lines[key] = body;
            rep << body << "\n";
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc) return rc;
        drop_graphs();
        if (cache) {
            std::ofstream out(cache, std::ios::trunc);
            if (!out) return fail(TWOLDG_EINVAL, std::string("cannot write the autotuner cache ") + cache);
            out << "{\n";
            size_t i = 0;
            for (auto& kv : lines) out << "  " << kv.second << (++i < lines.size() ? ",\n" : "\n");
            out << "}\n";
        }
        report = rep.str();
        return TWOLDG_OK;
    }

    int rk4(void* u, const double* dts, int nsteps, double t0 = 0.0) {
        if (!u) return fail(TWOLDG_EINVAL, "u is NULL");
        if (nsteps < 0) return fail(TWOLDG_EINVAL, "nsteps is negative");
        bool changed = false;
        for (int k = 0; k < nproblems; ++k) {
            if (!(dts[k] > 0) || !std::isfinite(dts[k])) return fail(TWOLDG_EINVAL, "dt must be positive and finite");
            if (dts[k] != h_dts[k]) changed = true;
        }
        if (changed) {
            std::copy(dts, dts + nproblems, h_dts.begin());
            for (int k = 0; k < nproblems; ++k) {
                const double c[4] = {dts[k] / 6, dts[k] / 3, dts[k] / 2, dts[k]};
                for (int q = 0; q < 4; ++q) {
                    unsigned char* dst = h_rk.data() + (k * 4 + q) * wsize;
                    if (wsize == 8) std::memcpy(dst, &c[q], 8);
                    else { float f = (float)c[q]; std::memcpy(dst, &f, 4); }
                }
            }
            CK(cudaMemcpyAsync(d_rk.p, h_rk.data(), h_rk.size(), cudaMemcpyHostToDevice, stream));
            CK(cudaStreamSynchronize(stream));
        }
        if (prec == TWOLDG_F32C && comp_u != u) {
            CK(cudaMemsetAsync(comp.p, 0, (size_t)total_words * wsize, stream));
            comp_u = u;
        }
        if (any_full()) {
            int rr = nsteps > 0 ? boundary_window(t0, dts[0], nsteps) : TWOLDG_OK;
            if (!rr) rr = set_time(t0, dts);
            if (rr) return rr;
        }
        if (nsteps == 0) return TWOLDG_OK;
        int r = export_all(u);
        if (!r) r = prime_cf();
        if (r) return r;
        const int chunk = std::min(nsteps, kChunk);
        cudaGraphExec_t gexec = nullptr;
        r = step_graph(u, chunk, &gexec);
        if (r) return r;
        for (int i = 0; i + chunk <= nsteps; i += chunk) CK(cudaGraphLaunch(gexec, stream));
        if (nsteps % chunk) {
            r = step_graph(u, nsteps % chunk, &gexec);
            if (r) return r;
            CK(cudaGraphLaunch(gexec, stream));
        }
        CK(cudaGetLastError());
        return TWOLDG_OK;
    }

    // The graph of `steps` steps on state u, captured at its first use.
    int step_graph(void* u, int steps, cudaGraphExec_t* out) {
        for (size_t i = 0; i < graphs.size(); ++i)
            if (graphs[i].u == u && graphs[i].steps == steps) {
                *out = graphs[i].exec;
                std::rotate(graphs.begin(), graphs.begin() + i, graphs.begin() + i + 1);
                return TWOLDG_OK;
            }
        cudaGraph_t graph;
        cudaGraphExec_t gexec = nullptr;
        CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        int r = enqueue_step(u, steps);
        cudaError_t e = cudaStreamEndCapture(stream, &graph);
        if (r) { if (e == cudaSuccess) cudaGraphDestroy(graph); return r; }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        if ((int)graphs.size() == kGraphs) {
            cudaGraphExecDestroy(graphs.back().exec);
            graphs.pop_back();
        }
        graphs.insert(graphs.begin(), StepGraph{u, steps, gexec});
        *out = gexec;
        return TWOLDG_OK;
    }
};

namespace twoldg {
void fm_advance_time_launch(double* tinfo, int nproblems, cudaStream_t s);
}

void twoldg_runner::fm_advance_time(cudaStream_t s) { fm_advance_time_launch((double*)d_tinfo.p, nproblems, s); }

struct twoldg_problem : twoldg_runner {
    int D = 0, P = 0, E = 0;
    int truncate = 1;
};

struct twoldg_batch : twoldg_runner {};

namespace twoldg {
// A problem's shape, precision (0: float64 fields, 1: float32), block count and
// stream, for the transfer's plans (transfer.cpp).
bool problem_shape(twoldg_problem* p, int* D, int* P, int* E, int* prec, int64_t* nblocks, cudaStream_t* stream) {
    if (!p) return false;
    *D = p->D;
    *P = p->P;
    *E = p->E;
    *prec = p->prec == TWOLDG_F64 ? 0 : 1;
    int64_t NN = 1;
    for (int d = 0; d < p->D; ++d) NN *= (int64_t)p->E * (p->P + 1);
    *nblocks = p->total_words / (2 * NN);
    *stream = p->stream;
    return true;
}
}  // namespace twoldg

extern "C" {

const char* twoldg_last_error(void) { return g_err.c_str(); }
const char* twoldg_version(void) { return "twoldg 0.1 (sm_103a)"; }

int twoldg_element_tables(int32_t order, int32_t precision, const char* name, void* out) {
    if (!name || !out) return fail(TWOLDG_EINVAL, "name and out must not be NULL");
    if (!tables().get(order)) return fail(TWOLDG_EINVAL, "order P must be 1.." + std::to_string(kMaxP));
    auto pickv = [&](auto& t) -> const void* {
        using V = typename std::decay_t<decltype(t.nodes)>;
        static_assert(sizeof(V) > 0, "");
        std::string n(name);
        const auto* v = &t.nodes;
        if (n == "nodes") v = &t.nodes;
        else if (n == "weights") v = &t.weights;
        else if (n == "offsets") v = &t.offsets;
        else if (n == "stencil") v = &t.stencil;
        else if (n == "truncate") v = &t.truncate;
        else if (n == "topmode") v = &t.topmode;
        else if (n == "topdual") v = &t.topdual;
        else if (n == "duals") v = &t.duals;
        else if (n == "prolong") v = &t.prolong;
        else if (n == "restrict") v = &t.restrict_;
        else return nullptr;
        std::memcpy(out, v->data(), v->size() * sizeof((*v)[0]));
        return out;
    };
    const void* r = precision == 0 ? pickv(tables().t64[order]) : pickv(tables().t32[order]);
    if (!r) return fail(TWOLDG_EINVAL, std::string("unknown table ") + name);
    return TWOLDG_OK;
}

int twoldg_problem_create(const twoldg_desc* desc, twoldg_problem** out) {
    if (!desc || !out) return fail(TWOLDG_EINVAL, "desc and out must not be NULL");
    *out = nullptr;
    std::unique_ptr<twoldg_problem> p(new twoldg_problem());
    int r = p->setup(1, desc);
    if (r) return r;
    p->D = desc->dim;
    p->P = desc->order;
    p->E = desc->elems;
    p->truncate = desc->truncate ? 1 : 0;
    *out = p.release();
    return TWOLDG_OK;
}

int twoldg_problem_destroy(twoldg_problem* p) {
    if (p) {
        cudaStreamSynchronize(p->stream);
        delete p;
    }
    return TWOLDG_OK;
}

int twoldg_state_words(const twoldg_problem* p, int64_t* words) {
    if (!p || !words) return fail(TWOLDG_EINVAL, "NULL argument");
    *words = p->total_words;
    return TWOLDG_OK;
}

int twoldg_min_spacing(const twoldg_problem* p, double* h) {
    if (!p || !h) return fail(TWOLDG_EINVAL, "NULL argument");
    *h = p->hmin[0];
    return TWOLDG_OK;
}

int twoldg_rhs(twoldg_problem* p, void* du, const void* u, double t) {
    if (!p || !du || !u) return fail(TWOLDG_EINVAL, "NULL argument");
    if (du == u) return fail(TWOLDG_EINVAL, "du and u must not alias: the right-hand side never writes u");
    int r = p->export_all(u);
    if (r) return r;
    Group& g = *p->groups[0];
    if (g.full) {
        r = p->boundary_window(t, 0.0, 0);
        if (!r) r = p->set_time(t, nullptr);
        if (r) return r;
        FmPtrs fp = p->fptrs(g, const_cast<void*>(u), 0);
        fp.du = du;
        r = p->fm_dense(g, fp, 1, p->stream);
        if (r) return r;
        CK(g.ops->fm_gradient((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, 0, fp, p->stream));
        r = p->fm_dense(g, fp, 3, p->stream);
        if (r) return r;
        CK(g.ops->fm_stage((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, 0, 0, fp, p->stream));
        return TWOLDG_OK;
    }
    r = p->cf_all(g, 0);
    if (r) return r;
    StagePtrs s = p->ptrs(g, const_cast<void*>(u), 0);
    s.du = du;
    CK(g.ops->stage((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, 0, 0, s, 0, p->stream));
    return TWOLDG_OK;
}

int twoldg_truncate(twoldg_problem* p, void* u) {
    if (!p || !u) return fail(TWOLDG_EINVAL, "NULL argument");
    Group& g = *p->groups[0];
    if (!g.truncate) return TWOLDG_OK;
    if (g.full) {
        FmPtrs fp = p->fptrs(g, u, 0);
        CK(g.ops->fm_truncate((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, fp, p->stream));
        return TWOLDG_OK;
    }
    CK(g.ops->truncate((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, u,
                       g.metric ? g.d_trm.p : nullptr, g.metric ? g.d_trd.p : nullptr, p->stream));
    return TWOLDG_OK;
}

int twoldg_rk4_step(twoldg_problem* p, void* u, double t, double dt, int32_t nsteps) {
    if (!p) return fail(TWOLDG_EINVAL, "NULL problem");
    return p->rk4(u, &dt, nsteps, t);
}

int twoldg_reset_compensation(twoldg_problem* p) {
    if (!p) return fail(TWOLDG_EINVAL, "NULL problem");
    if (p->comp.p) CK(cudaMemsetAsync(p->comp.p, 0, (size_t)p->total_words * p->wsize, p->stream));
    return TWOLDG_OK;
}

int twoldg_energy(twoldg_problem* p, const void* u, double t, double* energy) {
    if (!p || !u || !energy) return fail(TWOLDG_EINVAL, "NULL argument");
    int r = p->export_all(u);
    if (r) return r;
    Group& g = *p->groups[0];
    if (g.full) {
        r = p->boundary_window(t, 0.0, 0);
        if (!r) r = p->set_time(t, nullptr);
        if (r) return r;
        FmPtrs fp = p->fptrs(g, const_cast<void*>(u), 0);
        r = p->fm_dense(g, fp, 1, p->stream);
        if (r) return r;
        CK(g.ops->fm_gradient((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, 5, fp, p->stream));
        CK(g.ops->fm_energy((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, fp, p->stream));
    } else {
        r = p->cf_all(g, 0);
        if (r) return r;
        StagePtrs s = p->ptrs(g, const_cast<void*>(u), 0);
        CK(g.ops->energy((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, s, p->stream));
    }
    std::vector<double> part(g.items.size());
    CK(cudaMemcpyAsync(part.data(), g.d_part.p, part.size() * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    double e = 0;
    for (double x : part) e += x;
    *energy = e;
    return TWOLDG_OK;
}

int twoldg_norm(twoldg_problem* p, const void* u, const void* ref, int32_t pnorm, int32_t vars_mask, double* out) {
    if (!p || !u || !out) return fail(TWOLDG_EINVAL, "NULL argument");
    if (pnorm < 0) return fail(TWOLDG_EINVAL, "the norm takes an integer p >= 1, or 0 for the largest value");
    if (vars_mask < 1 || vars_mask > 3) return fail(TWOLDG_EINVAL, "vars_mask must select u (1), v (2) or both (3)");
    Group& g = *p->groups[0];
    CK(g.ops->norm((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, u, ref, pnorm, vars_mask,
                   (double*)g.d_part.p, (double*)g.d_part2.p, g.metric ? g.d_coef.p : nullptr,
                   g.full ? 1 + g.D * g.D : 1 + g.D, p->stream));
    std::vector<double> num(g.items.size()), vol(g.items.size());
    CK(cudaMemcpyAsync(num.data(), g.d_part.p, num.size() * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaMemcpyAsync(vol.data(), g.d_part2.p, vol.size() * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    if (pnorm == 0) {
        double m = 0;
        for (double x : num) m = std::fmax(m, x);
        *out = m;
        return TWOLDG_OK;
    }
    double a = 0, v = 0;
    for (size_t i = 0; i < num.size(); ++i) { a += num[i]; v += vol[i]; }
    *out = v == 0 ? 0.0 : std::pow(a / v, 1.0 / pnorm);
    return TWOLDG_OK;
}

static int indicator(twoldg_problem* p, const void* u, int var, int nq, const int* modes, const double* weights,
                     const double* pows, double post, void* tau) {
    if (!p || !u || !tau) return fail(TWOLDG_EINVAL, "NULL argument");
    if (var != 1 && var != 2) return fail(TWOLDG_EINVAL, "var must be 1 (u) or 2 (v)");
    Group& g = *p->groups[0];
    CK(g.ops->maxabs((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, u, var - 1, (double*)g.d_part.p,
                     p->stream));
    std::vector<double> part(g.items.size());
    CK(cudaMemcpyAsync(part.data(), g.d_part.p, part.size() * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    double peak = 0;
    for (double x : part) peak = std::fmax(peak, x);
    // A field that vanishes everywhere scores zero rather than NaN (src/refinement.jl:88-90).
    double scale = peak == 0 ? 0.0 : 1.0 / peak;
    std::vector<double> w(nq);
    for (int q = 0; q < nq; ++q) w[q] = weights[q] * scale;
    CK(g.ops->modes((const BlockItem*)g.d_items.p, (int)g.items.size(), g.E, u, var - 1, nq, modes, w.data(), pows,
                    post, tau, p->stream));
    return TWOLDG_OK;
}

static double doublefactorial(int m) {
    double r = 1;
    for (int k = 1; k <= 2 * m - 1; k += 2) r *= k;
    return r;
}

int twoldg_modal_indicator(twoldg_problem* p, const void* u, int32_t var, int32_t mode, void* tau_dev) {
    if (!p) return fail(TWOLDG_EINVAL, "NULL problem");
    // check_mode: mode 0 says nothing about resolution; the truncated scheme's last moving mode is P-1
    if (mode < 1 || mode > p->P)
        return fail(TWOLDG_EINVAL, "mode = " + std::to_string(mode) + " must be one of 1 .. P = " + std::to_string(p->P));
    std::vector<int> modes(mode);
    std::vector<double> weights(mode), pows(mode);
    for (int m = 1; m <= mode; ++m) {
        modes[m - 1] = m;
        weights[m - 1] = doublefactorial(m);
        pows[m - 1] = (double)mode / m;
    }
    return indicator(p, u, var, mode, modes.data(), weights.data(), pows.data(), 1.0 / doublefactorial(mode), tau_dev);
}

int twoldg_mode_amplitude(twoldg_problem* p, const void* u, int32_t var, int32_t mode, void* tau_dev) {
    if (!p) return fail(TWOLDG_EINVAL, "NULL problem");
    if (mode < 0 || mode > p->P)
        return fail(TWOLDG_EINVAL, "mode = " + std::to_string(mode) + " is not a Legendre mode of an element of order P = " +
                                       std::to_string(p->P));
    int m = mode;
    double w = 1, pw = 1;
    return indicator(p, u, var, 1, &m, &w, &pw, 1.0, tau_dev);
}

int twoldg_profile_step(twoldg_problem* p, void* u, double dt, float* stage_ms) {
    if (!p || !u || !stage_ms) return fail(TWOLDG_EINVAL, "NULL argument");
    double dts = dt;
    // make sure dt is on the device (rk4 with zero steps uploads it)
    int r = p->any_full() ? p->boundary_window(0.0, dt, 1) : TWOLDG_OK;
    if (!r) r = p->rk4(u, &dts, 0);
    if (r) return r;
    r = p->export_all(u);
    if (!r) r = p->prime_cf();
    if (r) return r;
    cudaEvent_t ev[5];
    for (int i = 0; i < 5; ++i) CK(cudaEventCreate(&ev[i]));
    CK(cudaEventRecord(ev[0], p->stream));
    for (int s = 1; s <= 4; ++s) {
        for (auto& gp : p->groups) {
            r = p->enqueue_stage(*gp, u, s, (s - 1) & 1, p->stream);
            if (r) return r;
        }
        CK(cudaEventRecord(ev[s], p->stream));
    }
    if (p->any_full()) {
        p->fm_advance_time(p->stream);
        CK(cudaGetLastError());
    }
    CK(cudaEventSynchronize(ev[4]));
    for (int s = 0; s < 4; ++s) CK(cudaEventElapsedTime(&stage_ms[s], ev[s], ev[s + 1]));
    for (int i = 0; i < 5; ++i) cudaEventDestroy(ev[i]);
    return TWOLDG_OK;
}

void* twoldg_stream(twoldg_problem* p) { return p ? (void*)p->stream : nullptr; }

int twoldg_profile_kernels(twoldg_problem* p, const void* u, float* ms, int32_t n) {
    if (!p || !u || !ms) return fail(TWOLDG_EINVAL, "NULL argument");
    if (n < 7) return fail(TWOLDG_EINVAL, "ms must hold 7 durations");
    Group& g = *p->groups[0];
    if (g.full) return fail(TWOLDG_EUNSUP, "the kernels timed here are the flat and diagonal ones");
    const BlockItem* items = (const BlockItem*)g.d_items.p;
    const int nitems = (int)g.items.size();
    // the truncation acts on a copy in the stage buffer, so u is not changed
    CK(cudaMemcpyAsync(p->y.p, u, (size_t)p->total_words * p->wsize, cudaMemcpyDeviceToDevice, p->stream));
    const int mode = p->P > 1 ? p->P - 1 : 1;
    std::vector<int> modes(mode);
    std::vector<double> w(mode), pw(mode);
    for (int m = 1; m <= mode; ++m) {
        modes[m - 1] = m;
        w[m - 1] = doublefactorial(m);
        pw[m - 1] = (double)mode / m;
    }
    cudaEvent_t ev[8];
    for (int i = 0; i < 8; ++i) CK(cudaEventCreate(&ev[i]));
    int r = TWOLDG_OK;
    auto step = [&](int i, cudaError_t e) {
        if (e != cudaSuccess && r == TWOLDG_OK) r = cuda_fail(e, "profile_kernels");
        cudaEventRecord(ev[i], p->stream);
    };
    cudaEventRecord(ev[0], p->stream);
    r = p->export_all(u);
    cudaEventRecord(ev[1], p->stream);
    if (!r) r = p->cf_all(g, 0);
    cudaEventRecord(ev[2], p->stream);
    StagePtrs sp = p->ptrs(g, const_cast<void*>(u), 0);
    step(3, g.ops->energy(items, nitems, g.E, sp, p->stream));
    step(4, g.ops->norm(items, nitems, g.E, u, p->y.p, 2, 3, (double*)g.d_part.p, (double*)g.d_part2.p,
                        g.metric ? g.d_coef.p : nullptr, 1 + g.D, p->stream));
    step(5, g.ops->maxabs(items, nitems, g.E, u, 0, (double*)g.d_part.p, p->stream));
    // the indicator's tau goes to the second accumulator half of the stage buffer
    step(6, g.ops->modes(items, nitems, g.E, u, 0, mode, modes.data(), w.data(), pw.data(),
                         1.0 / doublefactorial(mode), p->acc.p, p->stream));
    step(7, g.ops->truncate(items, nitems, g.E, p->y.p, g.metric ? g.d_trm.p : nullptr,
                            g.metric ? g.d_trd.p : nullptr, p->stream));
    cudaError_t e = cudaEventSynchronize(ev[7]);
    if (e != cudaSuccess && r == TWOLDG_OK) r = cuda_fail(e, "cudaEventSynchronize");
    for (int i = 0; i < 7 && r == TWOLDG_OK; ++i) {
        e = cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaEventElapsedTime");
    }
    for (int i = 0; i < 8; ++i) cudaEventDestroy(ev[i]);
    return r;
}

int twoldg_boundary_faces(twoldg_problem* p, int32_t* slots, int32_t* n) {
    if (!p || !n) return fail(TWOLDG_EINVAL, "NULL argument");
    Group& g = *p->groups[0];
    if (!g.full || g.boundary != 2)
        return fail(TWOLDG_EINVAL, "the problem does not take the caller's Dirichlet values (boundary 2)");
    if (slots)
        for (size_t q = 0; q < g.bidx.size(); ++q)
            if (g.bidx[q] >= 0) slots[g.bidx[q]] = (int32_t)q;
    *n = g.nbf;
    return TWOLDG_OK;
}

int twoldg_set_boundary_values(twoldg_problem* p, const double* values, int32_t nlevels, double t0, double dt) {
    if (!p || !values) return fail(TWOLDG_EINVAL, "NULL argument");
    Group& g = *p->groups[0];
    if (!g.full || g.boundary != 2)
        return fail(TWOLDG_EINVAL, "the problem does not take the caller's Dirichlet values (boundary 2)");
    if (nlevels < 1) return fail(TWOLDG_EINVAL, "nlevels must be at least 1");
    if (!(dt > 0) || !std::isfinite(dt) || !std::isfinite(t0))
        return fail(TWOLDG_EINVAL, "t0 must be finite and dt positive and finite");
    g.h_btab.values = values;
    g.h_btab.nlevels = nlevels;
    g.h_btab.nbf = g.nbf;
    g.h_btab.t0 = t0;
    g.h_btab.inv_half = 2.0 / dt;
    g.btab_dt = dt;
    g.btab_set = true;
    // ordered before every later launch on the problem's stream
    CK(cudaMemcpyAsync(g.d_btab.p, &g.h_btab, sizeof(BoundaryTable), cudaMemcpyHostToDevice, p->stream));
    return TWOLDG_OK;
}

int twoldg_synchronize(twoldg_problem* p) {
    if (!p) return fail(TWOLDG_EINVAL, "NULL problem");
    CK(cudaStreamSynchronize(p->stream));
    return TWOLDG_OK;
}

int twoldg_gather(twoldg_problem* p, const void* u, int32_t var, int64_t npoints, int32_t nper,
                  const int64_t* index, const void* weights, void* out) {
    if (!p || !u || (npoints > 0 && (!index || !weights || !out))) return fail(TWOLDG_EINVAL, "NULL argument");
    if (var != 1 && var != 2) return fail(TWOLDG_EINVAL, "var must be 1 (u) or 2 (v)");
    if (npoints < 0 || nper < 1) return fail(TWOLDG_EINVAL, "npoints must be >= 0 and nper >= 1");
    if (p->groups.empty()) return fail(TWOLDG_EINVAL, "the problem has no blocks");
    Group& g = *p->groups[0];
    CK(g.ops->gather(u, (var - 1) * g.NN, npoints, nper, index, weights, out, p->stream));
    return TWOLDG_OK;
}

int twoldg_transfer(const twoldg_desc* from, const void* u_from, const twoldg_desc* to, void* u_to, void* stream) {
    if (!from || !to || !u_from || !u_to) return fail(TWOLDG_EINVAL, "NULL argument");
    if (from->dim != to->dim || from->order != to->order || from->elems != to->elems ||
        from->precision != to->precision)
        return fail(TWOLDG_EINVAL, "the two forests must share dim, order, elems and precision");
    const int D = from->dim, P = from->order, E = from->elems;
    if (D < 1 || D > 3) return fail(TWOLDG_EINVAL, "dim must be 1, 2 or 3");
    if (E < 2 || E % 2) return fail(TWOLDG_EINVAL, "E must be even: a child block covers half its parent's elements");
    for (int k = 0; k < D; ++k)
        if (from->roots[k] != to->roots[k] || from->lo[k] != to->lo[k] || from->hi[k] != to->hi[k])
            return fail(TWOLDG_EINVAL, "the two forests must share roots and extents");
    if (from->coef || to->coef || from->face_nb || to->face_nb)
        return fail(TWOLDG_EUNSUP, "the transfer moves the state of flat brick forests");
    if (!tables().get(P)) return fail(TWOLDG_EUNSUP, "no kernels for P = " + std::to_string(P) + " (built: 1..6)");
    const int prec = from->precision;
    const int64_t N = (int64_t)E * (P + 1);
    int64_t NN = 1;
    for (int k = 0; k < D; ++k) NN *= N;
    // the old leaves by (level, corner)
    std::map<std::vector<int64_t>, int> old;
    for (int b = 0; b < from->nblocks; ++b) {
        std::vector<int64_t> key(1 + D);
        key[0] = from->level[b];
        for (int k = 0; k < D; ++k) key[1 + k] = from->corner[(int64_t)b * D + k];
        old[key] = b;
    }
    std::vector<TransferItem> items(to->nblocks);
    for (int b = 0; b < to->nblocks; ++b) {
        TransferItem& it = items[b];
        it.dst = (int64_t)b * 2 * NN;
        std::vector<int64_t> key(1 + D);
        key[0] = to->level[b];
        for (int k = 0; k < D; ++k) key[1 + k] = to->corner[(int64_t)b * D + k];
        auto same = old.find(key);
        if (same != old.end()) {
            it.mode = 0;
            it.src[0] = (int64_t)same->second * 2 * NN;
            continue;
        }
        if (key[0] > 0) {
            std::vector<int64_t> pk(key);
            pk[0] -= 1;
            int sub = 0;
            for (int k = 0; k < D; ++k) {
                sub |= (int)(key[1 + k] & 1) << k;
                pk[1 + k] = key[1 + k] >> 1;
            }
            auto par = old.find(pk);
            if (par != old.end()) {
                it.mode = 1;
                it.sub = sub;
                it.src[0] = (int64_t)par->second * 2 * NN;
                continue;
            }
        }
        bool all = true;
        for (int q = 0; q < (1 << D) && all; ++q) {
            std::vector<int64_t> ck(key);
            ck[0] += 1;
            for (int k = 0; k < D; ++k) ck[1 + k] = 2 * key[1 + k] + ((q >> k) & 1);
            auto ch = old.find(ck);
            if (ch == old.end()) all = false;
            else it.src[q] = (int64_t)ch->second * 2 * NN;
        }
        if (!all)
            return fail(TWOLDG_EINVAL, "block " + std::to_string(b) + " of the new forest is neither a leaf of the old "
                                       "one, nor a child of one, nor the parent of 2^D of them");
        it.mode = 2;
    }
    std::unique_ptr<Ops> ops;
    if (D == 1) ops.reset(make_ops_d1(prec, P, tables().t64[P], tables().t32[P]));
    if (D == 2) ops.reset(make_ops_d2(prec, P, tables().t64[P], tables().t32[P]));
    if (D == 3) ops.reset(make_ops_d3(prec, P, tables().t64[P], tables().t32[P]));
    if (!ops) return fail(TWOLDG_EINVAL, "precision must be TWOLDG_F64, TWOLDG_F32 or TWOLDG_F32C");
    cudaStream_t st = (cudaStream_t)stream;
    DevBuf d_items;
    CK(d_items.alloc(items.size() * sizeof(TransferItem)));
    CK(cudaMemcpyAsync(d_items.p, items.data(), items.size() * sizeof(TransferItem), cudaMemcpyHostToDevice, st));
    CK(ops->transfer((const TransferItem*)d_items.p, (int)items.size(), E, u_from, u_to, st));
    CK(cudaStreamSynchronize(st));
    return TWOLDG_OK;
}

int twoldg_batch_create(int32_t n, const twoldg_desc* descs, twoldg_batch** out) {
    if (!out) return fail(TWOLDG_EINVAL, "out must not be NULL");
    *out = nullptr;
    std::unique_ptr<twoldg_batch> b(new twoldg_batch());
    int r = b->setup(n, descs);
    if (r) return r;
    *out = b.release();
    return TWOLDG_OK;
}

int twoldg_batch_destroy(twoldg_batch* b) {
    if (b) {
        cudaStreamSynchronize(b->stream);
        delete b;
    }
    return TWOLDG_OK;
}

int twoldg_batch_offsets(const twoldg_batch* b, int64_t* offsets, int64_t* total_words) {
    if (!b) return fail(TWOLDG_EINVAL, "NULL batch");
    if (offsets) std::copy(b->offsets.begin(), b->offsets.end(), offsets);
    if (total_words) *total_words = b->total_words;
    return TWOLDG_OK;
}

int twoldg_batch_rk4_step(twoldg_batch* b, void* u, const double* dt, int32_t nsteps) {
    if (!b || !dt) return fail(TWOLDG_EINVAL, "NULL argument");
    return b->rk4(u, dt, nsteps);
}

static int tune_report(const std::string& rep, char* report, size_t report_len) {
    if (report && report_len) {
        const size_t n = std::min(rep.size(), report_len - 1);
        std::memcpy(report, rep.data(), n);
        report[n] = 0;
    }
    return TWOLDG_OK;
}

int twoldg_autotune(twoldg_problem* p, void* u, double dt, const char* cache, char* report, size_t report_len) {
    if (!p || !u) return fail(TWOLDG_EINVAL, "NULL argument");
    std::string rep;
    int r = p->autotune(u, &dt, cache, rep);
    if (r) return r;
    return tune_report(rep, report, report_len);
}

int twoldg_batch_autotune(twoldg_batch* b, void* u, const double* dt, const char* cache, char* report,
                          size_t report_len) {
    if (!b || !u || !dt) return fail(TWOLDG_EINVAL, "NULL argument");
    std::string rep;
    int r = b->autotune(u, dt, cache, rep);
    if (r) return r;
    return tune_report(rep, report, report_len);
}

void* twoldg_batch_stream(twoldg_batch* b) { return b ? (void*)b->stream : nullptr; }

int twoldg_batch_synchronize(twoldg_batch* b) {
    if (!b) return fail(TWOLDG_EINVAL, "NULL batch");
    CK(cudaStreamSynchronize(b->stream));
    return TWOLDG_OK;
}

}  // extern "C"
