// Mesh compiler. The neighbour of a block across a face is found by the
// leaf's integer coordinates, as TreeAMR's forest finds it: a block of the
// same level at the adjacent corner, else its parent-level block (this block
// is then the fine side of a coarse-fine face), else the 2^(D-1) children of
// the adjacent corner that touch the face (this block is the coarse side).
// A face outside the domain is periodic (wrapped) or a reflecting wall.
//
// Ghost semantics follow TreeAMR's element-local operators as the reference
// documents them (CODE.md, "The layout", "Reflecting walls", "The coupling"):
// same level and normal direction always injection of the neighbour's face
// node; walls mirror the block's own face node with u even and d_d u odd;
// across a coarse-fine face the fine ghost is the coarse element's
// polynomial at the fine nodes (I) and the coarse ghost its adjoint
// restriction R = M_c^-1 I^T M_f, tangentially.
#include "mesh.h"

#include <cmath>
#include <map>
#include <sstream>

namespace twoldg {

namespace {

struct Key {
    int level;
    int64_t c[3];
    bool operator<(const Key& o) const {
        if (level != o.level) return level < o.level;
        for (int k = 0; k < 3; ++k)
            if (c[k] != o.c[k]) return c[k] < o.c[k];
        return false;
    }
};

}  // namespace

// The faces of a refined brick patch inside an explicit face table (the
// ball's affine cube): the blocks whose faces are marked TWOLDG_FACE_BRICK
// are leaves of a brick of roots[d] root blocks, at their level and corner,
// and each such face is resolved as build_mesh resolves a brick's faces: a
// same-level neighbour by injection, a coarser one as the fine side of a
// coarse-fine face (I), 2^(D-1) finer ones as its coarse side (R).
static bool brick_faces(const twoldg_desc& d, Mesh& m, std::string& err) {
    std::ostringstream es;
    const int D = d.dim;
    std::map<Key, int> leaves;
    for (int b = 0; b < d.nblocks; ++b) {
        bool in = false;
        for (int f = 0; f < 2 * D; ++f) in = in || d.face_nb[b * 2 * D + f] == TWOLDG_FACE_BRICK;
        if (!in && d.level[b] == 0) continue;
        Key key{d.level[b], {0, 0, 0}};
        if (key.level < 0 || key.level > 20) { es << "block " << b << " has level " << key.level; err = es.str(); return false; }
        for (int k = 0; k < D; ++k) {
            key.c[k] = d.corner[(int64_t)b * D + k];
            const int64_t ext = (int64_t)d.roots[k] << key.level;
            if (key.c[k] < 0 || key.c[k] >= ext) {
                es << "block " << b << " corner[" << k << "] = " << key.c[k] << " is outside the brick [0, " << ext
                   << ")";
                err = es.str();
                return false;
            }
        }
        if (!leaves.emplace(key, b).second) { es << "block " << b << " duplicates another leaf"; err = es.str(); return false; }
    }
    auto slot = [&](int b, int f) { return b * 2 * D + f; };
    for (const auto& kv : leaves) {
        const int b = kv.second, lv = kv.first.level;
        const int64_t* c = kv.first.c;
        BlockItem& it = m.items[b];
        for (int f = 0; f < 2 * D; ++f) {
            if (d.face_nb[b * 2 * D + f] != TWOLDG_FACE_BRICK) continue;
            const int dd = f / 2, side = f % 2;
            Key n{lv, {c[0], c[1], c[2]}};
            n.c[dd] += side ? 1 : -1;
            if (n.c[dd] < 0 || n.c[dd] >= ((int64_t)d.roots[dd] << lv)) {
                es << "block " << b << " face " << f << " is marked a brick face and leaves the brick";
                err = es.str();
                return false;
            }
            auto same = leaves.find(n);
            if (same != leaves.end()) {
                it.nb[f] = slot(same->second, f ^ 1);
                m.nsame++;
                continue;
            }
            if (lv > 0) {
                Key p{lv - 1, {0, 0, 0}};
                for (int k = 0; k < D; ++k) p.c[k] = n.c[k] >> 1;
                auto coarse = leaves.find(p);
                if (coarse != leaves.end()) {
                    CfFace cf{};
                    cf.slot = slot(b, f);
                    cf.kind = 0;
                    cf.src[0] = slot(coarse->second, f ^ 1);
                    int bit = 0;
                    for (int k = 0; k < D; ++k) {
                        if (k == dd) continue;
                        cf.sub |= (int)(c[k] & 1) << bit;
                        ++bit;
                    }
                    cf.side = side;
                    cf.h = m.h[b];
                    m.cf.push_back(cf);
                    it.flags |= 1u << f;
                    continue;
                }
            }
            CfFace cf{};
            cf.slot = slot(b, f);
            cf.kind = 1;
            cf.side = side;
            cf.h = m.h[b];
            for (int q = 0; q < (1 << (D - 1)); ++q) {
                Key ch{lv + 1, {0, 0, 0}};
                int bit = 0;
                for (int k = 0; k < D; ++k) {
                    if (k == dd) ch.c[k] = 2 * n.c[k] + (side ? 0 : 1);
                    else { ch.c[k] = 2 * n.c[k] + ((q >> bit) & 1); ++bit; }
                }
                auto fine = leaves.find(ch);
                if (fine == leaves.end()) {
                    es << "block " << b << " face " << f << " has no neighbour one level apart at most: the brick "
                       << "must be 2:1 balanced across faces and tile its patch";
                    err = es.str();
                    return false;
                }
                cf.src[q] = slot(fine->second, f ^ 1);
            }
            m.cf.push_back(cf);
            it.flags |= 1u << f;
        }
    }
    return true;
}

// An explicit face table (a forest of glued patches): neighbours, faces and
// orientations as given; a face with no neighbour is a boundary face, and the
// faces marked TWOLDG_FACE_BRICK are those of a refined brick patch.
static bool build_explicit(const twoldg_desc& d, Mesh& m, std::string& err) {
    std::ostringstream es;
    const int D = d.dim;
    m.h.resize(d.nblocks);
    m.items.assign(d.nblocks, BlockItem{});
    m.hmin = INFINITY;
    const double cell = (d.hi[0] - d.lo[0]) / d.roots[0];
    bool brick = false;
    for (int b = 0; b < d.nblocks; ++b) {
        if (d.level[b] < 0 || d.level[b] > 20) {
            es << "block " << b << " has level " << d.level[b];
            err = es.str();
            return false;
        }
        m.h[b] = cell / std::ldexp(1.0, d.level[b]) / m.N;
        m.hmin = std::fmin(m.hmin, m.h[b]);
        BlockItem& it = m.items[b];
        it.off = (int64_t)b * 2 * m.NN;
        it.slot = b * 2 * D;
        it.h = m.h[b];
        for (int f = 0; f < 6; ++f) it.nb[f] = -1;
        for (int f = 0; f < 2 * D; ++f) {
            const int nb = d.face_nb[b * 2 * D + f];
            const int code = d.face_code[b * 2 * D + f];
            if (nb == TWOLDG_FACE_BRICK) { brick = true; continue; }
            if (nb < 0) { m.nwall++; continue; }
            const int nf = code & 15, o = (code >> 4) & 7;
            if (nb >= d.nblocks || nf >= 2 * D) {
                es << "block " << b << " face " << f << " names block " << nb << " face " << nf;
                err = es.str();
                return false;
            }
            if (d.face_nb[nb * 2 * D + nf] != b) {
                es << "block " << b << " face " << f << " and block " << nb << " face " << nf
                   << " do not name each other";
                err = es.str();
                return false;
            }
            if (d.level[nb] != d.level[b]) {
                es << "blocks " << b << " and " << nb << " meet across an explicit face at levels " << d.level[b]
                   << " and " << d.level[nb] << ": only a brick patch's faces join blocks of two levels";
                err = es.str();
                return false;
            }
            it.nb[f] = nb * 2 * D + nf;
            it.orient |= (uint32_t)o << (3 * f);
            m.nsame++;
        }
    }
    return !brick || brick_faces(d, m, err);
}

bool build_mesh(const twoldg_desc& d, Mesh& m, std::string& err) {
    std::ostringstream es;
    const int D = d.dim;
    if (D < 1 || D > 3) { es << "dim = " << D << " must be 1, 2 or 3"; err = es.str(); return false; }
    if (d.order < 1) { es << "the element order P must be at least 1, got " << d.order; err = es.str(); return false; }
    if (d.elems < 2 || d.elems % 2) {
        es << "E = " << d.elems << " elements per block must be even and at least 2: a block of a refined forest "
           << "covers half of its parent and has to cover whole elements of it (N must be a multiple of 2(P+1))";
        err = es.str();
        return false;
    }
    if (d.nblocks < 1 || !d.level || !d.corner) { err = "the forest has no blocks (nblocks, level, corner)"; return false; }
    m.D = D;
    m.P = d.order;
    m.E = d.elems;
    m.N = d.elems * (d.order + 1);
    m.nblocks = d.nblocks;
    m.NN = 1;
    for (int k = 0; k < D; ++k) m.NN *= m.N;
    double cell = 0;
    for (int k = 0; k < D; ++k) {
        if (d.roots[k] < 1) { es << "roots[" << k << "] = " << d.roots[k] << " must be positive"; err = es.str(); return false; }
        if (!(d.hi[k] > d.lo[k])) { es << "extent " << k << " is empty"; err = es.str(); return false; }
        if (d.periodic[k] && d.reflecting[k]) {
            es << "dimension " << k << " is both periodic and reflecting"; err = es.str(); return false;
        }
        if (!d.face_nb && !d.periodic[k] && !d.reflecting[k]) {
            es << "dimension " << k << " is neither periodic nor reflecting: the flat problem's outer faces are "
               << "filled by periodicity or by the wall's mirror";
            err = es.str();
            return false;
        }
        double c = (d.hi[k] - d.lo[k]) / d.roots[k];
        if (k == 0) cell = c;
        else if (std::fabs(c - cell) > 1e-12 * cell) {
            err = "root blocks must be cubes: one spacing per block, as the reference's per-block h";
            return false;
        }
    }
    if (d.face_nb) {
        if (!d.face_code) { err = "face_nb needs face_code"; return false; }
        return build_explicit(d, m, err);
    }
    std::map<Key, int> leaves;
    double volume = 0;
    for (int b = 0; b < d.nblocks; ++b) {
        Key key{d.level[b], {0, 0, 0}};
        if (key.level < 0 || key.level > 20) { es << "block " << b << " has level " << key.level; err = es.str(); return false; }
        for (int k = 0; k < D; ++k) {
            key.c[k] = d.corner[(int64_t)b * D + k];
            int64_t ext = (int64_t)d.roots[k] << key.level;
            if (key.c[k] < 0 || key.c[k] >= ext) {
                es << "block " << b << " corner[" << k << "] = " << key.c[k] << " is outside [0, " << ext << ")";
                err = es.str();
                return false;
            }
        }
        if (!leaves.emplace(key, b).second) { es << "block " << b << " duplicates another leaf"; err = es.str(); return false; }
        volume += std::ldexp(1.0, -D * key.level);
    }
    double rootsvol = 1;
    for (int k = 0; k < D; ++k) rootsvol *= d.roots[k];
    if (std::fabs(volume - rootsvol) > 1e-9 * rootsvol) {
        err = "the leaves do not tile the domain (their volume differs from the root blocks')";
        return false;
    }
    m.h.resize(d.nblocks);
    m.items.assign(d.nblocks, BlockItem{});
    m.hmin = INFINITY;
    for (int b = 0; b < d.nblocks; ++b) {
        m.h[b] = cell / std::ldexp(1.0, d.level[b]) / m.N;
        m.hmin = std::fmin(m.hmin, m.h[b]);
        BlockItem& it = m.items[b];
        it.off = (int64_t)b * 2 * m.NN;
        it.slot = b * 2 * D;
        it.flags = 0;
        it.problem = 0;
        it.h = m.h[b];
        for (int f = 0; f < 6; ++f) it.nb[f] = -1;
    }
    auto slot = [&](int b, int f) { return b * 2 * D + f; };
    for (int b = 0; b < d.nblocks; ++b) {
        const int lv = d.level[b];
        int64_t c[3] = {0, 0, 0};
        for (int k = 0; k < D; ++k) c[k] = d.corner[(int64_t)b * D + k];
        BlockItem& it = m.items[b];
        for (int f = 0; f < 2 * D; ++f) {
            const int dd = f / 2, side = f % 2;
            Key n{lv, {c[0], c[1], c[2]}};
            n.c[dd] += side ? 1 : -1;
            const int64_t ext = (int64_t)d.roots[dd] << lv;
            if (n.c[dd] < 0 || n.c[dd] >= ext) {
                if (d.periodic[dd]) {
                    n.c[dd] = (n.c[dd] + ext) % ext;
                } else {
                    it.nb[f] = slot(b, f);
                    it.flags |= 1u << (8 + f);
                    m.nwall++;
                    continue;
                }
            }
            auto same = leaves.find(n);
            if (same != leaves.end()) {
                it.nb[f] = slot(same->second, f ^ 1);
                m.nsame++;
                continue;
            }
            if (lv > 0) {
                Key p{lv - 1, {0, 0, 0}};
                for (int k = 0; k < D; ++k) p.c[k] = n.c[k] >> 1;
                auto coarse = leaves.find(p);
                if (coarse != leaves.end()) {
                    CfFace cf{};
                    cf.slot = slot(b, f);
                    cf.kind = 0;
                    cf.src[0] = slot(coarse->second, f ^ 1);
                    int bit = 0;
                    for (int k = 0; k < D; ++k) {
                        if (k == dd) continue;
                        cf.sub |= (int)(c[k] & 1) << bit;
                        ++bit;
                    }
                    cf.side = side;
                    cf.h = m.h[b];
                    m.cf.push_back(cf);
                    it.flags |= 1u << f;
                    continue;
                }
            }
            CfFace cf{};
            cf.slot = slot(b, f);
            cf.kind = 1;
            cf.side = side;
            cf.h = m.h[b];
            bool ok = true;
            for (int q = 0; q < (1 << (D - 1)); ++q) {
                Key ch{lv + 1, {0, 0, 0}};
                int bit = 0;
                for (int k = 0; k < D; ++k) {
                    if (k == dd) ch.c[k] = 2 * n.c[k] + (side ? 0 : 1);
                    else { ch.c[k] = 2 * n.c[k] + ((q >> bit) & 1); ++bit; }
                }
                auto fine = leaves.find(ch);
                if (fine == leaves.end()) { ok = false; break; }
                cf.src[q] = slot(fine->second, f ^ 1);
            }
            if (!ok) {
                es << "block " << b << " face " << f << " has no neighbour one level apart at most: the forest must "
                   << "be 2:1 balanced across faces and tile the domain";
                err = es.str();
                return false;
            }
            m.cf.push_back(cf);
            it.flags |= 1u << f;
        }
    }
    return true;
}

}  // namespace twoldg
