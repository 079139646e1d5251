// Element tables in double-double, rounded once to float64 and float32.
//
// Follows the reference's construction step by step: Gauss-Lobatto nodes by
// Newton's iteration on (1 - x^2) L_P'(x) from the Chebyshev-Gauss-Lobatto
// points, then symmetrised, with endpoints exactly +-1 (src/element.jl:95-114);
// weights 2 / (P(P+1) L_P(x)^2); the wide derivative D = d - (b - F)/2 per h,
// i.e. 2 d_hat / (P+1) with +-P/2 face terms (src/element.jl:138-150); the
// truncation projector and its rank-one form topmode (x) topdual, and the
// Legendre duals (src/element.jl:152-160); node offsets (P+1)(1+x)/2 with the
// faces exactly 0 and P+1 (src/element.jl:164-167). The coarse-fine operators
// are the element-local ghost operators the reference's CODE.md ("The
// coupling") describes: I, the coarse element's polynomial at the fine nodes,
// and R = M_c^-1 I^T M_f.
#include "tables.h"

#include "ddouble.h"

namespace twoldg {

namespace {

std::vector<dd> legendre_all(int P, dd x) {
    std::vector<dd> L(P + 1);
    L[0] = dd(1.0);
    if (P >= 1) L[1] = x;
    for (int k = 2; k <= P; ++k)
        L[k] = (dd(2.0 * k - 1) * x * L[k - 1] - dd(k - 1.0) * L[k - 2]) / dd((double)k);
    return L;
}

void gll(int P, std::vector<dd>& x, std::vector<dd>& w) {
    const double pi = 3.14159265358979323846;
    x.assign(P + 1, dd());
    for (int i = 0; i <= P; ++i) x[i] = dd(-std::cos(pi * i / P));
    x[0] = dd(-1.0);
    x[P] = dd(1.0);
    for (int it = 0; it < 200; ++it) {
        double worst = 0;
        std::vector<dd> delta(P + 1);
        for (int i = 0; i <= P; ++i) {
            std::vector<dd> L = legendre_all(P, x[i]);
            delta[i] = (x[i] * L[P] - L[P - 1]) / (dd((double)(P + 1)) * L[P]);
            worst = std::fmax(worst, std::fabs(delta[i].hi));
        }
        for (int i = 0; i <= P; ++i) x[i] = x[i] - delta[i];
        if (worst <= 1e-33) break;
    }
    std::vector<dd> s(P + 1);
    for (int i = 0; i <= P; ++i) s[i] = (x[i] - x[P - i]) / dd(2.0);
    s[0] = dd(-1.0);
    s[P] = dd(1.0);
    x = s;
    w.assign(P + 1, dd());
    for (int i = 0; i <= P; ++i) {
        dd LP = legendre_all(P, x[i])[P];
        w[i] = dd(2.0) / (dd((double)P * (P + 1)) * LP * LP);
    }
}

dd lagrange(const std::vector<dd>& xi, int j, dd x) {
    dd r(1.0);
    for (size_t k = 0; k < xi.size(); ++k)
        if ((int)k != j) r = r * ((x - xi[k]) / (xi[j] - xi[k]));
    return r;
}

template <typename T>
T round_to(dd v);
template <>
double round_to<double>(dd v) { return to_double(v); }
template <>
float round_to<float>(dd v) { return to_float(v); }

template <typename T>
void fill(ElementTables<T>& t, int P, const std::vector<dd>& nodes, const std::vector<dd>& w,
          const std::vector<dd>& offsets, const std::vector<dd>& W, const std::vector<dd>& Pi,
          const std::vector<dd>& LP, const std::vector<dd>& topdual, const std::vector<dd>& duals,
          const std::vector<dd>& I, const std::vector<dd>& R) {
    auto conv = [](const std::vector<dd>& v) {
        std::vector<T> o(v.size());
        for (size_t i = 0; i < v.size(); ++i) o[i] = round_to<T>(v[i]);
        return o;
    };
    t.P = P;
    t.nodes = conv(nodes);
    t.weights = conv(w);
    t.offsets = conv(offsets);
    t.stencil = conv(W);
    t.truncate = conv(Pi);
    t.topmode = conv(LP);
    t.topdual = conv(topdual);
    t.duals = conv(duals);
    t.prolong = conv(I);
    t.restrict_ = conv(R);
}

}  // namespace

bool build_tables(int P, ElementTables<double>& f64, ElementTables<float>& f32) {
    if (P < 1 || P > kMaxP) return false;
    const int P1 = P + 1, PW = P + 3;
    std::vector<dd> xi, wh;
    gll(P, xi, wh);
    std::vector<std::vector<dd>> Lall(P1);
    std::vector<dd> LP(P1);
    for (int i = 0; i < P1; ++i) {
        Lall[i] = legendre_all(P, xi[i]);
        LP[i] = Lall[i][P];
    }
    std::vector<dd> d(P1 * P1);
    for (int i = 0; i < P1; ++i)
        for (int j = 0; j < P1; ++j)
            if (i != j) d[i * P1 + j] = LP[i] / (LP[j] * (xi[i] - xi[j]));
    d[0] = -(dd((double)P) * dd((double)(P + 1)) / dd(4.0));
    d[P * P1 + P] = dd((double)P) * dd((double)(P + 1)) / dd(4.0);
    std::vector<dd> W(P1 * PW);
    for (int i = 0; i < P1; ++i)
        for (int j = 0; j < P1; ++j) W[i * PW + j + 1] = dd(2.0) * d[i * P1 + j] / dd((double)(P + 1));
    dd face = dd((double)P) / dd(2.0);
    W[0 * PW + 1] += face;
    W[0 * PW + 0] -= face;
    W[P * PW + P1] -= face;
    W[P * PW + P1 + 1] += face;
    dd gamma;
    for (int i = 0; i < P1; ++i) gamma += wh[i] * LP[i] * LP[i];
    std::vector<dd> Pi(P1 * P1);
    for (int i = 0; i < P1; ++i)
        for (int j = 0; j < P1; ++j)
            Pi[i * P1 + j] = dd(i == j ? 1.0 : 0.0) - LP[i] * wh[j] * LP[j] / gamma;
    std::vector<dd> duals(P1 * P1);
    for (int k = 0; k < P1; ++k) {
        dd g;
        for (int i = 0; i < P1; ++i) g += wh[i] * Lall[i][k] * Lall[i][k];
        for (int j = 0; j < P1; ++j) duals[k * P1 + j] = wh[j] * Lall[j][k] / g;
    }
    std::vector<dd> topdual(P1);
    for (int j = 0; j < P1; ++j) {
        topdual[j] = wh[j] * LP[j] / gamma;
        duals[P * P1 + j] = topdual[j];
    }
    std::vector<dd> offsets(P1);
    for (int i = 0; i < P1; ++i) offsets[i] = dd((double)(P + 1)) * (dd(1.0) + xi[i]) / dd(2.0);
    offsets[0] = dd(0.0);
    offsets[P] = dd((double)P1);
    std::vector<dd> I(2 * P1 * P1), R(P1 * 2 * P1);
    for (int half = 0; half < 2; ++half)
        for (int i = 0; i < P1; ++i) {
            dd xc = half == 0 ? (xi[i] - dd(1.0)) / dd(2.0) : (xi[i] + dd(1.0)) / dd(2.0);
            for (int j = 0; j < P1; ++j) I[(half * P1 + i) * P1 + j] = lagrange(xi, j, xc);
        }
    for (int j = 0; j < P1; ++j)
        for (int r = 0; r < 2 * P1; ++r)
            R[j * 2 * P1 + r] = I[r * P1 + j] * wh[r % P1] / (dd(2.0) * wh[j]);
    fill(f64, P, xi, wh, offsets, W, Pi, LP, topdual, duals, I, R);
    fill(f32, P, xi, wh, offsets, W, Pi, LP, topdual, duals, I, R);
    return true;
}

namespace {

// Gauss-Legendre nodes (ascending) and weights of n points
// (src/transfer.jl:44-62): Newton's iteration on L_n from the Chebyshev
// points -cos(pi (4i - 1) / (4n + 2)), then symmetrised so that
// x[i] == -x[n-1-i] holds after any rounding; w = 2 / ((1 - x^2) L_n'(x)^2).
void gauss_legendre(int n, std::vector<dd>& x, std::vector<dd>& w) {
    const double pi = 3.14159265358979323846;
    x.assign(n, dd());
    for (int i = 1; i <= n; ++i) x[i - 1] = dd(-std::cos(pi * (4.0 * i - 1) / (4.0 * n + 2)));
    auto value_and_slope = [&](dd t, dd& L, dd& dL) {
        std::vector<dd> all = legendre_all(n, t);
        L = all[n];
        dL = dd((double)n) * (t * all[n] - all[n - 1]) / (t * t - dd(1.0));
    };
    for (int it = 0; it < 200; ++it) {
        double worst = 0;
        std::vector<dd> delta(n);
        for (int i = 0; i < n; ++i) {
            dd L, dL;
            value_and_slope(x[i], L, dL);
            delta[i] = L / dL;
            worst = std::fmax(worst, std::fabs(delta[i].hi));
        }
        for (int i = 0; i < n; ++i) x[i] = x[i] - delta[i];
        if (worst <= 1e-31) break;
    }
    std::vector<dd> s(n);
    for (int i = 0; i < n; ++i) s[i] = (x[i] - x[n - 1 - i]) / dd(2.0);
    x = s;
    w.assign(n, dd());
    for (int i = 0; i < n; ++i) {
        dd L, dL;
        value_and_slope(x[i], L, dL);
        w[i] = dd(2.0) / ((dd(1.0) - x[i] * x[i]) * dL * dL);
    }
}

std::vector<dd> bary_dd(const std::vector<dd>& xi) {
    const int P1 = (int)xi.size();
    std::vector<dd> b(P1);
    for (int i = 0; i < P1; ++i) {
        dd p(1.0);
        for (int j = 0; j < P1; ++j)
            if (j != i) p = p * (xi[i] - xi[j]);
        b[i] = dd(1.0) / p;
    }
    return b;
}

}  // namespace

bool build_rule(int P, int q, RuleTables<double>& f64, RuleTables<float>& f32) {
    if (P < 1 || P > kMaxP || q < 1 || q > kMaxRule) return false;
    const int P1 = P + 1;
    std::vector<dd> xi, wh, xg, wg;
    gll(P, xi, wh);
    gauss_legendre(q, xg, wg);
    const std::vector<dd> bary = bary_dd(xi);
    std::vector<dd> lag(q * P1), con(P1 * q);
    for (int k = 0; k < q; ++k)
        for (int i = 0; i < P1; ++i) {
            dd phi = bary[i];
            for (int j = 0; j < P1; ++j)
                if (j != i) phi = phi * (xg[k] - xi[j]);
            lag[k * P1 + i] = phi;
            con[i * q + k] = wg[k] * phi / wh[i];
        }
    auto put = [&](auto& t, auto conv) {
        t.nodes.clear(); t.weights.clear(); t.lagrange.clear(); t.contract.clear();
        for (auto& v : xg) t.nodes.push_back(conv(v));
        for (auto& v : wg) t.weights.push_back(conv(v));
        for (auto& v : lag) t.lagrange.push_back(conv(v));
        for (auto& v : con) t.contract.push_back(conv(v));
    };
    put(f64, [](dd v) { return to_double(v); });
    put(f32, [](dd v) { return to_float(v); });
    return true;
}

bool build_bary(int P, std::vector<double>& f64, std::vector<float>& f32) {
    if (P < 1 || P > kMaxP) return false;
    std::vector<dd> xi, wh;
    gll(P, xi, wh);
    f64.clear();
    f32.clear();
    for (auto& v : bary_dd(xi)) {
        f64.push_back(to_double(v));
        f32.push_back(to_float(v));
    }
    return true;
}

}  // namespace twoldg
