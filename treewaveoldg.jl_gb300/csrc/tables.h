// Reference-element tables of order P, built in double-double and rounded
// once to the run's type.
#pragma once
#include <vector>

namespace twoldg {

constexpr int kMaxP = 8;

// All tables of one element order, in row-major layout, as the reference's
// Element{T,P1,PW} holds them (src/element.jl:58-67), plus the tangential
// coarse-fine operators of the element-local ghost fill.
template <typename T>
struct ElementTables {
    int P = 0;
    std::vector<T> nodes;     // P+1
    std::vector<T> weights;   // P+1
    std::vector<T> offsets;   // P+1
    std::vector<T> stencil;   // (P+1) x (P+3), columns are nodes -1 .. P+1
    std::vector<T> truncate;  // (P+1) x (P+1)
    std::vector<T> topmode;   // P+1
    std::vector<T> topdual;   // P+1
    std::vector<T> duals;     // (P+1) x (P+1), row k = dual of Legendre mode k
    std::vector<T> prolong;   // 2(P+1) x (P+1): coarse element polynomial at fine nodes
    std::vector<T> restrict_; // (P+1) x 2(P+1): M_c^-1 I^T M_f
};

// Builds the tables of order P (1 <= P <= kMaxP); returns false otherwise.
bool build_tables(int P, ElementTables<double>& f64, ElementTables<float>& f32);

// One Gauss-Legendre rule of the particle-grid transfer for elements of order
// P: its q nodes and weights on [-1, 1], the Lagrange table
// lagrange[k][i] = phi_i(x_k) (q x (P+1)) and the contraction
// contract[i][k] = w_k phi_i(x_k) / w^_i ((P+1) x q), the one-dimensional
// factor of the projection (P S)_n = (1/w_n) int S phi_n.
template <typename T>
struct RuleTables {
    std::vector<T> nodes, weights, lagrange, contract;
};

constexpr int kMaxRule = 256;

// The q-point rule's tables for order P (1 <= q <= kMaxRule); false otherwise.
bool build_rule(int P, int q, RuleTables<double>& f64, RuleTables<float>& f32);

// bary[i] = 1 / prod_{j != i} (x^_i - x^_j) over the element's Gauss-Lobatto
// nodes, so that phi_i(x) = bary[i] prod_{j != i} (x - x^_j) anywhere.
bool build_bary(int P, std::vector<double>& f64, std::vector<float>& f32);

}  // namespace twoldg
