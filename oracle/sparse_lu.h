// sparse_lu.h -- textbook sparse LU for the CPU oracle (test infrastructure only).
//
// The reference's CPU solver (p3s/cpp/nr_klu.cpp) takes its pivot order from SuiteSparse
// KLU 7.14.1 (klu_analyze / klu_factor, p3s/cpp/ci/build_klu.py:49-50), which is not
// available here. This file implements the published algorithms KLU is built from, in
// this project's own code:
//   * a minimum-degree fill-reducing ordering of the pattern of A + A^T
//     (elimination-graph formulation, ties broken by the lowest vertex index);
//   * the left-looking Gilbert-Peierls LU with threshold partial pivoting that prefers
//     the diagonal (|a_diag| >= tol * max|column| keeps the diagonal), no row scaling;
//   * a refactorization on a frozen pivot order and pattern, and triangular solves.
// It is used (a) behind a KLU-API shim to compile the reference's own nr_klu.cpp for
// validation and (b) by the oracle restatement in nr_oracle.cpp.
#pragma once

#include <vector>

namespace slu {

// Minimum-degree order of the symmetrised pattern of the n x n CSC matrix (Ap, Ai).
// Returns perm with perm[k] = the k-th eliminated row/column.
std::vector<int> min_degree_order(int n, const int* Ap, const int* Ai);

struct Factors {
    int n = 0;
    // LU = A(P, Q). P[k] = original row of pivot k, Q[k] = original column of step k.
    std::vector<int> P, Q, pinv;
    // L: unit lower, CSC by pivot column, row indices in pivot numbering, diagonal NOT
    // stored. U: CSC by pivot column, row indices in pivot numbering, ascending, the
    // diagonal last in each column.
    std::vector<int> Lp, Li, Up, Ui;
    std::vector<double> Lx, Ux;
};

// Factor A (CSC) with column order Q and threshold partial pivoting. Returns false on a
// structurally or numerically singular matrix (zero / non-finite pivot).
bool factor(int n, const int* Ap, const int* Ai, const double* Ax, const std::vector<int>& Q, double tol,
            Factors& F);

// Numeric refactorization on F's pivot order and pattern. Returns false on a zero or
// non-finite pivot (F's values are then undefined).
bool refactor(const int* Ap, const int* Ai, const double* Ax, Factors& F);

// Solve A x = b in place.
void solve(const Factors& F, double* b);

// min |U(k,k)| / max |U(k,k)|, 0 for an empty or non-finite factorization.
double pivot_ratio(const Factors& F);

}  // namespace slu
