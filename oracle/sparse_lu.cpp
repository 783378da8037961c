// sparse_lu.cpp -- see sparse_lu.h. Test infrastructure for the CPU oracle.
//
// Algorithms (published, restated in this project's own code):
//   * minimum degree on the elimination graph (Tinney scheme 2 / Rose), ties by index;
//   * Gilbert & Peierls, "Sparse partial pivoting in time proportional to arithmetic
//     operations" (1988): column-by-column sparse triangular solve over the reach of the
//     column in the graph of L (depth-first search, reverse post-order), threshold
//     partial pivoting with diagonal preference.
#include "sparse_lu.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <set>
#include <utility>

namespace slu {

static inline bool finite_bits(double x) {
    std::uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    return (b & 0x7ff0000000000000ULL) != 0x7ff0000000000000ULL;
}

std::vector<int> min_degree_order(int n, const int* Ap, const int* Ai) {
    std::vector<std::vector<int>> adj(n);
    for (int j = 0; j < n; ++j)
        for (int p = Ap[j]; p < Ap[j + 1]; ++p) {
            const int i = Ai[p];
            if (i == j || i < 0 || i >= n) continue;
            adj[i].push_back(j);
            adj[j].push_back(i);
        }
    std::set<std::pair<int, int>> queue;
    for (int v = 0; v < n; ++v) {
        auto& a = adj[v];
        std::sort(a.begin(), a.end());
        a.erase(std::unique(a.begin(), a.end()), a.end());
        queue.insert({(int)a.size(), v});
    }
    std::vector<int> perm;
    perm.reserve(n);
    std::vector<int> merged;
    while (!queue.empty()) {
        const int v = queue.begin()->second;
        queue.erase(queue.begin());
        perm.push_back(v);
        const std::vector<int> nb = adj[v];
        for (int u : nb) {
            auto& au = adj[u];
            queue.erase({(int)au.size(), u});
            merged.clear();
            std::set_union(au.begin(), au.end(), nb.begin(), nb.end(), std::back_inserter(merged));
            au.clear();
            for (int w : merged)
                if (w != u && w != v) au.push_back(w);
            queue.insert({(int)au.size(), u});
        }
        adj[v].clear();
    }
    return perm;
}

// Reach of column `col` of A in the graph of L (original row numbering), in topological
// order (the order the triangular solve must visit the rows). Returns the rows in `out`.
static void reach(int col, const int* Ap, const int* Ai, const std::vector<int>& pinv, const std::vector<int>& Lp,
                  const std::vector<int>& Li, std::vector<int>& mark, int stamp, std::vector<int>& stack,
                  std::vector<int>& pstack, std::vector<int>& out) {
    out.clear();
    for (int p = Ap[col]; p < Ap[col + 1]; ++p) {
        const int start = Ai[p];
        if (mark[start] == stamp) continue;
        int head = 0;
        stack[0] = start;
        while (head >= 0) {
            const int j = stack[head];
            const int jj = pinv[j];
            if (mark[j] != stamp) {
                mark[j] = stamp;
                pstack[head] = (jj < 0) ? 0 : Lp[jj];
            }
            bool done = true;
            const int pend = (jj < 0) ? 0 : Lp[jj + 1];
            for (int q = pstack[head]; q < pend; ++q) {
                const int i = Li[q];
                if (mark[i] == stamp) continue;
                pstack[head] = q + 1;
                stack[++head] = i;
                done = false;
                break;
            }
            if (done) {
                --head;
                out.push_back(j);  // post-order
            }
        }
    }
    std::reverse(out.begin(), out.end());
}

bool factor(int n, const int* Ap, const int* Ai, const double* Ax, const std::vector<int>& Q, double tol,
            Factors& F) {
    F = Factors();
    F.n = n;
    F.Q = Q;
    F.pinv.assign(n, -1);
    F.Lp.assign(n + 1, 0);
    F.Up.assign(n + 1, 0);
    std::vector<double> x(n, 0.0);
    std::vector<int> mark(n, -1), stack(n + 1), pstack(n + 1), rows;
    std::vector<std::pair<int, double>> ucol;
    for (int k = 0; k < n; ++k) {
        const int col = Q[k];
        reach(col, Ap, Ai, F.pinv, F.Lp, F.Li, mark, k, stack, pstack, rows);
        for (int p = Ap[col]; p < Ap[col + 1]; ++p) x[Ai[p]] += Ax[p];
        for (int j : rows) {
            const int jj = F.pinv[j];
            if (jj < 0) continue;
            const double xj = x[j];
            for (int p = F.Lp[jj]; p < F.Lp[jj + 1]; ++p) x[F.Li[p]] -= F.Lx[p] * xj;
        }
        int ipiv = -1;
        double amax = -1.0;
        for (int i : rows) {
            if (F.pinv[i] >= 0) continue;
            const double a = std::fabs(x[i]);
            if (a > amax) {
                amax = a;
                ipiv = i;
            }
        }
        if (ipiv < 0 || !(amax > 0.0) || !finite_bits(amax)) {
            for (int i : rows) x[i] = 0.0;
            return false;
        }
        if (F.pinv[col] < 0 && mark[col] == k && std::fabs(x[col]) >= tol * amax) ipiv = col;
        const double piv = x[ipiv];
        ucol.clear();
        for (int j : rows) {
            const int jj = F.pinv[j];
            if (jj >= 0) ucol.push_back({jj, x[j]});
        }
        std::sort(ucol.begin(), ucol.end());
        for (auto& e : ucol) {
            F.Ui.push_back(e.first);
            F.Ux.push_back(e.second);
        }
        F.Ui.push_back(k);
        F.Ux.push_back(piv);
        F.Up[k + 1] = (int)F.Ui.size();
        for (int i : rows) {
            if (F.pinv[i] >= 0 || i == ipiv) continue;
            F.Li.push_back(i);
            F.Lx.push_back(x[i] / piv);
        }
        F.Lp[k + 1] = (int)F.Li.size();
        F.pinv[ipiv] = k;
        for (int i : rows) x[i] = 0.0;
    }
    for (auto& r : F.Li) r = F.pinv[r];
    F.P.assign(n, 0);
    for (int i = 0; i < n; ++i) F.P[F.pinv[i]] = i;
    return true;
}

bool refactor(const int* Ap, const int* Ai, const double* Ax, Factors& F) {
    const int n = F.n;
    std::vector<double> x(n, 0.0);
    bool ok = true;
    for (int k = 0; k < n && ok; ++k) {
        const int col = F.Q[k];
        for (int p = Ap[col]; p < Ap[col + 1]; ++p) x[F.pinv[Ai[p]]] += Ax[p];
        const int ud = F.Up[k + 1] - 1;  // diagonal slot
        for (int p = F.Up[k]; p < ud; ++p) {
            const int jj = F.Ui[p];
            const double xj = x[jj];
            F.Ux[p] = xj;
            x[jj] = 0.0;
            for (int q = F.Lp[jj]; q < F.Lp[jj + 1]; ++q) x[F.Li[q]] -= F.Lx[q] * xj;
        }
        const double piv = x[k];
        x[k] = 0.0;
        F.Ux[ud] = piv;
        if (!(std::fabs(piv) > 0.0) || !finite_bits(piv)) ok = false;
        for (int q = F.Lp[k]; q < F.Lp[k + 1]; ++q) {
            F.Lx[q] = x[F.Li[q]] / piv;
            x[F.Li[q]] = 0.0;
        }
    }
    return ok;
}

void solve(const Factors& F, double* b) {
    const int n = F.n;
    std::vector<double> y(n);
    for (int k = 0; k < n; ++k) y[k] = b[F.P[k]];
    for (int k = 0; k < n; ++k) {
        const double yk = y[k];
        for (int q = F.Lp[k]; q < F.Lp[k + 1]; ++q) y[F.Li[q]] -= F.Lx[q] * yk;
    }
    for (int k = n - 1; k >= 0; --k) {
        const int ud = F.Up[k + 1] - 1;
        const double yk = y[k] / F.Ux[ud];
        y[k] = yk;
        for (int p = F.Up[k]; p < ud; ++p) y[F.Ui[p]] -= F.Ux[p] * yk;
    }
    for (int k = 0; k < n; ++k) b[F.Q[k]] = y[k];
}

double pivot_ratio(const Factors& F) {
    double pmin = INFINITY, pmax = 0.0;
    for (int k = 0; k < F.n; ++k) {
        const double a = std::fabs(F.Ux[F.Up[k + 1] - 1]);
        if (!finite_bits(a)) return 0.0;
        pmin = std::min(pmin, a);
        pmax = std::max(pmax, a);
    }
    if (!(pmax > 0.0)) return 0.0;
    return pmin / pmax;
}

}  // namespace slu
