// nr_oracle.cpp -- CPU oracle for batched polar Newton-Raphson power flow.
//
// TEST INFRASTRUCTURE ONLY: this file is the checker the GPU path is compared against
// (tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg). It is a C-ABI
// restatement, in this project's own code, of the algorithm of the reference's
// p3s/cpp/nr_klu.cpp (e2nIEE/parallel-pandapower-solver 1.2.2):
//   * Topology / J pattern and source map ..... nr_klu.cpp:86-125, 230-285, 732-759
//   * fused mismatch + Jacobian ................ nr_klu.cpp:311-424
//   * NaN-safe infinity norm / trial norm ...... nr_klu.cpp:426-488
//   * Newton loop with Armijo line search ...... nr_klu.cpp:541-711
//   * static-pivot refactorization ("lean") .... p3s/cpp/lean_lu.hpp:55-197
//   * per-column retry on a fresh pivoting LU .. nr_klu.cpp:837-857
//   * batch validation and error messages ...... nr_klu.cpp:1049-1166, 1184-1281
// The pivoting factorization KLU provides there is sparse_lu.cpp (textbook algorithms).
// Floating-point operations are written in the same order as the reference so that the
// oracle reproduces it to the last bit on the same pivot order.
#include <omp.h>

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "sparse_lu.h"

namespace {

using cd = std::complex<double>;

inline bool isfinite_bits(double x) {
    std::uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    return (b & 0x7ff0000000000000ULL) != 0x7ff0000000000000ULL;
}

constexpr double NONFINITE_NORM = 1.7976931348623157e308;  // DBL_MAX sentinel
constexpr double LS_BETA = 0.5;
constexpr int LS_MAX_TRIALS = 10;
constexpr double ARMIJO_C = 1e-4;
constexpr double REUSE_RCOND_RATIO = 1e-3;
constexpr double PIVOT_TOL = 0.001;

// Frozen static-pivot plan (lean_lu.hpp:33-50 restated).
struct Lean {
    bool valid = false;
    int n = 0;
    std::vector<int> P, Q, cp, dpos, row, aK, aSrc, aRow, dK, dU, dLb, dLe;
    double rcond0 = 0.0;
};

struct Topo {
    int n = 0, m = 0;
    std::vector<int> Yp, Yj, Ydiag, pv, pq, pvpq, pvpq_pos, pq_pos, Jp, Ji, src_k;
    std::vector<char> src_block;
    std::vector<double> Ym, Ya;
    std::vector<int> order;  // fill-reducing column order of J (the "analyze" step)
    Lean lean;
    // per column of the last batch call: 0 solved on the frozen (lean) order throughout, 1 a lean
    // refactorization failed its pivot check and the column went on with pivoting LU
    // (nr_klu.cpp:610-652), 2 re-run from its start on pivoting LU (nr_klu.cpp:845-857)
    std::vector<int> last_path;
};

struct State {
    std::vector<double> Jx, Vm, Va, Vm_ls, Va_ls, Pspec, Qspec, F, rhs, Ym, Ya, LU, lu_x, lu_y;
    std::vector<char> pin;
    std::unique_ptr<slu::Factors> num;  // pivoting factorization (fallback path)
    bool use_lean = true;
    bool left_lean = false;  // a lean refactorization of this column failed its pivot check
    explicit State(const Topo& t) {
        Jx.assign(t.Ji.size(), 0.0);
        Vm.assign(t.n, 0.0);
        Va.assign(t.n, 0.0);
        Vm_ls.assign(t.n, 0.0);
        Va_ls.assign(t.n, 0.0);
        Pspec.assign(t.n, 0.0);
        Qspec.assign(t.n, 0.0);
        F.assign(t.m, 0.0);
        rhs.assign(t.m, 0.0);
        if (t.lean.valid) {
            LU.assign(t.lean.row.size(), 0.0);
            lu_x.assign(t.m, 0.0);
            lu_y.assign(t.m, 0.0);
        }
    }
};

// ---- J pattern (nr_klu.cpp:230-285): CSC, dVa columns for pvpq then dVm for pq; in each
// column the P rows of the Ybus column's rows first, then the Q rows.
void build_pattern(Topo& w) {
    const int npvpq = (int)w.pvpq.size(), npq = (int)w.pq.size();
    w.m = npvpq + npq;
    std::vector<std::vector<std::pair<int, int>>> col(w.n);
    for (int r = 0; r < w.n; ++r)
        for (int k = w.Yp[r]; k < w.Yp[r + 1]; ++k) col[w.Yj[k]].push_back({r, k});
    w.Jp.assign(w.m + 1, 0);
    int c = 0;
    auto emit = [&](int bus, bool vm) {
        for (auto& e : col[bus]) {
            const int rp = w.pvpq_pos[e.first];
            if (rp != -1) {
                w.Ji.push_back(rp);
                w.src_k.push_back(e.second);
                w.src_block.push_back(vm ? 1 : 0);
            }
        }
        for (auto& e : col[bus]) {
            const int rq = w.pq_pos[e.first];
            if (rq != -1) {
                w.Ji.push_back(npvpq + rq);
                w.src_k.push_back(e.second);
                w.src_block.push_back(vm ? 3 : 2);
            }
        }
        w.Jp[++c] = (int)w.Ji.size();
    };
    for (int i = 0; i < npvpq; ++i) emit(w.pvpq[i], false);
    for (int i = 0; i < npq; ++i) emit(w.pq[i], true);
}

// ---- fused mismatch + Jacobian (nr_klu.cpp:311-424), same operation order.
void eval_FJ(const Topo& w, State& st, const double* Vm, const double* Va, double* F) {
    const int nnzY = (int)w.Yj.size();
    const double* Ym = st.Ym.empty() ? w.Ym.data() : st.Ym.data();
    const double* Ya = st.Ya.empty() ? w.Ya.data() : st.Ya.data();
    static thread_local std::vector<double> buf, Pc, Qc;
    if (buf.size() < (size_t)4 * nnzY) buf.resize((size_t)4 * nnzY);
    double* dPa = buf.data();
    double* dQa = buf.data() + nnzY;
    double* dPm = buf.data() + 2 * nnzY;
    double* dQm = buf.data() + 3 * nnzY;
    if ((int)Pc.size() < w.n) {
        Pc.resize(w.n);
        Qc.resize(w.n);
    }
    for (int r = 0; r < w.n; ++r) {
        const int d = w.Ydiag[r];
        if (d < 0) continue;
        dPa[d] = 0.0;
        dQa[d] = 0.0;
        dPm[d] = 0.0;
        dQm[d] = 0.0;
    }
    for (int r = 0; r < w.n; ++r) {
        const int d = w.Ydiag[r];
        double p = 0.0, q = 0.0;
        for (int k = w.Yp[r]; k < w.Yp[r + 1]; ++k) {
            const int c = w.Yj[k];
            const double delta = Va[r] - Ya[k] - Va[c];
            double s, co;
            ::sincos(delta, &s, &co);
            const double vy = Vm[r] * Ym[k];
            const double vij = vy * Vm[c];
            p += vij * co;
            q += vij * s;
            if (r != c) {
                const double a = vij * s;
                const double b = -vij * co;
                dPa[k] = a;
                dQa[k] = b;
                dPm[k] = vy * co;
                dQm[k] = vy * s;
                dPa[d] -= a;
                dQa[d] -= b;
                dPm[d] += Ym[k] * Vm[c] * co;
                dQm[d] += Ym[k] * Vm[c] * s;
            } else {
                dPm[d] += 2.0 * Vm[r] * Ym[k] * co;
                dQm[d] += 2.0 * Vm[r] * Ym[k] * s;
            }
        }
        Pc[r] = p;
        Qc[r] = q;
    }
    const int npvpq = (int)w.pvpq.size();
    for (int i = 0; i < npvpq; ++i) F[i] = Pc[w.pvpq[i]] - st.Pspec[w.pvpq[i]];
    for (int i = 0; i < (int)w.pq.size(); ++i) F[npvpq + i] = Qc[w.pq[i]] - st.Qspec[w.pq[i]];
    const double* blk[4] = {dPa, dPm, dQa, dQm};
    const int nzJ = (int)w.Ji.size();
    for (int p = 0; p < nzJ; ++p) st.Jx[p] = blk[(int)w.src_block[p]][w.src_k[p]];
    if (!st.pin.empty()) {
        for (int c = 0; c < w.m; ++c)
            for (int p = w.Jp[c]; p < w.Jp[c + 1]; ++p) {
                const int r = w.Ji[p];
                const int rb = r < npvpq ? w.pvpq[r] : w.pq[r - npvpq];
                if (st.pin[rb]) st.Jx[p] = (r == c) ? 1.0 : 0.0;
            }
        for (int r = 0; r < npvpq; ++r)
            if (st.pin[w.pvpq[r]]) F[r] = 0.0;
        for (int r = 0; r < (int)w.pq.size(); ++r)
            if (st.pin[w.pq[r]]) F[npvpq + r] = 0.0;
    }
}

double mismatch_norm(const double* F, int m) {
    double n = 0.0, sum = 0.0;
    for (int i = 0; i < m; ++i) {
        const double a = std::fabs(F[i]);
        sum += a;
        n = std::max(n, a);
    }
    return isfinite_bits(sum) ? n : NONFINITE_NORM;
}

// trial norm without Jacobian (nr_klu.cpp:456-488)
double eval_F_norm(const Topo& w, const State& st, const double* Vm, const double* Va) {
    const double* Ym = st.Ym.empty() ? w.Ym.data() : st.Ym.data();
    const double* Ya = st.Ya.empty() ? w.Ya.data() : st.Ya.data();
    const char* pin = st.pin.empty() ? nullptr : st.pin.data();
    double nrm = 0.0, sum = 0.0;
    for (int r : w.pvpq) {
        if (pin && pin[r]) continue;
        double p = 0.0;
        for (int k = w.Yp[r]; k < w.Yp[r + 1]; ++k) {
            const double delta = Va[r] - Ya[k] - Va[w.Yj[k]];
            p += Vm[r] * Ym[k] * Vm[w.Yj[k]] * std::cos(delta);
        }
        const double a = std::fabs(p - st.Pspec[r]);
        sum += a;
        nrm = std::max(nrm, a);
    }
    for (int r : w.pq) {
        if (pin && pin[r]) continue;
        double q = 0.0;
        for (int k = w.Yp[r]; k < w.Yp[r + 1]; ++k) {
            const double delta = Va[r] - Ya[k] - Va[w.Yj[k]];
            q += Vm[r] * Ym[k] * Vm[w.Yj[k]] * std::sin(delta);
        }
        const double a = std::fabs(q - st.Qspec[r]);
        sum += a;
        nrm = std::max(nrm, a);
    }
    return isfinite_bits(sum) ? nrm : NONFINITE_NORM;
}

// ---- static-pivot plan from one pivoting factorization (lean_lu.hpp:55-140 restated)
bool lean_build(Lean& pl, int n, const int* Ap, const int* Ai, const slu::Factors& F) {
    pl = Lean();
    pl.P = F.P;
    pl.Q = F.Q;
    pl.n = n;
    double pmin = INFINITY, pmax = 0.0;
    for (int k = 0; k < n; ++k) {
        const double a = std::fabs(F.Ux[F.Up[k + 1] - 1]);  // Rs = 1 (no row scaling)
        pmin = std::min(pmin, a);
        pmax = std::max(pmax, a);
    }
    if (!isfinite_bits(pmax) || !isfinite_bits(pmin) || !(pmax > 0.0) || !(pmin > 0.0)) return false;
    pl.rcond0 = pmin / pmax;
    std::vector<int> Pinv(n);
    for (int k = 0; k < n; ++k) Pinv[pl.P[k]] = k;
    pl.cp.assign(n + 1, 0);
    pl.dpos.assign(n, -1);
    for (int k = 0; k < n; ++k) {
        const int nu = F.Up[k + 1] - F.Up[k] - 1;
        const int nl = F.Lp[k + 1] - F.Lp[k];
        pl.cp[k + 1] = pl.cp[k] + nu + 1 + nl;
    }
    pl.row.resize(pl.cp[n]);
    std::vector<int> Lb(n), Le(n);
    for (int k = 0; k < n; ++k) {
        int q = pl.cp[k];
        for (int p = F.Up[k]; p < F.Up[k + 1] - 1; ++p) pl.row[q++] = F.Ui[p];  // ascending
        pl.dpos[k] = q;
        pl.row[q++] = k;
        Lb[k] = q;
        for (int p = F.Lp[k]; p < F.Lp[k + 1]; ++p) pl.row[q++] = F.Li[p];
        Le[k] = q;
    }
    std::vector<char> inpat(n, 0);
    pl.aK.assign(1, 0);
    pl.dK.assign(1, 0);
    for (int k = 0; k < n; ++k) {
        for (int q = pl.cp[k]; q < pl.cp[k + 1]; ++q) inpat[pl.row[q]] = 1;
        const int ac = pl.Q[k];
        for (int p = Ap[ac]; p < Ap[ac + 1]; ++p) {
            const int r = Pinv[Ai[p]];
            if (!inpat[r]) return false;
            pl.aSrc.push_back(p);
            pl.aRow.push_back(r);
        }
        pl.aK.push_back((int)pl.aSrc.size());
        for (int q = pl.cp[k]; q < pl.dpos[k]; ++q) {
            const int j = pl.row[q];
            pl.dU.push_back(q);
            pl.dLb.push_back(Lb[j]);
            pl.dLe.push_back(Le[j]);
        }
        pl.dK.push_back((int)pl.dU.size());
        for (int q = pl.cp[k]; q < pl.cp[k + 1]; ++q) inpat[pl.row[q]] = 0;
    }
    pl.valid = true;
    return true;
}

double lean_refactor(const Lean& pl, const double* Ax, double* LU, double* x) {
    const int* row = pl.row.data();
    double pmin = INFINITY, pmax = 0.0, asum = 0.0;
    bool finite = true;
    for (int k = 0; k < pl.n; ++k) {
        for (int e = pl.aK[k]; e < pl.aK[k + 1]; ++e) x[pl.aRow[e]] += Ax[pl.aSrc[e]];
        for (int d = pl.dK[k]; d < pl.dK[k + 1]; ++d) {
            const double u = x[row[pl.dU[d]]];
            if (u == 0.0) continue;
            for (int s = pl.dLb[d]; s < pl.dLe[d]; ++s) x[row[s]] -= u * LU[s];
        }
        const int dp = pl.dpos[k];
        for (int q = pl.cp[k]; q < dp; ++q) {
            const int r = row[q];
            LU[q] = x[r];
            x[r] = 0.0;
        }
        const double piv = x[k];
        x[k] = 0.0;
        LU[dp] = piv;
        const double a = std::fabs(piv);
        if (!(a > 0.0)) finite = false;
        asum += a;
        pmin = std::min(pmin, a);
        pmax = std::max(pmax, a);
        const double inv = 1.0 / piv;
        for (int q = dp + 1; q < pl.cp[k + 1]; ++q) {
            const int r = row[q];
            LU[q] = x[r] * inv;
            x[r] = 0.0;
        }
    }
    if (!finite || !isfinite_bits(asum) || pmax == 0.0) return 0.0;
    return pmin / pmax;
}

void lean_solve(const Lean& pl, const double* LU, double* b, double* y) {
    const int n = pl.n;
    const int* row = pl.row.data();
    for (int k = 0; k < n; ++k) y[k] = b[pl.P[k]];
    for (int k = 0; k < n; ++k) {
        const double yk = y[k];
        if (yk == 0.0) continue;
        for (int q = pl.dpos[k] + 1; q < pl.cp[k + 1]; ++q) y[row[q]] -= LU[q] * yk;
    }
    for (int k = n - 1; k >= 0; --k) {
        const double zk = y[k] / LU[pl.dpos[k]];
        y[k] = zk;
        if (zk == 0.0) continue;
        for (int q = pl.cp[k]; q < pl.dpos[k]; ++q) y[row[q]] -= LU[q] * zk;
    }
    for (int k = 0; k < n; ++k) b[pl.Q[k]] = y[k];
}

struct Result {
    int iterations;
    bool converged;
    int path = 0;  // Topo::last_path's code
};

// ---- Newton loop (nr_klu.cpp:569-711). `fresh` = no inherited pivoting factorization.
Result run_newton(const Topo& w, State& st, int max_iter, double tol, bool line_search) {
    const int npvpq = (int)w.pvpq.size(), npq = (int)w.pq.size();
    double *Vm = st.Vm.data(), *Va = st.Va.data(), *F = st.F.data(), *rhs = st.rhs.data();
    double *Vml = st.Vm_ls.data(), *Val = st.Va_ls.data();
    eval_FJ(w, st, Vm, Va, F);
    double nrm = mismatch_norm(F, w.m);
    int it = 0;
    bool converged = false;
    while (it < max_iter) {
        if (nrm < tol) {
            converged = true;
            break;
        }
        if (nrm >= NONFINITE_NORM) break;
        ++it;
        bool lean_done = false;
        if (st.use_lean && w.lean.valid) {
            const double rc = lean_refactor(w.lean, st.Jx.data(), st.LU.data(), st.lu_x.data());
            if (rc >= REUSE_RCOND_RATIO * w.lean.rcond0) {
                for (int i = 0; i < w.m; ++i) rhs[i] = -F[i];
                lean_solve(w.lean, st.LU.data(), rhs, st.lu_y.data());
                lean_done = true;
            } else {
                st.use_lean = false;
                st.left_lean = true;
                st.num.reset();
            }
        }
        if (!lean_done) {
            bool need_factor = !st.num;
            if (!need_factor && !slu::refactor(w.Jp.data(), w.Ji.data(), st.Jx.data(), *st.num)) {
                st.num.reset();
                need_factor = true;
            }
            if (need_factor) {
                st.num.reset(new slu::Factors);
                if (!slu::factor(w.m, w.Jp.data(), w.Ji.data(), st.Jx.data(), w.order, PIVOT_TOL, *st.num)) {
                    st.num.reset();
                    return {it, false};
                }
            }
            for (int i = 0; i < w.m; ++i) rhs[i] = -F[i];
            slu::solve(*st.num, rhs);
        }
        auto form_trial = [&](double a) {
            for (int i = 0; i < w.n; ++i) {
                Vml[i] = Vm[i];
                Val[i] = Va[i];
            }
            for (int i = 0; i < npvpq; ++i) Val[w.pvpq[i]] += a * rhs[i];
            for (int i = 0; i < npq; ++i) Vml[w.pq[i]] += a * rhs[npvpq + i];
        };
        auto commit = [&]() {
            for (int i = 0; i < npvpq; ++i) Va[w.pvpq[i]] = Val[w.pvpq[i]];
            for (int i = 0; i < npq; ++i) Vm[w.pq[i]] = Vml[w.pq[i]];
        };
        form_trial(1.0);
        eval_FJ(w, st, Vml, Val, F);
        const double nrm_full = mismatch_norm(F, w.m);
        if (!line_search || nrm_full <= (1.0 - ARMIJO_C) * nrm) {
            commit();
            nrm = nrm_full;
            continue;
        }
        double alpha = 1.0, best_alpha = 1.0, best_nrm = nrm_full;
        for (int trial = 1; trial <= LS_MAX_TRIALS; ++trial) {
            alpha *= LS_BETA;
            form_trial(alpha);
            const double nn = eval_F_norm(w, st, Vml, Val);
            if (nn < best_nrm) {
                best_nrm = nn;
                best_alpha = alpha;
            }
            if (nn <= (1.0 - ARMIJO_C * alpha) * nrm) break;
            if (trial == LS_MAX_TRIALS) {
                if (best_alpha != alpha) form_trial(best_alpha);
                break;
            }
        }
        commit();
        eval_FJ(w, st, Vm, Va, F);
        nrm = mismatch_norm(F, w.m);
    }
    return {it, converged};
}

// nr_klu.cpp:845-857: a column that does not converge on the frozen order is re-run
// from its start on a fresh pivoting factorization.
template <typename Init>
Result run_column(const Topo& w, State& s, Init&& init, int max_iter, double tol, bool ls) {
    const bool reused = w.lean.valid;
    init(s);
    s.use_lean = true;
    s.left_lean = false;
    s.num.reset();
    Result r = run_newton(w, s, max_iter, tol, ls);
    r.path = s.left_lean ? 1 : 0;
    if (r.converged || !reused) return r;
    s.num.reset();
    s.use_lean = false;
    init(s);
    Result r2 = run_newton(w, s, max_iter, tol, ls);
    r2.path = 2;
    return r2;
}

void build_topo(Topo& t, int n, const int* Yp, const int* Yj, const double* Yx, int nnz, const int* pv, int npv,
                const int* pq, int npq) {
    t.n = n;
    t.Yp.assign(Yp, Yp + n + 1);
    t.Yj.assign(Yj, Yj + nnz);
    t.Ym.resize(nnz);
    t.Ya.resize(nnz);
    for (int k = 0; k < nnz; ++k) {
        const cd y(Yx[2 * k], Yx[2 * k + 1]);
        t.Ym[k] = std::abs(y);
        t.Ya[k] = std::arg(y);
    }
    t.Ydiag.assign(n, -1);
    for (int r = 0; r < n; ++r)
        for (int k = t.Yp[r]; k < t.Yp[r + 1]; ++k)
            if (t.Yj[k] == r) {
                t.Ydiag[r] = k;
                break;
            }
    t.pv.assign(pv, pv + npv);
    t.pq.assign(pq, pq + npq);
    t.pvpq = t.pv;
    t.pvpq.insert(t.pvpq.end(), t.pq.begin(), t.pq.end());
    t.pvpq_pos.assign(n, -1);
    for (int i = 0; i < (int)t.pvpq.size(); ++i) t.pvpq_pos[t.pvpq[i]] = i;
    t.pq_pos.assign(n, -1);
    for (int i = 0; i < npq; ++i) t.pq_pos[t.pq[i]] = i;
    build_pattern(t);
    t.order = slu::min_degree_order(t.m, t.Jp.data(), t.Ji.data());
    // freeze the pivot order from one pivoting factorization at |V| = 1, angle 0
    State s(t);
    for (auto& v : s.Vm) v = 1.0;
    eval_FJ(t, s, s.Vm.data(), s.Va.data(), s.F.data());
    slu::Factors F;
    if (slu::factor(t.m, t.Jp.data(), t.Ji.data(), s.Jx.data(), t.order, PIVOT_TOL, F))
        lean_build(t.lean, t.m, t.Jp.data(), t.Ji.data(), F);
}

int n_workers(int n_threads, int T) {
    int nt = n_threads <= 0 ? omp_get_max_threads() : n_threads;
    nt = std::min(nt, omp_get_num_procs());
    nt = std::min(nt, T);
    return std::max(nt, 1);
}

void set_err(char* err, int len, const std::string& msg) {
    if (err && len > 0) {
        std::strncpy(err, msg.c_str(), (size_t)len - 1);
        err[len - 1] = 0;
    }
}

}  // namespace

extern "C" {

void* oracle_create(int n, const int* Yp, const int* Yj, const double* Yx, int nnz, const int* pv, int npv,
                    const int* pq, int npq, char* err, int errlen) {
    try {
        auto* t = new Topo;
        build_topo(*t, n, Yp, Yj, Yx, nnz, pv, npv, pq, npq);
        return t;
    } catch (const std::exception& e) {
        set_err(err, errlen, e.what());
        return nullptr;
    }
}

void oracle_destroy(void* h) { delete static_cast<Topo*>(h); }

int oracle_lean_active(void* h) { return static_cast<Topo*>(h)->lean.valid ? 1 : 0; }

// Path code of every column of the last batch call (see Topo::last_path); returns the count.
int oracle_last_paths(void* h, int* out, int n) {
    const auto& p = static_cast<Topo*>(h)->last_path;
    const int k = std::min(n, (int)p.size());
    for (int i = 0; i < k; ++i) out[i] = p[i];
    return (int)p.size();
}

void oracle_sizes(void* h, int* m, int* nnzJ) {
    auto* t = static_cast<Topo*>(h);
    *m = t->m;
    *nnzJ = (int)t->Ji.size();
}

int oracle_update_Y(void* h, const double* Yx, int nnz) {
    auto* t = static_cast<Topo*>(h);
    if (nnz != (int)t->Yj.size()) return -1;
    for (int k = 0; k < nnz; ++k) {
        const cd y(Yx[2 * k], Yx[2 * k + 1]);
        t->Ym[k] = std::abs(y);
        t->Ya[k] = std::arg(y);
    }
    return 0;
}

// S: (n, T) complex C order; V0: (n,) or (n, T); outputs V (n, T), iterations (T,), converged (T,)
int oracle_solve_batch(void* h, const double* S, int T, const double* V0, int v0_per_col, int max_iter, double tol,
                       int n_threads, int line_search, double* Vout, int* iters, unsigned char* conv, char* err,
                       int errlen) {
    const Topo& t = *static_cast<Topo*>(h);
    const int n = t.n;
    static_cast<Topo*>(h)->last_path.assign(T, 0);
    std::string first;
    const int nt = n_workers(n_threads, T);
#pragma omp parallel num_threads(nt)
    {
        State s(t);
#pragma omp for schedule(dynamic)
        for (int c = 0; c < T; ++c) {
            try {
                auto init = [&](State& cs) {
                    for (int i = 0; i < n; ++i) {
                        const size_t vo = v0_per_col ? ((size_t)i * T + c) : (size_t)i;
                        const double re = V0[2 * vo], im = V0[2 * vo + 1];
                        if (!isfinite_bits(re) || !isfinite_bits(im))
                            throw std::runtime_error("solve_batch: invalid initial voltage at bus " + std::to_string(i) +
                                                     ", step " + std::to_string(c));
                        const size_t so = (size_t)i * T + c;
                        cs.Pspec[i] = S[2 * so];
                        cs.Qspec[i] = S[2 * so + 1];
                        const cd v(re, im);
                        cs.Vm[i] = std::abs(v);
                        cs.Va[i] = std::arg(v);
                        if (cs.Vm[i] <= 0.0 || cs.Vm[i] > 10.0)
                            throw std::runtime_error("solve_batch: invalid voltage magnitude " +
                                                     std::to_string(cs.Vm[i]) + " at bus " + std::to_string(i));
                    }
                };
                Result r = run_column(t, s, init, max_iter, tol, line_search != 0);
                for (int i = 0; i < n; ++i) {
                    const cd v = std::polar(s.Vm[i], s.Va[i]);
                    Vout[2 * ((size_t)i * T + c)] = v.real();
                    Vout[2 * ((size_t)i * T + c) + 1] = v.imag();
                }
                iters[c] = r.iterations;
                conv[c] = r.converged ? 1 : 0;
                static_cast<Topo*>(h)->last_path[c] = r.path;
            } catch (const std::exception& e) {
#pragma omp critical
                {
                    if (first.empty()) first = e.what();
                }
            }
        }
    }
    if (!first.empty()) {
        set_err(err, errlen, first);
        return -1;
    }
    return 0;
}

// Ymag/Yang: (nnz, L) C order; S: (n,); V0: (n, L); pin: (n, L)
int oracle_solve_batch_contingency(void* h, const double* Ymag, const double* Yang, int L, const double* S,
                                   const double* V0, const unsigned char* pin, int max_iter, double tol,
                                   int n_threads, int line_search, double* Vout, int* iters, unsigned char* conv,
                                   char* err, int errlen) {
    const Topo& t = *static_cast<Topo*>(h);
    const int n = t.n, nnz = (int)t.Yj.size();
    static_cast<Topo*>(h)->last_path.assign(L, 0);
    std::string first;
    const int nt = n_workers(n_threads, L);
#pragma omp parallel num_threads(nt)
    {
        State s(t);
#pragma omp for schedule(dynamic)
        for (int c = 0; c < L; ++c) {
            try {
                auto init = [&](State& cs) {
                    cs.Ym.resize(nnz);
                    cs.Ya.resize(nnz);
                    for (int k = 0; k < nnz; ++k) {
                        cs.Ym[k] = Ymag[(size_t)k * L + c];
                        cs.Ya[k] = Yang[(size_t)k * L + c];
                    }
                    cs.pin.resize(n);
                    for (int i = 0; i < n; ++i) {
                        cs.pin[i] = (char)pin[(size_t)i * L + c];
                        cs.Pspec[i] = S[2 * i];
                        cs.Qspec[i] = S[2 * i + 1];
                        const size_t vo = (size_t)i * L + c;
                        const cd v(V0[2 * vo], V0[2 * vo + 1]);
                        cs.Vm[i] = std::abs(v);
                        cs.Va[i] = std::arg(v);
                    }
                };
                Result r = run_column(t, s, init, max_iter, tol, line_search != 0);
                for (int i = 0; i < n; ++i) {
                    const cd v = std::polar(s.Vm[i], s.Va[i]);
                    Vout[2 * ((size_t)i * L + c)] = v.real();
                    Vout[2 * ((size_t)i * L + c) + 1] = v.imag();
                }
                iters[c] = r.iterations;
                conv[c] = r.converged ? 1 : 0;
                static_cast<Topo*>(h)->last_path[c] = r.path;
            } catch (const std::exception& e) {
#pragma omp critical
                {
                    if (first.empty()) first = e.what();
                }
            }
        }
    }
    if (!first.empty()) {
        set_err(err, errlen, first);
        return -1;
    }
    return 0;
}

// Jacobian (CSC) at V0 (nr_klu.cpp:1284-1304): Jp (m+1), Ji (nnzJ), Jx (nnzJ); F (m) mismatch
void oracle_debug_J(void* h, const double* S, const double* V0, int* Jp, int* Ji, double* Jx, double* F) {
    const Topo& t = *static_cast<Topo*>(h);
    State s(t);
    for (int i = 0; i < t.n; ++i) {
        s.Pspec[i] = S[2 * i];
        s.Qspec[i] = S[2 * i + 1];
        const cd v(V0[2 * i], V0[2 * i + 1]);
        s.Vm[i] = std::abs(v);
        s.Va[i] = std::arg(v);
    }
    eval_FJ(t, s, s.Vm.data(), s.Va.data(), s.F.data());
    for (int i = 0; i <= t.m; ++i) Jp[i] = t.Jp[i];
    for (size_t p = 0; p < t.Ji.size(); ++p) {
        Ji[p] = t.Ji[p];
        Jx[p] = s.Jx[p];
    }
    if (F)
        for (int i = 0; i < t.m; ++i) F[i] = s.F[i];
}

}  // extern "C"
