// plan.cpp -- see plan.h.
#include "plan.h"

#include <cstring>
#include <string>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <queue>
#include <set>
#include <utility>

namespace gbpf {

namespace {

// Minimum-degree order of an undirected graph given as sorted adjacency lists
// (elimination graph: eliminating v turns its neighbourhood into a clique). Ties go to
// the lowest vertex index, so the order is deterministic.
std::vector<int> min_degree(std::vector<std::vector<int>> adj) {
    const int n = (int)adj.size();
    std::set<std::pair<int, int>> q;
    for (int v = 0; v < n; ++v) q.insert({(int)adj[v].size(), v});
    std::vector<int> order;
    order.reserve(n);
    std::vector<int> tmp;
    while (!q.empty()) {
        const int v = q.begin()->second;
        q.erase(q.begin());
        order.push_back(v);
        const std::vector<int> nb = std::move(adj[v]);
        adj[v].clear();
        for (int u : nb) {
            auto& a = adj[u];
            q.erase({(int)a.size(), u});
            tmp.clear();
            std::set_union(a.begin(), a.end(), nb.begin(), nb.end(), std::back_inserter(tmp));
            a.clear();
            for (int w : tmp)
                if (w != u && w != v) a.push_back(w);
            q.insert({(int)a.size(), u});
        }
    }
    return order;
}

inline int rank_in(const std::vector<int>& Li, int lo, int hi, int x) {
    return (int)(std::lower_bound(Li.begin() + lo, Li.begin() + hi, x) - (Li.begin() + lo));
}

// Deal tasks (weights) of one level to W workers: longest first, each onto the currently
// least-loaded worker (ties: lowest worker). Returns the worker of every task and the
// largest worker load.
int deal(const std::vector<long long>& weight, int W, std::vector<int>& who) {
    const int n = (int)weight.size();
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return weight[a] > weight[b]; });
    using E = std::pair<long long, int>;
    std::priority_queue<E, std::vector<E>, std::greater<E>> load;
    for (int w = 0; w < W; ++w) load.push({0, w});
    who.assign(n, 0);
    long long mx = 0;
    for (int i : idx) {
        E e = load.top();
        load.pop();
        who[i] = e.second;
        e.first += weight[i];
        mx = std::max(mx, e.first);
        load.push(e);
    }
    return (int)std::min<long long>(mx, 1LL << 30);
}

using Task = PlanTask;

// Reverse Cuthill-McKee order of the bus graph (the Ybus pattern): breadth-first from a
// least-connected unvisited bus of each component, neighbours by increasing degree, the
// whole sequence reversed (Cuthill & McKee 1969; George's reversal).
std::vector<int> rcm_order(int n, const int* Yp, const int* Yj) {
    std::vector<int> deg(n, 0);
    for (int i = 0; i < n; ++i)
        for (int k = Yp[i]; k < Yp[i + 1]; ++k) deg[i] += Yj[k] != i;
    auto lighter = [&](int a, int b) { return deg[a] != deg[b] ? deg[a] < deg[b] : a < b; };
    std::vector<int> starts(n);
    for (int i = 0; i < n; ++i) starts[i] = i;
    std::sort(starts.begin(), starts.end(), lighter);
    std::vector<char> seen(n, 0);
    std::vector<int> order, nb;
    order.reserve(n);
    for (int s0 : starts) {
        if (seen[s0]) continue;
        size_t head = order.size();
        order.push_back(s0);
        seen[s0] = 1;
        while (head < order.size()) {
            const int u = order[head++];
            nb.clear();
            for (int k = Yp[u]; k < Yp[u + 1]; ++k) {
                const int j = Yj[k];
                if (j != u && !seen[j]) {
                    seen[j] = 1;
                    nb.push_back(j);
                }
            }
            std::sort(nb.begin(), nb.end(), lighter);
            order.insert(order.end(), nb.begin(), nb.end());
        }
    }
    std::reverse(order.begin(), order.end());
    return order;
}

// Lay tasks out grouped by (level, worker); `four`: 4 ints per record (else 2). Chains
// (a diagonal and its L column) go to one worker; a chain heavier than its level's share of a
// worker (total weight / W) is cut into segments of at most that share (at least one L block
// each), every segment after the first led by a copy of the diagonal task flagged
// TASK_NOSTORE (it recomputes the inverse from the Jacobian's diagonal, which the pass
// leaves in place). Units are dealt longest-first onto the least-loaded worker.
void layout(const std::vector<Task>& tasks, int nlev, int W, std::vector<int>& out, std::vector<int>& ptr,
            std::vector<int>* level_work, bool four, const std::vector<int>* key = nullptr, double chain_cap = 1.0) {
    std::vector<std::vector<int>> by_level(nlev);
    for (int i = 0; i < (int)tasks.size(); ++i)
        if (tasks[i].head) by_level[tasks[i].level].push_back(i);
    ptr.assign((size_t)nlev * W + 1, 0);
    out.clear();
    std::vector<long long> wts;
    std::vector<int> who;
    std::vector<std::vector<int>> units;  // task indices; ~i = a recomputing copy of diagonal task i
    auto emit = [&](int q) {
        const Task& t = tasks[q < 0 ? ~q : q];
        out.push_back(t.dst);
        out.push_back(q < 0 ? (t.code | TASK_NOSTORE) : t.code);
        if (four) {
            out.push_back(t.p0);
            out.push_back(t.p1);
        }
    };
    for (int h = 0; h < nlev; ++h) {
        const auto& ids = by_level[h];
        long long total = 0;
        for (int id : ids)
            for (int q = id; q >= 0; q = tasks[q].next) total += tasks[q].w;
        // a chain heavier than chain_cap x the level's mean work per worker is cut into
        // segments (0: never cut)
        const long long cap = chain_cap > 0.0 ? std::max<long long>(1, (long long)std::ceil(chain_cap * (double)total / W))
                                              : std::numeric_limits<long long>::max();
        units.clear();
        wts.clear();
        for (int id : ids) {
            long long cw = 0;
            for (int q = id; q >= 0; q = tasks[q].next) cw += tasks[q].w;
            if (cw <= cap || tasks[id].next < 0) {
                units.emplace_back();
                for (int q = id; q >= 0; q = tasks[q].next) units.back().push_back(q);
                wts.push_back(cw);
                continue;
            }
            // segments: [diagonal, L...], then [recomputed diagonal, L...] ...
            units.emplace_back(1, id);
            long long uw = tasks[id].w;
            int nl = 0;
            for (int q = tasks[id].next; q >= 0; q = tasks[q].next) {
                if (nl > 0 && uw + tasks[q].w > cap) {
                    wts.push_back(uw);
                    units.emplace_back(1, ~id);
                    uw = tasks[id].w;
                    nl = 0;
                }
                units.back().push_back(q);
                uw += tasks[q].w;
                ++nl;
            }
            wts.push_back(uw);
        }
        const int mx = deal(wts, W, who);
        if (level_work) (*level_work)[h] += mx;
        // within a worker, units in the order of their key (the factor position they work
        // on): at any moment the workers of a CTA are at similar positions and share the
        // blocks they read in cache
        std::vector<int> mine;
        for (int w = 0; w < W; ++w) {
            ptr[(size_t)h * W + w] = four ? (int)(out.size() / 4) : (int)(out.size() / 2);
            mine.clear();
            for (size_t i = 0; i < units.size(); ++i)
                if (who[i] == w) mine.push_back((int)i);
            if (key)
                std::stable_sort(mine.begin(), mine.end(), [&](int a, int b) {
                    const int qa = units[a][0] < 0 ? ~units[a][0] : units[a][0];
                    const int qb = units[b][0] < 0 ? ~units[b][0] : units[b][0];
                    return (*key)[qa] < (*key)[qb];
                });
            for (int i : mine)
                for (int q : units[i]) emit(q);
        }
    }
    ptr[(size_t)nlev * W] = four ? (int)(out.size() / 4) : (int)(out.size() / 2);
}

}  // namespace

std::string build_plan(Plan& p, int n, const int* Yp, const int* Yj, int nnz, const int* pv, int npv,
                       const int* pq, int npq, int workers, double chain_cap) {
    p = Plan();
    p.n = n;
    p.nnzY = nnz;
    if (n <= 0) return "n_bus must be > 0";
    if (Yp[0] != 0 || Yp[n] != nnz) return "Ybus indptr inconsistent with nnz";
    for (int r = 0; r < n; ++r) {
        if (Yp[r + 1] < Yp[r]) return "Ybus indptr not monotone";
        for (int k = Yp[r]; k < Yp[r + 1]; ++k) {
            if (Yj[k] < 0 || Yj[k] >= n) return "Ybus column index out of range";
            if (k > Yp[r] && Yj[k] <= Yj[k - 1]) return "Ybus column indices must be sorted and unique per row";
        }
    }
    p.vidx.assign(n, -1);
    p.bus_pq.assign(n, 0);
    for (int i = 0; i < npv; ++i) {
        if (pv[i] < 0 || pv[i] >= n) return "pv index out of range";
        if (p.vidx[pv[i]] >= 0) return "bus listed twice in pv/pq";
        p.vidx[pv[i]] = (int)p.vbus.size();
        p.vbus.push_back(pv[i]);
    }
    for (int i = 0; i < npq; ++i) {
        if (pq[i] < 0 || pq[i] >= n) return "pq index out of range";
        if (p.vidx[pq[i]] >= 0) return "bus listed twice in pv/pq";
        p.vidx[pq[i]] = (int)p.vbus.size();
        p.vbus.push_back(pq[i]);
        p.bus_pq[pq[i]] = 1;
    }
    const int nv = p.nv = (int)p.vbus.size();
    p.ydiag.assign(n, -1);
    for (int r = 0; r < n; ++r)
        for (int k = Yp[r]; k < Yp[r + 1]; ++k)
            if (Yj[k] == r) p.ydiag[r] = k;

    // bus graph over variable buses (symmetrised)
    std::vector<std::vector<int>> adj(nv);
    for (int r = 0; r < n; ++r) {
        const int a = p.vidx[r];
        if (a < 0) continue;
        for (int k = Yp[r]; k < Yp[r + 1]; ++k) {
            const int b = p.vidx[Yj[k]];
            if (b < 0 || b == a) continue;
            adj[a].push_back(b);
            adj[b].push_back(a);
        }
    }
    for (auto& a : adj) {
        std::sort(a.begin(), a.end());
        a.erase(std::unique(a.begin(), a.end()), a.end());
    }
    p.perm = min_degree(adj);
    p.eval_order = rcm_order(n, Yp, Yj);
    p.pinv.assign(nv, -1);
    for (int k = 0; k < nv; ++k) p.pinv[p.perm[k]] = k;
    p.row_of_bus.assign(n, -1);
    p.bus_of_row.assign(nv, -1);
    p.row_pq.assign(nv, 0);
    for (int v = 0; v < nv; ++v) {
        const int row = p.pinv[v];
        p.row_of_bus[p.vbus[v]] = row;
        p.bus_of_row[row] = p.vbus[v];
        p.row_pq[row] = p.bus_pq[p.vbus[v]];
    }

    // symbolic factorization on the elimination tree (pivot numbering)
    p.Lp.assign(nv + 1, 0);
    p.Li.clear();
    p.parent.assign(nv, -1);
    std::vector<int> head(nv, -1), next(nv, -1), mark(nv, -1);
    for (int k = 0; k < nv; ++k) {
        const int start = (int)p.Li.size();
        mark[k] = k;
        for (int u : adj[p.perm[k]]) {
            const int i = p.pinv[u];
            if (i > k && mark[i] != k) {
                mark[i] = k;
                p.Li.push_back(i);
            }
        }
        for (int c = head[k]; c != -1; c = next[c])
            for (int q = p.Lp[c]; q < p.Lp[c + 1]; ++q) {
                const int i = p.Li[q];
                if (i > k && mark[i] != k) {
                    mark[i] = k;
                    p.Li.push_back(i);
                }
            }
        std::sort(p.Li.begin() + start, p.Li.end());
        p.Lp[k + 1] = (int)p.Li.size();
        if ((int)p.Li.size() > start) {
            const int par = p.Li[start];
            p.parent[k] = par;
            next[k] = head[par];
            head[par] = k;
        }
    }
    p.height.assign(nv, 0);
    for (int k = 0; k < nv; ++k)
        if (p.parent[k] >= 0) p.height[p.parent[k]] = std::max(p.height[p.parent[k]], p.height[k] + 1);
    p.depth.assign(nv, 0);
    for (int k = nv - 1; k >= 0; --k)
        if (p.parent[k] >= 0) p.depth[k] = p.depth[p.parent[k]] + 1;
    p.nlev = nv ? *std::max_element(p.height.begin(), p.height.end()) + 1 : 0;
    p.nblev = nv ? *std::max_element(p.depth.begin(), p.depth.end()) + 1 : 0;

    p.base.assign(nv + 1, 0);
    for (int t = 0; t < nv; ++t) p.base[t + 1] = p.base[t] + 1 + 2 * (p.Lp[t + 1] - p.Lp[t]);
    p.nblk = p.base[nv];
    if (((long long)p.nblk + p.nv) * 4 >= (1LL << 31)) return "factor pattern too large for int32 positions";
    if (p.nv >= (1 << (31 - TASK_ROW_SHIFT))) return "too many buses for the task code's row field";
    auto cnt = [&](int t) { return p.Lp[t + 1] - p.Lp[t]; };
    auto posU = [&](int t, int b) { return p.base[t] + 1 + rank_in(p.Li, p.Lp[t], p.Lp[t + 1], b); };
    auto posL = [&](int a, int t) { return p.base[t] + 1 + cnt(t) + rank_in(p.Li, p.Lp[t], p.Lp[t + 1], a); };
    auto pos = [&](int a, int b) { return a == b ? p.base[a] : (a > b ? posL(a, b) : posU(a, b)); };

    p.posmap.assign(nnz, -1);
    std::vector<uint8_t> inA(p.nblk, 0);
    for (int r = 0; r < n; ++r) {
        const int a = p.vidx[r];
        if (a < 0) continue;
        for (int k = Yp[r]; k < Yp[r + 1]; ++k) {
            const int b = p.vidx[Yj[k]];
            if (b < 0) continue;
            const int q = pos(p.pinv[a], p.pinv[b]);
            p.posmap[k] = q;
            inA[q] = 1;
        }
    }

    // pair lists grouped by target block, in ascending pivot order
    std::vector<int> pcount(p.nblk + 1, 0), fcount(nv + 1, 0);
    for (int s = 0; s < nv; ++s) {
        const int lo = p.Lp[s], hi = p.Lp[s + 1];
        for (int x = lo; x < hi; ++x) {
            ++fcount[p.Li[x]];
            for (int y = lo; y < hi; ++y) ++pcount[pos(p.Li[x], p.Li[y])];
        }
    }
    std::vector<int> poff(p.nblk + 1, 0), foff(nv + 1, 0);
    for (int q = 0; q < p.nblk; ++q) poff[q + 1] = poff[q] + pcount[q];
    for (int i = 0; i < nv; ++i) foff[i + 1] = foff[i] + fcount[i];
    std::vector<int> fpairs(2 * (size_t)poff[p.nblk]), fwd(2 * (size_t)foff[nv]);
    std::vector<int> pfill(poff.begin(), poff.end() - 1), ffill(foff.begin(), foff.end() - 1);
    for (int s = 0; s < nv; ++s) {
        const int lo = p.Lp[s], hi = p.Lp[s + 1];
        for (int x = lo; x < hi; ++x) {
            const int a = p.Li[x];
            const int la = posL(a, s);
            const int f = ffill[a]++;
            fwd[2 * f] = la;
            fwd[2 * f + 1] = s;
            for (int y = lo; y < hi; ++y) {
                const int b = p.Li[y];
                const int q = pfill[pos(a, b)]++;
                fpairs[2 * q] = la;
                fpairs[2 * q + 1] = posU(s, b);
            }
        }
    }

    // tasks
    const int W = p.W = std::max(1, workers);
    std::vector<Task> A, C;
    p.pairs.clear();
    auto add_pairs_factor = [&](int q, int& p0, int& p1) {
        p0 = (int)(p.pairs.size() / 2);
        for (int e = poff[q]; e < poff[q + 1]; ++e) {
            p.pairs.push_back(fpairs[2 * e]);
            p.pairs.push_back(fpairs[2 * e + 1]);
        }
        p1 = (int)(p.pairs.size() / 2);
    };
    for (int t = 0; t < nv; ++t) {
        const int h = p.height[t];
        int p0, p1;
        // diagonal, then its column of L on the same worker (each L block scaled by the
        // inverse diagonal the worker just computed)
        add_pairs_factor(p.base[t], p0, p1);
        int prev = (int)A.size();
        A.push_back({h, p.base[t], TK_DIAG | (inA[p.base[t]] ? 0 : TASK_FILL) | (t << TASK_ROW_SHIFT), p0, p1,
                     8LL * (p1 - p0) + 24});
        p.n_factor_pairs += p1 - p0;
        for (int x = p.Lp[t]; x < p.Lp[t + 1]; ++x) {
            const int j = p.Li[x];
            const int qu = posU(t, j), ql = posL(j, t);
            if (poff[qu + 1] > poff[qu] || !inA[qu]) {
                add_pairs_factor(qu, p0, p1);
                A.push_back({h, qu, TK_U | (inA[qu] ? 0 : TASK_FILL), p0, p1, 8LL * (p1 - p0) + 8});
                p.n_factor_pairs += p1 - p0;
            }
            add_pairs_factor(ql, p0, p1);
            const int me = (int)A.size();
            A.push_back({h, ql, TK_L | TASK_SCALE | (inA[ql] ? 0 : TASK_FILL), p0, p1, 8LL * (p1 - p0) + 12});
            A[me].head = false;
            A[prev].next = me;
            prev = me;
            p.n_factor_pairs += p1 - p0;
        }
        // forward substitution of block row t (its L row is final after lower levels)
        p0 = (int)(p.pairs.size() / 2);
        for (int e = foff[t]; e < foff[t + 1]; ++e) {
            p.pairs.push_back(fwd[2 * e]);
            p.pairs.push_back(fwd[2 * e + 1]);
        }
        p1 = (int)(p.pairs.size() / 2);
        p.n_fwd_pairs += p1 - p0;
        A.push_back({h, t, TK_FWD, p0, p1, 4LL * (p1 - p0) + 4});
        // backward substitution of block row t
        p0 = (int)(p.pairs.size() / 2);
        for (int x = p.Lp[t]; x < p.Lp[t + 1]; ++x) {
            p.pairs.push_back(posU(t, p.Li[x]));
            p.pairs.push_back(p.Li[x]);
        }
        p1 = (int)(p.pairs.size() / 2);
        p.n_bwd_pairs += p1 - p0;
        C.push_back({p.depth[t], t, p.nblk + t, p0, p1, 4LL * (p1 - p0) + 8});
    }
    if (p.pairs.size() / 2 >= (size_t)1 << 31) return "too many pairs";
    p.tasksA = std::move(A);
    p.tasksC = std::move(C);
    Schedule sc;
    make_schedule(p, W, sc, chain_cap);
    p.taskA = std::move(sc.taskA);
    p.ptrA = std::move(sc.ptrA);
    p.taskC = std::move(sc.taskC);
    p.ptrC = std::move(sc.ptrC);
    p.level_work = std::move(sc.level_work);
    return std::string();
}

void make_schedule(const Plan& p, int workers, Schedule& out, double chain_cap) {
    const int W = out.W = std::max(1, workers);
    out.level_work.assign(std::max(p.nlev, p.nblev), 0);
    // factor-level key: the task's destination block (a forward row: its diagonal block)
    std::vector<int> keyA(p.tasksA.size());
    for (size_t i = 0; i < p.tasksA.size(); ++i) {
        const Task& t = p.tasksA[i];
        keyA[i] = (t.code & 3) == TK_FWD ? p.base[t.dst] : t.dst;
    }
    layout(p.tasksA, p.nlev, W, out.taskA, out.ptrA, &out.level_work, true, &keyA, chain_cap);
    std::vector<int> keyC(p.tasksC.size());
    for (size_t i = 0; i < p.tasksC.size(); ++i) keyC[i] = p.tasksC[i].dst;
    layout(p.tasksC, p.nblev, W, out.taskC, out.ptrC, nullptr, true, &keyC, chain_cap);
}

// ----------------------------------------------------------------------------- host replica
void host_eval(const Plan& p, const int* Yp, const int* Yj, const double* Yx, const double* Vm, const double* Va,
               const double* S, const uint8_t* pin, double* blocks, double* R) {
    std::memset(blocks, 0, sizeof(double) * 4 * (size_t)p.nblk);
    for (int i = 0; i < p.n; ++i) {
        const int row = p.row_of_bus[i];
        if (row < 0) continue;
        const bool pqb = p.bus_pq[i] != 0;
        const bool pinned = pin && pin[i];
        const double vi = Vm[i], ci = std::cos(Va[i]), si = std::sin(Va[i]);
        double P = 0, Q = 0, dPa = 0, dQa = 0, dPm = 0, dQm = 0;
        for (int k = Yp[i]; k < Yp[i + 1]; ++k) {
            const int j = Yj[k];
            const double g = Yx[2 * k], b = Yx[2 * k + 1];
            if (j != i) {
                const double vj = Vm[j], cj = std::cos(Va[j]), sj = std::sin(Va[j]);
                const double wr = g * cj - b * sj, wi = g * sj + b * cj;
                const double xr = ci * wr + si * wi, xi = si * wr - ci * wi;
                const double vx = vi * xr, vy = vi * xi;
                const double Wr = vx * vj, Wi = vy * vj;
                P += Wr;
                Q += Wi;
                dPa -= Wi;
                dQa += Wr;
                dPm += vj * xr;
                dQm += vj * xi;
                const int q = p.posmap[k];
                if (q >= 0) {
                    const bool pqj = p.bus_pq[j] != 0;
                    double* o = blocks + 4 * (size_t)q;
                    if (pinned) {
                        o[0] = o[1] = o[2] = o[3] = 0.0;
                    } else {
                        o[0] = Wi;
                        o[1] = pqj ? vx : 0.0;
                        o[2] = pqb ? -Wr : 0.0;
                        o[3] = (pqb && pqj) ? vy : 0.0;
                    }
                }
            } else {
                P += vi * vi * g;
                Q -= vi * vi * b;
                dPm += 2.0 * vi * g;
                dQm -= 2.0 * vi * b;
            }
        }
        double* o = blocks + 4 * (size_t)p.base[row];
        if (pinned) {
            o[0] = 1.0;
            o[1] = 0.0;
            o[2] = 0.0;
            o[3] = 1.0;
        } else {
            o[0] = dPa;
            o[1] = pqb ? dPm : 0.0;
            o[2] = pqb ? dQa : 0.0;
            o[3] = pqb ? dQm : 1.0;
        }
        R[2 * row] = pinned ? 0.0 : S[2 * i] - P;
        R[2 * row + 1] = (pinned || !pqb) ? 0.0 : S[2 * i + 1] - Q;
    }
}

static inline void mm_sub(double* acc, const double* a, const double* b) {
    acc[0] -= a[0] * b[0] + a[1] * b[2];
    acc[1] -= a[0] * b[1] + a[1] * b[3];
    acc[2] -= a[2] * b[0] + a[3] * b[2];
    acc[3] -= a[2] * b[1] + a[3] * b[3];
}

bool host_factor(const Plan& p, double* blk, double* pmin, double* pmax) {
    double mn = INFINITY, mx = 0.0;
    bool ok = true;
    const int W = p.W;
    for (int h = 0; h < p.nlev; ++h) {
        for (int w = 0; w < W; ++w) {
            double dinv[4] = {0, 0, 0, 0};  // the worker's last inverse diagonal block
            for (int t = p.ptrA[(size_t)h * W + w]; t < p.ptrA[(size_t)h * W + w + 1]; ++t) {
                const int* T = &p.taskA[4 * (size_t)t];
                const int kind = T[1] & 3;
                if (kind == TK_FWD) continue;
                double acc[4] = {0, 0, 0, 0};
                if (!(T[1] & TASK_FILL))
                    for (int e = 0; e < 4; ++e) acc[e] = blk[4 * (size_t)T[0] + e];
                for (int q = T[2]; q < T[3]; ++q)
                    mm_sub(acc, blk + 4 * (size_t)p.pairs[2 * q], blk + 4 * (size_t)p.pairs[2 * q + 1]);
                double* o = blk + 4 * (size_t)T[0];
                if (kind == TK_DIAG) {
                    const int row = T[1] >> TASK_ROW_SHIFT;
                    const double det = acc[0] * acc[3] - acc[1] * acc[2];
                    const double inv = 1.0 / det;
                    dinv[0] = acc[3] * inv;
                    dinv[1] = -acc[1] * inv;
                    dinv[2] = -acc[2] * inv;
                    dinv[3] = acc[0] * inv;
                    if (T[1] & TASK_NOSTORE) continue;  // a segment's copy: the inverse stays in dinv
                    const double u0 = std::fabs(acc[0]);
                    const double u1 = std::fabs(det / acc[0]);
                    if (!(u0 > 0.0) || !std::isfinite(u0) || !std::isfinite(det)) ok = false;
                    mn = std::min(mn, u0);
                    mx = std::max(mx, u0);
                    if (p.row_pq[row]) {
                        if (!(u1 > 0.0) || !std::isfinite(u1)) ok = false;
                        mn = std::min(mn, u1);
                        mx = std::max(mx, u1);
                    }
                    for (int e = 0; e < 4; ++e) blk[4 * ((size_t)p.nblk + row) + e] = dinv[e];
                } else if (T[1] & TASK_SCALE) {
                    o[0] = acc[0] * dinv[0] + acc[1] * dinv[2];
                    o[1] = acc[0] * dinv[1] + acc[1] * dinv[3];
                    o[2] = acc[2] * dinv[0] + acc[3] * dinv[2];
                    o[3] = acc[2] * dinv[1] + acc[3] * dinv[3];
                } else {
                    for (int e = 0; e < 4; ++e) o[e] = acc[e];
                }
            }
        }
    }
    *pmin = mn;
    *pmax = mx;
    return ok;
}

void host_solve(const Plan& p, const double* blk, double* y) {
    for (int s = 0; s < p.nv; ++s) {
        const double y0 = y[2 * s], y1 = y[2 * s + 1];
        for (int x = p.Lp[s]; x < p.Lp[s + 1]; ++x) {
            const int a = p.Li[x];
            const double* l = blk + 4 * (size_t)(p.base[s] + 1 + (p.Lp[s + 1] - p.Lp[s]) + (x - p.Lp[s]));
            y[2 * a] -= l[0] * y0 + l[1] * y1;
            y[2 * a + 1] -= l[2] * y0 + l[3] * y1;
        }
    }
    for (int t = p.nv - 1; t >= 0; --t) {
        double r0 = y[2 * t], r1 = y[2 * t + 1];
        for (int x = p.Lp[t]; x < p.Lp[t + 1]; ++x) {
            const int j = p.Li[x];
            const double* u = blk + 4 * (size_t)(p.base[t] + 1 + (x - p.Lp[t]));
            r0 -= u[0] * y[2 * j] + u[1] * y[2 * j + 1];
            r1 -= u[2] * y[2 * j] + u[3] * y[2 * j + 1];
        }
        const double* d = blk + 4 * ((size_t)p.nblk + t);
        y[2 * t] = d[0] * r0 + d[1] * r1;
        y[2 * t + 1] = d[2] * r0 + d[3] * r1;
    }
}

}  // namespace gbpf

// ------------------------------------------------------------------ schedule self-test
namespace gbpf {

// Serial execution of the device schedule in double precision (the factor levels, which carry
// the forward substitution, then the backward levels), and a structural check that no task of
// a level reads what another task of the same level writes.
std::string schedule_selftest(const Plan& p, double* blk, const double* R, double* y) {
    const int W = p.W;
    std::vector<int> wstamp((size_t)p.nblk + p.nv, -1), ystamp(std::max(p.nv, 1), -1);
    for (int h = 0; h < p.nlev; ++h) {
        // structural: writes of the factor level
        for (int w = 0; w < W; ++w)
            for (int t = p.ptrA[(size_t)h * W + w]; t < p.ptrA[(size_t)h * W + w + 1]; ++t) {
                const int* T = &p.taskA[4 * (size_t)t];
                if ((T[1] & 3) == TK_FWD)
                    ystamp[T[0]] = h;
                else if ((T[1] & 3) == TK_DIAG) {  // writes its inverse; the Jacobian's block stays
                    if (!(T[1] & TASK_NOSTORE)) wstamp[(size_t)p.nblk + (T[1] >> TASK_ROW_SHIFT)] = h;
                } else
                    wstamp[T[0]] = h;
            }
        for (int w = 0; w < W; ++w)
            for (int t = p.ptrA[(size_t)h * W + w]; t < p.ptrA[(size_t)h * W + w + 1]; ++t) {
                const int* T = &p.taskA[4 * (size_t)t];
                const bool fwd = (T[1] & 3) == TK_FWD;
                if ((T[1] & 3) == TK_DIAG && wstamp[T[0]] == h)
                    return "level " + std::to_string(h) + ": a diagonal block is rewritten in its level";
                for (int q = T[2]; q < T[3]; ++q) {
                    const int a = p.pairs[2 * q], b = p.pairs[2 * q + 1];
                    if (wstamp[a] == h) return "level " + std::to_string(h) + ": a task reads a block written in its level";
                    if (!fwd && wstamp[b] == h) return "level " + std::to_string(h) + ": a task reads a block written in its level";
                    if (fwd && ystamp[b] == h) return "level " + std::to_string(h) + ": forward row reads a row of its level";
                }
            }
        // execute the level in reverse worker order (any order must give the same result)
        for (int w = W - 1; w >= 0; --w) {
            double dinv[4] = {0, 0, 0, 0};
            int dinv_level = -1;
            for (int t = p.ptrA[(size_t)h * W + w]; t < p.ptrA[(size_t)h * W + w + 1]; ++t) {
                const int* T = &p.taskA[4 * (size_t)t];
                const int kind = T[1] & 3;
                if (kind == TK_FWD) {
                    double y0 = R[2 * T[0]], y1 = R[2 * T[0] + 1];
                    for (int q = T[2]; q < T[3]; ++q) {
                        const double* l = blk + 4 * (size_t)p.pairs[2 * q];
                        const int srow = p.pairs[2 * q + 1];
                        y0 -= l[0] * y[2 * srow] + l[1] * y[2 * srow + 1];
                        y1 -= l[2] * y[2 * srow] + l[3] * y[2 * srow + 1];
                    }
                    y[2 * T[0]] = y0;
                    y[2 * T[0] + 1] = y1;
                    continue;
                }
                double acc[4] = {0, 0, 0, 0};
                if (!(T[1] & TASK_FILL))
                    for (int e = 0; e < 4; ++e) acc[e] = blk[4 * (size_t)T[0] + e];
                for (int q = T[2]; q < T[3]; ++q) {
                    const double* a = blk + 4 * (size_t)p.pairs[2 * q];
                    const double* b = blk + 4 * (size_t)p.pairs[2 * q + 1];
                    acc[0] -= a[0] * b[0] + a[1] * b[2];
                    acc[1] -= a[0] * b[1] + a[1] * b[3];
                    acc[2] -= a[2] * b[0] + a[3] * b[2];
                    acc[3] -= a[2] * b[1] + a[3] * b[3];
                }
                double* o = blk + 4 * (size_t)T[0];
                if (kind == TK_DIAG) {
                    const double det = acc[0] * acc[3] - acc[1] * acc[2];
                    if (!(std::fabs(det) > 0.0)) return "zero pivot block";
                    const double inv = 1.0 / det;
                    dinv[0] = acc[3] * inv;
                    dinv[1] = -acc[1] * inv;
                    dinv[2] = -acc[2] * inv;
                    dinv[3] = acc[0] * inv;
                    dinv_level = h;
                    if (!(T[1] & TASK_NOSTORE))
                        for (int e = 0; e < 4; ++e) blk[4 * ((size_t)p.nblk + (T[1] >> TASK_ROW_SHIFT)) + e] = dinv[e];
                } else if (T[1] & TASK_SCALE) {
                    if (dinv_level != h) return "level " + std::to_string(h) + ": an L block without its diagonal";
                    o[0] = acc[0] * dinv[0] + acc[1] * dinv[2];
                    o[1] = acc[0] * dinv[1] + acc[1] * dinv[3];
                    o[2] = acc[2] * dinv[0] + acc[3] * dinv[2];
                    o[3] = acc[2] * dinv[1] + acc[3] * dinv[3];
                } else {
                    for (int e = 0; e < 4; ++e) o[e] = acc[e];
                }
            }
        }
    }
    std::vector<int> bst(std::max(p.nv, 1), -1);
    for (int h = 0; h < p.nblev; ++h) {
        for (int w = 0; w < W; ++w)
            for (int t = p.ptrC[(size_t)h * W + w]; t < p.ptrC[(size_t)h * W + w + 1]; ++t) bst[p.taskC[4 * (size_t)t]] = h;
        for (int w = W - 1; w >= 0; --w)
            for (int t = p.ptrC[(size_t)h * W + w]; t < p.ptrC[(size_t)h * W + w + 1]; ++t) {
                const int* T = &p.taskC[4 * (size_t)t];
                double r0 = y[2 * T[0]], r1 = y[2 * T[0] + 1];
                for (int q = T[2]; q < T[3]; ++q) {
                    const double* u = blk + 4 * (size_t)p.pairs[2 * q];
                    const int j = p.pairs[2 * q + 1];
                    if (bst[j] == h) return "backward level " + std::to_string(h) + " reads a row of its level";
                    r0 -= u[0] * y[2 * j] + u[1] * y[2 * j + 1];
                    r1 -= u[2] * y[2 * j] + u[3] * y[2 * j + 1];
                }
                const double* d = blk + 4 * (size_t)T[1];
                y[2 * T[0]] = d[0] * r0 + d[1] * r1;
                y[2 * T[0] + 1] = d[2] * r0 + d[3] * r1;
            }
    }
    return std::string();
}

}  // namespace gbpf

// CPU-only check of the planner and the device schedule (no GPU needed): builds the plan
// for `workers` workers, evaluates the Jacobian at (Vm, Va), runs the schedule serially and
// returns the Newton step per bus (dx[2*bus] = angle, dx[2*bus+1] = magnitude, 0 for
// slack / PV magnitude). Returns 0, or -1 with the reason in `msg`.
extern "C" int gbpf_plan_selftest(int n, const int32_t* Yp, const int32_t* Yj, const double* Yx, int nnz,
                                  const int32_t* pv, int npv, const int32_t* pq, int npq, int workers,
                                  const double* Vm, const double* Va, const double* S, double* dx, int32_t* shape,
                                  char* msg, int msglen, double chain_cap) {
    gbpf::Plan p;
    std::string e = chain_cap >= 0.0 ? gbpf::build_plan(p, n, Yp, Yj, nnz, pv, npv, pq, npq, workers, chain_cap)
                                     : std::string("chain_cap must be >= 0");
    if (e.empty()) {
        std::vector<double> blk(4 * ((size_t)p.nblk + p.nv)), R(2 * (size_t)std::max(p.nv, 1)),
            y(2 * (size_t)std::max(p.nv, 1));
        gbpf::host_eval(p, Yp, Yj, Yx, Vm, Va, S, nullptr, blk.data(), R.data());
        e = gbpf::schedule_selftest(p, blk.data(), R.data(), y.data());
        if (e.empty()) {
            for (int b = 0; b < n; ++b) {
                const int r = p.row_of_bus[b];
                dx[2 * b] = r >= 0 ? y[2 * r] : 0.0;
                dx[2 * b + 1] = (r >= 0 && p.bus_pq[b]) ? y[2 * r + 1] : 0.0;
            }
            if (shape) {
                shape[0] = p.nv;
                shape[1] = p.nblk;
                shape[2] = p.nlev;
                shape[3] = p.nblev;
                shape[4] = (int)p.n_factor_pairs;
                shape[5] = (int)p.n_fwd_pairs;
                shape[6] = (int)p.n_bwd_pairs;
            }
        }
    }
    if (!e.empty()) {
        if (msg && msglen > 0) {
            std::strncpy(msg, e.c_str(), (size_t)msglen - 1);
            msg[msglen - 1] = 0;
        }
        return -1;
    }
    return 0;
}
