// plan.h -- topology-only setup of the batched polar Newton solver (host side).
//
// Counterpart of the reference's one-off setup: nr_klu.cpp:732-759 (build_topology,
// build_J_pattern), p3s/cuda/polar_topology.py:100-194 (Jacobian pattern + inverse map)
// and p3s/cuda/lean_lu_plan.py:205-321 (fill-reducing order, symbolic factorization,
// level schedule). Re-designed for the GB300 kernel:
//
//  * The Jacobian is factored in 2x2 BUS BLOCKS. Every non-slack bus owns the variable
//    pair (angle, magnitude) and the equation pair (P, Q); a PV bus's magnitude column
//    and Q row are carried as an identity dummy. A block pivot is a whole bus, so one
//    block multiply-subtract does 8 FMAs on 8 loaded values (the scalar form needs 16
//    loads for the same 8 FMAs), and the elimination tree is the bus graph's -- half the
//    height of the scalar one, i.e. half the barriers per factorization.
//  * The fill-reducing order is a minimum-degree order of the bus graph.
//  * Factor entries are computed in Crout form, one task per block; a pivot's diagonal block
//    and its column of L form one chain on one worker (the inverse diagonal stays in
//    registers and scales each L block as it is computed: no separate scaling pass, one
//    barrier per level). The inverse diagonal is stored apart, at block nblk + row, so the
//    Jacobian's diagonal block stays intact through the pass: a chain heavier than its
//    level's share of a worker is cut into segments, each later segment led by a copy of
//    the diagonal task that recomputes the inverse from it without storing anything. Tasks
//    and chain segments are grouped by elimination-tree height (level) and dealt to the
//    CTA's workers longest-first onto the least-loaded worker. The forward substitution
//    rides along in the same levels.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace gbpf {

enum TaskKind { TK_DIAG = 0, TK_U = 1, TK_L = 2, TK_FWD = 3 };
constexpr int TASK_SCALE = 1 << 3;  // L block: multiply by the inverse diagonal block computed just before
constexpr int TASK_FILL = 1 << 4;   // block not in the Jacobian: accumulate from zero
// (bit 5: the diagonal block has two real pivots -- a PQ row; set when a schedule is uploaded)
constexpr int TASK_NOSTORE = 1 << 6;  // diagonal recomputed for a chain segment: keep the inverse in registers
constexpr int TASK_ROW_SHIFT = 8;     // diagonal tasks: block row in code >> 8 (inverse at block nblk + row)

// One unit of factorization work before it is dealt to a worker: its level, destination
// block (or row), code, pair range and weight (the dealing key).
struct PlanTask {
    int level, dst, code, p0, p1;
    long long w;
    int next = -1;     // the next task of its chain (dealt to the same worker, laid out right after)
    bool head = true;  // first task of a chain (or a task on its own)
};

// The worker-dependent part of a plan: the level tasks dealt to W workers.
struct Schedule {
    int W = 0;
    std::vector<int> taskA, ptrA;   // entry tasks (4 ints) and per-(level, worker) ranges
    std::vector<int> taskC, ptrC;   // backward substitution tasks (4 ints)
    std::vector<int> level_work;    // per level: max worker load
};

struct Plan {
    int n = 0;    // buses
    int nnzY = 0;
    int nv = 0;   // variable (non-slack) buses = block rows
    std::vector<int> vbus;          // v -> bus (pv then pq)
    std::vector<int> vidx;          // bus -> v, -1 for slack
    std::vector<uint8_t> bus_pq;    // bus is PQ
    std::vector<int> perm, pinv;    // pivot order over v
    std::vector<int> row_of_bus;    // bus -> block row (pivot index) or -1
    std::vector<int> bus_of_row;    // block row -> bus
    std::vector<uint8_t> row_pq;    // block row is a PQ bus
    std::vector<int> eval_order;    // buses in reverse Cuthill-McKee order (the evaluation's sweep:
                                    // buses evaluated together share their neighbours' state)
    // symbolic (block level, pivot numbering)
    std::vector<int> Lp, Li;        // strict lower structure of each pivot column, ascending
    std::vector<int> parent, height, depth;
    std::vector<int> base;          // first block of each pivot (its diagonal), size nv+1
    int nblk = 0;                   // blocks of the pattern; factor arrays hold nblk + nv (the
                                    // inverse diagonal of row r at block nblk + r)
    std::vector<int> posmap;        // Ybus nnz -> block position, -1 if a slack is involved
    std::vector<int> ydiag;         // bus -> CSR index of its diagonal, -1 if none
    // schedule for W workers
    int W = 0;
    int nlev = 0, nblev = 0;
    std::vector<int> taskA;         // 4 ints per task: dst, kind|flags, p0, p1
    std::vector<int> ptrA;          // nlev*W + 1
    std::vector<int> taskC;         // backward: 4 ints: row, inverse-diagonal block, p0, p1
    std::vector<int> ptrC;          // nblev*W + 1
    std::vector<int> pairs;         // 2 ints per pair
    // undealt tasks (factor levels, backward), kept so other worker counts can be scheduled
    std::vector<PlanTask> tasksA, tasksC;
    // statistics
    long long n_factor_pairs = 0, n_fwd_pairs = 0, n_bwd_pairs = 0;
    double rcond0 = 0.0;            // pivot ratio of the flat-start factorization
    double jinv_est = 0.0;          // |J^-1| (infinity norm) estimate at the flat start
    double y_rowsum = 0.0;          // largest row sum of |Ybus|
    std::vector<int> level_work;    // per level: max worker load (critical path estimate)
};

// Build everything topology-only. Returns an empty string on success, else the error.
std::string build_plan(Plan& p, int n, const int* Yp, const int* Yj, int nnz, const int* pv, int npv,
                       const int* pq, int npq, int workers, double chain_cap = 1.0);

// Deal the plan's tasks to `workers` workers (longest first onto the least-loaded one); a
// level's diagonal-and-L chain heavier than chain_cap x the level's mean work per worker is
// cut into segments on different workers, each later one recomputing the diagonal inverse
// (0: chains are never cut).
void make_schedule(const Plan& p, int workers, Schedule& out, double chain_cap = 1.0);

// Host replica of the device algorithm (double precision): Jacobian blocks at (Vm, Va)
// written to `blocks` (nblk*4, zero where not in the Jacobian) and residual R (nv*2).
// host_factor / host_solve take arrays of (nblk + nv) * 4 (the inverse diagonals after them).
void host_eval(const Plan& p, const int* Yp, const int* Yj, const double* Yx, const double* Vm, const double* Va,
               const double* S, const uint8_t* pin, double* blocks, double* R);
// Serial block LU with the plan (in place); returns min/max real pivot in pmin/pmax and
// false on a zero / non-finite pivot.
bool host_factor(const Plan& p, double* blocks, double* pmin, double* pmax);
// Solve with factored blocks: b (nv*2, block-row order) -> x in place.
void host_solve(const Plan& p, const double* blocks, double* b);

}  // namespace gbpf
