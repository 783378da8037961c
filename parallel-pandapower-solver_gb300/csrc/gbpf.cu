// gbpf.cu -- host orchestration and C ABI (include/gbpf.h) of the batched Newton solver.
//
// The GB300 replacement of the reference's host drivers: nr_klu.cpp's Solver class
// (:964-1313) and PolarNewtonSolverCUDA's chunk loop (nr_polar_solver.py:598-1068). A
// solve is ONE launch of the persistent Newton kernel over the whole batch: no memory
// chunking (the per-CTA scratch is reused case after case, so device memory does not grow
// with the batch), no per-pass status read-back, no CPU hand-off.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "gbpf.h"
#include "gbpf_device.h"
#include "plan.h"

namespace {

thread_local std::string g_err;
thread_local cudaError_t g_copy_error = cudaSuccess;

int fail(const std::string& m) {
    g_err = m;
    return -1;
}

#define CK(x)                                                                                       \
    do {                                                                                            \
        cudaError_t e_ = (x);                                                                       \
        if (e_ != cudaSuccess) return fail(std::string(#x) + " failed: " + cudaGetErrorString(e_)); \
    } while (0)

struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    // Grows to at least b bytes; a buffer that had to grow takes half as much again (1 MiB
    // granules), so that a stream of slowly growing requests reallocates -- and synchronises
    // the device in cudaFree -- only a few times.
    cudaError_t ensure(size_t b) {
        if (b <= bytes && p) return cudaSuccess;
        size_t want = std::max<size_t>(b, 16);
        if (p) {
            want = std::max(want, bytes + bytes / 2);
            want = (want + (1u << 20) - 1) & ~(size_t)((1u << 20) - 1);
            cudaFree(p);
        }
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess && want > b) {  // no room for the headroom: exactly what is asked
            (void)cudaGetLastError();
            want = std::max<size_t>(b, 16);
            e = cudaMalloc(&p, want);
        }
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

template <typename T>
cudaError_t upload(DBuf& b, const std::vector<T>& v) {
    cudaError_t e = b.ensure(v.size() * sizeof(T));
    if (e != cudaSuccess) return e;
    if (!v.empty()) return cudaMemcpy(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return cudaSuccess;
}

int ilog2(int g) {
    int l = 0;
    while ((1 << l) < g) ++l;
    return l;
}

}  // namespace

void gbpf::set_error(const std::string& msg) { g_err = msg; }

gbpf::ScratchOffsets gbpf::scratch_offsets(int n, int nv, int nblk, int G, bool mixed) {
    ScratchOffsets o{};
    unsigned long long at = 0;
    auto take = [&](unsigned long long bytes) {
        const unsigned long long p = at;
        at += (bytes + 255) & ~255ULL;
        return p;
    };
    const unsigned long long g = (unsigned long long)G;
    // factor blocks, then the nv inverse diagonals
    const unsigned long long nf = (unsigned long long)nblk + nv;
    o.fac64 = take(nf * g * 32);
    o.fac32 = mixed ? take(nf * g * 16) : ~0ULL;
    o.fac32b = mixed ? take(nf * g * 16) : ~0ULL;
    o.R = take((unsigned long long)nv * g * 16);
    o.y64 = take((unsigned long long)nv * g * 16);
    o.y32 = mixed ? take((unsigned long long)nv * g * 8) : ~0ULL;
    o.Vc = take((unsigned long long)n * g * 32);
    o.Vt = take((unsigned long long)n * g * 32);
    o.Et = take((unsigned long long)n * g * 16);
    o.Ei = take((unsigned long long)n * g * 8);
    o.iv32 = take((unsigned long long)n * g * 4);
    o.pin = take((unsigned long long)n * g);
    o.total = at;
    return o;
}

// One CTA shape of the Newton kernel for a topology: threads per CTA, case slots per CTA,
// and the factorization schedule dealt to its NT / G workers (built on first use).
struct Shape {
    int NT = 0, G = 0, lg = 0, occ = 1;
    double chain_cap = 1.0;  // the schedule's chain segment cap (make_schedule)
    DBuf dtaskA, dptrA, dtaskC, dptrC, dheadA, dheadC, dtaskF, dheadF, dptrF;
    gbpf::DevPlan dp{};
    ~Shape() {
        for (DBuf* b : {&dtaskA, &dptrA, &dtaskC, &dptrC, &dheadA, &dheadC, &dtaskF, &dheadF, &dptrF})
            b->release();
    }
};

constexpr int N_SIZE_CLASSES = 48;  // batch sizes by ceil(log2(work items))

// Resources of one launch in flight: stream, events, scratch and buffers. The solver's own
// (synchronous calls) and every asynchronous slot have their own, so calls in different slots
// overlap (one's copies with another's kernel) without sharing anything they write.
struct ExecSlot {
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr, c0 = nullptr, c1 = nullptr;
    DBuf scr, bctl, btab, bjobs, bS, bV0, bV, bit, bcv, blane;
    unsigned long long* host_ctl = nullptr;  // page-locked copy of the control block
    bool pending = false;
    int grid = 0, G = 0, NT = 0;
    std::string who;
    ~ExecSlot() {
        for (DBuf* b : {&scr, &bctl, &btab, &bjobs, &bS, &bV0, &bV, &bit, &bcv, &blane}) b->release();
        for (cudaEvent_t e : {e0, e1, c0, c1})
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
        if (host_ctl) cudaFreeHost(host_ctl);
    }
};

struct gbpf_solver {
    gbpf::Plan plan;
    int n = 0, nnz = 0;
    std::vector<int> Yp, Yj;
    std::vector<double> Yx;  // interleaved complex
    int device = 0, nsm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr, c0 = nullptr, c1 = nullptr;
    int fixed_NT = 0, fixed_G = 0;               // CTA shape requested at creation (0: by batch size)
    int table_NT[N_SIZE_CLASSES] = {}, table_G[N_SIZE_CLASSES] = {};  // shapes set per size class
    std::vector<std::unique_ptr<Shape>> shapes;  // every shape built, kept for the solver's lifetime
    double chain_cap = 1.0;  // schedule of the shapes built from now on (gbpf_set_chain_cap)
    std::mutex shapes_mu;  // launches of several groups on this topology may look up shapes at once
    std::vector<std::unique_ptr<ExecSlot>> slots;  // asynchronous calls (gbpf_solve_lanes_async)
    // topology on the device
    DBuf dYp, dYj, dY, dY32, dposmap, drow_of_bus, dbus_pq, dpairs, drow_pq, dbus_of_row, ddpos, deval_order;
    gbpf::DevPlan dp{};  // topology part (schedule fields filled per shape)
    // scratch: one region per CTA (grow-only)
    DBuf scr;
    // per-call buffers (grow-only)
    DBuf bS, bV0, bV, bit, bcv, bctl, blane, bstp, bstk, bstv, bYd, bpin, btab, bjobs;
    DBuf bmis;            // final mismatch of every case of the last synchronous call
    long long mis_n = 0;  // its case count (0: none recorded)
    // islanding buffers (grow-only)
    DBuf iin, iscr, ibest, iout;
    // branch table for outage cases (gbpf_set_branches)
    int m = 0;
    DBuf dbr_f, dbr_t, dbr_live, dbr_pos, dbr_val, dslack, dprio;
    std::vector<int> br_pos;          // host copy of the stamp positions (m x 4)
    DBuf dg_ptr, dg_src, dshunt;      // Ybus gather lists (gbpf_update_Y_from_branches)
    bool gather_ready = false;
    gbpf_stats last{};
    ~gbpf_solver() {
        if (stream) cudaStreamSynchronize(stream);
        for (auto& sl : slots)
            if (sl->stream) cudaStreamSynchronize(sl->stream);
        slots.clear();
        shapes.clear();
        for (DBuf* b : {&dYp, &dYj, &dY, &dY32, &dposmap, &drow_of_bus, &dbus_pq, &dpairs, &drow_pq, &dbus_of_row, &deval_order,
                        &ddpos, &scr, &bS, &bV0, &bV, &bit, &bcv, &bctl, &blane, &bstp, &bstk, &bstv, &bYd, &bpin,
                        &btab, &bjobs, &bmis, &iin, &iscr, &ibest, &iout, &dbr_f, &dbr_t, &dbr_live, &dbr_pos, &dbr_val,
                        &dslack, &dprio, &dg_ptr, &dg_src, &dshunt})
            b->release();
        for (cudaEvent_t e : {e0, e1, c0, c1})
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

int upload_values(gbpf_solver* s) {
    std::vector<double> y(s->Yx);
    std::vector<float> y32(s->Yx.size());
    for (size_t i = 0; i < y.size(); ++i) y32[i] = (float)y[i];
    CK(upload(s->dY, y));
    CK(upload(s->dY32, y32));
    return 0;
}

// Pivot ratio of the frozen order on the base-grid Jacobian at a flat voltage, the
// reference value every later factorization is judged against (nr_klu.cpp:713-729,
// nr_polar_solver.py:409-427).
int compute_rcond0(gbpf_solver* s) {
    gbpf::Plan& p = s->plan;
    // largest row sum of |Y|: scales the rounding floor of a mismatch evaluated in double
    p.y_rowsum = 0.0;
    for (int r = 0; r < s->n; ++r) {
        double a = 0.0;
        for (int k = s->Yp[r]; k < s->Yp[r + 1]; ++k) a += std::hypot(s->Yx[2 * (size_t)k], s->Yx[2 * (size_t)k + 1]);
        p.y_rowsum = std::max(p.y_rowsum, a);
    }
    std::vector<double> Vm(s->n, 1.0), Va(s->n, 0.0), S(2 * (size_t)s->n, 0.0), blk(4 * ((size_t)p.nblk + p.nv)),
        R(2 * (size_t)std::max(p.nv, 1));
    gbpf::host_eval(p, s->Yp.data(), s->Yj.data(), s->Yx.data(), Vm.data(), Va.data(), S.data(), nullptr, blk.data(),
                    R.data());
    double mn = 0, mx = 0;
    if (p.nv == 0) {
        p.rcond0 = 1.0;
        p.jinv_est = 0.0;
        return 0;
    }
    if (!gbpf::host_factor(p, blk.data(), &mn, &mx) || !(mx > 0.0) || !(mn > 0.0) || !std::isfinite(mx)) {
        // no usable reference pivot ratio: every factorization on the device then fails its
        // pivot check and the cases end not converged (nr_klu.cpp's behaviour when its plan
        // cannot be built); gbpf_info reports rcond0 = NaN so callers can refuse the grid
        p.rcond0 = std::nan("");
        p.jinv_est = std::nan("");
        return 0;
    }
    p.rcond0 = mn / mx;
    // |J^-1| (infinity norm) estimate: the largest |J^-1 b| over a few sign vectors b
    // (all ones, P rows only, a fixed pseudo-random pattern); a lower bound that is usually
    // within a small factor
    std::vector<double> y(2 * (size_t)p.nv);
    double est = 0.0;
    unsigned rng = 12345u;
    for (int probe = 0; probe < 3; ++probe) {
        for (int r = 0; r < p.nv; ++r) {
            rng = rng * 1664525u + 1013904223u;
            const double sgn = probe == 2 ? ((rng >> 16) & 1 ? 1.0 : -1.0) : 1.0;
            y[2 * r] = sgn;
            y[2 * r + 1] = probe == 1 ? 0.0 : sgn * (p.row_pq[r] ? 1.0 : 0.0);
        }
        gbpf::host_solve(p, blk.data(), y.data());
        for (double v : y) est = std::max(est, std::fabs(v));
    }
    p.jinv_est = std::isfinite(est) ? est : std::nan("");
    return 0;
}

int setup(gbpf_solver* s, int cases_per_cta, int threads_per_cta) {
    CK(cudaGetDevice(&s->device));
    CK(cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, s->device));
    CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&s->e0));
    CK(cudaEventCreate(&s->e1));
    CK(cudaEventCreate(&s->c0));
    CK(cudaEventCreate(&s->c1));
    if (threads_per_cta != 0 && threads_per_cta != 256 && threads_per_cta != 512 && threads_per_cta != 1024)
        return fail("threads_per_cta must be 256, 512 or 1024");
    if (cases_per_cta != 0 && (cases_per_cta < 1 || cases_per_cta > gbpf::MAX_SLOTS || (cases_per_cta & (cases_per_cta - 1))))
        return fail("cases_per_cta must be a power of two in 1..32");
    s->fixed_NT = threads_per_cta;
    s->fixed_G = cases_per_cta;
    return 0;
}

// CTAs of a launch that needs `want` of them: at most the resident ones. Mixed-precision
// launches (latency-bound factorizations: a CTA's pass costs about the same however many of
// its slots are busy) take a whole number per SM when more than one per SM is needed, so
// that every SM gets the same share of the cases; double launches keep their slots full
// instead (the FP64 pipe is their bound, and a warp of half-empty slots still occupies it).
int grid_size(int nsm, int occ, long long want, bool balance) {
    const long long resident = (long long)nsm * std::max(1, occ);
    if (balance && want > nsm) want = (want + nsm - 1) / nsm * nsm;
    return (int)std::max<long long>(1, std::min(want, resident));
}

int size_class(long long units) {
    int c = 0;
    while (c + 1 < N_SIZE_CLASSES && (1LL << c) < units) ++c;
    return c;
}

// CTA shape for a batch of `units` work items. Case slots per SM: the batch's share of an
// SM rounded up to a power of two (measured on GB300, 2,000-bus grid: every batch from 1 to
// 8,760 cases is within a few percent of its best shape this way), at most 64 per SM
// (32 per SM above 4,096 variable buses, 16 above 16,384: the per-slot working set grows
// with the grid). Up to 4 slots per SM run as one 1,024-thread CTA (many workers per
// case); more run as two 512-thread CTAs per SM, whose phases overlap.
void choose_shape(const gbpf_solver* s, long long units, int* NT, int* G) {
    const int c = size_class(units);
    if (s->table_NT[c]) {
        *NT = s->table_NT[c];
        *G = s->table_G[c];
        return;
    }
    const int nv = std::max(1, s->plan.nv);
    const int cap = nv <= 4096 ? 64 : (nv <= 16384 ? 32 : 16);
    const long long share = (units + s->nsm - 1) / s->nsm;
    int per_sm = 1;
    while (per_sm < share && per_sm < cap) per_sm *= 2;
    int nt = s->fixed_NT, g = s->fixed_G;
    if (!nt && !g) {
        nt = per_sm <= 4 ? 1024 : 512;
    } else if (!nt) {
        nt = 512;
    }
    if (!g) g = std::min(gbpf::MAX_SLOTS, std::max(1, per_sm / (1024 / nt)));
    *NT = nt;
    *G = g;
}

// The schedule of one CTA shape: tasks dealt to NT / G workers, uploaded next to the
// shared topology arrays.
int get_shape(gbpf_solver* s, int NT, int G, Shape** out) {
    std::lock_guard<std::mutex> lock(s->shapes_mu);
    for (auto& sh : s->shapes)
        if (sh->NT == NT && sh->G == G && sh->chain_cap == s->chain_cap) {
            *out = sh.get();
            return 0;
        }
    std::unique_ptr<Shape> sh(new Shape);
    sh->NT = NT;
    sh->G = G;
    sh->chain_cap = s->chain_cap;
    sh->lg = ilog2(G);
    int occ = 1;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gbpf::newton_kernel_ptr(NT), NT, 0));
    sh->occ = std::max(1, occ);
    const gbpf::Plan& p = s->plan;
    gbpf::Schedule sc;
    gbpf::make_schedule(p, NT / G, sc, s->chain_cap);
    // DIAG tasks carry the "two real pivots" flag (PQ row) in bit 5 of their code
    for (size_t t = 0; t < sc.taskA.size() / 4; ++t) {
        if ((sc.taskA[4 * t + 1] & 3) == gbpf::TK_DIAG) {
            const int row = sc.taskA[4 * t + 1] >> gbpf::TASK_ROW_SHIFT;
            if (p.row_pq[row]) sc.taskA[4 * t + 1] |= 32;
        }
    }
    // the first two pairs of every task inline beside its record: a worker fetches them with
    // the record, one task ahead, and starts the task's block loads without first waiting for
    // its pair list
    auto head_pairs = [&](const std::vector<int>& tasks) {
        const size_t nt = tasks.size() / 4;
        std::vector<int> head(4 * nt, -1);
        for (size_t t = 0; t < nt; ++t) {
            const int p0 = tasks[4 * t + 2], p1 = tasks[4 * t + 3];
            for (int k = 0; k < 2 && p0 + k < p1; ++k) {
                head[4 * t + 2 * k] = p.pairs[2 * (size_t)(p0 + k)];
                head[4 * t + 2 * k + 1] = p.pairs[2 * (size_t)(p0 + k) + 1];
            }
        }
        return head;
    };
    CK(upload(sh->dheadA, head_pairs(sc.taskA)));
    CK(upload(sh->dheadC, head_pairs(sc.taskC)));
    // substitution-only lists for chord passes: every worker's forward tasks of each level,
    // the ones it runs inside the full factor-level lists
    std::vector<int> taskF, ptrF((size_t)p.nlev * sc.W + 1, 0);
    for (size_t q = 0; q + 1 < sc.ptrA.size(); ++q) {
        ptrF[q] = (int)(taskF.size() / 4);
        for (int t = sc.ptrA[q]; t < sc.ptrA[q + 1]; ++t)
            if ((sc.taskA[4 * (size_t)t + 1] & 3) == gbpf::TK_FWD)
                for (int k = 0; k < 4; ++k) taskF.push_back(sc.taskA[4 * (size_t)t + k]);
    }
    ptrF.back() = (int)(taskF.size() / 4);
    if (taskF.empty()) taskF.assign(4, 0);  // keeps the upload non-empty for a grid without forward tasks
    CK(upload(sh->dheadF, head_pairs(taskF)));
    CK(upload(sh->dtaskF, taskF));
    CK(upload(sh->dptrF, ptrF));
    CK(upload(sh->dtaskA, sc.taskA));
    CK(upload(sh->dptrA, sc.ptrA));
    CK(upload(sh->dtaskC, sc.taskC));
    CK(upload(sh->dptrC, sc.ptrC));
    sh->dp = s->dp;
    sh->dp.W = sc.W;
    sh->dp.taskA = sh->dtaskA.as<int4>();
    sh->dp.ptrA = sh->dptrA.as<int>();
    sh->dp.taskC = sh->dtaskC.as<int4>();
    sh->dp.ptrC = sh->dptrC.as<int>();
    sh->dp.headA = sh->dheadA.as<int4>();
    sh->dp.headC = sh->dheadC.as<int4>();
    sh->dp.taskF = sh->dtaskF.as<int4>();
    sh->dp.headF = sh->dheadF.as<int4>();
    sh->dp.ptrF = sh->dptrF.as<int>();
    *out = sh.get();
    s->shapes.push_back(std::move(sh));
    return 0;
}

int upload_plan(gbpf_solver* s) {
    const gbpf::Plan& p = s->plan;
    CK(upload(s->dYp, s->Yp));
    CK(upload(s->dYj, s->Yj));
    CK(upload(s->dposmap, p.posmap));
    CK(upload(s->drow_of_bus, p.row_of_bus));
    CK(upload(s->deval_order, p.eval_order));
    CK(upload(s->dbus_pq, p.bus_pq));
    CK(upload(s->dpairs, p.pairs));
    CK(upload(s->drow_pq, p.row_pq));
    CK(upload(s->dbus_of_row, p.bus_of_row));
    std::vector<int> dpos(p.base.begin(), p.base.begin() + p.nv);
    CK(upload(s->ddpos, dpos));
    if (int rc = upload_values(s)) return rc;
    gbpf::DevPlan& d = s->dp;
    d.n = p.n;
    d.nv = p.nv;
    d.nblk = p.nblk;
    d.W = 0;
    d.nlev = p.nlev;
    d.nblev = p.nblev;
    d.nnzY = p.nnzY;
    d.Yp = s->dYp.as<int>();
    d.Yj = s->dYj.as<int>();
    d.Y = s->dY.as<double2>();
    d.Y32 = s->dY32.as<float2>();
    d.posmap = s->dposmap.as<int>();
    d.row_of_bus = s->drow_of_bus.as<int>();
    d.eval_order = s->deval_order.as<int>();
    d.bus_pq = s->dbus_pq.as<uint8_t>();
    d.taskA = nullptr;
    d.ptrA = nullptr;
    d.taskC = nullptr;
    d.ptrC = nullptr;
    d.headA = nullptr;
    d.headC = nullptr;
    d.taskF = nullptr;
    d.headF = nullptr;
    d.ptrF = nullptr;
    d.pairs = s->dpairs.as<int2>();
    d.row_pq = s->drow_pq.as<uint8_t>();
    d.bus_of_row = s->dbus_of_row.as<int>();
    d.dpos = s->ddpos.as<int>();
    return 0;
}

gbpf::ScratchOffsets solver_offsets(const gbpf_solver* s, int G, bool mixed) {
    return gbpf::scratch_offsets(s->n, std::max(1, s->plan.nv), s->plan.nblk, G, mixed);
}

gbpf_params default_params() {
    gbpf_params p{};
    p.max_iter = 30;
    p.tol = 1e-8;
    p.line_search = 1;
    p.precision = 0;
    p.mixed_switch = 1e-3;
    p.check_v0 = 0;
    p.pivot_ratio_double = 1e-3;
    p.pivot_ratio_single = 1e-3;
    p.vote_rule = 1;
    p.polish = 1e-3;
    p.vtol = 1e-8;
    p.chord_tol = 1e-8;
    p.shared_start = 1;
    return p;
}

int check_params(const gbpf_params& p, const char* who) {
    if (p.max_iter <= 0) return fail(std::string(who) + ": max_iter must be > 0");
    if (!(p.tol > 0.0)) return fail(std::string(who) + ": tol must be > 0");
    if (p.precision != 0 && p.precision != 1) return fail(std::string(who) + ": precision must be 0 (double) or 1 (mixed)");
    return 0;
}

// A shared start pays for its one-CTA prologue only over enough cases starting from it.
constexpr long long SHARE_MIN_CASES = 16;

// The launch of `units` work items (cases, or lanes) enqueued on a stream with its own
// scratch and control block; read back with finish_launch.
struct LaunchRes {
    cudaStream_t stream;
    cudaEvent_t e0, e1;
    DBuf *scr, *bctl, *btab, *bjobs;
    unsigned long long* host_ctl;  // 32 entries
};

int enqueue_launch(gbpf_solver* s, LaunchRes& R, gbpf::Batch& b, long long units, const char* who, int* grid_out,
                   int* G_out, int* NT_out) {
    if (units <= 0) return fail(std::string(who) + ": empty batch");
    int NT = 0, G = 0;
    choose_shape(s, units, &NT, &G);
    Shape* sh = nullptr;
    if (int rc = get_shape(s, NT, G, &sh)) return rc;
    const int grid = grid_size(s->nsm, sh->occ, (units + G - 1) / G, b.mixed != 0);
    gbpf::Job job{};
    job.P = sh->dp;
    // the one-slot schedule for a CTA's last case (solo passes)
    Shape* sh1 = sh;
    if (G > 1)
        if (int rc = get_shape(s, NT, 1, &sh1)) return rc;
    job.P1 = sh1->dp;
    job.off = solver_offsets(s, G, b.mixed != 0);
    job.G = G;
    job.log2G = ilog2(G);
    CK(R.scr->ensure((size_t)grid * job.off.total));
    CK(R.bctl->ensure(64 * sizeof(unsigned long long)));
    auto* ctl = R.bctl->as<unsigned long long>();
    CK(cudaMemsetAsync(ctl, 0, 64 * sizeof(unsigned long long), R.stream));
    b.counter = reinterpret_cast<int*>(ctl + 16);
    b.stats = ctl;
    b.err = reinterpret_cast<int*>(ctl + 24);
    // shared start: every case from the same V0 on the base Ybus without pins -- its first
    // evaluation and factorization are computed once (start_kernel) for the whole launch
    const bool share = b.share_ok && units >= SHARE_MIN_CASES && b.v0_shared && b.ymode == 0 && !b.pin && !b.ref_bus &&
                       (!b.mixed || b.vote_rule == 1);
    gbpf::StartJob sj{};
    const size_t tab_bytes = ((size_t)s->n * 64 + 255) & ~(size_t)255;
    if (b.v0_shared) {
        const size_t need = tab_bytes + (share ? gbpf::start_bytes(s->n, s->plan.nv, s->plan.nblk, G, b.mixed != 0) : 0);
        CK(R.btab->ensure(need));
        b.v0tab = R.btab->as<double4_32a>();
    }
    if (share) {
        Shape* s1 = nullptr;
        if (int rc = get_shape(s, 1024, 1, &s1)) return rc;
        sj.P = s1->dp;
        sj.v0tab = b.v0tab;
        sj.mixed = b.mixed;
        sj.log2G = ilog2(G);
        sj.rcond_min = b.mixed ? b.rcond_min32 : b.rcond_min64;
        gbpf::start_carve(sj, R.btab->as<char>() + tab_bytes, s->n, s->plan.nv, s->plan.nblk, G, b.mixed != 0);
        b.R0 = sj.R0;
        b.fac0 = sj.facG;
        b.ok0 = sj.ok0;
    }
    job.B = b;
    const size_t job_bytes = (sizeof(gbpf::Job) + 255) & ~(size_t)255;
    CK(R.bjobs->ensure(job_bytes + sizeof(gbpf::StartJob)));
    CK(cudaMemcpyAsync(R.bjobs->p, &job, sizeof job, cudaMemcpyHostToDevice, R.stream));
    if (share)
        CK(cudaMemcpyAsync(R.bjobs->as<char>() + job_bytes, &sj, sizeof sj, cudaMemcpyHostToDevice, R.stream));
    gbpf::Launch L{};
    L.jobs = R.bjobs->as<gbpf::Job>();
    L.njobs = 1;
    L.scratch = R.scr->as<char>();
    L.cta_bytes = job.off.total;
    L.timed = b.timers;
    CK(cudaEventRecord(R.e0, R.stream));
    if (b.v0_shared)
        CK(gbpf::launch_v0_table(b.V0, s->n, b.check_v0, R.btab->as<double4_32a>(), b.err, R.stream));
    if (share)
        CK(gbpf::launch_start(reinterpret_cast<const gbpf::StartJob*>(R.bjobs->as<char>() + job_bytes), 1, R.stream));
    CK(gbpf::launch_newton(L, grid, NT, R.stream));
    CK(cudaEventRecord(R.e1, R.stream));
    CK(cudaMemcpyAsync(R.host_ctl, ctl, 32 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, R.stream));
    *grid_out = grid;
    *G_out = G;
    *NT_out = NT;
    return 0;
}

// After the launch's stream has finished: its counters into `st`, its device errors reported.
int finish_launch(const LaunchRes& R, int grid, int G, int NT, const char* who, gbpf_stats* st) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, R.e0, R.e1));
    const unsigned long long* host_ctl = R.host_ctl;
    st->single_factorizations = host_ctl[0];
    st->double_factorizations = host_ctl[1];
    st->single_rejected = host_ctl[2];
    st->double_rejected = host_ctl[3];
    st->macro_steps = host_ctl[4];
    st->chord_steps = host_ctl[5];
    st->first_steps = host_ctl[6];
    for (int k = 0; k < 6; ++k) st->phase_cycles[k] = host_ctl[8 + k];
    st->lazy_jacobians = host_ctl[14];
    st->jacobian_sweeps = host_ctl[7];
    st->grid = grid;
    st->cases_per_cta = G;
    st->threads_per_cta = NT;
    st->kernel_ms = ms;
    const int* err = reinterpret_cast<const int*>(host_ctl + 24);
    if (err[0] == gbpf::DE_V0_NONFINITE)
        return fail(std::string(who) + ": invalid initial voltage at bus " + std::to_string(err[1]) + ", step " +
                    std::to_string(err[2]));
    if (err[0] == gbpf::DE_V0_MAGNITUDE)
        return fail(std::string(who) + ": invalid voltage magnitude at bus " + std::to_string(err[1]) + ", step " +
                    std::to_string(err[2]));
    if (err[0] == gbpf::DE_STAMPS)
        return fail(std::string(who) + ": case " + std::to_string(err[2]) + " has " + std::to_string(err[1]) +
                    " outage stamp entries, more than the " + std::to_string(gbpf::MAX_STAMPS) + " supported");
    return 0;
}

// Run the persistent kernel over `units` work items on the solver's own stream and wait.
int run(gbpf_solver* s, gbpf::Batch& b, long long units, const char* who) {
    unsigned long long host_ctl[32];
    LaunchRes R{s->stream, s->e0, s->e1, &s->scr, &s->bctl, &s->btab, &s->bjobs, host_ctl};
    int grid = 0, G = 0, NT = 0;
    s->mis_n = 0;
    CK(s->bmis.ensure((size_t)b.B * 8));
    b.mis = s->bmis.as<double>();
    if (int rc = enqueue_launch(s, R, b, units, who, &grid, &G, &NT)) return rc;
    CK(cudaStreamSynchronize(s->stream));
    s->mis_n = b.B;
    return finish_launch(R, grid, G, NT, who, &s->last);
}

int record_call(gbpf_solver* s) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, s->c0, s->c1));
    s->last.call_ms = ms;
    return 0;
}

void fill_common(gbpf::Batch& b, const gbpf_solver* s, const gbpf_params& p) {
    b.max_iter = p.max_iter;
    b.tol = p.tol;
    b.line_search = p.line_search;
    b.mixed = p.precision == 1;
    b.mixed_switch = p.mixed_switch;
    b.vote_rule = p.vote_rule;
    // mixed (GB300 rule) cases polish to polish x tol, and further on ill-conditioned grids:
    // until |J^-1| x mismatch, a bound on the voltage error left, is below vtol -- but not
    // below twice the rounding floor of the double mismatch (eps x the largest row sum of
    // |Y|), which no step in double precision gets under reliably
    const double polish = p.polish > 0.0 && p.polish <= 1.0 ? p.polish : 1.0;
    b.tol_polish = p.tol * polish;
    const double k = s->plan.jinv_est;
    if (p.vtol > 0.0 && k > 0.0 && std::isfinite(k)) {
        const double floor_ = 2.0 * DBL_EPSILON * s->plan.y_rowsum;
        b.tol_polish = std::min(b.tol_polish, std::max(p.vtol / k, floor_));
    }
    // chord steps belong to the GB300 rule's float cases only (the double path refactors every
    // step like nr_klu)
    b.chord_tol = b.mixed && b.vote_rule == 1 && p.chord_tol > 0.0 ? p.chord_tol : 0.0;
    b.lazy_jac = b.chord_tol > 0.0 && !p.eager_jacobian;
    b.share_ok = p.shared_start != 0;
    b.timers = p.phase_timers != 0;
    b.check_v0 = p.check_v0;
    b.rcond_min64 = p.pivot_ratio_double * s->plan.rcond0;  // nr_klu.cpp:567 REUSE_RCOND_RATIO = 1e-3
    b.rcond_min32 = p.pivot_ratio_single * s->plan.rcond0;
}

// Shape rule for a launch over several topologies: threads per CTA by the batch-size rule of
// choose_shape on the total work; case slots per CTA per job: the batch-size rule's count,
// reduced for large topologies so that a job's CTA holds at most `slot_budget` (16,384)
// variable buses' worth of cases -- a large grid's cases then get many workers each, and
// they set the launch's critical path (measured on GB300, 256 grids of 30..19,423 buses x 16
// scenarios: one slot per CTA for the largest grids halves the launch).
void group_shape(int nsm, long long units, int* NT, int* Gmax) {
    const long long share = (units + nsm - 1) / nsm;
    int per_sm = 1;
    while (per_sm < share && per_sm < 64) per_sm *= 2;
    *NT = per_sm <= 4 ? 1024 : 512;
    *Gmax = std::min(gbpf::MAX_SLOTS, std::max(1, per_sm / (1024 / *NT)));
}

int job_slots(int Gmax, int nv, int budget) {
    int g = 1;
    while (g * 2 <= Gmax && (long long)(g * 2) * std::max(1, nv) <= budget) g *= 2;
    return g;
}

}  // namespace

// A launch context for several topologies at once: its own stream, scratch, control blocks
// and staging buffers. The topologies (gbpf_solver) keep their plans; a group launch borrows
// them and must not overlap a call on the same solver.
struct gbpf_group {
    int device = 0, nsm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr, c0 = nullptr, c1 = nullptr;
    DBuf scr, bjobs, bctl, btab, bin, bout, bisl;
    gbpf_stats last{};
    int fixed_NT = 0;              // threads per CTA (0: by the group rule)
    int slot_budget = 16384;       // variable buses x case slots a CTA may hold per job (measured best on the
                                   // 256-grid batch: 8,192 +5 %, 32,768 +8 % time)
    ~gbpf_group() {
        for (DBuf* b : {&scr, &bjobs, &bctl, &btab, &bin, &bout, &bisl}) b->release();
        for (cudaEvent_t e : {e0, e1, c0, c1})
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// One launch over `nj` jobs whose inputs and outputs are device pointers.
int group_run(gbpf_group* g, int nj, const gbpf_job* jobs, const gbpf_params& p, const char* who) {
    long long units = 0;
    for (int j = 0; j < nj; ++j) {
        const gbpf_job& J = jobs[j];
        if (!J.solver) return fail(std::string(who) + ": job without a solver");
        if (J.n_cases <= 0) return fail(std::string(who) + ": job " + std::to_string(j) + " has no cases");
        if (!J.S || !J.V0 || !J.V || !J.iterations || !J.converged)
            return fail(std::string(who) + ": job " + std::to_string(j) + " lacks an input or output array");
        if (J.cases_per_cta < 0 || J.cases_per_cta > gbpf::MAX_SLOTS || (J.cases_per_cta & (J.cases_per_cta - 1)))
            return fail(std::string(who) + ": job " + std::to_string(j) + ": cases_per_cta must be 0 or a power of two in 1..32");
        if (J.precision != 0)
            return fail(std::string(who) + ": job " + std::to_string(j) + ": a group launch takes its precision from its parameters (precision 0)");
        if (J.out_ptr) {
            if (!J.solver->m) return fail(std::string(who) + ": job " + std::to_string(j) + ": outage cases need the solver's branch table (gbpf_set_branches)");
            if (J.s_per_col || J.v0_per_col || !J.out_idx)
                return fail(std::string(who) + ": job " + std::to_string(j) + ": outage cases take one S and one V0 (n,) and out_ptr / out_idx");
        } else if (J.served) {
            return fail(std::string(who) + ": job " + std::to_string(j) + ": a served mask belongs to outage cases");
        }
        units += J.n_cases;
    }
    int NT = 0, Gmax = 0;
    group_shape(g->nsm, units, &NT, &Gmax);
    if (g->fixed_NT) NT = g->fixed_NT;
    const bool mixed = p.precision == 1;
    // largest work first, so the long jobs start early and the short ones fill the tail
    std::vector<int> order(nj);
    for (int j = 0; j < nj; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const double wa = (double)jobs[a].n_cases * jobs[a].solver->plan.nblk;
        const double wb = (double)jobs[b].n_cases * jobs[b].solver->plan.nblk;
        return wa > wb;
    });
    std::vector<gbpf::Job> hj(nj);
    std::vector<gbpf::StartJob> hs;  // shared starts (their pivot bound is set with the batch)
    std::vector<int> hs_batch;
    unsigned long long cta_bytes = 0;
    long long want = 0;
    int occ = 1 << 20;
    size_t tab_bytes = 0, isl_bytes = 0;
    auto up256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
    // a job whose cases all start from one V0 on the base Ybus without pins gets a shared start
    // (its first evaluation and factorization once, start_kernel)
    auto job_slots_of = [&](const gbpf_job& J) {
        return J.cases_per_cta ? J.cases_per_cta : job_slots(Gmax, J.solver->plan.nv, g->slot_budget);
    };
    auto shares = [&](const gbpf_job& J) {
        return p.shared_start && J.n_cases >= SHARE_MIN_CASES && !J.v0_per_col && !J.st_ptr && !J.out_ptr && !J.pin &&
               (!mixed || p.vote_rule == 1);
    };
    for (int j = 0; j < nj; ++j) {
        const gbpf_job& J = jobs[j];
        tab_bytes += J.v0_per_col ? 0 : up256((size_t)J.solver->n * 64);
        if (shares(J))
            tab_bytes += up256(gbpf::start_bytes(J.solver->n, J.solver->plan.nv, J.solver->plan.nblk, job_slots_of(J),
                                                 mixed));
        if (J.out_ptr) {
            const size_t n = J.solver->n, L = J.n_cases, gi = std::min<size_t>(L, 4 * (size_t)g->nsm);
            isl_bytes += 3 * up256(n * L * 4) + up256(L * 4) + up256(gi * 4 * n * 4) + up256(gi * n * 8);
        }
    }
    CK(g->bisl.ensure(std::max<size_t>(isl_bytes, 256)));
    size_t isl_at = 0;
    struct IslLaunch {
        const gbpf_solver* s;
        const gbpf_job* J;
        int *labels, *served_i, *ref_bus, *nis, *scr, *err;
        unsigned long long* best;
        int grid;
    };
    std::vector<IslLaunch> isl;
    CK(g->bctl.ensure((size_t)nj * 32 * sizeof(unsigned long long)));
    CK(g->btab.ensure(std::max<size_t>(tab_bytes, 64)));
    auto* ctl = g->bctl.as<unsigned long long>();
    CK(cudaMemsetAsync(ctl, 0, (size_t)nj * 32 * sizeof(unsigned long long), g->stream));
    size_t tab_at = 0;
    for (int q = 0; q < nj; ++q) {
        const int j = order[q];
        const gbpf_job& J = jobs[j];
        gbpf_solver* s = J.solver;
        const int G = job_slots_of(J);
        Shape* sh = nullptr;
        if (int rc = get_shape(s, NT, G, &sh)) return rc;
        occ = std::min(occ, sh->occ);
        gbpf::Job& o = hj[q];
        o.P = sh->dp;
        Shape* sh1 = sh;
        if (G > 1)
            if (int rc = get_shape(s, NT, 1, &sh1)) return rc;
        o.P1 = sh1->dp;
        o.off = solver_offsets(s, G, mixed);
        o.G = G;
        o.log2G = ilog2(G);
        o.seq = q;
        cta_bytes = std::max(cta_bytes, o.off.total);
        want += (J.n_cases + G - 1) / G;
        gbpf::Batch b{};
        b.B = J.n_cases;
        b.S = reinterpret_cast<const double2*>(J.S);
        b.s_shared = !J.s_per_col;
        b.sS = J.n_cases;
        b.V0 = reinterpret_cast<const double2*>(J.V0);
        b.v0_shared = !J.v0_per_col;
        b.sV0 = J.n_cases;
        if (b.v0_shared) {
            b.v0tab = reinterpret_cast<double4_32a*>(g->btab.as<char>() + tab_at);
            tab_at += up256((size_t)s->n * 64);
        }
        if (shares(J)) {
            Shape* s1 = nullptr;
            if (int rc = get_shape(s, 1024, 1, &s1)) return rc;
            gbpf::StartJob sj{};
            sj.P = s1->dp;
            sj.v0tab = b.v0tab;
            sj.mixed = mixed;
            sj.log2G = ilog2(G);
            gbpf::start_carve(sj, g->btab.as<char>() + tab_at, s->n, s->plan.nv, s->plan.nblk, G, mixed);
            tab_at += up256(gbpf::start_bytes(s->n, s->plan.nv, s->plan.nblk, G, mixed));
            b.R0 = sj.R0;
            b.fac0 = sj.facG;
            b.ok0 = sj.ok0;
            hs.push_back(sj);
            hs_batch.push_back(q);
        }
        if (J.pin) {
            b.pin = J.pin;
            b.spin = J.n_cases;
        }
        if (J.st_ptr) {
            b.ymode = 1;
            b.st_ptr = J.st_ptr;
            b.st_k = J.st_k;
            b.st_v = reinterpret_cast<const double2*>(J.st_val);
        }
        unsigned long long* c = ctl + (size_t)q * 32;
        if (J.out_ptr) {  // outage cases: islands on the device, stamps from the branch table
            const size_t n = s->n, L = J.n_cases;
            char* base = g->bisl.as<char>() + isl_at;
            IslLaunch il{};
            il.s = s;
            il.J = &J;
            il.labels = reinterpret_cast<int*>(base);
            il.ref_bus = reinterpret_cast<int*>(base + up256(n * L * 4));
            il.served_i = reinterpret_cast<int*>(base + 2 * up256(n * L * 4));
            il.nis = reinterpret_cast<int*>(base + 3 * up256(n * L * 4));
            il.grid = (int)std::min<size_t>(L, 4 * (size_t)g->nsm);
            il.scr = reinterpret_cast<int*>(base + 3 * up256(n * L * 4) + up256(L * 4));
            il.best = reinterpret_cast<unsigned long long*>(base + 3 * up256(n * L * 4) + up256(L * 4) +
                                                            up256((size_t)il.grid * 4 * n * 4));
            il.err = reinterpret_cast<int*>(c + 24) + 6;
            isl_at += 3 * up256(n * L * 4) + up256(L * 4) + up256((size_t)il.grid * 4 * n * 4) +
                      up256((size_t)il.grid * n * 8);
            isl.push_back(il);
            b.ymode = 3;
            b.out_ptr = J.out_ptr;
            b.out_idx = J.out_idx;
            b.ref_bus = il.ref_bus;
            b.sref = (long long)L;
        }
        b.Vout = reinterpret_cast<double2*>(J.V);
        b.sV = J.n_cases;
        b.iters = J.iterations;
        b.conv = J.converged;
        fill_common(b, s, p);
        b.counter = reinterpret_cast<int*>(c + 16);
        b.stats = c;
        b.err = reinterpret_cast<int*>(c + 24);
        o.B = b;
    }
    for (size_t k = 0; k < hs.size(); ++k) {
        const gbpf::Batch& b = hj[hs_batch[k]].B;
        hs[k].rcond_min = mixed ? b.rcond_min32 : b.rcond_min64;
    }
    const int grid = grid_size(g->nsm, occ, want, mixed);
    CK(g->scr.ensure((size_t)grid * cta_bytes));
    const size_t jobs_bytes = up256((size_t)nj * sizeof(gbpf::Job));
    CK(g->bjobs.ensure(jobs_bytes + hs.size() * sizeof(gbpf::StartJob)));
    CK(cudaMemcpyAsync(g->bjobs.p, hj.data(), (size_t)nj * sizeof(gbpf::Job), cudaMemcpyHostToDevice, g->stream));
    if (!hs.empty())
        CK(cudaMemcpyAsync(g->bjobs.as<char>() + jobs_bytes, hs.data(), hs.size() * sizeof(gbpf::StartJob),
                           cudaMemcpyHostToDevice, g->stream));
    gbpf::Launch L{};
    L.jobs = g->bjobs.as<gbpf::Job>();
    L.njobs = nj;
    L.scratch = g->scr.as<char>();
    L.cta_bytes = cta_bytes;
    CK(cudaEventRecord(g->e0, g->stream));
    for (int q = 0; q < nj; ++q) {
        const gbpf::Batch& b = hj[q].B;
        if (b.v0_shared)
            CK(gbpf::launch_v0_table(b.V0, hj[q].P.n, b.check_v0, const_cast<double4_32a*>(b.v0tab), b.err,
                                     g->stream));
    }
    if (!hs.empty())
        CK(gbpf::launch_start(reinterpret_cast<const gbpf::StartJob*>(g->bjobs.as<char>() + jobs_bytes),
                              (int)hs.size(), g->stream));
    for (const IslLaunch& il : isl) {
        const gbpf_solver* s = il.s;
        CK(gbpf::launch_islands(s->n, s->m, s->dbr_f.as<int>(), s->dbr_t.as<int>(), s->dbr_live.as<uint8_t>(),
                                il.J->n_cases, il.J->out_ptr, il.J->out_idx, s->dslack.as<uint8_t>(),
                                s->dprio.as<double>(), il.J->reslack, il.scr, il.best, il.labels,
                                reinterpret_cast<uint8_t*>(il.served_i), il.ref_bus, il.nis, il.err, il.grid,
                                g->stream));
        if (il.J->served)
            CK(cudaMemcpyAsync(il.J->served, il.served_i, (size_t)s->n * il.J->n_cases, cudaMemcpyDeviceToDevice,
                               g->stream));
    }
    CK(gbpf::launch_newton(L, grid, NT, g->stream));
    CK(cudaEventRecord(g->e1, g->stream));
    std::vector<unsigned long long> hc((size_t)nj * 32);
    CK(cudaMemcpyAsync(hc.data(), ctl, hc.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, g->e0, g->e1));
    gbpf_stats st{};
    for (int q = 0; q < nj; ++q) {
        const unsigned long long* c = hc.data() + (size_t)q * 32;
        st.single_factorizations += c[0];
        st.double_factorizations += c[1];
        st.single_rejected += c[2];
        st.double_rejected += c[3];
        st.macro_steps += c[4];
        st.chord_steps += c[5];
        st.first_steps += c[6];
        st.lazy_jacobians += c[14];
        st.jacobian_sweeps += c[7];
    }
    st.grid = grid;
    st.cases_per_cta = Gmax;
    st.threads_per_cta = NT;
    st.kernel_ms = ms;
    g->last = st;
    for (int q = 0; q < nj; ++q) {
        const int* err = reinterpret_cast<const int*>(hc.data() + (size_t)q * 32 + 24);
        const std::string job = std::string(who) + ": job " + std::to_string(order[q]) + ": ";
        if (err[0] == gbpf::DE_V0_NONFINITE)
            return fail(job + "invalid initial voltage at bus " + std::to_string(err[1]) + ", step " +
                        std::to_string(err[2]));
        if (err[0] == gbpf::DE_V0_MAGNITUDE)
            return fail(job + "invalid voltage magnitude at bus " + std::to_string(err[1]) + ", step " +
                        std::to_string(err[2]));
        if (err[0] == gbpf::DE_STAMPS)
            return fail(job + "case " + std::to_string(err[2]) + " has " + std::to_string(err[1]) +
                        " outage stamp entries, more than the " + std::to_string(gbpf::MAX_STAMPS) + " supported");
        if (err[0] == gbpf::DE_OUTAGE)
            return fail(job + "case " + std::to_string(err[2]) + " outages branch " + std::to_string(err[1]) +
                        ", which does not exist");
        if (err[6]) return fail(job + "island labels did not settle");
    }
    return 0;
}

}  // namespace

// =============================================================================== C ABI
extern "C" {

const char* gbpf_last_error(void) { return g_err.c_str(); }

int gbpf_version(void) { return 100; }

int gbpf_device_count(void) {
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return c;
}

gbpf_solver* gbpf_create(int n, const int32_t* Yp, const int32_t* Yj, const double* Yx, int nnz, const int32_t* pv,
                         int npv, const int32_t* pq, int npq, int cases_per_cta) {
    return gbpf_create_ex(n, Yp, Yj, Yx, nnz, pv, npv, pq, npq, cases_per_cta, 0);
}

gbpf_solver* gbpf_create_ex(int n, const int32_t* Yp, const int32_t* Yj, const double* Yx, int nnz,
                            const int32_t* pv, int npv, const int32_t* pq, int npq, int cases_per_cta,
                            int threads_per_cta) {
    if (n <= 0 || !Yp || (nnz > 0 && (!Yj || !Yx)) || npv < 0 || npq < 0) {
        fail("gbpf_create: invalid arguments");
        return nullptr;
    }
    std::unique_ptr<gbpf_solver> s(new gbpf_solver);
    s->n = n;
    s->nnz = nnz;
    s->Yp.assign(Yp, Yp + n + 1);
    s->Yj.assign(Yj, Yj + nnz);
    s->Yx.assign(Yx, Yx + 2 * (size_t)nnz);
    if (setup(s.get(), cases_per_cta, threads_per_cta)) return nullptr;
    std::string e = gbpf::build_plan(s->plan, n, Yp, Yj, nnz, pv, npv, pq, npq, 1);
    if (!e.empty()) {
        fail("gbpf_create: " + e);
        return nullptr;
    }
    if (compute_rcond0(s.get())) return nullptr;
    if (upload_plan(s.get())) return nullptr;
    return s.release();
}

void gbpf_destroy(gbpf_solver* s) { delete s; }

int gbpf_update_Y(gbpf_solver* s, const double* Yx, int nnz) {
    if (!s) return fail("null solver");
    if (nnz != s->nnz) return fail("update_Y: nnz mismatch (topology changed; rebuild Solver)");
    s->Yx.assign(Yx, Yx + 2 * (size_t)nnz);
    if (int rc = compute_rcond0(s)) return rc;
    return upload_values(s);
}

int gbpf_get_info(gbpf_solver* s, gbpf_info* o) {
    if (!s || !o) return fail("null argument");
    const gbpf::Plan& p = s->plan;
    o->n_bus = p.n;
    o->nnz_ybus = p.nnzY;
    o->n_var_bus = p.nv;
    o->n_blocks = p.nblk;
    o->n_levels = p.nlev;
    o->n_back_levels = p.nblev;
    int NT = 0, G = 0;  // the shape of a batch that fills the device
    choose_shape(s, 1LL << 40, &NT, &G);
    o->cases_per_cta = G;
    o->threads_per_cta = NT;
    o->workers = NT / G;
    o->factor_pairs = p.n_factor_pairs;
    o->forward_pairs = p.n_fwd_pairs;
    o->backward_pairs = p.n_bwd_pairs;
    o->rcond0 = p.rcond0;
    o->jinv_norm = p.jinv_est;
    return 0;
}

int gbpf_prepare_shapes(gbpf_solver* s, int max_cases_per_cta) {
    if (!s) return fail("null solver");
    const int cap = std::max(1, std::min(gbpf::MAX_SLOTS, max_cases_per_cta));
    for (int NT : {1024, 512})
        for (int G = 1; G <= (NT == 1024 ? std::min(cap, 4) : cap); G *= 2) {  // 1,024 threads: <= 4 slots
            Shape* sh = nullptr;
            if (int rc = get_shape(s, NT, G, &sh)) return rc;
        }
    return 0;
}

int gbpf_get_shape(gbpf_solver* s, long long units, int* threads_per_cta, int* cases_per_cta) {
    if (!s || !threads_per_cta || !cases_per_cta) return fail("null argument");
    if (units <= 0) return fail("get_shape: units must be > 0");
    choose_shape(s, units, threads_per_cta, cases_per_cta);
    return 0;
}

int gbpf_set_shape(gbpf_solver* s, long long units, int threads_per_cta, int cases_per_cta) {
    if (!s) return fail("null solver");
    if (units <= 0) return fail("set_shape: units must be > 0");
    const int c = size_class(units);
    if (threads_per_cta == 0 && cases_per_cta == 0) {
        s->table_NT[c] = s->table_G[c] = 0;
        return 0;
    }
    if (threads_per_cta != 256 && threads_per_cta != 512 && threads_per_cta != 1024)
        return fail("set_shape: threads_per_cta must be 256, 512 or 1024");
    if (cases_per_cta < 1 || cases_per_cta > gbpf::MAX_SLOTS || (cases_per_cta & (cases_per_cta - 1)))
        return fail("set_shape: cases_per_cta must be a power of two in 1..32");
    s->table_NT[c] = threads_per_cta;
    s->table_G[c] = cases_per_cta;
    return 0;
}

int gbpf_set_chain_cap(gbpf_solver* s, double chain_cap) {
    if (!s) return fail("null solver");
    if (!(chain_cap >= 0.0) || !std::isfinite(chain_cap)) return fail("set_chain_cap: chain_cap must be finite and >= 0");
    std::lock_guard<std::mutex> lock(s->shapes_mu);
    s->chain_cap = chain_cap;  // shapes of other caps stay built: launches may still hold them
    return 0;
}

int gbpf_get_mismatch(gbpf_solver* s, double* out, long long n) {
    if (!s || !out) return fail("get_mismatch: null argument");
    if (s->mis_n <= 0) return fail("get_mismatch: no synchronous solve recorded its cases' mismatch");
    if (n != s->mis_n)
        return fail("get_mismatch: the last call solved " + std::to_string(s->mis_n) + " cases, not " +
                    std::to_string(n));
    CK(cudaMemcpyAsync(out, s->bmis.p, (size_t)n * 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return 0;
}

int gbpf_get_stats(gbpf_solver* s, gbpf_stats* o) {
    if (!s || !o) return fail("null argument");
    *o = s->last;
    return 0;
}

int gbpf_get_Y(gbpf_solver* s, double* Yx) {
    if (!s || !Yx) return fail("null argument");
    std::copy(s->Yx.begin(), s->Yx.end(), Yx);
    return 0;
}

int gbpf_get_posmap(gbpf_solver* s, int32_t* out) {
    if (!s || !out) return fail("null argument");
    std::copy(s->plan.posmap.begin(), s->plan.posmap.end(), out);
    return 0;
}

int gbpf_get_row_of_bus(gbpf_solver* s, int32_t* out) {
    if (!s || !out) return fail("null argument");
    std::copy(s->plan.row_of_bus.begin(), s->plan.row_of_bus.end(), out);
    return 0;
}

int gbpf_solve_batch_device(gbpf_solver* s, int T, const double* dS, int s_per_col, const double* dV0,
                            int v0_per_col, const gbpf_params* pp, double* dV, int32_t* dit, uint8_t* dcv) {
    if (!s) return fail("null solver");
    const gbpf_params p = pp ? *pp : default_params();
    if (T <= 0) return fail("solve_batch: T (time steps) must be > 0");
    if (int rc = check_params(p, "solve_batch")) return rc;
    gbpf::Batch b{};
    b.B = T;
    b.S = reinterpret_cast<const double2*>(dS);
    b.s_shared = !s_per_col;
    b.sS = T;
    b.V0 = reinterpret_cast<const double2*>(dV0);
    b.v0_shared = !v0_per_col;
    b.sV0 = T;
    b.ymode = 0;
    b.Vout = reinterpret_cast<double2*>(dV);
    b.sV = T;
    b.iters = dit;
    b.conv = dcv;
    fill_common(b, s, p);
    return run(s, b, T, "solve_batch");
}

int gbpf_solve_batch(gbpf_solver* s, int T, const double* S, int s_per_col, const double* V0, int v0_per_col,
                     const gbpf_params* pp, double* V, int32_t* it, uint8_t* cv) {
    if (!s) return fail("null solver");
    if (T <= 0) return fail("solve_batch: T (time steps) must be > 0");
    const size_t n = s->n;
    const size_t sb = n * (s_per_col ? T : 1) * 16, vb = n * (v0_per_col ? T : 1) * 16, ob = n * (size_t)T * 16;
    CK(s->bS.ensure(sb));
    CK(s->bV0.ensure(vb));
    CK(s->bV.ensure(ob));
    CK(s->bit.ensure((size_t)T * 4));
    CK(s->bcv.ensure((size_t)T));
    CK(cudaEventRecord(s->c0, s->stream));
    CK(cudaMemcpyAsync(s->bS.p, S, sb, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->bV0.p, V0, vb, cudaMemcpyHostToDevice, s->stream));
    if (int rc = gbpf_solve_batch_device(s, T, s->bS.as<double>(), s_per_col, s->bV0.as<double>(), v0_per_col, pp,
                                         s->bV.as<double>(), s->bit.as<int32_t>(), s->bcv.as<uint8_t>()))
        return rc;
    CK(cudaMemcpyAsync(V, s->bV.p, ob, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(it, s->bit.p, (size_t)T * 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(cv, s->bcv.p, (size_t)T, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaEventRecord(s->c1, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return record_call(s);
}

int gbpf_solve_lanes_device(gbpf_solver* s, int T, const double* dS, const double* dV0, int K, const int64_t* doff,
                            const gbpf_params* pp, double* dV, int32_t* dit, uint8_t* dcv) {
    if (!s) return fail("null solver");
    const gbpf_params p = pp ? *pp : default_params();
    if (T <= 0) return fail("solve_lanes: T (time steps) must be > 0");
    if (K <= 0) return fail("solve_lanes: K (lanes) must be > 0");
    if (int rc = check_params(p, "solve_lanes")) return rc;
    gbpf::Batch b{};
    b.B = T;
    b.lanes = 1;
    b.K = K;
    b.lane_off = reinterpret_cast<const long long*>(doff);
    b.S = reinterpret_cast<const double2*>(dS);
    b.s_shared = 0;
    b.sS = T;
    b.V0 = reinterpret_cast<const double2*>(dV0);
    b.v0_shared = 1;
    b.sV0 = 0;
    b.ymode = 0;
    b.Vout = reinterpret_cast<double2*>(dV);
    b.sV = T;
    b.iters = dit;
    b.conv = dcv;
    fill_common(b, s, p);
    return run(s, b, K, "solve_lanes");
}

int gbpf_solve_lanes(gbpf_solver* s, int T, const double* S, const double* V0, int K, const int64_t* off,
                     const gbpf_params* pp, double* V, int32_t* it, uint8_t* cv) {
    if (!s) return fail("null solver");
    if (T <= 0 || K <= 0) return fail("solve_lanes: T and K must be > 0");
    if (off[0] != 0 || off[K] != T) return fail("solve_lanes: offsets must start at 0 and end at T");
    for (int l = 0; l < K; ++l)
        if (off[l + 1] < off[l]) return fail("solve_lanes: offsets must be non-decreasing");
    const size_t n = s->n;
    const size_t sb = n * (size_t)T * 16, vb = n * 16;
    CK(s->bS.ensure(sb));
    CK(s->bV0.ensure(vb));
    CK(s->bV.ensure(sb));
    CK(s->bit.ensure((size_t)T * 4));
    CK(s->bcv.ensure((size_t)T));
    CK(s->blane.ensure((size_t)(K + 1) * 8));
    CK(cudaEventRecord(s->c0, s->stream));
    CK(cudaMemcpyAsync(s->bS.p, S, sb, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->bV0.p, V0, vb, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->blane.p, off, (size_t)(K + 1) * 8, cudaMemcpyHostToDevice, s->stream));
    if (int rc = gbpf_solve_lanes_device(s, T, s->bS.as<double>(), s->bV0.as<double>(), K, s->blane.as<int64_t>(), pp,
                                         s->bV.as<double>(), s->bit.as<int32_t>(), s->bcv.as<uint8_t>()))
        return rc;
    CK(cudaMemcpyAsync(V, s->bV.p, sb, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(it, s->bit.p, (size_t)T * 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(cv, s->bcv.p, (size_t)T, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaEventRecord(s->c1, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return record_call(s);
}

int gbpf_solve_lanes_async(gbpf_solver* s, int slot, int T, const double* S, const double* V0, int K,
                           const int64_t* off, const gbpf_params* pp, double* V, int32_t* it, uint8_t* cv) {
    if (!s) return fail("null solver");
    if (slot < 0 || slot >= 8) return fail("solve_lanes_async: slot must be in 0..7");
    if (T <= 0 || K <= 0) return fail("solve_lanes_async: T and K must be > 0");
    if (off[0] != 0 || off[K] != T) return fail("solve_lanes_async: offsets must start at 0 and end at T");
    for (int l = 0; l < K; ++l)
        if (off[l + 1] < off[l]) return fail("solve_lanes_async: offsets must be non-decreasing");
    const gbpf_params p = pp ? *pp : default_params();
    if (int rc = check_params(p, "solve_lanes_async")) return rc;
    while ((int)s->slots.size() <= slot) {
        std::unique_ptr<ExecSlot> x(new ExecSlot);
        CK(cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking));
        CK(cudaEventCreate(&x->e0));
        CK(cudaEventCreate(&x->e1));
        CK(cudaEventCreate(&x->c0));
        CK(cudaEventCreate(&x->c1));
        CK(cudaMallocHost(&x->host_ctl, 32 * sizeof(unsigned long long)));
        s->slots.push_back(std::move(x));
    }
    ExecSlot& X = *s->slots[slot];
    if (X.pending) return fail("solve_lanes_async: slot " + std::to_string(slot) + " is still in flight (wait for it first)");
    s->mis_n = 0;  // asynchronous calls record no per-case mismatch
    const size_t n = s->n;
    const size_t sb = n * (size_t)T * 16, vb = n * 16;
    CK(X.bS.ensure(sb));
    CK(X.bV0.ensure(vb));
    CK(X.bV.ensure(sb));
    CK(X.bit.ensure((size_t)T * 4));
    CK(X.bcv.ensure((size_t)T));
    CK(X.blane.ensure((size_t)(K + 1) * 8));
    CK(cudaEventRecord(X.c0, X.stream));
    CK(cudaMemcpyAsync(X.bS.p, S, sb, cudaMemcpyHostToDevice, X.stream));
    CK(cudaMemcpyAsync(X.bV0.p, V0, vb, cudaMemcpyHostToDevice, X.stream));
    CK(cudaMemcpyAsync(X.blane.p, off, (size_t)(K + 1) * 8, cudaMemcpyHostToDevice, X.stream));
    gbpf::Batch b{};
    b.B = T;
    b.lanes = 1;
    b.K = K;
    b.lane_off = X.blane.as<long long>();
    b.S = X.bS.as<double2>();
    b.sS = T;
    b.V0 = X.bV0.as<double2>();
    b.v0_shared = 1;
    b.Vout = X.bV.as<double2>();
    b.sV = T;
    b.iters = X.bit.as<int32_t>();
    b.conv = X.bcv.as<uint8_t>();
    fill_common(b, s, p);
    LaunchRes R{X.stream, X.e0, X.e1, &X.scr, &X.bctl, &X.btab, &X.bjobs, X.host_ctl};
    if (int rc = enqueue_launch(s, R, b, K, "solve_lanes_async", &X.grid, &X.G, &X.NT)) return rc;
    CK(cudaMemcpyAsync(V, X.bV.p, sb, cudaMemcpyDeviceToHost, X.stream));
    CK(cudaMemcpyAsync(it, X.bit.p, (size_t)T * 4, cudaMemcpyDeviceToHost, X.stream));
    CK(cudaMemcpyAsync(cv, X.bcv.p, (size_t)T, cudaMemcpyDeviceToHost, X.stream));
    CK(cudaEventRecord(X.c1, X.stream));
    X.pending = true;
    return 0;
}

int gbpf_solve_wait(gbpf_solver* s, int slot) {
    if (!s) return fail("null solver");
    if (slot < 0 || slot >= (int)s->slots.size() || !s->slots[slot]->pending)
        return fail("solve_wait: nothing in flight in slot " + std::to_string(slot));
    ExecSlot& X = *s->slots[slot];
    X.pending = false;
    CK(cudaStreamSynchronize(X.stream));
    LaunchRes R{X.stream, X.e0, X.e1, &X.scr, &X.bctl, &X.btab, &X.bjobs, X.host_ctl};
    if (int rc = finish_launch(R, X.grid, X.G, X.NT, "solve_lanes_async", &s->last)) return rc;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, X.c0, X.c1));
    s->last.call_ms = ms;
    return 0;
}

int gbpf_solve_contingency(gbpf_solver* s, int L, const double* S, const double* V0, const uint8_t* pin,
                           const double* Yd, const int32_t* st_ptr, const int32_t* st_k, const double* st_val,
                           const gbpf_params* pp, double* V, int32_t* it, uint8_t* cv) {
    if (!s) return fail("null solver");
    const gbpf_params p = pp ? *pp : default_params();
    if (L <= 0) return fail("solve_batch_contingency: no cases");
    if (int rc = check_params(p, "solve_batch_contingency")) return rc;
    const size_t n = s->n, nnz = s->nnz;
    CK(s->bS.ensure(n * 16));
    CK(s->bV0.ensure(n * (size_t)L * 16));
    CK(s->bV.ensure(n * (size_t)L * 16));
    CK(s->bit.ensure((size_t)L * 4));
    CK(s->bcv.ensure((size_t)L));
    CK(cudaMemcpyAsync(s->bS.p, S, n * 16, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->bV0.p, V0, n * (size_t)L * 16, cudaMemcpyHostToDevice, s->stream));
    gbpf::Batch b{};
    b.B = L;
    b.S = s->bS.as<double2>();
    b.s_shared = 1;
    b.V0 = s->bV0.as<double2>();
    b.v0_shared = 0;
    b.sV0 = L;
    if (pin) {
        CK(s->bpin.ensure(n * (size_t)L));
        CK(cudaMemcpyAsync(s->bpin.p, pin, n * (size_t)L, cudaMemcpyHostToDevice, s->stream));
        b.pin = s->bpin.as<uint8_t>();
        b.spin = L;
    }
    if (Yd) {
        CK(s->bYd.ensure(nnz * (size_t)L * 16));
        CK(cudaMemcpyAsync(s->bYd.p, Yd, nnz * (size_t)L * 16, cudaMemcpyHostToDevice, s->stream));
        b.ymode = 2;
        b.Yd = s->bYd.as<double2>();
        b.sYd = L;
    } else if (st_ptr) {
        const int ne = st_ptr[L];
        for (int c = 0; c < L; ++c)
            if (st_ptr[c + 1] - st_ptr[c] > gbpf::MAX_STAMPS)
                return fail("solve_batch_contingency_stamp: case " + std::to_string(c) + " has more than " +
                            std::to_string(gbpf::MAX_STAMPS) + " stamp entries");
        for (int e = 0; e < ne; ++e)
            if (st_k[e] < 0 || st_k[e] >= (int)nnz) return fail("solve_batch_contingency_stamp: stamp row out of range");
        CK(s->bstp.ensure((size_t)(L + 1) * 4));
        CK(s->bstk.ensure((size_t)std::max(ne, 1) * 4));
        CK(s->bstv.ensure((size_t)std::max(ne, 1) * 16));
        CK(cudaMemcpyAsync(s->bstp.p, st_ptr, (size_t)(L + 1) * 4, cudaMemcpyHostToDevice, s->stream));
        if (ne) {
            CK(cudaMemcpyAsync(s->bstk.p, st_k, (size_t)ne * 4, cudaMemcpyHostToDevice, s->stream));
            CK(cudaMemcpyAsync(s->bstv.p, st_val, (size_t)ne * 16, cudaMemcpyHostToDevice, s->stream));
        }
        b.ymode = 1;
        b.st_ptr = s->bstp.as<int>();
        b.st_k = s->bstk.as<int>();
        b.st_v = s->bstv.as<double2>();
    }
    b.Vout = s->bV.as<double2>();
    b.sV = L;
    b.iters = s->bit.as<int32_t>();
    b.conv = s->bcv.as<uint8_t>();
    fill_common(b, s, p);
    if (int rc = run(s, b, L, "solve_batch_contingency")) return rc;
    CK(cudaMemcpyAsync(V, s->bV.p, n * (size_t)L * 16, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(it, s->bit.p, (size_t)L * 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(cv, s->bcv.p, (size_t)L, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return 0;
}

static int ensure_gather(gbpf_solver* s);

int gbpf_dc_start_batch(gbpf_solver* s, int T, const double* Pinj, const double* V0, const double* dc_stamps,
                        double* Vout, uint8_t* used) {
    if (!s || !Pinj || !V0 || !Vout) return fail("dc_start: null argument");
    if (T <= 0) return fail("dc_start: T must be > 0");
    if (dc_stamps && !s->m) return fail("dc_start: DC branch stamps need the branch table (gbpf_set_branches)");
    const size_t n = s->n, nb = s->plan.nblk, nv = std::max(1, s->plan.nv), nnz = s->nnz;
    Shape* sh = nullptr;
    if (int rc = get_shape(s, 1024, 1, &sh)) return rc;
    int dev = 0, nsm = 1;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int grid = std::max(1, std::min(T - 1, 2 * nsm));
    std::vector<double> th(n * (size_t)T);
    std::vector<double> th0(n);
    for (size_t i = 0; i < n; ++i) th0[i] = std::atan2(V0[2 * i + 1], V0[2 * i]);
    DBuf dP, dth, dfac, dR, dy, dout, dpiv, dB, dst, dsh;
    auto cleanup = [&]() {
        for (DBuf* b : {&dP, &dth, &dfac, &dR, &dy, &dout, &dpiv, &dB, &dst, &dsh}) b->release();
    };
    struct Guard {
        std::function<void()> f;
        ~Guard() { f(); }
    } guard{cleanup};
    const double2* Bx = nullptr;
    if (dc_stamps) {  // the DC stamps summed onto the Ybus pattern like the AC ones (COO order)
        if (int rc = ensure_gather(s)) return rc;
        CK(dst.ensure(64 * (size_t)s->m));
        CK(dsh.ensure(16 * n));
        CK(dB.ensure(16 * nnz));
        CK(cudaMemcpyAsync(dst.p, dc_stamps, 64 * (size_t)s->m, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemsetAsync(dsh.p, 0, 16 * n, s->stream));
        CK(gbpf::launch_ybus_gather((int)nnz, 4 * s->m, s->dg_ptr.as<int>(), s->dg_src.as<int>(), dst.as<double2>(),
                                    dsh.as<double2>(), dB.as<double2>(), nullptr, s->stream));
        Bx = dB.as<double2>();
    }
    CK(dP.ensure(n * 8 * T));
    CK(dth.ensure(n * 8));
    CK(dfac.ensure((nb + nv) * 32));
    CK(dR.ensure(nv * 16 * grid));
    CK(dy.ensure(nv * 16 * grid));
    CK(dout.ensure(n * 8 * T));
    CK(dpiv.ensure(16));
    CK(cudaMemcpyAsync(dP.p, Pinj, n * 8 * T, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(dth.p, th0.data(), n * 8, cudaMemcpyHostToDevice, s->stream));
    CK(gbpf::launch_dc(sh->dp, Bx, dP.as<double>(), T, dth.as<double>(), dfac.as<double4_32a>(), dR.as<double2>(),
                       dy.as<double2>(), dout.as<double>(), dpiv.as<unsigned long long>(), grid, s->stream));
    unsigned long long piv[2];
    CK(cudaMemcpyAsync(th.data(), dout.p, n * 8 * T, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(piv, dpiv.p, 16, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    // a zero or non-finite pivot (a DC island without a reference) or non-finite angles:
    // the case keeps the flat start (timeseries.py:244-247)
    double mn, mx;
    std::memcpy(&mn, &piv[0], 8);
    std::memcpy(&mx, &piv[1], 8);
    const bool piv_ok = std::isfinite(mx) && mn > 0.0;
    bool all = true;
    for (int c = 0; c < T; ++c) {
        bool ok = piv_ok;
        for (size_t i = 0; i < n && ok; ++i) ok = std::isfinite(th[i * T + c]);
        all = all && ok;
        if (used) used[c] = ok ? 1 : 0;
        for (size_t i = 0; i < n; ++i) {
            const size_t o = 2 * (i * T + c);
            if (!ok || s->plan.row_of_bus[i] < 0) {
                Vout[o] = V0[2 * i];
                Vout[o + 1] = V0[2 * i + 1];
            } else {
                const double vm = std::hypot(V0[2 * i], V0[2 * i + 1]);
                Vout[o] = vm * std::cos(th[i * T + c]);
                Vout[o + 1] = vm * std::sin(th[i * T + c]);
            }
        }
    }
    return all ? 0 : 1;
}

int gbpf_dc_start(gbpf_solver* s, const double* Pinj, const double* V0, double* Vout) {
    return gbpf_dc_start_batch(s, 1, Pinj, V0, nullptr, Vout, nullptr);
}

int gbpf_eval_jacobian(gbpf_solver* s, const double* S, const double* V, const uint8_t* pin, double* blocks,
                       double* residual) {
    if (!s) return fail("null solver");
    const size_t n = s->n, nb = s->plan.nblk, nv = std::max(1, s->plan.nv);
    DBuf dV, dSb, dpin, dVt, dEt, dEi, div32, dblk, dR;
    auto cleanup = [&]() {
        for (DBuf* b : {&dV, &dSb, &dpin, &dVt, &dEt, &dEi, &div32, &dblk, &dR}) b->release();
    };
    struct Guard {
        std::function<void()> f;
        ~Guard() { f(); }
    } guard{cleanup};
    CK(dV.ensure(n * 16));
    CK(dSb.ensure(n * 16));
    CK(dVt.ensure(n * 32));
    CK(dEt.ensure(n * 16));
    CK(dEi.ensure(n * 8));
    CK(div32.ensure(n * 4));
    CK(dblk.ensure(nb * 32));
    CK(dR.ensure(nv * 16));
    CK(cudaMemcpy(dV.p, V, n * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dSb.p, S, n * 16, cudaMemcpyHostToDevice));
    CK(cudaMemset(dblk.p, 0, nb * 32));
    CK(cudaMemset(dR.p, 0, nv * 16));
    if (pin) {
        CK(dpin.ensure(n));
        CK(cudaMemcpy(dpin.p, pin, n, cudaMemcpyHostToDevice));
    }
    CK(gbpf::launch_eval_debug(s->dp, dV.as<double2>(), dSb.as<double2>(), pin ? dpin.as<uint8_t>() : nullptr,
                               dVt.as<double4_32a>(), dEt.as<double2>(), dEi.as<double>(), div32.as<float>(),
                               dblk.as<double4_32a>(),
                               dR.as<double2>(), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpy(blocks, dblk.p, nb * 32, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(residual, dR.p, (size_t)s->plan.nv * 16, cudaMemcpyDeviceToHost));
    return 0;
}

int gbpf_selftest_conversions(const double* in, int n, float* d2f, double* f2d, float* d2f_small) {
    if (n <= 0) return 0;
    DBuf a, b, c, d;
    CK(a.ensure((size_t)n * 8));
    CK(b.ensure((size_t)n * 4));
    CK(c.ensure((size_t)n * 8));
    CK(d.ensure((size_t)n * 4));
    CK(cudaMemcpy(a.p, in, (size_t)n * 8, cudaMemcpyHostToDevice));
    CK(gbpf::launch_conversions(a.as<double>(), n, b.as<float>(), c.as<double>(), d.as<float>()));
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(d2f, b.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(f2d, c.p, (size_t)n * 8, cudaMemcpyDeviceToHost));
    if (d2f_small) CK(cudaMemcpy(d2f_small, d.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
    a.release();
    b.release();
    c.release();
    d.release();
    return 0;
}

int gbpf_selftest_math(const double* in, int n, double* recip, double* s_small, double* c_small, double* s_ref,
                       double* c_ref, const double* phasor, double* rot) {
    if (n <= 0) return 0;
    DBuf a, b, c;
    CK(a.ensure((size_t)n * 8));
    CK(b.ensure((size_t)n * 8 * 9));
    CK(c.ensure(16));
    double* o = b.as<double>();
    CK(cudaMemcpy(a.p, in, (size_t)n * 8, cudaMemcpyHostToDevice));
    if (phasor) CK(cudaMemcpy(c.p, phasor, 16, cudaMemcpyHostToDevice));
    CK(gbpf::launch_math(a.as<double>(), n, o, o + n, o + 2 * (size_t)n, o + 3 * (size_t)n, o + 4 * (size_t)n,
                         phasor ? c.as<double>() : nullptr, o + 5 * (size_t)n));
    CK(cudaDeviceSynchronize());
    double* outs[5] = {recip, s_small, c_small, s_ref, c_ref};
    for (int k = 0; k < 5; ++k) CK(cudaMemcpy(outs[k], o + k * (size_t)n, (size_t)n * 8, cudaMemcpyDeviceToHost));
    if (phasor && rot) CK(cudaMemcpy(rot, o + 5 * (size_t)n, (size_t)n * 32, cudaMemcpyDeviceToHost));
    a.release();
    b.release();
    c.release();
    return 0;
}

void* gbpf_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMallocHost(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
        fail("cudaMallocHost failed");
        return nullptr;
    }
    return p;
}

void gbpf_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

int gbpf_set_branches(gbpf_solver* s, int m, const int32_t* f, const int32_t* t, const int32_t* stamp_pos,
                      const double* stamp_val, const uint8_t* is_slack, const double* gen_prio) {
    if (!s) return fail("null solver");
    if (m <= 0 || !f || !t || !stamp_pos || !stamp_val || !is_slack) return fail("set_branches: invalid arguments");
    const int n = s->n;
    std::vector<uint8_t> live(m);
    for (int e = 0; e < m; ++e) {
        if (f[e] < 0 || f[e] >= n || t[e] < 0 || t[e] >= n) return fail("set_branches: branch end out of range");
        for (int q = 0; q < 4; ++q)
            if (stamp_pos[4 * e + q] < 0 || stamp_pos[4 * e + q] >= s->nnz)
                return fail("set_branches: stamp position out of range");
        // a branch couples its ends while its transfer admittances are nonzero
        live[e] = (stamp_val[8 * (size_t)e + 2] != 0.0 || stamp_val[8 * (size_t)e + 3] != 0.0 ||
                   stamp_val[8 * (size_t)e + 4] != 0.0 || stamp_val[8 * (size_t)e + 5] != 0.0);
    }
    std::vector<int> vf(f, f + m), vt(t, t + m), vp(stamp_pos, stamp_pos + 4 * (size_t)m);
    std::vector<double> vv(stamp_val, stamp_val + 8 * (size_t)m);
    std::vector<uint8_t> vs(is_slack, is_slack + n);
    std::vector<double> vprio(n, 0.0);
    if (gen_prio) vprio.assign(gen_prio, gen_prio + n);
    CK(upload(s->dbr_f, vf));
    CK(upload(s->dbr_t, vt));
    CK(upload(s->dbr_live, live));
    CK(upload(s->dbr_pos, vp));
    CK(upload(s->dbr_val, vv));
    CK(upload(s->dslack, vs));
    CK(upload(s->dprio, vprio));
    s->m = m;
    s->br_pos = vp;
    s->gather_ready = false;
    auto fill = [&](gbpf::DevPlan& d) {
        d.m = m;
        d.br_pos = s->dbr_pos.as<int4>();
        d.br_val = s->dbr_val.as<double2>();
        d.is_slack = s->dslack.as<uint8_t>();
    };
    fill(s->dp);
    std::lock_guard<std::mutex> lock(s->shapes_mu);
    for (auto& sh : s->shapes) fill(sh->dp);
    return 0;
}

// Gather lists of the Ybus sum: the contributions of every CSR entry in the order a COO sum of
// the stamps meets them (all Yff, then Yft, Ytf, Ytt, each in branch order; TwoPort.py:133-149),
// the bus shunt last. Built once per branch table.
static int ensure_gather(gbpf_solver* s) {
    if (s->gather_ready) return 0;
    const int m = s->m, n = s->n, nnz = s->nnz;
    std::vector<std::vector<int>> lists(nnz);
    for (int q = 0; q < 4; ++q)
        for (int e = 0; e < m; ++e) lists[s->br_pos[4 * (size_t)e + q]].push_back(4 * e + q);
    for (int i = 0; i < n; ++i)
        if (s->plan.ydiag[i] >= 0) lists[s->plan.ydiag[i]].push_back(4 * m + i);
    std::vector<int> ptr(nnz + 1, 0), src;
    for (int k = 0; k < nnz; ++k) {
        ptr[k + 1] = ptr[k] + (int)lists[k].size();
        src.insert(src.end(), lists[k].begin(), lists[k].end());
    }
    CK(upload(s->dg_ptr, ptr));
    CK(upload(s->dg_src, src));
    s->gather_ready = true;
    return 0;
}

int gbpf_update_Y_from_branches(gbpf_solver* s, const double* stamps, const double* bus_shunt) {
    if (!s || !stamps) return fail("update_Y_from_branches: null argument");
    if (!s->m) return fail("update_Y_from_branches: the branch table is not set (gbpf_set_branches)");
    const int m = s->m, n = s->n, nnz = s->nnz;
    if (int rc = ensure_gather(s)) return rc;
    std::vector<double> sh(2 * (size_t)n, 0.0);
    if (bus_shunt) sh.assign(bus_shunt, bus_shunt + 2 * (size_t)n);
    CK(upload(s->dshunt, sh));
    CK(cudaMemcpyAsync(s->dbr_val.p, stamps, 64 * (size_t)m, cudaMemcpyHostToDevice, s->stream));
    CK(gbpf::launch_ybus_gather(nnz, 4 * m, s->dg_ptr.as<int>(), s->dg_src.as<int>(), s->dbr_val.as<double2>(),
                                s->dshunt.as<double2>(), s->dY.as<double2>(), s->dY32.as<float2>(), s->stream));
    CK(cudaMemcpyAsync(s->Yx.data(), s->dY.p, 16 * (size_t)nnz, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    // branches whose transfer terms vanished (out of service, an open end) no longer couple
    std::vector<uint8_t> live(m);
    for (int e = 0; e < m; ++e)
        live[e] = (stamps[8 * (size_t)e + 2] != 0.0 || stamps[8 * (size_t)e + 3] != 0.0 ||
                   stamps[8 * (size_t)e + 4] != 0.0 || stamps[8 * (size_t)e + 5] != 0.0);
    CK(upload(s->dbr_live, live));
    return compute_rcond0(s);
}

int gbpf_solver_islands(gbpf_solver* s, int m, const int32_t* f, const int32_t* t, const uint8_t* live, int L,
                        const int32_t* out_ptr, const int32_t* out_idx, const uint8_t* is_slack, const double* gen_prio,
                        int reslack, int32_t* labels, uint8_t* served, int32_t* ref_bus, int32_t* n_islands) {
    if (!s) return fail("null solver");
    const int n = s->n;
    if (m < 0 || L <= 0 || !out_ptr || !is_slack || !labels || !served || !ref_bus || !n_islands ||
        (m > 0 && (!f || !t || !live)))
        return fail("solver_islands: invalid arguments");
    for (int e = 0; e < m; ++e)
        if (f[e] < 0 || f[e] >= n || t[e] < 0 || t[e] >= n) return fail("solver_islands: branch end out of range");
    if (out_ptr[0] != 0) return fail("solver_islands: outage pointers must start at 0");
    for (int c = 0; c < L; ++c)
        if (out_ptr[c + 1] < out_ptr[c]) return fail("solver_islands: outage pointers must not decrease");
    const int nout = out_ptr[L];
    for (int q = 0; q < nout; ++q)
        if (out_idx[q] < 0 || out_idx[q] >= m) return fail("solver_islands: outage index out of range");
    const int grid = std::max(1, std::min(L, 4 * s->nsm));
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t nl = (size_t)n * L;
    const size_t b_f = up((size_t)m * 4), b_l = up((size_t)m), b_op = up((size_t)(L + 1) * 4),
                 b_oi = up((size_t)std::max(nout, 1) * 4), b_s = up((size_t)n), b_p = up((size_t)n * 8);
    CK(s->iin.ensure(2 * b_f + b_l + b_op + b_oi + b_s + b_p));
    CK(s->iscr.ensure((size_t)grid * 4 * n * 4));
    CK(s->ibest.ensure((size_t)grid * n * 8));
    const size_t b_lab = up(nl * 4), b_sv = up(nl), b_ni = up((size_t)L * 4);
    CK(s->iout.ensure(2 * b_lab + b_sv + b_ni + 256));
    char* in = s->iin.as<char>();
    int* df = reinterpret_cast<int*>(in);
    int* dt = reinterpret_cast<int*>(in + b_f);
    uint8_t* dl = reinterpret_cast<uint8_t*>(in + 2 * b_f);
    int* dop = reinterpret_cast<int*>(in + 2 * b_f + b_l);
    int* doi = reinterpret_cast<int*>(in + 2 * b_f + b_l + b_op);
    uint8_t* ds = reinterpret_cast<uint8_t*>(in + 2 * b_f + b_l + b_op + b_oi);
    double* dp = reinterpret_cast<double*>(in + 2 * b_f + b_l + b_op + b_oi + b_s);
    char* out = s->iout.as<char>();
    int* dlab = reinterpret_cast<int*>(out);
    int* dref = reinterpret_cast<int*>(out + b_lab);
    uint8_t* dsv = reinterpret_cast<uint8_t*>(out + 2 * b_lab);
    int* dni = reinterpret_cast<int*>(out + 2 * b_lab + b_sv);
    int* derr = reinterpret_cast<int*>(out + 2 * b_lab + b_sv + b_ni);
    cudaStream_t st = s->stream;
    if (m) {
        CK(cudaMemcpyAsync(df, f, (size_t)m * 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dt, t, (size_t)m * 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dl, live, (size_t)m, cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemcpyAsync(dop, out_ptr, (size_t)(L + 1) * 4, cudaMemcpyHostToDevice, st));
    if (nout) CK(cudaMemcpyAsync(doi, out_idx, (size_t)nout * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ds, is_slack, (size_t)n, cudaMemcpyHostToDevice, st));
    if (gen_prio)
        CK(cudaMemcpyAsync(dp, gen_prio, (size_t)n * 8, cudaMemcpyHostToDevice, st));
    else
        CK(cudaMemsetAsync(dp, 0, (size_t)n * 8, st));
    CK(cudaMemsetAsync(derr, 0, 4, st));
    CK(gbpf::launch_islands(n, m, df, dt, dl, L, dop, doi, ds, dp, reslack, s->iscr.as<int>(),
                            s->ibest.as<unsigned long long>(), dlab, dsv, dref, dni, derr, grid, st));
    int kerr = 0;
    CK(cudaMemcpyAsync(&kerr, derr, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(labels, dlab, nl * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(served, dsv, nl, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(ref_bus, dref, nl * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(n_islands, dni, (size_t)L * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (kerr) return fail("solver_islands: label propagation did not settle");
    return 0;
}

gbpf_group* gbpf_group_create(void) {
    std::unique_ptr<gbpf_group> g(new gbpf_group);
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess) fail(std::string("gbpf_group_create: ") + cudaGetErrorString(e));
        return e == cudaSuccess;
    };
    if (!ok(cudaGetDevice(&g->device)) ||
        !ok(cudaDeviceGetAttribute(&g->nsm, cudaDevAttrMultiProcessorCount, g->device)) ||
        !ok(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking)) || !ok(cudaEventCreate(&g->e0)) ||
        !ok(cudaEventCreate(&g->e1)) || !ok(cudaEventCreate(&g->c0)) || !ok(cudaEventCreate(&g->c1)))
        return nullptr;
    return g.release();
}

void gbpf_group_destroy(gbpf_group* g) { delete g; }

int gbpf_group_solve_device(gbpf_group* g, int njobs, const gbpf_job* jobs, const gbpf_params* pp) {
    if (!g || !jobs || njobs <= 0) return fail("group_solve: no jobs");
    const gbpf_params p = pp ? *pp : default_params();
    if (int rc = check_params(p, "group_solve")) return rc;
    return group_run(g, njobs, jobs, p, "group_solve");
}

int gbpf_group_solve(gbpf_group* g, int njobs, const gbpf_job* jobs, const gbpf_params* pp) {
    if (!g || !jobs || njobs <= 0) return fail("group_solve: no jobs");
    const gbpf_params p = pp ? *pp : default_params();
    if (int rc = check_params(p, "group_solve")) return rc;
    // stage every job's inputs in one device buffer and its outputs in another
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    std::vector<size_t> in_at(njobs), out_at(njobs);
    size_t in_bytes = 0, out_bytes = 0;
    for (int j = 0; j < njobs; ++j) {
        const gbpf_job& J = jobs[j];
        if (!J.solver || J.n_cases <= 0) return fail("group_solve: job " + std::to_string(j) + " is empty");
        if (J.st_ptr) {
            const int ne = J.st_ptr[J.n_cases];
            for (int c = 0; c < J.n_cases; ++c)
                if (J.st_ptr[c + 1] - J.st_ptr[c] > gbpf::MAX_STAMPS)
                    return fail("group_solve: job " + std::to_string(j) + " case " + std::to_string(c) +
                                " has more than " + std::to_string(gbpf::MAX_STAMPS) + " stamp entries");
            for (int e = 0; e < ne; ++e)
                if (J.st_k[e] < 0 || J.st_k[e] >= J.solver->nnz)
                    return fail("group_solve: job " + std::to_string(j) + " stamp row out of range");
        }
        const size_t n = J.solver->n, T = J.n_cases;
        in_at[j] = in_bytes;
        in_bytes += up(n * (J.s_per_col ? T : 1) * 16) + up(n * (J.v0_per_col ? T : 1) * 16) + (J.pin ? up(n * T) : 0);
        if (J.st_ptr) in_bytes += up((T + 1) * 4) + up((size_t)std::max(J.st_ptr[T], 1) * 4) +
                                  up((size_t)std::max(J.st_ptr[T], 1) * 16);
        if (J.out_ptr) {
            if (!J.out_idx || J.out_ptr[0] != 0) return fail("group_solve: job " + std::to_string(j) + ": outage pointers must start at 0");
            for (size_t c = 0; c < T; ++c)
                if (J.out_ptr[c + 1] < J.out_ptr[c] || J.out_ptr[c + 1] - J.out_ptr[c] > gbpf::MAX_STAMPS / 4)
                    return fail("group_solve: job " + std::to_string(j) + " case " + std::to_string(c) +
                                ": at most " + std::to_string(gbpf::MAX_STAMPS / 4) + " outaged branches per case");
            for (int e = 0; e < J.out_ptr[T]; ++e)
                if (J.out_idx[e] < 0 || J.out_idx[e] >= J.solver->m)
                    return fail("group_solve: job " + std::to_string(j) + ": outage branch index out of range");
            in_bytes += up((T + 1) * 4) + up((size_t)std::max(J.out_ptr[T], 1) * 4);
        }
        out_at[j] = out_bytes;
        out_bytes += up(n * T * 16) + up(T * 4) + up(T) + (J.served ? up(n * T) : 0);
    }
    CK(g->bin.ensure(in_bytes));
    CK(g->bout.ensure(out_bytes));
    CK(cudaEventRecord(g->c0, g->stream));
    std::vector<gbpf_job> dj(jobs, jobs + njobs);
    for (int j = 0; j < njobs; ++j) {
        const gbpf_job& J = jobs[j];
        gbpf_job& D = dj[j];
        const size_t n = J.solver->n, T = J.n_cases;
        char* at = g->bin.as<char>() + in_at[j];
        auto put = [&](const void* src, size_t bytes) -> void* {
            void* dst = at;
            at += up(bytes);
            if (bytes) g_copy_error = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g->stream);
            return dst;
        };
        g_copy_error = cudaSuccess;
        D.S = static_cast<const double*>(put(J.S, n * (J.s_per_col ? T : 1) * 16));
        CK(g_copy_error);
        D.V0 = static_cast<const double*>(put(J.V0, n * (J.v0_per_col ? T : 1) * 16));
        CK(g_copy_error);
        if (J.pin) {
            D.pin = static_cast<const uint8_t*>(put(J.pin, n * T));
            CK(g_copy_error);
        }
        if (J.st_ptr) {
            const size_t ne = (size_t)J.st_ptr[T];
            D.st_ptr = static_cast<const int32_t*>(put(J.st_ptr, (T + 1) * 4));
            D.st_k = static_cast<const int32_t*>(put(J.st_k, ne * 4));
            D.st_val = static_cast<const double*>(put(J.st_val, ne * 16));
            CK(g_copy_error);
        }
        if (J.out_ptr) {
            D.out_ptr = static_cast<const int32_t*>(put(J.out_ptr, (T + 1) * 4));
            D.out_idx = static_cast<const int32_t*>(put(J.out_idx, (size_t)J.out_ptr[T] * 4));
            CK(g_copy_error);
        }
        char* o = g->bout.as<char>() + out_at[j];
        D.V = reinterpret_cast<double*>(o);
        D.iterations = reinterpret_cast<int32_t*>(o + up(n * T * 16));
        D.converged = reinterpret_cast<uint8_t*>(o + up(n * T * 16) + up(T * 4));
        if (J.served) D.served = reinterpret_cast<uint8_t*>(o + up(n * T * 16) + up(T * 4) + up(T));
    }
    if (int rc = group_run(g, njobs, dj.data(), p, "group_solve")) return rc;
    for (int j = 0; j < njobs; ++j) {
        const gbpf_job& J = jobs[j];
        const size_t n = J.solver->n, T = J.n_cases;
        CK(cudaMemcpyAsync(J.V, dj[j].V, n * T * 16, cudaMemcpyDeviceToHost, g->stream));
        CK(cudaMemcpyAsync(J.iterations, dj[j].iterations, T * 4, cudaMemcpyDeviceToHost, g->stream));
        CK(cudaMemcpyAsync(J.converged, dj[j].converged, T, cudaMemcpyDeviceToHost, g->stream));
        if (J.served) CK(cudaMemcpyAsync(J.served, dj[j].served, n * T, cudaMemcpyDeviceToHost, g->stream));
    }
    CK(cudaEventRecord(g->c1, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, g->c0, g->c1));
    g->last.call_ms = ms;
    return 0;
}

int gbpf_group_set_shape(gbpf_group* g, int threads_per_cta, int slot_budget) {
    if (!g) return fail("null group");
    if (threads_per_cta != 0 && threads_per_cta != 256 && threads_per_cta != 512 && threads_per_cta != 1024)
        return fail("group_set_shape: threads_per_cta must be 0, 256, 512 or 1024");
    if (slot_budget < 0) return fail("group_set_shape: slot_budget must be >= 0");
    g->fixed_NT = threads_per_cta;
    g->slot_budget = slot_budget ? slot_budget : 16384;
    return 0;
}

int gbpf_group_stats(gbpf_group* g, gbpf_stats* out) {
    if (!g || !out) return fail("null argument");
    *out = g->last;
    return 0;
}

}  // extern "C"

// ------------------------------------------------------------------------------ stream launch
// One persistent launch that serves jobs as they are submitted (see gbpf.h, gbpf_stream_*).
// Device control block (ints): [0] published, [1] stop, [2] status, [3] unused, then per job
// its written-back case count and its work counter; then the launch's 32 statistics words and
// 16 error words. Descriptors are never overwritten while the launch runs (the ring is filled
// front to back); a job's staged inputs take one 256-byte aligned block of a circular arena,
// released once the job and every older one are done -- the launch reads staged inputs past
// L1, so a block refilled for a later job is never read stale.
struct gbpf_stream {
    int device = 0, nsm = 0;
    cudaStream_t run = nullptr, sub = nullptr;  // the launch's stream; copies and islanding of submits
    cudaEvent_t ended = nullptr;
    DBuf scr, ring, ctl, arena;
    int* host_done = nullptr;            // page-locked, per job
    int* host_pub = nullptr;             // page-locked: the published count after each job
    int* host_one = nullptr;             // page-locked: the stop value
    gbpf::Job* host_jobs = nullptr;      // page-locked staging of the descriptors
    int capacity = 0, threads = 1024, ctas = 0, slot_budget = 8192;
    size_t arena_bytes = 0;
    // circular arena: live blocks from `tail` to `head` (wrapping past the end when `wrapped`);
    // job_beg / job_end: each job's block, released in job order from tail_job on
    size_t head = 0, tail = 0;
    bool wrapped = false;
    int tail_job = 0;
    std::vector<size_t> job_beg, job_end;
    unsigned long long cta_bytes = 0;
    int published = 0;
    bool running = false, mixed = false;
    gbpf_params p{};
    std::vector<gbpf_solver*> topo;  // the topologies the running launch was sized and scheduled for
    ~gbpf_stream() {
        if (run) cudaStreamSynchronize(run);
        if (sub) cudaStreamSynchronize(sub);
        for (DBuf* b : {&scr, &ring, &ctl, &arena}) b->release();
        for (void* h : {(void*)host_done, (void*)host_pub, (void*)host_one, (void*)host_jobs})
            if (h) cudaFreeHost(h);
        if (ended) cudaEventDestroy(ended);
        for (cudaStream_t st : {run, sub})
            if (st) cudaStreamDestroy(st);
    }
    int* dctl() { return ctl.as<int>(); }
    int* ddone() { return dctl() + 4; }
    int* dcounter() { return dctl() + 4 + capacity; }
    unsigned long long* dstats() {
        return reinterpret_cast<unsigned long long*>(ctl.as<char>() + (((size_t)(4 + 2 * capacity) * 4 + 255) & ~(size_t)255));
    }
    int* derr() { return reinterpret_cast<int*>(dstats() + 32); }
    size_t ctl_bytes() const { return (((size_t)(4 + 2 * capacity) * 4 + 255) & ~(size_t)255) + 32 * 8 + 16 * 4; }
    static size_t job_stride() { return sizeof(gbpf::Job); }  // the kernel's stride (a multiple of 256)
};

namespace {
constexpr unsigned STREAM_SLEEP_NS = 20000;  // a CTA without an open job polls every ~20 us

// Case slots a CTA may take per job of this topology: the slot budget's count, and at least
// two -- so that a large grid's job of more cases than the launch has CTAs runs in one wave of
// two-slot CTAs instead of two waves of one-slot CTAs
int stream_slots(const gbpf_stream* st, const gbpf_solver* s) {
    return std::max(2, job_slots(gbpf::MAX_SLOTS, s->plan.nv, st->slot_budget));
}

// Case slots of a job's CTAs: the slot budget's count, but no more than the job has cases (a
// single solve takes one slot, with all of the CTA's threads, for the lowest latency); and as
// many as it takes (up to two) for the job's cases to fit the launch's CTAs in one wave.
int stream_job_slots(const gbpf_stream* st, const gbpf_solver* s, int cases) {
    const int budget = job_slots(gbpf::MAX_SLOTS, s->plan.nv, st->slot_budget);
    int g = 1;
    while (g < cases && g < budget) g *= 2;
    if (g == 1 && cases > st->ctas) g = 2;
    return g;
}

size_t up256s(size_t b) { return (std::max<size_t>(b, 1) + 255) & ~(size_t)255; }

// A block of `need` bytes (a multiple of 256) of the circular arena for job `q`, after releasing
// the blocks of the completed jobs, oldest first; SIZE_MAX when it does not fit now.
size_t arena_block(gbpf_stream* st, int q, size_t need) {
    while (st->tail_job < st->published && *(volatile const int*)(st->host_done + st->tail_job)) {
        const int j = st->tail_job++;
        if (st->wrapped && st->job_beg[j] < st->tail) st->wrapped = false;  // the block after the wrap
        st->tail = st->job_end[j];
    }
    if (st->tail_job == st->published) {  // nothing live: the arena is empty
        st->head = st->tail = 0;
        st->wrapped = false;
    }
    size_t at = SIZE_MAX;
    if (!st->wrapped) {
        if (st->arena_bytes - st->head >= need) {
            at = st->head;
        } else if (st->tail > need) {  // wrap to the front (strictly below tail: full != empty)
            at = 0;
            st->wrapped = true;
        }
    } else if (st->tail - st->head > need) {
        at = st->head;
    }
    if (at == SIZE_MAX) return at;
    st->head = at + need;
    st->job_beg[q] = at;
    st->job_end[q] = at + need;
    return at;
}
}  // namespace

extern "C" {

gbpf_stream* gbpf_stream_create(int capacity, size_t arena_bytes, int threads, int ctas, int slot_budget) {
    if (capacity <= 0 || arena_bytes < 4096 || ctas < 0 || slot_budget < 0 ||
        (threads != 0 && threads != 512 && threads != 1024)) {
        fail("stream_create: capacity > 0, arena_bytes >= 4096, threads 0, 512 or 1024, ctas >= 0, slot_budget >= 0");
        return nullptr;
    }
    std::unique_ptr<gbpf_stream> st(new gbpf_stream);
    st->capacity = capacity;
    st->threads = threads ? threads : 1024;
    st->arena_bytes = arena_bytes & ~(size_t)255;
    st->job_beg.assign(capacity, 0);
    st->job_end.assign(capacity, 0);
    if (slot_budget) st->slot_budget = slot_budget;
    auto ok = [&](cudaError_t e) {
        if (e == cudaSuccess) return true;
        fail(std::string("stream_create: ") + cudaGetErrorString(e));
        return false;
    };
    if (!ok(cudaGetDevice(&st->device))) return nullptr;
    if (!ok(cudaDeviceGetAttribute(&st->nsm, cudaDevAttrMultiProcessorCount, st->device))) return nullptr;
    // every SM's room for Newton CTAs (one of 1,024 threads or two of 512), less 8 SMs' room kept
    // free for the submits' islanding and start-table kernels
    const int per_sm = 1024 / st->threads;
    st->ctas = ctas ? ctas : std::max(1, per_sm * (st->nsm - 8));
    if (!ok(cudaStreamCreateWithFlags(&st->run, cudaStreamNonBlocking))) return nullptr;
    if (!ok(cudaStreamCreateWithFlags(&st->sub, cudaStreamNonBlocking))) return nullptr;
    if (!ok(cudaEventCreateWithFlags(&st->ended, cudaEventDisableTiming))) return nullptr;
    if (!ok(st->ring.ensure((size_t)capacity * gbpf_stream::job_stride()))) return nullptr;
    if (!ok(st->ctl.ensure(st->ctl_bytes()))) return nullptr;
    if (!ok(st->arena.ensure(arena_bytes))) return nullptr;
    if (!ok(cudaMallocHost((void**)&st->host_done, (size_t)capacity * 4))) return nullptr;
    if (!ok(cudaMallocHost((void**)&st->host_pub, (size_t)capacity * 4))) return nullptr;
    if (!ok(cudaMallocHost((void**)&st->host_one, 4))) return nullptr;
    if (!ok(cudaMallocHost((void**)&st->host_jobs, (size_t)capacity * sizeof(gbpf::Job)))) return nullptr;
    for (int q = 0; q < capacity; ++q) st->host_pub[q] = q + 1;
    *st->host_one = 1;
    return st.release();
}

void gbpf_stream_destroy(gbpf_stream* st) {
    if (!st) return;
    if (st->running) gbpf_stream_stop(st);
    delete st;
}

int gbpf_stream_start(gbpf_stream* st, int nsolvers, gbpf_solver* const* solvers, const gbpf_params* pp,
                      double idle_seconds) {
    if (!st) return fail("null stream");
    if (st->running) return fail("stream_start: the launch is running (stop it first)");
    if (nsolvers <= 0 || !solvers) return fail("stream_start: no topology");
    if (!(idle_seconds > 0.0)) return fail("stream_start: idle_seconds must be > 0");
    const gbpf_params p = pp ? *pp : default_params();
    if (int rc = check_params(p, "stream_start")) return rc;
    st->p = p;
    st->p.shared_start = 0;   // no prologue kernels: jobs arrive while the launch runs
    st->p.phase_timers = 0;
    st->mixed = p.precision == 1;
    // every topology's schedules for its slot count, and scratch for the largest of them
    unsigned long long cta = 0;
    for (int k = 0; k < nsolvers; ++k) {
        gbpf_solver* s = solvers[k];
        if (!s) return fail("stream_start: null solver");
        if (s->device != st->device) return fail("stream_start: a solver lives on another device");
        const int G = stream_slots(st, s);
        for (int g = 1; g <= G; g *= 2) {  // a job takes any power of two up to G slots
            Shape* sh = nullptr;
            if (int rc = get_shape(s, st->threads, g, &sh)) return rc;
        }
        cta = std::max(cta, solver_offsets(s, G, st->mixed).total);
    }
    st->cta_bytes = cta;
    st->topo.assign(solvers, solvers + nsolvers);
    // the kernels that submits launch beside the running launch, loaded before it starts
    CK(gbpf::preload_v0_table());
    CK(gbpf::preload_islands());
    CK(st->scr.ensure((size_t)st->ctas * cta));
    // the control block is zero before the launch reads it and before any submit copies to it
    CK(cudaStreamSynchronize(st->sub));
    CK(cudaMemsetAsync(st->ctl.p, 0, st->ctl_bytes(), st->sub));
    CK(cudaStreamSynchronize(st->sub));
    std::memset(st->host_done, 0, (size_t)st->capacity * 4);
    st->head = st->tail = 0;
    st->wrapped = false;
    st->tail_job = 0;
    st->published = 0;
    gbpf::Launch L{};
    L.jobs = st->ring.as<gbpf::Job>();
    L.njobs = st->capacity;
    L.scratch = st->scr.as<char>();
    L.cta_bytes = cta;
    L.ring.published = st->dctl();
    L.ring.stop = st->dctl() + 1;
    L.ring.status = st->dctl() + 2;
    L.ring.done_cases = st->ddone();
    int* dflags = nullptr;
    CK(cudaHostGetDevicePointer((void**)&dflags, st->host_done, 0));
    L.ring.host_done = dflags;
    L.ring.sleep_ns = STREAM_SLEEP_NS;
    L.ring.idle_polls = std::max<long long>(1, (long long)(idle_seconds * 1e9 / STREAM_SLEEP_NS));
    CK(gbpf::launch_newton(L, st->ctas, st->threads, st->run));
    CK(cudaEventRecord(st->ended, st->run));
    st->running = true;
    return 0;
}

int gbpf_stream_alive(gbpf_stream* st) {
    if (!st) return fail("null stream");
    if (!st->running) return 0;
    const cudaError_t e = cudaEventQuery(st->ended);
    if (e == cudaErrorNotReady) return 1;
    if (e != cudaSuccess) return fail(std::string("stream_alive: ") + cudaGetErrorString(e));
    return 0;
}

int gbpf_stream_submit(gbpf_stream* st, const gbpf_job* J) {
    if (!st || !J) return fail("stream_submit: null argument");
    if (!st->running) return fail("stream_submit: the launch is not running (gbpf_stream_start)");
    const int alive = gbpf_stream_alive(st);
    if (alive < 0) return -1;
    if (!alive) return fail("stream_submit: the launch has ended (its idle limit passed); stop and start it again");
    gbpf_solver* s = J->solver;
    if (!s) return fail("stream_submit: job without a solver");
    if (std::find(st->topo.begin(), st->topo.end(), s) == st->topo.end())
        return fail("stream_submit: the job's topology was not given to gbpf_stream_start");
    if (J->n_cases <= 0) return fail("stream_submit: the job has no cases");
    if (!J->S || !J->V0 || !J->V || !J->iterations || !J->converged)
        return fail("stream_submit: the job lacks an input or output array");
    if (J->pin || J->st_ptr || J->v0_per_col)
        return fail("stream_submit: stream jobs take one start V0 (n,), no pins and no explicit stamps");
    // the job's own precision: double factors in any launch, mixed only where the launch's
    // scratch holds the float factor buffers (a launch started with mixed precision)
    gbpf_params pj = st->p;
    if (J->precision == 1)
        pj.precision = 0;
    else if (J->precision == 2 && st->mixed)
        pj.precision = 1;
    else if (J->precision != 0)
        return fail("stream_submit: precision must be 0 (the launch's), 1 (double) or 2 (mixed, in a mixed launch)");
    // every host array page-locked: the kernel writes the outputs directly, and a copy from
    // pageable memory would synchronize with the device -- that is, wait for the running launch
    for (const void* a : {(const void*)J->V, (const void*)J->iterations, (const void*)J->converged,
                          (const void*)J->served, (const void*)J->S, (const void*)J->V0, (const void*)J->out_ptr,
                          (const void*)J->out_idx}) {
        if (!a) continue;
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, a) != cudaSuccess || at.type != cudaMemoryTypeHost) {
            cudaGetLastError();
            return fail("stream_submit: inputs and outputs must be page-locked host memory (gbpf_host_alloc)");
        }
    }
    if (J->out_ptr) {
        if (!s->m) return fail("stream_submit: outage cases need the solver's branch table (gbpf_set_branches)");
        if (J->s_per_col || J->v0_per_col || !J->out_idx)
            return fail("stream_submit: outage cases take one S and one V0 (n,) and out_ptr / out_idx");
        if (J->out_ptr[0] != 0) return fail("stream_submit: outage pointers must start at 0");
        for (int c = 0; c < J->n_cases; ++c)
            if (J->out_ptr[c + 1] < J->out_ptr[c]) return fail("stream_submit: outage pointers must not decrease");
        for (int q = 0; q < J->out_ptr[J->n_cases]; ++q)
            if (J->out_idx[q] < 0 || J->out_idx[q] >= s->m) return fail("stream_submit: outage index out of range");
    } else if (J->served) {
        return fail("stream_submit: a served mask belongs to outage cases");
    }
    const int G = stream_job_slots(st, s, J->n_cases);
    if (st->published >= st->capacity) return -2;  // the ring is full: stop, then start again
    const size_t n = s->n, T = J->n_cases;
    const size_t sb = n * (J->s_per_col ? T : 1) * 16, vb = n * 16;
    const int nout = J->out_ptr ? J->out_ptr[T] : 0;
    const int igrid = (int)std::min<size_t>(T, 32);  // the islanding runs beside the launch, on spare SMs
    // the job's staging: S, V0, its start table, and for outage cases the lists and islanding
    const size_t parts[] = {sb, vb, n * 64, (T + 1) * 4, (size_t)std::max(nout, 1) * 4, n * T * 4, n * T * 4,
                            n * T, T * 4, (size_t)igrid * 4 * n * 4, (size_t)igrid * n * 8};
    const int nparts = J->out_ptr ? 11 : 3;
    size_t need = 0;
    for (int k = 0; k < nparts; ++k) need += up256s(parts[k]);
    if (need > st->arena_bytes) return fail("stream_submit: the job needs more staging than the arena holds");
    const int q = st->published;
    const size_t at = arena_block(st, q, need);
    if (at == SIZE_MAX) return -2;  // the arena is busy with earlier jobs: wait for them, or stop and start again
    char* blk[11] = {};
    size_t pos = at;
    for (int k = 0; k < nparts; ++k) {
        blk[k] = st->arena.as<char>() + pos;
        pos += up256s(parts[k]);
    }
    char *dS = blk[0], *dV0 = blk[1], *dtab = blk[2], *dop = blk[3], *doi = blk[4], *dlab = blk[5],
         *dref = blk[6], *dsv = blk[7], *dni = blk[8], *dscr = blk[9], *dbest = blk[10];
    CK(cudaMemcpyAsync(dS, J->S, sb, cudaMemcpyHostToDevice, st->sub));
    CK(cudaMemcpyAsync(dV0, J->V0, vb, cudaMemcpyHostToDevice, st->sub));
    gbpf::Job& o = st->host_jobs[q];
    o = gbpf::Job{};
    Shape* sh = nullptr;
    if (int rc = get_shape(s, st->threads, G, &sh)) return rc;  // (built by gbpf_stream_start)
    o.P = sh->dp;
    Shape* sh1 = sh;
    if (G > 1)
        if (int rc = get_shape(s, st->threads, 1, &sh1)) return rc;
    o.P1 = sh1->dp;
    o.off = solver_offsets(s, G, st->mixed);
    o.G = G;
    o.log2G = ilog2(G);
    o.seq = q;
    gbpf::Batch b{};
    b.B = (int)T;
    b.S = reinterpret_cast<const double2*>(dS);
    b.s_shared = !J->s_per_col;
    b.sS = (long long)T;
    b.V0 = reinterpret_cast<const double2*>(dV0);
    b.v0_shared = 1;
    b.v0tab = reinterpret_cast<const double4_32a*>(dtab);
    if (J->out_ptr) {
        CK(cudaMemcpyAsync(dop, J->out_ptr, (T + 1) * 4, cudaMemcpyHostToDevice, st->sub));
        if (nout) CK(cudaMemcpyAsync(doi, J->out_idx, (size_t)nout * 4, cudaMemcpyHostToDevice, st->sub));
        CK(gbpf::launch_islands(s->n, s->m, s->dbr_f.as<int>(), s->dbr_t.as<int>(), s->dbr_live.as<uint8_t>(),
                                (int)T, reinterpret_cast<const int*>(dop), reinterpret_cast<const int*>(doi),
                                s->dslack.as<uint8_t>(), s->dprio.as<double>(), J->reslack,
                                reinterpret_cast<int*>(dscr), reinterpret_cast<unsigned long long*>(dbest),
                                reinterpret_cast<int*>(dlab), reinterpret_cast<uint8_t*>(dsv),
                                reinterpret_cast<int*>(dref), reinterpret_cast<int*>(dni), st->derr() + 6, igrid,
                                st->sub));
        if (J->served) CK(cudaMemcpyAsync(J->served, dsv, n * T, cudaMemcpyDeviceToHost, st->sub));
        b.ymode = 3;
        b.out_ptr = reinterpret_cast<const int*>(dop);
        b.out_idx = reinterpret_cast<const int*>(doi);
        b.ref_bus = reinterpret_cast<const int*>(dref);
        b.sref = (long long)T;
    }
    b.Vout = reinterpret_cast<double2*>(J->V);
    b.sV = (long long)T;
    b.iters = J->iterations;
    b.conv = J->converged;
    fill_common(b, s, pj);
    b.counter = st->dcounter() + q;
    b.stats = st->dstats();
    b.err = st->derr();
    o.B = b;
    // the start table (run beside the launch on the submit stream, before the job is published)
    CK(gbpf::launch_v0_table(b.V0, s->n, b.check_v0, const_cast<double4_32a*>(b.v0tab), b.err, st->sub));
    // descriptor first, then the published count: stream order puts both behind the inputs
    CK(cudaMemcpyAsync(st->ring.as<char>() + (size_t)q * gbpf_stream::job_stride(), &o, sizeof(gbpf::Job),
                       cudaMemcpyHostToDevice, st->sub));
    CK(cudaMemcpyAsync(st->dctl(), st->host_pub + q, 4, cudaMemcpyHostToDevice, st->sub));
    st->published = q + 1;
    return q;
}

const int* gbpf_stream_flags(gbpf_stream* st) { return st ? st->host_done : nullptr; }

int gbpf_stream_done(gbpf_stream* st, int q) {
    if (!st) return fail("null stream");
    if (q < 0 || q >= st->published) return fail("stream_done: no such job in this launch");
    const int v = *(volatile const int*)(st->host_done + q);
    std::atomic_thread_fence(std::memory_order_acquire);  // the job's results are read after its flag
    return v ? 1 : 0;
}

int gbpf_stream_stop(gbpf_stream* st) {
    if (!st) return fail("null stream");
    if (!st->running) return 0;
    st->running = false;
    CK(cudaMemcpyAsync(st->dctl() + 1, st->host_one, 4, cudaMemcpyHostToDevice, st->sub));
    CK(cudaStreamSynchronize(st->sub));
    CK(cudaStreamSynchronize(st->run));
    int words[3] = {0, 0, 0}, err[16];
    CK(cudaMemcpy(words, st->dctl(), 12, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(err, st->derr(), sizeof err, cudaMemcpyDeviceToHost));
    if (err[0] == gbpf::DE_V0_NONFINITE || err[0] == gbpf::DE_V0_MAGNITUDE)
        return fail("stream: invalid initial voltage at bus " + std::to_string(err[1]));
    if (err[0] == gbpf::DE_STAMPS) return fail("stream: an outage case has too many stamp entries");
    if (err[6]) return fail("stream: label propagation of an outage job did not settle");
    if (words[2] == 2) return fail("stream: a job descriptor did not hold the job its index names");
    return words[2] ? 1 : 0;
}

}  // extern "C"
