/* gbpf.h -- C ABI of the GB300-native batched polar Newton-Raphson power-flow solver.
 *
 * Drop-in boundary for the batched Newton path of e2nIEE/parallel-pandapower-solver
 * (p3s 1.2.2). Every entry point replaces one call the reference's Python layer makes
 * into its compiled solvers; the reference interface each one replaces is cited next to
 * it. All arrays are caller-owned, C order; complex128 arrays are passed as interleaved
 * (re, im) doubles. Host-pointer entry points copy to and from the device themselves;
 * the *_device variants take device pointers. Functions return 0 on success and a
 * negative code on error, with a message from gbpf_last_error() (never an exception).
 * Non-convergence is not an error: it is reported per case in `converged`.
 */
#ifndef GBPF_H
#define GBPF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbpf_solver gbpf_solver;

/* Per-call solve parameters (nr_klu.cpp:1049-1052 keyword arguments, and the
 * PolarNewtonSolverCUDA attributes precision / mixed_switch / line_search,
 * p3s/cuda/nr_polar_solver.py:309-330). */
typedef struct gbpf_params {
    int max_iter;        /* 30 */
    double tol;          /* 1e-8: infinity norm of the mismatch, p.u. */
    int line_search;     /* 1: Armijo backtracking (nr_klu.cpp:541-567) */
    int precision;       /* 0: double factors; 1: mixed (float factors while the vote asks) */
    double mixed_switch; /* mismatch above which a case factors in float (mixed only) */
    int check_v0;        /* 1: reject non-finite / out-of-range start voltages like solve_batch */
    double pivot_ratio_double; /* accept a double factorization while min|piv|/max|piv| >= this x rcond0 (1e-3) */
    double pivot_ratio_single; /* the same bound for a float factorization (1e-3) */
    int vote_rule;       /* mixed: 0 = the reference's precision votes (nr_polar_kernels.cu:209-228),
                            1 = float until contraction stalls below mixed_switch */
    double polish;       /* vote_rule 1: a case on float factors iterates until its mismatch is
                            below polish * tol (1e-3) ... */
    double vtol;         /* ... and below vtol / |J^-1| (jinv_norm of gbpf_info), a bound on the
                            voltage error left (1e-8 p.u.; 0: no bound) -- though not below twice
                            the double mismatch's rounding floor -- so its voltage is as accurate
                            as a double solve's on ill-conditioned grids too */
    double chord_tol;    /* vote_rule 1: once an accepted float step leaves the mismatch below this
                            (1e-8 p.u.: the polish steps), the next step reuses the float factors it
                            was solved with (a chord step: substitutions only, no factorization) for
                            as long as each such step cuts the mismatch tenfold; 0: always refactor */
    int shared_start;    /* 1: a batch of at least 16 cases that all start from one V0 on the base
                            Ybus without pins evaluates and factors that start once (a one-CTA
                            prologue) and every case's first step solves with it -- for bulk
                            batches; 0: every case evaluates and factors its own start (no
                            prologue on the launch's critical path: latency-bound serving) */
    int phase_timers;    /* 1: the Newton kernel sums SM clock cycles per phase over its CTAs into
                            gbpf_stats.phase_cycles (single-topology launches; 0: off, the default) */
    int eager_jacobian;  /* mixed, vote_rule 1: 0 (default) leaves the float Jacobian out of an
                            evaluation after which no factorization is expected (after a chord
                            step, or a float step from below 100 x chord_tol) and builds it later
                            only if a step factors after all -- the same values, so the same
                            results; 1: every evaluation builds its Jacobian */
} gbpf_params;

/* Topology / schedule facts of a solver (for stats, rooflines and tests). */
typedef struct gbpf_info {
    int n_bus, nnz_ybus, n_var_bus, n_blocks, n_levels, n_back_levels;
    int cases_per_cta, threads_per_cta, workers;
    long long factor_pairs, forward_pairs, backward_pairs;
    double rcond0;
    double jinv_norm;    /* estimate of |J^-1| (infinity norm) at the flat start */
} gbpf_info;

/* Counters of the last solve (the reference's last_stats, nr_polar_solver.py:671-681). */
typedef struct gbpf_stats {
    unsigned long long single_factorizations, double_factorizations;
    unsigned long long single_rejected, double_rejected, macro_steps;
    int grid, cases_per_cta;
    double kernel_ms; /* device time of the Newton kernel, CUDA events on the solver's stream */
    double call_ms;   /* device time of the last host-pointer call: first copy in to last copy out */
    int threads_per_cta; /* CTA shape of the last launch (with cases_per_cta) */
    unsigned long long chord_steps; /* steps solved with the previous float factors (chord_tol) */
    unsigned long long first_steps; /* first steps solved with the shared start's factors: when every
                                       case starts from one V0 on the base Ybus without pins, the
                                       first mismatch's injections and J(V0) are computed and
                                       factored once per launch */
    unsigned long long phase_cycles[6]; /* with gbpf_params.phase_timers: SM cycles summed over the
                                           CTAs of the last launch per phase -- slot refill and case
                                           load, factorization with forward substitution, backward
                                           substitution, voltage update, mismatch / Jacobian
                                           evaluation, decision and write-back; 0 otherwise */
    unsigned long long lazy_jacobians;  /* mixed: evaluations that left the float Jacobian out (a
                                           chord step or the case's end was expected next) */
    unsigned long long jacobian_sweeps; /* of those, Jacobians built afterwards because the next
                                           step factored after all */
} gbpf_stats;

const char* gbpf_last_error(void);
int gbpf_version(void);
int gbpf_device_count(void);

/* Solver for one grid topology: pattern, bus types, fill-reducing order, symbolic
 * factorization and schedule, device upload.
 * Replaces nr_klu.Solver(Yp, Yj, Yx, pv, pq) (nr_klu.cpp:964-994, build_topology :732-759)
 * and PolarNewtonSolverCUDA(Yp, Yj, Yx, pv, pq) (nr_polar_solver.py:285-378).
 * cases_per_cta: 0 = chosen per batch size, else a power of two in 1..32. Returns NULL on error. */
gbpf_solver* gbpf_create(int n, const int32_t* Yp, const int32_t* Yj, const double* Yx, int nnz, const int32_t* pv,
                         int npv, const int32_t* pq, int npq, int cases_per_cta);
/* gbpf_create with the CTA shape fixed: threads_per_cta 256, 512 or 1024 and cases_per_cta a
 * power of two in 1..32; 0 leaves that part to the batch-size rule (gbpf_get_shape). CTAs of
 * 1024 / threads_per_cta threads share an SM. */
gbpf_solver* gbpf_create_ex(int n, const int32_t* Yp, const int32_t* Yj, const double* Yx, int nnz,
                            const int32_t* pv, int npv, const int32_t* pq, int npq, int cases_per_cta,
                            int threads_per_cta);
void gbpf_destroy(gbpf_solver* s);

/* Values-only Ybus refresh. Replaces Solver.update_Y (nr_klu.cpp:999-1011) and
 * PolarNewtonSolverCUDA.update_Y (nr_polar_solver.py:569-587). */
int gbpf_update_Y(gbpf_solver* s, const double* Yx, int nnz);

int gbpf_get_info(gbpf_solver* s, gbpf_info* out);
int gbpf_get_stats(gbpf_solver* s, gbpf_stats* out);
/* Final mismatch infinity norm (p.u.) of every case of the solver's last synchronous solve (n =
 * its case count). Times gbpf_info.jinv_norm it bounds each result's distance from the exact
 * power-flow solution to first order, and so from a converged FP64 solve (the per-result
 * accuracy statement of the mixed path). No reference counterpart. */
int gbpf_get_mismatch(gbpf_solver* s, double* out, long long n);
/* CTA shape (threads per CTA, case slots per CTA) the solver launches for a batch of
 * `units` work items (cases, or lanes), and an override per batch-size class
 * (ceil(log2(units))) -- what an autotuner sets after timing candidate shapes. Results do not
 * depend on the shape (every case runs the same arithmetic); only the speed does.
 * threads_per_cta = cases_per_cta = 0 removes the override. No reference counterpart (the
 * reference's lean LU kernel takes a fixed warps-per-block `slots` argument,
 * nr_polar_solver.py:285-300). */
int gbpf_get_shape(gbpf_solver* s, long long units, int* threads_per_cta, int* cases_per_cta);
int gbpf_set_shape(gbpf_solver* s, long long units, int threads_per_cta, int cases_per_cta);
/* Builds, ahead of use, the schedules of every CTA shape a launch of this topology may take
 * with up to max_cases_per_cta slots (512 threads: 1, 2, 4, ... slots; 1,024: up to 4), so that
 * no later launch builds one on its critical path (a serving loop's warm-up). No reference
 * counterpart. */
int gbpf_prepare_shapes(gbpf_solver* s, int max_cases_per_cta);
/* Factorization schedule knob (no reference counterpart; the reference deals each level's
 * tasks to a fixed number of lists, lean_lu_plan.py:172-190): within a level, a pivot's chain
 * of diagonal and L-column tasks heavier than chain_cap x the level's mean work per worker is
 * cut into segments on different workers, each later segment recomputing the diagonal's
 * inverse. 1.0 is the default; 0 never cuts. Applies to the CTA shapes used from now on
 * (shapes built with other caps stay cached); results do not change, only the speed. */
int gbpf_set_chain_cap(gbpf_solver* s, double chain_cap);

/* The solver's current Ybus values (nnz complex), e.g. after gbpf_update_Y_from_branches. */
int gbpf_get_Y(gbpf_solver* s, double* Yx);
/* Ybus nnz -> Jacobian block position (-1 for slack rows/columns), length nnz. */
int gbpf_get_posmap(gbpf_solver* s, int32_t* out);

/* Batch of operating points on one topology (time series).
 * S: (n, T) complex (s_per_col = 1) or (n,) shared; V0: (n, T) (v0_per_col = 1) or (n,).
 * Out: V (n, T) complex, iterations (T,), converged (T,).
 * Replaces Solver.solve_batch (nr_klu.cpp:1049-1166) and
 * PolarNewtonSolverCUDA.solve_batch (nr_polar_solver.py:466-481). */
int gbpf_solve_batch(gbpf_solver* s, int T, const double* S, int s_per_col, const double* V0, int v0_per_col,
                     const gbpf_params* p, double* V, int32_t* iterations, uint8_t* converged);
int gbpf_solve_batch_device(gbpf_solver* s, int T, const double* dS, int s_per_col, const double* dV0,
                            int v0_per_col, const gbpf_params* p, double* dV, int32_t* d_iterations,
                            uint8_t* d_converged);

/* Warm-start lanes: hours offsets[l] .. offsets[l+1]-1 of lane l are solved in order,
 * each from the converged voltage of the previous hour of its lane (from V0 for a
 * lane's first hour and after a non-converged hour). S (n, T); V0 (n,).
 * Extends solve_batch with per-column start voltages (nr_klu.cpp:1070-1090): the chain
 * is resolved on the device. */
int gbpf_solve_lanes(gbpf_solver* s, int T, const double* S, const double* V0, int K, const int64_t* offsets,
                     const gbpf_params* p, double* V, int32_t* iterations, uint8_t* converged);
int gbpf_solve_lanes_device(gbpf_solver* s, int T, const double* dS, const double* dV0, int K,
                            const int64_t* d_offsets, const gbpf_params* p, double* dV, int32_t* d_iterations,
                            uint8_t* d_converged);

/* gbpf_solve_lanes enqueued in `slot` (0..7) and returned at once: copies in, the launch and
 * copies out run on the slot's own stream with the slot's own scratch, so calls in different
 * slots overlap (one call's copies with another's kernel). S / V0 / offsets / V / iterations
 * / converged must stay valid until gbpf_solve_wait(slot), which waits, reports device errors
 * and sets the stats of that call. Page-locked host arrays (gbpf_host_alloc) let the copies
 * overlap; with pageable ones the call itself waits for them. No reference counterpart (the
 * reference's calls are synchronous). */
int gbpf_solve_lanes_async(gbpf_solver* s, int slot, int T, const double* S, const double* V0, int K,
                           const int64_t* offsets, const gbpf_params* p, double* V, int32_t* iterations,
                           uint8_t* converged);
int gbpf_solve_wait(gbpf_solver* s, int slot);

/* N-1 batch: per-case Ybus values on the shared pattern, per-case pin mask.
 * S: (n,) complex; V0: (n, L) complex; pin: (n, L) uint8 (NULL = none).
 * Per-case Ybus either dense Yd (nnz, L) complex (replaces
 * Solver.solve_batch_contingency, nr_klu.cpp:1184-1281, and
 * PolarNewtonSolverCUDA.solve_batch_contingency[_cx], nr_polar_solver.py:483-527) or, with
 * Yd == NULL, the base Ybus minus sparse stamps: case c subtracts st_val[e] at CSR
 * position st_k[e] for e in [st_ptr[c], st_ptr[c+1]) (replaces
 * solve_batch_contingency_stamp, nr_polar_solver.py:529-557). */
int gbpf_solve_contingency(gbpf_solver* s, int L, const double* S, const double* V0, const uint8_t* pin,
                           const double* Yd, const int32_t* st_ptr, const int32_t* st_k, const double* st_val,
                           const gbpf_params* p, double* V, int32_t* iterations, uint8_t* converged);

/* Jacobian blocks (n_blocks x 4, row-major 2x2 [dP/dth dP/dVm; dQ/dth dQ/dVm]) and residual
 * (n_var_bus x 2, block-row order, S - S(V)) evaluated on the device at one voltage.
 * Backs debug_J (nr_klu.cpp:1283-1304, 1332-1342). */
int gbpf_eval_jacobian(gbpf_solver* s, const double* S, const double* V, const uint8_t* pin, double* blocks,
                       double* residual);
/* DC start voltage (p3s/timeseries.py:200-247 dc_initial_voltage, NewtonPowerflowCpp.py:422-440
 * _pre_dc_solve): angles from B[pvpq, pvpq] theta = Pinj[pvpq] - B[pvpq, ref] theta_ref with
 * B the branch susceptance Laplacian (-Im Ybus off the diagonal, the diagonal their negated
 * row sum), factored and solved on the device by the solver's block LU; every non-slack
 * bus keeps its magnitude from V0 (n complex) with the DC angle, slack buses keep V0. Returns 0,
 * or 1 when the DC system is singular or gives non-finite angles (Vout = V0, the flat start). */
int gbpf_dc_start(gbpf_solver* s, const double* Pinj, const double* V0, double* Vout);
/* Batched DC start: T injection columns Pinj (n, T) [bus][case] (e.g. Sbus.real + the phase-shift
 * injection per time step or scenario), one shared V0 (n complex), B factored ONCE and every case
 * substituted on the device. dc_stamps (m x 4 complex, the DC branch stamps (Yff, Yft, Ytf, Ytt)
 * of the reference's models, TwoPort.py:169-189 create_y_dc_matrix, summed onto the Ybus pattern
 * at the positions of gbpf_set_branches; their imaginary parts are the reference's Bbus) or NULL
 * (B from the Ybus as gbpf_dc_start). Vout (n, T) complex; used (T, or NULL): 1 where the DC angles
 * were taken, 0 where the case keeps V0 (singular B or non-finite angles). Returns 0 when every case
 * took its DC angles, 1 otherwise, -1 on error. */
int gbpf_dc_start_batch(gbpf_solver* s, int T, const double* Pinj, const double* V0, const double* dc_stamps,
                        double* Vout, uint8_t* used);
/* Block row of each bus (-1 for slack), length n. */
int gbpf_get_row_of_bus(gbpf_solver* s, int32_t* out);

/* Device check of the kernels' integer-pipe float/double conversions: d2f[i] = in[i]
 * converted to float (round toward zero), f2d[i] = d2f[i] converted back to double, and
 * d2f_small[i] (optional, may be NULL) = in[i] through the short conversion the float
 * Jacobian applies to voltage components (equal to d2f[i] for finite |in[i]| < 2^128). No
 * reference counterpart (a GB300-specific helper). */
int gbpf_selftest_conversions(const double* in, int n, float* d2f, double* f2d, float* d2f_small);
/* Self-test of the kernels' own double-precision numerics (no reference counterpart): per
 * element, recip = the Newton-refined reciprocal (x > 0, else 0), s_small / c_small = the
 * small-angle series sine / cosine (|x| < 1/4, else CUDA's), s_ref / c_ref = CUDA's sincos;
 * with phasor (2 doubles, or NULL), rot (n x 4) = the phasor rotated by x as the voltage update
 * rotates a bus phasor, then as it does after a float step at a PQ bus (the increment formed
 * in float) (|x| < 1/4, else 0). */
int gbpf_selftest_math(const double* in, int n, double* recip, double* s_small, double* c_small, double* s_ref,
                       double* c_ref, const double* phasor, double* rot);

/* Page-locked host memory for fast transfers. */
void* gbpf_host_alloc(size_t bytes);
void gbpf_host_free(void* p);

/* ------------------------------------------------------------------ several topologies
 * One launch of the persistent kernel over jobs of different topologies (grids of uneven
 * size, requests of a serving loop): CTAs serve the jobs largest first, each job until its
 * cases run out, so short jobs fill the tail of long ones. A group owns the launch's
 * stream, scratch and staging buffers; the solvers lend their plans (no call on a solver
 * may overlap a group launch that uses it). No reference counterpart: the reference solves
 * one topology per call (nr_polar_solver.py:466-596). */
typedef struct gbpf_group gbpf_group;

typedef struct gbpf_job {
    gbpf_solver* solver;     /* the topology */
    int n_cases;
    const double* S;         /* (n, n_cases) complex (s_per_col = 1) or (n,) */
    int s_per_col;
    const double* V0;        /* (n, n_cases) (v0_per_col = 1) or (n,) */
    int v0_per_col;
    const uint8_t* pin;      /* (n, n_cases) or NULL */
    const int32_t* st_ptr;   /* outage stamps (gbpf_solve_contingency) or NULL */
    const int32_t* st_k;
    const double* st_val;
    double* V;               /* out: (n, n_cases) complex */
    int32_t* iterations;     /* out: (n_cases,) */
    uint8_t* converged;      /* out: (n_cases,) */
    int cases_per_cta;       /* 0: by the group rule (fewer for large grids), else a power of two <= 32 */
    /* Outage cases (the solver's branch table set by gbpf_set_branches; S and V0 (n,)): case c
     * removes branches out_idx[out_ptr[c] .. out_ptr[c+1]) (at most 8). Islands are found on the
     * device (gbpf_islands semantics, reslack as given); an island re-slacked to bus r starts
     * rotated so that r has angle 0 (r pinned at |V0[r]| + 0j); unserved buses are pinned at
     * 1 + 0j and returned as NaN. NULL: not an outage job. */
    const int32_t* out_ptr;
    const int32_t* out_idx;
    int reslack;
    uint8_t* served;         /* out, outage jobs: (n, n_cases) 1 where the bus's island is served
                                (the device islanding's mask, gbpf_islands semantics), or NULL */
    int precision;           /* stream launches: 0 = the launch's gbpf_params.precision, 1 = double
                                factors, 2 = mixed (a launch started with mixed precision); every
                                other parameter is the launch's. Group launches: 0 only. */
} gbpf_job;

gbpf_group* gbpf_group_create(void);
void gbpf_group_destroy(gbpf_group* g);
/* Host arrays: staged to the device, one launch, results copied back. */
int gbpf_group_solve(gbpf_group* g, int njobs, const gbpf_job* jobs, const gbpf_params* p);
/* Device arrays (every pointer of every job on the device). */
int gbpf_group_solve_device(gbpf_group* g, int njobs, const gbpf_job* jobs, const gbpf_params* p);
/* Launch shape of later group launches: threads per CTA (0: by the batch-size rule) and the
 * budget of variable buses x case slots a CTA holds per job (0: 16,384). */
int gbpf_group_set_shape(gbpf_group* g, int threads_per_cta, int slot_budget);
/* Counters of the last group launch (summed over its jobs). */
int gbpf_group_stats(gbpf_group* g, gbpf_stats* out);

/* ---------------------------------------------------------------- stream launch (serving)
 * ONE persistent launch of the Newton kernel that takes jobs while it runs: each submitted job
 * (gbpf_job: one topology's cases -- a single solve, a time-series chunk or N-1 outages) is
 * staged and appended to a ring, and the CTAs that find no open job take it as their slots free
 * up; its results are written straight into the caller's page-locked host arrays and its flag
 * (gbpf_stream_flags()[job]) is set once all its cases are written back. No reference
 * counterpart: the reference solves one call at a time (nr_polar_solver.py:466-596) and has no
 * serving loop.
 * create: capacity = jobs per launch; arena_bytes = device staging for the inputs of one launch;
 *   threads = threads per CTA, 512 or 1024 (0: 1024); ctas = CTAs (0: as many as fit on all
 *   SMs but 8, which keep room for the submits' islanding and start-table kernels); slot_budget
 *   = variable buses x case slots a CTA takes per job (0: 8,192). A job's CTAs take the
 *   smallest power of two of slots that holds its cases, up to that budget (a single solve
 *   runs on all of a CTA's threads), and two where one would leave more cases than the launch
 *   has CTAs (one wave instead of two).
 * start: launches the kernel for the given topologies (schedules built, scratch sized for them,
 *   the kernels that submits launch loaded into the context first; gbpf_params as for the other
 *   calls, the shared start off). A CTA without an open job polls every ~20 us; once no job has
 *   been published for idle_seconds it returns (status 1 at stop) -- the launch never waits
 *   without bound.
 * submit: returns the job's index, -2 when the ring of this launch is full (stop, start again,
 *   resubmit) or its staging arena is held by unfinished jobs (try again once some are done;
 *   a job's staging is released when it and every older job are done), -1 on error. Every
 *   host array of the job must be page-locked (gbpf_host_alloc; a copy from pageable memory
 *   would synchronize with the device, i.e. wait for the running launch): S, V0 and the outage
 *   lists are copied to the device asynchronously and must stay unchanged until the job's flag
 *   is set; V, iterations, converged (and served) are written by the kernel. Jobs take one
 *   start V0 (n,), no pins and no explicit stamps.
 * done: 1 once the job's results are in its host arrays (with an acquire fence), else 0.
 * alive: 1 while the launch runs. stop: marks the end of submits, waits for the launch (it
 *   serves every submitted job first) and returns 0, or 1 if its CTAs had returned at their
 *   idle limit, or -1 on a device error. After 1, a job whose flag is still 0 was published
 *   after the last CTA had left and was not started (none of its results written): submit it
 *   again to the next launch. A job some CTA started is always finished.
 * While a stream launch runs it holds most of the device's SMs: other solves on that device
 * wait until it is stopped (or its CTAs reach their idle limit) -- submit work to it instead. */
typedef struct gbpf_stream gbpf_stream;
gbpf_stream* gbpf_stream_create(int capacity, size_t arena_bytes, int threads, int ctas, int slot_budget);
void gbpf_stream_destroy(gbpf_stream* st);
int gbpf_stream_start(gbpf_stream* st, int nsolvers, gbpf_solver* const* solvers, const gbpf_params* p,
                      double idle_seconds);
int gbpf_stream_submit(gbpf_stream* st, const gbpf_job* job);
const int* gbpf_stream_flags(gbpf_stream* st);
int gbpf_stream_done(gbpf_stream* st, int job);
int gbpf_stream_alive(gbpf_stream* st);
int gbpf_stream_stop(gbpf_stream* st);

/* Islanding of N-1 cases on the device (case_generator.py:355-430 semantics).
 * Graph: n buses, m branches (f[e], t[e]); live[e] != 0 if the branch couples its ends.
 * Case c removes branches out_idx[out_ptr[c] .. out_ptr[c+1]). Labels are the connected
 * components numbered by their smallest bus (scipy's connected_components order).
 * Reference buses: slack buses (is_slack) keep their island served; with reslack, an
 * island without a slack is served from its generator bus of highest priority
 * (gen_prio[bus] > 0, ties to the lowest bus index); other islands are unserved.
 * Out: labels (n, L) int32, served (n, L) uint8, ref_bus (n, L) int32 (-1 if unserved),
 * reslack_bus (L,) int32 (-1 if none; the first re-slacked bus of the case). */
int gbpf_islands(int n, int m, const int32_t* f, const int32_t* t, const uint8_t* live, int L,
                 const int32_t* out_ptr, const int32_t* out_idx, const uint8_t* is_slack, const double* gen_prio,
                 int reslack, int32_t* labels, uint8_t* served, int32_t* ref_bus, int32_t* n_islands);

/* Branch table of the topology for outage cases: branch e joins f[e] - t[e]; its 2x2 stamp
 * (Yff, Yft, Ytf, Ytt) sits at CSR positions stamp_pos[4e .. 4e+3] with values stamp_val (4
 * complex per branch, the values an outage subtracts; case_generator.py:270-317, 505-524);
 * is_slack (n), gen_prio (n, re-slack ranking; NULL = none). */
int gbpf_set_branches(gbpf_solver* s, int m, const int32_t* f, const int32_t* t, const int32_t* stamp_pos,
                      const double* stamp_val, const uint8_t* is_slack, const double* gen_prio);

/* Branch stamps of the general two-port (p3s/models/TwoWindingTransformerModel.py:172-175; a
 * line is a = b = 1 with half its shunt admittance at each end, TransmissionLineModel.py:45-48):
 * Yff = (ys + y_from) / |a|^2, Yft = -ys / (conj a conj b), Ytf = -ys / (a b),
 * Ytt = (ys + y_to) / |b|^2 per branch (complex inputs of length m); out of service -> 0; an
 * open end Kron-eliminated (TwoPort.py:69-105). stamps: (m, 4) complex out. in_service /
 * open_from / open_to may be NULL (all in service, none open). */
int gbpf_branch_stamps(int m, const double* ys, const double* y_from, const double* y_to, const double* a,
                       const double* b, const uint8_t* in_service, const uint8_t* open_from, const uint8_t* open_to,
                       double* stamps);
int gbpf_branch_stamps_device(int m, const double* ys, const double* y_from, const double* y_to, const double* a,
                              const double* b, const uint8_t* in_service, const uint8_t* open_from,
                              const uint8_t* open_to, double* stamps, void* stream);
/* Ybus values of the solver's topology from branch stamps (m x 4 complex, at the positions set
 * by gbpf_set_branches) and bus shunts (n complex, or NULL), summed on the device
 * (TwoPort.py:133-149 create_y_matrix): the resident Ybus and the branch table take the new
 * values, like gbpf_update_Y (e.g. after tap changes). Replaces update_Y after a host rebuild
 * of the Ybus (NewtonPowerflowCuda.py:137-165). */
int gbpf_update_Y_from_branches(gbpf_solver* s, const double* stamps, const double* bus_shunt);

/* gbpf_islands for the topology of `s` (n = its bus count) on the solver's stream, with
 * device buffers the solver keeps and grows (no allocation once they are large enough):
 * for a caller that islands many batches of outages of one grid, e.g. a serving loop.
 * Replaces the same reference calls as gbpf_islands. */
int gbpf_solver_islands(gbpf_solver* s, int m, const int32_t* f, const int32_t* t, const uint8_t* live, int L,
                        const int32_t* out_ptr, const int32_t* out_idx, const uint8_t* is_slack, const double* gen_prio,
                        int reslack, int32_t* labels, uint8_t* served, int32_t* ref_bus, int32_t* n_islands);

/* gbpf_islands on caller-owned DEVICE buffers (same layouts; out_idx holds n_out entries),
 * allocating nothing: the kernel's scratch is a statically allocated 16 MiB device array,
 * so n may not exceed GBPF_ISLANDS_STATIC_MAX_BUS (larger n is rejected with an error).
 * Runs on `stream` (a cudaStream_t; NULL = the legacy default stream) and is synchronous:
 * it waits for `stream` and reads the validation and error words back to the host before it
 * returns. The first call on each device looks up the scratch address; make that first call
 * before any stream capture. The scratch is shared by every call on a device: calls that overlap
 * in time there (other streams or host threads) race. No reference counterpart: for callers
 * that must not allocate device memory (cudaMalloc / cudaFree synchronise the whole device,
 * stalling the solves a serving loop overlaps, and can fail under a memory budget). */
#define GBPF_ISLANDS_STATIC_MAX_BUS 65536
int gbpf_islands_device_static(int n, int m, const int32_t* d_f, const int32_t* d_t, const uint8_t* d_live, int L,
                               const int32_t* d_out_ptr, const int32_t* d_out_idx, int n_out,
                               const uint8_t* d_is_slack, const double* d_gen_prio, int reslack, int32_t* d_labels,
                               uint8_t* d_served, int32_t* d_ref_bus, int32_t* d_n_islands, void* stream);

/* ------------------------------------------------------------- either side of the path
 * Time-series injections (p3s/timeseries.py:36-141, build_sbus_matrix / _fill_sbus):
 * out[i, t] = s0[i] + sum_k coef[k] * (series[row[k] * T + t] - base[k]) over k = ptr[i] ..
 * ptr[i+1] - 1 in that order, added to the imaginary part where imag[k]. s0 (n) and out (n, T)
 * complex; series (R, T) float64 (every element-variable series stacked). Same operations and
 * order as the reference's loop, without fused multiply-adds. The _device variant takes device
 * pointers and runs on `stream` (a cudaStream_t; NULL = legacy default stream). */
int gbpf_build_sbus(int n, int T, int R, const double* s0, const int64_t* ptr, const int32_t* row, const double* coef,
                    const double* base, const uint8_t* imag, const double* series, double* out);
int gbpf_build_sbus_device(int n, int T, const double* s0, const int64_t* ptr, const int32_t* row, const double* coef,
                           const double* base, const uint8_t* imag, const double* series, double* out, void* stream);

/* Branch flows and loading of L solved cases (p3s/contingency/find_overloads.py:128-260,
 * compute_branch_loading): branch b joins f[b] -> t[b] with 2x2 admittance y[4b..4b+3] =
 * (Yff, Yft, Ytf, Ytt) complex; S_from = conj(Yff V_f + Yft V_t) V_f sn_mva, S_to likewise;
 * i_end = |S_end| / (vn_end |V_end| sqrt 3) (kA); i_max = max; loading = i_max / rating x 100
 * (kind 0, line: rating in kA) or max(i_from vn_from, i_to vn_to) sqrt 3 / rating x 100 (kind
 * 1, trafo: rating in MVA). Case c's outaged branches out_idx[out_ptr[c] ..] (out_ptr NULL:
 * none) report 0, non-converged cases NaN (end powers NaN + 0j, as the reference stores them), NaN
 * voltages propagate. V (n, L) complex; outputs
 * (nbr, L). */
int gbpf_branch_flows(int n, int nbr, int L, const int32_t* f, const int32_t* t, const double* y,
                      const double* vn_from, const double* vn_to, const double* rating, const uint8_t* kind,
                      double sn_mva, const double* V, const uint8_t* converged, const int32_t* out_ptr,
                      const int32_t* out_idx, double* S_from, double* S_to, double* i_from, double* i_to,
                      double* i_max, double* loading);
int gbpf_branch_flows_device(int nbr, int L, const int32_t* f, const int32_t* t, const double* y,
                             const double* vn_from, const double* vn_to, const double* rating, const uint8_t* kind,
                             double sn_mva, const double* V, const uint8_t* converged, const int32_t* out_ptr,
                             const int32_t* out_idx, double* S_from, double* S_to, double* i_from, double* i_to,
                             double* i_max, double* loading, void* stream);

/* Host-only check of the planner and the device schedule (runs without a GPU): plan for
 * `workers` workers, Jacobian at (Vm, Va) with injections S (n complex), the schedule
 * executed serially with a structural race check per level. dx (n x 2): Newton step per
 * bus (angle, magnitude). shape (7): n_var_bus, n_blocks, levels, back levels, factor /
 * forward / backward pairs. No reference counterpart: the reference's numpy plan executor
 * (lean_lu_plan.py:324-360) plays this role for its own plan. */
int gbpf_plan_selftest(int n, const int32_t* Yp, const int32_t* Yj, const double* Yx, int nnz, const int32_t* pv,
                       int npv, const int32_t* pq, int npq, int workers, const double* Vm, const double* Va,
                       const double* S, double* dx, int32_t* shape, char* msg, int msglen, double chain_cap);

#ifdef __cplusplus
}
#endif
#endif
