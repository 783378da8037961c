// gbpf_device.h -- structures shared by the host orchestration and the sm_103a kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace gbpf {

// slot states of the persistent Newton kernel
enum SlotState : int {
    SL_EMPTY = 0,      // needs a case
    SL_FRESH = 1,      // case loaded: evaluate at the start point
    SL_ACTIVE = 2,     // take a Newton step (factor + solve + full step)
    SL_BACKTRACK = 3,  // line search trial: mismatch only
    SL_NEEDJ = 4,      // line search done: mismatch + Jacobian at the accepted point
    SL_FINISH = 5,     // write the result back
    SL_RETIRED = 6,    // no more work
};

constexpr int MAX_SLOTS = 32;    // cases per CTA (G) upper bound
constexpr int MAX_STAMPS = 32;   // outage-stamp entries per case held in shared memory

// error codes written to Batch::err[0] (first error wins; err[1..2] = bus, case)
enum DevError : int {
    DE_NONE = 0,
    DE_V0_NONFINITE = 1,
    DE_V0_MAGNITUDE = 2,
    DE_STAMPS = 3,
    DE_OUTAGE = 4,           // a case's outage list is malformed (err[1] = index, err[2] = case)
};

struct DevPlan {
    int n, nv, nblk, W, nlev, nblev, nnzY;
    const int* Yp;
    const int* Yj;
    const double2* Y;        // base Ybus values (G + jB)
    const float2* Y32;       // float copy
    const int* posmap;       // Ybus nnz -> block, -1
    const int* row_of_bus;   // bus -> block row, -1 for slack
    const int* eval_order;   // the evaluation's bus sweep (reverse Cuthill-McKee)
    const uint8_t* bus_pq;
    const int4* taskA;
    const int* ptrA;
    const int4* taskC;
    const int* ptrC;
    const int4* headA;       // per taskA entry: its first two pairs inline (x0, y0, x1, y1; -1 = none)
    const int4* headC;       // per taskC entry: likewise
    const int4* taskF;       // chord passes: the forward tasks of taskA, same levels and workers
    const int4* headF;
    const int* ptrF;         // nlev*W + 1
    const int2* pairs;
    const uint8_t* row_pq;   // block row is PQ (two real pivots)
    const int* bus_of_row;
    const int* dpos;         // block row -> its diagonal block (base)
    // branch table (outage mode): per branch its 4 Ybus CSR positions and stamp values
    int m;
    const int4* br_pos;
    const double2* br_val;   // [branch][4]
    const uint8_t* is_slack; // [bus]
};

struct Batch {
    int B;                   // cases (independent mode) or total hours (lanes mode)
    int lanes;               // 0: independent cases; 1: warm-start lanes
    int K;                   // lanes
    const long long* lane_off;
    const double2* S;        // injections: S[bus * sS + case] or S[bus] if s_shared
    int s_shared;
    long long sS;
    const double2* V0;       // start voltage: V0[bus * sV0 + case] or V0[bus] if shared
    int v0_shared;
    long long sV0;
    const double4_32a* v0tab; // shared start: per bus (Vm, Va, cos, sin), (e, f, 1/Vm, 0)
    int check_v0;            // validate V0 like nr_klu's solve_batch
    int ymode;               // 0 base Ybus, 1 base minus per-case stamps, 2 dense per case,
                             // 3 base minus the stamps of per-case branch outages (out_ptr / out_idx)
    const int* st_ptr;       // stamps of case c: [st_ptr[c], st_ptr[c+1])
    const int* st_k;
    const double2* st_v;
    const double2* Yd;       // dense per-case Ybus Yd[k * sYd + case]
    long long sYd;
    const int* out_ptr;      // outage mode: case c removes branches out_idx[out_ptr[c] .. out_ptr[c+1])
    const int* out_idx;
    const int* ref_bus;      // island reference bus of every bus and case [bus * sref + case] (-1
    long long sref;          // unserved) or null: starts rotated to the reference, pins, NaN output
    const uint8_t* pin;      // pin[bus * spin + case] or null
    long long spin;
    double2* Vout;           // result Vout[bus * sV + case]
    long long sV;
    int* iters;
    uint8_t* conv;
    double* mis;             // or null: every case's final mismatch infinity norm (p.u.)
    int max_iter;
    double tol;
    int line_search;
    int mixed;               // 0: all factorizations double; 1: vote per case
    double mixed_switch;
    int vote_rule;           // 0: the reference's precision votes; 1: GB300 rule (see the kernel)
    double tol_polish;       // GB300 rule: float-factor cases iterate until mismatch < tol_polish
    double chord_tol;        // GB300 rule: below this mismatch a step reuses the last float factors (0: never)
    int lazy_jac;            // GB300 rule: evaluations expected to precede no factorization skip the float Jacobian
    // shared start (every case from the same V0 on the same Ybus, no pins): the injections and
    // the factors of J(V0), computed once by start_kernel; cases starting from V0 take their
    // first step with them (null: every case evaluates and factors its own start)
    const double2* R0;       // -(P, Q) at V0 per block row (0 for a PV row's Q)
    const void* fac0;        // factors of J(V0), one copy per case slot: [blk][slot], float4 / double4
    const int* ok0;          // 1 when the shared factorization passed its pivot check
    int share_ok;            // the caller allows a shared start (gbpf_params.shared_start)
    int timers;              // the launch counts SM cycles per phase into stats[8 .. 13] (gbpf_params.phase_timers)
    double rcond_min64;
    double rcond_min32;
    int* counter;            // work counter, zero before launch
    unsigned long long* stats;  // [0] fp32 factorizations [1] fp64 [2] fp32 rejected [3] fp64 rejected [4] macro steps
                                // [5] chord steps [6] first steps with the shared start's factors
                                // [8 .. 13] with timers: SM cycles summed over CTAs per phase (refill + load,
                                // factorization + forward substitution, backward substitution, voltage
                                // update, evaluation, decision + write-back)
    int* err;                // [0] code [1] bus [2] case
};

// Byte offsets of one job's scratch arrays inside a CTA's scratch region (G case slots;
// every array is [item][slot]); ~0 for an array the job does not use.
struct ScratchOffsets {
    unsigned long long fac64;  // [blk][slot] double 2x2 blocks (a00 a01 a10 a11)
    unsigned long long fac32;  // [blk][slot] float blocks (mixed precision): buffer 0 ...
    unsigned long long fac32b; // ... and 1 -- a slot's last float factors stay in one while the
                               // next Jacobian is written to the other
    unsigned long long R;      // [row][slot] residual (P, Q) = S - S(V)
    unsigned long long y64;    // [row][slot] step
    unsigned long long y32;
    unsigned long long Vc;     // [bus][slot] committed point (Vm, Va, cos, sin)
    unsigned long long Vt;     // [bus][slot] evaluation point (Vm, Va, cos, sin)
    unsigned long long Et;     // [bus][slot] evaluation point rectangular (e, f)
    unsigned long long Ei;     // [bus][slot] evaluation point 1 / Vm
    unsigned long long iv32;   // [bus][slot] 1 / Vm of the evaluation point in float (PQ buses)
    unsigned long long pin;    // [bus][slot]
    unsigned long long total;  // bytes of the job's region
};

// One job of a launch: a topology's plan (with the schedule of the launch's CTA shape), a
// batch of its cases, and where its scratch sits in a CTA's region.
// 256-byte aligned, so an array of jobs has one stride on the host and the device and no two
// jobs share a cache line.
struct alignas(256) Job {
    DevPlan P;
    DevPlan P1;              // the same topology with the one-slot schedule of the launch's CTA size
    Batch B;
    ScratchOffsets off;
    int G, log2G;            // case slots per CTA for this job (the schedule has NT / G workers)
    int seq;                 // its index in the launch's job array (checked by stream launches)
};
static_assert(sizeof(Job) % 256 == 0, "jobs are laid out at a 256-byte stride");

// A stream launch's job ring: the host appends job descriptors while the kernel runs and then
// raises `published` (both by copies on one stream, so a job's descriptor and inputs are in
// device memory before its index is published). The kernel serves published jobs in order,
// counts every job's written-back cases and, when a job is complete, sets its flag in
// page-locked host memory. A CTA that finds no open job polls, sleeping `sleep_ns` between
// polls, until `stop` is set or `idle_polls` polls have passed (then it sets status 1 and
// returns): no wait is unbounded.
struct Ring {
    const int* published;    // device: jobs published so far (null: not a stream launch)
    const int* stop;         // device: 1 once no more jobs will be published
    int* status;             // device: 1 if a CTA returned at its idle limit, 2 if a descriptor was not
                             // the job its index says (it is then not used)
    int* done_cases;         // device, per job: cases written back
    int* host_done;          // page-locked host memory, per job: 1 once all its cases are written back
    long long idle_polls;
    unsigned sleep_ns;
};

// A launch of the persistent Newton kernel: CTAs serve the jobs in order, each job until its
// cases run out; every CTA owns `cta_bytes` of scratch, reused job after job.
struct Launch {
    const Job* jobs;         // device array (a stream launch: its ring of descriptors)
    int njobs;
    char* scratch;
    unsigned long long cta_bytes;
    int timed;               // the instantiation that counts SM cycles per phase (stats[8 .. 13])
    Ring ring;
};

// Scratch layout of a job with n buses, nv block rows, nblk blocks and G slots.
ScratchOffsets scratch_offsets(int n, int nv, int nblk, int G, bool mixed);

// host-side launchers (gbpf_kernels.cu)
cudaError_t launch_newton(const Launch& L, int grid, int threads, cudaStream_t stream);
// DC start of T cases ([bus][case] injections and angles) with the block LU of a (1024 threads,
// 1 slot) schedule: B factored once (Bx: caller's susceptances on the Ybus pattern, or null:
// from the Ybus), every case substituted; R / y hold `grid` rows of nv; piv = (min, max) pivot bits
cudaError_t launch_dc(const DevPlan& P, const double2* Bx, const double* Pinj, int T, const double* theta_bus,
                      double4_32a* fac, double2* R, double2* y, double* theta, unsigned long long* piv, int grid,
                      cudaStream_t stream);
cudaError_t launch_eval_debug(const DevPlan& P, const double2* V, const double2* Sbus, const uint8_t* pin,
                              double4_32a* Vt, double2* Et, double* Ei, float* iv32, double4_32a* blocks,
                              double2* R, cudaStream_t stream);
cudaError_t launch_v0_table(const double2* V0, int n, int check, double4_32a* tab, int* err, cudaStream_t stream);

// One shared start of a launch: the plan with its 1,024-thread, one-slot schedule, the start
// table, and where the start's injections and factors go (replicated to the G slots of the
// Newton launch that uses them).
struct StartJob {
    DevPlan P;
    const double4_32a* v0tab;
    int mixed;               // float factors (the GB300 rule's first step) or double
    int log2G;               // slots per CTA of the Newton launch (the replication)
    double rcond_min;        // pivot-ratio bound of the factorization
    double2* R0;             // [row] -(P, Q) at V0
    void* fac1;              // [blk] the factors (nblk + nv blocks)
    void* facG;              // [blk][slot] the same, once per slot
    double2* y0;             // [row] scratch of the factorization's forward pass
    double2* Et0;            // [bus] scratch: the start's (e, f), 1 / Vm
    double* Ei0;
    float* iv0;
    int* ok0;
};
// Bytes of a shared start's buffers (R0, fac1, facG, y0, Et0, Ei0, iv0, ok0), each 256-aligned.
size_t start_bytes(int n, int nv, int nblk, int G, bool mixed);
// Carves those buffers from `base` into `sj`.
void start_carve(StartJob& sj, char* base, int n, int nv, int nblk, int G, bool mixed);
// One CTA of 1,024 threads per shared start.
cudaError_t launch_start(const StartJob* jobs, int njobs, cudaStream_t stream);
cudaError_t launch_conversions(const double* in, int n, float* d2f, double* f2d, float* d2f_small);
cudaError_t launch_math(const double* in, int n, double* recip, double* s_small, double* c_small, double* s_ref,
                        double* c_ref, const double* phasor, double* rot);
// Ybus values from stamps (postproc.cu)
cudaError_t launch_ybus_gather(int nnz, int m4, const int* ptr, const int* src, const double2* stamps,
                               const double2* shunt, double2* Y, float2* Y32, cudaStream_t stream);
// islanding kernel (islands.cu): scratch 4 n ints and n u64 per CTA of `grid`
cudaError_t launch_islands(int n, int m, const int* f, const int* t, const uint8_t* live, int L, const int* out_ptr,
                           const int* out_idx, const uint8_t* is_slack, const double* prio, int reslack, int* scratch,
                           unsigned long long* best, int* labels, uint8_t* served, int* ref_bus, int* n_islands,
                           int* err, int grid, cudaStream_t stream);
// Load a kernel's code into the context now (cudaFuncGetAttributes). With lazy module loading
// a kernel is otherwise loaded at its first launch, and loading waits for the kernels running on
// the device -- for a stream launch, until it ends; the stream launch preloads every kernel that
// its submits launch.
cudaError_t preload_v0_table();
cudaError_t preload_islands();
void set_error(const std::string& msg);  // message returned by gbpf_last_error()
const void* newton_kernel_ptr(int threads);

}  // namespace gbpf
