// gbpf_kernels.cu -- GB300 (sm_103a) kernels of the batched polar Newton-Raphson solver.
//
// One PERSISTENT kernel runs the whole Newton iteration of nr_klu.cpp:569-711 on the
// device for a batch of cases (time steps, outages, scenarios). Each CTA owns G case
// "slots" and loops: refill empty slots from a global work counter -> batched 2x2-block
// LU + substitutions for the slots that take a step -> voltage update -> fused mismatch /
// Jacobian evaluation -> per-slot Armijo/convergence decision -> write back finished
// cases. Cases retire independently and their slot is refilled at once (continuous
// batching inside the launch); there is no host round trip per Newton pass (the
// reference reads a status word back every pass, nr_polar_solver.py:932-933), no
// per-iteration launches, and no inter-CTA waiting of any kind (the only cross-CTA
// operation is the atomicAdd that hands out work; a stream launch's CTAs also poll the count
// of jobs the host has published, with a bounded wait).
//
// The per-CTA working set lives in global memory and is reused case after case: factor
// blocks [blk][slot] (the G slots of one block are contiguous, so a worker's G lanes read one
// 128/256-byte line per operand), residual and step [row][slot], voltage state [bus][slot].
// At about 1 MB per slot for the 2,000-bus grid (~10 GB over all slots) it does not fit the
// 129-MB L2: a pass streams it from DRAM (ncu: ~25 % L2 hit rate), which is what the
// per-case-iteration traffic measures.
//
// Precision: mismatch, power injections and convergence norm are always double, and so is the
// voltage state. With `mixed`, a slot's Jacobian, factors and substitutions are float while its
// vote says so (the vote rules of nr_polar_kernels.cu:209-228), double otherwise; a float
// factorization that fails the pivot check is redone in double within the same step; the
// phasor rotation of a float step at a PQ bus forms its increment in float (rotate_f32).
#include <cfloat>
#include <cstdint>

#include "gbpf_device.h"

namespace gbpf {


constexpr double ARMIJO_C = 1e-4;  // nr_klu.cpp:563
constexpr int LS_MAX_TRIALS = 10;  // nr_klu.cpp:562
constexpr double CHORD_RATE = 0.1; // a chord step must cut the mismatch tenfold for another one
constexpr double JAC_LAZY = 100.0; // a float step from below this x chord_tol skips its Jacobian
                                   // (near the solution such a step lands below chord_tol)
constexpr double BIG = DBL_MAX;    // nr_klu.cpp:434 NONFINITE_NORM

__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ __forceinline__ double bitsd(unsigned long long b) { return __longlong_as_double((long long)b); }
__device__ __forceinline__ bool finite_d(double x) {
    return (dbits(x) & 0x7ff0000000000000ULL) != 0x7ff0000000000000ULL;
}

// ---- float <-> double conversions on the integer pipes. GB300 runs double-precision
// instructions, conversions included, at 1/64 of the float rate; the float Jacobian / LU
// path converts a handful of values per bus and step, so these are done by IEEE-754 bit
// manipulation instead. float -> double is exact (float subnormals flush to zero);
// double -> float truncates the mantissa (round toward zero, within one float ulp),
// flushes magnitudes below 2^-126 to zero and saturates above the float range to infinity.
__device__ __forceinline__ float d2f_fast(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const unsigned de = (hi >> 20) & 0x7ffu;
    const int ex = (int)de - 1023 + 127;
    unsigned bits;
    if (de == 0x7ffu)
        bits = sign | 0x7f800000u | (((hi & 0xfffffu) | lo) ? 0x400000u : 0u);  // Inf / NaN
    else if (ex <= 0)
        bits = sign;
    else if (ex >= 255)
        bits = sign | 0x7f800000u;
    else
        bits = sign | ((unsigned)ex << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    return __uint_as_float(bits);
}

__device__ __forceinline__ double f2d_fast(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned sign = b & 0x80000000u;
    const unsigned ex = (b >> 23) & 0xffu;
    const unsigned man = b & 0x7fffffu;
    unsigned hi, lo = 0;
    if (ex == 0)
        hi = sign;
    else if (ex == 0xffu)
        hi = sign | 0x7ff00000u | (man ? 0x80000u : 0u);
    else {
        hi = sign | ((ex + 896u) << 20) | (man >> 3);
        lo = man << 29;
    }
    return __hiloint2double((int)hi, (int)lo);
}

// double -> float by truncation for finite |x| < 2^128 (voltage components): the bits
// d2f_fast gives there, in five integer operations -- the exponent is rebased by
// subtracting (1023 - 127) << 23 from the funnel-shifted exponent / mantissa, and
// magnitudes below 2^-126 go to a signed zero
__device__ __forceinline__ float d2f_trunc(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned a = hi & 0x7fffffffu;
    const unsigned m = __funnelshift_l(lo, a, 3) - (896u << 23);
    return __uint_as_float((hi & 0x80000000u) | (a >= (897u << 20) ? m : 0u));
}

// |x| as ordered bits (sign cleared): compares like the magnitudes, NaN above everything
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
}

// cos/sin of a small angle |d| <= 1/4 from their Maclaurin series (Horner in d^2), with as
// many terms as |d| needs (the first dropped term stays below double rounding); the
// truncation error is below 3e-18 on the whole range. Used to ROTATE a bus phasor by the
// Newton angle increment instead of evaluating sincos of the full angle.
__device__ __forceinline__ void sincos_small(double d, unsigned ahi, double* s, double* c) {
    const double z = d * d;
    if (ahi < 0x3F100000u) {  // |d| < 2^-14  // next terms below 2^-100: d^5/120 and d^4/24
        *s = fma(z * (-1.0 / 6.0), d, d);
        *c = fma(z, -0.5, 1.0);
        return;
    }
    if (ahi < 0x3F900000u) {  // |d| < 2^-6: next terms below 2^-60 relative: d^9/9! and d^8/8!
        double ps = -1.0 / 5040.0;
        ps = fma(ps, z, 1.0 / 120.0);
        ps = fma(ps, z, -1.0 / 6.0);
        *s = fma(ps * z, d, d);
        double pc = -1.0 / 720.0;
        pc = fma(pc, z, 1.0 / 24.0);
        pc = fma(pc, z, -0.5);
        *c = fma(pc, z, 1.0);
        return;
    }
    double ps = -1.0 / 39916800.0;
    ps = fma(ps, z, 1.0 / 362880.0);
    ps = fma(ps, z, -1.0 / 5040.0);
    ps = fma(ps, z, 1.0 / 120.0);
    ps = fma(ps, z, -1.0 / 6.0);
    *s = fma(ps * z, d, d);
    double pc = 1.0 / 479001600.0;
    pc = fma(pc, z, -1.0 / 3628800.0);
    pc = fma(pc, z, 1.0 / 40320.0);
    pc = fma(pc, z, -1.0 / 720.0);
    pc = fma(pc, z, 1.0 / 24.0);
    pc = fma(pc, z, -0.5);
    *c = fma(pc, z, 1.0);
}

// Rotation of a unit phasor (c, s) by a small angle d (|d| < 1/4) whose increment
// (c + js)(cos d - 1 + j sin d) is formed in float -- sin d - d and cos d - 1 from their
// Maclaurin series in d^2 (Horner; the first term left out is below 2^-30 relative) -- and
// added to the double phasor: within ~2^-21 |d| of the exact rotation, against ~1e-16 for
// sincos_small. For the mixed path's steps solved with float factors at PQ buses: such a
// step is itself off by ~cond(J) 2^-24 relative, and the Newton steps that follow correct
// both the angle and the magnitude of a PQ bus (a PV bus's magnitude is never corrected, so
// PV buses keep the double rotation).
__device__ __forceinline__ void rotate_f32(double c, double s, double d, double* cs, double* sn) {
    const float df = d2f_fast(d);
    const float z = df * df;
    const float sm = df * z * fmaf(fmaf(z, -1.f / 5040.f, 1.f / 120.f), z, -1.f / 6.f);               // sin d - d
    const float cm = z * fmaf(fmaf(fmaf(z, 1.f / 40320.f, -1.f / 720.f), z, 1.f / 24.f), z, -0.5f);  // cos d - 1
    const float c32 = d2f_trunc(c), s32 = d2f_trunc(s);
    const float sd = df + sm;
    *cs = c + f2d_fast(fmaf(c32, cm, -s32 * sd));
    *sn = s + f2d_fast(fmaf(s32, cm, c32 * sd));
}

// --------------------------------------------------------------------------------------
// Evaluation of one bus row for one slot, rectangular state e + jf = V.
//   I_i = sum_j Y_ij V_j                      (4 double FMAs per entry)
//   P_i + jQ_i = V_i conj(I_i),   residual R = S_spec - (P_i + jQ_i)
// The mismatch is computed with the same instructions in every mode, so the float and the
// double Jacobian paths see bit-identical residuals. Off-diagonal Jacobian block (i, j), with
// W = V_i conj(Y_ij V_j) (its real / imaginary part: the P / Q flow term of the entry):
//   [dP/dth_j dP/dVm_j; dQ/dth_j dQ/dVm_j] = [Im W, Re W / Vm_j; -Re W, Im W / Vm_j]
// and the diagonal block follows from P_i, Q_i and the self term S_ii = |V_i|^2 conj(Y_ii):
//   dP/dth_i = Q_ii - Q_i, dQ/dth_i = P_i - P_ii, dP/dVm_i = (P_i + P_ii)/Vm_i, dQ/dVm_i = (Q_i + Q_ii)/Vm_i
// -- the derivative formulas of nr_klu.cpp:344-378 (polar form, accumulated per entry there)
// rewritten without per-entry trigonometry. PV buses carry an identity dummy in their
// magnitude column and Q row; pinned buses (nr_klu.cpp:398-423) get identity rows and a
// zero residual. JM: 0 = mismatch only, 1 = double Jacobian, 2 = float Jacobian.
// --------------------------------------------------------------------------------------
struct EvalCtx {
    const DevPlan* P;
    const double2* Et;   // [bus][slot] (e, f)
    const double* Ei;    // [bus][slot] 1 / Vm
    const float* iv32;   // [bus][slot] 1 / Vm in float (PQ buses)
    int lg;
    int ymode;
    const double2* Yd;
    long long sYd;
    int ncase;
    int nst;
    const int* stk;
    const double2* stv;
};

__device__ __forceinline__ unsigned row_stamp_mask(const EvalCtx& c, int k0, int k1) {
    unsigned mask = 0;
    if (c.ymode == 1)
        for (int e = 0; e < c.nst; ++e)
            if (c.stk[e] >= k0 && c.stk[e] < k1) mask |= 1u << e;
    return mask;
}

__device__ __forceinline__ double2 ybus_val(const EvalCtx& c, int k, unsigned mask) {
    double2 y = c.ymode == 2 ? c.Yd[(size_t)k * c.sYd + c.ncase] : __ldg(&c.P->Y[k]);
    if (mask) {
        for (int e = 0; e < c.nst; ++e)
            if (((mask >> e) & 1u) && c.stk[e] == k) {
                y.x -= c.stv[e].x;
                y.y -= c.stv[e].y;
            }
    }
    return y;
}

__device__ __forceinline__ void put_block(double4_32a* fac, size_t at, double a, double b, double c, double d) {
    fac[at] = make_double4_32a(a, b, c, d);
}
__device__ __forceinline__ void put_block(float4* fac, size_t at, double a, double b, double c, double d) {
    fac[at] = make_float4((float)a, (float)b, (float)c, (float)d);
}

template <int JM, typename FacT>
__device__ unsigned long long eval_row(const EvalCtx& c, int i, int s, int row, bool pinned, bool pq_i, double2 Ssp,
                                       FacT* fac, double2* R, bool write_r) {
    const DevPlan& P = *c.P;
    const size_t si = ((size_t)i << c.lg) + s;
    const double2 ei = c.Et[si];
    // float copy of the evaluation point for the float Jacobian: (e, f) truncated from the
    // double phasor, 1 / Vm from its float array (read for PQ buses only)
    float4 vi32 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (JM == 2) vi32 = make_float4(d2f_trunc(ei.x), d2f_trunc(ei.y), pq_i ? c.iv32[si] : 0.f, 0.f);
    double Ir = 0.0, Ii = 0.0, gii = 0.0, bii = 0.0;
    float gii32 = 0.f, bii32 = 0.f;
    const int k0 = __ldg(&P.Yp[i]), k1 = __ldg(&P.Yp[i + 1]);
    const unsigned mask = row_stamp_mask(c, k0, k1);
    // the next nonzero's column and phasor are loaded while this one is worked on (the stores
    // of the Jacobian blocks would otherwise keep them from being issued early)
    int jn = k0 < k1 ? __ldg(&P.Yj[k0]) : 0;
    double2 en = k0 < k1 ? c.Et[((size_t)jn << c.lg) + s] : make_double2(0.0, 0.0);
    for (int k = k0; k < k1; ++k) {
        const int j = jn;
        const double2 ej = en;
        if (k + 1 < k1) {
            jn = __ldg(&P.Yj[k + 1]);
            en = c.Et[((size_t)jn << c.lg) + s];
        }
        const double2 y = ybus_val(c, k, mask);
        const size_t sj = ((size_t)j << c.lg) + s;
        Ir = fma(y.x, ej.x, Ir);
        Ir = fma(-y.y, ej.y, Ir);
        Ii = fma(y.x, ej.y, Ii);
        Ii = fma(y.y, ej.x, Ii);
        if (j == i) {
            gii = y.x;
            bii = y.y;
            if (JM == 2) {
                if (c.ymode == 0) {
                    const float2 y32 = __ldg(&P.Y32[k]);
                    gii32 = y32.x;
                    bii32 = y32.y;
                } else {
                    gii32 = d2f_fast(y.x);
                    bii32 = d2f_fast(y.y);
                }
            }
            continue;
        }
        if (JM == 0) continue;
        const int q = __ldg(&P.posmap[k]);
        if (q < 0) continue;
        const bool pq_j = __ldg(&P.bus_pq[j]) != 0;
        const size_t at = ((size_t)q << c.lg) + s;
        if (pinned) {
            put_block(fac, at, 0.0, 0.0, 0.0, 0.0);
            continue;
        }
        if (JM == 1) {
            const double wr = fma(-y.y, ej.y, y.x * ej.x), wi = fma(y.y, ej.x, y.x * ej.y);
            const double Wr = fma(ei.x, wr, ei.y * wi), Wi = fma(ei.y, wr, -ei.x * wi);
            const double ivj = c.Ei[sj];
            put_block(fac, at, Wi, pq_j ? Wr * ivj : 0.0, pq_i ? -Wr : 0.0, (pq_i && pq_j) ? Wi * ivj : 0.0);
        } else {
            float gx, gy;
            if (c.ymode == 0) {
                const float2 y32 = __ldg(&P.Y32[k]);
                gx = y32.x;
                gy = y32.y;
            } else {
                gx = d2f_fast(y.x);
                gy = d2f_fast(y.y);
            }
            const float4 vj = make_float4(d2f_trunc(ej.x), d2f_trunc(ej.y), pq_j ? c.iv32[sj] : 0.f, 0.f);
            const float wr = fmaf(-gy, vj.y, gx * vj.x), wi = fmaf(gy, vj.x, gx * vj.y);
            const float Wr = fmaf(vi32.x, wr, vi32.y * wi), Wi = fmaf(vi32.y, wr, -vi32.x * wi);
            reinterpret_cast<float4*>(fac)[at] =
                make_float4(Wi, pq_j ? Wr * vj.z : 0.f, pq_i ? -Wr : 0.f, (pq_i && pq_j) ? Wi * vj.z : 0.f);
        }
    }
    const double Pc = fma(ei.x, Ir, ei.y * Ii);
    const double Qc = fma(ei.y, Ir, -ei.x * Ii);
    if (JM == 1) {
        const size_t at = ((size_t)P.dpos[row] << c.lg) + s;
        if (pinned) {
            put_block(fac, at, 1.0, 0.0, 0.0, 1.0);
        } else {
            const double vi2 = fma(ei.x, ei.x, ei.y * ei.y);
            const double Ps = vi2 * gii, Qs = -vi2 * bii;
            const double ivi = c.Ei[si];
            put_block(fac, at, Qs - Qc, pq_i ? (Pc + Ps) * ivi : 0.0, pq_i ? Pc - Ps : 0.0,
                      pq_i ? (Qc + Qs) * ivi : 1.0);
        }
    } else if (JM == 2) {  // float diagonal block from float copies: no double arithmetic
        const size_t at = ((size_t)P.dpos[row] << c.lg) + s;
        float4 o;
        if (pinned) {
            o = make_float4(1.f, 0.f, 0.f, 1.f);
        } else {
            const float P32 = d2f_fast(Pc), Q32 = d2f_fast(Qc);
            const float vi2 = fmaf(vi32.x, vi32.x, vi32.y * vi32.y);
            const float Ps = vi2 * gii32, Qs = -vi2 * bii32;
            o = make_float4(Qs - Q32, pq_i ? (P32 + Ps) * vi32.z : 0.f, pq_i ? P32 - Ps : 0.f,
                            pq_i ? (Q32 + Qs) * vi32.z : 1.f);
        }
        reinterpret_cast<float4*>(fac)[at] = o;
    }
    const double rp = pinned ? 0.0 : Ssp.x - Pc;
    const double rq = (pinned || !pq_i) ? 0.0 : Ssp.y - Qc;
    if (write_r) R[((size_t)row << c.lg) + s] = make_double2(rp, rq);
    const unsigned long long a = abs_bits(rp), b = abs_bits(rq);
    return b > a ? b : a;
}

// Reciprocal of a positive double: float seed refined by two Newton-Raphson steps
// r <- r (2 - x r) (quadratic convergence: ~2^-24 -> 2^-48 -> below double rounding).
__device__ __forceinline__ double recip_nr(double x) {
    double r = (double)__frcp_rn((float)x);
    r = r * fma(-x, r, 2.0);
    r = r * fma(-x, r, 2.0);
    return r;
}

// Acquire load at GPU scope (a flag or count another agent writes) and release store at system
// scope (a flag the host reads).
__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_sys(int* p, int v) {
    asm volatile("st.release.sys.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// The next job a CTA serves (thread 0; -1: none left): the first job from *next_job on whose
// work counter is below its units. In a stream launch (published != null), a CTA that finds
// none polls until `stop` is set or no job has been published for idle_polls polls (status 1):
// every newly published job starts the idle window again, so the CTAs leave together, after
// the stream has been quiet for the whole window. Kept out of line: it runs once per job, and
// inlined its temporaries would crowd the solve's registers.
__device__ __noinline__ int bind_job(const Job* jobs, int njobs, const int* published, const int* stop, int* status,
                                     long long idle_polls, unsigned sleep_ns, int* next_job) {
    long long polls = 0;
    int seen = -1;
    for (;;) {
        // a stream launch: `stop` is read before `published` (the host raises it last)
        const bool stopping = published && ld_acquire(stop) != 0;
        const int pub = published ? ld_acquire(published) : njobs;
        if (pub != seen) {
            seen = pub;
            polls = 0;
        }
        for (; *next_job < pub; ++*next_job) {
            if (published && __ldcg(&jobs[*next_job].seq) != *next_job) {  // never use a wrong descriptor
                atomicExch(status, 2);
                return -1;
            }
            const Batch* b = &jobs[*next_job].B;
            const int* cnt = reinterpret_cast<const int*>(__ldcg(reinterpret_cast<const unsigned long long*>(&b->counter)));
            const int units = __ldcg(&b->lanes) ? __ldcg(&b->K) : __ldcg(&b->B);
            if (*(volatile const int*)cnt < units) return (*next_job)++;
        }
        if (!published || stopping) return -1;
        if (++polls > idle_polls) {  // no job for the whole idle window: return
            atomicCAS(status, 0, 1);
            return -1;
        }
        __nanosleep(sleep_ns);
    }
}

// A load of a job's staged input: past L1 in a stream launch, whose staging memory is refilled
// (by the copy engine, for a later job) while the kernel runs.
template <bool RING, typename T>
__device__ __forceinline__ T ld_in(const T* p) {
    if constexpr (RING) return __ldcg(p);
    else return *p;
}
__device__ __forceinline__ double4_32a ldcg4(const double4_32a* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    const double2 a = __ldcg(q), b = __ldcg(q + 1);
    return make_double4_32a(a.x, a.y, b.x, b.y);
}

// Per-phase clock (timed launches only): thread 0, just past a barrier that ends phase k, adds
// the SM cycles since the previous mark to the CTA's counter of phase k.
__device__ __forceinline__ void phase_mark(unsigned long long* ph, long long* clk, int k) {
    if (ph && threadIdx.x == 0) {
        const long long now = clock64();
        ph[k] += (unsigned long long)(now - *clk);
        *clk = now;
    }
}

// ---------------------------------------------------------------------------- block LU
template <typename T>
struct V4;
template <>
struct V4<double> {
    using t = double4_32a;
    using t2 = double2;
};
template <>
struct V4<float> {
    using t = float4;
    using t2 = float2;
};

template <typename T>
__device__ __forceinline__ T z4() {
    T r;
    r.x = r.y = r.z = r.w = 0;
    return r;
}

// Arithmetic of the factorization and substitutions with its rounding pinned: explicit fused
// multiply-adds, so every copy of the code (a case's own factorization, the shared start's,
// any CTA shape) rounds alike, and each 2x2 product costs two fused operations per entry.
__device__ __forceinline__ float fmadd(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmadd(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mulr(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mulr(double a, double b) { return __dmul_rn(a, b); }

// acc -= a * b (2x2 blocks, row-major)
template <typename B4>
__device__ __forceinline__ void mm_sub(B4& acc, const B4& a, const B4& b) {
    acc.x = fmadd(-a.y, b.z, fmadd(-a.x, b.x, acc.x));
    acc.y = fmadd(-a.y, b.w, fmadd(-a.x, b.y, acc.y));
    acc.z = fmadd(-a.w, b.z, fmadd(-a.z, b.x, acc.z));
    acc.w = fmadd(-a.w, b.w, fmadd(-a.z, b.y, acc.w));
}

// One batched factorization + substitution pass over the slots flagged in `on` (G <= 32).
// Worker w = (warp, lane / G) runs its task list of every level for its G slot lanes;
// the CTA meets at a barrier after each level, forward and backward. Pivot statistics per
// slot go to smin / smax (as ordered bits). With `solo` a slot index, P is the one-slot
// schedule and all threads work on that slot. Slots flagged in `chord` keep the factors already
// in `fac` and run the substitutions only; when every slot of the CTA does (factor_any false),
// the workers walk the substitution-only lists instead of skipping factor tasks one by one.
template <typename real, bool TIMED = false>
__device__ void lu_pass(const DevPlan& P, typename V4<real>::t* fac, const double2* R, typename V4<real>::t2* y,
                        const int* on, int lg, unsigned long long* smin, unsigned long long* smax,
                        const int* chord, bool factor_any, typename V4<real>::t* dinv_smem, int solo = -1,
                        unsigned long long* ph = nullptr, long long* clk = nullptr) {
    using B4 = typename V4<real>::t;
    using B2 = typename V4<real>::t2;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    // solo >= 0: one slot left in the CTA; P then carries the one-slot schedule (a worker per
    // thread) and every thread works on that slot
    const int s = solo >= 0 ? solo : lane & ((1 << lg) - 1);
    const int w = solo >= 0 ? tid : (tid >> 5) * (32 >> lg) + (lane >> lg);
    const int W = P.W;
    const bool act = on[s] != 0;
    const bool factor = !(chord && chord[s]);
    // float passes take each task's first two pairs from its head record (the double pass
    // keeps its registers for the wider blocks)
    constexpr bool HEAD = sizeof(real) == 4;
    real pmin = sizeof(real) == 4 ? (real)FLT_MAX : (real)DBL_MAX, pmax = 0;
    B4 dinv = z4<B4>();  // the worker's last inverse diagonal block: scales the L column after it
    for (int h = 0; h < P.nlev; ++h) {
        if (act) {
            const int* const PA = factor_any ? P.ptrA : P.ptrF;
            const int4* const TA = factor_any ? P.taskA : P.taskF;
            const int4* const HA = factor_any ? P.headA : P.headF;
            const int t0 = __ldg(&PA[h * W + w]), t1 = __ldg(&PA[h * W + w + 1]);
            // the next task's record and first two pairs are fetched while the current one
            // runs, so a task's block loads all go out at once when it starts
            int4 next = make_int4(0, 0, 0, 0), nhead = make_int4(0, 0, 0, 0);
            if (t0 < t1) {
                next = __ldg(&TA[t0]);
                if constexpr (HEAD) nhead = __ldg(&HA[t0]);
            }
            for (int t = t0; t < t1; ++t) {
                const int4 task = next, hd = nhead;
                if (t + 1 < t1) {
                    next = __ldg(&TA[t + 1]);
                    if constexpr (HEAD) nhead = __ldg(&HA[t + 1]);
                }
                const int kind = task.y & 3;
                const int np = HEAD ? min(task.w - task.z, 2) : 0;  // pairs taken from the head
                if (kind != 3 && !factor) continue;
                if (kind == 3) {  // forward substitution of block row task.x
                    const double2 r = R[((size_t)task.x << lg) + s];
                    real y0, y1;
                    if constexpr (sizeof(real) == 4) {
                        y0 = d2f_fast(r.x);
                        y1 = d2f_fast(r.y);
                    } else {
                        y0 = r.x;
                        y1 = r.y;
                    }
                    if (np > 0) {
                        const B4 l0 = fac[((size_t)hd.x << lg) + s];
                        const B2 u0 = y[((size_t)hd.y << lg) + s];
                        B4 l1 = z4<B4>();
                        B2 u1 = {};
                        if (np > 1) {
                            l1 = fac[((size_t)hd.z << lg) + s];
                            u1 = y[((size_t)hd.w << lg) + s];
                        }
                        y0 = fmadd(-l0.y, u0.y, fmadd(-l0.x, u0.x, y0));
                        y1 = fmadd(-l0.w, u0.y, fmadd(-l0.z, u0.x, y1));
                        if (np > 1) {
                            y0 = fmadd(-l1.y, u1.y, fmadd(-l1.x, u1.x, y0));
                            y1 = fmadd(-l1.w, u1.y, fmadd(-l1.z, u1.x, y1));
                        }
                    }
                    int p = task.z + np;
                    int2 n0 = make_int2(0, 0), n1 = make_int2(0, 0);
                    if (p < task.w) n0 = __ldg(&P.pairs[p]);
                    if (p + 1 < task.w) n1 = __ldg(&P.pairs[p + 1]);
                    for (; p + 1 < task.w; p += 2) {
                        const int2 q0 = n0, q1 = n1;
                        if (p + 2 < task.w) n0 = __ldg(&P.pairs[p + 2]);
                        if (p + 3 < task.w) n1 = __ldg(&P.pairs[p + 3]);
                        const B4 l0 = fac[((size_t)q0.x << lg) + s], l1 = fac[((size_t)q1.x << lg) + s];
                        const B2 u0 = y[((size_t)q0.y << lg) + s], u1 = y[((size_t)q1.y << lg) + s];
                        y0 = fmadd(-l0.y, u0.y, fmadd(-l0.x, u0.x, y0));
                        y1 = fmadd(-l0.w, u0.y, fmadd(-l0.z, u0.x, y1));
                        y0 = fmadd(-l1.y, u1.y, fmadd(-l1.x, u1.x, y0));
                        y1 = fmadd(-l1.w, u1.y, fmadd(-l1.z, u1.x, y1));
                    }
                    if (p < task.w) {
                        const int2 q0 = n0;
                        const B4 l0 = fac[((size_t)q0.x << lg) + s];
                        const B2 u0 = y[((size_t)q0.y << lg) + s];
                        y0 = fmadd(-l0.y, u0.y, fmadd(-l0.x, u0.x, y0));
                        y1 = fmadd(-l0.w, u0.y, fmadd(-l0.z, u0.x, y1));
                    }
                    B2 o;
                    o.x = y0;
                    o.y = y1;
                    y[((size_t)task.x << lg) + s] = o;
                    continue;
                }
                B4 acc = (task.y & 16) ? z4<B4>() : fac[((size_t)task.x << lg) + s];
                if (np > 0) {
                    const B4 a0 = fac[((size_t)hd.x << lg) + s], b0 = fac[((size_t)hd.y << lg) + s];
                    if (np > 1) {
                        const B4 a1 = fac[((size_t)hd.z << lg) + s], b1 = fac[((size_t)hd.w << lg) + s];
                        mm_sub(acc, a0, b0);
                        mm_sub(acc, a1, b1);
                    } else {
                        mm_sub(acc, a0, b0);
                    }
                }
                // the next two pairs' indices are fetched while this iteration's blocks load
                int p = task.z + np;
                int2 n0 = make_int2(0, 0), n1 = make_int2(0, 0);
                if (p < task.w) n0 = __ldg(&P.pairs[p]);
                if (p + 1 < task.w) n1 = __ldg(&P.pairs[p + 1]);
                for (; p + 1 < task.w; p += 2) {
                    const int2 q0 = n0, q1 = n1;
                    if (p + 2 < task.w) n0 = __ldg(&P.pairs[p + 2]);
                    if (p + 3 < task.w) n1 = __ldg(&P.pairs[p + 3]);
                    const B4 a0 = fac[((size_t)q0.x << lg) + s], b0 = fac[((size_t)q0.y << lg) + s];
                    const B4 a1 = fac[((size_t)q1.x << lg) + s], b1 = fac[((size_t)q1.y << lg) + s];
                    mm_sub(acc, a0, b0);
                    mm_sub(acc, a1, b1);
                }
                if (p < task.w) {
                    const int2 q0 = n0;
                    mm_sub(acc, fac[((size_t)q0.x << lg) + s], fac[((size_t)q0.y << lg) + s]);
                }
                if (kind == 0) {  // diagonal block: its inverse, kept for the L blocks that follow
                    const real det = fmadd(acc.x, acc.w, -mulr(acc.y, acc.z));
                    const real inv = (real)1 / det;
                    dinv.x = acc.w * inv;
                    dinv.y = -acc.y * inv;
                    dinv.z = -acc.z * inv;
                    dinv.w = acc.x * inv;
                    if (dinv_smem) dinv_smem[tid] = dinv;
                    // a chain segment's copy (TASK_NOSTORE) only recomputes it; the task itself
                    // records the pivots (a00 and det / a00) and stores the inverse apart, at
                    // block nblk + row (the Jacobian's diagonal stays for the copies)
                    if (!(task.y & 64)) {
                        const real u0 = fabs(acc.x);
                        pmin = fmin(pmin, u0);
                        pmax = (u0 > pmax || u0 != u0) ? u0 : pmax;
                        if (task.y & 32) {
                            const real u1 = fabs(det / acc.x);
                            pmin = fmin(pmin, u1);
                            pmax = (u1 > pmax || u1 != u1) ? u1 : pmax;
                        }
                        fac[((size_t)(P.nblk + (task.y >> 8)) << lg) + s] = dinv;
                    }
                } else if (task.y & 8) {  // L block: scaled by its column's inverse diagonal
                    B4 o;
                    const B4 dv = dinv_smem ? dinv_smem[tid] : dinv;
                    o.x = fmadd(acc.x, dv.x, mulr(acc.y, dv.z));
                    o.y = fmadd(acc.x, dv.y, mulr(acc.y, dv.w));
                    o.z = fmadd(acc.z, dv.x, mulr(acc.w, dv.z));
                    o.w = fmadd(acc.z, dv.y, mulr(acc.w, dv.w));
                    fac[((size_t)task.x << lg) + s] = o;
                } else {
                    fac[((size_t)task.x << lg) + s] = acc;
                }
            }
        }
        __syncthreads();
    }
    if constexpr (TIMED) phase_mark(ph, clk, 1);
    for (int h = 0; h < P.nblev; ++h) {
        if (act) {
            const int t0 = __ldg(&P.ptrC[h * W + w]), t1 = __ldg(&P.ptrC[h * W + w + 1]);
            int4 next = make_int4(0, 0, 0, 0), nhead = make_int4(0, 0, 0, 0);
            if (t0 < t1) {
                next = __ldg(&P.taskC[t0]);
                if constexpr (HEAD) nhead = __ldg(&P.headC[t0]);
            }
            for (int t = t0; t < t1; ++t) {
                const int4 task = next, hd = nhead;
                if (t + 1 < t1) {
                    next = __ldg(&P.taskC[t + 1]);
                    if constexpr (HEAD) nhead = __ldg(&P.headC[t + 1]);
                }
                const int np = HEAD ? min(task.w - task.z, 2) : 0;  // pairs taken from the head
                const B2 yr = y[((size_t)task.x << lg) + s];
                const B4 d = fac[((size_t)task.y << lg) + s];
                real r0 = yr.x, r1 = yr.y;
                if (np > 0) {
                    const B4 u0 = fac[((size_t)hd.x << lg) + s];
                    const B2 y0 = y[((size_t)hd.y << lg) + s];
                    B4 u1 = z4<B4>();
                    B2 y1 = {};
                    if (np > 1) {
                        u1 = fac[((size_t)hd.z << lg) + s];
                        y1 = y[((size_t)hd.w << lg) + s];
                    }
                    r0 = fmadd(-u0.y, y0.y, fmadd(-u0.x, y0.x, r0));
                    r1 = fmadd(-u0.w, y0.y, fmadd(-u0.z, y0.x, r1));
                    if (np > 1) {
                        r0 = fmadd(-u1.y, y1.y, fmadd(-u1.x, y1.x, r0));
                        r1 = fmadd(-u1.w, y1.y, fmadd(-u1.z, y1.x, r1));
                    }
                }
                int p = task.z + np;
                int2 n0 = make_int2(0, 0), n1 = make_int2(0, 0);
                if (p < task.w) n0 = __ldg(&P.pairs[p]);
                if (p + 1 < task.w) n1 = __ldg(&P.pairs[p + 1]);
                for (; p + 1 < task.w; p += 2) {
                    const int2 q0 = n0, q1 = n1;
                    if (p + 2 < task.w) n0 = __ldg(&P.pairs[p + 2]);
                    if (p + 3 < task.w) n1 = __ldg(&P.pairs[p + 3]);
                    const B4 u0 = fac[((size_t)q0.x << lg) + s], u1 = fac[((size_t)q1.x << lg) + s];
                    const B2 y0 = y[((size_t)q0.y << lg) + s], y1 = y[((size_t)q1.y << lg) + s];
                    r0 = fmadd(-u0.y, y0.y, fmadd(-u0.x, y0.x, r0));
                    r1 = fmadd(-u0.w, y0.y, fmadd(-u0.z, y0.x, r1));
                    r0 = fmadd(-u1.y, y1.y, fmadd(-u1.x, y1.x, r0));
                    r1 = fmadd(-u1.w, y1.y, fmadd(-u1.z, y1.x, r1));
                }
                if (p < task.w) {
                    const int2 q0 = n0;
                    const B4 u0 = fac[((size_t)q0.x << lg) + s];
                    const B2 y0 = y[((size_t)q0.y << lg) + s];
                    r0 = fmadd(-u0.y, y0.y, fmadd(-u0.x, y0.x, r0));
                    r1 = fmadd(-u0.w, y0.y, fmadd(-u0.z, y0.x, r1));
                }
                B2 o;
                o.x = fmadd(d.x, r0, mulr(d.y, r1));
                o.y = fmadd(d.z, r0, mulr(d.w, r1));
                y[((size_t)task.x << lg) + s] = o;
            }
        }
        __syncthreads();
    }
    if (act) {
        double dmin, dmax;
        if constexpr (sizeof(real) == 4) {
            dmin = f2d_fast((float)pmin);
            dmax = f2d_fast((float)pmax);
        } else {
            dmin = pmin;
            dmax = pmax;
        }
        atomicMin(&smin[s], dbits(dmin));
        atomicMax(&smax[s], dbits(dmax));
    }
    __syncthreads();
    if constexpr (TIMED) phase_mark(ph, clk, 2);
}

__device__ __forceinline__ bool pivots_ok(unsigned long long bmin, unsigned long long bmax, double rc) {
    if (bmax >= 0x7ff0000000000000ULL) return false;  // NaN / Inf pivot
    const double mn = bitsd(bmin), mx = bitsd(bmax);
    return mn > 0.0 && mn >= rc * mx;
}

// ------------------------------------------------------------------------- the kernel
// NTB threads per CTA and 1024 / NTB resident CTAs per SM (64 registers per thread in
// every variant): smaller CTAs let one CTA's latency-bound factorization overlap another's
// double-precision evaluation on the same SM.
template <int NTB, bool TIMED, bool RING>
__global__ void __launch_bounds__(NTB, 1024 / NTB) newton_kernel(const Launch L) {
    const int tid = threadIdx.x;
    const int NT = blockDim.x;
    char* const region = L.scratch + (size_t)blockIdx.x * L.cta_bytes;
    __shared__ DevPlan s_plan;
    __shared__ DevPlan s_plan1;  // the same topology with the one-slot schedule (solo passes)
    __shared__ Batch s_batch;
    __shared__ int s_solo;
    __shared__ double4_32a s_dinv64[NTB];  // double passes: each worker's inverse diagonal (off the registers)
    __shared__ int s_job;
    __shared__ ScratchOffsets s_off;
    __shared__ int s_G, s_lg, s_fin;
    int next_job = 0;  // thread 0: first job this CTA has not finished yet
    if (tid == 0) s_fin = 0;
    for (;;) {
    // ------------------------------------------------------------------ bind the next job
    // Jobs are taken in order; a job is open while its work counter is below its units.
    // Every CTA that finds a job open serves it until the job runs out of cases. Descriptors
    // are read past L1 (a stream launch's descriptors are written while the kernel runs).
    if constexpr (RING) {
        if (tid == 0)
            s_job = bind_job(L.jobs, L.njobs, L.ring.published, L.ring.stop, L.ring.status, L.ring.idle_polls,
                             L.ring.sleep_ns, &next_job);
    } else if (tid == 0) {
        int sel = -1;
        for (; next_job < L.njobs; ++next_job) {
            const Batch& b = L.jobs[next_job].B;
            if (*(volatile const int*)b.counter < (b.lanes ? b.K : b.B)) {
                sel = next_job++;
                break;
            }
        }
        s_job = sel;
    }
    __syncthreads();
    const int job = s_job;
    if (job < 0) break;
    {
        // (a stream launch's descriptors are written while the kernel runs: read past L1)
        const int* src = reinterpret_cast<const int*>(&L.jobs[job].P);
        int* dst = reinterpret_cast<int*>(&s_plan);
        for (int w = tid; w < (int)(sizeof(DevPlan) / 4); w += NT) dst[w] = RING ? __ldcg(src + w) : src[w];
        src = reinterpret_cast<const int*>(&L.jobs[job].B);
        dst = reinterpret_cast<int*>(&s_batch);
        for (int w = tid; w < (int)(sizeof(Batch) / 4); w += NT) dst[w] = RING ? __ldcg(src + w) : src[w];
        src = reinterpret_cast<const int*>(&L.jobs[job].P1);
        dst = reinterpret_cast<int*>(&s_plan1);
        for (int w = tid; w < (int)(sizeof(DevPlan) / 4); w += NT) dst[w] = RING ? __ldcg(src + w) : src[w];
        if constexpr (RING) {
            src = reinterpret_cast<const int*>(&L.jobs[job].off);
            dst = reinterpret_cast<int*>(&s_off);
            for (int w = tid; w < (int)(sizeof(ScratchOffsets) / 4); w += NT) dst[w] = __ldcg(src + w);
            if (tid == 0) {
                s_G = __ldcg(&L.jobs[job].G);
                s_lg = __ldcg(&L.jobs[job].log2G);
            }
        }
    }
    if constexpr (RING) __syncthreads();
    const ScratchOffsets& off = RING ? s_off : L.jobs[job].off;
    const int G = RING ? s_G : L.jobs[job].G, lg = RING ? s_lg : L.jobs[job].log2G;  // case slots of this job's CTAs
    double4_32a* fac64 = reinterpret_cast<double4_32a*>(region + off.fac64);
    float4* fac32 = off.fac32 != ~0ULL ? reinterpret_cast<float4*>(region + off.fac32) : nullptr;
    float4* fac32b = off.fac32b != ~0ULL ? reinterpret_cast<float4*>(region + off.fac32b) : nullptr;
    double2* R = reinterpret_cast<double2*>(region + off.R);
    double2* y64 = reinterpret_cast<double2*>(region + off.y64);
    float2* y32 = off.y32 != ~0ULL ? reinterpret_cast<float2*>(region + off.y32) : nullptr;
    // two state buffers per slot: the last evaluated point lives in Vb[s_tb[s]], the committed
    // point (while a line search backtracks) in the other -- accepting a step flips s_tb
    // instead of copying the state
    double4_32a* const Vb0 = reinterpret_cast<double4_32a*>(region + off.Vc);
    double4_32a* const Vb1 = reinterpret_cast<double4_32a*>(region + off.Vt);
    double2* Et = reinterpret_cast<double2*>(region + off.Et);
    double* Ei = reinterpret_cast<double*>(region + off.Ei);
    float* iv32 = reinterpret_cast<float*>(region + off.iv32);
    uint8_t* spin = reinterpret_cast<uint8_t*>(region + off.pin);
    __syncthreads();
    const DevPlan& P = s_plan;
    const Batch& Bt = s_batch;
    const int n = P.n;
    const int nG = n << lg;

    __shared__ int s_st[MAX_SLOTS], s_case[MAX_SLOTS], s_it[MAX_SLOTS], s_vote[MAX_SLOTS], s_trial[MAX_SLOTS];
    __shared__ int s_conv[MAX_SLOTS], s_jprec[MAX_SLOTS], s_yprec[MAX_SLOTS], s_warm[MAX_SLOTS];
    __shared__ int s_on32[MAX_SLOTS], s_on64[MAX_SLOTS], s_reeval[MAX_SLOTS];
    // s_nojac: the slot's last evaluation left the float Jacobian out (a chord step or the
    // case's end was expected next); a step that factors after all builds it first
    __shared__ int s_nojac[MAX_SLOTS];
    __shared__ long long s_lcur[MAX_SLOTS], s_lend[MAX_SLOTS];
    __shared__ double s_nrm[MAX_SLOTS], s_alpha[MAX_SLOTS], s_balpha[MAX_SLOTS], s_bnrm[MAX_SLOTS];
    __shared__ unsigned long long s_res[MAX_SLOTS], s_pmin[MAX_SLOTS], s_pmax[MAX_SLOTS];
    __shared__ int s_nst[MAX_SLOTS];
    __shared__ int s_tb[MAX_SLOTS];
    __shared__ int s_fb[MAX_SLOTS], s_chord[MAX_SLOTS];  // float factor buffer; next step is a chord step
    // s_first: the case started from the shared start and its first step uses the shared
    // factors; s_nofac: this step solves with factors it does not compute (chord or first)
    __shared__ int s_first[MAX_SLOTS], s_nofac[MAX_SLOTS];
    __shared__ int s_share;  // the launch's shared start is usable (its factorization passed)
    __shared__ int s_stk[MAX_SLOTS][MAX_STAMPS];
    __shared__ double2 s_stv[MAX_SLOTS][MAX_STAMPS];
    __shared__ unsigned long long s_ph[6];  // timed launches: SM cycles per phase of this CTA and job
    __shared__ long long s_clk;

    if (tid == 0) s_share = Bt.fac0 != nullptr && __ldg(Bt.ok0) == 1;  // written by the start kernel before this launch
    if (TIMED && tid == 0) {
        for (int k = 0; k < 6; ++k) s_ph[k] = 0ULL;
        s_clk = clock64();
    }
    // timed launches (a separate instantiation, so untimed ones carry no trace of the counters)
#define GBPF_PH (TIMED ? s_ph : nullptr)
    if (tid < G) {
        s_st[tid] = SL_EMPTY;
        s_lcur[tid] = s_lend[tid] = 0;
        s_warm[tid] = 0;
        s_nst[tid] = 0;
        s_jprec[tid] = 0;
        s_vote[tid] = 0;
        s_nojac[tid] = 0;
    }
    __syncthreads();

    // nr_klu.cpp:590-595 loop head of slot s on its mismatch s_nrm[s]. Under the GB300 vote
    // rule a case keeps stepping until its voltage is as exact as a double solve's: a float step
    // lands anywhere below tol (it contracts the error by ~cond(J) 2^-24 instead of squaring
    // it), so the case goes on until its mismatch is below tol_polish (the smaller of polish x
    // tol and a bound on the voltage error divided by the grid's |J^-1| estimate). `converged`
    // still means mismatch < tol.
    auto loop_head = [&](int s) {
        const bool polish = Bt.mixed && Bt.vote_rule == 1;
        const bool done = s_nrm[s] < (polish ? Bt.tol_polish : Bt.tol);
        if (s_it[s] >= Bt.max_iter) {
            s_st[s] = SL_FINISH;
            s_conv[s] = polish && s_nrm[s] < Bt.tol;
        } else if (done) {
            s_st[s] = SL_FINISH;
            s_conv[s] = 1;
        } else if (s_nrm[s] >= BIG) {
            s_st[s] = SL_FINISH;
            s_conv[s] = 0;
        } else {
            s_st[s] = SL_ACTIVE;
        }
    };

    for (;;) {
        // ---------------------------------------------------------------- refill
        if (tid < G) {
            const int s = tid;
            if (s_st[s] == SL_EMPTY) {
                long long c = -1;
                if (Bt.lanes) {
                    if (s_lcur[s] < s_lend[s]) {
                        c = s_lcur[s]++;
                    } else {
                        for (;;) {  // bounded: every pass consumes one lane
                            const int l = atomicAdd(Bt.counter, 1);
                            if (l >= Bt.K) break;
                            s_lcur[s] = Bt.lane_off[l];
                            s_lend[s] = Bt.lane_off[l + 1];
                            s_warm[s] = 0;
                            if (s_lcur[s] < s_lend[s]) {
                                c = s_lcur[s]++;
                                break;
                            }
                        }
                    }
                } else {
                    const int ci = atomicAdd(Bt.counter, 1);
                    if (ci < Bt.B) c = ci;
                }
                if (c < 0) {
                    s_st[s] = SL_RETIRED;
                } else {
                    s_case[s] = (int)c;
                    s_st[s] = SL_FRESH;
                    if (!s_warm[s]) s_tb[s] = 0;
                    s_fb[s] = 0;
                    s_chord[s] = 0;
                    s_first[s] = s_share && !s_warm[s];
                    s_nojac[s] = 0;
                    s_res[s] = 0ULL;
                    s_it[s] = 0;
                    s_conv[s] = 0;
                    s_vote[s] = Bt.mixed ? 1 : 0;
                    int nst = 0;
                    if (Bt.ymode == 3) {  // the stamps of the case's outaged branches
                        const int e0 = ld_in<RING>(Bt.out_ptr + c), e1 = ld_in<RING>(Bt.out_ptr + c + 1);
                        int nb = e1 - e0;
                        if (nb < 0 || 4 * nb > MAX_STAMPS) {
                            if (atomicCAS(&Bt.err[0], 0, DE_STAMPS) == 0) {
                                Bt.err[1] = 4 * nb;
                                Bt.err[2] = (int)c;
                            }
                            nb = nb < 0 ? 0 : MAX_STAMPS / 4;
                        }
                        for (int q = 0; q < nb; ++q) {
                            const int b = ld_in<RING>(Bt.out_idx + e0 + q);
                            if (b < 0 || b >= P.m) {  // never indexes the branch table out of range
                                if (atomicCAS(&Bt.err[0], 0, DE_OUTAGE) == 0) {
                                    Bt.err[1] = b;
                                    Bt.err[2] = (int)c;
                                }
                                continue;
                            }
                            const int4 pos = P.br_pos[b];
                            s_stk[s][nst] = pos.x;
                            s_stv[s][nst++] = P.br_val[4 * b];
                            s_stk[s][nst] = pos.y;
                            s_stv[s][nst++] = P.br_val[4 * b + 1];
                            s_stk[s][nst] = pos.z;
                            s_stv[s][nst++] = P.br_val[4 * b + 2];
                            s_stk[s][nst] = pos.w;
                            s_stv[s][nst++] = P.br_val[4 * b + 3];
                        }
                    } else if (Bt.ymode == 1) {
                        const int e0 = Bt.st_ptr[c], e1 = Bt.st_ptr[c + 1];
                        nst = e1 - e0;
                        if (nst > MAX_STAMPS) {
                            if (atomicCAS(&Bt.err[0], 0, DE_STAMPS) == 0) {
                                Bt.err[1] = nst;
                                Bt.err[2] = (int)c;
                            }
                            nst = MAX_STAMPS;
                        }
                        for (int e = 0; e < nst; ++e) {
                            s_stk[s][e] = Bt.st_k[e0 + e];
                            s_stv[s][e] = Bt.st_v[e0 + e];
                        }
                    }
                    s_nst[s] = nst;
                }
            }
            if (s_st[s] == SL_ACTIVE) s_it[s] += 1;
        }
        if (tid == 0) s_solo = -1;
        const int alive = __syncthreads_count(tid < G && s_st[tid] != SL_RETIRED);
        if (!alive) {
            if (TIMED && tid == 0)
                for (int k = 0; k < 6; ++k) atomicAdd(&Bt.stats[8 + k], s_ph[k]);
            break;
        }
        // one case left in the CTA (its tail): every thread works on that slot this pass
        if (alive == 1 && G > 1 && tid < G && s_st[tid] != SL_RETIRED) s_solo = tid;
        __syncthreads();
        // (read from shared memory where used: no register held across the pass)
        const int& solo = s_solo;
        auto nloop = [&]() { return s_solo >= 0 ? n : nG; };  // loop items of the per-bus phases

        // ---------------------------------------------------------------- load
        // The start goes to buffer 0 (a fresh case's committed point); buffer 1 gets it only at
        // slack buses, which no step rewrites -- every other bus's first trial is written to
        // buffer 1 before anything reads it.
        for (int k = tid; k < nloop(); k += NT) {
            const int idx = solo >= 0 ? (k << lg) + solo : k;
            const int s = idx & (G - 1);
            if (s_st[s] != SL_FRESH) continue;
            const int bus = idx >> lg;
            const bool fixed = P.row_of_bus[bus] < 0;
            const int c = s_case[s];
            if (s_warm[s]) {
                // previous hour of the lane converged here: its evaluated state is the start point
            } else if (Bt.v0_shared) {
                // shared start: the state table built once per launch (v0_table_kernel)
                const double4_32a t0 = RING ? ldcg4(Bt.v0tab + 2 * bus) : Bt.v0tab[2 * bus];
                Vb0[idx] = t0;
                if (fixed) Vb1[idx] = t0;
                // a case starting from the shared start evaluates its start with the shared
                // injections (no (e, f) or 1 / Vm read) and its first step rewrites them at every
                // moving bus before they are read: only the fixed buses' (e, f) are needed
                if (fixed || !s_first[s]) {
                    const double4_32a t1 = RING ? ldcg4(Bt.v0tab + 2 * bus + 1) : Bt.v0tab[2 * bus + 1];
                    Et[idx] = make_double2(t1.x, t1.y);
                    Ei[idx] = t1.z;
                    iv32[idx] = d2f_fast(t1.z);
                }
            } else {
                const double2 v0 = Bt.V0[(size_t)bus * Bt.sV0 + c];
                if (Bt.check_v0 && (!finite_d(v0.x) || !finite_d(v0.y))) {
                    if (atomicCAS(&Bt.err[0], 0, DE_V0_NONFINITE) == 0) {
                        Bt.err[1] = bus;
                        Bt.err[2] = c;
                    }
                }
                const double vm = hypot(v0.x, v0.y);
                const double va = atan2(v0.y, v0.x);
                if (Bt.check_v0 && (vm <= 0.0 || vm > 10.0) && finite_d(vm)) {
                    if (atomicCAS(&Bt.err[0], 0, DE_V0_MAGNITUDE) == 0) {
                        Bt.err[1] = bus;
                        Bt.err[2] = c;
                    }
                }
                double sn, cs;
                sincos(va, &sn, &cs);
                const double4_32a v = make_double4_32a(vm, va, cs, sn);
                Vb0[idx] = v;
                if (fixed) Vb1[idx] = v;
                const double e = vm * cs, f = vm * sn, iv = 1.0 / vm;
                Et[idx] = make_double2(e, f);
                Ei[idx] = iv;
                iv32[idx] = d2f_fast(iv);
            }
            uint8_t pinned = Bt.pin ? Bt.pin[(size_t)bus * Bt.spin + c] : (uint8_t)0;
            if (Bt.ref_bus) {
                // islands of an outage case (solver_cpp.py:121-134): an unserved bus is pinned at
                // 1 + 0j; an island re-slacked to bus r starts rotated so that r has angle 0 (r
                // itself at |v0| + 0j, pinned); islands holding a slack keep the start as it is
                const int r = ld_in<RING>(Bt.ref_bus + (size_t)bus * Bt.sref + c);
                if (r < 0 || !P.is_slack[r]) {
                    double4_32a v;
                    double iv;
                    if (r < 0) {
                        v = make_double4_32a(1.0, 0.0, 1.0, 0.0);
                        iv = 1.0;
                        pinned = 1;
                    } else {
                        const double4_32a t0 = Vb0[idx];
                        iv = Ei[idx];
                        if (r == bus) {
                            v = make_double4_32a(t0.x, 0.0, 1.0, 0.0);
                            pinned = 1;
                        } else {
                            const double4_32a tr = RING ? ldcg4(Bt.v0tab + 2 * r) : Bt.v0tab[2 * r];
                            v = make_double4_32a(t0.x, t0.y - tr.y, fma(t0.z, tr.z, t0.w * tr.w),
                                                 fma(t0.w, tr.z, -t0.z * tr.w));
                        }
                    }
                    Vb0[idx] = v;
                    if (fixed) Vb1[idx] = v;
                    const double e = v.x * v.z, f = v.x * v.w;
                    Et[idx] = make_double2(e, f);
                    Ei[idx] = iv;
                    iv32[idx] = d2f_fast(iv);
                }
            }
            spin[idx] = pinned;
            if (s_first[s]) {
                // a case from the shared start: its first mismatch S - S(V0) here, with S(V0)
                // computed once (the operation eval_row does, Ssp - Pc = Ssp + (-Pc)) -- so
                // it decides and takes its first step in this pass
                const int row = P.row_of_bus[bus];
                if (row >= 0) {
                    const double2 Ssp = ld_in<RING>(Bt.s_shared ? Bt.S + bus : Bt.S + (size_t)bus * Bt.sS + c);
                    const double2 r0 = __ldg(&Bt.R0[row]);
                    const double rp = Ssp.x + r0.x;
                    const double rq = P.bus_pq[bus] != 0 ? Ssp.y + r0.y : 0.0;
                    R[((size_t)row << lg) + s] = make_double2(rp, rq);
                    const unsigned long long a = abs_bits(rp), b = abs_bits(rq);
                    atomicMax(&s_res[s], b > a ? b : a);
                }
            }
        }
        __syncthreads();
        if (tid < G && s_st[tid] == SL_FRESH && s_first[tid]) {  // their loop head, now
            const int s = tid;
            double nw = bitsd(s_res[s]);
            if (!(nw < BIG)) nw = BIG;
            s_nrm[s] = nw;
            s_vote[s] = !Bt.mixed ? 0 : (Bt.vote_rule == 1 ? 1 : (nw > Bt.mixed_switch ? 1 : 0));
            // (what the start's own pass would have set: the precision of the start's Jacobian --
            // the shared one, float on the mixed path -- and the step count)
            s_jprec[s] = (Bt.mixed && s_vote[s] == 1) ? 1 : 0;
            loop_head(s);
            if (s_st[s] == SL_ACTIVE) s_it[s] = 1;
        }

        // ---------------------------------------------------------------- linear solve
        if (tid < G) {
            const int s = tid;
            const bool act = s_st[s] == SL_ACTIVE;
            const bool f32 = act && Bt.mixed && s_vote[s] == 1 && s_jprec[s] == 1;
            s_on32[s] = f32;
            s_on64[s] = act && !f32;
            s_reeval[s] = act && !f32 && s_jprec[s] == 1 && !s_first[s];
            s_nofac[s] = act && (s_chord[s] || s_first[s]);
            s_pmin[s] = ~0ULL;
            s_pmax[s] = 0ULL;
        }
        const int any32 = __syncthreads_or(tid < G && s_on32[tid]);
        if constexpr (TIMED) phase_mark(GBPF_PH, &s_clk, 0);
        // a float step that factors after an evaluation that left the Jacobian out: the
        // Jacobian at the same point first (the values that evaluation would have written)
        const int anylazy = __syncthreads_or(tid < G && s_on32[tid] && !s_nofac[tid] && s_nojac[tid]);
        if (anylazy) {
            for (int idx = tid; idx < nG; idx += NT) {
                const int s = idx & (G - 1);
                if (!(s_on32[s] && !s_nofac[s] && s_nojac[s])) continue;
                const int bus = idx >> lg;
                const int row = P.row_of_bus[bus];
                if (row < 0) continue;
                EvalCtx ec{&P, Et, Ei, iv32, lg, Bt.ymode == 3 ? 1 : Bt.ymode, Bt.Yd, Bt.sYd, s_case[s], s_nst[s], s_stk[s], s_stv[s]};
                eval_row<2>(ec, bus, s, row, spin[idx] != 0, P.bus_pq[bus] != 0, make_double2(0.0, 0.0),
                            s_fb[s] ? fac32 : fac32b, R, false);
            }
            __syncthreads();
            if (tid < G && s_on32[tid] && !s_nofac[tid] && s_nojac[tid]) atomicAdd(&Bt.stats[7], 1ULL);
        }
        if (any32) {
            // chord and first steps are decided per slot (a result never depends on the other
            // cases of its CTA); the factorization is left out altogether when no float slot
            // of the CTA factors
            const int all_chord = __syncthreads_and(!(tid < G && s_on32[tid]) || s_nofac[tid]);
            {
                // a slot factors the Jacobian in the buffer its last factors are not in; a chord
                // step solves with those factors, a first step with the shared start's
                const int sl = solo >= 0 ? solo : (tid & 31) & (G - 1);
                const int buf = s_chord[sl] ? s_fb[sl] : 1 - s_fb[sl];
                float4* const fl = s_first[sl] ? (float4*)Bt.fac0 : (buf ? fac32b : fac32);
                lu_pass<float, TIMED>(solo >= 0 ? s_plan1 : P, fl, R, y32, s_on32, lg, s_pmin, s_pmax, s_nofac, !all_chord,
                               nullptr, solo, GBPF_PH, &s_clk);
            }
            if (tid < G && s_on32[tid]) {
                const int s = tid;
                if (s_nofac[s]) {
                    atomicAdd(&Bt.stats[s_first[s] ? 6 : 5], 1ULL);
                } else {
                    atomicAdd(&Bt.stats[0], 1ULL);
                    if (!pivots_ok(s_pmin[s], s_pmax[s], Bt.rcond_min32)) {
                        atomicAdd(&Bt.stats[2], 1ULL);
                        s_vote[s] = -1;
                        s_on32[s] = 0;
                        s_on64[s] = 1;
                        s_reeval[s] = 1;
                    } else {
                        s_fb[s] ^= 1;  // the factors now live in the buffer the Jacobian was in
                    }
                }
                s_pmin[s] = ~0ULL;
                s_pmax[s] = 0ULL;
            }
        }
        const int anyre = __syncthreads_or(tid < G && s_reeval[tid]);
        if (anyre) {  // this step's factorization is double but the Jacobian was built in float
            for (int idx = tid; idx < nG; idx += NT) {
                const int s = idx & (G - 1);
                if (s_reeval[s]) Ei[idx] = recip_nr((s_tb[s] ? Vb1 : Vb0)[idx].x);
            }
            __syncthreads();
            for (int idx = tid; idx < nG; idx += NT) {
                const int s = idx & (G - 1);
                if (!s_reeval[s]) continue;
                const int bus = idx >> lg;
                const int row = P.row_of_bus[bus];
                if (row < 0) continue;
                EvalCtx ec{&P, Et, Ei, iv32, lg, Bt.ymode == 3 ? 1 : Bt.ymode, Bt.Yd, Bt.sYd, s_case[s], s_nst[s], s_stk[s], s_stv[s]};
                eval_row<1>(ec, bus, s, row, spin[idx] != 0, P.bus_pq[bus] != 0, make_double2(0.0, 0.0), fac64, R,
                            false);
            }
            __syncthreads();
            if (tid < G && s_reeval[tid]) s_jprec[tid] = 0;
        }
        const int any64 = __syncthreads_or(tid < G && s_on64[tid]);
        if (any64) {
            if (s_share) {
                // no double slot of the CTA factors (all take their first step): substitutions only
                const int all_first = __syncthreads_and(!(tid < G && s_on64[tid]) || s_nofac[tid]);
                const int sl = solo >= 0 ? solo : (tid & 31) & (G - 1);
                double4_32a* const fd = s_first[sl] ? (double4_32a*)Bt.fac0 : fac64;
                lu_pass<double, TIMED>(solo >= 0 ? s_plan1 : P, fd, R, y64, s_on64, lg, s_pmin, s_pmax, s_nofac, !all_first,
                                s_dinv64, solo, GBPF_PH, &s_clk);
            } else {
                lu_pass<double, TIMED>(solo >= 0 ? s_plan1 : P, fac64, R, y64, s_on64, lg, s_pmin, s_pmax, nullptr, true,
                                s_dinv64, solo, GBPF_PH, &s_clk);
            }
            if (tid < G && s_on64[tid]) {
                const int s = tid;
                if (s_nofac[s]) {
                    atomicAdd(&Bt.stats[s_first[s] ? 6 : 5], 1ULL);
                } else {
                    atomicAdd(&Bt.stats[1], 1ULL);
                    if (!pivots_ok(s_pmin[s], s_pmax[s], Bt.rcond_min64)) {
                        atomicAdd(&Bt.stats[3], 1ULL);
                        s_st[s] = SL_FINISH;  // no pivoting fallback on the device: not converged
                        s_conv[s] = 0;
                    }
                }
            }
        }
        if (tid < G && (s_on32[tid] || s_on64[tid])) {
            s_yprec[tid] = s_on64[tid] ? 0 : 1;
            s_first[tid] = 0;
        }
        __syncthreads();

        // ---------------------------------------------------------------- step
        // A thread's elements idx = tid + k NT all belong to slot tid & (G - 1) (NT is a
        // multiple of G) -- or all to the solo slot -- so the slot's state is read once and the
        // next element's committed point and step are loaded while the current one is worked on.
        {
            const int s = solo >= 0 ? solo : tid & (G - 1);
            const int st = s_st[s];
            if (st == SL_ACTIVE || st == SL_BACKTRACK || st == SL_NEEDJ) {
                const bool active = st == SL_ACTIVE;
                // committed point: the one evaluated last when it was accepted (ACTIVE), else
                // the other buffer; the new trial goes to the buffer that is not committed
                const int cb = active ? s_tb[s] : 1 - s_tb[s];
                const double4_32a* const Vc = cb ? Vb1 : Vb0;
                double4_32a* const Vt = cb ? Vb0 : Vb1;
                const bool ystep32 = s_yprec[s] != 0;
                const double alpha = s_alpha[s];
                const bool next_double = !Bt.mixed || s_vote[s] != 1;  // the next Jacobian is double
                auto fetch = [&](int at, int& row, double4_32a& vc, double& dth, double& dvm) {
                    row = P.row_of_bus[at >> lg];
                    vc = Vc[at];
                    if (row < 0) return;
                    if (ystep32) {
                        const float2 dd = y32[((size_t)row << lg) + s];
                        dth = f2d_fast(dd.x);
                        dvm = f2d_fast(dd.y);
                    } else {
                        const double2 dd = y64[((size_t)row << lg) + s];
                        dth = dd.x;
                        dvm = dd.y;
                    }
                };
                const int ksh = solo >= 0 ? lg : 0;  // element k -> idx = (k << ksh) + koff
                const int koff = solo >= 0 ? solo : 0;
                int rown = -1;
                double4_32a vcn = make_double4_32a(0.0, 0.0, 0.0, 0.0);
                double dthn = 0.0, dvmn = 0.0;
                if (tid < nloop()) fetch((tid << ksh) + koff, rown, vcn, dthn, dvmn);
                for (int k = tid; k < nloop(); k += NT) {
                    const int idx = (k << ksh) + koff;
                    const int row = rown;
                    const double4_32a vc = vcn;
                    const double dth = dthn, dvm = dvmn;
                    if (k + NT < nloop()) fetch(((k + NT) << ksh) + koff, rown, vcn, dthn, dvmn);
                    if (row < 0) continue;
                    const int bus = idx >> lg;
                    // trial point (nr_klu.cpp:665-669 form_trial): committed + alpha * step
                    const double d = active ? dth : alpha * dth;
                    const double va = vc.y + d;
                    const bool pq = __ldg(&P.bus_pq[bus]) != 0;
                    const double vm = !pq ? vc.x : (active ? vc.x + dvm : fma(alpha, dvm, vc.x));
                    double cs, sn;
                    const unsigned ahi = (unsigned)__double2hiint(d) & 0x7fffffffu;
                    if (ahi < 0x3FD00000u && ystep32 && pq) {  // a float step at a PQ bus
                        rotate_f32(vc.z, vc.w, d, &cs, &sn);
                    } else if (ahi < 0x3FD00000u) {  // |d| < 1/4: rotate the committed phasor by d
                        double sd, cd;
                        sincos_small(d, ahi, &sd, &cd);
                        cs = fma(vc.z, cd, -vc.w * sd);
                        sn = fma(vc.w, cd, vc.z * sd);
                    } else {
                        sincos(va, &sn, &cs);
                    }
                    Vt[idx] = make_double4_32a(vm, va, cs, sn);
                    const double e = vm * cs, f = vm * sn;
                    Et[idx] = make_double2(e, f);
                    if (pq) {  // PV buses keep the magnitude they were loaded with (and never read iv32)
                        if (next_double) {
                            const double iv = recip_nr(vm);
                            Ei[idx] = iv;
                            iv32[idx] = d2f_fast(iv);
                        } else {
                            iv32[idx] = __frcp_rn(d2f_fast(vm));
                        }
                    }
                }
            }
        }
        // The float Jacobian of this evaluation is left out where the next step should not
        // factor: after a chord step (another chord step or the case's end follows), or after a
        // float step from below JAC_LAZY x chord_tol (it lands below chord_tol). The lanes of a
        // warp are the case slots of one bus, so the choice is the CTA's: only when every
        // float full step of the CTA qualifies (mixed choices would run both paths per warp).
        int qual = 1;
        if (tid < G) {
            const int st = s_st[tid];
            if (st == SL_FRESH || st == SL_ACTIVE || st == SL_NEEDJ) s_jprec[tid] = (Bt.mixed && s_vote[tid] == 1) ? 1 : 0;
            if (st == SL_ACTIVE && s_jprec[tid])
                qual = Bt.lazy_jac && (s_chord[tid] || s_nrm[tid] < JAC_LAZY * Bt.chord_tol);
            s_res[tid] = 0ULL;
        }
        const int lazy = __syncthreads_and(qual);
        if (tid < G) {
            const int st = s_st[tid];
            if (st == SL_ACTIVE) {
                s_nojac[tid] = lazy && s_jprec[tid];
                if (s_nojac[tid]) atomicAdd(&Bt.stats[14], 1ULL);
            } else if (st == SL_FRESH || st == SL_NEEDJ) {
                s_nojac[tid] = 0;
            }
        }
        __syncthreads();
        if constexpr (TIMED) phase_mark(GBPF_PH, &s_clk, 3);

        // ---------------------------------------------------------------- evaluate
        // Buses are swept in reverse Cuthill-McKee order, so the buses a CTA evaluates at the
        // same time share their neighbours' state in cache.
        for (int k = tid; k < nloop(); k += NT) {
            const int s = solo >= 0 ? solo : k & (G - 1);
            const int st = s_st[s];
            if (st != SL_FRESH && st != SL_ACTIVE && st != SL_NEEDJ && st != SL_BACKTRACK) continue;
            const int bus = __ldg(&P.eval_order[solo >= 0 ? k : k >> lg]);
            const int row = P.row_of_bus[bus];
            if (row < 0) continue;
            const int c = s_case[s];
            const double2 Ssp = ld_in<RING>(Bt.s_shared ? Bt.S + bus : Bt.S + (size_t)bus * Bt.sS + c);
            const bool pq = P.bus_pq[bus] != 0;
            const bool pinned = spin[((size_t)bus << lg) + s] != 0;
            EvalCtx ec{&P, Et, Ei, iv32, lg, Bt.ymode == 3 ? 1 : Bt.ymode, Bt.Yd, Bt.sYd, c, s_nst[s], s_stk[s], s_stv[s]};
            unsigned long long worst;
            if (st == SL_BACKTRACK)
                worst = eval_row<0>(ec, bus, s, row, pinned, pq, Ssp, fac64, R, true);
            else if (Bt.mixed && s_jprec[s] && s_nojac[s])  // the mismatch only (lazy Jacobian)
                worst = eval_row<0>(ec, bus, s, row, pinned, pq, Ssp, fac64, R, true);
            else if (Bt.mixed && s_jprec[s])  // into the buffer the slot's last float factors are not in
                worst = eval_row<2>(ec, bus, s, row, pinned, pq, Ssp, s_fb[s] ? fac32 : fac32b, R, true);
            else
                worst = eval_row<1>(ec, bus, s, row, pinned, pq, Ssp, fac64, R, true);
            atomicMax(&s_res[s], worst);
        }
        __syncthreads();
        if constexpr (TIMED) phase_mark(GBPF_PH, &s_clk, 4);

        // ---------------------------------------------------------------- decide
        if (tid < G) {
            const int s = tid;
            const int st = s_st[s];
            if (st == SL_ACTIVE) s_tb[s] ^= 1;  // the trial just evaluated is in the other buffer
            double nw = bitsd(s_res[s]);
            if (!(nw < BIG)) nw = BIG;
            bool top = false;
            // Precision votes (mixed only). Reference rule (vote_rule 0, nr_polar_kernels.cu:209-228):
            // float while the mismatch is above mixed_switch, double below it, and double for
            // good once a float step fails to halve the mismatch or the line search engages.
            // GB300 rule (vote_rule 1): float throughout -- the double mismatch keeps the answer
            // exact and a float step near the solution still contracts by ~cond(J)*2^-24 --
            // and double for good only when contraction stalls near the solution (a float step
            // from below mixed_switch that does not halve the mismatch, or needs damping).
            if (st == SL_FRESH) {
                s_nrm[s] = nw;
                s_vote[s] = !Bt.mixed ? 0 : (Bt.vote_rule == 1 ? 1 : (nw > Bt.mixed_switch ? 1 : 0));
                top = true;
            } else if (st == SL_ACTIVE) {
                const double old = s_nrm[s];
                const bool was_chord = s_chord[s] != 0;
                s_chord[s] = 0;
                if (!Bt.line_search || nw <= (1.0 - ARMIJO_C) * old) {
                    if (Bt.mixed && s_vote[s] >= 0) {
                        if (Bt.vote_rule == 1) {
                            // (a chord step that contracts poorly only means: refactor next)
                            if (!was_chord && s_vote[s] == 1 && !(nw <= 0.5 * old) && old < Bt.mixed_switch)
                                s_vote[s] = -1;
                        } else if (s_vote[s] == 1 && !(nw <= 0.5 * old)) {
                            s_vote[s] = -1;
                        } else {
                            s_vote[s] = nw > Bt.mixed_switch ? 1 : 0;
                        }
                    }
                    s_nrm[s] = nw;
                    top = true;
                    // chord: near the solution the float factors of the last step are as good
                    // as fresh ones (a fresh float factorization is itself off by ~cond(J) 2^-24),
                    // so the next step reuses them while the mismatch is below chord_tol and each
                    // chord step cuts it at least CHORD_RATE-fold
                    if (Bt.chord_tol > 0.0 && s_vote[s] == 1 && s_yprec[s] == 1 && nw < Bt.chord_tol &&
                        (!was_chord || nw <= CHORD_RATE * old))
                        s_chord[s] = 1;
                } else {
                    s_balpha[s] = 1.0;
                    s_bnrm[s] = nw;
                    s_alpha[s] = 0.5;
                    s_trial[s] = 1;
                    s_st[s] = SL_BACKTRACK;
                    if (Bt.mixed && (Bt.vote_rule == 0 || old < Bt.mixed_switch)) s_vote[s] = -1;
                }
            } else if (st == SL_BACKTRACK) {
                const double a = s_alpha[s];
                if (nw < s_bnrm[s]) {
                    s_bnrm[s] = nw;
                    s_balpha[s] = a;
                }
                if (nw <= (1.0 - ARMIJO_C * a) * s_nrm[s]) {
                    s_st[s] = SL_NEEDJ;
                } else if (s_trial[s] >= LS_MAX_TRIALS) {
                    s_alpha[s] = s_balpha[s];
                    s_st[s] = SL_NEEDJ;
                } else {
                    s_trial[s] += 1;
                    s_alpha[s] = 0.5 * a;
                }
            } else if (st == SL_NEEDJ) {
                s_nrm[s] = nw;
                top = true;
            }
            if (top) loop_head(s);
        }
        if (tid == 0) atomicAdd(&Bt.stats[4], 1ULL);
        __syncthreads();

        // ---------------------------------------------------------------- write back
        for (int k = tid; k < nloop(); k += NT) {
            const int idx = solo >= 0 ? (k << lg) + solo : k;
            const int s = idx & (G - 1);
            if (s_st[s] != SL_FINISH) continue;
            const int bus = idx >> lg;
            const double4_32a v = (s_tb[s] ? Vb1 : Vb0)[idx];
            double2 o = make_double2(v.x * v.z, v.x * v.w);
            if (Bt.ref_bus && ld_in<RING>(Bt.ref_bus + (size_t)bus * Bt.sref + s_case[s]) < 0)
                o = make_double2(__longlong_as_double(0x7ff8000000000000LL), __longlong_as_double(0x7ff8000000000000LL));
            Bt.Vout[(size_t)bus * Bt.sV + s_case[s]] = o;
        }
        // a stream launch's results go to host memory: each writer makes its stores visible
        // to the host before the job's completion can be flagged
        if constexpr (RING) __threadfence_system();
        __syncthreads();
        if (tid < G && s_st[tid] == SL_FINISH) {
            const int s = tid;
            Bt.iters[s_case[s]] = s_it[s];
            Bt.conv[s_case[s]] = (uint8_t)s_conv[s];
            if (Bt.mis) Bt.mis[s_case[s]] = s_nrm[s];
            s_warm[s] = Bt.lanes && s_conv[s];
            s_st[s] = SL_EMPTY;
            if constexpr (RING) {
                __threadfence_system();
                atomicAdd(&s_fin, 1);
            }
        }
        __syncthreads();
        if (RING && tid == 0 && s_fin) {  // the job's last cases written back: flag it
            const int old = atomicAdd(&L.ring.done_cases[job], s_fin);
            if (old + s_fin == Bt.B) {
                __threadfence_system();
                st_release_sys(&L.ring.host_done[job], 1);
            }
            s_fin = 0;
        }
        if constexpr (TIMED) phase_mark(GBPF_PH, &s_clk, 5);
    }
#undef GBPF_PH
    }  // jobs
}

// Start-state table of a shared start voltage: per bus (Vm, Va, cos, sin) and (e, f, 1/Vm, 0),
// so that loading a case costs no trigonometry. Validates the voltages like nr_klu's
// solve_batch (nr_klu.cpp:1127-1139), reporting case 0.
__global__ void v0_table_kernel(const double2* V0, int n, int check, double4_32a* tab, int* err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double2 v0 = V0[i];
        if (check && (!finite_d(v0.x) || !finite_d(v0.y))) {
            if (atomicCAS(&err[0], 0, DE_V0_NONFINITE) == 0) {
                err[1] = i;
                err[2] = 0;
            }
        }
        const double vm = hypot(v0.x, v0.y), va = atan2(v0.y, v0.x);
        if (check && (vm <= 0.0 || vm > 10.0) && finite_d(vm)) {
            if (atomicCAS(&err[0], 0, DE_V0_MAGNITUDE) == 0) {
                err[1] = i;
                err[2] = 0;
            }
        }
        double sn, cs;
        sincos(va, &sn, &cs);
        tab[2 * i] = make_double4_32a(vm, va, cs, sn);
        tab[2 * i + 1] = make_double4_32a(vm * cs, vm * sn, 1.0 / vm, 0.0);
    }
}

// Conversion helpers applied elementwise (tests compare them with IEEE casts).
__global__ void conversions_kernel(const double* in, int n, float* d2f, double* f2d, float* d2f_small) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        d2f[i] = d2f_fast(in[i]);
        f2d[i] = f2d_fast(d2f[i]);
        d2f_small[i] = d2f_trunc(in[i]);
    }
}

// The project's own double-precision numerics applied elementwise (tests bound them against
// IEEE division and CUDA's sincos): recip_nr(x) for x > 0, and sincos_small(d) with CUDA's
// sincos(d) beside it for |d| < 1/4 (elements outside that range get sincos only).
__global__ void math_kernel(const double* in, int n, double* recip, double* s_small, double* c_small,
                            double* s_ref, double* c_ref, const double* phasor, double* rot) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double x = in[i];
        if (phasor) {  // the phasor (phasor[0], phasor[1]) rotated by x as the voltage update does, |x| < 1/4
            const unsigned ah = (unsigned)__double2hiint(x) & 0x7fffffffu;
            double rc = 0.0, rs = 0.0, fc = 0.0, fs = 0.0;
            if (ah < 0x3FD00000u) {
                double sd, cd;
                sincos_small(x, ah, &sd, &cd);
                rc = fma(phasor[0], cd, -phasor[1] * sd);
                rs = fma(phasor[1], cd, phasor[0] * sd);
                rotate_f32(phasor[0], phasor[1], x, &fc, &fs);  // a float step's rotation at a PQ bus
            }
            rot[4 * i] = rc;
            rot[4 * i + 1] = rs;
            rot[4 * i + 2] = fc;
            rot[4 * i + 3] = fs;
        }
        recip[i] = x > 0.0 ? recip_nr(x) : 0.0;
        double sr, cr;
        sincos(x, &sr, &cr);
        s_ref[i] = sr;
        c_ref[i] = cr;
        const unsigned ahi = (unsigned)__double2hiint(x) & 0x7fffffffu;
        if (ahi < 0x3FD00000u) {
            double sd, cd;
            sincos_small(x, ahi, &sd, &cd);
            s_small[i] = sd;
            c_small[i] = cd;
        } else {
            s_small[i] = sr;
            c_small[i] = cr;
        }
    }
}

cudaError_t launch_math(const double* in, int n, double* recip, double* s_small, double* c_small, double* s_ref,
                        double* c_ref, const double* phasor, double* rot) {
    math_kernel<<<(n + 255) / 256, 256>>>(in, n, recip, s_small, c_small, s_ref, c_ref, phasor, rot);
    return cudaGetLastError();
}

cudaError_t launch_conversions(const double* in, int n, float* d2f, double* f2d, float* d2f_small) {
    conversions_kernel<<<(n + 255) / 256, 256>>>(in, n, d2f, f2d, d2f_small);
    return cudaGetLastError();
}

cudaError_t launch_v0_table(const double2* V0, int n, int check, double4_32a* tab, int* err, cudaStream_t stream) {
    v0_table_kernel<<<(n + 255) / 256, 256, 0, stream>>>(V0, n, check, tab, err);
    return cudaGetLastError();
}

cudaError_t preload_v0_table() {
    cudaFuncAttributes a;
    return cudaFuncGetAttributes(&a, v0_table_kernel);
}

// DC start (NewtonPowerflowCpp.py:422-440 _pre_dc_solve, timeseries.py:200-247
// dc_initial_voltage): B[pvpq, pvpq] theta = Pinj[pvpq] - B[pvpq, ref] theta_ref, factored and
// solved by the Newton kernel's block LU (every 2x2 block carries B in its angle / P entry and
// the identity in its magnitude / Q entry). B is either the caller's DC susceptance matrix on
// the Ybus pattern (Bx: the imaginary parts of the summed DC branch stamps, diagonal included,
// as the reference's make_ybus builds its Bbus, NewtonPowerflowCpp.py:64-161) or, with Bx null,
// derived from the Ybus (-Im Y off the diagonal, the negated row sum on it). The plan's
// schedule has NTB workers and one slot.
template <bool BLOCKS>
__device__ void dc_assemble(const DevPlan& P, const double2* Bx, const double* Pinj, long long sP,
                            const double* theta_bus, double4_32a* fac, double2* R) {
    for (int i = threadIdx.x; i < P.n; i += blockDim.x) {
        const int row = P.row_of_bus[i];
        if (row < 0) continue;
        double rhs = Pinj[(size_t)i * sP], diag = 0.0;
        for (int k = P.Yp[i]; k < P.Yp[i + 1]; ++k) {
            const int j = P.Yj[k];
            if (j == i) {
                if (Bx) diag = Bx[k].y;
                continue;
            }
            const double b = Bx ? Bx[k].y : -P.Y[k].y;
            if (!Bx) diag -= b;
            const int q = P.posmap[k];
            if (q >= 0) {
                if (BLOCKS) fac[q] = make_double4_32a(b, 0.0, 0.0, 0.0);
            } else if (P.row_of_bus[j] < 0) {
                rhs -= b * theta_bus[j];  // coupling to a reference bus at its angle
            }
        }
        if (BLOCKS) fac[P.dpos[row]] = make_double4_32a(diag, 0.0, 0.0, 1.0);
        R[row] = make_double2(rhs, 0.0);
    }
}

// Case 0: factors B (one CTA) and solves its right-hand side; theta column 0.
template <int NTB>
__global__ void __launch_bounds__(NTB, 1) dc_kernel(const DevPlan P, const double2* Bx, const double* Pinj, long long sP,
                                                    const double* theta_bus, double4_32a* fac, double2* R, double2* y,
                                                    double* theta, long long sT, unsigned long long* piv) {
    __shared__ int s_on[1];
    __shared__ unsigned long long s_min[1], s_max[1];
    const int tid = threadIdx.x;
    if (tid == 0) {
        s_on[0] = 1;
        s_min[0] = ~0ULL;
        s_max[0] = 0ULL;
    }
    dc_assemble<true>(P, Bx, Pinj, sP, theta_bus, fac, R);
    __syncthreads();
    lu_pass<double>(P, fac, R, y, s_on, 0, s_min, s_max, nullptr, true, nullptr);
    for (int i = tid; i < P.n; i += NTB) {
        const int row = P.row_of_bus[i];
        theta[(size_t)i * sT] = row < 0 ? theta_bus[i] : y[row].x;
    }
    if (tid == 0) {
        piv[0] = s_min[0];
        piv[1] = s_max[0];
    }
}

// Cases 1 .. T-1: the factors of case 0 reused (B is the same for every case), substitutions
// only; each CTA takes cases blockIdx.x + 1, + gridDim.x, ... with its own R / y rows.
template <int NTB>
__global__ void __launch_bounds__(NTB, 1) dc_solve_kernel(const DevPlan P, const double2* Bx, const double* Pinj,
                                                          long long sP, int T, const double* theta_bus,
                                                          double4_32a* fac, double2* Rs, double2* ys, double* theta,
                                                          long long sT) {
    __shared__ int s_on[1], s_chord[1];
    __shared__ unsigned long long s_min[1], s_max[1];
    const int tid = threadIdx.x;
    const int nv = P.nv > 0 ? P.nv : 1;
    double2* R = Rs + (size_t)blockIdx.x * nv;
    double2* y = ys + (size_t)blockIdx.x * nv;
    if (tid == 0) {
        s_on[0] = 1;
        s_chord[0] = 1;
    }
    for (int c = blockIdx.x + 1; c < T; c += gridDim.x) {
        if (tid == 0) {
            s_min[0] = ~0ULL;
            s_max[0] = 0ULL;
        }
        dc_assemble<false>(P, Bx, Pinj + c, sP, theta_bus, fac, R);
        __syncthreads();
        lu_pass<double>(P, fac, R, y, s_on, 0, s_min, s_max, s_chord, false, nullptr);
        for (int i = tid; i < P.n; i += NTB) {
            const int row = P.row_of_bus[i];
            theta[(size_t)i * sT + c] = row < 0 ? theta_bus[i] : y[row].x;
        }
        __syncthreads();
    }
}

// Shared start of a launch (every case from the same V0 on the same Ybus, no pins): the
// injections S(V0) and the factors of J(V0) -- the same operations, in the same order, as
// every case's own first evaluation and factorization would do -- computed once, the factors
// then copied to every case slot of the Newton launch. One CTA per start; the start's plan
// carries the 1,024-thread, one-slot schedule.
template <int NTB>
__global__ void __launch_bounds__(NTB, 1) start_kernel(const StartJob* jobs) {
    __shared__ StartJob sj;
    __shared__ int s_on[1];
    __shared__ unsigned long long s_min[1], s_max[1];
    const int tid = threadIdx.x;
    {
        const int* src = reinterpret_cast<const int*>(&jobs[blockIdx.x]);
        int* dst = reinterpret_cast<int*>(&sj);
        for (int w = tid; w < (int)(sizeof(StartJob) / 4); w += NTB) dst[w] = src[w];
    }
    if (tid == 0) {
        s_on[0] = 1;
        s_min[0] = ~0ULL;
        s_max[0] = 0ULL;
    }
    __syncthreads();
    const DevPlan& P = sj.P;
    for (int i = tid; i < P.n; i += NTB) {  // as the Newton kernel loads a case from the table
        const double4_32a t1 = sj.v0tab[2 * i + 1];
        reinterpret_cast<double2*>(sj.Et0)[i] = make_double2(t1.x, t1.y);
        sj.Ei0[i] = t1.z;
        sj.iv0[i] = d2f_fast(t1.z);
    }
    __syncthreads();
    for (int i = tid; i < P.n; i += NTB) {
        const int row = P.row_of_bus[i];
        if (row < 0) continue;
        EvalCtx ec{&P, sj.Et0, sj.Ei0, sj.iv0, 0, 0, nullptr, 0, 0, 0, nullptr, nullptr};
        if (sj.mixed)
            eval_row<2>(ec, i, 0, row, false, P.bus_pq[i] != 0, make_double2(0.0, 0.0),
                        reinterpret_cast<float4*>(sj.fac1), sj.R0, true);
        else
            eval_row<1>(ec, i, 0, row, false, P.bus_pq[i] != 0, make_double2(0.0, 0.0),
                        reinterpret_cast<double4_32a*>(sj.fac1), sj.R0, true);
    }
    __syncthreads();
    if (sj.mixed)
        lu_pass<float>(P, reinterpret_cast<float4*>(sj.fac1), sj.R0, reinterpret_cast<float2*>(sj.y0), s_on, 0, s_min,
                       s_max, nullptr, true, nullptr);
    else
        lu_pass<double>(P, reinterpret_cast<double4_32a*>(sj.fac1), sj.R0, sj.y0, s_on, 0, s_min, s_max, nullptr, true,
                        nullptr);
    if (tid == 0) *sj.ok0 = pivots_ok(s_min[0], s_max[0], sj.rcond_min) ? 1 : 0;
}

// The start's factors copied to every case slot ([blk] -> [blk][slot]) by the whole device:
// blockIdx.y is the start, x and threads stride over its 16-byte words.
__global__ void replicate_kernel(const StartJob* jobs) {
    const StartJob& sj = jobs[blockIdx.y];
    const long long nb = (long long)sj.P.nblk + sj.P.nv;
    const int wpb = sj.mixed ? 1 : 2;  // 16-byte words per block
    const long long words = nb * wpb << sj.log2G;
    const float4* a = reinterpret_cast<const float4*>(sj.fac1);
    float4* b = reinterpret_cast<float4*>(sj.facG);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < words; q += (long long)gridDim.x * blockDim.x) {
        const long long blk = (q / wpb) >> sj.log2G, part = q % wpb;
        b[q] = a[blk * wpb + part];
    }
}

cudaError_t launch_start(const StartJob* jobs, int njobs, cudaStream_t stream) {
    if (njobs <= 0) return cudaSuccess;
    start_kernel<1024><<<njobs, 1024, 0, stream>>>(jobs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    replicate_kernel<<<dim3(256, njobs), 256, 0, stream>>>(jobs);
    return cudaGetLastError();
}

size_t start_bytes(int n, int nv, int nblk, int G, bool mixed) {
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t blk = mixed ? 16 : 32, nf = (size_t)nblk + nv, rows = (size_t)(nv > 0 ? nv : 1);
    return up(rows * 16) + up(nf * blk) + up(nf * blk * G) + up(rows * 16) + up((size_t)n * 16) + up((size_t)n * 8) +
           up((size_t)n * 4) + up(4);
}

void start_carve(StartJob& sj, char* base, int n, int nv, int nblk, int G, bool mixed) {
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t blk = mixed ? 16 : 32, nf = (size_t)nblk + nv, rows = (size_t)(nv > 0 ? nv : 1);
    size_t at = 0;
    auto take = [&](size_t b) {
        char* p = base + at;
        at += up(b);
        return p;
    };
    sj.R0 = reinterpret_cast<double2*>(take(rows * 16));
    sj.fac1 = take(nf * blk);
    sj.facG = take(nf * blk * G);
    sj.y0 = reinterpret_cast<double2*>(take(rows * 16));
    sj.Et0 = reinterpret_cast<double2*>(take((size_t)n * 16));
    sj.Ei0 = reinterpret_cast<double*>(take((size_t)n * 8));
    sj.iv0 = reinterpret_cast<float*>(take((size_t)n * 4));
    sj.ok0 = reinterpret_cast<int*>(take(4));
}

cudaError_t launch_dc(const DevPlan& P, const double2* Bx, const double* Pinj, int T, const double* theta_bus,
                      double4_32a* fac, double2* R, double2* y, double* theta, unsigned long long* piv, int grid,
                      cudaStream_t stream) {
    dc_kernel<1024><<<1, 1024, 0, stream>>>(P, Bx, Pinj, T, theta_bus, fac, R, y, theta, T, piv);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || T <= 1) return e;
    dc_solve_kernel<1024><<<grid, 1024, 0, stream>>>(P, Bx, Pinj, T, T, theta_bus, fac, R, y, theta, T);
    return cudaGetLastError();
}

// Jacobian blocks and residual at one given voltage (G = 1): debug_J and tests.
__global__ void eval_debug_kernel(const DevPlan P, const double2* V, const double2* Sbus, const uint8_t* pin,
                                  double4_32a* Vt, double2* Et, double* Ei, float* iv32, double4_32a* blocks,
                                  double2* R) {
    const int n = P.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double vm = hypot(V[i].x, V[i].y), va = atan2(V[i].y, V[i].x);
        double sn, cs;
        sincos(va, &sn, &cs);
        Vt[i] = make_double4_32a(vm, va, cs, sn);
        Et[i] = make_double2(vm * cs, vm * sn);
        Ei[i] = 1.0 / vm;
        iv32[i] = (float)(1.0 / vm);
    }
    __syncthreads();  // single-CTA launch
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int row = P.row_of_bus[i];
        if (row < 0) continue;
        EvalCtx ec{&P, Et, Ei, iv32, 0, 0, nullptr, 0, 0, 0, nullptr, nullptr};
        eval_row<1>(ec, i, 0, row, pin && pin[i], P.bus_pq[i] != 0, Sbus[i], blocks, R, true);
    }
}

cudaError_t launch_newton(const Launch& L, int grid, int threads, cudaStream_t stream) {
    if (L.ring.published) {  // a stream launch: untimed
        if (L.timed) return cudaErrorInvalidValue;
        if (threads == 1024)
            newton_kernel<1024, false, true><<<grid, 1024, 0, stream>>>(L);
        else if (threads == 512)
            newton_kernel<512, false, true><<<grid, 512, 0, stream>>>(L);
        else
            return cudaErrorInvalidValue;
    } else if (threads == 1024)
        L.timed ? newton_kernel<1024, true, false><<<grid, 1024, 0, stream>>>(L)
                : newton_kernel<1024, false, false><<<grid, 1024, 0, stream>>>(L);
    else if (threads == 512)
        L.timed ? newton_kernel<512, true, false><<<grid, 512, 0, stream>>>(L)
                : newton_kernel<512, false, false><<<grid, 512, 0, stream>>>(L);
    else if (threads == 256)
        L.timed ? newton_kernel<256, true, false><<<grid, 256, 0, stream>>>(L)
                : newton_kernel<256, false, false><<<grid, 256, 0, stream>>>(L);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_eval_debug(const DevPlan& P, const double2* V, const double2* Sbus, const uint8_t* pin,
                              double4_32a* Vt, double2* Et, double* Ei, float* iv32, double4_32a* blocks,
                              double2* R, cudaStream_t stream) {
    eval_debug_kernel<<<1, 256, 0, stream>>>(P, V, Sbus, pin, Vt, Et, Ei, iv32, blocks, R);
    return cudaGetLastError();
}

const void* newton_kernel_ptr(int threads) {
    if (threads == 1024) return (const void*)newton_kernel<1024, false, false>;
    if (threads == 512) return (const void*)newton_kernel<512, false, false>;
    return (const void*)newton_kernel<256, false, false>;
}

}  // namespace gbpf
