// islands.cu -- N-1 islanding and re-slacking on the device.
//
// Per contingency case: connected components of the live branch graph minus the case's
// outaged branches, numbered like scipy.sparse.csgraph.connected_components (ordered by
// each component's smallest bus), and the reference bus of every island: the lowest-index
// slack bus it contains, else (with reslack) its generator bus of highest priority (ties:
// lowest bus index), else none (unserved). Semantics of the reference's
// p3s/contingency/case_generator.py:355-430 (_components_after_outage, _resolve_references;
// the reference ranks generators by short-circuit impedance, this API by a caller-given
// priority, e.g. the scheduled active power).
//
// One CTA per case (persistent grid). Labels converge by min-label hooking with pointer
// jumping: every change lowers a label and no label drops below the smallest bus of its
// component, and the loop ends only when no edge joins two labels and every label is a
// root, so the fixed point labels every component with its smallest bus. The number of
// passes is bounded (checked and reported, never looped on).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "gbpf.h"
#include "gbpf_device.h"

namespace {

constexpr int NT = 256;
constexpr int NONE = 0x7fffffff;

__global__ void __launch_bounds__(NT) islands_kernel(int n, int m, const int* f, const int* t, const uint8_t* live,
                                                      int L, const int* out_ptr, const int* out_idx,
                                                      const uint8_t* is_slack, const double* prio, int reslack,
                                                      int* scratch, unsigned long long* best, int* labels,
                                                      uint8_t* served, int* ref_bus, int* n_islands, int* err) {
    int* lab = scratch + (size_t)blockIdx.x * 4 * n;
    int* id = lab + n;
    int* cslack = id + n;
    int* cgen = cslack + n;
    unsigned long long* cbest = best + (size_t)blockIdx.x * n;
    __shared__ int s_changed;
    __shared__ int s_unsettled;
    __shared__ int s_total;
    __shared__ int s_warp[NT / 32];
    const int tid = threadIdx.x;
    for (int c = blockIdx.x; c < L; c += gridDim.x) {
        const int o0 = out_ptr[c], o1 = out_ptr[c + 1];
        for (int v = tid; v < n; v += NT) lab[v] = v;
        if (tid == 0) s_unsettled = 0;
        __syncthreads();
        for (int pass = 0;; ++pass) {
            if (tid == 0) s_changed = 0;
            __syncthreads();
            for (int e = tid; e < m; e += NT) {
                if (!live[e]) continue;
                bool out = false;
                for (int q = o0; q < o1; ++q) out |= out_idx[q] == e;
                if (out) continue;
                const int a = lab[lab[f[e]]], b = lab[lab[t[e]]];
                if (a != b) {
                    const int lo = min(a, b), hi = max(a, b);
                    atomicMin(&lab[hi], lo);
                    atomicMin(&lab[f[e]], lo);
                    atomicMin(&lab[t[e]], lo);
                    s_changed = 1;
                }
            }
            __syncthreads();
            for (int v = tid; v < n; v += NT) {  // pointer jumping (bounded walk)
                const int l0 = lab[v];
                int l = l0;
                for (int k = 0; k < 64 && lab[l] != l; ++k) l = lab[l];
                if (l != l0) {
                    atomicMin(&lab[v], l);
                    s_changed = 1;
                }
            }
            __syncthreads();
            const int ch = s_changed;
            __syncthreads();
            if (!ch) break;
            if (pass > 2 * n + 64) {
                if (tid == 0) {
                    atomicCAS(err, 0, 1);
                    s_unsettled = 1;
                }
                __syncthreads();
                break;
            }
        }
        if (s_unsettled) {
            // labels that are not all roots would index the per-island words past this case's
            // islands: the case gets no islands (label -1, unserved, no reference bus) and the
            // error word, already set, is the call's only other effect
            for (int v = tid; v < n; v += NT) {
                labels[(size_t)v * L + c] = -1;
                served[(size_t)v * L + c] = 0;
                ref_bus[(size_t)v * L + c] = -1;
            }
            if (tid == 0) n_islands[c] = -1;
            __syncthreads();
            continue;
        }
        // component ids: exclusive prefix count of the roots (lab[v] == v), in bus order
        if (tid == 0) s_total = 0;
        __syncthreads();
        for (int base = 0; base < n; base += NT) {
            const int v = base + tid;
            const int r = (v < n && lab[v] == v) ? 1 : 0;
            const unsigned ball = __ballot_sync(0xffffffffu, r);
            const int lane = tid & 31, w = tid >> 5;
            if (lane == 0) s_warp[w] = __popc(ball);
            __syncthreads();
            int off = s_total;
            for (int k = 0; k < w; ++k) off += s_warp[k];
            if (r) id[v] = off + __popc(ball & ((1u << lane) - 1));
            __syncthreads();
            if (tid == 0) {
                int sum = 0;
                for (int k = 0; k < NT / 32; ++k) sum += s_warp[k];
                s_total += sum;
            }
            __syncthreads();
        }
        const int ncomp = s_total;
        for (int k = tid; k < ncomp; k += NT) {
            cslack[k] = NONE;
            cgen[k] = NONE;
            cbest[k] = 0ULL;
        }
        __syncthreads();
        // component id of every bus (roots hold theirs; read before any root is rewritten)
        for (int v = tid; v < n; v += NT) lab[v] = id[lab[v]];
        __syncthreads();
        for (int v = tid; v < n; v += NT) {
            const int k = lab[v];
            if (is_slack[v]) atomicMin(&cslack[k], v);
            if (reslack && prio[v] > 0.0) atomicMax(&cbest[k], (unsigned long long)__double_as_longlong(prio[v]));
        }
        __syncthreads();
        if (reslack)
            for (int v = tid; v < n; v += NT) {
                const int k = lab[v];
                if (prio[v] > 0.0 && (unsigned long long)__double_as_longlong(prio[v]) == cbest[k])
                    atomicMin(&cgen[k], v);
            }
        __syncthreads();
        for (int v = tid; v < n; v += NT) {
            const int k = lab[v];
            const int r = cslack[k] != NONE ? cslack[k] : (cgen[k] != NONE ? cgen[k] : -1);
            labels[(size_t)v * L + c] = k;
            served[(size_t)v * L + c] = r >= 0;
            ref_bus[(size_t)v * L + c] = r;
        }
        if (tid == 0) n_islands[c] = ncomp;
        __syncthreads();
    }
}

int ifail(const std::string& m) {
    gbpf::set_error(m);
    return -1;
}

}  // namespace

cudaError_t gbpf::launch_islands(int n, int m, const int* f, const int* t, const uint8_t* live, int L,
                                 const int* out_ptr, const int* out_idx, const uint8_t* is_slack, const double* prio,
                                 int reslack, int* scratch, unsigned long long* best, int* labels, uint8_t* served,
                                 int* ref_bus, int* n_islands, int* err, int grid, cudaStream_t stream) {
    islands_kernel<<<grid, NT, 0, stream>>>(n, m, f, t, live, L, out_ptr, out_idx, is_slack, prio, reslack, scratch,
                                            best, labels, served, ref_bus, n_islands, err);
    return cudaGetLastError();
}

cudaError_t gbpf::preload_islands() {
    cudaFuncAttributes a;
    return cudaFuncGetAttributes(&a, islands_kernel);
}

extern "C" int gbpf_islands(int n, int m, const int32_t* f, const int32_t* t, const uint8_t* live, int L,
                            const int32_t* out_ptr, const int32_t* out_idx, const uint8_t* is_slack,
                            const double* gen_prio, int reslack, int32_t* labels, uint8_t* served, int32_t* ref_bus,
                            int32_t* n_islands) {
    if (n <= 0 || m < 0 || L <= 0) return ifail("gbpf_islands: invalid sizes");
    for (int e = 0; e < m; ++e)
        if (f[e] < 0 || f[e] >= n || t[e] < 0 || t[e] >= n) return ifail("gbpf_islands: branch end out of range");
    if (out_ptr[0] != 0) return ifail("gbpf_islands: outage pointers must start at 0");
    for (int c = 0; c < L; ++c)
        if (out_ptr[c + 1] < out_ptr[c]) return ifail("gbpf_islands: outage pointers must not decrease");
    const int nout = out_ptr[L];
    for (int q = 0; q < nout; ++q)
        if (out_idx[q] < 0 || out_idx[q] >= m) return ifail("gbpf_islands: outage index out of range");
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int grid = std::max(1, std::min(L, 4 * nsm));
    void *df = nullptr, *dt = nullptr, *dl = nullptr, *dop = nullptr, *doi = nullptr, *ds = nullptr, *dp = nullptr,
         *dsc = nullptr, *dbest = nullptr, *dlab = nullptr, *dsv = nullptr, *dref = nullptr, *dni = nullptr,
         *derr = nullptr;
    auto al = [](void** p, size_t b) { return cudaMalloc(p, std::max<size_t>(b, 16)); };
    const size_t nl = (size_t)n * L;
    cudaError_t e = cudaSuccess;
    if (!e) e = al(&df, (size_t)m * 4);
    if (!e) e = al(&dt, (size_t)m * 4);
    if (!e) e = al(&dl, (size_t)m);
    if (!e) e = al(&dop, (size_t)(L + 1) * 4);
    if (!e) e = al(&doi, (size_t)std::max(nout, 1) * 4);
    if (!e) e = al(&ds, (size_t)n);
    if (!e) e = al(&dp, (size_t)n * 8);
    if (!e) e = al(&dsc, (size_t)grid * 4 * n * 4);
    if (!e) e = al(&dbest, (size_t)grid * n * 8);
    if (!e) e = al(&dlab, nl * 4);
    if (!e) e = al(&dsv, nl);
    if (!e) e = al(&dref, nl * 4);
    if (!e) e = al(&dni, (size_t)L * 4);
    if (!e) e = al(&derr, 16);
    if (!e && m) e = cudaMemcpy(df, f, (size_t)m * 4, cudaMemcpyHostToDevice);
    if (!e && m) e = cudaMemcpy(dt, t, (size_t)m * 4, cudaMemcpyHostToDevice);
    if (!e && m) e = cudaMemcpy(dl, live, (size_t)m, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(dop, out_ptr, (size_t)(L + 1) * 4, cudaMemcpyHostToDevice);
    if (!e && nout) e = cudaMemcpy(doi, out_idx, (size_t)nout * 4, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(ds, is_slack, (size_t)n, cudaMemcpyHostToDevice);
    if (!e && gen_prio) e = cudaMemcpy(dp, gen_prio, (size_t)n * 8, cudaMemcpyHostToDevice);
    if (!e && !gen_prio) e = cudaMemset(dp, 0, (size_t)n * 8);
    if (!e) e = cudaMemset(derr, 0, 16);
    if (!e) {
        islands_kernel<<<grid, NT>>>(n, m, (const int*)df, (const int*)dt, (const uint8_t*)dl, L, (const int*)dop,
                                     (const int*)doi, (const uint8_t*)ds, (const double*)dp, reslack, (int*)dsc,
                                     (unsigned long long*)dbest, (int*)dlab, (uint8_t*)dsv, (int*)dref, (int*)dni,
                                     (int*)derr);
        e = cudaGetLastError();
    }
    if (!e) e = cudaDeviceSynchronize();
    int kerr = 0;
    if (!e) e = cudaMemcpy(&kerr, derr, 4, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(labels, dlab, nl * 4, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(served, dsv, nl, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(ref_bus, dref, nl * 4, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(n_islands, dni, (size_t)L * 4, cudaMemcpyDeviceToHost);
    for (void* p : {df, dt, dl, dop, doi, ds, dp, dsc, dbest, dlab, dsv, dref, dni, derr})
        if (p) cudaFree(p);
    if (e) return ifail(std::string("gbpf_islands: ") + cudaGetErrorString(e));
    if (kerr) return ifail("gbpf_islands: label propagation did not settle");
    return 0;
}

// ---------------------------------------------------------------------------------------
// gbpf_islands_device_static: the islanding kernel on caller-owned device buffers with its
// scratch in statically allocated device memory, so a call allocates nothing (no
// cudaMalloc / cudaFree, no library routine that allocates). The scratch below is shared
// by every call on a device and keeps its last contents: the kernel initialises the label
// and per-island words it reads, and the error word is cleared before each launch. Calls
// that overlap in time on one device (other streams, other host threads) race on it.
namespace {

constexpr int STATIC_INTS = 1 << 21;  // 8 MiB: 4 n ints per CTA
constexpr int STATIC_BEST = 1 << 20;  // 8 MiB: n u64 per CTA
constexpr int STATIC_MAX_DEVICES = 64;
static_assert(GBPF_ISLANDS_STATIC_MAX_BUS <= STATIC_BEST, "one CTA must fit the static scratch");

static __device__ __align__(256) int g_static_ints[STATIC_INTS];
static __device__ __align__(256) unsigned long long g_static_best[STATIC_BEST];
static __device__ __align__(256) int g_static_err[64];

struct StaticScratch {
    int* ints = nullptr;
    unsigned long long* best = nullptr;
    int* err = nullptr;
    int nsm = 0;
    bool ready = false;
};
StaticScratch g_static[STATIC_MAX_DEVICES];
std::mutex g_static_mu;

// Validates the caller's device arrays before the islanding kernel indexes with them:
// bit 1 branch end out of range, bit 2 outage pointers not a non-decreasing 0..n_out run,
// bit 4 outage index out of range.
__global__ void islands_check_kernel(int n, int m, const int* f, const int* t, int L, const int* out_ptr,
                                     const int* out_idx, int n_out, int* err) {
    const int stride = gridDim.x * blockDim.x;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    int bad = 0;
    for (int e = i0; e < m; e += stride)
        if (f[e] < 0 || f[e] >= n || t[e] < 0 || t[e] >= n) bad |= 1;
    for (int c = i0; c <= L; c += stride) {
        const int p = out_ptr[c];
        if (c == 0 ? p != 0 : (p < out_ptr[c - 1] || p > n_out)) bad |= 2;
        if (c == L && p != n_out) bad |= 2;
    }
    for (int q = i0; q < n_out; q += stride)
        if (out_idx[q] < 0 || out_idx[q] >= m) bad |= 4;
    if (bad) atomicOr(err, bad);
}

int static_setup(StaticScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return ifail(std::string("gbpf_islands_device_static: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= STATIC_MAX_DEVICES) return ifail("gbpf_islands_device_static: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_static_mu);
    StaticScratch& s = g_static[dev];
    if (!s.ready) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_ints);
        if (e) return ifail(std::string("gbpf_islands_device_static: scratch address: ") + cudaGetErrorString(e));
        s.ints = static_cast<int*>(p);
        e = cudaGetSymbolAddress(&p, g_static_best);
        if (e) return ifail(std::string("gbpf_islands_device_static: scratch address: ") + cudaGetErrorString(e));
        s.best = static_cast<unsigned long long*>(p);
        e = cudaGetSymbolAddress(&p, g_static_err);
        if (e) return ifail(std::string("gbpf_islands_device_static: scratch address: ") + cudaGetErrorString(e));
        s.err = static_cast<int*>(p);
        e = cudaDeviceGetAttribute(&s.nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e) return ifail(std::string("gbpf_islands_device_static: ") + cudaGetErrorString(e));
        s.ready = true;
    }
    *out = &s;
    return 0;
}

}  // namespace

extern "C" int gbpf_islands_device_static(int n, int m, const int32_t* d_f, const int32_t* d_t,
                                          const uint8_t* d_live, int L, const int32_t* d_out_ptr,
                                          const int32_t* d_out_idx, int n_out, const uint8_t* d_is_slack,
                                          const double* d_gen_prio, int reslack, int32_t* d_labels,
                                          uint8_t* d_served, int32_t* d_ref_bus, int32_t* d_n_islands, void* stream) {
    if (n <= 0 || m < 0 || L <= 0 || n_out < 0) return ifail("gbpf_islands_device_static: invalid sizes");
    if (n > GBPF_ISLANDS_STATIC_MAX_BUS)
        return ifail("gbpf_islands_device_static: n = " + std::to_string(n) +
                     " buses exceeds the static scratch maximum of " + std::to_string(GBPF_ISLANDS_STATIC_MAX_BUS));
    if (!d_live || !d_out_ptr || !d_is_slack || !d_labels || !d_served || !d_ref_bus || !d_n_islands ||
        (m > 0 && (!d_f || !d_t)) || (n_out > 0 && !d_out_idx))
        return ifail("gbpf_islands_device_static: null device pointer");
    if (reslack && !d_gen_prio) return ifail("gbpf_islands_device_static: gen_prio is required with reslack");
    StaticScratch* s = nullptr;
    if (static_setup(&s)) return -1;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int per_cta = std::min(STATIC_INTS / (4 * n), STATIC_BEST / n);
    const int grid = std::max(1, std::min(std::min(L, 4 * s->nsm), per_cta));
    int herr = 0;
    cudaError_t e = cudaMemsetAsync(s->err, 0, sizeof(int), st);
    if (!e) {
        const int span = std::max(std::max(m, n_out), L + 1);
        const int cg = std::max(1, std::min((span + 255) / 256, 4 * s->nsm));
        islands_check_kernel<<<cg, 256, 0, st>>>(n, m, d_f, d_t, L, d_out_ptr, d_out_idx, n_out, s->err);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpyAsync(&herr, s->err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) return ifail(std::string("gbpf_islands_device_static: ") + cudaGetErrorString(e));
    if (herr & 1) return ifail("gbpf_islands_device_static: branch end out of range");
    if (herr & 2) return ifail("gbpf_islands_device_static: outage pointers must rise from 0 to n_out");
    if (herr & 4) return ifail("gbpf_islands_device_static: outage index out of range");
    islands_kernel<<<grid, NT, 0, st>>>(n, m, d_f, d_t, d_live, L, d_out_ptr, d_out_idx, d_is_slack, d_gen_prio,
                                        reslack, s->ints, s->best, d_labels, d_served, d_ref_bus, d_n_islands, s->err);
    e = cudaGetLastError();
    if (!e) e = cudaMemcpyAsync(&herr, s->err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) return ifail(std::string("gbpf_islands_device_static: ") + cudaGetErrorString(e));
    if (herr) return ifail("gbpf_islands_device_static: label propagation did not settle");
    return 0;
}
