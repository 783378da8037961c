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
    __shared__ int s_total;
    __shared__ int s_warp[NT / 32];
    const int tid = threadIdx.x;
    for (int c = blockIdx.x; c < L; c += gridDim.x) {
        const int o0 = out_ptr[c], o1 = out_ptr[c + 1];
        for (int v = tid; v < n; v += NT) lab[v] = v;
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
                if (tid == 0) atomicCAS(err, 0, 1);
                break;
            }
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

extern "C" int gbpf_islands(int n, int m, const int32_t* f, const int32_t* t, const uint8_t* live, int L,
                            const int32_t* out_ptr, const int32_t* out_idx, const uint8_t* is_slack,
                            const double* gen_prio, int reslack, int32_t* labels, uint8_t* served, int32_t* ref_bus,
                            int32_t* n_islands) {
    if (n <= 0 || m < 0 || L <= 0) return ifail("gbpf_islands: invalid sizes");
    for (int e = 0; e < m; ++e)
        if (f[e] < 0 || f[e] >= n || t[e] < 0 || t[e] >= n) return ifail("gbpf_islands: branch end out of range");
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
