// postproc.cu -- the steps either side of the Newton path, on the device.
//
// * Time-series injection assembly (p3s/timeseries.py:36-141, build_sbus_matrix / _fill_sbus):
//   out[i, t] = s0[i] + sum_k coef[k] * (series[row[k], t] - base[k])  (times j for imaginary
//   contributions) over bus i's contributions in their given order -- an HBM-bound scatter of
//   the element series into the (n, T) injection matrix the solver reads.
// * Branch flows and loading of solved cases (p3s/contingency/find_overloads.py:128-260,
//   compute_branch_loading): per branch end S = conj(Y_row V) V_end sn, currents |S| / (vn |V|
//   sqrt 3), loading against the line current or transformer MVA rating; outaged branches of
//   a case report 0, non-converged cases NaN.
//
// Both keep the reference's operation order with explicitly rounded operations (no fused
// multiply-add), so the results equal a straightforward double-precision evaluation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "gbpf.h"
#include "gbpf_device.h"

namespace {

int pfail(const std::string& m) {
    gbpf::set_error(m);
    return -1;
}

constexpr int TB = 256;

__global__ void __launch_bounds__(TB) sbus_kernel(int n, int T, const double2* __restrict__ s0,
                                                  const long long* __restrict__ ptr, const int* __restrict__ row,
                                                  const double* __restrict__ coef, const double* __restrict__ base,
                                                  const uint8_t* __restrict__ imag, const double* __restrict__ series,
                                                  double2* __restrict__ out) {
    const int t = blockIdx.x * TB + threadIdx.x;
    for (int i = blockIdx.y; i < n; i += gridDim.y) {
        if (t >= T) continue;
        double2 v = s0[i];
        const long long k0 = ptr[i], k1 = ptr[i + 1];
        for (long long k = k0; k < k1; ++k) {
            const double x = series[(size_t)row[k] * T + t];
            const double d = __dmul_rn(coef[k], __dsub_rn(x, base[k]));
            if (imag[k])
                v.y = __dadd_rn(v.y, d);
            else
                v.x = __dadd_rn(v.x, d);
        }
        out[(size_t)i * T + t] = v;
    }
}

// complex a * b, rounded like the host's (a.x b.x - a.y b.y, a.x b.y + a.y b.x)
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                        __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y)); }

__global__ void __launch_bounds__(TB) flow_kernel(int nbr, int L, const int* __restrict__ f, const int* __restrict__ t,
                                                  const double2* __restrict__ y, const double* __restrict__ vn_from,
                                                  const double* __restrict__ vn_to, const double* __restrict__ rating,
                                                  const uint8_t* __restrict__ kind, double sn,
                                                  const double2* __restrict__ V, const uint8_t* __restrict__ conv,
                                                  const int* __restrict__ out_ptr, const int* __restrict__ out_idx,
                                                  double2* __restrict__ Sf, double2* __restrict__ St,
                                                  double* __restrict__ If, double* __restrict__ It,
                                                  double* __restrict__ Imax, double* __restrict__ load) {
    const int c = blockIdx.x * TB + threadIdx.x;
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    const double sq3 = 1.7320508075688772;  // sqrt(3) rounded to double
    for (int b = blockIdx.y; b < nbr; b += gridDim.y) {
        if (c >= L) continue;
        const size_t o = (size_t)b * L + c;
        bool out = false;
        if (out_ptr)
            for (int q = out_ptr[c]; q < out_ptr[c + 1]; ++q) out |= out_idx[q] == b;
        if (out || !conv[c]) {  // a non-converged case wins over an outage (NaN, not 0)
            const double z = conv[c] ? 0.0 : nan;
            // the reference stores a real NaN into its complex end powers (find_overloads.py:
            // 246-250), i.e. NaN + 0j: the reactive powers of a non-converged case read 0
            Sf[o] = make_double2(z, 0.0);
            St[o] = make_double2(z, 0.0);
            If[o] = It[o] = Imax[o] = load[o] = z;
            continue;
        }
        const int fb = f[b], tb = t[b];
        const double2 vf = V[(size_t)fb * L + c], vt = V[(size_t)tb * L + c];
        const double2 yff = y[4 * b], yft = y[4 * b + 1], ytf = y[4 * b + 2], ytt = y[4 * b + 3];
        // row sums in column order, like the sparse product of the branch admittance rows
        const double2 inf = fb < tb ? cadd(cmul(yff, vf), cmul(yft, vt)) : cadd(cmul(yft, vt), cmul(yff, vf));
        const double2 itn = fb < tb ? cadd(cmul(ytf, vf), cmul(ytt, vt)) : cadd(cmul(ytt, vt), cmul(ytf, vf));
        double2 sf = cmul(make_double2(inf.x, -inf.y), vf);
        double2 st = cmul(make_double2(itn.x, -itn.y), vt);
        sf = make_double2(__dmul_rn(sf.x, sn), __dmul_rn(sf.y, sn));
        st = make_double2(__dmul_rn(st.x, sn), __dmul_rn(st.y, sn));
        const double vmf = hypot(vf.x, vf.y), vmt = hypot(vt.x, vt.y);
        const double i_f = __ddiv_rn(hypot(sf.x, sf.y), __dmul_rn(__dmul_rn(vn_from[b], vmf), sq3));
        const double i_t = __ddiv_rn(hypot(st.x, st.y), __dmul_rn(__dmul_rn(vn_to[b], vmt), sq3));
        const double im = fmax(i_f, i_t);
        double ld;
        if (kind[b] == 0) {
            ld = __dmul_rn(__ddiv_rn(im, rating[b]), 100.0);
        } else {
            const double smax = fmax(__dmul_rn(__dmul_rn(i_f, vn_from[b]), sq3), __dmul_rn(__dmul_rn(i_t, vn_to[b]), sq3));
            ld = __dmul_rn(__ddiv_rn(smax, rating[b]), 100.0);
        }
        Sf[o] = sf;
        St[o] = st;
        If[o] = i_f;
        It[o] = i_t;
        Imax[o] = (i_f != i_f || i_t != i_t) ? nan : im;
        load[o] = (i_f != i_f || i_t != i_t) ? nan : ld;
    }
}

__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {  // a / b, as (a conj(b)) / |b|^2
    const double d = __dadd_rn(__dmul_rn(b.x, b.x), __dmul_rn(b.y, b.y));
    const double2 num = cmul(a, make_double2(b.x, -b.y));
    return make_double2(__ddiv_rn(num.x, d), __ddiv_rn(num.y, d));
}

// Branch stamps (Yff, Yft, Ytf, Ytt) of the general two-port of p3s/models/TwoWindingTransformer
// Model.py:172-175 (a line is a = b = 1, y_from = y_to = half its shunt admittance,
// TransmissionLineModel.py:45-48): Yff = (ys + y_from) / |a|^2, Yft = -ys / (conj a conj b),
// Ytf = -ys / (a b), Ytt = (ys + y_to) / |b|^2; out of service -> 0; an open end Kron-eliminated
// (TwoPort.py:69-105): Yff' = Yff - Yft Ytf / Ytt with the to end open (the from end analogous),
// transfer terms 0, both ends open -> 0.
__global__ void __launch_bounds__(TB) stamp_kernel(int m, const double2* __restrict__ ys, const double2* __restrict__ yf,
                                                   const double2* __restrict__ yt, const double2* __restrict__ a,
                                                   const double2* __restrict__ b, const uint8_t* __restrict__ in_service,
                                                   const uint8_t* __restrict__ open_f, const uint8_t* __restrict__ open_t,
                                                   double2* __restrict__ out) {
    const int e = blockIdx.x * TB + threadIdx.x;
    if (e >= m) return;
    const double2 z = make_double2(0.0, 0.0);
    if (in_service && !in_service[e]) {
        out[4 * e] = out[4 * e + 1] = out[4 * e + 2] = out[4 * e + 3] = z;
        return;
    }
    const double2 s = ys[e], A = a[e], B = b[e];
    const double a2 = __dadd_rn(__dmul_rn(A.x, A.x), __dmul_rn(A.y, A.y));
    const double b2 = __dadd_rn(__dmul_rn(B.x, B.x), __dmul_rn(B.y, B.y));
    const double2 sf = cadd(s, yf[e]), st = cadd(s, yt[e]);
    double2 ff = make_double2(__ddiv_rn(sf.x, a2), __ddiv_rn(sf.y, a2));
    double2 tt = make_double2(__ddiv_rn(st.x, b2), __ddiv_rn(st.y, b2));
    const double2 ms = make_double2(-s.x, -s.y);
    double2 ft = cdiv(ms, cmul(make_double2(A.x, -A.y), make_double2(B.x, -B.y)));
    double2 tf = cdiv(ms, cmul(A, B));
    const bool of = open_f && open_f[e], ot = open_t && open_t[e];
    if (of || ot) {
        const bool tt0 = tt.x == 0.0 && tt.y == 0.0, ff0 = ff.x == 0.0 && ff.y == 0.0;
        const double2 ff_red = tt0 ? ff : make_double2(__dsub_rn(ff.x, cdiv(cmul(ft, tf), tt).x),
                                                       __dsub_rn(ff.y, cdiv(cmul(ft, tf), tt).y));
        const double2 tt_red = ff0 ? tt : make_double2(__dsub_rn(tt.x, cdiv(cmul(tf, ft), ff).x),
                                                       __dsub_rn(tt.y, cdiv(cmul(tf, ft), ff).y));
        const double2 nff = of ? z : (ot ? ff_red : ff);
        const double2 ntt = ot ? z : (of ? tt_red : tt);
        ff = nff;
        tt = ntt;
        ft = tf = z;
    }
    out[4 * e] = ff;
    out[4 * e + 1] = ft;
    out[4 * e + 2] = tf;
    out[4 * e + 3] = tt;
}

// Ybus values from branch stamps (TwoPort.py:133-149 create_y_matrix, then the bus shunts):
// Yx[k] = sum over the contributions of CSR entry k in order; a contribution below 4 m is
// stamp entry src of the branch table, 4 m + i the shunt of bus i.
__global__ void __launch_bounds__(TB) gather_kernel(int nnz, int m4, const int* __restrict__ ptr,
                                                    const int* __restrict__ src, const double2* __restrict__ stamps,
                                                    const double2* __restrict__ shunt, double2* __restrict__ Y,
                                                    float2* __restrict__ Y32) {
    const int k = blockIdx.x * TB + threadIdx.x;
    if (k >= nnz) return;
    double2 v = make_double2(0.0, 0.0);
    for (int q = ptr[k]; q < ptr[k + 1]; ++q) {
        const int s = src[q];
        v = cadd(v, s < m4 ? stamps[s] : shunt[s - m4]);
    }
    Y[k] = v;
    if (Y32) Y32[k] = make_float2((float)v.x, (float)v.y);
}

template <typename T>
struct DevVec {
    T* p = nullptr;
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)); }
    ~DevVec() {
        if (p) cudaFree(p);
    }
};

#define PK(x)                                                                                        \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) return pfail(std::string(#x) + " failed: " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

cudaError_t gbpf::launch_ybus_gather(int nnz, int m4, const int* ptr, const int* src, const double2* stamps,
                                     const double2* shunt, double2* Y, float2* Y32, cudaStream_t stream) {
    gather_kernel<<<(nnz + TB - 1) / TB, TB, 0, stream>>>(nnz, m4, ptr, src, stamps, shunt, Y, Y32);
    return cudaGetLastError();
}

extern "C" {

int gbpf_build_sbus_device(int n, int T, const double* s0, const int64_t* ptr, const int32_t* row, const double* coef,
                           const double* base, const uint8_t* imag, const double* series, double* out, void* stream) {
    if (n <= 0 || T <= 0) return pfail("build_sbus: n and T must be > 0");
    if (!s0 || !ptr || !out) return pfail("build_sbus: null argument");
    const dim3 grid((T + TB - 1) / TB, std::min(n, 65535));
    sbus_kernel<<<grid, TB, 0, static_cast<cudaStream_t>(stream)>>>(
        n, T, reinterpret_cast<const double2*>(s0), reinterpret_cast<const long long*>(ptr), row, coef, base, imag,
        series, reinterpret_cast<double2*>(out));
    PK(cudaGetLastError());
    return 0;
}

int gbpf_build_sbus(int n, int T, int R, const double* s0, const int64_t* ptr, const int32_t* row, const double* coef,
                    const double* base, const uint8_t* imag, const double* series, double* out) {
    if (n <= 0 || T <= 0 || R < 0) return pfail("build_sbus: n and T must be > 0");
    const long long K = ptr[n];
    if (ptr[0] != 0 || K < 0) return pfail("build_sbus: contribution pointers must start at 0");
    for (int i = 0; i < n; ++i)
        if (ptr[i + 1] < ptr[i]) return pfail("build_sbus: contribution pointers must not decrease");
    for (long long k = 0; k < K; ++k)
        if (row[k] < 0 || row[k] >= R) return pfail("build_sbus: series row out of range");
    DevVec<double> ds0, dcoef, dbase, dser, dout;
    DevVec<long long> dptr;
    DevVec<int> drow;
    DevVec<uint8_t> dimag;
    PK(ds0.alloc(2 * (size_t)n));
    PK(dptr.alloc(n + 1));
    PK(drow.alloc(K));
    PK(dcoef.alloc(K));
    PK(dbase.alloc(K));
    PK(dimag.alloc(K));
    PK(dser.alloc((size_t)R * T));
    PK(dout.alloc(2 * (size_t)n * T));
    PK(cudaMemcpy(ds0.p, s0, 16 * (size_t)n, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(dptr.p, ptr, 8 * (size_t)(n + 1), cudaMemcpyHostToDevice));
    if (K) {
        PK(cudaMemcpy(drow.p, row, 4 * (size_t)K, cudaMemcpyHostToDevice));
        PK(cudaMemcpy(dcoef.p, coef, 8 * (size_t)K, cudaMemcpyHostToDevice));
        PK(cudaMemcpy(dbase.p, base, 8 * (size_t)K, cudaMemcpyHostToDevice));
        PK(cudaMemcpy(dimag.p, imag, (size_t)K, cudaMemcpyHostToDevice));
    }
    if (R) PK(cudaMemcpy(dser.p, series, 8 * (size_t)R * T, cudaMemcpyHostToDevice));
    if (int rc = gbpf_build_sbus_device(n, T, ds0.p, reinterpret_cast<const int64_t*>(dptr.p), drow.p, dcoef.p,
                                        dbase.p, dimag.p, dser.p, dout.p, nullptr))
        return rc;
    PK(cudaDeviceSynchronize());
    PK(cudaMemcpy(out, dout.p, 16 * (size_t)n * T, cudaMemcpyDeviceToHost));
    return 0;
}

int gbpf_branch_stamps_device(int m, const double* ys, const double* y_from, const double* y_to, const double* a,
                              const double* b, const uint8_t* in_service, const uint8_t* open_from,
                              const uint8_t* open_to, double* stamps, void* stream) {
    if (m <= 0) return pfail("branch_stamps: m must be > 0");
    stamp_kernel<<<(m + TB - 1) / TB, TB, 0, static_cast<cudaStream_t>(stream)>>>(
        m, reinterpret_cast<const double2*>(ys), reinterpret_cast<const double2*>(y_from),
        reinterpret_cast<const double2*>(y_to), reinterpret_cast<const double2*>(a),
        reinterpret_cast<const double2*>(b), in_service, open_from, open_to, reinterpret_cast<double2*>(stamps));
    PK(cudaGetLastError());
    return 0;
}

int gbpf_branch_stamps(int m, const double* ys, const double* y_from, const double* y_to, const double* a,
                       const double* b, const uint8_t* in_service, const uint8_t* open_from, const uint8_t* open_to,
                       double* stamps) {
    if (m <= 0) return pfail("branch_stamps: m must be > 0");
    DevVec<double> d[6];
    DevVec<uint8_t> u[3];
    const double* hin[5] = {ys, y_from, y_to, a, b};
    for (int i = 0; i < 5; ++i) {
        PK(d[i].alloc(2 * (size_t)m));
        PK(cudaMemcpy(d[i].p, hin[i], 16 * (size_t)m, cudaMemcpyHostToDevice));
    }
    PK(d[5].alloc(8 * (size_t)m));
    const uint8_t* uin[3] = {in_service, open_from, open_to};
    for (int i = 0; i < 3; ++i)
        if (uin[i]) {
            PK(u[i].alloc(m));
            PK(cudaMemcpy(u[i].p, uin[i], (size_t)m, cudaMemcpyHostToDevice));
        }
    if (int rc = gbpf_branch_stamps_device(m, d[0].p, d[1].p, d[2].p, d[3].p, d[4].p, u[0].p, u[1].p, u[2].p, d[5].p,
                                           nullptr))
        return rc;
    PK(cudaDeviceSynchronize());
    PK(cudaMemcpy(stamps, d[5].p, 64 * (size_t)m, cudaMemcpyDeviceToHost));
    return 0;
}

int gbpf_branch_flows_device(int nbr, int L, const int32_t* f, const int32_t* t, const double* y,
                             const double* vn_from, const double* vn_to, const double* rating, const uint8_t* kind,
                             double sn_mva, const double* V, const uint8_t* converged, const int32_t* out_ptr,
                             const int32_t* out_idx, double* S_from, double* S_to, double* i_from, double* i_to,
                             double* i_max, double* loading, void* stream) {
    if (nbr <= 0 || L <= 0) return pfail("branch_flows: nbr and L must be > 0");
    const dim3 grid((L + TB - 1) / TB, std::min(nbr, 65535));
    flow_kernel<<<grid, TB, 0, static_cast<cudaStream_t>(stream)>>>(
        nbr, L, f, t, reinterpret_cast<const double2*>(y), vn_from, vn_to, rating, kind, sn_mva,
        reinterpret_cast<const double2*>(V), converged, out_ptr, out_idx, reinterpret_cast<double2*>(S_from),
        reinterpret_cast<double2*>(S_to), i_from, i_to, i_max, loading);
    PK(cudaGetLastError());
    return 0;
}

int gbpf_branch_flows(int n, int nbr, int L, const int32_t* f, const int32_t* t, const double* y,
                      const double* vn_from, const double* vn_to, const double* rating, const uint8_t* kind,
                      double sn_mva, const double* V, const uint8_t* converged, const int32_t* out_ptr,
                      const int32_t* out_idx, double* S_from, double* S_to, double* i_from, double* i_to,
                      double* i_max, double* loading) {
    if (n <= 0 || nbr <= 0 || L <= 0) return pfail("branch_flows: n, nbr and L must be > 0");
    for (int b = 0; b < nbr; ++b)
        if (f[b] < 0 || f[b] >= n || t[b] < 0 || t[b] >= n) return pfail("branch_flows: branch end out of range");
    int nout = 0;
    if (out_ptr) {
        if (out_ptr[0] != 0) return pfail("branch_flows: outage pointers must start at 0");
        for (int c = 0; c < L; ++c)
            if (out_ptr[c + 1] < out_ptr[c]) return pfail("branch_flows: outage pointers must not decrease");
        nout = out_ptr[L];
    }
    const size_t nl = (size_t)nbr * L;
    DevVec<int> df, dt, dop, doi;
    DevVec<double> dy, dvf, dvt, drt, dV, dsf, dst, dif, dit, dim, dld;
    DevVec<uint8_t> dk, dcv;
    PK(df.alloc(nbr));
    PK(dt.alloc(nbr));
    PK(dy.alloc(8 * (size_t)nbr));
    PK(dvf.alloc(nbr));
    PK(dvt.alloc(nbr));
    PK(drt.alloc(nbr));
    PK(dk.alloc(nbr));
    PK(dV.alloc(2 * (size_t)n * L));
    PK(dcv.alloc(L));
    PK(dsf.alloc(2 * nl));
    PK(dst.alloc(2 * nl));
    PK(dif.alloc(nl));
    PK(dit.alloc(nl));
    PK(dim.alloc(nl));
    PK(dld.alloc(nl));
    PK(cudaMemcpy(df.p, f, 4 * (size_t)nbr, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(dt.p, t, 4 * (size_t)nbr, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(dy.p, y, 64 * (size_t)nbr, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(dvf.p, vn_from, 8 * (size_t)nbr, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(dvt.p, vn_to, 8 * (size_t)nbr, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(drt.p, rating, 8 * (size_t)nbr, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(dk.p, kind, (size_t)nbr, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(dV.p, V, 16 * (size_t)n * L, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(dcv.p, converged, (size_t)L, cudaMemcpyHostToDevice));
    if (out_ptr) {
        PK(dop.alloc(L + 1));
        PK(doi.alloc(nout));
        PK(cudaMemcpy(dop.p, out_ptr, 4 * (size_t)(L + 1), cudaMemcpyHostToDevice));
        if (nout) PK(cudaMemcpy(doi.p, out_idx, 4 * (size_t)nout, cudaMemcpyHostToDevice));
    }
    if (int rc = gbpf_branch_flows_device(nbr, L, df.p, dt.p, dy.p, dvf.p, dvt.p, drt.p, dk.p, sn_mva, dV.p, dcv.p,
                                          out_ptr ? dop.p : nullptr, out_ptr ? doi.p : nullptr, dsf.p, dst.p, dif.p,
                                          dit.p, dim.p, dld.p, nullptr))
        return rc;
    PK(cudaDeviceSynchronize());
    PK(cudaMemcpy(S_from, dsf.p, 16 * nl, cudaMemcpyDeviceToHost));
    PK(cudaMemcpy(S_to, dst.p, 16 * nl, cudaMemcpyDeviceToHost));
    PK(cudaMemcpy(i_from, dif.p, 8 * nl, cudaMemcpyDeviceToHost));
    PK(cudaMemcpy(i_to, dit.p, 8 * nl, cudaMemcpyDeviceToHost));
    PK(cudaMemcpy(i_max, dim.p, 8 * nl, cudaMemcpyDeviceToHost));
    PK(cudaMemcpy(loading, dld.p, 8 * nl, cudaMemcpyDeviceToHost));
    return 0;
}

}  // extern "C"
