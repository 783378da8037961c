// klu_shim.cpp -- the KLU API of klu.h over oracle/sparse_lu.cpp (test infrastructure).
#include "klu.h"

#include <cstring>
#include <vector>

#include "../sparse_lu.h"

namespace {
struct Sym {
    std::vector<int> Q;
};
}  // namespace

extern "C" {

int klu_defaults(klu_common* c) {
    if (!c) return 0;
    std::memset(c, 0, sizeof *c);
    c->tol = 0.001;
    c->ordering = 0;
    c->btf = 1;
    c->rcond = 0.0;
    return 1;
}

klu_symbolic* klu_analyze(int n, int Ap[], int Ai[], klu_common* c) {
    if (n < 0 || !Ap || !Ai) return nullptr;
    auto* s = new klu_symbolic;
    auto* impl = new Sym;
    impl->Q = slu::min_degree_order(n, Ap, Ai);
    s->n = n;
    s->nblocks = 1;
    s->impl = impl;
    if (c) c->status = 0;
    return s;
}

klu_numeric* klu_factor(int Ap[], int Ai[], double Ax[], klu_symbolic* S, klu_common* c) {
    if (!S) return nullptr;
    auto* F = new slu::Factors;
    const double tol = c ? c->tol : 0.001;
    if (!slu::factor(S->n, Ap, Ai, Ax, static_cast<Sym*>(S->impl)->Q, tol, *F)) {
        delete F;
        if (c) c->status = 1;
        return nullptr;
    }
    auto* N = new klu_numeric;
    N->n = S->n;
    N->nzoff = 0;
    N->lnz = (int)F->Li.size() + S->n;
    N->unz = (int)F->Ui.size();
    N->impl = F;
    return N;
}

int klu_refactor(int Ap[], int Ai[], double Ax[], klu_symbolic* S, klu_numeric* N, klu_common* c) {
    (void)S;
    if (!N) return 0;
    const bool ok = slu::refactor(Ap, Ai, Ax, *static_cast<slu::Factors*>(N->impl));
    if (c) c->status = ok ? 0 : 1;
    return ok ? 1 : 0;
}

int klu_solve(klu_symbolic* S, klu_numeric* N, int ldim, int nrhs, double B[], klu_common* c) {
    (void)S;
    (void)c;
    if (!N || !B) return 0;
    for (int r = 0; r < nrhs; ++r) slu::solve(*static_cast<slu::Factors*>(N->impl), B + (size_t)r * ldim);
    return 1;
}

int klu_rcond(klu_symbolic* S, klu_numeric* N, klu_common* c) {
    (void)S;
    if (!N || !c) return 0;
    c->rcond = slu::pivot_ratio(*static_cast<slu::Factors*>(N->impl));
    return 1;
}

int klu_extract(klu_numeric* N, klu_symbolic* S, int* Lp, int* Li, double* Lx, int* Up, int* Ui, double* Ux, int* Fp,
                int* Fi, double* Fx, int* P, int* Q, double* Rs, int* R, klu_common* c) {
    (void)S;
    (void)Fp;
    (void)Fi;
    (void)Fx;
    (void)c;
    if (!N) return 0;
    const auto& F = *static_cast<slu::Factors*>(N->impl);
    const int n = F.n;
    if (Lp && Li && Lx) {  // unit diagonal first in each column, then the strict part
        int q = 0;
        for (int k = 0; k < n; ++k) {
            Lp[k] = q;
            Li[q] = k;
            Lx[q++] = 1.0;
            for (int p = F.Lp[k]; p < F.Lp[k + 1]; ++p) {
                Li[q] = F.Li[p];
                Lx[q++] = F.Lx[p];
            }
        }
        Lp[n] = q;
    }
    if (Up && Ui && Ux) {
        for (int k = 0; k <= n; ++k) Up[k] = F.Up[k];
        for (size_t p = 0; p < F.Ui.size(); ++p) {
            Ui[p] = F.Ui[p];
            Ux[p] = F.Ux[p];
        }
    }
    if (P)
        for (int k = 0; k < n; ++k) P[k] = F.P[k];
    if (Q)
        for (int k = 0; k < n; ++k) Q[k] = F.Q[k];
    if (Rs)
        for (int k = 0; k < n; ++k) Rs[k] = 1.0;
    if (R) {
        R[0] = 0;
        R[1] = n;
    }
    return 1;
}

int klu_free_symbolic(klu_symbolic** S, klu_common* c) {
    (void)c;
    if (S && *S) {
        delete static_cast<Sym*>((*S)->impl);
        delete *S;
        *S = nullptr;
    }
    return 1;
}

int klu_free_numeric(klu_numeric** N, klu_common* c) {
    (void)c;
    if (N && *N) {
        delete static_cast<slu::Factors*>((*N)->impl);
        delete *N;
        *N = nullptr;
    }
    return 1;
}

}  // extern "C"
