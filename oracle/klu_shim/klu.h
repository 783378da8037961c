/* klu.h -- KLU-API shim for the CPU oracle (test infrastructure only).
 *
 * The reference's CPU solver p3s/cpp/nr_klu.cpp and lean_lu.hpp include <klu.h> from
 * SuiteSparse KLU 7.14.1 (p3s/cpp/ci/build_klu.py:49-50), which is not installed here.
 * This header declares only the names, signatures and fields those two files use
 * (nr_klu.cpp:113-114,160-161,188,196-201,621-652,723-728,753-757; lean_lu.hpp:55-65),
 * implemented in klu_shim.cpp on top of this project's textbook sparse LU
 * (oracle/sparse_lu.cpp): minimum-degree ordering, threshold partial pivoting with
 * diagonal preference (tol 0.001), no row scaling (Rs = 1), a single block (no BTF).
 */
#ifndef GBPF_KLU_SHIM_H
#define GBPF_KLU_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct klu_common_struct {
    double tol;      /* partial-pivoting threshold */
    int ordering;    /* 0 = minimum degree (KLU: AMD); other values are treated alike */
    int btf;         /* ignored: always one block */
    double rcond;    /* set by klu_rcond */
    int status;
} klu_common;

typedef struct klu_symbolic_struct {
    int n;
    int nblocks;
    void* impl;
} klu_symbolic;

typedef struct klu_numeric_struct {
    int n;
    int nzoff;
    int lnz; /* entries of L including its unit diagonal */
    int unz; /* entries of U including its diagonal */
    void* impl;
} klu_numeric;

int klu_defaults(klu_common* Common);
klu_symbolic* klu_analyze(int n, int Ap[], int Ai[], klu_common* Common);
klu_numeric* klu_factor(int Ap[], int Ai[], double Ax[], klu_symbolic* Symbolic, klu_common* Common);
int klu_refactor(int Ap[], int Ai[], double Ax[], klu_symbolic* Symbolic, klu_numeric* Numeric, klu_common* Common);
int klu_solve(klu_symbolic* Symbolic, klu_numeric* Numeric, int ldim, int nrhs, double B[], klu_common* Common);
int klu_rcond(klu_symbolic* Symbolic, klu_numeric* Numeric, klu_common* Common);
int klu_extract(klu_numeric* Numeric, klu_symbolic* Symbolic, int* Lp, int* Li, double* Lx, int* Up, int* Ui,
                double* Ux, int* Fp, int* Fi, double* Fx, int* P, int* Q, double* Rs, int* R, klu_common* Common);
int klu_free_symbolic(klu_symbolic** Symbolic, klu_common* Common);
int klu_free_numeric(klu_numeric** Numeric, klu_common* Common);

#ifdef __cplusplus
}
#endif
#endif
