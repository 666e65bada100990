// Project-written replacement for the two Pardiso 6.0 entry points the
// reference calls (TissueFolding/TissueFolding/SourceCode/
// NewtonRaphsonSolver.cpp:411-415 prototypes, call sequence :481-682).
// Test infrastructure only: Pardiso is a closed, licence-checked binary that
// is not available here.  Semantics kept from Pardiso's documented interface:
// 1-based CSR input, mtype 11 (real unsymmetric), phase 11/22/33/-1,
// iparm[11] = 1 -> solve with the transposed matrix, iparm[7] = number of
// iterative-refinement steps.  The solve itself is tfb_solve_csr (RCM +
// banded LU with partial pivoting).
#include <cstdio>
#include <vector>

#include "../../tf_banded.h"

extern "C" void pardisoinit(void* pt, int* /*mtype*/, int* /*solver*/, int* iparm, double* /*dparm*/, int* error) {
    void** p = static_cast<void**>(pt);
    for (int i = 0; i < 64; ++i) p[i] = nullptr;
    for (int i = 0; i < 64; ++i) iparm[i] = 0;
    *error = 0;
}

extern "C" void pardiso(void* /*pt*/, int* /*maxfct*/, int* /*mnum*/, int* mtype, int* phase, int* n,
                        double* a, int* ia, int* ja, int* /*perm*/, int* /*nrhs*/, int* iparm,
                        int* /*msglvl*/, double* b, double* x, int* error, double* /*dparm*/) {
    *error = 0;
    if (*phase == -1 || *phase == 11 || *phase == 22) return;  // factorization happens in phase 33
    if (*phase != 33 && *phase != 23 && *phase != 13) { *error = -1; return; }
    if (*mtype != 11) { std::fprintf(stderr, "pardiso stand-in: only mtype 11 is provided\n"); *error = -1; return; }
    const int N = *n;
    const int nnz = ia[N] - 1;
    std::vector<int> ia0(N + 1), ja0(nnz);
    for (int i = 0; i <= N; ++i) ia0[i] = ia[i] - 1;
    for (int p = 0; p < nnz; ++p) ja0[p] = ja[p] - 1;
    const int transpose = (iparm[11] != 0) ? 1 : 0;
    const int refine = iparm[7] > 0 ? iparm[7] : 0;
    int rc = tfb_solve_csr(N, ia0.data(), ja0.data(), a, b, x, transpose, refine);
    if (rc != 0) *error = -4;  // Pardiso's "zero pivot, numerical factorization problem"
}
