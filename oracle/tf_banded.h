/*
 * Sparse direct solve by reverse Cuthill-McKee reordering followed by a
 * banded LU with partial pivoting.  TEST INFRASTRUCTURE ONLY (oracle): it is
 * the CPU stand-in for the reference's Pardiso solve
 * (TissueFolding/TissueFolding/SourceCode/NewtonRaphsonSolver.cpp:418-683,
 * mtype 11, phases 11/22/33) and is used by the oracle's Newton driver and by
 * the Pardiso replacement linked into oracle/_ref.  Pardiso itself is a
 * closed binary that is not available here.
 */
#ifndef TF_BANDED_H
#define TF_BANDED_H

#ifdef __cplusplus
extern "C" {
#endif

/* Solves A x = b (transpose == 0) or A^T x = b (transpose != 0) for the
 * n x n matrix A given in 0-based CSR (ia[n+1], ja[nnz], a[nnz]).  Performs
 * `refine` steps of iterative refinement.  Returns 0 on success, 1 on a zero
 * pivot, 2 on allocation failure. */
int tfb_solve_csr(int n, const int* ia, const int* ja, const double* a,
                  const double* b, double* x, int transpose, int refine);

#ifdef __cplusplus
}
#endif
#endif
