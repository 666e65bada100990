/*
 * Project-written stand-in for the subset of the GNU Scientific Library API
 * that the reference's element / Newton-Raphson translation units call.
 * Test infrastructure only: it lets the reference sources compile unmodified
 * into oracle/_ref so that they can serve as the parity oracle.  GSL itself
 * is not in this image.  Semantics follow GSL's published API documentation
 * (row-major gsl_matrix with a row stride `tda`, CBLAS transpose flags,
 * LU with partial pivoting); every routine is written here from that
 * description.  Routines the hot path never reaches (eigen solvers, SVD)
 * abort when called.
 */
#ifndef TF_GSL_SHIM_CORE_H
#define TF_GSL_SHIM_CORE_H

#include <stddef.h>
#include <math.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { size_t size; double* data; } gsl_block;

typedef struct {
    size_t size1;
    size_t size2;
    size_t tda;
    double* data;
    gsl_block* block;
    int owner;
} gsl_matrix;

typedef struct {
    size_t size;
    size_t stride;
    double* data;
    gsl_block* block;
    int owner;
} gsl_vector;

typedef struct { gsl_matrix matrix; } gsl_matrix_view;
typedef struct { gsl_vector vector; } gsl_vector_view;

typedef struct { size_t size; size_t* data; } gsl_permutation;

typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE_t;
typedef CBLAS_TRANSPOSE_t CBLAS_TRANSPOSE;

typedef enum {
    GSL_EIGEN_SORT_VAL_ASC, GSL_EIGEN_SORT_VAL_DESC,
    GSL_EIGEN_SORT_ABS_ASC, GSL_EIGEN_SORT_ABS_DESC
} gsl_eigen_sort_t;
typedef struct { size_t size; } gsl_eigen_symmv_workspace;

gsl_matrix* gsl_matrix_alloc(size_t n1, size_t n2);
gsl_matrix* gsl_matrix_calloc(size_t n1, size_t n2);
void gsl_matrix_free(gsl_matrix* m);
void gsl_matrix_set_zero(gsl_matrix* m);
void gsl_matrix_set_identity(gsl_matrix* m);
int gsl_matrix_memcpy(gsl_matrix* dest, const gsl_matrix* src);
int gsl_matrix_add(gsl_matrix* a, const gsl_matrix* b);
int gsl_matrix_sub(gsl_matrix* a, const gsl_matrix* b);
int gsl_matrix_scale(gsl_matrix* a, double x);
int gsl_matrix_transpose(gsl_matrix* m);
int gsl_matrix_transpose_memcpy(gsl_matrix* dest, const gsl_matrix* src);
gsl_matrix_view gsl_matrix_submatrix(gsl_matrix* m, size_t i, size_t j, size_t n1, size_t n2);

static inline double gsl_matrix_get(const gsl_matrix* m, size_t i, size_t j) {
    return m->data[i * m->tda + j];
}
static inline void gsl_matrix_set(gsl_matrix* m, size_t i, size_t j, double x) {
    m->data[i * m->tda + j] = x;
}

gsl_vector* gsl_vector_alloc(size_t n);
gsl_vector* gsl_vector_calloc(size_t n);
void gsl_vector_free(gsl_vector* v);
void gsl_vector_set_zero(gsl_vector* v);
int gsl_vector_scale(gsl_vector* v, double x);
static inline double gsl_vector_get(const gsl_vector* v, size_t i) {
    return v->data[i * v->stride];
}
static inline void gsl_vector_set(gsl_vector* v, size_t i, double x) {
    v->data[i * v->stride] = x;
}

gsl_permutation* gsl_permutation_alloc(size_t n);
void gsl_permutation_free(gsl_permutation* p);

int gsl_blas_dgemm(CBLAS_TRANSPOSE_t TransA, CBLAS_TRANSPOSE_t TransB, double alpha,
                   const gsl_matrix* A, const gsl_matrix* B, double beta, gsl_matrix* C);
double gsl_blas_dnrm2(const gsl_vector* x);

int gsl_linalg_LU_decomp(gsl_matrix* A, gsl_permutation* p, int* signum);
int gsl_linalg_LU_invert(const gsl_matrix* LU, const gsl_permutation* p, gsl_matrix* inverse);
int gsl_linalg_SV_decomp(gsl_matrix* A, gsl_matrix* V, gsl_vector* S, gsl_vector* work);

gsl_eigen_symmv_workspace* gsl_eigen_symmv_alloc(size_t n);
void gsl_eigen_symmv_free(gsl_eigen_symmv_workspace* w);
int gsl_eigen_symmv(gsl_matrix* A, gsl_vector* eval, gsl_matrix* evec, gsl_eigen_symmv_workspace* w);
int gsl_eigen_symmv_sort(gsl_vector* eval, gsl_matrix* evec, gsl_eigen_sort_t sort_type);

#ifdef __cplusplus
}
#endif

#endif
