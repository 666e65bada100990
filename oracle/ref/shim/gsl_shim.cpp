// Project-written implementation of the GSL subset declared in
// gsl/gsl_shim_core.h.  Test infrastructure for the oracle build only.
// Loop orders follow the plain definitions in GSL's documentation: dgemm
// accumulates over k in ascending order, LU is row-pivoted Doolittle
// elimination, LU_invert solves one unit column at a time.
#include "gsl/gsl_shim_core.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <cmath>
#include <vector>

extern "C" {

static void shim_fatal(const char* what) {
    std::fprintf(stderr, "gsl shim: %s is not provided by the oracle stand-in\n", what);
    std::abort();
}

gsl_matrix* gsl_matrix_alloc(size_t n1, size_t n2) {
    gsl_matrix* m = static_cast<gsl_matrix*>(std::malloc(sizeof(gsl_matrix)));
    m->size1 = n1;
    m->size2 = n2;
    m->tda = n2;
    m->data = static_cast<double*>(std::malloc(sizeof(double) * (n1 * n2 > 0 ? n1 * n2 : 1)));
    m->block = nullptr;
    m->owner = 1;
    return m;
}

gsl_matrix* gsl_matrix_calloc(size_t n1, size_t n2) {
    gsl_matrix* m = gsl_matrix_alloc(n1, n2);
    std::memset(m->data, 0, sizeof(double) * n1 * n2);
    return m;
}

void gsl_matrix_free(gsl_matrix* m) {
    if (!m) return;
    if (m->owner) std::free(m->data);
    std::free(m);
}

void gsl_matrix_set_zero(gsl_matrix* m) {
    for (size_t i = 0; i < m->size1; ++i)
        for (size_t j = 0; j < m->size2; ++j) m->data[i * m->tda + j] = 0.0;
}

void gsl_matrix_set_identity(gsl_matrix* m) {
    for (size_t i = 0; i < m->size1; ++i)
        for (size_t j = 0; j < m->size2; ++j) m->data[i * m->tda + j] = (i == j) ? 1.0 : 0.0;
}

int gsl_matrix_memcpy(gsl_matrix* dest, const gsl_matrix* src) {
    for (size_t i = 0; i < src->size1; ++i)
        for (size_t j = 0; j < src->size2; ++j) dest->data[i * dest->tda + j] = src->data[i * src->tda + j];
    return 0;
}

int gsl_matrix_add(gsl_matrix* a, const gsl_matrix* b) {
    for (size_t i = 0; i < a->size1; ++i)
        for (size_t j = 0; j < a->size2; ++j) a->data[i * a->tda + j] += b->data[i * b->tda + j];
    return 0;
}

int gsl_matrix_sub(gsl_matrix* a, const gsl_matrix* b) {
    for (size_t i = 0; i < a->size1; ++i)
        for (size_t j = 0; j < a->size2; ++j) a->data[i * a->tda + j] -= b->data[i * b->tda + j];
    return 0;
}

int gsl_matrix_scale(gsl_matrix* a, double x) {
    for (size_t i = 0; i < a->size1; ++i)
        for (size_t j = 0; j < a->size2; ++j) a->data[i * a->tda + j] *= x;
    return 0;
}

int gsl_matrix_transpose(gsl_matrix* m) {
    for (size_t i = 0; i < m->size1; ++i)
        for (size_t j = i + 1; j < m->size2; ++j) {
            double t = m->data[i * m->tda + j];
            m->data[i * m->tda + j] = m->data[j * m->tda + i];
            m->data[j * m->tda + i] = t;
        }
    return 0;
}

int gsl_matrix_transpose_memcpy(gsl_matrix* dest, const gsl_matrix* src) {
    for (size_t i = 0; i < dest->size1; ++i)
        for (size_t j = 0; j < dest->size2; ++j) dest->data[i * dest->tda + j] = src->data[j * src->tda + i];
    return 0;
}

gsl_matrix_view gsl_matrix_submatrix(gsl_matrix* m, size_t i, size_t j, size_t n1, size_t n2) {
    gsl_matrix_view v;
    v.matrix.size1 = n1;
    v.matrix.size2 = n2;
    v.matrix.tda = m->tda;
    v.matrix.data = m->data + i * m->tda + j;
    v.matrix.block = nullptr;
    v.matrix.owner = 0;
    return v;
}

gsl_vector* gsl_vector_alloc(size_t n) {
    gsl_vector* v = static_cast<gsl_vector*>(std::malloc(sizeof(gsl_vector)));
    v->size = n;
    v->stride = 1;
    v->data = static_cast<double*>(std::malloc(sizeof(double) * (n > 0 ? n : 1)));
    v->block = nullptr;
    v->owner = 1;
    return v;
}

gsl_vector* gsl_vector_calloc(size_t n) {
    gsl_vector* v = gsl_vector_alloc(n);
    std::memset(v->data, 0, sizeof(double) * n);
    return v;
}

void gsl_vector_free(gsl_vector* v) {
    if (!v) return;
    if (v->owner) std::free(v->data);
    std::free(v);
}

void gsl_vector_set_zero(gsl_vector* v) {
    for (size_t i = 0; i < v->size; ++i) v->data[i * v->stride] = 0.0;
}

int gsl_vector_scale(gsl_vector* v, double x) {
    for (size_t i = 0; i < v->size; ++i) v->data[i * v->stride] *= x;
    return 0;
}

gsl_permutation* gsl_permutation_alloc(size_t n) {
    gsl_permutation* p = static_cast<gsl_permutation*>(std::malloc(sizeof(gsl_permutation)));
    p->size = n;
    p->data = static_cast<size_t*>(std::malloc(sizeof(size_t) * (n > 0 ? n : 1)));
    for (size_t i = 0; i < n; ++i) p->data[i] = i;
    return p;
}

void gsl_permutation_free(gsl_permutation* p) {
    if (!p) return;
    std::free(p->data);
    std::free(p);
}

int gsl_blas_dgemm(CBLAS_TRANSPOSE_t TransA, CBLAS_TRANSPOSE_t TransB, double alpha,
                   const gsl_matrix* A, const gsl_matrix* B, double beta, gsl_matrix* C) {
    const size_t M = C->size1, N = C->size2;
    const size_t K = (TransA == CblasNoTrans) ? A->size2 : A->size1;
    for (size_t i = 0; i < M; ++i) {
        for (size_t j = 0; j < N; ++j) {
            double acc = 0.0;
            for (size_t k = 0; k < K; ++k) {
                double a = (TransA == CblasNoTrans) ? A->data[i * A->tda + k] : A->data[k * A->tda + i];
                double b = (TransB == CblasNoTrans) ? B->data[k * B->tda + j] : B->data[j * B->tda + k];
                acc += a * b;
            }
            double& c = C->data[i * C->tda + j];
            c = (beta == 0.0) ? alpha * acc : alpha * acc + beta * c;
        }
    }
    return 0;
}

double gsl_blas_dnrm2(const gsl_vector* x) {
    double s = 0.0;
    for (size_t i = 0; i < x->size; ++i) {
        double v = x->data[i * x->stride];
        s += v * v;
    }
    return std::sqrt(s);
}

int gsl_linalg_LU_decomp(gsl_matrix* A, gsl_permutation* p, int* signum) {
    const size_t N = A->size1;
    *signum = 1;
    for (size_t i = 0; i < N; ++i) p->data[i] = i;
    for (size_t j = 0; j + 1 < N; ++j) {
        double amax = std::fabs(A->data[j * A->tda + j]);
        size_t ipiv = j;
        for (size_t i = j + 1; i < N; ++i) {
            double a = std::fabs(A->data[i * A->tda + j]);
            if (a > amax) { amax = a; ipiv = i; }
        }
        if (ipiv != j) {
            for (size_t k = 0; k < N; ++k) {
                double t = A->data[j * A->tda + k];
                A->data[j * A->tda + k] = A->data[ipiv * A->tda + k];
                A->data[ipiv * A->tda + k] = t;
            }
            size_t t = p->data[j]; p->data[j] = p->data[ipiv]; p->data[ipiv] = t;
            *signum = -(*signum);
        }
        const double ajj = A->data[j * A->tda + j];
        if (ajj != 0.0) {
            for (size_t i = j + 1; i < N; ++i) {
                const double aij = A->data[i * A->tda + j] / ajj;
                A->data[i * A->tda + j] = aij;
                for (size_t k = j + 1; k < N; ++k) A->data[i * A->tda + k] -= aij * A->data[j * A->tda + k];
            }
        }
    }
    return 0;
}

int gsl_linalg_LU_invert(const gsl_matrix* LU, const gsl_permutation* p, gsl_matrix* inverse) {
    const size_t N = LU->size1;
    double x[64];
    if (N > 64) shim_fatal("LU_invert of order > 64");
    for (size_t c = 0; c < N; ++c) {
        // b = P e_c : x[i] = e_c[p[i]]
        for (size_t i = 0; i < N; ++i) x[i] = (p->data[i] == c) ? 1.0 : 0.0;
        for (size_t i = 0; i < N; ++i) {           // unit lower solve
            double s = x[i];
            for (size_t k = 0; k < i; ++k) s -= LU->data[i * LU->tda + k] * x[k];
            x[i] = s;
        }
        for (size_t ii = N; ii-- > 0;) {           // upper solve
            double s = x[ii];
            for (size_t k = ii + 1; k < N; ++k) s -= LU->data[ii * LU->tda + k] * x[k];
            x[ii] = s / LU->data[ii * LU->tda + ii];
        }
        for (size_t i = 0; i < N; ++i) inverse->data[i * inverse->tda + c] = x[i];
    }
    return 0;
}

// A = U S V^T by one-sided (Hestenes) Jacobi rotations: pairs of columns of
// A are rotated until orthogonal, the rotations accumulated in V; the
// singular values are the final column norms, U the normalised columns.
// Singular values descending, as GSL returns them.  On return A holds U.
int gsl_linalg_SV_decomp(gsl_matrix* A, gsl_matrix* V, gsl_vector* S, gsl_vector*) {
    const size_t M = A->size1, N = A->size2;
    auto a = [&](size_t i, size_t j) -> double& { return A->data[i * A->tda + j]; };
    auto v = [&](size_t i, size_t j) -> double& { return V->data[i * V->tda + j]; };
    for (size_t i = 0; i < N; ++i)
        for (size_t j = 0; j < N; ++j) v(i, j) = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        bool rotated = false;
        for (size_t p = 0; p + 1 < N; ++p)
            for (size_t q = p + 1; q < N; ++q) {
                double alpha = 0.0, beta = 0.0, gamma = 0.0;
                for (size_t i = 0; i < M; ++i) {
                    alpha += a(i, p) * a(i, p);
                    beta += a(i, q) * a(i, q);
                    gamma += a(i, p) * a(i, q);
                }
                if (gamma == 0.0 || std::fabs(gamma) <= 1e-17 * std::sqrt(alpha * beta)) continue;
                rotated = true;
                const double zeta = (beta - alpha) / (2.0 * gamma);
                const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / std::sqrt(1.0 + t * t), sn = c * t;
                for (size_t i = 0; i < M; ++i) {
                    const double x = a(i, p), y = a(i, q);
                    a(i, p) = c * x - sn * y;
                    a(i, q) = sn * x + c * y;
                }
                for (size_t i = 0; i < N; ++i) {
                    const double x = v(i, p), y = v(i, q);
                    v(i, p) = c * x - sn * y;
                    v(i, q) = sn * x + c * y;
                }
            }
        if (!rotated) break;
    }
    std::vector<double> sig(N);
    for (size_t j = 0; j < N; ++j) {
        double n2 = 0.0;
        for (size_t i = 0; i < M; ++i) n2 += a(i, j) * a(i, j);
        sig[j] = std::sqrt(n2);
        if (sig[j] > 0)
            for (size_t i = 0; i < M; ++i) a(i, j) /= sig[j];
    }
    for (size_t j = 0; j < N; ++j) {  // descending order
        size_t best = j;
        for (size_t k = j + 1; k < N; ++k)
            if (sig[k] > sig[best]) best = k;
        if (best == j) continue;
        std::swap(sig[j], sig[best]);
        for (size_t i = 0; i < M; ++i) std::swap(a(i, j), a(i, best));
        for (size_t i = 0; i < N; ++i) std::swap(v(i, j), v(i, best));
    }
    for (size_t j = 0; j < N; ++j) S->data[j * S->stride] = sig[j];
    return 0;
}

gsl_eigen_symmv_workspace* gsl_eigen_symmv_alloc(size_t) {
    shim_fatal("gsl_eigen_symmv_alloc");
    return nullptr;
}
void gsl_eigen_symmv_free(gsl_eigen_symmv_workspace*) { shim_fatal("gsl_eigen_symmv_free"); }
int gsl_eigen_symmv(gsl_matrix*, gsl_vector*, gsl_matrix*, gsl_eigen_symmv_workspace*) {
    shim_fatal("gsl_eigen_symmv");
    return -1;
}
int gsl_eigen_symmv_sort(gsl_vector*, gsl_matrix*, gsl_eigen_sort_t) {
    shim_fatal("gsl_eigen_symmv_sort");
    return -1;
}

}  // extern "C"
