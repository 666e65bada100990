// Project-written stand-in for the few Boost.uBLAS names that the reference's
// element sources mention (dense matrix/vector, identity_matrix,
// permutation_matrix, lu_factorize, lu_substitute, stream output).  They sit
// only on paths the oracle never executes (a uBLAS overload of the 3x3
// inverse and debug printers); they are implemented plainly so the reference
// translation units compile unmodified.  Test infrastructure only.
#ifndef TF_UBLAS_SHIM_HPP
#define TF_UBLAS_SHIM_HPP
#include <cmath>
#include <cstddef>
#include <ostream>
#include <vector>

namespace boost { namespace numeric { namespace ublas {

template <class T>
class identity_matrix {
public:
    explicit identity_matrix(std::size_t n) : n_(n) {}
    std::size_t size1() const { return n_; }
    std::size_t size2() const { return n_; }
    T operator()(std::size_t i, std::size_t j) const { return i == j ? T(1) : T(0); }
private:
    std::size_t n_;
};

template <class T>
class matrix {
public:
    matrix() : r_(0), c_(0) {}
    matrix(std::size_t r, std::size_t c) : r_(r), c_(c), d_(r * c, T(0)) {}
    std::size_t size1() const { return r_; }
    std::size_t size2() const { return c_; }
    T& operator()(std::size_t i, std::size_t j) { return d_[i * c_ + j]; }
    const T& operator()(std::size_t i, std::size_t j) const { return d_[i * c_ + j]; }
    void resize(std::size_t r, std::size_t c, bool = true) { r_ = r; c_ = c; d_.assign(r * c, T(0)); }
    template <class M>
    matrix& assign(const M& m) {
        resize(m.size1(), m.size2());
        for (std::size_t i = 0; i < r_; ++i)
            for (std::size_t j = 0; j < c_; ++j) (*this)(i, j) = m(i, j);
        return *this;
    }
private:
    std::size_t r_, c_;
    std::vector<T> d_;
};

template <class T>
class vector {
public:
    vector() {}
    explicit vector(std::size_t n) : d_(n, T(0)) {}
    std::size_t size() const { return d_.size(); }
    T& operator()(std::size_t i) { return d_[i]; }
    const T& operator()(std::size_t i) const { return d_[i]; }
    T& operator[](std::size_t i) { return d_[i]; }
    const T& operator[](std::size_t i) const { return d_[i]; }
private:
    std::vector<T> d_;
};

template <class I>
class permutation_matrix {
public:
    explicit permutation_matrix(std::size_t n) : p_(n) { for (std::size_t i = 0; i < n; ++i) p_[i] = i; }
    std::size_t size() const { return p_.size(); }
    I& operator()(std::size_t i) { return p_[i]; }
    const I& operator()(std::size_t i) const { return p_[i]; }
private:
    std::vector<I> p_;
};

// Row-pivoted LU in place; returns 0 on success, k+1 if the k-th pivot is 0.
template <class T, class I>
int lu_factorize(matrix<T>& A, permutation_matrix<I>& pm) {
    const std::size_t n = A.size1();
    int singular = 0;
    for (std::size_t j = 0; j < n; ++j) {
        std::size_t piv = j;
        for (std::size_t i = j + 1; i < n; ++i)
            if (std::fabs(A(i, j)) > std::fabs(A(piv, j))) piv = i;
        pm(j) = piv;
        if (piv != j)
            for (std::size_t k = 0; k < n; ++k) { T t = A(j, k); A(j, k) = A(piv, k); A(piv, k) = t; }
        if (A(j, j) == T(0)) { if (!singular) singular = static_cast<int>(j + 1); continue; }
        for (std::size_t i = j + 1; i < n; ++i) {
            A(i, j) /= A(j, j);
            for (std::size_t k = j + 1; k < n; ++k) A(i, k) -= A(i, j) * A(j, k);
        }
    }
    return singular;
}

// Solves A X = B in place for the factorization produced by lu_factorize.
template <class T, class I>
void lu_substitute(const matrix<T>& LU, const permutation_matrix<I>& pm, matrix<T>& B) {
    const std::size_t n = LU.size1(), m = B.size2();
    for (std::size_t j = 0; j < n; ++j)
        if (pm(j) != j)
            for (std::size_t k = 0; k < m; ++k) { T t = B(j, k); B(j, k) = B(pm(j), k); B(pm(j), k) = t; }
    for (std::size_t c = 0; c < m; ++c) {
        for (std::size_t i = 0; i < n; ++i)
            for (std::size_t k = 0; k < i; ++k) B(i, c) -= LU(i, k) * B(k, c);
        for (std::size_t ii = n; ii-- > 0;) {
            for (std::size_t k = ii + 1; k < n; ++k) B(ii, c) -= LU(ii, k) * B(k, c);
            B(ii, c) /= LU(ii, ii);
        }
    }
}

template <class T>
std::ostream& operator<<(std::ostream& os, const matrix<T>& m) {
    os << "[" << m.size1() << "," << m.size2() << "](";
    for (std::size_t i = 0; i < m.size1(); ++i) {
        os << "(";
        for (std::size_t j = 0; j < m.size2(); ++j) os << m(i, j) << (j + 1 < m.size2() ? "," : "");
        os << ")";
    }
    return os << ")";
}

template <class T>
std::ostream& operator<<(std::ostream& os, const vector<T>& v) {
    os << "[" << v.size() << "](";
    for (std::size_t i = 0; i < v.size(); ++i) os << v(i) << (i + 1 < v.size() ? "," : "");
    return os << ")";
}

}}}  // namespace boost::numeric::ublas
#endif
