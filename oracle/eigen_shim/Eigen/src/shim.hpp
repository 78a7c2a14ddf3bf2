#pragma once
// Minimal stand-in for the subset of Eigen 3.4's public API that the nonlocal
// (NonLocFEM) thermal path uses.  It exists only so that the reference's own
// headers (libraries/mesh, libraries/solvers) compile unchanged in this
// container, where Eigen is absent, and can be run as the parity oracle.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library includes this.
//
// Written from Eigen's documented behaviour (class and method names, argument
// meaning), not from its source.  Two pieces carry arithmetic of their own and
// are restatements of published methods:
//   * IncompleteCholesky<T, Upper, NaturalOrdering>: Lin & More (1999),
//     "Incomplete Cholesky factorizations with limited memory", SIAM J. Sci.
//     Comput. 21(1): l2 column scaling, diagonal shift alpha_S = 1e-3 doubled
//     on breakdown (at most 10 attempts), left-looking column factorisation that
//     keeps, per column, as many off-diagonal entries as the input column had
//     (the largest in magnitude).  Used by the reference as its "ILLT"
//     preconditioner (libraries/solvers/slae/eigen_preconditioner.hpp:57).
//   * SimplicialCholesky<..., Upper, NaturalOrdering>: a band LDL^T
//     factorisation (used by the 1D stationary solver,
//     libraries/solvers/solver_1d/thermal/stationary_heat_equation_solver_1d.hpp:99-105).
//   * ConjugateGradient<..., Upper> and BiCGSTAB with the diagonal
//     preconditioner: the textbook iterations (Hestenes & Stiefel 1952; van der
//     Vorst 1992) with Eigen's documented defaults (used by the nonlinear
//     boundary and non-symmetric branches of the stationary solver).
// The branch the configurations never reach (Eigen::SparseLU) throws
// std::logic_error.

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <stdexcept>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>   // Eigen/Core pulls this in when OpenMP is enabled
#endif

namespace Eigen {

enum { Dynamic = -1 };
enum StorageOptions { ColMajor = 0, RowMajor = 1 };
enum UpLoType { Lower = 1, Upper = 2 };
enum ComputationInfo { Success = 0, NumericalIssue = 1, NoConvergence = 2, InvalidInput = 3 };

template<class T, int Rows, int Cols> class Matrix;

// ---------------------------------------------------------------- dense vector
template<class T>
class Matrix<T, Dynamic, 1> {
    std::vector<T> _v;

public:
    using Scalar = T;
    Matrix() = default;
    explicit Matrix(long n) : _v(size_t(n), T{0}) {}
    Matrix(const Matrix&) = default;
    Matrix(Matrix&&) noexcept = default;
    Matrix& operator=(const Matrix&) = default;
    Matrix& operator=(Matrix&&) noexcept = default;

    static Matrix Zero(long n) { return Matrix(n); }
    static Matrix Constant(long n, const T v) { Matrix m(n); std::fill(m._v.begin(), m._v.end(), v); return m; }

    long size() const noexcept { return long(_v.size()); }
    long rows() const noexcept { return size(); }
    long cols() const noexcept { return 1; }
    void resize(long n) { _v.resize(size_t(n)); }
    void setZero() { std::fill(_v.begin(), _v.end(), T{0}); }
    void swap(Matrix& other) noexcept { _v.swap(other._v); }

    T* data() noexcept { return _v.data(); }
    const T* data() const noexcept { return _v.data(); }
    T& operator[](long i) { return _v[size_t(i)]; }
    const T& operator[](long i) const { return _v[size_t(i)]; }
    T& operator()(long i) { return _v[size_t(i)]; }
    const T& operator()(long i) const { return _v[size_t(i)]; }
    auto begin() noexcept { return _v.begin(); }
    auto end() noexcept { return _v.end(); }
    auto begin() const noexcept { return _v.begin(); }
    auto end() const noexcept { return _v.end(); }
    auto cbegin() const noexcept { return _v.cbegin(); }
    auto cend() const noexcept { return _v.cend(); }

    T dot(const Matrix& o) const {
        T s = T{0};
        for (size_t i = 0; i < _v.size(); ++i) s += _v[i] * o._v[i];
        return s;
    }
    T squaredNorm() const { return dot(*this); }
    T norm() const { return std::sqrt(squaredNorm()); }

    // Contiguous segment view: block(start, 0, length, 1).
    struct Block {
        T* p; long n;
        Block& operator+=(const Matrix& o) { for (long i = 0; i < n; ++i) p[i] += o[i]; return *this; }
        Block& operator-=(const Matrix& o) { for (long i = 0; i < n; ++i) p[i] -= o[i]; return *this; }
    };
    Block block(long start, long, long length, long) { return Block{_v.data() + start, length}; }

    Matrix& operator+=(const Matrix& o) { for (size_t i = 0; i < _v.size(); ++i) _v[i] += o._v[i]; return *this; }
    Matrix& operator-=(const Matrix& o) { for (size_t i = 0; i < _v.size(); ++i) _v[i] -= o._v[i]; return *this; }
    Matrix& operator*=(const T s) { for (T& x : _v) x *= s; return *this; }
    friend Matrix operator+(Matrix a, const Matrix& b) { a += b; return a; }
    friend Matrix operator-(Matrix a, const Matrix& b) { a -= b; return a; }
    friend Matrix operator*(const T s, Matrix a) { a *= s; return a; }
    friend Matrix operator*(Matrix a, const T s) { a *= s; return a; }
};

// ------------------------------------------------------- dense column-major matrix
template<class T>
class Matrix<T, Dynamic, Dynamic> {
    long _r = 0, _c = 0;
    std::vector<T> _v;

public:
    Matrix() = default;
    Matrix(long r, long c) : _r{r}, _c{c}, _v(size_t(r * c), T{0}) {}
    void resize(long r, long c) { _r = r; _c = c; _v.assign(size_t(r * c), T{0}); }
    long rows() const noexcept { return _r; }
    long cols() const noexcept { return _c; }
    T& operator()(long r, long c) { return _v[size_t(c * _r + r)]; }
    const T& operator()(long r, long c) const { return _v[size_t(c * _r + r)]; }

    struct Block {
        T* p; long n;
        void setZero() { std::fill(p, p + n, T{0}); }
        Block& operator+=(const Block& o) { for (long i = 0; i < n; ++i) p[i] += o.p[i]; return *this; }
        operator Matrix<T, Dynamic, 1>() const {
            Matrix<T, Dynamic, 1> v(n);
            std::copy(p, p + n, v.data());
            return v;
        }
    };
    Block col(long c) { return Block{_v.data() + c * _r, _r}; }
    Block col(long c) const { return Block{const_cast<T*>(_v.data()) + c * _r, _r}; }
    Block block(long r, long c, long h, long) { return Block{_v.data() + c * _r + r, h}; }
};

template<class T>
using VectorX = Matrix<T, Dynamic, 1>;

// ------------------------------------------------------------ CSR sparse matrix
template<class T, int Options, class I> class SparseMatrix;

template<class Sparse, int UpLo>
struct SelfAdjointView {
    const Sparse& m;
    template<class T>
    Matrix<T, Dynamic, 1> operator*(const Matrix<T, Dynamic, 1>& x) const { return m.symmetric_upper_product(x); }
};

template<class T, int Options, class I>
class SparseMatrix {
    static_assert(Options == RowMajor, "the oracle shim only provides row-major storage");
    long _rows = 0, _cols = 0;
    std::vector<I> _outer{I{0}};
    std::vector<I> _inner;
    std::vector<T> _values;

public:
    using Scalar = T;
    using StorageIndex = I;

    struct Storage {
        SparseMatrix& m;
        void resize(size_t n) { m._inner.resize(n); m._values.resize(n); }
    };

    SparseMatrix() = default;
    SparseMatrix(long r, long c) { resize(r, c); }
    template<int UpLo>
    explicit SparseMatrix(const SelfAdjointView<SparseMatrix, UpLo>& view) { *this = view.m.full_from_upper(); }

    void resize(long r, long c) {
        _rows = r; _cols = c;
        _outer.assign(size_t(r) + 1, I{0});
        _inner.clear(); _values.clear();
    }
    long rows() const noexcept { return _rows; }
    long cols() const noexcept { return _cols; }
    long outerSize() const noexcept { return _rows; }
    long nonZeros() const noexcept { return long(_outer[size_t(_rows)]); }
    I* outerIndexPtr() noexcept { return _outer.data(); }
    const I* outerIndexPtr() const noexcept { return _outer.data(); }
    I* innerIndexPtr() noexcept { return _inner.data(); }
    const I* innerIndexPtr() const noexcept { return _inner.data(); }
    T* valuePtr() noexcept { return _values.data(); }
    const T* valuePtr() const noexcept { return _values.data(); }
    Storage data() { return Storage{*this}; }
    void makeCompressed() {}

    long find(long r, long c) const {
        const I* b = _inner.data() + _outer[size_t(r)];
        const I* e = _inner.data() + _outer[size_t(r) + 1];
        const I* it = std::lower_bound(b, e, I(c));
        return (it != e && *it == I(c)) ? long(it - _inner.data()) : -1;
    }
    T coeff(long r, long c) const { const long k = find(r, c); return k < 0 ? T{0} : _values[size_t(k)]; }
    // Eigen inserts a missing entry; rows here are kept sorted, so the entry
    // goes at its ordered place (slow, only used outside hot loops).
    T& coeffRef(long r, long c) {
        long k = find(r, c);
        if (k >= 0) return _values[size_t(k)];
        const I* b = _inner.data() + _outer[size_t(r)];
        const I* e = _inner.data() + _outer[size_t(r) + 1];
        k = long(std::lower_bound(b, e, I(c)) - _inner.data());
        _inner.insert(_inner.begin() + k, I(c));
        _values.insert(_values.begin() + k, T{0});
        for (size_t i = size_t(r) + 1; i < _outer.size(); ++i) ++_outer[i];
        return _values[size_t(k)];
    }

    class InnerIterator {
        SparseMatrix& _m; long _k, _end, _row;
    public:
        InnerIterator(const SparseMatrix& m, long row)
            : _m{const_cast<SparseMatrix&>(m)}, _k{long(m._outer[size_t(row)])},
              _end{long(m._outer[size_t(row) + 1])}, _row{row} {}
        explicit operator bool() const noexcept { return _k < _end; }
        InnerIterator& operator++() { ++_k; return *this; }
        long index() const { return long(_m._inner[size_t(_k)]); }
        long col() const { return index(); }
        long row() const { return _row; }
        T value() const { return _m._values[size_t(_k)]; }
        T& valueRef() { return _m._values[size_t(_k)]; }
    };

    SparseMatrix& operator*=(const T s) { for (T& v : _values) v *= s; return *this; }

    // Union-pattern sum, rows kept sorted.
    SparseMatrix& operator+=(const SparseMatrix& o) {
        std::vector<I> outer(size_t(_rows) + 1, I{0}), inner;
        std::vector<T> values;
        inner.reserve(_inner.size()); values.reserve(_values.size());
        for (long r = 0; r < _rows; ++r) {
            long a = long(_outer[size_t(r)]), ae = long(_outer[size_t(r) + 1]);
            long b = long(o._outer[size_t(r)]), be = long(o._outer[size_t(r) + 1]);
            while (a < ae || b < be) {
                if (b >= be || (a < ae && _inner[size_t(a)] < o._inner[size_t(b)])) {
                    inner.push_back(_inner[size_t(a)]); values.push_back(_values[size_t(a)]); ++a;
                } else if (a >= ae || o._inner[size_t(b)] < _inner[size_t(a)]) {
                    inner.push_back(o._inner[size_t(b)]); values.push_back(o._values[size_t(b)]); ++b;
                } else {
                    inner.push_back(_inner[size_t(a)]); values.push_back(_values[size_t(a)] + o._values[size_t(b)]); ++a; ++b;
                }
            }
            outer[size_t(r) + 1] = I(inner.size());
        }
        _outer.swap(outer); _inner.swap(inner); _values.swap(values);
        return *this;
    }

    template<int UpLo>
    SelfAdjointView<SparseMatrix, UpLo> selfadjointView() const {
        static_assert(UpLo == Upper, "only upper storage is used by the reference path");
        return SelfAdjointView<SparseMatrix, UpLo>{*this};
    }

    Matrix<T, Dynamic, 1> operator*(const Matrix<T, Dynamic, 1>& x) const {
        Matrix<T, Dynamic, 1> y(_rows);
        for (long r = 0; r < _rows; ++r) {
            T s = T{0};
            for (I k = _outer[size_t(r)]; k < _outer[size_t(r) + 1]; ++k) s += _values[size_t(k)] * x[long(_inner[size_t(k)])];
            y[r] = s;
        }
        return y;
    }

    Matrix<T, Dynamic, 1> symmetric_upper_product(const Matrix<T, Dynamic, 1>& x) const {
        Matrix<T, Dynamic, 1> y(_rows);
        for (long r = 0; r < _rows; ++r)
            for (I k = _outer[size_t(r)]; k < _outer[size_t(r) + 1]; ++k) {
                const long c = long(_inner[size_t(k)]);
                if (c < r) continue;
                y[r] += _values[size_t(k)] * x[c];
                if (c != r) y[c] += _values[size_t(k)] * x[r];
            }
        return y;
    }

    SparseMatrix full_from_upper() const {
        std::vector<std::vector<std::pair<I, T>>> rows(static_cast<size_t>(_rows));
        for (long r = 0; r < _rows; ++r)
            for (I k = _outer[size_t(r)]; k < _outer[size_t(r) + 1]; ++k) {
                const long c = long(_inner[size_t(k)]);
                if (c < r) continue;
                rows[size_t(r)].push_back({I(c), _values[size_t(k)]});
                if (c != r && c < _rows) rows[size_t(c)].push_back({I(r), _values[size_t(k)]});
            }
        SparseMatrix f(_rows, _cols);
        for (long r = 0; r < _rows; ++r) {
            auto& row = rows[size_t(r)];
            std::sort(row.begin(), row.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
            for (const auto& [c, v] : row) { f._inner.push_back(c); f._values.push_back(v); }
            f._outer[size_t(r) + 1] = I(f._inner.size());
        }
        return f;
    }
};

template<class I> struct NaturalOrdering {};

// ------------------------------------------------------------ preconditioners
class IdentityPreconditioner {
public:
    IdentityPreconditioner() = default;
    template<class M> explicit IdentityPreconditioner(const M&) {}
    template<class M> IdentityPreconditioner& analyzePattern(const M&) { return *this; }
    template<class M> IdentityPreconditioner& factorize(const M&) { return *this; }
    template<class M> IdentityPreconditioner& compute(const M&) { return *this; }
    template<class V> V solve(const V& b) const { return b; }
    ComputationInfo info() { return Success; }
};

template<class T>
class DiagonalPreconditioner {
    Matrix<T, Dynamic, 1> _inv;
public:
    DiagonalPreconditioner() = default;
    template<class M> explicit DiagonalPreconditioner(const M& m) { compute(m); }
    template<class M> DiagonalPreconditioner& analyzePattern(const M&) { return *this; }
    template<class M> DiagonalPreconditioner& factorize(const M& m) { return compute(m); }
    template<class M> DiagonalPreconditioner& compute(const M& m) {
        _inv = Matrix<T, Dynamic, 1>::Constant(m.cols(), T{1});
        for (long r = 0; r < m.rows(); ++r) {
            const T d = m.coeff(r, r);
            if (d != T{0}) _inv[r] = T{1} / d;
        }
        return *this;
    }
    Matrix<T, Dynamic, 1> solve(const Matrix<T, Dynamic, 1>& b) const {
        Matrix<T, Dynamic, 1> x = b;
        for (long i = 0; i < x.size(); ++i) x[i] *= _inv[i];
        return x;
    }
    ComputationInfo info() { return Success; }
};

// Lin-More incomplete Cholesky with limited memory (p = 0 extra entries per
// column), natural ordering, on the symmetric matrix given by its upper part.
template<class T, int UpLo, class Ordering>
class IncompleteCholesky {
    long _n = 0;
    std::vector<long> _colptr;    // CSC of L (diagonal first in each column)
    std::vector<long> _rowidx;
    std::vector<T> _val;
    std::vector<T> _scale;
    ComputationInfo _info = InvalidInput;
    int _attempts = 0;
    T _shift = T{0};

public:
    static constexpr T initial_shift = T(1e-3);
    IncompleteCholesky() = default;
    template<class M> explicit IncompleteCholesky(const M& m) { compute(m); }
    template<class M> IncompleteCholesky& analyzePattern(const M&) { return *this; }
    template<class M> IncompleteCholesky& factorize(const M& m) { return compute(m); }
    ComputationInfo info() { return _info; }
    int attempts() const noexcept { return _attempts; }
    T shift() const noexcept { return _shift; }
    const std::vector<long>& colptr() const noexcept { return _colptr; }
    const std::vector<long>& rowidx() const noexcept { return _rowidx; }
    const std::vector<T>& values() const noexcept { return _val; }
    const std::vector<T>& scale() const noexcept { return _scale; }

    template<class M>
    IncompleteCholesky& compute(const M& m) {
        static_assert(UpLo == Upper, "only the upper-storage form is used by the reference path");
        _n = m.rows();
        const long n = _n;
        // Lower CSC of the symmetric matrix == row-major upper part.
        std::vector<long> cp(size_t(n) + 1, 0), ri;
        std::vector<T> va;
        for (long j = 0; j < n; ++j) {
            bool has_diag = false;
            for (auto k = m.outerIndexPtr()[j]; k < m.outerIndexPtr()[j + 1]; ++k) {
                const long c = long(m.innerIndexPtr()[k]);
                if (c < j) continue;
                if (c == j) has_diag = true;
                ri.push_back(c); va.push_back(m.valuePtr()[k]);
            }
            if (!has_diag) { _info = InvalidInput; return *this; }
            cp[size_t(j) + 1] = long(ri.size());
        }
        // l2 column norms of the full symmetric matrix -> D^{-1/2}.
        _scale.assign(size_t(n), T{0});
        for (long j = 0; j < n; ++j)
            for (long k = cp[size_t(j)]; k < cp[size_t(j) + 1]; ++k) {
                const long i = ri[size_t(k)];
                _scale[size_t(j)] += va[size_t(k)] * va[size_t(k)];
                if (i != j) _scale[size_t(i)] += va[size_t(k)] * va[size_t(k)];
            }
        for (T& s : _scale) {
            const T root = std::sqrt(std::sqrt(s));
            s = root > std::numeric_limits<T>::min() ? T{1} / root : T{1};
        }
        T mindiag = std::numeric_limits<T>::max();
        for (long j = 0; j < n; ++j) {
            for (long k = cp[size_t(j)]; k < cp[size_t(j) + 1]; ++k)
                va[size_t(k)] *= _scale[size_t(ri[size_t(k)])] * _scale[size_t(j)];
            mindiag = std::min(mindiag, va[size_t(cp[size_t(j)])]);
        }
        T shift = mindiag <= T{0} ? initial_shift - mindiag : T{0};
        _info = NumericalIssue;
        for (_attempts = 1; _attempts <= 10; ++_attempts) {
            if (factor_once(cp, ri, va, shift)) { _info = Success; _shift = shift; return *this; }
            shift = std::max(initial_shift, T{2} * shift);
        }
        return *this;
    }

    Matrix<T, Dynamic, 1> solve(const Matrix<T, Dynamic, 1>& b) const {
        Matrix<T, Dynamic, 1> x(_n);
        for (long i = 0; i < _n; ++i) x[i] = _scale[size_t(i)] * b[i];
        // L y = x (column oriented)
        for (long j = 0; j < _n; ++j) {
            const long k0 = _colptr[size_t(j)];
            x[j] /= _val[size_t(k0)];
            for (long k = k0 + 1; k < _colptr[size_t(j) + 1]; ++k) x[_rowidx[size_t(k)]] -= _val[size_t(k)] * x[j];
        }
        // L^T z = y
        for (long j = _n - 1; j >= 0; --j) {
            const long k0 = _colptr[size_t(j)];
            T s = x[j];
            for (long k = k0 + 1; k < _colptr[size_t(j) + 1]; ++k) s -= _val[size_t(k)] * x[_rowidx[size_t(k)]];
            x[j] = s / _val[size_t(k0)];
        }
        for (long i = 0; i < _n; ++i) x[i] *= _scale[size_t(i)];
        return x;
    }

private:
    bool factor_once(const std::vector<long>& cp, const std::vector<long>& ri, const std::vector<T>& va0, const T shift) {
        const long n = _n;
        std::vector<T> diag(static_cast<size_t>(n));
        for (long j = 0; j < n; ++j) diag[size_t(j)] = va0[size_t(cp[size_t(j)])] + shift;
        // Factor columns stored as (row, value) lists; `upd[j]` lists the
        // earlier columns k whose retained entries include row j.
        std::vector<std::vector<std::pair<long, T>>> cols(static_cast<size_t>(n));
        std::vector<std::vector<long>> upd(static_cast<size_t>(n));
        std::vector<T> acc(static_cast<size_t>(n), T{0});
        std::vector<char> mark(static_cast<size_t>(n), 0);
        std::vector<long> touched;
        for (long j = 0; j < n; ++j) {
            touched.clear();
            for (long k = cp[size_t(j)] + 1; k < cp[size_t(j) + 1]; ++k) {
                const long i = ri[size_t(k)];
                acc[size_t(i)] = va0[size_t(k)]; mark[size_t(i)] = 1; touched.push_back(i);
            }
            const long keep = cp[size_t(j) + 1] - cp[size_t(j)] - 1;
            for (const long k : upd[size_t(j)]) {
                T ljk = T{0};
                for (const auto& [i, v] : cols[size_t(k)]) if (i == j) { ljk = v; break; }
                for (const auto& [i, v] : cols[size_t(k)]) {
                    if (i <= j) continue;
                    if (!mark[size_t(i)]) { mark[size_t(i)] = 1; acc[size_t(i)] = T{0}; touched.push_back(i); }
                    acc[size_t(i)] -= v * ljk;
                }
            }
            const T d = diag[size_t(j)];
            if (!(d > T{0})) {
                for (const long i : touched) mark[size_t(i)] = 0;
                return false;
            }
            const T rd = std::sqrt(d);
            std::vector<std::pair<long, T>> entries;
            entries.reserve(touched.size());
            for (const long i : touched) {
                const T v = acc[size_t(i)] / rd;
                diag[size_t(i)] -= v * v;
                entries.push_back({i, v});
                mark[size_t(i)] = 0;
            }
            if (long(entries.size()) > keep) {
                std::stable_sort(entries.begin(), entries.end(), [](const auto& a, const auto& b) {
                    return std::abs(a.second) > std::abs(b.second) ||
                           (std::abs(a.second) == std::abs(b.second) && a.first < b.first);
                });
                entries.resize(size_t(keep));
            }
            std::sort(entries.begin(), entries.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
            for (const auto& [i, v] : entries) upd[size_t(i)].push_back(j);
            cols[size_t(j)] = std::move(entries);
            cols[size_t(j)].insert(cols[size_t(j)].begin(), {j, rd});
        }
        _colptr.assign(size_t(n) + 1, 0); _rowidx.clear(); _val.clear();
        for (long j = 0; j < n; ++j) {
            for (const auto& [i, v] : cols[size_t(j)]) { _rowidx.push_back(i); _val.push_back(v); }
            _colptr[size_t(j) + 1] = long(_rowidx.size());
        }
        return true;
    }
};

// Band LDL^T of the symmetric matrix given by its upper part, natural order.
template<class Sparse, int UpLo = Lower, class Ordering = NaturalOrdering<int>>
class SimplicialCholesky {
    using T = typename Sparse::Scalar;
    long _n = 0, _bw = 0;
    std::vector<T> _band;   // row-major band: _band[i * (bw+1) + (j - i)], j >= i
    std::vector<T> _d;
    ComputationInfo _info = InvalidInput;

public:
    SimplicialCholesky() = default;
    explicit SimplicialCholesky(const Sparse& m) { compute(m); }
    SimplicialCholesky& compute(const Sparse& m) {
        _n = m.rows(); _bw = 0;
        for (long r = 0; r < _n; ++r)
            for (auto k = m.outerIndexPtr()[r]; k < m.outerIndexPtr()[r + 1]; ++k)
                _bw = std::max(_bw, long(m.innerIndexPtr()[k]) - r);
        const long w = _bw + 1;
        _band.assign(size_t(_n * w), T{0});
        for (long r = 0; r < _n; ++r)
            for (auto k = m.outerIndexPtr()[r]; k < m.outerIndexPtr()[r + 1]; ++k) {
                const long c = long(m.innerIndexPtr()[k]);
                if (c >= r) _band[size_t(r * w + (c - r))] = m.valuePtr()[k];
            }
        // U^T D U with unit upper U stored in the band (overwrites A).
        _d.assign(size_t(_n), T{0});
        for (long i = 0; i < _n; ++i) {
            T di = _band[size_t(i * w)];
            for (long k = std::max(0L, i - _bw); k < i; ++k) {
                const T uki = _band[size_t(k * w + (i - k))];
                di -= uki * uki * _d[size_t(k)];
            }
            if (di == T{0}) { _info = NumericalIssue; return *this; }
            _d[size_t(i)] = di;
            for (long j = i + 1; j <= std::min(_n - 1, i + _bw); ++j) {
                T s = _band[size_t(i * w + (j - i))];
                for (long k = std::max(0L, j - _bw); k < i; ++k)
                    s -= _band[size_t(k * w + (i - k))] * _band[size_t(k * w + (j - k))] * _d[size_t(k)];
                _band[size_t(i * w + (j - i))] = s / di;
            }
        }
        _info = Success;
        return *this;
    }
    ComputationInfo info() const { return _info; }
    Matrix<T, Dynamic, 1> solve(const Matrix<T, Dynamic, 1>& b) const {
        const long w = _bw + 1;
        Matrix<T, Dynamic, 1> x = b;
        for (long i = 0; i < _n; ++i)            // U^T y = b
            for (long k = std::max(0L, i - _bw); k < i; ++k) x[i] -= _band[size_t(k * w + (i - k))] * x[k];
        for (long i = 0; i < _n; ++i) x[i] /= _d[size_t(i)];
        for (long i = _n - 1; i >= 0; --i)       // U x = z
            for (long j = i + 1; j <= std::min(_n - 1, i + _bw); ++j) x[i] -= _band[size_t(i * w + (j - i))] * x[j];
        return x;
    }
};

// Eigen::ConjugateGradient<SparseMatrix, Upper> as documented: the matrix is
// the self-adjoint view of its upper triangle, default DiagonalPreconditioner
// (inverse of the diagonal, 1 where it is zero), tolerance = machine epsilon on
// |r| / |b|, at most 2 n iterations, x0 = 0.  The iteration is the textbook
// preconditioned conjugate gradient (Hestenes & Stiefel 1952).
template<class Sparse, int UpLo = Lower>
struct ConjugateGradient {
    using T = typename Sparse::Scalar;
    using V = Matrix<T, Dynamic, 1>;
    const Sparse* _a = nullptr;
    V _inv;
    T _tol = std::numeric_limits<T>::epsilon();
    long _max = -1;
    mutable long _iters = 0;
    mutable T _error = T{0};
    explicit ConjugateGradient(const Sparse& a) : _a{&a}, _inv(a.rows()) {
        static_assert(UpLo == Upper, "only the upper-storage form is used by the reference path");
        const auto* op = a.outerIndexPtr();
        const auto* ip = a.innerIndexPtr();
        const T* vp = a.valuePtr();
        for (long r = 0; r < a.rows(); ++r) {
            T d = T{0};
            for (auto k = op[r]; k < op[r + 1]; ++k)
                if (long(ip[k]) == r) d = vp[k];
            _inv[r] = d != T{0} ? T{1} / d : T{1};
        }
    }
    void setTolerance(T t) { _tol = t; }
    void setMaxIterations(long m) { _max = m; }
    long iterations() const { return _iters; }
    T error() const { return _error; }
    ComputationInfo info() const { return Success; }
    V solve(const V& b) const { return solveWithGuess(b, V::Zero(b.size())); }
    V solveWithGuess(const V& b, const V& x0) const {
        const Sparse& A = *_a;
        const long n = b.size();
        const long maxit = _max < 0 ? 2 * n : _max;
        V x = x0;
        V r = b - A.template selfadjointView<Upper>() * x;
        const T bb = b.squaredNorm();
        _iters = 0;
        if (bb == T{0}) { _error = T{0}; return x; }
        const T threshold = std::max(_tol * _tol * bb, std::numeric_limits<T>::min());
        V z(n), p(n);
        for (long k = 0; k < n; ++k) p[k] = _inv[k] * r[k];
        T rz = r.dot(p);
        T rr = r.squaredNorm();
        long i = 0;
        while (rr > threshold && i < maxit) {
            const V q = A.template selfadjointView<Upper>() * p;
            const T alpha = rz / p.dot(q);
            for (long k = 0; k < n; ++k) { x[k] += alpha * p[k]; r[k] -= alpha * q[k]; }
            rr = r.squaredNorm();
            ++i;
            if (rr < threshold) break;
            for (long k = 0; k < n; ++k) z[k] = _inv[k] * r[k];
            const T rz_new = r.dot(z);
            const T beta = rz_new / rz;
            rz = rz_new;
            for (long k = 0; k < n; ++k) p[k] = z[k] + beta * p[k];
        }
        _iters = i;
        _error = std::sqrt(rr / bb);
        return x;
    }
};
// Eigen::BiCGSTAB<SparseMatrix> as documented: default DiagonalPreconditioner
// (inverse of the diagonal, 1 where it is zero), tolerance = machine epsilon
// on |r| / |b|, at most 2 n iterations.  The iteration is the right-
// preconditioned BiCGSTAB of van der Vorst (1992); when the shadow residual
// becomes orthogonal to the residual it restarts from the true residual.
template<class Sparse>
struct BiCGSTAB {
    using T = typename Sparse::Scalar;
    using V = Matrix<T, Dynamic, 1>;
    const Sparse* _a = nullptr;
    V _inv;
    T _tol = std::numeric_limits<T>::epsilon();
    long _max = -1;
    mutable long _iters = 0;
    mutable T _error = T{0};
    explicit BiCGSTAB(const Sparse& a) : _a{&a}, _inv(a.rows()) {
        const auto* op = a.outerIndexPtr();
        const auto* ip = a.innerIndexPtr();
        const T* vp = a.valuePtr();
        for (long r = 0; r < a.rows(); ++r) {
            T d = T{0};
            for (auto k = op[r]; k < op[r + 1]; ++k)
                if (long(ip[k]) == r) d = vp[k];
            _inv[r] = d != T{0} ? T{1} / d : T{1};
        }
    }
    void setTolerance(T t) { _tol = t; }
    void setMaxIterations(long m) { _max = m; }
    long iterations() const { return _iters; }
    T error() const { return _error; }
    ComputationInfo info() const { return Success; }
    V precond(const V& v) const {
        V z(v.size());
        for (long i = 0; i < v.size(); ++i) z[i] = _inv[i] * v[i];
        return z;
    }
    V solve(const V& b) const { return solveWithGuess(b, V::Zero(b.size())); }
    V solveWithGuess(const V& b, const V& x0) const {
        const Sparse& A = *_a;
        const long n = b.size();
        const long maxit = _max < 0 ? 2 * n : _max;
        V x = x0;
        V r = b - A * x;
        V r0 = r;
        const T bb = b.squaredNorm();
        const T tol2 = _tol * _tol * bb;
        T rho = 1, alpha = 1, w = 1;
        V v = V::Zero(n), p = V::Zero(n);
        long i = 0;
        T r0n2 = r0.squaredNorm();
        while (r.squaredNorm() > tol2 && i < maxit) {
            const T rho_old = rho;
            rho = r0.dot(r);
            if (std::abs(rho) < std::numeric_limits<T>::epsilon() * std::numeric_limits<T>::epsilon() * r0n2) {
                r = b - A * x;     // restart
                r0 = r;
                rho = r0n2 = r.squaredNorm();
                v = V::Zero(n);
                p = V::Zero(n);
                alpha = w = T{1};
                if (r0n2 == T{0}) break;
            }
            const T beta = (rho / rho_old) * (alpha / w);
            for (long k = 0; k < n; ++k) p[k] = r[k] + beta * (p[k] - w * v[k]);
            const V y = precond(p);
            v = A * y;
            alpha = rho / r0.dot(v);
            V s = r;
            for (long k = 0; k < n; ++k) s[k] -= alpha * v[k];
            const V z = precond(s);
            const V t = A * z;
            const T tt = t.squaredNorm();
            w = tt > T{0} ? t.dot(s) / tt : T{0};
            for (long k = 0; k < n; ++k) {
                x[k] += alpha * y[k] + w * z[k];
                r[k] = s[k] - w * t[k];
            }
            ++i;
        }
        _iters = i;
        _error = bb > T{0} ? std::sqrt(r.squaredNorm() / bb) : T{0};
        return x;
    }
};
template<class Sparse, class Ordering>
struct SparseLU {
    template<class... A> explicit SparseLU(const A&...) {
        throw std::logic_error{"Eigen::SparseLU is not part of the oracle build"};
    }
    template<class V> V solve(const V& b) const { return b; }
};

} // namespace Eigen
