// tt_matrix.h -- a small column-major matrix type that provides the subset of
// the Eigen 3 API used by maleadt/tracetransform's c++/ and openmp/ sources
// (Matrix, Block, comma initialiser, sum, cwiseSqrt, tail, transpose,
// products, JacobiSVD).  Written from Eigen's documented interface only; it is
// test infrastructure for building the reference sources as a CPU oracle.
//
// Evaluation orders that matter for float results:
//   - sum() adds coefficients in storage order (Eigen vectorises this;
//     that order is not reproduced);
//   - a product coefficient is a(i,0)*b(0,j) + a(i,1)*b(1,j) + ..., each
//     product rounded, summed left to right (Eigen's coefficient-based lazy
//     product for small fixed sizes without FMA).
#ifndef TT_SHIM_EIGEN_MATRIX_H
#define TT_SHIM_EIGEN_MATRIX_H

#include <algorithm>
#include <cassert>
#include <cerrno>
#include <climits>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iosfwd>
#include <sstream>
#include <string>
#include <limits>
#include <type_traits>
#include <vector>

namespace Eigen {

typedef std::ptrdiff_t Index;
const int Dynamic = -1;

enum DecompositionOptions {
    ComputeFullU = 0x04,
    ComputeThinU = 0x08,
    ComputeFullV = 0x10,
    ComputeThinV = 0x20
};
enum QRPreconditioners {
    NoQRPreconditioner,
    HouseholderQRPreconditioner,
    ColPivHouseholderQRPreconditioner,
    FullPivHouseholderQRPreconditioner
};

template <typename T, int R, int C> class Matrix;

// A rectangular view into a column-major matrix.
template <typename T> class Block {
  public:
    Block(T *base, Index ld, Index rows, Index cols)
        : p_(base), ld_(ld), rows_(rows), cols_(cols) {}
    Index rows() const { return rows_; }
    Index cols() const { return cols_; }
    Index size() const { return rows_ * cols_; }
    T &operator()(Index i, Index j) const { return p_[i + j * ld_]; }
    T &operator()(Index i) const { return at(i); }
    T &operator[](Index i) const { return at(i); }
    T sum() const {
        T s = 0;
        for (Index j = 0; j < cols_; j++)
            for (Index i = 0; i < rows_; i++)
                s += (*this)(i, j);
        return s;
    }
    template <int R, int C> Block &operator=(const Matrix<T, R, C> &m) {
        assert(m.rows() == rows_ && m.cols() == cols_);
        for (Index j = 0; j < cols_; j++)
            for (Index i = 0; i < rows_; i++)
                (*this)(i, j) = m(i, j);
        return *this;
    }

  private:
    T &at(Index i) const {
        return rows_ == 1 ? p_[i * ld_] : p_[i];
    }
    T *p_;
    Index ld_, rows_, cols_;
};

template <typename M> class CommaInitializer {
  public:
    CommaInitializer(M &m, typename M::Scalar first) : m_(m), pos_(0) {
        put(first);
    }
    template <typename S> CommaInitializer &operator,(const S &v) {
        put(static_cast<typename M::Scalar>(v));
        return *this;
    }

  private:
    void put(typename M::Scalar v) {
        // Eigen fills row by row.
        Index r = pos_ / m_.cols(), c = pos_ % m_.cols();
        m_(r, c) = v;
        pos_++;
    }
    M &m_;
    Index pos_;
};

template <typename T, int R, int C> class Matrix {
  public:
    typedef T Scalar;
    static const bool kFixed = (R != Dynamic && C != Dynamic);

    Matrix() : rows_(R == Dynamic ? 0 : R), cols_(C == Dynamic ? 0 : C) {
        d_.resize(rows_ * cols_);
    }
    // Vector of n coefficients (uninitialised in Eigen; zero here).
    template <typename I, typename std::enable_if<std::is_integral<I>::value,
                                                  int>::type = 0>
    explicit Matrix(I n) {
        static_assert(R == 1 || C == 1, "size constructor needs a vector");
        rows_ = (C == 1) ? (Index)n : 1;
        cols_ = (C == 1) ? 1 : (Index)n;
        d_.assign(rows_ * cols_, T(0));
    }
    // Two arguments: coefficients for fixed 2-vectors, sizes otherwise.
    template <typename A, typename B> Matrix(const A &a, const B &b) {
        if (kFixed) {
            rows_ = R;
            cols_ = C;
            d_.resize(R * C);
            assert(R * C == 2);
            d_[0] = static_cast<T>(a);
            d_[1] = static_cast<T>(b);
        } else {
            rows_ = (Index)a;
            cols_ = (Index)b;
            d_.assign(rows_ * cols_, T(0));
        }
    }
    Matrix(const Block<T> &b) : rows_(b.rows()), cols_(b.cols()) {
        d_.resize(rows_ * cols_);
        for (Index j = 0; j < cols_; j++)
            for (Index i = 0; i < rows_; i++)
                d_[i + j * rows_] = b(i, j);
    }
    Matrix(const Block<const T> &b) : rows_(b.rows()), cols_(b.cols()) {
        d_.resize(rows_ * cols_);
        for (Index j = 0; j < cols_; j++)
            for (Index i = 0; i < rows_; i++)
                d_[i + j * rows_] = b(i, j);
    }

    static Matrix Zero(Index rows, Index cols) {
        Matrix m;
        m.rows_ = rows;
        m.cols_ = cols;
        m.d_.assign(rows * cols, T(0));
        return m;
    }
    static Matrix Zero(Index n) {
        Matrix m(n);
        return m;
    }

    Index rows() const { return rows_; }
    Index cols() const { return cols_; }
    Index size() const { return rows_ * cols_; }
    T *data() { return d_.data(); }
    const T *data() const { return d_.data(); }

    T &operator()(Index i, Index j) { return d_[i + j * rows_]; }
    const T &operator()(Index i, Index j) const { return d_[i + j * rows_]; }
    T &operator()(Index i) { return d_[i]; }
    const T &operator()(Index i) const { return d_[i]; }
    T &operator[](Index i) { return d_[i]; }
    const T &operator[](Index i) const { return d_[i]; }
    T x() const { return d_[0]; }
    T y() const { return d_[1]; }

    Block<T> col(Index j) { return Block<T>(&d_[j * rows_], rows_, rows_, 1); }
    Block<T> col(Index j) const {
        return Block<T>(const_cast<T *>(&d_[j * rows_]), rows_, rows_, 1);
    }
    Block<T> block(Index i, Index j, Index r, Index c) {
        return Block<T>(&d_[i + j * rows_], rows_, r, c);
    }
    Block<T> block(Index i, Index j, Index r, Index c) const {
        return Block<T>(const_cast<T *>(&d_[i + j * rows_]), rows_, r, c);
    }

    T sum() const {
        T s = 0;
        for (Index i = 0; i < size(); i++)
            s += d_[i];
        return s;
    }
    Matrix cwiseSqrt() const {
        Matrix m(*this);
        for (Index i = 0; i < size(); i++)
            m.d_[i] = std::sqrt(d_[i]);
        return m;
    }
    Matrix tail(Index n) const {
        Matrix m(n);
        for (Index i = 0; i < n; i++)
            m.d_[i] = d_[size() - n + i];
        return m;
    }
    Matrix<T, C, R> transpose() const {
        Matrix<T, C, R> m = Matrix<T, C, R>::Zero(cols_, rows_);
        for (Index j = 0; j < cols_; j++)
            for (Index i = 0; i < rows_; i++)
                m(j, i) = (*this)(i, j);
        return m;
    }

    template <typename S> CommaInitializer<Matrix> operator<<(const S &v) {
        return CommaInitializer<Matrix>(*this, static_cast<T>(v));
    }

    Matrix &operator+=(const Matrix &o) {
        for (Index i = 0; i < size(); i++)
            d_[i] += o.d_[i];
        return *this;
    }
    Matrix &operator-=(const Matrix &o) {
        for (Index i = 0; i < size(); i++)
            d_[i] -= o.d_[i];
        return *this;
    }
    template <int R2, int C2> Matrix &operator*=(const Matrix<T, R2, C2> &o) {
        *this = product(*this, o);
        return *this;
    }
    Matrix operator-(const Matrix &o) const {
        Matrix m(*this);
        m -= o;
        return m;
    }
    Matrix operator+(const Matrix &o) const {
        Matrix m(*this);
        m += o;
        return m;
    }

    template <int R1, int C1, int R2, int C2>
    static Matrix product(const Matrix<T, R1, C1> &a,
                          const Matrix<T, R2, C2> &b) {
        Matrix m = Zero(a.rows(), b.cols());
        for (Index j = 0; j < b.cols(); j++) {
            for (Index i = 0; i < a.rows(); i++) {
                T acc = a(i, 0) * b(0, j);
                for (Index k = 1; k < a.cols(); k++)
                    acc += a(i, k) * b(k, j);
                m(i, j) = acc;
            }
        }
        return m;
    }

  private:
    template <typename, int, int> friend class Matrix;
    Index rows_, cols_;
    std::vector<T> d_;
};

template <typename T, int R1, int C1, int R2, int C2>
Matrix<T, Dynamic, Dynamic> operator*(const Matrix<T, R1, C1> &a,
                                      const Matrix<T, R2, C2> &b) {
    return Matrix<T, Dynamic, Dynamic>::product(a, b);
}
template <typename T, int R2, int C2>
Matrix<T, Dynamic, Dynamic> operator*(const Block<T> &a,
                                      const Matrix<T, R2, C2> &b) {
    Matrix<T, Dynamic, Dynamic> am(a);
    return Matrix<T, Dynamic, Dynamic>::product(am, b);
}

// Map over external column-major storage.  The stand-in copies on
// construction (Eigen's Map aliases the storage); enough for code that reads
// through a Map or converts it to a Matrix, as the engine's reference-side
// bindings do.
template <typename MatrixType> class Map : public MatrixType {
  public:
    typedef typename MatrixType::Scalar Scalar;
    Map(const Scalar *p, Index rows, Index cols) : MatrixType(rows, cols) {
        for (Index i = 0; i < rows * cols; i++)
            this->data()[i] = p[i];
    }
    Map(const Scalar *p, Index n) : MatrixType(n) {
        for (Index i = 0; i < n; i++)
            this->data()[i] = p[i];
    }
};

typedef Matrix<float, Dynamic, Dynamic> MatrixXf;
typedef Matrix<int, Dynamic, Dynamic> MatrixXi;
typedef Matrix<double, Dynamic, Dynamic> MatrixXd;
typedef Matrix<float, Dynamic, 1> VectorXf;
typedef Matrix<int, Dynamic, 1> VectorXi;
typedef Matrix<double, Dynamic, 1> VectorXd;
typedef Matrix<float, 2, 2> Matrix2f;
typedef Matrix<float, 1, 2> RowVector2f;
typedef Matrix<float, 2, 1> Vector2f;

// Singular value decomposition of a tall matrix by one-sided Jacobi
// rotations in double precision (Eigen runs two-sided Jacobi in the matrix's
// own scalar type after a QR preconditioner).  matrixU() is rows x rows with
// the leading min(rows, cols) columns set; matrixV() is cols x cols.
template <typename MatrixType, int QRPreconditioner = 0> class JacobiSVD {
  public:
    typedef typename MatrixType::Scalar Scalar;
    JacobiSVD(const MatrixType &a, unsigned int /*options*/) {
        const Index m = a.rows(), n = a.cols();
        assert(m >= n);
        std::vector<double> w(m * n), v(n * n, 0.0);
        for (Index j = 0; j < n; j++)
            for (Index i = 0; i < m; i++)
                w[i + j * m] = a(i, j);
        for (Index i = 0; i < n; i++)
            v[i + i * n] = 1.0;
        for (int sweep = 0; sweep < 80; sweep++) {
            bool rotated = false;
            for (Index p = 0; p + 1 < n; p++) {
                for (Index q = p + 1; q < n; q++) {
                    double *cp = &w[p * m], *cq = &w[q * m];
                    double a2 = 0, b2 = 0, g = 0;
                    for (Index i = 0; i < m; i++) {
                        a2 += cp[i] * cp[i];
                        b2 += cq[i] * cq[i];
                        g += cp[i] * cq[i];
                    }
                    if (g == 0 || std::fabs(g) <= 1e-15 * std::sqrt(a2 * b2))
                        continue;
                    rotated = true;
                    double zeta = (b2 - a2) / (2 * g);
                    double t = (zeta >= 0 ? 1.0 : -1.0) /
                               (std::fabs(zeta) + std::sqrt(1 + zeta * zeta));
                    double c = 1 / std::sqrt(1 + t * t), s = c * t;
                    for (Index i = 0; i < m; i++) {
                        double x = cp[i], y = cq[i];
                        cp[i] = c * x - s * y;
                        cq[i] = s * x + c * y;
                    }
                    double *vp = &v[p * n], *vq = &v[q * n];
                    for (Index i = 0; i < n; i++) {
                        double x = vp[i], y = vq[i];
                        vp[i] = c * x - s * y;
                        vq[i] = s * x + c * y;
                    }
                }
            }
            if (!rotated)
                break;
        }
        u_ = MatrixType::Zero(m, m);
        v_ = MatrixType::Zero(n, n);
        for (Index k = 0; k < n; k++) {
            double nrm = 0;
            for (Index i = 0; i < m; i++)
                nrm += w[i + k * m] * w[i + k * m];
            nrm = std::sqrt(nrm);
            for (Index i = 0; i < m; i++)
                u_(i, k) = (Scalar)(nrm > 0 ? w[i + k * m] / nrm : 0.0);
            for (Index i = 0; i < n; i++)
                v_(i, k) = (Scalar)v[i + k * n];
        }
        // keep the double-precision factors for an accurate U V^T
        wd_.swap(w);
        vd_.swap(v);
        m_ = m;
        n_ = n;
    }
    const MatrixType &matrixU() const { return u_; }
    const MatrixType &matrixV() const { return v_; }

  private:
    MatrixType u_, v_;
    std::vector<double> wd_, vd_;
    Index m_, n_;
};

} // namespace Eigen

#endif
