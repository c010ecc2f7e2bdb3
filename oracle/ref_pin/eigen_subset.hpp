// A small stand-in for the parts of Eigen's dense module that Thea's spatial-query headers use. Values are evaluated
// eagerly; every coefficient is computed with the operation order Eigen uses for small fixed-size, unvectorised
// expressions: coefficient-wise operations per coefficient, and sums (dot, squaredNorm, sum, products) as Eigen's
// unrolled reduction, which splits the range in halves: (e0 + (e1 + e2)) for three terms.
#pragma once

#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstddef>
#include <initializer_list>
#include <limits>
#include <ostream>
#include <type_traits>
#include <vector>

namespace Eigen {

typedef std::ptrdiff_t Index;
const int Dynamic = -1;
enum { ColMajor = 0, RowMajor = 0x1, AutoAlign = 0, DontAlign = 0x2 };
enum { Unaligned = 0, Aligned8 = 8, Aligned16 = 16, Aligned32 = 32, Aligned64 = 64, Aligned128 = 128, Aligned = 16 };
enum { RowMajorBit = 0x1 };

template <int O, int I> class Stride {
 public:
  Stride() {}
  Stride(Index, Index) {}
};
template <int I> class InnerStride : public Stride<0, I> {};
template <int O> class OuterStride : public Stride<O, 0> {};

namespace internal {
// Eigen's unrolled reduction: halves of the range combined with f
template <class S, class F> S redux(S const * v, Index start, Index len, F f) {
  if (len == 1) return v[start];
  Index h = len / 2;
  return f(redux(v, start, h, f), redux(v, start + h, len - h, f));
}
}  // namespace internal

template <typename Derived> class DenseBase {
 public:
  Derived & derived() { return *static_cast<Derived *>(this); }
  Derived const & derived() const { return *static_cast<Derived const *>(this); }
};
// Member functions reached through a MatrixBase<Derived> reference forward to the plain matrix
template <typename Derived> class MatrixBase : public DenseBase<Derived> {
 public:
  auto cwiseAbs() const { return this->derived().cwiseAbs(); }
  template <class I> auto maxCoeff(I * i) const { return this->derived().maxCoeff(i); }
  template <class I> auto minCoeff(I * i) const { return this->derived().minCoeff(i); }
  auto maxCoeff() const { return this->derived().maxCoeff(); }
  auto minCoeff() const { return this->derived().minCoeff(); }
  auto rows() const { return this->derived().rows(); }
  auto cols() const { return this->derived().cols(); }
  auto size() const { return this->derived().size(); }
  auto squaredNorm() const { return this->derived().squaredNorm(); }
  auto norm() const { return this->derived().norm(); }
  auto sum() const { return this->derived().sum(); }
};
template <typename Derived> class ArrayBase : public DenseBase<Derived> {};
template <typename Derived> class PlainObjectBase : public MatrixBase<Derived> {};

template <typename S, int R, int C, int O = 0, int MR = R, int MC = C> class Array;
template <typename S, int R, int C, int O = 0, int MR = R, int MC = C> class Matrix;

// Storage: fixed sizes in place, dynamic sizes in a vector (column-major order throughout)
template <typename S, int R, int C> struct Storage {
  S d[R * C > 0 ? R * C : 1];
  Index rows() const { return R; }
  Index cols() const { return C; }
  void resize(Index, Index) {}
  S * data() { return d; }
  S const * data() const { return d; }
};
template <typename S, int R, int C> struct DynStorage {
  std::vector<S> d;
  Index r = R > 0 ? R : 0, c = C > 0 ? C : 0;
  DynStorage() { d.resize((size_t)(r * c)); }
  Index rows() const { return r; }
  Index cols() const { return c; }
  void resize(Index rr, Index cc) {
    r = rr;
    c = cc;
    d.assign((size_t)(r * c), S());
  }
  S * data() { return d.data(); }
  S const * data() const { return d.data(); }
};

template <typename S, int R, int C, int O, int MR, int MC>
class Matrix : public PlainObjectBase<Matrix<S, R, C, O, MR, MC>> {
  typedef typename std::conditional<(R > 0 && C > 0), Storage<S, R, C>, DynStorage<S, R, C>>::type Store;
  Store st;

 public:
  typedef S Scalar;
  typedef S RealScalar;
  typedef S value_type;
  typedef Matrix PlainObject;
  enum { RowsAtCompileTime = R, ColsAtCompileTime = C, SizeAtCompileTime = (R > 0 && C > 0) ? R * C : Dynamic,
         IsRowMajor = (O & RowMajor) ? 1 : 0, Options = O, IsVectorAtCompileTime = (R == 1 || C == 1) ? 1 : 0,
         MaxRowsAtCompileTime = MR, MaxColsAtCompileTime = MC };

  Matrix() {}
  Matrix(Index r, Index c) { st.resize(r, c); }
  explicit Matrix(Index n) {
    if (R == 1) st.resize(1, n);
    else st.resize(n, 1);
  }
  Matrix(S x, S y) { (*this)[0] = x; (*this)[1] = y; }
  Matrix(S x, S y, S z) { (*this)[0] = x; (*this)[1] = y; (*this)[2] = z; }
  Matrix(S x, S y, S z, S w) { (*this)[0] = x; (*this)[1] = y; (*this)[2] = z; (*this)[3] = w; }
  // integer literals (Vector3(0, 0, 0) and the like)
  template <class A, class B, class = typename std::enable_if<std::is_arithmetic<A>::value && std::is_arithmetic<B>::value &&
                                                              !(std::is_same<A, S>::value && std::is_same<B, S>::value)>::type>
  Matrix(A x, B y) : Matrix((S)x, (S)y) {}
  template <class A, class B, class D,
            class = typename std::enable_if<std::is_arithmetic<A>::value && !(std::is_same<A, S>::value &&
                                                                               std::is_same<B, S>::value &&
                                                                               std::is_same<D, S>::value)>::type>
  Matrix(A x, B y, D z) : Matrix((S)x, (S)y, (S)z) {}
  template <int O2, int MR2, int MC2> Matrix(Matrix<S, R, C, O2, MR2, MC2> const & o) {
    st.resize(o.rows(), o.cols());
    for (Index i = 0; i < size(); ++i) data()[i] = o.data()[i];
  }
  template <int O2, int MR2, int MC2> Matrix & operator=(Matrix<S, R, C, O2, MR2, MC2> const & o) {
    st.resize(o.rows(), o.cols());
    for (Index i = 0; i < size(); ++i) data()[i] = o.data()[i];
    return *this;
  }

  Index rows() const { return st.rows(); }
  Index cols() const { return st.cols(); }
  Index size() const { return rows() * cols(); }
  S * data() { return st.data(); }
  S const * data() const { return st.data(); }
  void resize(Index r, Index c) { st.resize(r, c); }
  void resize(Index n) {
    if (R == 1) st.resize(1, n);
    else st.resize(n, 1);
  }

  S & operator[](Index i) { return data()[i]; }
  S const & operator[](Index i) const { return data()[i]; }
  S & operator()(Index i) { return data()[i]; }
  S const & operator()(Index i) const { return data()[i]; }
  S & operator()(Index i, Index j) { return data()[i + j * rows()]; }
  S const & operator()(Index i, Index j) const { return data()[i + j * rows()]; }
  S & coeffRef(Index i) { return data()[i]; }
  S coeff(Index i) const { return data()[i]; }
  S & coeffRef(Index i, Index j) { return (*this)(i, j); }
  S coeff(Index i, Index j) const { return (*this)(i, j); }
  S & x() { return data()[0]; }
  S & y() { return data()[1]; }
  S & z() { return data()[2]; }
  S & w() { return data()[3]; }
  S x() const { return data()[0]; }
  S y() const { return data()[1]; }
  S z() const { return data()[2]; }
  S w() const { return data()[3]; }

  template <class F> Matrix unary(F f) const {
    Matrix r(*this);
    for (Index i = 0; i < size(); ++i) r.data()[i] = f(data()[i]);
    return r;
  }
  template <class F> Matrix binary(Matrix const & o, F f) const {
    Matrix r(*this);
    for (Index i = 0; i < size(); ++i) r.data()[i] = f(data()[i], o.data()[i]);
    return r;
  }

  Matrix operator+(Matrix const & o) const { return binary(o, [](S a, S b) { return a + b; }); }
  Matrix operator-(Matrix const & o) const { return binary(o, [](S a, S b) { return a - b; }); }
  Matrix operator-() const { return unary([](S a) { return -a; }); }
  Matrix operator*(S s) const { return unary([s](S a) { return a * s; }); }
  Matrix operator/(S s) const { return unary([s](S a) { return a / s; }); }
  Matrix & operator+=(Matrix const & o) { return *this = *this + o; }
  Matrix & operator-=(Matrix const & o) { return *this = *this - o; }
  Matrix & operator*=(S s) { return *this = *this * s; }
  Matrix & operator/=(S s) { return *this = *this / s; }
  bool operator==(Matrix const & o) const {
    for (Index i = 0; i < size(); ++i)
      if (!(data()[i] == o.data()[i])) return false;
    return true;
  }
  bool operator!=(Matrix const & o) const { return !(*this == o); }

  S sum() const { return internal::redux(data(), 0, size(), [](S a, S b) { return a + b; }); }
  S prod() const { return internal::redux(data(), 0, size(), [](S a, S b) { return a * b; }); }
  S dot(Matrix const & o) const { return cwiseProduct(o).sum(); }
  S squaredNorm() const { return cwiseProduct(*this).sum(); }
  S norm() const { return std::sqrt(squaredNorm()); }
  Matrix normalized() const {
    S z = squaredNorm();
    return z > S(0) ? *this / std::sqrt(z) : *this;
  }
  void normalize() {
    S z = squaredNorm();
    if (z > S(0)) *this /= std::sqrt(z);
  }
  Matrix cross(Matrix const & b) const {
    Matrix const & a = *this;
    return Matrix(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
  }
  Matrix cwiseProduct(Matrix const & o) const { return binary(o, [](S a, S b) { return a * b; }); }
  Matrix cwiseQuotient(Matrix const & o) const { return binary(o, [](S a, S b) { return a / b; }); }
  Matrix cwiseMin(Matrix const & o) const { return binary(o, [](S a, S b) { return std::min(a, b); }); }
  Matrix cwiseMax(Matrix const & o) const { return binary(o, [](S a, S b) { return std::max(a, b); }); }
  Matrix cwiseMin(S s) const { return unary([s](S a) { return std::min(a, s); }); }
  Matrix cwiseMax(S s) const { return unary([s](S a) { return std::max(a, s); }); }
  Matrix cwiseAbs() const { return unary([](S a) { return std::abs(a); }); }
  Matrix cwiseInverse() const { return unary([](S a) { return S(1) / a; }); }
  Matrix cwiseSqrt() const { return unary([](S a) { return std::sqrt(a); }); }
  // minCoeff / maxCoeff: first index of the extremum (Eigen's visitors replace only on a strict comparison)
  S maxCoeff() const {
    S m = data()[0];
    for (Index i = 1; i < size(); ++i)
      if (data()[i] > m) m = data()[i];
    return m;
  }
  S minCoeff() const {
    S m = data()[0];
    for (Index i = 1; i < size(); ++i)
      if (data()[i] < m) m = data()[i];
    return m;
  }
  template <class I> S maxCoeff(I * idx) const {
    Index k = 0;
    for (Index i = 1; i < size(); ++i)
      if (data()[i] > data()[k]) k = i;
    if (idx) *idx = (I)k;
    return data()[k];
  }
  template <class I> S minCoeff(I * idx) const {
    Index k = 0;
    for (Index i = 1; i < size(); ++i)
      if (data()[i] < data()[k]) k = i;
    if (idx) *idx = (I)k;
    return data()[k];
  }
  bool hasNaN() const {
    for (Index i = 0; i < size(); ++i)
      if (data()[i] != data()[i]) return true;
    return false;
  }
  bool allFinite() const {
    for (Index i = 0; i < size(); ++i)
      if (!std::isfinite((double)data()[i])) return false;
    return true;
  }

  Matrix & setZero() { return fill(S(0)); }
  Matrix & setOnes() { return fill(S(1)); }
  Matrix & setConstant(S v) { return fill(v); }
  Matrix & fill(S v) {
    for (Index i = 0; i < size(); ++i) data()[i] = v;
    return *this;
  }
  Matrix & setIdentity() {
    for (Index i = 0; i < rows(); ++i)
      for (Index j = 0; j < cols(); ++j) (*this)(i, j) = i == j ? S(1) : S(0);
    return *this;
  }
  static Matrix Zero() { return Matrix().setZero(); }
  static Matrix Zero(Index n) { return Matrix(n).setZero(); }
  static Matrix Zero(Index r, Index c) { return Matrix(r, c).setZero(); }
  static Matrix Ones() { return Matrix().setOnes(); }
  static Matrix Constant(S v) { return Matrix().setConstant(v); }
  static Matrix Constant(Index n, S v) { return Matrix(n).setConstant(v); }
  static Matrix Identity() { return Matrix().setIdentity(); }
  static Matrix Identity(Index r, Index c) { return Matrix(r, c).setIdentity(); }
  static Matrix Unit(Index i) {
    Matrix m = Zero();
    m[i] = S(1);
    return m;
  }
  static Matrix UnitX() { return Unit(0); }
  static Matrix UnitY() { return Unit(1); }
  static Matrix UnitZ() { return Unit(2); }

  template <class U> Matrix<U, R, C, O, MR, MC> cast() const {
    Matrix<U, R, C, O, MR, MC> r(rows(), cols());
    for (Index i = 0; i < size(); ++i) r.data()[i] = (U)data()[i];
    return r;
  }
  Matrix<S, C, R, (O & DontAlign) | ((R == 1 && C != 1) ? 0 : 0), MC, MR> transpose() const {
    Matrix<S, C, R, (O & DontAlign), MC, MR> t(cols(), rows());
    for (Index i = 0; i < rows(); ++i)
      for (Index j = 0; j < cols(); ++j) t(j, i) = (*this)(i, j);
    return t;
  }
  Array<S, R, C, O, MR, MC> array() const;
  // 3 x 3: Eigen's cofactor inverse (cofactor(i, j) from the two other rows and columns, cyclically; det = column 0 of
  // the cofactors dotted with column 0; inverse(j, i) = cofactor(i, j) / det); other sizes by Gauss-Jordan elimination
  Matrix inverse() const {
    Matrix r(*this);
    Index n = rows();
    if (n == 3 && cols() == 3) {
      Matrix const & m = *this;
      S cof[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
          cof[i][j] = m(i1, j1) * m(i2, j2) - m(i1, j2) * m(i2, j1);
        }
      S det = cof[0][0] * m(0, 0) + (cof[1][0] * m(1, 0) + cof[2][0] * m(2, 0));
      S inv = S(1) / det;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r(j, i) = cof[i][j] * inv;
      return r;
    }
    Matrix a(*this);
    r.setIdentity();
    for (Index c = 0; c < n; ++c) {
      Index p = c;
      for (Index i = c + 1; i < n; ++i)
        if (std::abs(a(i, c)) > std::abs(a(p, c))) p = i;
      for (Index j = 0; j < n; ++j) {
        std::swap(a(c, j), a(p, j));
        std::swap(r(c, j), r(p, j));
      }
      S d = a(c, c);
      for (Index j = 0; j < n; ++j) {
        a(c, j) /= d;
        r(c, j) /= d;
      }
      for (Index i = 0; i < n; ++i)
        if (i != c) {
          S f = a(i, c);
          for (Index j = 0; j < n; ++j) {
            a(i, j) -= f * a(c, j);
            r(i, j) -= f * r(c, j);
          }
        }
    }
    return r;
  }
  S determinant() const {
    Matrix const & m = *this;
    if (rows() == 2) return m(0, 0) * m(1, 1) - m(0, 1) * m(1, 0);
    if (rows() == 3)
      return m(0, 0) * (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) - m(1, 0) * (m(0, 1) * m(2, 2) - m(0, 2) * m(2, 1)) +
             m(2, 0) * (m(0, 1) * m(1, 2) - m(0, 2) * m(1, 1));
    return S(0);
  }
  Matrix const & matrix() const { return *this; }
};

// Matrix products, coefficient (i, j) = the reduction over k of lhs(i, k) * rhs(k, j)
template <typename S, int R, int K, int C, int O1, int MR1, int MC1, int O2, int MR2, int MC2>
Matrix<S, R, C, O2, R, C> operator*(Matrix<S, R, K, O1, MR1, MC1> const & a, Matrix<S, K, C, O2, MR2, MC2> const & b) {
  Matrix<S, R, C, O2, R, C> r(a.rows(), b.cols());
  std::vector<S> t((size_t)a.cols());
  for (Index i = 0; i < a.rows(); ++i)
    for (Index j = 0; j < b.cols(); ++j) {
      for (Index k = 0; k < a.cols(); ++k) t[(size_t)k] = a(i, k) * b(k, j);
      r(i, j) = internal::redux(t.data(), 0, a.cols(), [](S x, S y) { return x + y; });
    }
  return r;
}

template <typename S, int R, int C, int O, int MR, int MC>
Matrix<S, R, C, O, MR, MC> operator*(S s, Matrix<S, R, C, O, MR, MC> const & m) {
  return m.unary([s](S a) { return s * a; });
}

template <typename S, int R, int C, int O, int MR, int MC>
std::ostream & operator<<(std::ostream & os, Matrix<S, R, C, O, MR, MC> const & m) {
  for (Index i = 0; i < m.size(); ++i) os << (i ? " " : "") << m.data()[i];
  return os;
}

// Coefficient-wise arrays (comparisons give boolean arrays)
template <typename S, int R, int C, int O, int MR, int MC>
class Array : public ArrayBase<Array<S, R, C, O, MR, MC>> {
 public:
  std::array<S, (R > 0 && C > 0) ? R * C : 4> d{};
  Index n = (R > 0 && C > 0) ? R * C : 0;
  Array() {}
  S & operator[](Index i) { return d[(size_t)i]; }
  S operator[](Index i) const { return d[(size_t)i]; }
  S & operator()(Index i) { return d[(size_t)i]; }
  S operator()(Index i) const { return d[(size_t)i]; }
  Index size() const { return n; }
  template <typename T2, int R2, int C2, int O2, int MR2, int MC2> Array(Array<T2, R2, C2, O2, MR2, MC2> const & o) {
    n = o.n;
    for (Index i = 0; i < n; ++i) d[(size_t)i] = (S)o[i];
  }
  template <class F> Array<bool, R, C, O, MR, MC> cmp(Array const & o, F f) const {
    Array<bool, R, C, O, MR, MC> r;
    r.n = n;
    for (Index i = 0; i < n; ++i) r[i] = f(d[(size_t)i], o.d[(size_t)i]);
    return r;
  }
  Array<bool, R, C, O, MR, MC> operator<=(Array const & o) const { return cmp(o, [](S a, S b) { return a <= b; }); }
  Array<bool, R, C, O, MR, MC> operator>=(Array const & o) const { return cmp(o, [](S a, S b) { return a >= b; }); }
  Array<bool, R, C, O, MR, MC> operator<(Array const & o) const { return cmp(o, [](S a, S b) { return a < b; }); }
  Array<bool, R, C, O, MR, MC> operator>(Array const & o) const { return cmp(o, [](S a, S b) { return a > b; }); }
  bool all() const {
    for (Index i = 0; i < n; ++i)
      if (!d[(size_t)i]) return false;
    return true;
  }
  bool any() const {
    for (Index i = 0; i < n; ++i)
      if (d[(size_t)i]) return true;
    return false;
  }
  Array abs() const {
    Array r(*this);
    for (Index i = 0; i < n; ++i) r[i] = std::abs(d[(size_t)i]);
    return r;
  }
};

template <typename S, int R, int C, int O, int MR, int MC>
Array<S, R, C, O, MR, MC> Matrix<S, R, C, O, MR, MC>::array() const {
  Array<S, R, C, O, MR, MC> a;
  a.n = size();
  for (Index i = 0; i < size(); ++i) a[i] = data()[i];
  return a;
}

template <typename P, int MO = Unaligned, typename St = Stride<0, 0>> class Map {};
template <typename T> class Quaternion {};
template <typename T> class AngleAxis {};
template <typename T> class Triplet {};
template <typename T, int O = 0, typename I = int> class SparseMatrix {};
template <typename T, int O = 0, typename I = int> class SparseVector {};
template <typename D> class SparseMatrixBase {};
template <typename M> class ColPivHouseholderQR {};

}  // namespace Eigen
