/*
 * Minimal stand-ins for the deal.II classes that the reference's cell kernels
 * (femgl/src/cell_mat_vec/*.cc) use, FullMatrix<double> and Vector<double>, and that
 * its PDW initial-state function (femgl/inc/pdw_config.h) uses: Point<3>, Function<3>
 * and the Assert macro.  TEST INFRASTRUCTURE ONLY: this header lets the oracle
 * build compile the reference's own kernel sources unmodified, so that their
 * outputs can pin the CPU restatement and the CUDA path.  Nothing in the
 * product links against it.
 *
 * Semantics follow the public deal.II documentation of these members:
 *   mmult(C, B, adding)  : C  = A * B      (C += A * B when adding)
 *   Tmmult(C, B, adding) : C  = A^T * B
 *   mTmult(C, B, adding) : C  = A * B^T
 *   add(a, A)            : this += a * A
 *   add(a, A, b, B)      : this += a * A + b * B
 *   trace()              : sum of the diagonal
 *   operator=(0.0)       : set every entry to zero
 *   Vector::operator*    : dot product
 */
#ifndef GLORACLE_DEALII_SHIM_H
#define GLORACLE_DEALII_SHIM_H

#include <cstddef>
#include <vector>

namespace dealii
{
  template <typename number>
  class FullMatrix
  {
  public:
    using size_type = std::size_t;

    FullMatrix(const size_type n = 0) : rows_(n), cols_(n), a_(n * n, number(0)) {}
    FullMatrix(const size_type m, const size_type n) : rows_(m), cols_(n), a_(m * n, number(0)) {}

    FullMatrix &operator=(const number d)
    {
      for (auto &x : a_) x = d;
      return *this;
    }

    size_type m() const { return rows_; }
    size_type n() const { return cols_; }

    number &operator()(const size_type i, const size_type j) { return a_[i * cols_ + j]; }
    const number &operator()(const size_type i, const size_type j) const { return a_[i * cols_ + j]; }
    void set(const size_type i, const size_type j, const number v) { a_[i * cols_ + j] = v; }

    void mmult(FullMatrix &C, const FullMatrix &B, const bool adding = false) const
    {
      for (size_type i = 0; i < rows_; ++i)
        for (size_type j = 0; j < B.cols_; ++j)
          {
            number s = 0;
            for (size_type k = 0; k < cols_; ++k) s += (*this)(i, k) * B(k, j);
            C(i, j) = adding ? C(i, j) + s : s;
          }
    }

    void Tmmult(FullMatrix &C, const FullMatrix &B, const bool adding = false) const
    {
      for (size_type i = 0; i < cols_; ++i)
        for (size_type j = 0; j < B.cols_; ++j)
          {
            number s = 0;
            for (size_type k = 0; k < rows_; ++k) s += (*this)(k, i) * B(k, j);
            C(i, j) = adding ? C(i, j) + s : s;
          }
    }

    void mTmult(FullMatrix &C, const FullMatrix &B, const bool adding = false) const
    {
      for (size_type i = 0; i < rows_; ++i)
        for (size_type j = 0; j < B.rows_; ++j)
          {
            number s = 0;
            for (size_type k = 0; k < cols_; ++k) s += (*this)(i, k) * B(j, k);
            C(i, j) = adding ? C(i, j) + s : s;
          }
    }

    void add(const number a, const FullMatrix &A)
    {
      for (size_type k = 0; k < a_.size(); ++k) a_[k] += a * A.a_[k];
    }

    void add(const number a, const FullMatrix &A, const number b, const FullMatrix &B)
    {
      for (size_type k = 0; k < a_.size(); ++k) a_[k] += a * A.a_[k] + b * B.a_[k];
    }

    number trace() const
    {
      number s = 0;
      for (size_type i = 0; i < rows_ && i < cols_; ++i) s += (*this)(i, i);
      return s;
    }

  private:
    size_type rows_, cols_;
    std::vector<number> a_;
  };

  template <typename number>
  class Vector
  {
  public:
    using size_type = std::size_t;
    Vector(const size_type n = 0) : v_(n, number(0)) {}
    Vector &operator=(const number d)
    {
      for (auto &x : v_) x = d;
      return *this;
    }
    number &operator()(const size_type i) { return v_[i]; }
    const number &operator()(const size_type i) const { return v_[i]; }
    number &operator[](const size_type i) { return v_[i]; }
    const number &operator[](const size_type i) const { return v_[i]; }
    Vector &operator+=(const Vector &o)
    {
      for (size_type i = 0; i < v_.size(); ++i) v_[i] += o.v_[i];
      return *this;
    }
    number operator*(const Vector &o) const
    {
      number s = 0;
      for (size_type i = 0; i < v_.size(); ++i) s += v_[i] * o.v_[i];
      return s;
    }
    size_type size() const { return v_.size(); }

  private:
    std::vector<number> v_;
  };

  // Point<dim>: coordinates read with operator()(i)
  template <int dim>
  class Point
  {
  public:
    Point() : c_{} {}
    Point(double x, double y, double z) : c_{x, y, z} {}
    double operator()(const unsigned int i) const { return c_[i]; }

  private:
    double c_[3];
  };

  // Function<dim>: a vector-valued function of n_components components
  template <int dim>
  class Function
  {
  public:
    explicit Function(const unsigned int n_components = 1) : n_components(n_components) {}
    virtual ~Function() = default;
    virtual void vector_value(const Point<dim> &, Vector<double> &) const {}
    virtual void vector_value_list(const std::vector<Point<dim>> &, std::vector<Vector<double>> &) const {}
    const unsigned int n_components;
  };

  struct ExcDimensionMismatch
  {
    ExcDimensionMismatch(std::size_t, std::size_t) {}
  };
} // namespace dealii

#ifndef Assert
#define Assert(cond, exc) ((void)0)
#endif

#endif
