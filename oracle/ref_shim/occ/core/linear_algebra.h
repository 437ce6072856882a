// Minimal stand-in for the one Eigen type that the reference's Lebedev table
// source needs (a dynamic-row, 4-column, row-major double matrix), so that the
// reference source compiles here without Eigen.  Only used to build the
// checker library under oracle/_ref; never shipped with the product.
#pragma once
#include <cstddef>
#include <vector>
namespace Eigen {
enum { Dynamic = -1, RowMajor = 1 };
template <typename T, int R, int C, int O> class Matrix {
public:
  Matrix(long rows, long cols) : r_(rows), c_(cols), d_(rows * cols) {}
  T *data() { return d_.data(); }
  const T *data() const { return d_.data(); }
  T &operator()(long i, long j) { return d_[i * c_ + j]; }
  long rows() const { return r_; }
  long cols() const { return c_; }
private:
  long r_, c_;
  std::vector<T> d_;
};
} // namespace Eigen
