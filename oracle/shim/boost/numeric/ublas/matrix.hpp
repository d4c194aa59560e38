// Stand-in for the part of boost/numeric/ublas/matrix.hpp that the jif3D box
// terms need: a dense row-major matrix with (i, j) access and data().
// Written for the oracle build only; it is not Boost code.
#ifndef ORACLE_SHIM_UBLAS_MATRIX_HPP
#define ORACLE_SHIM_UBLAS_MATRIX_HPP
#include <cstddef>
#include <vector>
namespace boost { namespace numeric { namespace ublas {
struct row_major {};
struct column_major {};
template <class T, class L = row_major> class matrix {
 public:
  typedef T value_type;
  matrix() : r_(0), c_(0) {}
  matrix(std::size_t r, std::size_t c) : r_(r), c_(c), d_(r * c) {}
  matrix(std::size_t r, std::size_t c, const T &v) : r_(r), c_(c), d_(r * c, v) {}
  T &operator()(std::size_t i, std::size_t j) { return d_[i * c_ + j]; }
  const T &operator()(std::size_t i, std::size_t j) const { return d_[i * c_ + j]; }
  std::vector<T> &data() { return d_; }
  const std::vector<T> &data() const { return d_; }
  std::size_t size1() const { return r_; }
  std::size_t size2() const { return c_; }
 private:
  std::size_t r_, c_;
  std::vector<T> d_;
};
template <class T, class L = row_major> class mapped_matrix {};
template <class T, class L = row_major> class compressed_matrix {};
}}}
#endif
