// Stand-in for boost/numeric/ublas/vector.hpp (oracle build only; not Boost code).
#ifndef ORACLE_SHIM_UBLAS_VECTOR_HPP
#define ORACLE_SHIM_UBLAS_VECTOR_HPP
#include <cstddef>
#include <vector>
namespace boost { namespace numeric { namespace ublas {
template <class T> class vector {
 public:
  vector() {}
  explicit vector(std::size_t n) : d_(n) {}
  vector(std::size_t n, const T &v) : d_(n, v) {}
  T &operator()(std::size_t i) { return d_[i]; }
  const T &operator()(std::size_t i) const { return d_[i]; }
  T &operator[](std::size_t i) { return d_[i]; }
  std::size_t size() const { return d_.size(); }
 private:
  std::vector<T> d_;
};
}}}
#endif
