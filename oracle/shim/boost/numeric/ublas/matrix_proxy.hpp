// Stand-in for boost/numeric/ublas/matrix_proxy.hpp (oracle build only; not Boost code).
#include "matrix.hpp"
#include "vector.hpp"
