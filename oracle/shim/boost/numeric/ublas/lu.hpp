// Stand-in for boost/numeric/ublas/lu.hpp (oracle build only; not Boost code).
#include "matrix.hpp"
#include "vector.hpp"
