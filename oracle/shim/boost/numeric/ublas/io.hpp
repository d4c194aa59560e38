// Stand-in for boost/numeric/ublas/io.hpp (oracle build only; not Boost code).
#include "matrix.hpp"
#include "vector.hpp"
