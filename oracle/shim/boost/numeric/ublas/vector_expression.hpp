// Stand-in for boost/numeric/ublas/vector_expression.hpp (oracle build only; not Boost code).
#include "matrix.hpp"
#include "vector.hpp"
