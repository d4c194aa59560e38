// Stand-in for boost/math/constants/constants.hpp: only pi<T>() is needed
// (oracle build only; not Boost code).
#ifndef ORACLE_SHIM_MATH_CONSTANTS_HPP
#define ORACLE_SHIM_MATH_CONSTANTS_HPP
namespace boost { namespace math { namespace constants {
template <class T> inline T pi() { return static_cast<T>(3.141592653589793238462643383279502884L); }
}}}
#endif
