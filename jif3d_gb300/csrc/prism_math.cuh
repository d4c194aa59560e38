// prism_math.cuh -- FP64 device arithmetic of the rectangular-prism terms.
//
// The geometric terms follow Li & Chouteau (1998) exactly as the reference
// evaluates them (Gravity/BasicGravElements.cpp):
//   g_z corner     x ln(y+r) + y ln(x+r) + z atan2(z r, x y), r >= eps      (:26-37)
//   diagonal FTG   atan2(a b, c r)                                           (:43-47)
//   off-diagonal   ln(max(v + r, eps))                                       (:53-59)
// A corner term depends only on the offset station - corner, so on a mesh
// whose corner coordinates are the running sums of the cell sizes every
// corner term is a function of one mesh NODE.  The kernels evaluate each node
// once per station ("node terms") and form the prism values from the eight
// nodes of a cell, instead of eight corner evaluations per cell.
//
// Products and sums that feed the corner terms use explicit round-to-nearest
// intrinsics so that no multiply-add is contracted: the operation sequence is
// the reference's.  The logarithms and arctangents are flog / fatan2
// (fp64_math.cuh): within about one unit in the last place, like the C
// library's, with a third of the FP64 operations of CUDA's log / atan2.
#pragma once
#include <cfloat>
#include <cstdint>

#include "fp64_math.cuh"

namespace j3g {

constexpr double kGravConst = 6.67428e-11;  // Gravity/BasicGravElements.h:22
constexpr double kEps = DBL_EPSILON;         // std::numeric_limits<double>::epsilon()

// Node-term components.  A kind needs a subset of them (see component masks).
enum NodeComp : int {
  NC_GZ = 0,  // g_z corner term
  NC_XX = 1,  // atan2(dy dz, dx r)   Uxx corner term
  NC_YY = 2,  // atan2(dx dz, dy r)   Uyy corner term
  NC_ZZ = 3,  // atan2(dx dy, dz r)   Uzz corner term
  NC_XY = 4,  // ln(max(dz + r, eps)) Uxy corner term
  NC_XZ = 5,  // ln(max(dy + r, eps)) Uxz corner term
  NC_YZ = 6,  // ln(max(dx + r, eps)) Uyz corner term
  NC_COUNT = 7
};

// Scale of each component when eight node terms are combined with the signs
// (-1)^(number of shifted coordinates):  g_z and the off-diagonal terms carry
// +G, the diagonal terms -G (the reference returns -sum*G, sum*G, -sum*G with
// sum = sum of (-1)^(shifts+1) terms).
__host__ __device__ constexpr double comp_scale(int c) {
  return (c >= NC_XX && c <= NC_ZZ) ? -kGravConst : kGravConst;
}

// Round-to-nearest products and sums that the compiler may not fuse.  Host
// code is built with -ffp-contract=off, so plain operators are the same there.
#ifdef __CUDA_ARCH__
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
#else
inline double mul(double a, double b) { return a * b; }
inline double add(double a, double b) { return a + b; }
inline double sub(double a, double b) { return a - b; }
#endif

// v < kEps on the integer pipe (the FP64 pipe is this kernel family's
// bound): negative values (sign bit set, -0 and -inf included) are below, a
// NaN of either sign is not, and non-negative doubles order as their bits.
__device__ __forceinline__ bool lt_eps(double v) {
  const long long b = __double_as_longlong(v);
  constexpr long long kEpsBits = 0x3cb0000000000000ll;  // 2^-52
  return b < 0 ? (b & 0x7fffffffffffffffll) <= 0x7ff0000000000000ll : b < kEpsBits;
}

// Clamp from below that keeps NaN, like std::max(v, eps).
__device__ __forceinline__ double clamp_eps(double v) { return lt_eps(v) ? kEps : v; }

// All node terms needed by `mask` (bit c set -> component c) for one offset
// (dx, dy, dz) = station - node.  One square root serves every component.
template <int MASK>
__device__ __forceinline__ void node_terms(double dx, double dy, double dz, double *out) {
  // fused: the node terms need r to FP64 accuracy, not the reference's
  // rounding (the eight-corner path keeps that)
  const double s2 = __fma_rn(dx, dx, __fma_rn(dy, dy, mul(dz, dz)));
  const double r = sqrt(s2);
  constexpr bool need_gz = MASK & (1 << NC_GZ);
  constexpr bool need_off = MASK & ((1 << NC_XY) | (1 << NC_XZ) | (1 << NC_YZ));
  double lx = 0.0, ly = 0.0;
  if (need_gz || need_off) {
    // ln(dx + r) and ln(dy + r) are shared by g_z and the Uyz / Uxz terms when
    // r >= eps (then g_z's clamped r equals the raw r).
    const double rg = clamp_eps(r);
    lx = flog(add(dx, rg));
    ly = flog(add(dy, rg));
    if (need_gz) {
      double a;
      if ((MASK & (1 << NC_ZZ)) && !lt_eps(r)) {
        // g_z's atan2(dz r, dx dy) and Uzz's atan2(dx dy, dz r) share their ratio
        double zz;
        fatan2_pair(mul(dz, rg), mul(dx, dy), a, zz);
        out[NC_ZZ] = zz;
      } else {
        a = fatan2(mul(dz, rg), mul(dx, dy));
        if (MASK & (1 << NC_ZZ)) out[NC_ZZ] = fatan2(mul(dx, dy), mul(dz, r));
      }
      out[NC_GZ] = __fma_rn(dx, ly, __fma_rn(dy, lx, mul(dz, a)));
    }
    if (need_off) {
      const bool shared = !lt_eps(r);
      const double ax = add(dx, r), ay = add(dy, r), az = add(dz, r);
      const double log_eps = fp64tab::kLogDblEps;  // log(DBL_EPSILON)
      if (MASK & (1 << NC_YZ))
        out[NC_YZ] = lt_eps(ax) ? log_eps : (shared ? lx : flog(ax));
      if (MASK & (1 << NC_XZ))
        out[NC_XZ] = lt_eps(ay) ? log_eps : (shared ? ly : flog(ay));
      if (MASK & (1 << NC_XY))
        out[NC_XY] = lt_eps(az) ? log_eps : flog(az);
    }
  }
  if (MASK & (1 << NC_XX)) out[NC_XX] = fatan2(mul(dy, dz), mul(dx, r));
  if (MASK & (1 << NC_YY)) out[NC_YY] = fatan2(mul(dx, dz), mul(dy, r));
  constexpr bool zz_done = (MASK & (1 << NC_GZ)) != 0;  // computed with g_z above
  if ((MASK & (1 << NC_ZZ)) && !zz_done) out[NC_ZZ] = fatan2(mul(dx, dy), mul(dz, r));
}

// Corner order of each component's eight-term sum, as bit triples
// (bit 2 = x shifted, bit 1 = y shifted, bit 0 = z shifted).  The reference
// evaluates Uyy, Uzz, Uxz and Uyz through argument permutations of the Uxx and
// Uxy routines (BasicGravElements.cpp:223-241), which permutes the order.
// Positions 0 / 1-3 / 4-6 / 7 are the zero / one / two / three-shift corners.
__host__ __device__ constexpr uint32_t comp_order(int c) {
  // packed 8 x 3 bits, position p in bits [3p, 3p+3)
  return c == NC_YY   ? (0u | 2u << 3 | 4u << 6 | 1u << 9 | 6u << 12 | 3u << 15 | 5u << 18 | 7u << 21)
         : c == NC_ZZ ? (0u | 1u << 3 | 4u << 6 | 2u << 9 | 5u << 12 | 3u << 15 | 6u << 18 | 7u << 21)
         : c == NC_XZ ? (0u | 4u << 3 | 1u << 6 | 2u << 9 | 5u << 12 | 6u << 15 | 3u << 18 | 7u << 21)
         : c == NC_YZ ? (0u | 1u << 3 | 2u << 6 | 4u << 9 | 3u << 12 | 5u << 15 | 6u << 18 | 7u << 21)
                      : (0u | 4u << 3 | 2u << 6 | 1u << 9 | 6u << 12 | 5u << 15 | 3u << 18 | 7u << 21);
}

// Prism value of component c from its eight node terms v[corner bits], summed
// in the reference's order and scaled as the reference scales it.
__device__ __forceinline__ double combine8(int c, const double *v) {
  const uint32_t ord = comp_order(c);
  double acc = -v[ord & 7u];
  acc = add(acc, v[(ord >> 3) & 7u]);
  acc = add(acc, v[(ord >> 6) & 7u]);
  acc = add(acc, v[(ord >> 9) & 7u]);
  acc = sub(acc, v[(ord >> 12) & 7u]);
  acc = sub(acc, v[(ord >> 15) & 7u]);
  acc = sub(acc, v[(ord >> 18) & 7u]);
  acc = add(acc, v[(ord >> 21) & 7u]);
  // g_z and off-diagonal: -acc*G ; diagonal: acc*G
  return (c >= NC_XX && c <= NC_ZZ) ? mul(acc, kGravConst) : mul(-acc, kGravConst);
}

// ---------------------------------------------------------------------------
// Reference-faithful single-prism terms (eight independent corner
// evaluations, each with the reference's own operand order).  Used for the
// background slabs and for meshes whose corners are not running sums.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double gz_corner(double x, double y, double z) {
  const double r = clamp_eps(sqrt(add(add(mul(x, x), mul(y, y)), mul(z, z))));
  double v = add(mul(x, flog(add(y, r))), mul(y, flog(add(x, r))));
  return add(v, mul(z, fatan2(mul(z, r), mul(x, y))));
}
__device__ __forceinline__ double diag_corner(double a, double b, double c) {
  return fatan2(mul(a, b), mul(c, sqrt(add(add(mul(a, a), mul(b, b)), mul(c, c)))));
}
__device__ __forceinline__ double offdiag_corner(double v, double x, double y, double z) {
  return flog(clamp_eps(add(v, sqrt(add(add(mul(x, x), mul(y, y)), mul(z, z))))));
}

// BasicGravElements.cpp:82-109
__device__ inline double grav_box(double mx, double my, double mz, double cx, double cy,
                                  double cz, double sx, double sy, double sz) {
  const double x0 = sub(mx, cx), x1 = sub(mx, add(cx, sx));
  const double y0 = sub(my, cy), y1 = sub(my, add(cy, sy));
  const double z0 = sub(mz, cz), z1 = sub(mz, add(cz, sz));
  double acc = -gz_corner(x0, y0, z0);
  acc = add(acc, gz_corner(x1, y0, z0));
  acc = add(acc, gz_corner(x0, y1, z0));
  acc = add(acc, gz_corner(x0, y0, z1));
  acc = sub(acc, gz_corner(x1, y1, z0));
  acc = sub(acc, gz_corner(x1, y0, z1));
  acc = sub(acc, gz_corner(x0, y1, z1));
  acc = add(acc, gz_corner(x1, y1, z1));
  return mul(-acc, kGravConst);
}
// BasicGravElements.cpp:125-152
__device__ inline double uxx_box(double mx, double my, double mz, double cx, double cy,
                                 double cz, double sx, double sy, double sz) {
  const double x0 = sub(mx, cx), x1 = sub(mx, add(cx, sx));
  const double y0 = sub(my, cy), y1 = sub(my, add(cy, sy));
  const double z0 = sub(mz, cz), z1 = sub(mz, add(cz, sz));
  double acc = -diag_corner(y0, z0, x0);
  acc = add(acc, diag_corner(y0, z0, x1));
  acc = add(acc, diag_corner(y1, z0, x0));
  acc = add(acc, diag_corner(y0, z1, x0));
  acc = sub(acc, diag_corner(y1, z0, x1));
  acc = sub(acc, diag_corner(y0, z1, x1));
  acc = sub(acc, diag_corner(y1, z1, x0));
  acc = add(acc, diag_corner(y1, z1, x1));
  return mul(acc, kGravConst);
}
// BasicGravElements.cpp:168-202
__device__ inline double uxy_box(double mx, double my, double mz, double cx, double cy,
                                 double cz, double sx, double sy, double sz) {
  const double x0 = sub(mx, cx), x1 = sub(mx, add(cx, sx));
  const double y0 = sub(my, cy), y1 = sub(my, add(cy, sy));
  const double z0 = sub(mz, cz), z1 = sub(mz, add(cz, sz));
  double acc = -offdiag_corner(z0, z0, y0, x0);
  acc = add(acc, offdiag_corner(z0, z0, y0, x1));
  acc = add(acc, offdiag_corner(z0, z0, y1, x0));
  acc = add(acc, offdiag_corner(z1, z1, y0, x0));
  acc = sub(acc, offdiag_corner(z0, z0, y1, x1));
  acc = sub(acc, offdiag_corner(z1, z1, y0, x1));
  acc = sub(acc, offdiag_corner(z1, z1, y1, x0));
  acc = add(acc, offdiag_corner(z1, z1, y1, x1));
  return mul(-acc, kGravConst);
}

// Unique prism components in node-component numbering (BasicGravElements.cpp:216-244).
__device__ inline void prism_components(int mask, double mx, double my, double mz, double cx,
                                        double cy, double cz, double sx, double sy, double sz,
                                        double *out) {
  if (mask & (1 << NC_GZ)) out[NC_GZ] = grav_box(mx, my, mz, cx, cy, cz, sx, sy, sz);
  if (mask & (1 << NC_XX)) out[NC_XX] = uxx_box(mx, my, mz, cx, cy, cz, sx, sy, sz);
  if (mask & (1 << NC_YY)) out[NC_YY] = uxx_box(my, mx, mz, cy, cx, cz, sy, sx, sz);
  if (mask & (1 << NC_ZZ)) out[NC_ZZ] = uxx_box(mz, mx, my, cz, cx, cy, sz, sx, sy);
  if (mask & (1 << NC_XY)) out[NC_XY] = uxy_box(mx, my, mz, cx, cy, cz, sx, sy, sz);
  if (mask & (1 << NC_XZ)) out[NC_XZ] = uxy_box(mx, mz, my, cx, cz, cy, sx, sz, sy);
  if (mask & (1 << NC_YZ)) out[NC_YZ] = uxy_box(mz, my, mx, cz, cy, cx, sz, sy, sx);
}

// Infinite-sheet terms, Gravity/BasicGravElements.h:51-75.
__device__ inline double inf_sheet(double mz, double top, double bottom) {
  const double pi = 3.141592653589793238462643383279502884;
  const double thick = sub(bottom, top);
  if ((mz <= top) || (mz >= bottom)) {
    const double sgn = (sub(top, mz) >= 0) ? 1.0 : -1.0;
    return mul(mul(mul(mul(2.0, pi), kGravConst), thick), sgn);
  }
  return mul(mul(mul(2.0, pi), kGravConst), sub(thick, mul(2.0, sub(mz, top))));
}
__device__ inline double uzz_inf_sheet(double mz, double top, double bottom) {
  const double pi = 3.141592653589793238462643383279502884;
  if ((mz <= top) || (mz >= bottom)) return 0.0;
  return mul(mul(4.0, pi), kGravConst);
}

}  // namespace j3g
