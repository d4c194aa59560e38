// kinds.h -- measurement kinds and their row layouts (host and device).
//
// Raw rows per station follow the reference implementations:
//   scalar   1 row  g_z                           (Gravity/ScalarOMPGravityImp.h)
//   tensor   9 rows Uxx Uxy Uxz Uyx Uyy Uyz Uzx Uzy Uzz, C order
//                                                 (Gravity/TensorOMPGravityImp.cpp:165-177)
//   magnetic 3 rows Bx By Bz                      (Magnetics/OMPMagneticSusceptibilityImp.cpp:187-190)
//   joint   10 rows g_z followed by the 9 tensor rows (one pass serving a
//           joint gravity + FTG inversion, which the reference runs as two
//           calculators over the same mesh)
#pragma once
#include "prism_math.cuh"

namespace j3g {

enum Kind : int { KIND_SCALAR = 1, KIND_TENSOR = 2, KIND_MAGNETIC = 3, KIND_JOINT = 4 };
enum Transform : int { TR_NONE = 0, TR_FTG_INVARIANT = 1, TR_TOTAL_FIELD = 2, TR_TFA = 3 };

constexpr int kTensorMask = (1 << NC_XX) | (1 << NC_YY) | (1 << NC_ZZ) | (1 << NC_XY) |
                            (1 << NC_XZ) | (1 << NC_YZ);

template <int KIND> struct KindTraits;
template <> struct KindTraits<KIND_SCALAR> {
  static constexpr int mask = 1 << NC_GZ;
  static constexpr int ncomp = 1;
  static constexpr int raw = 1;
};
template <> struct KindTraits<KIND_TENSOR> {
  static constexpr int mask = kTensorMask;
  static constexpr int ncomp = 6;
  static constexpr int raw = 9;
};
template <> struct KindTraits<KIND_MAGNETIC> {
  static constexpr int mask = kTensorMask;
  static constexpr int ncomp = 6;
  static constexpr int raw = 3;
};
template <> struct KindTraits<KIND_JOINT> {
  static constexpr int mask = (1 << NC_GZ) | kTensorMask;
  static constexpr int ncomp = 7;
  static constexpr int raw = 10;
};

__host__ __device__ inline int kind_mask(int kind) {
  return kind == KIND_SCALAR ? (1 << NC_GZ)
         : kind == KIND_JOINT ? ((1 << NC_GZ) | kTensorMask)
                              : kTensorMask;
}
__host__ __device__ inline int kind_raw(int kind) {
  return kind == KIND_SCALAR ? 1 : kind == KIND_TENSOR ? 9 : kind == KIND_MAGNETIC ? 3 : 10;
}
__host__ __device__ inline int kind_ncomp(int kind) {
  return kind == KIND_SCALAR ? 1 : kind == KIND_JOINT ? 7 : 6;
}
// Slot s of a kind's compact component list -> node component id.
__host__ __device__ inline int slot_comp(int kind, int s) {
  return (kind == KIND_SCALAR || kind == KIND_JOINT) ? s : s + 1;
}

// The magnetic projection B_k = F/(4 pi G) sum_j U_kj b_j with
// b = (cos I cos D, cos I sin D, sin I)
// (Magnetics/OMPMagneticSusceptibilityImp.cpp:116-118, 160-170).
struct MagField {
  double bx, by, bz;  // direction cosines of the inducing field
  double fs;          // field strength (nT)
  double factor;      // 1 / (4 pi G)
};

// Raw row values of one cell (or one station's gridded sums) from the node
// component values u[NC_*].  Operation order of the magnetic projection is
// the reference's: ((Uk0*bx + Uk1*by) + Uk2*bz) * fs * factor.
__host__ __device__ inline void raw_from_comps(int kind, const double *u, const MagField &m,
                                               double *raw) {
  if (kind == KIND_SCALAR) {
    raw[0] = u[NC_GZ];
    return;
  }
  double *t = raw;
  if (kind == KIND_JOINT) {
    raw[0] = u[NC_GZ];
    t = raw + 1;
  }
  if (kind == KIND_MAGNETIC) {
    raw[0] = mul(mul(add(add(mul(u[NC_XX], m.bx), mul(u[NC_XY], m.by)), mul(u[NC_XZ], m.bz)), m.fs), m.factor);
    raw[1] = mul(mul(add(add(mul(u[NC_XY], m.bx), mul(u[NC_YY], m.by)), mul(u[NC_YZ], m.bz)), m.fs), m.factor);
    raw[2] = mul(mul(add(add(mul(u[NC_XZ], m.bx), mul(u[NC_YZ], m.by)), mul(u[NC_ZZ], m.bz)), m.fs), m.factor);
    return;
  }
  t[0] = u[NC_XX];
  t[1] = u[NC_XY];
  t[2] = u[NC_XZ];
  t[3] = u[NC_XY];
  t[4] = u[NC_YY];
  t[5] = u[NC_YZ];
  t[6] = u[NC_XZ];
  t[7] = u[NC_YZ];
  t[8] = u[NC_ZZ];
}

// Adjoint of raw_from_comps: weights on the raw rows -> weights on the node
// components (duplicated tensor rows add up).
__host__ __device__ inline void comps_from_raw_weights(int kind, const double *w,
                                                       const MagField &m, double *u) {
  for (int c = 0; c < NC_COUNT; ++c) u[c] = 0.0;
  if (kind == KIND_SCALAR) {
    u[NC_GZ] = w[0];
    return;
  }
  const double *t = w;
  if (kind == KIND_JOINT) {
    u[NC_GZ] = w[0];
    t = w + 1;
  }
  if (kind == KIND_MAGNETIC) {
    const double f = m.fs * m.factor;
    u[NC_XX] = w[0] * m.bx * f;
    u[NC_XY] = (w[0] * m.by + w[1] * m.bx) * f;
    u[NC_XZ] = (w[0] * m.bz + w[2] * m.bx) * f;
    u[NC_YY] = w[1] * m.by * f;
    u[NC_YZ] = (w[1] * m.bz + w[2] * m.by) * f;
    u[NC_ZZ] = w[2] * m.bz * f;
    return;
  }
  u[NC_XX] = t[0];
  u[NC_XY] = t[1] + t[3];
  u[NC_XZ] = t[2] + t[6];
  u[NC_YY] = t[4];
  u[NC_YZ] = t[5] + t[7];
  u[NC_ZZ] = t[8];
}

}  // namespace j3g
