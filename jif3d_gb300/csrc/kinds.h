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
//   magnetic vertical gradient  1 row Bz(z) - Bz(z + 1 m)
//                                                 (Magnetics/OMPMagneticGradImp.cpp:13-106)
//   magnetisation  3 rows Bx By Bz of three magnetisation blocks Mx, My, Mz
//                  (3 ngrid parameters, no background)
//                                                 (Magnetics/OMPMagnetizationImp.cpp:25-117)
//
// The node kernels accumulate per station a kind's "virtual components": a
// node component (comp), the model block it multiplies (block: 0, or the
// magnetisation component 0-2) and the position it is evaluated at (at: the
// station, or 1 m below it for the vertical gradient).
#pragma once
#include "prism_math.cuh"

namespace j3g {

enum Kind : int {
  KIND_SCALAR = 1,
  KIND_TENSOR = 2,
  KIND_MAGNETIC = 3,
  KIND_JOINT = 4,
  KIND_MAG_GRADIENT = 5,
  KIND_MAGNETIZATION = 6
};
constexpr int kMaxVc = 9;  // largest number of virtual components of a kind
enum Transform : int { TR_NONE = 0, TR_FTG_INVARIANT = 1, TR_TOTAL_FIELD = 2, TR_TFA = 3 };

constexpr int kTensorMask = (1 << NC_XX) | (1 << NC_YY) | (1 << NC_ZZ) | (1 << NC_XY) |
                            (1 << NC_XZ) | (1 << NC_YZ);

// Kinds whose virtual components are the contiguous node components
// [off, off + ncomp) at the station, all on model block 0.
template <int MASK, int NCOMP, int RAW, int OFF> struct ContiguousTraits {
  static constexpr int mask = MASK;
  static constexpr int ncomp = NCOMP;  // virtual components per station
  static constexpr int raw = RAW;
  static constexpr int nblock = 1;
  static constexpr bool twin = false;
  static constexpr bool special = false;  // reduced to raw rows by the node path
  __host__ __device__ static constexpr int comp(int q) { return q + OFF; }
  __host__ __device__ static constexpr int block(int) { return 0; }
  __host__ __device__ static constexpr int at(int) { return 0; }
};

template <int KIND> struct KindTraits;
template <> struct KindTraits<KIND_SCALAR> : ContiguousTraits<1 << NC_GZ, 1, 1, 0> {};
template <> struct KindTraits<KIND_TENSOR> : ContiguousTraits<kTensorMask, 6, 9, 1> {};
template <> struct KindTraits<KIND_MAGNETIC> : ContiguousTraits<kTensorMask, 6, 3, 1> {};
template <> struct KindTraits<KIND_JOINT>
    : ContiguousTraits<(1 << NC_GZ) | kTensorMask, 7, 10, 0> {};
// Uxz, Uyz, Uzz at the station (q 0-2) and 1 m below it (q 3-5).
template <> struct KindTraits<KIND_MAG_GRADIENT> {
  static constexpr int mask = (1 << NC_XZ) | (1 << NC_YZ) | (1 << NC_ZZ);
  static constexpr int ncomp = 6;
  static constexpr int raw = 1;
  static constexpr int nblock = 1;
  static constexpr bool twin = true;
  static constexpr bool special = true;
  __host__ __device__ static constexpr int comp(int q) {
    return q % 3 == 0 ? NC_XZ : (q % 3 == 1 ? NC_YZ : NC_ZZ);
  }
  __host__ __device__ static constexpr int block(int) { return 0; }
  __host__ __device__ static constexpr int at(int q) { return q / 3; }
};
// U_kj against magnetisation block j, row-major in (k, j).
template <> struct KindTraits<KIND_MAGNETIZATION> {
  static constexpr int mask = kTensorMask;
  static constexpr int ncomp = 9;
  static constexpr int raw = 3;
  static constexpr int nblock = 3;
  static constexpr bool twin = false;
  static constexpr bool special = true;
  __host__ __device__ static constexpr int comp(int q) {
    return q == 0 ? NC_XX : q == 4 ? NC_YY : q == 8 ? NC_ZZ
         : (q == 1 || q == 3) ? NC_XY : (q == 2 || q == 6) ? NC_XZ : NC_YZ;
  }
  __host__ __device__ static constexpr int block(int q) { return q % 3; }
  __host__ __device__ static constexpr int at(int) { return 0; }
};

__host__ __device__ inline int kind_mask(int kind) {
  return kind == KIND_SCALAR        ? (1 << NC_GZ)
         : kind == KIND_JOINT       ? ((1 << NC_GZ) | kTensorMask)
         : kind == KIND_MAG_GRADIENT ? KindTraits<KIND_MAG_GRADIENT>::mask
                                    : kTensorMask;
}
__host__ __device__ constexpr inline int kind_raw(int kind) {
  return (kind == KIND_SCALAR || kind == KIND_MAG_GRADIENT) ? 1
         : kind == KIND_TENSOR                              ? 9
         : (kind == KIND_MAGNETIC || kind == KIND_MAGNETIZATION) ? 3
                                                            : 10;
}
// Virtual components per station.
__host__ __device__ constexpr inline int kind_ncomp(int kind) {
  return kind == KIND_SCALAR ? 1
         : kind == KIND_JOINT ? 7
         : kind == KIND_MAGNETIZATION ? 9
                                      : 6;
}
__host__ __device__ inline int kind_nblock(int kind) {
  return kind == KIND_MAGNETIZATION ? 3 : 1;
}
// The node path reduces these kinds to raw rows directly (no node-component
// layout); they have no background response.
__host__ __device__ constexpr inline bool kind_special(int kind) {
  return kind == KIND_MAG_GRADIENT || kind == KIND_MAGNETIZATION;
}
// Rows of the device-resident sensitivity per station: the raw rows for the
// magnetic kinds (Bx By Bz; the vertical gradient; the three field
// components over the three magnetisation blocks), else the kind's node
// components (scalar 1, tensor 6, joint 7), from which the raw rows follow.
__host__ __device__ constexpr inline bool stored_is_raw(int kind) {
  return kind == KIND_MAGNETIC || kind_special(kind);
}
__host__ __device__ constexpr inline int stored_rows(int kind) {
  return stored_is_raw(kind) ? kind_raw(kind) : kind_ncomp(kind);
}
// Slot s of a kind's compact component list -> node component id.
__host__ __device__ constexpr inline int slot_comp(int kind, int s) {
  return (kind == KIND_SCALAR || kind == KIND_JOINT) ? s : s + 1;
}

// The magnetic projection B_k = F/(4 pi G) sum_j U_kj b_j with
// b = (cos I cos D, cos I sin D, sin I)
// (Magnetics/OMPMagneticSusceptibilityImp.cpp:116-118, 160-170).
struct MagField {
  double bx, by, bz;  // direction cosines of the inducing field
  double fs;          // field strength (nT)
  double factor;      // 1 / (4 pi G); 1e-7 / G for the vertical gradient
                      // (OMPMagneticGradImp.cpp:66); 1e9 mu0 / (4 pi G) for
                      // magnetisation (OMPMagnetizationImp.cpp:58-59)
};

// Raw rows of the special kinds from their virtual components v[q] (already
// multiplied by comp_scale).  Vertical gradient: Bz at the station minus Bz
// 1 m below, Bz = ((Uxz bx + Uyz by) + Uzz bz) fs factor
// (OMPMagneticGradImp.cpp:67-71, 82-86, 103).  Magnetisation:
// B_k = ((c_k0 + c_k1) + c_k2) with c_kj = factor * U_kj . M_j
// (OMPMagnetizationImp.cpp:82-92).
__host__ __device__ inline void raw_from_vc(int kind, const double *v, const MagField &m,
                                            double *raw) {
  if (kind == KIND_MAG_GRADIENT) {
    const double bot = mul(mul(add(add(mul(v[0], m.bx), mul(v[1], m.by)), mul(v[2], m.bz)), m.fs), m.factor);
    const double top = mul(mul(add(add(mul(v[3], m.bx), mul(v[4], m.by)), mul(v[5], m.bz)), m.fs), m.factor);
    raw[0] = sub(bot, top);
    return;
  }
  for (int k = 0; k < 3; ++k)
    raw[k] = add(add(mul(m.factor, v[3 * k]), mul(m.factor, v[3 * k + 1])),
                 mul(m.factor, v[3 * k + 2]));
}

// Adjoint of raw_from_vc: raw weights -> virtual-component weights.
__host__ __device__ inline void vc_from_raw_weights(int kind, const double *w, const MagField &m,
                                                    double *u) {
  if (kind == KIND_MAG_GRADIENT) {
    const double f = w[0] * m.fs * m.factor;
    u[0] = f * m.bx;
    u[1] = f * m.by;
    u[2] = f * m.bz;
    u[3] = -u[0];
    u[4] = -u[1];
    u[5] = -u[2];
    return;
  }
  for (int q = 0; q < 9; ++q) u[q] = w[q / 3] * m.factor;
}

// Node component of virtual component q of a kind (host and device).
__host__ __device__ inline int vc_comp(int kind, int q) {
  switch (kind) {
    case KIND_SCALAR: return KindTraits<KIND_SCALAR>::comp(q);
    case KIND_TENSOR: return KindTraits<KIND_TENSOR>::comp(q);
    case KIND_MAGNETIC: return KindTraits<KIND_MAGNETIC>::comp(q);
    case KIND_JOINT: return KindTraits<KIND_JOINT>::comp(q);
    case KIND_MAG_GRADIENT: return KindTraits<KIND_MAG_GRADIENT>::comp(q);
    default: return KindTraits<KIND_MAGNETIZATION>::comp(q);
  }
}

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
