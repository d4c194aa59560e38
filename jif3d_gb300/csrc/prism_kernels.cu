// prism_kernels.cu -- FP64 matrix-free prism kernels for sm_103a.
//
// Work is organised around mesh NODES (see prism_math.cuh): for a station s
// every node n carries the corner terms F_c(s, n).  Three uses:
//   forward   U_c(s) = scale_c * sum_n F_c(s, n) * rho~(n)          (summation by parts)
//   adjoint   G(n)   = sum_s sum_c W_c(s) F_c(s, n),  grad(cell) = 2 * D3[G](cell)
//   J rows    T_c(s, cell) = eight-node sum in the reference's order
// where D3 is the signed eight-corner sum of a cell and rho~ its transpose
// applied to the model.  These reproduce ScalarOMPGravityImp::CalcGridded
// (Gravity/ScalarOMPGravityImp.cpp:138-180), TensorOMPGravityImp::CalcGridded
// (Gravity/TensorOMPGravityImp.cpp:125-182), the magnetic CalcGridded
// (Magnetics/OMPMagneticSusceptibilityImp.cpp:113-194) and the matrix-free
// LQDerivative (GravMag/ThreeDGravMagImplementation.h:177-231), with all
// stations in one launch and the reduction with the model on the device.
//
// All reductions have a fixed order, so results repeat bit for bit.
#include "prism_kernels.h"

namespace j3g {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ void decode_node(int n, int ny1, int nz1, int &i, int &j, int &k) {
  k = n % nz1;
  const int t = n / nz1;
  j = t % ny1;
  i = t / ny1;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <int KIND> struct Slots {
  static constexpr int off = (KIND == KIND_SCALAR || KIND == KIND_JOINT) ? 0 : 1;
};

// ---------------------------------------------------------------------------
// rho~(i,j,k) = sum_{a,b,c in {0,1}} (-1)^(a+b+c) rho(i-a, j-b, k-c), zero outside.
__global__ void k_rho_tilde(MeshView m, const double *__restrict__ rho, double *__restrict__ rt) {
  const int ny1 = m.ny + 1, nz1 = m.nz + 1;
  const int nn = (m.nx + 1) * ny1 * nz1;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  int i, j, k;
  decode_node(n, ny1, nz1, i, j, k);
  double v = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int a = (q >> 2) & 1, b = (q >> 1) & 1, c = q & 1;
    const int ci = i - a, cj = j - b, ck = k - c;
    if (ci < 0 || cj < 0 || ck < 0 || ci >= m.nx || cj >= m.ny || ck >= m.nz) continue;
    const double r = rho[((long long)ci * m.ny + cj) * m.nz + ck];
    v = ((a + b + c) & 1) ? v - r : v + r;
  }
  rt[n] = v;
}

// ---------------------------------------------------------------------------
// Forward partial sums.  Block (bx, by) covers nodes [bx*npb, (bx+1)*npb) and
// stations [by*spb, (by+1)*spb); each thread walks npb/256 nodes per station
// so the block reduction is amortised over several node evaluations.
template <int KIND>
__global__ void __launch_bounds__(kThreads)
    k_node_forward(MeshView m, StationView st, const double *__restrict__ rt,
                   double *__restrict__ partial, int npb, int spb) {
  using T = KindTraits<KIND>;
  constexpr int MASK = T::mask;
  constexpr int NCMP = T::ncomp;
  const int ny1 = m.ny + 1, nz1 = m.nz + 1;
  const int nn = (m.nx + 1) * ny1 * nz1;
  const int n0 = blockIdx.x * npb;
  const int n1 = min(nn, n0 + npb);
  const int s0 = blockIdx.y * spb;
  const int s1 = min(st.n, s0 + spb);
  __shared__ double red[kWarps][NCMP];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int s = s0; s < s1; ++s) {
    const double mx = st.x[s], my = st.y[s], mz = st.z[s];
    // the second position of the vertical gradient, z_meas + 1 as the
    // reference forms it (OMPMagneticGradImp.cpp:76-79)
    const double mz1 = T::twin ? add(mz, 1.0) : mz;
    double acc[NCMP];
#pragma unroll
    for (int q = 0; q < NCMP; ++q) acc[q] = 0.0;
    for (int n = n0 + threadIdx.x; n < n1; n += kThreads) {
      int i, j, k;
      decode_node(n, ny1, nz1, i, j, k);
      double F[T::twin ? 2 : 1][NC_COUNT];
      const double dx = sub(mx, m.X[i]), dy = sub(my, m.Y[j]);
      node_terms<MASK>(dx, dy, sub(mz, m.Z[k]), F[0]);
      if constexpr (T::twin) node_terms<MASK>(dx, dy, sub(mz1, m.Z[k]), F[T::twin ? 1 : 0]);
      double w[T::nblock];
#pragma unroll
      for (int b = 0; b < T::nblock; ++b) w[b] = rt[(long long)b * nn + n];
#pragma unroll
      for (int q = 0; q < NCMP; ++q) acc[q] = fma(F[T::at(q)][T::comp(q)], w[T::block(q)], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < NCMP; ++q) {
      const double v = warp_sum(acc[q]);
      if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < NCMP) {
      double v = 0.0;
#pragma unroll
      for (int w = 0; w < kWarps; ++w) v += red[w][threadIdx.x];
      partial[((long long)blockIdx.x * st.n + s) * NCMP + threadIdx.x] = v;
    }
    __syncthreads();
  }
}

template <int KIND>
__global__ void k_forward_reduce(int nmeas, int nblk, const double *__restrict__ partial,
                                 double *__restrict__ comps) {
  constexpr int NCMP = KindTraits<KIND>::ncomp;
  constexpr int OFF = Slots<KIND>::off;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nmeas * NC_COUNT) return;
  const int s = t / NC_COUNT, c = t % NC_COUNT;
  const int q = c - OFF;
  double v = 0.0;
  if (q >= 0 && q < NCMP && (KindTraits<KIND>::mask & (1 << c))) {
    for (int b = 0; b < nblk; ++b) v += partial[((long long)b * nmeas + s) * NCMP + q];
    v *= comp_scale(c);
  }
  comps[t] = v;
}

// The special kinds: virtual components straight to raw rows[nmeas][raw].
template <int KIND>
__global__ void k_forward_reduce_raw(int nmeas, int nblk, const double *__restrict__ partial,
                                     MagField mf, double *__restrict__ rawrows) {
  using T = KindTraits<KIND>;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nmeas) return;
  double v[kMaxVc];
#pragma unroll
  for (int q = 0; q < T::ncomp; ++q) {
    double a = 0.0;
    for (int b = 0; b < nblk; ++b) a += partial[((long long)b * nmeas + s) * T::ncomp + q];
    v[q] = a * comp_scale(T::comp(q));
  }
  double raw[3];
  raw_from_vc(KIND, v, mf, raw);
#pragma unroll
  for (int r = 0; r < T::raw; ++r) rawrows[(long long)s * T::raw + r] = raw[r];
}

// ---------------------------------------------------------------------------
// Background layer terms (GravityBackground.cpp:24-137).  A block takes 32
// stations of one layer; warp k evaluates one prism component (g_z, Uxx, Uyy,
// Uzz, Uxy, Uxz, Uyz; the eighth warp idles) for those 32 stations, each an
// eight-corner sum in the reference's order, so the serial chain of
// transcendentals per thread is one component long and no warp diverges.
// Warp 0 then combines them with the sheet terms exactly as the reference's
// per-station loop does.  A layer's top is summed from the
// thicknesses in layer order.  The kind is a template argument so that the
// term arrays stay in registers.
template <int KIND>
__global__ void __launch_bounds__(256) k_background(StationView st, int nbg,
                                                    const double *__restrict__ thick, double xo,
                                                    double yo, double zo, double xw, double yw,
                                                    double zw, MagField mf,
                                                    double *__restrict__ bgsens) {
  constexpr int kind = KIND;
  constexpr int raw = kind_raw(kind);
  const int slot = threadIdx.x >> 5, li = threadIdx.x & 31;  // component, station
  const int s = blockIdx.x * 32 + li;
  const int j = blockIdx.y;
  const bool live = s < st.n;
  if constexpr (kind_special(kind)) {  // no background response (OMPMagneticGradImp.h:32-40)
    if (live && slot < raw) bgsens[((long long)s * raw + slot) * nbg + j] = 0.0;
    return;
  } else {
    __shared__ double terms[32][8];
    double mx = 0.0, my = 0.0, mz = 0.0;
    if (live) {
      mx = st.x[s];
      my = st.y[s];
      mz = st.z[s];
    }
    double top = zo;
    for (int i = 0; i < j; ++i) top = add(top, thick[i]);
    const double th = thick[j];
    const double bottom = add(top, th);
    // the slab inside the gridded depth, whole or cut at its bottom
    const bool have = top < zw;
    const double h = bottom <= zw ? th : sub(zw, top);
    constexpr bool kGz = kind == KIND_SCALAR || kind == KIND_JOINT;
    constexpr bool kTensor = kind != KIND_SCALAR;
    double b = 0.0;
    if (live && have) {
      if (slot == 0 && kGz) b = grav_box(mx, my, mz, xo, yo, top, xw, yw, h);
      if (kTensor) {
        if (slot == 1) b = uxx_box(mx, my, mz, xo, yo, top, xw, yw, h);
        if (slot == 2) b = uxx_box(my, mx, mz, yo, xo, top, yw, xw, h);
        if (slot == 3) b = uxx_box(mz, mx, my, top, xo, yo, h, xw, yw);
        if (slot == 4) b = uxy_box(mx, my, mz, xo, yo, top, xw, yw, h);
        if (slot == 5) b = uxy_box(mx, mz, my, xo, top, yo, xw, h, yw);
        if (slot == 6) b = uxy_box(mz, my, mx, top, yo, xo, h, yw, xw);
      }
    }
    terms[li][slot] = b;
    __syncthreads();
    if (!live || slot != 0) return;
    const double *t = terms[li];
    double v[raw];
    if constexpr (kGz) {
      double g = inf_sheet(mz, top, bottom);
      if (have) g = sub(g, t[0]);
      v[0] = g;
    }
    if constexpr (kTensor) {
      // 3 x 3 tensor from the unique components (BasicGravElements.cpp:216-244)
      const double box[9] = {t[1], t[4], t[5], t[4], t[2], t[6], t[5], t[6], t[3]};
      double u[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      u[8] = uzz_inf_sheet(mz, top, bottom);
      if (have) {
#pragma unroll
        for (int c = 0; c < 9; ++c) u[c] = sub(u[c], box[c]);
      }
      if constexpr (kind == KIND_MAGNETIC) {
        const double f1 = mf.fs, f2 = mf.factor;
        v[0] = mul(mul(add(add(mul(u[0], mf.bx), mul(u[1], mf.by)), mul(u[2], mf.bz)), f1), f2);
        v[1] = mul(mul(add(add(mul(u[3], mf.bx), mul(u[4], mf.by)), mul(u[5], mf.bz)), f1), f2);
        v[2] = mul(mul(add(add(mul(u[6], mf.bx), mul(u[7], mf.by)), mul(u[8], mf.bz)), f1), f2);
      } else {
        constexpr int o = kind == KIND_JOINT ? 1 : 0;
#pragma unroll
        for (int c = 0; c < 9; ++c) v[o + c] = u[c];
      }
    }
#pragma unroll
    for (int r = 0; r < raw; ++r) bgsens[((long long)s * raw + r) * nbg + j] = v[r];
  }
}

// ---------------------------------------------------------------------------
__device__ double apply_transform(int transform, const double *raw, double bx, double by,
                                  double bz) {
  switch (transform) {
    case TR_FTG_INVARIANT:  // Gravity/GravityTransforms.h:33-37
      return sub(sub(sub(add(add(mul(raw[0], raw[4]), mul(raw[4], raw[8])), mul(raw[0], raw[8])),
                         mul(raw[3], raw[1])),
                     mul(raw[7], raw[5])),
                 mul(raw[2], raw[6]));
    case TR_TOTAL_FIELD:  // Magnetics/MagneticTransforms.h:27-30
      return sqrt(add(add(mul(raw[0], raw[0]), mul(raw[1], raw[1])), mul(raw[2], raw[2])));
    case TR_TFA:  // Magnetics/MagneticTransforms.h:122-129
      return add(add(mul(bx, raw[0]), mul(by, raw[1])), mul(bz, raw[2]));
    default:
      return raw[0];
  }
}

__global__ void k_assemble(int kind, int transform, double tbx, double tby, double tbz,
                           int nmeas, const double *__restrict__ comps, int comps_ld,
                           const double *__restrict__ bgsens, int nbg,
                           const double *__restrict__ bgval, MagField mf,
                           double *__restrict__ raw_out, double *__restrict__ data_out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nmeas) return;
  const int raw = kind_raw(kind);
  double r[10];
  if (comps_ld == NC_COUNT) {
    double u[NC_COUNT];
    for (int c = 0; c < NC_COUNT; ++c) u[c] = comps[(long long)s * NC_COUNT + c];
    raw_from_comps(kind, u, mf, r);
  } else {  // comps already hold raw gridded rows
    for (int c = 0; c < raw; ++c) r[c] = comps[(long long)s * comps_ld + c];
  }
  for (int c = 0; c < raw; ++c) {
    double bg = 0.0;
    for (int j = 0; j < nbg; ++j)
      bg = add(bg, mul(bgsens[((long long)s * raw + c) * nbg + j], bgval[j]));
    r[c] = add(r[c], bg);
    if (raw_out) raw_out[(long long)s * raw + c] = r[c];
  }
  if (transform == TR_NONE) {
    for (int c = 0; c < raw; ++c) data_out[(long long)s * raw + c] = r[c];
  } else {
    data_out[s] = apply_transform(transform, r, tbx, tby, tbz);
  }
}

// w_raw = misfit * dT/draw (GravityTransforms.h:72-93, MagneticTransforms.h:65-75,136-145);
// without a transform the misfit is the raw weight.
__global__ void k_backproject(int kind, int transform, double tbx, double tby, double tbz,
                              int nmeas, const double *__restrict__ misfit,
                              const double *__restrict__ rawd, double *__restrict__ w_raw) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nmeas) return;
  const int raw = kind_raw(kind);
  if (transform == TR_NONE) {
    for (int c = 0; c < raw; ++c) w_raw[(long long)s * raw + c] = misfit[(long long)s * raw + c];
    return;
  }
  const double m = misfit[s];
  const double *d = rawd + (long long)s * raw;
  double *w = w_raw + (long long)s * raw;
  if (transform == TR_FTG_INVARIANT) {
    w[0] = mul(m, add(d[4], d[8]));
    w[1] = mul(m, -d[3]);
    w[2] = mul(m, -d[6]);
    w[3] = mul(m, -d[1]);
    w[4] = mul(m, add(d[0], d[8]));
    w[5] = mul(m, -d[7]);
    w[6] = mul(m, -d[2]);
    w[7] = mul(m, -d[5]);
    w[8] = mul(m, add(d[0], d[4]));
  } else if (transform == TR_TOTAL_FIELD) {
    const double t = sqrt(add(add(mul(d[0], d[0]), mul(d[1], d[1])), mul(d[2], d[2])));
    for (int c = 0; c < 3; ++c) w[c] = mul(m, d[c] / t);
  } else {  // TFA
    w[0] = mul(m, tbx);
    w[1] = mul(m, tby);
    w[2] = mul(m, tbz);
  }
}

__global__ void k_comp_weights(int kind, int nmeas, const double *__restrict__ w_raw, MagField mf,
                               double *__restrict__ W) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nmeas) return;
  const int raw = kind_raw(kind);
  double w[10];
  for (int c = 0; c < raw; ++c) w[c] = w_raw[(long long)s * raw + c];
  if (kind_special(kind)) {  // virtual-component weights [nmeas][ncomp]
    const int nv = kind_ncomp(kind);
    double u[kMaxVc];
    vc_from_raw_weights(kind, w, mf, u);
    for (int q = 0; q < nv; ++q)
      W[(long long)s * nv + q] = u[q] * comp_scale(vc_comp(kind, q));
    return;
  }
  double u[NC_COUNT];
  comps_from_raw_weights(kind, w, mf, u);
  for (int c = 0; c < NC_COUNT; ++c) W[(long long)s * NC_COUNT + c] = u[c] * comp_scale(c);
}

// ---------------------------------------------------------------------------
// Adjoint: one thread per node, stations of one chunk staged through shared
// memory 64 at a time.
constexpr int kStage = 64;

template <int KIND>
__global__ void __launch_bounds__(kThreads)
    k_node_adjoint(MeshView m, StationView st, const double *__restrict__ W, int spc,
                   const int *__restrict__ chunk_start, double *__restrict__ Gpart) {
  using T = KindTraits<KIND>;
  constexpr int MASK = T::mask;
  constexpr int NCMP = T::ncomp;
  // weights: node-component layout [nmeas][NC_COUNT], or [nmeas][ncomp] for
  // the special kinds
  constexpr int WLD = T::special ? NCMP : NC_COUNT;
  const int ny1 = m.ny + 1, nz1 = m.nz + 1;
  const int nn = (m.nx + 1) * ny1 * nz1;
  const int n = blockIdx.x * kThreads + threadIdx.x;
  const int chunk = blockIdx.y;
  // stations of this chunk: spc apiece, or the ranges of chunk_start (chunks
  // that never straddle a station subset)
  const int s0 = chunk_start ? chunk_start[chunk] : chunk * spc;
  const int s1 = chunk_start ? chunk_start[chunk + 1] : min(st.n, s0 + spc);
  __shared__ double sx[kStage], sy[kStage], sz[kStage], sw[kStage][NCMP];
  int i = 0, j = 0, k = 0;
  if (n < nn) decode_node(n, ny1, nz1, i, j, k);
  const double X = (n < nn) ? m.X[i] : 0.0, Y = (n < nn) ? m.Y[j] : 0.0,
               Z = (n < nn) ? m.Z[k] : 0.0;
  double acc[T::nblock];
#pragma unroll
  for (int b = 0; b < T::nblock; ++b) acc[b] = 0.0;
  for (int base = s0; base < s1; base += kStage) {
    const int cnt = min(kStage, s1 - base);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt; t += kThreads) {
      sx[t] = st.x[base + t];
      sy[t] = st.y[base + t];
      sz[t] = st.z[base + t];
#pragma unroll
      for (int q = 0; q < NCMP; ++q)
        sw[t][q] = W[(long long)(base + t) * WLD + (T::special ? q : T::comp(q))];
    }
    __syncthreads();
    if (n < nn) {
      for (int t = 0; t < cnt; ++t) {
        double F[T::twin ? 2 : 1][NC_COUNT];
        const double dx = sub(sx[t], X), dy = sub(sy[t], Y);
        node_terms<MASK>(dx, dy, sub(sz[t], Z), F[0]);
        if constexpr (T::twin) node_terms<MASK>(dx, dy, sub(add(sz[t], 1.0), Z), F[T::twin ? 1 : 0]);
#pragma unroll
        for (int q = 0; q < NCMP; ++q)
          acc[T::block(q)] = fma(sw[t][q], F[T::at(q)][T::comp(q)], acc[T::block(q)]);
      }
    }
  }
  if (n < nn) {
#pragma unroll
    for (int b = 0; b < T::nblock; ++b)
      Gpart[((long long)chunk * T::nblock + b) * nn + n] = acc[b];
  }
}

// G[n] = sum_c Gpart[c * stride + n] (stride = blocks x nodes per chunk).
__global__ void k_sum_chunks(int nn, int nchunk, long long stride,
                             const double *__restrict__ Gpart, double *__restrict__ G) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  double v = 0.0;
  for (int c = 0; c < nchunk; ++c) v += Gpart[(long long)c * stride + n];
  G[n] = v;
}

// grad(cell) = 2 * sum_{a,b,c} (-1)^(a+b+c) G(i+a, j+b, k+c)
__global__ void k_adjoint_combine(MeshView m, const double *__restrict__ G,
                                  double *__restrict__ grad) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= m.ngrid()) return;
  const int k = cell % m.nz;
  const long long t = cell / m.nz;
  const int j = t % m.ny;
  const int i = t / m.ny;
  const int ny1 = m.ny + 1, nz1 = m.nz + 1;
  double v = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int a = (q >> 2) & 1, b = (q >> 1) & 1, c = q & 1;
    const double g = G[((long long)(i + a) * ny1 + (j + b)) * nz1 + (k + c)];
    v = ((a + b + c) & 1) ? v - g : v + g;
  }
  grad[cell] = 2.0 * v;
}

__global__ void k_background_grad(int kind, int nmeas, int nbg, const double *__restrict__ w_raw,
                                  const double *__restrict__ bgsens, double *__restrict__ gbg) {
  const int j = blockIdx.x;
  const int raw = kind_raw(kind);
  double acc = 0.0;
  for (int s = threadIdx.x; s < nmeas; s += blockDim.x)
    for (int r = 0; r < raw; ++r)
      acc = fma(w_raw[(long long)s * raw + r], bgsens[((long long)s * raw + r) * nbg + j], acc);
  __shared__ double red[kWarps];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < kWarps; ++w) v += red[w];
    gbg[j] = 2.0 * v;
  }
}

// ---------------------------------------------------------------------------
// Sensitivity rows.
template <int KIND>
__global__ void __launch_bounds__(kThreads)
    k_node_eval(MeshView m, StationView st, int s0, double *__restrict__ F) {
  using T = KindTraits<KIND>;
  constexpr int MASK = T::mask;
  constexpr int NCMP = T::ncomp;
  const int ny1 = m.ny + 1, nz1 = m.nz + 1;
  const int nn = (m.nx + 1) * ny1 * nz1;
  const int n = blockIdx.x * kThreads + threadIdx.x;
  const int sl = blockIdx.y;
  if (n >= nn) return;
  int i, j, k;
  decode_node(n, ny1, nz1, i, j, k);
  const int s = s0 + sl;
  double v[T::twin ? 2 : 1][NC_COUNT];
  const double dx = sub(st.x[s], m.X[i]), dy = sub(st.y[s], m.Y[j]);
  node_terms<MASK>(dx, dy, sub(st.z[s], m.Z[k]), v[0]);
  if constexpr (T::twin) node_terms<MASK>(dx, dy, sub(add(st.z[s], 1.0), m.Z[k]), v[T::twin ? 1 : 0]);
#pragma unroll
  for (int q = 0; q < NCMP; ++q) F[((long long)sl * NCMP + q) * nn + n] = v[T::at(q)][T::comp(q)];
}

// Raw rows of one cell from its virtual-component box values u[q]:
// the ordinary kinds through raw_from_comps, the vertical gradient through
// raw_from_vc (BzSensBot - BzSensTop, OMPMagneticGradImp.cpp:88-99) and
// magnetisation as factor * U_kj in row k, column block j
// (OMPMagnetizationImp.cpp:58-68, 93-104).
template <int KIND, class OutT = double>
__device__ __forceinline__ void store_cell_rows(const double *u, const MagField &mf,
                                                long long ngrid, long long cell, OutT *rows,
                                                long long ld) {
  using T = KindTraits<KIND>;
  if constexpr (KIND == KIND_MAGNETIZATION) {
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int jb = 0; jb < 3; ++jb)
        rows[(long long)k * ld + jb * ngrid + cell] = (OutT)mul(mf.factor, u[3 * k + jb]);
  } else if constexpr (KIND == KIND_MAG_GRADIENT) {
    double raw[3];
    raw_from_vc(KIND, u, mf, raw);
    rows[cell] = (OutT)raw[0];
  } else {
    double c[NC_COUNT];
#pragma unroll
    for (int q = 0; q < T::ncomp; ++q) c[T::comp(q)] = u[q];
    double raw[10];
    raw_from_comps(KIND, c, mf, raw);
#pragma unroll
    for (int r = 0; r < T::raw; ++r) rows[(long long)r * ld + cell] = (OutT)raw[r];
  }
}

template <int KIND>
__global__ void __launch_bounds__(kThreads)
    k_cell_rows(MeshView m, const double *__restrict__ F, MagField mf, double *__restrict__ rows,
                long long ld) {
  using T = KindTraits<KIND>;
  constexpr int NCMP = T::ncomp;
  const long long cell = (long long)blockIdx.x * kThreads + threadIdx.x;
  const int sl = blockIdx.y;
  if (cell >= m.ngrid()) return;
  const int k = cell % m.nz;
  const long long t = cell / m.nz;
  const int j = t % m.ny;
  const int i = t / m.ny;
  const int ny1 = m.ny + 1, nz1 = m.nz + 1;
  const int nn = (m.nx + 1) * ny1 * nz1;
  double u[kMaxVc];
#pragma unroll
  for (int q = 0; q < NCMP; ++q) {
    const double *f = F + ((long long)sl * NCMP + q) * nn;
    double v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c)
      v[c] = f[((i + ((c >> 2) & 1)) * ny1 + (j + ((c >> 1) & 1))) * nz1 + (k + (c & 1))];
    u[q] = combine8(T::comp(q), v);
  }
  store_cell_rows<KIND>(u, mf, m.ngrid(), cell, rows + (long long)sl * T::raw * ld, ld);
}

// Stored rows for the device-resident sensitivity: the node components of the
// kind (scalar 1, tensor 6, joint 7) or the raw magnetic rows (3 of Bx By Bz;
// 1 of the vertical gradient; 3 over the three magnetisation blocks, columns
// block * ngrid + cell), one row per (station, stored component), written as
// OutT (double or float).
template <int KIND> struct StoredRows {
  static constexpr int n = stored_rows(KIND);
};

template <int KIND, class OutT>
__global__ void __launch_bounds__(kThreads)
    k_cell_stored(MeshView m, const double *__restrict__ F, MagField mf, OutT *__restrict__ rows,
                  long long ld) {
  constexpr int NCMP = KindTraits<KIND>::ncomp;
  constexpr int OFF = Slots<KIND>::off;
  constexpr int NS = StoredRows<KIND>::n;
  const long long cell = (long long)blockIdx.x * kThreads + threadIdx.x;
  const int sl = blockIdx.y;
  if (cell >= m.ngrid()) return;
  const int k = cell % m.nz;
  const long long t = cell / m.nz;
  const int j = t % m.ny;
  const int i = t / m.ny;
  const int ny1 = m.ny + 1, nz1 = m.nz + 1;
  const int nn = (m.nx + 1) * ny1 * nz1;
  if constexpr (KindTraits<KIND>::special) {
    // the raw rows, as k_cell_rows forms them
    double u[kMaxVc];
#pragma unroll
    for (int q = 0; q < NCMP; ++q) {
      const double *f = F + ((long long)sl * NCMP + q) * nn;
      double v[8];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        v[c] = f[((i + ((c >> 2) & 1)) * ny1 + (j + ((c >> 1) & 1))) * nz1 + (k + (c & 1))];
      u[q] = combine8(KindTraits<KIND>::comp(q), v);
    }
    store_cell_rows<KIND, OutT>(u, mf, m.ngrid(), cell, rows + (long long)sl * NS * ld, ld);
  } else {
    double u[NC_COUNT];
#pragma unroll
    for (int q = 0; q < NCMP; ++q) {
      const double *f = F + ((long long)sl * NCMP + q) * nn;
      double v[8];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        v[c] = f[((i + ((c >> 2) & 1)) * ny1 + (j + ((c >> 1) & 1))) * nz1 + (k + (c & 1))];
      u[q + OFF] = combine8(q + OFF, v);
    }
    if (KIND == KIND_MAGNETIC) {
      double raw[10];
      raw_from_comps(KIND, u, mf, raw);
#pragma unroll
      for (int r = 0; r < 3; ++r) rows[((long long)sl * NS + r) * ld + cell] = (OutT)raw[r];
    } else {
#pragma unroll
      for (int q = 0; q < NCMP; ++q) rows[((long long)sl * NS + q) * ld + cell] = (OutT)u[q + OFF];
    }
  }
}

template <int KIND>
__global__ void __launch_bounds__(kThreads)
    k_cell_direct(MeshView m, StationView st, int s0, MagField mf, double *__restrict__ rows,
                  long long ld) {
  using T = KindTraits<KIND>;
  constexpr int MASK = T::mask;
  const long long cell = (long long)blockIdx.x * kThreads + threadIdx.x;
  const int sl = blockIdx.y;
  if (cell >= m.ngrid()) return;
  const int k = cell % m.nz;
  const long long t = cell / m.nz;
  const int j = t % m.ny;
  const int i = t / m.ny;
  const int s = s0 + sl;
  double c[T::twin ? 2 : 1][NC_COUNT];
  prism_components(MASK, st.x[s], st.y[s], st.z[s], m.X[i], m.Y[j], m.Z[k], m.xs[i], m.ys[j],
                   m.zs[k], c[0]);
  if constexpr (T::twin)
    prism_components(MASK, st.x[s], st.y[s], add(st.z[s], 1.0), m.X[i], m.Y[j], m.Z[k], m.xs[i],
                     m.ys[j], m.zs[k], c[T::twin ? 1 : 0]);
  double u[kMaxVc];
#pragma unroll
  for (int q = 0; q < T::ncomp; ++q) u[q] = c[T::at(q)][T::comp(q)];
  store_cell_rows<KIND>(u, mf, m.ngrid(), cell, rows + (long long)sl * T::raw * ld, ld);
}

__global__ void k_rows_dot(int raw, long long ngrid, const double *__restrict__ rows,
                           long long ld, const double *__restrict__ rho, double *__restrict__ out) {
  const int row = blockIdx.x;  // sl * raw + r
  const double *p = rows + (long long)row * ld;
  double acc = 0.0;
  for (long long c = threadIdx.x; c < ngrid; c += blockDim.x) acc = fma(p[c], rho[c], acc);
  __shared__ double red[kWarps];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < kWarps; ++w) v += red[w];
    out[row] = v;
  }
}

// grad[cell] += sum_{sl, r} w[(sl*raw + r)] * rows[(sl*raw + r)*ld + cell]
__global__ void k_rows_tdot(int nrow, long long ngrid, const double *__restrict__ rows, long long ld,
                            const double *__restrict__ w, double *__restrict__ grad) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ngrid) return;
  double acc = grad[cell];
  for (int r = 0; r < nrow; ++r) acc = fma(w[r], rows[(long long)r * ld + cell], acc);
  grad[cell] = acc;
}

__global__ void k_scale(long long n, double f, double *__restrict__ v) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) v[t] *= f;
}

__global__ void k_fp64_probe(double *out, int n_iter) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1.0, a2 = a0 + 2.0, a3 = a0 + 3.0;
  const double b = 0.999999, c = 1e-7;
  for (int it = 0; it < n_iter; ++it) {
    a0 = fma(a0, b, c);
    a1 = fma(a1, b, c);
    a2 = fma(a2, b, c);
    a3 = fma(a3, b, c);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3;
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
#define J3G_DISPATCH4(kind, CALL, OTHER)                                     \
  switch (kind) {                                                            \
    case KIND_SCALAR: { constexpr int K = KIND_SCALAR; CALL; } break;        \
    case KIND_TENSOR: { constexpr int K = KIND_TENSOR; CALL; } break;        \
    case KIND_MAGNETIC: { constexpr int K = KIND_MAGNETIC; CALL; } break;    \
    case KIND_JOINT: { constexpr int K = KIND_JOINT; CALL; } break;          \
    OTHER                                                                    \
    default: return cudaErrorInvalidValue;                                   \
  }
// every kind
#define J3G_DISPATCH(kind, CALL)                                                       \
  J3G_DISPATCH4(kind, CALL,                                                            \
                case KIND_MAG_GRADIENT: { constexpr int K = KIND_MAG_GRADIENT; CALL; } break; \
                case KIND_MAGNETIZATION: { constexpr int K = KIND_MAGNETIZATION; CALL; } break;)
// the kinds with a node-component layout (node reduce)
#define J3G_DISPATCH_ORDINARY(kind, CALL) J3G_DISPATCH4(kind, CALL, )

cudaError_t launch_rho_tilde(const MeshView &m, const double *rho, double *rho_t,
                             cudaStream_t st) {
  const long long nn = m.nnodes();
  k_rho_tilde<<<cdiv(nn, kThreads), kThreads, 0, st>>>(m, rho, rho_t);
  return cudaGetLastError();
}

cudaError_t launch_node_forward(int kind, const MeshView &m, const StationView &s,
                                const double *rho_t, double *partial, int nblk, int npb, int spb,
                                cudaStream_t st) {
  dim3 grid(nblk, cdiv(s.n, spb));
  J3G_DISPATCH(kind, (k_node_forward<K><<<grid, kThreads, 0, st>>>(m, s, rho_t, partial, npb, spb)));
  return cudaGetLastError();
}

cudaError_t launch_forward_reduce(int kind, int nmeas, int nblk, const double *partial,
                                  const MagField &mf, double *comps, cudaStream_t st) {
  if (kind == KIND_MAG_GRADIENT) {
    k_forward_reduce_raw<KIND_MAG_GRADIENT><<<cdiv(nmeas, kThreads), kThreads, 0, st>>>(
        nmeas, nblk, partial, mf, comps);
    return cudaGetLastError();
  }
  if (kind == KIND_MAGNETIZATION) {
    k_forward_reduce_raw<KIND_MAGNETIZATION><<<cdiv(nmeas, kThreads), kThreads, 0, st>>>(
        nmeas, nblk, partial, mf, comps);
    return cudaGetLastError();
  }
  const int n = nmeas * NC_COUNT;
  J3G_DISPATCH_ORDINARY(kind, (k_forward_reduce<K><<<cdiv(n, kThreads), kThreads, 0, st>>>(nmeas, nblk, partial, comps)));
  return cudaGetLastError();
}

cudaError_t launch_background(int kind, const MeshView &m, const StationView &s, int nbg,
                              const double *bg_thick, double xo, double yo, double zo, double xw,
                              double yw, double zw, const MagField &mf, double *bgsens,
                              cudaStream_t st) {
  (void)m;
  if (nbg == 0 || s.n == 0) return cudaSuccess;
  if (nbg > 65535) return cudaErrorInvalidValue;
  const dim3 grid(cdiv(s.n, 32), nbg);
  J3G_DISPATCH(kind, (k_background<K><<<grid, 256, 0, st>>>(s, nbg, bg_thick, xo, yo, zo, xw, yw,
                                                              zw, mf, bgsens)));
  return cudaGetLastError();
}

cudaError_t launch_assemble(int kind, int transform, double tbx, double tby, double tbz,
                            int nmeas, const double *comps, int comps_ld, const double *bgsens,
                            int nbg, const double *bgval, const MagField &mf, double *raw_out,
                            double *data_out, cudaStream_t st) {
  k_assemble<<<cdiv(nmeas, 128), 128, 0, st>>>(kind, transform, tbx, tby, tbz, nmeas, comps,
                                                comps_ld, bgsens, nbg, bgval, mf, raw_out,
                                                data_out);
  return cudaGetLastError();
}

cudaError_t launch_backproject(int kind, int transform, double tbx, double tby, double tbz,
                               int nmeas, const double *misfit, const double *raw,
                               double *w_raw, cudaStream_t st) {
  k_backproject<<<cdiv(nmeas, 128), 128, 0, st>>>(kind, transform, tbx, tby, tbz, nmeas, misfit,
                                                  raw, w_raw);
  return cudaGetLastError();
}

cudaError_t launch_comp_weights(int kind, int nmeas, const double *w_raw, const MagField &mf,
                                double *W, cudaStream_t st) {
  k_comp_weights<<<cdiv(nmeas, 128), 128, 0, st>>>(kind, nmeas, w_raw, mf, W);
  return cudaGetLastError();
}

cudaError_t launch_node_adjoint(int kind, const MeshView &m, const StationView &s,
                                const double *W, int spc, int nchunk, const int *chunk_start,
                                double *Gpart, cudaStream_t st) {
  dim3 grid(cdiv(m.nnodes(), kThreads), nchunk);
  J3G_DISPATCH(kind, (k_node_adjoint<K><<<grid, kThreads, 0, st>>>(m, s, W, spc, chunk_start, Gpart)));
  return cudaGetLastError();
}

cudaError_t launch_adjoint_combine(const MeshView &m, int nchunk, int nblock, const double *Gpart,
                                   double *G, double *grad, cudaStream_t st) {
  const long long nn = m.nnodes();
  for (int b = 0; b < nblock; ++b) {
    k_sum_chunks<<<cdiv(nn, kThreads), kThreads, 0, st>>>((int)nn, nchunk, nblock * nn,
                                                           Gpart + b * nn, G + b * nn);
    k_adjoint_combine<<<cdiv(m.ngrid(), kThreads), kThreads, 0, st>>>(m, G + b * nn,
                                                                      grad + b * m.ngrid());
  }
  return cudaGetLastError();
}

cudaError_t launch_background_grad(int kind, int nmeas, int nbg, const double *w_raw,
                                   const double *bgsens, double *grad_bg, cudaStream_t st) {
  if (nbg == 0) return cudaSuccess;
  k_background_grad<<<nbg, kThreads, 0, st>>>(kind, nmeas, nbg, w_raw, bgsens, grad_bg);
  return cudaGetLastError();
}

cudaError_t launch_sens_rows(int kind, bool node_exact, const MeshView &m, const StationView &s,
                             int s0, int ns, const MagField &mf, double *F, double *rows,
                             long long ld, cudaStream_t st) {
  if (node_exact) {
    dim3 g1(cdiv(m.nnodes(), kThreads), ns);
    dim3 g2(cdiv(m.ngrid(), kThreads), ns);
    J3G_DISPATCH(kind, (k_node_eval<K><<<g1, kThreads, 0, st>>>(m, s, s0, F),
                        k_cell_rows<K><<<g2, kThreads, 0, st>>>(m, F, mf, rows, ld)));
  } else {
    dim3 g2(cdiv(m.ngrid(), kThreads), ns);
    J3G_DISPATCH(kind, (k_cell_direct<K><<<g2, kThreads, 0, st>>>(m, s, s0, mf, rows, ld)));
  }
  return cudaGetLastError();
}

int stored_rows_per_station(int kind) {
  return stored_rows(kind);
}

cudaError_t launch_stored_rows(int kind, const MeshView &m, const StationView &s, int s0, int ns,
                               const MagField &mf, double *F, double *rows64, float *rows32,
                               long long ld, cudaStream_t st) {
  dim3 g1(cdiv(m.nnodes(), kThreads), ns);
  dim3 g2(cdiv(m.ngrid(), kThreads), ns);
  if (rows64) {
    J3G_DISPATCH(kind, (k_node_eval<K><<<g1, kThreads, 0, st>>>(m, s, s0, F),
                        k_cell_stored<K, double><<<g2, kThreads, 0, st>>>(m, F, mf, rows64, ld)));
  } else {
    J3G_DISPATCH(kind, (k_node_eval<K><<<g1, kThreads, 0, st>>>(m, s, s0, F),
                        k_cell_stored<K, float><<<g2, kThreads, 0, st>>>(m, F, mf, rows32, ld)));
  }
  return cudaGetLastError();
}

cudaError_t launch_rows_dot(int raw, int ns, long long ngrid, const double *rows, long long ld,
                            const double *rho, double *out, cudaStream_t st) {
  k_rows_dot<<<ns * raw, kThreads, 0, st>>>(raw, ngrid, rows, ld, rho, out);
  return cudaGetLastError();
}

cudaError_t launch_rows_tdot(int nrow, long long ngrid, const double *rows, long long ld,
                             const double *w, double *grad, cudaStream_t st) {
  k_rows_tdot<<<cdiv(ngrid, kThreads), kThreads, 0, st>>>(nrow, ngrid, rows, ld, w, grad);
  return cudaGetLastError();
}

cudaError_t launch_scale(long long n, double f, double *v, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_scale<<<cdiv(n, kThreads), kThreads, 0, st>>>(n, f, v);
  return cudaGetLastError();
}

cudaError_t launch_fp64_probe(double *out, int blocks, int threads, int n_iter,
                              cudaStream_t st) {
  k_fp64_probe<<<blocks, threads, 0, st>>>(out, n_iter);
  return cudaGetLastError();
}

}  // namespace j3g
