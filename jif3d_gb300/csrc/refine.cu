// Model refinement: axis refinement and cell walks (host), projection of
// cell values and combination of gradients (device).  The device passes are
// HBM-bound copies and sums; both follow the reference's index walk exactly,
// so their results are bit-identical to it.
#include <algorithm>
#include <cstdint>

#include "refine.h"

namespace j3g {

int refine_axis(int ncoarse, const double *coarse_coords, const double *coarse_sizes, int nref,
                const double *ref_coords, std::vector<double> &fine_sizes) {
  // the refined axis keeps every coarse corner and inserts the refinement
  // coordinates that lie inside each coarse cell (ModelRefiner.cpp:29-50);
  // a refinement coordinate equal to a coarse corner is consumed, not doubled
  const size_t nr = (size_t)nref - 1;
  size_t r = 0;
  std::vector<double> corners;
  corners.reserve((size_t)ncoarse + nr);
  for (int i = 0; i < ncoarse; ++i) {
    corners.push_back(coarse_coords[i]);
    if (r < nr && ref_coords[r] == coarse_coords[i]) ++r;
    const double limit = coarse_coords[i] + coarse_sizes[i];
    while (r < nr && ref_coords[r] < limit) corners.push_back(ref_coords[r++]);
  }
  // sizes are the corner differences; the last cell ends where the coarse
  // domain ends (:53-71)
  fine_sizes.assign(corners.size(), 0.0);
  for (size_t k = 0; k + 1 < corners.size(); ++k) fine_sizes[k] = corners[k + 1] - corners[k];
  double last = coarse_sizes[ncoarse - 1];
  if (r > 0) last += coarse_coords[ncoarse - 1] - corners.back();
  if (!(last > 0.0)) return 1;
  fine_sizes.back() = last;
  return 0;
}

void refine_ranges(int ncoarse, const double *coarse_sizes, int nfine, const double *fine_sizes,
                   int *begin, int *end, int *owner) {
  std::fill(owner, owner + nfine, -1);
  int start = 0;
  for (int i = 0; i < ncoarse; ++i) {
    double covered = 0.0;
    int stop = start;
    while (covered < coarse_sizes[i] && stop < nfine) covered += fine_sizes[stop++];
    begin[i] = start;
    end[i] = stop;
    for (int f = start; f < stop; ++f) owner[f] = i;
    start = stop;
  }
}

namespace {

constexpr int kThreads = 256;

// Projection: one warp per refined (x, y) row, lanes along z.  A row needs
// only its two owner lookups and one coarse row pointer; when a row has at
// most 32 lane items (cells, or cell pairs) each lane keeps its z owners in
// registers for the whole kernel, and a warp gathers four rows before it
// stores them, so four rows of loads are in flight.
// PAIRS: the host has checked that every row starts on a 16-byte boundary
// (even row length, even model stride, aligned base), so a lane writes two
// cells with one streaming 16-byte store (evict-first: this pass does not
// read the refined values again).
template <bool PAIRS>
__global__ void __launch_bounds__(kThreads)
k_refine_project(RefineMaps m, int nmb, int nblock, int nextra, const double *__restrict__ coarse,
                 double *__restrict__ fine, long long cngrid, long long fngrid) {
  constexpr int R = 4;
  const long long ldc = nblock * cngrid + nextra, ldf = nblock * fngrid + nextra;
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * (unsigned)blockDim.x) >> 5);
  const int fn1 = m.fn[1], fn2 = m.fn[2], cn1 = m.cn[1], cn2 = m.cn[2];
  const int nrows = m.fn[0] * fn1;
  const int items = PAIRS ? fn2 >> 1 : fn2;
  const int *__restrict__ ozv = m.owner[2];
  const bool lane_owned = items <= 32;
  int oz0 = -1, oz1 = -1;
  if (lane_owned && lane < items) {
    oz0 = ozv[PAIRS ? 2 * lane : lane];
    if (PAIRS) oz1 = ozv[2 * lane + 1];
  }
  for (int mb = blockIdx.y; mb < nmb; mb += gridDim.y) {
    const int model = mb / nblock, blk = mb - model * nblock;
    const double *src = coarse + model * ldc + blk * cngrid;
    double *dst = fine + model * ldf + blk * fngrid;
    if (lane_owned) {
      for (int row0 = warp * R; row0 < nrows; row0 += nwarps * R) {
        double a[R], b[R];
        unsigned ok = 0;  // rows with a coarse cell, one bit each
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int row = row0 + r;
          a[r] = b[r] = 0.0;
          if (row < nrows) {
            const int fi = row / fn1, fj = row - fi * fn1;
            const int ox = m.owner[0][fi], oy = m.owner[1][fj];
            if (ox >= 0 && oy >= 0 && lane < items) {
              const double *s = src + ((long long)ox * cn1 + oy) * cn2;
              ok |= 1u << r;
              if (oz0 >= 0) a[r] = s[oz0];
              if (PAIRS && oz1 >= 0) b[r] = s[oz1];
            }
          }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (!(ok >> r & 1u)) continue;
          double *d = dst + (long long)(row0 + r) * fn2;
          if (PAIRS) {
            if (oz0 >= 0 && oz1 >= 0) {
              __stcs(reinterpret_cast<double2 *>(d) + lane, make_double2(a[r], b[r]));
            } else {
              if (oz0 >= 0) d[2 * lane] = a[r];
              if (oz1 >= 0) d[2 * lane + 1] = b[r];
            }
          } else if (oz0 >= 0) {
            __stcs(d + lane, a[r]);
          }
        }
      }
    } else {
      for (int row = warp; row < nrows; row += nwarps) {
        const int fi = row / fn1, fj = row - fi * fn1;
        const int ox = m.owner[0][fi], oy = m.owner[1][fj];
        if (ox < 0 || oy < 0) continue;
        const double *s = src + ((long long)ox * cn1 + oy) * cn2;
        double *d = dst + (long long)row * fn2;
        for (int k = lane; k < fn2; k += 32) {
          const int oz = ozv[k];
          if (oz >= 0) d[k] = s[oz];
        }
      }
    }
    if (blk == 0 && blockIdx.x == 0)
      for (int e = threadIdx.x; e < nextra; e += blockDim.x)
        fine[model * ldf + nblock * fngrid + e] = coarse[model * ldc + nblock * cngrid + e];
  }
}

// 0.0 + v without the FP64 pipe: v itself, except that -0.0 becomes +0.0
// (the first add of a sum that starts at 0.0, as CombineValues' does).
__device__ __forceinline__ double zero_plus(double v) {
  return (__double_as_longlong(v) << 1) == 0 ? 0.0 : v;
}

// Combination: one warp per coarse (x, y) row, lanes along coarse z.  The
// refined rows (i, j) of the coarse row are warp-uniform and are walked in x,
// then y order; each lane adds its z run of every row in z order -- so each
// coarse sum is the reference's x, y, z sequence (CombineValues,
// ModelRefiner.cpp:114-122), bit for bit.  The adds run on GB300's narrow
// FP64 pipe, which bounds this kernel: each (row, z slot) costs one warp-wide
// add, so KR > 0 unrolls the z run to exactly its longest length, the first
// add of every sum (onto 0.0) is done with integer operations, and the loads
// of RB rows are issued before their adds.  KR = 0 runs any length.
template <int KR>
__global__ void __launch_bounds__(kThreads)
k_refine_combine(RefineMaps m, int nmb, int nblock, int nextra, const double *__restrict__ fine,
                 double *__restrict__ coarse, long long cngrid, long long fngrid) {
  constexpr int RB = KR == 0 ? 1 : (KR <= 2 ? 4 : 2);
  constexpr int KU = KR == 0 ? 1 : KR;
  const long long ldc = nblock * cngrid + nextra, ldf = nblock * fngrid + nextra;
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * (unsigned)blockDim.x) >> 5);
  const int fn1 = m.fn[1], fn2 = m.fn[2], cn1 = m.cn[1], cn2 = m.cn[2];
  const int crows = m.cn[0] * cn1;
  const long long rstride = (long long)fn1 * fn2;
  for (int mb = blockIdx.y; mb < nmb; mb += gridDim.y) {
    const int model = mb / nblock, blk = mb - model * nblock;
    const double *src = fine + model * ldf + blk * fngrid;
    double *dst = coarse + model * ldc + blk * cngrid;
    for (int crow = warp; crow < crows; crow += nwarps) {
      const int ci = crow / cn1, cj = crow - ci * cn1;
      const int i0 = m.begin[0][ci], ni = m.end[0][ci] - i0;
      const int j0 = m.begin[1][cj], nj = m.end[1][cj] - j0;
      const int nr = ni * nj;
      const double *row00 = src + ((long long)i0 * fn1 + j0) * fn2;
      for (int ck0 = 0; ck0 < cn2; ck0 += 32) {
        const int ck = ck0 + lane;
        int k0 = 0, nk = 0;
        if (ck < cn2) {
          k0 = m.begin[2][ck];
          nk = m.end[2][ck] - k0;
        }
        double sum = 0.0;
        if (KR == 0) {
          int i = 0, j = 0;
          bool first = true;
          for (int r = 0; r < nr; ++r) {
            const double *p = row00 + i * rstride + (long long)j * fn2 + k0;
            for (int u = 0; u < nk; ++u) {
              sum = first ? zero_plus(p[u]) : sum + p[u];
              first = false;
            }
            if (++j == nj) j = 0, ++i;
          }
        } else if (nr > 0) {
          // the first refined row: its first value starts the sum
          {
            double v[KU];
#pragma unroll
            for (int u = 0; u < KU; ++u)
              if (u < nk) v[u] = row00[k0 + u];
            if (nk > 0) sum = zero_plus(v[0]);
#pragma unroll
            for (int u = 1; u < KU; ++u)
              if (u < nk) sum += v[u];
          }
          int i = nj == 1 ? 1 : 0, j = nj == 1 ? 0 : 1;
          for (int r0 = 1; r0 < nr; r0 += RB) {
            double v[RB][KU];
#pragma unroll
            for (int r = 0; r < RB; ++r) {
              if (r0 + r < nr) {
                const double *p = row00 + i * rstride + (long long)j * fn2 + k0;
#pragma unroll
                for (int u = 0; u < KU; ++u)
                  if (u < nk) v[r][u] = p[u];
                if (++j == nj) j = 0, ++i;
              }
            }
#pragma unroll
            for (int r = 0; r < RB; ++r)
              if (r0 + r < nr) {
#pragma unroll
                for (int u = 0; u < KU; ++u)
                  if (u < nk) sum += v[r][u];
              }
          }
        }
        if (ck < cn2) dst[(long long)crow * cn2 + ck] = sum;
      }
    }
    if (blk == 0 && blockIdx.x == 0)
      for (int e = threadIdx.x; e < nextra; e += blockDim.x)
        coarse[model * ldc + nblock * cngrid + e] = fine[model * ldf + nblock * fngrid + e];
  }
}

dim3 grid_for(long long work_blocks, int nmb) {
  const int gy = std::min(nmb, 65535);
  // enough CTAs for several waves over 152 SMs, spread across the models
  const long long cap = std::max<long long>(4, 152LL * 32 / gy);
  return dim3((unsigned)std::max<long long>(1, std::min(work_blocks, cap)), (unsigned)gy);
}

}  // namespace

cudaError_t launch_refine_project(const RefineMaps &m, int nmodels, int nblock, int nextra,
                                  const double *coarse, double *fine, cudaStream_t st) {
  const long long cngrid = (long long)m.cn[0] * m.cn[1] * m.cn[2];
  const long long fngrid = (long long)m.fn[0] * m.fn[1] * m.fn[2];
  const int nmb = nmodels * nblock;
  if (nmb <= 0) return cudaSuccess;
  const long long rows = (long long)m.fn[0] * m.fn[1];
  const dim3 grid = grid_for((rows + kThreads / 32 - 1) / (kThreads / 32), nmb);
  // every row start (model stride, block stride, row length) on 16 bytes
  const long long ldf = (long long)nblock * fngrid + nextra;
  const bool pairs = (reinterpret_cast<uintptr_t>(fine) % 16 == 0) && m.fn[2] % 2 == 0 &&
                     (nmodels == 1 || ldf % 2 == 0);
  if (pairs)
    k_refine_project<true><<<grid, kThreads, 0, st>>>(m, nmb, nblock, nextra, coarse, fine,
                                                      cngrid, fngrid);
  else
    k_refine_project<false><<<grid, kThreads, 0, st>>>(m, nmb, nblock, nextra, coarse, fine,
                                                       cngrid, fngrid);
  return cudaGetLastError();
}

cudaError_t launch_refine_combine(const RefineMaps &m, int nmodels, int nblock, int nextra,
                                  const double *fine, double *coarse, cudaStream_t st) {
  const long long cngrid = (long long)m.cn[0] * m.cn[1] * m.cn[2];
  const long long fngrid = (long long)m.fn[0] * m.fn[1] * m.fn[2];
  const int nmb = nmodels * nblock;
  if (nmb <= 0) return cudaSuccess;
  const long long crows = (long long)m.cn[0] * m.cn[1];
  const dim3 grid = grid_for((crows + kThreads / 32 - 1) / (kThreads / 32), nmb);
  const int zr = m.zrun_max;
  if (zr <= 1)
    k_refine_combine<1><<<grid, kThreads, 0, st>>>(m, nmb, nblock, nextra, fine, coarse, cngrid,
                                                   fngrid);
  else if (zr <= 2)
    k_refine_combine<2><<<grid, kThreads, 0, st>>>(m, nmb, nblock, nextra, fine, coarse, cngrid,
                                                   fngrid);
  else if (zr <= 3)
    k_refine_combine<3><<<grid, kThreads, 0, st>>>(m, nmb, nblock, nextra, fine, coarse, cngrid,
                                                   fngrid);
  else if (zr <= 4)
    k_refine_combine<4><<<grid, kThreads, 0, st>>>(m, nmb, nblock, nextra, fine, coarse, cngrid,
                                                   fngrid);
  else
    k_refine_combine<0><<<grid, kThreads, 0, st>>>(m, nmb, nblock, nextra, fine, coarse, cngrid,
                                                   fngrid);
  return cudaGetLastError();
}

}  // namespace j3g
