// Model refinement: axis refinement and cell walks (host), projection of
// cell values and combination of gradients (device).  The device passes are
// HBM-bound copies and sums; both follow the reference's index walk exactly,
// so their results are bit-identical to it.
#include <algorithm>

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

// One warp per refined (x, y) row: each lane writes every 32nd cell of the
// row from the coarse row its owners select (coalesced 8-byte stores; the
// coarse row is read through L1/L2).
__global__ void __launch_bounds__(kThreads)
k_refine_project(RefineMaps m, int nmb, int nblock, int nextra, const double *__restrict__ coarse,
                 double *__restrict__ fine, long long cngrid, long long fngrid) {
  const long long ldc = nblock * cngrid + nextra, ldf = nblock * fngrid + nextra;
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * (unsigned)blockDim.x) >> 5);
  const int nrows = m.fn[0] * m.fn[1];
  for (int mb = blockIdx.y; mb < nmb; mb += gridDim.y) {
    const int model = mb / nblock, blk = mb - model * nblock;
    const double *src = coarse + model * ldc + blk * cngrid;
    double *dst = fine + model * ldf + blk * fngrid;
    for (int row = warp; row < nrows; row += nwarps) {
      const int fi = row / m.fn[1], fj = row - fi * m.fn[1];
      const int ox = m.owner[0][fi], oy = m.owner[1][fj];
      if (ox < 0 || oy < 0) continue;
      const double *s = src + ((long long)ox * m.cn[1] + oy) * m.cn[2];
      double *d = dst + (long long)row * m.fn[2];
      for (int k = lane; k < m.fn[2]; k += 32) {
        const int oz = m.owner[2][k];
        if (oz >= 0) d[k] = s[oz];
      }
    }
    if (blk == 0 && blockIdx.x == 0)
      for (int e = threadIdx.x; e < nextra; e += blockDim.x)
        fine[model * ldf + nblock * fngrid + e] = coarse[model * ldc + nblock * cngrid + e];
  }
}

// One thread per coarse cell: the sum of its refined cells in x, y, z order
// (CombineValues, ModelRefiner.cpp:114-122).  Neighbouring threads read
// neighbouring z runs, so a warp's loads cover whole sectors over the loop.
__global__ void __launch_bounds__(kThreads)
k_refine_combine(RefineMaps m, int nmb, int nblock, int nextra, const double *__restrict__ fine,
                 double *__restrict__ coarse, long long cngrid, long long fngrid) {
  const long long ldc = nblock * cngrid + nextra, ldf = nblock * fngrid + nextra;
  const int cyz = m.cn[1] * m.cn[2];
  for (int mb = blockIdx.y; mb < nmb; mb += gridDim.y) {
    const int model = mb / nblock, blk = mb - model * nblock;
    const double *src = fine + model * ldf + blk * fngrid;
    double *dst = coarse + model * ldc + blk * cngrid;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < (int)cngrid;
         c += gridDim.x * blockDim.x) {
      const int ci = c / cyz, rem = c - ci * cyz;
      const int cj = rem / m.cn[2], ck = rem - cj * m.cn[2];
      const int i1 = m.end[0][ci], j0 = m.begin[1][cj], j1 = m.end[1][cj];
      const int k0 = m.begin[2][ck], k1 = m.end[2][ck];
      double sum = 0.0;
      for (int i = m.begin[0][ci]; i < i1; ++i)
        for (int j = j0; j < j1; ++j) {
          const double *p = src + ((long long)i * m.fn[1] + j) * m.fn[2];
          for (int k = k0; k < k1; ++k) sum += p[k];
        }
      dst[c] = sum;
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
  k_refine_project<<<grid, kThreads, 0, st>>>(m, nmb, nblock, nextra, coarse, fine, cngrid,
                                              fngrid);
  return cudaGetLastError();
}

cudaError_t launch_refine_combine(const RefineMaps &m, int nmodels, int nblock, int nextra,
                                  const double *fine, double *coarse, cudaStream_t st) {
  const long long cngrid = (long long)m.cn[0] * m.cn[1] * m.cn[2];
  const long long fngrid = (long long)m.fn[0] * m.fn[1] * m.fn[2];
  const int nmb = nmodels * nblock;
  if (nmb <= 0) return cudaSuccess;
  const dim3 grid = grid_for((cngrid + kThreads - 1) / kThreads, nmb);
  k_refine_combine<<<grid, kThreads, 0, st>>>(m, nmb, nblock, nextra, fine, coarse, cngrid,
                                              fngrid);
  return cudaGetLastError();
}

}  // namespace j3g
