// Model refinement between an inversion (coarse) grid and the forward grid:
// the axis refinement and the cell walks on the host, the projection of cell
// values and the combination of gradients on the device
// (ModelBase/ModelRefiner.cpp:17-218).
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace j3g {

// RefineOneAxis (ModelBase/ModelRefiner.cpp:17-72).  coarse_coords holds
// ncoarse + 1 corners, ref_coords nref values of which the last is not used
// (the reference walks size() - 1 of them).  Returns 0, or 1 when the last
// refined cell has a non-positive size.
int refine_axis(int ncoarse, const double *coarse_coords, const double *coarse_sizes, int nref,
                const double *ref_coords, std::vector<double> &fine_sizes);

// The walk of FindEnd (ModelRefiner.cpp:92-102) as ProjectValues and
// CombineGradient run it along one axis (:136-167): coarse cell i covers
// refined cells [begin[i], end[i]), taken in order until their summed sizes
// reach the coarse size.  owner[f] is the coarse cell of refined cell f, or
// -1 for a refined cell past the last range.
void refine_ranges(int ncoarse, const double *coarse_sizes, int nfine, const double *fine_sizes,
                   int *begin, int *end, int *owner);

// Device view of the three axes' walks (int arrays on the device).
struct RefineMaps {
  const int *owner[3];  // per refined index along x, y, z
  const int *begin[3];  // per coarse index
  const int *end[3];
  int cn[3];            // coarse cells per axis
  int fn[3];            // refined cells per axis
  int zrun_max;         // longest z run of refined cells of one coarse cell
};

// ProjectValues (:124-168) for nmodels models of nblock cell blocks followed
// by nextra extra parameters: refined[.] = coarse[owner]; refined cells that
// no coarse cell covers are not written; the extra parameters are copied.
cudaError_t launch_refine_project(const RefineMaps &m, int nmodels, int nblock, int nextra,
                                  const double *coarse, double *fine, cudaStream_t st);
// CombineGradient (:170-218): coarse[c] = sum over its refined cells in x, y,
// z order (FP64, the reference's order, so bit-identical); extras copied.
cudaError_t launch_refine_combine(const RefineMaps &m, int nmodels, int nblock, int nextra,
                                  const double *fine, double *coarse, cudaStream_t st);

}  // namespace j3g
