// GB300ModelRefiner.h -- jif3D's ModelRefiner (ModelBase/ModelRefiner.h:33-128)
// with the cell passes on a GB300 through the C ABI of libjif3d_gb300.so.
//
// Same interface and meaning as jif3D::ModelRefiner: Set{X,Y,Z}Coordinates
// take the refinement coordinates (the fine model's corners), RefineAxes
// builds the refined axes (RefineOneAxis, on the host), ProjectValues copies
// each coarse value onto its refined cells and CombineGradient sums a refined
// gradient over each coarse cell -- both on the device, bit-identical to the
// reference (the same FindEnd walk, the same x, y, z order of the adds).
// ThreeDModelObjective (Inversion/ThreeDModelObjective.h:73) holds its
// refiner by value; declaring that member as jif3D::GB300ModelRefiner is the
// whole change that moves its refinement onto the GPU.
//
// Inside a jif3D source tree the real jif3D headers are included; elsewhere
// define JIF3D_GB300_STANDALONE to use the stand-ins of jif3d_compat.h.
#pragma once

#include <string>
#include <vector>

#include "jif3d_gb300.h"

#ifdef JIF3D_GB300_STANDALONE
#include "jif3d_compat.h"
#else
#include "../Global/FatalException.h"
#include "../Global/VecMat.h"
#include "../ModelBase/ThreeDModelBase.h"
#endif

namespace jif3D {

namespace gb300_refine_detail {
#ifdef JIF3D_GB300_STANDALONE
inline const double *cells(const ThreeDModelBase &m) { return m.GetData().data(); }
inline double *cells(ThreeDModelBase &m) { return m.SetData().data(); }
inline void resize_cells(ThreeDModelBase &m, size_t nx, size_t ny, size_t nz) {
  m.SetData().resize(nx * ny * nz);
}
#else
inline const double *cells(const ThreeDModelBase &m) { return m.GetData().origin(); }
inline double *cells(ThreeDModelBase &m) { return m.SetData().origin(); }
inline void resize_cells(ThreeDModelBase &m, size_t nx, size_t ny, size_t nz) {
  m.SetData().resize(boost::extents[nx][ny][nz]);
}
#endif
}  // namespace gb300_refine_detail

class GB300ModelRefiner {
 public:
  typedef ThreeDModelBase::t3DModelDim t3DModelDim;

  explicit GB300ModelRefiner(int device = 0) : device_(device) {}
  ~GB300ModelRefiner() {
    if (ctx_) j3g_destroy(ctx_);
  }
  // copies get their own context (the reference's refiner is copied with the
  // objective function, ThreeDModelObjective.h:248 clone)
  GB300ModelRefiner(const GB300ModelRefiner &o)
      : refx_(o.refx_), refy_(o.refy_), refz_(o.refz_), device_(o.device_) {}
  GB300ModelRefiner &operator=(const GB300ModelRefiner &o) {
    if (this != &o) {
      refx_ = o.refx_, refy_ = o.refy_, refz_ = o.refz_, device_ = o.device_;
      if (ctx_) j3g_destroy(ctx_);
      ctx_ = nullptr;
      fine_key_.clear();
      coarse_key_.clear();
    }
    return *this;
  }

  void SetXCoordinates(const t3DModelDim &X) { refx_ = X; }
  void SetYCoordinates(const t3DModelDim &Y) { refy_ = Y; }
  void SetZCoordinates(const t3DModelDim &Z) { refz_ = Z; }

  // RefineAxes (ModelRefiner.cpp:74-90): the refined cell sizes of the three
  // axes; the refined model's data are resized, their values left as they are.
  void RefineAxes(const ThreeDModelBase &InputModel, ThreeDModelBase &RefinedModel) {
    RefinedModel.SetXCellSizes(RefineOneAxis(InputModel.GetXCoordinates(),
                                             InputModel.GetXCellSizes(), refx_));
    RefinedModel.SetYCellSizes(RefineOneAxis(InputModel.GetYCoordinates(),
                                             InputModel.GetYCellSizes(), refy_));
    RefinedModel.SetZCellSizes(RefineOneAxis(InputModel.GetZCoordinates(),
                                             InputModel.GetZCellSizes(), refz_));
    gb300_refine_detail::resize_cells(RefinedModel, RefinedModel.GetXCellSizes().size(),
                                      RefinedModel.GetYCellSizes().size(),
                                      RefinedModel.GetZCellSizes().size());
  }
  // ProjectValues (:124-168) on the device.
  void ProjectValues(const ThreeDModelBase &InputModel, ThreeDModelBase &RefinedModel) {
    Prepare(InputModel, RefinedModel);
    Check(j3g_refine_project(ctx_, 1, gb300_refine_detail::cells(InputModel),
                             gb300_refine_detail::cells(RefinedModel)),
          "j3g_refine_project");
  }
  void RefineModel(const ThreeDModelBase &InputModel, ThreeDModelBase &RefinedModel) {
    RefineAxes(InputModel, RefinedModel);
    ProjectValues(InputModel, RefinedModel);
  }
  // CombineGradient (:170-218) on the device.
  rvec CombineGradient(const rvec &FineGradient, const ThreeDModelBase &CoarseModel,
                       const ThreeDModelBase &RefinedModel) {
    Prepare(CoarseModel, RefinedModel);
    const size_t nfine = RefinedModel.GetXCellSizes().size() *
                         RefinedModel.GetYCellSizes().size() *
                         RefinedModel.GetZCellSizes().size();
    if (FineGradient.size() != nfine)
      throw FatalException("Fine gradient does not match the refined model", __FILE__,
                           __LINE__);
    std::vector<double> fine(FineGradient.begin(), FineGradient.end());
    const size_t ncoarse = CoarseModel.GetXCellSizes().size() *
                           CoarseModel.GetYCellSizes().size() *
                           CoarseModel.GetZCellSizes().size();
    std::vector<double> out(ncoarse);
    Check(j3g_refine_combine(ctx_, 1, fine.data(), out.data()), "j3g_refine_combine");
    rvec CoarseGradient(ncoarse);
    for (size_t i = 0; i < ncoarse; ++i) CoarseGradient(i) = out[i];
    return CoarseGradient;
  }

 private:
  static t3DModelDim RefineOneAxis(const t3DModelDim &coords, const t3DModelDim &sizes,
                                   const t3DModelDim &ref) {
    t3DModelDim out(sizes.size() + ref.size());
    int n = 0;
    const int rc = j3g_refine_axis((int)sizes.size(), coords.data(), sizes.data(),
                                   (int)ref.size(), ref.data(), (int)out.size(), out.data(), &n);
    if (rc != J3G_OK) {
      if (n < 0)
        throw FatalException("Negative cell size in model refinement !", __FILE__, __LINE__);
      throw FatalException("Model refinement: no refinement coordinates or an empty axis",
                           __FILE__, __LINE__);
    }
    out.resize(n);
    return out;
  }
  static std::vector<double> Key(const ThreeDModelBase &m) {
    std::vector<double> k(m.GetXCellSizes().begin(), m.GetXCellSizes().end());
    k.push_back(-1.0);
    k.insert(k.end(), m.GetYCellSizes().begin(), m.GetYCellSizes().end());
    k.push_back(-1.0);
    k.insert(k.end(), m.GetZCellSizes().begin(), m.GetZCellSizes().end());
    return k;
  }
  // the context's mesh is the refined grid, its refinement the coarse grid;
  // both are set again only when the cell sizes change
  void Prepare(const ThreeDModelBase &Coarse, const ThreeDModelBase &Refined) {
    if (!ctx_) {
      if (j3g_create(&ctx_, device_) != J3G_OK) {
        ctx_ = nullptr;
        throw FatalException("j3g_create failed (a CUDA device is required)", __FILE__,
                             __LINE__);
      }
    }
    const std::vector<double> fk = Key(Refined), ck = Key(Coarse);
    if (fk != fine_key_) {
      const t3DModelDim &X = Refined.GetXCoordinates(), &Y = Refined.GetYCoordinates(),
                        &Z = Refined.GetZCoordinates();
      Check(j3g_set_mesh(ctx_, (int)Refined.GetXCellSizes().size(),
                         (int)Refined.GetYCellSizes().size(), (int)Refined.GetZCellSizes().size(),
                         X.data(), Y.data(), Z.data(), Refined.GetXCellSizes().data(),
                         Refined.GetYCellSizes().data(), Refined.GetZCellSizes().data()),
            "j3g_set_mesh");
      fine_key_ = fk;
      coarse_key_.clear();
    }
    if (ck != coarse_key_) {
      Check(j3g_set_refinement(ctx_, (int)Coarse.GetXCellSizes().size(),
                               (int)Coarse.GetYCellSizes().size(),
                               (int)Coarse.GetZCellSizes().size(), Coarse.GetXCellSizes().data(),
                               Coarse.GetYCellSizes().data(), Coarse.GetZCellSizes().data()),
            "j3g_set_refinement");
      coarse_key_ = ck;
    }
  }
  void Check(int rc, const char *what) {
    if (rc != J3G_OK) {
      const char *msg = ctx_ ? j3g_last_error(ctx_) : nullptr;
      throw FatalException(std::string(what) + ": " + (msg && *msg ? msg : j3g_status_string(rc)),
                           __FILE__, __LINE__);
    }
  }

  t3DModelDim refx_, refy_, refz_;
  int device_ = 0;
  j3g_context *ctx_ = nullptr;
  std::vector<double> fine_key_, coarse_key_;
};

}  // namespace jif3D
