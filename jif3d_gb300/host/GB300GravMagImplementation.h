// GB300GravMagImplementation.h -- jif3D implementation objects that run the
// gravity / FTG / magnetic prism path on a GB300 through the C ABI of
// libjif3d_gb300.so (include/jif3d_gb300.h).
//
// Drop-in for the implementation classes of jif3D's bridge
// (GravMag/ThreeDGravMagImplementation.h:39-84): the calculators
// (MinMem / Cached / FullSensitivityGravMagCalculator) and the objective /
// L-BFGS chain call them unchanged.  Calculate and LQDerivative are
// overridden as whole-survey calls (one launch over all stations instead of
// the base class's station loop); the per-station CalcGridded / CalcBackground
// that the base declares are implemented too, through a one-station context.
//
// Inside a jif3D source tree the real jif3D headers are included; elsewhere
// (tests, this repository) define JIF3D_GB300_STANDALONE to use the stand-in
// declarations of jif3d_compat.h.
//
// Transforms: jif3D's base class keeps its VectorTransform private and its
// SetDataTransform is not virtual, so an implementation cannot see which
// transform a calculator set -- only GetDataPerMeasurement.  Two routes:
//  * unchanged callers that set the transform through the calculator only
//    (Joint/SetupMagnetics.cpp:206, 254 and the like): the device computes
//    the raw data (and rows) of all stations in one call; Calculate then runs
//    the base class's station loop over them, so the base applies its own
//    transform and calls HandleSensitivities; LQDerivative back-projects each
//    station's misfit through the base class's own derivative loop (run on a
//    one-station survey and a model of `raw` parameters whose rows are the
//    identity, which yields 2 T_i'^T m_i), and the device forms 2 J^T of the
//    back-projected raw misfit.  A transform that keeps the number of data
//    per station (jif3D's only one for these data is CopyTransform, the
//    identity) is not visible and is not needed;
//  * SetGB300Transform names the transform to the device as well, which then
//    applies it in the fused epilogues (no per-station host work); Calculate
//    checks that both give the same number of data per station.  The
//    device-resident calculator needs this route.
#pragma once

#include <cstring>
#include <string>
#include <vector>

#include "jif3d_gb300.h"

#ifdef JIF3D_GB300_STANDALONE
#include "jif3d_compat.h"
#else
#include "../GravMag/ThreeDGravMagImplementation.h"
#include "../Global/FatalException.h"
#include "../Gravity/ScalarGravityData.h"
#include "../Gravity/TensorGravityData.h"
#include "../Magnetics/ThreeComponentMagneticData.h"
#include "../Magnetics/ThreeDMagnetizationModel.h"
#include "../Magnetics/TotalFieldMagneticData.h"
#endif

namespace jif3D {

namespace gb300_detail {
// Background layer thicknesses of a model; magnetisation models have no
// background parameters (Magnetics/ThreeDMagnetizationModel.h:66-69).
template <class M>
std::vector<double> background_thicknesses(const M &m) {
  return std::vector<double>(m.GetBackgroundThicknesses().begin(),
                             m.GetBackgroundThicknesses().end());
}
inline std::vector<double> background_thicknesses(const ThreeDMagnetizationModel &) {
  return std::vector<double>();
}
template <class V>
std::vector<double> to_vector(const V &v) {
  return std::vector<double>(v.begin(), v.end());
}
}  // namespace gb300_detail

template <class DataType>
class GB300GravMagImplementation : public ThreeDGravMagImplementation<DataType> {
 public:
  typedef typename DataType::ModelType ModelType;

  // kind: J3G_SCALAR, J3G_TENSOR, J3G_MAGNETIC, J3G_MAG_GRADIENT or
  // J3G_MAGNETIZATION; inclination / declination in radians, field strength
  // in nT (magnetic kinds).  The context is created on CUDA device `device`.
  GB300GravMagImplementation(int kind, double inclination = 0.0, double declination = 0.0,
                             double field_strength = 0.0, int device = 0)
      : kind_(kind), inc_(inclination), dec_(declination), fs_(field_strength),
        device_(device) {
    Check(nullptr, j3g_create(&ctx_, device_), "j3g_create");
    Check(ctx_, j3g_set_kind(ctx_, kind_, inc_, dec_, fs_), "j3g_set_kind");
  }
  virtual ~GB300GravMagImplementation() {
    if (ctx_) j3g_destroy(ctx_);
    if (one_) j3g_destroy(one_);
  }
  GB300GravMagImplementation(const GB300GravMagImplementation &) = delete;
  GB300GravMagImplementation &operator=(const GB300GravMagImplementation &) = delete;

  virtual size_t RawDataPerMeasurement() override {
    switch (kind_) {
      case J3G_SCALAR:
      case J3G_MAG_GRADIENT: return 1;
      case J3G_TENSOR: return 9;
      case J3G_JOINT: return 10;
      default: return 3;
    }
  }

  // Device data transform: J3G_T_NONE, J3G_T_FTG_INVARIANT (tensor),
  // J3G_T_TOTAL_FIELD or J3G_T_TFA (three-component magnetics, with the
  // anomaly direction's inclination / declination in radians).  Give the
  // calculator the matching jif3D transform (FTGInvariant, TotalField,
  // TotalFieldAnomaly).
  void SetGB300Transform(int transform, double inclination = 0.0, double declination = 0.0) {
    Check(ctx_, j3g_set_transform(ctx_, transform, inclination, declination),
          "j3g_set_transform");
    transform_ = transform;
    tinc_ = inclination;
    tdec_ = declination;
  }

  // ThreeDGravMagImplementation::Calculate (ThreeDGravMagImplementation.h:116-168)
  // for all stations in one call.  When the calculator's current-sensitivity
  // matrix is large enough (FullSensitivityGravMagCalculator), the raw rows of
  // every station are delivered through it and HandleSensitivities(i) is
  // called in station order, as the base class does.
  virtual rvec Calculate(const ModelType &Model, const DataType &Data,
                         ThreeDGravMagCalculator<DataType> &Calculator) override {
    Upload(ctx_, Model, Data, Data.GetMeasPosX().size(), 0);
    if (CalculatorTransformOnly()) return ServedCalculate(Model, Data, Calculator);
    CheckTransform();
    const size_t nmeas = Data.GetMeasPosX().size();
    const size_t raw = RawDataPerMeasurement();
    const size_t nparm = Model.GetNModelParm();
    const std::vector<double> params = gb300_detail::to_vector(Model.GetModelParameters());
    std::vector<double> out(nmeas * this->GetDataPerMeasurement());
    rmat &cur = Calculator.SetCurrentSensitivities();
    if (nmeas > 0 && cur.size1() >= raw && cur.size2() >= nparm) {
      std::vector<double> J(nmeas * raw * nparm);
      Check(ctx_, j3g_forward_sens(ctx_, params.data(), out.data(), J.data()), "j3g_forward_sens");
      for (size_t i = 0; i < nmeas; ++i) {
        for (size_t r = 0; r < raw; ++r)
          for (size_t c = 0; c < nparm; ++c) cur(r, c) = J[(i * raw + r) * nparm + c];
        Calculator.HandleSensitivities(i);
      }
    } else if (nmeas > 0) {
      Check(ctx_, j3g_forward(ctx_, params.data(), out.data()), "j3g_forward");
    }
    return ToRvec(out);
  }

  // ThreeDGravMagImplementation::LQDerivative (ThreeDGravMagImplementation.h:177-231):
  // 2 J^T (transform-derivative-weighted misfit), matrix-free on the device.
  virtual rvec LQDerivative(const ModelType &Model, const DataType &Data,
                            const rvec &Misfit) override {
    Upload(ctx_, Model, Data, Data.GetMeasPosX().size(), 0);
    const bool served = CalculatorTransformOnly();
    if (!served) CheckTransform();
    const size_t nmeas = Data.GetMeasPosX().size();
    if (Misfit.size() != nmeas * this->GetDataPerMeasurement())
      throw FatalException("Misfit does not have the size of the data", __FILE__, __LINE__);
    const std::vector<double> params = gb300_detail::to_vector(Model.GetModelParameters());
    const std::vector<double> misfit =
        served ? BackProjectedMisfit(params, Data, Misfit) : gb300_detail::to_vector(Misfit);
    std::vector<double> grad(Model.GetNModelParm());
    Check(ctx_, j3g_lqderivative(ctx_, params.data(), misfit.data(), grad.data()),
          "j3g_lqderivative");
    return ToRvec(grad);
  }

  // -- Device-resident sensitivities (GB300DeviceSensitivityCalculator) ----
  // Loads the model's geometry and the stations (nothing is sent when they
  // are unchanged; any change drops the stored J) and tells whether J is
  // held in HBM in `storage` (J3G_STORE_FP32 / J3G_STORE_F16X2) for them.
  bool HasStoredSensitivity(const ModelType &Model, const DataType &Data, int storage) {
    Upload(ctx_, Model, Data, Data.GetMeasPosX().size(), 0);
    CheckTransform();
    int have = 0;
    Check(ctx_, j3g_sensitivity_info(ctx_, &have, nullptr, nullptr, nullptr),
          "j3g_sensitivity_info");
    return have == storage;
  }
  // Builds J for the geometry last loaded by HasStoredSensitivity.
  void BuildStoredSensitivity(int storage) {
    Check(ctx_, j3g_build_sensitivity(ctx_, storage), "j3g_build_sensitivity");
  }
  // nmodels models [nmodels][nparm] -> data [nmodels][nmeas * data per
  // station] with the stored J (the geometry of the last
  // HasStoredSensitivity call).
  std::vector<double> StoredForward(const std::vector<double> &models, int nmodels) {
    int nmeas = 0, dpm = 0;
    Check(ctx_, j3g_get_sizes(ctx_, nullptr, nullptr, &nmeas, nullptr, &dpm), "j3g_get_sizes");
    std::vector<double> data((size_t)nmodels * nmeas * dpm);
    Check(ctx_, j3g_batched_forward(ctx_, nmodels, models.data(), data.data()),
          "j3g_batched_forward");
    return data;
  }
  // Gradients [nmodels][nparm] of the misfits [nmodels][nmeas * data per
  // station] at the models, with the stored J.
  std::vector<double> StoredLQDerivative(const std::vector<double> &models,
                                         const std::vector<double> &misfits, int nmodels) {
    long long nparm = 0;
    Check(ctx_, j3g_get_sizes(ctx_, nullptr, &nparm, nullptr, nullptr, nullptr), "j3g_get_sizes");
    std::vector<double> grads((size_t)nmodels * nparm);
    Check(ctx_, j3g_batched_lqderivative(ctx_, nmodels, models.data(), misfits.data(),
                                         grads.data()),
          "j3g_batched_lqderivative");
    return grads;
  }

 private:
  // What CalcGridded / CalcBackground return while the base class's loops
  // run over data computed beforehand (see ServedCalculate,
  // BackProjectedMisfit): nothing (the per-station contexts), the raw data
  // of each station (with its rows when the calculator keeps them), or one
  // station's raw data with identity rows.
  enum class Serve { kNone, kData, kRows, kUnit };

  // A transform was set through the calculator only: the base class's
  // GetDataPerMeasurement differs from the raw count and no device
  // transform was named.
  bool CalculatorTransformOnly() {
    return transform_ == J3G_T_NONE && this->GetDataPerMeasurement() != RawDataPerMeasurement();
  }

  // Calculate with the calculator's transform: the raw data (and rows) of
  // every station in one device call, then the base class's station loop
  // over them -- it applies its transform per station and calls
  // HandleSensitivities in station order (ThreeDGravMagImplementation.h:116-168).
  rvec ServedCalculate(const ModelType &Model, const DataType &Data,
                       ThreeDGravMagCalculator<DataType> &Calculator) {
    const size_t nmeas = Data.GetMeasPosX().size();
    const size_t raw = RawDataPerMeasurement();
    const size_t nparm = Model.GetNModelParm();
    const std::vector<double> params = gb300_detail::to_vector(Model.GetModelParameters());
    served_.assign(nmeas * raw, 0.0);
    rmat &cur = Calculator.SetCurrentSensitivities();
    const bool rows = cur.size1() >= raw && cur.size2() >= nparm;
    served_rows_.assign(rows ? nmeas * raw * nparm : 0, 0.0);
    served_nparm_ = nparm;
    if (nmeas > 0 && rows)
      Check(ctx_, j3g_forward_sens(ctx_, params.data(), served_.data(), served_rows_.data()),
            "j3g_forward_sens");
    else if (nmeas > 0)
      Check(ctx_, j3g_forward(ctx_, params.data(), served_.data()), "j3g_forward");
    ServeScope scope(this, rows ? Serve::kRows : Serve::kData);
    return ThreeDGravMagImplementation<DataType>::Calculate(Model, Data, Calculator);
  }

  // The raw-length misfit T_i'^T m_i of every station i for a transform set
  // through the calculator: the raw data from the device, then for each
  // station the base class's own LQDerivative on a one-station survey and a
  // model of `raw` parameters whose rows are the identity, which returns
  // 2 T_i'^T m_i (ThreeDGravMagImplementation.h:177-231).
  std::vector<double> BackProjectedMisfit(const std::vector<double> &params, const DataType &Data,
                                          const rvec &Misfit) {
    const size_t nmeas = Data.GetMeasPosX().size();
    const size_t raw = RawDataPerMeasurement(), dpm = this->GetDataPerMeasurement();
    served_.assign(nmeas * raw, 0.0);
    if (nmeas > 0) Check(ctx_, j3g_forward(ctx_, params.data(), served_.data()), "j3g_forward");
    ModelType unit;
    unit.SetMeshSize(raw, 1, 1);
    if (unit.GetNModelParm() != raw) unit.SetMeshSize(1, 1, 1);  // magnetisation: 3 blocks
    if (unit.GetNModelParm() != raw)
      throw FatalException("No model of the raw data size for the transform's derivative",
                           __FILE__, __LINE__);
    const std::vector<double> X = gb300_detail::to_vector(Data.GetMeasPosX()),
                              Y = gb300_detail::to_vector(Data.GetMeasPosY()),
                              Z = gb300_detail::to_vector(Data.GetMeasPosZ());
    std::vector<double> out(nmeas * raw);
    ServeScope scope(this, Serve::kUnit);
    rvec m(dpm);
    for (size_t i = 0; i < nmeas; ++i) {
      DataType one;
      one.AddMeasurementPoint(X[i], Y[i], Z[i]);
      for (size_t j = 0; j < dpm; ++j) m(j) = Misfit(i * dpm + j);
      serve_station_ = i;
      const rvec g = ThreeDGravMagImplementation<DataType>::LQDerivative(unit, one, m);
      for (size_t r = 0; r < raw; ++r) out[i * raw + r] = 0.5 * g(r);
    }
    return out;
  }

  struct ServeScope {
    GB300GravMagImplementation *imp;
    ServeScope(GB300GravMagImplementation *i, Serve mode) : imp(i) { imp->serve_ = mode; }
    ~ServeScope() {
      imp->serve_ = Serve::kNone;
      imp->served_rows_ = std::vector<double>();
    }
  };

  // Per-station parts of the base class's station loops: served from data
  // computed beforehand (above), or else through a context holding the one
  // station: the gridded response and rows (columns of the cell blocks), and
  // the background response and rows (columns ngrid..).
  virtual rvec CalcGridded(const size_t measindex, const ModelType &Model,
                           const DataType &Data, rmat &Sensitivities) override {
    if (serve_ != Serve::kNone) return Served(measindex, Sensitivities);
    return OneStation(measindex, Model, Data, Sensitivities, true);
  }
  virtual rvec CalcBackground(const size_t measindex, const double, const double,
                              const double, const ModelType &Model, const DataType &Data,
                              rmat &Sensitivities) override {
    if (serve_ != Serve::kNone) return rvec(RawDataPerMeasurement());  // in the gridded part
    return OneStation(measindex, Model, Data, Sensitivities, false);
  }

  rvec Served(size_t measindex, rmat &Sens) {
    const size_t raw = RawDataPerMeasurement();
    const size_t i = serve_ == Serve::kUnit ? serve_station_ : measindex;
    rvec out(raw);
    for (size_t r = 0; r < raw; ++r) out(r) = served_[i * raw + r];
    if (serve_ == Serve::kUnit) {
      for (size_t r = 0; r < raw; ++r)
        for (size_t c = 0; c < Sens.size2(); ++c) Sens(r, c) = r == c ? 1.0 : 0.0;
    } else if (serve_ == Serve::kRows && Sens.size1() >= raw && Sens.size2() >= served_nparm_) {
      const double *J = served_rows_.data() + i * raw * served_nparm_;
      for (size_t r = 0; r < raw; ++r)
        for (size_t c = 0; c < served_nparm_; ++c) Sens(r, c) = J[r * served_nparm_ + c];
    }
    return out;
  }

  rvec OneStation(size_t i, const ModelType &Model, const DataType &Data, rmat &Sens,
                  bool gridded) {
    if (!one_) {
      Check(nullptr, j3g_create(&one_, device_), "j3g_create");
      Check(one_, j3g_set_kind(one_, kind_, inc_, dec_, fs_), "j3g_set_kind");
    }
    Upload(one_, Model, Data, 1, i);
    long long ngrid = 0, nparm = 0;
    Check(one_, j3g_get_sizes(one_, &ngrid, &nparm, nullptr, nullptr, nullptr), "j3g_get_sizes");
    const long long ncell = nparm - (long long)gb300_detail::background_thicknesses(Model).size();
    std::vector<double> params = gb300_detail::to_vector(Model.GetModelParameters());
    // keep only the part asked for: cell blocks or background values
    for (long long c = 0; c < nparm; ++c)
      if ((c < ncell) != gridded) params[c] = 0.0;
    const size_t raw = RawDataPerMeasurement();
    std::vector<double> out(raw), J(raw * nparm);
    Check(one_, j3g_forward_sens(one_, params.data(), out.data(), J.data()), "j3g_forward_sens");
    if (Sens.size1() >= raw && Sens.size2() >= (size_t)nparm) {
      const long long c0 = gridded ? 0 : ncell, c1 = gridded ? ncell : nparm;
      for (size_t r = 0; r < raw; ++r)
        for (long long c = c0; c < c1; ++c) Sens(r, c) = J[r * nparm + c];
    }
    return ToRvec(out);
  }

  // Geometry, stations and transform of a context, re-sent only when they
  // change (the context drops its stored state on any change).
  void Upload(j3g_context *ctx, const ModelType &Model, const DataType &Data, size_t nst,
              size_t first) {
    Geometry g;
    g.xc = gb300_detail::to_vector(Model.GetXCoordinates());
    g.yc = gb300_detail::to_vector(Model.GetYCoordinates());
    g.zc = gb300_detail::to_vector(Model.GetZCoordinates());
    g.xs = gb300_detail::to_vector(Model.GetXCellSizes());
    g.ys = gb300_detail::to_vector(Model.GetYCellSizes());
    g.zs = gb300_detail::to_vector(Model.GetZCellSizes());
    g.bg = gb300_detail::background_thicknesses(Model);
    const std::vector<double> X = gb300_detail::to_vector(Data.GetMeasPosX()),
                              Y = gb300_detail::to_vector(Data.GetMeasPosY()),
                              Z = gb300_detail::to_vector(Data.GetMeasPosZ());
    if (first + nst > X.size())
      throw FatalException("Station index beyond the data", __FILE__, __LINE__);
    g.sx.assign(X.begin() + first, X.begin() + first + nst);
    g.sy.assign(Y.begin() + first, Y.begin() + first + nst);
    g.sz.assign(Z.begin() + first, Z.begin() + first + nst);
    g.transform = ctx == ctx_ ? transform_ : J3G_T_NONE;
    Geometry &have = ctx == ctx_ ? main_geo_ : one_geo_;
    if (have.valid && have == g) return;
    if (g.xs.size() + 1 != g.xc.size() || g.ys.size() + 1 != g.yc.size() ||
        g.zs.size() + 1 != g.zc.size())
      throw FatalException("Corner coordinates must have one value more than the cell sizes",
                           __FILE__, __LINE__);
    Check(ctx, j3g_set_mesh(ctx, (int)g.xs.size(), (int)g.ys.size(), (int)g.zs.size(),
                            g.xc.data(), g.yc.data(), g.zc.data(), g.xs.data(), g.ys.data(),
                            g.zs.data()),
          "j3g_set_mesh");
    Check(ctx, j3g_set_background(ctx, (int)g.bg.size(), g.bg.empty() ? nullptr : g.bg.data()),
          "j3g_set_background");
    Check(ctx, j3g_set_stations(ctx, (int)nst, g.sx.data(), g.sy.data(), g.sz.data()),
          "j3g_set_stations");
    Check(ctx, j3g_set_transform(ctx, g.transform, tinc_, tdec_), "j3g_set_transform");
    g.valid = true;
    have = g;
  }

  void CheckTransform() {
    int dpm = 0;
    Check(ctx_, j3g_get_sizes(ctx_, nullptr, nullptr, nullptr, nullptr, &dpm), "j3g_get_sizes");
    if ((size_t)dpm != this->GetDataPerMeasurement())
      throw FatalException(
          "The calculator's data transform and SetGB300Transform give different numbers of data "
          "per station",
          __FILE__, __LINE__);
  }

  static rvec ToRvec(const std::vector<double> &v) {
    rvec r(v.size());
    for (size_t i = 0; i < v.size(); ++i) r(i) = v[i];
    return r;
  }

  static void Check(j3g_context *ctx, int rc, const char *what) {
    if (rc == J3G_OK) return;
    std::string msg = std::string(what) + ": " + j3g_status_string(rc);
    if (ctx && j3g_last_error(ctx)[0]) msg += std::string(" (") + j3g_last_error(ctx) + ")";
    throw FatalException(msg, __FILE__, __LINE__);
  }

  struct Geometry {
    std::vector<double> xc, yc, zc, xs, ys, zs, bg, sx, sy, sz;
    int transform = J3G_T_NONE;
    bool valid = false;
    bool operator==(const Geometry &o) const {
      return xc == o.xc && yc == o.yc && zc == o.zc && xs == o.xs && ys == o.ys && zs == o.zs &&
             bg == o.bg && sx == o.sx && sy == o.sy && sz == o.sz && transform == o.transform;
    }
  };

  int kind_;
  double inc_, dec_, fs_;
  int device_;
  int transform_ = J3G_T_NONE;
  double tinc_ = 0.0, tdec_ = 0.0;
  j3g_context *ctx_ = nullptr;  // all stations
  j3g_context *one_ = nullptr;  // one station (CalcGridded / CalcBackground)
  Geometry main_geo_, one_geo_;
  Serve serve_ = Serve::kNone;
  std::vector<double> served_, served_rows_;  // raw data [nmeas][raw], rows [nmeas][raw][nparm]
  size_t served_nparm_ = 0, serve_station_ = 0;
};

// Replaces ScalarOMPGravityImp / ScalarCudaGravityImp.
class ScalarGB300GravityImp : public GB300GravMagImplementation<ScalarGravityData> {
 public:
  explicit ScalarGB300GravityImp(int device = 0)
      : GB300GravMagImplementation<ScalarGravityData>(J3G_SCALAR, 0.0, 0.0, 0.0, device) {}
};

// Replaces TensorOMPGravityImp / TensorCudaGravityImp.
class TensorGB300GravityImp : public GB300GravMagImplementation<TensorGravityData> {
 public:
  explicit TensorGB300GravityImp(int device = 0)
      : GB300GravMagImplementation<TensorGravityData>(J3G_TENSOR, 0.0, 0.0, 0.0, device) {}
};

// Replaces OMPMagneticSusceptibilityImp(Inc, Dec, Fs) (three raw components).
class GB300MagneticSusceptibilityImp
    : public GB300GravMagImplementation<TotalFieldMagneticData> {
 public:
  GB300MagneticSusceptibilityImp(double Inc = 0.0, double Dec = 0.0, double Fs = 1.0,
                                 int device = 0)
      : GB300GravMagImplementation<TotalFieldMagneticData>(J3G_MAGNETIC, Inc, Dec, Fs, device) {}
};

// Replaces OMPMagneticGradImp(Inc, Dec, Fs): Bz(z) - Bz(z + 1 m).
class GB300MagneticGradImp : public GB300GravMagImplementation<TotalFieldMagneticData> {
 public:
  GB300MagneticGradImp(double Inc = 0.0, double Dec = 0.0, double Fs = 1.0, int device = 0)
      : GB300GravMagImplementation<TotalFieldMagneticData>(J3G_MAG_GRADIENT, Inc, Dec, Fs,
                                                           device) {}
};

// Replaces OMPMagnetizationImp (three magnetisation blocks).
class GB300MagnetizationImp : public GB300GravMagImplementation<ThreeComponentMagneticData> {
 public:
  explicit GB300MagnetizationImp(int device = 0)
      : GB300GravMagImplementation<ThreeComponentMagneticData>(J3G_MAGNETIZATION, 0.0, 0.0, 0.0,
                                                               device) {}
};

}  // namespace jif3D
