// GB300DeviceSensitivityCalculator.h -- a jif3D calculator that keeps the
// sensitivity matrix in GPU memory (HBM) across calls: the device twin of
// FullSensitivityGravMagCalculator (GravMag/FullSensitivityGravMagCalculator.h
// :33-221) over the caching logic of CachedGravMagCalculator
// (GravMag/CachedGravMagCalculator.h:28-143).
//
//   first call on a geometry   FP64 box terms through the implementation
//                              object (as the reference's first call), then
//                              j3g_build_sensitivity keeps J on the device;
//   later calls                d = T(J m) and 2 J^T (T' r) with the stored J
//                              (FP32 streaming or fp16 hi / lo tensor-core
//                              products, relative error <= 1e-6), no box terms.
//
// The cache key is the whole geometry -- cell sizes, origin, background
// thicknesses, kind, transform and the station positions -- held by the
// implementation's context, which drops J when any of them changes.  (The
// reference's GridBackgroundModelCache compares the model grid but not the
// stations, ModelBase/GridBackgroundModelCache.h:37-85, so its cached
// result can belong to other stations.)  Model values are not part of the
// key: J does not depend on them.
//
// CalculateBatch / LQDerivativeBatch run many models of one geometry at once
// (rows of a parameter matrix), e.g. the trial models of a line search or
// Monte-Carlo samples; with J3G_STORE_F16X2 they are tensor-core products.
#pragma once

#include <memory>
#include <vector>

#include "GB300GravMagImplementation.h"

namespace jif3D {

namespace gb300_detail {
#ifdef JIF3D_GB300_STANDALONE
template <class T>
using shared = std::shared_ptr<T>;
#else
template <class T>
using shared = boost::shared_ptr<T>;
#endif
}  // namespace gb300_detail

template <class DataType>
class GB300DeviceSensitivityCalculator : public ThreeDGravMagCalculator<DataType> {
 public:
  typedef typename DataType::ModelType ModelType;
  typedef GB300GravMagImplementation<DataType> ImpType;

  // storage: J3G_STORE_FP32 (the default: one copy of J, streamed at HBM
  // speed, the right choice for one model per call) or J3G_STORE_F16X2
  // (J and its transpose as fp16 hi / lo, tensor-core products: the faster
  // choice for CalculateBatch / LQDerivativeBatch over many models).
  explicit GB300DeviceSensitivityCalculator(gb300_detail::shared<ImpType> imp,
                                            int storage = J3G_STORE_FP32)
      : ThreeDGravMagCalculator<DataType>(imp), imp_(imp), storage_(storage) {}

  virtual rvec Calculate(const ModelType &Model, const DataType &Data) override {
    this->CheckModelConsistency(Model);
    if (imp_->HasStoredSensitivity(Model, Data, storage_))
      return ToRvec(imp_->StoredForward(Params(Model), 1));
    // no host rows: the implementation computes the data only
    this->SetCurrentSensitivities().resize(0, 0);
    rvec result = imp_->Calculate(Model, Data, *this);
    imp_->BuildStoredSensitivity(storage_);
    return result;
  }

  virtual rvec LQDerivative(const ModelType &Model, const DataType &Data,
                            const rvec &Misfit) override {
    this->CheckModelConsistency(Model);
    if (!imp_->HasStoredSensitivity(Model, Data, storage_))
      return imp_->LQDerivative(Model, Data, Misfit);  // FP64 matrix-free
    CheckMisfit(Data, Misfit.size());
    return ToRvec(imp_->StoredLQDerivative(Params(Model), ToVector(Misfit), 1));
  }

  // Data of every row of Parameters ([nmodels][nparm]) on the geometry of
  // Model (whose own values are not used): [nmodels][nmeas * data per
  // station].  Builds J first if this geometry has none.
  rmat CalculateBatch(const ModelType &Model, const DataType &Data, const rmat &Parameters) {
    this->CheckModelConsistency(Model);
    const int n = Rows(Model, Parameters);
    Ensure(Model, Data);
    return ToRmat(imp_->StoredForward(Flatten(Parameters), n), n);
  }

  // Gradients [nmodels][nparm] of the rows of Misfits at the rows of
  // Parameters, on the geometry of Model.
  rmat LQDerivativeBatch(const ModelType &Model, const DataType &Data, const rmat &Parameters,
                         const rmat &Misfits) {
    this->CheckModelConsistency(Model);
    const int n = Rows(Model, Parameters);
    if (Misfits.size1() != (size_t)n)
      throw FatalException("One misfit row per model is needed", __FILE__, __LINE__);
    Ensure(Model, Data);
    CheckMisfit(Data, Misfits.size2());
    return ToRmat(imp_->StoredLQDerivative(Flatten(Parameters), Flatten(Misfits), n), n);
  }

  // No host rows are kept: J lives on the device only.
  virtual void HandleSensitivities(const size_t) override {}

 private:
  void Ensure(const ModelType &Model, const DataType &Data) {
    if (!imp_->HasStoredSensitivity(Model, Data, storage_)) imp_->BuildStoredSensitivity(storage_);
  }

  void CheckMisfit(const DataType &Data, size_t n) {
    if (n != Data.GetMeasPosX().size() * imp_->GetDataPerMeasurement())
      throw FatalException("Misfit does not have the size of the data", __FILE__, __LINE__);
  }

  static int Rows(const ModelType &Model, const rmat &Parameters) {
    if (Parameters.size2() != Model.GetNModelParm())
      throw FatalException("Parameter rows do not match the model's parameter count", __FILE__,
                           __LINE__);
    return (int)Parameters.size1();
  }

  static std::vector<double> Params(const ModelType &Model) {
    return gb300_detail::to_vector(Model.GetModelParameters());
  }
  static std::vector<double> ToVector(const rvec &v) { return gb300_detail::to_vector(v); }

  static std::vector<double> Flatten(const rmat &m) {
    std::vector<double> v(m.size1() * m.size2());
    for (size_t r = 0; r < m.size1(); ++r)
      for (size_t c = 0; c < m.size2(); ++c) v[r * m.size2() + c] = m(r, c);
    return v;
  }

  static rmat ToRmat(const std::vector<double> &v, int rows) {
    const size_t cols = rows ? v.size() / rows : 0;
    rmat m(rows, cols);
    for (size_t r = 0; r < (size_t)rows; ++r)
      for (size_t c = 0; c < cols; ++c) m(r, c) = v[r * cols + c];
    return m;
  }

  static rvec ToRvec(const std::vector<double> &v) {
    rvec r(v.size());
    for (size_t i = 0; i < v.size(); ++i) r(i) = v[i];
    return r;
  }

  gb300_detail::shared<ImpType> imp_;
  int storage_;
};

}  // namespace jif3D
