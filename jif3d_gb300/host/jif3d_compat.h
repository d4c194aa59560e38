// jif3d_compat.h -- minimal stand-ins for the jif3D declarations that
// GB300GravMagImplementation.h uses, for building it outside a jif3D source
// tree (jif3D itself needs Boost and NetCDF).  Same class and member names as
// jif3D so that the implementation header compiles unchanged against either;
// only what the implementation and its tests touch is provided:
//   rvec / rmat                     (Global/VecMat.h)
//   FatalException                  (Global/FatalException.h)
//   VectorTransform + FTGInvariant, TotalField, TotalFieldAnomaly (sizes only)
//   ThreeDModelBase and the gravity / susceptibility / magnetisation models
//   the data classes with their ModelType
//   ThreeDGravMagCalculator, MinMemGravMagCalculator,
//   FullSensitivityGravMagCalculator (host-stored rows, FP64 products)
//   ThreeDGravMagImplementation with the generic per-station loop
//     (GravMag/ThreeDGravMagImplementation.h:116-168), so that the
//     per-station overrides can be exercised
#pragma once

#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

namespace jif3D {

class rvec {
 public:
  rvec() {}
  explicit rvec(size_t n, double v = 0.0) : d_(n, v) {}
  size_t size() const { return d_.size(); }
  double &operator()(size_t i) { return d_[i]; }
  double operator()(size_t i) const { return d_[i]; }
  double &operator[](size_t i) { return d_[i]; }
  double operator[](size_t i) const { return d_[i]; }
  std::vector<double>::const_iterator begin() const { return d_.begin(); }
  std::vector<double>::const_iterator end() const { return d_.end(); }

 private:
  std::vector<double> d_;
};

class rmat {
 public:
  rmat() {}
  rmat(size_t r, size_t c) : r_(r), c_(c), d_(r * c, 0.0) {}
  size_t size1() const { return r_; }
  size_t size2() const { return c_; }
  void resize(size_t r, size_t c) {
    r_ = r;
    c_ = c;
    d_.assign(r * c, 0.0);
  }
  double &operator()(size_t i, size_t j) { return d_[i * c_ + j]; }
  double operator()(size_t i, size_t j) const { return d_[i * c_ + j]; }

 private:
  size_t r_ = 0, c_ = 0;
  std::vector<double> d_;
};

class FatalException : public std::runtime_error {
 public:
  FatalException(const std::string &what, const std::string &file = std::string(), int line = 0)
      : std::runtime_error(what + (file.empty() ? "" : " (" + file + ":" + std::to_string(line) + ")")) {}
};

class VectorTransform {
 public:
  virtual ~VectorTransform() {}
  virtual size_t GetInputSize() const = 0;
  virtual size_t GetOutputSize() const = 0;
};
class FTGInvariant : public VectorTransform {
 public:
  size_t GetInputSize() const override { return 9; }
  size_t GetOutputSize() const override { return 1; }
};
class TotalField : public VectorTransform {
 public:
  size_t GetInputSize() const override { return 3; }
  size_t GetOutputSize() const override { return 1; }
};
class TotalFieldAnomaly : public VectorTransform {
 public:
  size_t GetInputSize() const override { return 3; }
  size_t GetOutputSize() const override { return 1; }
};

// Rectilinear mesh: origin + cell sizes, corner coordinates as running sums
// (ModelBase/ThreeDModelBase.cpp:96-113), values z fastest.
// The cell values are one flat block, z fastest (the reference keeps a
// boost::multi_array, ThreeDModelBase.h:49-51, 119-128).
class ThreeDModelBase {
 public:
  typedef std::vector<double> t3DModelDim;
  typedef std::vector<double> t3DModelData;
  virtual ~ThreeDModelBase() {}
  void SetMesh(const std::vector<double> &xs, const std::vector<double> &ys,
               const std::vector<double> &zs, double x0, double y0, double z0) {
    xs_ = xs;
    ys_ = ys;
    zs_ = zs;
    xc_ = Coords(x0, xs);
    yc_ = Coords(y0, ys);
    zc_ = Coords(z0, zs);
  }
  // the origin stays, the corners are recomputed (ThreeDModelBase.h:74-90)
  void SetXCellSizes(const t3DModelDim &v) { xs_ = v, xc_ = Coords(Origin(xc_), v); }
  void SetYCellSizes(const t3DModelDim &v) { ys_ = v, yc_ = Coords(Origin(yc_), v); }
  void SetZCellSizes(const t3DModelDim &v) { zs_ = v, zc_ = Coords(Origin(zc_), v); }
  t3DModelData &SetData() { return data_; }
  const t3DModelData &GetData() const { return data_; }
  size_t GetNModelElements() const { return data_.size(); }
  const std::vector<double> &GetXCellSizes() const { return xs_; }
  const std::vector<double> &GetYCellSizes() const { return ys_; }
  const std::vector<double> &GetZCellSizes() const { return zs_; }
  const std::vector<double> &GetXCoordinates() const { return xc_; }
  const std::vector<double> &GetYCoordinates() const { return yc_; }
  const std::vector<double> &GetZCoordinates() const { return zc_; }
  size_t NCells() const { return xs_.size() * ys_.size() * zs_.size(); }

 private:
  static double Origin(const std::vector<double> &c) { return c.empty() ? 0.0 : c[0]; }
  static std::vector<double> Coords(double o, const std::vector<double> &s) {
    std::vector<double> c(1, o);
    double v = o;
    for (double w : s) c.push_back(v += w);
    return c;
  }
  std::vector<double> xs_, ys_, zs_, xc_, yc_, zc_;
  t3DModelData data_;
};

// One cell block plus background layers (ThreeDGravityModel.h:91-104,
// ThreeDSusceptibilityModel.h:42-55).
class ThreeDLayeredModel : public ThreeDModelBase {
 public:
  std::vector<double> &SetValues() { return SetData(); }
  std::vector<double> &SetBackgroundValues() { return bgv_; }
  std::vector<double> &SetBackgroundThicknesses() { return bgt_; }
  const std::vector<double> &GetBackgroundThicknesses() const { return bgt_; }
  rvec GetModelParameters() const {
    const std::vector<double> &values = GetData();
    rvec p(values.size() + bgv_.size());
    for (size_t i = 0; i < values.size(); ++i) p(i) = values[i];
    for (size_t i = 0; i < bgv_.size(); ++i) p(values.size() + i) = bgv_[i];
    return p;
  }
  size_t GetNModelParm() const { return GetData().size() + bgv_.size(); }

 private:
  std::vector<double> bgv_, bgt_;
};
class ThreeDGravityModel : public ThreeDLayeredModel {};
class ThreeDSusceptibilityModel : public ThreeDLayeredModel {};

// Three magnetisation blocks, no background parameters
// (ThreeDMagnetizationModel.h:53-70).
class ThreeDMagnetizationModel : public ThreeDModelBase {
 public:
  std::vector<double> &SetMagnetization_X() { return SetData(); }
  std::vector<double> &SetMagnetization_Y() { return my_; }
  std::vector<double> &SetMagnetization_Z() { return mz_; }
  rvec GetModelParameters() const {
    const std::vector<double> &mx_ = GetData();
    const size_t n = mx_.size();
    rvec p(3 * n);
    for (size_t i = 0; i < n; ++i) {
      p(i) = mx_[i];
      p(n + i) = my_[i];
      p(2 * n + i) = mz_[i];
    }
    return p;
  }
  size_t GetNModelParm() const { return 3 * GetData().size(); }

 private:
  std::vector<double> my_, mz_;
};

class GeneralData {
 public:
  void AddMeasurementPoint(double x, double y, double z) {
    x_.push_back(x);
    y_.push_back(y);
    z_.push_back(z);
  }
  const std::vector<double> &GetMeasPosX() const { return x_; }
  const std::vector<double> &GetMeasPosY() const { return y_; }
  const std::vector<double> &GetMeasPosZ() const { return z_; }

 private:
  std::vector<double> x_, y_, z_;
};
class ScalarGravityData : public GeneralData {
 public:
  typedef ThreeDGravityModel ModelType;
};
class TensorGravityData : public GeneralData {
 public:
  typedef ThreeDGravityModel ModelType;
};
class TotalFieldMagneticData : public GeneralData {
 public:
  typedef ThreeDSusceptibilityModel ModelType;
};
class ThreeComponentMagneticData : public GeneralData {
 public:
  typedef ThreeDMagnetizationModel ModelType;
};

template <class DataType> class ThreeDGravMagImplementation;

template <class DataType>
class ThreeDGravMagCalculator {
 public:
  typedef typename DataType::ModelType ModelType;
  explicit ThreeDGravMagCalculator(std::shared_ptr<ThreeDGravMagImplementation<DataType>> imp)
      : Imp(imp) {}
  virtual ~ThreeDGravMagCalculator() {}
  void SetDataTransform(std::shared_ptr<VectorTransform> t) {
    Transform = t;
    Imp->SetDataTransform(t);
  }
  virtual rvec Calculate(const ModelType &Model, const DataType &Data) {
    return Imp->Calculate(Model, Data, *this);
  }
  virtual rvec LQDerivative(const ModelType &Model, const DataType &Data, const rvec &Misfit) {
    return Imp->LQDerivative(Model, Data, Misfit);
  }
  rmat &SetCurrentSensitivities() { return CurrentSensitivities; }
  virtual void HandleSensitivities(const size_t measindex) = 0;

 protected:
  // the cell values match the cell sizes (ThreeDGravMagCalculator.h:122-145)
  void CheckModelConsistency(const ModelType &Model) {
    if (Model.GetData().size() != Model.NCells())
      throw FatalException("Model values do not match the cell sizes");
  }
  rmat CurrentSensitivities;
  std::shared_ptr<VectorTransform> Transform;
  std::shared_ptr<ThreeDGravMagImplementation<DataType>> Imp;
};

template <class DataType>
class MinMemGravMagCalculator : public ThreeDGravMagCalculator<DataType> {
 public:
  using ThreeDGravMagCalculator<DataType>::ThreeDGravMagCalculator;
  rvec Calculate(const typename DataType::ModelType &Model, const DataType &Data) override {
    this->CurrentSensitivities.resize(0, 0);
    return ThreeDGravMagCalculator<DataType>::Calculate(Model, Data);
  }
  void HandleSensitivities(const size_t) override {}
};

// Keeps every station's raw rows (host memory), as
// FullSensitivityGravMagCalculator.h:98-130 does on its first call.
template <class DataType>
class FullSensitivityGravMagCalculator : public ThreeDGravMagCalculator<DataType> {
 public:
  using ThreeDGravMagCalculator<DataType>::ThreeDGravMagCalculator;
  rvec Calculate(const typename DataType::ModelType &Model, const DataType &Data) override {
    const size_t raw = this->Imp->RawDataPerMeasurement();
    this->CurrentSensitivities.resize(raw, Model.GetNModelParm());
    Sensitivities.resize(Data.GetMeasPosX().size() * raw, Model.GetNModelParm());
    return ThreeDGravMagCalculator<DataType>::Calculate(Model, Data);
  }
  void HandleSensitivities(const size_t measindex) override {
    const size_t raw = this->CurrentSensitivities.size1();
    for (size_t r = 0; r < raw; ++r)
      for (size_t c = 0; c < Sensitivities.size2(); ++c)
        Sensitivities(measindex * raw + r, c) = this->CurrentSensitivities(r, c);
  }
  const rmat &GetSensitivities() const { return Sensitivities; }

 private:
  rmat Sensitivities;
};

template <class DataType>
class ThreeDGravMagImplementation {
 public:
  typedef typename DataType::ModelType ThreeDModelType;
  virtual ~ThreeDGravMagImplementation() {}
  virtual size_t RawDataPerMeasurement() = 0;
  void SetDataTransform(std::shared_ptr<VectorTransform> t) { Transform = t; }
  size_t GetDataPerMeasurement() {
    return Transform ? Transform->GetOutputSize() : RawDataPerMeasurement();
  }
  // The generic station loop: gridded + background per station, then
  // HandleSensitivities(i).  Without a transform only (stand-in).
  virtual rvec Calculate(const ThreeDModelType &Model, const DataType &Data,
                         ThreeDGravMagCalculator<DataType> &Calculator) {
    if (Transform)
      throw FatalException("the stand-in station loop has no data transforms");
    const size_t nmeas = Data.GetMeasPosX().size(), raw = RawDataPerMeasurement();
    const double xw = std::accumulate(Model.GetXCellSizes().begin(), Model.GetXCellSizes().end(), 0.0);
    const double yw = std::accumulate(Model.GetYCellSizes().begin(), Model.GetYCellSizes().end(), 0.0);
    const double zw = std::accumulate(Model.GetZCellSizes().begin(), Model.GetZCellSizes().end(), 0.0);
    rvec out(nmeas * raw);
    for (size_t i = 0; i < nmeas; ++i) {
      rvec g = CalcGridded(i, Model, Data, Calculator.SetCurrentSensitivities());
      rvec b = CalcBackground(i, xw, yw, zw, Model, Data, Calculator.SetCurrentSensitivities());
      for (size_t r = 0; r < raw; ++r) out(i * raw + r) = g(r) + b(r);
      Calculator.HandleSensitivities(i);
    }
    return out;
  }
  virtual rvec LQDerivative(const ThreeDModelType &Model, const DataType &Data,
                            const rvec &Misfit) = 0;

 protected:
  std::shared_ptr<VectorTransform> Transform;

 private:
  virtual rvec CalcBackground(const size_t measindex, const double xwidth, const double ywidth,
                              const double zwidth, const ThreeDModelType &Model,
                              const DataType &Data, rmat &Sensitivities) = 0;
  virtual rvec CalcGridded(const size_t measindex, const ThreeDModelType &Model,
                           const DataType &Data, rmat &Sensitivities) = 0;
};

}  // namespace jif3D
