// jif3d_compat.h -- minimal stand-ins for the jif3D declarations that
// GB300GravMagImplementation.h uses, for building it outside a jif3D source
// tree (jif3D itself needs Boost and NetCDF).  Same class and member names as
// jif3D so that the implementation header compiles unchanged against either;
// only what the implementation and its tests touch is provided:
//   rvec / rmat                     (Global/VecMat.h)
//   FatalException                  (Global/FatalException.h)
//   VectorTransform + FTGInvariant, TotalField, TotalFieldAnomaly (Transform
//     and Derivative, Gravity/GravityTransforms.h:25-100,
//     Magnetics/MagneticTransforms.h:19-156)
//   ThreeDModelBase and the gravity / susceptibility / magnetisation models
//   the data classes with their ModelType
//   ThreeDGravMagCalculator, MinMemGravMagCalculator,
//   FullSensitivityGravMagCalculator (host-stored rows, FP64 products)
//   ThreeDGravMagImplementation with its private transform and the generic
//     per-station Calculate and LQDerivative loops
//     (GravMag/ThreeDGravMagImplementation.h:39-231), so that the
//     per-station overrides and transforms set through a calculator can be
//     exercised
#pragma once

#include <cmath>
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

// Per-station data transforms: Transform maps the raw data of a station to
// its transformed data, Derivative gives the output x input Jacobian.
class VectorTransform {
 public:
  virtual ~VectorTransform() {}
  virtual size_t GetInputSize() const = 0;
  virtual size_t GetOutputSize() const = 0;
  virtual rvec Transform(const rvec &in) const = 0;
  virtual rmat Derivative(const rvec &in) const = 0;
};
// The second invariant of the tensor Uxx..Uzz (3 x 3, C order).
class FTGInvariant : public VectorTransform {
 public:
  size_t GetInputSize() const override { return 9; }
  size_t GetOutputSize() const override { return 1; }
  rvec Transform(const rvec &u) const override {
    rvec r(1);
    r(0) = u(0) * u(4) + u(4) * u(8) + u(0) * u(8) - u(3) * u(1) - u(7) * u(5) - u(2) * u(6);
    return r;
  }
  rmat Derivative(const rvec &u) const override {
    rmat d(1, 9);
    d(0, 0) = u(4) + u(8);
    d(0, 1) = -u(3);
    d(0, 2) = -u(6);
    d(0, 3) = -u(1);
    d(0, 4) = u(0) + u(8);
    d(0, 5) = -u(7);
    d(0, 6) = -u(2);
    d(0, 7) = -u(5);
    d(0, 8) = u(0) + u(4);
    return d;
  }
};
// |B| of the three components.
class TotalField : public VectorTransform {
 public:
  size_t GetInputSize() const override { return 3; }
  size_t GetOutputSize() const override { return 1; }
  rvec Transform(const rvec &b) const override {
    rvec r(1);
    r(0) = std::sqrt(b(0) * b(0) + b(1) * b(1) + b(2) * b(2));
    return r;
  }
  rmat Derivative(const rvec &b) const override {
    const double t = std::sqrt(b(0) * b(0) + b(1) * b(1) + b(2) * b(2));
    rmat d(1, 3);
    for (size_t k = 0; k < 3; ++k) d(0, k) = b(k) / t;
    return d;
  }
};
// The projection of the anomalous field on the inducing field's direction
// (inclination and declination in radians).
class TotalFieldAnomaly : public VectorTransform {
 public:
  explicit TotalFieldAnomaly(double Inclination = 0.0, double Declination = 0.0)
      : bx_(std::cos(Inclination) * std::cos(Declination)),
        by_(std::cos(Inclination) * std::sin(Declination)),
        bz_(std::sin(Inclination)) {}
  size_t GetInputSize() const override { return 3; }
  size_t GetOutputSize() const override { return 1; }
  rvec Transform(const rvec &b) const override {
    rvec r(1);
    r(0) = bx_ * b(0) + by_ * b(1) + bz_ * b(2);
    return r;
  }
  rmat Derivative(const rvec &) const override {
    rmat d(1, 3);
    d(0, 0) = bx_;
    d(0, 1) = by_;
    d(0, 2) = bz_;
    return d;
  }

 private:
  double bx_, by_, bz_;
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
  // cell counts; sizes zero, corners at the origin (ThreeDModelBase.h:146-155)
  virtual void SetMeshSize(size_t nx, size_t ny, size_t nz) {
    xs_.assign(nx, 0.0);
    ys_.assign(ny, 0.0);
    zs_.assign(nz, 0.0);
    xc_.assign(nx + 1, 0.0);
    yc_.assign(ny + 1, 0.0);
    zc_.assign(nz + 1, 0.0);
    data_.assign(nx * ny * nz, 0.0);
  }
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
  void SetMeshSize(size_t nx, size_t ny, size_t nz) override {
    ThreeDModelBase::SetMeshSize(nx, ny, nz);
    my_.assign(nx * ny * nz, 0.0);
    mz_.assign(nx * ny * nz, 0.0);
  }

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
  // not virtual, and the transform is private: a derived class sees only
  // GetDataPerMeasurement (ThreeDGravMagImplementation.h:44-75)
  void SetDataTransform(std::shared_ptr<VectorTransform> t) { Transform = t; }
  size_t GetDataPerMeasurement() {
    return Transform ? Transform->GetOutputSize() : RawDataPerMeasurement();
  }
  // The generic station loop (:116-168): gridded + background per station,
  // the transform applied per station, then HandleSensitivities(i).
  virtual rvec Calculate(const ThreeDModelType &Model, const DataType &Data,
                         ThreeDGravMagCalculator<DataType> &Calculator) {
    const size_t nmeas = Data.GetMeasPosX().size(), raw = RawDataPerMeasurement();
    const size_t dpm = GetDataPerMeasurement();
    const double xw = Width(Model.GetXCellSizes()), yw = Width(Model.GetYCellSizes()),
                 zw = Width(Model.GetZCellSizes());
    rvec out(nmeas * dpm);
    for (size_t i = 0; i < nmeas; ++i) {
      rvec cur = CalcGridded(i, Model, Data, Calculator.SetCurrentSensitivities());
      rvec b = CalcBackground(i, xw, yw, zw, Model, Data, Calculator.SetCurrentSensitivities());
      for (size_t r = 0; r < raw; ++r) cur(r) += b(r);
      const rvec res = Transform ? Transform->Transform(cur) : cur;
      for (size_t k = 0; k < dpm; ++k) out(i * dpm + k) = res(k);
      Calculator.HandleSensitivities(i);
    }
    return out;
  }
  // The generic least-squares derivative (:177-231): per station the raw
  // rows, multiplied by the transform's derivative at the raw data, summed
  // with the misfit as weights; times 2.
  virtual rvec LQDerivative(const ThreeDModelType &Model, const DataType &Data,
                            const rvec &Misfit) {
    const size_t nmeas = Data.GetMeasPosX().size(), raw = RawDataPerMeasurement();
    const size_t dpm = GetDataPerMeasurement(), nmod = Model.GetNModelParm();
    if (Misfit.size() != nmeas * dpm) throw FatalException("misfit size");
    const double xw = Width(Model.GetXCellSizes()), yw = Width(Model.GetYCellSizes()),
                 zw = Width(Model.GetZCellSizes());
    rvec deriv(nmod);
    rmat sens(raw, nmod);
    for (size_t i = 0; i < nmeas; ++i) {
      rvec cur = CalcGridded(i, Model, Data, sens);
      rvec b = CalcBackground(i, xw, yw, zw, Model, Data, sens);
      for (size_t r = 0; r < raw; ++r) cur(r) += b(r);
      rmat td(dpm, raw);
      if (Transform)
        td = Transform->Derivative(cur);
      else
        for (size_t r = 0; r < raw; ++r) td(r, r) = 1.0;
      for (size_t j = 0; j < dpm; ++j)
        for (size_t c = 0; c < nmod; ++c) {
          double v = 0.0;
          for (size_t r = 0; r < raw; ++r) v += td(j, r) * sens(r, c);
          deriv(c) += Misfit(i * dpm + j) * v;
        }
    }
    for (size_t c = 0; c < nmod; ++c) deriv(c) *= 2.0;
    return deriv;
  }

 private:
  static double Width(const std::vector<double> &v) {
    return std::accumulate(v.begin(), v.end(), 0.0);
  }
  std::shared_ptr<VectorTransform> Transform;
  virtual rvec CalcBackground(const size_t measindex, const double xwidth, const double ywidth,
                              const double zwidth, const ThreeDModelType &Model,
                              const DataType &Data, rmat &Sensitivities) = 0;
  virtual rvec CalcGridded(const size_t measindex, const ThreeDModelType &Model,
                           const DataType &Data, rmat &Sensitivities) = 0;
};

}  // namespace jif3D
