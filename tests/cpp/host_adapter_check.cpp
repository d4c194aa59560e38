// Drives the C++ implementation objects of jif3d_gb300/host through the
// stand-in calculators, on a problem read from a text file, and writes what
// they return for tests/test_gpu_host_adapter.py to compare with the oracle.
//
// usage: host_adapter_check problem.txt out.txt
//
// problem.txt (whitespace separated):
//   kind inc dec fs transform t_inc t_dec
//   nx ny nz, then nx / ny / nz cell sizes, then the origin x y z
//   nbg, nbg thicknesses
//   nmeas, nmeas x y z triples
//   nparm, nparm model values
//   nmisfit, nmisfit misfit values
// out.txt: lines "name count values..." for
//   minmem (MinMem calculator), full (FullSensitivity calculator), rows
//   (its sensitivity matrix, row-major), grad (LQDerivative), loop (the base
//   class's per-station loop, no transform only), and "exception ok" when a
//   wrong misfit size raised FatalException; with a transform, the same with
//   the transform set through the calculators only (a second implementation
//   object, no SetGB300Transform): calcminmem, calcfull, calcrows, calcgrad
//   (MinMem) and calcfullgrad (FullSensitivity, first call uncached).  Then the device-resident
//   calculator (GB300DeviceSensitivityCalculator, fp16 hi / lo storage):
//   devfirst (first call, FP64), devcached (second call, stored J), devgrad,
//   devbatch / devbatchgrad (rows k = 0, 1, 2: the model times 1 + 0.1 k and
//   the misfit times k + 1), devmoved (station 0 moved by +1 m in x: a new
//   geometry, FP64 again) and "devexception ok" for a misfit row count that
//   does not match the models; dev32cached / dev32grad: the same calculator
//   with its default FP32 storage.
#define JIF3D_GB300_STANDALONE
#include <cstdio>
#include <fstream>
#include <memory>

#include "GB300DeviceSensitivityCalculator.h"
#include "GB300GravMagImplementation.h"

using namespace jif3D;

namespace {

struct Problem {
  int kind = 0, transform = 0;
  double inc = 0, dec = 0, fs = 0, tinc = 0, tdec = 0;
  std::vector<double> xs, ys, zs, bg, st, model, misfit;
  double x0 = 0, y0 = 0, z0 = 0;
};

std::vector<double> read_vec(std::istream &in, size_t n) {
  std::vector<double> v(n);
  for (auto &x : v) in >> x;
  return v;
}

Problem read_problem(const char *path) {
  std::ifstream in(path);
  Problem p;
  in >> p.kind >> p.inc >> p.dec >> p.fs >> p.transform >> p.tinc >> p.tdec;
  size_t nx, ny, nz, n;
  in >> nx >> ny >> nz;
  p.xs = read_vec(in, nx);
  p.ys = read_vec(in, ny);
  p.zs = read_vec(in, nz);
  in >> p.x0 >> p.y0 >> p.z0 >> n;
  p.bg = read_vec(in, n);
  in >> n;
  p.st = read_vec(in, 3 * n);
  in >> n;
  p.model = read_vec(in, n);
  in >> n;
  p.misfit = read_vec(in, n);
  if (!in) throw FatalException("cannot read the problem file");
  return p;
}

rvec flatten(const rmat &m) {
  rvec v(m.size1() * m.size2());
  for (size_t r = 0; r < m.size1(); ++r)
    for (size_t c = 0; c < m.size2(); ++c) v(r * m.size2() + c) = m(r, c);
  return v;
}

void put(std::FILE *f, const char *name, const rvec &v) {
  std::fprintf(f, "%s %zu", name, v.size());
  for (size_t i = 0; i < v.size(); ++i) std::fprintf(f, " %.17g", v(i));
  std::fprintf(f, "\n");
}

template <class Model>
void fill_layered(Model &m, const Problem &p) {
  const size_t n = p.xs.size() * p.ys.size() * p.zs.size();
  m.SetValues().assign(p.model.begin(), p.model.begin() + n);
  m.SetBackgroundValues().assign(p.model.begin() + n, p.model.end());
  m.SetBackgroundThicknesses() = p.bg;
}
void fill(ThreeDGravityModel &m, const Problem &p) { fill_layered(m, p); }
void fill(ThreeDSusceptibilityModel &m, const Problem &p) { fill_layered(m, p); }
void fill(ThreeDMagnetizationModel &m, const Problem &p) {
  const size_t n = p.xs.size() * p.ys.size() * p.zs.size();
  m.SetMagnetization_X().assign(p.model.begin(), p.model.begin() + n);
  m.SetMagnetization_Y().assign(p.model.begin() + n, p.model.begin() + 2 * n);
  m.SetMagnetization_Z().assign(p.model.begin() + 2 * n, p.model.begin() + 3 * n);
}

std::shared_ptr<VectorTransform> transform_of(int code, double inc, double dec) {
  switch (code) {
    case J3G_T_FTG_INVARIANT: return std::make_shared<FTGInvariant>();
    case J3G_T_TOTAL_FIELD: return std::make_shared<TotalField>();
    case J3G_T_TFA: return std::make_shared<TotalFieldAnomaly>(inc, dec);
    default: return nullptr;
  }
}

// The transform set through the calculators only, as unchanged jif3D callers
// do (no SetGB300Transform on this implementation object).
template <class DataType>
void run_calculator_transform(const Problem &p,
                              std::shared_ptr<GB300GravMagImplementation<DataType>> imp,
                              typename DataType::ModelType &model, const DataType &data,
                              const rvec &mis, std::FILE *out) {
  auto t = transform_of(p.transform, p.tinc, p.tdec);
  if (!t) return;
  MinMemGravMagCalculator<DataType> minmem(imp);
  FullSensitivityGravMagCalculator<DataType> full(imp);
  minmem.SetDataTransform(t);
  full.SetDataTransform(t);
  put(out, "calcminmem", minmem.Calculate(model, data));
  put(out, "calcfull", full.Calculate(model, data));
  put(out, "calcrows", flatten(full.GetSensitivities()));
  put(out, "calcgrad", minmem.LQDerivative(model, data, mis));
  put(out, "calcfullgrad", full.LQDerivative(model, data, mis));
}

template <class DataType>
void run(const Problem &p, std::shared_ptr<GB300GravMagImplementation<DataType>> imp,
         std::shared_ptr<GB300GravMagImplementation<DataType>> plain, std::FILE *out) {
  typename DataType::ModelType model;
  model.SetMesh(p.xs, p.ys, p.zs, p.x0, p.y0, p.z0);
  fill(model, p);
  DataType data;
  for (size_t i = 0; i + 2 < p.st.size(); i += 3)
    data.AddMeasurementPoint(p.st[i], p.st[i + 1], p.st[i + 2]);
  imp->SetGB300Transform(p.transform, p.tinc, p.tdec);

  MinMemGravMagCalculator<DataType> minmem(imp);
  FullSensitivityGravMagCalculator<DataType> full(imp);
  if (auto t = transform_of(p.transform, p.tinc, p.tdec)) {
    minmem.SetDataTransform(t);
    full.SetDataTransform(t);
  }
  put(out, "minmem", minmem.Calculate(model, data));
  put(out, "full", full.Calculate(model, data));
  const rmat &J = full.GetSensitivities();
  rvec rows(J.size1() * J.size2());
  for (size_t r = 0; r < J.size1(); ++r)
    for (size_t c = 0; c < J.size2(); ++c) rows(r * J.size2() + c) = J(r, c);
  put(out, "rows", rows);
  rvec mis(p.misfit.size());
  for (size_t i = 0; i < p.misfit.size(); ++i) mis(i) = p.misfit[i];
  put(out, "grad", minmem.LQDerivative(model, data, mis));
  if (p.transform == J3G_T_NONE) {
    // the base class's station loop over the per-station overrides
    FullSensitivityGravMagCalculator<DataType> loopcalc(imp);
    loopcalc.Calculate(model, data);  // sizes its matrices
    put(out, "loop", imp->ThreeDGravMagImplementation<DataType>::Calculate(model, data, loopcalc));
    const rmat &L = loopcalc.GetSensitivities();
    rvec lrows(L.size1() * L.size2());
    for (size_t r = 0; r < L.size1(); ++r)
      for (size_t c = 0; c < L.size2(); ++c) lrows(r * L.size2() + c) = L(r, c);
    put(out, "looprows", lrows);
  }
  try {
    minmem.LQDerivative(model, data, rvec(mis.size() + 1));
  } catch (const FatalException &) {
    std::fprintf(out, "exception ok\n");
  }
  run_calculator_transform(p, plain, model, data, mis, out);

  GB300DeviceSensitivityCalculator<DataType> dev(imp, J3G_STORE_F16X2);
  if (auto t = transform_of(p.transform, p.tinc, p.tdec)) dev.SetDataTransform(t);
  put(out, "devfirst", dev.Calculate(model, data));
  put(out, "devcached", dev.Calculate(model, data));
  put(out, "devgrad", dev.LQDerivative(model, data, mis));
  const rvec params = model.GetModelParameters();
  rmat P(3, params.size()), M(3, mis.size());
  for (size_t k = 0; k < 3; ++k) {
    for (size_t c = 0; c < params.size(); ++c) P(k, c) = params(c) * (1.0 + 0.1 * k);
    for (size_t c = 0; c < mis.size(); ++c) M(k, c) = mis(c) * (k + 1.0);
  }
  put(out, "devbatch", flatten(dev.CalculateBatch(model, data, P)));
  put(out, "devbatchgrad", flatten(dev.LQDerivativeBatch(model, data, P, M)));
  DataType moved;
  for (size_t i = 0; i + 2 < p.st.size(); i += 3)
    moved.AddMeasurementPoint(p.st[i] + (i == 0 ? 1.0 : 0.0), p.st[i + 1], p.st[i + 2]);
  put(out, "devmoved", dev.Calculate(model, moved));
  try {
    dev.LQDerivativeBatch(model, data, P, rmat(2, mis.size()));
  } catch (const FatalException &) {
    std::fprintf(out, "devexception ok\n");
  }
  // the default storage (FP32 J) on the original stations
  GB300DeviceSensitivityCalculator<DataType> dev32(imp);
  if (auto t = transform_of(p.transform, p.tinc, p.tdec)) dev32.SetDataTransform(t);
  dev32.Calculate(model, data);  // FP64, builds the FP32 J
  put(out, "dev32cached", dev32.Calculate(model, data));
  put(out, "dev32grad", dev32.LQDerivative(model, data, mis));
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s problem.txt out.txt\n", argv[0]);
    return 2;
  }
  try {
    const Problem p = read_problem(argv[1]);
    std::FILE *out = std::fopen(argv[2], "w");
    if (!out) return 3;
    switch (p.kind) {
      case J3G_SCALAR:
        run<ScalarGravityData>(p, std::make_shared<ScalarGB300GravityImp>(),
                               std::make_shared<ScalarGB300GravityImp>(), out);
        break;
      case J3G_TENSOR:
        run<TensorGravityData>(p, std::make_shared<TensorGB300GravityImp>(),
                               std::make_shared<TensorGB300GravityImp>(), out);
        break;
      case J3G_MAGNETIC:
        run<TotalFieldMagneticData>(
            p, std::make_shared<GB300MagneticSusceptibilityImp>(p.inc, p.dec, p.fs),
            std::make_shared<GB300MagneticSusceptibilityImp>(p.inc, p.dec, p.fs), out);
        break;
      case J3G_MAG_GRADIENT:
        run<TotalFieldMagneticData>(p, std::make_shared<GB300MagneticGradImp>(p.inc, p.dec, p.fs),
                                    std::make_shared<GB300MagneticGradImp>(p.inc, p.dec, p.fs),
                                    out);
        break;
      case J3G_MAGNETIZATION:
        run<ThreeComponentMagneticData>(p, std::make_shared<GB300MagnetizationImp>(),
                                        std::make_shared<GB300MagnetizationImp>(), out);
        break;
      default:
        std::fprintf(stderr, "unknown kind %d\n", p.kind);
        return 2;
    }
    std::fclose(out);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
