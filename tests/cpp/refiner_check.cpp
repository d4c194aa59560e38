// Drives jif3D::GB300ModelRefiner (jif3d_gb300/host/GB300ModelRefiner.h) the
// way ThreeDModelObjective drives its refiner (SetFineModelGeometry, then
// RefineModel before the forward and CombineGradient after the gradient,
// Inversion/ThreeDModelObjective.h:188-201, 254-260, 310-324), and writes
// what it returns for tests/test_gpu_refine.py to compare with the oracle.
//
// usage: refiner_check problem.txt out.txt
//
// problem.txt (whitespace separated):
//   coarse origin x y z
//   for x, y, z: n, n coarse sizes
//   for x, y, z: m, m refinement coordinates
//   ncoarse, coarse cell values
//   nfine, refined gradient values
// out.txt: lines "name count values..." for xsizes / ysizes / zsizes (the
//   refined axes), fine (the projected values), coarse_grad (the combined
//   gradient), copy_grad (the same through a copied refiner), and
//   "exception ok" when a last coarse cell of zero size raised FatalException.
#define JIF3D_GB300_STANDALONE
#include <cstdio>
#include <fstream>

#include "GB300ModelRefiner.h"

using namespace jif3D;

namespace {

std::vector<double> read_vec(std::istream &in) {
  size_t n = 0;
  in >> n;
  std::vector<double> v(n);
  for (auto &x : v) in >> x;
  return v;
}

void write(FILE *f, const char *name, const std::vector<double> &v) {
  std::fprintf(f, "%s %zu", name, v.size());
  for (double x : v) std::fprintf(f, " %.17g", x);
  std::fprintf(f, "\n");
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: refiner_check problem.txt out.txt\n");
    return 2;
  }
  try {
    std::ifstream in(argv[1]);
    double x0, y0, z0;
    in >> x0 >> y0 >> z0;
    std::vector<double> xs = read_vec(in), ys = read_vec(in), zs = read_vec(in);
    std::vector<double> rx = read_vec(in), ry = read_vec(in), rz = read_vec(in);
    std::vector<double> values = read_vec(in), fgrad = read_vec(in);
    if (!in) throw FatalException("cannot read the problem file");

    ThreeDGravityModel coarse, fine;
    coarse.SetMesh(xs, ys, zs, x0, y0, z0);
    coarse.SetData() = values;
    fine.SetMesh(std::vector<double>(1, 1.0), std::vector<double>(1, 1.0),
                 std::vector<double>(1, 1.0), x0, y0, z0);

    GB300ModelRefiner refiner;
    refiner.SetXCoordinates(rx);
    refiner.SetYCoordinates(ry);
    refiner.SetZCoordinates(rz);
    refiner.RefineModel(coarse, fine);

    FILE *out = std::fopen(argv[2], "w");
    write(out, "xsizes", fine.GetXCellSizes());
    write(out, "ysizes", fine.GetYCellSizes());
    write(out, "zsizes", fine.GetZCellSizes());
    write(out, "fine", fine.GetData());
    rvec g(fgrad.size());
    for (size_t i = 0; i < fgrad.size(); ++i) g(i) = fgrad[i];
    const rvec cg = refiner.CombineGradient(g, coarse, fine);
    write(out, "coarse_grad", std::vector<double>(cg.begin(), cg.end()));
    GB300ModelRefiner copy(refiner);
    const rvec cg2 = copy.CombineGradient(g, coarse, fine);
    write(out, "copy_grad", std::vector<double>(cg2.begin(), cg2.end()));

    // a last coarse cell of zero size: the reference throws
    ThreeDGravityModel bad, badfine;
    std::vector<double> bz = zs;
    bz.back() = 0.0;
    bad.SetMesh(xs, ys, bz, x0, y0, z0);
    try {
      refiner.RefineAxes(bad, badfine);
    } catch (const FatalException &) {
      std::fprintf(out, "exception ok\n");
    }
    std::fclose(out);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
