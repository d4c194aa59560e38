// C entry points around the reference's own box-term functions, so that the
// oracle's restatement can be checked against the reference arithmetic.
// Built by oracle/Makefile from Gravity/BasicGravElements.cpp of the jif3D
// source tree (compiled unmodified, with the stand-in headers in oracle/shim);
// the output goes to oracle/_ref/ and never ships.  TEST INFRASTRUCTURE ONLY.
#include "Gravity/BasicGravElements.h"

extern "C" {
double ref_grav_box(double mx, double my, double mz, double cx, double cy, double cz,
                    double sx, double sy, double sz) {
  return jif3D::CalcGravBoxTerm(mx, my, mz, cx, cy, cz, sx, sy, sz);
}
void ref_tensor_box(double mx, double my, double mz, double cx, double cy, double cz,
                    double sx, double sy, double sz, double *out) {
  jif3D::rmat m = jif3D::CalcTensorBoxTerm(mx, my, mz, cx, cy, cz, sx, sy, sz);
  for (int i = 0; i < 9; ++i) out[i] = m.data()[i];
}
double ref_uxx_box(double mx, double my, double mz, double cx, double cy, double cz,
                   double sx, double sy, double sz) {
  return jif3D::CalcUxxTerm(mx, my, mz, cx, cy, cz, sx, sy, sz);
}
double ref_uxy_box(double mx, double my, double mz, double cx, double cy, double cz,
                   double sx, double sy, double sz) {
  return jif3D::CalcUxyTerm(mx, my, mz, cx, cy, cz, sx, sy, sz);
}
double ref_inf_sheet(double mz, double top, double bottom) {
  return jif3D::CalcInfSheetTerm(mz, top, bottom);
}
double ref_uzz_inf_sheet(double mz, double top, double bottom) {
  return jif3D::CalcUzzInfSheetTerm(mz, top, bottom);
}
}
