/*
 * prism_oracle.c -- FP64 CPU oracle for the jif3D gravity / FTG / magnetic
 * prism path.  TEST INFRASTRUCTURE ONLY: it is the checker that the CUDA path
 * is compared against (tests, the smoke check and the CPU-baseline leg of the
 * benchmark); nothing in the product library links or calls it.
 *
 * Every function restates, in the same operation order, the reference code it
 * cites (paths relative to the jif3D source tree).  It is compiled with
 * -ffp-contract=off so that x86-64 and aarch64 hosts give the same bits.
 *
 * Layout conventions (ModelBase/ThreeDModelBase.h:157-168):
 *   model cell (xi, yi, zi) sits at offset (xi*ny + yi)*nz + zi  (z fastest),
 *   xcoord[i] is the upper-left-front corner of cell column i,
 *   the cell spans [xcoord[i], xcoord[i] + xsize[i]].
 * Sensitivity rows are row-major, one row per raw datum, columns ngrid + nbg
 * (Gravity/ThreeDGravityModel.h:91-104).
 */
#include <float.h>
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_GRAV_CONST 6.67428e-11 /* Gravity/BasicGravElements.h:22 */
#define ORC_PI 3.141592653589793238462643383279502884

enum { ORC_SCALAR = 1, ORC_TENSOR = 2, ORC_MAGNETIC = 3, ORC_MAG_GRADIENT = 5,
       ORC_MAGNETIZATION = 6 };
enum { ORC_T_NONE = 0, ORC_T_FTG_INVARIANT = 1, ORC_T_TOTAL_FIELD = 2, ORC_T_TFA = 3 };

/* ---------------------------------------------------------------------------
 * Box terms.  Gravity/BasicGravElements.cpp
 * ------------------------------------------------------------------------- */

/* One corner of the g_z term: x ln(y+r) + y ln(x+r) + z atan2(z r, x y), with
 * r clamped from below at DBL_EPSILON.  BasicGravElements.cpp:26-37. */
static double gz_corner(double x, double y, double z)
{
  double r = sqrt(x * x + y * y + z * z);
  if (r < DBL_EPSILON) /* std::max(r, eps) keeps NaN, so does this test */
    r = DBL_EPSILON;
  double v = x * log(y + r) + y * log(x + r);
  v += z * atan2(z * r, x * y);
  return v;
}

/* Diagonal FTG corner term atan2(a b, c sqrt(a^2+b^2+c^2)).
 * BasicGravElements.cpp:43-47. */
static double ftg_diag_corner(double a, double b, double c)
{
  return atan2(a * b, c * sqrt(a * a + b * b + c * c));
}

/* Off-diagonal FTG corner term ln(max(v + sqrt(x^2+y^2+z^2), eps)).
 * BasicGravElements.cpp:53-59. */
static double ftg_offdiag_corner(double v, double x, double y, double z)
{
  double arg = v + sqrt(x * x + y * y + z * z);
  if (arg < DBL_EPSILON)
    arg = DBL_EPSILON;
  return log(arg);
}

/* g_z geometric term of one prism, corners summed in the reference order
 * (000, x, y, z, xy, xz, yz, xyz).  BasicGravElements.cpp:82-109. */
double orc_grav_box(double mx, double my, double mz, double cx, double cy, double cz,
                    double sx, double sy, double sz)
{
  const double x0 = mx - cx, x1 = mx - (cx + sx);
  const double y0 = my - cy, y1 = my - (cy + sy);
  const double z0 = mz - cz, z1 = mz - (cz + sz);
  double acc = -gz_corner(x0, y0, z0);
  acc += gz_corner(x1, y0, z0);
  acc += gz_corner(x0, y1, z0);
  acc += gz_corner(x0, y0, z1);
  acc -= gz_corner(x1, y1, z0);
  acc -= gz_corner(x1, y0, z1);
  acc -= gz_corner(x0, y1, z1);
  acc += gz_corner(x1, y1, z1);
  return -acc * ORC_GRAV_CONST;
}

/* Uxx geometric term (and Uyy/Uzz with permuted arguments).
 * BasicGravElements.cpp:125-152. */
double orc_uxx_box(double mx, double my, double mz, double cx, double cy, double cz,
                   double sx, double sy, double sz)
{
  const double x0 = mx - cx, x1 = mx - (cx + sx);
  const double y0 = my - cy, y1 = my - (cy + sy);
  const double z0 = mz - cz, z1 = mz - (cz + sz);
  double acc = -ftg_diag_corner(y0, z0, x0);
  acc += ftg_diag_corner(y0, z0, x1);
  acc += ftg_diag_corner(y1, z0, x0);
  acc += ftg_diag_corner(y0, z1, x0);
  acc -= ftg_diag_corner(y1, z0, x1);
  acc -= ftg_diag_corner(y0, z1, x1);
  acc -= ftg_diag_corner(y1, z1, x0);
  acc += ftg_diag_corner(y1, z1, x1);
  return acc * ORC_GRAV_CONST;
}

/* Uxy geometric term (and Uxz/Uyz with permuted arguments).
 * BasicGravElements.cpp:168-202. */
double orc_uxy_box(double mx, double my, double mz, double cx, double cy, double cz,
                   double sx, double sy, double sz)
{
  const double x0 = mx - cx, x1 = mx - (cx + sx);
  const double y0 = my - cy, y1 = my - (cy + sy);
  const double z0 = mz - cz, z1 = mz - (cz + sz);
  double acc = -ftg_offdiag_corner(z0, z0, y0, x0);
  acc += ftg_offdiag_corner(z0, z0, y0, x1);
  acc += ftg_offdiag_corner(z0, z0, y1, x0);
  acc += ftg_offdiag_corner(z1, z1, y0, x0);
  acc -= ftg_offdiag_corner(z0, z0, y1, x1);
  acc -= ftg_offdiag_corner(z1, z1, y0, x1);
  acc -= ftg_offdiag_corner(z1, z1, y1, x0);
  acc += ftg_offdiag_corner(z1, z1, y1, x1);
  return -acc * ORC_GRAV_CONST;
}

/* Full 3x3 tensor, row-major, symmetric.  BasicGravElements.cpp:216-244. */
void orc_tensor_box(double mx, double my, double mz, double cx, double cy, double cz,
                    double sx, double sy, double sz, double *u)
{
  u[0] = orc_uxx_box(mx, my, mz, cx, cy, cz, sx, sy, sz);
  u[4] = orc_uxx_box(my, mx, mz, cy, cx, cz, sy, sx, sz);
  u[8] = orc_uxx_box(mz, mx, my, cz, cx, cy, sz, sx, sy);
  u[1] = orc_uxy_box(mx, my, mz, cx, cy, cz, sx, sy, sz);
  u[3] = u[1];
  u[2] = orc_uxy_box(mx, mz, my, cx, cz, cy, sx, sz, sy);
  u[6] = u[2];
  u[5] = orc_uxy_box(mz, my, mx, cz, cy, cx, sz, sy, sx);
  u[7] = u[5];
}

static double sign_of(double n) { return n >= 0 ? 1.0 : -1.0; } /* Global/NumUtil.h:26-33 */

/* Infinite sheet g_z term.  Gravity/BasicGravElements.h:51-63. */
double orc_inf_sheet(double mz, double top, double bottom)
{
  const double thick = bottom - top;
  if ((mz <= top) || (mz >= bottom))
    return 2.0 * ORC_PI * ORC_GRAV_CONST * thick * sign_of(top - mz);
  return 2.0 * ORC_PI * ORC_GRAV_CONST * (thick - 2.0 * (mz - top));
}

/* Infinite sheet Uzz term.  Gravity/BasicGravElements.h:65-75. */
double orc_uzz_inf_sheet(double mz, double top, double bottom)
{
  if ((mz <= top) || (mz >= bottom))
    return 0.0;
  return 4.0 * ORC_PI * ORC_GRAV_CONST;
}

/* ---------------------------------------------------------------------------
 * Problem description shared by the drivers below.
 * ------------------------------------------------------------------------- */
typedef struct {
  int nx, ny, nz;
  const double *xc, *yc, *zc; /* corner coordinates, at least nx / ny / nz used (+1 for origin) */
  const double *xs, *ys, *zs; /* cell sizes */
  int nbg;
  const double *bg_thick;     /* nbg background layer thicknesses */
  int nmeas;
  const double *mx, *my, *mz; /* station coordinates */
  int kind;                   /* ORC_SCALAR / ORC_TENSOR / ORC_MAGNETIC */
  double inc, dec, fs;        /* magnetic inducing field (radians, nT) */
  int transform;              /* ORC_T_* */
  double t_inc, t_dec;        /* angles of a TotalFieldAnomaly transform */
  int nthreads;
} orc_problem;

static int raw_per_meas(int kind)
{
  return (kind == ORC_SCALAR || kind == ORC_MAG_GRADIENT) ? 1 : (kind == ORC_TENSOR ? 9 : 3);
}

/* Model parameters per cell block: three magnetisation components
 * (Magnetics/ThreeDMagnetizationModel.h:53-70: x block, y block, z block,
 * no background parameters), else one value per cell plus the background. */
static size_t ncols_of(int kind, int ngrid, int nbg)
{
  return kind == ORC_MAGNETIZATION ? (size_t)3 * ngrid : (size_t)ngrid + nbg;
}

static int out_per_meas(const orc_problem *p)
{
  return p->transform == ORC_T_NONE ? raw_per_meas(p->kind) : 1;
}

/* Magnetic projection of a tensor sensitivity onto B.
 * Magnetics/OMPMagneticSusceptibilityImp.cpp:116-118, 160-170. */
static void mag_project(const orc_problem *p, const double *u, double *b)
{
  const double bx = cos(p->inc) * cos(p->dec);
  const double by = cos(p->inc) * sin(p->dec);
  const double bz = sin(p->inc);
  const double factor = 1.0 / (4 * ORC_PI * ORC_GRAV_CONST);
  b[0] = (u[0] * bx + u[1] * by + u[2] * bz) * p->fs * factor;
  b[1] = (u[3] * bx + u[4] * by + u[5] * bz) * p->fs * factor;
  b[2] = (u[6] * bx + u[7] * by + u[8] * bz) * p->fs * factor;
}

/* z component of the field of one cell at (mx, my, mz) for the vertical
 * gradient: Magnetics/OMPMagneticGradImp.cpp:20-22, 58-73 (factor 1e-7 / G). */
static double grad_bz(const orc_problem *p, double mx, double my, double mz, int xi, int yi,
                      int zi)
{
  const double bx = cos(p->inc) * cos(p->dec);
  const double by = cos(p->inc) * sin(p->dec);
  const double bz = sin(p->inc);
  double u[9];
  orc_tensor_box(mx, my, mz, p->xc[xi], p->yc[yi], p->zc[zi], p->xs[xi], p->ys[yi], p->zs[zi],
                 u);
  const double factor = 1e-7 / ORC_GRAV_CONST;
  return (u[6] * bx + u[7] * by + u[8] * bz) * p->fs * factor;
}

/* Raw sensitivities of one cell for one station (1, 9 or 3 values; for the
 * vertical gradient the two fields Bz(z) and Bz(z + 1), whose difference is
 * the row; for magnetisation the 3 x 3 block factor * U, row-major). */
static void cell_sens(const orc_problem *p, int s, int xi, int yi, int zi, double *out)
{
  const double mx = p->mx[s], my = p->my[s], mz = p->mz[s];
  if (p->kind == ORC_MAG_GRADIENT) {
    out[0] = grad_bz(p, mx, my, mz, xi, yi, zi);       /* OMPMagneticGradImp.cpp:58-71 */
    out[1] = grad_bz(p, mx, my, mz + 1, xi, yi, zi);   /* :76-86 */
    return;
  }
  if (p->kind == ORC_MAGNETIZATION) {
    /* Magnetics/OMPMagnetizationImp.cpp:58-68: currvalue = factor * U */
    const double mag_mu = 4e-7 * ORC_PI;
    const double factor = 1.0e9 * mag_mu / (4 * ORC_PI * ORC_GRAV_CONST);
    double u[9];
    orc_tensor_box(mx, my, mz, p->xc[xi], p->yc[yi], p->zc[zi], p->xs[xi], p->ys[yi],
                   p->zs[zi], u);
    for (int c = 0; c < 9; ++c)
      out[c] = factor * u[c];
    return;
  }
  if (p->kind == ORC_SCALAR) {
    out[0] = orc_grav_box(mx, my, mz, p->xc[xi], p->yc[yi], p->zc[zi], p->xs[xi],
                          p->ys[yi], p->zs[zi]);
  } else {
    double u[9];
    orc_tensor_box(mx, my, mz, p->xc[xi], p->yc[yi], p->zc[zi], p->xs[xi], p->ys[yi],
                   p->zs[zi], u);
    if (p->kind == ORC_TENSOR)
      memcpy(out, u, sizeof(u));
    else
      mag_project(p, u, out);
  }
}

/* Gridded part for one station: Gravity/ScalarOMPGravityImp.cpp:138-180,
 * Gravity/TensorOMPGravityImp.cpp:125-182,
 * Magnetics/OMPMagneticSusceptibilityImp.cpp:113-194.
 * The cell loop is one flat loop over the z-fastest offset.  With one thread
 * the sum is taken in offset order; with more, OpenMP splits it in contiguous
 * chunks and adds the chunk sums (the reference's reduction(+)).
 * sens: raw x ncol row-major (ncol >= ngrid) or NULL. */
/* Per-cell accumulation of the two new kinds (into acc[0..2]) and their rows.
 * Vertical gradient: BzBot += BzSensBot * chi, BzTop += BzSensTop * chi, row
 * BzSensBot - BzSensTop (OMPMagneticGradImp.cpp:71-100).  Magnetisation:
 * B_k += (c_k0 mx + c_k1 my) + c_k2 mz, rows c_kj at column offset + j*ngrid
 * (OMPMagnetizationImp.cpp:70-104). */
static void accumulate_special(const orc_problem *p, const double *v, const double *model,
                               int offset, int ngrid, double *acc, double *sens, size_t ncol)
{
  if (p->kind == ORC_MAG_GRADIENT) {
    const double chi = model[offset];
    acc[0] += v[0] * chi;
    acc[1] += v[1] * chi;
    if (sens)
      sens[offset] = v[0] - v[1];
    return;
  }
  const double m0 = model[offset], m1 = model[offset + ngrid], m2 = model[offset + 2 * ngrid];
  for (int k = 0; k < 3; ++k) {
    acc[k] += (v[3 * k] * m0 + v[3 * k + 1] * m1 + v[3 * k + 2] * m2);
    if (sens)
      for (int j = 0; j < 3; ++j)
        sens[(size_t)k * ncol + offset + (size_t)j * ngrid] = v[3 * k + j];
  }
}

static void gridded(const orc_problem *p, int s, const double *model, double *result,
                    double *sens, size_t ncol)
{
  const int ngrid = p->nx * p->ny * p->nz;
  const int raw = raw_per_meas(p->kind);
  const int special = p->kind == ORC_MAG_GRADIENT || p->kind == ORC_MAGNETIZATION;
  const int nacc = p->kind == ORC_MAG_GRADIENT ? 2 : raw;
  double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#ifdef _OPENMP
#pragma omp parallel num_threads(p->nthreads > 0 ? p->nthreads : 1)
  {
    double local[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma omp for schedule(static)
    for (int offset = 0; offset < ngrid; ++offset) {
      const int zi = offset % p->nz;
      const int rest = offset / p->nz;
      const int yi = rest % p->ny;
      const int xi = rest / p->ny;
      double v[9];
      cell_sens(p, s, xi, yi, zi, v);
      if (special) {
        accumulate_special(p, v, model, offset, ngrid, local, sens, ncol);
        continue;
      }
      const double rho = model[offset];
      for (int c = 0; c < raw; ++c) {
        local[c] += v[c] * rho;
        if (sens)
          sens[(size_t)c * ncol + offset] = v[c];
      }
    }
#pragma omp for ordered schedule(static, 1)
    for (int t = 0; t < omp_get_num_threads(); ++t) {
#pragma omp ordered
      for (int c = 0; c < nacc; ++c)
        acc[c] += local[c];
    }
  }
#else
  for (int offset = 0; offset < ngrid; ++offset) {
    const int zi = offset % p->nz;
    const int rest = offset / p->nz;
    const int yi = rest % p->ny;
    const int xi = rest / p->ny;
    double v[9];
    cell_sens(p, s, xi, yi, zi, v);
    if (special) {
      accumulate_special(p, v, model, offset, ngrid, acc, sens, ncol);
      continue;
    }
    const double rho = model[offset];
    for (int c = 0; c < raw; ++c) {
      acc[c] += v[c] * rho;
      if (sens)
        sens[(size_t)c * ncol + offset] = v[c];
    }
  }
#endif
  if (p->kind == ORC_MAG_GRADIENT) {
    result[0] = acc[0] - acc[1]; /* returnvalue(0) = BzBot - BzTop */
    return;
  }
  for (int c = 0; c < raw; ++c)
    result[c] = acc[c];
}

/* 1-D background for one station.  Gravity/GravityBackground.cpp:24-72 (g_z),
 * 87-137 (tensor), Magnetics/OMPMagneticSusceptibilityImp.cpp:31-101 (B).
 * The depth test compares an absolute depth with the grid thickness, exactly
 * as the reference does (GravityBackground.cpp:49,56). */
static void background(const orc_problem *p, int s, double xw, double yw, double zw,
                       const double *bgval, double *result, double *sens, size_t ncol,
                       int ngrid)
{
  const int raw = raw_per_meas(p->kind);
  if (p->kind == ORC_MAG_GRADIENT || p->kind == ORC_MAGNETIZATION) {
    /* no background response: OMPMagneticGradImp.h:32-40, OMPMagnetizationImp.cpp:16-22
     * (the gradient's background columns stay zero; magnetisation has none) */
    for (int c = 0; c < raw; ++c)
      result[c] = 0.0;
    if (sens && p->kind == ORC_MAG_GRADIENT)
      for (int j = 0; j < p->nbg; ++j)
        sens[(size_t)ngrid + j] = 0.0;
    return;
  }
  const double mx = p->mx[s], my = p->my[s], mz = p->mz[s];
  double top = p->zc[0];
  double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int j = 0; j < p->nbg; ++j) {
    const double thick = p->bg_thick[j];
    const double bottom = top + thick;
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (p->kind == ORC_SCALAR) {
      v[0] = orc_inf_sheet(mz, top, bottom);
      if (top < zw && (bottom <= zw))
        v[0] -= orc_grav_box(mx, my, mz, p->xc[0], p->yc[0], top, xw, yw, thick);
      if (top < zw && bottom > zw)
        v[0] -= orc_grav_box(mx, my, mz, p->xc[0], p->yc[0], top, xw, yw, (zw - top));
    } else {
      double u[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      u[8] = orc_uzz_inf_sheet(mz, top, bottom);
      double b[9];
      if (top < zw && (bottom <= zw)) {
        orc_tensor_box(mx, my, mz, p->xc[0], p->yc[0], top, xw, yw, thick, b);
        for (int c = 0; c < 9; ++c)
          u[c] -= b[c];
      }
      if (top < zw && bottom > zw) {
        orc_tensor_box(mx, my, mz, p->xc[0], p->yc[0], top, xw, yw, (zw - top), b);
        for (int c = 0; c < 9; ++c)
          u[c] -= b[c];
      }
      if (p->kind == ORC_TENSOR)
        memcpy(v, u, sizeof(u));
      else
        mag_project(p, u, v);
    }
    for (int c = 0; c < raw; ++c) {
      if (sens)
        sens[(size_t)c * ncol + ngrid + j] = v[c];
      acc[c] += v[c] * bgval[j];
    }
    top += thick;
  }
  for (int c = 0; c < raw; ++c)
    result[c] = acc[c];
}

/* Data transforms.  Gravity/GravityTransforms.h:33-37 (I2 invariant),
 * Magnetics/MagneticTransforms.h:27-30 (total field), 122-129 (TFA). */
static double apply_transform(const orc_problem *p, const double *raw)
{
  switch (p->transform) {
  case ORC_T_FTG_INVARIANT:
    return raw[0] * raw[4] + raw[4] * raw[8] + raw[0] * raw[8] - raw[3] * raw[1] -
           raw[7] * raw[5] - raw[2] * raw[6];
  case ORC_T_TOTAL_FIELD:
    return sqrt(raw[0] * raw[0] + raw[1] * raw[1] + raw[2] * raw[2]);
  case ORC_T_TFA: {
    const double bx = cos(p->t_inc) * cos(p->t_dec);
    const double by = cos(p->t_inc) * sin(p->t_dec);
    const double bz = sin(p->t_inc);
    return (bx * raw[0] + by * raw[1] + bz * raw[2]);
  }
  default:
    return raw[0];
  }
}

/* 1 x raw Jacobian of the transform.  GravityTransforms.h:72-93,
 * MagneticTransforms.h:65-75, 136-145. */
static void transform_derivative(const orc_problem *p, const double *raw, double *d)
{
  switch (p->transform) {
  case ORC_T_FTG_INVARIANT:
    d[0] = raw[4] + raw[8];
    d[1] = -raw[3];
    d[2] = -raw[6];
    d[3] = -raw[1];
    d[4] = raw[0] + raw[8];
    d[5] = -raw[7];
    d[6] = -raw[2];
    d[7] = -raw[5];
    d[8] = raw[0] + raw[4];
    break;
  case ORC_T_TOTAL_FIELD: {
    const double t = sqrt(raw[0] * raw[0] + raw[1] * raw[1] + raw[2] * raw[2]);
    d[0] = raw[0] / t;
    d[1] = raw[1] / t;
    d[2] = raw[2] / t;
    break;
  }
  case ORC_T_TFA:
    d[0] = cos(p->t_inc) * cos(p->t_dec);
    d[1] = cos(p->t_inc) * sin(p->t_dec);
    d[2] = sin(p->t_inc);
    break;
  default:
    break;
  }
}

static double width_sum(const double *v, int n)
{
  double s = 0.0; /* std::accumulate, ThreeDGravMagImplementation.h:132-137 */
  for (int i = 0; i < n; ++i)
    s += v[i];
  return s;
}

static orc_problem make_problem(int nx, int ny, int nz, const double *xc, const double *yc,
                                const double *zc, const double *xs, const double *ys,
                                const double *zs, int nbg, const double *bg_thick, int nmeas,
                                const double *mx, const double *my, const double *mz,
                                int kind, double inc, double dec, double fs, int transform,
                                double t_inc, double t_dec, int nthreads)
{
  orc_problem p;
  p.nx = nx; p.ny = ny; p.nz = nz;
  p.xc = xc; p.yc = yc; p.zc = zc;
  p.xs = xs; p.ys = ys; p.zs = zs;
  p.nbg = nbg; p.bg_thick = bg_thick;
  p.nmeas = nmeas; p.mx = mx; p.my = my; p.mz = mz;
  p.kind = kind; p.inc = inc; p.dec = dec; p.fs = fs;
  p.transform = transform; p.t_inc = t_inc; p.t_dec = t_dec;
  p.nthreads = nthreads;
  return p;
}

/* Forward response of all stations, optionally with the raw sensitivity
 * matrix (rows nmeas*raw, columns ngrid+nbg).  The station loop of
 * GravMag/ThreeDGravMagImplementation.h:116-168: gridded + background, then
 * the transform.  model holds ngrid grid values followed by nbg background
 * values (Gravity/ThreeDGravityModel.h:91-99).  Returns 0 on success. */
int orc_forward(int nx, int ny, int nz, const double *xc, const double *yc, const double *zc,
                const double *xs, const double *ys, const double *zs, int nbg,
                const double *bg_thick, int nmeas, const double *mx, const double *my,
                const double *mz, int kind, double inc, double dec, double fs, int transform,
                double t_inc, double t_dec, int nthreads, const double *model, double *data,
                double *sens)
{
  orc_problem p = make_problem(nx, ny, nz, xc, yc, zc, xs, ys, zs, nbg, bg_thick, nmeas, mx,
                               my, mz, kind, inc, dec, fs, transform, t_inc, t_dec, nthreads);
  const int ngrid = nx * ny * nz;
  const size_t ncol = ncols_of(kind, ngrid, nbg);
  const int raw = raw_per_meas(kind);
  const int dpm = out_per_meas(&p);
  const double xw = width_sum(xs, nx), yw = width_sum(ys, ny), zw = width_sum(zs, nz);
  for (int s = 0; s < nmeas; ++s) {
    double g[9], b[9], cur[9];
    double *rows = sens ? sens + (size_t)s * raw * ncol : NULL;
    gridded(&p, s, model, g, rows, ncol);
    background(&p, s, xw, yw, zw, model + ngrid, b, rows, ncol, ngrid);
    for (int c = 0; c < raw; ++c)
      cur[c] = g[c] + b[c];
    if (transform != ORC_T_NONE)
      data[s] = apply_transform(&p, cur);
    else
      for (int c = 0; c < raw; ++c)
        data[(size_t)s * dpm + c] = cur[c];
  }
  return 0;
}

/* Least-squares derivative 2 * sum_i (T_i' J_i)^T misfit_i, the matrix-free
 * loop of GravMag/ThreeDGravMagImplementation.h:177-231.  With `data` not
 * NULL the same station loop also stores the forward response, as
 * orc_forward computes it (the rows and the gridded + background sums of a
 * station are the same in both loops), so that a test needs one pass over
 * the box terms for both outputs. */
int orc_forward_lqderivative(int nx, int ny, int nz, const double *xc, const double *yc,
                             const double *zc, const double *xs, const double *ys,
                             const double *zs, int nbg, const double *bg_thick, int nmeas,
                             const double *mx, const double *my, const double *mz, int kind,
                             double inc, double dec, double fs, int transform, double t_inc,
                             double t_dec, int nthreads, const double *model,
                             const double *misfit, double *data, double *grad)
{
  orc_problem p = make_problem(nx, ny, nz, xc, yc, zc, xs, ys, zs, nbg, bg_thick, nmeas, mx,
                               my, mz, kind, inc, dec, fs, transform, t_inc, t_dec, nthreads);
  const int ngrid = nx * ny * nz;
  const size_t ncol = ncols_of(kind, ngrid, nbg);
  const int raw = raw_per_meas(kind);
  const int dpm = out_per_meas(&p);
  const double xw = width_sum(xs, nx), yw = width_sum(ys, ny), zw = width_sum(zs, nz);
  double *rows = (double *)malloc(sizeof(double) * raw * ncol);
  if (!rows)
    return 3;
  for (size_t c = 0; c < ncol; ++c)
    grad[c] = 0.0;
  for (int s = 0; s < nmeas; ++s) {
    double g[9], b[9], cur[9];
    gridded(&p, s, model, g, rows, ncol);
    background(&p, s, xw, yw, zw, model + ngrid, b, rows, ncol, ngrid);
    for (int c = 0; c < raw; ++c)
      cur[c] = g[c] + b[c];
    if (data) {
      if (transform != ORC_T_NONE)
        data[s] = apply_transform(&p, cur);
      else
        for (int c = 0; c < raw; ++c)
          data[(size_t)s * dpm + c] = cur[c];
    }
    if (transform != ORC_T_NONE) {
      /* NewSensitivities = TransDeriv * CurrentSensitivities (1 x raw times raw x ncol) */
      double d[9];
      transform_derivative(&p, cur, d);
      const double w = misfit[s];
      for (size_t col = 0; col < ncol; ++col) {
        double v = 0.0;
        for (int c = 0; c < raw; ++c)
          v += d[c] * rows[(size_t)c * ncol + col];
        grad[col] += w * v;
      }
    } else {
      for (int c = 0; c < raw; ++c) {
        const double w = misfit[(size_t)s * dpm + c];
        const double *row = rows + (size_t)c * ncol;
        for (size_t col = 0; col < ncol; ++col)
          grad[col] += w * row[col];
      }
    }
  }
  for (size_t c = 0; c < ncol; ++c)
    grad[c] = 2.0 * grad[c];
  free(rows);
  return 0;
}

int orc_lqderivative(int nx, int ny, int nz, const double *xc, const double *yc,
                     const double *zc, const double *xs, const double *ys, const double *zs,
                     int nbg, const double *bg_thick, int nmeas, const double *mx,
                     const double *my, const double *mz, int kind, double inc, double dec,
                     double fs, int transform, double t_inc, double t_dec, int nthreads,
                     const double *model, const double *misfit, double *grad)
{
  return orc_forward_lqderivative(nx, ny, nz, xc, yc, zc, xs, ys, zs, nbg, bg_thick, nmeas, mx,
                                  my, mz, kind, inc, dec, fs, transform, t_inc, t_dec, nthreads,
                                  model, misfit, NULL, grad);
}

/* Cached-sensitivity products of GravMag/FullSensitivityGravMagCalculator.h:
 * raw data = J m (136-152) and 2 J^T r (214-221), J row-major nrow x ncol.
 * The J^T r accumulation runs over rows in order, as ublas prod(trans(J), r). */
void orc_sens_matvec(int nrow, int ncol, const double *J, const double *m, double *d)
{
  for (int i = 0; i < nrow; ++i) {
    double v = 0.0;
    const double *row = J + (size_t)i * ncol;
    for (int c = 0; c < ncol; ++c)
      v += row[c] * m[c];
    d[i] = v;
  }
}

void orc_sens_rmatvec2(int nrow, int ncol, const double *J, const double *r, double *g)
{
  for (int c = 0; c < ncol; ++c)
    g[c] = 0.0;
  for (int i = 0; i < nrow; ++i) {
    const double *row = J + (size_t)i * ncol;
    for (int c = 0; c < ncol; ++c)
      g[c] += row[c] * r[i];
  }
  for (int c = 0; c < ncol; ++c)
    g[c] = 2.0 * g[c];
}

int orc_version(void) { return 1; }
