// capi.cu -- the C ABI of include/jif3d_gb300.h: context, geometry upload,
// scratch management and the forward / adjoint / sensitivity drivers.
//
// The reference's CUDA layer (Gravity/gravcuda.cu) allocates and frees its
// buffers on every Calculate and launches one kernel per station followed by a
// blocking copy of the whole sensitivity row to the host.  Here the geometry
// stays resident in the context, all stations go in one launch, the
// reduction with the model happens on the device, and only data / gradients
// cross to the host (sensitivity rows only when asked for).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/jif3d_gb300.h"
#include "prism_kernels.h"

using namespace j3g;

namespace {

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
};

}  // namespace

struct j3g_context {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;

  // geometry (host copies)
  int nx = 0, ny = 0, nz = 0;
  bool mesh_set = false;
  bool node_exact = true;
  std::vector<double> X, Y, Z, xs, ys, zs;
  double xw = 0, yw = 0, zw = 0;
  std::vector<double> bg;
  int nmeas = 0;
  bool stations_set = false;
  int kind = 0;
  double inc = 0, dec = 0, fs = 0;
  int transform = J3G_T_NONE;
  double tinc = 0, tdec = 0;
  bool bg_dirty = true;
  long long launches = 0;  // kernels queued by this context

  // device copies of the geometry
  DevBuf dX, dY, dZ, dxs, dys, dzs, dbg, dsx, dsy, dsz;
  // scratch
  DevBuf model, data, misfit, grad, rhot, partial, comps, bgsens, rawd, wraw, W, Gpart, G, F,
      rows, rowsum, probe;

  long long ngrid() const { return (long long)nx * ny * nz; }
  long long nparm() const { return ngrid() + (long long)bg.size(); }
  long long nnodes() const { return (long long)(nx + 1) * (ny + 1) * (nz + 1); }
  int raw() const { return kind_raw(kind); }
  int dpm() const { return transform == J3G_T_NONE ? raw() : 1; }
};

namespace {

int fail(j3g_context *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(j3g_context *c, cudaError_t e, const char *where) {
  return fail(c, J3G_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define J3G_CUDA(ctx, call)                                 \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

// A launcher call: check its error and count the kernels it queued (each
// launcher queues one kernel; the two-kernel launchers add one more below).
#define J3G_LAUNCH(ctx, call)                               \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    ++(ctx)->launches;                                      \
  } while (0)

int ensure(j3g_context *c, DevBuf &b, size_t bytes) {
  if (bytes == 0) bytes = 8;
  if (b.cap >= bytes) return J3G_OK;
  if (b.p) {
    cudaError_t e = cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaFree");
  }
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    b.p = nullptr;
    cudaGetLastError();
    return fail(c, J3G_ERR_NOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
  }
  b.cap = bytes;
  return J3G_OK;
}

#define J3G_TRY(expr)              \
  do {                             \
    int rc_ = (expr);              \
    if (rc_ != J3G_OK) return rc_; \
  } while (0)

template <class T> T *ptr(DevBuf &b) { return static_cast<T *>(b.p); }

int upload(j3g_context *c, DevBuf &b, const std::vector<double> &v) {
  J3G_TRY(ensure(c, b, v.size() * sizeof(double)));
  if (!v.empty())
    J3G_CUDA(c, cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(double),
                                cudaMemcpyHostToDevice, c->stream));
  return J3G_OK;
}

MeshView mesh_view(j3g_context *c) {
  MeshView m;
  m.nx = c->nx;
  m.ny = c->ny;
  m.nz = c->nz;
  m.X = ptr<double>(c->dX);
  m.Y = ptr<double>(c->dY);
  m.Z = ptr<double>(c->dZ);
  m.xs = ptr<double>(c->dxs);
  m.ys = ptr<double>(c->dys);
  m.zs = ptr<double>(c->dzs);
  return m;
}

StationView station_view(j3g_context *c) {
  StationView s;
  s.n = c->nmeas;
  s.x = ptr<double>(c->dsx);
  s.y = ptr<double>(c->dsy);
  s.z = ptr<double>(c->dsz);
  return s;
}

MagField mag_field(const j3g_context *c) {
  MagField m;
  // Magnetics/OMPMagneticSusceptibilityImp.cpp:116-118 and :160
  m.bx = std::cos(c->inc) * std::cos(c->dec);
  m.by = std::cos(c->inc) * std::sin(c->dec);
  m.bz = std::sin(c->inc);
  m.fs = c->fs;
  m.factor = 1.0 / (4 * 3.141592653589793238462643383279502884 * kGravConst);
  return m;
}

void tfa_dir(const j3g_context *c, double &bx, double &by, double &bz) {
  // Magnetics/MagneticTransforms.h:146-152
  bx = std::cos(c->tinc) * std::cos(c->tdec);
  by = std::cos(c->tinc) * std::sin(c->tdec);
  bz = std::sin(c->tinc);
}

int check_ready(j3g_context *c) {
  if (!c) return J3G_ERR_ARG;
  if (!c->mesh_set) return fail(c, J3G_ERR_STATE, "mesh not set");
  if (!c->stations_set) return fail(c, J3G_ERR_STATE, "stations not set");
  if (c->kind == 0) return fail(c, J3G_ERR_STATE, "kind not set");
  if (c->ngrid() > (long long)0x7fffffff || c->nnodes() > (long long)0x7fffffff)
    return fail(c, J3G_ERR_ARG, "mesh too large (more than 2^31 cells or nodes)");
  return J3G_OK;
}

// Background sensitivities of every station (cached until geometry changes).
int ensure_background(j3g_context *c) {
  const int nbg = (int)c->bg.size();
  if (nbg == 0) return J3G_OK;
  if (!c->bg_dirty) return J3G_OK;
  J3G_TRY(ensure(c, c->bgsens, sizeof(double) * (size_t)c->nmeas * c->raw() * nbg));
  if (c->nmeas > 0) {
    // model origin = first corner coordinate (ThreeDModelBase::GetXOrigin)
    const double xo = c->X[0], yo = c->Y[0], zo = c->Z[0];
    J3G_LAUNCH(c, launch_background(c->kind, mesh_view(c), station_view(c), nbg, ptr<double>(c->dbg),
                                  xo, yo, zo, c->xw, c->yw, c->zw, mag_field(c),
                                  ptr<double>(c->bgsens), c->stream));
  }
  c->bg_dirty = false;
  return J3G_OK;
}

constexpr int kTargetBlocks = 152 * 8;

// Gridded node-component sums comps[nmeas][NC_COUNT] for the model d_model.
int gridded_node_forward(j3g_context *c, const double *d_model) {
  const long long nn = c->nnodes();
  J3G_TRY(ensure(c, c->rhot, sizeof(double) * nn));
  MeshView m = mesh_view(c);
  J3G_LAUNCH(c, launch_rho_tilde(m, d_model, ptr<double>(c->rhot), c->stream));
  int npb = 2048, spb = 4;
  auto blocks = [&](int a, int b) {
    return ((nn + a - 1) / a) * (long long)((c->nmeas + b - 1) / b);
  };
  while (npb > 256 && blocks(npb, spb) < kTargetBlocks) npb >>= 1;
  while (spb > 1 && blocks(npb, spb) < kTargetBlocks) spb >>= 1;
  const int nblk = (int)((nn + npb - 1) / npb);
  const int ncomp = kind_ncomp(c->kind);
  J3G_TRY(ensure(c, c->partial, sizeof(double) * (size_t)nblk * c->nmeas * ncomp));
  J3G_TRY(ensure(c, c->comps, sizeof(double) * (size_t)c->nmeas * NC_COUNT));
  J3G_LAUNCH(c, launch_node_forward(c->kind, m, station_view(c), ptr<double>(c->rhot),
                                  ptr<double>(c->partial), nblk, npb, spb, c->stream));
  J3G_LAUNCH(c, launch_forward_reduce(c->kind, c->nmeas, nblk, ptr<double>(c->partial),
                                    ptr<double>(c->comps), c->stream));
  return J3G_OK;
}

// Station chunk for row generation, bounded by ~1 GiB of row scratch.
int row_chunk(j3g_context *c, long long ld) {
  const long long per = (long long)c->raw() * ld * 8 +
                        (c->node_exact ? (long long)kind_ncomp(c->kind) * c->nnodes() * 8 : 0);
  long long ch = (1LL << 30) / (per > 0 ? per : 1);
  if (ch < 1) ch = 1;
  if (ch > c->nmeas) ch = c->nmeas;
  if (ch > 65535) ch = 65535;
  return (int)ch;
}

// Raw gridded data from explicit sensitivity rows: rowsum[nmeas][raw].
// Optionally copies each chunk's rows (with background columns) to h_sens.
int gridded_rows_forward(j3g_context *c, const double *d_model, double *h_sens) {
  const long long ngrid = c->ngrid(), nparm = c->nparm();
  const int raw = c->raw(), nbg = (int)c->bg.size();
  const long long ld = h_sens ? nparm : ngrid;
  const int chunk = row_chunk(c, ld);
  J3G_TRY(ensure(c, c->rows, sizeof(double) * (size_t)chunk * raw * ld));
  if (c->node_exact)
    J3G_TRY(ensure(c, c->F, sizeof(double) * (size_t)chunk * kind_ncomp(c->kind) * c->nnodes()));
  J3G_TRY(ensure(c, c->rowsum, sizeof(double) * (size_t)c->nmeas * raw));
  MeshView m = mesh_view(c);
  StationView s = station_view(c);
  const MagField mf = mag_field(c);
  for (int s0 = 0; s0 < c->nmeas; s0 += chunk) {
    const int ns = std::min(chunk, c->nmeas - s0);
    if (ngrid > 0) {
      J3G_LAUNCH(c, launch_sens_rows(c->kind, c->node_exact, m, s, s0, ns, mf, ptr<double>(c->F),
                                   ptr<double>(c->rows), ld, c->stream));
      if (c->node_exact) ++c->launches;  // node terms + cell combine
      J3G_LAUNCH(c, launch_rows_dot(raw, ns, ngrid, ptr<double>(c->rows), ld, d_model,
                                  ptr<double>(c->rowsum) + (size_t)s0 * raw, c->stream));
    } else {
      J3G_CUDA(c, cudaMemsetAsync(ptr<double>(c->rowsum) + (size_t)s0 * raw, 0,
                                  sizeof(double) * ns * raw, c->stream));
    }
    if (h_sens) {
      if (nbg > 0)
        J3G_CUDA(c, cudaMemcpy2DAsync(ptr<double>(c->rows) + ngrid, ld * sizeof(double),
                                      ptr<double>(c->bgsens) + (size_t)s0 * raw * nbg,
                                      nbg * sizeof(double), nbg * sizeof(double),
                                      (size_t)ns * raw, cudaMemcpyDeviceToDevice, c->stream));
      J3G_CUDA(c, cudaMemcpyAsync(h_sens + (size_t)s0 * raw * nparm, c->rows.p,
                                  sizeof(double) * (size_t)ns * raw * nparm,
                                  cudaMemcpyDeviceToHost, c->stream));
      J3G_CUDA(c, cudaStreamSynchronize(c->stream));
    }
  }
  return J3G_OK;
}

// Forward with every buffer on the device.  raw_out (device, nmeas*raw) optional.
int forward_device(j3g_context *c, const double *d_model, double *d_data, double *raw_out,
                   double *h_sens) {
  J3G_TRY(check_ready(c));
  if (c->nmeas == 0) return J3G_OK;
  J3G_TRY(ensure_background(c));
  double tbx, tby, tbz;
  tfa_dir(c, tbx, tby, tbz);
  const int nbg = (int)c->bg.size();
  const double *bgval = d_model + c->ngrid();
  const double *bgsens = nbg ? ptr<double>(c->bgsens) : nullptr;
  if (h_sens || (!c->node_exact && c->ngrid() > 0)) {
    J3G_TRY(gridded_rows_forward(c, d_model, h_sens));
    J3G_LAUNCH(c, launch_assemble(c->kind, c->transform, tbx, tby, tbz, c->nmeas,
                                ptr<double>(c->rowsum), c->raw(), bgsens, nbg, bgval,
                                mag_field(c), raw_out, d_data, c->stream));
  } else {
    if (c->ngrid() > 0) {
      J3G_TRY(gridded_node_forward(c, d_model));
    } else {
      J3G_TRY(ensure(c, c->comps, sizeof(double) * (size_t)c->nmeas * NC_COUNT));
      J3G_CUDA(c, cudaMemsetAsync(c->comps.p, 0, sizeof(double) * c->nmeas * NC_COUNT, c->stream));
    }
    J3G_LAUNCH(c, launch_assemble(c->kind, c->transform, tbx, tby, tbz, c->nmeas,
                                ptr<double>(c->comps), NC_COUNT, bgsens, nbg, bgval, mag_field(c),
                                raw_out, d_data, c->stream));
  }
  return J3G_OK;
}

int adjoint_device(j3g_context *c, const double *d_model, const double *d_misfit,
                   double *d_grad) {
  J3G_TRY(check_ready(c));
  const long long ngrid = c->ngrid(), nparm = c->nparm();
  if (c->nmeas == 0) {
    J3G_CUDA(c, cudaMemsetAsync(d_grad, 0, sizeof(double) * (size_t)nparm, c->stream));
    return J3G_OK;
  }
  J3G_TRY(ensure_background(c));
  const int raw = c->raw(), nbg = (int)c->bg.size();
  double tbx, tby, tbz;
  tfa_dir(c, tbx, tby, tbz);
  const double *rawd = nullptr;
  if (c->transform == J3G_T_FTG_INVARIANT || c->transform == J3G_T_TOTAL_FIELD) {
    // non-linear transforms need the raw data at the current model
    J3G_TRY(ensure(c, c->rawd, sizeof(double) * (size_t)c->nmeas * raw));
    J3G_TRY(ensure(c, c->data, sizeof(double) * (size_t)c->nmeas * c->dpm()));
    J3G_TRY(forward_device(c, d_model, ptr<double>(c->data), ptr<double>(c->rawd), nullptr));
    rawd = ptr<double>(c->rawd);
  }
  J3G_TRY(ensure(c, c->wraw, sizeof(double) * (size_t)c->nmeas * raw));
  J3G_LAUNCH(c, launch_backproject(c->kind, c->transform, tbx, tby, tbz, c->nmeas, d_misfit, rawd,
                                 ptr<double>(c->wraw), c->stream));
  MeshView m = mesh_view(c);
  StationView s = station_view(c);
  if (ngrid > 0 && c->node_exact) {
    J3G_TRY(ensure(c, c->W, sizeof(double) * (size_t)c->nmeas * NC_COUNT));
    J3G_LAUNCH(c, launch_comp_weights(c->kind, c->nmeas, ptr<double>(c->wraw), mag_field(c),
                                    ptr<double>(c->W), c->stream));
    const long long nn = c->nnodes();
    const long long nodeblocks = (nn + 255) / 256;
    long long want = (kTargetBlocks + nodeblocks - 1) / nodeblocks;
    long long maxchunk = (c->nmeas + 15) / 16;
    int nchunk = (int)std::max(1LL, std::min(want, maxchunk));
    const int spc = (c->nmeas + nchunk - 1) / nchunk;
    nchunk = (c->nmeas + spc - 1) / spc;
    J3G_TRY(ensure(c, c->Gpart, sizeof(double) * (size_t)nchunk * nn));
    J3G_TRY(ensure(c, c->G, sizeof(double) * (size_t)nn));
    J3G_LAUNCH(c, launch_node_adjoint(c->kind, m, s, ptr<double>(c->W), spc, nchunk,
                                    ptr<double>(c->Gpart), c->stream));
    J3G_LAUNCH(c, launch_adjoint_combine(m, nchunk, ptr<double>(c->Gpart), ptr<double>(c->G),
                                       d_grad, c->stream));
    ++c->launches;  // chunk sum + cell combine
  } else if (ngrid > 0) {
    // eight-corner rows, accumulated chunk by chunk
    J3G_CUDA(c, cudaMemsetAsync(d_grad, 0, sizeof(double) * (size_t)ngrid, c->stream));
    const int chunk = row_chunk(c, ngrid);
    J3G_TRY(ensure(c, c->rows, sizeof(double) * (size_t)chunk * raw * ngrid));
    const MagField mf = mag_field(c);
    for (int s0 = 0; s0 < c->nmeas; s0 += chunk) {
      const int ns = std::min(chunk, c->nmeas - s0);
      J3G_LAUNCH(c, launch_sens_rows(c->kind, false, m, s, s0, ns, mf, nullptr,
                                   ptr<double>(c->rows), ngrid, c->stream));
      J3G_LAUNCH(c, launch_rows_tdot(ns * raw, ngrid, ptr<double>(c->rows), ngrid,
                                   ptr<double>(c->wraw) + (size_t)s0 * raw, d_grad, c->stream));
    }
    J3G_LAUNCH(c, launch_scale(ngrid, 2.0, d_grad, c->stream));
  }
  if (nbg > 0)
    J3G_LAUNCH(c, launch_background_grad(c->kind, c->nmeas, nbg, ptr<double>(c->wraw),
                                       ptr<double>(c->bgsens), d_grad + ngrid, c->stream));
  return J3G_OK;
}

bool valid_kind(int k) { return k >= J3G_SCALAR && k <= J3G_JOINT; }

}  // namespace

// ===========================================================================
extern "C" {

const char *j3g_status_string(int status) {
  switch (status) {
    case J3G_OK: return "ok";
    case J3G_ERR_ARG: return "invalid argument";
    case J3G_ERR_CUDA: return "CUDA error";
    case J3G_ERR_NOMEM: return "out of memory";
    case J3G_ERR_STATE: return "context not ready";
    case J3G_ERR_UNSUPPORTED: return "unsupported combination";
    case J3G_ERR_SCRATCH_LIMIT: return "problem exceeds the fixed scratch of j3g_forward_noalloc";
    default: return "unknown status";
  }
}

const char *j3g_last_error(const j3g_context *ctx) { return ctx ? ctx->err.c_str() : ""; }

int j3g_create(j3g_context **out, int device) {
  if (!out) return J3G_ERR_ARG;
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return J3G_ERR_CUDA;
  }
  if (device < 0 || device >= count) return J3G_ERR_ARG;
  j3g_context *c = new (std::nothrow) j3g_context();
  if (!c) return J3G_ERR_NOMEM;
  c->device = device;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return J3G_ERR_CUDA;
  }
  c->stream = c->own_stream;
  *out = c;
  return J3G_OK;
}

int j3g_destroy(j3g_context *c) {
  if (!c) return J3G_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  DevBuf *bufs[] = {&c->dX, &c->dY, &c->dZ, &c->dxs, &c->dys, &c->dzs, &c->dbg, &c->dsx,
                    &c->dsy, &c->dsz, &c->model, &c->data, &c->misfit, &c->grad, &c->rhot,
                    &c->partial, &c->comps, &c->bgsens, &c->rawd, &c->wraw, &c->W, &c->Gpart,
                    &c->G, &c->F, &c->rows, &c->rowsum, &c->probe};
  for (DevBuf *b : bufs)
    if (b->p) cudaFree(b->p);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
  return J3G_OK;
}

int j3g_set_stream(j3g_context *c, void *stream) {
  if (!c) return J3G_ERR_ARG;
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  return J3G_OK;
}

int j3g_set_mesh(j3g_context *c, int nx, int ny, int nz, const double *xc, const double *yc,
                 const double *zc, const double *xs, const double *ys, const double *zs) {
  if (!c) return J3G_ERR_ARG;
  if (nx < 0 || ny < 0 || nz < 0) return fail(c, J3G_ERR_ARG, "negative mesh size");
  const bool empty = (nx == 0 || ny == 0 || nz == 0);
  if (!empty && (!xc || !yc || !zc || !xs || !ys || !zs))
    return fail(c, J3G_ERR_ARG, "null coordinate or size array");
  cudaSetDevice(c->device);
  c->nx = empty ? 0 : nx;
  c->ny = empty ? 0 : ny;
  c->nz = empty ? 0 : nz;
  auto nodes = [&](int n, const double *co, const double *sz, std::vector<double> &N,
                   std::vector<double> &S, double &width) {
    N.assign(n + 1, 0.0);
    S.assign(sz, sz + n);
    // the origin of an empty axis is 0 (ThreeDModelBase::GetXOrigin)
    if (n == 0) {
      N[0] = co ? co[0] : 0.0;
      width = 0.0;
      return true;
    }
    bool exact = true;
    for (int i = 0; i < n; ++i) N[i] = co[i];
    // the upper corner of the last cell is the reference's ul_corner + size
    N[n] = co[n - 1] + sz[n - 1];
    for (int i = 0; i + 1 < n; ++i)
      if (!(co[i] + sz[i] == co[i + 1])) exact = false;
    width = 0.0;  // std::accumulate over the sizes (ThreeDGravMagImplementation.h:132-137)
    for (int i = 0; i < n; ++i) width += sz[i];
    return exact;
  };
  bool ex = true;
  ex &= nodes(c->nx, empty ? (xc ? xc : nullptr) : xc, xs, c->X, c->xs, c->xw);
  ex &= nodes(c->ny, empty ? (yc ? yc : nullptr) : yc, ys, c->Y, c->ys, c->yw);
  ex &= nodes(c->nz, empty ? (zc ? zc : nullptr) : zc, zs, c->Z, c->zs, c->zw);
  c->node_exact = ex;
  J3G_TRY(upload(c, c->dX, c->X));
  J3G_TRY(upload(c, c->dY, c->Y));
  J3G_TRY(upload(c, c->dZ, c->Z));
  J3G_TRY(upload(c, c->dxs, c->xs));
  J3G_TRY(upload(c, c->dys, c->ys));
  J3G_TRY(upload(c, c->dzs, c->zs));
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  c->mesh_set = true;
  c->bg_dirty = true;
  return J3G_OK;
}

int j3g_set_background(j3g_context *c, int nbg, const double *thick) {
  if (!c) return J3G_ERR_ARG;
  if (nbg < 0 || (nbg > 0 && !thick)) return fail(c, J3G_ERR_ARG, "bad background arrays");
  cudaSetDevice(c->device);
  c->bg.assign(thick, thick + nbg);
  J3G_TRY(upload(c, c->dbg, c->bg));
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  c->bg_dirty = true;
  return J3G_OK;
}

int j3g_set_stations(j3g_context *c, int n, const double *x, const double *y, const double *z) {
  if (!c) return J3G_ERR_ARG;
  if (n < 0 || (n > 0 && (!x || !y || !z))) return fail(c, J3G_ERR_ARG, "bad station arrays");
  cudaSetDevice(c->device);
  std::vector<double> vx(x, x + n), vy(y, y + n), vz(z, z + n);
  J3G_TRY(upload(c, c->dsx, vx));
  J3G_TRY(upload(c, c->dsy, vy));
  J3G_TRY(upload(c, c->dsz, vz));
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  c->nmeas = n;
  c->stations_set = true;
  c->bg_dirty = true;
  return J3G_OK;
}

int j3g_set_kind(j3g_context *c, int kind, double inc, double dec, double fs) {
  if (!c) return J3G_ERR_ARG;
  if (!valid_kind(kind)) return fail(c, J3G_ERR_ARG, "unknown kind");
  c->kind = kind;
  c->inc = inc;
  c->dec = dec;
  c->fs = fs;
  c->bg_dirty = true;
  if (c->transform != J3G_T_NONE) {
    const bool ok = (c->transform == J3G_T_FTG_INVARIANT && kind == J3G_TENSOR) ||
                    ((c->transform == J3G_T_TOTAL_FIELD || c->transform == J3G_T_TFA) &&
                     kind == J3G_MAGNETIC);
    if (!ok) c->transform = J3G_T_NONE;
  }
  return J3G_OK;
}

int j3g_set_transform(j3g_context *c, int transform, double inc, double dec) {
  if (!c) return J3G_ERR_ARG;
  if (transform < J3G_T_NONE || transform > J3G_T_TFA)
    return fail(c, J3G_ERR_ARG, "unknown transform");
  if (transform == J3G_T_FTG_INVARIANT && c->kind != J3G_TENSOR)
    return fail(c, J3G_ERR_UNSUPPORTED, "the FTG invariant needs tensor data");
  if ((transform == J3G_T_TOTAL_FIELD || transform == J3G_T_TFA) && c->kind != J3G_MAGNETIC)
    return fail(c, J3G_ERR_UNSUPPORTED, "total-field transforms need magnetic data");
  c->transform = transform;
  c->tinc = inc;
  c->tdec = dec;
  return J3G_OK;
}

int j3g_get_sizes(const j3g_context *c, long long *ngrid, long long *nparm, int *nmeas,
                  int *raw, int *dpm) {
  if (!c) return J3G_ERR_ARG;
  if (ngrid) *ngrid = c->ngrid();
  if (nparm) *nparm = c->nparm();
  if (nmeas) *nmeas = c->nmeas;
  if (raw) *raw = c->kind ? c->raw() : 0;
  if (dpm) *dpm = c->kind ? c->dpm() : 0;
  return J3G_OK;
}

int j3g_forward_device(j3g_context *c, const double *d_model, double *d_data) {
  if (!c || !d_model || !d_data) return fail(c, J3G_ERR_ARG, "null pointer");
  cudaSetDevice(c->device);
  return forward_device(c, d_model, d_data, nullptr, nullptr);
}

int j3g_lqderivative_device(j3g_context *c, const double *d_model, const double *d_misfit,
                            double *d_grad) {
  if (!c || !d_model || !d_misfit || !d_grad) return fail(c, J3G_ERR_ARG, "null pointer");
  cudaSetDevice(c->device);
  return adjoint_device(c, d_model, d_misfit, d_grad);
}

static int host_forward(j3g_context *c, const double *h_model, double *h_data, double *h_sens) {
  if (!c || !h_model || !h_data) return fail(c, J3G_ERR_ARG, "null pointer");
  J3G_TRY(check_ready(c));
  cudaSetDevice(c->device);
  const size_t np = (size_t)c->nparm(), nd = (size_t)c->nmeas * c->dpm();
  J3G_TRY(ensure(c, c->model, sizeof(double) * np));
  J3G_TRY(ensure(c, c->data, sizeof(double) * nd));
  J3G_CUDA(c, cudaMemcpyAsync(c->model.p, h_model, sizeof(double) * np, cudaMemcpyHostToDevice,
                              c->stream));
  J3G_TRY(forward_device(c, ptr<double>(c->model), ptr<double>(c->data), nullptr, h_sens));
  if (nd)
    J3G_CUDA(c, cudaMemcpyAsync(h_data, c->data.p, sizeof(double) * nd, cudaMemcpyDeviceToHost,
                                c->stream));
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  return J3G_OK;
}

int j3g_forward(j3g_context *c, const double *h_model, double *h_data) {
  return host_forward(c, h_model, h_data, nullptr);
}

int j3g_forward_sens(j3g_context *c, const double *h_model, double *h_data, double *h_sens) {
  if (!h_sens) return fail(c, J3G_ERR_ARG, "null sensitivity buffer");
  return host_forward(c, h_model, h_data, h_sens);
}

int j3g_lqderivative(j3g_context *c, const double *h_model, const double *h_misfit,
                     double *h_grad) {
  if (!c || !h_model || !h_misfit || !h_grad) return fail(c, J3G_ERR_ARG, "null pointer");
  J3G_TRY(check_ready(c));
  cudaSetDevice(c->device);
  const size_t np = (size_t)c->nparm(), nd = (size_t)c->nmeas * c->dpm();
  J3G_TRY(ensure(c, c->model, sizeof(double) * np));
  J3G_TRY(ensure(c, c->misfit, sizeof(double) * nd));
  J3G_TRY(ensure(c, c->grad, sizeof(double) * np));
  J3G_CUDA(c, cudaMemcpyAsync(c->model.p, h_model, sizeof(double) * np, cudaMemcpyHostToDevice,
                              c->stream));
  if (nd)
    J3G_CUDA(c, cudaMemcpyAsync(c->misfit.p, h_misfit, sizeof(double) * nd,
                                cudaMemcpyHostToDevice, c->stream));
  J3G_TRY(adjoint_device(c, ptr<double>(c->model), ptr<double>(c->misfit), ptr<double>(c->grad)));
  J3G_CUDA(c, cudaMemcpyAsync(h_grad, c->grad.p, sizeof(double) * np, cudaMemcpyDeviceToHost,
                              c->stream));
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  return J3G_OK;
}

int j3g_launch_count(const j3g_context *c, long long *count) {
  if (!c || !count) return J3G_ERR_ARG;
  *count = c->launches;
  return J3G_OK;
}

int j3g_synchronize(j3g_context *c) {
  if (!c) return J3G_ERR_ARG;
  cudaSetDevice(c->device);
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  return J3G_OK;
}

int j3g_probe_fp64(j3g_context *c, double *gflops) {
  if (!c || !gflops) return J3G_ERR_ARG;
  cudaSetDevice(c->device);
  int sms = 0;
  J3G_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const int threads = 256, blocks = sms * 8, iters = 1 << 14;
  J3G_TRY(ensure(c, c->probe, sizeof(double) * blocks * threads));
  cudaEvent_t a, b;
  J3G_CUDA(c, cudaEventCreate(&a));
  J3G_CUDA(c, cudaEventCreate(&b));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    J3G_CUDA(c, cudaEventRecord(a, c->stream));
    J3G_LAUNCH(c, launch_fp64_probe(ptr<double>(c->probe), blocks, threads, iters, c->stream));
    J3G_CUDA(c, cudaEventRecord(b, c->stream));
    J3G_CUDA(c, cudaEventSynchronize(b));
    float ms = 0;
    J3G_CUDA(c, cudaEventElapsedTime(&ms, a, b));
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  const double flops = 2.0 * 4.0 * iters * (double)blocks * threads;
  *gflops = flops / (best * 1e-3) / 1e9;
  return J3G_OK;
}

}  // extern "C"
