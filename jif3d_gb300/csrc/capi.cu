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

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <array>
#include <functional>
#include <initializer_list>
#include <map>
#include <string>
#include <vector>

#include "../../include/jif3d_gb300.h"
#include "prism_kernels.h"
#include "refine.h"
#include "stored.h"

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

  // device-resident sensitivity (j3g_build_sensitivity)
  int storage = 0;             // 0 none, J3G_STORE_FP32, J3G_STORE_F16X2
  long long st_rows = 0;       // nmeas * stored rows per station
  long long st_ld = 0;         // cells padded to a multiple of 64
  long long st_ldT = 0;        // rows padded to a multiple of 64 (transposed copy)
  DevBuf J32, Jhi, Jlo, JThi, JTlo, rowscale, Jrowsum;
  DevBuf x32, sums, part, Bhi, Blo, P, wst, wrawb, rawb, gerr, mscale, mmean, swork, sexp;

  // tensor-core product plans (j3g_set_autotune): key direction, rows, padded
  // models, K; the plan last used per direction is kept for j3g_get_gemm_plan
  struct GemmPlan {
    int nsplit = 0, tile = 0;
    float ms = 0.0f;  // timed by the autotuner (0 for the fixed rule)
  };
  bool autotune = false;
  bool pinned[2] = {false, false};  // plans fixed by j3g_set_gemm_plan, per direction
  GemmPlan pinned_plan[2];

  // station subsets (j3g_subsets_*): a context over the concatenated subset
  // stations, rebuilt when the subsets or this context's setup change
  long long gen = 0;  // bumped by every set_* call
  // bumped by everything a captured product depends on beyond its arguments:
  // set_* calls, buffer (re)allocation, product plans, timing
  long long prod_gen = 0;
  std::vector<double> hsx, hsy, hsz;
  j3g_context *child = nullptr;
  std::vector<int> child_off, child_idx;
  long long child_gen = -1;
  DevBuf chunks;  // chunk station ranges of a subset adjoint
  std::vector<int> chunks_h;  // the table now in chunks
  std::map<std::array<long long, 4>, GemmPlan> plans;
  GemmPlan last_plan[2];

  // model refinement (j3g_set_refinement): the coarse (inversion) grid over
  // this context's mesh, as the cell walks of the three axes on the device
  bool refine_set = false;
  bool refine_covers_all = true;  // every mesh cell belongs to a coarse cell
  int cn[3] = {0, 0, 0};
  DevBuf rmaps, rcoarse, rfine;
  RefineMaps rm{};

  // pipelined host-buffer products (j3g_batched_*_async): inputs copied in and
  // outputs out on copy streams of the call's direction, the products on the
  // context's stream; a ring of device slots lets one call's copies overlap
  // another call's work
  struct Slot {
    DevBuf in, in2, out;
    cudaEvent_t h2d = nullptr, done = nullptr, d2h = nullptr;
    int *flag = nullptr;    // page-locked copy of the tensor-core error flag
    long long ticket = -1;  // call in flight in this slot, -1 if free
    // per direction (forward, derivative): the product replayed as a CUDA
    // graph, valid while prod_gen and the model count are those it was
    // captured under, and the state of the last eager product
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    long long exec_gen[2] = {-1, -1}, exec_launches[2] = {0, 0};
    int exec_nmod[2] = {0, 0};
    long long warm_gen[2] = {-1, -1};
    int warm_nmod[2] = {0, 0};
  };
  static constexpr int kSlots = 4;
  Slot slots[kSlots];
  // copy streams per direction (forward, derivative): a forward's data (a few
  // MB) does not queue behind a derivative's gradients (the size of the
  // models) on the way out, nor a derivative's misfits behind a forward's
  // models on the way in
  cudaStream_t h2d_stream[2] = {nullptr, nullptr}, d2h_stream[2] = {nullptr, nullptr};
  long long next_ticket = 0;
  // failure codes of calls whose slot was reused before they were waited for
  std::map<long long, int> failed_tickets;
  // j3g_set_test_fault: the fault the tensor-core launches simulate (0: none)
  int test_fault = 0;

  // optional per-category kernel timing (j3g_set_timing): event pairs
  // recorded on the context's stream around the dominant launches
  bool timing = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> timed;

  long long ngrid() const { return (long long)nx * ny * nz; }
  // model blocks: magnetisation has three cell blocks and no background
  // parameters (Magnetics/ThreeDMagnetizationModel.h:66-69)
  long long nparm() const {
    return kind == J3G_MAGNETIZATION ? 3 * ngrid() : ngrid() + (long long)bg.size();
  }
  long long ngrid_cols() const { return (long long)kind_nblock(kind) * ngrid(); }
  // background layers that respond (none for the vertical gradient and
  // magnetisation: OMPMagneticGradImp.h:32-40, OMPMagnetizationImp.cpp:16-22)
  int nbg_active() const { return kind_special(kind) ? 0 : (int)bg.size(); }
  // background parameters of a model; those of the vertical gradient have
  // no response, so their gradient entries are zero
  int nbg_params() const { return (int)(nparm() - ngrid_cols()); }
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

// Records a start event now and a stop event when it goes out of scope, if
// the context's timing is on.
struct TimedScope {
  j3g_context *c;
  int cat;
  cudaEvent_t a = nullptr, b = nullptr;
  TimedScope(j3g_context *ctx, int category) : c(ctx), cat(category) {
    if (!c->timing) return;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
      a = b = nullptr;
      return;
    }
    cudaEventRecord(a, c->stream);
  }
  ~TimedScope() {
    if (!a) return;
    cudaEventRecord(b, c->stream);
    c->timed.push_back({cat, {a, b}});
  }
};

int ensure(j3g_context *c, DevBuf &b, size_t bytes) {
  if (bytes == 0) bytes = 8;
  if (b.cap >= bytes) return J3G_OK;
  if (b.p) {
    cudaError_t e = cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaFree");
  }
  ++c->prod_gen;  // captured products hold the old address
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
  const double pi = 3.141592653589793238462643383279502884;
  if (c->kind == J3G_MAG_GRADIENT) {
    m.factor = 1e-7 / kGravConst;  // Magnetics/OMPMagneticGradImp.cpp:66
  } else if (c->kind == J3G_MAGNETIZATION) {
    const double mag_mu = 4e-7 * pi;  // Magnetics/OMPMagnetizationImp.cpp:29, 58-59
    m.factor = 1.0e9 * mag_mu / (4 * pi * kGravConst);
  } else {
    m.factor = 1.0 / (4 * pi * kGravConst);
  }
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
  const int nbg = c->nbg_active();
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
  const int nblock = kind_nblock(c->kind);
  J3G_TRY(ensure(c, c->rhot, sizeof(double) * nn * nblock));
  MeshView m = mesh_view(c);
  for (int b = 0; b < nblock; ++b)
    J3G_LAUNCH(c, launch_rho_tilde(m, d_model + (size_t)b * c->ngrid(),
                                   ptr<double>(c->rhot) + (size_t)b * nn, c->stream));
  int npb = 2048, spb = 4;
  auto blocks = [&](int a, int b) {
    return ((nn + a - 1) / a) * (long long)((c->nmeas + b - 1) / b);
  };
  while (npb > 256 && blocks(npb, spb) < kTargetBlocks) npb >>= 1;
  while (spb > 1 && blocks(npb, spb) < kTargetBlocks) spb >>= 1;
  // station blocks run over grid y: at most 65535 of them
  spb = std::max(spb, (c->nmeas + 65534) / 65535);
  const int nblk = (int)((nn + npb - 1) / npb);
  const int ncomp = kind_ncomp(c->kind);
  J3G_TRY(ensure(c, c->partial, sizeof(double) * (size_t)nblk * c->nmeas * ncomp));
  J3G_TRY(ensure(c, c->comps, sizeof(double) * (size_t)c->nmeas * NC_COUNT));
  {
    TimedScope ts(c, J3G_TIMER_NODE_FORWARD);
    J3G_LAUNCH(c, launch_node_forward(c->kind, m, station_view(c), ptr<double>(c->rhot),
                                      ptr<double>(c->partial), nblk, npb, spb, c->stream));
  }
  J3G_LAUNCH(c, launch_forward_reduce(c->kind, c->nmeas, nblk, ptr<double>(c->partial),
                                      mag_field(c), ptr<double>(c->comps), c->stream));
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
  const long long ngrid = c->ngrid(), nparm = c->nparm(), ncolg = c->ngrid_cols();
  const int raw = c->raw(), nbg = c->nbg_active();
  // background columns without a response (vertical gradient) are zero
  const int nbg_zero = c->kind == J3G_MAG_GRADIENT ? (int)c->bg.size() : 0;
  const long long ld = h_sens ? nparm : ncolg;
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
      J3G_LAUNCH(c, launch_rows_dot(raw, ns, ncolg, ptr<double>(c->rows), ld, d_model,
                                  ptr<double>(c->rowsum) + (size_t)s0 * raw, c->stream));
    } else {
      J3G_CUDA(c, cudaMemsetAsync(ptr<double>(c->rowsum) + (size_t)s0 * raw, 0,
                                  sizeof(double) * ns * raw, c->stream));
    }
    if (h_sens) {
      if (nbg_zero > 0)
        J3G_CUDA(c, cudaMemset2DAsync(ptr<double>(c->rows) + ngrid, ld * sizeof(double), 0,
                                      nbg_zero * sizeof(double), (size_t)ns * raw, c->stream));
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
  const int nbg = c->nbg_active();
  const double *bgval = d_model + c->ngrid();
  const double *bgsens = nbg ? ptr<double>(c->bgsens) : nullptr;
  // node sums per station: node components, or raw rows for the special kinds
  const int comps_ld = kind_special(c->kind) ? c->raw() : NC_COUNT;
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
                                ptr<double>(c->comps), comps_ld, bgsens, nbg, bgval, mag_field(c),
                                raw_out, d_data, c->stream));
  }
  return J3G_OK;
}

// Adjoint of all stations into d_grad, or, with sub (nsub + 1 station
// offsets, sub->back() == nmeas), one gradient per station subset into
// d_grad + k * nparm; the node path then keeps every chunk of stations
// inside one subset and sums each subset's chunks on its own.
int adjoint_device(j3g_context *c, const double *d_model, const double *d_misfit,
                   double *d_grad, const std::vector<int> *sub = nullptr) {
  J3G_TRY(check_ready(c));
  const long long ngrid = c->ngrid(), nparm = c->nparm();
  const std::vector<int> all{0, c->nmeas};
  const std::vector<int> &off = sub ? *sub : all;
  const int nsub = (int)off.size() - 1;
  if (c->nmeas == 0) {
    J3G_CUDA(c, cudaMemsetAsync(d_grad, 0, sizeof(double) * (size_t)nparm * nsub, c->stream));
    return J3G_OK;
  }
  J3G_TRY(ensure_background(c));
  const int raw = c->raw(), nbg = c->nbg_active();
  const long long ncolg = c->ngrid_cols();
  const int nblock = kind_nblock(c->kind);
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
    J3G_TRY(ensure(c, c->W, sizeof(double) * (size_t)c->nmeas * std::max<int>(NC_COUNT, kMaxVc)));
    J3G_LAUNCH(c, launch_comp_weights(c->kind, c->nmeas, ptr<double>(c->wraw), mag_field(c),
                                    ptr<double>(c->W), c->stream));
    const long long nn = c->nnodes();
    const long long nodeblocks = (nn + 255) / 256;
    long long want = (kTargetBlocks + nodeblocks - 1) / nodeblocks;
    long long maxchunk = (c->nmeas + 15) / 16;
    int nchunk = (int)std::max(1LL, std::min(want, maxchunk));
    const int spc = (c->nmeas + nchunk - 1) / nchunk;
    nchunk = (c->nmeas + spc - 1) / spc;
    // chunks of at most spc stations that never straddle a subset
    std::vector<int> starts, first_chunk;
    const int *d_starts = nullptr;
    if (sub) {
      for (int k = 0; k < nsub; ++k) {
        first_chunk.push_back((int)starts.size());
        for (int a = off[k]; a < off[k + 1]; a += spc) starts.push_back(a);
      }
      first_chunk.push_back((int)starts.size());
      starts.push_back(c->nmeas);
      nchunk = (int)starts.size() - 1;
      // uploaded only when the subsets' chunk layout changes: a repeated call
      // on the same subsets queues kernels only (and can be graph-captured)
      if (starts != c->chunks_h) {
        J3G_TRY(ensure(c, c->chunks, sizeof(int) * starts.size()));
        J3G_CUDA(c, cudaMemcpyAsync(c->chunks.p, starts.data(), sizeof(int) * starts.size(),
                                    cudaMemcpyHostToDevice, c->stream));
        J3G_CUDA(c, cudaStreamSynchronize(c->stream));  // the host table is a local
        c->chunks_h = starts;
      }
      d_starts = ptr<int>(c->chunks);
    } else {
      first_chunk = {0, nchunk};
    }
    J3G_TRY(ensure(c, c->Gpart, sizeof(double) * (size_t)std::max(nchunk, 1) * nblock * nn));
    J3G_TRY(ensure(c, c->G, sizeof(double) * (size_t)nblock * nn));
    if (nchunk > 0) {
      TimedScope ts(c, J3G_TIMER_NODE_ADJOINT);
      J3G_LAUNCH(c, launch_node_adjoint(c->kind, m, s, ptr<double>(c->W), spc, nchunk, d_starts,
                                        ptr<double>(c->Gpart), c->stream));
    }
    for (int k = 0; k < nsub; ++k) {
      const int c0 = first_chunk[k], nk = first_chunk[k + 1] - c0;
      J3G_LAUNCH(c, launch_adjoint_combine(m, nk, nblock,
                                           ptr<double>(c->Gpart) + (size_t)c0 * nblock * nn,
                                           ptr<double>(c->G), d_grad + (size_t)k * nparm,
                                           c->stream));
      c->launches += 2 * nblock - 1;  // chunk sum + cell combine per block
    }
  } else if (ngrid > 0) {
    // eight-corner rows, accumulated chunk by chunk within each subset
    const int chunk = row_chunk(c, ncolg);
    J3G_TRY(ensure(c, c->rows, sizeof(double) * (size_t)chunk * raw * ncolg));
    const MagField mf = mag_field(c);
    for (int k = 0; k < nsub; ++k) {
      double *gk = d_grad + (size_t)k * nparm;
      J3G_CUDA(c, cudaMemsetAsync(gk, 0, sizeof(double) * (size_t)ncolg, c->stream));
      for (int s0 = off[k]; s0 < off[k + 1]; s0 += chunk) {
        const int ns = std::min(chunk, off[k + 1] - s0);
        J3G_LAUNCH(c, launch_sens_rows(c->kind, false, m, s, s0, ns, mf, nullptr,
                                     ptr<double>(c->rows), ncolg, c->stream));
        J3G_LAUNCH(c, launch_rows_tdot(ns * raw, ncolg, ptr<double>(c->rows), ncolg,
                                     ptr<double>(c->wraw) + (size_t)s0 * raw, gk, c->stream));
      }
      J3G_LAUNCH(c, launch_scale(ncolg, 2.0, gk, c->stream));
    }
  }
  for (int k = 0; k < nsub; ++k) {
    double *gk = d_grad + (size_t)k * nparm;
    if (c->kind == J3G_MAG_GRADIENT && !c->bg.empty())  // background parameters do not respond
      J3G_CUDA(c, cudaMemsetAsync(gk + ngrid, 0, sizeof(double) * c->bg.size(), c->stream));
    if (nbg > 0)
      J3G_LAUNCH(c, launch_background_grad(c->kind, off[k + 1] - off[k], nbg,
                                           ptr<double>(c->wraw) + (size_t)off[k] * raw,
                                           ptr<double>(c->bgsens) + (size_t)off[k] * raw * nbg,
                                           gk + ngrid, c->stream));
  }
  return J3G_OK;
}

bool valid_kind(int k) { return k >= J3G_SCALAR && k <= J3G_MAGNETIZATION; }

// ---------------------------------------------------------------------------
// Device-resident sensitivity (the GPU side of FullSensitivityGravMagCalculator)

void free_buf(DevBuf &b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
}

void drop_stored(j3g_context *c) {
  if (!c || c->storage == 0) return;
  cudaStreamSynchronize(c->stream);
  free_buf(c->J32);
  free_buf(c->Jhi);
  free_buf(c->Jlo);
  free_buf(c->JThi);
  free_buf(c->JTlo);
  free_buf(c->rowscale);
  free_buf(c->Jrowsum);
  c->storage = 0;
}

long long round64(long long v) { return (v + 63) / 64 * 64; }
int nstored(const j3g_context *c) { return stored_rows_per_station(c->kind); }

int build_stored(j3g_context *c, int storage) {
  J3G_TRY(check_ready(c));
  if (storage != J3G_STORE_FP32 && storage != J3G_STORE_F16X2)
    return fail(c, J3G_ERR_ARG, "unknown storage");
  if (!c->node_exact)
    return fail(c, J3G_ERR_UNSUPPORTED,
                "device sensitivity needs corner coordinates that are running sums of the sizes");
  if (c->ngrid() == 0 || c->nmeas == 0) return fail(c, J3G_ERR_ARG, "empty mesh or survey");
  drop_stored(c);
  J3G_TRY(ensure_background(c));
  const long long K = c->ngrid_cols(), ldK = round64(K);
  const int NS = nstored(c);
  const long long R = (long long)c->nmeas * NS, ldR = round64(R);
  const size_t need = storage == J3G_STORE_FP32
                          ? (size_t)R * ldK * 4
                          : (size_t)(tiled_rows(R) * ldK + tiled_rows(K) * ldR) * 4;
  size_t fr = 0, tot = 0;
  J3G_CUDA(c, cudaMemGetInfo(&fr, &tot));
  if (need + (size_t)(1ull << 31) > fr)
    return fail(c, J3G_ERR_NOMEM, "sensitivity of " + std::to_string(need) + " bytes does not fit");
  c->st_rows = R;
  c->st_ld = ldK;
  c->st_ldT = ldR;
  // station chunks bounded by ~1 GiB of FP64 rows + node scratch
  const long long per = (long long)NS * K * 8 + (long long)kind_ncomp(c->kind) * c->nnodes() * 8;
  int chunk = (int)std::max(1LL, std::min<long long>(c->nmeas, (1LL << 30) / per));
  chunk = std::min(chunk, 65535);
  J3G_TRY(ensure(c, c->F, sizeof(double) * (size_t)chunk * kind_ncomp(c->kind) * c->nnodes()));
  MeshView m = mesh_view(c);
  StationView s = station_view(c);
  const MagField mf = mag_field(c);
  if (storage == J3G_STORE_FP32) {
    J3G_TRY(ensure(c, c->J32, sizeof(float) * (size_t)R * ldK));
    J3G_CUDA(c, cudaMemsetAsync(c->J32.p, 0, sizeof(float) * (size_t)R * ldK, c->stream));
    for (int s0 = 0; s0 < c->nmeas; s0 += chunk) {
      const int ns = std::min(chunk, c->nmeas - s0);
      J3G_LAUNCH(c, launch_stored_rows(c->kind, m, s, s0, ns, mf, ptr<double>(c->F), nullptr,
                                       ptr<float>(c->J32) + (size_t)s0 * NS * ldK, ldK,
                                       c->stream));
      ++c->launches;
    }
  } else {
    // tiled layout; the padding rows of the last row block stay zero
    const size_t bj = 2 * (size_t)tiled_rows(R) * ldK, bjt = 2 * (size_t)tiled_rows(K) * ldR;
    J3G_TRY(ensure(c, c->Jhi, bj));
    J3G_TRY(ensure(c, c->Jlo, bj));
    J3G_TRY(ensure(c, c->JThi, bjt));
    J3G_TRY(ensure(c, c->JTlo, bjt));
    J3G_CUDA(c, cudaMemsetAsync(c->Jhi.p, 0, bj, c->stream));
    J3G_CUDA(c, cudaMemsetAsync(c->Jlo.p, 0, bj, c->stream));
    J3G_CUDA(c, cudaMemsetAsync(c->JThi.p, 0, bjt, c->stream));
    J3G_CUDA(c, cudaMemsetAsync(c->JTlo.p, 0, bjt, c->stream));
    J3G_TRY(ensure(c, c->rowscale, sizeof(float) * (size_t)R));
    J3G_TRY(ensure(c, c->Jrowsum, sizeof(double) * (size_t)R));
    J3G_TRY(ensure(c, c->rows, sizeof(double) * (size_t)chunk * NS * K));
    J3G_TRY(ensure(c, c->gerr, sizeof(int)));
    J3G_CUDA(c, cudaMemsetAsync(c->gerr.p, 0, sizeof(int), c->stream));
    for (int s0 = 0; s0 < c->nmeas; s0 += chunk) {
      const int ns = std::min(chunk, c->nmeas - s0);
      J3G_LAUNCH(c, launch_stored_rows(c->kind, m, s, s0, ns, mf, ptr<double>(c->F),
                                       ptr<double>(c->rows), nullptr, K, c->stream));
      ++c->launches;
      J3G_LAUNCH(c, launch_split_rows(ptr<double>(c->rows), K, K, ns * NS, c->Jhi.p, c->Jlo.p,
                                      ldK, ptr<float>(c->rowscale), ptr<double>(c->Jrowsum),
                                      (long long)s0 * NS, c->stream));
    }
    J3G_LAUNCH(c, launch_transpose16(c->Jhi.p, ldK, R, K, c->JThi.p, ldR, c->stream));
    J3G_LAUNCH(c, launch_transpose16(c->Jlo.p, ldK, R, K, c->JTlo.p, ldR, c->stream));
  }
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  c->storage = storage;
  return J3G_OK;
}

int check_stored(j3g_context *c) {
  J3G_TRY(check_ready(c));
  if (c->storage == 0) return fail(c, J3G_ERR_STATE, "no device sensitivity: call j3g_build_sensitivity");
  return J3G_OK;
}

int batched_forward_impl(j3g_context *c, int nmod, const double *d_models, double *d_data,
                         double *raw_out);

// d = J m through the FP32 streaming product (one model), then background + transform.
int stored_forward_f32(j3g_context *c, const double *d_model, double *d_data, double *raw_out) {
  const long long K = c->ngrid_cols(), ldK = c->st_ld, R = c->st_rows;
  double tbx, tby, tbz;
  tfa_dir(c, tbx, tby, tbz);
  J3G_TRY(ensure(c, c->x32, sizeof(float) * (size_t)ldK));
  J3G_TRY(ensure(c, c->sums, sizeof(double) * (size_t)R));
  J3G_LAUNCH(c, launch_to_f32(d_model, K, ldK, ptr<float>(c->x32), c->stream));
  {
    TimedScope ts(c, J3G_TIMER_STREAM_FORWARD);
    J3G_LAUNCH(c, launch_gemv_f32(ptr<float>(c->J32), ldK, (int)R, ptr<float>(c->x32),
                                  ptr<double>(c->sums), c->stream));
  }
  const int nbg = c->nbg_active();
  J3G_LAUNCH(c, launch_stored_assemble(c->kind, c->transform, tbx, tby, tbz, c->nmeas, 1,
                                       ptr<double>(c->sums), R, nbg ? ptr<double>(c->bgsens) : nullptr,
                                       nbg, d_model, c->nparm(), K, mag_field(c), raw_out, d_data,
                                       (long long)c->nmeas * c->dpm(), c->stream));
  return J3G_OK;
}

// Gradient entries of background parameters without a response (vertical
// gradient): zero, for nmod gradients [nmod][nparm].
int zero_inert_background(j3g_context *c, int nmod, double *d_grads) {
  const int ninert = c->nbg_params() - c->nbg_active();
  if (ninert <= 0 || nmod == 0) return J3G_OK;
  const size_t np = c->nparm();
  J3G_CUDA(c, cudaMemset2DAsync(d_grads + (np - ninert), np * sizeof(double), 0,
                                ninert * sizeof(double), nmod, c->stream));
  return J3G_OK;
}

int stored_adjoint_f32(j3g_context *c, const double *d_model, const double *d_misfit,
                       double *d_grad) {
  const long long K = c->ngrid_cols(), ldK = c->st_ld, R = c->st_rows;
  const int raw = c->raw(), nbg = c->nbg_active();
  double tbx, tby, tbz;
  tfa_dir(c, tbx, tby, tbz);
  const double *rawd = nullptr;
  if (c->transform == J3G_T_FTG_INVARIANT || c->transform == J3G_T_TOTAL_FIELD) {
    J3G_TRY(ensure(c, c->rawb, sizeof(double) * (size_t)c->nmeas * raw));
    J3G_TRY(ensure(c, c->data, sizeof(double) * (size_t)c->nmeas * c->dpm()));
    J3G_TRY(stored_forward_f32(c, d_model, ptr<double>(c->data), ptr<double>(c->rawb)));
    rawd = ptr<double>(c->rawb);
  }
  J3G_TRY(ensure(c, c->wrawb, sizeof(double) * (size_t)c->nmeas * raw));
  J3G_TRY(ensure(c, c->wst, sizeof(double) * (size_t)R));
  J3G_TRY(ensure(c, c->part, sizeof(double) * (size_t)gemv_t_chunks((int)R) * ldK));
  J3G_LAUNCH(c, launch_stored_weights(c->kind, c->transform, tbx, tby, tbz, c->nmeas, 1, d_misfit,
                                      (long long)c->nmeas * c->dpm(), rawd, mag_field(c),
                                      ptr<double>(c->wrawb), ptr<double>(c->wst), R, c->stream));
  {
    TimedScope ts(c, J3G_TIMER_STREAM_ADJOINT);
    J3G_LAUNCH(c, launch_gemv_t_f32(ptr<float>(c->J32), ldK, (int)R, ptr<double>(c->wst),
                                    ptr<double>(c->part), K, 2.0, d_grad, c->stream));
  }
  ++c->launches;  // column-block sums + chunk reduction
  if (nbg)
    J3G_LAUNCH(c, launch_bg_grad_batched(raw, c->nmeas, nbg, 1, ptr<double>(c->wrawb),
                                         ptr<double>(c->bgsens), d_grad, c->nparm(), K, c->stream));
  return zero_inert_background(c, 1, d_grad);
}

// K-splits of a tensor-core product: at most kMaxKbPerSplit k-blocks per
// split keep the kernel's FP32 register sums short (the splits are added as
// FP32 two-sum pairs), and at least about six waves of CTAs over the 152 SMs.
// 128 k-blocks (8192 products, 256 drained sums per register) keep every
// output group of the config-4 products within 3e-7 of FP64 and the FTG
// invariant's within 4e-7 (bound 1e-6); 64 gave 1e-7 / 3e-7 with twice the
// partial sums to add.
constexpr long long kMaxKbPerSplit = 128;
int choose_splits(long long m, int ntiles, long long ld) {
  const long long mt = (m + 127) / 128, kb = ld / 64;
  const long long s = std::max<long long>((kb + kMaxKbPerSplit - 1) / kMaxKbPerSplit,
                                          (6 * 152 + mt * ntiles - 1) / (mt * ntiles));
  return (int)std::max<long long>(1, std::min(s, kb));
}

// The split-sum kernel's arguments for one product (launch_splitk_reduce).
struct SplitSums {
  double *out = nullptr;
  long long ld_out = 0;
  const float *rowscale = nullptr, *modscale = nullptr;
  const int *sexp = nullptr;  // per-split model scales (forward), [models][splits]
  const double *modmean = nullptr, *rowsum = nullptr;
  double factor = 1.0;
};

// One tensor-core product and its split sums, timed as the direction's
// product and the split sums.
cudaError_t product_launches(j3g_context *c, int dir, const GemmOperands &g, int nsplit, int tile,
                             long long ldp, long long slice, const SplitSums &ss) {
  cudaError_t e;
  {
    TimedScope ts(c, dir ? J3G_TIMER_GEMM_ADJOINT : J3G_TIMER_GEMM_FORWARD);
    e = launch_gemm_x3(g, nsplit, ptr<float>(c->P), ldp, slice, ptr<int>(c->gerr), c->stream,
                       tile);
  }
  if (e != cudaSuccess) return e;
  ++c->launches;
  TimedScope ts(c, J3G_TIMER_REDUCE);
  e = launch_splitk_reduce(ptr<float>(c->P), gemm_splits_used(g.ld, nsplit), slice, (int)g.n,
                           (int)g.m, ldp, ss.rowscale, ss.modscale, ss.sexp, ss.modmean,
                           ss.rowsum, ss.factor, ss.out, ss.ld_out, c->stream);
  if (e == cudaSuccess) ++c->launches;
  return e;
}

// Plan of one tensor-core product (K splits and N tile), with the partial-sum
// buffer c->P sized for it.  Without autotuning, the fixed rule: choose_splits
// and gemm_n_tile.  With autotuning, the first product of a shape times each
// candidate -- the fixed plan, split counts that fill the last wave of CTAs on
// the SMs, and one-SM 128-wide tiles where the pair kernel would run -- once
// after an untimed run (CUDA events on the context's stream), keeps the
// fastest for the context's lifetime and reuses it.  A candidate is timed
// as `run` queues it (operands, nsplit, tile): the product with its split
// sums, and for the forward the models' split, which follows the product's K
// splits.
// Every candidate keeps at most kMaxKbPerSplit k-blocks per split, the bound
// that holds the FP32 register sums to their accuracy.
int gemm_plan(j3g_context *c, int dir, const GemmOperands &g, long long slice,
              const std::function<cudaError_t(const GemmOperands &, int, int)> &run,
              j3g_context::GemmPlan &plan) {
  const int tile0 = gemm_n_tile((int)g.n);
  plan.tile = tile0;
  plan.nsplit = choose_splits(g.m, (int)(g.n_pad / tile0), g.ld);
  plan.ms = 0.0f;
  if (c->pinned[dir]) {
    const auto &pp = c->pinned_plan[dir];
    if (pp.tile == 0 || g.n_pad % pp.tile == 0) {  // a tile that fits the batch
      plan.nsplit = pp.nsplit;
      if (pp.tile) plan.tile = pp.tile;
      return ensure(c, c->P,
                    sizeof(float) * (size_t)gemm_splits_used(g.ld, plan.nsplit) * slice);
    }
  }
  const std::array<long long, 4> key{dir, g.m, g.n_pad, g.ld};
  auto it = c->autotune ? c->plans.find(key) : c->plans.end();
  if (!c->autotune || it != c->plans.end()) {
    if (it != c->plans.end()) plan = it->second;
    return ensure(c, c->P, sizeof(float) * (size_t)gemm_splits_used(g.ld, plan.nsplit) * slice);
  }
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  const long long kb = g.ld / 64, smin = (kb + kMaxKbPerSplit - 1) / kMaxKbPerSplit;
  std::vector<std::pair<int, int>> cand;  // (tile, nsplit)
  for (int tile : {tile0, tile0 == 256 ? 128 : 0}) {
    if (!tile || g.n_pad % tile) continue;
    const int base = choose_splits(g.m, (int)(g.n_pad / tile), g.ld);
    const long long smax = std::min<long long>(kb, 4LL * base);
    cand.push_back({tile, base});
    // CTAs per split: 128-row tiles (a pair counts two) x N tiles; one CTA per SM
    const long long per = (tile == 256 ? 2 * ((g.m + 255) / 256) : (g.m + 127) / 128) *
                          (g.n_pad / tile);
    int added = 0;
    for (long long w = 1; w <= 256 && added < 3; ++w) {
      const long long s = w * sms / per;
      if (s < std::max<long long>(smin, base) || s > smax) continue;
      const int used = gemm_splits_used(g.ld, (int)s);
      const long long rem = (long long)used * per % sms;
      if (rem > sms / 10 && rem < sms * 9 / 10) continue;  // much of the last wave idle
      bool seen = false;
      for (auto &p : cand) seen |= (p.first == tile && gemm_splits_used(g.ld, p.second) == used);
      if (!seen) {
        cand.push_back({tile, (int)s});
        ++added;
      }
    }
  }
  int nsp_max = 1;
  for (auto &p : cand) nsp_max = std::max(nsp_max, gemm_splits_used(g.ld, p.second));

  J3G_TRY(ensure(c, c->P, sizeof(float) * (size_t)nsp_max * slice));
  GemmOperands gt = g;
  gt.fault = 0;  // candidates are timed on the normal path
  cudaEvent_t a, b;
  J3G_CUDA(c, cudaEventCreate(&a));
  J3G_CUDA(c, cudaEventCreate(&b));
  const bool timing = c->timing;
  c->timing = false;  // the candidates stay out of the phase timers
  float best = 0.0f;
  for (auto &p : cand) {
    float ms = 0.0f;
    cudaError_t e = run(gt, p.second, p.first);
    if (e == cudaSuccess) e = cudaEventRecord(a, c->stream);
    if (e == cudaSuccess) e = run(gt, p.second, p.first);
    if (e == cudaSuccess) e = cudaEventRecord(b, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (e != cudaSuccess) {
      c->timing = timing;
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      return cuda_fail(c, e, "gemm autotune");
    }
    if (best == 0.0f || ms < best) {
      best = ms;
      plan.tile = p.first;
      plan.nsplit = p.second;
      plan.ms = ms;
    }
  }
  c->timing = timing;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  c->plans[key] = plan;
  ++c->prod_gen;
  return J3G_OK;
}

// Models per pass of the batched products: the model index of the split,
// reduction and epilogue kernels runs over grid y (at most 65535 blocks) and
// the product pads the batch to a multiple of 256.
constexpr int kMaxBatch = 32768;

int batched_forward_pass(j3g_context *c, int nmod, const double *d_models, double *d_data,
                         double *raw_out) {
  const long long K = c->ngrid_cols(), ldK = c->st_ld, R = c->st_rows, np = c->nparm();
  double tbx, tby, tbz;
  tfa_dir(c, tbx, tby, tbz);
  const int nbg = c->nbg_active();
  J3G_TRY(ensure(c, c->sums, sizeof(double) * (size_t)nmod * R));
  if (c->storage == J3G_STORE_FP32) {
    for (int n = 0; n < nmod; ++n) {
      J3G_TRY(ensure(c, c->x32, sizeof(float) * (size_t)ldK));
      J3G_LAUNCH(c, launch_to_f32(d_models + (size_t)n * np, K, ldK, ptr<float>(c->x32), c->stream));
      J3G_LAUNCH(c, launch_gemv_f32(ptr<float>(c->J32), ldK, (int)R, ptr<float>(c->x32),
                                    ptr<double>(c->sums) + (size_t)n * R, c->stream));
    }
  } else {
    const int tile = gemm_n_tile(nmod);
    const long long npad = (nmod + tile - 1) / tile * tile;
    J3G_TRY(ensure(c, c->Bhi, 2 * (size_t)npad * ldK));
    J3G_TRY(ensure(c, c->Blo, 2 * (size_t)npad * ldK));
    J3G_TRY(ensure(c, c->mmean, sizeof(double) * (size_t)npad));
    // split exponents [npad][splits] and the sampled row exponents after them
    J3G_TRY(ensure(c, c->sexp, sizeof(int) * (size_t)npad * (ldK / 64 + 1)));
    const long long slice = (long long)nmod * R;
    GemmOperands g{c->Jhi.p, c->Jlo.p, R, c->Bhi.p, c->Blo.p, nmod, npad, ldK, true};
    g.fault = c->test_fault;
    J3G_TRY(ensure(c, c->gerr, sizeof(int)));
    // sums = rowscale * (split sums, each split at its models' scale)
    //        + centre * (J 1)
    SplitSums ss;
    ss.out = ptr<double>(c->sums);
    ss.ld_out = R;
    ss.rowscale = ptr<float>(c->rowscale);
    ss.sexp = ptr<int>(c->sexp);
    ss.modmean = ptr<double>(c->mmean);
    ss.rowsum = ptr<double>(c->Jrowsum);
    // models are centred (m - an estimate of their mean over cells; centre *
    // (J 1) is added back in FP64 after the product, so a large uniform part
    // of a model -- whose tensor response is nearly zero -- does not eat into
    // the FP32 accuracy) and split with one scale per K split of the product
    auto run = [&](const GemmOperands &go, int nsplit, int tile) -> cudaError_t {
      const int nsp = gemm_splits_used(ldK, nsplit);
      cudaError_t e;
      {
        TimedScope ts(c, J3G_TIMER_SPLIT);
        e = launch_split_models(d_models, np, nmod, K, c->Bhi.p, c->Blo.p, ldK, (int)npad,
                                64LL * gemm_kb_per_split(ldK, nsplit), nsp,
                                ptr<double>(c->mmean), ptr<int>(c->sexp), c->stream);
      }
      if (e != cudaSuccess) return e;
      c->launches += 2;
      return product_launches(c, 0, go, nsplit, tile, R, slice, ss);
    };
    j3g_context::GemmPlan plan;
    J3G_TRY(gemm_plan(c, 0, g, slice, run, plan));
    c->last_plan[0] = plan;
    const cudaError_t e = run(g, plan.nsplit, plan.tile);
    if (e != cudaSuccess) return cuda_fail(c, e, "forward product");
  }
  TimedScope ts(c, J3G_TIMER_EPILOGUE);
  J3G_LAUNCH(c, launch_stored_assemble(c->kind, c->transform, tbx, tby, tbz, c->nmeas, nmod,
                                       ptr<double>(c->sums), R, nbg ? ptr<double>(c->bgsens) : nullptr,
                                       nbg, d_models, np, K, mag_field(c), raw_out, d_data,
                                       (long long)c->nmeas * c->dpm(), c->stream));
  return J3G_OK;
}

// Batches of more than kMaxBatch models run as consecutive passes.
int batched_forward_impl(j3g_context *c, int nmod, const double *d_models, double *d_data,
                         double *raw_out) {
  const size_t np = c->nparm(), nd = (size_t)c->nmeas * c->dpm(), nr = (size_t)c->nmeas * c->raw();
  for (int n0 = 0; n0 < nmod; n0 += kMaxBatch)
    J3G_TRY(batched_forward_pass(c, std::min(kMaxBatch, nmod - n0), d_models + n0 * np,
                                 d_data + n0 * nd, raw_out ? raw_out + n0 * nr : nullptr));
  return J3G_OK;
}

int batched_adjoint_pass(j3g_context *c, int nmod, const double *d_models,
                         const double *d_misfits, double *d_grads) {
  const long long K = c->ngrid_cols(), ldK = c->st_ld, R = c->st_rows, ldR = c->st_ldT,
                  np = c->nparm();
  const int raw = c->raw(), nbg = c->nbg_active();
  double tbx, tby, tbz;
  tfa_dir(c, tbx, tby, tbz);
  const double *rawd = nullptr;
  if (c->transform == J3G_T_FTG_INVARIANT || c->transform == J3G_T_TOTAL_FIELD) {
    J3G_TRY(ensure(c, c->rawb, sizeof(double) * (size_t)nmod * c->nmeas * raw));
    J3G_TRY(ensure(c, c->data, sizeof(double) * (size_t)nmod * c->nmeas * c->dpm()));
    J3G_TRY(batched_forward_pass(c, nmod, d_models, ptr<double>(c->data), ptr<double>(c->rawb)));
    rawd = ptr<double>(c->rawb);
  }
  J3G_TRY(ensure(c, c->wrawb, sizeof(double) * (size_t)nmod * c->nmeas * raw));
  const int tile = gemm_n_tile(nmod);
  const long long npad = (nmod + tile - 1) / tile * tile;
  // fp16 products on a survey that fits one cluster per model: the weights and
  // their split in one launch (the same values as the two launches below)
  const bool fused = c->storage != J3G_STORE_FP32 && weights_split_fits(c->nmeas, ldR, (int)npad);
  if (!fused) {
    J3G_TRY(ensure(c, c->wst, sizeof(double) * (size_t)nmod * R));
    TimedScope ts(c, J3G_TIMER_EPILOGUE);
    J3G_LAUNCH(c, launch_stored_weights(c->kind, c->transform, tbx, tby, tbz, c->nmeas, nmod,
                                        d_misfits, (long long)c->nmeas * c->dpm(), rawd,
                                        mag_field(c), ptr<double>(c->wrawb), ptr<double>(c->wst),
                                        R, c->stream));
  }
  if (c->storage == J3G_STORE_FP32) {
    J3G_TRY(ensure(c, c->part, sizeof(double) * (size_t)gemv_t_chunks((int)R) * ldK));
    for (int n = 0; n < nmod; ++n) {
      J3G_LAUNCH(c, launch_gemv_t_f32(ptr<float>(c->J32), ldK, (int)R,
                                      ptr<double>(c->wst) + (size_t)n * R, ptr<double>(c->part), K,
                                      2.0, d_grads + (size_t)n * np, c->stream));
      ++c->launches;
    }
  } else {
    J3G_TRY(ensure(c, c->Bhi, 2 * (size_t)npad * std::max(ldR, ldK)));
    J3G_TRY(ensure(c, c->Blo, 2 * (size_t)npad * std::max(ldR, ldK)));
    J3G_TRY(ensure(c, c->mscale, sizeof(float) * (size_t)npad));
    // residual weights carry the row scale of J: J = s_r (hi + lo)
    if (fused) {
      TimedScope ts(c, J3G_TIMER_SPLIT);
      J3G_LAUNCH(c, launch_weights_split(c->kind, c->transform, tbx, tby, tbz, c->nmeas, nmod,
                                         (int)npad, d_misfits, (long long)c->nmeas * c->dpm(),
                                         rawd, mag_field(c), ptr<double>(c->wrawb),
                                         ptr<float>(c->rowscale), ptr<float>(c->mscale),
                                         c->Bhi.p, c->Blo.p, ldR, c->stream));
    } else {
      J3G_TRY(ensure(c, c->swork, sizeof(double) * (size_t)split_matrix_work((int)npad, ldR)));
      TimedScope ts(c, J3G_TIMER_SPLIT);
      J3G_LAUNCH(c, launch_split_matrix(ptr<double>(c->wst), R, nmod, R, ptr<float>(c->rowscale),
                                        c->Bhi.p, c->Blo.p, ldR, (int)npad, ptr<float>(c->mscale),
                                        ptr<double>(c->swork), c->stream));
      c->launches += split_matrix_launches(ldR) - 1;
    }
    const long long slice = (long long)nmod * K;
    GemmOperands g{c->JThi.p, c->JTlo.p, K, c->Bhi.p, c->Blo.p, nmod, npad, ldR, true};
    g.fault = c->test_fault;
    J3G_TRY(ensure(c, c->gerr, sizeof(int)));
    SplitSums ss;  // gradients = 2 * modscale * (split sums)
    ss.out = d_grads;
    ss.ld_out = np;
    ss.modscale = ptr<float>(c->mscale);
    ss.factor = 2.0;
    auto run = [&](const GemmOperands &go, int nsplit, int tile) {
      return product_launches(c, 1, go, nsplit, tile, K, slice, ss);
    };
    j3g_context::GemmPlan plan;
    J3G_TRY(gemm_plan(c, 1, g, slice, run, plan));
    c->last_plan[1] = plan;
    const cudaError_t e = product_launches(c, 1, g, plan.nsplit, plan.tile, K, slice, ss);
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint product");
  }
  if (nbg) {
    TimedScope ts(c, J3G_TIMER_EPILOGUE);
    J3G_LAUNCH(c, launch_bg_grad_batched(raw, c->nmeas, nbg, nmod, ptr<double>(c->wrawb),
                                         ptr<double>(c->bgsens), d_grads, np, K, c->stream));
  }
  return zero_inert_background(c, nmod, d_grads);
}

int batched_adjoint_impl(j3g_context *c, int nmod, const double *d_models,
                         const double *d_misfits, double *d_grads) {
  const size_t np = c->nparm(), nd = (size_t)c->nmeas * c->dpm();
  for (int n0 = 0; n0 < nmod; n0 += kMaxBatch)
    J3G_TRY(batched_adjoint_pass(c, std::min(kMaxBatch, nmod - n0),
                                 d_models ? d_models + n0 * np : nullptr, d_misfits + n0 * nd,
                                 d_grads + n0 * np));
  return J3G_OK;
}

// Error flag of the tensor-core pipeline (bounded waits that expired).
int check_gemm_flag(j3g_context *c) {
  if (!c->gerr.p) return J3G_OK;
  int v = 0;
  J3G_CUDA(c, cudaMemcpyAsync(&v, c->gerr.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  if (v != 0) {
    cudaMemsetAsync(c->gerr.p, 0, sizeof(int), c->stream);
    return fail(c, J3G_ERR_CUDA, "tensor-core pipeline wait expired (code " + std::to_string(v) + ")");
  }
  return J3G_OK;
}

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
                    &c->G, &c->F, &c->rows, &c->rowsum, &c->probe, &c->J32, &c->Jhi,
                    &c->Jlo, &c->JThi, &c->JTlo, &c->rowscale, &c->x32, &c->sums, &c->part,
                    &c->Bhi, &c->Blo, &c->P, &c->wst, &c->wrawb, &c->rawb, &c->gerr,
                    &c->mscale, &c->Jrowsum, &c->mmean, &c->swork, &c->sexp, &c->chunks, &c->rmaps,
                    &c->rcoarse, &c->rfine};
  for (DevBuf *b : bufs)
    if (b->p) cudaFree(b->p);
  for (auto &sl : c->slots) {
    if (sl.ticket >= 0 && sl.d2h) cudaEventSynchronize(sl.d2h);
    for (DevBuf *b : {&sl.in, &sl.in2, &sl.out})
      if (b->p) cudaFree(b->p);
    for (cudaEvent_t e : {sl.h2d, sl.done, sl.d2h})
      if (e) cudaEventDestroy(e);
    for (cudaGraphExec_t g : sl.exec)
      if (g) cudaGraphExecDestroy(g);
    if (sl.flag) cudaFreeHost(sl.flag);
  }
  for (int d = 0; d < 2; ++d) {
    if (c->h2d_stream[d]) cudaStreamDestroy(c->h2d_stream[d]);
    if (c->d2h_stream[d]) cudaStreamDestroy(c->d2h_stream[d]);
  }
  for (auto &t : c->timed) {
    cudaEventDestroy(t.second.first);
    cudaEventDestroy(t.second.second);
  }
  if (c->child) j3g_destroy(c->child);
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
  c->refine_set = false;  // the walks belong to the old mesh
  c->bg_dirty = true;
  drop_stored(c);  // the stored sensitivity belongs to the old geometry
  ++c->gen;
  ++c->prod_gen;
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
  drop_stored(c);  // the stored sensitivity belongs to the old geometry
  ++c->gen;
  ++c->prod_gen;
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
  c->hsx.swap(vx);
  c->hsy.swap(vy);
  c->hsz.swap(vz);
  c->stations_set = true;
  c->bg_dirty = true;
  drop_stored(c);  // the stored sensitivity belongs to the old geometry
  ++c->gen;
  ++c->prod_gen;
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
  drop_stored(c);  // the stored sensitivity belongs to the old geometry
  if (c->transform != J3G_T_NONE) {
    const bool ok = (c->transform == J3G_T_FTG_INVARIANT && kind == J3G_TENSOR) ||
                    ((c->transform == J3G_T_TOTAL_FIELD || c->transform == J3G_T_TFA) &&
                     (kind == J3G_MAGNETIC || kind == J3G_MAGNETIZATION));
    if (!ok) c->transform = J3G_T_NONE;
  }
  ++c->gen;
  ++c->prod_gen;
  return J3G_OK;
}

int j3g_set_transform(j3g_context *c, int transform, double inc, double dec) {
  if (!c) return J3G_ERR_ARG;
  if (transform < J3G_T_NONE || transform > J3G_T_TFA)
    return fail(c, J3G_ERR_ARG, "unknown transform");
  if (transform == J3G_T_FTG_INVARIANT && c->kind != J3G_TENSOR)
    return fail(c, J3G_ERR_UNSUPPORTED, "the FTG invariant needs tensor data");
  if ((transform == J3G_T_TOTAL_FIELD || transform == J3G_T_TFA) && c->kind != J3G_MAGNETIC &&
      c->kind != J3G_MAGNETIZATION)
    return fail(c, J3G_ERR_UNSUPPORTED, "total-field transforms need three-component magnetic data");
  c->transform = transform;
  c->tinc = inc;
  c->tdec = dec;
  ++c->gen;
  ++c->prod_gen;
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

// The context over the concatenated stations of a batch of station subsets
// (same mesh, background, kind and transform as c, work on c's stream).
static int subset_child(j3g_context *c, int nsub, const int *off, const int *idx,
                        j3g_context **out) {
  J3G_TRY(check_ready(c));
  if (nsub < 1 || !off || off[0] != 0) return fail(c, J3G_ERR_ARG, "bad subset offsets");
  for (int k = 0; k < nsub; ++k)
    if (off[k + 1] < off[k]) return fail(c, J3G_ERR_ARG, "subset offsets must not decrease");
  const int total = off[nsub];
  if (total > 0 && !idx) return fail(c, J3G_ERR_ARG, "null subset station index");
  for (int i = 0; i < total; ++i)
    if (idx[i] < 0 || idx[i] >= c->nmeas)
      return fail(c, J3G_ERR_ARG, "subset station index outside the survey");
  std::vector<int> voff(off, off + nsub + 1), vidx(idx, idx + total);
  if (!c->child) {
    int rc = j3g_create(&c->child, c->device);
    if (rc != J3G_OK) return fail(c, rc, "cannot create the subset context");
  }
  j3g_context *ch = c->child;
  j3g_set_stream(ch, c->stream);
  if (c->child_gen != c->gen || voff != c->child_off || vidx != c->child_idx) {
    int rc = j3g_set_mesh(ch, c->nx, c->ny, c->nz, c->X.data(), c->Y.data(), c->Z.data(),
                          c->xs.data(), c->ys.data(), c->zs.data());
    if (rc == J3G_OK) rc = j3g_set_background(ch, (int)c->bg.size(), c->bg.data());
    if (rc == J3G_OK) rc = j3g_set_kind(ch, c->kind, c->inc, c->dec, c->fs);
    if (rc == J3G_OK) rc = j3g_set_transform(ch, c->transform, c->tinc, c->tdec);
    std::vector<double> x(total), y(total), z(total);
    for (int i = 0; i < total; ++i) {
      x[i] = c->hsx[idx[i]];
      y[i] = c->hsy[idx[i]];
      z[i] = c->hsz[idx[i]];
    }
    if (rc == J3G_OK) rc = j3g_set_stations(ch, total, x.data(), y.data(), z.data());
    if (rc != J3G_OK) return fail(c, rc, ch->err);
    c->child_off.swap(voff);
    c->child_idx.swap(vidx);
    c->child_gen = c->gen;
  }
  *out = ch;
  return J3G_OK;
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

int j3g_build_sensitivity(j3g_context *c, int storage) {
  if (!c) return J3G_ERR_ARG;
  cudaSetDevice(c->device);
  return build_stored(c, storage);
}

int j3g_drop_sensitivity(j3g_context *c) {
  if (!c) return J3G_ERR_ARG;
  cudaSetDevice(c->device);
  drop_stored(c);
  return J3G_OK;
}

int j3g_sensitivity_info(const j3g_context *c, int *storage, long long *rows, long long *cols,
                         long long *bytes) {
  if (!c) return J3G_ERR_ARG;
  if (storage) *storage = c->storage;
  if (rows) *rows = c->storage ? c->st_rows : 0;
  if (cols) *cols = c->storage ? c->ngrid_cols() : 0;
  if (bytes)
    *bytes = c->storage == J3G_STORE_FP32     ? c->st_rows * c->st_ld * 4
             : c->storage == J3G_STORE_F16X2 ? 2 * (tiled_rows(c->st_rows) * c->st_ld * 2) +
                                                   2 * (tiled_rows(c->ngrid_cols()) * c->st_ldT * 2)
                                              : 0;
  return J3G_OK;
}

int j3g_stored_forward_device(j3g_context *c, const double *d_model, double *d_data) {
  if (!c || !d_model || !d_data) return fail(c, J3G_ERR_ARG, "null pointer");
  cudaSetDevice(c->device);
  J3G_TRY(check_stored(c));
  if (c->storage == J3G_STORE_FP32) return stored_forward_f32(c, d_model, d_data, nullptr);
  return batched_forward_impl(c, 1, d_model, d_data, nullptr);
}

int j3g_stored_lqderivative_device(j3g_context *c, const double *d_model, const double *d_misfit,
                                   double *d_grad) {
  if (!c || !d_model || !d_misfit || !d_grad) return fail(c, J3G_ERR_ARG, "null pointer");
  cudaSetDevice(c->device);
  J3G_TRY(check_stored(c));
  if (c->storage == J3G_STORE_FP32) return stored_adjoint_f32(c, d_model, d_misfit, d_grad);
  return batched_adjoint_impl(c, 1, d_model, d_misfit, d_grad);
}

int j3g_batched_forward_device(j3g_context *c, int nmodels, const double *d_models,
                               double *d_data) {
  if (!c || nmodels < 0 || (nmodels > 0 && (!d_models || !d_data)))
    return fail(c, J3G_ERR_ARG, "bad batched arguments");
  cudaSetDevice(c->device);
  J3G_TRY(check_stored(c));
  if (nmodels == 0) return J3G_OK;
  return batched_forward_impl(c, nmodels, d_models, d_data, nullptr);
}

int j3g_batched_lqderivative_device(j3g_context *c, int nmodels, const double *d_models,
                                    const double *d_misfits, double *d_grads) {
  if (!c || nmodels < 0 || (nmodels > 0 && (!d_models || !d_misfits || !d_grads)))
    return fail(c, J3G_ERR_ARG, "bad batched arguments");
  cudaSetDevice(c->device);
  J3G_TRY(check_stored(c));
  if (nmodels == 0) return J3G_OK;
  return batched_adjoint_impl(c, nmodels, d_models, d_misfits, d_grads);
}

int j3g_batched_forward(j3g_context *c, int nmodels, const double *h_models, double *h_data) {
  if (!c || nmodels < 0 || (nmodels > 0 && (!h_models || !h_data)))
    return fail(c, J3G_ERR_ARG, "bad batched arguments");
  cudaSetDevice(c->device);
  J3G_TRY(check_stored(c));
  if (nmodels == 0) return J3G_OK;
  const size_t nm = (size_t)nmodels * c->nparm(), nd = (size_t)nmodels * c->nmeas * c->dpm();
  J3G_TRY(ensure(c, c->model, sizeof(double) * nm));
  J3G_TRY(ensure(c, c->data, sizeof(double) * nd));
  J3G_CUDA(c, cudaMemcpyAsync(c->model.p, h_models, sizeof(double) * nm, cudaMemcpyHostToDevice,
                              c->stream));
  J3G_TRY(batched_forward_impl(c, nmodels, ptr<double>(c->model), ptr<double>(c->data), nullptr));
  J3G_CUDA(c, cudaMemcpyAsync(h_data, c->data.p, sizeof(double) * nd, cudaMemcpyDeviceToHost,
                              c->stream));
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  return check_gemm_flag(c);
}

int j3g_batched_lqderivative(j3g_context *c, int nmodels, const double *h_models,
                             const double *h_misfits, double *h_grads) {
  if (!c || nmodels < 0 || (nmodels > 0 && (!h_misfits || !h_grads)))
    return fail(c, J3G_ERR_ARG, "bad batched arguments");
  cudaSetDevice(c->device);
  J3G_TRY(check_stored(c));
  if (nmodels == 0) return J3G_OK;
  // only the data-dependent transforms read the models (their forward data)
  const bool needs_models =
      c->transform == J3G_T_FTG_INVARIANT || c->transform == J3G_T_TOTAL_FIELD;
  if (needs_models && !h_models) return fail(c, J3G_ERR_ARG, "this transform needs the models");
  const size_t nm = (size_t)nmodels * c->nparm(), nd = (size_t)nmodels * c->nmeas * c->dpm();
  J3G_TRY(ensure(c, c->model, sizeof(double) * nm));
  J3G_TRY(ensure(c, c->misfit, sizeof(double) * nd));
  J3G_TRY(ensure(c, c->grad, sizeof(double) * nm));
  if (needs_models)
    J3G_CUDA(c, cudaMemcpyAsync(c->model.p, h_models, sizeof(double) * nm,
                                cudaMemcpyHostToDevice, c->stream));
  J3G_CUDA(c, cudaMemcpyAsync(c->misfit.p, h_misfits, sizeof(double) * nd,
                              cudaMemcpyHostToDevice, c->stream));
  J3G_TRY(batched_adjoint_impl(c, nmodels, ptr<double>(c->model), ptr<double>(c->misfit),
                               ptr<double>(c->grad)));
  J3G_CUDA(c, cudaMemcpyAsync(h_grads, c->grad.p, sizeof(double) * nm, cudaMemcpyDeviceToHost,
                              c->stream));
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  return check_gemm_flag(c);
}

namespace {
// The next slot of the pipeline ring, its previous call complete; the copy
// streams and events are made on first use.
int pipeline_slot(j3g_context *c, j3g_context::Slot *&slot) {
  for (int d = 0; d < 2; ++d)
    if (!c->h2d_stream[d]) {
      J3G_CUDA(c, cudaStreamCreateWithFlags(&c->h2d_stream[d], cudaStreamNonBlocking));
      J3G_CUDA(c, cudaStreamCreateWithFlags(&c->d2h_stream[d], cudaStreamNonBlocking));
    }
  slot = &c->slots[c->next_ticket % j3g_context::kSlots];
  if (!slot->h2d) {
    J3G_CUDA(c, cudaEventCreateWithFlags(&slot->h2d, cudaEventDisableTiming));
    J3G_CUDA(c, cudaEventCreateWithFlags(&slot->done, cudaEventDisableTiming));
    J3G_CUDA(c, cudaEventCreateWithFlags(&slot->d2h, cudaEventDisableTiming));
    J3G_CUDA(c, cudaMallocHost(&slot->flag, sizeof(int)));
  }
  if (slot->ticket >= 0) {  // the call before in this slot must have finished
    J3G_CUDA(c, cudaEventSynchronize(slot->d2h));
    // that call was never waited for: keep its failure for j3g_batched_wait
    if (*slot->flag != 0) {
      c->failed_tickets[slot->ticket] = *slot->flag;
      *slot->flag = 0;
      cudaMemsetAsync(c->gerr.p, 0, sizeof(int), c->stream);
    }
    slot->ticket = -1;
  }
  return J3G_OK;
}

// Queue the copies around a product: inputs (host -> slot buffers) on the
// direction's H2D stream, the product on the context's stream once they are
// in, the output back on the direction's D2H stream once the product is done.
struct PipeCopy {
  const double *host;
  DevBuf *dev;
  size_t n;
};
// The product of a pipelined call on the context's stream: replayed from the
// slot's CUDA graph when one was captured under the current state, captured
// when the previous eager product of this shape left the state unchanged (no
// buffer grew, no plan was tuned), else run eagerly.  With timing on, eager.
int pipeline_product(j3g_context *c, j3g_context::Slot *slot, int dir, int nmod,
                     const std::function<int(void)> &product) {
  if (!c->timing && slot->exec[dir] && slot->exec_gen[dir] == c->prod_gen &&
      slot->exec_nmod[dir] == nmod) {
    J3G_CUDA(c, cudaGraphLaunch(slot->exec[dir], c->stream));
    c->launches += slot->exec_launches[dir];
    return J3G_OK;
  }
  if (!c->timing && slot->warm_gen[dir] == c->prod_gen && slot->warm_nmod[dir] == nmod) {
    if (slot->exec[dir]) {
      cudaGraphExecDestroy(slot->exec[dir]);
      slot->exec[dir] = nullptr;
    }
    const long long gen0 = c->prod_gen, l0 = c->launches;
    J3G_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = product();
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(c->stream, &graph);
    cudaGraphExec_t exec = nullptr;
    if (rc == J3G_OK && ec == cudaSuccess && graph && c->prod_gen == gen0 &&
        cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
      cudaGraphDestroy(graph);
      slot->exec[dir] = exec;
      slot->exec_gen[dir] = gen0;
      slot->exec_nmod[dir] = nmod;
      slot->exec_launches[dir] = c->launches - l0;
      J3G_CUDA(c, cudaGraphLaunch(exec, c->stream));
      return J3G_OK;
    }
    // not capturable under this state: nothing ran, run it eagerly
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    c->launches = l0;
    slot->warm_gen[dir] = -1;
  }
  const long long gen0 = c->prod_gen;
  J3G_TRY(product());
  if (c->prod_gen == gen0) {
    slot->warm_gen[dir] = gen0;
    slot->warm_nmod[dir] = nmod;
  }
  return J3G_OK;
}

int pipeline_run(j3g_context *c, j3g_context::Slot *slot, int dir, int nmod,
                 std::initializer_list<PipeCopy> ins, double *h_out, size_t n_out,
                 long long *ticket, const std::function<int(void)> &product) {
  cudaStream_t h2d = c->h2d_stream[dir], d2h = c->d2h_stream[dir];
  for (const PipeCopy &in : ins) {
    if (!in.host) continue;
    J3G_TRY(ensure(c, *in.dev, sizeof(double) * in.n));
    J3G_CUDA(c, cudaMemcpyAsync(in.dev->p, in.host, sizeof(double) * in.n,
                                cudaMemcpyHostToDevice, h2d));
  }
  J3G_TRY(ensure(c, slot->out, sizeof(double) * n_out));
  J3G_CUDA(c, cudaEventRecord(slot->h2d, h2d));
  J3G_CUDA(c, cudaStreamWaitEvent(c->stream, slot->h2d, 0));
  J3G_TRY(pipeline_product(c, slot, dir, nmod, product));
  J3G_CUDA(c, cudaEventRecord(slot->done, c->stream));
  J3G_CUDA(c, cudaStreamWaitEvent(d2h, slot->done, 0));
  J3G_CUDA(c, cudaMemcpyAsync(h_out, slot->out.p, sizeof(double) * n_out, cudaMemcpyDeviceToHost,
                              d2h));
  // the error flag of the bounded waits, as it stands after this product
  *slot->flag = 0;
  if (c->gerr.p)
    J3G_CUDA(c, cudaMemcpyAsync(slot->flag, c->gerr.p, sizeof(int), cudaMemcpyDeviceToHost, d2h));
  J3G_CUDA(c, cudaEventRecord(slot->d2h, d2h));
  slot->ticket = c->next_ticket++;
  if (ticket) *ticket = slot->ticket;
  return J3G_OK;
}
}  // namespace

int j3g_batched_forward_async(j3g_context *c, int nmodels, const double *h_models,
                              double *h_data, long long *ticket) {
  if (!c || nmodels < 1 || !h_models || !h_data)
    return fail(c, J3G_ERR_ARG, "bad batched arguments");
  cudaSetDevice(c->device);
  J3G_TRY(check_stored(c));
  j3g_context::Slot *slot;
  J3G_TRY(pipeline_slot(c, slot));
  const size_t nm = (size_t)nmodels * c->nparm(), nd = (size_t)nmodels * c->nmeas * c->dpm();
  return pipeline_run(c, slot, 0, nmodels, {{h_models, &slot->in, nm}}, h_data, nd, ticket,
                      [&]() {
    return batched_forward_impl(c, nmodels, ptr<double>(slot->in), ptr<double>(slot->out),
                                nullptr);
  });
}

int j3g_batched_lqderivative_async(j3g_context *c, int nmodels, const double *h_models,
                                   const double *h_misfits, double *h_grads, long long *ticket) {
  if (!c || nmodels < 1 || !h_misfits || !h_grads)
    return fail(c, J3G_ERR_ARG, "bad batched arguments");
  cudaSetDevice(c->device);
  J3G_TRY(check_stored(c));
  const bool needs_models =
      c->transform == J3G_T_FTG_INVARIANT || c->transform == J3G_T_TOTAL_FIELD;
  if (needs_models && !h_models) return fail(c, J3G_ERR_ARG, "this transform needs the models");
  j3g_context::Slot *slot;
  J3G_TRY(pipeline_slot(c, slot));
  const size_t nm = (size_t)nmodels * c->nparm(), nd = (size_t)nmodels * c->nmeas * c->dpm();
  return pipeline_run(c, slot, 1, nmodels,
                      {{needs_models ? h_models : nullptr, &slot->in, nm},
                       {h_misfits, &slot->in2, nd}},
                      h_grads, nm, ticket, [&]() {
                        return batched_adjoint_impl(
                            c, nmodels, needs_models ? ptr<double>(slot->in) : nullptr,
                            ptr<double>(slot->in2), ptr<double>(slot->out));
                      });
}

int j3g_batched_wait(j3g_context *c, long long ticket) {
  if (!c || ticket < 0 || ticket >= c->next_ticket)
    return fail(c, J3G_ERR_ARG, "no such pipelined call");
  cudaSetDevice(c->device);
  // a call that is no longer in its slot has completed (its slot was reused);
  // a failure seen when its slot was reused is reported now
  auto f = c->failed_tickets.find(ticket);
  if (f != c->failed_tickets.end()) {
    const int code = f->second;
    c->failed_tickets.erase(f);
    return fail(c, J3G_ERR_CUDA,
                "tensor-core pipeline wait expired (code " + std::to_string(code) + ")");
  }
  for (auto &sl : c->slots)
    if (sl.ticket == ticket) {
      J3G_CUDA(c, cudaEventSynchronize(sl.d2h));
      sl.ticket = -1;
      if (*sl.flag != 0) {
        const int code = *sl.flag;
        *sl.flag = 0;
        cudaMemsetAsync(c->gerr.p, 0, sizeof(int), c->stream);
        return fail(c, J3G_ERR_CUDA,
                    "tensor-core pipeline wait expired (code " + std::to_string(code) + ")");
      }
    }
  return J3G_OK;
}

static void clear_timing(j3g_context *c) {
  for (auto &t : c->timed) {
    cudaEventDestroy(t.second.first);
    cudaEventDestroy(t.second.second);
  }
  c->timed.clear();
}

int j3g_set_timing(j3g_context *c, int enable) {
  if (!c) return J3G_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  clear_timing(c);
  c->timing = enable != 0;
  ++c->prod_gen;
  return J3G_OK;
}

int j3g_get_timing(j3g_context *c, int category, double *total_ms, long long *launches) {
  if (!c || !total_ms || !launches) return J3G_ERR_ARG;
  cudaSetDevice(c->device);
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  double ms = 0.0;
  long long n = 0;
  for (auto &t : c->timed) {
    if (t.first != category) continue;
    float v = 0.0f;
    J3G_CUDA(c, cudaEventElapsedTime(&v, t.second.first, t.second.second));
    ms += v;
    ++n;
  }
  *total_ms = ms;
  *launches = n;
  return J3G_OK;
}

int j3g_subsets_forward_device(j3g_context *c, int nsub, const int *h_offsets,
                               const int *h_index, const double *d_model, double *d_data) {
  if (!c || !d_model || !d_data) return fail(c, J3G_ERR_ARG, "null pointer");
  cudaSetDevice(c->device);
  j3g_context *ch = nullptr;
  J3G_TRY(subset_child(c, nsub, h_offsets, h_index, &ch));
  const long long l0 = ch->launches;
  const int rc = forward_device(ch, d_model, d_data, nullptr, nullptr);
  c->launches += ch->launches - l0;
  return rc == J3G_OK ? J3G_OK : fail(c, rc, ch->err);
}

int j3g_subsets_lqderivative_device(j3g_context *c, int nsub, const int *h_offsets,
                                    const int *h_index, const double *d_model,
                                    const double *d_misfit, double *d_grads) {
  if (!c || !d_model || !d_misfit || !d_grads) return fail(c, J3G_ERR_ARG, "null pointer");
  cudaSetDevice(c->device);
  j3g_context *ch = nullptr;
  J3G_TRY(subset_child(c, nsub, h_offsets, h_index, &ch));
  const std::vector<int> off(h_offsets, h_offsets + nsub + 1);
  const long long l0 = ch->launches;
  const int rc = adjoint_device(ch, d_model, d_misfit, d_grads, &off);
  c->launches += ch->launches - l0;
  return rc == J3G_OK ? J3G_OK : fail(c, rc, ch->err);
}

int j3g_set_autotune(j3g_context *c, int enable) {
  if (!c) return J3G_ERR_ARG;
  c->autotune = enable != 0;
  ++c->prod_gen;
  return J3G_OK;
}

int j3g_set_test_fault(j3g_context *c, int fault) {
  if (!c || fault < 0 || fault > 1) return J3G_ERR_ARG;
  c->test_fault = fault;
  ++c->prod_gen;  // captured products hold the old kernel arguments
  return J3G_OK;
}

int j3g_set_gemm_plan(j3g_context *c, int direction, int nsplit, int tile) {
  if (!c || direction < 0 || direction > 1) return J3G_ERR_ARG;
  ++c->prod_gen;
  if (nsplit <= 0) {  // back to the fixed rule / the autotuner
    c->pinned[direction] = false;
    return J3G_OK;
  }
  if (tile != 0 && tile != 64 && tile != 128 && tile != 256)
    return fail(c, J3G_ERR_ARG, "tile must be 0, 64, 128 or 256");
  c->pinned[direction] = true;
  c->pinned_plan[direction].nsplit = nsplit;
  c->pinned_plan[direction].tile = tile;
  c->pinned_plan[direction].ms = 0.0f;
  return J3G_OK;
}

int j3g_get_gemm_plan(const j3g_context *c, int direction, int *nsplit, int *tile,
                      double *tuned_ms) {
  if (!c || direction < 0 || direction > 1) return J3G_ERR_ARG;
  const auto &p = c->last_plan[direction];
  if (nsplit) *nsplit = p.nsplit;
  if (tile) *tile = p.tile;
  if (tuned_ms) *tuned_ms = p.ms;
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
  return check_gemm_flag(c);
}

int j3g_refine_axis(int ncoarse, const double *coarse_coords, const double *coarse_sizes,
                    int nref, const double *ref_coords, int capacity, double *fine_sizes,
                    int *nfine) {
  if (ncoarse < 1 || !coarse_coords || !coarse_sizes || nref < 1 || !ref_coords || !nfine ||
      capacity < 0 || (capacity > 0 && !fine_sizes))
    return J3G_ERR_ARG;
  std::vector<double> f;
  if (refine_axis(ncoarse, coarse_coords, coarse_sizes, nref, ref_coords, f) != 0) {
    *nfine = -1;  // non-positive last cell: the reference throws
    return J3G_ERR_ARG;
  }
  *nfine = (int)f.size();
  if ((int)f.size() > capacity) return J3G_ERR_ARG;
  std::copy(f.begin(), f.end(), fine_sizes);
  return J3G_OK;
}

int j3g_set_refinement(j3g_context *c, int cnx, int cny, int cnz, const double *cxs,
                       const double *cys, const double *czs) {
  if (!c) return J3G_ERR_ARG;
  if (!c->mesh_set || c->ngrid() == 0) return fail(c, J3G_ERR_STATE, "set the forward mesh first");
  if (cnx < 1 || cny < 1 || cnz < 1 || !cxs || !cys || !czs)
    return fail(c, J3G_ERR_ARG, "bad coarse grid");
  if ((long long)cnx * cny * cnz >= (1LL << 30) || c->ngrid() >= (1LL << 30))
    return fail(c, J3G_ERR_ARG, "grids of 2^30 cells or more are not supported");
  cudaSetDevice(c->device);
  const int fn[3] = {c->nx, c->ny, c->nz}, cn[3] = {cnx, cny, cnz};
  const double *cs[3] = {cxs, cys, czs};
  const std::vector<double> *fs[3] = {&c->xs, &c->ys, &c->zs};
  // int layout: owners (fn per axis), begins (cn per axis), ends (cn per axis)
  std::vector<int> h((size_t)fn[0] + fn[1] + fn[2] + 2 * ((size_t)cnx + cny + cnz));
  size_t off[3][3], o = 0;
  for (int a = 0; a < 3; ++a) off[a][0] = o, o += fn[a];
  for (int a = 0; a < 3; ++a) off[a][1] = o, o += cn[a];
  for (int a = 0; a < 3; ++a) off[a][2] = o, o += cn[a];
  bool all = true;
  for (int a = 0; a < 3; ++a) {
    int *owner = h.data() + off[a][0];
    refine_ranges(cn[a], cs[a], fn[a], fs[a]->data(), h.data() + off[a][1], h.data() + off[a][2],
                  owner);
    for (int f = 0; f < fn[a]; ++f) all &= owner[f] >= 0;
  }
  J3G_TRY(ensure(c, c->rmaps, h.size() * sizeof(int)));
  J3G_CUDA(c, cudaMemcpyAsync(c->rmaps.p, h.data(), h.size() * sizeof(int),
                              cudaMemcpyHostToDevice, c->stream));
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  const int *d = ptr<int>(c->rmaps);
  for (int a = 0; a < 3; ++a) {
    c->rm.owner[a] = d + off[a][0];
    c->rm.begin[a] = d + off[a][1];
    c->rm.end[a] = d + off[a][2];
    c->rm.cn[a] = cn[a];
    c->rm.fn[a] = fn[a];
    c->cn[a] = cn[a];
  }
  c->rm.zrun_max = 0;
  for (int k = 0; k < cnz; ++k)
    c->rm.zrun_max = std::max(c->rm.zrun_max, h[off[2][2] + k] - h[off[2][1] + k]);
  c->refine_covers_all = all;
  c->refine_set = true;
  return J3G_OK;
}

namespace {
// cell blocks and extra parameters of a model vector of this context's kind
void refine_layout(const j3g_context *c, int &nblock, int &nextra) {
  nblock = c->kind == J3G_MAGNETIZATION ? 3 : 1;
  nextra = c->kind == J3G_MAGNETIZATION ? 0 : (int)c->bg.size();
}
long long coarse_nparm(const j3g_context *c) {
  int nblock, nextra;
  refine_layout(c, nblock, nextra);
  return (long long)nblock * c->cn[0] * c->cn[1] * c->cn[2] + nextra;
}
}  // namespace

int j3g_refinement_info(const j3g_context *c, long long *coarse_cells, long long *coarse_nparm_out,
                        int *covers_all) {
  if (!c) return J3G_ERR_ARG;
  if (!c->refine_set) return J3G_ERR_STATE;
  if (coarse_cells) *coarse_cells = (long long)c->cn[0] * c->cn[1] * c->cn[2];
  if (coarse_nparm_out) *coarse_nparm_out = coarse_nparm(c);
  if (covers_all) *covers_all = c->refine_covers_all ? 1 : 0;
  return J3G_OK;
}

int j3g_refine_project_device(j3g_context *c, int nmodels, const double *d_coarse,
                              double *d_fine) {
  if (!c || nmodels < 0 || (nmodels > 0 && (!d_coarse || !d_fine)))
    return fail(c, J3G_ERR_ARG, "bad refinement arguments");
  if (!c->refine_set) return fail(c, J3G_ERR_STATE, "no refinement set for this mesh");
  cudaSetDevice(c->device);
  int nblock, nextra;
  refine_layout(c, nblock, nextra);
  J3G_LAUNCH(c, launch_refine_project(c->rm, nmodels, nblock, nextra, d_coarse, d_fine,
                                      c->stream));
  return J3G_OK;
}

int j3g_refine_combine_device(j3g_context *c, int nmodels, const double *d_fine,
                              double *d_coarse) {
  if (!c || nmodels < 0 || (nmodels > 0 && (!d_coarse || !d_fine)))
    return fail(c, J3G_ERR_ARG, "bad refinement arguments");
  if (!c->refine_set) return fail(c, J3G_ERR_STATE, "no refinement set for this mesh");
  cudaSetDevice(c->device);
  int nblock, nextra;
  refine_layout(c, nblock, nextra);
  J3G_LAUNCH(c, launch_refine_combine(c->rm, nmodels, nblock, nextra, d_fine, d_coarse,
                                      c->stream));
  return J3G_OK;
}

int j3g_refine_project(j3g_context *c, int nmodels, const double *h_coarse, double *h_fine) {
  if (!c || nmodels < 0 || (nmodels > 0 && (!h_coarse || !h_fine)))
    return fail(c, J3G_ERR_ARG, "bad refinement arguments");
  if (!c->refine_set) return fail(c, J3G_ERR_STATE, "no refinement set for this mesh");
  if (nmodels == 0) return J3G_OK;
  cudaSetDevice(c->device);
  const size_t nc = (size_t)nmodels * coarse_nparm(c), nf = (size_t)nmodels * c->nparm();
  J3G_TRY(ensure(c, c->rcoarse, nc * sizeof(double)));
  J3G_TRY(ensure(c, c->rfine, nf * sizeof(double)));
  J3G_CUDA(c, cudaMemcpyAsync(c->rcoarse.p, h_coarse, nc * sizeof(double),
                              cudaMemcpyHostToDevice, c->stream));
  if (!c->refine_covers_all)  // uncovered cells keep the caller's values
    J3G_CUDA(c, cudaMemcpyAsync(c->rfine.p, h_fine, nf * sizeof(double), cudaMemcpyHostToDevice,
                                c->stream));
  J3G_TRY(j3g_refine_project_device(c, nmodels, ptr<double>(c->rcoarse), ptr<double>(c->rfine)));
  J3G_CUDA(c, cudaMemcpyAsync(h_fine, c->rfine.p, nf * sizeof(double), cudaMemcpyDeviceToHost,
                              c->stream));
  J3G_CUDA(c, cudaStreamSynchronize(c->stream));
  return J3G_OK;
}

int j3g_refine_combine(j3g_context *c, int nmodels, const double *h_fine, double *h_coarse) {
  if (!c || nmodels < 0 || (nmodels > 0 && (!h_coarse || !h_fine)))
    return fail(c, J3G_ERR_ARG, "bad refinement arguments");
  if (!c->refine_set) return fail(c, J3G_ERR_STATE, "no refinement set for this mesh");
  if (nmodels == 0) return J3G_OK;
  cudaSetDevice(c->device);
  const size_t nc = (size_t)nmodels * coarse_nparm(c), nf = (size_t)nmodels * c->nparm();
  J3G_TRY(ensure(c, c->rcoarse, nc * sizeof(double)));
  J3G_TRY(ensure(c, c->rfine, nf * sizeof(double)));
  J3G_CUDA(c, cudaMemcpyAsync(c->rfine.p, h_fine, nf * sizeof(double), cudaMemcpyHostToDevice,
                              c->stream));
  J3G_TRY(j3g_refine_combine_device(c, nmodels, ptr<double>(c->rfine), ptr<double>(c->rcoarse)));
  J3G_CUDA(c, cudaMemcpyAsync(h_coarse, c->rcoarse.p, nc * sizeof(double),
                              cudaMemcpyDeviceToHost, c->stream));
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
