// noalloc.cu -- the allocation-free gridded forward (j3g_forward_noalloc).
//
// Some hosts cannot let this library call cudaMalloc: an application that
// reserves all device memory for its own pool allocator at start-up (a
// cudaMalloc from here would fail or fragment that pool), or a solver loop
// that must not take the device-wide synchronisation that cudaMalloc/cudaFree
// imply.  For them this file offers one entry point whose only scratch
// memory is the fixed file-scope device array below; inputs and outputs are
// caller-owned device buffers and nothing is allocated or freed.
//
// The array is part of the library image: every GPU that loads the library
// holds its 16 MiB until the process exits.  All calls share it, so calls
// that overlap on the GPU (different streams, or several host threads) race
// on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "../../include/jif3d_gb300.h"
#include "prism_kernels.h"

using namespace j3g;

namespace {

constexpr long long kScratchDoubles = 2LL << 20;  // 2 Mi doubles = 16 MiB
constexpr long long kAlign = 32;                   // regions start on 256-byte boundaries
constexpr int kMaxDevices = 64;

// Shared scratch of every j3g_forward_noalloc call on this device.  In host
// code this name is only a stand-in for the symbol, not a device address;
// kernels receive the address obtained from cudaGetSymbolAddress.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

std::mutex g_setup_mutex;
double *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device`, with that device current.
// Outside stream capture the address is looked up on every call: a device
// reset (cudaDeviceReset) or a new primary context loads the library's module
// again, possibly at another address, so a remembered address could be stale.
// While `stream` is being captured, the address remembered from the last call
// outside capture is used (looking a symbol up may load the module, which a
// capturing stream must not see); a first call inside capture is refused.
int scratch_for(int device, cudaStream_t stream, double **out) {
  if (device < 0 || device >= kMaxDevices) return J3G_ERR_ARG;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) {
    cudaGetLastError();
    return J3G_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (cap == cudaStreamCaptureStatusNone) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return J3G_ERR_CUDA;
    }
    g_scratch_ptr[device] = static_cast<double *>(p);
  } else if (!g_scratch_ptr[device]) {
    return J3G_ERR_STATE;
  }
  *out = g_scratch_ptr[device];
  return J3G_OK;
}

long long round_up(long long v) { return (v + kAlign - 1) / kAlign * kAlign; }

}  // namespace

extern "C" int j3g_forward_noalloc(int kind, int nx, int ny, int nz, const double *d_xnode,
                                   const double *d_ynode, const double *d_znode, int nmeas,
                                   const double *d_sx, const double *d_sy, const double *d_sz,
                                   double inclination, double declination,
                                   double field_strength, const double *d_model, double *d_data,
                                   void *stream) {
  if (kind < KIND_SCALAR || kind > KIND_JOINT) return J3G_ERR_ARG;
  if (nx <= 0 || ny <= 0 || nz <= 0 || nmeas < 0) return J3G_ERR_ARG;
  if (!d_xnode || !d_ynode || !d_znode || !d_model || !d_data) return J3G_ERR_ARG;
  if (nmeas > 0 && (!d_sx || !d_sy || !d_sz)) return J3G_ERR_ARG;
  if (nmeas == 0) return J3G_OK;

  // scratch plan: rho~ (one value per node), per-station component sums,
  // and the per-block partial sums of the node reduction
  const long long nn = (long long)(nx + 1) * (ny + 1) * (nz + 1);
  const int ncomp = kind_ncomp(kind);
  const long long rho_len = round_up(nn);
  const long long comps_len = round_up((long long)nmeas * NC_COUNT);
  const long long left = kScratchDoubles - rho_len - comps_len;
  const long long per_block = (long long)nmeas * ncomp;
  if (left < per_block) return J3G_ERR_SCRATCH_LIMIT;
  const long long max_blocks = left / per_block;
  int npb = 2048;
  while ((nn + npb - 1) / npb > max_blocks) {
    if (npb > (1 << 26)) return J3G_ERR_SCRATCH_LIMIT;
    npb <<= 1;
  }
  int spb = 4;
  auto blocks = [&](int a, int b) {
    return ((nn + a - 1) / a) * (long long)((nmeas + b - 1) / b);
  };
  // smaller node blocks for parallelism, as long as their partials still fit
  while (npb > 256 && blocks(npb, spb) < 152 * 8 &&
         (nn + (npb >> 1) - 1) / (npb >> 1) <= max_blocks)
    npb >>= 1;
  while (spb > 1 && blocks(npb, spb) < 152 * 8) spb >>= 1;
  // station blocks run over grid y: at most 65535 of them
  spb = std::max(spb, (nmeas + 65534) / 65535);
  const int nblk = (int)((nn + npb - 1) / npb);

  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return J3G_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double *scratch = nullptr;
  int rc = scratch_for(device, st, &scratch);
  if (rc != J3G_OK) return rc;
  double *rho_t = scratch;
  double *comps = scratch + rho_len;
  double *partial = comps + comps_len;

  MeshView m;
  m.nx = nx;
  m.ny = ny;
  m.nz = nz;
  m.X = d_xnode;
  m.Y = d_ynode;
  m.Z = d_znode;
  m.xs = m.ys = m.zs = nullptr;  // not used by the node-term forward
  StationView s;
  s.n = nmeas;
  s.x = d_sx;
  s.y = d_sy;
  s.z = d_sz;
  MagField mf;
  mf.bx = std::cos(inclination) * std::cos(declination);
  mf.by = std::cos(inclination) * std::sin(declination);
  mf.bz = std::sin(inclination);
  mf.fs = field_strength;
  mf.factor = 1.0 / (4 * 3.141592653589793238462643383279502884 * kGravConst);

  // every scratch value read below is written first in the same call, so no
  // clearing is needed: rho~ covers all nodes, the partials all (block,
  // station, component) triples and the sums all (station, component) pairs
  if (launch_rho_tilde(m, d_model, rho_t, st) != cudaSuccess) return J3G_ERR_CUDA;
  if (launch_node_forward(kind, m, s, rho_t, partial, nblk, npb, spb, st) != cudaSuccess)
    return J3G_ERR_CUDA;
  if (launch_forward_reduce(kind, nmeas, nblk, partial, mf, comps, st) != cudaSuccess)
    return J3G_ERR_CUDA;
  if (launch_assemble(kind, TR_NONE, 0.0, 0.0, 0.0, nmeas, comps, NC_COUNT, nullptr, 0, nullptr,
                      mf, nullptr, d_data, st) != cudaSuccess)
    return J3G_ERR_CUDA;
  return J3G_OK;
}
