// prism_kernels.h -- launchers of the FP64 prism kernels (internal interface
// between the C-ABI layer and the kernels; no CUDA types leak past capi.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include "kinds.h"

namespace j3g {

// Device view of the mesh.  Node coordinates X[0..nx], Y[0..ny], Z[0..nz];
// cell i spans [X[i], X[i] + xs[i]].  When node_exact is true every
// X[i] + xs[i] equals X[i+1] bit for bit, so a corner term is a node term.
struct MeshView {
  int nx, ny, nz;
  const double *X, *Y, *Z;     // nodes (n + 1 each)
  const double *xs, *ys, *zs;  // cell sizes (n each)
  __host__ __device__ long long ngrid() const { return (long long)nx * ny * nz; }
  __host__ __device__ long long nnodes() const {
    return (long long)(nx + 1) * (ny + 1) * (nz + 1);
  }
};

struct StationView {
  int n;
  const double *x, *y, *z;
};

// Forward, node formulation:  per station and component
//   U_c(s) = scale_c * sum_nodes F_c(s, node) * rho~(node)
// rho~ = third mixed backward difference of the zero-padded model (one model
// block; magnetisation runs it once per block into rho_t + block * nnodes).
cudaError_t launch_rho_tilde(const MeshView &m, const double *rho, double *rho_t,
                             cudaStream_t st);
// partial: [nblk][nmeas][ncomp] virtual-component sums; rho_t holds one
// nnodes block per model block of the kind.
cudaError_t launch_node_forward(int kind, const MeshView &m, const StationView &s,
                                const double *rho_t, double *partial, int nblk,
                                int nodes_per_block, int stations_per_block, cudaStream_t st);
// comps: [nmeas][NC_COUNT] node-component sums (scaled), unused comps zero;
// for the vertical gradient and magnetisation the raw rows [nmeas][raw].
cudaError_t launch_forward_reduce(int kind, int nmeas, int nblk, const double *partial,
                                  const MagField &mf, double *comps, cudaStream_t st);

// Background: bgsens[s][raw][j] for each layer j (GravityBackground.cpp:24-137,
// OMPMagneticSusceptibilityImp.cpp:31-101).
cudaError_t launch_background(int kind, const MeshView &m, const StationView &s, int nbg,
                              const double *bg_thick, double xorig, double yorig, double zorig,
                              double xw, double yw, double zw, const MagField &mf,
                              double *bgsens, cudaStream_t st);

// Per station: raw = raw_from_comps(comps) (+ sum_j bgsens * bgval) and the
// optional transform.  raw_out [nmeas][raw] (may be null), data_out [nmeas][dpm].
cudaError_t launch_assemble(int kind, int transform, double t_bx, double t_by, double t_bz,
                            int nmeas, const double *comps, int comps_ld, const double *bgsens,
                            int nbg, const double *bgval, const MagField &mf, double *raw_out,
                            double *data_out, cudaStream_t st);

// Adjoint.  w_raw [nmeas][raw] are the raw-row weights (misfit already
// back-projected through the transform).  W [nmeas][NC_COUNT] receives the
// node-component weights with the component scale folded in ([nmeas][ncomp]
// virtual-component weights for the vertical gradient and magnetisation).
cudaError_t launch_backproject(int kind, int transform, double t_bx, double t_by, double t_bz,
                               int nmeas, const double *misfit, const double *raw,
                               double *w_raw, cudaStream_t st);
cudaError_t launch_comp_weights(int kind, int nmeas, const double *w_raw, const MagField &mf,
                                double *W, cudaStream_t st);
// Gpart [nchunk][nblock][nnodes] = sum over the chunk's stations of
// sum_q W_q * F_q, per model block.
// chunk_start (device, nchunk + 1 values, may be null): explicit station
// ranges of the chunks instead of stations_per_chunk apiece.
cudaError_t launch_node_adjoint(int kind, const MeshView &m, const StationView &s,
                                const double *W, int stations_per_chunk, int nchunk,
                                const int *chunk_start, double *Gpart, cudaStream_t st);
// grad[b * ngrid + cell] = 2 * sum_corners (-1)^shifts * sum_chunks
// Gpart[chunk][b][node] for each model block b; G: nblock * nnodes scratch.
cudaError_t launch_adjoint_combine(const MeshView &m, int nchunk, int nblock, const double *Gpart,
                                   double *G, double *grad, cudaStream_t st);
// grad[ngrid + j] = 2 * sum_s sum_r w_raw[s][r] * bgsens[s][r][j]
cudaError_t launch_background_grad(int kind, int nmeas, int nbg, const double *w_raw,
                                   const double *bgsens, double *grad_bg, cudaStream_t st);

// Sensitivity rows (reference per-cell order).  rows[(sl*raw + r) * ld + cell]
// for stations s0 .. s0+ns-1 (sl = s - s0); magnetisation rows carry the three
// blocks at columns b * ngrid + cell.  node_exact selects the node-term
// path (F scratch of ns * ncomp * nnodes doubles), otherwise eight corner
// evaluations per cell.
cudaError_t launch_sens_rows(int kind, bool node_exact, const MeshView &m,
                             const StationView &s, int s0, int ns, const MagField &mf,
                             double *F, double *rows, long long ld, cudaStream_t st);
// Rows of the device-resident sensitivity for stations s0..s0+ns-1: per
// station the kind's node components (scalar 1, tensor 6 = xx yy zz xy xz yz,
// joint 7 = gz + tensor) or, for magnetics, the 3 raw rows Bx By Bz.  Written
// as double (rows64) or float (rows32), row (sl*nstored + q) at stride ld.
int stored_rows_per_station(int kind);
cudaError_t launch_stored_rows(int kind, const MeshView &m, const StationView &s, int s0, int ns,
                               const MagField &mf, double *F, double *rows64, float *rows32,
                               long long ld, cudaStream_t st);

// d[(s0+sl)*raw + r] = sum_cell rows[(sl*raw + r)*ld + cell] * rho[cell]
cudaError_t launch_rows_dot(int raw, int ns, long long ngrid, const double *rows, long long ld,
                            const double *rho, double *out, cudaStream_t st);

// grad[cell] += sum_r w[r] * rows[r*ld + cell] over nrow rows.
cudaError_t launch_rows_tdot(int nrow, long long ngrid, const double *rows, long long ld,
                             const double *w, double *grad, cudaStream_t st);
cudaError_t launch_scale(long long n, double f, double *v, cudaStream_t st);

// FP64 peak probe: n_iter dependent-chain FMAs per thread (measurement only).
cudaError_t launch_fp64_probe(double *out, int blocks, int threads, int n_iter,
                              cudaStream_t st);

}  // namespace j3g
