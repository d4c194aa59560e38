// stored.h -- device-resident sensitivity storage and its products (internal).
#pragma once
#include <cuda_runtime.h>

#include "kinds.h"

namespace j3g {

// Tiled layout of the stored fp16 sensitivity (the A operand of the
// tensor-core products): tiles of 128 rows x 64 columns, each 16 KB
// contiguous and row-major inside, ordered by column block within a row
// block.  A matrix with rows padded to ld columns (a multiple of 64) and to a
// multiple of 128 rows (tiled_rows) keeps element (r, c) at tiled_index.  One
// TMA box of the products is one tile: a single contiguous 16 KB read,
// where the row-major layout needed 128 separate 128-byte pieces.
__host__ __device__ inline long long tiled_index(long long r, long long c, long long ld) {
  return ((r >> 7) * (ld >> 6) + (c >> 6)) * 8192 + (r & 127) * 64 + (c & 63);
}
inline long long tiled_rows(long long rows) { return (rows + 127) / 128 * 128; }

// fp16 hi / lo split of FP64 rows with a power-of-two row scale
// (scale[row0 + r]): row = scale * (hi + lo), max|hi| in (2^13, 2^14];
// hi / lo in the tiled layout with ld_out columns (padding columns zero).
// rowsum (optional) receives the FP64 row sums J 1.
cudaError_t launch_split_rows(const double *rows, long long ld_in, long long ncol, int nrows,
                              void *hi, void *lo, long long ld_out, float *scale, double *rowsum,
                              long long row0, cudaStream_t st);
// out(c, r) = in(r, c) for r < rows (zero for rows <= r < ld_out), c < cols;
// 16-bit elements, both matrices in the tiled layout (in: ld_in columns,
// out: ld_out columns).
cudaError_t launch_transpose16(const void *in, long long ld_in, long long rows, long long cols,
                               void *out, long long ld_out, cudaStream_t st);
// FP64 [nrow][ld_src] (column c times colscale[c] when given) -> fp16 hi / lo
// [nrow_pad][ld_dst] with a power-of-two scale per row into rowscale[r]; rows
// beyond nrow and columns beyond ncol are zero.  work:
// split_matrix_work(nrow_pad, ld_dst) doubles.
long long split_matrix_work(int nrow_pad, long long ld_dst);
// Kernel launches of one launch_split_matrix call (1 for short rows, else 3).
int split_matrix_launches(long long ld_dst);
cudaError_t launch_split_matrix(const double *src, long long ld_src, int nrow, long long ncol,
                                const float *colscale, void *hi, void *lo, long long ld_dst,
                                int nrow_pad, float *rowscale, double *work, cudaStream_t st);
cudaError_t launch_to_f32(const double *src, long long n, long long npad, float *dst,
                          cudaStream_t st);
// d[r] = sum_c J[r][c] x[c] (FP32 J, FP32 x, FP64 result), ld multiple of 4.
cudaError_t launch_gemv_f32(const float *J, long long ld, int nrows, const float *x, double *out,
                            cudaStream_t st);
// out[c] = factor * sum_r J[r][c] w[r]; part needs gemv_t_chunks(nrows) * ld doubles.
int gemv_t_chunks(int nrows);
cudaError_t launch_gemv_t_f32(const float *J, long long ld, int nrows, const double *w,
                              double *part, long long ncol, double factor, double *out,
                              cudaStream_t st);
// out[n][r] = factor * rowscale[r] * modscale[n] * sum_s 2^sexp[n][s] P[s][n][r]
// (P float, out double; modscale and sexp optional, sexp [nmod][nsplit])
// + modmean[n] * rowsum[r] when modmean is given (adds back a centred mean).
cudaError_t launch_splitk_reduce(const float *P, int nsplit, long long slice, int nmod, int nrow,
                                 long long ldp, const float *rowscale, const float *modscale,
                                 const int *sexp, const double *modmean, const double *rowsum,
                                 double factor, double *out, long long ld_out, cudaStream_t st);
// Models [nrow][ld_src] (ncol values each) -> fp16 hi / lo [nrow_pad][ld_dst]
// for the forward product with nsp K splits of cols_per_split columns, in one
// pass: centre[r] an estimate of row r's mean (removed before the split), and
// per split the power-of-two scale 2^sexp[r][s]: row r = centre[r] + the
// split's 2^sexp * (hi + lo) on its columns.  Rows beyond nrow are zero.
// sexp holds nrow_pad * (nsp + 1) ints: the table, then the rows' sampled
// exponents.
cudaError_t launch_split_models(const double *src, long long ld_src, int nrow, long long ncol,
                                void *hi, void *lo, long long ld_dst, int nrow_pad,
                                long long cols_per_split, int nsp, double *centre, int *sexp,
                                cudaStream_t st);

// Batched epilogues of the stored products (grid over station x model).
cudaError_t launch_stored_assemble(int kind, int transform, double tbx, double tby, double tbz,
                                   int nmeas, int nmod, const double *sums, long long ld_sums,
                                   const double *bgsens, int nbg, const double *models,
                                   long long ld_models, long long ngrid, const MagField &mf,
                                   double *raw_out, double *data, long long ld_data,
                                   cudaStream_t st);
cudaError_t launch_stored_weights(int kind, int transform, double tbx, double tby, double tbz,
                                  int nmeas, int nmod, const double *misfit, long long ld_misfit,
                                  const double *rawd, const MagField &mf, double *w_raw,
                                  double *w_st, long long ld_w, cudaStream_t st);
// The weights of launch_stored_weights and their split (launch_split_matrix
// without centring, colscale = J's row scales) in one launch, for surveys
// that fit one cluster of CTAs per model (weights_split_fits): w_raw as
// launch_stored_weights writes it, hi / lo / rowscale as the split does.
bool weights_split_fits(int nmeas, long long ld_dst, int nrow_pad);
cudaError_t launch_weights_split(int kind, int transform, double tbx, double tby, double tbz,
                                 int nmeas, int nmod, int nrow_pad, const double *misfit,
                                 long long ld_misfit, const double *rawd, const MagField &mf,
                                 double *w_raw, const float *colscale, float *rowscale, void *hi,
                                 void *lo, long long ld_dst, cudaStream_t st);
cudaError_t launch_bg_grad_batched(int raw, int nmeas, int nbg, int nmod, const double *w_raw,
                                   const double *bgsens, double *grads, long long ld_grads,
                                   long long ngrid, cudaStream_t st);

// Tensor-core products.  A: m rows x ld columns in the tiled layout (buffers of
// tiled_rows(m) rows); B: [n_pad][ld] row-major; both K-major fp16 (or bf16),
// ld a multiple of 64, n_pad a multiple of gemm_n_tile(n), 16-byte aligned bases.
struct GemmOperands {
  const void *a_hi, *a_lo;  // 16-bit elements: bf16, or fp16 when f16 is set
  long long m;
  const void *b_hi, *b_lo;
  long long n, n_pad;
  long long ld;
  bool f16;
  // 1: test the failure path of the bounded waits -- the drain warps
  // withhold their accumulator releases, so the MMA issuer's wait for one
  // expires (after 20 ms) and the launch reports an error code (j3g_set_test_fault)
  int fault = 0;
};
int gemm_n_tile(int n);
int gemm_splits_used(long long ld, int nsplit);
// k-blocks (64 columns) per K split: split s covers k-blocks [s kb, (s + 1) kb).
int gemm_kb_per_split(long long ld, int nsplit);
// P[split][n][ldp] (split stride `slice`) = per-split sums of
// Ahi Bhi + Ahi Blo + Alo Bhi; err receives a non-zero code if a bounded
// wait expired.
// tile: 0 picks gemm_n_tile(n); 64 or 128 force one-SM tiles of that N, 256
// the CTA-pair kernel (n_pad must be a multiple of the tile).
cudaError_t launch_gemm_x3(const GemmOperands &g, int nsplit, float *P, long long ldp,
                           long long slice, int *err, cudaStream_t st, int tile = 0);

}  // namespace j3g
