/*
 * jif3d_gb300.h -- C ABI of the GB300 gravity / FTG / magnetic prism engine.
 *
 * One opaque context per implementation object, bound to one CUDA device and
 * one stream.  Every call returns an int status (J3G_OK on success) and never
 * exits the process; j3g_last_error() gives the message of the last failure.
 * Calls on one context are not thread-safe (one caller at a time), as the
 * reference's CUDA layer is not (Gravity/GravityInterface.h:19-20).
 *
 * Conventions (identical to jif3D, so no transposes are needed):
 *   model cell (xi, yi, zi) at offset (xi*ny + yi)*nz + zi, z fastest, z down
 *     (ModelBase/ThreeDModelBase.h:157-168);
 *   model vectors hold ngrid grid values followed by nbg background values
 *     (Gravity/ThreeDGravityModel.h:91-99), magnetisation models three ngrid
 *     blocks (x, y, z) and no background;
 *   raw data per station: scalar 1 (g_z), tensor 9 (Uxx..Uzz, C order),
 *     magnetic 3 (Bx, By, Bz), joint 10 (g_z then the 9 tensor values),
 *     vertical magnetic gradient 1, magnetisation 3 (Bx, By, Bz);
 *   sensitivity rows are row-major, nmeas*raw rows of ngrid+nbg columns
 *     (GravMag/FullSensitivityGravMagCalculator.h:116-130);
 *   angles in radians, field strength in nT, densities in kg/m^3, SI output.
 *
 * Pointer arguments named h_* are host memory; d_* are device memory of the
 * context's device.
 */
#ifndef JIF3D_GB300_H_
#define JIF3D_GB300_H_

#ifdef __cplusplus
extern "C" {
#endif

typedef struct j3g_context j3g_context;

enum j3g_status {
  J3G_OK = 0,
  J3G_ERR_ARG = 1,         /* bad argument or size */
  J3G_ERR_CUDA = 2,        /* CUDA runtime error (message in j3g_last_error) */
  J3G_ERR_NOMEM = 3,       /* device or host allocation failed */
  J3G_ERR_STATE = 4,       /* call made before the mesh / stations / kind were set */
  J3G_ERR_UNSUPPORTED = 5, /* combination not supported (e.g. I2 transform on scalar data) */
  J3G_ERR_SCRATCH_LIMIT = 6 /* problem too large for j3g_forward_noalloc's fixed scratch */
};

enum j3g_kind {
  J3G_SCALAR = 1,   /* g_z,             ScalarOMPGravityImp / ScalarCudaGravityImp */
  J3G_TENSOR = 2,   /* FTG 9 components, TensorOMPGravityImp / TensorCudaGravityImp */
  J3G_MAGNETIC = 3, /* induced B,        OMPMagneticSusceptibilityImp / CudaMagneticSusceptibilityImp */
  J3G_JOINT = 4,    /* g_z + FTG in one pass (no single reference counterpart) */
  /* vertical gradient of Bz, one datum per station: Bz(z) - Bz(z + 1 m),
   * Magnetics/OMPMagneticGradImp.cpp:13-106.  Model ngrid susceptibilities +
   * nbg background values, the background does not respond (its gradient is
   * zero, OMPMagneticGradImp.h:32-40).  Transform: none. */
  J3G_MAG_GRADIENT = 5,
  /* remanent magnetisation, Bx By Bz per station,
   * Magnetics/OMPMagnetizationImp.cpp:25-117.  Model 3 * ngrid values: the x,
   * y and z magnetisation blocks (ThreeDMagnetizationModel.h:53-70), no
   * background.  Transforms: none, total field, total-field anomaly.  Not
   * available for the device-resident sensitivity (j3g_build_sensitivity). */
  J3G_MAGNETIZATION = 6
};

enum j3g_transform {
  J3G_T_NONE = 0,
  J3G_T_FTG_INVARIANT = 1, /* FTGInvariant, Gravity/GravityTransforms.h:25-100 */
  J3G_T_TOTAL_FIELD = 2,   /* TotalField, Magnetics/MagneticTransforms.h:19-82 */
  J3G_T_TFA = 3            /* TotalFieldAnomaly, Magnetics/MagneticTransforms.h:84-156 */
};

/* Text of a status code. */
const char *j3g_status_string(int status);
/* Message of the last failing call on ctx (empty string if none). */
const char *j3g_last_error(const j3g_context *ctx);

/* Create a context on CUDA device `device` with its own stream.  Replaces the
 * device probing of PrepareData (Gravity/gravcuda.cu:38-77), minus its exit()
 * calls and its search for an unused device. */
int j3g_create(j3g_context **ctx, int device);
/* Free every device buffer of ctx.  Replaces FreeData (Gravity/gravcuda.cu:8-26);
 * it never resets the device (the reference destructors call cudaDeviceReset,
 * ScalarCudaGravityImp.cpp:52). */
int j3g_destroy(j3g_context *ctx);
/* Launch on a caller-owned stream (cudaStream_t passed as void*; NULL restores
 * the context's own stream). */
int j3g_set_stream(j3g_context *ctx, void *stream);

/* Mesh: corner coordinates (n+1 values each, ThreeDModelBase::GetXCoordinates)
 * and cell sizes (n values each).  Replaces the allocation and H2D copies of
 * PrepareData (Gravity/gravcuda.cu:79-106). */
int j3g_set_mesh(j3g_context *ctx, int nx, int ny, int nz, const double *h_xcoord,
                 const double *h_ycoord, const double *h_zcoord, const double *h_xsize,
                 const double *h_ysize, const double *h_zsize);
/* Background layer thicknesses (ThreeDGravityModel::GetBackgroundThicknesses);
 * the layer densities / susceptibilities are the last nbg model values. */
int j3g_set_background(j3g_context *ctx, int nbg, const double *h_thick);
/* Measurement positions (GeneralData::GetMeasPosX/Y/Z). */
int j3g_set_stations(j3g_context *ctx, int nmeas, const double *h_x, const double *h_y,
                     const double *h_z);
/* Kind of data and, for J3G_MAGNETIC, the inducing field: inclination and
 * declination in radians, field strength in nT
 * (OMPMagneticSusceptibilityImp(Inc, Dec, Fs), Magnetics/OMPMagneticSusceptibilityImp.cpp:196). */
int j3g_set_kind(j3g_context *ctx, int kind, double inclination, double declination,
                 double field_strength);
/* Output transform (ThreeDGravMagImplementation::SetDataTransform,
 * GravMag/ThreeDGravMagImplementation.h:67-70); angles used by J3G_T_TFA. */
int j3g_set_transform(j3g_context *ctx, int transform, double inclination, double declination);
/* Sizes implied by the current setup (any pointer may be NULL). */
int j3g_get_sizes(const j3g_context *ctx, long long *ngrid, long long *nparm, int *nmeas,
                  int *raw_per_meas, int *data_per_meas);

/* Forward response of all stations (host buffers): model nparm values ->
 * data nmeas*data_per_meas values.  Matrix-free, no sensitivities kept.
 * Replaces ThreeDGravMagImplementation::Calculate
 * (GravMag/ThreeDGravMagImplementation.h:116-168) driven by
 * MinMemGravMagCalculator, and the per-station SingleScalarMeas /
 * SingleFTGMeas launches (Gravity/gravcuda.cu:117-197). */
int j3g_forward(j3g_context *ctx, const double *h_model, double *h_data);
/* As j3g_forward, and also the raw sensitivity rows (nmeas*raw x nparm,
 * row-major) that FullSensitivityGravMagCalculator stores through
 * HandleSensitivities (GravMag/FullSensitivityGravMagCalculator.h:98-130).
 * The data are formed from the rows, cell by cell, as CalcGridded does. */
int j3g_forward_sens(j3g_context *ctx, const double *h_model, double *h_data, double *h_sens);
/* Least-squares derivative 2 * J^T (T' misfit), length nparm, computed
 * matrix-free (box terms recomputed, nothing stored).  misfit has
 * nmeas*data_per_meas values (already C_d^-1 weighted).  Replaces
 * ThreeDGravMagImplementation::LQDerivative (GravMag/ThreeDGravMagImplementation.h:177-231). */
int j3g_lqderivative(j3g_context *ctx, const double *h_model, const double *h_misfit,
                     double *h_grad);

/* Device-resident variants of j3g_forward / j3g_lqderivative (pointers on
 * the context's device, work queued on the context's stream; no host sync). */
int j3g_forward_device(j3g_context *ctx, const double *d_model, double *d_data);
int j3g_lqderivative_device(j3g_context *ctx, const double *d_model, const double *d_misfit,
                            double *d_grad);

/* ---- Station subsets ---------------------------------------------------------
 * A batch of station subsets of uneven size on the current mesh, model and
 * kind -- e.g. survey lines or blocks inverted separately -- in one node-term
 * launch per direction instead of one Calculate / LQDerivative per subset.
 * Subset k holds the stations h_index[h_offsets[k] .. h_offsets[k+1]) (host
 * arrays: nsub + 1 non-decreasing offsets from 0, indices into the stations
 * set with j3g_set_stations; a station may belong to several subsets).
 * Forward: data of every listed station, subset after subset
 * (h_offsets[nsub] * data_per_meas values).  Adjoint: d_misfit in the same
 * layout; one gradient per subset, nsub x nparm values, each
 * 2 J_k^T (T' misfit_k) over that subset's stations only.  No single reference
 * counterpart (the reference evaluates each subset with its own calculator). */
int j3g_subsets_forward_device(j3g_context *ctx, int nsub, const int *h_offsets,
                               const int *h_index, const double *d_model, double *d_data);
int j3g_subsets_lqderivative_device(j3g_context *ctx, int nsub, const int *h_offsets,
                                    const int *h_index, const double *d_model,
                                    const double *d_misfit, double *d_grads);

/* ---- Model refinement -------------------------------------------------------
 * An inversion on a coarse grid with the forward calculation on a refined
 * grid: ModelRefiner (ModelBase/ModelRefiner.h:33-128, ModelRefiner.cpp:17-218)
 * as ThreeDModelObjective uses it on either side of the forward and the
 * gradient (Inversion/ThreeDModelObjective.h:188-201, 254-260, 310-324).
 *
 * j3g_refine_axis is RefineOneAxis (ModelRefiner.cpp:17-72): the refined cell
 * sizes of one axis from the coarse corners (ncoarse + 1 values, as
 * GetXCoordinates returns them), the coarse sizes and nref refinement
 * coordinates (the fine model's GetXCoordinates; as in the reference the last
 * one, the end of the domain, is not used).  Every coarse corner is kept, the
 * refinement coordinates inside each coarse cell are inserted and the last
 * cell ends where the coarse domain ends.  Writes the count to *nfine and at
 * most capacity sizes (capacity 0 queries the count).  J3G_ERR_ARG when the
 * last refined cell would not have a positive size (the reference's
 * FatalException; *nfine = -1), when nref < 1, or when capacity is too small.
 * Host only: no context and no GPU needed. */
int j3g_refine_axis(int ncoarse, const double *h_coarse_coords, const double *h_coarse_sizes,
                    int nref, const double *h_ref_coords, int capacity, double *h_fine_sizes,
                    int *nfine);
/* Attach the coarse (inversion) grid to a context whose mesh is the refined
 * forward grid.  Along each axis a coarse cell takes refined cells in order
 * until their summed sizes reach its own size (FindEnd, ModelRefiner.cpp:
 * 92-102).  Coarse models are [cnx][cny][cnz] cell blocks (three for
 * magnetisation) followed by the background parameters; j3g_set_mesh clears
 * the refinement. */
int j3g_set_refinement(j3g_context *ctx, int cnx, int cny, int cnz, const double *h_xsizes,
                       const double *h_ysizes, const double *h_zsizes);
/* Cells and parameters of one coarse model; *covers_all is 0 when some
 * refined cells lie outside every coarse cell's run (rounding in the walk). */
int j3g_refinement_info(const j3g_context *ctx, long long *coarse_cells, long long *coarse_nparm,
                        int *covers_all);
/* ProjectValues (ModelRefiner.cpp:124-168) for nmodels models: every refined
 * cell takes the value of its coarse cell; refined cells outside every run
 * keep their values; the background parameters are copied, as the objective's
 * ExtraParameterSetter does (ThreeDModelObjective.h:238-248).  Bit-exact. */
int j3g_refine_project_device(j3g_context *ctx, int nmodels, const double *d_coarse,
                              double *d_fine);
/* CombineGradient (ModelRefiner.cpp:170-218): each coarse entry is the sum of
 * the refined entries of its cell, added in x, y, z order as the reference
 * adds them (bit-exact); the background entries are copied
 * (ThreeDModelObjective.h:319-323). */
int j3g_refine_combine_device(j3g_context *ctx, int nmodels, const double *d_fine,
                              double *d_coarse);
/* Host-buffer forms of the two (copy in, run, copy out, synchronise). */
int j3g_refine_project(j3g_context *ctx, int nmodels, const double *h_coarse, double *h_fine);
int j3g_refine_combine(j3g_context *ctx, int nmodels, const double *h_fine, double *h_coarse);

/* ---- Device-resident sensitivity matrix ------------------------------------
 * The GPU counterpart of FullSensitivityGravMagCalculator's cached path
 * (GravMag/FullSensitivityGravMagCalculator.h:116-221): J is built once per
 * geometry from the FP64 box terms and kept in HBM; later products reuse it
 * without recomputing any box term.  Stored rows per station: scalar 1 (g_z),
 * tensor 6 (Uxx Uyy Uzz Uxy Uxz Uyz), joint 7 (g_z + the 6), magnetic 3
 * (Bx By Bz); the background columns stay FP64.  Any set_mesh / set_stations
 * / set_kind / set_background call drops it.  Needs corner coordinates that
 * are running sums of the cell sizes (as jif3D builds them). */
enum j3g_storage {
  J3G_STORE_FP32 = 1, /* FP32 J, streamed by FP32-FMA products with FP64 sums */
  J3G_STORE_F16X2 = 2 /* J = s_r (hi + lo), fp16 hi / lo (22 significant bits) with a
                         power-of-two row scale s_r, plus the transposed copy; products on
                         the tensor cores.  (A bf16 hi / lo pair keeps only 16 bits, which
                         leaves ~2e-6 relative error on FTG rows.) */
};
int j3g_build_sensitivity(j3g_context *ctx, int storage);
int j3g_drop_sensitivity(j3g_context *ctx);
/* storage kind, stored rows, columns (cells) and device bytes of the stored J. */
int j3g_sensitivity_info(const j3g_context *ctx, int *storage, long long *rows, long long *cols,
                         long long *bytes);
/* Cached forward d = T(J m) and derivative 2 J^T (T' misfit) of one model
 * with the stored J (FullSensitivityGravMagCalculator::CalculateCachedResult
 * :154-167 and CachedLQDerivative :169-221). */
int j3g_stored_forward_device(j3g_context *ctx, const double *d_model, double *d_data);
int j3g_stored_lqderivative_device(j3g_context *ctx, const double *d_model,
                                   const double *d_misfit, double *d_grad);
/* The same for nmodels models at once (line-search trials, Monte-Carlo
 * samples): models [nmodels][nparm], data [nmodels][nmeas*data_per_meas],
 * misfits like data, gradients like models.  With J3G_STORE_F16X2 storage
 * the products run on the tensor cores: models and scaled misfits are split
 * into fp16 hi / lo parts with power-of-two scales, J M ~= Jhi Mhi + Jhi Mlo
 * + Jlo Mhi; all three products of every 32 cells go to a fresh TMEM
 * accumulator (cross terms first), which is drained into FP32 register sums;
 * K splits of at most 4096 cells are summed as FP32 two-sum pairs and in FP64
 * (about 1e-7 relative error).
 * The _device forms queue work only; the host forms copy in and out and
 * synchronise (page-locked host buffers copy at full link speed).  The
 * derivative reads the models only under the FTG-invariant and total-field
 * transforms, whose derivative depends on the data; otherwise the host form
 * does not copy them (h_models may then be NULL). */
int j3g_batched_forward_device(j3g_context *ctx, int nmodels, const double *d_models,
                               double *d_data);
int j3g_batched_lqderivative_device(j3g_context *ctx, int nmodels, const double *d_models,
                                    const double *d_misfits, double *d_grads);
int j3g_batched_forward(j3g_context *ctx, int nmodels, const double *h_models, double *h_data);
int j3g_batched_lqderivative(j3g_context *ctx, int nmodels, const double *h_models,
                             const double *h_misfits, double *h_grads);
/* Pipelined host-buffer forms: the call queues the copy of its inputs in,
 * the product and the copy of its output back, and returns a ticket; the
 * copies run on streams of the context's own, one in and one out per
 * direction (forward, derivative), so they overlap the products of the calls
 * before and after, and a forward's data or a derivative's misfits do not
 * queue behind the other direction's model-sized copies.  j3g_batched_wait(ticket)
 * blocks until that call's output is in host memory.  Up to four calls are
 * in flight (a fifth waits for the first: enough to queue a forward two
 * steps ahead of the misfit it feeds).  A call's product is replayed from a
 * CUDA graph of its slot once the same shape has run with no buffer grown or
 * plan tuned; any set_*, plan, timing or sensitivity change retires the
 * graphs.  The host buffers must stay
 * valid and unchanged until the call is waited for, and page-locked host
 * buffers are needed for the copies to overlap. */
int j3g_batched_forward_async(j3g_context *ctx, int nmodels, const double *h_models,
                              double *h_data, long long *ticket);
int j3g_batched_lqderivative_async(j3g_context *ctx, int nmodels, const double *h_models,
                                   const double *h_misfits, double *h_grads, long long *ticket);
int j3g_batched_wait(j3g_context *ctx, long long ticket);

/* ---- NetCDF files: jif3D's on-disk data and models ---------------------------
 * jif3D stores data and models with netCDF (Gravity/ReadWriteGravityData.cpp,
 * Magnetics/ReadWriteMagneticData.cpp, ModelBase/NetCDFModelTools.cpp); this
 * library reads and writes those files itself, with no NetCDF or HDF5
 * library.  Readers take NetCDF classic files (CDF-1, CDF-2, CDF-5) and
 * netCDF-4 files (HDF5: compact or contiguous datasets, compact or
 * symbol-table groups, as netCDF-4 writes jif3D's files); chunked datasets
 * are J3G_ERR_ARG with a message.  The writer produces CDF-2 (64-bit offset)
 * files, which jif3D's netCDF-C++ reads like its own.  Values are exchanged
 * as double.  Host only: no context and no GPU.  On failure the message is
 * j3g_nc_last_error() (per thread). */
typedef struct j3g_ncfile j3g_ncfile;
typedef struct j3g_ncwriter j3g_ncwriter;
enum { J3G_NC_BYTE = 1, J3G_NC_CHAR = 2, J3G_NC_SHORT = 3, J3G_NC_INT = 4, J3G_NC_FLOAT = 5,
       J3G_NC_DOUBLE = 6 };
const char *j3g_nc_last_error(void);
/* Read a whole file (NcFile(filename, NcFile::read)). */
int j3g_nc_open(const char *path, j3g_ncfile **file);
int j3g_nc_close(j3g_ncfile *file);
/* 1, 2, 5: classic CDF-1 / CDF-2 / CDF-5; 4: netCDF-4 (HDF5). */
int j3g_nc_format(const j3g_ncfile *file, int *format);
int j3g_nc_nvars(const j3g_ncfile *file, int *nvars);
int j3g_nc_var_name(const j3g_ncfile *file, int index, int capacity, char *name);
/* Shape of a variable (getVar(name).getDims()); J3G_ERR_ARG if it is absent. */
int j3g_nc_var_shape(const j3g_ncfile *file, const char *var, int capacity, int *ndims,
                     long long *shape);
/* All values of a variable, row-major, as double (ReadVec, Global/NetCDFTools.h). */
int j3g_nc_read_var(const j3g_ncfile *file, const char *var, long long count, double *values);
/* Length of a dimension (getDim(name).getSize()). */
int j3g_nc_dim_len(const j3g_ncfile *file, const char *dim, long long *len);
/* A text attribute of a variable, or of the file when var is NULL. */
int j3g_nc_text_att(const j3g_ncfile *file, const char *var, const char *att, int capacity,
                    char *value);
/* Writer (NcFile(filename, NcFile::replace), addDim, addVar, putAtt, putVar);
 * the file is written by j3g_nc_close_writer, which also frees the writer. */
int j3g_nc_create(const char *path, j3g_ncwriter **writer);
int j3g_nc_def_dim(j3g_ncwriter *writer, const char *name, long long len);
int j3g_nc_def_var(j3g_ncwriter *writer, const char *name, int type, int ndims,
                   const char *const *dims);
int j3g_nc_put_text_att(j3g_ncwriter *writer, const char *var, const char *name,
                        const char *value);
int j3g_nc_put_var(j3g_ncwriter *writer, const char *var, long long count,
                   const double *values);
int j3g_nc_close_writer(j3g_ncwriter *writer);
/* Free a writer without writing its file. */
int j3g_nc_discard_writer(j3g_ncwriter *writer);

/* Block until the context's stream is idle; reports J3G_ERR_CUDA if a
 * bounded wait inside a tensor-core kernel expired since the last check. */
int j3g_synchronize(j3g_context *ctx);
/* Number of CUDA kernels this context has queued since it was created. */
int j3g_launch_count(const j3g_context *ctx, long long *count);

/* Kernel timing (for rooflines): while enabled, the dominant launches of each
 * category are bracketed by CUDA events on the context's stream.
 * j3g_set_timing(ctx, 1) starts a new measurement (clears old records);
 * j3g_get_timing synchronises and returns the summed device time (ms) and
 * the number of timed launches of one category. */
enum j3g_timer {
  J3G_TIMER_NODE_FORWARD = 0,   /* k_node_forward */
  J3G_TIMER_NODE_ADJOINT = 1,   /* k_node_adjoint */
  J3G_TIMER_STREAM_FORWARD = 2, /* FP32 J m streaming product */
  J3G_TIMER_STREAM_ADJOINT = 3, /* FP32 J^T r streaming product (column blocks) */
  J3G_TIMER_GEMM_FORWARD = 4,   /* tensor-core J M */
  J3G_TIMER_GEMM_ADJOINT = 5,   /* tensor-core J^T R */
  J3G_TIMER_SPLIT = 6,          /* fp16 hi / lo split of models and residual weights */
  J3G_TIMER_REDUCE = 7,         /* FP64 sums of the per-split tensor-core partials */
  J3G_TIMER_EPILOGUE = 8        /* batched data assembly, residual weights, background */
};
int j3g_set_timing(j3g_context *ctx, int enable);
int j3g_get_timing(j3g_context *ctx, int category, double *total_ms, long long *launches);

/* Autotuning of the tensor-core products (J3G_STORE_F16X2 batched calls); no
 * reference counterpart.  Off by default: a fixed rule picks the K-split count
 * and the N tile (about six waves of CTAs, at most 128 k-blocks per split), so
 * a caller that never calls this -- the unchanged jif3D calculators through
 * the C++ implementation, for one -- runs untuned plans.  With enable = 1, the first product of each shape (direction,
 * rows, models, K) times a few candidate plans -- split counts that fill the
 * last wave of CTAs, and one-SM 128-wide tiles in place of CTA pairs -- and
 * keeps the fastest for the context's lifetime.  Every candidate keeps the
 * accuracy bound of the fixed rule (at most 128 k-blocks per split).  Tuning
 * synchronises the context's stream, so the first call of a shape must not be
 * made while the stream is being captured into a CUDA graph; results can
 * differ from the fixed plan's in the last bits (another summation order). */
int j3g_set_autotune(j3g_context *ctx, int enable);
/* Fix the plan of one direction (0 forward, 1 adjoint): K splits and N tile
 * (0 = by the number of models, 64, 128, 256; a tile the batch does not fill
 * falls back to the automatic plan).  nsplit <= 0 returns to the fixed rule or
 * the autotuner.  For reproducible runs with a plan found by tuning; more
 * than 128 k-blocks per split loses accuracy (the split sums are FP32). */
int j3g_set_gemm_plan(j3g_context *ctx, int direction, int nsplit, int tile);
/* The plan the last batched product used: direction 0 forward (J M), 1
 * adjoint (J^T R); K splits requested, N tile (64, 128 or 256 = CTA pair) and
 * the autotuner's time of that plan in ms (0 for the fixed rule). */
int j3g_get_gemm_plan(const j3g_context *ctx, int direction, int *nsplit, int *tile,
                      double *tuned_ms);
/* Failure-path test of the tensor-core products' bounded waits; no
 * counterpart in the reference (whose CUDA layer exits on any error,
 * Global/CudaError.h:13-22).  With fault = 1, every later tensor-core product
 * launch of this context simulates a stalled pipeline without faulting the
 * GPU: its drain warps withhold the releases of their TMEM accumulators, the
 * MMA issuer gives up on one after 20 ms, stops issuing and waits for the
 * MMAs and copies it has issued (each wait bounded by 2 s), and the launch
 * records an error code; the call that checks the flag (j3g_synchronize,
 * j3g_batched_forward / _lqderivative, j3g_batched_wait) returns
 * J3G_ERR_CUDA and clears it, and the context stays usable.  A launch
 * takes about 2 s in this mode and its results are not defined.  fault = 0
 * restores the normal path.  Test use only. */
int j3g_set_test_fault(j3g_context *ctx, int fault);

/* Allocation-free gridded forward, for callers that cannot let a library
 * allocate device memory: hosts that reserve all device memory for their own
 * pool allocator at start-up, or loops that must not take the device-wide
 * synchronisation of cudaMalloc / cudaFree.  No counterpart in the reference.
 *
 * Computes the raw gridded data (no background layers, no transform) of
 * every station, nmeas * raw values into d_data, for the model d_model
 * (nx*ny*nz values).  d_xnode / d_ynode / d_znode are the nx+1 / ny+1 / nz+1
 * mesh node coordinates, i.e. corner coordinates that are the running sums of
 * the cell sizes (ThreeDModelBase::CalcCoords).  All pointers are device
 * memory of the current device; work is queued on `stream` (a cudaStream_t,
 * NULL for the legacy default stream) and the call does not synchronise.
 *
 * Scratch is a fixed 16 MiB device array inside the library (held by every
 * GPU that loads the library until the process exits): the call allocates and
 * frees nothing.  It needs (nx+1)(ny+1)(nz+1) + 7*nmeas doubles plus at least
 * one block of nmeas*ncomp doubles (ncomp = 1 scalar, 6 tensor / magnetic,
 * 7 joint), all rounded up to 32 doubles, within 2^21 doubles; larger problems
 * return J3G_ERR_SCRATCH_LIMIT without touching d_data.  Every call shares
 * the array and leaves its last contents behind (each call writes all it
 * reads, nothing needs to start at zero), so calls that overlap on the GPU
 * race on it and must be serialised by the caller.  Each call made outside
 * stream capture looks up the array's device address on the current device
 * (cudaGetSymbolAddress), so a device reset between calls is harmless; a call
 * on a capturing stream reuses the address of the device's last call outside
 * capture and returns J3G_ERR_STATE if there was none, so make the first call
 * on a device (and the first after a device reset) before any stream capture. */
int j3g_forward_noalloc(int kind, int nx, int ny, int nz, const double *d_xnode,
                        const double *d_ynode, const double *d_znode, int nmeas,
                        const double *d_sx, const double *d_sy, const double *d_sz,
                        double inclination, double declination, double field_strength,
                        const double *d_model, double *d_data, void *stream);

/* Measured FP64 FMA rate of the device in GFLOP/s (2 flops per FMA), from
 * independent FMA chains in a probe kernel of this library; the denominator of
 * the FP64 roofline fractions that the benchmark reports (no vendor-published
 * or externally measured FP64 figure is available for the device).  No
 * counterpart in the reference. */
int j3g_probe_fp64(j3g_context *ctx, double *gflops);

#ifdef __cplusplus
}
#endif
#endif /* JIF3D_GB300_H_ */
