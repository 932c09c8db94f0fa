/*
 * tomoj_gb300.h -- C ABI of the GB300 projection / backprojection engine.
 *
 * The engine is a drop-in for TomoJ's Projector plug-in surface
 * (TomoJ_Base/src/main/java/fr/curie/tomoj/tomography/projectors/Projector.java)
 * and for the iteration drivers that call it
 * (TomoJ_Base/src/main/java/fr/curie/tomoj/tomography/TomoReconstruction2.java).
 * Every entry point is a plain C function taking POD structs, pointers and
 * sizes, returns a tomo_status (0 = success), and never throws; the last error
 * message of the calling thread is available from tomo_last_error().
 *
 * Data layouts (identical to the reference's in-memory layouts):
 *   volume      float32 [D][H][W]   (D slices of W x H, x fastest;
 *                                    TomoReconstruction2 ImageStack)
 *   tilt-series float32 [N][h][w]   (TiltSeries ImageStack)
 *   euler       float64 [N][3][3]   row-major (AffineAlignment.getEulerMatrix)
 *   transform   float64 [N][6]      java.awt.geom.AffineTransform flat matrix
 *                                    {m00, m10, m01, m11, m02, m12}
 *
 * A handle is thread-compatible (one thread at a time).  All device work of a
 * handle runs on its stream (tomo_set_stream; default: a stream the handle
 * creates).  Calls that take host pointers copy synchronously on that stream.
 */
#ifndef TOMOJ_GB300_H
#define TOMOJ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TOMO_ABI_VERSION 1

typedef int32_t tomo_status;
#define TOMO_OK 0
#define TOMO_ERR_INVALID (-1)     /* bad argument or size */
#define TOMO_ERR_CUDA (-2)        /* CUDA runtime error (message in tomo_last_error) */
#define TOMO_ERR_NOMEM (-3)       /* admission control: not enough free HBM under the limit */
#define TOMO_ERR_STATE (-4)       /* call out of order (e.g. backproject with no projection) */
#define TOMO_ERR_UNSUPPORTED (-5) /* geometry or option not supported by the engine */
#define TOMO_ERR_CANCELLED (-6)   /* tomo_cancel() was called */
#define TOMO_ERR_DEVICE (-7)      /* a kernel reported an error status (bounded wait expired) */

/* TiltSeries fill types (TiltSeries.FILL_*) used when aligning projections. */
#define TOMO_FILL_NONE 0
#define TOMO_FILL_AVG 1
#define TOMO_FILL_NAN 2

/* WBP weighting filters.  RADERMACHER is FFTWeighting (FFTWeighting.java:31-112);
 * RAMP and HAMMING_RAMP are row filters with no counterpart in the reference. */
#define TOMO_WEIGHT_NONE 0
#define TOMO_WEIGHT_RADERMACHER 1
#define TOMO_WEIGHT_RAMP 2
#define TOMO_WEIGHT_HAMMING_RAMP 3

/* Storage precision of the volume (accumulation is always FP32).  BF16 and FP16
 * keep each volume row (an XZ slab) as value / scale in 16 bits with a per-row
 * power-of-two scale; backprojection sums are Kahan-compensated FP32 and residual
 * norms FP64.  These modes have no counterpart in the reference (float volumes). */
#define TOMO_PREC_FP32 0
#define TOMO_PREC_BF16 1
#define TOMO_PREC_FP16 2

typedef struct tomo_geom {
    int32_t W, H, D;        /* volume width (x), height (y: tilt-axis rows), depth (z) */
    int32_t w, h;           /* projection width, height */
    int32_t nproj;          /* projections in the tilt-series */
    double vol_center[3];   /* TomoReconstruction2 centres; NaN = default (n-1)/2 */
    double proj_center[4];  /* TiltSeries centerX, centerY (forward projection) and
                               projectionCenterX, projectionCenterY (backprojection);
                               NaN = default (n-1)/2 */
    double scale;           /* projection/volume scale (VoxelProjector3D.setScale); 0 = 1 */
} tomo_geom;

typedef struct tomo_params {
    int32_t positivity;     /* VoxelProjector3D.setPositivityConstraint */
    int32_t long_object;    /* VoxelProjector3D.setLongObjectCompensation */
    int32_t fill;           /* TOMO_FILL_* for tomo_load_series alignment */
    int32_t normalize;      /* TiltSeries.setNormalize: (x-mean)/stdDev per tilt */
    int32_t precision;      /* TOMO_PREC_* */
    int32_t reserved[3];
} tomo_params;

typedef struct tomo_projector tomo_projector;

/* ---- library ---------------------------------------------------------- */
int32_t tomo_abi_version(void);
const char* tomo_last_error(void);
/* Upper bound on device bytes the library may hold across all handles
 * (admission control; 0 = no limit besides free HBM). */
tomo_status tomo_set_memory_limit(uint64_t bytes);
uint64_t tomo_memory_in_use(void);
/* Free and total bytes of the current device (ProjectorGPU.computeMaximumSizeForVolume
 * sizes a volume from them, ProjectorGPU.java:162-166).  Free counts the idle blocks of
 * the engine's device memory pool: handle buffers are carved from one stream-ordered pool
 * per device that keeps what destroyed handles return, so that retiring a handle does not
 * wait for the whole device. */
tomo_status tomo_device_memory(uint64_t* free_bytes, uint64_t* total_bytes);
/* Number of kernels this library launched since load (all handles). */
uint64_t tomo_kernel_launches(void);

/* ---- lifetime ----------------------------------------------------------
 * Replaces the Projector constructor (Projector.java:30-40), which captures
 * dimensions and centres from the TiltSeries and TomoReconstruction2. */
tomo_status tomo_create(const tomo_geom* geom, const tomo_params* params, tomo_projector** out);
tomo_status tomo_destroy(tomo_projector* p);
/* cudaStream_t passed as void*; NULL returns to the handle's own stream. */
tomo_status tomo_set_stream(tomo_projector* p, void* stream);
/* Recreates the handle's own stream at a scheduling priority (no counterpart in the
 * reference; same scale as tomo_batch_set_priority: 0 default, larger more urgent). */
tomo_status tomo_set_priority(tomo_projector* p, int32_t priority);

/* ---- data ---------------------------------------------------------------
 * Uploads the unaligned tilt-series and per-tilt geometry and builds the
 * aligned projections that TiltSeries.getPixels(i) returns
 * (TiltSeries.java:678-687 -> AffineAlignment.applyTransformOnImage,
 * AffineAlignment.java:136-259).  transforms may be NULL (identity); stats
 * (per tilt {mean, stdDev}) may be NULL (0, 1).  pixels_on_device != 0 means
 * `pixels` is a device pointer. */
tomo_status tomo_load_series(tomo_projector* p, const float* pixels, int32_t pixels_on_device, const double* euler,
                             const double* transforms, const double* stats);
/* TiltSeries.setFillType: re-aligns the resident series with another fill policy
 * (WBP uses FILL_AVG, iterative methods FILL_NAN; WBPReconstructionApplication.java:52,
 * IterativeReconstructionApplication.java:196). */
tomo_status tomo_set_fill(tomo_projector* p, int32_t fill);
/* The aligned projection `index` as the projector sees it (host copy). */
tomo_status tomo_get_aligned(tomo_projector* p, int32_t index, float* out_host);
/* Volume rows [y0,y1) from/to a host or device buffer laid out [D][y1-y0][W]. */
tomo_status tomo_set_volume(tomo_projector* p, const float* src, int32_t on_device, int32_t y0, int32_t y1);
tomo_status tomo_get_volume(tomo_projector* p, float* dst, int32_t on_device, int32_t y0, int32_t y1);
tomo_status tomo_fill_volume(tomo_projector* p, float value);
/* Device pointer of the resident volume [D][H][W] (valid until tomo_destroy). */
tomo_status tomo_volume_device_ptr(tomo_projector* p, float** out);
/* Two projectors on one TomoReconstruction2 (the dual-axis drivers ADASIRT / ADOSSART,
 * TomoReconstruction2.java:880-1100, build projector1 and projector2 on the same rec):
 * p works in place on owner's volume (same W, H, D; FP32 storage) and on owner's
 * stream, so their calls run in order; p's own volume is released.  owner must stay
 * alive while shared.  owner == NULL gives p a private copy of the volume it sees. */
tomo_status tomo_share_volume(tomo_projector* p, tomo_projector* owner);

/* ---- Projector surface (Projector.java:130-156) ------------------------- */
tomo_status tomo_add_projection(tomo_projector* p, int32_t index);          /* addProjection(int) */
tomo_status tomo_clear_projections(tomo_projector* p);                      /* clearAllProjections() */
tomo_status tomo_project(tomo_projector* p, int32_t y0, int32_t y1);       /* project(y0,y1) */
/* projectAndDifference(factor,y0,y1): err_out[k] = sum of squared differences of
 * the k-th added projection (may be NULL). */
tomo_status tomo_project_and_difference(tomo_projector* p, double factor, int32_t y0, int32_t y1, double* err_out);
tomo_status tomo_backproject(tomo_projector* p, int32_t y0, int32_t y1);   /* backproject(y0,y1) */
tomo_status tomo_start_iteration(tomo_projector* p);                        /* startOfIteration() */
tomo_status tomo_end_iteration(tomo_projector* p);                          /* endOfIteration() */
/* getProjection(k): forward projection of the k-th added projection (w*h floats). */
tomo_status tomo_get_projection(tomo_projector* p, int32_t k, float* out_host);
tomo_status tomo_get_norm(tomo_projector* p, int32_t k, float* out_host);
tomo_status tomo_get_difference(tomo_projector* p, int32_t k, float* out_host);
int32_t tomo_projection_count(tomo_projector* p);

/* ---- options ------------------------------------------------------------ */
/* VoxelProjector3D setters (VoxelProjector3D.java:78-104): positivity constraint,
 * long-object compensation, and the projection / reconstruction scale (the geometry
 * tables are rebuilt when a series is loaded).  setNbRaysPerPixels has no engine
 * call: the Joseph projector of the reference ignores it (projectJosephPartial reads
 * one ray per pixel; projectPartial resets it to 1, VoxelProjector3D.java:471). */
tomo_status tomo_set_positivity(tomo_projector* p, int32_t enabled);
/* OS-SART iterations over K (1..4) row ranges on K streams: volume rows are
 * independent with a vertical tilt axis, so the forward projection of one range can
 * overlap the backprojection of another.  Used for whole-row centre offsets, scale 1
 * geometry, FP32 storage and no long-object compensation; otherwise one stream. */
tomo_status tomo_set_row_streams(tomo_projector* p, int32_t k);
tomo_status tomo_set_long_object(tomo_projector* p, int32_t enabled);
tomo_status tomo_set_scale(tomo_projector* p, double scale);
/* Projector.setVolumeCenters(cx, cy, cz) / setProjectionCenter(...) (Projector.java:52-108):
 * vol_center {cx, cy, cz}, proj_center {centerX, centerY, projectionCenterX,
 * projectionCenterY}; NULL or NaN entries keep their value.  Rebuilds the geometry
 * tables of a loaded series. */
tomo_status tomo_set_centers(tomo_projector* p, const double* vol_center, const double* proj_center);
/* WBP weighting applied before every backprojection (VoxelProjector3D.java:163-166),
 * replacing new FFTWeighting(ts, radius * w) (ReconstructionParameters.java:320,
 * FFTWeighting.java:22-24).  tilt_deg: per-tilt ts.getTiltAngle(i) in degrees (NULL =
 * read from the Euler matrices, which then must have a vertical axis); tilt_axes:
 * per-tilt ts.getTiltAxis(i) in degrees (NULL = 0).  A zero axis filters rows; any
 * other axis applies the 2-D mask through 2-D transforms (Radermacher only, w and h
 * up to 4096). */
tomo_status tomo_set_weighting(tomo_projector* p, int32_t kind, double radius, const double* tilt_deg,
                               const double* tilt_axes);
/* TVM regularisation run at endOfIteration (TVMProjector3D.java:135-157):
 * ROF denoise with theta, g, dt for `iterations` inner steps; iterations 0 disables. */
tomo_status tomo_set_tvm(tomo_projector* p, float theta, float g, float dt, int32_t iterations);
/* FISTA momentum wrapper (FistaProjector3D.java). */
tomo_status tomo_set_fista(tomo_projector* p, int32_t enabled);
/* BayesianVoxelProjector3D (TomoJ_AdvancedReconstruction/.../projectors/
 * BayesianVoxelProjector3D.java): startOfIteration sets a distance volume to
 * -lambda times the 27-point [1,-2,1]^3 stencil of the volume, every update's
 * differences are backprojected into it instead of the volume, and
 * endOfIteration adds alpha times it to the volume (then positivity, if set).
 * FP32 volumes only. */
tomo_status tomo_set_bayesian(tomo_projector* p, double lambda, double alpha, int32_t enabled);
/* BgARTVoxelProjector3D (TomoJ_AdvancedReconstruction/.../projectors/
 * BgARTVoxelProjector3D.java): a 7-point cross median before every iteration
 * (do_median), and after every iteration the histogram collapse filter: voxels
 * on the background side of mode +/- k sigma become the background value (the
 * histogram mode, or bg_value when it is not NaN).  Enabling applies the
 * collapse once to the current volume, as the reference's constructor does.
 * FP32 volumes only. */
tomo_status tomo_set_bgart(tomo_projector* p, double k, int32_t dark_bg, int32_t do_median, double bg_value,
                           int32_t enabled);
/* CompressedSensingProjector (TomoJ_AdvancedReconstruction/.../projectors/
 * CompressedSensingProjector.java:34-155; the reference's setters setWaveletType,
 * setWaveletDegree, setWaveletShift, setSoftThresholdingPercentageOfZeros and
 * setWaveletsIterations): after every iteration the volume goes through the
 * separable 3-D fractional spline wavelet transform (wavelet_type 0 orthonormal,
 * 3 B-spline, 6 dual; degree > -0.5; shift), is soft-thresholded at the level that
 * zeroes fraction_zeros of the coefficients, and is transformed back.
 * levels = {x, y, z} transform levels, or NULL for the reference's default (the
 * same count on every axis, from the width).  Every level's line length must be
 * even (TOMO_ERR_UNSUPPORTED otherwise).  FP32 volumes only. */
tomo_status tomo_set_compressed_sensing(tomo_projector* p, int32_t wavelet_type, double degree, double shift,
                                       double fraction_zeros, const int32_t* levels, int32_t enabled);
/* The soft threshold of the last wavelet filter (synchronises the handle's stream). */
tomo_status tomo_compressed_sensing_threshold(tomo_projector* p, double* out);

/* ---- drivers (TomoReconstruction2) --------------------------------------- */
/* WBP(ts, projector, params, y0, y1) with update 0 (TomoReconstruction2.java:499-538). */
tomo_status tomo_run_wbp(tomo_projector* p, int32_t y0, int32_t y1);
/* OSSART(ts, projector, params, y0, y1) (TomoReconstruction2.java:548-634):
 * update 0 = SIRT (all projections per update), 1 = ART.  The first projection
 * of every iteration's ordering comes from tomo_first_index(seed, iteration)
 * instead of Math.random().  err_out (n_iter*5, may be NULL) receives
 * {average, min, argmin, max, argmax} per iteration.  Iterations run as one
 * CUDA graph per iteration when use_graph != 0. */
tomo_status tomo_run_ossart(tomo_projector* p, int32_t n_iter, double relax, int32_t update, uint64_t seed,
                            int32_t y0, int32_t y1, int32_t use_graph, double* err_out);
/* Deterministic replacement for the random first index of orderShuffleART. */
int32_t tomo_first_index(uint64_t seed, int32_t iteration, int32_t nproj);
/* orderShuffleART ordering (TomoReconstruction2.java:735-781) for a first index. */
tomo_status tomo_order(tomo_projector* p, int32_t first, int32_t* order_out);
/* Same ordering for explicit Euler matrices (nproj x 9); needs no handle or GPU. */
tomo_status tomo_order_shuffle(int32_t nproj, const double* euler, int32_t first, int32_t* order_out);
/* Cooperative cancel, polled between updates (TomoReconstruction2.interrupt). */
tomo_status tomo_cancel(tomo_projector* p);

/* ---- batching (no counterpart in the reference) ------------------------------
 * A batch runs iterations of many handles together (heterogeneous tilt-series:
 * sizes, tilt counts and schemes may differ): for every update index one
 * forward-projection launch per kernel variant covers that update of every
 * member, then one residual reduction and one backprojection launch.  Members
 * keep their own volumes, series and options (TVM, positivity...); the batch
 * only references them, so destroy the batch before its handles.  A step's
 * launches are captured as one CUDA graph and replayed while the membership
 * and update sizes are unchanged.  Members must live on one device. */
typedef struct tomo_batch tomo_batch;
tomo_status tomo_batch_create(tomo_batch** out);
tomo_status tomo_batch_destroy(tomo_batch* b);
/* Scheduling priority of the batch's stream (no counterpart in the reference): 0 is the
 * device default, each step above asks for the next more urgent stream priority, clamped
 * to the device's range.  As SMs free up, CTAs of a more urgent stream are dispatched
 * first, so a batch of small series is not held behind the long launches of a batch of
 * large ones. */
tomo_status tomo_batch_set_priority(tomo_batch* b, int32_t priority);
/* cudaStream_t passed as void* for the batch's work (NULL: the batch's own stream).
 * Members' own streams must be idle at each iteration, as with the batch's own stream. */
tomo_status tomo_batch_set_stream(tomo_batch* b, void* stream);
/* Persistent launches (no counterpart in the reference; default off): each forward phase
 * is one launch per CTA size (256 threads up to 512 detector columns, 512 above) and each
 * backprojection phase one launch per storage type and rule set, of resident CTAs that
 * take work items from a device list, longest first, through an atomic cursor.  Off: one
 * launch per kernel variant with a CTA per item, which measured faster on GB300 (64
 * heterogeneous series: 0.97 against 0.85-0.88 T voxel-updates/s).  Results are bitwise
 * the same.  on: 0 off, 1 on; for tuning, a sum of 2 (forward phase persistent), 4
 * (backprojection persistent), 8 (lists in plan order instead of longest first) and 16
 * (launches of a phase one after another instead of side by side). */
tomo_status tomo_batch_set_persistent(tomo_batch* b, int32_t on);
/* Replaces the membership (n handles). */
tomo_status tomo_batch_set(tomo_batch* b, tomo_projector* const* members, int32_t n);
/* One OS-SART iteration of every member (osartIteration, TomoReconstruction2.java:636-733):
 * relax[m], update[m] (0 = SIRT) and the ordering's first index first[m] per member;
 * err_out (n*5, may be NULL) receives each member's {average, min, argmin, max, argmax}. */
tomo_status tomo_batch_iteration(tomo_batch* b, const double* relax, const int32_t* update, const int32_t* first,
                                 int32_t use_graph, double* err_out);

/* ---- measurement (no counterpart in the reference; Chrono-style timing) ----
 * When enabled, tomo_run_ossart records CUDA events around every forward
 * projection (+ residual reduction) and backprojection launch on the handle's
 * stream; tomo_profile_read returns {fp_ms, fp_launches, bp_ms, bp_launches}
 * accumulated since profiling was enabled. */
tomo_status tomo_set_profiling(tomo_projector* p, int32_t enabled);
tomo_status tomo_profile_read(tomo_projector* p, double* out4);
/* Tilts per forward-projection CTA (0 = automatic; tuning knob). */
tomo_status tomo_set_tilts_per_cta(tomo_projector* p, int32_t n);
/* Volume rows per backprojection thread (tuning knob, no counterpart in the reference):
 * 0 = by size and storage type, 1 = one row, 2 = two rows (FP32 volumes with a vertical
 * tilt axis and whole-row centre offsets; otherwise one row).  Results are bitwise the
 * same either way. */
tomo_status tomo_set_bp_rows(tomo_projector* p, int32_t rows);
/* Autotuner (no counterpart in the reference): times the forward projection with
 * difference and the backprojection of one update of `update` tilts (0: all) of the
 * loaded series under each candidate kernel shape -- forward-projection tilts per CTA
 * (automatic grouping, the register maximum and 3/4, 1/2, 1/4 of it) and backprojection
 * rows per thread (1, 2) -- with CUDA events over `reps` launches each (0: 3), and keeps
 * the fastest on the handle (tomo_set_tilts_per_cta / tomo_set_bp_rows; batches use each
 * member's choice).  The added projections are cleared; the volume is saved and put back.
 * Every candidate computes the same values, up to the FP32 summation order where a tilt
 * grouping changes the depth split of a small grid.  out4 (may be NULL): {tilts per CTA
 * (0 = automatic), rows per thread, forward ms, backprojection ms} of the choice. */
tomo_status tomo_autotune(tomo_projector* p, int32_t update, int32_t reps, double* out4);
/* Failure-path test hook (no counterpart in the reference): while enabled, the
 * forward projector of this handle does not issue the bulk copies of each CTA's
 * first plane chunk, so that chunk's bounded mbarrier wait runs out, the CTA
 * records the timeout in the device status word and returns with nothing in
 * flight; the call reports TOMO_ERR_DEVICE and the handle stays usable.  Only
 * volumes whose rows are staged with bulk copies (W * element size a multiple
 * of 16 bytes) are affected. */
tomo_status tomo_debug_hold_first_copy(tomo_projector* p, int32_t enabled);

/* ---- projection + difference without allocation ----------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a JVM that keeps all device memory in its own pre-sized pool, a serving loop
 * that may not take cudaMalloc's implicit synchronisation mid-request, code held
 * to a fixed memory budget): the forward projection + difference of one update
 * (projectAndDifference) on the caller's device buffers, with no handle.
 *   volume  device float32 [D][H][W]      meas  device float32 [nproj][h][w] (aligned)
 *   proj, norm, diff  device float32 [T][h][w] outputs (slot b = tilts[b])
 *   err_out host double [T]               euler host double [nproj][9]
 * Its scratch lives in one static device array of about 5 MiB that every GPU
 * loading the library keeps until exit.  Limits: nproj <= 128, T <= 64,
 * w, h <= 2048, W up to about 9500 (one plane row in the forward projector's
 * shared memory), vertical tilt axis.  Long-object compensation is not applied
 * (the plain projector's norms and differences).  The first call on a device sets up the
 * scratch address (make it before any stream capture).  Calls share the
 * scratch: calls that overlap on the GPU, or run concurrently, race.
 * Synchronous on `stream` (cudaStream_t as void*, NULL = default stream). */
tomo_status tomo_project_and_difference_noalloc(const tomo_geom* geom, const double* euler, const int32_t* tilts,
                                                int32_t T, double factor, const float* volume, const float* meas,
                                                float* proj, float* norm, float* diff, double* err_out,
                                                void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TOMOJ_GB300_H */
