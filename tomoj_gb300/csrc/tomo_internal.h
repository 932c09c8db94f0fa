// Internal declarations of the GB300 projection / backprojection engine.
//
// Geometry convention ("separable" fast path): with the tilt axis vertical
// (AffineAlignment keeps tiltAxisVertical = true, AffineAlignment.java:18, 389-395)
// every Euler matrix is [[c,0,-s],[0,1,0],[s,0,c]], so projection row j only
// sees volume row r = j - (pc1 - vc1) and the forward projector and
// backprojector work on independent XZ planes.  Positions along a plane are
// kept in 32.32 fixed point so that interpolation weights match the
// reference's double-precision geometry to ~1e-7 pixel; which samples are
// inside the volume / projection is decided on the host with the reference's
// exact double arithmetic and shipped as per-ray / per-column z intervals.
#pragma once
#include <atomic>
#include <functional>
#include <vector>
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace tomo {

constexpr double kFix = 4294967296.0;  // 2^32: fixed-point scale of positions

// Forward-projector occupancy: rays per thread (tilts per CTA x detector columns per
// thread) and resident CTAs per SM, which sets the shared-memory budget of a CTA.
#ifndef TOMO_FP_RAYS
#define TOMO_FP_RAYS 16
#endif
constexpr int kFpRays = TOMO_FP_RAYS;
// CTA shape by detector width: 256 threads, two CTAs per SM, up to 512 columns; 512
// threads, one CTA per SM, above (twice the rays per CTA, so a staged plane serves twice
// the tilts: 1.4x faster at 2048 columns, slower at 512).
constexpr int kFpMaxThreads = 512;
constexpr int fp_ctas_per_sm(int nt) { return nt <= 256 ? 2 : 1; }
constexpr size_t fp_smem_budget(int nt) { return (size_t)(nt <= 256 ? 112 : 226) * 1024; }

// Device status word bits written by kernels (never trap: the host reads them).
constexpr int kStatusTimeout = 1;       // an mbarrier wait exceeded its iteration budget
constexpr unsigned kStatusRange = 4u;   // a volume value left the FP16 range of its slab scale

// One forward-projection ray (tilt t, detector column i).  The ray is inside
// the volume for z in [za, za + cnt); x(z) = X0 + z * step in 32.32 fixed point.
struct alignas(16) FpRay {
    int32_t zab;    // za | cnt << 16 (cnt = 0: the ray misses the volume)
    float norm;     // exact float ray length the reference accumulates (VoxelProjector3D.java:774-783)
    long long X0;   // fixed-point x at z = 0
};

struct alignas(16) FpTilt {
    long long step;  // fixed-point dirX
    double ninc;     // normIncrement
};

// Backprojection of tilt t: xx(x, z) = K + x * C + z * S (fixed point, volume
// indices x, z); voxels of column x are inside the projection for z in
// [zlo, zlo + cnt) (per-column table).
struct alignas(8) BpTilt {
    long long K, C, S;
};

// Generic-geometry forward projection constants of one tilt, the reference's
// expressions of R (VoxelProjector3D.java:682-694).
struct GenericFpTilt {
    double icF, zcF, divY, yFx, zFx, divX, dirX, dirY, ninc;
};

// Per-handle geometry constants (host-computed).
struct Geometry {
    int W, H, D, w, h, N;
    double vc[3], pc[4], scale;
    bool separable;   // all tilts have the vertical-axis form: the XZ-plane kernels apply
    bool fractional;  // ... but rows map with a blend (scale != 1 or centres not a whole row apart)
    int fp_row_off;   // integral rows: r = j - fp_row_off for the forward projector
    int bp_row_off;   // integral rows: j = r + bp_row_off for the backprojector
};

// Host-side table builders (geometry.cpp).  Return false if the tilt is not separable.
bool tilt_is_separable(const double* R, const Geometry& g);
// The vertical-axis form of R (any scale and centres): the XZ-plane kernels apply with
// row maps (fractional rows).
bool tilt_is_vertical(const double* R);
// Row maps of the fractional-row form.  Forward: projection rows [j0, h) of a
// projection whose 2-row tasks start at j0 (VoxelProjector3D.project) -> volume row
// (-1 outside) and float blend weight.  Backward: volume rows [0, H) -> projection row
// (-1 outside) and blend weight (ImageJ getInterpolatedValue's y weight).
void build_fp_rowmap(const Geometry& g, int j0, int* row, float* yf);
void build_bp_rowmap(const Geometry& g, int* row, float* yf);
// normtab_scratch: D + 2 floats the builder may use (nullptr: it allocates its own).
void build_fp_tables(const Geometry& g, const double* R, FpTilt* tilt, FpRay* rays /* w entries */,
                     float* normtab_scratch = nullptr);
void build_bp_tables(const Geometry& g, const double* R, BpTilt* tilt, int32_t* zint /* W entries */);
void build_generic_fp_tilt(const double* R, GenericFpTilt* out);
// M-point spectrum (M a power of two >= 2w - 1) of the real circular kernel
// h = IDFT_w(mask_row), zero-padded: the row filter as a convolution.
void row_filter_spectrum(const float* mask_row, int w, int M, float2* H);
void order_shuffle(int n, const double* euler, int first, int* out);
// fn(begin, end) over [0, n) split into contiguous ranges on up to 16 host threads,
// at least min_per_thread items each (the calling thread takes the first range).
void parallel_ranges(int n, int min_per_thread, const std::function<void(int, int)>& fn);
// In-place radix-2 FFT in double (forward, e^{-2 pi i kn/M}); M a power of two.
void fft_host_forward(std::vector<double>& re, std::vector<double>& im);
int first_index(uint64_t seed, int iteration, int nproj);
void weighting_row_filter(int kind, int w, int nproj, const double* sint, const double* tilts_deg, double diameter,
                          float* mask_row);

// Volume storage types (values of tomo_params.precision).  Reduced types hold
// value / vscale[r] per volume row r (an XZ slab), vscale a power of two.
enum VolType : int { kVolF32 = 0, kVolBF16 = 1, kVolF16 = 2 };
#ifdef __CUDACC__
#define TOMO_HD __host__ __device__
#else
#define TOMO_HD
#endif
TOMO_HD inline size_t vol_elem_bytes(int vt) { return vt == kVolF32 ? 4 : 2; }

// Device kernels (launch wrappers in the .cu files).  All return cudaError_t of the launch.
struct FpLaunch {
    const void* vol;        // [D][H][W] of vtype
    int vtype;              // VolType
    const float* vscale;    // [H] slab scales (reduced types), else nullptr
    const float* meas;      // aligned measured [N][h][w] (nullptr: projection only)
    const int* tilts;       // batch tilt indices [T]
    int T;                  // projections in the batch
    const FpTilt* ftilt;    // [N]
    const FpRay* rays;      // [N][w]
    float* proj;            // [T][h][w]
    float* norm;            // [T][h][w]
    float* diff;            // [T][h][w] (written when meas != nullptr)
    double* errpart;        // [T][h] per-row sum of squared differences
    double factor;          // relaxation factor passed to projectAndDifference
    int j0, j1;             // projection rows to compute
    int tilts_per_cta;
    int W, H, D, w, h;
    int row_off;
    int* status;            // device error word
    // Depth split: zparts CTAs share each (tilt group, row), each summing its own run of
    // planes; partial ray sums go to part[zparts][T][h][w] and the last CTA of the group
    // (ticket in tickets[groups][h], left at zero) adds them in part order and finishes.
    int zparts;             // 0 or 1: no split
    float* part;
    unsigned* tickets;
    // Fractional rows (scale != 1 or centres not a whole row apart): projection row j
    // samples volume rows rowmap[j] and rowmap[j] + 1 blended with weight rowyf[j]
    // (rowmap[j] < 0: the row misses the volume).  nullptr: row j - row_off, no blend.
    const int* rowmap;
    const float* rowyf;
    int two_rows;           // shared memory holds both rows of every plane
    // Failure-path test hook (tomo_debug_hold_first_copy): the first chunk's bulk copies
    // are never issued, so its mbarrier wait runs out after kHoldWaitTries polls and the
    // CTA reports kStatusTimeout and returns (nothing is in flight).  0 in normal use.
    int hold_first_copy;
};
constexpr uint32_t kHoldWaitTries = 1u << 12;
cudaError_t launch_fp_separable(const FpLaunch& a, cudaStream_t s);
// Any geometry (kernels_generic.cu): one thread per ray / voxel in the reference's
// double arithmetic.  proj/norm are [T][h][w] in batch order.
struct FpGenericLaunch {
    const float* vol;
    const int* tilts;
    int T;
    const GenericFpTilt* gtilt;  // [N]
    float* proj;
    float* norm;
    int j0, j1;                  // projection rows; row j0 starts the first 2-row task
    int W, H, D, w, h;
    double pc0x, pc0y, scale, vcx, vcy, vcz, bXmax, bYmax, acc;
};
cudaError_t launch_fp_generic(const FpGenericLaunch& a, cudaStream_t s);
struct BpGenericLaunch {
    float* vol;
    const float* img;            // [T][h][w] batch order
    const int* tilts;
    int T;
    const double* euler;         // [N][9]
    int y0, y1;
    int W, H, D, w, h;
    double vc0, vc1, vc2, cix, ciy, scale;
    int positivity;
};
cudaError_t launch_bp_generic(const BpGenericLaunch& a, cudaStream_t s);

// Depth parts for `ctas` (tilt group, row) CTAs: balances the grid over the resident
// CTA slots of the device (1 = no split).
int fp_zparts(int ctas, int D, int zc, int sms, int ctas_per_sm);
// Plane rows are staged with bulk copies when every row starts on a 16-byte boundary.
inline int fp_use_tma(int W, int vtype, const void* vol) {
    return ((W * vol_elem_bytes(vtype)) % 16 == 0) && ((reinterpret_cast<uintptr_t>(vol) & 15) == 0);
}

struct BpLaunch {
    // Fractional rows: volume row r reads projection rows bprow[r] and bprow[r] + 1
    // (clamped) blended with weight bpyf[r]; bprow[r] < 0: outside.  nullptr: row r + row_off.
    const int* bprow;
    const float* bpyf;
    void* vol;              // [D][H][W] of vtype
    int vtype;              // VolType; reduced types add with Kahan compensation
    const float* vscale;    // [H] slab scales (reduced types)
    unsigned* vmax;         // [H] running max |value| per row as float bits (reduced types)
    const float* img;       // [T][h][w] images to backproject, batch order
    const int* tilts;       // [T] tilt index of each image (for geometry)
    int T;
    const BpTilt* btilt;    // [N]
    const int32_t* zint;    // [N][W]
    int y0, y1;             // volume rows
    int W, H, D, w, h;
    int row_off;
    int positivity;
    int sanitize;           // apply NaN/Inf checks of the reference (images may be non-finite)
    int* status;
    int wide_seg;           // tile footprints up to 192 image columns (scale up to ~2.1)
    int sms;                // multiprocessors of the device (grid-size choices; 0: unknown)
    int rows_mode;          // volume rows per thread: 0 by size and type, 1 one, 2 two (where allowed)
};
cudaError_t launch_bp_separable(const BpLaunch& a, cudaStream_t s);
// Batched backprojection: CTA b runs items[b] = {descriptor, x tile, z tile, row} (with `pairs`, the
// first row of a pair of rows; z tiles of bp_pair_tile_z()).
cudaError_t launch_bp_batch(bool sanitize, bool positivity, int vtype, bool pairs, const BpLaunch* descs,
                            const int4* items, int n_items, cudaStream_t s);
// Persistent batched backprojection: `grid` resident CTAs take items in list order through
// the atomic *cursor (zero before the launch).
cudaError_t launch_bp_persist(bool sanitize, bool positivity, int vtype, bool pairs, const BpLaunch* descs,
                              const int4* items, int n_items, int* cursor, int grid, cudaStream_t s);
int bp_persist_ctas_per_sm(int vtype, bool pairs);
int bp_tile_x();
int bp_tile_z();
// Whole-row backprojections of this kind run two volume rows per CTA (batch items then
// name the first row of each pair, every other row), with z tiles of bp_pair_tile_z().
bool bp_row_pairs(int vtype, bool sanitize, bool positivity);
int bp_pair_tile_z(int vtype);
cudaError_t bp_init_attributes();
// Image columns a BP tile may span for one tilt (segment pairs staged per tilt).
int bp_segment_pairs(bool wide);

cudaError_t launch_align(const float* raw, float* out, const double* tinv /*[N][6]*/, const double* stats, int N,
                         int w, int h, int normalize, int fill, const unsigned char* identity, cudaStream_t s);
// Row filters: bad (optional, one flag per image of rows_per_img rows) turns every row
// of a flagged image into NaN, as the reference's 2-D transform does.
cudaError_t launch_row_filter_tw(float* img, const float* mask_row, const float2* tw, int rows, int w,
                                 const int* bad, int rows_per_img, cudaStream_t s);
// Row filter of any width as a circular convolution (spectrum H and twiddles of M points,
// M a power of two >= 2w - 1, at most kRowConvMaxM).
constexpr int kRowConvMaxM = 8192;
cudaError_t launch_row_filter_conv(float* img, const float2* H, const float2* tw, int rows, int w, int M,
                                   const int* bad, int rows_per_img, cudaStream_t s);
// bad[t] = 1 when image t (npix floats) holds a NaN or an Inf, else 0.
cudaError_t launch_image_nonfinite(const float* imgs, int T, size_t npix, int* bad, cudaStream_t s);
// One DFT length for the 2-D weighting: radix-2 when n is a power of two (M == n),
// otherwise Bluestein on M >= 2n - 1 points.  Device tables: chirp (n), bspec (M),
// tw (M) as built by dft_row_tables.
struct DftRowPlan {
    int n, M, logM;
    const float2* chirp;
    const float2* bspec;
    const float2* tw;
};
constexpr int kDft2MaxN = 4096;
int dft_grid_size(int n);  // M for length n (n <= kDft2MaxN)
void dft_row_tables(int n, int M, float2* chirp, float2* bspec, float2* tw);
// FFTWeighting.createWeightingMask (FFTWeighting.java:31-65), transposed: maskT[i * h + j]
// is the weight of column frequency i, row frequency j.
void weighting_mask_2d(int w, int h, int nproj, const double* tilt_deg, const double* axis_deg, double diameter,
                       float* maskT);
// 2-D weighting of T images (w x h) in place; sa, sb scratch of T*w*h complex each.
cudaError_t launch_weighting_2d(float* imgs, int T, int w, int h, const float* maskT, const DftRowPlan& Pw,
                                const DftRowPlan& Ph, float2* sa, float2* sb, cudaStream_t s);
cudaError_t launch_diff(const float* meas, const int* tilts, const float* th, const float* norm, float* diff,
                        double* errpart, int T, int w, int h, int j0, int j1, double factor, cudaStream_t s);
cudaError_t launch_gather(float* dst, const float* src, const int* tilts, int T, size_t npix, cudaStream_t s);
cudaError_t launch_scan_nonfinite(const float* p, size_t n, int* flags, cudaStream_t s);
int fp_max_tilts_per_cta(int w);
int fp_threads(int w);  // threads per CTA for w detector columns
int fp_qp(int w);       // detector columns per thread (0: w too wide)
int fp_choose_zc(int W, int rows, int vtype, int nt);
size_t fp_smem_bytes(int ZC, int W, int qp, int rows = 1, int vtype = kVolF32);
// Batched forward projection: CTA b runs items[b] = {descriptor, first tilt, row, use_tma};
// pk = 1 when every descriptor of the launch has a 16-bit volume, 0 when all are FP32.
cudaError_t launch_fp_batch(int qp, int nt, const FpLaunch* descs, const int4* items, int n_items, int zc,
                            size_t smem, int pk, cudaStream_t s);
// Persistent batched forward projection: `grid` resident CTAs of nt threads take items
// {descriptor, first tilt, row, flags} in list order through the atomic *cursor (zero
// before the launch); flags: bit 0 bulk copies, bits 1-3 log2 QP, bit 4 16-bit pairs.
// One kernel per (nt, zc) serves every QP of its block size and both pair kinds.
bool fp_persist_supported(int nt, int zc);
cudaError_t launch_fp_persist(int nt, int zc, const FpLaunch* descs, const int4* items, int n_items, int* cursor,
                              int grid, size_t smem, cudaStream_t s);
cudaError_t fp_init_attributes();
cudaError_t misc_init_attributes();
cudaError_t launch_reduce_err(const double* errpart, double* err, int T, int h, cudaStream_t s);
// Batched residual sums: problem b sums errpart[b][T_b][h_b] into err[b][T_b].
struct ErrReduce {
    const double* errpart;
    double* err;
    int T, h;
};
cudaError_t launch_reduce_err_batch(const ErrReduce* jobs, int n_jobs, int max_T, cudaStream_t s);
// One fused TV inner step p_b = updateP(updateU(f, p_a), p_a) (first: p_a = 0), and the
// closing updateU written in place over f.
cudaError_t launch_tv_step(const float* f, const float* const pa[3], float* const pb[3], bool first, int W, int H,
                           int D, float theta, float g, float dt, cudaStream_t s);
cudaError_t launch_tv_final(float* fu, const float* const p[3], int W, int H, int D, float theta, cudaStream_t s);
cudaError_t launch_fill(float* p, size_t n, float v, cudaStream_t s);
cudaError_t launch_fista(float* rec, const float* prev, size_t n, double factor, cudaStream_t s);
cudaError_t launch_long_object(float* norm, int T, int h, int w, cudaStream_t s);
// Bayesian regularisation (BayesianVoxelProjector3D): dist = factor * stencil(rec); and
// dist *= alpha, rec += dist (+ positivity).
cudaError_t launch_bayes_conv(const float* rec, float* dist, int W, int H, int D, double factor, cudaStream_t s);
cudaError_t launch_bayes_apply(float* rec, float* dist, size_t n, double alpha, int positivity, cudaStream_t s);
// BgART (BgARTVoxelProjector3D): histogram collapse filter (scratch: kBgScratchBytes) and
// the 7-point cross median (tmp: a volume-sized copy).
constexpr size_t kBgScratchBytes = 16 + 256 * 8 + 3 * 8;
cudaError_t launch_bgart_collapse(float* vol, size_t n, double k, int dark_bg, double bg_value, void* scratch,
                                  cudaStream_t s);
cudaError_t launch_bgart_median(float* vol, float* tmp, int W, int H, int D, cudaStream_t s);

// Compressed sensing (CompressedSensingProjector.endOfIteration, kernels_wavelet.cu): FP64
// separable fractional spline wavelet transform of the volume, soft threshold at the level
// that zeroes the requested fraction of coefficients, inverse transform, back into the FP32
// volume.  The threshold search runs kWaveletThresholdPasses histogram rounds at most.
constexpr int kWaveletThresholdPasses = 16;
struct WaveletPlan;
// nullptr (with *why) when the parameters or sizes are not supported
WaveletPlan* wavelet_plan_create(int W, int H, int D, const int iters[3], int type, double alpha, double tau,
                                 double fraction_zeros, const char** why);
size_t wavelet_plan_table_bytes(const WaveletPlan* P);
size_t wavelet_plan_state_bytes();
// uploads the tables into d_tables (wavelet_plan_table_bytes) and binds the FP64 buffer
// (W * H * D doubles) and the state (wavelet_plan_state_bytes)
cudaError_t wavelet_plan_bind(WaveletPlan* P, void* d_tables, double* d_buf, void* d_state, cudaStream_t s);
void wavelet_plan_destroy(WaveletPlan* P);
cudaError_t launch_wavelet_filter(const WaveletPlan* P, float* vol, cudaStream_t s);
cudaError_t wavelet_read_threshold(const WaveletPlan* P, double* out, cudaStream_t s);

// Reduced-precision volume storage (kernels_vol.cu).  `src`/`dst` float buffers are
// laid out [D][rows][W] and cover volume rows [y0, y0 + rows).
// Max |value| of each of the rows into vmax[y0 + row] (float bits; vmax zeroed by the caller).
cudaError_t launch_vol_rowmax(const float* src, int rows, int y0, int W, int H, int D, unsigned* vmax,
                              cudaStream_t s);
// vmax holds H + 1 entries: the row maxima and, in entry H, the volume's maximum.
// Picks each row's scale from its maximum (slab_scale_for) or, with `floor`, from its
// maximum and the volume's (vmax[H] set here first; slab_scale_target), and packs src
// into the reduced volume.
cudaError_t launch_vol_pack(const float* src, int rows, int y0, int W, int H, int D, int vtype, void* vol,
                            float* vscale, unsigned* vmax, bool floor, int* status, cudaStream_t s);
cudaError_t launch_vol_unpack(const void* vol, int vtype, const float* vscale, int rows, int y0, int W, int H,
                              int D, float* dst, cudaStream_t s);
// Sets vmax[H] from the row maxima, then re-scales the rows whose scale
// slab_needs_rescale rejects (before a backprojection: rows under the floor; after it:
// rows whose maximum left the band as well).
cudaError_t launch_vol_rescale(void* vol, int vtype, float* vscale, unsigned* vmax, int W, int H, int D,
                               int* status, cudaStream_t s);
// The slab-scale passes around a backprojection for many 16-bit volumes in one launch each
// (a batch's members): before (rows under the floor raised, row maxima zeroed) or after (rows
// whose maximum left the band re-scaled); the same per-volume work as launch_vol_rescale.
struct VolJob {
    void* vol;
    float* vscale;
    unsigned* vmax;
    int vtype, W, H, D;
    int* status;
};
cudaError_t launch_vol_hooks_batch(const VolJob* jobs, int n_jobs, int max_H, bool before, cudaStream_t s);
// Fills the volume with `value`: scales, row maxima and the volume's maximum follow.
cudaError_t launch_vol_fill(void* vol, int vtype, float* vscale, unsigned* vmax, size_t nvox, int H, float value,
                            cudaStream_t s);
cudaError_t launch_scan_nonfinite_vol(const void* vol, int vtype, size_t n, int* flags, cudaStream_t s);

// Streaming multiprocessors of the current device (queried once per device ordinal and
// cached; 1 if the query fails).  Grid sizes of the grid-stride kernels scale with it.
int device_sms();

// Sets the calling thread's message for tomo_last_error.
void set_last_error(const char* msg);

// Counts kernels launched by this library (tomo_kernel_launches).
void count_launch(int n = 1);
extern std::atomic<uint64_t> g_launches;

}  // namespace tomo
