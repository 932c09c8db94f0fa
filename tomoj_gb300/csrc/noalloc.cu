// Projection + difference for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a JVM that hands the
// library only buffers from its own pre-sized device pool (the Java host must
// keep device memory under its own accounting), a serving loop that may not
// take cudaMalloc's implicit device synchronisation or its latency in the
// middle of a request, and code that must stay within a fixed, pre-reserved
// memory budget.  tomo_project_and_difference_noalloc gives them the forward
// projection + difference step on their own device buffers: the caller passes
// the volume, the aligned measurements and the output images; the scratch the
// step needs (ray tables, per-row residual partials, the residual vector and
// the kernel status word) lives in one file-scope __device__ array of
// kNoAllocScratchBytes, which every GPU that loads the library holds until the
// process exits.  Host-side scratch is file-scope static as well, so the call
// allocates nothing on the device, and nothing on the host unless it fails (the
// error message for tomo_last_error).
//
// Limits: nproj <= 128 tilts in the series, <= 64 tilts per call, w <= 2048,
// h <= 2048, D <= 65535, W such that one plane row and its pairs fit the forward
// projector's shared memory (W up to about 9500), vertical tilt axis (separable
// geometry); larger sizes are rejected with TOMO_ERR_INVALID / TOMO_ERR_UNSUPPORTED.
// Long-object compensation (setLongObjectCompensation) is not applied: the norms
// and differences are those of the plain projector.
//
// The first call on each device does the set-up (cudaGetSymbolAddress of the
// scratch array and the kernels' shared-memory attributes) with that device
// current; make that first call before any stream capture.  All calls share
// the one scratch array and its contents persist between calls (the call
// clears what must start at zero), so calls that overlap on the GPU race, and
// the host-side tables are shared too: do not run two calls concurrently.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/tomoj_gb300.h"
#include "tomo_internal.h"

namespace tomo {
namespace {

constexpr int kMaxNproj = 128;
constexpr int kMaxBatch = 64;
constexpr int kMaxW = 2048;
constexpr int kMaxH = 2048;
constexpr int kMaxD = 65535;
constexpr int kMaxDevices = 64;

// Device scratch layout (bytes): ray tables | tilt steps | per-row residuals |
// residuals | batch indices | status word.
constexpr size_t kRaysOff = 0;
constexpr size_t kRaysBytes = sizeof(FpRay) * (size_t)kMaxNproj * kMaxW;          // 4 MiB
constexpr size_t kTiltOff = kRaysOff + kRaysBytes;
constexpr size_t kTiltBytes = sizeof(FpTilt) * (size_t)kMaxNproj;                   // 2 KiB
constexpr size_t kErrpartOff = kTiltOff + kTiltBytes;
constexpr size_t kErrpartBytes = sizeof(double) * (size_t)kMaxBatch * kMaxH;        // 1 MiB
constexpr size_t kErrOff = kErrpartOff + kErrpartBytes;
constexpr size_t kErrBytes = sizeof(double) * (size_t)kMaxBatch;
constexpr size_t kBatchOff = kErrOff + kErrBytes;
constexpr size_t kBatchBytes = sizeof(int) * (size_t)kMaxBatch;
constexpr size_t kStatusOff = kBatchOff + kBatchBytes;
constexpr size_t kNoAllocScratchBytes = kStatusOff + 256;                              // ~5.0 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Host-side scratch (file scope: the call does not touch the heap).  Every tilt of a
// call has its own ray-table slot, so all uploads are queued before one synchronisation.
static FpRay h_rays[kMaxBatch][kMaxW];
static FpTilt h_tilts[kMaxNproj];
static float h_normtab[kMaxD + 2];
static int h_batch[kMaxBatch];

static std::mutex g_setup_mu;
static void* g_dev_scratch[kMaxDevices];

// Reported through tomo_last_error (only error paths touch the message string).
tomo_status nerr(tomo_status code, const char* msg) {
    set_last_error(msg);
    return code;
}

tomo_status device_scratch(unsigned char** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return nerr(TOMO_ERR_CUDA, "no current CUDA device");
    }
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_dev_scratch[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            cudaGetLastError();
            return nerr(TOMO_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
        }
        if (fp_init_attributes() != cudaSuccess) {
            cudaGetLastError();
            return nerr(TOMO_ERR_CUDA, "cannot configure forward-projector shared memory");
        }
        g_dev_scratch[dev] = ptr;
    }
    *out = static_cast<unsigned char*>(g_dev_scratch[dev]);
    return TOMO_OK;
}

}  // namespace
}  // namespace tomo

using namespace tomo;

extern "C" tomo_status tomo_project_and_difference_noalloc(const tomo_geom* geom, const double* euler,
                                                           const int32_t* tilts, int32_t T, double factor,
                                                           const float* d_volume, const float* d_meas,
                                                           float* d_proj, float* d_norm, float* d_diff,
                                                           double* err_out, void* stream) {
    if (!geom || !euler || !tilts || !d_volume || !d_meas || !d_proj || !d_norm || !d_diff || !err_out)
        return nerr(TOMO_ERR_INVALID, "null argument");
    if (T <= 0 || T > kMaxBatch) return nerr(TOMO_ERR_INVALID, "between 1 and 64 tilts per call");
    if (geom->nproj <= 0 || geom->nproj > kMaxNproj) return nerr(TOMO_ERR_INVALID, "at most 128 tilts in the series");
    if (geom->w <= 0 || geom->w > kMaxW || geom->h <= 0 || geom->h > kMaxH)
        return nerr(TOMO_ERR_INVALID, "projections larger than 2048 x 2048");
    if (geom->W <= 0 || geom->H <= 0 || geom->D <= 0 || geom->D > kMaxD)
        return nerr(TOMO_ERR_INVALID, "bad volume size");
    // the forward projector stages at least one plane row of W voxels (and its pairs) in
    // shared memory: wider volumes are refused before anything is uploaded
    if (fp_qp(geom->w) == 0 || fp_smem_bytes(1, geom->W, fp_qp(geom->w), 1) > fp_smem_budget(fp_threads(geom->w)))
        return nerr(TOMO_ERR_INVALID, "volume width W too large for the forward projector's shared memory");
    Geometry g{};
    g.W = geom->W;
    g.H = geom->H;
    g.D = geom->D;
    g.w = geom->w;
    g.h = geom->h;
    g.N = geom->nproj;
    const double dvc[3] = {(g.W - 1) / 2.0, (g.H - 1) / 2.0, (g.D - 1) / 2.0};
    const double dpc[4] = {(g.w - 1.0) / 2, (g.h - 1.0) / 2, (g.w - 1) / 2.0, (g.h - 1) / 2.0};
    for (int k = 0; k < 3; k++) g.vc[k] = std::isnan(geom->vol_center[k]) ? dvc[k] : geom->vol_center[k];
    for (int k = 0; k < 4; k++) g.pc[k] = std::isnan(geom->proj_center[k]) ? dpc[k] : geom->proj_center[k];
    g.scale = geom->scale == 0.0 ? 1.0 : geom->scale;
    for (int b = 0; b < T; b++) {
        if (tilts[b] < 0 || tilts[b] >= g.N) return nerr(TOMO_ERR_INVALID, "tilt index out of range");
        if (!tilt_is_separable(euler + 9 * (size_t)tilts[b], g))
            return nerr(TOMO_ERR_UNSUPPORTED, "needs a vertical tilt axis, scale 1 and integral row offsets");
    }
    unsigned char* scr = nullptr;
    tomo_status st = device_scratch(&scr);
    if (st != TOMO_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    FpRay* d_rays = reinterpret_cast<FpRay*>(scr + kRaysOff);
    FpTilt* d_ft = reinterpret_cast<FpTilt*>(scr + kTiltOff);
    double* d_errpart = reinterpret_cast<double*>(scr + kErrpartOff);
    double* d_err = reinterpret_cast<double*>(scr + kErrOff);
    int* d_batch = reinterpret_cast<int*>(scr + kBatchOff);
    int* d_status = reinterpret_cast<int*>(scr + kStatusOff);
    // ray tables of the requested tilts (the closed-form intervals of the handle path; only
    // rays that graze a border replay the reference's accumulation), in their series slots
    for (int b = 0; b < T; b++) {
        const int t = tilts[b];
        build_fp_tables(g, euler + 9 * (size_t)t, &h_tilts[t], h_rays[b], h_normtab);
        if (cudaMemcpyAsync(d_rays + (size_t)t * g.w, h_rays[b], sizeof(FpRay) * g.w, cudaMemcpyHostToDevice, s) !=
                cudaSuccess ||
            cudaMemcpyAsync(d_ft + t, &h_tilts[t], sizeof(FpTilt), cudaMemcpyHostToDevice, s) != cudaSuccess) {
            cudaGetLastError();
            return nerr(TOMO_ERR_CUDA, "table upload failed");
        }
        h_batch[b] = t;
    }
    const int offset = (g.h > g.H && g.scale == 1) ? (g.h - g.H) / 2 : 0;
    const int j0 = std::max(0, (int)std::floor(offset * g.scale + 0.5));
    const int j1 = g.h;
    const size_t npix = (size_t)g.w * g.h;
    bool ok = cudaMemcpyAsync(d_batch, h_batch, sizeof(int) * T, cudaMemcpyHostToDevice, s) == cudaSuccess;
    // scratch that must start at zero: rows the kernel does not write, and the status word
    ok = ok && cudaMemsetAsync(d_errpart, 0, sizeof(double) * (size_t)T * g.h, s) == cudaSuccess;
    ok = ok && cudaMemsetAsync(d_status, 0, sizeof(int), s) == cudaSuccess;
    if (j0 > 0)
        for (int b = 0; b < T && ok; b++) {
            const size_t rowbytes = sizeof(float) * (size_t)std::min(j0, g.h) * g.w;
            ok = cudaMemsetAsync(d_proj + b * npix, 0, rowbytes, s) == cudaSuccess &&
                 cudaMemsetAsync(d_norm + b * npix, 0, rowbytes, s) == cudaSuccess &&
                 cudaMemsetAsync(d_diff + b * npix, 0, rowbytes, s) == cudaSuccess;
        }
    if (!ok) {
        cudaGetLastError();
        return nerr(TOMO_ERR_CUDA, "scratch clear failed");
    }
    if (j0 < j1) {
        FpLaunch a{};
        a.vol = d_volume;
        a.meas = d_meas;
        a.tilts = d_batch;
        a.T = T;
        a.ftilt = d_ft;
        a.rays = d_rays;
        a.proj = d_proj;
        a.norm = d_norm;
        a.diff = d_diff;
        a.errpart = d_errpart;
        a.factor = factor;
        a.j0 = j0;
        a.j1 = j1;
        const int tgmax = fp_max_tilts_per_cta(g.w);
        const int groups = (T + tgmax - 1) / tgmax;
        a.tilts_per_cta = (T + groups - 1) / groups;
        a.W = g.W;
        a.H = g.H;
        a.D = g.D;
        a.w = g.w;
        a.h = g.h;
        a.row_off = (int)(g.pc[1] - g.vc[1]);
        a.status = d_status;
        if (launch_fp_separable(a, s) != cudaSuccess) {
            cudaGetLastError();
            return nerr(TOMO_ERR_CUDA, "forward-projection launch failed");
        }
    }
    int status = 0;
    if (launch_reduce_err(d_errpart, d_err, T, g.h, s) != cudaSuccess ||
        cudaMemcpyAsync(err_out, d_err, sizeof(double) * T, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return nerr(TOMO_ERR_CUDA, "projection failed");
    }
    if (status != 0) return nerr(TOMO_ERR_DEVICE, "a bounded wait in the projection kernel expired");
    return TOMO_OK;
}
