// The projector handle (shared by the C-ABI translation units).
#pragma once
#include <atomic>
#include <vector>

#include "../../include/tomoj_gb300.h"
#include "tomo_internal.h"


struct tomo_projector {
    tomo::Geometry g{};
    tomo_params params{};
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    int device = 0;
    size_t npix = 0, nvox = 0;
    std::vector<void*> allocs;
    uint64_t bytes = 0;

    float* d_vol = nullptr;        // FP32 volume (precision TOMO_PREC_FP32)
    tomo_projector* vol_owner = nullptr;  // d_vol belongs to this handle (tomo_share_volume)
    std::vector<tomo_projector*> vol_sharers;  // handles working on this handle's d_vol
    int vtype = tomo::kVolF32;          // volume storage type (tomo_params.precision)
    uint16_t* d_vol16 = nullptr;   // reduced volume [D][H][W] (BF16 / FP16 bit patterns)
    float* d_vscale = nullptr;     // [H] slab scales of the reduced volume
    unsigned* d_vmax = nullptr;    // [H] row max |value| after the last backprojection
    float* d_vtmp = nullptr;       // FP32 staging rows for set/get of a reduced volume (lazy)
    size_t vtmp_rows = 0;          // volume rows d_vtmp holds
    float* d_tv_f = nullptr;       // FP32 copy of a reduced volume for the TV step (lazy)
    void* vol() const { return vtype == tomo::kVolF32 ? static_cast<void*>(d_vol) : static_cast<void*>(d_vol16); }
    float* d_raw = nullptr;
    float* d_meas = nullptr;
    float* d_proj = nullptr;
    float* d_norm = nullptr;
    float* d_diff = nullptr;
    float* d_obatch = nullptr;
    double* d_errpart = nullptr;
    double* d_err = nullptr;
    int* d_batch = nullptr;
    int* d_orders = nullptr;
    int orders_cap = 0;
    int* d_status = nullptr;
    int* d_flags = nullptr;
    tomo::FpTilt* d_ftilt = nullptr;
    tomo::FpRay* d_rays = nullptr;
    tomo::BpTilt* d_btilt = nullptr;
    // fractional rows: forward row map for the task start fprow_j0, backward row map
    int* d_fprow = nullptr;
    float* d_fpyf = nullptr;
    int* d_bprow = nullptr;
    float* d_bpyf = nullptr;
    int fprow_j0 = -1;
    int bp_wide = 0;        // backprojection tiles need the 192-column segments
    bool bp_generic = false;  // ... or are wider still: the generic backprojector
    std::vector<int> h_fprow;
    std::vector<float> h_fpyf;
    tomo::GenericFpTilt* d_gtilt = nullptr;  // generic geometry: per-tilt FP constants
    double* d_euler = nullptr;               // generic geometry: [N][9] Euler matrices
    int32_t* d_zint = nullptr;
    double* d_tinv = nullptr;
    double* d_stats = nullptr;
    unsigned char* d_identity = nullptr;
    float* d_mask = nullptr;
    float2* d_tw = nullptr;
    float2* d_convH = nullptr;   // non-power-of-two widths: spectrum of the circular kernel
    float2* d_convTw = nullptr;  // and twiddles, conv_M points
    int conv_M = 0;
    int* d_imgbad = nullptr;  // per-image non-finite flags for the row filters
    int imgbad_cap = 0;
    // 2-D weighting (tilt axis not vertical): transposed mask, DFT tables, scratch
    bool weight2d = false;
    float* d_w2mask = nullptr;
    float2* d_w2tab = nullptr;
    float2 *d_w2a = nullptr, *d_w2b = nullptr;
    int w2chunk = 0;
    tomo::DftRowPlan w2pw{}, w2ph{};
    float *d_px = nullptr, *d_py = nullptr, *d_pz = nullptr;  // TV dual field, two buffers (lazy)
    float *d_qx = nullptr, *d_qy = nullptr, *d_qz = nullptr;
    float* d_prev = nullptr;

    std::vector<double> euler;
    std::vector<int> batch;
    bool batch_uploaded = false;
    bool series_loaded = false;
    bool diffs_valid = false;
    bool projected = false;
    bool obatch_valid = false;
    bool meas_has_nan = false, meas_has_inf = false;
    bool vol_nonfinite = false;
    // the flag of the volume this handle works on (the owner's when shared)
    bool& vol_flag() { return vol_owner ? vol_owner->vol_nonfinite : vol_nonfinite; }
    int weight_kind = TOMO_WEIGHT_NONE;
    float tv_theta = 25.0f, tv_g = 1.0f, tv_dt = 0.1f;
    int tv_iters = 0;
    bool fista = false;
    double fista_t = 0.0;
    // BayesianVoxelProjector3D: differences go to d_dist, applied at the end of an iteration
    bool bayes = false;
    double bayes_lambda = 0.1, bayes_alpha = 0.1;
    float* d_dist = nullptr;
    // BgARTVoxelProjector3D: cross median before, histogram collapse after every iteration
    bool bgart = false;
    double bg_k = 0.0, bg_value = 0.0;
    int bg_dark = 1, bg_median = 1;
    void* d_bgscratch = nullptr;
    float* d_bgtmp = nullptr;
    // CompressedSensingProjector: wavelet soft threshold after every iteration
    bool cs = false;
    tomo::WaveletPlan* wav = nullptr;
    double* d_wbuf = nullptr;
    void* d_wtab = nullptr;
    size_t wtab_bytes = 0;
    void* d_wstate = nullptr;
    // volume a backprojection of differences adds to
    void* bp_target() const { return bayes ? static_cast<void*>(d_dist) : vol(); }
    std::atomic<int> cancel{0};
    int tilts_per_cta = 0;  // forward projector tilt grouping (0 = automatic)
    int bp_rows = 0;        // backprojection rows per thread (0 = automatic, 1, 2)
    int hold_first_copy = 0;  // failure-path test hook of the forward projector (tomo_debug_hold_first_copy)
    // row streams: K row ranges of an OS-SART iteration run on K streams (rows are
    // independent), so that forward and backprojections of different rows overlap
    int row_streams = 1;
    cudaStream_t rs[4] = {};
    cudaStream_t rs_reduce = nullptr;
    std::vector<cudaEvent_t> rs_ev;  // fork, per-(subset, range) forward-done, joins
    int sms = 0;            // multiprocessors of the device
    // forward-projector depth split scratch (partial ray sums, per-group tickets)
    float* d_fppart = nullptr;
    size_t fppart_cap = 0;  // floats
    unsigned* d_tickets = nullptr;
    size_t tickets_cap = 0;
    // per-kernel timing of the OS-SART driver (tomo_set_profiling)
    bool profile = false;
    std::vector<cudaEvent_t> ev;
    double prof_ms[2] = {0, 0};  // forward projection (+ residual reduction), backprojection
    long long prof_n[2] = {0, 0};
};

namespace tomo {
// Helpers of tomo_abi.cu used by the batch driver.
// Device buffers from the engine's stream-ordered pool; pool_free orders the release after
// the work queued on `stream`.
cudaError_t pool_malloc(void** ptr, size_t bytes);
void pool_free(void* ptr, cudaStream_t stream);
tomo_status handle_fail(tomo_status code, const char* msg);
tomo_status handle_need_series(tomo_projector* p);
tomo_status handle_start_iteration(tomo_projector* p);
tomo_status handle_end_iteration(tomo_projector* p);
int handle_tilts_per_cta(const tomo_projector* p, int T);
}  // namespace tomo
