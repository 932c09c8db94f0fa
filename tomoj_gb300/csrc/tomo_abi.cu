// C ABI of the engine: handles, admission control, the Projector surface and
// the TomoReconstruction2 drivers.  See include/tomoj_gb300.h for the contract.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tomoj_gb300.h"
#include "tomo_internal.h"
#include "tomo_handle.h"

namespace tomo {
std::atomic<uint64_t> g_launches{0};
void count_launch(int n) { g_launches += (uint64_t)n; }
}  // namespace tomo

using namespace tomo;

namespace {

thread_local std::string g_err;
std::atomic<uint64_t> g_in_use{0};
std::atomic<uint64_t> g_limit{0};

tomo_status fail(tomo_status code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define CK(expr)                                                                                      \
    do {                                                                                              \
        cudaError_t _e = (expr);                                                                      \
        if (_e != cudaSuccess)                                                                        \
            return fail(TOMO_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));           \
    } while (0)

#define CKS(expr)                     \
    do {                              \
        tomo_status _s = (expr);      \
        if (_s != TOMO_OK) return _s; \
    } while (0)

}  // namespace

void tomo::set_last_error(const char* msg) { g_err = msg; }


namespace {

// Handle buffers come from one stream-ordered memory pool per device that keeps the blocks
// it gets back (release threshold unlimited).  Destroying a handle returns its buffers with
// cudaFreeAsync, which does not wait for the whole device as cudaFree does (a server that
// retires a request would otherwise stall every other request's kernels), and the next
// handle's buffers are carved from those blocks.  Admission counts the pool's idle blocks
// as free HBM.  Allocations are made on a private stream and completed before use.
struct DevicePool {
    cudaMemPool_t pool = nullptr;
    cudaStream_t stream = nullptr;
    bool tried = false;
};
std::mutex g_pool_mu;
DevicePool g_pools[64];

DevicePool* device_pool() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_pool_mu);
    DevicePool& d = g_pools[dev];
    if (!d.tried) {
        d.tried = true;
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        if (cudaMemPoolCreate(&d.pool, &props) != cudaSuccess ||
            cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            if (d.pool) cudaMemPoolDestroy(d.pool);
            d.pool = nullptr;
        } else {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(d.pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    return d.pool ? &d : nullptr;
}

size_t pool_idle_bytes(const DevicePool* d) {
    if (!d) return 0;
    uint64_t reserved = 0, used = 0;
    cudaMemPoolGetAttribute(d->pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
    cudaMemPoolGetAttribute(d->pool, cudaMemPoolAttrUsedMemCurrent, &used);
    return reserved > used ? (size_t)(reserved - used) : 0;
}

// Returns a buffer; `stream` orders the release after the work queued there.
void dfree(void* ptr, cudaStream_t stream) {
    if (!ptr) return;
    DevicePool* d = device_pool();
    if (d) {
        if (cudaFreeAsync(ptr, stream) != cudaSuccess) cudaGetLastError();
    } else {
        cudaFree(ptr);
    }
}

tomo_status dalloc(tomo_projector* p, void** ptr, size_t bytes) {
    if (bytes == 0) bytes = 16;
    const uint64_t lim = g_limit.load();
    if (lim != 0 && g_in_use.load() + bytes > lim)
        return fail(TOMO_ERR_NOMEM, "admission: " + std::to_string(bytes) + " bytes exceed the memory limit");
    DevicePool* d = device_pool();
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && bytes > free_b + pool_idle_bytes(d))
        return fail(TOMO_ERR_NOMEM, "admission: " + std::to_string(bytes) + " bytes exceed free HBM");
    cudaError_t e;
    if (d) {
        e = cudaMallocFromPoolAsync(ptr, bytes, d->pool, d->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
    } else {
        e = cudaMalloc(ptr, bytes);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(TOMO_ERR_NOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
    }
    p->allocs.push_back(*ptr);
    p->bytes += bytes;
    g_in_use += bytes;
    return TOMO_OK;
}

template <class T>
tomo_status alloc_n(tomo_projector* p, T** ptr, size_t n) {
    return dalloc(p, reinterpret_cast<void**>(ptr), n * sizeof(T));
}

// Frees one of the handle's allocations early (bytes as allocated) and clears *ptr.
template <class T>
void free_n(tomo_projector* p, T** ptr, size_t n) {
    if (!*ptr) return;
    dfree(*ptr, p->stream);  // after the handle's queued work that may still read it
    for (auto& a : p->allocs)
        if (a == (void*)*ptr) a = nullptr;
    g_in_use -= n * sizeof(T);
    p->bytes -= n * sizeof(T);
    *ptr = nullptr;
}

tomo_status check_status(tomo_projector* p) {
    int st = 0;
    CK(cudaMemcpyAsync(&st, p->d_status, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    if (st != 0) {
        CK(cudaMemsetAsync(p->d_status, 0, sizeof(int), p->stream));
        // a kernel that gave up may have left depth-split tickets behind
        if (p->d_tickets) CK(cudaMemsetAsync(p->d_tickets, 0, sizeof(unsigned) * p->tickets_cap, p->stream));
        std::string why;
        if (st & kStatusTimeout) why += " (bounded wait expired)";
        if (st & (int)kStatusRange) why += " (a volume value left the FP16 range of its slab scale)";
        return fail(TOMO_ERR_DEVICE, "a kernel reported status " + std::to_string(st) + why);
    }
    return TOMO_OK;
}

tomo_status upload_batch(tomo_projector* p) {
    if (p->batch_uploaded) return TOMO_OK;
    if (!p->batch.empty())
        CK(cudaMemcpyAsync(p->d_batch, p->batch.data(), p->batch.size() * sizeof(int), cudaMemcpyHostToDevice,
                           p->stream));
    // the host vector may change after this call: make the copy complete first
    CK(cudaStreamSynchronize(p->stream));
    p->batch_uploaded = true;
    return TOMO_OK;
}

// Projection row range of project(y0,y1) (VoxelProjector3D.java:338-352): from
// round((y0 + offset) * scale) to the projection height.
void fp_rows(const tomo_projector* p, int y0, int* j0, int* j1) {
    const Geometry& g = p->g;
    const int offset = (g.h > g.H && g.scale == 1) ? (g.h - g.H) / 2 : 0;
    int s = (int)std::floor((y0 + offset) * g.scale + 0.5);
    if (s < 0) s = 0;
    *j0 = s;
    *j1 = g.h;
}

// Tilts per forward-projection CTA: the widest grouping the registers allow, split
// evenly (every CTA re-stages the row's XZ plane, so fewer, wider groups reuse
// each staged plane more; measured faster than splitting for occupancy).
int auto_tilts_per_cta(const tomo_projector* p, int T, int rows) {
    (void)rows;
    const int tgmax = fp_max_tilts_per_cta(p->g.w);
    if (p->tilts_per_cta > 0) return std::min(p->tilts_per_cta, tgmax);
    const int groups = (T + tgmax - 1) / tgmax;
    return (T + groups - 1) / groups;
}

// Depth split of a forward projection of T tilts over rows [j0, j1): the number of
// parts, after making sure the scratch exists.  Scratch is only allocated outside
// stream capture; a captured launch that lacks it runs unsplit.
int fp_split(tomo_projector* p, int T, int rows, int tpc) {
    const Geometry& g = p->g;
    const int groups = (T + tpc - 1) / tpc;
    const int nt = fp_threads(g.w);
    const int P = fp_zparts(groups * rows, g.D, fp_choose_zc(g.W, g.fractional ? 2 : 1, p->vtype, nt), p->sms,
                            fp_ctas_per_sm(nt));
    if (P <= 1) return 1;
    const size_t need_part = (size_t)P * T * p->npix;
    const size_t need_tk = (size_t)groups * g.h;
    if (need_part <= p->fppart_cap && need_tk <= p->tickets_cap) return P;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(p->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return 1;
    if (need_part > p->fppart_cap) {
        free_n(p, &p->d_fppart, p->fppart_cap);
        p->fppart_cap = 0;
        if (alloc_n(p, &p->d_fppart, need_part) != TOMO_OK) return 1;
        p->fppart_cap = need_part;
    }
    if (need_tk > p->tickets_cap) {
        free_n(p, &p->d_tickets, p->tickets_cap);
        p->tickets_cap = 0;
        if (alloc_n(p, &p->d_tickets, need_tk) != TOMO_OK) return 1;
        if (cudaMemsetAsync(p->d_tickets, 0, sizeof(unsigned) * need_tk, p->stream) != cudaSuccess) return 1;
        p->tickets_cap = need_tk;
    }
    return P;
}

// Forward row map of the fractional-row form for projections whose tasks start at
// row j0 (uploaded when j0 changes; the host copy stays alive for captured copies).
tomo_status ensure_fp_rowmap(tomo_projector* p, int j0) {
    if (p->fprow_j0 == j0) return TOMO_OK;
    const Geometry& g = p->g;
    p->h_fprow.assign(g.h, -1);
    p->h_fpyf.assign(g.h, 0.0f);
    build_fp_rowmap(g, j0, p->h_fprow.data(), p->h_fpyf.data());
    CK(cudaMemcpyAsync(p->d_fprow, p->h_fprow.data(), sizeof(int) * g.h, cudaMemcpyHostToDevice, p->stream));
    CK(cudaMemcpyAsync(p->d_fpyf, p->h_fpyf.data(), sizeof(float) * g.h, cudaMemcpyHostToDevice, p->stream));
    p->fprow_j0 = j0;
    return TOMO_OK;
}

// Forward projection of the current batch, with the fused difference when meas is given.
tomo_status run_fp(tomo_projector* p, const int* d_tilts, int T, int y0, bool with_diff, double factor,
                   int slot0) {
    const Geometry& g = p->g;
    int j0, j1;
    fp_rows(p, y0, &j0, &j1);
    float* proj = p->d_proj + (size_t)slot0 * p->npix;
    float* norm = p->d_norm + (size_t)slot0 * p->npix;
    float* diff = p->d_diff + (size_t)slot0 * p->npix;
    double* errpart = p->d_errpart + (size_t)slot0 * g.h;
    if (j0 > 0) {
        // rows the reference leaves untouched stay zero (fresh FloatProcessors)
        for (int b = 0; b < T; b++) {
            CK(cudaMemsetAsync(proj + (size_t)b * p->npix, 0, sizeof(float) * (size_t)std::min(j0, g.h) * g.w,
                               p->stream));
            CK(cudaMemsetAsync(norm + (size_t)b * p->npix, 0, sizeof(float) * (size_t)std::min(j0, g.h) * g.w,
                               p->stream));
            if (with_diff)
                CK(cudaMemsetAsync(diff + (size_t)b * p->npix, 0, sizeof(float) * (size_t)std::min(j0, g.h) * g.w,
                                   p->stream));
        }
        if (with_diff) CK(cudaMemsetAsync(errpart, 0, sizeof(double) * (size_t)T * g.h, p->stream));
    }
    if (j0 >= j1) return TOMO_OK;
    if (!g.separable) {
        // any geometry: reference arithmetic per ray, then the difference pass
        FpGenericLaunch ga{};
        ga.vol = p->d_vol;
        ga.tilts = d_tilts;
        ga.T = T;
        ga.gtilt = p->d_gtilt;
        ga.proj = proj;
        ga.norm = norm;
        ga.j0 = j0;
        ga.j1 = j1;
        ga.W = g.W;
        ga.H = g.H;
        ga.D = g.D;
        ga.w = g.w;
        ga.h = g.h;
        ga.pc0x = g.pc[0];
        ga.pc0y = g.pc[1];
        ga.scale = g.scale;
        ga.vcx = g.vc[0];
        ga.vcy = g.vc[1];
        ga.vcz = g.vc[2];
        ga.bXmax = (double)((float)g.W + 1e-10f);  // int + float ACCURACY rounds to W (VoxelProjector3D.java:33)
        ga.bYmax = (double)((float)g.H + 1e-10f);
        ga.acc = (double)1e-10f;
        CK(launch_fp_generic(ga, p->stream));
        if (p->params.long_object) CK(launch_long_object(norm, T, g.h, g.w, p->stream));
        if (with_diff) {
            CK(launch_diff(p->d_meas, d_tilts, proj, norm, diff, errpart, T, g.w, g.h, j0, j1, factor, p->stream));
            CK(launch_reduce_err(errpart, p->d_err + slot0, T, g.h, p->stream));
        }
        return TOMO_OK;
    }
    FpLaunch a{};
    a.vol = p->vol();
    a.vtype = p->vtype;
    a.vscale = p->vtype == kVolF32 ? nullptr : p->d_vscale;
    a.meas = (with_diff && !p->params.long_object) ? p->d_meas : nullptr;
    a.tilts = d_tilts;
    a.T = T;
    a.ftilt = p->d_ftilt;
    a.rays = p->d_rays;
    a.proj = proj;
    a.norm = norm;
    a.diff = diff;
    a.errpart = errpart;
    a.factor = factor;
    a.j0 = j0;
    a.j1 = j1;
    a.tilts_per_cta = auto_tilts_per_cta(p, T, j1 - j0);
    a.zparts = fp_split(p, T, j1 - j0, a.tilts_per_cta);
    a.part = p->d_fppart;
    a.tickets = p->d_tickets;
    if (g.fractional) {
        CKS(ensure_fp_rowmap(p, j0));
        a.rowmap = p->d_fprow;
        a.rowyf = p->d_fpyf;
        a.two_rows = 1;
    }
    a.W = g.W;
    a.H = g.H;
    a.D = g.D;
    a.w = g.w;
    a.h = g.h;
    a.row_off = g.fp_row_off;
    a.status = p->d_status;
    a.hold_first_copy = p->hold_first_copy;
    CK(launch_fp_separable(a, p->stream));
    if (p->params.long_object) {
        CK(launch_long_object(norm, T, g.h, g.w, p->stream));
        if (with_diff)
            CK(launch_diff(p->d_meas, d_tilts, proj, norm, diff, errpart, T, g.w, g.h, j0, j1, factor, p->stream));
    }
    if (with_diff) CK(launch_reduce_err(errpart, p->d_err + slot0, T, g.h, p->stream));
    return TOMO_OK;
}

// Forward projection + difference of projection rows [j0, j1) only (separable FP32
// geometry), on p->stream, no depth split and no residual reduction: one row range
// of a row-stream iteration.
tomo_status run_fp_range(tomo_projector* p, const int* d_tilts, int T, int j0, int j1, double factor, int slot0) {
    const Geometry& g = p->g;
    if (j0 >= j1) return TOMO_OK;
    FpLaunch a{};
    a.vol = p->vol();
    a.vtype = p->vtype;
    a.meas = p->d_meas;
    a.tilts = d_tilts;
    a.T = T;
    a.ftilt = p->d_ftilt;
    a.rays = p->d_rays;
    a.proj = p->d_proj + (size_t)slot0 * p->npix;
    a.norm = p->d_norm + (size_t)slot0 * p->npix;
    a.diff = p->d_diff + (size_t)slot0 * p->npix;
    a.errpart = p->d_errpart + (size_t)slot0 * g.h;
    a.factor = factor;
    a.j0 = j0;
    a.j1 = j1;
    a.tilts_per_cta = auto_tilts_per_cta(p, T, j1 - j0);
    a.zparts = 1;
    a.W = g.W;
    a.H = g.H;
    a.D = g.D;
    a.w = g.w;
    a.h = g.h;
    a.row_off = g.fp_row_off;
    a.status = p->d_status;
    a.hold_first_copy = p->hold_first_copy;
    CK(launch_fp_separable(a, p->stream));
    return TOMO_OK;
}

tomo_status apply_weighting(tomo_projector* p, float* imgs, int T) {
    if (p->weight_kind == TOMO_WEIGHT_NONE || T <= 0) return TOMO_OK;
    const Geometry& g = p->g;
    if (p->weight2d) {
        for (int t0 = 0; t0 < T; t0 += p->w2chunk) {
            const int tc = std::min(p->w2chunk, T - t0);
            CK(launch_weighting_2d(imgs + (size_t)t0 * p->npix, tc, g.w, g.h, p->d_w2mask, p->w2pw, p->w2ph, p->d_w2a,
                                   p->d_w2b, p->stream));
        }
        return TOMO_OK;
    }
    // the row filter is the 2-D filter for a vertical axis, except that the 2-D
    // transform spreads a non-finite pixel over the whole image: flag such images
    for (int t0 = 0; t0 < T; t0 += p->imgbad_cap) {
        const int tc = std::min(p->imgbad_cap, T - t0);
        float* im = imgs + (size_t)t0 * p->npix;
        CK(launch_image_nonfinite(im, tc, p->npix, p->d_imgbad, p->stream));
        if (p->conv_M > 0)
            CK(launch_row_filter_conv(im, p->d_convH, p->d_convTw, tc * g.h, g.w, p->conv_M, p->d_imgbad, g.h,
                                      p->stream));
        else
            CK(launch_row_filter_tw(im, p->d_mask, p->d_tw, tc * g.h, g.w, p->d_imgbad, g.h, p->stream));
    }
    return TOMO_OK;
}

// Reduced storage: before a backprojection, rows whose scale is under the floor set by
// the volume's maximum get room to grow to that level (a row of tiny values next to rows
// of ordinary ones would otherwise leave FP16's range at the first update); row maxima
// are then rebuilt by the backprojection, and slabs whose maximum left the target band
// are re-scaled (no-op launches for most rows).
tomo_status bp_pre(tomo_projector* p, cudaStream_t s) {
    if (p->vtype == kVolF32) return TOMO_OK;
    CK(launch_vol_rescale(p->vol(), p->vtype, p->d_vscale, p->d_vmax, p->g.W, p->g.H, p->g.D, p->d_status, s));
    CK(cudaMemsetAsync(p->d_vmax, 0, sizeof(unsigned) * p->g.H, s));
    return TOMO_OK;
}

tomo_status bp_post(tomo_projector* p, cudaStream_t s) {
    if (p->vtype == kVolF32) return TOMO_OK;
    CK(launch_vol_rescale(p->vol(), p->vtype, p->d_vscale, p->d_vmax, p->g.W, p->g.H, p->g.D, p->d_status, s));
    return TOMO_OK;
}

// Backprojection of T images into volume rows [y0, y1).  `diffs`: the images are
// differences of an update, which a Bayesian handle adds to its distance volume.
tomo_status run_bp(tomo_projector* p, const float* imgs, const int* d_tilts, int T, int y0, int y1, bool sanitize,
                   bool diffs) {
    const Geometry& g = p->g;
    y0 = std::max(0, y0);
    y1 = std::min(g.H, y1);
    if (y1 <= y0 || T <= 0) return TOMO_OK;
    const bool to_dist = diffs && p->bayes;
    if (!g.separable || p->bp_generic) {
        BpGenericLaunch ga{};
        ga.vol = to_dist ? p->d_dist : p->d_vol;
        ga.img = imgs;
        ga.tilts = d_tilts;
        ga.T = T;
        ga.euler = p->d_euler;
        ga.y0 = y0;
        ga.y1 = y1;
        ga.W = g.W;
        ga.H = g.H;
        ga.D = g.D;
        ga.w = g.w;
        ga.h = g.h;
        ga.vc0 = g.vc[0];
        ga.vc1 = g.vc[1];
        ga.vc2 = g.vc[2];
        ga.cix = g.pc[2];
        ga.ciy = g.pc[3];
        ga.scale = g.scale;
        ga.positivity = p->params.positivity;
        CK(launch_bp_generic(ga, p->stream));
        return TOMO_OK;
    }
    BpLaunch a{};
    if (g.fractional) {
        a.bprow = p->d_bprow;
        a.bpyf = p->d_bpyf;
    }
    a.wide_seg = p->bp_wide;
    a.vol = to_dist ? p->bp_target() : p->vol();
    a.vtype = to_dist ? kVolF32 : p->vtype;
    a.vscale = p->d_vscale;
    a.vmax = p->d_vmax;
    a.img = imgs;
    a.tilts = d_tilts;
    a.T = T;
    a.btilt = p->d_btilt;
    a.zint = p->d_zint;
    a.y0 = y0;
    a.y1 = y1;
    a.W = g.W;
    a.H = g.H;
    a.D = g.D;
    a.w = g.w;
    a.h = g.h;
    a.row_off = g.bp_row_off;
    a.positivity = p->params.positivity;
    a.sanitize = sanitize || p->vol_flag();
    a.status = p->d_status;
    a.sms = p->sms;
    a.rows_mode = p->bp_rows;
    if (to_dist) {
        CK(launch_bp_separable(a, p->stream));
        return TOMO_OK;
    }
    CKS(bp_pre(p, p->stream));
    CK(launch_bp_separable(a, p->stream));
    CKS(bp_post(p, p->stream));
    return TOMO_OK;
}

tomo_status need_series(tomo_projector* p) {
    if (!p->series_loaded) return fail(TOMO_ERR_STATE, "no tilt-series loaded (tomo_load_series)");
    return TOMO_OK;
}

tomo_status tv_denoise(tomo_projector* p) {
    const Geometry& g = p->g;
    if (p->tv_iters <= 0) return TOMO_OK;
    // reduced storage: the step runs on an FP32 copy f and packs u back with fresh slab scales
    const bool red = p->vtype != kVolF32;
    float* f = red ? p->d_tv_f : p->d_vol;
    if (red) CK(launch_vol_unpack(p->vol(), p->vtype, p->d_vscale, g.H, 0, g.W, g.H, g.D, p->d_tv_f, p->stream));
    float* a[3] = {p->d_px, p->d_py, p->d_pz};
    float* b[3] = {p->d_qx, p->d_qy, p->d_qz};
    for (int it = 0; it < p->tv_iters; it++) {
        CK(launch_tv_step(f, a, b, it == 0, g.W, g.H, g.D, p->tv_theta, p->tv_g, p->tv_dt, p->stream));
        std::swap(a, b);
    }
    CK(launch_tv_final(f, a, g.W, g.H, g.D, p->tv_theta, p->stream));
    if (red) {
        CK(cudaMemsetAsync(p->d_vmax, 0, sizeof(unsigned) * g.H, p->stream));
        CK(launch_vol_rowmax(p->d_tv_f, g.H, 0, g.W, g.H, g.D, p->d_vmax, p->stream));
        // iteration-time pack: scales floored by the volume's maximum (a row the step
        // flattened keeps room for the next update)
        CK(launch_vol_pack(p->d_tv_f, g.H, 0, g.W, g.H, g.D, p->vtype, p->vol(), p->d_vscale, p->d_vmax, true,
                           p->d_status, p->stream));
    }
    return TOMO_OK;
}

tomo_status end_iteration(tomo_projector* p) {
    if (p->bayes)
        CK(launch_bayes_apply(p->d_vol, p->d_dist, p->nvox, p->bayes_alpha, p->params.positivity, p->stream));
    if (p->bgart)
        CK(launch_bgart_collapse(p->d_vol, p->nvox, p->bg_k, p->bg_dark, p->bg_value, p->d_bgscratch, p->stream));
    CKS(tv_denoise(p));
    if (p->cs) CK(launch_wavelet_filter(p->wav, p->d_vol, p->stream));
    if (p->fista) {
        const double t_1 = p->fista_t;
        p->fista_t = (1 + std::sqrt(1 + 4 * p->fista_t * p->fista_t)) / 2;
        const double factor = (t_1 - 1) / p->fista_t;
        CK(launch_fista(p->d_vol, p->d_prev, p->nvox, factor, p->stream));
    }
    return TOMO_OK;
}

tomo_status start_iteration(tomo_projector* p) {
    if (p->bgart && p->bg_median) CK(launch_bgart_median(p->d_vol, p->d_bgtmp, p->g.W, p->g.H, p->g.D, p->stream));
    if (p->bayes)
        CK(launch_bayes_conv(p->d_vol, p->d_dist, p->g.W, p->g.H, p->g.D, -p->bayes_lambda, p->stream));
    if (p->fista)
        CK(cudaMemcpyAsync(p->d_prev, p->d_vol, sizeof(float) * p->nvox, cudaMemcpyDeviceToDevice, p->stream));
    return TOMO_OK;
}

}  // namespace

namespace tomo {
// Buffers outside a handle (batch plans) from the same stream-ordered pool: no device-wide
// synchronisation when a plan grows while other streams run.
cudaError_t pool_malloc(void** ptr, size_t bytes) {
    DevicePool* d = device_pool();
    if (!d) return cudaMalloc(ptr, bytes);
    cudaError_t e = cudaMallocFromPoolAsync(ptr, bytes, d->pool, d->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
    return e;
}
void pool_free(void* ptr, cudaStream_t stream) { dfree(ptr, stream); }
tomo_status handle_fail(tomo_status code, const char* msg) { return fail(code, msg); }
tomo_status handle_need_series(tomo_projector* p) { return need_series(p); }
tomo_status handle_start_iteration(tomo_projector* p) { return start_iteration(p); }
tomo_status handle_end_iteration(tomo_projector* p) { return end_iteration(p); }
int handle_tilts_per_cta(const tomo_projector* p, int T) { return auto_tilts_per_cta(p, T, 0); }
}  // namespace tomo

extern "C" {

int32_t tomo_abi_version(void) { return TOMO_ABI_VERSION; }
const char* tomo_last_error(void) { return g_err.c_str(); }

tomo_status tomo_set_memory_limit(uint64_t bytes) {
    g_limit = bytes;
    return TOMO_OK;
}
uint64_t tomo_memory_in_use(void) { return g_in_use.load(); }
tomo_status tomo_device_memory(uint64_t* free_bytes, uint64_t* total_bytes) {
    if (!free_bytes || !total_bytes) return fail(TOMO_ERR_INVALID, "null argument");
    size_t f = 0, t = 0;
    CK(cudaMemGetInfo(&f, &t));
    *free_bytes = f + pool_idle_bytes(device_pool());  // idle blocks of the handles' pool are free to handles
    *total_bytes = t;
    return TOMO_OK;
}
uint64_t tomo_kernel_launches(void) { return g_launches.load(); }

tomo_status tomo_create(const tomo_geom* geom, const tomo_params* params, tomo_projector** out) {
    if (!geom || !out) return fail(TOMO_ERR_INVALID, "null argument");
    *out = nullptr;
    if (geom->W <= 0 || geom->H <= 0 || geom->D <= 0 || geom->w <= 0 || geom->h <= 0 || geom->nproj <= 0)
        return fail(TOMO_ERR_INVALID, "dimensions must be positive");
    if (geom->D > 65535 || geom->w > 4096 || geom->W > 65535)
        return fail(TOMO_ERR_UNSUPPORTED, "D <= 65535, W <= 65535 and w <= 4096 are supported");
    // the backprojector addresses a thread's 16 voxels with 32-bit offsets of k * H * W
    if ((uint64_t)geom->W * (uint64_t)geom->H * 16u >= (1ull << 32))
        return fail(TOMO_ERR_UNSUPPORTED, "W * H must be below 2^28");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(TOMO_ERR_CUDA, "no CUDA device");
    }
    tomo_projector* p = new tomo_projector();
    Geometry& g = p->g;
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
    if (params) p->params = *params;
    if (p->params.precision < TOMO_PREC_FP32 || p->params.precision > TOMO_PREC_FP16) {
        delete p;
        return fail(TOMO_ERR_INVALID, "precision must be TOMO_PREC_FP32, TOMO_PREC_BF16 or TOMO_PREC_FP16");
    }
    p->vtype = p->params.precision;  // TOMO_PREC_* values equal the storage types
    cudaGetDevice(&p->device);
    if (cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess) {
        cudaGetLastError();
        p->sms = 1;
    }
    p->npix = (size_t)g.w * g.h;
    p->nvox = (size_t)g.W * g.H * g.D;
    const size_t N = (size_t)g.N;
    tomo_status st = TOMO_OK;
    auto A = [&](tomo_status s) {
        if (st == TOMO_OK) st = s;
    };
    if (p->vtype == kVolF32) {
        A(alloc_n(p, &p->d_vol, p->nvox));
    } else {
        A(alloc_n(p, &p->d_vol16, p->nvox));
        A(alloc_n(p, &p->d_vscale, (size_t)g.H));
        A(alloc_n(p, &p->d_vmax, (size_t)g.H + 1));  // row maxima, then the volume's maximum
    }
    A(alloc_n(p, &p->d_raw, N * p->npix));
    A(alloc_n(p, &p->d_meas, N * p->npix));
    A(alloc_n(p, &p->d_proj, N * p->npix));
    A(alloc_n(p, &p->d_norm, N * p->npix));
    A(alloc_n(p, &p->d_diff, N * p->npix));
    A(alloc_n(p, &p->d_obatch, N * p->npix));
    A(alloc_n(p, &p->d_errpart, N * g.h));
    A(alloc_n(p, &p->d_err, N));
    A(alloc_n(p, &p->d_batch, N));
    A(alloc_n(p, &p->d_status, 1));
    A(alloc_n(p, &p->d_flags, 1));
    A(alloc_n(p, &p->d_ftilt, N));
    A(alloc_n(p, &p->d_rays, N * g.w));
    A(alloc_n(p, &p->d_btilt, N));
    A(alloc_n(p, &p->d_zint, N * g.W));
    A(alloc_n(p, &p->d_tinv, N * 6));
    A(alloc_n(p, &p->d_stats, N * 2));
    A(alloc_n(p, &p->d_identity, N));
    A(alloc_n(p, &p->d_mask, (size_t)g.w));
    A(alloc_n(p, &p->d_tw, (size_t)g.w));
    if (st == TOMO_OK) {
        if (cudaStreamCreateWithFlags(&p->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            st = fail(TOMO_ERR_CUDA, "cudaStreamCreate failed");
        }
    }
    if (st != TOMO_OK) {
        std::string msg = g_err;
        tomo_destroy(p);
        g_err = msg;
        return st;
    }
    p->stream = p->own_stream;
    if (fp_init_attributes() != cudaSuccess || misc_init_attributes() != cudaSuccess ||
        bp_init_attributes() != cudaSuccess) {
        tomo_destroy(p);
        return fail(TOMO_ERR_CUDA, "cannot configure kernel shared memory");
    }
    if (p->vtype == kVolF32) {
        cudaMemsetAsync(p->d_vol, 0, sizeof(float) * p->nvox, p->stream);
    } else {
        launch_vol_fill(p->d_vol16, p->vtype, p->d_vscale, p->d_vmax, p->nvox, g.H, 0.0f, p->stream);
    }
    cudaMemsetAsync(p->d_status, 0, sizeof(int), p->stream);
    cudaMemsetAsync(p->d_err, 0, sizeof(double) * N, p->stream);
    if (cudaStreamSynchronize(p->stream) != cudaSuccess) {
        tomo_destroy(p);
        return fail(TOMO_ERR_CUDA, "initialisation failed");
    }
    *out = p;
    return TOMO_OK;
}

tomo_status tomo_destroy(tomo_projector* p) {
    if (!p) return TOMO_OK;
    if (p->stream) cudaStreamSynchronize(p->stream);
    // handles sharing this volume keep it: the allocation passes to the first of them,
    // which becomes the owner of the others; a sharer leaves its owner
    if (!p->vol_sharers.empty()) {
        tomo_projector* q0 = p->vol_sharers.front();
        for (void*& a : p->allocs)
            if (a == static_cast<void*>(p->d_vol)) a = nullptr;
        q0->allocs.push_back(p->d_vol);
        p->bytes -= sizeof(float) * p->nvox;
        q0->bytes += sizeof(float) * p->nvox;
        q0->vol_owner = nullptr;
        q0->stream = q0->own_stream;
        q0->vol_nonfinite = p->vol_nonfinite;
        for (tomo_projector* q : p->vol_sharers) {
            if (q == q0) continue;
            q->vol_owner = q0;
            q->stream = q0->stream;
            q0->vol_sharers.push_back(q);
        }
        p->vol_sharers.clear();
        p->d_vol = nullptr;
    }
    if (p->vol_owner) {
        auto& v = p->vol_owner->vol_sharers;
        v.erase(std::remove(v.begin(), v.end(), p), v.end());
    }
    for (cudaEvent_t e : p->ev) cudaEventDestroy(e);
    {
        // the handle's stream is drained above; its row-stream work joins that stream
        DevicePool* d = device_pool();
        for (void* a : p->allocs) dfree(a, d ? d->stream : nullptr);
    }
    g_in_use -= p->bytes;
    for (cudaEvent_t e : p->rs_ev) cudaEventDestroy(e);
    for (cudaStream_t q : p->rs)
        if (q) cudaStreamDestroy(q);
    if (p->rs_reduce) cudaStreamDestroy(p->rs_reduce);
    if (p->own_stream) cudaStreamDestroy(p->own_stream);
    if (p->wav) wavelet_plan_destroy(p->wav);
    delete p;
    return TOMO_OK;
}

tomo_status tomo_set_priority(tomo_projector* p, int32_t priority) {
    if (!p || priority < 0) return fail(TOMO_ERR_INVALID, "bad argument");
    if (p->vol_owner) return fail(TOMO_ERR_STATE, "this handle works on another handle's volume");
    int least = 0, greatest = 0;  // numerically: least >= greatest, lower is more urgent
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    cudaStream_t s = nullptr;
    CK(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, std::max(greatest, least - priority)));
    CK(cudaStreamSynchronize(p->stream));
    const bool own = (p->stream == p->own_stream);
    cudaStreamDestroy(p->own_stream);
    p->own_stream = s;
    if (own) {
        p->stream = s;
        for (tomo_projector* q : p->vol_sharers) q->stream = s;
    }
    return TOMO_OK;
}

tomo_status tomo_set_stream(tomo_projector* p, void* stream) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (p->vol_owner)
        return fail(TOMO_ERR_STATE, "this handle works on another handle's volume: set the owner's stream");
    CK(cudaStreamSynchronize(p->stream));
    p->stream = stream ? static_cast<cudaStream_t>(stream) : p->own_stream;
    for (tomo_projector* q : p->vol_sharers) q->stream = p->stream;  // one volume, one stream
    return TOMO_OK;
}

// Geometry tables of the loaded Euler matrices and the handle's geometry (scale,
// centres): the kernel family (separable, fractional rows, generic) and its tables.
static tomo_status setup_geometry(tomo_projector* p) {
    Geometry& g = p->g;
    const int N = g.N;
    bool integral = true, vertical = true;
    for (int t = 0; t < N; t++) {
        integral = integral && tilt_is_separable(&p->euler[9 * t], g);
        vertical = vertical && tilt_is_vertical(&p->euler[9 * t]);
    }
    // vertical-axis tilts run on the XZ-plane kernels; rows that are not a whole row
    // apart (scale != 1, half-row centre offsets) blend two rows (16-bit volumes excepted)
    const bool sep = integral || (vertical && p->vtype == kVolF32);
    g.separable = sep;
    g.fractional = sep && !integral;
    if (g.fractional) {
        if (!p->d_fprow) {
            CKS(alloc_n(p, &p->d_fprow, (size_t)g.h));
            CKS(alloc_n(p, &p->d_fpyf, (size_t)g.h));
            CKS(alloc_n(p, &p->d_bprow, (size_t)g.H));
            CKS(alloc_n(p, &p->d_bpyf, (size_t)g.H));
        }
        std::vector<int> br(g.H);
        std::vector<float> by(g.H);
        build_bp_rowmap(g, br.data(), by.data());
        CK(cudaMemcpyAsync(p->d_bprow, br.data(), sizeof(int) * g.H, cudaMemcpyHostToDevice, p->stream));
        CK(cudaMemcpyAsync(p->d_bpyf, by.data(), sizeof(float) * g.H, cudaMemcpyHostToDevice, p->stream));
        CK(cudaStreamSynchronize(p->stream));
        p->fprow_j0 = -1;
    }
    // image columns one backprojection tile (64 x 64 voxels) may span for a tilt
    p->bp_wide = 0;
    p->bp_generic = false;
    if (sep) {
        double span = 0;
        for (int t = 0; t < N; t++) {
            const double* R = &p->euler[9 * t];
            span = std::max(span, (bp_tile_x() - 1) * std::fabs(R[0] * g.scale) +
                                      (bp_tile_z() - 1) * std::fabs(R[2] * g.scale) + 3.0);
        }
        if (span > bp_segment_pairs(true)) p->bp_generic = true;
        else if (span > bp_segment_pairs(false)) p->bp_wide = 1;
        if ((p->bp_generic || p->bp_wide) && p->vtype != kVolF32)
            return fail(TOMO_ERR_UNSUPPORTED, "16-bit volume storage needs scale 1");
    }
    if (sep) {
        g.fp_row_off = (int)(g.pc[1] - g.vc[1]);
        g.bp_row_off = (int)(g.pc[3] - g.vc[1]);
        std::vector<FpTilt> ft(N);
        std::vector<FpRay> rays((size_t)N * g.w);
        std::vector<BpTilt> bt(N);
        std::vector<int32_t> zint((size_t)N * g.W);
        // tilts are independent: their tables are built on the host threads
        parallel_ranges(N, 4, [&](int t0, int t1) {
            for (int t = t0; t < t1; t++) {
                build_fp_tables(g, &p->euler[9 * t], &ft[t], &rays[(size_t)t * g.w]);
                build_bp_tables(g, &p->euler[9 * t], &bt[t], &zint[(size_t)t * g.W]);
            }
        });
        CK(cudaMemcpyAsync(p->d_ftilt, ft.data(), sizeof(FpTilt) * N, cudaMemcpyHostToDevice, p->stream));
        CK(cudaMemcpyAsync(p->d_rays, rays.data(), sizeof(FpRay) * rays.size(), cudaMemcpyHostToDevice, p->stream));
        CK(cudaMemcpyAsync(p->d_btilt, bt.data(), sizeof(BpTilt) * N, cudaMemcpyHostToDevice, p->stream));
        CK(cudaMemcpyAsync(p->d_zint, zint.data(), sizeof(int32_t) * zint.size(), cudaMemcpyHostToDevice,
                           p->stream));
        CK(cudaStreamSynchronize(p->stream));
    }
    if (!sep || p->bp_generic) {
        if (p->vtype != kVolF32)
            return fail(TOMO_ERR_UNSUPPORTED,
                        "16-bit volume storage needs a vertical tilt axis, scale 1 and whole-row centre offsets");
        if (!p->d_gtilt) CKS(alloc_n(p, &p->d_gtilt, (size_t)N));
        if (!p->d_euler) CKS(alloc_n(p, &p->d_euler, (size_t)N * 9));
        std::vector<GenericFpTilt> gt(N);
        for (int t = 0; t < N; t++) build_generic_fp_tilt(&p->euler[9 * t], &gt[t]);
        CK(cudaMemcpyAsync(p->d_gtilt, gt.data(), sizeof(GenericFpTilt) * N, cudaMemcpyHostToDevice, p->stream));
        CK(cudaMemcpyAsync(p->d_euler, p->euler.data(), sizeof(double) * 9 * N, cudaMemcpyHostToDevice, p->stream));
        CK(cudaStreamSynchronize(p->stream));
    }
    return TOMO_OK;
}

tomo_status tomo_load_series(tomo_projector* p, const float* pixels, int32_t pixels_on_device, const double* euler,
                             const double* transforms, const double* stats) {
    if (!p || !pixels || !euler) return fail(TOMO_ERR_INVALID, "null argument");
    Geometry& g = p->g;
    const int N = g.N;
    CK(cudaMemcpyAsync(p->d_raw, pixels, sizeof(float) * N * p->npix,
                       pixels_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, p->stream));
    p->euler.assign(euler, euler + 9 * (size_t)N);
    CKS(setup_geometry(p));
    // alignment: Tinv = AffineTransform.createInverse (general case)
    std::vector<double> tinv((size_t)N * 6), st((size_t)N * 2);
    std::vector<unsigned char> ident(N);
    for (int t = 0; t < N; t++) {
        double T[6] = {1, 0, 0, 1, 0, 0};
        if (transforms) std::memcpy(T, transforms + 6 * t, sizeof(T));
        ident[t] = (T[0] == 1.0 && T[1] == 0.0 && T[2] == 0.0 && T[3] == 1.0 && T[4] == 0.0 && T[5] == 0.0);
        const double m00 = T[0], m10 = T[1], m01 = T[2], m11 = T[3], m02 = T[4], m12 = T[5];
        const double det = m00 * m11 - m01 * m10;
        if (!ident[t] && !(std::fabs(det) > 4.9e-324))
            return fail(TOMO_ERR_INVALID, "transform " + std::to_string(t) + " is not invertible");
        double* I = &tinv[6 * (size_t)t];
        I[0] = m11 / det;
        I[1] = -m10 / det;
        I[2] = -m01 / det;
        I[3] = m00 / det;
        I[4] = (m01 * m12 - m11 * m02) / det;
        I[5] = (m10 * m02 - m00 * m12) / det;
        st[2 * t] = stats ? stats[2 * t] : 0.0;
        st[2 * t + 1] = stats ? stats[2 * t + 1] : 1.0;
    }
    CK(cudaMemcpyAsync(p->d_tinv, tinv.data(), sizeof(double) * tinv.size(), cudaMemcpyHostToDevice, p->stream));
    CK(cudaMemcpyAsync(p->d_stats, st.data(), sizeof(double) * st.size(), cudaMemcpyHostToDevice, p->stream));
    CK(cudaMemcpyAsync(p->d_identity, ident.data(), N, cudaMemcpyHostToDevice, p->stream));
    CK(launch_align(p->d_raw, p->d_meas, p->d_tinv, p->d_stats, N, g.w, g.h, p->params.normalize, p->params.fill,
                    p->d_identity, p->stream));
    int flags = 0;
    CK(cudaMemsetAsync(p->d_flags, 0, sizeof(int), p->stream));
    CK(launch_scan_nonfinite(p->d_meas, (size_t)N * p->npix, p->d_flags, p->stream));
    CK(cudaMemcpyAsync(&flags, p->d_flags, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    p->meas_has_nan = (flags & 1) != 0;
    p->meas_has_inf = (flags & 2) != 0;
    p->series_loaded = true;
    p->batch.clear();
    p->batch_uploaded = false;
    p->diffs_valid = p->projected = p->obatch_valid = false;
    return TOMO_OK;
}

tomo_status tomo_set_row_streams(tomo_projector* p, int32_t k) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (k < 1 || k > 4) return fail(TOMO_ERR_INVALID, "1 to 4 row streams");
    for (int i = 1; i < k; i++)
        if (!p->rs[i]) CK(cudaStreamCreateWithFlags(&p->rs[i], cudaStreamNonBlocking));
    if (k > 1 && !p->rs[0]) CK(cudaStreamCreateWithFlags(&p->rs[0], cudaStreamNonBlocking));
    if (k > 1 && !p->rs_reduce) CK(cudaStreamCreateWithFlags(&p->rs_reduce, cudaStreamNonBlocking));
    p->row_streams = k;
    return TOMO_OK;
}

tomo_status tomo_set_positivity(tomo_projector* p, int32_t enabled) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    p->params.positivity = enabled ? 1 : 0;
    return TOMO_OK;
}

tomo_status tomo_set_long_object(tomo_projector* p, int32_t enabled) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    p->params.long_object = enabled ? 1 : 0;
    return TOMO_OK;
}

tomo_status tomo_set_scale(tomo_projector* p, double scale) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (!(scale > 0) || !std::isfinite(scale)) return fail(TOMO_ERR_INVALID, "scale must be positive");
    const double old = p->g.scale;
    p->g.scale = scale;
    if (!p->series_loaded) return TOMO_OK;
    const tomo_status st = setup_geometry(p);
    if (st != TOMO_OK) {
        const std::string why = tomo_last_error();
        p->g.scale = old;
        setup_geometry(p);
        return fail(st, why);
    }
    p->fprow_j0 = -1;
    p->diffs_valid = p->projected = false;
    return TOMO_OK;
}

tomo_status tomo_set_centers(tomo_projector* p, const double* vol_center, const double* proj_center) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    Geometry& g = p->g;
    double vc[3], pc[4];
    std::memcpy(vc, g.vc, sizeof(vc));
    std::memcpy(pc, g.pc, sizeof(pc));
    for (int k = 0; k < 3; k++)
        if (vol_center && !std::isnan(vol_center[k])) g.vc[k] = vol_center[k];
    for (int k = 0; k < 4; k++)
        if (proj_center && !std::isnan(proj_center[k])) g.pc[k] = proj_center[k];
    if (!p->series_loaded) return TOMO_OK;
    const tomo_status st = setup_geometry(p);
    if (st != TOMO_OK) {
        const std::string why = tomo_last_error();
        std::memcpy(g.vc, vc, sizeof(vc));
        std::memcpy(g.pc, pc, sizeof(pc));
        setup_geometry(p);
        return fail(st, why);
    }
    p->fprow_j0 = -1;
    p->diffs_valid = p->projected = false;
    return TOMO_OK;
}

tomo_status tomo_set_fill(tomo_projector* p, int32_t fill) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (fill < TOMO_FILL_NONE || fill > TOMO_FILL_NAN) return fail(TOMO_ERR_INVALID, "unknown fill type");
    p->params.fill = fill;
    if (!p->series_loaded) return TOMO_OK;
    const Geometry& g = p->g;
    CK(launch_align(p->d_raw, p->d_meas, p->d_tinv, p->d_stats, g.N, g.w, g.h, p->params.normalize, fill,
                    p->d_identity, p->stream));
    int flags = 0;
    CK(cudaMemsetAsync(p->d_flags, 0, sizeof(int), p->stream));
    CK(launch_scan_nonfinite(p->d_meas, (size_t)g.N * p->npix, p->d_flags, p->stream));
    CK(cudaMemcpyAsync(&flags, p->d_flags, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    p->meas_has_nan = (flags & 1) != 0;
    p->meas_has_inf = (flags & 2) != 0;
    p->obatch_valid = false;
    return TOMO_OK;
}

tomo_status tomo_get_aligned(tomo_projector* p, int32_t index, float* out_host) {
    if (!p || !out_host) return fail(TOMO_ERR_INVALID, "null argument");
    if (!p->series_loaded) return fail(TOMO_ERR_STATE, "no tilt-series loaded");
    if (index < 0 || index >= p->g.N) return fail(TOMO_ERR_INVALID, "index out of range");
    CK(cudaMemcpyAsync(out_host, p->d_meas + (size_t)index * p->npix, sizeof(float) * p->npix,
                       cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    return TOMO_OK;
}

// FP32 staging of a reduced volume: enough rows for about 64 MB (at least one row).
static tomo_status ensure_vtmp(tomo_projector* p, size_t* rows_out) {
    const Geometry& g = p->g;
    const size_t row_bytes = sizeof(float) * (size_t)g.W * g.D;
    size_t rows = std::max<size_t>(1, ((size_t)64 << 20) / row_bytes);
    rows = std::min<size_t>(rows, (size_t)g.H);
    if (!p->d_vtmp) {
        CKS(alloc_n(p, &p->d_vtmp, rows * (size_t)g.W * g.D));
        p->vtmp_rows = rows;
    }
    *rows_out = p->vtmp_rows;
    return TOMO_OK;
}

static tomo_status volume_copy(tomo_projector* p, float* host_or_dev, int on_device, int y0, int y1, bool to_dev) {
    const Geometry& g = p->g;
    if (y0 < 0 || y1 > g.H || y1 < y0) return fail(TOMO_ERR_INVALID, "row range outside the volume");
    if (y1 == y0) return TOMO_OK;
    const size_t rows = (size_t)(y1 - y0);
    // [D][rows][W] <-> [D][H][W] rows y0..y1 of every slice
    cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice
                                    : (to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost);
    if (p->vtype == kVolF32) {
        float* dev = p->d_vol + (size_t)y0 * g.W;
        if (to_dev)
            CK(cudaMemcpy2DAsync(dev, sizeof(float) * g.W * g.H, host_or_dev, sizeof(float) * g.W * rows,
                                 sizeof(float) * g.W * rows, g.D, kind, p->stream));
        else
            CK(cudaMemcpy2DAsync(host_or_dev, sizeof(float) * g.W * rows, dev, sizeof(float) * g.W * g.H,
                                 sizeof(float) * g.W * rows, g.D, kind, p->stream));
        CK(cudaStreamSynchronize(p->stream));
        return TOMO_OK;
    }
    // reduced storage: blocks of rows through the FP32 staging buffer
    size_t cap = 0;
    CKS(ensure_vtmp(p, &cap));
    // a whole new volume: the old row maxima must not count towards its maximum
    if (to_dev && rows == (size_t)g.H) CK(cudaMemsetAsync(p->d_vmax, 0, sizeof(unsigned) * g.H, p->stream));
    kind = on_device ? cudaMemcpyDeviceToDevice : (to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost);
    for (size_t a = 0; a < rows; a += cap) {
        const size_t n = std::min(cap, rows - a);
        float* user = host_or_dev + a * g.W;  // row a of the caller's [D][rows][W] buffer
        const int r0 = y0 + (int)a;
        if (to_dev) {
            CK(cudaMemcpy2DAsync(p->d_vtmp, sizeof(float) * g.W * n, user, sizeof(float) * g.W * rows,
                                 sizeof(float) * g.W * n, g.D, kind, p->stream));
            CK(cudaMemsetAsync(p->d_vmax + r0, 0, sizeof(unsigned) * n, p->stream));
            CK(launch_vol_rowmax(p->d_vtmp, (int)n, r0, g.W, g.H, g.D, p->d_vmax, p->stream));
            CK(launch_vol_pack(p->d_vtmp, (int)n, r0, g.W, g.H, g.D, p->vtype, p->vol(), p->d_vscale, p->d_vmax, false,
                               p->d_status, p->stream));
        } else {
            CK(launch_vol_unpack(p->vol(), p->vtype, p->d_vscale, (int)n, r0, g.W, g.H, g.D, p->d_vtmp, p->stream));
            CK(cudaMemcpy2DAsync(user, sizeof(float) * g.W * rows, p->d_vtmp, sizeof(float) * g.W * n,
                                 sizeof(float) * g.W * n, g.D, kind, p->stream));
        }
        // the staging buffer is reused by the next block
        CK(cudaStreamSynchronize(p->stream));
    }
    return to_dev ? check_status(p) : TOMO_OK;
}

tomo_status tomo_set_volume(tomo_projector* p, const float* src, int32_t on_device, int32_t y0, int32_t y1) {
    if (!p || !src) return fail(TOMO_ERR_INVALID, "null argument");
    CKS(volume_copy(p, const_cast<float*>(src), on_device, y0, y1, true));
    int flags = 0;
    CK(cudaMemsetAsync(p->d_flags, 0, sizeof(int), p->stream));
    CK(launch_scan_nonfinite_vol(p->vol(), p->vtype, p->nvox, p->d_flags, p->stream));
    CK(cudaMemcpyAsync(&flags, p->d_flags, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    p->vol_flag() = flags != 0;
    return TOMO_OK;
}

tomo_status tomo_get_volume(tomo_projector* p, float* dst, int32_t on_device, int32_t y0, int32_t y1) {
    if (!p || !dst) return fail(TOMO_ERR_INVALID, "null argument");
    return volume_copy(p, dst, on_device, y0, y1, false);
}

tomo_status tomo_fill_volume(tomo_projector* p, float value) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (p->vtype == kVolF32)
        CK(launch_fill(p->d_vol, p->nvox, value, p->stream));
    else
        CK(launch_vol_fill(p->vol(), p->vtype, p->d_vscale, p->d_vmax, p->nvox, p->g.H, value, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    p->vol_flag() = !std::isfinite(value);
    return TOMO_OK;
}

tomo_status tomo_volume_device_ptr(tomo_projector* p, float** out) {
    if (!p || !out) return fail(TOMO_ERR_INVALID, "null argument");
    if (p->vtype != kVolF32)
        return fail(TOMO_ERR_UNSUPPORTED, "the volume is stored in 16 bits with slab scales; use tomo_get_volume");
    *out = p->d_vol;
    return TOMO_OK;
}

tomo_status tomo_share_volume(tomo_projector* p, tomo_projector* owner) {
    if (!p || p == owner) return fail(TOMO_ERR_INVALID, "null or self handle");
    if (p->vtype != kVolF32 || (owner && owner->vtype != kVolF32))
        return fail(TOMO_ERR_UNSUPPORTED, "volume sharing needs FP32 storage");
    if (!owner) {
        if (!p->vol_owner) return TOMO_OK;  // already private
        float* mine = nullptr;
        CKS(alloc_n(p, &mine, p->nvox));
        CK(cudaMemcpyAsync(mine, p->d_vol, sizeof(float) * p->nvox, cudaMemcpyDeviceToDevice, p->stream));
        CK(cudaStreamSynchronize(p->stream));
        p->vol_nonfinite = p->vol_flag();
        auto& v = p->vol_owner->vol_sharers;
        v.erase(std::remove(v.begin(), v.end(), p), v.end());
        p->d_vol = mine;
        p->vol_owner = nullptr;
        p->stream = p->own_stream;
        return TOMO_OK;
    }
    if (owner->vol_owner) return fail(TOMO_ERR_INVALID, "the owner shares another handle's volume");
    if (!p->vol_sharers.empty()) return fail(TOMO_ERR_INVALID, "other handles share this handle's volume");
    if (p->vol_owner == owner) return TOMO_OK;
    if (p->vol_owner) CKS(tomo_share_volume(p, nullptr));
    if (p->g.W != owner->g.W || p->g.H != owner->g.H || p->g.D != owner->g.D)
        return fail(TOMO_ERR_INVALID, "volume sizes differ");
    CK(cudaStreamSynchronize(p->stream));
    CK(cudaStreamSynchronize(owner->stream));
    if (!p->vol_owner) free_n(p, &p->d_vol, p->nvox);
    p->d_vol = owner->d_vol;
    p->vol_owner = owner;
    p->stream = owner->stream;
    owner->vol_sharers.push_back(p);
    return TOMO_OK;
}

tomo_status tomo_add_projection(tomo_projector* p, int32_t index) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (!p->series_loaded) return fail(TOMO_ERR_STATE, "no tilt-series loaded");
    if (index < 0 || index >= p->g.N) return fail(TOMO_ERR_INVALID, "projection index out of range");
    if ((int)p->batch.size() >= p->g.N) return fail(TOMO_ERR_INVALID, "more projections added than slots");
    p->batch.push_back(index);
    p->batch_uploaded = false;
    p->obatch_valid = false;
    return TOMO_OK;
}

tomo_status tomo_clear_projections(tomo_projector* p) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    p->batch.clear();
    p->batch_uploaded = false;
    p->diffs_valid = p->projected = p->obatch_valid = false;
    return TOMO_OK;
}

int32_t tomo_projection_count(tomo_projector* p) { return p ? (int32_t)p->batch.size() : 0; }

tomo_status tomo_project(tomo_projector* p, int32_t y0, int32_t y1) {
    (void)y1;
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    CKS(need_series(p));
    CKS(upload_batch(p));
    CKS(run_fp(p, p->d_batch, (int)p->batch.size(), y0, false, 0.0, 0));
    CKS(check_status(p));
    p->projected = true;
    p->diffs_valid = false;
    return TOMO_OK;
}

tomo_status tomo_project_and_difference(tomo_projector* p, double factor, int32_t y0, int32_t y1, double* err_out) {
    (void)y1;
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    CKS(need_series(p));
    CKS(upload_batch(p));
    const int T = (int)p->batch.size();
    CKS(run_fp(p, p->d_batch, T, y0, true, factor, 0));
    if (err_out && T > 0)
        CK(cudaMemcpyAsync(err_out, p->d_err, sizeof(double) * T, cudaMemcpyDeviceToHost, p->stream));
    CKS(check_status(p));
    p->projected = true;
    p->diffs_valid = true;
    return TOMO_OK;
}

tomo_status tomo_backproject(tomo_projector* p, int32_t y0, int32_t y1) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    CKS(need_series(p));
    CKS(upload_batch(p));
    const int T = (int)p->batch.size();
    if (T == 0) return TOMO_OK;
    const float* imgs;
    bool sanitize;
    // BayesianVoxelProjector3D.backproject only acts on differences (:77-116)
    if (p->bayes && !p->diffs_valid) return TOMO_OK;
    if (p->diffs_valid) {
        CKS(apply_weighting(p, p->d_diff, T));
        imgs = p->d_diff;
        sanitize = p->meas_has_inf;
    } else {
        if (!p->obatch_valid) {
            CK(launch_gather(p->d_obatch, p->d_meas, p->d_batch, T, p->npix, p->stream));
            p->obatch_valid = true;
        }
        CKS(apply_weighting(p, p->d_obatch, T));
        imgs = p->d_obatch;
        sanitize = p->meas_has_nan || p->meas_has_inf;
    }
    CKS(run_bp(p, imgs, p->d_batch, T, y0, y1, sanitize, p->diffs_valid));
    CKS(check_status(p));
    return TOMO_OK;
}

tomo_status tomo_start_iteration(tomo_projector* p) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    CKS(start_iteration(p));
    return TOMO_OK;
}

tomo_status tomo_end_iteration(tomo_projector* p) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    CKS(end_iteration(p));
    CK(cudaStreamSynchronize(p->stream));
    return TOMO_OK;
}

static tomo_status get_slot(tomo_projector* p, const float* base, int32_t k, float* out, bool need) {
    if (!p || !out) return fail(TOMO_ERR_INVALID, "null argument");
    if (!need) return fail(TOMO_ERR_STATE, "nothing projected for the current projections");
    if (k < 0 || k >= (int)p->batch.size()) return fail(TOMO_ERR_INVALID, "projection slot out of range");
    CK(cudaMemcpyAsync(out, base + (size_t)k * p->npix, sizeof(float) * p->npix, cudaMemcpyDeviceToHost,
                       p->stream));
    CK(cudaStreamSynchronize(p->stream));
    return TOMO_OK;
}

tomo_status tomo_get_projection(tomo_projector* p, int32_t k, float* out_host) {
    return get_slot(p, p ? p->d_proj : nullptr, k, out_host, p && p->projected);
}
tomo_status tomo_get_norm(tomo_projector* p, int32_t k, float* out_host) {
    return get_slot(p, p ? p->d_norm : nullptr, k, out_host, p && p->projected);
}
tomo_status tomo_get_difference(tomo_projector* p, int32_t k, float* out_host) {
    return get_slot(p, p ? p->d_diff : nullptr, k, out_host, p && p->diffs_valid);
}

// FFTWeighting(ts, diameter) (FFTWeighting.java:22-24, 31-81): the mask reads
// ts.getTiltAngle(i) and ts.getTiltAxis(i).
tomo_status set_weighting_2d(tomo_projector* p, double diameter, const std::vector<double>& deg,
                             const double* tilt_axes) {
    const Geometry& g = p->g;
    if (g.w > kDft2MaxN || g.h > kDft2MaxN)
        return fail(TOMO_ERR_UNSUPPORTED, "2-D weighting supports projections up to 4096 x 4096");
    const int Mw = dft_grid_size(g.w), Mh = dft_grid_size(g.h);
    const size_t tw_n = (size_t)g.w + 2 * (size_t)Mw, th_n = (size_t)g.h + 2 * (size_t)Mh;
    std::vector<float2> tab(tw_n + th_n);
    dft_row_tables(g.w, Mw, tab.data(), tab.data() + g.w, tab.data() + g.w + Mw);
    dft_row_tables(g.h, Mh, tab.data() + tw_n, tab.data() + tw_n + g.h, tab.data() + tw_n + g.h + Mh);
    std::vector<float> maskT(p->npix);
    weighting_mask_2d(g.w, g.h, g.N, deg.data(), tilt_axes, diameter, maskT.data());
    // scratch for up to 2^24 complex values per buffer (256 MB for both)
    const int want = (int)std::max<size_t>(1, std::min<size_t>({(size_t)g.N, 65535, ((size_t)1 << 24) / p->npix}));
    if (!p->d_w2mask) {
        CKS(alloc_n(p, &p->d_w2mask, p->npix));
        CKS(alloc_n(p, &p->d_w2tab, tab.size()));
    }
    if (p->w2chunk < want) {
        free_n(p, &p->d_w2a, (size_t)p->w2chunk * p->npix);
        free_n(p, &p->d_w2b, (size_t)p->w2chunk * p->npix);
        p->w2chunk = 0;
        CKS(alloc_n(p, &p->d_w2a, (size_t)want * p->npix));
        CKS(alloc_n(p, &p->d_w2b, (size_t)want * p->npix));
        p->w2chunk = want;
    }
    CK(cudaMemcpyAsync(p->d_w2mask, maskT.data(), sizeof(float) * p->npix, cudaMemcpyHostToDevice, p->stream));
    CK(cudaMemcpyAsync(p->d_w2tab, tab.data(), sizeof(float2) * tab.size(), cudaMemcpyHostToDevice, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    auto plan = [](int n, int M, const float2* base) {
        DftRowPlan P;
        P.n = n;
        P.M = M;
        P.logM = 0;
        while ((1 << P.logM) < M) P.logM++;
        P.chirp = base;
        P.bspec = base + n;
        P.tw = base + n + M;
        return P;
    };
    p->w2pw = plan(g.w, Mw, p->d_w2tab);
    p->w2ph = plan(g.h, Mh, p->d_w2tab + tw_n);
    p->weight2d = true;
    return TOMO_OK;
}

tomo_status tomo_set_weighting(tomo_projector* p, int32_t kind, double radius, const double* tilt_deg,
                               const double* tilt_axes) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (kind < TOMO_WEIGHT_NONE || kind > TOMO_WEIGHT_HAMMING_RAMP) return fail(TOMO_ERR_INVALID, "unknown filter");
    if (kind == TOMO_WEIGHT_NONE) {
        p->weight_kind = kind;
        return TOMO_OK;
    }
    if (!p->series_loaded) return fail(TOMO_ERR_STATE, "load the tilt-series before setting the weighting");
    const Geometry& g = p->g;
    bool tilted = false;
    if (tilt_axes)
        for (int t = 0; t < g.N; t++) tilted = tilted || tilt_axes[t] != 0.0;
    if (tilted && kind != TOMO_WEIGHT_RADERMACHER)
        return fail(TOMO_ERR_UNSUPPORTED, "ramp filters need a zero tilt-axis angle");
    if (kind == TOMO_WEIGHT_RADERMACHER && !(radius > 0))
        return fail(TOMO_ERR_INVALID, "Radermacher weighting needs a positive radius");
    std::vector<double> sint(g.N), deg(g.N);
    for (int t = 0; t < g.N; t++) {
        if (tilt_deg) {
            deg[t] = tilt_deg[t];
            sint[t] = std::sin(tilt_deg[t] * (M_PI / 180.0));
        } else {
            sint[t] = p->euler[9 * t + 6];  // eulerAngles2Matrix(0, theta, 0) row 2 = (sin(theta), 0, cos(theta))
            deg[t] = std::atan2(p->euler[9 * t + 6], p->euler[9 * t + 8]) * (180.0 / M_PI);
        }
    }
    if (tilted) {
        CKS(set_weighting_2d(p, radius * g.w, deg, tilt_axes));
        p->weight_kind = kind;
        return TOMO_OK;
    }
    p->weight2d = false;
    if (p->imgbad_cap < g.N) {
        free_n(p, &p->d_imgbad, (size_t)p->imgbad_cap);
        p->imgbad_cap = 0;
        CKS(alloc_n(p, &p->d_imgbad, (size_t)g.N));
        p->imgbad_cap = g.N;
    }
    std::vector<float> mask(g.w);
    weighting_row_filter(kind, g.w, g.N, sint.data(), deg.data(), radius * g.w, mask.data());
    if ((g.w & (g.w - 1)) != 0) {
        // any width: circular convolution with h = IDFT_w(mask) through an M-point FFT
        int M = 1;
        while (M < 2 * g.w - 1) M <<= 1;
        if (M > kRowConvMaxM) return fail(TOMO_ERR_UNSUPPORTED, "weighting supports widths up to 4096");
        std::vector<float2> H(M), twm(M);
        row_filter_spectrum(mask.data(), g.w, M, H.data());
        for (int k = 0; k < M; k++) {
            const double a = -2.0 * M_PI * k / M;
            twm[k] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        if (p->conv_M < M) {
            CKS(alloc_n(p, &p->d_convH, (size_t)M));
            CKS(alloc_n(p, &p->d_convTw, (size_t)M));
        }
        CK(cudaMemcpyAsync(p->d_convH, H.data(), sizeof(float2) * M, cudaMemcpyHostToDevice, p->stream));
        CK(cudaMemcpyAsync(p->d_convTw, twm.data(), sizeof(float2) * M, cudaMemcpyHostToDevice, p->stream));
        CK(cudaStreamSynchronize(p->stream));
        p->conv_M = M;
        p->weight_kind = kind;
        return TOMO_OK;
    }
    std::vector<float2> tw(g.w);
    for (int k = 0; k < g.w; k++) {
        const double a = -2.0 * M_PI * k / g.w;
        tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    CK(cudaMemcpyAsync(p->d_mask, mask.data(), sizeof(float) * g.w, cudaMemcpyHostToDevice, p->stream));
    CK(cudaMemcpyAsync(p->d_tw, tw.data(), sizeof(float2) * g.w, cudaMemcpyHostToDevice, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    p->weight_kind = kind;
    return TOMO_OK;
}

tomo_status tomo_set_tvm(tomo_projector* p, float theta, float g, float dt, int32_t iterations) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (iterations < 0) return fail(TOMO_ERR_INVALID, "negative iteration count");
    if (iterations > 0 && !p->d_px) {
        CKS(alloc_n(p, &p->d_px, p->nvox));
        CKS(alloc_n(p, &p->d_py, p->nvox));
        CKS(alloc_n(p, &p->d_pz, p->nvox));
        CKS(alloc_n(p, &p->d_qx, p->nvox));
        CKS(alloc_n(p, &p->d_qy, p->nvox));
        CKS(alloc_n(p, &p->d_qz, p->nvox));
    }
    if (iterations > 0 && p->vtype != kVolF32 && !p->d_tv_f) CKS(alloc_n(p, &p->d_tv_f, p->nvox));
    p->tv_theta = theta;
    p->tv_g = g;
    p->tv_dt = dt;
    p->tv_iters = iterations;
    return TOMO_OK;
}

tomo_status tomo_set_fista(tomo_projector* p, int32_t enabled) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (enabled && p->vtype != kVolF32)
        return fail(TOMO_ERR_UNSUPPORTED, "FISTA momentum needs the FP32 volume (precision TOMO_PREC_FP32)");
    if (enabled && !p->d_prev) CKS(alloc_n(p, &p->d_prev, p->nvox));
    p->fista = enabled != 0;
    p->fista_t = 0.0;
    return TOMO_OK;
}

tomo_status tomo_set_bayesian(tomo_projector* p, double lambda, double alpha, int32_t enabled) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (enabled && p->vtype != kVolF32)
        return fail(TOMO_ERR_UNSUPPORTED, "the Bayesian regulariser needs the FP32 volume (precision TOMO_PREC_FP32)");
    if (enabled && !p->d_dist) CKS(alloc_n(p, &p->d_dist, p->nvox));
    p->bayes = enabled != 0;
    p->bayes_lambda = lambda;
    p->bayes_alpha = alpha;
    return TOMO_OK;
}

tomo_status tomo_set_bgart(tomo_projector* p, double k, int32_t dark_bg, int32_t do_median, double bg_value,
                           int32_t enabled) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (enabled && p->vtype != kVolF32)
        return fail(TOMO_ERR_UNSUPPORTED, "the BgART filters need the FP32 volume (precision TOMO_PREC_FP32)");
    if (enabled && !p->d_bgscratch) CKS(dalloc(p, &p->d_bgscratch, kBgScratchBytes));
    if (enabled && do_median && !p->d_bgtmp) CKS(alloc_n(p, &p->d_bgtmp, p->nvox));
    p->bgart = enabled != 0;
    p->bg_k = k;
    p->bg_dark = dark_bg != 0;
    p->bg_median = do_median != 0;
    p->bg_value = bg_value;
    if (p->bgart) {
        // the reference's constructor collapses the starting volume once (BgARTVoxelProjector3D.java:22-27)
        CK(launch_bgart_collapse(p->d_vol, p->nvox, k, p->bg_dark, bg_value, p->d_bgscratch, p->stream));
        CK(cudaStreamSynchronize(p->stream));
    }
    return TOMO_OK;
}

tomo_status tomo_set_compressed_sensing(tomo_projector* p, int32_t wavelet_type, double degree, double shift,
                                       double fraction_zeros, const int32_t* levels, int32_t enabled) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    if (!enabled) {
        p->cs = false;
        return TOMO_OK;
    }
    if (p->vtype != kVolF32)
        return fail(TOMO_ERR_UNSUPPORTED, "the wavelet filter needs the FP32 volume (precision TOMO_PREC_FP32)");
    const Geometry& g = p->g;
    int it[3];
    if (levels) {
        for (int a = 0; a < 3; a++) it[a] = levels[a];
    } else {
        // findBestWaveletsIteration (CompressedSensingProjector.java:127-151): every axis
        // from the width
        int n = 1;
        for (long long s = 64; s < g.W; s *= 2) n++;
        it[0] = it[1] = it[2] = n;
    }
    const char* why = nullptr;
    WaveletPlan* plan = wavelet_plan_create(g.W, g.H, g.D, it, wavelet_type, degree, shift, fraction_zeros, &why);
    if (!plan) {
        const bool sizes = std::strstr(why, "levels") != nullptr;
        return fail(sizes ? TOMO_ERR_UNSUPPORTED : TOMO_ERR_INVALID, why);
    }
    CK(cudaStreamSynchronize(p->stream));
    const size_t tb = wavelet_plan_table_bytes(plan);
    tomo_status st = TOMO_OK;
    if (!p->d_wbuf) st = alloc_n(p, &p->d_wbuf, p->nvox);
    if (st == TOMO_OK && !p->d_wstate) st = dalloc(p, &p->d_wstate, wavelet_plan_state_bytes());
    if (st == TOMO_OK && p->d_wtab && p->wtab_bytes < tb) free_n(p, reinterpret_cast<char**>(&p->d_wtab), p->wtab_bytes);
    if (st == TOMO_OK && !p->d_wtab) {
        st = dalloc(p, &p->d_wtab, tb);
        if (st == TOMO_OK) p->wtab_bytes = tb;
    }
    if (st != TOMO_OK) {
        wavelet_plan_destroy(plan);
        return st;
    }
    cudaError_t e = wavelet_plan_bind(plan, p->d_wtab, p->d_wbuf, p->d_wstate, p->stream);
    if (e != cudaSuccess) {
        wavelet_plan_destroy(plan);
        CK(e);
    }
    if (p->wav) wavelet_plan_destroy(p->wav);
    p->wav = plan;
    p->cs = true;
    return TOMO_OK;
}

tomo_status tomo_compressed_sensing_threshold(tomo_projector* p, double* out) {
    if (!p || !out) return fail(TOMO_ERR_INVALID, "null argument");
    if (!p->wav) return fail(TOMO_ERR_STATE, "no wavelet filter set (tomo_set_compressed_sensing)");
    CK(wavelet_read_threshold(p->wav, out, p->stream));
    return TOMO_OK;
}

tomo_status tomo_set_profiling(tomo_projector* p, int32_t enabled) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    p->profile = enabled != 0;
    p->prof_ms[0] = p->prof_ms[1] = 0;
    p->prof_n[0] = p->prof_n[1] = 0;
    return TOMO_OK;
}

tomo_status tomo_profile_read(tomo_projector* p, double* out4) {
    if (!p || !out4) return fail(TOMO_ERR_INVALID, "null argument");
    out4[0] = p->prof_ms[0];
    out4[1] = (double)p->prof_n[0];
    out4[2] = p->prof_ms[1];
    out4[3] = (double)p->prof_n[1];
    return TOMO_OK;
}

tomo_status tomo_set_bp_rows(tomo_projector* p, int32_t rows) {
    if (!p || rows < 0 || rows > 2) return fail(TOMO_ERR_INVALID, "rows per backprojection thread: 0, 1 or 2");
    p->bp_rows = rows;
    return TOMO_OK;
}

// Autotuner: candidate kernel shapes timed on one update of this handle's series.
tomo_status tomo_autotune(tomo_projector* p, int32_t update, int32_t reps, double* out4) {
    if (!p || reps < 0) return fail(TOMO_ERR_INVALID, "bad argument");
    CKS(need_series(p));
    const Geometry& g = p->g;
    const bool tunable = g.separable && !p->bp_generic;
    const int T = (update <= 0 || update > g.N) ? g.N : update;
    if (reps == 0) reps = 3;
    double best_fp = 0, best_bp = 0;
    if (tunable) {
        // the trials use the projection slots and overwrite the volume: clear the added
        // projections, keep a copy of the volume (and slab scales) and put it back afterwards
        CKS(tomo_clear_projections(p));
        const size_t vbytes = p->nvox * (p->vtype == kVolF32 ? sizeof(float) : sizeof(uint16_t));
        unsigned char* save = nullptr;
        float* save_sc = nullptr;
        unsigned* save_mx = nullptr;
        CKS(alloc_n(p, &save, vbytes));
        if (p->vtype != kVolF32 &&
            (alloc_n(p, &save_sc, (size_t)g.H) != TOMO_OK || alloc_n(p, &save_mx, (size_t)g.H + 1) != TOMO_OK)) {
            free_n(p, &save, vbytes);
            free_n(p, &save_sc, (size_t)g.H);
            free_n(p, &save_mx, (size_t)g.H + 1);
            return TOMO_ERR_NOMEM;
        }
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        tomo_status st = TOMO_OK;
        auto ck = [&](cudaError_t e) {
            if (e != cudaSuccess && st == TOMO_OK) st = fail(TOMO_ERR_CUDA, cudaGetErrorString(e));
        };
        ck(cudaMemcpyAsync(save, p->vol(), vbytes, cudaMemcpyDeviceToDevice, p->stream));
        if (save_sc) ck(cudaMemcpyAsync(save_sc, p->d_vscale, sizeof(float) * g.H, cudaMemcpyDeviceToDevice, p->stream));
        if (save_mx)
            ck(cudaMemcpyAsync(save_mx, p->d_vmax, sizeof(unsigned) * (g.H + 1), cudaMemcpyDeviceToDevice, p->stream));
        ck(cudaEventCreate(&e0));
        ck(cudaEventCreate(&e1));
        for (int i = 0; i < T; i++) p->batch.push_back(i);
        if (st == TOMO_OK) st = upload_batch(p);
        const double factor = 1.0 / T;
        // time `reps` launches of fn after one untimed one
        auto timed = [&](const std::function<tomo_status()>& fn) -> double {
            if (st != TOMO_OK) return 0;
            if ((st = fn()) != TOMO_OK) return 0;
            ck(cudaEventRecord(e0, p->stream));
            for (int r = 0; r < reps && st == TOMO_OK; r++) st = fn();
            ck(cudaEventRecord(e1, p->stream));
            ck(cudaEventSynchronize(e1));
            float ms = 0;
            ck(cudaEventElapsedTime(&ms, e0, e1));
            return st == TOMO_OK ? ms / reps : 0;
        };
        // forward projection: tilts per CTA (0 = the balanced automatic grouping)
        const int tgmax = fp_max_tilts_per_cta(g.w);
        std::vector<int> cands = {0, tgmax, (3 * tgmax + 3) / 4, (tgmax + 1) / 2, (tgmax + 3) / 4};
        std::sort(cands.begin() + 1, cands.end());
        cands.erase(std::unique(cands.begin() + 1, cands.end()), cands.end());
        int best_c = 0;
        best_fp = 1e30;
        for (int c : cands) {
            if (c > T) continue;
            p->tilts_per_cta = c;
            const double ms = timed([&] { return run_fp(p, p->d_batch, T, 0, true, factor, 0); });
            if (st == TOMO_OK && ms < best_fp) {
                best_fp = ms;
                best_c = c;
            }
        }
        p->tilts_per_cta = best_c;
        // backprojection of the differences: volume rows per thread
        std::vector<int> rows = {0};
        if (p->vtype == kVolF32 && !g.fractional && !p->bp_wide) rows = {1, 2};
        int best_r = 0;
        best_bp = 1e30;
        for (int r : rows) {
            p->bp_rows = r;
            const double ms = timed([&] { return run_bp(p, p->d_diff, p->d_batch, T, 0, g.H, false, false); });
            if (st == TOMO_OK && ms < best_bp) {
                best_bp = ms;
                best_r = r;
            }
        }
        p->bp_rows = best_r;
        ck(cudaMemcpyAsync(p->vol(), save, vbytes, cudaMemcpyDeviceToDevice, p->stream));
        if (save_sc) ck(cudaMemcpyAsync(p->d_vscale, save_sc, sizeof(float) * g.H, cudaMemcpyDeviceToDevice, p->stream));
        if (save_mx)
            ck(cudaMemcpyAsync(p->d_vmax, save_mx, sizeof(unsigned) * (g.H + 1), cudaMemcpyDeviceToDevice, p->stream));
        ck(cudaStreamSynchronize(p->stream));
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        free_n(p, &save, vbytes);
        free_n(p, &save_sc, (size_t)g.H);
        free_n(p, &save_mx, (size_t)g.H + 1);
        tomo_clear_projections(p);
        if (st != TOMO_OK) return st;
    }
    if (out4) {
        out4[0] = p->tilts_per_cta;
        out4[1] = p->bp_rows;
        out4[2] = best_fp;
        out4[3] = best_bp;
    }
    return TOMO_OK;
}

tomo_status tomo_set_tilts_per_cta(tomo_projector* p, int32_t n) {
    if (!p || n < 0) return fail(TOMO_ERR_INVALID, "bad argument");
    p->tilts_per_cta = n;
    return TOMO_OK;
}

tomo_status tomo_debug_hold_first_copy(tomo_projector* p, int32_t enabled) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    p->hold_first_copy = enabled != 0;
    return TOMO_OK;
}

tomo_status tomo_cancel(tomo_projector* p) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    p->cancel = 1;
    return TOMO_OK;
}

int32_t tomo_first_index(uint64_t seed, int32_t iteration, int32_t nproj) {
    return first_index(seed, iteration, nproj);
}

tomo_status tomo_order(tomo_projector* p, int32_t first, int32_t* order_out) {
    if (!p || !order_out) return fail(TOMO_ERR_INVALID, "null argument");
    if (!p->series_loaded) return fail(TOMO_ERR_STATE, "no tilt-series loaded");
    if (first < 0 || first >= p->g.N) return fail(TOMO_ERR_INVALID, "first index out of range");
    order_shuffle(p->g.N, p->euler.data(), first, order_out);
    return TOMO_OK;
}

tomo_status tomo_order_shuffle(int32_t nproj, const double* euler, int32_t first, int32_t* order_out) {
    if (!euler || !order_out || nproj <= 0) return fail(TOMO_ERR_INVALID, "null argument or empty series");
    if (first < 0 || first >= nproj) return fail(TOMO_ERR_INVALID, "first index out of range");
    order_shuffle(nproj, euler, first, order_out);
    return TOMO_OK;
}

tomo_status tomo_run_wbp(tomo_projector* p, int32_t y0, int32_t y1) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    CKS(need_series(p));
    const int N = p->g.N;
    std::vector<int> all(N);
    for (int t = 0; t < N; t++) all[t] = t;
    CK(cudaMemcpyAsync(p->d_batch, all.data(), sizeof(int) * N, cudaMemcpyHostToDevice, p->stream));
    CK(launch_gather(p->d_obatch, p->d_meas, p->d_batch, N, p->npix, p->stream));
    CKS(apply_weighting(p, p->d_obatch, N));
    CKS(run_bp(p, p->d_obatch, p->d_batch, N, y0, y1, p->meas_has_nan || p->meas_has_inf, false));
    CKS(check_status(p));
    p->batch.clear();
    p->batch_uploaded = false;
    p->diffs_valid = p->projected = p->obatch_valid = false;
    return TOMO_OK;
}

tomo_status tomo_run_ossart(tomo_projector* p, int32_t n_iter, double relax, int32_t update, uint64_t seed,
                            int32_t y0, int32_t y1, int32_t use_graph, double* err_out) {
    if (!p) return fail(TOMO_ERR_INVALID, "null handle");
    CKS(need_series(p));
    if (n_iter < 0 || update < 0) return fail(TOMO_ERR_INVALID, "negative iteration count or update size");
    const Geometry& g = p->g;
    const int N = g.N;
    const int upd = (update == 0) ? N : std::min(update, N);
    const double factor = (double)(float)(relax / upd);  // float factorimg (TomoReconstruction2.java:646)
    if (p->orders_cap < n_iter) {
        free_n(p, &p->d_orders, (size_t)p->orders_cap * N);
        CKS(alloc_n(p, &p->d_orders, (size_t)std::max(n_iter, 1) * N));
        p->orders_cap = std::max(n_iter, 1);
    }
    std::vector<int> orders((size_t)n_iter * N);
    for (int it = 0; it < n_iter; it++)
        order_shuffle(N, p->euler.data(), first_index(seed, it, N), &orders[(size_t)it * N]);
    if (n_iter > 0)
        CK(cudaMemcpyAsync(p->d_orders, orders.data(), sizeof(int) * orders.size(), cudaMemcpyHostToDevice,
                           p->stream));
    std::vector<double> errs((size_t)N);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const int nsub = (N + upd - 1) / upd;
    if (p->profile && (int)p->ev.size() < 4 * nsub) {
        while ((int)p->ev.size() < 4 * nsub) {
            cudaEvent_t e;
            CK(cudaEventCreate(&e));
            p->ev.push_back(e);
        }
    }
    {
        // depth-split scratch for the subset sizes of this run, before any capture
        int j0, j1;
        fp_rows(p, y0, &j0, &j1);
        for (int T : {upd, N - (nsub - 1) * upd})
            if (T > 0) fp_split(p, T, j1 - j0, auto_tilts_per_cta(p, T, j1 - j0));
        if (g.separable && g.fractional) CKS(ensure_fp_rowmap(p, j0));
    }
    // row streams: integral separable FP32 geometry without long-object compensation
    // (its norm maximum couples the rows of a projection)
    const int K = (p->row_streams > 1 && g.separable && !g.fractional && !p->bp_generic && p->vtype == kVolF32 &&
                   !p->params.long_object && g.fp_row_off == g.bp_row_off)
                      ? p->row_streams
                      : 1;
    int rj0 = 0, rj1 = 0;
    fp_rows(p, y0, &rj0, &rj1);
    const int ry0 = std::max(0, y0), ry1 = std::min(g.H, y1);
    if (K > 1) {
        const size_t need = 1 + (size_t)nsub * K + K + 1;
        while (p->rs_ev.size() < need) {
            cudaEvent_t e;
            CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            p->rs_ev.push_back(e);
        }
    }
    auto body_rows = [&](const int* d_ord) -> tomo_status {
        CKS(start_iteration(p));
        cudaStream_t main = p->stream;
        struct Restore {  // the handle's stream comes back on every exit path
            tomo_projector* p;
            cudaStream_t s;
            ~Restore() { p->stream = s; }
        } restore{p, main};
        if (rj0 > 0) {
            // rows the reference leaves untouched stay zero, for every slot of the iteration
            for (int b = 0; b < N; b++) {
                const size_t o = (size_t)b * p->npix, n = sizeof(float) * (size_t)std::min(rj0, g.h) * g.w;
                CK(cudaMemsetAsync(p->d_proj + o, 0, n, main));
                CK(cudaMemsetAsync(p->d_norm + o, 0, n, main));
                CK(cudaMemsetAsync(p->d_diff + o, 0, n, main));
            }
            CK(cudaMemsetAsync(p->d_errpart, 0, sizeof(double) * (size_t)N * g.h, main));
        }
        cudaEvent_t* ev = p->rs_ev.data();
        CK(cudaEventRecord(ev[0], main));
        CK(cudaStreamWaitEvent(p->rs_reduce, ev[0], 0));
        // volume rows [yb[k], yb[k+1]) and the projection rows they see
        std::vector<int> yb(K + 1), jb(K + 1);
        for (int k = 0; k <= K; k++) {
            yb[k] = ry0 + (int)((long long)(ry1 - ry0) * k / K);
            jb[k] = std::min(std::max(yb[k] + g.fp_row_off, rj0), rj1);
        }
        jb[0] = rj0;
        jb[K] = rj1;
        tomo_status st = TOMO_OK;
        for (int s = 0, q = 0; s < N && st == TOMO_OK; s += upd, q++) {
            const int T = std::min(upd, N - s);
            for (int k = 0; k < K && st == TOMO_OK; k++) {
                p->stream = p->rs[k];
                if (q == 0) CK(cudaStreamWaitEvent(p->stream, ev[0], 0));
                if (p->profile && k == 0)
                    CK(cudaEventRecordWithFlags(p->ev[4 * q + 0], p->stream, cudaEventRecordExternal));
                st = run_fp_range(p, d_ord + s, T, jb[k], jb[k + 1], factor, s);
                if (p->profile && k == 0)
                    CK(cudaEventRecordWithFlags(p->ev[4 * q + 1], p->stream, cudaEventRecordExternal));
                CK(cudaEventRecord(ev[1 + (size_t)q * K + k], p->stream));
            }
            for (int k = 0; k < K; k++) CK(cudaStreamWaitEvent(p->rs_reduce, ev[1 + (size_t)q * K + k], 0));
            CK(launch_reduce_err(p->d_errpart + (size_t)s * g.h, p->d_err + s, T, g.h, p->rs_reduce));
            for (int k = 0; k < K && st == TOMO_OK; k++) {
                p->stream = p->rs[k];
                st = run_bp(p, p->d_diff + (size_t)s * p->npix, d_ord + s, T, yb[k], yb[k + 1], p->meas_has_inf,
                            true);
                if (p->profile && k == 0)
                    CK(cudaEventRecordWithFlags(p->ev[4 * q + 2], p->stream, cudaEventRecordExternal));
            }
        }
        p->stream = main;
        const size_t j = 1 + (size_t)nsub * K;
        for (int k = 0; k < K; k++) {
            CK(cudaEventRecord(ev[j + k], p->rs[k]));
            CK(cudaStreamWaitEvent(main, ev[j + k], 0));
        }
        CK(cudaEventRecord(ev[j + K], p->rs_reduce));
        CK(cudaStreamWaitEvent(main, ev[j + K], 0));
        CKS(st);
        CKS(end_iteration(p));
        return TOMO_OK;
    };
    auto body = [&](const int* d_ord) -> tomo_status {
        if (K > 1) return body_rows(d_ord);
        CKS(start_iteration(p));
        for (int s = 0, k = 0; s < N; s += upd, k++) {
            const int T = std::min(upd, N - s);
            if (p->profile) CK(cudaEventRecordWithFlags(p->ev[4 * k + 0], p->stream, cudaEventRecordExternal));
            CKS(run_fp(p, d_ord + s, T, y0, true, factor, s));
            if (p->profile) CK(cudaEventRecordWithFlags(p->ev[4 * k + 1], p->stream, cudaEventRecordExternal));
            CKS(run_bp(p, p->d_diff + (size_t)s * p->npix, d_ord + s, T, y0, y1, p->meas_has_inf, true));
            if (p->profile) CK(cudaEventRecordWithFlags(p->ev[4 * k + 2], p->stream, cudaEventRecordExternal));
        }
        CKS(end_iteration(p));
        return TOMO_OK;
    };
    uint64_t graph_kernels = 0;
    int* d_cur = p->d_batch;  // the graph reads the iteration's order from here
    tomo_status result = TOMO_OK;
    for (int it = 0; it < n_iter && result == TOMO_OK; it++) {
        if (p->cancel.exchange(0)) {
            result = fail(TOMO_ERR_CANCELLED, "cancelled");
            break;
        }
        CK(cudaMemcpyAsync(d_cur, p->d_orders + (size_t)it * N, sizeof(int) * N, cudaMemcpyDeviceToDevice,
                           p->stream));
        if (use_graph && !p->fista) {
            if (!exec) {
                const uint64_t before = tomo::g_launches.load();
                CK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
                tomo_status bs = body(d_cur);
                cudaError_t ce = cudaStreamEndCapture(p->stream, &graph);
                // kernels are counted when the graph runs, not when it is captured
                graph_kernels = tomo::g_launches.load() - before;
                tomo::g_launches -= graph_kernels;
                if (bs != TOMO_OK) return bs;
                CK(ce);
                CK(cudaGraphInstantiate(&exec, graph, 0));
            }
            CK(cudaGraphLaunch(exec, p->stream));
            tomo::count_launch((int)graph_kernels);
        } else {
            CKS(body(d_cur));
        }
        CK(cudaMemcpyAsync(errs.data(), p->d_err, sizeof(double) * N, cudaMemcpyDeviceToHost, p->stream));
        CK(cudaStreamSynchronize(p->stream));
        if (p->profile) {
            for (int k = 0; k < nsub; k++) {
                float a = 0, b = 0;
                CK(cudaEventElapsedTime(&a, p->ev[4 * k + 0], p->ev[4 * k + 1]));
                CK(cudaEventElapsedTime(&b, p->ev[4 * k + 1], p->ev[4 * k + 2]));
                p->prof_ms[0] += a;
                p->prof_ms[1] += b;
                p->prof_n[0]++;
                p->prof_n[1]++;
            }
        }
        if (err_out) {
            // osartIteration's error summary (TomoReconstruction2.java:692-730), including its
            // else-if: a new maximum is never also tested as a minimum.
            const int* ord = &orders[(size_t)it * N];
            double som = 0, errmin = 3.4028234663852886e38, errmax = 0;
            int imin = 0, imax = 0;
            for (int t = 0; t < N; t++) {
                const double e = errs[t];
                som += e;
                if (e > errmax) {
                    errmax = e;
                    imax = ord[t];
                } else if (e < errmin) {
                    errmin = e;
                    imin = ord[t];
                }
            }
            double* o = err_out + 5 * (size_t)it;
            o[0] = std::sqrt(som / (double)((long long)N * g.W * g.H));
            o[1] = std::sqrt(errmin / (double)(g.W * g.H));
            o[2] = imin;
            o[3] = std::sqrt(errmax / (double)(g.W * g.H));
            o[4] = imax;
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (result != TOMO_OK) return result;
    CKS(check_status(p));
    p->batch.clear();
    p->batch_uploaded = false;
    p->diffs_valid = p->projected = p->obatch_valid = false;
    return TOMO_OK;
}

}  // extern "C"
