// Batched execution of many handles (heterogeneous tilt-series).
//
// A batch references existing handles (each keeps its own volume, series,
// tables and options) and runs one OS-SART iteration of all of them together:
// for every update index s, one forward-projection launch per kernel variant
// covers update s of every member that has one (each CTA reads its
// {descriptor, tilt group, row} work item), one batched residual reduction
// follows, and one backprojection launch covers all members' tiles.  Optionally
// (tomo_batch_set_persistent) each phase is one persistent launch per CTA size
// instead: resident CTAs take items from a list, longest first, through an
// atomic cursor, and the launches of a phase run side by side.  The
// per-member descriptors and work lists are rebuilt only when the membership
// or the update sizes change, and the step's launches are captured once as a
// CUDA graph and replayed while they stay valid; every iteration only uploads
// the members' new orderings (orderShuffleART with the given first index) and
// reads their residuals back.
#include <algorithm>
#include <cmath>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "tomo_handle.h"

using namespace tomo;

// Page-locked host staging of a batch's per-iteration orderings, residuals and status
// words.  Copies from or to pageable memory go through the driver's staging path, where a
// small copy of one lane waited behind the large series uploads of requests being
// admitted on other threads.
template <class T>
struct Pinned {
    T* p = nullptr;
    size_t cap = 0;
    cudaError_t reserve(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        const size_t c = std::max<size_t>(std::max<size_t>(n, cap + cap / 2), 64);
        cap = 0;
        const cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&p), c * sizeof(T), cudaHostAllocDefault);
        if (e == cudaSuccess) cap = c;
        else p = nullptr;
        return e;
    }
    T& operator[](size_t i) { return p[i]; }
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
};

struct tomo_batch {
    std::vector<tomo_projector*> members;
    std::vector<int> upd;        // update size of each member in the cached plan
    std::vector<double> factor;  // relaxation factor of each member in the cached plan
    bool plan_valid = false;
    cudaStream_t stream = nullptr;      // where the batch's work runs
    cudaStream_t own_stream = nullptr;  // the stream the batch created
    // device plan
    FpLaunch* d_fp = nullptr;
    BpLaunch* d_bp = nullptr;
    ErrReduce* d_red = nullptr;
    int4* d_fp_items = nullptr;
    int4* d_bp_items = nullptr;
    size_t cap_fp = 0, cap_bp = 0, cap_fpi = 0, cap_bpi = 0, cap_red = 0;
    struct FpSeg {
        int s, qp, nt, zc, pk;
        size_t smem;
        int off, n;
    };
    struct BpSeg {
        int s;
        bool sanitize, pos;
        int vt;
        bool pairs;
        int off, n;
    };
    struct RedSeg {
        int s, off, n, maxT;
    };
    struct VolSeg {  // the 16-bit members with an update s (slab-scale passes)
        int s, off, n, maxH;
    };
    std::vector<VolSeg> vol_segs;
    VolJob* d_vjobs = nullptr;
    size_t cap_vjobs = 0;
    // persistent launches: one per (s, block size, chunk depth) for the forward phase and
    // per (s, flags, storage type, row pairs) for the backprojection; cursor: its slot of
    // d_cursor, zeroed at the start of every iteration
    struct FpPSeg {
        int s, nt, zc;
        size_t smem;
        int off, n, cursor, grid;
    };
    struct BpPSeg {
        int s;
        bool sanitize, pos;
        int vt;
        bool pairs;
        int off, n, cursor, grid;
    };
    std::vector<FpSeg> fp_segs;
    std::vector<BpSeg> bp_segs;
    std::vector<RedSeg> red_segs;
    std::vector<FpPSeg> fp_psegs;
    std::vector<BpPSeg> bp_psegs;
    int persistent = 0;  // tomo_batch_set_persistent mode (default: a launch per kernel variant)
    int* d_cursor = nullptr;
    size_t cap_cursor = 0;
    int n_cursor = 0;
    int priority = 0;
    // side streams and events for launches of one phase that run side by side
    std::vector<cudaStream_t> aux;
    std::vector<cudaEvent_t> ev_join;
    cudaEvent_t ev_fork = nullptr;
    int max_nsub = 0;
    bool has_fista = false;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    uint64_t graph_kernels = 0;
    Pinned<int> host_orders;
    Pinned<double> host_err;
    Pinned<int> host_status;
};

namespace {

// tomo_batch_set_persistent modes (1 = forward and backprojection persistent, longest first)
constexpr int kPersistFp = 2, kPersistBp = 4, kPersistListOrder = 8, kPersistSerial = 16;

#define BCK(expr)                                                                              \
    do {                                                                                       \
        cudaError_t _e = (expr);                                                               \
        if (_e != cudaSuccess) {                                                               \
            cudaGetLastError();                                                                \
            return handle_fail(TOMO_ERR_CUDA, (std::string(#expr) + ": " + cudaGetErrorString(_e)).c_str()); \
        }                                                                                      \
    } while (0)

#define BCKS(expr)                    \
    do {                              \
        tomo_status _s = (expr);      \
        if (_s != TOMO_OK) return _s; \
    } while (0)

// Plan buffers grow by half again and come from the engine's stream-ordered pool: a batch
// whose membership grows while other batches run never waits for the whole device.
template <class T>
tomo_status ensure(T** ptr, size_t* cap, size_t n, cudaStream_t s) {
    if (n <= *cap && *ptr) return TOMO_OK;
    if (*ptr) pool_free(*ptr, s);
    *ptr = nullptr;
    size_t c = std::max<size_t>(std::max<size_t>(n, *cap + *cap / 2), 16);
    if (pool_malloc(reinterpret_cast<void**>(ptr), c * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        *cap = 0;
        return handle_fail(TOMO_ERR_NOMEM, "batch plan allocation failed");
    }
    *cap = c;
    return TOMO_OK;
}

void drop_graph(tomo_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// Descriptors and work lists of one iteration for the current membership.
tomo_status build_plan(tomo_batch* b) {
    std::vector<FpLaunch> fp;
    std::vector<BpLaunch> bp;
    std::vector<ErrReduce> red;
    // work items grouped by (s, qp, zc, pair kind) for FP and (s, sanitize, pos, storage type) for BP
    std::map<std::tuple<int, int, int, int, int>, std::vector<int4>> fpi;
    std::map<std::tuple<int, int, int, int, int>, size_t> fpsmem;
    std::map<std::tuple<int, int, int, int, int>, std::vector<int4>> bpi;
    std::map<std::tuple<int, int, int, int, int>, std::vector<double>> fpcost, bpcost;  // per item, persistent
    std::map<std::tuple<int, int, int, int, int>, std::vector<int>> fpclass;  // kernel body of a persistent item
    std::map<int, std::vector<ErrReduce>> reds;
    std::map<int, std::vector<VolJob>> vjobs;
    b->max_nsub = 0;
    b->has_fista = false;
    const int tx = bp_tile_x(), tz = bp_tile_z();
    for (size_t m = 0; m < b->members.size(); m++) {
        tomo_projector* p = b->members[m];
        const Geometry& g = p->g;
        if (!g.separable || g.fractional || p->bp_wide || p->bp_generic)
            return handle_fail(TOMO_ERR_UNSUPPORTED,
                               "batched iterations need a vertical tilt axis, scale 1 and whole-row centre offsets");
        if (p->vol_owner)
            return handle_fail(TOMO_ERR_UNSUPPORTED, "a handle sharing another handle's volume cannot join a batch");
        const int N = g.N, upd = b->upd[m];
        const int nsub = (N + upd - 1) / upd;
        b->max_nsub = std::max(b->max_nsub, nsub);
        b->has_fista = b->has_fista || p->fista;
        // rows the forward projector never writes must read as zero residual
        BCK(cudaMemsetAsync(p->d_errpart, 0, sizeof(double) * (size_t)N * g.h, b->stream));
        const int qp = fp_qp(g.w), nt = fp_threads(g.w);
        const int zc = fp_choose_zc(g.W, 1, p->vtype, nt);
        const int pk = p->vtype != kVolF32 ? 1 : 0;
        const int use_tma = fp_use_tma(g.W, p->vtype, p->vol());
        int lq = 0;
        while ((1 << lq) < qp) lq++;
        const bool fp_persist = (b->persistent & kPersistFp) && fp_persist_supported(nt, zc);
        const int offset = (g.h > g.H && g.scale == 1) ? (g.h - g.H) / 2 : 0;
        const int j0 = std::max(0, (int)std::floor(offset * g.scale + 0.5));
        for (int s = 0; s < nsub; s++) {
            const int T = std::min(upd, N - s * upd);
            const int slot = s * upd;
            FpLaunch a{};
            a.vol = p->vol();
            a.vtype = p->vtype;
            a.vscale = p->vtype == kVolF32 ? nullptr : p->d_vscale;
            a.meas = p->d_meas;
            a.tilts = p->d_batch + slot;
            a.T = T;
            a.ftilt = p->d_ftilt;
            a.rays = p->d_rays;
            a.proj = p->d_proj + (size_t)slot * p->npix;
            a.norm = p->d_norm + (size_t)slot * p->npix;
            a.diff = p->d_diff + (size_t)slot * p->npix;
            a.errpart = p->d_errpart + (size_t)slot * g.h;
            a.factor = b->factor[m];
            a.j0 = j0;
            a.j1 = g.h;
            a.tilts_per_cta = handle_tilts_per_cta(p, T);
            a.W = g.W;
            a.H = g.H;
            a.D = g.D;
            a.w = g.w;
            a.h = g.h;
            a.row_off = g.fp_row_off;
            a.status = p->d_status;
            const int di = (int)fp.size();
            fp.push_back(a);
            // persistent launches group by block size and chunk depth only (qp = pk = -1)
            const auto key = fp_persist ? std::make_tuple(s, -1, nt, zc, -1) : std::make_tuple(s, qp, nt, zc, pk);
            fpsmem[key] = std::max(fpsmem[key], fp_smem_bytes(zc, g.W, qp, 1, p->vtype));
            auto& items = fpi[key];
            // a row's tilt groups one after another: the staged planes are read again from L2
            const int flags = use_tma | (fp_persist ? (lq << 1) | (pk << 4) : 0);
            const double cost = (double)g.D * g.w * a.tilts_per_cta;  // ray-steps of a full item
            for (int j = j0; j < g.h; j++)
                for (int g0 = 0; g0 < T; g0 += a.tilts_per_cta) {
                    items.push_back(make_int4(di, g0, j, flags));
                    if (fp_persist) {
                        fpcost[key].push_back(cost);
                        fpclass[key].push_back(lq * 2 + pk);
                    }
                }
            reds[s].push_back(ErrReduce{a.errpart, p->d_err + slot, T, g.h});
            if (p->vtype != kVolF32)
                vjobs[s].push_back(VolJob{p->vol(), p->d_vscale, p->d_vmax, p->vtype, g.W, g.H, g.D, p->d_status});
            BpLaunch c{};
            c.vol = p->bp_target();
            c.vtype = p->bayes ? kVolF32 : p->vtype;
            c.vscale = p->d_vscale;
            c.vmax = p->d_vmax;
            c.img = a.diff;
            c.tilts = a.tilts;
            c.T = T;
            c.btilt = p->d_btilt;
            c.zint = p->d_zint;
            c.y0 = 0;
            c.y1 = g.H;
            c.W = g.W;
            c.H = g.H;
            c.D = g.D;
            c.w = g.w;
            c.h = g.h;
            c.row_off = g.bp_row_off;
            c.positivity = p->params.positivity;
            c.sanitize = p->meas_has_inf || p->vol_flag();
            c.status = p->d_status;
            const int bi = (int)bp.size();
            bp.push_back(c);
            // row pairs unless the member's tuning asks for one row per thread
            const bool pairs = bp_row_pairs(c.vtype, c.sanitize != 0, c.positivity != 0) && p->bp_rows != 1;
            auto& bitems = bpi[std::make_tuple(s, c.sanitize, c.positivity, c.vtype, pairs ? 1 : 0)];
            const int rstep = pairs ? 2 : 1, tzr = pairs ? bp_pair_tile_z(c.vtype) : tz;
            for (int r = 0; r < g.H; r += rstep) {
                bool reached = false;  // a row of the item sees a projection row
                for (int q = 0; q < rstep && r + q < g.H; q++) {
                    const int jp = r + q + g.bp_row_off;
                    reached = reached || (jp >= 0 && jp < g.h);
                }
                if (!reached) continue;
                for (int zt = 0; zt < (g.D + tzr - 1) / tzr; zt++)
                    for (int xt = 0; xt < (g.W + tx - 1) / tx; xt++) {
                        bitems.push_back(make_int4(bi, xt, zt, r));
                        bpcost[std::make_tuple(s, c.sanitize, c.positivity, c.vtype, pairs ? 1 : 0)].push_back(
                            (double)T * std::min(tzr, g.D - zt * tzr));
                    }
            }
        }
    }
    // flatten; the lists of persistent launches go longest item first (stable, so a row's
    // tilt groups stay together)
    // by kernel body first (CTAs that run the same body side by side share the instruction
    // cache), then longest first
    auto by_cost = [](std::vector<int4>& items, const std::vector<double>& cost, const std::vector<int>* cls) {
        std::vector<size_t> idx(items.size());
        for (size_t i = 0; i < idx.size(); i++) idx[i] = i;
        std::stable_sort(idx.begin(), idx.end(), [&](size_t x, size_t y) {
            if (cls && (*cls)[x] != (*cls)[y]) return (*cls)[x] < (*cls)[y];
            return cost[x] > cost[y];
        });
        std::vector<int4> out(items.size());
        for (size_t i = 0; i < idx.size(); i++) out[i] = items[idx[i]];
        items.swap(out);
    };
    const int sms = device_sms();
    std::vector<int4> fp_all, bp_all;
    b->fp_segs.clear();
    b->bp_segs.clear();
    b->red_segs.clear();
    b->fp_psegs.clear();
    b->bp_psegs.clear();
    b->n_cursor = 0;
    for (auto& kv : fpi) {
        const int s = std::get<0>(kv.first), nt = std::get<2>(kv.first), zc = std::get<3>(kv.first);
        if (std::get<1>(kv.first) < 0) {
            if (!(b->persistent & kPersistListOrder)) by_cost(kv.second, fpcost[kv.first], &fpclass[kv.first]);
            const int n = (int)kv.second.size();
            const int grid = std::min(n, fp_ctas_per_sm(nt) * sms);
            b->fp_psegs.push_back(tomo_batch::FpPSeg{s, nt, zc, fpsmem[kv.first], (int)fp_all.size(), n,
                                                     b->n_cursor++, grid});
        } else {
            b->fp_segs.push_back(tomo_batch::FpSeg{s, std::get<1>(kv.first), nt, zc, std::get<4>(kv.first),
                                                   fpsmem[kv.first], (int)fp_all.size(), (int)kv.second.size()});
        }
        fp_all.insert(fp_all.end(), kv.second.begin(), kv.second.end());
    }
    for (auto& kv : bpi) {
        const int s = std::get<0>(kv.first), vt = std::get<3>(kv.first);
        const bool san = std::get<1>(kv.first) != 0, pos = std::get<2>(kv.first) != 0, pairs = std::get<4>(kv.first) != 0;
        if (b->persistent & kPersistBp) {
            if (!(b->persistent & kPersistListOrder)) by_cost(kv.second, bpcost[kv.first], nullptr);
            const int n = (int)kv.second.size();
            const int grid = std::min(n, bp_persist_ctas_per_sm(vt, pairs) * sms);
            b->bp_psegs.push_back(tomo_batch::BpPSeg{s, san, pos, vt, pairs, (int)bp_all.size(), n, b->n_cursor++,
                                                     grid});
        } else {
            b->bp_segs.push_back(tomo_batch::BpSeg{s, san, pos, vt, pairs, (int)bp_all.size(), (int)kv.second.size()});
        }
        bp_all.insert(bp_all.end(), kv.second.begin(), kv.second.end());
    }
    BCKS(ensure(&b->d_cursor, &b->cap_cursor, (size_t)std::max(b->n_cursor, 1), b->stream));
    std::vector<VolJob> vall;
    b->vol_segs.clear();
    for (auto& kv : vjobs) {
        int maxH = 0;
        for (auto& j : kv.second) maxH = std::max(maxH, j.H);
        b->vol_segs.push_back(tomo_batch::VolSeg{kv.first, (int)vall.size(), (int)kv.second.size(), maxH});
        vall.insert(vall.end(), kv.second.begin(), kv.second.end());
    }
    BCKS(ensure(&b->d_vjobs, &b->cap_vjobs, std::max<size_t>(vall.size(), 1), b->stream));
    if (!vall.empty())
        BCK(cudaMemcpyAsync(b->d_vjobs, vall.data(), sizeof(VolJob) * vall.size(), cudaMemcpyHostToDevice, b->stream));
    for (auto& kv : reds) {
        int maxT = 0;
        for (auto& r : kv.second) maxT = std::max(maxT, r.T);
        b->red_segs.push_back(tomo_batch::RedSeg{kv.first, (int)red.size(), (int)kv.second.size(), maxT});
        red.insert(red.end(), kv.second.begin(), kv.second.end());
    }
    BCKS(ensure(&b->d_fp, &b->cap_fp, fp.size(), b->stream));
    BCKS(ensure(&b->d_bp, &b->cap_bp, bp.size(), b->stream));
    BCKS(ensure(&b->d_red, &b->cap_red, red.size(), b->stream));
    BCKS(ensure(&b->d_fp_items, &b->cap_fpi, fp_all.size(), b->stream));
    BCKS(ensure(&b->d_bp_items, &b->cap_bpi, bp_all.size(), b->stream));
    BCK(cudaMemcpyAsync(b->d_fp, fp.data(), sizeof(FpLaunch) * fp.size(), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->d_bp, bp.data(), sizeof(BpLaunch) * bp.size(), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->d_red, red.data(), sizeof(ErrReduce) * red.size(), cudaMemcpyHostToDevice, b->stream));
    if (!fp_all.empty())
        BCK(cudaMemcpyAsync(b->d_fp_items, fp_all.data(), sizeof(int4) * fp_all.size(), cudaMemcpyHostToDevice,
                            b->stream));
    if (!bp_all.empty())
        BCK(cudaMemcpyAsync(b->d_bp_items, bp_all.data(), sizeof(int4) * bp_all.size(), cudaMemcpyHostToDevice,
                            b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    b->plan_valid = true;
    drop_graph(b);
    return TOMO_OK;
}

// Runs the launches of one phase: the first on the batch stream, the others on side
// streams forked from it and joined back, so that one launch's tail overlaps the next.
tomo_status run_side_by_side(tomo_batch* b, const std::vector<std::function<cudaError_t(cudaStream_t)>>& jobs) {
    if (jobs.empty()) return TOMO_OK;
    if (b->persistent & kPersistSerial) {
        for (auto& j : jobs) BCK(j(b->stream));
        return TOMO_OK;
    }
    const size_t side = jobs.size() - 1;
    while (b->aux.size() < side) {
        int least = 0, greatest = 0;
        BCK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        cudaStream_t q = nullptr;
        cudaEvent_t e = nullptr;
        BCK(cudaStreamCreateWithPriority(&q, cudaStreamNonBlocking, std::max(greatest, least - b->priority)));
        b->aux.push_back(q);
        BCK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b->ev_join.push_back(e);
    }
    if (side > 0) {
        if (!b->ev_fork) BCK(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
        BCK(cudaEventRecord(b->ev_fork, b->stream));
    }
    for (size_t k = 1; k < jobs.size(); k++) {
        BCK(cudaStreamWaitEvent(b->aux[k - 1], b->ev_fork, 0));
        BCK(jobs[k](b->aux[k - 1]));
        BCK(cudaEventRecord(b->ev_join[k - 1], b->aux[k - 1]));
    }
    BCK(jobs[0](b->stream));
    for (size_t k = 1; k < jobs.size(); k++) BCK(cudaStreamWaitEvent(b->stream, b->ev_join[k - 1], 0));
    return TOMO_OK;
}

tomo_status launch_step(tomo_batch* b) {
    for (tomo_projector* p : b->members) BCKS(handle_start_iteration(p));
    if (b->n_cursor > 0) BCK(cudaMemsetAsync(b->d_cursor, 0, sizeof(int) * b->n_cursor, b->stream));
    for (int s = 0; s < b->max_nsub; s++) {
        std::vector<std::function<cudaError_t(cudaStream_t)>> jobs;
        for (auto& sg : b->fp_psegs)
            if (sg.s == s)
                jobs.push_back([b, sg](cudaStream_t q) {
                    return launch_fp_persist(sg.nt, sg.zc, b->d_fp, b->d_fp_items + sg.off, sg.n,
                                             b->d_cursor + sg.cursor, sg.grid, sg.smem, q);
                });
        BCKS(run_side_by_side(b, jobs));
        for (auto& sg : b->fp_segs)
            if (sg.s == s)
                BCK(launch_fp_batch(sg.qp, sg.nt, b->d_fp, b->d_fp_items + sg.off, sg.n, sg.zc, sg.smem, sg.pk, b->stream));
        for (auto& sg : b->red_segs)
            if (sg.s == s) BCK(launch_reduce_err_batch(b->d_red + sg.off, sg.n, sg.maxT, b->stream));
        // slab-scale passes of the 16-bit members that have an update s, one launch each
        for (auto& vs : b->vol_segs)
            if (vs.s == s) BCK(launch_vol_hooks_batch(b->d_vjobs + vs.off, vs.n, vs.maxH, true, b->stream));
        std::vector<std::function<cudaError_t(cudaStream_t)>> bjobs;
        for (auto& sg : b->bp_psegs)
            if (sg.s == s)
                bjobs.push_back([b, sg](cudaStream_t q) {
                    return launch_bp_persist(sg.sanitize, sg.pos, sg.vt, sg.pairs, b->d_bp, b->d_bp_items + sg.off,
                                             sg.n, b->d_cursor + sg.cursor, sg.grid, q);
                });
        BCKS(run_side_by_side(b, bjobs));
        for (auto& sg : b->bp_segs)
            if (sg.s == s)
                BCK(launch_bp_batch(sg.sanitize, sg.pos, sg.vt, sg.pairs, b->d_bp, b->d_bp_items + sg.off, sg.n,
                                    b->stream));
        for (auto& vs : b->vol_segs)
            if (vs.s == s) BCK(launch_vol_hooks_batch(b->d_vjobs + vs.off, vs.n, vs.maxH, false, b->stream));
    }
    for (tomo_projector* p : b->members) BCKS(handle_end_iteration(p));
    return TOMO_OK;
}

}  // namespace

extern "C" {

tomo_status tomo_batch_create(tomo_batch** out) {
    if (!out) return handle_fail(TOMO_ERR_INVALID, "null argument");
    tomo_batch* b = new tomo_batch();
    if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return handle_fail(TOMO_ERR_CUDA, "cannot create the batch stream");
    }
    b->stream = b->own_stream;
    *out = b;
    return TOMO_OK;
}

tomo_status tomo_batch_set_priority(tomo_batch* b, int32_t priority) {
    if (!b || priority < 0) return handle_fail(TOMO_ERR_INVALID, "bad argument");
    int least = 0, greatest = 0;  // numerically: least >= greatest, lower is more urgent
    BCK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int prio = std::max(greatest, least - priority);
    cudaStream_t s = nullptr;
    BCK(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio));
    // a captured iteration is launched into whatever stream the batch holds
    cudaStreamSynchronize(b->stream);
    const bool own = b->stream == b->own_stream;
    cudaStreamDestroy(b->own_stream);
    b->own_stream = s;
    if (own) b->stream = s;
    b->priority = priority;
    for (cudaStream_t& q : b->aux) {  // side streams follow
        cudaStreamSynchronize(q);
        cudaStreamDestroy(q);
        BCK(cudaStreamCreateWithPriority(&q, cudaStreamNonBlocking, prio));
    }
    drop_graph(b);  // captured with the old side streams' dependencies
    return TOMO_OK;
}

tomo_status tomo_batch_set_stream(tomo_batch* b, void* stream) {
    if (!b) return handle_fail(TOMO_ERR_INVALID, "null batch");
    BCK(cudaStreamSynchronize(b->stream));
    b->stream = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
    return TOMO_OK;
}

tomo_status tomo_batch_set_persistent(tomo_batch* b, int32_t on) {
    if (!b) return handle_fail(TOMO_ERR_INVALID, "null batch");
    BCK(cudaStreamSynchronize(b->stream));
    if (on < 0 || on > 31) return handle_fail(TOMO_ERR_INVALID, "persistent mode out of range");
    b->persistent = on == 1 ? (kPersistFp | kPersistBp) : on;
    b->plan_valid = false;
    drop_graph(b);
    return TOMO_OK;
}

tomo_status tomo_batch_destroy(tomo_batch* b) {
    if (!b) return TOMO_OK;
    cudaStreamSynchronize(b->stream);
    drop_graph(b);
    for (void* q : {(void*)b->d_fp, (void*)b->d_bp, (void*)b->d_red, (void*)b->d_fp_items, (void*)b->d_bp_items,
                    (void*)b->d_cursor, (void*)b->d_vjobs})
        if (q) pool_free(q, b->stream);
    cudaStreamSynchronize(b->stream);
    for (cudaStream_t q : b->aux) {
        cudaStreamSynchronize(q);
        cudaStreamDestroy(q);
    }
    for (cudaEvent_t e : b->ev_join) cudaEventDestroy(e);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->stream != b->own_stream) cudaStreamSynchronize(b->stream);
    cudaStreamDestroy(b->own_stream);
    delete b;
    return TOMO_OK;
}

tomo_status tomo_batch_set(tomo_batch* b, tomo_projector* const* members, int32_t n) {
    if (!b || (n > 0 && !members) || n < 0) return handle_fail(TOMO_ERR_INVALID, "bad argument");
    for (int i = 0; i < n; i++) {
        if (!members[i]) return handle_fail(TOMO_ERR_INVALID, "null member");
        BCKS(handle_need_series(members[i]));
        for (int k = 0; k < i; k++)
            if (members[k] == members[i]) return handle_fail(TOMO_ERR_INVALID, "a handle appears twice");
    }
    BCK(cudaStreamSynchronize(b->stream));
    b->members.assign(members, members + n);
    b->plan_valid = false;
    drop_graph(b);
    return TOMO_OK;
}

tomo_status tomo_batch_iteration(tomo_batch* b, const double* relax, const int32_t* update, const int32_t* first,
                                 int32_t use_graph, double* err_out) {
    if (!b || !relax || !update || !first) return handle_fail(TOMO_ERR_INVALID, "null argument");
    const size_t M = b->members.size();
    if (M == 0) return TOMO_OK;
    // the members' own streams must be idle: their buffers are used on the batch stream
    for (tomo_projector* p : b->members) BCK(cudaStreamSynchronize(p->stream));
    std::vector<int> upd(M);
    std::vector<double> fac(M);
    for (size_t m = 0; m < M; m++) {
        const int N = b->members[m]->g.N;
        if (update[m] < 0) return handle_fail(TOMO_ERR_INVALID, "negative update size");
        if (first[m] < 0 || first[m] >= N) return handle_fail(TOMO_ERR_INVALID, "first index out of range");
        upd[m] = update[m] == 0 ? N : std::min(update[m], N);
        fac[m] = (double)(float)(relax[m] / upd[m]);  // float factorimg (TomoReconstruction2.java:646)
    }
    if (!b->plan_valid || upd != b->upd || fac != b->factor) {
        b->upd = upd;
        b->factor = fac;
        BCKS(build_plan(b));
    }
    // orderings of this iteration into each member's batch buffer
    size_t total = 0;
    for (size_t m = 0; m < M; m++) total += b->members[m]->g.N;
    BCK(b->host_orders.reserve(total));
    BCK(b->host_err.reserve(total));
    BCK(b->host_status.reserve(M));
    size_t o = 0;
    for (size_t m = 0; m < M; m++) {
        tomo_projector* p = b->members[m];
        order_shuffle(p->g.N, p->euler.data(), first[m], &b->host_orders[o]);
        BCK(cudaMemcpyAsync(p->d_batch, &b->host_orders[o], sizeof(int) * p->g.N, cudaMemcpyHostToDevice,
                            b->stream));
        o += p->g.N;
    }
    // the members' start/end-of-iteration work (TVM, FISTA) joins the batch stream
    std::vector<cudaStream_t> saved(M);
    for (size_t m = 0; m < M; m++) {
        saved[m] = b->members[m]->stream;
        b->members[m]->stream = b->stream;
    }
    struct Restore {
        tomo_batch* b;
        std::vector<cudaStream_t>& s;
        ~Restore() {
            for (size_t m = 0; m < b->members.size(); m++) b->members[m]->stream = s[m];
        }
    } restore{b, saved};
    if (use_graph && !b->has_fista) {
        if (!b->exec) {
            const uint64_t before = g_launches.load();
            BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            tomo_status st = launch_step(b);
            cudaError_t ce = cudaStreamEndCapture(b->stream, &b->graph);
            b->graph_kernels = g_launches.load() - before;
            g_launches -= b->graph_kernels;
            if (st != TOMO_OK) {
                drop_graph(b);
                return st;
            }
            BCK(ce);
            BCK(cudaGraphInstantiate(&b->exec, b->graph, 0));
        }
        BCK(cudaGraphLaunch(b->exec, b->stream));
        count_launch((int)b->graph_kernels);
    } else {
        BCKS(launch_step(b));
    }
    // residuals and status words on the batch stream (a copy on the legacy default stream
    // waited for every other stream's work here: a small batch's iteration took as long as
    // a large batch's running beside it)
    for (size_t m = 0; m < M; m++) b->host_status[m] = 0;
    o = 0;
    for (size_t m = 0; m < M; m++) {
        tomo_projector* p = b->members[m];
        BCK(cudaMemcpyAsync(&b->host_err[o], p->d_err, sizeof(double) * p->g.N, cudaMemcpyDeviceToHost, b->stream));
        BCK(cudaMemcpyAsync(&b->host_status[m], p->d_status, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
        o += p->g.N;
    }
    BCK(cudaStreamSynchronize(b->stream));
    o = 0;
    for (size_t m = 0; m < M; m++) {
        tomo_projector* p = b->members[m];
        const int st = b->host_status[m];
        if (st != 0) {
            cudaMemsetAsync(p->d_status, 0, sizeof(int), b->stream);
            cudaStreamSynchronize(b->stream);
            std::string why = "member " + std::to_string(m) + ": a kernel reported status " + std::to_string(st);
            if (st & kStatusTimeout) why += " (bounded wait expired)";
            if (st & (int)kStatusRange) why += " (a volume value left the FP16 range of its slab scale)";
            return handle_fail(TOMO_ERR_DEVICE, why.c_str());
        }
        if (err_out) {
            const int N = p->g.N;
            const int* ord = &b->host_orders[o];
            double som = 0, errmin = 3.4028234663852886e38, errmax = 0;
            int imin = 0, imax = 0;
            for (int t = 0; t < N; t++) {
                const double e = b->host_err[o + t];
                som += e;
                if (e > errmax) {
                    errmax = e;
                    imax = ord[t];
                } else if (e < errmin) {
                    errmin = e;
                    imin = ord[t];
                }
            }
            const double wh = (double)p->g.W * p->g.H;
            double* e5 = err_out + 5 * m;
            e5[0] = std::sqrt(som / ((double)N * wh));
            e5[1] = std::sqrt(errmin / wh);
            e5[2] = imin;
            e5[3] = std::sqrt(errmax / wh);
            e5[4] = imax;
        }
        o += p->g.N;
    }
    for (tomo_projector* p : b->members) {
        p->batch.clear();
        p->batch_uploaded = false;
        p->diffs_valid = p->projected = p->obatch_valid = false;
    }
    return TOMO_OK;
}

}  // extern "C"
