// Host-side geometry: per-ray and per-column tables built with the reference's
// exact double arithmetic, the orderShuffleART ordering and the WBP row filters.
// Compiled with -ffp-contract=off so that a*b+c is rounded twice, as in Java.
#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <functional>
#include <thread>
#include <utility>
#include <vector>

#include "tomo_internal.h"

namespace tomo {

namespace {

constexpr double kAcc = (double)1e-10f;  // VoxelProjector3D.ACCURACY, a float constant (VoxelProjector3D.java:33)

long long to_fix(double v) { return (long long)std::llrint(v * kFix); }

// Finds the contiguous run of z in [0, n) where in(z) holds, starting from real
// estimates za, zb of its two ends.  `in` must describe an interval.
template <class F>
void find_interval(int n, double za, double zb, F in, int* lo_out, int* cnt_out) {
    if (za > zb) std::swap(za, zb);
    *lo_out = 0;
    *cnt_out = 0;
    if (n <= 0) return;
    auto clampi = [n](double v) -> int {
        if (!(v == v)) return 0;
        if (v < 0) return 0;
        if (v > n - 1) return n - 1;
        return (int)v;
    };
    // A point inside the interval, if any, is within a couple of steps of the estimate.
    int seed = -1;
    const int cands[] = {clampi(std::ceil(za)), clampi(std::floor(zb)), clampi(std::floor(0.5 * (za + zb))),
                         clampi(std::ceil(za) + 1), clampi(std::floor(zb) - 1), clampi(std::ceil(za) - 1),
                         clampi(std::floor(zb) + 1)};
    for (int c : cands)
        if (in(c)) { seed = c; break; }
    if (seed < 0) return;
    // Bisect both ends: every probe evaluates the exact predicate, and the last probes
    // of each search are the two planes on either side of that end.
    int a = 0, b = seed;  // in(b); everything below a is outside
    while (a < b) {
        const int m = a + (b - a) / 2;
        if (in(m)) b = m;
        else a = m + 1;
    }
    const int lo = a;
    a = seed;
    b = n - 1;  // in(a); everything above b is outside
    while (a < b) {
        const int m = a + (b - a + 1) / 2;
        if (in(m)) a = m;
        else b = m - 1;
    }
    *lo_out = lo;
    *cnt_out = a - lo + 1;
}

}  // namespace

bool tilt_is_vertical(const double* R) {
    return R[0] != 0.0 && R[1] == 0.0 && R[3] == 0.0 && R[4] == 1.0 && R[5] == 0.0;
}

// projectJosephPartial on a vertical-axis tilt (VoxelProjector3D.java:716-760): icF, zcF and
// dirY are signed zeros and divY is 1, so the ray's y is the task-stepped jcentered plus
// the volume centre, constant along the ray; getPixel (TomoReconstruction2.java:154-190)
// then takes ybase = (int)y and yFraction = (float)y - ybase.
void build_fp_rowmap(const Geometry& g, int j0, int* row, float* yf) {
    const double jinc = 1.0 / g.scale;
    const double bYmax = (double)((float)g.H + 1e-10f);
    for (int j = 0; j < g.h; j++) {
        row[j] = -1;
        yf[j] = 0.0f;
        if (j < j0) continue;
        const int s = j0 + 2 * ((j - j0) / 2);  // first row of the reference's 2-row task
        double jc = (s - 1.0 - g.pc[1]) / g.scale;
        jc = jc + jinc;
        if (j == s + 1) jc = jc + jinc;
        const double y = jc + g.vc[1];
        if (!(y + kAcc >= 0 && y < bYmax)) continue;
        const int yb = (y < 0) ? 0 : (int)y;
        row[j] = yb;
        yf[j] = (y < 0) ? 0.0f : (float)y - (float)yb;
    }
}

// backProjectPartial on a vertical-axis tilt (VoxelProjector3D.java:266-283): the x~ R10
// and z~ R12 terms are signed zeros, so yy = y~ * scale + cy for the whole row, and the
// voxel is inside when 0 <= yy < h.
void build_bp_rowmap(const Geometry& g, int* row, float* yf) {
    for (int r = 0; r < g.H; r++) {
        const double yy = (r - g.vc[1]) * g.scale + g.pc[3];
        row[r] = -1;
        yf[r] = 0.0f;
        if (!(yy >= 0 && yy < g.h)) continue;
        const int yb = (int)yy;
        row[r] = yb;
        yf[r] = (float)(yy - yb);
    }
}

bool tilt_is_separable(const double* R, const Geometry& g) {
    if (g.scale != 1.0) return false;
    if (!(R[0] != 0.0)) return false;
    if (R[1] != 0.0 || R[3] != 0.0 || R[4] != 1.0 || R[5] != 0.0) return false;
    const double o1 = g.pc[1] - g.vc[1], o3 = g.pc[3] - g.vc[1];
    return o1 == std::floor(o1) && o3 == std::floor(o3);
}

void build_generic_fp_tilt(const double* R, GenericFpTilt* o) {
    // VoxelProjector3D.projectJosephPartial (VoxelProjector3D.java:682-694), same operation order
    o->icF = R[3] / R[0];
    o->zcF = (R[5] - (R[3] * R[2] / R[0]));
    o->divY = R[4] - (R[3] * R[1] / R[0]);
    o->yFx = R[1];
    o->zFx = R[2];
    o->divX = R[0];
    o->dirY = -(R[5] - R[3] * R[2] / R[0]) / (R[4] - R[3] * R[1] / R[0]);
    o->dirX = (R[1] * (-o->dirY) - R[2]) / R[0];
    o->ninc = std::sqrt(o->dirX * o->dirX + o->dirY * o->dirY + 1);
}

// Forward-projection ray table of one tilt, following
// VoxelProjector3D.projectJosephPartial (VoxelProjector3D.java:671-821) for a
// separable tilt: the x position of ray i at plane z is the accumulated double
// oldx + (z+1) dirX + volcenterx; the ray counts a plane when
// x + ACCURACY >= 0 && x < W, and one extra normIncrement when it leaves the
// volume laterally.
void build_fp_tables(const Geometry& g, const double* R, FpTilt* tilt, FpRay* rays, float* normtab_scratch) {
    const double dirY = -(R[5] - R[3] * R[2] / R[0]) / (R[4] - R[3] * R[1] / R[0]);
    const double dirX = (R[1] * (-dirY) - R[2]) / R[0];
    const double ninc = std::sqrt(dirX * dirX + dirY * dirY + 1);
    const double vcx = g.vc[0], vcz = g.vc[2];
    const double bXmax = (double)((float)g.W + 1e-10f);
    tilt->step = to_fix(dirX);
    tilt->ninc = ninc;
    const int D = g.D;
    // norm_sum is a float accumulating a double increment: norm(k) for k increments.
    std::vector<float> own;
    float* normtab = normtab_scratch;
    if (!normtab) {
        own.assign((size_t)D + 2, 0.0f);
        normtab = own.data();
    }
    normtab[0] = 0.0f;
    for (int k = 1; k < D + 2; k++) normtab[k] = (float)((double)normtab[k - 1] + ninc);

    for (int i = 0; i < g.w; i++) {
        const double icentered = (i - g.pc[0]) / g.scale;
        // oldy is jcentered on a separable tilt and R[1] * oldy is a signed zero.
        double oldx0 = icentered - R[1] * 0.0 - R[2] * (-1 - vcz);
        oldx0 /= R[0];
        auto in_exact = [&](double x) { return x + kAcc >= 0 && x < bXmax; };
        auto x_of = [&](int z) { return oldx0 + (z + 1) * dirX + vcx; };
        bool near = false;
        auto in_fast = [&](int z) {
            const double x = x_of(z);
            if (std::fabs(x + kAcc) < 1e-8 || std::fabs(x - bXmax) < 1e-8) near = true;
            return in_exact(x);
        };
        int lo = 0, cnt = 0;
        if (dirX == 0.0) {
            if (in_exact(oldx0 + vcx)) { lo = 0; cnt = D; }
        } else {
            const double za = (-kAcc - vcx - oldx0) / dirX - 1.0;
            const double zb = (bXmax - vcx - oldx0) / dirX - 1.0;
            find_interval(D, za, zb, in_fast, &lo, &cnt);
            if (near) {
                // Replay the reference's accumulation exactly for rays that graze a border:
                // the first run of inside planes (the reference stops at the plane after it).
                double oldx = oldx0;
                int first = -1, run = 0;
                for (int z = 0; z < D; z++) {
                    const double xc = oldx + dirX;
                    if (in_exact(xc + vcx)) {
                        if (first < 0) first = z;
                        run++;
                    } else if (first >= 0) {
                        break;
                    }
                    oldx = xc;
                }
                lo = first < 0 ? 0 : first;
                cnt = run;
            }
        }
        int incr = cnt;
        if (cnt > 0 && lo + cnt - 1 < D - 1) incr++;  // extra increment when the ray exits the volume
        FpRay r;
        r.zab = (int32_t)((uint32_t)lo | ((uint32_t)cnt << 16));
        r.norm = cnt > 0 ? normtab[incr] : 0.0f;
        r.X0 = to_fix(oldx0 + dirX + vcx);
        rays[i] = r;
    }
}

// Backprojection tables of one tilt, following VoxelProjector3D.backProjectPartial
// (VoxelProjector3D.java:221-308): xx = ((x~ R00 + y~ R01) + z~ R02) * scale + cix,
// and a voxel contributes when 0 <= xx < w.  On a separable tilt y~ R01 is a
// signed zero, so the decision depends on (x, z) only.
void build_bp_tables(const Geometry& g, const double* R, BpTilt* tilt, int32_t* zint) {
    const double cix = g.pc[2];
    const double sc = g.scale;
    tilt->C = to_fix(R[0] * sc);
    tilt->S = to_fix(R[2] * sc);
    tilt->K = to_fix(cix - g.vc[0] * R[0] * sc - g.vc[2] * R[2] * sc);
    for (int x = 0; x < g.W; x++) {
        const double xt = x - g.vc[0];
        const double a = xt * R[0] + 0.0 * R[1];
        auto xx_of = [&](int k) {
            const double z = k - g.vc[2];
            return (a + z * R[2]) * g.scale + cix;
        };
        auto in = [&](int k) {
            const double xx = xx_of(k);
            return xx >= 0 && xx < g.w;
        };
        int lo = 0, cnt = 0;
        if (R[2] == 0.0) {
            if (in(0)) { lo = 0; cnt = g.D; }
        } else {
            const double za = (0.0 - cix - a) / R[2] + g.vc[2];
            const double zb = ((double)g.w - cix - a) / R[2] + g.vc[2];
            find_interval(g.D, za, zb, in, &lo, &cnt);
        }
        zint[x] = (int32_t)((uint32_t)lo | ((uint32_t)cnt << 16));
    }
}

// TomoReconstruction2.orderShuffleART (TomoReconstruction2.java:735-781) with a
// given first index: then repeatedly the remaining projection whose beam
// direction (row 2 of its Euler matrix) is most perpendicular to the last one.
void order_shuffle(int n, const double* euler, int first, int* out) {
    std::vector<char> todo((size_t)n, 1);
    int cc = 0, im = first;
    while (cc < n) {
        if (cc != 0) {
            double mini = 1.7976931348623157e308;
            int omini = -1;
            const double* a = euler + 9 * im + 6;
            for (int o = 0; o < n; o++) {
                if (!todo[o]) continue;
                const double* b = euler + 9 * o + 6;
                const double sp = std::fabs(a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
                if (sp < mini) { mini = sp; omini = o; }
            }
            im = omini;
        }
        if (todo[im]) { out[cc++] = im; todo[im] = 0; }
    }
}

// SplitMix64 of (seed, iteration): the deterministic stand-in for Math.random().
int first_index(uint64_t seed, int iteration, int nproj) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ULL * (uint64_t)(iteration + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    return nproj > 0 ? (int)(z % (uint64_t)nproj) : 0;
}

// One row of the WBP frequency mask (row filters only depend on the column frequency).
//  RADERMACHER: FFTWeighting.createWeightingMask (FFTWeighting.java:31-65) with a
//               zero tilt-axis angle, where the mask is independent of the row.
//  RAMP:        d_theta * |k| / w, DC term d_theta / (4 w).
//  HAMMING_RAMP: RAMP * (0.54 + 0.46 cos(2 pi k / w)).
// d_theta is the mean tilt spacing in radians (pi / N for a single tilt).
void weighting_row_filter(int kind, int w, int nproj, const double* sint, const double* tilts_deg, double diameter,
                          float* mask_row) {
    const double cx = w / 2.0;
    if (kind == 1) {
        for (int i = 0; i < w; i++) {
            const double ci = (i > cx) ? i - w : i;
            double weight = 0;
            for (int p = 0; p < nproj; p++) {
                const double zj = (ci * sint[p] * 1.0 + 0.0 * sint[p] * 0.0) / w;
                double value = diameter * M_PI * zj;
                if (value == 0)
                    value = 1;
                else
                    value = std::sin(value) / value;
                weight += value;
            }
            if (weight < 0.005) weight = (double)0.005f;
            weight *= diameter;
            mask_row[i] = (float)(1 / weight);
        }
        return;
    }
    double tmin = 0, tmax = 0;
    for (int p = 0; p < nproj; p++) {
        if (p == 0 || tilts_deg[p] < tmin) tmin = tilts_deg[p];
        if (p == 0 || tilts_deg[p] > tmax) tmax = tilts_deg[p];
    }
    const double dtheta = nproj > 1 ? (tmax - tmin) * (M_PI / 180.0) / (nproj - 1) : M_PI;
    for (int i = 0; i < w; i++) {
        const double ci = (i > cx) ? i - w : i;
        double m = (ci == 0) ? dtheta / (4.0 * w) : dtheta * std::fabs(ci) / w;
        if (kind == 3) m *= 0.54 + 0.46 * std::cos(2.0 * M_PI * ci / w);
        mask_row[i] = (float)m;
    }
}

}  // namespace tomo

namespace tomo {

namespace {

// In-place iterative radix-2 FFT in double, forward (e^{-2 pi i kn/M}); M a power of two.
void fft_host(std::vector<double>& re, std::vector<double>& im) {
    const int M = (int)re.size();
    int logM = 0;
    while ((1 << logM) < M) logM++;
    for (int i = 0; i < M; i++) {
        int r = 0;
        for (int b = 0; b < logM; b++) r |= ((i >> b) & 1) << (logM - 1 - b);
        if (r > i) {
            std::swap(re[i], re[r]);
            std::swap(im[i], im[r]);
        }
    }
    for (int len = 2; len <= M; len <<= 1) {
        const int half = len / 2;
        for (int i = 0; i < M; i += len)
            for (int k = 0; k < half; k++) {
                const double a = -2.0 * M_PI * k / len;
                const double wr = std::cos(a), wi = std::sin(a);
                const double xr = re[i + k + half], xi = im[i + k + half];
                const double tr = xr * wr - xi * wi, ti = xr * wi + xi * wr;
                re[i + k + half] = re[i + k] - tr;
                im[i + k + half] = im[i + k] - ti;
                re[i + k] += tr;
                im[i + k] += ti;
            }
    }
}

}  // namespace

void fft_host_forward(std::vector<double>& re, std::vector<double>& im) { fft_host(re, im); }

// The row filter of a non-power-of-two width as a convolution: h[n] = (1/w) sum_k
// mask[k] e^{2 pi i k n / w} (real for the even masks used here; the real part is
// kept), zero-padded to M points and transformed by an M-point radix-2 FFT in double.
void row_filter_spectrum(const float* mask_row, int w, int M, float2* H) {
    std::vector<double> re((size_t)M, 0.0), im((size_t)M, 0.0);
    for (int n = 0; n < w; n++) {
        double acc = 0.0;
        for (int k = 0; k < w; k++) {
            const long long kn = ((long long)k * n) % w;
            acc += (double)mask_row[k] * std::cos(2.0 * M_PI * (double)kn / w);
        }
        re[n] = acc / w;
    }
    fft_host(re, im);
    for (int m = 0; m < M; m++) H[m] = make_float2((float)re[m], (float)im[m]);
}

int dft_grid_size(int n) {
    if ((n & (n - 1)) == 0) return n;
    int M = 1;
    while (M < 2 * n - 1) M <<= 1;
    return M;
}

// Bluestein tables: chirp c[k] = exp(-i pi k^2 / n) (k^2 reduced mod 2n in integers so
// the angle stays exact), bspec = M-point spectrum of conj(c) wrapped to negative
// indices (b[m] = b[M - m] = conj(c[m])), twiddles exp(-2 pi i k / M).  For a power of
// two n == M only the twiddles are used.
void dft_row_tables(int n, int M, float2* chirp, float2* bspec, float2* tw) {
    for (int k = 0; k < M; k++) {
        const double a = -2.0 * M_PI * k / M;
        tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    if (M == n) {
        for (int k = 0; k < n; k++) chirp[k] = make_float2(1.0f, 0.0f);
        for (int k = 0; k < M; k++) bspec[k] = make_float2(1.0f, 0.0f);
        return;
    }
    std::vector<double> cr(n), ci(n);
    for (int k = 0; k < n; k++) {
        const double a = -M_PI * (double)(((long long)k * k) % (2LL * n)) / n;
        cr[k] = std::cos(a);
        ci[k] = std::sin(a);
        chirp[k] = make_float2((float)cr[k], (float)ci[k]);
    }
    std::vector<double> re((size_t)M, 0.0), im((size_t)M, 0.0);
    re[0] = cr[0];
    im[0] = -ci[0];
    for (int k = 1; k < n; k++) {
        re[k] = re[M - k] = cr[k];
        im[k] = im[M - k] = -ci[k];
    }
    fft_host(re, im);
    for (int m = 0; m < M; m++) bspec[m] = make_float2((float)re[m], (float)im[m]);
}

// FFTWeighting.createWeightingMask (FFTWeighting.java:31-65) for per-tilt axis angles,
// stored transposed (column frequency major) for the column pass.
void weighting_mask_2d(int w, int h, int nproj, const double* tilt_deg, const double* axis_deg, double diameter,
                       float* maskT) {
    const double cx = w / 2.0, cy = h / 2.0;
    std::vector<double> sint(nproj), cosp(nproj), sinp(nproj);
    for (int p = 0; p < nproj; p++) {
        sint[p] = std::sin(tilt_deg[p] * (M_PI / 180.0));
        cosp[p] = std::cos(axis_deg[p] * (M_PI / 180.0));
        sinp[p] = std::sin(axis_deg[p] * (M_PI / 180.0));
    }
    // w * h * nproj sines: rows are split over the host threads
    parallel_ranges(h, 8, [&](int ja, int jb) {
        for (int j = ja; j < jb; j++) {
            const double cj = (j > cy) ? j - h : j;
            for (int i = 0; i < w; i++) {
                const double ci = (i > cx) ? i - w : i;
                double weight = 0;
                for (int p = 0; p < nproj; p++) {
                    const double zj = (ci * sint[p] * cosp[p] + cj * sint[p] * sinp[p]) / w;
                    double value = diameter * M_PI * zj;
                    if (value == 0)
                        value = 1;
                    else
                        value = std::sin(value) / value;
                    weight += value;
                }
                if (weight < 0.005) weight = (double)0.005f;
                weight *= diameter;
                maskT[(size_t)i * h + j] = (float)(1 / weight);
            }
        }
    });
}

void parallel_ranges(int n, int min_per_thread, const std::function<void(int, int)>& fn) {
    if (n <= 0) return;
    const int hw = std::max(1, (int)std::thread::hardware_concurrency());
    const int nt = std::max(1, std::min({hw, 16, (n + min_per_thread - 1) / std::max(1, min_per_thread)}));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++) pool.emplace_back(fn, (int)((long long)n * t / nt), (int)((long long)n * (t + 1) / nt));
    fn(0, (int)((long long)n / nt));
    for (auto& th : pool) th.join();
}

}  // namespace tomo
