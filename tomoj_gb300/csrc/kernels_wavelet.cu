// Compressed-sensing regularisation of CompressedSensingProjector.endOfIteration
// (TomoJ_AdvancedReconstruction/.../projectors/CompressedSensingProjector.java:34-71): the
// volume goes to an FP64 buffer, through the separable 3-D fractional spline wavelet
// transform of fr.curie.wavelets.WaveletProcessing (doTransform3D), is soft-thresholded at
// the level that zeroes the requested fraction of coefficients (findThreshold, :80-125),
// transformed back (doInverse3D) and rounded into the FP32 volume (copyBufferToRec).
//
// Filters: the published fractional spline wavelets of Unser and Blu, the third-party
// library the reference calls (Fractional_Splines_Wavelets 1.0).  H(w) = sqrt(2)
// |cos(w/2)|^(alpha+1) exp(-i tau w) on (-pi, pi]; A(w) = |2 sin(w/2)|^(2 alpha+2)
// sum_k |w + 2 pi k|^-(2 alpha+2) (|k| <= 256, the tail from its integral and the first
// Euler-Maclaurin correction).
// Orthonormal: Ho = H sqrt(A(w)/A(2w)), Go = e^{-iw} conj(Ho(w+pi)); B-spline: synthesis
// H, e^{-iw} conj(H(w+pi)) A(w+pi), analysis H A(w)/A(2w), e^{-iw} conj(H(w+pi))/A(2w);
// dual: the B-spline pair exchanged.  All filter values are computed on the host in
// double; the device does only FFTs (radix 4, Bluestein for other lengths) and products.
//
// A level along an axis of length n runs a group of threads per pair of lines: DFT_n, the two analysis
// products folded to n/2 frequencies, two inverse DFT_{n/2} into [low | high].  The
// synthesis inverts it.  Levels act on the low-pass corner: x, y, z forward and z, y, x
// backward.  The threshold search runs on the device (fixed number of histogram passes,
// each skipped once the search is done), so the whole filter is graph-capturable.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "tomo_internal.h"

namespace tomo {

namespace {

constexpr int kWavThreads = 256;
constexpr int kWavTwN = 8192;      // twiddle table e^{-2 pi i k / 8192}, k < 6144
constexpr int kWavMaxPow2 = 8192;  // longest power-of-two line
constexpr int kWavMaxOther = 4096; // longest other line (Bluestein grid <= 8192)
constexpr int kWavTailK = 256;

struct WavState {
    unsigned long long maxkey;  // max |v| as double bits (non-negative: ordered as integers)
    int done;
    int index;
    long long nbpixels;
    double histomax, histoscale, threshold;
    unsigned long long hist[256];
};

struct WavDft {
    int n, logn;  // logn < 0: not a power of two (Bluestein)
    int M, logM;
    const double2* chirp;  // e^{-i pi (k^2 mod 2n) / n}, k < n
    const double2* bspec;  // DFT_M of the conjugate chirp, / M
};

struct WavLines {
    double* buf;
    int n;
    int nu, nv;
    int groups;  // line pairs per CTA (a power of two; blockDim.x / groups threads each)
    int stride;  // shared-memory entries per group: n + Bluestein scratch
    long long es, su, sv;  // element stride along a line, strides of the line indices u, v
    WavDft full, half;
    const double2* lo;  // analysis: conj(filter) / 2; synthesis: filter
    const double2* hi;
    const double2* tw;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// The threads of one line pair: index within the group, group size.  Every group of a CTA
// runs the same lengths, so the barriers below are reached by all threads together.
struct Grp {
    int t, nt;
};

// In-place DFT of s[0, n) (natural order in and out), n = 2^logn >= 2, unnormalised; inverse
// uses e^{+2 pi i kn/n}.  Decimation in time after a bit-reversal permutation: one radix-2
// stage when logn is odd, then radix-4 passes, each doing the radix-2 stages of spans h and
// 2h at once: with w = e^{-2 pi i pos / 4h}, the inputs take w^2, w and w^3 and a 4-point
// DFT whose only products are by -i (+i inverse).  Ends with a barrier.
__device__ void fft_pow2(double2* s, int n, int logn, const double2* __restrict__ tw, bool inverse, Grp g) {
    for (int k = g.t; k < n; k += g.nt) {
        const int r = (int)(__brev((unsigned)k) >> (32 - logn));
        if (k < r) {
            const double2 t = s[k];
            s[k] = s[r];
            s[r] = t;
        }
    }
    __syncthreads();
    int lg = 1;
    if (logn & 1) {
        for (int j = g.t; j < (n >> 1); j += g.nt) {
            const double2 a = s[2 * j], b = s[2 * j + 1];
            s[2 * j] = cadd(a, b);
            s[2 * j + 1] = csub(a, b);
        }
        __syncthreads();
        lg = 2;
    }
    for (; lg < logn; lg += 2) {
        const int h = 1 << (lg - 1);
        const int step = kWavTwN >> (lg + 1);  // e^{-2 pi i pos / 4h} = tw[pos * step]
        for (int j = g.t; j < (n >> 2); j += g.nt) {
            const int pos = j & (h - 1);
            const int i0 = ((j >> (lg - 1)) << (lg + 1)) + pos;
            const double2 a0 = s[i0];
            double2 a1 = s[i0 + h], a2 = s[i0 + 2 * h], a3 = s[i0 + 3 * h];
            if (pos != 0) {
                double2 w1 = tw[2 * pos * step], w2 = tw[pos * step], w3 = tw[3 * pos * step];
                if (inverse) {
                    w1.y = -w1.y;
                    w2.y = -w2.y;
                    w3.y = -w3.y;
                }
                a1 = cmul(a1, w1);
                a2 = cmul(a2, w2);
                a3 = cmul(a3, w3);
            }
            const double2 b0 = cadd(a0, a1), b1 = csub(a0, a1), b2 = cadd(a2, a3), b3 = csub(a2, a3);
            // -i b3 forward, +i b3 inverse
            const double2 t = inverse ? make_double2(-b3.y, b3.x) : make_double2(b3.y, -b3.x);
            s[i0] = cadd(b0, b2);
            s[i0 + 2 * h] = csub(b0, b2);
            s[i0 + h] = cadd(b1, t);
            s[i0 + 3 * h] = csub(b1, t);
        }
        __syncthreads();
    }
}

// DFT of x[0, n) in place (a: Bluestein scratch of P.M entries); unnormalised.
__device__ void dft_any(double2* x, double2* a, const WavDft& P, const double2* __restrict__ tw, bool inverse,
                        Grp g) {
    if (P.n <= 1) return;
    if (P.logn >= 0) {
        fft_pow2(x, P.n, P.logn, tw, inverse, g);
        return;
    }
    // inverse DFT = conj(DFT(conj(x)))
    const double cs = inverse ? -1.0 : 1.0;
    for (int k = g.t; k < P.M; k += g.nt)
        a[k] = k < P.n ? cmul(make_double2(x[k].x, cs * x[k].y), P.chirp[k]) : make_double2(0.0, 0.0);
    __syncthreads();
    fft_pow2(a, P.M, P.logM, tw, false, g);
    for (int k = g.t; k < P.M; k += g.nt) a[k] = cmul(a[k], P.bspec[k]);
    __syncthreads();
    fft_pow2(a, P.M, P.logM, tw, true, g);
    for (int k = g.t; k < P.n; k += g.nt) {
        const double2 v = cmul(a[k], P.chirp[k]);
        x[k] = make_double2(v.x, cs * v.y);
    }
    __syncthreads();
}

// One wavelet level on every line of a corner: analysis (SYN false) writes [low | high]
// over the line, synthesis (SYN true) reads [low | high] and writes the line.  A CTA takes
// the lines u and u + 1 as the real and imaginary parts of one complex signal (the
// filters have real impulse responses, so both stay separable through the products, the
// folding and the inverse transforms), as WaveletProcessing pairs neighbouring rows.
template <bool SYN>
__global__ void __launch_bounds__(kWavThreads) wav_lines_kernel(const WavLines L) {
    extern __shared__ double2 wsm[];
    const int nt = blockDim.x / L.groups;
    const int gi = threadIdx.x / nt;
    const Grp g{(int)threadIdx.x - gi * nt, nt};
    double2* x = wsm + (size_t)gi * L.stride;
    double2* a = x + L.n;
    const int npair = (L.nu + 1) >> 1;
    // pair index over (u pairs, v); a group past the end computes on zeros and stores nothing
    const long long pidx = (long long)blockIdx.x * L.groups + gi;
    const bool live = pidx < (long long)npair * L.nv;
    const int u0 = live ? 2 * (int)(pidx % npair) : 0;
    const int u1 = u0 + 1 < L.nu ? u0 + 1 : u0;
    const int v = live ? (int)(pidx / npair) : 0;
    double* line0 = L.buf + (long long)u0 * L.su + (long long)v * L.sv;
    double* line1 = L.buf + (long long)u1 * L.su + (long long)v * L.sv;
    const int n = L.n, m = n >> 1;
    for (int j = g.t; j < n; j += g.nt)
        x[j] = live ? make_double2(line0[(long long)j * L.es], u1 != u0 ? line1[(long long)j * L.es] : 0.0)
                    : make_double2(0.0, 0.0);
    __syncthreads();
    double scale;
    if (!SYN) {
        dft_any(x, a, L.full, L.tw, false, g);
        for (int k = g.t; k < m; k += g.nt) {
            const double2 x0 = x[k], x1 = x[k + m];
            x[k] = cadd(cmul(x0, L.lo[k]), cmul(x1, L.lo[k + m]));
            x[k + m] = cadd(cmul(x0, L.hi[k]), cmul(x1, L.hi[k + m]));
        }
        __syncthreads();
        dft_any(x, a, L.half, L.tw, true, g);
        dft_any(x + m, a, L.half, L.tw, true, g);
        scale = 1.0 / m;
    } else {
        dft_any(x, a, L.half, L.tw, false, g);
        dft_any(x + m, a, L.half, L.tw, false, g);
        for (int k = g.t; k < m; k += g.nt) {
            const double2 c = x[k], d = x[k + m];
            x[k] = cadd(cmul(c, L.lo[k]), cmul(d, L.hi[k]));
            x[k + m] = cadd(cmul(c, L.lo[k + m]), cmul(d, L.hi[k + m]));
        }
        __syncthreads();
        dft_any(x, a, L.full, L.tw, true, g);
        scale = 1.0 / n;
    }
    if (!live) return;
    for (int j = g.t; j < n; j += g.nt) {
        line0[(long long)j * L.es] = x[j].x * scale;
        if (u1 != u0) line1[(long long)j * L.es] = x[j].y * scale;
    }
}

__global__ void wav_from_volume_kernel(const float* __restrict__ vol, double* __restrict__ buf, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        buf[i] = (double)vol[i];
}

__global__ void wav_to_volume_kernel(const double* __restrict__ buf, float* __restrict__ vol, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        vol[i] = (float)buf[i];
}

__global__ void wav_maxabs_kernel(const double* __restrict__ buf, size_t n, WavState* st) {
    unsigned long long best = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long k = (unsigned long long)__double_as_longlong(fabs(buf[i]));
        best = k > best ? k : best;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_down_sync(0xffffffffu, best, o);
        best = t > best ? t : best;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(&st->maxkey, best);
}

// findThreshold's start: histomax = max |v| (an all-zero buffer gives threshold 0)
__global__ void wav_thr_init_kernel(WavState* st, long long nbpixels) {
    if (threadIdx.x != 0) return;
    const double hm = __longlong_as_double((long long)st->maxkey);
    st->nbpixels = nbpixels;
    st->histomax = hm;
    st->index = -1;
    for (int i = 0; i < 256; i++) st->hist[i] = 0;
    if (hm == 0.0) {
        st->threshold = 0.0;
        st->done = 1;
    } else {
        st->histoscale = 256.0 / hm;
        st->done = 0;
    }
}

// computeAbsHistogram: bin (int)(histoscale |v|), clamped to 255
__global__ void wav_hist_kernel(const double* __restrict__ buf, size_t n, WavState* st) {
    __shared__ unsigned int h[256];
    if (*(volatile int*)&st->done) return;
    const double scale = st->histoscale;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double s = scale * fabs(buf[i]);
        const int b = s >= 255.0 ? 255 : (int)s;
        atomicAdd(&h[b], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        if (h[i]) atomicAdd(&st->hist[i], (unsigned long long)h[i]);
}

// one round of findThreshold's refinement loop
__global__ void wav_thr_decide_kernel(WavState* st) {
    if (threadIdx.x != 0 || st->done) return;
    const long long nb = st->nbpixels;
    long long sum = 0;
    int index = -1;
    while (sum < nb && index < 255) {
        index++;
        sum += (long long)st->hist[index];
    }
    st->index = index;
    st->threshold = index / st->histoscale;
    if (nb > 0 && (double)sum / (double)nb > 1.01) {
        const double nm = fabs((index + 1) / st->histoscale);
        if (nm < st->histomax) {
            st->histomax = nm;
            st->histoscale = 256.0 / nm;
            for (int i = 0; i < 256; i++) st->hist[i] = 0;
            return;
        }
    }
    st->done = 1;
}

__global__ void wav_soft_kernel(double* __restrict__ buf, size_t n, const WavState* st) {
    const double t = st->threshold;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double v = buf[i];
        buf[i] = v > t ? v - t : (v < -t ? v + t : 0.0);
    }
}

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
int log2i(int n) {
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}

// A(w) of the degree-alpha fractional B-spline
double autocorr(double w, double alpha) {
    const double p = 2.0 * alpha + 2.0;
    w = std::remainder(w, 2.0 * M_PI);  // (-pi, pi]
    if (w == 0.0) return 1.0;
    double s = std::pow(std::fabs(w), -p);
    for (int k = 1; k <= kWavTailK; k++)
        s += std::pow(std::fabs(w + 2.0 * M_PI * k), -p) + std::pow(std::fabs(w - 2.0 * M_PI * k), -p);
    // the tail k > K: integral from K + 1/2 plus the midpoint-rule Euler-Maclaurin term
    const double a = 2.0 * M_PI * (kWavTailK + 0.5);
    s += (std::pow(a + w, 1.0 - p) + std::pow(a - w, 1.0 - p)) / (2.0 * M_PI * (p - 1.0));
    s -= 2.0 * M_PI * p / 24.0 * (std::pow(a + w, -p - 1.0) + std::pow(a - w, -p - 1.0));
    return std::pow(std::fabs(2.0 * std::sin(w / 2.0)), p) * s;
}

// refinement filter of the (alpha, tau) fractional B-spline
void refine(double w, double alpha, double tau, double& re, double& im) {
    w = std::remainder(w, 2.0 * M_PI);
    if (w == -M_PI) w = M_PI;
    const double mag = std::sqrt(2.0) * std::pow(std::fabs(std::cos(w / 2.0)), alpha + 1.0);
    re = mag * std::cos(tau * w);
    im = -mag * std::sin(tau * w);
}

}  // namespace

struct WaveletPlan {
    struct Dft {
        int n = 0, logn = -1, M = 0, logM = 0;
        size_t chirp = 0, bspec = 0;  // offsets (double2) in the tables
    };
    struct Pass {
        bool syn = false;
        int n = 0, nu = 0, nv = 0;
        long long es = 0, su = 0, sv = 0;
        Dft full, half;
        size_t lo = 0, hi = 0;
        int groups = 1, nt = kWavThreads, stride = 0;
        size_t smem = 0;
    };
    int W = 0, H = 0, D = 0;
    long long nbpixels = 0;
    std::vector<double2> tables;  // twiddles at offset 0, then chirps, spectra and filters
    std::vector<Pass> passes;     // forward levels then inverse levels
    size_t smem_max = 0;
    double2* d_tables = nullptr;
    double* d_buf = nullptr;
    WavState* d_state = nullptr;
};

namespace {

WaveletPlan::Dft make_dft(WaveletPlan& P, std::map<int, WaveletPlan::Dft>& cache, int n) {
    auto it = cache.find(n);
    if (it != cache.end()) return it->second;
    WaveletPlan::Dft d;
    d.n = n;
    if (is_pow2(n)) {
        d.logn = log2i(n);
    } else {
        d.logn = -1;
        d.M = 1;
        while (d.M < 2 * n - 1) d.M <<= 1;
        d.logM = log2i(d.M);
        d.chirp = P.tables.size();
        std::vector<double> cr(n), ci(n);
        for (int k = 0; k < n; k++) {
            const long long q = ((long long)k * k) % (2LL * n);
            const double ang = -M_PI * (double)q / n;
            cr[k] = std::cos(ang);
            ci[k] = std::sin(ang);
            P.tables.push_back(make_double2(cr[k], ci[k]));
        }
        std::vector<double> br(d.M, 0.0), bi(d.M, 0.0);
        for (int k = 0; k < n; k++) {
            br[k] = cr[k];
            bi[k] = -ci[k];
            if (k > 0) {
                br[d.M - k] = cr[k];
                bi[d.M - k] = -ci[k];
            }
        }
        fft_host_forward(br, bi);
        d.bspec = P.tables.size();
        for (int k = 0; k < d.M; k++) P.tables.push_back(make_double2(br[k] / d.M, bi[k] / d.M));
    }
    cache[n] = d;
    return d;
}

size_t dft_scratch(const WaveletPlan::Dft& d) { return d.logn >= 0 ? 0 : (size_t)d.M; }

// filters of one level length n: analysis (conj / 2) or synthesis, appended to the tables
void make_filters(WaveletPlan& P, int n, int type, double alpha, double tau, bool syn, size_t& lo, size_t& hi) {
    std::vector<double2> L(n), G(n);
    for (int k = 0; k < n; k++) {
        const double w = 2.0 * M_PI * (k > n / 2 ? k - n : k) / n;
        double hr, hi_, pr, pi_;
        refine(w, alpha, tau, hr, hi_);
        refine(w + M_PI, alpha, tau, pr, pi_);
        const double A = autocorr(w, alpha), Ap = autocorr(w + M_PI, alpha), A2 = autocorr(2.0 * w, alpha);
        const double er = std::cos(w), ei = -std::sin(w);  // e^{-iw}
        double lr, li, gr, gi;
        if (type == 0) {
            const double so = std::sqrt(A / A2), sp = std::sqrt(Ap / A2);
            lr = hr * so;
            li = hi_ * so;
            // e^{-iw} conj(Ho(w + pi))
            const double cr = pr * sp, ci = -pi_ * sp;
            gr = er * cr - ei * ci;
            gi = er * ci + ei * cr;
        } else {
            // B-spline synthesis pair (type 3) or, for the dual (type 6), its analysis pair
            const bool bspline_filter = (type == 3) == syn;
            const double fl = bspline_filter ? 1.0 : A / A2;
            const double fg = bspline_filter ? Ap : 1.0 / A2;
            lr = hr * fl;
            li = hi_ * fl;
            const double cr = pr * fg, ci = -pi_ * fg;
            gr = er * cr - ei * ci;
            gi = er * ci + ei * cr;
        }
        if (syn) {
            L[k] = make_double2(lr, li);
            G[k] = make_double2(gr, gi);
        } else {
            L[k] = make_double2(lr / 2, -li / 2);
            G[k] = make_double2(gr / 2, -gi / 2);
        }
    }
    lo = P.tables.size();
    P.tables.insert(P.tables.end(), L.begin(), L.end());
    hi = P.tables.size();
    P.tables.insert(P.tables.end(), G.begin(), G.end());
}

}  // namespace

WaveletPlan* wavelet_plan_create(int W, int H, int D, const int iters[3], int type, double alpha, double tau,
                                 double fraction_zeros, const char** why) {
    static const char* kWhy[] = {
        "wavelet type must be 0 (orthonormal), 3 (B-spline) or 6 (dual)",
        "wavelet degree must be above -0.5",
        "fraction of zeros must be in [0, 1]",
        "wavelet levels must be >= 0 and every level's length even and at most 8192 (4096 when not a power of two)",
    };
    if (type != 0 && type != 3 && type != 6) return *why = kWhy[0], nullptr;
    if (!(alpha > -0.5) || !std::isfinite(alpha) || !std::isfinite(tau)) return *why = kWhy[1], nullptr;
    if (!(fraction_zeros >= 0.0 && fraction_zeros <= 1.0)) return *why = kWhy[2], nullptr;
    const int dims[3] = {W, H, D};
    for (int a = 0; a < 3; a++) {
        if (iters[a] < 0 || iters[a] > 30) return *why = kWhy[3], nullptr;
        int n = dims[a];
        for (int l = 0; l < iters[a]; l++) {
            if (n < 2 || (n & 1) || n > (is_pow2(n) ? kWavMaxPow2 : kWavMaxOther)) return *why = kWhy[3], nullptr;
            n >>= 1;
        }
    }
    auto* P = new WaveletPlan();
    P->W = W;
    P->H = H;
    P->D = D;
    // (long)(percentageOfZeros * X * Y * Z), evaluated left to right
    P->nbpixels = (long long)(fraction_zeros * W * H * D);
    P->tables.resize(3 * kWavTwN / 4);
    for (int k = 0; k < 3 * kWavTwN / 4; k++) {
        const double ang = -2.0 * M_PI * k / kWavTwN;
        P->tables[k] = make_double2(std::cos(ang), std::sin(ang));
    }
    std::map<int, WaveletPlan::Dft> cache;
    const long long sx = 1, sy = W, sz = (long long)W * H;
    auto add_pass = [&](bool syn, int axis, const int size[3]) {
        WaveletPlan::Pass q;
        q.syn = syn;
        q.n = size[axis];
        if (axis == 0) {
            q.es = sx, q.nu = size[1], q.su = sy, q.nv = size[2], q.sv = sz;
        } else if (axis == 1) {
            q.es = sy, q.nu = size[0], q.su = sx, q.nv = size[2], q.sv = sz;
        } else {
            q.es = sz, q.nu = size[0], q.su = sx, q.nv = size[1], q.sv = sy;
        }
        q.full = make_dft(*P, cache, q.n);
        q.half = make_dft(*P, cache, q.n / 2);
        make_filters(*P, q.n, type, alpha, tau, syn, q.lo, q.hi);
        // threads per line pair: one per radix-4 butterfly of the longest transform (4 to
        // 256); line pairs per CTA: up to 256 threads, fewer when the pass would otherwise
        // leave less than two CTAs per SM
        const long long pairs = (long long)((q.nu + 1) / 2) * q.nv;
        const int work = std::max(q.full.logn >= 0 ? q.n : q.full.M, q.half.logn >= 0 ? q.n / 2 : q.half.M) / 4;
        q.nt = 4;
        while (q.nt < kWavThreads && q.nt < work) q.nt <<= 1;
        q.groups = kWavThreads / q.nt;
        while (q.groups > 1 && pairs / q.groups < 2LL * device_sms()) q.groups >>= 1;
        q.stride = q.n + (int)std::max(dft_scratch(q.full), dft_scratch(q.half));
        q.smem = sizeof(double2) * (size_t)q.groups * q.stride;
        P->smem_max = std::max(P->smem_max, q.smem);
        P->passes.push_back(q);
    };
    const int maxit = std::max(iters[0], std::max(iters[1], iters[2]));
    int size[3] = {W, H, D};
    for (int level = 1; level <= maxit; level++) {
        for (int a = 0; a < 3; a++)
            if (level <= iters[a]) add_pass(false, a, size);
        for (int a = 0; a < 3; a++)
            if (level <= iters[a]) size[a] >>= 1;
    }
    for (int level = maxit; level >= 1; level--) {
        for (int a = 0; a < 3; a++)
            if (level <= iters[a]) size[a] <<= 1;
        for (int a = 2; a >= 0; a--)
            if (level <= iters[a]) add_pass(true, a, size);
    }
    return P;
}

size_t wavelet_plan_table_bytes(const WaveletPlan* P) { return sizeof(double2) * P->tables.size(); }
size_t wavelet_plan_state_bytes() { return sizeof(WavState); }

cudaError_t wavelet_plan_bind(WaveletPlan* P, void* d_tables, double* d_buf, void* d_state, cudaStream_t s) {
    P->d_tables = static_cast<double2*>(d_tables);
    P->d_buf = d_buf;
    P->d_state = static_cast<WavState*>(d_state);
    cudaError_t e = cudaMemcpyAsync(d_tables, P->tables.data(), wavelet_plan_table_bytes(P), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    {
        // the limit is per kernel, shared by every handle: only ever raised
        static std::mutex mu;
        static size_t attr = 48 * 1024;
        std::lock_guard<std::mutex> lock(mu);
        if (P->smem_max > attr) {
            e = cudaFuncSetAttribute(wav_lines_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)P->smem_max);
            if (e != cudaSuccess) return e;
            e = cudaFuncSetAttribute(wav_lines_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)P->smem_max);
            if (e != cudaSuccess) return e;
            attr = P->smem_max;
        }
    }
    return cudaStreamSynchronize(s);
}

void wavelet_plan_destroy(WaveletPlan* P) { delete P; }

int wavelet_plan_passes(const WaveletPlan* P) { return (int)P->passes.size(); }

cudaError_t launch_wavelet_filter(const WaveletPlan* P, float* vol, cudaStream_t s) {
    const size_t n = (size_t)P->W * P->H * P->D;
    if (n == 0) return cudaSuccess;
    const int blocks = (int)std::min<size_t>((n + kWavThreads - 1) / kWavThreads, device_sms() * 8);
    auto dft_of = [&](const WaveletPlan::Dft& d) {
        WavDft r;
        r.n = d.n;
        r.logn = d.logn;
        r.M = d.M;
        r.logM = d.logM;
        r.chirp = d.logn >= 0 ? nullptr : P->d_tables + d.chirp;
        r.bspec = d.logn >= 0 ? nullptr : P->d_tables + d.bspec;
        return r;
    };
    wav_from_volume_kernel<<<blocks, kWavThreads, 0, s>>>(vol, P->d_buf, n);
    count_launch();
    const size_t nfwd = P->passes.size() / 2;
    auto run_pass = [&](const WaveletPlan::Pass& q) {
        WavLines L;
        L.buf = P->d_buf;
        L.n = q.n;
        L.nu = q.nu;
        L.nv = q.nv;
        L.groups = q.groups;
        L.stride = q.stride;
        L.es = q.es;
        L.su = q.su;
        L.sv = q.sv;
        L.full = dft_of(q.full);
        L.half = dft_of(q.half);
        L.lo = P->d_tables + q.lo;
        L.hi = P->d_tables + q.hi;
        L.tw = P->d_tables;
        const long long pairs = (long long)((q.nu + 1) / 2) * q.nv;
        const unsigned grid = (unsigned)((pairs + q.groups - 1) / q.groups);
        const int block = q.groups * q.nt;
        if (q.syn)
            wav_lines_kernel<true><<<grid, block, q.smem, s>>>(L);
        else
            wav_lines_kernel<false><<<grid, block, q.smem, s>>>(L);
        count_launch();
    };
    for (size_t i = 0; i < nfwd; i++) run_pass(P->passes[i]);
    cudaError_t e = cudaMemsetAsync(&P->d_state->maxkey, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    wav_maxabs_kernel<<<blocks, kWavThreads, 0, s>>>(P->d_buf, n, P->d_state);
    wav_thr_init_kernel<<<1, 32, 0, s>>>(P->d_state, P->nbpixels);
    count_launch(2);
    for (int pass = 0; pass < kWaveletThresholdPasses; pass++) {
        wav_hist_kernel<<<blocks, kWavThreads, 0, s>>>(P->d_buf, n, P->d_state);
        wav_thr_decide_kernel<<<1, 32, 0, s>>>(P->d_state);
        count_launch(2);
    }
    wav_soft_kernel<<<blocks, kWavThreads, 0, s>>>(P->d_buf, n, P->d_state);
    count_launch();
    for (size_t i = nfwd; i < P->passes.size(); i++) run_pass(P->passes[i]);
    wav_to_volume_kernel<<<blocks, kWavThreads, 0, s>>>(P->d_buf, vol, n);
    count_launch();
    return cudaGetLastError();
}

cudaError_t wavelet_read_threshold(const WaveletPlan* P, double* out, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(out, &P->d_state->threshold, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}

}  // namespace tomo
