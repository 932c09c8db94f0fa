// Supporting kernels: per-tilt alignment resample, WBP row filter (batched FFT),
// deterministic residual reductions, TV denoise stencils, FISTA momentum, fills
// and the long-object normalisation.  The library is compiled with -fmad=false,
// so every a*b+c here rounds twice like the Java reference unless fmaf is used.
#include <cmath>

#include "device_util.cuh"
#include "tomo_internal.h"

namespace tomo {
namespace {

// AffineAlignment.applyTransformOnImage (TomoJ_Base/.../align/AffineAlignment.java:136-259):
// inverse-map every output pixel through Tinv around (w/2, h/2), Java (int) truncation,
// bilinear in double with the floor pixel on the last row/column, optional
// (x - mean) / stdDev, and the TiltSeries fill policy outside the image.
__global__ void align_kernel(const float* __restrict__ raw, float* __restrict__ out, const double* __restrict__ tinv,
                             const double* __restrict__ stats, int w, int h, int normalize, int fill,
                             const unsigned char* __restrict__ identity) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    const int t = blockIdx.z;
    if (i >= w) return;
    const float* un = raw + (size_t)t * w * h;
    const double mean = stats ? stats[2 * t] : 0.0;
    const double sd = stats ? stats[2 * t + 1] : 1.0;
    float pix;
    if (identity[t]) {
        const float v = un[(size_t)j * w + i];
        pix = normalize ? __double2float_rn(__ddiv_rn(__dsub_rn((double)v, mean), sd)) : v;
    } else {
        const double* T = tinv + 6 * t;  // {i00, i10, i01, i11, i02, i12}
        const double cx = w / 2.0, cy = h / 2.0;
        const double px = (double)i - cx, jc = (double)j - cy;
        const double xx = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(T[0], px), __dmul_rn(T[2], jc)), T[4]), cx);
        const double yy = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(T[1], px), __dmul_rn(T[3], jc)), T[5]), cy);
        const int ix0 = __double2int_rz(xx), iy0 = __double2int_rz(yy);
        const double dx0 = __dsub_rn(xx, (double)ix0), dy0 = __dsub_rn(yy, (double)iy0);
        if (ix0 >= 0 && ix0 < w && iy0 >= 0 && iy0 < h) {
            if (ix0 == w - 1 || iy0 == h - 1) {
                pix = un[ix0 + (size_t)iy0 * w];
            } else {
                const double fac4 = __dmul_rn(dx0, dy0);
                const size_t pos = ix0 + (size_t)iy0 * w;
                const double v1 = un[pos], v3 = un[pos + w], v2 = un[pos + 1], v4 = un[pos + 1 + w];
                const double w1 = __dadd_rn(__dsub_rn(__dsub_rn(1.0, dx0), dy0), fac4);
                const double acc = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(v1, w1), __dmul_rn(v2, __dsub_rn(dx0, fac4))),
                                                       __dmul_rn(v3, __dsub_rn(dy0, fac4))),
                                             __dmul_rn(v4, fac4));
                pix = __double2float_rn(acc);
            }
            if (normalize) pix = __double2float_rn(__ddiv_rn(__dsub_rn((double)pix, mean), sd));
        } else if (fill == 1) {
            pix = normalize ? 0.0f : __double2float_rn(mean);
        } else if (fill == 2) {
            pix = __int_as_float(0x7fc00000);
        } else {
            pix = 0.0f;
        }
    }
    out[(size_t)t * w * h + (size_t)j * w + i] = pix;
}

// --- WBP row filter --------------------------------------------------------------
// FFTWeighting.weighting (FFTWeighting.java:87-112) multiplies the 2-D spectrum by
// a mask that, for a zero tilt-axis angle, depends on the column frequency only;
// the 2-D filter is then exactly a filter of every row.  Two real rows are packed
// into one complex sequence (the mask is real and even, so the packed halves
// stay separate), transformed by an in-shared-memory radix-2 FFT, multiplied by
// the mask, transformed back and scaled by 1/w.
__device__ __forceinline__ unsigned bitrev(unsigned v, int bits) { return __brev(v) >> (32 - bits); }

__device__ void fft_stages(float2* s, const float2* __restrict__ tw, int n, int logn, bool inverse) {
    for (int len = 2, stage = 0; len <= n; len <<= 1, stage++) {
        const int half = len >> 1;
        const int tstride = n / len;
        __syncthreads();
        for (int b = threadIdx.x; b < n / 2; b += blockDim.x) {
            const int grp = b / half, k = b % half;
            const int ia = grp * len + k, ib = ia + half;
            float2 wv = tw[k * tstride];
            if (inverse) wv.y = -wv.y;
            const float2 xb = s[ib], xa = s[ia];
            const float2 t = make_float2(xb.x * wv.x - xb.y * wv.y, xb.x * wv.y + xb.y * wv.x);
            s[ib] = make_float2(xa.x - t.x, xa.y - t.y);
            s[ia] = make_float2(xa.x + t.x, xa.y + t.y);
        }
    }
    __syncthreads();
}

// bad (optional): per-image flag of a non-finite pixel.  The reference's 2-D transform
// spreads one NaN or Inf over the whole image; a row filter alone would keep it in
// its row, so rows of a flagged image are written as NaN.
__device__ __forceinline__ bool image_bad(const int* bad, int row, int rows_per_img) {
    return bad != nullptr && bad[row / rows_per_img] != 0;
}

__global__ void row_filter_kernel(float* img, const float* __restrict__ mask, const float2* __restrict__ tw, int rows,
                                  int n, int logn, const int* __restrict__ bad, int rows_per_img) {
    extern __shared__ float2 sbuf[];
    float2* a = sbuf;
    float2* b = sbuf + n;
    const int r0 = 2 * blockIdx.x, r1 = r0 + 1;
    float* row0 = img + (size_t)r0 * n;
    float* row1 = (r1 < rows) ? img + (size_t)r1 * n : nullptr;
    for (int k = threadIdx.x; k < n; k += blockDim.x)
        a[bitrev(k, logn)] = make_float2(row0[k], row1 ? row1[k] : 0.0f);
    fft_stages(a, tw, n, logn, false);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const float m = mask[k];
        const float2 v = a[k];
        b[bitrev(k, logn)] = make_float2(v.x * m, v.y * m);
    }
    fft_stages(b, tw, n, logn, true);
    const float inv = 1.0f / (float)n;
    const bool bad0 = image_bad(bad, r0, rows_per_img), bad1 = row1 && image_bad(bad, r1, rows_per_img);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        row0[k] = bad0 ? __int_as_float(0x7fc00000) : b[k].x * inv;
        if (row1) row1[k] = bad1 ? __int_as_float(0x7fc00000) : b[k].y * inv;
    }
}

// Any width: the row filter is a circular convolution of length w with the real
// kernel h = IDFT_w(mask).  Rows are laid out twice ([row, row], the periodic
// extension) in a zero-padded power-of-two buffer of M >= 2w - 1 points; the linear
// convolution with h (spectrum H, M points) equals the circular one on outputs
// [w, 2w).  Two real rows are packed into one complex sequence as above (h is real).
__global__ void row_filter_conv_kernel(float* img, const float2* __restrict__ H, const float2* __restrict__ tw, int rows,
                                       int w, int M, int logM, const int* __restrict__ bad, int rows_per_img) {
    extern __shared__ float2 sbuf[];
    float2* a = sbuf;
    const int r0 = 2 * blockIdx.x, r1 = r0 + 1;
    float* row0 = img + (size_t)r0 * w;
    float* row1 = (r1 < rows) ? img + (size_t)r1 * w : nullptr;
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        float2 v = make_float2(0.0f, 0.0f);
        if (k < 2 * w) {
            const int m = k < w ? k : k - w;
            v = make_float2(row0[m], row1 ? row1[m] : 0.0f);
        }
        a[bitrev(k, logM)] = v;
    }
    fft_stages(a, tw, M, logM, false);
    float2* b = sbuf + M;
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        const float2 v = a[k], f = H[k];
        b[bitrev(k, logM)] = make_float2(v.x * f.x - v.y * f.y, v.x * f.y + v.y * f.x);
    }
    fft_stages(b, tw, M, logM, true);
    const float inv = 1.0f / (float)M;
    const bool bad0 = image_bad(bad, r0, rows_per_img), bad1 = row1 && image_bad(bad, r1, rows_per_img);
    for (int k = threadIdx.x; k < w; k += blockDim.x) {
        row0[k] = bad0 ? __int_as_float(0x7fc00000) : b[w + k].x * inv;
        if (row1) row1[k] = bad1 ? __int_as_float(0x7fc00000) : b[w + k].y * inv;
    }
}

// --- 2-D weighting (tilt axis not vertical) ----------------------------------------
// FFTWeighting.weighting (FFTWeighting.java:87-112) with a mask that depends on both
// frequencies: forward DFT of every row, transpose, per column (now a row) forward
// DFT, multiply by the mask, inverse DFT, transpose back, inverse DFT of every row,
// real part scaled by 1/(w h).  Each transform runs in shared memory: radix-2 when
// the length is a power of two, otherwise Bluestein's chirp-z algorithm on a radix-2
// grid of M >= 2n - 1 points:
//   X[k] = c[k] * sum_j (x[j] c[j]) conj(c[k - j]),  c[j] = exp(-i pi j^2 / n),
// the convolution done by an M-point FFT with the precomputed spectrum of the
// wrapped conj(c).  Inverse transforms are conj(DFT(conj(x))).
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Forward DFT (conjugated on input and output when conj_io: the inverse) of x[0, n)
// in shared memory, in place; a and b are M-point work buffers.
__device__ void dft_row(float2* x, float2* a, float2* b, const DftRowPlan& P, bool conj_io) {
    const int n = P.n, M = P.M, logM = P.logM;
    const float cs = conj_io ? -1.0f : 1.0f;
    if (M == n) {
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            const float2 v = x[k];
            a[bitrev(k, logM)] = make_float2(v.x, cs * v.y);
        }
        fft_stages(a, P.tw, M, logM, false);
        for (int k = threadIdx.x; k < n; k += blockDim.x) x[k] = make_float2(a[k].x, cs * a[k].y);
        __syncthreads();
        return;
    }
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        float2 v = make_float2(0.0f, 0.0f);
        if (k < n) v = cmulf(make_float2(x[k].x, cs * x[k].y), P.chirp[k]);
        a[bitrev(k, logM)] = v;
    }
    fft_stages(a, P.tw, M, logM, false);
    for (int k = threadIdx.x; k < M; k += blockDim.x) b[bitrev(k, logM)] = cmulf(a[k], P.bspec[k]);
    fft_stages(b, P.tw, M, logM, true);
    const float inv = 1.0f / (float)M;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const float2 v = cmulf(b[k], P.chirp[k]);
        x[k] = make_float2(v.x * inv, cs * v.y * inv);
    }
    __syncthreads();
}

// MODE 0: real rows -> spectra; 1: spectra x mask row (row index mod mask_rows),
// inverse; 2: spectra -> real rows (real part x scale).  One row per CTA.
template <int MODE>
__global__ void dft2_rows_kernel(const float* __restrict__ rin, float2* cio, float* rout, const float* __restrict__ mask,
                                 DftRowPlan P, int mask_rows, float scale) {
    extern __shared__ float2 sbuf[];
    float2* x = sbuf;
    float2* a = sbuf + P.n;
    float2* b = a + P.M;
    const size_t r = blockIdx.x;
    const int n = P.n;
    for (int k = threadIdx.x; k < n; k += blockDim.x)
        x[k] = MODE == 0 ? make_float2(rin[r * n + k], 0.0f) : cio[r * n + k];
    __syncthreads();
    dft_row(x, a, b, P, MODE == 2);
    if (MODE == 1) {
        const float* m = mask + (size_t)(r % (size_t)mask_rows) * n;
        for (int k = threadIdx.x; k < n; k += blockDim.x) x[k] = make_float2(x[k].x * m[k], x[k].y * m[k]);
        __syncthreads();
        dft_row(x, a, b, P, true);
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        if (MODE == 2)
            rout[r * n + k] = x[k].x * scale;
        else
            cio[r * n + k] = x[k];
    }
}

// [T][R][C] -> [T][C][R], 32 x 32 tiles.
__global__ void transpose_c_kernel(const float2* __restrict__ in, float2* __restrict__ out, int R, int Cc) {
    __shared__ float2 tile[32][33];
    const size_t base = (size_t)blockIdx.z * R * Cc;
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int r = r0 + dy, c = c0 + threadIdx.x;
        if (r < R && c < Cc) tile[dy][threadIdx.x] = in[base + (size_t)r * Cc + c];
    }
    __syncthreads();
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int c = c0 + dy, r = r0 + threadIdx.x;
        if (r < R && c < Cc) out[base + (size_t)c * R + r] = tile[threadIdx.x][dy];
    }
}

// bad[t] = 1 when image t holds a NaN or an Inf.
__global__ void image_nonfinite_kernel(const float* __restrict__ imgs, size_t npix, int* bad) {
    const float* im = imgs + (size_t)blockIdx.y * npix;
    int f = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix; i += (size_t)gridDim.x * blockDim.x)
        f |= !isfinite(im[i]);
    f = __reduce_or_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && f) atomicOr(bad + blockIdx.y, 1);
}

// Sum over rows of the per-row residuals, one thread per tilt, fixed order.
// Sum of one projection's per-row residual sums by one warp: lane l adds rows
// l, l + 32, ... in order, then a fixed butterfly combines the lanes (deterministic).
__device__ __forceinline__ double warp_row_sum(const double* __restrict__ rows, int h) {
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    for (int j = lane; j < h; j += 32) s += rows[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

constexpr int kErrWarps = 4;  // projections per 128-thread block

__global__ void reduce_err_kernel(const double* __restrict__ errpart, double* __restrict__ err, int T, int h) {
    const int t = blockIdx.x * kErrWarps + (threadIdx.x >> 5);
    if (t >= T) return;
    const double s = warp_row_sum(errpart + (size_t)t * h, h);
    if ((threadIdx.x & 31) == 0) err[t] = s;
}

__global__ void reduce_err_batch_kernel(const ErrReduce* __restrict__ jobs) {
    const ErrReduce j = jobs[blockIdx.y];
    const int t = blockIdx.x * kErrWarps + (threadIdx.x >> 5);
    if (t >= j.T) return;
    const double s = warp_row_sum(j.errpart + (size_t)t * j.h, j.h);
    if ((threadIdx.x & 31) == 0) j.err[t] = s;
}

// TotalVariationDenoising_3D (Filters/.../TotalVariationDenoising_3D.java:84-202): inner
// steps of updateP (:115-156) then updateU (:158-202), fused.  The step k -> k + 1 needs
// u_k = f - theta * div p_k only where updateP reads it (the voxel and its +x, +y, +z
// neighbours), so one kernel rebuilds u_k plane by plane in shared memory from p_k and f
// and writes p_{k+1}; u itself is never stored between steps.  p is double-buffered
// (a CTA reads p_k of its -x / -y / -z neighbours while others write p_{k+1}).  Every
// value is computed with updateU's and updateP's float expressions in their order, so
// the result is the unfused sequence's bit for bit.

// u = f - theta * div p at flat index o = (z, y, x), with updateU's boundary rules.
__device__ __forceinline__ float tv_u_point(const float* f, const float* __restrict__ px, const float* __restrict__ py,
                                            const float* __restrict__ pz, size_t o, int x, int y, int z, int W, int H,
                                            int D, float theta) {
    float div;
    if (x == 0) div = px[o];
    else if (x == W - 1) div = -px[o];
    else div = px[o] - px[o - 1];
    if (y == 0) div += py[o];
    else if (y == H - 1) div += -py[o];
    else div += py[o] - py[o - W];
    if (z == 0) div += pz[o];
    else if (z == D - 1) div += -pz[o];
    else div += pz[o] - pz[o - (size_t)W * H];
    return f[o] - theta * div;
}

constexpr int kTvX = 32, kTvY = 8, kTvZ = 32;  // CTA: 32 x 8 columns, marching 32 planes
// One thread per element of the tile and its +x / +y halo (33 x 9): every u of a plane is
// one thread's, computed once.  A thread keeps its column's p_k of the current plane in
// registers (the update reads them, and pz of the plane is the next plane's -z neighbour),
// so a plane costs it f, px, py, pz and the -x / -y neighbours (L1 hits of the adjacent
// threads' loads).
constexpr int kTvFX = kTvX + 1, kTvFY = kTvY + 1, kTvThreads = kTvFX * kTvFY;

// One inner step: p_b = updateP(u_a, p_a) with u_a = updateU(f, p_a); FIRST: p_a = 0, u_a = f.
template <bool FIRST>
__global__ void __launch_bounds__(kTvThreads) tv_step_kernel(const float* __restrict__ f, const float* __restrict__ pxa,
                                                           const float* __restrict__ pya, const float* __restrict__ pza,
                                                           float* __restrict__ pxb, float* __restrict__ pyb,
                                                           float* __restrict__ pzb, int W, int H, int D, float theta,
                                                           float g, float dt) {
    __shared__ float us[2][kTvFY][kTvFX];  // u of planes z and z + 1 over the tile and its halo
    const int lx = threadIdx.x % kTvFX, ly = threadIdx.x / kTvFX;
    const int x = blockIdx.x * kTvX + lx, y = blockIdx.y * kTvY + ly;
    const int z0 = blockIdx.z * kTvZ, z1 = min(z0 + kTvZ, D);
    const size_t WH = (size_t)W * H;
    const bool in = x < W && y < H;
    const bool inner = in && lx < kTvX && ly < kTvY;  // writes p_b
    const float k = dt / theta;
    // A plane's inputs are loaded one iteration before its u is computed, so the loads
    // overlap the update of the plane before.
    struct In {
        float f, px, py, pz, pxm, pym;  // pxm / pym: the -x / -y neighbours' p (0 where unused)
    };
    auto load = [&](int z) -> In {
        In v{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        if (!in) return v;
        const size_t o = (size_t)z * WH + (size_t)y * W + x;
        v.f = f[o];
        if (!FIRST) {
            v.px = pxa[o];
            v.py = pya[o];
            v.pz = pza[o];
            if (x > 0 && x < W - 1) v.pxm = pxa[o - 1];
            if (y > 0 && y < H - 1) v.pym = pya[o - W];
        }
        return v;
    };
    // pz of this column at the plane before the one whose u is computed next
    float pzm = 0.0f;
    if (!FIRST && in && z0 > 0 && z0 < D - 1) pzm = pza[(size_t)(z0 - 1) * WH + (size_t)y * W + x];
    // u from loaded inputs (updateU's expressions and order, as tv_u_point)
    auto u_of = [&](const In& v, int z) -> float {
        if (!in) return 0.0f;
        if (FIRST) return v.f;
        float div;
        if (x == 0) div = v.px;
        else if (x == W - 1) div = -v.px;
        else div = v.px - v.pxm;
        if (y == 0) div += v.py;
        else if (y == H - 1) div += -v.py;
        else div += v.py - v.pym;
        if (z == 0) div += v.pz;
        else if (z == D - 1) div += -v.pz;
        else div += v.pz - pzm;
        pzm = v.pz;
        return v.f - theta * div;
    };
    In c = load(z0);                             // plane z0
    In nx = z0 + 1 < D ? load(z0 + 1) : c;      // plane z0 + 1, in flight
    us[0][ly][lx] = u_of(c, z0);
    int cur = 0;
    for (int z = z0; z < z1; z++) {
        const float cpx = c.px, cpy = c.py, cpz = c.pz;  // p_a at (x, y, z)
        if (z + 1 < D) {
            us[cur ^ 1][ly][lx] = u_of(nx, z + 1);
            c = nx;
            if (z + 2 < D && z + 1 < z1) nx = load(z + 2);
        }
        __syncthreads();
        if (inner) {
            const size_t o = (size_t)z * WH + (size_t)y * W + x;
            const float u0 = us[cur][ly][lx];
            const float duy = (y < H - 1) ? us[cur][ly + 1][lx] - u0 : 0.0f;
            const float dux = (x < W - 1) ? us[cur][ly][lx + 1] - u0 : 0.0f;
            const float duz = (z < D - 1) ? us[cur ^ 1][ly][lx] - u0 : 0.0f;
            const float s = duy * duy + dux * dux + duz * duz;
            const float dd1 = 1.0f + dt / theta / g * fabsf(__fsqrt_rn(s));
            pxb[o] = __fdiv_rn(cpx - k * dux, dd1);
            pyb[o] = __fdiv_rn(cpy - k * duy, dd1);
            pzb[o] = __fdiv_rn(cpz - k * duz, dd1);
        }
        __syncthreads();
        cur ^= 1;
    }
}

// The closing updateU, in place: fu holds f and receives u (each voxel reads only its own f).
__global__ void tv_final_kernel(float* fu, const float* __restrict__ px, const float* __restrict__ py,
                                const float* __restrict__ pz, int W, int H, int D, float theta) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= W) return;
    const size_t o = ((size_t)z * H + y) * W + x;
    fu[o] = tv_u_point(fu, px, py, pz, o, x, y, z, W, H, D, theta);
}

__global__ void fill_kernel(float* p, size_t n, float v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// FistaProjector3D.endOfIteration (FistaProjector3D.java:43-59) with addToPixel's NaN skip.
__global__ void fista_kernel(float* rec, const float* __restrict__ prev, size_t n, double factor) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double val = __dmul_rn(factor, (double)(rec[i] - prev[i]));
        if (!isnan(val)) rec[i] = rec[i] + __double2float_rn(val);
    }
}

// BayesianVoxelProjector3D.startOfIteration -> convolve(rec, kernel, distanceVolume, -lambda)
// (TomoJ_AdvancedReconstruction/.../projectors/BayesianVoxelProjector3D.java:131-134, 168-194):
// the 27-point stencil [1,-2,1]^3 over TomoReconstruction2.getCubicNeightborhoodWithClamp
// (TomoReconstruction2.java:317-339), whose out-of-volume neighbours read 0 through getPixel;
// float products (exact: the weights are powers of two) summed in double in the reference's
// neighbour order (x offset outermost, z innermost), times factor, rounded to float.
__global__ void bayes_conv_kernel(const float* __restrict__ rec, float* __restrict__ dist, int W, int H, int D,
                                  double factor) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= W) return;
    const float k1[3] = {1.0f, -2.0f, 1.0f};
    double total = 0.0;
#pragma unroll
    for (int i = -1; i <= 1; i++)
#pragma unroll
        for (int j = -1; j <= 1; j++)
#pragma unroll
            for (int k = -1; k <= 1; k++) {
                const int xx = x + i, yy = y + j, zz = z + k;
                float v = 0.0f;
                if (xx >= 0 && xx < W && yy >= 0 && yy < H && zz >= 0 && zz < D)
                    v = rec[((size_t)zz * H + yy) * W + xx];
                total = __dadd_rn(total, (double)__fmul_rn(v, k1[i + 1] * k1[j + 1] * k1[k + 1]));
            }
    dist[((size_t)z * H + y) * W + x] = __double2float_rn(__dmul_rn(total, factor));
}

// BayesianVoxelProjector3D.endOfIteration (:119-129): distance *= alpha (float pixel times
// double, rounded to float), volume += distance (float), then positivity (max with 0).
__global__ void bayes_apply_kernel(float* rec, float* dist, size_t n, double alpha, int positivity) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float d = __double2float_rn(__dmul_rn((double)dist[i], alpha));
        dist[i] = d;
        float v = __fadd_rn(d, rec[i]);
        if (positivity && 0.0f > v) v = 0.0f;
        rec[i] = v;
    }
}

// ---- BgARTVoxelProjector3D (TomoJ_AdvancedReconstruction/.../BgARTVoxelProjector3D.java) ----

// Order-preserving unsigned key of a float (-0.0 before 0.0), and back.
__device__ __forceinline__ unsigned float_key(float f) {
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_float(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}
// Java's Arrays.sort(float[]) order: as float_key, with NaN last.
__device__ __forceinline__ unsigned java_sort_key(float f) { return isnan(f) ? 0xFFFFFFFFu : float_key(f); }

// keys[0] = min key, keys[1] = max key over the non-NaN voxels (keys preset to ~0 / 0).
__global__ void bg_minmax_kernel(const float* __restrict__ v, size_t n, unsigned* keys) {
    unsigned lo = 0xFFFFFFFFu, hi = 0u;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float f = v[i];
        if (isnan(f)) continue;
        const unsigned k = float_key(f);
        lo = min(lo, k);
        hi = max(hi, k);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(keys, lo);
        atomicMax(keys + 1, hi);
    }
}

// ImageJ StackStatistics histogram of 32-bit data: 256 bins over [min, max], bin
// (int)((v - min) * (256 / (max - min))) clamped to 255, all in bin 0 when max == min.
__global__ void bg_hist_kernel(const float* __restrict__ v, size_t n, const unsigned* keys,
                               unsigned long long* hist) {
    __shared__ unsigned h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const double lo = key_float(keys[0]), hi = key_float(keys[1]);
    const double scale = __ddiv_rn(256.0, hi - lo);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float f = v[i];
        if (isnan(f)) continue;
        int b = 0;
        if (hi > lo) {
            b = (int)__dmul_rn((double)f - lo, scale);  // truncation toward zero, as Java's (int)
            if (b > 255) b = 255;
        }
        atomicAdd(&h[b], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        if (h[i]) atomicAdd(hist + i, (unsigned long long)h[i]);
}

// collapseFilter thresholds (:29-83) in one thread: out = {background, th1, th2}.
__global__ void bg_finalize_kernel(const unsigned* keys, const unsigned long long* hist, double k, double bg_value,
                                   double* out) {
    const double histmin = key_float(keys[0]), histmax = key_float(keys[1]);
    const double bin = (histmax - histmin) / 256;
    double best = 0;
    int max_index = 0;
    for (int i = 0; i < 256; i++)
        if ((double)hist[i] > best) {
            best = (double)hist[i];
            max_index = i;
        }
    const double bg = isnan(bg_value) ? __dadd_rn(histmin, __dmul_rn((double)max_index, bin)) : bg_value;
    double sigma = 0;
    long long count = 0;
    for (int i = 0; i < max_index; i++) {
        const double d = __dsub_rn(__dadd_rn(histmin, __dmul_rn((double)i, bin)), bg);
        sigma = __dadd_rn(sigma, __dmul_rn(__dmul_rn(d, d), (double)hist[i]));
        count += (long long)hist[i];
    }
    sigma = __dsqrt_rn(__ddiv_rn(sigma, (double)count));
    out[0] = bg;
    out[1] = __dsub_rn(bg, __dmul_rn(k, sigma));
    out[2] = __dadd_rn(bg, __dmul_rn(k, sigma));
}

__global__ void bg_apply_kernel(float* v, size_t n, const double* out, int dark_bg) {
    const double bg = out[0], th1 = out[1], th2 = out[2];
    const float bgf = __double2float_rn(bg);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double val = v[i];
        if (dark_bg && val < th2) v[i] = bgf;
        if (!dark_bg && val > th1) v[i] = bgf;
    }
}

// medianFilter3Dcross (:117-145) from the copy `src` into `dst`: the voxel, its z
// neighbours (0 outside) and its in-plane neighbours by flat index within the slice
// (x neighbours wrap across rows; -1 / -W need an index > 0, +1 / +W one < W*H).
__global__ void median_cross_kernel(const float* __restrict__ src, float* __restrict__ dst, int W, int H, int D) {
    const long long P = (long long)W * H;
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    if (idx >= P) return;
    const float* cur = src + P * z;
    float nb[7];
    nb[0] = z > 0 ? cur[idx - P] : 0.0f;
    nb[1] = z < D - 1 ? cur[idx + P] : 0.0f;
    nb[2] = cur[idx];
    nb[3] = (idx + 1 < P) ? cur[idx + 1] : 0.0f;
    nb[4] = (idx - 1 > 0) ? cur[idx - 1] : 0.0f;
    nb[5] = (idx - W > 0) ? cur[idx - W] : 0.0f;
    nb[6] = (idx + W < P) ? cur[idx + W] : 0.0f;
    unsigned key[7];
#pragma unroll
    for (int a = 0; a < 7; a++) key[a] = java_sort_key(nb[a]);
    // rank selection: the element with 3 keys below it (ties broken by position) is the median
    float med = nb[0];
#pragma unroll
    for (int a = 0; a < 7; a++) {
        int below = 0;
#pragma unroll
        for (int b = 0; b < 7; b++) below += (key[b] < key[a]) || (key[b] == key[a] && b < a);
        if (below == 3) med = nb[a];
    }
    dst[P * z + idx] = med;
}

// Long-object compensation: every norm pixel of a projection becomes the projection's maximum.
__global__ void long_object_kernel(float* norm, int npix) {
    __shared__ float red[32];
    float* n = norm + (size_t)blockIdx.x * npix;
    float m = 0.0f;
    for (int i = threadIdx.x; i < npix; i += blockDim.x) m = fmaxf(m, n[i]);
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = (threadIdx.x < blockDim.x / 32) ? red[threadIdx.x] : 0.0f;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) red[0] = m;
    }
    __syncthreads();
    m = red[0];
    for (int i = threadIdx.x; i < npix; i += blockDim.x) n[i] = m;
}

// VoxelProjector3D.difference (VoxelProjector3D.java:414-433) over precomputed projections
// (used when long-object compensation replaces the norms after projection).
__global__ void diff_kernel(const float* __restrict__ meas, const int* __restrict__ tilts, const float* __restrict__ th,
                            const float* __restrict__ norm, float* __restrict__ diff, double* __restrict__ errpart,
                            int w, int h, int j0, int j1, double factor) {
    __shared__ double red[32];
    const int b = blockIdx.y;
    const int j = blockIdx.x;
    double e2 = 0.0;
    if (j >= j0 && j < j1) {
        const float* e = meas + ((size_t)tilts[b] * h + j) * w;
        const size_t o = ((size_t)b * h + j) * w;
        for (int i = threadIdx.x; i < w; i += blockDim.x) {
            const float ev = e[i], tv = th[o + i];
            float d = 0.0f;
            if (!isnan(ev) && !isnan(tv)) {
                const float q = __fdiv_rn(ev - tv, norm[o + i]);
                const double v = (double)q * factor;
                d = __double2float_rn(v);
                e2 += v * v;
            }
            diff[o + i] = d;
        }
    } else {
        const size_t o = ((size_t)b * h + j) * w;
        for (int i = threadIdx.x; i < w; i += blockDim.x) diff[o + i] = 0.0f;
    }
    e2 = warp_sum(e2);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < (int)blockDim.x / 32; k++) s += red[k];
        errpart[(size_t)b * h + j] = s;
    }
}

// Copies image tilts[b] of src into slot b of dst (addProjection's fresh copy).
__global__ void gather_kernel(float* __restrict__ dst, const float* __restrict__ src, const int* __restrict__ tilts,
                              size_t npix) {
    const int b = blockIdx.y;
    const float* s = src + (size_t)tilts[b] * npix;
    float* d = dst + (size_t)b * npix;
    if ((npix & 3) == 0) {  // every image starts 16-byte aligned
        const float4* s4 = reinterpret_cast<const float4*>(s);
        float4* d4 = reinterpret_cast<float4*>(d);
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix / 4;
             i += (size_t)gridDim.x * blockDim.x)
            d4[i] = s4[i];
    } else {
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix; i += (size_t)gridDim.x * blockDim.x)
            d[i] = s[i];
    }
}

// flags[0] |= 1 if any NaN, flags[0] |= 2 if any +-Inf.
__global__ void scan_nonfinite_kernel(const float* __restrict__ p, size_t n, int* flags) {
    int f = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float v = p[i];
        if (isnan(v)) f |= 1;
        else if (isinf(v)) f |= 2;
    }
    f = __reduce_or_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && f) atomicOr(flags, f);
}

}  // namespace

cudaError_t misc_init_attributes() {
    cudaError_t e = cudaFuncSetAttribute(row_filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         2 * 4096 * (int)sizeof(float2));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(row_filter_conv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             2 * kRowConvMaxM * (int)sizeof(float2));
    if (e != cudaSuccess) return e;
    const int dft_smem = (kDft2MaxN + 2 * kRowConvMaxM) * (int)sizeof(float2);
    e = cudaFuncSetAttribute(dft2_rows_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, dft_smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(dft2_rows_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, dft_smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(dft2_rows_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, dft_smem);
}

int device_sms() {
    constexpr int kMaxDevices = 64;
    static std::atomic<int> cache[kMaxDevices];  // 0: not queried yet
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return 1;
    }
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v > 0) return v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
        cudaGetLastError();
        v = 1;
    }
    cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

cudaError_t launch_gather(float* dst, const float* src, const int* tilts, int T, size_t npix, cudaStream_t s) {
    if (T <= 0) return cudaSuccess;
    dim3 grid((unsigned)std::min<size_t>((npix / 4 + 255) / 256 + 1, 64), T);
    gather_kernel<<<grid, 256, 0, s>>>(dst, src, tilts, npix);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_scan_nonfinite(const float* p, size_t n, int* flags, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, device_sms() * 8);
    scan_nonfinite_kernel<<<blocks, 256, 0, s>>>(p, n, flags);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_align(const float* raw, float* out, const double* tinv, const double* stats, int N, int w, int h,
                         int normalize, int fill, const unsigned char* identity, cudaStream_t s) {
    dim3 grid((w + 127) / 128, h, N);
    align_kernel<<<grid, 128, 0, s>>>(raw, out, tinv, stats, w, h, normalize, fill, identity);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_row_filter_tw(float* img, const float* mask_row, const float2* tw, int rows, int w,
                                 const int* bad, int rows_per_img, cudaStream_t s) {
    int logn = 0;
    while ((1 << logn) < w) logn++;
    if ((1 << logn) != w) return cudaErrorInvalidValue;
    const size_t smem = 2 * (size_t)w * sizeof(float2);
    row_filter_kernel<<<(rows + 1) / 2, 256, smem, s>>>(img, mask_row, tw, rows, w, logn, bad, rows_per_img);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_row_filter_conv(float* img, const float2* H, const float2* tw, int rows, int w, int M,
                                   const int* bad, int rows_per_img, cudaStream_t s) {
    int logM = 0;
    while ((1 << logM) < M) logM++;
    if ((1 << logM) != M || M < 2 * w - 1 || M > kRowConvMaxM) return cudaErrorInvalidValue;
    const size_t smem = 2 * (size_t)M * sizeof(float2);
    row_filter_conv_kernel<<<(rows + 1) / 2, 256, smem, s>>>(img, H, tw, rows, w, M, logM, bad, rows_per_img);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_image_nonfinite(const float* imgs, int T, size_t npix, int* bad, cudaStream_t s) {
    if (T <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(int) * (size_t)T, s);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)std::min<size_t>((npix + 255) / 256, 32), T);
    image_nonfinite_kernel<<<grid, 256, 0, s>>>(imgs, npix, bad);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_weighting_2d(float* imgs, int T, int w, int h, const float* maskT, const DftRowPlan& Pw,
                                const DftRowPlan& Ph, float2* sa, float2* sb, cudaStream_t s) {
    if (T <= 0) return cudaSuccess;
    if (Pw.n != w || Ph.n != h || w > kDft2MaxN || h > kDft2MaxN || T > 65535) return cudaErrorInvalidValue;
    const size_t smw = (size_t)(Pw.n + 2 * Pw.M) * sizeof(float2);
    const size_t smh = (size_t)(Ph.n + 2 * Ph.M) * sizeof(float2);
    const float scale = (float)(1.0 / ((double)w * (double)h));
    const dim3 tb(32, 8);
    dft2_rows_kernel<0><<<(unsigned)T * h, 256, smw, s>>>(imgs, sa, nullptr, nullptr, Pw, 1, 1.0f);
    count_launch();
    transpose_c_kernel<<<dim3((w + 31) / 32, (h + 31) / 32, T), tb, 0, s>>>(sa, sb, h, w);
    count_launch();
    dft2_rows_kernel<1><<<(unsigned)T * w, 256, smh, s>>>(nullptr, sb, nullptr, maskT, Ph, w, 1.0f);
    count_launch();
    transpose_c_kernel<<<dim3((h + 31) / 32, (w + 31) / 32, T), tb, 0, s>>>(sb, sa, w, h);
    count_launch();
    dft2_rows_kernel<2><<<(unsigned)T * h, 256, smw, s>>>(nullptr, sa, imgs, nullptr, Pw, 1, scale);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_reduce_err(const double* errpart, double* err, int T, int h, cudaStream_t s) {
    if (T <= 0) return cudaSuccess;
    reduce_err_kernel<<<(T + kErrWarps - 1) / kErrWarps, 32 * kErrWarps, 0, s>>>(errpart, err, T, h);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_reduce_err_batch(const ErrReduce* jobs, int n_jobs, int max_T, cudaStream_t s) {
    if (n_jobs <= 0) return cudaSuccess;
    reduce_err_batch_kernel<<<dim3((max_T + kErrWarps - 1) / kErrWarps, n_jobs), 32 * kErrWarps, 0, s>>>(jobs);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_tv_step(const float* f, const float* const pa[3], float* const pb[3], bool first, int W, int H,
                           int D, float theta, float g, float dt, cudaStream_t s) {
    dim3 grid((W + kTvX - 1) / kTvX, (H + kTvY - 1) / kTvY, (D + kTvZ - 1) / kTvZ);
    if (first)
        tv_step_kernel<true><<<grid, kTvThreads, 0, s>>>(f, pa[0], pa[1], pa[2], pb[0], pb[1], pb[2], W, H, D, theta,
                                                         g, dt);
    else
        tv_step_kernel<false><<<grid, kTvThreads, 0, s>>>(f, pa[0], pa[1], pa[2], pb[0], pb[1], pb[2], W, H, D, theta,
                                                          g, dt);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_tv_final(float* fu, const float* const p[3], int W, int H, int D, float theta, cudaStream_t s) {
    dim3 grid((W + 127) / 128, H, D);
    tv_final_kernel<<<grid, 128, 0, s>>>(fu, p[0], p[1], p[2], W, H, D, theta);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_fill(float* p, size_t n, float v, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, device_sms() * 16);
    fill_kernel<<<blocks, 256, 0, s>>>(p, n, v);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_fista(float* rec, const float* prev, size_t n, double factor, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, device_sms() * 16);
    fista_kernel<<<blocks, 256, 0, s>>>(rec, prev, n, factor);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_bayes_conv(const float* rec, float* dist, int W, int H, int D, double factor, cudaStream_t s) {
    dim3 grid((W + 127) / 128, H, D);
    bayes_conv_kernel<<<grid, 128, 0, s>>>(rec, dist, W, H, D, factor);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_bayes_apply(float* rec, float* dist, size_t n, double alpha, int positivity, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, device_sms() * 16);
    bayes_apply_kernel<<<blocks, 256, 0, s>>>(rec, dist, n, alpha, positivity);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_bgart_collapse(float* vol, size_t n, double k, int dark_bg, double bg_value, void* scratch,
                                  cudaStream_t s) {
    unsigned* keys = static_cast<unsigned*>(scratch);
    unsigned long long* hist = reinterpret_cast<unsigned long long*>(static_cast<char*>(scratch) + 16);
    double* out = reinterpret_cast<double*>(static_cast<char*>(scratch) + 16 + 256 * 8);
    cudaError_t e;
    if ((e = cudaMemsetAsync(keys, 0xFF, 4, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(keys + 1, 0, 4, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(hist, 0, 256 * 8, s)) != cudaSuccess) return e;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, device_sms() * 8);
    bg_minmax_kernel<<<blocks, 256, 0, s>>>(vol, n, keys);
    bg_hist_kernel<<<blocks, 256, 0, s>>>(vol, n, keys, hist);
    bg_finalize_kernel<<<1, 1, 0, s>>>(keys, hist, k, bg_value, out);
    bg_apply_kernel<<<blocks, 256, 0, s>>>(vol, n, out, dark_bg);
    count_launch(4);
    return cudaGetLastError();
}

cudaError_t launch_bgart_median(float* vol, float* tmp, int W, int H, int D, cudaStream_t s) {
    const size_t n = (size_t)W * H * D;
    cudaError_t e = cudaMemcpyAsync(tmp, vol, sizeof(float) * n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    const long long P = (long long)W * H;
    median_cross_kernel<<<dim3((unsigned)((P + 255) / 256), D), 256, 0, s>>>(tmp, vol, W, H, D);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_long_object(float* norm, int T, int h, int w, cudaStream_t s) {
    if (T <= 0) return cudaSuccess;
    long_object_kernel<<<T, 512, 0, s>>>(norm, h * w);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_diff(const float* meas, const int* tilts, const float* th, const float* norm, float* diff,
                        double* errpart, int T, int w, int h, int j0, int j1, double factor, cudaStream_t s) {
    if (T <= 0) return cudaSuccess;
    diff_kernel<<<dim3(h, T), 256, 0, s>>>(meas, tilts, th, norm, diff, errpart, w, h, j0, j1, factor);
    count_launch();
    return cudaGetLastError();
}

}  // namespace tomo
