// Forward projection and backprojection for any geometry (tilt axis not vertical,
// full 3-D alignment matrices, scale != 1, non-integral centre offsets): the path
// the separable kernels do not cover.
//
// Both follow the reference's double-precision arithmetic step by step, so which
// samples fall inside the volume or the projection, and every interpolation
// weight, are the reference's:
//   * forward: VoxelProjector3D.projectJosephPartial (TomoJ_Base/.../projectors/
//     VoxelProjector3D.java:671-821) with TomoReconstruction2.getPixel
//     (TomoReconstruction2.java:154-190); one thread per ray, positions stepped in
//     double from the row's 2-row task start exactly as the reference's tasks do;
//   * backward: VoxelProjector3D.backProjectPartial (:221-308) with ImageJ's
//     bilinear getInterpolatedValue; one thread per voxel, every tilt of the update
//     added in order in a register.
// The double stepping makes these kernels FP64-bound; they are the fallback when
// the separable fast path does not apply.
#include <cmath>

#include "tomo_internal.h"

namespace tomo {
namespace {

constexpr int kGThreads = 128;

__device__ __forceinline__ float g_get_pixel(const float* __restrict__ vol, int W, int H, int D, double x, double y,
                                             int z) {
    const int xbase = (x < 0) ? 0 : (int)x;
    const int ybase = (y < 0) ? 0 : (int)y;
    const float* im = vol + (size_t)z * W * H;
    if (xbase == W - 1 || ybase == H - 1 || z == D - 1) return im[xbase + ybase * W];
    const float xf = (x < 0) ? 0.0f : __fsub_rn(__double2float_rn(x), (float)xbase);
    const float yf = (y < 0) ? 0.0f : __fsub_rn(__double2float_rn(y), (float)ybase);
    const int index = ybase * W + xbase;
    const float xyz = im[index];
    const float xy1z = im[index + W];
    const float lower = __fadd_rn(xyz, __fmul_rn(xf, __fsub_rn(im[index + 1], xyz)));
    const float upper = __fadd_rn(xy1z, __fmul_rn(xf, __fsub_rn(im[index + W + 1], xy1z)));
    return __fadd_rn(lower, __fmul_rn(yf, __fsub_rn(upper, lower)));
}

__global__ void __launch_bounds__(kGThreads) fp_generic_kernel(const __grid_constant__ FpGenericLaunch a) {
    const int i = blockIdx.x * kGThreads + threadIdx.x;
    const int j = a.j0 + blockIdx.y;
    const int b = blockIdx.z;
    if (i >= a.w) return;
    const GenericFpTilt gt = a.gtilt[a.tilts[b]];
    // the reference's 2-row task starting at row s steps jcentered from (s - 1 - pc1) / scale
    const int s = a.j0 + 2 * ((j - a.j0) / 2);
    const double jinc = 1.0 / a.scale;
    double jcentered = (s - 1.0 - a.pc0y) / a.scale;
    jcentered = jcentered + jinc;
    if (j == s + 1) jcentered = jcentered + jinc;
    const double icentered = (i - a.pc0x) / a.scale;
    const double ijPartForY = jcentered - gt.icF * icentered;
    double oldy = (ijPartForY - gt.zcF * (-1 - a.vcz)) / gt.divY;
    double oldx = icentered - gt.yFx * oldy - gt.zFx * (-1 - a.vcz);
    oldx = oldx / gt.divX;
    float ray_sum = 0.0f, norm_sum = 0.0f;
    bool entered = false;
    for (int z = 0; z < a.D; z++) {
        const double xc = oldx + gt.dirX;
        const double yc = oldy + gt.dirY;
        const double x = xc + a.vcx;
        const double y = yc + a.vcy;
        if (x + a.acc >= 0 && x < a.bXmax && y + a.acc >= 0 && y < a.bYmax) {
            ray_sum = __fadd_rn(ray_sum, g_get_pixel(a.vol, a.W, a.H, a.D, x, y, z));
            norm_sum = __double2float_rn((double)norm_sum + gt.ninc);
            entered = true;
        } else if (entered) {
            norm_sum = __double2float_rn((double)norm_sum + gt.ninc);
            break;
        }
        oldx = xc;
        oldy = yc;
    }
    const size_t o = ((size_t)b * a.h + j) * a.w + i;
    if (norm_sum > 0) {
        a.proj[o] = __double2float_rn((double)ray_sum * gt.ninc);
        a.norm[o] = norm_sum;
    } else {
        a.proj[o] = __int_as_float(0x7fc00000);
        a.norm[o] = 0.0f;
    }
}

__device__ __forceinline__ double ij_pixel(const float* p, int w, int x, int y) { return (double)p[x + y * w]; }

__device__ __forceinline__ double ij_edge(const float* p, int w, int h, int x, int y) {
    if (x <= 0) x = 0;
    if (x >= w) x = w - 1;
    if (y <= 0) y = 0;
    if (y >= h) y = h - 1;
    return ij_pixel(p, w, x, y);
}

// ImageJ FloatProcessor.getInterpolatedValue(x, y): bilinear, edge values inside the
// last column / row, 0 further out.
__device__ __forceinline__ double ij_interpolated_value(const float* p, int w, int h, double x, double y) {
    double ll, lr, ur, ul, xf, yf;
    if (x < 0.0 || y < 0.0 || x >= w - 1.0 || y >= h - 1.0) {
        if (x < -1.0 || y < -1.0 || x >= w || y >= h) return 0.0;
        const int xbase = (int)floor(x);
        const int ybase = (int)floor(y);
        xf = x - xbase;
        yf = y - ybase;
        if (xf < 0.0) xf = 0.0;
        if (yf < 0.0) yf = 0.0;
        ll = ij_edge(p, w, h, xbase, ybase);
        lr = ij_edge(p, w, h, xbase + 1, ybase);
        ur = ij_edge(p, w, h, xbase + 1, ybase + 1);
        ul = ij_edge(p, w, h, xbase, ybase + 1);
    } else {
        const int xbase = (int)x;
        const int ybase = (int)y;
        xf = x - xbase;
        yf = y - ybase;
        if (xf < 0.0) xf = 0.0;
        if (yf < 0.0) yf = 0.0;
        ll = ij_pixel(p, w, xbase, ybase);
        lr = ij_pixel(p, w, xbase + 1, ybase);
        ur = ij_pixel(p, w, xbase + 1, ybase + 1);
        ul = ij_pixel(p, w, xbase, ybase + 1);
    }
    const double ua = ul + xf * (ur - ul);
    const double la = ll + xf * (lr - ll);
    return la + yf * (ua - la);
}

__global__ void __launch_bounds__(kGThreads) bp_generic_kernel(const __grid_constant__ BpGenericLaunch a) {
    const int i = blockIdx.x * kGThreads + threadIdx.x;
    const int j = a.y0 + blockIdx.y;
    const int k = blockIdx.z;
    if (i >= a.W) return;
    float* vp = a.vol + ((size_t)k * a.H + j) * a.W + i;
    float v = *vp;
    const double x = i - a.vc0, y = j - a.vc1, z = k - a.vc2;
    const size_t npix = (size_t)a.w * a.h;
    for (int b = 0; b < a.T; b++) {
        const double* R = a.euler + 9 * (size_t)a.tilts[b];
        const double ztx = z * R[2];
        const double zty = z * R[5];
        const double ytx = y * R[1];
        const double yty = y * R[4];
        const double xx = (x * R[0] + ytx + ztx) * a.scale + a.cix;
        const double yy = (x * R[3] + yty + zty) * a.scale + a.ciy;
        if (xx >= 0 && xx < a.w && yy >= 0 && yy < a.h) {
            const float value = __double2float_rn(ij_interpolated_value(a.img + b * npix, a.w, a.h, xx, yy));
            if (!isnan(value)) {
                float t = __fadd_rn(v, value);
                if (isnan(t) || isinf(t)) t = 0.0f;
                if (a.positivity && t < 0.0f) t = 0.0f;
                v = t;
            }
        }
    }
    *vp = v;
}

}  // namespace

cudaError_t launch_fp_generic(const FpGenericLaunch& a, cudaStream_t s) {
    if (a.T <= 0 || a.j1 <= a.j0) return cudaSuccess;
    dim3 grid((a.w + kGThreads - 1) / kGThreads, a.j1 - a.j0, a.T);
    fp_generic_kernel<<<grid, kGThreads, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_bp_generic(const BpGenericLaunch& a, cudaStream_t s) {
    if (a.T <= 0 || a.y1 <= a.y0) return cudaSuccess;
    dim3 grid((a.W + kGThreads - 1) / kGThreads, a.y1 - a.y0, a.D);
    bp_generic_kernel<<<grid, kGThreads, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

}  // namespace tomo
