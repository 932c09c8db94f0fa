/*
 * tomo_oracle.c -- CPU restatement of TomoJ's projection / backprojection path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline.  It is never linked into, loaded by, or called from the GPU engine
 * (tomoj_gb300/); only tests/, __graft_entry__.smoke() and bench.py's CPU legs
 * may use it.
 *
 * Parity status: UNPINNED.  The reference (a Java 8 ImageJ plug-in) ships no
 * tests, golden vectors or fixtures for this path, and it cannot be compiled or
 * run without a JDK and its third-party jars.  The restatement is therefore
 * checked against analytic known-answer cases and against an independent FP64
 * numpy twin (oracle/np_oracle.py).
 *
 * Arithmetic follows the Java source operation by operation: float where the
 * reference declares float, double where it declares double, no fused
 * multiply-add (build with -ffp-contract=off), Java's truncating (int) casts,
 * and Java's Math.round.  Reference citations are paths inside the TomoJ tree.
 *
 * Third-party arithmetic that the reference calls and that is absent from its
 * tree is restated from the libraries' published behaviour:
 *   - net.imagej:ij:1.53a  ImageProcessor.getInterpolatedValue(x,y): documented
 *     as bilinear interpolation (the BICUBIC interpolation method set by
 *     VoxelProjector3D.backProjectPartial only affects getInterpolatedPixel),
 *     with clamp-to-edge sampling in the last column/row.
 *   - net.sourceforge.parallelcolt:parallelcolt:0.10.1  DenseFloatMatrix2D
 *     getFft2()/ifft2(true): an unnormalised forward 2-D DFT and a 1/(w*h)
 *     scaled inverse.  Restated as an exact double-precision DFT.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_ACCURACY 1e-10f /* VoxelProjector3D.java:33 (float constant) */

typedef struct {
    int W, H, D;       /* volume width (x), height (y, tilt axis), depth (z) */
    int w, h;          /* projection width, height */
    double vc[3];      /* volume centres, TomoReconstruction2.java:63-66 */
    double pc[4];      /* centerX, centerY, projectionCenterX, projectionCenterY (Projector.java:52-58) */
    double scale;      /* ts.W / rec.W when rescaleData (ReconstructionParameters.java:328) */
    int positivity;    /* VoxelProjector3D.positivityConstraint */
    int long_object;   /* VoxelProjector3D.longObjectCompensation */
} or_geom;

/* ------------------------------------------------------------------------ */
/* Small persistent thread pool: the reference submits 2-row tasks to a      */
/* fixed pool of Prefs.getThreads() workers and waits on every future after  */
/* each projection (VoxelProjector3D.java:162-206, :341-374).                */
/* ------------------------------------------------------------------------ */
typedef void (*or_task_fn)(void* ctx, int task);

typedef struct {
    pthread_t* th;
    int n;
    pthread_mutex_t mu;
    pthread_cond_t cv_work, cv_done;
    or_task_fn fn;
    void* ctx;
    int n_tasks, next_task, done_tasks;
    long generation;
    int quit;
} or_pool;

static or_pool* g_pool = NULL;
static int g_pool_threads = 1;

static void* or_worker(void* arg) {
    or_pool* p = (or_pool*)arg;
    long seen = 0;
    pthread_mutex_lock(&p->mu);
    for (;;) {
        while (!p->quit && p->generation == seen) pthread_cond_wait(&p->cv_work, &p->mu);
        if (p->quit) break;
        seen = p->generation;
        while (p->next_task < p->n_tasks) {
            int t = p->next_task++;
            or_task_fn fn = p->fn;
            void* ctx = p->ctx;
            pthread_mutex_unlock(&p->mu);
            fn(ctx, t);
            pthread_mutex_lock(&p->mu);
            if (++p->done_tasks == p->n_tasks) pthread_cond_broadcast(&p->cv_done);
        }
    }
    pthread_mutex_unlock(&p->mu);
    return NULL;
}

static void or_pool_stop(void) {
    if (!g_pool) return;
    pthread_mutex_lock(&g_pool->mu);
    g_pool->quit = 1;
    pthread_cond_broadcast(&g_pool->cv_work);
    pthread_mutex_unlock(&g_pool->mu);
    for (int i = 0; i < g_pool->n; i++) pthread_join(g_pool->th[i], NULL);
    free(g_pool->th);
    free(g_pool);
    g_pool = NULL;
}

/* Number of worker threads used by every parallel loop (1 = run inline). */
void or_set_threads(int n) {
    if (n < 1) n = 1;
    or_pool_stop();
    g_pool_threads = n;
    if (n == 1) return;
    g_pool = (or_pool*)calloc(1, sizeof(or_pool));
    g_pool->n = n;
    g_pool->th = (pthread_t*)calloc((size_t)n, sizeof(pthread_t));
    pthread_mutex_init(&g_pool->mu, NULL);
    pthread_cond_init(&g_pool->cv_work, NULL);
    pthread_cond_init(&g_pool->cv_done, NULL);
    for (int i = 0; i < n; i++) pthread_create(&g_pool->th[i], NULL, or_worker, g_pool);
}

int or_get_threads(void) { return g_pool_threads; }

static void or_parallel(int n_tasks, or_task_fn fn, void* ctx) {
    if (n_tasks <= 0) return;
    if (!g_pool) {
        for (int t = 0; t < n_tasks; t++) fn(ctx, t);
        return;
    }
    pthread_mutex_lock(&g_pool->mu);
    g_pool->fn = fn;
    g_pool->ctx = ctx;
    g_pool->n_tasks = n_tasks;
    g_pool->next_task = 0;
    g_pool->done_tasks = 0;
    g_pool->generation++;
    pthread_cond_broadcast(&g_pool->cv_work);
    while (g_pool->done_tasks < g_pool->n_tasks) pthread_cond_wait(&g_pool->cv_done, &g_pool->mu);
    pthread_mutex_unlock(&g_pool->mu);
}

/* Java (int) cast of a double: truncation toward zero, NaN -> 0, saturating. */
static inline int jint(double v) {
    if (v != v) return 0;
    if (v >= 2147483647.0) return 2147483647;
    if (v <= -2147483648.0) return (-2147483647 - 1);
    return (int)v;
}

/* Java Math.round(double) as used for int results: floor(x + 0.5). */
static inline int jround(double v) { return jint(floor(v + 0.5)); }

/* ------------------------------------------------------------------------ */
/* Geometry                                                                  */
/* ------------------------------------------------------------------------ */

/* MatrixUtils.eulerAngles2Matrix (Utility/.../MatrixUtils.java:226-251).
 * Row-major 3x3 into R. Angles in degrees. */
void or_euler(double phi, double theta, double psi, double* R) {
    phi = phi * (M_PI / 180.0);
    theta = theta * (M_PI / 180.0);
    psi = psi * (M_PI / 180.0);
    double cphi = cos(phi), sphi = sin(phi);
    double ctheta = cos(theta), stheta = sin(theta);
    double cpsi = cos(psi), spsi = sin(psi);
    R[0] = cpsi * ctheta * cphi - spsi * sphi;
    R[1] = cpsi * ctheta * sphi + spsi * cphi;
    R[2] = -cpsi * stheta;
    R[3] = -spsi * ctheta * cphi - cpsi * sphi;
    R[4] = -spsi * ctheta * sphi + cpsi * cphi;
    R[5] = spsi * stheta;
    R[6] = stheta * cphi;
    R[7] = stheta * sphi;
    R[8] = ctheta;
}

/* ------------------------------------------------------------------------ */
/* Forward projection                                                        */
/* ------------------------------------------------------------------------ */

/* TomoReconstruction2.getPixel(double,double,int), TomoReconstruction2.java:154-190.
 * Bilinear in XY at integer z; raw floor voxel on the last column, row or plane. */
static inline float or_get_pixel(const float* vol, int W, int H, int D, double x, double y, int z) {
    const int xbase = (x < 0) ? 0 : jint(x);
    const int ybase = (y < 0) ? 0 : jint(y);
    const float* im = vol + (size_t)z * W * H;
    if (xbase == W - 1 || ybase == H - 1 || z == D - 1) return im[xbase + ybase * W];
    const float xFraction = (x < 0) ? 0.0f : (float)x - (float)xbase;
    const float yFraction = (y < 0) ? 0.0f : (float)y - (float)ybase;
    const int index = ybase * W + xbase;
    const float xyz = im[index];
    const float xy1z = im[index + W];
    const float lower = xyz + xFraction * (im[index + 1] - xyz);
    return lower + yFraction * ((xy1z + xFraction * (im[index + W + 1] - xy1z)) - lower);
}

/* VoxelProjector3D.projectJosephPartial, VoxelProjector3D.java:671-821 (no mask,
 * no global deformation).  Fills rows [starty,endy) of proj/norm; returns the
 * task's norm maximum (used for long-object compensation). */
static float or_fp_rows(const float* vol, const or_geom* g, const double* R, float* proj, float* norm,
                        int starty, int endy) {
    const int W = g->W, H = g->H, D = g->D, psx = g->w;
    const double icF = R[3] / R[0];
    const double zcF = (R[5] - (R[3] * R[2] / R[0]));
    const double divY = R[4] - (R[3] * R[1] / R[0]);
    const double yFx = R[1], zFx = R[2], divX = R[0];
    const double dirY = -(R[5] - R[3] * R[2] / R[0]) / (R[4] - R[3] * R[1] / R[0]);
    const double dirX = (R[1] * (-dirY) - R[2]) / R[0];
    const double ninc = sqrt(dirX * dirX + dirY * dirY + 1);
    const double vcx = g->vc[0], vcy = g->vc[1], vcz = g->vc[2];
    /* borderXmax = volumeWidth + ACCURACY is an int+float sum in Java: it rounds to (float)W. */
    const double bXmax = (double)((float)W + OR_ACCURACY);
    const double bYmax = (double)((float)H + OR_ACCURACY);
    const double acc = (double)OR_ACCURACY;
    float norm_max = 0;
    int jj = (starty - 1) * psx;
    double jcentered = (starty - 1.0 - g->pc[1]) / g->scale;
    const double jinc = 1.0 / g->scale;
    for (int j = starty; j < endy; j++) {
        jj += psx;
        jcentered += jinc;
        if (j >= 0 && j < g->h) {
            for (int i = 0; i < psx; i++) {
                const double icentered = (i - g->pc[0]) / g->scale;
                float ray_sum = 0, norm_sum = 0;
                const double ijPartForY = jcentered - icF * icentered;
                double oldy = (ijPartForY - zcF * (-1 - vcz)) / divY;
                double oldx = icentered - yFx * oldy - zFx * (-1 - vcz);
                oldx /= divX;
                int entered = 0;
                for (int z = 0; z < D; z++) {
                    const double xc = oldx + dirX;
                    const double yc = oldy + dirY;
                    const double x = xc + vcx;
                    const double y = yc + vcy;
                    if (x + acc >= 0 && x < bXmax && y + acc >= 0 && y < bYmax) {
                        ray_sum += or_get_pixel(vol, W, H, D, x, y, z);
                        norm_sum = (float)((double)norm_sum + ninc);
                        entered = 1;
                    } else if (entered) {
                        norm_sum = (float)((double)norm_sum + ninc);
                        break;
                    }
                    oldx = xc;
                    oldy = yc;
                }
                if (norm_sum > 0) {
                    proj[jj + i] = (float)((double)ray_sum * ninc);
                    norm[jj + i] = norm_sum;
                    if (norm_sum > norm_max) norm_max = norm_sum;
                } else {
                    proj[jj + i] = NAN;
                    norm[jj + i] = 0;
                }
            }
        }
    }
    return norm_max;
}

typedef struct {
    const float* vol;
    const or_geom* g;
    const double* R;
    float* proj;
    float* norm;
    int start, end;
    float* task_max;
} fp_ctx;

static void fp_task(void* c, int t) {
    fp_ctx* x = (fp_ctx*)c;
    int s = x->start + 2 * t;
    int e = (s + 2 < x->g->h) ? s + 2 : x->g->h;
    x->task_max[t] = or_fp_rows(x->vol, x->g, x->R, x->proj, x->norm, s, e);
}

/* VoxelProjector3D.project(startY,endY) for one projection, VoxelProjector3D.java:333-376.
 * proj and norm (w*h) are zeroed here, like the fresh FloatProcessors of the reference.
 * Long-object compensation: the reference lets every 2-row task overwrite the whole
 * norm image with its own maximum (a race); this restatement uses the maximum over
 * the whole projection, the deterministic reading of that code. */
void or_project(const float* vol, const or_geom* g, const double* R, int startY, int endY, float* proj,
                float* norm) {
    (void)endY; /* the reference computes every row from start to the projection height */
    memset(proj, 0, sizeof(float) * (size_t)g->w * g->h);
    memset(norm, 0, sizeof(float) * (size_t)g->w * g->h);
    const int offset = (g->h > g->H && g->scale == 1) ? (g->h - g->H) / 2 : 0;
    const int start = jround((startY + offset) * g->scale);
    const int end = g->h;
    if (start >= end) return;
    int n_tasks = (end - start + 1) / 2;
    float* tmax = (float*)calloc((size_t)n_tasks, sizeof(float));
    fp_ctx c = {vol, g, R, proj, norm, start, end, tmax};
    or_parallel(n_tasks, fp_task, &c);
    if (g->long_object) {
        float m = 0;
        for (int t = 0; t < n_tasks; t++)
            if (tmax[t] > m) m = tmax[t];
        for (size_t i = 0; i < (size_t)g->w * g->h; i++) norm[i] = m;
    }
    free(tmax);
}

/* VoxelProjector3D.difference, VoxelProjector3D.java:414-433.  diff must be zeroed
 * by the caller (a fresh FloatProcessor).  Returns the sum of squared diffs. */
double or_difference(const float* expv, const float* th, const float* norm, float* diff, int n, double factor) {
    double error = 0;
    for (int pos = 0; pos < n; pos++) {
        const float nn = norm[pos];
        const float e = expv[pos];
        const float t = th[pos];
        if (!isnan(e) && !isnan(t)) {
            const float q = (e - t) / nn;
            const double value = (double)q * factor;
            diff[pos] = (float)value;
            error += value * value;
        }
    }
    return error;
}

/* ------------------------------------------------------------------------ */
/* Backprojection                                                            */
/* ------------------------------------------------------------------------ */

static inline double ij_pixel(const float* p, int w, int x, int y) { return (double)p[x + y * w]; }

static inline double ij_edge(const float* p, int w, int h, int x, int y) {
    if (x <= 0) x = 0;
    if (x >= w) x = w - 1;
    if (y <= 0) y = 0;
    if (y >= h) y = h - 1;
    return ij_pixel(p, w, x, y);
}

/* ImageJ 1.53a ImageProcessor.getInterpolatedValue(x,y) on a FloatProcessor:
 * bilinear interpolation; inside the last column/row the edge value is used. */
static inline double ij_interpolated_value(const float* p, int w, int h, double x, double y) {
    if (x < 0.0 || y < 0.0 || x >= w - 1.0 || y >= h - 1.0) {
        if (x < -1.0 || y < -1.0 || x >= w || y >= h) return 0.0;
        const int xbase = jint(floor(x));
        const int ybase = jint(floor(y));
        double xf = x - xbase, yf = y - ybase;
        if (xf < 0.0) xf = 0.0;
        if (yf < 0.0) yf = 0.0;
        const double ll = ij_edge(p, w, h, xbase, ybase);
        const double lr = ij_edge(p, w, h, xbase + 1, ybase);
        const double ur = ij_edge(p, w, h, xbase + 1, ybase + 1);
        const double ul = ij_edge(p, w, h, xbase, ybase + 1);
        const double ua = ul + xf * (ur - ul);
        const double la = ll + xf * (lr - ll);
        return la + yf * (ua - la);
    }
    const int xbase = jint(x);
    const int ybase = jint(y);
    double xf = x - xbase, yf = y - ybase;
    if (xf < 0.0) xf = 0.0;
    if (yf < 0.0) yf = 0.0;
    const double ll = ij_pixel(p, w, xbase, ybase);
    const double lr = ij_pixel(p, w, xbase + 1, ybase);
    const double ur = ij_pixel(p, w, xbase + 1, ybase + 1);
    const double ul = ij_pixel(p, w, xbase, ybase + 1);
    const double ua = ul + xf * (ur - ul);
    const double la = ll + xf * (lr - ll);
    return la + yf * (ua - la);
}

/* VoxelProjector3D.backProjectPartial, VoxelProjector3D.java:221-308 (no mask, no
 * global deformation), for volume rows [starty,endy). */
static void or_bp_rows(float* vol, const or_geom* g, const double* R, const float* proj, int starty, int endy) {
    const double cix = g->pc[2], ciy = g->pc[3];
    const int W = g->W, H = g->H;
    for (int k = 0; k < g->D; k++) {
        const double z = k - g->vc[2];
        float* planez = vol + (size_t)k * W * H;
        for (int j = starty; j < endy; j++) {
            const double y = j - g->vc[1];
            for (int i = 0; i < W; i++) {
                const double x = i - g->vc[0];
                const double ztx = z * R[2];
                const double zty = z * R[5];
                const double ytx = y * R[1];
                const double yty = y * R[4];
                const int jj = j * W;
                const double xx = (x * R[0] + ytx + ztx) * g->scale + cix;
                const double yy = (x * R[3] + yty + zty) * g->scale + ciy;
                if (xx >= 0 && xx < g->w && yy >= 0 && yy < g->h) {
                    const float value = (float)ij_interpolated_value(proj, g->w, g->h, xx, yy);
                    if (!isnan(value)) {
                        float v = planez[i + jj] + value;
                        if (isnan(v)) v = 0;
                        if (isinf(v)) v = 0;
                        if (g->positivity && v < 0) v = 0;
                        planez[i + jj] = v;
                    }
                }
            }
        }
    }
}

typedef struct {
    float* vol;
    const or_geom* g;
    const double* R;
    const float* proj;
    int startY, endY;
} bp_ctx;

static void bp_task(void* c, int t) {
    bp_ctx* x = (bp_ctx*)c;
    int s = x->startY + 2 * t;
    int e = (s + 2 < x->endY) ? s + 2 : x->endY;
    or_bp_rows(x->vol, x->g, x->R, x->proj, s, e);
}

/* Backprojection of one projection into volume rows [startY,endY)
 * (VoxelProjector3D.backproject inner body, VoxelProjector3D.java:167-204). */
void or_backproject(float* vol, const or_geom* g, const double* R, const float* proj, int startY, int endY) {
    if (endY <= startY) return;
    bp_ctx c = {vol, g, R, proj, startY, endY};
    or_parallel((endY - startY + 1) / 2, bp_task, &c);
}

/* ------------------------------------------------------------------------ */
/* Per-tilt 2-D alignment: AffineAlignment.applyTransformOnImage             */
/* (TomoJ_Base/.../align/AffineAlignment.java:136-259).                      */
/* T is java.awt.geom.AffineTransform's flat matrix {m00,m10,m01,m11,m02,m12}.*/
/* fill: 0 = FILL_NONE (zero), 1 = FILL_AVG, 2 = FILL_NaN.                    */
/* Returns 0, or -1 when T is not invertible.                                 */
/* ------------------------------------------------------------------------ */
int or_align(const float* un, int width, int height, const double* T, int normalize, double mean, double stdDev,
             int fill, float* out) {
    const int identity = (T[0] == 1.0 && T[1] == 0.0 && T[2] == 0.0 && T[3] == 1.0 && T[4] == 0.0 && T[5] == 0.0);
    const size_t n = (size_t)width * height;
    if (identity) {
        for (size_t i = 0; i < n; i++) out[i] = normalize ? (float)(((double)un[i] - mean) / stdDev) : un[i];
        return 0;
    }
    memset(out, 0, sizeof(float) * n);
    /* AffineTransform.createInverse, general case */
    const double m00 = T[0], m10 = T[1], m01 = T[2], m11 = T[3], m02 = T[4], m12 = T[5];
    const double det = m00 * m11 - m01 * m10;
    if (fabs(det) <= 4.9e-324) return -1;
    const double i00 = m11 / det, i10 = -m10 / det, i01 = -m01 / det, i11 = m00 / det;
    const double i02 = (m01 * m12 - m11 * m02) / det, i12 = (m10 * m02 - m00 * m12) / det;
    const double centerx = width / 2.0, centery = height / 2.0;
    for (int j = 0; j < height; j++) {
        const int jj = j * width;
        const double jc = j - centery;
        for (int i = 0; i < width; i++) {
            const double px = i - centerx;
            const double xx = (i00 * px + i01 * jc + i02) + centerx;
            const double yy = (i10 * px + i11 * jc + i12) + centery;
            const int ix0 = jint(xx), iy0 = jint(yy);
            const double dx0 = xx - ix0, dy0 = yy - iy0;
            if (ix0 >= 0 && ix0 < width && iy0 >= 0 && iy0 < height) {
                float pix;
                if (ix0 == width - 1 || iy0 == height - 1) {
                    pix = un[ix0 + iy0 * width];
                    if (normalize) pix = (float)(((double)pix - mean) / stdDev);
                } else {
                    const double fac4 = dx0 * dy0;
                    int pos = ix0 + iy0 * width;
                    const float v1 = un[pos];
                    const float v3 = un[pos + width];
                    const float v2 = un[++pos];
                    const float v4 = un[pos + width];
                    pix = (float)(v1 * (1 - dx0 - dy0 + fac4) + v2 * (dx0 - fac4) + v3 * (dy0 - fac4) + v4 * fac4);
                    if (normalize) pix = (float)(((double)pix - mean) / stdDev);
                }
                out[jj + i] = pix;
            } else if (fill == 1) {
                if (!normalize) out[jj + i] = (float)mean;
            } else if (fill == 2) {
                out[jj + i] = NAN;
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* WBP weighting: FFTWeighting (TomoJ_Base/.../filters/FFTWeighting.java)   */
/* ------------------------------------------------------------------------ */

/* FFTWeighting.createWeightingMask, FFTWeighting.java:31-65.  tilt and axis in degrees. */
void or_weighting_mask(int sx, int sy, int nproj, const double* tilt, const double* axis, double diameter,
                       float* mask) {
    const double cx = sx / 2.0, cy = sy / 2.0;
    double* sint = (double*)malloc(sizeof(double) * (size_t)nproj);
    double* cosp = (double*)malloc(sizeof(double) * (size_t)nproj);
    double* sinp = (double*)malloc(sizeof(double) * (size_t)nproj);
    for (int i = 0; i < nproj; i++) {
        sint[i] = sin(tilt[i] * (M_PI / 180.0));
        cosp[i] = cos(axis[i] * (M_PI / 180.0));
        sinp[i] = sin(axis[i] * (M_PI / 180.0));
    }
    for (int j = 0; j < sy; j++) {
        const int jj = j * sx;
        const double cj = (j > cy) ? j - sy : j;
        for (int i = 0; i < sx; i++) {
            const double ci = (i > cx) ? i - sx : i;
            double weight = 0;
            for (int p = 0; p < nproj; p++) {
                const double zj = (ci * sint[p] * cosp[p] + cj * sint[p] * sinp[p]) / sx;
                double value = diameter * M_PI * zj;
                if (value == 0)
                    value = 1;
                else
                    value = sin(value) / value;
                weight += value;
            }
            if (weight < 0.005) weight = (double)0.005f;
            weight *= diameter;
            mask[jj + i] = (float)(1 / weight);
        }
    }
    free(sint);
    free(cosp);
    free(sinp);
}

/* In-place complex DFT of length n (double).  Radix-2 for powers of two, otherwise
 * Bluestein's chirp-z on a radix-2 grid.  sign=-1 forward, +1 inverse (unscaled). */
static void fft_pow2(double* re, double* im, int n, int sign) {
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double t = re[i]; re[i] = re[j]; re[j] = t;
            t = im[i]; im[i] = im[j]; im[j] = t;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        const double ang = sign * 2.0 * M_PI / len;
        for (int i = 0; i < n; i += len) {
            for (int k = 0; k < len / 2; k++) {
                const double wr = cos(ang * k), wi = sin(ang * k);
                const int a = i + k, b = i + k + len / 2;
                const double xr = re[b] * wr - im[b] * wi;
                const double xi = re[b] * wi + im[b] * wr;
                re[b] = re[a] - xr; im[b] = im[a] - xi;
                re[a] += xr; im[a] += xi;
            }
        }
    }
}

static void dft(double* re, double* im, int n, int sign) {
    if (n <= 1) return;
    if ((n & (n - 1)) == 0) { fft_pow2(re, im, n, sign); return; }
    int m = 1;
    while (m < 2 * n - 1) m <<= 1;
    double* ar = (double*)calloc((size_t)m, sizeof(double));
    double* ai = (double*)calloc((size_t)m, sizeof(double));
    double* br = (double*)calloc((size_t)m, sizeof(double));
    double* bi = (double*)calloc((size_t)m, sizeof(double));
    double* cr = (double*)malloc(sizeof(double) * (size_t)n);
    double* ci = (double*)malloc(sizeof(double) * (size_t)n);
    for (int k = 0; k < n; k++) {
        const double ang = sign * M_PI * (double)(((long long)k * k) % (2LL * n)) / n;
        cr[k] = cos(ang); ci[k] = sin(ang);
        ar[k] = re[k] * cr[k] - im[k] * ci[k];
        ai[k] = re[k] * ci[k] + im[k] * cr[k];
    }
    br[0] = cr[0]; bi[0] = -ci[0];
    for (int k = 1; k < n; k++) { br[k] = br[m - k] = cr[k]; bi[k] = bi[m - k] = -ci[k]; }
    fft_pow2(ar, ai, m, -1);
    fft_pow2(br, bi, m, -1);
    for (int k = 0; k < m; k++) {
        const double r = ar[k] * br[k] - ai[k] * bi[k];
        const double i = ar[k] * bi[k] + ai[k] * br[k];
        ar[k] = r; ai[k] = i;
    }
    fft_pow2(ar, ai, m, 1);
    for (int k = 0; k < n; k++) {
        const double r = ar[k] / m, i = ai[k] / m;
        re[k] = r * cr[k] - i * ci[k];
        im[k] = r * ci[k] + i * cr[k];
    }
    free(ar); free(ai); free(br); free(bi); free(cr); free(ci);
}

/* FFTWeighting.weighting, FFTWeighting.java:87-112: forward 2-D DFT, multiply the
 * real and imaginary parts by the mask, scaled inverse 2-D DFT, keep the real part. */
void or_weighting_apply(float* pix, int sx, int sy, const float* mask) {
    const size_t n = (size_t)sx * sy;
    double* re = (double*)malloc(sizeof(double) * n);
    double* im = (double*)calloc(n, sizeof(double));
    int mx = sx > sy ? sx : sy;
    double* tr = (double*)malloc(sizeof(double) * (size_t)mx);
    double* ti = (double*)malloc(sizeof(double) * (size_t)mx);
    for (size_t i = 0; i < n; i++) re[i] = pix[i];
    for (int dir = -1; dir <= 1; dir += 2) {
        for (int j = 0; j < sy; j++) dft(re + (size_t)j * sx, im + (size_t)j * sx, sx, dir);
        for (int i = 0; i < sx; i++) {
            for (int j = 0; j < sy; j++) { tr[j] = re[(size_t)j * sx + i]; ti[j] = im[(size_t)j * sx + i]; }
            dft(tr, ti, sy, dir);
            for (int j = 0; j < sy; j++) { re[(size_t)j * sx + i] = tr[j]; im[(size_t)j * sx + i] = ti[j]; }
        }
        if (dir == -1)
            for (size_t i = 0; i < n; i++) { re[i] *= (double)mask[i]; im[i] *= (double)mask[i]; }
    }
    for (size_t i = 0; i < n; i++) pix[i] = (float)(re[i] / (double)n);
    free(re); free(im); free(tr); free(ti);
}

/* ------------------------------------------------------------------------ */
/* TV denoise: TotalVariationDenoising_3D.denoise3D/updateP/updateU          */
/* (Filters/src/main/java/fr/curie/filters/TotalVariationDenoising_3D.java:84-202). */
/* ------------------------------------------------------------------------ */
typedef struct {
    const float* u;
    float* p;
    int W, H, D;
    float theta, g, dt;
} tvp_ctx;

static void tv_p_task(void* c, int zi) {
    tvp_ctx* a = (tvp_ctx*)c;
    const int W = a->W, H = a->H, D = a->D;
    const int zz = zi + 1; /* 1-based slice index as in the reference */
    const float* u = a->u + (size_t)zi * W * H;
    const float* u1 = a->u + (size_t)((zz + 1 < D ? zz + 1 : D) - 1) * W * H;
    float* p = a->p + (size_t)zi * W * H * 3;
    const float dt = a->dt, theta = a->theta, g = a->g;
    for (int y = 0; y < H; y++) {
        for (int x = 0; x < W; x++) {
            const float duy = (y < H - 1) ? u[x + W * (y + 1)] - u[x + W * y] : 0;
            const float dux = (x < W - 1) ? u[x + 1 + W * y] - u[x + W * y] : 0;
            const float duz = (zz <= D - 1) ? u1[x + W * y] - u[x + W * y] : 0;
            const float dd1 = 1 + dt / theta / g * fabsf((float)sqrt((double)(duy * duy + dux * dux + duz * duz)));
            float* q = p + x * 3 + W * 3 * y;
            q[0] = (q[0] - dt / theta * dux) / dd1;
            q[1] = (q[1] - dt / theta * duy) / dd1;
            q[2] = (q[2] - dt / theta * duz) / dd1;
        }
    }
}

typedef struct {
    const float* f;
    float* u;
    const float* p;
    int W, H, D;
    float theta;
} tvu_ctx;

static void tv_u_task(void* c, int zi) {
    tvu_ctx* a = (tvu_ctx*)c;
    const int W = a->W, H = a->H, D = a->D;
    const int zz = zi + 1;
    const float* p = a->p + (size_t)zi * W * H * 3;
    const float* p_1 = a->p + (size_t)((zz - 1 > 1 ? zz - 1 : 1) - 1) * W * H * 3;
    const float* f = a->f + (size_t)zi * W * H;
    float* u = a->u + (size_t)zi * W * H;
    for (int y = 0; y < H; y++) {
        for (int x = 0; x < W; x++) {
            float div_p;
            if (x == 0) div_p = p[x * 3 + W * 3 * y];
            else if (x == W - 1) div_p = -p[x * 3 + W * 3 * y];
            else div_p = p[x * 3 + W * 3 * y] - p[(x - 1) * 3 + W * 3 * y];
            if (y == 0) div_p += p[x * 3 + 1 + W * 3 * y];
            else if (y == H - 1) div_p += -p[x * 3 + 1 + W * 3 * y];
            else div_p += p[x * 3 + 1 + W * 3 * y] - p[x * 3 + 1 + W * 3 * (y - 1)];
            if (zz == 1) div_p += p[x * 3 + 2 + W * 3 * y];
            else if (zz == D) div_p += -p[x * 3 + 2 + W * 3 * y];
            else div_p += p[x * 3 + 2 + W * 3 * y] - p_1[x * 3 + 2 + W * 3 * y];
            u[x + W * y] = f[x + W * y] - a->theta * div_p;
        }
    }
}

/* denoise3D: u = f, p = 0; iterations x (updateP, updateU); f <- u. */
void or_tv_denoise(float* f, int W, int H, int D, float theta, float g, float dt, int iterations) {
    const size_t n = (size_t)W * H * D;
    float* u = (float*)malloc(sizeof(float) * n);
    float* p = (float*)calloc(n * 3, sizeof(float));
    memcpy(u, f, sizeof(float) * n);
    for (int it = 0; it < iterations; it++) {
        tvp_ctx pc = {u, p, W, H, D, theta, g, dt};
        or_parallel(D, tv_p_task, &pc);
        tvu_ctx uc = {f, u, p, W, H, D, theta};
        or_parallel(D, tv_u_task, &uc);
    }
    memcpy(f, u, sizeof(float) * n);
    free(u);
    free(p);
}

/* ------------------------------------------------------------------------ */
/* OS-SART driver (TomoReconstruction2.java:548-781)                         */
/* ------------------------------------------------------------------------ */

/* orderShuffleART (TomoReconstruction2.java:735-781) with the random first index
 * replaced by `first`.  euler: nproj row-major 3x3 matrices. */
void or_order_shuffle(int nproj, const double* euler, int first, int* indexes) {
    char* todo = (char*)malloc((size_t)nproj);
    memset(todo, 1, (size_t)nproj);
    int cc = 0, im = first;
    while (cc < nproj) {
        if (cc != 0) {
            double mini = 1.7976931348623157e308;
            int omini = -1;
            const double* a = euler + 9 * im + 6;
            for (int o = 0; o < nproj; o++) {
                if (todo[o]) {
                    const double* b = euler + 9 * o + 6;
                    const double sp = fabs(a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
                    if (sp < mini) { mini = sp; omini = o; }
                }
            }
            im = omini;
        }
        if (todo[im]) { indexes[cc] = im; todo[im] = 0; cc++; }
    }
    free(todo);
}

/* One OS-SART iteration over aligned measured projections `meas` (nproj*w*h).
 * Follows osartIteration (TomoReconstruction2.java:636-733) with the projector
 * calls of VoxelProjector3D.  order: the projection order for this iteration.
 * err5 receives {average, min, argmin, max, argmax} as the reference computes them.
 * err_per_proj (nproj, may be NULL) receives each projection's sum of squares. */
static void ossart_iteration_into(float* vol, float* bp_vol, const or_geom* g, const double* euler,
                                  const float* meas, int nproj, const int* order, double relax, int update,
                                  int startY, int endY, double* err5, double* err_per_proj);

void or_ossart_iteration(float* vol, const or_geom* g, const double* euler, const float* meas, int nproj,
                         const int* order, double relax, int update, int startY, int endY, double* err5,
                         double* err_per_proj) {
    ossart_iteration_into(vol, vol, g, euler, meas, nproj, order, relax, update, startY, endY, err5, err_per_proj);
}

/* The same iteration projecting `vol` but backprojecting into `bp_vol`
 * (BayesianVoxelProjector3D.backproject adds the differences to its distance
 * volume, BayesianVoxelProjector3D.java:77-116). */
void or_ossart_iteration_into(float* vol, float* bp_vol, const or_geom* g, const double* euler, const float* meas,
                              int nproj, const int* order, double relax, int update, int startY, int endY,
                              double* err5) {
    ossart_iteration_into(vol, bp_vol, g, euler, meas, nproj, order, relax, update, startY, endY, err5, NULL);
}

static void ossart_iteration_into(float* vol, float* bp_vol, const or_geom* g, const double* euler,
                                  const float* meas, int nproj, const int* order, double relax, int update,
                                  int startY, int endY, double* err5, double* err_per_proj) {
    const int upd = (update == 0) ? nproj : update;
    const float factorimg = (float)(relax / upd);
    const size_t npix = (size_t)g->w * g->h;
    float* proj = (float*)malloc(sizeof(float) * npix * (size_t)upd);
    float* norm = (float*)malloc(sizeof(float) * npix * (size_t)upd);
    float* diff = (float*)malloc(sizeof(float) * npix * (size_t)upd);
    int* batch = (int*)malloc(sizeof(int) * (size_t)upd);
    int diffIndex = 0;
    double som = 0, errmin = 3.4028234663852886e38, errmax = 0;
    int imin = 0, imax = 0;
    for (int t = 0; t < nproj; t++) {
        batch[diffIndex++] = order[t];
        if (diffIndex == upd || t == nproj - 1) {
            for (int e = 0; e < diffIndex; e++) {
                const int p = batch[e];
                or_project(vol, g, euler + 9 * p, startY, endY, proj + npix * e, norm + npix * e);
                memset(diff + npix * e, 0, sizeof(float) * npix);
                const double err = or_difference(meas + npix * p, proj + npix * e, norm + npix * e, diff + npix * e,
                                                 (int)npix, (double)factorimg);
                if (err_per_proj) err_per_proj[p] = err;
                som += err;
                if (err > errmax) { errmax = err; imax = order[t - diffIndex + e + 1]; }
                else if (err < errmin) { errmin = err; imin = order[t - diffIndex + e + 1]; }
            }
            for (int e = 0; e < diffIndex; e++)
                or_backproject(bp_vol, g, euler + 9 * batch[e], diff + npix * e, startY, endY);
            diffIndex = 0;
        }
    }
    if (err5) {
        err5[0] = sqrt(som / (double)((long long)nproj * g->W * g->H));
        err5[1] = sqrt(errmin / (double)(g->W * g->H));
        err5[2] = imin;
        err5[3] = sqrt(errmax / (double)(g->W * g->H));
        err5[4] = imax;
    }
    free(proj); free(norm); free(diff); free(batch);
}

/* WBP(ts, projector, params, startY, endY) with update 0 (TomoReconstruction2.java:499-538):
 * every projection (optionally weighted in place with `mask`) is backprojected alone,
 * in index order.  meas is modified when mask != NULL (the reference weights the
 * projector's own copy). */
void or_wbp(float* vol, const or_geom* g, const double* euler, float* meas, int nproj, const float* mask,
            int startY, int endY) {
    const size_t npix = (size_t)g->w * g->h;
    for (int p = 0; p < nproj; p++) {
        if (mask) or_weighting_apply(meas + npix * p, g->w, g->h, mask);
        or_backproject(vol, g, euler + 9 * p, meas + npix * p, startY, endY);
    }
}

/* FistaProjector3D.endOfIteration momentum step (FistaProjector3D.java:43-59):
 * t <- (1+sqrt(1+4t^2))/2 ; rec += ((t_prev-1)/t) (rec - prev).  Returns new t. */
double or_fista_step(float* rec, const float* prev, size_t n, double t) {
    const double t_1 = t;
    t = (1 + sqrt(1 + 4 * t * t)) / 2;
    const double factor = (t_1 - 1) / t;
    for (size_t i = 0; i < n; i++) {
        /* getPixel() values are floats, so the difference is a float subtraction;
         * addToPixel skips NaN and adds (float)value (TomoReconstruction2.java:365-370). */
        const double val = factor * (double)(rec[i] - prev[i]);
        if (!isnan(val)) rec[i] = rec[i] + (float)val;
    }
    return t;
}

/* ------------------------------------------------------------------------ */
/* BayesianVoxelProjector3D (TomoJ_AdvancedReconstruction/.../projectors/    */
/* BayesianVoxelProjector3D.java).                                           */
/* ------------------------------------------------------------------------ */

/* startOfIteration -> convolve(rec, kernel, distanceVolume, -lambda) (:131-134, :168-194):
 * dist = (float)(factor * sum_n neighbour_n * kernel_n) over the 3x3x3 neighbourhood of
 * TomoReconstruction2.getCubicNeightborhoodWithClamp (TomoReconstruction2.java:317-339),
 * which reads getPixel(x+i, y+j, z+k) for i, j, k = -1..1 (i outermost): despite its
 * name, out-of-volume neighbours are 0 (getPixel, :241-246).  The kernel is
 * [1,-2,1] x [1,-2,1] x [1,-2,1]; products are float, the sum double. */
void or_bayes_start(const float* rec, float* dist, int W, int H, int D, double lambda) {
    static const float kern[27] = {1, -2, 1, -2, 4, -2, 1, -2, 1, -2, 4, -2, 4, -8, 4, -2, 4, -2,
                                   1, -2, 1, -2, 4, -2, 1, -2, 1};
    const double factor = -lambda;
    for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                double total = 0;
                int idx = 0;
                for (int i = -1; i <= 1; i++)
                    for (int j = -1; j <= 1; j++)
                        for (int k = -1; k <= 1; k++) {
                            const int xx = x + i, yy = y + j, zz = z + k;
                            float v = 0.0f;
                            if (xx >= 0 && xx < W && yy >= 0 && yy < H && zz >= 0 && zz < D)
                                v = rec[((size_t)zz * H + yy) * W + xx];
                            total += (double)(v * kern[idx++]);
                        }
                dist[((size_t)z * H + y) * W + x] = (float)(total * factor);
            }
}

/* endOfIteration (:119-129): distanceVolume *= alpha (FloatProcessor.multiply: float
 * pixel times double, rounded to float), rec += distanceVolume (FloatBlitter.ADD,
 * float), then the positivity constraint (FloatBlitter.MAX with zeros) when set. */
void or_bayes_end(float* rec, float* dist, size_t n, double alpha, int positivity) {
    for (size_t i = 0; i < n; i++) {
        dist[i] = (float)((double)dist[i] * alpha);
        float v = dist[i] + rec[i];
        if (positivity && 0.0f > v) v = 0.0f;
        rec[i] = v;
    }
}

/* ------------------------------------------------------------------------ */
/* BgARTVoxelProjector3D (TomoJ_AdvancedReconstruction/.../projectors/       */
/* BgARTVoxelProjector3D.java).                                              */
/* ------------------------------------------------------------------------ */

/* Stack histogram as ImageJ's StackStatistics computes it for 32-bit data (ij 1.53a,
 * a dependency absent from the reference tree; restated from its documented
 * behaviour): min and max over the non-NaN voxels, 256 bins over [min, max], bin
 * (int)((v - min) * (256 / (max - min))) clamped to 255; every voxel falls in bin 0
 * when max == min. */
static void ij_stack_histogram(const float* v, size_t n, double* mn, double* mx, long long* hist) {
    double lo = INFINITY, hi = -INFINITY;
    for (size_t i = 0; i < n; i++) {
        if (isnan(v[i])) continue;
        if (v[i] < lo) lo = v[i];
        if (v[i] > hi) hi = v[i];
    }
    memset(hist, 0, sizeof(long long) * 256);
    const double scale = 256.0 / (hi - lo);
    for (size_t i = 0; i < n; i++) {
        if (isnan(v[i])) continue;
        int b = 0;
        if (hi > lo) {
            b = jint((v[i] - lo) * scale);
            if (b > 255) b = 255;
        }
        hist[b]++;
    }
    *mn = lo;
    *mx = hi;
}

/* collapseFilter (:29-90): the background is the histogram mode (or bgValue when it is
 * not NaN), sigma the spread of the bins below the mode around it; with a dark
 * background every voxel below mode + k sigma becomes the background, otherwise every
 * voxel above mode - k sigma.  Returns the background value. */
double or_bgart_collapse(float* vol, size_t n, double k, int dark_bg, double bg_value) {
    long long hist[256];
    double histmin, histmax;
    ij_stack_histogram(vol, n, &histmin, &histmax, hist);
    const double bin = (histmax - histmin) / 256;
    double best = 0;
    int max_index = 0;
    for (int i = 0; i < 256; i++)
        if ((double)hist[i] > best) {
            best = (double)hist[i];
            max_index = i;
        }
    const double bg = isnan(bg_value) ? histmin + max_index * bin : bg_value;
    double sigma = 0;
    long long count = 0;
    for (int i = 0; i < max_index; i++) {
        const double d = histmin + i * bin - bg;
        sigma += d * d * (double)hist[i];
        count += hist[i];
    }
    sigma = sqrt(sigma / (double)count);
    const double th1 = bg - k * sigma, th2 = bg + k * sigma;
    for (size_t i = 0; i < n; i++) {
        const double val = vol[i];
        if (dark_bg && val < th2) vol[i] = (float)bg;
        if (!dark_bg && val > th1) vol[i] = (float)bg;
    }
    return bg;
}

/* Java's Arrays.sort(float[]) order as an unsigned key: -0.0 before 0.0, NaN last. */
static inline uint32_t java_float_key(float f) {
    uint32_t b;
    if (isnan(f)) return 0xFFFFFFFFu;
    memcpy(&b, &f, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

/* medianFilter3Dcross (:117-145): median of the voxel, its two z neighbours (0 outside
 * the stack) and four in-plane neighbours addressed by flat index within the slice,
 * so x neighbours wrap across rows, indices must be > 0 for the -1 and -W neighbours
 * and < W*H for the +1 and +W neighbours (0 otherwise); all reads from a copy. */
void or_bgart_median_cross(float* vol, int W, int H, int D) {
    const size_t P = (size_t)W * H, n = P * D;
    float* tmp = (float*)malloc(sizeof(float) * n);
    memcpy(tmp, vol, sizeof(float) * n);
    for (int z = 0; z < D; z++) {
        const float* cur = tmp + P * z;
        const float* lo = z > 0 ? tmp + P * (z - 1) : NULL;
        const float* hi = z < D - 1 ? tmp + P * (z + 1) : NULL;
        for (long long idx = 0; idx < (long long)P; idx++) {
            float nb[7];
            nb[0] = lo ? lo[idx] : 0.0f;
            nb[1] = hi ? hi[idx] : 0.0f;
            nb[2] = cur[idx];
            nb[3] = (idx + 1 < (long long)P) ? cur[idx + 1] : 0.0f;
            nb[4] = (idx - 1 > 0) ? cur[idx - 1] : 0.0f;
            nb[5] = (idx - W > 0) ? cur[idx - W] : 0.0f;
            nb[6] = (idx + W < (long long)P) ? cur[idx + W] : 0.0f;
            /* insertion sort by Java's float order */
            for (int a = 1; a < 7; a++) {
                const float f = nb[a];
                const uint32_t kf = java_float_key(f);
                int b = a - 1;
                while (b >= 0 && java_float_key(nb[b]) > kf) {
                    nb[b + 1] = nb[b];
                    b--;
                }
                nb[b + 1] = f;
            }
            vol[P * z + idx] = nb[3];
        }
    }
    free(tmp);
}
