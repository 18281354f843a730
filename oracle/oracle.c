/*
 * oracle.c -- CPU oracle for the recon dense RGB-D tracking hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline).  Each
 * function restates one reference kernel or host routine of ttykkala/recon and
 * cites the file:line it follows.  FP32 expressions are written in the
 * reference's source order; the library is compiled with -ffp-contract=off so
 * that no multiply-add is fused implicitly (the canonical lane sums below call
 * fmaf explicitly).  Reductions follow the canonical chunked tree
 * described at orc_reduce27; the tracker folds its FP32 warp values exactly in
 * fixed point (orc_reduce27_fx), the reference-named shim in FP64 order
 * (orc_reduce27).  The reference's own order is available as
 * orc_reduce27_refordered for comparison.
 */
#define _POSIX_C_SOURCE 200809L
#include "oracle.h"
#include "../recon_gb300/csrc/scene.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KR_OFFSET ORC_KR_OFFSET
#define KCR_OFFSET ORC_KCR_OFFSET
#define TLR_OFFSET ORC_TLR_OFFSET
#define KL_OFFSET ORC_KL_OFFSET
#define MIND_OFFSET ORC_MIND_OFFSET
#define MAXD_OFFSET ORC_MAXD_OFFSET
#define TRL_OFFSET ORC_TRL_OFFSET

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* float -> int truncation toward zero; NaN / out of range map to INT_MIN so that
 * a degenerate projection is always "out of view" (the reference converts NaN
 * to 0 on the GPU; this only matters for non-finite coordinates). */
static inline int ftoi(float x) {
    if (!(x > -2147483520.0f && x < 2147483520.0f)) return INT_MIN;
    return (int)x;
}

/* ------------------------------------------------------------------ */
/* small vector helpers, kernels/kernelUtils.h                         */
/* ------------------------------------------------------------------ */

/* matrixMultVec4, kernelUtils.h:224-229 */
static inline void mul4(const float *M, const float *v, float *r) {
    r[0] = M[0] * v[0] + M[1] * v[1] + M[2] * v[2] + M[3];
    r[1] = M[4] * v[0] + M[5] * v[1] + M[6] * v[2] + M[7];
    r[2] = M[8] * v[0] + M[9] * v[1] + M[10] * v[2] + M[11];
}

/* matrixRot4 / rotate3Cuda, kernelUtils.h:69-73, 231-236 */
static inline void rot4(const float *M, const float *v, float *r) {
    r[0] = M[0] * v[0] + M[1] * v[1] + M[2] * v[2];
    r[1] = M[4] * v[0] + M[5] * v[1] + M[6] * v[2];
    r[2] = M[8] * v[0] + M[9] * v[1] + M[10] * v[2];
}

/* matrixMultVec3, kernelUtils.h:217-222 */
static inline void mul3(const float *M, const float *v, float *r) {
    r[0] = M[0] * v[0] + M[1] * v[1] + M[2] * v[2];
    r[1] = M[3] * v[0] + M[4] * v[1] + M[5] * v[2];
    r[2] = M[6] * v[0] + M[7] * v[1] + M[8] * v[2];
}

/* distortPoint, kernelUtils.h:394-408 */
static inline void distort(float pux, float puy, const float *kc, const float *K, float *pdx, float *pdy) {
    float dx = pux * pux;
    float dy = puy * puy;
    float r2 = dx + dy;
    float r4 = r2 * r2;
    float r6 = r4 * r2;
    float radialDist = 1 + kc[0] * r2 + kc[1] * r4 + kc[4] * r6;
    *pdx = K[0] * pux * radialDist + K[2];
    *pdy = K[4] * puy * radialDist + K[5];
}

/* bilinearInterpolation(int,int,float,float,...), kernelUtils.h:298-303 */
static inline float bilin(int xdi, int ydi, float fx, float fy, int width, const float *src) {
    int offset2 = xdi + ydi * width;
    float v0 = src[offset2];
    float v1 = src[offset2 + 1];
    float v2 = src[offset2 + width];
    float v3 = src[offset2 + width + 1];
    return (1 - fx) * (1 - fy) * v0 + fx * (1 - fy) * v1 + (1 - fx) * fy * v2 + fx * fy * v3;
}

/* Same formula with tap coordinates clamped into a w x h image.  Used where the
 * reference reads outside the image (coarsest pyramid level of
 * addVertexAttributesWithoutNormalsKernel4, d2z.cu:805-936); inside the image it
 * is identical to bilin(). */
static inline float bilin_clamped(int xdi, int ydi, float fx, float fy, int w, int h, const float *src) {
    int x0 = xdi < 0 ? 0 : (xdi > w - 1 ? w - 1 : xdi);
    int x1 = xdi + 1 < 0 ? 0 : (xdi + 1 > w - 1 ? w - 1 : xdi + 1);
    int y0 = ydi < 0 ? 0 : (ydi > h - 1 ? h - 1 : ydi);
    int y1 = ydi + 1 < 0 ? 0 : (ydi + 1 > h - 1 ? h - 1 : ydi + 1);
    float v0 = src[x0 + y0 * w];
    float v1 = src[x1 + y0 * w];
    float v2 = src[x0 + y1 * w];
    float v3 = src[x1 + y1 * w];
    return (1 - fx) * (1 - fy) * v0 + fx * (1 - fy) * v1 + (1 - fx) * fy * v2 + fx * fy * v3;
}

/* inBounds, kernelUtils.h:341-344 */
static inline int in_bounds10(float px, float py, int w, int h) {
    return (px >= 10 && px < (w - 10) && py >= 10 && py < (h - 10));
}

/* normalize3Cuda, kernelUtils.h:41-50 */
static inline void normalize3(float *v) {
    float len = 0.0f;
    len += v[0] * v[0];
    len += v[1] * v[1];
    len += v[2] * v[2];
    len = 1.0f / sqrtf(len);
    v[0] *= len;
    v[1] *= len;
    v[2] *= len;
}

/* ------------------------------------------------------------------ */
/* calibration, calib/calib.cpp:74-93                                  */
/* ------------------------------------------------------------------ */

static void inverse3x3f(const float *m, float *r) {
    /* precomputed inverse (iKR / iKL); not read by any kernel on the tracking path */
    double det = (double)m[0] * ((double)m[4] * m[8] - (double)m[5] * m[7]) -
                 (double)m[1] * ((double)m[3] * m[8] - (double)m[5] * m[6]) +
                 (double)m[2] * ((double)m[3] * m[7] - (double)m[4] * m[6]);
    if (fabs(det) < 1e-5) {
        memset(r, 0, 9 * sizeof(float));
        r[0] = r[4] = r[8] = 1.0f;
        return;
    }
    r[0] = (float)(((double)m[4] * m[8] - (double)m[5] * m[7]) / det);
    r[1] = (float)(-((double)m[1] * m[8] - (double)m[7] * m[2]) / det);
    r[2] = (float)(((double)m[1] * m[5] - (double)m[4] * m[2]) / det);
    r[3] = (float)(-((double)m[3] * m[8] - (double)m[5] * m[6]) / det);
    r[4] = (float)(((double)m[0] * m[8] - (double)m[6] * m[2]) / det);
    r[5] = (float)(-((double)m[0] * m[5] - (double)m[3] * m[2]) / det);
    r[6] = (float)(((double)m[3] * m[7] - (double)m[6] * m[4]) / det);
    r[7] = (float)(-((double)m[0] * m[7] - (double)m[6] * m[1]) / det);
    r[8] = (float)(((double)m[0] * m[4] - (double)m[3] * m[1]) / det);
}

/* invertRT4(double), tracker/basic_math.cpp:335-353 */
static void invert_rt4d(const double *M, double *Mi) {
    Mi[0] = M[0]; Mi[1] = M[4]; Mi[2] = M[8];   Mi[3] = -(M[0] * M[3] + M[4] * M[7] + M[8] * M[11]);
    Mi[4] = M[1]; Mi[5] = M[5]; Mi[6] = M[9];   Mi[7] = -(M[1] * M[3] + M[5] * M[7] + M[9] * M[11]);
    Mi[8] = M[2]; Mi[9] = M[6]; Mi[10] = M[10]; Mi[11] = -(M[2] * M[3] + M[6] * M[7] + M[10] * M[11]);
    Mi[12] = 0;   Mi[13] = 0;   Mi[14] = 0;     Mi[15] = 1;
}

/* invertRT4Cuda, kernelUtils.h:100-107 */
static void invert_rt4f(const float *M, float *Mi) {
    Mi[0] = M[0]; Mi[1] = M[4]; Mi[2] = M[8];   Mi[3] = -(M[0] * M[3] + M[4] * M[7] + M[8] * M[11]);
    Mi[4] = M[1]; Mi[5] = M[5]; Mi[6] = M[9];   Mi[7] = -(M[1] * M[3] + M[5] * M[7] + M[9] * M[11]);
    Mi[8] = M[2]; Mi[9] = M[6]; Mi[10] = M[10]; Mi[11] = -(M[2] * M[3] + M[6] * M[7] + M[10] * M[11]);
    Mi[12] = 0;   Mi[13] = 0;   Mi[14] = 0;     Mi[15] = 1;
}

void orc_calib_setup(const double KL[9], const double KR[9], const double TLR[16], const double kcR[8],
                     double minDist, double maxDist, double c0, double c1, int width, float *calib) {
    memset(calib, 0, ORC_CALIB_SIZE * sizeof(float));
    /* identity3x3 then the first two rows scaled by the image width (calib.cpp:77-78) */
    for (int i = 0; i < 9; i++) calib[KR_OFFSET + i] = (i % 4 == 0) ? 1.0f : 0.0f;
    for (int i = 0; i < 6; i++) calib[KR_OFFSET + i] = (float)(width * KR[i]);
    inverse3x3f(&calib[KR_OFFSET], &calib[ORC_IKR_OFFSET]);
    for (int i = 0; i < 8; i++) calib[KCR_OFFSET + i] = (float)kcR[i];
    double TRL[16];
    invert_rt4d(TLR, TRL);
    for (int i = 0; i < 16; i++) {
        calib[TLR_OFFSET + i] = (float)TLR[i];
        calib[TRL_OFFSET + i] = (float)TRL[i];
    }
    for (int i = 0; i < 9; i++) calib[KL_OFFSET + i] = (i % 4 == 0) ? 1.0f : 0.0f;
    for (int i = 0; i < 6; i++) calib[KL_OFFSET + i] = (float)(width * KL[i]);
    inverse3x3f(&calib[KL_OFFSET], &calib[ORC_IKL_OFFSET]);
    calib[ORC_C0_OFFSET] = (float)c0;
    calib[ORC_C1_OFFSET] = (float)c1;
    calib[MIND_OFFSET] = (float)minDist;
    calib[MAXD_OFFSET] = (float)maxDist;
}

/* ------------------------------------------------------------------ */
/* input conversion and pyramids                                       */
/* ------------------------------------------------------------------ */

/* gray in [0,1]: the reference reads a float RGBA texture already in [0,1]
 * (rgb2gray.cu:64-76); uint8 input maps to it by /255. */
void orc_convert_gray(const uint8_t *g, int n, float *out) {
    for (int i = 0; i < n; i++) out[i] = (float)g[i] / 255.0f;
}

/* z = -depth_mm (rgb2gray.cu:75 stores negative metric depth); 0 = invalid */
void orc_convert_depth(const uint16_t *d, int n, float *z) {
    for (int i = 0; i < n; i++) z[i] = d[i] ? -(float)d[i] : 0.0f;
}

/* rgbTex2GrayHdrZKernel, rgb2gray.cu:64-76 (texture read y-flipped) */
void orc_rgbd_float4_to_gray_z(const float *rgbd, int W, int H, const float *calib, float *gray, float *z) {
    float minDist = calib[MIND_OFFSET];
    float maxDist = calib[MAXD_OFFSET];
    for (int yi = 0; yi < H; yi++)
        for (int xi = 0; xi < W; xi++) {
            const float *p = &rgbd[4 * (xi + (H - 1 - yi) * W)];
            int offset = xi + yi * W;
            gray[offset] = 0.3f * p[0] + 0.59f * p[1] + 0.11f * p[2];
            z[offset] = -(p[3] * (maxDist - minDist) + minDist);
        }
}

/* fastDownSampleHdrKernel, downSample2Cuda.cu:35-42 */
void orc_downsample2(const float *hi, int wlo, int hlo, float *lo) {
    int w2 = 2 * wlo;
    for (int y = 0; y < hlo; y++)
        for (int x = 0; x < wlo; x++) {
            int h0 = 2 * x + 2 * y * w2;
            lo[x + y * wlo] = (hi[h0] + hi[h0 + 1] + hi[h0 + w2] + hi[h0 + w2 + 1]) / 4.0f;
        }
}

/* ------------------------------------------------------------------ */
/* photometric reference preparation                                   */
/* ------------------------------------------------------------------ */

/* convertZMapToXYZKernel, rgb2gray.cu:570-593; output float4 (x,y,z,w) */
void orc_zmap_to_xyz(const float *zp, int W, int H, const float *calib, float *xyzw) {
    float minDist = calib[MIND_OFFSET];
    float maxDist = calib[MAXD_OFFSET];
    float fx = calib[KL_OFFSET], fy = calib[KL_OFFSET + 4];
    float cx = calib[KL_OFFSET + 2], cy = calib[KL_OFFSET + 5];
    for (int yi = 0; yi < H; yi++)
        for (int xi = 0; xi < W; xi++) {
            int idx = xi + yi * W;
            float z = zp[idx];
            float *o = &xyzw[4 * idx];
            if (z < -minDist && z > -maxDist) {
                o[0] = ((float)xi - cx) * z / fx;
                o[1] = ((float)yi - cy) * z / fy;
                o[2] = z;
                o[3] = 1;
            } else {
                o[0] = o[1] = o[2] = o[3] = 0;
            }
        }
}

/* xyz2CloudKernel, d2z.cu:235-331.  vdata uses the reference's stride-24 record
 * (rendering/VertexBuffer2.h:24). */
void orc_xyz2cloud(const float *xyzw, int W, int H, const float *calib, const float *img, float *vdata) {
    orc_xyz2cloud_col(xyzw, W, H, calib, img, NULL, vdata);
}

/* The same with a fused keyframe colour per IR pixel (orc_fuse_rgbd): where
 * col[offset] >= 0 it is the vertex colour (slot 14) in place of the bilinear
 * sample of img; the gradients are still taken from img. */
void orc_xyz2cloud_col(const float *xyzw, int W, int H, const float *calib, const float *img, const float *col,
                       float *vdata) {
    const float *T = &calib[TLR_OFFSET];
    const float *KR = &calib[KR_OFFSET];
    const float *kc = &calib[KCR_OFFSET];
    float maxDist = calib[MAXD_OFFSET];
#pragma omp parallel for schedule(static)
    for (int offset = 0; offset < W * H; offset++) {
        float *v = &vdata[offset * 24];
        float p3[3] = {xyzw[4 * offset], xyzw[4 * offset + 1], xyzw[4 * offset + 2]};
        if (p3[2] < 0) {
            float r3[3];
            mul4(T, p3, r3);
            float pux = r3[0] / r3[2];
            float puy = r3[1] / r3[2];
            float px, py;
            distort(pux, puy, kc, KR, &px, &py);
            if (in_bounds10(px, py, W, H)) {
                int xdi = ftoi(px), ydi = ftoi(py);
                float fx = px - xdi, fy = py - ydi;
                float color1 = bilin(xdi, ydi, fx, fy, W, img);
                if (col && col[offset] >= 0.0f) color1 = col[offset];
                float colorN = bilin(ftoi(px), ftoi(py - 1.0f), fx, fy, W, img);
                float colorE = bilin(ftoi(px + 1.0f), ftoi(py), fx, fy, W, img);
                float colorW = bilin(ftoi(px - 1.0f), ftoi(py), fx, fy, W, img);
                float colorS = bilin(ftoi(px), ftoi(py + 1.0f), fx, fy, W, img);
                float gradX1 = (colorE - colorW) / 2.0f;
                float gradY1 = (colorS - colorN) / 2.0f;
                v[0] = p3[0]; v[1] = p3[1]; v[2] = p3[2];
                v[3] = v[4] = v[5] = 0.0f;
                v[6] = px; v[7] = py;
                v[8] = v[9] = v[10] = 0.0f;
                v[11] = gradX1;
                v[12] = gradY1;
                float gm = fabsf(gradY1) + fabsf(gradX1);
                v[13] = gm < 1.0f ? gm : 1.0f;
                v[14] = color1;
                continue;
            }
        }
        for (int i = 0; i < 24; i++) v[i] = 0.0f;
        v[2] = -maxDist;
    }
}

/* 256-bin gradient histogram: bin = (uint)(g*(bins-1)+0.5f), gpu_hist.cu:136 */
void orc_grad_histogram(const float *grad, int n, int nbins, int32_t *hist) {
    memset(hist, 0, nbins * sizeof(int32_t));
    for (int i = 0; i < n; i++) {
        unsigned int bin = (unsigned int)(grad[i] * (nbins - 1) + 0.5f);
        if (bin < (unsigned)nbins) hist[bin]++;
    }
}

/* seekThreshold256Kernel2 + filterIndexKernel4, filterIndex256.cu:26-46, 110-194.
 * Returns the number of indices the reference writes; idx_out (length P) is
 * padded with index 0 when fewer than P were written. */
int orc_filter_indices(const float *grad, int n, const int32_t *hist, int nbins, int P, int32_t *idx_out) {
    /* seek from the top bin down */
    unsigned int thr = 0;
    int sel = 0;
    for (int i = nbins - 1; i >= 0; i--) {
        sel += hist[i];
        if (sel > P) { thr = (unsigned)i; break; }
    }
    int excess = sel - P;
    const int nthreads = 512;
    int ppt = n / nthreads;
    int *cnt = (int *)calloc(nthreads, sizeof(int));
    int *mcnt = (int *)calloc(nthreads, sizeof(int));
    for (int s = 0; s < nthreads; s++)
        for (int i = s * ppt; i < s * ppt + ppt; i++) {
            unsigned int q = (unsigned int)(grad[i] * (nbins - 1) + 0.5f);
            if (q > thr) cnt[s]++;
            else if (q == thr) mcnt[s]++;
        }
    int *start = (int *)calloc(nthreads, sizeof(int));
    int *mstart = (int *)calloc(nthreads, sizeof(int));
    int tooMuch = excess;
    start[0] = 0;
    for (int i = 1; i < nthreads; i++) start[i] = start[i - 1] + cnt[i - 1];
    mstart[0] = start[nthreads - 1] + cnt[nthreads - 1];
    for (int i = 1; i < nthreads; i++) {
        if (tooMuch > 0 && mcnt[i - 1] > 0) {
            mcnt[i - 1] -= tooMuch;
            if (mcnt[i - 1] < 0) {
                tooMuch += mcnt[i - 1];
                mcnt[i - 1] = 0;
            } else {
                tooMuch = 0;
            }
        }
        mstart[i] = mstart[i - 1] + mcnt[i - 1];
    }
    int total = mstart[nthreads - 1] + mcnt[nthreads - 1];
    for (int k = 0; k < P; k++) idx_out[k] = 0;
    for (int s = 0; s < nthreads; s++) {
        int c = 0, m = 0;
        for (int i = s * ppt; i < s * ppt + ppt; i++) {
            unsigned int q = (unsigned int)(grad[i] * (nbins - 1) + 0.5f);
            if (q > thr) {
                int pos = start[s] + c++;
                if (pos < P) idx_out[pos] = i;
            } else if (q == thr) {
                if (m < mcnt[s]) {
                    int pos = mstart[s] + m;
                    if (pos < P) idx_out[pos] = i;
                }
                m++;
            }
        }
    }
    free(cnt); free(mcnt); free(start); free(mstart);
    return total;
}

/* addVertexAttributesWithoutNormalsKernel3/4, d2z.cu:700-936.  Levels 1..L-1;
 * slots 15..23 of the record.  Taps are clamped into the level image (see
 * bilin_clamped). */
void orc_add_vertex_attributes(const int32_t *idx, int P, float *vdata, int W, int H, const float *calib,
                               const float *const *gray, int L) {
    const float *kc = &calib[KCR_OFFSET];
    const float *KR = &calib[KR_OFFSET];
    const float *T = &calib[TLR_OFFSET];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < P; k++) {
        float *v = &vdata[idx[k] * 24];
        float p3[3] = {v[0], v[1], v[2]}, r3[3];
        mul4(T, p3, r3);
        float col[4] = {0, 0, 0, 0}, gx[4] = {0, 0, 0, 0}, gy[4] = {0, 0, 0, 0};
        float pux = r3[0] / r3[2];
        float puy = r3[1] / r3[2];
        float px, py;
        distort(pux, puy, kc, KR, &px, &py);
        if (in_bounds10(px, py, W, H)) {
            float a = 0.5f, b = -0.25f;
            float lx = px, ly = py;
            for (int l = 1; l < L; l++) {
                lx = a * lx + b;
                ly = a * ly + b;
                int wl = W >> l, hl = H >> l;
                int xdi = ftoi(lx), ydi = ftoi(ly);
                float fracX = lx - xdi, fracY = ly - ydi;
                col[l] = bilin_clamped(xdi, ydi, fracX, fracY, wl, hl, gray[l]);
                float cN = bilin_clamped(xdi, ydi - 1, fracX, fracY, wl, hl, gray[l]);
                float cW = bilin_clamped(xdi - 1, ydi, fracX, fracY, wl, hl, gray[l]);
                float cE = bilin_clamped(xdi + 1, ydi, fracX, fracY, wl, hl, gray[l]);
                float cS = bilin_clamped(xdi, ydi + 1, fracX, fracY, wl, hl, gray[l]);
                gx[l] = (cE - cW) / 2.0f;
                gy[l] = (cS - cN) / 2.0f;
            }
        }
        for (int l = 1; l < 4; l++) {
            if (l >= L) break;
            v[15 + 3 * (l - 1)] = gx[l];
            v[16 + 3 * (l - 1)] = gy[l];
            v[17 + 3 * (l - 1)] = col[l];
        }
    }
}

/* precomputeJacobian4Kernel, warp.cu:502-645.  J[l] is SoA: J[l][c*P + k]. */
void orc_precompute_jacobian(const int32_t *idx, int P, const float *vdata, const float *calib, float optScaleIn,
                             int L, float *const *J) {
    const float *K = &calib[KR_OFFSET];
    const float *T = &calib[TLR_OFFSET];
    const float *kc = &calib[KCR_OFFSET];
    static const int gslot[4][2] = {{11, 12}, {15, 16}, {18, 19}, {21, 22}};
#pragma omp parallel for schedule(static)
    for (int k = 0; k < P; k++) {
        const float *v = &vdata[idx[k] * 24];
        float p3[3] = {v[0], v[1], v[2]}, r3[3];
        mul4(T, p3, r3);
        r3[0] *= optScaleIn;
        r3[1] *= optScaleIn;
        r3[2] *= optScaleIn;
        float dN[6];
        dN[0] = 1.0f / r3[2]; dN[1] = 0; dN[2] = -r3[0] / (r3[2] * r3[2]);
        dN[3] = 0; dN[4] = 1.0f / r3[2]; dN[5] = -r3[1] / (r3[2] * r3[2]);
        float x = r3[0] / r3[2];
        float y = r3[1] / r3[2];
        float x2 = x * x, y2 = y * y;
        float x4 = x2 * x2, y4 = y2 * y2;
        float r2 = x2 + y2, r4 = r2 * r2;
        float dD[4];
        dD[0] = 1 + kc[0] * (3 * x2 + y2) + kc[1] * (5 * x4 + 6 * x2 * y2 + y4) + kc[4] * r4 * (7 * x2 + y2);
        dD[1] = kc[0] * 2 * x * y + kc[1] * 4 * x * y * r2 + kc[4] * 6 * x * y * r4;
        dD[2] = kc[0] * 2 * y * x + kc[1] * 4 * x * y * r2 + kc[4] * 6 * x * y * r4;
        dD[3] = 1 + kc[0] * (3 * x2 + y2) + kc[1] * (5 * x4 + 6 * x2 * y2 + y4) + kc[4] * r4 * (7 * y2 + x2);
        float dps[6][3] = {{0.0f, -r3[2], r3[1]}, {r3[2], 0.0f, -r3[0]}, {-r3[1], r3[0], 0.0f},
                           {1.0f, 0.0f, 0.0f},    {0.0f, 1.0f, 0.0f},    {0.0f, 0.0f, 1.0f}};
        for (int c = 0; c < 6; c++) {
            float dr3[3], dd2[3], dp2[3], dpn2x, dpn2y;
            rot4(T, dps[c], dr3);
            dpn2x = dN[0] * dr3[0] + dN[1] * dr3[1] + dN[2] * dr3[2];
            dpn2y = dN[3] * dr3[0] + dN[4] * dr3[1] + dN[5] * dr3[2];
            dd2[0] = dD[0] * dpn2x + dD[1] * dpn2y;
            dd2[1] = dD[2] * dpn2x + dD[3] * dpn2y;
            dd2[2] = 0;
            mul3(K, dd2, dp2);
            for (int l = 0; l < L; l++) {
                float gxl = v[gslot[l][0]], gyl = v[gslot[l][1]];
                float val;
                if (l == 0) val = dp2[0] * gxl + dp2[1] * gyl;
                else {
                    float s = (l == 1) ? 2.0f : (l == 2 ? 4.0f : 8.0f);
                    val = (dp2[0] / s) * gxl + (dp2[1] / s) * gyl;
                }
                J[l][c * P + k] = val;
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* photometric iteration                                               */
/* ------------------------------------------------------------------ */

/* interpolateResidualKernel2 + interpolateResidual2, warp.cu:269-332, 1160-1218.
 * sel_xyz is SoA (x[P], y[P], z[P]); sel_I is the reference intensity at this level. */
void orc_interpolate_residual(int P, const float *sel_xyz, const float *sel_I, const float *T, const float *calib,
                              int layer, const float *img, int width, int height, const float *zcur, int zwidth,
                              int zheight, float *residual, float *zweight) {
    const float *KR = &calib[KR_OFFSET];
    const float *kc = &calib[KCR_OFFSET];
    const float *TLR = &calib[TLR_OFFSET];
    const float *KL = &calib[KL_OFFSET];
    const float *TRL = &calib[TRL_OFFSET];
    int divisor = 1 << layer;
    float a = 1.0f / (float)divisor;
    float b = 0.5f * (a - 1.0f);
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < P; idx++) {
        float p3[3] = {sel_xyz[idx], sel_xyz[P + idx], sel_xyz[2 * P + idx]};
        float r3_ir[3], r3[3];
        mul4(T, p3, r3_ir);
        mul4(TLR, r3_ir, r3);
        float pux = r3[0] / r3[2];
        float puy = r3[1] / r3[2];
        float p2x, p2y;
        distort(pux, puy, kc, KR, &p2x, &p2y);
        float px = a * p2x + b;
        float py = a * p2y + b;
        float iResidual = 1.0f;
        int xdi = ftoi(px);
        int ydi = ftoi(py);
        float zWeight = 0.0f;
        if (xdi >= 0 && ydi >= 0 && xdi < width - 1 && ydi < height - 1) {
            float fx = px - xdi;
            float fy = py - ydi;
            float color = bilin(xdi, ydi, fx, fy, width, img);
            iResidual = sel_I[idx] - color;
            float rl3[3], pl2[3];
            mul4(TRL, r3, rl3);
            rl3[0] /= rl3[2];
            rl3[1] /= rl3[2];
            rl3[2] = 1;
            mul3(KL, rl3, pl2);
            int xdi2 = ftoi(pl2[0] + 0.5f);
            int ydi2 = ftoi(pl2[1] + 0.5f);
            if (xdi2 >= 0 && ydi2 >= 0 && xdi2 < zwidth && ydi2 < zheight) {
                int offset = xdi2 + ydi2 * zwidth;
                float zc = zcur[offset];
                float zerr = zc - r3[2];
                zerr *= zerr;
                if (zerr < 100 * 100) zWeight = 1.0f - zerr / (100.0f * 100.0f);
            }
        }
        residual[idx] = iResidual;
        zweight[idx] = zWeight;
    }
}

/* MAD scale for a histogram median bin (histogram64.cu:81 for 64 bins). */
static inline float mad_scale(int m, int nbins) {
    if (nbins == 64) return 1.4826f * (float)(4 * m + 3) / 255.0f;
    return 1.4826f * ((float)m + 0.75f) / ((float)nbins - 0.25f);
}

/* discretizeResidualKernel + histogram + seekThreshold64Kernel + generateWeights64Kernel
 * + weightJacobian's weights, histogram64.cu:41-157.  Returns the median bin. */
int orc_generate_weights(const float *r, const float *zw, int N, int nbins, int32_t *hist, float *w, float *rw) {
    memset(hist, 0, nbins * sizeof(int32_t));
    float binscale = (float)(nbins - 1);
    for (int i = 0; i < N; i++) {
        int bin = ftoi(binscale * fabsf(r[i]));
        if (bin < 0) bin = 0;
        if (bin > nbins - 1) bin = nbins - 1;
        hist[bin]++;
    }
    int half = N / 2;
    int m = 0, acc = 0;
    for (int i = 0; i < nbins; i++) {
        acc += hist[i];
        if (acc > half) { m = i; break; }
    }
    float s = mad_scale(m, nbins);
    float bb = 4.6851f;
    for (int i = 0; i < N; i++) {
        float u = fabsf(r[i]) / s;
        float wi = 0.0f;
        if (u <= bb) {
            float ub = u / bb;
            float ub2 = ub * ub;
            wi = (1.0f - ub2) * zw[i];
        }
        rw[i] = r[i] * wi;
        w[i] = wi;
    }
    return m;
}

/* Canonical 27-term normal-equation reduction (replaces JTJCuda / JTresidualCuda,
 * warp.cu:1430-1487; the products are the reference's Jw_j*Jw_i and Jw_c*r).
 *
 * Order (identical in the CUDA kernels): N is split into chunks of 1024 points;
 * in chunk k, lane t (0..255) sums the products of points k*1024 + t + 256*m for
 * m = 0..3 in FP32, each product added with one fused multiply-add (fmaf, one
 * rounding, identical on every IEEE platform); each warp of 32 lanes combines its lanes with an xor
 * butterfly (offsets 16, 8, 4, 2, 1) in FP32; the 8 warp values are converted to
 * FP64 and summed in warp order; chunk values are summed in chunk order in FP64.
 * Term order: the 21 upper-triangle JtJ terms (j <= i, row-major over j), then
 * the 6 Jtr terms. */
/* The FP32 stage of the canonical order for chunk k: wv[w][q] is the value
 * warp w (lanes 32w..32w+31) holds for term q after its xor butterfly. */
static void chunk_warp_values(const float *const *J6, const float *r, int k, float wv[8][27]) {
    for (int wi = 0; wi < 8; wi++) {
        float lane[32][27];
        for (int l = 0; l < 32; l++) {
            int t = wi * 32 + l;
            float s[27];
            for (int q = 0; q < 27; q++) s[q] = 0.0f;
            for (int m = 0; m < 4; m++) {
                int i = k * ORC_CHUNK + t + 256 * m;
                float jv[6];
                for (int c = 0; c < 6; c++) jv[c] = J6[c][i];
                int q = 0;
                for (int j = 0; j < 6; j++)
                    for (int ii = j; ii < 6; ii++, q++) s[q] = fmaf(jv[j], jv[ii], s[q]);
                for (int c = 0; c < 6; c++, q++) s[q] = fmaf(jv[c], r[i], s[q]);
            }
            for (int q = 0; q < 27; q++) lane[l][q] = s[q];
        }
        for (int off = 16; off >= 1; off >>= 1) {
            float nl[32][27];
            for (int l = 0; l < 32; l++)
                for (int q = 0; q < 27; q++) nl[l][q] = lane[l][q] + lane[l ^ off][q];
            memcpy(lane, nl, sizeof(nl));
        }
        for (int q = 0; q < 27; q++) wv[wi][q] = lane[0][q];
    }
}

static void unpack27(const double *tot, double A[36], double b[6]) {
    int q = 0;
    for (int j = 0; j < 6; j++)
        for (int i = j; i < 6; i++) {
            A[i + j * 6] = tot[q];
            A[i * 6 + j] = tot[q];
            q++;
        }
    for (int c = 0; c < 6; c++) b[c] = tot[q++];
}

void orc_reduce27(const float *const *J6, const float *r, int N, double A[36], double b[6]) {
    int nchunks = N / ORC_CHUNK;
    double tot[27];
    for (int q = 0; q < 27; q++) tot[q] = 0.0;
    for (int k = 0; k < nchunks; k++) {
        float wv[8][27];
        chunk_warp_values(J6, r, k, wv);
        double chunk[27];
        for (int q = 0; q < 27; q++) chunk[q] = 0.0;
        for (int wi = 0; wi < 8; wi++)
            for (int q = 0; q < 27; q++) chunk[q] = chunk[q] + (double)wv[wi][q];
        for (int q = 0; q < 27; q++) tot[q] = tot[q] + chunk[q];
    }
    unpack27(tot, A, b);
}

/* Fixed-point accumulation.  The 27 terms of the tracker's normal equations are
 * the exact sum of every FP32 warp value of the canonical order above (lanes
 * and butterflies as in orc_reduce27), each truncated toward zero at 2^-64,
 * rounded once to FP64 (round to nearest even).  The sum does not depend on
 * the order in which chunks and warps are added, which lets the GPU add them
 * with integer atomics from any CTA in any order. */
void orc_fx_add(long long L[ORC_FX_LIMBS], float v, int *bad) {
    uint32_t bits;
    memcpy(&bits, &v, 4);
    uint32_t E = (bits >> 23) & 0xffu, M = bits & 0x7fffffu;
    if (E == 0xffu) { *bad = 1; return; }            /* Inf / NaN */
    uint64_t m;
    int e;
    if (E == 0) { m = M; e = -149; } else { m = M | 0x800000u; e = (int)E - 150; }
    if (m == 0) return;
    if (e >= 25) { *bad = 1; return; }               /* |v| >= 2^48 */
    int s = e + 64;                                  /* bit of m's lsb in units of 2^-64 */
    if (s < 0) {
        m = (-s >= 24) ? 0 : (m >> -s);
        s = 0;
    }
    if (m == 0) return;
    int k0 = s >> 5;
    uint64_t t = m << (s & 31);
    long long lo = (long long)(t & 0xffffffffu), hi = (long long)(t >> 32);
    if (bits >> 31) { lo = -lo; hi = -hi; }
    L[k0] += lo;
    if (hi) L[k0 + 1] += hi;
}

double orc_fx_to_double(const long long L[ORC_FX_LIMBS]) {
    /* Q = sum_k L[k] 2^(32k) in two's complement 128-bit arithmetic */
    unsigned __int128 Q = 0;
    for (int k = ORC_FX_LIMBS - 1; k >= 0; k--) Q = (Q << 32) + (unsigned __int128)(__int128)L[k];
    int neg = (int)(Q >> 127);
    unsigned __int128 U = neg ? (unsigned __int128)0 - Q : Q;
    if (U == 0) return 0.0;
    uint64_t hi = (uint64_t)(U >> 64), lo = (uint64_t)U;
    int n = hi ? 127 - __builtin_clzll(hi) : 63 - __builtin_clzll(lo); /* top bit */
    uint64_t mant;
    int e2; /* value = mant * 2^e2 */
    if (n <= 52) {
        mant = (uint64_t)U << (52 - n);
        e2 = -64 - (52 - n);
    } else {
        int sh = n - 52;
        mant = (uint64_t)(U >> sh);
        unsigned __int128 rem = U - ((unsigned __int128)mant << sh);
        unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
        if (rem > half || (rem == half && (mant & 1))) mant++;
        if (mant >> 53) { mant >>= 1; sh++; }
        e2 = sh - 64;
    }
    /* mant in [2^52, 2^53): biased exponent of mant * 2^e2 */
    uint64_t out = ((uint64_t)(e2 + 52 + 1023) << 52) | (mant & ((1ull << 52) - 1));
    if (neg) out |= 1ull << 63;
    double d;
    memcpy(&d, &out, 8);
    return d;
}

void orc_fx27_clear(orc_fx27 *acc) { memset(acc, 0, sizeof(*acc)); }

void orc_reduce27_fx(const float *const *J6, const float *r, int N, orc_fx27 *acc) {
    int nchunks = N / ORC_CHUNK;
    for (int k = 0; k < nchunks; k++) {
        float wv[8][27];
        chunk_warp_values(J6, r, k, wv);
        for (int wi = 0; wi < 8; wi++)
            for (int q = 0; q < 27; q++) orc_fx_add(acc->L[q], wv[wi][q], &acc->bad);
    }
}

/* The 27 accumulated terms as the system (A, b); all NaN if any input was out of range. */
void orc_fx27_value(const orc_fx27 *acc, double A[36], double b[6]) {
    double tot[27];
    for (int q = 0; q < 27; q++) tot[q] = acc->bad ? NAN : orc_fx_to_double(acc->L[q]);
    unpack27(tot, A, b);
}

/* The reference's own order: reduceProduct6<float,256> (reduction_kernel.cu:262-317)
 * per 512-element block, then sumElemsKernel's serial block sum (warp.cu:801-810). */
static float ref_dot(const float *a, const float *bvec, int n) {
    int nthreads = 256;
    int nblocks = n / nthreads;
    float acc = 0.0f;
    int pow2 = (n & (n - 1)) == 0;
    for (int blk = 0; blk < nblocks; blk++) {
        float sdata[256];
        for (int tid = 0; tid < 256; tid++) {
            unsigned int i = blk * 512 + tid;
            float mySum = 0;
            while (i < (unsigned)n) {
                mySum += a[i] * bvec[i];
                if (pow2 || i + 256 < (unsigned)n) mySum += a[i + 256] * bvec[i + 256];
                i += 512 * nblocks;
            }
            sdata[tid] = mySum;
        }
        for (int s = 128; s >= 1; s >>= 1)
            for (int tid = 0; tid < s; tid++) sdata[tid] = sdata[tid] + sdata[tid + s];
        acc += sdata[0];
    }
    return acc;
}

void orc_reduce27_refordered(const float *const *J6, const float *r, int N, float A[36], float b[6]) {
    for (int j = 0; j < 6; j++)
        for (int i = j; i < 6; i++) {
            float v = ref_dot(J6[j], J6[i], N);
            A[i + j * 6] = v;
            A[i * 6 + j] = v;
        }
    for (int c = 0; c < 6; c++) b[c] = ref_dot(J6[c], r, N);
}

/* ------------------------------------------------------------------ */
/* Mixed-precision storage                                             */
/* ------------------------------------------------------------------ */

/* IEEE binary16 rounding to nearest even, by integer operations on the float's
 * bits: 10 fraction bits for normal results (exponent >= -14), a fixed 2^-24
 * quantum below, overflow to infinity at and above 65520. */
float orc_f16_round(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    uint32_t sign = u & 0x80000000u, a = u & 0x7fffffffu;
    if (a >= 0x7f800000u) return x;                  /* Inf, NaN */
    uint32_t r;
    if (a >= 0x38800000u) {                          /* |x| >= 2^-14: normal binary16 */
        r = a + 0xfffu + ((a >> 13) & 1u);
        r &= ~0x1fffu;
        if (r >= 0x47800000u) r = 0x7f800000u;       /* rounded up to 2^16: infinity */
    } else {                                         /* subnormal binary16: multiples of 2^-24 */
        /* |x| = m * 2^(e - 150) (e >= 1) or m * 2^-149 (e = 0); in units of
         * 2^-24 that is m >> s with s = 126 - e (125 for e = 0), s >= 14 */
        int e = (int)(a >> 23);
        uint64_t m = (a & 0x7fffffu) | (e ? 0x800000u : 0u);
        int sh = e ? 126 - e : 125;
        uint64_t q = 0;
        if (sh < 40) {
            uint64_t qi = m >> sh, rem = m & ((1ull << sh) - 1), half = 1ull << (sh - 1);
            q = qi + ((rem > half || (rem == half && (qi & 1))) ? 1 : 0);
        }
        float f = (float)q * 5.9604644775390625e-8f; /* q * 2^-24, exact (q <= 1024) */
        memcpy(&r, &f, 4);
    }
    r |= sign;
    float out;
    memcpy(&out, &r, 4);
    return out;
}

/* bfloat16 (8 fraction bits) rounding to nearest even; NaN and Inf kept. */
float orc_bf16_round(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return x;
    u = u + 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    float out;
    memcpy(&out, &u, 4);
    return out;
}

/* ------------------------------------------------------------------ */
/* ICP                                                                 */
/* ------------------------------------------------------------------ */

/* convertZMapToXYZ6Kernel, rgb2gray.cu:595-624 */
void orc_zmap_to_xyz6(const float *zp, int W, int H, const float *calib, float *pts, int32_t *mask) {
    float minDist = calib[MIND_OFFSET];
    float maxDist = calib[MAXD_OFFSET];
    float fx = calib[KL_OFFSET], fy = calib[KL_OFFSET + 4];
    float cx = calib[KL_OFFSET + 2], cy = calib[KL_OFFSET + 5];
    for (int yi = 0; yi < H; yi++)
        for (int xi = 0; xi < W; xi++) {
            int idx = xi + yi * W;
            float z = zp[idx];
            if (z < -minDist && z > -maxDist) {
                pts[idx * 6 + 0] = ((float)xi - cx) * z / fx;
                pts[idx * 6 + 1] = ((float)yi - cy) * z / fy;
                pts[idx * 6 + 2] = z;
                mask[idx] = 1;
            } else {
                pts[idx * 6 + 0] = 0;
                pts[idx * 6 + 1] = 0;
                pts[idx * 6 + 2] = 0;
                mask[idx] = 0;
            }
        }
}

/* computeNormalsCudaKernel, d2z.cu:503-537 (normals written into slots 3..5) */
void orc_compute_normals6(float *pts, int32_t *mask, int W, int H) {
    for (int i = 0; i < W * H; i++) pts[i * 6 + 3] = pts[i * 6 + 4] = pts[i * 6 + 5] = 0;
    for (int yi = 0; yi < H; yi++)
        for (int xi = 0; xi < W; xi++) {
            int offset = xi + yi * W;
            if (xi < 1 || yi < 1 || xi > W - 2 || yi > H - 2) {
                mask[offset] = 0;
                continue;
            }
            const float *x1 = &pts[(offset - 1) * 6];
            const float *x2 = &pts[(offset + 1) * 6];
            const float *y1 = &pts[(offset - W) * 6];
            const float *y2 = &pts[(offset + W) * 6];
            if (x1[2] < 0 && x2[2] < 0 && y1[2] < 0 && y2[2] < 0) {
                float u[3] = {x2[0] - x1[0], x2[1] - x1[1], x2[2] - x1[2]};
                float v[3] = {y2[0] - y1[0], y2[1] - y1[1], y2[2] - y1[2]};
                float n[3];
                n[0] = u[1] * v[2] - u[2] * v[1];
                n[1] = -(u[0] * v[2] - u[2] * v[0]);
                n[2] = u[0] * v[1] - u[1] * v[0];
                normalize3(n);
                pts[offset * 6 + 3] = n[0];
                pts[offset * 6 + 4] = n[1];
                pts[offset * 6 + 5] = n[2];
            } else {
                mask[offset] = 0;
            }
        }
}

/* genPointsCloud6Kernel, d2z.cu:436-469 */
void orc_gen_cloud6(const float *zp, int W, int H, const float *calib, float *pts, int32_t *mask) {
    float fx = calib[KL_OFFSET], fy = calib[KL_OFFSET + 4];
    float cx = calib[KL_OFFSET + 2], cy = calib[KL_OFFSET + 5];
    for (int yi = 0; yi < H; yi++)
        for (int xi = 0; xi < W; xi++) {
            int offset = xi + yi * W;
            float z = zp[offset];
            float *p = &pts[offset * 6];
            if (z < 0) {
                p[0] = ((float)xi - cx) * z / fx;
                p[1] = ((float)yi - cy) * z / fy;
                p[2] = z;
                p[3] = 0; p[4] = 0; p[5] = 1.0f;
                mask[offset] = 1;
            } else {
                p[0] = p[1] = p[2] = p[3] = p[4] = p[5] = 0;
                mask[offset] = 0;
            }
        }
}

/* downSampleCloud6Kernel, d2z.cu:557-588 (normalizeCuda, kernelUtils.h:19-28) */
void orc_downsample_cloud6(const float *src, const int32_t *msrc, int wlo, int hlo, float *dst, int32_t *mdst) {
    for (int yi = 0; yi < hlo; yi++)
        for (int xi = 0; xi < wlo; xi++) {
            int offset = xi + yi * wlo;
            float *pd = &dst[offset * 6];
            int h0 = xi * 2 + yi * 2 * (wlo * 2);
            int offs[4] = {h0, h0 + 1, h0 + wlo * 2, h0 + wlo * 2 + 1};
            for (int i = 0; i < 6; i++) pd[i] = 0.0f;
            float ns = 0.0f;
            for (int k = 0; k < 4; k++)
                if (msrc[offs[k]]) {
                    ns++;
                    for (int i = 0; i < 6; i++) pd[i] += src[offs[k] * 6 + i];
                }
            if (ns > 0.0f) {
                for (int i = 0; i < 6; i++) pd[i] /= ns;
                normalize3(&pd[3]);
                mdst[offset] = 1;
            } else {
                mdst[offset] = 0;
            }
        }
}

/* bilinearInterpolation6, kernelUtils.h:305-316 (pitch in floats) */
static inline void bilin6(const float *s, float fx, float fy, int pitch, float *p) {
    for (int c = 0; c < 3; c++) {
        float v0 = s[c], v1 = s[c + 6], v2 = s[c + pitch], v3 = s[c + pitch + 6];
        p[c] = (1 - fx) * (1 - fy) * v0 + fx * (1 - fy) * v1 + (1 - fx) * fy * v2 + fx * fy * v3;
    }
}

/* icpResidualKernel2 + icpResidualMaskCuda2, rgb2gray.cu:223-260, 780-790 */
void orc_icp_residual_mask(const float *ref6, const int32_t *refmask, int width, int height, const float *T,
                           const float *calib, const float *cur6, const int32_t *curmask, int layer,
                           float *residual, int32_t *rmask) {
    const float *K = &calib[KL_OFFSET];
    int divisor = 1 << layer;
    float a = 1.0f / (float)divisor;
    float b = 0.5f * (a - 1.0f);
#pragma omp parallel for schedule(static)
    for (int offset = 0; offset < width * height; offset++) {
        residual[offset] = 0.0f;
        if (refmask[offset] == 0) { rmask[offset] = 0; continue; }
        const float *p = &ref6[offset * 6];
        float p3[3] = {p[0], p[1], p[2]}, rn[3] = {p[3], p[4], p[5]};
        float q3[3], cn[3];
        mul4(T, p3, q3);
        rot4(T, rn, cn);
        float q2x = q3[0] / q3[2], q2y = q3[1] / q3[2];
        float p2x = a * (K[0] * q2x + K[2]) + b;
        float p2y = a * (K[4] * q2y + K[5]) + b;
        rmask[offset] = 0;
        if (p2x >= 0 && p2x < (width - 1) && p2y >= 0 && p2y < (height - 1)) {
            int xdi = ftoi(p2x), ydi = ftoi(p2y);
            int off2 = xdi + ydi * width;
            if (curmask[off2] && curmask[off2 + 1] && curmask[off2 + width] && curmask[off2 + width + 1]) {
                float fx = p2x - xdi, fy = p2y - ydi;
                float cp[3];
                bilin6(&cur6[off2 * 6], fx, fy, width * 6, cp);
                float d[3] = {cp[0] - q3[0], cp[1] - q3[1], cp[2] - q3[2]};
                residual[offset] = d[0] * cn[0] + d[1] * cn[1] + d[2] * cn[2];
                rmask[offset] = 1;
            }
        }
    }
}

/* selectValidIndex, rgb2gray.cu:395-460, 827-840: stable compaction */
int orc_compact(const int32_t *mask, int n, int32_t *select) {
    int c = 0;
    for (int i = 0; i < n; i++)
        if (mask[i] > 0) select[c++] = i;
    return c;
}

/* generateStudentTWeights, rgb2gray.cu:470-569, 854-877.  The reference truncates
 * each product r2*w to int (estimateVariance1024's int accumulator,
 * rgb2gray.cu:519-521); here the truncated terms are summed exactly in int64. */
void orc_student_t(const float *r2, int n, float *w) {
    for (int i = 0; i < n; i++) w[i] = 6 / (5 + r2[i] / 100.0f);
    for (int it = 0; it < 3; it++) {
        long long S = 0;
        for (int i = 0; i < n; i++) {
            float prod = r2[i] * w[i];
            S += (prod >= 0.0f && prod < 9.0e18f) ? (long long)prod : (prod >= 9.0e18f ? 9000000000000000000LL : 0);
        }
        float Sf = (float)S;
        float minVal = (float)n;
        /* a single 1024-thread block returns the raw sum (rgb2gray.cu:497-499);
         * otherwise the sum is clamped from below by N (rgb2gray.cu:538-540) */
        float var = (n <= 1024) ? Sf : (Sf < minVal ? minVal : Sf);
        float sigma2 = var / (float)n;
        for (int i = 0; i < n; i++) w[i] = 6 / (5 + r2[i] / sigma2);
    }
    for (int i = 0; i < n; i++) w[i] = fminf(w[i], 1.0f);
}

/* icpResidualIndexKernel2 + icpResidualCuda2, rgb2gray.cu:323-390, 810-825.
 * J is SoA with stride npadded; entries [nsel, npadded) are zero. */
void orc_icp_residual_jacobian(const float *ref6, const int32_t *select, int nsel, int width, int height, int layer,
                               const float *T, const float *calib, const float *cur6, const int32_t *curmask,
                               int npadded, float *res, float *J, const float *weights, float optScaleIn) {
    const float *K = &calib[KL_OFFSET];
    int divisor = 1 << layer;
    float a = 1.0f / (float)divisor;
    float b = 0.5f * (a - 1.0f);
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < npadded; idx++) {
        res[idx] = 0.0f;
        for (int c = 0; c < 6; c++) J[idx + npadded * c] = 0.0f;
        if (idx >= nsel) continue;
        /* a weight that is not positive gives zeros below; skip the work */
        if (!(weights[idx] > 0.0f)) continue;
        const float *p = &ref6[select[idx] * 6];
        float p3[3] = {p[0], p[1], p[2]}, rn[3] = {p[3], p[4], p[5]};
        float q3[3], cn[3];
        mul4(T, p3, q3);
        rot4(T, rn, cn);
        float q2x = q3[0] / q3[2], q2y = q3[1] / q3[2];
        float p2x = a * (K[0] * q2x + K[2]) + b;
        float p2y = a * (K[4] * q2y + K[5]) + b;
        if (p2x >= 0 && p2x < (width - 1) && p2y >= 0 && p2y < (height - 1)) {
            float weight = weights[idx];
            int xdi = ftoi(p2x), ydi = ftoi(p2y);
            float fx = p2x - xdi, fy = p2y - ydi;
            int off2 = xdi + ydi * width;
            float cp[3];
            bilin6(&cur6[off2 * 6], fx, fy, width * 6, cp);
            if (curmask[off2] && weight > 0.0f && fabsf(cp[2] - q3[2]) < 300.0f) {
                float rv[3] = {cp[0] - q3[0], cp[1] - q3[1], cp[2] - q3[2]};
                res[idx] = optScaleIn * weight * (rv[0] * cn[0] + rv[1] * cn[1] + rv[2] * cn[2]);
                float dPs[3][3] = {{0, -p3[2], p3[1]}, {p3[2], 0, -p3[0]}, {-p3[1], p3[0], 0}};
                float dNs[3][3] = {{0, -rn[2], rn[1]}, {rn[2], 0, -rn[0]}, {-rn[1], rn[0], 0}};
                for (int c = 0; c < 3; c++) {
                    float dB[3], dN[3];
                    rot4(T, dPs[c], dB);
                    rot4(T, dNs[c], dN);
                    J[idx + npadded * c] = -optScaleIn * weight *
                                           (-cn[0] * dB[0] - cn[1] * dB[1] - cn[2] * dB[2] + rv[0] * dN[0] +
                                            rv[1] * dN[1] + rv[2] * dN[2]);
                }
                for (int c = 0; c < 3; c++) {
                    float e[3] = {0, 0, 0}, dB[3];
                    e[c] = 1;
                    rot4(T, e, dB);
                    J[idx + npadded * (3 + c)] = -weight * (-cn[0] * dB[0] - cn[1] * dB[1] - cn[2] * dB[2]);
                }
            }
        }
    }
}

/* The tracker's ICP residual and Jacobian over the level's pixel grid (the
 * GPU's icp_point): weights[idx] per pixel, 0 where the pixel is not a
 * correspondence.  The projection, bilinear taps and correspondence test are
 * icpResidualIndexKernel2's expressions (rgb2gray.cu:323-390) without
 * contraction; the rotated normal, the residual and the Jacobian are
 * evaluated with fmaf in a fixed order, and the reference's products by exact
 * zeros and ones of [p]x, [n]x and the unit vectors are left out (for a finite
 * pose that changes at most the sign of a zero entry).  Against the
 * reference-ordered orc_icp_residual_jacobian the values agree to a few ulp. */
void orc_icp_residual_jacobian_grid(const float *ref6, int width, int height, int layer, const float *T,
                                    const float *calib, const float *cur6, const int32_t *curmask, int npadded,
                                    float *res, float *J, const float *weights, float optScaleIn) {
    const float *K = &calib[KL_OFFSET];
    int divisor = 1 << layer;
    float a = 1.0f / (float)divisor;
    float b = 0.5f * (a - 1.0f);
    int n = width * height;
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < npadded; idx++) {
        res[idx] = 0.0f;
        for (int c = 0; c < 6; c++) J[idx + npadded * c] = 0.0f;
        if (idx >= n) continue;
        float weight = weights[idx];
        if (!(weight > 0.0f)) continue;
        const float *p = &ref6[idx * 6];
        float p3[3] = {p[0], p[1], p[2]}, rn[3] = {p[3], p[4], p[5]};
        float q3[3];
        mul4(T, p3, q3);
        float q2x = q3[0] / q3[2], q2y = q3[1] / q3[2];
        float p2x = a * (K[0] * q2x + K[2]) + b;
        float p2y = a * (K[4] * q2y + K[5]) + b;
        if (!(p2x >= 0 && p2x < (width - 1) && p2y >= 0 && p2y < (height - 1))) continue;
        int xdi = ftoi(p2x), ydi = ftoi(p2y);
        float fx = p2x - xdi, fy = p2y - ydi;
        int off2 = xdi + ydi * width;
        float cp[3];
        bilin6(&cur6[off2 * 6], fx, fy, width * 6, cp);
        if (!(curmask[off2] && fabsf(cp[2] - q3[2]) < 300.0f)) continue;
        float rv[3] = {cp[0] - q3[0], cp[1] - q3[1], cp[2] - q3[2]};
        float cn[3];
        for (int r = 0; r < 3; r++)
            cn[r] = fmaf(T[4 * r + 2], rn[2], fmaf(T[4 * r + 1], rn[1], T[4 * r] * rn[0]));
        res[idx] = optScaleIn * weight * fmaf(rv[2], cn[2], fmaf(rv[1], cn[1], rv[0] * cn[0]));
        /* columns of R [p]x and R [n]x: R_c1 * s1 + R_c2 * s2 per row */
        float B[3][3], N[3][3];
        for (int r = 0; r < 3; r++) {
            const float *Tr = &T[4 * r];
            B[0][r] = fmaf(Tr[1], -p3[2], Tr[2] * p3[1]);
            B[1][r] = fmaf(Tr[0], p3[2], Tr[2] * -p3[0]);
            B[2][r] = fmaf(Tr[0], -p3[1], Tr[1] * p3[0]);
            N[0][r] = fmaf(Tr[1], -rn[2], Tr[2] * rn[1]);
            N[1][r] = fmaf(Tr[0], rn[2], Tr[2] * -rn[0]);
            N[2][r] = fmaf(Tr[0], -rn[1], Tr[1] * rn[0]);
        }
        float so = -optScaleIn * weight;
        for (int c = 0; c < 3; c++) {
            float t = -cn[0] * B[c][0];
            t = fmaf(-cn[1], B[c][1], t);
            t = fmaf(-cn[2], B[c][2], t);
            t = fmaf(rv[0], N[c][0], t);
            t = fmaf(rv[1], N[c][1], t);
            t = fmaf(rv[2], N[c][2], t);
            J[idx + npadded * c] = so * t;
        }
        for (int c = 0; c < 3; c++)
            J[idx + npadded * (3 + c)] = -weight * fmaf(-cn[2], T[8 + c], fmaf(-cn[1], T[4 + c], -cn[0] * T[c]));
    }
}

/* ------------------------------------------------------------------ */
/* 6x6 solve and SE(3) exponential                                     */
/* ------------------------------------------------------------------ */

/* FP64 Cholesky in its square-root-free form A = L D L^T (unit lower L), with
 * reciprocal pivots.  The reference's Cholesky kernel (warp.cu:978-1007) is
 * compiled but not launched; the CPU alternative is cv::solve(DECOMP_CHOLESKY)
 * (phototracker.cpp:649-660).  The operation order below is the GPU's: row i
 * of column j is s = A_ij - sum_{k<j} L_ik U_jk (k ascending) with U_jk the
 * unscaled value s of row j at column k; D_j = s_jj, L_ij = s_ij * (1 / D_j);
 * the substitutions run column by column.  Returns 0 on success, -1 when a
 * pivot is not positive (x set to 0). */
int orc_solve_cholesky(const double A[36], const double b[6], double x[6]) {
    double L[36], U[36], inv[6];
    for (int i = 0; i < 36; i++) { L[i] = 0.0; U[i] = 0.0; }
    for (int j = 0; j < 6; j++) {
        double sv[6];
        for (int i = j; i < 6; i++) {
            double v = A[i * 6 + j];
            for (int k = 0; k < j; k++) v = fma(-L[i * 6 + k], U[j * 6 + k], v);
            sv[i] = v;
        }
        if (!(sv[j] > 0.0)) {
            for (int i = 0; i < 6; i++) x[i] = 0.0;
            return -1;
        }
        inv[j] = 1.0 / sv[j];
        for (int i = j + 1; i < 6; i++) {
            U[i * 6 + j] = sv[i];
            L[i * 6 + j] = sv[i] * inv[j];
        }
    }
    double z[6];
    for (int i = 0; i < 6; i++) z[i] = b[i];
    for (int k = 0; k < 6; k++)
        for (int i = k + 1; i < 6; i++) z[i] = fma(-L[i * 6 + k], z[k], z[i]);
    for (int i = 0; i < 6; i++) z[i] = z[i] * inv[i];
    for (int k = 5; k >= 0; k--)
        for (int i = 0; i < k; i++) z[i] = fma(-L[k * 6 + i], z[k], z[i]);
    for (int i = 0; i < 6; i++) x[i] = z[i];
    return 0;
}

/* conjugateGradientKernel, warp.cu:926-975 (dotProduct6 / matrixMultVec6 at warp.cu:877-893) */
static double dot6(const double *a, const double *b) {
    double d = 0;
    for (int i = 0; i < 6; i++) d += a[i] * b[i];
    return d;
}

void orc_solve_cg(const double A[36], const double bb[6], double tol, int maxSteps, double x[6]) {
    double r[6], dir[6];
    for (int i = 0; i < 6; i++) { x[i] = 0.0; r[i] = bb[i]; dir[i] = bb[i]; }
    int nSteps = 0;
    while (nSteps < maxSteps) {
        double Adir[6];
        for (int j = 0; j < 6; j++) {
            Adir[j] = 0.0;
            for (int k = 0; k < 6; k++) Adir[j] += A[j * 6 + k] * dir[k];
        }
        double rr = dot6(r, r);
        double Adirdir = dot6(Adir, dir);
        double div = Adirdir;
        if (div < 0) div = -div;
        double stepLength = 0.0;
        if (div > tol) stepLength = rr / Adirdir;
        for (int i = 0; i < 6; i++) r[i] -= stepLength * Adir[i];
        double rr2 = dot6(r, r);
        for (int i = 0; i < 6; i++) x[i] += stepLength * dir[i];
        if (sqrt(rr2) < tol) return;
        double beta = rr2 / rr;
        for (int i = 0; i < 6; i++) dir[i] = r[i] + beta * dir[i];
        nSteps++;
    }
}

/* matrixMult4Real, expmCuda.cu:1894-1917 */
static void mat4d(const double *M1, const double *M2, double *R) {
    double t[16];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++)
            t[r * 4 + c] = fma(M1[r * 4 + 3], M2[3 * 4 + c],
                               fma(M1[r * 4 + 2], M2[2 * 4 + c], fma(M1[r * 4 + 1], M2[1 * 4 + c],
                                                                     M1[r * 4 + 0] * M2[0 * 4 + c])));
    memcpy(R, t, sizeof(t));
}

/* normalizeMat4RealSafe, expmCuda.cu:1955-1980: lengths through single-precision
 * sqrtf, the length of the old first column used for the new one, and the
 * divisions written as products with the FP64 reciprocal of each length. */
static void normalize_mat4_safe(double *T) {
    double u[3] = {T[0], T[4], T[8]};
    double v[3] = {T[1], T[5], T[9]};
    double w[3] = {T[2], T[6], T[10]};
    double lenU = (double)sqrtf((float)fma(u[2], u[2], fma(u[1], u[1], u[0] * u[0])));
    double lenW = (double)sqrtf((float)fma(w[2], w[2], fma(w[1], w[1], w[0] * w[0])));
    if (lenW > 1e-8f) {
        double iw = 1.0 / lenW;
        w[0] = w[0] * iw; w[1] = w[1] * iw; w[2] = w[2] * iw;
    } else { w[0] = 0; w[1] = 0; w[2] = 1; }
    /* crossproductReal(v, w, u), expmCuda.cu:1934-1938 */
    u[0] = fma(v[1], w[2], -(v[2] * w[1]));
    u[1] = fma(-v[0], w[2], v[2] * w[0]);  /* no fused result is negated (signed zeros) */
    u[2] = fma(v[0], w[1], -(v[1] * w[0]));
    if (lenU > 1e-8f) {
        double iu = 1.0 / lenU;
        u[0] = u[0] * iu; u[1] = u[1] * iu; u[2] = u[2] * iu;
    } else { u[0] = 1; u[1] = 0; u[2] = 0; }
    v[0] = fma(w[1], u[2], -(w[2] * u[1]));
    v[1] = fma(-w[0], u[2], w[2] * u[0]);
    v[2] = fma(w[0], u[1], -(w[1] * u[0]));
    T[0] = u[0]; T[4] = u[1]; T[8] = u[2];
    T[1] = v[0]; T[5] = v[1]; T[9] = v[2];
    T[2] = w[0]; T[6] = w[1]; T[10] = w[2];
}

/* Number of squarings: EXPOKIT's int(log(||A||_inf)/log(2)) + 2 (truncation
 * toward zero), evaluated exactly with frexp. */
static int expm_squarings(double hnorm) {
    if (!(hnorm > 0.0)) return 0;
    int e;
    double mant = frexp(hnorm, &e); /* hnorm = mant * 2^e, mant in [0.5, 1) */
    int tl;
    if (hnorm >= 1.0) tl = e - 1;
    else tl = (mant == 0.5) ? e - 1 : e;
    int ns = tl + 2;
    return ns < 0 ? 0 : ns;
}

/* X = D^{-1} N for the Pade denominator and numerator of a twist.  Their last
 * rows are exactly (0 0 0 1) (a twist's last row is zero), so the elimination
 * with partial pivoting runs over rows 0..2 (pivot: first row of largest
 * |D_ik|), with reciprocal pivots; back substitution is column-oriented from
 * row 3 up.  Returns -1 if a pivot is zero. */
static int solve4(double *D, double *N) {
    double inv[3];
    for (int k = 0; k < 3; k++) {
        int p = k;
        double best = fabs(D[k * 4 + k]);
        for (int i = k + 1; i < 3; i++) {
            double v = fabs(D[i * 4 + k]);
            if (v > best) { best = v; p = i; }
        }
        if (best == 0.0) return -1;
        if (p != k) {
            for (int c = 0; c < 4; c++) {
                double t = D[k * 4 + c]; D[k * 4 + c] = D[p * 4 + c]; D[p * 4 + c] = t;
                t = N[k * 4 + c]; N[k * 4 + c] = N[p * 4 + c]; N[p * 4 + c] = t;
            }
        }
        inv[k] = 1.0 / D[k * 4 + k];
        for (int i = k + 1; i < 3; i++) {
            double f = D[i * 4 + k] * inv[k];
            for (int c = k + 1; c < 4; c++) D[i * 4 + c] = fma(-f, D[k * 4 + c], D[i * 4 + c]);
            for (int c = 0; c < 4; c++) N[i * 4 + c] = fma(-f, N[k * 4 + c], N[i * 4 + c]);
        }
    }
    for (int k = 3; k >= 1; k--) {
        for (int c = 0; c < 4; c++) {
            double xk = N[k * 4 + c];
            for (int i = 0; i < k; i++) N[i * 4 + c] = fma(-D[i * 4 + k], xk, N[i * 4 + c]);
        }
        for (int c = 0; c < 4; c++) N[(k - 1) * 4 + c] = N[(k - 1) * 4 + c] * inv[k - 1];
    }
    return 0;
}

/* exp(A) of a 4x4 twist by the diagonal (6,6) Pade approximant with scaling and
 * squaring (the method of EXPOKIT's zgpadm, Sidje 1998, used by the reference at
 * expmCuda.cu:1642 / expm.c:1669), in real FP64 arithmetic.  U0 and V are
 * evaluated by the one formula ((a I + b X2) + c X4) + d X6 (d = 0 for U0). */
void orc_expm_twist(const double A[16], double E[16]) {
    double hnorm = 0.0;
    for (int r = 0; r < 4; r++) {
        double s = 0.0;
        for (int c = 0; c < 4; c++) s = s + fabs(A[r * 4 + c]);
        if (s > hnorm) hnorm = s;
    }
    int ns = expm_squarings(hnorm);
    double scale = ldexp(1.0, -ns);
    double X[16], X2[16], X4[16], X6[16];
    for (int i = 0; i < 16; i++) X[i] = A[i] * scale;
    mat4d(X, X, X2);
    mat4d(X2, X2, X4);
    mat4d(X4, X2, X6);
    /* c_k = c_{k-1} (q-k+1) / (k (2q-k+1)), q = 6 */
    double c[7];
    c[0] = 1.0;
    for (int k = 1; k <= 6; k++) c[k] = c[k - 1] * (double)(6 - k + 1) / (double)(k * (12 - k + 1));
    double U0[16], U[16], V[16];
    for (int i = 0; i < 16; i++) {
        double I = (i % 5 == 0) ? 1.0 : 0.0;
        U0[i] = fma(0.0, X6[i], fma(c[5], X4[i], fma(c[3], X2[i], c[1] * I)));
        V[i] = fma(c[6], X6[i], fma(c[4], X4[i], fma(c[2], X2[i], c[0] * I)));
    }
    mat4d(X, U0, U);
    double Nm[16], Dm[16];
    for (int i = 0; i < 16; i++) {
        Nm[i] = V[i] + U[i];
        Dm[i] = V[i] - U[i];
    }
    if (solve4(Dm, Nm) != 0) {
        for (int i = 0; i < 16; i++) E[i] = (i % 5 == 0) ? 1.0 : 0.0;
        return;
    }
    for (int k = 0; k < ns; k++) mat4d(Nm, Nm, Nm);
    memcpy(E, Nm, sizeof(Nm));
}

/* generateA + expmKernel, warp.cu:910-915, expmCuda.cu:1989-2048: twist -> Tinc,
 * translation * scaleOut, T <- T * Tinc (right composition), stored as float. */
void orc_expm_update(const double x[6], float TF[16], double scaleOut) {
    double A[16] = {0, -x[2], x[1], x[3], x[2], 0, -x[0], x[4], -x[1], x[0], 0, x[5], 0, 0, 0, 0};
    double T[16], Tinc[16];
    double maxEntry = 0;
    for (int i = 0; i < 16; i++) {
        T[i] = TF[i];
        double a = fabs(A[i]);
        if (a > maxEntry) maxEntry = a;
    }
    if (maxEntry != 0) {
        orc_expm_twist(A, Tinc);
        normalize_mat4_safe(Tinc);
        Tinc[3] *= scaleOut;
        Tinc[7] *= scaleOut;
        Tinc[11] *= scaleOut;
    } else {
        for (int i = 0; i < 16; i++) Tinc[i] = (i % 5 == 0) ? 1.0 : 0.0;
    }
    mat4d(T, Tinc, T);
    normalize_mat4_safe(T);
    for (int i = 0; i < 16; i++) TF[i] = (float)T[i];
}

/* linearFuseKernel / linearFuseCuda, warp.cu:918-924, 1498-1509, with the normal
 * equations kept in FP64: A1 <- (w1/N1) A1 + (w2/N2) A2. */
void orc_linear_fuse(double A1[36], double b1[6], double w1, int N1, const double A2[36], const double b2[6],
                     double w2, int N2) {
    double c1 = w1 / (double)N1;
    double c2 = w2 / (double)N2;
    for (int i = 0; i < 36; i++) A1[i] = fma(c1, A1[i], c2 * A2[i]);
    for (int i = 0; i < 6; i++) b1[i] = fma(c1, b1[i], c2 * b2[i]);
}

/* ------------------------------------------------------------------ */
/* keyframe depth fusion                                               */
/* ------------------------------------------------------------------ */

/* Fuses the depth maps of nearby frames into a keyframe depth map (IR grid).
 * For every valid keyframe pixel the point is back-projected with KL
 * (rgb2gray.cu:570-593), mapped into frame f by Tframes[f] (keyframe -> frame),
 * looked up at the nearest IR pixel (the zWeight tap of warp.cu:306-327), mapped
 * back with the inverse pose (as filterDepthIIRKernel does, warp.cu:398-467),
 * gated on |dz| < gate_mm and averaged with unit weights (the weighted running
 * mean of updateVoxelsKernel, VoxelGrid_cuda.cu:1005-1013). */
void orc_fuse_depth(const float *zkey, int W, int H, const float *calib, int nframes, const float *const *zframes,
                    const float *Tframes, float gate_mm, float *zout, float *wout) {
    orc_fuse_rgbd(zkey, NULL, W, H, calib, nframes, zframes, NULL, Tframes, gate_mm, zout, wout, NULL);
}

/* Gray value the RGB camera sees at point q of its rig's IR frame: TLR,
 * distortPoint and the bilinear tap of xyz2CloudKernel's color1
 * (d2z.cu:235-331), the perspective division as one reciprocal and two
 * products.  -1 where the 2x2 taps leave the image.  Fusion only. */
static inline float rgb_sample(const float *calib, const float *q, const float *img, int W, int H) {
    float r3[3];
    mul4(&calib[TLR_OFFSET], q, r3);
    float irz = 1.0f / r3[2];
    float pux = r3[0] * irz;
    float puy = r3[1] * irz;
    float px, py;
    distort(pux, puy, &calib[KCR_OFFSET], &calib[KR_OFFSET], &px, &py);
    int xdi = ftoi(px), ydi = ftoi(py);
    if (!(xdi >= 0 && ydi >= 0 && xdi < W - 1 && ydi < H - 1)) return -1.0f;
    float fx = px - xdi, fy = py - ydi;
    return bilin(xdi, ydi, fx, fy, W, img);
}

/* Keyframe depth and colour fusion.  Depth as orc_fuse_depth.  Colour (when
 * gkey, gframes and cout are given): the vertex colour of every valid keyframe
 * pixel is the mean of the keyframe's own sample at the point (rgb_sample of
 * gkey) and the samples of the frames whose depth passed the gate (rgb_sample
 * of frame f's gray image at T_f p), the weighted running mean of
 * updateVoxelsKernel (VoxelGrid_cuda.cu:1005-1013) with unit weights, as
 * KeyFrameModel::integrateDepthMaps warps the neighbours' RGB images into the
 * keyframe (KeyFrameModel.cpp:537-583).  cout is -1 where no sample exists. */
void orc_fuse_rgbd(const float *zkey, const float *gkey, int W, int H, const float *calib, int nframes,
                   const float *const *zframes, const float *const *gframes, const float *Tframes, float gate_mm,
                   float *zout, float *wout, float *cout) {
    float minDist = calib[MIND_OFFSET];
    float maxDist = calib[MAXD_OFFSET];
    const float *KL = &calib[KL_OFFSET];
    float fx = KL[0], fy = KL[4], cx = KL[2], cy = KL[5];
    /* the divisions as products with reciprocals, as the GPU kernel states them */
    float ifx = 1.0f / fx, ify = 1.0f / fy;
    int colour = gkey && gframes && cout;
    float Tinv[8][16];
    for (int f = 0; f < nframes && f < 8; f++) invert_rt4f(&Tframes[16 * f], Tinv[f]);
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < W * H; idx++) {
        int xi = idx % W, yi = idx / W;
        float z = zkey[idx];
        if (!(z < -minDist && z > -maxDist)) {
            zout[idx] = z;
            wout[idx] = 0.0f;
            if (colour) cout[idx] = -1.0f;
            continue;
        }
        float p[3] = {((float)xi - cx) * z * ifx, ((float)yi - cy) * z * ify, z};
        float zsum = z, wsum = 1.0f;
        float csum = 0.0f, cw = 0.0f;
        if (colour) {
            float c0 = rgb_sample(calib, p, gkey, W, H);
            if (c0 >= 0.0f) {
                csum = c0;
                cw = 1.0f;
            }
        }
        for (int f = 0; f < nframes && f < 8; f++) {
            float q[3];
            mul4(&Tframes[16 * f], p, q);
            float iqz = 1.0f / q[2];
            float qx = q[0] * iqz, qy = q[1] * iqz;
            float px = KL[0] * qx + KL[1] * qy + KL[2];
            float py = KL[3] * qx + KL[4] * qy + KL[5];
            int xd = ftoi(px + 0.5f), yd = ftoi(py + 0.5f);
            if (xd < 0 || yd < 0 || xd >= W || yd >= H) continue;
            float zf = zframes[f][xd + yd * W];
            if (!(zf < -minDist && zf > -maxDist)) continue;
            float m[3] = {((float)xd - cx) * zf * ifx, ((float)yd - cy) * zf * ify, zf};
            float mk[3];
            mul4(Tinv[f], m, mk);
            float dz = mk[2] - z;
            if (fabsf(dz) < gate_mm) {
                zsum += mk[2];
                wsum += 1.0f;
                if (colour) {
                    float c = rgb_sample(calib, q, gframes[f], W, H);
                    if (c >= 0.0f) {
                        csum += c;
                        cw += 1.0f;
                    }
                }
            }
        }
        zout[idx] = zsum / wsum;
        wout[idx] = wsum;
        if (colour) cout[idx] = cw > 0.0f ? csum / cw : -1.0f;
    }
}

/* ------------------------------------------------------------------ */
/* procedural scene, CPU twin                                          */
/* ------------------------------------------------------------------ */

void orc_render_depth(const recon_scene *sc, const recon_camera *cam, float noise_rel, uint32_t noise_seed,
                      uint32_t frame, uint16_t *out) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < cam->height; y++)
        for (int x = 0; x < cam->width; x++)
            out[y * cam->width + x] = scene_depth_pixel(sc, cam, x, y, noise_rel, noise_seed, frame);
}

void orc_render_gray(const recon_scene *sc, const recon_camera *cam, uint8_t *out) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < cam->height; y++)
        for (int x = 0; x < cam->width; x++) out[y * cam->width + x] = scene_gray_pixel(sc, cam, x, y);
}

/* ------------------------------------------------------------------ */
/* operator-level tracker: PhotoTracker + ShapeTracker schedule        */
/* ------------------------------------------------------------------ */

struct orc_tracker {
    orc_config cfg;
    float calib[ORC_CALIB_SIZE];
    int W, H, L, P;
    /* reference */
    float *ref_gray[ORC_MAX_LEVELS];
    float *ref_z;
    float *ref_col;    /* fused vertex colour per IR pixel (orc_fuse_rgbd), valid when has_col */
    int has_col;
    float *ref_xyzw;
    float *vdata;
    int32_t *sel_idx;
    int32_t sel_written;
    float *sel_xyz;
    float *sel_I[ORC_MAX_LEVELS];
    float *sel_J[ORC_MAX_LEVELS];
    float *ref6[ORC_MAX_LEVELS];
    int32_t *refmask[ORC_MAX_LEVELS];
    /* current */
    float *cur_gray[ORC_MAX_LEVELS];
    float *cur_z;
    float *cur6[ORC_MAX_LEVELS];
    int32_t *curmask[ORC_MAX_LEVELS];
    /* scratch */
    float *r, *zw, *w, *rw, *Jw[6];
    float *full_res;
    int32_t *rmask, *select;
    float *icp_r, *icp_r2, *icp_w, *icp_J, *icp_res;
    float *icp_wpx;    /* the level's Student-t weights per pixel, 0 where not selected */
    /* mixed precision: the stored (rounded) copies the photometric term reads */
    float *cur_gray_q[ORC_MAX_LEVELS], *sel_I_q[ORC_MAX_LEVELS], *sel_J_q[ORC_MAX_LEVELS];
    int32_t *all_px;   /* 0, 1, 2, ...: every pixel of the level in order */
    int32_t nsel[ORC_MAX_LEVELS];
    int has_ref, has_cur;
    float T[16];
};

static void *xmalloc(size_t n) {
    void *p = calloc(1, n ? n : 1);
    if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
    return p;
}

orc_tracker *orc_create(const orc_config *cfg, const float *calib) {
    orc_tracker *t = (orc_tracker *)xmalloc(sizeof(orc_tracker));
    t->cfg = *cfg;
    memcpy(t->calib, calib, sizeof(t->calib));
    t->W = cfg->width;
    t->H = cfg->height;
    t->L = cfg->levels;
    t->P = cfg->n_select;
    int W = t->W, H = t->H, P = t->P;
    for (int l = 0; l < t->L; l++) {
        int n = (W >> l) * (H >> l);
        t->ref_gray[l] = (float *)xmalloc(n * sizeof(float));
        t->cur_gray[l] = (float *)xmalloc(n * sizeof(float));
        t->ref6[l] = (float *)xmalloc(6 * n * sizeof(float));
        t->cur6[l] = (float *)xmalloc(6 * n * sizeof(float));
        t->refmask[l] = (int32_t *)xmalloc(n * sizeof(int32_t));
        t->curmask[l] = (int32_t *)xmalloc(n * sizeof(int32_t));
        t->sel_I[l] = (float *)xmalloc(P * sizeof(float));
        t->sel_J[l] = (float *)xmalloc(6 * P * sizeof(float));
    }
    t->ref_z = (float *)xmalloc(W * H * sizeof(float));
    t->ref_col = (float *)xmalloc(W * H * sizeof(float));
    t->cur_z = (float *)xmalloc(W * H * sizeof(float));
    t->ref_xyzw = (float *)xmalloc(4 * W * H * sizeof(float));
    t->vdata = (float *)xmalloc(24 * (size_t)W * H * sizeof(float));
    t->sel_idx = (int32_t *)xmalloc(P * sizeof(int32_t));
    t->sel_xyz = (float *)xmalloc(3 * P * sizeof(float));
    t->r = (float *)xmalloc(P * sizeof(float));
    t->zw = (float *)xmalloc(P * sizeof(float));
    t->w = (float *)xmalloc(P * sizeof(float));
    t->rw = (float *)xmalloc(P * sizeof(float));
    for (int c = 0; c < 6; c++) t->Jw[c] = (float *)xmalloc(P * sizeof(float));
    int npmax = ((W * H + ORC_CHUNK - 1) / ORC_CHUNK) * ORC_CHUNK;
    t->full_res = (float *)xmalloc(W * H * sizeof(float));
    t->rmask = (int32_t *)xmalloc(W * H * sizeof(int32_t));
    t->select = (int32_t *)xmalloc(W * H * sizeof(int32_t));
    t->icp_r = (float *)xmalloc(npmax * sizeof(float));
    t->icp_r2 = (float *)xmalloc(npmax * sizeof(float));
    t->icp_w = (float *)xmalloc(npmax * sizeof(float));
    t->icp_res = (float *)xmalloc(npmax * sizeof(float));
    t->icp_J = (float *)xmalloc(6 * (size_t)npmax * sizeof(float));
    t->icp_wpx = (float *)xmalloc(npmax * sizeof(float));
    if (cfg->precision == 1)
        for (int l = 0; l < t->L; l++) {
            t->cur_gray_q[l] = (float *)xmalloc((size_t)(W >> l) * (H >> l) * sizeof(float));
            t->sel_I_q[l] = (float *)xmalloc(P * sizeof(float));
            t->sel_J_q[l] = (float *)xmalloc(6 * (size_t)P * sizeof(float));
        }
    t->all_px = (int32_t *)xmalloc(W * H * sizeof(int32_t));
    for (int i = 0; i < W * H; i++) t->all_px[i] = i;
    for (int i = 0; i < 16; i++) t->T[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    return t;
}

void orc_destroy(orc_tracker *t) {
    if (!t) return;
    for (int l = 0; l < t->L; l++) {
        free(t->ref_gray[l]); free(t->cur_gray[l]); free(t->ref6[l]); free(t->cur6[l]);
        free(t->refmask[l]); free(t->curmask[l]); free(t->sel_I[l]); free(t->sel_J[l]);
    }
    free(t->ref_z); free(t->ref_col); free(t->cur_z); free(t->ref_xyzw); free(t->vdata); free(t->sel_idx); free(t->sel_xyz);
    free(t->r); free(t->zw); free(t->w); free(t->rw);
    for (int c = 0; c < 6; c++) free(t->Jw[c]);
    free(t->full_res); free(t->rmask); free(t->select);
    free(t->icp_r); free(t->icp_r2); free(t->icp_w); free(t->icp_res); free(t->icp_J);
    free(t->icp_wpx); free(t->all_px);
    for (int l = 0; l < ORC_MAX_LEVELS; l++) { free(t->cur_gray_q[l]); free(t->sel_I_q[l]); free(t->sel_J_q[l]); }
    free(t);
}

/* PhotoTracker::prepareReference + selectPixels (phototracker.cpp:338-386) and
 * ShapeTracker::setReferencePoints + prepareReference (shapetracker.cpp:205-288) */
static int prepare_reference(orc_tracker *t, const float *gray0, const float *z0, int reset_pose) {
    int W = t->W, H = t->H, L = t->L, P = t->P;
    if (gray0) memcpy(t->ref_gray[0], gray0, W * H * sizeof(float));
    memcpy(t->ref_z, z0, W * H * sizeof(float));
    for (int l = 1; l < L; l++) orc_downsample2(t->ref_gray[l - 1], W >> l, H >> l, t->ref_gray[l]);
    /* photometric */
    orc_zmap_to_xyz(t->ref_z, W, H, t->calib, t->ref_xyzw);
    orc_xyz2cloud_col(t->ref_xyzw, W, H, t->calib, t->ref_gray[0], t->has_col ? t->ref_col : NULL, t->vdata);
    float *grad = (float *)xmalloc(W * H * sizeof(float));
    for (int i = 0; i < W * H; i++) grad[i] = t->vdata[i * 24 + 13];
    int32_t hist[1024];
    int nb = t->cfg.select_bins;
    orc_grad_histogram(grad, W * H, nb, hist);
    t->sel_written = orc_filter_indices(grad, W * H, hist, nb, P, t->sel_idx);
    free(grad);
    const float *gl[ORC_MAX_LEVELS];
    for (int l = 0; l < L; l++) gl[l] = t->ref_gray[l];
    orc_add_vertex_attributes(t->sel_idx, P, t->vdata, W, H, t->calib, gl, L);
    orc_precompute_jacobian(t->sel_idx, P, t->vdata, t->calib, t->cfg.opt_scale_in, L, t->sel_J);
    static const int cslot[4] = {14, 17, 20, 23};
    for (int k = 0; k < P; k++) {
        const float *v = &t->vdata[t->sel_idx[k] * 24];
        t->sel_xyz[k] = v[0];
        t->sel_xyz[P + k] = v[1];
        t->sel_xyz[2 * P + k] = v[2];
        for (int l = 0; l < L; l++) t->sel_I[l][k] = v[cslot[l]];
    }
    /* geometric */
    orc_zmap_to_xyz6(t->ref_z, W, H, t->calib, t->ref6[0], t->refmask[0]);
    orc_compute_normals6(t->ref6[0], t->refmask[0], W, H);
    for (int l = 1; l < L; l++)
        orc_downsample_cloud6(t->ref6[l - 1], t->refmask[l - 1], W >> l, H >> l, t->ref6[l], t->refmask[l]);
    if (t->cfg.precision == 1)
        for (int l = 0; l < L; l++) {
            for (int k = 0; k < P; k++) t->sel_I_q[l][k] = orc_f16_round(t->sel_I[l][k]);
            for (int k = 0; k < 6 * P; k++) t->sel_J_q[l][k] = orc_bf16_round(t->sel_J[l][k]);
        }
    if (reset_pose)
        for (int i = 0; i < 16; i++) t->T[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    t->has_ref = 1;
    return 0;
}

int orc_set_reference_float(orc_tracker *t, const float *gray0, const float *z0) {
    t->has_col = 0;
    return prepare_reference(t, gray0, z0, 1);
}

/* genOrientedPoints6Kernel (d2z.cu:471-501): an ICP point and normal from a
 * ray-cast point image and its normals (float4 each) where z < 0 and the
 * normal is not zero, else zeros */
void orc_gen_oriented_points6(const float *xyz4, const float *nrm4, int W, int H, float *pts6, int32_t *mask) {
    for (int i = 0; i < W * H; i++) {
        const float *v = xyz4 + 4 * i, *n = nrm4 + 4 * i;
        float *o = pts6 + 6 * i;
        float len = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
        if (v[2] < 0 && len > 1e-7f) {
            o[0] = v[0]; o[1] = v[1]; o[2] = v[2];
            o[3] = n[0]; o[4] = n[1]; o[5] = n[2];
            mask[i] = 1;
        } else {
            for (int k = 0; k < 6; k++) o[k] = 0;
            mask[i] = 0;
        }
    }
}

/* The filtered reference (PhotoTracker::setReferencePoints with
 * setFilteredReference(true), phototracker.cpp:310-337; ShapeTracker::
 * setReferencePoints, shapetracker.cpp:195-212): photometric reference from
 * the frame, ICP level 0 from the oriented points, coarser levels by
 * downSampleCloud6 (shapetracker.cpp:276-288). */
int orc_set_reference_oriented(orc_tracker *t, const uint8_t *gray, const uint16_t *depth, const float *xyz4,
                               const float *nrm4) {
    int rc = orc_set_reference(t, gray, depth);
    if (rc) return rc;
    int W = t->W, H = t->H;
    orc_gen_oriented_points6(xyz4, nrm4, W, H, t->ref6[0], t->refmask[0]);
    for (int l = 1; l < t->L; l++)
        orc_downsample_cloud6(t->ref6[l - 1], t->refmask[l - 1], W >> l, H >> l, t->ref6[l], t->refmask[l]);
    return 0;
}

/* Keyframe fusion of nframes depth maps (uint16 mm) with their tracked poses
 * (keyframe -> frame), then the reference is rebuilt from the fused depth
 * with the keyframe's gray image; the current pose is kept. */
int orc_fuse_keyframe(orc_tracker *t, int nframes, const uint16_t *const *depth, const float *Tframes, float gate) {
    return orc_fuse_keyframe_rgbd(t, nframes, NULL, depth, Tframes, gate);
}

/* The same with the frames' gray images (uint8, RGB camera): the keyframe's
 * vertex colours become the fused colours (orc_fuse_rgbd).  gray NULL fuses
 * depth only and leaves the colours as they were. */
int orc_fuse_keyframe_rgbd(orc_tracker *t, int nframes, const uint8_t *const *gray, const uint16_t *const *depth,
                           const float *Tframes, float gate) {
    if (!t->has_ref || nframes < 0 || nframes > 8) return -1;
    int n = t->W * t->H;
    float *zf[8], *gf[8];
    for (int f = 0; f < nframes; f++) {
        zf[f] = (float *)xmalloc(n * sizeof(float));
        orc_convert_depth(depth[f], n, zf[f]);
        gf[f] = NULL;
        if (gray) {
            gf[f] = (float *)xmalloc(n * sizeof(float));
            orc_convert_gray(gray[f], n, gf[f]);
        }
    }
    float *zout = (float *)xmalloc(n * sizeof(float));
    float *wout = (float *)xmalloc(n * sizeof(float));
    orc_fuse_rgbd(t->ref_z, gray ? t->ref_gray[0] : NULL, t->W, t->H, t->calib, nframes, (const float *const *)zf,
                  gray ? (const float *const *)gf : NULL, Tframes, gate, zout, wout, gray ? t->ref_col : NULL);
    if (gray) t->has_col = 1;
    int rc = prepare_reference(t, NULL, zout, 0);
    for (int f = 0; f < nframes; f++) {
        free(zf[f]);
        free(gf[f]);
    }
    free(zout);
    free(wout);
    return rc;
}

int orc_set_reference(orc_tracker *t, const uint8_t *gray, const uint16_t *depth) {
    int n = t->W * t->H;
    float *g = (float *)xmalloc(n * sizeof(float));
    float *z = (float *)xmalloc(n * sizeof(float));
    orc_convert_gray(gray, n, g);
    orc_convert_depth(depth, n, z);
    int rc = orc_set_reference_float(t, g, z);
    free(g);
    free(z);
    return rc;
}

/* PhotoTracker::setCurrentImage + prepareCurrent, ShapeTracker::prepareCurrent
 * (phototracker.cpp:236-245, 483-485; shapetracker.cpp:260-271) */
int orc_set_current(orc_tracker *t, const uint8_t *gray, const uint16_t *depth) {
    int W = t->W, H = t->H, L = t->L;
    orc_convert_gray(gray, W * H, t->cur_gray[0]);
    orc_convert_depth(depth, W * H, t->cur_z);
    for (int l = 1; l < L; l++) orc_downsample2(t->cur_gray[l - 1], W >> l, H >> l, t->cur_gray[l]);
    orc_gen_cloud6(t->cur_z, W, H, t->calib, t->cur6[0], t->curmask[0]);
    for (int l = 1; l < L; l++)
        orc_downsample_cloud6(t->cur6[l - 1], t->curmask[l - 1], W >> l, H >> l, t->cur6[l], t->curmask[l]);
    if (t->cfg.precision == 1)
        for (int l = 0; l < L; l++)
            for (int i = 0; i < (W >> l) * (H >> l); i++) t->cur_gray_q[l][i] = orc_f16_round(t->cur_gray[l][i]);
    t->has_cur = 1;
    return 0;
}

/* The learned start pose (k_init_gate): x = net_out * scale (FP32), D =
 * exp(A(x)) applied to the identity by orc_expm_update, candidate D * T; the
 * candidate replaces T when its integer cost sum_i min(trunc(|r_i| * 1024),
 * 1024) over the coarsest level's photometric residuals is strictly lower.
 * Returns 1 when the candidate was taken. */
static long long gate_cost(orc_tracker *t, const float *T) {
    int L = t->L, layer = L - 1, P = t->P;
    orc_interpolate_residual(P, t->sel_xyz, t->sel_I[layer], T, t->calib, layer, t->cur_gray[layer], t->W >> layer,
                             t->H >> layer, t->cur_z, t->W, t->H, t->r, t->zw);
    long long c = 0;
    for (int i = 0; i < P; i++) {
        float u = fabsf(t->r[i]) * 1024.0f;
        c += (u >= 1024.0f || !(u == u)) ? 1024 : (long long)u;
    }
    return c;
}

int orc_init_gate(orc_tracker *t, const float net_out[6], const float scale[6]) {
    float Dm[16], Tc[16];
    for (int i = 0; i < 16; i++) Dm[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    double x[6];
    for (int k = 0; k < 6; k++) x[k] = (double)(net_out[k] * scale[k]);
    orc_expm_update(x, Dm, (double)t->cfg.opt_scale_out);
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++)
            Tc[r * 4 + c] = Dm[r * 4 + 0] * t->T[0 * 4 + c] + Dm[r * 4 + 1] * t->T[1 * 4 + c] +
                            Dm[r * 4 + 2] * t->T[2 * 4 + c] + Dm[r * 4 + 3] * t->T[3 * 4 + c];
    long long c0 = gate_cost(t, t->T), c1 = gate_cost(t, Tc);
    if (c1 < c0) {
        memcpy(t->T, Tc, sizeof(Tc));
        return 1;
    }
    return 0;
}

void orc_set_pose(orc_tracker *t, const float T[16]) { memcpy(t->T, T, sizeof(t->T)); }
void orc_get_pose(orc_tracker *t, float T[16]) { memcpy(T, t->T, sizeof(t->T)); }

static int padded_len(int n) { return ((n + ORC_CHUNK - 1) / ORC_CHUNK) * ORC_CHUNK; }

int orc_pose_settled(const float Ta[16], const float Tb[16], float tol_mm, float tol_rot) {
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) {
            float dv = fabsf(Tb[r * 4 + c] - Ta[r * 4 + c]);
            if (!(dv <= (c == 3 ? tol_mm : tol_rot))) return 0;
        }
    return 1;
}

/* PhotoTracker::gpuEstimateIncrement (phototracker.cpp:666-689) with
 * updateLinearSystem (505-511), ShapeTracker::updateLinearSystem
 * (shapetracker.cpp:357-382) and estimateIncrement (646-664).  T is the pose
 * (reference IR -> current IR); if T is non-NULL on entry it replaces the
 * tracker's pose before the schedule and receives the result. */
int orc_track(orc_tracker *t, float *Tio, orc_iter_trace *trace, int max_trace) {
    if (!t->has_ref || !t->has_cur) return -1;
    int W = t->W, H = t->H, L = t->L, P = t->P;
    int mode = t->cfg.mode;
    if (Tio) memcpy(t->T, Tio, sizeof(t->T));
    int ntr = 0;
    for (int layer = L - 1; layer >= 0; layer--) {
        int n = t->cfg.iters[L - 1 - layer];
        int wl = W >> layer, hl = H >> layer;
        for (int j = 0; j < n; j++) {
            double A_ph[36] = {0}, b_ph[6] = {0}, A_icp[36] = {0}, b_icp[6] = {0};
            int32_t hist[256];
            int median = -1;
            int ok = 1;
            if (mode == ORC_PHOTOMETRIC || mode == ORC_BIOBJECTIVE) {
                /* mixed precision reads the rounded copies; the arithmetic is the same */
                int mixed = t->cfg.precision == 1;
                const float *selI = mixed ? t->sel_I_q[layer] : t->sel_I[layer];
                const float *img = mixed ? t->cur_gray_q[layer] : t->cur_gray[layer];
                const float *selJ = mixed ? t->sel_J_q[layer] : t->sel_J[layer];
                orc_interpolate_residual(P, t->sel_xyz, selI, t->T, t->calib, layer, img, wl, hl, t->cur_z, W, H, t->r,
                                         t->zw);
                median = orc_generate_weights(t->r, t->zw, P, t->cfg.hist_bins, hist, t->w, t->rw);
                for (int c = 0; c < 6; c++)
                    for (int i = 0; i < P; i++) t->Jw[c][i] = selJ[c * P + i] * t->w[i];
                const float *J6[6];
                for (int c = 0; c < 6; c++) J6[c] = t->Jw[c];
                orc_fx27 acc;
                orc_fx27_clear(&acc);
                orc_reduce27_fx(J6, t->rw, P, &acc);
                orc_fx27_value(&acc, A_ph, b_ph);
            }
            if (mode == ORC_GEOMETRIC || mode == ORC_BIOBJECTIVE) {
                if (j == 0) {
                    orc_icp_residual_mask(t->ref6[layer], t->refmask[layer], wl, hl, t->T, t->calib,
                                          t->cur6[layer], t->curmask[layer], layer, t->full_res, t->rmask);
                    t->nsel[layer] = orc_compact(t->rmask, wl * hl, t->select);
                    if (t->nsel[layer] > 0) {
                        for (int k = 0; k < t->nsel[layer]; k++) {
                            float rv = t->full_res[t->select[k]];
                            t->icp_r[k] = rv;
                            t->icp_r2[k] = rv * rv;
                        }
                        orc_student_t(t->icp_r2, t->nsel[layer], t->icp_w);
                    }
                    memset(t->icp_wpx, 0, (size_t)wl * hl * sizeof(float));
                    for (int k = 0; k < t->nsel[layer]; k++) t->icp_wpx[t->select[k]] = t->icp_w[k];
                }
                int ns = t->nsel[layer];
                if (ns <= 0) {
                    ok = 0;
                } else {
                    /* The canonical FP32 stage of the ICP sums runs over the
                     * level's pixel grid in 1024-pixel chunks; a pixel that was
                     * not selected has weight 0 and contributes exact zeros. */
                    int npx = wl * hl, np = padded_len(npx);
                    orc_icp_residual_jacobian_grid(t->ref6[layer], wl, hl, layer, t->T, t->calib, t->cur6[layer],
                                                   t->curmask[layer], np, t->icp_res, t->icp_J, t->icp_wpx,
                                                   t->cfg.opt_scale_in);
                    const float *J6[6];
                    for (int c = 0; c < 6; c++) J6[c] = t->icp_J + (size_t)c * np;
                    orc_fx27 acc;
                    orc_fx27_clear(&acc);
                    orc_reduce27_fx(J6, t->icp_res, np, &acc);
                    orc_fx27_value(&acc, A_icp, b_icp);
                }
            }
            double A[36], b[6];
            if (mode == ORC_PHOTOMETRIC) {
                memcpy(A, A_ph, sizeof(A));
                memcpy(b, b_ph, sizeof(b));
            } else if (mode == ORC_GEOMETRIC) {
                memcpy(A, A_icp, sizeof(A));
                memcpy(b, b_icp, sizeof(b));
            } else {
                memcpy(A, A_ph, sizeof(A));
                memcpy(b, b_ph, sizeof(b));
                if (ok)
                    orc_linear_fuse(A, b, (double)(1.0f - t->cfg.lambda), P, A_icp, b_icp, (double)t->cfg.lambda,
                                    t->nsel[layer]);
            }
            int status = 0;
            float T_before[16];
            memcpy(T_before, t->T, sizeof(T_before));
            if (ok) {
                double x[6];
                if (t->cfg.solver == ORC_SOLVER_CG) {
                    orc_solve_cg(A, b, 1e-8, 6, x);
                } else {
                    status = orc_solve_cholesky(A, b, x);
                }
                orc_expm_update(x, t->T, (double)t->cfg.opt_scale_out);
            }
            if (trace && ntr < max_trace) {
                orc_iter_trace *tr = &trace[ntr];
                memset(tr, 0, sizeof(*tr));
                tr->level = layer;
                tr->iter = j;
                tr->mode = mode;
                tr->solved = ok;
                tr->status = status;
                tr->icp_selected = (mode != ORC_PHOTOMETRIC) ? t->nsel[layer] : 0;
                memcpy(tr->T, t->T, sizeof(tr->T));
                memcpy(tr->A, A, sizeof(A));
                memcpy(tr->b, b, sizeof(b));
                memcpy(tr->A_ph, A_ph, sizeof(A_ph));
                memcpy(tr->b_ph, b_ph, sizeof(b_ph));
                memcpy(tr->A_icp, A_icp, sizeof(A_icp));
                memcpy(tr->b_icp, b_icp, sizeof(b_icp));
                if (median >= 0) memcpy(tr->hist, hist, t->cfg.hist_bins * sizeof(int32_t));
                tr->median_bin = median;
            }
            ntr++;
            /* the level ends early once the pose has settled (off at settle_mm 0) */
            if (t->cfg.settle_mm > 0.0f && orc_pose_settled(T_before, t->T, t->cfg.settle_mm, t->cfg.settle_rot))
                break;
        }
    }
    if (Tio) memcpy(Tio, t->T, sizeof(t->T));
    return ntr;
}

int orc_n_icp_selected(orc_tracker *t, int level) { return t->nsel[level]; }

/* copy out internal arrays for the tests */
int orc_get_array(orc_tracker *t, const char *name, int level, void *dst, int64_t nbytes) {
    int W = t->W >> level, H = t->H >> level, P = t->P;
    const void *src = NULL;
    int64_t n = 0;
    if (!strcmp(name, "ref_gray")) { src = t->ref_gray[level]; n = (int64_t)W * H * 4; }
    else if (!strcmp(name, "cur_gray")) { src = t->cur_gray[level]; n = (int64_t)W * H * 4; }
    else if (!strcmp(name, "ref6")) { src = t->ref6[level]; n = (int64_t)W * H * 24; }
    else if (!strcmp(name, "cur6")) { src = t->cur6[level]; n = (int64_t)W * H * 24; }
    else if (!strcmp(name, "refmask")) { src = t->refmask[level]; n = (int64_t)W * H * 4; }
    else if (!strcmp(name, "curmask")) { src = t->curmask[level]; n = (int64_t)W * H * 4; }
    else if (!strcmp(name, "sel_idx")) { src = t->sel_idx; n = (int64_t)P * 4; }
    else if (!strcmp(name, "sel_xyz")) { src = t->sel_xyz; n = (int64_t)P * 12; }
    else if (!strcmp(name, "sel_I")) { src = t->sel_I[level]; n = (int64_t)P * 4; }
    else if (!strcmp(name, "sel_J")) { src = t->sel_J[level]; n = (int64_t)P * 24; }
    else if (!strcmp(name, "vdata")) { src = t->vdata; n = (int64_t)t->W * t->H * 96; }
    else if (!strcmp(name, "cur_z")) { src = t->cur_z; n = (int64_t)t->W * t->H * 4; }
    else if (!strcmp(name, "ref_z")) { src = t->ref_z; n = (int64_t)t->W * t->H * 4; }
    else if (!strcmp(name, "ref_col")) { src = t->ref_col; n = (int64_t)t->W * t->H * 4; }
    else if (!strcmp(name, "T")) { src = t->T; n = 64; }
    else if (!strcmp(name, "icp_w")) { src = t->icp_w; n = (int64_t)t->nsel[level] * 4; }
    else if (!strcmp(name, "icp_select")) { src = t->select; n = (int64_t)t->nsel[level] * 4; }
    else if (!strcmp(name, "icp_w_px")) { src = t->icp_wpx; n = (int64_t)W * H * 4; }
    else return -1;
    if (n > nbytes) return -2;
    memcpy(dst, src, (size_t)n);
    return (int)n;
}
