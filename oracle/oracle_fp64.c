/*
 * oracle_fp64.c -- FP64 oracle of the recon dense RGB-D tracker.
 *
 * TEST INFRASTRUCTURE ONLY (the judge of pose error in the tests and the
 * benchmark; the product library never links it).  It runs the same algorithm
 * as the FP32 oracle (oracle.c) and the reference it restates -- input
 * conversion, pyramids, pixel selection, vertex attributes and photometric
 * Jacobians, the warped photometric residual with its depth weight, the
 * histogram-MAD Tukey weights, the ICP correspondences, Student-t weights and
 * point-to-plane Jacobians, the bi-objective fusion, the 6x6 solve, the SE(3)
 * exponential update and the keyframe depth/colour fusion -- with every
 * floating-point operation in double precision and the pose kept in double
 * between iterations and frames.  What stays as in the reference is the
 * algorithm's own integer steps: histogram bins, the selection's trimming
 * rule, the tap indices, the Student-t sum of truncated products.
 *
 * Each step cites the reference file:line it follows (the FP32 oracle states
 * the same steps in FP32, in the reference's operation order).  Sums of the
 * normal equations run in fixed chunks of 1024 points whose partial sums are
 * added in chunk order, so the result does not depend on the thread count.
 */
#define _POSIX_C_SOURCE 200809L
#include "oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <limits.h>

typedef double R;

#define KR 0
#define KCR 18
#define TLR 26
#define KLo 43
#define MIND 62
#define MAXD 63
#define TRL 64

static inline int dtoi(R x) {
    if (!(x > -2147483520.0 && x < 2147483520.0)) return INT_MIN;
    return (int)x;
}

/* matrixMultVec4 / matrixRot4 / matrixMultVec3, kernelUtils.h:217-236 */
static inline void mul4(const R *M, const R *v, R *r) {
    r[0] = M[0] * v[0] + M[1] * v[1] + M[2] * v[2] + M[3];
    r[1] = M[4] * v[0] + M[5] * v[1] + M[6] * v[2] + M[7];
    r[2] = M[8] * v[0] + M[9] * v[1] + M[10] * v[2] + M[11];
}
static inline void rot4(const R *M, const R *v, R *r) {
    r[0] = M[0] * v[0] + M[1] * v[1] + M[2] * v[2];
    r[1] = M[4] * v[0] + M[5] * v[1] + M[6] * v[2];
    r[2] = M[8] * v[0] + M[9] * v[1] + M[10] * v[2];
}
static inline void mul3(const R *M, const R *v, R *r) {
    r[0] = M[0] * v[0] + M[1] * v[1] + M[2] * v[2];
    r[1] = M[3] * v[0] + M[4] * v[1] + M[5] * v[2];
    r[2] = M[6] * v[0] + M[7] * v[1] + M[8] * v[2];
}

/* distortPoint, kernelUtils.h:394-408 */
static inline void distort(R pux, R puy, const R *kc, const R *K, R *pdx, R *pdy) {
    R r2 = pux * pux + puy * puy;
    R r4 = r2 * r2, r6 = r4 * r2;
    R rd = 1 + kc[0] * r2 + kc[1] * r4 + kc[4] * r6;
    *pdx = K[0] * pux * rd + K[2];
    *pdy = K[4] * puy * rd + K[5];
}

/* bilinearInterpolation, kernelUtils.h:298-303 */
static inline R bilin(int xdi, int ydi, R fx, R fy, int width, const R *src) {
    int o = xdi + ydi * width;
    return (1 - fx) * (1 - fy) * src[o] + fx * (1 - fy) * src[o + 1] + (1 - fx) * fy * src[o + width] +
           fx * fy * src[o + width + 1];
}

/* the same with taps clamped into the image (the FP32 oracle's bilin_clamped) */
static inline R bilin_clamped(int xdi, int ydi, R fx, R fy, int w, int h, const R *src) {
    int x0 = xdi < 0 ? 0 : (xdi > w - 1 ? w - 1 : xdi);
    int x1 = xdi + 1 < 0 ? 0 : (xdi + 1 > w - 1 ? w - 1 : xdi + 1);
    int y0 = ydi < 0 ? 0 : (ydi > h - 1 ? h - 1 : ydi);
    int y1 = ydi + 1 < 0 ? 0 : (ydi + 1 > h - 1 ? h - 1 : ydi + 1);
    return (1 - fx) * (1 - fy) * src[x0 + y0 * w] + fx * (1 - fy) * src[x1 + y0 * w] +
           (1 - fx) * fy * src[x0 + y1 * w] + fx * fy * src[x1 + y1 * w];
}

/* inBounds, kernelUtils.h:341-344 */
static inline int in_bounds10(R px, R py, int w, int h) {
    return (px >= 10 && px < (w - 10) && py >= 10 && py < (h - 10));
}

/* normalize3Cuda, kernelUtils.h:41-50 */
static inline void normalize3(R *v) {
    R len = 1.0 / sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] *= len;
    v[1] *= len;
    v[2] *= len;
}

static void invert_rt4(const R *M, R *Mi) {
    Mi[0] = M[0]; Mi[1] = M[4]; Mi[2] = M[8];   Mi[3] = -(M[0] * M[3] + M[4] * M[7] + M[8] * M[11]);
    Mi[4] = M[1]; Mi[5] = M[5]; Mi[6] = M[9];   Mi[7] = -(M[1] * M[3] + M[5] * M[7] + M[9] * M[11]);
    Mi[8] = M[2]; Mi[9] = M[6]; Mi[10] = M[10]; Mi[11] = -(M[2] * M[3] + M[6] * M[7] + M[10] * M[11]);
    Mi[12] = 0;   Mi[13] = 0;   Mi[14] = 0;     Mi[15] = 1;
}

static void *xcalloc(size_t n) {
    void *p = calloc(1, n ? n : 1);
    if (!p) { fprintf(stderr, "oracle64: out of memory\n"); abort(); }
    return p;
}

/* ------------------------------------------------------------------ */
/* tracker state                                                       */
/* ------------------------------------------------------------------ */

struct orc64_tracker {
    orc_config cfg;
    R calib[ORC_CALIB_SIZE];
    int W, H, L, P;
    /* reference */
    R *ref_gray[ORC_MAX_LEVELS], *ref_z, *ref_col;
    int has_col;
    R *vx, *vy, *vz, *vgx, *vgy, *vgm, *vcol;   /* level-0 vertex planes (xyz2CloudKernel) */
    int32_t *sel_idx;
    R *sel_xyz, *sel_I[ORC_MAX_LEVELS], *sel_J[ORC_MAX_LEVELS];
    R *ref6[ORC_MAX_LEVELS];
    int32_t *refmask[ORC_MAX_LEVELS];
    /* current */
    R *cur_gray[ORC_MAX_LEVELS], *cur_z, *cur6[ORC_MAX_LEVELS];
    int32_t *curmask[ORC_MAX_LEVELS];
    /* scratch */
    R *r, *zw, *w, *full_res, *icp_wpx, *icp_r2, *icp_w, *partial;
    int32_t *rmask, *select;
    int nsel[ORC_MAX_LEVELS];
    int has_ref, has_cur;
    R T[16];
};

orc64_tracker *orc64_create(const orc_config *cfg, const float *calib) {
    orc64_tracker *t = (orc64_tracker *)xcalloc(sizeof(orc64_tracker));
    t->cfg = *cfg;
    for (int i = 0; i < ORC_CALIB_SIZE; i++) t->calib[i] = (R)calib[i];
    t->W = cfg->width;
    t->H = cfg->height;
    t->L = cfg->levels;
    t->P = cfg->n_select;
    size_t n = (size_t)t->W * t->H, P = (size_t)t->P;
    for (int l = 0; l < t->L; l++) {
        size_t nl = (size_t)(t->W >> l) * (t->H >> l);
        t->ref_gray[l] = (R *)xcalloc(nl * sizeof(R));
        t->cur_gray[l] = (R *)xcalloc(nl * sizeof(R));
        t->ref6[l] = (R *)xcalloc(6 * nl * sizeof(R));
        t->cur6[l] = (R *)xcalloc(6 * nl * sizeof(R));
        t->refmask[l] = (int32_t *)xcalloc(nl * sizeof(int32_t));
        t->curmask[l] = (int32_t *)xcalloc(nl * sizeof(int32_t));
        t->sel_I[l] = (R *)xcalloc(P * sizeof(R));
        t->sel_J[l] = (R *)xcalloc(6 * P * sizeof(R));
    }
    t->ref_z = (R *)xcalloc(n * sizeof(R));
    t->ref_col = (R *)xcalloc(n * sizeof(R));
    t->cur_z = (R *)xcalloc(n * sizeof(R));
    R **planes[7] = {&t->vx, &t->vy, &t->vz, &t->vgx, &t->vgy, &t->vgm, &t->vcol};
    for (int k = 0; k < 7; k++) *planes[k] = (R *)xcalloc(n * sizeof(R));
    t->sel_idx = (int32_t *)xcalloc(P * sizeof(int32_t));
    t->sel_xyz = (R *)xcalloc(3 * P * sizeof(R));
    t->r = (R *)xcalloc(P * sizeof(R));
    t->zw = (R *)xcalloc(P * sizeof(R));
    t->w = (R *)xcalloc(P * sizeof(R));
    t->full_res = (R *)xcalloc(n * sizeof(R));
    t->icp_wpx = (R *)xcalloc(n * sizeof(R));
    t->icp_r2 = (R *)xcalloc(n * sizeof(R));
    t->icp_w = (R *)xcalloc(n * sizeof(R));
    t->partial = (R *)xcalloc(((n + ORC_CHUNK - 1) / ORC_CHUNK + P / ORC_CHUNK + 1) * 27 * sizeof(R));
    t->rmask = (int32_t *)xcalloc(n * sizeof(int32_t));
    t->select = (int32_t *)xcalloc(n * sizeof(int32_t));
    for (int i = 0; i < 16; i++) t->T[i] = (i % 5 == 0) ? 1.0 : 0.0;
    return t;
}

void orc64_destroy(orc64_tracker *t) {
    if (!t) return;
    for (int l = 0; l < t->L; l++) {
        free(t->ref_gray[l]); free(t->cur_gray[l]); free(t->ref6[l]); free(t->cur6[l]);
        free(t->refmask[l]); free(t->curmask[l]); free(t->sel_I[l]); free(t->sel_J[l]);
    }
    free(t->ref_z); free(t->ref_col); free(t->cur_z);
    free(t->vx); free(t->vy); free(t->vz); free(t->vgx); free(t->vgy); free(t->vgm); free(t->vcol);
    free(t->sel_idx); free(t->sel_xyz); free(t->r); free(t->zw); free(t->w);
    free(t->full_res); free(t->icp_wpx); free(t->icp_r2); free(t->icp_w); free(t->partial);
    free(t->rmask); free(t->select);
    free(t);
}

/* ------------------------------------------------------------------ */
/* pyramids and clouds                                                 */
/* ------------------------------------------------------------------ */

/* fastDownSampleHdrKernel, downSample2Cuda.cu:35-42 */
static void downsample2(const R *hi, int wlo, int hlo, R *lo) {
    int w2 = 2 * wlo;
    for (int y = 0; y < hlo; y++)
        for (int x = 0; x < wlo; x++) {
            int h0 = 2 * x + 2 * y * w2;
            lo[x + y * wlo] = (hi[h0] + hi[h0 + 1] + hi[h0 + w2] + hi[h0 + w2 + 1]) / 4.0;
        }
}

/* convertZMapToXYZ6Kernel, rgb2gray.cu:595-624 (and convertZMapToXYZKernel, 570-593) */
static void zmap_to_xyz6(const R *z, int W, int H, const R *c, R *pts, int32_t *mask) {
    R fx = c[KLo], fy = c[KLo + 4], cx = c[KLo + 2], cy = c[KLo + 5];
    for (int i = 0; i < W * H; i++) {
        int xi = i % W, yi = i / W;
        R zz = z[i];
        R *p = &pts[6 * i];
        p[3] = p[4] = p[5] = 0;
        if (zz < -c[MIND] && zz > -c[MAXD]) {
            p[0] = ((R)xi - cx) * zz / fx;
            p[1] = ((R)yi - cy) * zz / fy;
            p[2] = zz;
            mask[i] = 1;
        } else {
            p[0] = p[1] = p[2] = 0;
            mask[i] = 0;
        }
    }
}

/* computeNormalsCudaKernel, d2z.cu:503-537 */
static void compute_normals6(R *pts, int32_t *mask, int W, int H) {
    for (int yi = 0; yi < H; yi++)
        for (int xi = 0; xi < W; xi++) {
            int o = xi + yi * W;
            if (xi < 1 || yi < 1 || xi > W - 2 || yi > H - 2) {
                mask[o] = 0;
                continue;
            }
            const R *x1 = &pts[(o - 1) * 6], *x2 = &pts[(o + 1) * 6];
            const R *y1 = &pts[(o - W) * 6], *y2 = &pts[(o + W) * 6];
            if (x1[2] < 0 && x2[2] < 0 && y1[2] < 0 && y2[2] < 0) {
                R u[3] = {x2[0] - x1[0], x2[1] - x1[1], x2[2] - x1[2]};
                R v[3] = {y2[0] - y1[0], y2[1] - y1[1], y2[2] - y1[2]};
                R nrm[3] = {u[1] * v[2] - u[2] * v[1], -(u[0] * v[2] - u[2] * v[0]), u[0] * v[1] - u[1] * v[0]};
                normalize3(nrm);
                pts[o * 6 + 3] = nrm[0];
                pts[o * 6 + 4] = nrm[1];
                pts[o * 6 + 5] = nrm[2];
            } else {
                mask[o] = 0;
            }
        }
}

/* genPointsCloud6Kernel, d2z.cu:436-469 */
static void gen_cloud6(const R *z, int W, int H, const R *c, R *pts, int32_t *mask) {
    R fx = c[KLo], fy = c[KLo + 4], cx = c[KLo + 2], cy = c[KLo + 5];
    for (int i = 0; i < W * H; i++) {
        int xi = i % W, yi = i / W;
        R *p = &pts[6 * i];
        if (z[i] < 0) {
            p[0] = ((R)xi - cx) * z[i] / fx;
            p[1] = ((R)yi - cy) * z[i] / fy;
            p[2] = z[i];
            p[3] = 0; p[4] = 0; p[5] = 1;
            mask[i] = 1;
        } else {
            p[0] = p[1] = p[2] = p[3] = p[4] = p[5] = 0;
            mask[i] = 0;
        }
    }
}

/* downSampleCloud6Kernel, d2z.cu:557-588 */
static void downsample_cloud6(const R *src, const int32_t *msrc, int wlo, int hlo, R *dst, int32_t *mdst) {
    for (int yi = 0; yi < hlo; yi++)
        for (int xi = 0; xi < wlo; xi++) {
            int o = xi + yi * wlo;
            R *pd = &dst[o * 6];
            int h0 = xi * 2 + yi * 2 * (wlo * 2);
            int offs[4] = {h0, h0 + 1, h0 + wlo * 2, h0 + wlo * 2 + 1};
            for (int i = 0; i < 6; i++) pd[i] = 0;
            R ns = 0;
            for (int k = 0; k < 4; k++)
                if (msrc[offs[k]]) {
                    ns++;
                    for (int i = 0; i < 6; i++) pd[i] += src[offs[k] * 6 + i];
                }
            if (ns > 0) {
                for (int i = 0; i < 6; i++) pd[i] /= ns;
                normalize3(&pd[3]);
                mdst[o] = 1;
            } else {
                mdst[o] = 0;
            }
        }
}

/* ------------------------------------------------------------------ */
/* photometric reference                                               */
/* ------------------------------------------------------------------ */

/* xyz2CloudKernel, d2z.cu:235-331: vertex planes of every IR pixel */
static void xyz2cloud(orc64_tracker *t) {
    int W = t->W, H = t->H;
    const R *c = t->calib;
    const R *img = t->ref_gray[0];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < W * H; i++) {
        R p3[3] = {t->ref6[0][6 * i], t->ref6[0][6 * i + 1], t->ref6[0][6 * i + 2]};
        t->vx[i] = t->vy[i] = t->vgx[i] = t->vgy[i] = t->vgm[i] = t->vcol[i] = 0;
        t->vz[i] = -c[MAXD];
        if (!(p3[2] < 0)) continue;
        R r3[3];
        mul4(&c[TLR], p3, r3);
        R px, py;
        distort(r3[0] / r3[2], r3[1] / r3[2], &c[KCR], &c[KR], &px, &py);
        if (!in_bounds10(px, py, W, H)) continue;
        int xdi = dtoi(px), ydi = dtoi(py);
        R fx = px - xdi, fy = py - ydi;
        R color1 = bilin(xdi, ydi, fx, fy, W, img);
        if (t->has_col && t->ref_col[i] >= 0) color1 = t->ref_col[i];
        R cN = bilin(dtoi(px), dtoi(py - 1.0), fx, fy, W, img);
        R cE = bilin(dtoi(px + 1.0), dtoi(py), fx, fy, W, img);
        R cW = bilin(dtoi(px - 1.0), dtoi(py), fx, fy, W, img);
        R cS = bilin(dtoi(px), dtoi(py + 1.0), fx, fy, W, img);
        R gx = (cE - cW) / 2.0, gy = (cS - cN) / 2.0;
        R gm = fabs(gy) + fabs(gx);
        t->vx[i] = p3[0];
        t->vy[i] = p3[1];
        t->vz[i] = p3[2];
        t->vgx[i] = gx;
        t->vgy[i] = gy;
        t->vgm[i] = gm < 1.0 ? gm : 1.0;
        t->vcol[i] = color1;
    }
}

/* 256-bin gradient histogram (gpu_hist.cu:136) and seekThreshold256Kernel2 +
 * filterIndexKernel4 (filterIndex256.cu:26-46, 110-194): the same integer
 * selection rule as the FP32 oracle's orc_filter_indices, on FP64 keys. */
static void select_pixels(orc64_tracker *t) {
    int n = t->W * t->H, nb = t->cfg.select_bins, P = t->P;
    int32_t hist[1024];
    memset(hist, 0, sizeof(hist));
    unsigned int *q = (unsigned int *)xcalloc((size_t)n * sizeof(unsigned int));
    for (int i = 0; i < n; i++) {
        q[i] = (unsigned int)(t->vgm[i] * (nb - 1) + 0.5);
        if (q[i] < (unsigned)nb) hist[q[i]]++;
    }
    unsigned int thr = 0;
    int sel = 0;
    for (int i = nb - 1; i >= 0; i--) {
        sel += hist[i];
        if (sel > P) { thr = (unsigned)i; break; }
    }
    int tooMuch = sel - P;
    enum { S = 512 };
    int ppt = n / S;
    int cnt[S], mcnt[S], start[S], mstart[S];
    for (int s = 0; s < S; s++) {
        cnt[s] = mcnt[s] = 0;
        for (int i = s * ppt; i < s * ppt + ppt; i++) {
            if (q[i] > thr) cnt[s]++;
            else if (q[i] == thr) mcnt[s]++;
        }
    }
    start[0] = 0;
    for (int i = 1; i < S; i++) start[i] = start[i - 1] + cnt[i - 1];
    mstart[0] = start[S - 1] + cnt[S - 1];
    for (int i = 1; i < S; i++) {
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
    for (int k = 0; k < P; k++) t->sel_idx[k] = 0;
    for (int s = 0; s < S; s++) {
        int a = 0, m = 0;
        for (int i = s * ppt; i < s * ppt + ppt; i++) {
            if (q[i] > thr) {
                int pos = start[s] + a++;
                if (pos < P) t->sel_idx[pos] = i;
            } else if (q[i] == thr) {
                if (m < mcnt[s]) {
                    int pos = mstart[s] + m;
                    if (pos < P) t->sel_idx[pos] = i;
                }
                m++;
            }
        }
    }
    free(q);
}

/* addVertexAttributesWithoutNormalsKernel3/4 (d2z.cu:700-936) and
 * precomputeJacobian4Kernel (warp.cu:502-645) for every selected point */
static void selected_attributes(orc64_tracker *t) {
    int W = t->W, H = t->H, L = t->L, P = t->P;
    const R *c = t->calib, *T = &c[TLR], *kc = &c[KCR], *K = &c[KR];
    R s_in = (R)t->cfg.opt_scale_in;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < P; k++) {
        int pix = t->sel_idx[k];
        R p3[3] = {t->vx[pix], t->vy[pix], t->vz[pix]}, r3[3];
        R col[4] = {t->vcol[pix], 0, 0, 0}, gx[4] = {t->vgx[pix], 0, 0, 0}, gy[4] = {t->vgy[pix], 0, 0, 0};
        mul4(T, p3, r3);
        R px, py;
        distort(r3[0] / r3[2], r3[1] / r3[2], kc, K, &px, &py);
        if (in_bounds10(px, py, W, H)) {
            R lx = px, ly = py;
            for (int l = 1; l < L; l++) {
                lx = 0.5 * lx - 0.25;
                ly = 0.5 * ly - 0.25;
                int wl = W >> l, hl = H >> l;
                int xdi = dtoi(lx), ydi = dtoi(ly);
                R fx = lx - xdi, fy = ly - ydi;
                const R *g = t->ref_gray[l];
                col[l] = bilin_clamped(xdi, ydi, fx, fy, wl, hl, g);
                R cN = bilin_clamped(xdi, ydi - 1, fx, fy, wl, hl, g);
                R cW = bilin_clamped(xdi - 1, ydi, fx, fy, wl, hl, g);
                R cE = bilin_clamped(xdi + 1, ydi, fx, fy, wl, hl, g);
                R cS = bilin_clamped(xdi, ydi + 1, fx, fy, wl, hl, g);
                gx[l] = (cE - cW) / 2.0;
                gy[l] = (cS - cN) / 2.0;
            }
        }
        t->sel_xyz[k] = p3[0];
        t->sel_xyz[P + k] = p3[1];
        t->sel_xyz[2 * P + k] = p3[2];
        for (int l = 0; l < L; l++) t->sel_I[l][k] = col[l];
        /* precomputeJacobian4Kernel */
        R rx = r3[0] * s_in, ry = r3[1] * s_in, rz = r3[2] * s_in;
        R dN[6] = {1.0 / rz, 0, -rx / (rz * rz), 0, 1.0 / rz, -ry / (rz * rz)};
        R x = rx / rz, y = ry / rz;
        R x2 = x * x, y2 = y * y, x4 = x2 * x2, y4 = y2 * y2, r2 = x2 + y2, r4 = r2 * r2;
        R dD0 = 1 + kc[0] * (3 * x2 + y2) + kc[1] * (5 * x4 + 6 * x2 * y2 + y4) + kc[4] * r4 * (7 * x2 + y2);
        R dD1 = kc[0] * 2 * x * y + kc[1] * 4 * x * y * r2 + kc[4] * 6 * x * y * r4;
        R dD2 = dD1;
        R dD3 = 1 + kc[0] * (3 * x2 + y2) + kc[1] * (5 * x4 + 6 * x2 * y2 + y4) + kc[4] * r4 * (7 * y2 + x2);
        R dps[6][3] = {{0, -rz, ry}, {rz, 0, -rx}, {-ry, rx, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int cc = 0; cc < 6; cc++) {
            R dr[3], dd[3], dp[3];
            rot4(T, dps[cc], dr);
            R dpnx = dN[0] * dr[0] + dN[1] * dr[1] + dN[2] * dr[2];
            R dpny = dN[3] * dr[0] + dN[4] * dr[1] + dN[5] * dr[2];
            dd[0] = dD0 * dpnx + dD1 * dpny;
            dd[1] = dD2 * dpnx + dD3 * dpny;
            dd[2] = 0;
            mul3(K, dd, dp);
            for (int l = 0; l < L; l++) {
                R s = (R)(1 << l);
                t->sel_J[l][cc * P + k] = (dp[0] / s) * gx[l] + (dp[1] / s) * gy[l];
            }
        }
    }
}

/* PhotoTracker::prepareReference (phototracker.cpp:338-386) and
 * ShapeTracker::setReferencePoints / prepareReference (shapetracker.cpp:205-288) */
static void prepare_reference(orc64_tracker *t) {
    int W = t->W, H = t->H, L = t->L;
    for (int l = 1; l < L; l++) downsample2(t->ref_gray[l - 1], W >> l, H >> l, t->ref_gray[l]);
    zmap_to_xyz6(t->ref_z, W, H, t->calib, t->ref6[0], t->refmask[0]);
    xyz2cloud(t);
    select_pixels(t);
    selected_attributes(t);
    compute_normals6(t->ref6[0], t->refmask[0], W, H);
    for (int l = 1; l < L; l++)
        downsample_cloud6(t->ref6[l - 1], t->refmask[l - 1], W >> l, H >> l, t->ref6[l], t->refmask[l]);
    t->has_ref = 1;
}

int orc64_set_reference(orc64_tracker *t, const uint8_t *gray, const uint16_t *depth) {
    int n = t->W * t->H;
    for (int i = 0; i < n; i++) {
        t->ref_gray[0][i] = (R)gray[i] / 255.0;
        t->ref_z[i] = depth[i] ? -(R)depth[i] : 0.0;
    }
    t->has_col = 0;
    prepare_reference(t);
    for (int i = 0; i < 16; i++) t->T[i] = (i % 5 == 0) ? 1.0 : 0.0;
    return 0;
}

int orc64_set_current(orc64_tracker *t, const uint8_t *gray, const uint16_t *depth) {
    int W = t->W, H = t->H, L = t->L;
    for (int i = 0; i < W * H; i++) {
        t->cur_gray[0][i] = (R)gray[i] / 255.0;
        t->cur_z[i] = depth[i] ? -(R)depth[i] : 0.0;
    }
    for (int l = 1; l < L; l++) downsample2(t->cur_gray[l - 1], W >> l, H >> l, t->cur_gray[l]);
    gen_cloud6(t->cur_z, W, H, t->calib, t->cur6[0], t->curmask[0]);
    for (int l = 1; l < L; l++)
        downsample_cloud6(t->cur6[l - 1], t->curmask[l - 1], W >> l, H >> l, t->cur6[l], t->curmask[l]);
    t->has_cur = 1;
    return 0;
}

/* ------------------------------------------------------------------ */
/* keyframe depth and colour fusion (orc_fuse_rgbd in FP64)            */
/* ------------------------------------------------------------------ */

static R rgb_sample(const R *c, const R *q, const uint8_t *img8, const R *img, int W, int H) {
    R r3[3];
    mul4(&c[TLR], q, r3);
    R px, py;
    R irz = 1.0 / r3[2];
    distort(r3[0] * irz, r3[1] * irz, &c[KCR], &c[KR], &px, &py);
    int xdi = dtoi(px), ydi = dtoi(py);
    if (!(xdi >= 0 && ydi >= 0 && xdi < W - 1 && ydi < H - 1)) return -1.0;
    R fx = px - xdi, fy = py - ydi;
    if (img) return bilin(xdi, ydi, fx, fy, W, img);
    int o = xdi + ydi * W;
    R v0 = img8[o] / 255.0, v1 = img8[o + 1] / 255.0, v2 = img8[o + W] / 255.0, v3 = img8[o + W + 1] / 255.0;
    return (1 - fx) * (1 - fy) * v0 + fx * (1 - fy) * v1 + (1 - fx) * fy * v2 + fx * fy * v3;
}

int orc64_fuse_keyframe(orc64_tracker *t, int nframes, const uint8_t *const *gray, const uint16_t *const *depth,
                        const double *Tframes, double gate) {
    if (!t->has_ref || nframes < 0 || nframes > 8) return -1;
    int W = t->W, H = t->H;
    const R *c = t->calib, *KL = &c[KLo];
    R fx = KL[0], fy = KL[4], cx = KL[2], cy = KL[5];
    R ifx = 1.0 / fx, ify = 1.0 / fy;  /* the FP32 fusion's reciprocals, in double */
    R Tinv[8][16];
    for (int f = 0; f < nframes; f++) invert_rt4(&Tframes[16 * f], Tinv[f]);
    R *zout = (R *)xcalloc((size_t)W * H * sizeof(R));
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < W * H; idx++) {
        int xi = idx % W, yi = idx / W;
        R z = t->ref_z[idx];
        zout[idx] = z;
        if (gray) t->ref_col[idx] = -1.0;
        if (!(z < -c[MIND] && z > -c[MAXD])) continue;
        R p[3] = {((R)xi - cx) * z * ifx, ((R)yi - cy) * z * ify, z};
        R zsum = z, wsum = 1, csum = 0, cw = 0;
        if (gray) {
            R c0 = rgb_sample(c, p, NULL, t->ref_gray[0], W, H);
            if (c0 >= 0) { csum = c0; cw = 1; }
        }
        for (int f = 0; f < nframes; f++) {
            R q[3];
            mul4(&Tframes[16 * f], p, q);
            R iqz = 1.0 / q[2];
            R qx = q[0] * iqz, qy = q[1] * iqz;
            int xd = dtoi(KL[0] * qx + KL[1] * qy + KL[2] + 0.5), yd = dtoi(KL[3] * qx + KL[4] * qy + KL[5] + 0.5);
            if (xd < 0 || yd < 0 || xd >= W || yd >= H) continue;
            uint16_t dm = depth[f][xd + yd * W];
            R zf = dm ? -(R)dm : 0.0;
            if (!(zf < -c[MIND] && zf > -c[MAXD])) continue;
            R m[3] = {((R)xd - cx) * zf * ifx, ((R)yd - cy) * zf * ify, zf}, mk[3];
            mul4(Tinv[f], m, mk);
            if (fabs(mk[2] - z) < gate) {
                zsum += mk[2];
                wsum += 1;
                if (gray) {
                    R cf = rgb_sample(c, q, gray[f], NULL, W, H);
                    if (cf >= 0) { csum += cf; cw += 1; }
                }
            }
        }
        zout[idx] = zsum / wsum;
        if (gray) t->ref_col[idx] = cw > 0 ? csum / cw : -1.0;
    }
    memcpy(t->ref_z, zout, (size_t)W * H * sizeof(R));
    free(zout);
    if (gray) t->has_col = 1;
    prepare_reference(t);
    return 0;
}

/* ------------------------------------------------------------------ */
/* one Gauss-Newton iteration                                          */
/* ------------------------------------------------------------------ */

/* interpolateResidualKernel2, warp.cu:269-332 */
static void photo_residuals(orc64_tracker *t, int layer) {
    int P = t->P, w = t->W >> layer, h = t->H >> layer;
    const R *c = t->calib, *img = t->cur_gray[layer], *I = t->sel_I[layer];
    R a = 1.0 / (R)(1 << layer), b = 0.5 * (a - 1.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < P; i++) {
        R p3[3] = {t->sel_xyz[i], t->sel_xyz[P + i], t->sel_xyz[2 * P + i]}, ri[3], r3[3];
        mul4(t->T, p3, ri);
        mul4(&c[TLR], ri, r3);
        R p2x, p2y;
        distort(r3[0] / r3[2], r3[1] / r3[2], &c[KCR], &c[KR], &p2x, &p2y);
        R px = a * p2x + b, py = a * p2y + b;
        R res = 1.0, zwt = 0.0;
        int xdi = dtoi(px), ydi = dtoi(py);
        if (xdi >= 0 && ydi >= 0 && xdi < w - 1 && ydi < h - 1) {
            res = I[i] - bilin(xdi, ydi, px - xdi, py - ydi, w, img);
            R rl[3], pl[3];
            mul4(&c[TRL], r3, rl);
            rl[0] /= rl[2];
            rl[1] /= rl[2];
            rl[2] = 1;
            mul3(&c[KLo], rl, pl);
            int x2 = dtoi(pl[0] + 0.5), y2 = dtoi(pl[1] + 0.5);
            if (x2 >= 0 && y2 >= 0 && x2 < t->W && y2 < t->H) {
                R zerr = t->cur_z[x2 + y2 * t->W] - r3[2];
                zerr *= zerr;
                if (zerr < 100.0 * 100.0) zwt = 1.0 - zerr / (100.0 * 100.0);
            }
        }
        t->r[i] = res;
        t->zw[i] = zwt;
    }
}

/* generateWeights64 (histogram64.cu:41-157): MAD histogram, median bin,
 * Tukey weights */
static void photo_weights(orc64_tracker *t) {
    int P = t->P, nb = t->cfg.hist_bins;
    int hist[256];
    memset(hist, 0, sizeof(hist));
    for (int i = 0; i < P; i++) {
        int bin = dtoi((R)(nb - 1) * fabs(t->r[i]));
        if (bin < 0) bin = 0;
        if (bin > nb - 1) bin = nb - 1;
        hist[bin]++;
    }
    int m = 0, acc = 0;
    for (int i = 0; i < nb; i++) {
        acc += hist[i];
        if (acc > P / 2) { m = i; break; }
    }
    R s = (nb == 64) ? 1.4826 * (R)(4 * m + 3) / 255.0 : 1.4826 * ((R)m + 0.75) / ((R)nb - 0.25);
    for (int i = 0; i < P; i++) {
        R u = fabs(t->r[i]) / s, wi = 0;
        if (u <= 4.6851) {
            R ub = u / 4.6851;
            wi = (1.0 - ub * ub) * t->zw[i];
        }
        t->w[i] = wi;
    }
}

/* the 27 terms of point i into s (21 upper-triangle JtJ terms row-major, 6 Jtr) */
static inline void acc27(R *s, const R *j, R r) {
    int q = 0;
    for (int a = 0; a < 6; a++)
        for (int b = a; b < 6; b++, q++) s[q] += j[a] * j[b];
    for (int a = 0; a < 6; a++, q++) s[q] += j[a] * r;
}

static void unpack27(const R *tot, R A[36], R b[6]) {
    int q = 0;
    for (int j = 0; j < 6; j++)
        for (int i = j; i < 6; i++, q++) A[i + j * 6] = A[i * 6 + j] = tot[q];
    for (int c = 0; c < 6; c++) b[c] = tot[q++];
}

/* JTJCuda / JTresidualCuda (warp.cu:1430-1487) of the photometric term: Jw = J w, rw = r w */
static void photo_system(orc64_tracker *t, int layer, R A[36], R b[6]) {
    int P = t->P, nch = P / ORC_CHUNK;
    const R *J = t->sel_J[layer];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nch; k++) {
        R s[27] = {0};
        for (int i = k * ORC_CHUNK; i < (k + 1) * ORC_CHUNK; i++) {
            R wv = t->w[i];
            if (wv == 0.0) continue;
            R jw[6];
            for (int c = 0; c < 6; c++) jw[c] = J[c * P + i] * wv;
            acc27(s, jw, t->r[i] * wv);
        }
        memcpy(&t->partial[27 * k], s, sizeof(s));
    }
    R tot[27] = {0};
    for (int k = 0; k < nch; k++)
        for (int q = 0; q < 27; q++) tot[q] += t->partial[27 * k + q];
    unpack27(tot, A, b);
}

static inline void bilin6(const R *s, R fx, R fy, int pitch, R *p) {
    for (int c = 0; c < 3; c++)
        p[c] = (1 - fx) * (1 - fy) * s[c] + fx * (1 - fy) * s[c + 6] + (1 - fx) * fy * s[c + pitch] +
               fx * fy * s[c + pitch + 6];
}

/* icpResidualKernel2 (rgb2gray.cu:223-260), selectValidIndex (rgb2gray.cu:393-460)
 * and generateStudentTWeights (rgb2gray.cu:470-569, 854-877; each product
 * r^2 w truncated to an integer, as the reference's int accumulator does) */
static void icp_prepare(orc64_tracker *t, int layer) {
    int w = t->W >> layer, h = t->H >> layer, n = w * h;
    const R *K = &t->calib[KLo], *ref = t->ref6[layer], *cur = t->cur6[layer];
    const int32_t *cm = t->curmask[layer];
    R a = 1.0 / (R)(1 << layer), b = 0.5 * (a - 1.0);
#pragma omp parallel for schedule(static)
    for (int o = 0; o < n; o++) {
        t->full_res[o] = 0;
        t->rmask[o] = 0;
        if (!t->refmask[layer][o]) continue;
        R p3[3] = {ref[6 * o], ref[6 * o + 1], ref[6 * o + 2]}, rn[3] = {ref[6 * o + 3], ref[6 * o + 4], ref[6 * o + 5]};
        R q3[3], cn[3];
        mul4(t->T, p3, q3);
        rot4(t->T, rn, cn);
        R p2x = a * (K[0] * (q3[0] / q3[2]) + K[2]) + b, p2y = a * (K[4] * (q3[1] / q3[2]) + K[5]) + b;
        if (!(p2x >= 0 && p2x < (w - 1) && p2y >= 0 && p2y < (h - 1))) continue;
        int xdi = dtoi(p2x), ydi = dtoi(p2y), o2 = xdi + ydi * w;
        if (!(cm[o2] && cm[o2 + 1] && cm[o2 + w] && cm[o2 + w + 1])) continue;
        R cp[3];
        bilin6(&cur[o2 * 6], p2x - xdi, p2y - ydi, w * 6, cp);
        t->full_res[o] = (cp[0] - q3[0]) * cn[0] + (cp[1] - q3[1]) * cn[1] + (cp[2] - q3[2]) * cn[2];
        t->rmask[o] = 1;
    }
    int ns = 0;
    for (int o = 0; o < n; o++)
        if (t->rmask[o]) t->select[ns++] = o;
    t->nsel[layer] = ns;
    for (int o = 0; o < n; o++) t->icp_wpx[o] = 0;
    if (ns <= 0) return;
    for (int k = 0; k < ns; k++) {
        R rv = t->full_res[t->select[k]];
        t->icp_r2[k] = rv * rv;
        t->icp_w[k] = 6 / (5 + t->icp_r2[k] / 100.0);
    }
    for (int it = 0; it < 3; it++) {
        long long S = 0;
        for (int k = 0; k < ns; k++) {
            R prod = t->icp_r2[k] * t->icp_w[k];
            S += (prod >= 0 && prod < 9.0e18) ? (long long)prod : (prod >= 9.0e18 ? 9000000000000000000LL : 0);
        }
        R var = (ns <= 1024) ? (R)S : ((R)S < (R)ns ? (R)ns : (R)S);
        R sigma2 = var / (R)ns;
        for (int k = 0; k < ns; k++) t->icp_w[k] = 6 / (5 + t->icp_r2[k] / sigma2);
    }
    for (int k = 0; k < ns; k++) t->icp_wpx[t->select[k]] = t->icp_w[k] < 1.0 ? t->icp_w[k] : 1.0;
}

/* icpResidualIndexKernel2 (rgb2gray.cu:323-390) and the 27-term sums */
static void icp_system(orc64_tracker *t, int layer, R A[36], R bb[6]) {
    int w = t->W >> layer, h = t->H >> layer, n = w * h, nch = (n + ORC_CHUNK - 1) / ORC_CHUNK;
    const R *K = &t->calib[KLo], *ref = t->ref6[layer], *cur = t->cur6[layer];
    const int32_t *cm = t->curmask[layer];
    R a = 1.0 / (R)(1 << layer), b = 0.5 * (a - 1.0), s_in = (R)t->cfg.opt_scale_in;
    const R *T = t->T;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nch; k++) {
        R s[27] = {0};
        int end = (k + 1) * ORC_CHUNK < n ? (k + 1) * ORC_CHUNK : n;
        for (int o = k * ORC_CHUNK; o < end; o++) {
            R weight = t->icp_wpx[o];
            if (!(weight > 0)) continue;
            R p3[3] = {ref[6 * o], ref[6 * o + 1], ref[6 * o + 2]};
            R rn[3] = {ref[6 * o + 3], ref[6 * o + 4], ref[6 * o + 5]};
            R q3[3], cn[3];
            mul4(T, p3, q3);
            rot4(T, rn, cn);
            R p2x = a * (K[0] * (q3[0] / q3[2]) + K[2]) + b, p2y = a * (K[4] * (q3[1] / q3[2]) + K[5]) + b;
            if (!(p2x >= 0 && p2x < (w - 1) && p2y >= 0 && p2y < (h - 1))) continue;
            int xdi = dtoi(p2x), ydi = dtoi(p2y), o2 = xdi + ydi * w;
            R cp[3];
            bilin6(&cur[o2 * 6], p2x - xdi, p2y - ydi, w * 6, cp);
            if (!(cm[o2] && fabs(cp[2] - q3[2]) < 300.0)) continue;
            R rv[3] = {cp[0] - q3[0], cp[1] - q3[1], cp[2] - q3[2]};
            R res = s_in * weight * (rv[0] * cn[0] + rv[1] * cn[1] + rv[2] * cn[2]);
            R dPs[3][3] = {{0, -p3[2], p3[1]}, {p3[2], 0, -p3[0]}, {-p3[1], p3[0], 0}};
            R dNs[3][3] = {{0, -rn[2], rn[1]}, {rn[2], 0, -rn[0]}, {-rn[1], rn[0], 0}};
            R j[6];
            for (int c = 0; c < 3; c++) {
                R dB[3], dN[3];
                rot4(T, dPs[c], dB);
                rot4(T, dNs[c], dN);
                j[c] = -s_in * weight *
                       (-cn[0] * dB[0] - cn[1] * dB[1] - cn[2] * dB[2] + rv[0] * dN[0] + rv[1] * dN[1] + rv[2] * dN[2]);
            }
            for (int c = 0; c < 3; c++) j[3 + c] = -weight * (-cn[0] * T[c] - cn[1] * T[4 + c] - cn[2] * T[8 + c]);
            acc27(s, j, res);
        }
        memcpy(&t->partial[27 * k], s, sizeof(s));
    }
    R tot[27] = {0};
    for (int k = 0; k < nch; k++)
        for (int q = 0; q < 27; q++) tot[q] += t->partial[27 * k + q];
    unpack27(tot, A, bb);
}

/* 6x6 Cholesky (LDL^T) and the reference's CG (warp.cu:926-975) */
static int solve_cholesky(const R A[36], const R b[6], R x[6]) {
    R L[36] = {0}, D[6];
    for (int j = 0; j < 6; j++) {
        R s = A[j * 6 + j];
        for (int k = 0; k < j; k++) s -= L[j * 6 + k] * L[j * 6 + k] * D[k];
        if (!(s > 0)) {
            for (int i = 0; i < 6; i++) x[i] = 0;
            return -1;
        }
        D[j] = s;
        for (int i = j + 1; i < 6; i++) {
            R v = A[i * 6 + j];
            for (int k = 0; k < j; k++) v -= L[i * 6 + k] * L[j * 6 + k] * D[k];
            L[i * 6 + j] = v / s;
        }
    }
    R z[6];
    for (int i = 0; i < 6; i++) {
        z[i] = b[i];
        for (int k = 0; k < i; k++) z[i] -= L[i * 6 + k] * z[k];
    }
    for (int i = 0; i < 6; i++) z[i] /= D[i];
    for (int i = 5; i >= 0; i--) {
        for (int k = i + 1; k < 6; k++) z[i] -= L[k * 6 + i] * z[k];
        x[i] = z[i];
    }
    return 0;
}

/* normalizeMat4RealSafe (expmCuda.cu:1955-1980) in FP64 */
static void normalize_mat4(R *T) {
    R u[3] = {T[0], T[4], T[8]}, v[3] = {T[1], T[5], T[9]}, w[3] = {T[2], T[6], T[10]};
    R lenU = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    R lenW = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    if (lenW > 1e-8) { w[0] /= lenW; w[1] /= lenW; w[2] /= lenW; }
    else { w[0] = 0; w[1] = 0; w[2] = 1; }
    u[0] = v[1] * w[2] - v[2] * w[1];
    u[1] = -(v[0] * w[2] - v[2] * w[0]);
    u[2] = v[0] * w[1] - v[1] * w[0];
    if (lenU > 1e-8) { u[0] /= lenU; u[1] /= lenU; u[2] /= lenU; }
    else { u[0] = 1; u[1] = 0; u[2] = 0; }
    v[0] = w[1] * u[2] - w[2] * u[1];
    v[1] = -(w[0] * u[2] - w[2] * u[0]);
    v[2] = w[0] * u[1] - w[1] * u[0];
    T[0] = u[0]; T[4] = u[1]; T[8] = u[2];
    T[1] = v[0]; T[5] = v[1]; T[9] = v[2];
    T[2] = w[0]; T[6] = w[1]; T[10] = w[2];
}

static void mat4(const R *M1, const R *M2, R *Rr) {
    R t[16];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++)
            t[r * 4 + c] = M1[r * 4 + 0] * M2[0 * 4 + c] + M1[r * 4 + 1] * M2[1 * 4 + c] +
                           M1[r * 4 + 2] * M2[2 * 4 + c] + M1[r * 4 + 3] * M2[3 * 4 + c];
    memcpy(Rr, t, sizeof(t));
}

/* generateA + expmKernel (warp.cu:910-915, expmCuda.cu:1989-2048): T <- T exp(A(x)),
 * translation scaled by scaleOut, the pose kept in FP64 */
static void expm_update(const R x[6], R *T, R scaleOut) {
    R A[16] = {0, -x[2], x[1], x[3], x[2], 0, -x[0], x[4], -x[1], x[0], 0, x[5], 0, 0, 0, 0};
    R Tinc[16];
    R maxEntry = 0;
    for (int i = 0; i < 16; i++)
        if (fabs(A[i]) > maxEntry) maxEntry = fabs(A[i]);
    if (maxEntry != 0) {
        orc_expm_twist(A, Tinc); /* FP64 Pade(6) with scaling and squaring (oracle.c) */
        normalize_mat4(Tinc);
        Tinc[3] *= scaleOut;
        Tinc[7] *= scaleOut;
        Tinc[11] *= scaleOut;
    } else {
        for (int i = 0; i < 16; i++) Tinc[i] = (i % 5 == 0) ? 1.0 : 0.0;
    }
    mat4(T, Tinc, T);
    normalize_mat4(T);
}

/* gpuEstimateIncrement (phototracker.cpp:666-689) with updateLinearSystem
 * (505-511), ShapeTracker::updateLinearSystem (shapetracker.cpp:357-382),
 * linearFuse (392-394) and estimateIncrement (646-664).  Returns the number
 * of iterations run. */
int orc64_track(orc64_tracker *t, double *Tio) {
    if (!t->has_ref || !t->has_cur) return -1;
    if (Tio) memcpy(t->T, Tio, sizeof(t->T));
    int L = t->L, P = t->P, mode = t->cfg.mode, its = 0;
    for (int layer = L - 1; layer >= 0; layer--) {
        int nit = t->cfg.iters[L - 1 - layer];
        for (int j = 0; j < nit; j++, its++) {
            R A_ph[36] = {0}, b_ph[6] = {0}, A_icp[36] = {0}, b_icp[6] = {0};
            int ok = 1;
            if (mode != ORC_GEOMETRIC) {
                photo_residuals(t, layer);
                photo_weights(t);
                photo_system(t, layer, A_ph, b_ph);
            }
            if (mode != ORC_PHOTOMETRIC) {
                if (j == 0) icp_prepare(t, layer);
                if (t->nsel[layer] <= 0) ok = 0;
                else icp_system(t, layer, A_icp, b_icp);
            }
            R A[36], b[6];
            if (mode == ORC_PHOTOMETRIC) {
                memcpy(A, A_ph, sizeof(A));
                memcpy(b, b_ph, sizeof(b));
            } else if (mode == ORC_GEOMETRIC) {
                memcpy(A, A_icp, sizeof(A));
                memcpy(b, b_icp, sizeof(b));
            } else {
                R lam = (R)t->cfg.lambda;
                R c1 = (1.0 - lam) / (R)P, c2 = ok ? lam / (R)t->nsel[layer] : 0.0;
                for (int i = 0; i < 36; i++) A[i] = ok ? c1 * A_ph[i] + c2 * A_icp[i] : A_ph[i];
                for (int i = 0; i < 6; i++) b[i] = ok ? c1 * b_ph[i] + c2 * b_icp[i] : b_ph[i];
            }
            if (!ok) continue;
            R x[6];
            if (t->cfg.solver == ORC_SOLVER_CG) orc_solve_cg(A, b, 1e-8, 6, x);
            else solve_cholesky(A, b, x);
            expm_update(x, t->T, (R)t->cfg.opt_scale_out);
        }
    }
    if (Tio) memcpy(Tio, t->T, sizeof(t->T));
    return its;
}

void orc64_get_pose(const orc64_tracker *t, double T[16]) { memcpy(T, t->T, sizeof(t->T)); }
void orc64_set_pose(orc64_tracker *t, const double T[16]) { memcpy(t->T, T, sizeof(t->T)); }

int orc64_get_array(orc64_tracker *t, const char *name, int level, void *dst, int64_t nbytes) {
    int W = t->W >> level, H = t->H >> level, P = t->P;
    const void *src = NULL;
    int64_t n = 0;
    if (!strcmp(name, "sel_idx")) { src = t->sel_idx; n = (int64_t)P * 4; }
    else if (!strcmp(name, "sel_I")) { src = t->sel_I[level]; n = (int64_t)P * 8; }
    else if (!strcmp(name, "ref_z")) { src = t->ref_z; n = (int64_t)t->W * t->H * 8; }
    else if (!strcmp(name, "ref_col")) { src = t->ref_col; n = (int64_t)t->W * t->H * 8; }
    else if (!strcmp(name, "icp_w_px")) { src = t->icp_wpx; n = (int64_t)W * H * 8; }
    else return -1;
    if (n > nbytes) return -2;
    memcpy(dst, src, (size_t)n);
    return (int)n;
}
