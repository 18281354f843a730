/*
 * oracle_kinect.c -- CPU oracle of the Kinect pre-processing: disparity ->
 * depth, RGB -> gray, and the undistortion of a gray image.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Each function restates one
 * routine of tracker/multicore/multicore.cpp (OMPFunctions) and cites its
 * lines; FP32 expressions in the reference's order, built with
 * -ffp-contract=off.
 *
 * Conversions: the reference forms a source pixel as `unsigned int sxi = xi +
 * xOff` with a float offset (-4, -3 for the Kinect's IR/disparity shift).  For
 * a negative sum that conversion is undefined; on the x86 machines the
 * reference ran on it wraps to a huge value, so the pixel fails the bounds
 * test and gets no depth.  These functions take that behaviour: a source
 * coordinate is the integer truncation of the float sum and must lie in
 * [0, size - 1).
 */
#include "oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* truncation of a float pixel coordinate; negative sums are out of range */
static inline int src_coord(int i, float off, int *ok) {
    float s = (float)i + off;
    if (!(s >= 0.0f && s < 2147483520.0f)) {
        *ok = 0;
        return 0;
    }
    return (int)s;
}

/* OMPFunctions::d2Z (multicore.cpp:240-275): z = |1 / (c0 + c1 d)| in mm from
 * 11-bit disparity (2047 = none), 0 outside [min_dist, max_dist]; the source
 * pixel is shifted by (x_off, y_off) and must lie inside [0, W-1) x [0, H-1).
 * Rows are processed in 4 blocks of H / 4 (rows past 4 * (H / 4) stay 0). */
void orc_kinect_d2z(const uint16_t *disp, int W, int H, float c0, float c1, float min_dist, float max_dist,
                    float x_off, float y_off, float *z) {
    memset(z, 0, sizeof(float) * (size_t)W * H);
    int rows = 4 * (H / 4);
    for (int yi = 0; yi < rows; yi++)
        for (int xi = 0; xi < W; xi++) {
            int okx = 1, oky = 1;
            int sx = src_coord(xi, x_off, &okx), sy = src_coord(yi, y_off, &oky);
            float out = 0.0f;
            if (okx && oky && sx < W - 1 && sy < H - 1) {
                float d = (float)disp[sx + sy * W];
                if (d < 2047) {
                    float zz = fabsf(1.0f / (c0 + c1 * d));
                    if (zz > max_dist || zz < min_dist) zz = 0.0f;
                    out = zz;
                }
            }
            z[xi + yi * W] = out;
        }
}

/* OMPFunctions::d2ZLow (multicore.cpp:189-238): the half-resolution map
 * (Wl x Hl from a 2Wl x 2Hl disparity), the smallest disparity of each 2x2
 * block, all four below 2047 */
void orc_kinect_d2z_low(const uint16_t *disp, int Wl, int Hl, float c0, float c1, float min_dist, float max_dist,
                        float x_off, float y_off, float *z) {
    memset(z, 0, sizeof(float) * (size_t)Wl * Hl);
    int W2 = 2 * Wl, H2 = 2 * Hl;
    int rows = 4 * (Hl / 4);
    for (int yi = 0; yi < rows; yi++)
        for (int xi = 0; xi < Wl; xi++) {
            int okx = 1, oky = 1;
            int sx = src_coord(2 * xi, x_off, &okx), sy = src_coord(2 * yi, y_off, &oky);
            float out = 0.0f;
            if (okx && oky && sx < W2 - 1 && sy < H2 - 1) {
                float d1 = (float)disp[sx + sy * W2];
                float d2 = (float)disp[sx + 1 + sy * W2];
                float d3 = (float)disp[sx + 1 + (sy + 1) * W2];
                float d4 = (float)disp[sx + (sy + 1) * W2];
                if (d1 < 2047 && d2 < 2047 && d3 < 2047 && d4 < 2047) {
                    float d = d1;
                    if (d2 < d) d = d2;
                    if (d3 < d) d = d3;
                    if (d4 < d) d = d4;
                    float zz = fabsf(1.0f / (c0 + c1 * d));
                    if (zz > max_dist || zz < min_dist) zz = 0.0f;
                    out = zz;
                }
            }
            z[xi + yi * Wl] = out;
        }
}

/* OMPFunctions::convert2Gray (multicore.cpp:634-652): 3 bytes per pixel
 * (channel order as stored), gray = (c0*19588 + c1*38469 + c2*7471) >> 16;
 * rows are processed in 4 blocks of H / 4 (pixels of later rows are left as
 * they are) */
void orc_kinect_rgb2gray(const uint8_t *rgb, int W, int H, uint8_t *gray) {
    int m = 4 * W * (H / 4);
    for (int i = 0; i < m; i++)
        gray[i] = (uint8_t)(((unsigned)rgb[3 * i] * 19588u + (unsigned)rgb[3 * i + 1] * 38469u +
                             (unsigned)rgb[3 * i + 2] * 7471u) >> 16);
}

/* OMPFunctions::undistort / undistortLookup (multicore.cpp:654-770): each
 * output pixel samples the distorted image at K (radial(iK p)) with 8-bit
 * fixed-point bilinear weights; the first call stores the sampling offsets
 * p - (x, y) and every later call samples at offset + (x, y), which is what
 * this computes (points outside [0, W-2) x [0, H-2) get offset -(x, y), i.e.
 * pixel (0, 0), whose 2x2 block the routine sets to 0).  Rows are processed in
 * 6 blocks of H / 6.  int(p) truncates toward zero, so a sampling point in
 * (-1, 0) passes the bounds test; its weight (unsigned)(frac * 256) then
 * converts a negative float, which on x86 wraps modulo 2^32 -- taken here as
 * (uint32_t)(int64_t). */
static inline unsigned wrap_u32(float v) { return (unsigned)(int64_t)v; }

void orc_kinect_undistort(const uint8_t *src_in, int W, int H, const float *K, const float *iK, const float *kc,
                          uint8_t *dst) {
    size_t n = (size_t)W * H;
    uint8_t *src = (uint8_t *)malloc(n);
    memcpy(src, src_in, n);
    src[0] = 0;
    src[1] = 0;
    src[W] = 0;
    src[W + 1] = 0;
    int rows = 6 * (H / 6);
    for (int yi = 0; yi < rows; yi++)
        for (int xi = 0; xi < W; xi++) {
            float pu0 = (float)xi, pu1 = (float)yi;
            float pd0 = iK[0] * pu0 + iK[1] * pu1 + iK[2];
            float pd1 = iK[3] * pu0 + iK[4] * pu1 + iK[5];
            float r2 = (pd0 * pd0) + (pd1 * pd1), r4 = r2 * r2, r6 = r4 * r2;
            float rd = 1 + kc[0] * r2 + kc[1] * r4 + kc[4] * r6;
            pd0 *= rd;
            pd1 *= rd;
            float p0 = K[0] * pd0 + K[1] * pd1 + K[2];
            float p1 = K[3] * pd0 + K[4] * pd1 + K[5];
            /* int(p) in [0, size - 2) */
            float dx, dy;
            if (p0 > -1.0f && p1 > -1.0f && p0 < (float)(W - 2) && p1 < (float)(H - 2)) {
                dx = p0 - (float)xi;
                dy = p1 - (float)yi;
            } else {
                dx = 0.0f - (float)xi;
                dy = 0.0f - (float)yi;
            }
            /* undistortLookup */
            float q0 = dx + (float)xi, q1 = dy + (float)yi;
            int xq = (int)q0, yq = (int)q1;
            unsigned fx = wrap_u32((q0 - (float)xq) * 256.0f);
            unsigned fy = wrap_u32((q1 - (float)yq) * 256.0f);
            const uint8_t *p = &src[xq + (size_t)yq * W];
            unsigned i1 = p[0], i2 = p[1], i4 = p[W], i3 = p[W + 1];
            unsigned c = fx * fy;
            unsigned a = 65536 - ((fy + fx) << 8) + c;
            unsigned b = (fx << 8) - c;
            unsigned d = 65536 - a - b - c;
            dst[xi + (size_t)yi * W] = (uint8_t)((a * i1 + b * i2 + c * i3 + d * i4) >> 16);
        }
    free(src);
}

/* ---- the GPU capture path: the reference's CUDA kernels of
 * capture/VideoPreProcessorGPU.cpp:120-175 and reconstruct/TrackFrame.cpp:
 * 430-465.  These run on the GPU, where a float -> unsigned conversion
 * saturates (a negative value gives 0, NaN gives 0); the restatement does the
 * same, so a negative shifted coordinate reads row or column 0. ---- */

static inline unsigned gpu_f2u(float v) {
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xffffffffu;
    return (unsigned)v;
}

/* undistortDisparityKernel (d2z.cu:68-85): the disparity as float, 65535 where
 * it is 2047 or more (the polynomial correction there is commented out) */
void orc_kinect_disparity_to_float(const uint16_t *disp, int n, float *out) {
    for (int i = 0; i < n; i++) {
        float d = (float)disp[i];
        out[i] = d < 2047 ? d : (float)0xffff;
    }
}

/* d2ZLowKernel / d2ZLowHdrKernel (d2z.cu:88-170): the W/2 x H/2 depth, from
 * 16-bit (disp_u16) or float (disp_f32) disparity: at (2x + x_off, 2y + y_off)
 * inside [0, W-1) x [0, H-1) and all four 2x2 disparities below 2047, z =
 * |1 / (c0 + c1 min d)| (0 outside [min_dist, max_dist]) and the output is
 * (z - min_dist) / (max_dist - min_dist); otherwise 0. */
void orc_kinect_depth_normalized(const uint16_t *disp_u16, const float *disp_f32, int W, int H, float c0, float c1,
                                 float min_dist, float max_dist, float x_off, float y_off, float *z_low) {
    int Wl = W / 2, Hl = H / 2;
    for (int yi = 0; yi < Hl; yi++)
        for (int xi = 0; xi < Wl; xi++) {
            unsigned sx = gpu_f2u((float)(2 * xi) + x_off), sy = gpu_f2u((float)(2 * yi) + y_off);
            float out = 0.0f;
            if (sx < (unsigned)(W - 1) && sy < (unsigned)(H - 1)) {
                size_t o = sx + (size_t)sy * W;
                float d1, d2, d3, d4;
                if (disp_f32) {
                    d1 = disp_f32[o];
                    d2 = disp_f32[o + 1];
                    d3 = disp_f32[o + 1 + W];
                    d4 = disp_f32[o + W];
                } else {
                    d1 = (float)disp_u16[o];
                    d2 = (float)disp_u16[o + 1];
                    d3 = (float)disp_u16[o + 1 + W];
                    d4 = (float)disp_u16[o + W];
                }
                if (d1 < 2047 && d2 < 2047 && d3 < 2047 && d4 < 2047) {
                    float d = d1;
                    if (d2 < d) d = d2;
                    if (d3 < d) d = d3;
                    if (d4 < d) d = d4;
                    float z = fabsf(1.0f / (c0 + c1 * d));
                    if (z > max_dist || z < min_dist) z = 0.0f;
                    out = (z - min_dist) / (max_dist - min_dist);
                }
            }
            z_low[xi + (size_t)yi * Wl] = out;
        }
}

/* convertHdrRGBKernel (rgb2gray.cu:634-647): every channel / 255 */
void orc_kinect_rgb_to_hdr(const uint8_t *rgb, int n, float *rgb_hdr) {
    for (int i = 0; i < 3 * n; i++) rgb_hdr[i] = ((float)rgb[i]) / 255.0f;
}

/* rgb2GrayHdrKernel (rgb2gray.cu:41-50): the integer gray of convert2Gray as float */
void orc_kinect_rgb_to_gray_hdr(const uint8_t *rgb, int n, float *gray) {
    for (int i = 0; i < n; i++)
        gray[i] = (float)((rgb[3 * i] * 19588 + rgb[3 * i + 1] * 38469 + rgb[3 * i + 2] * 7471) >> 16);
}

/* rgbF2GrayHdrKernel (rgb2gray.cu:53-62) */
void orc_kinect_rgb_hdr_to_gray(const float *rgb_hdr, int n, float *gray) {
    for (int i = 0; i < n; i++)
        gray[i] = 0.3f * rgb_hdr[3 * i] + 0.59f * rgb_hdr[3 * i + 1] + 0.11f * rgb_hdr[3 * i + 2];
}

/* undistortHdrRGBKernel (undistort.cu:110-170): each channel of the RGB image
 * sampled at K (radial(iK (x, y))) with float bilinear weights of the /255
 * values; 0 where int(p) leaves [0, W-2) x [0, H-2) */
void orc_kinect_undistort_rgb_hdr(const uint8_t *rgb, int W, int H, const float *K, const float *iK, const float *kc,
                                  float *rgb_hdr) {
    int pitch = 3 * W;
    for (int yi = 0; yi < H; yi++)
        for (int xi = 0; xi < W; xi++) {
            size_t oR = 3 * (size_t)xi + (size_t)yi * pitch;
            float pu0 = (float)xi, pu1 = (float)yi;
            float pd0 = iK[0] * pu0 + iK[1] * pu1 + iK[2];
            float pd1 = iK[3] * pu0 + iK[4] * pu1 + iK[5];
            float r2 = (pd0 * pd0) + (pd1 * pd1), r4 = r2 * r2, r6 = r4 * r2;
            float rd = 1 + kc[0] * r2 + kc[1] * r4 + kc[4] * r6;
            pd0 *= rd;
            pd1 *= rd;
            float p0 = K[0] * pd0 + K[1] * pd1 + K[2];
            float p1 = K[3] * pd0 + K[4] * pd1 + K[5];
            /* int(p) of a value far out of range: the GPU saturates, and either
             * way the bounds test below fails */
            int xdi = (p0 > -2147483648.0f && p0 < 2147483648.0f) ? (int)p0 : (p0 > 0 ? 2147483647 : -2147483647 - 1);
            int ydi = (p1 > -2147483648.0f && p1 < 2147483648.0f) ? (int)p1 : (p1 > 0 ? 2147483647 : -2147483647 - 1);
            if (p0 != p0) xdi = 0;
            if (p1 != p1) ydi = 0;
            if (xdi >= 0 && ydi >= 0 && (unsigned)xdi < (unsigned)(W - 2) && (unsigned)ydi < (unsigned)(H - 2)) {
                size_t o2 = 3 * (size_t)xdi + (size_t)ydi * pitch;
                float fx = p0 - xdi, fy = p1 - ydi;
                float a = (1 - fx) * (1 - fy), b = fx * (1 - fy), c = (1 - fx) * fy, d = fx * fy;
                for (int ch = 0; ch < 3; ch++) {
                    size_t q = o2 + ch;
                    float v0 = (float)rgb[q] / 255.0f, v1 = (float)rgb[q + 3] / 255.0f;
                    float v2 = (float)rgb[q + pitch] / 255.0f, v3 = (float)rgb[q + pitch + 3] / 255.0f;
                    rgb_hdr[oR + ch] = a * v0 + b * v1 + c * v2 + d * v3;
                }
            } else {
                rgb_hdr[oR] = rgb_hdr[oR + 1] = rgb_hdr[oR + 2] = 0.0f;
            }
        }
}
