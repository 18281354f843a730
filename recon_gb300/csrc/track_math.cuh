// track_math.cuh -- per-point device math of the tracking hot path.
//
// Every FP32 expression is written in the reference kernel's source order
// (the cited file:line) and the translation unit is compiled with -fmad=false,
// so each value is bit-identical to the reference semantics evaluated without
// fused multiply-adds.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#define RC_KR 0
#define RC_KCR 18
#define RC_TLR 26
#define RC_KL 43
#define RC_MIND 62
#define RC_MAXD 63
#define RC_TRL 64

namespace rt {

// float -> int truncation; NaN / out of range -> INT_MIN (always "out of view")
__device__ __forceinline__ int ftoi(float x) {
    if (!(x > -2147483520.0f && x < 2147483520.0f)) return INT32_MIN;
    return (int)x;
}

// matrixMultVec4, kernels/kernelUtils.h:224-229
__device__ __forceinline__ void mul4(const float *M, float x, float y, float z, float &rx, float &ry, float &rz) {
    rx = M[0] * x + M[1] * y + M[2] * z + M[3];
    ry = M[4] * x + M[5] * y + M[6] * z + M[7];
    rz = M[8] * x + M[9] * y + M[10] * z + M[11];
}

// matrixRot4 / rotate3Cuda, kernelUtils.h:69-73, 231-236
__device__ __forceinline__ void rot4(const float *M, float x, float y, float z, float &rx, float &ry, float &rz) {
    rx = M[0] * x + M[1] * y + M[2] * z;
    ry = M[4] * x + M[5] * y + M[6] * z;
    rz = M[8] * x + M[9] * y + M[10] * z;
}

// matrixMultVec3, kernelUtils.h:217-222
__device__ __forceinline__ void mul3(const float *M, float x, float y, float z, float &rx, float &ry, float &rz) {
    rx = M[0] * x + M[1] * y + M[2] * z;
    ry = M[3] * x + M[4] * y + M[5] * z;
    rz = M[6] * x + M[7] * y + M[8] * z;
}

// distortPoint, kernelUtils.h:394-408
__device__ __forceinline__ void distort(float pux, float puy, const float *kc, const float *K, float &pdx,
                                        float &pdy) {
    float dx = pux * pux;
    float dy = puy * puy;
    float r2 = dx + dy;
    float r4 = r2 * r2;
    float r6 = r4 * r2;
    float radialDist = 1 + kc[0] * r2 + kc[1] * r4 + kc[4] * r6;
    pdx = K[0] * pux * radialDist + K[2];
    pdy = K[4] * puy * radialDist + K[5];
}

// a stored value widened to FP32 (exact for FP16 and BF16)
__device__ __forceinline__ float ldf(const float *p) { return __ldg(p); }
__device__ __forceinline__ float ldf(const __half *p) { return __half2float(__ldg(p)); }
__device__ __forceinline__ float ldf(const __nv_bfloat16 *p) { return __bfloat162float(__ldg(p)); }
// a uint8 gray value in [0, 1] (the input conversion's (float)g / 255)
__device__ __forceinline__ float ldf(const uint8_t *p) { return (float)__ldg(p) / 255.0f; }

// bilinearInterpolation(int,int,float,float,...), kernelUtils.h:298-303
template <typename TImg>
__device__ __forceinline__ float bilin(int xdi, int ydi, float fx, float fy, int width, const TImg *src) {
    int o = xdi + ydi * width;
    float v0 = ldf(src + o);
    float v1 = ldf(src + o + 1);
    float v2 = ldf(src + o + width);
    float v3 = ldf(src + o + width + 1);
    return (1 - fx) * (1 - fy) * v0 + fx * (1 - fy) * v1 + (1 - fx) * fy * v2 + fx * fy * v3;
}

// the same with taps clamped into the image (coarsest level of d2z.cu:805-936)
__device__ __forceinline__ float bilin_clamped(int xdi, int ydi, float fx, float fy, int w, int h, const float *src) {
    int x0 = xdi < 0 ? 0 : (xdi > w - 1 ? w - 1 : xdi);
    int x1 = xdi + 1 < 0 ? 0 : (xdi + 1 > w - 1 ? w - 1 : xdi + 1);
    int y0 = ydi < 0 ? 0 : (ydi > h - 1 ? h - 1 : ydi);
    int y1 = ydi + 1 < 0 ? 0 : (ydi + 1 > h - 1 ? h - 1 : ydi + 1);
    float v0 = __ldg(src + x0 + y0 * w);
    float v1 = __ldg(src + x1 + y0 * w);
    float v2 = __ldg(src + x0 + y1 * w);
    float v3 = __ldg(src + x1 + y1 * w);
    return (1 - fx) * (1 - fy) * v0 + fx * (1 - fy) * v1 + (1 - fx) * fy * v2 + fx * fy * v3;
}

// inBounds, kernelUtils.h:341-344
__device__ __forceinline__ bool in_bounds10(float px, float py, int w, int h) {
    return (px >= 10 && px < (w - 10) && py >= 10 && py < (h - 10));
}

// normalize3Cuda / normalizeCuda, kernelUtils.h:19-28, 41-50
__device__ __forceinline__ void normalize3(float &x, float &y, float &z) {
    float len = 0.0f;
    len += x * x;
    len += y * y;
    len += z * z;
    len = 1.0f / sqrtf(len);
    x *= len;
    y *= len;
    z *= len;
}

// MAD scale from the histogram median bin, histogram64.cu:81
__device__ __forceinline__ float mad_scale(int m, int nbins) {
    if (nbins == 64) return 1.4826f * (float)(4 * m + 3) / 255.0f;
    return 1.4826f * ((float)m + 0.75f) / ((float)nbins - 0.25f);
}

// generateWeights64Kernel, histogram64.cu:79-94
__device__ __forceinline__ float tukey_weight(float r, float zw, float s) {
    float bb = 4.6851f;
    float u = fabsf(r) / s;
    float w = 0.0f;
    if (u <= bb) {
        float ub = u / bb;
        float ub2 = ub * ub;
        w = (1.0f - ub2) * zw;
    }
    return w;
}

__device__ __forceinline__ int mad_bin(float r, int nbins) {
    int bin = ftoi((float)(nbins - 1) * fabsf(r));
    if (bin < 0) bin = 0;
    if (bin > nbins - 1) bin = nbins - 1;
    return bin;
}

// interpolateResidualKernel2, warp.cu:269-332: photometric residual and depth
// consistency weight of one keyframe point at pyramid layer `layer` (the image
// stored in FP32, or in FP16 for the mixed-precision mode).
template <typename TImg>
__device__ __forceinline__ void photo_residual(const float *calib, const float *T, float a, float b, float px3,
                                               float py3, float pz3, float Iref, const TImg *img, int width,
                                               int height, const float *zcur, int zwidth, int zheight, float &res,
                                               float &zweight) {
    const float *KR = calib + RC_KR;
    const float *kc = calib + RC_KCR;
    const float *TLR = calib + RC_TLR;
    float rix, riy, riz, rx, ry, rz;
    mul4(T, px3, py3, pz3, rix, riy, riz);
    mul4(TLR, rix, riy, riz, rx, ry, rz);
    float pux = rx / rz;
    float puy = ry / rz;
    float p2x, p2y;
    distort(pux, puy, kc, KR, p2x, p2y);
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
        iResidual = Iref - color;
        const float *KL = calib + RC_KL;
        const float *TRL = calib + RC_TRL;
        float lx, ly, lz;
        mul4(TRL, rx, ry, rz, lx, ly, lz);
        lx /= lz;
        ly /= lz;
        lz = 1;
        float qx, qy, qz;
        mul3(KL, lx, ly, lz, qx, qy, qz);
        int xdi2 = ftoi(qx + 0.5f);
        int ydi2 = ftoi(qy + 0.5f);
        if (xdi2 >= 0 && ydi2 >= 0 && xdi2 < zwidth && ydi2 < zheight) {
            float zc = __ldg(zcur + xdi2 + ydi2 * zwidth);
            float zerr = zc - rz;
            zerr *= zerr;
            if (zerr < 100 * 100) zWeight = 1.0f - zerr / (100.0f * 100.0f);
        }
    }
    res = iResidual;
    zweight = zWeight;
}

// bilinearInterpolation6 of float4 (x,y,z,mask) cloud taps, kernelUtils.h:305-316
__device__ __forceinline__ void bilin_pts(const float4 *cur, int off2, int width, float fx, float fy, float &cx,
                                          float &cy, float &cz, float &m00, float &m10, float &m01, float &m11) {
    float4 v0 = __ldg(cur + off2);
    float4 v1 = __ldg(cur + off2 + 1);
    float4 v2 = __ldg(cur + off2 + width);
    float4 v3 = __ldg(cur + off2 + width + 1);
    cx = (1 - fx) * (1 - fy) * v0.x + fx * (1 - fy) * v1.x + (1 - fx) * fy * v2.x + fx * fy * v3.x;
    cy = (1 - fx) * (1 - fy) * v0.y + fx * (1 - fy) * v1.y + (1 - fx) * fy * v2.y + fx * fy * v3.y;
    cz = (1 - fx) * (1 - fy) * v0.z + fx * (1 - fy) * v1.z + (1 - fx) * fy * v2.z + fx * fy * v3.z;
    m00 = v0.w;
    m10 = v1.w;
    m01 = v2.w;
    m11 = v3.w;
}

}  // namespace rt
