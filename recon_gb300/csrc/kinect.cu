// kinect.cu -- the Kinect pre-processing of the capture path on the GPU:
// disparity -> depth (full and half resolution), RGB -> gray, and the
// undistortion of a gray image (tracker/multicore/multicore.cpp, OMPFunctions
// d2Z, d2ZLow, convert2Gray, undistort / undistortLookup); and the reference's
// own GPU capture path (d2z.cu, rgb2gray.cu, undistort.cu: disparity as float,
// normalised half-resolution depth, RGB -> float RGB -> float gray, RGB
// undistortion into float RGB), further below.
//
// Each kernel computes the reference routine's values bit for bit (FP32 in
// its order, -fmad=false), one thread per output pixel, including what the
// routines leave untouched: they split the rows into 4 (d2Z, d2ZLow,
// convert2Gray) or 6 (undistort) equal blocks, so the rows past the last full
// block are zero (d2Z, d2ZLow) or not written (convert2Gray, undistort).
// Two conversions the reference leaves to the compiler are fixed the way they
// behave on the x86 machines it ran on: a negative shifted source coordinate
// is out of range, and a negative bilinear weight wraps modulo 2^32.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>

#include "../../include/recon_track.h"
#include "../../include/recon_kinect.h"

namespace rt {
void set_last_error(const char *msg);
void add_launches(long long n);
}  // namespace rt

namespace kinect {

// a source coordinate: truncation of i + off, -1 when the sum is negative
__device__ __forceinline__ int src_coord(int i, float off) {
    const float s = (float)i + off;
    return (s >= 0.0f && s < 2147483520.0f) ? (int)s : -1;
}

__device__ __forceinline__ float z_of(float d, float c0, float c1, float min_dist, float max_dist) {
    float z = fabsf(1.0f / (c0 + c1 * d));
    if (z > max_dist || z < min_dist) z = 0.0f;
    return z;
}

// OMPFunctions::d2Z (multicore.cpp:240-275)
__global__ void k_d2z(const uint16_t *__restrict__ disp, int W, int H, float c0, float c1, float min_dist,
                      float max_dist, float x_off, float y_off, float *__restrict__ z) {
    const int xi = blockIdx.x * blockDim.x + threadIdx.x, yi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi >= W || yi >= H) return;
    float out = 0.0f;
    if (yi < 4 * (H / 4)) {
        const int sx = src_coord(xi, x_off), sy = src_coord(yi, y_off);
        if (sx >= 0 && sy >= 0 && sx < W - 1 && sy < H - 1) {
            const float d = (float)disp[sx + (size_t)sy * W];
            if (d < 2047) out = z_of(d, c0, c1, min_dist, max_dist);
        }
    }
    z[xi + (size_t)yi * W] = out;
}

// OMPFunctions::d2ZLow (multicore.cpp:189-238): Wl x Hl from 2Wl x 2Hl
__global__ void k_d2z_low(const uint16_t *__restrict__ disp, int Wl, int Hl, float c0, float c1, float min_dist,
                          float max_dist, float x_off, float y_off, float *__restrict__ z) {
    const int xi = blockIdx.x * blockDim.x + threadIdx.x, yi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi >= Wl || yi >= Hl) return;
    const int W2 = 2 * Wl, H2 = 2 * Hl;
    float out = 0.0f;
    if (yi < 4 * (Hl / 4)) {
        const int sx = src_coord(2 * xi, x_off), sy = src_coord(2 * yi, y_off);
        if (sx >= 0 && sy >= 0 && sx < W2 - 1 && sy < H2 - 1) {
            const size_t o = sx + (size_t)sy * W2;
            const float d1 = (float)disp[o], d2 = (float)disp[o + 1];
            const float d3 = (float)disp[o + 1 + W2], d4 = (float)disp[o + W2];
            if (d1 < 2047 && d2 < 2047 && d3 < 2047 && d4 < 2047) {
                float d = d1;
                if (d2 < d) d = d2;
                if (d3 < d) d = d3;
                if (d4 < d) d = d4;
                out = z_of(d, c0, c1, min_dist, max_dist);
            }
        }
    }
    z[xi + (size_t)yi * Wl] = out;
}

// OMPFunctions::convert2Gray (multicore.cpp:634-652)
__global__ void k_rgb2gray(const uint8_t *__restrict__ rgb, int n, uint8_t *__restrict__ gray) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned r = rgb[3 * (size_t)i], g = rgb[3 * (size_t)i + 1], b = rgb[3 * (size_t)i + 2];
    gray[i] = (uint8_t)((r * 19588u + g * 38469u + b * 7471u) >> 16);
}

// OMPFunctions::undistort and undistortLookup (multicore.cpp:654-770): the
// sampling offset p - (x, y) of the mapping, then the lookup at offset + (x, y)
// with 8-bit fixed-point bilinear weights; the routine zeroes the source's
// upper-left 2x2 pixels (read here as 0, the input is not changed)
__global__ void k_undistort(const uint8_t *__restrict__ src, int W, int H, KinectUndistort u,
                            uint8_t *__restrict__ dst) {
    const int xi = blockIdx.x * blockDim.x + threadIdx.x, yi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi >= W || yi >= 6 * (H / 6)) return;
    const float pu0 = (float)xi, pu1 = (float)yi;
    float pd0 = u.iK[0] * pu0 + u.iK[1] * pu1 + u.iK[2];
    float pd1 = u.iK[3] * pu0 + u.iK[4] * pu1 + u.iK[5];
    const float r2 = (pd0 * pd0) + (pd1 * pd1), r4 = r2 * r2, r6 = r4 * r2;
    const float rd = 1 + u.kc[0] * r2 + u.kc[1] * r4 + u.kc[4] * r6;
    pd0 *= rd;
    pd1 *= rd;
    const float p0 = u.K[0] * pd0 + u.K[1] * pd1 + u.K[2];
    const float p1 = u.K[3] * pd0 + u.K[4] * pd1 + u.K[5];
    float dx, dy;
    // int(p) in [0, size - 2)
    if (p0 > -1.0f && p1 > -1.0f && p0 < (float)(W - 2) && p1 < (float)(H - 2)) {
        dx = p0 - (float)xi;
        dy = p1 - (float)yi;
    } else {
        dx = 0.0f - (float)xi;
        dy = 0.0f - (float)yi;
    }
    const float q0 = dx + (float)xi, q1 = dy + (float)yi;
    const int xq = (int)q0, yq = (int)q1;
    const unsigned fx = (unsigned)(long long)((q0 - (float)xq) * 256.0f);
    const unsigned fy = (unsigned)(long long)((q1 - (float)yq) * 256.0f);
    const size_t o = xq + (size_t)yq * W;
    auto px = [&](size_t i) -> unsigned { return (i == 0 || i == 1 || i == (size_t)W || i == (size_t)W + 1) ? 0u : src[i]; };
    const unsigned i1 = px(o), i2 = px(o + 1), i4 = px(o + W), i3 = px(o + W + 1);
    const unsigned c = fx * fy;
    const unsigned a = 65536 - ((fy + fx) << 8) + c;
    const unsigned b = (fx << 8) - c;
    const unsigned d = 65536 - a - b - c;
    dst[xi + (size_t)yi * W] = (uint8_t)((a * i1 + b * i2 + c * i3 + d * i4) >> 16);
}

// ---- the GPU capture path (d2z.cu, rgb2gray.cu, undistort.cu) ----

// float -> unsigned as the GPU converts it: truncation that saturates
// (negative and NaN give 0)
__device__ __forceinline__ unsigned f2u_sat(float v) {
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xffffffffu;
    return (unsigned)v;
}

// undistortDisparityKernel (d2z.cu:68-85)
__global__ void k_disp_float(const uint16_t *__restrict__ disp, int n, float *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float d = (float)disp[i];
    out[i] = d < 2047 ? d : (float)0xffff;
}

// d2ZLowKernel / d2ZLowHdrKernel (d2z.cu:88-170), T = uint16_t or float
template <typename T>
__global__ void k_depth_normalized(const T *__restrict__ disp, int W, int H, float c0, float c1, float min_dist,
                                   float max_dist, float x_off, float y_off, float *__restrict__ z) {
    const int xi = blockIdx.x * blockDim.x + threadIdx.x, yi = blockIdx.y * blockDim.y + threadIdx.y;
    const int Wl = W / 2;
    if (xi >= Wl || yi >= H / 2) return;
    const unsigned sx = f2u_sat((float)(2 * xi) + x_off), sy = f2u_sat((float)(2 * yi) + y_off);
    float out = 0.0f;
    if (sx < (unsigned)(W - 1) && sy < (unsigned)(H - 1)) {
        const size_t o = sx + (size_t)sy * W;
        const float d1 = (float)disp[o], d2 = (float)disp[o + 1];
        const float d3 = (float)disp[o + 1 + W], d4 = (float)disp[o + W];
        if (d1 < 2047 && d2 < 2047 && d3 < 2047 && d4 < 2047) {
            float d = d1;
            if (d2 < d) d = d2;
            if (d3 < d) d = d3;
            if (d4 < d) d = d4;
            float zz = fabsf(1.0f / (c0 + c1 * d));
            if (zz > max_dist || zz < min_dist) zz = 0.0f;
            out = (zz - min_dist) / (max_dist - min_dist);
        }
    }
    z[xi + (size_t)yi * Wl] = out;
}

// convertHdrRGBKernel (rgb2gray.cu:634-647), one thread per byte
__global__ void k_rgb_hdr(const uint8_t *__restrict__ rgb, int n3, float *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n3) out[i] = ((float)rgb[i]) / 255.0f;
}

// rgb2GrayHdrKernel / rgbF2GrayHdrKernel (rgb2gray.cu:41-62)
__global__ void k_gray_hdr(const uint8_t *__restrict__ rgb, const float *__restrict__ rgbf, int n,
                           float *__restrict__ gray) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t o = 3 * (size_t)i;
    if (rgb)
        gray[i] = (float)((rgb[o] * 19588 + rgb[o + 1] * 38469 + rgb[o + 2] * 7471) >> 16);
    else
        gray[i] = 0.3f * rgbf[o] + 0.59f * rgbf[o + 1] + 0.11f * rgbf[o + 2];
}

// undistortHdrRGBKernel (undistort.cu:110-170)
__global__ void k_undistort_rgb_hdr(const uint8_t *__restrict__ rgb, int W, int H, KinectUndistort u,
                                    float *__restrict__ out) {
    const int xi = blockIdx.x * blockDim.x + threadIdx.x, yi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi >= W || yi >= H) return;
    const size_t pitch = 3 * (size_t)W, oR = 3 * (size_t)xi + yi * pitch;
    const float pu0 = (float)xi, pu1 = (float)yi;
    float pd0 = u.iK[0] * pu0 + u.iK[1] * pu1 + u.iK[2];
    float pd1 = u.iK[3] * pu0 + u.iK[4] * pu1 + u.iK[5];
    const float r2 = (pd0 * pd0) + (pd1 * pd1), r4 = r2 * r2, r6 = r4 * r2;
    const float rd = 1 + u.kc[0] * r2 + u.kc[1] * r4 + u.kc[4] * r6;
    pd0 *= rd;
    pd1 *= rd;
    const float p0 = u.K[0] * pd0 + u.K[1] * pd1 + u.K[2];
    const float p1 = u.K[3] * pd0 + u.K[4] * pd1 + u.K[5];
    // int(p): the GPU's conversion saturates (NaN gives 0)
    const int xdi = __float2int_rz(p0), ydi = __float2int_rz(p1);
    if (xdi >= 0 && ydi >= 0 && (unsigned)xdi < (unsigned)(W - 2) && (unsigned)ydi < (unsigned)(H - 2)) {
        const size_t o2 = 3 * (size_t)xdi + ydi * pitch;
        const float fx = p0 - xdi, fy = p1 - ydi;
        const float a = (1 - fx) * (1 - fy), b = fx * (1 - fy), c = (1 - fx) * fy, d = fx * fy;
#pragma unroll
        for (int ch = 0; ch < 3; ch++) {
            const size_t q = o2 + ch;
            const float v0 = (float)rgb[q] / 255.0f, v1 = (float)rgb[q + 3] / 255.0f;
            const float v2 = (float)rgb[q + pitch] / 255.0f, v3 = (float)rgb[q + pitch + 3] / 255.0f;
            out[oR + ch] = a * v0 + b * v1 + c * v2 + d * v3;
        }
    } else {
        out[oR] = out[oR + 1] = out[oR + 2] = 0.0f;
    }
}

int fail(int code, const char *msg) {
    rt::set_last_error(msg);
    return code;
}

// Launches through cudaLaunchKernelEx, whose return value is the launch's own
// status: an error another part of the process left pending is neither
// reported as this library's nor cleared.
template <typename... KArgs, typename... Args>
int launch(void (*kern)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.stream = s;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
    if (e != cudaSuccess) {
        std::string m = std::string("kernel launch: ") + cudaGetErrorString(e);
        rt::set_last_error(m.c_str());
        return RECON_ERR_CUDA;
    }
    rt::add_launches(1);
    return RECON_OK;
}

}  // namespace kinect

using namespace kinect;

extern "C" {

int recon_kinect_disparity_to_depth(const uint16_t *disp, int32_t width, int32_t height, float c0, float c1,
                                    float min_dist, float max_dist, float x_off, float y_off,
                                    int32_t half_resolution, float *z, void *stream) {
    if (!disp || !z || width < 2 || height < 2 || width > 16384 || height > 16384)
        return fail(RECON_ERR_INVALID_ARG, "bad argument");
    if (half_resolution && (width % 2 || height % 2)) return fail(RECON_ERR_INVALID_ARG, "odd disparity size");
    cudaStream_t s = (cudaStream_t)stream;
    dim3 blk(32, 8);
    if (half_resolution) {
        const int Wl = width / 2, Hl = height / 2;
        return launch(k_d2z_low, dim3((Wl + 31) / 32, (Hl + 7) / 8), blk, s, disp, Wl, Hl, c0, c1, min_dist, max_dist,
                      x_off, y_off, z);
    }
    return launch(k_d2z, dim3((width + 31) / 32, (height + 7) / 8), blk, s, disp, width, height, c0, c1, min_dist,
                  max_dist, x_off, y_off, z);
}

int recon_kinect_rgb_to_gray(const uint8_t *rgb, int32_t width, int32_t height, uint8_t *gray, void *stream) {
    if (!rgb || !gray || width < 1 || height < 1) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    const int n = 4 * width * (height / 4);
    if (n == 0) return RECON_OK;
    return launch(k_rgb2gray, dim3((n + 255) / 256), dim3(256), (cudaStream_t)stream, rgb, n, gray);
}

int recon_kinect_undistort_gray(const uint8_t *src, int32_t width, int32_t height, const float K[9], const float iK[9],
                                const float kc[5], uint8_t *dst, void *stream) {
    if (!src || !dst || !K || !iK || !kc || width < 4 || height < 6) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    KinectUndistort u;
    for (int i = 0; i < 9; i++) {
        u.K[i] = K[i];
        u.iK[i] = iK[i];
    }
    for (int i = 0; i < 5; i++) u.kc[i] = kc[i];
    return launch(k_undistort, dim3((width + 31) / 32, (6 * (height / 6) + 7) / 8), dim3(32, 8), (cudaStream_t)stream, src,
                  width, height, u, dst);
}

int recon_kinect_disparity_to_float(const uint16_t *disp, int32_t width, int32_t height, float *out, void *stream) {
    if (!disp || !out || width < 1 || height < 1 || width > 16384 || height > 16384)
        return fail(RECON_ERR_INVALID_ARG, "bad argument");
    const int n = width * height;
    return launch(k_disp_float, dim3((n + 255) / 256), dim3(256), (cudaStream_t)stream, disp, n, out);
}

int recon_kinect_depth_normalized(const uint16_t *disp_u16, const float *disp_f32, int32_t width, int32_t height,
                                  float c0, float c1, float min_dist, float max_dist, float x_off, float y_off,
                                  float *z_low, void *stream) {
    if ((!disp_u16) == (!disp_f32) || !z_low || width < 2 || height < 2 || width > 16384 || height > 16384 ||
        width % 2 || height % 2)
        return fail(RECON_ERR_INVALID_ARG, "bad argument (one disparity input, even size)");
    const int Wl = width / 2, Hl = height / 2;
    const dim3 grid((Wl + 31) / 32, (Hl + 7) / 8), blk(32, 8);
    cudaStream_t s = (cudaStream_t)stream;
    if (disp_u16)
        return launch(k_depth_normalized<uint16_t>, grid, blk, s, disp_u16, width, height, c0, c1, min_dist, max_dist,
                      x_off, y_off, z_low);
    return launch(k_depth_normalized<float>, grid, blk, s, disp_f32, width, height, c0, c1, min_dist, max_dist, x_off,
                  y_off, z_low);
}

int recon_kinect_rgb_to_hdr(const uint8_t *rgb, int32_t width, int32_t height, float *rgb_hdr, void *stream) {
    if (!rgb || !rgb_hdr || width < 1 || height < 1 || width > 16384 || height > 16384)
        return fail(RECON_ERR_INVALID_ARG, "bad argument");
    const int n3 = 3 * width * height;
    return launch(k_rgb_hdr, dim3((n3 + 255) / 256), dim3(256), (cudaStream_t)stream, rgb, n3, rgb_hdr);
}

int recon_kinect_rgb_to_gray_hdr(const uint8_t *rgb, const float *rgb_hdr, int32_t width, int32_t height,
                                 float *gray, void *stream) {
    if ((!rgb) == (!rgb_hdr) || !gray || width < 1 || height < 1 || width > 16384 || height > 16384)
        return fail(RECON_ERR_INVALID_ARG, "bad argument (one image input)");
    const int n = width * height;
    return launch(k_gray_hdr, dim3((n + 255) / 256), dim3(256), (cudaStream_t)stream, rgb, rgb_hdr, n, gray);
}

int recon_kinect_undistort_rgb_hdr(const uint8_t *rgb, int32_t width, int32_t height, const float K[9],
                                   const float iK[9], const float kc[5], float *rgb_hdr, void *stream) {
    if (!rgb || !rgb_hdr || !K || !iK || !kc || width < 3 || height < 3 || width > 16384 || height > 16384)
        return fail(RECON_ERR_INVALID_ARG, "bad argument");
    KinectUndistort u;
    for (int i = 0; i < 9; i++) {
        u.K[i] = K[i];
        u.iK[i] = iK[i];
    }
    for (int i = 0; i < 5; i++) u.kc[i] = kc[i];
    return launch(k_undistort_rgb_hdr, dim3((width + 31) / 32, (height + 7) / 8), dim3(32, 8), (cudaStream_t)stream,
                  rgb, width, height, u, rgb_hdr);
}

}  // extern "C"
