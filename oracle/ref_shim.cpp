// ref_shim.cpp -- host build of reference kernels (test infrastructure).
//
// Compiled only by oracle/build_ref.py into oracle/_ref/libreconref.so.  It
// supplies the CUDA built-ins used by the reference's kernels (float2/3/4,
// threadIdx/blockIdx/blockDim, __global__/__device__, __shared__,
// __syncthreads, a point-sampled tex2D), includes the reference's own
// kernels/kernelUtils.h and the kernel bodies extracted verbatim from the
// reference tree into oracle/_ref/frag_*.inc, and exports ref_* launchers that
// run each kernel over its grid: one-thread-per-element kernels sequentially,
// one-block kernels with barriers as one host thread per CUDA thread.
#include <algorithm>
#include <barrier>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

using std::fabs;
using std::max;
using std::min;
using std::sqrt;

struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
static inline float3 make_float3(float a, float b, float c) { float3 r = {a, b, c}; return r; }
struct uint3_ { unsigned int x, y, z; };
// per host thread, so that a block's threads can run concurrently
static thread_local uint3_ threadIdx, blockIdx, blockDim, gridDim;
typedef unsigned int uint;

#define __global__ static
#define __device__ static inline
#define __host__
// one block at a time: a __shared__ array is a function-level static that the
// block's host threads share, and __syncthreads is a barrier across them
#define __shared__ static
static std::barrier<> *g_block_barrier = nullptr;
#define __syncthreads() g_block_barrier->arrive_and_wait()
typedef double doublereal;

// texture<float4, 2> with point sampling, unnormalised coordinates (the
// reference sets no filter mode): tex2D(t, x, y) is texel (x, y)
struct RgbdTexShim {
    const float4 *data = nullptr;
    int width = 0;
};
static RgbdTexShim rgbdTex;
static inline float4 tex2D(const RgbdTexShim &t, int x, int y) { return t.data[x + y * t.width]; }

// the PhotoTracker method extracted from phototracker.cpp, on its own
struct PhotoTracker {
    bool poseDifferenceExceeded(float *dT, float translationThreshold, float rotationThreshold);
};
void rot2Quaternion(float *m, int n, float *q);  // basic_math.cpp
void normalizeQuaternion(float *qr);
void invertRT4(double *M, double *iM);
void matrixMult4x4(double *M1, double *M2, double *R);
void double_precision4(float *m4, double *m4_dbl);
void float_precision4(double *m4, float *m4_flt);

#include "calib/calib.h"
#define VERTEXBUFFER_STRIDE 24
#define HISTOGRAM64_BIN_COUNT 64

namespace refk {
#include "kernelUtils.h"
#include "frag_warp.inc"
#include "frag_histogram64.inc"
#include "frag_d2z.inc"
#include "frag_rgb2gray.inc"
#include "frag_downSample2Cuda.inc"
#include "frag_filterIndex256.inc"
#include "frag_undistort.inc"
}  // namespace refk

#include "frag_phototracker.inc"

// ---- tracker/kernels/VoxelGrid_cuda.cu (reconstruction stream) ----
// The voxel kernels use the CUDA samples' helper_math.h vector operators
// (componentwise float3 / float4 arithmetic, dot, clamp), restated here, the
// reference's SimParams (kernels/particles_kernel.cuh, included as is) in a
// global `params`, and uint3 values converted from float the way the GPU does
// it: truncation that saturates (negative and NaN give 0), also for the
// `uint += float` steps of the voxel traversal.
void invertRT4(float *M, float *Mi);  // basic_math.cpp:355-368
#include <cfloat>
namespace refv {
using refk::normalize3Cuda;
using refk::rotate3Cuda;
static inline unsigned gpu_f2u(float v) {
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xffffffffu;
    return (unsigned)v;
}
struct SatU {
    unsigned v;
    operator unsigned() const { return v; }
    SatU &operator+=(float f) { v = gpu_f2u((float)v + f); return *this; }
};
struct uint3 { SatU x, y, z; };
static inline uint3 make_uint3(float a, float b, float c) {
    uint3 r = {{gpu_f2u(a)}, {gpu_f2u(b)}, {gpu_f2u(c)}};
    return r;
}
static inline float4 make_float4(float a, float b, float c, float d) { float4 r = {a, b, c, d}; return r; }
static inline float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
static inline float3 operator/(float s, float3 a) { return make_float3(s / a.x, s / a.y, s / a.z); }
static inline float4 operator-(float4 a, float4 b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float clamp(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
static inline float max(float a, float b) { return fmaxf(a, b); }
static inline float min(float a, float b) { return fminf(a, b); }
#include "particles_kernel.cuh"
static SimParams params;
#include "frag_VoxelGrid_cuda.inc"
}  // namespace refv

void expm(float *x, float *Tmotion, float scaleOut);  // tracker/tracker/expm.c:2084 (C++ linkage)

namespace {
template <class F> void launch1d(int n, int block, F f) {
    blockDim = {(unsigned)block, 1, 1};
    int grid = (n + block - 1) / block;
    gridDim = {(unsigned)grid, 1, 1};
    for (int b = 0; b < grid; b++)
        for (int t = 0; t < block; t++) {
            blockIdx = {(unsigned)b, 0, 0};
            threadIdx = {(unsigned)t, 0, 0};
            if (b * block + t < n) f();
        }
}
template <class F> void launch2d(int w, int h, F f) {
    blockDim = {1, 1, 1};
    gridDim = {(unsigned)w, (unsigned)h, 1};
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            blockIdx = {(unsigned)x, (unsigned)y, 0};
            threadIdx = {0, 0, 0};
            f();
        }
}
}  // namespace

extern "C" {

void ref_convertZMapToXYZ(float *z, float *xyzw, float *calib, int W, int H) {
    launch2d(W, H, [&] { refk::convertZMapToXYZKernel(z, (float4 *)xyzw, calib, W); });
}

void ref_convertZMapToXYZ6(float *z, float *pts, int *mask, float *calib, int W, int H) {
    launch2d(W, H, [&] { refk::convertZMapToXYZ6Kernel(z, pts, mask, calib, W); });
}

void ref_xyz2Cloud(float *xyzw, int W, int H, float *calib, float *vdata, float *img) {
    launch2d(W, H, [&] { refk::xyz2CloudKernel((float4 *)xyzw, W, H, calib, vdata, img, 24); });
}

void ref_extractGradient(float *vdata, int n, float *out) {
    launch1d(n, 1024, [&] { refk::extractGradientKernel(vdata, 24, 13, out); });
}

void ref_addVertexAttributes(int *idx, int n, float *vdata, int W, int H, float *calib, float *g1, float *g2,
                             float *g3, float *g4, int L) {
    if (L == 3)
        launch1d(n, 512, [&] { refk::addVertexAttributesWithoutNormalsKernel3(idx, vdata, W, H, calib, g1, g2, g3, 24); });
    else
        launch1d(n, 512, [&] { refk::addVertexAttributesWithoutNormalsKernel4(idx, vdata, W, H, calib, g1, g2, g3, g4, 24); });
}

void ref_precomputeJacobian4(int *idx, int n, float *vdata, float *calib, float *J1, float *J2, float *J3, float *J4,
                             float optScaleIn) {
    launch1d(n, 512, [&] { refk::precomputeJacobian4Kernel(idx, vdata, calib, n, J1, J2, J3, J4, 24, optScaleIn); });
}

void ref_interpolateResidual2(int *idx, int n, float *vdata, float *T, float *calib, int layer, float *img, int w,
                              int h, float *zcur, int zw, int zh, float *residual, float *zweight) {
    int colorOffset = layer == 0 ? 14 : (layer == 1 ? 17 : (layer == 2 ? 20 : 23));
    int divisor = 1 << layer;
    float a = 1.0f / float(divisor);
    float b = 0.5f * (a - 1.0f);
    launch1d(n, 1024, [&] {
        refk::interpolateResidualKernel2(idx, vdata, T, calib, a, b, colorOffset, img, w, h, zcur, zweight, residual,
                                         24, zw, zh);
    });
}

// discretizeResidualKernel -> 64-bin histogram -> seekThreshold64Kernel ->
// generateWeights64Kernel, histogram64.cu:115-157
int ref_generateWeights64(float *residual, int n, float *weights, float *zweights, float *wres, int *hist64) {
    std::vector<int> disc(n);
    launch1d(n, 1024, [&] { refk::discretizeResidualKernel(residual, disc.data()); });
    std::vector<int> h(64, 0);
    for (int i = 0; i < n; i++) h[disc[i]]++;
    if (hist64) memcpy(hist64, h.data(), 64 * sizeof(int));
    launch1d(1, 1, [&] { refk::seekThreshold64Kernel(h.data(), n / 2); });
    int median = h[0];
    launch1d(n, 1024, [&] { refk::generateWeights64Kernel(residual, h.data(), weights, zweights, wres); });
    return median;
}

void ref_weightJacobian(float *J, float *w, int n, float *Jw) {
    launch1d(n, 1024, [&] { refk::weightJacobianKernel(J, w, n, Jw); });
}

void ref_fastDownSampleHdr(float *hi, int wlo, int hlo, float *lo) {
    launch2d(wlo, hlo, [&] { refk::fastDownSampleHdrKernel(hi, 2 * wlo, lo, wlo); });
}

void ref_genPointsCloud6(float *z, int W, int H, float *calib, float *pts, int *mask) {
    launch2d(W, H, [&] { refk::genPointsCloud6Kernel(z, W, H, calib, pts, mask); });
}

void ref_genOrientedPoints6(float *xyz4, float *nrm4, int W, int H, float *calib, float *pts, int *mask) {
    launch2d(W, H, [&] { refk::genOrientedPoints6Kernel((float4 *)xyz4, (float4 *)nrm4, W, H, calib, pts, mask); });
}

// the GPU capture path (d2z.cu, rgb2gray.cu, undistort.cu).  Compiled for the
// host, a negative float converted to unsigned wraps instead of saturating as
// on the GPU, so the disparity kernels differ from the GPU where 2x + x_off or
// 2y + y_off is negative.
void ref_undistortDisparity(unsigned short *d, float *u, int W, int H, float *calib) {
    launch2d(W, H, [&] { refk::undistortDisparityKernel(d, u, W, H, calib); });
}

void ref_d2ZLowGpu(unsigned short *d, float *z, int W, int H, float *calib, float xoff, float yoff) {
    launch2d(W / 2, H / 2, [&] { refk::d2ZLowKernel(d, z, W, H, calib, xoff, yoff); });
}

void ref_d2ZLowHdrGpu(float *d, float *z, int W, int H, float *calib, float xoff, float yoff) {
    launch2d(W / 2, H / 2, [&] { refk::d2ZLowHdrKernel(d, z, W, H, calib, xoff, yoff); });
}

void ref_convertHdrRGB(unsigned char *src, float *dst, int W, int H) {
    launch2d(W, H, [&] { refk::convertHdrRGBKernel(src, dst, (unsigned)W, (unsigned)H); });
}

void ref_rgb2GrayHdr(unsigned char *rgb, float *gray, int W, int H) {
    launch2d(W, H, [&] { refk::rgb2GrayHdrKernel(rgb, gray, W); });
}

void ref_rgbF2GrayHdr(float *rgb, float *gray, int W, int H) {
    launch2d(W, H, [&] { refk::rgbF2GrayHdrKernel(rgb, gray, W); });
}

void ref_undistortHdrRGB(unsigned char *src, float *dst, int W, int H, float *calib) {
    launch2d(W, H, [&] { refk::undistortHdrRGBKernel(src, dst, (unsigned)W, (unsigned)H, calib); });
}

void ref_computeNormals(float *pts, int *mask, int W, int H) {
    launch2d(W, H, [&] { refk::computeNormalsCudaKernel(pts, mask, W, H); });
}

void ref_downSampleCloud6(float *src, int *msrc, float *dst, int *mdst, int wlo, int hlo) {
    launch2d(wlo, hlo, [&] { refk::downSampleCloud6Kernel(dst, mdst, wlo, hlo, src, msrc); });
}

void ref_icpResidualMask2(float *ref6, int *refmask, int w, int h, float *T, float *calib, float *cur6, int *curmask,
                          int layer, float *residual, int *rmask) {
    int divisor = 1 << layer;
    float a = 1.0f / float(divisor);
    float b = 0.5f * (a - 1.0f);
    launch2d(w, h, [&] { refk::icpResidualKernel2(ref6, refmask, w, h, T, calib, cur6, curmask, a, b, residual, rmask); });
}

void ref_icpResidual2(float *ref6, int *select, int nsel, int w, int h, int layer, float *T, float *calib, float *cur6,
                      int *curmask, int npadded, float *res, float *J, float *weights, float optScaleIn) {
    int divisor = 1 << layer;
    float a = 1.0f / float(divisor);
    float b = 0.5f * (a - 1.0f);
    memset(res, 0, sizeof(float) * npadded);
    memset(J, 0, sizeof(float) * 6 * npadded);
    launch1d(nsel, 1024, [&] {
        refk::icpResidualIndexKernel2(ref6, select, nsel, w, h, T, calib, cur6, curmask, a, b, npadded, res, J,
                                      weights, optScaleIn);
    });
}

void ref_packIndex(int *select, int n, float *full, float *r, float *r2) {
    launch1d(n, 1024, [&] { refk::packIndexKernel(select, full, n, r, r2); });
}

// generateStudentTWeights (rgb2gray.cu:854-877) with estimateVariance1024's
// reduction order (rgb2gray.cu:478-547): int truncation per thread, float tree
// per 1024-thread block, int sum over block partials in the last block.
static float ref_estimate_variance(const float *r2, const float *w, int n) {
    int grid = (n + 1023) / 1024;
    std::vector<float> blockSum(grid);
    auto tree = [](float *p) {
        for (int s = 512; s >= 1; s >>= 1)
            for (int t = 0; t < s; t++) p[t] += p[t + s];
        return p[0];
    };
    for (int b = 0; b < grid; b++) {
        float s[1024];
        for (int t = 0; t < 1024; t++) {
            int sum = 0;
            for (long i = (long)b * 1024 + t; i < n; i += 1024L * grid) sum += r2[i] * w[i];
            s[t] = sum;
        }
        blockSum[b] = tree(s);
    }
    if (grid == 1) return blockSum[0]; /* single block: no lower clamp (rgb2gray.cu:497-499) */
    float s[1024];
    for (int t = 0; t < 1024; t++) {
        int sum = 0;
        for (int i = t; i < grid; i += 1024) sum += blockSum[i];
        s[t] = sum;
    }
    float v = tree(s);
    float minVal = float(n);
    if (v < minVal) v = minVal;
    return v;
}

void ref_studentT(float *r2, int n, float *w) {
    launch1d(n, 1024, [&] { refk::initWeightsKernel(r2, n, 100.0f, w); });
    for (int it = 0; it < 3; it++) {
        float var = ref_estimate_variance(r2, w, n);
        launch1d(n, 1024, [&] { refk::updateWeightsKernel(r2, n, &var, w); });
    }
    launch1d(n, 1024, [&] { refk::clampWeightsKernel(w, n); });
}

void ref_conjugateGradient(float *A, float *b, double *x) {
    double Adev[16];
    launch1d(1, 1, [&] { refk::conjugateGradientKernel(A, b, 1e-8, 6, Adev); });
    x[0] = Adev[9]; x[1] = Adev[2]; x[2] = Adev[4];
    x[3] = Adev[3]; x[4] = Adev[7]; x[5] = Adev[11];
}

void ref_linearFuse(float *A1, float *b1, float w1, float iN1, float *A2, float *b2, float w2, float iN2) {
    launch1d(36, 36, [&] { refk::linearFuseKernel(A1, b1, w1, iN1, A2, b2, w2, iN2); });
}

void ref_expm(float *x, float *T, float scaleOut) { expm(x, T, scaleOut); }

// filterIndices4 (filterIndex256.cu:172-194): seekThreshold256Kernel2 in one
// thread, then filterIndexKernel4 as one block of 512 threads whose two
// __syncthreads phases run as barriers across 512 host threads.  hist: the
// float histogram (overwritten with the threshold and surplus, as the
// reference does); index: the selected pixel indices, nVertices entries (the
// reference's index buffer: its surplus trimming skips the last segment, so
// it can write past entry P).
void ref_filterIndices4(float *grad, float *hist, int *index, int nVertices, int P, int nbins) {
    blockIdx = {0, 0, 0};
    threadIdx = {0, 0, 0};
    refk::seekThreshold256Kernel2(hist, P, nbins);
    const int nthreads = 512;
    int ppt = nVertices / nthreads;
    std::barrier<> bar(nthreads);
    g_block_barrier = &bar;
    std::vector<std::thread> th;
    th.reserve(nthreads);
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([=] {
            threadIdx = {(unsigned)t, 0, 0};
            blockIdx = {0, 0, 0};
            blockDim = {(unsigned)nthreads, 1, 1};
            gridDim = {1, 1, 1};
            refk::filterIndexKernel4(grad, hist, index, nthreads, ppt, nbins);
        });
    for (auto &x : th) x.join();
    g_block_barrier = nullptr;
}

// rgbTex2GrayHdrZKernel / rgbdTex2DepthKernel (rgb2gray.cu:64-87) over the
// float4 RGBA-D frame bound as the texture
void ref_rgbTex2GrayHdrZ(float *rgbd, int W, int H, float *calib, float *gray, float *z, float *z2) {
    rgbdTex.data = (const float4 *)rgbd;
    rgbdTex.width = W;
    launch2d(W, H, [&] { refk::rgbTex2GrayHdrZKernel(gray, W, H, z, calib); });
    launch2d(W, H, [&] { refk::rgbdTex2DepthKernel(W, H, z2, calib); });
    rgbdTex.data = nullptr;
}

// PhotoTracker::poseDifferenceExceeded (phototracker.cpp:268-288)
int ref_poseDifferenceExceeded(float *dT, float dist, float angle) {
    PhotoTracker p;
    return p.poseDifferenceExceeded(dT, dist, angle) ? 1 : 0;
}

// PhotoTracker::applyIncrement's pose arithmetic (phototracker.cpp:514-531)
// with the reference's basic_math.cpp: T (host, current -> reference, float)
// and the global pose are updated from the tracked pose Trel.
void ref_applyIncrement(float *T, double *globalPose, float *Trel) {
    double TdblPrev[16];
    double_precision4(T, &TdblPrev[0]);
    double iTprev[16];
    invertRT4(&TdblPrev[0], &iTprev[0]);
    double iTdbl[16], Tdbl[16], Tinc[16];
    double_precision4(Trel, &iTdbl[0]);
    invertRT4(&iTdbl[0], &Tdbl[0]);
    float_precision4(&Tdbl[0], T);
    matrixMult4x4(&iTprev[0], &Tdbl[0], &Tinc[0]);
    matrixMult4x4(&globalPose[0], &Tinc[0], &globalPose[0]);
}

}  // extern "C"

// ---- reconstruction stream launchers: every kernel over its whole grid ----
// SimParams as VoxelGrid's constructor and setCameraParams fill it
// (VoxelGrid.cpp:48-106, 266-273): voxelSize = cubeDim / gridResolution,
// T = invertRT4(Tcur) (world -> camera), iT = Tcur, K normalised.
static void ref_tsdf_params(int R, const float *origin, const float *dim, int W, int H, float min_dist, float max_dist,
                            const float *Tcur, const float *K) {
    refv::SimParams &p = refv::params;
    memset(&p, 0, sizeof(p));
    p.maxDist = max_dist;
    p.minDist = min_dist;
    p.winWidth = W;
    p.winHeight = H;
    p.cubeOrigin = make_float3(origin[0], origin[1], origin[2]);
    p.cubeDim = make_float3(dim[0], dim[1], dim[2]);
    p.gridResolution = R;
    p.voxelSize = make_float3(p.cubeDim.x / R, p.cubeDim.y / R, p.cubeDim.z / R);
    if (Tcur) {
        float Tc[16], iTc[16];
        memcpy(Tc, Tcur, sizeof(Tc));
        invertRT4(Tc, iTc);
        memcpy(p.T.m, iTc, sizeof(iTc));
        memcpy(p.iT.m, Tc, sizeof(Tc));
    }
    if (K) memcpy(p.K.m, K, 9 * sizeof(float));
}

template <class F> static void launch3d(int R, F f) {
    blockDim = {1, 1, 1};
    gridDim = {(unsigned)R, (unsigned)R, (unsigned)R};
    threadIdx = {0, 0, 0};
    for (int z = 0; z < R; z++)
        for (int y = 0; y < R; y++)
            for (int x = 0; x < R; x++) {
                blockIdx = {(unsigned)x, (unsigned)y, (unsigned)z};
                f();
            }
}

extern "C" {

void ref_tsdf_reset(float *grid, int nvox) {
    launch1d(nvox, 1024, [&] { refv::resetKernel((float2 *)grid, 1.0f, 0.0f); });
}

void ref_tsdf_reconstruction(float *rgbd, int W, int H, float min_dist, float max_dist, float *dist) {
    ref_tsdf_params(8, (const float[3]){0, 0, 0}, (const float[3]){1, 1, 1}, W, H, min_dist, max_dist, nullptr,
                    nullptr);
    rgbdTex.data = (const float4 *)rgbd;
    rgbdTex.width = W;
    launch2d(W, H, [&] { refv::reconstructionKernel(dist, W, H); });
    rgbdTex.data = nullptr;
}

void ref_tsdf_update(float *grid, int R, float *origin, float *dim, int W, int H, float min_dist, float max_dist,
                     float *Tcur, float *K, float *dist) {
    ref_tsdf_params(R, origin, dim, W, H, min_dist, max_dist, Tcur, K);
    launch3d(R, [&] { refv::updateVoxelsKernel((float2 *)grid, dist); });
}

void ref_tsdf_raycast(float *grid, int R, float *origin, float *dim, int W, int H, float min_dist, float max_dist,
                      float *Tcur, float *K, int filtering, float *xyz) {
    ref_tsdf_params(R, origin, dim, W, H, min_dist, max_dist, Tcur, K);
    launch2d(W, H, [&] { refv::rayCastVoxelsKernel((float2 *)grid, W, H, filtering != 0, (float4 *)xyz); });
}

void ref_tsdf_shade(float *xyz, int W, int H, float *shaded, float *normal) {
    launch2d(W, H, [&] { refv::shadingKernel((float4 *)xyz, W, H, (float4 *)shaded, (float4 *)normal); });
}

void ref_tsdf_resample(float *dst, float *src, int R, float *origin, float *dim, float *Tcur) {
    ref_tsdf_params(R, origin, dim, 8, 8, 0, 1, Tcur, nullptr);
    launch3d(R, [&] { refv::resampleVoxelsKernel((float2 *)dst, (float2 *)src); });
}

}  // extern "C"
