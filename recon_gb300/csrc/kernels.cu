// kernels.cu -- sm_103a kernels of the dense RGB-D tracking hot path.
//
// Compiled with -fmad=false: every FP32/FP64 expression is rounded operation by
// operation in the reference's source order, so the results reproduce the
// reference semantics (and the CPU oracle) bit for bit.  One launch serves all
// tracker instances of a batch (blockIdx.y = instance).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstddef>
#include <mutex>

#include "scene.h"
#include "exact_arith.cuh"
#include "fx.cuh"
#include "solve.cuh"
#include "track_kernels.cuh"
#include "track_math.cuh"

namespace rt {

#define INST_DESC const InstDesc &d = D[blockIdx.y]

// Copies an instance descriptor (pointers, sizes, calibration) into shared
// memory with one parallel load instead of a chain of dependent global loads.
__device__ __forceinline__ void load_desc(InstDesc &sd, const InstDesc *src_desc) {
    const int *src = reinterpret_cast<const int *>(src_desc);
    int *dst = reinterpret_cast<int *>(&sd);
    for (int k = threadIdx.x; k < (int)(sizeof(InstDesc) / sizeof(int)); k += blockDim.x) dst[k] = __ldg(src + k);
}

// ------------------------------------------------------------------
// input conversion and pyramids
// ------------------------------------------------------------------

// The reference frame's level 0: uint8 gray -> [0,1], uint16 mm -> z = -mm
// (rgb2gray.cu:64-76 for the u8/u16 form, or the float4 RGBA+depth frame with
// its y-flip, rgbTex2GrayHdrZKernel), and its xyz + mask
// (convertZMapToXYZ6Kernel, rgb2gray.cu:595-624; the same formula as
// convertZMapToXYZKernel, 570-593).  The current frame uses
// k_prep_current_pyramid.
__device__ __forceinline__ void convert_pixel(const InstDesc &d, const uint8_t *gp, const uint16_t *dp, const float *fp,
                                              int i, int xi, int yi, float &g, float &z) {
    if (fp) {
        // rgbTex2GrayHdrZKernel: texture read at (x, H-1-y)
        float4 p = __ldg((const float4 *)fp + xi + (d.H - 1 - yi) * d.W);
        g = 0.3f * p.x + 0.59f * p.y + 0.11f * p.z;
        float minDist = d.calib[RC_MIND], maxDist = d.calib[RC_MAXD];
        z = -(p.w * (maxDist - minDist) + minDist);
    } else {
        g = (float)__ldg(gp + i) / 255.0f;
        uint16_t dm = __ldg(dp + i);
        z = dm ? -(float)dm : 0.0f;
    }
}

__global__ void k_convert_level0(const InstDesc *D, const uint8_t *const *in_gray, const uint16_t *const *in_depth,
                                 const float *const *in_rgbd) {
    INST_DESC;
    const uint8_t *gp = in_gray[blockIdx.y];
    const uint16_t *dp = in_depth[blockIdx.y];
    const float *fp = in_rgbd[blockIdx.y];
    if (!fp && (!gp || !dp)) return;  // instance not updated by this call
    int n = d.W * d.H;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int xi = i % d.W, yi = i / d.W;
    float g, z;
    convert_pixel(d, gp, dp, fp, i, xi, yi, g, z);
    float fx = d.calib[RC_KL], fy = d.calib[RC_KL + 4];
    float cx = d.calib[RC_KL + 2], cy = d.calib[RC_KL + 5];
    d.ref_gray[0][i] = g;
    d.ref_z[i] = z;
    d.ref_col[i] = -1.0f;  // a new keyframe has no fused colour
    float minDist = d.calib[RC_MIND], maxDist = d.calib[RC_MAXD];
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    if (z < -minDist && z > -maxDist) {
        o.x = ((float)xi - cx) * z / fx;
        o.y = ((float)yi - cy) * z / fy;
        o.z = z;
        o.w = 1.0f;
    }
    d.ref_pts[0][i] = o;
}

// The current frame's whole pyramid in one pass: the level-0 conversion
// (convert_pixel, and genPointsCloud6Kernel, d2z.cu:436-469, for the cloud)
// and the 2x2 reductions of fastDownSampleHdrKernel and downSampleCloud6Kernel
// for the coarser levels (the expressions of k_downsample, in its order), so
// every value is identical to the separate kernels'.  A CTA of 256 threads
// takes a 32x32 tile of level 0: each thread converts one 2x2 block and
// reduces it to its level-1 pixel in registers; levels 2 and 3 come from the
// level-1 tile in shared memory.  Level 0 is never read back.
constexpr int kPyrTile = 32;

__device__ __forceinline__ void cloud_point(const InstDesc &d, int xi, int yi, float z, float4 &o) {
    float fx = d.calib[RC_KL], fy = d.calib[RC_KL + 4];
    float cx = d.calib[RC_KL + 2], cy = d.calib[RC_KL + 5];
    o = make_float4(0.f, 0.f, 0.f, 0.f);
    if (z < 0) {
        o.x = ((float)xi - cx) * z / fx;
        o.y = ((float)yi - cy) * z / fy;
        o.z = z;
        o.w = 1.0f;
    }
}

// downSampleCloud6Kernel's average of the valid points among four (d2z.cu:557-588)
__device__ __forceinline__ float4 down_points(const float4 &a, const float4 &b, const float4 &c, const float4 &e) {
    float p0 = 0.0f, p1 = 0.0f, p2 = 0.0f, ns = 0.0f;
    const float4 *q[4] = {&a, &b, &c, &e};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (q[k]->w != 0.0f) {
            ns++;
            p0 += q[k]->x;
            p1 += q[k]->y;
            p2 += q[k]->z;
        }
    }
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ns > 0.0f) o = make_float4(p0 / ns, p1 / ns, p2 / ns, 1.0f);
    return o;
}

// In a sequence the kernel also does the per-frame bookkeeping in CTA 0 of
// each instance (saving two launches a frame): with `store_prev` it stores the
// previous frame's tracked pose (k_store_pose), with `begin` it resets the
// frame's statistics and sums (k_begin_track without an initial pose).
__global__ void __launch_bounds__(256) k_prep_current_pyramid(const InstDesc *D, const uint8_t *const *in_gray,
                                                              const uint16_t *const *in_depth,
                                                              const float *const *in_rgbd, int tiles_x,
                                                              float *store_prev, int begin) {
    __shared__ InstDesc sd;
    __shared__ float sg[2][256];   // gray of levels 1 (16x16) and 2 (8x8)
    __shared__ float4 sp[2][256];  // points of levels 1 and 2
    load_desc(sd, D + blockIdx.y);
    __syncthreads();
    const InstDesc &d = sd;
    if (blockIdx.x == 0) {
        int t = threadIdx.x;
        if (store_prev && t < 16) store_prev[16 * blockIdx.y + t] = d.T[t];
        if (begin) {
            if (t < ST_COUNT) d.stats[t] = 0;
            if (t == 0) {
                *d.counter = 0u;
                if (d.trace_count) *d.trace_count = 0;
            }
            for (int k = t; k < 2 * 27 * kFxLimbs; k += blockDim.x) d.fx[k] = 0ull;
            if (t < 2) d.fx_bad[t] = 0;
        }
    }
    const uint8_t *gp = in_gray[blockIdx.y];
    const uint16_t *dp = in_depth[blockIdx.y];
    const float *fp = in_rgbd[blockIdx.y];
    if (!fp && (!gp || !dp)) return;  // instance not updated by this call
    int W = d.W, H = d.H;
    int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    if (tx * kPyrTile >= W || ty * kPyrTile >= H) return;
    int t = threadIdx.x;
    int bx = t % 16, by = t / 16;
    int x0 = tx * kPyrTile + 2 * bx, y0 = ty * kPyrTile + 2 * by;
    // level 0: the 2x2 block (x0, y0) .. (x0 + 1, y0 + 1), in k_downsample's order
    float g[4];
    float4 pt[4];
    bool in0 = x0 < W && y0 < H;
    if (in0) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            int xi = x0 + (k & 1), yi = y0 + (k >> 1);
            g[k] = 0.0f;
            pt[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (xi >= W || yi >= H) continue;
            int i = xi + yi * W;
            float z;
            convert_pixel(d, gp, dp, fp, i, xi, yi, g[k], z);
            cloud_point(d, xi, yi, z, pt[k]);
            d.cur_gray[0][i] = g[k];
            if (d.cur_grayh[0]) d.cur_grayh[0][i] = __float2half_rn(g[k]);  // mixed precision
            d.cur_z[i] = z;
            d.cur_pts[0][i] = pt[k];
        }
    }
    if (d.L < 2) return;
    // level 1 in registers (its pixel exists iff the whole block does)
    int w1 = W >> 1, h1 = H >> 1;
    int x1 = x0 >> 1, y1 = y0 >> 1;
    if (in0 && x1 < w1 && y1 < h1) {
        float gl = (g[0] + g[1] + g[2] + g[3]) / 4.0f;
        float4 o = down_points(pt[0], pt[1], pt[2], pt[3]);
        int i = x1 + y1 * w1;
        d.cur_gray[1][i] = gl;
        if (d.cur_grayh[1]) d.cur_grayh[1][i] = __float2half_rn(gl);
        d.cur_pts[1][i] = o;
        sg[0][t] = gl;
        sp[0][t] = o;
    }
    // levels 2 and 3 from the 16x16 level-1 tile (slot 0), level 2 in slot 1
    int side = 16;
    for (int l = 2; l < d.L; l++) {
        __syncthreads();
        int src = (l - 2) & 1;
        int hs = side;
        side >>= 1;
        int wl = W >> l, hl = H >> l;
        if (t < side * side) {
            int ox = t % side, oy = t / side;
            int gx = tx * (kPyrTile >> l) + ox, gy = ty * (kPyrTile >> l) + oy;
            if (gx < wl && gy < hl) {
                int c0 = 2 * ox + 2 * oy * hs;
                float gl = (sg[src][c0] + sg[src][c0 + 1] + sg[src][c0 + hs] + sg[src][c0 + hs + 1]) / 4.0f;
                float4 o = down_points(sp[src][c0], sp[src][c0 + 1], sp[src][c0 + hs], sp[src][c0 + hs + 1]);
                int i = gx + gy * wl;
                d.cur_gray[l][i] = gl;
                if (d.cur_grayh[l]) d.cur_grayh[l][i] = __float2half_rn(gl);
                d.cur_pts[l][i] = o;
                sg[1 - src][t] = gl;
                sp[1 - src][t] = o;
            }
        }
    }
}

// fastDownSampleHdrKernel (downSample2Cuda.cu:35-42) for the reference gray
// pyramid and downSampleCloud6Kernel (d2z.cu:557-588) for its point and normal
// pyramid.
__global__ void k_downsample(const InstDesc *D, int level, const int *active) {
    INST_DESC;
    if (!active[blockIdx.y]) return;
    if (level >= d.L) return;
    int wlo = d.W >> level, hlo = d.H >> level;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= wlo * hlo) return;
    int x = i % wlo, y = i / wlo;
    int w2 = 2 * wlo;
    int h0 = 2 * x + 2 * y * w2;
    const float *hi = d.ref_gray[level - 1];
    d.ref_gray[level][i] = (hi[h0] + hi[h0 + 1] + hi[h0 + w2] + hi[h0 + w2 + 1]) / 4.0f;

    const float4 *src = d.ref_pts[level - 1];
    int offs[4] = {h0, h0 + 1, h0 + w2, h0 + w2 + 1};
    float p0 = 0.0f, p1 = 0.0f, p2 = 0.0f, n0 = 0.0f, n1 = 0.0f, n2 = 0.0f;
    float ns = 0.0f;
    for (int k = 0; k < 4; k++) {
        float4 s = src[offs[k]];
        if (s.w != 0.0f) {
            ns++;
            p0 += s.x;
            p1 += s.y;
            p2 += s.z;
            float4 nn = d.ref_nrm[level - 1][offs[k]];
            n0 += nn.x;
            n1 += nn.y;
            n2 += nn.z;
        }
    }
    if (ns > 0.0f) {
        p0 /= ns;
        p1 /= ns;
        p2 /= ns;
        n0 /= ns;
        n1 /= ns;
        n2 /= ns;
        normalize3(n0, n1, n2);
        d.ref_nrm[level][i] = make_float4(n0, n1, n2, 0.0f);
        d.ref_pts[level][i] = make_float4(p0, p1, p2, 1.0f);
    } else {
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
        d.ref_pts[level][i] = o;
        d.ref_nrm[level][i] = o;
    }
}

// Gray value the RGB camera sees at point (qx, qy, qz) of its rig's IR frame
// (TLR, distortPoint and the bilinear color1 tap of xyz2CloudKernel,
// d2z.cu:235-331, with the perspective division as one reciprocal and two
// products), from a float image or a uint8 image scaled by 1/255; -1 where
// the 2x2 taps leave the image.  Used by the keyframe fusion only.
template <typename TImg>
__device__ __forceinline__ float rgb_sample(const float *calib, float qx, float qy, float qz, const TImg *img, int W,
                                            int H) {
    float rx, ry, rz;
    mul4(calib + RC_TLR, qx, qy, qz, rx, ry, rz);
    float irz = 1.0f / rz;
    float pux = rx * irz, puy = ry * irz;
    float px, py;
    distort(pux, puy, calib + RC_KCR, calib + RC_KR, px, py);
    int xdi = ftoi(px), ydi = ftoi(py);
    if (!(xdi >= 0 && ydi >= 0 && xdi < W - 1 && ydi < H - 1)) return -1.0f;
    float fx = px - xdi, fy = py - ydi;
    return bilin(xdi, ydi, fx, fy, W, img);
}

// Keyframe depth and colour fusion (the oracle's orc_fuse_rgbd restates the
// same steps): every valid keyframe pixel is back-projected with KL
// (rgb2gray.cu:570-593), mapped into frame f by its tracked pose, looked up at
// the nearest IR pixel (the zWeight tap of warp.cu:306-327), mapped back with
// the inverse pose (as filterDepthIIRKernel does, warp.cu:398-467), gated on
// |dz| < gate and averaged with unit weights (the running mean of
// updateVoxelsKernel, VoxelGrid_cuda.cu:1005-1013).  The divisions are
// written as products with reciprocals (of fx, fy per instance, of the
// depth once per projection); the oracle states the same.  With gray images the
// vertex colour is fused under the same gate: the mean of the keyframe's own
// sample at the point and the accepted frames' samples at T_f p
// (KeyFrameModel::integrateDepthMaps warps the neighbours' RGB images into the
// keyframe, KeyFrameModel.cpp:537-583).  Writes the fused depth in place into
// ref_z and the colour into ref_col (-1 where no sample exists).
// depth / gray: nframes x n_inst frame pointers (gray may be null: depth only,
// colours kept); Tf: nframes x n_inst x 16 poses.
// 8 CTAs per SM (32 registers, a few bytes of spill): more warps to hide the
// per-frame gathers, 447 against 496 us per 30 x 5-frame launch at 44 registers
#ifndef RECON_FUSE_MIN_BLOCKS
#define RECON_FUSE_MIN_BLOCKS 8
#endif
__global__ void __launch_bounds__(256, RECON_FUSE_MIN_BLOCKS) k_fuse_depth(const InstDesc *D, int nframes, int n_inst, const uint16_t *const *depth,
                             const uint8_t *const *gray, const float *Tf, float gate, const int *active) {
    INST_DESC;
    if (!active[blockIdx.y]) return;
    __shared__ float sT[8][16], sTi[8][16];
    if (threadIdx.x < nframes && threadIdx.x < 8) {
        const float *M = Tf + ((size_t)threadIdx.x * n_inst + blockIdx.y) * 16;
        float *Mi = sTi[threadIdx.x];
        for (int k = 0; k < 16; k++) sT[threadIdx.x][k] = M[k];
        // invertRT4Cuda, kernelUtils.h:100-107
        Mi[0] = M[0]; Mi[1] = M[4]; Mi[2] = M[8];   Mi[3] = -(M[0] * M[3] + M[4] * M[7] + M[8] * M[11]);
        Mi[4] = M[1]; Mi[5] = M[5]; Mi[6] = M[9];   Mi[7] = -(M[1] * M[3] + M[5] * M[7] + M[9] * M[11]);
        Mi[8] = M[2]; Mi[9] = M[6]; Mi[10] = M[10]; Mi[11] = -(M[2] * M[3] + M[6] * M[7] + M[10] * M[11]);
        Mi[12] = 0;   Mi[13] = 0;   Mi[14] = 0;     Mi[15] = 1;
    }
    __syncthreads();
    int W = d.W, H = d.H;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W * H) return;
    float minDist = d.calib[RC_MIND], maxDist = d.calib[RC_MAXD];
    const float *KL = d.calib + RC_KL;
    float fx = KL[0], fy = KL[4], cx = KL[2], cy = KL[5];
    float ifx = 1.0f / fx, ify = 1.0f / fy;
    int xi = idx % W, yi = idx / W;
    float z = d.ref_z[idx];
    const bool colour = gray != nullptr;
    if (!(z < -minDist && z > -maxDist)) {
        if (colour) d.ref_col[idx] = -1.0f;
        return;
    }
    float px3 = ((float)xi - cx) * z * ifx, py3 = ((float)yi - cy) * z * ify, pz3 = z;
    float zsum = z, wsum = 1.0f;
    float csum = 0.0f, cw = 0.0f;
    if (colour) {
        float c0 = rgb_sample(d.calib, px3, py3, pz3, d.ref_gray[0], W, H);
        if (c0 >= 0.0f) {
            csum = c0;
            cw = 1.0f;
        }
    }
    for (int f = 0; f < nframes && f < 8; f++) {
        float qx, qy, qz;
        mul4(sT[f], px3, py3, pz3, qx, qy, qz);
        float iqz = 1.0f / qz;
        float q2x = qx * iqz, q2y = qy * iqz;
        float pxl = KL[0] * q2x + KL[1] * q2y + KL[2];
        float pyl = KL[3] * q2x + KL[4] * q2y + KL[5];
        int xd = ftoi(pxl + 0.5f), yd = ftoi(pyl + 0.5f);
        if (xd < 0 || yd < 0 || xd >= W || yd >= H) continue;
        uint16_t dm = depth[(size_t)f * n_inst + blockIdx.y][xd + yd * W];
        float zf = dm ? -(float)dm : 0.0f;
        if (!(zf < -minDist && zf > -maxDist)) continue;
        float mx = ((float)xd - cx) * zf * ifx, my = ((float)yd - cy) * zf * ify, mz = zf;
        float kx, ky, kz;
        mul4(sTi[f], mx, my, mz, kx, ky, kz);
        float dz = kz - z;
        if (fabsf(dz) < gate) {
            zsum += kz;
            wsum += 1.0f;
            if (colour) {
                float c = rgb_sample(d.calib, qx, qy, qz, gray[(size_t)f * n_inst + blockIdx.y], W, H);
                if (c >= 0.0f) {
                    csum += c;
                    cw += 1.0f;
                }
            }
        }
    }
    d.ref_z[idx] = zsum / wsum;
    if (colour) d.ref_col[idx] = cw > 0.0f ? csum / cw : -1.0f;
}

// reference level-0 points from ref_z (convertZMapToXYZ6Kernel, rgb2gray.cu:595-624)
__global__ void k_ref_from_z(const InstDesc *D, const int *active) {
    INST_DESC;
    if (!active[blockIdx.y]) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.W * d.H) return;
    int xi = i % d.W, yi = i / d.W;
    float fx = d.calib[RC_KL], fy = d.calib[RC_KL + 4];
    float cx = d.calib[RC_KL + 2], cy = d.calib[RC_KL + 5];
    float minDist = d.calib[RC_MIND], maxDist = d.calib[RC_MAXD];
    float z = d.ref_z[i];
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    if (z < -minDist && z > -maxDist) {
        o.x = ((float)xi - cx) * z / fx;
        o.y = ((float)yi - cy) * z / fy;
        o.z = z;
        o.w = 1.0f;
    }
    d.ref_pts[0][i] = o;
}

// genOrientedPoints6Kernel (d2z.cu:471-501): the filtered reference's level-0
// ICP points and normals from a ray-cast point image and its normals (float4
// maps of the keyframe's pixels, camera frame); replaces what k_normals wrote
// for the instances whose point pointer is set
__global__ void k_oriented_points(const InstDesc *D, const float *const *in_pts, const float *const *in_nrm) {
    INST_DESC;
    const float4 *pts = reinterpret_cast<const float4 *>(in_pts[blockIdx.y]);
    const float4 *nrm = reinterpret_cast<const float4 *>(in_nrm[blockIdx.y]);
    if (!pts || !nrm) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.W * d.H) return;
    const float4 v = pts[i], n = nrm[i];
    const float len = n.x * n.x + n.y * n.y + n.z * n.z;
    if (v.z < 0 && len > 1e-7f) {
        d.ref_pts[0][i] = make_float4(v.x, v.y, v.z, 1.0f);
        d.ref_nrm[0][i] = make_float4(n.x, n.y, n.z, 0.0f);
    } else {
        d.ref_pts[0][i] = make_float4(0.f, 0.f, 0.f, 0.f);
        d.ref_nrm[0][i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// computeNormalsCudaKernel, d2z.cu:503-537 (reference level 0)
__global__ void k_normals(const InstDesc *D, const int *active) {
    INST_DESC;
    if (!active[blockIdx.y]) return;
    int W = d.W, H = d.H;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * H) return;
    int xi = i % W, yi = i / W;
    float4 me = d.ref_pts[0][i];
    float4 nrm = make_float4(0.f, 0.f, 0.f, 0.f);
    float mask = me.w;
    if (xi < 1 || yi < 1 || xi > W - 2 || yi > H - 2) {
        mask = 0.0f;
    } else {
        float4 x1 = d.ref_pts[0][i - 1], x2 = d.ref_pts[0][i + 1];
        float4 y1 = d.ref_pts[0][i - W], y2 = d.ref_pts[0][i + W];
        if (x1.z < 0 && x2.z < 0 && y1.z < 0 && y2.z < 0) {
            float ux = x2.x - x1.x, uy = x2.y - x1.y, uz = x2.z - x1.z;
            float vx = y2.x - y1.x, vy = y2.y - y1.y, vz = y2.z - y1.z;
            float nx = uy * vz - uz * vy;
            float ny = -(ux * vz - uz * vx);
            float nz = ux * vy - uy * vx;
            normalize3(nx, ny, nz);
            nrm = make_float4(nx, ny, nz, 0.0f);
        } else {
            mask = 0.0f;
        }
    }
    d.ref_nrm[0][i] = nrm;
    // only .w changes; neighbours read x/y/z of this element, which stay the same
    d.ref_pts[0][i].w = mask;
}

// ------------------------------------------------------------------
// photometric reference: vertex records, gradient histogram, selection
// ------------------------------------------------------------------

// The vertex record of keyframe pixel i (xyz2CloudKernel, d2z.cu:235-331):
// v = x y z px py gx gy gmag gray, zero with z = -maxDist where the point is
// invalid or projects within 10 pixels of the border.  The keyframe kernels
// evaluate it twice with the same operations: for every pixel to find the
// gradient magnitude that selects the points, and again for the selected
// points only (so that the other eight planes are never stored).  The point
// is the back-projection of the keyframe depth ref_z, formed as
// k_convert_level0 and k_ref_from_z form the level-0 ICP points (zero out of
// range: xyz alone carries the validity), so a filtered reference's oriented
// points, which later replace those, do not enter it.
__device__ __forceinline__ void vertex_record(const InstDesc &d, int i, int W, int H, float *v) {
    for (int k = 0; k < kVtxPlanes; k++) v[k] = 0.0f;
    v[2] = -d.calib[RC_MAXD];
    float p3x = 0.0f, p3y = 0.0f, p3z = 0.0f;
    {
        float z = d.ref_z[i];
        float minDist = d.calib[RC_MIND], maxDist = d.calib[RC_MAXD];
        if (z < -minDist && z > -maxDist) {
            float fx = d.calib[RC_KL], fy = d.calib[RC_KL + 4];
            float cx = d.calib[RC_KL + 2], cy = d.calib[RC_KL + 5];
            p3x = ((float)(i % W) - cx) * z / fx;
            p3y = ((float)(i / W) - cy) * z / fy;
            p3z = z;
        }
    }
    if (p3z < 0) {
        const float *T = d.calib + RC_TLR;
        float rx, ry, rz;
        mul4(T, p3x, p3y, p3z, rx, ry, rz);
        float pux = rx / rz, puy = ry / rz;
        float px, py;
        distort(pux, puy, d.calib + RC_KCR, d.calib + RC_KR, px, py);
        if (in_bounds10(px, py, W, H)) {
            const float *img = d.ref_gray[0];
            int xdi = ftoi(px), ydi = ftoi(py);
            float fx = px - xdi, fy = py - ydi;
            float color1 = bilin(xdi, ydi, fx, fy, W, img);
            float fused = d.ref_col[i];  // the keyframe fusion's vertex colour, if any
            if (fused >= 0.0f) color1 = fused;
            float colorN = bilin(ftoi(px), ftoi(py - 1.0f), fx, fy, W, img);
            float colorE = bilin(ftoi(px + 1.0f), ftoi(py), fx, fy, W, img);
            float colorW = bilin(ftoi(px - 1.0f), ftoi(py), fx, fy, W, img);
            float colorS = bilin(ftoi(px), ftoi(py + 1.0f), fx, fy, W, img);
            float gradX1 = (colorE - colorW) / 2.0f;
            float gradY1 = (colorS - colorN) / 2.0f;
            float gm = fabsf(gradY1) + fabsf(gradX1);
            v[0] = p3x; v[1] = p3y; v[2] = p3z;
            v[3] = px; v[4] = py;
            v[5] = gradX1; v[6] = gradY1;
            v[7] = gm < 1.0f ? gm : 1.0f;
            v[8] = color1;
        }
    }
}

// The gradient magnitude of every keyframe pixel (xyz2CloudKernel's gmag
// plane) and its 256-bin histogram (gpu_hist.cu:136, cuda_hist.cu:100-152)
// with privatised shared-memory integer atomics.
__global__ void k_xyz2cloud(const InstDesc *D, const int *active) {
    INST_DESC;
    if (!active[blockIdx.y]) return;
    __shared__ int sh[1024];
    int nb = d.select_bins;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) sh[k] = 0;
    __syncthreads();
    int W = d.W, H = d.H, n = W * H;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float v[kVtxPlanes];
        vertex_record(d, i, W, H, v);
        d.gmag[i] = v[7];
        unsigned int bin = (unsigned int)(v[7] * (nb - 1) + 0.5f);
        if (bin < (unsigned)nb) atomicAdd(&sh[bin], 1);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nb; k += blockDim.x)
        if (sh[k]) atomicAdd(&d.grad_hist[k], sh[k]);
}

// seekThreshold256Kernel2 (filterIndex256.cu:26-46) + per-segment counts of
// filterIndexKernel4 (filterIndex256.cu:110-133).  seg layout:
// [0,512) cnt, [512,1024) mcnt, [1024,1536) start, [1536,2048) mstart,
// [2048,2560) kept, [3072] thr, [3073] excess, [3074] written.
__global__ void k_seg_count(const InstDesc *D, const int *active) {
    INST_DESC;
    if (!active[blockIdx.y]) return;
    int nb = d.select_bins, P = d.P;
    __shared__ unsigned int s_thr;
    __shared__ int s_excess;
    __shared__ int s_hist[1024];
    // the histogram in shared memory in one parallel load; the threshold
    // search (from the top bin down) then reads shared memory only
    for (int k = threadIdx.x; k < nb; k += blockDim.x) s_hist[k] = __ldcg(d.grad_hist + k);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int thr = 0;
        int sel = 0;
        for (int k = nb - 1; k >= 0; k--) {
            sel += s_hist[k];
            if (sel > P) { thr = (unsigned)k; break; }
        }
        s_thr = thr;
        s_excess = sel - P;
        if (blockIdx.x == 0) {
            d.seg[3072] = (int)thr;
            d.seg[3073] = sel - P;
        }
    }
    __syncthreads();
    int n = d.W * d.H;
    int ppt = n / kSegments;
    int warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    int lane = threadIdx.x & 31;
    if (warp >= kSegments) return;
    const float *grad = d.gmag;
    unsigned int thr = s_thr;
    int cnt = 0, mcnt = 0;
    for (int base = warp * ppt; base < warp * ppt + ppt; base += 32) {
        int i = base + lane;
        bool in = i < warp * ppt + ppt;
        unsigned int q = in ? (unsigned int)(grad[i] * (nb - 1) + 0.5f) : 0u;
        unsigned int ab = __ballot_sync(0xffffffffu, in && q > thr);
        unsigned int me = __ballot_sync(0xffffffffu, in && q == thr);
        cnt += __popc(ab);
        mcnt += __popc(me);
    }
    if (lane == 0) {
        d.seg[warp] = cnt;
        d.seg[512 + warp] = mcnt;
    }
}

// Exclusive prefix sum of kSegments (512) values in shared memory by the
// CTA's 512 threads: warp scans by shuffles, then the warps' totals.
__device__ __forceinline__ int block_exclusive_scan512(int v, int *warp_tot) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        int t = lane < kSegments / 32 ? warp_tot[lane] : 0;
        int ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, ti, o);
            if (lane >= o) ti += u;
        }
        if (lane < kSegments / 32) warp_tot[lane] = ti - t;  // exclusive warp offsets
    }
    __syncthreads();
    return warp_tot[w] + incl - v;
}

// segment start offsets and the reference's sequential trimming of surplus
// threshold-bin points (filterIndex256.cu:136-157), one CTA of kSegments
// threads per instance: the start offsets are an exclusive prefix sum of the
// counts; the trimming walks the segments in order only while a surplus is
// left (after that it changes nothing), then the threshold-bin offsets are
// an exclusive prefix sum of what was kept, after the last start.
__global__ void k_seg_scan(const InstDesc *D, const int *active) {
    INST_DESC;
    if (!active[blockIdx.y]) return;
    __shared__ int s_kept[kSegments];
    __shared__ int warp_tot[kSegments / 32];
    int t = threadIdx.x;
    int *cnt = d.seg, *mcnt = d.seg + 512, *start = d.seg + 1024, *mstart = d.seg + 1536, *kept = d.seg + 2048;
    int c = __ldcg(cnt + t);
    s_kept[t] = __ldcg(mcnt + t);
    int st = block_exclusive_scan512(c, warp_tot);  // synchronises: s_kept is complete
    start[t] = st;
    if (t == 0) {
        int tooMuch = __ldcg(d.seg + 3073);
        for (int i = 1; i < kSegments && tooMuch > 0; i++) {
            if (s_kept[i - 1] > 0) {
                s_kept[i - 1] -= tooMuch;
                if (s_kept[i - 1] < 0) {
                    tooMuch += s_kept[i - 1];
                    s_kept[i - 1] = 0;
                } else {
                    tooMuch = 0;
                }
            }
        }
    }
    __syncthreads();
    // the total of the counts (the last start plus the last count) begins the threshold-bin offsets
    __shared__ int s_base;
    if (t == kSegments - 1) s_base = st + c;
    int k = s_kept[t];
    int ms = block_exclusive_scan512(k, warp_tot);  // synchronises: s_base is visible
    mstart[t] = s_base + ms;
    kept[t] = k;
    if (t == kSegments - 1) d.seg[3074] = s_base + ms + k;
}

// filterIndexKernel4's scatter (filterIndex256.cu:159-168): one warp per segment
__global__ void k_seg_scatter(const InstDesc *D, const int *active) {
    INST_DESC;
    if (!active[blockIdx.y]) return;
    int nb = d.select_bins, P = d.P;
    int n = d.W * d.H;
    int ppt = n / kSegments;
    int warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    int lane = threadIdx.x & 31;
    if (warp >= kSegments) return;
    const float *grad = d.gmag;
    unsigned int thr = (unsigned int)d.seg[3072];
    int pos_a = d.seg[1024 + warp];
    int pos_m = d.seg[1536 + warp];
    int kept = d.seg[2048 + warp];
    int m = 0;
    unsigned int lower = (1u << lane) - 1u;
    for (int base = warp * ppt; base < warp * ppt + ppt; base += 32) {
        int i = base + lane;
        bool in = i < warp * ppt + ppt;
        unsigned int q = in ? (unsigned int)(grad[i] * (nb - 1) + 0.5f) : 0u;
        bool ia = in && q > thr, im = in && q == thr;
        unsigned int ab = __ballot_sync(0xffffffffu, ia);
        unsigned int me = __ballot_sync(0xffffffffu, im);
        if (ia) {
            int pos = pos_a + __popc(ab & lower);
            if (pos < P) d.sel_idx[pos] = i;
        }
        if (im) {
            int r = m + __popc(me & lower);
            if (r < kept) {
                int pos = pos_m + r;
                if (pos < P) d.sel_idx[pos] = i;
            }
        }
        pos_a += __popc(ab);
        m += __popc(me);
    }
}

// addVertexAttributesWithoutNormalsKernel3/4 (d2z.cu:700-936) and
// precomputeJacobian4Kernel (warp.cu:502-645), fused per selected point.
__global__ void k_attr_jac(const InstDesc *D, const int *active) {
    INST_DESC;
    if (!active[blockIdx.y]) return;
    int P = d.P, L = d.L, W = d.W, H = d.H, n = W * H;
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P) return;
    int pix = d.sel_idx[k];
    float v[kVtxPlanes];
    vertex_record(d, pix, W, H, v);
    float p3x = v[0], p3y = v[1], p3z = v[2];
    float gx[kMaxLevels] = {0, 0, 0, 0}, gy[kMaxLevels] = {0, 0, 0, 0}, col[kMaxLevels] = {0, 0, 0, 0};
    gx[0] = v[5];
    gy[0] = v[6];
    col[0] = v[8];
    const float *T = d.calib + RC_TLR;
    const float *kc = d.calib + RC_KCR;
    const float *KR = d.calib + RC_KR;
    float rx, ry, rz;
    mul4(T, p3x, p3y, p3z, rx, ry, rz);
    {
        float pux = rx / rz, puy = ry / rz;
        float px, py;
        distort(pux, puy, kc, KR, px, py);
        if (in_bounds10(px, py, W, H)) {
            float a = 0.5f, b = -0.25f;
            float lx = px, ly = py;
            for (int l = 1; l < L; l++) {
                lx = a * lx + b;
                ly = a * ly + b;
                int wl = W >> l, hl = H >> l;
                int xdi = ftoi(lx), ydi = ftoi(ly);
                float fracX = lx - xdi, fracY = ly - ydi;
                const float *g = d.ref_gray[l];
                col[l] = bilin_clamped(xdi, ydi, fracX, fracY, wl, hl, g);
                float cN = bilin_clamped(xdi, ydi - 1, fracX, fracY, wl, hl, g);
                float cW = bilin_clamped(xdi - 1, ydi, fracX, fracY, wl, hl, g);
                float cE = bilin_clamped(xdi + 1, ydi, fracX, fracY, wl, hl, g);
                float cS = bilin_clamped(xdi, ydi + 1, fracX, fracY, wl, hl, g);
                gx[l] = (cE - cW) / 2.0f;
                gy[l] = (cS - cN) / 2.0f;
            }
        }
    }
    d.sel_xyz[k] = p3x;
    d.sel_xyz[P + k] = p3y;
    d.sel_xyz[2 * P + k] = p3z;
    for (int l = 0; l < L; l++) {
        d.sel_I[l][k] = col[l];
        if (d.sel_Ih[l]) d.sel_Ih[l][k] = __float2half_rn(col[l]);  // mixed precision
    }

    // precomputeJacobian4Kernel
    float optScaleIn = d.opt_in;
    rx *= optScaleIn;
    ry *= optScaleIn;
    rz *= optScaleIn;
    float dN0 = 1.0f / rz, dN1 = 0, dN2 = -rx / (rz * rz);
    float dN3 = 0, dN4 = 1.0f / rz, dN5 = -ry / (rz * rz);
    float x = rx / rz;
    float y = ry / rz;
    float x2 = x * x, y2 = y * y;
    float x4 = x2 * x2, y4 = y2 * y2;
    float r2 = x2 + y2, r4 = r2 * r2;
    float dD0 = 1 + kc[0] * (3 * x2 + y2) + kc[1] * (5 * x4 + 6 * x2 * y2 + y4) + kc[4] * r4 * (7 * x2 + y2);
    float dD1 = kc[0] * 2 * x * y + kc[1] * 4 * x * y * r2 + kc[4] * 6 * x * y * r4;
    float dD2 = kc[0] * 2 * y * x + kc[1] * 4 * x * y * r2 + kc[4] * 6 * x * y * r4;
    float dD3 = 1 + kc[0] * (3 * x2 + y2) + kc[1] * (5 * x4 + 6 * x2 * y2 + y4) + kc[4] * r4 * (7 * y2 + x2);
    const float dps[6][3] = {{0.0f, -rz, ry}, {rz, 0.0f, -rx}, {-ry, rx, 0.0f},
                             {1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}};
#pragma unroll
    for (int c = 0; c < 6; c++) {
        float drx, dry, drz;
        rot4(T, dps[c][0], dps[c][1], dps[c][2], drx, dry, drz);
        float dpnx = dN0 * drx + dN1 * dry + dN2 * drz;
        float dpny = dN3 * drx + dN4 * dry + dN5 * drz;
        float ddx = dD0 * dpnx + dD1 * dpny;
        float ddy = dD2 * dpnx + dD3 * dpny;
        float ddz = 0;
        float dp2x, dp2y, dp2z;
        mul3(KR, ddx, ddy, ddz, dp2x, dp2y, dp2z);
        for (int l = 0; l < L; l++) {
            float val;
            if (l == 0) val = dp2x * gx[0] + dp2y * gy[0];
            else {
                float s = (l == 1) ? 2.0f : (l == 2 ? 4.0f : 8.0f);
                val = (dp2x / s) * gx[l] + (dp2y / s) * gy[l];
            }
            d.sel_J[l][c * P + k] = val;
            if (d.sel_Jb[l]) d.sel_Jb[l][c * P + k] = __float2bfloat16_rn(val);  // mixed precision
        }
    }
}

// ------------------------------------------------------------------
// ICP: correspondence mask, compaction, Student-t weights
// ------------------------------------------------------------------

// (long long)x for 0 <= x < 2^63 (or x = -0) from the bits of x with integer
// operations: the float -> int64 conversion instruction issues on the FP64
// pipe, which is narrow on this GPU.
__device__ __forceinline__ long long trunc_f32_nonneg(float x) {
    uint32_t bits = __float_as_uint(x) & 0x7fffffffu;
    int E = (int)(bits >> 23);
    if (E < 127) return 0;  // x < 1
    uint64_t m = (uint64_t)((bits & 0x7fffffu) | 0x800000u);
    int sh = E - 150;
    return (long long)(sh >= 0 ? (m << sh) : (m >> -sh));
}

// the reference's int truncation of r^2 w (estimateVariance1024, rgb2gray.cu:519-521)
__device__ __forceinline__ long long trunc_prod(float r2, float w) {
    float prod = r2 * w;
    if (prod >= 0.0f && prod < 8388608.0f) return trunc_small(prod);
    return (prod >= 0.0f && prod < 9.0e18f) ? trunc_f32_nonneg(prod) : (prod >= 9.0e18f ? 9000000000000000000LL : 0);
}

// The Student-t weight (rgb2gray.cu:537-540; the first pass's sigma^2 is 100,
// rgb2gray.cu:827-850)
__device__ __forceinline__ float student_w(float r2, float sigma2) { return 6 / (5 + r2 / sigma2); }

// The residual and mask of pixel i of the level (icpResidualKernel2) from its
// loaded reference point p and normal rn; returns the mask, sets r2.
__device__ __forceinline__ uint8_t icp_mask_pixel(const InstDesc &d, const float *T, int level, float4 p, float4 rn,
                                                  float &r2) {
    r2 = 0.0f;
    if (p.w == 0.0f) return 0;
    int w = d.W >> level, h = d.H >> level;
    const float *K = d.calib + RC_KL;
    float a = 1.0f / (float)(1 << level);
    float b = 0.5f * (a - 1.0f);
    float qx, qy, qz, cnx, cny, cnz;
    mul4(T, p.x, p.y, p.z, qx, qy, qz);
    rot4(T, rn.x, rn.y, rn.z, cnx, cny, cnz);
    float q2x = qx / qz, q2y = qy / qz;
    float p2x = a * (K[0] * q2x + K[2]) + b;
    float p2y = a * (K[4] * q2y + K[5]) + b;
    if (!(p2x >= 0 && p2x < (w - 1) && p2y >= 0 && p2y < (h - 1))) return 0;
    int xdi = ftoi(p2x), ydi = ftoi(p2y);
    int off2 = xdi + ydi * w;
    float fx = p2x - xdi, fy = p2y - ydi;
    float cx, cy, cz, m0, m1, m2, m3;
    bilin_pts(d.cur_pts[level], off2, w, fx, fy, cx, cy, cz, m0, m1, m2, m3);
    if (!(m0 != 0.0f && m1 != 0.0f && m2 != 0.0f && m3 != 0.0f)) return 0;
    float dx = cx - qx, dy = cy - qy, dz = cz - qz;
    float res = dx * cnx + dy * cny + dz * cnz;
    r2 = res * res;
    return 1;
}

// Whether this CTA is the last of the instance's `nblk` CTAs of the launch to
// finish its partial total (written by thread 0 before the call): thread 0 makes
// the total visible, then takes a ticket from the instance's counter; the CTA
// holding the last ticket resets the counter for the next launch and may read
// every partial total.  No CTA waits for another.
__device__ __forceinline__ bool icp_last_block(const InstDesc &d, int nblk) {
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int k = atomicAdd(d.counter + 1, 1u);
        s_last = (k == (unsigned int)nblk - 1u);
        if (s_last) {
            atomicExch(d.counter + 1, 0u);
            __threadfence();
        }
    }
    __syncthreads();
    return s_last != 0;
}

// icpResidualKernel2 (rgb2gray.cu:223-260) with initWeightsKernel's first
// Student-t weight (rgb2gray.cu:827-850): per pixel of the level, whether it is
// a correspondence at the level's start pose and its squared residual; per
// block of 1024 pixels the number of correspondences and the exact int64 sum
// of the truncated r^2 w0 products (the first variance sum).  The ICP sums of
// the iterations run over the pixel grid, so no compacted list is built.
// 6 CTAs per SM (40 registers): more gathers in flight, 63 against 73 us per
// 30-instance launch at 44 registers
#ifndef RECON_MASK_MIN_BLOCKS
#define RECON_MASK_MIN_BLOCKS 6
#endif
__global__ void __launch_bounds__(kLanes, RECON_MASK_MIN_BLOCKS) k_icp_mask(const InstDesc *D, int level) {
    pdl_trigger();
    __shared__ InstDesc sd;
    __shared__ float sT[16];
    __shared__ int s_cnt[kLanes / 32];
    __shared__ long long s_var[kLanes / 32];
    load_desc(sd, D + blockIdx.y);
    __syncthreads();
    const InstDesc &d = sd;
    if (level >= d.L || d.mode == RECON_PHOTOMETRIC) return;
    if (d.iters[d.L - 1 - level] <= 0) return;
    int n = (d.W >> level) * (d.H >> level);
    // the grid covers the batch's largest level; this instance has fewer blocks
    // (its per-block arrays hold exactly that many entries)
    if ((int)blockIdx.x >= (n + kChunk - 1) / kChunk) return;
    pdl_wait();
    if (threadIdx.x < 16) sT[threadIdx.x] = __ldcg(d.T + threadIdx.x);
    if (blockIdx.x == 0 && threadIdx.x == 0) d.work[2] += (unsigned long long)n;
    __syncthreads();
    int cnt = 0;
    long long vsum = 0;
#pragma unroll
    for (int g = 0; g < 2; g++) {
        // two pixels at a time: point and normal loads in flight together
        int i0 = blockIdx.x * kChunk + threadIdx.x + kLanes * (2 * g);
        float4 p[2], rn[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            int i = i0 + kLanes * u;
            p[u] = rn[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (i < n) {
                p[u] = __ldg(d.ref_pts[level] + i);
                rn[u] = __ldg(d.ref_nrm[level] + i);
            }
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            int i = i0 + kLanes * u;
            if (i >= n) continue;
            float r2;
            uint8_t ok = icp_mask_pixel(d, sT, level, p[u], rn[u], r2);
            if (ok) {
                float w0 = student_w(r2, 100.0f);
                vsum += trunc_prod(r2, w0);
            }
            d.icp_r2[i] = r2;
            d.icp_mask[i] = ok;
            cnt += ok;
        }
    }
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    for (int o = 16; o > 0; o >>= 1) vsum += __shfl_xor_sync(0xffffffffu, vsum, o);
    int wid = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_cnt[wid] = cnt;
        s_var[wid] = vsum;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int c = 0;
        long long v = 0;
        for (int k = 0; k < kLanes / 32; k++) {
            c += s_cnt[k];
            v += s_var[k];
        }
        d.icp_blkcnt[blockIdx.x] = c;
        d.icp_blkvar[blockIdx.x] = v;
    }
}

// Student-t pass `pass` (1..3) of a level (updateWeightsKernel /
// clampWeightsKernel, rgb2gray.cu:549-569) over the level's pixel grid: CTA x
// of instance blockIdx.y takes the 1024-pixel blocks [x K, (x+1) K) of the
// instance, K = blocks_per_cta (about one wave of CTAs over the batch), a
// thread four consecutive pixels of each block with the loads of four blocks
// in flight.  Every correspondence is weighed with the variance of the
// previous pass; passes 1 and 2 add the truncated products r^2 w into the
// CTA's partial sum (icp_part) and the instance's last CTA forms the total
// icp_var[pass]; pass 3 clamps at 1 and writes every pixel's weight (0 where
// the pixel is not a correspondence).  Pass 1 first adds up k_icp_mask's block
// totals (every CTA, from L2): the correspondence count and the first
// variance sum, which CTA 0 stores.  The sums are exact int64 sums, so the
// result does not depend on how the pixels are split; one launch per pass
// keeps every SM busy without any CTA waiting on another.  48 registers: five
// CTAs per SM (kPassCtaSlots).
__global__ void __launch_bounds__(kLanes) k_icp_student_pass(const InstDesc *D, int level, int pass,
                                                             int blocks_per_cta) {
    pdl_trigger();
    __shared__ InstDesc sd;
    __shared__ long long s_var[kLanes / 32];
    __shared__ int s_cnt[kLanes / 32];
    load_desc(sd, D + blockIdx.y);
    __syncthreads();
    const InstDesc &d = sd;
    if (level >= d.L || d.mode == RECON_PHOTOMETRIC) return;
    if (d.iters[d.L - 1 - level] <= 0) return;
    int n = (d.W >> level) * (d.H >> level);
    int nblk = (n + kChunk - 1) / kChunk;
    int nctas = (nblk + blocks_per_cta - 1) / blocks_per_cta;
    if ((int)blockIdx.x >= nctas) return;
    int b_first = blockIdx.x * blocks_per_cta;
    int b_last = min(b_first + blocks_per_cta, nblk);
    int wid = threadIdx.x >> 5;
    pdl_wait();
    int nsel;
    long long var;
    if (pass == 1) {
        int c = 0;
        long long v = 0;
        for (int k = threadIdx.x; k < nblk; k += kLanes) {
            c += __ldcg(d.icp_blkcnt + k);
            v += __ldcg(d.icp_blkvar + k);
        }
        c = __reduce_add_sync(0xffffffffu, c);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) {
            s_cnt[wid] = c;
            s_var[wid] = v;
        }
        __syncthreads();
        nsel = 0;
        var = 0;
        for (int k = 0; k < kLanes / 32; k++) {
            nsel += s_cnt[k];
            var += s_var[k];
        }
        __syncthreads();  // s_var is reused for this pass's sum
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            d.icp_nsel[level] = nsel;
            // ICP weight of the fused system, kept off the iteration's critical path
            d.fuse_c2[level] = (double)d.lambda / (double)nsel;
            d.icp_var[0] = (unsigned long long)var;
        }
    } else {
        nsel = __ldcg(d.icp_nsel + level);
        var = (long long)__ldcg(d.icp_var + pass - 1);
    }
    float Sf = (float)var;
    float minVal = (float)nsel;
    float vv = (nsel <= 1024) ? Sf : (Sf < minVal ? minVal : Sf);
    float sigma2 = vv / (float)nsel;
    long long vsum = 0;
    for (int b0 = b_first; b0 < b_last; b0 += 4) {
        float4 r[4];
        uchar4 m[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            int i = (b0 + u) * kChunk + 4 * threadIdx.x;
            r[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            m[u] = make_uchar4(0, 0, 0, 0);
            if (b0 + u >= b_last || i >= n) continue;
            if (i + 3 < n) {
                // 16- and 4-byte aligned: the arrays start on 256-byte boundaries
                r[u] = __ldg(reinterpret_cast<const float4 *>(d.icp_r2 + i));
                m[u] = __ldg(reinterpret_cast<const uchar4 *>(d.icp_mask + i));
            } else {
                // the instance's last pixels (n not a multiple of 4)
                r[u].x = __ldg(d.icp_r2 + i);
                m[u].x = __ldg(d.icp_mask + i);
                if (i + 1 < n) {
                    r[u].y = __ldg(d.icp_r2 + i + 1);
                    m[u].y = __ldg(d.icp_mask + i + 1);
                }
                if (i + 2 < n) {
                    r[u].z = __ldg(d.icp_r2 + i + 2);
                    m[u].z = __ldg(d.icp_mask + i + 2);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            int i = (b0 + u) * kChunk + 4 * threadIdx.x;
            if (b0 + u >= b_last || i >= n) continue;
            if (pass == 3) {
                float4 w = make_float4(m[u].x ? fminf(student_w(r[u].x, sigma2), 1.0f) : 0.0f,
                                       m[u].y ? fminf(student_w(r[u].y, sigma2), 1.0f) : 0.0f,
                                       m[u].z ? fminf(student_w(r[u].z, sigma2), 1.0f) : 0.0f,
                                       m[u].w ? fminf(student_w(r[u].w, sigma2), 1.0f) : 0.0f);
                if (i + 3 < n) {
                    *reinterpret_cast<float4 *>(d.icp_w + i) = w;
                } else {
                    d.icp_w[i] = w.x;
                    if (i + 1 < n) d.icp_w[i + 1] = w.y;
                    if (i + 2 < n) d.icp_w[i + 2] = w.z;
                }
            } else {
                // pixels past the end have mask 0
                if (m[u].x) vsum += trunc_prod(r[u].x, student_w(r[u].x, sigma2));
                if (m[u].y) vsum += trunc_prod(r[u].y, student_w(r[u].y, sigma2));
                if (m[u].z) vsum += trunc_prod(r[u].z, student_w(r[u].z, sigma2));
                if (m[u].w) vsum += trunc_prod(r[u].w, student_w(r[u].w, sigma2));
            }
        }
    }
    if (pass == 3) return;
    for (int o = 16; o > 0; o >>= 1) vsum += __shfl_xor_sync(0xffffffffu, vsum, o);
    if ((threadIdx.x & 31) == 0) s_var[wid] = vsum;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long v = 0;
        for (int k = 0; k < kLanes / 32; k++) v += s_var[k];
        d.icp_part[blockIdx.x] = v;
    }
    if (!icp_last_block(d, nctas)) return;
    long long v = 0;
    for (int k = threadIdx.x; k < nctas; k += kLanes) v += __ldcg(d.icp_part + k);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_var[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long tot = 0;
        for (int k = 0; k < kLanes / 32; k++) tot += s_var[k];
        d.icp_var[pass] = (unsigned long long)tot;
    }
}

// ------------------------------------------------------------------
// one Gauss-Newton iteration for every instance
// ------------------------------------------------------------------

constexpr int kIterThreads = kIterBlock;  // one canonical lane (4 points of a chunk) per thread
constexpr int kCluster = kIterCluster;
constexpr int kFxTerms = 27 * kFxLimbs;

// 16-byte aligned: J is the destination of 16-byte cp.async copies
struct __align__(16) IterShared {
    float T[16];
    long long fx[27][kFxLimbs];  // this CTA's fixed-point sums of its warp totals
    int fx_bad;
    double A_ph[27];    // the allocation-free entry point's photometric terms
    // photometric CTAs: the Jacobian of the CTA's first chunk; ICP CTAs: the
    // Jacobians of the chunk being reduced (with R, its residuals)
    __align__(16) float J[6][kChunk];
    float R[kChunk];
    int hist[256];      // this CTA's photometric histogram (read by its cluster)
    int hist_all[256];  // the instance's histogram
    int median;
    SolveScratch S;     // the allocation-free entry point's solve
};

static_assert(alignof(IterShared) >= 16 && offsetof(IterShared, J) % 16 == 0 && (kChunk * sizeof(float)) % 16 == 0,
              "cp.async destinations must be 16-byte aligned");

struct SolveShared {
    float T[16];
    double A_ph[27], A_icp[27];
    SolveScratch S;
    // scalars loaded with the sums
    double fuse_c2;
    unsigned long long work0, work1;
    int nsel, median, st_iters, st_solves, st_nonspd, trace_slot;
};

__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory"); }

// address of `p` (a shared-memory variable of this CTA) in CTA `rank` of the cluster
template <class T> __device__ __forceinline__ T *cluster_peer(T *p, int rank) {
    unsigned long long out;
    asm volatile("mapa.u64 %0, %1, %2;\n" : "=l"(out) : "l"((unsigned long long)p), "r"(rank));
    return reinterpret_cast<T *>(out);
}

__device__ __forceinline__ void fx_clear(IterShared &sh) {
    for (int k = threadIdx.x; k < kFxTerms; k += blockDim.x) (&sh.fx[0][0])[k] = 0;
    if (threadIdx.x == 0) sh.fx_bad = 0;
}

// Adds warp total v of term q (lane q of warp_terms) to the CTA's fixed-point
// sums; the 8 warps of a CTA add to the same limbs with shared-memory atomics.
__device__ __forceinline__ void fx_add_term(IterShared &sh, int q, float v) {
    int k0, bad = 0;
    long long lo, hi;
    fx_split(v, k0, lo, hi, bad);
    if (lo) atomicAdd(reinterpret_cast<unsigned long long *>(&sh.fx[q][k0]), (unsigned long long)lo);
    if (hi) atomicAdd(reinterpret_cast<unsigned long long *>(&sh.fx[q][k0 + 1]), (unsigned long long)hi);
    if (bad) sh.fx_bad = 1;
}

// Adds the CTA's fixed-point sums to the instance's (after a __syncthreads).
__device__ __forceinline__ void fx_flush(const IterShared &sh, unsigned long long *dst, int *dst_bad) {
    if (threadIdx.x < kFxTerms) {
        long long v = (&sh.fx[0][0])[threadIdx.x];
        if (v) atomicAdd(dst + threadIdx.x, (unsigned long long)v);
    }
    if (threadIdx.x == 0 && sh.fx_bad) atomicOr(dst_bad, 1);
}

// canonical per-lane accumulation of the 27 normal-equation terms, one fused
// multiply-add per product (the oracle's fmaf)
__device__ __forceinline__ void acc27(float *s, const float *j, float r) {
    int q = 0;
#pragma unroll
    for (int a = 0; a < 6; a++)
#pragma unroll
        for (int c = a; c < 6; c++, q++) s[q] = __fmaf_rn(j[a], j[c], s[q]);
#pragma unroll
    for (int c = 0; c < 6; c++, q++) s[q] = __fmaf_rn(j[c], r, s[q]);
}

// Warp totals of the 27 terms by recursive halving: at the step with offset o
// each lane keeps half of its values and adds the partner's copy of them, so
// lane q ends with term q.  Every addition pairs the same two partial sums as
// the canonical xor butterfly (offsets 16, 8, 4, 2, 1), so the totals are the
// butterfly's bit for bit, with 31 shuffles instead of 135.
__device__ __forceinline__ float warp_terms(const float *v) {
    int lane = threadIdx.x & 31;
    float a[16];
    bool h = lane & 16;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        float x = v[i], y = (i + 16 < 27) ? v[i + 16] : 0.0f;
        float send = h ? x : y, keep = h ? y : x;
        a[i] = keep + __shfl_xor_sync(kFull, send, 16);
    }
    float b[8];
    h = lane & 8;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        float send = h ? a[i] : a[i + 8], keep = h ? a[i + 8] : a[i];
        b[i] = keep + __shfl_xor_sync(kFull, send, 8);
    }
    float c[4];
    h = lane & 4;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float send = h ? b[i] : b[i + 4], keep = h ? b[i + 4] : b[i];
        c[i] = keep + __shfl_xor_sync(kFull, send, 4);
    }
    float e[2];
    h = lane & 2;
#pragma unroll
    for (int i = 0; i < 2; i++) {
        float send = h ? c[i] : c[i + 2], keep = h ? c[i + 2] : c[i];
        e[i] = keep + __shfl_xor_sync(kFull, send, 2);
    }
    h = lane & 1;
    float send = h ? e[0] : e[1], keep = h ? e[1] : e[0];
    return keep + __shfl_xor_sync(kFull, send, 1);
}

// Median bin of an instance histogram (seekThreshold64Kernel,
// histogram64.cu:48-61): first bin whose cumulative count exceeds P/2.  Warp 0.
__device__ __forceinline__ void hist_median(IterShared &sh, const int *hist, int nb, int P) {
    if (threadIdx.x >= 32) return;
    int lane = threadIdx.x;
    int per = (nb + 31) / 32;
    int loc = 0;
    for (int k = 0; k < per; k++) {
        int bin = lane * per + k;
        if (bin < nb) loc += hist[bin];
    }
    int incl = loc;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    int half = P / 2;
    unsigned int over = __ballot_sync(0xffffffffu, incl > half);
    if (over) {
        int l0 = __ffs(over) - 1;
        if (lane == l0) {
            int acc = incl - loc, med = 0;
            for (int k = 0; k < per; k++) {
                int bin = lane * per + k;
                if (bin < nb) {
                    acc += hist[bin];
                    if (acc > half) { med = bin; break; }
                }
            }
            sh.median = med;
        }
    } else if (lane == 0) {
        sh.median = 0;
    }
}

// One photometric iteration by a single 256-thread CTA (the allocation-free
// entry point): residuals, histogram, median, weights and the fixed-point sums
// of all P points; the 27 terms end in sh.A_ph.
__device__ void photo_iteration(const InstDesc &d, IterShared &sh, int level) {
    int P = d.P;
    int w = d.W >> level, h = d.H >> level;
    float a = 1.0f / (float)(1 << level);
    float b = 0.5f * (a - 1.0f);
    const float *img = d.cur_gray[level];
    const float *I = d.sel_I[level];
    int nb = d.hist_bins;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) sh.hist[k] = 0;
    fx_clear(sh);
    __syncthreads();
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        float r, zw;
        photo_residual(d.calib, sh.T, a, b, d.sel_xyz[i], d.sel_xyz[P + i], d.sel_xyz[2 * P + i], I[i], img, w, h,
                       d.cur_z, d.W, d.H, r, zw);
        d.ph_r[i] = r;
        d.ph_zw[i] = zw;
        atomicAdd(&sh.hist[mad_bin(r, nb)], 1);
    }
    __syncthreads();
    hist_median(sh, sh.hist, nb, P);
    __syncthreads();
    float s = mad_scale(sh.median, nb);
    const float *J = d.sel_J[level];
    int t = threadIdx.x, lane = t & 31;
    for (int c = 0; c < P / kChunk; c++) {
        float acc[27];
#pragma unroll
        for (int q = 0; q < 27; q++) acc[q] = 0.0f;
        for (int m = 0; m < 4; m++) {
            int i = c * kChunk + t + kLanes * m;
            float r = d.ph_r[i];
            float wv = tukey_weight(r, d.ph_zw[i], s);
            float jw[6];
#pragma unroll
            for (int k = 0; k < 6; k++) jw[k] = J[k * P + i] * wv;
            acc27(acc, jw, r * wv);
        }
        float v = warp_terms(acc);
        if (lane < 27) fx_add_term(sh, lane, v);
    }
    __syncthreads();
    if (threadIdx.x < 27) {
        long long L[kFxLimbs];
#pragma unroll
        for (int k = 0; k < kFxLimbs; k++) L[k] = sh.fx[threadIdx.x][k];
        sh.A_ph[threadIdx.x] = sh.fx_bad ? __longlong_as_double(0x7ff8000000000000LL) : fx_to_double(L);
    }
}

// The inputs of ICP pixel `idx` of the level: its last Student-t weight and
// its reference point and normal (weight 0 past the end of the grid).  (A
// packed 24-byte point + normal layout was measured: no change, the kernel is
// bound by latency and issue, not by these bytes.)
__device__ __forceinline__ void icp_load(const InstDesc &d, int level, int idx, int npix, float &weight, float4 &p,
                                         float4 &rn) {
    weight = 0.0f;
    p = rn = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (idx < npix) {
        weight = __ldg(d.icp_w + idx);
        p = __ldg(d.ref_pts[level] + idx);
        rn = __ldg(d.ref_nrm[level] + idx);
    }
}

// icpResidualIndexKernel2, rgb2gray.cu:323-390, for one pixel of the level.  A
// pixel that is not a correspondence has weight 0, and the reference's test
// `weight > 0` then gives zeros.  The projection, the bilinear taps and the
// correspondence test are the reference's expressions without contraction
// (they decide which pixels count); the rotated normal, the residual and the
// Jacobian, continuous terms of the normal equations only, are evaluated with
// fused multiply-adds (one rounding per multiply-add; the oracle's
// orc_icp_residual_jacobian_grid states the same sequence with fmaf).
__device__ __forceinline__ void icp_point(const InstDesc &d, const float *T, int level, float weight, float4 p,
                                          float4 rn, float *j, float &res) {
    res = 0.0f;
#pragma unroll
    for (int c = 0; c < 6; c++) j[c] = 0.0f;
    if (!(weight > 0.0f)) return;
    int w = d.W >> level, h = d.H >> level;
    const float *K = d.calib + RC_KL;
    float a = 1.0f / (float)(1 << level);
    float b = 0.5f * (a - 1.0f);
    float qx, qy, qz;
    mul4(T, p.x, p.y, p.z, qx, qy, qz);
    float q2x = qx / qz, q2y = qy / qz;
    float p2x = a * (K[0] * q2x + K[2]) + b;
    float p2y = a * (K[4] * q2y + K[5]) + b;
    if (!(p2x >= 0 && p2x < (w - 1) && p2y >= 0 && p2y < (h - 1))) return;
    int xdi = ftoi(p2x), ydi = ftoi(p2y);
    float fx = p2x - xdi, fy = p2y - ydi;
    int off2 = xdi + ydi * w;
    float cx, cy, cz, m0, m1, m2, m3;
    bilin_pts(d.cur_pts[level], off2, w, fx, fy, cx, cy, cz, m0, m1, m2, m3);
    if (!(m0 != 0.0f && fabsf(cz - qz) < 300.0f)) return;
    float optScaleIn = d.opt_in;
    float rvx = cx - qx, rvy = cy - qy, rvz = cz - qz;
    float cnx = __fmaf_rn(T[2], rn.z, __fmaf_rn(T[1], rn.y, T[0] * rn.x));
    float cny = __fmaf_rn(T[6], rn.z, __fmaf_rn(T[5], rn.y, T[4] * rn.x));
    float cnz = __fmaf_rn(T[10], rn.z, __fmaf_rn(T[9], rn.y, T[8] * rn.x));
    res = optScaleIn * weight * __fmaf_rn(rvz, cnz, __fmaf_rn(rvy, cny, rvx * cnx));
    // The reference rotates the columns of [p]x and [n]x and the unit vectors
    // with full 3x3 products.  The terms it multiplies by an exact 0 or 1 are
    // dropped here: for a finite pose that changes at most the sign of a zero
    // Jacobian entry, and signed zeros add nothing to the fixed-point sums.
    float b0x = __fmaf_rn(T[1], -p.z, T[2] * p.y), b0y = __fmaf_rn(T[5], -p.z, T[6] * p.y),
          b0z = __fmaf_rn(T[9], -p.z, T[10] * p.y);
    float b1x = __fmaf_rn(T[0], p.z, T[2] * -p.x), b1y = __fmaf_rn(T[4], p.z, T[6] * -p.x),
          b1z = __fmaf_rn(T[8], p.z, T[10] * -p.x);
    float b2x = __fmaf_rn(T[0], -p.y, T[1] * p.x), b2y = __fmaf_rn(T[4], -p.y, T[5] * p.x),
          b2z = __fmaf_rn(T[8], -p.y, T[9] * p.x);
    float n0x = __fmaf_rn(T[1], -rn.z, T[2] * rn.y), n0y = __fmaf_rn(T[5], -rn.z, T[6] * rn.y),
          n0z = __fmaf_rn(T[9], -rn.z, T[10] * rn.y);
    float n1x = __fmaf_rn(T[0], rn.z, T[2] * -rn.x), n1y = __fmaf_rn(T[4], rn.z, T[6] * -rn.x),
          n1z = __fmaf_rn(T[8], rn.z, T[10] * -rn.x);
    float n2x = __fmaf_rn(T[0], -rn.y, T[1] * rn.x), n2y = __fmaf_rn(T[4], -rn.y, T[5] * rn.x),
          n2z = __fmaf_rn(T[8], -rn.y, T[9] * rn.x);
    float so = -optScaleIn * weight;
    // -cn . b + rv . n, accumulated left to right
    auto row = [&](float bx, float by, float bz, float nx, float ny, float nz) {
        float t = -cnx * bx;
        t = __fmaf_rn(-cny, by, t);
        t = __fmaf_rn(-cnz, bz, t);
        t = __fmaf_rn(rvx, nx, t);
        t = __fmaf_rn(rvy, ny, t);
        return __fmaf_rn(rvz, nz, t);
    };
    j[0] = so * row(b0x, b0y, b0z, n0x, n0y, n0z);
    j[1] = so * row(b1x, b1y, b1z, n1x, n1y, n1z);
    j[2] = so * row(b2x, b2y, b2z, n2x, n2y, n2z);
#pragma unroll
    for (int c = 0; c < 3; c++)
        j[3 + c] = -weight * __fmaf_rn(-cnz, T[8 + c], __fmaf_rn(-cny, T[4 + c], -cnx * T[c]));
}

// The arrays the photometric term reads: FP32, or (mixed precision) the FP16
// current image and reference intensities and the BF16 Jacobian.  Widening a
// stored FP16 / BF16 value to FP32 is exact, so the arithmetic that follows is
// the FP32 path's on rounded inputs.
template <bool kMixed> struct PhotoArrays;
template <> struct PhotoArrays<false> {
    using TI = float;
    using TJ = float;
    static __device__ const float *img(const InstDesc &d, int l) { return d.cur_gray[l]; }
    static __device__ const float *I(const InstDesc &d, int l) { return d.sel_I[l]; }
    static __device__ const float *J(const InstDesc &d, int l) { return d.sel_J[l]; }
};
template <> struct PhotoArrays<true> {
    using TI = __half;
    using TJ = __nv_bfloat16;
    static __device__ const __half *img(const InstDesc &d, int l) { return d.cur_grayh[l]; }
    static __device__ const __half *I(const InstDesc &d, int l) { return d.sel_Ih[l]; }
    static __device__ const __nv_bfloat16 *J(const InstDesc &d, int l) { return d.sel_Jb[l]; }
};

// Photometric residuals of lane t's 4 points of chunk c
// (interpolateResidualKernel2, warp.cu:269-332).
template <bool kMixed>
__device__ __forceinline__ void photo_lane_residuals(const InstDesc &d, const float *T, int level, int c, int t,
                                                     float *r, float *zw) {
    int P = d.P;
    int w = d.W >> level, h = d.H >> level;
    float a = 1.0f / (float)(1 << level);
    float b = 0.5f * (a - 1.0f);
    const auto *img = PhotoArrays<kMixed>::img(d, level);
    const auto *I = PhotoArrays<kMixed>::I(d, level);
#pragma unroll
    for (int m = 0; m < 4; m++) {
        int i = c * kChunk + t + kLanes * m;
        photo_residual(d.calib, T, a, b, __ldg(d.sel_xyz + i), __ldg(d.sel_xyz + P + i), __ldg(d.sel_xyz + 2 * P + i),
                       ldf(I + i), img, w, h, d.cur_z, d.W, d.H, r[m], zw[m]);
    }
}

// The photometric term of an instance by its cluster of 8 CTAs: CTA `rank`
// evaluates chunks rank, rank + 8, ...; the cluster adds its histograms
// (histogram64.cu:115-145) through distributed shared memory, every CTA finds
// the median bin (seekThreshold64Kernel, histogram64.cu:48-61) and weighs its
// own points (generateWeights64Kernel, 79-94) into the CTA's fixed-point sums.
// Returns whether this CTA had a chunk.
template <bool kMixed>
__device__ bool photo_cluster(const InstDesc &d, IterShared &sh, int level, int rank) {
    using TJ = typename PhotoArrays<kMixed>::TJ;
    int P = d.P, nph = P / kChunk, nb = d.hist_bins;
    int t = threadIdx.x, lane = t & 31;
    const TJ *J = PhotoArrays<kMixed>::J(d, level);
    // the Jacobian tile in shared memory, in its stored type (a BF16 tile uses
    // the first half of sh.J)
    TJ(*sJ)[kChunk] = reinterpret_cast<TJ(*)[kChunk]>(&sh.J[0][0]);
    constexpr int kPer16 = 16 / sizeof(TJ);  // values per 16-byte copy
    // the first chunk's Jacobian does not depend on the pose: copy it to shared
    // memory asynchronously while the residuals are evaluated
    if (rank < nph) {
        for (int k = t; k < 6 * (kChunk / kPer16); k += blockDim.x) {
            int col = k / (kChunk / kPer16), q = k % (kChunk / kPer16);
            const TJ *src = J + (size_t)col * P + rank * kChunk + kPer16 * q;
            unsigned int dst = (unsigned int)__cvta_generic_to_shared(&sJ[col][kPer16 * q]);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    for (int k = t; k < nb; k += blockDim.x) sh.hist[k] = 0;
    __syncthreads();
    float r0[4], zw0[4];
    for (int c = rank; c < nph; c += kCluster) {
        float r[4], zw[4];
        photo_lane_residuals<kMixed>(d, sh.T, level, c, t, r, zw);
#pragma unroll
        for (int m = 0; m < 4; m++) {
            // one shared-memory atomic per distinct bin of the warp
            int bin = mad_bin(r[m], nb);
            unsigned int peers = __match_any_sync(kFull, bin);
            if ((t & 31) == __ffs(peers) - 1) atomicAdd(&sh.hist[bin], __popc(peers));
            if (c == rank) {
                r0[m] = r[m];
                zw0[m] = zw[m];
            } else {  // later chunks of this CTA go through global scratch
                int i = c * kChunk + t + kLanes * m;
                d.ph_r[i] = r[m];
                d.ph_zw[i] = zw[m];
            }
        }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    cluster_arrive();
    cluster_wait();  // every CTA's histogram is complete
    for (int k = t; k < nb; k += blockDim.x) {
        int s = 0;
#pragma unroll
        for (int q = 0; q < kCluster; q++) s += *cluster_peer(&sh.hist[k], q);
        sh.hist_all[k] = s;
    }
    cluster_arrive();  // done reading the others' histograms; the wait is before this CTA leaves
    __syncthreads();
    hist_median(sh, sh.hist_all, nb, P);
    __syncthreads();
    if (rank == 0) {
        for (int k = t; k < nb; k += blockDim.x) d.ph_hist[256 + k] = sh.hist_all[k];  // for the trace
        if (t == 0) d.ph_hist[512] = sh.median;
    }
    float s = mad_scale(sh.median, nb);
    for (int c = rank; c < nph; c += kCluster) {
        float acc[27];
#pragma unroll
        for (int q = 0; q < 27; q++) acc[q] = 0.0f;
#pragma unroll
        for (int m = 0; m < 4; m++) {
            int i = c * kChunk + t + kLanes * m;
            float r, zw, jv[6];
            if (c == rank) {
                r = r0[m];
                zw = zw0[m];
#pragma unroll
                for (int k = 0; k < 6; k++) jv[k] = (float)sJ[k][t + kLanes * m];
            } else {
                r = d.ph_r[i];  // written by this thread above
                zw = d.ph_zw[i];
#pragma unroll
                for (int k = 0; k < 6; k++) jv[k] = ldf(J + k * P + i);
            }
            float wv = tukey_weight(r, zw, s);
            float jw[6];
#pragma unroll
            for (int k = 0; k < 6; k++) jw[k] = jv[k] * wv;
            acc27(acc, jw, r * wv);
        }
        float v = warp_terms(acc);
        if (lane < 27) fx_add_term(sh, lane, v);
    }
    cluster_wait();
    return rank < nph;
}

// L2 prefetch of [p, p + bytes) (cp.async.bulk.prefetch.L2: a 16-byte aligned
// global address and a multiple of 16 bytes; a smaller tail is left out).  A
// prefetch changes no value anywhere, it only brings lines into L2 early.
__device__ __forceinline__ void prefetch_l2(const void *p, unsigned bytes) {
    bytes &= ~15u;
    if (bytes == 0) return;
    unsigned long long g;
    asm("cvta.to.global.u64 %0, %1;\n" : "=l"(g) : "l"(p));
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(g), "r"(bytes) : "memory");
}

// Prefetches what ICP chunk c of the level reads: its reference points,
// normals and weights (contiguous streams) and the rows of the current point
// cloud that its bilinear taps read at small motion (the chunk's own rows and
// the one below).  Issued by one thread, a chunk ahead of its use.
__device__ __forceinline__ void icp_prefetch_chunk(const InstDesc &d, int level, int c, int npix) {
    int i0 = c * kChunk;
    if (c < 0 || i0 >= npix) return;
    int n = min(kChunk, npix - i0);
    prefetch_l2(d.ref_pts[level] + i0, (unsigned)n * 16u);
    prefetch_l2(d.ref_nrm[level] + i0, (unsigned)n * 16u);
    prefetch_l2(d.icp_w + i0, (unsigned)n * 4u);
    int w = d.W >> level, h = d.H >> level;
    int y0 = i0 / w, y1 = min((i0 + n - 1) / w + 1, h - 1);
    prefetch_l2(d.cur_pts[level] + (size_t)y0 * w, (unsigned)((y1 - y0 + 1) * w) * 16u);
}

// ICP chunks [c0, c1) of 1024 pixels of the level: lane t evaluates pixels
// t + 256m of each chunk (icpResidualIndexKernel2 and the reference's per-point
// Jacobian), the warp totals of each chunk go into the CTA's fixed-point sums.
__device__ void icp_chunks(const InstDesc &d, IterShared &sh, int level, int c0, int c1, int npix) {
    int t = threadIdx.x, lane = t & 31;
    for (int c = c0; c < c1; c++) {
        if (t == 0 && c + 1 < c1) icp_prefetch_chunk(d, level, c + 1, npix);
        // Phase 1: the lane's four pixels with no accumulators live; each
        // result goes to the lane's own shared slots.
#pragma unroll
        for (int g = 0; g < 2; g++) {
            // two pixels at a time: both loads in flight, then both evaluated
            float w[2];
            float4 p[2], n[2];
#pragma unroll
            for (int u = 0; u < 2; u++) icp_load(d, level, c * kChunk + t + kLanes * (2 * g + u), npix, w[u], p[u], n[u]);
#pragma unroll
            for (int u = 0; u < 2; u++) {
                int m = 2 * g + u;
                float j[6], r;
                icp_point(d, sh.T, level, w[u], p[u], n[u], j, r);
#pragma unroll
                for (int k = 0; k < 6; k++) sh.J[k][t + kLanes * m] = j[k];
                sh.R[t + kLanes * m] = r;
            }
        }
        // Phase 2: the canonical per-lane sums in point order, from the slots
        // this thread wrote (no barrier needed).
        float acc[27];
#pragma unroll
        for (int q = 0; q < 27; q++) acc[q] = 0.0f;
#pragma unroll
        for (int m = 0; m < 4; m++) {
            float j[6];
#pragma unroll
            for (int k = 0; k < 6; k++) j[k] = sh.J[k][t + kLanes * m];
            acc27(acc, j, sh.R[t + kLanes * m]);
        }
        float v = warp_terms(acc);
        if (lane < 27) fx_add_term(sh, lane, v);
    }
}

__device__ __forceinline__ int packed_index(int r, int c) {
    int a = r < c ? r : c, b = r < c ? c : r;
    return a * 6 - (a * (a - 1)) / 2 + (b - a);
}

// The end of an iteration of an instance: the accumulated terms in FP64 (reset
// for the next iteration), the system of the mode (fused in FP64 for
// BIOBJECTIVE with weights precomputed off this path, linearFuseKernel
// warp.cu:918-924), the solve and SE(3) update (warp 0), the statistics and
// the optional trace.  Every global value it reads is loaded in one round trip
// at the start (threads 54..63 fetch the scalars), since the FP64 solve that
// follows is a long serial chain.
__device__ __forceinline__ void finalize_iter(const InstDesc &d, SolveShared &sh, int level, int it, bool use_ph,
                                              bool use_icp) {
    int t = threadIdx.x;
    SolveScratch &S = sh.S;
    long long L[kFxLimbs];
    int bad = 0;
    unsigned long long *src = nullptr;
    if (t < 54) {
        int set = t / 27, q = t % 27;
        src = d.fx + set * kFxTerms + q * kFxLimbs;
#pragma unroll
        for (int k = 0; k < kFxLimbs; k++) L[k] = (long long)__ldcg(src + k);
        bad = __ldcg(d.fx_bad + set);
    } else if (t == 54) {
        sh.nsel = use_icp ? __ldcg(d.icp_nsel + level) : 0;
    } else if (t == 55) {
        sh.fuse_c2 = __ldcg(d.fuse_c2 + level);
    } else if (t == 56) {
        sh.median = use_ph ? __ldcg(d.ph_hist + 512) : -1;
    } else if (t == 57) {
        sh.st_iters = __ldcg(d.stats + ST_ITERS);
        sh.st_solves = __ldcg(d.stats + ST_SOLVES);
        sh.st_nonspd = __ldcg(d.stats + ST_NONSPD);
    } else if (t == 58) {
        sh.work0 = __ldcg(d.work + 0);
        sh.work1 = __ldcg(d.work + 1);
    } else if (t == 59) {
        sh.trace_slot = d.trace ? __ldcg(d.trace_count) : 0;
    }
    if (t < 16) sh.T[t] = __ldcg(d.T + t);
    if (t < 54) {
        double v = bad ? __longlong_as_double(0x7ff8000000000000LL) : fx_to_double(L);
        (t >= 27 ? sh.A_icp : sh.A_ph)[t % 27] = v;
#pragma unroll
        for (int k = 0; k < kFxLimbs; k++) src[k] = 0ull;
    }
    __syncthreads();
    if (t < 2) d.fx_bad[t] = 0;
    int nsel = sh.nsel;
    bool ok = !(use_icp && nsel <= 0);  // ShapeTracker "not enough points": no solve
    int slot = sh.trace_slot;
    bool tr_on = d.trace && slot < d.trace_max;
    recon_iter_trace *tr = tr_on ? d.trace + slot : nullptr;
    if (t < 42) {
        int q = (t < 36) ? packed_index(t / 6, t % 6) : 21 + (t - 36);
        double aph = sh.A_ph[q], aic = sh.A_icp[q];
        double v;
        if (d.mode == RECON_PHOTOMETRIC) v = aph;
        else if (d.mode == RECON_GEOMETRIC) v = aic;
        else v = ok ? __fma_rn(d.fuse_c1, aph, sh.fuse_c2 * aic) : aph;  // (1-lambda)/P * photo + lambda/N * icp
        if (t < 36) S.A[t] = v;
        else S.b[t - 36] = v;
        if (tr) {
            if (t < 36) {
                tr->A[t] = v;
                tr->A_ph[t] = aph;
                tr->A_icp[t] = aic;
            } else {
                tr->b[t - 36] = v;
                tr->b_ph[t - 36] = aph;
                tr->b_icp[t - 36] = aic;
            }
        }
    }
    int median = sh.median;
    if (tr) {
        for (int k = t; k < 256; k += blockDim.x)
            tr->hist[k] = (use_ph && k < d.hist_bins) ? __ldcg(d.ph_hist + 256 + k) : 0;
    }
    __syncthreads();
    if (t >= 32) return;
    int lane = t;
    int st = 0;
    float T_before = lane < 16 ? sh.T[lane] : 0.0f;
    if (ok) st = wsolve_update(S, d.solver, sh.T, (double)d.opt_out, lane);
    __syncwarp();
    if (d.settle_mm > 0.0f) {
        // settle rule (orc_pose_settled): every translation entry moved by at
        // most settle_mm and every rotation entry by at most settle_rot; the
        // instance's remaining iterations of this level are skipped
        bool small = true;
        if (lane < 12) small = fabsf(sh.T[lane] - T_before) <= ((lane & 3) == 3 ? d.settle_mm : d.settle_rot);
        if (__all_sync(0xffffffffu, small) && lane == 0) d.stats[ST_SETTLED] = level + 1;
    }
    if (lane < 16) d.T[lane] = sh.T[lane];
    if (tr && lane < 16) tr->T[lane] = sh.T[lane];
    if (lane == 0) {
        int *stt = d.stats;
        unsigned long long *wk = d.work;
        stt[ST_ITERS] = sh.st_iters + 1;
        if (ok) stt[ST_SOLVES] = sh.st_solves + 1;
        if (st != 0) stt[ST_NONSPD] = sh.st_nonspd + 1;
        if (use_ph) stt[ST_MEDIAN] = median;
        if (use_ph) wk[0] = sh.work0 + (unsigned long long)d.P;
        if (use_icp) wk[1] = sh.work1 + (unsigned long long)nsel;
        if (use_icp) stt[ST_ICPSEL0 + level] = nsel;
        if (tr) {
            tr->level = level;
            tr->iter = it;
            tr->mode = d.mode;
            tr->solved = ok ? 1 : 0;
            tr->status = st;
            tr->icp_selected = use_icp ? nsel : 0;
            tr->median_bin = median;
        }
        if (d.trace) *d.trace_count = slot + 1;
    }
}


// The linearisation of one GN iteration at `level`, iteration `it`, for every
// instance.  The grid is one row: blocks [0, 8n) are the photometric clusters
// of the n instances (cluster i = instance i; updateLinearSystem,
// phototracker.cpp:505-511), then icp_ctas blocks per instance, block j of an
// instance taking ICP chunks [j K, (j+1) K) of 1024 pixels, K = icp_per_cta
// (ShapeTracker::updateLinearSystem, shapetracker.cpp:376-381).  The
// photometric clusters, the longest dependent chains of the iteration
// (residuals, a cluster-wide histogram, then the weighted sums), come first so
// that they all start in the first wave and the short ICP CTAs fill in around
// them.  Every CTA adds its fixed-point sums to the instance's with integer
// atomics, so the result does not depend on K or on the order in which CTAs
// finish; k_solve then fuses, solves and updates the pose.
//
// Even iterations visit the instances, and the chunks within each, in reverse
// order (CTAs start roughly in block order): a level-0 pass streams several
// times L2's capacity, and the lines it touched last (or k_icp_mask touched
// last, before iteration 0) are the ones the next pass then starts with.
#ifndef RECON_ITER_MIN_BLOCKS
#define RECON_ITER_MIN_BLOCKS 4
#endif
__global__ void __cluster_dims__(kCluster, 1, 1) __launch_bounds__(kIterThreads, RECON_ITER_MIN_BLOCKS)
    k_iter(const InstDesc *D, int level, int it, int icp_per_cta, int n_inst, int icp_ctas) {
    pdl_trigger();
    const bool rev = (it & 1) == 0;
    int slot, role;  // instance slot of the block, and its role within the instance
    if ((int)blockIdx.x < kCluster * n_inst) {
        slot = blockIdx.x / kCluster;
        role = blockIdx.x % kCluster;
    } else {
        int j = blockIdx.x - kCluster * n_inst;
        if (icp_ctas <= 0) return;
        slot = j / icp_ctas;
        role = kCluster + j % icp_ctas;
        if (slot >= n_inst) return;  // rounding of the grid to whole clusters
    }
    __shared__ InstDesc sd;
    load_desc(sd, D + (rev ? n_inst - 1 - slot : slot));
    __syncthreads();
    const InstDesc &d = sd;
    if (level >= d.L) return;
    if (it >= d.iters[d.L - 1 - level]) return;
    if (role >= kCluster && threadIdx.x == 0 && d.mode != RECON_PHOTOMETRIC) {
        // the first chunk's inputs, while the previous kernel finishes
        int np = (d.W >> level) * (d.H >> level);
        int nall = ((np + kChunk - 1) / kChunk + icp_per_cta - 1) / icp_per_cta;
        int jj = role - kCluster;
        if (jj < nall) icp_prefetch_chunk(d, level, (rev ? nall - 1 - jj : jj) * icp_per_cta, np);
    }
    pdl_wait();
    // the instance left this level early (settle rule; uniform over a cluster)
    if (d.settle_mm > 0.0f && __ldcg(d.stats + ST_SETTLED) == level + 1) return;
    bool use_ph = d.mode != RECON_GEOMETRIC;
    bool use_icp = d.mode != RECON_PHOTOMETRIC;
    int nsel = use_icp ? __ldcg(d.icp_nsel + level) : 0;
    int npix = (d.W >> level) * (d.H >> level);
    int nchunks = (npix + kChunk - 1) / kChunk;
    int nicp = nsel > 0 ? (nchunks + icp_per_cta - 1) / icp_per_cta : 0;
    int set;  // which sums this CTA adds to: 0 photometric, 1 ICP
    if (role < kCluster) {
        if (!use_ph) return;
        set = 0;
    } else {
        if (role - kCluster >= nicp) return;
        set = 1;
    }
    __shared__ IterShared sh;
    if (threadIdx.x < 16) sh.T[threadIdx.x] = __ldcg(d.T + threadIdx.x);
    fx_clear(sh);
    __syncthreads();
    if (set == 0) {
        bool had = d.precision == RECON_PRECISION_MIXED ? photo_cluster<true>(d, sh, level, role)
                                                        : photo_cluster<false>(d, sh, level, role);
        if (!had) return;
    } else {
        int j = role - kCluster;
        int c0 = (rev ? nicp - 1 - j : j) * icp_per_cta;
        icp_chunks(d, sh, level, c0, min(c0 + icp_per_cta, nchunks), npix);
    }
    __syncthreads();
    fx_flush(sh, d.fx + set * kFxTerms, d.fx_bad + set);
}

// The rest of a GN iteration, one CTA per instance after k_iter: the normal
// equations from the fixed-point sums, fusion, solve and SE(3) update
// (estimateIncrement, phototracker.cpp:646-664; linearFuse,
// shapetracker.cpp:392-394).
__global__ void __launch_bounds__(kSolveThreads) k_solve(const InstDesc *D, int level, int it) {
    pdl_trigger();
    __shared__ InstDesc sd;
    load_desc(sd, D + blockIdx.x);
    __syncthreads();
    const InstDesc &d = sd;
    if (level >= d.L) return;
    if (it >= d.iters[d.L - 1 - level]) return;
    pdl_wait();
    if (d.settle_mm > 0.0f && __ldcg(d.stats + ST_SETTLED) == level + 1) return;
    bool use_ph = d.mode != RECON_GEOMETRIC;
    bool use_icp = d.mode != RECON_PHOTOMETRIC;
    __shared__ SolveShared sh;
    finalize_iter(d, sh, level, it, use_ph, use_icp);
}

// The whole ICP preparation of a small level in one launch: the level's
// correspondences (k_icp_mask's per-pixel work), their count and first
// variance sum, and the three Student-t passes (updateWeightsKernel /
// clampWeightsKernel, rgb2gray.cu:549-569): each pass weighs every
// correspondence with the variance of the previous pass; the final pass
// clamps at 1 and writes every pixel's weight (0 where the pixel is not a
// correspondence), the first two produce only their variance sums (exact int64
// sums of truncated products).  An 8-CTA cluster per instance (blockIdx.y)
// splits the pixels, every thread reading back only what it wrote, and
// exchanges the CTAs' sums through distributed shared memory, so no pass waits
// for a separate launch.  Two CTAs fit on an SM, so a batch of up to 38
// instances runs in one wave.
constexpr int kStudentThreads = 1024;

__device__ __forceinline__ void student_body(const InstDesc *D, int level) {
    __shared__ InstDesc sd;
    __shared__ float sT[16];
    __shared__ long long part[3];
    __shared__ int part_cnt;
    __shared__ long long warp_sum[kStudentThreads / 32];
    __shared__ int warp_cnt[kStudentThreads / 32];
    __shared__ long long s_var0;
    __shared__ int s_nsel;
    load_desc(sd, D + blockIdx.y);
    __syncthreads();
    const InstDesc &d = sd;
    if (level >= d.L || d.mode == RECON_PHOTOMETRIC) return;
    if (d.iters[d.L - 1 - level] <= 0) return;  // uniform over the cluster
    pdl_wait();
    int n = (d.W >> level) * (d.H >> level);
    int rank = blockIdx.x, t = threadIdx.x, lane = t & 31, wid = t >> 5;
    int stride = kIterCluster * kStudentThreads;
    int c = 0;
    long long v = 0;
    {
        if (t < 16) sT[t] = __ldcg(d.T + t);
        if (rank == 0 && t == 0) d.work[2] += (unsigned long long)n;
        __syncthreads();
        for (int i0 = rank * kStudentThreads + t; i0 < n; i0 += 2 * stride) {
            // two pixels at a time: point and normal loads in flight together
            float4 p[2], rn[2];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                int i = i0 + u * stride;
                p[u] = rn[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (i < n) {
                    p[u] = __ldg(d.ref_pts[level] + i);
                    rn[u] = __ldg(d.ref_nrm[level] + i);
                }
            }
#pragma unroll
            for (int u = 0; u < 2; u++) {
                int i = i0 + u * stride;
                if (i >= n) continue;
                float r2;
                uint8_t ok = icp_mask_pixel(d, sT, level, p[u], rn[u], r2);
                if (ok) v += trunc_prod(r2, student_w(r2, 100.0f));
                d.icp_r2[i] = r2;
                d.icp_mask[i] = ok;
                c += ok;
            }
        }
    }
    c = __reduce_add_sync(0xffffffffu, c);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) {
        warp_cnt[wid] = c;
        warp_sum[wid] = v;
    }
    __syncthreads();
    if (t == 0) {
        int cs = 0;
        long long vs = 0;
        for (int w = 0; w < kStudentThreads / 32; w++) {
            cs += warp_cnt[w];
            vs += warp_sum[w];
        }
        part[2] = vs;
        part_cnt = cs;
    }
    cluster_arrive();
    cluster_wait();  // every CTA's count and first sum are in its shared memory
    if (t == 0) {
        int cs = 0;
        long long vs = 0;
#pragma unroll
        for (int r = 0; r < kIterCluster; r++) {
            cs += *cluster_peer(&part_cnt, r);
            vs += *cluster_peer(&part[2], r);
        }
        s_nsel = cs;
        s_var0 = vs;
    }
    __syncthreads();
    int nsel = s_nsel;
    long long var = s_var0;
    if (rank == 0 && t == 0) {
        d.icp_nsel[level] = nsel;
        // ICP weight of the fused system, kept off the iteration's critical path
        d.fuse_c2[level] = (double)d.lambda / (double)nsel;
        d.icp_var[0] = (unsigned long long)var;
    }
    for (int pass = 1; pass <= 3; pass++) {
        float Sf = (float)var;
        float minVal = (float)nsel;
        float vv = (nsel <= 1024) ? Sf : (Sf < minVal ? minVal : Sf);
        float sigma2 = vv / (float)nsel;
        long long vsum = 0;
        int i = rank * kStudentThreads + t;
        float r_next = 0.0f;
        uint8_t m_next = 0;
        if (i < n) {
            r_next = __ldg(d.icp_r2 + i);
            m_next = __ldg(d.icp_mask + i);
        }
        for (; i < n; i += stride) {
            // the next pixel's loads are in flight while this one is weighed
            float r = r_next;
            uint8_t mk = m_next;
            if (i + stride < n) {
                r_next = __ldg(d.icp_r2 + i + stride);
                m_next = __ldg(d.icp_mask + i + stride);
            }
            if (pass == 3) {
                d.icp_w[i] = mk ? fminf(student_w(r, sigma2), 1.0f) : 0.0f;
            } else if (mk) {
                vsum += trunc_prod(r, student_w(r, sigma2));
            }
        }
        if (pass == 3) break;
        for (int o = 16; o > 0; o >>= 1) vsum += __shfl_xor_sync(0xffffffffu, vsum, o);
        if (lane == 0) warp_sum[wid] = vsum;
        __syncthreads();
        if (t == 0) {
            long long sum = 0;
            for (int w = 0; w < kStudentThreads / 32; w++) sum += warp_sum[w];
            part[pass - 1] = sum;
        }
        cluster_arrive();
        cluster_wait();  // every CTA's sum of this pass is in its shared memory
        long long tot = 0;
#pragma unroll
        for (int r = 0; r < kIterCluster; r++) tot += *cluster_peer(&part[pass - 1], r);
        var = tot;
        if (rank == 0 && t == 0) d.icp_var[pass] = (unsigned long long)tot;
        __syncthreads();  // warp_sum is rewritten by the next pass
    }
    // no CTA leaves while another may still read its sums
    cluster_arrive();
    cluster_wait();
}

// The coarser levels' ICP preparation, where the grid is small enough for one
// cluster per instance to evaluate it.  Two CTAs per SM (a few registers spill
// in the mask phase; measured faster than one CTA per SM at 30 instances).
__global__ void __cluster_dims__(kIterCluster, 1, 1) __launch_bounds__(kStudentThreads, 2)
    k_icp_prepare(const InstDesc *D, int level) {
    pdl_trigger();
    student_body(D, level);
}

// ------------------------------------------------------------------
// learned initialisation: network inputs and the start-pose gate
// ------------------------------------------------------------------

// Coarse network image ([60][80][2] BF16: gray, depth in metres / 4) of each
// instance's uint8 / uint16 input frame, from the input pointer table
// (gray pointers, then depth pointers); the formula of recon_initnet_coarse.
__global__ void __launch_bounds__(256) k_net_coarse(const InstDesc *D, const uint8_t *const *in_gray,
                                                     const uint16_t *const *in_depth, const __nv_bfloat16 *prev,
                                                     __nv_bfloat16 *out, __nv_bfloat16 *net_in) {
    const InstDesc &d = D[blockIdx.y];
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kNetW * kNetH) return;
    const uint8_t *g = in_gray[blockIdx.y];
    const uint16_t *dp = in_depth[blockIdx.y];
    if (!g || !dp) return;
    int W = d.W, bx = d.W / kNetW, by = d.H / kNetH;
    int ox = p % kNetW, oy = p / kNetW;
    int gs = 0, cnt = 0;
    long long ds = 0;
    for (int y = 0; y < by; y++)
        for (int x = 0; x < bx; x++) {
            long long o = (long long)(oy * by + y) * W + ox * bx + x;
            gs += __ldg(g + o);
            int dv = __ldg(dp + o);
            if (dv) {
                ds += dv;
                cnt++;
            }
        }
    float gv = (float)gs / (255.0f * (float)(bx * by));
    float dv = cnt ? ((float)ds / (float)cnt) / 4000.0f : 0.0f;
    long long q = (long long)blockIdx.y * kNetW * kNetH + p;
    __nv_bfloat16 bg = __float2bfloat16_rn(gv), bd = __float2bfloat16_rn(dv);
    out[2 * q] = bg;
    out[2 * q + 1] = bd;
    if (net_in) {  // the network input (previous gray, depth, current gray, depth)
        net_in[4 * q + 0] = prev[2 * q];
        net_in[4 * q + 1] = prev[2 * q + 1];
        net_in[4 * q + 2] = bg;
        net_in[4 * q + 3] = bd;
    }
}

// Integer start-pose cost of one point: min(trunc(|r| * 1024), 1024) of its
// photometric residual at `level`.
__device__ __forceinline__ long long gate_cost_point(const InstDesc &d, const float *T, int level, int i) {
    int P = d.P, w = d.W >> level, h = d.H >> level;
    float a = 1.0f / (float)(1 << level);
    float b = 0.5f * (a - 1.0f);
    float r, zw;
    photo_residual(d.calib, T, a, b, __ldg(d.sel_xyz + i), __ldg(d.sel_xyz + P + i), __ldg(d.sel_xyz + 2 * P + i),
                   __ldg(d.sel_I[level] + i), d.cur_gray[level], w, h, d.cur_z, d.W, d.H, r, zw);
    float u = fabsf(r) * 1024.0f;
    return (u >= 1024.0f || !(u == u)) ? 1024 : (long long)(int)u;  // 0 <= u < 1024: a 32-bit conversion
}

// The learned start pose, step 1 (one warp per instance, no pose needed, so it
// runs with the network): the network's twist x = out * scale (FP32) mapped to
// D = exp(A(x)) applied to the identity (wexpm_update, FP64, the tracker's own
// pose update), stored as the float matrix the candidate D * T is formed from.
__global__ void __launch_bounds__(32) k_gate_twist(const InstDesc *D, const float *net_out, const float *scale,
                                                   float *Dout) {
    const InstDesc &d = D[blockIdx.x];
    __shared__ float Dm[16];
    __shared__ SolveScratch S;
    int t = threadIdx.x;
    if (t < 16) Dm[t] = (t % 5 == 0) ? 1.0f : 0.0f;
    __syncwarp();
    double x[6];
    for (int k = 0; k < 6; k++) x[k] = (double)(net_out[blockIdx.x * 6 + k] * scale[k]);
    wexpm_update(S, x, Dm, (double)d.opt_out, t);
    if (t < 16) Dout[16 * blockIdx.x + t] = Dm[t];
}

// Step 2 (grid: point blocks x instances): the candidate Tc = D * T from the
// previous pose T (FP32, as the oracle forms it), the integer costs of T and of
// Tc at the coarsest level (exact integer sums, any order), and in the
// instance's last CTA to finish (an atomic ticket) the choice: Tc replaces T
// when its cost is strictly lower.  That CTA resets the costs and the ticket
// for the next frame.
__global__ void __launch_bounds__(256) k_gate(const InstDesc *D, const float *Dm_all, long long *cost,
                                              unsigned int *ticket, float *cand, int *choice) {
    __shared__ InstDesc sd;
    __shared__ float Tp[16], Tc[16];
    __shared__ long long part[2][8];
    __shared__ bool last;
    load_desc(sd, D + blockIdx.y);
    __syncthreads();
    const InstDesc &d = sd;
    int t = threadIdx.x, inst = blockIdx.y;
    if (t < 16) Tp[t] = __ldcg(d.T + t);
    __syncthreads();
    if (t < 16) {
        const float *Dm = Dm_all + 16 * inst;
        int r = t >> 2, c = t & 3;
        Tc[t] = Dm[r * 4 + 0] * Tp[0 * 4 + c] + Dm[r * 4 + 1] * Tp[1 * 4 + c] + Dm[r * 4 + 2] * Tp[2 * 4 + c] +
                Dm[r * 4 + 3] * Tp[3 * 4 + c];
    }
    __syncthreads();
    int level = d.L - 1;
    long long c0 = 0, c1 = 0;
    for (int i = blockIdx.x * blockDim.x + t; i < d.P; i += gridDim.x * blockDim.x) {
        c0 += gate_cost_point(d, Tp, level, i);
        c1 += gate_cost_point(d, Tc, level, i);
    }
    for (int o = 16; o > 0; o >>= 1) {
        c0 += __shfl_xor_sync(0xffffffffu, c0, o);
        c1 += __shfl_xor_sync(0xffffffffu, c1, o);
    }
    if ((t & 31) == 0) {
        part[0][t >> 5] = c0;
        part[1][t >> 5] = c1;
    }
    __syncthreads();
    if (t == 0) {
        long long s0 = 0, s1 = 0;
        for (int w = 0; w < 8; w++) {
            s0 += part[0][w];
            s1 += part[1][w];
        }
        atomicAdd(reinterpret_cast<unsigned long long *>(cost + 2 * inst), (unsigned long long)s0);
        atomicAdd(reinterpret_cast<unsigned long long *>(cost + 2 * inst + 1), (unsigned long long)s1);
        __threadfence();
        last = atomicAdd(ticket + inst, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // every CTA's costs are in: the choice
    __threadfence();
    long long k0 = (long long)__ldcg(reinterpret_cast<unsigned long long *>(cost + 2 * inst));
    long long k1 = (long long)__ldcg(reinterpret_cast<unsigned long long *>(cost + 2 * inst + 1));
    bool take = k1 < k0;
    if (t < 16) {
        cand[16 * inst + t] = Tc[t];
        if (take) d.T[t] = Tc[t];
    }
    if (t == 0) {
        if (choice) choice[inst] = take ? 1 : 0;
        cost[2 * inst] = 0;
        cost[2 * inst + 1] = 0;
        ticket[inst] = 0u;
    }
}

// ------------------------------------------------------------------
// procedural renderer
// ------------------------------------------------------------------

__global__ void k_render_depth(recon_scene sc, recon_camera cam, float noise_rel, uint32_t seed, uint32_t frame,
                               uint16_t *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cam.width * cam.height) return;
    out[i] = scene_depth_pixel(&sc, &cam, i % cam.width, i / cam.width, noise_rel, seed, frame);
}

__global__ void k_render_gray(recon_scene sc, recon_camera cam, uint8_t *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cam.width * cam.height) return;
    out[i] = scene_gray_pixel(&sc, &cam, i % cam.width, i / cam.width);
}

}  // namespace rt

// ====================================================================
// Allocation-free photometric iteration.
//
// Some callers cannot allocate device memory while they track: a host that
// runs the tracker inside a real-time frame loop, where a cudaMalloc can
// synchronise the device and stall the frame, or a host framework that owns
// all device memory through its own allocator and hands plug-ins only the
// buffers it created.  For them this variant of the photometric GN iteration
// keeps its scratch (per-point residuals and depth weights) in a file-scope
// device array instead of per-instance buffers from cudaMalloc.
//
// The array is a static __device__ symbol: every GPU that loads the library
// holds it until the process exits, and every call shares it and finds the
// previous call's contents there.  Calls that overlap on the GPU (different
// streams, or different host threads on the same device) race on it and must
// be serialised by the caller.  Nothing in it has to start at zero: the
// residual and weight slots for the call's points are written before they
// are read, and the partial sums live in shared memory.
// ====================================================================

namespace rt {

constexpr int kNoAllocMaxPoints = RECON_NOALLOC_MAX_POINTS;

// residual[P], depth weight[P]: 128 KB for the 16384-point maximum
static __device__ __align__(256) float g_noalloc_scratch[2 * kNoAllocMaxPoints];

__global__ void __launch_bounds__(256) k_photo_iter_noalloc(recon_photo_view v, float *scratch, float *T) {
    __shared__ IterShared sh;
    __shared__ InstDesc d;  // view of the caller's buffers in the layout photo_iteration reads
    if (threadIdx.x == 0) {
        d.W = v.depth_width;
        d.H = v.depth_height;
        d.P = v.n_points;
        d.hist_bins = v.hist_bins;
        for (int i = 0; i < RECON_CALIB_SIZE; i++) d.calib[i] = v.calib[i];
        for (int l = 0; l < kMaxLevels; l++) {
            d.cur_gray[l] = nullptr;
            d.sel_I[l] = nullptr;
            d.sel_J[l] = nullptr;
        }
        d.cur_gray[v.level] = const_cast<float *>(v.img);
        d.sel_I[v.level] = const_cast<float *>(v.intensity);
        d.sel_J[v.level] = const_cast<float *>(v.jacobian);
        d.sel_xyz = const_cast<float *>(v.xyz);
        d.cur_z = const_cast<float *>(v.depth);
        d.ph_r = scratch;
        d.ph_zw = scratch + kNoAllocMaxPoints;
    }
    if (threadIdx.x < 16) sh.T[threadIdx.x] = T[threadIdx.x];
    __syncthreads();
    photo_iteration(d, sh, v.level);
    __syncthreads();
    if (threadIdx.x >= 32) return;
    int lane = threadIdx.x;
    SolveScratch &S = sh.S;
    for (int k = lane; k < 42; k += 32) {
        int q = (k < 36) ? packed_index(k / 6, k % 6) : 21 + (k - 36);
        if (k < 36) S.A[k] = sh.A_ph[q];
        else S.b[k - 36] = sh.A_ph[q];
    }
    __syncwarp();
    wsolve_update(S, v.solver, sh.T, (double)v.opt_scale_out, lane);
    if (lane < 16) T[lane] = sh.T[lane];
}

}  // namespace rt

namespace rt {
void set_last_error(const char *msg);
}

namespace {
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {nullptr};

int noalloc_reject(const char *msg) {
    rt::set_last_error(msg);
    return RECON_ERR_INVALID_ARG;
}
}  // namespace

extern "C" int recon_photometric_iteration_noalloc(const recon_photo_view *v, float *T_dev, void *stream) {
    if (!v || !T_dev || !v->xyz || !v->intensity || !v->jacobian || !v->img || !v->depth)
        return noalloc_reject("recon_photometric_iteration_noalloc: null pointer");
    if (v->n_points <= 0 || v->n_points % rt::kChunk)
        return noalloc_reject("recon_photometric_iteration_noalloc: n_points must be a positive multiple of 1024");
    if (v->n_points > rt::kNoAllocMaxPoints)
        return noalloc_reject("recon_photometric_iteration_noalloc: n_points exceeds RECON_NOALLOC_MAX_POINTS "
                              "(16384), the size of the built-in scratch array");
    if (v->level < 0 || v->level >= rt::kMaxLevels || v->hist_bins < 2 || v->hist_bins > 256)
        return noalloc_reject("recon_photometric_iteration_noalloc: level must be 0..3 and hist_bins 2..256");
    if (v->img_width < 2 || v->img_height < 2 || v->img_width != (v->depth_width >> v->level) ||
        v->img_height != (v->depth_height >> v->level))
        return noalloc_reject("recon_photometric_iteration_noalloc: img must be the depth size >> level");
    if (v->solver < 0 || v->solver > 1) return noalloc_reject("recon_photometric_iteration_noalloc: bad solver");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        rt::set_last_error("recon_photometric_iteration_noalloc: no current CUDA device");
        return RECON_ERR_CUDA;
    }
    void *ptr = nullptr;
    {
        // set-up, once per device with that device current: the host-side name
        // of a __device__ array is not a device address, so look it up
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            cudaError_t e = cudaGetSymbolAddress(&g_noalloc_ptr[dev], rt::g_noalloc_scratch);
            if (e != cudaSuccess) {
                g_noalloc_ptr[dev] = nullptr;
                rt::set_last_error("recon_photometric_iteration_noalloc: cudaGetSymbolAddress failed");
                return RECON_ERR_CUDA;
            }
        }
        ptr = g_noalloc_ptr[dev];
    }
    // the launch status comes from the launch call itself, so an error the
    // caller's own earlier work left pending is neither cleared nor taken for ours
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(1);
    cfg.blockDim = dim3(rt::kLanes);
    cfg.stream = (cudaStream_t)stream;
    cudaError_t e = cudaLaunchKernelEx(&cfg, rt::k_photo_iter_noalloc, *v, (float *)ptr, T_dev);
    if (e != cudaSuccess) {
        rt::set_last_error("recon_photometric_iteration_noalloc: kernel launch failed");
        return RECON_ERR_CUDA;
    }
    return RECON_OK;
}
