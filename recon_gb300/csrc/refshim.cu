// refshim.cu -- the reference tracker's kernel-level launchers
// (tracker/kernels/cuda_funcs.h:36-111) re-implemented for sm_103a on the
// reference's data layouts (include/recon_ref_shim.h).  The per-element math
// is the same as the fused product kernels (track_math.cuh, solve.cuh) and is
// compiled with -fmad=false, so every output equals the reference semantics
// bit for bit; the 27-term reductions use the library's canonical order.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/recon_ref_shim.h"
#include "solve.cuh"
#include "track_kernels.cuh"
#include "track_math.cuh"

namespace rs {
using namespace rt;

constexpr int kMaxBins = 1024;
constexpr int kMaxChunks = 4096;  // 4M points per reduction

// module-static scratch, process global like the reference's
// initHistogram64 / initCudaDotProduct buffers (histogram64.cu:96-113, warp.cu:1412-1427)
__device__ int g_hist[kMaxBins];
__device__ int g_seg[3076];
__device__ double g_part[kMaxChunks * 27];
__device__ int g_blk[kMaxChunks];
__device__ unsigned long long g_var[4];

thread_local int t_status = 0;

__global__ void k_downsample(const float *hi, int wlo, int hlo, float *lo) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= wlo * hlo) return;
    int x = i % wlo, y = i / wlo, w2 = 2 * wlo;
    int h0 = 2 * x + 2 * y * w2;
    lo[i] = (hi[h0] + hi[h0 + 1] + hi[h0 + w2] + hi[h0 + w2 + 1]) / 4.0f;
}

__global__ void k_zmap_xyz(const float *zp, float *out, int *mask, const float *calib, int W, int H, int six) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * H) return;
    int xi = i % W, yi = i / W;
    float minDist = calib[RC_MIND], maxDist = calib[RC_MAXD];
    float fx = calib[RC_KL], fy = calib[RC_KL + 4], cx = calib[RC_KL + 2], cy = calib[RC_KL + 5];
    float z = zp[i];
    bool ok = (z < -minDist && z > -maxDist);
    float x = 0, y = 0, zz = 0;
    if (ok) {
        x = ((float)xi - cx) * z / fx;
        y = ((float)yi - cy) * z / fy;
        zz = z;
    }
    if (six) {
        out[i * 6 + 0] = x;
        out[i * 6 + 1] = y;
        out[i * 6 + 2] = zz;
        mask[i] = ok ? 1 : 0;
    } else {
        out[i * 4 + 0] = x;
        out[i * 4 + 1] = y;
        out[i * 4 + 2] = zz;
        out[i * 4 + 3] = ok ? 1.0f : 0.0f;
    }
}

// xyz2CloudKernel, d2z.cu:235-331
__global__ void k_xyz2cloud(const float4 *xyzw, int W, int H, const float *calib, const float *img, float *vdata,
                            int stride) {
    int offset = blockIdx.x * blockDim.x + threadIdx.x;
    if (offset >= W * H) return;
    float *v = vdata + (size_t)offset * stride;
    float4 pt = xyzw[offset];
    if (pt.z < 0) {
        float rx, ry, rz;
        mul4(calib + RC_TLR, pt.x, pt.y, pt.z, rx, ry, rz);
        float px, py;
        distort(rx / rz, ry / rz, calib + RC_KCR, calib + RC_KR, px, py);
        if (in_bounds10(px, py, W, H)) {
            int xdi = ftoi(px), ydi = ftoi(py);
            float fx = px - xdi, fy = py - ydi;
            float color1 = bilin(xdi, ydi, fx, fy, W, img);
            float colorN = bilin(ftoi(px), ftoi(py - 1.0f), fx, fy, W, img);
            float colorE = bilin(ftoi(px + 1.0f), ftoi(py), fx, fy, W, img);
            float colorW = bilin(ftoi(px - 1.0f), ftoi(py), fx, fy, W, img);
            float colorS = bilin(ftoi(px), ftoi(py + 1.0f), fx, fy, W, img);
            float gradX1 = (colorE - colorW) / 2.0f;
            float gradY1 = (colorS - colorN) / 2.0f;
            v[0] = pt.x; v[1] = pt.y; v[2] = pt.z;
            v[3] = v[4] = v[5] = 0.0f;
            v[6] = px; v[7] = py;
            v[8] = v[9] = v[10] = 0.0f;
            v[11] = gradX1;
            v[12] = gradY1;
            float gm = fabsf(gradY1) + fabsf(gradX1);
            v[13] = gm < 1.0f ? gm : 1.0f;
            v[14] = color1;
            return;
        }
    }
    for (int k = 0; k < stride; k++) v[k] = 0.0f;
    v[2] = -calib[RC_MAXD];
}

__global__ void k_extract(const float *vdata, int stride, int n, float *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = vdata[(size_t)i * stride + 13];
}

// gpuHista's bin formula (gpu_hist.cu:136), exact integer counts
__global__ void k_hist(const float *src, int n, int bins) {
    __shared__ int sh[kMaxBins];
    for (int k = threadIdx.x; k < bins; k += blockDim.x) sh[k] = 0;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned int bin = (unsigned int)(src[i] * (bins - 1) + 0.5f);
        if (bin < (unsigned)bins) atomicAdd(&sh[bin], 1);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < bins; k += blockDim.x)
        if (sh[k]) atomicAdd(&g_hist[k], sh[k]);
}

__global__ void k_hist_out(float *hist, int bins) {
    for (int k = threadIdx.x; k < bins; k += blockDim.x) hist[k] = (float)g_hist[k];
}

__global__ void k_zero_hist() {
    for (int k = threadIdx.x; k < kMaxBins; k += blockDim.x) g_hist[k] = 0;
}

// seekThreshold256Kernel2 + segment counts of filterIndexKernel4 (filterIndex256.cu:26-46, 110-133)
__global__ void k_seg_count(const float *grad, const float *histf, int n, int nbins, int P) {
    __shared__ unsigned int s_thr;
    if (threadIdx.x == 0) {
        unsigned int thr = 0;
        int sel = 0;
        for (int k = nbins - 1; k >= 0; k--) {
            sel += (unsigned int)histf[k];
            if (sel > P) { thr = (unsigned)k; break; }
        }
        s_thr = thr;
        if (blockIdx.x == 0) {
            g_seg[3072] = (int)thr;
            g_seg[3073] = sel - P;
        }
    }
    __syncthreads();
    int ppt = n / kSegments;
    int warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (warp >= kSegments) return;
    int cnt = 0, mcnt = 0;
    for (int base = warp * ppt; base < warp * ppt + ppt; base += 32) {
        int i = base + lane;
        bool in = i < warp * ppt + ppt;
        unsigned int q = in ? (unsigned int)(grad[i] * (nbins - 1) + 0.5f) : 0u;
        cnt += __popc(__ballot_sync(0xffffffffu, in && q > s_thr));
        mcnt += __popc(__ballot_sync(0xffffffffu, in && q == s_thr));
    }
    if (lane == 0) {
        g_seg[warp] = cnt;
        g_seg[512 + warp] = mcnt;
    }
}

__global__ void k_seg_scan() {
    int *cnt = g_seg, *mcnt = g_seg + 512, *start = g_seg + 1024, *mstart = g_seg + 1536, *kept = g_seg + 2048;
    int tooMuch = g_seg[3073];
    start[0] = 0;
    for (int i = 1; i < kSegments; i++) start[i] = start[i - 1] + cnt[i - 1];
    for (int i = 0; i < kSegments; i++) kept[i] = mcnt[i];
    mstart[0] = start[kSegments - 1] + cnt[kSegments - 1];
    for (int i = 1; i < kSegments; i++) {
        if (tooMuch > 0 && kept[i - 1] > 0) {
            kept[i - 1] -= tooMuch;
            if (kept[i - 1] < 0) {
                tooMuch += kept[i - 1];
                kept[i - 1] = 0;
            } else {
                tooMuch = 0;
            }
        }
        mstart[i] = mstart[i - 1] + kept[i - 1];
    }
}

__global__ void k_seg_scatter(const float *grad, int n, int nbins, int P, int *idx_out) {
    int ppt = n / kSegments;
    int warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (warp >= kSegments) return;
    unsigned int thr = (unsigned int)g_seg[3072];
    int pos_a = g_seg[1024 + warp], pos_m = g_seg[1536 + warp], kept = g_seg[2048 + warp], m = 0;
    unsigned int lower = (1u << lane) - 1u;
    for (int base = warp * ppt; base < warp * ppt + ppt; base += 32) {
        int i = base + lane;
        bool in = i < warp * ppt + ppt;
        unsigned int q = in ? (unsigned int)(grad[i] * (nbins - 1) + 0.5f) : 0u;
        bool ia = in && q > thr, im = in && q == thr;
        unsigned int ab = __ballot_sync(0xffffffffu, ia), me = __ballot_sync(0xffffffffu, im);
        if (ia) {
            int pos = pos_a + __popc(ab & lower);
            if (pos < P) idx_out[pos] = i;
        }
        if (im) {
            int r = m + __popc(me & lower);
            if (r < kept && pos_m + r < P) idx_out[pos_m + r] = i;
        }
        pos_a += __popc(ab);
        m += __popc(me);
    }
}

__global__ void k_fill(int *p, int n, int v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

// addVertexAttributesWithoutNormalsKernel3/4, d2z.cu:700-936 (taps clamped into the image)
__global__ void k_attr(const int *idx, int P, float *vdata, int stride, int W, int H, const float *calib,
                       const float *g1, const float *g2, const float *g3, int L) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P) return;
    float *v = vdata + (size_t)idx[k] * stride;
    float rx, ry, rz;
    mul4(calib + RC_TLR, v[0], v[1], v[2], rx, ry, rz);
    float col[4] = {0, 0, 0, 0}, gx[4] = {0, 0, 0, 0}, gy[4] = {0, 0, 0, 0};
    float px, py;
    distort(rx / rz, ry / rz, calib + RC_KCR, calib + RC_KR, px, py);
    const float *g[4] = {nullptr, g1, g2, g3};
    if (in_bounds10(px, py, W, H)) {
        float a = 0.5f, b = -0.25f, lx = px, ly = py;
        for (int l = 1; l < L; l++) {
            lx = a * lx + b;
            ly = a * ly + b;
            int wl = W >> l, hl = H >> l;
            int xdi = ftoi(lx), ydi = ftoi(ly);
            float fX = lx - xdi, fY = ly - ydi;
            col[l] = bilin_clamped(xdi, ydi, fX, fY, wl, hl, g[l]);
            float cN = bilin_clamped(xdi, ydi - 1, fX, fY, wl, hl, g[l]);
            float cW = bilin_clamped(xdi - 1, ydi, fX, fY, wl, hl, g[l]);
            float cE = bilin_clamped(xdi + 1, ydi, fX, fY, wl, hl, g[l]);
            float cS = bilin_clamped(xdi, ydi + 1, fX, fY, wl, hl, g[l]);
            gx[l] = (cE - cW) / 2.0f;
            gy[l] = (cS - cN) / 2.0f;
        }
    }
    for (int l = 1; l < L && l < 4; l++) {
        v[15 + 3 * (l - 1)] = gx[l];
        v[16 + 3 * (l - 1)] = gy[l];
        v[17 + 3 * (l - 1)] = col[l];
    }
}

// precomputeJacobian4Kernel, warp.cu:502-645
__global__ void k_jac(const int *idx, int P, const float *vdata, int stride, const float *calib, float *J1, float *J2,
                      float *J3, float *J4, float optScaleIn) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P) return;
    const float *v = vdata + (size_t)idx[k] * stride;
    const float *T = calib + RC_TLR, *K = calib + RC_KR, *kc = calib + RC_KCR;
    float rx, ry, rz;
    mul4(T, v[0], v[1], v[2], rx, ry, rz);
    rx *= optScaleIn;
    ry *= optScaleIn;
    rz *= optScaleIn;
    float dN0 = 1.0f / rz, dN1 = 0, dN2 = -rx / (rz * rz), dN3 = 0, dN4 = 1.0f / rz, dN5 = -ry / (rz * rz);
    float x = rx / rz, y = ry / rz, x2 = x * x, y2 = y * y, x4 = x2 * x2, y4 = y2 * y2, r2 = x2 + y2, r4 = r2 * r2;
    float dD0 = 1 + kc[0] * (3 * x2 + y2) + kc[1] * (5 * x4 + 6 * x2 * y2 + y4) + kc[4] * r4 * (7 * x2 + y2);
    float dD1 = kc[0] * 2 * x * y + kc[1] * 4 * x * y * r2 + kc[4] * 6 * x * y * r4;
    float dD2 = kc[0] * 2 * y * x + kc[1] * 4 * x * y * r2 + kc[4] * 6 * x * y * r4;
    float dD3 = 1 + kc[0] * (3 * x2 + y2) + kc[1] * (5 * x4 + 6 * x2 * y2 + y4) + kc[4] * r4 * (7 * y2 + x2);
    const float dps[6][3] = {{0.0f, -rz, ry}, {rz, 0.0f, -rx}, {-ry, rx, 0.0f},
                             {1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}};
    float *J[4] = {J1, J2, J3, J4};
    const int gs[4][2] = {{11, 12}, {15, 16}, {18, 19}, {21, 22}};
    for (int c = 0; c < 6; c++) {
        float drx, dry, drz, px, py, pz;
        rot4(T, dps[c][0], dps[c][1], dps[c][2], drx, dry, drz);
        float dpnx = dN0 * drx + dN1 * dry + dN2 * drz;
        float dpny = dN3 * drx + dN4 * dry + dN5 * drz;
        mul3(K, dD0 * dpnx + dD1 * dpny, dD2 * dpnx + dD3 * dpny, 0.0f, px, py, pz);
        for (int l = 0; l < 4; l++) {
            if (!J[l]) continue;
            float gxl = v[gs[l][0]], gyl = v[gs[l][1]];
            float val;
            if (l == 0) val = px * gxl + py * gyl;
            else {
                float s = (l == 1) ? 2.0f : (l == 2 ? 4.0f : 8.0f);
                val = (px / s) * gxl + (py / s) * gyl;
            }
            J[l][c * P + k] = val;
        }
    }
}

// interpolateResidualKernel2, warp.cu:269-332
__global__ void k_interp(const int *idx, int P, const float *vdata, int stride, const float *T, const float *calib,
                         float a, float b, int colorOffset, const float *img, int w, int h, const float *zcur, int zw,
                         int zh, float *residual, float *zweight) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P) return;
    const float *v = vdata + (size_t)idx[k] * stride;
    float r, z;
    photo_residual(calib, T, a, b, v[0], v[1], v[2], v[colorOffset], img, w, h, zcur, zw, zh, r, z);
    residual[k] = r;
    zweight[k] = z;
}

// histogram64.cu:41-157: 64-bin histogram of (int)(63|r|), median, Tukey weights
__global__ void k_w64_hist(const float *r, int n) {
    __shared__ int sh[64];
    if (threadIdx.x < 64) sh[threadIdx.x] = 0;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&sh[mad_bin(r[i], 64)], 1);
    __syncthreads();
    if (threadIdx.x < 64 && sh[threadIdx.x]) atomicAdd(&g_hist[threadIdx.x], sh[threadIdx.x]);
}

__global__ void k_w64_apply(const float *r, int n, float *w, const float *ext, float *wr) {
    __shared__ int s_med;
    if (threadIdx.x == 0) {
        int half = n / 2, acc = 0, m = 0;
        for (int k = 0; k < 64; k++) {
            acc += g_hist[k];
            if (acc > half) { m = k; break; }
        }
        s_med = m;
    }
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = mad_scale(s_med, 64);
    float wi = tukey_weight(r[i], ext[i], s);
    wr[i] = r[i] * wi;
    w[i] = wi;
}

__global__ void k_weight_jac(const float *J, const float *w, int n, float *Jw) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float wi = w[i];
    for (int c = 0; c < 6; c++) Jw[c * n + i] = J[c * n + i] * wi;
}

// canonical 27-term reduction: one CTA per 1024-point chunk
__global__ void __launch_bounds__(256) k_reduce27(const float *J, const float *r, int n) {
    __shared__ double wpart[8][27];
    int c = blockIdx.x, t = threadIdx.x, lane = t & 31, wid = t >> 5;
    float acc[27];
#pragma unroll
    for (int q = 0; q < 27; q++) acc[q] = 0.0f;
    for (int m = 0; m < 4; m++) {
        int i = c * kChunk + t + kLanes * m;
        float j[6];
        for (int k = 0; k < 6; k++) j[k] = J[k * n + i];
        float rv = r ? r[i] : 0.0f;
        int q = 0;
        for (int aa = 0; aa < 6; aa++)
            for (int cc = aa; cc < 6; cc++, q++) acc[q] = __fmaf_rn(j[aa], j[cc], acc[q]);
        for (int cc = 0; cc < 6; cc++, q++) acc[q] = __fmaf_rn(j[cc], rv, acc[q]);
    }
    for (int q = 0; q < 27; q++) {
        float v = acc[q];
        for (int o = 16; o > 0; o >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) wpart[wid][q] = (double)v;
    }
    __syncthreads();
    if (t < 27) {
        double s = 0.0;
        for (int w = 0; w < 8; w++) s = s + wpart[w][t];
        g_part[(size_t)c * 27 + t] = s;
    }
}

__global__ void k_reduce_out(int nchunks, float *jtj, float *jtr) {
    __shared__ double tot[27];
    int q = threadIdx.x;
    if (q < 27) {
        double s = 0.0;
        for (int c = 0; c < nchunks; c++) s = s + g_part[(size_t)c * 27 + q];
        tot[q] = s;
    }
    __syncthreads();
    if (q == 0) {
        int k = 0;
        for (int j = 0; j < 6; j++)
            for (int i = j; i < 6; i++) {
                if (jtj) {
                    jtj[i + j * 6] = (float)tot[k];
                    jtj[i * 6 + j] = (float)tot[k];
                }
                k++;
            }
        if (jtr)
            for (int c = 0; c < 6; c++) jtr[c] = (float)tot[21 + c];
    }
}

// linearFuseKernel, warp.cu:918-924
__global__ void k_fuse(float *A1, float *b1, float w1, float iN1, const float *A2, const float *b2, float w2,
                       float iN2) {
    int idx = threadIdx.x;
    if (idx < 6) b1[idx] = iN1 * w1 * b1[idx] + iN2 * w2 * b2[idx];
    if (idx < 36) A1[idx] = iN1 * w1 * A1[idx] + iN2 * w2 * A2[idx];
}

// conjugateGradientKernel + expmKernel, warp.cu:926-975, expmCuda.cu:1989-2048
__global__ void k_solve_motion(const float *JtJ, const float *b, float *TDev, float scaleOut) {
    __shared__ SolveScratch S;
    __shared__ float T[16];
    int lane = threadIdx.x;
    for (int i = lane; i < 36; i += 32) S.A[i] = (double)JtJ[i];
    if (lane < 6) S.b[lane] = (double)b[lane];
    if (lane < 16) T[lane] = TDev[lane];
    __syncwarp();
    wsolve_update(S, 1, T, (double)scaleOut, lane);
    if (lane < 16) TDev[lane] = T[lane];
}

// genPointsCloud6Kernel, d2z.cu:436-469
__global__ void k_gencloud6(const float *zp, int W, int H, const float *calib, float *pts, int *mask) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * H) return;
    int xi = i % W, yi = i / W;
    float fx = calib[RC_KL], fy = calib[RC_KL + 4], cx = calib[RC_KL + 2], cy = calib[RC_KL + 5];
    float z = zp[i];
    float *p = pts + (size_t)i * 6;
    if (z < 0) {
        p[0] = ((float)xi - cx) * z / fx;
        p[1] = ((float)yi - cy) * z / fy;
        p[2] = z;
        p[3] = 0;
        p[4] = 0;
        p[5] = 1.0f;
        mask[i] = 1;
    } else {
        for (int k = 0; k < 6; k++) p[k] = 0;
        mask[i] = 0;
    }
}

// computeNormalsCudaKernel, d2z.cu:503-537
__global__ void k_normals6(float *pts, int *mask, int W, int H) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * H) return;
    int xi = i % W, yi = i / W;
    float *me = pts + (size_t)i * 6;
    if (xi < 1 || yi < 1 || xi > W - 2 || yi > H - 2) {
        me[3] = me[4] = me[5] = 0;
        mask[i] = 0;
        return;
    }
    const float *x1 = pts + (size_t)(i - 1) * 6, *x2 = pts + (size_t)(i + 1) * 6;
    const float *y1 = pts + (size_t)(i - W) * 6, *y2 = pts + (size_t)(i + W) * 6;
    if (x1[2] < 0 && x2[2] < 0 && y1[2] < 0 && y2[2] < 0) {
        float ux = x2[0] - x1[0], uy = x2[1] - x1[1], uz = x2[2] - x1[2];
        float vx = y2[0] - y1[0], vy = y2[1] - y1[1], vz = y2[2] - y1[2];
        float nx = uy * vz - uz * vy, ny = -(ux * vz - uz * vx), nz = ux * vy - uy * vx;
        normalize3(nx, ny, nz);
        me[3] = nx;
        me[4] = ny;
        me[5] = nz;
        return;
    }
    me[3] = me[4] = me[5] = 0;
    mask[i] = 0;
}

// downSampleCloud6Kernel, d2z.cu:557-588
__global__ void k_ds6(const float *src, const int *msrc, float *dst, int *mdst, int wlo, int hlo) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= wlo * hlo) return;
    int xi = i % wlo, yi = i / wlo;
    int h0 = xi * 2 + yi * 2 * (wlo * 2);
    int offs[4] = {h0, h0 + 1, h0 + wlo * 2, h0 + wlo * 2 + 1};
    float pd[6] = {0, 0, 0, 0, 0, 0};
    float ns = 0.0f;
    for (int k = 0; k < 4; k++)
        if (msrc[offs[k]]) {
            ns++;
            for (int c = 0; c < 6; c++) pd[c] += src[(size_t)offs[k] * 6 + c];
        }
    if (ns > 0.0f) {
        for (int c = 0; c < 6; c++) pd[c] /= ns;
        normalize3(pd[3], pd[4], pd[5]);
        mdst[i] = 1;
    } else {
        mdst[i] = 0;
    }
    for (int c = 0; c < 6; c++) dst[(size_t)i * 6 + c] = pd[c];
}

__device__ __forceinline__ void bilin6(const float *s, float fx, float fy, int pitch, float &px, float &py,
                                       float &pz) {
    float o[3];
    for (int c = 0; c < 3; c++) {
        float v0 = s[c], v1 = s[c + 6], v2 = s[c + pitch], v3 = s[c + pitch + 6];
        o[c] = (1 - fx) * (1 - fy) * v0 + fx * (1 - fy) * v1 + (1 - fx) * fy * v2 + fx * fy * v3;
    }
    px = o[0];
    py = o[1];
    pz = o[2];
}

// icpResidualKernel2, rgb2gray.cu:223-260
__global__ void k_icpmask(const float *ref6, const int *refmask, int w, int h, const float *T, const float *calib,
                          const float *cur6, const int *curmask, float a, float b, float *residual, int *rmask) {
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= w * h) return;
    if (refmask[o] == 0) {
        rmask[o] = 0;
        return;
    }
    const float *K = calib + RC_KL, *p = ref6 + (size_t)o * 6;
    float qx, qy, qz, nx, ny, nz;
    mul4(T, p[0], p[1], p[2], qx, qy, qz);
    rot4(T, p[3], p[4], p[5], nx, ny, nz);
    float q2x = qx / qz, q2y = qy / qz;
    float p2x = a * (K[0] * q2x + K[2]) + b, p2y = a * (K[4] * q2y + K[5]) + b;
    if (p2x >= 0 && p2x < (w - 1) && p2y >= 0 && p2y < (h - 1)) {
        int xdi = ftoi(p2x), ydi = ftoi(p2y), off2 = xdi + ydi * w;
        if (curmask[off2] && curmask[off2 + 1] && curmask[off2 + w] && curmask[off2 + w + 1]) {
            float cx, cy, cz;
            bilin6(cur6 + (size_t)off2 * 6, p2x - xdi, p2y - ydi, w * 6, cx, cy, cz);
            residual[o] = (cx - qx) * nx + (cy - qy) * ny + (cz - qz) * nz;
            rmask[o] = 1;
            return;
        }
    }
    rmask[o] = 0;
}

__global__ void k_blkcount(const int *mask, int n) {
    __shared__ int s;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int f = (i < n && mask[i] > 0) ? 1 : 0;
    int c = __reduce_add_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0) atomicAdd(&s, c);
    __syncthreads();
    if (threadIdx.x == 0) g_blk[blockIdx.x] = s;
}

// selectValidIndex's stable compaction (rgb2gray.cu:395-460), 1024 pixels per block
__global__ void k_compact(const int *mask, int n, int nblk, int *select, int *total) {
    __shared__ int s_base, s_warp[32];
    if (threadIdx.x < 32) {
        int pre = 0, tot = 0;
        for (int k = threadIdx.x; k < nblk; k += 32) {
            tot += g_blk[k];
            if (k < (int)blockIdx.x) pre += g_blk[k];
        }
        pre = __reduce_add_sync(0xffffffffu, pre);
        tot = __reduce_add_sync(0xffffffffu, tot);
        if (threadIdx.x == 0) {
            s_base = pre;
            if (blockIdx.x == 0) *total = tot;
        }
    }
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int f = (i < n && mask[i] > 0) ? 1 : 0;
    unsigned int bal = __ballot_sync(0xffffffffu, f);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) s_warp[wid] = __popc(bal);
    __syncthreads();
    int wbase = 0;
    for (int k = 0; k < wid; k++) wbase += s_warp[k];
    if (f) select[s_base + wbase + __popc(bal & ((1u << lane) - 1u))] = i;
}

__global__ void k_pack(const int *sel, int n, const float *full, float *r, float *r2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v = full[sel[i]];
    r[i] = v;
    r2[i] = v * v;
}

__device__ __forceinline__ long long trunc_prod2(float r2, float w) {
    float prod = r2 * w;
    return (prod >= 0.0f && prod < 9.0e18f) ? (long long)prod : (prod >= 9.0e18f ? 9000000000000000000LL : 0);
}

// generateStudentTWeights, rgb2gray.cu:470-569, 854-877 (exact int64 sum of the truncated terms)
__global__ void k_student(const float *r2, int n, float *w, int pass) {
    __shared__ long long s_acc;
    if (threadIdx.x == 0) s_acc = 0;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    long long v = 0;
    if (i < n) {
        float wv;
        if (pass == 0) {
            wv = 6 / (5 + r2[i] / 100.0f);
        } else {
            float Sf = (float)(long long)g_var[pass - 1];
            float minVal = (float)n;
            float var = (n <= 1024) ? Sf : (Sf < minVal ? minVal : Sf);
            wv = 6 / (5 + r2[i] / (var / (float)n));
        }
        if (pass == 3) wv = fminf(wv, 1.0f);
        else v = trunc_prod2(r2[i], wv);
        w[i] = wv;
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd((unsigned long long *)&s_acc, (unsigned long long)v);
    __syncthreads();
    if (threadIdx.x == 0 && pass < 3 && s_acc) atomicAdd(&g_var[pass], (unsigned long long)s_acc);
}

__global__ void k_zero_var() {
    if (threadIdx.x < 4) g_var[threadIdx.x] = 0ull;
}

// icpResidualIndexKernel2, rgb2gray.cu:323-390
__global__ void k_icpres(const float *ref6, const int *select, int nsel, int w, int h, const float *T,
                         const float *calib, const float *cur6, const int *curmask, float a, float b, int npadded,
                         float *res, float *J, const float *weights, float optScaleIn) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nsel) return;
    const float *K = calib + RC_KL, *p = ref6 + (size_t)select[idx] * 6;
    float qx, qy, qz, cnx, cny, cnz;
    mul4(T, p[0], p[1], p[2], qx, qy, qz);
    rot4(T, p[3], p[4], p[5], cnx, cny, cnz);
    float q2x = qx / qz, q2y = qy / qz;
    float p2x = a * (K[0] * q2x + K[2]) + b, p2y = a * (K[4] * q2y + K[5]) + b;
    if (p2x >= 0 && p2x < (w - 1) && p2y >= 0 && p2y < (h - 1)) {
        float weight = weights[idx];
        int xdi = ftoi(p2x), ydi = ftoi(p2y), off2 = xdi + ydi * w;
        float cx, cy, cz;
        bilin6(cur6 + (size_t)off2 * 6, p2x - xdi, p2y - ydi, w * 6, cx, cy, cz);
        if (curmask[off2] && weight > 0.0f && fabsf(cz - qz) < 300.0f) {
            float rvx = cx - qx, rvy = cy - qy, rvz = cz - qz;
            res[idx] = optScaleIn * weight * (rvx * cnx + rvy * cny + rvz * cnz);
            const float dP[3][3] = {{0, -p[2], p[1]}, {p[2], 0, -p[0]}, {-p[1], p[0], 0}};
            const float dNv[3][3] = {{0, -p[5], p[4]}, {p[5], 0, -p[3]}, {-p[4], p[3], 0}};
            for (int c = 0; c < 3; c++) {
                float bx, by, bz, nx, ny, nz;
                rot4(T, dP[c][0], dP[c][1], dP[c][2], bx, by, bz);
                rot4(T, dNv[c][0], dNv[c][1], dNv[c][2], nx, ny, nz);
                J[idx + npadded * c] =
                    -optScaleIn * weight * (-cnx * bx - cny * by - cnz * bz + rvx * nx + rvy * ny + rvz * nz);
            }
            for (int c = 0; c < 3; c++) {
                float bx, by, bz;
                rot4(T, c == 0 ? 1.0f : 0.0f, c == 1 ? 1.0f : 0.0f, c == 2 ? 1.0f : 0.0f, bx, by, bz);
                J[idx + npadded * (3 + c)] = -weight * (-cnx * bx - cny * by - cnz * bz);
            }
            return;
        }
    }
    res[idx] = 0.0f;
    for (int c = 0; c < 6; c++) J[idx + npadded * c] = 0.0f;
}

inline unsigned g1d(int n, int b = 256) { return (unsigned)((n + b - 1) / b); }

bool launched(int code_if_bad) {
    cudaError_t e = cudaGetLastError();
    t_status = (e == cudaSuccess) ? code_if_bad : RECON_ERR_CUDA;
    return e == cudaSuccess;
}

}  // namespace rs

using namespace rs;

extern "C" {

int recon_last_status(void) { return t_status; }

#define SHIM_BEGIN() (void)cudaGetLastError()
#define BAD() \
    do {      \
        t_status = RECON_ERR_INVALID_ARG; \
        return; \
    } while (0)

void downSample2Pyramid(recon_pyramid *p, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!p || p->nLayers < 1 || p->nLayers > RECON_MAX_LEVELS) BAD();
    for (int l = 1; l < p->nLayers; l++) {
        if (!p->devPtr[l - 1] || !p->devPtr[l] || p->width[l] * 2 != p->width[l - 1]) BAD();
        int n = p->width[l] * p->height[l];
        k_downsample<<<g1d(n), 256, 0, stream>>>(p->devPtr[l - 1], p->width[l], p->height[l], p->devPtr[l]);
    }
    launched(RECON_OK);
}

void convertZmapToXYZCuda(float *z, float *pts, float *calib, int width, int height, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!z || !pts || !calib || width < 1 || height < 1) BAD();
    k_zmap_xyz<<<g1d(width * height), 256, 0, stream>>>(z, pts, nullptr, calib, width, height, 0);
    launched(RECON_OK);
}

void convertZmapToXYZ6Cuda(float *z, float *pts, int *mask, float *calib, int width, int height,
                           recon_stream_t stream) {
    SHIM_BEGIN();
    if (!z || !pts || !mask || !calib || width < 1 || height < 1) BAD();
    k_zmap_xyz<<<g1d(width * height), 256, 0, stream>>>(z, pts, mask, calib, width, height, 1);
    launched(RECON_OK);
}

void xyz2CloudCuda(float *xyz, float *calib, recon_vbuffer *vb, recon_pyramid *gp, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!xyz || !calib || !vb || !vb->devPtr || !gp || !gp->devPtr[0] || vb->stride < 24) BAD();
    int W = gp->width[0], H = gp->height[0];
    vb->vertexCount = W * H;
    k_xyz2cloud<<<g1d(W * H), 256, 0, stream>>>((const float4 *)xyz, W, H, calib, gp->devPtr[0], vb->devPtr,
                                                vb->stride);
    launched(RECON_OK);
}

void extractGradientMagnitudes(recon_vbuffer *vb, float *out, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!vb || !vb->devPtr || !out || vb->stride != 24 || vb->vertexCount % 1024) BAD();
    k_extract<<<g1d(vb->vertexCount), 256, 0, stream>>>(vb->devPtr, vb->stride, vb->vertexCount, out);
    launched(RECON_OK);
}

double cudaHista(float *src, float *hist, int length, int bins, float *d_hist, recon_stream_t stream) {
    (void)d_hist;
    SHIM_BEGIN();
    if (!src || !hist || length < 1 || bins < 2 || bins > kMaxBins) {
        t_status = RECON_ERR_INVALID_ARG;
        return 0.0;
    }
    k_zero_hist<<<1, 256, 0, stream>>>();
    k_hist<<<256, 256, 0, stream>>>(src, length, bins);
    k_hist_out<<<1, 256, 0, stream>>>(hist, bins);
    launched(RECON_OK);
    return 0.0;
}

void filterIndices4(recon_vbuffer *vb, float *grad, float *histf, int P, int nbins, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!vb || !vb->indexDevPtr || !grad || !histf || P < 1 || nbins < 2 || vb->stride != 24 ||
        vb->vertexCount / kSegments > 1024)
        BAD();
    int n = vb->vertexCount;
    k_fill<<<g1d(P), 256, 0, stream>>>(vb->indexDevPtr, P, 0);
    k_seg_count<<<kSegments / 8, 256, 0, stream>>>(grad, histf, n, nbins, P);
    k_seg_scan<<<1, 1, 0, stream>>>();
    k_seg_scatter<<<kSegments / 8, 256, 0, stream>>>(grad, n, nbins, P, vb->indexDevPtr);
    vb->elementsCount = P;
    launched(RECON_OK);
}

void addVertexAttributesWithoutNormalsCuda(float *calib, recon_vbuffer *vb, recon_pyramid *gp, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!calib || !vb || !vb->devPtr || !vb->indexDevPtr || !gp || gp->nLayers < 3 || gp->nLayers > 4 ||
        vb->elementsCount % 512)
        BAD();
    k_attr<<<g1d(vb->elementsCount), 256, 0, stream>>>(vb->indexDevPtr, vb->elementsCount, vb->devPtr, vb->stride,
                                                       gp->width[0], gp->height[0], calib, gp->devPtr[1],
                                                       gp->devPtr[2], gp->nLayers > 3 ? gp->devPtr[3] : nullptr,
                                                       gp->nLayers);
    launched(RECON_OK);
}

void precomputeJacobian4Cuda(recon_vbuffer *vb, float *calib, float *J1, float *J2, float *J3, float *J4,
                             float optScaleIn, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!vb || !vb->devPtr || !vb->indexDevPtr || !J1 || !J2 || !J3 || !J4 || vb->elementsCount % 1024) BAD();
    k_jac<<<g1d(vb->elementsCount), 256, 0, stream>>>(vb->indexDevPtr, vb->elementsCount, vb->devPtr, vb->stride,
                                                      calib, J1, J2, J3, J4, optScaleIn);
    launched(RECON_OK);
}

void interpolateResidual2(recon_vbuffer *vb, float *T, float *calib, recon_pyramid *gp, int layer, float *zcur,
                          float *zw, float *residual, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!vb || !T || !vb->devPtr || !vb->indexDevPtr || !calib || !residual || !zcur || !zw) BAD();
    if (vb->elementsCount % 1024 != 0 || !gp || layer < 0 || layer > gp->nLayers - 1 || !gp->devPtr[layer]) BAD();
    int colorOffset = layer == 0 ? 14 : (layer == 1 ? 17 : (layer == 2 ? 20 : 23));
    float a = 1.0f / (float)(1 << layer);
    float b = 0.5f * (a - 1.0f);
    k_interp<<<g1d(vb->elementsCount), 256, 0, stream>>>(vb->indexDevPtr, vb->elementsCount, vb->devPtr, vb->stride,
                                                         T, calib, a, b, colorOffset, gp->devPtr[layer],
                                                         gp->width[layer], gp->height[layer], zcur, gp->width[0],
                                                         gp->height[0], residual, zw);
    launched(RECON_OK);
}

void generateWeights64(float *r, int count, float *w, float *ext, float *wr, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!r || count < 1024 || !w || !wr || !ext || count % 1024) BAD();
    k_zero_hist<<<1, 256, 0, stream>>>();
    k_w64_hist<<<g1d(count), 256, 0, stream>>>(r, count);
    k_w64_apply<<<g1d(count), 256, 0, stream>>>(r, count, w, ext, wr);
    launched(RECON_OK);
}

void weightJacobian(float *J, float *w, int count, float *Jw, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!J || count < 1024 || !Jw || !w || count % 1024) BAD();
    k_weight_jac<<<g1d(count), 256, 0, stream>>>(J, w, count, Jw);
    launched(RECON_OK);
}

static void reduce_shim(float *JT, float *r, int count, float *jtj, float *jtr, recon_stream_t stream) {
    int nch = count / kChunk;
    k_reduce27<<<nch, kLanes, 0, stream>>>(JT, r, count);
    k_reduce_out<<<1, 32, 0, stream>>>(nch, jtj, jtr);
    launched(RECON_OK);
}

void JTJCuda(float *JT, int count, float *JtJ, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!JT || count < 1024 || !JtJ || count % 1024 || count / kChunk > kMaxChunks) BAD();
    reduce_shim(JT, nullptr, count, JtJ, nullptr, stream);
}

void JTresidualCuda(float *JT, float *r, int count, float *result6, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!JT || !r || count < 1024 || !result6 || count % 1024 || count / kChunk > kMaxChunks) BAD();
    reduce_shim(JT, r, count, nullptr, result6, stream);
}

void linearFuseCuda(float *A1, float *b1, float w1, int N1, float *A2, float *b2, float w2, int N2,
                    recon_stream_t stream) {
    SHIM_BEGIN();
    if (!A1 || !A2 || !b1 || !b2) BAD();
    double invN1 = 1.0 / double(N1), invN2 = 1.0 / double(N2);
    k_fuse<<<1, 36, 0, stream>>>(A1, b1, w1, float(invN1), A2, b2, w2, float(invN2));
    launched(RECON_OK);
}

void solveMotionCuda(float *JtJ, float *b, float *T, float scaleOut, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!JtJ || !b || !T) BAD();
    k_solve_motion<<<1, 32, 0, stream>>>(JtJ, b, T, scaleOut);
    launched(RECON_OK);
}

void genPointCloud6Cuda(float *z, int W, int H, float *pts, int *mask, float *calib, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!z || W < 1 || H < 1 || !pts || !calib || !mask) BAD();
    k_gencloud6<<<g1d(W * H), 256, 0, stream>>>(z, W, H, calib, pts, mask);
    launched(RECON_OK);
}

void computeNormals6Cuda(float *pts, int *mask, int W, int H, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!pts || !mask || W < 1 || H < 1) BAD();
    k_normals6<<<g1d(W * H), 256, 0, stream>>>(pts, mask, W, H);
    launched(RECON_OK);
}

void downSampleCloud6Cuda(float *src, int *msrc, float *dst, int *mdst, int w, int h, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!src || !dst || w < 1 || h < 1 || !msrc || !mdst) BAD();
    k_ds6<<<g1d(w * h), 256, 0, stream>>>(src, msrc, dst, mdst, w, h);
    launched(RECON_OK);
}

void icpResidualMaskCuda2(float *ref6, int *selMask, int w, int h, float *T, float *calib, float *cur6, int *curMask,
                          int layer, float *residual, int *rmask, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!cur6 || !selMask || !T || !calib || !ref6 || !curMask || !residual || !rmask) BAD();
    float a = 1.0f / (float)(1 << layer);
    float b = 0.5f * (a - 1.0f);
    k_icpmask<<<g1d(w * h), 256, 0, stream>>>(ref6, selMask, w, h, T, calib, cur6, curMask, a, b, residual, rmask);
    launched(RECON_OK);
}

void selectValidIndex(int *mask, int n, int *partialSumIntDev, int maxBlocks, int *select, recon_stream_t stream) {
    SHIM_BEGIN();
    int nblk = (n + 1023) / 1024;
    if (n <= 0 || !partialSumIntDev || !select || !mask || (n + 511) / 512 > maxBlocks || nblk > kMaxChunks) BAD();
    k_blkcount<<<nblk, 1024, 0, stream>>>(mask, n);
    k_compact<<<nblk, 1024, 0, stream>>>(mask, n, nblk, select, partialSumIntDev);
    launched(RECON_OK);
}

void packIndex(int *sel, int n, float *full, float *r, float *r2, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!sel || !r || n <= 0 || !full || !r2) BAD();
    k_pack<<<g1d(n), 256, 0, stream>>>(sel, n, full, r, r2);
    launched(RECON_OK);
}

void generateStudentTWeights(float *r2, int n, float *partialSumDev, int maxBlocks, float *w, recon_stream_t stream) {
    SHIM_BEGIN();
    if (!r2 || n <= 0 || !w || !partialSumDev || maxBlocks < 1 || (n + 1023) / 1024 > maxBlocks) BAD();
    k_zero_var<<<1, 32, 0, stream>>>();
    for (int pass = 0; pass <= 3; pass++) k_student<<<g1d(n), 256, 0, stream>>>(r2, n, w, pass);
    launched(RECON_OK);
}

void icpResidualCuda2(float *ref6, int *select, int nsel, int w, int h, int layer, float *T, float *calib, float *cur6,
                      int *curMask, int nPadded, float *res, float *J, float *weights, float optScaleIn,
                      recon_stream_t stream) {
    SHIM_BEGIN();
    if (!cur6 || !select || !T || !calib || !ref6 || !res || !J || !weights || !curMask || nPadded % 1024) BAD();
    float a = 1.0f / (float)(1 << layer);
    float b = 0.5f * (a - 1.0f);
    if (nsel > 0)
        k_icpres<<<g1d(nsel), 256, 0, stream>>>(ref6, select, nsel, w, h, T, calib, cur6, curMask, a, b, nPadded,
                                                res, J, weights, optScaleIn);
    launched(RECON_OK);
}

}  // extern "C"
