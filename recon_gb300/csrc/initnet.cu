// initnet.cu -- the learned initialisation network (include/recon_initnet.h):
// BF16 tensor-core convolutions (mma.sync m16n8k16, FP32 accumulation) for the
// forward pass and for the backward pass's weight and input gradients, FP32
// CUDA-core kernels for the head and Adam.
//
// Every kernel reduces in a fixed order (no floating-point atomics), so a
// training run is deterministic.  The shapes are small (about 10 MFLOP per
// sample): a CTA computes a 16-pixel by Cout output tile directly from the NHWC
// input (implicit GEMM, no im2col buffer).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <math.h>

#include <algorithm>
#include <string>

#include "../../include/recon_initnet.h"
#include "../../include/recon_track.h"

namespace rt {
void set_last_error(const char *msg);
}

namespace nn {

constexpr int kLayers = 6;
constexpr int kCin[kLayers] = {4, 16, 32, 64, 64, 128};
constexpr int kCout[kLayers] = {16, 32, 64, 64, 128, 128};
constexpr int kHt[kLayers + 1] = {60, 30, 15, 8, 4, 2, 1};
constexpr int kWd[kLayers + 1] = {80, 40, 20, 10, 5, 3, 2};
constexpr int kFeat = 128;
constexpr int kOut = RECON_NET_OUT;

constexpr int kpad(int cin) { return (9 * cin + 15) / 16 * 16; }

struct Offsets {
    int64_t w[kLayers], b[kLayers], wfc, bfc, scale, total;
};

Offsets offsets() {
    Offsets o;
    int64_t p = 0;
    for (int l = 0; l < kLayers; l++) {
        o.w[l] = p;
        p += (int64_t)kCout[l] * kpad(kCin[l]);
        o.b[l] = p;
        p += kCout[l];
    }
    o.wfc = p;
    p += (int64_t)kOut * kFeat;
    o.bfc = p;
    p += kOut;
    o.scale = p;
    p += kOut;
    o.total = p;
    return o;
}

__device__ __forceinline__ float bf(const __nv_bfloat16 *p) { return __bfloat162float(*p); }

// out[m][co] = relu(bias[co] + sum_k A[m][k] W[co][k]) with A the 3x3 / stride 2
// / pad 1 patches of `in` (k = tap * Cin + c).  One CTA of 16 warps per 16
// output pixels and K split (blockIdx.y of gridDim.y): the split covers a
// contiguous range of 16-wide K steps, warp w takes output-channel group
// w % NG and the steps j0 + w / NG, + KS, ...; the KS partial tiles are added in
// ascending order in shared memory.  With one split the CTA adds the bias,
// applies the ReLU and stores BF16; with several it stores its FP32 tile to
// `partial` and k_conv_split_finish adds the splits in ascending order.  Every
// order is fixed, so the result does not depend on scheduling.
constexpr int kConvWarps = 16;

template <int COUT>
__global__ void __launch_bounds__(kConvWarps * 32) k_conv_fwd(const __nv_bfloat16 *in, int N, int H, int W, int Cin,
                                                              int Kp, const __nv_bfloat16 *w, const float *bias,
                                                              __nv_bfloat16 *out, int Ho, int Wo, float *partial) {
    constexpr int NF = COUT / 8;             // 8-column fragments
    constexpr int NG = NF < 8 ? NF : 8;      // warps across the columns
    constexpr int FPW = NF / NG;             // fragments per warp
    constexpr int KS = kConvWarps / NG;      // warps across K
    __shared__ float red[KS][16][COUT];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int ng = warp % NG, ks = warp / NG;
    long long M = (long long)N * Ho * Wo;
    long long m0 = (long long)blockIdx.x * 16;
    int g = lane >> 2, tig = lane & 3;
    long long rr[2] = {m0 + g, m0 + g + 8};
    bool rv[2];
    int rn[2], ry[2], rx[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        rv[h] = rr[h] < M;
        long long mm = rv[h] ? rr[h] : 0;
        rx[h] = (int)(mm % Wo);
        ry[h] = (int)((mm / Wo) % Ho);
        rn[h] = (int)(mm / ((long long)Wo * Ho));
    }
    float acc[FPW][4];
#pragma unroll
    for (int f = 0; f < FPW; f++) acc[f][0] = acc[f][1] = acc[f][2] = acc[f][3] = 0.0f;
    int K = 9 * Cin, nk = Kp / 16;
    int S = gridDim.y, per = (nk + S - 1) / S;
    int j0 = blockIdx.y * per, j1 = min(nk, j0 + per);
#pragma unroll 2
    for (int j = j0 + ks; j < j1; j += KS) {
        int kb = 16 * j;
        // A fragment: a0 (row g, k 2t..2t+1), a1 (row g+8), a2 (row g, k+8), a3 (row g+8, k+8)
        uint32_t a[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int h = q & 1;
            int k = kb + 2 * tig + ((q >> 1) ? 8 : 0);
            uint32_t v = 0;
            if (rv[h] && k < K) {
                int tap = k / Cin, c = k - tap * Cin;
                int ky = tap / 3, kx = tap - ky * 3;
                int iy = 2 * ry[h] - 1 + ky, ix = 2 * rx[h] - 1 + kx;
                if (iy >= 0 && iy < H && ix >= 0 && ix < W)
                    v = *reinterpret_cast<const uint32_t *>(in + (((long long)rn[h] * H + iy) * W + ix) * Cin + c);
            }
            a[q] = v;
        }
#pragma unroll
        for (int f = 0; f < FPW; f++) {
            // B fragment: b0 (k 2t..2t+1, n g), b1 (k + 8)
            const __nv_bfloat16 *wr = w + (long long)((ng * FPW + f) * 8 + g) * Kp + kb + 2 * tig;
            uint32_t b0 = *reinterpret_cast<const uint32_t *>(wr);
            uint32_t b1 = *reinterpret_cast<const uint32_t *>(wr + 8);
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                "{%0,%1,%2,%3};\n"
                : "+f"(acc[f][0]), "+f"(acc[f][1]), "+f"(acc[f][2]), "+f"(acc[f][3])
                : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
        }
    }
    // C fragment: c0 c1 (row g, cols 2t, 2t+1), c2 c3 (row g+8)
#pragma unroll
    for (int f = 0; f < FPW; f++) {
        int col = (ng * FPW + f) * 8 + 2 * tig;
        red[ks][g][col] = acc[f][0];
        red[ks][g][col + 1] = acc[f][1];
        red[ks][g + 8][col] = acc[f][2];
        red[ks][g + 8][col + 1] = acc[f][3];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 16 * COUT / 2; e += blockDim.x) {
        int row = e / (COUT / 2), col = 2 * (e % (COUT / 2));
        long long m = m0 + row;
        if (m >= M) continue;
        float v0 = 0.0f, v1 = 0.0f;
#pragma unroll
        for (int q = 0; q < KS; q++) {
            v0 += red[q][row][col];
            v1 += red[q][row][col + 1];
        }
        if (S > 1) {
            float *pp = partial + ((long long)blockIdx.y * M + m) * COUT + col;
            pp[0] = v0;
            pp[1] = v1;
            continue;
        }
        v0 = v0 + bias[col];
        v1 = v1 + bias[col + 1];
        v0 = v0 > 0.0f ? v0 : 0.0f;
        v1 = v1 > 0.0f ? v1 : 0.0f;
        *reinterpret_cast<__nv_bfloat162 *>(out + m * COUT + col) = __floats2bfloat162_rn(v0, v1);
    }
}

// The same convolution for the wide, shallow layers (few channels, K of at
// most a few 16-wide steps): each warp owns a 16-pixel tile and all its
// columns and runs the whole K loop in ascending order, so no warp idles and
// no partial tiles are added.  8 warps (128 pixels) per CTA.
constexpr int kConvPxWarps = 8;

template <int COUT>
__global__ void __launch_bounds__(kConvPxWarps * 32) k_conv_fwd_px(const __nv_bfloat16 *in, int N, int H, int W,
                                                                   int Cin, int Kp, const __nv_bfloat16 *w,
                                                                   const float *bias, __nv_bfloat16 *out, int Ho,
                                                                   int Wo) {
    constexpr int NF = COUT / 8;
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    long long M = (long long)N * Ho * Wo;
    long long m0 = ((long long)blockIdx.x * kConvPxWarps + warp) * 16;
    if (m0 >= M) return;
    int g = lane >> 2, tig = lane & 3;
    long long rr[2] = {m0 + g, m0 + g + 8};
    bool rv[2];
    int rn[2], ry[2], rx[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        rv[h] = rr[h] < M;
        long long mm = rv[h] ? rr[h] : 0;
        rx[h] = (int)(mm % Wo);
        ry[h] = (int)((mm / Wo) % Ho);
        rn[h] = (int)(mm / ((long long)Wo * Ho));
    }
    float acc[NF][4];
#pragma unroll
    for (int f = 0; f < NF; f++) acc[f][0] = acc[f][1] = acc[f][2] = acc[f][3] = 0.0f;
    int K = 9 * Cin, nk = Kp / 16;
    for (int j = 0; j < nk; j++) {
        int kb = 16 * j;
        uint32_t a[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int h = q & 1;
            int k = kb + 2 * tig + ((q >> 1) ? 8 : 0);
            uint32_t v = 0;
            if (rv[h] && k < K) {
                int tap = k / Cin, c = k - tap * Cin;
                int ky = tap / 3, kx = tap - ky * 3;
                int iy = 2 * ry[h] - 1 + ky, ix = 2 * rx[h] - 1 + kx;
                if (iy >= 0 && iy < H && ix >= 0 && ix < W)
                    v = *reinterpret_cast<const uint32_t *>(in + (((long long)rn[h] * H + iy) * W + ix) * Cin + c);
            }
            a[q] = v;
        }
#pragma unroll
        for (int f = 0; f < NF; f++) {
            const __nv_bfloat16 *wr = w + (long long)(f * 8 + g) * Kp + kb + 2 * tig;
            uint32_t b0 = *reinterpret_cast<const uint32_t *>(wr);
            uint32_t b1 = *reinterpret_cast<const uint32_t *>(wr + 8);
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                "{%0,%1,%2,%3};\n"
                : "+f"(acc[f][0]), "+f"(acc[f][1]), "+f"(acc[f][2]), "+f"(acc[f][3])
                : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
        }
    }
#pragma unroll
    for (int f = 0; f < NF; f++) {
        int col = f * 8 + 2 * tig;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if (!rv[h]) continue;
            float v0 = acc[f][2 * h] + bias[col], v1 = acc[f][2 * h + 1] + bias[col + 1];
            v0 = v0 > 0.0f ? v0 : 0.0f;
            v1 = v1 > 0.0f ? v1 : 0.0f;
            *reinterpret_cast<__nv_bfloat162 *>(out + rr[h] * COUT + col) = __floats2bfloat162_rn(v0, v1);
        }
    }
}

// The K splits of a convolution added in ascending order, bias, ReLU, BF16.
template <int COUT>
__global__ void k_conv_split_finish(const float *partial, int S, long long M, const float *bias,
                                    __nv_bfloat16 *out) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= M * (COUT / 2)) return;
    long long m = e / (COUT / 2);
    int col = 2 * (int)(e % (COUT / 2));
    float v0 = 0.0f, v1 = 0.0f;
#pragma unroll 4
    for (int q = 0; q < S; q++) {
        const float *pp = partial + ((long long)q * M + m) * COUT + col;
        v0 += pp[0];
        v1 += pp[1];
    }
    v0 = v0 + bias[col];
    v1 = v1 + bias[col + 1];
    v0 = v0 > 0.0f ? v0 : 0.0f;
    v1 = v1 > 0.0f ? v1 : 0.0f;
    *reinterpret_cast<__nv_bfloat162 *>(out + m * COUT + col) = __floats2bfloat162_rn(v0, v1);
}

// global average pooling of the last activation and the linear layer; one CTA
// (kFeat threads) per sample
__global__ void k_head_fwd(const __nv_bfloat16 *a6, int P, const float *wfc, const float *bfc, float *feat, float *y) {
    __shared__ float f[kFeat];
    int n = blockIdx.x, c = threadIdx.x;
    float s = 0.0f;
    for (int p = 0; p < P; p++) s += bf(a6 + ((long long)n * P + p) * kFeat + c);
    s = s / (float)P;
    f[c] = s;
    feat[(long long)n * kFeat + c] = s;
    __syncthreads();
    if (c < kOut) {
        float v = bfc[c];
        for (int k = 0; k < kFeat; k++) v += wfc[c * kFeat + k] * f[k];
        y[(long long)n * kOut + c] = v;
    }
}

// loss, and the gradients of the linear layer (one CTA of kOut*kFeat
// threads): the output gradients of kHeadChunk samples at a time are staged
// in shared memory, thread (j, c) adds its products over the samples in order,
// and the loss is every thread's squared errors (its entries in order) added
// by a fixed tree.
constexpr int kHeadChunk = 128;
__global__ void k_head_grad(const float *y, const float *t, const float *feat, int N, float *gwfc, float *gbfc,
                            float *loss) {
    static_assert(kOut * kFeat == 768, "the loss tree folds 3 x 256 partial sums");
    __shared__ float sdy[kHeadChunk * kOut];
    __shared__ float red[kOut * kFeat];
    int i = threadIdx.x;  // j * kFeat + c
    int j = i / kFeat, c = i % kFeat;
    float inv = 2.0f / (float)(kOut * N);
    float s = 0.0f, sb = 0.0f, l = 0.0f;
    for (int n0 = 0; n0 < N; n0 += kHeadChunk) {
        int cnt = N - n0 < kHeadChunk ? N - n0 : kHeadChunk;
        __syncthreads();  // the previous chunk is consumed
        for (int e = i; e < cnt * kOut; e += blockDim.x) {
            float d = y[(long long)n0 * kOut + e] - t[(long long)n0 * kOut + e];
            l += d * d;
            sdy[e] = d * inv;
        }
        __syncthreads();
        for (int n = 0; n < cnt; n++) {
            float dy = sdy[n * kOut + j];
            s += dy * feat[(long long)(n0 + n) * kFeat + c];
            sb += dy;
        }
    }
    gwfc[i] = s;
    if (c == 0) gbfc[j] = sb;
    red[i] = l;
    __syncthreads();
    if (i < 256) red[i] = (red[i] + red[i + 256]) + red[i + 512];
    for (int w = 128; w > 0; w >>= 1) {
        __syncthreads();
        if (i < w) red[i] += red[i + w];
    }
    if (i == 0) *loss = red[0] / (float)(kOut * N);
}

// gradient at the last convolution's pre-activation: d feat / P through the
// pooling, masked by the ReLU
__global__ void k_head_back(const float *y, const float *t, const float *wfc, const __nv_bfloat16 *a6, int N, int P,
                            float *dz6) {
    int n = blockIdx.x, c = threadIdx.x;
    float inv = 2.0f / (float)(kOut * N);
    float df = 0.0f;
    for (int j = 0; j < kOut; j++) df += wfc[j * kFeat + c] * ((y[n * kOut + j] - t[n * kOut + j]) * inv);
    df = df / (float)P;
    for (int p = 0; p < P; p++) {
        long long o = ((long long)n * P + p) * kFeat + c;
        dz6[o] = bf(a6 + o) > 0.0f ? df : 0.0f;
    }
}

// two FP32 values rounded to BF16 (round to nearest even) in one 32-bit word,
// the first in the low half (the mma.sync operand order)
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Weight and bias gradients of a convolution on the tensor cores:
// gW[co][k] = sum_m dz[m][co] X[m][k], X the 3x3 / stride 2 / pad 1 patches
// of the layer input (k = tap * Cin + c), a GEMM whose reduction runs over
// the output pixels m, with BF16 operands (dz rounded to nearest even) and
// FP32 accumulation (mma.sync m16n8k16).  CTA (x, s) computes columns
// [64 x, 64 x + 64) for every co over split s of the pixels, staging 64 pixels
// at a time in shared memory transposed (two consecutive pixels per 32-bit
// word, rows padded so that fragment loads hit distinct banks).  Warp w owns
// fragment tiles [w FPW, (w + 1) FPW) of the (co / 16) x (column / 8) grid.
// Split s covers pixels [s per, (s + 1) per).  Writes partial[e][s] for the
// entries e = co (Kp + 1) + k, k < Kp, and, from CTA column 0, the bias
// gradient at k = Kp: the split's FP32 sum of dz (each thread adds its pixel
// pairs in order, the threads of a co are then added in thread order).
constexpr int kWgKT = 64, kWgMS = 64, kWgThreads = 128;
template <int COUT>
__global__ void __launch_bounds__(kWgThreads) k_conv_wgrad_tc(const float *dz, const __nv_bfloat16 *in, int N,
                                                              int H, int W, int Cin, int Kp, int Ho, int Wo,
                                                              int nsplit, int per, float *partial) {
    constexpr int RT = COUT / 16, FPW = RT * 2;  // 8 column fragments per row tile, over 4 warps
    constexpr int LD = kWgMS / 2 + 4;            // words per staged row
    constexpr int TPC = kWgThreads / COUT;       // threads per co in the staging of dz
    static_assert(kWgThreads % COUT == 0 && RT * 8 == 4 * FPW, "tile split");
    __shared__ uint32_t sD[COUT][LD];
    __shared__ uint32_t sX[kWgKT][LD];
    __shared__ int s_n[kWgMS], s_oy[kWgMS], s_ox[kWgMS];
    __shared__ int s_c[kWgKT], s_ky[kWgKT], s_kx[kWgKT];
    __shared__ float s_bias[kWgThreads];
    const uint16_t *inb = reinterpret_cast<const uint16_t *>(in);
    int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    int K = 9 * Cin, kb = blockIdx.x * kWgKT, s = blockIdx.y;
    long long M = (long long)N * Ho * Wo;
    long long mb = (long long)per * s, me = mb + per < M ? mb + per : M;
    if (tid < kWgKT) {
        int k = kb + tid;
        int tap = k / Cin;
        s_c[tid] = k < K ? k - tap * Cin : -1;
        s_ky[tid] = tap / 3;
        s_kx[tid] = tap - (tap / 3) * 3;
    }
    float acc[FPW][4];
#pragma unroll
    for (int q = 0; q < FPW; q++) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.0f;
    float bsum = 0.0f;
    for (long long m0 = mb; m0 < me; m0 += kWgMS) {
        __syncthreads();  // the previous stage is consumed
        if (tid < kWgMS) {
            long long m = m0 + tid;
            s_n[tid] = -1;
            if (m < me) {
                s_ox[tid] = (int)(m % Wo);
                s_oy[tid] = (int)((m / Wo) % Ho);
                s_n[tid] = (int)(m / ((long long)Wo * Ho));
            }
        }
        // dz^T: thread tid always stages co = tid % COUT
        for (int e = tid; e < COUT * (kWgMS / 2); e += kWgThreads) {
            int co = e % COUT, mp = e / COUT;
            long long m = m0 + 2 * mp;
            float v0 = m < me ? dz[m * COUT + co] : 0.0f;
            float v1 = m + 1 < me ? dz[(m + 1) * COUT + co] : 0.0f;
            bsum += v0;
            bsum += v1;
            sD[co][mp] = pack_bf16(v0, v1);
        }
        __syncthreads();  // the pixel decode is visible
        for (int e = tid; e < kWgKT * (kWgMS / 2); e += kWgThreads) {
            int kk = e % kWgKT, mp = e / kWgKT;
            int c = s_c[kk];
            uint32_t word = 0;
            if (c >= 0) {
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    int i = 2 * mp + h, n = s_n[i];
                    if (n < 0) continue;
                    int iy = 2 * s_oy[i] - 1 + s_ky[kk], ix = 2 * s_ox[i] - 1 + s_kx[kk];
                    if (iy >= 0 && iy < H && ix >= 0 && ix < W)
                        word |= (uint32_t)inb[(((long long)n * H + iy) * W + ix) * Cin + c] << (16 * h);
                }
            }
            sX[kk][mp] = word;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < kWgMS / 16; ks++) {
#pragma unroll
            for (int q = 0; q < FPW; q++) {
                int qq = warp * FPW + q, r = qq / 8, f = qq % 8;
                uint32_t a[4] = {sD[16 * r + g][ks * 8 + t], sD[16 * r + g + 8][ks * 8 + t],
                                 sD[16 * r + g][ks * 8 + t + 4], sD[16 * r + g + 8][ks * 8 + t + 4]};
                mma_bf16(acc[q], a, sX[8 * f + g][ks * 8 + t], sX[8 * f + g][ks * 8 + t + 4]);
            }
        }
    }
    int row = Kp + 1;
#pragma unroll
    for (int q = 0; q < FPW; q++) {
        int qq = warp * FPW + q, r = qq / 8, f = qq % 8;
        int k = kb + 8 * f + 2 * t;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            int co = 16 * r + g + 8 * h;
            long long e = (long long)co * row + k;
            if (k < Kp) partial[e * nsplit + s] = acc[q][2 * h];
            if (k + 1 < Kp) partial[(e + 1) * nsplit + s] = acc[q][2 * h + 1];
        }
    }
    if (blockIdx.x == 0) {
        s_bias[tid] = bsum;
        __syncthreads();
        if (tid < COUT) {
            float b = 0.0f;
#pragma unroll
            for (int j = 0; j < TPC; j++) b += s_bias[tid + j * COUT];
            partial[((long long)tid * row + Kp) * nsplit + s] = b;
        }
    }
}

// Sums the splits of every entry of partial[e][s] (e = co (Kp + 1) + k) in a
// fixed order into the flat gradient (weights, then the bias): with few
// splits a thread per entry adds them in order; with many a warp per entry,
// lane q adding splits q, q + 32, ... in order and the lanes then added by a
// fixed butterfly.
__global__ void k_wgrad_reduce(const float *partial, int nsplit, int Cout, int Kp, float *gw, float *gb) {
    int row = Kp + 1;
    long long ne = (long long)Cout * row;
    long long e;
    float v = 0.0f;
    if (nsplit <= 8) {
        e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
        if (e >= ne) return;
        for (int q = 0; q < nsplit; q++) v += partial[e * nsplit + q];
    } else {
        e = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        int lane = threadIdx.x & 31;
        if (e >= ne) return;  // uniform over the warp
        for (int q = lane; q < nsplit; q += 32) v += partial[e * nsplit + q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane) return;
    }
    int co = (int)(e / row), k = (int)(e % row);
    if (k == Kp) gb[co] = v;
    else gw[(long long)co * Kp + k] = v;
}

// Input gradient of a convolution on the tensor cores (the transposed
// convolution of dz, masked by the previous layer's ReLU output a_prev):
// dprev[p][c] = sum over the taps and co of W[co][tap Cin + c] dz[o(p, tap)][co],
// o(p, tap) the output pixel that pixel p feeds through the tap (stride 2: by
// the parity of p's coordinates only 1, 2 or 4 of the 9 taps exist).  A GEMM
// of the input pixels (rows) by Cin (columns) with BF16 operands (dz rounded to
// nearest even, the weights as [9][Cin][Cout] in wt) and FP32 accumulation,
// the taps and co in ascending order.  The rows are the input pixels in parity
// class order ((y & 1, x & 1) outermost, then image, row, column), so the 16
// rows of a warp almost always share their taps and a tap that none of them
// has is skipped.  A CTA has 4 warps: 4 / KS row tiles of 16 rows, each
// reduced by KS warps (warp group kg takes the co steps kg, kg + KS, ... of
// every tap), whose tiles are then added in group order (the deep layers
// have few rows and long reductions).
template <int CIN, int KS>
__global__ void __launch_bounds__(128) k_conv_dgrad_tc(const float *dz, const __nv_bfloat16 *wt,
                                                       const __nv_bfloat16 *a_prev, int N, int H, int W, int Cout,
                                                       int Ho, int Wo, float *dz_prev) {
    constexpr int NF = CIN / 8;
    static_assert(KS == 1 || KS == 2 || KS == 4, "4 warps per CTA");
    __shared__ float red[KS > 1 ? 4 : 1][KS > 1 ? 16 : 1][KS > 1 ? CIN : 1];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    int kg = warp % KS, tile = warp / KS;
    long long rbase = ((long long)blockIdx.x * (4 / KS) + tile) * 16;
    long long pix[2];
    int yy[2], xx[2], nn[2];
    bool ok[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        long long r = rbase + g + 8 * h;
        ok[h] = false;
        pix[h] = 0;
        yy[h] = xx[h] = nn[h] = 0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int py = q >> 1, px = q & 1;
            int hq = (H + 1 - py) / 2, wq = (W + 1 - px) / 2;
            long long cnt = (long long)N * hq * wq;
            if (!ok[h] && r >= 0 && r < cnt) {
                int n = (int)(r / ((long long)hq * wq));
                int rem = (int)(r - (long long)n * hq * wq);
                nn[h] = n;
                yy[h] = 2 * (rem / wq) + py;
                xx[h] = 2 * (rem % wq) + px;
                pix[h] = ((long long)n * H + yy[h]) * W + xx[h];
                ok[h] = true;
            }
            r -= cnt;
        }
    }
    float acc[NF][4];
#pragma unroll
    for (int f = 0; f < NF; f++) acc[f][0] = acc[f][1] = acc[f][2] = acc[f][3] = 0.0f;
    for (int tap = 0; tap < 9; tap++) {
        int ky = tap / 3, kx = tap - ky * 3;
        long long o[2];
        bool v[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            int ty = yy[h] + 1 - ky, tx = xx[h] + 1 - kx;
            v[h] = ok[h] && ty >= 0 && tx >= 0 && !(ty & 1) && !(tx & 1) && (ty >> 1) < Ho && (tx >> 1) < Wo;
            o[h] = v[h] ? (((long long)nn[h] * Ho + (ty >> 1)) * Wo + (tx >> 1)) * Cout : 0;
        }
        if (!__any_sync(0xffffffffu, v[0] || v[1])) continue;
        const uint32_t *wtap = reinterpret_cast<const uint32_t *>(wt + (long long)tap * CIN * Cout);
        for (int co0 = 16 * kg; co0 < Cout; co0 += 16 * KS) {
            uint32_t a[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                int h = q & 1, col = co0 + 2 * t + ((q >> 1) ? 8 : 0);
                float2 d = v[h] ? *reinterpret_cast<const float2 *>(dz + o[h] + col) : make_float2(0.0f, 0.0f);
                a[q] = pack_bf16(d.x, d.y);
            }
#pragma unroll
            for (int f = 0; f < NF; f++) {
                int wi = ((8 * f + g) * Cout + co0 + 2 * t) >> 1;
                mma_bf16(acc[f], a, __ldg(wtap + wi), __ldg(wtap + wi + 4));
            }
        }
    }
    if (KS > 1) {
        // groups 1.. leave their tiles in shared memory, group 0 adds them in order
#pragma unroll
        for (int k = 1; k < KS; k++) {
            if (kg == k) {
#pragma unroll
                for (int f = 0; f < NF; f++)
#pragma unroll
                    for (int q = 0; q < 4; q++) red[warp][g + 8 * (q >> 1)][8 * f + 2 * t + (q & 1)] = acc[f][q];
            }
        }
        __syncthreads();
        if (kg != 0) return;
#pragma unroll
        for (int k = 1; k < KS; k++)
#pragma unroll
            for (int f = 0; f < NF; f++)
#pragma unroll
                for (int q = 0; q < 4; q++) acc[f][q] += red[warp + k][g + 8 * (q >> 1)][8 * f + 2 * t + (q & 1)];
    }
#pragma unroll
    for (int h = 0; h < 2; h++) {
        if (!ok[h]) continue;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            int c = 8 * f + 2 * t;
            long long idx = pix[h] * CIN + c;
            float2 out;
            out.x = bf(a_prev + idx) > 0.0f ? acc[f][2 * h] : 0.0f;
            out.y = bf(a_prev + idx + 1) > 0.0f ? acc[f][2 * h + 1] : 0.0f;
            *reinterpret_cast<float2 *>(dz_prev + idx) = out;
        }
    }
}

// The convolution weights of every layer as [9][Cin][Cout] (BF16) for the
// input-gradient kernel: wt[tap][c][co] = w[co][tap Cin + c].
struct WtLayout {
    int64_t src[kLayers], dst[kLayers];
    int cin[kLayers], cout[kLayers];
};
__global__ void k_wt_transpose(const __nv_bfloat16 *pbf, __nv_bfloat16 *wt, WtLayout lay) {
    int l = blockIdx.y;
    int Cin = lay.cin[l], Cout = lay.cout[l], Kp = (9 * Cin + 15) / 16 * 16;
    int tot = 9 * Cin * Cout;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
        int co = e % Cout, k = e / Cout;  // k = tap * Cin + c
        wt[lay.dst[l] + e] = pbf[lay.src[l] + (int64_t)co * Kp + k];
    }
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, int64_t n, float lr, float bc1, float bc2) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float gi = g[i];
    float mi = b1 * m[i] + (1.0f - b1) * gi;
    float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

__global__ void k_to_bf16(const float *p, __nv_bfloat16 *q, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) q[i] = __float2bfloat16_rn(p[i]);
}

__global__ void k_coarse(const uint8_t *gray, const uint16_t *depth, int n, int W, int H, __nv_bfloat16 *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int per = RECON_NET_W * RECON_NET_H;
    if (i >= n * per) return;
    int f = i / per, p = i % per;
    int ox = p % RECON_NET_W, oy = p / RECON_NET_W;
    int bx = W / RECON_NET_W, by = H / RECON_NET_H;
    const uint8_t *g = gray + (long long)f * W * H;
    const uint16_t *dp = depth + (long long)f * W * H;
    int gs = 0, cnt = 0;
    long long ds = 0;
    for (int y = 0; y < by; y++)
        for (int x = 0; x < bx; x++) {
            long long o = (long long)(oy * by + y) * W + ox * bx + x;
            gs += g[o];
            int dv = dp[o];
            if (dv) {
                ds += dv;
                cnt++;
            }
        }
    float gv = (float)gs / (255.0f * (float)(bx * by));
    float dv = cnt ? ((float)ds / (float)cnt) / 4000.0f : 0.0f;
    out[2 * (long long)i] = __float2bfloat16_rn(gv);
    out[2 * (long long)i + 1] = __float2bfloat16_rn(dv);
}

__global__ void k_pair(const __nv_bfloat16 *prev, const __nv_bfloat16 *cur, int n, __nv_bfloat16 *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int per = RECON_NET_W * RECON_NET_H;
    if (i >= n * per) return;
    out[4 * (long long)i + 0] = prev[2 * (long long)i];
    out[4 * (long long)i + 1] = prev[2 * (long long)i + 1];
    out[4 * (long long)i + 2] = cur[2 * (long long)i];
    out[4 * (long long)i + 3] = cur[2 * (long long)i + 1];
}

}  // namespace nn

using namespace nn;

struct recon_initnet {
    int max_batch = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    Offsets off;
    float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *pbf = nullptr;
    __nv_bfloat16 *wt = nullptr;  // the convolution weights as [9][Cin][Cout] per layer
    WtLayout wt_lay;
    __nv_bfloat16 *act[kLayers] = {nullptr};
    float *dz[kLayers] = {nullptr};
    float *feat = nullptr, *y = nullptr, *partial = nullptr, *loss = nullptr;
    float *fpart = nullptr;  // forward K-split tiles
    int64_t partial_floats = 0;
    int64_t step = 0;
};

namespace {

int net_fail(int code, const std::string &msg) {
    rt::set_last_error(msg.c_str());
    return code;
}

#define NCK(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return net_fail(RECON_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int64_t act_count(int l, int n) { return (int64_t)n * kHt[l + 1] * kWd[l + 1] * kCout[l]; }

// Output pixels per split of layer l's weight gradient for a batch of n: a
// multiple of the 64-pixel stage, so that the layer's CTAs (splits x 64-column
// tiles) number about 1024.
int wg_per_split(int l, int n) {
    long long M = (long long)n * kHt[l + 1] * kWd[l + 1];
    long long kt = (kpad(kCin[l]) + kWgKT - 1) / kWgKT;
    long long per = (M * kt + 1023) / 1024;
    per = (per + kWgMS - 1) / kWgMS * kWgMS;
    return (int)(per < kWgMS ? kWgMS : per);
}
int nsplit_for(int l, int n) {
    long long M = (long long)n * kHt[l + 1] * kWd[l + 1];
    int per = wg_per_split(l, n);
    return (int)((M + per - 1) / per);
}

// K splits of layer l's forward convolution for a batch of n: enough CTAs for
// about two per SM when the layer has few output pixels (the deep layers), at
// least one 16-wide K step per warp and split.
bool pixel_parallel(int l, int n);
int fsplit_for(int l, int n) {
    long long M = (long long)n * kHt[l + 1] * kWd[l + 1];
    long long ctas = (M + 15) / 16;
    int NF = kCout[l] / 8, NG = NF < 8 ? NF : 8, KS = kConvWarps / NG;
    int nk = kpad(kCin[l]) / 16;
    if (ctas > 76) return 1;  // at least half the SMs busy: the finishing pass would cost more
    long long s = (2 * 152) / ctas;
    if (s > nk / KS) s = nk / KS;
    return (int)(s < 1 ? 1 : s);
}

// Layers whose 16 warps would mostly idle in k_conv_fwd (fewer K steps than the
// warps it spreads over K), and layers of a batch with at least 4096 tiles of
// 16 output pixels (a training batch: enough warps to fill the GPU many times
// over without splitting K), run as k_conv_fwd_px.
bool pixel_parallel(int l, int n) {
    int NF = kCout[l] / 8, NG = NF < 8 ? NF : 8, KS = kConvWarps / NG;
    long long tiles = ((long long)n * kHt[l + 1] * kWd[l + 1] + 15) / 16;
    return kpad(kCin[l]) / 16 < KS || tiles >= 4096;
}

template <int COUT>
void conv_launch(recon_initnet *net, int l, const __nv_bfloat16 *in, int n) {
    int Cin = kCin[l], Kp = kpad(Cin);
    long long M = (long long)n * kHt[l + 1] * kWd[l + 1];
    if (pixel_parallel(l, n)) {
        long long tiles = (M + 15) / 16;
        k_conv_fwd_px<COUT><<<(unsigned)((tiles + kConvPxWarps - 1) / kConvPxWarps), kConvPxWarps * 32, 0,
                               net->stream>>>(in, n, kHt[l], kWd[l], Cin, Kp, net->pbf + net->off.w[l],
                                              net->params + net->off.b[l], net->act[l], kHt[l + 1], kWd[l + 1]);
        return;
    }
    int S = fsplit_for(l, n);
    dim3 grid((unsigned)((M + 15) / 16), (unsigned)S);
    const __nv_bfloat16 *w = net->pbf + net->off.w[l];
    const float *b = net->params + net->off.b[l];
    k_conv_fwd<COUT><<<grid, kConvWarps * 32, 0, net->stream>>>(in, n, kHt[l], kWd[l], Cin, Kp, w, b, net->act[l],
                                                                kHt[l + 1], kWd[l + 1], net->fpart);
    if (S > 1) {
        long long pairs = M * (COUT / 2);
        k_conv_split_finish<COUT><<<(unsigned)((pairs + 255) / 256), 256, 0, net->stream>>>(net->fpart, S, M, b,
                                                                                           net->act[l]);
    }
}

int conv_forward(recon_initnet *net, int l, const __nv_bfloat16 *in, int n) {
    switch (kCout[l]) {
        case 16: conv_launch<16>(net, l, in, n); break;
        case 32: conv_launch<32>(net, l, in, n); break;
        case 64: conv_launch<64>(net, l, in, n); break;
        default: conv_launch<128>(net, l, in, n); break;
    }
    return RECON_OK;
}

int forward(recon_initnet *net, const __nv_bfloat16 *in, int n) {
    const __nv_bfloat16 *x = in;
    for (int l = 0; l < kLayers; l++) {
        conv_forward(net, l, x, n);
        x = net->act[l];
    }
    int P = kHt[kLayers] * kWd[kLayers];
    k_head_fwd<<<n, kFeat, 0, net->stream>>>(net->act[kLayers - 1], P, net->params + net->off.wfc,
                                             net->params + net->off.bfc, net->feat, net->y);
    NCK(cudaGetLastError());
    return RECON_OK;
}

int backward(recon_initnet *net, const __nv_bfloat16 *in, const float *target, int n, float *grad, float *loss) {
    int P = kHt[kLayers] * kWd[kLayers];
    k_head_grad<<<1, kOut * kFeat, 0, net->stream>>>(net->y, target, net->feat, n, grad + net->off.wfc,
                                                    grad + net->off.bfc, loss);
    k_head_back<<<n, kFeat, 0, net->stream>>>(net->y, target, net->params + net->off.wfc, net->act[kLayers - 1], n, P,
                                              net->dz[kLayers - 1]);
    for (int l = kLayers - 1; l >= 0; l--) {
        int Cin = kCin[l], Cout = kCout[l], Kp = kpad(Cin);
        int H = kHt[l], W = kWd[l], Ho = kHt[l + 1], Wo = kWd[l + 1];
        const __nv_bfloat16 *lin = l ? net->act[l - 1] : in;
        int ns = nsplit_for(l, n), per = wg_per_split(l, n);
        int row = Kp + 1;
        dim3 g1((Kp + kWgKT - 1) / kWgKT, ns);
        switch (Cout) {
            case 16: k_conv_wgrad_tc<16><<<g1, kWgThreads, 0, net->stream>>>(net->dz[l], lin, n, H, W, Cin, Kp, Ho, Wo, ns, per, net->partial); break;
            case 32: k_conv_wgrad_tc<32><<<g1, kWgThreads, 0, net->stream>>>(net->dz[l], lin, n, H, W, Cin, Kp, Ho, Wo, ns, per, net->partial); break;
            case 64: k_conv_wgrad_tc<64><<<g1, kWgThreads, 0, net->stream>>>(net->dz[l], lin, n, H, W, Cin, Kp, Ho, Wo, ns, per, net->partial); break;
            default: k_conv_wgrad_tc<128><<<g1, kWgThreads, 0, net->stream>>>(net->dz[l], lin, n, H, W, Cin, Kp, Ho, Wo, ns, per, net->partial); break;
        }
        long long red_threads = (long long)Cout * row * (ns <= 8 ? 1 : 32);
        k_wgrad_reduce<<<(unsigned)((red_threads + 127) / 128), 128, 0, net->stream>>>(
            net->partial, ns, Cout, Kp, grad + net->off.w[l], grad + net->off.b[l]);
        if (l > 0) {
            // rows of 16 per tile; the reduction split over 2 or 4 warps when the
            // layer has fewer than 8 or 4 tiles per SM (and co steps to share)
            long long rows = (long long)n * H * W, tiles = (rows + 15) / 16;
            int ks = 1;
            if (tiles < 8 * 152) ks = 2;
            if (tiles < 4 * 152) ks = 4;
            while (ks > 1 && Cout / 16 < ks) ks >>= 1;
            unsigned blocks = (unsigned)((tiles + 4 / ks - 1) / (4 / ks));
            const __nv_bfloat16 *wt = net->wt + net->wt_lay.dst[l];
            const __nv_bfloat16 *ap = net->act[l - 1];
            float *dp = net->dz[l - 1];
#define RECON_DGRAD(CI, K) k_conv_dgrad_tc<CI, K><<<blocks, 128, 0, net->stream>>>(net->dz[l], wt, ap, n, H, W, Cout, Ho, Wo, dp)
#define RECON_DGRAD_KS(CI) (ks == 4 ? RECON_DGRAD(CI, 4) : ks == 2 ? RECON_DGRAD(CI, 2) : RECON_DGRAD(CI, 1))
            switch (Cin) {
                case 16: RECON_DGRAD_KS(16); break;
                case 32: RECON_DGRAD_KS(32); break;
                case 64: RECON_DGRAD_KS(64); break;
                default: RECON_DGRAD_KS(128); break;
            }
#undef RECON_DGRAD_KS
#undef RECON_DGRAD
        }
    }
    NCK(cudaMemsetAsync(grad + net->off.scale, 0, kOut * sizeof(float), net->stream));
    NCK(cudaGetLastError());
    return RECON_OK;
}

int check_batch(recon_initnet *net, int n) {
    if (!net) return net_fail(RECON_ERR_INVALID_ARG, "null network");
    if (n <= 0 || n > net->max_batch) return net_fail(RECON_ERR_INVALID_ARG, "batch size outside 1..max_batch");
    return RECON_OK;
}

void refresh_bf16(recon_initnet *net) {
    int64_t tot = net->off.total;
    k_to_bf16<<<(unsigned)((tot + 255) / 256), 256, 0, net->stream>>>(net->params, net->pbf, tot);
    k_wt_transpose<<<dim3(64, kLayers), 256, 0, net->stream>>>(net->pbf, net->wt, net->wt_lay);
}

}  // namespace

namespace nn {
// forward pass on another stream (the tracker's), output to `out` [n][6]
int forward_on(recon_initnet *net, const uint16_t *in_bf16, int n, float *out, cudaStream_t s) {
    int rc = check_batch(net, n);
    if (rc) return rc;
    cudaStream_t keep = net->stream;
    net->stream = s;
    rc = forward(net, reinterpret_cast<const __nv_bfloat16 *>(in_bf16), n);
    if (!rc && cudaMemcpyAsync(out, net->y, (int64_t)n * kOut * 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        rc = net_fail(RECON_ERR_CUDA, "initnet output copy");
    net->stream = keep;
    return rc;
}
const float *scale_dev(recon_initnet *net) { return net->params + net->off.scale; }
// kernels one forward pass of a batch of n launches: the convolutions, their
// split-K finishing kernels and the pooling + linear layer
int forward_kernels(int n) {
    int k = kLayers + 1;
    for (int l = 0; l < kLayers; l++) k += (!pixel_parallel(l, n) && fsplit_for(l, n) > 1) ? 1 : 0;
    return k;
}
}  // namespace nn

extern "C" {

int64_t recon_initnet_param_count(void) { return offsets().total; }

int recon_initnet_create(int32_t max_batch, void *stream, recon_initnet **out) {
    if (!out || max_batch <= 0) return net_fail(RECON_ERR_INVALID_ARG, "bad argument");
    *out = nullptr;
    recon_initnet *net = new recon_initnet();
    net->max_batch = max_batch;
    net->off = offsets();
    net->stream = (cudaStream_t)stream;  // NULL: the legacy default stream
    int64_t P = net->off.total;
    int64_t nwt = 0;
    for (int l = 0; l < kLayers; l++) {
        net->wt_lay.src[l] = net->off.w[l];
        net->wt_lay.dst[l] = nwt;
        net->wt_lay.cin[l] = kCin[l];
        net->wt_lay.cout[l] = kCout[l];
        nwt += 9LL * kCin[l] * kCout[l];
    }
    int64_t part = 0;
    for (int l = 0; l < kLayers; l++) {
        for (int nb = 1; nb <= max_batch; nb++) {
            int64_t s = (int64_t)nsplit_for(l, nb) * kCout[l] * (kpad(kCin[l]) + 1);
            if (s > part) part = s;
        }
    }
    net->partial_floats = part;
    int64_t fpart = 1;
    for (int l = 0; l < kLayers; l++)
        for (int nb = 1; nb <= max_batch; nb++) {
            int S = fsplit_for(l, nb);
            if (S > 1) fpart = std::max(fpart, (int64_t)S * nb * kHt[l + 1] * kWd[l + 1] * kCout[l]);
        }
    bool ok = cudaMalloc(&net->params, P * 4) == cudaSuccess && cudaMalloc(&net->grad, P * 4) == cudaSuccess &&
              cudaMalloc(&net->m, P * 4) == cudaSuccess && cudaMalloc(&net->v, P * 4) == cudaSuccess &&
              cudaMalloc(&net->pbf, P * 2) == cudaSuccess && cudaMalloc(&net->wt, nwt * 2) == cudaSuccess &&
              cudaMalloc(&net->feat, (int64_t)max_batch * kFeat * 4) == cudaSuccess &&
              cudaMalloc(&net->y, (int64_t)max_batch * kOut * 4) == cudaSuccess &&
              cudaMalloc(&net->partial, part * 4) == cudaSuccess && cudaMalloc(&net->fpart, fpart * 4) == cudaSuccess &&
              cudaMalloc(&net->loss, 16) == cudaSuccess;
    for (int l = 0; ok && l < kLayers; l++) {
        ok = cudaMalloc(&net->act[l], act_count(l, max_batch) * 2) == cudaSuccess &&
             cudaMalloc(&net->dz[l], act_count(l, max_batch) * 4) == cudaSuccess;
    }
    if (!ok) {
        recon_initnet_destroy(net);
        return net_fail(RECON_ERR_CUDA, "cudaMalloc(initnet)");
    }
    cudaMemsetAsync(net->params, 0, P * 4, net->stream);
    cudaMemsetAsync(net->m, 0, P * 4, net->stream);
    cudaMemsetAsync(net->v, 0, P * 4, net->stream);
    cudaMemsetAsync(net->grad, 0, P * 4, net->stream);
    refresh_bf16(net);
    if (cudaStreamSynchronize(net->stream) != cudaSuccess) {
        recon_initnet_destroy(net);
        return net_fail(RECON_ERR_CUDA, "initnet set-up");
    }
    *out = net;
    return RECON_OK;
}

int recon_initnet_destroy(recon_initnet *net) {
    if (!net) return RECON_OK;
    if (net->stream) cudaStreamSynchronize(net->stream);
    cudaFree(net->params);
    cudaFree(net->grad);
    cudaFree(net->m);
    cudaFree(net->v);
    cudaFree(net->pbf);
    cudaFree(net->wt);
    cudaFree(net->feat);
    cudaFree(net->y);
    cudaFree(net->partial);
    cudaFree(net->fpart);
    cudaFree(net->loss);
    for (int l = 0; l < kLayers; l++) {
        cudaFree(net->act[l]);
        cudaFree(net->dz[l]);
    }
    if (net->own_stream) cudaStreamDestroy(net->stream);
    delete net;
    return RECON_OK;
}

int recon_initnet_set_params(recon_initnet *net, const float *params, int32_t on_device) {
    if (!net || !params) return net_fail(RECON_ERR_INVALID_ARG, "null argument");
    (void)cudaGetLastError();
    NCK(cudaMemcpyAsync(net->params, params, net->off.total * 4,
                        on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, net->stream));
    NCK(cudaMemsetAsync(net->m, 0, net->off.total * 4, net->stream));
    NCK(cudaMemsetAsync(net->v, 0, net->off.total * 4, net->stream));
    net->step = 0;
    refresh_bf16(net);
    NCK(cudaStreamSynchronize(net->stream));
    return RECON_OK;
}

int recon_initnet_get_params(recon_initnet *net, float *params_host) {
    if (!net || !params_host) return net_fail(RECON_ERR_INVALID_ARG, "null argument");
    (void)cudaGetLastError();
    NCK(cudaMemcpyAsync(params_host, net->params, net->off.total * 4, cudaMemcpyDeviceToHost, net->stream));
    NCK(cudaStreamSynchronize(net->stream));
    return RECON_OK;
}

int recon_initnet_forward(recon_initnet *net, const uint16_t *in_bf16, int32_t n, float *out) {
    int rc = check_batch(net, n);
    if (rc) return rc;
    if (!in_bf16 || !out) return net_fail(RECON_ERR_INVALID_ARG, "null argument");
    (void)cudaGetLastError();
    rc = forward(net, reinterpret_cast<const __nv_bfloat16 *>(in_bf16), n);
    if (rc) return rc;
    NCK(cudaMemcpyAsync(out, net->y, (int64_t)n * kOut * 4, cudaMemcpyDeviceToDevice, net->stream));
    return RECON_OK;
}

int recon_initnet_gradient(recon_initnet *net, const uint16_t *in_bf16, const float *target, int32_t n, float *grad,
                           float *loss_dev) {
    int rc = check_batch(net, n);
    if (rc) return rc;
    if (!in_bf16 || !target || !grad || !loss_dev) return net_fail(RECON_ERR_INVALID_ARG, "null argument");
    (void)cudaGetLastError();
    const __nv_bfloat16 *in = reinterpret_cast<const __nv_bfloat16 *>(in_bf16);
    rc = forward(net, in, n);
    if (rc) return rc;
    return backward(net, in, target, n, grad, loss_dev);
}

int recon_initnet_train_step(recon_initnet *net, const uint16_t *in_bf16, const float *target, int32_t n, float lr,
                             float *loss_dev) {
    int rc = check_batch(net, n);
    if (rc) return rc;
    if (!in_bf16 || !target || !loss_dev) return net_fail(RECON_ERR_INVALID_ARG, "null argument");
    (void)cudaGetLastError();
    const __nv_bfloat16 *in = reinterpret_cast<const __nv_bfloat16 *>(in_bf16);
    rc = forward(net, in, n);
    if (rc) return rc;
    rc = backward(net, in, target, n, net->grad, loss_dev);
    if (rc) return rc;
    net->step++;
    float bc1 = 1.0f - powf(0.9f, (float)net->step), bc2 = 1.0f - powf(0.999f, (float)net->step);
    int64_t ntrain = net->off.scale;  // the output scale is not trained
    k_adam<<<(unsigned)((ntrain + 255) / 256), 256, 0, net->stream>>>(net->params, net->grad, net->m, net->v, ntrain,
                                                                      lr, bc1, bc2);
    refresh_bf16(net);
    NCK(cudaGetLastError());
    return RECON_OK;
}

int recon_initnet_coarse(const uint8_t *gray, const uint16_t *depth, int32_t n, int32_t width, int32_t height,
                         uint16_t *out_bf16, void *stream) {
    if (!gray || !depth || !out_bf16 || n <= 0) return net_fail(RECON_ERR_INVALID_ARG, "null argument");
    if (width < RECON_NET_W || height < RECON_NET_H || width % RECON_NET_W || height % RECON_NET_H)
        return net_fail(RECON_ERR_INVALID_ARG, "frame size must be a multiple of 80 x 60");
    (void)cudaGetLastError();
    int tot = n * RECON_NET_W * RECON_NET_H;
    k_coarse<<<(tot + 255) / 256, 256, 0, (cudaStream_t)stream>>>(gray, depth, n, width, height,
                                                                  reinterpret_cast<__nv_bfloat16 *>(out_bf16));
    NCK(cudaGetLastError());
    return RECON_OK;
}

int recon_initnet_pair(const uint16_t *prev_coarse, const uint16_t *cur_coarse, int32_t n, uint16_t *in_bf16,
                       void *stream) {
    if (!prev_coarse || !cur_coarse || !in_bf16 || n <= 0) return net_fail(RECON_ERR_INVALID_ARG, "null argument");
    (void)cudaGetLastError();
    int tot = n * RECON_NET_W * RECON_NET_H;
    k_pair<<<(tot + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const __nv_bfloat16 *>(prev_coarse), reinterpret_cast<const __nv_bfloat16 *>(cur_coarse), n,
        reinterpret_cast<__nv_bfloat16 *>(in_bf16));
    NCK(cudaGetLastError());
    return RECON_OK;
}

}  // extern "C"
