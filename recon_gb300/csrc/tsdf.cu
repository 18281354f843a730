// tsdf.cu -- the reconstruction stream: TSDF fusion of distance maps into a
// voxel grid, ray casting and shading of the fused surface, resampling of a
// grid into a moved frame, and the distance map of an RGB-D frame.
//
// Reference: tracker/kernels/VoxelGrid_cuda.cu (kernels) and
// tracker/reconstruct/VoxelGrid.cpp (host object).  Every per-voxel and
// per-pixel value is the reference's arithmetic in its source order (the
// library is built with -fmad=false; divisions and square roots are IEEE);
// float -> unsigned conversions saturate as the reference's make_uint3 and
// `uint += float` do on the GPU.  What differs is how the work is mapped:
//
//  * update: one CTA per 32x8x8 block of voxels, each thread a run of 8 voxels
//    along z at one (x, y), so that a warp reads and writes 32 consecutive
//    float2 (256 bytes).  A block whose voxel centres all project outside the
//    image (tested at its 8 corners, with a margin for rounding) is skipped
//    as a whole: the projection is a linear-fractional map, so over a box on
//    one side of the camera plane its extremes lie at the corners.  A voxel is
//    written only when its value changes.
//  * ray cast: one thread per pixel, one warp per 8x4 tile.  A byte per 8x8x8 brick
//    records whether any voxel of the brick may be negative; the traversal
//    steps through bricks without one using only its step arithmetic (the
//    reference's coarse test, tsdf < 0, cannot pass there), so empty space
//    costs no grid reads.  The byte is set whenever a negative value is
//    stored and cleared only by a reset or a rebuild, so it never hides a
//    negative voxel.
//  * where the reference would read past the end of the grid array (its
//    bounds checks are commented out), a ray reports no hit.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>
#include <string.h>

#include <cmath>
#include <string>
#include <utility>
#include <vector>

#include "../../include/recon_track.h"
#include "../../include/recon_tsdf.h"

namespace rt {
void set_last_error(const char *msg);
void add_launches(long long n);
}  // namespace rt

namespace tsdf {

constexpr int kBrick = 8;    // voxels per side of a flag brick
constexpr int kTileX = 32;   // update CTA: 32 x 8 columns of 8 voxels along z
constexpr int kTileY = 8;
constexpr int kRunZ = 8;
constexpr int kRayTileX = 8;  // ray cast CTA: one warp on 8 x 4 pixels (rays differ widely in length;
constexpr int kRayTileY = 4;  // one-warp CTAs let the block scheduler balance the SMs)
constexpr int kKinds = 5;     // timing kinds: update, ray cast, shading, distance map, reset / resample

struct Geom {
    int R, B, SB, W, H;             // voxels, 8^3 bricks and 32^3 super bricks per side, image size
    int nb;                         // B^3: offset of the super-brick bytes
    float T[12];                    // update: world -> camera; ray cast / resample: camera -> world
    float K0, K2, K4, K5, Wf, Hf, Wm2, Hm2;
    float sx, sy, sz;               // centre of voxel 0 (start)
    float vx2, vy2, vz2;            // voxel spacing (2 * voxelSize)
    float lim, tol, slope;          // update gates
    float b0x, b0y, b0z, b1x, b1y, b1z;  // grid bounds
    float ib0x, ib0y, ib0z;         // interpolation origin
    float ivx, ivy, ivz;            // 1 / voxel spacing (voxelize's invVoxelDim)
    float min_dist, max_dist;
};

__device__ __forceinline__ unsigned f2u(float v) { return __float2uint_rz(v); }

__device__ __forceinline__ size_t brick_of(const Geom &g, unsigned x, unsigned y, unsigned z) {
    return ((size_t)(z >> 3) * g.B + (y >> 3)) * g.B + (x >> 3);
}
__device__ __forceinline__ size_t super_of(const Geom &g, unsigned x, unsigned y, unsigned z) {
    return (size_t)g.nb + ((size_t)(z >> 5) * g.SB + (y >> 5)) * g.SB + (x >> 5);
}
// marks the brick and super brick of a voxel that holds a negative value
__device__ __forceinline__ void mark_negative(uint8_t *flags, const Geom &g, unsigned x, unsigned y, unsigned z) {
    flags[brick_of(g, x, y, z)] = 1;
    flags[super_of(g, x, y, z)] = 1;
}

// ---------------------------------------------------------------- update --

// updateVoxelsKernel (VoxelGrid_cuda.cu:944-1014).  counts (kCount): voxels
// [projected into the image, fused, changed].
template <bool kCount>
__global__ void __launch_bounds__(kTileX * kTileY)
    k_update(float2 *__restrict__ grid, uint8_t *__restrict__ flags, const float *__restrict__ dist, Geom g,
             unsigned long long *__restrict__ counts) {
    __shared__ int s_skip;
    const int lane = threadIdx.x & 31;
    const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * kTileY, z0 = blockIdx.z * kRunZ;
    if (threadIdx.x < 32) {
        // the block's corner voxel centres (lanes 8..31 repeat lanes 0..7)
        const int c = lane & 7;
        const int cx = min(x0 + ((c & 1) ? kTileX - 1 : 0), g.R - 1);
        const int cy = y0 + ((c & 2) ? kTileY - 1 : 0), cz = z0 + ((c & 4) ? kRunZ - 1 : 0);
        const float px = g.sx + (float)cx * g.vx2, py = g.sy + (float)cy * g.vy2, pz = g.sz + (float)cz * g.vz2;
        const float rx = g.T[0] * px + g.T[1] * py + g.T[2] * pz + g.T[3];
        const float ry = g.T[4] * px + g.T[5] * py + g.T[6] * pz + g.T[7];
        const float rz = g.T[8] * px + g.T[9] * py + g.T[10] * pz + g.T[11];
        float ux = (rx / rz * g.K0 + g.K2) * g.Wf, uy = (ry / rz * g.K4 + g.K5) * g.Hf;
        float lo_x = ux, hi_x = ux, lo_y = uy, hi_y = uy;
        for (int o = 1; o < 8; o <<= 1) {
            lo_x = fminf(lo_x, __shfl_xor_sync(0xffffffffu, lo_x, o));
            hi_x = fmaxf(hi_x, __shfl_xor_sync(0xffffffffu, hi_x, o));
            lo_y = fminf(lo_y, __shfl_xor_sync(0xffffffffu, lo_y, o));
            hi_y = fmaxf(hi_y, __shfl_xor_sync(0xffffffffu, hi_y, o));
        }
        // |rz| >= 16 mm at every corner keeps the rounding of the projected
        // coordinates far below the 4-pixel margin
        const unsigned front = __ballot_sync(0xffffffffu, rz < -16.0f) & 0xffu;
        const unsigned behind = __ballot_sync(0xffffffffu, rz > 16.0f) & 0xffu;
        const bool one_side = (front == 0xffu) || (behind == 0xffu);
        const bool outside = !(hi_x >= -3.0f) || !(lo_x < g.Wf + 2.0f) || !(hi_y >= -3.0f) || !(lo_y < g.Hf + 2.0f);
        if (lane == 0) s_skip = one_side && outside;
    }
    __syncthreads();
    if (s_skip) return;
    const int ix = x0 + lane, iy = y0 + (threadIdx.x >> 5);
    if (ix >= g.R) return;
    const float px = g.sx + (float)ix * g.vx2;
    const float py = g.sy + (float)iy * g.vy2;
    // T p summed left to right: the first two products do not depend on z
    const float ax = g.T[0] * px + g.T[1] * py, ay = g.T[4] * px + g.T[5] * py, az = g.T[8] * px + g.T[9] * py;
    unsigned n_proj = 0, n_fused = 0, n_changed = 0;
    const int W = g.W;
#pragma unroll 2
    for (int k = 0; k < kRunZ; k++) {
        const int iz = z0 + k;
        const float pz = g.sz + (float)iz * g.vz2;
        float rx = ax + g.T[2] * pz + g.T[3];
        float ry = ay + g.T[6] * pz + g.T[7];
        const float rz = az + g.T[10] * pz + g.T[11];
        const float voxel_dist = -rz;
        rx /= rz;
        ry /= rz;
        const float ux = (rx * g.K0 + g.K2) * g.Wf;
        const float uy = (ry * g.K4 + g.K5) * g.Hf;
        // int(u) in [1, size - 2): the reference's safeBorder of 1
        if (!(ux >= 1.0f && ux < g.Wm2 && uy >= 1.0f && uy < g.Hm2)) continue;
        n_proj++;
        const int ui = (int)ux, vi = (int)uy;
        const float *dp = dist + (size_t)vi * W + ui;
        const float a = __ldg(dp), b = __ldg(dp + 1), c = __ldg(dp + W), d = __ldg(dp + W + 1);
        if (a < g.lim || b < g.lim || c < g.lim || d < g.lim) continue;
        const float fu = ux - (float)ui;
        const float fv = uy - (float)vi;
        const float z = (1 - fu) * (1 - fv) * a + fu * (1 - fv) * b + (1 - fu) * fv * c + fu * fv * d;
        if (fabsf(z - a) > g.tol || fabsf(z - b) > g.tol || fabsf(z - c) > g.tol || fabsf(z - d) > g.tol) continue;
        const float sdf = -(voxel_dist - z) / g.slope;
        if (sdf < -1.25f) continue;
        n_fused++;
        const float nt = fmaxf(fminf(1.0f, sdf), -1.0f);
        float2 *gp = grid + ((size_t)iz * g.R + iy) * g.R + ix;
        const float2 old = *gp;
        const float nx = (old.y * old.x + 1.0f * nt) / (old.y + 1.0f);
        const float ny = fminf(1.0f + old.y, 16.0f);
        if (__float_as_uint(nx) != __float_as_uint(old.x) || __float_as_uint(ny) != __float_as_uint(old.y)) {
            *gp = make_float2(nx, ny);
            n_changed++;
        }
        if (nx < 0.0f) mark_negative(flags, g, ix, iy, iz);
    }
    if (kCount) {
        n_proj = __reduce_add_sync(0xffffffffu, n_proj);
        n_fused = __reduce_add_sync(0xffffffffu, n_fused);
        n_changed = __reduce_add_sync(0xffffffffu, n_changed);
        if (lane == 0) {
            atomicAdd(&counts[0], (unsigned long long)n_proj);
            atomicAdd(&counts[1], (unsigned long long)n_fused);
            atomicAdd(&counts[2], (unsigned long long)n_changed);
        }
    }
}

// -------------------------------------------------------------- ray cast --

// trilinearDensity / trilinearWeight (VoxelGrid_cuda.cu:181-260) at q (voxel
// units), channel ch; false when a corner lies past the end of the array
__device__ __forceinline__ bool trilinear(const float2 *__restrict__ grid, const Geom &g, float qx, float qy,
                                          float qz, int ch, float *out) {
    const unsigned ix = f2u(qx), iy = f2u(qy), iz = f2u(qz);
    const float fx = qx - (float)ix, fy = qy - (float)iy, fz = qz - (float)iz;
    const size_t ys = (size_t)g.R, zs = ys * g.R;
    const size_t o = (size_t)ix + (size_t)iy * ys + (size_t)iz * zs;
    if (o + 1 + ys + zs >= zs * g.R) return false;
    const float *f = reinterpret_cast<const float *>(grid) + ch;
    const float d000 = __ldg(f + 2 * o);
    const float d001 = __ldg(f + 2 * (o + zs));
    const float d010 = __ldg(f + 2 * (o + ys));
    const float d011 = __ldg(f + 2 * (o + ys + zs));
    const float d100 = __ldg(f + 2 * (o + 1));
    const float d101 = __ldg(f + 2 * (o + 1 + zs));
    const float d110 = __ldg(f + 2 * (o + 1 + ys));
    const float d111 = __ldg(f + 2 * (o + 1 + ys + zs));
    const float x00 = (1 - fx) * d000 + fx * d100;
    const float x01 = (1 - fx) * d001 + fx * d101;
    const float x10 = (1 - fx) * d010 + fx * d110;
    const float x11 = (1 - fx) * d011 + fx * d111;
    const float z0 = (1 - fy) * x00 + fy * x10;
    const float z1 = (1 - fy) * x01 + fy * x11;
    *out = (1 - fz) * z0 + fz * z1;
    return true;
}

// estimateLinearZero (VoxelGrid_cuda.cu:553-557)
__device__ __forceinline__ float linear_zero(float tA, float dA, float tB, float dB) {
    const float s = fmaxf(0.0f, fminf(dA / (dA - dB), 1.0f));
    return tA + s * (tB - tA);
}

struct Ray {
    float ox, oy, oz, dx, dy, dz;
};

__device__ __forceinline__ bool sample(const float2 *__restrict__ grid, const Geom &g, const Ray &r, float ivx,
                                       float ivy, float ivz, float t, float *out) {
    return trilinear(grid, g, (r.ox + t * r.dx - g.ib0x) * ivx, (r.oy + t * r.dy - g.ib0y) * ivy,
                     (r.oz + t * r.dz - g.ib0z) * ivz, 0, out);
}

// 2: the voxel's 32^3 super brick holds no negative value; 1: its 8^3 brick
// holds none; 0: the voxel may be negative, or lies outside [0, R)^3 (where
// the reference's flattened index wraps into the next row or slice)
__device__ __forceinline__ int empty_level(const uint8_t *__restrict__ flags, const Geom &g, int x, int y, int z) {
    const unsigned R = (unsigned)g.R;
    if (!((unsigned)x < R && (unsigned)y < R && (unsigned)z < R)) return 0;
    if (__ldg(flags + super_of(g, x, y, z)) == 0) return 2;
    return __ldg(flags + brick_of(g, x, y, z)) == 0 ? 1 : 0;
}

// traverseVoxelsCuda's fine search once the coarse test passed
// (VoxelGrid_cuda.cu:674-704): 1 hit, 0 no hit (the traversal ends), 2 the
// trilinear value at the voxel is not negative (the traversal goes on)
__device__ __forceinline__ int refine(const float2 *__restrict__ grid, const Geom &g, const Ray &r, float ivx,
                                      float ivy, float ivz, float vpx, float vpy, float vpz, float enterT,
                                      float exitT, int iter, int max_back, float *t_hit) {
    const float dv = (vpx - r.ox) * r.dx + (vpy - r.oy) * r.dy + (vpz - r.oz) * r.dz;
    float t1 = fmaxf(enterT, fminf(dv, exitT));
    float e1;
    if (!sample(grid, g, r, ivx, ivy, ivz, t1, &e1)) return 0;
    if (!(e1 < 0.0f)) return 2;
    float t0 = t1 - g.vx2 / 2;
    int back = 0;
    while (t0 > enterT) {
        if (++back > max_back) return 0;
        float e0;
        if (!sample(grid, g, r, ivx, ivy, ivz, t0, &e0)) return 0;
        if (e0 > 0.0f) {
            float tx = linear_zero(t0, e0, t1, e1);
            while (iter > 0) {
                float ex;
                if (!sample(grid, g, r, ivx, ivy, ivz, tx, &ex)) return 0;
                if (ex < 0.0f) {
                    t1 = tx;
                    e1 = ex;
                } else {
                    t0 = tx;
                    e0 = ex;
                }
                tx = linear_zero(t0, e0, t1, e1);
                iter--;
            }
            *t_hit = tx;
            return 1;
        } else if (e0 > e1) {
            t1 = t0;
            e1 = e0;
        }
        t0 -= g.vx2 * 0.5f;
    }
    return 0;
}

// One axis of the voxel walk: the next plane-crossing time and its step, the
// voxel corner coordinate and its step, the voxel index and its direction.
struct Axis {
    float tn, ts, vp, gs;
    int c, d;
    __device__ __forceinline__ void step() {
        tn += ts;
        vp += gs;
        c = max(c + d, 0);
    }
    // events of this axis before the one that leaves the current S-block
    // (S = 8 or 32, the block also ending at R); -1 when no event leaves it
    // (the index saturates at 0 in block 0)
    __device__ __forceinline__ int to_boundary(int S, int R) const {
        return d > 0 ? min(S - 1 - (c & (S - 1)), R - 1 - c) : (c >= S ? (c & (S - 1)) : -1);
    }
    // the time of the event after b more events: the same additions as b steps
    __device__ __forceinline__ float time_after(int b) const {
        float T = tn;
        for (int i = 0; i < b; i++) T += ts;
        return T;
    }
};

// traverseVoxelsCuda (VoxelGrid_cuda.cu:628-730).  The voxel coordinates are
// kept as ints: the reference steps them with `uint += float` by +-1, which
// for coordinates below 2^24 is an integer step that saturates at 0.
//
// The reference's walk is a merge of three per-axis event sequences (plane
// crossings at tn, tn + ts, ...; each value depends only on how many steps its
// own axis took): at every step it takes the axis with the smallest tn, ties
// going to z, then y, then x.  So the order of all events is the order of
// (time, z < y < x).  A block of voxels (a 32^3 super brick or an 8^3 brick)
// that holds no negative value is crossed axis by axis: the event that leaves
// the block is the smallest (time, axis) among the three axes' boundary
// events, and each axis takes exactly its events ordered before that one --
// the same float additions in the same order as the reference's walk, and no
// grid reads.  The boundary times are first estimated with one rounding; only
// the axes whose estimate may be the smallest are summed exactly.  Other
// voxels (blocks that may hold a negative value, voxels outside [0, R)^3) are
// visited one by one, as the reference does.
__device__ bool traverse(const float2 *__restrict__ grid, const uint8_t *__restrict__ flags, const Geom &g,
                         const Ray &r, float idx, float idy, float idz, int s0, int s1, int s2, float enterT,
                         float exitT, int iter, float *t_hit) {
    const float vdx = g.vx2, vdy = g.vy2, vdz = g.vz2;
    enterT += vdx * 2;
    exitT -= vdx * 2;
    if (enterT < 0) enterT = 0;
    if (enterT + vdx * 2 > exitT) return false;
    const float ivx = g.ivx, ivy = g.ivy, ivz = g.ivz;
    const unsigned vx = f2u((r.ox + enterT * r.dx - g.ib0x) * ivx);
    const unsigned vy = f2u((r.oy + enterT * r.dy - g.ib0y) * ivy);
    const unsigned vz = f2u((r.oz + enterT * r.dz - g.ib0z) * ivz);
    // the start point lies in the grid box, so its voxel is in [0, R]^3
    if (vx > (unsigned)g.R + 1 || vy > (unsigned)g.R + 1 || vz > (unsigned)g.R + 1) return false;
    Axis X, Y, Z;
    X.vp = g.ib0x + (float)vx * vdx;
    Y.vp = g.ib0y + (float)vy * vdy;
    Z.vp = g.ib0z + (float)vz * vdz;
    const float sgx = (float)(1 - 2 * s0), sgy = (float)(1 - 2 * s1), sgz = (float)(1 - 2 * s2);
    X.gs = sgx * vdx;
    Y.gs = sgy * vdy;
    Z.gs = sgz * vdz;
    X.tn = (X.vp + X.gs - r.ox) * idx;
    Y.tn = (Y.vp + Y.gs - r.oy) * idy;
    Z.tn = (Z.vp + Z.gs - r.oz) * idz;
    X.ts = X.gs * idx;
    Y.ts = Y.gs * idy;
    Z.ts = Z.gs * idz;
    X.d = 1 - 2 * s0;
    Y.d = 1 - 2 * s1;
    Z.d = 1 - 2 * s2;
    X.c = (int)vx;
    Y.c = (int)vy;
    Z.c = (int)vz;
    const size_t R = (size_t)g.R, RR = R * R, nvox = RR * R;
    const float *gx = reinterpret_cast<const float *>(grid);
    // a ray crosses at most R + 2 voxel planes per axis inside the grid and
    // the fine search steps back at most 4R + 4 half voxels; the caps end the
    // loops only where float steps stall (a grid far from the origin with tiny
    // voxels), where the reference's loops would not end
    const int max_steps = 3 * g.R + 16, max_back = 4 * g.R + 16;
    const float inf = __int_as_float(0x7f800000);
    int steps = 0;
    int lvl = empty_level(flags, g, X.c, Y.c, Z.c);
    float t = enterT;
    while (t < exitT) {
        if (lvl > 0) {
            const int S = lvl == 2 ? 32 : 8;
            const int bx = X.to_boundary(S, g.R), by = Y.to_boundary(S, g.R), bz = Z.to_boundary(S, g.R);
            if (bx >= 0 || by >= 0 || bz >= 0) {
                // estimates E (one rounding) and bounds on their distance from
                // the exact sums: b + 1 roundings of at most 2^-24 of the
                // partial sums, taken four times over.  A NaN estimate (0 x inf)
                // fails every comparison and is summed exactly.
                const float Ex = bx >= 0 ? __fmaf_rn((float)bx, X.ts, X.tn) : inf;
                const float Ey = by >= 0 ? __fmaf_rn((float)by, Y.ts, Y.tn) : inf;
                const float Ez = bz >= 0 ? __fmaf_rn((float)bz, Z.ts, Z.tn) : inf;
                const float ex = (float)(bx + 2) * 2.384185791e-7f * (fabsf(X.tn) + fabsf(Ex)) + 1e-30f;
                const float ey = (float)(by + 2) * 2.384185791e-7f * (fabsf(Y.tn) + fabsf(Ey)) + 1e-30f;
                const float ez = (float)(bz + 2) * 2.384185791e-7f * (fabsf(Z.tn) + fabsf(Ez)) + 1e-30f;
                float thr = inf;
                if (bx >= 0) thr = fminf(thr, Ex + ex);
                if (by >= 0) thr = fminf(thr, Ey + ey);
                if (bz >= 0) thr = fminf(thr, Ez + ez);
                // exact boundary times of the candidates; the first in (time, z < y < x) order
                int ea = -1;
                float Te = 0.0f;
                if (bz >= 0 && !(Ez - ez > thr)) {
                    ea = 2;
                    Te = Z.time_after(bz);
                }
                if (by >= 0 && !(Ey - ey > thr)) {
                    const float Ty = Y.time_after(by);
                    if (ea < 0 || Ty < Te) {
                        ea = 1;
                        Te = Ty;
                    }
                }
                if (bx >= 0 && !(Ex - ex > thr)) {
                    const float Tx = X.time_after(bx);
                    if (ea < 0 || Tx < Te) {
                        ea = 0;
                        Te = Tx;
                    }
                }
                // the walk ends inside this block: nothing can be hit there
                if (!(Te < exitT)) return false;
                int nx = 0, ny = 0, nz = 0;
                if (ea == 0) {
                    nx = bx + 1;
                    for (int i = 0; i < nx; i++) {
                        X.tn += X.ts;
                        X.vp += X.gs;
                    }
                } else {
                    while (X.tn < Te && nx <= max_steps) {
                        X.tn += X.ts;
                        X.vp += X.gs;
                        nx++;
                    }
                }
                if (ea == 1) {
                    ny = by + 1;
                    for (int i = 0; i < ny; i++) {
                        Y.tn += Y.ts;
                        Y.vp += Y.gs;
                    }
                } else {
                    // y before x at equal times
                    while ((Y.tn < Te || (Y.tn == Te && ea == 0)) && ny <= max_steps) {
                        Y.tn += Y.ts;
                        Y.vp += Y.gs;
                        ny++;
                    }
                }
                if (ea == 2) {
                    nz = bz + 1;
                    for (int i = 0; i < nz; i++) {
                        Z.tn += Z.ts;
                        Z.vp += Z.gs;
                    }
                } else {
                    // z before x and y at equal times
                    while (Z.tn <= Te && nz <= max_steps) {
                        Z.tn += Z.ts;
                        Z.vp += Z.gs;
                        nz++;
                    }
                }
                X.c = max(X.c + X.d * nx, 0);
                Y.c = max(Y.c + Y.d * ny, 0);
                Z.c = max(Z.c + Z.d * nz, 0);
                steps += nx + ny + nz;
                if (steps > max_steps) return false;
                t = Te;
                lvl = empty_level(flags, g, X.c, Y.c, Z.c);
                continue;
            }
        }
        if (++steps > max_steps) return false;
        if (lvl == 0) {
            const size_t off = (size_t)X.c + (size_t)Y.c * R + (size_t)Z.c * RR;
            if (off >= nvox) return false;
            if (__ldg(gx + 2 * off) < 0.0f) {
                const int rr =
                    refine(grid, g, r, ivx, ivy, ivz, X.vp, Y.vp, Z.vp, enterT, exitT, iter, max_back, t_hit);
                if (rr != 2) return rr == 1;
            }
        }
        // one event of the reference's walk (x when tnx < tny and tnx < tnz,
        // y when tny <= tnx and tny < tnz, else z)
        const int ox = X.c, oy = Y.c, oz = Z.c;
        if (X.tn < Y.tn) {
            if (X.tn < Z.tn) {
                t = X.tn;
                X.step();
            } else {
                t = Z.tn;
                Z.step();
            }
        } else {
            if (Y.tn < Z.tn) {
                t = Y.tn;
                Y.step();
            } else {
                t = Z.tn;
                Z.step();
            }
        }
        if (((ox ^ X.c) | (oy ^ Y.c) | (oz ^ Z.c)) >> 3) lvl = empty_level(flags, g, X.c, Y.c, Z.c);
    }
    return false;
}

// rayCastVoxelsKernel (VoxelGrid_cuda.cu:734-770) with initRay (118-141) and
// intersectVoxelGridCuda (144-163); g.T = camera -> world
__global__ void __launch_bounds__(kRayTileX * kRayTileY, 32)
    k_raycast(const float2 *__restrict__ grid, const uint8_t *__restrict__ flags, Geom g, int iter,
              float4 *__restrict__ xyz) {
    const int xi = blockIdx.x * kRayTileX + (threadIdx.x % kRayTileX);
    const int yi = blockIdx.y * kRayTileY + (threadIdx.x / kRayTileX);
    if (xi >= g.W || yi >= g.H) return;
    const float pdx = (float)xi / g.Wf, pdy = (float)yi / g.Hf;
    float cx = -(pdx - g.K2) / g.K0, cy = -(pdy - g.K5) / g.K4, cz = -1;
    float len = 0.0f;
    len += cx * cx;
    len += cy * cy;
    len += cz * cz;
    len = 1.0f / sqrtf(len);
    cx *= len;
    cy *= len;
    cz *= len;
    Ray r;
    r.dx = g.T[0] * cx + g.T[1] * cy + g.T[2] * cz;
    r.dy = g.T[4] * cx + g.T[5] * cy + g.T[6] * cz;
    r.dz = g.T[8] * cx + g.T[9] * cy + g.T[10] * cz;
    r.ox = g.T[3];
    r.oy = g.T[7];
    r.oz = g.T[11];
    const int s0 = r.dx < 0, s1 = r.dy < 0, s2 = r.dz < 0;
    const float idx = (fabsf(r.dx) > 1e-6f) ? 1.0f / r.dx : (float)(1 - 2 * s0) * FLT_MAX;
    const float idy = (fabsf(r.dy) > 1e-6f) ? 1.0f / r.dy : (float)(1 - 2 * s1) * FLT_MAX;
    const float idz = (fabsf(r.dz) > 1e-6f) ? 1.0f / r.dz : (float)(1 - 2 * s2) * FLT_MAX;
    const float x0 = ((s0 ? g.b1x : g.b0x) - r.ox) * idx, x1 = ((s0 ? g.b0x : g.b1x) - r.ox) * idx;
    const float y0 = ((s1 ? g.b1y : g.b0y) - r.oy) * idy, y1 = ((s1 ? g.b0y : g.b1y) - r.oy) * idy;
    const float z0 = ((s2 ? g.b1z : g.b0z) - r.oz) * idz, z1 = ((s2 ? g.b0z : g.b1z) - r.oz) * idz;
    const float tmin = fmaxf(x0, fmaxf(y0, z0));
    const float tmax = fminf(x1, fminf(y1, z1));
    float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float th;
    if (!(tmin >= tmax || tmax <= 0) && traverse(grid, flags, g, r, idx, idy, idz, s0, s1, s2, tmin, tmax, iter, &th))
        out = make_float4(th * cx, th * cy, th * cz, (th > g.min_dist && th < g.max_dist) ? 1.0f : 0.0f);
    xyz[(size_t)yi * g.W + xi] = out;
}

// shadingKernel (VoxelGrid_cuda.cu:844-891) with filter3 (772-789)
__global__ void k_shade(const float4 *__restrict__ xyz, int W, int H, float4 *__restrict__ shaded,
                        float4 *__restrict__ normal) {
    const int xi = blockIdx.x * blockDim.x + threadIdx.x, yi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi >= W || yi >= H) return;
    const size_t off = (size_t)yi * W + xi;
    float4 pix = make_float4(0.0f, 0.0f, 0.0f, 1.0f), nrm = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (xi < W - 3 && yi < H - 3 && xi >= 3 && yi >= 3) {
        const float4 p1x = xyz[off + 1], p0x = xyz[off - 1], p1y = xyz[off + W], p0y = xyz[off - W];
        if (p1x.w > 0.0f && p0x.w > 0.0f && p1y.w > 0.0f && p0y.w > 0.0f) {
            const float ux = p1x.x - p0x.x, uy = p1x.y - p0x.y, uz = p1x.z - p0x.z;
            const float vx = p0y.x - p1y.x, vy = p0y.y - p1y.y, vz = p0y.z - p1y.z;
            float nx = uy * vz - uz * vy;
            float ny = -(ux * vz - uz * vx);
            float nz = ux * vy - uy * vx;
            float len = 0.0f;
            len += nx * nx;
            len += ny * ny;
            len += nz * nz;
            len = 1.0f / sqrtf(len);
            nx *= len;
            ny *= len;
            nz *= len;
            const float color = nx * 0.0f + ny * 0.0f + nz * 1.0f;
            if (color > 0.0f) {
                pix = make_float4(color, color, color, 1.0f);
                nrm = make_float4(nx, ny, nz, 0.0f);
            }
        }
    }
    shaded[off] = pix;
    normal[off] = nrm;
}

// ------------------------------------------------- grid and measurement --

// resetKernel (VoxelGrid_cuda.cu:113-118) with (1, 0): two voxels per store
__global__ void k_reset(float4 *__restrict__ grid2, size_t n2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x)
        grid2[i] = make_float4(1.0f, 0.0f, 1.0f, 0.0f);
}

// the brick bytes of a grid given as a whole (after a copy-in or a resample)
__global__ void k_flags(const float2 *__restrict__ grid, uint8_t *__restrict__ flags, Geom g) {
    const size_t n = (size_t)g.R * g.R * g.R;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (grid[i].x < 0.0f) {
            const unsigned x = (unsigned)(i % g.R), y = (unsigned)((i / g.R) % g.R), z = (unsigned)(i / ((size_t)g.R * g.R));
            mark_negative(flags, g, x, y, z);
        }
}

// reconstructionKernel (VoxelGrid_cuda.cu:1090-1112): rows of the RGB-D
// frame are stored bottom-up
__global__ void k_dist_rgbd(const float4 *__restrict__ rgbd, int W, int H, float min_dist, float max_dist,
                            float *__restrict__ dist) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const float tol = 1e-4f;
    const float w = rgbd[(size_t)(H - 1 - y) * W + x].w;
    dist[(size_t)y * W + x] = (w > tol && w < (1.0f - tol)) ? w * (max_dist - min_dist) + min_dist : 0.0f;
}

__global__ void k_dist_depth16(const uint16_t *__restrict__ depth, size_t n, float *__restrict__ dist) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dist[i] = (float)depth[i];
}

// resampleVoxelsKernel (VoxelGrid_cuda.cu:896-941); g.T = camera -> world
__global__ void k_resample(float2 *__restrict__ dst, const float2 *__restrict__ src, Geom g) {
    const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y, iz = blockIdx.z;
    if (ix >= g.R) return;
    const float px = g.sx + (float)ix * g.vx2, py = g.sy + (float)iy * g.vy2, pz = g.sz + (float)iz * g.vz2;
    const float rx = g.T[0] * px + g.T[1] * py + g.T[2] * pz + g.T[3];
    const float ry = g.T[4] * px + g.T[5] * py + g.T[6] * pz + g.T[7];
    const float rz = g.T[8] * px + g.T[9] * py + g.T[10] * pz + g.T[11];
    const float qx = (rx - g.sx) / g.vx2, qy = (ry - g.sy) / g.vy2, qz = (rz - g.sz) / g.vz2;
    const float hi = (float)(g.R - 2);
    const bool oob = (qx < 0 || qx > hi) || (qy < 0 || qy > hi) || (qz < 0 || qz > hi);
    float2 v = make_float2(1.0f, 0.0f);
    float d, w;
    if (!oob && trilinear(src, g, qx, qy, qz, 0, &d) && trilinear(src, g, qx, qy, qz, 1, &w)) v = make_float2(d, w);
    dst[((size_t)iz * g.R + iy) * g.R + ix] = v;
}

}  // namespace tsdf

// ================================================================= host ==

using namespace tsdf;

struct recon_tsdf {
    recon_tsdf_params p{};
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    float2 *grid = nullptr;
    uint8_t *flags = nullptr;
    float *dist = nullptr;
    float4 *xyz = nullptr, *shaded = nullptr, *normal = nullptr;
    void *staging = nullptr;  // device copy of a host measurement (uint16 or float4 frame)
    size_t staging_bytes = 0;
    unsigned long long *counts = nullptr;
    bool counting = false;
    bool timing = false;
    double ms[kKinds] = {};
    int64_t launches[kKinds] = {};
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    std::vector<cudaEvent_t> spare;
};

namespace {

int fail(int code, const char *msg) {
    rt::set_last_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char *where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    rt::set_last_error(m.c_str());
    return RECON_ERR_CUDA;
}

#define TCK(call)                                            \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
    } while (0)

size_t n_voxels(const recon_tsdf_params &p) {
    return (size_t)p.grid_resolution * p.grid_resolution * p.grid_resolution;
}
size_t n_bricks(const recon_tsdf_params &p) {
    const size_t b = (size_t)p.grid_resolution / kBrick;
    return b * b * b;
}
// the flag bytes: one per 8^3 brick, then one per 32^3 super brick
size_t n_flag_bytes(const recon_tsdf_params &p) {
    const size_t sb = ((size_t)p.grid_resolution + 31) / 32;
    return n_bricks(p) + sb * sb * sb;
}
size_t n_pixels(const recon_tsdf_params &p) { return (size_t)p.width * p.height; }

// invertRT4 (basic_math.cpp:355-368): VoxelGrid::setCameraParams's world ->
// camera pose, in float, translation summed left to right
void invert_rt4(const float *M, float *Mi) {
    Mi[0] = M[0]; Mi[1] = M[4]; Mi[2] = M[8];
    Mi[3] = -(M[0] * M[3] + M[4] * M[7] + M[8] * M[11]);
    Mi[4] = M[1]; Mi[5] = M[5]; Mi[6] = M[9];
    Mi[7] = -(M[1] * M[3] + M[5] * M[7] + M[9] * M[11]);
    Mi[8] = M[2]; Mi[9] = M[6]; Mi[10] = M[10];
    Mi[11] = -(M[2] * M[3] + M[6] * M[7] + M[10] * M[11]);
    Mi[12] = 0; Mi[13] = 0; Mi[14] = 0; Mi[15] = 1;
}

// the launch constants of SimParams (VoxelGrid.cpp:48-106; kernel prologues
// VoxelGrid_cuda.cu:745-756, 957-965): T3x4 is the first three rows of the
// pose the kernel uses
Geom make_geom(const recon_tsdf_params &p, const float *T3x4, const float *K) {
    Geom g;
    memset(&g, 0, sizeof(g));
    const int R = p.grid_resolution;
    g.R = R;
    g.B = R / kBrick;
    g.SB = (R + 31) / 32;
    g.nb = g.B * g.B * g.B;
    g.W = p.width;
    g.H = p.height;
    if (T3x4) memcpy(g.T, T3x4, sizeof(g.T));
    if (K) {
        g.K0 = K[0];
        g.K2 = K[2];
        g.K4 = K[4];
        g.K5 = K[5];
    }
    g.Wf = (float)p.width;
    g.Hf = (float)p.height;
    g.Wm2 = (float)(p.width - 2);
    g.Hm2 = (float)(p.height - 2);
    const float vsx = p.cube_dim[0] / (float)R, vsy = p.cube_dim[1] / (float)R, vsz = p.cube_dim[2] / (float)R;
    g.sx = p.cube_origin[0] - p.cube_dim[0] + vsx;
    g.sy = p.cube_origin[1] - p.cube_dim[1] + vsy;
    g.sz = p.cube_origin[2] - p.cube_dim[2] + vsz;
    g.vx2 = vsx * 2;
    g.vy2 = vsy * 2;
    g.vz2 = vsz * 2;
    g.lim = vsx * 2;
    g.tol = p.cube_dim[0] / 200.0f;
    g.slope = p.cube_dim[0] * 0.030f;
    g.b0x = p.cube_origin[0] - p.cube_dim[0];
    g.b0y = p.cube_origin[1] - p.cube_dim[1];
    g.b0z = p.cube_origin[2] - p.cube_dim[2];
    g.b1x = p.cube_origin[0] + p.cube_dim[0];
    g.b1y = p.cube_origin[1] + p.cube_dim[1];
    g.b1z = p.cube_origin[2] + p.cube_dim[2];
    g.ib0x = g.b0x + vsx;
    g.ib0y = g.b0y + vsy;
    g.ib0z = g.b0z + vsz;
    // 2.0f * voxelSize (VoxelGrid_cuda.cu:753) equals vs * 2
    g.ivx = 1.0f / g.vx2;
    g.ivy = 1.0f / g.vy2;
    g.ivz = 1.0f / g.vz2;
    g.min_dist = p.min_dist;
    g.max_dist = p.max_dist;
    return g;
}

struct Timed {
    recon_tsdf *v;
    int kind;
    cudaEvent_t a = nullptr, b = nullptr;
    Timed(recon_tsdf *v_, int kind_) : v(v_), kind(kind_) {
        if (!v->timing) return;
        for (cudaEvent_t *e : {&a, &b}) {
            if (!v->spare.empty()) {
                *e = v->spare.back();
                v->spare.pop_back();
            } else if (cudaEventCreate(e) != cudaSuccess) {
                *e = nullptr;
            }
        }
        if (a) cudaEventRecord(a, v->stream);
    }
    ~Timed() {
        if (!v->timing || !a || !b) return;
        cudaEventRecord(b, v->stream);
        v->pending.push_back({kind, {a, b}});
    }
};

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
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    rt::add_launches(1);
    return RECON_OK;
}

int check_pose(const float *T, const float *K) {
    if (!T) return fail(RECON_ERR_INVALID_ARG, "pose is NULL");
    for (int i = 0; i < 16; i++)
        if (!std::isfinite(T[i])) return fail(RECON_ERR_INVALID_ARG, "pose is not finite");
    if (K) {
        for (int i = 0; i < 9; i++)
            if (!std::isfinite(K[i])) return fail(RECON_ERR_INVALID_ARG, "K is not finite");
        if (K[0] == 0.0f || K[4] == 0.0f) return fail(RECON_ERR_INVALID_ARG, "K has a zero focal length");
    }
    return RECON_OK;
}

int ensure_staging(recon_tsdf *v, size_t bytes) {
    if (v->staging_bytes >= bytes) return RECON_OK;
    if (v->staging) {
        TCK(cudaStreamSynchronize(v->stream));
        cudaFree(v->staging);
        v->staging = nullptr;
        v->staging_bytes = 0;
    }
    TCK(cudaMalloc(&v->staging, bytes));
    v->staging_bytes = bytes;
    return RECON_OK;
}

int rebuild_flags(recon_tsdf *v, float2 *grid, uint8_t *flags) {
    TCK(cudaMemsetAsync(flags, 0, n_flag_bytes(v->p), v->stream));
    Geom g = make_geom(v->p, nullptr, nullptr);
    return launch(k_flags, dim3(1216), dim3(256), v->stream, grid, flags, g);
}

}  // namespace

extern "C" {

void recon_tsdf_default_params(int32_t grid_resolution, int32_t width, int32_t height, float min_dist,
                               float max_dist, recon_tsdf_params *out) {
    if (!out) return;
    memset(out, 0, sizeof(*out));
    out->grid_resolution = grid_resolution;
    out->cube_origin[0] = 0.0f;
    out->cube_origin[1] = 0.01f;
    out->cube_origin[2] = -1600.01f;
    out->cube_dim[0] = out->cube_dim[1] = out->cube_dim[2] = 1500.0f;
    out->width = width;
    out->height = height;
    out->min_dist = min_dist;
    out->max_dist = max_dist;
}

int recon_tsdf_create(const recon_tsdf_params *p, void *stream, recon_tsdf **out) {
    if (!p || !out) return fail(RECON_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    const int R = p->grid_resolution;
    if (R < 8 || R % kBrick || R > 2048) return fail(RECON_ERR_INVALID_ARG, "grid_resolution must be a multiple of 8 in 8..2048");
    if (p->width < 8 || p->height < 8 || p->width > 16384 || p->height > 16384)
        return fail(RECON_ERR_INVALID_ARG, "image size must be 8..16384");
    for (int i = 0; i < 3; i++) {
        if (!(p->cube_dim[i] > 0.0f) || !std::isfinite(p->cube_dim[i]) || !std::isfinite(p->cube_origin[i]))
            return fail(RECON_ERR_INVALID_ARG, "cube_dim must be positive and finite");
    }
    if (!(p->min_dist >= 0.0f && p->max_dist > p->min_dist)) return fail(RECON_ERR_INVALID_ARG, "need 0 <= min_dist < max_dist");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        (void)cudaGetLastError();  // this call's own error
        return fail(RECON_ERR_NO_DEVICE, "no CUDA device");
    }
    recon_tsdf *v = new recon_tsdf();
    v->p = *p;
    cudaGetDevice(&v->device);
    int rc = RECON_OK;
    auto alloc = [&](void **ptr, size_t bytes) {
        if (rc != RECON_OK) return;
        cudaError_t e = cudaMalloc(ptr, bytes);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc");
    };
    if (stream) {
        v->stream = (cudaStream_t)stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&v->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamCreate");
        v->own_stream = rc == RECON_OK;
    }
    alloc((void **)&v->grid, n_voxels(*p) * sizeof(float2));
    alloc((void **)&v->flags, n_flag_bytes(*p));
    alloc((void **)&v->dist, n_pixels(*p) * sizeof(float));
    alloc((void **)&v->xyz, n_pixels(*p) * sizeof(float4));
    alloc((void **)&v->shaded, n_pixels(*p) * sizeof(float4));
    alloc((void **)&v->normal, n_pixels(*p) * sizeof(float4));
    alloc((void **)&v->counts, 4 * sizeof(unsigned long long));
    if (rc == RECON_OK) {
        cudaMemsetAsync(v->dist, 0, n_pixels(*p) * sizeof(float), v->stream);
        cudaMemsetAsync(v->xyz, 0, n_pixels(*p) * sizeof(float4), v->stream);
        cudaMemsetAsync(v->shaded, 0, n_pixels(*p) * sizeof(float4), v->stream);
        cudaMemsetAsync(v->normal, 0, n_pixels(*p) * sizeof(float4), v->stream);
        cudaMemsetAsync(v->counts, 0, 4 * sizeof(unsigned long long), v->stream);
        rc = recon_tsdf_reset(v);
    }
    if (rc != RECON_OK) {
        recon_tsdf_destroy(v);
        return rc;
    }
    *out = v;
    return RECON_OK;
}

int recon_tsdf_destroy(recon_tsdf *v) {
    if (!v) return RECON_OK;
    if (v->stream) cudaStreamSynchronize(v->stream);
    for (auto &pe : v->pending) {
        cudaEventDestroy(pe.second.first);
        cudaEventDestroy(pe.second.second);
    }
    for (cudaEvent_t e : v->spare) cudaEventDestroy(e);
    cudaFree(v->grid);
    cudaFree(v->flags);
    cudaFree(v->dist);
    cudaFree(v->xyz);
    cudaFree(v->shaded);
    cudaFree(v->normal);
    cudaFree(v->staging);
    cudaFree(v->counts);
    if (v->own_stream) cudaStreamDestroy(v->stream);
    delete v;
    return RECON_OK;
}

int recon_tsdf_reset(recon_tsdf *v) {
    if (!v) return fail(RECON_ERR_INVALID_ARG, "NULL grid");
    Timed tm(v, 4);
    TCK(cudaMemsetAsync(v->flags, 0, n_flag_bytes(v->p), v->stream));
    return launch(k_reset, dim3(152 * 8), dim3(256), v->stream, reinterpret_cast<float4 *>(v->grid), n_voxels(v->p) / 2);
}

int recon_tsdf_set_dist_map(recon_tsdf *v, const float *dist, int32_t on_device) {
    if (!v || !dist) return fail(RECON_ERR_INVALID_ARG, "NULL argument");
    TCK(cudaMemcpyAsync(v->dist, dist, n_pixels(v->p) * sizeof(float),
                        on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, v->stream));
    return RECON_OK;
}

int recon_tsdf_set_dist_rgbd_float4(recon_tsdf *v, const float *rgbd, int32_t on_device) {
    if (!v || !rgbd) return fail(RECON_ERR_INVALID_ARG, "NULL argument");
    const float4 *src = reinterpret_cast<const float4 *>(rgbd);
    if (!on_device) {
        int rc = ensure_staging(v, n_pixels(v->p) * sizeof(float4));
        if (rc) return rc;
        TCK(cudaMemcpyAsync(v->staging, rgbd, n_pixels(v->p) * sizeof(float4), cudaMemcpyHostToDevice, v->stream));
        src = reinterpret_cast<const float4 *>(v->staging);
    }
    Timed tm(v, 3);
    dim3 blk(32, 8), grd((v->p.width + 31) / 32, (v->p.height + 7) / 8);
    return launch(k_dist_rgbd, grd, blk, v->stream, src, v->p.width, v->p.height, v->p.min_dist, v->p.max_dist, v->dist);
}

int recon_tsdf_set_dist_depth16(recon_tsdf *v, const uint16_t *depth, int32_t on_device) {
    if (!v || !depth) return fail(RECON_ERR_INVALID_ARG, "NULL argument");
    const uint16_t *src = depth;
    if (!on_device) {
        int rc = ensure_staging(v, n_pixels(v->p) * sizeof(uint16_t));
        if (rc) return rc;
        TCK(cudaMemcpyAsync(v->staging, depth, n_pixels(v->p) * sizeof(uint16_t), cudaMemcpyHostToDevice, v->stream));
        src = reinterpret_cast<const uint16_t *>(v->staging);
    }
    Timed tm(v, 3);
    return launch(k_dist_depth16, dim3((unsigned)((n_pixels(v->p) + 255) / 256)), dim3(256), v->stream, src,
                  n_pixels(v->p), v->dist);
}

int recon_tsdf_update(recon_tsdf *v, const float T[16], const float K[9]) {
    if (!v || !K) return fail(RECON_ERR_INVALID_ARG, "NULL argument");
    int rc = check_pose(T, K);
    if (rc) return rc;
    float Tin[16], Tw2c[16];
    memcpy(Tin, T, sizeof(Tin));
    invert_rt4(Tin, Tw2c);
    Geom g = make_geom(v->p, Tw2c, K);
    const int R = v->p.grid_resolution;
    dim3 grd((R + kTileX - 1) / kTileX, R / kTileY, R / kRunZ);
    Timed tm(v, 0);
    if (v->counting)
        return launch(k_update<true>, grd, dim3(kTileX * kTileY), v->stream, v->grid, v->flags, v->dist, g, v->counts);
    return launch(k_update<false>, grd, dim3(kTileX * kTileY), v->stream, v->grid, v->flags, v->dist, g,
                  (unsigned long long *)nullptr);
}

int recon_tsdf_raycast(recon_tsdf *v, const float T[16], const float K[9], int32_t cubic_filter) {
    if (!v || !K) return fail(RECON_ERR_INVALID_ARG, "NULL argument");
    int rc = check_pose(T, K);
    if (rc) return rc;
    Geom g = make_geom(v->p, T, K);
    dim3 grd((v->p.width + kRayTileX - 1) / kRayTileX, (v->p.height + kRayTileY - 1) / kRayTileY);
    {
        Timed tm(v, 1);
        rc = launch(k_raycast, grd, dim3(kRayTileX * kRayTileY), v->stream, v->grid, v->flags, g, cubic_filter ? 3 : 0,
                    v->xyz);
        if (rc) return rc;
    }
    Timed tm(v, 2);
    dim3 blk(32, 8), grd2((v->p.width + 31) / 32, (v->p.height + 7) / 8);
    return launch(k_shade, grd2, blk, v->stream, v->xyz, v->p.width, v->p.height, v->shaded, v->normal);
}

int recon_tsdf_resample(recon_tsdf *dst, recon_tsdf *src, const float T[16]) {
    if (!dst || !src || dst == src) return fail(RECON_ERR_INVALID_ARG, "need two different grids");
    if (memcmp(&dst->p, &src->p, sizeof(recon_tsdf_params)) != 0)
        return fail(RECON_ERR_INVALID_ARG, "the grids have different parameters");
    int rc = check_pose(T, nullptr);
    if (rc) return rc;
    if (src->stream != dst->stream) {
        cudaEvent_t e;
        TCK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        cudaEventRecord(e, src->stream);
        cudaStreamWaitEvent(dst->stream, e, 0);
        cudaEventDestroy(e);
    }
    Geom g = make_geom(dst->p, T, nullptr);
    const int R = dst->p.grid_resolution;
    {
        Timed tm(dst, 4);
        rc = launch(k_resample, dim3((R + 127) / 128, R, R), dim3(128), dst->stream, dst->grid, src->grid, g);
        if (rc) return rc;
    }
    rc = rebuild_flags(dst, dst->grid, dst->flags);
    if (rc) return rc;
    if (src->stream != dst->stream) {
        // src must not be changed before the resample has read it
        cudaEvent_t e;
        TCK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        cudaEventRecord(e, dst->stream);
        cudaStreamWaitEvent(src->stream, e, 0);
        cudaEventDestroy(e);
    }
    return RECON_OK;
}

void *recon_tsdf_device_array(recon_tsdf *v, const char *name) {
    if (!v || !name) return nullptr;
    if (!strcmp(name, "tsdf")) return v->grid;
    if (!strcmp(name, "dist")) return v->dist;
    if (!strcmp(name, "xyz")) return v->xyz;
    if (!strcmp(name, "shaded")) return v->shaded;
    if (!strcmp(name, "normal")) return v->normal;
    if (!strcmp(name, "flags")) return v->flags;
    return nullptr;
}

int64_t recon_tsdf_get(recon_tsdf *v, const char *name, void *host_dst, int64_t nbytes) {
    if (!v || !name || !host_dst) return fail(RECON_ERR_INVALID_ARG, "NULL argument");
    void *src = recon_tsdf_device_array(v, name);
    if (!src) return fail(RECON_ERR_INVALID_ARG, "unknown array");
    size_t bytes;
    if (!strcmp(name, "tsdf"))
        bytes = n_voxels(v->p) * sizeof(float2);
    else if (!strcmp(name, "dist"))
        bytes = n_pixels(v->p) * sizeof(float);
    else if (!strcmp(name, "flags"))
        bytes = n_bricks(v->p);
    else
        bytes = n_pixels(v->p) * sizeof(float4);
    if ((int64_t)bytes > nbytes) return fail(RECON_ERR_INVALID_ARG, "destination too small");
    TCK(cudaMemcpyAsync(host_dst, src, bytes, cudaMemcpyDeviceToHost, v->stream));
    TCK(cudaStreamSynchronize(v->stream));
    return (int64_t)bytes;
}

int recon_tsdf_set_grid(recon_tsdf *v, const float *grid, int32_t on_device) {
    if (!v || !grid) return fail(RECON_ERR_INVALID_ARG, "NULL argument");
    TCK(cudaMemcpyAsync(v->grid, grid, n_voxels(v->p) * sizeof(float2),
                        on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, v->stream));
    return rebuild_flags(v, v->grid, v->flags);
}

void *recon_tsdf_stream(recon_tsdf *v) { return v ? (void *)v->stream : nullptr; }

int recon_tsdf_enable_timing(recon_tsdf *v, int32_t on) {
    if (!v) return fail(RECON_ERR_INVALID_ARG, "NULL grid");
    v->timing = on != 0;
    return RECON_OK;
}

int recon_tsdf_get_timing(recon_tsdf *v, double ms[5], int64_t launches[5], int32_t reset) {
    if (!v) return fail(RECON_ERR_INVALID_ARG, "NULL grid");
    TCK(cudaStreamSynchronize(v->stream));
    for (auto &pe : v->pending) {
        float t = 0.0f;
        if (cudaEventElapsedTime(&t, pe.second.first, pe.second.second) == cudaSuccess) {
            v->ms[pe.first] += t;
            v->launches[pe.first] += 1;
        }
        v->spare.push_back(pe.second.first);
        v->spare.push_back(pe.second.second);
    }
    v->pending.clear();
    for (int k = 0; k < kKinds; k++) {
        if (ms) ms[k] = v->ms[k];
        if (launches) launches[k] = v->launches[k];
        if (reset) {
            v->ms[k] = 0.0;
            v->launches[k] = 0;
        }
    }
    return RECON_OK;
}

int recon_tsdf_enable_counting(recon_tsdf *v, int32_t on) {
    if (!v) return fail(RECON_ERR_INVALID_ARG, "NULL grid");
    v->counting = on != 0;
    return RECON_OK;
}

int recon_tsdf_get_counts(recon_tsdf *v, int64_t counts[3], int32_t reset) {
    if (!v || !counts) return fail(RECON_ERR_INVALID_ARG, "NULL argument");
    unsigned long long h[4];
    TCK(cudaMemcpyAsync(h, v->counts, sizeof(h), cudaMemcpyDeviceToHost, v->stream));
    TCK(cudaStreamSynchronize(v->stream));
    for (int i = 0; i < 3; i++) counts[i] = (int64_t)h[i];
    if (reset) TCK(cudaMemsetAsync(v->counts, 0, sizeof(h), v->stream));
    return RECON_OK;
}

}  // extern "C"
