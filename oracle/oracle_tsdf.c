/*
 * oracle_tsdf.c -- CPU oracle of the reconstruction stream: TSDF fusion,
 * ray cast, shading, resampling and the distance map of an RGB-D frame.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline).  Each
 * function restates one reference kernel of tracker/kernels/VoxelGrid_cuda.cu
 * (or host routine of tracker/reconstruct/VoxelGrid.cpp) and cites the lines
 * it follows.  FP32 expressions are written in the reference's source order and
 * the library is built with -ffp-contract=off, so every multiply and add is
 * rounded separately, as in the CUDA kernels built with -fmad=false.
 *
 * Conversions follow the GPU: float -> unsigned truncates and saturates
 * (negative and NaN give 0), as make_uint3(float...) and `uint += float` do in
 * the reference's kernels.  Where the reference reads outside the grid array
 * (its bounds checks are commented out: VoxelGrid_cuda.cu:192-195, 658) the
 * ray reports no hit instead; every in-array read is the reference's.  The
 * traversal's loops are capped (3R + 16 voxel steps, 4R + 16 half-voxel steps
 * back): a ray crosses at most R + 2 voxel planes per axis, so the caps only
 * end loops whose float steps stall (a grid far from the origin with tiny
 * voxels), which in the reference would not end.
 *
 * Grid layout: float2 (tsdf, weight) per voxel, x fastest, then y, then z
 * (VoxelGrid_cuda.cu:952, idx = ix + iy*R + iz*R*R).
 */
#include "oracle.h"
#include <float.h>
#include <math.h>
#include <string.h>

typedef struct { float x, y, z; } v3;

/* float -> unsigned as the GPU converts it (cvt.rzi.u32.f32: truncation,
 * saturating; NaN -> 0) */
static inline unsigned f2u(float v) {
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xffffffffu;
    return (unsigned)v;
}

/* invertRT4 (basic_math.cpp:355-368): rigid inverse in float, the
 * translation as -(R^T t) summed left to right */
void orc_tsdf_invert_rt4(const float *M, float *Mi) {
    Mi[0] = M[0]; Mi[1] = M[4]; Mi[2] = M[8];
    Mi[3] = -(M[0] * M[3] + M[4] * M[7] + M[8] * M[11]);
    Mi[4] = M[1]; Mi[5] = M[5]; Mi[6] = M[9];
    Mi[7] = -(M[1] * M[3] + M[5] * M[7] + M[9] * M[11]);
    Mi[8] = M[2]; Mi[9] = M[6]; Mi[10] = M[10];
    Mi[11] = -(M[2] * M[3] + M[6] * M[7] + M[10] * M[11]);
    Mi[12] = 0; Mi[13] = 0; Mi[14] = 0; Mi[15] = 1;
}

/* voxelSize = cubeDim / gridResolution (VoxelGrid.cpp:104) */
static v3 voxel_size(const orc_tsdf_params *p) {
    v3 v = {p->dim[0] / (float)p->R, p->dim[1] / (float)p->R, p->dim[2] / (float)p->R};
    return v;
}

/* resetKernel (VoxelGrid_cuda.cu:113-118) with VoxelGrid::clear's (1, 0) */
void orc_tsdf_reset(float *grid, int64_t nvox) {
    for (int64_t i = 0; i < nvox; i++) {
        grid[2 * i] = 1.0f;
        grid[2 * i + 1] = 0.0f;
    }
}

/* reconstructionKernel (VoxelGrid_cuda.cu:1090-1112): the distance map of a
 * float4 RGB-D frame (w = normalised depth, rows stored bottom-up) */
void orc_tsdf_dist_from_rgbd(const float *rgbd, int W, int H, float min_dist, float max_dist, float *dist) {
    const float tol = 1e-4f;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            float w = rgbd[4 * ((int64_t)(H - 1 - y) * W + x) + 3];
            dist[(int64_t)y * W + x] = (w > tol && w < (1.0f - tol)) ? w * (max_dist - min_dist) + min_dist : 0.0f;
        }
}

/* updateVoxelsKernel (VoxelGrid_cuda.cu:944-1014) for every voxel, with the
 * world -> camera pose invertRT4(Tcur) of VoxelGrid::setCameraParams
 * (VoxelGrid.cpp:266-273).  K: normalised 3x3 intrinsics (main.cpp:878-882). */
void orc_tsdf_update(float *grid, const orc_tsdf_params *p, const float *dist, const float Tcur[16], const float K[9]) {
    float T[16];
    orc_tsdf_invert_rt4(Tcur, T);
    const int R = p->R, W = p->W, H = p->H;
    const v3 vs = voxel_size(p);
    const v3 start = {p->origin[0] - p->dim[0] + vs.x, p->origin[1] - p->dim[1] + vs.y,
                      p->origin[2] - p->dim[2] + vs.z};
    const v3 vs2 = {vs.x * 2, vs.y * 2, vs.z * 2};
    const float lim = vs.x * 2;
    const float tol = p->dim[0] / 200.0f;
    const float slope = p->dim[0] * 0.030f;
#pragma omp parallel for schedule(static)
    for (int iz = 0; iz < R; iz++)
        for (int iy = 0; iy < R; iy++)
            for (int ix = 0; ix < R; ix++) {
                float px = start.x + (float)ix * vs2.x;
                float py = start.y + (float)iy * vs2.y;
                float pz = start.z + (float)iz * vs2.z;
                float rx = T[0] * px + T[1] * py + T[2] * pz + T[3];
                float ry = T[4] * px + T[5] * py + T[6] * pz + T[7];
                float rz = T[8] * px + T[9] * py + T[10] * pz + T[11];
                float voxel_dist = -rz;
                rx /= rz;
                ry /= rz;
                float ux = (rx * K[0] + K[2]) * (float)W;
                float uy = (ry * K[4] + K[5]) * (float)H;
                /* int(u) in [1, W-2): safeBorder 1 (VoxelGrid_cuda.cu:984-985) */
                if (!(ux >= 1.0f && ux < (float)(W - 2) && uy >= 1.0f && uy < (float)(H - 2))) continue;
                int ui = (int)ux, vi = (int)uy;
                int64_t off = ui + (int64_t)vi * W;
                float a = dist[off], b = dist[off + 1], c = dist[off + W], d = dist[off + W + 1];
                if (a < lim || b < lim || c < lim || d < lim) continue;
                float fu = ux - (float)ui;
                float fv = uy - (float)vi;
                float z = (1 - fu) * (1 - fv) * a + fu * (1 - fv) * b + (1 - fu) * fv * c + fu * fv * d;
                if (fabsf(z - a) > tol || fabsf(z - b) > tol || fabsf(z - c) > tol || fabsf(z - d) > tol) continue;
                float sdf = -(voxel_dist - z) / slope;
                if (sdf < -1.25f) continue;
                float nt = fmaxf(fminf(1.0f, sdf), -1.0f);
                float *g = grid + 2 * ((int64_t)ix + (int64_t)iy * R + (int64_t)iz * R * R);
                g[0] = (g[1] * g[0] + 1.0f * nt) / (g[1] + 1.0f);
                g[1] = fminf(1.0f + g[1], 16.0f);
            }
}

/* trilinearDensity / trilinearWeight (VoxelGrid_cuda.cu:181-260); ch = 0 / 1.
 * Returns 0 when a corner lies outside the array (the reference reads past it). */
static int trilinear(const float *grid, int R, v3 q, int ch, float *out) {
    unsigned ix = f2u(q.x), iy = f2u(q.y), iz = f2u(q.z);
    float fx = q.x - (float)ix, fy = q.y - (float)iy, fz = q.z - (float)iz;
    const int64_t ys = R, zs = (int64_t)R * R;
    int64_t o = (int64_t)ix + (int64_t)iy * ys + (int64_t)iz * zs;
    if (o + 1 + ys + zs >= zs * R) return 0;
    float d000 = grid[2 * o + ch];
    float d001 = grid[2 * (o + zs) + ch];
    float d010 = grid[2 * (o + ys) + ch];
    float d011 = grid[2 * (o + ys + zs) + ch];
    float d100 = grid[2 * (o + 1) + ch];
    float d101 = grid[2 * (o + 1 + zs) + ch];
    float d110 = grid[2 * (o + 1 + ys) + ch];
    float d111 = grid[2 * (o + 1 + ys + zs) + ch];
    float x00 = (1 - fx) * d000 + fx * d100;
    float x01 = (1 - fx) * d001 + fx * d101;
    float x10 = (1 - fx) * d010 + fx * d110;
    float x11 = (1 - fx) * d011 + fx * d111;
    float z0 = (1 - fy) * x00 + fy * x10;
    float z1 = (1 - fy) * x01 + fy * x11;
    *out = (1 - fz) * z0 + fz * z1;
    return 1;
}

/* estimateLinearZero (VoxelGrid_cuda.cu:553-557) */
static inline float linear_zero(float tA, float dA, float tB, float dB) {
    float s = fmaxf(0.0f, fminf(dA / (dA - dB), 1.0f));
    return tA + s * (tB - tA);
}

/* sample point of ray parameter t in voxel units: (origin + t*dir - ib0) * inv */
static inline v3 ray_voxel(v3 o, v3 dir, float t, v3 ib0, v3 inv) {
    v3 q = {(o.x + t * dir.x - ib0.x) * inv.x, (o.y + t * dir.y - ib0.y) * inv.y, (o.z + t * dir.z - ib0.z) * inv.z};
    return q;
}

/* traverseVoxelsCuda (VoxelGrid_cuda.cu:628-730).  Returns 1 on a hit. */
static int traverse(const float *grid, int R, v3 o, v3 dir, v3 invdir, const int *sgn, float enterT, float exitT,
                    v3 ib0, v3 vd, int filtering, float *t_hit) {
    enterT += vd.x * 2;
    exitT -= vd.x * 2;
    if (enterT < 0) enterT = 0;
    if (enterT + vd.x * 2 > exitT) return 0;
    /* voxelize (VoxelGrid_cuda.cu:165-179) */
    v3 ivd = {1.0f / vd.x, 1.0f / vd.y, 1.0f / vd.z};
    unsigned vx = f2u((o.x + enterT * dir.x - ib0.x) * ivd.x);
    unsigned vy = f2u((o.y + enterT * dir.y - ib0.y) * ivd.y);
    unsigned vz = f2u((o.z + enterT * dir.z - ib0.z) * ivd.z);
    v3 inv = {1.0f / vd.x, 1.0f / vd.y, 1.0f / vd.z};
    v3 vp = {ib0.x + (float)vx * vd.x, ib0.y + (float)vy * vd.y, ib0.z + (float)vz * vd.z};
    v3 sg = {(float)(1 - 2 * sgn[0]), (float)(1 - 2 * sgn[1]), (float)(1 - 2 * sgn[2])};
    v3 gs = {sg.x * vd.x, sg.y * vd.y, sg.z * vd.z};
    v3 tn = {(vp.x + gs.x - o.x) * invdir.x, (vp.y + gs.y - o.y) * invdir.y, (vp.z + gs.z - o.z) * invdir.z};
    v3 ts = {gs.x * invdir.x, gs.y * invdir.y, gs.z * invdir.z};
    int iter = filtering ? 3 : 0;
    const int64_t nvox = (int64_t)R * R * R;
    /* step caps: never reached unless float steps stall (see the header) */
    const int max_steps = 3 * R + 16, max_back = 4 * R + 16;
    int steps = 0;
    float t = enterT;
    while (t < exitT) {
        int64_t off = (int64_t)vx + (int64_t)vy * R + (int64_t)vz * R * R;
        if (off >= nvox || ++steps > max_steps) return 0;
        if (grid[2 * off] < 0.0f) {
            float dv = (vp.x - o.x) * dir.x + (vp.y - o.y) * dir.y + (vp.z - o.z) * dir.z;
            float t1 = fmaxf(enterT, fminf(dv, exitT));
            float e1;
            if (!trilinear(grid, R, ray_voxel(o, dir, t1, ib0, inv), 0, &e1)) return 0;
            if (e1 < 0.0f) {
                float t0 = t1 - vd.x / 2;
                int back = 0;
                while (t0 > enterT) {
                    if (++back > max_back) return 0;
                    float e0;
                    if (!trilinear(grid, R, ray_voxel(o, dir, t0, ib0, inv), 0, &e0)) return 0;
                    if (e0 > 0.0f) {
                        float tx = linear_zero(t0, e0, t1, e1);
                        while (iter > 0) {
                            float ex;
                            if (!trilinear(grid, R, ray_voxel(o, dir, tx, ib0, inv), 0, &ex)) return 0;
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
                    t0 -= vd.x * 0.5f;
                }
                return 0;
            }
        }
        if (tn.x < tn.y) {
            if (tn.x < tn.z) {
                t = tn.x; vp.x += gs.x; vx = f2u((float)vx + sg.x); tn.x += ts.x;
            } else {
                t = tn.z; vp.z += gs.z; vz = f2u((float)vz + sg.z); tn.z += ts.z;
            }
        } else {
            if (tn.y < tn.z) {
                t = tn.y; vp.y += gs.y; vy = f2u((float)vy + sg.y); tn.y += ts.y;
            } else {
                t = tn.z; vp.z += gs.z; vz = f2u((float)vz + sg.z); tn.z += ts.z;
            }
        }
    }
    return 0;
}

/* rayCastVoxelsKernel (VoxelGrid_cuda.cu:734-770) with initRay (118-141) and
 * intersectVoxelGridCuda (144-163), for every pixel; Tcur: camera -> world
 * (VoxelGrid::rayCastImage, VoxelGrid.cpp:286-300).  xyz: W*H float4. */
void orc_tsdf_raycast(const float *grid, const orc_tsdf_params *p, const float Tcur[16], const float K[9],
                      int filtering, float *xyz) {
    const int R = p->R, W = p->W, H = p->H;
    const v3 vs = voxel_size(p);
    const v3 b0 = {p->origin[0] - p->dim[0], p->origin[1] - p->dim[1], p->origin[2] - p->dim[2]};
    const v3 b1 = {p->origin[0] + p->dim[0], p->origin[1] + p->dim[1], p->origin[2] + p->dim[2]};
    const v3 ib0 = {b0.x + vs.x, b0.y + vs.y, b0.z + vs.z};
    const v3 vd = {2.0f * vs.x, 2.0f * vs.y, 2.0f * vs.z};
    const float *T = Tcur;
#pragma omp parallel for schedule(dynamic, 4)
    for (int yi = 0; yi < H; yi++)
        for (int xi = 0; xi < W; xi++) {
            float pdx = (float)xi / (float)W, pdy = (float)yi / (float)H;
            v3 cam = {-(pdx - K[2]) / K[0], -(pdy - K[5]) / K[4], -1};
            float len = 0.0f;
            len += cam.x * cam.x;
            len += cam.y * cam.y;
            len += cam.z * cam.z;
            len = 1.0f / sqrtf(len);
            cam.x *= len;
            cam.y *= len;
            cam.z *= len;
            v3 dir = {T[0] * cam.x + T[1] * cam.y + T[2] * cam.z, T[4] * cam.x + T[5] * cam.y + T[6] * cam.z,
                      T[8] * cam.x + T[9] * cam.y + T[10] * cam.z};
            v3 o = {T[3], T[7], T[11]};
            int sgn[3] = {dir.x < 0, dir.y < 0, dir.z < 0};
            v3 inv;
            inv.x = (fabsf(dir.x) > 1e-6f) ? 1.0f / dir.x : (float)(1 - 2 * sgn[0]) * FLT_MAX;
            inv.y = (fabsf(dir.y) > 1e-6f) ? 1.0f / dir.y : (float)(1 - 2 * sgn[1]) * FLT_MAX;
            inv.z = (fabsf(dir.z) > 1e-6f) ? 1.0f / dir.z : (float)(1 - 2 * sgn[2]) * FLT_MAX;
            float *px = xyz + 4 * ((int64_t)yi * W + xi);
            px[0] = px[1] = px[2] = px[3] = 0.0f;
            /* intersectVoxelGridCuda */
            float x0 = ((sgn[0] ? b1.x : b0.x) - o.x) * inv.x;
            float x1 = ((sgn[0] ? b0.x : b1.x) - o.x) * inv.x;
            float y0 = ((sgn[1] ? b1.y : b0.y) - o.y) * inv.y;
            float y1 = ((sgn[1] ? b0.y : b1.y) - o.y) * inv.y;
            float z0 = ((sgn[2] ? b1.z : b0.z) - o.z) * inv.z;
            float z1 = ((sgn[2] ? b0.z : b1.z) - o.z) * inv.z;
            float tmin = fmaxf(x0, fmaxf(y0, z0));
            float tmax = fminf(x1, fminf(y1, z1));
            if (tmin >= tmax || tmax <= 0) continue;
            float th;
            if (!traverse(grid, R, o, dir, inv, sgn, tmin, tmax, ib0, vd, filtering, &th)) continue;
            px[0] = th * cam.x;
            px[1] = th * cam.y;
            px[2] = th * cam.z;
            px[3] = (th > p->min_dist && th < p->max_dist) ? 1.0f : 0.0f;
        }
}

/* shadingKernel (VoxelGrid_cuda.cu:844-891) with filter3 (772-789): shaded
 * image and normals of a ray-cast xyz image (all W*H float4) */
void orc_tsdf_shade(const float *xyz, int W, int H, float *shaded, float *normal) {
#pragma omp parallel for schedule(static)
    for (int yi = 0; yi < H; yi++)
        for (int xi = 0; xi < W; xi++) {
            int64_t off = (int64_t)yi * W + xi;
            float *pix = shaded + 4 * off, *nrm = normal + 4 * off;
            pix[0] = pix[1] = pix[2] = 0.0f;
            pix[3] = 1.0f;
            nrm[0] = nrm[1] = nrm[2] = nrm[3] = 0.0f;
            if (xi >= W - 3 || yi >= H - 3 || xi < 3 || yi < 3) continue;
            const float *p1x = xyz + 4 * (off + 1), *p0x = xyz + 4 * (off - 1);
            const float *p1y = xyz + 4 * (off + W), *p0y = xyz + 4 * (off - W);
            if (p1x[3] <= 0.0f || p0x[3] <= 0.0f || p1y[3] <= 0.0f || p0y[3] <= 0.0f) continue;
            float ux = p1x[0] - p0x[0], uy = p1x[1] - p0x[1], uz = p1x[2] - p0x[2];
            float vx = p0y[0] - p1y[0], vy = p0y[1] - p1y[1], vz = p0y[2] - p1y[2];
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
            float color = nx * 0.0f + ny * 0.0f + nz * 1.0f;
            if (color > 0.0f) {
                pix[0] = pix[1] = pix[2] = color;
                nrm[0] = nx;
                nrm[1] = ny;
                nrm[2] = nz;
            }
        }
}

/* resampleVoxelsKernel (VoxelGrid_cuda.cu:896-941): dst voxel centres mapped
 * by Tcur (camera -> world of the new grid, VoxelGrid::setCameraParams) into
 * src, trilinear tsdf and weight there, (1, 0) outside */
void orc_tsdf_resample(float *dst, const float *src, const orc_tsdf_params *p, const float Tcur[16]) {
    const int R = p->R;
    const v3 vs = voxel_size(p);
    const v3 start = {p->origin[0] - p->dim[0] + vs.x, p->origin[1] - p->dim[1] + vs.y,
                      p->origin[2] - p->dim[2] + vs.z};
    const v3 vs2 = {vs.x * 2, vs.y * 2, vs.z * 2};
    const float *iT = Tcur;
    const float hi = (float)(R - 2);
#pragma omp parallel for schedule(static)
    for (int iz = 0; iz < R; iz++)
        for (int iy = 0; iy < R; iy++)
            for (int ix = 0; ix < R; ix++) {
                float px = start.x + (float)ix * vs2.x;
                float py = start.y + (float)iy * vs2.y;
                float pz = start.z + (float)iz * vs2.z;
                float rx = iT[0] * px + iT[1] * py + iT[2] * pz + iT[3];
                float ry = iT[4] * px + iT[5] * py + iT[6] * pz + iT[7];
                float rz = iT[8] * px + iT[9] * py + iT[10] * pz + iT[11];
                v3 iv = {(rx - start.x) / vs2.x, (ry - start.y) / vs2.y, (rz - start.z) / vs2.z};
                float *g = dst + 2 * ((int64_t)ix + (int64_t)iy * R + (int64_t)iz * R * R);
                int oob = 0;
                if (iv.x < 0 || iv.x > hi) oob = 1;
                if (iv.y < 0 || iv.y > hi) oob = 1;
                if (iv.z < 0 || iv.z > hi) oob = 1;
                float dx, wx;
                if (!oob && trilinear(src, R, iv, 0, &dx) && trilinear(src, R, iv, 1, &wx)) {
                    g[0] = dx;
                    g[1] = wx;
                } else {
                    g[0] = 1;
                    g[1] = 0;
                }
            }
}
