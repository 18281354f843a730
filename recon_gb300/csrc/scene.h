/*
 * Procedural RGB-D scene: seeded textured room + boxes, ray-cast into an
 * IR (depth) camera and an RGB (gray) camera.
 *
 * The reference renders its synthetic input with OpenGL (a teapot drawn into
 * an FBO, utils/src/Renderer.cpp:137-175, depth packed by the shader at
 * utils/src/Shaders.cpp:206-216).  No graphics stack exists on the target
 * machines, so the inputs are produced by this ray caster instead.  The same
 * functions are compiled for the GPU (render kernel) and for the host (CPU
 * twin), and they use only IEEE-exact operations (+ - * / floor, integer
 * hashing, no transcendentals), so both produce bit-identical images when
 * compiled without FMA contraction.
 *
 * Conventions follow the reference tracker: cameras look down -z (points in
 * front of the camera have z < 0), pixel (x, y) is sampled at integer
 * coordinates, and the intrinsics carry a negative x focal length
 * (calib/calib.cpp:150,174 negate K[0]).
 */
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define SCENE_HD __host__ __device__ __forceinline__
#else
#define SCENE_HD static inline
#endif

#define RECON_SCENE_MAX_BOXES 16

typedef struct recon_scene {
    float room_min[3];
    float room_max[3];
    int32_t n_boxes;
    uint32_t seed;
    float box_c[RECON_SCENE_MAX_BOXES][3];
    float box_h[RECON_SCENE_MAX_BOXES][3];
    float box_R[RECON_SCENE_MAX_BOXES][9]; /* world -> box-local rotation, row-major */
} recon_scene;

/* Camera description for one render pass. */
typedef struct recon_camera {
    float K[9];       /* row-major 3x3, already scaled to pixels (fx < 0) */
    float kc[5];      /* radial distortion k1, k2, (unused), (unused), k3 */
    float Rcw[9];     /* camera -> world rotation, row-major */
    float tcw[3];     /* camera centre in world coordinates (mm) */
    int32_t width, height;
} recon_camera;

SCENE_HD uint32_t scene_hash(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU;
    x ^= x >> 15; x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

SCENE_HD float scene_u01(uint32_t h) { return (float)(h >> 8) * (1.0f / 16777216.0f); }

SCENE_HD float scene_lattice(int32_t ix, int32_t iy, uint32_t seed) {
    uint32_t h = scene_hash((uint32_t)ix * 0x9E3779B1u ^ scene_hash((uint32_t)iy + seed * 0x85EBCA77u));
    return scene_u01(h);
}

SCENE_HD float scene_floor(float x) {
    /* floor for |x| < 2^23 without calling libm, identical on host and device */
    int32_t i = (int32_t)x;
    float fi = (float)i;
    return (fi > x) ? fi - 1.0f : fi;
}

SCENE_HD float scene_value_noise(float x, float y, uint32_t seed) {
    float fx = scene_floor(x), fy = scene_floor(y);
    int32_t ix = (int32_t)fx, iy = (int32_t)fy;
    float tx = x - fx, ty = y - fy;
    float sx = tx * tx * (3.0f - 2.0f * tx);
    float sy = ty * ty * (3.0f - 2.0f * ty);
    float a = scene_lattice(ix, iy, seed);
    float b = scene_lattice(ix + 1, iy, seed);
    float c = scene_lattice(ix, iy + 1, seed);
    float d = scene_lattice(ix + 1, iy + 1, seed);
    float ab = a + (b - a) * sx;
    float cd = c + (d - c) * sx;
    return ab + (cd - ab) * sy;
}

/* Albedo in [0,1): four octaves of value noise (feature sizes 230, 97, 41, 17 mm). */
SCENE_HD float scene_texture(float u, float v, uint32_t seed) {
    float t = 0.45f * scene_value_noise(u * 0.004347826f, v * 0.004347826f, seed);
    t += 0.25f * scene_value_noise(u * 0.010309278f, v * 0.010309278f, seed + 17u);
    t += 0.17f * scene_value_noise(u * 0.024390243f, v * 0.024390243f, seed + 39u);
    t += 0.13f * scene_value_noise(u * 0.058823529f, v * 0.058823529f, seed + 71u);
    return t;
}

/* Undistorted normalised image coordinates of pixel (x, y): inverts
 * pd = K * pu * (1 + k1 r^2 + k2 r^4 + k3 r^6) (kernels/kernelUtils.h:394-408)
 * by a fixed number of fixed-point iterations. */
SCENE_HD void scene_pixel_ray(const recon_camera *cam, float x, float y, float *dx, float *dy) {
    float qx = (x - cam->K[2]) / cam->K[0];
    float qy = (y - cam->K[5]) / cam->K[4];
    float px = qx, py = qy;
    if (cam->kc[0] != 0.0f || cam->kc[1] != 0.0f || cam->kc[4] != 0.0f) {
        for (int it = 0; it < 12; it++) {
            float r2 = px * px + py * py;
            float r4 = r2 * r2;
            float r6 = r4 * r2;
            float rad = 1.0f + cam->kc[0] * r2 + cam->kc[1] * r4 + cam->kc[4] * r6;
            px = qx / rad;
            py = qy / rad;
        }
    }
    /* camera looks down -z: a point at z = -1 has pu = (x/z, y/z) = (-x, -y) */
    *dx = -px;
    *dy = -py;
}

/* Casts one ray; returns depth along the camera -z axis (mm), or -1 for no hit.
 * *albedo receives the texture value at the hit point. */
SCENE_HD float scene_cast(const recon_scene *sc, const recon_camera *cam, int32_t xi, int32_t yi, float *albedo) {
    float cx, cy;
    scene_pixel_ray(cam, (float)xi, (float)yi, &cx, &cy);
    const float cz = -1.0f;
    const float *R = cam->Rcw;
    float d[3], o[3];
    d[0] = R[0] * cx + R[1] * cy + R[2] * cz;
    d[1] = R[3] * cx + R[4] * cy + R[5] * cz;
    d[2] = R[6] * cx + R[7] * cy + R[8] * cz;
    o[0] = cam->tcw[0]; o[1] = cam->tcw[1]; o[2] = cam->tcw[2];

    /* room interior: first exit face */
    float tbest = 3.0e38f;
    int face = -1;
    for (int a = 0; a < 3; a++) {
        float ta = 3.0e38f;
        int f = -1;
        if (d[a] > 0.0f) { ta = (sc->room_max[a] - o[a]) / d[a]; f = 2 * a + 1; }
        else if (d[a] < 0.0f) { ta = (sc->room_min[a] - o[a]) / d[a]; f = 2 * a; }
        if (f >= 0 && ta < tbest) { tbest = ta; face = f; }
    }
    float hu = 0.0f, hv = 0.0f;
    uint32_t tseed = sc->seed;
    if (face >= 0) {
        int a = face >> 1;
        float p[3];
        p[0] = o[0] + tbest * d[0];
        p[1] = o[1] + tbest * d[1];
        p[2] = o[2] + tbest * d[2];
        hu = p[(a + 1) % 3];
        hv = p[(a + 2) % 3];
        tseed = sc->seed + 101u * (uint32_t)(face + 1);
    }
    /* boxes: slab test in box-local coordinates */
    for (int b = 0; b < sc->n_boxes; b++) {
        const float *Rb = sc->box_R[b];
        float oc[3], ol[3], dl[3];
        oc[0] = o[0] - sc->box_c[b][0];
        oc[1] = o[1] - sc->box_c[b][1];
        oc[2] = o[2] - sc->box_c[b][2];
        ol[0] = Rb[0] * oc[0] + Rb[1] * oc[1] + Rb[2] * oc[2];
        ol[1] = Rb[3] * oc[0] + Rb[4] * oc[1] + Rb[5] * oc[2];
        ol[2] = Rb[6] * oc[0] + Rb[7] * oc[1] + Rb[8] * oc[2];
        dl[0] = Rb[0] * d[0] + Rb[1] * d[1] + Rb[2] * d[2];
        dl[1] = Rb[3] * d[0] + Rb[4] * d[1] + Rb[5] * d[2];
        dl[2] = Rb[6] * d[0] + Rb[7] * d[1] + Rb[8] * d[2];
        float tmin = -3.0e38f, tmax = 3.0e38f;
        int amin = 0;
        int ok = 1;
        for (int a = 0; a < 3; a++) {
            float h = sc->box_h[b][a];
            if (dl[a] == 0.0f) {
                if (ol[a] < -h || ol[a] > h) ok = 0;
                continue;
            }
            float t1 = (-h - ol[a]) / dl[a];
            float t2 = (h - ol[a]) / dl[a];
            float tn = t1 < t2 ? t1 : t2;
            float tf = t1 < t2 ? t2 : t1;
            if (tn > tmin) { tmin = tn; amin = a; }
            if (tf < tmax) tmax = tf;
        }
        if (ok && tmin <= tmax && tmin > 1.0f && tmin < tbest) {
            tbest = tmin;
            float pl[3];
            pl[0] = ol[0] + tmin * dl[0];
            pl[1] = ol[1] + tmin * dl[1];
            pl[2] = ol[2] + tmin * dl[2];
            hu = pl[(amin + 1) % 3];
            hv = pl[(amin + 2) % 3];
            tseed = sc->seed + 7919u * (uint32_t)(b + 1) + 13u * (uint32_t)amin;
            face = 6 + b;
        }
    }
    if (face < 0) { *albedo = 0.0f; return -1.0f; }
    *albedo = scene_texture(hu, hv, tseed);
    /* d was built from a camera ray with z = -1, so the ray parameter is the depth */
    return tbest;
}

/* Irwin-Hall(4) approximation of a unit normal variate, from a counter hash. */
SCENE_HD float scene_gauss(uint32_t seed, uint32_t frame, uint32_t pix) {
    uint32_t h = scene_hash(seed * 0x27d4eb2fu ^ scene_hash(frame * 0x165667b1u ^ scene_hash(pix)));
    float s = 0.0f;
    for (int k = 0; k < 4; k++) {
        h = scene_hash(h + 0x9E3779B9u);
        s += scene_u01(h);
    }
    return (s - 2.0f) * 1.7320508f;
}

/* Depth pixel (uint16 mm, 0 = invalid) with multiplicative noise sigma = noise_rel * depth. */
SCENE_HD uint16_t scene_depth_pixel(const recon_scene *sc, const recon_camera *cam, int32_t xi, int32_t yi,
                                    float noise_rel, uint32_t noise_seed, uint32_t frame) {
    float alb;
    float z = scene_cast(sc, cam, xi, yi, &alb);
    if (z <= 0.0f) return 0;
    if (noise_rel != 0.0f) {
        float n = scene_gauss(noise_seed, frame, (uint32_t)(yi * cam->width + xi));
        z = z + z * noise_rel * n;
    }
    if (!(z >= 0.5f && z < 65535.0f)) return 0;
    return (uint16_t)(z + 0.5f);
}

/* Gray pixel (uint8): albedo mapped to [0.1, 0.9]. */
SCENE_HD uint8_t scene_gray_pixel(const recon_scene *sc, const recon_camera *cam, int32_t xi, int32_t yi) {
    float alb;
    float z = scene_cast(sc, cam, xi, yi, &alb);
    if (z <= 0.0f) return 0;
    float g = 0.1f + 0.8f * alb;
    int32_t v = (int32_t)(g * 255.0f + 0.5f);
    if (v < 0) v = 0;
    if (v > 255) v = 255;
    return (uint8_t)v;
}
