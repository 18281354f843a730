/* recon_tsdf.h -- C ABI of the reconstruction stream: TSDF fusion of depth
 * maps into a voxel grid and ray casting of the fused surface.
 *
 * Replaces VoxelGrid (tracker/reconstruct/VoxelGrid.h, VoxelGrid.cpp) and the
 * kernels it launches (tracker/kernels/VoxelGrid_cuda.cu).  A handle owns one
 * grid of R^3 voxels, each a float2 (tsdf, weight) in the reference's layout
 * (x fastest, then y, then z; VoxelGrid_cuda.cu:952), the distance map of the
 * last measurement and the ray-cast images.  Every call is asynchronous on the
 * handle's stream (one stream per grid: the reference runs its voxel grid on
 * its own GPU, main.cpp:923-989) except the *_get copies, which synchronise.
 * Results are bit-identical to the reference's kernel arithmetic compiled
 * without multiply-add contraction.
 *
 * Poses are row-major 4x4 float, camera -> world (the reference's Tcur /
 * tsdfPose).  K is the normalised 3x3 intrinsic matrix of getNormalizedK
 * (main.cpp:878-882): K[0] = fx / width, K[2] = cx / width, K[4] = fy /
 * height, K[5] = cy / height.
 */
#ifndef RECON_TSDF_H
#define RECON_TSDF_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct recon_tsdf recon_tsdf;

/* SimParams (tracker/kernels/particles_kernel.cuh:38-51) without the camera
 * fields, which each call passes. */
typedef struct recon_tsdf_params {
    int32_t grid_resolution; /* voxels per side; a multiple of 8 (main.cpp:78) */
    float cube_origin[3];    /* centre of the grid (VoxelGrid.cpp:62: 0, 0.01, -1600.01) */
    float cube_dim[3];       /* half the side length (VoxelGrid.cpp:63: 1500) */
    int32_t width, height;   /* distance map and ray-cast image size */
    float min_dist, max_dist; /* depth range of the RGB-D frames (calibration minDist / maxDist) */
} recon_tsdf_params;

/* The reference's grid placement (VoxelGrid.cpp:48-106) for R voxels per side. */
void recon_tsdf_default_params(int32_t grid_resolution, int32_t width, int32_t height, float min_dist,
                               float max_dist, recon_tsdf_params *out);

/* VoxelGrid::VoxelGrid + initialize (VoxelGrid.cpp:48-132): allocates the grid
 * (8 * R^3 bytes) and the images and clears the grid.  stream: a cudaStream_t
 * for all work of the grid, or NULL to create one. */
int recon_tsdf_create(const recon_tsdf_params *p, void *stream, recon_tsdf **out);
int recon_tsdf_destroy(recon_tsdf *v);
/* VoxelGrid::clear / reset (VoxelGrid.cpp:316-327): every voxel (1, 0). */
int recon_tsdf_reset(recon_tsdf *v);

/* The measurement: a distance map (width x height float, positive depth along
 * the optical axis in mm, 0 = none), from
 *  - the distance map itself,
 *  - the reference's float4 RGB-D frame (w = depth normalised to [min_dist,
 *    max_dist], rows stored bottom-up): VoxelGrid::preprocessMeasurementRGBD
 *    and reconstructionKernel (VoxelGrid.cpp:253-264, VoxelGrid_cuda.cu:1090-1112),
 *  - a uint16 depth map in mm (0 = none), top row first.
 * on_device: the input pointer is device memory (else host memory, copied). */
int recon_tsdf_set_dist_map(recon_tsdf *v, const float *dist, int32_t on_device);
int recon_tsdf_set_dist_rgbd_float4(recon_tsdf *v, const float *rgbd, int32_t on_device);
int recon_tsdf_set_dist_depth16(recon_tsdf *v, const uint16_t *depth, int32_t on_device);

/* VoxelGrid::update (VoxelGrid.cpp:275-284, updateVoxelsKernel
 * VoxelGrid_cuda.cu:944-1014): fuses the distance map seen from T into the
 * grid (running mean of the truncated signed distance, weight capped at 16). */
int recon_tsdf_update(recon_tsdf *v, const float T[16], const float K[9]);

/* VoxelGrid::rayCastImage (VoxelGrid.cpp:286-300, rayCastVoxelsKernel and
 * shadingKernel, VoxelGrid_cuda.cu:734-770, 844-891): per pixel the first
 * zero crossing of the grid along the ray from T, as a camera-frame point
 * (float4 xyz, w = 1 when the ray length is inside (min_dist, max_dist)), the
 * shaded image (float4 gray) and the surface normals (float4).  cubic_filter:
 * three extra interpolation steps of the crossing (the reference passes 1). */
int recon_tsdf_raycast(recon_tsdf *v, const float T[16], const float K[9], int32_t cubic_filter);

/* resampleVoxelGrid (main.cpp:884-891, resampleVoxelsKernel
 * VoxelGrid_cuda.cu:896-941): dst's voxels are mapped by T (camera -> world of
 * dst's frame) into src and take its trilinear tsdf and weight, (1, 0) outside.
 * Both grids must have the same parameters.  Runs on dst's stream after src's
 * pending work. */
int recon_tsdf_resample(recon_tsdf *dst, recon_tsdf *src, const float T[16]);

/* Device arrays of the grid: "tsdf" (R^3 float2), "dist" (float), "xyz",
 * "shaded", "normal" (width*height float4: getRayCastXYZImage,
 * getRayCastImage, getRayCastNormalImage).  NULL for an unknown name. */
void *recon_tsdf_device_array(recon_tsdf *v, const char *name);
/* Copies one of those arrays to host memory (synchronises); returns bytes. */
int64_t recon_tsdf_get(recon_tsdf *v, const char *name, void *host_dst, int64_t nbytes);
/* Replaces the grid (R^3 float2, host or device memory). */
int recon_tsdf_set_grid(recon_tsdf *v, const float *grid, int32_t on_device);
void *recon_tsdf_stream(recon_tsdf *v);

/* Measurement hooks (no reference counterpart).  With timing on, every
 * launch is bracketed with CUDA events; totals per kind (0 update, 1 ray
 * cast, 2 shading, 3 distance map, 4 reset / resample) are read with
 * recon_tsdf_get_timing.  With counting on, the update also counts voxels
 * [projected, fused, changed]; the grid traffic of an update is 8 bytes read
 * per fused voxel and 8 bytes written per changed one. */
int recon_tsdf_enable_timing(recon_tsdf *v, int32_t on);
int recon_tsdf_get_timing(recon_tsdf *v, double ms[5], int64_t launches[5], int32_t reset);
int recon_tsdf_enable_counting(recon_tsdf *v, int32_t on);
int recon_tsdf_get_counts(recon_tsdf *v, int64_t counts[3], int32_t reset);

#ifdef __cplusplus
}
#endif
#endif
