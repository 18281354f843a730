/* recon_kinect.h -- C ABI of the Kinect pre-processing of the capture path
 * (tracker/multicore/multicore.cpp, OMPFunctions; used by ZConv::d2z,
 * zconv.cpp:395-445, and the file source, capture/fileSource.cpp:170-230).
 *
 * All pointers are device memory; the work is queued on `stream` (a
 * cudaStream_t, NULL for the default stream) and the calls do not wait.
 * Results are bit-identical to the reference routines on x86 (where a
 * negative shifted source coordinate is out of range and a negative bilinear
 * weight wraps modulo 2^32).  The Bayer demosaic of the capture path is
 * OpenCV's cvtColor(COLOR_BayerGB2RGB) and has no counterpart here. */
#ifndef RECON_KINECT_H
#define RECON_KINECT_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* OMPFunctions::d2Z / d2ZLow (multicore.cpp:189-275): depth z = |1 / (c0 +
 * c1 d)| in mm of 11-bit disparity d (2047: none), 0 outside [min_dist,
 * max_dist]; the source pixel is (x + x_off, y + y_off) (the Kinect's
 * disparity shift is -4, -3 when the calibration asks for it, zconv.cpp:411-413)
 * and must lie in [0, width-1) x [0, height-1).  half_resolution: the output
 * is width/2 x height/2, each pixel the smallest disparity of its 2x2 block
 * (all four valid).  Rows past the last of 4 equal row blocks are 0.
 * c0, c1, min_dist, max_dist: calibData[61], [42], minDist, maxDist. */
int recon_kinect_disparity_to_depth(const uint16_t *disp, int32_t width, int32_t height, float c0, float c1,
                                    float min_dist, float max_dist, float x_off, float y_off,
                                    int32_t half_resolution, float *z, void *stream);

/* OMPFunctions::convert2Gray (multicore.cpp:634-652): gray = (p0*19588 +
 * p1*38469 + p2*7471) >> 16 of 3-byte pixels in their stored channel order;
 * pixels past the last of 4 equal row blocks are not written. */
int recon_kinect_rgb_to_gray(const uint8_t *rgb, int32_t width, int32_t height, uint8_t *gray, void *stream);

/* OMPFunctions::undistort (multicore.cpp:654-738) as every call after the first
 * computes it (undistortLookup, 740-770): dst(x, y) samples src at K
 * (radial(iK (x, y))) -- kc[0], kc[1], kc[4] the radial terms -- with 8-bit
 * fixed-point bilinear weights, 0 where that point leaves [0, width-2) x
 * [0, height-2).  Rows past the last of 6 equal row blocks are not written. */
int recon_kinect_undistort_gray(const uint8_t *src, int32_t width, int32_t height, const float K[9], const float iK[9],
                                const float kc[5], uint8_t *dst, void *stream);

#ifdef __cplusplus
}

/* launch constants of the undistortion (C++ only) */
struct KinectUndistort {
    float K[9], iK[9], kc[5];
};
#endif
#endif
