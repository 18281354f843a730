/* recon_kinect.h -- C ABI of the Kinect pre-processing of the capture path
 * (tracker/multicore/multicore.cpp, OMPFunctions; used by ZConv::d2z,
 * zconv.cpp:395-445, and the file source, capture/fileSource.cpp:170-230).
 *
 * All pointers are device memory; the work is queued on `stream` (a
 * cudaStream_t, NULL for the default stream) and the calls do not wait.
 * Results of the host routines' counterparts are bit-identical to the
 * reference routines on x86 (where a negative shifted source coordinate is
 * out of range and a negative bilinear weight wraps modulo 2^32); those of
 * the GPU capture path to the reference kernels on the GPU.  The Bayer demosaic of the capture path is
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

/* ---- the GPU capture path: the reference's CUDA kernels as
 * capture/VideoPreProcessorGPU.cpp:120-175 and reconstruct/TrackFrame.cpp:
 * 430-465 call them (undistortDisparityCuda -> d2ZCudaHdr for depth,
 * convertToHDRCuda -> rgb2GrayCuda for gray).  Every pixel of the output is
 * written (the reference's 32 x 30 blocks cover sizes that are multiples of
 * them).  The reference converts a shifted float coordinate to unsigned,
 * which on the GPU saturates: where 2x + x_off or 2y + y_off is negative the
 * depth reads row or column 0 (unlike the host routines above). ---- */

/* undistortDisparityCuda (d2z.cu:1098-1104, undistortDisparityKernel
 * d2z.cu:68-85): the disparity as float, 65535 where it is 2047 or more. */
int recon_kinect_disparity_to_float(const uint16_t *disp, int32_t width, int32_t height, float *out, void *stream);

/* d2ZCuda / d2ZCudaHdr (d2z.cu:1073-1088; d2ZLowKernel / d2ZLowHdrKernel,
 * d2z.cu:88-170): the width/2 x height/2 depth of 16-bit (disp_u16) or float
 * (disp_f32; exactly one of the two non-null) disparity.  At (2x + x_off,
 * 2y + y_off) inside [0, width-1) x [0, height-1) with all four 2x2
 * disparities below 2047: z = |1 / (c0 + c1 min d)|, 0 outside [min_dist,
 * max_dist], and the output is (z - min_dist) / (max_dist - min_dist) (so a
 * depth outside the range gives -min_dist / (max_dist - min_dist));
 * elsewhere 0. */
int recon_kinect_depth_normalized(const uint16_t *disp_u16, const float *disp_f32, int32_t width, int32_t height,
                                  float c0, float c1, float min_dist, float max_dist, float x_off, float y_off,
                                  float *z_low, void *stream);

/* convertToHDRCuda (rgb2gray.cu:880-888, convertHdrRGBKernel 634-647): every
 * byte of the 3-channel image / 255 as float. */
int recon_kinect_rgb_to_hdr(const uint8_t *rgb, int32_t width, int32_t height, float *rgb_hdr, void *stream);

/* rgb2GrayCuda (rgb2gray.cu:649-662): from 3-byte pixels (rgb2GrayHdrKernel,
 * 41-50: float((p0*19588 + p1*38469 + p2*7471) >> 16)) or from float RGB
 * (rgbF2GrayHdrKernel, 53-62: 0.3 r + 0.59 g + 0.11 b); exactly one of rgb
 * and rgb_hdr non-null. */
int recon_kinect_rgb_to_gray_hdr(const uint8_t *rgb, const float *rgb_hdr, int32_t width, int32_t height,
                                 float *gray, void *stream);

/* undistortRGBCuda (undistort.cu:231-239, undistortHdrRGBKernel 110-170):
 * every channel of the 3-byte image sampled at K (radial(iK (x, y))) with
 * float bilinear weights of the values / 255, into float RGB; 0 where int(p)
 * leaves [0, width-2) x [0, height-2).  K, iK, kc: calibData[0..8], [9..17],
 * [18..22] (kc[0], kc[1], kc[4] the radial terms). */
int recon_kinect_undistort_rgb_hdr(const uint8_t *rgb, int32_t width, int32_t height, const float K[9],
                                   const float iK[9], const float kc[5], float *rgb_hdr, void *stream);

#ifdef __cplusplus
}

/* launch constants of the undistortion (C++ only) */
struct KinectUndistort {
    float K[9], iK[9], kc[5];
};
#endif
#endif
