/*
 * recon_ref_shim.h -- the reference tracker's kernel-level C ABI, re-implemented
 * for sm_103a.
 *
 * The functions keep the names, argument order and argument meaning of the
 * reference's extern "C" launchers (tracker/kernels/cuda_funcs.h:36-111,
 * histogram_common.h:31-34), so the reference's PhotoTracker / ShapeTracker
 * call sites compile against this header after one substitution: the C++
 * container objects they pass (VertexBuffer2, rendering/VertexBuffer2.h:28-78;
 * ImagePyramid2, image2/ImagePyramid2.h:35-78) become the POD views below.
 * Data layouts are the reference's: stride-24 vertex records, stride-6 ICP
 * clouds, SoA Jacobians J[c*count + i], 96-float calibData in device memory.
 *
 * Like the reference, the functions return void and validate their arguments
 * by printing nothing and returning early; the status of the last call is
 * available from recon_last_status() (0 = OK, negative = RECON_ERR_*).
 * Module-static scratch (histograms, segment tables, block sums) is process
 * global as in the reference (initHistogram64 / initCudaDotProduct,
 * histogram64.cu:96-113, warp.cu:1412-1427): calls must not overlap on the GPU.
 * Reductions use the library's canonical order, not the reference's
 * per-dot-product launches (warp.cu:1430-1487).
 */
#pragma once
#include <stdint.h>

#include "recon_track.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *recon_stream_t; /* cudaStream_t */

typedef struct recon_vbuffer { /* VertexBuffer2 */
    float *devPtr;             /* vertexCount records of `stride` floats */
    int32_t *indexDevPtr;      /* elementsCount selected record indices */
    int32_t stride;            /* 24 (VERTEXBUFFER_STRIDE, VertexBuffer2.h:24) */
    int32_t vertexCount;
    int32_t elementsCount;     /* set by filterIndices4 */
} recon_vbuffer;

typedef struct recon_pyramid { /* ImagePyramid2 of 1-channel float images */
    int32_t nLayers;
    int32_t width[RECON_MAX_LEVELS], height[RECON_MAX_LEVELS];
    float *devPtr[RECON_MAX_LEVELS];
} recon_pyramid;

int recon_last_status(void);

/* downSample2Cuda.cu:43-77 */
void downSample2Pyramid(recon_pyramid *pyramid, recon_stream_t stream);
/* rgb2gray.cu:665-670, 672-678 */
void convertZmapToXYZCuda(float *zReferenceDev, float *refPointsDev /* float4 */, float *calibDataDev, int width,
                          int height, recon_stream_t stream);
void convertZmapToXYZ6Cuda(float *zReferenceDev, float *refPointsDev, int *selectionMask, float *calibDataDev,
                           int width, int height, recon_stream_t stream);
/* d2z.cu:1107-1128 */
void xyz2CloudCuda(float *xyzImage /* float4 */, float *calibDataDev, recon_vbuffer *vbuffer,
                   recon_pyramid *grayPyramid, recon_stream_t stream);
/* d2z.cu:1297-1322 */
void extractGradientMagnitudes(recon_vbuffer *vbuffer, float *gradientScratchDev, recon_stream_t stream);
/* cuda_hist.cu:100-152 (returns 0, like the reference) */
double cudaHista(float *src, float *hist, int length, int bins, float *d_hist, recon_stream_t stream);
/* filterIndex256.cu:171-194 */
void filterIndices4(recon_vbuffer *vbuffer, float *gradientData, float *histogramDev, int pixelSelectionAmount,
                    int nbins, recon_stream_t stream);
/* d2z.cu:1229-1265 */
void addVertexAttributesWithoutNormalsCuda(float *calibDataDev, recon_vbuffer *vbuffer, recon_pyramid *grayPyramid,
                                           recon_stream_t stream);
/* warp.cu:1336-1354 */
void precomputeJacobian4Cuda(recon_vbuffer *vbuffer, float *calibDataDev, float *jacobian1Dev, float *jacobian2Dev,
                             float *jacobian3Dev, float *jacobian4Dev, float optScaleIn, recon_stream_t stream);
/* warp.cu:1160-1218 */
void interpolateResidual2(recon_vbuffer *vbuffer, float *T, float *calibDataDev, recon_pyramid *grayPyramid,
                          int layer, float *zCurrentDev, float *zWeightsDev, float *residual, recon_stream_t stream);
/* histogram64.cu:115-157 */
void generateWeights64(float *residualDev, int count, float *weightsDev, float *extWeightsDev,
                       float *weightedResidualDev, recon_stream_t stream);
/* warp.cu:1396-1409 */
void weightJacobian(float *jacobianTDev, float *weights, int count, float *weightedJacobianTDev,
                    recon_stream_t stream);
/* warp.cu:1472-1487, 1453-1470 */
void JTJCuda(float *JT, int count, float *JtJDev, recon_stream_t stream);
void JTresidualCuda(float *JT, float *residual, int count, float *result6, recon_stream_t stream);
/* warp.cu:1498-1509 */
void linearFuseCuda(float *JtJDevExt, float *residual6DevExt, float weight1, int N1, float *JtJDev,
                    float *residual6Dev, float weight2, int N2, recon_stream_t stream);
/* warp.cu:1512-1601: FP64 CG (6 steps, tol 1e-8), then T <- T * expm(x) */
void solveMotionCuda(float *JtJDev, float *b, float *TDev, float scaleOut, recon_stream_t stream);
/* d2z.cu:1158-1166, 1287-1295, 1184-1195 */
void genPointCloud6Cuda(float *zCurrentDev, int texWidth, int texHeight, float *curPointsDev, int *selectionMaskDev,
                        float *calibDataDev, recon_stream_t stream);
void computeNormals6Cuda(float *refPointsDev, int *selectionMask, int texWidth, int texHeight,
                         recon_stream_t stream);
void downSampleCloud6Cuda(float *xyz6DevSrc, int *maskSrc, float *xyz6DevDst, int *maskDst, int dstTexWidth,
                          int dstTexHeight, recon_stream_t stream);
/* rgb2gray.cu:780-790, 827-877, 810-825 */
void icpResidualMaskCuda2(float *refPointsDev, int *selectionMask, int width, int height, float *TDev,
                          float *calibDataDev, float *curPointsDev, int *selectionMaskRef, int layer,
                          float *residualDev, int *residualMaskDev, recon_stream_t stream);
void selectValidIndex(int *residualMaskDev, int nElems, int *partialSumIntDev, int maxBlocks, int *selectionIndexDev,
                      recon_stream_t stream);
void packIndex(int *selectionIndexDev, int totalSelected, float *fullResidualDev, float *residualDev,
               float *residual2Dev, recon_stream_t stream);
void generateStudentTWeights(float *residual2Dev, int nElems, float *partialSumDev, int maxBlocks, float *weightsDev,
                             recon_stream_t stream);
void icpResidualCuda2(float *refPointsDev, int *select, int nSelect, int width, int height, int layer, float *TDev,
                      float *calibDataDev, float *curPointsDev, int *curMask, int nPadded, float *residualDev,
                      float *jacobianDev, float *weightsDev, float optScaleIn, recon_stream_t stream);

#ifdef __cplusplus
}
#endif
