/*
 * recon_track.h -- C ABI of the GB300 dense RGB-D tracking library
 * (librecon_track.so, hand-written sm_103a CUDA behind plain C entry points).
 *
 * It replaces the tracking hot path of ttykkala/recon: the PhotoTracker /
 * ShapeTracker operator classes (tracker/tracker/phototracker.h:33-154,
 * tracker/tracker/shapetracker.h:29-137) and the extern "C" kernel launchers
 * they call (tracker/kernels/cuda_funcs.h:36-111, histogram_common.h:31-34,
 * expmCuda.h).  All signatures use plain pointers and sizes; every call returns
 * a status code (the reference prints and returns, hostUtils.cpp:27-33).
 *
 * Pointers: "host" arguments are host memory; functions taking `on_device`
 * accept either host (0) or device (1) image pointers.  All device work of one
 * tracker/batch runs on the stream given at creation (NULL = the library's own
 * stream); the reference's second GPU becomes a second stream (fusion).
 * Device inputs are read on that stream: work that writes them on another
 * stream must be ordered before the call (an event the batch's stream,
 * recon_batch_stream, waits for, or a synchronisation).
 */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define RECON_OK 0
#define RECON_ERR_INVALID_ARG -1
#define RECON_ERR_NOT_ENOUGH_POINTS -2 /* shapetracker.cpp:365 "not enough points" */
#define RECON_ERR_NON_SPD -3           /* a Cholesky pivot was not positive; pose kept */
#define RECON_ERR_TIMEOUT -4           /* reserved: no kernel of this library waits on a flag */
#define RECON_ERR_CUDA -5
#define RECON_ERR_STATE -6             /* reference or current frame missing */
#define RECON_ERR_NO_DEVICE -7

#define RECON_CALIB_SIZE 96 /* calibData layout of tracker/calib/calib.h:22-37 */
#define RECON_MAX_LEVELS 4

/* TrackMode, phototracker.h:30 */
#define RECON_GEOMETRIC 0
#define RECON_PHOTOMETRIC 1
#define RECON_BIOBJECTIVE 2

#define RECON_SOLVER_CHOLESKY 0 /* FP64 Cholesky (reference: dead choleskyKernel, warp.cu:978-1007) */
#define RECON_SOLVER_CG 1       /* FP64 CG, 6 steps, tol 1e-8 (reference live solver, warp.cu:926-975) */

#define RECON_PRECISION_FP32 0
#define RECON_PRECISION_MIXED 1 /* FP16 image pyramids, BF16 Jacobians, FP32 math, FP64 reduction fold */

typedef struct recon_config {
    int32_t width, height, levels; /* level-0 size; 3 levels at 320 wide, 4 at 640 (phototracker.cpp:777-784) */
    int32_t n_select;              /* photometric points, multiple of 1024 (phototracker.cpp:48: 8192) */
    int32_t hist_bins;             /* MAD histogram bins (histogram64.cu: 64) */
    int32_t select_bins;           /* pixel-selection histogram bins (phototracker.cpp:346: 256) */
    int32_t solver;                /* RECON_SOLVER_* */
    int32_t mode;                  /* RECON_GEOMETRIC / PHOTOMETRIC / BIOBJECTIVE */
    float lambda;                  /* bi-objective weight of the ICP term (setLambda, phototracker.cpp:160-165) */
    int32_t iters[RECON_MAX_LEVELS]; /* GN iterations, coarse -> fine (setIterationCounts, phototracker.cpp:488-490) */
    float opt_scale_in;            /* 1e-3 (phototracker.cpp:50) */
    float opt_scale_out;           /* 1e3  (phototracker.cpp:51) */
    int32_t precision;             /* RECON_PRECISION_* */
    float settle_mm;               /* > 0: a level ends early once one GN iteration moves every
                                      translation entry of the pose by <= settle_mm (mm) and every
                                      rotation entry by <= settle_rot; 0 (default): the fixed
                                      schedule of the reference */
    float settle_rot;
    int32_t reserved[5];
} recon_config;

typedef struct recon_track_stats {
    int32_t status;                   /* RECON_OK; RECON_ERR_NON_SPD if a solve was rejected; else
                                         RECON_ERR_NOT_ENOUGH_POINTS if an iteration was skipped for
                                         lack of ICP correspondences (the pose is kept in both cases) */
    int32_t iterations;               /* GN iterations executed */
    int32_t solves;                   /* iterations that updated the pose */
    int32_t icp_selected[RECON_MAX_LEVELS]; /* valid ICP correspondences per level (0 if unused) */
    int32_t photo_median_bin;         /* MAD histogram median bin of the last photometric iteration */
    int32_t non_spd;                  /* solves rejected by a non-positive pivot */
    int32_t reserved[5];
} recon_track_stats;

/* Per-iteration record (for parity checks): pose after the update and the
 * normal equations that produced it. */
typedef struct recon_iter_trace {
    int32_t level, iter, mode, solved, icp_selected, status;
    float T[16];
    double A[36];
    double b[6];
    double A_ph[36], b_ph[6], A_icp[36], b_icp[6];
    int32_t hist[256];
    int32_t median_bin;
    int32_t pad_;
} recon_iter_trace;

typedef struct recon_batch recon_batch;

/* ---- library ---- */
const char *recon_last_error(void);
int recon_device_count(void);

/* calibData from raw calibration (Calibration::setupCalibDataBuffer, calib.cpp:74-93). */
int recon_calib_setup(const double KL[9], const double KR[9], const double TLR[16], const double kcR[8],
                      double min_dist, double max_dist, double c0, double c1, int32_t width, float *calib_out);

/* ---- batch of tracker instances (one instance = one PhotoTracker + ShapeTracker) ----
 * Every instance has its own configuration and calibration; one launch serves
 * all instances.  The single-tracker calls below are batches of one. */
int recon_batch_create(int32_t n, const recon_config *cfgs, const float *calibs, void *stream, recon_batch **out);
int recon_batch_destroy(recon_batch *b);
int recon_batch_size(const recon_batch *b);

/* Reference (keyframe) images for instances [0, n): uint8 gray (RGB camera) and
 * uint16 depth in mm (IR camera, 0 = invalid).  Rebuilds the photometric
 * selection and Jacobians and the ICP reference pyramid and resets the pose to
 * identity (PhotoTracker::prepareReference, phototracker.cpp:360-386;
 * ShapeTracker::setReferencePoints/prepareReference, shapetracker.cpp:205-288).
 * gray[i] / depth[i] may be NULL to leave instance i unchanged. */
int recon_batch_set_reference(recon_batch *b, const uint8_t *const *gray, const uint16_t *const *depth,
                              int32_t on_device);
/* The filtered reference (setFilteredReference(true); PhotoTracker::
 * setReferencePoints and ShapeTracker::setReferencePoints, phototracker.cpp:
 * 310-337, shapetracker.cpp:195-212): the photometric reference from gray and
 * depth as recon_batch_set_reference, the ICP reference from oriented points
 * -- points[i] and normals[i] are width x height float4 maps in instance i's
 * depth-camera frame, typically the ray cast of a fused volume
 * (recon_tsdf_device_array "xyz" and "normal"); a pixel whose point has z < 0
 * and whose normal is not zero becomes an ICP point with that normal
 * (genOrientedPoints6Kernel, d2z.cu:471-501), coarser levels are 2x2 means
 * as for a raw reference.  points / normals may hold NULL for instances that
 * take the raw path (normals from the depth).  A later keyframe fusion
 * rebuilds the ICP reference from the fused depth. */
int recon_batch_set_reference_oriented(recon_batch *b, const uint8_t *const *gray, const uint16_t *const *depth,
                                       const float *const *points, const float *const *normals, int32_t on_device);
/* Reference given as the reference's float4 RGBA + normalised depth frame
 * (rgbTex2GrayHdrZKernel, rgb2gray.cu:64-76; rows stored bottom-up). */
int recon_batch_set_reference_rgbd_float4(recon_batch *b, int32_t inst, const float *rgbd, int32_t on_device);
/* Current frame (setCurrentImage + prepareCurrent, phototracker.cpp:236-245, 483-485). */
int recon_batch_set_current(recon_batch *b, const uint8_t *const *gray, const uint16_t *const *depth,
                            int32_t on_device);
int recon_batch_set_current_rgbd_float4(recon_batch *b, int32_t inst, const float *rgbd, int32_t on_device);

/* Runs the coarse-to-fine Gauss-Newton schedule for every instance
 * (gpuEstimateIncrement, phototracker.cpp:666-689).  T_io: n x 16 floats,
 * row-major, reference IR -> current IR; when non-NULL it is the initial pose
 * and receives the result.  stats: n entries or NULL.  Synchronises. */
int recon_batch_track(recon_batch *b, float *T_io, recon_track_stats *stats);
/* Same, asynchronous: poses stay on the device (recon_batch_get_poses). */
int recon_batch_track_async(recon_batch *b, const float *T_init_host);
int recon_batch_get_poses(recon_batch *b, float *T_out, recon_track_stats *stats);

/* Tracks nf consecutive current frames for every instance against its present
 * reference, each frame starting from the previous frame's pose (the
 * reference tracker's behaviour between reference updates,
 * phototracker.cpp:691-728).  gray/depth: nf x n pointers, row f = frame f of
 * every instance.  Host inputs are copied on a second stream into one device
 * slot per frame, overlapping frame f+1's upload with frame f's tracking
 * (pinned host memory makes the copies asynchronous); the slots keep the
 * frames until the next call (recon_batch_fuse_sequence reads them).  T_out:
 * nf x n x 16 floats (host) or NULL; stats: statistics of the last frame.
 * Synchronises once at the end. */
int recon_batch_track_sequence(recon_batch *b, int32_t nf, const uint8_t *const *gray, const uint16_t *const *depth,
                               int32_t on_device, float *T_out, recon_track_stats *stats);

/* Learned initialisation (include/recon_initnet.h; no counterpart in the
 * reference, which starts every frame from the previous frame's pose).  With a
 * network attached, each tracked frame (recon_batch_track without a T_init,
 * recon_batch_track_sequence) first predicts the motion from the previous
 * frame (the keyframe for the first frame) to the current one, takes the
 * predicted start pose where its coarse-level photometric residual is lower,
 * and runs `iters` (coarse to fine) instead of each instance's own schedule.
 * Frames must be uint8 / uint16 and a multiple of 80x60.  net = NULL restores
 * the plain tracker and the configured schedules.  The network object must
 * outlive its use by the batch. */
typedef struct recon_initnet recon_initnet;
int recon_batch_set_init_net(recon_batch *b, recon_initnet *net, const int32_t iters[RECON_MAX_LEVELS]);
/* The last frame's gate decisions (1: learned start pose) and network outputs [n][6]. */
int recon_batch_get_init(recon_batch *b, int32_t *choice, float *net_out);

/* Keyframe depth and colour fusion: fuses nframes (1..8) tracked frames into
 * every instance's keyframe.  depth: nframes x n uint16 mm maps; gray:
 * nframes x n uint8 images, or NULL to fuse depth only (the vertex colours are
 * then kept).  T: nframes x n x 16 keyframe -> frame poses (host memory) as
 * returned by tracking.  Every valid keyframe pixel is warped into each frame and back;
 * a frame's depth that agrees within gate_mm enters the running mean of the
 * pixel's depth, and its gray sample at the point enters the running mean of
 * the pixel's vertex colour (which then replaces the keyframe's own sample as
 * the photometric reference intensity at level 0).  The photometric selection
 * and Jacobians and the ICP reference pyramid are rebuilt from the fused depth
 * with the keyframe's gray image; the current pose is kept.  Runs on the
 * batch's second (reconstruction) stream; later tracking on the pose stream
 * waits for it.  Reference analogues: filterDepthIIRKernel (warp.cu:398-467,
 * disabled), updateVoxelsKernel's running mean (VoxelGrid_cuda.cu:1005-1013),
 * KeyFrameModel::integrateDepthMaps, which warps the neighbours' depth and RGB
 * into the keyframe (KeyFrameModel.cpp:537-583, not compiled). */
int recon_batch_fuse_keyframe_rgbd(recon_batch *b, int32_t nframes, const uint8_t *const *gray,
                                   const uint16_t *const *depth, const float *T, int32_t on_device, float gate_mm);
/* The same fusion (depth and colour) of the first nframes frames of the last
 * recon_batch_track_sequence call, with their tracked poses: frames, poses and
 * pointer tables are all taken on the device (the caller's device frames, or
 * the library's device copies of host frames), so nothing is copied and the
 * host does not wait.  It fails with RECON_ERR_STATE if that sequence had
 * fewer frames. */
int recon_batch_fuse_sequence(recon_batch *b, int32_t nframes, float gate_mm);
/* Depth only, host poses: recon_batch_fuse_keyframe_rgbd with gray = NULL. */
int recon_batch_fuse_keyframe(recon_batch *b, int32_t nframes, const uint16_t *const *depth, const float *T_host,
                              int32_t on_device, float gate_mm);

int recon_batch_set_iterations(recon_batch *b, int32_t inst, const int32_t iters[RECON_MAX_LEVELS]);
int recon_batch_set_mode(recon_batch *b, int32_t inst, int32_t mode, float lambda);
/* Settle rule of instance `inst` (recon_config.settle_mm / settle_rot): with
 * tol_mm > 0 the instance leaves a pyramid level once one GN iteration has
 * moved every translation entry of its pose by at most tol_mm and every
 * rotation entry by at most tol_rot; the level's iteration count is the cap.
 * tol_mm = 0 restores the reference's fixed schedule (gpuEstimateIncrement,
 * phototracker.cpp:666-689, has no early exit).  Both must be finite, >= 0. */
int recon_batch_set_settle(recon_batch *b, int32_t inst, float tol_mm, float tol_rot);

/* Tile shape of the linearisation kernel at each pyramid level: ICP chunks of
 * 1024 pixels per CTA, 1..64, or 0 for the built-in choice.  Poses and sums do
 * not depend on it (the normal equations are exact integer sums); only the
 * speed does.  recon_gb300.tune.autotune_icp_chunks picks it by timing.  No
 * reference counterpart: the reference launches fixed 1024-thread blocks. */
int recon_batch_set_icp_chunks_per_cta(recon_batch *b, const int32_t per_level[RECON_MAX_LEVELS]);
/* The values in effect (the built-in choice resolved), 0 for unused levels. */
int recon_batch_get_icp_chunks_per_cta(recon_batch *b, int32_t per_level[RECON_MAX_LEVELS]);

/* Per-iteration trace of instance `inst` (enabled with max_iters > 0). */
int recon_batch_enable_trace(recon_batch *b, int32_t max_iters);
int recon_batch_get_trace(recon_batch *b, int32_t inst, recon_iter_trace *out, int32_t max);

/* Measurement hooks (used by the benchmark).  Timing brackets every launch of
 * the schedule with CUDA events on the batch's stream; totals per kernel kind
 * (0 GN iteration linearisation, 1 ICP mask, 2 Student-t passes, 3
 * current-frame preparation, 4 reference preparation, 5 GN iteration solve and
 * pose update, 6 ICP preparation of a small level in one launch, 7 keyframe
 * fusion) accumulate in
 * recon_batch_get_poses and are read with recon_batch_get_timing.  Work
 * counters: per instance [photometric point-iterations, ICP point-iterations,
 * ICP mask pixels, 0]. */
int recon_batch_enable_timing(recon_batch *b, int32_t on);
int recon_batch_get_timing(recon_batch *b, double *ms, int64_t *launches, int32_t reset);
int recon_batch_get_work(recon_batch *b, uint64_t *out, int32_t reset);
void *recon_batch_stream(recon_batch *b); /* the cudaStream_t all work of the batch runs on */
int64_t recon_launch_count(void);         /* kernels launched by the library so far (graph replays included) */

/* Copies an internal device array of instance `inst` to host memory (tests).
 * Names: ref_gray, cur_gray, ref_z, ref_col, cur_z, ref_pts, ref_nrm, cur_pts, sel_idx,
 * sel_xyz, sel_I, sel_J, gmag, grad_hist, icp_nsel, and icp_mask (uint8) /
 * icp_w (float) per pixel of the last level the ICP term prepared (`level`
 * gives its size; icp_w is 0 where the pixel is not a correspondence).
 * Returns bytes. */
int64_t recon_batch_get_array(recon_batch *b, int32_t inst, const char *name, int32_t level, void *host_dst,
                              int64_t nbytes);

/* ---- allocation-free photometric iteration ----
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they track -- a real-time frame loop where a cudaMalloc could
 * synchronise the device and stall the frame, or a host framework that owns
 * all device memory and hands a plug-in only buffers it created -- this runs
 * one photometric Gauss-Newton iteration (residuals and depth weights,
 * histogram-MAD Tukey weights, 27-term normal equations, FP64 solve, SE(3)
 * update of T_dev) without allocating anything.  Its scratch is a fixed
 * device array inside the library, sized for RECON_NOALLOC_MAX_POINTS points
 * (128 KB, held on every GPU that loads the library until the process exits);
 * larger n_points is rejected with RECON_ERR_INVALID_ARG.  Every call shares
 * that array, so calls that overlap on the GPU (other streams or host threads)
 * race and must be serialised by the caller.  The first call on a device looks
 * up the array's device address and keeps it; make that first call before any
 * stream capture, and do not call it again on a device after cudaDeviceReset
 * (the kept address belongs to the reset context).  All pointers in the view
 * and T_dev are device memory; the result equals one iteration of
 * recon_batch_track in PHOTOMETRIC mode.  A solve whose pivot is not positive
 * leaves T_dev where it was (re-orthonormalised) and is not reported here;
 * the batch entry point counts it in recon_track_stats.non_spd. */
#define RECON_NOALLOC_MAX_POINTS 16384
typedef struct recon_photo_view {
    int32_t n_points;                 /* selected points P, multiple of 1024, <= RECON_NOALLOC_MAX_POINTS */
    int32_t level;                    /* pyramid level of img */
    int32_t img_width, img_height;    /* size of img: (depth_width >> level) x (depth_height >> level) */
    int32_t depth_width, depth_height; /* level-0 size of depth */
    int32_t hist_bins;                /* MAD histogram bins (64 in the reference) */
    int32_t solver;                   /* RECON_SOLVER_* */
    float opt_scale_out;              /* 1e3 */
    float calib[RECON_CALIB_SIZE];
    const float *xyz;                 /* 3 x P keyframe points (x block, y block, z block) */
    const float *intensity;           /* P keyframe intensities at `level` */
    const float *jacobian;            /* 6 x P precomputed photometric Jacobian at `level` */
    const float *img;                 /* current gray image at `level`, values in [0,1] */
    const float *depth;               /* current level-0 depth, z = -mm (0 = invalid) */
} recon_photo_view;
int recon_photometric_iteration_noalloc(const recon_photo_view *view, float *T_dev, void *stream);

/* ---- self-test of the Student-t truncation (no reference counterpart) ----
 * The Student-t passes truncate r2 * w in [0, 2^23) to an integer with a
 * round-toward-zero add of 2^23 instead of a conversion.  This compares the
 * two for every float in [0, 2^23) on the current GPU and stores the number of
 * mismatches (0 on a correct device). */
int recon_selftest_exact_arith(int64_t *mismatches);

/* ---- single tracker (PhotoTracker-style handle = batch of one) ---- */
typedef recon_batch recon_tracker;
int recon_tracker_create(const recon_config *cfg, const float *calib, void *stream, recon_tracker **out);
int recon_tracker_destroy(recon_tracker *t);
int recon_set_reference(recon_tracker *t, const uint8_t *gray, const uint16_t *depth, int32_t on_device);
int recon_set_reference_oriented(recon_tracker *t, const uint8_t *gray, const uint16_t *depth, const float *points,
                                 const float *normals, int32_t on_device);
int recon_set_current(recon_tracker *t, const uint8_t *gray, const uint16_t *depth, int32_t on_device);
int recon_track(recon_tracker *t, float T_io[16], recon_track_stats *stats);
int recon_set_iterations(recon_tracker *t, const int32_t iters[RECON_MAX_LEVELS]);
int recon_set_mode(recon_tracker *t, int32_t mode, float lambda);
int recon_set_settle(recon_tracker *t, float tol_mm, float tol_rot); /* recon_batch_set_settle */
/* getRelativePose / getGlobalPose / resetTracking (phototracker.cpp:223-262).
 * After each recon_track the host pose bookkeeping follows applyIncrement
 * (phototracker.cpp:514-531): the relative pose T is the tracked pose
 * inverted in double and stored as float (current -> reference), the
 * increment inv(double(T_previous)) * inv(double(T_tracked)) is accumulated
 * into the double global pose.  A new reference resets T to the identity and
 * keeps the global pose; recon_reset clears both. */
int recon_get_relative_pose(recon_tracker *t, float T[16]);
int recon_get_global_pose(recon_tracker *t, double T[16]);
int recon_reset(recon_tracker *t);

/* Keyframe trigger (setReferenceUpdating, poseDifferenceExceeded,
 * referenceOutdated; phototracker.cpp:62-68, 268-296, thresholds 125 mm /
 * 12.5 deg at phototracker.cpp:127-128).  recon_pose_difference_exceeded: 1
 * when the translation of dT is longer than dist_mm or its rotation angle
 * (from the unit quaternion) exceeds angle_deg, else 0.
 * recon_reference_outdated: 1 when the tracker has no reference, or when
 * reference updating is on and its relative pose exceeds the thresholds (the
 * caller then sets a new reference), else 0.  The batch form tests every
 * instance's tracked pose (inverted in double, stored as float, as the
 * reference tests its host pose) into outdated[n]. */
int recon_pose_difference_exceeded(const float dT[16], float dist_mm, float angle_deg);
int recon_set_reference_updating(recon_tracker *t, int32_t on, float dist_mm, float angle_deg);
int recon_reference_outdated(recon_tracker *t);
int recon_batch_reference_outdated(recon_batch *b, float dist_mm, float angle_deg, int32_t *outdated);

/* ---- result files (tracker/calib/ResultTxt.cpp:17-76, TrackingParams.cpp:50-95) ----
 * recon_trajectory_save: ResultTxt::save -- n poses (n x 16 float, row-major,
 * e.g. the global poses of successive frames as float, main.cpp:942) are
 * left-multiplied by the inverse of the first (canonize, float arithmetic in
 * the reference's order) and written one per line as "i: " and 16 values in
 * %e; transpose / inverse as ResultTxt::save's flags (the reference writes
 * transpose 1, inverse 0: the row-major matrix; main.cpp:383).  At most 10000
 * poses are written (MAX_POSE_COUNT).
 * recon_trajectory_load: reads such a file back (transpose as it was written);
 * returns the number of poses.
 * recon_track_params_load: TrackingParams::init -- lines "frame mode error",
 * mode geometric (lambda 1), photometric (lambda 0) or biobjective-lambda<x>;
 * returns the number of entries (all are counted, max_n are stored) or an
 * error naming the line of an unknown mode.
 * recon_track_params_lookup: TrackingParams::getParams -- index of the entry
 * whose frame is nearest to `frame` (the first on ties), -1 without entries
 * (the reference then uses GEOMETRIC). */
int recon_trajectory_save(const char *path, const float *poses, int32_t n, int32_t transpose, int32_t inverse);
int32_t recon_trajectory_load(const char *path, float *poses, int32_t max_n, int32_t transpose);
int32_t recon_track_params_load(const char *path, int32_t *frames, int32_t *modes, float *lambdas, int32_t max_n);
int32_t recon_track_params_lookup(const int32_t *frames, int32_t n, int32_t frame);

/* ---- procedural RGB-D renderer (inputs for tests and benchmarks) ----
 * scene / camera: the recon_scene / recon_camera structs of
 * recon_gb300/csrc/scene.h.  Output pointers are device memory. */
int recon_render_depth(const void *scene, const void *camera, float noise_rel, uint32_t noise_seed, uint32_t frame,
                       uint16_t *depth_dev, void *stream);
int recon_render_gray(const void *scene, const void *camera, uint8_t *gray_dev, void *stream);

#ifdef __cplusplus
}
#endif
