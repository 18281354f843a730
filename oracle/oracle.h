/*
 * oracle.h -- CPU oracle for the recon dense RGB-D tracking hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain-C restatement of the
 * reference tracker's GPU kernels (ttykkala/recon, the .cu files under tracker/kernels) and of
 * its per-level Gauss-Newton schedule (tracker/tracker/phototracker.cpp,
 * shapetracker.cpp).  It is used by the tests as the checker, by bench.py as the
 * timed CPU baseline, and by nothing else: the product library never links it.
 *
 * Floating point: every FP32 expression is evaluated in the reference's source
 * order with no FMA contraction (compile with -ffp-contract=off), so results are
 * bit-identical to a GPU build of the same expressions with -fmad=false.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* calibData layout, tracker/calib/calib.h:22-37 */
#define ORC_KR_OFFSET 0
#define ORC_IKR_OFFSET 9
#define ORC_KCR_OFFSET 18
#define ORC_TLR_OFFSET 26
#define ORC_C1_OFFSET 42
#define ORC_KL_OFFSET 43
#define ORC_IKL_OFFSET 52
#define ORC_C0_OFFSET 61
#define ORC_MIND_OFFSET 62
#define ORC_MAXD_OFFSET 63
#define ORC_TRL_OFFSET 64
#define ORC_CALIB_SIZE 96

/* tracker modes, tracker/tracker/phototracker.h:30 */
#define ORC_GEOMETRIC 0
#define ORC_PHOTOMETRIC 1
#define ORC_BIOBJECTIVE 2

#define ORC_SOLVER_CHOLESKY 0
#define ORC_SOLVER_CG 1

#define ORC_MAX_LEVELS 4
#define ORC_CHUNK 1024 /* canonical reduction chunk (points) */

typedef struct orc_config {
    int32_t width, height, levels;
    int32_t n_select;    /* photometric points, phototracker.cpp:48 */
    int32_t hist_bins;   /* MAD histogram bins, histogram64.cu (64) */
    int32_t select_bins; /* pixel-selection histogram bins, phototracker.cpp:346 (256) */
    int32_t solver;
    int32_t mode;
    float lambda;
    int32_t iters[ORC_MAX_LEVELS]; /* coarse -> fine, phototracker.cpp:148-149 */
    float opt_scale_in;            /* phototracker.cpp:50 */
    float opt_scale_out;           /* phototracker.cpp:51 */
    int32_t precision;             /* 0 FP32; 1 mixed: FP16 current images and reference
                                      intensities, BF16 photometric Jacobians (values rounded
                                      to nearest even on storage, FP32 arithmetic) */
    float settle_mm;               /* > 0: a level ends early once one iteration moves every
                                      translation entry by <= settle_mm and every rotation entry
                                      by <= settle_rot (orc_pose_settled); 0: fixed schedule */
    float settle_rot;
} orc_config;

/* float -> nearest binary16 / bfloat16 value (ties to even), widened back to float */
float orc_f16_round(float x);
float orc_bf16_round(float x);

typedef struct orc_iter_trace {
    int32_t level, iter, mode, solved, icp_selected, status;
    float T[16];
    double A[36];
    double b[6];
    double A_ph[36], b_ph[6], A_icp[36], b_icp[6];
    int32_t hist[256];
    int32_t median_bin;
    int32_t pad_;
} orc_iter_trace;

typedef struct orc_tracker orc_tracker;

/* ---- calibration (calib.cpp:74-93) ---- */
void orc_calib_setup(const double KL[9], const double KR[9], const double TLR[16], const double kcR[8],
                     double minDist, double maxDist, double c0, double c1, int width, float *calib);

/* ---- input conversion (rgb2gray.cu:64-87 restated for uint8 gray / uint16 mm depth) ---- */
void orc_convert_gray(const uint8_t *g, int n, float *out);
void orc_convert_depth(const uint16_t *d, int n, float *z);
void orc_rgbd_float4_to_gray_z(const float *rgbd, int W, int H, const float *calib, float *gray, float *z);
void orc_downsample2(const float *hi, int wlo, int hlo, float *lo);

/* ---- photometric reference preparation ---- */
void orc_zmap_to_xyz(const float *z, int W, int H, const float *calib, float *xyzw);
void orc_xyz2cloud(const float *xyzw, int W, int H, const float *calib, const float *gray0, float *vdata);
void orc_xyz2cloud_col(const float *xyzw, int W, int H, const float *calib, const float *gray0, const float *col,
                       float *vdata);
void orc_grad_histogram(const float *grad, int n, int nbins, int32_t *hist);
int orc_filter_indices(const float *grad, int n, const int32_t *hist, int nbins, int P, int32_t *idx_out);
void orc_add_vertex_attributes(const int32_t *idx, int P, float *vdata, int W, int H, const float *calib,
                               const float *const *gray, int L);
void orc_precompute_jacobian(const int32_t *idx, int P, const float *vdata, const float *calib, float optScaleIn,
                             int L, float *const *J);

/* ---- photometric iteration ---- */
void orc_interpolate_residual(int P, const float *sel_xyz, const float *sel_I, const float *T, const float *calib,
                              int layer, const float *img, int w, int h, const float *zcur, int zw, int zh,
                              float *residual, float *zweight);
int orc_generate_weights(const float *r, const float *zw, int N, int nbins, int32_t *hist, float *w, float *rw);
void orc_reduce27(const float *const *J6, const float *r, int N, double A[36], double b[6]);
void orc_reduce27_refordered(const float *const *J6, const float *r, int N, float A[36], float b[6]);

/* Exact fixed-point accumulation of FP32 values (the tracker's reduction): a
 * value v is the integer sum_k L[k] * 2^(32k) in units of 2^-64; FP32 inputs
 * are truncated toward zero at 2^-64 and must satisfy |v| < 2^48 (else `bad`). */
#define ORC_FX_LIMBS 4
typedef struct orc_fx27 {
    long long L[27][ORC_FX_LIMBS];
    int bad;
} orc_fx27;
void orc_fx_add(long long L[ORC_FX_LIMBS], float v, int *bad);
double orc_fx_to_double(const long long L[ORC_FX_LIMBS]);
void orc_fx27_clear(orc_fx27 *acc);
void orc_reduce27_fx(const float *const *J6, const float *r, int N, orc_fx27 *acc);
void orc_fx27_value(const orc_fx27 *acc, double A[36], double b[6]);

/* ---- ICP ---- */
void orc_zmap_to_xyz6(const float *z, int W, int H, const float *calib, float *pts6, int32_t *mask);
void orc_compute_normals6(float *pts6, int32_t *mask, int W, int H);
void orc_gen_cloud6(const float *z, int W, int H, const float *calib, float *pts6, int32_t *mask);
void orc_downsample_cloud6(const float *src6, const int32_t *msrc, int wlo, int hlo, float *dst6, int32_t *mdst);
void orc_icp_residual_mask(const float *ref6, const int32_t *refmask, int w, int h, const float *T,
                           const float *calib, const float *cur6, const int32_t *curmask, int layer,
                           float *residual, int32_t *rmask);
int orc_compact(const int32_t *mask, int n, int32_t *select);
void orc_student_t(const float *r2, int n, float *w);
void orc_icp_residual_jacobian(const float *ref6, const int32_t *select, int nsel, int w, int h, int layer,
                               const float *T, const float *calib, const float *cur6, const int32_t *curmask,
                               int npadded, float *r, float *J, const float *weights, float optScaleIn);
/* the tracker's form over the pixel grid (fused multiply-adds in the continuous terms) */
void orc_icp_residual_jacobian_grid(const float *ref6, int w, int h, int layer, const float *T, const float *calib,
                                    const float *cur6, const int32_t *curmask, int npadded, float *r, float *J,
                                    const float *weights, float optScaleIn);

/* ---- solve and SE(3) update ---- */
int orc_solve_cholesky(const double A[36], const double b[6], double x[6]);
void orc_solve_cg(const double A[36], const double b[6], double tol, int maxSteps, double x[6]);
void orc_expm_update(const double x[6], float T[16], double scaleOut);
void orc_expm_twist(const double A[16], double E[16]);
void orc_linear_fuse(double A1[36], double b1[6], double w1, int N1, const double A2[36], const double b2[6],
                     double w2, int N2);

/* ---- keyframe fusion ---- */
void orc_fuse_depth(const float *zkey, int W, int H, const float *calib, int nframes, const float *const *zframes,
                    const float *Tframes, float gate_mm, float *zout, float *wout);
void orc_fuse_rgbd(const float *zkey, const float *gkey, int W, int H, const float *calib, int nframes,
                   const float *const *zframes, const float *const *gframes, const float *Tframes, float gate_mm,
                   float *zout, float *wout, float *cout);

/* ---- whole tracker (operator level, phototracker.cpp / shapetracker.cpp) ---- */
orc_tracker *orc_create(const orc_config *cfg, const float *calib);
/* 1 if no translation entry of the pose moved by more than tol_mm and no
 * rotation entry by more than tol_rot between Ta and Tb (float differences,
 * exact comparisons: the GPU takes the same decision from the same poses) */
int orc_pose_settled(const float Ta[16], const float Tb[16], float tol_mm, float tol_rot);
void orc_destroy(orc_tracker *t);
int orc_set_reference(orc_tracker *t, const uint8_t *gray, const uint16_t *depth);
int orc_set_reference_float(orc_tracker *t, const float *gray0, const float *z0);
int orc_set_current(orc_tracker *t, const uint8_t *gray, const uint16_t *depth);
void orc_gen_oriented_points6(const float *xyz4, const float *nrm4, int W, int H, float *pts6, int32_t *mask);
int orc_set_reference_oriented(orc_tracker *t, const uint8_t *gray, const uint16_t *depth, const float *xyz4,
                               const float *nrm4);
int orc_fuse_keyframe(orc_tracker *t, int nframes, const uint16_t *const *depth, const float *Tframes, float gate);
int orc_fuse_keyframe_rgbd(orc_tracker *t, int nframes, const uint8_t *const *gray, const uint16_t *const *depth,
                           const float *Tframes, float gate);
int orc_track(orc_tracker *t, float *T, orc_iter_trace *trace, int max_trace);
/* learned start pose gate (k_init_gate); 1 when the network's candidate was taken */
int orc_init_gate(orc_tracker *t, const float net_out[6], const float scale[6]);
void orc_set_pose(orc_tracker *t, const float T[16]);
void orc_get_pose(orc_tracker *t, float T[16]);
int orc_get_array(orc_tracker *t, const char *name, int level, void *dst, int64_t nbytes);
int orc_n_icp_selected(orc_tracker *t, int level);

/* ---- FP64 oracle (oracle_fp64.c): the same tracker with every operation in
 * double and the pose kept in double; the judge of pose error ---- */
typedef struct orc64_tracker orc64_tracker;
orc64_tracker *orc64_create(const orc_config *cfg, const float *calib);
void orc64_destroy(orc64_tracker *t);
int orc64_set_reference(orc64_tracker *t, const uint8_t *gray, const uint16_t *depth);
int orc64_set_current(orc64_tracker *t, const uint8_t *gray, const uint16_t *depth);
/* depth and (gray non-NULL) colour fusion of nframes frames, poses keyframe -> frame */
int orc64_fuse_keyframe(orc64_tracker *t, int nframes, const uint8_t *const *gray, const uint16_t *const *depth,
                        const double *Tframes, double gate);
/* the plain schedule from T (NULL: the tracker's pose); returns iterations run */
int orc64_track(orc64_tracker *t, double *T);
void orc64_get_pose(const orc64_tracker *t, double T[16]);
void orc64_set_pose(orc64_tracker *t, const double T[16]);
int orc64_get_array(orc64_tracker *t, const char *name, int level, void *dst, int64_t nbytes);

/* ---- reconstruction stream (oracle_tsdf.c): TSDF fusion and ray cast,
 * tracker/kernels/VoxelGrid_cuda.cu; grid = R^3 float2 (tsdf, weight), x fastest ---- */
typedef struct orc_tsdf_params {
    int32_t R;           /* voxels per side (SimParams.gridResolution) */
    float origin[3];     /* SimParams.cubeOrigin */
    float dim[3];        /* SimParams.cubeDim: half the side length */
    int32_t W, H;        /* SimParams.winWidth / winHeight */
    float min_dist, max_dist;
} orc_tsdf_params;
void orc_tsdf_invert_rt4(const float *M, float *Mi);
void orc_tsdf_reset(float *grid, int64_t nvox);
void orc_tsdf_dist_from_rgbd(const float *rgbd, int W, int H, float min_dist, float max_dist, float *dist);
void orc_tsdf_update(float *grid, const orc_tsdf_params *p, const float *dist, const float Tcur[16], const float K[9]);
void orc_tsdf_raycast(const float *grid, const orc_tsdf_params *p, const float Tcur[16], const float K[9],
                      int filtering, float *xyz);
void orc_tsdf_shade(const float *xyz, int W, int H, float *shaded, float *normal);
void orc_tsdf_resample(float *dst, const float *src, const orc_tsdf_params *p, const float Tcur[16]);

/* ---- Kinect pre-processing (oracle_kinect.c, tracker/multicore/multicore.cpp) ---- */
void orc_kinect_d2z(const uint16_t *disp, int W, int H, float c0, float c1, float min_dist, float max_dist,
                    float x_off, float y_off, float *z);
void orc_kinect_d2z_low(const uint16_t *disp, int Wl, int Hl, float c0, float c1, float min_dist, float max_dist,
                        float x_off, float y_off, float *z);
void orc_kinect_rgb2gray(const uint8_t *rgb, int W, int H, uint8_t *gray);
/* the GPU capture path (tracker/kernels/d2z.cu, rgb2gray.cu, undistort.cu) */
void orc_kinect_disparity_to_float(const uint16_t *disp, int n, float *out);
void orc_kinect_depth_normalized(const uint16_t *disp_u16, const float *disp_f32, int W, int H, float c0, float c1,
                                 float min_dist, float max_dist, float x_off, float y_off, float *z_low);
void orc_kinect_rgb_to_hdr(const uint8_t *rgb, int n, float *rgb_hdr);
void orc_kinect_rgb_to_gray_hdr(const uint8_t *rgb, int n, float *gray);
void orc_kinect_rgb_hdr_to_gray(const float *rgb_hdr, int n, float *gray);
void orc_kinect_undistort_rgb_hdr(const uint8_t *rgb, int W, int H, const float *K, const float *iK, const float *kc,
                                  float *rgb_hdr);
void orc_kinect_undistort(const uint8_t *src, int W, int H, const float *K, const float *iK, const float *kc,
                          uint8_t *dst);

/* ---- procedural scene (CPU twin of the GPU renderer) ---- */
struct recon_scene;
struct recon_camera;
void orc_render_depth(const struct recon_scene *sc, const struct recon_camera *cam, float noise_rel,
                      uint32_t noise_seed, uint32_t frame, uint16_t *out);
void orc_render_gray(const struct recon_scene *sc, const struct recon_camera *cam, uint8_t *out);

int orc_num_threads(void);
void orc_set_threads(int n);

#ifdef __cplusplus
}
#endif
