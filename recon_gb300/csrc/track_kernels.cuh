// track_kernels.cuh -- device-side instance descriptor shared by the kernels
// and the host code of librecon_track.so.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/recon_track.h"

namespace rt {

constexpr int kMaxLevels = 4;
constexpr int kChunk = 1024;     // canonical reduction chunk (points)
constexpr int kLanes = 256;      // lanes per chunk, 4 points each
constexpr int kSegments = 512;   // pixel-selection segments (filterIndex256.cu:183)
constexpr int kVtxPlanes = 9;    // a vertex record: x y z px py gx gy gmag gray
constexpr int kIterCluster = 8;  // CTAs of the photometric cluster of the GN iteration kernel
constexpr int kIterBlock = 256;  // threads of a GN iteration CTA
constexpr int kIterCtaSlots = 4 * 152;  // GN iteration CTAs resident on a 152-SM GB300
constexpr int kPassCtaSlots = 5 * 152;  // 256-thread Student-t pass CTAs resident on a 152-SM GB300
constexpr int kSolveThreads = 64;        // threads of the per-instance solve CTA
constexpr int kFxLimbs = 4;      // limbs of a fixed-point sum (fx.cuh)
constexpr int kNetW = 80, kNetH = 60;  // coarse image of the learned initialisation

// ST_SETTLED: level + 1 of the level the instance left early (settle rule), 0 if none this frame
enum StatSlot { ST_ITERS = 0, ST_SOLVES, ST_NONSPD, ST_STATUS, ST_MEDIAN, ST_ICPSEL0, ST_SETTLED = 9, ST_COUNT = 16 };

struct InstDesc {
    int W, H, L, P;
    int hist_bins, select_bins, mode, solver;
    float lambda, opt_in, opt_out;
    int precision;
    double fuse_c1;  // (double)(1 - lambda) / P, the photometric weight of the fused system
    int iters[kMaxLevels];
    float settle_mm, settle_rot;  // settle rule (recon_config); off at settle_mm 0
    float calib[RECON_CALIB_SIZE];
    // reference (keyframe)
    float *ref_gray[kMaxLevels];
    float *ref_z;
    float *ref_col;               // W*H fused vertex colour (keyframe fusion), -1 where none
    float4 *ref_pts[kMaxLevels];  // x y z mask
    float4 *ref_nrm[kMaxLevels];  // nx ny nz 0
    float *gmag;                  // W*H: the keyframe pixels' gradient magnitudes
    int *grad_hist;               // select_bins
    int *seg;                     // segment tables, 6 * kSegments + 4
    int *sel_idx;                 // P
    float *sel_xyz;               // 3 * P (SoA)
    float *sel_I[kMaxLevels];     // P
    float *sel_J[kMaxLevels];     // 6 * P (SoA)
    // mixed precision (precision == RECON_PRECISION_MIXED): the FP16 / BF16
    // copies the photometric term reads instead of sel_I, sel_J and cur_gray
    __half *sel_Ih[kMaxLevels];         // P
    __nv_bfloat16 *sel_Jb[kMaxLevels];  // 6 * P (SoA)
    __half *cur_grayh[kMaxLevels];      // W*H of the level
    // current frame
    float *cur_gray[kMaxLevels];
    float *cur_z;
    float4 *cur_pts[kMaxLevels];  // x y z mask
    // photometric scratch
    float *ph_r, *ph_zw;
    int *ph_hist;     // [256,512) the last histogram (for the trace), [512] its median bin
    // ICP scratch
    uint8_t *icp_mask;       // W*H: the pixel is a correspondence of the level
    float *icp_r2;           // W*H: its squared residual at the level's start pose
    float *icp_w;            // W*H: its Student-t weight, 0 where not selected
    int *icp_blkcnt;         // per 1024-pixel block: correspondences
    long long *icp_blkvar;   // per 1024-pixel block: first variance sum
    long long *icp_part;     // per Student-t pass CTA (at most one per block): its partial sum
    unsigned long long *icp_var;  // 4: the variance sums of the passes
    int *icp_nsel;           // kMaxLevels
    double *fuse_c2;         // kMaxLevels: lambda / (ICP correspondences) of the level
    // fixed-point sums of the current iteration: [0,108) photometric, [108,216) ICP
    unsigned long long *fx;
    int *fx_bad;             // 2: an accumulated value was out of range
    unsigned long long *work; // [0] photometric point-iterations, [1] ICP point-iterations, [2] ICP mask pixels
    unsigned int *counter;   // 4: [1] the Student-t passes' last-CTA ticket (k_icp_student_pass; reset by its last taker)
    float *T;                // 16, device pose (reference IR -> current IR)
    int *stats;              // ST_COUNT
    recon_iter_trace *trace;
    int trace_max;
    int *trace_count;
};

// Programmatic dependent launch.  The kernels of the per-frame schedule are
// launched so that the next kernel may start while this one finishes:
// pdl_trigger lets it be scheduled, and pdl_wait (griddepcontrol.wait) returns
// once every earlier kernel of the stream has completed and its writes are
// visible.  Before pdl_wait a kernel reads only the instance descriptors (not
// written by any kernel of the schedule) and writes nothing.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

// k_iter copies a descriptor into shared memory as 32-bit words
static_assert(sizeof(InstDesc) % sizeof(int) == 0, "InstDesc must be a whole number of words");

}  // namespace rt
