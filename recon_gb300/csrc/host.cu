// host.cu -- host side of librecon_track.so: instance memory, the per-frame
// launch schedule (captured as a CUDA graph) and the C ABI of
// include/recon_track.h.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/recon_initnet.h"
#include "scene.h"
#include "track_kernels.cuh"

namespace rt {
__global__ void k_convert_level0(const InstDesc *D, const uint8_t *const *in_gray, const uint16_t *const *in_depth,
                                 const float *const *in_rgbd);
__global__ void k_downsample(const InstDesc *D, int level, const int *active);
__global__ void k_normals(const InstDesc *D, const int *active);
__global__ void k_oriented_points(const InstDesc *D, const float *const *in_pts, const float *const *in_nrm);
__global__ void k_xyz2cloud(const InstDesc *D, const int *active);
__global__ void k_seg_count(const InstDesc *D, const int *active);
__global__ void k_seg_scan(const InstDesc *D, const int *active);
__global__ void k_seg_scatter(const InstDesc *D, const int *active);
__global__ void k_attr_jac(const InstDesc *D, const int *active);
__global__ void k_icp_mask(const InstDesc *D, int level);
constexpr int kPyrTile = 32;  // level-0 tile of k_prep_current_pyramid
__global__ void k_prep_current_pyramid(const InstDesc *D, const uint8_t *const *in_gray,
                                       const uint16_t *const *in_depth, const float *const *in_rgbd, int tiles_x,
                                       float *store_prev, int begin);
__global__ void k_icp_student_pass(const InstDesc *D, int level, int pass, int blocks_per_cta);
__global__ void k_icp_prepare(const InstDesc *D, int level);
__global__ void k_iter(const InstDesc *D, int level, int it, int icp_per_cta, int n_inst, int icp_ctas);
__global__ void k_solve(const InstDesc *D, int level, int it);
__global__ void k_render_depth(recon_scene sc, recon_camera cam, float noise_rel, uint32_t seed, uint32_t frame,
                               uint16_t *out);
__global__ void k_render_gray(recon_scene sc, recon_camera cam, uint8_t *out);
__global__ void k_reset_pose(const InstDesc *D, const int *active);
__global__ void k_begin_track(const InstDesc *D, const float *T_init, int have_init);
__global__ void k_clear_ref(const InstDesc *D, const int *active);
__global__ void k_store_pose(const InstDesc *D, float *dst);
__global__ void k_gather_results(const InstDesc *D, int *dst);
__global__ void k_fuse_depth(const InstDesc *D, int nframes, int n_inst, const uint16_t *const *depth,
                             const uint8_t *const *gray, const float *Tf, float gate, const int *active);
__global__ void k_ref_from_z(const InstDesc *D, const int *active);
__global__ void k_net_coarse(const InstDesc *D, const uint8_t *const *in_gray, const uint16_t *const *in_depth,
                             const __nv_bfloat16 *prev, __nv_bfloat16 *out, __nv_bfloat16 *net_in);
__global__ void k_gate_twist(const InstDesc *D, const float *net_out, const float *scale, float *Dout);
__global__ void k_gate(const InstDesc *D, const float *Dm_all, long long *cost, unsigned int *ticket, float *cand,
                       int *choice);
}  // namespace rt

namespace nn {
int forward_on(recon_initnet *net, const uint16_t *in_bf16, int n, float *out, cudaStream_t s);
const float *scale_dev(recon_initnet *net);
int forward_kernels(int n);
}  // namespace nn

using namespace rt;

namespace {

thread_local std::string g_last_error;
std::atomic<long long> g_launches{0};  // kernels launched by this library (graph replays included)

int fail(int code, const char *msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return RECON_ERR_CUDA;
}

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);        \
    } while (0)

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// The runtime's last-error slot is per host thread and shared with every other
// CUDA user in the process; an error left there by unrelated code must not be
// reported as a failure of this library's launches.
void clear_stale_error() { (void)cudaGetLastError(); }

}  // namespace

namespace rt {
// lets other translation units of the library report a message through recon_last_error
void set_last_error(const char *msg) { g_last_error = msg; }
void add_launches(long long n) { g_launches += n; }
}  // namespace rt

namespace {

struct Arena {
    size_t off = 0;
    char *base = nullptr;
    template <class T> T *take(size_t count) {
        size_t o = off;
        off = align256(off + count * sizeof(T));
        return base ? reinterpret_cast<T *>(base + o) : nullptr;
    }
};

}  // namespace

struct recon_batch {
    int n = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::vector<recon_config> cfg;
    std::vector<InstDesc> desc;
    std::vector<void *> arenas;
    InstDesc *d_desc = nullptr;
    // input pointer tables (5 x n: gray, depth, float4 RGB-D, oriented points,
    // their normals) and staging for host uploads
    const void **d_inptr = nullptr;
    std::vector<const void *> h_inptr;
    int *d_active = nullptr;
    uint8_t *d_stage = nullptr;
    size_t stage_bytes = 0;
    float *d_Tinit = nullptr;
    // [n][32] words: each instance's pose (16 floats) and statistics (16 ints),
    // gathered by one kernel so the results come back in one copy
    int *d_results = nullptr;
    int *h_results = nullptr;  // pinned
    int trace_max = 0;
    recon_iter_trace *d_trace = nullptr;
    int *d_trace_count = nullptr;
    bool have_ref = false, have_cur = false;
    // schedule graph
    cudaGraphExec_t graph = nullptr;
    bool graph_dirty = true;
    int max_pix = 0, max_L = 0, max_P = 0;
    long long graph_kernels = 0;
    // ICP chunks of 1024 pixels per k_iter CTA at each level (0: built-in choice)
    int icp_cpc[kMaxLevels] = {0, 0, 0, 0};
    // optional per-launch CUDA-event timing (kinds: see TimingKind)
    bool timing = false;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> graph_events, direct_events;
    std::vector<cudaEvent_t> event_pool;  // reused by timed direct launches
    size_t pool_next = 0;
    double t_ms[8] = {0};
    long long t_cnt[8] = {0};
    // sequence tracking: pointer tables, pose history, host-input double buffer
    const void **d_seqptr = nullptr;
    size_t seqptr_cap = 0;
    const void **h_seqptr = nullptr;  // pinned
    float *d_Tseq = nullptr;
    size_t Tseq_cap = 0;
    int seq_frames = 0;  // frames of the last recon_batch_track_sequence call (their poses are in d_Tseq)
    // host-input sequences: one device slot per frame of the call (kept after
    // the call, so that recon_batch_fuse_sequence can read the frames), in two
    // sets used by alternate calls: a call's copies need not wait for a
    // fusion that still reads the previous call's frames
    uint8_t *d_slots = nullptr;
    size_t set_bytes = 0;  // bytes of one set
    int next_set = 0;
    int seq_set = -1;  // the set of the last sequence (-1: device frames)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copied[2] = {nullptr, nullptr};
    // the last reads of each set: the tracking of the call that used it (batch
    // stream) and a fusion of its frames (reconstruction stream)
    cudaEvent_t ev_set_read[2] = {nullptr, nullptr}, ev_set_fused[2] = {nullptr, nullptr};
    // keyframe fusion runs on a second stream (the reference's reconstruction GPU)
    cudaStream_t recon_stream = nullptr;
    cudaEvent_t ev_pose = nullptr, ev_fused = nullptr;
    uint8_t *d_fuse = nullptr;
    size_t fuse_bytes = 0;
    const void **d_fuse_ptr = nullptr;
    const void **h_fuse_ptr = nullptr;  // pinned: the fusion's pointer table
    int *d_all_active = nullptr;        // [n] ones: the fusion updates every instance
    float *d_fuse_T = nullptr;
    size_t fuse_cap = 0;
    // host pose bookkeeping for the single-tracker API (applyIncrement):
    // T_host is the reference's host pose T, current -> reference, float
    double global_pose[16];
    float T_host[16];
    // keyframe policy (setReferenceUpdating / referenceOutdated)
    bool ref_updating = false;
    float ref_dist_mm = 125.0f, ref_angle_deg = 12.5f;  // phototracker.cpp:127-128
    // learned initialisation (recon_batch_set_init_net)
    recon_initnet *net = nullptr;
    uint16_t *d_coarse[2] = {nullptr, nullptr};  // coarse images [n][60][80][2] BF16: previous / current frame
    int coarse_prev = 0;
    uint16_t *d_netin = nullptr;  // [n][60][80][4]
    float *d_netout = nullptr;    // [n][6]
    // sequences: the network runs one frame ahead on net_stream (its input
    // does not depend on the poses), into alternate output buffers
    float *d_netout_seq[2] = {nullptr, nullptr};
    const float *netout_last = nullptr;  // the outputs recon_batch_get_init reports
    cudaStream_t net_stream = nullptr;
    cudaEvent_t ev_net[2] = {nullptr, nullptr}, ev_gate[2] = {nullptr, nullptr}, ev_seq = nullptr;
    int *d_choice = nullptr;      // [n]: 1 where the learned start pose was taken
    float *d_cand = nullptr;      // [n][16]: candidate start poses
    long long *d_cost = nullptr;  // [n][2]: gate costs of the current pose and the candidate (0 between frames)
    unsigned int *d_ticket = nullptr;  // [n]: CTAs of the gate that finished (0 between frames)
    float *d_gateD = nullptr;     // [n][16]: exp of the network twist (single-frame path)
    float *d_gateD_seq[2] = {nullptr, nullptr};  // the same for alternate frames of a sequence
    std::vector<std::vector<int>> plain_iters;  // schedules restored when the network is detached
};

namespace {

void identity16(float *T) {
    for (int i = 0; i < 16; i++) T[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}
void identity16d(double *T) {
    for (int i = 0; i < 16; i++) T[i] = (i % 5 == 0) ? 1.0 : 0.0;
}

int validate(const recon_config &c) {
    if (c.width < 32 || c.height < 16) return fail(RECON_ERR_INVALID_ARG, "image too small");
    if (c.levels < 1 || c.levels > RECON_MAX_LEVELS) return fail(RECON_ERR_INVALID_ARG, "levels must be 1..4");
    int m = 1 << (c.levels - 1);
    if (c.width % m || c.height % m) return fail(RECON_ERR_INVALID_ARG, "size not divisible by 2^(levels-1)");
    if (c.n_select <= 0 || c.n_select % kChunk) return fail(RECON_ERR_INVALID_ARG, "n_select must be a positive multiple of 1024");
    if (c.n_select > c.width * c.height) return fail(RECON_ERR_INVALID_ARG, "n_select exceeds the pixel count");
    if ((c.width * c.height) / kSegments > 1024) return fail(RECON_ERR_INVALID_ARG, "image too large for the 512-segment selection");
    if (c.hist_bins < 2 || c.hist_bins > 256) return fail(RECON_ERR_INVALID_ARG, "hist_bins must be 2..256");
    if (c.select_bins < 2 || c.select_bins > 1024) return fail(RECON_ERR_INVALID_ARG, "select_bins must be 2..1024");
    if (c.mode < 0 || c.mode > 2) return fail(RECON_ERR_INVALID_ARG, "bad mode");
    if (c.solver < 0 || c.solver > 1) return fail(RECON_ERR_INVALID_ARG, "bad solver");
    for (int l = 0; l < RECON_MAX_LEVELS; l++)
        if (c.iters[l] < 0 || c.iters[l] > 1000) return fail(RECON_ERR_INVALID_ARG, "bad iteration count");
    if (!(c.lambda >= 0.0f && c.lambda <= 1.0f)) return fail(RECON_ERR_INVALID_ARG, "lambda must be in [0,1]");
    if (c.precision != RECON_PRECISION_FP32 && c.precision != RECON_PRECISION_MIXED)
        return fail(RECON_ERR_INVALID_ARG, "bad precision");
    if (!(c.settle_mm >= 0.0f && c.settle_mm <= FLT_MAX && c.settle_rot >= 0.0f && c.settle_rot <= FLT_MAX))
        return fail(RECON_ERR_INVALID_ARG, "settle tolerances must be finite and >= 0");
    return RECON_OK;
}

// lays out (base == nullptr: sizes only) the device buffers of one instance
size_t layout(InstDesc &d, char *base) {
    Arena a;
    a.base = base;
    int W = d.W, H = d.H, n = W * H, P = d.P;
    for (int l = 0; l < kMaxLevels; l++) {
        int nl = (l < d.L) ? (W >> l) * (H >> l) : 0;
        d.ref_gray[l] = nl ? a.take<float>(nl) : nullptr;
        d.cur_gray[l] = nl ? a.take<float>(nl) : nullptr;
        d.ref_pts[l] = nl ? a.take<float4>(nl) : nullptr;
        d.ref_nrm[l] = nl ? a.take<float4>(nl) : nullptr;
        d.cur_pts[l] = nl ? a.take<float4>(nl) : nullptr;
        d.sel_I[l] = (l < d.L) ? a.take<float>(P) : nullptr;
        d.sel_J[l] = (l < d.L) ? a.take<float>(6 * (size_t)P) : nullptr;
        bool mixed = d.precision == RECON_PRECISION_MIXED && l < d.L;
        d.sel_Ih[l] = mixed ? a.take<__half>(P) : nullptr;
        d.sel_Jb[l] = mixed ? a.take<__nv_bfloat16>(6 * (size_t)P) : nullptr;
        d.cur_grayh[l] = mixed ? a.take<__half>(nl) : nullptr;
    }
    d.ref_z = a.take<float>(n);
    d.ref_col = a.take<float>(n);
    d.cur_z = a.take<float>(n);
    d.gmag = a.take<float>(n);
    d.grad_hist = a.take<int>(1024);
    d.seg = a.take<int>(3076);
    d.sel_idx = a.take<int>(P);
    d.sel_xyz = a.take<float>(3 * (size_t)P);
    d.ph_r = a.take<float>(P);
    d.ph_zw = a.take<float>(P);
    d.ph_hist = a.take<int>(1024);
    d.icp_mask = a.take<uint8_t>(n);
    d.icp_r2 = a.take<float>(n);
    d.icp_w = a.take<float>(n);
    int nblk = (n + kChunk - 1) / kChunk;
    d.icp_blkcnt = a.take<int>(nblk);
    d.icp_blkvar = a.take<long long>(nblk);
    d.icp_part = a.take<long long>(nblk);
    d.icp_var = a.take<unsigned long long>(4);
    d.icp_nsel = a.take<int>(kMaxLevels);
    d.fuse_c2 = a.take<double>(kMaxLevels);
    d.fx = a.take<unsigned long long>(2 * 27 * kFxLimbs);
    d.fx_bad = a.take<int>(2);
    d.work = a.take<unsigned long long>(4);
    d.counter = a.take<unsigned int>(4);
    d.T = a.take<float>(16);
    d.stats = a.take<int>(ST_COUNT);
    return a.off;
}

int ensure_stage(recon_batch *b, size_t bytes) {
    if (bytes <= b->stage_bytes) return RECON_OK;
    if (b->d_stage) cudaFree(b->d_stage);
    b->d_stage = nullptr;
    b->stage_bytes = 0;
    CK(cudaMalloc(&b->d_stage, bytes));
    b->stage_bytes = bytes;
    return RECON_OK;
}

// uploads host images to staging (if needed) and fills the device pointer table
// Host-to-device copies of one image per instance, dst[i] <- src[i] (bytes[i];
// a null src copies nothing): one 2-D copy when every instance has an image,
// all of one size, and the sources and the destinations are each evenly
// spaced (frames picked from one host stack at a fixed step into one device
// arena), else one copy per image.
cudaError_t copy_images(const void *const *src, void *const *dst, const size_t *bytes, int n, cudaStream_t s) {
    bool one = n >= 2;
    size_t sp = 0, dp = 0;
    if (one) {
        const char *s0 = (const char *)src[0], *s1 = (const char *)src[1];
        const char *d0 = (const char *)dst[0], *d1 = (const char *)dst[1];
        one = s0 && s1 && s1 > s0 && d1 > d0;
        if (one) {
            sp = (size_t)(s1 - s0);
            dp = (size_t)(d1 - d0);
            one = sp >= bytes[0] && dp >= bytes[0];
        }
        for (int i = 0; one && i < n; i++)
            one = src[i] && bytes[i] == bytes[0] && (const char *)src[i] == s0 + i * sp &&
                  (const char *)dst[i] == d0 + i * dp;
    }
    if (one) return cudaMemcpy2DAsync(dst[0], dp, src[0], sp, bytes[0], n, cudaMemcpyHostToDevice, s);
    for (int i = 0; i < n; i++) {
        if (!src[i]) continue;
        cudaError_t e = cudaMemcpyAsync(dst[i], src[i], bytes[i], cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

int stage_inputs(recon_batch *b, const uint8_t *const *gray, const uint16_t *const *depth, const float *const *rgbd,
                 int on_device, const float *const *opts = nullptr, const float *const *onrm = nullptr) {
    int n = b->n;
    b->h_inptr.assign(5 * (size_t)n, nullptr);
    std::vector<int> active(n, 0);
    size_t need = 0;
    if (!on_device) {
        for (int i = 0; i < n; i++) {
            size_t px = (size_t)b->cfg[i].width * b->cfg[i].height;
            if (rgbd && rgbd[i]) need += align256(px * 16);
            else if (gray && depth && gray[i] && depth[i]) need += align256(px) + align256(px * 2);
            if (opts && onrm && opts[i] && onrm[i]) need += 2 * align256(px * 16);
        }
        int rc = ensure_stage(b, need ? need : 256);
        if (rc) return rc;
    }
    // the staging arena holds, per instance, its images one after the other;
    // the copies go out per image kind (5 kinds: gray, depth, RGB-D, points,
    // normals) so that evenly spaced images take one 2-D copy each
    std::vector<const void *> src(5 * (size_t)n, nullptr);
    std::vector<void *> dst(5 * (size_t)n, nullptr);
    std::vector<size_t> bytes(5 * (size_t)n, 0);
    size_t off = 0;
    auto place = [&](int kind, int i, const void *p, size_t nb) -> const void * {
        if (on_device) return p;
        size_t k = (size_t)kind * n + i;
        src[k] = p;
        dst[k] = b->d_stage + off;
        bytes[k] = nb;
        off += align256(nb);
        return dst[k];
    };
    for (int i = 0; i < n; i++) {
        size_t px = (size_t)b->cfg[i].width * b->cfg[i].height;
        if (rgbd && rgbd[i]) {
            b->h_inptr[2 * (size_t)n + i] = place(2, i, rgbd[i], px * 16);
            active[i] = 1;
        } else if (gray && depth && gray[i] && depth[i]) {
            b->h_inptr[i] = place(0, i, gray[i], px);
            b->h_inptr[(size_t)n + i] = place(1, i, depth[i], px * 2);
            active[i] = 1;
        }
        if (active[i] && opts && onrm && opts[i] && onrm[i]) {
            b->h_inptr[3 * (size_t)n + i] = place(3, i, opts[i], px * 16);
            b->h_inptr[4 * (size_t)n + i] = place(4, i, onrm[i], px * 16);
        }
    }
    if (!on_device)
        for (int kind = 0; kind < 5; kind++)
            CK(copy_images(src.data() + (size_t)kind * n, dst.data() + (size_t)kind * n,
                           bytes.data() + (size_t)kind * n, n, b->stream));
    CK(cudaMemcpyAsync(b->d_inptr, b->h_inptr.data(), 5 * (size_t)n * sizeof(void *), cudaMemcpyHostToDevice,
                       b->stream));
    CK(cudaMemcpyAsync(b->d_active, active.data(), n * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    // the pageable source vectors must stay valid until the copies complete
    CK(cudaStreamSynchronize(b->stream));
    return RECON_OK;
}

dim3 grid_pix(int pix, int n, int block = 256) { return dim3((pix + block - 1) / block, n, 1); }

enum TimingKind {
    TK_ITER = 0, TK_ICP_MASK, TK_ICP_STUDENT, TK_PREP_CUR, TK_PREP_REF, TK_SOLVE, TK_ICP_PREP, TK_FUSE, TK_COUNT
};
static_assert(TK_COUNT <= 8, "timing slots");

// brackets one launch with a pair of events when timing is enabled; events
// recorded during stream capture become graph nodes and are re-recorded by
// every replay
struct TimedScope {
    recon_batch *b;
    cudaStream_t s;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> *list;
    cudaEvent_t e1 = nullptr, e2 = nullptr;
    int kind;
    unsigned int flags;
    TimedScope(recon_batch *b_, cudaStream_t s_, int kind_, bool in_graph) : b(b_), s(s_), kind(kind_) {
        list = in_graph ? &b->graph_events : &b->direct_events;
        // inside a capture an event record must be external to become a graph node
        flags = in_graph ? cudaEventRecordExternal : cudaEventRecordDefault;
        if (!b->timing) return;
        if (in_graph) {
            cudaEventCreate(&e1);
            cudaEventCreate(&e2);
        } else {
            e1 = take();
            e2 = take();
        }
        cudaEventRecordWithFlags(e1, s, flags);
    }
    cudaEvent_t take() {
        if (b->pool_next == b->event_pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            b->event_pool.push_back(e);
        }
        return b->event_pool[b->pool_next++];
    }
    ~TimedScope() {
        if (!b->timing) return;
        cudaEventRecordWithFlags(e2, s, flags);
        list->push_back({kind, {e1, e2}});
    }
};

// pooled: the direct-launch events return to the pool instead of being destroyed
void collect_events(recon_batch *b, std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> &list,
                    bool pooled) {
    for (auto &ev : list) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ev.second.first, ev.second.second) == cudaSuccess) {
            b->t_ms[ev.first] += ms;
            b->t_cnt[ev.first] += 1;
        }
    }
    if (pooled) {
        list.clear();
        b->pool_next = 0;
    }
}

// reference preparation; from_inputs: convert the staged images (else rebuild
// from the current ref_z, keeping the keyframe gray); reset_pose: T <- I
int prepare_reference(recon_batch *b, bool from_inputs = true, bool reset_pose = true,
                      cudaStream_t st = nullptr, const int *active_flags = nullptr, bool oriented = false) {
    cudaStream_t s = st ? st : b->stream;
    TimedScope ts(b, s, TK_PREP_REF, false);
    int n = b->n;
    auto D = b->d_desc;
    auto in = b->d_inptr;
    const int *active = active_flags ? active_flags : b->d_active;
    if (from_inputs)
        k_convert_level0<<<grid_pix(b->max_pix, n), 256, 0, s>>>(
            D, (const uint8_t *const *)in, (const uint16_t *const *)(in + n), (const float *const *)(in + 2 * n));
    else
        k_ref_from_z<<<grid_pix(b->max_pix, n), 256, 0, s>>>(D, active);
    k_normals<<<grid_pix(b->max_pix, n), 256, 0, s>>>(D, active);
    // the photometric vertex records take the points of the keyframe depth
    // (ref_z), not the level-0 ICP points that oriented points may replace
    k_clear_ref<<<dim3(1, n), 256, 0, s>>>(D, active);
    k_xyz2cloud<<<grid_pix(b->max_pix, n), 256, 0, s>>>(D, active);
    if (oriented) {
        k_oriented_points<<<grid_pix(b->max_pix, n), 256, 0, s>>>(D, (const float *const *)(in + 3 * n),
                                                                   (const float *const *)(in + 4 * n));
        g_launches += 1;
    }
    for (int l = 1; l < b->max_L; l++)
        k_downsample<<<grid_pix(b->max_pix >> (2 * l), n), 256, 0, s>>>(D, l, active);
    k_seg_count<<<dim3(kSegments / 8, n), 256, 0, s>>>(D, active);
    k_seg_scan<<<dim3(1, n), kSegments, 0, s>>>(D, active);
    k_seg_scatter<<<dim3(kSegments / 8, n), 256, 0, s>>>(D, active);
    k_attr_jac<<<grid_pix(b->max_P, n), 256, 0, s>>>(D, active);
    if (reset_pose) k_reset_pose<<<dim3(1, n), 32, 0, s>>>(D, active);
    g_launches += 9 + (b->max_L - 1) + (reset_pose ? 1 : 0);
    CK(cudaGetLastError());
    return RECON_OK;
}

// the current frame's level-0 conversion and pyramid in one launch
// (in sequences the same launch stores the previous frame's pose into
// `store_prev` and, with `begin`, starts the frame as k_begin_track does)
int prepare_current(recon_batch *b, const void **in = nullptr, float *store_prev = nullptr, bool begin = false) {
    TimedScope ts(b, b->stream, TK_PREP_CUR, false);
    int n = b->n;
    if (!in) in = b->d_inptr;
    int maxw = 0, maxh = 0;
    for (auto &c : b->cfg) {
        maxw = std::max(maxw, c.width);
        maxh = std::max(maxh, c.height);
    }
    int tx = (maxw + kPyrTile - 1) / kPyrTile, ty = (maxh + kPyrTile - 1) / kPyrTile;
    k_prep_current_pyramid<<<dim3(tx * ty, n), 256, 0, b->stream>>>(
        b->d_desc, (const uint8_t *const *)in, (const uint16_t *const *)(in + n), (const float *const *)(in + 2 * n),
        tx, store_prev, begin ? 1 : 0);
    g_launches += 1;
    CK(cudaGetLastError());
    return RECON_OK;
}

// Levels with at most this many pixels per instance prepare their ICP
// correspondences and weights in one cluster launch (k_icp_prepare, at most 4
// pixels per thread); larger ones use the wide mask grid and one wide launch
// per Student-t pass (k_icp_student_pass), whose many small CTAs hide the
// gathers' latency better and keep every SM busy.
#ifndef RECON_PREPARE_FUSED_MAX_PIX
#define RECON_PREPARE_FUSED_MAX_PIX (4 * 8 * 1024)
#endif
constexpr int kPrepareFusedMaxPix = RECON_PREPARE_FUSED_MAX_PIX;

// Launches a kernel of the per-frame schedule as a programmatic dependent of
// the previous kernel in the stream (a programmatic edge inside a graph): it
// may start while that kernel finishes and waits for it with pdl_wait.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// ICP chunks per k_iter CTA at `level` for a level whose largest instance has
// `nchunk` chunks: the tuned value, else about five waves of CTAs over the
// batch's chunks, at most 8 chunks each.  The result does not depend on it.
int icp_per_cta(const recon_batch *b, int level, int nchunk) {
    if (b->icp_cpc[level] > 0) return b->icp_cpc[level];
    int waves = 5 * kIterCtaSlots;
    return std::min(8, std::max(1, (b->n * nchunk + waves / 2) / waves));
}

// the per-frame Gauss-Newton schedule (gpuEstimateIncrement, phototracker.cpp:666-689)
int launch_schedule(recon_batch *b, cudaStream_t s, bool in_graph) {
    int n = b->n;
    auto D = b->d_desc;
    bool any_icp = false;
    for (auto &c : b->cfg) any_icp |= (c.mode != RECON_PHOTOMETRIC);
    for (int level = b->max_L - 1; level >= 0; level--) {
        int maxit = 0, maxpix = 0;
        for (int i = 0; i < n; i++) {
            const recon_config &c = b->cfg[i];
            if (level >= c.levels) continue;
            int it = c.iters[c.levels - 1 - level];
            if (it > maxit) maxit = it;
            int px = (c.width >> level) * (c.height >> level);
            if (px > maxpix) maxpix = px;
        }
        if (maxit == 0) continue;
        int nchunk = (maxpix + kChunk - 1) / kChunk;
        if (any_icp && maxpix <= kPrepareFusedMaxPix) {
            // small grid: mask and Student-t passes in one cluster launch
            TimedScope ts(b, s, TK_ICP_PREP, in_graph);
            CK(launch_pdl(k_icp_prepare, dim3(kIterCluster, n), dim3(1024), s, D, level));
            b->graph_kernels += 1;
        } else if (any_icp) {
            {
                TimedScope ts(b, s, TK_ICP_MASK, in_graph);
                CK(launch_pdl(k_icp_mask, dim3(nchunk, n), dim3(kLanes), s, D, level));
            }
            {
                // about one wave of CTAs over the blocks of the instances that
                // run the level (sized by their actual blocks, so that a batch
                // of mixed resolutions is spread as evenly as a uniform one)
                long long blocks = 0;
                for (int i = 0; i < n; i++) {
                    const recon_config &c = b->cfg[i];
                    if (level >= c.levels || c.mode == RECON_PHOTOMETRIC || c.iters[c.levels - 1 - level] <= 0)
                        continue;
                    blocks += ((c.width >> level) * (c.height >> level) + kChunk - 1) / kChunk;
                }
                int per = (int)std::max(1LL, (blocks + kPassCtaSlots - 1) / kPassCtaSlots);
                int gx = (nchunk + per - 1) / per;
                TimedScope ts(b, s, TK_ICP_STUDENT, in_graph);
                for (int pass = 1; pass <= 3; pass++)
                    CK(launch_pdl(k_icp_student_pass, dim3(gx, n), dim3(kLanes), s, D, level, pass, per));
            }
            b->graph_kernels += 4;
        }
        int per_cta = icp_per_cta(b, level, nchunk);
        int ncta = any_icp ? (nchunk + per_cta - 1) / per_cta : 0;
        // every instance's photometric cluster, then ncta ICP CTAs per
        // instance, the total rounded up to whole clusters
        int gx = kIterCluster * n + (n * ncta + kIterCluster - 1) / kIterCluster * kIterCluster;
        for (int it = 0; it < maxit; it++) {
            {
                TimedScope ts(b, s, TK_ITER, in_graph);
                CK(launch_pdl(k_iter, dim3(gx, 1), dim3(kIterBlock), s, D, level, it, per_cta, n, ncta));
            }
            {
                TimedScope ts(b, s, TK_SOLVE, in_graph);
                CK(launch_pdl(k_solve, dim3(n), dim3(kSolveThreads), s, D, level, it));
            }
            b->graph_kernels += 2;
        }
    }
    CK(cudaGetLastError());
    return RECON_OK;
}

int run_schedule(recon_batch *b) {
    if (b->timing) {
        // timed runs launch directly so that every launch keeps its own events
        b->graph_kernels = 0;
        int rc = launch_schedule(b, b->stream, false);
        g_launches += b->graph_kernels;
        b->graph_dirty = true;
        return rc;
    }
    if (b->graph_dirty) {
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        for (auto &ev : b->graph_events) {
            cudaEventDestroy(ev.second.first);
            cudaEventDestroy(ev.second.second);
        }
        b->graph_events.clear();
        cudaStream_t cs;
        CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t g;
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaStreamDestroy(cs);
            return cuda_fail(e, "cudaStreamBeginCapture");
        }
        b->graph_kernels = 0;
        int rc = launch_schedule(b, cs, true);
        e = cudaStreamEndCapture(cs, &g);
        cudaStreamDestroy(cs);
        if (rc) return rc;
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        b->graph_dirty = false;
    }
    CK(cudaGraphLaunch(b->graph, b->stream));
    g_launches += b->graph_kernels;
    return RECON_OK;
}

// Learned start poses for the frame whose uint8 / uint16 inputs the pointer
// table `row` (gray pointers, then depth pointers) holds: coarse image, network
// on (previous, current), gate.  The current coarse image becomes the previous.
// The network part on stream s: the coarse image of the frame whose inputs
// `row` holds, the network input (previous, current) and the forward pass into
// `out`.  The current coarse image becomes the previous.
int learned_net(recon_batch *b, const void **row, cudaStream_t s, float *out, float *gateD) {
    int n = b->n;
    int cur = 1 - b->coarse_prev;
    k_net_coarse<<<dim3((kNetW * kNetH + 255) / 256, n), 256, 0, s>>>(
        b->d_desc, (const uint8_t *const *)row, (const uint16_t *const *)(row + n),
        (const __nv_bfloat16 *)b->d_coarse[b->coarse_prev], (__nv_bfloat16 *)b->d_coarse[cur],
        (__nv_bfloat16 *)b->d_netin);
    g_launches += 1;
    int rc = nn::forward_on(b->net, b->d_netin, n, out, s);
    if (rc) return rc;
    g_launches += nn::forward_kernels(n);
    k_gate_twist<<<n, 32, 0, s>>>(b->d_desc, out, nn::scale_dev(b->net), gateD);
    g_launches += 1;
    b->coarse_prev = cur;
    CK(cudaGetLastError());
    return RECON_OK;
}

// The gate on the batch stream (one launch): candidate pose from the network's
// exp(twist) `gateD` and the previous pose, the two coarse costs, the choice.
int learned_gate(recon_batch *b, const float *out, const float *gateD) {
    int n = b->n;
    k_gate<<<dim3((b->max_P + 255) / 256, n), 256, 0, b->stream>>>(b->d_desc, gateD, b->d_cost, b->d_ticket,
                                                                    b->d_cand, b->d_choice);
    g_launches += 1;
    b->netout_last = out;
    CK(cudaGetLastError());
    return RECON_OK;
}

int learned_start(recon_batch *b, const void **row) {
    int rc = learned_net(b, row, b->stream, b->d_netout, b->d_gateD);
    if (rc) return rc;
    return learned_gate(b, b->d_netout, b->d_gateD);
}

// coarse image of the keyframe: the "previous frame" of the first tracked frame
int learned_keyframe(recon_batch *b) {
    if (!b->net) return RECON_OK;
    int n = b->n;
    const void **row = b->d_inptr;
    k_net_coarse<<<dim3((kNetW * kNetH + 255) / 256, n), 256, 0, b->stream>>>(
        b->d_desc, (const uint8_t *const *)row, (const uint16_t *const *)(row + n), nullptr,
        (__nv_bfloat16 *)b->d_coarse[b->coarse_prev], nullptr);
    g_launches += 1;
    CK(cudaGetLastError());
    return RECON_OK;
}

// Fusion buffers (second stream, events, pointer tables for cnt frame-instance pairs).
int fuse_prepare(recon_batch *b, size_t cnt) {
    if (!b->recon_stream) {
        CK(cudaStreamCreateWithFlags(&b->recon_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&b->ev_pose, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&b->ev_fused, cudaEventDisableTiming));
        std::vector<int> ones(b->n, 1);
        CK(cudaMalloc(&b->d_all_active, b->n * sizeof(int)));
        CK(cudaMemcpy(b->d_all_active, ones.data(), b->n * sizeof(int), cudaMemcpyHostToDevice));
    }
    if (cnt > b->fuse_cap) {
        // the previous fusion may still read the tables
        CK(cudaStreamSynchronize(b->recon_stream));
        if (b->d_fuse_ptr) cudaFree(b->d_fuse_ptr);
        if (b->h_fuse_ptr) cudaFreeHost(b->h_fuse_ptr);
        if (b->d_fuse_T) cudaFree(b->d_fuse_T);
        b->d_fuse_ptr = nullptr;
        b->h_fuse_ptr = nullptr;
        b->d_fuse_T = nullptr;
        b->fuse_cap = 0;
        CK(cudaMalloc(&b->d_fuse_ptr, 2 * cnt * sizeof(void *)));
        CK(cudaMallocHost(&b->h_fuse_ptr, 2 * cnt * sizeof(void *)));
        CK(cudaMalloc(&b->d_fuse_T, cnt * 16 * sizeof(float)));
        b->fuse_cap = cnt;
    } else {
        // the pinned table is rewritten by the host: the previous fusion's copy of it is done
        CK(cudaStreamSynchronize(b->recon_stream));
    }
    return RECON_OK;
}

int prepare_reference(recon_batch *b, bool from_inputs, bool reset_pose, cudaStream_t st, const int *active_flags,
                      bool oriented);

// The fusion kernel and the reference rebuild on the second stream, reading
// the device table d_fuse_ptr (depth, then gray) and poses Tdev; the pose
// stream then waits for the fused keyframe.
int fuse_launch(recon_batch *b, int nframes, bool colour, const float *Tdev, float gate_mm) {
    int n = b->n;
    size_t cnt = (size_t)nframes * n;
    {
        TimedScope ts(b, b->recon_stream, TK_FUSE, false);
        k_fuse_depth<<<grid_pix(b->max_pix, n), 256, 0, b->recon_stream>>>(
            b->d_desc, nframes, n, (const uint16_t *const *)b->d_fuse_ptr,
            colour ? (const uint8_t *const *)(b->d_fuse_ptr + cnt) : nullptr, Tdev, gate_mm, b->d_all_active);
    }
    g_launches += 1;
    int rc = prepare_reference(b, false, false, b->recon_stream, b->d_all_active);
    if (rc) return rc;
    CK(cudaEventRecord(b->ev_fused, b->recon_stream));
    CK(cudaStreamWaitEvent(b->stream, b->ev_fused, 0));
    return RECON_OK;
}

int upload_desc(recon_batch *b) {
    CK(cudaMemcpyAsync(b->d_desc, b->desc.data(), b->n * sizeof(InstDesc), cudaMemcpyHostToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return RECON_OK;
}

}  // namespace

namespace rt {

__global__ void k_reset_pose(const InstDesc *D, const int *active) {
    const InstDesc &d = D[blockIdx.y];
    if (!active[blockIdx.y]) return;
    if (threadIdx.x < 16) d.T[threadIdx.x] = (threadIdx.x % 5 == 0) ? 1.0f : 0.0f;
}

__global__ void k_clear_ref(const InstDesc *D, const int *active) {
    const InstDesc &d = D[blockIdx.y];
    if (!active[blockIdx.y]) return;
    for (int k = threadIdx.x; k < 1024; k += blockDim.x) d.grad_hist[k] = 0;
    for (int k = threadIdx.x; k < d.P; k += blockDim.x) d.sel_idx[k] = 0;
}

__global__ void k_store_pose(const InstDesc *D, float *dst) {
    const InstDesc &d = D[blockIdx.y];
    if (threadIdx.x < 16) dst[16 * blockIdx.y + threadIdx.x] = d.T[threadIdx.x];
}

__global__ void k_gather_results(const InstDesc *D, int *dst) {
    const InstDesc &d = D[blockIdx.y];
    int t = threadIdx.x;
    if (t < 16) dst[32 * blockIdx.y + t] = __float_as_int(d.T[t]);
    else if (t < 16 + ST_COUNT) dst[32 * blockIdx.y + t] = d.stats[t - 16];
}

__global__ void k_begin_track(const InstDesc *D, const float *T_init, int have_init) {
    const InstDesc &d = D[blockIdx.y];
    int t = threadIdx.x;
    if (have_init && t < 16) d.T[t] = T_init[16 * blockIdx.y + t];
    if (t < ST_COUNT) d.stats[t] = 0;
    if (t == 0) {
        *d.counter = 0u;
        if (d.trace_count) *d.trace_count = 0;
    }
    for (int k = t; k < 2 * 27 * kFxLimbs; k += blockDim.x) d.fx[k] = 0ull;
    if (t < 2) d.fx_bad[t] = 0;
}

}  // namespace rt

// ====================================================================
// C ABI
// ====================================================================
extern "C" {

const char *recon_last_error(void) { return g_last_error.c_str(); }

int recon_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

int recon_calib_setup(const double KL[9], const double KR[9], const double TLR[16], const double kcR[8],
                      double min_dist, double max_dist, double c0, double c1, int32_t width, float *calib) {
    if (!KL || !KR || !TLR || !kcR || !calib || width <= 0) return fail(RECON_ERR_INVALID_ARG, "null argument");
    memset(calib, 0, RECON_CALIB_SIZE * sizeof(float));
    auto putK = [&](int off, const double *K) {
        for (int i = 0; i < 9; i++) calib[off + i] = (i % 4 == 0) ? 1.0f : 0.0f;
        for (int i = 0; i < 6; i++) calib[off + i] = (float)(width * K[i]);
        const float *m = calib + off;
        double det = (double)m[0] * ((double)m[4] * m[8] - (double)m[5] * m[7]) -
                     (double)m[1] * ((double)m[3] * m[8] - (double)m[5] * m[6]) +
                     (double)m[2] * ((double)m[3] * m[7] - (double)m[4] * m[6]);
        float *r = calib + off + 9;
        if (std::fabs(det) < 1e-5) {
            for (int i = 0; i < 9; i++) r[i] = (i % 4 == 0) ? 1.0f : 0.0f;
            return;
        }
        r[0] = (float)(((double)m[4] * m[8] - (double)m[5] * m[7]) / det);
        r[1] = (float)(-((double)m[1] * m[8] - (double)m[7] * m[2]) / det);
        r[2] = (float)(((double)m[1] * m[5] - (double)m[4] * m[2]) / det);
        r[3] = (float)(-((double)m[3] * m[8] - (double)m[5] * m[6]) / det);
        r[4] = (float)(((double)m[0] * m[8] - (double)m[6] * m[2]) / det);
        r[5] = (float)(-((double)m[0] * m[5] - (double)m[3] * m[2]) / det);
        r[6] = (float)(((double)m[3] * m[7] - (double)m[6] * m[4]) / det);
        r[7] = (float)(-((double)m[0] * m[7] - (double)m[6] * m[1]) / det);
        r[8] = (float)(((double)m[0] * m[4] - (double)m[3] * m[1]) / det);
    };
    putK(0, KR);
    for (int i = 0; i < 8; i++) calib[18 + i] = (float)kcR[i];
    double TRL[16] = {TLR[0], TLR[4], TLR[8],  -(TLR[0] * TLR[3] + TLR[4] * TLR[7] + TLR[8] * TLR[11]),
                      TLR[1], TLR[5], TLR[9],  -(TLR[1] * TLR[3] + TLR[5] * TLR[7] + TLR[9] * TLR[11]),
                      TLR[2], TLR[6], TLR[10], -(TLR[2] * TLR[3] + TLR[6] * TLR[7] + TLR[10] * TLR[11]),
                      0,      0,      0,       1};
    for (int i = 0; i < 16; i++) {
        calib[26 + i] = (float)TLR[i];
        calib[64 + i] = (float)TRL[i];
    }
    putK(43, KL);
    calib[61] = (float)c0;
    calib[42] = (float)c1;
    calib[62] = (float)min_dist;
    calib[63] = (float)max_dist;
    return RECON_OK;
}

int recon_batch_create(int32_t n, const recon_config *cfgs, const float *calibs, void *stream, recon_batch **out) {
    clear_stale_error();
    if (!out || !cfgs || !calibs || n <= 0) return fail(RECON_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(RECON_ERR_NO_DEVICE, "no CUDA device");
    for (int i = 0; i < n; i++) {
        int rc = validate(cfgs[i]);
        if (rc) return rc;
    }
    recon_batch *b = new recon_batch();
    b->n = n;
    b->cfg.assign(cfgs, cfgs + n);
    b->desc.resize(n);
    identity16d(b->global_pose);
    identity16(b->T_host);
    if (stream) {
        b->stream = (cudaStream_t)stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete b;
            return cuda_fail(e, "cudaStreamCreate");
        }
        b->own_stream = true;
    }
    for (int i = 0; i < n; i++) {
        const recon_config &c = cfgs[i];
        InstDesc &d = b->desc[i];
        memset(&d, 0, sizeof(d));
        d.W = c.width;
        d.H = c.height;
        d.L = c.levels;
        d.P = c.n_select;
        d.hist_bins = c.hist_bins;
        d.select_bins = c.select_bins;
        d.mode = c.mode;
        d.solver = c.solver;
        d.lambda = c.lambda;
        d.fuse_c1 = (double)(1.0f - c.lambda) / (double)c.n_select;
        d.opt_in = c.opt_scale_in;
        d.opt_out = c.opt_scale_out;
        d.precision = c.precision;
        for (int l = 0; l < kMaxLevels; l++) d.iters[l] = c.iters[l];
        d.settle_mm = c.settle_mm;
        d.settle_rot = c.settle_rot;
        memcpy(d.calib, calibs + (size_t)RECON_CALIB_SIZE * i, sizeof(d.calib));
        size_t bytes = layout(d, nullptr);
        void *mem = nullptr;
        cudaError_t e = cudaMalloc(&mem, bytes);
        if (e != cudaSuccess) {
            recon_batch_destroy(b);
            return cuda_fail(e, "cudaMalloc(instance)");
        }
        b->arenas.push_back(mem);
        cudaMemsetAsync(mem, 0, bytes, b->stream);
        layout(d, (char *)mem);
        b->max_pix = std::max(b->max_pix, c.width * c.height);
        b->max_L = std::max(b->max_L, c.levels);
        b->max_P = std::max(b->max_P, c.n_select);
    }
    cudaError_t e = cudaMalloc(&b->d_desc, n * sizeof(InstDesc));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_inptr, 5 * (size_t)n * sizeof(void *));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_active, n * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_Tinit, 16 * (size_t)n * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_results, 32 * (size_t)n * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_results, 32 * (size_t)n * sizeof(int));
    if (e != cudaSuccess) {
        recon_batch_destroy(b);
        return cuda_fail(e, "cudaMalloc(batch)");
    }
    for (int i = 0; i < n; i++) {
        float I[16];
        identity16(I);
        cudaMemcpyAsync(b->desc[i].T, I, sizeof(I), cudaMemcpyHostToDevice, b->stream);
        cudaStreamSynchronize(b->stream);
    }
    int rc = upload_desc(b);
    if (rc) {
        recon_batch_destroy(b);
        return rc;
    }
    *out = b;
    return RECON_OK;
}

int recon_batch_destroy(recon_batch *b) {
    if (!b) return RECON_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (void *p : b->arenas) cudaFree(p);
    if (b->d_desc) cudaFree(b->d_desc);
    if (b->d_inptr) cudaFree(b->d_inptr);
    if (b->d_active) cudaFree(b->d_active);
    if (b->d_stage) cudaFree(b->d_stage);
    if (b->d_Tinit) cudaFree(b->d_Tinit);
    if (b->d_results) cudaFree(b->d_results);
    if (b->h_results) cudaFreeHost(b->h_results);
    if (b->d_trace) cudaFree(b->d_trace);
    if (b->d_trace_count) cudaFree(b->d_trace_count);
    if (b->d_seqptr) cudaFree(b->d_seqptr);
    if (b->h_seqptr) cudaFreeHost(b->h_seqptr);
    if (b->d_Tseq) cudaFree(b->d_Tseq);
    if (b->d_slots) cudaFree(b->d_slots);
    for (int k = 0; k < 2; k++) {
        if (b->ev_copied[k]) cudaEventDestroy(b->ev_copied[k]);
        if (b->ev_set_read[k]) cudaEventDestroy(b->ev_set_read[k]);
        if (b->ev_set_fused[k]) cudaEventDestroy(b->ev_set_fused[k]);
    }
    if (b->copy_stream) cudaStreamDestroy(b->copy_stream);
    for (int k = 0; k < 2; k++) {
        if (b->d_netout_seq[k]) cudaFree(b->d_netout_seq[k]);
        if (b->ev_net[k]) cudaEventDestroy(b->ev_net[k]);
        if (b->ev_gate[k]) cudaEventDestroy(b->ev_gate[k]);
    }
    if (b->ev_seq) cudaEventDestroy(b->ev_seq);
    if (b->net_stream) cudaStreamDestroy(b->net_stream);
    if (b->recon_stream) cudaStreamDestroy(b->recon_stream);
    if (b->ev_pose) cudaEventDestroy(b->ev_pose);
    if (b->ev_fused) cudaEventDestroy(b->ev_fused);
    if (b->d_fuse) cudaFree(b->d_fuse);
    if (b->d_fuse_ptr) cudaFree(b->d_fuse_ptr);
    if (b->h_fuse_ptr) cudaFreeHost(b->h_fuse_ptr);
    if (b->d_fuse_T) cudaFree(b->d_fuse_T);
    if (b->d_all_active) cudaFree(b->d_all_active);
    for (auto &ev : b->graph_events) {
        cudaEventDestroy(ev.second.first);
        cudaEventDestroy(ev.second.second);
    }
    for (cudaEvent_t e : b->event_pool) cudaEventDestroy(e);
    for (int k = 0; k < 2; k++)
        if (b->d_coarse[k]) cudaFree(b->d_coarse[k]);
    if (b->d_netin) cudaFree(b->d_netin);
    if (b->d_netout) cudaFree(b->d_netout);
    if (b->d_choice) cudaFree(b->d_choice);
    if (b->d_cand) cudaFree(b->d_cand);
    if (b->d_cost) cudaFree(b->d_cost);
    if (b->d_ticket) cudaFree(b->d_ticket);
    if (b->d_gateD) cudaFree(b->d_gateD);
    for (int k = 0; k < 2; k++)
        if (b->d_gateD_seq[k]) cudaFree(b->d_gateD_seq[k]);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return RECON_OK;
}

int recon_batch_size(const recon_batch *b) { return b ? b->n : 0; }

int recon_batch_set_reference(recon_batch *b, const uint8_t *const *gray, const uint16_t *const *depth,
                              int32_t on_device) {
    clear_stale_error();
    if (!b || !gray || !depth) return fail(RECON_ERR_INVALID_ARG, "null argument");
    int rc = stage_inputs(b, gray, depth, nullptr, on_device);
    if (rc) return rc;
    rc = prepare_reference(b);
    if (rc) return rc;
    rc = learned_keyframe(b);
    if (rc) return rc;
    CK(cudaStreamSynchronize(b->stream));
    b->have_ref = true;
    return RECON_OK;
}

int recon_batch_set_reference_oriented(recon_batch *b, const uint8_t *const *gray, const uint16_t *const *depth,
                                       const float *const *points, const float *const *normals, int32_t on_device) {
    clear_stale_error();
    if (!b || !gray || !depth || !points || !normals) return fail(RECON_ERR_INVALID_ARG, "null argument");
    int rc = stage_inputs(b, gray, depth, nullptr, on_device, points, normals);
    if (rc) return rc;
    rc = prepare_reference(b, true, true, nullptr, nullptr, true);
    if (rc) return rc;
    rc = learned_keyframe(b);
    if (rc) return rc;
    CK(cudaStreamSynchronize(b->stream));
    b->have_ref = true;
    return RECON_OK;
}

int recon_batch_set_reference_rgbd_float4(recon_batch *b, int32_t inst, const float *rgbd, int32_t on_device) {
    clear_stale_error();
    if (!b || !rgbd || inst < 0 || inst >= b->n) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    std::vector<const float *> p(b->n, nullptr);
    p[inst] = rgbd;
    int rc = stage_inputs(b, nullptr, nullptr, p.data(), on_device);
    if (rc) return rc;
    rc = prepare_reference(b);
    if (rc) return rc;
    CK(cudaStreamSynchronize(b->stream));
    b->have_ref = true;
    return RECON_OK;
}

int recon_batch_set_current(recon_batch *b, const uint8_t *const *gray, const uint16_t *const *depth,
                            int32_t on_device) {
    clear_stale_error();
    if (!b || !gray || !depth) return fail(RECON_ERR_INVALID_ARG, "null argument");
    int rc = stage_inputs(b, gray, depth, nullptr, on_device);
    if (rc) return rc;
    rc = prepare_current(b);
    if (rc) return rc;
    b->have_cur = true;
    return RECON_OK;
}

int recon_batch_set_current_rgbd_float4(recon_batch *b, int32_t inst, const float *rgbd, int32_t on_device) {
    clear_stale_error();
    if (!b || !rgbd || inst < 0 || inst >= b->n) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    std::vector<const float *> p(b->n, nullptr);
    p[inst] = rgbd;
    int rc = stage_inputs(b, nullptr, nullptr, p.data(), on_device);
    if (rc) return rc;
    rc = prepare_current(b);
    if (rc) return rc;
    b->have_cur = true;
    return RECON_OK;
}

int recon_batch_track_async(recon_batch *b, const float *T_init_host) {
    clear_stale_error();
    if (!b) return fail(RECON_ERR_INVALID_ARG, "null batch");
    if (!b->have_ref || !b->have_cur) return fail(RECON_ERR_STATE, "reference or current frame missing");
    if (T_init_host)
        CK(cudaMemcpyAsync(b->d_Tinit, T_init_host, 16 * (size_t)b->n * sizeof(float), cudaMemcpyHostToDevice,
                           b->stream));
    k_begin_track<<<dim3(1, b->n), 32, 0, b->stream>>>(b->d_desc, b->d_Tinit, T_init_host ? 1 : 0);
    g_launches += 1;
    CK(cudaGetLastError());
    if (b->net && !T_init_host) {
        int rc = learned_start(b, b->d_inptr);
        if (rc) return rc;
    }
    return run_schedule(b);
}

int recon_batch_get_poses(recon_batch *b, float *T_out, recon_track_stats *stats) {
    clear_stale_error();
    if (!b) return fail(RECON_ERR_INVALID_ARG, "null batch");
    int n = b->n;
    if (T_out || stats) {
        static_assert(16 + ST_COUNT <= 32, "results record");
        k_gather_results<<<dim3(1, n), 32, 0, b->stream>>>(b->d_desc, b->d_results);
        g_launches += 1;
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(b->h_results, b->d_results, 32 * (size_t)n * sizeof(int), cudaMemcpyDeviceToHost,
                           b->stream));
    }
    CK(cudaStreamSynchronize(b->stream));
    if (T_out)
        for (int i = 0; i < n; i++) memcpy(T_out + 16 * (size_t)i, b->h_results + 32 * (size_t)i, 64);
    if (b->timing) {
        collect_events(b, b->graph_events, false);
        collect_events(b, b->direct_events, true);
    }
    if (stats) {
        for (int i = 0; i < b->n; i++) {
            const int *s = b->h_results + 32 * (size_t)i + 16;
            recon_track_stats &o = stats[i];
            memset(&o, 0, sizeof(o));
            o.iterations = s[ST_ITERS];
            o.solves = s[ST_SOLVES];
            o.non_spd = s[ST_NONSPD];
            o.photo_median_bin = s[ST_MEDIAN];
            for (int l = 0; l < RECON_MAX_LEVELS; l++) o.icp_selected[l] = s[ST_ICPSEL0 + l];
            // a rejected pivot first; else an iteration skipped for lack of ICP
            // correspondences (ShapeTracker's "not enough points",
            // shapetracker.cpp:365); the pose is kept in both cases
            o.status = o.non_spd ? RECON_ERR_NON_SPD
                                 : (o.solves < o.iterations ? RECON_ERR_NOT_ENOUGH_POINTS : RECON_OK);
        }
    }
    return RECON_OK;
}

int recon_batch_track(recon_batch *b, float *T_io, recon_track_stats *stats) {
    int rc = recon_batch_track_async(b, T_io);
    if (rc) return rc;
    return recon_batch_get_poses(b, T_io, stats);
}

int recon_batch_set_iterations(recon_batch *b, int32_t inst, const int32_t iters[RECON_MAX_LEVELS]) {
    clear_stale_error();
    if (!b || !iters || inst < 0 || inst >= b->n) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    recon_config c = b->cfg[inst];
    for (int l = 0; l < RECON_MAX_LEVELS; l++) c.iters[l] = iters[l];
    int rc = validate(c);
    if (rc) return rc;
    b->cfg[inst] = c;
    for (int l = 0; l < kMaxLevels; l++) b->desc[inst].iters[l] = iters[l];
    b->graph_dirty = true;
    return upload_desc(b);
}

int recon_batch_set_settle(recon_batch *b, int32_t inst, float tol_mm, float tol_rot) {
    clear_stale_error();
    if (!b || inst < 0 || inst >= b->n) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    recon_config c = b->cfg[inst];
    c.settle_mm = tol_mm;
    c.settle_rot = tol_rot;
    int rc = validate(c);
    if (rc) return rc;
    b->cfg[inst] = c;
    b->desc[inst].settle_mm = tol_mm;
    b->desc[inst].settle_rot = tol_rot;
    return upload_desc(b);  // the launches do not change: the kernels read the rule from the descriptor
}

int recon_batch_set_icp_chunks_per_cta(recon_batch *b, const int32_t per_level[RECON_MAX_LEVELS]) {
    clear_stale_error();
    if (!b || !per_level) return fail(RECON_ERR_INVALID_ARG, "null argument");
    for (int l = 0; l < kMaxLevels; l++)
        if (per_level[l] < 0 || per_level[l] > 64) return fail(RECON_ERR_INVALID_ARG, "chunks per CTA out of [0, 64]");
    CK(cudaStreamSynchronize(b->stream));
    for (int l = 0; l < kMaxLevels; l++) b->icp_cpc[l] = per_level[l];
    b->graph_dirty = true;
    return RECON_OK;
}

int recon_batch_get_icp_chunks_per_cta(recon_batch *b, int32_t per_level[RECON_MAX_LEVELS]) {
    clear_stale_error();
    if (!b || !per_level) return fail(RECON_ERR_INVALID_ARG, "null argument");
    for (int l = 0; l < kMaxLevels; l++) {
        int maxpix = 0;
        for (int i = 0; i < b->n; i++) {
            const recon_config &c = b->cfg[i];
            if (l < c.levels) maxpix = std::max(maxpix, (c.width >> l) * (c.height >> l));
        }
        per_level[l] = maxpix ? icp_per_cta(b, l, (maxpix + kChunk - 1) / kChunk) : 0;
    }
    return RECON_OK;
}

int recon_batch_set_mode(recon_batch *b, int32_t inst, int32_t mode, float lambda) {
    clear_stale_error();
    if (!b || inst < 0 || inst >= b->n) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    recon_config c = b->cfg[inst];
    c.mode = mode;
    c.lambda = lambda < 0.0f ? 0.0f : (lambda > 1.0f ? 1.0f : lambda);  // setLambda clamps, phototracker.cpp:160-165
    int rc = validate(c);
    if (rc) return rc;
    b->cfg[inst] = c;
    b->desc[inst].mode = c.mode;
    b->desc[inst].lambda = c.lambda;
    b->desc[inst].fuse_c1 = (double)(1.0f - c.lambda) / (double)c.n_select;
    b->graph_dirty = true;
    return upload_desc(b);
}

int recon_batch_enable_trace(recon_batch *b, int32_t max_iters) {
    clear_stale_error();
    if (!b || max_iters < 0) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    if (b->d_trace) cudaFree(b->d_trace);
    if (b->d_trace_count) cudaFree(b->d_trace_count);
    b->d_trace = nullptr;
    b->d_trace_count = nullptr;
    b->trace_max = max_iters;
    if (max_iters > 0) {
        CK(cudaMalloc(&b->d_trace, (size_t)b->n * max_iters * sizeof(recon_iter_trace)));
        CK(cudaMalloc(&b->d_trace_count, (size_t)b->n * sizeof(int)));
        CK(cudaMemset(b->d_trace, 0, (size_t)b->n * max_iters * sizeof(recon_iter_trace)));
        CK(cudaMemset(b->d_trace_count, 0, (size_t)b->n * sizeof(int)));
    }
    for (int i = 0; i < b->n; i++) {
        b->desc[i].trace = max_iters > 0 ? b->d_trace + (size_t)i * max_iters : nullptr;
        b->desc[i].trace_max = max_iters;
        b->desc[i].trace_count = max_iters > 0 ? b->d_trace_count + i : nullptr;
    }
    return upload_desc(b);
}

int recon_batch_get_trace(recon_batch *b, int32_t inst, recon_iter_trace *out, int32_t max) {
    clear_stale_error();
    if (!b || inst < 0 || inst >= b->n || !out) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    if (!b->d_trace) return 0;
    int cnt = 0;
    CK(cudaMemcpy(&cnt, b->d_trace_count + inst, sizeof(int), cudaMemcpyDeviceToHost));
    if (cnt > b->trace_max) cnt = b->trace_max;
    if (cnt > max) cnt = max;
    if (cnt > 0)
        CK(cudaMemcpy(out, b->d_trace + (size_t)inst * b->trace_max, cnt * sizeof(recon_iter_trace),
                      cudaMemcpyDeviceToHost));
    return cnt;
}

int64_t recon_batch_get_array(recon_batch *b, int32_t inst, const char *name, int32_t level, void *host_dst,
                              int64_t nbytes) {
    clear_stale_error();
    if (!b || inst < 0 || inst >= b->n || !name || !host_dst) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    const InstDesc &d = b->desc[inst];
    if (level < 0 || level >= d.L) return fail(RECON_ERR_INVALID_ARG, "bad level");
    int W = d.W >> level, H = d.H >> level, P = d.P, n0 = d.W * d.H;
    const void *src = nullptr;
    int64_t sz = 0;
    std::string nm(name);
    if (nm == "ref_gray") { src = d.ref_gray[level]; sz = (int64_t)W * H * 4; }
    else if (nm == "cur_gray") { src = d.cur_gray[level]; sz = (int64_t)W * H * 4; }
    else if (nm == "ref_z") { src = d.ref_z; sz = (int64_t)n0 * 4; }
    else if (nm == "ref_col") { src = d.ref_col; sz = (int64_t)n0 * 4; }
    else if (nm == "cur_z") { src = d.cur_z; sz = (int64_t)n0 * 4; }
    else if (nm == "ref_pts") { src = d.ref_pts[level]; sz = (int64_t)W * H * 16; }
    else if (nm == "ref_nrm") { src = d.ref_nrm[level]; sz = (int64_t)W * H * 16; }
    else if (nm == "cur_pts") { src = d.cur_pts[level]; sz = (int64_t)W * H * 16; }
    else if (nm == "sel_idx") { src = d.sel_idx; sz = (int64_t)P * 4; }
    else if (nm == "sel_xyz") { src = d.sel_xyz; sz = (int64_t)P * 12; }
    else if (nm == "sel_I") { src = d.sel_I[level]; sz = (int64_t)P * 4; }
    else if (nm == "sel_J") { src = d.sel_J[level]; sz = (int64_t)P * 24; }
    else if (nm == "gmag") { src = d.gmag; sz = (int64_t)n0 * 4; }
    else if (nm == "grad_hist") { src = d.grad_hist; sz = (int64_t)d.select_bins * 4; }
    else if (nm == "T") { src = d.T; sz = 64; }
    else if (nm == "icp_nsel") { src = d.icp_nsel; sz = 16; }
    else if (nm == "icp_mask") { src = d.icp_mask; sz = (int64_t)W * H; }
    else if (nm == "icp_w") { src = d.icp_w; sz = (int64_t)W * H * 4; }
    else return fail(RECON_ERR_INVALID_ARG, "unknown array");
    if (sz > nbytes) return fail(RECON_ERR_INVALID_ARG, "destination too small");
    CK(cudaStreamSynchronize(b->stream));
    CK(cudaMemcpy(host_dst, src, sz, cudaMemcpyDeviceToHost));
    return sz;
}

int recon_batch_enable_timing(recon_batch *b, int32_t on) {
    clear_stale_error();
    if (!b) return fail(RECON_ERR_INVALID_ARG, "null batch");
    CK(cudaStreamSynchronize(b->stream));
    if ((bool)on != b->timing) b->graph_dirty = true;
    b->timing = on != 0;
    for (int k = 0; k < 8; k++) { b->t_ms[k] = 0.0; b->t_cnt[k] = 0; }
    return RECON_OK;
}

int recon_batch_get_timing(recon_batch *b, double *ms, int64_t *launches, int32_t reset) {
    clear_stale_error();
    if (!b || !ms || !launches) return fail(RECON_ERR_INVALID_ARG, "null argument");
    CK(cudaStreamSynchronize(b->stream));
    collect_events(b, b->direct_events, true);
    for (int k = 0; k < TK_COUNT; k++) {
        ms[k] = b->t_ms[k];
        launches[k] = b->t_cnt[k];
        if (reset) { b->t_ms[k] = 0.0; b->t_cnt[k] = 0; }
    }
    return TK_COUNT;
}

int recon_batch_get_work(recon_batch *b, uint64_t *out, int32_t reset) {
    clear_stale_error();
    if (!b || !out) return fail(RECON_ERR_INVALID_ARG, "null argument");
    CK(cudaStreamSynchronize(b->stream));
    for (int i = 0; i < b->n; i++) {
        CK(cudaMemcpy(out + 4 * (size_t)i, b->desc[i].work, 4 * sizeof(uint64_t), cudaMemcpyDeviceToHost));
        if (reset) CK(cudaMemset(b->desc[i].work, 0, 4 * sizeof(uint64_t)));
    }
    return RECON_OK;
}

void *recon_batch_stream(recon_batch *b) { return b ? (void *)b->stream : nullptr; }

int64_t recon_launch_count(void) { return g_launches.load(); }

int recon_batch_track_sequence(recon_batch *b, int32_t nf, const uint8_t *const *gray, const uint16_t *const *depth,
                               int32_t on_device, float *T_out, recon_track_stats *stats) {
    clear_stale_error();
    if (!b || nf <= 0 || !gray || !depth) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    if (!b->have_ref) return fail(RECON_ERR_STATE, "reference frame missing");
    int n = b->n;
    for (size_t k = 0; k < (size_t)nf * n; k++)
        if (!gray[k] || !depth[k]) return fail(RECON_ERR_INVALID_ARG, "null frame pointer");
    size_t need_ptr = (size_t)nf * 3 * n;
    size_t need_T = (size_t)nf * n * 16;
    std::vector<size_t> px(n);
    size_t frame_bytes = 0;
    for (int i = 0; i < n; i++) {
        px[i] = (size_t)b->cfg[i].width * b->cfg[i].height;
        frame_bytes += align256(px[i]) + align256(2 * px[i]);
    }
    // a keyframe fusion may still read the last sequence's poses and slots:
    // let it finish before any buffer is reallocated
    if (b->recon_stream && (need_ptr > b->seqptr_cap || need_T > b->Tseq_cap ||
                            (!on_device && frame_bytes * nf > b->set_bytes)))
        CK(cudaStreamSynchronize(b->recon_stream));
    if (need_ptr > b->seqptr_cap) {
        if (b->d_seqptr) cudaFree(b->d_seqptr);
        if (b->h_seqptr) cudaFreeHost(b->h_seqptr);
        b->d_seqptr = nullptr;
        b->h_seqptr = nullptr;
        b->seqptr_cap = 0;
        CK(cudaMalloc(&b->d_seqptr, need_ptr * sizeof(void *)));
        CK(cudaMallocHost(&b->h_seqptr, need_ptr * sizeof(void *)));
        b->seqptr_cap = need_ptr;
    }
    if (need_T > b->Tseq_cap) {
        if (b->d_Tseq) cudaFree(b->d_Tseq);
        b->d_Tseq = nullptr;
        b->Tseq_cap = 0;
        CK(cudaMalloc(&b->d_Tseq, need_T * sizeof(float)));
        b->Tseq_cap = need_T;
    }
    b->seq_frames = 0;
    b->seq_set = -1;
    int set = 0;
    if (!on_device) {
        if (frame_bytes * nf > b->set_bytes) {
            // the previous calls' tracking has been waited for (their poses
            // were read back) and the fusion above
            if (b->d_slots) cudaFree(b->d_slots);
            b->d_slots = nullptr;
            b->set_bytes = 0;
            CK(cudaMalloc(&b->d_slots, 2 * frame_bytes * nf));
            b->set_bytes = frame_bytes * nf;
        }
        if (!b->copy_stream) CK(cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; k++) {
            if (!b->ev_copied[k]) CK(cudaEventCreateWithFlags(&b->ev_copied[k], cudaEventDisableTiming));
            if (!b->ev_set_read[k]) CK(cudaEventCreateWithFlags(&b->ev_set_read[k], cudaEventDisableTiming));
            if (!b->ev_set_fused[k]) CK(cudaEventCreateWithFlags(&b->ev_set_fused[k], cudaEventDisableTiming));
        }
        // this call's set was last read by the call before the previous one and
        // by a fusion of its frames: the copies into it wait for both (an event
        // never recorded is no wait)
        set = b->next_set;
        b->next_set ^= 1;
        CK(cudaStreamWaitEvent(b->copy_stream, b->ev_set_read[set], 0));
        CK(cudaStreamWaitEvent(b->copy_stream, b->ev_set_fused[set], 0));
        // frame f is copied into slot f, the only source of row f of the pointer table
        for (int f = 0; f < nf; f++) {
            size_t off = b->set_bytes * set + frame_bytes * f;
            for (int i = 0; i < n; i++) {
                b->h_seqptr[(size_t)f * 3 * n + i] = b->d_slots + off;
                off += align256(px[i]);
                b->h_seqptr[(size_t)f * 3 * n + n + i] = b->d_slots + off;
                off += align256(2 * px[i]);
                b->h_seqptr[(size_t)f * 3 * n + 2 * n + i] = nullptr;
            }
        }
    } else {
        for (int f = 0; f < nf; f++)
            for (int i = 0; i < n; i++) {
                b->h_seqptr[(size_t)f * 3 * n + i] = gray[(size_t)f * n + i];
                b->h_seqptr[(size_t)f * 3 * n + n + i] = depth[(size_t)f * n + i];
                b->h_seqptr[(size_t)f * 3 * n + 2 * n + i] = nullptr;
            }
    }
    CK(cudaMemcpyAsync(b->d_seqptr, b->h_seqptr, need_ptr * sizeof(void *), cudaMemcpyHostToDevice, b->stream));
    // the input row of frame f
    auto row_of = [&](int f) -> const void ** { return b->d_seqptr + (size_t)f * 3 * n; };
    // copy frame f into its slot on the copy stream (ev_copied[f & 1] marks it;
    // frame f's copies are issued after frame f - 1's, so the event recorded
    // later on the same stream also covers the earlier frames)
    // one 2-D copy per image kind when the instances' host images of a frame
    // and their slots are evenly spaced with one size (copy_images)
    std::vector<size_t> gbytes(n), dbytes(n);
    for (int i = 0; i < n; i++) {
        gbytes[i] = px[i];
        dbytes[i] = 2 * px[i];
    }
    auto stage = [&](int f) -> int {
        if (on_device) return RECON_OK;
        void *const *slots = (void *const *)(b->h_seqptr + (size_t)f * 3 * n);
        CK(copy_images((const void *const *)(gray + (size_t)f * n), slots, gbytes.data(), n, b->copy_stream));
        CK(copy_images((const void *const *)(depth + (size_t)f * n), slots + n, dbytes.data(), n, b->copy_stream));
        CK(cudaEventRecord(b->ev_copied[f & 1], b->copy_stream));
        return RECON_OK;
    };
    // The network input of a frame is two images, not a pose, so the network
    // runs one frame ahead on its own stream while the batch stream tracks the
    // previous frame; only the gate (which needs the previous pose) waits for it.
    // Frame f's outputs go to d_netout_seq[f & 1], free once gate(f - 2) ran.
    auto net_ahead = [&](int f) -> int {
        int k = f & 1;
        if (!on_device) CK(cudaStreamWaitEvent(b->net_stream, b->ev_copied[k], 0));
        CK(cudaStreamWaitEvent(b->net_stream, b->ev_gate[k], 0));
        int rc = learned_net(b, row_of(f), b->net_stream, b->d_netout_seq[k], b->d_gateD_seq[k]);
        if (rc) return rc;
        CK(cudaEventRecord(b->ev_net[k], b->net_stream));
        return RECON_OK;
    };
    if (b->net) {
        if (!b->net_stream) CK(cudaStreamCreateWithFlags(&b->net_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; k++) {
            if (!b->ev_net[k]) CK(cudaEventCreateWithFlags(&b->ev_net[k], cudaEventDisableTiming));
            if (!b->ev_gate[k]) CK(cudaEventCreateWithFlags(&b->ev_gate[k], cudaEventDisableTiming));
        }
        if (!b->ev_seq) CK(cudaEventCreateWithFlags(&b->ev_seq, cudaEventDisableTiming));
        // the pointer table and the keyframe's coarse image are written on the batch stream
        CK(cudaEventRecord(b->ev_seq, b->stream));
        CK(cudaStreamWaitEvent(b->net_stream, b->ev_seq, 0));
    }
    int rc0 = stage(0);
    if (rc0) return rc0;
    if (b->net && (rc0 = net_ahead(0))) return rc0;
    for (int f = 0; f < nf; f++) {
        const void **row = row_of(f);
        if (f + 1 < nf) {
            int rc = stage(f + 1);
            if (rc) return rc;
            if (b->net && (rc = net_ahead(f + 1))) return rc;
        }
        if (!on_device) CK(cudaStreamWaitEvent(b->stream, b->ev_copied[f & 1], 0));
        int rc = prepare_current(b, row, f > 0 ? b->d_Tseq + (size_t)(f - 1) * n * 16 : nullptr, true);
        if (rc) return rc;
        if (b->net) {
            CK(cudaStreamWaitEvent(b->stream, b->ev_net[f & 1], 0));
            rc = learned_gate(b, b->d_netout_seq[f & 1], b->d_gateD_seq[f & 1]);
            if (rc) return rc;
            CK(cudaEventRecord(b->ev_gate[f & 1], b->stream));
        }
        rc = run_schedule(b);
        if (rc) return rc;
        CK(cudaGetLastError());
    }
    // the last frame's pose (the earlier ones were stored by the next frame's pyramid launch)
    k_store_pose<<<dim3(1, n), 32, 0, b->stream>>>(b->d_desc, b->d_Tseq + (size_t)(nf - 1) * n * 16);
    g_launches += 1;
    if (!on_device) {
        CK(cudaEventRecord(b->ev_set_read[set], b->stream));
        b->seq_set = set;
    }
    b->have_cur = true;
    b->seq_frames = nf;
    if (T_out) CK(cudaMemcpyAsync(T_out, b->d_Tseq, need_T * sizeof(float), cudaMemcpyDeviceToHost, b->stream));
    return recon_batch_get_poses(b, nullptr, stats);
}

int recon_batch_set_init_net(recon_batch *b, recon_initnet *net, const int32_t iters[RECON_MAX_LEVELS]) {
    clear_stale_error();
    if (!b) return fail(RECON_ERR_INVALID_ARG, "null batch");
    int n = b->n;
    if (!net) {
        if (b->net) {
            for (int i = 0; i < n; i++) {
                for (int l = 0; l < kMaxLevels; l++) {
                    b->cfg[i].iters[l] = b->plain_iters[i][l];
                    b->desc[i].iters[l] = b->plain_iters[i][l];
                }
            }
        }
        b->net = nullptr;
        b->graph_dirty = true;
        return upload_desc(b);
    }
    if (!iters) return fail(RECON_ERR_INVALID_ARG, "null schedule");
    for (int i = 0; i < n; i++) {
        const recon_config &c = b->cfg[i];
        if (c.width % kNetW || c.height % kNetH)
            return fail(RECON_ERR_INVALID_ARG, "the learned initialisation needs frames of a multiple of 80x60");
        recon_config t = c;
        for (int l = 0; l < RECON_MAX_LEVELS; l++) t.iters[l] = iters[l];
        int rc = validate(t);
        if (rc) return rc;
    }
    if (!b->d_netin) {
        size_t px = (size_t)n * kNetW * kNetH;
        for (int k = 0; k < 2; k++) CK(cudaMalloc(&b->d_coarse[k], px * 2 * sizeof(uint16_t)));
        CK(cudaMalloc(&b->d_netin, px * 4 * sizeof(uint16_t)));
        CK(cudaMalloc(&b->d_netout, (size_t)n * 6 * sizeof(float)));
        for (int k = 0; k < 2; k++) CK(cudaMalloc(&b->d_netout_seq[k], (size_t)n * 6 * sizeof(float)));
        b->netout_last = b->d_netout;
        CK(cudaMalloc(&b->d_choice, (size_t)n * sizeof(int)));
        CK(cudaMalloc(&b->d_cand, (size_t)n * 16 * sizeof(float)));
        CK(cudaMalloc(&b->d_cost, (size_t)n * 2 * sizeof(long long)));
        CK(cudaMalloc(&b->d_ticket, (size_t)n * sizeof(unsigned int)));
        CK(cudaMalloc(&b->d_gateD, (size_t)n * 16 * sizeof(float)));
        for (int k = 0; k < 2; k++) CK(cudaMalloc(&b->d_gateD_seq[k], (size_t)n * 16 * sizeof(float)));
        CK(cudaMemsetAsync(b->d_cost, 0, (size_t)n * 2 * sizeof(long long), b->stream));
        CK(cudaMemsetAsync(b->d_ticket, 0, (size_t)n * sizeof(unsigned int), b->stream));
        CK(cudaMemsetAsync(b->d_coarse[0], 0, px * 2 * sizeof(uint16_t), b->stream));
        CK(cudaMemsetAsync(b->d_coarse[1], 0, px * 2 * sizeof(uint16_t), b->stream));
    }
    if (!b->net) {
        b->plain_iters.assign(n, std::vector<int>(kMaxLevels));
        for (int i = 0; i < n; i++)
            for (int l = 0; l < kMaxLevels; l++) b->plain_iters[i][l] = b->cfg[i].iters[l];
    }
    for (int i = 0; i < n; i++)
        for (int l = 0; l < kMaxLevels; l++) {
            b->cfg[i].iters[l] = iters[l];
            b->desc[i].iters[l] = iters[l];
        }
    b->net = net;
    b->graph_dirty = true;
    int rc = upload_desc(b);
    if (rc) return rc;
    if (b->have_ref) return learned_keyframe(b);
    return RECON_OK;
}

int recon_batch_get_init(recon_batch *b, int32_t *choice, float *net_out) {
    clear_stale_error();
    if (!b || !b->net) return fail(RECON_ERR_STATE, "no network attached");
    if (choice) CK(cudaMemcpyAsync(choice, b->d_choice, (size_t)b->n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    if (net_out)
        CK(cudaMemcpyAsync(net_out, b->netout_last, (size_t)b->n * 6 * sizeof(float), cudaMemcpyDeviceToHost,
                           b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return RECON_OK;
}

int recon_batch_fuse_keyframe(recon_batch *b, int32_t nframes, const uint16_t *const *depth, const float *T_host,
                              int32_t on_device, float gate_mm) {
    return recon_batch_fuse_keyframe_rgbd(b, nframes, nullptr, depth, T_host, on_device, gate_mm);
}

int recon_batch_fuse_sequence(recon_batch *b, int32_t nframes, float gate_mm) {
    clear_stale_error();
    if (!b || nframes < 1 || nframes > 8 || !(gate_mm > 0.0f))
        return fail(RECON_ERR_INVALID_ARG, "bad argument (1..8 frames, positive gate)");
    if (!b->have_ref) return fail(RECON_ERR_STATE, "reference frame missing");
    if (nframes > b->seq_frames) return fail(RECON_ERR_STATE, "the last sequence has fewer frames");
    int rc = fuse_prepare(b, (size_t)nframes * b->n);
    if (rc) return rc;
    int n = b->n;
    size_t cnt = (size_t)nframes * n;
    // depth pointers [cnt], then gray pointers [cnt], from the sequence's rows
    for (int f = 0; f < nframes; f++)
        for (int i = 0; i < n; i++) {
            size_t k = (size_t)f * n + i;
            b->h_fuse_ptr[k] = b->h_seqptr[(size_t)f * 3 * n + n + i];
            b->h_fuse_ptr[cnt + k] = b->h_seqptr[(size_t)f * 3 * n + i];
        }
    CK(cudaEventRecord(b->ev_pose, b->stream));
    CK(cudaStreamWaitEvent(b->recon_stream, b->ev_pose, 0));
    CK(cudaMemcpyAsync(b->d_fuse_ptr, b->h_fuse_ptr, 2 * cnt * sizeof(void *), cudaMemcpyHostToDevice,
                       b->recon_stream));
    rc = fuse_launch(b, nframes, true, b->d_Tseq, gate_mm);
    if (rc) return rc;
    // the frames of a host-input sequence live in its slot set until this fusion is done
    if (b->seq_set >= 0) CK(cudaEventRecord(b->ev_set_fused[b->seq_set], b->recon_stream));
    return RECON_OK;
}

int recon_batch_fuse_keyframe_rgbd(recon_batch *b, int32_t nframes, const uint8_t *const *gray,
                                   const uint16_t *const *depth, const float *T, int32_t on_device, float gate_mm) {
    clear_stale_error();
    if (!b || nframes < 1 || nframes > 8 || !depth || !T || !(gate_mm > 0.0f))
        return fail(RECON_ERR_INVALID_ARG, "bad argument (1..8 frames, poses, positive gate)");
    if (!b->have_ref) return fail(RECON_ERR_STATE, "reference frame missing");
    int n = b->n;
    size_t cnt = (size_t)nframes * n;
    for (size_t k = 0; k < cnt; k++)
        if (!depth[k] || (gray && !gray[k])) return fail(RECON_ERR_INVALID_ARG, "null frame pointer");
    int rc = fuse_prepare(b, cnt);
    if (rc) return rc;
    std::vector<size_t> px(n);
    size_t bytes = 0;
    for (int i = 0; i < n; i++) {
        px[i] = (size_t)b->cfg[i].width * b->cfg[i].height;
        bytes += (size_t)nframes * (align256(2 * px[i]) + (gray ? align256(px[i]) : 0));
    }
    // the fusion waits for the pose stream's pending work (tracked frames)
    CK(cudaEventRecord(b->ev_pose, b->stream));
    CK(cudaStreamWaitEvent(b->recon_stream, b->ev_pose, 0));
    // pointer table: depth pointers [cnt], then gray pointers [cnt]
    for (size_t k = 0; k < 2 * cnt; k++) b->h_fuse_ptr[k] = nullptr;
    if (!on_device) {
        if (bytes > b->fuse_bytes) {
            if (b->d_fuse) cudaFree(b->d_fuse);
            b->d_fuse = nullptr;
            b->fuse_bytes = 0;
            CK(cudaMalloc(&b->d_fuse, bytes));
            b->fuse_bytes = bytes;
        }
        size_t off = 0;
        for (int f = 0; f < nframes; f++)
            for (int i = 0; i < n; i++) {
                size_t k = (size_t)f * n + i;
                uint8_t *dst = b->d_fuse + off;
                CK(cudaMemcpyAsync(dst, depth[k], 2 * px[i], cudaMemcpyHostToDevice, b->recon_stream));
                b->h_fuse_ptr[k] = dst;
                off += align256(2 * px[i]);
                if (gray) {
                    dst = b->d_fuse + off;
                    CK(cudaMemcpyAsync(dst, gray[k], px[i], cudaMemcpyHostToDevice, b->recon_stream));
                    b->h_fuse_ptr[cnt + k] = dst;
                    off += align256(px[i]);
                }
            }
    } else {
        for (size_t k = 0; k < cnt; k++) {
            b->h_fuse_ptr[k] = depth[k];
            if (gray) b->h_fuse_ptr[cnt + k] = gray[k];
        }
    }
    CK(cudaMemcpyAsync(b->d_fuse_ptr, b->h_fuse_ptr, 2 * cnt * sizeof(void *), cudaMemcpyHostToDevice,
                       b->recon_stream));
    CK(cudaMemcpyAsync(b->d_fuse_T, T, cnt * 16 * sizeof(float), cudaMemcpyHostToDevice, b->recon_stream));
    rc = fuse_launch(b, nframes, gray != nullptr, b->d_fuse_T, gate_mm);
    if (rc) return rc;
    // pageable sources (the frames, T) must outlive the copies
    CK(cudaStreamSynchronize(b->recon_stream));
    return RECON_OK;
}

// ---- single tracker ----
int recon_tracker_create(const recon_config *cfg, const float *calib, void *stream, recon_tracker **out) {
    return recon_batch_create(1, cfg, calib, stream, out);
}
int recon_tracker_destroy(recon_tracker *t) { return recon_batch_destroy(t); }
int recon_set_reference(recon_tracker *t, const uint8_t *gray, const uint16_t *depth, int32_t on_device) {
    if (!t) return fail(RECON_ERR_INVALID_ARG, "null tracker");
    int rc = recon_batch_set_reference(t, &gray, &depth, on_device);
    if (rc == RECON_OK) identity16(t->T_host);  // prepareReference clears T (phototracker.cpp:362-368)
    return rc;
}
int recon_set_reference_oriented(recon_tracker *t, const uint8_t *gray, const uint16_t *depth, const float *points,
                                 const float *normals, int32_t on_device) {
    if (!t) return fail(RECON_ERR_INVALID_ARG, "null tracker");
    int rc = recon_batch_set_reference_oriented(t, &gray, &depth, &points, &normals, on_device);
    if (rc == RECON_OK) identity16(t->T_host);
    return rc;
}
int recon_set_current(recon_tracker *t, const uint8_t *gray, const uint16_t *depth, int32_t on_device) {
    return recon_batch_set_current(t, &gray, &depth, on_device);
}

// invertRT4 (basic_math.cpp:335-353) in double
static void invert_rt4d(const double *M, double *Mi) {
    Mi[0] = M[0]; Mi[1] = M[4]; Mi[2] = M[8];   Mi[3] = -(M[0] * M[3] + M[4] * M[7] + M[8] * M[11]);
    Mi[4] = M[1]; Mi[5] = M[5]; Mi[6] = M[9];   Mi[7] = -(M[1] * M[3] + M[5] * M[7] + M[9] * M[11]);
    Mi[8] = M[2]; Mi[9] = M[6]; Mi[10] = M[10]; Mi[11] = -(M[2] * M[3] + M[6] * M[7] + M[10] * M[11]);
    Mi[12] = 0;   Mi[13] = 0;   Mi[14] = 0;     Mi[15] = 1;
}

// matrixMult4x4 in double, each entry the left-to-right sum of its four
// products (basic_math.cpp:183-207); the product may alias an input
static void mult4x4d(const double *A, const double *B, double *C) {
    double t2[16];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++)
            t2[r * 4 + c] = A[r * 4 + 0] * B[0 * 4 + c] + A[r * 4 + 1] * B[1 * 4 + c] + A[r * 4 + 2] * B[2 * 4 + c] +
                            A[r * 4 + 3] * B[3 * 4 + c];
    memcpy(C, t2, sizeof(t2));
}

// PhotoTracker::applyIncrement (phototracker.cpp:514-531).  Trel is the
// tracked pose (reference -> current, the device pose).  The host pose T is
// kept as the reference keeps it: current -> reference, inverted in double
// and stored as float; the increment from the previous frame is
// inv(double(T_prev)) * inv(double(Trel)) and is accumulated into the double
// global pose.
static void apply_increment(recon_tracker *t, const float *Trel) {
    double TdblPrev[16], iTprev[16], iTdbl[16], Tdbl[16], Tinc[16];
    for (int i = 0; i < 16; i++) {
        TdblPrev[i] = (double)t->T_host[i];
        iTdbl[i] = (double)Trel[i];
    }
    invert_rt4d(TdblPrev, iTprev);
    invert_rt4d(iTdbl, Tdbl);
    for (int i = 0; i < 16; i++) t->T_host[i] = (float)Tdbl[i];
    mult4x4d(iTprev, Tdbl, Tinc);
    mult4x4d(t->global_pose, Tinc, t->global_pose);
}

// PhotoTracker::poseDifferenceExceeded (phototracker.cpp:268-288): the
// translation length of dT, and the rotation angle of dT from its unit
// quaternion (the identity rotation, to 1e-5 on the diagonal, is angle 0).
static bool pose_difference_exceeded(const float *dT, float dist_mm, float angle_deg) {
    double dx = dT[3], dy = dT[7], dz = dT[11];
    float dist = (float)std::sqrt(dx * dx + dy * dy + dz * dz + 1e-12f);
    if (dist > dist_mm) return true;
    float angle = 0.0f;
    if (std::fabs(dT[0] - 1.0f) > 1e-5 || std::fabs(dT[5] - 1.0f) > 1e-5 || std::fabs(dT[10] - 1.0f) > 1e-5) {
        // rotation -> unit quaternion (w, x, y, z), branching on the largest
        // diagonal term for stability (rot2Quaternion, basic_math.cpp:943-973)
        float q[4];
        float tr = dT[0] + dT[5] + dT[10];
        if (tr > 0) {
            float sc = 0.5f / std::sqrt(tr + 1.0f);
            q[0] = 0.25f / sc;
            q[1] = (dT[9] - dT[6]) * sc;
            q[2] = (dT[2] - dT[8]) * sc;
            q[3] = (dT[4] - dT[1]) * sc;
        } else if (dT[0] > dT[5] && dT[0] > dT[10]) {
            float sc = 2.0f * std::sqrt(1.0f + dT[0] - dT[5] - dT[10]);
            q[0] = (dT[9] - dT[6]) / sc;
            q[1] = 0.25f * sc;
            q[2] = (dT[1] + dT[4]) / sc;
            q[3] = (dT[2] + dT[8]) / sc;
        } else if (dT[5] > dT[10]) {
            float sc = 2.0f * std::sqrt(1.0f + dT[5] - dT[0] - dT[10]);
            q[0] = (dT[2] - dT[8]) / sc;
            q[1] = (dT[1] + dT[4]) / sc;
            q[2] = 0.25f * sc;
            q[3] = (dT[6] + dT[9]) / sc;
        } else {
            float sc = 2.0f * std::sqrt(1.0f + dT[10] - dT[0] - dT[5]);
            q[0] = (dT[4] - dT[1]) / sc;
            q[1] = (dT[2] + dT[8]) / sc;
            q[2] = (dT[6] + dT[9]) / sc;
            q[3] = 0.25f * sc;
        }
        // normalizeQuaternion (basic_math.cpp:1006-1013)
        float len = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3] + 1e-7f);
        for (int k = 0; k < 4; k++) q[k] /= len;
        angle = (float)(std::acos((double)q[0]) * 2.0f * 180.0f / 3.141592653f);
    }
    return angle > angle_deg;
}

int recon_track(recon_tracker *t, float T_io[16], recon_track_stats *stats) {
    if (!t) return fail(RECON_ERR_INVALID_ARG, "null tracker");
    float T[16];
    if (T_io) memcpy(T, T_io, sizeof(T));
    int rc = recon_batch_track_async(t, T_io ? T : nullptr);
    if (rc) return rc;
    rc = recon_batch_get_poses(t, T, stats);
    if (rc) return rc;
    apply_increment(t, T);
    if (T_io) memcpy(T_io, T, sizeof(T));
    return stats ? stats[0].status : RECON_OK;
}
int recon_set_iterations(recon_tracker *t, const int32_t iters[RECON_MAX_LEVELS]) {
    return recon_batch_set_iterations(t, 0, iters);
}
int recon_set_mode(recon_tracker *t, int32_t mode, float lambda) { return recon_batch_set_mode(t, 0, mode, lambda); }
int recon_set_settle(recon_tracker *t, float tol_mm, float tol_rot) { return recon_batch_set_settle(t, 0, tol_mm, tol_rot); }
int recon_get_relative_pose(recon_tracker *t, float T[16]) {
    if (!t || !T) return fail(RECON_ERR_INVALID_ARG, "null argument");
    memcpy(T, t->T_host, sizeof(t->T_host));
    return RECON_OK;
}

int recon_set_reference_updating(recon_tracker *t, int32_t on, float dist_mm, float angle_deg) {
    if (!t || !(dist_mm > 0.0f) || !(angle_deg > 0.0f)) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    t->ref_updating = on != 0;
    t->ref_dist_mm = dist_mm;
    t->ref_angle_deg = angle_deg;
    return RECON_OK;
}

int recon_reference_outdated(recon_tracker *t) {
    if (!t) return fail(RECON_ERR_INVALID_ARG, "null tracker");
    if (!t->have_ref) return 1;
    return (t->ref_updating && pose_difference_exceeded(t->T_host, t->ref_dist_mm, t->ref_angle_deg)) ? 1 : 0;
}

int recon_pose_difference_exceeded(const float dT[16], float dist_mm, float angle_deg) {
    if (!dT) return fail(RECON_ERR_INVALID_ARG, "null pose");
    return pose_difference_exceeded(dT, dist_mm, angle_deg) ? 1 : 0;
}

int recon_batch_reference_outdated(recon_batch *b, float dist_mm, float angle_deg, int32_t *outdated) {
    clear_stale_error();
    if (!b || !outdated || !(dist_mm > 0.0f) || !(angle_deg > 0.0f)) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    if (!b->have_ref) {
        for (int i = 0; i < b->n; i++) outdated[i] = 1;
        return RECON_OK;
    }
    std::vector<float> T(16 * (size_t)b->n);
    int rc = recon_batch_get_poses(b, T.data(), nullptr);
    if (rc) return rc;
    for (int i = 0; i < b->n; i++) {
        // the reference tests its host pose T = inv(Trel), inverted in double and stored as float
        double Td[16], Ti[16];
        float Tf[16];
        for (int k = 0; k < 16; k++) Td[k] = (double)T[16 * (size_t)i + k];
        invert_rt4d(Td, Ti);
        for (int k = 0; k < 16; k++) Tf[k] = (float)Ti[k];
        outdated[i] = pose_difference_exceeded(Tf, dist_mm, angle_deg) ? 1 : 0;
    }
    return RECON_OK;
}
int recon_get_global_pose(recon_tracker *t, double T[16]) {
    if (!t || !T) return fail(RECON_ERR_INVALID_ARG, "null argument");
    memcpy(T, t->global_pose, sizeof(t->global_pose));
    return RECON_OK;
}
int recon_reset(recon_tracker *t) {
    clear_stale_error();
    if (!t) return fail(RECON_ERR_INVALID_ARG, "null tracker");
    identity16d(t->global_pose);
    identity16(t->T_host);
    float I[16];
    identity16(I);
    CK(cudaMemcpyAsync(t->desc[0].T, I, sizeof(I), cudaMemcpyHostToDevice, t->stream));
    CK(cudaStreamSynchronize(t->stream));
    t->have_ref = false;
    t->have_cur = false;
    return RECON_OK;
}

// ---- renderer ----
int recon_render_depth(const void *scene, const void *camera, float noise_rel, uint32_t noise_seed, uint32_t frame,
                       uint16_t *depth_dev, void *stream) {
    clear_stale_error();
    if (!scene || !camera || !depth_dev) return fail(RECON_ERR_INVALID_ARG, "null argument");
    recon_scene sc;
    recon_camera cam;
    memcpy(&sc, scene, sizeof(sc));
    memcpy(&cam, camera, sizeof(cam));
    int n = cam.width * cam.height;
    k_render_depth<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(sc, cam, noise_rel, noise_seed, frame, depth_dev);
    g_launches += 1;
    CK(cudaGetLastError());
    return RECON_OK;
}

int recon_render_gray(const void *scene, const void *camera, uint8_t *gray_dev, void *stream) {
    clear_stale_error();
    if (!scene || !camera || !gray_dev) return fail(RECON_ERR_INVALID_ARG, "null argument");
    recon_scene sc;
    recon_camera cam;
    memcpy(&sc, scene, sizeof(sc));
    memcpy(&cam, camera, sizeof(cam));
    int n = cam.width * cam.height;
    k_render_gray<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(sc, cam, gray_dev);
    g_launches += 1;
    CK(cudaGetLastError());
    return RECON_OK;
}

}  // extern "C"
