// trajio.cu -- the reference's result files on the host: the estimated
// trajectory (ResultTxt, tracker/calib/ResultTxt.cpp:17-76) and the
// per-segment tracking mode list (TrackingParams, tracker/calib/
// TrackingParams.cpp:50-95, e.g. data/best-method.tst).
//
// The file formats have to be the reference's to interoperate with its
// evaluation scripts: one line per pose, "i: " and 16 numbers in %e, after
// every pose is left-multiplied by the inverse of the first (canonize, in
// float, with invertRT4 and matrixMult4x4's summation order); one line per
// segment, "frame mode error" with mode geometric, photometric or
// biobjective-lambda<value>.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <climits>
#include <string>
#include <vector>

#include "../../include/recon_track.h"

namespace rt {
void set_last_error(const char *msg);
}  // namespace rt

namespace {

constexpr int kMaxPoses = 10000;  // MAX_POSE_COUNT (ResultTxt.h:19)

int fail(int code, const std::string &msg) {
    rt::set_last_error(msg.c_str());
    return code;
}

// invertRT4 (basic_math.cpp:355-368) in float
void invert_rt4f(const float *M, float *Mi) {
    Mi[0] = M[0]; Mi[1] = M[4]; Mi[2] = M[8];
    Mi[3] = -(M[0] * M[3] + M[4] * M[7] + M[8] * M[11]);
    Mi[4] = M[1]; Mi[5] = M[5]; Mi[6] = M[9];
    Mi[7] = -(M[1] * M[3] + M[5] * M[7] + M[9] * M[11]);
    Mi[8] = M[2]; Mi[9] = M[6]; Mi[10] = M[10];
    Mi[11] = -(M[2] * M[3] + M[6] * M[7] + M[10] * M[11]);
    Mi[12] = 0; Mi[13] = 0; Mi[14] = 0; Mi[15] = 1;
}

// matrixMult4x4 (basic_math.cpp:85-112) in float: each element summed left to right
void mult4x4f(const float *A, const float *B, float *R) {
    float t[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            t[i * 4 + j] = A[i * 4] * B[j] + A[i * 4 + 1] * B[4 + j] + A[i * 4 + 2] * B[8 + j] + A[i * 4 + 3] * B[12 + j];
    memcpy(R, t, sizeof(t));
}

}  // namespace

extern "C" {

int recon_trajectory_save(const char *path, const float *poses, int32_t n, int32_t transpose, int32_t inverse) {
    if (!path || (n > 0 && !poses) || n < 0) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    if (n == 0) return RECON_OK;  // ResultTxt::save writes nothing without poses
    if (n > kMaxPoses) n = kMaxPoses;  // ResultTxt::addPose keeps the first MAX_POSE_COUNT
    std::vector<float> data(poses, poses + 16 * (size_t)n);
    float mi[16];
    invert_rt4f(&data[0], mi);
    for (int i = 0; i < n; i++) mult4x4f(mi, &data[16 * (size_t)i], &data[16 * (size_t)i]);
    FILE *f = fopen(path, "wb");
    if (!f) return fail(RECON_ERR_INVALID_ARG, std::string("cannot open ") + path);
    for (int i = 0; i < n; i++) {
        const float *m = &data[16 * (size_t)i];
        float a[16], b[16];
        if (inverse)
            invert_rt4f(m, a);
        else
            memcpy(a, m, sizeof(a));
        // transpose4x4 (basic_math.cpp:221-227)
        if (transpose)
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++) b[c + r * 4] = a[r + c * 4];
        else
            memcpy(b, a, sizeof(b));
        fprintf(f, "%d: %e %e %e %e %e %e %e %e %e %e %e %e %e %e %e %e\n", i + 1, b[0], b[4], b[8], b[12], b[1], b[5],
                b[9], b[13], b[2], b[6], b[10], b[14], b[3], b[7], b[11], b[15]);
    }
    if (fclose(f) != 0) return fail(RECON_ERR_INVALID_ARG, std::string("cannot write ") + path);
    return RECON_OK;
}

int32_t recon_trajectory_load(const char *path, float *poses, int32_t max_n, int32_t transpose) {
    if (!path || !poses || max_n < 0) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    FILE *f = fopen(path, "rb");
    if (!f) return fail(RECON_ERR_INVALID_ARG, std::string("cannot open ") + path);
    int32_t n = 0;
    char line[1024];
    while (n < max_n && fgets(line, sizeof(line), f)) {
        int idx = 0;
        float v[16];
        int got = sscanf(line, "%d: %e %e %e %e %e %e %e %e %e %e %e %e %e %e %e %e", &idx, &v[0], &v[1], &v[2], &v[3],
                         &v[4], &v[5], &v[6], &v[7], &v[8], &v[9], &v[10], &v[11], &v[12], &v[13], &v[14], &v[15]);
        if (got != 17) continue;
        // the line is b[0], b[4], b[8], b[12], b[1], ... of the written matrix b
        float b[16];
        for (int c = 0; c < 4; c++)
            for (int r = 0; r < 4; r++) b[r * 4 + c] = v[c * 4 + r];
        float *m = poses + 16 * (size_t)n;
        if (transpose)
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++) m[r * 4 + c] = b[c * 4 + r];
        else
            memcpy(m, b, sizeof(b));
        n++;
    }
    fclose(f);
    return n;
}

int32_t recon_track_params_load(const char *path, int32_t *frames, int32_t *modes, float *lambdas, int32_t max_n) {
    if (!path || !frames || !modes || !lambdas || max_n < 0) return fail(RECON_ERR_INVALID_ARG, "bad argument");
    FILE *f = fopen(path, "rb");
    if (!f) return fail(RECON_ERR_INVALID_ARG, std::string("cannot open ") + path);
    int32_t n = 0;
    int lineno = 0;
    char line[1024];
    int rc = RECON_OK;
    while (fgets(line, sizeof(line), f)) {
        lineno++;
        int frame = 0;
        char mode[512] = {0};
        float err = 0.0f;
        if (sscanf(line, "%d %511s %e", &frame, mode, &err) < 2) continue;
        int m;
        float lam;
        if (!strcmp(mode, "geometric")) {
            m = RECON_GEOMETRIC;
            lam = 1.0f;
        } else if (!strcmp(mode, "photometric")) {
            m = RECON_PHOTOMETRIC;
            lam = 0.0f;
        } else if (!strncmp(mode, "biobjective", strlen("biobjective"))) {
            m = RECON_BIOBJECTIVE;
            // atof of what follows "biobjective-lambda" (TrackingParams.cpp:88)
            lam = strlen(mode) >= strlen("biobjective-lambda") ? (float)atof(mode + strlen("biobjective-lambda")) : 0.0f;
        } else {
            rc = fail(RECON_ERR_INVALID_ARG, std::string(path) + ":" + std::to_string(lineno) + ": invalid mode " + mode);
            break;
        }
        if (n < max_n) {
            frames[n] = frame;
            modes[n] = m;
            lambdas[n] = lam;
        }
        n++;
    }
    fclose(f);
    return rc == RECON_OK ? n : rc;
}

int32_t recon_track_params_lookup(const int32_t *frames, int32_t n, int32_t frame) {
    if (!frames || n <= 0) return -1;
    int best = 0;
    long long best_d = LLONG_MAX;
    for (int i = 0; i < n; i++) {
        long long d = llabs((long long)frames[i] - frame);
        if (d < best_d) {
            best_d = d;
            best = i;
        }
    }
    return best;
}

}  // extern "C"
