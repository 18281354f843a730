// solve.cuh -- FP64 6x6 solve and SE(3) pose update, executed by one warp.
//
// The arithmetic of every matrix element is the same sequence of FP64
// operations as the oracle's restatement, so the results are bit-identical;
// lanes only evaluate independent elements concurrently.  GB300's FP64 rate is
// low (~1.25 TFLOP/s per GPU), so spreading the 4x4 products over 16 lanes
// matters more than it would on a datacenter part with full FP64.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace rt {

struct SolveScratch {
    double A[36], b[6], x[6], L[36], y[6];
    double M[6][16];  // X, X2, X4, X6 / U0, V / N, D
    double E[16], T[16], Tinc[16];
    double red[2];
    int piv;
    int ns;
    int status;
};

// 4x4 product R = M1 * M2 (matrixMult4Real, expmCuda.cu:1894-1917); R may alias.
__device__ __forceinline__ void wmat4(const double *M1, const double *M2, double *R, int lane) {
    double t = 0.0;
    if (lane < 16) {
        int r = lane >> 2, c = lane & 3;
        t = M1[r * 4 + 0] * M2[0 * 4 + c] + M1[r * 4 + 1] * M2[1 * 4 + c] + M1[r * 4 + 2] * M2[2 * 4 + c] +
            M1[r * 4 + 3] * M2[3 * 4 + c];
    }
    __syncwarp();
    if (lane < 16) R[lane] = t;
    __syncwarp();
}

// normalizeMat4RealSafe, expmCuda.cu:1955-1980 (lane 0)
__device__ __forceinline__ void normalize_mat4_safe(double *T) {
    double u0 = T[0], u1 = T[4], u2 = T[8];
    double v0 = T[1], v1 = T[5], v2 = T[9];
    double w0 = T[2], w1 = T[6], w2 = T[10];
    double lenU = (double)sqrtf((float)(u0 * u0 + u1 * u1 + u2 * u2));
    double lenW = (double)sqrtf((float)(w0 * w0 + w1 * w1 + w2 * w2));
    if (lenW > 1e-8f) { w0 /= lenW; w1 /= lenW; w2 /= lenW; }
    else { w0 = 0; w1 = 0; w2 = 1; }
    u0 = v1 * w2 - v2 * w1;
    u1 = -(v0 * w2 - v2 * w0);
    u2 = v0 * w1 - v1 * w0;
    if (lenU > 1e-8f) { u0 /= lenU; u1 /= lenU; u2 /= lenU; }
    else { u0 = 1; u1 = 0; u2 = 0; }
    v0 = w1 * u2 - w2 * u1;
    v1 = -(w0 * u2 - w2 * u0);
    v2 = w0 * u1 - w1 * u0;
    T[0] = u0; T[4] = u1; T[8] = u2;
    T[1] = v0; T[5] = v1; T[9] = v2;
    T[2] = w0; T[6] = w1; T[10] = w2;
}

__device__ __forceinline__ int expm_squarings(double hnorm) {
    if (!(hnorm > 0.0)) return 0;
    int e;
    double mant = frexp(hnorm, &e);
    int tl;
    if (hnorm >= 1.0) tl = e - 1;
    else tl = (mant == 0.5) ? e - 1 : e;
    int ns = tl + 2;
    return ns < 0 ? 0 : ns;
}

// exp(A) by the diagonal (6,6) Pade approximant with scaling and squaring (the
// method of EXPOKIT zgpadm used at expmCuda.cu:1642), real FP64.  Result in S.E.
static __device__ void wexpm_twist(SolveScratch &S, const double *A, int lane) {
    if (lane == 0) {
        double hnorm = 0.0;
        for (int r = 0; r < 4; r++) {
            double s = 0.0;
            for (int c = 0; c < 4; c++) s = s + fabs(A[r * 4 + c]);
            if (s > hnorm) hnorm = s;
        }
        S.ns = expm_squarings(hnorm);
    }
    __syncwarp();
    int ns = S.ns;
    double scale = ldexp(1.0, -ns);
    double *X = S.M[0], *X2 = S.M[1], *X4 = S.M[2], *X6 = S.M[3], *U0 = S.M[4], *V = S.M[5];
    if (lane < 16) X[lane] = A[lane] * scale;
    __syncwarp();
    wmat4(X, X, X2, lane);
    wmat4(X2, X2, X4, lane);
    wmat4(X4, X2, X6, lane);
    double c[7];
    c[0] = 1.0;
    for (int k = 1; k <= 6; k++) c[k] = c[k - 1] * (double)(6 - k + 1) / (double)(k * (12 - k + 1));
    if (lane < 16) {
        double I = (lane % 5 == 0) ? 1.0 : 0.0;
        U0[lane] = c[1] * I + c[3] * X2[lane] + c[5] * X4[lane];
        V[lane] = c[0] * I + c[2] * X2[lane] + c[4] * X4[lane] + c[6] * X6[lane];
    }
    __syncwarp();
    double *U = S.M[1];  // X2 no longer needed
    wmat4(X, U0, U, lane);
    double *Nm = S.M[2], *Dm = S.M[3];
    if (lane < 16) {
        Nm[lane] = V[lane] + U[lane];
        Dm[lane] = V[lane] - U[lane];
    }
    __syncwarp();
    // LU with partial pivoting, X = D^{-1} N (same operation order as the oracle)
    int singular = 0;
    for (int k = 0; k < 4; k++) {
        if (lane == 0) {
            int p = k;
            double best = fabs(Dm[k * 4 + k]);
            for (int i = k + 1; i < 4; i++) {
                double v = fabs(Dm[i * 4 + k]);
                if (v > best) { best = v; p = i; }
            }
            S.piv = (best == 0.0) ? -1 : p;
        }
        __syncwarp();
        int p = S.piv;
        if (p < 0) { singular = 1; break; }
        if (p != k && lane < 4) {
            double t = Dm[k * 4 + lane]; Dm[k * 4 + lane] = Dm[p * 4 + lane]; Dm[p * 4 + lane] = t;
            t = Nm[k * 4 + lane]; Nm[k * 4 + lane] = Nm[p * 4 + lane]; Nm[p * 4 + lane] = t;
        }
        __syncwarp();
        // lanes (i - k - 1) * 8 + col: col 0..3 -> D, 4..7 -> N
        int i = k + 1 + (lane >> 3);
        int col = lane & 7;
        double nv = 0.0;
        bool act = (i < 4);
        if (act) {
            double f = Dm[i * 4 + k] / Dm[k * 4 + k];
            if (col < 4) {
                if (col >= k) nv = Dm[i * 4 + col] - f * Dm[k * 4 + col];
                else act = false;
            } else {
                nv = Nm[i * 4 + (col - 4)] - f * Nm[k * 4 + (col - 4)];
            }
        }
        __syncwarp();
        if (act) {
            if (col < 4) Dm[i * 4 + col] = nv;
            else Nm[i * 4 + (col - 4)] = nv;
        }
        __syncwarp();
    }
    if (singular) {
        if (lane < 16) S.E[lane] = (lane % 5 == 0) ? 1.0 : 0.0;
        __syncwarp();
        return;
    }
    if (lane < 4) {
        int c2 = lane;
        for (int i = 3; i >= 0; i--) {
            double s = Nm[i * 4 + c2];
            for (int k = i + 1; k < 4; k++) s = s - Dm[i * 4 + k] * Nm[k * 4 + c2];
            Nm[i * 4 + c2] = s / Dm[i * 4 + i];
        }
    }
    __syncwarp();
    for (int k = 0; k < ns; k++) wmat4(Nm, Nm, Nm, lane);
    if (lane < 16) S.E[lane] = Nm[lane];
    __syncwarp();
}

// generateA + expmKernel (warp.cu:910-915, expmCuda.cu:1989-2048): T <- T * exp(A(x)),
// translation scaled by scaleOut, stored as float.  TF is shared memory or global.
static __device__ void wexpm_update(SolveScratch &S, const double *x, float *TF, double scaleOut, int lane) {
    double A[16] = {0, -x[2], x[1], x[3], x[2], 0, -x[0], x[4], -x[1], x[0], 0, x[5], 0, 0, 0, 0};
    double maxEntry = 0;
    for (int i = 0; i < 16; i++) {
        double a = fabs(A[i]);
        if (a > maxEntry) maxEntry = a;
    }
    if (lane < 16) S.T[lane] = (double)TF[lane];
    __syncwarp();
    if (maxEntry != 0) {
        wexpm_twist(S, A, lane);
        if (lane == 0) {
            for (int i = 0; i < 16; i++) S.Tinc[i] = S.E[i];
            normalize_mat4_safe(S.Tinc);
            S.Tinc[3] *= scaleOut;
            S.Tinc[7] *= scaleOut;
            S.Tinc[11] *= scaleOut;
        }
    } else {
        if (lane < 16) S.Tinc[lane] = (lane % 5 == 0) ? 1.0 : 0.0;
    }
    __syncwarp();
    wmat4(S.T, S.Tinc, S.T, lane);
    if (lane == 0) normalize_mat4_safe(S.T);
    __syncwarp();
    if (lane < 16) TF[lane] = (float)S.T[lane];
    __syncwarp();
}

// FP64 Cholesky + substitutions (same order as the oracle). Returns 0 / -1.
static __device__ int wcholesky(SolveScratch &S, int lane) {
    const double *A = S.A;
    double *L = S.L;
    if (lane < 36) {
        for (int i = lane; i < 36; i += 32) L[i] = 0.0;
    }
    __syncwarp();
    for (int j = 0; j < 6; j++) {
        if (lane == 0) {
            double d = A[j * 6 + j];
            for (int k = 0; k < j; k++) d = d - L[j * 6 + k] * L[j * 6 + k];
            if (!(d > 0.0)) {
                S.status = -1;
            } else {
                L[j * 6 + j] = sqrt(d);
            }
        }
        __syncwarp();
        if (S.status != 0) return -1;
        int i = j + 1 + lane;
        double v = 0.0;
        if (i < 6) {
            double s = A[i * 6 + j];
            for (int k = 0; k < j; k++) s = s - L[i * 6 + k] * L[j * 6 + k];
            v = s / L[j * 6 + j];
        }
        __syncwarp();
        if (i < 6) L[i * 6 + j] = v;
        __syncwarp();
    }
    if (lane == 0) {
        for (int i = 0; i < 6; i++) {
            double s = S.b[i];
            for (int k = 0; k < i; k++) s = s - L[i * 6 + k] * S.y[k];
            S.y[i] = s / L[i * 6 + i];
        }
        for (int i = 5; i >= 0; i--) {
            double s = S.y[i];
            for (int k = i + 1; k < 6; k++) s = s - L[k * 6 + i] * S.x[k];
            S.x[i] = s / L[i * 6 + i];
        }
    }
    __syncwarp();
    return 0;
}

// conjugateGradientKernel, warp.cu:926-975 (lane 0)
static __device__ void cg_solve(const double *A, const double *bb, double tol, int maxSteps, double *x) {
    double r[6], dir[6];
    for (int i = 0; i < 6; i++) { x[i] = 0.0; r[i] = bb[i]; dir[i] = bb[i]; }
    int nSteps = 0;
    while (nSteps < maxSteps) {
        double Adir[6];
        for (int j = 0; j < 6; j++) {
            Adir[j] = 0.0;
            for (int k = 0; k < 6; k++) Adir[j] += A[j * 6 + k] * dir[k];
        }
        double rr = 0, Adirdir = 0;
        for (int i = 0; i < 6; i++) rr += r[i] * r[i];
        for (int i = 0; i < 6; i++) Adirdir += Adir[i] * dir[i];
        double dv = Adirdir;
        if (dv < 0) dv = -dv;
        double stepLength = 0.0;
        if (dv > tol) stepLength = rr / Adirdir;
        for (int i = 0; i < 6; i++) r[i] -= stepLength * Adir[i];
        double rr2 = 0;
        for (int i = 0; i < 6; i++) rr2 += r[i] * r[i];
        for (int i = 0; i < 6; i++) x[i] += stepLength * dir[i];
        if (sqrt(rr2) < tol) return;
        double beta = rr2 / rr;
        for (int i = 0; i < 6; i++) dir[i] = r[i] + beta * dir[i];
        nSteps++;
    }
}

// Solve S.A x = S.b and apply the update to TF.  Returns the solve status.
static __device__ int wsolve_update(SolveScratch &S, int solver, float *TF, double scaleOut, int lane) {
    if (lane == 0) S.status = 0;
    __syncwarp();
    int st = 0;
    if (solver == 1) {
        if (lane == 0) cg_solve(S.A, S.b, 1e-8, 6, S.x);
        __syncwarp();
    } else {
        st = wcholesky(S, lane);
        if (st != 0) {
            if (lane < 6) S.x[lane] = 0.0;
            __syncwarp();
        }
    }
    double x[6];
    for (int i = 0; i < 6; i++) x[i] = S.x[i];
    wexpm_update(S, x, TF, scaleOut, lane);
    return st;
}

}  // namespace rt
