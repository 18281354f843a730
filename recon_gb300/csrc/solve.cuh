// solve.cuh -- FP64 6x6 solve and SE(3) pose update, executed by one warp.
//
// Every matrix element goes through the same sequence of FP64 operations as the
// oracle's restatement (orc_solve_cholesky, orc_expm_update), so the results
// are bit-identical; lanes only evaluate independent elements concurrently.
// On GB300 an FP64 warp instruction occupies its SM sub-partition for about 64
// cycles whether or not it depends on the previous one, and a divide or square
// root costs about ten of them.  The layout below therefore keeps the serial
// FP64 chain short: every product added to a sum is one fused multiply-add
// (the oracle's fma, one rounding), one reciprocal per pivot instead of a
// divide per element, lane-parallel substitutions, and comparisons of
// magnitudes on the integer bit patterns instead of FP64 compares.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace rt {

constexpr unsigned kFull = 0xffffffffu;

struct SolveScratch {
    double A[36], b[6], x[6], L[36], U[36], inv[6];
    double M[6][16];  // X, X2, X4, X6 / U0, V / N, D
    double E[16], T[16], Tinc[16];
    double lu_inv[3];
    int status;
};

// Pade (6,6) coefficients c_k = c_{k-1} (q-k+1) / (k (2q-k+1)), q = 6, in the
// oracle's FP64 evaluation order.
__device__ __constant__ const double kPade[7] = {0x1.0000000000000p+0, 0x1.0000000000000p-1, 0x1.d1745d1745d17p-4,
                                                 0x1.f07c1f07c1f07p-7, 0x1.4afd6a052bf5ap-10, 0x1.08cabb37565e2p-14,
                                                 0x1.937e11175f095p-20};

// |v| as an integer: for non-NaN values its order is the order of |v|
__device__ __forceinline__ long long abs_bits(double v) { return __double_as_longlong(v) & 0x7fffffffffffffffLL; }
constexpr long long kInfBits = 0x7ff0000000000000LL;

// 4x4 product R = M1 * M2 (matrixMult4Real, expmCuda.cu:1894-1917), each entry
// the first product then three fused multiply-adds; R may alias.
__device__ __forceinline__ void wmat4(const double *M1, const double *M2, double *R, int lane) {
    double t = 0.0;
    if (lane < 16) {
        int r = lane >> 2, c = lane & 3;
        t = M1[r * 4 + 0] * M2[0 * 4 + c];
        t = __fma_rn(M1[r * 4 + 1], M2[1 * 4 + c], t);
        t = __fma_rn(M1[r * 4 + 2], M2[2 * 4 + c], t);
        t = __fma_rn(M1[r * 4 + 3], M2[3 * 4 + c], t);
    }
    __syncwarp();
    if (lane < 16) R[lane] = t;
    __syncwarp();
}

// normalizeMat4RealSafe, expmCuda.cu:1955-1980, as the oracle states it: lengths
// through sqrtf, the old first column's length for the new one, products with
// the reciprocal lengths.  Lane i < 3 handles row i of the three columns.
__device__ __forceinline__ void wnormalize(double *T, int lane) {
    double len = 0.0;
    if (lane < 2) {
        int c = lane ? 2 : 0;
        double a = T[c], b = T[4 + c], e = T[8 + c];
        len = (double)sqrtf((float)__fma_rn(e, e, __fma_rn(b, b, a * a)));
    }
    double lenU = __shfl_sync(kFull, len, 0), lenW = __shfl_sync(kFull, len, 1);
    bool okU = lenU > 1e-8f, okW = lenW > 1e-8f;
    double il = 0.0;
    if (lane < 2 && (lane ? okW : okU)) il = 1.0 / len;
    double iu = __shfl_sync(kFull, il, 0), iw = __shfl_sync(kFull, il, 1);
    int i = lane < 3 ? lane : 0;
    double wi = okW ? T[4 * i + 2] * iw : (i == 2 ? 1.0 : 0.0);
    double vi = T[4 * i + 1];
    // crossproductReal (expmCuda.cu:1934-1938): component i uses rows ia, ib
    int ia = (i == 0) ? 1 : 0, ib = (i == 2) ? 1 : 2;
    double w_a = __shfl_sync(kFull, wi, ia), w_b = __shfl_sync(kFull, wi, ib);
    double v_a = __shfl_sync(kFull, vi, ia), v_b = __shfl_sync(kFull, vi, ib);
    // component 1 is v0 w2 - v2 w0 negated: written as -v0 w2 + v2 w0 so that
    // no fused result is negated (a negated zero sum would flip its sign)
    double ui = (i == 1) ? __fma_rn(-v_a, w_b, v_b * w_a) : __fma_rn(v_a, w_b, -(v_b * w_a));
    ui = okU ? ui * iu : (i == 0 ? 1.0 : 0.0);
    double u_a = __shfl_sync(kFull, ui, ia), u_b = __shfl_sync(kFull, ui, ib);
    double vn = (i == 1) ? __fma_rn(-w_a, u_b, w_b * u_a) : __fma_rn(w_a, u_b, -(w_b * u_a));
    __syncwarp();
    if (lane < 3) {
        T[4 * i] = ui;
        T[4 * i + 1] = vn;
        T[4 * i + 2] = wi;
    }
    __syncwarp();
}

// EXPOKIT's number of squarings, int(log2 ||A||_inf) + 2 truncated toward zero
// (at least 0), from the bits of the norm (the oracle evaluates it with frexp).
__device__ __forceinline__ int expm_squarings_bits(long long hb) {
    if (hb <= 0) return 0;
    int Eb = (int)(hb >> 52);
    if (Eb == 0) return 0;   // subnormal: far below 1
    if (Eb == 0x7ff) return 1;  // infinite norm (frexp leaves the exponent 0)
    bool frac0 = (hb & ((1LL << 52) - 1)) == 0;
    int tl = (Eb >= 1023) ? Eb - 1023 : (frac0 ? Eb - 1023 : Eb - 1022);
    int ns = tl + 2;
    return ns < 0 ? 0 : ns;
}

// exp(A) of a twist by the diagonal (6,6) Pade approximant with scaling and
// squaring (the method of EXPOKIT zgpadm used at expmCuda.cu:1642), real FP64.
// Result in S.E.
static __device__ void wexpm_twist(SolveScratch &S, const double *A, int lane) {
    long long sb = 0;
    if (lane < 4) {
        double s = fabs(A[lane * 4 + 0]);
        s = s + fabs(A[lane * 4 + 1]);
        s = s + fabs(A[lane * 4 + 2]);
        s = s + fabs(A[lane * 4 + 3]);
        sb = __double_as_longlong(s);
    }
    long long hb = 0;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        long long v = __shfl_sync(kFull, sb, r);
        if (v <= kInfBits && v > hb) hb = v;  // NaN row sums never win, as in the oracle
    }
    int ns = expm_squarings_bits(hb);
    double scale = __longlong_as_double((long long)(1023 - ns) << 52);
    double *X = S.M[0], *X2 = S.M[1], *X4 = S.M[2], *X6 = S.M[3], *U0 = S.M[4], *V = S.M[5];
    if (lane < 16) X[lane] = A[lane] * scale;
    __syncwarp();
    wmat4(X, X, X2, lane);
    wmat4(X2, X2, X4, lane);
    wmat4(X4, X2, X6, lane);
    {
        // lanes 0-15: U0 = ((c1 I + c3 X2) + c5 X4) + 0 X6; lanes 16-31: V with c0, c2, c4, c6
        int e = lane & 15;
        bool isV = lane >= 16;
        double ca = isV ? kPade[0] : kPade[1], cb = isV ? kPade[2] : kPade[3];
        double cc = isV ? kPade[4] : kPade[5], cd = isV ? kPade[6] : 0.0;
        double I = (e % 5 == 0) ? 1.0 : 0.0;
        double o = __fma_rn(cd, X6[e], __fma_rn(cc, X4[e], __fma_rn(cb, X2[e], ca * I)));
        (isV ? V : U0)[e] = o;
    }
    __syncwarp();
    double *U = S.M[1];  // X2 no longer needed
    wmat4(X, U0, U, lane);
    double *Nm = S.M[2], *Dm = S.M[3];
    {
        int e = lane & 15;
        if (lane < 16) Nm[e] = V[e] + U[e];
        else Dm[e] = V[e] - U[e];
    }
    __syncwarp();
    // elimination over rows 0..2 (the last rows of D and N are exactly e4)
    int row = lane >> 3, col = lane & 7;  // col 0..3 -> D, 4..7 -> N
    for (int k = 0; k < 3; k++) {
        int p = k;
        long long best = abs_bits(Dm[k * 4 + k]);
        bool best_nan = best > kInfBits;
        for (int i = k + 1; i < 3; i++) {
            long long v = abs_bits(Dm[i * 4 + k]);
            if (!best_nan && v <= kInfBits && v > best) {
                best = v;
                p = i;
            }
        }
        if (best == 0) {  // singular: exp replaced by the identity, as the oracle does
            if (lane < 16) S.E[lane] = (lane % 5 == 0) ? 1.0 : 0.0;
            __syncwarp();
            return;
        }
        if (p != k) {
            double t = 0.0;
            int src = (row == k) ? p : k;
            bool sw = (row == k || row == p);
            if (sw) t = (col < 4) ? Dm[src * 4 + col] : Nm[src * 4 + col - 4];
            __syncwarp();
            if (sw) {
                if (col < 4) Dm[row * 4 + col] = t;
                else Nm[row * 4 + col - 4] = t;
            }
            __syncwarp();
        }
        double inv = 1.0 / Dm[k * 4 + k];
        double nv = 0.0;
        bool act = (row > k && row < 3) && (col >= 4 || col >= k + 1);
        if (act) {
            double f = Dm[row * 4 + k] * inv;
            if (col < 4) nv = __fma_rn(-f, Dm[k * 4 + col], Dm[row * 4 + col]);
            else nv = __fma_rn(-f, Nm[k * 4 + col - 4], Nm[row * 4 + col - 4]);
        }
        __syncwarp();
        if (act) {
            if (col < 4) Dm[row * 4 + col] = nv;
            else Nm[row * 4 + col - 4] = nv;
        }
        if (lane == 0) S.lu_inv[k] = inv;
        __syncwarp();
    }
    // column-oriented back substitution from row 3 up; lanes (row, c) of N
    int c = col - 4;
    for (int k = 3; k >= 1; k--) {
        double nv = 0.0;
        bool act = (col >= 4) && (row < k);
        if (act) nv = __fma_rn(-Dm[row * 4 + k], Nm[k * 4 + c], Nm[row * 4 + c]);
        __syncwarp();
        if (act) Nm[row * 4 + c] = nv;
        __syncwarp();
        if (col >= 4 && row == k - 1) Nm[row * 4 + c] = Nm[row * 4 + c] * S.lu_inv[k - 1];
        __syncwarp();
    }
    for (int k = 0; k < ns; k++) wmat4(Nm, Nm, Nm, lane);
    if (lane < 16) S.E[lane] = Nm[lane];
    __syncwarp();
}

// generateA + expmKernel (warp.cu:910-915, expmCuda.cu:1989-2048): T <- T * exp(A(x)),
// translation scaled by scaleOut, stored as float.  TF is shared memory or global.
static __device__ void wexpm_update(SolveScratch &S, const double *x, float *TF, double scaleOut, int lane) {
    // the twist matrix lives in S.Tinc until exp(A) replaces it
    if (lane == 0) {
        double *A = S.Tinc;
        A[0] = 0.0; A[1] = -x[2]; A[2] = x[1]; A[3] = x[3];
        A[4] = x[2]; A[5] = 0.0; A[6] = -x[0]; A[7] = x[4];
        A[8] = -x[1]; A[9] = x[0]; A[10] = 0.0; A[11] = x[5];
        A[12] = 0.0; A[13] = 0.0; A[14] = 0.0; A[15] = 0.0;
    }
    // the largest |entry| is nonzero iff some x_k is nonzero and not NaN
    bool nonzero = false;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        long long v = abs_bits(x[k]);
        nonzero |= (v != 0 && v <= kInfBits);
    }
    if (lane < 16) S.T[lane] = (double)TF[lane];
    __syncwarp();
    if (nonzero) {
        wexpm_twist(S, S.Tinc, lane);
        if (lane < 16) S.Tinc[lane] = S.E[lane];
        __syncwarp();
        wnormalize(S.Tinc, lane);
        if (lane < 3) S.Tinc[4 * lane + 3] *= scaleOut;
    } else {
        if (lane < 16) S.Tinc[lane] = (lane % 5 == 0) ? 1.0 : 0.0;
    }
    __syncwarp();
    wmat4(S.T, S.Tinc, S.T, lane);
    wnormalize(S.T, lane);
    if (lane < 16) TF[lane] = (float)S.T[lane];
    __syncwarp();
}

// FP64 square-root-free Cholesky A = L D L^T with reciprocal pivots and
// column-oriented substitutions (orc_solve_cholesky).  Lane i < 6 owns row i.
// Returns 0, or -1 when a pivot is not positive.
static __device__ int wcholesky(SolveScratch &S, int lane) {
    const double *A = S.A;
    double *L = S.L, *U = S.U;
    for (int k = lane; k < 36; k += 32) {
        L[k] = 0.0;
        U[k] = 0.0;
    }
    __syncwarp();
    int i = lane;
    for (int j = 0; j < 6; j++) {
        double v = 0.0;
        if (i >= j && i < 6) {
            v = A[i * 6 + j];
            for (int k = 0; k < j; k++) v = __fma_rn(-L[i * 6 + k], U[j * 6 + k], v);
        }
        double dj = __shfl_sync(kFull, v, j);
        if (!(dj > 0.0)) return -1;
        double inv = 1.0 / dj;
        if (lane == 0) S.inv[j] = inv;
        if (i > j && i < 6) {
            U[i * 6 + j] = v;
            L[i * 6 + j] = v * inv;
        }
        __syncwarp();
    }
    double z = (i < 6) ? S.b[i] : 0.0;
    for (int k = 0; k < 6; k++) {
        double zk = __shfl_sync(kFull, z, k);
        if (i > k && i < 6) z = __fma_rn(-L[i * 6 + k], zk, z);
    }
    if (i < 6) z = z * S.inv[i];
    for (int k = 5; k >= 0; k--) {
        double zk = __shfl_sync(kFull, z, k);
        if (i < k) z = __fma_rn(-L[k * 6 + i], zk, z);
    }
    if (i < 6) S.x[i] = z;
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
