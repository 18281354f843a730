/*
 * initnet_oracle.c -- CPU oracle of the learned initialisation network
 * (include/recon_initnet.h).  TEST INFRASTRUCTURE ONLY: the checker of the GPU
 * forward and backward kernels.  There is no counterpart in the reference.
 *
 * Everything is computed in FP64.  With exact = 0 the values the GPU stores in
 * BF16 (convolution weights and activations) are rounded to BF16 (round to
 * nearest even) at the same points, and so are the pre-activation gradients
 * where the backward pass multiplies them on the tensor cores (the weight and
 * input gradients; the bias gradient sums them unrounded), so GPU and oracle
 * agree to FP32 accumulation-order rounding; with exact = 1 nothing is rounded
 * and the gradient is the exact derivative of the FP64 loss (for finite
 * differences).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NL 6
static const int CIN[NL] = {4, 16, 32, 64, 64, 128};
static const int COUT[NL] = {16, 32, 64, 64, 128, 128};
static const int HT[NL + 1] = {60, 30, 15, 8, 4, 2, 1};
static const int WD[NL + 1] = {80, 40, 20, 10, 5, 3, 2};
#define FEAT 128
#define NOUT 6

static int kpad(int cin) { return (9 * cin + 15) / 16 * 16; }

typedef struct {
    int64_t w[NL], b[NL], wfc, bfc, scale, total;
} net_off;

static net_off offs(void) {
    net_off o;
    int64_t p = 0;
    for (int l = 0; l < NL; l++) {
        o.w[l] = p;
        p += (int64_t)COUT[l] * kpad(CIN[l]);
        o.b[l] = p;
        p += COUT[l];
    }
    o.wfc = p;
    p += NOUT * FEAT;
    o.bfc = p;
    p += NOUT;
    o.scale = p;
    p += NOUT;
    o.total = p;
    return o;
}

int64_t orc_net_param_count(void) { return offs().total; }

/* float -> bf16 bits, round to nearest even (NaN kept quiet) */
static uint16_t f2bf(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40);
    uint32_t r = u + 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(r >> 16);
}
static float bf2f(uint16_t b) {
    uint32_t u = (uint32_t)b << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static double rbf(double v, int exact) { return exact ? v : (double)bf2f(f2bf((float)v)); }

/* coarse image, the GPU's k_coarse */
void orc_net_coarse(const uint8_t *gray, const uint16_t *depth, int n, int W, int H, uint16_t *out) {
    int bx = W / 80, by = H / 60;
    for (int f = 0; f < n; f++)
        for (int oy = 0; oy < 60; oy++)
            for (int ox = 0; ox < 80; ox++) {
                const uint8_t *g = gray + (int64_t)f * W * H;
                const uint16_t *dp = depth + (int64_t)f * W * H;
                int gs = 0, cnt = 0;
                long long ds = 0;
                for (int y = 0; y < by; y++)
                    for (int x = 0; x < bx; x++) {
                        int64_t o = (int64_t)(oy * by + y) * W + ox * bx + x;
                        gs += g[o];
                        if (dp[o]) {
                            ds += dp[o];
                            cnt++;
                        }
                    }
                float gv = (float)gs / (255.0f * (float)(bx * by));
                float dv = cnt ? ((float)ds / (float)cnt) / 4000.0f : 0.0f;
                int64_t i = ((int64_t)f * 60 + oy) * 80 + ox;
                out[2 * i] = f2bf(gv);
                out[2 * i + 1] = f2bf(dv);
            }
}

/* forward pass; acts[l] (n*HT*WD*COUT doubles) keep the post-ReLU activations,
 * feat the pooled features, y the outputs */
static void forward(const float *params, const uint16_t *in, int n, int exact, double **acts, double *feat,
                    double *y) {
    net_off o = offs();
    int64_t inN = (int64_t)n * 60 * 80 * 4;
    double *x = malloc(sizeof(double) * inN);
    for (int64_t i = 0; i < inN; i++) x[i] = bf2f(in[i]);
    const double *cur = x;
    for (int l = 0; l < NL; l++) {
        int Cin = CIN[l], Cout = COUT[l], Kp = kpad(Cin), H = HT[l], W = WD[l], Ho = HT[l + 1], Wo = WD[l + 1];
        const float *w = params + o.w[l], *b = params + o.b[l];
        double *out = acts[l];
        for (int nn = 0; nn < n; nn++)
            for (int oy = 0; oy < Ho; oy++)
                for (int ox = 0; ox < Wo; ox++)
                    for (int co = 0; co < Cout; co++) {
                        double acc = 0.0;
                        for (int k = 0; k < 9 * Cin; k++) {
                            int tap = k / Cin, c = k % Cin, ky = tap / 3, kx = tap % 3;
                            int iy = 2 * oy - 1 + ky, ix = 2 * ox - 1 + kx;
                            if (iy < 0 || iy >= H || ix < 0 || ix >= W) continue;
                            acc += cur[(((int64_t)nn * H + iy) * W + ix) * Cin + c] * rbf(w[co * Kp + k], exact);
                        }
                        double v = (exact ? acc : (double)(float)acc) + (double)b[co];
                        if (!exact) v = (double)(float)v;
                        v = v > 0.0 ? v : 0.0;
                        out[(((int64_t)nn * Ho + oy) * Wo + ox) * Cout + co] = rbf(v, exact);
                    }
        cur = out;
    }
    int P = HT[NL] * WD[NL];
    for (int nn = 0; nn < n; nn++) {
        for (int c = 0; c < FEAT; c++) {
            double s = 0.0;
            for (int p = 0; p < P; p++) s += cur[((int64_t)nn * P + p) * FEAT + c];
            feat[nn * FEAT + c] = exact ? s / P : (double)((float)s / (float)P);
        }
        for (int j = 0; j < NOUT; j++) {
            double v = params[o.bfc + j];
            for (int c = 0; c < FEAT; c++) v += (double)params[o.wfc + j * FEAT + c] * feat[nn * FEAT + c];
            y[nn * NOUT + j] = exact ? v : (double)(float)v;
        }
    }
    free(x);
}

static double **alloc_acts(int n) {
    double **a = malloc(sizeof(double *) * NL);
    for (int l = 0; l < NL; l++) a[l] = calloc((size_t)n * HT[l + 1] * WD[l + 1] * COUT[l], sizeof(double));
    return a;
}
static void free_acts(double **a) {
    for (int l = 0; l < NL; l++) free(a[l]);
    free(a);
}

void orc_net_forward(const float *params, const uint16_t *in, int n, int exact, double *out) {
    double **acts = alloc_acts(n);
    double *feat = malloc(sizeof(double) * n * FEAT);
    forward(params, in, n, exact, acts, feat, out);
    free(feat);
    free_acts(acts);
}

/* loss = mean over samples and outputs of (y - t)^2; the gradient of every
 * parameter into grad (the output scale entries: 0). */
double orc_net_loss_grad(const float *params, const uint16_t *in, const float *target, int n, int exact,
                         double *grad) {
    net_off o = offs();
    double **acts = alloc_acts(n);
    double *feat = malloc(sizeof(double) * n * FEAT);
    double *y = malloc(sizeof(double) * n * NOUT);
    forward(params, in, n, exact, acts, feat, y);
    memset(grad, 0, sizeof(double) * o.total);
    double loss = 0.0;
    double *dy = malloc(sizeof(double) * n * NOUT);
    for (int i = 0; i < n * NOUT; i++) {
        double d = y[i] - (double)target[i];
        loss += d * d;
        dy[i] = 2.0 * d / (double)(NOUT * n);
    }
    loss /= (double)(NOUT * n);
    for (int j = 0; j < NOUT; j++)
        for (int nn = 0; nn < n; nn++) {
            grad[o.bfc + j] += dy[nn * NOUT + j];
            for (int c = 0; c < FEAT; c++) grad[o.wfc + j * FEAT + c] += dy[nn * NOUT + j] * feat[nn * FEAT + c];
        }
    int P = HT[NL] * WD[NL];
    /* dz: gradient at the pre-activation of the current layer */
    double *dz = calloc((size_t)n * P * FEAT, sizeof(double));
    for (int nn = 0; nn < n; nn++)
        for (int c = 0; c < FEAT; c++) {
            double df = 0.0;
            for (int j = 0; j < NOUT; j++) df += (double)params[o.wfc + j * FEAT + c] * dy[nn * NOUT + j];
            df /= (double)P;
            for (int p = 0; p < P; p++) {
                int64_t idx = ((int64_t)nn * P + p) * FEAT + c;
                dz[idx] = acts[NL - 1][idx] > 0.0 ? df : 0.0;
            }
        }
    int64_t inN = (int64_t)n * 60 * 80 * 4;
    double *x = malloc(sizeof(double) * inN);
    for (int64_t i = 0; i < inN; i++) x[i] = bf2f(in[i]);
    for (int l = NL - 1; l >= 0; l--) {
        int Cin = CIN[l], Cout = COUT[l], Kp = kpad(Cin), H = HT[l], W = WD[l], Ho = HT[l + 1], Wo = WD[l + 1];
        const double *lin = l ? acts[l - 1] : x;
        const float *w = params + o.w[l];
        for (int nn = 0; nn < n; nn++)
            for (int oy = 0; oy < Ho; oy++)
                for (int ox = 0; ox < Wo; ox++)
                    for (int co = 0; co < Cout; co++) {
                        double d = dz[(((int64_t)nn * Ho + oy) * Wo + ox) * Cout + co];
                        if (d == 0.0) continue;
                        grad[o.b[l] + co] += d;
                        double dr = rbf(d, exact);
                        for (int k = 0; k < 9 * Cin; k++) {
                            int tap = k / Cin, c = k % Cin, ky = tap / 3, kx = tap % 3;
                            int iy = 2 * oy - 1 + ky, ix = 2 * ox - 1 + kx;
                            if (iy < 0 || iy >= H || ix < 0 || ix >= W) continue;
                            grad[o.w[l] + co * Kp + k] += dr * lin[(((int64_t)nn * H + iy) * W + ix) * Cin + c];
                        }
                    }
        if (l == 0) break;
        double *dprev = calloc((size_t)n * H * W * Cin, sizeof(double));
        for (int nn = 0; nn < n; nn++)
            for (int oy = 0; oy < Ho; oy++)
                for (int ox = 0; ox < Wo; ox++)
                    for (int co = 0; co < Cout; co++) {
                        double d = dz[(((int64_t)nn * Ho + oy) * Wo + ox) * Cout + co];
                        if (d == 0.0) continue;
                        d = rbf(d, exact);
                        for (int k = 0; k < 9 * Cin; k++) {
                            int tap = k / Cin, c = k % Cin, ky = tap / 3, kx = tap % 3;
                            int iy = 2 * oy - 1 + ky, ix = 2 * ox - 1 + kx;
                            if (iy < 0 || iy >= H || ix < 0 || ix >= W) continue;
                            dprev[(((int64_t)nn * H + iy) * W + ix) * Cin + c] += rbf(w[co * Kp + k], exact) * d;
                        }
                    }
        for (int64_t i = 0; i < (int64_t)n * H * W * Cin; i++) dprev[i] = acts[l - 1][i] > 0.0 ? dprev[i] : 0.0;
        free(dz);
        dz = dprev;
    }
    free(dz);
    free(x);
    free(dy);
    free(y);
    free(feat);
    free_acts(acts);
    return loss;
}
