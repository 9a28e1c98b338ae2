/* CPU FP64 restatement of the plate / ball vote surrogate: the MLP
 * 28 -> 64 -> 64 -> 64 -> 6 (GELU, tanh form) over the 28 features of the
 * raw input (d, n, flag) -- the input itself, d_i d_j and n_i n_j (i <= j),
 * d_i n_j -- and its backward pass, and the "plain orientation integral" the
 * surrogate is trained on.  Test infrastructure: the GPU training kernels'
 * gradients and the GPU sample generator are checked against these.
 *
 * Parameter layout (float64 here, float32 master copy on the GPU), padded to
 * 8 outputs with zero rows:
 *   W1[64][28] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[8][64] b4[8]
 * Quantised forward (quant != 0): weights and each hidden layer's input
 * rounded to bfloat16 (round to nearest even of the float32 value), each
 * feature formed in float32 (a product rounded once) and taken as
 * bf16(f) + bf16(f - bf16(f)) (the tensor-core form feeds each feature and
 * its residual against the same weight), as the tensor-core inference
 * computes; the backward pass treats the rounding as identity.
 * quant == 1: GELU exact, then rounded to bfloat16 (the GPU's FP32 GELU);
 * quant == 2: the activation as the GPU's training forward pass and its
 * tcgen05 inference compute it: for units j with j % 8 < 6 the GELU in packed
 * BF16 arithmetic (every product or fused multiply-add rounded to bfloat16
 * once, tanh exact then rounded; the hardware's tanh approximation may differ
 * from that in the last bit), for j % 8 >= 6 z * phi(z) with phi a clamped
 * odd polynomial evaluated in float32 (exactly as the GPU does), rounded to
 * bfloat16. */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "tvoracle.h"

#define PI_D 3.14159265358979323846
#define MLP_IN 28
#define MLP_X 8     /* floats per sample row of X (7 used) */
#define MLP_H 64
#define MLP_OUT 8

static double bf16r(double x) {
    float f = (float)x;
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) != 0x7f800000u) {            /* finite: round to nearest even at bit 16 */
        u += 0x7fffu + ((u >> 16) & 1u);
    }
    u &= 0xffff0000u;
    memcpy(&f, &u, 4);
    return (double)f;
}

static const double GELU_K = 0.7978845608028654;   /* sqrt(2 / pi) */
static const double GELU_A = 0.044715;

static double gelu(double z) { return 0.5 * z * (1.0 + tanh(GELU_K * (z + GELU_A * z * z * z))); }
static double gelu_bf16(double z) {
    const double zb = bf16r(z);
    const double ka = bf16r((float)GELU_K * (float)GELU_A), k = bf16r(GELU_K);
    const double u = bf16r(zb * bf16r(bf16r(zb * zb) * ka + k));
    const double t = bf16r(tanh(u));
    const double h = bf16r(zb * 0.5);
    return bf16r(h * t + h);
}
static double gelu_poly(double zd) {
    const float z = (float)zd;
    const float h = fminf(fmaxf(z, -3.0f), 3.0f);
    const float s = h * h;
    float p = fmaf(s, -0.000222746943f, 0.00561482186f);
    p = fmaf(p, s, -0.0578609677f);
    p = fmaf(p, s, 0.394045958f);
    const float phi = fmaf(h, p, 0.5f);
    return bf16r((double)(z * phi));
}
static double act(double z, int quant, int unit) {
    if (quant == 2) return (unit & 7) >= 6 ? gelu_poly(z) : gelu_bf16(z);
    return quant ? bf16r(gelu(z)) : gelu(z);
}
static double gelu_d(double z) {
    const double t = tanh(GELU_K * (z + GELU_A * z * z * z));
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GELU_K * (1.0 + 3.0 * GELU_A * z * z);
}

/* the 28 features of a raw input x = (d0, d1, d2, n0, n1, n2, flag); with
 * quant, x is float32 and each product is rounded to float32 once */
static void features(const double* x, int quant, double* f) {
    const double* d = x;
    const double* nv = x + 3;
    int k = 0;
    for (int i = 0; i < 7; ++i) f[k++] = quant ? (double)(float)x[i] : x[i];
#define OR_PROD(a, b) (quant ? (double)((float)(a) * (float)(b)) : (a) * (b))
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) f[k++] = OR_PROD(d[i], d[j]);
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) f[k++] = OR_PROD(nv[i], nv[j]);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) f[k++] = OR_PROD(d[i], nv[j]);
#undef OR_PROD
}

int or_mlp_param_count(void) { return MLP_H * MLP_IN + MLP_H + 2 * (MLP_H * MLP_H + MLP_H) + MLP_OUT * MLP_H + MLP_OUT; }

/* forward + backward over B samples (X: B x 8, T: B x 8 targets; only the
 * first 6 outputs count): loss = sum over samples and 6 outputs of
 * (y - t)^2 / B, grad (same layout as params) accumulates d loss / d param. */
double or_mlp_loss_grad(const double* P, const double* X, const double* T, int B, int quant, double* grad, double* Y) {
    const double* W1 = P;
    const double* b1 = W1 + MLP_H * MLP_IN;
    const double* W2 = b1 + MLP_H;
    const double* b2 = W2 + MLP_H * MLP_H;
    const double* W3 = b2 + MLP_H;
    const double* b3 = W3 + MLP_H * MLP_H;
    const double* W4 = b3 + MLP_H;
    const double* b4 = W4 + MLP_OUT * MLP_H;
    const int np = or_mlp_param_count();
    double Wq[MLP_H * MLP_IN + 2 * MLP_H * MLP_H + MLP_OUT * MLP_H];
    double* W1q = Wq;
    double* W2q = W1q + MLP_H * MLP_IN;
    double* W3q = W2q + MLP_H * MLP_H;
    double* W4q = W3q + MLP_H * MLP_H;
    for (int i = 0; i < MLP_H * MLP_IN; ++i) W1q[i] = quant ? bf16r(W1[i]) : W1[i];
    for (int i = 0; i < MLP_H * MLP_H; ++i) { W2q[i] = quant ? bf16r(W2[i]) : W2[i]; W3q[i] = quant ? bf16r(W3[i]) : W3[i]; }
    for (int i = 0; i < MLP_OUT * MLP_H; ++i) W4q[i] = quant ? bf16r(W4[i]) : W4[i];
    if (grad) memset(grad, 0, sizeof(double) * (size_t)np);
    double* g1 = grad;
    double* gb1 = g1 ? g1 + MLP_H * MLP_IN : 0;
    double* g2 = g1 ? gb1 + MLP_H : 0;
    double* gb2 = g1 ? g2 + MLP_H * MLP_H : 0;
    double* g3 = g1 ? gb2 + MLP_H : 0;
    double* gb3 = g1 ? g3 + MLP_H * MLP_H : 0;
    double* g4 = g1 ? gb3 + MLP_H : 0;
    double* gb4 = g1 ? g4 + MLP_OUT * MLP_H : 0;
    double loss = 0.0;
    for (int s = 0; s < B; ++s) {
        double h0[MLP_IN], z1[MLP_H], h1[MLP_H], z2[MLP_H], h2[MLP_H], z3[MLP_H], h3[MLP_H];
        /* quantised: each feature as bf16(f) + bf16(f - bf16(f)), the network's first layer taking both */
        double f[MLP_IN];
        features(X + s * MLP_X, quant, f);
        for (int k = 0; k < MLP_IN; ++k) h0[k] = quant ? bf16r(f[k]) + bf16r(f[k] - bf16r(f[k])) : f[k];
        for (int j = 0; j < MLP_H; ++j) {
            double a = b1[j];
            for (int k = 0; k < MLP_IN; ++k) a += W1q[j * MLP_IN + k] * h0[k];
            z1[j] = a;
            h1[j] = act(a, quant, j);
        }
        for (int j = 0; j < MLP_H; ++j) {
            double a = b2[j];
            for (int k = 0; k < MLP_H; ++k) a += W2q[j * MLP_H + k] * h1[k];
            z2[j] = a;
            h2[j] = act(a, quant, j);
        }
        for (int j = 0; j < MLP_H; ++j) {
            double a = b3[j];
            for (int k = 0; k < MLP_H; ++k) a += W3q[j * MLP_H + k] * h2[k];
            z3[j] = a;
            h3[j] = act(a, quant, j);
        }
        double dy[MLP_OUT];
        for (int o = 0; o < MLP_OUT; ++o) {
            double a = b4[o];
            for (int k = 0; k < MLP_H; ++k) a += W4q[o * MLP_H + k] * h3[k];
            const double d = o < 6 ? a - T[s * MLP_OUT + o] : 0.0;
            loss += d * d / B;
            dy[o] = 2.0 * d / B;
            if (Y) Y[s * MLP_OUT + o] = a;
        }
        if (!grad) continue;
        double dh3[MLP_H], dz3[MLP_H], dh2[MLP_H], dz2[MLP_H], dh1[MLP_H], dz1[MLP_H];
        for (int o = 0; o < MLP_OUT; ++o) {
            gb4[o] += dy[o];
            for (int k = 0; k < MLP_H; ++k) g4[o * MLP_H + k] += dy[o] * h3[k];
        }
        for (int k = 0; k < MLP_H; ++k) {
            double a = 0.0;
            for (int o = 0; o < MLP_OUT; ++o) a += W4q[o * MLP_H + k] * dy[o];
            dh3[k] = a;
            dz3[k] = a * gelu_d(z3[k]);
        }
        for (int j = 0; j < MLP_H; ++j) {
            gb3[j] += dz3[j];
            for (int k = 0; k < MLP_H; ++k) g3[j * MLP_H + k] += dz3[j] * h2[k];
        }
        for (int k = 0; k < MLP_H; ++k) {
            double a = 0.0;
            for (int j = 0; j < MLP_H; ++j) a += W3q[j * MLP_H + k] * dz3[j];
            dh2[k] = a;
            dz2[k] = a * gelu_d(z2[k]);
        }
        for (int j = 0; j < MLP_H; ++j) {
            gb2[j] += dz2[j];
            for (int k = 0; k < MLP_H; ++k) g2[j * MLP_H + k] += dz2[j] * h1[k];
        }
        for (int k = 0; k < MLP_H; ++k) {
            double a = 0.0;
            for (int j = 0; j < MLP_H; ++j) a += W2q[j * MLP_H + k] * dz2[j];
            dh1[k] = a;
            dz1[k] = a * gelu_d(z1[k]);
        }
        for (int j = 0; j < MLP_H; ++j) {
            gb1[j] += dz1[j];
            for (int k = 0; k < MLP_IN; ++k) g1[j * MLP_IN + k] += dz1[j] * h0[k];
        }
        (void)dh1; (void)dh2; (void)dh3;
    }
    return loss;
}

/* The plain orientation integral the surrogate learns, for sigma2 = 0,
 * power 1 and o != 0, with the Gaussian c1 = exp(-|o|^2 / sigma^2) taken out:
 * the unit-scale vote's angular part F (xx, xy, xz, yy, yz, zz) at offset
 * direction d for
 *   plate (n = plate normal): (1/S) sum_i (1 - (q_i.d)^2) r_i r_i^T over
 *     S = 64 orientations q_i = cos(i pi/S) u + sin(i pi/S) v on the great
 *     circle normal to n (the reference's basis, tensorvote.h:2467-2469);
 *   ball: the same summand averaged over the sphere with an 8 x 8 rule
 *     (Gauss-Legendre in cos(theta), uniform in phi).
 * r = q - 2 (q.d) d.  The rules are exact for this degree-4 integrand. */
static void stick_unit(const double* q, const double* d, double w, double* F) {
    const double qd = q[0] * d[0] + q[1] * d[1] + q[2] * d[2];
    const double eta = w * (1.0 - qd * qd);
    const double r[3] = {q[0] - 2 * qd * d[0], q[1] - 2 * qd * d[1], q[2] - 2 * qd * d[2]};
    F[0] += eta * r[0] * r[0]; F[1] += eta * r[0] * r[1]; F[2] += eta * r[0] * r[2];
    F[3] += eta * r[1] * r[1]; F[4] += eta * r[1] * r[2]; F[5] += eta * r[2] * r[2];
}

void or_surrogate_target(const double* dir, const double* n, int plate, double* F) {
    double d[3] = {dir[0], dir[1], dir[2]};
    const double dl = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    for (int k = 0; k < 6; ++k) F[k] = 0.0;
    if (dl == 0.0) return;
    d[0] /= dl; d[1] /= dl; d[2] /= dl;
    if (plate) {
        double u[3], v[3];
        if (fabs(n[2]) < 0.999) { u[0] = n[1]; u[1] = -n[0]; u[2] = 0.0; }    /* n x z */
        else { u[0] = 0.0; u[1] = n[2]; u[2] = -n[1]; }                        /* n x x */
        const double ul = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        u[0] /= ul; u[1] /= ul; u[2] /= ul;
        v[0] = n[1] * u[2] - n[2] * u[1]; v[1] = n[2] * u[0] - n[0] * u[2]; v[2] = n[0] * u[1] - n[1] * u[0];
        for (int i = 0; i < 64; ++i) {
            const double a = PI_D * i / 64.0;
            const double q[3] = {cos(a) * u[0] + sin(a) * v[0], cos(a) * u[1] + sin(a) * v[1],
                                 cos(a) * u[2] + sin(a) * v[2]};
            stick_unit(q, d, 1.0 / 64.0, F);
        }
    } else {
        static const double x8[8] = {-0.9602898564975363, -0.7966664774136267, -0.5255324099163290,
                                     -0.1834346424956498, 0.1834346424956498,  0.5255324099163290,
                                     0.7966664774136267,  0.9602898564975363};
        static const double w8[8] = {0.1012285362903763, 0.2223810344533745, 0.3137066458778873,
                                     0.3626837833783620, 0.3626837833783620, 0.3137066458778873,
                                     0.2223810344533745, 0.1012285362903763};
        for (int a = 0; a < 8; ++a)
            for (int b = 0; b < 8; ++b) {
                const double ct = x8[a], st = sqrt(1.0 - ct * ct), ph = 2.0 * PI_D * b / 8.0;
                const double q[3] = {st * cos(ph), st * sin(ph), ct};
                stick_unit(q, d, w8[a] / 2.0 / 8.0, F);
            }
    }
}
