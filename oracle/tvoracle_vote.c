/*
 * tvoracle_vote.c -- CPU restatement of tiralib's tensor-voting functions.
 *
 * TEST INFRASTRUCTURE ONLY (see tvoracle_eig.c for the rules that apply).
 *
 * FP32 routines restate, in the same order of operations:
 *   build_neighbors3d            tira/functions/tensorvote.h:1411
 *   sticknorm3                   tira/functions/tensorvote.h:1163
 *   stickvote3_accumulate_kernel tira/functions/tensorvote.h:1184
 *   cpu::tk_stickvote            tira/functions/tensorvote.h:1513
 *   cpu::tk_plate_numerical      tira/functions/tensorvote.h:1651
 *   cpu::tk_plate_analytic       tira/functions/tensorvote.h:1564
 *   cpu::tk_platevote            tira/functions/tensorvote.h:1714
 *   cpu::tensorvote_tk (3D)      tira/functions/tensorvote.h:1776
 *   cpu::tensorvote3             tira/functions/tensorvote.h:1819
 *   atv (3D) / atv_H / atv_window3 / tensorvote3_atv   tensorvote.h:607,710,1443,1485
 *   2D: Neighbor2D :776, tk_stick_eta_2d :804, tk_stick_norm_2d :843,
 *       tk_stickvote_2d :872, tk_stick_window :939, tk_plate_numerical (2D) :1048,
 *       tk_plate_window :1091, build_neighbors2d :1223, cpu::tensorvote_tk (2D) :1336,
 *       cpu::tensorvote :1381, atv (2D) :225, atv_window :288, cpu::tensorvote_atv :1298
 * Differences from the reference, on purpose:
 *   - cpu::tk_platevote adds the plate vote only to the entries [i][j], i < j, of
 *     the column-major glm::mat3 (tensorvote.h:1750-1753), so the reference CPU
 *     output is not symmetric; the reference GPU kernel (tensorvote.h:2630-2632)
 *     writes both halves.  This restatement writes the symmetric tensor, i.e.
 *     the GPU behaviour, which equals the reference CPU output on the six entries
 *     {0,1,2,4,5,8} that eigen.h reads back.
 * The FP64 routines (or_tensorvote3_f64, ball vote) are the precision oracle
 * and have no counterpart in the reference.
 */
#include "tvoracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_D 3.14159265358979323846
#define TV_EPS 1e-12

typedef struct { float x, y, z; } v3;
static v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static v3 cross(v3 a, v3 b) { return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
static v3 vnorm(v3 a) { float s = 1.0f / sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); return mk(a.x * s, a.y * s, a.z * s); }

/* ---------------- 3D neighbour table ---------------- */
typedef struct { int du, dv, dw; float dx, dy, dz, c1, c2; } nb3;

static nb3* build_nb3(int w, float s1, float s2, int* count) {
    int hw = w / 2, n = 0;
    nb3* t = (nb3*)malloc(sizeof(nb3) * (size_t)w * w * w);
    const float inv1 = s1 > 0 ? 1.0f / (s1 * s1) : 0.0f;
    const float inv2 = s2 > 0 ? 1.0f / (s2 * s2) : 0.0f;
    for (int dw = -hw; dw <= hw; dw++)
        for (int dv = -hw; dv <= hw; dv++)
            for (int du = -hw; du <= hw; du++) {
                nb3 e; e.du = du; e.dv = dv; e.dw = dw;
                const float l2 = (float)(du * du + dv * dv + dw * dw);
                if (l2 == 0.0f) { e.dx = e.dy = e.dz = 0.0f; }
                else { float L = sqrtf(l2); e.dx = (float)du / L; e.dy = (float)dv / L; e.dz = (float)dw / L; }
                e.c1 = s1 == 0.0f ? (l2 > TV_EPS ? 0.0f : 1.0f) : expf(-l2 * inv1);
                e.c2 = s2 == 0.0f ? (l2 > TV_EPS ? 0.0f : 1.0f) : expf(-l2 * inv2);
                t[n++] = e;
            }
    *count = n;
    return t;
}

static double factorial_d(unsigned n) { double f = 1; for (unsigned i = 1; i <= n; i++) f *= i; return f; }

float or_sticknorm3(float s1, float s2, unsigned p) {
    float pi_term = (float)(PI_D * sqrt(PI_D) / 2.0);
    float sig1_3 = s1 * s1 * s1, sig2_3 = s2 * s2 * s2;
    float num1 = (float)(pow(2, 2 * p + 1) * factorial_d(p) * factorial_d(p));
    float num2 = 2.0f;
    float den1 = (float)factorial_d(2 * p + 1);
    float den2 = (float)(2 * p + 1);
    return pi_term * ((sig1_3 * num1 / den1) + (sig2_3 * num2 / den2));
}

static void stick_acc(float* m, v3 d, float c1, float c2, v3 q, unsigned power, float scale) {
    const float qTd = q.x * d.x + q.y * d.y + q.z * d.z;
    const float qTd2 = qTd * qTd;
    float eta;
    if (power == 1) eta = c1 * (1.0f - qTd2) + c2 * qTd2;
    else {
        const float t1 = 1.0f - qTd2, t2 = qTd2;
        float e1 = t1, e2 = t2;
        for (unsigned i = 1; i < power; ++i) { e1 *= t1; e2 *= t2; }
        eta = c1 * e1 + c2 * e2;
    }
    const float rx = q.x - 2.0f * qTd * d.x, ry = q.y - 2.0f * qTd * d.y, rz = q.z - 2.0f * qTd * d.z;
    const float term = scale * eta;
    m[0] += term * rx * rx; m[1] += term * rx * ry; m[2] += term * rx * rz;
    m[3] += term * ry * ry; m[4] += term * ry * rz; m[5] += term * rz * rz;
}

/* plate basis of tk_plate_numerical / tk_plate_analytic (CPU versions) */
static void plate_basis(v3 n, v3* u, v3* v) {
    if (fabsf(n.z) < 0.999f) *u = vnorm(cross(mk(0, 0, 1), n));
    else *u = vnorm(cross(mk(1, 0, 0), n));
    *v = cross(n, *u);
}

static void plate_numerical(float* V, v3 dn, float c1, float c2, unsigned power, v3 n, unsigned samples) {
    for (int i = 0; i < 6; ++i) V[i] = 0.0f;
    const float n2 = n.x * n.x + n.y * n.y + n.z * n.z;
    if (samples == 0 || !((double)n2 > TV_EPS)) return;
    v3 u, v;
    plate_basis(n, &u, &v);
    const float dbeta = (float)PI_D / (float)samples;
    for (unsigned i = 0; i < samples; ++i) {
        const float beta = dbeta * (float)i;
        const float cb = cosf(beta), sb = sinf(beta);
        v3 q = mk(cb * u.x + sb * v.x, cb * u.y + sb * v.y, cb * u.z + sb * v.z);
        stick_acc(V, dn, c1, c2, q, power, 1.0f);
    }
    for (int i = 0; i < 6; ++i) V[i] *= dbeta;
}

/* terminating 2F1(-p, b; c; z), the series of hyp2f1_neg_p_device (tensorvote.h:2364) */
static double hyp2f1_neg(unsigned p, double b, double c, double z) {
    double sum = 1.0, term = 1.0;
    for (unsigned k = 0; k < p; ++k) {
        double kd = (double)k;
        term *= ((-(double)p + kd) * (b + kd)) / ((kd + 1.0) * (c + kd)) * z;
        sum += term;
    }
    return sum;
}
static double beta_fn(double a, double b) { return exp(lgamma(a) + lgamma(b) - lgamma(a + b)); }

/* column-major 3x3 helpers for the analytic plate (glm::mat3 semantics) */
typedef struct { float m[3][3]; } m3;   /* m[col][row] */
static m3 mmul(m3 a, m3 b) {
    m3 r;
    for (int c = 0; c < 3; ++c)
        for (int row = 0; row < 3; ++row)
            r.m[c][row] = a.m[0][row] * b.m[c][0] + a.m[1][row] * b.m[c][1] + a.m[2][row] * b.m[c][2];
    return r;
}
static m3 mtr(m3 a) { m3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[j][i]; return r; }

static void plate_analytic(float* V, v3 dn, float c1, float c2, unsigned power, v3 n, double K0, double K1) {
    v3 u, v;
    plate_basis(n, &u, &v);
    m3 Z = {{{u.x, u.y, u.z}, {v.x, v.y, v.z}, {n.x, n.y, n.z}}};
    m3 Zt = mtr(Z);
    const float dx = Zt.m[0][0] * dn.x + Zt.m[1][0] * dn.y + Zt.m[2][0] * dn.z;
    const float dy = Zt.m[0][1] * dn.x + Zt.m[1][1] * dn.y + Zt.m[2][1] * dn.z;
    const float dz = Zt.m[0][2] * dn.x + Zt.m[1][2] * dn.y + Zt.m[2][2] * dn.z;
    const float alpha = sqrtf(dx * dx + dy * dy);
    const float a2 = alpha * alpha;
    const float phi = atan2f(dy, dx);
    const double a2d = fmin((double)a2, 1.0);
    const double J0 = 0.5 * PI_D * hyp2f1_neg(power, 1.5, 2.0, a2d);
    const double J1 = PI_D * hyp2f1_neg(power, 0.5, 1.0, a2d);
    m3 A, B;
    memset(&A, 0, sizeof A); memset(&B, 0, sizeof B);
    const float t = 1.0f - 2.0f * a2;
    A.m[0][0] = (t * t) * (float)J0;
    A.m[0][2] = -2.0f * alpha * dz * t * (float)J0;
    A.m[2][0] = -2.0f * alpha * dz * t * (float)J0;
    A.m[1][1] = (float)(J1 - J0);
    A.m[2][2] = 4.0f * a2 * (dz * dz) * (float)J0;
    const float a2p = powf(a2, (float)power);
    B.m[0][0] = a2p * (t * t) * (float)K0;
    B.m[0][2] = -2.0f * alpha * a2p * dz * t * (float)K0;
    B.m[2][0] = -2.0f * alpha * a2p * dz * t * (float)K0;
    B.m[1][1] = a2p * (float)(K1 - K0);
    B.m[2][2] = 4.0f * a2p * a2 * (dz * dz) * (float)K0;
    m3 Rz; memset(&Rz, 0, sizeof Rz);
    const float cph = cosf(phi), sph = sinf(phi);
    Rz.m[0][0] = cph; Rz.m[0][1] = -sph; Rz.m[1][0] = sph; Rz.m[1][1] = cph; Rz.m[2][2] = 1.0f;
    m3 Rzr = mtr(Rz);
    m3 ta = mmul(mmul(Rzr, A), Rz), tb = mmul(mmul(Rzr, B), Rz);
    m3 ga = mmul(mmul(Z, ta), Zt), gb = mmul(mmul(Z, tb), Zt);
    float P[3][3];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) P[c][r] = c1 * ga.m[c][r] + c2 * gb.m[c][r];
    /* the upper-triangle entries the reference accumulates (tensorvote.h:1750-1753) */
    V[0] = P[0][0]; V[1] = P[0][1]; V[2] = P[0][2]; V[3] = P[1][1]; V[4] = P[1][2]; V[5] = P[2][2];
}

/* ATV 3D closed-form vote, tensorvote.h:607 (atv_H) and :710 (atv) */
static void atv3(float l0, float l1, float l2, v3 e1, v3 e2, float rx, float ry, float rz, float sigma, float* V) {
    const float dist = sqrtf(rx * rx + ry * ry + rz * rz);
    const float c = sigma == 0.0f ? ((double)dist > TV_EPS ? 0.0f : 1.0f) : expf(-(dist * dist) / (sigma * sigma));
    float dx, dy, dz;
    if (dist == 0.0f) { dx = dy = dz = 0.0f; } else { dx = rx / dist; dy = ry / dist; dz = rz / dist; }
    const float Ra = 1.0f - 2.0f * dx * dx, Rb = 0.0f - 2.0f * dx * dy, Rc = 1.0f - 2.0f * dy * dy;
    const float Rd = 0.0f - 2.0f * dx * dz, Re = 0.0f - 2.0f * dy * dz, Rf = 1.0f - 2.0f * dz * dz;
    float T[3][6];
    T[0][0] = e2.x * e2.x; T[0][1] = e2.x * e2.y; T[0][2] = e2.y * e2.y; T[0][3] = e2.x * e2.z; T[0][4] = e2.y * e2.z; T[0][5] = e2.z * e2.z;
    T[1][0] = e1.x * e1.x; T[1][1] = e1.x * e1.y; T[1][2] = e1.y * e1.y; T[1][3] = e1.x * e1.z; T[1][4] = e1.y * e1.z; T[1][5] = e1.z * e1.z;
    for (int i = 0; i < 6; ++i) T[1][i] += T[0][i];
    T[2][0] = 1; T[2][1] = 0; T[2][2] = 1; T[2][3] = 0; T[2][4] = 0; T[2][5] = 1;
    float vTvT[3][6], TvvT[3][6];
    for (int k = 0; k < 3; ++k) {
        const float* t = T[k];  /* a b c d e f = xx xy yy xz yz zz */
        const float tvx = t[0] * dx + t[1] * dy + t[3] * dz;
        const float tvy = t[1] * dx + t[2] * dy + t[4] * dz;
        const float tvz = t[3] * dx + t[4] * dy + t[5] * dz;
        const float vTv = dx * tvx + dy * tvy + dz * tvz;
        for (int i = 0; i < 6; ++i) vTvT[k][i] = t[i] * vTv;
        TvvT[k][0] = tvx * tvx; TvvT[k][1] = tvx * tvy; TvvT[k][2] = tvy * tvy;
        TvvT[k][3] = tvx * tvz; TvvT[k][4] = tvy * tvz; TvvT[k][5] = tvz * tvz;
    }
    const float s[3] = {l2 - l1, l1 - l0, l0};
    const float inv[3] = {1.0f / 3.0f, 1.0f / 4.0f, 1.0f / 5.0f};
    float H[6];
    for (int i = 0; i < 6; ++i)
        H[i] = s[0] * (T[0][i] - inv[0] * (vTvT[0][i] + 2.0f * TvvT[0][i]))
             + s[1] * (T[1][i] - inv[1] * (vTvT[1][i] + 2.0f * TvvT[1][i]))
             + s[2] * (T[2][i] - inv[2] * (vTvT[2][i] + 2.0f * TvvT[2][i]));
    const float R00 = Ra, R01 = Rb, R02 = Rd, R10 = Rb, R11 = Rc, R12 = Re, R20 = Rd, R21 = Re, R22 = Rf;
    const float H00 = H[0], H01 = H[1], H02 = H[3], H10 = H[1], H11 = H[2], H12 = H[4], H20 = H[3], H21 = H[4], H22 = H[5];
    const float m00 = R00 * H00 + R01 * H10 + R02 * H20, m01 = R00 * H01 + R01 * H11 + R02 * H21, m02 = R00 * H02 + R01 * H12 + R02 * H22;
    const float m10 = R10 * H00 + R11 * H10 + R12 * H20, m11 = R10 * H01 + R11 * H11 + R12 * H21, m12 = R10 * H02 + R11 * H12 + R12 * H22;
    const float m20 = R20 * H00 + R21 * H10 + R22 * H20, m21 = R20 * H01 + R21 * H11 + R22 * H21, m22 = R20 * H02 + R21 * H12 + R22 * H22;
    /* stored as xx, xy, xz, yy, yz, zz */
    V[0] = c * (m00 * R00 + m01 * R10 + m02 * R20);
    V[1] = c * (m00 * R01 + m01 * R11 + m02 * R21);
    V[2] = c * (m00 * R02 + m01 * R12 + m02 * R22);
    V[3] = c * (m10 * R01 + m11 * R11 + m12 * R21);
    V[4] = c * (m10 * R02 + m11 * R12 + m12 * R22);
    V[5] = c * (m20 * R02 + m21 * R12 + m22 * R22);
}

/* Per-voxel voter data exactly as cpu::tensorvote3 prepares it (:1822-1849):
 * lambdas from evals3, spherical eigenvectors, spherical_to_cartesian. */
typedef struct { float* L; v3* large; v3* mid; v3* small; } voters3;

static voters3 prep_voters3(const float* in9, size_t n) {
    voters3 P;
    P.L = (float*)malloc(sizeof(float) * 3 * n);
    float* th = (float*)malloc(sizeof(float) * 6 * n);
    P.large = (v3*)malloc(sizeof(v3) * n);
    P.mid = (v3*)malloc(sizeof(v3) * n);
    P.small = (v3*)malloc(sizeof(v3) * n);
    or_evals3(in9, n, P.L);
    or_evecs3spherical(in9, P.L, n, th);
    for (size_t i = 0; i < n; ++i) {
        float c[3];
        or_spherical_to_cartesian(th[6 * i + 4], th[6 * i + 5], c); P.large[i] = mk(c[0], c[1], c[2]);
        or_spherical_to_cartesian(th[6 * i + 2], th[6 * i + 3], c); P.mid[i] = mk(c[0], c[1], c[2]);
        or_spherical_to_cartesian(th[6 * i + 0], th[6 * i + 1], c); P.small[i] = mk(c[0], c[1], c[2]);
    }
    free(th);
    return P;
}
static void free_voters3(voters3* P) { free(P->L); free(P->large); free(P->mid); free(P->small); }

/* One receiver of cpu::tensorvote_tk (3D): sticknorm * stick + platenorm * plate,
 * as 6 unique entries (xx, xy, xz, yy, yz, zz). */
static void tk3_receiver(const voters3* P, const nb3* NB, int nbc, unsigned power, unsigned s0, unsigned s1, unsigned s2,
                         int x0, int x1, int x2, int stick, int plate, unsigned samples,
                         float sticknorm, float platenorm, double K0, double K1, float* out6) {
    float vote[6] = {0, 0, 0, 0, 0, 0};
    if (stick) {
        float m[6] = {0, 0, 0, 0, 0, 0};
        for (int k = 0; k < nbc; ++k) {
            const nb3* e = &NB[k];
            const int r0 = x0 + e->dw; if ((unsigned)r0 >= s0) continue;
            const int r1 = x1 + e->dv; if ((unsigned)r1 >= s1) continue;
            const int r2 = x2 + e->du; if ((unsigned)r2 >= s2) continue;
            const size_t b = (size_t)r0 * s1 * s2 + (size_t)r1 * s2 + r2;
            const float l1 = P->L[3 * b + 1], l2 = P->L[3 * b + 2];
            const float scale = copysignf(fabsf(l2) - fabsf(l1), l2);
            stick_acc(m, mk(e->dx, e->dy, e->dz), e->c1, e->c2, P->large[b], power, scale);
        }
        for (int i = 0; i < 6; ++i) vote[i] += sticknorm * m[i];
    }
    if (plate) {
        float R[6] = {0, 0, 0, 0, 0, 0};
        for (int k = 0; k < nbc; ++k) {
            const nb3* e = &NB[k];
            const int r0 = x0 + e->dw; if ((unsigned)r0 >= s0) continue;
            const int r1 = x1 + e->dv; if ((unsigned)r1 >= s1) continue;
            const int r2 = x2 + e->du; if ((unsigned)r2 >= s2) continue;
            const size_t b = (size_t)r0 * s1 * s2 + (size_t)r1 * s2 + r2;
            const float l0 = P->L[3 * b + 0], l1 = P->L[3 * b + 1];
            const float scale = copysignf(fabsf(l1) - fabsf(l0), l1);
            float V[6];
            if (samples > 0) plate_numerical(V, mk(e->dx, e->dy, e->dz), e->c1, e->c2, power, P->small[b], samples);
            else plate_analytic(V, mk(e->dx, e->dy, e->dz), e->c1, e->c2, power, P->small[b], K0, K1);
            for (int i = 0; i < 6; ++i) R[i] += scale * V[i];
        }
        for (int i = 0; i < 6; ++i) vote[i] += platenorm * R[i];
    }
    for (int i = 0; i < 6; ++i) out6[i] = vote[i];
}

static void atv3_receiver(const voters3* P, float sigma, unsigned w, unsigned s0, unsigned s1, unsigned s2,
                          int x0, int x1, int x2, float* out6) {
    float R[6] = {0, 0, 0, 0, 0, 0};
    const int hw = (int)w / 2;
    for (int dz = -hw; dz <= hw; ++dz) {
        const int r0 = x0 + dz; if (r0 < 0 || r0 >= (int)s0) continue;
        for (int dy = -hw; dy <= hw; ++dy) {
            const int r1 = x1 + dy; if (r1 < 0 || r1 >= (int)s1) continue;
            for (int dx = -hw; dx <= hw; ++dx) {
                const int r2 = x2 + dx; if (r2 < 0 || r2 >= (int)s2) continue;
                const size_t idx = ((size_t)r0 * s1 + r1) * s2 + r2;
                float V[6];
                atv3(P->L[3 * idx], P->L[3 * idx + 1], P->L[3 * idx + 2], P->mid[idx], P->large[idx],
                     (float)dx, (float)dy, (float)dz, sigma, V);
                for (int i = 0; i < 6; ++i) R[i] += V[i];
            }
        }
    }
    for (int i = 0; i < 6; ++i) out6[i] = R[i];
}

static void put9(float* o9, const float* v6) {
    o9[0] = v6[0]; o9[1] = v6[1]; o9[2] = v6[2];
    o9[3] = v6[1]; o9[4] = v6[3]; o9[5] = v6[4];
    o9[6] = v6[2]; o9[7] = v6[4]; o9[8] = v6[5];
}

/* cpu::tensorvote3 (tensorvote.h:1819): 9 floats per voxel in and out.
 * If `receivers` is non-NULL only those flat voxel indices are computed (into
 * out9 at the same positions); `threads` > 1 spreads receivers over OpenMP
 * threads (a harness loop, the arithmetic per receiver is unchanged). */
void or_tensorvote3_sel(const float* in9, float* out9, unsigned s0, unsigned s1, unsigned s2,
                        float sigma1, float sigma2, unsigned w, unsigned power, int stick, int plate,
                        unsigned samples, int is_atv, const long long* receivers, long long n_recv, int threads) {
    const size_t n = (size_t)s0 * s1 * s2;
    voters3 P = prep_voters3(in9, n);
    int nbc = 0;
    nb3* NB = build_nb3((int)w, sigma1, sigma2, &nbc);
    const float sticknorm = 1.0f / or_sticknorm3(sigma1, sigma2, power);
    const float platenorm = 1.0f / (float)PI_D;
    double K0 = 0, K1 = 0;
    if (samples == 0) { K0 = beta_fn(0.5, (double)power + 1.5); K1 = beta_fn(0.5, (double)power + 0.5); }
    const long long total = receivers ? n_recv : (long long)n;
#ifdef _OPENMP
    if (threads < 1) threads = 1;
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads)
#endif
    for (long long t = 0; t < total; ++t) {
        const long long idx = receivers ? receivers[t] : t;
        const int x0 = (int)(idx / ((long long)s1 * s2));
        const int x1 = (int)((idx / s2) % s1);
        const int x2 = (int)(idx % s2);
        float v6[6];
        if (is_atv) atv3_receiver(&P, sigma1, w, s0, s1, s2, x0, x1, x2, v6);
        else tk3_receiver(&P, NB, nbc, power, s0, s1, s2, x0, x1, x2, stick, plate, samples,
                          sticknorm, platenorm, K0, K1, v6);
        put9(out9 + 9 * idx, v6);
    }
    (void)threads;
    free(NB);
    free_voters3(&P);
}

void or_tensorvote3(const float* in9, float* out9, unsigned s0, unsigned s1, unsigned s2,
                    float sigma1, float sigma2, unsigned w, unsigned power, int stick, int plate,
                    unsigned samples, int is_atv) {
    or_tensorvote3_sel(in9, out9, s0, s1, s2, sigma1, sigma2, w, power, stick, plate, samples, is_atv, NULL, 0, 1);
}

/* ---------------- 2D ---------------- */

typedef struct { int du, dv; float dx, dy, c1, c2, Ra, Rb, Rc, Va, Vb, Vc; } nb2;   /* Neighbor2D, 48 B */

static float stick_norm_2d(float s1, float s2, unsigned p) {
    if (p < 1) p = 1;
    float ratio = 1.0f;
    for (unsigned k = 1; k <= p; ++k) ratio *= (float)(2 * k) / (float)(2 * k - 1);
    return ratio / ((float)PI_D * (s1 * s1 + s2 * s2));
}

static float atten(float dist, float sigma) {
    if (sigma == 0.0f) return ((double)dist > TV_EPS) ? 0.0f : 1.0f;
    return expf(-(dist * dist) / (sigma * sigma));
}

static void stickvote_2d(float rx, float ry, float s1, float s2, unsigned power, float theta, float* Va, float* Vb, float* Vc) {
    const float qx = cosf(theta), qy = sinf(theta);
    const float dist = sqrtf(rx * rx + ry * ry);
    float dx, dy;
    if (dist == 0.0f) { dx = 0.0f; dy = 0.0f; } else { dx = rx / dist; dy = ry / dist; }
    const float qTd = qx * dx + qy * dy;
    unsigned p = power < 1 ? 1 : power;
    const float c1 = atten(dist, s1), c2 = atten(dist, s2);
    const float qTd2 = qTd * qTd, t1 = 1.0f - qTd2, t2 = qTd2;
    float D;
    if (p == 1) D = c1 * t1 + c2 * t2;
    else { float e1 = t1, e2 = t2; for (unsigned i = 1; i < p; ++i) { e1 *= t1; e2 *= t2; } D = c1 * e1 + c2 * e2; }
    const float eta_s = stick_norm_2d(s1, s2, power);
    const float factor = D * eta_s;
    const float Ra = 1 - 2 * dx * dx, Rb = -2 * dx * dy, Rc = 1 - 2 * dy * dy;
    const float Rqx = Ra * qx + Rb * qy, Rqy = Rb * qx + Rc * qy;
    *Va = Rqx * Rqx * factor; *Vb = Rqx * Rqy * factor; *Vc = Rqy * Rqy * factor;
}

static void plate_numerical_2d(float rx, float ry, float s1, float s2, unsigned power, float* oa, float* ob, float* oc, unsigned n) {
    *oa = *ob = *oc = 0;
    if (n == 0) return;
    const float dtheta = (float)(PI_D / (double)(float)n);
    for (unsigned i = 0; i < n; ++i) {
        const float theta = dtheta * (float)i;
        float a, b, c;
        stickvote_2d(rx, ry, s1, s2, power, theta, &a, &b, &c);
        *oa += a; *ob += b; *oc += c;
    }
    const float wb = (float)PI_D / (float)n;
    *oa *= wb; *ob *= wb; *oc *= wb;
}

/* build_neighbors2d, tensorvote.h:1223; table written in the 48-byte layout */
int or_build_neighbors2d(int w, float s1, float s2, unsigned power, unsigned samples, int stick, int plate, void* out) {
    if (w <= 0) return 0;
    const int hw = w / 2;
    nb2* t = (nb2*)out;
    int k = 0;
    const float inv1 = s1 > 0 ? 1.0f / (s1 * s1) : 0.0f, inv2 = s2 > 0 ? 1.0f / (s2 * s2) : 0.0f;
    for (int dv = -hw; dv <= hw; dv++)
        for (int du = -hw; du <= hw; du++) {
            nb2 e; memset(&e, 0, sizeof e);
            e.du = du; e.dv = dv;
            const float l2 = (float)(du * du + dv * dv);
            if (stick) {
                if (l2 == 0.0f) { e.dx = 0; e.dy = 0; }
                else { const float il = 1.0f / sqrtf(l2); e.dx = (float)du * il; e.dy = (float)dv * il; }
                e.c1 = s1 == 0.0f ? (l2 > TV_EPS ? 0.0f : 1.0f) : expf(-l2 * inv1);
                e.c2 = s2 == 0.0f ? (l2 > TV_EPS ? 0.0f : 1.0f) : expf(-l2 * inv2);
                e.Ra = 1.0f - 2.0f * e.dx * e.dx; e.Rb = 0.0f - 2.0f * e.dx * e.dy; e.Rc = 1.0f - 2.0f * e.dy * e.dy;
            }
            if (plate && samples > 0) plate_numerical_2d((float)du, (float)dv, s1, s2, power, &e.Va, &e.Vb, &e.Vc, samples);
            if (t) t[k] = e;
            k++;
        }
    return k;
}

/* cpu::tensorvote_tk (2D, tensorvote.h:1336) given eigenvalues and polar angles */
static void tk2(float* out4, const float* lam, const float* th, float s1, float s2, unsigned power, unsigned w,
                unsigned S0, unsigned S1, int stick, int plate, unsigned samples, const nb2* NB, int nbc) {
    const int use_plate = plate && samples > 0;
    const float eta_s = stick_norm_2d(s1, s2, power < 1 ? 1 : power);
    unsigned p = power < 1 ? 1 : power;
    for (int x0 = 0; x0 < (int)S0; x0++)
        for (int x1 = 0; x1 < (int)S1; x1++) {
            float oa = 0, ob = 0, oc = 0;
            if (stick) {
                float a = 0, b = 0, c = 0;
                for (int k = 0; k < nbc; ++k) {
                    const int r0 = x0 + NB[k].dv; if ((unsigned)r0 >= S0) continue;
                    const int r1 = x1 + NB[k].du; if ((unsigned)r1 >= S1) continue;
                    const int idx = r0 * (int)S1 * 2 + r1 * 2;
                    const float theta = th[idx + 1];
                    const float qx = cosf(theta), qy = sinf(theta);
                    const float qTd = qx * NB[k].dx + qy * NB[k].dy;
                    const float q2 = qTd * qTd, t1 = 1.0f - q2, t2 = q2;
                    float D;
                    if (p == 1) D = NB[k].c1 * t1 + NB[k].c2 * t2;
                    else { float e1 = t1, e2 = t2; for (unsigned i = 1; i < p; ++i) { e1 *= t1; e2 *= t2; } D = NB[k].c1 * e1 + NB[k].c2 * e2; }
                    const float Rqx = NB[k].Ra * qx + NB[k].Rb * qy, Rqy = NB[k].Rb * qx + NB[k].Rc * qy;
                    const float factor = D * eta_s;
                    const float Va = Rqx * Rqx * factor, Vb = Rqx * Rqy * factor, Vc = Rqy * Rqy * factor;
                    const float l0 = lam[idx], l1 = lam[idx + 1];
                    float scale = fabsf(l1) - fabsf(l0);
                    if (l1 < 0.0f) scale = scale * -1.0f;
                    a += scale * Va; b += scale * Vb; c += scale * Vc;
                }
                oa += a; ob += b; oc += c;
            }
            if (plate) {
                float a = 0, b = 0, c = 0;
                if (use_plate)
                    for (int k = 0; k < nbc; ++k) {
                        const int r0 = x0 + NB[k].dv; if ((unsigned)r0 >= S0) continue;
                        const int r1 = x1 + NB[k].du; if ((unsigned)r1 >= S1) continue;
                        const int idx = r0 * (int)S1 * 2 + r1 * 2;
                        const float l0 = lam[idx];
                        if (l0 == 0.0f) continue;
                        a += l0 * NB[k].Va; b += l0 * NB[k].Vb; c += l0 * NB[k].Vc;
                    }
                oa += a; ob += b; oc += c;
            }
            const size_t o = ((size_t)x0 * S1 + x1) * 4;
            out4[o] = oa; out4[o + 1] = ob; out4[o + 2] = ob; out4[o + 3] = oc;
        }
}

/* 2D ATV, tensorvote.h:161 (atv_H), :225 (atv), :288 (atv_window) */
static void atv2(float l0, float l1, float e0x, float e0y, float e1x, float e1y, float rx, float ry, float sigma,
                 float* Va, float* Vb, float* Vc) {
    const float dist = sqrtf(rx * rx + ry * ry);
    const float c = atten(dist, sigma);
    float dx, dy;
    if (dist == 0) { dx = 0; dy = 0; } else { dx = rx / dist; dy = ry / dist; }
    const float Ra = 1 - 2 * dx * dx, Rb = -2 * dx * dy, Rc = 1 - 2 * dy * dy;
    float T1a = e1x * e1x, T1b = e1x * e1y, T1c = e1y * e1y;
    float T0a = e0x * e0x + T1a, T0b = e0x * e0y + T1b, T0c = e0y * e0y + T1c;
    const float v0 = dx * (dx * T0a + dy * T0b) + dy * (dx * T0b + dy * T0c);
    const float v1 = dx * (dx * T1a + dy * T1b) + dy * (dx * T1b + dy * T1c);
    const float t0x = T0a * dx + T0b * dy, t0y = T0b * dx + T0c * dy;
    const float t1x = T1a * dx + T1b * dy, t1y = T1b * dx + T1c * dy;
    const float s1 = l1 - l0, inv3 = 1.0f / 3.0f, inv4 = 1.0f / 4.0f;
    float Ha = s1 * (T1a - inv3 * (T1a * v1 + 2 * (t1x * t1x)));
    float Hb = s1 * (T1b - inv3 * (T1b * v1 + 2 * (t1x * t1y)));
    float Hc = s1 * (T1c - inv3 * (T1c * v1 + 2 * (t1y * t1y)));
    const float s0 = l0;
    Ha += s0 * (T0a - inv4 * (T0a * v0 + 2 * (t0x * t0x)));
    Hb += s0 * (T0b - inv4 * (T0b * v0 + 2 * (t0x * t0y)));
    Hc += s0 * (T0c - inv4 * (T0c * v0 + 2 * (t0y * t0y)));
    const float Ra2 = Ra * Ra, Rb2 = Rb * Rb, Rc2 = Rc * Rc, Rab = Ra * Rb, Rbc = Rb * Rc, Rac = Ra * Rc;
    *Va = c * (Ra2 * Ha + 2 * Rab * Hb + Rb2 * Hc);
    *Vb = c * (Rb2 * Hb + Rab * Ha + Rac * Hb + Rbc * Hc);
    *Vc = c * (Rb2 * Ha + 2 * Rbc * Hb + Rc2 * Hc);
}

static void atv2_field(float* out4, const float* lam, const float* th, float sigma, unsigned w, unsigned S0, unsigned S1) {
    const int hw = (int)w / 2;
    for (int x0 = 0; x0 < (int)S0; x0++)
        for (int x1 = 0; x1 < (int)S1; x1++) {
            float oa = 0, ob = 0, oc = 0;
            for (int v = -hw; v <= hw; v++) {
                const int r0 = x0 + v;
                if (r0 < 0 || r0 >= (int)S0) continue;
                for (int u = -hw; u <= hw; u++) {
                    const int r1 = x1 + u;
                    if (r1 < 0 || r1 >= (int)S1) continue;
                    const int idx = r0 * (int)S1 * 2 + r1 * 2;
                    const float t0 = th[idx], t1 = th[idx + 1];
                    float a, b, c;
                    atv2(lam[idx], lam[idx + 1], cosf(t0), sinf(t0), cosf(t1), sinf(t1), (float)u, (float)v, sigma, &a, &b, &c);
                    oa += a; ob += b; oc += c;
                }
            }
            const size_t o = ((size_t)x0 * S1 + x1) * 4;
            out4[o] = oa; out4[o + 1] = ob; out4[o + 2] = ob; out4[o + 3] = oc;
        }
}

/* cpu::tensorvote (2D, tensorvote.h:1381): [a,b,b,c] per pixel in and out. */
void or_tensorvote2(float* out4, const float* in4, float s1, float s2, int power, unsigned w,
                    unsigned S0, unsigned S1, int stick, int plate, unsigned samples, int is_atv) {
    const size_t n = (size_t)S0 * S1;
    float* lam = (float*)malloc(sizeof(float) * 2 * n);
    float* th = (float*)malloc(sizeof(float) * 2 * n);
    or_evals2(in4, n, lam);
    or_evecs2polar(in4, lam, n, th);
    if (is_atv) atv2_field(out4, lam, th, s1, w, S0, S1);
    else {
        const int use_plate = plate && samples > 0;
        nb2* NB = NULL; int nbc = 0;
        if (stick || use_plate) {
            NB = (nb2*)malloc(sizeof(nb2) * (size_t)w * w);
            nbc = or_build_neighbors2d((int)w, s1, s2, (unsigned)power, samples, stick, use_plate, NB);
        }
        tk2(out4, lam, th, s1, s2, (unsigned)power, w, S0, S1, stick, plate, samples, NB, nbc);
        free(NB);
    }
    free(lam); free(th);
}

/* 2D TK with a caller-supplied Neighbor2D table (tensorvote_prebuilt, :2237) */
void or_tensorvote2_prebuilt(float* out4, const float* in4, const void* nb, int nbc, float s1, float s2, int power,
                             unsigned w, unsigned S0, unsigned S1, int stick, int plate, unsigned samples) {
    const size_t n = (size_t)S0 * S1;
    float* lam = (float*)malloc(sizeof(float) * 2 * n);
    float* th = (float*)malloc(sizeof(float) * 2 * n);
    or_evals2(in4, n, lam);
    or_evecs2polar(in4, lam, n, th);
    tk2(out4, lam, th, s1, s2, (unsigned)power, w, S0, S1, stick, plate, samples, (const nb2*)nb, nbc);
    free(lam); free(th);
}

/* ---------------- FP64 precision oracle for 3D TK (no reference counterpart) ----
 * Voters from the FP64 Jacobi eigensolver of each (float) input tensor; stick
 * and plate in double; the plate is the exact orientation integral, i.e. the
 * limit the reference's S-sample rule reaches for S >= power + 2, evaluated
 * with the (power + 2)-point rule (exact for that integrand); the ball vote
 * is the mean of unit stick votes over the sphere (Gauss-Legendre in cos(theta)
 * x uniform in phi, exact for the degree-(2 power + 2) integrand), scaled by
 * lambda0.  Output 6 unique entries per voxel (xx, xy, xz, yy, yz, zz). */
typedef struct { double x, y, z; } d3;

static void stick_acc_d(double* m, d3 d, double c1, double c2, d3 q, unsigned power, double scale) {
    const double t = q.x * d.x + q.y * d.y + q.z * d.z, t2 = t * t;
    double e1 = 1.0 - t2, e2 = t2, a = e1, b = e2;
    for (unsigned i = 1; i < power; ++i) { a *= e1; b *= e2; }
    const double eta = c1 * a + c2 * b;
    const double rx = q.x - 2 * t * d.x, ry = q.y - 2 * t * d.y, rz = q.z - 2 * t * d.z;
    const double term = scale * eta;
    m[0] += term * rx * rx; m[1] += term * rx * ry; m[2] += term * rx * rz;
    m[3] += term * ry * ry; m[4] += term * ry * rz; m[5] += term * rz * rz;
}

static void gauss_legendre(int n, double* x, double* w) {
    for (int i = 0; i < n; ++i) {
        double z = cos(PI_D * (i + 0.75) / (n + 0.5)), pp = 0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1, p2 = 0;
            for (int j = 0; j < n; ++j) { double p3 = p2; p2 = p1; p1 = ((2 * j + 1) * z * p2 - j * p3) / (j + 1); }
            pp = n * (z * p1 - p2) / (z * z - 1);
            double z1 = z; z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-15) break;
        }
        x[i] = z; w[i] = 2 / ((1 - z * z) * pp * pp);
    }
}

void or_tensorvote3_f64(const float* in9, double* out6, unsigned s0, unsigned s1, unsigned s2,
                        double sigma1, double sigma2, unsigned w, unsigned power, int stick, int plate, int ball,
                        const long long* receivers, long long n_recv, int threads) {
    const size_t n = (size_t)s0 * s1 * s2;
    double* L = (double*)malloc(sizeof(double) * 3 * n);
    d3* E2 = (d3*)malloc(sizeof(d3) * n);
    d3* E0 = (d3*)malloc(sizeof(d3) * n);
    for (size_t i = 0; i < n; ++i) {
        const float* m = in9 + 9 * i;
        double s6[6] = {m[0], m[1], m[2], m[4], m[5], m[8]}, ev[9];
        or_eig3_f64(s6, L + 3 * i, ev);
        E0[i].x = ev[0]; E0[i].y = ev[1]; E0[i].z = ev[2];
        E2[i].x = ev[6]; E2[i].y = ev[7]; E2[i].z = ev[8];
    }
    /* sticknorm3 in double */
    const double pt = PI_D * sqrt(PI_D) / 2.0;
    const double sn = pt * (sigma1 * sigma1 * sigma1 * pow(2, 2 * power + 1) * factorial_d(power) * factorial_d(power) / factorial_d(2 * power + 1)
                          + sigma2 * sigma2 * sigma2 * 2.0 / (2 * power + 1));
    const int M = (int)power + 2;           /* exact plate rule */
    const int NG = (int)power + 3, NP = 2 * (int)power + 5;
    double gx[64], gw[64];
    gauss_legendre(NG, gx, gw);
    const int hw = (int)w / 2;
    const long long total = receivers ? n_recv : (long long)n;
#ifdef _OPENMP
    if (threads < 1) threads = 1;
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
#endif
    for (long long t = 0; t < total; ++t) {
        const long long idx = receivers ? receivers[t] : t;
        const int x0 = (int)(idx / ((long long)s1 * s2)), x1 = (int)((idx / s2) % s1), x2 = (int)(idx % s2);
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int dw = -hw; dw <= hw; ++dw) {
            const int r0 = x0 + dw; if (r0 < 0 || r0 >= (int)s0) continue;
            for (int dv = -hw; dv <= hw; ++dv) {
                const int r1 = x1 + dv; if (r1 < 0 || r1 >= (int)s1) continue;
                for (int du = -hw; du <= hw; ++du) {
                    const int r2 = x2 + du; if (r2 < 0 || r2 >= (int)s2) continue;
                    const size_t b = ((size_t)r0 * s1 + r1) * s2 + r2;
                    const double l2 = (double)(du * du + dv * dv + dw * dw);
                    d3 d = {0, 0, 0};
                    if (l2 > 0) { double il = 1.0 / sqrt(l2); d.x = du * il; d.y = dv * il; d.z = dw * il; }
                    const double c1 = sigma1 == 0 ? (l2 > 0 ? 0 : 1) : exp(-l2 / (sigma1 * sigma1));
                    const double c2 = sigma2 == 0 ? (l2 > 0 ? 0 : 1) : exp(-l2 / (sigma2 * sigma2));
                    const double* lam = L + 3 * b;
                    if (stick) {
                        double m[6] = {0, 0, 0, 0, 0, 0};
                        const double sc = copysign(fabs(lam[2]) - fabs(lam[1]), lam[2]);
                        stick_acc_d(m, d, c1, c2, E2[b], power, sc);
                        for (int i = 0; i < 6; ++i) acc[i] += m[i] / sn;
                    }
                    if (plate) {
                        d3 nn = E0[b], u, v;
                        /* any orthonormal basis of the plane normal to nn */
                        if (fabs(nn.z) < 0.9) { u.x = -nn.y; u.y = nn.x; u.z = 0; }
                        else { u.x = 0; u.y = -nn.z; u.z = nn.y; }
                        double un = sqrt(u.x * u.x + u.y * u.y + u.z * u.z);
                        u.x /= un; u.y /= un; u.z /= un;
                        v.x = nn.y * u.z - nn.z * u.y; v.y = nn.z * u.x - nn.x * u.z; v.z = nn.x * u.y - nn.y * u.x;
                        double m[6] = {0, 0, 0, 0, 0, 0};
                        for (int i = 0; i < M; ++i) {
                            const double be = PI_D * i / M;
                            d3 q = {cos(be) * u.x + sin(be) * v.x, cos(be) * u.y + sin(be) * v.y, cos(be) * u.z + sin(be) * v.z};
                            stick_acc_d(m, d, c1, c2, q, power, 1.0);
                        }
                        const double sc = copysign(fabs(lam[1]) - fabs(lam[0]), lam[1]);
                        for (int i = 0; i < 6; ++i) acc[i] += sc * m[i] * (PI_D / M) / PI_D;
                    }
                    if (ball) {
                        double m[6] = {0, 0, 0, 0, 0, 0};
                        for (int i = 0; i < NG; ++i)
                            for (int j = 0; j < NP; ++j) {
                                const double ct = gx[i], st = sqrt(1 - ct * ct), ph = 2 * PI_D * j / NP;
                                d3 q = {st * cos(ph), st * sin(ph), ct};
                                stick_acc_d(m, d, c1, c2, q, power, gw[i] * (2 * PI_D / NP));
                            }
                        for (int i = 0; i < 6; ++i) acc[i] += lam[0] * m[i] / (4 * PI_D);
                    }
                }
            }
        }
        for (int i = 0; i < 6; ++i) out6[6 * idx + i] = acc[i];
    }
    (void)threads;
    free(L); free(E2); free(E0);
}
