/*
 * tvoracle_eig.c -- CPU restatement of tiralib's symmetric eigensolvers.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this file:
 * it is loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg, and only as the checker / the timed CPU reference.
 *
 * Parity: the float routines restate tira/functions/eigen.h operation for
 * operation (FP32, same branches, same thresholds) and are pinned against the
 * reference's own code compiled in oracle/_ref and against the committed
 * fixtures in tests/golden/.  The double routines (Jacobi) are the FP64
 * precision oracle, which has no counterpart in the reference.
 */
#include "tvoracle.h"
#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EIG_EPS 1e-6f          /* tira::constant::TIRA_EIGEN_EPSILON<float>, eigen.h:13 */
#define PI_D 3.14159265358979323846

static void swapf(float* a, float* b) { float t = *a; *a = *b; *b = t; }
static float sgn_plus(float a) { return a < 0.0f ? -1.0f : 1.0f; }          /* eigen.h:29 */
static float dot3f(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void cross3f(const float* a, const float* b, float* r) {             /* eigen.h:68 */
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}
static void normalize3f(float* v) {                                          /* eigen.h:56 */
    float n = sqrtf(dot3f(v, v));
    if (n > EIG_EPS) {
        float inv = 1.0f / n;
        v[0] *= inv; v[1] *= inv; v[2] *= inv;
    }
}

/* ---------------- 2x2 ---------------- */

/* quad_root, eigen.h:90 */
static void quad_root(float b, float c, float* r0, float* r1) {
    float disc = (b * b) - 4.0f * c;
    if (disc < 0.0f) disc = 0.0f;
    float q = -0.5f * (b + sgn_plus(b) * sqrtf(disc));
    *r1 = q;
    if (q == 0.0f) *r0 = 0.0f; else *r0 = c / q;
    if (*r0 > *r1) swapf(r0, r1);
}

/* eval2_symmetric, eigen.h:119 */
void or_eval2(float a, float b, float c, float* e0, float* e1) {
    float tr = a + c;
    float det = a * c - b * b;
    quad_root(-tr, det, e0, e1);
    const float scale = (fabsf(*e1) > 1.0f) ? fabsf(*e1) : 1.0f;
    const float tol = EIG_EPS * scale;
    if (*e0 < 0.0f && *e0 > -tol) *e0 = 0.0f;
    if (*e1 < 0.0f && *e1 > -tol) *e1 = 0.0f;
}

/* evec2polar_symmetric, eigen.h:150 */
void or_evec2polar(float a, float b, float c, const float* lambdas, float* theta0, float* theta1) {
    const float pi = (float)PI_D;
    float l0 = lambdas[0];
    float vx0 = -b, vy0 = a - l0;
    float vx1 = c - l0, vy1 = -b;
    const float n0 = vx0 * vx0 + vy0 * vy0;
    const float n1 = vx1 * vx1 + vy1 * vy1;
    float vx = (n0 >= n1) ? vx0 : vx1;
    float vy = (n0 >= n1) ? vy0 : vy1;
    float n = sqrtf(vx * vx + vy * vy);
    if (n < EIG_EPS) { vx = 1.0f; vy = 0.0f; n = 1.0f; }
    else { const float inv = 1.0f / n; vx *= inv; vy *= inv; }
    if (fabsf(vx) >= fabsf(vy)) { if (vx < 0.0f) { vx = -vx; vy = -vy; } }
    else { if (vy < 0.0f) { vx = -vx; vy = -vy; } }
    *theta0 = atan2f(vy, vx);
    float ux = -vy, uy = vx;
    if (fabsf(ux) >= fabsf(uy)) { if (ux < 0.0f) { ux = -ux; uy = -uy; } }
    else { if (uy < 0.0f) { ux = -ux; uy = -uy; } }
    *theta1 = atan2f(uy, ux);
    if (*theta0 <= -pi) *theta0 += 2.0f * pi;
    if (*theta1 <= -pi) *theta1 += 2.0f * pi;
    if (*theta0 > pi) *theta0 -= 2.0f * pi;
    if (*theta1 > pi) *theta1 -= 2.0f * pi;
}

/* cpu::evals2_symmetric / evecs2polar_symmetric, eigen.h:573,598 (input [a,b,b,c]) */
void or_evals2(const float* mats4, size_t n, float* evals2) {
    for (size_t i = 0; i < n; ++i)
        or_eval2(mats4[4 * i + 0], mats4[4 * i + 1], mats4[4 * i + 3], &evals2[2 * i], &evals2[2 * i + 1]);
}
void or_evecs2polar(const float* mats4, const float* evals2, size_t n, float* thetas2) {
    for (size_t i = 0; i < n; ++i)
        or_evec2polar(mats4[4 * i + 0], mats4[4 * i + 1], mats4[4 * i + 3], &evals2[2 * i],
                      &thetas2[2 * i], &thetas2[2 * i + 1]);
}

/* ---------------- 3x3 ---------------- */

/* determinant3, eigen.h:46: | a b d ; b c e ; d e f | */
static float det3f(float a, float b, float c, float d, float e, float f) {
    return a * (c * f - e * e) - b * (b * f - e * d) + d * (b * e - c * d);
}

/* eval3_symmetric (Smith's trigonometric method), eigen.h:392 */
void or_eval3(float a, float b, float c, float d, float e, float f, float* e0, float* e1, float* e2) {
    const float p1 = b * b + d * d + e * e;
    if (p1 < EIG_EPS) {
        *e0 = a; *e1 = c; *e2 = f;
        if (*e0 > *e1) swapf(e0, e1);
        if (*e1 > *e2) swapf(e1, e2);
        if (*e0 > *e1) swapf(e0, e1);
        return;
    }
    const float tr = a + c + f;
    const float q = tr / 3.0f;
    const float aq = a - q, cq = c - q, fq = f - q;
    const float p2 = aq * aq + cq * cq + fq * fq + 2.0f * p1;
    float p = sqrtf(p2 / 6.0f);
    const float p_inv = 1.0f / p;
    const float Ba = p_inv * aq, Bb = p_inv * b, Bc = p_inv * cq;
    const float Bd = p_inv * d, Be = p_inv * e, Bf = p_inv * fq;
    const float det_B = Ba * (Bc * Bf - Be * Be) - Bb * (Bb * Bf - Bd * Be) + Bd * (Bb * Be - Bd * Bc);
    float r = det_B / 2.0f;
    float phi;
    const float pif = (float)PI_D;
    if (r < -1.0f) phi = pif / 3.0f;
    else if (r >= 1.0f) phi = 0.0f;
    else phi = acosf(r) / 3.0f;
    *e2 = q + 2.0f * p * cosf(phi);
    *e0 = q + 2.0f * p * cosf(phi + (2.0f * pif / 3.0f));
    *e1 = tr - *e0 - *e2;
}

/* evec3_symmetric_0: eigenvector from the largest cofactor row of A - l I, eigen.h:248 */
static void evec3_0(float a, float b, float c, float d, float e, float f, float ev, float* out) {
    float m00 = a - ev, m01 = b, m02 = d;
    float m10 = b, m11 = c - ev, m12 = e;
    float m20 = d, m21 = e, m22 = f - ev;
    float c00 = m11 * m22 - m12 * m21, c01 = m12 * m20 - m10 * m22, c02 = m10 * m21 - m11 * m20;
    float c10 = m02 * m21 - m01 * m22, c11 = m00 * m22 - m02 * m20, c12 = m01 * m20 - m00 * m21;
    float c20 = m01 * m12 - m02 * m11, c21 = m02 * m10 - m00 * m12, c22 = m00 * m11 - m01 * m10;
    float r0 = c00 * c00 + c01 * c01 + c02 * c02;
    float r1 = c10 * c10 + c11 * c11 + c12 * c12;
    float r2 = c20 * c20 + c21 * c21 + c22 * c22;
    if (r0 >= r1 && r0 >= r2) { out[0] = c00; out[1] = c01; out[2] = c02; }
    else if (r1 >= r0 && r1 >= r2) { out[0] = c10; out[1] = c11; out[2] = c12; }
    else { out[0] = c20; out[1] = c21; out[2] = c22; }
    normalize3f(out);
}

/* ComputeOrthogonalComplement, eigen.h:218 */
static void ortho_complement(const float* ev, float* U, float* V) {
    const float ax = fabsf(ev[0]), ay = fabsf(ev[1]), az = fabsf(ev[2]);
    float t[3];
    if (ay - ax > EIG_EPS) {
        if (az - ax > EIG_EPS) { t[0] = 1; t[1] = 0; t[2] = 0; }
        else { t[0] = 0; t[1] = 0; t[2] = 1; }
    } else {
        if (az - ay > EIG_EPS) { t[0] = 0; t[1] = 1; t[2] = 0; }
        else { t[0] = 0; t[1] = 0; t[2] = 1; }
    }
    cross3f(ev, t, U);
    normalize3f(U);
    cross3f(ev, U, V);
}

/* evec3_symmetric_1: second eigenvector from the 2x2 problem on {U,V}, eigen.h:291 */
static void evec3_1(float a, float b, float c, float d, float e, float f, float ev1, const float* evec0, float* out) {
    float U[3], V[3];
    ortho_complement(evec0, U, V);
    const float AU[3] = {a * U[0] + b * U[1] + d * U[2], b * U[0] + c * U[1] + e * U[2], d * U[0] + e * U[1] + f * U[2]};
    const float AV[3] = {a * V[0] + b * V[1] + d * V[2], b * V[0] + c * V[1] + e * V[2], d * V[0] + e * V[1] + f * V[2]};
    float m00 = dot3f(U, AU) - ev1;
    float m01 = dot3f(U, AV);
    float m11 = dot3f(V, AV) - ev1;
    float am00 = fabsf(m00), am01 = fabsf(m01), am11 = fabsf(m11);
    if (am00 >= am11) {
        if (am00 > EIG_EPS || am01 > EIG_EPS) {
            if (am00 >= am01) { m01 /= m00; float il = 1.0f / sqrtf(1.0f + m01 * m01); m00 = il; m01 *= il; }
            else { m00 /= m01; float il = 1.0f / sqrtf(1.0f + m00 * m00); m01 = il; m00 *= il; }
            for (int k = 0; k < 3; ++k) out[k] = m01 * U[k] - m00 * V[k];
        } else { out[0] = U[0]; out[1] = U[1]; out[2] = U[2]; }
    } else {
        if (am11 > EIG_EPS || am01 > EIG_EPS) {
            if (am11 >= am01) { m01 /= m11; float il = 1.0f / sqrtf(1.0f + m01 * m01); m11 = il; m01 *= il; }
            else { m11 /= m01; float il = 1.0f / sqrtf(1.0f + m11 * m11); m01 = il; m11 *= il; }
            for (int k = 0; k < 3; ++k) out[k] = m11 * U[k] - m01 * V[k];
        } else { out[0] = U[0]; out[1] = U[1]; out[2] = U[2]; }
    }
}

/* evec3_symmetric, eigen.h:452: three cartesian eigenvectors for ascending evals */
void or_evec3(float a, float b, float c, float d, float e, float f, const float* evals,
              float* ev0, float* ev1, float* ev2) {
    const float udn = b * b + d * d + e * e;
    if (udn < EIG_EPS) {
        float val[3] = {a, c, f};
        int idx[3] = {0, 1, 2};
        /* bubble sort of (eval, index) pairs, eigen.h:470-472 */
        if (val[0] > val[1]) { swapf(&val[0], &val[1]); int t = idx[0]; idx[0] = idx[1]; idx[1] = t; }
        if (val[1] > val[2]) { swapf(&val[1], &val[2]); int t = idx[1]; idx[1] = idx[2]; idx[2] = t; }
        if (val[0] > val[1]) { swapf(&val[0], &val[1]); int t = idx[0]; idx[0] = idx[1]; idx[1] = t; }
        float* outs[3] = {ev0, ev1, ev2};
        for (int k = 0; k < 3; ++k) {
            outs[k][0] = idx[k] == 0; outs[k][1] = idx[k] == 1; outs[k][2] = idx[k] == 2;
        }
        return;
    }
    const float q = (a + c + f) / 3.0f;
    const float p2 = (a - q) * (a - q) + (c - q) * (c - q) + (f - q) * (f - q) + 2.0f * udn;
    const float p = sqrtf(p2 / 6.0f);
    float halfDet;
    if (p < EIG_EPS) halfDet = 0.0f;
    else halfDet = det3f(a - q, b, c - q, d, e, f - q) / (2.0f * (p * p * p));
    halfDet = (halfDet < -1.0f) ? -1.0f : ((halfDet > 1.0f) ? 1.0f : halfDet);
    if (halfDet >= 0.0f) {
        evec3_0(a, b, c, d, e, f, evals[2], ev2);
        evec3_1(a, b, c, d, e, f, evals[1], ev2, ev1);
        cross3f(ev1, ev2, ev0);
    } else {
        evec3_0(a, b, c, d, e, f, evals[0], ev0);
        evec3_1(a, b, c, d, e, f, evals[1], ev0, ev1);
        cross3f(ev0, ev1, ev2);
        normalize3f(ev2);
    }
}

/* the sign rule of evec3spherical_symmetric, eigen.h:524-537 */
static void canonical_sign(float* v) {
    float ax = fabsf(v[0]), ay = fabsf(v[1]), az = fabsf(v[2]);
    int k = 0; float amax = ax;
    if (ay > amax) { k = 1; amax = ay; }
    if (az > amax) { k = 2; amax = az; }
    if (v[k] < 0.0f) { v[0] = -v[0]; v[1] = -v[1]; v[2] = -v[2]; }
}

/* evec3spherical_symmetric, eigen.h:515: (theta, phi) per eigenvector */
void or_evec3spherical(float a, float b, float c, float d, float e, float f, const float* evals, float* out6) {
    float v[3][3];
    or_evec3(a, b, c, d, e, f, evals, v[0], v[1], v[2]);
    for (int k = 0; k < 3; ++k) {
        canonical_sign(v[k]);
        v[k][2] = (v[k][2] < -1.0f) ? -1.0f : ((v[k][2] > 1.0f) ? 1.0f : v[k][2]);
        out6[2 * k + 0] = atan2f(v[k][1], v[k][0]);
        out6[2 * k + 1] = acosf(v[k][2]);
    }
}

/* spherical_to_cartesian, tira/functions/tensor.h:26 */
void or_spherical_to_cartesian(float theta, float phi, float* out3) {
    const float st = sinf(theta), ct = cosf(theta), sp = sinf(phi), cp = cosf(phi);
    out3[0] = ct * sp; out3[1] = st * sp; out3[2] = cp;
}

/* cpu::evals3_symmetric / evecs3spherical_symmetric, eigen.h:621,652 (glm::mat3 input,
 * reading entries {0,1,2,4,5,8} as a, b, d, c, e, f) */
void or_evals3(const float* m9, size_t n, float* evals3) {
    for (size_t i = 0; i < n; ++i) {
        const float* m = m9 + 9 * i;
        or_eval3(m[0], m[1], m[4], m[2], m[5], m[8], &evals3[3 * i], &evals3[3 * i + 1], &evals3[3 * i + 2]);
    }
}
void or_evecs3spherical(const float* m9, const float* evals3, size_t n, float* out6) {
    for (size_t i = 0; i < n; ++i) {
        const float* m = m9 + 9 * i;
        or_evec3spherical(m[0], m[1], m[4], m[2], m[5], m[8], evals3 + 3 * i, out6 + 6 * i);
    }
}
void or_evecs3cart(const float* m9, const float* evals3, size_t n, float* out9) {
    for (size_t i = 0; i < n; ++i) {
        const float* m = m9 + 9 * i;
        or_evec3(m[0], m[1], m[4], m[2], m[5], m[8], evals3 + 3 * i, out9 + 9 * i, out9 + 9 * i + 3, out9 + 9 * i + 6);
    }
}

/* cpu::evals3_symmetric + evecs3 over a batch, spread over OpenMP threads
 * (a harness loop for timing the reference's CPU eigensolver on all cores;
 * the per-matrix arithmetic is or_eval3 / or_evec3 unchanged). */
void or_eig3_batch_threads(const float* m9, size_t n, float* evals3, float* evecs9, int threads) {
#ifdef _OPENMP
    if (threads < 1) threads = 1;
#pragma omp parallel for schedule(static) num_threads(threads)
#endif
    for (long long i = 0; i < (long long)n; ++i) {
        const float* m = m9 + 9 * i;
        or_eval3(m[0], m[1], m[4], m[2], m[5], m[8], &evals3[3 * i], &evals3[3 * i + 1], &evals3[3 * i + 2]);
        or_evec3(m[0], m[1], m[4], m[2], m[5], m[8], evals3 + 3 * i, evecs9 + 9 * i, evecs9 + 9 * i + 3,
                 evecs9 + 9 * i + 6);
    }
    (void)threads;
}

/* ---------------- FP64 precision oracle (no reference counterpart) ----------------
 * Cyclic Jacobi on a symmetric 3x3 matrix in double precision, iterated to
 * convergence; eigenvalues ascending, eigenvectors as the columns of V
 * (returned as three rows ev0, ev1, ev2, unit length, sign canonicalised as
 * in eigen.h so the two solvers can be compared directly). */
void or_eig3_f64(const double* s6, double* evals3, double* evecs9) {
    /* s6 = (xx, xy, xz, yy, yz, zz) */
    double A[3][3] = {{s6[0], s6[1], s6[2]}, {s6[1], s6[3], s6[4]}, {s6[2], s6[4], s6[5]}};
    double V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        double diag = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
        if (off <= 1e-36 * diag || off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (A[p][q] == 0.0) continue;
                double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
                for (int k = 0; k < 3; ++k) {  /* A <- A J */
                    double akp = A[k][p], akq = A[k][q];
                    A[k][p] = cs * akp - sn * akq; A[k][q] = sn * akp + cs * akq;
                }
                for (int k = 0; k < 3; ++k) {  /* A <- J^T A */
                    double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = cs * apk - sn * aqk; A[q][k] = sn * apk + cs * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = cs * vkp - sn * vkq; V[k][q] = sn * vkp + cs * vkq;
                }
            }
    }
    int idx[3] = {0, 1, 2};
    double ev[3] = {A[0][0], A[1][1], A[2][2]};
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2 - i; ++j)
            if (ev[idx[j]] > ev[idx[j + 1]]) { int t = idx[j]; idx[j] = idx[j + 1]; idx[j + 1] = t; }
    for (int k = 0; k < 3; ++k) {
        int c = idx[k];
        evals3[k] = ev[c];
        double v[3] = {V[0][c], V[1][c], V[2][c]};
        double nrm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        int m = 0; double am = fabs(v[0]);
        if (fabs(v[1]) > am) { m = 1; am = fabs(v[1]); }
        if (fabs(v[2]) > am) { m = 2; }
        double s = (v[m] < 0 ? -1.0 : 1.0) / nrm;
        evecs9[3 * k + 0] = v[0] * s; evecs9[3 * k + 1] = v[1] * s; evecs9[3 * k + 2] = v[2] * s;
    }
}

void or_eig3_f64_batch(const double* s6, size_t n, double* evals3, double* evecs9) {
    for (size_t i = 0; i < n; ++i) or_eig3_f64(s6 + 6 * i, evals3 + 3 * i, evecs9 + 9 * i);
}
