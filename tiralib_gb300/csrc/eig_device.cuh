// Device eigensolvers for symmetric 2x2 / 3x3 tensors.
//
// Parity flavour: tiralib's FP32 closed forms, operation for operation, so
// results match the reference within FP32 rounding:
//   quad_root / eval2_symmetric / evec2polar_symmetric  eigen.h:90,119,150
//   eval3_symmetric (Smith's trigonometric method)      eigen.h:392
//   evec3_symmetric (+ _0 cofactor rows, _1 2x2 on the orthogonal
//   complement, ComputeOrthogonalComplement)            eigen.h:452,248,291,218
//   evec3spherical_symmetric sign rule + (theta, phi)   eigen.h:515
//   spherical_to_cartesian                              tensor.h:26
// Precise flavour (no reference counterpart): see "precise mode" below; FP64
// is used only for a pair closer than 1e-4 |lambda_max|.
#pragma once
#include <cuda_runtime.h>

namespace tvgb {

#define TVGB_EIG_EPS 1e-6f   // tira::constant::TIRA_EIGEN_EPSILON<float>, eigen.h:13
#define TVGB_PI_F 3.14159265358979323846f

__device__ __forceinline__ void swapf_d(float& a, float& b) { float t = a; a = b; b = t; }
__device__ __forceinline__ float dot3_d(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ __forceinline__ void cross3_d(const float* a, const float* b, float* r) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ void normalize3_d(float* v) {
    float n = sqrtf(dot3_d(v, v));
    if (n > TVGB_EIG_EPS) {
        float inv = 1.0f / n;
        v[0] *= inv; v[1] *= inv; v[2] *= inv;
    }
}

// ------------------------------------------------------------------ 2x2
__device__ __forceinline__ void eval2_d(float a, float b, float c, float& e0, float& e1) {
    const float tr = a + c, det = a * c - b * b;
    const float bq = -tr;
    float disc = bq * bq - 4.0f * det;
    if (disc < 0.0f) disc = 0.0f;
    const float q = -0.5f * (bq + (bq < 0.0f ? -1.0f : 1.0f) * sqrtf(disc));
    e1 = q;
    e0 = (q == 0.0f) ? 0.0f : det / q;
    if (e0 > e1) swapf_d(e0, e1);
    const float scale = fabsf(e1) > 1.0f ? fabsf(e1) : 1.0f;
    const float tol = TVGB_EIG_EPS * scale;
    if (e0 < 0.0f && e0 > -tol) e0 = 0.0f;
    if (e1 < 0.0f && e1 > -tol) e1 = 0.0f;
}

__device__ __forceinline__ void evec2polar_d(float a, float b, float c, float l0, float& th0, float& th1) {
    float vx0 = -b, vy0 = a - l0, vx1 = c - l0, vy1 = -b;
    const float n0 = vx0 * vx0 + vy0 * vy0, n1 = vx1 * vx1 + vy1 * vy1;
    float vx = n0 >= n1 ? vx0 : vx1, vy = n0 >= n1 ? vy0 : vy1;
    float n = sqrtf(vx * vx + vy * vy);
    if (n < TVGB_EIG_EPS) { vx = 1.0f; vy = 0.0f; }
    else { const float inv = 1.0f / n; vx *= inv; vy *= inv; }
    if (fabsf(vx) >= fabsf(vy)) { if (vx < 0.0f) { vx = -vx; vy = -vy; } }
    else if (vy < 0.0f) { vx = -vx; vy = -vy; }
    th0 = atan2f(vy, vx);
    float ux = -vy, uy = vx;
    if (fabsf(ux) >= fabsf(uy)) { if (ux < 0.0f) { ux = -ux; uy = -uy; } }
    else if (uy < 0.0f) { ux = -ux; uy = -uy; }
    th1 = atan2f(uy, ux);
    const float pi = TVGB_PI_F;
    if (th0 <= -pi) th0 += 2.0f * pi;
    if (th1 <= -pi) th1 += 2.0f * pi;
    if (th0 > pi) th0 -= 2.0f * pi;
    if (th1 > pi) th1 -= 2.0f * pi;
}

// ------------------------------------------------------------------ 3x3 (eigen.h semantics)
// matrix | a b d ; b c e ; d e f |
__device__ __forceinline__ void eval3_d(float a, float b, float c, float d, float e, float f,
                                        float& e0, float& e1, float& e2) {
    const float p1 = b * b + d * d + e * e;
    if (p1 < TVGB_EIG_EPS) {
        e0 = a; e1 = c; e2 = f;
        if (e0 > e1) swapf_d(e0, e1);
        if (e1 > e2) swapf_d(e1, e2);
        if (e0 > e1) swapf_d(e0, e1);
        return;
    }
    const float tr = a + c + f;
    const float q = tr / 3.0f;
    const float aq = a - q, cq = c - q, fq = f - q;
    const float p2 = aq * aq + cq * cq + fq * fq + 2.0f * p1;
    const float p = sqrtf(p2 / 6.0f);
    const float pinv = 1.0f / p;
    const float Ba = pinv * aq, Bb = pinv * b, Bc = pinv * cq, Bd = pinv * d, Be = pinv * e, Bf = pinv * fq;
    const float detB = Ba * (Bc * Bf - Be * Be) - Bb * (Bb * Bf - Bd * Be) + Bd * (Bb * Be - Bd * Bc);
    const float r = detB / 2.0f;
    float phi;
    if (r < -1.0f) phi = TVGB_PI_F / 3.0f;
    else if (r >= 1.0f) phi = 0.0f;
    else phi = acosf(r) / 3.0f;
    e2 = q + 2.0f * p * cosf(phi);
    e0 = q + 2.0f * p * cosf(phi + (2.0f * TVGB_PI_F / 3.0f));
    e1 = tr - e0 - e2;
}

__device__ __forceinline__ void evec3_0_d(float a, float b, float c, float d, float e, float f, float ev, float* out) {
    const float m00 = a - ev, m01 = b, m02 = d, m10 = b, m11 = c - ev, m12 = e, m20 = d, m21 = e, m22 = f - ev;
    const float c00 = m11 * m22 - m12 * m21, c01 = m12 * m20 - m10 * m22, c02 = m10 * m21 - m11 * m20;
    const float c10 = m02 * m21 - m01 * m22, c11 = m00 * m22 - m02 * m20, c12 = m01 * m20 - m00 * m21;
    const float c20 = m01 * m12 - m02 * m11, c21 = m02 * m10 - m00 * m12, c22 = m00 * m11 - m01 * m10;
    const float r0 = c00 * c00 + c01 * c01 + c02 * c02;
    const float r1 = c10 * c10 + c11 * c11 + c12 * c12;
    const float r2 = c20 * c20 + c21 * c21 + c22 * c22;
    if (r0 >= r1 && r0 >= r2) { out[0] = c00; out[1] = c01; out[2] = c02; }
    else if (r1 >= r0 && r1 >= r2) { out[0] = c10; out[1] = c11; out[2] = c12; }
    else { out[0] = c20; out[1] = c21; out[2] = c22; }
    normalize3_d(out);
}

__device__ __forceinline__ void ortho_complement_d(const float* ev, float* U, float* V) {
    const float ax = fabsf(ev[0]), ay = fabsf(ev[1]), az = fabsf(ev[2]);
    float t[3];
    if (ay - ax > TVGB_EIG_EPS) {
        if (az - ax > TVGB_EIG_EPS) { t[0] = 1; t[1] = 0; t[2] = 0; }
        else { t[0] = 0; t[1] = 0; t[2] = 1; }
    } else {
        if (az - ay > TVGB_EIG_EPS) { t[0] = 0; t[1] = 1; t[2] = 0; }
        else { t[0] = 0; t[1] = 0; t[2] = 1; }
    }
    cross3_d(ev, t, U);
    normalize3_d(U);
    cross3_d(ev, U, V);
}

__device__ __forceinline__ void evec3_1_d(float a, float b, float c, float d, float e, float f, float ev1,
                                          const float* evec0, float* out) {
    float U[3], V[3];
    ortho_complement_d(evec0, U, V);
    const float AU[3] = {a * U[0] + b * U[1] + d * U[2], b * U[0] + c * U[1] + e * U[2], d * U[0] + e * U[1] + f * U[2]};
    const float AV[3] = {a * V[0] + b * V[1] + d * V[2], b * V[0] + c * V[1] + e * V[2], d * V[0] + e * V[1] + f * V[2]};
    float m00 = dot3_d(U, AU) - ev1, m01 = dot3_d(U, AV), m11 = dot3_d(V, AV) - ev1;
    const float am00 = fabsf(m00), am01 = fabsf(m01), am11 = fabsf(m11);
    if (am00 >= am11) {
        if (am00 > TVGB_EIG_EPS || am01 > TVGB_EIG_EPS) {
            if (am00 >= am01) { m01 /= m00; const float il = 1.0f / sqrtf(1.0f + m01 * m01); m00 = il; m01 *= il; }
            else { m00 /= m01; const float il = 1.0f / sqrtf(1.0f + m00 * m00); m01 = il; m00 *= il; }
            for (int k = 0; k < 3; ++k) out[k] = m01 * U[k] - m00 * V[k];
        } else { out[0] = U[0]; out[1] = U[1]; out[2] = U[2]; }
    } else {
        if (am11 > TVGB_EIG_EPS || am01 > TVGB_EIG_EPS) {
            if (am11 >= am01) { m01 /= m11; const float il = 1.0f / sqrtf(1.0f + m01 * m01); m11 = il; m01 *= il; }
            else { m11 /= m01; const float il = 1.0f / sqrtf(1.0f + m11 * m11); m01 = il; m11 *= il; }
            for (int k = 0; k < 3; ++k) out[k] = m11 * U[k] - m01 * V[k];
        } else { out[0] = U[0]; out[1] = U[1]; out[2] = U[2]; }
    }
}

// three cartesian eigenvectors for ascending evals (eigen.h:452)
__device__ __forceinline__ void evec3_d(float a, float b, float c, float d, float e, float f, const float* ev,
                                        float* v0, float* v1, float* v2) {
    const float udn = b * b + d * d + e * e;
    if (udn < TVGB_EIG_EPS) {
        float val[3] = {a, c, f};
        int idx[3] = {0, 1, 2};
        if (val[0] > val[1]) { swapf_d(val[0], val[1]); int t = idx[0]; idx[0] = idx[1]; idx[1] = t; }
        if (val[1] > val[2]) { swapf_d(val[1], val[2]); int t = idx[1]; idx[1] = idx[2]; idx[2] = t; }
        if (val[0] > val[1]) { swapf_d(val[0], val[1]); int t = idx[0]; idx[0] = idx[1]; idx[1] = t; }
        v0[0] = idx[0] == 0; v0[1] = idx[0] == 1; v0[2] = idx[0] == 2;
        v1[0] = idx[1] == 0; v1[1] = idx[1] == 1; v1[2] = idx[1] == 2;
        v2[0] = idx[2] == 0; v2[1] = idx[2] == 1; v2[2] = idx[2] == 2;
        return;
    }
    const float q = (a + c + f) / 3.0f;
    const float p2 = (a - q) * (a - q) + (c - q) * (c - q) + (f - q) * (f - q) + 2.0f * udn;
    const float p = sqrtf(p2 / 6.0f);
    float hd;
    if (p < TVGB_EIG_EPS) hd = 0.0f;
    else {
        const float A = a - q, C = c - q, F = f - q;
        hd = (A * (C * F - e * e) - b * (b * F - e * d) + d * (b * e - C * d)) / (2.0f * (p * p * p));
    }
    hd = hd < -1.0f ? -1.0f : (hd > 1.0f ? 1.0f : hd);
    if (hd >= 0.0f) {
        evec3_0_d(a, b, c, d, e, f, ev[2], v2);
        evec3_1_d(a, b, c, d, e, f, ev[1], v2, v1);
        cross3_d(v1, v2, v0);
    } else {
        evec3_0_d(a, b, c, d, e, f, ev[0], v0);
        evec3_1_d(a, b, c, d, e, f, ev[1], v0, v1);
        cross3_d(v0, v1, v2);
        normalize3_d(v2);
    }
}

// sign rule of evec3spherical_symmetric (eigen.h:524-537): the largest-|.|
// component is made non-negative
__device__ __forceinline__ void canonical_sign_d(float* v) {
    const float ax = fabsf(v[0]), ay = fabsf(v[1]), az = fabsf(v[2]);
    int k = 0;
    float am = ax;
    if (ay > am) { k = 1; am = ay; }
    if (az > am) k = 2;
    const float vk = k == 0 ? v[0] : (k == 1 ? v[1] : v[2]);
    if (vk < 0.0f) { v[0] = -v[0]; v[1] = -v[1]; v[2] = -v[2]; }
}

__device__ __forceinline__ void to_spherical_d(float* v, float& theta, float& phi) {
    canonical_sign_d(v);
    const float z = v[2] < -1.0f ? -1.0f : (v[2] > 1.0f ? 1.0f : v[2]);
    theta = atan2f(v[1], v[0]);
    phi = acosf(z);
}

__device__ __forceinline__ void from_spherical_d(float theta, float phi, float* v) {
    const float st = sinf(theta), ct = cosf(theta), sp = sinf(phi), cp = cosf(phi);
    v[0] = ct * sp; v[1] = st * sp; v[2] = cp;
}

// ------------------------------------------------------------------ precise mode
// (no reference counterpart)  The matrix is scaled by a power of two so its
// largest entry is in [1, 2) (exact), which turns eigen.h's absolute 1e-6
// thresholds into relative ones.  Smith's formula gives the three
// eigenvalues; only the one farthest from its neighbour ("isolated") is kept:
// its eigenvector comes from the largest cofactor row of A - l I (eigen.h's
// evec3_symmetric_0), the other two from a symmetric 2x2 Jacobi solve on the
// plane normal to it, and every eigenvalue is re-taken as a Rayleigh
// quotient.  When the remaining pair is closer than 1e-4 |lambda_max| the
// plane projection, the 2x2 solve and the frame are redone in FP64.

// the plane normal to unit w, the 2x2 problem on it, Rayleigh quotients;
// A = (xx, xy, xz, yy, yz, zz), entries scaled into [-2, 2].  Outputs lx <= ly
// with vectors x, y; lw and the squared residual rw of (lw, w).  Unit
// lengths come from the hardware reciprocal square root (2 ulp): the FP32
// results carry ~1e-7 relative rounding either way.
__device__ __forceinline__ void complement_solve(const float* A, const float* w, float& lx, float& ly, float* x,
                                                 float* y, float& lw, float& rw) {
    // U = w x e_k for the axis k of the smallest |w_k| (two non-zero components), V = w x U
    const float aw0 = fabsf(w[0]), aw1 = fabsf(w[1]), aw2 = fabsf(w[2]);
    float U[3];
    if (aw0 <= aw1 && aw0 <= aw2) { U[0] = 0.0f; U[1] = w[2]; U[2] = -w[1]; }
    else if (aw1 <= aw2) { U[0] = -w[2]; U[1] = 0.0f; U[2] = w[0]; }
    else { U[0] = w[1]; U[1] = -w[0]; U[2] = 0.0f; }
    const float nu = rsqrtf(fmaf(U[0], U[0], fmaf(U[1], U[1], U[2] * U[2])));
    U[0] *= nu; U[1] *= nu; U[2] *= nu;
    const float V[3] = {w[1] * U[2] - w[2] * U[1], w[2] * U[0] - w[0] * U[2], w[0] * U[1] - w[1] * U[0]};
    auto mv = [&](const float* v, float* r) {
        r[0] = fmaf(A[0], v[0], fmaf(A[1], v[1], A[2] * v[2]));
        r[1] = fmaf(A[1], v[0], fmaf(A[3], v[1], A[4] * v[2]));
        r[2] = fmaf(A[2], v[0], fmaf(A[4], v[1], A[5] * v[2]));
    };
    float AU[3], AV[3], AW[3];
    mv(U, AU); mv(V, AV); mv(w, AW);
    const float h00 = fmaf(U[0], AU[0], fmaf(U[1], AU[1], U[2] * AU[2]));
    const float h01 = fmaf(U[0], AV[0], fmaf(U[1], AV[1], U[2] * AV[2]));
    const float h11 = fmaf(V[0], AV[0], fmaf(V[1], AV[1], V[2] * AV[2]));
    lw = fmaf(w[0], AW[0], fmaf(w[1], AW[1], w[2] * AW[2]));
    {   // squared residual of the isolated pair (lw, w)
        const float r0 = fmaf(-lw, w[0], AW[0]), r1 = fmaf(-lw, w[1], AW[1]), r2 = fmaf(-lw, w[2], AW[2]);
        rw = fmaf(r0, r0, fmaf(r1, r1, r2 * r2));
    }
    float cs = 1.0f, sn = 0.0f;
    if (h01 != 0.0f) {     // Jacobi rotation zeroing h01: tt = tan of the angle, |tt| <= 1
        const float th = __fdividef(h11 - h00, 2.0f * h01);
        const float ath = fabsf(th);
        // for |th| > 2^60, th^2 + 1 would overflow; tt -> 1 / (2 th) there
        const float den = ath > 1.0e18f ? 2.0f * ath : ath + sqrtf(fmaf(th, th, 1.0f));
        const float tt = copysignf(__fdividef(1.0f, den), th);
        cs = rsqrtf(fmaf(tt, tt, 1.0f));
        sn = tt * cs;
    }
    for (int k = 0; k < 3; ++k) { x[k] = cs * U[k] - sn * V[k]; y[k] = fmaf(sn, U[k], cs * V[k]); }
    float Ax[3], Ay[3];
    mv(x, Ax); mv(y, Ay);
    lx = fmaf(x[0], Ax[0], fmaf(x[1], Ax[1], x[2] * Ax[2]));
    ly = fmaf(y[0], Ay[0], fmaf(y[1], Ay[1], y[2] * Ay[2]));
    if (lx > ly) {
        float tmp;
        for (int k = 0; k < 3; ++k) { tmp = x[k]; x[k] = y[k]; y[k] = tmp; }
        tmp = lx; lx = ly; ly = tmp;
    }
}

// assemble an ascending, right-handed frame from (w, lw) and the pair
template <class T>
__device__ __forceinline__ void assemble(bool iso_high, T lw, const T* w, T lx, T ly, const T* x, const T* y,
                                         float* ev, float* v0, float* v1, float* v2, float unscale) {
    T o0[3], o1[3], o2[3], l0, l1, l2;
    if (iso_high) {   // w is the largest eigenvector
        for (int k = 0; k < 3; ++k) { o0[k] = x[k]; o1[k] = y[k]; }
        l0 = lx; l1 = ly; l2 = lw;
        o2[0] = o0[1] * o1[2] - o0[2] * o1[1]; o2[1] = o0[2] * o1[0] - o0[0] * o1[2]; o2[2] = o0[0] * o1[1] - o0[1] * o1[0];
    } else {
        for (int k = 0; k < 3; ++k) { o1[k] = x[k]; o2[k] = y[k]; }
        l0 = lw; l1 = lx; l2 = ly;
        o0[0] = o1[1] * o2[2] - o1[2] * o2[1]; o0[1] = o1[2] * o2[0] - o1[0] * o2[2]; o0[2] = o1[0] * o2[1] - o1[1] * o2[0];
    }
    ev[0] = float(l0) * unscale; ev[1] = float(l1) * unscale; ev[2] = float(l2) * unscale;
    for (int k = 0; k < 3; ++k) { v0[k] = float(o0[k]); v1[k] = float(o1[k]); v2[k] = float(o2[k]); }
    // Rayleigh quotients may reorder values closer than rounding: keep ascending
    if (ev[0] > ev[1]) { swapf_d(ev[0], ev[1]); for (int k = 0; k < 3; ++k) swapf_d(v0[k], v1[k]); }
    if (ev[1] > ev[2]) { swapf_d(ev[1], ev[2]); for (int k = 0; k < 3; ++k) swapf_d(v1[k], v2[k]); }
    if (ev[0] > ev[1]) { swapf_d(ev[0], ev[1]); for (int k = 0; k < 3; ++k) swapf_d(v0[k], v1[k]); }
}

// FP32 phase.  Returns 0 when done (ev / v* set); otherwise w and iso_high
// are set and the return value selects the FP64 phase: 1 = the remaining
// pair is closer than 1e-4 |lambda_max| (project onto the plane in FP64),
// 2 = Smith's formula isolated no eigenvalue (a near-triple cluster: Jacobi).
// Only the isolated eigenvalue is taken from Smith's formula: the largest
// when det(A - qI) >= 0 (phi <= pi/6), else the smallest.
__device__ __forceinline__ int eig3_precise_fp32(float a, float b, float c, float d, float e, float f, float* ev,
                                                 float* v0, float* v1, float* v2, float* w, bool& iso_high) {
    const float amax = fmaxf(fmaxf(fmaxf(fabsf(a), fabsf(b)), fmaxf(fabsf(c), fabsf(d))), fmaxf(fabsf(e), fabsf(f)));
    iso_high = true;
    if (amax == 0.0f || !(amax < INFINITY)) {
        ev[0] = ev[1] = ev[2] = amax == 0.0f ? 0.0f : NAN;
        v0[0] = 1; v0[1] = 0; v0[2] = 0; v1[0] = 0; v1[1] = 1; v1[2] = 0; v2[0] = 0; v2[1] = 0; v2[2] = 1;
        return 0;
    }
    int ex;
    frexpf(amax, &ex);
    const float sc = ldexpf(1.0f, 1 - ex), unsc = ldexpf(1.0f, ex - 1);   // entries scaled into [1, 2)
    const float A[6] = {a * sc, b * sc, d * sc, c * sc, e * sc, f * sc};   // xx xy xz yy yz zz
    // Smith: A = qI + pB, det(B) / 2 = cos(3 phi)
    const float q = (A[0] + A[3] + A[5]) * (1.0f / 3.0f);
    const float aq = A[0] - q, cq = A[3] - q, fq = A[5] - q;
    const float p6 = fmaf(aq, aq, fmaf(cq, cq, fmaf(fq, fq, 2.0f * fmaf(A[1], A[1], fmaf(A[2], A[2], A[4] * A[4]))))) *
                     (1.0f / 6.0f);
    float l = q;
    if (p6 > 0.0f) {
        const float rp = rsqrtf(p6), p = p6 * rp;
        const float det = aq * fmaf(cq, fq, -A[4] * A[4]) - A[1] * fmaf(A[1], fq, -A[4] * A[2]) +
                          A[2] * fmaf(A[1], A[4], -cq * A[2]);
        const float r = fminf(fmaxf(0.5f * det * (rp * rp * rp), -1.0f), 1.0f);
        iso_high = r >= 0.0f;
        const float phi = acosf(r) * (1.0f / 3.0f);
        l = fmaf(2.0f * p, cosf(iso_high ? phi : phi + 2.0f * TVGB_PI_F / 3.0f), q);
    }
    // w: the largest cofactor row of A - l I (eigen.h's evec3_symmetric_0 rule)
    {
        const float m00 = A[0] - l, m11 = A[3] - l, m22 = A[5] - l, m01 = A[1], m02 = A[2], m12 = A[4];
        const float c0[3] = {m11 * m22 - m12 * m12, m12 * m02 - m01 * m22, m01 * m12 - m11 * m02};
        const float c1[3] = {m02 * m12 - m01 * m22, m00 * m22 - m02 * m02, m01 * m02 - m00 * m12};
        const float c2[3] = {m01 * m12 - m02 * m11, m02 * m01 - m00 * m12, m00 * m11 - m01 * m01};
        const float r0 = fmaf(c0[0], c0[0], fmaf(c0[1], c0[1], c0[2] * c0[2]));
        const float r1 = fmaf(c1[0], c1[0], fmaf(c1[1], c1[1], c1[2] * c1[2]));
        const float r2 = fmaf(c2[0], c2[0], fmaf(c2[1], c2[1], c2[2] * c2[2]));
        const bool s0 = r0 >= r1 && r0 >= r2, s1 = !s0 && r1 >= r2;
        const float rb = s0 ? r0 : (s1 ? r1 : r2);
        if (rb > 1e-12f) {
            const float iw = rsqrtf(rb);
            w[0] = (s0 ? c0[0] : (s1 ? c1[0] : c2[0])) * iw;
            w[1] = (s0 ? c0[1] : (s1 ? c1[1] : c2[1])) * iw;
            w[2] = (s0 ? c0[2] : (s1 ? c1[2] : c2[2])) * iw;
        } else {                       // cofactors vanished: A ~ l I
            w[0] = 0.0f; w[1] = 0.0f; w[2] = 1.0f;
        }
    }
    float lx, ly, lw, rw, x[3], y[3];
    complement_solve(A, w, lx, ly, x, y, lw, rw);
    if (rw > 1e-10f) return 2;      // w's residual well above FP32 rounding
    const float lm = fmaxf(fmaxf(fabsf(lx), fabsf(ly)), fabsf(lw));
    if ((ly - lx) < 1e-4f * lm) return 1;
    assemble<float>(iso_high, lw, w, lx, ly, x, y, ev, v0, v1, v2, unsc);
    return 0;
}

// Conversions between FP32 and FP64 on the integer pipe.  GB300's FP64 pipe
// executes conversions at its own low rate, and in the FP64 phase below they
// were as many as its arithmetic operations.
// widen_f32: exact for normal floats; zero and subnormal inputs give a signed
// zero; the input is finite.
__device__ __forceinline__ double widen_f32(float x) {
    const unsigned u = __float_as_uint(x), mag = u & 0x7fffffffu;
    const bool nrm = mag >= 0x00800000u;
    const unsigned hi = (u & 0x80000000u) | (nrm ? (mag >> 3) + (896u << 20) : 0u);   // exponent bias 1023 - 127
    return __hiloint2double(int(hi), int(nrm ? u << 29 : 0u));
}
// narrow_trunc: the mantissa truncated to 24 bits (relative error < 2^-23);
// magnitudes below the FP32 normal range give a signed zero; |x| < 2^128.
__device__ __forceinline__ float narrow_trunc(double x) {
    const unsigned hi = unsigned(__double2hiint(x)), lo = unsigned(__double2loint(x));
    const unsigned mag = hi & 0x7fffffffu, sgn = hi & 0x80000000u;
    if ((mag >> 20) <= 896u) return __uint_as_float(sgn);
    return __uint_as_float(sgn | ((mag - (896u << 20)) << 3) | (lo >> 29));
}

// FP64 phase.  code 1: the pair is resolved on the plane normal to w.  The
// plane basis is exact: U = e_k x w copies two components of w (k = the
// smallest |w_k|), V = w x U is formed in FP64, so w, U, V are orthogonal to
// FP64 rounding and |V|^2 = |w|^2 |U|^2.  The work is done in the frame
// rotated cyclically to put axis k first, where U = (0, -w2, w1) and
// V = (w1^2 + w2^2, -w0 w1, -w0 w2) (products of two floats, exact in FP64).
// The 2x2 matrix H = [U V]^T A [U V] is formed in FP64; with the Gram scaling
// folded in (H' = diag(1, 1/|w|) H diag(1, 1/|w|) / |U|^2, |w|^2 = 1 +
// O(eps32) so 1/|w| and 1/|w|^2 are two-term series) its difference and
// off-diagonal, which cancel for a close pair, are exact to FP64 rounding.
// The Jacobi angle needs only FP32 relative accuracy from those two numbers,
// the pair's eigenvalues come from the rotated FP64 diagonal, and the frame
// is completed in FP32.  41 FP64 arithmetic operations, and two conversions
// (the pair's eigenvalues to FP32).
// code 2: cyclic Jacobi on the whole matrix in FP64.
__device__ __forceinline__ void eig3_precise_fp64(float a, float b, float c, float d, float e, float f, const float* w,
                                                  bool iso_high, int code, float* ev, float* v0, float* v1, float* v2) {
    const float amax = fmaxf(fmaxf(fmaxf(fabsf(a), fabsf(b)), fmaxf(fabsf(c), fabsf(d))), fmaxf(fabsf(e), fabsf(f)));
    int ex;
    frexpf(amax, &ex);
    const float sc = ldexpf(1.0f, 1 - ex), unsc = ldexpf(1.0f, ex - 1);
    if (code == 1) {
        const float Af[6] = {a * sc, b * sc, d * sc, c * sc, e * sc, f * sc};   // xx xy xz yy yz zz
        const float aw0 = fabsf(w[0]), aw1 = fabsf(w[1]), aw2 = fabsf(w[2]);
        const int k = (aw0 <= aw1 && aw0 <= aw2) ? 0 : (aw1 <= aw2 ? 1 : 2);
        // A and w in the frame (k, k + 1, k + 2 mod 3)
        float p00, p01, p02, p11, p12, p22, s0, s1, s2;
        if (k == 0) {
            p00 = Af[0]; p11 = Af[3]; p22 = Af[5]; p01 = Af[1]; p02 = Af[2]; p12 = Af[4];
            s0 = w[0]; s1 = w[1]; s2 = w[2];
        } else if (k == 1) {
            p00 = Af[3]; p11 = Af[5]; p22 = Af[0]; p01 = Af[4]; p02 = Af[1]; p12 = Af[2];
            s0 = w[1]; s1 = w[2]; s2 = w[0];
        } else {
            p00 = Af[5]; p11 = Af[0]; p22 = Af[3]; p01 = Af[2]; p02 = Af[4]; p12 = Af[1];
            s0 = w[2]; s1 = w[0]; s2 = w[1];
        }
        const double P00 = widen_f32(p00), P01 = widen_f32(p01), P02 = widen_f32(p02), P11 = widen_f32(p11),
                     P12 = widen_f32(p12), P22 = widen_f32(p22);
        const double W0 = widen_f32(s0), W1 = widen_f32(s1), W2 = widen_f32(s2);
        const double V0 = fma(W1, W1, W2 * W2), V1 = -(W0 * W1), V2 = -(W0 * W2);
        const double nw = fma(W0, W0, V0);
        const double AU0 = fma(P02, W1, -(P01 * W2));                 // A U, U = (0, -W2, W1)
        const double AU1 = fma(P12, W1, -(P11 * W2));
        const double AU2 = fma(P22, W1, -(P12 * W2));
        const double AV0 = fma(P00, V0, fma(P01, V1, P02 * V2));
        const double AV1 = fma(P01, V0, fma(P11, V1, P12 * V2));
        const double AV2 = fma(P02, V0, fma(P12, V1, P22 * V2));
        const double h00 = fma(W1, AU2, -(W2 * AU1));
        const double h01 = fma(V0, AU0, fma(V1, AU1, V2 * AU2));
        const double h11 = fma(V0, AV0, fma(V1, AV1, V2 * AV2));
        const double dn = nw - 1.0;                                  // |dn| ~ 1e-7
        const double inw = fma(dn, dn, 1.0 - dn);                    // 1 / |w|^2
        const double isq = fma(0.375 * dn, dn, 1.0 - 0.5 * dn);      // 1 / |w|
        const double g11 = h11 * inw, g01 = h01 * isq;               // |U|^2 H'
        // Jacobi rotation of [[h00, g01], [g01, g11]] in FP32 from exact inputs
        const float ddf = narrow_trunc(g11 - h00), g01f = narrow_trunc(g01);
        float cs = 1.0f, sn = 0.0f, tt = 0.0f;
        if (g01f != 0.0f) {
            const float th = ddf / (2.0f * g01f);
            tt = (th >= 0.0f ? 1.0f : -1.0f) / (fabsf(th) + sqrtf(fmaf(th, th, 1.0f)));
            cs = rsqrtf(fmaf(tt, tt, 1.0f));
            sn = tt * cs;
        }
        const double ttd = widen_f32(tt);
        const double lxd = fma(-ttd, g01, h00), lyd = fma(ttd, g01, g11);
        const float nU = fmaf(s1, s1, s2 * s2);                      // |U|^2 = V0
        float lx = float(lxd) / nU, ly = float(lyd) / nU;
        const float iu = rsqrtf(nU), iv = rsqrtf(fmaf(s0, s0, nU) * nU);
        const float Ur[3] = {0.0f, -s2, s1}, Vr[3] = {nU, -s0 * s1, -s0 * s2};
        float xr[3], yr[3];
        for (int i = 0; i < 3; ++i) {
            const float u = Ur[i] * iu, v = Vr[i] * iv;
            xr[i] = cs * u - sn * v;
            yr[i] = fmaf(sn, u, cs * v);
        }
        // back to the original frame: x[(k + j) % 3] = xr[j]
        float x[3], y[3];
        x[0] = k == 0 ? xr[0] : (k == 1 ? xr[2] : xr[1]);
        x[1] = k == 0 ? xr[1] : (k == 1 ? xr[0] : xr[2]);
        x[2] = k == 0 ? xr[2] : (k == 1 ? xr[1] : xr[0]);
        y[0] = k == 0 ? yr[0] : (k == 1 ? yr[2] : yr[1]);
        y[1] = k == 0 ? yr[1] : (k == 1 ? yr[0] : yr[2]);
        y[2] = k == 0 ? yr[2] : (k == 1 ? yr[1] : yr[0]);
        // ly - lx = dd + 2 tt g01, and tt g01 has the sign of dd (of g01 when
        // dd is 0), so the order follows from signs: no FP64 comparison
        if (ddf != 0.0f ? ddf < 0.0f : g01f < 0.0f) {
            float tmp;
            for (int i = 0; i < 3; ++i) { tmp = x[i]; x[i] = y[i]; y[i] = tmp; }
            tmp = lx; lx = ly; ly = tmp;
        }
        // the isolated eigenvalue: FP32 Rayleigh quotient of w
        const float Aw0 = fmaf(Af[0], w[0], fmaf(Af[1], w[1], Af[2] * w[2]));
        const float Aw1 = fmaf(Af[1], w[0], fmaf(Af[3], w[1], Af[4] * w[2]));
        const float Aw2 = fmaf(Af[2], w[0], fmaf(Af[4], w[1], Af[5] * w[2]));
        const float lw = fmaf(w[0], Aw0, fmaf(w[1], Aw1, w[2] * Aw2)) / fmaf(s0, s0, nU);
        assemble<float>(iso_high, lw, w, lx, ly, x, y, ev, v0, v1, v2, unsc);
        return;
    }
    const double A[6] = {double(a * sc), double(b * sc), double(d * sc), double(c * sc), double(e * sc), double(f * sc)};
    // no eigenvalue is isolated (a near-triple cluster): cyclic Jacobi in FP64
    double M[3][3] = {{A[0], A[1], A[2]}, {A[1], A[3], A[4]}, {A[2], A[4], A[5]}};
    double Q[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 8; ++sweep) {
        const double off = M[0][1] * M[0][1] + M[0][2] * M[0][2] + M[1][2] * M[1][2];
        const double dg = M[0][0] * M[0][0] + M[1][1] * M[1][1] + M[2][2] * M[2][2];
        if (!(off > 1e-32 * dg)) break;
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            if (M[p][q] == 0.0) continue;
            const double th = (M[q][q] - M[p][p]) / (2.0 * M[p][q]);
            const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
            const double cc = 1.0 / sqrt(t * t + 1.0), ss = t * cc;
            for (int k = 0; k < 3; ++k) {
                const double mkp = M[k][p], mkq = M[k][q];
                M[k][p] = cc * mkp - ss * mkq; M[k][q] = ss * mkp + cc * mkq;
            }
            for (int k = 0; k < 3; ++k) {
                const double mpk = M[p][k], mqk = M[q][k];
                M[p][k] = cc * mpk - ss * mqk; M[q][k] = ss * mpk + cc * mqk;
            }
            for (int k = 0; k < 3; ++k) {
                const double qkp = Q[k][p], qkq = Q[k][q];
                Q[k][p] = cc * qkp - ss * qkq; Q[k][q] = ss * qkp + cc * qkq;
            }
        }
    }
    int o[3] = {0, 1, 2};
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2 - i; ++j)
            if (M[o[j]][o[j]] > M[o[j + 1]][o[j + 1]]) { const int t = o[j]; o[j] = o[j + 1]; o[j + 1] = t; }
    float* vs[3] = {v0, v1, v2};
    for (int k = 0; k < 3; ++k) {
        ev[k] = float(M[o[k]][o[k]]) * unsc;
        for (int r = 0; r < 3; ++r) vs[k][r] = float(Q[r][o[k]]);
    }
}

// both phases in one call (per-thread use); true when FP64 ran
__device__ __forceinline__ bool eig3_precise_d(float a, float b, float c, float d, float e, float f, float* ev,
                                               float* v0, float* v1, float* v2) {
    float w[3];
    bool hi;
    const int code = eig3_precise_fp32(a, b, c, d, e, f, ev, v0, v1, v2, w, hi);
    if (!code) return false;
    eig3_precise_fp64(a, b, c, d, e, f, w, hi, code, ev, v0, v1, v2);
    return true;
}

}  // namespace tvgb
