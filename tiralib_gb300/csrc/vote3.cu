// 3D tensor voting on sm_103a: voter preparation, the stick + closed-form
// plate (+ ball) vote with its fused eigendecomposition, the generic path
// (any power / sample count, ATV) and the C ABI.
//
// Reference path replaced (tira/functions/tensorvote.h):
//   tira::cuda::tensorvote3 :2817 -> evals3/evecs3spherical (eigen.h:896,945)
//   -> serial host spherical->cartesian loop :2831-2858 -> _tensorvote3_tk :2741
//   -> global_stickvote3 :2412 + global_platevote3 :2589 (two launches, each a
//   read-modify-write of a 36-byte glm::mat3, neighbour table in global
//   memory for w > 11, plate = `samples` stick votes per pair with a basis
//   rebuilt per pair), or global_tensorvote3_atv :2640.
//
// Here:
//   k_prep3      one pass over the input field: eigen.h's solve, the
//                reference's spherical round trip of the eigenvectors
//                (parity mode), and per-voter scales -> voter records.
//   k_vote3_fast power = 1 with an exact plate (samples == 0 or >= 3):
//                receivers tiled 32 x 8 x R per CTA, voter rows with their
//                sigma-halo staged in shared memory, per-offset weights from
//                a radial table (they depend on |offset|^2 only), stick and
//                plate accumulated in registers in one pass, FP32 row
//                partials folded into per-voxel Kahan sums, eigensolve fused
//                into the epilogue.
//   k_vote3_generic every other case (power > 1, samples < power + 2, ball
//                with power > 1, ATV): one receiver per thread, exact
//                reference arithmetic per pair.
//
// The plate closed form.  For voter plate normal n (unit), offset d = o/|o|,
// c1 = exp(-|o|^2/s1^2), c2 likewise and ct = c2 - c1, the reference's plate
// is (1/pi) * (pi/S) sum_i stick(q_i), q_i = cos(i pi/S) u + sin(i pi/S) v.
// The summand is a trigonometric polynomial of degree 2 power + 2 in the
// angle, so for S >= power + 2 the S-point rule equals the integral over
// [0, pi).  With R = I - 2 d d^T, P = I - n n^T and p = P d the integral is
//   (1/pi) R [ (pi/2) c1 P + (pi/8) ct (|p|^2 P + 2 p p^T) ] R
// = (c1/2 + ct |p|^2 / 8) (I - m m^T) + (ct / 4) (R p)(R p)^T,   m = R n,
// and with v = n.o, g = 1/|o|^2:  m = n - 2 v g o,  R p = -(o + v m)/|o|,
// |p|^2 = [o != 0] - v^2 g.  The ball term (mean of unit stick votes over the
// sphere, scaled by lambda0) is (c1/3 + ct [o != 0] / 15) I + (2 ct g / 15) o o^T.
#include "tvgb_internal.cuh"
#include "eig_device.cuh"
#include <algorithm>
#include <vector>

namespace tvgb {

constexpr int VX = 32;   // receivers per CTA along x (one warp)
constexpr int VY = 8;    // rows of warps per CTA

// ------------------------------------------------------------------ voter preparation

struct PrepOut {
    float4* A;   // (q, stick scale * sticknorm)  -- largest eigenvector
    float4* B;   // (n, plate scale)               -- smallest eigenvector (unit)
    float* C;    // lambda0 (ball)
    float4* L;   // (lambda0, lambda1, lambda2, 0) -- ATV / generic
    float4* E1;  // middle eigenvector (ATV)
    int atv;     // A, B, C hold the ATV scales: lambda2 - lambda1, lambda1 - lambda0, lambda0
};

template <int LAYOUT>
__device__ __forceinline__ void read_tensor(const float* __restrict__ in, size_t n, size_t i, float& a, float& b,
                                            float& c, float& d, float& e, float& f) {
    if (LAYOUT == 9) {
        const float* m = in + i * 9;
        a = __ldg(m); b = __ldg(m + 1); d = __ldg(m + 2); c = __ldg(m + 4); e = __ldg(m + 5); f = __ldg(m + 8);
    } else if (LAYOUT == 6) {
        const float* m = in + i * 6;
        a = __ldg(m); b = __ldg(m + 1); d = __ldg(m + 2); c = __ldg(m + 3); e = __ldg(m + 4); f = __ldg(m + 5);
    } else {
        a = __ldg(in + i); b = __ldg(in + n + i); d = __ldg(in + 2 * n + i);
        c = __ldg(in + 3 * n + i); e = __ldg(in + 4 * n + i); f = __ldg(in + 5 * n + i);
    }
}

template <int LAYOUT>
__global__ void __launch_bounds__(256) k_prep3(const float* __restrict__ in, size_t n, PrepOut o, float sticknorm,
                                                int parity) {
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        float a, b, c, d, e, f;
        read_tensor<LAYOUT>(in, n, i, a, b, c, d, e, f);
        float ev[3], v0[3], v1[3], v2[3];
        if (parity) {
            eval3_d(a, b, c, d, e, f, ev[0], ev[1], ev[2]);
            evec3_d(a, b, c, d, e, f, ev, v0, v1, v2);
            // cpu::tensorvote3 / cuda::tensorvote3 pass the eigenvectors through
            // float (theta, phi) and back (tensorvote.h:1831-1849, 2831-2858)
            float th, ph;
            to_spherical_d(v0, th, ph); from_spherical_d(th, ph, v0);
            to_spherical_d(v1, th, ph); from_spherical_d(th, ph, v1);
            to_spherical_d(v2, th, ph); from_spherical_d(th, ph, v2);
        } else {
            eig3_precise_d(a, b, c, d, e, f, ev, v0, v1, v2);
        }
        if (o.A) {
            // TK: tensorvote.h:1537; ATV: atv_H's s1 = lambda2 - lambda1 (:660), no normaliser
            const float ss = o.atv ? ev[2] - ev[1] : copysignf(fabsf(ev[2]) - fabsf(ev[1]), ev[2]) * sticknorm;
            o.A[i] = make_float4(v2[0], v2[1], v2[2], ss);
        }
        if (o.B) {
            // plate3_numerical_device normalises the normal and skips a zero one (:2461-2465)
            const float nn = v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2];
            // TK: :2616; ATV: atv_H's s2 = lambda1 - lambda0 on the plane normal to n (:661)
            float sp = o.atv ? ev[1] - ev[0] : copysignf(fabsf(ev[1]) - fabsf(ev[0]), ev[1]);
            float inv = 0.0f;
            if (nn > 1e-12f) inv = rsqrtf(nn); else sp = 0.0f;
            o.B[i] = make_float4(v0[0] * inv, v0[1] * inv, v0[2] * inv, sp);
        }
        if (o.C) o.C[i] = ev[0];
        if (o.L) o.L[i] = make_float4(ev[0], ev[1], ev[2], 0.0f);
        if (o.E1) o.E1[i] = make_float4(v1[0], v1[1], v1[2], 0.0f);
    }
}

// ------------------------------------------------------------------ radial table
// entry (8 floats) for integer |o|^2 = L2:
//   a = (c1, ct * g, 2 g, c1/2 + ct [L2>0] / 8)
//   b = (ct g / 8, ct g / 4, c1/3 + ct [L2>0] / 15, 2 ct g / 15)
__device__ __forceinline__ void radial_entry(int L2, float s1, float s2, float4& a, float4& b) {
    const float l2 = float(L2);
    const float inv1 = s1 > 0.0f ? 1.0f / (s1 * s1) : 0.0f;
    const float inv2 = s2 > 0.0f ? 1.0f / (s2 * s2) : 0.0f;
    // build_neighbors3d's weights, including the sigma == 0 rule (tensorvote.h:1431-1432)
    const float c1 = s1 == 0.0f ? (l2 > 1e-12f ? 0.0f : 1.0f) : expf(-l2 * inv1);
    const float c2 = s2 == 0.0f ? (l2 > 1e-12f ? 0.0f : 1.0f) : expf(-l2 * inv2);
    const float ct = c2 - c1;
    const float g = L2 > 0 ? 1.0f / l2 : 0.0f;
    const float dd = L2 > 0 ? 1.0f : 0.0f;
    a = make_float4(c1, ct * g, 2.0f * g, 0.5f * c1 + 0.125f * ct * dd);
    b = make_float4(0.125f * ct * g, 0.25f * ct * g, c1 * (1.0f / 3.0f) + ct * dd * (1.0f / 15.0f),
                    ct * g * (2.0f / 15.0f));
}

// ATV (tensorvote.h:710) in the same closed-form terms.  With d the unit
// offset (zero at the voter itself), R = I - 2 d d^T, c the attenuation
// exp(-|o|^2 / sigma^2) and the voter's eigenpairs (l_k, e_k):
//   stick  c (l2 - l1) (1 - (e2.d)^2) (R e2)(R e2)^T
//   plate  c (l1 - l0) [(1 - |Pd|^2 / 4)(I - m m^T) - (R Pd)(R Pd)^T / 2],
//          P = I - e0 e0^T = e1 e1^T + e2 e2^T, m = R e0, |Pd|^2 = 1 - (e0.d)^2
//   ball   c l0 [(1 - |d|^2 / 5) I - (2 / 5) d d^T]
// which is c R H R of atv_H (:607): for T = q q^T the H term reduces to
// (1 - (q.d)^2) q q^T, R I R = I and R d = -d.  These are the basis tensors
// the TK kernels accumulate (R q, I - m m^T, h = o + (n.o) m = -|o| R Pd,
// and o o^T), so ATV runs on them with this radial table:
//   a = (c, -c g, 2 g, A0),  b = (A1, Bp, ball I, ball oo^T),  g = 1 / |o|^2,
//   A0 = c (3/4 for o != 0, 1 at o = 0), A1 = -c g / 4, Bp = -c g / 2,
//   ball I = c (4/5 for o != 0, 1 at o = 0), ball oo^T = -2 c g / 5,
// and voter records A = (e2, l2 - l1), B = (e0, l1 - l0), C = l0.
__device__ __forceinline__ void radial_entry_atv(int L2, float sigma, float4& a, float4& b) {
    const float l2 = float(L2);
    const float c = sigma == 0.0f ? (l2 > 1e-12f ? 0.0f : 1.0f) : expf(-l2 / (sigma * sigma));   // atv_attenuation :35
    const float g = L2 > 0 ? 1.0f / l2 : 0.0f;
    const bool o0 = L2 == 0;
    a = make_float4(c, -c * g, 2.0f * g, o0 ? c : 0.75f * c);
    b = make_float4(-0.25f * c * g, -0.5f * c * g, o0 ? c : 0.8f * c, -0.4f * c * g);
}

// ------------------------------------------------------------------ fast kernel

struct FastArgs {
    const float4* A;
    const float4* B;
    const float* C;
    int s0, s1, s2, hw, rows;   // rows: voter rows (offsets) staged per stage
    float sig1, sig2;
    float* out;
    int out_layout;
    float* evals;
    float* evecs;
    int evec_fmt;
    int precise_eig;
    int zr0, zr1;               // receivers voted: planes [zr0, zr1) (launch_fast: [0, s0) if empty)
    int atv;                    // ATV weights (radial_entry_atv, sigma = sig1) instead of TK's
};

__device__ __forceinline__ void fast_radial_entry(const FastArgs& a, int L2, float4& ea, float4& eb) {
    if (a.atv) radial_entry_atv(L2, a.sig1, ea, eb);
    else radial_entry(L2, a.sig1, a.sig2, ea, eb);
}

__device__ __forceinline__ void kahan_add(float& sum, float& comp, float x) {
    const float y = x - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

#ifndef TVGB_FAST_R
#define TVGB_FAST_R 4          // receivers per thread along z
#endif
#ifndef TVGB_FAST_MINB
#define TVGB_FAST_MINB 2       // resident CTAs per SM the register budget is sized for
#endif
#ifndef TVGB_FOLD_PLANE
#define TVGB_FOLD_PLANE 1      // 1: FP32 partials span a whole voter plane before the Kahan fold
#endif
#ifndef TVGB_DUNROLL
#define TVGB_DUNROLL 2         // unroll factor of the +-ox loop
#endif
constexpr int kDUnroll = TVGB_DUNROLL;

// Block coordinates from the launch order: CTAs run roughly in linear-index
// order (x fastest), and the plain mapping keeps z-neighbours, which share
// most of their voter planes, a whole xy-layer apart.  In groups of ZG
// z-blocks the order is x, then z within the group, then y, so the CTAs
// resident at one time share their halos in L2.
constexpr int ZG = 8;
__device__ __forceinline__ void swizzled_block(int& bx, int& by, int& bz) {
    const int gx = gridDim.x, gy = gridDim.y, gz = gridDim.z;
    const int L = blockIdx.x + gx * (blockIdx.y + gy * blockIdx.z);
    const int per = ZG * gx * gy;
    const int g = L / per, rem = L - g * per;
    const int gsz = min(ZG, gz - g * ZG);
    bx = rem % gx;
    const int t = rem / gx;
    bz = g * ZG + t % gsz;
    by = t / gsz;
}

// one (receiver, voter) pair: stick + closed-form plate (+ ball) into P[0..6]
template <bool STICK, bool PLATE, bool BALL>
__device__ __forceinline__ void vote_pair(const float4& A, const float4& B, float lb, float ub, float vb, float oxf,
                                          float oyf, float oz, const float4& ta, const float4& tb, float* P) {
    if (STICK) {
        // stickvote3_accumulate_kernel (tensorvote.h:1184) with power = 1
        const float u = fmaf(A.z, oz, ub);             // q . o
        const float k = u * ta.z;                       // 2 (q.o) / |o|^2
        const float rx = fmaf(-k, oxf, A.x);            // r = q - 2 (q.d) d
        const float ry = fmaf(-k, oyf, A.y);
        const float rz = fmaf(-k, oz, A.z);
        const float eta = fmaf(ta.y, u * u, ta.x);      // c1 + (c2 - c1) (q.d)^2
        const float term = A.w * eta;
        const float t0 = term * rx, t1 = term * ry, t2 = term * rz;
        P[0] = fmaf(t0, rx, P[0]);
        P[1] = fmaf(t0, ry, P[1]);
        P[2] = fmaf(t0, rz, P[2]);
        P[3] = fmaf(t1, ry, P[3]);
        P[4] = fmaf(t1, rz, P[4]);
        P[5] = fmaf(t2, rz, P[5]);
    }
    if (PLATE) {
        const float v = fmaf(B.z, oz, vb);             // n . o
        const float k = v * ta.z;
        const float mx = fmaf(-k, oxf, B.x);            // m = R n
        const float my = fmaf(-k, oyf, B.y);
        const float mz = fmaf(-k, oz, B.z);
        const float hx = fmaf(v, mx, oxf);              // h = o + v m = -|o| R p
        const float hy = fmaf(v, my, oyf);
        const float hz = fmaf(v, mz, oz);
        const float cA = fmaf(-tb.x, v * v, ta.w);      // c1/2 + (c2 - c1) |p|^2 / 8
        const float sA = B.w * cA;
        const float sB = B.w * tb.y;                    // (c2 - c1) / (4 |o|^2)
        P[6] += sA;
        const float ax = sA * mx, ay = sA * my, az = sA * mz;
        const float bx = sB * hx, by = sB * hy, bz = sB * hz;
        P[0] = fmaf(bx, hx, fmaf(-ax, mx, P[0]));
        P[1] = fmaf(bx, hy, fmaf(-ax, my, P[1]));
        P[2] = fmaf(bx, hz, fmaf(-ax, mz, P[2]));
        P[3] = fmaf(by, hy, fmaf(-ay, my, P[3]));
        P[4] = fmaf(by, hz, fmaf(-ay, mz, P[4]));
        P[5] = fmaf(bz, hz, fmaf(-az, mz, P[5]));
    }
    if (BALL) {
        P[6] = fmaf(lb, tb.z, P[6]);
        const float wb = lb * tb.w;
        const float wx = wb * oxf, wy = wb * oyf, wz = wb * oz;
        P[0] = fmaf(wx, oxf, P[0]);
        P[1] = fmaf(wx, oyf, P[1]);
        P[2] = fmaf(wx, oz, P[2]);
        P[3] = fmaf(wy, oyf, P[3]);
        P[4] = fmaf(wy, oz, P[4]);
        P[5] = fmaf(wz, oz, P[5]);
    }
}

// one row of voters (fixed vz, oy) against receivers j in [JLO, JHI].  The
// weights depend on ox^2 only, so the voters at +ox and -ox are taken together
// and share each table load.  rA / rB / rC point at this thread's ox = 0 voter.
template <int R>
__device__ __forceinline__ void fold_partials(float (&P)[R][7], float (&tot)[R][6], float (&cmp)[R][6], int jlo,
                                              int jhi) {
#pragma unroll
    for (int j = 0; j < R; ++j) {
        if (j < jlo || j > jhi) continue;
        kahan_add(tot[j][0], cmp[j][0], P[j][0] + P[j][6]);
        kahan_add(tot[j][1], cmp[j][1], P[j][1]);
        kahan_add(tot[j][2], cmp[j][2], P[j][2]);
        kahan_add(tot[j][3], cmp[j][3], P[j][3] + P[j][6]);
        kahan_add(tot[j][4], cmp[j][4], P[j][4]);
        kahan_add(tot[j][5], cmp[j][5], P[j][5] + P[j][6]);
#pragma unroll
        for (int k = 0; k < 7; ++k) P[j][k] = 0.0f;
    }
}

template <int R, int JLO, int JHI, bool STICK, bool PLATE, bool BALL>
__device__ __forceinline__ void vote_row(const float4* __restrict__ rA, const float4* __restrict__ rB,
                                         const float* __restrict__ rC, const float4* __restrict__ tbl,
                                         const int (&zoff)[R], const float (&ozf)[R], float oyf, int L2y, int hw,
                                         float (&tot)[R][6], float (&cmp)[R][6], float (&Pp)[R][7]) {
#if TVGB_FOLD_PLANE
    float (&P)[R][7] = Pp;
#else
    (void)Pp;
    float P[R][7];
#pragma unroll
    for (int j = 0; j < R; ++j)
#pragma unroll
        for (int k = 0; k < 7; ++k) P[j][k] = 0.0f;
#endif
    const float4 Z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    {   // ox = 0
        const float4 A = STICK ? rA[0] : Z4, B = PLATE ? rB[0] : Z4;
        const float lb = BALL ? rC[0] : 0.0f;
        const float ub = A.y * oyf, vb = B.y * oyf;
        const int off = 2 * L2y;
#pragma unroll
        for (int j = JLO; j <= JHI; ++j) {
            const float4 ta = tbl[zoff[j] + off];
            const float4 tb = (PLATE || BALL) ? tbl[zoff[j] + off + 1] : Z4;
            vote_pair<STICK, PLATE, BALL>(A, B, lb, ub, vb, 0.0f, oyf, ozf[j], ta, tb, P[j]);
        }
    }
    float oxf = 1.0f;
    int off = 2 * (1 + L2y);
    int step = 6;                        // 2 * (2 ox + 1) for ox = 1
#pragma unroll kDUnroll
    for (int d = 1; d <= hw; ++d) {
        const float4 Ap = STICK ? rA[d] : Z4, Am = STICK ? rA[-d] : Z4;
        const float4 Bp = PLATE ? rB[d] : Z4, Bm = PLATE ? rB[-d] : Z4;
        const float lp = BALL ? rC[d] : 0.0f, lm = BALL ? rC[-d] : 0.0f;
        const float ubp = fmaf(Ap.x, oxf, Ap.y * oyf), ubm = fmaf(-Am.x, oxf, Am.y * oyf);
        const float vbp = fmaf(Bp.x, oxf, Bp.y * oyf), vbm = fmaf(-Bm.x, oxf, Bm.y * oyf);
#pragma unroll
        for (int j = JLO; j <= JHI; ++j) {
            const float4 ta = tbl[zoff[j] + off];
            const float4 tb = (PLATE || BALL) ? tbl[zoff[j] + off + 1] : Z4;
            vote_pair<STICK, PLATE, BALL>(Ap, Bp, lp, ubp, vbp, oxf, oyf, ozf[j], ta, tb, P[j]);
            vote_pair<STICK, PLATE, BALL>(Am, Bm, lm, ubm, vbm, -oxf, oyf, ozf[j], ta, tb, P[j]);
        }
        off += step;
        step += 4;
        oxf += 1.0f;
    }
#if !TVGB_FOLD_PLANE
    // fold the row partials into the per-voxel Kahan sums
    fold_partials<R>(P, tot, cmp, JLO, JHI);
#endif
}

template <int R, int JLO, int JHI, bool S, bool PL, bool BA>
__device__ __forceinline__ void row_if(int jlo, int jhi, const float4* rA, const float4* rB, const float* rC,
                                       const float4* tbl, const int (&zoff)[R], const float (&ozf)[R], float oyf,
                                       int L2y, int hw, float (&tot)[R][6], float (&cmp)[R][6], float (&P)[R][7]) {
    if (jlo == JLO && jhi == JHI)
        vote_row<R, JLO, JHI, S, PL, BA>(rA, rB, rC, tbl, zoff, ozf, oyf, L2y, hw, tot, cmp, P);
}

// every (jlo, jhi) with 0 <= jlo <= jhi < R
template <int R, int JLO, int JHI, bool S, bool PL, bool BA>
__device__ __forceinline__ void row_dispatch(int jlo, int jhi, const float4* rA, const float4* rB, const float* rC,
                                             const float4* tbl, const int (&zoff)[R], const float (&ozf)[R],
                                             float oyf, int L2y, int hw, float (&tot)[R][6], float (&cmp)[R][6],
                                             float (&P)[R][7]) {
    row_if<R, JLO, JHI, S, PL, BA>(jlo, jhi, rA, rB, rC, tbl, zoff, ozf, oyf, L2y, hw, tot, cmp, P);
    if constexpr (JHI + 1 < R)
        row_dispatch<R, JLO, JHI + 1, S, PL, BA>(jlo, jhi, rA, rB, rC, tbl, zoff, ozf, oyf, L2y, hw, tot, cmp, P);
    else if constexpr (JLO + 1 < R)
        row_dispatch<R, JLO + 1, JLO + 1, S, PL, BA>(jlo, jhi, rA, rB, rC, tbl, zoff, ozf, oyf, L2y, hw, tot, cmp, P);
}

__device__ __forceinline__ void write_receiver(const FastArgs& a, size_t idx, size_t n, const float* m6) {
    float* out = a.out;
    if (out) {
        if (a.out_layout == TVGB_LAYOUT_MAT3) {
            float* o = out + idx * 9;
            o[0] = m6[0]; o[1] = m6[1]; o[2] = m6[2];
            o[3] = m6[1]; o[4] = m6[3]; o[5] = m6[4];
            o[6] = m6[2]; o[7] = m6[4]; o[8] = m6[5];
        } else if (a.out_layout == TVGB_LAYOUT_SYM6) {
            float* o = out + idx * 6;
            for (int k = 0; k < 6; ++k) o[k] = m6[k];
        } else {
            for (int k = 0; k < 6; ++k) out[k * n + idx] = m6[k];
        }
    }
    if (a.evals || a.evecs) {
        float ev[3], v[9];
        if (a.precise_eig) {
            eig3_precise_d(m6[0], m6[1], m6[3], m6[2], m6[4], m6[5], ev, v, v + 3, v + 6);
        } else {
            eval3_d(m6[0], m6[1], m6[3], m6[2], m6[4], m6[5], ev[0], ev[1], ev[2]);
            if (a.evecs) evec3_d(m6[0], m6[1], m6[3], m6[2], m6[4], m6[5], ev, v, v + 3, v + 6);
        }
        if (a.evals) { a.evals[idx * 3] = ev[0]; a.evals[idx * 3 + 1] = ev[1]; a.evals[idx * 3 + 2] = ev[2]; }
        if (a.evecs) {
            if (a.evec_fmt == TVGB_EVEC_CARTESIAN) {
                for (int k = 0; k < 9; ++k) a.evecs[idx * 9 + k] = v[k];
            } else {
                float th, ph;
                to_spherical_d(v, th, ph); a.evecs[idx * 6] = th; a.evecs[idx * 6 + 1] = ph;
                to_spherical_d(v + 3, th, ph); a.evecs[idx * 6 + 2] = th; a.evecs[idx * 6 + 3] = ph;
                to_spherical_d(v + 6, th, ph); a.evecs[idx * 6 + 4] = th; a.evecs[idx * 6 + 5] = ph;
            }
        }
    }
}

// No term votes: every receiver's voted tensor is zero.  Writes the zero
// tensor and, where asked for, its eigendecomposition through the same
// epilogue as the vote kernels, so the outputs match a vote whose terms all
// contribute nothing.
__global__ void __launch_bounds__(256) k_vote3_none(FastArgs a) {
    const size_t n = size_t(a.s0) * a.s1 * a.s2, plane = size_t(a.s1) * a.s2;
    const size_t i1 = size_t(a.zr1) * plane;      // receivers of planes [zr0, zr1)
    const float zero6[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    for (size_t i = size_t(a.zr0) * plane + size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < i1;
         i += size_t(gridDim.x) * blockDim.x)
        write_receiver(a, i, n, zero6);
}

template <int R, bool STICK, bool PLATE, bool BALL>
__global__ void __launch_bounds__(VX * VY, TVGB_FAST_MINB) k_vote3_fast(FastArgs a) {
    extern __shared__ __align__(16) float4 smem[];
    const int hw = a.hw;
    const int nt = 3 * hw * hw + 1;          // radial table entries
    const int SW = VX + 2 * hw;              // staged row width
    const int SR = VY + a.rows - 1;          // staged rows
    float4* tbl = smem;                      // 2 * nt float4
    float4* sA = tbl + 2 * nt;               // SR * SW
    float4* sB = sA + (STICK ? SR * SW : 0);
    float* sC = reinterpret_cast<float*>(sB + (PLATE ? SR * SW : 0));
    const int tid = threadIdx.y * VX + threadIdx.x;
    const int nthr = VX * VY;

    for (int L2 = tid; L2 < nt; L2 += nthr) {
        float4 ea, eb;
        fast_radial_entry(a, L2, ea, eb);
        tbl[2 * L2] = ea;
        tbl[2 * L2 + 1] = eb;
    }

    int bx, by, bz;
    swizzled_block(bx, by, bz);
    const int x0 = bx * VX, y0 = by * VY, z0 = a.zr0 + bz * R;
    const int s0 = a.s0, s1 = a.s1, s2 = a.s2;
    const size_t plane = size_t(s1) * s2;

    float tot[R][6], cmp[R][6];
#pragma unroll
    for (int j = 0; j < R; ++j)
#pragma unroll
        for (int k = 0; k < 6; ++k) { tot[j][k] = 0.0f; cmp[j][k] = 0.0f; }

    const int vz_lo = max(0, z0 - hw), vz_hi = min(s0 - 1, z0 + R - 1 + hw);
    for (int vz = vz_lo; vz <= vz_hi; ++vz) {
        const int dzp = vz - z0;
        const int jlo = max(0, dzp - hw), jhi = min(R - 1, dzp + hw);
        int zoff[R];
        float ozf[R];
        float P[R][7];   // plane partials (TVGB_FOLD_PLANE); otherwise unused
#pragma unroll
        for (int j = 0; j < R; ++j) {
            const int oz = dzp - j;
            zoff[j] = 2 * oz * oz;
            ozf[j] = float(oz);
#pragma unroll
            for (int k = 0; k < 7; ++k) P[j][k] = 0.0f;
        }
        for (int oy0 = -hw; oy0 <= hw; oy0 += a.rows) {
            const int oy1 = min(hw, oy0 + a.rows - 1);
            const int nrows = VY + (oy1 - oy0);
            __syncthreads();   // previous stage fully consumed (and table built)
            // stage voter rows y0+oy0 .. y0+VY-1+oy1, columns x0-hw .. x0+VX-1+hw
            const int nst = nrows * SW;
            for (int e = tid; e < nst; e += nthr) {
                const int r = e / SW, c = e - r * SW;
                const int gy = y0 + oy0 + r, gx = x0 - hw + c;
                const bool in = (unsigned)gy < (unsigned)s1 && (unsigned)gx < (unsigned)s2;
                const size_t gi = size_t(vz) * plane + size_t(gy) * s2 + gx;
                if (STICK) sA[e] = in ? __ldg(a.A + gi) : make_float4(0, 0, 0, 0);
                if (PLATE) sB[e] = in ? __ldg(a.B + gi) : make_float4(0, 0, 0, 0);
                if (BALL) sC[e] = in ? __ldg(a.C + gi) : 0.0f;
            }
            __syncthreads();
            for (int oy = oy0; oy <= oy1; ++oy) {
                // a voter row outside the volume only holds zero records: skip it
                // (threadIdx.y is uniform within a warp, so is this branch)
                if ((unsigned)(y0 + int(threadIdx.y) + oy) >= (unsigned)s1) continue;
                const int rr = threadIdx.y + (oy - oy0);
                const int base = rr * SW + threadIdx.x + hw;   // column of ox = 0
                row_dispatch<R, 0, 0, STICK, PLATE, BALL>(jlo, jhi, sA + base, sB + base, sC + base, tbl, zoff, ozf,
                                                          float(oy), oy * oy, hw, tot, cmp, P);
            }
        }
#if TVGB_FOLD_PLANE
        fold_partials<R>(P, tot, cmp, jlo, jhi);
#endif
    }

    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= s2 || y >= s1) return;
    const size_t n = size_t(s0) * plane;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const int z = z0 + j;
        if (z >= a.zr1) break;
        float m6[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) m6[k] = tot[j][k];
        write_receiver(a, size_t(z) * plane + size_t(y) * s2 + x, n, m6);
    }
}

// ------------------------------------------------------------------ packed variant
// The same arithmetic as k_vote3_fast with the two z-neighbour receivers
// (j, j + 1) of a thread in the two lanes of Blackwell's packed FP32
// instructions (FFMA2 / FMUL2 / FADD2): both see the same voter, so the
// voter's components are broadcast and only the per-offset weights differ.
// Those depend on |o|^2 = ox^2 + oy^2 + oz^2, so at each voter plane the CTA
// builds a paired table indexed by ox^2 + oy^2 whose fields are already the
// (j, j + 1) float2 pairs: a 128-bit load yields two packed operands.  One
// packed instruction does two receivers' work, halving the FP32 issue slots
// per pair.  Measured (256^3, sigma 4): 55 -> 35 instructions per pair,
// issue active 77 % -> 49 %, but the FMA pipe, not issue, then bounds it
// (a packed instruction holds the pipe twice as long): 420.7 ms against
// 424.8 ms for k_vote3_fast.  With the ball term the packed kernel spills,
// so ball votes keep k_vote3_fast.  Accumulation (plane partials into
// per-voxel Kahan sums) is unchanged.
#ifndef TVGB_PACKED
#define TVGB_PACKED 1
#endif
#ifndef TVGB_PK_UNROLL
#define TVGB_PK_UNROLL 2
#endif
constexpr int kPkUnroll = TVGB_PK_UNROLL;

__device__ __forceinline__ float2 bc2(float x) { return make_float2(x, x); }

// paired-table entry: X = (c1, ctg), Y = (-2g, A0), Z = (-A1, Bp), W = (ball I, ball oo^T), each a (j, j+1) pair
template <bool STICK, bool PLATE, bool BALL>
__device__ __forceinline__ void vote_pair_pk(const float4& A, const float4& B, float lb, float ub, float vb,
                                             const float2& ox2, const float2& oy2, const float2& oz2, const float4& X,
                                             const float4& Y, const float4& Z, const float4& W, float2 (&P)[7]) {
    const float2 F2n = make_float2(Y.x, Y.y);
    if (STICK) {
        const float2 u = __ffma2_rn(bc2(A.z), oz2, bc2(ub));            // q . o
        const float2 kn = __fmul2_rn(u, F2n);                             // -2 (q.o) / |o|^2
        const float2 rx = __ffma2_rn(kn, ox2, bc2(A.x));
        const float2 ry = __ffma2_rn(kn, oy2, bc2(A.y));
        const float2 rz = __ffma2_rn(kn, oz2, bc2(A.z));
        const float2 eta = __ffma2_rn(make_float2(X.z, X.w), __fmul2_rn(u, u), make_float2(X.x, X.y));
        const float2 term = __fmul2_rn(bc2(A.w), eta);
        const float2 t0 = __fmul2_rn(term, rx), t1 = __fmul2_rn(term, ry), t2 = __fmul2_rn(term, rz);
        P[0] = __ffma2_rn(t0, rx, P[0]);
        P[1] = __ffma2_rn(t0, ry, P[1]);
        P[2] = __ffma2_rn(t0, rz, P[2]);
        P[3] = __ffma2_rn(t1, ry, P[3]);
        P[4] = __ffma2_rn(t1, rz, P[4]);
        P[5] = __ffma2_rn(t2, rz, P[5]);
    }
    if (PLATE) {
        const float2 v = __ffma2_rn(bc2(B.z), oz2, bc2(vb));            // n . o
        const float2 kn = __fmul2_rn(v, F2n);
        const float2 mx = __ffma2_rn(kn, ox2, bc2(B.x));                  // m = R n
        const float2 my = __ffma2_rn(kn, oy2, bc2(B.y));
        const float2 mz = __ffma2_rn(kn, oz2, bc2(B.z));
        const float2 hx = __ffma2_rn(v, mx, ox2);                         // h = o + v m
        const float2 hy = __ffma2_rn(v, my, oy2);
        const float2 hz = __ffma2_rn(v, mz, oz2);
        const float2 cA = __ffma2_rn(make_float2(Z.x, Z.y), __fmul2_rn(v, v), make_float2(Y.z, Y.w));
        const float2 nsA = __fmul2_rn(bc2(-B.w), cA);                     // -sA
        const float2 sB = __fmul2_rn(bc2(B.w), make_float2(Z.z, Z.w));
        P[6] = __fadd2_rn(P[6], nsA);                                     // the identity term, negated
        const float2 ax = __fmul2_rn(nsA, mx), ay = __fmul2_rn(nsA, my), az = __fmul2_rn(nsA, mz);
        const float2 bx = __fmul2_rn(sB, hx), by = __fmul2_rn(sB, hy), bz = __fmul2_rn(sB, hz);
        P[0] = __ffma2_rn(bx, hx, __ffma2_rn(ax, mx, P[0]));
        P[1] = __ffma2_rn(bx, hy, __ffma2_rn(ax, my, P[1]));
        P[2] = __ffma2_rn(bx, hz, __ffma2_rn(ax, mz, P[2]));
        P[3] = __ffma2_rn(by, hy, __ffma2_rn(ay, my, P[3]));
        P[4] = __ffma2_rn(by, hz, __ffma2_rn(ay, mz, P[4]));
        P[5] = __ffma2_rn(bz, hz, __ffma2_rn(az, mz, P[5]));
    }
    if (BALL) {
        P[6] = __ffma2_rn(bc2(-lb), make_float2(W.x, W.y), P[6]);
        const float2 wb = __fmul2_rn(bc2(lb), make_float2(W.z, W.w));
        const float2 wx = __fmul2_rn(wb, ox2), wy = __fmul2_rn(wb, oy2), wz = __fmul2_rn(wb, oz2);
        P[0] = __ffma2_rn(wx, ox2, P[0]);
        P[1] = __ffma2_rn(wx, oy2, P[1]);
        P[2] = __ffma2_rn(wx, oz2, P[2]);
        P[3] = __ffma2_rn(wy, oy2, P[3]);
        P[4] = __ffma2_rn(wy, oz2, P[4]);
        P[5] = __ffma2_rn(wz, oz2, P[5]);
    }
}

// one voter row (fixed vz, oy) against the receiver pair of this paired table
template <bool STICK, bool PLATE, bool BALL>
__device__ __forceinline__ void vote_row_pk(const float4* __restrict__ rA, const float4* __restrict__ rB,
                                            const float* __restrict__ rC, const float4* __restrict__ pt, int NQ,
                                            const float2& oz2, float oyf, int L2y, int hw, float2 (&P)[7]) {
    const float4 Z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float2 oy2 = bc2(oyf);
    {   // ox = 0
        const float4 A = STICK ? rA[0] : Z4, B = PLATE ? rB[0] : Z4;
        const float lb = BALL ? rC[0] : 0.0f;
        const float4* e = pt + NQ * L2y;
        const float4 X = e[0], Y = e[1], Zt = e[2], W = BALL ? e[3] : Z4;
        vote_pair_pk<STICK, PLATE, BALL>(A, B, lb, A.y * oyf, B.y * oyf, bc2(0.0f), oy2, oz2, X, Y, Zt, W, P);
    }
    float oxf = 1.0f;
    int e2 = 1 + L2y;
    int step = 3;                        // (ox + 1)^2 - ox^2 for ox = 1
#pragma unroll kPkUnroll
    for (int d = 1; d <= hw; ++d) {
        const float4 Ap = STICK ? rA[d] : Z4, Am = STICK ? rA[-d] : Z4;
        const float4 Bp = PLATE ? rB[d] : Z4, Bm = PLATE ? rB[-d] : Z4;
        const float lp = BALL ? rC[d] : 0.0f, lm = BALL ? rC[-d] : 0.0f;
        const float4* e = pt + NQ * e2;
        const float4 X = e[0], Y = e[1], Zt = e[2], W = BALL ? e[3] : Z4;
        const float2 oxp = bc2(oxf), oxm = bc2(-oxf);
        vote_pair_pk<STICK, PLATE, BALL>(Ap, Bp, lp, fmaf(Ap.x, oxf, Ap.y * oyf), fmaf(Bp.x, oxf, Bp.y * oyf), oxp, oy2,
                                         oz2, X, Y, Zt, W, P);
        vote_pair_pk<STICK, PLATE, BALL>(Am, Bm, lm, fmaf(-Am.x, oxf, Am.y * oyf), fmaf(-Bm.x, oxf, Bm.y * oyf), oxm,
                                         oy2, oz2, X, Y, Zt, W, P);
        e2 += step;
        step += 2;
        oxf += 1.0f;
    }
}

// both receiver pairs of a thread on one voter row: each voter record and its
// (q.o, n.o) partial sums are read / formed once for the two pairs
#ifndef TVGB_PK_FUSE
#define TVGB_PK_FUSE 1         // both receiver pairs per voter-row pass
#endif
#ifndef TVGB_PK_BALL
#define TVGB_PK_BALL 1         // the packed kernel also for votes with the ball term
#endif
#ifndef TVGB_PK2_UNROLL
#define TVGB_PK2_UNROLL 3      // unroll factor of that pass's +-ox loop
#endif
constexpr int kPk2Unroll = TVGB_PK2_UNROLL;
template <bool STICK, bool PLATE, bool BALL>
__device__ __forceinline__ void vote_row_pk2(const float4* __restrict__ rA, const float4* __restrict__ rB,
                                             const float* __restrict__ rC, const float4* __restrict__ pt0,
                                             const float4* __restrict__ pt1, int NQ, const float2& oz20,
                                             const float2& oz21, float oyf, int L2y, int hw, float2 (&P0)[7],
                                             float2 (&P1)[7]) {
    const float4 Z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float2 oy2 = bc2(oyf);
    {   // ox = 0
        const float4 A = STICK ? rA[0] : Z4, B = PLATE ? rB[0] : Z4;
        const float lb = BALL ? rC[0] : 0.0f;
        const float ub = A.y * oyf, vb = B.y * oyf;
        const float4* e0 = pt0 + NQ * L2y;
        const float4* e1 = pt1 + NQ * L2y;
        vote_pair_pk<STICK, PLATE, BALL>(A, B, lb, ub, vb, bc2(0.0f), oy2, oz20, e0[0], e0[1], e0[2],
                                         BALL ? e0[3] : Z4, P0);
        vote_pair_pk<STICK, PLATE, BALL>(A, B, lb, ub, vb, bc2(0.0f), oy2, oz21, e1[0], e1[1], e1[2],
                                         BALL ? e1[3] : Z4, P1);
    }
    float oxf = 1.0f;
    int e2 = 1 + L2y;
    int step = 3;                        // (ox + 1)^2 - ox^2 for ox = 1
#pragma unroll kPk2Unroll
    for (int d = 1; d <= hw; ++d) {
        const float4 Ap = STICK ? rA[d] : Z4, Am = STICK ? rA[-d] : Z4;
        const float4 Bp = PLATE ? rB[d] : Z4, Bm = PLATE ? rB[-d] : Z4;
        const float lp = BALL ? rC[d] : 0.0f, lm = BALL ? rC[-d] : 0.0f;
        const float ubp = fmaf(Ap.x, oxf, Ap.y * oyf), ubm = fmaf(-Am.x, oxf, Am.y * oyf);
        const float vbp = fmaf(Bp.x, oxf, Bp.y * oyf), vbm = fmaf(-Bm.x, oxf, Bm.y * oyf);
        const float2 oxp = bc2(oxf), oxm = bc2(-oxf);
        {
            const float4* e = pt0 + NQ * e2;
            const float4 X = e[0], Y = e[1], Zt = e[2], W = BALL ? e[3] : Z4;
            vote_pair_pk<STICK, PLATE, BALL>(Ap, Bp, lp, ubp, vbp, oxp, oy2, oz20, X, Y, Zt, W, P0);
            vote_pair_pk<STICK, PLATE, BALL>(Am, Bm, lm, ubm, vbm, oxm, oy2, oz20, X, Y, Zt, W, P0);
        }
        {
            const float4* e = pt1 + NQ * e2;
            const float4 X = e[0], Y = e[1], Zt = e[2], W = BALL ? e[3] : Z4;
            vote_pair_pk<STICK, PLATE, BALL>(Ap, Bp, lp, ubp, vbp, oxp, oy2, oz21, X, Y, Zt, W, P1);
            vote_pair_pk<STICK, PLATE, BALL>(Am, Bm, lm, ubm, vbm, oxm, oy2, oz21, X, Y, Zt, W, P1);
        }
        e2 += step;
        step += 2;
        oxf += 1.0f;
    }
}

template <bool STICK, bool PLATE, bool BALL, bool TBL>
__global__ void __launch_bounds__(VX * VY, TVGB_FAST_MINB) k_vote3_pk(FastArgs a) {
    constexpr int R = 4;
    constexpr int NQ = BALL ? 4 : 3;         // float4 per paired-table entry
    extern __shared__ __align__(16) float4 smem[];
    const int hw = a.hw;
    const int ne = 2 * hw * hw + 1;          // paired-table entries (ox^2 + oy^2)
    const int SW = VX + 2 * hw;
    const int SR = VY + a.rows - 1;
    // TBL: the radial table (2 nt float4) in shared memory.  Without it (the largest windows) each plane's
    // paired table takes its entries from fast_radial_entry directly (4 ne evaluations per plane and CTA,
    // under 1% of the plane's work), which leaves room for two CTAs per SM with several voter rows per stage
    const int nt = TBL ? 3 * hw * hw + 1 : 0;
    float4* tbl = smem;                      // 2 nt
    float4* ptab = tbl + 2 * nt;             // 2 pairs x ne x NQ
    float4* sA = ptab + 2 * ne * NQ;
    float4* sB = sA + (STICK ? SR * SW : 0);
    float* sC = reinterpret_cast<float*>(sB + (PLATE ? SR * SW : 0));
    const int tid = threadIdx.y * VX + threadIdx.x;
    const int nthr = VX * VY;
    for (int L2 = tid; L2 < nt; L2 += nthr) {
        float4 ea, eb;
        fast_radial_entry(a, L2, ea, eb);
        tbl[2 * L2] = ea;
        tbl[2 * L2 + 1] = eb;
    }
    int bx, by, bz;
    swizzled_block(bx, by, bz);
    const int x0 = bx * VX, y0 = by * VY, z0 = a.zr0 + bz * R;
    const int s0 = a.s0, s1 = a.s1, s2 = a.s2;
    const size_t plane = size_t(s1) * s2;
    float tot[R][6], cmp[R][6];
#pragma unroll
    for (int j = 0; j < R; ++j)
#pragma unroll
        for (int k = 0; k < 6; ++k) { tot[j][k] = 0.0f; cmp[j][k] = 0.0f; }

    const int vz_lo = max(0, z0 - hw), vz_hi = min(s0 - 1, z0 + R - 1 + hw);
    for (int vz = vz_lo; vz <= vz_hi; ++vz) {
        const int dzp = vz - z0;
        float2 P[2][7];
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
            for (int k = 0; k < 7; ++k) P[p][k] = make_float2(0.0f, 0.0f);
        // receiver pair p = (2p, 2p + 1): oz = dzp - j; a pair with neither receiver in reach is skipped
        bool pv[2];
        float2 oz2[2];
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const int oa = dzp - 2 * p, ob = oa - 1;
            pv[p] = abs(oa) <= hw || abs(ob) <= hw;
            oz2[p] = make_float2(float(oa), float(ob));
        }
        for (int oy0 = -hw; oy0 <= hw; oy0 += a.rows) {
            const int oy1 = min(hw, oy0 + a.rows - 1);
            const int nrows = VY + (oy1 - oy0);
            __syncthreads();   // previous stage fully consumed (and table built)
            if (oy0 == -hw) {  // this plane's paired table (zero weights for a receiver out of reach)
                for (int i = tid; i < 2 * ne; i += nthr) {
                    const int p = i / ne, e = i - p * ne;
                    const int oa = dzp - 2 * p, ob = oa - 1;
                    float4 ta = make_float4(0, 0, 0, 0), tba = ta, tb = ta, tbb = ta;
                    if (abs(oa) <= hw) {
                        if (TBL) { ta = tbl[2 * (e + oa * oa)]; tba = tbl[2 * (e + oa * oa) + 1]; }
                        else fast_radial_entry(a, e + oa * oa, ta, tba);
                    }
                    if (abs(ob) <= hw) {
                        if (TBL) { tb = tbl[2 * (e + ob * ob)]; tbb = tbl[2 * (e + ob * ob) + 1]; }
                        else fast_radial_entry(a, e + ob * ob, tb, tbb);
                    }
                    float4* q = ptab + (size_t(p) * ne + e) * NQ;
                    // radial entry a = (c1, ct g, 2 g, A0), b = (A1, Bp, ball I, ball oo^T)
                    q[0] = make_float4(ta.x, tb.x, ta.y, tb.y);
                    q[1] = make_float4(-ta.z, -tb.z, ta.w, tb.w);
                    q[2] = make_float4(-tba.x, -tbb.x, tba.y, tbb.y);
                    if (BALL) q[3] = make_float4(tba.z, tbb.z, tba.w, tbb.w);
                }
            }
            const int nst = nrows * SW;
            for (int e = tid; e < nst; e += nthr) {
                const int r = e / SW, c = e - r * SW;
                const int gy = y0 + oy0 + r, gx = x0 - hw + c;
                const bool in = (unsigned)gy < (unsigned)s1 && (unsigned)gx < (unsigned)s2;
                const size_t gi = size_t(vz) * plane + size_t(gy) * s2 + gx;
                if (STICK) sA[e] = in ? __ldg(a.A + gi) : make_float4(0, 0, 0, 0);
                if (PLATE) sB[e] = in ? __ldg(a.B + gi) : make_float4(0, 0, 0, 0);
                if (BALL) sC[e] = in ? __ldg(a.C + gi) : 0.0f;
            }
            __syncthreads();
            for (int oy = oy0; oy <= oy1; ++oy) {
                if ((unsigned)(y0 + int(threadIdx.y) + oy) >= (unsigned)s1) continue;   // warp-uniform
                const int rr = threadIdx.y + (oy - oy0);
                const int base = rr * SW + threadIdx.x + hw;
#if TVGB_PK_FUSE
                if (pv[0] && pv[1]) {
                    vote_row_pk2<STICK, PLATE, BALL>(sA + base, sB + base, sC + base, ptab, ptab + size_t(ne) * NQ, NQ,
                                                     oz2[0], oz2[1], float(oy), oy * oy, hw, P[0], P[1]);
                    continue;
                }
#endif
#pragma unroll
                for (int p = 0; p < 2; ++p)
                    if (pv[p])
                        vote_row_pk<STICK, PLATE, BALL>(sA + base, sB + base, sC + base, ptab + size_t(p) * ne * NQ,
                                                        NQ, oz2[p], float(oy), oy * oy, hw, P[p]);
            }
        }
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const float2 d6 = P[p][6];   // negated identity term
            kahan_add(tot[2 * p][0], cmp[2 * p][0], P[p][0].x - d6.x);
            kahan_add(tot[2 * p][1], cmp[2 * p][1], P[p][1].x);
            kahan_add(tot[2 * p][2], cmp[2 * p][2], P[p][2].x);
            kahan_add(tot[2 * p][3], cmp[2 * p][3], P[p][3].x - d6.x);
            kahan_add(tot[2 * p][4], cmp[2 * p][4], P[p][4].x);
            kahan_add(tot[2 * p][5], cmp[2 * p][5], P[p][5].x - d6.x);
            kahan_add(tot[2 * p + 1][0], cmp[2 * p + 1][0], P[p][0].y - d6.y);
            kahan_add(tot[2 * p + 1][1], cmp[2 * p + 1][1], P[p][1].y);
            kahan_add(tot[2 * p + 1][2], cmp[2 * p + 1][2], P[p][2].y);
            kahan_add(tot[2 * p + 1][3], cmp[2 * p + 1][3], P[p][3].y - d6.y);
            kahan_add(tot[2 * p + 1][4], cmp[2 * p + 1][4], P[p][4].y);
            kahan_add(tot[2 * p + 1][5], cmp[2 * p + 1][5], P[p][5].y - d6.y);
        }
    }

    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= s2 || y >= s1) return;
    const size_t n = size_t(s0) * plane;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const int z = z0 + j;
        if (z >= a.zr1) break;
        float m6[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) m6[k] = tot[j][k];
        write_receiver(a, size_t(z) * plane + size_t(y) * s2 + x, n, m6);
    }
}

// ------------------------------------------------------------------ generic kernel
// One receiver per thread, straight gather with the reference's arithmetic;
// handles any power, a literal samples-point plate when samples < power + 2
// (with the reference's (u, v) basis, tensorvote.h:2467-2469), the ball term
// for any power (Gauss-Legendre x uniform-phi rule, exact for the integrand)
// and ATV (tensorvote.h:710, :2640).

struct GenArgs {
    const float4* A;
    const float4* B;
    const float* C;
    const float4* L;
    const float4* E1;
    int s0, s1, s2, hw;
    float sig1, sig2;
    unsigned power;
    int plate_m;          // samples used for the plate (literal rule)
    int stick, plate, ball, atv;
    int ng, np;           // ball rule sizes
    const float* gl;      // Gauss-Legendre nodes/weights (2 * ng floats), device
    FastArgs o;           // output description
};

__device__ __forceinline__ void stick_pair(float* m, float dx, float dy, float dz, float c1, float c2, float qx, float qy,
                                           float qz, unsigned power, float scale) {
    const float qTd = qx * dx + qy * dy + qz * dz;
    const float qTd2 = qTd * qTd;
    float eta;
    if (power == 1) eta = c1 * (1.0f - qTd2) + c2 * qTd2;
    else {
        const float t1 = 1.0f - qTd2, t2 = qTd2;
        float e1 = t1, e2 = t2;
        for (unsigned i = 1; i < power; ++i) { e1 *= t1; e2 *= t2; }
        eta = c1 * e1 + c2 * e2;
    }
    const float rx = qx - 2.0f * qTd * dx, ry = qy - 2.0f * qTd * dy, rz = qz - 2.0f * qTd * dz;
    const float term = scale * eta;
    m[0] += term * rx * rx; m[1] += term * rx * ry; m[2] += term * rx * rz;
    m[3] += term * ry * ry; m[4] += term * ry * rz; m[5] += term * rz * rz;
}

// atv (tensorvote.h:710) with atv_H (:607); m gets xx, xy, xz, yy, yz, zz
__device__ __forceinline__ void atv_pair(float* m, float l0, float l1, float l2, float4 e1, float4 e2, float rx, float ry,
                                         float rz, float sigma) {
    const float dist = sqrtf(rx * rx + ry * ry + rz * rz);
    const float c = sigma == 0.0f ? (dist > 1e-12f ? 0.0f : 1.0f) : expf(-(dist * dist) / (sigma * sigma));
    float dx = 0.0f, dy = 0.0f, dz = 0.0f;
    if (dist != 0.0f) { dx = rx / dist; dy = ry / dist; dz = rz / dist; }
    const float R00 = 1.0f - 2.0f * dx * dx, R01 = -2.0f * dx * dy, R02 = -2.0f * dx * dz;
    const float R11 = 1.0f - 2.0f * dy * dy, R12 = -2.0f * dy * dz, R22 = 1.0f - 2.0f * dz * dz;
    float T[3][6];
    T[0][0] = e2.x * e2.x; T[0][1] = e2.x * e2.y; T[0][2] = e2.x * e2.z; T[0][3] = e2.y * e2.y; T[0][4] = e2.y * e2.z; T[0][5] = e2.z * e2.z;
    T[1][0] = e1.x * e1.x + T[0][0]; T[1][1] = e1.x * e1.y + T[0][1]; T[1][2] = e1.x * e1.z + T[0][2];
    T[1][3] = e1.y * e1.y + T[0][3]; T[1][4] = e1.y * e1.z + T[0][4]; T[1][5] = e1.z * e1.z + T[0][5];
    T[2][0] = 1; T[2][1] = 0; T[2][2] = 0; T[2][3] = 1; T[2][4] = 0; T[2][5] = 1;
    const float s[3] = {l2 - l1, l1 - l0, l0};
    const float inv[3] = {1.0f / 3.0f, 1.0f / 4.0f, 1.0f / 5.0f};
    float H[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float* t = T[k];   // xx xy xz yy yz zz
        const float tvx = t[0] * dx + t[1] * dy + t[2] * dz;
        const float tvy = t[1] * dx + t[3] * dy + t[4] * dz;
        const float tvz = t[2] * dx + t[4] * dy + t[5] * dz;
        const float vTv = dx * tvx + dy * tvy + dz * tvz;
        const float tv[6] = {tvx * tvx, tvx * tvy, tvx * tvz, tvy * tvy, tvy * tvz, tvz * tvz};
#pragma unroll
        for (int i = 0; i < 6; ++i) H[i] += s[k] * (t[i] - inv[k] * (t[i] * vTv + 2.0f * tv[i]));
    }
    // V = c R H R
    const float Hm[3][3] = {{H[0], H[1], H[2]}, {H[1], H[3], H[4]}, {H[2], H[4], H[5]}};
    const float Rm[3][3] = {{R00, R01, R02}, {R01, R11, R12}, {R02, R12, R22}};
    float M[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) M[i][j] = Rm[i][0] * Hm[0][j] + Rm[i][1] * Hm[1][j] + Rm[i][2] * Hm[2][j];
    const int ii[6] = {0, 0, 0, 1, 1, 2}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int q = 0; q < 6; ++q)
        m[q] += c * (M[ii[q]][0] * Rm[0][jj[q]] + M[ii[q]][1] * Rm[1][jj[q]] + M[ii[q]][2] * Rm[2][jj[q]]);
}

__global__ void __launch_bounds__(128) k_vote3_generic(GenArgs g) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int z = blockIdx.z;
    if (x >= g.s2) return;
    const int hw = g.hw;
    const size_t plane = size_t(g.s1) * g.s2;
    const float inv1 = g.sig1 > 0.0f ? 1.0f / (g.sig1 * g.sig1) : 0.0f;
    const float inv2 = g.sig2 > 0.0f ? 1.0f / (g.sig2 * g.sig2) : 0.0f;
    float acc[6] = {0, 0, 0, 0, 0, 0};
    for (int dw = -hw; dw <= hw; ++dw) {
        const int r0 = z + dw;
        if ((unsigned)r0 >= (unsigned)g.s0) continue;
        float row[6] = {0, 0, 0, 0, 0, 0};
        for (int dv = -hw; dv <= hw; ++dv) {
            const int r1 = y + dv;
            if ((unsigned)r1 >= (unsigned)g.s1) continue;
            for (int du = -hw; du <= hw; ++du) {
                const int r2 = x + du;
                if ((unsigned)r2 >= (unsigned)g.s2) continue;
                const size_t b = size_t(r0) * plane + size_t(r1) * g.s2 + r2;
                if (g.atv) {
                    const float4 L = g.L[b];
                    atv_pair(row, L.x, L.y, L.z, g.E1[b], g.A[b], float(du), float(dv), float(dw), g.sig1);
                    continue;
                }
                const float l2 = float(du * du + dv * dv + dw * dw);
                float dx = 0.0f, dy = 0.0f, dz = 0.0f;
                if (l2 != 0.0f) { const float L = sqrtf(l2); dx = float(du) / L; dy = float(dv) / L; dz = float(dw) / L; }
                const float c1 = g.sig1 == 0.0f ? (l2 > 1e-12f ? 0.0f : 1.0f) : expf(-l2 * inv1);
                const float c2 = g.sig2 == 0.0f ? (l2 > 1e-12f ? 0.0f : 1.0f) : expf(-l2 * inv2);
                if (g.stick) {
                    const float4 A = g.A[b];
                    stick_pair(row, dx, dy, dz, c1, c2, A.x, A.y, A.z, g.power, A.w);
                }
                if (g.plate) {
                    const float4 B = g.B[b];
                    if (B.w != 0.0f) {
                        const float ax = fabsf(B.z) < 0.999f ? 0.0f : 1.0f, az = fabsf(B.z) < 0.999f ? 1.0f : 0.0f;
                        // u = normalize(cross(a, n)), v = cross(n, u)   (tensorvote.h:2467-2469)
                        float ux = 0.0f * B.z - az * B.y, uy = az * B.x - ax * B.z, uz = ax * B.y - 0.0f * B.x;
                        const float ul = ux * ux + uy * uy + uz * uz;
                        if (ul > 0.0f) { const float il = rsqrtf(ul); ux *= il; uy *= il; uz *= il; }
                        const float vx = B.y * uz - B.z * uy, vy = B.z * ux - B.x * uz, vz = B.x * uy - B.y * ux;
                        const float db = 3.14159265358979323846f / float(g.plate_m);
                        float p[6] = {0, 0, 0, 0, 0, 0};
                        for (int i = 0; i < g.plate_m; ++i) {
                            float sb, cb;
                            sincosf(db * float(i), &sb, &cb);
                            stick_pair(p, dx, dy, dz, c1, c2, cb * ux + sb * vx, cb * uy + sb * vy, cb * uz + sb * vz,
                                       g.power, 1.0f);
                        }
                        const float sw = B.w * db * (1.0f / 3.14159265358979323846f);
                        for (int k = 0; k < 6; ++k) row[k] += sw * p[k];
                    }
                }
                if (g.ball) {
                    const float lb = g.C[b];
                    if (lb != 0.0f) {
                        float p[6] = {0, 0, 0, 0, 0, 0};
                        for (int i = 0; i < g.ng; ++i) {
                            const float ct = g.gl[i], wgt = g.gl[g.ng + i], st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
                            for (int k = 0; k < g.np; ++k) {
                                float sp, cp;
                                sincosf(6.28318530717958647692f * float(k) / float(g.np), &sp, &cp);
                                stick_pair(p, dx, dy, dz, c1, c2, st * cp, st * sp, ct, g.power,
                                           wgt * (6.28318530717958647692f / float(g.np)));
                            }
                        }
                        const float sw = lb * (1.0f / (4.0f * 3.14159265358979323846f));
                        for (int k = 0; k < 6; ++k) row[k] += sw * p[k];
                    }
                }
            }
        }
        for (int k = 0; k < 6; ++k) acc[k] += row[k];
    }
    write_receiver(g.o, size_t(z) * plane + size_t(y) * g.s2 + x, size_t(g.s0) * plane, acc);
}

// ------------------------------------------------------------------ host side

static double factorial_d(unsigned n) {
    double f = 1;
    for (unsigned i = 1; i <= n; i++) f *= i;
    return f;
}

// sticknorm3 (tensorvote.h:1163), evaluated with the reference's float steps
static float sticknorm3_f(float s1, float s2, unsigned p) {
    const double pi = 3.14159265358979323846;
    const float pi_term = float(pi * std::sqrt(pi) / 2.0);
    const float sig1_3 = s1 * s1 * s1, sig2_3 = s2 * s2 * s2;
    const float num1 = float(std::pow(2.0, double(2 * p + 1)) * factorial_d(p) * factorial_d(p));
    const float num2 = 2.0f;
    const float den1 = float(factorial_d(2 * p + 1));
    const float den2 = float(2 * p + 1);
    return pi_term * ((sig1_3 * num1 / den1) + (sig2_3 * num2 / den2));
}

static void gauss_legendre(int n, double* x, double* w) {
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < n; ++i) {
        double z = std::cos(pi * (i + 0.75) / (n + 0.5)), pp = 0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1, p2 = 0;
            for (int j = 0; j < n; ++j) { const double p3 = p2; p2 = p1; p1 = ((2 * j + 1) * z * p2 - j * p3) / (j + 1); }
            pp = n * (z * p1 - p2) / (z * z - 1);
            const double z1 = z;
            z = z1 - p1 / pp;
            if (std::fabs(z - z1) < 1e-15) break;
        }
        x[i] = z;
        w[i] = 2 / ((1 - z * z) * pp * pp);
    }
}

template <int R, bool S, bool P, bool B>
static int launch_fast_t(const FastArgs& a, cudaStream_t st) {
    const int hw = a.hw;
    const int nt = 3 * hw * hw + 1;
    const int SW = VX + 2 * hw;
    const int SR = VY + a.rows - 1;
    const size_t smem = size_t(2 * nt) * 16 + (S ? size_t(SR) * SW * 16 : 0) + (P ? size_t(SR) * SW * 16 : 0) +
                        (B ? size_t(SR) * SW * 4 : 0);
    TVGB_CUDA(cudaFuncSetAttribute(k_vote3_fast<R, S, P, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    dim3 grid(ceil_div(a.s2, VX), ceil_div(a.s1, VY), ceil_div(size_t(a.zr1 - a.zr0), R));
    {
        KernelTimer kt_("k_vote3_fast", st);
        k_vote3_fast<R, S, P, B><<<grid, dim3(VX, VY), smem, st>>>(a);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    return TVGB_OK;
}

constexpr int FAST_R = TVGB_FAST_R;

static size_t fast_smem(int hw, int rows, bool S, bool P, bool B) {
    const int nt = 3 * hw * hw + 1, SW = VX + 2 * hw, SR = VY + rows - 1;
    return size_t(2 * nt) * 16 + (S ? size_t(SR) * SW * 16 : 0) + (P ? size_t(SR) * SW * 16 : 0) +
           (B ? size_t(SR) * SW * 4 : 0);
}

template <bool S, bool P, bool B, bool T>
static int launch_pk_tt(const FastArgs& a, size_t smem, cudaStream_t st) {
    TVGB_CUDA(cudaFuncSetAttribute(k_vote3_pk<S, P, B, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    dim3 grid(ceil_div(a.s2, VX), ceil_div(a.s1, VY), ceil_div(size_t(a.zr1 - a.zr0), 4));
    {
        KernelTimer kt_("k_vote3_fast", st);
        k_vote3_pk<S, P, B, T><<<grid, dim3(VX, VY), smem, st>>>(a);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    return TVGB_OK;
}

template <bool S, bool P, bool B>
static int launch_pk_t(const FastArgs& a, size_t smem, bool tbl, cudaStream_t st) {
    return tbl ? launch_pk_tt<S, P, B, true>(a, smem, st) : launch_pk_tt<S, P, B, false>(a, smem, st);
}

static size_t pk_smem(int hw, int rows, bool S, bool P, bool B, bool tbl) {
    const size_t ne = size_t(2) * hw * hw + 1, nt = size_t(3) * hw * hw + 1;
    return fast_smem(hw, rows, S, P, B) - (tbl ? 0 : 2 * nt * 16) + 2 * ne * (B ? 4 : 3) * 16;
}

static int launch_none(const FastArgs& a, cudaStream_t st) {
    const size_t n = size_t(a.zr1 - a.zr0) * a.s1 * a.s2;
    if (n == 0) return TVGB_OK;
    const size_t blocks = std::min<size_t>((n + 255) / 256, 152 * 8);
    {
        KernelTimer kt_("k_vote3_none", st);
        k_vote3_none<<<unsigned(blocks), 256, 0, st>>>(a);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    return TVGB_OK;
}

static int launch_fast(FastArgs a, bool S, bool P, bool B, cudaStream_t st) {
    if (a.zr1 <= a.zr0) { a.zr0 = 0; a.zr1 = a.s0; }   // every receiver plane
    if (a.zr1 <= a.zr0) return TVGB_OK;
    if (!S && !P && !B) return launch_none(a, st);
    // rows per stage: the largest count that keeps TVGB_FAST_MINB CTAs per SM
    const int w = 2 * a.hw + 1;
    const size_t budget = (TVGB_FAST_MINB >= 3 ? 72 : 100) * 1024;
    if (TVGB_PACKED && FAST_R == 4 && (TVGB_PK_BALL || !B)) {
        // two CTAs per SM: 228 KB of shared memory less 1 KB reserved per CTA.  The radial table stays in shared
        // memory unless leaving it out lets a stage hold more voter rows
        const size_t pk_budget = (TVGB_FAST_MINB >= 3 ? 72 : 112) * 1024;
        int rows_t = w, rows_n = w;
        while (rows_t > 1 && pk_smem(a.hw, rows_t, S, P, B, true) > pk_budget) rows_t = (rows_t + 1) / 2;
        while (rows_n > 1 && pk_smem(a.hw, rows_n, S, P, B, false) > pk_budget) rows_n = (rows_n + 1) / 2;
        const bool tbl = rows_t >= rows_n && pk_smem(a.hw, rows_t, S, P, B, true) <= pk_budget;
        const int rows = tbl ? rows_t : rows_n;
        const size_t smem = pk_smem(a.hw, rows, S, P, B, tbl);
        if (smem <= 200 * 1024) {
            a.rows = rows;
            const int code = (S ? 4 : 0) | (P ? 2 : 0) | (B ? 1 : 0);
            switch (code) {
                case 4: return launch_pk_t<true, false, false>(a, smem, tbl, st);
                case 2: return launch_pk_t<false, true, false>(a, smem, tbl, st);
                case 6: return launch_pk_t<true, true, false>(a, smem, tbl, st);
                case 7: return launch_pk_t<true, true, true>(a, smem, tbl, st);
                case 5: return launch_pk_t<true, false, true>(a, smem, tbl, st);
                case 3: return launch_pk_t<false, true, true>(a, smem, tbl, st);
                case 1: return launch_pk_t<false, false, true>(a, smem, tbl, st);
                default: return TVGB_OK;
            }
        }
    }
    int rows = w;
    while (rows > 1 && fast_smem(a.hw, rows, S, P, B) > budget) rows = (rows + 1) / 2;
    if (fast_smem(a.hw, rows, S, P, B) > 200 * 1024) {
        set_error("vote window too large for the shared-memory tile (w = %d)", w);
        return TVGB_ERR_UNSUPPORTED;
    }
    a.rows = rows;
    const int code = (S ? 4 : 0) | (P ? 2 : 0) | (B ? 1 : 0);
    switch (code) {
        case 4: return launch_fast_t<FAST_R, true, false, false>(a, st);
        case 2: return launch_fast_t<FAST_R, false, true, false>(a, st);
        case 6: return launch_fast_t<FAST_R, true, true, false>(a, st);
        case 7: return launch_fast_t<FAST_R, true, true, true>(a, st);
        case 5: return launch_fast_t<FAST_R, true, false, true>(a, st);
        case 3: return launch_fast_t<FAST_R, false, true, true>(a, st);
        case 1: return launch_fast_t<FAST_R, false, false, true>(a, st);
        default: return TVGB_OK;
    }
}

template <int LAYOUT>
static int launch_prep_t(const float* in, size_t n, PrepOut o, float sn, int parity, cudaStream_t st) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    size_t blocks = (n + 255) / 256;
    if (blocks > size_t(sms) * 16) blocks = size_t(sms) * 16;
    {
        KernelTimer kt_("k_prep3", st);
        k_prep3<LAYOUT><<<unsigned(blocks ? blocks : 1), 256, 0, st>>>(in, n, o, sn, parity);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    return TVGB_OK;
}

static int launch_prep(const float* in, int layout, size_t n, PrepOut o, float sn, int parity, cudaStream_t st) {
    if (layout == TVGB_LAYOUT_MAT3) return launch_prep_t<9>(in, n, o, sn, parity, st);
    if (layout == TVGB_LAYOUT_SYM6) return launch_prep_t<6>(in, n, o, sn, parity, st);
    return launch_prep_t<60>(in, n, o, sn, parity, st);
}

int vote3_device(const float* in, int in_layout, unsigned s0, unsigned s1, unsigned s2, const tvgb_vote3_params& p,
                 float* out, int out_layout, float* evals3, float* evecs, int evec_format, cudaStream_t st,
                 const SlabHook* hook) {
    const size_t n = size_t(s0) * s1 * s2;
    if (n == 0) return TVGB_OK;
    const unsigned w = p.w ? p.w : auto_window(p.sigma1, p.sigma2);
    const int hw = int(w / 2);
    const unsigned power = p.power < 1 ? 1 : p.power;
    const bool atv = p.is_atv != 0;
    const bool S = !atv && p.stick, P = !atv && p.plate, B = !atv && p.ball;
    // exact plate whenever the rule has at least power + 2 points (or is the closed form)
    const bool plate_exact = p.samples == 0 || p.samples >= power + 2;
    // ATV runs on the fast kernel's stick, plate and ball terms with its own weights
    // (radial_entry_atv) whenever the window's tables fit in shared memory
    const bool atv_fast = atv && fast_smem(hw, 1, true, true, true) <= 200 * 1024;
    const bool fast = atv_fast || (!atv && power == 1 && (!P || plate_exact));
    const bool KS = S || atv_fast, KP = P || atv_fast, KB = B || atv_fast;   // terms of the fast kernel

    Scratch sA, sB, sC, sL, sE1, sGL;
    PrepOut po{};
    po.atv = atv_fast ? 1 : 0;
    if (KS || atv) { TVGB_TRY(sA.alloc(n * 16, st)); po.A = sA.get<float4>(); }
    if (KP) { TVGB_TRY(sB.alloc(n * 16, st)); po.B = sB.get<float4>(); }
    if (KB) { TVGB_TRY(sC.alloc(n * 4, st)); po.C = sC.get<float>(); }
    if (atv && !atv_fast) {
        TVGB_TRY(sL.alloc(n * 16, st)); po.L = sL.get<float4>();
        TVGB_TRY(sE1.alloc(n * 16, st)); po.E1 = sE1.get<float4>();
    }
    const float sn = S ? 1.0f / sticknorm3_f(p.sigma1, p.sigma2, power) : 1.0f;
    TVGB_TRY(launch_prep(in, in_layout, n, po, sn, p.parity, st));

    FastArgs fa{};
    fa.A = po.A; fa.B = po.B; fa.C = po.C;
    fa.s0 = int(s0); fa.s1 = int(s1); fa.s2 = int(s2); fa.hw = hw;
    fa.sig1 = p.sigma1; fa.sig2 = p.sigma2;
    fa.out = out; fa.out_layout = out_layout; fa.evals = evals3; fa.evecs = evecs; fa.evec_fmt = evec_format;
    fa.precise_eig = p.parity ? 0 : 1;
    fa.atv = atv_fast ? 1 : 0;
    if (!S && !P && !B && !atv) {
        // nothing votes: the reference leaves the zeroed output
        if (out) TVGB_CUDA(cudaMemsetAsync(out, 0, n * (out_layout == TVGB_LAYOUT_MAT3 ? 36 : 24), st));
        if (!evals3 && !evecs) return TVGB_OK;
    }
    if (fast) {
        if (!hook || hook->slab == 0) return launch_fast(fa, KS, KP, KB, st);
        // receivers in z-slabs of hook->slab planes; the hook follows each slab's launch
        for (unsigned z = 0; z < s0; z += hook->slab) {
            fa.zr0 = int(z);
            fa.zr1 = int(std::min(s0, z + hook->slab));
            TVGB_TRY(launch_fast(fa, KS, KP, KB, st));
            TVGB_TRY(hook->fn(hook->ctx, unsigned(fa.zr0), unsigned(fa.zr1)));
        }
        return TVGB_OK;
    }

    GenArgs g{};
    g.A = po.A; g.B = po.B; g.C = po.C; g.L = po.L; g.E1 = po.E1;
    g.s0 = int(s0); g.s1 = int(s1); g.s2 = int(s2); g.hw = hw;
    g.sig1 = p.sigma1; g.sig2 = p.sigma2; g.power = power;
    g.plate_m = int(plate_exact ? power + 2 : p.samples);
    g.stick = S; g.plate = P; g.ball = B; g.atv = atv;
    g.o = fa;
    if (B) {
        g.ng = int(power) + 3;
        g.np = 2 * int(power) + 5;
        double gx[64], gw[64];
        gauss_legendre(g.ng, gx, gw);
        float h[128];
        for (int i = 0; i < g.ng; ++i) { h[i] = float(gx[i]); h[g.ng + i] = float(gw[i]); }
        TVGB_TRY(sGL.alloc(sizeof(float) * 2 * g.ng, st));
        TVGB_CUDA(cudaMemcpyAsync(sGL.p, h, sizeof(float) * 2 * g.ng, cudaMemcpyHostToDevice, st));
        TVGB_CUDA(cudaStreamSynchronize(st));   // h is a stack buffer
        g.gl = sGL.get<float>();
    }
    dim3 grid(ceil_div(s2, 128), s1, s0);
    {
        KernelTimer kt_("k_vote3_generic", st);
        k_vote3_generic<<<grid, 128, 0, st>>>(g);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    if (hook && hook->slab) TVGB_TRY(hook->fn(hook->ctx, 0u, s0));   // one slab: the whole volume
    return TVGB_OK;
}

// Host outputs of a large vote: the receivers are voted in z-slabs and each
// slab's results go to the host on a second stream while the next slab
// votes.  A device->host copy into host memory the GPU has not touched for a
// while runs well below the link's rate, so leaving the whole result for the
// end cost a fifth of the 384^3 pipeline's time.
struct SlabCopy {
    cudaStream_t compute = nullptr, copy = nullptr;
    std::vector<cudaEvent_t> events;
    const HostOut* outs = nullptr;
    int nout = 0;
    size_t plane = 0, n = 0;   // voxels per z-plane, voxels in all
};

static int slab_copy(void* ctx, unsigned z0, unsigned z1) {
    SlabCopy& c = *static_cast<SlabCopy*>(ctx);
    cudaEvent_t e = nullptr;
    TVGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c.events.push_back(e);
    TVGB_CUDA(cudaEventRecord(e, c.compute));
    TVGB_CUDA(cudaStreamWaitEvent(c.copy, e, 0));
    const size_t v0 = size_t(z0) * c.plane, nv = size_t(z1 - z0) * c.plane;
    for (int i = 0; i < c.nout; ++i) {
        const HostOut& o = c.outs[i];
        KernelTimer kt_("copy_d2h", c.copy);
        if (o.planes) {
            for (size_t k = 0; k < o.per; ++k)
                TVGB_CUDA(cudaMemcpyAsync(o.host + k * c.n + v0, o.dev + k * c.n + v0, nv * sizeof(float),
                                          cudaMemcpyDeviceToHost, c.copy));
        } else {
            TVGB_CUDA(cudaMemcpyAsync(o.host + v0 * o.per, o.dev + v0 * o.per, nv * o.per * sizeof(float),
                                      cudaMemcpyDeviceToHost, c.copy));
        }
        kt_.stop();
    }
    return TVGB_OK;
}

int vote3_to_host(const float* in, int in_layout, unsigned s0, unsigned s1, unsigned s2, const tvgb_vote3_params& p,
                  float* out, int out_layout, float* evals3, float* evecs, int evec_format, const HostOut* outs,
                  int nouts, cudaStream_t st) {
    SlabCopy c;
    c.compute = st;
    c.plane = size_t(s1) * s2;
    c.n = size_t(s0) * c.plane;
    c.outs = outs;
    c.nout = nouts;
    TVGB_CUDA(cudaStreamCreateWithFlags(&c.copy, cudaStreamNonBlocking));
    // about 8 slabs, each a multiple of the kernels' 4-plane receiver groups
    SlabHook hook{slab_copy, &c, std::max(4u, ((s0 + 7) / 8 + 3) / 4 * 4)};
    const int rc = vote3_device(in, in_layout, s0, s1, s2, p, out, out_layout, evals3, evecs, evec_format, st, &hook);
    // join the copy stream before the caller releases the device temporaries on st
    cudaEvent_t done = nullptr;
    if (cudaEventCreateWithFlags(&done, cudaEventDisableTiming) == cudaSuccess &&
        cudaEventRecord(done, c.copy) == cudaSuccess) {
        cudaStreamWaitEvent(st, done, 0);
    } else {
        cudaStreamSynchronize(c.copy);
    }
    const cudaError_t se = cudaStreamSynchronize(st);
    if (done) cudaEventDestroy(done);
    for (cudaEvent_t e : c.events) cudaEventDestroy(e);
    cudaStreamDestroy(c.copy);
    if (rc != TVGB_OK) return rc;
    if (se != cudaSuccess) {
        set_error("vote with host outputs: %s", cudaGetErrorString(se));
        return TVGB_ERR_CUDA;
    }
    return TVGB_OK;
}

}  // namespace tvgb

using namespace tvgb;

extern "C" {

double tvgb_sticknorm3(float sigma1, float sigma2, unsigned power) { return sticknorm3_f(sigma1, sigma2, power); }

// Host table of tira::Neighbor3D records (tensorvote.h:1147, built by
// cpu::build_neighbors3d :1411): 32 bytes each, int32 du, dv, dw, float32
// d.x, d.y, d.z, c1, c2, with du on the fast axis and dw on the slow one, in
// the reference's loop order (dw outermost) and float steps.  The vote
// kernels here index a radial table instead; this exists for callers that
// inspect or reuse the reference's table.
int tvgb_build_neighbors3d(int w, float sigma1, float sigma2, void* out, int* count) {
    TVGB_CHECK_ARG(count, "tvgb_build_neighbors3d: count is NULL");
    TVGB_CHECK_ARG(w >= 0, "tvgb_build_neighbors3d: w must be >= 0");
    TVGB_CHECK_ARG(w <= 1025, "tvgb_build_neighbors3d: w = %d too large", w);
    struct Nb3 { int du, dv, dw; float dx, dy, dz, c1, c2; };
    static_assert(sizeof(Nb3) == 32, "Neighbor3D must be 32 bytes");
    const int hw = w / 2;
    const float inv1 = sigma1 > 0 ? 1.0f / (sigma1 * sigma1) : 0.0f, inv2 = sigma2 > 0 ? 1.0f / (sigma2 * sigma2) : 0.0f;
    Nb3* o = static_cast<Nb3*>(out);
    int k = 0;
    for (int dw = -hw; dw <= hw; dw++)
        for (int dv = -hw; dv <= hw; dv++)
            for (int du = -hw; du <= hw; du++, k++) {
                if (!o) continue;
                Nb3 e{};
                e.du = du; e.dv = dv; e.dw = dw;
                const float l2 = float(du * du + dv * dv + dw * dw);
                if (l2 != 0.0f) {
                    const float len = std::sqrt(l2);
                    e.dx = float(du) / len; e.dy = float(dv) / len; e.dz = float(dw) / len;
                }
                e.c1 = sigma1 == 0.0f ? (l2 > 1e-12f ? 0.0f : 1.0f) : std::exp(-l2 * inv1);
                e.c2 = sigma2 == 0.0f ? (l2 > 1e-12f ? 0.0f : 1.0f) : std::exp(-l2 * inv2);
                o[k] = e;
            }
    *count = k;
    return TVGB_OK;
}

static int check_params(const tvgb_vote3_params* p, const char* fn) {
    TVGB_CHECK_ARG(p, "%s: params is NULL", fn);
    TVGB_CHECK_ARG(p->sigma1 >= 0.0f && p->sigma2 >= 0.0f, "%s: sigmas must be >= 0", fn);
    TVGB_CHECK_ARG(p->is_atv || p->sigma1 > 0.0f || p->sigma2 > 0.0f, "%s: sigma1 and sigma2 are both 0", fn);
    TVGB_CHECK_ARG(p->w == 0 || (p->w % 2) == 1, "%s: window w must be odd (got %u)", fn, p->w);
    TVGB_CHECK_ARG(p->w <= 129, "%s: window w = %u exceeds the supported maximum 129", fn, p->w);
    TVGB_CHECK_ARG(p->power <= 32, "%s: power = %u exceeds the supported maximum 32", fn, p->power);
    return TVGB_OK;
}

int tvgb_vote3(const float* in, int in_layout, unsigned s0, unsigned s1, unsigned s2, const tvgb_vote3_params* p,
               float* out, int out_layout, float* evals3, float* evecs, int evec_format, void* stream) {
    TVGB_TRY(check_params(p, "tvgb_vote3"));
    TVGB_CHECK_ARG(in_layout == TVGB_LAYOUT_MAT3 || in_layout == TVGB_LAYOUT_SYM6 || in_layout == TVGB_LAYOUT_SYM6_PLANES,
                   "tvgb_vote3: in_layout must be 9, 6 or 60");
    TVGB_CHECK_ARG(out_layout == TVGB_LAYOUT_MAT3 || out_layout == TVGB_LAYOUT_SYM6 || out_layout == TVGB_LAYOUT_SYM6_PLANES,
                   "tvgb_vote3: out_layout must be 9, 6 or 60");
    TVGB_CHECK_ARG(evec_format >= 0 && evec_format <= 2, "tvgb_vote3: evec_format must be 0, 1 or 2");
    const size_t n = size_t(s0) * s1 * s2;
    if (n == 0) return TVGB_OK;
    TVGB_CHECK_ARG(in, "tvgb_vote3: input is NULL");
    cudaStream_t st = as_stream(stream);
    const size_t nin = in_layout == TVGB_LAYOUT_MAT3 ? 9 : 6, nout = out_layout == TVGB_LAYOUT_MAT3 ? 9 : 6;
    const size_t nv = evec_format == 1 ? 9 : (evec_format == 2 ? 6 : 0);
    DevArray din, dout, dev_, dvec;
    TVGB_TRY(din.in(in, n * nin * 4, st));
    TVGB_TRY(dout.out(out, n * nout * 4, st));
    TVGB_TRY(dev_.out(evals3, n * 12, st));
    TVGB_TRY(dvec.out(nv ? evecs : nullptr, n * nv * 4, st));
    const bool host_out = dout.owned || dev_.owned || dvec.owned;
    if (host_out && n >= (size_t(1) << 22)) {   // large volume, host outputs: copies overlapped with the vote
        HostOut outs[3];
        int no_ = 0;
        if (dout.owned) outs[no_++] = {out, dout.get<float>(), nout, out_layout == TVGB_LAYOUT_SYM6_PLANES};
        if (dev_.owned) outs[no_++] = {evals3, dev_.get<float>(), 3, false};
        if (dvec.owned) outs[no_++] = {evecs, dvec.get<float>(), nv, false};
        return vote3_to_host(din.get<float>(), in_layout, s0, s1, s2, *p, dout.get<float>(), out_layout,
                             dev_.get<float>(), dvec.get<float>(), nv ? evec_format : 0, outs, no_, st);
    }
    TVGB_TRY(vote3_device(din.get<float>(), in_layout, s0, s1, s2, *p, dout.get<float>(), out_layout,
                          dev_.get<float>(), dvec.get<float>(), nv ? evec_format : 0, st));
    TVGB_TRY(dout.finish());
    TVGB_TRY(dev_.finish());
    TVGB_TRY(dvec.finish());
    return sync_if(din.owned || host_out, st);
}

int tvgb_tensorvote3(const float* input_field, float* output_field, unsigned s0, unsigned s1, unsigned s2, float sigma,
                     float sigma2, unsigned w, unsigned power, int device, int stick, int plate, unsigned samples,
                     int is_atv, void* stream) {
    TVGB_CHECK_ARG(input_field && output_field, "tvgb_tensorvote3: NULL field pointer");
    TVGB_CHECK_ARG(w >= 1 && (w % 2) == 1, "tvgb_tensorvote3: window w must be odd and >= 1 (got %u)", w);
    // the reference runs on device `device` (tensorvote.h:2820); a negative
    // index selects its CPU eigen path (eigen.h:897), which this library has not
    TVGB_CHECK_ARG(device >= 0, "tvgb_tensorvote3: device %d: negative indices select the reference's CPU path, "
                   "which this GPU library does not provide", device);
    TVGB_CUDA(cudaSetDevice(device));
    tvgb_vote3_params p{};
    p.sigma1 = sigma; p.sigma2 = sigma2; p.w = w; p.power = power; p.samples = samples;
    p.stick = stick; p.plate = plate; p.ball = 0; p.is_atv = is_atv; p.parity = 1;
    return tvgb_vote3(input_field, TVGB_LAYOUT_MAT3, s0, s1, s2, &p, output_field, TVGB_LAYOUT_MAT3, nullptr, nullptr,
                      0, stream);
}

}  // extern "C"

// ------------------------------------------------------------------ allocation-free 3D vote
// tvgb_vote3_noalloc: the same preparation and fast vote kernels as tvgb_vote3,
// for callers that may not allocate device memory while they run -- code
// inside a host-side real-time loop or plugin callback that forbids
// allocation, or a process whose device memory is owned by another
// allocator.  The per-voxel voter records (the only scratch this path uses)
// live in the file-scope arrays below instead of stream-ordered
// allocations: every GPU that loads the library holds them until exit.
#include <mutex>

namespace tvgb {

constexpr size_t NOALLOC_MAX_VOXELS = size_t(1) << 19;   // 524288 voxels (e.g. 80^3): 18 MiB per GPU

static __device__ __align__(256) float4 g_noalloc_stick[NOALLOC_MAX_VOXELS];
static __device__ __align__(256) float4 g_noalloc_plate[NOALLOC_MAX_VOXELS];
static __device__ __align__(256) float g_noalloc_ball[NOALLOC_MAX_VOXELS];

struct NoallocScratch {
    float4* stick;
    float4* plate;
    float* ball;
};

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::mutex g_noalloc_mu;
static bool g_noalloc_ready[NOALLOC_MAX_DEVICES];
static NoallocScratch g_noalloc_addr[NOALLOC_MAX_DEVICES];
static void* g_noalloc_ctx[NOALLOC_MAX_DEVICES];

// The current CUDA context (driver API, looked up through the runtime since
// the library links only the runtime); null if unavailable.
static void* current_context() {
    using GetCtx = int (*)(void**);
    static std::once_flag once;
    static GetCtx fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<GetCtx>(p);
        else
            cudaGetLastError();
    });
    void* ctx = nullptr;
    if (fn && fn(&ctx) != 0) ctx = nullptr;
    return ctx;
}

// Device addresses of the arrays on the current device (the array names are
// host-side stand-ins in host code), looked up on the first call in each
// context of a device: a device reset (cudaDeviceReset, or another library
// resetting the primary context) makes a new context, whose module copy of
// the arrays may sit elsewhere, so the cached addresses follow the context.
static int noalloc_scratch(NoallocScratch& s) {
    int dev = 0;
    TVGB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        set_error("tvgb_vote3_noalloc: device %d beyond the supported %d", dev, NOALLOC_MAX_DEVICES);
        return TVGB_ERR_UNSUPPORTED;
    }
    // the caller's arrays were classified (cudaPointerGetAttributes) before this, so the device's context
    // is current; without one the addresses are looked up again on every call
    void* ctx = current_context();
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_ready[dev] || !ctx || ctx != g_noalloc_ctx[dev]) {
        NoallocScratch a{};
        TVGB_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&a.stick), g_noalloc_stick));
        TVGB_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&a.plate), g_noalloc_plate));
        TVGB_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&a.ball), g_noalloc_ball));
        g_noalloc_addr[dev] = a;
        g_noalloc_ready[dev] = true;
        g_noalloc_ctx[dev] = ctx;
    }
    s = g_noalloc_addr[dev];
    return TVGB_OK;
}

}  // namespace tvgb

extern "C" int tvgb_vote3_noalloc(const float* in, int in_layout, unsigned s0, unsigned s1, unsigned s2,
                                  const tvgb_vote3_params* p, float* out, int out_layout, float* evals3, float* evecs,
                                  int evec_format, void* stream) {
    TVGB_TRY(check_params(p, "tvgb_vote3_noalloc"));
    TVGB_CHECK_ARG(in_layout == TVGB_LAYOUT_MAT3 || in_layout == TVGB_LAYOUT_SYM6 || in_layout == TVGB_LAYOUT_SYM6_PLANES,
                   "tvgb_vote3_noalloc: in_layout must be 9, 6 or 60");
    TVGB_CHECK_ARG(out_layout == TVGB_LAYOUT_MAT3 || out_layout == TVGB_LAYOUT_SYM6 || out_layout == TVGB_LAYOUT_SYM6_PLANES,
                   "tvgb_vote3_noalloc: out_layout must be 9, 6 or 60");
    TVGB_CHECK_ARG(evec_format >= 0 && evec_format <= 2, "tvgb_vote3_noalloc: evec_format must be 0, 1 or 2");
    const size_t n = size_t(s0) * s1 * s2;
    if (n == 0) return TVGB_OK;
    TVGB_CHECK_ARG(n <= NOALLOC_MAX_VOXELS,
                   "tvgb_vote3_noalloc: %zu voxels exceed the maximum of %zu (use tvgb_vote3 for larger volumes)",
                   n, NOALLOC_MAX_VOXELS);
    TVGB_CHECK_ARG(!p->is_atv, "tvgb_vote3_noalloc: ATV is not available without allocation (use tvgb_vote3)");
    const unsigned power = p->power < 1 ? 1 : p->power;
    TVGB_CHECK_ARG(power == 1 && (!p->plate || p->samples == 0 || p->samples >= 3),
                   "tvgb_vote3_noalloc: only power 1 with an exact plate (samples 0 or >= 3) runs without "
                   "allocation (use tvgb_vote3)");
    // the caller passes device arrays: staging host memory would allocate
    TVGB_CHECK_ARG(in && is_device_ptr(in), "tvgb_vote3_noalloc: input must be device memory");
    TVGB_CHECK_ARG(!out || is_device_ptr(out), "tvgb_vote3_noalloc: out must be device memory");
    TVGB_CHECK_ARG(!evals3 || is_device_ptr(evals3), "tvgb_vote3_noalloc: evals3 must be device memory");
    TVGB_CHECK_ARG(!evecs || !evec_format || is_device_ptr(evecs), "tvgb_vote3_noalloc: evecs must be device memory");
    NoallocScratch sc;
    TVGB_TRY(noalloc_scratch(sc));
    cudaStream_t st = as_stream(stream);
    const bool S = p->stick != 0, P = p->plate != 0, B = p->ball != 0;
    const unsigned w = p->w ? p->w : auto_window(p->sigma1, p->sigma2);
    PrepOut po{};
    po.A = S ? sc.stick : nullptr;
    po.B = P ? sc.plate : nullptr;
    po.C = B ? sc.ball : nullptr;
    const float sn = S ? 1.0f / sticknorm3_f(p->sigma1, p->sigma2, power) : 1.0f;
    TVGB_TRY(launch_prep(in, in_layout, n, po, sn, p->parity, st));
    FastArgs fa{};
    fa.A = po.A; fa.B = po.B; fa.C = po.C;
    fa.s0 = int(s0); fa.s1 = int(s1); fa.s2 = int(s2); fa.hw = int(w / 2);
    fa.sig1 = p->sigma1; fa.sig2 = p->sigma2;
    fa.out = out; fa.out_layout = out_layout; fa.evals = evals3;
    fa.evecs = evec_format ? evecs : nullptr; fa.evec_fmt = evec_format;
    fa.precise_eig = p->parity ? 0 : 1;
    // with no term voting, launch_fast writes the zero tensor and its eigendecomposition
    return launch_fast(fa, S, P, B, st);
}

// ------------------------------------------------------------------ learned plate / ball vote
// tvgb_vote3_surrogate: the stick vote exact (as k_vote3_fast), the plate
// vote by one of three rules, chosen so that they can be timed side by side
// in the same kernel skeleton (one receiver per lane, 32 x 4 receivers per
// CTA, voters read through L1 / L2):
//   PLATE_SURROGATE  the MLP of surrogate_mlp.cuh on the tensor cores
//                    (sur_tc.cuh): for each voter offset the CTA runs its
//                    128 (receiver, voter) pairs as one tile; o = 0 is voted
//                    exactly.  A judge then votes the plate of the CTA's
//                    first 32 receivers exactly; if the surrogate's plate
//                    differs from it by more than tol x the norm of the full
//                    voted tensors, normwise over those 32 receivers (the
//                    tile's sampled error), the whole CTA's plate is
//                    recomputed exactly.
//   PLATE_CLOSED     the exact closed form of k_vote3_fast.
//   PLATE_PLAIN64    the plain orientation integral with 64 orientations
//                    (the reference's plate3_numerical_device rule,
//                    tensorvote.h:2457, basis :2467-2469).
// The ball vote (lambda0 x the mean unit stick vote over the sphere) depends
// on the offset only: it is tabulated per offset by the same rule (network
// with flag 0 / closed form / 8 x 8 sphere rule) and applied per pair.
#include "sur_tc.cuh"
#include <algorithm>
#include <cmath>
#include <vector>

namespace tvgb {

enum { PLATE_SURROGATE = 0, PLATE_CLOSED = 1, PLATE_PLAIN64 = 2 };

struct SurVoteArgs {
    FastArgs f;
    const uint4* img;         // the network's weight image (PLATE_SURROGATE, sur_tc.cuh)
    const float* ball_tab;    // (2 hw + 1)^3 x 8 floats, or NULL
    const float* ball_exact;  // the exact ball table (the judge's), PLATE_SURROGATE only
    float inv_sig;
    float tol;
    unsigned* stats;          // [0] CTAs, [1] CTAs whose plate was recomputed exactly
    int* err;                 // set when a tensor-core wait gave up
};

__constant__ float c_cs64[64], c_sn64[64];
// 8-point Gauss-Legendre rule on [-1, 1] (nodes, weights)
__constant__ float c_gl8x_v[8] = {-0.9602898564975363f, -0.7966664774136267f, -0.5255324099163290f,
                                  -0.1834346424956498f, 0.1834346424956498f,  0.5255324099163290f,
                                  0.7966664774136267f,  0.9602898564975363f};
__constant__ float c_gl8w_v[8] = {0.1012285362903763f, 0.2223810344533745f, 0.3137066458778873f,
                                  0.3626837833783620f, 0.3626837833783620f, 0.3137066458778873f,
                                  0.2223810344533745f, 0.1012285362903763f};

// the plain orientation integral's plate for one pair (sigma2 = 0 rule via the radial table)
__device__ __forceinline__ void plate_plain64(const float4& B, float ox, float oy, float oz, const float4& ta,
                                              float L2, float* P) {
    if (B.w == 0.0f) return;
    const float n0 = B.x, n1 = B.y, n2 = B.z;
    float u0, u1, u2;
    if (fabsf(n2) < 0.999f) { u0 = n1; u1 = -n0; u2 = 0.0f; } else { u0 = 0.0f; u1 = n2; u2 = -n1; }
    const float iu = rsqrtf(u0 * u0 + u1 * u1 + u2 * u2);
    u0 *= iu; u1 *= iu; u2 *= iu;
    const float v0 = n1 * u2 - n2 * u1, v1 = n2 * u0 - n0 * u2, v2 = n0 * u1 - n1 * u0;
    const float c1 = ta.x, ctg = ta.y, g2 = ta.z;        // c1, (c2 - c1)/|o|^2, 2/|o|^2
    const float ws = B.w * (1.0f / 64.0f);
    float a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0;
#pragma unroll 4
    for (int i = 0; i < 64; ++i) {
        const float cs = c_cs64[i], sn = c_sn64[i];
        const float q0 = fmaf(cs, u0, sn * v0), q1 = fmaf(cs, u1, sn * v1), q2 = fmaf(cs, u2, sn * v2);
        const float qo = fmaf(q0, ox, fmaf(q1, oy, q2 * oz));
        const float eta = fmaf(ctg, qo * qo, c1);
        const float k = qo * g2;
        const float r0 = fmaf(-k, ox, q0), r1 = fmaf(-k, oy, q1), r2 = fmaf(-k, oz, q2);
        const float t0 = eta * r0, t1 = eta * r1, t2 = eta * r2;
        a0 = fmaf(t0, r0, a0); a1 = fmaf(t0, r1, a1); a2 = fmaf(t0, r2, a2);
        a3 = fmaf(t1, r1, a3); a4 = fmaf(t1, r2, a4); a5 = fmaf(t2, r2, a5);
    }
    (void)L2;
    P[0] = fmaf(ws, a0, P[0]); P[1] = fmaf(ws, a1, P[1]); P[2] = fmaf(ws, a2, P[2]);
    P[3] = fmaf(ws, a3, P[3]); P[4] = fmaf(ws, a4, P[4]); P[5] = fmaf(ws, a5, P[5]);
}

// the exact plate (closed form) of this lane's receiver over the window
// without o = 0 (that term is always voted exactly in the main loop)
template <bool BALL>
__device__ __forceinline__ void plate_exact_sum(const SurVoteArgs& a, const float4* tbl, int x, int y, int z,
                                                float* E) {
    const FastArgs& f = a.f;
    const int hw = f.hw, W = 2 * hw + 1;
    for (int k = 0; k < 7; ++k) E[k] = 0.0f;
    const float4 Z4 = make_float4(0, 0, 0, 0);
    for (int oz = -hw; oz <= hw; ++oz) {
        const int vz = z + oz;
        if ((unsigned)vz >= (unsigned)f.s0) continue;
        for (int oy = -hw; oy <= hw; ++oy) {
            const int vy = y + oy;
            if ((unsigned)vy >= (unsigned)f.s1) continue;
            for (int ox = -hw; ox <= hw; ++ox) {
                const int vx = x + ox;
                const bool in = (unsigned)vx < (unsigned)f.s2;
                const float4 B = in ? __ldg(f.B + (size_t(vz) * f.s1 + vy) * f.s2 + vx) : Z4;
                const int L2 = ox * ox + oy * oy + oz * oz;
                if (BALL) {   // the exact ball, every offset
                    const float lb = in ? __ldg(f.C + (size_t(vz) * f.s1 + vy) * f.s2 + vx) : 0.0f;
                    const float4* bt = reinterpret_cast<const float4*>(
                        a.ball_exact + 8 * (size_t((oz + hw) * W + (oy + hw)) * W + (ox + hw)));
                    const float4 b0 = __ldg(bt), b1 = __ldg(bt + 1);
                    E[0] = fmaf(lb, b0.x, E[0]); E[1] = fmaf(lb, b0.y, E[1]); E[2] = fmaf(lb, b0.z, E[2]);
                    E[3] = fmaf(lb, b0.w, E[3]); E[4] = fmaf(lb, b1.x, E[4]); E[5] = fmaf(lb, b1.y, E[5]);
                }
                if (L2 == 0) continue;
                const float4 ta = tbl[2 * L2], tb = tbl[2 * L2 + 1];
                vote_pair<false, true, false>(Z4, B, 0.0f, 0.0f, fmaf(B.x, float(ox), B.y * float(oy)), float(ox),
                                              float(oy), float(oz), ta, tb, E);
            }
        }
    }
}

// The exact plate rules (PLATE_CLOSED, PLATE_PLAIN64) in the surrogate
// kernel's skeleton, for timing side by side with it.
template <int MODE, bool STICK, bool BALL>
__global__ void __launch_bounds__(128) k_vote3_sur(SurVoteArgs a) {
    extern __shared__ __align__(16) float4 sm4[];
    const FastArgs& f = a.f;
    const int hw = f.hw;
    const int nt = 3 * hw * hw + 1;
    float4* tbl = sm4;                                               // 2 nt float4
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int L2 = tid; L2 < nt; L2 += 128) {
        float4 ea, eb;
        radial_entry(L2, f.sig1, f.sig2, ea, eb);
        tbl[2 * L2] = ea;
        tbl[2 * L2 + 1] = eb;
    }
    __syncthreads();

    const int x = blockIdx.x * 32 + lane, y = blockIdx.y * 4 + warp, z = blockIdx.z;
    const bool yin = y < f.s1;
    const float4 Z4 = make_float4(0, 0, 0, 0);
    float tot[6], cmp[6];
    for (int k = 0; k < 6; ++k) { tot[k] = 0.0f; cmp[k] = 0.0f; }
    const int W = 2 * hw + 1;
    for (int oz = -hw; oz <= hw; ++oz) {
        const int vz = z + oz;
        if ((unsigned)vz >= (unsigned)f.s0) continue;
        float P[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int oy = -hw; oy <= hw; ++oy) {
            const int vy = y + oy;
            if (!yin || (unsigned)vy >= (unsigned)f.s1) continue;   // warp-uniform
            const size_t row = (size_t(vz) * f.s1 + vy) * f.s2;
            for (int ox = -hw; ox <= hw; ++ox) {
                const int vx = x + ox;
                const bool in = (unsigned)vx < (unsigned)f.s2;
                const float4 A = (STICK && in) ? __ldg(f.A + row + vx) : Z4;
                const float4 B = in ? __ldg(f.B + row + vx) : Z4;
                const int L2 = ox * ox + oy * oy + oz * oz;
                const float4 ta = tbl[2 * L2], tb = tbl[2 * L2 + 1];
                const float oxf = float(ox), oyf = float(oy), ozf = float(oz);
                if (STICK)
                    vote_pair<true, false, false>(A, Z4, 0.0f, fmaf(A.x, oxf, A.y * oyf), 0.0f, oxf, oyf, ozf, ta, tb, P);
                if (BALL) {
                    const float lb = in ? __ldg(f.C + row + vx) : 0.0f;
                    const float4* bt = reinterpret_cast<const float4*>(
                        a.ball_tab + 8 * (size_t((oz + hw) * W + (oy + hw)) * W + (ox + hw)));
                    const float4 b0 = __ldg(bt), b1 = __ldg(bt + 1);
                    P[0] = fmaf(lb, b0.x, P[0]); P[1] = fmaf(lb, b0.y, P[1]); P[2] = fmaf(lb, b0.z, P[2]);
                    P[3] = fmaf(lb, b0.w, P[3]); P[4] = fmaf(lb, b1.x, P[4]); P[5] = fmaf(lb, b1.y, P[5]);
                }
                if (MODE == PLATE_CLOSED || L2 == 0)
                    vote_pair<false, true, false>(Z4, B, 0.0f, 0.0f, fmaf(B.x, oxf, B.y * oyf), oxf, oyf, ozf, ta, tb, P);
                else
                    plate_plain64(B, oxf, oyf, ozf, ta, float(L2), P);
            }
        }
        kahan_add(tot[0], cmp[0], P[0] + P[6]);
        kahan_add(tot[1], cmp[1], P[1]);
        kahan_add(tot[2], cmp[2], P[2]);
        kahan_add(tot[3], cmp[3], P[3] + P[6]);
        kahan_add(tot[4], cmp[4], P[4]);
        kahan_add(tot[5], cmp[5], P[5] + P[6]);
    }
    if (x >= f.s2 || !yin) return;
    const size_t plane = size_t(f.s1) * f.s2, n = size_t(f.s0) * plane;
    write_receiver(f, size_t(z) * plane + size_t(y) * f.s2 + x, n, tot);
}

// The surrogate vote on the tensor cores.  A CTA is 32 x 4 receivers (one per
// thread, = one row of the M = 128 tile); for each voter offset o != 0 the
// CTA runs one tile through the network (sur_tc.cuh): row r holds (o / |o|,
// n of receiver r's voter, 1).  Offsets are visited in the same order by
// every thread (the tile's MMAs synchronise the CTA): rows whose voter lies
// outside the volume carry a zero record and vote zero.  While the tensor
// core runs layer 1, the same threads vote the stick exactly.  The network's
// plate (and ball) accumulate apart from the exact terms, so that the judge
// can compare them with the exact plate of the CTA's first 32 receivers.
template <bool STICK, bool BALL>
__global__ void __launch_bounds__(128) k_vote3_surtc(SurVoteArgs a) {
    extern __shared__ __align__(128) float4 sm4[];
    const FastArgs& f = a.f;
    const int hw = f.hw;
    const int nt = 3 * hw * hw + 1;
    uint4* img_s = reinterpret_cast<uint4*>(sm4);                    // weight image
    float4* tbl = sm4 + TC_IMG_BYTES / 16;                           // 2 nt float4
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) uint64_t bar;
    __shared__ int s_fail;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int L2 = tid; L2 < nt; L2 += 128) {
        float4 ea, eb;
        radial_entry(L2, f.sig1, f.sig2, ea, eb);
        tbl[2 * L2] = ea;
        tbl[2 * L2 + 1] = eb;
    }
    if (tid == 0) s_fail = 0;
    SurTc tcs;
    sur_tc_setup(tcs, a.img, img_s, &tmem_slot, &bar);   // ends with __syncthreads

    const int x = blockIdx.x * 32 + lane, y = blockIdx.y * 4 + warp, z = blockIdx.z;
    const int y0 = blockIdx.y * 4;
    const bool yin = y < f.s1;
    const float4 Z4 = make_float4(0, 0, 0, 0);
    const uint32_t tA = tcs.tmem + tc_lane_base() + TC_A, tD = tcs.tmem + tc_lane_base() + TC_D;
    float tot[6], cmp[6], net[6], bs[6];
    for (int k = 0; k < 6; ++k) { tot[k] = 0.0f; cmp[k] = 0.0f; net[k] = 0.0f; bs[k] = 0.0f; }
    const int W = 2 * hw + 1;
    // rows oy for which any of the CTA's 4 receiver rows has its voter inside the volume
    const int oy_lo = max(-hw, -(y0 + 3)), oy_hi = min(hw, f.s1 - 1 - y0);
    bool ok = true;
    for (int oz = -hw; oz <= hw && ok; ++oz) {
        const int vz = z + oz;
        if ((unsigned)vz >= (unsigned)f.s0) continue;                // CTA-uniform
        float P[7] = {0, 0, 0, 0, 0, 0, 0};
        float Q[6] = {0, 0, 0, 0, 0, 0};
        for (int oy = oy_lo; oy <= oy_hi && ok; ++oy) {
            const int vy = y + oy;
            const bool rin = yin && (unsigned)vy < (unsigned)f.s1;
            const size_t row = (size_t(vz) * f.s1 + (rin ? vy : 0)) * f.s2;
            for (int ox = -hw; ox <= hw; ++ox) {
                const int vx = x + ox;
                const bool in = rin && (unsigned)vx < (unsigned)f.s2;
                const float4 A = (STICK && in) ? __ldg(f.A + row + vx) : Z4;
                const float4 B = in ? __ldg(f.B + row + vx) : Z4;
                const int L2 = ox * ox + oy * oy + oz * oz;
                const float4 ta = tbl[2 * L2], tb = tbl[2 * L2 + 1];
                const float oxf = float(ox), oyf = float(oy), ozf = float(oz);
                if (L2 == 0) {                                       // CTA-uniform: o = 0 is voted exactly
                    if (STICK)
                        vote_pair<true, false, false>(A, Z4, 0.0f, fmaf(A.x, oxf, A.y * oyf), 0.0f, oxf, oyf, ozf, ta,
                                                      tb, P);
                    vote_pair<false, true, false>(Z4, B, 0.0f, 0.0f, fmaf(B.x, oxf, B.y * oyf), oxf, oyf, ozf, ta, tb, P);
                } else {
                    const float il = rsqrtf(float(L2));
                    float dv[3] = {oxf * il, oyf * il, ozf * il}, nv[3] = {B.x, B.y, B.z};
                    sur_canonical(dv, nv, true);
                    // layer 1's row: the features, the bias pair, the features' BF16 residuals (sur_row64)
                    const float xin[SUR_X] = {dv[0], dv[1], dv[2], nv[0], nv[1], nv[2], 1.0f};
                    uint32_t row[SUR_K1 / 2];
                    sur_row64(xin, row);
                    if (!tcs.failed) tc::tmem_st32(tA, row);
                    if (!sur_tc_layer<1>(tcs)) { ok = false; break; }
                    // the exact stick vote while layer 1 runs
                    if (STICK)
                        vote_pair<true, false, false>(A, Z4, 0.0f, fmaf(A.x, oxf, A.y * oyf), 0.0f, oxf, oyf, ozf, ta,
                                                      tb, P);
                    sur_tc_hidden<1>(tcs);
                    if (!sur_tc_layer<2>(tcs)) { ok = false; break; }
                    sur_tc_hidden<1>(tcs);
                    if (!sur_tc_layer<3>(tcs)) { ok = false; break; }
                    sur_tc_hidden<1>(tcs);
                    if (!sur_tc_layer<4>(tcs) || tcs.failed) { ok = false; break; }
                    uint32_t r[16];
                    tc::tmem_ld16(tD, r);
                    const float w = B.w * ta.x;                      // plate scale x c1(|o|)
#pragma unroll
                    for (int k = 0; k < 6; ++k) Q[k] = fmaf(w, __uint_as_float(r[k]), Q[k]);
                }
                if (BALL) {   // the tabulated ball (network, exact at o = 0), judged with the plate
                    const float lb = in ? __ldg(f.C + row + vx) : 0.0f;
                    const float4* bt = reinterpret_cast<const float4*>(
                        a.ball_tab + 8 * (size_t((oz + hw) * W + (oy + hw)) * W + (ox + hw)));
                    const float4 b0 = __ldg(bt), b1 = __ldg(bt + 1);
                    bs[0] = fmaf(lb, b0.x, bs[0]); bs[1] = fmaf(lb, b0.y, bs[1]); bs[2] = fmaf(lb, b0.z, bs[2]);
                    bs[3] = fmaf(lb, b0.w, bs[3]); bs[4] = fmaf(lb, b1.x, bs[4]); bs[5] = fmaf(lb, b1.y, bs[5]);
                }
            }
        }
        // exact terms (stick, o = 0 plate) into the Kahan sums; the network's plate apart
        kahan_add(tot[0], cmp[0], P[0] + P[6]);
        kahan_add(tot[1], cmp[1], P[1]);
        kahan_add(tot[2], cmp[2], P[2]);
        kahan_add(tot[3], cmp[3], P[3] + P[6]);
        kahan_add(tot[4], cmp[4], P[4]);
        kahan_add(tot[5], cmp[5], P[5] + P[6]);
        for (int k = 0; k < 6; ++k) net[k] += Q[k];
    }
    if (!sur_tc_teardown(tcs) || !ok) {
        if (tid == 0) atomicExch(a.err, 1);
        return;
    }
    float plate[6];
    for (int k = 0; k < 6; ++k) plate[k] = net[k] + bs[k];
    // judge: the first warp's receivers against the exact plate (and ball)
    const bool mine = x < f.s2 && yin;
    if (warp == 0) {
        float E[7];
        plate_exact_sum<BALL>(a, tbl, x, y, z, E);
        const float e6[6] = {E[0] + E[6], E[1], E[2], E[3] + E[6], E[4], E[5] + E[6]};
        // the tile's sampled error, normwise over its 32 sampled receivers (Frobenius norms, off-diagonal
        // entries twice): || plate_net - plate_exact || against tol x || voted tensor ||
        float dn = 0.0f, tn = 0.0f;
        if (mine)
            for (int k = 0; k < 6; ++k) {
                const float wgt = (k == 0 || k == 3 || k == 5) ? 1.0f : 2.0f;
                const float d = plate[k] - e6[k], tt = tot[k] + e6[k];
                dn = fmaf(wgt * d, d, dn);
                tn = fmaf(wgt * tt, tt, tn);
            }
        for (int off = 16; off > 0; off >>= 1) {
            dn += __shfl_xor_sync(0xffffffffu, dn, off);
            tn += __shfl_xor_sync(0xffffffffu, tn, off);
        }
        if (lane == 0 && !(dn <= a.tol * a.tol * tn)) s_fail = 1;
    }
    __syncthreads();
    if (s_fail) {
        float E[7];
        plate_exact_sum<BALL>(a, tbl, x, y, z, E);
        plate[0] = E[0] + E[6]; plate[1] = E[1]; plate[2] = E[2];
        plate[3] = E[3] + E[6]; plate[4] = E[4]; plate[5] = E[5] + E[6];
    }
    if (tid == 0 && a.stats) {
        atomicAdd(a.stats, 1u);
        if (s_fail) atomicAdd(a.stats + 1, 1u);
    }
    if (!mine) return;
    const size_t plane = size_t(f.s1) * f.s2, n = size_t(f.s0) * plane;
    float m6[6];
    for (int k = 0; k < 6; ++k) m6[k] = tot[k] + plate[k];
    write_receiver(f, size_t(z) * plane + size_t(y) * f.s2 + x, n, m6);
}

// the per-offset ball table: lambda0-unit ball vote at each offset of the window
template <int MODE>
__global__ void k_ball_table(int hw, float sig1, float sig2, float inv_sig, const float* __restrict__ Fnet,
                             float* __restrict__ tab) {
    const int W = 2 * hw + 1;
    const int n = W * W * W;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ox = i % W - hw, oy = (i / W) % W - hw, oz = i / (W * W) - hw;
        const int L2 = ox * ox + oy * oy + oz * oz;
        float4 ea, eb;
        radial_entry(L2, sig1, sig2, ea, eb);
        float F[6] = {0, 0, 0, 0, 0, 0};
        if (MODE == PLATE_CLOSED || L2 == 0) {
            // (c1/3 + ct [o != 0]/15) I + (2 ct g / 15) o o^T: eb.z, eb.w
            const float o[3] = {float(ox), float(oy), float(oz)};
            F[0] = eb.z + eb.w * o[0] * o[0]; F[1] = eb.w * o[0] * o[1]; F[2] = eb.w * o[0] * o[2];
            F[3] = eb.z + eb.w * o[1] * o[1]; F[4] = eb.w * o[1] * o[2]; F[5] = eb.z + eb.w * o[2] * o[2];
        } else if (MODE == PLATE_PLAIN64) {
            const float il = rsqrtf(float(L2));
            const float d[3] = {ox * il, oy * il, oz * il};
            const float c1 = ea.x, c2 = c1 + ea.y * float(L2);
            for (int ia = 0; ia < 8; ++ia)
                for (int ib = 0; ib < 8; ++ib) {
                    const float ct = c_gl8x_v[ia], st = sqrtf(1.0f - ct * ct);
                    float sp, cp;
                    sincospif(float(ib) / 4.0f, &sp, &cp);
                    const float q[3] = {st * cp, st * sp, ct};
                    const float qd = q[0] * d[0] + q[1] * d[1] + q[2] * d[2];
                    const float eta = c_gl8w_v[ia] * (1.0f / 16.0f) * (c1 * (1.0f - qd * qd) + c2 * qd * qd);
                    const float r[3] = {q[0] - 2 * qd * d[0], q[1] - 2 * qd * d[1], q[2] - 2 * qd * d[2]};
                    F[0] += eta * r[0] * r[0]; F[1] += eta * r[0] * r[1]; F[2] += eta * r[0] * r[2];
                    F[3] += eta * r[1] * r[1]; F[4] += eta * r[1] * r[2]; F[5] += eta * r[2] * r[2];
                }
        } else {
            for (int k = 0; k < 6; ++k) F[k] = ea.x * Fnet[size_t(i) * 8 + k];
        }
        for (int k = 0; k < 6; ++k) tab[size_t(i) * 8 + k] = F[k];
        tab[size_t(i) * 8 + 6] = 0.0f;
        tab[size_t(i) * 8 + 7] = 0.0f;
    }
}

template <int MODE>
static int launch_sur(const SurVoteArgs& a, bool S, bool B, dim3 grid, size_t smem, cudaStream_t st) {
    const void* fn;
    if (MODE == PLATE_SURROGATE) {
        if (S && B) fn = (const void*)k_vote3_surtc<true, true>;
        else if (S) fn = (const void*)k_vote3_surtc<true, false>;
        else if (B) fn = (const void*)k_vote3_surtc<false, true>;
        else fn = (const void*)k_vote3_surtc<false, false>;
    } else {
        if (S && B) fn = (const void*)k_vote3_sur<MODE, true, true>;
        else if (S) fn = (const void*)k_vote3_sur<MODE, true, false>;
        else if (B) fn = (const void*)k_vote3_sur<MODE, false, true>;
        else fn = (const void*)k_vote3_sur<MODE, false, false>;
    }
    TVGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    SurVoteArgs arg = a;
    void* args[] = {&arg};
    {
        KernelTimer kt_(MODE == PLATE_SURROGATE ? "k_vote3_surtc" : (MODE == PLATE_CLOSED ? "k_vote3_sur_closed"
                                                                                         : "k_vote3_sur_plain64"), st);
        TVGB_CUDA(cudaLaunchKernel(fn, grid, dim3(128), args, smem, st));
        kt_.stop();
    }
    TVGB_LAUNCHED();
    return TVGB_OK;
}

static int sur_constants() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    TVGB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && done[dev]) return TVGB_OK;
    float cs[64], sn[64];
    for (int i = 0; i < 64; ++i) {
        cs[i] = float(std::cos(3.14159265358979323846 * i / 64.0));
        sn[i] = float(std::sin(3.14159265358979323846 * i / 64.0));
    }
    TVGB_CUDA(cudaMemcpyToSymbol(c_cs64, cs, sizeof(cs)));
    TVGB_CUDA(cudaMemcpyToSymbol(c_sn64, sn, sizeof(sn)));
    if (dev >= 0 && dev < 64) done[dev] = true;
    return TVGB_OK;
}

}  // namespace tvgb

extern "C" int tvgb_vote3_surrogate(const float* in, int in_layout, unsigned s0, unsigned s1, unsigned s2,
                                    const tvgb_vote3_params* p, const float* net_params, int plate_mode, float tol,
                                    float* out, int out_layout, float* evals3, float* evecs, int evec_format,
                                    unsigned long long* stats, void* stream) {
    using namespace tvgb;
    TVGB_TRY(check_params(p, "tvgb_vote3_surrogate"));
    TVGB_CHECK_ARG(!p->is_atv && (p->power <= 1) && p->sigma2 == 0.0f && p->sigma1 > 0.0f,
                   "tvgb_vote3_surrogate: TK with power 1 and sigma2 = 0 only (the surrogate's training domain)");
    TVGB_CHECK_ARG(plate_mode >= 0 && plate_mode <= 2, "tvgb_vote3_surrogate: plate_mode must be 0, 1 or 2");
    TVGB_CHECK_ARG(plate_mode != 0 || net_params, "tvgb_vote3_surrogate: plate_mode 0 needs the network parameters");
    TVGB_CHECK_ARG(tol >= 0.0f, "tvgb_vote3_surrogate: tol must be >= 0");
    TVGB_CHECK_ARG(in_layout == TVGB_LAYOUT_MAT3 || in_layout == TVGB_LAYOUT_SYM6 || in_layout == TVGB_LAYOUT_SYM6_PLANES,
                   "tvgb_vote3_surrogate: in_layout must be 9, 6 or 60");
    TVGB_CHECK_ARG(out_layout == TVGB_LAYOUT_MAT3 || out_layout == TVGB_LAYOUT_SYM6 || out_layout == TVGB_LAYOUT_SYM6_PLANES,
                   "tvgb_vote3_surrogate: out_layout must be 9, 6 or 60");
    TVGB_CHECK_ARG(evec_format >= 0 && evec_format <= 2, "tvgb_vote3_surrogate: evec_format must be 0, 1 or 2");
    const size_t n = size_t(s0) * s1 * s2;
    if (stats) { stats[0] = 0; stats[1] = 0; }
    if (n == 0) return TVGB_OK;
    TVGB_CHECK_ARG(in, "tvgb_vote3_surrogate: input is NULL");
    cudaStream_t st = as_stream(stream);
    TVGB_TRY(sur_constants());
    const size_t nin = in_layout == TVGB_LAYOUT_MAT3 ? 9 : 6, nout = out_layout == TVGB_LAYOUT_MAT3 ? 9 : 6;
    const size_t nv = evec_format == 1 ? 9 : (evec_format == 2 ? 6 : 0);
    DevArray din, dout, dev_, dvec;
    TVGB_TRY(din.in(in, n * nin * 4, st));
    TVGB_TRY(dout.out(out, n * nout * 4, st));
    TVGB_TRY(dev_.out(evals3, n * 12, st));
    TVGB_TRY(dvec.out(nv ? evecs : nullptr, n * nv * 4, st));

    const unsigned w = p->w ? p->w : auto_window(p->sigma1, p->sigma2);
    const int hw = int(w / 2), W = int(w);
    const bool S = p->stick != 0, P = p->plate != 0, B = p->ball != 0;
    Scratch sA, sB, sC, stab, stabx, snet, sX, sY, sst;
    PrepOut po{};
    TVGB_TRY(sA.alloc(n * 16, st)); po.A = sA.get<float4>();
    TVGB_TRY(sB.alloc(n * 16, st)); po.B = sB.get<float4>();
    if (B) { TVGB_TRY(sC.alloc(n * 4, st)); po.C = sC.get<float>(); }
    const float sn = S ? 1.0f / sticknorm3_f(p->sigma1, p->sigma2, 1) : 1.0f;
    TVGB_TRY(launch_prep(din.get<float>(), in_layout, n, po, sn, p->parity, st));
    if (!P) TVGB_CUDA(cudaMemsetAsync(po.B, 0, n * 16, st));   // no plate: zero plate records

    SurVoteArgs a{};
    FastArgs& fa = a.f;
    fa.A = po.A; fa.B = po.B; fa.C = po.C;
    fa.s0 = int(s0); fa.s1 = int(s1); fa.s2 = int(s2); fa.hw = hw;
    fa.sig1 = p->sigma1; fa.sig2 = p->sigma2;
    fa.out = dout.get<float>(); fa.out_layout = out_layout; fa.evals = dev_.get<float>(); fa.evecs = dvec.get<float>();
    fa.evec_fmt = nv ? evec_format : 0;
    fa.precise_eig = p->parity ? 0 : 1;
    a.inv_sig = 1.0f / p->sigma1;
    a.tol = tol;
    // the network's weight image, then an error flag for the tensor-core waits
    TVGB_TRY(snet.alloc(TC_IMG_BYTES + 16, st));
    a.err = reinterpret_cast<int*>(static_cast<char*>(snet.p) + TC_IMG_BYTES);
    TVGB_CUDA(cudaMemsetAsync(a.err, 0, sizeof(int), st));
    if (plate_mode == PLATE_SURROGATE) {
        a.img = snet.get<uint4>();
        TVGB_TRY(sur_upload_tc(net_params, snet.p, st));
    }
    if (B) {
        const size_t nt3 = size_t(W) * W * W;
        TVGB_TRY(stab.alloc(nt3 * 32, st));
        const float* Fnet = nullptr;
        if (plate_mode == PLATE_SURROGATE) {
            std::vector<float> X(nt3 * 8, 0.0f);
            for (size_t i = 0; i < nt3; ++i) {
                const int ox = int(i % W) - hw, oy = int((i / W) % W) - hw, oz = int(i / (size_t(W) * W)) - hw;
                const int L2 = ox * ox + oy * oy + oz * oz;
                const float il = L2 ? 1.0f / std::sqrt(float(L2)) : 0.0f;   // o = 0 is tabulated exactly
                float dv[3] = {ox * il, oy * il, oz * il}, nv[3];
                sur_canonical(dv, nv, false);       // the ball does not depend on the normal
                X[i * 8 + 0] = dv[0]; X[i * 8 + 1] = dv[1]; X[i * 8 + 2] = dv[2];
                X[i * 8 + 3] = nv[0]; X[i * 8 + 4] = nv[1]; X[i * 8 + 5] = nv[2];
            }
            TVGB_TRY(sX.alloc(nt3 * 32, st));
            TVGB_TRY(sY.alloc(nt3 * 32, st));
            TVGB_CUDA(cudaMemcpyAsync(sX.p, X.data(), nt3 * 32, cudaMemcpyHostToDevice, st));
            TVGB_TRY(sur_eval_tc_device(snet.p, sX.get<float>(), nt3, sY.get<float>(), 1, a.err, st));
            TVGB_CUDA(cudaStreamSynchronize(st));   // X leaves scope
            Fnet = sY.get<float>();
        }
        const unsigned gb = unsigned(std::min<size_t>((nt3 + 255) / 256, 4096));
        if (plate_mode == PLATE_SURROGATE) {
            TVGB_TRY(stabx.alloc(nt3 * 32, st));
            k_ball_table<PLATE_CLOSED><<<gb, 256, 0, st>>>(hw, p->sigma1, p->sigma2, a.inv_sig, nullptr,
                                                           stabx.get<float>());
            TVGB_LAUNCHED();
            a.ball_exact = stabx.get<float>();
        }
        if (plate_mode == PLATE_SURROGATE)
            k_ball_table<PLATE_SURROGATE><<<gb, 256, 0, st>>>(hw, p->sigma1, p->sigma2, a.inv_sig, Fnet, stab.get<float>());
        else if (plate_mode == PLATE_CLOSED)
            k_ball_table<PLATE_CLOSED><<<gb, 256, 0, st>>>(hw, p->sigma1, p->sigma2, a.inv_sig, Fnet, stab.get<float>());
        else
            k_ball_table<PLATE_PLAIN64><<<gb, 256, 0, st>>>(hw, p->sigma1, p->sigma2, a.inv_sig, Fnet, stab.get<float>());
        TVGB_LAUNCHED();
        a.ball_tab = stab.get<float>();
    }
    TVGB_TRY(sst.alloc(16, st));
    TVGB_CUDA(cudaMemsetAsync(sst.p, 0, 16, st));
    a.stats = sst.get<unsigned>();
    const int nt = 3 * hw * hw + 1;
    size_t smem = size_t(2) * nt * 16;
    if (plate_mode == PLATE_SURROGATE) {
        // the weight image before the radial table; at least TC_SMEM_PER_CTA, so
        // that no more CTAs share an SM than its tensor memory holds
        smem += TC_IMG_BYTES;
        if (smem < size_t(TC_SMEM_PER_CTA)) smem = TC_SMEM_PER_CTA;
    }
    TVGB_CHECK_ARG(smem <= 200 * 1024, "tvgb_vote3_surrogate: window w = %u too large", w);
    dim3 grid(ceil_div(s2, 32u), ceil_div(s1, 4u), s0);
    if (plate_mode == PLATE_SURROGATE) TVGB_TRY(launch_sur<PLATE_SURROGATE>(a, S, B, grid, smem, st));
    else if (plate_mode == PLATE_CLOSED) TVGB_TRY(launch_sur<PLATE_CLOSED>(a, S, B, grid, smem, st));
    else TVGB_TRY(launch_sur<PLATE_PLAIN64>(a, S, B, grid, smem, st));
    unsigned hst[2] = {0, 0};
    int herr = 0;
    TVGB_CUDA(cudaMemcpyAsync(hst, sst.p, 8, cudaMemcpyDeviceToHost, st));
    TVGB_CUDA(cudaMemcpyAsync(&herr, a.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    TVGB_TRY(dout.finish());
    TVGB_TRY(dev_.finish());
    TVGB_TRY(dvec.finish());
    TVGB_CUDA(cudaStreamSynchronize(st));
    if (herr) {
        set_error("tvgb_vote3_surrogate: a tensor-core wait timed out");
        return TVGB_ERR_CUDA;
    }
    if (stats) { stats[0] = hst[0]; stats[1] = hst[1]; }
    return TVGB_OK;
}
