// The learned plate / ball vote: training data from the plain orientation
// integral, quantisation-aware training of the MLP (surrogate_mlp.cuh) by
// this file's own forward / backward / Adam kernels, and its tensor-core
// evaluation.  The vote kernel that uses it is in vote3.cu.
//
// What is learned.  For sigma2 = 0 and power 1 the plate vote of a voter with
// unit plate scale and normal n at offset o != 0 is c1(|o|) F_plate(o/|o|, n)
// and the ball vote is c1(|o|) F_ball(o/|o|), c1 = exp(-|o|^2 / sigma^2).
// The network maps (o / |o|, n, flag) -> F (6 components, xx xy xz yy yz
// zz; flag 1 = plate, 0 = ball); the Gaussian is applied analytically, so
// the offset enters as its direction (fed as o / sigma, the network had 4x
// the error: it must then learn the normalisation, singular at o = 0).  The
// training targets are the plain orientation integral with 64 orientations:
// (1/64) sum_i (1 - (q_i.d)^2) r_i r_i^T over q_i on the great circle normal
// to n (the reference's plate rule, tensorvote.h:2457 plate3_numerical_device,
// with its (u, v) basis) or over an 8 x 8 sphere rule (ball), r = q - 2 (q.d) d.
#include "tvgb_internal.cuh"
#include "surrogate_mlp.cuh"
#include "sur_tc.cuh"
#include <cmath>
#include <cstring>
#include <vector>

namespace tvgb {

// ---------------------------------------------------------------- host helpers

static uint16_t bf16_bits(float f) {          // round to nearest even
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) != 0x7f800000u) u += 0x7fffu + ((u >> 16) & 1u);
    return uint16_t(u >> 16);
}

// a bias as the two BF16 values whose sum the MMA forms in FP32
static void bias_split(float b, float& hi, float& lo) {
    const uint32_t u = uint32_t(bf16_bits(b)) << 16;
    std::memcpy(&hi, &u, 4);
    lo = b - hi;
}

// layer 1's weight meeting K column k of the input row (sur_row64's layout):
// W1 for a feature or its residual, the split b1 for the bias pair
static float w1_at(const float* P, int j, int k) {
    if (k < SUR_IN) return P[SUR_W1 + j * SUR_IN + k];
    if (k == SUR_IN || k == SUR_IN + 1) {
        float hi, lo;
        bias_split(P[SUR_B1 + j], hi, lo);
        return k == SUR_IN ? hi : lo;
    }
    if (k >= 32 && k < 32 + SUR_IN) return P[SUR_W1 + j * SUR_IN + (k - 32)];
    return 0.0f;
}

void sur_make_fragments(const float* P, uint2* frag, float* bias) {
    struct L { int w, kin, nout, kt, nt, fbase; };
    const L layers[4] = {{SUR_W1, SUR_K1, SUR_H, 4, 8, SUR_F1}, {SUR_W2, SUR_H, SUR_H, 4, 8, SUR_F2},
                         {SUR_W3, SUR_H, SUR_H, 4, 8, SUR_F3}, {SUR_W4, SUR_H, SUR_OUT, 4, 1, SUR_F4}};
    for (const L& l : layers) {
        auto w = [&](int j, int k) {
            if (l.fbase == SUR_F1) return w1_at(P, j, k);
            return k < l.kin ? P[l.w + j * l.kin + k] : 0.0f;
        };
        for (int kt = 0; kt < l.kt; ++kt)
            for (int nt = 0; nt < l.nt; ++nt)
                for (int lane = 0; lane < 32; ++lane) {
                    const int g = lane >> 2, t = lane & 3, j = nt * 8 + g, k0 = kt * 16 + 2 * t;
                    uint2 f;
                    f.x = uint32_t(bf16_bits(w(j, k0))) | (uint32_t(bf16_bits(w(j, k0 + 1))) << 16);
                    f.y = uint32_t(bf16_bits(w(j, k0 + 8))) | (uint32_t(bf16_bits(w(j, k0 + 9))) << 16);
                    frag[(l.fbase + kt * l.nt + nt) * 32 + lane] = f;
                }
    }
    for (int i = 0; i < SUR_H; ++i) {
        bias[i] = P[SUR_B1 + i];
        bias[SUR_H + i] = P[SUR_B2 + i];
        bias[2 * SUR_H + i] = P[SUR_B3 + i];
    }
    for (int i = 0; i < SUR_OUT; ++i) bias[3 * SUR_H + i] = P[SUR_B4 + i];
}

void sur_make_tc_image(const float* P, uint16_t* img) {
    std::memset(img, 0, TC_IMG_BYTES);
    // element (n, k) of an N x K K-major matrix in 8 x 8 core matrices (no swizzle)
    auto put = [&](int base, int K, int n, int k, float v) {
        const int byte = base + (n >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (n & 7) * 16 + (k & 7) * 2;
        img[byte / 2] = bf16_bits(v);
    };
    // a bias as the two BF16 values whose sum the MMA forms in FP32
    auto put_bias = [&](int base, int K, int n, int k, float b) {
        float hi, lo;
        bias_split(b, hi, lo);
        put(base, K, n, k, hi);
        put(base, K, n, k + 1, lo);
    };
    for (int n = 0; n < SUR_H; ++n) {
        // layer 1: features, the bias pair, the features' residuals (sur_row64's K layout)
        for (int k = 0; k < TC_K1; ++k) put(TC_B1, TC_K1, n, k, w1_at(P, n, k));
        for (int k = 0; k < SUR_H; ++k) {
            put(TC_B2, TC_KH, n, k, P[SUR_W2 + n * SUR_H + k]);
            put(TC_B3, TC_KH, n, k, P[SUR_W3 + n * SUR_H + k]);
        }
        put_bias(TC_B2, TC_KH, n, SUR_H, P[SUR_B2 + n]);
        put_bias(TC_B3, TC_KH, n, SUR_H, P[SUR_B3 + n]);
    }
    for (int n = 0; n < SUR_OUT; ++n) {
        for (int k = 0; k < SUR_H; ++k) put(TC_B4, TC_KH, n, k, P[SUR_W4 + n * SUR_H + k]);
        put_bias(TC_B4, TC_KH, n, SUR_H, P[SUR_B4 + n]);
    }
}

// ---------------------------------------------------------------- training data

// splitmix64 (Steele, Lea and Flood's SplitMix generator, as published by
// Vigna): a counter-based stream per sample
__device__ __forceinline__ uint64_t smix(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ float u01(uint64_t& s) {
    s = smix(s);
    return (float(s >> 40) + 0.5f) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ float gauss(uint64_t& s) {     // Box-Muller
    const float a = u01(s), b = u01(s);
    return sqrtf(-2.0f * logf(a)) * cospif(2.0f * b);
}

__device__ __forceinline__ void stick_unit_f(const float* q, const float* d, float w, float* F) {
    const float qd = q[0] * d[0] + q[1] * d[1] + q[2] * d[2];
    const float eta = w * (1.0f - qd * qd);
    const float r0 = q[0] - 2.0f * qd * d[0], r1 = q[1] - 2.0f * qd * d[1], r2 = q[2] - 2.0f * qd * d[2];
    F[0] += eta * r0 * r0; F[1] += eta * r0 * r1; F[2] += eta * r0 * r2;
    F[3] += eta * r1 * r1; F[4] += eta * r1 * r2; F[5] += eta * r2 * r2;
}

__constant__ float c_gl8x[8] = {-0.9602898564975363f, -0.7966664774136267f, -0.5255324099163290f,
                                -0.1834346424956498f, 0.1834346424956498f,  0.5255324099163290f,
                                0.7966664774136267f,  0.9602898564975363f};
__constant__ float c_gl8w[8] = {0.1012285362903763f, 0.2223810344533745f, 0.3137066458778873f,
                                0.3626837833783620f, 0.3626837833783620f, 0.3137066458778873f,
                                0.2223810344533745f, 0.1012285362903763f};

// Inputs: the offset direction d uniform on the sphere (for sigma2 = 0 the
// vote's angular part depends on the direction only: the Gaussian carries
// the radius), n uniform on the sphere, plate or ball with probability 1/2.
__global__ void k_sur_samples(size_t n, unsigned long long seed, float* __restrict__ X, float* __restrict__ T) {
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        uint64_t s = smix(seed ^ smix(i + 0x51ed2701ull));
        float x[3] = {gauss(s), gauss(s), gauss(s)};
        float xl = sqrtf(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        if (!(xl > 1e-6f)) { x[0] = 1; x[1] = 0; x[2] = 0; xl = 1; }
        for (int k = 0; k < 3; ++k) x[k] /= xl;
        float nv[3] = {gauss(s), gauss(s), gauss(s)};
        float nl = sqrtf(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
        if (!(nl > 1e-6f)) { nv[0] = 0; nv[1] = 0; nv[2] = 1; nl = 1; }
        for (int k = 0; k < 3; ++k) nv[k] /= nl;
        const bool plate = u01(s) < 0.5f;
        const float dl = sqrtf(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        const float d[3] = {x[0] / dl, x[1] / dl, x[2] / dl};
        float F[6] = {0, 0, 0, 0, 0, 0};
        if (plate) {
            float u[3];
            if (fabsf(nv[2]) < 0.999f) { u[0] = nv[1]; u[1] = -nv[0]; u[2] = 0.0f; }
            else { u[0] = 0.0f; u[1] = nv[2]; u[2] = -nv[1]; }
            const float ul = sqrtf(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
            for (int k = 0; k < 3; ++k) u[k] /= ul;
            const float v[3] = {nv[1] * u[2] - nv[2] * u[1], nv[2] * u[0] - nv[0] * u[2], nv[0] * u[1] - nv[1] * u[0]};
            for (int q = 0; q < 64; ++q) {
                float sn, cs;
                sincospif(float(q) / 64.0f, &sn, &cs);
                const float qq[3] = {cs * u[0] + sn * v[0], cs * u[1] + sn * v[1], cs * u[2] + sn * v[2]};
                stick_unit_f(qq, d, 1.0f / 64.0f, F);
            }
        } else {
            for (int a = 0; a < 8; ++a)
                for (int b = 0; b < 8; ++b) {
                    const float ct = c_gl8x[a], st = sqrtf(1.0f - ct * ct);
                    float sp, cp;
                    sincospif(float(b) / 4.0f, &sp, &cp);
                    const float qq[3] = {st * cp, st * sp, ct};
                    stick_unit_f(qq, d, c_gl8w[a] * (1.0f / 16.0f), F);
                }
        }
        float* xo = X + i * 8;
        float* to = T + i * 8;
        sur_canonical(x, nv, plate);      // the target is the same at the canonical inputs
        xo[0] = x[0]; xo[1] = x[1]; xo[2] = x[2]; xo[3] = nv[0]; xo[4] = nv[1]; xo[5] = nv[2];
        xo[6] = plate ? 1.0f : 0.0f; xo[7] = 0.0f;
        for (int k = 0; k < 6; ++k) to[k] = F[k];
        to[6] = 0.0f; to[7] = 0.0f;
    }
}

// ---------------------------------------------------------------- training

constexpr int TRB = 32;          // samples per CTA
constexpr int TRS = SUR_H + 1;   // transposed weight row stride (conflict-free both ways)

__device__ __forceinline__ float bq(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float gelu_grad(float z) {
    const float t = tanhf(GELU_K * (z + GELU_A * z * z * z));
    return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * GELU_K * (1.0f + 3.0f * GELU_A * z * z);
}

struct TrainShared {
    float w1t[SUR_IN * TRS];     // [k][j] = bf16(W1[j][k])
    float w2t[SUR_H * TRS];
    float w3t[SUR_H * TRS];
    float w4t[SUR_H * 9];        // [k][o]
    float b[SUR_NBIAS];
    float h0[TRB * SUR_IN];
    float z1[TRB * SUR_H], h1[TRB * SUR_H], z2[TRB * SUR_H], h2[TRB * SUR_H], z3[TRB * SUR_H], h3[TRB * SUR_H];
    float dy[TRB * SUR_OUT];
    float loss[8];
};

// Forward + backward of TRB samples per CTA (the quantised forward of the
// tensor-core inference, its packed-BF16 GELU included; the rounding is the
// identity in the backward pass, which differentiates the smooth GELU).
// Each CTA writes its gradient sum and loss sum to part[blockIdx] (NPARAM + 1
// floats): the reduction over CTAs happens in k_sur_adam in a fixed order.
__global__ void __launch_bounds__(256) k_sur_fwd_bwd(const float* __restrict__ P, const float* __restrict__ X,
                                                     const float* __restrict__ T, size_t n, size_t first, int batch,
                                                     float* __restrict__ part) {
    extern __shared__ __align__(16) float sm_raw[];
    TrainShared& S = *reinterpret_cast<TrainShared*>(sm_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int e = tid; e < SUR_H * SUR_IN; e += 256) { const int j = e / SUR_IN, k = e % SUR_IN; S.w1t[k * TRS + j] = bq(P[SUR_W1 + e]); }
    for (int e = tid; e < SUR_H * SUR_H; e += 256) {
        const int j = e / SUR_H, k = e % SUR_H;
        S.w2t[k * TRS + j] = bq(P[SUR_W2 + e]);
        S.w3t[k * TRS + j] = bq(P[SUR_W3 + e]);
    }
    for (int e = tid; e < SUR_OUT * SUR_H; e += 256) { const int o = e / SUR_H, k = e % SUR_H; S.w4t[k * 9 + o] = bq(P[SUR_W4 + e]); }
    for (int e = tid; e < SUR_H; e += 256) { S.b[e] = P[SUR_B1 + e]; S.b[SUR_H + e] = P[SUR_B2 + e]; S.b[2 * SUR_H + e] = P[SUR_B3 + e]; }
    if (tid < SUR_OUT) S.b[3 * SUR_H + tid] = P[SUR_B4 + tid];
    const size_t base = first + size_t(blockIdx.x) * TRB;
    // each feature as the first layer sees it: bf16(f) + bf16 of its residual
    if (tid < TRB) {
        const float* xs = X + ((base + tid) % n) * 8;
        float x[SUR_X], f[SUR_IN];
        for (int k = 0; k < SUR_X; ++k) x[k] = xs[k];
        sur_features(x, f);
        for (int k = 0; k < SUR_IN; ++k) S.h0[tid * SUR_IN + k] = bq(f[k]) + bq(bf16_residual(f[k]));
    }
    __syncthreads();

    // hidden layers: thread (warp, lane) -> outputs j = lane, lane + 32 of samples warp + 8 i
    auto hidden = [&](const float* in, int kin, const float* wt, const float* bb, float* z, float* h) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int s = warp + 8 * i;
            float a0 = bb[lane], a1 = bb[lane + 32];
            for (int k = 0; k < kin; ++k) {
                const float x = in[s * kin + k];
                a0 = fmaf(wt[k * TRS + lane], x, a0);
                a1 = fmaf(wt[k * TRS + lane + 32], x, a1);
            }
            z[s * SUR_H + lane] = a0; z[s * SUR_H + lane + 32] = a1;
            // the inference's activation of units lane and lane + 32 (the same kind)
            const uint32_t g2 = gelu_unit_pair(a0, a1, gelu_is_poly(lane));
            h[s * SUR_H + lane] = __uint_as_float(g2 << 16);
            h[s * SUR_H + lane + 32] = __uint_as_float(g2 & 0xffff0000u);
        }
    };
    hidden(S.h0, SUR_IN, S.w1t, S.b, S.z1, S.h1);
    __syncthreads();
    hidden(S.h1, SUR_H, S.w2t, S.b + SUR_H, S.z2, S.h2);
    __syncthreads();
    hidden(S.h2, SUR_H, S.w3t, S.b + 2 * SUR_H, S.z3, S.h3);
    __syncthreads();
    {   // output layer, loss and dL/dy: thread -> (sample tid / 8, output tid % 8)
        const int s = tid >> 3, o = tid & 7;
        float y = S.b[3 * SUR_H + o];
        for (int k = 0; k < SUR_H; ++k) y = fmaf(S.w4t[k * 9 + o], S.h3[s * SUR_H + k], y);
        float d = 0.0f;
        if (o < 6) d = y - T[((base + s) % n) * 8 + o];
        S.dy[s * SUR_OUT + o] = 2.0f * d / float(batch);
        float l = d * d / float(batch);
        for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
        if (lane == 0) S.loss[warp] = l;
    }
    __syncthreads();
    float* g = part + size_t(blockIdx.x) * (SUR_NPARAM + 1);
    // dz3 = (W4q^T dy) * gelu'(z3), in place of z3
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int s = warp + 8 * i;
        for (int kk = 0; kk < 2; ++kk) {
            const int k = lane + 32 * kk;
            float a = 0.0f;
            for (int o = 0; o < SUR_OUT; ++o) a = fmaf(S.w4t[k * 9 + o], S.dy[s * SUR_OUT + o], a);
            S.z3[s * SUR_H + k] = a * gelu_grad(S.z3[s * SUR_H + k]);
        }
    }
    // gradients of the output layer
    for (int e = tid; e < SUR_OUT * SUR_H; e += 256) {
        const int o = e / SUR_H, k = e % SUR_H;
        float a = 0.0f;
        for (int s = 0; s < TRB; ++s) a = fmaf(S.dy[s * SUR_OUT + o], S.h3[s * SUR_H + k], a);
        g[SUR_W4 + e] = a;
    }
    if (tid < SUR_OUT) {
        float a = 0.0f;
        for (int s = 0; s < TRB; ++s) a += S.dy[s * SUR_OUT + tid];
        g[SUR_B4 + tid] = a;
    }
    if (tid == 0) {
        float l = 0.0f;
        for (int w = 0; w < 8; ++w) l += S.loss[w];
        g[SUR_NPARAM] = l;
    }
    __syncthreads();
    // hidden layers, from the top: dz_{l-1} = (Wl_q^T dz_l) * gelu'(z_{l-1}); grad Wl = dz_l h_{l-1}^T
    auto back = [&](const float* wt, const float* dz, const float* hprev, int kin, float* zprev, int woff, int boff) {
        if (zprev) {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int s = warp + 8 * i;
                for (int kk = 0; kk < 2; ++kk) {
                    const int k = lane + 32 * kk;
                    float a = 0.0f;
                    for (int j = 0; j < SUR_H; ++j) a = fmaf(wt[k * TRS + j], dz[s * SUR_H + j], a);
                    zprev[s * SUR_H + k] = a * gelu_grad(zprev[s * SUR_H + k]);
                }
            }
        }
        for (int e = tid; e < SUR_H * kin; e += 256) {
            const int j = e / kin, k = e % kin;
            float a = 0.0f;
            for (int s = 0; s < TRB; ++s) a = fmaf(dz[s * SUR_H + j], hprev[s * kin + k], a);
            g[woff + e] = a;
        }
        if (tid < SUR_H) {
            float a = 0.0f;
            for (int s = 0; s < TRB; ++s) a += dz[s * SUR_H + tid];
            g[boff + tid] = a;
        }
    };
    back(S.w3t, S.z3, S.h2, SUR_H, S.z2, SUR_W3, SUR_B3);
    __syncthreads();
    back(S.w2t, S.z2, S.h1, SUR_H, S.z1, SUR_W2, SUR_B2);
    __syncthreads();
    back(S.w1t, S.z1, S.h0, SUR_IN, nullptr, SUR_W1, SUR_B1);
}

// Adam over the CTA partial sums (fixed order: deterministic); the padded
// parameters get zero gradients and stay zero.  part[b][NPARAM] is the loss.
__global__ void k_sur_adam(float* __restrict__ P, float* __restrict__ M, float* __restrict__ V,
                           const float* __restrict__ part, int nblk, float lr, float bc1, float bc2,
                           float* __restrict__ loss_out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > SUR_NPARAM) return;
    float gsum = 0.0f;
    for (int b = 0; b < nblk; ++b) gsum += part[size_t(b) * (SUR_NPARAM + 1) + p];
    if (p == SUR_NPARAM) {
        if (loss_out) *loss_out = gsum;
        return;
    }
    const float m = 0.9f * M[p] + 0.1f * gsum;
    const float v = 0.999f * V[p] + 0.001f * gsum * gsum;
    M[p] = m;
    V[p] = v;
    P[p] -= lr * (m / bc1) / (sqrtf(v / bc2) + 1e-8f);
}

// the CTA partials summed in a fixed order: grad[0 .. NPARAM) and *loss
__global__ void k_sur_gradsum(const float* __restrict__ part, int nblk, float* __restrict__ grad,
                              float* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > SUR_NPARAM) return;
    float s = 0.0f;
    for (int b = 0; b < nblk; ++b) s += part[size_t(b) * (SUR_NPARAM + 1) + p];
    if (p < SUR_NPARAM) grad[p] = s;
    else *loss = s;
}

// ---------------------------------------------------------------- tensor-core evaluation

__global__ void __launch_bounds__(128) k_sur_eval(const uint2* __restrict__ frag_g, const float* __restrict__ bias_g,
                                                  const float* __restrict__ X, size_t n, float* __restrict__ Y) {
    __shared__ uint2 frag[SUR_NFRAG * 32];
    __shared__ float bias[SUR_NBIAS];
    for (int e = threadIdx.x; e < SUR_NFRAG * 32; e += blockDim.x) frag[e] = frag_g[e];
    for (int e = threadIdx.x; e < SUR_NBIAS; e += blockDim.x) bias[e] = bias_g[e];
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const size_t warps = size_t(gridDim.x) * (blockDim.x >> 5);
    for (size_t tile = size_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 16 < n; tile += warps) {
        const size_t r0 = tile * 16 + g, r1 = r0 + 8;
        float x0[SUR_X] = {0, 0, 0, 0, 0, 0, 0}, x1[SUR_X] = {0, 0, 0, 0, 0, 0, 0};
        if (r0 < n) for (int k = 0; k < SUR_X; ++k) x0[k] = X[r0 * 8 + k];
        if (r1 < n) for (int k = 0; k < SUR_X; ++k) x1[k] = X[r1 * 8 + k];
        uint32_t row0[SUR_K1 / 2], row1[SUR_K1 / 2];
        sur_row64(x0, row0);
        sur_row64(x1, row1);
        if (r0 >= n) for (int i = 0; i < SUR_K1 / 2; ++i) row0[i] = 0u;
        if (r1 >= n) for (int i = 0; i < SUR_K1 / 2; ++i) row1[i] = 0u;
        // A fragment of k-tile kt: rows g / g + 8, columns 16 kt + 2 t (pair 8 kt + t) and + 8 (pair 8 kt + 4 + t)
        uint32_t a[4][4];
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            a[kt][0] = row0[8 * kt + t];
            a[kt][1] = row1[8 * kt + t];
            a[kt][2] = row0[8 * kt + 4 + t];
            a[kt][3] = row1[8 * kt + 4 + t];
        }
        float out[4];
        sur_mlp16(frag, bias, a, out);
        if (r0 < n) { Y[r0 * 8 + 2 * t] = out[0]; Y[r0 * 8 + 2 * t + 1] = out[1]; }
        if (r1 < n) { Y[r1 * 8 + 2 * t] = out[2]; Y[r1 * 8 + 2 * t + 1] = out[3]; }
    }
}

// The network on tcgen05: one 128-sample tile per CTA iteration (sur_tc.cuh).
template <int GM>
__global__ void __launch_bounds__(128) k_sur_eval_tc(const uint4* __restrict__ img_g, const float* __restrict__ X,
                                                     size_t n, float* __restrict__ Y, int* __restrict__ err,
                                                     uint32_t wait_limit) {
    extern __shared__ __align__(128) uint4 img_s[];
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) uint64_t bar;
    SurTc s;
    sur_tc_setup(s, img_g, img_s, &tmem_slot, &bar, wait_limit);
    const size_t ntiles = (n + 127) / 128;
    for (size_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const size_t row = tile * 128 + threadIdx.x;
        float4 x0 = make_float4(0, 0, 0, 0), x1 = x0;
        if (row < n) {
            x0 = reinterpret_cast<const float4*>(X)[row * 2];
            x1 = reinterpret_cast<const float4*>(X)[row * 2 + 1];
        }
        const float x[SUR_X] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z};
        uint32_t in[SUR_K1 / 2];
        sur_row64(x, in);
        float out[8];
        if (!sur_tc_forward<GM>(s, in, out)) break;
        if (row < n) {
            reinterpret_cast<float4*>(Y)[row * 2] = make_float4(out[0], out[1], out[2], out[3]);
            reinterpret_cast<float4*>(Y)[row * 2 + 1] = make_float4(out[4], out[5], out[6], out[7]);
        }
    }
    if (!sur_tc_teardown(s) && threadIdx.x == 0) atomicExch(err, 1);
}

// the weight image on the device (TC_IMG_BYTES)
int sur_upload_tc(const float* params_host_or_dev, void* img_dev, cudaStream_t st) {
    std::vector<float> P(SUR_NPARAM);
    if (is_device_ptr(params_host_or_dev)) {
        TVGB_CUDA(cudaMemcpyAsync(P.data(), params_host_or_dev, SUR_NPARAM * 4, cudaMemcpyDeviceToHost, st));
        TVGB_CUDA(cudaStreamSynchronize(st));
    } else {
        std::memcpy(P.data(), params_host_or_dev, SUR_NPARAM * 4);
    }
    std::vector<uint16_t> img(TC_IMG_BYTES / 2);
    sur_make_tc_image(P.data(), img.data());
    TVGB_CUDA(cudaMemcpyAsync(img_dev, img.data(), TC_IMG_BYTES, cudaMemcpyHostToDevice, st));
    TVGB_CUDA(cudaStreamSynchronize(st));   // the host vector goes out of scope
    return TVGB_OK;
}

int sur_eval_tc_device(const void* img, const float* X, size_t n, float* Y, int gelu_mode, int* err,
                       cudaStream_t st, uint32_t wait_limit) {
    if (n == 0) return TVGB_OK;
    const size_t tiles = (n + 127) / 128;
    const unsigned grid = unsigned(tiles < 152 * 4 ? tiles : 152 * 4);
    const int smem = TC_SMEM_PER_CTA;
    const void* fn = gelu_mode == 0 ? (const void*)k_sur_eval_tc<0> : (const void*)k_sur_eval_tc<1>;
    TVGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const uint4* img4 = static_cast<const uint4*>(img);
    void* args[] = {&img4, &X, &n, &Y, &err, &wait_limit};
    {
        KernelTimer kt_("k_sur_eval_tc", st);
        TVGB_CUDA(cudaLaunchKernel(fn, dim3(grid), dim3(128), args, smem, st));
        kt_.stop();
    }
    TVGB_LAUNCHED();
    return TVGB_OK;
}

int sur_upload(const float* params_host_or_dev, uint2* frag_dev, float* bias_dev, cudaStream_t st) {
    std::vector<float> P(SUR_NPARAM);
    if (is_device_ptr(params_host_or_dev)) {
        TVGB_CUDA(cudaMemcpyAsync(P.data(), params_host_or_dev, SUR_NPARAM * 4, cudaMemcpyDeviceToHost, st));
        TVGB_CUDA(cudaStreamSynchronize(st));
    } else {
        std::memcpy(P.data(), params_host_or_dev, SUR_NPARAM * 4);
    }
    std::vector<uint2> frag(SUR_NFRAG * 32);
    std::vector<float> bias(SUR_NBIAS);
    sur_make_fragments(P.data(), frag.data(), bias.data());
    TVGB_CUDA(cudaMemcpyAsync(frag_dev, frag.data(), frag.size() * sizeof(uint2), cudaMemcpyHostToDevice, st));
    TVGB_CUDA(cudaMemcpyAsync(bias_dev, bias.data(), bias.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    TVGB_CUDA(cudaStreamSynchronize(st));   // the host vectors go out of scope
    return TVGB_OK;
}

static unsigned grid_n(size_t n, unsigned per);

int sur_eval_device(const uint2* frag, const float* bias, const float* X, size_t n, float* Y, cudaStream_t st) {
    if (n == 0) return TVGB_OK;
    size_t b = ((n + 15) / 16 + 3) / 4;
    if (b > 152 * 16) b = 152 * 16;
    {
        KernelTimer kt_("k_sur_eval", st);
        k_sur_eval<<<unsigned(b), 128, 0, st>>>(frag, bias, X, n, Y);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    return TVGB_OK;
}

static unsigned grid_n(size_t n, unsigned per) {
    size_t b = (n + per - 1) / per;
    if (b > 152 * 16) b = 152 * 16;
    return unsigned(b ? b : 1);
}

static int fwd_bwd_launch(const float* P, const float* X, const float* T, size_t n, size_t first, int batch,
                          float* part, cudaStream_t st) {
    const size_t smem = sizeof(TrainShared);
    TVGB_CUDA(cudaFuncSetAttribute(k_sur_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    {
        KernelTimer kt_("k_sur_fwd_bwd", st);
        k_sur_fwd_bwd<<<batch / TRB, 256, smem, st>>>(P, X, T, n, first, batch, part);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    return TVGB_OK;
}

}  // namespace tvgb

using namespace tvgb;

extern "C" {

int tvgb_surrogate_param_count(void) { return SUR_NPARAM; }

int tvgb_surrogate_samples(size_t n, unsigned long long seed, float* X, float* T, void* stream) {
    TVGB_CHECK_ARG(X && T, "tvgb_surrogate_samples: NULL pointer");
    if (n == 0) return TVGB_OK;
    cudaStream_t st = as_stream(stream);
    DevArray dx, dt;
    TVGB_TRY(dx.out(X, n * 32, st));
    TVGB_TRY(dt.out(T, n * 32, st));
    {
        KernelTimer kt_("k_sur_samples", st);
        k_sur_samples<<<grid_n(n, 256), 256, 0, st>>>(n, seed, dx.get<float>(), dt.get<float>());
        kt_.stop();
    }
    TVGB_LAUNCHED();
    TVGB_TRY(dx.finish());
    TVGB_TRY(dt.finish());
    return sync_if(dx.owned || dt.owned, st);
}

int tvgb_surrogate_grad(const float* params, const float* X, const float* T, int batch, float* grad, float* loss,
                        void* stream) {
    TVGB_CHECK_ARG(params && X && T && grad, "tvgb_surrogate_grad: NULL pointer");
    TVGB_CHECK_ARG(batch > 0 && batch % TRB == 0 && batch <= (1 << 22),
                   "tvgb_surrogate_grad: batch must be a positive multiple of %d (at most 2^22)", TRB);
    cudaStream_t st = as_stream(stream);
    DevArray dp, dx, dt, dg;
    TVGB_TRY(dp.in(params, SUR_NPARAM * 4, st));
    TVGB_TRY(dx.in(X, size_t(batch) * 32, st));
    TVGB_TRY(dt.in(T, size_t(batch) * 32, st));
    TVGB_TRY(dg.out(grad, SUR_NPARAM * 4, st));
    const int nblk = batch / TRB;
    Scratch part, lbuf;
    TVGB_TRY(part.alloc(size_t(nblk) * (SUR_NPARAM + 1) * 4, st));
    TVGB_TRY(lbuf.alloc(16, st));
    TVGB_TRY(fwd_bwd_launch(dp.get<float>(), dx.get<float>(), dt.get<float>(), size_t(batch), 0, batch,
                            part.get<float>(), st));
    k_sur_gradsum<<<(SUR_NPARAM + 256) / 256, 256, 0, st>>>(part.get<float>(), nblk, dg.get<float>(),
                                                            lbuf.get<float>());
    TVGB_LAUNCHED();
    TVGB_TRY(dg.finish());
    if (loss) {
        TVGB_CUDA(cudaMemcpyAsync(loss, lbuf.get<float>(), 4, cudaMemcpyDeviceToHost, st));
    }
    TVGB_CUDA(cudaStreamSynchronize(st));
    return TVGB_OK;
}

int tvgb_surrogate_train(float* params, const float* X, const float* T, size_t n, int batch, int steps, float lr,
                         float* loss_history, void* stream) {
    TVGB_CHECK_ARG(params && X && T, "tvgb_surrogate_train: NULL pointer");
    TVGB_CHECK_ARG(batch > 0 && batch % TRB == 0 && batch <= (1 << 22),
                   "tvgb_surrogate_train: batch must be a positive multiple of %d (at most 2^22)", TRB);
    TVGB_CHECK_ARG(n >= size_t(batch) && steps >= 0 && lr > 0.0f, "tvgb_surrogate_train: bad sizes or rate");
    cudaStream_t st = as_stream(stream);
    DevArray dp, dx, dt, dl;
    TVGB_TRY(dp.in(params, SUR_NPARAM * 4, st));
    dp.output = true;                      // copied back by finish()
    TVGB_TRY(dx.in(X, n * 32, st));
    TVGB_TRY(dt.in(T, n * 32, st));
    if (loss_history) TVGB_TRY(dl.out(loss_history, size_t(steps) * 4, st));
    const int nblk = batch / TRB;
    Scratch part, mv;
    TVGB_TRY(part.alloc(size_t(nblk) * (SUR_NPARAM + 1) * 4, st));
    TVGB_TRY(mv.alloc(size_t(2) * SUR_NPARAM * 4, st));
    TVGB_CUDA(cudaMemsetAsync(mv.get<float>(), 0, size_t(2) * SUR_NPARAM * 4, st));
    double b1 = 1.0, b2 = 1.0;
    for (int s = 0; s < steps; ++s) {
        b1 *= 0.9; b2 *= 0.999;
        // cosine decay to 1 % of the initial rate
        const float f = 0.01f + 0.99f * 0.5f * (1.0f + std::cos(3.14159265f * float(s) / float(steps)));
        TVGB_TRY(fwd_bwd_launch(dp.get<float>(), dx.get<float>(), dt.get<float>(), n, (size_t(s) * batch) % n, batch,
                                part.get<float>(), st));
        {
            KernelTimer kt_("k_sur_adam", st);
            k_sur_adam<<<(SUR_NPARAM + 256) / 256, 256, 0, st>>>(
                dp.get<float>(), mv.get<float>(), mv.get<float>() + SUR_NPARAM, part.get<float>(), nblk, lr * f,
                float(1.0 - b1), float(1.0 - b2), loss_history ? dl.get<float>() + s : nullptr);
            kt_.stop();
        }
        TVGB_LAUNCHED();
    }
    TVGB_TRY(dp.finish());
    TVGB_TRY(dl.finish());
    TVGB_CUDA(cudaStreamSynchronize(st));
    return TVGB_OK;
}

int tvgb_surrogate_eval(const float* params, const float* X, size_t n, float* Y, void* stream) {
    TVGB_CHECK_ARG(params && X && Y, "tvgb_surrogate_eval: NULL pointer");
    if (n == 0) return TVGB_OK;
    cudaStream_t st = as_stream(stream);
    DevArray dx, dy;
    TVGB_TRY(dx.in(X, n * 32, st));
    TVGB_TRY(dy.out(Y, n * 32, st, true));
    Scratch net;
    TVGB_TRY(net.alloc(SUR_NFRAG * 32 * sizeof(uint2) + SUR_NBIAS * 4, st));
    uint2* frag = net.get<uint2>();
    float* bias = reinterpret_cast<float*>(frag + SUR_NFRAG * 32);
    TVGB_TRY(sur_upload(params, frag, bias, st));
    TVGB_TRY(sur_eval_device(frag, bias, dx.get<float>(), n, dy.get<float>(), st));
    TVGB_TRY(dy.finish());
    return sync_if(dx.owned || dy.owned, st);
}

int tvgb_surrogate_eval_tc(const float* params, const float* X, size_t n, float* Y, int gelu_mode, void* stream) {
    return tvgb_surrogate_eval_tc_limit(params, X, n, Y, gelu_mode, -1, stream);
}

int tvgb_surrogate_eval_tc_limit(const float* params, const float* X, size_t n, float* Y, int gelu_mode,
                                 long long wait_limit, void* stream) {
    TVGB_CHECK_ARG(params && X && Y, "tvgb_surrogate_eval_tc: NULL pointer");
    TVGB_CHECK_ARG(gelu_mode == 0 || gelu_mode == 1, "tvgb_surrogate_eval_tc: gelu_mode must be 0 or 1");
    TVGB_CHECK_ARG(wait_limit <= (long long)TC_WAIT_LIMIT,
                   "tvgb_surrogate_eval_tc_limit: wait_limit above the default %u", TC_WAIT_LIMIT);
    const uint32_t limit = wait_limit < 0 ? TC_WAIT_LIMIT : uint32_t(wait_limit);
    if (n == 0) return TVGB_OK;
    cudaStream_t st = as_stream(stream);
    DevArray dx, dy;
    TVGB_TRY(dx.in(X, n * 32, st));
    TVGB_TRY(dy.out(Y, n * 32, st, true));
    Scratch net;
    TVGB_TRY(net.alloc(TC_IMG_BYTES + 16, st));
    int* err = reinterpret_cast<int*>(static_cast<char*>(net.p) + TC_IMG_BYTES);
    TVGB_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    TVGB_TRY(sur_upload_tc(params, net.p, st));
    TVGB_TRY(sur_eval_tc_device(net.p, dx.get<float>(), n, dy.get<float>(), gelu_mode, err, st, limit));
    int herr = 0;
    TVGB_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    TVGB_TRY(dy.finish());
    TVGB_CUDA(cudaStreamSynchronize(st));
    if (herr) {
        set_error("tvgb_surrogate_eval_tc: a tensor-core wait timed out");
        return TVGB_ERR_CUDA;
    }
    return TVGB_OK;
}

}  // extern "C"
