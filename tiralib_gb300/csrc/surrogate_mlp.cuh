// The plate / ball vote surrogate's network on the tensor cores.
//
// MLP 28 -> 64 -> 64 -> 64 -> 6 (GELU) from the 28 features of (offset
// direction d = o / |o|, plate normal n, flag 1 plate / 0 ball): d, n, the
// flag, and the degree-2 monomials d_i d_j, n_i n_j (6 each) and d_i n_j (9).
// The vote's angular part is a polynomial in d and n (degree 6), so the
// monomials give the network part of its structure for free: trained alike,
// its held-out error fell from 0.40% to 0.24% against the 7 raw inputs.
// Outputs padded to 8.  Weights and activations are bfloat16, accumulation
// FP32: mma.sync.m16n8k16 (BF16) with each warp carrying 16 samples.  A
// layer's FP32 accumulators, after GELU, are packed to bfloat16 and become
// the next layer's A fragments in the same registers: the accumulator of
// n-tiles 2k and 2k+1 is exactly the A fragment of k-tile k, so the whole
// network runs without touching shared memory for activations.  Weights are
// pre-arranged per (layer, k-tile, n-tile, lane) as the B fragment each lane
// holds (two 32-bit registers), so each MMA needs one 64-bit shared load.
//
// Layer 1's input row (K = 64, sur_row64): the 28 features at K 0..27, a
// (1, 1) pair at K 28, 29 that meets the bias split as bf16(b1) and
// bf16(b1 - bf16(b1)) in the weights, and the features' BF16 residuals at
// K 32..59 against the same weights as the features, so each feature
// reaches the tensor cores with ~16 significant bits.  Layers 2..4 take
// their bias as the accumulator's initial value (mma.sync) or through a
// constant K block (tcgen05, sur_tc.cuh).
//
// Parameter layout (FP32 master copy):
//   W1[64][28] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[8][64] b4[8]
// with W[out][in]; W4[6..7][.] and b4[6..7] stay zero.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace tvgb {

constexpr int SUR_X = 7;                         // raw inputs (d, n, flag); sample rows hold 8 floats
constexpr int SUR_IN = 28, SUR_H = 64, SUR_OUT = 8;
constexpr int SUR_K1 = 64;                       // layer 1's K: features, bias pair, residuals
constexpr int SUR_W1 = 0;
constexpr int SUR_B1 = SUR_W1 + SUR_H * SUR_IN;
constexpr int SUR_W2 = SUR_B1 + SUR_H;
constexpr int SUR_B2 = SUR_W2 + SUR_H * SUR_H;
constexpr int SUR_W3 = SUR_B2 + SUR_H;
constexpr int SUR_B3 = SUR_W3 + SUR_H * SUR_H;
constexpr int SUR_W4 = SUR_B3 + SUR_H;
constexpr int SUR_B4 = SUR_W4 + SUR_OUT * SUR_H;
constexpr int SUR_NPARAM = SUR_B4 + SUR_OUT;     // 10696
// B fragments: layer 1 (4 k-tiles x 8 n-tiles), 2 and 3 (4 x 8), 4 (4 x 1)
constexpr int SUR_F1 = 0, SUR_F2 = 32, SUR_F3 = 64, SUR_F4 = 96, SUR_NFRAG = 100;
constexpr int SUR_NBIAS = 3 * SUR_H + SUR_OUT;   // b1 b2 b3 b4

constexpr float GELU_K = 0.7978845608028654f;    // sqrt(2 / pi)
constexpr float GELU_A = 0.044715f;

// The network's inputs in canonical form.  The plate vote is even in the
// offset direction d and in the normal n (R = I - 2 d d^T, m m^T and
// (R p)(R p)^T with p = (I - n n^T) d are unchanged by either sign), and the
// ball vote is even in d and does not depend on n.  So n is taken with
// n_z >= 0 and d with d.n >= 0 (ball: d_z >= 0 and n = e_z): the network
// learns each function on a quarter (plate) or half (ball) of its domain.
// Training samples, the vote and the ball table all pass through here.
__host__ __device__ __forceinline__ void sur_canonical(float* d, float* n, bool plate) {
    if (plate) {
        if (n[2] < 0.0f) { n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2]; }
        if (d[0] * n[0] + d[1] * n[1] + d[2] * n[2] < 0.0f) { d[0] = -d[0]; d[1] = -d[1]; d[2] = -d[2]; }
    } else {
        n[0] = 0.0f; n[1] = 0.0f; n[2] = 1.0f;
        if (d[2] < 0.0f) { d[0] = -d[0]; d[1] = -d[1]; d[2] = -d[2]; }
    }
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);   // .x (low half) = lo
    return *reinterpret_cast<const uint32_t*>(&v);
}

// x - bf16(x): the part of an input that its BF16 rounding drops (exact in
// FP32).  The network's first layer takes each input twice, as bf16(x) and as
// bf16 of this residual, against the same weight, so the inputs reach the
// tensor cores with ~16 significant bits instead of 8.
__host__ __device__ __forceinline__ float bf16_residual(float x) {
    return x - __bfloat162float(__float2bfloat16_rn(x));
}

// The network's 28 features of a raw input x = (d0, d1, d2, n0, n1, n2,
// flag): x itself, then d_i d_j (i <= j), n_i n_j (i <= j), d_i n_j, each
// product rounded to FP32 once.
__host__ __device__ __forceinline__ void sur_features(const float* x, float* f) {
    const float* d = x;
    const float* nv = x + 3;
#pragma unroll
    for (int k = 0; k < SUR_X; ++k) f[k] = x[k];
    f[7] = d[0] * d[0]; f[8] = d[0] * d[1]; f[9] = d[0] * d[2];
    f[10] = d[1] * d[1]; f[11] = d[1] * d[2]; f[12] = d[2] * d[2];
    f[13] = nv[0] * nv[0]; f[14] = nv[0] * nv[1]; f[15] = nv[0] * nv[2];
    f[16] = nv[1] * nv[1]; f[17] = nv[1] * nv[2]; f[18] = nv[2] * nv[2];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) f[19 + 3 * i + j] = d[i] * nv[j];
}

// Layer 1's input row as 32 BF16 pairs (lower half = even K): the features,
// the bias pair (1, 1), two zeros, the features' residuals, four zeros.
// Each feature pair is packed once (cvt.rn.bf16x2), unpacked to FP32 by bit
// moves, and its residual pair formed by one packed subtraction.
__device__ __forceinline__ void sur_row64(const float* x, uint32_t (&row)[SUR_K1 / 2]) {
    float f[SUR_IN];
    sur_features(x, f);
#pragma unroll
    for (int i = 0; i < SUR_IN / 2; ++i) {
        const uint32_t hb = pack_bf16x2(f[2 * i], f[2 * i + 1]);
        row[i] = hb;
        const float2 hf = make_float2(__uint_as_float(hb << 16), __uint_as_float(hb & 0xffff0000u));
        const float2 r = __ffma2_rn(hf, make_float2(-1.0f, -1.0f), make_float2(f[2 * i], f[2 * i + 1]));   // exact
        row[16 + i] = pack_bf16x2(r.x, r.y);
    }
    row[14] = pack_bf16x2(1.0f, 1.0f);
    row[15] = 0u;
    row[30] = 0u;
    row[31] = 0u;
}

__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// GELU, tanh form, with the hardware tanh approximation (inference)
__device__ __forceinline__ float gelu_fast(float z) {
    const float u = GELU_K * fmaf(GELU_A * z, z * z, z);
    const float h = 0.5f * z;
    return fmaf(h, tanh_fast(u), h);
}

__device__ __forceinline__ void mma_bf16_16816(float (&c)[4], const uint32_t (&a)[4], uint2 b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// One 16-sample tile through the network.  a_in[kt]: this lane's A fragment
// of k-tile kt of the 16 x 64 layer-1 input (sur_row64's layout: rows g,
// g + 8; columns 16 kt + 2 t, + 1 in registers 0 / 1, 16 kt + 8 + 2 t, + 1
// in registers 2 / 3).  frag: the SUR_NFRAG x 32 B fragments (shared memory;
// layer 1's carry b1 in the rows that meet the bias pair), bias: b1 b2 b3 b4
// (b1 unused).  Returns the lane's output accumulator: rows g (out[0..1]) and
// g + 8 (out[2..3]), output columns 2 t, 2 t + 1, with g = lane / 4,
// t = lane % 4.
__device__ __forceinline__ void sur_mlp16(const uint2* __restrict__ frag, const float* __restrict__ bias,
                                          const uint32_t (&a_in)[4][4], float (&out)[4]) {
    const int lane = threadIdx.x & 31, t = lane & 3;
    float c[8][4];
    uint32_t a[4][4];
    // layer 1 (its bias rides in K)
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        c[nt][0] = 0.0f; c[nt][1] = 0.0f; c[nt][2] = 0.0f; c[nt][3] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) mma_bf16_16816(c[nt], a_in[kt], frag[(SUR_F1 + kt * 8 + nt) * 32 + lane]);
    }
#pragma unroll
    for (int layer = 0; layer < 2; ++layer) {
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            a[kt][0] = pack_bf16x2(gelu_fast(c[2 * kt][0]), gelu_fast(c[2 * kt][1]));
            a[kt][1] = pack_bf16x2(gelu_fast(c[2 * kt][2]), gelu_fast(c[2 * kt][3]));
            a[kt][2] = pack_bf16x2(gelu_fast(c[2 * kt + 1][0]), gelu_fast(c[2 * kt + 1][1]));
            a[kt][3] = pack_bf16x2(gelu_fast(c[2 * kt + 1][2]), gelu_fast(c[2 * kt + 1][3]));
        }
        const int fbase = layer == 0 ? SUR_F2 : SUR_F3;
        const float* bl = bias + SUR_H * (layer + 1);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float b0 = bl[nt * 8 + 2 * t], b1 = bl[nt * 8 + 2 * t + 1];
            c[nt][0] = b0; c[nt][1] = b1; c[nt][2] = b0; c[nt][3] = b1;
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) mma_bf16_16816(c[nt], a[kt], frag[(fbase + kt * 8 + nt) * 32 + lane]);
        }
    }
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        a[kt][0] = pack_bf16x2(gelu_fast(c[2 * kt][0]), gelu_fast(c[2 * kt][1]));
        a[kt][1] = pack_bf16x2(gelu_fast(c[2 * kt][2]), gelu_fast(c[2 * kt][3]));
        a[kt][2] = pack_bf16x2(gelu_fast(c[2 * kt + 1][0]), gelu_fast(c[2 * kt + 1][1]));
        a[kt][3] = pack_bf16x2(gelu_fast(c[2 * kt + 1][2]), gelu_fast(c[2 * kt + 1][3]));
    }
    const float* b4 = bias + 3 * SUR_H;
    out[0] = b4[2 * t]; out[1] = b4[2 * t + 1]; out[2] = out[0]; out[3] = out[1];
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) mma_bf16_16816(out, a[kt], frag[(SUR_F4 + kt) * 32 + lane]);
}

// Host-side: the B fragments and bias vector of a parameter vector (FP32
// master copy, layout above).  frag: SUR_NFRAG * 32 uint2, bias: SUR_NBIAS floats.
void sur_make_fragments(const float* params, uint2* frag, float* bias);

}  // namespace tvgb
