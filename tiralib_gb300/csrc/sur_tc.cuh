// The surrogate's MLP (surrogate_mlp.cuh: 28 features -> 64 -> 64 -> 64 -> 6,
// GELU, BF16 weights and activations, FP32 accumulation) on the
// fifth-generation tensor cores: tcgen05.mma with M = 128 rows (one
// (receiver, voter) pair or one sample per row, one row per thread of a
// 128-thread CTA), the activations in tensor memory (TMEM) as the A operand,
// the weights in shared memory as the B operand.
//
// TMEM columns of the CTA's allocation (128):
//   [0, 64)    D: the FP32 accumulator of the current layer (N = 64; the
//              output layer uses [0, 16))
//   [64, 96)   A: the current layer's input, BF16 pairs (64 values): layer
//              1's row of 64 (sur_row64: features, the bias pair, residuals),
//              then each hidden layer's activations
//   [96, 104)  a constant block: (1, 1, 0, ..., 0) in BF16.  The weight image
//              carries each hidden and output bias as bf16(b) and
//              bf16(b - bf16(b)) in the two K columns that meet it, so the
//              MMA adds the bias in FP32 to ~2^-16 relative and no epilogue
//              instruction is spent on it.  (Layer 1's bias pair is part of
//              its own row.)
//
// Weight image (shared memory, bytes), each matrix N x K, K-major, in 8 x 8
// core matrices without swizzle (LBO = 128 B along K, SBO = (K / 8) * 128 B
// along N):  B1 64 x 64 at 0, B2 64 x 80 at 8192, B3 64 x 80 at 18432,
// B4 16 x 80 at 28672; 31232 bytes in all.
//
// Where the time goes (GB300, measured): the three GELU epilogues per tile.
// With every unit on the tanh form the MUFU pipe was 71% busy; with one unit
// in four on the FMA-pipe polynomial form the kernel is held by the chain of
// four dependent MMA rounds per tile, with only 4 tiles in flight per SM
// (512 TMEM columns).
#pragma once
#include "surrogate_mlp.cuh"
#include "tc_sm100.cuh"

namespace tvgb {

constexpr int TC_COLS = 128;                    // TMEM columns per CTA
constexpr int TC_D = 0, TC_A = 64, TC_ONE = 96;
constexpr int TC_B1 = 0, TC_B2 = 8192, TC_B3 = 18432, TC_B4 = 28672, TC_IMG_BYTES = 31232;
constexpr int TC_K1 = SUR_K1, TC_KH = 80;       // K of layer 1 and of layers 2..4
constexpr uint32_t TC_WAIT_LIMIT = 1u << 24;    // mbarrier polls before a kernel gives up
// dynamic shared memory requested per CTA: at most 4 CTAs (4 x TC_COLS = all
// 512 TMEM columns) fit on an SM, so no CTA waits in tcgen05.alloc
constexpr int TC_SMEM_PER_CTA = 52 * 1024;

// GELU of a pair of FP32 pre-activations, returned as a BF16 pair (lower half
// = z0).  Mode 0: FP32 arithmetic with the hardware tanh, rounded once.
// Mode 1: packed BF16 arithmetic, one MUFU operation per pair:
//   zb = bf16(z); u = zb (K + K A zb^2); h = zb / 2; gelu = h + h tanh(u),
// every product and fused multiply-add rounded to BF16 once.  Mode 1, with
// the polynomial form below on one unit in four, is the activation of the
// training forward pass and of the surrogate vote.
template <int GM>
__device__ __forceinline__ uint32_t gelu_pair(float z0, float z1) {
    if (GM == 0) return pack_bf16x2(gelu_fast(z0), gelu_fast(z1));
    const __nv_bfloat162 zb = __floats2bfloat162_rn(z0, z1);
    const __nv_bfloat162 ka = __float2bfloat162_rn(GELU_K * GELU_A), k = __float2bfloat162_rn(GELU_K);
    const __nv_bfloat162 half = __float2bfloat162_rn(0.5f);
    const __nv_bfloat162 u = __hmul2(zb, __hfma2(__hmul2(zb, zb), ka, k));
    uint32_t ui = *reinterpret_cast<const uint32_t*>(&u), ti;
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(ti) : "r"(ui));
    const __nv_bfloat162 t = *reinterpret_cast<const __nv_bfloat162*>(&ti);
    const __nv_bfloat162 h = __hmul2(zb, half);
    const __nv_bfloat162 g = __hfma2(h, t, h);
    return *reinterpret_cast<const uint32_t*>(&g);
}

// The polynomial form of the GELU, for one unit in four (the units 8 u + 6 and
// 8 u + 7): z * phi(z), phi the normal CDF as a clamped odd polynomial
//   phi(z) = 1/2 + h (A1 + A3 s + A5 s^2 + A7 s^3),  h = clamp(z, -3, 3), s = h^2,
// a weighted least-squares fit on [-3, 3] (max deviation 1.5e-3 from the
// normal CDF), in FP32 arithmetic, rounded once to BF16.  It runs on the FMA
// pipe while the other units' tanh occupy the MUFU pipe: with three units in
// four on the MUFU the two pipes finish together.
constexpr float GELU_PC = 3.0f;
constexpr float GELU_P1 = 0.394045958f, GELU_P3 = -0.0578609677f, GELU_P5 = 0.00561482186f,
                GELU_P7 = -0.000222746943f;
__host__ __device__ constexpr bool gelu_is_poly(int col) { return (col & 7) >= 6; }

__device__ __forceinline__ uint32_t gelu_poly_pair(float z0, float z1) {
    const float2 z = make_float2(z0, z1);
    const float2 h = make_float2(fminf(fmaxf(z0, -GELU_PC), GELU_PC), fminf(fmaxf(z1, -GELU_PC), GELU_PC));
    const float2 s = __fmul2_rn(h, h);
    float2 p = __ffma2_rn(s, make_float2(GELU_P7, GELU_P7), make_float2(GELU_P5, GELU_P5));
    p = __ffma2_rn(p, s, make_float2(GELU_P3, GELU_P3));
    p = __ffma2_rn(p, s, make_float2(GELU_P1, GELU_P1));
    const float2 phi = __ffma2_rn(h, p, make_float2(0.5f, 0.5f));
    const float2 g = __fmul2_rn(z, phi);
    return pack_bf16x2(g.x, g.y);
}

// the activation of the unit pair (col, col + 1) or, in training, of two
// units of the same kind: the polynomial form for gelu_is_poly units, the
// packed-BF16 tanh form otherwise
__device__ __forceinline__ uint32_t gelu_unit_pair(float z0, float z1, bool poly) {
    return poly ? gelu_poly_pair(z0, z1) : gelu_pair<1>(z0, z1);
}

// this thread's TMEM lane quarter (warp w owns lanes 32 (w % 4) ..)
__device__ __forceinline__ uint32_t tc_lane_base() { return uint32_t(((threadIdx.x >> 5) & 3) * 32) << 16; }

// Per-CTA state of the tensor-core MLP (one copy per thread).
struct SurTc {
    uint32_t tmem;       // base address of the allocation
    uint32_t img;        // shared-memory address of the weight image
    uint64_t* bar;       // MMA completion barrier
    uint32_t phase;      // parity of the next completion
    uint32_t wait_limit; // polls of each layer's MMA barrier before the thread gives up
    int failed;          // this thread's wait gave up
};

// Setup by all 128 threads: weight image global -> shared memory, barrier,
// TMEM allocation (warp 0), the constant block.  tmem_slot and bar are
// __shared__ variables of the caller.  wait_limit bounds each layer's wait
// for its MMAs (polls; 0 gives up at once, which only tests the error path).
// Ends with a CTA barrier.
__device__ __forceinline__ void sur_tc_setup(SurTc& s, const uint4* __restrict__ img_g, uint4* img_s,
                                             uint32_t* tmem_slot, uint64_t* bar,
                                             uint32_t wait_limit = TC_WAIT_LIMIT) {
    const int tid = threadIdx.x;
    for (int i = tid; i < TC_IMG_BYTES / 16; i += blockDim.x) img_s[i] = img_g[i];
    if (tid == 0) tc::mbar_init(bar, 1);
    if (tid < 32) {
        tc::tmem_alloc(tmem_slot, TC_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    s.tmem = *tmem_slot;
    s.img = tc::smem_u32(img_s);
    s.bar = bar;
    s.phase = 0;
    s.wait_limit = wait_limit;
    s.failed = 0;
    const uint32_t one[8] = {0x3F803F80u, 0, 0, 0, 0, 0, 0, 0};   // bf16 (1, 1)
    tc::tmem_st8(s.tmem + tc_lane_base() + TC_ONE, one);
}

// Issue one layer's MMAs (thread 0) after every thread's TMEM writes, then
// wait for them.  The barrier that opens the call also tells every thread
// whether any thread's previous wait gave up; then all return false together
// (a thread whose wait gave up goes on to this barrier with stale data).
template <int LAYER>
__device__ __forceinline__ bool sur_tc_layer(SurTc& s) {
    tc::fence_before_sync();
    if (__syncthreads_or(s.failed)) return false;
    if (threadIdx.x == 0) {
        tc::fence_after_sync();
        if (LAYER == 1) {
            const uint32_t idesc = tc::idesc_bf16_f32(128, 64);
#pragma unroll
            for (int k = 0; k < TC_K1 / 16; ++k)
                tc::mma_ts(s.tmem + TC_D, s.tmem + TC_A + 8 * k, tc::smem_desc(s.img + TC_B1 + 256 * k, 128, 1024),
                           idesc, k > 0 ? 1u : 0u);
        } else {
            const uint32_t b = s.img + (LAYER == 2 ? TC_B2 : (LAYER == 3 ? TC_B3 : TC_B4));
            const uint32_t idesc = tc::idesc_bf16_f32(128, LAYER == 4 ? 16 : 64);
#pragma unroll
            for (int k = 0; k < TC_KH / 16; ++k)
                tc::mma_ts(s.tmem + TC_D, s.tmem + TC_A + 8 * k, tc::smem_desc(b + 256 * k, 128, 1280), idesc,
                           k > 0 ? 1u : 0u);
        }
        tc::mma_commit(s.bar);
    }
    if (tc::mbar_wait(s.bar, s.phase, s.wait_limit)) s.phase ^= 1u;
    else s.failed = 1;            // the phase stays: teardown waits for it
    tc::fence_after_sync();
    return true;
}

// GELU of this thread's row of D into its row of A.  A thread whose wait
// gave up leaves tensor memory alone: its MMAs may still be in flight.
template <int GM>
__device__ __forceinline__ void sur_tc_hidden(const SurTc& s) {
    if (s.failed) return;
    const uint32_t t = s.tmem + tc_lane_base();
    uint32_t act[32];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        uint32_t r[32];
        tc::tmem_ld32(t + TC_D + 32 * h, r);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float z0 = __uint_as_float(r[2 * i]), z1 = __uint_as_float(r[2 * i + 1]);
            act[16 * h + i] = GM == 1 ? gelu_unit_pair(z0, z1, gelu_is_poly(32 * h + 2 * i)) : gelu_pair<0>(z0, z1);
        }
    }
    tc::tmem_st32(t + TC_A, act);
}

// Layers 1..4 after the caller stored this thread's layer-1 input row
// (sur_row64: 32 BF16 pairs) into TMEM at TC_A; leaves the 16 output columns
// in D.  Returns false if a wait gave up.
template <int GM>
__device__ __forceinline__ bool sur_tc_layers(SurTc& s) {
    if (!sur_tc_layer<1>(s)) return false;
    sur_tc_hidden<GM>(s);
    if (!sur_tc_layer<2>(s)) return false;
    sur_tc_hidden<GM>(s);
    if (!sur_tc_layer<3>(s)) return false;
    sur_tc_hidden<GM>(s);
    return sur_tc_layer<4>(s);
}

// One 128-row tile through the network: in = this thread's layer-1 input
// row (sur_row64), out = its 8 output columns (6 used).  Returns false if a
// wait gave up.
template <int GM>
__device__ __forceinline__ bool sur_tc_forward(SurTc& s, const uint32_t (&in)[SUR_K1 / 2], float (&out)[8]) {
    const uint32_t t = s.tmem + tc_lane_base();
    if (!s.failed) tc::tmem_st32(t + TC_A, in);
    if (!sur_tc_layers<GM>(s) || s.failed) return false;
    uint32_t r[16];
    tc::tmem_ld16(t + TC_D, r);
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = __uint_as_float(r[i]);
    return true;
}

// Teardown by all threads: TMEM freed by warp 0.  Returns false if a wait
// gave up anywhere in the CTA; then the MMAs still in flight are waited for
// before the columns are released, always with the full TC_WAIT_LIMIT
// whatever the layers' limit was.  Only thread 0's own phase can still be
// pending: once any wait gives up no further MMA is issued, and if thread 0's
// last wait succeeded, the MMAs it issued have completed.
__device__ __forceinline__ bool sur_tc_teardown(SurTc& s) {
    tc::fence_before_sync();
    const int bad = __syncthreads_or(s.failed);
    if (bad && threadIdx.x == 0 && s.failed) tc::mbar_wait(s.bar, s.phase, TC_WAIT_LIMIT);
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x < 32) tc::tmem_dealloc(s.tmem, TC_COLS);
    return !bad;
}

// Host side: the weight image of a parameter vector (FP32 master copy, layout
// of surrogate_mlp.cuh) as TC_IMG_BYTES / 2 BF16 values.
void sur_make_tc_image(const float* params, uint16_t* img);

}  // namespace tvgb
