// Batched symmetric eigendecomposition kernels (3x3 and 2x2) and their C ABI.
//
// Replaces the reference launchers tira::cuda::evals3_symmetric /
// evecs3spherical_symmetric / evals2_symmetric / evecs2polar_symmetric
// (tira/functions/eigen.h:896,945,769,828) whose kernels read 36-byte AoS
// records with strided per-thread loads and run eigenvalues and
// eigenvectors as two passes over HBM.  Here one pass does both: a block
// stages its tile of AoS records into shared memory with 16-byte coalesced
// loads, each thread solves one tensor, and results leave through shared
// memory with 16-byte coalesced stores.  HBM traffic is the algorithmic
// minimum (read the tensor once, write each output once).  Each block keeps
// two input tiles in shared memory: the next tile's copy (cp.async) runs
// while the current one is solved.
//
// Precise mode (k_eig3w): a scale-invariant FP32 solve for every tensor;
// tensors whose remaining pair is closer than 1e-4 |lambda_max| go to a
// per-warp queue in shared memory, which the warp finishes in FP64, 32 at a
// time, while the other warps go on with their FP32 work (no block-wide
// barrier).  Each tensor is read from HBM once and each result written once
// (the FP64 results overwrite their FP32 placeholders a few tiles later,
// normally still in L2), and the FP64 pipe only sees flagged tensors (27% of
// the C3 recipe's), packed into whole warps.
#include "tvgb_common.cuh"
#include "eig_device.cuh"
#include <algorithm>
#include <mutex>

namespace tvgb {

constexpr int EIG_BLOCK = 256;
// resident blocks per SM the precise kernel is compiled for: 3 (80 registers,
// almost no spills) measured faster than 4 or 5 (64 / 48 registers, with the
// FP64 phase spilling): 4.24 ms against 4.67 / 4.81 ms for 2^27 tensors
#ifndef TVGB_EIG_MINB
#define TVGB_EIG_MINB 3
#endif

// in_layout: 9 (mat3 AoS), 6 (sym6 AoS), 60 (sym6 planes)
template <int IN_LAYOUT>
__device__ __forceinline__ void load_tile(const float* __restrict__ in, size_t n, size_t base, int cnt, float* s_in,
                                          bool aligned) {
    constexpr int NF = IN_LAYOUT == 9 ? 9 : 6;
    if (IN_LAYOUT == 60) {
        // planes: component c of tensor i at in[c * n + i]; store AoS into smem
        for (int c = 0; c < 6; ++c)
            for (int i = threadIdx.x; i < cnt; i += EIG_BLOCK) s_in[i * 6 + c] = __ldg(in + c * n + base + i);
        return;
    }
    const float* src = in + base * NF;
    const int nfl = cnt * NF;
    if (aligned && cnt == EIG_BLOCK) {
        const float4* s4 = reinterpret_cast<const float4*>(src);
        float4* d4 = reinterpret_cast<float4*>(s_in);
        for (int i = threadIdx.x; i < nfl / 4; i += EIG_BLOCK) d4[i] = __ldg(s4 + i);
    } else {
        for (int i = threadIdx.x; i < nfl; i += EIG_BLOCK) s_in[i] = __ldg(src + i);
    }
}

// The next tile's AoS records copied into shared memory asynchronously
// (16-byte cp.async per thread, no registers held), so the copy runs while
// the block solves the current tile.  Full, 16-byte aligned AoS tiles only.
__device__ __forceinline__ void load_tile_async(const float* __restrict__ src, int nfl, float* s_in) {
    const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(s_in));
    for (int i = threadIdx.x; i < nfl / 4; i += EIG_BLOCK)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 16u * i), "l"(src + 4 * i) : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void wait_tile_async() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void store_tile(float* __restrict__ dst, const float* s, int nfl, bool aligned, bool full) {
    if (aligned && full && (nfl % 4) == 0) {
        float4* d4 = reinterpret_cast<float4*>(dst);
        const float4* s4 = reinterpret_cast<const float4*>(s);
        for (int i = threadIdx.x; i < nfl / 4; i += EIG_BLOCK) d4[i] = s4[i];
    } else {
        for (int i = threadIdx.x; i < nfl; i += EIG_BLOCK) dst[i] = s[i];
    }
}

// Parity mode (eigen.h's closed forms).  EVEC_FMT: 0 none, 1 cartesian (9),
// 2 spherical (6).  EVALS_IN: take the eigenvalues from `evals_in` (the
// reference's evecs3spherical contract).
template <int IN_LAYOUT, int EVEC_FMT, bool EVALS_IN>
__global__ void __launch_bounds__(EIG_BLOCK) k_eig3(const float* __restrict__ in, size_t n,
                                                    const float* __restrict__ evals_in, float* __restrict__ evals,
                                                    float* __restrict__ evecs, int aligned_in, int aligned_out) {
    constexpr int NF = IN_LAYOUT == 9 ? 9 : 6;
    constexpr int NV = EVEC_FMT == 1 ? 9 : (EVEC_FMT == 2 ? 6 : 0);
    __shared__ __align__(16) float s_in2[2][EIG_BLOCK * NF];   // the current tile and the next one
    __shared__ __align__(16) float s_ev[EIG_BLOCK * 3];
    __shared__ __align__(16) float s_vec[EIG_BLOCK * 9];

    const size_t stride = size_t(gridDim.x) * EIG_BLOCK;
    // tile at `base` into buffer `buf`: asynchronous when full, aligned and AoS
    auto fetch = [&](size_t base, int buf) {
        const int cnt = int(min(size_t(EIG_BLOCK), n - base));
        if (IN_LAYOUT != 60 && aligned_in && cnt == EIG_BLOCK)
            load_tile_async(in + base * NF, EIG_BLOCK * NF, s_in2[buf]);
        else
            load_tile<IN_LAYOUT>(in, n, base, cnt, s_in2[buf], aligned_in);
    };
    int it = 0;   // tiles done by this block: tile it sits in buffer it & 1
    if (size_t(blockIdx.x) * EIG_BLOCK < n) fetch(size_t(blockIdx.x) * EIG_BLOCK, 0);
    for (size_t base = size_t(blockIdx.x) * EIG_BLOCK; base < n; base += stride, ++it) {
        const int cnt = int(min(size_t(EIG_BLOCK), n - base));
        const float* s_in = s_in2[it & 1];
        if (EVALS_IN)
            for (int i = threadIdx.x; i < cnt * 3; i += EIG_BLOCK) s_ev[i] = __ldg(evals_in + base * 3 + i);
        wait_tile_async();
        __syncthreads();
        // the other buffer was last read before the barrier that ended the previous tile
        if (base + stride < n) fetch(base + stride, (it + 1) & 1);
        const int t = threadIdx.x;
        if (t < cnt) {
            const float* m = s_in + t * NF;
            float a, b, c, d, e, f;
            if (NF == 9) { a = m[0]; b = m[1]; d = m[2]; c = m[4]; e = m[5]; f = m[8]; }
            else { a = m[0]; b = m[1]; d = m[2]; c = m[3]; e = m[4]; f = m[5]; }
            float ev[3], v[9];
            if (EVALS_IN) { ev[0] = s_ev[t * 3]; ev[1] = s_ev[t * 3 + 1]; ev[2] = s_ev[t * 3 + 2]; }
            else eval3_d(a, b, c, d, e, f, ev[0], ev[1], ev[2]);
            if (EVEC_FMT != 0) evec3_d(a, b, c, d, e, f, ev, v, v + 3, v + 6);
            if (!EVALS_IN) { s_ev[t * 3] = ev[0]; s_ev[t * 3 + 1] = ev[1]; s_ev[t * 3 + 2] = ev[2]; }
            if (EVEC_FMT != 0)
                for (int k = 0; k < 9; ++k) s_vec[t * 9 + k] = v[k];
        }
        __syncthreads();
        if (EVEC_FMT == 2) {
            // spherical output, packed 6 per tensor into the front of s_vec
            float sph[6];
            if (t < cnt) {
                float w[9];
                for (int k = 0; k < 9; ++k) w[k] = s_vec[t * 9 + k];
                to_spherical_d(w, sph[0], sph[1]);
                to_spherical_d(w + 3, sph[2], sph[3]);
                to_spherical_d(w + 6, sph[4], sph[5]);
            }
            __syncthreads();
            if (t < cnt)
                for (int k = 0; k < 6; ++k) s_vec[t * 6 + k] = sph[k];
            __syncthreads();
        }
        const bool full = cnt == EIG_BLOCK;
        if (evals && !EVALS_IN) store_tile(evals + base * 3, s_ev, cnt * 3, aligned_out, full);
        if (NV && evecs) store_tile(evecs + base * NV, s_vec, cnt * NV, aligned_out, full);
        __syncthreads();
    }
}

// Precise mode, warp-tiled.  Each warp owns tiles of 32 consecutive tensors
// (tile t of the batch goes to warp t mod (warps in the grid)) and works on
// them without any block-wide barrier:
//   * the next tile's records are copied into the warp's shared buffer with
//     cp.async while the current one is solved;
//   * every lane solves its tensor in FP32 (eig3_precise_fp32); a tensor
//     whose remaining pair is closer than 1e-4 |lambda_max| is appended to
//     the warp's queue in shared memory (its six entries, w and its place);
//   * the tile's results leave through the warp's staging buffer with
//     16-byte coalesced stores;
//   * once the queue holds 32 tensors, the warp finishes them in FP64, one
//     per lane, and writes their results over the FP32 ones (the tiles they
//     came from were stored a few tiles earlier and are normally still in
//     L2).  The rest of the queue is finished at the end.
// A warp busy in FP64 holds up no other warp, so the FP64 pipe works while
// the other warps issue the FP32 phase.
constexpr int EIGW_QCAP = 64;          // queue entries per warp (at most 31 + 32 between drains)
constexpr int EIGW_QF = 11;            // floats per entry: 6 entries, w0..w2, tile, key

template <int IN_LAYOUT, int EVEC_FMT>
__global__ void __launch_bounds__(EIG_BLOCK, TVGB_EIG_MINB) k_eig3w(const float* __restrict__ in, size_t n,
                                                                      float* __restrict__ evals,
                                                                      float* __restrict__ evecs,
                                                                      unsigned long long* __restrict__ n_refined,
                                                                      int aligned_in, int aligned_out) {
    constexpr int NF = IN_LAYOUT == 9 ? 9 : 6;
    constexpr int NV = EVEC_FMT == 1 ? 9 : (EVEC_FMT == 2 ? 6 : 0);
    constexpr int NW = EIG_BLOCK / 32;
    __shared__ __align__(16) float s_in[NW][32 * NF];
    __shared__ __align__(16) float s_ev[NW][32 * 3];
    __shared__ __align__(16) float s_vec[NW][32 * (NV ? NV : 1)];
    __shared__ float s_q[NW][EIGW_QCAP * EIGW_QF];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t nwarps = size_t(gridDim.x) * NW;
    const size_t ntiles = (n + 31) / 32;
    float* sin = s_in[warp];
    float* sq = s_q[warp];
    int qn = 0;                         // warp-uniform queue length
    unsigned long long refined = 0;

    // the tile's AoS records into the warp buffer: asynchronous when whole and aligned
    auto fetch = [&](size_t t) {
        if (IN_LAYOUT == 60) return;
        const size_t base = t * 32;
        const int cnt = int(min(size_t(32), n - base));
        const float* src = in + base * NF;
        if (aligned_in && cnt == 32) {
            const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(sin));
            for (int i = lane; i < 32 * NF / 4; i += 32)
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 16u * i), "l"(src + 4 * i)
                             : "memory");
            asm volatile("cp.async.commit_group;" ::: "memory");
        } else {
            for (int i = lane; i < cnt * NF; i += 32) sin[i] = __ldg(src + i);
        }
    };
    // FP64 phase of queue entries [q0, q0 + cnt) (one per lane), results written to global memory
    auto drain = [&](int q0, int cnt) {
        if (lane < cnt) {
            const float* e = sq + (q0 + lane) * EIGW_QF;
            const unsigned key = __float_as_uint(e[10]);
            const size_t i = size_t(__float_as_uint(e[9])) * 32 + (key & 31u);
            const int code = int((key >> 5) & 3u);
            const bool hi = (key >> 7) & 1u;
            const float w[3] = {e[6], e[7], e[8]};
            float ev[3], v[9];
            eig3_precise_fp64(e[0], e[1], e[2], e[3], e[4], e[5], w, hi, code, ev, v, v + 3, v + 6);
            if (evals) { evals[i * 3] = ev[0]; evals[i * 3 + 1] = ev[1]; evals[i * 3 + 2] = ev[2]; }
            if (EVEC_FMT == 1 && evecs)
                for (int k = 0; k < 9; ++k) evecs[i * 9 + k] = v[k];
            if (EVEC_FMT == 2 && evecs) {
                float th, ph;
                to_spherical_d(v, th, ph); evecs[i * 6] = th; evecs[i * 6 + 1] = ph;
                to_spherical_d(v + 3, th, ph); evecs[i * 6 + 2] = th; evecs[i * 6 + 3] = ph;
                to_spherical_d(v + 6, th, ph); evecs[i * 6 + 4] = th; evecs[i * 6 + 5] = ph;
            }
        }
        refined += unsigned(cnt);
    };

    size_t t = blockIdx.x * size_t(NW) + warp;
    if (t < ntiles) fetch(t);
    for (; t < ntiles; t += nwarps) {
        const size_t base = t * 32;
        const int cnt = int(min(size_t(32), n - base));
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncwarp();
        float a = 0, b = 0, c = 0, d = 0, e = 0, f = 0;
        if (lane < cnt) {
            if (IN_LAYOUT == 60) {
                const size_t i = base + lane;
                a = __ldg(in + i); b = __ldg(in + n + i); d = __ldg(in + 2 * n + i);
                c = __ldg(in + 3 * n + i); e = __ldg(in + 4 * n + i); f = __ldg(in + 5 * n + i);
            } else if (NF == 9) {
                const float* m = sin + lane * 9;
                a = m[0]; b = m[1]; d = m[2]; c = m[4]; e = m[5]; f = m[8];
            } else {
                const float* m = sin + lane * 6;
                a = m[0]; b = m[1]; d = m[2]; c = m[3]; e = m[4]; f = m[5];
            }
        }
        __syncwarp();                                       // the buffer is read: the next copy may land
        if (t + nwarps < ntiles) fetch(t + nwarps);
        float ev[3] = {0, 0, 0}, v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, w[3];
        bool hi = true;
        int code = 0;
        if (lane < cnt) code = eig3_precise_fp32(a, b, c, d, e, f, ev, v, v + 3, v + 6, w, hi);
        const unsigned flag = __ballot_sync(0xffffffffu, code != 0);
        if (code) {   // queue slot: after the lanes below with a flagged tensor
            float* q = sq + (qn + __popc(flag & ((1u << lane) - 1u))) * EIGW_QF;
            q[0] = a; q[1] = b; q[2] = c; q[3] = d; q[4] = e; q[5] = f;
            q[6] = w[0]; q[7] = w[1]; q[8] = w[2];
            q[9] = __uint_as_float(unsigned(t));
            q[10] = __uint_as_float(unsigned(lane) | (unsigned(code) << 5) | ((hi ? 1u : 0u) << 7));
        }
        qn += __popc(flag);
        // the tile's FP32 results (flagged tensors: overwritten by their FP64 phase later)
        float* se = s_ev[warp];
        se[lane * 3] = ev[0]; se[lane * 3 + 1] = ev[1]; se[lane * 3 + 2] = ev[2];
        if (NV) {
            float* sv = s_vec[warp];
            if (EVEC_FMT == 1) {
                for (int k = 0; k < 9; ++k) sv[lane * 9 + k] = v[k];
            } else {
                float sph[6];
                to_spherical_d(v, sph[0], sph[1]);
                to_spherical_d(v + 3, sph[2], sph[3]);
                to_spherical_d(v + 6, sph[4], sph[5]);
                for (int k = 0; k < 6; ++k) sv[lane * 6 + k] = sph[k];
            }
        }
        __syncwarp();
        const bool full = cnt == 32 && aligned_out;
        if (evals) {
            if (full) {
                const float4* s4 = reinterpret_cast<const float4*>(se);
                float4* d4 = reinterpret_cast<float4*>(evals + base * 3);
                for (int i = lane; i < 24; i += 32) d4[i] = s4[i];
            } else {
                for (int i = lane; i < cnt * 3; i += 32) evals[base * 3 + i] = se[i];
            }
        }
        if (NV && evecs) {
            const float* sv = s_vec[warp];
            if (full) {
                const float4* s4 = reinterpret_cast<const float4*>(sv);
                float4* d4 = reinterpret_cast<float4*>(evecs + base * NV);
                for (int i = lane; i < 8 * NV; i += 32) d4[i] = s4[i];
            } else {
                for (int i = lane; i < cnt * NV; i += 32) evecs[base * NV + i] = sv[i];
            }
        }
        __syncwarp();                                       // tile stores ordered before the FP64 results
        if (qn >= 32) {
            drain(qn - 32, 32);
            qn -= 32;
            __syncwarp();
        }
    }
    if (qn > 0) drain(0, qn);
    if (n_refined && lane == 0 && refined) atomicAdd(n_refined, refined);
}

__global__ void k_eval2(const float4* __restrict__ m4, size_t n, float2* __restrict__ ev2) {
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const float4 m = __ldg(m4 + i);
        float e0, e1;
        eval2_d(m.x, m.y, m.w, e0, e1);
        ev2[i] = make_float2(e0, e1);
    }
}

__global__ void k_evec2(const float4* __restrict__ m4, const float2* __restrict__ ev2, size_t n, float2* __restrict__ th2) {
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const float4 m = __ldg(m4 + i);
        float t0, t1;
        evec2polar_d(m.x, m.y, m.w, __ldg(ev2 + i).x, t0, t1);
        th2[i] = make_float2(t0, t1);
    }
}

static int grid_for(size_t items, int per_block) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    size_t blocks = (items + per_block - 1) / per_block;
    size_t cap = size_t(sms) * 8;   // persistent-style grid: a multiple of the SM count
    if (blocks > cap) blocks = cap;
    return int(blocks ? blocks : 1);
}

// Grid of a grid-stride kernel: as many blocks as fit on the GPU at once, so
// every block is resident from the start and all finish together.  (A grid of
// a fixed 8 blocks per SM ran k_eig3, 6 resident per SM, in a full wave and a
// third of a wave.)
template <class Kernel>
static int resident_grid(Kernel kern, int block, size_t items) {
    struct Entry { const void* k; int dev, block, resident; };
    static std::mutex mu;
    static Entry cache[32];
    static int used = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    int resident = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        for (int i = 0; i < used; ++i)
            if (cache[i].k == reinterpret_cast<const void*>(kern) && cache[i].dev == dev && cache[i].block == block)
                resident = cache[i].resident;
    }
    if (resident == 0) {
        int sms = 152, p = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, kern, block, 0) != cudaSuccess || p < 1) {
            cudaGetLastError();
            p = 1;
        }
        resident = sms * p;
        std::lock_guard<std::mutex> lk(mu);
        if (used < 32) cache[used++] = Entry{reinterpret_cast<const void*>(kern), dev, block, resident};
    }
    size_t blocks = (items + block - 1) / block;
    const size_t cap = size_t(resident);
    if (blocks > cap) blocks = cap;
    return int(blocks ? blocks : 1);
}

template <int IL, int EF, bool PR, bool EI>
static int launch_eig3_t(const float* in, size_t n, const float* ev_in, float* ev, float* vec, unsigned long long* nref,
                         cudaStream_t s) {
    const int ai = (reinterpret_cast<uintptr_t>(in) % 16) == 0;
    const int ao = (!ev || reinterpret_cast<uintptr_t>(ev) % 16 == 0) && (!vec || reinterpret_cast<uintptr_t>(vec) % 16 == 0);
    KernelTimer kt_("k_eig3", s);
    if constexpr (PR) {   // precise: the warp-tiled kernel
        k_eig3w<IL, EF><<<resident_grid(k_eig3w<IL, EF>, EIG_BLOCK, n), EIG_BLOCK, 0, s>>>(in, n, ev, vec, nref, ai,
                                                                                            ao);
    } else {
        k_eig3<IL, EF, EI><<<resident_grid(k_eig3<IL, EF, EI>, EIG_BLOCK, n), EIG_BLOCK, 0, s>>>(in, n, ev_in, ev, vec,
                                                                                                ai, ao);
    }
    kt_.stop();
    TVGB_LAUNCHED();
    return TVGB_OK;
}

template <int IL>
static int launch_eig3_l(const float* in, size_t n, float* ev, float* vec, int fmt, bool precise,
                         unsigned long long* nref, cudaStream_t s) {
    if (precise) {
        if (fmt == 1) return launch_eig3_t<IL, 1, true, false>(in, n, nullptr, ev, vec, nref, s);
        if (fmt == 2) return launch_eig3_t<IL, 2, true, false>(in, n, nullptr, ev, vec, nref, s);
        return launch_eig3_t<IL, 0, true, false>(in, n, nullptr, ev, vec, nref, s);
    }
    if (fmt == 1) return launch_eig3_t<IL, 1, false, false>(in, n, nullptr, ev, vec, nref, s);
    if (fmt == 2) return launch_eig3_t<IL, 2, false, false>(in, n, nullptr, ev, vec, nref, s);
    return launch_eig3_t<IL, 0, false, false>(in, n, nullptr, ev, vec, nref, s);
}

// device-pointer entry used by the other translation units too
int eig3_device(const float* in, int layout, size_t n, float* ev, float* vec, int fmt, bool precise,
                unsigned long long* nref, cudaStream_t s) {
    if (n == 0) return TVGB_OK;
    if (layout == TVGB_LAYOUT_MAT3) return launch_eig3_l<9>(in, n, ev, vec, fmt, precise, nref, s);
    if (layout == TVGB_LAYOUT_SYM6) return launch_eig3_l<6>(in, n, ev, vec, fmt, precise, nref, s);
    return launch_eig3_l<60>(in, n, ev, vec, fmt, precise, nref, s);
}

}  // namespace tvgb

using namespace tvgb;

extern "C" {

// Host arrays in, host arrays out: the batch is cut into chunks that flow
// through a ring of device buffers on their own streams, so the host->device
// copy of one chunk, the solve of another and the device->host copy of a
// third run at the same time (separate copy engines each way).  Ordered after
// the caller's stream's earlier work, and the caller's stream after the last
// chunk.
static int eig3_streamed(const float* mats, int in_layout, size_t n, float* evals3, float* evecs, int fmt,
                         bool precise, unsigned long long* nref, cudaStream_t s) {
    constexpr size_t CH = size_t(1) << 22;
    constexpr int NB = 3;
    const size_t nf = in_layout == TVGB_LAYOUT_MAT3 ? 9 : 6;
    const size_t nv = fmt == 1 ? 9 : (fmt == 2 ? 6 : 0);
    const size_t per = CH * (nf + 3 + nv);
    Scratch buf;
    TVGB_TRY(buf.alloc(NB * per * sizeof(float), s));
    cudaStream_t ss[NB] = {};
    cudaEvent_t fork = nullptr, join[NB] = {};
    int rc = TVGB_OK;
    auto cuda = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess && rc == TVGB_OK) {
            set_error("tvgb_eig3 (streamed): %s failed: %s", what, cudaGetErrorString(e));
            rc = TVGB_ERR_CUDA;
        }
        return e == cudaSuccess;
    };
    bool ok = cuda(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "cudaEventCreate");
    for (int b = 0; ok && b < NB; ++b)
        ok = cuda(cudaStreamCreateWithFlags(&ss[b], cudaStreamNonBlocking), "cudaStreamCreate") &&
             cuda(cudaEventCreateWithFlags(&join[b], cudaEventDisableTiming), "cudaEventCreate");
    ok = ok && cuda(cudaEventRecord(fork, s), "cudaEventRecord");
    for (int b = 0; ok && b < NB; ++b) ok = cuda(cudaStreamWaitEvent(ss[b], fork, 0), "cudaStreamWaitEvent");
    size_t i = 0;
    for (size_t c = 0; ok && c < n; c += CH, ++i) {
        const int b = int(i % NB);
        const size_t m = n - c < CH ? n - c : CH;
        float* din = buf.get<float>() + b * per;
        float* dev = din + CH * nf;
        float* dvec = dev + CH * 3;
        ok = cuda(cudaMemcpyAsync(din, mats + c * nf, m * nf * sizeof(float), cudaMemcpyHostToDevice, ss[b]),
                  "cudaMemcpyAsync");
        if (ok) {
            const int r = eig3_device(din, in_layout, m, dev, nv ? dvec : nullptr, fmt, precise, nref, ss[b]);
            if (r != TVGB_OK) {
                rc = r;
                ok = false;
            }
        }
        ok = ok && cuda(cudaMemcpyAsync(evals3 + c * 3, dev, m * 3 * sizeof(float), cudaMemcpyDeviceToHost, ss[b]),
                        "cudaMemcpyAsync");
        if (ok && nv)
            ok = cuda(cudaMemcpyAsync(evecs + c * nv, dvec, m * nv * sizeof(float), cudaMemcpyDeviceToHost, ss[b]),
                      "cudaMemcpyAsync");
    }
    // join every stream that was created, also after a failure, before the buffers are released on s
    for (int b = 0; b < NB; ++b) {
        if (ss[b] && join[b] && cudaEventRecord(join[b], ss[b]) == cudaSuccess) cudaStreamWaitEvent(s, join[b], 0);
        else if (ss[b]) cudaStreamSynchronize(ss[b]);
    }
    for (int b = 0; b < NB; ++b) {
        if (join[b]) cudaEventDestroy(join[b]);
        if (ss[b]) cudaStreamDestroy(ss[b]);
    }
    if (fork) cudaEventDestroy(fork);
    return rc;
}

int tvgb_eig3(const float* mats, int in_layout, size_t n, float* evals3, float* evecs, int evec_format, int mode,
              size_t* n_refined, void* stream) {
    TVGB_CHECK_ARG(mats || n == 0, "tvgb_eig3: mats is NULL");
    TVGB_CHECK_ARG(in_layout == TVGB_LAYOUT_MAT3 || in_layout == TVGB_LAYOUT_SYM6 || in_layout == TVGB_LAYOUT_SYM6_PLANES,
                   "tvgb_eig3: in_layout must be 9, 6 or 60 (got %d)", in_layout);
    TVGB_CHECK_ARG(evec_format >= 0 && evec_format <= 2, "tvgb_eig3: evec_format must be 0, 1 or 2");
    TVGB_CHECK_ARG(mode == TVGB_EIG_PARITY || mode == TVGB_EIG_PRECISE, "tvgb_eig3: mode must be 0 or 1");
    if (n_refined) *n_refined = 0;
    if (n == 0) return TVGB_OK;
    cudaStream_t s = as_stream(stream);
    const size_t nf = in_layout == TVGB_LAYOUT_MAT3 ? 9 : 6;
    const size_t nv = evec_format == 1 ? 9 : (evec_format == 2 ? 6 : 0);
    Scratch cnt;
    if (n_refined && mode == TVGB_EIG_PRECISE) {
        TVGB_TRY(cnt.alloc(sizeof(unsigned long long), s));
        TVGB_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), s));
    }
    // large batches wholly in host memory (interleaved layouts): copies overlapped with the solve
    if (n >= (size_t(1) << 23) && in_layout != TVGB_LAYOUT_SYM6_PLANES && evals3 && !is_device_ptr(mats) &&
        !is_device_ptr(evals3) && (!nv || (evecs && !is_device_ptr(evecs)))) {
        TVGB_TRY(eig3_streamed(mats, in_layout, n, evals3, evecs, evec_format, mode == TVGB_EIG_PRECISE,
                               cnt.get<unsigned long long>(), s));
        if (cnt.p) {
            unsigned long long h = 0;
            TVGB_CUDA(cudaMemcpyAsync(&h, cnt.p, sizeof(h), cudaMemcpyDeviceToHost, s));
            *n_refined = size_t(h);
        }
        TVGB_CUDA(cudaStreamSynchronize(s));
        return TVGB_OK;
    }
    DevArray din, dev_, dvec;
    TVGB_TRY(din.in(mats, n * nf * sizeof(float), s));
    TVGB_TRY(dev_.out(evals3, n * 3 * sizeof(float), s));
    TVGB_TRY(dvec.out(nv ? evecs : nullptr, n * nv * sizeof(float), s));
    TVGB_TRY(eig3_device(din.get<float>(), in_layout, n, dev_.get<float>(), dvec.get<float>(), evec_format,
                         mode == TVGB_EIG_PRECISE, cnt.get<unsigned long long>(), s));
    TVGB_TRY(dev_.finish());
    TVGB_TRY(dvec.finish());
    bool need_sync = din.owned || dev_.owned || dvec.owned;
    if (cnt.p) {
        unsigned long long h = 0;
        TVGB_CUDA(cudaMemcpyAsync(&h, cnt.p, sizeof(h), cudaMemcpyDeviceToHost, s));
        TVGB_CUDA(cudaStreamSynchronize(s));
        *n_refined = size_t(h);
        need_sync = false;
    }
    return sync_if(need_sync, s);
}

int tvgb_evals3_symmetric(const float* mats9, size_t n, float* evals3, void* stream) {
    TVGB_CHECK_ARG(evals3 || n == 0, "tvgb_evals3_symmetric: evals3 is NULL");
    return tvgb_eig3(mats9, TVGB_LAYOUT_MAT3, n, evals3, nullptr, TVGB_EVEC_NONE, TVGB_EIG_PARITY, nullptr, stream);
}

int tvgb_evecs3spherical_symmetric(const float* mats9, const float* evals3, size_t n, float* evecs6, void* stream) {
    TVGB_CHECK_ARG((mats9 && evals3 && evecs6) || n == 0, "tvgb_evecs3spherical_symmetric: NULL argument");
    if (n == 0) return TVGB_OK;
    cudaStream_t s = as_stream(stream);
    DevArray din, dev_, dvec;
    TVGB_TRY(din.in(mats9, n * 9 * sizeof(float), s));
    TVGB_TRY(dev_.in(evals3, n * 3 * sizeof(float), s));
    TVGB_TRY(dvec.out(evecs6, n * 6 * sizeof(float), s));
    TVGB_TRY((launch_eig3_t<9, 2, false, true>(din.get<float>(), n, dev_.get<float>(), nullptr, dvec.get<float>(),
                                                nullptr, s)));
    TVGB_TRY(dvec.finish());
    return sync_if(din.owned || dev_.owned || dvec.owned, s);
}

int tvgb_evals2_symmetric(const float* mats4, size_t n, float* evals2, void* stream) {
    TVGB_CHECK_ARG((mats4 && evals2) || n == 0, "tvgb_evals2_symmetric: NULL argument");
    if (n == 0) return TVGB_OK;
    cudaStream_t s = as_stream(stream);
    DevArray din, dout;
    TVGB_TRY(din.in(mats4, n * 16, s));
    TVGB_TRY(dout.out(evals2, n * 8, s));
    TVGB_CHECK_ARG(reinterpret_cast<uintptr_t>(din.dev) % 16 == 0 && reinterpret_cast<uintptr_t>(dout.dev) % 8 == 0,
                   "tvgb_evals2_symmetric: device arrays must be 16/8-byte aligned");
    {
        KernelTimer kt_("k_eval2", s);
        k_eval2<<<grid_for(n, 256), 256, 0, s>>>(din.get<float4>(), n, dout.get<float2>());
        kt_.stop();
    }
    TVGB_LAUNCHED();
    TVGB_TRY(dout.finish());
    return sync_if(din.owned || dout.owned, s);
}

int tvgb_evecs2polar_symmetric(const float* mats4, const float* evals2, size_t n, float* thetas2, void* stream) {
    TVGB_CHECK_ARG((mats4 && evals2 && thetas2) || n == 0, "tvgb_evecs2polar_symmetric: NULL argument");
    if (n == 0) return TVGB_OK;
    cudaStream_t s = as_stream(stream);
    DevArray din, dev_, dout;
    TVGB_TRY(din.in(mats4, n * 16, s));
    TVGB_TRY(dev_.in(evals2, n * 8, s));
    TVGB_TRY(dout.out(thetas2, n * 8, s));
    TVGB_CHECK_ARG(reinterpret_cast<uintptr_t>(din.dev) % 16 == 0 && reinterpret_cast<uintptr_t>(dev_.dev) % 8 == 0 &&
                       reinterpret_cast<uintptr_t>(dout.dev) % 8 == 0,
                   "tvgb_evecs2polar_symmetric: device arrays must be 16/8-byte aligned");
    {
        KernelTimer kt_("k_evec2", s);
        k_evec2<<<grid_for(n, 256), 256, 0, s>>>(din.get<float4>(), dev_.get<float2>(), n, dout.get<float2>());
        kt_.stop();
    }
    TVGB_LAUNCHED();
    TVGB_TRY(dout.finish());
    return sync_if(din.owned || dev_.owned || dout.owned, s);
}

}  // extern "C"
