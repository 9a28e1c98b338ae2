// Structure tensor and separable Gaussian filters.
//
// Reference path replaced: the caller computes volume<T>::gradient per axis
// (tira/volume.h:974, a host triple loop), forms the outer product itself,
// and blurs each of the six components with tira::cuda::gaussian_filter3d
// (tira/functions/filter.h:401): three launches per component (z, y, x
// passes, cuda_convolve3z/3y/3x :275,259,243) with the kernel in global
// memory, intermediates in HBM and a device synchronise after each pass.
//
// Here one kernel does it all (k_st3<K> for K = 3..13 taps, k_st3_any
// above): a CTA owns a 32 x 8 output column and marches through the input
// z-planes.  Per plane it forms the gradients (central inside, one-sided at
// the faces) and their six products on the haloed xy tile from the last three
// raw planes in shared memory, blurs them along y (one thread per channel and
// column, the column held in registers) and along x (64-bit row loads), and
// feeds each thread's two x outputs of three channels into a register window
// of K partial sums per output, which completes the z blur: each finished
// output plane is written once.  The raw planes are staged either by each
// thread's own loads one plane ahead (k_st3) or, for volumes whose rows meet
// the TMA rules, by cp.async.bulk.tensor boxes issued six planes ahead
// (k_st3_tma).  HBM traffic ~ one read of the volume plus one write of the six
// components (28 B per voxel).
//
// tvgb_gaussian_filter3d / tvgb_gaussian_convolve2 keep the reference's
// scalar, valid-convolution contract (filter.h:401, :305) with a coalesced
// per-axis pass kernel.
#include "tvgb_internal.cuh"
#include "tma_sm100.cuh"
#include <vector>
#include <cmath>

namespace tvgb {

// filter.h:405-410 (3D) / :308 (2D) window rules
static unsigned ksize3(float sigma) {
    unsigned k = unsigned(std::ceil(6.0f * sigma));
    if (k % 2 == 0) k++;
    return k;
}
static unsigned ksize2(float sigma) { return unsigned(6.0f * sigma); }

// cpu::gaussian1d (filter.h:38) with mu = 0, dx = 1: taps at cell centres,
// normalised to sum 1 (float steps as the reference)
static void gaussian1d(unsigned K, float sigma, float* k) {
    const float half = float(K) / 2.0f;
    const float start = -half + 0.5f;
    const float s2 = sigma * sigma;
    const float pi = 3.14159265358979323846f;
    const float nrm = 1.0f / std::sqrt(2.0f * pi * s2);
    float sum = 0.0f;
    for (unsigned i = 0; i < K; ++i) {
        const float x = start + float(i);
        k[i] = nrm * std::exp(-(x * x) / (2.0f * s2));
        sum += k[i];
    }
    if (sum > 0.0f) {
        const float inv = 1.0f / sum;
        for (unsigned i = 0; i < K; ++i) k[i] *= inv;
    }
}

constexpr int STX = 32, STY = 8, MAXK = 41;

struct StArgs {
    const float* vol;
    int s0, s1, s2;       // input
    int o0, o1, o2;       // output dims
    int K, off;           // taps, input offset of output index 0 (0 valid, K/2 same)
    int zchunk;           // output planes per CTA
    float g[MAXK];
    float* out;
    int layout;
    int pair_store;       // planes layout, even o2, 8-byte aligned out: 64-bit stores of x pairs
};

// d/d(axis) at an in-volume voxel: volume<T>::gradient's rule
__device__ __forceinline__ float grad1(float lo, float c, float hi, int p, int S) {
    if (S < 2) return 0.0f;
    if (p == 0) return hi - c;
    if (p == S - 1) return c - lo;
    return (hi - lo) * 0.5f;
}

// Shared memory (floats), with EX = 32 + K - 1, EY = 8 + K - 1:
//   raw   3 x (EY + 2) x (EX + 2)   input planes iz-1, iz, iz+1 (ring by plane index mod 3)
//   sT    6 x EY x EX               gradient products of plane iz on the haloed region
//   sY    6 x 8 x EX                blurred along y
//   ring  K x 6 x 8 x 32            blurred along y and x, last K planes
__global__ void __launch_bounds__(STX * STY) k_st3_any(StArgs a) {
    extern __shared__ __align__(16) float sm[];
    const int K = a.K;
    const int EX = STX + K - 1, EY = STY + K - 1;
    const int RX = EX + 2, RY = EY + 2;
    float* raw = sm;
    float* sT = raw + 3 * RY * RX;
    float* sY = sT + 6 * EY * EX;
    float* ring = sY + 6 * STY * EX;
    __shared__ float g[MAXK];
    const int tid = threadIdx.y * STX + threadIdx.x;
    const int nthr = STX * STY;
    if (tid < K) g[tid] = a.g[tid];

    const int ox0 = blockIdx.x * STX, oy0 = blockIdx.y * STY;
    const int oz_lo = blockIdx.z * a.zchunk, oz_hi = min(a.o0 - 1, oz_lo + a.zchunk - 1);
    const int iz_lo = oz_lo - a.off, iz_hi = oz_hi + K - 1 - a.off;   // input planes feeding [oz_lo, oz_hi]
    const int ix0 = ox0 - a.off, iy0 = oy0 - a.off;                     // input coords of the product region
    const size_t on = size_t(a.o0) * a.o1 * a.o2;

    // raw plane p -> slot, region x in [ix0 - 1, ix0 + EX], y in [iy0 - 1, iy0 + EY]
    auto load_raw = [&](int p) {
        float* dst = raw + (((p % 3) + 3) % 3) * RY * RX;
        const bool zin = p >= 0 && p < a.s0;
        for (int e = tid; e < RY * RX; e += nthr) {
            const int ry = e / RX, rx = e - ry * RX;
            const int x = ix0 - 1 + rx, y = iy0 - 1 + ry;
            float v = 0.0f;
            if (zin && (unsigned)x < (unsigned)a.s2 && (unsigned)y < (unsigned)a.s1)
                v = __ldg(a.vol + (size_t(p) * a.s1 + y) * a.s2 + x);
            dst[e] = v;
        }
    };
    load_raw(iz_lo - 1);
    load_raw(iz_lo);
    for (int iz = iz_lo; iz <= iz_hi; ++iz) {
        load_raw(iz + 1);
        __syncthreads();
        // gradient products on the haloed region (zero outside the volume)
        {
            const float* R0 = raw + ((((iz - 1) % 3) + 3) % 3) * RY * RX;
            const float* R1 = raw + (((iz % 3) + 3) % 3) * RY * RX;
            const float* R2 = raw + ((((iz + 1) % 3) + 3) % 3) * RY * RX;
            const bool zin = iz >= 0 && iz < a.s0;
            const int ps = EY * EX;
            for (int e = tid; e < ps; e += nthr) {
                const int ry = e / EX, rx = e - ry * EX;
                const int x = ix0 + rx, y = iy0 + ry;
                float gx = 0.0f, gy = 0.0f, gz = 0.0f;
                if (zin && (unsigned)x < (unsigned)a.s2 && (unsigned)y < (unsigned)a.s1) {
                    const int c = (ry + 1) * RX + rx + 1;
                    gx = grad1(R1[c - 1], R1[c], R1[c + 1], x, a.s2);
                    gy = grad1(R1[c - RX], R1[c], R1[c + RX], y, a.s1);
                    gz = grad1(R0[c], R1[c], R2[c], iz, a.s0);
                }
                sT[e] = gx * gx; sT[ps + e] = gx * gy; sT[2 * ps + e] = gx * gz;
                sT[3 * ps + e] = gy * gy; sT[4 * ps + e] = gy * gz; sT[5 * ps + e] = gz * gz;
            }
        }
        __syncthreads();
        // blur along y: sY[c][ty][rx]
        for (int e = tid; e < 6 * STY * EX; e += nthr) {
            const int c = e / (STY * EX), r = e - c * STY * EX, ty = r / EX, rx = r - ty * EX;
            const float* src = sT + c * EY * EX + ty * EX + rx;
            float sacc = 0.0f;
            for (int k = 0; k < K; ++k) sacc = fmaf(g[k], src[k * EX], sacc);
            sY[e] = sacc;
        }
        __syncthreads();
        // blur along x into the ring slot of this plane
        {
            float* slot = ring + ((iz - iz_lo) % K) * 6 * STY * STX;
            for (int e = tid; e < 6 * STY * STX; e += nthr) {
                const int c = e / (STY * STX), r = e - c * STY * STX, ty = r / STX, tx = r - ty * STX;
                const float* src = sY + c * STY * EX + ty * EX + tx;
                float sacc = 0.0f;
                for (int k = 0; k < K; ++k) sacc = fmaf(g[k], src[k], sacc);
                slot[e] = sacc;
            }
        }
        __syncthreads();
        // output plane oz = iz - (K - 1) + off is complete: blur along z and write
        const int oz = iz - (K - 1) + a.off;
        if (oz >= oz_lo && oz <= oz_hi) {
            const int x = ox0 + threadIdx.x, y = oy0 + threadIdx.y;
            float v[6];
            for (int c = 0; c < 6; ++c) v[c] = 0.0f;
            for (int k = 0; k < K; ++k) {
                const float* sl = ring + ((oz + k - a.off - iz_lo) % K) * 6 * STY * STX + threadIdx.y * STX + threadIdx.x;
                for (int c = 0; c < 6; ++c) v[c] = fmaf(g[k], sl[c * STY * STX], v[c]);
            }
            if (x < a.o2 && y < a.o1) {
                const size_t idx = (size_t(oz) * a.o1 + y) * a.o2 + x;
                if (a.layout == TVGB_LAYOUT_SYM6_PLANES) {
                    for (int c = 0; c < 6; ++c) a.out[c * on + idx] = v[c];
                } else if (a.layout == TVGB_LAYOUT_SYM6) {
                    for (int c = 0; c < 6; ++c) a.out[idx * 6 + c] = v[c];
                } else {
                    float* o = a.out + idx * 9;
                    o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; o[3] = v[1]; o[4] = v[3];
                    o[5] = v[4]; o[6] = v[2]; o[7] = v[4]; o[8] = v[5];
                }
            }
        }
        // the next iteration's raw load writes the slot of plane iz - 1, last
        // read before the barrier that follows the products; its ring write
        // (slot of plane iz + 1 - K, read just above) comes after two barriers
    }
}

// Fixed-K variant (odd K <= ST_MAXT).  Same arithmetic, reorganised so that
// each shared-memory value feeds several FMAs:
//   * y blur: one thread per (channel, haloed column) computes the tile's 8
//     rows from one pass down the column, kept in registers;
//   * x blur: one thread per (channel triple, row, pair of x) reads its row
//     segment with 64-bit loads and produces both outputs;
//   * z blur: each thread keeps, for its 6 outputs, the K partial sums of the
//     planes in flight in registers; slot (plane mod K) is resolved by a
//     warp-uniform dispatch so every index is static;
//   * the next raw plane is fetched into registers before the products and
//     stored after them, so its global latency overlaps two stages.
constexpr int ST_MAXT = 13;

template <int K, int J>
__device__ __forceinline__ void st_zstep(float (&acc)[6][K], const float (&v)[6], const float (&gw)[K],
                                         float (&done)[6]) {
#pragma unroll
    for (int m = 0; m < K; ++m) {
        const int sl = (J - m + K) % K;
#pragma unroll
        for (int o = 0; o < 6; ++o) acc[o][sl] = fmaf(gw[m], v[o], acc[o][sl]);
    }
    constexpr int sd = (J + 1) % K;
#pragma unroll
    for (int o = 0; o < 6; ++o) { done[o] = acc[o][sd]; acc[o][sd] = 0.0f; }
}

// slot j of the z-window, resolved by one indexed branch
template <int K>
__device__ __forceinline__ void st_zdispatch(int j, float (&acc)[6][K], const float (&v)[6], const float (&gw)[K],
                                             float (&done)[6]) {
#define TVGB_ZCASE(J) \
    case J:           \
        if constexpr (J < K) st_zstep<K, J>(acc, v, gw, done); \
        break;
    switch (j) {
        TVGB_ZCASE(0) TVGB_ZCASE(1) TVGB_ZCASE(2) TVGB_ZCASE(3) TVGB_ZCASE(4) TVGB_ZCASE(5) TVGB_ZCASE(6)
        TVGB_ZCASE(7) TVGB_ZCASE(8) TVGB_ZCASE(9) TVGB_ZCASE(10) TVGB_ZCASE(11) TVGB_ZCASE(12)
        default: break;
    }
#undef TVGB_ZCASE
}

// twice volume<T>::gradient's rule (central difference inside, one-sided at
// the edges); the factor 4 on the products is taken out by the z weights
__device__ __forceinline__ float grad2(float lo, float c, float hi, int p, int S) {
    if (S < 2) return 0.0f;
    if (p == 0) return 2.0f * (hi - c);
    if (p == S - 1) return 2.0f * (c - lo);
    return hi - lo;
}

template <int K>
__global__ void __launch_bounds__(STX * STY, 2) k_st3(StArgs a) {
    static_assert(K <= ST_MAXT, "fixed-tap kernel");
    constexpr int EX = STX + K - 1, EY = STY + K - 1;   // EX even: 64-bit row loads stay aligned
    constexpr int RX = EX + 2, RY = EY + 2;
    constexpr int NT = STX * STY;
    constexpr int NR = (RY * RX + NT - 1) / NT;          // raw elements per thread per plane
    constexpr int PS = EY * EX;                          // product points per plane
    constexpr int NP = (PS + NT - 1) / NT;               // product points per thread
    __shared__ __align__(16) float raw[3 * RY * RX];
    __shared__ __align__(16) float sT[6 * PS];
    __shared__ __align__(16) float sY[6 * STY * EX];
    const int tid = threadIdx.x;
    float gw[K], gz[K];
#pragma unroll
    for (int k = 0; k < K; ++k) { gw[k] = a.g[k]; gz[k] = 0.25f * a.g[k]; }

    const int ox0 = blockIdx.x * STX, oy0 = blockIdx.y * STY;
    const int oz_lo = blockIdx.z * a.zchunk, oz_hi = min(a.o0 - 1, oz_lo + a.zchunk - 1);
    const int iz_lo = oz_lo - a.off, iz_hi = oz_hi + K - 1 - a.off;
    const int ix0 = ox0 - a.off, iy0 = oy0 - a.off;
    const size_t on = size_t(a.o0) * a.o1 * a.o2;
    const size_t plane = size_t(a.s1) * a.s2;
    // every product point and its x/y neighbours inside the volume: no edge rules in x, y
    const bool inner = ix0 >= 1 && ix0 + EX <= a.s2 - 1 && iy0 >= 1 && iy0 + EY <= a.s1 - 1;

    // owned outputs: channels 3h..3h+2 at (x0 + {0,1}, y) of every plane
    const int h = tid >> 7, ty = (tid >> 4) & 7, px = (tid & 15) * 2;
    const int y = oy0 + ty, x0 = ox0 + px;

    // raw elements of this thread: in-plane offset, or -1 outside the volume / region
    int foff[NR];
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        const int e = tid + r * NT;
        const int ry = e / RX, rx = e - ry * RX;
        const int gxr = ix0 - 1 + rx, gyr = iy0 - 1 + ry;
        foff[r] = (e < RY * RX && (unsigned)gxr < (unsigned)a.s2 && (unsigned)gyr < (unsigned)a.s1) ? gyr * a.s2 + gxr
                                                                                                  : -1;
    }
    float pre[NR];
    auto fetch = [&](int p) {
        const bool zin = p >= 0 && p < a.s0;
        const float* src = a.vol + size_t(zin ? p : 0) * plane;
#pragma unroll
        for (int r = 0; r < NR; ++r) pre[r] = (zin && foff[r] >= 0) ? __ldg(src + foff[r]) : 0.0f;
    };
    auto store = [&](int p) {
        float* dst = raw + (((p % 3) + 3) % 3) * RY * RX;
#pragma unroll
        for (int r = 0; r < NR; ++r)
            if (tid + r * NT < RY * RX) dst[tid + r * NT] = pre[r];
    };
    fetch(iz_lo - 1); store(iz_lo - 1);
    fetch(iz_lo); store(iz_lo);
    fetch(iz_lo + 1); store(iz_lo + 1);

    float acc[6][K];
#pragma unroll
    for (int o = 0; o < 6; ++o)
#pragma unroll
        for (int k = 0; k < K; ++k) acc[o][k] = 0.0f;

    for (int iz = iz_lo; iz <= iz_hi; ++iz) {
        const bool zin = iz >= 0 && iz < a.s0;
        fetch(iz + 2);
        __syncthreads();   // raw plane iz + 1 stored; previous x blur done with sY
        if (zin) {
            const float* R0 = raw + ((((iz - 1) % 3) + 3) % 3) * RY * RX;
            const float* R1 = raw + (((iz % 3) + 3) % 3) * RY * RX;
            const float* R2 = raw + ((((iz + 1) % 3) + 3) % 3) * RY * RX;
            if (inner && iz >= 1 && iz <= a.s0 - 2) {
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    const int e = tid + q * NT;
                    if (e < PS) {
                        const int ry = e / EX, rx = e - ry * EX;
                        const int c = (ry + 1) * RX + rx + 1;
                        const float gx = R1[c + 1] - R1[c - 1];
                        const float gy = R1[c + RX] - R1[c - RX];
                        const float gzv = R2[c] - R0[c];
                        sT[e] = gx * gx; sT[PS + e] = gx * gy; sT[2 * PS + e] = gx * gzv;
                        sT[3 * PS + e] = gy * gy; sT[4 * PS + e] = gy * gzv; sT[5 * PS + e] = gzv * gzv;
                    }
                }
            } else {
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    const int e = tid + q * NT;
                    if (e < PS) {
                        const int ry = e / EX, rx = e - ry * EX;
                        const int gxp = ix0 + rx, gyp = iy0 + ry;
                        float gx = 0.0f, gy = 0.0f, gzv = 0.0f;
                        if ((unsigned)gxp < (unsigned)a.s2 && (unsigned)gyp < (unsigned)a.s1) {
                            const int c = (ry + 1) * RX + rx + 1;
                            gx = grad2(R1[c - 1], R1[c], R1[c + 1], gxp, a.s2);
                            gy = grad2(R1[c - RX], R1[c], R1[c + RX], gyp, a.s1);
                            gzv = grad2(R0[c], R1[c], R2[c], iz, a.s0);
                        }
                        sT[e] = gx * gx; sT[PS + e] = gx * gy; sT[2 * PS + e] = gx * gzv;
                        sT[3 * PS + e] = gy * gy; sT[4 * PS + e] = gy * gzv; sT[5 * PS + e] = gzv * gzv;
                    }
                }
            }
        }
        __syncthreads();   // products ready; raw plane iz - 1 no longer read
        store(iz + 2);
        if (zin) {
            for (int it = tid; it < 6 * EX; it += NT) {
                const int c = it / EX, rx = it - c * EX;
                const float* col = sT + c * PS + rx;
                float cv[EY];
#pragma unroll
                for (int r = 0; r < EY; ++r) cv[r] = col[r * EX];
#pragma unroll
                for (int t = 0; t < STY; ++t) {
                    float s = 0.0f;
#pragma unroll
                    for (int k = 0; k < K; ++k) s = fmaf(gw[k], cv[t + k], s);
                    sY[(c * STY + t) * EX + rx] = s;
                }
            }
        }
        __syncthreads();   // y blur ready
        float v[6];
        if (zin) {
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                const float2* row = reinterpret_cast<const float2*>(sY + ((3 * h + cc) * STY + ty) * EX + px);
                float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
                for (int q = 0; q < (K + 1) / 2; ++q) {
                    const float2 u = row[q];
                    // u.x = sY[px + 2q], u.y = sY[px + 2q + 1]
                    if (2 * q < K) s0 = fmaf(gw[2 * q], u.x, s0);
                    if (2 * q + 1 < K) s0 = fmaf(gw[2 * q + 1], u.y, s0);
                    if (2 * q >= 1) s1 = fmaf(gw[2 * q - 1], u.x, s1);
                    s1 = fmaf(gw[2 * q], u.y, s1);
                }
                v[2 * cc] = s0; v[2 * cc + 1] = s1;
            }
        } else {
#pragma unroll
            for (int o = 0; o < 6; ++o) v[o] = 0.0f;
        }
        float done[6];
        st_zdispatch<K>((iz - iz_lo) % K, acc, v, gz, done);
        // the slot just completed began at plane iz - K + 1: output oz
        const int oz = iz - (K - 1) + a.off;
        if (oz >= oz_lo && y < a.o1 && a.pair_store) {
            // planes, even row length, 8-byte aligned output: the thread's two x neighbours as one 64-bit store per
            // channel (x0 even, so both are in the row or neither)
            if (x0 < a.o2) {
                float2* o = reinterpret_cast<float2*>(a.out + (3 * h) * on + (size_t(oz) * a.o1 + y) * a.o2 + x0);
                const size_t on2 = on / 2;
                o[0] = make_float2(done[0], done[1]);
                o[on2] = make_float2(done[2], done[3]);
                o[2 * on2] = make_float2(done[4], done[5]);
            }
        } else if (oz >= oz_lo && y < a.o1) {
            const size_t row0 = (size_t(oz) * a.o1 + y) * a.o2;
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int x = x0 + u;
                if (x >= a.o2) continue;
                const size_t idx = row0 + x;
                const float c0 = done[u], c1 = done[2 + u], c2 = done[4 + u];   // channels 3h, 3h+1, 3h+2
                if (a.layout == TVGB_LAYOUT_SYM6_PLANES) {
                    a.out[(3 * h) * on + idx] = c0; a.out[(3 * h + 1) * on + idx] = c1; a.out[(3 * h + 2) * on + idx] = c2;
                } else if (a.layout == TVGB_LAYOUT_SYM6) {
                    float* o = a.out + idx * 6 + 3 * h;
                    o[0] = c0; o[1] = c1; o[2] = c2;
                } else {
                    float* o = a.out + idx * 9;
                    if (h == 0) { o[0] = c0; o[1] = c1; o[3] = c1; o[2] = c2; o[6] = c2; }
                    else { o[4] = c0; o[5] = c1; o[7] = c1; o[8] = c2; }
                }
            }
        }
    }
}

// ------------------------------------------------------------------ TMA-staged raw planes
// k_st3 with its raw z-planes staged by the Tensor Memory Accelerator, for
// volumes whose rows meet the TMA rules (s2 % 4 == 0, 16-byte aligned): one
// thread issues a cp.async.bulk.tensor box per plane (the tile with its halo,
// zero outside the volume) ST_TMA_AHEAD planes ahead into a ring of
// ST_TMA_SLOTS slots with one mbarrier each.  The other threads spend no
// registers or load instructions on the staging and wait only on the
// mbarrier; one block barrier per plane goes (two remain).  Every wait is
// bounded: a wait that runs out ends the CTA's loop at its next barrier and
// thread 0 waits, bounded, for the copies still in flight before the CTA
// exits (g_st3_faults counts such CTAs).
constexpr int ST_TMA_SLOTS = 8, ST_TMA_AHEAD = 6;   // slots >= ahead + 2: a slot is reused two planes after its last read
constexpr uint32_t ST_TMA_WAIT_LIMIT = 1u << 24;    // mbarrier polls before a CTA gives up

template <int K>
struct St3TmaGeom {
    static constexpr int EX = STX + K - 1, EY = STY + K - 1;
    static constexpr int BX = (EX + 2 + 3 + 3) / 4 * 4;  // box width: raw columns EX + 2 after a shift rs <= 3
    static constexpr int BY = EY + 2;
    static constexpr int SLOT = (BX * BY + 31) / 32 * 32;   // floats per ring slot (128-byte multiples)
    static constexpr uint32_t BOX_BYTES = uint32_t(BX) * BY * 4;
    // channel strides of the products and of the y-blurred rows, padded to EX mod 32 words: a warp's 32
    // consecutive (channel, column) tasks of the y blur that cross into the next channel then continue on the
    // next banks instead of meeting their own first lanes (2-way conflicts for 5 of a CTA's 8 warps otherwise)
    static constexpr int PSP = EY * EX + ((EX - EY * EX) % 32 + 32) % 32;
    static constexpr int SYP = STY * EX + ((EX - STY * EX) % 32 + 32) % 32;
    // raw ring, products sT[6][PSP], y-blurred rows sY[6][SYP], then the slots' mbarriers
    static constexpr size_t SMEM = sizeof(float) * (size_t(ST_TMA_SLOTS) * SLOT + 6 * PSP + 6 * SYP) + 8 * ST_TMA_SLOTS;
};

static __device__ unsigned g_st3_faults;             // CTAs whose plane wait timed out

template <int K>
__global__ void __launch_bounds__(STX * STY, 2) k_st3_tma(const __grid_constant__ CUtensorMap vmap, StArgs a) {
    static_assert(K <= ST_MAXT, "fixed-tap kernel");
    constexpr int EX = STX + K - 1, EY = STY + K - 1;   // EX even: 64-bit row loads stay aligned
    using G = St3TmaGeom<K>;
    constexpr int RX = G::BX, RY = EY + 2;                // raw row pitch: the TMA box width
    constexpr int NT = STX * STY;
    constexpr int PS = EY * EX;                          // product points per plane
    constexpr int NP = (PS + NT - 1) / NT;               // product points per thread
    extern __shared__ __align__(128) float smem[];
    float* raw = smem;                                   // ST_TMA_SLOTS slots of G::SLOT floats
    float* sT = raw + ST_TMA_SLOTS * G::SLOT;
    constexpr int PSP = G::PSP, SYP = G::SYP;            // padded channel strides
    float* sY = sT + 6 * PSP;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sY + 6 * SYP);
    const int tid = threadIdx.x;
    float gw[K], gz[K];
#pragma unroll
    for (int k = 0; k < K; ++k) { gw[k] = a.g[k]; gz[k] = 0.25f * a.g[k]; }

    const int ox0 = blockIdx.x * STX, oy0 = blockIdx.y * STY;
    const int oz_lo = blockIdx.z * a.zchunk, oz_hi = min(a.o0 - 1, oz_lo + a.zchunk - 1);
    const int iz_lo = oz_lo - a.off, iz_hi = oz_hi + K - 1 - a.off;
    const int ix0 = ox0 - a.off, iy0 = oy0 - a.off;
    const size_t on = size_t(a.o0) * a.o1 * a.o2;
    const size_t plane = size_t(a.s1) * a.s2;
    // every product point and its x/y neighbours inside the volume: no edge rules in x, y
    const bool inner = ix0 >= 1 && ix0 + EX <= a.s2 - 1 && iy0 >= 1 && iy0 + EY <= a.s1 - 1;

    // owned outputs: channels 3h..3h+2 at (x0 + {0,1}, y) of every plane
    const int h = tid >> 7, ty = (tid >> 4) & 7, px = (tid & 15) * 2;
    const int y = oy0 + ty, x0 = ox0 + px;

    // raw tile: columns ix0 - 1 .. ix0 + EX, rows iy0 - 1 .. iy0 + EY; the box starts rs columns further left so
    // that its x coordinate is a multiple of 4 (the TMA rule), and element (ry, rx) sits at ry * RX + rx + rs
    const int rs = ((-a.off - 1) % 4 + 4) % 4;
    const int bx0 = ix0 - 1 - rs, by0 = iy0 - 1;
    const int P0 = iz_lo - 1, qmax = iz_hi + 1 - P0;     // raw planes P0 + q, q = 0 .. qmax
    if (tid == 0)
        for (int i = 0; i < ST_TMA_SLOTS; ++i) tc::mbar_init(&bars[i], 1);
    __syncthreads();
    auto issue = [&](int q) {   // thread 0: raw plane P0 + q into slot q % SLOTS
        uint64_t* b = &bars[q % ST_TMA_SLOTS];
        tma::fence_proxy_async();
        tma::arrive_expect_tx(b, G::BOX_BYTES);
        tma::load_3d(raw + (q % ST_TMA_SLOTS) * G::SLOT, &vmap, bx0, by0, P0 + q, b);
    };
    if (tid == 0)
        for (int q = 0; q <= min(ST_TMA_AHEAD, qmax); ++q) issue(q);
    int issued = min(ST_TMA_AHEAD, qmax);
    bool timed_out = false;
    auto wait = [&](int q) {
        if (!tc::mbar_wait(&bars[q % ST_TMA_SLOTS], uint32_t(q / ST_TMA_SLOTS) & 1u, ST_TMA_WAIT_LIMIT))
            timed_out = true;
    };
    wait(0);
    wait(1);

    float acc[6][K];
#pragma unroll
    for (int o = 0; o < 6; ++o)
#pragma unroll
        for (int k = 0; k < K; ++k) acc[o][k] = 0.0f;

    int qfail = -1;
    for (int iz = iz_lo; iz <= iz_hi; ++iz) {
        const bool zin = iz >= 0 && iz < a.s0;
        const int qz = iz - P0;                          // this plane's ring index; its neighbours qz - 1, qz + 1
        // the plane ST_TMA_AHEAD ahead goes into the slot of plane qz + AHEAD - SLOTS <= qz - 2, last read by the
        // products of the previous plane, before the barrier that followed them
        if (tid == 0 && issued < qmax) issue(++issued);
        wait(qz + 1);
        if (zin) {
            const float* R0 = raw + ((qz - 1) % ST_TMA_SLOTS) * G::SLOT + rs;
            const float* R1 = raw + (qz % ST_TMA_SLOTS) * G::SLOT + rs;
            const float* R2 = raw + ((qz + 1) % ST_TMA_SLOTS) * G::SLOT + rs;
            if (inner && iz >= 1 && iz <= a.s0 - 2) {
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    const int e = tid + q * NT;
                    if (e < PS) {
                        const int ry = e / EX, rx = e - ry * EX;
                        const int c = (ry + 1) * RX + rx + 1;
                        const float gx = R1[c + 1] - R1[c - 1];
                        const float gy = R1[c + RX] - R1[c - RX];
                        const float gzv = R2[c] - R0[c];
                        sT[e] = gx * gx; sT[PSP + e] = gx * gy; sT[2 * PSP + e] = gx * gzv;
                        sT[3 * PSP + e] = gy * gy; sT[4 * PSP + e] = gy * gzv; sT[5 * PSP + e] = gzv * gzv;
                    }
                }
            } else {
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    const int e = tid + q * NT;
                    if (e < PS) {
                        const int ry = e / EX, rx = e - ry * EX;
                        const int gxp = ix0 + rx, gyp = iy0 + ry;
                        float gx = 0.0f, gy = 0.0f, gzv = 0.0f;
                        if ((unsigned)gxp < (unsigned)a.s2 && (unsigned)gyp < (unsigned)a.s1) {
                            const int c = (ry + 1) * RX + rx + 1;
                            gx = grad2(R1[c - 1], R1[c], R1[c + 1], gxp, a.s2);
                            gy = grad2(R1[c - RX], R1[c], R1[c + RX], gyp, a.s1);
                            gzv = grad2(R0[c], R1[c], R2[c], iz, a.s0);
                        }
                        sT[e] = gx * gx; sT[PSP + e] = gx * gy; sT[2 * PSP + e] = gx * gzv;
                        sT[3 * PSP + e] = gy * gy; sT[4 * PSP + e] = gy * gzv; sT[5 * PSP + e] = gzv * gzv;
                    }
                }
            }
        }
        // products ready; raw plane iz - 1 no longer read.  A wait that ran out ends the loop here, for all threads
        if (__syncthreads_or(timed_out)) { qfail = qz; break; }
        if (zin) {
            for (int it = tid; it < 6 * EX; it += NT) {
                const int c = it / EX, rx = it - c * EX;
                const float* col = sT + c * PSP + rx;
                float cv[EY];
#pragma unroll
                for (int r = 0; r < EY; ++r) cv[r] = col[r * EX];
#pragma unroll
                for (int t = 0; t < STY; ++t) {
                    float s = 0.0f;
#pragma unroll
                    for (int k = 0; k < K; ++k) s = fmaf(gw[k], cv[t + k], s);
                    sY[c * SYP + t * EX + rx] = s;
                }
            }
        }
        __syncthreads();   // y blur ready
        float v[6];
        if (zin) {
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                const float2* row = reinterpret_cast<const float2*>(sY + (3 * h + cc) * SYP + ty * EX + px);
                float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
                for (int q = 0; q < (K + 1) / 2; ++q) {
                    const float2 u = row[q];
                    // u.x = sY[px + 2q], u.y = sY[px + 2q + 1]
                    if (2 * q < K) s0 = fmaf(gw[2 * q], u.x, s0);
                    if (2 * q + 1 < K) s0 = fmaf(gw[2 * q + 1], u.y, s0);
                    if (2 * q >= 1) s1 = fmaf(gw[2 * q - 1], u.x, s1);
                    s1 = fmaf(gw[2 * q], u.y, s1);
                }
                v[2 * cc] = s0; v[2 * cc + 1] = s1;
            }
        } else {
#pragma unroll
            for (int o = 0; o < 6; ++o) v[o] = 0.0f;
        }
        float done[6];
        st_zdispatch<K>((iz - iz_lo) % K, acc, v, gz, done);
        // the slot just completed began at plane iz - K + 1: output oz
        const int oz = iz - (K - 1) + a.off;
        if (oz >= oz_lo && y < a.o1 && a.pair_store) {
            // planes, even row length, 8-byte aligned output: the thread's two x neighbours as one 64-bit store per
            // channel (x0 even, so both are in the row or neither)
            if (x0 < a.o2) {
                float2* o = reinterpret_cast<float2*>(a.out + (3 * h) * on + (size_t(oz) * a.o1 + y) * a.o2 + x0);
                const size_t on2 = on / 2;
                o[0] = make_float2(done[0], done[1]);
                o[on2] = make_float2(done[2], done[3]);
                o[2 * on2] = make_float2(done[4], done[5]);
            }
        } else if (oz >= oz_lo && y < a.o1) {
            const size_t row0 = (size_t(oz) * a.o1 + y) * a.o2;
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int x = x0 + u;
                if (x >= a.o2) continue;
                const size_t idx = row0 + x;
                const float c0 = done[u], c1 = done[2 + u], c2 = done[4 + u];   // channels 3h, 3h+1, 3h+2
                if (a.layout == TVGB_LAYOUT_SYM6_PLANES) {
                    a.out[(3 * h) * on + idx] = c0; a.out[(3 * h + 1) * on + idx] = c1; a.out[(3 * h + 2) * on + idx] = c2;
                } else if (a.layout == TVGB_LAYOUT_SYM6) {
                    float* o = a.out + idx * 6 + 3 * h;
                    o[0] = c0; o[1] = c1; o[2] = c2;
                } else {
                    float* o = a.out + idx * 9;
                    if (h == 0) { o[0] = c0; o[1] = c1; o[3] = c1; o[2] = c2; o[6] = c2; }
                    else { o[4] = c0; o[5] = c1; o[7] = c1; o[8] = c2; }
                }
            }
        }
    }
    if (qfail >= 0 && tid == 0) {
        // the planes from qfail + 1 on may still be in flight (each slot holds at most one of them): wait for them
        // before the shared memory is released
        atomicAdd(&g_st3_faults, 1u);
        for (int q = qfail + 1; q <= issued; ++q)
            tc::mbar_wait(&bars[q % ST_TMA_SLOTS], uint32_t(q / ST_TMA_SLOTS) & 1u, ST_TMA_WAIT_LIMIT);
    }
}

void structure_tensor3_dims(unsigned s0, unsigned s1, unsigned s2, float sigma, int mode, unsigned* d) {
    const unsigned K = ksize3(sigma);
    if (mode == 0) {
        d[0] = s0 >= K ? s0 - K + 1 : 0;
        d[1] = s1 >= K ? s1 - K + 1 : 0;
        d[2] = s2 >= K ? s2 - K + 1 : 0;
    } else {
        d[0] = s0; d[1] = s1; d[2] = s2;
    }
}

int structure_tensor3_device(const float* vol, unsigned s0, unsigned s1, unsigned s2, float sigma, int mode,
                             float* out, int out_layout, unsigned* out_dims, cudaStream_t st) {
    const unsigned K = ksize3(sigma);
    if (K > MAXK) { set_error("structure tensor: sigma %g gives %u taps (max %d)", sigma, K, MAXK); return TVGB_ERR_UNSUPPORTED; }
    unsigned d[3];
    structure_tensor3_dims(s0, s1, s2, sigma, mode, d);
    if (out_dims) { out_dims[0] = d[0]; out_dims[1] = d[1]; out_dims[2] = d[2]; }
    if (size_t(d[0]) * d[1] * d[2] == 0) return TVGB_OK;
    StArgs a{};
    a.vol = vol; a.s0 = int(s0); a.s1 = int(s1); a.s2 = int(s2);
    a.o0 = int(d[0]); a.o1 = int(d[1]); a.o2 = int(d[2]);
    a.K = int(K); a.off = mode == 0 ? 0 : int(K / 2);
    gaussian1d(K, sigma, a.g);
    a.out = out; a.layout = out_layout;
    a.pair_store = out_layout == TVGB_LAYOUT_SYM6_PLANES && d[2] % 2 == 0 && reinterpret_cast<uintptr_t>(out) % 8 == 0;
    const unsigned gx = ceil_div(d[2], STX), gy = ceil_div(d[1], STY);
    const bool fixed = K <= unsigned(ST_MAXT);
    const int EX = STX + int(K) - 1, EY = STY + int(K) - 1;
    size_t smem = fixed ? 0
                        : sizeof(float) * (size_t(3) * (EY + 2) * (EX + 2) + size_t(6) * EY * EX +
                                                 size_t(6) * STY * EX + size_t(K) * 6 * STY * STX);
    // the TMA kernel when the volume's rows meet the TMA rules (16-byte aligned rows)
    CUtensorMap vmap;
    bool tma = false;
    size_t tma_smem = 0;
    const void* tfn = nullptr;
    switch (K) {
        case 3: tfn = (const void*)k_st3_tma<3>; tma_smem = St3TmaGeom<3>::SMEM; break;
        case 5: tfn = (const void*)k_st3_tma<5>; tma_smem = St3TmaGeom<5>::SMEM; break;
        case 7: tfn = (const void*)k_st3_tma<7>; tma_smem = St3TmaGeom<7>::SMEM; break;
        case 9: tfn = (const void*)k_st3_tma<9>; tma_smem = St3TmaGeom<9>::SMEM; break;
        case 11: tfn = (const void*)k_st3_tma<11>; tma_smem = St3TmaGeom<11>::SMEM; break;
        case 13: tfn = (const void*)k_st3_tma<13>; tma_smem = St3TmaGeom<13>::SMEM; break;
        default: break;
    }
    if (tfn && s2 % 4 == 0) {
        unsigned bx = 0, by = 0;
        switch (K) {
            case 3: bx = St3TmaGeom<3>::BX; by = St3TmaGeom<3>::BY; break;
            case 5: bx = St3TmaGeom<5>::BX; by = St3TmaGeom<5>::BY; break;
            case 7: bx = St3TmaGeom<7>::BX; by = St3TmaGeom<7>::BY; break;
            case 9: bx = St3TmaGeom<9>::BX; by = St3TmaGeom<9>::BY; break;
            case 11: bx = St3TmaGeom<11>::BX; by = St3TmaGeom<11>::BY; break;
            case 13: bx = St3TmaGeom<13>::BX; by = St3TmaGeom<13>::BY; break;
            default: break;
        }
        tma = make_tmap_3d_f32(&vmap, vol, s2, s1, s0, bx, by);
    }
    const void* fn = nullptr;
    switch (K) {
        case 3: fn = (const void*)k_st3<3>; break;
        case 5: fn = (const void*)k_st3<5>; break;
        case 7: fn = (const void*)k_st3<7>; break;
        case 9: fn = (const void*)k_st3<9>; break;
        case 11: fn = (const void*)k_st3<11>; break;
        case 13: fn = (const void*)k_st3<13>; break;
        default: fn = (const void*)k_st3_any; break;
    }
    if (tma) {
        fn = tfn;
        smem = tma_smem;
        TVGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    } else if (!fixed) {
        TVGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    }
    // z chunk.  Each CTA walks zc + K - 1 planes (K - 1 of them ramp).  Cost
    // model: the busiest SM's planes, divided by the speed-up of running n
    // CTAs side by side on one SM (taken as n^0.7, n up to the occupancy).
    int dev = 0, sms = 0, per_sm = 0;
    TVGB_CUDA(cudaGetDevice(&dev));
    TVGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TVGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, STX * STY, smem));
    sms = std::max(1, sms);
    per_sm = std::max(1, per_sm);
    int zchunk = int(d[0]);
    double best = 0.0;
    for (int zc = int(d[0]); zc >= 1; zc = zc > 64 ? zc - zc / 16 : zc - 1) {
        const size_t ctas = size_t(gx) * gy * ceil_div(d[0], unsigned(zc));
        const size_t per = (ctas + size_t(sms) - 1) / size_t(sms);
        const double conc = std::pow(double(std::min(per, size_t(per_sm))), 0.7);
        const double cost = double(per) * double(zc + int(K) - 1) / conc;
        if (best == 0.0 || cost < best) { best = cost; zchunk = zc; }
    }
    a.zchunk = zchunk;
    dim3 grid(gx, gy, ceil_div(d[0], unsigned(zchunk)));
    {
        KernelTimer kt_(tma ? "k_st3_tma" : "k_st3", st);
        if (tma) {
            void* args[] = {&vmap, &a};
            TVGB_CUDA(cudaLaunchKernel(fn, grid, dim3(STX * STY), args, smem, st));
        } else if (fixed) {
            void* args[] = {&a};
            TVGB_CUDA(cudaLaunchKernel(fn, grid, dim3(STX * STY), args, 0, st));
        } else {
            k_st3_any<<<grid, dim3(STX, STY), smem, st>>>(a);
        }
        kt_.stop();
    }
    TVGB_LAUNCHED();
    return TVGB_OK;
}

// ------------------------------------------------------------------ 2D structure tensor
struct St2Args {
    const float* img;
    int s0, s1, o0, o1, K, offl;
    float g[MAXK];
    float* out4;
};

// np.gradient(..., edge_order=2) along one line at position p of S samples
__device__ __forceinline__ float grad_eo2(const float* f, size_t stride, int p, int S) {
    if (S < 3) return 0.0f;
    if (p == 0) return (-3.0f * f[0] + 4.0f * f[stride] - f[2 * stride]) / 2.0f;
    if (p == S - 1) return (3.0f * f[0] - 4.0f * f[-ptrdiff_t(stride)] + f[-2 * ptrdiff_t(stride)]) / 2.0f;
    return (f[stride] - f[-ptrdiff_t(stride)]) / 2.0f;
}

__global__ void k_st2(St2Args a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= a.o1 || y >= a.o0) return;
    float s[3] = {0, 0, 0};
    for (int i = 0; i < a.K; ++i) {
        const int r = y + i - a.offl;
        if (r < 0 || r >= a.s0) continue;
        float row[3] = {0, 0, 0};
        for (int j = 0; j < a.K; ++j) {
            const int c = x + j - a.offl;
            if (c < 0 || c >= a.s1) continue;
            const float* f = a.img + size_t(r) * a.s1 + c;
            const float gx = grad_eo2(f, 1, c, a.s1);
            const float gy = grad_eo2(f, size_t(a.s1), r, a.s0);
            row[0] = fmaf(a.g[j], gx * gx, row[0]);
            row[1] = fmaf(a.g[j], gx * gy, row[1]);
            row[2] = fmaf(a.g[j], gy * gy, row[2]);
        }
        for (int k = 0; k < 3; ++k) s[k] = fmaf(a.g[i], row[k], s[k]);
    }
    float4* o = reinterpret_cast<float4*>(a.out4) + size_t(y) * a.o1 + x;
    *o = make_float4(s[0], s[1], s[1], s[2]);
}

// ------------------------------------------------------------------ scalar separable pass
struct PassArgs {
    const float* src;
    float* dst;
    int sx, sy, sz;   // source dims (x fastest)
    int axis, K;
    float g[MAXK];
};

__global__ void k_pass(PassArgs a) {
    const int ox = a.sx - (a.axis == 0 ? a.K - 1 : 0);
    const int oy = a.sy - (a.axis == 1 ? a.K - 1 : 0);
    const int oz = a.sz - (a.axis == 2 ? a.K - 1 : 0);
    const size_t n = size_t(ox) * oy * oz;
    const size_t stride = a.axis == 0 ? 1 : (a.axis == 1 ? size_t(a.sx) : size_t(a.sx) * a.sy);
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const int x = int(i % ox), y = int((i / ox) % oy), z = int(i / (size_t(ox) * oy));
        const float* p = a.src + (size_t(z) * a.sy + y) * a.sx + x;
        float s = 0.0f;
        for (int k = 0; k < a.K; ++k) s += a.g[k] * __ldg(p + k * stride);
        a.dst[i] = s;
    }
}

static int pass(const float* src, float* dst, int sx, int sy, int sz, int axis, unsigned K, float sigma, cudaStream_t st) {
    PassArgs a{};
    a.src = src; a.dst = dst; a.sx = sx; a.sy = sy; a.sz = sz; a.axis = axis; a.K = int(K);
    gaussian1d(K, sigma, a.g);
    const size_t n = size_t(sx - (axis == 0 ? K - 1 : 0)) * (sy - (axis == 1 ? K - 1 : 0)) * (sz - (axis == 2 ? K - 1 : 0));
    size_t blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    {
        KernelTimer kt_("k_pass", st);
        k_pass<<<unsigned(blocks ? blocks : 1), 256, 0, st>>>(a);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    return TVGB_OK;
}

}  // namespace tvgb

using namespace tvgb;

extern "C" {

int tvgb_structure_tensor3(const float* volume, unsigned s0, unsigned s1, unsigned s2, float sigma, int mode, float* out,
                           int out_layout, unsigned* out_dims, void* stream) {
    TVGB_CHECK_ARG(volume && out, "tvgb_structure_tensor3: NULL pointer");
    TVGB_CHECK_ARG(sigma > 0.0f, "tvgb_structure_tensor3: sigma must be > 0");
    TVGB_CHECK_ARG(mode == 0 || mode == 1, "tvgb_structure_tensor3: mode must be 0 (valid) or 1 (same)");
    TVGB_CHECK_ARG(out_layout == TVGB_LAYOUT_MAT3 || out_layout == TVGB_LAYOUT_SYM6 || out_layout == TVGB_LAYOUT_SYM6_PLANES,
                   "tvgb_structure_tensor3: out_layout must be 9, 6 or 60");
    unsigned d[3];
    structure_tensor3_dims(s0, s1, s2, sigma, mode, d);
    TVGB_CHECK_ARG(mode == 1 || (s0 >= ksize3(sigma) && s1 >= ksize3(sigma) && s2 >= ksize3(sigma)),
                   "tvgb_structure_tensor3: volume smaller than the %u-tap window (valid mode)", ksize3(sigma));
    if (out_dims) { out_dims[0] = d[0]; out_dims[1] = d[1]; out_dims[2] = d[2]; }
    const size_t n = size_t(s0) * s1 * s2, no = size_t(d[0]) * d[1] * d[2];
    if (no == 0) return TVGB_OK;
    cudaStream_t st = as_stream(stream);
    DevArray din, dout;
    TVGB_TRY(din.in(volume, n * 4, st));
    TVGB_TRY(dout.out(out, no * (out_layout == TVGB_LAYOUT_MAT3 ? 36 : 24), st));
    TVGB_TRY(structure_tensor3_device(din.get<float>(), s0, s1, s2, sigma, mode, dout.get<float>(), out_layout, nullptr, st));
    TVGB_TRY(dout.finish());
    return sync_if(din.owned || dout.owned, st);
}

int tvgb_structure_tensor2(const float* image, unsigned s0, unsigned s1, float sigma, int mode, float* out4,
                           unsigned* out_dims, void* stream) {
    TVGB_CHECK_ARG(image && out4, "tvgb_structure_tensor2: NULL pointer");
    TVGB_CHECK_ARG(sigma > 0.0f, "tvgb_structure_tensor2: sigma must be > 0");
    TVGB_CHECK_ARG(mode == 0 || mode == 1, "tvgb_structure_tensor2: mode must be 0 or 1");
    const unsigned K = ksize2(sigma);
    TVGB_CHECK_ARG(K >= 1 && K <= MAXK, "tvgb_structure_tensor2: window (unsigned)(6 sigma) = %u out of range", K);
    TVGB_CHECK_ARG(mode == 1 || (s0 >= K && s1 >= K), "tvgb_structure_tensor2: image smaller than the window");
    St2Args a{};
    a.img = nullptr; a.s0 = int(s0); a.s1 = int(s1); a.K = int(K);
    a.offl = mode == 0 ? 0 : int((K - 1) / 2);
    a.o0 = mode == 0 ? int(s0 - K + 1) : int(s0);
    a.o1 = mode == 0 ? int(s1 - K + 1) : int(s1);
    gaussian1d(K, sigma, a.g);
    if (out_dims) { out_dims[0] = unsigned(a.o0); out_dims[1] = unsigned(a.o1); }
    const size_t n = size_t(s0) * s1, no = size_t(a.o0) * a.o1;
    if (no == 0) return TVGB_OK;
    cudaStream_t st = as_stream(stream);
    DevArray din, dout;
    TVGB_TRY(din.in(image, n * 4, st));
    TVGB_TRY(dout.out(out4, no * 16, st));
    TVGB_CHECK_ARG(reinterpret_cast<uintptr_t>(dout.dev) % 16 == 0, "tvgb_structure_tensor2: out4 must be 16-byte aligned");
    a.img = din.get<float>();
    a.out4 = dout.get<float>();
    dim3 blk(32, 8), grid(ceil_div(a.o1, 32), ceil_div(a.o0, 8));
    {
        KernelTimer kt_("k_st2", st);
        k_st2<<<grid, blk, 0, st>>>(a);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    TVGB_TRY(dout.finish());
    return sync_if(din.owned || dout.owned, st);
}

int tvgb_gaussian_filter3d(const float* src, unsigned width, unsigned height, unsigned depth, float sigma_w,
                           float sigma_h, float sigma_d, float* dst, unsigned* out_dims, void* stream) {
    TVGB_CHECK_ARG(src && dst, "tvgb_gaussian_filter3d: NULL pointer");
    TVGB_CHECK_ARG(sigma_w > 0 && sigma_h > 0 && sigma_d > 0, "tvgb_gaussian_filter3d: sigmas must be > 0");
    const unsigned kw = ksize3(sigma_w), kh = ksize3(sigma_h), kd = ksize3(sigma_d);
    TVGB_CHECK_ARG(kw <= MAXK && kh <= MAXK && kd <= MAXK, "tvgb_gaussian_filter3d: window too large");
    TVGB_CHECK_ARG(width >= kw && height >= kh && depth >= kd, "tvgb_gaussian_filter3d: volume smaller than the window");
    const unsigned ow = width - kw + 1, oh = height - kh + 1, od = depth - kd + 1;
    if (out_dims) { out_dims[0] = ow; out_dims[1] = oh; out_dims[2] = od; }
    cudaStream_t st = as_stream(stream);
    DevArray din, dout;
    TVGB_TRY(din.in(src, size_t(width) * height * depth * 4, st));
    TVGB_TRY(dout.out(dst, size_t(ow) * oh * od * 4, st));
    Scratch t1, t2;
    // same pass order as the reference GPU path: z, then y, then x (filter.h:471-511)
    TVGB_TRY(t1.alloc(size_t(width) * height * od * 4, st));
    TVGB_TRY(t2.alloc(size_t(width) * oh * od * 4, st));
    TVGB_TRY(pass(din.get<float>(), t1.get<float>(), int(width), int(height), int(depth), 2, kd, sigma_d, st));
    TVGB_TRY(pass(t1.get<float>(), t2.get<float>(), int(width), int(height), int(od), 1, kh, sigma_h, st));
    TVGB_TRY(pass(t2.get<float>(), dout.get<float>(), int(width), int(oh), int(od), 0, kw, sigma_w, st));
    TVGB_TRY(dout.finish());
    return sync_if(din.owned || dout.owned, st);
}

int tvgb_gaussian_convolve2(const float* src, unsigned in_sx, unsigned in_sy, float sigma1, float sigma2, float* dst,
                            unsigned* out_dims, void* stream) {
    TVGB_CHECK_ARG(src && dst, "tvgb_gaussian_convolve2: NULL pointer");
    TVGB_CHECK_ARG(sigma1 > 0 && sigma2 > 0, "tvgb_gaussian_convolve2: sigmas must be > 0");
    const unsigned kw = ksize2(sigma1), kh = ksize2(sigma2);
    TVGB_CHECK_ARG(kw >= 1 && kh >= 1 && kw <= MAXK && kh <= MAXK, "tvgb_gaussian_convolve2: window out of range");
    TVGB_CHECK_ARG(in_sx >= kw && in_sy >= kh, "tvgb_gaussian_convolve2: image smaller than the window");
    const unsigned ow = in_sx - kw + 1, oh = in_sy - kh + 1;
    if (out_dims) { out_dims[0] = ow; out_dims[1] = oh; }
    cudaStream_t st = as_stream(stream);
    DevArray din, dout;
    TVGB_TRY(din.in(src, size_t(in_sx) * in_sy * 4, st));
    TVGB_TRY(dout.out(dst, size_t(ow) * oh * 4, st));
    Scratch t1;
    // y pass then x pass, as cuda_convolve2y / 2x (filter.h:360-375)
    TVGB_TRY(t1.alloc(size_t(in_sx) * oh * 4, st));
    TVGB_TRY(pass(din.get<float>(), t1.get<float>(), int(in_sx), int(in_sy), 1, 1, kh, sigma2, st));
    TVGB_TRY(pass(t1.get<float>(), dout.get<float>(), int(in_sx), int(oh), 1, 0, kw, sigma1, st));
    TVGB_TRY(dout.finish());
    return sync_if(din.owned || dout.owned, st);
}

int tvgb_pipeline3(const float* volume, unsigned s0, unsigned s1, unsigned s2, float sigma_st, int st_mode,
                   const tvgb_vote3_params* p, float* out, int out_layout, float* evals3, float* evecs, int evec_format,
                   unsigned* out_dims, void* stream) {
    TVGB_CHECK_ARG(volume && p, "tvgb_pipeline3: NULL pointer");
    TVGB_CHECK_ARG(sigma_st > 0.0f, "tvgb_pipeline3: sigma_st must be > 0");
    TVGB_CHECK_ARG(st_mode == 0 || st_mode == 1, "tvgb_pipeline3: st_mode must be 0 or 1");
    TVGB_CHECK_ARG(out_layout == TVGB_LAYOUT_MAT3 || out_layout == TVGB_LAYOUT_SYM6 || out_layout == TVGB_LAYOUT_SYM6_PLANES,
                   "tvgb_pipeline3: out_layout must be 9, 6 or 60");
    TVGB_CHECK_ARG(evec_format >= 0 && evec_format <= 2, "tvgb_pipeline3: evec_format must be 0, 1 or 2");
    unsigned d[3];
    structure_tensor3_dims(s0, s1, s2, sigma_st, st_mode, d);
    TVGB_CHECK_ARG(st_mode == 1 || (s0 >= ksize3(sigma_st) && s1 >= ksize3(sigma_st) && s2 >= ksize3(sigma_st)),
                   "tvgb_pipeline3: volume smaller than the structure-tensor window (valid mode)");
    if (out_dims) { out_dims[0] = d[0]; out_dims[1] = d[1]; out_dims[2] = d[2]; }
    const size_t n = size_t(s0) * s1 * s2, no = size_t(d[0]) * d[1] * d[2];
    if (no == 0) return TVGB_OK;
    cudaStream_t st = as_stream(stream);
    const size_t nout = out_layout == TVGB_LAYOUT_MAT3 ? 9 : 6;
    const size_t nv = evec_format == 1 ? 9 : (evec_format == 2 ? 6 : 0);
    DevArray din, dout, dev_, dvec;
    TVGB_TRY(din.in(volume, n * 4, st));
    TVGB_TRY(dout.out(out, no * nout * 4, st));
    TVGB_TRY(dev_.out(evals3, no * 12, st));
    TVGB_TRY(dvec.out(nv ? evecs : nullptr, no * nv * 4, st));
    Scratch tensor;
    TVGB_TRY(tensor.alloc(no * 24, st));
    TVGB_TRY(structure_tensor3_device(din.get<float>(), s0, s1, s2, sigma_st, st_mode, tensor.get<float>(),
                                      TVGB_LAYOUT_SYM6_PLANES, nullptr, st));
    const bool host_out = dout.owned || dev_.owned || dvec.owned;
    if (!host_out || no < (size_t(1) << 22)) {
        TVGB_TRY(vote3_device(tensor.get<float>(), TVGB_LAYOUT_SYM6_PLANES, d[0], d[1], d[2], *p, dout.get<float>(),
                              out_layout, dev_.get<float>(), dvec.get<float>(), nv ? evec_format : 0, st));
        TVGB_TRY(dout.finish());
        TVGB_TRY(dev_.finish());
        TVGB_TRY(dvec.finish());
        return sync_if(din.owned || host_out, st);
    }
    // host outputs of a large volume: z-slabs, copies overlapped with the vote
    HostOut outs[3];
    int no_ = 0;
    if (dout.owned) outs[no_++] = {out, dout.get<float>(), nout, out_layout == TVGB_LAYOUT_SYM6_PLANES};
    if (dev_.owned) outs[no_++] = {evals3, dev_.get<float>(), 3, false};
    if (dvec.owned) outs[no_++] = {evecs, dvec.get<float>(), nv, false};
    TVGB_TRY(vote3_to_host(tensor.get<float>(), TVGB_LAYOUT_SYM6_PLANES, d[0], d[1], d[2], *p, dout.get<float>(),
                           out_layout, dev_.get<float>(), dvec.get<float>(), nv ? evec_format : 0, outs, no_, st));
    return TVGB_OK;
}

}  // extern "C"
