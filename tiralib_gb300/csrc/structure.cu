// Structure tensor and separable Gaussian filters.
//
// Reference path replaced: the caller computes volume<T>::gradient per axis
// (tira/volume.h:974, a host triple loop), forms the outer product itself,
// and blurs each of the six components with tira::cuda::gaussian_filter3d
// (tira/functions/filter.h:401): three launches per component (z, y, x
// passes, cuda_convolve3z/3y/3x :275,259,243) with the kernel in global
// memory, intermediates in HBM and a device synchronise after each pass.
//
// Here one kernel does it all: a CTA owns a 32 x 8 output column and marches
// through the input z-planes; per plane it forms the gradient (central
// inside, one-sided at the faces), the six products on the haloed xy region,
// blurs them along x and y in shared memory, and keeps the last K xy-blurred
// planes in a shared-memory ring from which each finished output plane is
// blurred along z and written once.  HBM traffic ~ one read of the volume
// plus one write of the six components (28 B per voxel).
//
// tvgb_gaussian_filter3d / tvgb_gaussian_convolve2 keep the reference's
// scalar, valid-convolution contract (filter.h:401, :305) with a coalesced
// per-axis pass kernel.
#include "tvgb_internal.cuh"
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
};

__device__ __forceinline__ float vol_at(const StArgs& a, int z, int y, int x) {
    return __ldg(a.vol + (size_t(z) * a.s1 + y) * a.s2 + x);
}

// d/d(axis) at an in-volume voxel: volume<T>::gradient's rule
__device__ __forceinline__ float grad1(float lo, float c, float hi, int p, int S) {
    if (S < 2) return 0.0f;
    if (p == 0) return hi - c;
    if (p == S - 1) return c - lo;
    return (hi - lo) * 0.5f;
}

__global__ void __launch_bounds__(STX * STY) k_st3(StArgs a) {
    extern __shared__ __align__(16) float sm[];
    const int K = a.K;
    const int EX = STX + K - 1, EY = STY + K - 1;
    float* sT = sm;                          // 6 x EY x EX products
    float* sX = sT + 6 * EY * EX;            // 6 x EY x STX x-blurred
    float* ring = sX + 6 * EY * STX;         // K x 6 x STY x STX xy-blurred
    __shared__ float g[MAXK];
    const int tid = threadIdx.y * STX + threadIdx.x;
    if (tid < K) g[tid] = a.g[tid];

    const int ox0 = blockIdx.x * STX, oy0 = blockIdx.y * STY;
    const int oz_lo = blockIdx.z * a.zchunk, oz_hi = min(a.o0 - 1, oz_lo + a.zchunk - 1);
    // input z-planes feeding outputs [oz_lo, oz_hi]: iz = oz + c - off, c in [0, K)
    const int iz_lo = oz_lo - a.off, iz_hi = oz_hi + K - 1 - a.off;
    const int ix0 = ox0 - a.off, iy0 = oy0 - a.off;   // input coords of region origin
    const size_t on = size_t(a.o0) * a.o1 * a.o2;

    for (int iz = iz_lo; iz <= iz_hi; ++iz) {
        const bool zin = iz >= 0 && iz < a.s0;
        // (b) products on the haloed region
        for (int e = tid; e < EY * EX; e += STX * STY) {
            const int ry = e / EX, rx = e - ry * EX;
            const int x = ix0 + rx, y = iy0 + ry;
            float gx = 0.0f, gy = 0.0f, gz = 0.0f;
            if (zin && x >= 0 && x < a.s2 && y >= 0 && y < a.s1) {
                const float c = vol_at(a, iz, y, x);
                const float xl = x > 0 ? vol_at(a, iz, y, x - 1) : c, xh = x + 1 < a.s2 ? vol_at(a, iz, y, x + 1) : c;
                const float yl = y > 0 ? vol_at(a, iz, y - 1, x) : c, yh = y + 1 < a.s1 ? vol_at(a, iz, y + 1, x) : c;
                const float zl = iz > 0 ? vol_at(a, iz - 1, y, x) : c, zh = iz + 1 < a.s0 ? vol_at(a, iz + 1, y, x) : c;
                gx = grad1(xl, c, xh, x, a.s2);
                gy = grad1(yl, c, yh, y, a.s1);
                gz = grad1(zl, c, zh, iz, a.s0);
            }
            const int ps = EY * EX;
            sT[e] = gx * gx; sT[ps + e] = gx * gy; sT[2 * ps + e] = gx * gz;
            sT[3 * ps + e] = gy * gy; sT[4 * ps + e] = gy * gz; sT[5 * ps + e] = gz * gz;
        }
        __syncthreads();
        // (c) blur along x: sX[c][ry][tx]
        for (int e = tid; e < 6 * EY * STX; e += STX * STY) {
            const int c = e / (EY * STX), r = e - c * EY * STX, ry = r / STX, tx = r - ry * STX;
            const float* src = sT + c * EY * EX + ry * EX + tx;
            float s = 0.0f;
            for (int k = 0; k < K; ++k) s = fmaf(g[k], src[k], s);
            sX[e] = s;
        }
        __syncthreads();
        // (d) blur along y into the ring slot of this plane
        float* slot = ring + ((iz - iz_lo) % K) * 6 * STY * STX;
        for (int e = tid; e < 6 * STY * STX; e += STX * STY) {
            const int c = e / (STY * STX), r = e - c * STY * STX, ty = r / STX, tx = r - ty * STX;
            const float* src = sX + c * EY * STX + ty * STX + tx;
            float s = 0.0f;
            for (int k = 0; k < K; ++k) s = fmaf(g[k], src[k * STX], s);
            slot[e] = s;
        }
        __syncthreads();
        // (e) output plane oz = iz - (K - 1) + off is complete
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
        // the next plane's step (b) overwrites sT only; the ring slot it later
        // writes is not read by (e) of this iteration after this barrier
        __syncthreads();
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
    const unsigned gx = ceil_div(d[2], STX), gy = ceil_div(d[1], STY);
    // enough CTAs for ~4 waves on 152 SMs, but chunks long enough to amortise the K-1 plane ramp
    int zchunk = int(d[0]);
    const size_t target = 152 * 8;
    while (zchunk > 4 * int(K) && size_t(gx) * gy * ceil_div(d[0], unsigned(zchunk)) < target) zchunk = (zchunk + 1) / 2;
    a.zchunk = zchunk;
    const int EX = STX + int(K) - 1, EY = STY + int(K) - 1;
    const size_t smem = sizeof(float) * (size_t(6) * EY * EX + size_t(6) * EY * STX + size_t(K) * 6 * STY * STX);
    TVGB_CUDA(cudaFuncSetAttribute(k_st3, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    dim3 grid(gx, gy, ceil_div(d[0], unsigned(zchunk)));
    {
        KernelTimer kt_("k_st3", st);
        k_st3<<<grid, dim3(STX, STY), smem, st>>>(a);
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
    TVGB_TRY(vote3_device(tensor.get<float>(), TVGB_LAYOUT_SYM6_PLANES, d[0], d[1], d[2], *p, dout.get<float>(),
                          out_layout, dev_.get<float>(), dvec.get<float>(), nv ? evec_format : 0, st));
    TVGB_TRY(dout.finish());
    TVGB_TRY(dev_.finish());
    TVGB_TRY(dvec.finish());
    return sync_if(din.owned || dout.owned || dev_.owned || dvec.owned, st);
}

}  // extern "C"
