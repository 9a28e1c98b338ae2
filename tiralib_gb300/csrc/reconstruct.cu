// Consumers of a voted 2D field on sm_103a: stick saliency, Otsu's
// threshold, saliency thresholding with optional closing + hole filling, and
// the scale-invariant mean Frobenius distance (SIMF) used as the objective
// of tiralib's parameter sweeps.
//
// Reference (python/tira/tensors_lib):
//   reconstruct.py:14  stick_saliency      |lambda|max - |lambda|min per pixel
//   reconstruct.py:34  _otsu_threshold     256-bin histogram over [0, max], between-class variance
//   reconstruct.py:66  saliency_threshold  s > thr, optionally binary_closing + binary_fill_holes
//   metrics.py:37      simf                mean || A - alpha B ||_F, alpha = <A,B> / <B,B>
// Fields are (H, W) pixels of [a, b, b, c] (float4), as the 2D vote writes them.
#include "tvgb_internal.cuh"
#include <cmath>

namespace tvgb {

// |lambda|max - |lambda|min of [[a, b], [b, c]]: with d = lambda+ - lambda- =
// 2 hypot((a - c)/2, b) >= 0 and t = lambda+ + lambda- = a + c, it is d when
// both eigenvalues share a sign and |t| otherwise, i.e. min(d, |t|).
__device__ __forceinline__ float saliency2(float4 m) {
    const float d = 2.0f * hypotf(0.5f * (m.x - m.w), m.y);
    return fminf(d, fabsf(m.x + m.w));
}

__global__ void k_saliency2(const float4* __restrict__ in, size_t n, float* __restrict__ sal,
                            unsigned* __restrict__ vmax_bits) {
    float mx = 0.0f;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const float s = saliency2(__ldg(in + i));
        if (sal) sal[i] = s;
        mx = fmaxf(mx, s);
    }
    if (vmax_bits) {
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if ((threadIdx.x & 31) == 0) atomicMax(vmax_bits, __float_as_uint(mx));   // s >= 0: bits order as values
    }
}

__global__ void k_vmax(const float* __restrict__ v, size_t n, unsigned* __restrict__ vmax_bits) {
    float mx = 0.0f;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        mx = fmaxf(mx, v[i]);
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(vmax_bits, __float_as_uint(mx));
}

// np.histogram(values, bins=256, range=(0, vmax)) bin of v for float32
// values: NumPy builds the edges in the values' type, float32 here
// (linspace(0, vmax, 257): i * (vmax / 256) rounded to float, the last edge
// vmax), takes int(v / vmax * 256) in FP64 as the first guess and corrects
// it against the float32 edges.
__device__ __forceinline__ float hist_edge(int i, double vmax) {
    return i >= 256 ? float(vmax) : float(double(i) * (vmax / 256.0));
}
__device__ __forceinline__ int hist_bin(float v, double vmax) {
    int i = int((double(v) / vmax) * 256.0);
    if (i >= 256) i = 255;
    if (i < 0) i = 0;
    if (v < hist_edge(i, vmax)) --i;
    else if (i != 255 && v >= hist_edge(i + 1, vmax)) ++i;
    return i;
}

__global__ void k_hist256(const float* __restrict__ v, size_t n, const unsigned* __restrict__ vmax_bits,
                          unsigned long long* __restrict__ hist) {
    __shared__ unsigned h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const double vmax = double(__uint_as_float(*vmax_bits));
    if (vmax > 0.0) {
        for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
            const float x = v[i];
            if (x >= 0.0f && double(x) <= vmax) atomicAdd(&h[hist_bin(x, vmax)], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        if (h[i]) atomicAdd(hist + i, (unsigned long long)h[i]);
}

// Otsu on the histogram, one thread (reconstruct.py:44-63): bin centres are
// float32 like the edges, the class weights and means FP64, the first
// maximum of the between-class variance wins.
__global__ void k_otsu(const unsigned long long* __restrict__ hist, const unsigned* __restrict__ vmax_bits,
                       double* __restrict__ thr) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double vmax = double(__uint_as_float(*vmax_bits));
    if (!(vmax > 0.0)) { *thr = 0.0; return; }
    double total = 0.0;
    for (int i = 0; i < 256; ++i) total += double(hist[i]);
    if (total == 0.0) { *thr = 0.0; return; }
    auto centre = [&](int i) { return (hist_edge(i, vmax) + hist_edge(i + 1, vmax)) / 2.0f; };
    double cum_all = 0.0;
    for (int i = 0; i < 256; ++i) cum_all += double(hist[i]) * double(centre(i));
    double w0 = 0.0, cum = 0.0, best = -1.0, best_c = 0.0;
    for (int i = 0; i < 256; ++i) {
        const double c = double(centre(i));
        w0 += double(hist[i]);
        cum += double(hist[i]) * c;
        const double w1 = total - w0;
        const double mu0 = w0 > 0.0 ? cum / w0 : 0.0;
        const double mu1 = w1 > 0.0 ? (cum_all - cum) / w1 : 0.0;
        const double dm = mu0 - mu1;
        const double b = (w0 * w1) * (dm * dm);
        if (b > best) { best = b; best_c = c; }
    }
    *thr = best_c;
}

// s > thr with the threshold in FP64, as NumPy compares a float32 map with a Python float
__global__ void k_threshold(const float* __restrict__ s, size_t n, const double* __restrict__ thr,
                            unsigned char* __restrict__ mask) {
    const double t = *thr;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        mask[i] = double(s[i]) > t ? 1 : 0;
}

// square (2 r + 1) structuring element, one axis at a time; pixels outside
// the image count as 0 (scipy's border_value = 0): dilation ORs, erosion ANDs
template <bool DILATE, bool ALONG_X>
__global__ void k_morph(const unsigned char* __restrict__ in, unsigned char* __restrict__ out, int H, int W, int r) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    unsigned char acc = DILATE ? 0 : 1;
    for (int k = -r; k <= r; ++k) {
        const int xx = ALONG_X ? x + k : x, yy = ALONG_X ? y : y + k;
        const unsigned char v = (xx >= 0 && xx < W && yy >= 0 && yy < H) ? in[size_t(yy) * W + xx] : 0;
        if (DILATE) acc |= v; else acc &= v;
    }
    out[size_t(y) * W + x] = acc;
}

// Hole filling: background reachable from the border through 4-connected
// background stays background; the rest becomes foreground.  Each launch
// propagates `reach` inside 32 x 32 tiles (plus the one-pixel halo read from
// the previous state) until the tile settles, and reports whether anything
// changed; the host repeats launches until nothing does.
constexpr int FT = 32;
__global__ void k_fill_reach(const unsigned char* __restrict__ fg, unsigned char* __restrict__ reach, int H, int W,
                             int* __restrict__ changed) {
    __shared__ unsigned char r[FT + 2][FT + 2];
    __shared__ unsigned char b[FT + 2][FT + 2];
    __shared__ int tile_changed, any;
    const int tx = threadIdx.x, ty = threadIdx.y;        // 32 x 8 threads, 4 rows each
    const int x0 = blockIdx.x * FT, y0 = blockIdx.y * FT;
    for (int e = ty * FT + tx; e < (FT + 2) * (FT + 2); e += FT * 8) {
        const int ly = e / (FT + 2), lx = e - ly * (FT + 2);
        const int gx = x0 + lx - 1, gy = y0 + ly - 1;
        const bool in = gx >= 0 && gx < W && gy >= 0 && gy < H;
        // outside the image: reached background (the dilation's border_value = 1)
        r[ly][lx] = in ? reach[size_t(gy) * W + gx] : 1;
        b[ly][lx] = in ? (fg[size_t(gy) * W + gx] ? 0 : 1) : 1;
    }
    if (tx == 0 && ty == 0) any = 0;
    __syncthreads();
    for (int it = 0; it < FT * FT; ++it) {
        if (tx == 0 && ty == 0) tile_changed = 0;
        __syncthreads();
        for (int k = 0; k < 4; ++k) {
            const int ly = ty * 4 + k + 1, lx = tx + 1;
            if (y0 + ly - 1 < H && x0 + lx - 1 < W && b[ly][lx] && !r[ly][lx] &&
                (r[ly - 1][lx] | r[ly + 1][lx] | r[ly][lx - 1] | r[ly][lx + 1])) {
                r[ly][lx] = 1;
                tile_changed = 1;
            }
        }
        __syncthreads();
        const int c = tile_changed;
        if (c && tx == 0 && ty == 0) any = 1;
        __syncthreads();
        if (!c) break;
    }
    for (int k = 0; k < 4; ++k) {
        const int ly = ty * 4 + k + 1, lx = tx + 1;
        const int gx = x0 + lx - 1, gy = y0 + ly - 1;
        if (gx < W && gy < H) reach[size_t(gy) * W + gx] = r[ly][lx];
    }
    if (tx == 0 && ty == 0 && any) atomicOr(changed, 1);
}

__global__ void k_fill_finish(const unsigned char* __restrict__ reach, size_t n, unsigned char* __restrict__ mask) {
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        mask[i] = reach[i] ? 0 : 1;
}

// SIMF passes: <A,B>, <B,B> (pass 1) and sum_p || A_p - alpha B_p ||_F (pass 2), FP64 accumulation
__device__ __forceinline__ void block_add(double v, double* dst) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(dst, v);
}

__global__ void k_simf_dots(const float4* __restrict__ A, const float4* __restrict__ B, size_t n, double* acc) {
    double ab = 0.0, bb = 0.0;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const float4 a = __ldg(A + i), b = __ldg(B + i);
        ab += double(a.x) * b.x + double(a.y) * b.y + double(a.z) * b.z + double(a.w) * b.w;
        bb += double(b.x) * b.x + double(b.y) * b.y + double(b.z) * b.z + double(b.w) * b.w;
    }
    block_add(ab, acc);
    block_add(bb, acc + 1);
}

__global__ void k_simf_norms(const float4* __restrict__ A, const float4* __restrict__ B, size_t n,
                             const double* __restrict__ dots, double* __restrict__ acc) {
    const double alpha = dots[1] < 1e-8 ? 0.0 : dots[0] / dots[1];   // metrics.py:137-146
    const float al = float(alpha);
    double s = 0.0;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const float4 a = __ldg(A + i), b = __ldg(B + i);
        const float d0 = fmaf(-al, b.x, a.x), d1 = fmaf(-al, b.y, a.y), d2 = fmaf(-al, b.z, a.z),
                    d3 = fmaf(-al, b.w, a.w);
        s += sqrt(double(d0) * d0 + double(d1) * d1 + double(d2) * d2 + double(d3) * d3);
    }
    block_add(s, acc);
}

static unsigned grid1(size_t n) {
    size_t b = (n + 255) / 256;
    if (b > 152 * 8) b = 152 * 8;
    return unsigned(b ? b : 1);
}

int simf2_device(const float4* A, const float4* B, size_t n, double* dev_acc3, cudaStream_t st) {
    TVGB_CUDA(cudaMemsetAsync(dev_acc3, 0, 3 * sizeof(double), st));
    k_simf_dots<<<grid1(n), 256, 0, st>>>(A, B, n, dev_acc3);
    TVGB_LAUNCHED();
    k_simf_norms<<<grid1(n), 256, 0, st>>>(A, B, n, dev_acc3, dev_acc3 + 2);
    TVGB_LAUNCHED();
    return TVGB_OK;
}

}  // namespace tvgb

using namespace tvgb;

extern "C" {

int tvgb_stick_saliency2(const float* field, size_t n, float* saliency, void* stream) {
    TVGB_CHECK_ARG(field && saliency, "tvgb_stick_saliency2: NULL pointer");
    if (n == 0) return TVGB_OK;
    cudaStream_t st = as_stream(stream);
    DevArray din, dout;
    TVGB_TRY(din.in(field, n * 16, st));
    TVGB_TRY(dout.out(saliency, n * 4, st));
    TVGB_CHECK_ARG(reinterpret_cast<uintptr_t>(din.dev) % 16 == 0, "tvgb_stick_saliency2: field must be 16-byte aligned");
    {
        KernelTimer kt_("k_saliency2", st);
        k_saliency2<<<grid1(n), 256, 0, st>>>(din.get<float4>(), n, dout.get<float>(), nullptr);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    TVGB_TRY(dout.finish());
    return sync_if(din.owned || dout.owned, st);
}

static int otsu_device(const float* v, size_t n, unsigned* vmax_bits, bool have_max, unsigned long long* hist,
                       double* thr, cudaStream_t st) {
    if (!have_max) {
        TVGB_CUDA(cudaMemsetAsync(vmax_bits, 0, sizeof(unsigned), st));
        k_vmax<<<grid1(n), 256, 0, st>>>(v, n, vmax_bits);
        TVGB_LAUNCHED();
    }
    TVGB_CUDA(cudaMemsetAsync(hist, 0, 256 * sizeof(unsigned long long), st));
    {
        KernelTimer kt_("k_hist256", st);
        k_hist256<<<grid1(n), 256, 0, st>>>(v, n, vmax_bits, hist);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    k_otsu<<<1, 32, 0, st>>>(hist, vmax_bits, thr);
    TVGB_LAUNCHED();
    return TVGB_OK;
}

int tvgb_otsu_threshold(const float* values, size_t n, double* threshold, void* stream) {
    TVGB_CHECK_ARG(values && threshold, "tvgb_otsu_threshold: NULL pointer");
    cudaStream_t st = as_stream(stream);
    if (n == 0) { *threshold = 0.0; return TVGB_OK; }
    DevArray din;
    TVGB_TRY(din.in(values, n * 4, st));
    Scratch sc;
    TVGB_TRY(sc.alloc(256 * 8 + 16 + 8, st));
    unsigned long long* hist = sc.get<unsigned long long>();
    double* thr = reinterpret_cast<double*>(hist + 256);
    unsigned* vmax = reinterpret_cast<unsigned*>(thr + 1);
    TVGB_TRY(otsu_device(din.get<float>(), n, vmax, false, hist, thr, st));
    TVGB_CUDA(cudaMemcpyAsync(threshold, thr, sizeof(double), cudaMemcpyDeviceToHost, st));
    TVGB_CUDA(cudaStreamSynchronize(st));
    return TVGB_OK;
}

int tvgb_saliency_threshold2(const float* field, unsigned s0, unsigned s1, int fill, int use_otsu, double threshold,
                             int close_radius, unsigned char* mask, double* threshold_used, void* stream) {
    TVGB_CHECK_ARG(field && mask, "tvgb_saliency_threshold2: NULL pointer");
    TVGB_CHECK_ARG(close_radius >= 0 && close_radius <= 4096, "tvgb_saliency_threshold2: bad close_radius %d",
                   close_radius);
    const size_t n = size_t(s0) * s1;
    if (n == 0) return TVGB_OK;
    cudaStream_t st = as_stream(stream);
    DevArray din, dmask;
    TVGB_TRY(din.in(field, n * 16, st));
    TVGB_TRY(dmask.out(mask, n, st));
    TVGB_CHECK_ARG(reinterpret_cast<uintptr_t>(din.dev) % 16 == 0,
                   "tvgb_saliency_threshold2: field must be 16-byte aligned");
    Scratch sc;
    TVGB_TRY(sc.alloc(n * 4 + 2 * n + 256 * 8 + 64, st));
    unsigned long long* hist = sc.get<unsigned long long>();
    double* thr = reinterpret_cast<double*>(hist + 256);
    unsigned* vmax = reinterpret_cast<unsigned*>(thr + 1);
    int* changed = reinterpret_cast<int*>(vmax + 1);
    float* sal = reinterpret_cast<float*>(reinterpret_cast<char*>(hist) + 256 * 8 + 64);
    unsigned char* b0 = reinterpret_cast<unsigned char*>(sal + n);
    unsigned char* b1 = b0 + n;
    TVGB_CUDA(cudaMemsetAsync(vmax, 0, sizeof(unsigned), st));
    {
        KernelTimer kt_("k_saliency2", st);
        k_saliency2<<<grid1(n), 256, 0, st>>>(din.get<float4>(), n, sal, vmax);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    if (use_otsu) {
        TVGB_TRY(otsu_device(sal, n, vmax, true, hist, thr, st));
    } else {
        TVGB_CUDA(cudaMemcpyAsync(thr, &threshold, sizeof(double), cudaMemcpyHostToDevice, st));
    }
    unsigned char* out = dmask.get<unsigned char>();
    k_threshold<<<grid1(n), 256, 0, st>>>(sal, n, thr, fill ? b0 : out);
    TVGB_LAUNCHED();
    if (fill) {
        const int H = int(s0), W = int(s1);
        dim3 blk(32, 8), g(ceil_div(s1, 32u), ceil_div(s0, 8u));
        unsigned char* cur = b0;
        if (close_radius > 0) {   // binary_closing: dilation then erosion, border value 0
            k_morph<true, true><<<g, blk, 0, st>>>(b0, b1, H, W, close_radius);
            k_morph<true, false><<<g, blk, 0, st>>>(b1, out, H, W, close_radius);
            k_morph<false, true><<<g, blk, 0, st>>>(out, b1, H, W, close_radius);
            k_morph<false, false><<<g, blk, 0, st>>>(b1, b0, H, W, close_radius);
            for (int i = 0; i < 4; ++i) TVGB_LAUNCHED();
        }
        // binary_fill_holes: reach from the border through 4-connected background
        unsigned char* reach = b1;
        TVGB_CUDA(cudaMemsetAsync(reach, 0, n, st));
        dim3 gf(ceil_div(s1, unsigned(FT)), ceil_div(s0, unsigned(FT))), bf(32, 8);
        for (size_t round = 0; round <= n; ++round) {   // each round adds a pixel or ends it
            int h_changed = 0;
            TVGB_CUDA(cudaMemsetAsync(changed, 0, sizeof(int), st));
            k_fill_reach<<<gf, bf, 0, st>>>(cur, reach, H, W, changed);
            TVGB_LAUNCHED();
            TVGB_CUDA(cudaMemcpyAsync(&h_changed, changed, sizeof(int), cudaMemcpyDeviceToHost, st));
            TVGB_CUDA(cudaStreamSynchronize(st));
            if (!h_changed) break;
        }
        k_fill_finish<<<grid1(n), 256, 0, st>>>(reach, n, out);
        TVGB_LAUNCHED();
    }
    if (threshold_used) {
        TVGB_CUDA(cudaMemcpyAsync(threshold_used, thr, sizeof(double), cudaMemcpyDeviceToHost, st));
        TVGB_CUDA(cudaStreamSynchronize(st));
    }
    TVGB_TRY(dmask.finish());
    return sync_if(din.owned || dmask.owned, st);
}

int tvgb_simf2(const float* A, const float* B, size_t n, double* simf, void* stream) {
    TVGB_CHECK_ARG(A && B && simf, "tvgb_simf2: NULL pointer");
    if (n == 0) { *simf = 0.0; return TVGB_OK; }
    cudaStream_t st = as_stream(stream);
    DevArray da, db;
    TVGB_TRY(da.in(A, n * 16, st));
    TVGB_TRY(db.in(B, n * 16, st));
    TVGB_CHECK_ARG(reinterpret_cast<uintptr_t>(da.dev) % 16 == 0 && reinterpret_cast<uintptr_t>(db.dev) % 16 == 0,
                   "tvgb_simf2: fields must be 16-byte aligned");
    Scratch sc;
    TVGB_TRY(sc.alloc(3 * sizeof(double), st));
    TVGB_TRY(simf2_device(da.get<float4>(), db.get<float4>(), n, sc.get<double>(), st));
    double h[3];
    TVGB_CUDA(cudaMemcpyAsync(h, sc.get<double>(), sizeof(h), cudaMemcpyDeviceToHost, st));
    TVGB_CUDA(cudaStreamSynchronize(st));
    *simf = h[2] / double(n);
    return TVGB_OK;
}

}  // extern "C"
