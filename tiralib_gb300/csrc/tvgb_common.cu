// Host-side support of libtvgb: error state, pointer classification and
// stream-ordered device temporaries.
#include "tvgb_common.cuh"
#include "tma_sm100.cuh"
#include <cudaTypedefs.h>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace tvgb {

static thread_local char g_last_error[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

std::atomic<unsigned long long>& launch_counter() {
    static std::atomic<unsigned long long> c{0};
    return c;
}

namespace {
std::atomic<int> g_prof_on{0};
std::mutex g_prof_mu;
struct Pending { const char* name; cudaEvent_t a, b; };
std::vector<Pending>& pending() { static std::vector<Pending> v; return v; }
}  // namespace

KernelTimer::KernelTimer(const char* n, cudaStream_t s) : name(n), stream(s) {
    if (!g_prof_on.load(std::memory_order_relaxed)) return;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) { a = b = nullptr; return; }
    cudaEventRecord(a, s);
}

void KernelTimer::stop() {
    if (!a) return;
    cudaEventRecord(b, stream);
    std::lock_guard<std::mutex> g(g_prof_mu);
    pending().push_back({name, a, b});
    a = b = nullptr;
}

bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();  // unregistered host memory on old runtimes
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// The library's stream-ordered allocations come from its own memory pool,
// one per device, which keeps freed memory for the next call (release
// threshold at the maximum).  The device's default pool returns freed memory
// to the driver at every synchronisation, and mapping it again cost ~20 ms per
// call of the 3D pipeline on host arrays.  tvgb_release_cached_memory trims
// the pools.
constexpr int kMaxPoolDevices = 64;
static std::mutex g_pool_mu;
static cudaMemPool_t g_pools[kMaxPoolDevices];

static int device_pool(cudaMemPool_t& pool) {
    int dev = 0;
    TVGB_CUDA(cudaGetDevice(&dev));
    TVGB_CHECK_ARG(dev >= 0 && dev < kMaxPoolDevices, "device %d beyond the library's pool table", dev);
    std::lock_guard<std::mutex> g(g_pool_mu);
    if (!g_pools[dev]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        TVGB_CUDA(cudaMemPoolCreate(&p, &props));
        unsigned long long keep = ~0ull;   // the attribute is a 64-bit value
        const cudaError_t e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        if (e != cudaSuccess) {
            cudaMemPoolDestroy(p);
            set_error("cudaMemPoolSetAttribute failed: %s", cudaGetErrorString(e));
            return TVGB_ERR_CUDA;
        }
        g_pools[dev] = p;
    }
    pool = g_pools[dev];
    return TVGB_OK;
}

static int pool_alloc(void** ptr, size_t bytes, cudaStream_t s) {
    cudaMemPool_t pool;
    TVGB_TRY(device_pool(pool));
    TVGB_CUDA(cudaMallocFromPoolAsync(ptr, bytes, pool, s));
    return TVGB_OK;
}

int DevArray::in(const void* p, size_t nbytes, cudaStream_t s) {
    user = const_cast<void*>(p);
    bytes = nbytes;
    stream = s;
    output = false;
    if (!p || nbytes == 0) return TVGB_OK;
    if (is_device_ptr(p)) {
        dev = user;
        return TVGB_OK;
    }
    TVGB_TRY(pool_alloc(&dev, nbytes, s));
    owned = true;
    scratch_track((long long)nbytes);
    KernelTimer kt_("copy_h2d", s);   // the profile times staging copies beside the kernels
    TVGB_CUDA(cudaMemcpyAsync(dev, p, nbytes, cudaMemcpyHostToDevice, s));
    kt_.stop();
    return TVGB_OK;
}

int DevArray::out(void* p, size_t nbytes, cudaStream_t s, bool zero) {
    user = p;
    bytes = nbytes;
    stream = s;
    output = true;
    if (!p || nbytes == 0) return TVGB_OK;
    if (is_device_ptr(p)) {
        dev = p;
    } else {
        TVGB_TRY(pool_alloc(&dev, nbytes, s));
        owned = true;
        scratch_track((long long)nbytes);
    }
    if (zero) TVGB_CUDA(cudaMemsetAsync(dev, 0, nbytes, s));
    return TVGB_OK;
}

int DevArray::finish() {
    if (output && owned && dev && user) {
        KernelTimer kt_("copy_d2h", stream);
        TVGB_CUDA(cudaMemcpyAsync(user, dev, bytes, cudaMemcpyDeviceToHost, stream));
        kt_.stop();
    }
    return TVGB_OK;
}

int Scratch::alloc(size_t bytes, cudaStream_t s) {
    stream = s;
    if (bytes == 0) return TVGB_OK;
    TVGB_TRY(pool_alloc(&p, bytes, s));
    this->bytes = bytes;
    scratch_track((long long)bytes);
    return TVGB_OK;
}

static std::atomic<long long> g_scratch_cur{0}, g_scratch_peak{0};

void scratch_track(long long delta) {
    const long long now = g_scratch_cur.fetch_add(delta) + delta;
    long long pk = g_scratch_peak.load();
    while (now > pk && !g_scratch_peak.compare_exchange_weak(pk, now)) {
    }
}

// FP32 FMA throughput: every thread runs 8 independent chains of packed
// FP32x2 fused multiply-adds (16 FMAs per iteration).  Each CTA records its
// SM-clock cycles and its global-timer nanoseconds, so the host learns the SM
// clock the kernel ran at.
__global__ void __launch_bounds__(256) k_fp32_peak(int iters, float* __restrict__ sink,
                                                   unsigned long long* __restrict__ clk) {
    float2 a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = make_float2(1e-3f * float(threadIdx.x + i), 2e-3f * float(i));
    const float2 m = make_float2(0.9999f, 0.9998f), c = make_float2(1e-6f, 2e-6f);
    unsigned long long t0, t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    const long long c0 = clock64();
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = __ffma2_rn(a[i], m, c);
    }
    const long long c1 = clock64();
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i].x + a[i].y;
    if (s == 1234.5f) sink[0] = s;   // keeps the chains alive
    if (threadIdx.x == 0) {
        atomicAdd(clk, (unsigned long long)(c1 - c0));
        atomicAdd(clk + 1, t1 - t0);
    }
}

// MUFU throughput: 8 independent chains of tanh.approx per thread, FP32
// (MODE 0) or packed BF16 pairs (MODE 1).
template <int MODE>
__global__ void __launch_bounds__(256) k_tanh_rate(int iters, float* __restrict__ sink) {
    float a[8];
    uint32_t b[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        a[i] = 1e-3f * float(threadIdx.x + i);
        b[i] = 0x3C003C00u + uint32_t(i);
    }
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            if (MODE == 0) asm volatile("tanh.approx.f32 %0, %0;" : "+f"(a[i]));
            else asm volatile("tanh.approx.bf16x2 %0, %0;" : "+r"(b[i]));
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i] + __uint_as_float(b[i]);
    if (s == 1234.5f) sink[0] = s;
}

// ------------------------------------------------------------------ TMA tensor maps
// cuTensorMapEncodeTiled is a driver API function; the library links only the
// runtime, so its address is looked up once through the runtime.
bool make_tmap_3d_f32(CUtensorMap* map, const float* base, unsigned s2, unsigned s1, unsigned s0, unsigned bx,
                      unsigned by) {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    std::call_once(once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        else
            cudaGetLastError();
    });
    if (!encode) return false;
    if (reinterpret_cast<uintptr_t>(base) % 16 != 0 || (size_t(s2) * 4) % 16 != 0 || (bx * 4) % 16 != 0) return false;
    const cuuint64_t dims[3] = {s2, s1, s0};
    const cuuint64_t strides[2] = {cuuint64_t(s2) * 4, cuuint64_t(s2) * s1 * 4};
    const cuuint32_t box[3] = {bx, by, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUtensorMap m;
    const CUresult r = encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    *map = m;
    return true;
}

}  // namespace tvgb

extern "C" {

int tvgb_pipe_rates(double* rates, void* stream) {
    using namespace tvgb;
    TVGB_CHECK_ARG(rates, "tvgb_pipe_rates: rates is NULL");
    double tf = 0.0, mhz = 0.0;
    TVGB_TRY(tvgb_fp32_peak(&tf, &mhz, stream));
    TVGB_CHECK_ARG(mhz > 0.0, "tvgb_pipe_rates: the SM clock could not be measured");
    cudaStream_t st = as_stream(stream);
    int dev = 0, sms = 0;
    TVGB_CUDA(cudaGetDevice(&dev));
    TVGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int ctas = sms * 8, iters = 1 << 13;
    Scratch scr;
    TVGB_TRY(scr.alloc(16, st));
    cudaEvent_t e0, e1;
    TVGB_CUDA(cudaEventCreate(&e0));
    TVGB_CUDA(cudaEventCreate(&e1));
    rates[0] = tf * 1e12 / 2.0 / (double(sms) * mhz * 1e6);   // FP32 FMAs per SM clock
    for (int mode = 0; mode < 2; ++mode) {
        auto launch = [&](int n) {
            if (mode == 0) k_tanh_rate<0><<<ctas, 256, 0, st>>>(n, scr.get<float>());
            else k_tanh_rate<1><<<ctas, 256, 0, st>>>(n, scr.get<float>());
        };
        launch(iters / 8);   // warm-up
        TVGB_CUDA(cudaEventRecord(e0, st));
        launch(iters);
        TVGB_CUDA(cudaEventRecord(e1, st));
        TVGB_LAUNCHED();
        TVGB_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        TVGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        const double results = double(ctas) * 256.0 * iters * 8.0 * (mode == 1 ? 2.0 : 1.0);
        rates[1 + mode] = results / (double(ms) * 1e-3) / (double(sms) * mhz * 1e6);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    rates[3] = mhz;
    return TVGB_OK;
}

int tvgb_fp32_peak(double* tflops, double* sm_mhz, void* stream) {
    using namespace tvgb;
    TVGB_CHECK_ARG(tflops, "tvgb_fp32_peak: tflops is NULL");
    cudaStream_t st = as_stream(stream);
    int dev = 0, sms = 0;
    TVGB_CUDA(cudaGetDevice(&dev));
    TVGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int ctas = sms * 8, iters = 1 << 18;
    Scratch scr;
    TVGB_TRY(scr.alloc(64, st));
    unsigned long long* clk = scr.get<unsigned long long>();
    cudaEvent_t e0, e1;
    TVGB_CUDA(cudaEventCreate(&e0));
    TVGB_CUDA(cudaEventCreate(&e1));
    k_fp32_peak<<<ctas, 256, 0, st>>>(iters / 8, reinterpret_cast<float*>(clk + 2), clk);   // warm-up
    TVGB_CUDA(cudaMemsetAsync(clk, 0, 16, st));
    TVGB_CUDA(cudaEventRecord(e0, st));
    k_fp32_peak<<<ctas, 256, 0, st>>>(iters, reinterpret_cast<float*>(clk + 2), clk);
    TVGB_CUDA(cudaEventRecord(e1, st));
    TVGB_LAUNCHED();
    unsigned long long h[2] = {0, 0};
    TVGB_CUDA(cudaMemcpyAsync(h, clk, 16, cudaMemcpyDeviceToHost, st));
    TVGB_CUDA(cudaStreamSynchronize(st));
    float ms = 0.0f;
    TVGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * 16.0 * double(iters) * double(ctas) * 256.0;
    *tflops = flops / (double(ms) * 1e-3) / 1e12;
    if (sm_mhz) *sm_mhz = h[1] ? 1e3 * double(h[0]) / double(h[1]) : 0.0;
    return TVGB_OK;
}

const char* tvgb_last_error(void) { return tvgb::g_last_error; }
int tvgb_version(void) { return 100; }
unsigned long long tvgb_launch_count(void) { return tvgb::launch_counter().load(); }

int tvgb_memory_stats(unsigned long long* scratch_bytes, unsigned long long* scratch_peak_bytes, int reset_peak) {
    const long long cur = tvgb::g_scratch_cur.load();
    if (scratch_bytes) *scratch_bytes = (unsigned long long)(cur > 0 ? cur : 0);
    if (scratch_peak_bytes) *scratch_peak_bytes = (unsigned long long)tvgb::g_scratch_peak.load();
    if (reset_peak) tvgb::g_scratch_peak.store(cur > 0 ? cur : 0);
    return TVGB_OK;
}

int tvgb_release_cached_memory(void) {
    std::lock_guard<std::mutex> g(tvgb::g_pool_mu);
    for (int d = 0; d < tvgb::kMaxPoolDevices; ++d)
        if (tvgb::g_pools[d] && cudaMemPoolTrimTo(tvgb::g_pools[d], 0) != cudaSuccess) {
            tvgb::set_error("cudaMemPoolTrimTo failed on device %d", d);
            return TVGB_ERR_CUDA;
        }
    return TVGB_OK;
}

int tvgb_profile_enable(int on) {
    tvgb::g_prof_on.store(on ? 1 : 0);
    return TVGB_OK;
}

// Resolves every recorded launch (synchronising on its events) and writes
// "name count total_ms\n" lines, one per kernel, into buf; resets the record.
int tvgb_profile_read(char* buf, size_t buflen) {
    std::vector<tvgb::Pending> v;
    {
        std::lock_guard<std::mutex> g(tvgb::g_prof_mu);
        v.swap(tvgb::pending());
    }
    std::map<std::string, std::pair<long, double>> agg;
    int status = TVGB_OK;
    for (auto& r : v) {
        float ms = 0.0f;
        if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) {
            tvgb::set_error("tvgb_profile_read: event timing failed");
            status = TVGB_ERR_CUDA;
        }
        auto& e = agg[r.name];
        e.first += 1;
        e.second += ms;
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    std::string out;
    char line[256];
    for (auto& kv : agg) {
        snprintf(line, sizeof line, "%s %ld %.6f\n", kv.first.c_str(), kv.second.first, kv.second.second);
        out += line;
    }
    if (buf && buflen) {
        strncpy(buf, out.c_str(), buflen - 1);
        buf[buflen - 1] = 0;
    }
    return status;
}

}  // extern "C"
