// Shared host/device helpers of libtvgb: status codes and the per-thread
// error message, pointer classification (host vs device, as the reference's
// _is_device, tira/functions/tensorvote.h:1880), stream-ordered device
// buffers and the launch counter.
#pragma once
#include <cuda_runtime.h>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <atomic>
#include "../../include/tvgb.h"

namespace tvgb {

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
std::atomic<unsigned long long>& launch_counter();

#define TVGB_CHECK_ARG(cond, ...)                    \
    do {                                             \
        if (!(cond)) {                               \
            ::tvgb::set_error(__VA_ARGS__);          \
            return TVGB_ERR_ARG;                     \
        }                                            \
    } while (0)

#define TVGB_CUDA(call)                                                                     \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            ::tvgb::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),       \
                              __FILE__, __LINE__);                                          \
            return e_ == cudaErrorMemoryAllocation ? TVGB_ERR_NOMEM : TVGB_ERR_CUDA;        \
        }                                                                                   \
    } while (0)

// after a <<<>>> launch
#define TVGB_LAUNCHED()                                                                     \
    do {                                                                                    \
        ::tvgb::launch_counter().fetch_add(1, std::memory_order_relaxed);                   \
        cudaError_t e_ = cudaGetLastError();                                                \
        if (e_ != cudaSuccess) {                                                            \
            ::tvgb::set_error("kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_),   \
                              __FILE__, __LINE__);                                          \
            return TVGB_ERR_CUDA;                                                           \
        }                                                                                   \
    } while (0)

#define TVGB_TRY(expr)                 \
    do {                               \
        int s_ = (expr);               \
        if (s_ != TVGB_OK) return s_;  \
    } while (0)

// ---------------------------------------------------------------- opt-in kernel timing
// When enabled (tvgb_profile_enable), each launch site records a CUDA event
// pair on its stream; tvgb_profile_read() resolves and aggregates them per
// kernel name.  Off by default: then a KernelTimer costs one atomic load.
struct KernelTimer {
    const char* name;
    cudaStream_t stream;
    cudaEvent_t a = nullptr, b = nullptr;
    KernelTimer(const char* n, cudaStream_t s);
    void stop();
};

// ---------------------------------------------------------------- pointers
// Device (or managed) memory -> true; host / unregistered -> false.
bool is_device_ptr(const void* p);

// A device view of a caller array: the caller's pointer if it is device
// memory, else a stream-ordered temporary (filled from the host for inputs,
// copied back by finish() for outputs).
// Device bytes held by the library's own temporaries (stream-ordered
// allocations, counted when enqueued / released), and their high-water mark.
void scratch_track(long long delta);

struct DevArray {
    void* user = nullptr;
    void* dev = nullptr;
    size_t bytes = 0;
    bool owned = false;
    bool output = false;
    cudaStream_t stream = nullptr;

    DevArray() = default;
    DevArray(const DevArray&) = delete;
    DevArray& operator=(const DevArray&) = delete;
    ~DevArray() {
        if (owned && dev) {
            cudaFreeAsync(dev, stream);
            scratch_track(-(long long)bytes);
        }
    }
    template <class T> T* get() const { return static_cast<T*>(dev); }
    // input: copy host data in
    int in(const void* p, size_t nbytes, cudaStream_t s);
    // output: allocate if host; optionally zero
    int out(void* p, size_t nbytes, cudaStream_t s, bool zero = false);
    // copy a host output back (asynchronously; caller synchronises)
    int finish();
};

// Plain stream-ordered scratch buffer.
struct Scratch {
    void* p = nullptr;
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
    Scratch() = default;
    Scratch(const Scratch&) = delete;
    Scratch& operator=(const Scratch&) = delete;
    ~Scratch() {
        if (p) {
            cudaFreeAsync(p, stream);
            scratch_track(-(long long)bytes);
        }
    }
    int alloc(size_t bytes, cudaStream_t s);
    template <class T> T* get() const { return static_cast<T*>(p); }
};

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// Synchronise when any caller array was host memory (its data must be in
// place before returning).
inline int sync_if(bool need, cudaStream_t s) {
    if (need) TVGB_CUDA(cudaStreamSynchronize(s));
    return TVGB_OK;
}

inline unsigned ceil_div(size_t a, unsigned b) { return unsigned((a + b - 1) / b); }

}  // namespace tvgb
