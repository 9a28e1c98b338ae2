// tira_gb300/tensorvote.h -- header-only C++ shims with tiralib's entry-point
// names and signatures, forwarding to libtvgb's C ABI (include/tvgb.h).
//
// A C++ caller of tiralib's tensor-voting path replaces
//     #include <tira/functions/tensorvote.h>   (and eigen.h / filter.h)
// with
//     #include <tira_gb300/tensorvote.h>
// and links libtvgb.so.  Behaviour follows the reference:
//   * synchronous: each call finishes its work on the default stream before
//     returning (the reference synchronises after its kernels);
//   * host or device pointers, classified per call (tensorvote.h:1880);
//   * the eigen / filter functions return newly allocated arrays, new[] /
//     malloc for host input and cudaMalloc for device input, as the reference
//     (eigen.h:933-941, 996-1006; filter.h:518-526); the caller frees them;
//   * a negative device index, which the reference's eigen launchers send to
//     their CPU code (eigen.h:897,946), is an error here: this library has no
//     CPU path.  Those calls report it and return nullptr;
//   * errors are printed and execution continues, as HANDLE_ERROR does
//     (tira/cuda/error.h:11-15); define TIRA_GB300_THROW to throw
//     std::runtime_error instead.
// Only float is implemented (the reference path is FP32); other types fail
// to compile.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>
#include <cuda_runtime.h>

#include "../tvgb.h"

namespace tira_gb300 {

inline void check(int status, const char* fn) {
    if (status == TVGB_OK) return;
#ifdef TIRA_GB300_THROW
    throw std::runtime_error(std::string(fn) + ": " + tvgb_last_error());
#else
    std::printf("%s failed: %s\n", fn, tvgb_last_error());
#endif
}

// Reports a failure the way check() does, for errors found in the shim itself.
inline void fail(const char* fn, const std::string& what) {
#ifdef TIRA_GB300_THROW
    throw std::runtime_error(std::string(fn) + ": " + what);
#else
    std::printf("%s failed: %s\n", fn, what.c_str());
#endif
}

// The reference's eigen launchers take a device index and run on the CPU
// when it is negative (eigen.h:897,946).  This library has no CPU path, so a
// negative index is an error, and so is a device that cannot be made current.
inline bool select_device(int device, const char* fn) {
    if (device < 0) {
        fail(fn, "device " + std::to_string(device) +
                     " requests the reference's CPU path, which this GPU library does not provide");
        return false;
    }
    const cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(fn, "cudaSetDevice(" + std::to_string(device) + "): " + cudaGetErrorString(e));
        return false;
    }
    return true;
}

inline bool on_device(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

template <class T>
inline T* alloc_like(const void* ref, size_t count) {
    T* p = nullptr;
    if (on_device(ref)) {
        if (cudaMalloc(&p, sizeof(T) * count) != cudaSuccess) p = nullptr;
    } else {
        p = new T[count];
    }
    return p;
}

template <class T>
using only_float = std::enable_if_t<std::is_same<T, float>::value, int>;

}  // namespace tira_gb300

namespace tira {

// tira::Neighbor2D (tensorvote.h:776), byte-compatible
struct Neighbor2D {
    int du, dv;
    float dx, dy, c1, c2, Ra, Rb, Rc, Va, Vb, Vc;
};
static_assert(sizeof(Neighbor2D) == 48, "Neighbor2D must be 48 bytes");

// tira::Neighbor3D (tensorvote.h:1147), byte-compatible.  The reference's d
// is a glm::vec3; here it is a plain three-float struct with the same
// layout (x, y, z), so the shim does not need glm.
struct Neighbor3D {
    struct vec3 {
        float x, y, z;
        float& operator[](int i) { return (&x)[i]; }
        const float& operator[](int i) const { return (&x)[i]; }
    };
    int du, dv, dw;   // offsets along x2 (fast), x1, x0 (slow)
    vec3 d;           // unit direction of (du, dv, dw); zero at the centre
    float c1, c2;     // exp(-l2 / sigma1^2), exp(-l2 / sigma2^2)
};
static_assert(sizeof(Neighbor3D) == 32, "Neighbor3D must be 32 bytes");

namespace cpu {
// tira::cpu::build_neighbors2d (tensorvote.h:1222-1223): the w*w table, as a vector
inline std::vector<Neighbor2D> build_neighbors2d(const int w, const float sigma1, const float sigma2,
                                                 const unsigned power, const unsigned samples, const bool stick,
                                                 const bool plate) {
    std::vector<Neighbor2D> nb;
    int count = 0;
    const int st = tvgb_build_neighbors2d(w, sigma1, sigma2, power, samples, stick, plate, nullptr, &count);
    tira_gb300::check(st, "tira::cpu::build_neighbors2d");
    if (st != TVGB_OK || count <= 0) return nb;
    nb.resize(std::size_t(count));
    tira_gb300::check(tvgb_build_neighbors2d(w, sigma1, sigma2, power, samples, stick, plate, nb.data(), &count),
                      "tira::cpu::build_neighbors2d");
    return nb;
}

// tira::cpu::build_neighbors3d (tensorvote.h:1411): the w*w*w table.  sigma is
// any (x, y) pair type, e.g. glm::vec2 as in the reference, read as
// (sigma1, sigma2).
template <class Vec2>
inline std::vector<Neighbor3D> build_neighbors3d(int w, Vec2 sigma) {
    std::vector<Neighbor3D> nb;
    int count = 0;
    const int st = tvgb_build_neighbors3d(w, float(sigma.x), float(sigma.y), nullptr, &count);
    tira_gb300::check(st, "tira::cpu::build_neighbors3d");
    if (st != TVGB_OK || count <= 0) return nb;
    nb.resize(std::size_t(count));
    tira_gb300::check(tvgb_build_neighbors3d(w, float(sigma.x), float(sigma.y), nb.data(), &count),
                      "tira::cpu::build_neighbors3d");
    return nb;
}
}  // namespace cpu

namespace cuda {

// tira::cuda::tensorvote3 (tensorvote.h:2817)
template <class Type, tira_gb300::only_float<Type> = 0>
void tensorvote3(const Type* input_field, Type* output_field, unsigned int s0, unsigned int s1, unsigned int s2,
                 float sigma, float sigma2, unsigned int w, unsigned int power, int device, bool stick, bool plate,
                 unsigned samples, bool is_atv) {
    tira_gb300::check(tvgb_tensorvote3(input_field, output_field, s0, s1, s2, sigma, sigma2, w, power, device, stick,
                                       plate, samples, is_atv, nullptr),
                      "tira::cuda::tensorvote3");
    cudaDeviceSynchronize();
}

// tira::cuda::tensorvote (tensorvote.h:2201)
template <class Type, tira_gb300::only_float<Type> = 0>
void tensorvote(Type* t_out, const Type* t_in, const Type sigma1, const Type sigma2, const int power, const unsigned w,
                const unsigned shape0, const unsigned shape1, const bool stick = true, const bool plate = true,
                const unsigned samples = 10, const bool is_atv = false, const bool debug = false) {
    (void)debug;
    tira_gb300::check(tvgb_tensorvote(t_out, t_in, sigma1, sigma2, power, w, shape0, shape1, stick, plate, samples,
                                      is_atv, nullptr),
                      "tira::cuda::tensorvote");
    cudaDeviceSynchronize();
}

// tira::cuda::tensorvote_prebuilt (tensorvote.h:2237)
template <class Type, tira_gb300::only_float<Type> = 0>
void tensorvote_prebuilt(Type* t_out, const Type* t_in, const Neighbor2D* host_nb, int nb_count, const Type sigma1,
                         const Type sigma2, const int power, const unsigned w, const unsigned shape0,
                         const unsigned shape1, const bool stick = true, const bool plate = true,
                         const unsigned samples = 10) {
    tira_gb300::check(tvgb_tensorvote_prebuilt(t_out, t_in, host_nb, nb_count, sigma1, sigma2, power, w, shape0,
                                               shape1, stick, plate, samples, nullptr),
                      "tira::cuda::tensorvote_prebuilt");
    cudaDeviceSynchronize();
}

// tira::cuda::evals3_symmetric (eigen.h:896): returns a new (3 n) array
template <class Type, tira_gb300::only_float<Type> = 0>
Type* evals3_symmetric(const Type* mats, const size_t n, int device) {
    if (!tira_gb300::select_device(device, "tira::cuda::evals3_symmetric")) return nullptr;
    Type* out = tira_gb300::alloc_like<Type>(mats, 3 * n);
    tira_gb300::check(tvgb_evals3_symmetric(mats, n, out, nullptr), "tira::cuda::evals3_symmetric");
    cudaDeviceSynchronize();
    return out;
}

// tira::cuda::evecs3spherical_symmetric (eigen.h:945): returns a new (6 n)
// array, on the device if either input is device memory
template <class Type, tira_gb300::only_float<Type> = 0>
Type* evecs3spherical_symmetric(const Type* mats, const Type* lambda, const size_t n, int device) {
    if (!tira_gb300::select_device(device, "tira::cuda::evecs3spherical_symmetric")) return nullptr;
    const void* ref = tira_gb300::on_device(mats) ? static_cast<const void*>(mats) : static_cast<const void*>(lambda);
    Type* out = tira_gb300::alloc_like<Type>(ref, 6 * n);
    tira_gb300::check(tvgb_evecs3spherical_symmetric(mats, lambda, n, out, nullptr),
                      "tira::cuda::evecs3spherical_symmetric");
    cudaDeviceSynchronize();
    return out;
}

// tira::cuda::evals2_symmetric (eigen.h:769)
template <class Type, tira_gb300::only_float<Type> = 0>
Type* evals2_symmetric(const Type* mats, const size_t n, int device) {
    if (!tira_gb300::select_device(device, "tira::cuda::evals2_symmetric")) return nullptr;
    Type* out = tira_gb300::alloc_like<Type>(mats, 2 * n);
    tira_gb300::check(tvgb_evals2_symmetric(mats, n, out, nullptr), "tira::cuda::evals2_symmetric");
    cudaDeviceSynchronize();
    return out;
}

// tira::cuda::evecs2polar_symmetric (eigen.h:828)
template <class Type, tira_gb300::only_float<Type> = 0>
Type* evecs2polar_symmetric(const Type* mats, const Type* evals, size_t n, int device) {
    if (!tira_gb300::select_device(device, "tira::cuda::evecs2polar_symmetric")) return nullptr;
    const void* ref = tira_gb300::on_device(mats) ? static_cast<const void*>(mats) : static_cast<const void*>(evals);
    Type* out = tira_gb300::alloc_like<Type>(ref, 2 * n);
    tira_gb300::check(tvgb_evecs2polar_symmetric(mats, evals, n, out, nullptr), "tira::cuda::evecs2polar_symmetric");
    cudaDeviceSynchronize();
    return out;
}

// tira::cuda::gaussian_filter3d (filter.h:401): returns a new volume (malloc
// for host input, cudaMalloc for device input)
template <typename ImageType, typename KernelType = float, tira_gb300::only_float<ImageType> = 0>
ImageType* gaussian_filter3d(const ImageType* source, unsigned int width, unsigned int height, unsigned int depth,
                             float sigma_w, float sigma_h, float sigma_d, unsigned int& out_width,
                             unsigned int& out_height, unsigned int& out_depth) {
    auto ks = [](float s) { unsigned k = unsigned(std::ceil(6.0f * s)); return k % 2 ? k : k + 1; };
    out_width = width - (ks(sigma_w) - 1);
    out_height = height - (ks(sigma_h) - 1);
    out_depth = depth - (ks(sigma_d) - 1);
    const size_t n = size_t(out_width) * out_height * out_depth;
    ImageType* out = nullptr;
    if (tira_gb300::on_device(source)) {
        if (cudaMalloc(&out, n * sizeof(ImageType)) != cudaSuccess) out = nullptr;
    } else {
        out = static_cast<ImageType*>(std::malloc(n * sizeof(ImageType)));
    }
    unsigned dims[3];
    tira_gb300::check(tvgb_gaussian_filter3d(source, width, height, depth, sigma_w, sigma_h, sigma_d, out, dims,
                                             nullptr),
                      "tira::cuda::gaussian_filter3d");
    cudaDeviceSynchronize();
    return out;
}

// tira::cuda::gaussian_convolve2 (filter.h:305)
template <typename ImageType, typename KernelType = float, tira_gb300::only_float<ImageType> = 0>
ImageType* gaussian_convolve2(const ImageType* source, const unsigned in_sx, const unsigned in_sy, float sigma1,
                              float sigma2, unsigned int& out_width, unsigned int& out_height) {
    out_width = in_sx - (unsigned(sigma1 * 6) - 1);
    out_height = in_sy - (unsigned(sigma2 * 6) - 1);
    const size_t n = size_t(out_width) * out_height;
    ImageType* out = nullptr;
    if (tira_gb300::on_device(source)) {
        if (cudaMalloc(&out, n * sizeof(ImageType)) != cudaSuccess) out = nullptr;
    } else {
        out = static_cast<ImageType*>(std::malloc(n * sizeof(ImageType)));
    }
    unsigned dims[2];
    tira_gb300::check(tvgb_gaussian_convolve2(source, in_sx, in_sy, sigma1, sigma2, out, dims, nullptr),
                      "tira::cuda::gaussian_convolve2");
    cudaDeviceSynchronize();
    return out;
}

}  // namespace cuda
}  // namespace tira
