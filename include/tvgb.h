/*
 * tvgb.h -- C ABI of libtvgb.so, the GB300 (sm_103a) implementation of
 * tiralib's tensor-voting path: separable-Gaussian structure tensor, 2D/3D
 * stick / plate / ball vote accumulation, and batched 2x2 / 3x3 symmetric
 * eigendecomposition.
 *
 * Conventions shared by every entry point
 *   - Every function returns an int status: TVGB_OK (0) or one of the
 *     TVGB_ERR_* codes; tvgb_last_error() gives a message for the calling
 *     thread's most recent failure.  (The reference prints CUDA errors and
 *     carries on, tira/cuda/error.h:11-15; its pybind layer throws
 *     std::runtime_error on bad arguments, cuda_ext/tensorvote_tk.cu:73-83.)
 *   - Array arguments may be host or device pointers; each is classified
 *     per call with cudaPointerGetAttributes, as the reference does
 *     (tensorvote.h:1880-1890, eigen.h:910-919).  Host inputs are staged to
 *     the device and host outputs are copied back before the call returns.
 *     A call whose arrays are all device memory is asynchronous on `stream`.
 *   - `stream` is a cudaStream_t (NULL = the legacy default stream).  The
 *     reference runs synchronously on the default stream; the C++ shims in
 *     include/tira_gb300/ pass NULL and synchronise.
 *   - The current CUDA device is used unless a `device` argument says
 *     otherwise (tira::cuda::tensorvote3 selects the device, :2820).
 *   - No global mutable state: calls on different streams may overlap.
 *     (The reference keeps its 3D neighbour table in one __constant__
 *     symbol, tensorvote.h:2316, and is not reentrant.)
 *   - Layouts: 3D volumes are (s0, s1, s2) slow to fast, voxel index
 *     (x0 * s1 + x1) * s2 + x2; a "mat3" tensor is 9 floats per voxel
 *     (glm::mat3, symmetric, so row/column order does not matter); "sym6"
 *     is 6 unique entries (xx, xy, xz, yy, yz, zz) with x the fast axis.
 *     2D tensors are 4 floats per pixel [a, b, b, c], row-major (s0, s1).
 */
#ifndef TVGB_H
#define TVGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TVGB_OK 0
#define TVGB_ERR_ARG 1          /* invalid argument (shape, sigma, window, null pointer) */
#define TVGB_ERR_CUDA 2         /* CUDA runtime or launch error */
#define TVGB_ERR_NOMEM 3        /* device allocation failed */
#define TVGB_ERR_UNSUPPORTED 4  /* valid request this build does not implement */

/* layouts / formats */
#define TVGB_LAYOUT_MAT3 9      /* 9 floats per voxel, AoS */
#define TVGB_LAYOUT_SYM6 6      /* 6 floats per voxel, AoS (xx, xy, xz, yy, yz, zz) */
#define TVGB_LAYOUT_SYM6_PLANES 60  /* 6 planes of n floats (component-major) */
#define TVGB_EVEC_NONE 0
#define TVGB_EVEC_CARTESIAN 1   /* 9 floats: e0, e1, e2 (ascending eigenvalue order) */
#define TVGB_EVEC_SPHERICAL 2   /* 6 floats: (theta, phi) of e0, e1, e2, as eigen.h:515 */
#define TVGB_EIG_PARITY 0       /* eigen.h's FP32 closed form, operation for operation */
#define TVGB_EIG_PRECISE 1      /* FP32 closed form + FP64 refinement of near-degenerate pairs */

const char* tvgb_last_error(void);
int tvgb_version(void);

/* ----------------------------------------------------------------------------
 * Symmetric eigendecomposition
 * ------------------------------------------------------------------------- */

/* Replaces tira::cuda::evals3_symmetric (tira/functions/eigen.h:896).
 * mats9: n glm::mat3; evals3: n x 3 ascending.  The reference returns a new
 * array; here the caller owns evals3 (host or device). */
int tvgb_evals3_symmetric(const float* mats9, size_t n, float* evals3, void* stream);

/* Replaces tira::cuda::evecs3spherical_symmetric (eigen.h:945): 6 floats per
 * matrix, (theta, phi) of the eigenvectors for evals3[0..2]. */
int tvgb_evecs3spherical_symmetric(const float* mats9, const float* evals3, size_t n, float* evecs6,
                                   void* stream);

/* Replaces tira::cuda::evals2_symmetric (eigen.h:769): mats4 [a,b,b,c]. */
int tvgb_evals2_symmetric(const float* mats4, size_t n, float* evals2, void* stream);

/* Replaces tira::cuda::evecs2polar_symmetric (eigen.h:828): theta0, theta1. */
int tvgb_evecs2polar_symmetric(const float* mats4, const float* evals2, size_t n, float* thetas2,
                               void* stream);

/* Fused one-pass 3x3 solve (no single reference function; it merges
 * eigen.h:896 and :945).  in_layout TVGB_LAYOUT_MAT3 / _SYM6 / _SYM6_PLANES;
 * evec_format TVGB_EVEC_*; mode TVGB_EIG_PARITY or TVGB_EIG_PRECISE.
 * evals3 or evecs may be NULL to skip that output.  n_refined (may be NULL)
 * receives the number of matrices the precise mode refined in FP64. */
int tvgb_eig3(const float* mats, int in_layout, size_t n, float* evals3, float* evecs, int evec_format,
              int mode, size_t* n_refined, void* stream);

/* ----------------------------------------------------------------------------
 * Separable Gaussian filter and structure tensor
 * ------------------------------------------------------------------------- */

/* Replaces tira::cuda::gaussian_filter3d (tira/functions/filter.h:401): valid
 * separable convolution of one scalar volume (width = fast axis), window
 * ceil(6 sigma) made odd per axis.  dst holds the output; out_dims receives
 * (out_width, out_height, out_depth). */
int tvgb_gaussian_filter3d(const float* src, unsigned width, unsigned height, unsigned depth,
                           float sigma_w, float sigma_h, float sigma_d, float* dst, unsigned* out_dims,
                           void* stream);

/* Replaces tira::cuda::gaussian_convolve2 (filter.h:305): valid separable 2D
 * convolution, window (unsigned)(6 sigma) per axis.  out_dims = (out_w, out_h). */
int tvgb_gaussian_convolve2(const float* src, unsigned in_sx, unsigned in_sy, float sigma1, float sigma2,
                            float* dst, unsigned* out_dims, void* stream);

/* 3D structure tensor of a scalar volume: central-difference gradient
 * (volume<T>::gradient, tira/volume.h:974) -> outer product -> separable
 * Gaussian per component (gaussian_filter3d, filter.h:401), fused.
 * mode 0: valid (output s_i - K + 1 per axis, as the reference);
 * mode 1: same size, tensor field zero outside the volume.
 * out_layout TVGB_LAYOUT_MAT3, _SYM6 or _SYM6_PLANES.
 * out_dims receives (s0', s1', s2'). */
int tvgb_structure_tensor3(const float* volume, unsigned s0, unsigned s1, unsigned s2, float sigma, int mode,
                           float* out, int out_layout, unsigned* out_dims, void* stream);

/* 2D structure tensor as the reference's 2D workload assembles it:
 * np.gradient(edge_order=2) (python/tira/tensors.py:36-37) -> outer product
 * [a,b,b,c] (tensors.py:40-51) -> gaussian_convolve2 (filter.h:305) per
 * component.  mode 0 valid, 1 same size. out_dims = (s0', s1'). */
int tvgb_structure_tensor2(const float* image, unsigned s0, unsigned s1, float sigma, int mode, float* out4,
                           unsigned* out_dims, void* stream);

/* ----------------------------------------------------------------------------
 * Tensor voting
 * ------------------------------------------------------------------------- */

/* Replaces template tira::cuda::tensorvote3<float> (tira/functions/tensorvote.h:2817):
 * input_field / output_field are n glm::mat3 (host or device).  TK when
 * is_atv == 0 (stick: largest eigenvector, plate: orientation integral of
 * stick votes about the smallest eigenvector; samples = 0 is the closed form,
 * samples > 0 the reference's samples-point rule, which equals the closed
 * form whenever samples >= power + 2); ATV (tensorvote.h:2640) when is_atv
 * != 0, with sigma as the ATV sigma.  The output is symmetric (the reference
 * GPU kernels write both halves, tensorvote.h:2452-2454, 2630-2632). */
int tvgb_tensorvote3(const float* input_field, float* output_field, unsigned s0, unsigned s1, unsigned s2,
                     float sigma, float sigma2, unsigned w, unsigned power, int device, int stick, int plate,
                     unsigned samples, int is_atv, void* stream);

/* Replaces template tira::cuda::tensorvote<float> (tensorvote.h:2201): 2D TK
 * (is_atv = 0) or ATV (is_atv = 1; sigma1 is the ATV sigma) on [a,b,b,c]. */
int tvgb_tensorvote(float* t_out, const float* t_in, float sigma1, float sigma2, int power, unsigned w,
                    unsigned shape0, unsigned shape1, int stick, int plate, unsigned samples, int is_atv,
                    void* stream);

/* Replaces tira::cuda::tensorvote_prebuilt<float> (tensorvote.h:2237): 2D TK
 * with a caller-built host table of nb_count tira::Neighbor2D records (48
 * bytes each: int32 du, dv; float32 dx, dy, c1, c2, Ra, Rb, Rc, Va, Vb, Vc). */
int tvgb_tensorvote_prebuilt(float* t_out, const float* t_in, const void* host_nb, int nb_count, float sigma1,
                             float sigma2, int power, unsigned w, unsigned shape0, unsigned shape1, int stick,
                             int plate, unsigned samples, void* stream);

/* Replaces tira::cpu::build_neighbors2d (tensorvote.h:1223), host only: writes
 * w*w Neighbor2D records to out (may be NULL) and their count to count. */
int tvgb_build_neighbors2d(int w, float sigma1, float sigma2, unsigned power, unsigned samples, int stick,
                           int plate, void* out, int* count);

/* Extended 3D voting (no single reference function; the options below extend
 * tira::cuda::tensorvote3, tensorvote.h:2817). */
typedef struct tvgb_vote3_params {
    float sigma1;       /* TK sigma1 (ATV sigma when is_atv) */
    float sigma2;       /* TK sigma2 */
    unsigned w;         /* odd window side; 0 = 2 * ceil(3 * max(sigma1, sigma2)) + 1 */
    unsigned power;     /* refinement exponent, >= 1 */
    unsigned samples;   /* plate orientation samples; 0 = closed form */
    int stick, plate;   /* TK terms */
    int ball;           /* TK ball term: lambda0 x mean of unit stick votes over the sphere (no reference counterpart) */
    int is_atv;         /* analytical tensor voting instead of TK */
    int parity;         /* 1: voter eigenvectors through eigen.h's spherical round trip (reference parity);
                           0: cartesian eigenvectors straight from the solver */
} tvgb_vote3_params;

/* in: n tensors in in_layout; out: voted tensors in out_layout (may be NULL);
 * evals3 / evecs: eigendecomposition of the voted tensor fused onto the vote
 * kernel (either may be NULL). */
int tvgb_vote3(const float* in, int in_layout, unsigned s0, unsigned s1, unsigned s2, const tvgb_vote3_params* p,
               float* out, int out_layout, float* evals3, float* evecs, int evec_format, void* stream);

/* Allocation-free variant of tvgb_vote3 (no counterpart in the reference).
 * For callers that must not allocate device memory while they run: code in
 * a host-side real-time loop or plugin callback where allocation is
 * forbidden, or processes whose device memory belongs to another allocator.
 * It calls no cudaMalloc / cudaMallocAsync / cudaFree and allocates nothing
 * else: its scratch (the per-voxel voter records) is a file-scope device
 * array of at most 524288 voxels (e.g. 80^3; 18 MiB held by every GPU that
 * loads the library, until the process exits).  Limits:
 *   - all arrays are device memory (in, out, evals3, evecs);
 *   - s0 * s1 * s2 <= 524288, else TVGB_ERR_ARG;
 *   - TK with power 1 and samples 0 or >= 3 (the fast kernel), no ATV, else
 *     TVGB_ERR_ARG;
 *   - the first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress) and should come before any stream capture;
 *   - every call shares the one array: calls whose work overlaps on the GPU
 *     (different streams, or host threads without ordering) race and must be
 *     serialised by the caller.  Nothing in the array needs zeroing: each
 *     call overwrites the records it reads. */
int tvgb_vote3_noalloc(const float* in, int in_layout, unsigned s0, unsigned s1, unsigned s2,
                       const tvgb_vote3_params* p, float* out, int out_layout, float* evals3, float* evecs,
                       int evec_format, void* stream);

/* Whole path on one volume: structure tensor (sigma_st, st_mode as
 * tvgb_structure_tensor3) -> TK vote -> fused eigendecomposition.  Outputs
 * as tvgb_vote3; out_dims receives the voted field's (s0', s1', s2'). */
int tvgb_pipeline3(const float* volume, unsigned s0, unsigned s1, unsigned s2, float sigma_st, int st_mode,
                   const tvgb_vote3_params* p, float* out, int out_layout, float* evals3, float* evecs,
                   int evec_format, unsigned* out_dims, void* stream);

/* Sticknorm of the 3D stick vote (tira::sticknorm3, tensorvote.h:1163), host. */
double tvgb_sticknorm3(float sigma1, float sigma2, unsigned power);

/* Counts every kernel launch this library has issued in the calling process
 * (for launch accounting in benchmarks). */
unsigned long long tvgb_launch_count(void);

/* Device bytes the library itself holds in stream-ordered temporaries (host
 * staging of caller arrays, voter records) and their high-water mark since
 * the last reset (no reference counterpart: for footprint reports).  Caller
 * arrays are not counted.  reset_peak != 0 restarts the mark at the current
 * value after reading it. */
int tvgb_memory_stats(unsigned long long* scratch_bytes, unsigned long long* scratch_peak_bytes, int reset_peak);

/* Opt-in per-kernel timing (no reference counterpart; the reference has no
 * timers): while enabled, every launch is bracketed by a CUDA event pair on
 * its stream.  tvgb_profile_read resolves the recorded launches (waiting on
 * their events), writes one "kernel launches total_ms" line per kernel into
 * buf and clears the record.  The switch is process-wide. */
int tvgb_profile_enable(int on);
int tvgb_profile_read(char* buf, size_t buflen);

#ifdef __cplusplus
}
#endif
#endif /* TVGB_H */
