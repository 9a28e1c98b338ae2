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
#define TVGB_ERR_UNSUPPORTED 4  /* a valid request the library does not implement */

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
/* device must be >= 0 and is made current (the reference's negative index
 * selects its CPU eigen path, eigen.h:897, which is not provided): a
 * negative index returns TVGB_ERR_ARG. */
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

/* Replaces tira::cpu::build_neighbors3d (tensorvote.h:1411), host only: writes
 * w*w*w tira::Neighbor3D records (tensorvote.h:1147; 32 bytes each: int32
 * du, dv, dw, float32 d.x, d.y, d.z, c1, c2) to out (may be NULL) and their
 * count to count. */
int tvgb_build_neighbors3d(int w, float sigma1, float sigma2, void* out, int* count);

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
 *     the lookup is repeated after the device's context changes (a
 *     cudaDeviceReset, or another library resetting the primary context),
 *     so that first call after a reset should also precede any capture;
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

/* ---- Consumers of a voted 2D field (tiralib's Python layer,
 * python/tira/tensors_lib/reconstruct.py and metrics.py, has no C or CUDA
 * counterpart; these replace its NumPy / SciPy code for this path).  Fields
 * are n pixels of [a, b, b, c] float32 (the 2D vote's layout); host or
 * device pointers. */

/* Replaces reconstruct.py:14 stick_saliency: |lambda|max - |lambda|min per
 * pixel into saliency (n floats). */
int tvgb_stick_saliency2(const float* field, size_t n, float* saliency, void* stream);

/* Replaces reconstruct.py:34 _otsu_threshold: Otsu's threshold of n
 * non-negative values (256-bin histogram over [0, max], NumPy's bin rules),
 * written to *threshold (host). */
int tvgb_otsu_threshold(const float* values, size_t n, double* threshold, void* stream);

/* Replaces reconstruct.py:66 saliency_threshold on an s0 x s1 field: mask =
 * saliency > threshold (Otsu's when use_otsu != 0); with fill != 0 the mask
 * is closed with a (2 close_radius + 1)^2 square (border value 0) and its
 * holes (background not 4-connected to the border) are filled, as
 * scipy.ndimage.binary_closing + binary_fill_holes.  mask: s0 * s1 bytes
 * (0 / 1).  threshold_used (host, may be NULL) receives the threshold. */
int tvgb_saliency_threshold2(const float* field, unsigned s0, unsigned s1, int fill, int use_otsu, double threshold,
                             int close_radius, unsigned char* mask, double* threshold_used, void* stream);

/* Replaces metrics.py:37 simf: mean over pixels of ||A - alpha B||_F with
 * alpha = <A,B> / <B,B> (0 when <B,B> < 1e-8), written to *simf (host). */
int tvgb_simf2(const float* A, const float* B, size_t n, double* simf, void* stream);

/* The objective evaluations of optimize.py:256 optimize_tk as one call: K
 * parameter sets params[3k..3k+2] = (sigma1, sigma2, power) (power rounded
 * down, >= 1) voted on t_in (TK stick + plate with `samples` plate samples
 * when plate != 0; window 2 int(3 max(sigma1, sigma2)) + 1 as
 * optimize.py:_w_from_sigma), each scored by simf against G into simf[k]
 * (host).  The input is solved once for all K sets.  t_out, if not NULL,
 * receives the K voted fields (K * shape0 * shape1 * 4 floats). */
int tvgb_tensorvote_sweep(const float* t_in, const float* G, unsigned shape0, unsigned shape1, const double* params,
                          int K, unsigned samples, int plate, double* simf, float* t_out, void* stream);

/* ---- Learned plate / ball vote (no reference counterpart: a learned
 * stand-in for the reference's plate3_numerical_device, tensorvote.h:2457).
 * The network is an MLP 28 -> 64 -> 64 -> 64 -> 6 (GELU; BF16 weights and
 * activations on the tensor cores, FP32 accumulation) from the features of
 * (offset direction d = o / |o|, plate normal n, flag: 1 plate / 0 ball) --
 * the seven inputs, then d_i d_j and n_i n_j (i <= j) and d_i n_j -- to the
 * vote's angular part (xx, xy, xz, yy, yz, zz) for sigma2 = 0, power 1,
 * o != 0; the Gaussian exp(-|o|^2 / sigma^2) is applied analytically.  Parameters: a
 * float32 vector of tvgb_surrogate_param_count() values, layout
 * W1[64][28] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[8][64] b4[8]
 * (W[out][in]; W4[6..7][.], b4[6..7] zero).  Arrays are host or device
 * pointers; X and T hold 8 floats per sample (the seven raw inputs padded
 * with a zero, targets with two); the features are formed on the device. */
int tvgb_surrogate_param_count(void);

/* n training samples from the plain orientation integral (64 orientations;
 * offset directions and normals uniform on the sphere, plate or ball with
 * probability 1/2; counter-based random stream `seed`). */
int tvgb_surrogate_samples(size_t n, unsigned long long seed, float* X, float* T, void* stream);

/* One quantisation-aware forward + backward pass over batch samples (batch a
 * multiple of 32): grad (param_count floats) = d loss / d params, *loss
 * (host) = sum over samples and the 6 outputs of (y - t)^2 / batch. */
int tvgb_surrogate_grad(const float* params, const float* X, const float* T, int batch, float* grad, float* loss,
                        void* stream);

/* `steps` Adam steps (batch samples each, cycling through the n samples;
 * learning rate lr with cosine decay to lr / 100); params updated in place;
 * loss_history (steps floats, may be NULL) gets each step's loss. */
int tvgb_surrogate_train(float* params, const float* X, const float* T, size_t n, int batch, int steps, float lr,
                         float* loss_history, void* stream);

/* The network on the tensor cores: Y (n x 8 floats, 6 used) from X. */
int tvgb_surrogate_eval(const float* params, const float* X, size_t n, float* Y, void* stream);

/* The same network on the fifth-generation tensor cores (tcgen05.mma, the
 * activations in tensor memory, 128 samples per tile).  gelu_mode 0: GELU in
 * FP32 with the hardware tanh, as tvgb_surrogate_eval; 1: GELU in packed
 * BF16 arithmetic (the arithmetic of the training forward pass and of the
 * surrogate vote).  Returns TVGB_ERR_CUDA if a tensor-core wait timed out. */
int tvgb_surrogate_eval_tc(const float* params, const float* X, size_t n, float* Y, int gelu_mode, void* stream);

/* tvgb_surrogate_eval_tc with the bound on each layer's wait for its MMAs
 * made explicit (no reference counterpart): wait_limit < 0 is the default
 * (2^24 mbarrier polls), 0 <= wait_limit <= 2^24 that many polls.  A wait
 * that runs out makes every thread of the CTA stop at its next layer; the
 * MMAs still in flight are then waited for with the full default bound
 * before the tensor memory is released, and the call returns TVGB_ERR_CUDA
 * with the device context intact.  wait_limit = 0 gives up at once: it
 * exists to test that path. */
int tvgb_surrogate_eval_tc_limit(const float* params, const float* X, size_t n, float* Y, int gelu_mode,
                                 long long wait_limit, void* stream);

/* tvgb_vote3 (TK, power 1, sigma2 = 0) with the plate (and ball) vote by
 * plate_mode: 0 the network (judged per CTA of 32 x 4 receivers: if its
 * first 32 receivers' plate differs from the exact plate by more than tol x
 * the norm of their voted tensors, normwise over the 32, the CTA's plate is
 * voted exactly), 1 the exact closed form, 2 the plain 64-orientation
 * integral.  The stick vote
 * is exact in every mode.  stats (2 values, host, may be NULL): CTAs, and
 * CTAs recomputed exactly. */
int tvgb_vote3_surrogate(const float* in, int in_layout, unsigned s0, unsigned s1, unsigned s2,
                         const tvgb_vote3_params* params, const float* net_params, int plate_mode, float tol,
                         float* out, int out_layout, float* evals3, float* evecs, int evec_format,
                         unsigned long long* stats, void* stream);

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

/* Device memory the library has freed stays in its own per-device pool for
 * the next call (no reference counterpart: the reference allocates and frees
 * per call).  This returns every pool's unused memory to the driver. */
int tvgb_release_cached_memory(void);

/* Opt-in per-kernel timing (no reference counterpart; the reference has no
 * timers): while enabled, every launch is bracketed by a CUDA event pair on
 * its stream.  tvgb_profile_read resolves the recorded launches (waiting on
 * their events), writes one "kernel launches total_ms" line per kernel into
 * buf and clears the record.  The switch is process-wide. */
int tvgb_profile_enable(int on);
int tvgb_profile_read(char* buf, size_t buflen);

/* Measured FP32 peak (no reference counterpart; the denominator of the
 * voting kernels' roofline): a kernel of independent packed FP32 fused
 * multiply-add chains on every SM for ~40 ms.  *tflops gets its rate (an FMA
 * = 2 flops), *sm_mhz (may be NULL) the mean SM clock it ran at, from the
 * SMs' cycle counters against the global timer. */
int tvgb_fp32_peak(double* tflops, double* sm_mhz, void* stream);

/* Measured pipe rates per SM clock (no reference counterpart; they bound the
 * learned vote's activations): rates[0] FP32 FMAs, rates[1] tanh.approx.f32
 * results, rates[2] tanh.approx.bf16x2 results (two per instruction),
 * rates[3] the SM clock in MHz, all from throughput kernels on every SM. */
int tvgb_pipe_rates(double* rates, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TVGB_H */
