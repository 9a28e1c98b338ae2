/* tvoracle.h -- CPU restatement of tiralib's tensor-voting path.
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU baseline leg of bench.py as the checker / timed CPU reference; the
 * product (tiralib_gb300, libtvgb.so) never links or calls it. */
#pragma once
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
/* eigen (tira/functions/eigen.h) */
void or_eval2(float a, float b, float c, float* e0, float* e1);
void or_evec2polar(float a, float b, float c, const float* lambdas, float* theta0, float* theta1);
void or_evals2(const float* mats4, size_t n, float* evals2);
void or_evecs2polar(const float* mats4, const float* evals2, size_t n, float* thetas2);
void or_eval3(float a, float b, float c, float d, float e, float f, float* e0, float* e1, float* e2);
void or_evec3(float a, float b, float c, float d, float e, float f, const float* evals, float* ev0, float* ev1, float* ev2);
void or_evec3spherical(float a, float b, float c, float d, float e, float f, const float* evals, float* out6);
void or_spherical_to_cartesian(float theta, float phi, float* out3);
void or_evals3(const float* m9, size_t n, float* evals3);
void or_evecs3spherical(const float* m9, const float* evals3, size_t n, float* out6);
void or_evecs3cart(const float* m9, const float* evals3, size_t n, float* out9);
void or_eig3_batch_threads(const float* m9, size_t n, float* evals3, float* evecs9, int threads);
void or_eig3_f64(const double* s6, double* evals3, double* evecs9);
void or_eig3_f64_batch(const double* s6, size_t n, double* evals3, double* evecs9);
/* filter / gradient / structure tensor (tira/functions/filter.h, tira/volume.h) */
unsigned or_ksize3(float sigma);
unsigned or_ksize2(float sigma);
void or_gaussian1d(unsigned ksize, float sigma, float* k);
void or_gaussian_convolve3(const float* in, unsigned sx, unsigned sy, unsigned sz, float sw, float sh, float sd, float* out, unsigned* out_dims);
void or_gaussian_convolve2(const float* in, unsigned sx, unsigned sy, float sigma, float* out, unsigned* out_dims);
void or_gradient3(const float* vol, unsigned s0, unsigned s1, unsigned s2, int axis, float* out);
void or_structure_tensor3(const float* vol, unsigned s0, unsigned s1, unsigned s2, float sigma, int mode, float* out6, unsigned* out_dims);
void or_structure_tensor2(const float* img, unsigned s0, unsigned s1, float sigma, int mode, float* out4, unsigned* out_dims);
/* voting (tira/functions/tensorvote.h) */
float or_sticknorm3(float s1, float s2, unsigned p);
void or_tensorvote3(const float* in9, float* out9, unsigned s0, unsigned s1, unsigned s2, float sigma1, float sigma2,
                    unsigned w, unsigned power, int stick, int plate, unsigned samples, int is_atv);
void or_tensorvote3_sel(const float* in9, float* out9, unsigned s0, unsigned s1, unsigned s2, float sigma1, float sigma2,
                        unsigned w, unsigned power, int stick, int plate, unsigned samples, int is_atv,
                        const long long* receivers, long long n_recv, int threads);
void or_tensorvote3_f64(const float* in9, double* out6, unsigned s0, unsigned s1, unsigned s2, double sigma1, double sigma2,
                        unsigned w, unsigned power, int stick, int plate, int ball, const long long* receivers, long long n_recv, int threads);
int or_build_neighbors2d(int w, float s1, float s2, unsigned power, unsigned samples, int stick, int plate, void* out);
void or_tensorvote2(float* out4, const float* in4, float s1, float s2, int power, unsigned w, unsigned S0, unsigned S1,
                    int stick, int plate, unsigned samples, int is_atv);
void or_tensorvote2_prebuilt(float* out4, const float* in4, const void* nb, int nbc, float s1, float s2, int power,
                             unsigned w, unsigned S0, unsigned S1, int stick, int plate, unsigned samples);
/* plate / ball vote surrogate: FP64 MLP and its training target */
int or_mlp_param_count(void);
double or_mlp_loss_grad(const double* P, const double* X, const double* T, int B, int quant, double* grad, double* Y);
void or_surrogate_target(const double* dir, const double* n, int plate, double* F);
#ifdef __cplusplus
}
#endif
