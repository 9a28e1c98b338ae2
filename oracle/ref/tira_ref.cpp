// C-ABI wrappers around tiralib's OWN CPU functions for the tensor-voting
// path, compiled straight from the reference headers (include path set by
// oracle/build_ref.sh) with the glm / Boost stand-ins in oracle/shim.
//
// Test infrastructure only: the library this file builds (oracle/_ref/) is
// used by tests/ to validate the C restatement in oracle/tvoracle.c and by
// tests/golden/make_golden.py to produce committed fixtures.  Nothing in the
// product links it.
//
// Wrapped reference functions (file:line within tiralib):
//   tira::cpu::evals3_symmetric            tira/functions/eigen.h:621
//   tira::cpu::evecs3spherical_symmetric   tira/functions/eigen.h:652
//   tira::cpu::evals2_symmetric            tira/functions/eigen.h:573
//   tira::cpu::evecs2polar_symmetric       tira/functions/eigen.h:598
//   tira::evec3_symmetric (cartesian)      tira/functions/eigen.h:452
//   tira::cpu::gaussian1d                  tira/functions/filter.h:38
//   tira::cpu::gaussian_convolve2          tira/functions/filter.h:159
//   tira::cpu::gaussian_convolve3          tira/functions/filter.h:175
//   tira::cpu::build_neighbors2d           tira/functions/tensorvote.h:1223
//   tira::cpu::tensorvote (2D TK / ATV)    tira/functions/tensorvote.h:1381
//   tira::cpu::tensorvote3 (3D TK / ATV)   tira/functions/tensorvote.h:1819
//   tira::sticknorm3                       tira/functions/tensorvote.h:1163
#include <cstdlib>
#include <cstring>
#include <tira/functions/tensorvote.h>
#include <tira/functions/filter.h>

extern "C" {

void ref_evals3(const float* mats9, size_t n, float* out3) {
    float* e = tira::cpu::evals3_symmetric<float>(mats9, n);
    std::memcpy(out3, e, sizeof(float) * 3 * n);
    delete[] e;
}

void ref_evecs3spherical(const float* mats9, const float* evals3, size_t n, float* out6) {
    float* e = tira::cpu::evecs3spherical_symmetric<float>(mats9, evals3, n);
    std::memcpy(out6, e, sizeof(float) * 6 * n);
    delete[] e;
}

void ref_evecs3cart(const float* mats9, const float* evals3, size_t n, float* out9) {
    for (size_t i = 0; i < n; ++i) {
        const float* m = mats9 + 9 * i;
        tira::evec3_symmetric<float>(m[0], m[1], m[4], m[2], m[5], m[8], evals3 + 3 * i,
                                     out9 + 9 * i, out9 + 9 * i + 3, out9 + 9 * i + 6);
    }
}

void ref_evals2(const float* mats4, size_t n, float* out2) {
    float* e = tira::cpu::evals2_symmetric<float>(mats4, n);
    std::memcpy(out2, e, sizeof(float) * 2 * n);
    delete[] e;
}

void ref_evecs2polar(const float* mats4, const float* evals2, size_t n, float* out2) {
    float* e = tira::cpu::evecs2polar_symmetric<float>(mats4, evals2, n);
    std::memcpy(out2, e, sizeof(float) * 2 * n);
    delete[] e;
}

void ref_gaussian1d(unsigned ksize, float sigma, float* out) {
    float* k = tira::cpu::gaussian1d<float>(ksize, 0.0f, sigma, 1.0f);
    std::memcpy(out, k, sizeof(float) * ksize);
    delete[] k;
}

// out must hold the valid-convolution size; returns it through out_dims.
void ref_gaussian_convolve3(const float* in, unsigned sx, unsigned sy, unsigned sz,
                            float sw, float sh, float sd, float* out, unsigned* out_dims) {
    unsigned ox, oy, oz;
    float* r = tira::cpu::gaussian_convolve3<float, float>(in, sx, sy, sz, sw, sh, sd, ox, oy, oz);
    std::memcpy(out, r, sizeof(float) * size_t(ox) * oy * oz);
    delete[] r;
    out_dims[0] = ox; out_dims[1] = oy; out_dims[2] = oz;
}

void ref_gaussian_convolve2(const float* in, unsigned sx, unsigned sy, float sigma,
                            float* out, unsigned* out_dims) {
    unsigned ox, oy;
    float* r = tira::cpu::gaussian_convolve2<float, float>(in, sx, sy, sigma, ox, oy);
    std::memcpy(out, r, sizeof(float) * size_t(ox) * oy);
    std::free(r);
    out_dims[0] = ox; out_dims[1] = oy;
}

// Writes count * 48 bytes (tira::Neighbor2D) into out; returns the count.
int ref_build_neighbors2d(int w, float sigma1, float sigma2, unsigned power, unsigned samples,
                          int stick, int plate, void* out) {
    std::vector<tira::Neighbor2D> nb =
        tira::cpu::build_neighbors2d(w, sigma1, sigma2, power, samples, stick != 0, plate != 0);
    if (out) std::memcpy(out, nb.data(), nb.size() * sizeof(tira::Neighbor2D));
    return int(nb.size());
}

int ref_sizeof_neighbor2d(void) { return int(sizeof(tira::Neighbor2D)); }

// Writes count * 32 bytes (tira::Neighbor3D) into out; returns the count.
int ref_build_neighbors3d(int w, float sigma1, float sigma2, void* out) {
    std::vector<tira::Neighbor3D> nb = tira::cpu::build_neighbors3d(w, glm::vec2(sigma1, sigma2));
    if (out) std::memcpy(out, nb.data(), nb.size() * sizeof(tira::Neighbor3D));
    return int(nb.size());
}

int ref_sizeof_neighbor3d(void) { return int(sizeof(tira::Neighbor3D)); }

void ref_tensorvote2(float* out4, const float* in4, float sigma1, float sigma2, int power, unsigned w,
                     unsigned s0, unsigned s1, int stick, int plate, unsigned samples, int is_atv) {
    tira::cpu::tensorvote<float>(out4, in4, sigma1, sigma2, power, w, s0, s1,
                                 stick != 0, plate != 0, samples, is_atv != 0);
}

void ref_tensorvote3(const float* in9, float* out9, unsigned s0, unsigned s1, unsigned s2,
                     float sigma1, float sigma2, unsigned w, unsigned power,
                     int stick, int plate, unsigned samples, int is_atv) {
    tira::cpu::tensorvote3(reinterpret_cast<glm::mat3*>(out9), reinterpret_cast<const glm::mat3*>(in9),
                           glm::vec2(sigma1, sigma2), power, w, s0, s1, s2,
                           stick != 0, plate != 0, samples, is_atv != 0);
}

double ref_sticknorm3(float sigma1, float sigma2, unsigned power) {
    return tira::sticknorm3<float>(sigma1, sigma2, power);
}

}  // extern "C"
