/*
 * tvoracle_filter.c -- CPU restatement of tiralib's separable Gaussian filter,
 * central-difference gradient and the structure-tensor assembly of the path.
 *
 * TEST INFRASTRUCTURE ONLY (see tvoracle_eig.c for the rules that apply).
 *
 * Reference anchors:
 *   normaldist                 tira/functions/filter.h:15
 *   cpu::gaussian1d            tira/functions/filter.h:38
 *   cpu::convolve2 / convolve3 tira/functions/filter.h:67,108 (valid convolution)
 *   cpu::gaussian_convolve2    tira/functions/filter.h:159 (ksize = (unsigned)(6 sigma))
 *   cpu::gaussian_convolve3    tira/functions/filter.h:175 (ksize = ceil(6 sigma), made odd)
 *   volume<T>::gradient        tira/volume.h:974 (central inside, one-sided at the edges)
 *   np.gradient(edge_order=2)  python/tira/tensors.py:36-37 (2D structure tensor)
 * The 3D structure-tensor assembly (outer product of the gradient) has no
 * helper in the reference; the caller writes it (tensors.py:40-51 is the 2D form).
 */
#include "tvoracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PI_D 3.14159265358979323846

unsigned or_ksize3(float sigma) {            /* filter.h:178-183, 405-410 */
    unsigned k = (unsigned)ceilf(6.0f * sigma);
    if (k % 2 == 0) k++;
    return k;
}
unsigned or_ksize2(float sigma) { return (unsigned)(6.0f * sigma); }   /* filter.h:163, 308 */

/* normaldist + gaussian1d (mu = 0, dx = 1) */
void or_gaussian1d(unsigned ksize, float sigma, float* k) {
    const float halfwidth = (float)ksize * 1.0f / 2.0f;
    const float startx = -halfwidth + (1.0f / 2.0f);
    const float sigma_sq = sigma * sigma;
    const float pi = (float)PI_D;
    const float nrm = 1.0f / sqrtf(2.0f * pi * sigma_sq);
    float sum = 0.0f;
    for (unsigned i = 0; i < ksize; ++i) {
        const float x = startx + (float)i * 1.0f;
        k[i] = nrm * expf(-((x - 0.0f) * (x - 0.0f)) / (2.0f * sigma_sq));
        sum += k[i];
    }
    if (sum > 0.0f) {
        float inv = 1.0f / sum;
        for (unsigned i = 0; i < ksize; ++i) k[i] *= inv;
    }
}

/* one valid 1-D pass of a separable convolution along `axis` (0 = x fast,
 * 1 = y, 2 = z) of a (sx, sy, sz) volume; dst has the axis shortened by K-1. */
static void conv_axis(const float* src, unsigned sx, unsigned sy, unsigned sz,
                      const float* k, unsigned K, int axis, float* dst) {
    unsigned ox = sx - (axis == 0 ? K - 1 : 0);
    unsigned oy = sy - (axis == 1 ? K - 1 : 0);
    unsigned oz = sz - (axis == 2 ? K - 1 : 0);
    for (unsigned z = 0; z < oz; ++z)
        for (unsigned y = 0; y < oy; ++y)
            for (unsigned x = 0; x < ox; ++x) {
                float s = 0.0f;
                for (unsigned i = 0; i < K; ++i) {
                    unsigned xx = x + (axis == 0 ? i : 0), yy = y + (axis == 1 ? i : 0), zz = z + (axis == 2 ? i : 0);
                    s += k[i] * src[((size_t)zz * sy + yy) * sx + xx];
                }
                dst[((size_t)z * oy + y) * ox + x] = s;
            }
}

/* gaussian_convolve3: x pass, then y, then z (CPU order, filter.h:189-191) */
void or_gaussian_convolve3(const float* in, unsigned sx, unsigned sy, unsigned sz,
                           float sw, float sh, float sd, float* out, unsigned* out_dims) {
    unsigned kw = or_ksize3(sw), kh = or_ksize3(sh), kd = or_ksize3(sd);
    float* gw = (float*)malloc(sizeof(float) * kw);
    float* gh = (float*)malloc(sizeof(float) * kh);
    float* gd = (float*)malloc(sizeof(float) * kd);
    or_gaussian1d(kw, sw, gw); or_gaussian1d(kh, sh, gh); or_gaussian1d(kd, sd, gd);
    unsigned ox = sx - (kw - 1), oy = sy - (kh - 1), oz = sz - (kd - 1);
    float* t1 = (float*)malloc(sizeof(float) * (size_t)ox * sy * sz);
    float* t2 = (float*)malloc(sizeof(float) * (size_t)ox * oy * sz);
    conv_axis(in, sx, sy, sz, gw, kw, 0, t1);
    conv_axis(t1, ox, sy, sz, gh, kh, 1, t2);
    conv_axis(t2, ox, oy, sz, gd, kd, 2, out);
    out_dims[0] = ox; out_dims[1] = oy; out_dims[2] = oz;
    free(t1); free(t2); free(gw); free(gh); free(gd);
}

/* gaussian_convolve2: x pass then y pass, both with ksize = (unsigned)(6 sigma) */
void or_gaussian_convolve2(const float* in, unsigned sx, unsigned sy, float sigma,
                           float* out, unsigned* out_dims) {
    unsigned K = or_ksize2(sigma);
    float* g = (float*)malloc(sizeof(float) * (K ? K : 1));
    or_gaussian1d(K, sigma, g);
    unsigned ox = sx - (K - 1), oy = sy - (K - 1);
    float* t1 = (float*)malloc(sizeof(float) * (size_t)ox * sy);
    conv_axis(in, sx, sy, 1, g, K, 0, t1);
    conv_axis(t1, ox, sy, 1, g, K, 1, out);
    out_dims[0] = ox; out_dims[1] = oy;
    free(t1); free(g);
}

/* volume<T>::gradient(axis) with unit spacing: (b - a) / 2 inside, (b - a) at
 * the two faces normal to the axis.  Volume extents (s0, s1, s2) slow to fast;
 * axis 0 = x (fast, s2), 1 = y (s1), 2 = z (slow, s0), as in volume.h. */
void or_gradient3(const float* vol, unsigned s0, unsigned s1, unsigned s2, int axis, float* out) {
    const size_t stride = axis == 0 ? 1 : (axis == 1 ? s2 : (size_t)s1 * s2);
    const unsigned S = axis == 0 ? s2 : (axis == 1 ? s1 : s0);
    for (unsigned z = 0; z < s0; ++z)
        for (unsigned y = 0; y < s1; ++y)
            for (unsigned x = 0; x < s2; ++x) {
                const size_t i = ((size_t)z * s1 + y) * s2 + x;
                const unsigned c = axis == 0 ? x : (axis == 1 ? y : z);
                float g;
                if (S == 1) g = 0.0f;
                else if (c == 0) g = (float)((double)(vol[i + stride] - vol[i]) / 1.0);
                else if (c == S - 1) g = (float)((double)(vol[i] - vol[i - stride]) / 1.0);
                else g = (float)((double)(vol[i + stride] - vol[i - stride]) / 2.0);
                out[i] = g;
            }
}

/* 3-D structure tensor of the path: gradient -> outer product (components
 * xx, xy, xz, yy, yz, zz, x fastest) -> separable Gaussian per component.
 * mode 0: the reference's valid convolution (output s_i - K + 1 per axis).
 * mode 1: same-size output, the tensor field taken as zero outside the volume.
 * out6 is component-major planes: out6[c * n_out + voxel]. */
void or_structure_tensor3(const float* vol, unsigned s0, unsigned s1, unsigned s2, float sigma, int mode,
                          float* out6, unsigned* out_dims) {
    const size_t n = (size_t)s0 * s1 * s2;
    float* g[3];
    for (int a = 0; a < 3; ++a) { g[a] = (float*)malloc(sizeof(float) * n); or_gradient3(vol, s0, s1, s2, a, g[a]); }
    unsigned K = or_ksize3(sigma), R = K / 2;
    float* k = (float*)malloc(sizeof(float) * K);
    or_gaussian1d(K, sigma, k);
    unsigned px = mode ? s2 + 2 * R : s2, py = mode ? s1 + 2 * R : s1, pz = mode ? s0 + 2 * R : s0;
    unsigned ox = px - (K - 1), oy = py - (K - 1), oz = pz - (K - 1);
    size_t np_ = (size_t)px * py * pz, no = (size_t)ox * oy * oz;
    float* t = (float*)calloc(np_, sizeof(float));
    float* t1 = (float*)malloc(sizeof(float) * (size_t)ox * py * pz);
    float* t2 = (float*)malloc(sizeof(float) * (size_t)ox * oy * pz);
    const int ca[6] = {0, 0, 0, 1, 1, 2}, cb[6] = {0, 1, 2, 1, 2, 2};
    unsigned off = mode ? R : 0;
    for (int c = 0; c < 6; ++c) {
        for (unsigned z = 0; z < s0; ++z)
            for (unsigned y = 0; y < s1; ++y)
                for (unsigned x = 0; x < s2; ++x) {
                    size_t i = ((size_t)z * s1 + y) * s2 + x;
                    t[((size_t)(z + off) * py + (y + off)) * px + (x + off)] = g[ca[c]][i] * g[cb[c]][i];
                }
        conv_axis(t, px, py, pz, k, K, 0, t1);
        conv_axis(t1, ox, py, pz, k, K, 1, t2);
        conv_axis(t2, ox, oy, pz, k, K, 2, out6 + c * no);
    }
    out_dims[0] = oz; out_dims[1] = oy; out_dims[2] = ox;   /* (s0', s1', s2') slow to fast */
    free(t); free(t1); free(t2); free(k);
    for (int a = 0; a < 3; ++a) free(g[a]);
}

/* 2-D structure tensor as the C1 workload assembles it: np.gradient with
 * edge_order = 2 (tensors.py:36-37), outer product (tensors.py:40-51) stored
 * as [a, b, b, c] per pixel, then cpu::gaussian_convolve2 per component
 * (valid).  mode 1 keeps the size (field zero outside the image). */
void or_structure_tensor2(const float* img, unsigned s0, unsigned s1, float sigma, int mode,
                          float* out4, unsigned* out_dims) {
    const size_t n = (size_t)s0 * s1;
    float* gx = (float*)malloc(sizeof(float) * n);
    float* gy = (float*)malloc(sizeof(float) * n);
    for (unsigned r = 0; r < s0; ++r)
        for (unsigned c = 0; c < s1; ++c) {
            const float* f = img + (size_t)r * s1;
            float v;
            if (s1 < 3) v = 0.0f;
            else if (c == 0) v = (-3.0f * f[0] + 4.0f * f[1] - f[2]) / 2.0f;
            else if (c == s1 - 1) v = (3.0f * f[c] - 4.0f * f[c - 1] + f[c - 2]) / 2.0f;
            else v = (f[c + 1] - f[c - 1]) / 2.0f;
            gx[(size_t)r * s1 + c] = v;
            float w;
#define IMG(rr) img[(size_t)(rr) * s1 + c]
            if (s0 < 3) w = 0.0f;
            else if (r == 0) w = (-3.0f * IMG(0) + 4.0f * IMG(1) - IMG(2)) / 2.0f;
            else if (r == s0 - 1) w = (3.0f * IMG(r) - 4.0f * IMG(r - 1) + IMG(r - 2)) / 2.0f;
            else w = (IMG(r + 1) - IMG(r - 1)) / 2.0f;
#undef IMG
            gy[(size_t)r * s1 + c] = w;
        }
    unsigned K = or_ksize2(sigma), Rl = (K - 1) / 2, Rr = K - 1 - Rl;
    float* k = (float*)malloc(sizeof(float) * (K ? K : 1));
    or_gaussian1d(K, sigma, k);
    unsigned px = mode ? s1 + K - 1 : s1, py = mode ? s0 + K - 1 : s0;
    unsigned ox = px - (K - 1), oy = py - (K - 1);
    float* t = (float*)calloc((size_t)px * py, sizeof(float));
    float* t1 = (float*)malloc(sizeof(float) * (size_t)ox * py);
    float* o = (float*)malloc(sizeof(float) * (size_t)ox * oy);
    unsigned offl = mode ? Rl : 0;
    (void)Rr;
    for (int comp = 0; comp < 3; ++comp) {
        for (unsigned r = 0; r < s0; ++r)
            for (unsigned c = 0; c < s1; ++c) {
                size_t i = (size_t)r * s1 + c;
                float v = comp == 0 ? gx[i] * gx[i] : (comp == 1 ? gx[i] * gy[i] : gy[i] * gy[i]);
                t[(size_t)(r + offl) * px + (c + offl)] = v;
            }
        conv_axis(t, px, py, 1, k, K, 0, t1);
        conv_axis(t1, ox, py, 1, k, K, 1, o);
        for (size_t i = 0; i < (size_t)ox * oy; ++i) {
            if (comp == 0) out4[4 * i + 0] = o[i];
            else if (comp == 1) { out4[4 * i + 1] = o[i]; out4[4 * i + 2] = o[i]; }
            else out4[4 * i + 3] = o[i];
        }
    }
    out_dims[0] = oy; out_dims[1] = ox;
    free(t); free(t1); free(o); free(k); free(gx); free(gy);
}
