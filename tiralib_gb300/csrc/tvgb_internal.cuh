// Device-pointer entry points shared between libtvgb's translation units.
#pragma once
#include "tvgb_common.cuh"

namespace tvgb {

// eigen.cu: batched 3x3 solve on device arrays
int eig3_device(const float* in, int layout, size_t n, float* ev, float* vec, int fmt, bool precise,
                unsigned long long* nref, cudaStream_t s);

// structure.cu: fused gradient -> outer product -> separable Gaussian
int structure_tensor3_device(const float* vol, unsigned s0, unsigned s1, unsigned s2, float sigma, int mode,
                             float* out, int out_layout, unsigned* out_dims, cudaStream_t s);
void structure_tensor3_dims(unsigned s0, unsigned s1, unsigned s2, float sigma, int mode, unsigned* dims);

// vote3.cu: voting on device arrays (in / out in the given layouts)
// Called by vote3_device after the launch that votes receiver planes [z0, z1)
// (in order, every plane once) when slab > 0.
struct SlabHook {
    int (*fn)(void* ctx, unsigned z0, unsigned z1);
    void* ctx;
    unsigned slab;   // receiver planes per launch; 0: one launch, no calls
};
int vote3_device(const float* in, int in_layout, unsigned s0, unsigned s1, unsigned s2, const tvgb_vote3_params& p,
                 float* out, int out_layout, float* evals3, float* evecs, int evec_format, cudaStream_t s,
                 const SlabHook* hook = nullptr);
// A host output of a vote and the device temporary it is computed in.
struct HostOut {
    float* host;
    const float* dev;
    size_t per;      // floats per voxel
    bool planes;     // per component planes of n floats rather than interleaved
};
// vote3_device in z-slabs, each slab's part of every HostOut copied to the
// host on a second stream while the next slab votes; returns after all of
// it has completed (st synchronised).
int vote3_to_host(const float* in, int in_layout, unsigned s0, unsigned s1, unsigned s2, const tvgb_vote3_params& p,
                  float* out, int out_layout, float* evals3, float* evecs, int evec_format, const HostOut* outs,
                  int nouts, cudaStream_t s);

// reconstruct.cu: SIMF of two (n, 4) fields into acc[0..2] = (<A,B>, <B,B>, sum of norms)
int simf2_device(const float4* A, const float4* B, size_t n, double* acc3, cudaStream_t s);

// surrogate.cu: the network's tensor-core form from a parameter vector
// (host or device), and its evaluation on n inputs (n x 8 floats)
int sur_upload(const float* params, uint2* frag_dev, float* bias_dev, cudaStream_t s);
int sur_eval_device(const uint2* frag, const float* bias, const float* X, size_t n, float* Y, cudaStream_t s);
// the tcgen05 network (sur_tc.cuh): weight image upload and evaluation
int sur_upload_tc(const float* params, void* img_dev, cudaStream_t s);
int sur_eval_tc_device(const void* img, const float* X, size_t n, float* Y, int gelu_mode, int* err, cudaStream_t s,
                       uint32_t wait_limit = 1u << 24);

// window rule of the reference's Python layer (tensorvote_tk.cu:88-95)
inline unsigned auto_window(float s1, float s2) {
    const float sm = s2 > s1 ? s2 : s1;
    int w = 2 * int(3.0f * sm) + 1;
    if (w < 3) w = 3;
    if (w % 2 == 0) w += 1;
    return unsigned(w);
}

}  // namespace tvgb
