// Tensor Memory Accelerator (TMA) loads for sm_100-family GPUs (built here
// for sm_103a): a tiled box of a global tensor copied into shared memory by
// cp.async.bulk.tensor, its completion signalled on an mbarrier with a
// transaction byte count.  Plain loads of this GPU's own memory into the
// issuing CTA's shared memory: no cluster multicast.
//
// Rules the callers keep:
//   * the tensor map (built on the host by make_tmap_3d_f32) describes a
//     16-byte aligned global array whose row strides are multiples of 16
//     bytes, and a box whose innermost extent is a multiple of 16 bytes;
//   * the innermost box coordinate x of every load is a multiple of 4
//     (float32: x * 4 bytes a multiple of 16).  The other coordinates may be
//     negative or past the end: those elements read as zero;
//   * the shared-memory destination is 128-byte aligned;
//   * every wait on the mbarrier is bounded (tc::mbar_wait).
#pragma once
#include <cuda.h>
#include <stdint.h>
#include "tc_sm100.cuh"

namespace tvgb {
namespace tma {

// one thread: arrive on the barrier and announce the bytes the next copy delivers
__device__ __forceinline__ void arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// box at (x, y, z) of a rank-3 tensor map into dst; completes bytes on bar
__device__ __forceinline__ void load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(tc::smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(tc::smem_u32(bar))
        : "memory");
}

// generic-proxy accesses of shared memory ordered before later async-proxy (TMA) writes
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

}  // namespace tma

// Host: a rank-3 float32 tensor map of dims (x, y, z) = (s2, s1, s0), x
// fastest, dense rows, box (bx, by, 1), zero fill outside.  Returns false
// (map untouched) when the driver entry point is missing or the encoding
// is refused (alignment rules above).
bool make_tmap_3d_f32(CUtensorMap* map, const float* base, unsigned s2, unsigned s1, unsigned s0, unsigned bx,
                      unsigned by);

}  // namespace tvgb
