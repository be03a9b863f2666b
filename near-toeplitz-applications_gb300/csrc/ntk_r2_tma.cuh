// ntk_r2_tma.cuh -- TMA (cp.async.bulk.tensor), mbarrier and CTA-barrier
// helpers of the paired-chunk kernels (ntk_r2.cu, ntk_r2_adi.cu), and the
// host-side tensor-map encoding.
#pragma once
#include <cuda.h>

#include <mutex>

#include "ntk_internal.h"
#include "ntk_r2.cuh"

namespace ntk {
namespace r2 {

constexpr unsigned FULL = 0xffffffffu;
constexpr unsigned STATUS_TIMEOUT = 2u;
constexpr unsigned RANGE_MAG = 1151u << 20;  // high word of 2^128

// ---------------------------------------------------------------------------
// mbarrier / TMA (cp.async.bulk.tensor) helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Bounded wait for phase `parity` of the barrier: false when it did not
// complete within the limit (then the caller raises STATUS_TIMEOUT).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}
// Fetch a box into L2 only (no shared-memory destination, no completion to
// wait for): the load that follows finds the box in L2.
__device__ __forceinline__ void tma_prefetch_l2(const CUtensorMap* map, int c0, int c1, int c2, int c3) {
  asm volatile("cp.async.bulk.prefetch.tensor.4d.L2.global [%0, {%1, %2, %3, %4}];" ::"l"(map), "r"(c0), "r"(c1),
               "r"(c2), "r"(c3)
               : "memory");
}
__device__ __forceinline__ void tma_store(const CUtensorMap* map, int c0, int c1, int c2, int c3, const void* src) {
  asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%1, %2, %3, %4}], [%5];" ::"l"(map),
               "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void tma_store_commit_and_wait() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ unsigned char* align1024(unsigned char* p) {
  return reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~(uintptr_t)1023);
}

// Barriers over the threads that work on one group: the whole CTA, or a
// named barrier (id 1..15) over `count` threads of it.  all(v): a barrier
// that also returns whether v holds in every participating thread.
struct SyncAll {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
  __device__ __forceinline__ bool all(bool v) const { return __syncthreads_and(v) != 0; }
};
struct SyncBar {
  int id, count;
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
  }
  __device__ __forceinline__ bool all(bool v) const {
    unsigned r;
    asm volatile(
        "{ .reg .pred p, q; setp.ne.u32 p, %1, 0; bar.red.and.pred q, %2, %3, p; selp.u32 %0, 1, 0, q; }"
        : "=r"(r)
        : "r"((unsigned)v), "r"(id), "r"(count)
        : "memory");
    return r != 0;
  }
};

// Offset (in doubles) of rows 2i, 2i+1 of chunk j in a 4 KB system tile
// written by TMA with the 128-byte swizzle: 16-byte unit i XOR (j mod 8).
__device__ __forceinline__ int xpair(int j, int i) { return j * 16 + ((i ^ (j & 7)) << 1); }

// ---------------------------------------------------------------------------
// host: tensor maps
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// Rank-4 map (unused trailing dimensions of extent 1) over `base`.
inline int encode(CUtensorMap* m, const double* base, const cuuint64_t dims[4], const cuuint64_t strides[3],
           const cuuint32_t box[4], CUtensorMapSwizzle sw) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return NTK_ERR_UNSUPPORTED;
  }
  const cuuint32_t es[4] = {1, 1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, const_cast<double*>(base), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return NTK_ERR_UNSUPPORTED;
  }
  return NTK_OK;
}

}  // namespace r2
}  // namespace ntk
