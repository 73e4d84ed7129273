// TMA (cp.async.bulk.tensor) and mbarrier helpers, inline PTX for sm_103a.
//
// Every wait is bounded: a wait that gives up records an error code in a
// device word the host reads after the call (SC_ERR_TIMEOUT), waits once more
// (again bounded) for the copies it issued, and the kernel returns.  No trap,
// no unbounded spin.
#pragma once
#include <cuda.h>
#include <stdint.h>

#include "sc_common.cuh"

namespace sc {

constexpr int kTmaTimeout = 4;          // matches SC_ERR_TIMEOUT
constexpr int kSpinLimit = 4096;        // try_wait rounds (each suspends <= 0.2 ms): <= 0.8 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// First 128-byte aligned address in the dynamic shared-memory window (TMA
// destinations must be 128-byte aligned; the window itself is only
// guaranteed 16).  Launches reserve kSmemAlignPad extra bytes for this.
constexpr size_t kSmemAlignPad = 128;
__device__ __forceinline__ unsigned char* align128(unsigned char* p) {
  const uint32_t a = smem_u32(p);
  return p + ((128u - (a & 127u)) & 127u);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make mbarrier initialisation and prior generic-proxy accesses of shared
// memory visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(200000)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of `bar`.  On give-up: record the error,
// wait once more (bounded) so no copy is left writing into this CTA's shared
// memory, and return false; the caller then returns from the kernel.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* err) {
  for (int it = 0; it < kSpinLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  if (err) atomicExch(err, kTmaTimeout);
  for (int it = 0; it < kSpinLimit; ++it)
    if (mbar_try_wait(bar, parity)) break;
  return false;
}

// True once any CTA of the launch gave up a wait: later CTAs return before
// issuing copies.
__device__ __forceinline__ bool launch_failed(const int* err) {
  return err && *reinterpret_cast<const volatile int*>(err) != 0;
}

// 4D tiled load global -> shared, completion counted on `bar` (bytes).
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0,
                                            int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}

// Bulk tensor store of one box from shared memory, tracked by bulk groups.
// The threads that wrote the box fence their writes (fence_proxy_async) and
// meet at a barrier before one thread issues the store; that thread commits
// the group and waits for its reads (tma_store_wait_read) before the source
// is written again or the CTA exits.
__device__ __forceinline__ void tma_store_4d(const CUtensorMap* map, const void* src, int c0, int c1, int c2,
                                             int c3) {
  asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%2, %3, %4, %5}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(smem_u32(src)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
               : "memory");
}
__device__ __forceinline__ void tma_store_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// at most N of the most recent committed groups still reading
template <int N = 0> __device__ __forceinline__ void tma_store_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}

// 1D bulk copy global -> shared of `bytes` (both addresses 16-byte aligned,
// bytes a multiple of 16), completion counted on `bar`.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// L2 prefetch of one box of a tensor map (the copy engine fetches it; no
// completion to wait for, boxes outside the tensor fetch nothing).
__device__ __forceinline__ void tma_prefetch_4d(const CUtensorMap* map, int c0, int c1, int c2, int c3) {
  asm volatile("cp.async.bulk.prefetch.tensor.4d.L2.global.tile [%0, {%1, %2, %3, %4}];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(c0), "r"(c1), "r"(c2), "r"(c3)
               : "memory");
}

// Tensor view of `nf` equally spaced fields for the strided-axis passes:
// dims (x: nxh complex in 8-byte units, y: ny, z: nz, field), rows of pitch
// nxp.  Columns beyond nxh are outside the tensor and load as zero.
struct TmaFields {
  CUtensorMap map;
  int nf;
};

}  // namespace sc
