// Tensor Memory Accelerator helpers (inline PTX, sm_90+): tensor-map
// creation on the host through the driver entry point (no link-time
// dependency on libcuda), mbarrier set-up and bounded waits, tiled bulk
// loads and bulk reduce-adds.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pmgb {

// Encodes a tiled tensor map over a float32 array with `rank` dimensions
// (dims/box innermost first; strides in bytes for dims 1..rank-1).  Returns
// PMGB_OK or an error status.
int make_tensor_map(CUtensorMap *map, const void *base, int rank, const uint64_t *dims,
                    const uint64_t *strides_bytes, const uint32_t *box);

// Spin limit of an mbarrier wait: far above any real transfer time, so a
// wait that reaches it means the copy will not complete.
constexpr uint32_t MBAR_SPIN_LIMIT = 1u << 24;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// Makes mbarrier initialisation and generic-proxy shared-memory writes
// visible to the async proxy (TMA).
__device__ __forceinline__ void fence_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// Waits for phase `parity` of the barrier to complete; returns false if
// `limit` polls went by first.
__device__ __forceinline__ bool mbar_wait_limit(uint64_t *bar, uint32_t parity, uint32_t limit) {
  const uint32_t a = smem_addr(bar);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// The same with the library's spin limit.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  return mbar_wait_limit(bar, parity, MBAR_SPIN_LIMIT);
}

// Host side: PMGB_OK, or PMGB_ERR_CUDA when the counters a tile kernel kept
// (stats[2]) show that one of its mbarrier waits reached its spin limit.
// Waits for `stream` (the counters are read back).
int check_wait_stats(const uint32_t *stats, cudaStream_t stream);

// Host side: launches a one-CTA kernel that arms an mbarrier for 16 bytes,
// issues no copy and waits with a limit of `limit` polls; *status_dev (a
// device word) becomes 1 if the wait ran out, 0 if it completed.
int test_wait_timeout(uint32_t limit, uint32_t *status_dev, cudaStream_t stream);

// 4-D tiled load of the tensor-map box at (c0, c1, c2, c3) into shared
// memory, completing on `bar`.
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            int c2, int c3, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
      "r"(smem_addr(bar))
      : "memory");
}

// 3-D tiled reduce-add of a shared-memory box into global memory at
// (c0, c1, c2) (float32 add performed by the memory system).
__device__ __forceinline__ void tma_reduce_add_3d(const CUtensorMap *map, int c0, int c1, int c2,
                                                  const void *src) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group"
      " [%0, {%1, %2, %3}], [%4];" ::"l"(reinterpret_cast<uint64_t>(map)),
      "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(src))
      : "memory");
}

// 4-D tiled reduce-add of a shared-memory box into global memory.
__device__ __forceinline__ void tma_reduce_add_4d(const CUtensorMap *map, int c0, int c1, int c2,
                                                  int c3, const void *src) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.4d.global.shared::cta.add.tile.bulk_group"
      " [%0, {%1, %2, %3, %4}], [%5];" ::"l"(reinterpret_cast<uint64_t>(map)),
      "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(src))
      : "memory");
}

// 3-D tiled load of the tensor-map box at (c0, c1, c2), completing on `bar`.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            int c2, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// Waits until the committed bulk operations have finished reading shared
// memory (the source may then be overwritten).
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// The same, except for the most recently committed group (still in flight).
__device__ __forceinline__ void bulk_wait_read_prior() {
  asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
}

// Waits until the committed bulk operations have completed.
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

}  // namespace pmgb
