// Host side of the TMA helpers: tensor-map encoding through the driver entry
// point obtained from the runtime (so libpmgb has no link-time dependency on
// libcuda and still loads on machines without a GPU driver).
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"
#include "tma.cuh"

namespace pmgb {
namespace {

std::mutex g_mu;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int encoder(PFN_cuTensorMapEncodeTiled_v12000 *out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
      return fail(PMGB_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  *out = g_encode;
  return PMGB_OK;
}

// Arms the barrier for 16 bytes that no copy will ever deliver and waits
// with a bounded poll count: the wait must run out and report it.  Nothing
// is in flight, so the CTA can leave at once.
__global__ void wait_timeout_probe_kernel(uint32_t limit, uint32_t *status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_async_shared();
    mbar_expect_tx(&bar, 16);
  }
  __syncthreads();
  const bool ok = mbar_wait_limit(&bar, 0, limit);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) *status = 1u;
  else if (threadIdx.x == 0) *status = 0u;
}

}  // namespace

int check_wait_stats(const uint32_t *stats, cudaStream_t stream) {
  if (!stats) return PMGB_OK;
  uint32_t h[3] = {0, 0, 0};
  PMGB_CUDA(cudaMemcpyAsync(h, stats, sizeof(h), cudaMemcpyDeviceToHost, stream));
  PMGB_CUDA(cudaStreamSynchronize(stream));
  if (h[2] != 0)
    return fail(PMGB_ERR_CUDA,
                "an mbarrier wait of a tile-staged kernel reached its spin limit (a TMA copy "
                "did not arrive): the results of the calls since the counters were zeroed "
                "are invalid");
  return PMGB_OK;
}

int test_wait_timeout(uint32_t limit, uint32_t *status_dev, cudaStream_t stream) {
  wait_timeout_probe_kernel<<<1, 32, 0, stream>>>(limit, status_dev);
  PMGB_LAUNCHED("wait_timeout_probe_kernel");
  return PMGB_OK;
}

int make_tensor_map(CUtensorMap *map, const void *base, int rank, const uint64_t *dims,
                    const uint64_t *strides_bytes, const uint32_t *box) {
  PFN_cuTensorMapEncodeTiled_v12000 enc;
  PMGB_TRY(encoder(&enc));
  cuuint64_t d[5], s[4];
  cuuint32_t b[5], es[5];
  for (int i = 0; i < rank; ++i) {
    d[i] = dims[i];
    b[i] = box[i];
    es[i] = 1;
    if (i + 1 < rank) s[i] = strides_bytes[i];
  }
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)rank, const_cast<void *>(base),
                   d, s, b, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(PMGB_ERR_CUDA, "cuTensorMapEncodeTiled failed with CUresult " + std::to_string((int)r));
  return PMGB_OK;
}

}  // namespace pmgb
