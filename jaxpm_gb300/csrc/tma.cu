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

}  // namespace

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
