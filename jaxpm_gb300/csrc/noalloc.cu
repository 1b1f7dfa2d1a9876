// Deterministic CIC paint that allocates nothing.
//
// The deterministic painter needs an 8-byte fixed-point accumulator per
// mesh cell.  pmgb_cic_paint_f32 takes that scratch from the caller's
// workspace; this variant keeps it in a file-scope device array instead,
// for callers that cannot hand out device memory: a framework whose custom
// call receives only the buffers its allocator created (XLA FFI handlers,
// plugins inside another runtime), or code that must not call cudaMalloc
// while the device memory is owned by someone else's pool.  The array is
// sized for meshes up to 128^3 cells (16 MiB, held by every GPU that loads
// the library until the process exits).
#include <mutex>
#include <string>

#include "common.cuh"
#include "kernels.cuh"

namespace pmgb {
namespace {

constexpr int64_t NOALLOC_MAX_CELLS = (int64_t)128 * 128 * 128;

static __device__ __align__(256) unsigned long long g_fixed_scratch[NOALLOC_MAX_CELLS];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
unsigned long long *g_scratch_addr[MAX_DEVICES] = {nullptr};

// The device address of g_fixed_scratch on the current device.  In host code
// the array's name only stands for the symbol, so the address is looked up
// once per device (with that device current) and cached.
int scratch_address(unsigned long long **out) {
  int dev = 0;
  PMGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES)
    return fail(PMGB_ERR_UNSUPPORTED, "device index beyond the scratch table");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_fixed_scratch);
    if (e != cudaSuccess)
      return fail(PMGB_ERR_CUDA,
                  std::string("cudaGetSymbolAddress(g_fixed_scratch): ") + cudaGetErrorString(e));
    g_scratch_addr[dev] = static_cast<unsigned long long *>(p);
  }
  *out = g_scratch_addr[dev];
  return PMGB_OK;
}

}  // namespace
}  // namespace pmgb

using namespace pmgb;

extern "C" int pmgb_cic_paint_deterministic_noalloc_f32(float *mesh, int nx, int ny, int nz,
                                                        const float *pos, int64_t np,
                                                        const float *weights,
                                                        float weight_scale, int accumulate,
                                                        pmgb_stream_t stream) {
  clear_error();
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_REQUIRE(np >= 0, "np is negative");
  PMGB_REQUIRE(mesh != nullptr, "mesh is NULL");
  if (np > 0) PMGB_REQUIRE(pos != nullptr, "pos is NULL");
  const int64_t ncell = (int64_t)nx * ny * nz;
  if (ncell > NOALLOC_MAX_CELLS)
    return fail(PMGB_ERR_INVALID_ARGUMENT,
                "pmgb_cic_paint_deterministic_noalloc_f32 handles at most " +
                    std::to_string(NOALLOC_MAX_CELLS) + " cells (128^3); got " +
                    std::to_string(ncell) + "; use pmgb_cic_paint_f32 with a workspace");
  unsigned long long *acc = nullptr;
  PMGB_TRY(scratch_address(&acc));
  return paint_fixed_into(acc, mesh, nx, ny, nz, pos, np, weights, weight_scale, accumulate,
                          stream);
}
