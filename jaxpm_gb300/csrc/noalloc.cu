// Deterministic CIC paint that allocates nothing.
//
// The deterministic painter needs an 8-byte fixed-point accumulator per
// mesh cell.  pmgb_cic_paint_f32 takes that scratch from the caller's
// workspace; this variant keeps it in a file-scope device array instead,
// for callers that cannot hand out device memory: a framework whose custom
// call receives only the buffers its allocator created (XLA FFI handlers,
// plugins inside another runtime), or code that must not call cudaMalloc
// while the device memory is owned by someone else's pool.  The array is
// sized for meshes up to 128^3 cells (16 MiB).  With lazy module loading
// (the CUDA default since 12.2) a context takes those 16 MiB when this
// module is first used in it, i.e. at the first call; with
// CUDA_MODULE_LOADING=EAGER every context takes them when it is created.
// They are held until the context is destroyed.
#include <cudaTypedefs.h>

#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace pmgb {
namespace {

constexpr int64_t NOALLOC_MAX_CELLS = (int64_t)128 * 128 * 128;

static __device__ __align__(256) unsigned long long g_fixed_scratch[NOALLOC_MAX_CELLS];

std::mutex g_mu;
// Device addresses of g_fixed_scratch, one per CUDA context that used it,
// keyed by the context's unique id (cuCtxGetId): a device reset, or a caller
// that runs the library under its own (non-primary) context, gets a new id
// and so a fresh lookup instead of a stale or foreign address.
std::vector<std::pair<unsigned long long, unsigned long long *>> g_addr;
constexpr size_t MAX_CACHED_CONTEXTS = 64;
PFN_cuCtxGetCurrent_v4000 g_ctx_current = nullptr;
PFN_cuCtxGetId_v12000 g_ctx_id = nullptr;

int driver_fn(const char *name, int version, void **out) {
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion(name, out, version, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !*out)
    return fail(PMGB_ERR_UNSUPPORTED, std::string(name) + " is not available");
  return PMGB_OK;
}

int lookup(unsigned long long **out) {
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_fixed_scratch);
  if (e != cudaSuccess)
    return fail(PMGB_ERR_CUDA,
                std::string("cudaGetSymbolAddress(g_fixed_scratch): ") + cudaGetErrorString(e));
  *out = static_cast<unsigned long long *>(p);
  return PMGB_OK;
}

// The device address of g_fixed_scratch in the current context.  In host
// code the array's name only stands for the symbol, so the address is looked
// up (cudaGetSymbolAddress, with the context current) once per context and
// cached under its id.
int scratch_address(unsigned long long **out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ctx_current) {
    void *f = nullptr;
    PMGB_TRY(driver_fn("cuCtxGetCurrent", 4000, &f));
    g_ctx_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
    PMGB_TRY(driver_fn("cuCtxGetId", 12000, &f));
    g_ctx_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f);
  }
  CUcontext ctx = nullptr;
  if (g_ctx_current(&ctx) != CUDA_SUCCESS)
    return fail(PMGB_ERR_CUDA, "cuCtxGetCurrent failed");
  if (!ctx) {
    // no context bound yet: the runtime binds the device's primary context
    // on its first call that needs one (this lookup)
    unsigned long long *unused = nullptr;
    PMGB_TRY(lookup(&unused));
    if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx)
      return fail(PMGB_ERR_CUDA, "no CUDA context is current");
  }
  unsigned long long id = 0;
  if (g_ctx_id(ctx, &id) != CUDA_SUCCESS) return fail(PMGB_ERR_CUDA, "cuCtxGetId failed");
  for (const auto &e : g_addr)
    if (e.first == id) {
      *out = e.second;
      return PMGB_OK;
    }
  unsigned long long *addr = nullptr;
  PMGB_TRY(lookup(&addr));
  if (g_addr.size() >= MAX_CACHED_CONTEXTS) g_addr.erase(g_addr.begin());
  g_addr.emplace_back(id, addr);
  *out = addr;
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
