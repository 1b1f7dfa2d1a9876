// Exported C ABI of libpmgb (declared in include/pmgb.h): argument checks,
// per-thread error messages, then a call into the kernels' host code.
#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "common.cuh"
#include "kernels.cuh"
#include "tma.cuh"

namespace pmgb {

namespace {
thread_local std::string t_err;
std::mutex g_sm_mu;
std::map<int, int> g_sm;
}  // namespace

std::atomic<uint64_t> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int fail(int code, const std::string &msg) {
  t_err = msg;
  return code;
}

void clear_error() { t_err.clear(); }

int sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  std::lock_guard<std::mutex> lk(g_sm_mu);
  auto it = g_sm.find(dev);
  if (it != g_sm.end()) return it->second;
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
    n = 148;
  g_sm[dev] = n;
  return n;
}

int64_t l2_bytes() {
  static std::mutex mu;
  static std::map<int, int64_t> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  int b = 0;
  if (cudaDeviceGetAttribute(&b, cudaDevAttrL2CacheSize, dev) != cudaSuccess || b < 0) b = 0;
  cache[dev] = b;
  return b;
}

int resident_ctas(const void *kernel, int threads, size_t smem) {
  static std::mutex mu;
  static std::map<std::tuple<const void *, int, int, size_t>, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return sm_count();
  const auto key = std::make_tuple(kernel, dev, threads, smem);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const int n = per_sm * sm_count();
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = n;
  return n;
}

int check_mesh(int nx, int ny, int nz) {
  const int lim = 1 << 24;
  if (nx <= 0 || ny <= 0 || nz <= 0 || nx >= lim || ny >= lim || nz >= lim)
    return fail(PMGB_ERR_INVALID_ARGUMENT,
                "mesh shape must be positive and below 2^24 per axis, got (" +
                    std::to_string(nx) + ", " + std::to_string(ny) + ", " +
                    std::to_string(nz) + ")");
  if ((double)nx * ny * nz >= 1099511627776.0)
    return fail(PMGB_ERR_INVALID_ARGUMENT, "mesh has 2^40 cells or more");
  return PMGB_OK;
}

}  // namespace pmgb

using namespace pmgb;

#define BEGIN() clear_error()
#define NEED(ptr) PMGB_REQUIRE((ptr) != nullptr, std::string(#ptr) + " is NULL")
#define NONNEG(np) PMGB_REQUIRE((np) >= 0, std::string(#np) + " is negative")

static int check_mode(int mode) {
  PMGB_REQUIRE(mode == PMGB_PAINT_ATOMIC || mode == PMGB_PAINT_BINNED ||
                   mode == PMGB_PAINT_DETERMINISTIC,
               "unknown paint mode " + std::to_string(mode));
  return PMGB_OK;
}

extern "C" {

int pmgb_version(void) { return 102; }

uint64_t pmgb_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

const char *pmgb_last_error(void) { return t_err.c_str(); }

size_t pmgb_cic_paint_workspace_size(int nx, int ny, int nz, int64_t np, int mode) {
  return paint_workspace_size(nx, ny, nz, np, mode);
}

int pmgb_cic_paint_f32(float *mesh, int nx, int ny, int nz, const float *pos, int64_t np,
                       const float *weights, float weight_scale, int mode, int accumulate,
                       void *workspace, size_t workspace_bytes, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_TRY(check_mode(mode));
  NONNEG(np);
  NEED(mesh);
  if (np > 0) NEED(pos);
  return paint(mesh, nx, ny, nz, pos, np, weights, weight_scale, mode, accumulate, workspace,
               workspace_bytes, stream);
}

int pmgb_cic_read_f32(const float *mesh, int nx, int ny, int nz, const float *pos, int64_t np,
                      float *out, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NONNEG(np);
  if (np == 0) return PMGB_OK;
  NEED(mesh);
  NEED(pos);
  NEED(out);
  return read(mesh, nx, ny, nz, pos, np, out, stream);
}

int pmgb_cic_read3_f32(const float *mesh3, int64_t comp_stride, int nx, int ny, int nz,
                       const float *pos, int64_t np, float *out3, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NONNEG(np);
  PMGB_REQUIRE(comp_stride >= (int64_t)nx * ny * nz, "comp_stride smaller than the mesh");
  if (np == 0) return PMGB_OK;
  NEED(mesh3);
  NEED(pos);
  NEED(out3);
  return read3(mesh3, comp_stride, nx, ny, nz, pos, np, out3, stream);
}

int pmgb_cic_weights_f32(const float *pos, int64_t np, int nx, int ny, int nz, int32_t *idx,
                         float *w, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NONNEG(np);
  if (np == 0) return PMGB_OK;
  NEED(pos);
  NEED(idx);
  NEED(w);
  return cic_weights(pos, np, nx, ny, nz, idx, w, stream);
}

int pmgb_cic_paint_vjp_f32(const float *g_mesh, int nx, int ny, int nz, const float *pos,
                           int64_t np, const float *weights, float weight_scale, float *g_pos,
                           float *g_w, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NONNEG(np);
  if (np == 0) return PMGB_OK;
  NEED(g_mesh);
  NEED(pos);
  return paint_vjp(g_mesh, nx, ny, nz, pos, np, weights, weight_scale, g_pos, g_w, stream);
}

int pmgb_cic_read_vjp_f32(const float *mesh, int nx, int ny, int nz, const float *pos,
                          int64_t np, const float *g_out, float *g_mesh, float *g_pos,
                          pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NONNEG(np);
  if (np == 0) return PMGB_OK;
  NEED(pos);
  NEED(g_out);
  if (g_pos) NEED(mesh);
  return read_vjp(mesh, nx, ny, nz, pos, np, g_out, g_mesh, g_pos, stream);
}

int pmgb_cic_paint_dx_f32(float *mesh, int nx, int ny, int nz, const float *disp,
                          const float *weights, float weight_scale, int accumulate,
                          pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NEED(mesh);
  NEED(disp);
  return paint_dx(mesh, nx, ny, nz, disp, weights, weight_scale, accumulate, stream);
}

int pmgb_cic_read_dx_f32(const float *mesh, int nx, int ny, int nz, const float *disp,
                         float *out, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NEED(mesh);
  NEED(disp);
  NEED(out);
  return read_dx(mesh, nx, ny, nz, disp, out, stream);
}

int pmgb_enmesh_f32(const float *disp, int nx, int ny, int nz, int32_t *idx, float *w,
                    pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NEED(disp);
  NEED(idx);
  NEED(w);
  return enmesh(disp, nx, ny, nz, idx, w, stream);
}

int pmgb_fft_r2c_f32(const float *in, void *out, int nx, int ny, int nz, int batch,
                     pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_REQUIRE(batch >= 1, "batch must be >= 1");
  NEED(in);
  NEED(out);
  return fft_r2c(in, out, nx, ny, nz, batch, stream);
}

int pmgb_fft_c2r_f32(void *in, float *out, int nx, int ny, int nz, int batch, int normalize,
                     pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_REQUIRE(batch >= 1, "batch must be >= 1");
  NEED(in);
  NEED(out);
  PMGB_TRY(fft_c2r(in, out, nx, ny, nz, batch, stream));
  if (normalize) {
    const int64_t n = (int64_t)nx * ny * nz;
    PMGB_TRY(scale_inplace(out, n * batch, 1.0f / (float)n, stream));
  }
  return PMGB_OK;
}

int pmgb_fft3_supported(int nx, int ny, int nz) {
  return spectral_supported(nx, ny, nz) ? 1 : 0;
}

int pmgb_fft3_pitch(int nz) { return nz > 0 ? spectral_pitch(nz) : 0; }

int pmgb_set_fft_path(int path) {
  BEGIN();
  PMGB_REQUIRE(path == PMGB_FFT_CUFFT || path == PMGB_FFT_FUSED || path == PMGB_FFT_OWN,
               "unknown FFT path");
  set_spectral(path);
  return PMGB_OK;
}

int pmgb_fft_path(void) { return spectral_mode(); }

int pmgb_set_run_timing(int enable) {
  BEGIN();
  PMGB_REQUIRE(enable == 0 || enable == 1, "enable must be 0 or 1");
  return set_run_timing(enable != 0);
}

int pmgb_run_timing(double *gather_ms, double *forces_ms, double *resort_ms, int *steps) {
  BEGIN();
  return run_timing(gather_ms, forces_ms, resort_ms, steps);
}

int pmgb_get_tuning(pmgb_tuning *out) {
  BEGIN();
  NEED(out);
  const Tuning t = tuning();
  *out = pmgb_tuning{};
  out->gather_static_quarters = t.gather_static_quarters;
  out->gather_ctas_per_sm = t.gather_ctas_per_sm;
  out->resort_ctas_per_sm = t.resort_ctas_per_sm;
  out->resort_priority = t.resort_priority;
  return PMGB_OK;
}

int pmgb_set_tuning(const pmgb_tuning *in) {
  BEGIN();
  NEED(in);
  PMGB_REQUIRE(in->gather_static_quarters >= 0 && in->gather_static_quarters <= 4,
               "gather_static_quarters must lie in [0, 4]");
  PMGB_REQUIRE(in->gather_ctas_per_sm >= 0 && in->gather_ctas_per_sm <= 32,
               "gather_ctas_per_sm must lie in [0, 32]");
  PMGB_REQUIRE(in->resort_ctas_per_sm >= 0 && in->resort_ctas_per_sm <= 32,
               "resort_ctas_per_sm must lie in [0, 32]");
  PMGB_REQUIRE(in->resort_priority == 0 || in->resort_priority == 1,
               "resort_priority must be 0 or 1");
  Tuning t;
  t.gather_static_quarters = in->gather_static_quarters;
  t.gather_ctas_per_sm = in->gather_ctas_per_sm;
  t.resort_ctas_per_sm = in->resort_ctas_per_sm;
  t.resort_priority = in->resort_priority;
  set_tuning(t);
  return PMGB_OK;
}

int pmgb_fft3_r2c_f32(const float *in, void *out, int nx, int ny, int nz, int batch,
                      pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_REQUIRE(batch >= 1, "batch must be >= 1");
  NEED(in);
  NEED(out);
  PMGB_REQUIRE(reinterpret_cast<uintptr_t>(in) % 16 == 0, "input must be 16-byte aligned");
  return spectral_r2c(in, out, nx, ny, nz, batch, stream);
}

int pmgb_fft3_c2r_f32(void *in, float *out, int nx, int ny, int nz, int batch,
                      pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_REQUIRE(batch >= 1, "batch must be >= 1");
  NEED(in);
  NEED(out);
  PMGB_REQUIRE(reinterpret_cast<uintptr_t>(out) % 16 == 0, "output must be 16-byte aligned");
  return spectral_c2r(in, out, nx, ny, nz, batch, stream);
}

static int check_kspace(int nx, int ny, int nz, int grad_order, int fd) {
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_REQUIRE(grad_order == 0 || grad_order == 1, "grad_order must be 0 or 1");
  PMGB_REQUIRE(fd == 0 || fd == 1, "fd_laplace must be 0 or 1");
  return PMGB_OK;
}

size_t pmgb_mesh_forces_workspace_size(int nx, int ny, int nz) {
  if (nx <= 0 || ny <= 0 || nz <= 0) return 0;
  return mesh_forces_workspace_size(nx, ny, nz);
}

int pmgb_mesh_forces_f32(const float *mesh, float *force3, int nx, int ny, int nz,
                         float r_split, void *workspace, size_t workspace_bytes,
                         pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NEED(mesh);
  NEED(force3);
  return mesh_forces_ws(mesh, force3, nx, ny, nz, r_split, workspace, workspace_bytes, stream);
}

int pmgb_mesh_potential_f32(const float *mesh, float *pot, int nx, int ny, int nz,
                            float r_split, void *workspace, size_t workspace_bytes,
                            pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NEED(mesh);
  NEED(pot);
  PMGB_REQUIRE(r_split >= 0.0f, "r_split must be non-negative");
  return mesh_potential_ws(mesh, pot, nx, ny, nz, r_split, workspace, workspace_bytes, stream);
}

int pmgb_mesh_forces_vjp_f32(const float *g_force3, float *g_mesh, int nx, int ny, int nz,
                             float r_split, void *workspace, size_t workspace_bytes,
                             pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NEED(g_force3);
  NEED(g_mesh);
  return mesh_forces_vjp_ws(g_force3, g_mesh, nx, ny, nz, r_split, workspace, workspace_bytes,
                            stream);
}

int pmgb_kspace_forces_f32(const void *delta_k, void *force_k, int64_t comp_stride, int nx,
                           int ny, int nz, float r_split, int grad_order, int fd_laplace,
                           float scale, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_kspace(nx, ny, nz, grad_order, fd_laplace));
  NEED(delta_k);
  NEED(force_k);
  PMGB_REQUIRE(comp_stride >= (int64_t)nx * ny * (nz / 2 + 1),
               "comp_stride smaller than the half spectrum");
  return kspace_forces(delta_k, force_k, comp_stride, nx, ny, nz, r_split, grad_order,
                       fd_laplace, scale, stream);
}

int pmgb_kspace_forces_vjp_f32(const void *g_force_k, int64_t comp_stride, void *g_delta_k,
                               int nx, int ny, int nz, float r_split, int grad_order,
                               int fd_laplace, float scale, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_kspace(nx, ny, nz, grad_order, fd_laplace));
  NEED(g_force_k);
  NEED(g_delta_k);
  PMGB_REQUIRE(comp_stride >= (int64_t)nx * ny * (nz / 2 + 1),
               "comp_stride smaller than the half spectrum");
  return kspace_forces_vjp(g_force_k, comp_stride, g_delta_k, nx, ny, nz, r_split, grad_order,
                           fd_laplace, scale, stream);
}

int pmgb_kspace_invlaplace_f32(void *spec, int nx, int ny, int nz, int fd_laplace, float scale,
                               pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_kspace(nx, ny, nz, 1, fd_laplace));
  NEED(spec);
  return kspace_invlaplace(spec, nx, ny, nz, fd_laplace, scale, stream);
}

int pmgb_kspace_longrange_f32(void *spec, int nx, int ny, int nz, float r_split,
                              pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NEED(spec);
  return kspace_longrange(spec, nx, ny, nz, r_split, stream);
}

int pmgb_kspace_gradient_f32(const void *in, void *out, int nx, int ny, int nz, int direction,
                             int grad_order, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_kspace(nx, ny, nz, grad_order, 0));
  PMGB_REQUIRE(direction >= 0 && direction < 3, "direction must be 0, 1 or 2");
  NEED(in);
  NEED(out);
  return kspace_gradient(in, out, nx, ny, nz, direction, grad_order, stream);
}

int pmgb_read3_kick_drift_f32(const float *force3, int64_t comp_stride, int nx, int ny, int nz,
                              float *pos, float *vel, int64_t np, float kick, float drift,
                              float *forces_out, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NONNEG(np);
  PMGB_REQUIRE(comp_stride >= (int64_t)nx * ny * nz, "comp_stride smaller than the mesh");
  if (np == 0) return PMGB_OK;
  NEED(force3);
  NEED(pos);
  NEED(vel);
  return read3_kick_drift(force3, comp_stride, nx, ny, nz, pos, vel, np, kick, drift,
                          forces_out, stream);
}

int pmgb_kick_f32(float *vel, const float *forces, int64_t np, float k, pmgb_stream_t stream) {
  BEGIN();
  NONNEG(np);
  if (np == 0) return PMGB_OK;
  NEED(vel);
  NEED(forces);
  return kick(vel, forces, np, k, stream);
}

int pmgb_drift_f32(float *pos, const float *vel, int64_t np, float d, pmgb_stream_t stream) {
  BEGIN();
  NONNEG(np);
  if (np == 0) return PMGB_OK;
  NEED(pos);
  NEED(vel);
  return drift(pos, vel, np, d, stream);
}

size_t pmgb_pm_workspace_size(int nx, int ny, int nz, int64_t np, int paint_mode) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || np < 0) return 0;
  return pm_workspace_size(nx, ny, nz, np, paint_mode);
}

int pmgb_pm_forces_f32(const float *pos, int64_t np, int nx, int ny, int nz, float r_split,
                       int paint_mode, float *forces, void *workspace, size_t workspace_bytes,
                       pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_TRY(check_mode(paint_mode));
  NONNEG(np);
  if (np > 0) {
    NEED(pos);
    NEED(forces);
  }
  return pm_forces(pos, np, nx, ny, nz, r_split, paint_mode, forces, workspace, workspace_bytes,
                   stream);
}

int pmgb_fpm_step_f32(float *pos, float *vel, int64_t np, int nx, int ny, int nz, float kick,
                      float drift, float r_split, int paint_mode, void *workspace,
                      size_t workspace_bytes, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_TRY(check_mode(paint_mode));
  NONNEG(np);
  if (np > 0) {
    NEED(pos);
    NEED(vel);
  }
  return fpm_step(pos, vel, np, nx, ny, nz, kick, drift, r_split, paint_mode, workspace,
                  workspace_bytes, stream);
}

int pmgb_fpm_step_plain_f32(float *pos, float *vel, int64_t np, int nx, int ny, int nz,
                            float kick, float drift, float r_split, void *workspace,
                            size_t workspace_bytes, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NONNEG(np);
  if (np > 0) {
    NEED(pos);
    NEED(vel);
  }
  return fpm_step_plain(pos, vel, np, nx, ny, nz, kick, drift, r_split, workspace,
                        workspace_bytes, stream);
}

int pmgb_pm_forces_vjp_f32(const float *pos, int64_t np, int nx, int ny, int nz, float r_split,
                           int paint_mode, const float *g_forces, float *g_pos,
                           void *workspace, size_t workspace_bytes, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_TRY(check_mode(paint_mode));
  NONNEG(np);
  if (np > 0) {
    NEED(pos);
    NEED(g_forces);
    NEED(g_pos);
  }
  return pm_forces_vjp(pos, np, nx, ny, nz, r_split, paint_mode, g_forces, g_pos, workspace,
                       workspace_bytes, stream);
}

size_t pmgb_tile_sort_workspace_size(int nx, int ny, int nz, int64_t np) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || np < 0) return 0;
  return sort_workspace_size(nx, ny, nz, np);
}

static int check_sortable(int nx, int ny, int nz, int64_t np) {
  PMGB_TRY(check_mesh(nx, ny, nz));
  NONNEG(np);
  PMGB_REQUIRE(np < (int64_t)UINT32_MAX, "the sorted path indexes particles with 32 bits");
  PMGB_REQUIRE(tile_key_count(nx, ny, nz) <= ((int64_t)1 << 24),
               "the sorted path supports at most 256 tiles (2048 cells) per axis");
  return PMGB_OK;
}

int pmgb_tile_sort_f32(const float *pos, const float *vel, const uint32_t *id, int64_t np, int nx,
                       int ny, int nz, float *pos_out, float *vel_out, uint32_t *id_out,
                       void *workspace, size_t workspace_bytes, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  if (np == 0) return PMGB_OK;
  NEED(pos);
  NEED(pos_out);
  NEED(id_out);
  PMGB_REQUIRE((vel == nullptr) == (vel_out == nullptr), "vel and vel_out must both be given");
  PMGB_REQUIRE(pos != pos_out && (!vel || vel != vel_out) && (!id || id != id_out),
               "the sort cannot run in place");
  return tile_sort(pos, vel, id, np, nx, ny, nz, pos_out, vel_out, id_out, workspace,
                   workspace_bytes, stream);
}

int pmgb_unpermute3_f32(const float *in, const uint32_t *id, int64_t np, float *out,
                        pmgb_stream_t stream) {
  BEGIN();
  NONNEG(np);
  if (np == 0) return PMGB_OK;
  NEED(in);
  NEED(id);
  NEED(out);
  PMGB_REQUIRE(in != out, "unpermute cannot run in place");
  return unpermute3(in, id, np, out, stream);
}

int pmgb_tile_sort_dest_f32(const float *pos, const float *vel, const uint32_t *id, int64_t np,
                            int nx, int ny, int nz, float *pos_out, float *vel_out,
                            uint32_t *id_out, uint32_t *dest, void *workspace,
                            size_t workspace_bytes, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  if (np == 0) return PMGB_OK;
  NEED(pos);
  NEED(pos_out);
  NEED(id_out);
  NEED(dest);
  PMGB_REQUIRE((vel == nullptr) == (vel_out == nullptr), "vel and vel_out must both be given");
  PMGB_REQUIRE(pos != pos_out && (!vel || vel != vel_out) && (!id || id != id_out),
               "the sort cannot run in place");
  return tile_sort(pos, vel, id, np, nx, ny, nz, pos_out, vel_out, id_out, workspace,
                   workspace_bytes, stream, dest);
}

int pmgb_gather3_f32(const float *in, int64_t n_in, const uint32_t *idx, int64_t n, float *out,
                     pmgb_stream_t stream) {
  BEGIN();
  NONNEG(n_in);
  NONNEG(n);
  if (n == 0) return PMGB_OK;
  NEED(in);
  NEED(idx);
  NEED(out);
  PMGB_REQUIRE(out + 3 * n <= in || in + 3 * n_in <= out, "the gather cannot overlap its source");
  return gather3(in, n_in, idx, n, out, stream);
}

int pmgb_permute3_f32(const float *in, const uint32_t *id, int64_t np, float *out,
                      pmgb_stream_t stream) {
  BEGIN();
  NONNEG(np);
  if (np == 0) return PMGB_OK;
  NEED(in);
  NEED(id);
  NEED(out);
  PMGB_REQUIRE(in != out, "permute cannot run in place");
  return permute3(in, id, np, out, stream);
}

int pmgb_read3_kick_drift_binned_f32(const float *force3, int64_t comp_stride, int nx, int ny,
                                     int nz, float *pos, float *vel, int64_t np, float kick,
                                     float drift, void *sort_workspace,
                                     size_t sort_workspace_bytes, uint32_t *stats,
                                     pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  PMGB_REQUIRE(comp_stride >= (int64_t)nx * ny * nz, "comp_stride smaller than the mesh");
  if (np == 0) return PMGB_OK;
  NEED(force3);
  NEED(pos);
  NEED(vel);
  NEED(sort_workspace);
  return rkd_sorted(force3, comp_stride, nx, ny, nz, pos, pos, vel, np, kick, drift,
                    sort_workspace, sort_workspace_bytes, stats, stream);
}

int pmgb_read3_kick_drift_paint_binned_f32(const float *force3, int64_t comp_stride, int nx,
                                           int ny, int nz, float *pos, float *vel, int64_t np,
                                           float kick, float drift, float *mesh_next,
                                           void *sort_workspace, size_t sort_workspace_bytes,
                                           uint32_t *stats, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  PMGB_REQUIRE(comp_stride >= (int64_t)nx * ny * nz, "comp_stride smaller than the mesh");
  NEED(mesh_next);
  if (np == 0) {
    PMGB_CUDA(cudaMemsetAsync(mesh_next, 0, (size_t)nx * ny * nz * sizeof(float), stream));
    return PMGB_OK;
  }
  NEED(force3);
  NEED(pos);
  NEED(vel);
  NEED(sort_workspace);
  PMGB_REQUIRE(mesh_next != force3, "mesh_next must not alias the force meshes");
  return rkd_sorted(force3, comp_stride, nx, ny, nz, pos, pos, vel, np, kick, drift,
                    sort_workspace, sort_workspace_bytes, stats, stream, mesh_next);
}

int pmgb_read_potential_kick_drift_paint_binned_f32(const float *pot, int nx, int ny, int nz,
                                                    float *pos, float *vel, int64_t np,
                                                    float kick, float drift, float *mesh_next,
                                                    void *sort_workspace,
                                                    size_t sort_workspace_bytes, uint32_t *stats,
                                                    pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  if (np == 0) {
    if (mesh_next)
      PMGB_CUDA(cudaMemsetAsync(mesh_next, 0, (size_t)nx * ny * nz * sizeof(float), stream));
    return PMGB_OK;
  }
  NEED(pot);
  NEED(pos);
  NEED(vel);
  NEED(sort_workspace);
  PMGB_REQUIRE(mesh_next != pot, "mesh_next must not alias the potential");
  return rkd_sorted(pot, (int64_t)nx * ny * nz, nx, ny, nz, pos, pos, vel, np, kick, drift,
                    sort_workspace, sort_workspace_bytes, stats, stream, mesh_next, true);
}

int pmgb_read_potential_kick_drift_paint_perm_f32(
    const float *pot, int nx, int ny, int nz, const float *pos, const float *vel,
    const uint32_t *perm, float *pos_out, float *vel_out, int64_t np, float kick, float drift,
    float *mesh_next, void *sort_workspace, size_t sort_workspace_bytes, uint32_t *stats,
    pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  if (np == 0) {
    if (mesh_next)
      PMGB_CUDA(cudaMemsetAsync(mesh_next, 0, (size_t)nx * ny * nz * sizeof(float), stream));
    return PMGB_OK;
  }
  NEED(pot);
  NEED(pos);
  NEED(vel);
  NEED(pos_out);
  NEED(vel_out);
  NEED(sort_workspace);
  PMGB_REQUIRE(mesh_next != pot, "mesh_next must not alias the potential");
  if (perm)
    PMGB_REQUIRE(pos_out != pos && vel_out != vel,
                 "with a permutation the outputs must not alias the inputs");
  else
    PMGB_REQUIRE((pos_out == pos) == (vel_out == vel),
                 "without a permutation the outputs alias both inputs or neither");
  PMGB_TRY(check_sort_workspace(sort_workspace, sort_workspace_bytes, nx, ny, nz, np));
  PermIO io;
  io.perm = perm;
  io.vel_out = vel_out;
  perm_scratch(sort_workspace, nx, ny, nz, np, &io);
  return rkd_sorted(pot, (int64_t)nx * ny * nz, nx, ny, nz, pos, pos_out,
                    const_cast<float *>(vel), np, kick, drift, sort_workspace,
                    sort_workspace_bytes, stats, stream, mesh_next, true, io);
}

int pmgb_tile_resort_index(int64_t np, int nx, int ny, int nz, const uint32_t *perm_old,
                           uint32_t *perm_new, const uint32_t *id_in, uint32_t *id_out,
                           void *sort_workspace, size_t sort_workspace_bytes,
                           pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  NEED(sort_workspace);
  if (np > 0) NEED(perm_new);
  if (np > 0 && perm_old) {
    NEED(id_in);
    NEED(id_out);
    PMGB_REQUIRE(perm_old != perm_new && id_in != id_out,
                 "perm_old/perm_new and id_in/id_out must be distinct buffers");
  }
  return index_resort(np, nx, ny, nz, perm_old, perm_new, perm_old ? id_in : nullptr,
                      perm_old ? id_out : nullptr, sort_workspace, sort_workspace_bytes,
                      stream);
}

int pmgb_gather_u32(const uint32_t *in, const uint32_t *idx, int64_t np, uint32_t *out,
                    pmgb_stream_t stream) {
  BEGIN();
  PMGB_REQUIRE(np >= 0, "np is negative");
  if (np == 0) return PMGB_OK;
  NEED(in);
  NEED(idx);
  NEED(out);
  PMGB_REQUIRE(in != out, "in and out must be distinct buffers");
  return gather_u32(in, idx, np, out, stream);
}

static int run_sorted_record(float *xs, float *vel_a, uint32_t *id_a, float *vel_b,
                             uint32_t *id_b, float *pos_out, int64_t np, int nx, int ny, int nz,
                             int n_steps, const float *kick, const float *drift, float r_split,
                             void *workspace, size_t workspace_bytes, void *sort_workspace,
                             size_t sort_workspace_bytes, float *force3s, uint32_t *dests,
                             uint32_t *offsets, uint32_t *stats, pmgb_stream_t stream, bool pot) {
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  PMGB_REQUIRE(n_steps >= 0, "n_steps is negative");
  PMGB_REQUIRE(r_split >= 0.0f, "r_split must be non-negative");
  if (n_steps == 0) return PMGB_OK;
  NEED(xs);
  NEED(vel_a);
  NEED(id_a);
  NEED(vel_b);
  NEED(id_b);
  NEED(pos_out);
  NEED(kick);
  NEED(drift);
  NEED(sort_workspace);
  NEED(force3s);
  NEED(dests);
  NEED(offsets);
  return fpm_run_sorted_record(xs, vel_a, id_a, vel_b, id_b, pos_out, np, nx, ny, nz, n_steps,
                               kick, drift, r_split, workspace, workspace_bytes, sort_workspace,
                               sort_workspace_bytes, force3s, dests, offsets, stats, stream, pot);
}

int pmgb_fpm_run_sorted_record_f32(float *xs, float *vel_a, uint32_t *id_a, float *vel_b,
                                   uint32_t *id_b, float *pos_out, int64_t np, int nx, int ny,
                                   int nz, int n_steps, const float *kick, const float *drift,
                                   float r_split, void *workspace, size_t workspace_bytes,
                                   void *sort_workspace, size_t sort_workspace_bytes,
                                   float *force3s, uint32_t *dests, uint32_t *offsets,
                                   uint32_t *stats, pmgb_stream_t stream) {
  BEGIN();
  return run_sorted_record(xs, vel_a, id_a, vel_b, id_b, pos_out, np, nx, ny, nz, n_steps, kick,
                           drift, r_split, workspace, workspace_bytes, sort_workspace,
                           sort_workspace_bytes, force3s, dests, offsets, stats, stream, false);
}

int pmgb_fpm_run_sorted_record_pot_f32(float *xs, float *vel_a, uint32_t *id_a, float *vel_b,
                                       uint32_t *id_b, float *pos_out, int64_t np, int nx,
                                       int ny, int nz, int n_steps, const float *kick,
                                       const float *drift, float r_split, void *workspace,
                                       size_t workspace_bytes, void *sort_workspace,
                                       size_t sort_workspace_bytes, float *potentials,
                                       uint32_t *dests, uint32_t *offsets, uint32_t *stats,
                                       pmgb_stream_t stream) {
  BEGIN();
  return run_sorted_record(xs, vel_a, id_a, vel_b, id_b, pos_out, np, nx, ny, nz, n_steps, kick,
                           drift, r_split, workspace, workspace_bytes, sort_workspace,
                           sort_workspace_bytes, potentials, dests, offsets, stats, stream, true);
}

int pmgb_fpm_run_sorted_f32(float *pos_a, float *vel_a, uint32_t *id_a, float *pos_b,
                            float *vel_b, uint32_t *id_b, int64_t np, int nx, int ny, int nz,
                            int n_steps, const float *kick, const float *drift, float r_split,
                            void *workspace, size_t workspace_bytes, void *sort_workspace,
                            size_t sort_workspace_bytes, uint32_t *stats,
                            pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  PMGB_REQUIRE(n_steps >= 0, "n_steps is negative");
  if (n_steps == 0) return PMGB_OK;
  NEED(kick);
  NEED(drift);
  if (np > 0) {
    NEED(pos_a);
    NEED(vel_a);
    NEED(id_a);
    NEED(pos_b);
    NEED(vel_b);
    NEED(id_b);
    PMGB_REQUIRE(pos_a != pos_b && vel_a != vel_b && id_a != id_b,
                 "the two state buffers must be distinct");
  }
  return fpm_run_sorted(pos_a, vel_a, id_a, pos_b, vel_b, id_b, np, nx, ny, nz, n_steps, kick,
                        drift, r_split, workspace, workspace_bytes, sort_workspace,
                        sort_workspace_bytes, stats, stream);
}

int pmgb_check_stats(const uint32_t *stats, pmgb_stream_t stream) {
  BEGIN();
  return check_wait_stats(stats, stream);
}

int pmgb_test_wait_timeout(uint32_t spin_limit, uint32_t *status, pmgb_stream_t stream) {
  BEGIN();
  NEED(status);
  PMGB_REQUIRE(spin_limit >= 1 && spin_limit <= (1u << 20),
               "spin_limit must lie in [1, 2^20]");
  return test_wait_timeout(spin_limit, status, stream);
}

int pmgb_cic_paint_sorted_f32(float *mesh, int nx, int ny, int nz, const float *pos,
                              int64_t np, void *sort_workspace, size_t sort_workspace_bytes,
                              uint32_t *stats, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  NEED(mesh);
  NEED(sort_workspace);
  if (np > 0) NEED(pos);
  return paint_sorted(mesh, nx, ny, nz, pos, np, sort_workspace, sort_workspace_bytes, stats,
                      stream);
}

int pmgb_tile_scatter_f32(const float *pos, const float *vel, const uint32_t *id, int64_t np,
                          int nx, int ny, int nz, float *pos_out, float *vel_out,
                          uint32_t *id_out, uint32_t *dest_out, void *sort_workspace,
                          size_t sort_workspace_bytes, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  if (np > 0) {
    NEED(pos);
    NEED(pos_out);
    NEED(id_out);
    PMGB_REQUIRE((vel == nullptr) == (vel_out == nullptr), "vel and vel_out must both be given");
    PMGB_REQUIRE(pos != pos_out && (!vel || vel != vel_out) && (!id || id != id_out),
                 "the scatter cannot run in place");
  }
  return tile_scatter(pos, vel, id, np, nx, ny, nz, pos_out, vel_out, id_out, dest_out,
                      sort_workspace, sort_workspace_bytes, stream);
}

int pmgb_fpm_step_sorted_f32(const float *pos, float *vel, const uint32_t *id, float *pos_out,
                             float *vel_out,
                             uint32_t *id_out, int64_t np, int nx, int ny, int nz, float kick,
                             float drift, float r_split, void *workspace, size_t workspace_bytes,
                             void *sort_workspace, size_t sort_workspace_bytes,
                             float *force3_out, uint32_t *dest_out, uint32_t *offsets_out,
                             uint32_t *stats, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  if (np > 0) {
    NEED(pos);
    NEED(vel);
    NEED(id);
    NEED(pos_out);
    NEED(vel_out);
    NEED(id_out);
    PMGB_REQUIRE(pos != pos_out && vel != vel_out && id != id_out,
                 "the sorted step writes to separate output buffers");
  }
  return fpm_step_sorted(pos, vel, id, pos_out, vel_out, id_out, np, nx, ny, nz, kick, drift,
                         r_split, workspace, workspace_bytes, sort_workspace,
                         sort_workspace_bytes, force3_out, dest_out, offsets_out, stats, stream);
}

int64_t pmgb_tile_key_count(int nx, int ny, int nz) {
  if (nx <= 0 || ny <= 0 || nz <= 0) return 0;
  return tile_key_count(nx, ny, nz);
}

static int step_sorted_vjp(const float *pos, const float *force3, const uint32_t *dest,
                           const uint32_t *tile_offsets, const float *g_pos_in,
                           const float *g_vel_in, float *g_pos_out, float *g_vel_out, int64_t np,
                           int nx, int ny, int nz, float kick, float drift, float r_split,
                           void *workspace, size_t workspace_bytes, uint32_t *stats,
                           pmgb_stream_t stream, bool pot) {
  PMGB_TRY(check_sortable(nx, ny, nz, np));
  NEED(force3);
  NEED(tile_offsets);
  if (np > 0) {
    NEED(pos);
    NEED(g_pos_in);
    NEED(g_vel_in);
    NEED(g_pos_out);
    NEED(g_vel_out);
    PMGB_REQUIRE(g_pos_in != g_pos_out && g_vel_in != g_vel_out && g_pos_out != g_vel_out,
                 "the reverse step writes to separate output buffers");
  }
  return fpm_step_sorted_vjp(pos, force3, dest, tile_offsets, g_pos_in, g_vel_in, g_pos_out,
                             g_vel_out, np, nx, ny, nz, kick, drift, r_split, workspace,
                             workspace_bytes, stats, stream, pot);
}

int pmgb_fpm_step_sorted_vjp_f32(const float *pos, const float *force3, const uint32_t *dest,
                                 const uint32_t *tile_offsets, const float *g_pos_in,
                                 const float *g_vel_in, float *g_pos_out, float *g_vel_out,
                                 int64_t np, int nx, int ny, int nz, float kick, float drift,
                                 float r_split, void *workspace, size_t workspace_bytes,
                                 uint32_t *stats, pmgb_stream_t stream) {
  BEGIN();
  return step_sorted_vjp(pos, force3, dest, tile_offsets, g_pos_in, g_vel_in, g_pos_out,
                         g_vel_out, np, nx, ny, nz, kick, drift, r_split, workspace,
                         workspace_bytes, stats, stream, false);
}

int pmgb_fpm_coef_cotangents_f32(const float *pos, const float *pos_next, const uint32_t *dest,
                                  const float *force3, int64_t comp_stride, int nx, int ny,
                                  int nz, const float *g_pos_next, const float *g_vel,
                                  int64_t np, double *out, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NONNEG(np);
  if (np == 0) return PMGB_OK;
  NEED(pos);
  NEED(pos_next);
  NEED(force3);
  NEED(g_pos_next);
  NEED(g_vel);
  NEED(out);
  PMGB_REQUIRE(comp_stride >= (int64_t)nx * ny * nz,
               "comp_stride must be at least nx*ny*nz");
  return coef_cotangents(pos, pos_next, dest, force3, comp_stride, nx, ny, nz, g_pos_next,
                         g_vel, np, out, stream);
}

int pmgb_fpm_step_sorted_vjp_pot_f32(const float *pos, const float *potential,
                                     const uint32_t *dest, const uint32_t *tile_offsets,
                                     const float *g_pos_in, const float *g_vel_in,
                                     float *g_pos_out, float *g_vel_out, int64_t np, int nx,
                                     int ny, int nz, float kick, float drift, float r_split,
                                     void *workspace, size_t workspace_bytes, uint32_t *stats,
                                     pmgb_stream_t stream) {
  BEGIN();
  return step_sorted_vjp(pos, potential, dest, tile_offsets, g_pos_in, g_vel_in, g_pos_out,
                         g_vel_out, np, nx, ny, nz, kick, drift, r_split, workspace,
                         workspace_bytes, stats, stream, true);
}

int pmgb_linear_field_colour_f32(void *spec, int nx, int ny, int nz, float box_x, float box_y,
                                 float box_z, const float *table_k, const float *table_p,
                                 int n_table, float scale, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_REQUIRE(box_x > 0 && box_y > 0 && box_z > 0, "box lengths must be positive");
  PMGB_REQUIRE(n_table >= 2, "the power table needs at least two entries");
  NEED(spec);
  NEED(table_k);
  NEED(table_p);
  return linear_field_colour(spec, nx, ny, nz, box_x, box_y, box_z, table_k, table_p, n_table,
                             scale, stream);
}

size_t pmgb_lpt2_source_workspace_size(int nx, int ny, int nz) {
  if (nx <= 0 || ny <= 0 || nz <= 0) return 0;
  return lpt2_source_workspace_size(nx, ny, nz);
}

int pmgb_lpt2_source_vjp_f32(const float *ic, const float *g_delta2, float *g_ic, int nx, int ny,
                             int nz, void *workspace, size_t workspace_bytes,
                             pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NEED(ic);
  NEED(g_delta2);
  NEED(g_ic);
  return lpt2_source_vjp(ic, g_delta2, g_ic, nx, ny, nz, workspace, workspace_bytes, stream);
}

int pmgb_lpt2_source_f32(const void *delta_k, float *delta2, int nx, int ny, int nz,
                         void *workspace, size_t workspace_bytes, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  NEED(delta_k);
  NEED(delta2);
  return lpt2_source(delta_k, delta2, nx, ny, nz, workspace, workspace_bytes, stream);
}

int pmgb_lpt_combine_f32(const float *a, const float *b, int64_t n, float ca, float cb,
                         float *out, pmgb_stream_t stream) {
  BEGIN();
  NONNEG(n);
  if (n == 0) return PMGB_OK;
  NEED(a);
  NEED(out);
  return lpt_combine(a, b, n, ca, cb, out, stream);
}

int pmgb_power_spectrum_f32(const void *spec, int nx, int ny, int nz, double box_x, double box_y,
                            double box_z, const double *kedges, int n_edges, double *psum,
                            double *pcount, double *ksum, pmgb_stream_t stream) {
  BEGIN();
  PMGB_TRY(check_mesh(nx, ny, nz));
  PMGB_REQUIRE(n_edges >= 1 && n_edges <= 2000, "n_edges must be in 1..2000");
  PMGB_REQUIRE(box_x > 0 && box_y > 0 && box_z > 0, "box lengths must be positive");
  NEED(spec);
  NEED(kedges);
  NEED(psum);
  NEED(pcount);
  NEED(ksum);
  return power_spectrum(spec, nx, ny, nz, box_x, box_y, box_z, kedges, n_edges, psum, pcount,
                        ksum, stream);
}

size_t pmgb_batch_workspace_size(const pmgb_sim *sims, int n_sims) {
  BEGIN();
  return batch_workspace_size(sims, n_sims);
}

int pmgb_batch_init(const pmgb_sim *sims, int n_sims, void *workspace, size_t workspace_bytes,
                    pmgb_stream_t stream) {
  BEGIN();
  return batch_init(sims, n_sims, workspace, workspace_bytes, stream);
}

int pmgb_batch_release(const void *workspace) {
  BEGIN();
  return batch_release(workspace);
}

int pmgb_batch_counts(const pmgb_sim *sims, int n_sims, int64_t *np_total, int64_t *cells_total) {
  BEGIN();
  return batch_counts(sims, n_sims, np_total, cells_total);
}

int pmgb_cic_paint_batched_f32(const pmgb_sim *sims, int n_sims, float *meshes, const float *pos,
                               void *workspace, size_t workspace_bytes, pmgb_stream_t stream) {
  BEGIN();
  NEED(meshes);
  NEED(pos);
  return cic_paint_batched(sims, n_sims, meshes, pos, workspace, workspace_bytes, stream);
}

int pmgb_pm_forces_batched_f32(const pmgb_sim *sims, int n_sims, const float *pos, float *forces,
                               float r_split, void *workspace, size_t workspace_bytes,
                               pmgb_stream_t stream) {
  BEGIN();
  NEED(pos);
  NEED(forces);
  PMGB_REQUIRE(r_split >= 0.0f, "r_split must be non-negative");
  return pm_forces_batched(sims, n_sims, pos, forces, r_split, workspace, workspace_bytes,
                           stream);
}

int pmgb_fpm_step_batched_f32(const pmgb_sim *sims, int n_sims, float *pos, float *vel,
                              const float *kick, const float *drift, float r_split,
                              float *pos_before, void *workspace, size_t workspace_bytes,
                              pmgb_stream_t stream) {
  BEGIN();
  NEED(pos);
  NEED(vel);
  NEED(kick);
  NEED(drift);
  PMGB_REQUIRE(r_split >= 0.0f, "r_split must be non-negative");
  return fpm_step_batched(sims, n_sims, pos, vel, kick, drift, r_split, pos_before, workspace,
                          workspace_bytes, stream);
}

int pmgb_fpm_step_batched_vjp_f32(const pmgb_sim *sims, int n_sims, const float *pos,
                                  float *g_pos, float *g_vel, const float *kick,
                                  const float *drift, float r_split, void *workspace,
                                  size_t workspace_bytes, pmgb_stream_t stream) {
  BEGIN();
  NEED(pos);
  NEED(g_pos);
  NEED(g_vel);
  NEED(kick);
  NEED(drift);
  PMGB_REQUIRE(r_split >= 0.0f, "r_split must be non-negative");
  return fpm_step_batched_vjp(sims, n_sims, pos, g_pos, g_vel, kick, drift, r_split, workspace,
                              workspace_bytes, stream);
}

size_t pmgb_npy_header(const char *descr, const int64_t *shape, int ndim, char *buf,
                       size_t cap) {
  BEGIN();
  if (!descr || ndim < 0 || ndim > 32 || (ndim > 0 && !shape)) return 0;
  return npy_header(descr, shape, ndim, buf, cap);
}

int pmgb_snapshot_begin_npy(const char *path, const void *array, const char *descr,
                            int itemsize, const int64_t *shape, int ndim, void *staging,
                            size_t staging_bytes, pmgb_stream_t stream,
                            pmgb_snapshot **snapshot) {
  BEGIN();
  NEED(path);
  NEED(array);
  NEED(descr);
  NEED(snapshot);
  PMGB_REQUIRE(ndim >= 0 && ndim <= 32, "ndim must be in 0..32");
  PMGB_REQUIRE(ndim == 0 || shape != nullptr, "shape is NULL");
  PMGB_REQUIRE(itemsize > 0 && itemsize <= 16, "itemsize must be in 1..16");
  return snapshot_begin_npy(path, array, descr, itemsize, shape, ndim, staging, staging_bytes,
                            stream, reinterpret_cast<Snapshot **>(snapshot));
}

int pmgb_snapshot_wait(pmgb_snapshot *snapshot) {
  BEGIN();
  return snapshot_wait(reinterpret_cast<Snapshot *>(snapshot));
}

}  // extern "C"
