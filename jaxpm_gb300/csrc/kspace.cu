// Fourier-space operators on half spectra [nx][ny][nz/2+1] (complex64).
//
// Reference: jaxpm/pm.py:49-56 (pot_k = delta_k * invlaplace * longrange;
// force_k_i = -gradient_kernel(kvec, i) * pot_k) with the kernels of
// jaxpm/kernels.py:41-115 and wave numbers 2*pi*fftfreq(n) (fftk,
// kernels.py:10-23).  Per-axis quantities (w, w^2, the order-1 and order-0
// gradient factors and the finite-difference w^2) are tabulated once per
// (device, n) in float32 with the reference's operation order, so the
// per-element work is a few multiplies: the fused kernel reads delta_k once
// and writes the three force spectra, 32 bytes per complex element.
#include <cmath>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "kspace.cuh"

namespace pmgb {
namespace {

std::mutex g_mu;
std::map<std::pair<int, int>, AxisEntry *> g_tables;

// Builds (once) and returns the device table for an axis of length n.
int axis_table(int n, const AxisEntry **out) {
  int dev = 0;
  PMGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  auto key = std::make_pair(dev, n);
  auto it = g_tables.find(key);
  if (it != g_tables.end()) {
    *out = it->second;
    return PMGB_OK;
  }
  std::vector<AxisEntry> h(n);
  const double twopi = 2.0 * M_PI;
  const double inv_n = 1.0 / n;
  const float c6 = (float)(1.0 / 6.0);
  const float twopi_f = (float)twopi;
  const float pi_f = (float)M_PI;
  for (int i = 0; i < n; ++i) {
    int m = i < (n + 1) / 2 ? i : i - n;  // numpy fftfreq ordering
    float w = (float)(twopi * ((double)m * inv_n));
    AxisEntry e;
    e.w = w;
    e.k2 = w * w;
    float s1 = std::sin(w), s2 = std::sin(2.0f * w);
    float t = 8.0f * s1;
    e.g1 = c6 * (t - s2);
    e.g0 = (i == n / 2) ? 0.0f : w;
    float x = w / twopi_f;
    float px = pi_f * x;
    float sinc = (px == 0.0f) ? 1.0f : std::sin(px) / px;
    float kf = w * sinc;
    e.fdk2 = kf * kf;
    e.pad[0] = e.pad[1] = e.pad[2] = 0.0f;
    h[i] = e;
  }
  AxisEntry *d = nullptr;
  PMGB_CUDA(cudaMalloc(&d, n * sizeof(AxisEntry)));
  cudaError_t err = cudaMemcpy(d, h.data(), n * sizeof(AxisEntry), cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    cudaFree(d);
    return fail(PMGB_ERR_CUDA, std::string("axis table upload: ") + cudaGetErrorString(err));
  }
  g_tables[key] = d;
  *out = d;
  return PMGB_OK;
}

__device__ __forceinline__ Elem element(const Tables &t, uint32_t e, uint32_t ny, uint32_t nzh) {
  uint32_t k = e % nzh, r = e / nzh, j = r % ny, i = r / ny;
  Elem el;
  el.X = t.x[i];
  el.Y = t.y[j];
  el.Z = t.z[k];
  return el;
}

__global__ void __launch_bounds__(256)
forces_kernel(const float2 *__restrict__ dk, float2 *__restrict__ fk, int64_t cs,
              Tables t, uint32_t ny, uint32_t nzh, uint32_t total, float r2, int order,
              int fd, float scale) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += gridDim.x * blockDim.x) {
    float2 f[3];
    force_modes(element(t, e, ny, nzh), dk[e], r2, order, fd, scale, f);
#pragma unroll
    for (int c = 0; c < 3; ++c) fk[c * cs + e] = f[c];
  }
}

__global__ void __launch_bounds__(256)
forces_vjp_kernel(const float2 *__restrict__ gfk, int64_t cs, float2 *__restrict__ gdk,
                  Tables t, uint32_t ny, uint32_t nzh, uint32_t total, float r2, int order,
                  int fd, float scale) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += gridDim.x * blockDim.x) {
    const float2 v[3] = {gfk[e], gfk[cs + e], gfk[2 * cs + e]};
    gdk[e] = force_modes_adjoint(element(t, e, ny, nzh), v, r2, order, fd, scale);
  }
}

__global__ void invlaplace_kernel(float2 *__restrict__ spec, Tables t, uint32_t ny,
                                  uint32_t nzh, uint32_t total, int fd, float scale) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += gridDim.x * blockDim.x) {
    Elem el = element(t, e, ny, nzh);
    float inv = inv_laplace(el, fd);
    float2 d = spec[e];
    spec[e] = make_float2(__fmul_rn(d.x, inv) * scale, __fmul_rn(d.y, inv) * scale);
  }
}

__global__ void longrange_kernel(float2 *__restrict__ spec, Tables t, uint32_t ny,
                                 uint32_t nzh, uint32_t total, float r2) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += gridDim.x * blockDim.x) {
    Elem el = element(t, e, ny, nzh);
    float L = long_range(el, r2);
    float2 d = spec[e];
    spec[e] = make_float2(d.x * L, d.y * L);
  }
}

__global__ void gradient_kernel(const float2 *__restrict__ in, float2 *__restrict__ out,
                                Tables t, uint32_t ny, uint32_t nzh, uint32_t total, int dir,
                                int order) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += gridDim.x * blockDim.x) {
    Elem el = element(t, e, ny, nzh);
    const AxisEntry &A = dir == 0 ? el.X : (dir == 1 ? el.Y : el.Z);
    float g = order ? A.g1 : A.g0;
    float2 d = in[e];
    out[e] = make_float2(g * d.y, -g * d.x);
  }
}

int geometry(int nx, int ny, int nz, uint32_t *total, uint32_t *nzh) {
  int64_t h = nz / 2 + 1;
  int64_t tot = (int64_t)nx * ny * h;
  if (tot >= (int64_t)UINT32_MAX)
    return fail(PMGB_ERR_UNSUPPORTED, "half spectrum larger than 2^32 elements");
  *total = (uint32_t)tot;
  *nzh = (uint32_t)h;
  return PMGB_OK;
}

}  // namespace

int tables(int nx, int ny, int nz, Tables *t) {
  PMGB_TRY(axis_table(nx, &t->x));
  PMGB_TRY(axis_table(ny, &t->y));
  PMGB_TRY(axis_table(nz, &t->z));
  return PMGB_OK;
}

int kspace_forces(const void *dk, void *fk, int64_t cs, int nx, int ny, int nz, float r_split,
                  int order, int fd, float scale, cudaStream_t s) {
  Tables t;
  uint32_t total, nzh;
  PMGB_TRY(geometry(nx, ny, nz, &total, &nzh));
  PMGB_TRY(tables(nx, ny, nz, &t));
  forces_kernel<<<wave_grid(forces_kernel, total, 256), 256, 0, s>>>(
      static_cast<const float2 *>(dk), static_cast<float2 *>(fk), cs, t, ny, nzh, total,
      r_split * r_split, order, fd, scale);
  PMGB_LAUNCHED("forces_kernel");
  return PMGB_OK;
}

int kspace_forces_vjp(const void *gfk, int64_t cs, void *gdk, int nx, int ny, int nz,
                      float r_split, int order, int fd, float scale, cudaStream_t s) {
  Tables t;
  uint32_t total, nzh;
  PMGB_TRY(geometry(nx, ny, nz, &total, &nzh));
  PMGB_TRY(tables(nx, ny, nz, &t));
  forces_vjp_kernel<<<wave_grid(forces_vjp_kernel, total, 256), 256, 0, s>>>(
      static_cast<const float2 *>(gfk), cs, static_cast<float2 *>(gdk), t, ny, nzh, total,
      r_split * r_split, order, fd, scale);
  PMGB_LAUNCHED("forces_vjp_kernel");
  return PMGB_OK;
}

int kspace_invlaplace(void *spec, int nx, int ny, int nz, int fd, float scale, cudaStream_t s) {
  Tables t;
  uint32_t total, nzh;
  PMGB_TRY(geometry(nx, ny, nz, &total, &nzh));
  PMGB_TRY(tables(nx, ny, nz, &t));
  invlaplace_kernel<<<wave_grid(invlaplace_kernel, total, 256), 256, 0, s>>>(
      static_cast<float2 *>(spec), t, ny, nzh, total, fd, scale);
  PMGB_LAUNCHED("invlaplace_kernel");
  return PMGB_OK;
}

int kspace_longrange(void *spec, int nx, int ny, int nz, float r_split, cudaStream_t s) {
  Tables t;
  uint32_t total, nzh;
  PMGB_TRY(geometry(nx, ny, nz, &total, &nzh));
  PMGB_TRY(tables(nx, ny, nz, &t));
  longrange_kernel<<<wave_grid(longrange_kernel, total, 256), 256, 0, s>>>(
      static_cast<float2 *>(spec), t, ny, nzh, total, r_split * r_split);
  PMGB_LAUNCHED("longrange_kernel");
  return PMGB_OK;
}

int kspace_gradient(const void *in, void *out, int nx, int ny, int nz, int dir, int order,
                    cudaStream_t s) {
  Tables t;
  uint32_t total, nzh;
  PMGB_TRY(geometry(nx, ny, nz, &total, &nzh));
  PMGB_TRY(tables(nx, ny, nz, &t));
  gradient_kernel<<<wave_grid(gradient_kernel, total, 256), 256, 0, s>>>(
      static_cast<const float2 *>(in), static_cast<float2 *>(out), t, ny, nzh, total, dir, order);
  PMGB_LAUNCHED("gradient_kernel");
  return PMGB_OK;
}

}  // namespace pmgb
