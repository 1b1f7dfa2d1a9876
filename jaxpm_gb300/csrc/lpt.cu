// Initial-condition kernels on either side of the step loop.
//
// linear_field colouring: jaxpm/pm.py:134-143 -- the spectrum of a white
// noise field is multiplied by sqrt(pk(|k|) * N^3 / V), with pk the linear
// interpolation of a (k, P) table (the closure the reference's tests pass,
// tests/conftest.py:90-94).
// 2LPT source: jaxpm/pm.py:88-111 -- six second-derivative fields
// ifft3d(grad_i grad_j * delta_k * invlaplace), combined into
// sum_{i<j} (phi_ii phi_jj - phi_ij^2) in the reference's accumulation order.
// LPT combination: jaxpm/pm.py:85-87,118-124 as out = a1*F1 + a2*F2.
#include <cmath>

#include "common.cuh"
#include "kernels.cuh"

namespace pmgb {

namespace {

__device__ __forceinline__ float fftfreq_w(int i, int n) {
  int m = i < (n + 1) / 2 ? i : i - n;
  return (float)(6.283185307179586 * ((double)m * (1.0 / n)));
}

__device__ __forceinline__ float order1_grad(float w) {
  return (float)(1.0 / 6.0) * (8.0f * sinf(w) - sinf(2.0f * w));
}

// jnp.interp: clamp outside the table, linear inside.
__device__ float interp(float x, const float *__restrict__ xp, const float *__restrict__ fp,
                        int n) {
  if (x <= xp[0]) return fp[0];
  if (x >= xp[n - 1]) return fp[n - 1];
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (xp[mid] <= x) lo = mid; else hi = mid;
  }
  float t = (x - xp[lo]) / (xp[hi] - xp[lo]);
  return fp[lo] + t * (fp[hi] - fp[lo]);
}

__global__ void colour_kernel(float2 *__restrict__ spec, int nx, int ny, int nz, float bx,
                              float by, float bz, const float *__restrict__ tk,
                              const float *__restrict__ tp, int nt, float norm, float scale) {
  const int nzh = nz / 2 + 1;
  const int64_t total = (int64_t)nx * ny * nzh;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int k = (int)(e % nzh);
    int64_t r = e / nzh;
    int j = (int)(r % ny), i = (int)(r / ny);
    float kx = fftfreq_w(i, nx) / bx * (float)nx;
    float ky = fftfreq_w(j, ny) / by * (float)ny;
    float kz = fftfreq_w(k, nz) / bz * (float)nz;
    float kmesh = sqrtf(kx * kx + ky * ky + kz * kz);
    float amp = sqrtf(interp(kmesh, tk, tp, nt) * norm) * scale;
    float2 v = spec[e];
    spec[e] = make_float2(v.x * amp, v.y * amp);
  }
}

// The six spectra -grad_i grad_j * invlaplace * delta_k (pairs 00,01,02,11,12,22).
__global__ void shear_kernel(const float2 *__restrict__ dk, float2 *__restrict__ out,
                             int64_t cs, int nx, int ny, int nz, float scale) {
  const int nzh = nz / 2 + 1;
  const int64_t total = (int64_t)nx * ny * nzh;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int k = (int)(e % nzh);
    int64_t r = e / nzh;
    int j = (int)(r % ny), i = (int)(r / ny);
    float w[3] = {fftfreq_w(i, nx), fftfreq_w(j, ny), fftfreq_w(k, nz)};
    float kk = __fadd_rn(__fadd_rn(w[0] * w[0], w[1] * w[1]), w[2] * w[2]);
    float inv = kk == 0.0f ? 0.0f : -__frcp_rn(kk);
    float2 d = dk[e];
    float px = d.x * inv, py = d.y * inv;
    float g[3] = {order1_grad(w[0]), order1_grad(w[1]), order1_grad(w[2])};
    int c = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = a; b < 3; ++b) {
        float m = -(g[a] * g[b]) * scale;  // (i g_a)(i g_b) = -g_a g_b
        out[c * cs + e] = make_float2(px * m, py * m);
        ++c;
      }
  }
}

// delta2 = sum_{i<j}(s_ii s_jj - s_ij^2), accumulated as in jaxpm/pm.py:96-109.
__global__ void source_kernel(const float *__restrict__ s, int64_t cs, float *__restrict__ d2,
                              int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    float s00 = s[e], s01 = s[cs + e], s02 = s[2 * cs + e], s11 = s[3 * cs + e],
          s12 = s[4 * cs + e], s22 = s[5 * cs + e];
    float d = __fmul_rn(s00, 0.0f);
    d = __fsub_rn(d, __fmul_rn(s01, s01));
    d = __fsub_rn(d, __fmul_rn(s02, s02));
    d = __fadd_rn(d, __fmul_rn(s11, s00));
    float acc = __fadd_rn(s00, s11);
    d = __fsub_rn(d, __fmul_rn(s12, s12));
    d = __fadd_rn(d, __fmul_rn(s22, acc));
    d2[e] = d;
  }
}

__global__ void combine_kernel(const float *__restrict__ a, const float *__restrict__ b,
                               int64_t n, float ca, float cb, float *__restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    out[e] = b ? ca * a[e] + cb * b[e] : ca * a[e];
}

// Adjoint of source_kernel: with d = sum_{i<j}(s_ii s_jj - s_ij^2),
// s_bar_ii = g * (sum of the other two diagonal entries), s_bar_ij = -2 g s_ij
// (in place over the six shear meshes).
__global__ void source_vjp_kernel(float *__restrict__ s, int64_t cs,
                                  const float *__restrict__ g, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const float s00 = s[e], s01 = s[cs + e], s02 = s[2 * cs + e], s11 = s[3 * cs + e],
                s12 = s[4 * cs + e], s22 = s[5 * cs + e];
    const float ge = g[e];
    s[e] = ge * (s11 + s22);
    s[cs + e] = -2.0f * ge * s01;
    s[2 * cs + e] = -2.0f * ge * s02;
    s[3 * cs + e] = ge * (s00 + s22);
    s[4 * cs + e] = -2.0f * ge * s12;
    s[5 * cs + e] = ge * (s00 + s11);
  }
}

// Adjoint of shear_kernel + C2R: each map delta -> s_ab is a real circular
// convolution with an even kernel (multiplier -g_a g_b invlaplace, real and
// even in k), hence self-adjoint; the six transformed cotangents are
// combined into one spectrum, in place over the first (elementwise).
__global__ void shear_vjp_kernel(float2 *__restrict__ spec, int64_t cs, int nx, int ny, int nz,
                                 float scale) {
  const int nzh = nz / 2 + 1;
  const int64_t total = (int64_t)nx * ny * nzh;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int k = (int)(e % nzh);
    int64_t r = e / nzh;
    int j = (int)(r % ny), i = (int)(r / ny);
    float w[3] = {fftfreq_w(i, nx), fftfreq_w(j, ny), fftfreq_w(k, nz)};
    float kk = __fadd_rn(__fadd_rn(w[0] * w[0], w[1] * w[1]), w[2] * w[2]);
    float inv = kk == 0.0f ? 0.0f : -__frcp_rn(kk);
    float g[3] = {order1_grad(w[0]), order1_grad(w[1]), order1_grad(w[2])};
    float ax = 0.f, ay = 0.f;
    int c = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = a; b < 3; ++b) {
        const float m = -(g[a] * g[b]) * scale * inv;
        const float2 v = spec[c * cs + e];
        ax += m * v.x;
        ay += m * v.y;
        ++c;
      }
    spec[e] = make_float2(ax, ay);
  }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

int linear_field_colour(void *spec, int nx, int ny, int nz, float bx, float by, float bz,
                        const float *tk, const float *tp, int nt, float scale, cudaStream_t s) {
  const int64_t total = (int64_t)nx * ny * (nz / 2 + 1);
  float norm = (float)((double)nx * ny * nz / ((double)bx * by * bz));
  colour_kernel<<<wave_grid(colour_kernel, total, 256), 256, 0, s>>>(
      static_cast<float2 *>(spec), nx, ny, nz, bx, by, bz, tk, tp, nt, norm, scale);
  PMGB_LAUNCHED("colour_kernel");
  return PMGB_OK;
}

size_t lpt2_source_workspace_size(int nx, int ny, int nz) {
  const size_t ncell = (size_t)nx * ny * nz;
  const size_t nhalf = (size_t)nx * ny * (nz / 2 + 1);
  return align256(6 * nhalf * 8) + align256(6 * ncell * 4);
}

int lpt2_source(const void *dk, float *delta2, int nx, int ny, int nz, void *ws, size_t bytes,
                cudaStream_t s) {
  const size_t need = lpt2_source_workspace_size(nx, ny, nz);
  if (!ws || bytes < need)
    return fail(PMGB_ERR_WORKSPACE, "2LPT source needs " + std::to_string(need) +
                                        " workspace bytes");
  const int64_t ncell = (int64_t)nx * ny * nz;
  const int64_t nhalf = (int64_t)nx * ny * (nz / 2 + 1);
  float2 *spec = static_cast<float2 *>(ws);
  float *shear = reinterpret_cast<float *>(static_cast<char *>(ws) + align256(6 * nhalf * 8));
  shear_kernel<<<wave_grid(shear_kernel, nhalf, 256), 256, 0, s>>>(
      static_cast<const float2 *>(dk), spec, nhalf, nx, ny, nz, 1.0f / (float)ncell);
  PMGB_LAUNCHED("shear_kernel");
  PMGB_TRY(fft_c2r(spec, shear, nx, ny, nz, 6, s));
  source_kernel<<<wave_grid(source_kernel, ncell, 256), 256, 0, s>>>(shear, ncell, delta2, ncell);
  PMGB_LAUNCHED("source_kernel");
  return PMGB_OK;
}

int lpt2_source_vjp(const float *ic, const float *g, float *g_ic, int nx, int ny, int nz, void *ws,
                    size_t bytes, cudaStream_t s) {
  const size_t need = lpt2_source_workspace_size(nx, ny, nz);
  if (!ws || bytes < need)
    return fail(PMGB_ERR_WORKSPACE, "2LPT source adjoint needs " + std::to_string(need) +
                                        " workspace bytes");
  const int64_t ncell = (int64_t)nx * ny * nz;
  const int64_t nhalf = (int64_t)nx * ny * (nz / 2 + 1);
  float2 *spec = static_cast<float2 *>(ws);
  float *shear = reinterpret_cast<float *>(static_cast<char *>(ws) + align256(6 * nhalf * 8));
  const float scale = 1.0f / (float)ncell;
  // forward recompute of the six shear meshes (delta_k staged in the shear
  // meshes' region, which holds one spectrum and is overwritten next)
  float2 *dk = reinterpret_cast<float2 *>(shear);
  PMGB_TRY(fft_r2c(ic, dk, nx, ny, nz, 1, s));
  shear_kernel<<<wave_grid(shear_kernel, nhalf, 256), 256, 0, s>>>(
      dk, spec, nhalf, nx, ny, nz, scale);
  PMGB_LAUNCHED("shear_kernel");
  PMGB_TRY(fft_c2r(spec, shear, nx, ny, nz, 6, s));
  source_vjp_kernel<<<wave_grid(source_vjp_kernel, ncell, 256), 256, 0, s>>>(
      shear, ncell, g, ncell);
  PMGB_LAUNCHED("source_vjp_kernel");
  PMGB_TRY(fft_r2c(shear, spec, nx, ny, nz, 6, s));
  shear_vjp_kernel<<<wave_grid(shear_vjp_kernel, nhalf, 256), 256, 0, s>>>(
      spec, nhalf, nx, ny, nz, scale);
  PMGB_LAUNCHED("shear_vjp_kernel");
  return fft_c2r(spec, g_ic, nx, ny, nz, 1, s);
}

int lpt_combine(const float *a, const float *b, int64_t n, float ca, float cb, float *out,
                cudaStream_t s) {
  if (n == 0) return PMGB_OK;
  combine_kernel<<<wave_grid(combine_kernel, n, 256), 256, 0, s>>>(a, b, n, ca, cb, out);
  PMGB_LAUNCHED("combine_kernel");
  return PMGB_OK;
}

}  // namespace pmgb
