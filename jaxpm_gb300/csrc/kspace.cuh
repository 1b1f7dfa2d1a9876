// Per-axis Fourier tables and the per-element k-space operators shared by
// the k-space kernels (kspace.cu) and the fused spectral pipeline
// (spectral.cu).  Wave numbers 2*pi*fftfreq(n) (jaxpm/kernels.py:10-23);
// gradient, inverse Laplacian and long-range kernels of jaxpm/kernels.py:41-115.
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace pmgb {

struct AxisEntry {
  float w;     // 2*pi*fftfreq(n)[i], radians per cell
  float k2;    // w*w
  float g1;    // (8 sin w - sin 2w)/6, order-1 gradient factor
  float g0;    // w with the Nyquist entry zeroed, order-0 gradient factor
  float fdk2;  // (w * sinc(w / 2pi))^2, finite-difference Laplacian term
  float pad[3];
};

struct Tables {
  const AxisEntry *x, *y, *z;
};

// Builds (once per device and n) the device tables of the three axes.
int tables(int nx, int ny, int nz, Tables *t);

struct Elem {
  AxisEntry X, Y, Z;
};

// -1/k^2 with k=0 -> 0 (kernels.py:87-92): kk summed as ((0 + kx^2) + ky^2) + kz^2.
__device__ __forceinline__ float inv_laplace(const Elem &el, int fd) {
  float kk = fd ? __fadd_rn(__fadd_rn(el.X.fdk2, el.Y.fdk2), el.Z.fdk2)
                : __fadd_rn(__fadd_rn(el.X.k2, el.Y.k2), el.Z.k2);
  return kk == 0.0f ? 0.0f : -__frcp_rn(kk);
}

// exp(-k^2 r^2) or 1 (kernels.py:111-115).
__device__ __forceinline__ float long_range(const Elem &el, float r2) {
  if (r2 == 0.0f) return 1.0f;
  float kk = __fadd_rn(__fadd_rn(el.X.k2, el.Y.k2), el.Z.k2);
  return expf(-kk * r2);
}

// The three force spectra of one element of delta_k (pm.py:49-56):
// pot = (delta * invlaplace) * longrange, F_c = -(i g_c) pot * scale.
__device__ __forceinline__ void force_modes(const Elem &el, float2 d, float r2, int order,
                                            int fd, float scale, float2 f[3]) {
  const float inv = inv_laplace(el, fd);
  const float L = long_range(el, r2);
  const float px = __fmul_rn(__fmul_rn(d.x, inv), L), py = __fmul_rn(__fmul_rn(d.y, inv), L);
  const float g[3] = {order ? el.X.g1 : el.X.g0, order ? el.Y.g1 : el.Y.g0,
                      order ? el.Z.g1 : el.Z.g0};
#pragma unroll
  for (int c = 0; c < 3; ++c)
    // -(i g) * (px + i py) = g*py - i g*px
    f[c] = make_float2(__fmul_rn(g[c], py) * scale, -__fmul_rn(g[c], px) * scale);
}

// Adjoint of force_modes: sum_c conj(K_c) v_c with conj(K_c) = (i g_c) m.
__device__ __forceinline__ float2 force_modes_adjoint(const Elem &el, const float2 v[3],
                                                      float r2, int order, int fd,
                                                      float scale) {
  const float m = inv_laplace(el, fd) * long_range(el, r2) * scale;
  const float g[3] = {order ? el.X.g1 : el.X.g0, order ? el.Y.g1 : el.Y.g0,
                      order ? el.Z.g1 : el.Z.g0};
  float ax = 0.f, ay = 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    // (i g)(vx + i vy) = -g vy + i g vx
    ax -= g[c] * v[c].y;
    ay += g[c] * v[c].x;
  }
  return make_float2(ax * m, ay * m);
}

}  // namespace pmgb
