// CIC painting and reading on a periodic float32 mesh.
//
// Reference semantics: jaxpm/painting.py:15-45 (paint), :78-106 (read),
// jaxpm/painting_utils.py:28-187 (relative mode).  Weights are computed
// with the exact float32 operation order of the reference (common.cuh), so
// indices and per-neighbour weights are bit-identical; only the order in
// which contributions are summed into a cell differs (atomics).
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace pmgb {

// ---------------------------------------------------------------------------
// Plain painter: one thread per particle, eight fp32 global atomics.
// ---------------------------------------------------------------------------
// The eight weights are those of the reference's neighbour list; the two
// z-neighbours of each (x, y) pair go out as one vector reduction when
// they share a 16-byte group (red_zpair).
__global__ void __launch_bounds__(256)
paint_atomic_kernel(float *__restrict__ mesh, int nx, int ny, int nz,
                    const float *__restrict__ pos, int64_t np,
                    const float *__restrict__ weights, float wscale, bool vec) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float x, y, z;
    load3(pos, p, x, y, z);
    float wp = weights ? __fmul_rn(wscale, __ldg(weights + p)) : wscale;
    Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int cx = c & 1, cy = c >> 1;
      const float kxy = __fmul_rn(cx ? ax.k1 : ax.k0, cy ? ay.k1 : ay.k0);
      float *row = mesh + cell_index(cx ? ax.i1 : ax.i0, cy ? ay.i1 : ay.i0, 0, ny, nz);
      red_zpair(row, az.i0, az.i1, __fmul_rn(wp, __fmul_rn(kxy, az.k0)),
                __fmul_rn(wp, __fmul_rn(kxy, az.k1)), vec);
    }
  }
}

// ---------------------------------------------------------------------------
// Deterministic painter: every contribution is rounded to a signed 32.32
// fixed-point integer and summed with 64-bit integer atomics, which are
// associative, so the result does not depend on the order of arrival.
// ---------------------------------------------------------------------------
constexpr float DET_SCALE = 4294967296.0f;  // 2^32

__global__ void __launch_bounds__(256)
paint_fixed_kernel(unsigned long long *__restrict__ acc, int nx, int ny, int nz,
                   const float *__restrict__ pos, int64_t np,
                   const float *__restrict__ weights, float wscale) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float x, y, z;
    load3(pos, p, x, y, z);
    float wp = weights ? __fmul_rn(wscale, __ldg(weights + p)) : wscale;
    Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      float w = __fmul_rn(wp, __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0,
                                                  conn_y(n) ? ay.k1 : ay.k0),
                                        conn_z(n) ? az.k1 : az.k0));
      long long q = __float2ll_rn(w * DET_SCALE);
      atomicAdd(acc + cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                                 conn_z(n) ? az.i1 : az.i0, ny, nz),
                (unsigned long long)q);
    }
  }
}

__global__ void fixed_to_float_kernel(float *__restrict__ mesh,
                                      const unsigned long long *__restrict__ acc,
                                      int64_t n, int accumulate) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float v = (float)((double)(long long)acc[i] * (1.0 / 4294967296.0));
    mesh[i] = accumulate ? mesh[i] + v : v;
  }
}

// ---------------------------------------------------------------------------
// Readers.
// ---------------------------------------------------------------------------
// out[p * ostride] = the CIC read of `mesh` at particle p.
__global__ void __launch_bounds__(256)
read_kernel(const float *__restrict__ mesh, int nx, int ny, int nz,
            const float *__restrict__ pos, int64_t np, float *__restrict__ out, int ostride) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float x, y, z;
    load3(pos, p, x, y, z);
    Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
    float s = 0.0f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      float w = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                          conn_z(n) ? az.k1 : az.k0);
      s += __ldg(mesh + cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                                   conn_z(n) ? az.i1 : az.i0, ny, nz)) * w;
    }
    out[p * ostride] = s;
  }
}

__global__ void __launch_bounds__(256)
read3_kernel(const float *__restrict__ m, int64_t cs, int nx, int ny, int nz,
             const float *__restrict__ pos, int64_t np, float *__restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float x, y, z;
    load3(pos, p, x, y, z);
    Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      float w = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                          conn_z(n) ? az.k1 : az.k0);
      int64_t c = cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                             conn_z(n) ? az.i1 : az.i0, ny, nz);
      s0 += __ldg(m + c) * w;
      s1 += __ldg(m + cs + c) * w;
      s2 += __ldg(m + 2 * cs + c) * w;
    }
    out[3 * p] = s0;
    out[3 * p + 1] = s1;
    out[3 * p + 2] = s2;
  }
}

__global__ void weights_kernel(const float *__restrict__ pos, int64_t np, int nx,
                               int ny, int nz, int32_t *__restrict__ idx,
                               float *__restrict__ wout) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float x, y, z;
    load3(pos, p, x, y, z);
    Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      wout[8 * p + n] = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                                  conn_z(n) ? az.k1 : az.k0);
      idx[24 * p + 3 * n] = conn_x(n) ? ax.i1 : ax.i0;
      idx[24 * p + 3 * n + 1] = conn_y(n) ? ay.i1 : ay.i0;
      idx[24 * p + 3 * n + 2] = conn_z(n) ? az.i1 : az.i0;
    }
  }
}

// Gradient of the interpolated field at p: g[d] = sum_c dW/dx_d * mesh[c].
__device__ __forceinline__ void interp_grad(const float *__restrict__ mesh, int nx,
                                            int ny, int nz, float x, float y, float z,
                                            float &gx, float &gy, float &gz, float &val) {
  Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
  AxisGrad dx = cic_axis_grad(x), dy = cic_axis_grad(y), dz = cic_axis_grad(z);
  gx = gy = gz = val = 0.f;
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    float kx = conn_x(n) ? ax.k1 : ax.k0, ky = conn_y(n) ? ay.k1 : ay.k0,
          kz = conn_z(n) ? az.k1 : az.k0;
    float ddx = conn_x(n) ? dx.d1 : dx.d0, ddy = conn_y(n) ? dy.d1 : dy.d0,
          ddz = conn_z(n) ? dz.d1 : dz.d0;
    float m = __ldg(mesh + cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                                      conn_z(n) ? az.i1 : az.i0, ny, nz));
    gx += m * ddx * ky * kz;
    gy += m * kx * ddy * kz;
    gz += m * kx * ky * ddz;
    val += m * kx * ky * kz;
  }
}

__global__ void __launch_bounds__(256)
paint_vjp_kernel(const float *__restrict__ g_mesh, int nx, int ny, int nz,
                 const float *__restrict__ pos, int64_t np,
                 const float *__restrict__ weights, float wscale,
                 float *__restrict__ g_pos, float *__restrict__ g_w) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float x, y, z, gx, gy, gz, v;
    load3(pos, p, x, y, z);
    interp_grad(g_mesh, nx, ny, nz, x, y, z, gx, gy, gz, v);
    float wp = weights ? wscale * __ldg(weights + p) : wscale;
    if (g_pos) {
      g_pos[3 * p] = wp * gx;
      g_pos[3 * p + 1] = wp * gy;
      g_pos[3 * p + 2] = wp * gz;
    }
    if (g_w) g_w[p] = v;
  }
}

__global__ void __launch_bounds__(256)
read_vjp_pos_kernel(const float *__restrict__ mesh, int nx, int ny, int nz,
                    const float *__restrict__ pos, int64_t np,
                    const float *__restrict__ g_out, float *__restrict__ g_pos) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float x, y, z, gx, gy, gz, v;
    load3(pos, p, x, y, z);
    interp_grad(mesh, nx, ny, nz, x, y, z, gx, gy, gz, v);
    float g = __ldg(g_out + p);
    g_pos[3 * p] = g * gx;
    g_pos[3 * p + 1] = g * gy;
    g_pos[3 * p + 2] = g * gz;
  }
}

// ---------------------------------------------------------------------------
// Relative mode (jaxpm/painting_utils.py:47-69,84-96).  Particle i sits at
// lattice point unravel(i) plus disp[i]; the periodic wrap is taken in float
// before the floor, the displacement is re-centred with rint(d/L)*L, and a
// neighbour whose wrapped coordinate rounds up to L is dropped (the
// reference's scatter and gather both drop out-of-range indices).
// ---------------------------------------------------------------------------
struct RelAxis {
  int i[2];
  float w[2];
};

__device__ __forceinline__ float jnp_remainder(float x, float L) {
  float r = fmodf(x, L);
  if (r != 0.0f && ((r < 0.0f) != (L < 0.0f))) r = __fadd_rn(r, L);
  return r;
}

__device__ __forceinline__ RelAxis rel_axis(int lattice, float disp, int n) {
  RelAxis a;
  const float L = (float)n;
  float p = __fadd_rn((float)lattice, disp);
#pragma unroll
  for (int o = 0; o < 2; ++o) {
    float t = o ? __fadd_rn(p, 1.0f) : p;
    float r = floorf(jnp_remainder(t, L));
    float d = __fsub_rn(p, r);
    d = __fsub_rn(d, __fmul_rn(rintf(__fdiv_rn(d, L)), L));
    a.w[o] = __fsub_rn(1.0f, fabsf(d));
    a.i[o] = (r >= 0.0f && r < L) ? (int)r : -1;  // -1: dropped
  }
  return a;
}

__global__ void __launch_bounds__(256)
paint_dx_kernel(float *__restrict__ mesh, int nx, int ny, int nz,
                const float *__restrict__ disp, const float *__restrict__ weights,
                float wscale) {
  const int64_t np = (int64_t)nx * ny * nz;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    int iz = (int)(p % nz), iy = (int)((p / nz) % ny), ix = (int)(p / ((int64_t)ny * nz));
    float x, y, z;
    load3(disp, p, x, y, z);
    RelAxis ax = rel_axis(ix, x, nx), ay = rel_axis(iy, y, ny), az = rel_axis(iz, z, nz);
    float wp = weights ? __fmul_rn(wscale, __ldg(weights + p)) : wscale;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      int ox = n & 1, oy = (n >> 1) & 1, oz = (n >> 2) & 1;
      if (ax.i[ox] < 0 || ay.i[oy] < 0 || az.i[oz] < 0) continue;
      float w = __fmul_rn(wp, __fmul_rn(__fmul_rn(ax.w[ox], ay.w[oy]), az.w[oz]));
      atomicAdd(mesh + cell_index(ax.i[ox], ay.i[oy], az.i[oz], ny, nz), w);
    }
  }
}

__global__ void __launch_bounds__(256)
read_dx_kernel(const float *__restrict__ mesh, int nx, int ny, int nz,
               const float *__restrict__ disp, float *__restrict__ out) {
  const int64_t np = (int64_t)nx * ny * nz;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    int iz = (int)(p % nz), iy = (int)((p / nz) % ny), ix = (int)(p / ((int64_t)ny * nz));
    float x, y, z;
    load3(disp, p, x, y, z);
    RelAxis ax = rel_axis(ix, x, nx), ay = rel_axis(iy, y, ny), az = rel_axis(iz, z, nz);
    float s = 0.f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      int ox = n & 1, oy = (n >> 1) & 1, oz = (n >> 2) & 1;
      if (ax.i[ox] < 0 || ay.i[oy] < 0 || az.i[oz] < 0) continue;
      float w = __fmul_rn(__fmul_rn(ax.w[ox], ay.w[oy]), az.w[oz]);
      s += __ldg(mesh + cell_index(ax.i[ox], ay.i[oy], az.i[oz], ny, nz)) * w;
    }
    out[p] = s;
  }
}

__global__ void enmesh_kernel(const float *__restrict__ disp, int nx, int ny, int nz,
                              int32_t *__restrict__ idx, float *__restrict__ wout) {
  const int64_t np = (int64_t)nx * ny * nz;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    int iz = (int)(p % nz), iy = (int)((p / nz) % ny), ix = (int)(p / ((int64_t)ny * nz));
    float x, y, z;
    load3(disp, p, x, y, z);
    RelAxis ax = rel_axis(ix, x, nx), ay = rel_axis(iy, y, ny), az = rel_axis(iz, z, nz);
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      int ox = n & 1, oy = (n >> 1) & 1, oz = (n >> 2) & 1;
      wout[8 * p + n] = __fmul_rn(__fmul_rn(ax.w[ox], ay.w[oy]), az.w[oz]);
      idx[24 * p + 3 * n] = ax.i[ox];
      idx[24 * p + 3 * n + 1] = ay.i[oy];
      idx[24 * p + 3 * n + 2] = az.i[oz];
    }
  }
}

// ---------------------------------------------------------------------------
// Host entry points (internal; the C ABI wrappers live in abi.cu).
// ---------------------------------------------------------------------------
size_t paint_workspace_size(int nx, int ny, int nz, int64_t np, int mode) {
  (void)np;
  if (mode == PMGB_PAINT_DETERMINISTIC)
    return (size_t)nx * ny * nz * sizeof(unsigned long long);
  return 0;
}

int paint(float *mesh, int nx, int ny, int nz, const float *pos, int64_t np,
          const float *weights, float wscale, int mode, int accumulate,
          void *ws, size_t ws_bytes, cudaStream_t s) {
  const int64_t ncell = (int64_t)nx * ny * nz;
  if (mode == PMGB_PAINT_DETERMINISTIC) {
    size_t need = paint_workspace_size(nx, ny, nz, np, mode);
    if (!ws || ws_bytes < need)
      return fail(PMGB_ERR_WORKSPACE, "deterministic paint needs " +
                                          std::to_string(need) + " workspace bytes");
    auto *acc = static_cast<unsigned long long *>(ws);
    PMGB_CUDA(cudaMemsetAsync(acc, 0, need, s));
    if (np > 0) {
      paint_fixed_kernel<<<wave_grid(paint_fixed_kernel, np, 256), 256, 0, s>>>(
          acc, nx, ny, nz, pos, np, weights, wscale);
      PMGB_LAUNCHED("paint_fixed_kernel");
    }
    fixed_to_float_kernel<<<wave_grid(fixed_to_float_kernel, ncell, 256), 256, 0, s>>>(
        mesh, acc, ncell, accumulate);
    PMGB_LAUNCHED("fixed_to_float_kernel");
    return PMGB_OK;
  }
  if (!accumulate) PMGB_CUDA(cudaMemsetAsync(mesh, 0, ncell * sizeof(float), s));
  if (np == 0) return PMGB_OK;
  if (mode == PMGB_PAINT_ATOMIC) {
    // 8 CTAs per SM requested rather than one wave of the 6 resident: the
    // atomics-bound paint runs faster with the extra CTAs queued (16.7M
    // particles on 256^3: 0.41 against 0.44 ms uniform, 0.44 against 0.46 ms
    // clustered)
    paint_atomic_kernel<<<grid_for(np, 256), 256, 0, s>>>(
        mesh, nx, ny, nz, pos, np, weights, wscale, zpair_vec_ok(mesh, nz));
    PMGB_LAUNCHED("paint_atomic_kernel");
    return PMGB_OK;
  }
  if (mode == PMGB_PAINT_BINNED) return paint_box(mesh, nx, ny, nz, pos, np, weights, wscale,
                                                  nullptr, s);
  return fail(PMGB_ERR_INVALID_ARGUMENT, "unknown paint mode " + std::to_string(mode));
}

// Deterministic paint into a caller-provided fixed-point accumulator of
// nx*ny*nz 64-bit words (cleared here): the kernels of the deterministic
// mode, for callers that supply the scratch themselves.
int paint_fixed_into(unsigned long long *acc, float *mesh, int nx, int ny, int nz,
                     const float *pos, int64_t np, const float *weights, float wscale,
                     int accumulate, cudaStream_t s) {
  const int64_t ncell = (int64_t)nx * ny * nz;
  PMGB_CUDA(cudaMemsetAsync(acc, 0, ncell * sizeof(unsigned long long), s));
  if (np > 0) {
    paint_fixed_kernel<<<wave_grid(paint_fixed_kernel, np, 256), 256, 0, s>>>(
        acc, nx, ny, nz, pos, np, weights, wscale);
    PMGB_LAUNCHED("paint_fixed_kernel");
  }
  fixed_to_float_kernel<<<wave_grid(fixed_to_float_kernel, ncell, 256), 256, 0, s>>>(
      mesh, acc, ncell, accumulate);
  PMGB_LAUNCHED("fixed_to_float_kernel");
  return PMGB_OK;
}

int read(const float *mesh, int nx, int ny, int nz, const float *pos, int64_t np,
         float *out, cudaStream_t s) {
  if (np == 0) return PMGB_OK;
  read_kernel<<<wave_grid(read_kernel, np, 256), 256, 0, s>>>(mesh, nx, ny, nz, pos, np, out,
                                                              1);
  PMGB_LAUNCHED("read_kernel");
  return PMGB_OK;
}

// Three components in one pass when their meshes fit in L2 together (or
// none does), else one pass per component: a particle order that is random
// over the mesh then keeps one mesh resident in L2 at a time instead of
// missing in all three (16.7M particles on 256^3, 64 MB per mesh: uniform
// 3.75 ms in one pass, 1.23 ms in three; clustered 0.70 -> 0.48 ms), for
// 12 B more of positions per particle and pass.
int read3(const float *mesh3, int64_t cs, int nx, int ny, int nz, const float *pos,
          int64_t np, float *out, cudaStream_t s) {
  if (np == 0) return PMGB_OK;
  const int64_t mesh_bytes = (int64_t)nx * ny * nz * (int64_t)sizeof(float);
  const int64_t l2 = l2_bytes();
  if (l2 > 0 && 3 * mesh_bytes > (l2 * 3) / 4 && 2 * mesh_bytes <= l2) {
    for (int c = 0; c < 3; ++c) {
      read_kernel<<<wave_grid(read_kernel, np, 256), 256, 0, s>>>(mesh3 + c * cs, nx, ny, nz,
                                                                  pos, np, out + c, 3);
      PMGB_LAUNCHED("read_kernel");
    }
    return PMGB_OK;
  }
  read3_kernel<<<wave_grid(read3_kernel, np, 256), 256, 0, s>>>(
      mesh3, cs, nx, ny, nz, pos, np, out);
  PMGB_LAUNCHED("read3_kernel");
  return PMGB_OK;
}

int cic_weights(const float *pos, int64_t np, int nx, int ny, int nz, int32_t *idx,
                float *w, cudaStream_t s) {
  if (np == 0) return PMGB_OK;
  weights_kernel<<<wave_grid(weights_kernel, np, 256), 256, 0, s>>>(pos, np, nx, ny, nz, idx, w);
  PMGB_LAUNCHED("weights_kernel");
  return PMGB_OK;
}

int paint_vjp(const float *g_mesh, int nx, int ny, int nz, const float *pos, int64_t np,
              const float *weights, float wscale, float *g_pos, float *g_w,
              cudaStream_t s) {
  if (np == 0 || (!g_pos && !g_w)) return PMGB_OK;
  paint_vjp_kernel<<<wave_grid(paint_vjp_kernel, np, 256), 256, 0, s>>>(
      g_mesh, nx, ny, nz, pos, np, weights, wscale, g_pos, g_w);
  PMGB_LAUNCHED("paint_vjp_kernel");
  return PMGB_OK;
}

int read_vjp(const float *mesh, int nx, int ny, int nz, const float *pos, int64_t np,
             const float *g_out, float *g_mesh, float *g_pos, cudaStream_t s) {
  if (np == 0) return PMGB_OK;
  if (g_mesh) {
    paint_atomic_kernel<<<grid_for(np, 256), 256, 0, s>>>(
        g_mesh, nx, ny, nz, pos, np, g_out, 1.0f, zpair_vec_ok(g_mesh, nz));
    PMGB_LAUNCHED("paint_atomic_kernel");
  }
  if (g_pos) {
    read_vjp_pos_kernel<<<wave_grid(read_vjp_pos_kernel, np, 256), 256, 0, s>>>(
        mesh, nx, ny, nz, pos, np, g_out, g_pos);
    PMGB_LAUNCHED("read_vjp_pos_kernel");
  }
  return PMGB_OK;
}

int paint_dx(float *mesh, int nx, int ny, int nz, const float *disp, const float *weights,
             float wscale, int accumulate, cudaStream_t s) {
  const int64_t n = (int64_t)nx * ny * nz;
  if (!accumulate) PMGB_CUDA(cudaMemsetAsync(mesh, 0, n * sizeof(float), s));
  paint_dx_kernel<<<wave_grid(paint_dx_kernel, n, 256), 256, 0, s>>>(
      mesh, nx, ny, nz, disp, weights, wscale);
  PMGB_LAUNCHED("paint_dx_kernel");
  return PMGB_OK;
}

int read_dx(const float *mesh, int nx, int ny, int nz, const float *disp, float *out,
            cudaStream_t s) {
  const int64_t n = (int64_t)nx * ny * nz;
  read_dx_kernel<<<wave_grid(read_dx_kernel, n, 256), 256, 0, s>>>(mesh, nx, ny, nz, disp, out);
  PMGB_LAUNCHED("read_dx_kernel");
  return PMGB_OK;
}

int enmesh(const float *disp, int nx, int ny, int nz, int32_t *idx, float *w,
           cudaStream_t s) {
  const int64_t n = (int64_t)nx * ny * nz;
  enmesh_kernel<<<wave_grid(enmesh_kernel, n, 256), 256, 0, s>>>(disp, nx, ny, nz, idx, w);
  PMGB_LAUNCHED("enmesh_kernel");
  return PMGB_OK;
}

}  // namespace pmgb
