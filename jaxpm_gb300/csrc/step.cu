// The FastPM step: fused gather + kick + drift, its one-kernel-per-op
// counterpart, the pm_forces adjoint, and the composite calls that chain
// paint -> R2C -> k-space -> C2R -> read through a caller-provided
// workspace.
//
// Reference: jaxpm/pm.py:12-58 (pm_forces), jaxpm/ode.py:20-80 (FastPM
// drift / kick / first_kick).  The kick and drift coefficients are host
// scalars (growth-factor differences of ode.py times the step, with
// 1.5*Omega_m folded into the kick).
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace pmgb {

// vel += kick * read3(force meshes at pos); pos += drift * vel.
__global__ void __launch_bounds__(256)
read3_kick_drift_kernel(const float *__restrict__ m, int64_t cs, int nx, int ny, int nz,
                        float *__restrict__ pos, float *__restrict__ vel, int64_t np,
                        float kick, float drift, float *__restrict__ fout) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float x = pos[3 * p], y = pos[3 * p + 1], z = pos[3 * p + 2];
    float vx = vel[3 * p], vy = vel[3 * p + 1], vz = vel[3 * p + 2];
    Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
    float f0 = 0.f, f1 = 0.f, f2 = 0.f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      float w = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                          conn_z(n) ? az.k1 : az.k0);
      int64_t c = cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                             conn_z(n) ? az.i1 : az.i0, ny, nz);
      f0 += __ldg(m + c) * w;
      f1 += __ldg(m + cs + c) * w;
      f2 += __ldg(m + 2 * cs + c) * w;
    }
    if (fout) {
      fout[3 * p] = f0;
      fout[3 * p + 1] = f1;
      fout[3 * p + 2] = f2;
    }
    vx += kick * f0;
    vy += kick * f1;
    vz += kick * f2;
    vel[3 * p] = vx;
    vel[3 * p + 1] = vy;
    vel[3 * p + 2] = vz;
    pos[3 * p] = x + drift * vx;
    pos[3 * p + 1] = y + drift * vy;
    pos[3 * p + 2] = z + drift * vz;
  }
}

__global__ void axpy3_kernel(float *__restrict__ y, const float *__restrict__ x, int64_t n,
                             float a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}

// One component of a read, written with a stride (the plain form's three
// separate gathers into an [np][3] force array).
__global__ void __launch_bounds__(256)
read_strided_kernel(const float *__restrict__ mesh, int nx, int ny, int nz,
                    const float *__restrict__ pos, int64_t np, float *__restrict__ out,
                    int stride) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float x, y, z;
    load3(pos, p, x, y, z);
    Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
    float s = 0.f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      float w = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                          conn_z(n) ? az.k1 : az.k0);
      s += __ldg(mesh + cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                                   conn_z(n) ? az.i1 : az.i0, ny, nz)) * w;
    }
    out[(int64_t)stride * p] = s;
  }
}

// Paints the three components of per-particle vectors g[p][c] into three
// meshes (the cotangent paint of the read adjoint).
__global__ void __launch_bounds__(256)
paint3_kernel(float *__restrict__ m, int64_t cs, int nx, int ny, int nz,
              const float *__restrict__ pos, int64_t np, const float *__restrict__ g) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float x, y, z, g0, g1, g2;
    load3(pos, p, x, y, z);
    load3(g, p, g0, g1, g2);
    Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      float w = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                          conn_z(n) ? az.k1 : az.k0);
      int64_t c = cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                             conn_z(n) ? az.i1 : az.i0, ny, nz);
      atomicAdd(m + c, g0 * w);
      atomicAdd(m + cs + c, g1 * w);
      atomicAdd(m + 2 * cs + c, g2 * w);
    }
  }
}

// Both position terms of the pm_forces adjoint in one gather:
// g_pos[p][d] = sum_i g[p][i] * d/dx_d read(F_i)(x_p) + d/dx_d read(rho_bar)(x_p).
__global__ void __launch_bounds__(256)
forces_vjp_gather_kernel(const float *__restrict__ f3, int64_t cs,
                         const float *__restrict__ rbar, int nx, int ny, int nz,
                         const float *__restrict__ pos, int64_t np,
                         const float *__restrict__ g, float *__restrict__ gpos) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    float x, y, z, g0, g1, g2;
    load3(pos, p, x, y, z);
    load3(g, p, g0, g1, g2);
    Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
    AxisGrad dx = cic_axis_grad(x), dy = cic_axis_grad(y), dz = cic_axis_grad(z);
    float ox = 0.f, oy = 0.f, oz = 0.f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      float kx = conn_x(n) ? ax.k1 : ax.k0, ky = conn_y(n) ? ay.k1 : ay.k0,
            kz = conn_z(n) ? az.k1 : az.k0;
      float ddx = conn_x(n) ? dx.d1 : dx.d0, ddy = conn_y(n) ? dy.d1 : dy.d0,
            ddz = conn_z(n) ? dz.d1 : dz.d0;
      int64_t c = cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                             conn_z(n) ? az.i1 : az.i0, ny, nz);
      // contracted field: rho_bar + g . F at this cell
      float v = __ldg(rbar + c) + g0 * __ldg(f3 + c) + g1 * __ldg(f3 + cs + c) +
                g2 * __ldg(f3 + 2 * cs + c);
      ox += v * ddx * ky * kz;
      oy += v * kx * ddy * kz;
      oz += v * kx * ky * ddz;
    }
    gpos[3 * p] = ox;
    gpos[3 * p + 1] = oy;
    gpos[3 * p + 2] = oz;
  }
}

// ---------------------------------------------------------------------------
// Workspace of the composite calls (every region 256-byte aligned).
// ---------------------------------------------------------------------------
struct Layout {
  size_t mesh, dk, fk, f3, g3, forces, work, det, total;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static Layout layout(int nx, int ny, int nz, int64_t np, int mode) {
  const size_t ncell = (size_t)nx * ny * nz;
  // spectra sized for the padded rows of the spectral pipeline (a superset
  // of cuFFT's [nx][ny][nz/2+1])
  const size_t nspec = (size_t)nx * ny * spectral_pitch(nz);
  Layout L;
  size_t o = 0;
  L.mesh = o; o = align256(o + ncell * 4);
  L.dk = o; o = align256(o + nspec * 8);
  L.fk = o; o = align256(o + 3 * nspec * 8);
  L.f3 = o; o = align256(o + 3 * ncell * 4);
  L.g3 = o; o = align256(o + 3 * ncell * 4);
  L.forces = o; o = align256(o + (size_t)np * 12);
  L.work = o; o = align256(o + 16);  // tile counter of the dynamically scheduled kernels
  L.det = o;
  if (mode == PMGB_PAINT_DETERMINISTIC) o = align256(o + ncell * 8);
  L.total = o;
  return L;
}

size_t pm_workspace_size(int nx, int ny, int nz, int64_t np, int mode) {
  return layout(nx, ny, nz, np, mode).total;
}

static int check_ws(void *ws, size_t bytes, const Layout &L) {
  if (!ws || bytes < L.total)
    return fail(PMGB_ERR_WORKSPACE, "composite call needs " + std::to_string(L.total) +
                                        " workspace bytes, got " + std::to_string(bytes));
  if (reinterpret_cast<uintptr_t>(ws) % 256 != 0)
    return fail(PMGB_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  return PMGB_OK;
}

#define WS(T, off) reinterpret_cast<T *>(static_cast<char *>(ws) + (off))

static bool aligned16(const void *p) { return reinterpret_cast<uintptr_t>(p) % 16 == 0; }

static bool use_spectral(int nx, int ny, int nz, const void *in, const void *out) {
  return spectral_enabled() && spectral_supported(nx, ny, nz) && aligned16(in) && aligned16(out);
}

// density mesh -> the three force meshes f3: the spectral pipeline where
// the mesh shape allows it (and it is enabled), else R2C -> fused k-space
// kernel -> batched C2R through cuFFT.  dk / fk: one and three spectra of
// spectral_pitch rows.
int mesh_forces(const float *mesh, int nx, int ny, int nz, float r_split, void *dk, void *fk,
                float *f3, cudaStream_t s) {
  const int64_t ncell = (int64_t)nx * ny * nz;
  const int64_t nhalf = (int64_t)nx * ny * (nz / 2 + 1);
  if (use_spectral(nx, ny, nz, mesh, f3))
    return spectral_forces(mesh, dk, fk, f3, nx, ny, nz, r_split, 1, 0, 1.0f / (float)ncell, s);
  PMGB_TRY(fft_r2c(mesh, dk, nx, ny, nz, 1, s));
  PMGB_TRY(kspace_forces(dk, fk, nhalf, nx, ny, nz, r_split, 1, 0, 1.0f / (float)ncell, s));
  return fft_c2r(fk, f3, nx, ny, nz, 3, s);
}

// Adjoint of mesh_forces: the three force-mesh cotangents g3 (read only)
// -> the density-mesh cotangent rbar.
int mesh_forces_vjp(const float *g3, int nx, int ny, int nz, float r_split, void *dk,
                    void *fk, float *rbar, cudaStream_t s) {
  const int64_t ncell = (int64_t)nx * ny * nz;
  const int64_t nhalf = (int64_t)nx * ny * (nz / 2 + 1);
  if (use_spectral(nx, ny, nz, g3, rbar))
    return spectral_forces_vjp(g3, fk, dk, rbar, nx, ny, nz, r_split, 1, 0,
                               1.0f / (float)ncell, s);
  PMGB_TRY(fft_r2c(g3, fk, nx, ny, nz, 3, s));
  PMGB_TRY(kspace_forces_vjp(fk, nhalf, dk, nx, ny, nz, r_split, 1, 0, 1.0f / (float)ncell, s));
  return fft_c2r(dk, rbar, nx, ny, nz, 1, s);
}

// Workspace of the standalone mesh-force calls: one spectrum then three.
size_t mesh_forces_workspace_size(int nx, int ny, int nz) {
  const size_t nspec = (size_t)nx * ny * spectral_pitch(nz);
  return align256(nspec * 8) + align256(3 * nspec * 8);
}

static int mesh_ws(void *ws, size_t bytes, int nx, int ny, int nz, void **dk, void **fk) {
  const size_t need = mesh_forces_workspace_size(nx, ny, nz);
  if (!ws || bytes < need)
    return fail(PMGB_ERR_WORKSPACE, "mesh-force call needs " + std::to_string(need) +
                                        " workspace bytes, got " + std::to_string(bytes));
  if (reinterpret_cast<uintptr_t>(ws) % 256 != 0)
    return fail(PMGB_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  *dk = ws;
  *fk = static_cast<char *>(ws) + align256((size_t)nx * ny * spectral_pitch(nz) * 8);
  return PMGB_OK;
}

int mesh_forces_ws(const float *mesh, float *f3, int nx, int ny, int nz, float r_split,
                   void *ws, size_t bytes, cudaStream_t s) {
  void *dk, *fk;
  PMGB_TRY(mesh_ws(ws, bytes, nx, ny, nz, &dk, &fk));
  return mesh_forces(mesh, nx, ny, nz, r_split, dk, fk, f3, s);
}

int mesh_potential_ws(const float *mesh, float *pot, int nx, int ny, int nz, float r_split,
                      void *ws, size_t bytes, cudaStream_t s) {
  void *dk, *fk;
  PMGB_TRY(mesh_ws(ws, bytes, nx, ny, nz, &dk, &fk));
  if (!spectral_supported(nx, ny, nz))
    return fail(PMGB_ERR_UNSUPPORTED,
                "the potential pipeline needs power-of-two nx in [8,1024], ny in [64,512], "
                "nz in [16,512]");
  return spectral_potential(mesh, dk, pot, nx, ny, nz, r_split,
                            1.0f / (float)((int64_t)nx * ny * nz), s);
}

int mesh_forces_vjp_ws(const float *g3, float *rbar, int nx, int ny, int nz, float r_split,
                       void *ws, size_t bytes, cudaStream_t s) {
  void *dk, *fk;
  PMGB_TRY(mesh_ws(ws, bytes, nx, ny, nz, &dk, &fk));
  return mesh_forces_vjp(g3, nx, ny, nz, r_split, dk, fk, rbar, s);
}

// paint -> the three force meshes at WS(float, L.f3).
static int force_meshes(const float *pos, int64_t np, int nx, int ny, int nz, float r_split,
                        int mode, void *ws, const Layout &L, cudaStream_t s) {
  const int64_t ncell = (int64_t)nx * ny * nz;
  float *mesh = WS(float, L.mesh);
  PMGB_TRY(paint(mesh, nx, ny, nz, pos, np, nullptr, 1.0f, mode, 0, WS(void, L.det),
                 mode == PMGB_PAINT_DETERMINISTIC ? (size_t)ncell * 8 : 0, s));
  return mesh_forces(mesh, nx, ny, nz, r_split, WS(void, L.dk), WS(void, L.fk),
                     WS(float, L.f3), s);
}

int pm_workspace_regions(void *ws, size_t bytes, int nx, int ny, int nz, int64_t np,
                         float **mesh, void **dk, void **fk, float **f3, float **g3,
                         unsigned **work) {
  Layout L = layout(nx, ny, nz, np, PMGB_PAINT_BINNED);
  PMGB_TRY(check_ws(ws, bytes, L));
  *mesh = WS(float, L.mesh);
  *dk = WS(void, L.dk);
  *fk = WS(void, L.fk);
  *f3 = WS(float, L.f3);
  *g3 = WS(float, L.g3);
  *work = WS(unsigned, L.work);
  return PMGB_OK;
}

float *pm_workspace_particles(void *ws, size_t bytes, int nx, int ny, int nz, int64_t np) {
  Layout L = layout(nx, ny, nz, np, PMGB_PAINT_BINNED);
  if (check_ws(ws, bytes, L) != PMGB_OK) return nullptr;
  return WS(float, L.forces);
}

int force_meshes_sorted(const float *pos, int64_t np, int nx, int ny, int nz, float r_split,
                        void *ws, size_t bytes, void *sort_ws, size_t sort_bytes,
                        unsigned *stats, float *f3_out, float **f3, cudaStream_t s) {
  Layout L = layout(nx, ny, nz, np, PMGB_PAINT_BINNED);
  PMGB_TRY(check_ws(ws, bytes, L));
  float *mesh = WS(float, L.mesh);
  PMGB_TRY(paint_sorted(mesh, nx, ny, nz, pos, np, sort_ws, sort_bytes, stats, s));
  *f3 = f3_out ? f3_out : WS(float, L.f3);
  return mesh_forces(mesh, nx, ny, nz, r_split, WS(void, L.dk), WS(void, L.fk), *f3, s);
}

int pm_forces(const float *pos, int64_t np, int nx, int ny, int nz, float r_split, int mode,
              float *forces, void *ws, size_t bytes, cudaStream_t s) {
  Layout L = layout(nx, ny, nz, np, mode);
  PMGB_TRY(check_ws(ws, bytes, L));
  PMGB_TRY(force_meshes(pos, np, nx, ny, nz, r_split, mode, ws, L, s));
  PMGB_TRY(read3(WS(float, L.f3), (int64_t)nx * ny * nz, nx, ny, nz, pos, np, forces, s));
  return PMGB_OK;
}

int read3_kick_drift(const float *f3, int64_t cs, int nx, int ny, int nz, float *pos,
                     float *vel, int64_t np, float kick, float drift, float *fout,
                     cudaStream_t s) {
  if (np == 0) return PMGB_OK;
  read3_kick_drift_kernel<<<wave_grid(read3_kick_drift_kernel, np, 256), 256, 0, s>>>(
      f3, cs, nx, ny, nz, pos, vel, np, kick, drift, fout);
  PMGB_LAUNCHED("read3_kick_drift_kernel");
  return PMGB_OK;
}

int fpm_step(float *pos, float *vel, int64_t np, int nx, int ny, int nz, float kick,
             float drift, float r_split, int mode, void *ws, size_t bytes, cudaStream_t s) {
  Layout L = layout(nx, ny, nz, np, mode);
  PMGB_TRY(check_ws(ws, bytes, L));
  PMGB_TRY(force_meshes(pos, np, nx, ny, nz, r_split, mode, ws, L, s));
  PMGB_TRY(read3_kick_drift(WS(float, L.f3), (int64_t)nx * ny * nz, nx, ny, nz, pos, vel, np,
                            kick, drift, nullptr, s));
  return PMGB_OK;
}

int kick(float *vel, const float *forces, int64_t np, float k, cudaStream_t s) {
  if (np == 0) return PMGB_OK;
  axpy3_kernel<<<wave_grid(axpy3_kernel, 3 * np, 256), 256, 0, s>>>(vel, forces, 3 * np, k);
  PMGB_LAUNCHED("kick(axpy3_kernel)");
  return PMGB_OK;
}

int drift(float *pos, const float *vel, int64_t np, float d, cudaStream_t s) {
  if (np == 0) return PMGB_OK;
  axpy3_kernel<<<wave_grid(axpy3_kernel, 3 * np, 256), 256, 0, s>>>(pos, vel, 3 * np, d);
  PMGB_LAUNCHED("drift(axpy3_kernel)");
  return PMGB_OK;
}

int fpm_step_plain(float *pos, float *vel, int64_t np, int nx, int ny, int nz, float kk,
                   float dd, float r_split, void *ws, size_t bytes, cudaStream_t s) {
  Layout L = layout(nx, ny, nz, np, PMGB_PAINT_ATOMIC);
  PMGB_TRY(check_ws(ws, bytes, L));
  const int64_t ncell = (int64_t)nx * ny * nz;
  const int64_t nhalf = (int64_t)nx * ny * (nz / 2 + 1);
  float *mesh = WS(float, L.mesh);
  float2 *dk = WS(float2, L.dk);
  float2 *fk = WS(float2, L.fk);
  float *f3 = WS(float, L.f3);
  float *forces = WS(float, L.forces);
  PMGB_TRY(paint(mesh, nx, ny, nz, pos, np, nullptr, 1.0f, PMGB_PAINT_ATOMIC, 0, nullptr, 0, s));
  PMGB_TRY(fft_r2c(mesh, dk, nx, ny, nz, 1, s));
  PMGB_TRY(kspace_invlaplace(dk, nx, ny, nz, 0, 1.0f / (float)ncell, s));
  if (r_split != 0.0f) PMGB_TRY(kspace_longrange(dk, nx, ny, nz, r_split, s));
  for (int d = 0; d < 3; ++d) {
    PMGB_TRY(kspace_gradient(dk, fk + d * nhalf, nx, ny, nz, d, 1, s));
    PMGB_TRY(fft_c2r(fk + d * nhalf, f3 + d * ncell, nx, ny, nz, 1, s));
  }
  if (np > 0) {
    for (int d = 0; d < 3; ++d) {
      read_strided_kernel<<<wave_grid(read_strided_kernel, np, 256), 256, 0, s>>>(
          f3 + d * ncell, nx, ny, nz, pos, np, forces + d, 3);
      PMGB_LAUNCHED("read_strided_kernel");
    }
  }
  PMGB_TRY(kick(vel, forces, np, kk, s));
  PMGB_TRY(drift(pos, vel, np, dd, s));
  return PMGB_OK;
}

int pm_forces_vjp(const float *pos, int64_t np, int nx, int ny, int nz, float r_split,
                  int mode, const float *g, float *gpos, void *ws, size_t bytes,
                  cudaStream_t s) {
  Layout L = layout(nx, ny, nz, np, mode);
  PMGB_TRY(check_ws(ws, bytes, L));
  const int64_t ncell = (int64_t)nx * ny * nz;
  PMGB_TRY(force_meshes(pos, np, nx, ny, nz, r_split, mode, ws, L, s));
  float *g3 = WS(float, L.g3);
  PMGB_CUDA(cudaMemsetAsync(g3, 0, 3 * ncell * sizeof(float), s));
  if (np > 0) {
    paint3_kernel<<<wave_grid(paint3_kernel, np, 256), 256, 0, s>>>(
        g3, ncell, nx, ny, nz, pos, np, g);
    PMGB_LAUNCHED("paint3_kernel");
  }
  float *rbar = WS(float, L.mesh);
  PMGB_TRY(mesh_forces_vjp(g3, nx, ny, nz, r_split, WS(void, L.dk), WS(void, L.fk), rbar, s));
  if (np > 0) {
    forces_vjp_gather_kernel<<<wave_grid(forces_vjp_gather_kernel, np, 256), 256, 0, s>>>(
        WS(float, L.f3), ncell, rbar, nx, ny, nz, pos, np, g, gpos);
    PMGB_LAUNCHED("forces_vjp_gather_kernel");
  }
  return PMGB_OK;
}

}  // namespace pmgb
