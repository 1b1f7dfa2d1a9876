// Batched FastPM: many independent simulations, of possibly different mesh
// shapes, advanced together with each phase of a step issued once for the
// whole batch.  The reference batches independent simulations with
// jax.vmap over its step (README.md:29; tests/test_distributed_pm.py:335-409
// vmap independent simulations); the per-simulation arithmetic is that of
// the single-simulation step (pm.py:12-58 forces, ode.py:13-82 kick/drift).
//
// Layout.  Simulations are grouped by mesh shape: groups in order of first
// appearance in the table, the simulations of a group in table order.  A
// group's meshes and spectra are contiguous with a uniform stride, so one
// batched cuFFT plan transforms the whole group:
//   mesh pool  [group][sim][nx][ny][nz]           f32  (density, then potential;
//                                                       adjoint: potential cotangent, rho_bar)
//   dk pool    [group][sim][nx][ny][nz/2+1]       c64
//   f3 pool    [group][sim][3][nx][ny][nz]        f32  (force meshes)
//   g3 pool    [group][sim][3][nx][ny][nz]        f32  (adjoint: force-mesh cotangents)
// Particles are the concatenation, in table order, of every simulation's
// [np][3] positions (and velocities).
//
// Kernels.  The particle kernels (paint, gather + kick + drift, and the two
// adjoint kernels) are one launch over every particle of the batch with one
// particle per thread: block b belongs to the simulation whose first block
// is the largest not above b (binary search of the device descriptor
// table), so a block never straddles two simulations and reads its own mesh
// shape, pool offsets and kick/drift coefficients.  The forces come from the
// potentials: one batched cuFFT R2C per group, one k-space launch over all
// groups' spectra (the potential multiply, in place), one batched C2R per
// group, and the order-1 gradient as its real-space stencil (one launch per
// group); plans are made when the workspace is initialised (so that a step
// can be captured in a CUDA graph).
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "kspace.cuh"

namespace pmgb {

namespace {

constexpr int BT = 256;            // threads per block, one particle per thread
constexpr int MAX_KGROUPS = 8;     // shape groups per k-space launch
constexpr int MAX_SIMS = 1 << 16;  // simulations per table

// Device descriptor of one simulation (table order).
struct BatchSim {
  int nx, ny, nz, group;
  int64_t p0, np;  // particle range in the concatenated arrays
  int64_t blk0;    // first block of its particles in the particle kernels
  int64_t mesh;    // float offset of its density mesh in the mesh pool
  int64_t f3;      // float offset of its force meshes in the f3 / g3 pools
  int64_t cell0;   // float offset of its mesh in a table-ordered mesh set
};

struct Group {
  int nx, ny, nz, n;  // shape and number of simulations
  int64_t mesh;       // float offset of its first mesh in the mesh pool
  int64_t spec;       // complex offset of its first spectrum in the dk pool
};

struct Plan {
  std::vector<BatchSim> sims;
  std::vector<Group> groups;
  int64_t np = 0, cells = 0, specs = 0, blocks = 0;
  size_t o_desc = 0, o_mesh = 0, o_dk = 0, o_f3 = 0, o_g3 = 0, total = 0;
  uint64_t key = 0;
};

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

uint64_t fnv(uint64_t h, int64_t v) {
  for (int i = 0; i < 8; ++i) {
    h ^= (uint64_t)((v >> (8 * i)) & 0xff);
    h *= 1099511628211ull;
  }
  return h;
}

int make_plan(const pmgb_sim *t, int n, Plan *P) {
  PMGB_REQUIRE(t != nullptr, "sims is NULL");
  PMGB_REQUIRE(n >= 1 && n <= MAX_SIMS,
               "n_sims must be in [1, " + std::to_string(MAX_SIMS) + "], got " +
                   std::to_string(n));
  P->sims.assign(n, BatchSim{});
  P->groups.clear();
  uint64_t key = 1469598103934665603ull;
  key = fnv(key, n);
  std::vector<int> gid(n);
  for (int i = 0; i < n; ++i) {
    PMGB_TRY(check_mesh(t[i].nx, t[i].ny, t[i].nz));
    PMGB_REQUIRE(t[i].np >= 0, "sims[" + std::to_string(i) + "].np is negative");
    const int64_t half = (int64_t)t[i].nx * t[i].ny * (t[i].nz / 2 + 1);
    PMGB_REQUIRE(half < (int64_t)INT32_MAX,
                 "sims[" + std::to_string(i) + "]: mesh too large for a batched simulation");
    int g = -1;
    for (size_t k = 0; k < P->groups.size(); ++k)
      if (P->groups[k].nx == t[i].nx && P->groups[k].ny == t[i].ny && P->groups[k].nz == t[i].nz)
        g = (int)k;
    if (g < 0) {
      P->groups.push_back(Group{t[i].nx, t[i].ny, t[i].nz, 0, 0, 0});
      g = (int)P->groups.size() - 1;
    }
    gid[i] = g;
    P->groups[g].n++;
    key = fnv(fnv(fnv(fnv(key, t[i].nx), t[i].ny), t[i].nz), t[i].np);
  }
  // group pools, each group starting on a 256-byte boundary (cuFFT wants
  // aligned batches; the vector reductions of the painters 16 bytes)
  int64_t mesh = 0, spec = 0;
  for (Group &g : P->groups) {
    g.mesh = mesh;
    g.spec = spec;
    mesh += ((int64_t)g.n * g.nx * g.ny * g.nz + 63) / 64 * 64;
    spec += ((int64_t)g.n * g.nx * g.ny * (g.nz / 2 + 1) + 31) / 32 * 32;
  }
  P->cells = mesh;
  P->specs = spec;
  // simulations: particle ranges and blocks in table order, pool slots in group order
  std::vector<int> used(P->groups.size(), 0);
  int64_t p0 = 0, blk = 0, cell0 = 0;
  for (int i = 0; i < n; ++i) {
    const Group &g = P->groups[gid[i]];
    const int64_t nc = (int64_t)g.nx * g.ny * g.nz;
    BatchSim &d = P->sims[i];
    d.nx = g.nx;
    d.ny = g.ny;
    d.nz = g.nz;
    d.group = gid[i];
    d.p0 = p0;
    d.np = t[i].np;
    d.blk0 = blk;
    const int slot = used[gid[i]]++;
    d.mesh = g.mesh + slot * nc;
    d.f3 = 3 * g.mesh + slot * 3 * nc;
    d.cell0 = cell0;
    p0 += t[i].np;
    blk += (t[i].np + BT - 1) / BT;
    cell0 += nc;
  }
  PMGB_REQUIRE(blk < (int64_t)INT32_MAX, "too many particles in the batch");
  P->np = p0;
  P->blocks = blk;
  size_t o = 0;
  P->o_desc = o; o = al256(o + (size_t)n * sizeof(BatchSim));
  P->o_mesh = o; o = al256(o + (size_t)P->cells * 4);
  P->o_dk = o;   o = al256(o + (size_t)P->specs * 8);
  P->o_f3 = o;   o = al256(o + (size_t)P->cells * 3 * 4);
  P->o_g3 = o;   o = al256(o + (size_t)P->cells * 3 * 4);
  P->total = o;
  P->key = key;
  return PMGB_OK;
}

// workspace -> key of the table it was initialised for
std::mutex g_mu;
std::map<const void *, uint64_t> g_ready;

// Builds the plan and checks that `ws` was initialised for this table.
int bind(const pmgb_sim *t, int n, void *ws, size_t bytes, Plan *P) {
  PMGB_TRY(make_plan(t, n, P));
  PMGB_REQUIRE(ws != nullptr, "workspace is NULL");
  if (bytes < P->total)
    return fail(PMGB_ERR_WORKSPACE, "batched call needs " + std::to_string(P->total) +
                                        " workspace bytes, got " + std::to_string(bytes));
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_ready.find(ws);
  if (it == g_ready.end() || it->second != P->key)
    return fail(PMGB_ERR_INVALID_ARGUMENT,
                "workspace was not initialised for this simulation table "
                "(call pmgb_batch_init first)");
  return PMGB_OK;
}

#define BW(T, off) reinterpret_cast<T *>(static_cast<char *>(ws) + (off))

// ---------------------------------------------------------------------------
// Particle kernels
// ---------------------------------------------------------------------------

__device__ __forceinline__ int sim_of_block(const BatchSim *__restrict__ sims, int n, int64_t b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sims[mid].blk0 <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// This thread's simulation and particle; false past the simulation's end.
__device__ __forceinline__ bool locate(const BatchSim *__restrict__ sims, int n, int &s,
                                       BatchSim &d, int64_t &p) {
  s = sim_of_block(sims, n, blockIdx.x);
  d = sims[s];
  const int64_t local = ((int64_t)blockIdx.x - d.blk0) * BT + threadIdx.x;
  p = d.p0 + local;
  return local < d.np;
}

__device__ __forceinline__ float corner_weight(const Axis &ax, const Axis &ay, const Axis &az,
                                               int n) {
  return __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                   conn_z(n) ? az.k1 : az.k0);
}

__device__ __forceinline__ int64_t corner_cell(const Axis &ax, const Axis &ay, const Axis &az,
                                               int n, int ny, int nz) {
  return cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                    conn_z(n) ? az.i1 : az.i0, ny, nz);
}

// Unit-mass CIC paint of every simulation into its mesh (pool slot, or the
// table-ordered slot when `table_order`).
__global__ void __launch_bounds__(BT)
batch_paint_kernel(const BatchSim *__restrict__ sims, int n, float *__restrict__ meshes,
                   int table_order, const float *__restrict__ pos, bool vec_ok) {
  int s;
  BatchSim d;
  int64_t p;
  if (!locate(sims, n, s, d, p)) return;
  float x, y, z;
  load3(pos, p, x, y, z);
  const int64_t off = table_order ? d.cell0 : d.mesh;
  float *m = meshes + off;
  const Axis ax = cic_axis(x, d.nx), ay = cic_axis(y, d.ny), az = cic_axis(z, d.nz);
  // vector reductions need every row 16-byte aligned: base, mesh offset and nz
  const bool vec = vec_ok && (d.nz & 3) == 0 && (off & 3) == 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int cx = c & 1, cy = c >> 1;
    const float kxy = __fmul_rn(cx ? ax.k1 : ax.k0, cy ? ay.k1 : ay.k0);
    red_zpair(m + cell_index(cx ? ax.i1 : ax.i0, cy ? ay.i1 : ay.i0, 0, d.ny, d.nz), az.i0,
              az.i1, __fmul_rn(kxy, az.k0), __fmul_rn(kxy, az.k1), vec);
  }
}

// Three-component read at the particles (forces of pm_forces).
__global__ void __launch_bounds__(BT)
batch_read3_kernel(const BatchSim *__restrict__ sims, int n, const float *__restrict__ f3pool,
                   const float *__restrict__ pos, float *__restrict__ out) {
  int s;
  BatchSim d;
  int64_t p;
  if (!locate(sims, n, s, d, p)) return;
  float x, y, z;
  load3(pos, p, x, y, z);
  const float *m = f3pool + d.f3;
  const int64_t cs = (int64_t)d.nx * d.ny * d.nz;
  const Axis ax = cic_axis(x, d.nx), ay = cic_axis(y, d.ny), az = cic_axis(z, d.nz);
  float f0 = 0.f, f1 = 0.f, f2 = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const float w = corner_weight(ax, ay, az, c);
    const int64_t e = corner_cell(ax, ay, az, c, d.ny, d.nz);
    f0 += __ldg(m + e) * w;
    f1 += __ldg(m + cs + e) * w;
    f2 += __ldg(m + 2 * cs + e) * w;
  }
  out[3 * p] = f0;
  out[3 * p + 1] = f1;
  out[3 * p + 2] = f2;
}

// Gather of the three force meshes + kick + drift with the simulation's own
// coefficients (ode.py:13-82: v += kick F(x); x += drift v).  `pos_before`
// (optional) receives the positions before the step.
__global__ void __launch_bounds__(BT)
batch_rkd_kernel(const BatchSim *__restrict__ sims, int n, const float *__restrict__ f3pool,
                 float *__restrict__ pos, float *__restrict__ vel,
                 const float *__restrict__ kick, const float *__restrict__ drift,
                 float *__restrict__ pos_before) {
  int s;
  BatchSim d;
  int64_t p;
  if (!locate(sims, n, s, d, p)) return;
  const float x = pos[3 * p], y = pos[3 * p + 1], z = pos[3 * p + 2];
  float vx = vel[3 * p], vy = vel[3 * p + 1], vz = vel[3 * p + 2];
  const float *m = f3pool + d.f3;
  const int64_t cs = (int64_t)d.nx * d.ny * d.nz;
  const Axis ax = cic_axis(x, d.nx), ay = cic_axis(y, d.ny), az = cic_axis(z, d.nz);
  float f0 = 0.f, f1 = 0.f, f2 = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const float w = corner_weight(ax, ay, az, c);
    const int64_t e = corner_cell(ax, ay, az, c, d.ny, d.nz);
    f0 += __ldg(m + e) * w;
    f1 += __ldg(m + cs + e) * w;
    f2 += __ldg(m + 2 * cs + e) * w;
  }
  const float kk = __ldg(kick + s), dd = __ldg(drift + s);
  if (pos_before) {
    pos_before[3 * p] = x;
    pos_before[3 * p + 1] = y;
    pos_before[3 * p + 2] = z;
  }
  vx += kk * f0;
  vy += kk * f1;
  vz += kk * f2;
  vel[3 * p] = vx;
  vel[3 * p + 1] = vy;
  vel[3 * p + 2] = vz;
  pos[3 * p] = x + dd * vx;
  pos[3 * p + 1] = y + dd * vy;
  pos[3 * p + 2] = z + dd * vz;
}

// Adjoint, first pass: u = g_vel + drift g_pos (the velocity cotangent
// after the drift transpose), painted as kick*u at the step's starting
// positions into the three force-mesh cotangents (the read transpose).
__global__ void __launch_bounds__(BT)
batch_adj_paint_kernel(const BatchSim *__restrict__ sims, int n, float *__restrict__ g3pool,
                       const float *__restrict__ pos, const float *__restrict__ gpos,
                       const float *__restrict__ gvel, const float *__restrict__ kick,
                       const float *__restrict__ drift, bool vec_ok) {
  int s;
  BatchSim d;
  int64_t p;
  if (!locate(sims, n, s, d, p)) return;
  float x, y, z, gx, gy, gz, vx, vy, vz;
  load3(pos, p, x, y, z);
  load3(gpos, p, gx, gy, gz);
  load3(gvel, p, vx, vy, vz);
  const float kk = __ldg(kick + s), dd = __ldg(drift + s);
  const float u0 = kk * (vx + dd * gx), u1 = kk * (vy + dd * gy), u2 = kk * (vz + dd * gz);
  float *m = g3pool + d.f3;
  const int64_t cs = (int64_t)d.nx * d.ny * d.nz;
  const Axis ax = cic_axis(x, d.nx), ay = cic_axis(y, d.ny), az = cic_axis(z, d.nz);
  // vector reductions need every row of the three meshes 16-byte aligned
  const bool vec = vec_ok && (d.nz & 3) == 0 && (d.f3 & 3) == 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int cx = c & 1, cy = c >> 1;
    const float kxy = __fmul_rn(cx ? ax.k1 : ax.k0, cy ? ay.k1 : ay.k0);
    const float wa = __fmul_rn(kxy, az.k0), wb = __fmul_rn(kxy, az.k1);
    float *row = m + cell_index(cx ? ax.i1 : ax.i0, cy ? ay.i1 : ay.i0, 0, d.ny, d.nz);
    red_zpair(row, az.i0, az.i1, u0 * wa, u0 * wb, vec);
    red_zpair(row + cs, az.i0, az.i1, u1 * wa, u1 * wb, vec);
    red_zpair(row + 2 * cs, az.i0, az.i1, u2 * wa, u2 * wb, vec);
  }
}

// Adjoint, second pass: g_pos += d/dx [read(rho_bar) + (kick u) . read(F)]
// at the starting positions (the position terms of the read and of the
// paint), and g_vel = u.
__global__ void __launch_bounds__(BT)
batch_adj_gather_kernel(const BatchSim *__restrict__ sims, int n,
                        const float *__restrict__ f3pool, const float *__restrict__ rbar_pool,
                        const float *__restrict__ pos, float *__restrict__ gpos,
                        float *__restrict__ gvel, const float *__restrict__ kick,
                        const float *__restrict__ drift) {
  int s;
  BatchSim d;
  int64_t p;
  if (!locate(sims, n, s, d, p)) return;
  float x, y, z;
  load3(pos, p, x, y, z);
  float gx = gpos[3 * p], gy = gpos[3 * p + 1], gz = gpos[3 * p + 2];
  const float vx = gvel[3 * p], vy = gvel[3 * p + 1], vz = gvel[3 * p + 2];
  const float kk = __ldg(kick + s), dd = __ldg(drift + s);
  const float w0 = vx + dd * gx, w1 = vy + dd * gy, w2 = vz + dd * gz;  // u
  const float u0 = kk * w0, u1 = kk * w1, u2 = kk * w2;
  const float *f3 = f3pool + d.f3;
  const float *rb = rbar_pool + d.mesh;
  const int64_t cs = (int64_t)d.nx * d.ny * d.nz;
  const Axis ax = cic_axis(x, d.nx), ay = cic_axis(y, d.ny), az = cic_axis(z, d.nz);
  const AxisGrad dx = cic_axis_grad(x), dy = cic_axis_grad(y), dz = cic_axis_grad(z);
  float ox = 0.f, oy = 0.f, oz = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const float kx = conn_x(c) ? ax.k1 : ax.k0, ky = conn_y(c) ? ay.k1 : ay.k0,
                kz = conn_z(c) ? az.k1 : az.k0;
    const float ddx = conn_x(c) ? dx.d1 : dx.d0, ddy = conn_y(c) ? dy.d1 : dy.d0,
                ddz = conn_z(c) ? dz.d1 : dz.d0;
    const int64_t e = corner_cell(ax, ay, az, c, d.ny, d.nz);
    const float v = __ldg(rb + e) + u0 * __ldg(f3 + e) + u1 * __ldg(f3 + cs + e) +
                    u2 * __ldg(f3 + 2 * cs + e);
    ox += v * ddx * ky * kz;
    oy += v * kx * ddy * kz;
    oz += v * kx * ky * ddz;
  }
  gpos[3 * p] = gx + ox;
  gpos[3 * p + 1] = gy + oy;
  gpos[3 * p + 2] = gz + oz;
  gvel[3 * p] = w0;
  gvel[3 * p + 1] = w1;
  gvel[3 * p + 2] = w2;
}

// ---------------------------------------------------------------------------
// k-space: one launch over the spectra of up to MAX_KGROUPS shape groups
// ---------------------------------------------------------------------------

struct KGroup {
  Tables t;
  uint32_t ny, nzh, total;  // per-simulation half spectrum
  float scale;              // 1 / ncell
  int64_t start;            // first element of the group in the dk pool
  int64_t count;            // elements of the group (simulations x total)
};

struct KGroups {
  KGroup g[MAX_KGROUPS];
  int count;
  int64_t begin, end;  // element range of this launch in the dk pool
};

__device__ __forceinline__ int kgroup_of(const KGroups &G, int64_t e) {
  int k = 0;
#pragma unroll
  for (int i = 1; i < MAX_KGROUPS; ++i)
    if (i < G.count && e >= G.g[i].start) k = i;
  return k;
}

__device__ __forceinline__ Elem kelement(const KGroup &g, uint32_t el) {
  const uint32_t k = el % g.nzh, r = el / g.nzh, j = r % g.ny, i = r / g.ny;
  Elem E;
  E.X = g.t.x[i];
  E.Y = g.t.y[j];
  E.Z = g.t.z[k];
  return E;
}

// dk [sim][half] *= invlaplace * longrange * scale, in place: the spectra of
// the potentials (the forces are their order-1 stencil gradients).
__global__ void __launch_bounds__(256)
batch_potential_kernel(float2 *__restrict__ dk, KGroups G, float r2) {
  for (int64_t e = G.begin + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < G.end;
       e += (int64_t)gridDim.x * blockDim.x) {
    const KGroup &g = G.g[kgroup_of(G, e)];
    const int64_t local = e - g.start;
    if (local >= g.count) continue;  // padding between groups
    const int64_t inst = local / g.total;
    const uint32_t el = (uint32_t)(local - inst * g.total);
    const Elem E = kelement(g, el);
    const float inv = inv_laplace(E, 0), L = long_range(E, r2);
    const float2 d = dk[e];
    dk[e] = make_float2(__fmul_rn(__fmul_rn(d.x, inv), L) * g.scale,
                        __fmul_rn(__fmul_rn(d.y, inv), L) * g.scale);
  }
}

// The potentials' spectra for every group, in place (one launch per
// MAX_KGROUPS groups).  The multiply is symmetric, so the adjoint is the
// same operation.
int kspace_potential_batched(const Plan &P, float2 *dk, float r_split, cudaStream_t s) {
  const size_t ng = P.groups.size();
  for (size_t g0 = 0; g0 < ng; g0 += MAX_KGROUPS) {
    KGroups G;
    std::memset(&G, 0, sizeof(G));
    G.count = (int)std::min(ng - g0, (size_t)MAX_KGROUPS);
    for (int k = 0; k < G.count; ++k) {
      const Group &gr = P.groups[g0 + k];
      KGroup &kg = G.g[k];
      PMGB_TRY(tables(gr.nx, gr.ny, gr.nz, &kg.t));
      kg.ny = (uint32_t)gr.ny;
      kg.nzh = (uint32_t)(gr.nz / 2 + 1);
      kg.total = (uint32_t)((int64_t)gr.nx * gr.ny * kg.nzh);
      kg.scale = 1.0f / (float)((int64_t)gr.nx * gr.ny * gr.nz);
      kg.start = gr.spec;
      kg.count = (int64_t)gr.n * kg.total;
    }
    G.begin = G.g[0].start;
    const Group &last = P.groups[g0 + G.count - 1];
    G.end = last.spec + (int64_t)last.n * last.nx * last.ny * (last.nz / 2 + 1);
    batch_potential_kernel<<<wave_grid(batch_potential_kernel, G.end - G.begin, 256), 256, 0, s>>>(
        dk, G, r_split * r_split);
    PMGB_LAUNCHED("batch_potential_kernel");
  }
  return PMGB_OK;
}

// density pool -> f3 pool through the potentials: R2C per group, one
// k-space launch (in place), C2R per group into the mesh pool (the density
// is no longer needed), then the order-1 gradient as a real-space stencil
// per group (jaxpm/kernels.py:41-66: the multiplier i g(w) is the transfer
// function of the stencil), one inverse transform per simulation instead of
// three.
int batch_mesh_forces(const Plan &P, void *ws, float r_split, cudaStream_t s) {
  float *mesh = BW(float, P.o_mesh);
  float2 *dk = BW(float2, P.o_dk);
  float *f3 = BW(float, P.o_f3);
  for (const Group &g : P.groups)
    PMGB_TRY(fft_r2c(mesh + g.mesh, dk + g.spec, g.nx, g.ny, g.nz, g.n, s));
  PMGB_TRY(kspace_potential_batched(P, dk, r_split, s));
  for (const Group &g : P.groups) {
    PMGB_TRY(fft_c2r(dk + g.spec, mesh + g.mesh, g.nx, g.ny, g.nz, g.n, s));
    PMGB_TRY(stencil_forces(mesh + g.mesh, f3 + 3 * g.mesh, g.nx, g.ny, g.nz, g.n, s));
  }
  return PMGB_OK;
}

// g3 pool -> rho_bar in the mesh pool (adjoint of batch_mesh_forces): the
// potential cotangents sum_c D_c g_c by the stencil, then the symmetric
// k-space multiply between one R2C and one C2R per group.
int batch_mesh_forces_vjp(const Plan &P, void *ws, float r_split, cudaStream_t s) {
  float *rbar = BW(float, P.o_mesh);
  float2 *dk = BW(float2, P.o_dk);
  float *g3 = BW(float, P.o_g3);
  for (const Group &g : P.groups) {
    PMGB_TRY(stencil_adjoint(g3 + 3 * g.mesh, rbar + g.mesh, g.nx, g.ny, g.nz, g.n, s));
    PMGB_TRY(fft_r2c(rbar + g.mesh, dk + g.spec, g.nx, g.ny, g.nz, g.n, s));
  }
  PMGB_TRY(kspace_potential_batched(P, dk, r_split, s));
  for (const Group &g : P.groups)
    PMGB_TRY(fft_c2r(dk + g.spec, rbar + g.mesh, g.nx, g.ny, g.nz, g.n, s));
  return PMGB_OK;
}

const BatchSim *desc(const Plan &P, void *ws) { return BW(const BatchSim, P.o_desc); }

// paint of every simulation's density into the mesh pool
int batch_density(const Plan &P, void *ws, const float *pos, cudaStream_t s) {
  float *mesh = BW(float, P.o_mesh);
  PMGB_CUDA(cudaMemsetAsync(mesh, 0, (size_t)P.cells * 4, s));
  if (P.blocks == 0) return PMGB_OK;
  // scalar reductions: lattice-ordered particles of a warp hit consecutive
  // cells, which the vector form would serialise (measured slower here)
  batch_paint_kernel<<<(unsigned)P.blocks, BT, 0, s>>>(desc(P, ws), (int)P.sims.size(), mesh, 0,
                                                       pos, false);
  PMGB_LAUNCHED("batch_paint_kernel");
  return PMGB_OK;
}

}  // namespace

size_t batch_workspace_size(const pmgb_sim *t, int n) {
  Plan P;
  if (make_plan(t, n, &P) != PMGB_OK) return 0;
  return P.total;
}

int batch_init(const pmgb_sim *t, int n, void *ws, size_t bytes, cudaStream_t s) {
  Plan P;
  PMGB_TRY(make_plan(t, n, &P));
  PMGB_REQUIRE(ws != nullptr, "workspace is NULL");
  if (bytes < P.total)
    return fail(PMGB_ERR_WORKSPACE, "batched call needs " + std::to_string(P.total) +
                                        " workspace bytes, got " + std::to_string(bytes));
  if (reinterpret_cast<uintptr_t>(ws) % 256 != 0)
    return fail(PMGB_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  // the descriptor table (the copy from pageable memory returns once the
  // host data has been staged)
  PMGB_CUDA(cudaMemcpyAsync(BW(void, P.o_desc), P.sims.data(), P.sims.size() * sizeof(BatchSim),
                            cudaMemcpyHostToDevice, s));
  // FFT plans and k-space tables of every group, made now so that the
  // steps launch work only
  for (const Group &g : P.groups) {
    PMGB_TRY(fft_prepare(g.nx, g.ny, g.nz, g.n, 1));
    PMGB_TRY(fft_prepare(g.nx, g.ny, g.nz, g.n, 0));
    Tables tb;
    PMGB_TRY(tables(g.nx, g.ny, g.nz, &tb));
  }
  std::lock_guard<std::mutex> lk(g_mu);
  g_ready[ws] = P.key;
  return PMGB_OK;
}

int batch_release(const void *ws) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_ready.erase(ws);
  return PMGB_OK;
}

int cic_paint_batched(const pmgb_sim *t, int n, float *meshes, const float *pos, void *ws,
                      size_t bytes, cudaStream_t s) {
  Plan P;
  PMGB_TRY(bind(t, n, ws, bytes, &P));
  PMGB_CUDA(cudaMemsetAsync(meshes, 0, (size_t)P.cells * 4, s));
  if (P.blocks == 0) return PMGB_OK;
  const bool vec = reinterpret_cast<uintptr_t>(meshes) % 16 == 0;
  batch_paint_kernel<<<(unsigned)P.blocks, BT, 0, s>>>(desc(P, ws), n, meshes, 1, pos, vec);
  PMGB_LAUNCHED("batch_paint_kernel");
  return PMGB_OK;
}

int pm_forces_batched(const pmgb_sim *t, int n, const float *pos, float *forces, float r_split,
                      void *ws, size_t bytes, cudaStream_t s) {
  Plan P;
  PMGB_TRY(bind(t, n, ws, bytes, &P));
  PMGB_TRY(batch_density(P, ws, pos, s));
  PMGB_TRY(batch_mesh_forces(P, ws, r_split, s));
  if (P.blocks == 0) return PMGB_OK;
  batch_read3_kernel<<<(unsigned)P.blocks, BT, 0, s>>>(desc(P, ws), n, BW(float, P.o_f3), pos,
                                                       forces);
  PMGB_LAUNCHED("batch_read3_kernel");
  return PMGB_OK;
}

int fpm_step_batched(const pmgb_sim *t, int n, float *pos, float *vel, const float *kick,
                     const float *drift, float r_split, float *pos_before, void *ws,
                     size_t bytes, cudaStream_t s) {
  Plan P;
  PMGB_TRY(bind(t, n, ws, bytes, &P));
  PMGB_TRY(batch_density(P, ws, pos, s));
  PMGB_TRY(batch_mesh_forces(P, ws, r_split, s));
  if (P.blocks == 0) return PMGB_OK;
  batch_rkd_kernel<<<(unsigned)P.blocks, BT, 0, s>>>(desc(P, ws), n, BW(float, P.o_f3), pos, vel,
                                                     kick, drift, pos_before);
  PMGB_LAUNCHED("batch_rkd_kernel");
  return PMGB_OK;
}

int fpm_step_batched_vjp(const pmgb_sim *t, int n, const float *pos, float *gpos, float *gvel,
                         const float *kick, const float *drift, float r_split, void *ws,
                         size_t bytes, cudaStream_t s) {
  Plan P;
  PMGB_TRY(bind(t, n, ws, bytes, &P));
  // forces at the step's starting positions (recomputed)
  PMGB_TRY(batch_density(P, ws, pos, s));
  PMGB_TRY(batch_mesh_forces(P, ws, r_split, s));
  float *g3 = BW(float, P.o_g3);
  PMGB_CUDA(cudaMemsetAsync(g3, 0, (size_t)P.cells * 3 * 4, s));
  if (P.blocks > 0) {
    batch_adj_paint_kernel<<<(unsigned)P.blocks, BT, 0, s>>>(desc(P, ws), n, g3, pos, gpos,
                                                             gvel, kick, drift, false);
    PMGB_LAUNCHED("batch_adj_paint_kernel");
  }
  PMGB_TRY(batch_mesh_forces_vjp(P, ws, r_split, s));
  if (P.blocks > 0) {
    batch_adj_gather_kernel<<<(unsigned)P.blocks, BT, 0, s>>>(
        desc(P, ws), n, BW(float, P.o_f3), BW(float, P.o_mesh), pos, gpos, gvel, kick, drift);
    PMGB_LAUNCHED("batch_adj_gather_kernel");
  }
  return PMGB_OK;
}

int batch_counts(const pmgb_sim *t, int n, int64_t *np_total, int64_t *cells_total) {
  Plan P;
  PMGB_TRY(make_plan(t, n, &P));
  if (np_total) *np_total = P.np;
  if (cells_total) *cells_total = P.cells;
  return PMGB_OK;
}

}  // namespace pmgb
