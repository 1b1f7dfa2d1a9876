// Tile-sorted particle kernels: counting sort by mesh tile, shared-memory
// box painting and box-staged gather + kick + drift.
//
// Particles are kept physically ordered by the 8^3-cell mesh tile that holds
// them (tiles in Morton order), so a CTA's chunk of consecutive particles
// covers a compact box of cells.  The painter accumulates that box in shared
// memory and flushes it with 16-byte vector atomics; the gather stages the
// box of the three force meshes in shared memory and interpolates from
// there.  The sort is a counting sort: the gather kernel, which computes the
// new positions, also counts them per tile and records each particle's rank
// in its tile (warp-aggregated atomics); an exclusive scan turns counts into
// offsets; a scatter pass moves (pos, vel, id) to offset + rank.
//
// Reference semantics are unchanged: every particle's CIC indices and
// weights are computed exactly as in jaxpm/painting.py:21-37 (common.cuh)
// from its own unwrapped position; the box only changes where partial sums
// are accumulated and where mesh values are read from.
#include <map>
#include <mutex>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "tma.cuh"

namespace pmgb {

constexpr int TILE = 8;               // cells per tile edge
constexpr int BOX_THREADS = 256;
constexpr int PAINT_PER_THREAD = 8;   // paint chunk: 2048 particles
constexpr int PAINT_CHUNK = BOX_THREADS * PAINT_PER_THREAD;
constexpr int PAINT_CAP = 16384;      // cells of the paint box (64 KB)

// ---------------------------------------------------------------------------
// tile keys
// ---------------------------------------------------------------------------
__host__ __device__ inline int tile_bits(int nx, int ny, int nz) {
  int t = std::max(std::max((nx + TILE - 1) / TILE, (ny + TILE - 1) / TILE), (nz + TILE - 1) / TILE);
  int b = 0;
  while ((1 << b) < t) ++b;
  return b;
}

__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  v &= 0x3ff;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// Morton key of the tile holding the (wrapped) cell of position (x, y, z).
__device__ __forceinline__ uint32_t tile_key(float x, float y, float z, int nx, int ny, int nz) {
  uint32_t tx = wrap_index((int)floorf(x), nx) / TILE;
  uint32_t ty = wrap_index((int)floorf(y), ny) / TILE;
  uint32_t tz = wrap_index((int)floorf(z), nz) / TILE;
  return (spread3(tx) << 2) | (spread3(ty) << 1) | spread3(tz);
}

__device__ __forceinline__ uint32_t compact3(uint32_t v) {
  v &= 0x09249249u;
  v = (v | (v >> 2)) & 0x030C30C3u;
  v = (v | (v >> 4)) & 0x0300F00Fu;
  v = (v | (v >> 8)) & 0x030000FFu;
  v = (v | (v >> 16)) & 0x000003FFu;
  return v;
}

// Warp-aggregated count of `key` (valid lanes only); returns the lane's rank
// among the particles of that key counted so far.
__device__ __forceinline__ uint32_t count_and_rank(unsigned *__restrict__ counts, uint32_t key,
                                                   unsigned active) {
  const int lane = threadIdx.x & 31;
  // common case: every active lane has the same key (vote + shuffle only)
  const int first = __ffs(active) - 1;
  const uint32_t k0 = __shfl_sync(active, key, first);
  unsigned peers;
  if (__all_sync(active, key == k0))
    peers = active;
  else
    peers = __match_any_sync(active, key);
  int leader = __ffs(peers) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(counts + key, (unsigned)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + __popc(peers & ((1u << lane) - 1u));
}

// The gather's tile histogram: particles that stay in the tile being
// processed (`home`) are added by one warp-level reduction, the others one
// each; no value is returned, so nothing waits on the atomics (the scatter
// claims the slots).  All 32 lanes call it.
__device__ __forceinline__ void count_home(unsigned *__restrict__ counts, uint32_t key,
                                           uint32_t home, bool valid) {
  const unsigned stay = __ballot_sync(0xffffffffu, valid && key == home);
  if (stay && (threadIdx.x & 31) == __ffs(stay) - 1) atomicAdd(counts + home, (unsigned)__popc(stay));
  if (valid && key != home) atomicAdd(counts + key, 1u);
}

// count_home that also ranks the particles that stay in `home` with the
// shared counter *stay (one warp-aggregated shared atomic): returns a
// stayer's rank among the tile's stayers, ~0 for a particle that left.
__device__ __forceinline__ unsigned count_home_rank(unsigned *__restrict__ counts, uint32_t key,
                                                    uint32_t home, bool valid, unsigned *stay) {
  const int lane = threadIdx.x & 31;
  const unsigned sm = __ballot_sync(0xffffffffu, valid && key == home);
  unsigned b = 0;
  if (sm && lane == __ffs(sm) - 1) {
    atomicAdd(counts + home, (unsigned)__popc(sm));
    b = atomicAdd(stay, (unsigned)__popc(sm));
  }
  if (valid && key != home) atomicAdd(counts + key, 1u);
  b = __shfl_sync(0xffffffffu, b, sm ? __ffs(sm) - 1 : 0);
  return (sm >> lane) & 1u ? b + __popc(sm & ((1u << lane) - 1u)) : 0xffffffffu;
}

// Fixed-point scale of a paint box whose tile holds `count` (< 2^20)
// particles: 2^s with s = min(24, clz(count)), so that count * 2^s < 2^32
// (a cell receives at most one contribution, <= 2^s, per particle) and the
// box sums stay exact in one 32-bit word.
__device__ __forceinline__ int paint_shift(unsigned count) {
  const int s = __clz(count);
  return s < 24 ? s : 24;
}

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }

// ---------------------------------------------------------------------------
// chunk boxes in coordinates relative to a reference cell (so a chunk that
// straddles the periodic boundary, or whose particles carry different
// numbers of box lengths, stays compact)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int rel_coord(int f, int r, int n) {
  int d = (f - r) % n;
  if (d < 0) d += n;
  if (d >= (n + 1) / 2) d -= n;  // into [-(n/2), (n+1)/2)
  return d;
}

struct BoxGeom {
  int rx, ry, rz;  // reference cell (unwrapped floor of the chunk's first particle)
  int lx, ly, lz;  // relative coordinate of box cell 0
  int ex, ey, ez;  // extents
  bool fits;
};

template <int NWARPS>
__device__ BoxGeom chunk_box(int lo0, int lo1, int lo2, int hi0, int hi1, int hi2, int rx,
                             int ry, int rz, int cap, int zalign, int nz) {
  __shared__ int red[6][NWARPS];
  __shared__ int fin[6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int v[6] = {lo0, lo1, lo2, hi0, hi1, hi2};
#pragma unroll
  for (int d = 0; d < 6; ++d) {
    int x = v[d];
    for (int o = 16; o > 0; o >>= 1) {
      int y = __shfl_xor_sync(0xffffffffu, x, o);
      x = d < 3 ? min(x, y) : max(x, y);
    }
    if (lane == 0) red[d][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    int d = threadIdx.x, x = red[d][0];
    for (int w = 1; w < NWARPS; ++w) x = d < 3 ? min(x, red[d][w]) : max(x, red[d][w]);
    fin[d] = x;
  }
  __syncthreads();
  BoxGeom g;
  g.rx = rx; g.ry = ry; g.rz = rz;
  g.lx = fin[0]; g.ly = fin[1]; g.lz = fin[2];
  if (zalign > 1) {  // start the box on a z-cell that is a multiple of zalign
    int gz = ((rz + g.lz) % nz + nz) % nz;
    g.lz -= gz % zalign;
  }
  int64_t ex = (int64_t)fin[3] - g.lx + 2, ey = (int64_t)fin[4] - g.ly + 2,
          ez = (int64_t)fin[5] - g.lz + 2;
  if (zalign > 1) ez = (ez + zalign - 1) / zalign * zalign;
  g.fits = ex <= cap && ey <= cap && ez <= cap && ex * ey * ez <= cap;
  g.ex = (int)(ex < cap ? ex : cap);
  g.ey = (int)(ey < cap ? ey : cap);
  g.ez = (int)(ez < cap ? ez : cap);
  __syncthreads();  // red/fin are reused by the next call
  return g;
}

// Relative floor coordinates of a particle w.r.t. the reference cell; a
// non-finite or huge coordinate forces the chunk out of the box path.
__device__ __forceinline__ void rel_bounds(float x, int r, int n, int &lo, int &hi, int &rel) {
  float f = floorf(x);
  if (fabsf(f) < 1e9f) {
    rel = rel_coord((int)f, r, n);
    lo = min(lo, rel);
    hi = max(hi, rel);
  } else {
    rel = 0;
    lo = INT_MIN / 4;
    hi = INT_MAX / 4;
  }
}

__device__ __forceinline__ int ref_floor(float x) {
  float f = floorf(x);
  return fabsf(f) < 1e9f ? (int)f : 0;
}

// ---------------------------------------------------------------------------
// Box painter (PMGB_PAINT_BINNED).  Works for particles in any order; it is
// fast when they are tile sorted, because a chunk's box is then small.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(BOX_THREADS)
paint_box_kernel(float *__restrict__ mesh, int nx, int ny, int nz, const float *__restrict__ pos,
                 int64_t np, const float *__restrict__ weights, float wscale,
                 unsigned *__restrict__ stats, int zal) {
  // zal = 4: flush with 16-byte atomics (nz % 4 == 0, mesh 16-byte aligned)
  extern __shared__ float box[];
  const int tid = threadIdx.x;
  for (int64_t chunk = blockIdx.x; chunk * PAINT_CHUNK < np; chunk += gridDim.x) {
    const int64_t base = chunk * PAINT_CHUNK;
    const int rx = ref_floor(__ldg(pos + 3 * base)), ry = ref_floor(__ldg(pos + 3 * base + 1)),
              rz = ref_floor(__ldg(pos + 3 * base + 2));
    float px[PAINT_PER_THREAD], py[PAINT_PER_THREAD], pz[PAINT_PER_THREAD];
    int qx[PAINT_PER_THREAD], qy[PAINT_PER_THREAD], qz[PAINT_PER_THREAD];
    int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
#pragma unroll
    for (int j = 0; j < PAINT_PER_THREAD; ++j) {
      int64_t p = base + tid + j * BOX_THREADS;
      if (p < np) {
        load3(pos, p, px[j], py[j], pz[j]);
        rel_bounds(px[j], rx, nx, lo[0], hi[0], qx[j]);
        rel_bounds(py[j], ry, ny, lo[1], hi[1], qy[j]);
        rel_bounds(pz[j], rz, nz, lo[2], hi[2], qz[j]);
      }
    }
    BoxGeom g = chunk_box<BOX_THREADS / 32>(lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], rx, ry, rz,
                                            PAINT_CAP, zal, nz);
    if (!g.fits) {
      if (stats && tid == 0) atomicAdd(stats, 1u);
#pragma unroll
      for (int j = 0; j < PAINT_PER_THREAD; ++j) {
        int64_t p = base + tid + j * BOX_THREADS;
        if (p >= np) continue;
        float wp = weights ? __fmul_rn(wscale, __ldg(weights + p)) : wscale;
        Axis ax = cic_axis(px[j], nx), ay = cic_axis(py[j], ny), az = cic_axis(pz[j], nz);
#pragma unroll
        for (int n = 0; n < 8; ++n) {
          float w = __fmul_rn(wp, __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0,
                                                      conn_y(n) ? ay.k1 : ay.k0),
                                            conn_z(n) ? az.k1 : az.k0));
          atomicAdd(mesh + cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                                      conn_z(n) ? az.i1 : az.i0, ny, nz), w);
        }
      }
      continue;
    }
    const int eyz = g.ey * g.ez, vol = g.ex * eyz;
    for (int q = tid; q < vol; q += BOX_THREADS) box[q] = 0.0f;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PAINT_PER_THREAD; ++j) {
      int64_t p = base + tid + j * BOX_THREADS;
      if (p >= np) continue;
      float wp = weights ? __fmul_rn(wscale, __ldg(weights + p)) : wscale;
      Axis ax = cic_axis(px[j], nx), ay = cic_axis(py[j], ny), az = cic_axis(pz[j], nz);
      int q0 = ((qx[j] - g.lx) * g.ey + (qy[j] - g.ly)) * g.ez + (qz[j] - g.lz);
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        float w = __fmul_rn(wp, __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0,
                                                    conn_y(n) ? ay.k1 : ay.k0),
                                          conn_z(n) ? az.k1 : az.k0));
        atomicAdd(box + q0 + conn_x(n) * eyz + conn_y(n) * g.ez + conn_z(n), w);
      }
    }
    __syncthreads();
    if (zal == 4) {
      // flush groups of four z-consecutive cells with one 16-byte atomic
      const int ez4 = g.ez >> 2, groups = g.ex * g.ey * ez4;
      for (int q = tid; q < groups; q += BOX_THREADS) {
        int c4 = q % ez4, r = q / ez4, b = r % g.ey, a = r / g.ey;
        const float4 v = *reinterpret_cast<const float4 *>(box + (a * g.ey + b) * g.ez + 4 * c4);
        if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) {
          int gx = wrap_index(rx + g.lx + a, nx), gy = wrap_index(ry + g.ly + b, ny);
          int gz = wrap_index(rz + g.lz + 4 * c4, nz);
          atomicAdd(reinterpret_cast<float4 *>(mesh + cell_index(gx, gy, gz, ny, nz)), v);
        }
      }
    } else {
      for (int q = tid; q < vol; q += BOX_THREADS) {
        float v = box[q];
        if (v != 0.0f) {
          int c = q % g.ez, r = q / g.ez, b = r % g.ey, a = r / g.ey;
          atomicAdd(mesh + cell_index(wrap_index(rx + g.lx + a, nx), wrap_index(ry + g.ly + b, ny),
                                      wrap_index(rz + g.lz + c, nz), ny, nz), v);
        }
      }
    }
    __syncthreads();  // the box is reused by the next chunk
  }
}

// ---------------------------------------------------------------------------
// Tile kernels of the sorted loop.  Right after a sort, particles
// offsets[k] .. offsets[k+1]-1 all have their (wrapped) cell inside tile k,
// so one CTA per tile works on the fixed box tile + 1-cell halo,
// 9 x 9 x 9 cells, stored with a z stride of 12 so that a box row is a
// whole number of 16-byte units (the TMA box is 12 x 9 x 9).  A particle
// found outside its tile (only possible if the ranges are stale) takes the
// global-memory path and is counted in stats[0] (paint) / stats[1] (gather).
// An mbarrier wait that reaches its spin limit sets stats[2] and ends the
// CTA's work.
//
// Interior tiles (box inside the mesh: ox+9 <= nx, oy+9 <= ny, oz+12 <= nz)
// move their boxes with the Tensor Memory Accelerator: the paint flushes its
// box with one cp.reduce.async.bulk.tensor add, and the gather prefetches
// the next tile's force box with cp.async.bulk.tensor into the other of two
// shared-memory buffers while it works on the current one.  Tiles on the
// periodic boundary use plain loads and 16-byte atomics with wrapped
// indices.
// ---------------------------------------------------------------------------
constexpr int TB = TILE + 1;   // box edge (cells)
constexpr int TBZ = 12;        // z stride of a box row (16-byte multiple)
constexpr int TBOX = TB * TB * TBZ;
constexpr int TILE_THREADS = 256;

__device__ __forceinline__ bool box_interior(int ox, int oy, int oz, int nx, int ny, int nz) {
  return ox + TB <= nx && oy + TB <= ny && oz + TBZ <= nz;
}

// The paint boxes accumulate CIC weights (in [0, 1]) in fixed point with
// native (fire-and-forget) 32-bit shared atomics: round(w * 2^s) with s =
// paint_shift(count of the tile's particles), which keeps every cell's sum
// exact and below 2^32 (2^22 for a tile of 512 particles, 2^20 below 4096).
// Each box is converted to float once per cell.  Tiles of 2^20 particles or
// more paint with global float atomics instead.
constexpr unsigned FIX_SAFE_COUNT = 1u << 20;

// Warp-per-tile painter: each warp of a CTA owns a private box (reused as
// the float box for the flush) and takes tiles from a global counter, so
// warps never wait on each other and a heavy tile delays only its own warp.
constexpr int PAINT_WARPS = 8;
constexpr int PAINT_ILP = 4;
constexpr int WBOX_WORDS = (TBOX + 31) / 32 * 32;  // one word per cell, 128-byte multiple
constexpr int PAINT_SMEM = PAINT_WARPS * WBOX_WORDS * 4;

__global__ void __launch_bounds__(PAINT_WARPS * 32)
paint_tiles_kernel(float *__restrict__ mesh, int nx, int ny, int nz,
                   const float *__restrict__ pos, const unsigned *__restrict__ offsets,
                   uint32_t nkeys, unsigned *__restrict__ next_tile,
                   unsigned *__restrict__ stats, int vec,
                   const __grid_constant__ CUtensorMap tmap, int use_tma) {
  extern __shared__ __align__(128) unsigned wbox[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned *lo = wbox + warp * WBOX_WORDS;
  float *fbox = reinterpret_cast<float *>(lo);
  for (;;) {
    uint32_t key = 0;
    if (lane == 0) key = atomicAdd(next_tile, 1u);
    key = __shfl_sync(0xffffffffu, key, 0);
    if (key >= nkeys) break;
    const unsigned beg = __ldg(offsets + key), end = __ldg(offsets + key + 1);
    if (beg == end) continue;  // uniform across the warp
    const int ox = (int)compact3(key >> 2) * TILE, oy = (int)compact3(key >> 1) * TILE,
              oz = (int)compact3(key) * TILE;
    const bool boxed = end - beg < FIX_SAFE_COUNT;  // uniform
    const int shift = paint_shift(end - beg);
    const float S = pow2f(shift);
    {
      uint4 *z4 = reinterpret_cast<uint4 *>(lo);  // 16-byte aligned
      for (int q = lane; q < TBOX / 4; q += 32) z4[q] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncwarp();
    for (unsigned p0 = beg + lane; p0 < end; p0 += 32 * PAINT_ILP) {
     float px[PAINT_ILP], py[PAINT_ILP], pz[PAINT_ILP];
#pragma unroll
     for (int j = 0; j < PAINT_ILP; ++j) {  // loads of several particles in flight
       const unsigned p = p0 + 32 * j;
       if (p < end) {
         px[j] = __ldg(pos + 3 * (int64_t)p);
         py[j] = __ldg(pos + 3 * (int64_t)p + 1);
         pz[j] = __ldg(pos + 3 * (int64_t)p + 2);
       }
     }
#pragma unroll
     for (int j = 0; j < PAINT_ILP; ++j) {
      if (p0 + 32 * j >= end) break;
      const float x = px[j], y = py[j], z = pz[j];
      Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
      const int lx = ax.i0 - ox, ly = ay.i0 - oy, lz = az.i0 - oz;
      if (boxed && (unsigned)lx < (unsigned)TILE && (unsigned)ly < (unsigned)TILE &&
          (unsigned)lz < (unsigned)TILE) {
        const int q0 = (lx * TB + ly) * TBZ + lz;
#pragma unroll
        for (int n = 0; n < 8; ++n) {
          float w = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                              conn_z(n) ? az.k1 : az.k0);
          atomicAdd(lo + q0 + conn_x(n) * TB * TBZ + conn_y(n) * TBZ + conn_z(n),
                    __float2uint_rn(w * S));
        }
      } else {
        if (stats && boxed) atomicAdd(stats, 1u);
#pragma unroll
        for (int n = 0; n < 8; ++n) {
          float w = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                              conn_z(n) ? az.k1 : az.k0);
          atomicAdd(mesh + cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                                      conn_z(n) ? az.i1 : az.i0, ny, nz), w);
        }
      }
     }
    }
    __syncwarp();
    // fixed point -> float in place (each lane reads and rewrites its own cells)
    {
      const float inv = pow2f(-shift);
      for (int q = lane; q < TBOX; q += 32) fbox[q] = (float)lo[q] * inv;
    }
    const bool tma = use_tma && box_interior(ox, oy, oz, nx, ny, nz);
    if (tma) fence_async_shared();  // generic-proxy writes of fbox -> TMA
    __syncwarp();
    if (tma) {
      if (lane == 0) {
        tma_reduce_add_3d(&tmap, oz, oy, ox, fbox);
        bulk_commit();
        bulk_wait_read();  // the box may be rewritten after this
      }
    } else if (vec) {
      // 9 x 9 rows of three 16-byte groups starting at z = oz, oz+4, oz+8
      for (int q = lane; q < TB * TB * 3; q += 32) {
        const int g = q % 3, r = q / 3, b = r % TB, a = r / TB;
        const float4 v = *reinterpret_cast<const float4 *>(fbox + (a * TB + b) * TBZ + 4 * g);
        if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) {
          const int gx = wrap_index(ox + a, nx), gy = wrap_index(oy + b, ny),
                    gz = wrap_index(oz + 4 * g, nz);
          atomicAdd(reinterpret_cast<float4 *>(mesh + cell_index(gx, gy, gz, ny, nz)), v);
        }
      }
    } else {
      for (int q = lane; q < TB * TB * TB; q += 32) {
        const int c = q % TB, r = q / TB, b = r % TB, a = r / TB;
        const float v = fbox[(a * TB + b) * TBZ + c];
        if (v != 0.f)
          atomicAdd(mesh + cell_index(wrap_index(ox + a, nx), wrap_index(oy + b, ny),
                                      wrap_index(oz + c, nz), ny, nz), v);
      }
    }
    __syncwarp();  // the box is reused by the warp's next tile
  }
  if (use_tma && lane == 0) bulk_wait_all();  // reductions complete before the kernel ends
}

constexpr int FBOX = 3 * TBOX;  // three force components, [c][x][y][z(12)]
constexpr uint32_t FBOX_BYTES = FBOX * sizeof(float);
constexpr int FBOX_STRIDE = (FBOX + 31) / 32 * 32;  // buffers 128-byte aligned

// Potential box of the gather that derives the forces from the potential
// (the run loop): the tile's force box needs the potential two cells beyond
// it on each side along each axis (the order-1 gradient kernel
// (8 sin w - sin 2w)/6 of jaxpm/kernels.py:41-66 is the transfer function
// of the stencil (8 (p[+1] - p[-1]) - (p[+2] - p[-2])) / 12), so 13 x 13
// cells in x and y; in z the box starts 4 cells before the tile (a TMA
// load's innermost coordinate must be 16-byte aligned) and spans 16.
constexpr int PBX = TB + 4, PBY = TB + 4, PBZ = 16;
constexpr int PBOX = PBX * PBY * PBZ;
constexpr uint32_t PBOX_BYTES = PBOX * sizeof(float);
static_assert(PBOX <= FBOX_STRIDE, "potential box must fit a force-box buffer");

__device__ __forceinline__ bool pot_interior(int ox, int oy, int oz, int nx, int ny, int nz) {
  return ox >= 2 && oy >= 2 && oz >= 4 && ox + TB + 2 <= nx && oy + TB + 2 <= ny &&
         oz + PBZ - 4 <= nz;
}

// -(i g(w)) applied to the potential along `axis` at mesh cell (ix, iy, iz),
// from the potential in global memory (wrapped neighbours): the force
// component, (t2 - 8 t1) / 12 with t1 = p[+1] - p[-1], t2 = p[+2] - p[-2]
// (the gather's box path computes the same expression), for particles found
// outside their tile.
__device__ __forceinline__ float stencil_force_global(const float *__restrict__ pot, int ix,
                                                      int iy, int iz, int axis, int nx, int ny,
                                                      int nz) {
  float v[5];
#pragma unroll
  for (int d = -2; d <= 2; ++d) {
    if (d == 0) continue;
    const int x = axis == 0 ? wrap_index(ix + d, nx) : ix;
    const int y = axis == 1 ? wrap_index(iy + d, ny) : iy;
    const int z = axis == 2 ? wrap_index(iz + d, nz) : iz;
    v[d + 2] = __ldg(pot + cell_index(x, y, z, ny, nz));
  }
  const float t1 = v[3] - v[1], t2 = v[4] - v[0];
  return (t2 - 8.0f * t1) * (1.0f / 12.0f);
}

// The CIC-interpolated force of a particle (axes ax, ay, az) from the
// potential in global memory; out of line, it is the rare path and would
// otherwise crowd the gather's registers.
__device__ __noinline__ void pot_gather_global(const float *__restrict__ pot, Axis ax, Axis ay,
                                               Axis az, int nx, int ny, int nz, float *a) {
  float a0 = 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll 1
  for (int n = 0; n < 8; ++n) {
    const float w = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                              conn_z(n) ? az.k1 : az.k0);
    const int ix = conn_x(n) ? ax.i1 : ax.i0, iy = conn_y(n) ? ay.i1 : ay.i0,
              iz = conn_z(n) ? az.i1 : az.i0;
    a0 += stencil_force_global(pot, ix, iy, iz, 0, nx, ny, nz) * w;
    a1 += stencil_force_global(pot, ix, iy, iz, 1, nx, ny, nz) * w;
    a2 += stencil_force_global(pot, ix, iy, iz, 2, nx, ny, nz) * w;
  }
  a[0] = a0;
  a[1] = a1;
  a[2] = a2;
}

// The tile's force box (three components [c][x][y][z(12)], TBOX apart) from
// its potential box `pbox` (PBX x PBY x PBZ, force-box cell (a, b, c) is
// potential entry (a + 2, b + 2, c + 4)): -(i g(w)) of the order-1 gradient
// kernel (8 sin w - sin 2w)/6 of jaxpm/kernels.py:41-66 as the stencil
// (t2 - 8 t1) / 12, t1 = p[+1] - p[-1], t2 = p[+2] - p[-2], four z cells per
// item with 16-byte shared loads: rows of 16 potentials, c0 = 0, 4, 8 (cells
// 9..11 are the rows' padding; their neighbours may read the next row,
// which stays inside the buffer).  The caller synchronises afterwards.
__device__ __forceinline__ void force_box_from_potential(const float *__restrict__ box,
                                                         float *__restrict__ ff, int tid) {
  for (int q = tid; q < TB * TB * 3; q += TILE_THREADS) {
    const int c0 = 4 * (q % 3), r = q / 3, b = r % TB, a = r / TB;
    const float *row = box + ((a + 2) * PBY + b + 2) * PBZ + c0;
    const float4 z0 = *reinterpret_cast<const float4 *>(row);
    const float4 zc = *reinterpret_cast<const float4 *>(row + 4);
    const float4 z2 = *reinterpret_cast<const float4 *>(row + 8);
    const float zz[12] = {z0.x, z0.y, z0.z, z0.w, zc.x, zc.y, zc.z, zc.w,
                          z2.x, z2.y, z2.z, z2.w};
    auto nb = [&](int off) { return *reinterpret_cast<const float4 *>(row + 4 + off); };
    const float4 xm2 = nb(-2 * PBY * PBZ), xm1 = nb(-PBY * PBZ), xp1 = nb(PBY * PBZ),
                 xp2 = nb(2 * PBY * PBZ);
    const float4 ym2 = nb(-2 * PBZ), ym1 = nb(-PBZ), yp1 = nb(PBZ), yp2 = nb(2 * PBZ);
    auto f = [](float m2, float m1, float p1, float p2) {
      const float t1 = p1 - m1, t2 = p2 - m2;
      return (t2 - 8.0f * t1) * (1.0f / 12.0f);
    };
    float4 fx, fy, fz;
    fx.x = f(xm2.x, xm1.x, xp1.x, xp2.x);
    fx.y = f(xm2.y, xm1.y, xp1.y, xp2.y);
    fx.z = f(xm2.z, xm1.z, xp1.z, xp2.z);
    fx.w = f(xm2.w, xm1.w, xp1.w, xp2.w);
    fy.x = f(ym2.x, ym1.x, yp1.x, yp2.x);
    fy.y = f(ym2.y, ym1.y, yp1.y, yp2.y);
    fy.z = f(ym2.z, ym1.z, yp1.z, yp2.z);
    fy.w = f(ym2.w, ym1.w, yp1.w, yp2.w);
    fz.x = f(zz[2], zz[3], zz[5], zz[6]);
    fz.y = f(zz[3], zz[4], zz[6], zz[7]);
    fz.z = f(zz[4], zz[5], zz[7], zz[8]);
    fz.w = f(zz[5], zz[6], zz[8], zz[9]);
    const int o = (a * TB + b) * TBZ + c0;
    *reinterpret_cast<float4 *>(ff + o) = fx;
    *reinterpret_cast<float4 *>(ff + TBOX + o) = fy;
    *reinterpret_cast<float4 *>(ff + 2 * TBOX + o) = fz;
  }
}

struct TileInfo {
  unsigned beg, end;
  int ox, oy, oz;
  bool tma;
};

__device__ __forceinline__ TileInfo tile_info(const unsigned *__restrict__ offsets, uint32_t key,
                                              int nx, int ny, int nz, int use_tma,
                                              bool pot = false) {
  TileInfo t;
  t.beg = __ldg(offsets + key);
  t.end = __ldg(offsets + key + 1);
  t.ox = (int)compact3(key >> 2) * TILE;
  t.oy = (int)compact3(key >> 1) * TILE;
  t.oz = (int)compact3(key) * TILE;
  t.tma = use_tma && t.beg != t.end &&
          (pot ? pot_interior(t.ox, t.oy, t.oz, nx, ny, nz)
               : box_interior(t.ox, t.oy, t.oz, nx, ny, nz));
  return t;
}

// Tile schedule of the gather kernels.  CTA b first takes the static tiles
// b, b + G, b + 2G, ... below S = max(2G, `quarters` quarters of the keys
// rounded down to a multiple of G), G = gridDim.x; the rest of the keys go to
// whichever CTA asks first: the c-th grab from the counter *work (zero at
// launch) is tile S + c.  In the gather that paints (three quarters static)
// the static part keeps the tiles processed at the same time spread over the
// mesh once the CTAs drift apart: a schedule that is dynamic throughout keeps
// every CTA on neighbouring keys, and with large steps the global atomics of
// the particles leaving their tiles then pile up on the same cells (gather of
// a 6-step 512^3 run 5.1 ms dynamic, 4.5 ms static or hybrid).  The dynamic
// tail absorbs the uneven particle counts of the tiles (40-step run: 4.2 ms
// static, 3.8 ms dynamic or hybrid).  Every key is processed exactly once.
struct TileSchedule {
  uint32_t nstatic;  // static tiles per CTA (S / G)
  uint32_t S;
  __device__ __forceinline__ TileSchedule(uint32_t nkeys, uint32_t quarters) {
    const uint32_t G = gridDim.x;
    nstatic = max(2u, (uint32_t)(((uint64_t)nkeys * quarters / 4u) / G));
    S = nstatic * G;
  }
  // the key of this CTA's i-th tile (i >= nstatic: takes a counter value)
  __device__ __forceinline__ uint32_t key(uint32_t i, unsigned *work) const {
    return i < nstatic ? blockIdx.x + i * gridDim.x : S + atomicAdd(work, 1u);
  }
};

constexpr int RKD_ILP = 2;

// Paint box of the fused gather (the next step's density from the new
// positions): the tile's own 9 x 9 x 12-cell box, so particles that stay in
// the tile paint into shared memory and the few that left it paint with
// global atomics.  Two boxes in turn (the TMA reduce of one drains while
// the next tile paints the other), one fixed-point word per cell
// (paint_shift), x-planes padded to 128 bytes for the per-plane reduces.
constexpr int NB = TB;
constexpr int NBZ = TBZ;
constexpr int NPS = (NB * NBZ + 31) / 32 * 32;  // x-plane stride (128-byte multiple)
constexpr int NBOX_WORDS = NB * NPS;
constexpr int RKDP_SMEM = 2 * NBOX_WORDS * 4;

__device__ __forceinline__ void zero_words(unsigned *p, int words, int tid) {
  uint4 *z4 = reinterpret_cast<uint4 *>(p);
  for (int q = tid; q < words / 4; q += TILE_THREADS) z4[q] = make_uint4(0u, 0u, 0u, 0u);
}

// POT: f3 is the potential mesh (cs unused) and tmap its 3-D map; each
// tile's force box is computed from the staged potential box.
template <bool PAINT, bool POT = false>
__global__ void __launch_bounds__(TILE_THREADS, 4)
rkd_tiles_kernel(const float *__restrict__ f3, int64_t cs, int nx, int ny, int nz,
                 const float *pos, float *pos_out, float *vel,
                 const unsigned *__restrict__ offsets, uint32_t nkeys, float kick, float drift,
                 unsigned *__restrict__ counts, unsigned *__restrict__ rank,
                 unsigned *__restrict__ stats, const __grid_constant__ CUtensorMap tmap,
                 int use_tma, float *__restrict__ mesh_next, int pvec,
                 const __grid_constant__ CUtensorMap pmap, int use_ptma,
                 unsigned *__restrict__ work, const PermIO io, int quarters) {
  __shared__ __align__(128) float fb[2][FBOX_STRIDE];
  __shared__ __align__(16) float ff[POT ? FBOX : 4];  // POT: the tile's force box
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t s_grab[2];  // the tile after next, as grabbed by thread 0
  __shared__ unsigned s_stay;     // permuted mode: particles of the tile that stayed
  extern __shared__ __align__(128) unsigned pbox[];  // PAINT: 2 x NBOX_WORDS
  constexpr uint32_t BOX_BYTES = POT ? PBOX_BYTES : FBOX_BYTES;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_async_shared();
  }
  if (PAINT) zero_words(pbox, NBOX_WORDS, tid);
  __syncthreads();
  int pbuf = 0;
  uint32_t phase0 = 0u, phase1 = 0u;  // parity of the next completion of bar[0] / bar[1]
  // TileSchedule; thread 0 fixes each tile two tiles ahead, so a grab's
  // latency hides behind a tile's work.
  uint32_t key = blockIdx.x;
  if (key >= nkeys) return;
  const TileSchedule sched(nkeys, (uint32_t)quarters);
  uint32_t knext = gridDim.x + blockIdx.x;  // tiles 0 and 1 are static
  uint32_t it = 0;                          // index of the current tile
  TileInfo cur = tile_info(offsets, key, nx, ny, nz, use_tma, POT);
  if (cur.tma && tid == 0) {
    mbar_expect_tx(&bar[0], BOX_BYTES);
    if (POT) tma_load_3d(fb[0], &tmap, cur.oz - 4, cur.oy - 2, cur.ox - 2, &bar[0]);
    else tma_load_4d(fb[0], &tmap, cur.oz, cur.oy, cur.ox, 0, &bar[0]);
  }
  // permuted mode: the indices of a tile's first chunk are loaded one tile
  // ahead, so that its particle loads do not wait on them
  unsigned qpre[RKD_ILP];
  auto prefetch_perm = [&](const TileInfo &t) {
#pragma unroll
    for (int j = 0; j < RKD_ILP; ++j) {
      const unsigned p = t.beg + tid + j * TILE_THREADS;
      qpre[j] = (io.perm && p < t.end) ? __ldg(io.perm + p) : p;
    }
  };
  prefetch_perm(cur);
  int buf = 0;
  while (key < nkeys) {
    uint32_t kgrab = 0xffffffffu;  // thread 0: the tile after next
    if (tid == 0 && knext < nkeys) kgrab = sched.key(it + 2, work);
    if (tid == 0) s_stay = 0u;  // read by this thread last, after the tile's barrier
    // prefetch the next tile's box into the other buffer (freed by the
    // barrier at the end of the previous iteration)
    TileInfo nxt;
    nxt.tma = false;
    if (knext < nkeys) {
      nxt = tile_info(offsets, knext, nx, ny, nz, use_tma, POT);
      if (nxt.tma && tid == 0) {
        fence_async_shared();
        mbar_expect_tx(&bar[buf ^ 1], BOX_BYTES);
        if (POT)
          tma_load_3d(fb[buf ^ 1], &tmap, nxt.oz - 4, nxt.oy - 2, nxt.ox - 2, &bar[buf ^ 1]);
        else
          tma_load_4d(fb[buf ^ 1], &tmap, nxt.oz, nxt.oy, nxt.ox, 0, &bar[buf ^ 1]);
      }
    }
    float px[RKD_ILP], py[RKD_ILP], pz[RKD_ILP], pu[RKD_ILP], pv[RKD_ILP], pw[RKD_ILP];
    auto load_chunk = [&](unsigned p0) {
#pragma unroll
      for (int j = 0; j < RKD_ILP; ++j) {
        const unsigned p = p0 + tid + j * TILE_THREADS;
        if (p < cur.end) {
          // slot p's particle: at index perm[p] in the permuted mode
          const int64_t q = p0 == cur.beg ? (int64_t)qpre[j]
                            : io.perm    ? (int64_t)__ldg(io.perm + p)
                                         : (int64_t)p;
          px[j] = pos[3 * q];
          py[j] = pos[3 * q + 1];
          pz[j] = pos[3 * q + 2];
          pu[j] = vel[3 * q];
          pv[j] = vel[3 * q + 1];
          pw[j] = vel[3 * q + 2];
        }
      }
    };
    if (cur.beg != cur.end) {
      load_chunk(cur.beg);  // in flight during the box wait (and the force box)
      if (knext < nkeys) prefetch_perm(nxt);
      float *box = fb[buf];
      if (cur.tma) {
        const bool ok = mbar_wait(&bar[buf], buf ? phase1 : phase0);
        if (__syncthreads_or(!ok)) {  // uniform: every thread leaves together
          if (stats && tid == 0) atomicExch(stats + 2, 1u);
          if (nxt.tma) mbar_wait(&bar[buf ^ 1], buf ? phase0 : phase1);  // drain the prefetch
          if (PAINT && use_ptma && (tid & 31) == 0) bulk_wait_all();  // paint reductions
          return;
        }
        if (buf) phase1 ^= 1u; else phase0 ^= 1u;
      } else if (POT) {
        for (int q = tid; q < PBOX; q += TILE_THREADS) {
          const int zc = q % PBZ, r = q / PBZ, yc = r % PBY, xc = r / PBY;
          box[q] = __ldg(f3 + cell_index(wrap_index(cur.ox - 2 + xc, nx),
                                         wrap_index(cur.oy - 2 + yc, ny),
                                         wrap_index(cur.oz - 4 + zc, nz), ny, nz));
        }
        __syncthreads();
      } else {
        for (int q = tid; q < 3 * TB * TB * TB; q += TILE_THREADS) {
          const int c = q % TB, r = q / TB, b = r % TB, r2 = r / TB, a = r2 % TB, comp = r2 / TB;
          const int64_t cell = cell_index(wrap_index(cur.ox + a, nx), wrap_index(cur.oy + b, ny),
                                          wrap_index(cur.oz + c, nz), ny, nz);
          box[((comp * TB + a) * TB + b) * TBZ + c] = __ldg(f3 + comp * cs + cell);
        }
        __syncthreads();
      }
      if (POT) {
        force_box_from_potential(box, ff, tid);
        __syncthreads();
        box = ff;
      }
      if (tid == 0) s_grab[buf] = kgrab;  // returned by now; frees its register
      // every lane of a warp runs the same iterations (ballot / match inside);
      // each thread loads RKD_ILP particles before computing any of them
      for (unsigned p0 = cur.beg; p0 < cur.end; p0 += TILE_THREADS * RKD_ILP) {
       if (p0 != cur.beg) load_chunk(p0);
#pragma unroll
       for (int j = 0; j < RKD_ILP; ++j) {
        const unsigned p = p0 + tid + j * TILE_THREADS;
        const bool valid = p < cur.end;
        uint32_t k = 0;
        if (valid) {
          const float x = px[j], y = py[j], z = pz[j];
          const float v0 = pu[j], v1 = pv[j], v2 = pw[j];
          Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
          float a0 = 0.f, a1 = 0.f, a2 = 0.f;
          const int lx = ax.i0 - cur.ox, ly = ay.i0 - cur.oy, lz = az.i0 - cur.oz;
          if ((unsigned)lx < (unsigned)TILE && (unsigned)ly < (unsigned)TILE &&
              (unsigned)lz < (unsigned)TILE) {
            const int q0 = (lx * TB + ly) * TBZ + lz;
#pragma unroll
            for (int n = 0; n < 8; ++n) {
              float w = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                                  conn_z(n) ? az.k1 : az.k0);
              const int q = q0 + conn_x(n) * TB * TBZ + conn_y(n) * TBZ + conn_z(n);
              a0 += box[q] * w;
              a1 += box[TBOX + q] * w;
              a2 += box[2 * TBOX + q] * w;
            }
          } else if (POT) {
            if (stats) atomicAdd(stats + 1, 1u);
            float a[3];
            pot_gather_global(f3, ax, ay, az, nx, ny, nz, a);
            a0 = a[0];
            a1 = a[1];
            a2 = a[2];
          } else {
            if (stats) atomicAdd(stats + 1, 1u);
#pragma unroll
            for (int n = 0; n < 8; ++n) {
              float w = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                                  conn_z(n) ? az.k1 : az.k0);
              const int64_t c = cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                                           conn_z(n) ? az.i1 : az.i0, ny, nz);
              a0 += __ldg(f3 + c) * w;
              a1 += __ldg(f3 + cs + c) * w;
              a2 += __ldg(f3 + 2 * cs + c) * w;
            }
          }
          const float vx = v0 + kick * a0, vy = v1 + kick * a1, vz = v2 + kick * a2;
          float *vo = io.vel_out ? io.vel_out : vel;
          vo[3 * (int64_t)p] = vx;
          vo[3 * (int64_t)p + 1] = vy;
          vo[3 * (int64_t)p + 2] = vz;
          const float xn = x + drift * vx, yn = y + drift * vy, zn = z + drift * vz;
          pos_out[3 * (int64_t)p] = xn;
          pos_out[3 * (int64_t)p + 1] = yn;
          pos_out[3 * (int64_t)p + 2] = zn;
          // the new cell (cic_axis wraps floor(x) as the tile key does)
          const Axis bx = cic_axis(xn, nx), by = cic_axis(yn, ny), bz = cic_axis(zn, nz);
          const int cx = bx.i0 - cur.ox, cy = by.i0 - cur.oy, cz = bz.i0 - cur.oz;
          const bool stays = (unsigned)cx < (unsigned)TILE && (unsigned)cy < (unsigned)TILE &&
                             (unsigned)cz < (unsigned)TILE;
          k = stays ? key  // most particles stay
                    : (spread3((uint32_t)bx.i0 / TILE) << 2) |
                          (spread3((uint32_t)by.i0 / TILE) << 1) | spread3((uint32_t)bz.i0 / TILE);
          if (PAINT) {  // the next step's density: the new position into the paint box
            const unsigned cnt = cur.end - cur.beg;
            unsigned *plo = pbox + pbuf * NBOX_WORDS;
            if (stays && cnt < FIX_SAFE_COUNT) {
              const int q0 = cx * NPS + cy * NBZ + cz;
              const float S = pow2f(paint_shift(cnt));
#pragma unroll
              for (int n = 0; n < 8; ++n) {
                const float w =
                    __fmul_rn(__fmul_rn(conn_x(n) ? bx.k1 : bx.k0, conn_y(n) ? by.k1 : by.k0),
                              conn_z(n) ? bz.k1 : bz.k0);
                const int q = q0 + conn_x(n) * NPS + conn_y(n) * NBZ + conn_z(n);
                atomicAdd(plo + q, __float2uint_rn(w * S));
              }
            } else {  // left the tile (the normal case for ~1 in 10): global atomics
#pragma unroll
              for (int n = 0; n < 8; ++n) {
                const float w =
                    __fmul_rn(__fmul_rn(conn_x(n) ? bx.k1 : bx.k0, conn_y(n) ? by.k1 : by.k0),
                              conn_z(n) ? bz.k1 : bz.k0);
                atomicAdd(mesh_next + cell_index(conn_x(n) ? bx.i1 : bx.i0,
                                                 conn_y(n) ? by.i1 : by.i0,
                                                 conn_z(n) ? bz.i1 : bz.i0, ny, nz),
                          w);
              }
            }
          }
        }
        if (io.key_out) {
          // the stayers' ranks in the tile come from one shared counter
          // (warp-aggregated), so the re-sort places them without atomics
          const unsigned r = count_home_rank(counts, k, key, valid, &s_stay);
          if (valid) *reinterpret_cast<uint2 *>(io.key_out + 2 * (int64_t)p) = make_uint2(k, r);
        } else if (counts) {
          count_home(counts, k, key, valid);
        }
       }
      }
    } else {
      if (knext < nkeys) prefetch_perm(nxt);
      if (tid == 0) s_grab[buf] = kgrab;
    }
    __syncthreads();  // buffer `buf` is free for the prefetch two tiles ahead
    const uint32_t kafter = s_grab[buf];  // rewritten two iterations later, after a barrier
    if (io.stay_out && tid == 0) io.stay_out[key] = s_stay;
    if (PAINT && cur.beg != cur.end) {
      // flush the paint box, each warp its x-planes (w and w + 8): fixed
      // point -> float in place, one TMA reduce-add per plane into the mesh
      // (16-byte atomics where the box wraps), then the warp zeroes its
      // planes of the other box for the next tile (once its previous
      // reduce has read them).  No CTA barrier: the next tile's barrier
      // orders the zeroing before its atomics.
      const int lane = tid & 31, warp = tid >> 5;
      const unsigned cnt = cur.end - cur.beg;
      float *pf = reinterpret_cast<float *>(pbox + pbuf * NBOX_WORDS);
      const float inv = pow2f(-paint_shift(cnt));
      const bool ptma = use_ptma && box_interior(cur.ox, cur.oy, cur.oz, nx, ny, nz);
      for (int a = warp; a < NB; a += TILE_THREADS / 32) {
        uint4 *pl = reinterpret_cast<uint4 *>(pf + a * NPS);
        for (int q = lane; q < NB * NBZ / 4; q += 32) {
          const uint4 u = pl[q];
          reinterpret_cast<float4 *>(pl)[q] =
              make_float4((float)u.x * inv, (float)u.y * inv, (float)u.z * inv, (float)u.w * inv);
        }
      }
      if (ptma) fence_async_shared();
      __syncwarp();
      if (ptma) {
        if (lane == 0) {
          for (int a = warp; a < NB; a += TILE_THREADS / 32)
            tma_reduce_add_3d(&pmap, cur.oz, cur.oy, cur.ox + a, pf + a * NPS);
          bulk_commit();
        }
      } else {
        for (int a = warp; a < NB; a += TILE_THREADS / 32) {
          for (int q = lane; q < NB * NBZ / 4; q += 32) {
            const int g = q % (NBZ / 4), b = q / (NBZ / 4);
            const float *src = pf + a * NPS + b * NBZ + 4 * g;
            const int64_t row = cell_index(wrap_index(cur.ox + a, nx),
                                           wrap_index(cur.oy + b, ny), 0, ny, nz);
            if (pvec) {
              const float4 v = *reinterpret_cast<const float4 *>(src);
              if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f)
                atomicAdd(reinterpret_cast<float4 *>(mesh_next + row +
                                                     wrap_index(cur.oz + 4 * g, nz)),
                          v);
            } else {
#pragma unroll
              for (int c = 0; c < 4; ++c)
                if (src[c] != 0.f)
                  atomicAdd(mesh_next + row + wrap_index(cur.oz + 4 * g + c, nz), src[c]);
            }
          }
        }
      }
      // the warp's planes of the other box: free once this lane 0's previous
      // reduce group has read them
      if (use_ptma && lane == 0) {
        if (ptma) bulk_wait_read_prior();  // all but the group just committed
        else bulk_wait_read();             // nothing committed for this tile
      }
      __syncwarp();
      unsigned *other = pbox + (pbuf ^ 1) * NBOX_WORDS;
      for (int a = warp; a < NB; a += TILE_THREADS / 32) {
        uint4 *pl = reinterpret_cast<uint4 *>(other + a * NPS);
        for (int q = lane; q < NB * NBZ / 4; q += 32) pl[q] = make_uint4(0u, 0u, 0u, 0u);
      }
      pbuf ^= 1;
    }
    cur = nxt;
    key = knext;
    knext = kafter;
    ++it;
    buf ^= 1;
  }
  if (PAINT && use_ptma && (tid & 31) == 0) bulk_wait_all();  // reductions done before exit
}

// Histogram + rank of the current positions (the first sort of a run).
__global__ void __launch_bounds__(256)
tile_rank_kernel(const float *__restrict__ pos, int64_t np, int nx, int ny, int nz,
                 unsigned *__restrict__ counts, unsigned *__restrict__ rank) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // every lane of a warp runs the same number of iterations (match/shfl)
  for (int64_t p0 = blockIdx.x * (int64_t)blockDim.x; p0 < np; p0 += stride) {
    int64_t p = p0 + threadIdx.x;
    bool valid = p < np;
    uint32_t key = 0;
    if (valid) key = tile_key(__ldg(pos + 3 * p), __ldg(pos + 3 * p + 1), __ldg(pos + 3 * p + 2),
                              nx, ny, nz);
    unsigned active = __ballot_sync(0xffffffffu, valid);
    if (valid) rank[p] = count_and_rank(counts, key, active);
  }
}

// Each scatter thread carries SCATTER_ILP particles so that their loads are
// in flight together.
constexpr int SCATTER_ILP = 4;

// Slot claims of ILP particles per thread (particle b0 + threadIdx.x +
// j * blockDim.x has tile key k[j]): r[j] becomes its slot in the tile,
// taken from the per-tile `cursor`.  Warp-aggregated: lanes whose key equals
// the first valid lane's (most of a warp, since neighbouring particles
// share their tile) take consecutive slots from one atomic, the others
// claim one each; all ILP atomics are in flight before any result is used.
// Every lane of the warp must call it (votes and shuffles).
template <int ILP>
__device__ __forceinline__ void claim_slots(const uint32_t (&k)[ILP], int64_t b0, int64_t np,
                                            unsigned *__restrict__ cursor, unsigned (&r)[ILP]) {
  const int lane = threadIdx.x & 31;
  unsigned same[ILP], base[ILP];
  uint32_t lead[ILP];
#pragma unroll
  for (int j = 0; j < ILP; ++j) {
    const bool valid = b0 + threadIdx.x + j * (int64_t)blockDim.x < np;
    const unsigned act = __ballot_sync(0xffffffffu, valid);
    lead[j] = __shfl_sync(0xffffffffu, k[j], act ? __ffs(act) - 1 : 0);
    same[j] = __ballot_sync(0xffffffffu, valid && k[j] == lead[j]);
    base[j] = 0;
    if (same[j] && lane == __ffs(same[j]) - 1)
      base[j] = atomicAdd(cursor + lead[j], (unsigned)__popc(same[j]));
    r[j] = (valid && k[j] != lead[j]) ? atomicAdd(cursor + k[j], 1u) : 0u;
  }
#pragma unroll
  for (int j = 0; j < ILP; ++j) {
    const unsigned b = __shfl_sync(0xffffffffu, base[j], same[j] ? __ffs(same[j]) - 1 : 0);
    if ((same[j] >> lane) & 1u) r[j] = b + __popc(same[j] & ((1u << lane) - 1u));
  }
}

// The permuted run loop's re-sort: the particle in slot p (the order its
// step started from) has the new tile key and, if it stayed in its tile,
// its rank among the tile's stayers (key_rank[p], from the gather).  A stayer's
// new slot is offsets[key] + rank, with no atomics; a leaver (rank ~0)
// claims the next slot after the stayers from cursor[key] (the stayer
// count), warp-aggregated by key.  perm_new[d] = p tells the next gather
// where slot d's particle is.  With perm_old the ids follow the gather,
// which read slot p's particle from index perm_old[p]:
// id_out[p] = id_in[perm_old[p]].
constexpr int ISCATTER_ILP = 2;
__global__ void __launch_bounds__(256)
index_scatter_kernel(const uint2 *__restrict__ key_rank, int64_t np, const unsigned *__restrict__ offsets,
                     unsigned *__restrict__ cursor, unsigned *__restrict__ perm_new,
                     const unsigned *__restrict__ perm_old, const unsigned *__restrict__ id_in,
                     unsigned *__restrict__ id_out) {
  const int lane = threadIdx.x & 31;
  const int64_t span = (int64_t)blockDim.x * ISCATTER_ILP;
  for (int64_t b0 = blockIdx.x * span; b0 < np; b0 += gridDim.x * span) {
    uint32_t k[ISCATTER_ILP];
    unsigned r[ISCATTER_ILP];
#pragma unroll
    for (int j = 0; j < ISCATTER_ILP; ++j) {
      const int64_t p = b0 + threadIdx.x + j * (int64_t)blockDim.x;
      const uint2 kr = p < np ? __ldg(key_rank + p) : make_uint2(0u, 0u);
      k[j] = kr.x;
      r[j] = kr.y;
      if (perm_old && p < np) id_out[p] = __ldg(id_in + __ldg(perm_old + p));
    }
#pragma unroll
    for (int j = 0; j < ISCATTER_ILP; ++j) {
      const bool leave = r[j] == 0xffffffffu;  // invalid lanes hold r = 0
      const unsigned lm = __ballot_sync(0xffffffffu, leave);
      if (leave) {
        const unsigned peers = __match_any_sync(lm, k[j]);
        const int leader = __ffs(peers) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(cursor + k[j], (unsigned)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        r[j] = base + __popc(peers & ((1u << lane) - 1u));
      }
    }
#pragma unroll
    for (int j = 0; j < ISCATTER_ILP; ++j) {
      const int64_t p = b0 + threadIdx.x + j * (int64_t)blockDim.x;
      if (p < np) perm_new[__ldg(offsets + k[j]) + r[j]] = (unsigned)p;
    }
  }
}

__global__ void gather_u32_kernel(const unsigned *__restrict__ in,
                                  const unsigned *__restrict__ idx, int64_t np,
                                  unsigned *__restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x)
    out[p] = __ldg(in + __ldg(idx + p));
}

// Moves particle p to offsets[key] + its rank in the tile: rank[p] when the
// ranks were recorded (the first sort), else a slot claimed from `cursor`
// (the zeroed tile counters) here (claim_slots), so the gather only counts.
// The loop is warp-uniform (the claims vote across the warp).
__global__ void __launch_bounds__(256, 3)
scatter_kernel(const float *__restrict__ pos, const float *__restrict__ vel,
               const unsigned *__restrict__ id, const unsigned *__restrict__ rank, int64_t np,
               int nx, int ny, int nz, const unsigned *__restrict__ offsets,
               unsigned *__restrict__ cursor, float *__restrict__ pos2,
               float *__restrict__ vel2, unsigned *__restrict__ id2, unsigned *__restrict__ dest) {
  const int64_t span = (int64_t)blockDim.x * SCATTER_ILP;
  for (int64_t b0 = blockIdx.x * span; b0 < np; b0 += gridDim.x * span) {
    float x[SCATTER_ILP], y[SCATTER_ILP], z[SCATTER_ILP], u[SCATTER_ILP], v[SCATTER_ILP],
        w[SCATTER_ILP];
    unsigned r[SCATTER_ILP], ident[SCATTER_ILP];
#pragma unroll
    for (int j = 0; j < SCATTER_ILP; ++j) {
      const int64_t p = b0 + threadIdx.x + j * (int64_t)blockDim.x;
      if (p < np) {
        x[j] = __ldg(pos + 3 * p);
        y[j] = __ldg(pos + 3 * p + 1);
        z[j] = __ldg(pos + 3 * p + 2);
        if (rank) r[j] = __ldg(rank + p);
        if (vel) {
          u[j] = __ldg(vel + 3 * p);
          v[j] = __ldg(vel + 3 * p + 1);
          w[j] = __ldg(vel + 3 * p + 2);
        }
        ident[j] = id ? __ldg(id + p) : (unsigned)p;
      }
    }
    uint32_t k[SCATTER_ILP];
#pragma unroll
    for (int j = 0; j < SCATTER_ILP; ++j) {
      const int64_t p = b0 + threadIdx.x + j * (int64_t)blockDim.x;
      k[j] = p < np ? tile_key(x[j], y[j], z[j], nx, ny, nz) : 0u;
    }
    if (!rank) claim_slots<SCATTER_ILP>(k, b0, np, cursor, r);
#pragma unroll
    for (int j = 0; j < SCATTER_ILP; ++j) {
      const int64_t p = b0 + threadIdx.x + j * (int64_t)blockDim.x;
      if (p < np) r[j] += __ldg(offsets + k[j]);
    }
#pragma unroll
    for (int j = 0; j < SCATTER_ILP; ++j) {
      const int64_t p = b0 + threadIdx.x + j * (int64_t)blockDim.x;
      if (p < np) {
        const int64_t d = r[j];
        pos2[3 * d] = x[j];
        pos2[3 * d + 1] = y[j];
        pos2[3 * d + 2] = z[j];
        if (vel) {
          vel2[3 * d] = u[j];
          vel2[3 * d + 1] = v[j];
          vel2[3 * d + 2] = w[j];
        }
        id2[d] = ident[j];
        if (dest) dest[p] = (unsigned)d;  // where particle p went (for adjoints)
      }
    }
  }
}

// out[id[p]] = in[p] for [np][3] arrays (back to the caller's order).
__global__ void unpermute3_kernel(const float *__restrict__ in, const unsigned *__restrict__ id,
                                  int64_t np, float *__restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    int64_t d = __ldg(id + p);
    if (d >= np) continue;  // not a permutation entry: skipped
    out[3 * d] = __ldg(in + 3 * p);
    out[3 * d + 1] = __ldg(in + 3 * p + 1);
    out[3 * d + 2] = __ldg(in + 3 * p + 2);
  }
}

// out[p] = in[id[p]] for [np][3] arrays (caller's order -> tile order).
// out[p] = in[id[p]] for p < np, id indexing an [n_in][3] array
__global__ void permute3_kernel(const float *__restrict__ in, const unsigned *__restrict__ id,
                                int64_t np, float *__restrict__ out, int64_t n_in) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = __ldg(id + p);
    if (s >= n_in) continue;  // not an entry of the source: skipped
    out[3 * p] = __ldg(in + 3 * s);
    out[3 * p + 1] = __ldg(in + 3 * s + 1);
    out[3 * p + 2] = __ldg(in + 3 * s + 2);
  }
}

// ---------------------------------------------------------------------------
// Exclusive scan of the tile counts (two levels: 4096 per block, then the
// block totals in one block).
// ---------------------------------------------------------------------------
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_PER_THREAD = 4;
constexpr int SCAN_BLOCK = SCAN_THREADS * SCAN_PER_THREAD;

__device__ unsigned block_exclusive_scan(unsigned v, unsigned *total) {
  __shared__ unsigned warp_sums[SCAN_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned x = v;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned s = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < SCAN_THREADS / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  unsigned before = (warp > 0 ? warp_sums[warp - 1] : 0u) + x - v;
  *total = warp_sums[SCAN_THREADS / 32 - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_blocks_kernel(const unsigned *__restrict__ in, unsigned *__restrict__ out, int64_t n,
                   unsigned *__restrict__ sums) {
  const int64_t b0 = (int64_t)blockIdx.x * SCAN_BLOCK + threadIdx.x * SCAN_PER_THREAD;
  unsigned v[SCAN_PER_THREAD], s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; ++i) {
    v[i] = b0 + i < n ? in[b0 + i] : 0u;
    s += v[i];
  }
  unsigned total;
  unsigned run = block_exclusive_scan(s, &total);
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; ++i) {
    if (b0 + i < n) out[b0 + i] = run;
    run += v[i];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
  if (gridDim.x == 1 && threadIdx.x == 0) out[n] = total;  // one block: the grand total
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_sums_kernel(unsigned *__restrict__ sums, int nb) {
  unsigned v[SCAN_PER_THREAD], s = 0;
  const int b0 = threadIdx.x * SCAN_PER_THREAD;
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; ++i) {
    v[i] = b0 + i < nb ? sums[b0 + i] : 0u;
    s += v[i];
  }
  unsigned total;
  unsigned run = block_exclusive_scan(s, &total);
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; ++i) {
    if (b0 + i < nb) sums[b0 + i] = run;
    run += v[i];
  }
}

__global__ void scan_add_kernel(unsigned *__restrict__ out, int64_t n,
                                const unsigned *__restrict__ sums, unsigned grand_total) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] += sums[i / SCAN_BLOCK];
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = grand_total;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int64_t tile_key_count(int nx, int ny, int nz) { return (int64_t)1 << (3 * tile_bits(nx, ny, nz)); }

namespace {
std::mutex g_tune_mu;
Tuning g_tune;
}  // namespace

Tuning tuning() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  return g_tune;
}

void set_tuning(const Tuning &t) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune = t;
}

static int set_smem(const void *fn, int bytes) {
  PMGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  return PMGB_OK;
}

int paint_box(float *mesh, int nx, int ny, int nz, const float *pos, int64_t np,
              const float *weights, float wscale, unsigned *stats, cudaStream_t s) {
  static bool ready[64] = {false};
  int dev = 0;
  PMGB_CUDA(cudaGetDevice(&dev));
  if (dev >= 64 || !ready[dev]) {
    PMGB_TRY(set_smem((const void *)paint_box_kernel, PAINT_CAP * (int)sizeof(float)));
    if (dev < 64) ready[dev] = true;
  }
  if (np == 0) return PMGB_OK;
  const int zal = (nz % 4 == 0 && reinterpret_cast<uintptr_t>(mesh) % 16 == 0) ? 4 : 1;
  int64_t chunks = (np + PAINT_CHUNK - 1) / PAINT_CHUNK;
  unsigned grid = (unsigned)std::min<int64_t>(chunks, (int64_t)sm_count() * 3);
  paint_box_kernel<<<grid, BOX_THREADS, PAINT_CAP * sizeof(float), s>>>(
      mesh, nx, ny, nz, pos, np, weights, wscale, stats, zal);
  PMGB_LAUNCHED("paint_box_kernel");
  return PMGB_OK;
}

int exclusive_scan(const unsigned *in, unsigned *out, int64_t n, unsigned *sums,
                   unsigned grand_total, cudaStream_t s) {
  int64_t nb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
  if (nb > SCAN_BLOCK) return fail(PMGB_ERR_UNSUPPORTED, "too many tiles for the scan");
  scan_blocks_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n, sums);
  PMGB_LAUNCHED("scan_blocks_kernel");
  if (nb > 1) {
    scan_sums_kernel<<<1, SCAN_THREADS, 0, s>>>(sums, (int)nb);
    PMGB_LAUNCHED("scan_sums_kernel");
    scan_add_kernel<<<wave_grid(scan_add_kernel, n, 256), 256, 0, s>>>(out, n, sums, grand_total);
    PMGB_LAUNCHED("scan_add_kernel");
  }
  return PMGB_OK;
}

// Scratch of the sort: tile counts (keys), tile offsets (keys + 1: the last
// entry is the particle count), scan block sums, two words per particle
// (a rank, or the permuted gather's key and stayer rank), the stayer counts
// (keys).
size_t sort_workspace_size(int nx, int ny, int nz, int64_t np) {
  const size_t keys = (size_t)tile_key_count(nx, ny, nz);
  auto a = [](size_t b) { return (b + 255) & ~(size_t)255; };
  return a(keys * 4) + a((keys + 1) * 4) + a(((keys + SCAN_BLOCK - 1) / SCAN_BLOCK) * 4) +
         a((size_t)np * 8) + a(keys * 4) + 256;
}

struct SortScratch {
  // rank: ranks of the first sort (np words), or (from the permuted gather)
  // np pairs of the new tile key and the particle's rank among those that
  // stayed in their tile (~0 for the others); stay: per tile, how many
  // stayed (the leavers' slot cursor of the re-sort)
  unsigned *counts, *offsets, *sums, *rank, *stay, *work;
};

static SortScratch sort_scratch(void *ws, int nx, int ny, int nz, int64_t np) {
  const size_t keys = (size_t)tile_key_count(nx, ny, nz);
  auto a = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char *c = static_cast<char *>(ws);
  SortScratch sc;
  sc.counts = reinterpret_cast<unsigned *>(c);
  c += a(keys * 4);
  sc.offsets = reinterpret_cast<unsigned *>(c);
  c += a((keys + 1) * 4);
  sc.sums = reinterpret_cast<unsigned *>(c);
  c += a(((keys + SCAN_BLOCK - 1) / SCAN_BLOCK) * 4);
  sc.rank = reinterpret_cast<unsigned *>(c);  // np words, or np (key, rank) pairs
  c += a((size_t)np * 8);
  sc.stay = reinterpret_cast<unsigned *>(c);
  c += a(keys * 4);
  sc.work = reinterpret_cast<unsigned *>(c);
  return sc;
}

static int check_sort_ws(void *ws, size_t bytes, int nx, int ny, int nz, int64_t np) {
  if (!ws || bytes < sort_workspace_size(nx, ny, nz, np))
    return fail(PMGB_ERR_WORKSPACE, "the sorted path needs " +
                                        std::to_string(sort_workspace_size(nx, ny, nz, np)) +
                                        " sort workspace bytes");
  if (reinterpret_cast<uintptr_t>(ws) % 256 != 0)
    return fail(PMGB_ERR_WORKSPACE, "the sort workspace must be 256-byte aligned");
  return PMGB_OK;
}

static unsigned tile_grid(int64_t keys) {
  return (unsigned)std::min<int64_t>(keys, (int64_t)sm_count() * 8);
}

// The scatter's grid: one wave of resident CTAs (every CTA strides over the
// same number of 1024-particle chunks, so a partial last wave would leave
// SMs idle for a third of the kernel).
static unsigned scatter_grid(int64_t np) {
  return wave_grid(scatter_kernel, (np + SCATTER_ILP - 1) / SCATTER_ILP, 256);
}

int tile_sort(const float *pos, const float *vel, const unsigned *id, int64_t np, int nx, int ny,
              int nz, float *pos2, float *vel2, unsigned *id2, void *ws, size_t bytes,
              cudaStream_t s, unsigned *dest) {
  PMGB_TRY(check_sort_ws(ws, bytes, nx, ny, nz, np));
  const int64_t keys = tile_key_count(nx, ny, nz);
  SortScratch sc = sort_scratch(ws, nx, ny, nz, np);
  PMGB_CUDA(cudaMemsetAsync(sc.counts, 0, keys * 4, s));
  if (np > 0) {
    tile_rank_kernel<<<wave_grid(tile_rank_kernel, np, 256), 256, 0, s>>>(
        pos, np, nx, ny, nz, sc.counts, sc.rank);
    PMGB_LAUNCHED("tile_rank_kernel");
  }
  PMGB_TRY(exclusive_scan(sc.counts, sc.offsets, keys, sc.sums, (unsigned)np, s));
  if (np > 0) {
    scatter_kernel<<<scatter_grid(np), 256, 0, s>>>(pos, vel, id, sc.rank, np, nx, ny, nz,
                                                    sc.offsets, nullptr, pos2, vel2, id2, dest);
    PMGB_LAUNCHED("scatter_kernel");
  }
  return PMGB_OK;
}

int unpermute3(const float *in, const unsigned *id, int64_t np, float *out, cudaStream_t s) {
  if (np == 0) return PMGB_OK;
  unpermute3_kernel<<<wave_grid(unpermute3_kernel, np, 256), 256, 0, s>>>(in, id, np, out);
  PMGB_LAUNCHED("unpermute3_kernel");
  return PMGB_OK;
}

int permute3(const float *in, const unsigned *id, int64_t np, float *out, cudaStream_t s) {
  if (np == 0) return PMGB_OK;
  permute3_kernel<<<wave_grid(permute3_kernel, np, 256), 256, 0, s>>>(in, id, np, out, np);
  PMGB_LAUNCHED("permute3_kernel");
  return PMGB_OK;
}

int gather3(const float *in, int64_t n_in, const unsigned *idx, int64_t n, float *out,
            cudaStream_t s) {
  if (n == 0) return PMGB_OK;
  permute3_kernel<<<wave_grid(permute3_kernel, n, 256), 256, 0, s>>>(in, idx, n, out, n_in);
  PMGB_LAUNCHED("permute3_kernel");
  return PMGB_OK;
}

// Paint of tile-sorted particles (ranges from the last sort); the mesh is
// overwritten.
int paint_sorted(float *mesh, int nx, int ny, int nz, const float *pos, int64_t np,
                 void *sort_ws, size_t sort_bytes, unsigned *stats, cudaStream_t s) {
  PMGB_TRY(check_sort_ws(sort_ws, sort_bytes, nx, ny, nz, np));
  PMGB_CUDA(cudaMemsetAsync(mesh, 0, (size_t)nx * ny * nz * sizeof(float), s));
  if (np == 0) return PMGB_OK;
  const int64_t keys = tile_key_count(nx, ny, nz);
  SortScratch sc = sort_scratch(sort_ws, nx, ny, nz, np);
  const int vec = (nz % 4 == 0 && reinterpret_cast<uintptr_t>(mesh) % 16 == 0) ? 1 : 0;
  // TMA flush of interior tiles: a 3-D map over the mesh, box 12 x 9 x 9
  CUtensorMap map;
  memset(&map, 0, sizeof(map));
  int use_tma = 0;
  if (vec && nz >= TBZ && ny >= TB && nx >= TB) {
    const uint64_t dims[3] = {(uint64_t)nz, (uint64_t)ny, (uint64_t)nx};
    const uint64_t strides[2] = {(uint64_t)nz * 4, (uint64_t)ny * nz * 4};
    const uint32_t box[3] = {TBZ, TB, TB};
    use_tma = make_tensor_map(&map, mesh, 3, dims, strides, box) == PMGB_OK ? 1 : 0;
    clear_error();
  }
  static bool ready[64] = {false};
  int dev = 0;
  PMGB_CUDA(cudaGetDevice(&dev));
  if (dev >= 64 || !ready[dev]) {
    PMGB_TRY(set_smem((const void *)paint_tiles_kernel, PAINT_SMEM));
    if (dev < 64) ready[dev] = true;
  }
  PMGB_CUDA(cudaMemsetAsync(sc.work, 0, sizeof(unsigned), s));
  const unsigned grid = (unsigned)std::min<int64_t>((keys + PAINT_WARPS - 1) / PAINT_WARPS,
                                                    (int64_t)sm_count() * 3);
  paint_tiles_kernel<<<grid, PAINT_WARPS * 32, PAINT_SMEM, s>>>(
      mesh, nx, ny, nz, pos, sc.offsets, (uint32_t)keys, sc.work, stats, vec, map, use_tma);
  PMGB_LAUNCHED("paint_tiles_kernel");
  return PMGB_OK;
}

// Tile-staged gather + kick + drift of tile-sorted particles; counts the new
// positions per tile and records each particle's rank in its new tile.  The
// drifted positions go to pos_out (pos itself for an in-place update).  With
// mesh_next, the new positions are also painted there (overwritten): the
// density of the next step.
// f3: the three force meshes (component stride cs), or with `pot` the
// potential mesh from which the gather derives them.
int rkd_sorted(const float *f3, int64_t cs, int nx, int ny, int nz, const float *pos,
               float *pos_out, float *vel, int64_t np, float kick, float drift, void *sort_ws,
               size_t sort_bytes, unsigned *stats, cudaStream_t s, float *mesh_next, bool pot,
               const PermIO &io) {
  PMGB_TRY(check_sort_ws(sort_ws, sort_bytes, nx, ny, nz, np));
  const int64_t keys = tile_key_count(nx, ny, nz);
  SortScratch sc = sort_scratch(sort_ws, nx, ny, nz, np);
  PMGB_CUDA(cudaMemsetAsync(sc.counts, 0, keys * 4, s));
  if (np == 0) return PMGB_OK;
  // TMA prefetch of interior boxes: forces, a 4-D map (z, y, x, component)
  // with box 12 x 9 x 9 x 3; potential, a 3-D map with box 16 x 13 x 13
  CUtensorMap map;
  memset(&map, 0, sizeof(map));
  int use_tma = 0;
  const bool al = nz % 4 == 0 && reinterpret_cast<uintptr_t>(f3) % 16 == 0;
  if (pot) {
    if (al && nz >= PBZ && ny >= PBY && nx >= PBX) {
      const uint64_t dims[3] = {(uint64_t)nz, (uint64_t)ny, (uint64_t)nx};
      const uint64_t strides[2] = {(uint64_t)nz * 4, (uint64_t)ny * nz * 4};
      const uint32_t box[3] = {PBZ, PBY, PBX};
      use_tma = make_tensor_map(&map, f3, 3, dims, strides, box) == PMGB_OK ? 1 : 0;
      clear_error();
    }
  } else if (al && cs % 4 == 0 && nz >= TBZ && ny >= TB && nx >= TB) {
    const uint64_t dims[4] = {(uint64_t)nz, (uint64_t)ny, (uint64_t)nx, 3};
    const uint64_t strides[3] = {(uint64_t)nz * 4, (uint64_t)ny * nz * 4, (uint64_t)cs * 4};
    const uint32_t box[4] = {TBZ, TB, TB, 3};
    use_tma = make_tensor_map(&map, f3, 4, dims, strides, box) == PMGB_OK ? 1 : 0;
    clear_error();
  }
  CUtensorMap pmap;
  memset(&pmap, 0, sizeof(pmap));
  // per variant and device: shared-memory opt-in done, and the resident CTAs
  // per SM (the grid of the dynamic tile schedule)
  static int resident[4][64] = {{0}};
  int dev = 0;
  PMGB_CUDA(cudaGetDevice(&dev));
  const int variant = (mesh_next ? 1 : 0) + (pot ? 2 : 0);
  const void *fn = variant == 0   ? (const void *)rkd_tiles_kernel<false, false>
                   : variant == 1 ? (const void *)rkd_tiles_kernel<true, false>
                   : variant == 2 ? (const void *)rkd_tiles_kernel<false, true>
                                  : (const void *)rkd_tiles_kernel<true, true>;
  const size_t dsmem = mesh_next ? RKDP_SMEM : 0;
  int per_sm = dev < 64 ? resident[variant][dev] : 0;
  if (per_sm == 0) {
    PMGB_TRY(set_smem(fn, dsmem));
    PMGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, TILE_THREADS, dsmem));
    per_sm = std::max(per_sm, 1);
    if (dev < 64) resident[variant][dev] = per_sm;
  }
  int use_ptma = 0;
  bool aligned = false;
  if (mesh_next) {
    const int64_t ncell = (int64_t)nx * ny * nz;
    PMGB_CUDA(cudaMemsetAsync(mesh_next, 0, ncell * sizeof(float), s));
    aligned = nz % 4 == 0 && reinterpret_cast<uintptr_t>(mesh_next) % 16 == 0;
    if (aligned && nz >= NBZ && ny >= NB && nx >= NB) {
      // 3-D map of the density mesh, box 12 x 9 x 1 (one x-plane of the paint box)
      const uint64_t dims[3] = {(uint64_t)nz, (uint64_t)ny, (uint64_t)nx};
      const uint64_t strides[2] = {(uint64_t)nz * 4, (uint64_t)ny * nz * 4};
      const uint32_t box[3] = {NBZ, NB, 1};
      use_ptma = make_tensor_map(&pmap, mesh_next, 3, dims, strides, box) == PMGB_OK ? 1 : 0;
      clear_error();
    }
  }
  // the tile counter of the dynamic schedule (the word after the painter's)
  unsigned *work = sc.work + 1;
  PMGB_CUDA(cudaMemsetAsync(work, 0, sizeof(unsigned), s));
#define RKD_ARGS                                                                             \
  f3, cs, nx, ny, nz, pos, pos_out, vel, sc.offsets, (uint32_t)keys, kick, drift, sc.counts, \
      sc.rank, stats, map, use_tma, mesh_next, aligned ? 1 : 0, pmap, use_ptma, work, io, \
      tu.gather_static_quarters
  const Tuning tu = tuning();
  const int use_sm = tu.gather_ctas_per_sm > 0 ? std::min(per_sm, tu.gather_ctas_per_sm) : per_sm;
  const unsigned grid = (unsigned)std::min<int64_t>(keys, (int64_t)sm_count() * use_sm);
  switch (variant) {
    case 0: rkd_tiles_kernel<false, false><<<grid, TILE_THREADS, dsmem, s>>>(RKD_ARGS); break;
    case 1: rkd_tiles_kernel<true, false><<<grid, TILE_THREADS, dsmem, s>>>(RKD_ARGS); break;
    case 2: rkd_tiles_kernel<false, true><<<grid, TILE_THREADS, dsmem, s>>>(RKD_ARGS); break;
    default: rkd_tiles_kernel<true, true><<<grid, TILE_THREADS, dsmem, s>>>(RKD_ARGS); break;
  }
#undef RKD_ARGS
  PMGB_LAUNCHED("rkd_tiles_kernel");
  return PMGB_OK;
}

// Scan of the tile counts left by rkd_sorted, then the scatter of
// (pos, vel, id) to (pos2, vel2, id2) in tile order; dest (nullable)
// receives each particle's new index.
int tile_scatter(const float *pos, const float *vel, const unsigned *id, int64_t np, int nx,
                 int ny, int nz, float *pos2, float *vel2, unsigned *id2, unsigned *dest,
                 void *sort_ws, size_t sort_bytes, cudaStream_t s) {
  PMGB_TRY(check_sort_ws(sort_ws, sort_bytes, nx, ny, nz, np));
  const int64_t keys = tile_key_count(nx, ny, nz);
  SortScratch sc = sort_scratch(sort_ws, nx, ny, nz, np);
  PMGB_TRY(exclusive_scan(sc.counts, sc.offsets, keys, sc.sums, (unsigned)np, s));
  // the counts become the per-tile slot cursors of the scatter
  PMGB_CUDA(cudaMemsetAsync(sc.counts, 0, keys * 4, s));
  if (np > 0) {
    scatter_kernel<<<scatter_grid(np), 256, 0, s>>>(pos, vel, id, nullptr, np, nx, ny, nz,
                                                    sc.offsets, sc.counts, pos2, vel2, id2,
                                                    dest);
    PMGB_LAUNCHED("scatter_kernel");
  }
  return PMGB_OK;
}

// The permuted loop's re-sort: scan of the tile counts the gather left,
// then perm (where each new slot's particle is) from the keys the gather
// wrote (the sort workspace's rank array).
int index_resort(int64_t np, int nx, int ny, int nz, const unsigned *perm_old,
                 unsigned *perm_new, const unsigned *id_in, unsigned *id_out, void *sort_ws,
                 size_t sort_bytes, cudaStream_t s) {
  PMGB_TRY(check_sort_ws(sort_ws, sort_bytes, nx, ny, nz, np));
  const int64_t keys = tile_key_count(nx, ny, nz);
  SortScratch sc = sort_scratch(sort_ws, nx, ny, nz, np);
  PMGB_TRY(exclusive_scan(sc.counts, sc.offsets, keys, sc.sums, (unsigned)np, s));
  if (np > 0) {
    unsigned grid = wave_grid(index_scatter_kernel, (np + ISCATTER_ILP - 1) / ISCATTER_ILP, 256);
    const Tuning tu = tuning();
    if (tu.resort_ctas_per_sm > 0)
      grid = (unsigned)std::min<int64_t>(grid, (int64_t)sm_count() * tu.resort_ctas_per_sm);
    index_scatter_kernel<<<grid, 256, 0, s>>>(reinterpret_cast<const uint2 *>(sc.rank), np,
                                        sc.offsets, sc.stay, perm_new, perm_old, id_in, id_out);
    PMGB_LAUNCHED("index_scatter_kernel");
  }
  return PMGB_OK;
}

int gather_u32(const unsigned *in, const unsigned *idx, int64_t np, unsigned *out,
               cudaStream_t s) {
  if (np == 0) return PMGB_OK;
  gather_u32_kernel<<<wave_grid(gather_u32_kernel, np, 256), 256, 0, s>>>(in, idx, np, out);
  PMGB_LAUNCHED("gather_u32_kernel");
  return PMGB_OK;
}

void perm_scratch(void *sort_ws, int nx, int ny, int nz, int64_t np, PermIO *io) {
  const SortScratch sc = sort_scratch(sort_ws, nx, ny, nz, np);
  io->key_out = sc.rank;  // np (key, stayer rank) pairs
  io->stay_out = sc.stay;
}

int check_sort_workspace(void *ws, size_t bytes, int nx, int ny, int nz, int64_t np) {
  return check_sort_ws(ws, bytes, nx, ny, nz, np);
}

// The tile ranges (nkeys + 1 offsets) of the current order.
const unsigned *tile_offsets(void *sort_ws, int nx, int ny, int nz, int64_t np) {
  return sort_scratch(sort_ws, nx, ny, nz, np).offsets;
}

// One FastPM step on tile-sorted particles.  Reads (pos, vel, id), writes
// the advanced state, sorted by the new positions, to (pos2, vel2, id2).
// `mesh_ws` is the composite workspace (pm_workspace_size); `sort_ws` the
// sort scratch holding the ranges of the current order; `stats` (nullable)
// counts particles found outside their tile (stale ranges).  For adjoints
// the step can record (each nullable): the force meshes [3][nx][ny][nz]
// (written there instead of the workspace), each particle's index after the
// step (dest), and the tile ranges of the order it started from (offsets).
int fpm_step_sorted(const float *pos, float *vel, const unsigned *id, float *pos2, float *vel2,
                    unsigned *id2, int64_t np, int nx, int ny, int nz, float kick, float drift,
                    float r_split, void *mesh_ws, size_t mesh_bytes, void *sort_ws,
                    size_t sort_bytes, float *force3_out, unsigned *dest_out,
                    unsigned *offsets_out, unsigned *stats, cudaStream_t s) {
  PMGB_TRY(check_sort_ws(sort_ws, sort_bytes, nx, ny, nz, np));
  if (offsets_out)
    PMGB_CUDA(cudaMemcpyAsync(offsets_out, tile_offsets(sort_ws, nx, ny, nz, np),
                              (tile_key_count(nx, ny, nz) + 1) * sizeof(unsigned),
                              cudaMemcpyDeviceToDevice, s));
  float *f3 = nullptr;
  PMGB_TRY(force_meshes_sorted(pos, np, nx, ny, nz, r_split, mesh_ws, mesh_bytes, sort_ws,
                               sort_bytes, stats, force3_out, &f3, s));
  // the drifted positions go to workspace scratch, so pos keeps the
  // positions the step started from (the reverse step needs them)
  float *drifted = pm_workspace_particles(mesh_ws, mesh_bytes, nx, ny, nz, np);
  if (!drifted) return PMGB_ERR_WORKSPACE;
  PMGB_TRY(rkd_sorted(f3, (int64_t)nx * ny * nz, nx, ny, nz, pos, drifted, vel, np, kick, drift,
                      sort_ws, sort_bytes, stats, s));
  return tile_scatter(drifted, vel, id, np, nx, ny, nz, pos2, vel2, id2, dest_out, sort_ws,
                      sort_bytes, s);
}

// A run of sorted steps: the density of the first step is painted from the
// tile ranges in sort_ws; every later density is painted by the previous
// step's gather (rkd_tiles_kernel<true>) from the new positions, before the
// re-sort, so each step reads the particles once.
// Second stream and events of the run loop's fork/join (one set per host
// thread and device, created on first use: make the first run call outside
// any stream capture).
struct Aux {
  cudaStream_t s2 = nullptr;   // the highest priority
  cudaStream_t s2d = nullptr;  // the default priority
  cudaEvent_t gathered = nullptr, sorted = nullptr;
};

static int aux_stream(Aux **out) {
  thread_local std::map<int, Aux> aux;
  int dev = 0;
  PMGB_CUDA(cudaGetDevice(&dev));
  Aux &x = aux[dev];
  if (!x.s2) {
    // the sort's stream at the highest priority: its blocks are placed ahead
    // of the concurrent FFT kernels' as SMs free up (measured 8.05 -> 7.89
    // ms per step at 512^3 against the default priority)
    int least = 0, greatest = 0;
    PMGB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    PMGB_CUDA(cudaStreamCreateWithPriority(&x.s2, cudaStreamNonBlocking, greatest));
    PMGB_CUDA(cudaStreamCreateWithFlags(&x.s2d, cudaStreamNonBlocking));
    PMGB_CUDA(cudaEventCreateWithFlags(&x.gathered, cudaEventDisableTiming));
    PMGB_CUDA(cudaEventCreateWithFlags(&x.sorted, cudaEventDisableTiming));
  }
  *out = &x;
  return PMGB_OK;
}

// Launch timing of the run loop (set_run_timing): while on, a run records
// CUDA events around each of its gathers, force evaluations and re-sorts, on
// the streams they run on; run_timing reads the last timed run's pairs back.
// Event slots of step i: 6i + {0, 1} its gather, {2, 3} the force
// evaluation issued after it (the next step's), {4, 5} its re-sort; the
// force evaluation before step 0 takes 6n + {0, 1}.
static std::mutex g_rt_mu;
static bool g_rt_on = false;
static int g_rt_dev = -1;
static std::vector<cudaEvent_t> g_rt_ev;
static int g_rt_steps = 0;  // steps of the last completed timed run (0: none)

int set_run_timing(bool on) {
  std::lock_guard<std::mutex> lk(g_rt_mu);
  g_rt_on = on;
  g_rt_steps = 0;
  return PMGB_OK;
}

// Holds the timing lock for the whole run while timing is on, so that two
// host threads' runs cannot interleave their event slots.
class RunTimer {
 public:
  int begin(int n) {
    std::unique_lock<std::mutex> lk(g_rt_mu);
    if (!g_rt_on) return PMGB_OK;
    int dev = 0;
    PMGB_CUDA(cudaGetDevice(&dev));
    if (dev != g_rt_dev) {
      for (cudaEvent_t e : g_rt_ev) cudaEventDestroy(e);
      g_rt_ev.clear();
      g_rt_dev = dev;
    }
    while (g_rt_ev.size() < 6 * (size_t)n + 2) {
      cudaEvent_t e = nullptr;
      PMGB_CUDA(cudaEventCreate(&e));
      g_rt_ev.push_back(e);
    }
    g_rt_steps = 0;
    n_ = n;
    lk_ = std::move(lk);
    return PMGB_OK;
  }
  int mark(int slot, cudaStream_t s) {
    if (lk_.owns_lock()) PMGB_CUDA(cudaEventRecord(g_rt_ev[slot], s));
    return PMGB_OK;
  }
  void done() {
    if (lk_.owns_lock()) g_rt_steps = n_;
  }

 private:
  std::unique_lock<std::mutex> lk_;
  int n_ = 0;
};

int run_timing(double *gather_ms, double *forces_ms, double *resort_ms, int *steps) {
  std::lock_guard<std::mutex> lk(g_rt_mu);
  if (g_rt_steps <= 0)
    return fail(PMGB_ERR_INVALID_ARGUMENT,
                "no timed run: switch timing on (pmgb_set_run_timing) before the run");
  const int n = g_rt_steps;
  auto span = [&](int a, double *acc) -> int {
    float ms = 0.f;
    const cudaError_t e = cudaEventElapsedTime(&ms, g_rt_ev[a], g_rt_ev[a + 1]);
    if (e == cudaErrorNotReady) {
      cudaGetLastError();
      return fail(PMGB_ERR_CUDA, "the timed run has not finished: synchronise its stream first");
    }
    if (e != cudaSuccess) return fail(PMGB_ERR_CUDA, std::string("cudaEventElapsedTime: ") +
                                                         cudaGetErrorString(e));
    *acc += ms;
    return PMGB_OK;
  };
  double g = 0.0, f = 0.0, r = 0.0;
  PMGB_TRY(span(6 * n, &f));
  for (int i = 0; i < n; ++i) {
    PMGB_TRY(span(6 * i, &g));
    if (i + 1 < n) {
      PMGB_TRY(span(6 * i + 2, &f));
      PMGB_TRY(span(6 * i + 4, &r));
    }
  }
  if (gather_ms) *gather_ms = g / n;
  if (forces_ms) *forces_ms = f / n;
  if (resort_ms) *resort_ms = n > 1 ? r / (n - 1) : 0.0;
  if (steps) *steps = n;
  return PMGB_OK;
}

int fpm_run_sorted(float *pos_a, float *vel_a, unsigned *id_a, float *pos_b, float *vel_b,
                   unsigned *id_b, int64_t np, int nx, int ny, int nz, int n_steps,
                   const float *kick, const float *drift, float r_split, void *mesh_ws,
                   size_t mesh_bytes, void *sort_ws, size_t sort_bytes, unsigned *stats,
                   cudaStream_t s) {
  PMGB_TRY(check_sort_ws(sort_ws, sort_bytes, nx, ny, nz, np));
  float *mesh, *f3, *g3;
  void *dk, *fk;
  unsigned *work;
  PMGB_TRY(pm_workspace_regions(mesh_ws, mesh_bytes, nx, ny, nz, np, &mesh, &dk, &fk, &f3, &g3,
                                &work));
  (void)g3;
  (void)work;
  float *drifted = pm_workspace_particles(mesh_ws, mesh_bytes, nx, ny, nz, np);
  if (!drifted) return PMGB_ERR_WORKSPACE;
  if (n_steps <= 0) return PMGB_OK;
  float *P[2] = {pos_a, pos_b}, *V[2] = {vel_a, vel_b};
  unsigned *I[2] = {id_a, id_b};
  Aux *aux;
  PMGB_TRY(aux_stream(&aux));
  // the re-sort's stream (Tuning::resort_priority)
  cudaStream_t s2 = tuning().resort_priority ? aux->s2d : aux->s2;
  // Forces from the potential where the spectral pipeline serves the mesh:
  // one inverse transform instead of three, the order-1 gradient taken by
  // the gather as the equivalent real-space stencil (f3 then holds the
  // potential).
  const bool pot = spectral_enabled() && spectral_supported(nx, ny, nz) && nz % 4 == 0 &&
                   reinterpret_cast<uintptr_t>(mesh) % 16 == 0 &&
                   reinterpret_cast<uintptr_t>(f3) % 16 == 0;
  const float scale = 1.0f / (float)((int64_t)nx * ny * nz);
  auto forces = [&]() -> int {
    if (pot) return spectral_potential(mesh, dk, f3, nx, ny, nz, r_split, scale, s);
    return mesh_forces(mesh, nx, ny, nz, r_split, dk, fk, f3, s);
  };
  // The particles stay where the gather writes them: step i's gather reads
  // slot p of the tile ranges from index perm[p] of buffer `cur` and writes
  // it to index p of the other buffer (step 0, whose input is already in
  // tile order, updates buffer a in place), with its new tile key; the
  // re-sort between steps then only rebuilds perm (index_resort, 8 bytes
  // per particle instead of 56), and one full scatter after the last gather
  // puts the state in tile order.  perm lives in the workspace's particle
  // region, the keys in the sort workspace's rank array.
  // two permutations in turn (the re-sort reads the one the gather used)
  unsigned *perm[2] = {reinterpret_cast<unsigned *>(drifted),
                       reinterpret_cast<unsigned *>(drifted) + np};
  SortScratch sc = sort_scratch(sort_ws, nx, ny, nz, np);
  RunTimer rt;
  PMGB_TRY(rt.begin(n_steps));
  PMGB_TRY(paint_sorted(mesh, nx, ny, nz, pos_a, np, sort_ws, sort_bytes, stats, s));
  PMGB_TRY(rt.mark(6 * n_steps, s));
  PMGB_TRY(forces());
  PMGB_TRY(rt.mark(6 * n_steps + 1, s));
  int cur = 0, pc = 0;  // buffer holding the state; perm[pc] its permutation
  for (int i = 0; i < n_steps; ++i) {
    const bool last = i + 1 == n_steps;
    const int out = i == 0 ? cur : cur ^ 1;
    // the gather of step i needs step i-1's re-sort (perm, tile offsets) and
    // step i's forces (issued on s)
    if (i > 0) PMGB_CUDA(cudaStreamWaitEvent(s, aux->sorted, 0));
    PermIO io;
    io.perm = i == 0 ? nullptr : perm[pc];
    io.vel_out = V[out];
    perm_scratch(sort_ws, nx, ny, nz, np, &io);
    PMGB_TRY(rt.mark(6 * i, s));
    PMGB_TRY(rkd_sorted(f3, (int64_t)nx * ny * nz, nx, ny, nz, P[cur], P[out], V[cur], np,
                        kick[i], drift[i], sort_ws, sort_bytes, stats, s,
                        last ? nullptr : mesh, pot, io));
    PMGB_TRY(rt.mark(6 * i + 1, s));
    // the re-sort of step i (on the second stream) and the forces of step
    // i+1 (from the density the gather just painted) are independent: they
    // touch disjoint buffers and overlap
    PMGB_CUDA(cudaEventRecord(aux->gathered, s));
    PMGB_CUDA(cudaStreamWaitEvent(s2, aux->gathered, 0));
    PMGB_TRY(rt.mark(6 * i + 4, s2));
    if (!last) {
      // ids follow the gather (from the order it read), perm is rebuilt
      PMGB_TRY(index_resort(np, nx, ny, nz, i == 0 ? nullptr : perm[pc], perm[pc ^ 1],
                            I[cur], I[out], sort_ws, sort_bytes, s2));
      pc ^= 1;
      cur = out;
    } else {
      if (i > 0) PMGB_TRY(gather_u32(I[cur], perm[pc], np, I[out], s2));
      cur = out;
      PMGB_TRY(tile_scatter(P[cur], V[cur], I[cur], np, nx, ny, nz, P[cur ^ 1], V[cur ^ 1],
                            I[cur ^ 1], nullptr, sort_ws, sort_bytes, s2));
      cur ^= 1;
    }
    PMGB_TRY(rt.mark(6 * i + 5, s2));
    PMGB_CUDA(cudaEventRecord(aux->sorted, s2));
    if (!last) {
      PMGB_TRY(rt.mark(6 * i + 2, s));
      PMGB_TRY(forces());
      PMGB_TRY(rt.mark(6 * i + 3, s));
    }
  }
  // the state ends in buffer n_steps & 1 (one buffer change per step: none
  // in step 0, one in each later gather, one in the final scatter)
  (void)cur;
  // join: everything of the run is ordered before later work on s
  PMGB_CUDA(cudaStreamWaitEvent(s, aux->sorted, 0));
  rt.done();
  return PMGB_OK;
}

int fpm_run_sorted_record(float *xs, float *vel_a, unsigned *id_a, float *vel_b, unsigned *id_b,
                          float *pos_out, int64_t np, int nx, int ny, int nz, int n_steps,
                          const float *kick, const float *drift, float r_split, void *mesh_ws,
                          size_t mesh_bytes, void *sort_ws, size_t sort_bytes, float *f3s,
                          unsigned *dests, unsigned *offs, unsigned *stats, cudaStream_t s,
                          bool pot) {
  if (pot && !spectral_supported(nx, ny, nz))
    return fail(PMGB_ERR_UNSUPPORTED,
                "recording the potential needs the potential pipeline's mesh shapes "
                "(power-of-two nx in [8,1024], ny in [64,512], nz in [16,512])");
  PMGB_TRY(check_sort_ws(sort_ws, sort_bytes, nx, ny, nz, np));
  float *mesh, *f3, *g3;
  void *dk, *fk;
  unsigned *work;
  PMGB_TRY(pm_workspace_regions(mesh_ws, mesh_bytes, nx, ny, nz, np, &mesh, &dk, &fk, &f3, &g3,
                                &work));
  (void)f3;
  (void)g3;
  (void)work;
  float *drifted = pm_workspace_particles(mesh_ws, mesh_bytes, nx, ny, nz, np);
  if (!drifted) return PMGB_ERR_WORKSPACE;
  if (n_steps <= 0) return PMGB_OK;
  const int64_t ncell = (int64_t)nx * ny * nz, keys = tile_key_count(nx, ny, nz);
  float *V[2] = {vel_a, vel_b};
  unsigned *I[2] = {id_a, id_b};
  Aux *aux;
  PMGB_TRY(aux_stream(&aux));
  // step i's forces: three meshes at f3s + i*3ncell, or the potential at
  // f3s + i*ncell
  const int64_t per = pot ? ncell : 3 * ncell;
  const float scale = 1.0f / (float)ncell;
  auto forces = [&](int i) -> int {
    if (pot) return spectral_potential(mesh, dk, f3s + per * i, nx, ny, nz, r_split, scale, s);
    return mesh_forces(mesh, nx, ny, nz, r_split, dk, fk, f3s + per * i, s);
  };
  PMGB_TRY(paint_sorted(mesh, nx, ny, nz, xs, np, sort_ws, sort_bytes, stats, s));
  PMGB_TRY(forces(0));
  for (int i = 0; i < n_steps; ++i) {
    const int a = i & 1, b = a ^ 1;
    float *x = xs + 3 * np * (int64_t)i;
    float *xn = i + 1 < n_steps ? x + 3 * np : pos_out;
    if (i > 0) PMGB_CUDA(cudaStreamWaitEvent(s, aux->sorted, 0));
    PMGB_CUDA(cudaMemcpyAsync(offs + (keys + 1) * (int64_t)i,
                              tile_offsets(sort_ws, nx, ny, nz, np),
                              (keys + 1) * sizeof(unsigned), cudaMemcpyDeviceToDevice, s));
    PMGB_TRY(rkd_sorted(f3s + per * i, ncell, nx, ny, nz, x, drifted, V[a], np, kick[i],
                        drift[i], sort_ws, sort_bytes, stats, s,
                        i + 1 < n_steps ? mesh : nullptr, pot));
    PMGB_CUDA(cudaEventRecord(aux->gathered, s));
    PMGB_CUDA(cudaStreamWaitEvent(aux->s2, aux->gathered, 0));
    PMGB_TRY(tile_scatter(drifted, V[a], I[a], np, nx, ny, nz, xn, V[b], I[b],
                          dests + np * (int64_t)i, sort_ws, sort_bytes, aux->s2));
    PMGB_CUDA(cudaEventRecord(aux->sorted, aux->s2));
    if (i + 1 < n_steps) PMGB_TRY(forces(i + 1));
  }
  PMGB_CUDA(cudaStreamWaitEvent(s, aux->sorted, 0));
  return PMGB_OK;
}

// ---------------------------------------------------------------------------
// Adjoint of the sorted step.
//
// Forward step (particles in tile order i): v' = v + kick F(x),
// x' = x + drift v', then the sort moves particle p to dest[p] (order i+1).
// Given the cotangents (g, h) of (x', v') in order i+1, the cotangents of
// (x, v) in order i are
//   u = h[dest] + drift g[dest],   gv = u,
//   gx = g[dest] + (dF/dx)^T (kick u),
// with (dF/dx)^T w = sum_c w_c grad F_c(x) + grad rho_bar(x) and
// rho_bar = sum_c A_c^T paint(w_c) (A_c the k-space operator of force
// component c, A_c^T its conjugate multiplier between an R2C and a C2R).
// ---------------------------------------------------------------------------
// The adjoint paint: a CTA of four warps paints one tile at a time into one
// shared box (11.8 KB), ten CTAs (40 warps) to an SM.  Measured on the
// 512^3 forward+adjoint step: one tile per warp with four boxes per CTA
// (16 warps per SM) 16.64 ms, two warps per box 16.28, three or four 15.97.
constexpr int ADJ_THREADS = 128;
constexpr int ADJ_BOX_WORDS = (3 * TBOX + 31) / 32 * 32;  // three components, 128-byte multiple
constexpr int ADJ_PAINT_SMEM = ADJ_BOX_WORDS * 4;
constexpr unsigned ADJ_BOX_COUNT = 8192;  // larger tiles paint with global atomics

__device__ __forceinline__ void adj_cotangent(const float *__restrict__ gx,
                                              const float *__restrict__ gv,
                                              const unsigned *__restrict__ dest, unsigned p,
                                              float kick, float drift, float g[3], float u[3],
                                              float w[3]) {
  const int64_t d = dest ? (int64_t)__ldg(dest + p) : (int64_t)p;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    g[c] = __ldg(gx + 3 * d + c);
    u[c] = __ldg(gv + 3 * d + c) + drift * g[c];
    w[c] = kick * u[c];
  }
}

// Paint of the three components of w = kick * u, one tile per CTA at a
// time (tiles from a counter).  The cotangents have no fixed
// range, so each tile uses block floating point: a first pass finds max |w|
// over the tile, the box then accumulates round(W * w * S) in int32 with
// native shared atomics, S a power of two chosen so that no cell can
// overflow (|sum| <= count * max * S <= 2^30).
__global__ void __launch_bounds__(ADJ_THREADS)
adj_paint3_tiles_kernel(float *__restrict__ g3, int64_t cs, int nx, int ny, int nz,
                        const float *__restrict__ pos, const unsigned *__restrict__ dest,
                        const float *__restrict__ gx, const float *__restrict__ gv, float kick,
                        float drift, const unsigned *__restrict__ offsets, uint32_t nkeys,
                        unsigned *__restrict__ next_tile, unsigned *__restrict__ stats, int vec,
                        const __grid_constant__ CUtensorMap tmap, int use_tma) {
  extern __shared__ __align__(128) int abox[];
  __shared__ uint32_t s_key[2];  // the grabbed tile, alternating between iterations
  __shared__ float s_max[ADJ_THREADS / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int *acc = abox;
  float *fb = reinterpret_cast<float *>(acc);
  for (uint32_t it = 0;; ++it) {
    // every branch below is uniform across the CTA (it depends on the tile only)
    if (tid == 0) s_key[it & 1] = atomicAdd(next_tile, 1u);
    __syncthreads();
    const uint32_t key = s_key[it & 1];
    if (key >= nkeys) break;
    const unsigned beg = __ldg(offsets + key), end = __ldg(offsets + key + 1);
    if (beg == end) continue;
    const int ox = (int)compact3(key >> 2) * TILE, oy = (int)compact3(key >> 1) * TILE,
              oz = (int)compact3(key) * TILE;
    const unsigned count = end - beg;
    // pass 1: the tile's largest cotangent component
    float m = 0.f;
    for (unsigned p = beg + tid; p < end; p += ADJ_THREADS) {
      float g[3], u[3], w[3];
      adj_cotangent(gx, gv, dest, p, kick, drift, g, u, w);
      m = fmaxf(m, fmaxf(fabsf(w[0]), fmaxf(fabsf(w[1]), fabsf(w[2]))));
      if (isnan(w[0] + w[1] + w[2])) m = INFINITY;  // fmaxf drops NaN: keep it visible
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) s_max[warp] = m;
    __syncthreads();
    m = s_max[0];
#pragma unroll
    for (int k = 1; k < ADJ_THREADS / 32; ++k) m = fmaxf(m, s_max[k]);
    if (m == 0.f) continue;  // nothing to paint
    // non-finite cotangents skip the box and propagate through global atomics
    const bool boxed = count < ADJ_BOX_COUNT && isfinite(m);
    int e = 0;
    if (boxed) {
      // S = 2^e with m * S * count <= 2^30
      e = (int)floorf(30.0f - log2f((float)count) - log2f(m));
      e = max(-120, min(120, e));
      for (int q = tid; q < 3 * TBOX; q += ADJ_THREADS) acc[q] = 0;
    }
    const float S = ldexpf(1.0f, e);
    __syncthreads();
    for (unsigned p = beg + tid; p < end; p += ADJ_THREADS) {
      float g[3], u[3], w[3];
      adj_cotangent(gx, gv, dest, p, kick, drift, g, u, w);
      const float x = __ldg(pos + 3 * (int64_t)p), y = __ldg(pos + 3 * (int64_t)p + 1),
                  z = __ldg(pos + 3 * (int64_t)p + 2);
      Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
      const int lx = ax.i0 - ox, ly = ay.i0 - oy, lz = az.i0 - oz;
      if (boxed && (unsigned)lx < (unsigned)TILE && (unsigned)ly < (unsigned)TILE &&
          (unsigned)lz < (unsigned)TILE) {
        const int q0 = (lx * TB + ly) * TBZ + lz;
        const float ws0 = w[0] * S, ws1 = w[1] * S, ws2 = w[2] * S;
#pragma unroll
        for (int n = 0; n < 8; ++n) {
          const float W = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                                    conn_z(n) ? az.k1 : az.k0);
          const int q = q0 + conn_x(n) * TB * TBZ + conn_y(n) * TBZ + conn_z(n);
          atomicAdd(acc + q, __float2int_rn(W * ws0));
          atomicAdd(acc + TBOX + q, __float2int_rn(W * ws1));
          atomicAdd(acc + 2 * TBOX + q, __float2int_rn(W * ws2));
        }
      } else {
        if (stats && boxed) atomicAdd(stats, 1u);
#pragma unroll
        for (int n = 0; n < 8; ++n) {
          const float W = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                                    conn_z(n) ? az.k1 : az.k0);
          const int64_t c = cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                                       conn_z(n) ? az.i1 : az.i0, ny, nz);
          atomicAdd(g3 + c, W * w[0]);
          atomicAdd(g3 + cs + c, W * w[1]);
          atomicAdd(g3 + 2 * cs + c, W * w[2]);
        }
      }
    }
    if (!boxed) continue;
    __syncthreads();
    const float inv = ldexpf(1.0f, -e);
    for (int q = tid; q < 3 * TBOX; q += ADJ_THREADS) fb[q] = (float)acc[q] * inv;
    const bool tma = use_tma && box_interior(ox, oy, oz, nx, ny, nz);
    if (tma) fence_async_shared();
    __syncthreads();
    if (tma) {
      if (tid == 0) {
        tma_reduce_add_4d(&tmap, oz, oy, ox, 0, fb);
        bulk_commit();
        bulk_wait_read();
      }
    } else if (vec) {
      for (int q = tid; q < 3 * TB * TB * 3; q += ADJ_THREADS) {
        const int gq = q % 3, r = q / 3, b = r % TB, r2 = r / TB, a = r2 % TB, c = r2 / TB;
        const float4 v =
            *reinterpret_cast<const float4 *>(fb + c * TBOX + (a * TB + b) * TBZ + 4 * gq);
        if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) {
          const int64_t cell = cell_index(wrap_index(ox + a, nx), wrap_index(oy + b, ny),
                                          wrap_index(oz + 4 * gq, nz), ny, nz);
          atomicAdd(reinterpret_cast<float4 *>(g3 + c * cs + cell), v);
        }
      }
    } else {
      for (int q = tid; q < 3 * TB * TB * TB; q += ADJ_THREADS) {
        const int cz = q % TB, r = q / TB, b = r % TB, r2 = r / TB, a = r2 % TB, c = r2 / TB;
        const float v = fb[c * TBOX + (a * TB + b) * TBZ + cz];
        if (v != 0.f)
          atomicAdd(g3 + c * cs + cell_index(wrap_index(ox + a, nx), wrap_index(oy + b, ny),
                                             wrap_index(oz + cz, nz), ny, nz), v);
      }
    }
    __syncthreads();  // the box is free for the next tile once the reduce has read it
  }
  if (use_tma && tid == 0) bulk_wait_all();
}

// Both position terms of the adjoint in one tile-staged gather (one CTA per
// tile, the boxes of the three force meshes and of rho_bar fetched by TMA
// and double buffered), plus the cotangent update:
// gx_out = g + sum_n (rho_bar + w . F)(c_n) dW_n/dx,  gv_out = u.
constexpr int RBOX_STRIDE = (TBOX + 31) / 32 * 32;
constexpr uint32_t RBOX_BYTES = TBOX * sizeof(float);

// POT: f3 is the potential the step's forces came from (cs unused, fmap its
// 3-D map with the 16 x 13 x 13 box of the forward gather) and each tile's
// force box is computed from the staged potential box, as in
// rkd_tiles_kernel<., true>.
template <bool POT>
__global__ void __launch_bounds__(TILE_THREADS)
adj_gather_tiles_kernel(const float *__restrict__ f3, int64_t cs, const float *__restrict__ rbar,
                        int nx, int ny, int nz, const float *__restrict__ pos,
                        const unsigned *__restrict__ dest, const float *__restrict__ gx,
                        const float *__restrict__ gv, float *__restrict__ gx_out,
                        float *__restrict__ gv_out, float kick, float drift,
                        const unsigned *__restrict__ offsets, uint32_t nkeys,
                        unsigned *__restrict__ stats, const __grid_constant__ CUtensorMap fmap,
                        const __grid_constant__ CUtensorMap rmap, int use_tma,
                        unsigned *__restrict__ work) {
  __shared__ __align__(128) float fb[2][FBOX_STRIDE];
  __shared__ __align__(128) float rb[2][RBOX_STRIDE];
  __shared__ __align__(16) float ff[POT ? FBOX : 4];  // POT: the tile's force box
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t s_grab[2];
  constexpr uint32_t BOX_BYTES = (POT ? PBOX_BYTES : FBOX_BYTES) + RBOX_BYTES;
  const int tid = threadIdx.x;
  // the tile's boxes by TMA, completing on `b`
  auto issue = [&](float *fdst, float *rdst, const TileInfo &t, uint64_t *b) {
    if (POT) tma_load_3d(fdst, &fmap, t.oz - 4, t.oy - 2, t.ox - 2, b);
    else tma_load_4d(fdst, &fmap, t.oz, t.oy, t.ox, 0, b);
    tma_load_3d(rdst, &rmap, t.oz, t.oy, t.ox, b);
  };
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_async_shared();
  }
  __syncthreads();
  uint32_t phase0 = 0u, phase1 = 0u;
  // TileSchedule, each tile fixed two tiles ahead by thread 0
  uint32_t key = blockIdx.x;
  if (key >= nkeys) return;
  const TileSchedule sched(nkeys, 0);  // no global atomics: dynamic
  uint32_t knext = gridDim.x + blockIdx.x;  // tiles 0 and 1 are static
  uint32_t it = 0;                          // index of the current tile
  TileInfo cur = tile_info(offsets, key, nx, ny, nz, use_tma, POT);
  if (cur.tma && tid == 0) {
    mbar_expect_tx(&bar[0], BOX_BYTES);
    issue(fb[0], rb[0], cur, &bar[0]);
  }
  int buf = 0;
  while (key < nkeys) {
    uint32_t kgrab = 0xffffffffu;
    if (tid == 0 && knext < nkeys) kgrab = sched.key(it + 2, work);
    TileInfo nxt;
    nxt.tma = false;
    if (knext < nkeys) {
      nxt = tile_info(offsets, knext, nx, ny, nz, use_tma, POT);
      if (nxt.tma && tid == 0) {
        fence_async_shared();
        mbar_expect_tx(&bar[buf ^ 1], BOX_BYTES);
        issue(fb[buf ^ 1], rb[buf ^ 1], nxt, &bar[buf ^ 1]);
      }
    }
    if (cur.beg != cur.end) {
      float *box = fb[buf];
      float *rbox = rb[buf];
      if (cur.tma) {
        const bool ok = mbar_wait(&bar[buf], buf ? phase1 : phase0);
        if (__syncthreads_or(!ok)) {
          if (stats && tid == 0) atomicExch(stats + 2, 1u);
          if (nxt.tma) mbar_wait(&bar[buf ^ 1], buf ? phase0 : phase1);
          return;
        }
        if (buf) phase1 ^= 1u; else phase0 ^= 1u;
      } else if (POT) {
        for (int q = tid; q < PBOX; q += TILE_THREADS) {
          const int zc = q % PBZ, r = q / PBZ, yc = r % PBY, xc = r / PBY;
          box[q] = __ldg(f3 + cell_index(wrap_index(cur.ox - 2 + xc, nx),
                                         wrap_index(cur.oy - 2 + yc, ny),
                                         wrap_index(cur.oz - 4 + zc, nz), ny, nz));
        }
        for (int q = tid; q < TB * TB * TB; q += TILE_THREADS) {
          const int c = q % TB, r = q / TB, b = r % TB, a = r / TB;
          rbox[(a * TB + b) * TBZ + c] =
              __ldg(rbar + cell_index(wrap_index(cur.ox + a, nx), wrap_index(cur.oy + b, ny),
                                      wrap_index(cur.oz + c, nz), ny, nz));
        }
        __syncthreads();
      } else {
        for (int q = tid; q < 4 * TB * TB * TB; q += TILE_THREADS) {
          const int c = q % TB, r = q / TB, b = r % TB, r2 = r / TB, a = r2 % TB, comp = r2 / TB;
          const int64_t cell = cell_index(wrap_index(cur.ox + a, nx), wrap_index(cur.oy + b, ny),
                                          wrap_index(cur.oz + c, nz), ny, nz);
          const int li = (a * TB + b) * TBZ + c;
          if (comp < 3) box[comp * TBOX + li] = __ldg(f3 + comp * cs + cell);
          else rbox[li] = __ldg(rbar + cell);
        }
        __syncthreads();
      }
      if (POT) {
        force_box_from_potential(box, ff, tid);
        __syncthreads();
        box = ff;
      }
      if (tid == 0) s_grab[buf] = kgrab;
      for (unsigned p = cur.beg + tid; p < cur.end; p += TILE_THREADS) {
        float g[3], u[3], w[3];
        adj_cotangent(gx, gv, dest, p, kick, drift, g, u, w);
        const float x = __ldg(pos + 3 * (int64_t)p), y = __ldg(pos + 3 * (int64_t)p + 1),
                    z = __ldg(pos + 3 * (int64_t)p + 2);
        Axis ax = cic_axis(x, nx), ay = cic_axis(y, ny), az = cic_axis(z, nz);
        AxisGrad dx = cic_axis_grad(x), dy = cic_axis_grad(y), dz = cic_axis_grad(z);
        const int lx = ax.i0 - cur.ox, ly = ay.i0 - cur.oy, lz = az.i0 - cur.oz;
        const bool in = (unsigned)lx < (unsigned)TILE && (unsigned)ly < (unsigned)TILE &&
                        (unsigned)lz < (unsigned)TILE;
        if (!in && stats) atomicAdd(stats + 1, 1u);
        float o0 = 0.f, o1 = 0.f, o2 = 0.f;
#pragma unroll
        for (int n = 0; n < 8; ++n) {
          const float kx = conn_x(n) ? ax.k1 : ax.k0, ky = conn_y(n) ? ay.k1 : ay.k0,
                      kz = conn_z(n) ? az.k1 : az.k0;
          const float ddx = conn_x(n) ? dx.d1 : dx.d0, ddy = conn_y(n) ? dy.d1 : dy.d0,
                      ddz = conn_z(n) ? dz.d1 : dz.d0;
          float v;
          if (in) {
            const int q = ((lx + conn_x(n)) * TB + ly + conn_y(n)) * TBZ + lz + conn_z(n);
            v = rbox[q] + w[0] * box[q] + w[1] * box[TBOX + q] + w[2] * box[2 * TBOX + q];
          } else if (POT) {
            const int ix = conn_x(n) ? ax.i1 : ax.i0, iy = conn_y(n) ? ay.i1 : ay.i0,
                      iz = conn_z(n) ? az.i1 : az.i0;
            v = __ldg(rbar + cell_index(ix, iy, iz, ny, nz)) +
                w[0] * stencil_force_global(f3, ix, iy, iz, 0, nx, ny, nz) +
                w[1] * stencil_force_global(f3, ix, iy, iz, 1, nx, ny, nz) +
                w[2] * stencil_force_global(f3, ix, iy, iz, 2, nx, ny, nz);
          } else {
            const int64_t c = cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                                         conn_z(n) ? az.i1 : az.i0, ny, nz);
            v = __ldg(rbar + c) + w[0] * __ldg(f3 + c) + w[1] * __ldg(f3 + cs + c) +
                w[2] * __ldg(f3 + 2 * cs + c);
          }
          o0 += v * ddx * ky * kz;
          o1 += v * kx * ddy * kz;
          o2 += v * kx * ky * ddz;
        }
        gx_out[3 * (int64_t)p] = g[0] + o0;
        gx_out[3 * (int64_t)p + 1] = g[1] + o1;
        gx_out[3 * (int64_t)p + 2] = g[2] + o2;
        gv_out[3 * (int64_t)p] = u[0];
        gv_out[3 * (int64_t)p + 1] = u[1];
        gv_out[3 * (int64_t)p + 2] = u[2];
      }
    } else if (tid == 0) {
      s_grab[buf] = kgrab;
    }
    __syncthreads();
    const uint32_t kafter = s_grab[buf];  // rewritten two iterations later, after a barrier
    cur = nxt;
    key = knext;
    knext = kafter;
    ++it;
    buf ^= 1;
  }
}

// The cotangents of step i's kick and drift coefficients, one pass over
// the particles of order i (kick: <u, F(x)>, u the velocity cotangent the
// reverse step returned and F the CIC read of the step's force meshes at
// the positions it started from; drift: <g_x', x' - x> = drift <g_x', v'>,
// x' and g_x' the positions the step ended with and their cotangents,
// pulled from order i+1 by dest).  Float64 sums per block, then one double
// atomic per block and quantity.
__global__ void __launch_bounds__(256)
coef_cotangent_kernel(const float *__restrict__ x, const float *__restrict__ xn,
                      const unsigned *__restrict__ dest, const float *__restrict__ f3, int64_t cs,
                      int nx, int ny, int nz, const float *__restrict__ gxn,
                      const float *__restrict__ u, int64_t np, double *__restrict__ out) {
  double gk = 0.0, gd = 0.0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    const float x0 = __ldg(x + 3 * p), x1 = __ldg(x + 3 * p + 1), x2 = __ldg(x + 3 * p + 2);
    Axis ax = cic_axis(x0, nx), ay = cic_axis(x1, ny), az = cic_axis(x2, nz);
    float F0 = 0.f, F1 = 0.f, F2 = 0.f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const float w = __fmul_rn(__fmul_rn(conn_x(n) ? ax.k1 : ax.k0, conn_y(n) ? ay.k1 : ay.k0),
                                conn_z(n) ? az.k1 : az.k0);
      const int64_t c = cell_index(conn_x(n) ? ax.i1 : ax.i0, conn_y(n) ? ay.i1 : ay.i0,
                                   conn_z(n) ? az.i1 : az.i0, ny, nz);
      F0 += __ldg(f3 + c) * w;
      F1 += __ldg(f3 + cs + c) * w;
      F2 += __ldg(f3 + 2 * cs + c) * w;
    }
    gk += (double)__ldg(u + 3 * p) * F0 + (double)__ldg(u + 3 * p + 1) * F1 +
          (double)__ldg(u + 3 * p + 2) * F2;
    const int64_t d = dest ? (int64_t)__ldg(dest + p) : p;
    if (d < np)
      gd += (double)__ldg(gxn + 3 * d) * (__ldg(xn + 3 * d) - x0) +
            (double)__ldg(gxn + 3 * d + 1) * (__ldg(xn + 3 * d + 1) - x1) +
            (double)__ldg(gxn + 3 * d + 2) * (__ldg(xn + 3 * d + 2) - x2);
  }
  for (int o = 16; o > 0; o >>= 1) {
    gk += __shfl_xor_sync(0xffffffffu, gk, o);
    gd += __shfl_xor_sync(0xffffffffu, gd, o);
  }
  __shared__ double part[2][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    part[0][warp] = gk;
    part[1][warp] = gd;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += part[0][w];
      b += part[1][w];
    }
    atomicAdd(out, a);
    atomicAdd(out + 1, b);
  }
}

int coef_cotangents(const float *pos, const float *pos_next, const unsigned *dest,
                    const float *force3, int64_t cs, int nx, int ny, int nz,
                    const float *g_pos_next, const float *g_vel, int64_t np, double *out,
                    cudaStream_t s) {
  if (np == 0) return PMGB_OK;
  coef_cotangent_kernel<<<wave_grid(coef_cotangent_kernel, np, 256), 256, 0, s>>>(
      pos, pos_next, dest, force3, cs, nx, ny, nz, g_pos_next, g_vel, np, out);
  PMGB_LAUNCHED("coef_cotangent_kernel");
  return PMGB_OK;
}

// One reverse step of the sorted loop (see the block comment above).
// pos: the positions the step started from (order i); force3: the force
// meshes the step used, or with `pot` the potential they were derived from
// (the order-1 stencil, as in the run loop); dest: where each particle went
// (order i -> i+1; NULL = identity); offsets: the tile ranges of order i
// (nkeys + 1 entries); (gx_in, gv_in) in order i+1 -> (gx_out, gv_out) in
// order i.
int fpm_step_sorted_vjp(const float *pos, const float *force3, const unsigned *dest,
                        const unsigned *offsets, const float *gx_in, const float *gv_in,
                        float *gx_out, float *gv_out, int64_t np, int nx, int ny, int nz,
                        float kick, float drift, float r_split, void *mesh_ws, size_t mesh_bytes,
                        unsigned *stats, cudaStream_t s, bool pot) {
  float *mesh, *f3w, *g3;
  void *dk, *fk;
  unsigned *work;
  PMGB_TRY(pm_workspace_regions(mesh_ws, mesh_bytes, nx, ny, nz, np, &mesh, &dk, &fk, &f3w, &g3,
                                &work));
  (void)f3w;
  const int64_t ncell = (int64_t)nx * ny * nz;
  const int64_t keys = tile_key_count(nx, ny, nz);
  PMGB_CUDA(cudaMemsetAsync(g3, 0, 3 * ncell * sizeof(float), s));
  if (np == 0) return PMGB_OK;
  const bool aligned = nz % 4 == 0 && ncell % 4 == 0 &&
                       reinterpret_cast<uintptr_t>(g3) % 16 == 0 &&
                       reinterpret_cast<uintptr_t>(force3) % 16 == 0 &&
                       reinterpret_cast<uintptr_t>(mesh) % 16 == 0 && nz >= TBZ && ny >= TB &&
                       nx >= TB;
  const uint64_t dims4[4] = {(uint64_t)nz, (uint64_t)ny, (uint64_t)nx, 3};
  const uint64_t strides4[3] = {(uint64_t)nz * 4, (uint64_t)ny * nz * 4, (uint64_t)ncell * 4};
  const uint32_t box4[4] = {TBZ, TB, TB, 3};
  const uint64_t dims3[3] = {(uint64_t)nz, (uint64_t)ny, (uint64_t)nx};
  const uint32_t box3[3] = {TBZ, TB, TB};
  const uint32_t pbox3[3] = {PBZ, PBY, PBX};
  CUtensorMap gmap, fmap, rmap;
  memset(&gmap, 0, sizeof(gmap));
  memset(&fmap, 0, sizeof(fmap));
  memset(&rmap, 0, sizeof(rmap));
  int use_tma = 0, use_gtma = 0;  // the paint's map; the gather's two maps
  if (aligned) {
    use_tma = make_tensor_map(&gmap, g3, 4, dims4, strides4, box4) == PMGB_OK;
    if (pot)
      use_gtma = nz >= PBZ && ny >= PBY && nx >= PBX &&
                 make_tensor_map(&fmap, force3, 3, dims3, strides4, pbox3) == PMGB_OK;
    else
      use_gtma = make_tensor_map(&fmap, force3, 4, dims4, strides4, box4) == PMGB_OK;
    use_gtma = use_gtma && make_tensor_map(&rmap, mesh, 3, dims3, strides4, box3) == PMGB_OK;
    clear_error();
  }
  static bool ready[64] = {false};
  int dev = 0;
  PMGB_CUDA(cudaGetDevice(&dev));
  if (dev >= 64 || !ready[dev]) {
    PMGB_TRY(set_smem((const void *)adj_paint3_tiles_kernel, ADJ_PAINT_SMEM));
    if (dev < 64) ready[dev] = true;
  }
  // 1. paint of the cotangent-weighted forces
  PMGB_CUDA(cudaMemsetAsync(work, 0, sizeof(unsigned), s));
  const unsigned pgrid = (unsigned)std::min<int64_t>(
      keys, (int64_t)resident_ctas((const void *)adj_paint3_tiles_kernel, ADJ_THREADS,
                                   ADJ_PAINT_SMEM));
  adj_paint3_tiles_kernel<<<pgrid, ADJ_THREADS, ADJ_PAINT_SMEM, s>>>(
      g3, ncell, nx, ny, nz, pos, dest, gx_in, gv_in, kick, drift, offsets, (uint32_t)keys, work,
      stats, aligned ? 1 : 0, gmap, use_tma);
  PMGB_LAUNCHED("adj_paint3_tiles_kernel");
  // 2. rho_bar = sum_c A_c^T (painted component c)
  PMGB_TRY(mesh_forces_vjp(g3, nx, ny, nz, r_split, dk, fk, mesh, s));
  // 3. gather of both position terms and the cotangent update
  const void *gfn = pot ? (const void *)adj_gather_tiles_kernel<true>
                        : (const void *)adj_gather_tiles_kernel<false>;
  const unsigned ggrid =
      (unsigned)std::min<int64_t>(keys, (int64_t)resident_ctas(gfn, TILE_THREADS, 0));
  PMGB_CUDA(cudaMemsetAsync(work + 1, 0, sizeof(unsigned), s));
#define ADJ_GATHER_ARGS                                                                     \
  force3, ncell, mesh, nx, ny, nz, pos, dest, gx_in, gv_in, gx_out, gv_out, kick, drift, \
      offsets, (uint32_t)keys, stats, fmap, rmap, use_gtma, work + 1
  if (pot)
    adj_gather_tiles_kernel<true><<<ggrid, TILE_THREADS, 0, s>>>(ADJ_GATHER_ARGS);
  else
    adj_gather_tiles_kernel<false><<<ggrid, TILE_THREADS, 0, s>>>(ADJ_GATHER_ARGS);
#undef ADJ_GATHER_ARGS
  PMGB_LAUNCHED("adj_gather_tiles_kernel");
  return PMGB_OK;
}

}  // namespace pmgb
