// Shared helpers of libpmgb: status handling, launch geometry and the CIC
// arithmetic that every painter and reader uses.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <climits>
#include <string>

#include "../../include/pmgb.h"

namespace pmgb {

// Records `msg` as the calling thread's last error and returns `code`.
int fail(int code, const std::string &msg);
// Clears the calling thread's last error.
void clear_error();

// Number of SMs of the current device (cached per device).
int sm_count();
// L2 cache bytes of the current device (cached per device).
int64_t l2_bytes();

#define PMGB_CUDA(call)                                                     \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess)                                                  \
      return ::pmgb::fail(PMGB_ERR_CUDA, std::string(#call) + ": " +       \
                                             cudaGetErrorString(e_));       \
  } while (0)

// Counts the kernels this library has launched (every launch site checks
// its launch with PMGB_LAUNCHED, which also counts it).
void count_launch();

#define PMGB_LAUNCHED(name)                                                 \
  do {                                                                      \
    cudaError_t e_ = cudaGetLastError();                                    \
    if (e_ != cudaSuccess)                                                  \
      return ::pmgb::fail(PMGB_ERR_CUDA, std::string(name) + " launch: " + \
                                             cudaGetErrorString(e_));       \
    ::pmgb::count_launch();                                                 \
  } while (0)

#define PMGB_REQUIRE(cond, msg)                                             \
  do {                                                                      \
    if (!(cond)) return ::pmgb::fail(PMGB_ERR_INVALID_ARGUMENT, msg);       \
  } while (0)

#define PMGB_TRY(call)                                                      \
  do {                                                                      \
    int s_ = (call);                                                        \
    if (s_ != PMGB_OK) return s_;                                           \
  } while (0)

// Validates a mesh shape: positive, and small enough that cell indices and
// the float32 cell coordinates stay exact (< 2^24 per axis, < 2^40 cells).
int check_mesh(int nx, int ny, int nz);

// Grid size for a grid-stride loop over n items with `threads` per block:
// enough blocks to fill every SM `per_sm` times, never more than needed.
inline unsigned grid_for(int64_t n, int threads, int per_sm = 8) {
  int64_t need = (n + threads - 1) / threads;
  int64_t cap = (int64_t)sm_count() * per_sm;
  if (need < 1) need = 1;
  return (unsigned)(need < cap ? need : cap);
}

// CTAs of `kernel` resident on the whole device at once (its occupancy at
// `threads` per block and `smem` dynamic shared bytes, times the SM count),
// cached per kernel and device.
int resident_ctas(const void *kernel, int threads, size_t smem);

// Grid of a grid-stride loop over n items whose chunks all cost about the
// same: at most one wave of the kernel's resident CTAs.  A fixed cap of
// 8 CTAs per SM leaves a partial last wave (SMs idle for part of the kernel)
// whenever the kernel's registers allow fewer than 8 per SM.
template <typename K>
inline unsigned wave_grid(K *kernel, int64_t n, int threads, size_t smem = 0) {
  int64_t need = (n + threads - 1) / threads;
  const int64_t cap = resident_ctas(reinterpret_cast<const void *>(kernel), threads, smem);
  if (need < 1) need = 1;
  return (unsigned)(need < cap ? need : cap);
}

// ---------------------------------------------------------------------------
// CIC arithmetic, absolute mode (reference: jaxpm/painting.py:21-37).
// Every operation is rounded separately (no FMA contraction) so that the
// float32 weights equal the reference's bit for bit:
//   c0 = floor(x), c1 = floor(x) + 1 (in float),
//   k0 = 1 - |x - c0|, k1 = 1 - |x - c1|,
//   cell = int32(c) floor-mod n.
// ---------------------------------------------------------------------------

// Floor-modulo i mod n (n > 0); the integer division only runs for indices
// outside [0, n), which unwrapped positions rarely are.
__device__ __forceinline__ int wrap_index(int i, int n) {
  if ((unsigned)i < (unsigned)n) return i;
  int r = i % n;
  return r < 0 ? r + n : r;
}

struct Axis {
  int i0, i1;    // wrapped cells of the lower and upper neighbour
  float k0, k1;  // their CIC factors
};

// The upper neighbour's cell int32(floor(x) + 1) mod n equals
// (i0 + 1) mod n for every position with |x| < 2^24.
__device__ __forceinline__ Axis cic_axis(float x, int n) {
  Axis a;
  float f = floorf(x);
  float c1 = __fadd_rn(f, 1.0f);
  a.k0 = __fsub_rn(1.0f, fabsf(__fsub_rn(x, f)));
  a.k1 = __fsub_rn(1.0f, fabsf(__fsub_rn(x, c1)));
  a.i0 = wrap_index((int)f, n);
  a.i1 = (fabsf(f) < 16777216.0f) ? (a.i0 + 1 == n ? 0 : a.i0 + 1) : wrap_index((int)c1, n);
  return a;
}

// Derivative of each factor w.r.t. x: d(1 - |x - c|)/dx = -1 for x >= c,
// +1 otherwise (JAX's select(u >= 0, g, -g) rule for abs; floor has zero
// derivative).
struct AxisGrad {
  float d0, d1;
};

__device__ __forceinline__ AxisGrad cic_axis_grad(float x) {
  AxisGrad g;
  float f = floorf(x);
  float c1 = __fadd_rn(f, 1.0f);
  g.d0 = (__fsub_rn(x, f) >= 0.0f) ? -1.0f : 1.0f;
  g.d1 = (__fsub_rn(x, c1) >= 0.0f) ? -1.0f : 1.0f;
  return g;
}

// Neighbour n of the reference's connection list (painting.py:24-25):
// (0,0,0),(1,0,0),(0,1,0),(0,0,1),(1,1,0),(1,0,1),(0,1,1),(1,1,1).
__host__ __device__ constexpr int conn_x(int n) {
  return (n == 1 || n == 4 || n == 5 || n == 7) ? 1 : 0;
}
__host__ __device__ constexpr int conn_y(int n) {
  return (n == 2 || n == 4 || n == 6 || n == 7) ? 1 : 0;
}
__host__ __device__ constexpr int conn_z(int n) {
  return (n == 3 || n == 5 || n == 6 || n == 7) ? 1 : 0;
}

__device__ __forceinline__ int64_t cell_index(int ix, int iy, int iz, int ny,
                                              int nz) {
  return ((int64_t)ix * ny + iy) * nz + iz;
}

// Adds wa to row[iz0] and wb to row[iz1] (iz1 the upper z neighbour of iz0,
// wrapped): one 16-byte vector reduction when both cells lie in one aligned
// group of four (3 cases in 4 when `vec` -- rows 16-byte aligned, nz a
// multiple of 4), else two scalar reductions.  The other two lanes of the
// vector add +0.0f, which leaves any value unchanged.  Halves the L2 sector
// operations of a CIC paint, whose z-neighbour pairs are adjacent words.
__device__ __forceinline__ void red_zpair(float *row, int iz0, int iz1, float wa, float wb,
                                         bool vec) {
  const int q = iz0 & 3;
  if (vec && q != 3 && iz1 == iz0 + 1) {
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (q == 0) { v.x = wa; v.y = wb; }
    else if (q == 1) { v.y = wa; v.z = wb; }
    else { v.z = wa; v.w = wb; }
    atomicAdd(reinterpret_cast<float4 *>(row + (iz0 - q)), v);
  } else {
    atomicAdd(row + iz0, wa);
    atomicAdd(row + iz1, wb);
  }
}

// Whether red_zpair may use vector reductions on a mesh at `mesh` with
// rows of nz floats.
inline bool zpair_vec_ok(const void *mesh, int nz) {
  return nz % 4 == 0 && reinterpret_cast<uintptr_t>(mesh) % 16 == 0;
}

// Loads particle p's three coordinates from an [np][3] array.
__device__ __forceinline__ void load3(const float *__restrict__ a, int64_t p,
                                      float &x, float &y, float &z) {
  const float *q = a + 3 * p;
  x = __ldg(q);
  y = __ldg(q + 1);
  z = __ldg(q + 2);
}

}  // namespace pmgb
