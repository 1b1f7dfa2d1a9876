// The spectral part of the PM force (jaxpm/pm.py:30-56: fft3d of the
// density, the k-space kernels, three ifft3d) and of its adjoint, as
// hand-written FFTs in three passes over HBM for power-of-two meshes:
//
//   plane pass (forward): each x-plane [ny][nz] of a real mesh is transformed
//     along z (real-to-complex, nz/2+1 modes) and y.  By default cuFFT's
//     batched 2-D transforms do this (fft.cu); the library's own plane
//     kernels (path 2) use one thread-block cluster of CL CTAs per plane (16
//     for ny >= 256, else 8).  CTA r holds the rows y = r + CL*l
//     (l < M = ny/CL) in shared memory, transforms them along z, then along
//     l (an M-point DFT per column); the last radix-CL step of the y
//     transform reads the CL partial results of every column from the
//     cluster's shared memories (DSMEM) and writes the plane's spectrum
//     [ky][kz] (row pitch `pitch` complex) to HBM.  For nz, ny in {256, 512}
//     the row and column transforms run in registers (plane_*_reg_kernel).
//   x pass: one CTA per (ky, XW consecutive kz) transforms the nx values of
//     each column along x; in the force pipeline it also multiplies by the
//     three force kernels and transforms each product back along x, so the
//     density spectrum and the three force spectra never exist in HBM in
//     full-3-D transformed form.
//   plane pass (inverse): the mirror of the forward plane pass, per
//     component, writing the real force meshes.
//
// Each pass reads and writes its data once: 6.5 GB per force evaluation at
// 512^3 against about 16 GB through cuFFT plus a separate k-space kernel.
//
// The 1-D transforms are in-place radix-8 Cooley-Tukey: forward stages are
// decimation in frequency (natural order in, digit-reversed order out),
// inverse stages decimation in time (digit-reversed in, natural out), so no
// reordering pass is needed between a forward and an inverse transform.
// Twiddles come from float32 tables exp(-2 pi i k / n) computed in double
// precision on the host.  Inverse transforms are unnormalised (as cuFFT's
// and the 1/N^3 of the force pipeline is folded into the k-space multiply).
#include <cooperative_groups.h>

#include <atomic>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <utility>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "kspace.cuh"

namespace cg = cooperative_groups;

namespace pmgb {
namespace {

// Plane passes: planes with ny >= 256 rows go to 16-CTA clusters of 256
// threads (a 512^2 plane's rows in 66 KB of shared memory per CTA, three
// CTAs per SM, so that the load, transform and store phases of different
// clusters overlap); narrower planes to 8-CTA clusters of 512 threads.
constexpr int PLANE_CL = 8;  // the smaller cluster; ny >= PLANE_CL^2
constexpr int PLANE_CL_WIDE = 16;
constexpr int XW = 8;               // kz columns per x-pass CTA (64-byte segments)
constexpr int XPASS_THREADS = 256;

// ---- complex helpers ------------------------------------------------------

__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  return make_float2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  return make_float2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// a * (-i) (forward) or a * (+i) (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_ni(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---- small DFTs: y[k] = sum_m v[m] exp(-+2 pi i m k / R), in place ------------

template <bool INV>
__device__ __forceinline__ void dft2(float2 *v) {
  const float2 a = v[0];
  v[0] = cadd(a, v[1]);
  v[1] = csub(a, v[1]);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2 *v) {
  const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  const float2 t2 = cadd(v[1], v[3]), t3 = mul_ni<INV>(csub(v[1], v[3]));
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}

// radix 2 x 4: u_m = v_m + v_{m+4} feed the even outputs, (v_m - v_{m+4}) w8^m
// the odd ones.
template <bool INV>
__device__ __forceinline__ void dft8(float2 *v) {
  const float r = 0.70710678118654752f;
  float2 u[4], w[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    u[m] = cadd(v[m], v[m + 4]);
    w[m] = csub(v[m], v[m + 4]);
  }
  {
    const float2 d = w[1];
    w[1] = INV ? make_float2(r * (d.x - d.y), r * (d.x + d.y))
               : make_float2(r * (d.x + d.y), r * (d.y - d.x));
  }
  w[2] = mul_ni<INV>(w[2]);
  {
    const float2 d = w[3];
    w[3] = INV ? make_float2(-r * (d.x + d.y), r * (d.x - d.y))
               : make_float2(r * (d.y - d.x), -r * (d.x + d.y));
  }
  dft4<INV>(u);
  dft4<INV>(w);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    v[2 * j] = u[j];
    v[2 * j + 1] = w[j];
  }
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float2 *v) {
  if (R == 8) dft8<INV>(v);
  else if (R == 4) dft4<INV>(v);
  else dft2<INV>(v);
}

// radix 2 x 8: the even and odd inputs' 8-point DFTs E, O, then
// y[k] = E[k] + w16^k O[k], y[k+8] = E[k] - w16^k O[k] (w16 = exp(-+2 pi i / 16)).
template <bool INV>
__device__ __forceinline__ void dft16(float2 *v) {
  constexpr float c1 = 0.92387953251128674f, s1 = 0.38268343236508978f,
                  r = 0.70710678118654752f;
  constexpr float C[8] = {1.f, c1, r, s1, 0.f, -s1, -r, -c1};  // cos(pi k / 8)
  constexpr float S[8] = {0.f, s1, r, c1, 1.f, c1, r, s1};     // sin(pi k / 8)
  float2 e[8], o[8];
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    e[m] = v[2 * m];
    o[m] = v[2 * m + 1];
  }
  dft8<INV>(e);
  dft8<INV>(o);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float2 t = cmul(o[k], make_float2(C[k], INV ? S[k] : -S[k]));
    v[k] = cadd(e[k], t);
    v[k + 8] = csub(e[k], t);
  }
}

template <int CL, bool INV>
__device__ __forceinline__ void dft_cl(float2 *v) {
  if constexpr (CL == 16) dft16<INV>(v);
  else dft8<INV>(v);
}

// ---- in-place radix-8 stages ------------------------------------------------
//
// A transform of length n = 2^lgn runs stages with block length L = 2^lg
// (lg = lgn first), radix R = 2^rb (rb = min(3, lg)) and span S = L / R.
// Forward (DIF) butterfly (block, j < S): elements base + S m, m < R:
// DFT_R, then output k2 times w_L^(j k2).  Inverse (DIT) butterfly: the
// conjugate twiddles first, then the inverse DFT_R; its stages run in the
// opposite order.  The forward transform leaves frequency k at position
// dif_pos(k).

__device__ __forceinline__ int dif_pos(int k, int lgn) {
  int p = 0;
  for (int lg = lgn; lg > 0;) {
    const int rb = lg >= 3 ? 3 : lg, sb = lg - rb;
    p |= (k & ((1 << rb) - 1)) << sb;
    k >>= rb;
    lg = sb;
  }
  return p;
}

__device__ __forceinline__ int dif_freq(int p, int lgn) {
  int k = 0, sh = 0;
  for (int lg = lgn; lg > 0;) {
    const int rb = lg >= 3 ? 3 : lg, sb = lg - rb;
    k |= (p >> sb) << sh;
    p &= (1 << sb) - 1;
    sh += rb;
    lg = sb;
  }
  return k;
}

// One butterfly; `tw` is a table of 2^lgtw entries exp(-2 pi i t / 2^lgtw).
template <bool INV, int R>
__device__ __forceinline__ void butterfly(float2 *base, int sstride, int j, int lg,
                                          const float2 *__restrict__ tw, int lgtw) {
  float2 v[R];
#pragma unroll
  for (int m = 0; m < R; ++m) v[m] = base[m * sstride];
  const int sh = lgtw - lg;
  if (INV) {
#pragma unroll
    for (int m = 1; m < R; ++m) v[m] = cmulc(v[m], __ldg(tw + ((j * m) << sh)));
    dft<R, true>(v);
  } else {
    dft<R, false>(v);
#pragma unroll
    for (int m = 1; m < R; ++m) v[m] = cmul(v[m], __ldg(tw + ((j * m) << sh)));
  }
#pragma unroll
  for (int m = 0; m < R; ++m) base[m * sstride] = v[m];
}

// One stage over `batch` sequences: element e of sequence q at d[q*qs + e*es].
// Threads tid, tid+nth, ... take the butterflies, sequence index fastest.
template <bool INV>
__device__ __forceinline__ void stage(float2 *d, int lgn, int lg, int es, int qs, int batch,
                                      const float2 *__restrict__ tw, int lgtw, int tid,
                                      int nth) {
  const int rb = lg >= 3 ? 3 : lg, sb = lg - rb;
  const int total = batch << (lgn - rb);
  for (int t = tid; t < total; t += nth) {
    const int b = t / batch, q = t - b * batch;
    const int blk = b >> sb, j = b & ((1 << sb) - 1);
    float2 *base = d + q * qs + ((blk << lg) + j) * es;
    if (rb == 3) butterfly<INV, 8>(base, es << sb, j, lg, tw, lgtw);
    else if (rb == 2) butterfly<INV, 4>(base, es << sb, j, lg, tw, lgtw);
    else butterfly<INV, 2>(base, es << sb, j, lg, tw, lgtw);
  }
}

// Whole transforms; SYNC is __syncwarp or __syncthreads between stages.
template <bool CTA>
__device__ __forceinline__ void group_sync() {
  if (CTA) __syncthreads();
  else __syncwarp();
}

template <bool CTA>
__device__ void fft_forward(float2 *d, int lgn, int es, int qs, int batch,
                            const float2 *__restrict__ tw, int lgtw, int tid, int nth) {
  for (int lg = lgn; lg > 0;) {
    stage<false>(d, lgn, lg, es, qs, batch, tw, lgtw, tid, nth);
    group_sync<CTA>();
    lg -= lg >= 3 ? 3 : lg;
  }
}

template <bool CTA>
__device__ void fft_inverse(float2 *d, int lgn, int es, int qs, int batch,
                            const float2 *__restrict__ tw, int lgtw, int tid, int nth) {
  if (lgn == 0) return;
  int lg = lgn % 3 == 0 ? 3 : lgn % 3;
  for (;;) {
    stage<true>(d, lgn, lg, es, qs, batch, tw, lgtw, tid, nth);
    group_sync<CTA>();
    if (lg == lgn) break;
    lg += 3;
  }
}

// ---- real <-> half-complex rows (z axis), one warp per row ---------------------
//
// A real row x[0..nz) is packed as z[m] = x[2m] + i x[2m+1] (H = nz/2
// complex).  After the forward H-point transform (digit-reversed Z), the
// modes X[k], k = 0..H, are E + w^k O and conj(E - w^k O) for the pair
// (k, H-k), E = (Z[k] + conj Z[H-k])/2, O = -i (Z[k] - conj Z[H-k])/2,
// w = exp(-2 pi i / nz).  They are written in natural order (H+1 slots).

constexpr int ROW_PAIRS = (256 / 2 + 1 + 31) / 32;  // pairs per lane for H <= 256

__device__ void row_r2c_finish(float2 *row, int lgh, const float2 *__restrict__ twz, int lane) {
  const int H = 1 << lgh;
  float2 xa[ROW_PAIRS], xb[ROW_PAIRS];
#pragma unroll
  for (int i = 0; i < ROW_PAIRS; ++i) {
    const int j = lane + 32 * i;
    if (j <= H / 2) {
      const float2 a = row[dif_pos(j, lgh)];
      const float2 b = conjf2(row[dif_pos((H - j) & (H - 1), lgh)]);
      const float2 e = cscale(cadd(a, b), 0.5f);
      const float2 o = cscale(mul_ni<false>(csub(a, b)), 0.5f);
      const float2 t = cmul(__ldg(twz + j), o);
      xa[i] = cadd(e, t);
      xb[i] = conjf2(csub(e, t));
    }
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < ROW_PAIRS; ++i) {
    const int j = lane + 32 * i;
    if (j <= H / 2) {
      row[j] = xa[i];
      row[H - j] = xb[i];
    }
  }
  __syncwarp();
}

// Inverse: natural X[0..H] -> packed Z'[k] = P + T, Z'[H-k] = conj(P - T),
// P = X[k] + conj X[H-k], T = i w^-k (X[k] - conj X[H-k]), written at the
// digit-reversed positions the inverse H-point transform expects; the
// imaginary parts of X[0] and X[H] are dropped (a real row's modes 0 and
// nz/2 are real).
__device__ void row_c2r_start(float2 *row, int lgh, const float2 *__restrict__ twz, int lane) {
  const int H = 1 << lgh;
  float2 za[ROW_PAIRS], zb[ROW_PAIRS];
#pragma unroll
  for (int i = 0; i < ROW_PAIRS; ++i) {
    const int j = lane + 32 * i;
    if (j <= H / 2) {
      float2 a = row[j], b = row[H - j];
      if (j == 0) {
        a.y = 0.f;
        b.y = 0.f;
      }
      const float2 p = cadd(a, conjf2(b));
      const float2 q = csub(a, conjf2(b));
      const float2 t = mul_ni<true>(cmulc(q, __ldg(twz + j)));
      za[i] = cadd(p, t);
      zb[i] = conjf2(csub(p, t));
    }
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < ROW_PAIRS; ++i) {
    const int j = lane + 32 * i;
    if (j <= H / 2) {
      row[dif_pos(j, lgh)] = za[i];
      if (j > 0 && j < H / 2) row[dif_pos(H - j, lgh)] = zb[i];
    }
  }
  __syncwarp();
}

// ---- plane passes -------------------------------------------------------------

struct PlaneGeom {
  int ny, nz, lgy, lgz;  // plane size
  int M, lgm;            // rows per CTA (ny / CL)
  int sp;                // shared row pitch (complex), even, >= nz/2 + 1
  int pitch;             // HBM spectrum row pitch (complex), >= nz/2 + 1
};

// Forward: real planes in[plane][ny][nz] -> out[plane][ky][kz] (pitch),
// padding columns kz > nz/2 zeroed.
// Launched in clusters of CL CTAs (a launch attribute), one cluster per plane.
template <int CL, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
plane_r2c_kernel(const float *__restrict__ in, float2 *__restrict__ out, PlaneGeom g,
                 const float2 *__restrict__ twy, const float2 *__restrict__ twz) {
  extern __shared__ __align__(16) float2 sm[];
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int64_t plane = blockIdx.x / CL;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = NT / 32;
  const int lgh = g.lgz - 1, H = 1 << lgh;
  // 1. rows y = r + CL*l: load, H-point forward transform, real finish
  for (int l = warp; l < g.M; l += nwarp) {
    const int y = r + CL * l;
    const float4 *src =
        reinterpret_cast<const float4 *>(in + (plane * g.ny + y) * (int64_t)g.nz);
    float4 *dst = reinterpret_cast<float4 *>(sm + l * g.sp);
    for (int i = lane; i < g.nz / 4; i += 32) dst[i] = __ldg(src + i);
    __syncwarp();
    fft_forward<false>(sm + l * g.sp, lgh, 1, 0, 1, twz, g.lgz, lane, 32);
    row_r2c_finish(sm + l * g.sp, lgh, twz, lane);
  }
  __syncthreads();
  // 2. M-point forward transform along l of the H+1 columns (w_M = w_ny^CL)
  fft_forward<true>(sm, g.lgm, g.sp, 1, H + 1, twy, g.lgy, tid, NT);
  cluster.sync();
  // 3. the last radix-CL step: X[k2 + M k1] = sum_s w_CL^(s k1) w_ny^(s k2) Y_s[k2]
  const int kb = g.M / CL;
  for (int t = tid; t < kb * g.pitch; t += NT) {
    const int kk = t / g.pitch, kz = t - kk * g.pitch;
    const int k2 = r * kb + kk;
    float2 v[CL];
    if (kz <= H) {
      const int row = dif_pos(k2, g.lgm);
#pragma unroll
      for (int s = 0; s < CL; ++s) {
        const float2 *rem = cluster.map_shared_rank(sm, s);
        v[s] = cmul(rem[row * g.sp + kz], __ldg(twy + s * k2));
      }
      dft_cl<CL, false>(v);
    } else {
#pragma unroll
      for (int s = 0; s < CL; ++s) v[s] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k1 = 0; k1 < CL; ++k1)
      out[(plane * g.ny + k2 + g.M * k1) * (int64_t)g.pitch + kz] = v[k1];
  }
  cluster.sync();  // keep this CTA's shared memory alive while others read it
}

// Inverse: in[plane][ky][kz] (pitch) -> real planes out[plane][ny][nz]
// (unnormalised).
template <int CL, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
plane_c2r_kernel(const float2 *__restrict__ in, float *__restrict__ out, PlaneGeom g,
                 const float2 *__restrict__ twy, const float2 *__restrict__ twz) {
  extern __shared__ __align__(16) float2 sm[];
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int64_t plane = blockIdx.x / CL;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = NT / 32;
  const int lgh = g.lgz - 1, H = 1 << lgh;
  cluster.sync();  // every CTA of the cluster runs before any remote store
  // 1. first radix-CL step of the inverse y transform, scattered to the
  //    cluster: V_s[k2] = w_ny^(-s k2) sum_k1 w_CL^(-s k1) X[k2 + M k1]
  const int kb = g.M / CL;
  for (int t = tid; t < kb * (H + 1); t += NT) {
    const int kk = t / (H + 1), kz = t - kk * (H + 1);
    const int k2 = r * kb + kk;
    float2 v[CL];
#pragma unroll
    for (int k1 = 0; k1 < CL; ++k1)
      v[k1] = __ldg(in + (plane * g.ny + k2 + g.M * k1) * (int64_t)g.pitch + kz);
    dft_cl<CL, true>(v);
    const int row = dif_pos(k2, g.lgm);
#pragma unroll
    for (int s = 0; s < CL; ++s) {
      float2 *rem = cluster.map_shared_rank(sm, s);
      rem[row * g.sp + kz] = cmulc(v[s], __ldg(twy + s * k2));
    }
  }
  cluster.sync();
  // 2. inverse M-point transform along the columns -> natural l
  fft_inverse<true>(sm, g.lgm, g.sp, 1, H + 1, twy, g.lgy, tid, NT);
  // 3. rows: half-complex -> packed, inverse H-point transform, store
  for (int l = warp; l < g.M; l += nwarp) {
    const int y = r + CL * l;
    float2 *row = sm + l * g.sp;
    row_c2r_start(row, lgh, twz, lane);
    fft_inverse<false>(row, lgh, 1, 0, 1, twz, g.lgz, lane, 32);
    float4 *dst = reinterpret_cast<float4 *>(out + (plane * g.ny + y) * (int64_t)g.nz);
    const float4 *src = reinterpret_cast<const float4 *>(row);
    for (int i = lane; i < g.nz / 4; i += 32) dst[i] = src[i];
  }
}

// ---- x pass -------------------------------------------------------------------

enum XMode { X_FORWARD = 0, X_INVERSE = 1, X_FORCES = 2, X_FORCES_ADJ = 3, X_POTENTIAL = 4 };

struct XGeom {
  int nx, ny, lgx, nzh, pitch, chunks;
  int64_t cs_in, cs_out;  // component strides (complex elements)
};

// CTA per (ky, chunk of XW columns); buf[x][w].  X_FORWARD: natural x ->
// natural kx (in place allowed).  X_INVERSE: natural kx -> natural x
// (unnormalised).  X_FORCES: forward, then for each force component the
// k-space product and the inverse transform, out + c*cs_out.
// X_FORCES_ADJ: for each component the forward transform of in + c*cs_in,
// the conjugate products summed, then the inverse transform.
template <int MODE>
__global__ void __launch_bounds__(XPASS_THREADS)
xpass_kernel(const float2 *in, float2 *out, XGeom g, const float2 *__restrict__ twx, Tables t,
             float r2, int order, int fd, float scale) {
  extern __shared__ __align__(16) float2 xs[];
  float2 *b0 = xs, *b1 = xs + g.nx * XW;
  const int tid = threadIdx.x;
  const int ky = blockIdx.x / g.chunks, kz0 = (blockIdx.x - ky * g.chunks) * XW;
  const int n = g.nx * XW;
  auto gidx = [&](int x, int w) -> int64_t {
    return ((int64_t)x * g.ny + ky) * g.pitch + kz0 + w;
  };
  if (MODE == X_FORCES_ADJ) {
    for (int c = 0; c < 3; ++c) {
      for (int i = tid; i < n; i += XPASS_THREADS)
        b1[i] = in[c * g.cs_in + gidx(i / XW, i % XW)];
      __syncthreads();
      fft_forward<true>(b1, g.lgx, XW, 1, XW, twx, g.lgx, tid, XPASS_THREADS);
      const AxisEntry Y = t.y[ky];
      for (int i = tid; i < n; i += XPASS_THREADS) {
        const int p = i / XW, w = i % XW, kz = kz0 + w;
        if (kz >= g.nzh) {
          b0[i] = make_float2(0.f, 0.f);
          continue;
        }
        const AxisEntry X = t.x[dif_freq(p, g.lgx)], Z = t.z[kz];
        const float gc = c == 0 ? (order ? X.g1 : X.g0)
                                : (c == 1 ? (order ? Y.g1 : Y.g0) : (order ? Z.g1 : Z.g0));
        const float2 v = b1[i];
        float2 acc = c == 0 ? make_float2(0.f, 0.f) : b0[i];
        acc.x -= gc * v.y;
        acc.y += gc * v.x;
        if (c == 2) {
          Elem el;
          el.X = X;
          el.Y = Y;
          el.Z = Z;
          const float m = inv_laplace(el, fd) * long_range(el, r2) * scale;
          acc = make_float2(acc.x * m, acc.y * m);
        }
        b0[i] = acc;
      }
      __syncthreads();
    }
    fft_inverse<true>(b0, g.lgx, XW, 1, XW, twx, g.lgx, tid, XPASS_THREADS);
    for (int i = tid; i < n; i += XPASS_THREADS) out[gidx(i / XW, i % XW)] = b0[i];
    return;
  }
  // load (X_INVERSE: natural kx into digit-reversed positions)
  for (int i = tid; i < n; i += XPASS_THREADS) {
    const int x = i / XW, w = i % XW;
    const int p = MODE == X_INVERSE ? dif_pos(x, g.lgx) : x;
    b0[p * XW + w] = in[gidx(x, w)];
  }
  __syncthreads();
  if (MODE == X_INVERSE) {
    fft_inverse<true>(b0, g.lgx, XW, 1, XW, twx, g.lgx, tid, XPASS_THREADS);
    for (int i = tid; i < n; i += XPASS_THREADS) out[gidx(i / XW, i % XW)] = b0[i];
    return;
  }
  fft_forward<true>(b0, g.lgx, XW, 1, XW, twx, g.lgx, tid, XPASS_THREADS);
  if (MODE == X_FORWARD) {
    for (int i = tid; i < n; i += XPASS_THREADS) {
      const int kx = i / XW, w = i % XW;
      out[gidx(kx, w)] = b0[dif_pos(kx, g.lgx) * XW + w];
    }
    return;
  }
  if (MODE == X_POTENTIAL) {
    // pot = (delta * invlaplace) * longrange * scale, inverse x transform
    const AxisEntry Y = t.y[ky];
    for (int i = tid; i < n; i += XPASS_THREADS) {
      const int p = i / XW, w = i % XW, kz = kz0 + w;
      float2 pv = make_float2(0.f, 0.f);
      if (kz < g.nzh) {
        Elem el;
        el.X = t.x[dif_freq(p, g.lgx)];
        el.Y = Y;
        el.Z = t.z[kz];
        const float inv = inv_laplace(el, fd), L = long_range(el, r2);
        const float2 d = b0[i];
        pv = make_float2(__fmul_rn(__fmul_rn(d.x, inv), L) * scale,
                         __fmul_rn(__fmul_rn(d.y, inv), L) * scale);
      }
      b1[i] = pv;
    }
    __syncthreads();
    fft_inverse<true>(b1, g.lgx, XW, 1, XW, twx, g.lgx, tid, XPASS_THREADS);
    for (int i = tid; i < n; i += XPASS_THREADS) out[gidx(i / XW, i % XW)] = b1[i];
    return;
  }
  // X_FORCES
  const AxisEntry Y = t.y[ky];
  for (int c = 0; c < 3; ++c) {
    for (int i = tid; i < n; i += XPASS_THREADS) {
      const int p = i / XW, w = i % XW, kz = kz0 + w;
      float2 f[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
      if (kz < g.nzh) {
        Elem el;
        el.X = t.x[dif_freq(p, g.lgx)];
        el.Y = Y;
        el.Z = t.z[kz];
        force_modes(el, b0[i], r2, order, fd, scale, f);
      }
      b1[i] = c == 0 ? f[0] : (c == 1 ? f[1] : f[2]);
    }
    __syncthreads();
    fft_inverse<true>(b1, g.lgx, XW, 1, XW, twx, g.lgx, tid, XPASS_THREADS);
    for (int i = tid; i < n; i += XPASS_THREADS)
      out[c * g.cs_out + gidx(i / XW, i % XW)] = b1[i];
    __syncthreads();
  }
}

// ---- x pass, register-resident transforms (nx = 2^LG, 64 <= nx <= 1024) --------
//
// Each column of nx values is transformed by nx/8 threads holding 8
// elements each; a CTA takes XW columns (w fastest in the thread index, so
// each warp reads and writes 64-byte segments).  A stage's butterfly is
// computed in registers; between stages the values move through a padded
// shared buffer (two buffers used in turn, one barrier per exchange).  The
// first forward stage reads HBM directly, the last inverse stage writes it,
// and the last forward stage and the first inverse stage work on the same
// 8 positions, so the k-space multiply happens in registers.

// float2 of padding per 8 positions: with 8, every exchange pattern of every
// stage reads and writes in the minimum two wavefronts per warp
constexpr int XPAD = 8;

template <int LG>
struct XPlan {
  static constexpr int N = 1 << LG;
  static constexpr int T = N / 8;                   // threads per column
  static constexpr int NS = (LG + 2) / 3;           // stages
  static constexpr int BUF = N * XW + (N / 8) * XPAD;  // one exchange buffer (float2)
};

__device__ __forceinline__ int xaddr(int p, int w) { return p * XW + w + (p >> 3) * XPAD; }

// position of element m of thread b in stage s (block length 2^(LG-3s))
template <int LG, int S_>
__device__ __forceinline__ int xpos(int b, int m) {
  constexpr int lg = LG - 3 * S_;
  if constexpr (lg >= 3) {
    constexpr int sb = lg - 3;
    return ((b >> sb) << lg) + (b & ((1 << sb) - 1)) + (m << sb);
  } else {
    return 8 * b + m;
  }
}

// frequency held at DIF output position p
template <int LG>
__device__ __forceinline__ int xfreq(int p) {
  int k = 0, sh = 0;
#pragma unroll
  for (int lg = LG; lg > 0;) {
    const int rb = lg >= 3 ? 3 : lg, sb = lg - rb;
    k |= (p >> sb) << sh;
    p &= (1 << sb) - 1;
    sh += rb;
    lg = sb;
  }
  return k;
}

// Twiddles of the radix-8 stages with span S > 1, packed per stage as
// [j][m-1] = w_L^(j m) (j < S, m = 1..7) so a thread reads its seven at
// consecutive addresses; xtw_offset(s) is where stage s's table starts.
template <int LG>
__host__ __device__ constexpr int xtw_offset(int s) {
  int off = 0;
  for (int q = 0; q < s; ++q) {
    const int lg = LG - 3 * q;
    if (lg >= 4) off += 7 << (lg - 3);
  }
  return off;
}

template <int LG, int S_ = 0>
__device__ __forceinline__ void xload_twiddles(float2 *tw, const float2 *__restrict__ twx,
                                               int tid, int nth) {
  constexpr int lg = LG - 3 * S_;
  if constexpr (lg >= 4) {
    constexpr int S = 1 << (lg - 3), sh = LG - lg, off = xtw_offset<LG>(S_);
    for (int i = tid; i < 7 * S; i += nth) {
      const int j = i / 7, m = i - 7 * j + 1;
      tw[off + i] = __ldg(twx + ((j * m) << sh));
    }
    xload_twiddles<LG, S_ + 1>(tw, twx, tid, nth);
  }
}

template <int LG, int S_, bool INV>
__device__ __forceinline__ void xstage(float2 *v, int b, const float2 *tw) {
  constexpr int lg = LG - 3 * S_;
  if constexpr (lg >= 3) {
    constexpr int sb = lg - 3;
    if constexpr (sb > 0) {
      const int j = b & ((1 << sb) - 1);
      const float2 *tj = tw + xtw_offset<LG>(S_) + 7 * j;
      if (INV) {
#pragma unroll
        for (int m = 1; m < 8; ++m) v[m] = cmulc(v[m], tj[m - 1]);
        dft8<true>(v);
      } else {
        dft8<false>(v);
#pragma unroll
        for (int m = 1; m < 8; ++m) v[m] = cmul(v[m], tj[m - 1]);
      }
    } else {
      dft8<INV>(v);
    }
  } else if constexpr (lg == 2) {
    dft4<INV>(v);
    dft4<INV>(v + 4);
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) dft2<INV>(v + 2 * q);
  }
}

// Exchange addresses of stage S_: element m of thread b sits at
// xaddr(base + m*S) = xaddr(base) + m*S*XW + ((m*S) >> 3)*XPAD, base =
// xpos(b, 0): the low three bits of base plus (m*S mod 8) never carry
// (base's low bits are j < S when S < 8, zero otherwise), so the per-m part
// is a compile-time offset.
template <int LG, int S_>
__device__ __forceinline__ int xbase(int b, int w) {
  return xaddr(xpos<LG, S_>(b, 0), w);
}

template <int LG, int S_>
__device__ __forceinline__ constexpr int xoff(int m) {
  constexpr int lg = LG - 3 * S_;
  constexpr int S = lg >= 3 ? 1 << (lg - 3) : 1;
  return m * S * XW + ((m * S) >> 3) * XPAD;
}

// write the values at stage A's positions, read them at stage B's
template <int LG, int SA, int SB>
__device__ __forceinline__ void xexchange(float2 *v, int b, int w, float2 *buf) {
  float2 *pa = buf + xbase<LG, SA>(b, w);
#pragma unroll
  for (int m = 0; m < 8; ++m) pa[xoff<LG, SA>(m)] = v[m];
  __syncthreads();
  const float2 *pb = buf + xbase<LG, SB>(b, w);
#pragma unroll
  for (int m = 0; m < 8; ++m) v[m] = pb[xoff<LG, SB>(m)];
}

// Forward transform from natural order (v at stage-0 positions) to the last
// stage's positions; `flip` tracks which exchange buffer is next.
template <int LG, int S_ = 0>
__device__ __forceinline__ void xforward(float2 *v, int b, int w, const float2 *tw, float2 *buf0,
                                         float2 *buf1, int &flip) {
  xstage<LG, S_, false>(v, b, tw);
  if constexpr (S_ + 1 < XPlan<LG>::NS) {
    xexchange<LG, S_, S_ + 1>(v, b, w, flip ? buf1 : buf0);
    flip ^= 1;
    xforward<LG, S_ + 1>(v, b, w, tw, buf0, buf1, flip);
  }
}

// Inverse transform from the last stage's positions to natural order.
template <int LG, int S_ = XPlan<LG>::NS - 1>
__device__ __forceinline__ void xinverse(float2 *v, int b, int w, const float2 *tw, float2 *buf0,
                                         float2 *buf1, int &flip) {
  xstage<LG, S_, true>(v, b, tw);
  if constexpr (S_ > 0) {
    xexchange<LG, S_, S_ - 1>(v, b, w, flip ? buf1 : buf0);
    flip ^= 1;
    xinverse<LG, S_ - 1>(v, b, w, tw, buf0, buf1, flip);
  }
}

template <int LG, int MODE>
__global__ void __launch_bounds__(XPlan<LG>::T * XW, 1024 / (XPlan<LG>::T * XW))
xpass_reg_kernel(const float2 *in, float2 *out, XGeom g, const float2 *__restrict__ twx,
                 Tables t, float r2, int order, int fd, float scale) {
  using PL = XPlan<LG>;
  constexpr int N = PL::N, T = PL::T, NS = PL::NS;
  extern __shared__ __align__(16) float2 xsm[];
  float2 *tw = xsm;  // per-stage twiddle tables (xtw_offset), fewer than N entries
  float2 *buf0 = xsm + N, *buf1 = buf0 + PL::BUF;
  float2 *xk = buf1 + PL::BUF;  // per kx: (k2 or fd k2, gradient factor) for the k-space modes
  const int tid = threadIdx.x, w = tid % XW, b = tid / XW;
  const int ky = blockIdx.x / g.chunks, kz0 = (blockIdx.x - ky * g.chunks) * XW;
  const int kz = kz0 + w;
  xload_twiddles<LG>(tw, twx, tid, T * XW);
  if (MODE == X_FORCES || MODE == X_FORCES_ADJ || MODE == X_POTENTIAL) {
    for (int i = tid; i < N; i += T * XW) {
      const AxisEntry X = t.x[i];
      xk[i] = make_float2(fd ? X.fdk2 : X.k2, order ? X.g1 : X.g0);
    }
  }
  __syncthreads();
  auto gidx = [&](int x) -> int64_t { return ((int64_t)x * g.ny + ky) * g.pitch + kz; };
  int flip = 0;
  float2 v[8];
  if (MODE == X_FORWARD || MODE == X_FORCES || MODE == X_POTENTIAL) {
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = in[gidx(b + T * m)];
    xforward<LG>(v, b, w, tw, buf0, buf1, flip);
  }
  if (MODE == X_FORWARD) {
#pragma unroll
    for (int m = 0; m < 8; ++m) out[gidx(xfreq<LG>(xpos<LG, NS - 1>(b, m)))] = v[m];
    return;
  }
  if (MODE == X_INVERSE) {
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = in[gidx(xfreq<LG>(xpos<LG, NS - 1>(b, m)))];
    xinverse<LG>(v, b, w, tw, buf0, buf1, flip);
#pragma unroll
    for (int m = 0; m < 8; ++m) out[gidx(b + T * m)] = v[m];
    return;
  }
  const bool live = kz < g.nzh;
  const AxisEntry Y = t.y[ky];
  const AxisEntry Z = t.z[live ? kz : 0];
  const float yk2 = fd ? Y.fdk2 : Y.k2, zk2 = fd ? Z.fdk2 : Z.k2;
  const float gy = order ? Y.g1 : Y.g0, gz = order ? Z.g1 : Z.g0;
  // per element: the inverse Laplacian times the long-range factor, as in
  // inv_laplace / long_range (kk = ((kx^2 + ky^2) + kz^2); r2 uses k^2)
  auto kfactor = [&](int kx, float &inv, float &L) {
    const float2 xe = xk[kx];
    const float kk = __fadd_rn(__fadd_rn(xe.x, yk2), zk2);
    inv = kk == 0.0f ? 0.0f : -__frcp_rn(kk);
    L = 1.0f;
    if (r2 != 0.0f) {
      const float k2 = fd ? __fadd_rn(__fadd_rn(t.x[kx].k2, Y.k2), Z.k2) : kk;
      L = expf(-k2 * r2);
    }
  };
  if (MODE == X_POTENTIAL) {
    // pot = (delta * invlaplace) * longrange * scale, one inverse transform
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int kx = xfreq<LG>(xpos<LG, NS - 1>(b, m));
      float inv, L;
      kfactor(kx, inv, L);
      v[m] = live ? make_float2(__fmul_rn(__fmul_rn(v[m].x, inv), L) * scale,
                                __fmul_rn(__fmul_rn(v[m].y, inv), L) * scale)
                  : make_float2(0.f, 0.f);
    }
    xinverse<LG>(v, b, w, tw, buf0, buf1, flip);
#pragma unroll
    for (int m = 0; m < 8; ++m) out[gidx(b + T * m)] = v[m];
    return;
  }
  if (MODE == X_FORCES) {
    // pot = (delta * invlaplace) * longrange.  F_c = -(i g_c) pot: the x
    // component needs its own inverse x transform; g_y and g_z are constant
    // along x, so F_y and F_z are -(i g_y) and -(i g_z) times one inverse
    // transform of pot.  pot is kept (times the normalisation) in v after
    // the x component is written.
    float2 pot[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int kx = xfreq<LG>(xpos<LG, NS - 1>(b, m));
      float inv, L;
      kfactor(kx, inv, L);
      pot[m] = make_float2(__fmul_rn(__fmul_rn(v[m].x, inv), L),
                           __fmul_rn(__fmul_rn(v[m].y, inv), L));
      if (!live) pot[m] = make_float2(0.f, 0.f);
      const float gc = xk[kx].y;
      // -(i g) * (px + i py) = g*py - i g*px
      v[m] = make_float2(__fmul_rn(gc, pot[m].y) * scale, -__fmul_rn(gc, pot[m].x) * scale);
    }
    xinverse<LG>(v, b, w, tw, buf0, buf1, flip);
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      out[gidx(b + T * m)] = v[m];
      v[m] = make_float2(pot[m].x * scale, pot[m].y * scale);
    }
    xinverse<LG>(v, b, w, tw, buf0, buf1, flip);
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      out[g.cs_out + gidx(b + T * m)] = make_float2(gy * v[m].y, -gy * v[m].x);
      out[2 * g.cs_out + gidx(b + T * m)] = make_float2(gz * v[m].y, -gz * v[m].x);
    }
    return;
  }
  // X_FORCES_ADJ: acc = sum_c (i g_c) V_c, then times invlaplace * longrange
  // * scale.  g_y and g_z are constant along x, so the y and z cotangents
  // are combined before one forward transform: (i g_y) V_y + (i g_z) V_z =
  // FFT_x((i g_y) G_y + (i g_z) G_z).
  float2 acc[8];
#pragma unroll
  for (int m = 0; m < 8; ++m) v[m] = in[gidx(b + T * m)];
  xforward<LG>(v, b, w, tw, buf0, buf1, flip);
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const float gc = xk[xfreq<LG>(xpos<LG, NS - 1>(b, m))].y;
    acc[m] = make_float2(-gc * v[m].y, gc * v[m].x);
  }
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const float2 a = in[g.cs_in + gidx(b + T * m)], c = in[2 * g.cs_in + gidx(b + T * m)];
    // (i g_y) a + (i g_z) c
    v[m] = make_float2(-(gy * a.y + gz * c.y), gy * a.x + gz * c.x);
  }
  xforward<LG>(v, b, w, tw, buf0, buf1, flip);
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const int kx = xfreq<LG>(xpos<LG, NS - 1>(b, m));
    float inv, L;
    kfactor(kx, inv, L);
    const float mm = inv * L * scale;
    const float ax = acc[m].x + v[m].x, ay = acc[m].y + v[m].y;
    v[m] = live ? make_float2(ax * mm, ay * mm) : make_float2(0.f, 0.f);
  }
  xinverse<LG>(v, b, w, tw, buf0, buf1, flip);
#pragma unroll
  for (int m = 0; m < 8; ++m) out[gidx(b + T * m)] = v[m];
}

// ---- register-resident plane passes (16-CTA clusters; nz, ny in {256, 512}) ----
//
// The decomposition of plane_r2c_kernel / plane_c2r_kernel (CTA r of a
// 16-CTA cluster holds the rows y = r + 16 l, l < M = ny/16), with the
// transforms in registers: the CTA's rows are copied into shared memory at
// once (cp.async, every copy in flight together), each group of 8 rows is
// transformed along z by the x pass's register machinery (xforward /
// xinverse: 8 elements per thread, radix-8 stages, padded exchanges), and
// each column's M-point transform along l runs in one thread's registers.
// Columns and rows stay in natural order, so the cluster step indexes row k2
// directly.

constexpr int PREG_THREADS = 256;

// w32^e = exp(-2 pi i e / 32): cos and sin of pi e / 16, e < 22
__device__ __constant__ float C32[22] = {
    1.f, 0.98078528040323043f, 0.92387953251128674f, 0.83146961230254524f,
    0.70710678118654752f, 0.55557023301960218f, 0.38268343236508978f, 0.19509032201612825f,
    0.f, -0.19509032201612825f, -0.38268343236508978f, -0.55557023301960218f,
    -0.70710678118654752f, -0.83146961230254524f, -0.92387953251128674f, -0.98078528040323043f,
    -1.f, -0.98078528040323043f, -0.92387953251128674f, -0.83146961230254524f,
    -0.70710678118654752f, -0.55557023301960218f};
__device__ __constant__ float S32[22] = {
    0.f, 0.19509032201612825f, 0.38268343236508978f, 0.55557023301960218f,
    0.70710678118654752f, 0.83146961230254524f, 0.92387953251128674f, 0.98078528040323043f,
    1.f, 0.98078528040323043f, 0.92387953251128674f, 0.83146961230254524f,
    0.70710678118654752f, 0.55557023301960218f, 0.38268343236508978f, 0.19509032201612825f,
    0.f, -0.19509032201612825f, -0.38268343236508978f, -0.55557023301960218f,
    -0.70710678118654752f, -0.83146961230254524f};

// 32-point DFT in place, radix 4 x 8: x[8a + b] -> DFT4 over a for each b,
// times w32^(b c), then DFT8 over b for each c.  Slot 8c + d ends holding
// X[c + 4d] (col_slot_freq).
template <bool INV>
__device__ __forceinline__ void dft32(float2 *v) {
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    float2 t[4] = {v[b], v[8 + b], v[16 + b], v[24 + b]};
    dft4<INV>(t);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int e = b * c;
      v[8 * c + b] =
          e == 0 ? t[c] : cmul(t[c], make_float2(C32[e], INV ? S32[e] : -S32[e]));
    }
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) dft8<INV>(v + 8 * c);
}

// the M-point column transform (natural order in) and the frequency its
// slot s holds afterwards
template <int M, bool INV>
__device__ __forceinline__ void dft_col(float2 *v) {
  if constexpr (M == 32) dft32<INV>(v);
  else dft16<INV>(v);
}
template <int M>
__device__ __forceinline__ constexpr int col_slot_freq(int s) {
  return M == 32 ? (s >> 3) + 4 * (s & 7) : s;
}

template <int LGH, int M>
struct PregPlan {
  using PL = XPlan<LGH>;
  static constexpr int H = 1 << LGH;
  static constexpr int GPR = PREG_THREADS / (PL::T * XW);  // row groups per pass
  static constexpr int PASSES = M / (8 * GPR);
  static constexpr int TW = xtw_offset<LGH>(PL::NS);  // packed row twiddles
  static constexpr int XBUF = 2 * GPR * PL::BUF;
};

template <int LGH, int M>
size_t preg_smem(int sp) {
  using P = PregPlan<LGH, M>;
  return ((size_t)M * sp + P::XBUF + P::TW) * sizeof(float2);
}

// cp.async of the CTA's M rows (nz floats each) into rows[l * sp]
template <int LGH, int M>
__device__ __forceinline__ void preg_load_rows(const float *in, float2 *rows, int64_t row0,
                                               int ny_stride, int sp, int tid) {
  constexpr int PER_ROW = (2 << LGH) / 4;  // 16-byte pieces per row
  const uint32_t base = static_cast<uint32_t>(__cvta_generic_to_shared(rows));
  for (int i = tid; i < M * PER_ROW; i += PREG_THREADS) {
    const int l = i / PER_ROW, c = i - l * PER_ROW;
    const float *src = in + (row0 + (int64_t)ny_stride * l) * (2 << LGH) + 4 * c;
    const uint32_t dst = base + (uint32_t)(l * sp * (int)sizeof(float2) + 16 * c);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

template <int LGH, int M>
__global__ void __launch_bounds__(PREG_THREADS, 2)
plane_r2c_reg_kernel(const float *__restrict__ in, float2 *__restrict__ out, PlaneGeom g,
                     const float2 *__restrict__ twh, const float2 *__restrict__ twy,
                     const float2 *__restrict__ twz) {
  using P = PregPlan<LGH, M>;
  using PL = typename P::PL;
  constexpr int H = P::H, T = PL::T, NS = PL::NS, CL = PLANE_CL_WIDE, KB = M / CL;
  extern __shared__ __align__(16) float2 sm[];
  float2 *rows = sm;
  float2 *xbuf = rows + M * g.sp;
  float2 *tw = xbuf + P::XBUF;
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int64_t plane = blockIdx.x / CL;
  const int tid = threadIdx.x;
  preg_load_rows<LGH, M>(in, rows, plane * g.ny + r, CL, g.sp, tid);
  xload_twiddles<LGH>(tw, twh, tid, PREG_THREADS);
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncthreads();
  // 1. rows, 8 per group: the H-point forward transform of the packed row
  //    z[p] = x[2p] + i x[2p+1], written back in natural frequency order
  const int grp = tid / (T * XW), gt = tid - grp * (T * XW), w = gt % XW, b = gt / XW;
  float2 *buf0 = xbuf + 2 * grp * PL::BUF, *buf1 = buf0 + PL::BUF;
  int flip = 0;
  for (int q = 0; q < P::PASSES; ++q) {
    float2 *row = rows + ((q * P::GPR + grp) * 8 + w) * g.sp;
    float2 v[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = row[b + T * m];
    xforward<LGH>(v, b, w, tw, buf0, buf1, flip);  // every read of row precedes its barriers
#pragma unroll
    for (int m = 0; m < 8; ++m) row[xfreq<LGH>(xpos<LGH, NS - 1>(b, m))] = v[m];
  }
  __syncthreads();
  // real finish in place, one thread per mode pair (j, H - j): X[j] = E + w^j O,
  // X[H-j] = conj(E - w^j O) (as row_r2c_finish)
  for (int i = tid; i < M * (H / 2 + 1); i += PREG_THREADS) {
    const int l = i / (H / 2 + 1), j = i - l * (H / 2 + 1);
    float2 *row = rows + l * g.sp;
    const float2 a = row[j];
    const float2 c = conjf2(row[(H - j) & (H - 1)]);
    const float2 e = cscale(cadd(a, c), 0.5f);
    const float2 o = cscale(mul_ni<false>(csub(a, c)), 0.5f);
    const float2 t = cmul(__ldg(twz + j), o);
    row[j] = cadd(e, t);
    row[H - j] = conjf2(csub(e, t));
  }
  __syncthreads();
  // 2. columns: the M-point forward transform along l of each of the H + 1
  //    columns in one thread's registers
  for (int kz = tid; kz <= H; kz += PREG_THREADS) {
    float2 v[M];
#pragma unroll
    for (int l = 0; l < M; ++l) v[l] = rows[l * g.sp + kz];
    dft_col<M, false>(v);
#pragma unroll
    for (int s = 0; s < M; ++s) rows[col_slot_freq<M>(s) * g.sp + kz] = v[s];
  }
  cluster.sync();
  // 3. the last radix-16 step: X[k2 + M k1] = sum_s w16^(s k1) w_ny^(s k2) Y_s[k2]
  for (int t = tid; t < KB * g.pitch; t += PREG_THREADS) {
    const int kk = t / g.pitch, kz = t - kk * g.pitch;
    const int k2 = r * KB + kk;
    float2 v[CL];
    if (kz <= H) {
#pragma unroll
      for (int s = 0; s < CL; ++s) {
        const float2 *rem = cluster.map_shared_rank(rows, s);
        v[s] = cmul(rem[k2 * g.sp + kz], __ldg(twy + s * k2));
      }
      dft16<false>(v);
    } else {
#pragma unroll
      for (int s = 0; s < CL; ++s) v[s] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k1 = 0; k1 < CL; ++k1)
      out[(plane * g.ny + k2 + M * k1) * (int64_t)g.pitch + kz] = v[k1];
  }
  cluster.sync();  // keep this CTA's shared memory alive while others read it
}

template <int LGH, int M>
__global__ void __launch_bounds__(PREG_THREADS, 2)
plane_c2r_reg_kernel(const float2 *__restrict__ in, float *__restrict__ out, PlaneGeom g,
                     const float2 *__restrict__ twh, const float2 *__restrict__ twy,
                     const float2 *__restrict__ twz) {
  using P = PregPlan<LGH, M>;
  using PL = typename P::PL;
  constexpr int H = P::H, T = PL::T, NS = PL::NS, CL = PLANE_CL_WIDE, KB = M / CL;
  extern __shared__ __align__(16) float2 sm[];
  float2 *rows = sm;
  float2 *xbuf = rows + M * g.sp;
  float2 *tw = xbuf + P::XBUF;
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int64_t plane = blockIdx.x / CL;
  const int tid = threadIdx.x;
  xload_twiddles<LGH>(tw, twh, tid, PREG_THREADS);
  cluster.sync();  // every CTA of the cluster runs before any remote store
  // 1. first radix-16 step of the inverse y transform, scattered to the
  //    cluster: V_s[k2] = w_ny^(-s k2) sum_k1 w16^(-s k1) X[k2 + M k1]
  for (int t = tid; t < KB * (H + 1); t += PREG_THREADS) {
    const int kk = t / (H + 1), kz = t - kk * (H + 1);
    const int k2 = r * KB + kk;
    float2 v[CL];
#pragma unroll
    for (int k1 = 0; k1 < CL; ++k1)
      v[k1] = __ldg(in + (plane * g.ny + k2 + M * k1) * (int64_t)g.pitch + kz);
    dft16<true>(v);
#pragma unroll
    for (int s = 0; s < CL; ++s) {
      float2 *rem = cluster.map_shared_rank(rows, s);
      rem[k2 * g.sp + kz] = cmulc(v[s], __ldg(twy + s * k2));
    }
  }
  cluster.sync();
  // 2. columns: the inverse M-point transform, natural k in, natural l out
  for (int kz = tid; kz <= H; kz += PREG_THREADS) {
    float2 v[M];
#pragma unroll
    for (int k = 0; k < M; ++k) v[k] = rows[k * g.sp + kz];
    dft_col<M, true>(v);
#pragma unroll
    for (int s = 0; s < M; ++s) rows[col_slot_freq<M>(s) * g.sp + kz] = v[s];
  }
  __syncthreads();
  // 3. rows: half-complex -> packed in place, one thread per mode pair (as
  //    row_c2r_start, natural order), then the H-point inverse transform of
  //    8 rows per group and the real rows to HBM
  for (int i = tid; i < M * (H / 2 + 1); i += PREG_THREADS) {
    const int l = i / (H / 2 + 1), j = i - l * (H / 2 + 1);
    float2 *row = rows + l * g.sp;
    float2 a = row[j], c = row[H - j];
    if (j == 0) {
      a.y = 0.f;
      c.y = 0.f;
    }
    const float2 p = cadd(a, conjf2(c));
    const float2 d = csub(a, conjf2(c));
    const float2 t = mul_ni<true>(cmulc(d, __ldg(twz + j)));
    row[j] = cadd(p, t);
    if (j > 0 && j < H / 2) row[H - j] = conjf2(csub(p, t));
  }
  __syncthreads();
  const int grp = tid / (T * XW), gt = tid - grp * (T * XW), w = gt % XW, b = gt / XW;
  float2 *buf0 = xbuf + 2 * grp * PL::BUF, *buf1 = buf0 + PL::BUF;
  int flip = 0;
  for (int q = 0; q < P::PASSES; ++q) {
    const int l = (q * P::GPR + grp) * 8 + w;
    const float2 *row = rows + l * g.sp;
    float2 v[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = row[xfreq<LGH>(xpos<LGH, NS - 1>(b, m))];
    xinverse<LGH>(v, b, w, tw, buf0, buf1, flip);
    float2 *dst =
        reinterpret_cast<float2 *>(out + (plane * g.ny + r + CL * l) * (int64_t)(2 * H));
#pragma unroll
    for (int m = 0; m < 8; ++m) dst[b + T * m] = v[m];
  }
}

// ---- host side ----------------------------------------------------------------

std::mutex g_tw_mu;
std::map<std::pair<int, int>, float2 *> g_twiddles;

// exp(-2 pi i k / n), k < n, per (device, n).
int twiddles(int n, const float2 **out) {
  int dev = 0;
  PMGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_tw_mu);
  auto key = std::make_pair(dev, n);
  auto it = g_twiddles.find(key);
  if (it != g_twiddles.end()) {
    *out = it->second;
    return PMGB_OK;
  }
  std::vector<float2> h(n);
  for (int k = 0; k < n; ++k) {
    const double a = -2.0 * M_PI * (double)k / (double)n;
    h[k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  float2 *d = nullptr;
  PMGB_CUDA(cudaMalloc(&d, n * sizeof(float2)));
  cudaError_t err = cudaMemcpy(d, h.data(), n * sizeof(float2), cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    cudaFree(d);
    return fail(PMGB_ERR_CUDA, std::string("twiddle upload: ") + cudaGetErrorString(err));
  }
  g_twiddles[key] = d;
  *out = d;
  return PMGB_OK;
}

int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

PlaneGeom plane_geom(int ny, int nz, int pitch, int cl) {
  PlaneGeom g;
  g.ny = ny;
  g.nz = nz;
  g.lgy = ilog2(ny);
  g.lgz = ilog2(nz);
  g.M = ny / cl;
  g.lgm = ilog2(g.M);
  g.sp = (nz / 2 + 2) & ~1;
  g.pitch = pitch;
  return g;
}

size_t plane_smem(const PlaneGeom &g) { return (size_t)g.M * g.sp * sizeof(float2); }

int set_dyn_smem(const void *fn, size_t bytes) {
  PMGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return PMGB_OK;
}

// One cluster of CL CTAs per plane (cluster size as a launch attribute; 16
// is above the portable 8 and needs the function's opt-in).
template <typename Fn, typename... Args>
int launch_planes(Fn fn, int cl, int nt, int nplanes, size_t smem, cudaStream_t s,
                  Args... args) {
  PMGB_TRY(set_dyn_smem((const void *)fn, smem));
  if (cl > 8)
    PMGB_CUDA(cudaFuncSetAttribute((const void *)fn,
                                   cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)nplanes * cl);
  cfg.blockDim = dim3(nt);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  PMGB_CUDA(cudaLaunchKernelEx(&cfg, fn, args...));
  return PMGB_OK;
}

// Whether 16-CTA clusters of `fn` (nt threads, smem bytes of dynamic shared
// memory) can be resident on this device; queried once per (device, kernel,
// smem).  Where they cannot, the 8-CTA kernels run.
bool clusters_fit(const void *fn, int nt, size_t smem) {
  static std::mutex mu;
  static std::map<std::tuple<int, const void *, size_t>, bool> known;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_tuple(dev, fn, smem);
  auto it = known.find(key);
  if (it != known.end()) return it->second;
  int n = 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(PLANE_CL_WIDE);
  cfg.blockDim = dim3(nt);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = PLANE_CL_WIDE;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const bool ok =
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
          cudaSuccess &&
      cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
          cudaSuccess &&
      cudaOccupancyMaxActiveClusters(&n, fn, &cfg) == cudaSuccess && n >= 1;
  cudaGetLastError();  // a refused query leaves no sticky error behind
  known[key] = ok;
  return ok;
}

// The register-resident kernels' shapes: nz and ny each 256 or 512.
template <bool FWD, int LGH, int M>
const void *preg_fn() {
  return FWD ? (const void *)plane_r2c_reg_kernel<LGH, M>
             : (const void *)plane_c2r_reg_kernel<LGH, M>;
}

template <bool FWD, int LGH, int M>
int preg_try(const void *in, void *out, int nplanes, int ny, int nz, int pitch, cudaStream_t s,
             bool *done) {
  const PlaneGeom g = plane_geom(ny, nz, pitch, PLANE_CL_WIDE);
  const size_t smem = preg_smem<LGH, M>(g.sp);
  *done = false;
  if (!clusters_fit(preg_fn<FWD, LGH, M>(), PREG_THREADS, smem)) return PMGB_OK;
  const float2 *twh, *twy, *twz;
  PMGB_TRY(twiddles(1 << LGH, &twh));
  PMGB_TRY(twiddles(ny, &twy));
  PMGB_TRY(twiddles(nz, &twz));
  if (FWD)
    PMGB_TRY(launch_planes(plane_r2c_reg_kernel<LGH, M>, PLANE_CL_WIDE, PREG_THREADS, nplanes,
                           smem, s, static_cast<const float *>(in), static_cast<float2 *>(out),
                           g, twh, twy, twz));
  else
    PMGB_TRY(launch_planes(plane_c2r_reg_kernel<LGH, M>, PLANE_CL_WIDE, PREG_THREADS, nplanes,
                           smem, s, static_cast<const float2 *>(in), static_cast<float *>(out),
                           g, twh, twy, twz));
  *done = true;
  return PMGB_OK;
}

template <bool FWD>
int preg_dispatch(const void *in, void *out, int nplanes, int ny, int nz, int pitch,
                  cudaStream_t s, bool *done) {
  *done = false;
  if (nz == 512 && ny == 512) return preg_try<FWD, 8, 32>(in, out, nplanes, ny, nz, pitch, s, done);
  if (nz == 512 && ny == 256) return preg_try<FWD, 8, 16>(in, out, nplanes, ny, nz, pitch, s, done);
  if (nz == 256 && ny == 512) return preg_try<FWD, 7, 32>(in, out, nplanes, ny, nz, pitch, s, done);
  if (nz == 256 && ny == 256) return preg_try<FWD, 7, 16>(in, out, nplanes, ny, nz, pitch, s, done);
  return PMGB_OK;
}

int plane_r2c(const float *in, float2 *out, int nplanes, int ny, int nz, int pitch,
              cudaStream_t s) {
  bool done = false;
  PMGB_TRY(preg_dispatch<true>(in, out, nplanes, ny, nz, pitch, s, &done));
  if (done) {
    PMGB_LAUNCHED("plane_r2c_reg_kernel");
    return PMGB_OK;
  }
  bool wide = ny >= PLANE_CL_WIDE * PLANE_CL_WIDE;
  const PlaneGeom g = plane_geom(ny, nz, pitch, wide ? PLANE_CL_WIDE : PLANE_CL);
  const size_t smem = plane_smem(g);
  wide = wide && clusters_fit((const void *)plane_r2c_kernel<PLANE_CL_WIDE, 256, 3>, 256, smem);
  const PlaneGeom g8 = wide ? g : plane_geom(ny, nz, pitch, PLANE_CL);
  const float2 *twy, *twz;
  PMGB_TRY(twiddles(ny, &twy));
  PMGB_TRY(twiddles(nz, &twz));
  if (wide)
    PMGB_TRY(launch_planes(plane_r2c_kernel<PLANE_CL_WIDE, 256, 3>, PLANE_CL_WIDE, 256, nplanes,
                           smem, s, in, out, g, twy, twz));
  else
    PMGB_TRY(launch_planes(plane_r2c_kernel<PLANE_CL, 512, 1>, PLANE_CL, 512, nplanes,
                           plane_smem(g8), s, in, out, g8, twy, twz));
  PMGB_LAUNCHED("plane_r2c_kernel");
  return PMGB_OK;
}

int plane_c2r(const float2 *in, float *out, int nplanes, int ny, int nz, int pitch,
              cudaStream_t s) {
  bool done = false;
  PMGB_TRY(preg_dispatch<false>(in, out, nplanes, ny, nz, pitch, s, &done));
  if (done) {
    PMGB_LAUNCHED("plane_c2r_reg_kernel");
    return PMGB_OK;
  }
  bool wide = ny >= PLANE_CL_WIDE * PLANE_CL_WIDE;
  const PlaneGeom g = plane_geom(ny, nz, pitch, wide ? PLANE_CL_WIDE : PLANE_CL);
  const size_t smem = plane_smem(g);
  wide = wide && clusters_fit((const void *)plane_c2r_kernel<PLANE_CL_WIDE, 256, 3>, 256, smem);
  const PlaneGeom g8 = wide ? g : plane_geom(ny, nz, pitch, PLANE_CL);
  const float2 *twy, *twz;
  PMGB_TRY(twiddles(ny, &twy));
  PMGB_TRY(twiddles(nz, &twz));
  if (wide)
    PMGB_TRY(launch_planes(plane_c2r_kernel<PLANE_CL_WIDE, 256, 3>, PLANE_CL_WIDE, 256, nplanes,
                           smem, s, in, out, g, twy, twz));
  else
    PMGB_TRY(launch_planes(plane_c2r_kernel<PLANE_CL, 512, 1>, PLANE_CL, 512, nplanes,
                           plane_smem(g8), s, in, out, g8, twy, twz));
  PMGB_LAUNCHED("plane_c2r_kernel");
  return PMGB_OK;
}

template <int LG, int MODE>
int xpass_reg(const float2 *in, float2 *out, const XGeom &g, const float2 *twx, const Tables &t,
              float r2, int order, int fd, float scale, cudaStream_t s) {
  using PL = XPlan<LG>;
  const size_t smem = (2 * (size_t)PL::N + 2 * (size_t)PL::BUF) * sizeof(float2);
  PMGB_TRY(set_dyn_smem((const void *)xpass_reg_kernel<LG, MODE>, smem));
  xpass_reg_kernel<LG, MODE><<<g.ny * g.chunks, PL::T * XW, smem, s>>>(in, out, g, twx, t, r2,
                                                                       order, fd, scale);
  PMGB_LAUNCHED("xpass_reg_kernel");
  return PMGB_OK;
}

template <int MODE>
int xpass(const float2 *in, float2 *out, int nx, int ny, int nz, int pitch, int64_t cs_in,
          int64_t cs_out, float r_split, int order, int fd, float scale, cudaStream_t s) {
  XGeom g;
  g.nx = nx;
  g.ny = ny;
  g.lgx = ilog2(nx);
  g.nzh = nz / 2 + 1;
  g.pitch = pitch;
  g.chunks = (g.nzh + XW - 1) / XW;
  g.cs_in = cs_in;
  g.cs_out = cs_out;
  const float2 *twx;
  PMGB_TRY(twiddles(nx, &twx));
  Tables t{nullptr, nullptr, nullptr};
  if (MODE == X_FORCES || MODE == X_FORCES_ADJ || MODE == X_POTENTIAL)
    PMGB_TRY(tables(nx, ny, nz, &t));
  const float r2 = r_split * r_split;
  switch (g.lgx) {
    case 6: return xpass_reg<6, MODE>(in, out, g, twx, t, r2, order, fd, scale, s);
    case 7: return xpass_reg<7, MODE>(in, out, g, twx, t, r2, order, fd, scale, s);
    case 8: return xpass_reg<8, MODE>(in, out, g, twx, t, r2, order, fd, scale, s);
    case 9: return xpass_reg<9, MODE>(in, out, g, twx, t, r2, order, fd, scale, s);
    case 10: return xpass_reg<10, MODE>(in, out, g, twx, t, r2, order, fd, scale, s);
    default: break;
  }
  const size_t smem = 2 * (size_t)nx * XW * sizeof(float2);
  PMGB_TRY(set_dyn_smem((const void *)xpass_kernel<MODE>, smem));
  xpass_kernel<MODE><<<ny * g.chunks, XPASS_THREADS, smem, s>>>(in, out, g, twx, t,
                                                                  r_split * r_split, order, fd,
                                                                  scale);
  PMGB_LAUNCHED("xpass_kernel");
  return PMGB_OK;
}

}  // namespace

// 0: cuFFT 3-D + k-space kernel; 1 (default): cuFFT 2-D planes + the fused
// x pass; 2: the library's plane kernels + the fused x pass.
static std::atomic<int> g_spectral{1};

bool spectral_enabled() { return g_spectral.load() != 0; }

int spectral_mode() { return g_spectral.load(); }

int set_spectral(int mode) { return g_spectral.exchange(mode); }

// plane transforms of the composite pipeline: cuFFT's batched 2-D or ours
static int planes_r2c(const float *in, float2 *out, int nplanes, int ny, int nz, int pitch,
                      cudaStream_t s) {
  if (g_spectral.load() == 2) return plane_r2c(in, out, nplanes, ny, nz, pitch, s);
  return fft_planes_r2c(in, out, nplanes, ny, nz, pitch, s);
}

static int planes_c2r(float2 *in, float *out, int nplanes, int ny, int nz, int pitch,
                      cudaStream_t s) {
  if (g_spectral.load() == 2) return plane_c2r(in, out, nplanes, ny, nz, pitch, s);
  return fft_planes_c2r(in, out, nplanes, ny, nz, pitch, s);
}

int spectral_pitch(int nz) { return (nz / 2 + 1 + XW - 1) / XW * XW; }

bool spectral_supported(int nx, int ny, int nz) {
  return pow2(nx) && pow2(ny) && pow2(nz) && nx >= 8 && nx <= 1024 &&
         ny >= PLANE_CL * PLANE_CL && ny <= 512 && nz >= 16 && nz <= 512;
}

static int check_spectral(int nx, int ny, int nz) {
  if (!spectral_supported(nx, ny, nz))
    return fail(PMGB_ERR_UNSUPPORTED,
                "the spectral pipeline needs power-of-two nx in [8,1024], ny in [64,512], "
                "nz in [16,512]");
  return PMGB_OK;
}

int spectral_r2c(const float *in, void *out, int nx, int ny, int nz, int batch,
                 cudaStream_t s) {
  PMGB_TRY(check_spectral(nx, ny, nz));
  const int pitch = spectral_pitch(nz);
  float2 *o = static_cast<float2 *>(out);
  PMGB_TRY(planes_r2c(in, o, nx * batch, ny, nz, pitch, s));
  if (g_spectral.load() != 2) {
    // cuFFT writes the nz/2+1 modes of each row; the padding is zeroed here
    const int nzh = nz / 2 + 1;
    PMGB_CUDA(cudaMemset2DAsync(o + nzh, pitch * sizeof(float2), 0,
                                (pitch - nzh) * sizeof(float2), (size_t)nx * ny * batch, s));
  }
  const int64_t cs = (int64_t)nx * ny * pitch;
  for (int b = 0; b < batch; ++b)
    PMGB_TRY(xpass<X_FORWARD>(o + b * cs, o + b * cs, nx, ny, nz, pitch, cs, cs, 0.f, 1, 0,
                              1.f, s));
  return PMGB_OK;
}

int spectral_c2r(void *in, float *out, int nx, int ny, int nz, int batch, cudaStream_t s) {
  PMGB_TRY(check_spectral(nx, ny, nz));
  const int pitch = spectral_pitch(nz);
  float2 *i2 = static_cast<float2 *>(in);
  const int64_t cs = (int64_t)nx * ny * pitch;
  for (int b = 0; b < batch; ++b)
    PMGB_TRY(xpass<X_INVERSE>(i2 + b * cs, i2 + b * cs, nx, ny, nz, pitch, cs, cs, 0.f, 1, 0,
                              1.f, s));
  PMGB_TRY(planes_c2r(i2, out, nx * batch, ny, nz, pitch, s));
  return PMGB_OK;
}

// ---- real-space order-1 gradient -------------------------------------------
//
// The order-1 gradient multiplier i g(w), g(w) = (8 sin w - sin 2w)/6
// (jaxpm/kernels.py:41-66), is the transfer function of the stencil
// D p = (8 (p[+1] - p[-1]) - (p[+2] - p[-2])) / 12 along each axis; D is
// antisymmetric (D^T = -D).  One thread per cell, z fastest: the twelve
// neighbours come through L1 / L2 (each potential value is read by 13
// threads), one potential read and three force writes per cell from DRAM.

__device__ __forceinline__ float d_stencil(float m2, float m1, float p1, float p2) {
  const float t1 = p1 - m1, t2 = p2 - m2;
  return (8.0f * t1 - t2) * (1.0f / 12.0f);
}

// f3[c] = -D_c pot: the forces of the potential (spectral_forces' result).
__global__ void __launch_bounds__(256)
stencil_forces_kernel(const float *__restrict__ pot, float *__restrict__ f3, int nx, int ny,
                      int nz) {
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(e % nz);
    const int64_t r = e / nz;
    const int y = (int)(r % ny), x = (int)(r / ny);
    auto at = [&](int xx, int yy, int zz) {
      return __ldg(pot + ((int64_t)xx * ny + yy) * nz + zz);
    };
    const int xm1 = x == 0 ? nx - 1 : x - 1, xm2 = x < 2 ? x - 2 + nx : x - 2;
    const int xp1 = x + 1 == nx ? 0 : x + 1, xp2 = x + 2 >= nx ? x + 2 - nx : x + 2;
    const int ym1 = y == 0 ? ny - 1 : y - 1, ym2 = y < 2 ? y - 2 + ny : y - 2;
    const int yp1 = y + 1 == ny ? 0 : y + 1, yp2 = y + 2 >= ny ? y + 2 - ny : y + 2;
    const int zm1 = z == 0 ? nz - 1 : z - 1, zm2 = z < 2 ? z - 2 + nz : z - 2;
    const int zp1 = z + 1 == nz ? 0 : z + 1, zp2 = z + 2 >= nz ? z + 2 - nz : z + 2;
    f3[e] = -d_stencil(at(xm2, y, z), at(xm1, y, z), at(xp1, y, z), at(xp2, y, z));
    f3[n + e] = -d_stencil(at(x, ym2, z), at(x, ym1, z), at(x, yp1, z), at(x, yp2, z));
    f3[2 * n + e] = -d_stencil(at(x, y, zm2), at(x, y, zm1), at(x, y, zp1), at(x, y, zp2));
  }
}

// out = sum_c D_c g3[c]: the potential cotangent of force-mesh cotangents
// (the transpose of stencil_forces_kernel, -D_c^T = D_c).
__global__ void __launch_bounds__(256)
stencil_adjoint_kernel(const float *__restrict__ g3, float *__restrict__ out, int nx, int ny,
                       int nz) {
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(e % nz);
    const int64_t r = e / nz;
    const int y = (int)(r % ny), x = (int)(r / ny);
    auto at = [&](int c, int xx, int yy, int zz) {
      return __ldg(g3 + c * n + ((int64_t)xx * ny + yy) * nz + zz);
    };
    const int xm1 = x == 0 ? nx - 1 : x - 1, xm2 = x < 2 ? x - 2 + nx : x - 2;
    const int xp1 = x + 1 == nx ? 0 : x + 1, xp2 = x + 2 >= nx ? x + 2 - nx : x + 2;
    const int ym1 = y == 0 ? ny - 1 : y - 1, ym2 = y < 2 ? y - 2 + ny : y - 2;
    const int yp1 = y + 1 == ny ? 0 : y + 1, yp2 = y + 2 >= ny ? y + 2 - ny : y + 2;
    const int zm1 = z == 0 ? nz - 1 : z - 1, zm2 = z < 2 ? z - 2 + nz : z - 2;
    const int zp1 = z + 1 == nz ? 0 : z + 1, zp2 = z + 2 >= nz ? z + 2 - nz : z + 2;
    out[e] = d_stencil(at(0, xm2, y, z), at(0, xm1, y, z), at(0, xp1, y, z), at(0, xp2, y, z)) +
             d_stencil(at(1, x, ym2, z), at(1, x, ym1, z), at(1, x, yp1, z), at(1, x, yp2, z)) +
             d_stencil(at(2, x, y, zm2), at(2, x, y, zm1), at(2, x, y, zp1), at(2, x, y, zp2));
  }
}

// Tiled forms of the two stencils: a CTA takes a 32 (z) x 8 (y) tile and
// marches along ST_XCH planes of x, keeping each thread's column along x in a
// register window (the x stencil) and staging the current plane (with the
// halo its y and z stencils need) in shared memory, so each input value
// comes from DRAM about once.  The values of the plane two ahead are loaded
// into registers while the current plane is computed, so two planes' loads
// are in flight.  Needs nz % 32 == 0, ny % 8 == 0, nx % ST_XCH == 0.
constexpr int ST_TZ = 32, ST_TY = 8, ST_XCH = 32;
constexpr int ST_THREADS = ST_TZ * ST_TY;
static_assert(ST_XCH % 2 == 0, "the tiled stencils march two planes per loop trip");

__device__ __forceinline__ int wrap_lo_hi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

__global__ void __launch_bounds__(ST_THREADS)
stencil_forces_tiled_kernel(const float *__restrict__ pot, float *__restrict__ f3, int nx, int ny,
                            int nz) {
  constexpr int HALO = (ST_TY + 4) * (ST_TZ + 4);  // the plane tile with its y and z halo
  constexpr int PER = (HALO + ST_THREADS - 1) / ST_THREADS;
  __shared__ float pl[ST_TY + 4][ST_TZ + 4];
  const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * ST_TZ + tz;
  const int xch = nx / ST_XCH, b = blockIdx.z / xch;
  const int zb = blockIdx.x * ST_TZ, yb = blockIdx.y * ST_TY, x0 = (blockIdx.z - b * xch) * ST_XCH;
  const int x1 = x0 + ST_XCH;
  const int64_t plane = (int64_t)ny * nz, n = plane * nx;
  pot += b * n;  // batch entry b: [b][nx][ny][nz] in, [b][3][nx][ny][nz] out
  f3 += 3 * b * n;
  const int64_t col = (int64_t)(yb + ty) * nz + zb + tz;
  auto load_tile = [&](int x, float (&v)[PER]) {
    const float *P = pot + (int64_t)x * plane;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int q = tid + ST_THREADS * i;
      if (q < HALO) {
        const int r = q / (ST_TZ + 4), c = q - r * (ST_TZ + 4);
        v[i] = __ldg(P + (int64_t)wrap_lo_hi(yb + r - 2, ny) * nz + wrap_lo_hi(zb + c - 2, nz));
      }
    }
  };
  auto at_col = [&](int x) { return __ldg(pot + wrap_lo_hi(x, nx) * plane + col); };
  // the x window: pot at x-2, x-1, x+1, x+2 for plane x, and x+3 already
  // loaded (two planes ahead, like the tiles)
  float w0 = at_col(x0 - 2), w1 = at_col(x0 - 1), w3 = at_col(x0 + 1), w4 = at_col(x0 + 2);
  float w5 = at_col(x0 + 3);
  float ta[PER], tb[PER];  // tiles of planes x and x + 1 (x even within the run)
  load_tile(x0, ta);
  load_tile(x0 + 1, tb);
  // one plane: its tile into shared memory, the loads of two planes ahead
  // issued into the registers it frees, then the stencils
  auto step = [&](int x, float (&tile)[PER]) {
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int q = tid + ST_THREADS * i;
      if (q < HALO) (&pl[0][0])[q] = tile[i];
    }
    __syncthreads();
    float w6 = 0.f;
    if (x + 2 < x1) {
      load_tile(x + 2, tile);
      w6 = at_col(x + 4);
    }
    const int64_t e = (int64_t)x * plane + col;
    f3[e] = -d_stencil(w0, w1, w3, w4);
    f3[n + e] = -d_stencil(pl[ty][tz + 2], pl[ty + 1][tz + 2], pl[ty + 3][tz + 2],
                           pl[ty + 4][tz + 2]);
    f3[2 * n + e] = -d_stencil(pl[ty + 2][tz], pl[ty + 2][tz + 1], pl[ty + 2][tz + 3],
                               pl[ty + 2][tz + 4]);
    const float w2 = pl[ty + 2][tz + 2];  // pot at plane x: the next window's x-1 value
    __syncthreads();
    w0 = w1;
    w1 = w2;
    w3 = w4;
    w4 = w5;
    w5 = w6;
  };
  for (int x = x0; x < x1; x += 2) {  // ST_XCH is even
    step(x, ta);
    step(x + 1, tb);
  }
}

__global__ void __launch_bounds__(ST_THREADS)
stencil_adjoint_tiled_kernel(const float *__restrict__ g3, float *__restrict__ out, int nx,
                             int ny, int nz) {
  constexpr int HY = (ST_TY + 4) * ST_TZ, HZ = ST_TY * (ST_TZ + 4);  // y and z halo tiles
  constexpr int PER = (HY + HZ + ST_THREADS - 1) / ST_THREADS;
  __shared__ float gy[ST_TY + 4][ST_TZ];
  __shared__ float gz[ST_TY][ST_TZ + 4];
  const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * ST_TZ + tz;
  const int xch = nx / ST_XCH, b = blockIdx.z / xch;
  const int zb = blockIdx.x * ST_TZ, yb = blockIdx.y * ST_TY, x0 = (blockIdx.z - b * xch) * ST_XCH;
  const int x1 = x0 + ST_XCH;
  const int64_t plane = (int64_t)ny * nz, n = plane * nx;
  g3 += 3 * b * n;  // batch entry b: [b][3][nx][ny][nz] in, [b][nx][ny][nz] out
  out += b * n;
  const int64_t col = (int64_t)(yb + ty) * nz + zb + tz;
  // item q < HY: gy[r][c] of the y component; else gz of the z component
  auto load_tiles = [&](int x, float (&v)[PER]) {
    const float *Py = g3 + n + (int64_t)x * plane, *Pz = g3 + 2 * n + (int64_t)x * plane;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int q = tid + ST_THREADS * i;
      if (q < HY) {
        const int r = q / ST_TZ, c = q - r * ST_TZ;
        v[i] = __ldg(Py + (int64_t)wrap_lo_hi(yb + r - 2, ny) * nz + zb + c);
      } else if (q < HY + HZ) {
        const int qz = q - HY, r = qz / (ST_TZ + 4), c = qz - r * (ST_TZ + 4);
        v[i] = __ldg(Pz + (int64_t)(yb + r) * nz + wrap_lo_hi(zb + c - 2, nz));
      }
    }
  };
  auto at_col = [&](int x) { return __ldg(g3 + wrap_lo_hi(x, nx) * plane + col); };
  float w0 = at_col(x0 - 2), w1 = at_col(x0 - 1), w2 = at_col(x0), w3 = at_col(x0 + 1),
        w4 = at_col(x0 + 2), w5 = at_col(x0 + 3);
  float ta[PER], tb[PER];  // tiles of planes x and x + 1 (x even within the run)
  load_tiles(x0, ta);
  load_tiles(x0 + 1, tb);
  auto step = [&](int x, float (&tiles)[PER]) {
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int q = tid + ST_THREADS * i;
      if (q < HY) (&gy[0][0])[q] = tiles[i];
      else if (q < HY + HZ) (&gz[0][0])[q - HY] = tiles[i];
    }
    __syncthreads();
    float w6 = 0.f;
    if (x + 2 < x1) {
      load_tiles(x + 2, tiles);
      w6 = at_col(x + 4);
    }
    out[(int64_t)x * plane + col] =
        d_stencil(w0, w1, w3, w4) +
        d_stencil(gy[ty][tz], gy[ty + 1][tz], gy[ty + 3][tz], gy[ty + 4][tz]) +
        d_stencil(gz[ty][tz], gz[ty][tz + 1], gz[ty][tz + 3], gz[ty][tz + 4]);
    __syncthreads();
    w0 = w1;
    w1 = w2;
    w2 = w3;
    w3 = w4;
    w4 = w5;
    w5 = w6;
  };
  for (int x = x0; x < x1; x += 2) {  // ST_XCH is even
    step(x, ta);
    step(x + 1, tb);
  }
}

static bool stencil_tiled(int nx, int ny, int nz, int batch) {
  return nz % ST_TZ == 0 && ny % ST_TY == 0 && nx % ST_XCH == 0 &&
         (int64_t)batch * (nx / ST_XCH) <= 65535;
}

int stencil_forces(const float *pot, float *f3, int nx, int ny, int nz, int batch,
                   cudaStream_t s) {
  const int64_t n = (int64_t)nx * ny * nz;
  if (stencil_tiled(nx, ny, nz, batch)) {
    stencil_forces_tiled_kernel<<<dim3(nz / ST_TZ, ny / ST_TY, batch * (nx / ST_XCH)),
                                  dim3(ST_TZ, ST_TY), 0, s>>>(pot, f3, nx, ny, nz);
    PMGB_LAUNCHED("stencil_forces_tiled_kernel");
    return PMGB_OK;
  }
  for (int b = 0; b < batch; ++b) {
    stencil_forces_kernel<<<wave_grid(stencil_forces_kernel, n, 256), 256, 0, s>>>(
        pot + b * n, f3 + 3 * b * n, nx, ny, nz);
    PMGB_LAUNCHED("stencil_forces_kernel");
  }
  return PMGB_OK;
}

int stencil_adjoint(const float *g3, float *out, int nx, int ny, int nz, int batch,
                    cudaStream_t s) {
  const int64_t n = (int64_t)nx * ny * nz;
  if (stencil_tiled(nx, ny, nz, batch)) {
    stencil_adjoint_tiled_kernel<<<dim3(nz / ST_TZ, ny / ST_TY, batch * (nx / ST_XCH)),
                                   dim3(ST_TZ, ST_TY), 0, s>>>(g3, out, nx, ny, nz);
    PMGB_LAUNCHED("stencil_adjoint_tiled_kernel");
    return PMGB_OK;
  }
  for (int b = 0; b < batch; ++b) {
    stencil_adjoint_kernel<<<wave_grid(stencil_adjoint_kernel, n, 256), 256, 0, s>>>(
        g3 + 3 * b * n, out + b * n, nx, ny, nz);
    PMGB_LAUNCHED("stencil_adjoint_kernel");
  }
  return PMGB_OK;
}

int spectral_forces(const float *mesh, void *spec, void *fspec, float *f3, int nx, int ny,
                    int nz, float r_split, int order, int fd, float scale, cudaStream_t s) {
  PMGB_TRY(check_spectral(nx, ny, nz));
  const int pitch = spectral_pitch(nz);
  const int64_t cs = (int64_t)nx * ny * pitch;
  float2 *d = static_cast<float2 *>(spec), *f = static_cast<float2 *>(fspec);
  if (order == 1 && fd == 0) {
    // one inverse transform of the potential (into fspec's memory), then
    // the order-1 gradient as its real-space stencil
    float *pot = reinterpret_cast<float *>(f);
    PMGB_TRY(spectral_potential(mesh, d, pot, nx, ny, nz, r_split, scale, s));
    return stencil_forces(pot, f3, nx, ny, nz, 1, s);
  }
  PMGB_TRY(planes_r2c(mesh, d, nx, ny, nz, pitch, s));
  PMGB_TRY(xpass<X_FORCES>(d, f, nx, ny, nz, pitch, cs, cs, r_split, order, fd, scale, s));
  PMGB_TRY(planes_c2r(f, f3, 3 * nx, ny, nz, pitch, s));
  return PMGB_OK;
}

// mesh -> spec -> the potential pot = IFFT(delta_k * invlaplace * longrange
// * scale) as a real mesh [nx][ny][nz]: the forces' pipeline with one
// inverse transform instead of three (the order-1 gradient is then the
// real-space stencil whose transfer function it is).  The x pass runs in
// place on spec.
int spectral_potential(const float *mesh, void *spec, float *pot, int nx, int ny, int nz,
                       float r_split, float scale, cudaStream_t s) {
  PMGB_TRY(check_spectral(nx, ny, nz));
  const int pitch = spectral_pitch(nz);
  const int64_t cs = (int64_t)nx * ny * pitch;
  float2 *d = static_cast<float2 *>(spec);
  PMGB_TRY(planes_r2c(mesh, d, nx, ny, nz, pitch, s));
  PMGB_TRY(xpass<X_POTENTIAL>(d, d, nx, ny, nz, pitch, cs, cs, r_split, 1, 0, scale, s));
  PMGB_TRY(planes_c2r(d, pot, nx, ny, nz, pitch, s));
  return PMGB_OK;
}

int spectral_forces_vjp(const float *g3, void *spec3, void *dspec, float *rbar, int nx, int ny,
                        int nz, float r_split, int order, int fd, float scale,
                        cudaStream_t s) {
  PMGB_TRY(check_spectral(nx, ny, nz));
  const int pitch = spectral_pitch(nz);
  const int64_t cs = (int64_t)nx * ny * pitch;
  float2 *a = static_cast<float2 *>(spec3), *d = static_cast<float2 *>(dspec);
  if (order == 1 && fd == 0) {
    // the potential cotangent sum_c D_c g_c in real space (into spec3's
    // memory), then the symmetric k-space multiply of the potential
    float *pbar = reinterpret_cast<float *>(a);
    PMGB_TRY(stencil_adjoint(g3, pbar, nx, ny, nz, 1, s));
    return spectral_potential(pbar, d, rbar, nx, ny, nz, r_split, scale, s);
  }
  PMGB_TRY(planes_r2c(g3, a, 3 * nx, ny, nz, pitch, s));
  PMGB_TRY(xpass<X_FORCES_ADJ>(a, d, nx, ny, nz, pitch, cs, cs, r_split, order, fd, scale, s));
  PMGB_TRY(planes_c2r(d, rbar, nx, ny, nz, pitch, s));
  return PMGB_OK;
}

}  // namespace pmgb
