// Binned power spectrum of a half spectrum.
//
// Reference: jaxpm/utils.py:14-128 (_initialize_pk, power_spectrum with
// multipoles=0): |k| = sqrt(sum_i (2 pi n_i / L_i * fftfreq(n_i))^2) in
// float64, bins from np.digitize(|k|, kedges) (bin b holds
// kedges[b-1] <= |k| < kedges[b]), power |X|^2 of the ortho-normalised FFT.
// The half spectrum stands for the full one: a mode with 0 < kz < nz/2
// also stands for its mirror (-k), which has the same |k| and |X|^2, so it
// counts twice.  Each CTA accumulates its own float64 histogram in shared
// memory, then adds it to the global one.
#include "common.cuh"

namespace pmgb {
namespace {

__global__ void power_kernel(const float2 *__restrict__ spec, int nx, int ny, int nz, double sx,
                             double sy, double sz, const double *__restrict__ edges,
                             int n_edges, double inv_norm, double *__restrict__ psum,
                             double *__restrict__ pcount, double *__restrict__ ksum) {
  extern __shared__ double sh[];
  const int nb = n_edges + 1;
  double *hp = sh, *hc = sh + nb, *hk = sh + 2 * nb;
  for (int b = threadIdx.x; b < 3 * nb; b += blockDim.x) sh[b] = 0.0;
  __syncthreads();
  const int nzh = nz / 2 + 1;
  const int64_t total = (int64_t)nx * ny * nzh;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int k = (int)(e % nzh);
    int64_t r = e / nzh;
    int j = (int)(r % ny), i = (int)(r / ny);
    int mi = i < (nx + 1) / 2 ? i : i - nx;
    int mj = j < (ny + 1) / 2 ? j : j - ny;
    int mk = k < (nz + 1) / 2 ? k : k - nz;
    double kx = __dmul_rn(sx, __dmul_rn((double)mi, 1.0 / nx));
    double ky = __dmul_rn(sy, __dmul_rn((double)mj, 1.0 / ny));
    double kz = __dmul_rn(sz, __dmul_rn((double)mk, 1.0 / nz));
    // Summed in float64 as NumPy does (no fused multiply-adds); the square
    // root is taken in float32 because jnp.sqrt converts its float64 input
    // to float32 (x64 disabled, the reference default).
    double kk = __dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz));
    double km = (double)sqrtf((float)kk);
    // digitize: number of edges <= km
    int lo = 0, hi = n_edges;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (edges[mid] <= km) lo = mid + 1; else hi = mid;
    }
    double mult = (k == 0 || (nz % 2 == 0 && k == nz / 2)) ? 1.0 : 2.0;
    float2 v = spec[e];
    double p = ((double)v.x * v.x + (double)v.y * v.y) * inv_norm;
    atomicAdd(hp + lo, mult * p);
    atomicAdd(hc + lo, mult);
    atomicAdd(hk + lo, mult * km);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    if (hc[b] != 0.0) {
      atomicAdd(psum + b, hp[b]);
      atomicAdd(pcount + b, hc[b]);
      atomicAdd(ksum + b, hk[b]);
    }
  }
}

}  // namespace

int power_spectrum(const void *spec, int nx, int ny, int nz, double bx, double by, double bz,
                   const double *edges, int n_edges, double *psum, double *pcount, double *ksum,
                   cudaStream_t s) {
  const int nb = n_edges + 1;
  PMGB_CUDA(cudaMemsetAsync(psum, 0, nb * sizeof(double), s));
  PMGB_CUDA(cudaMemsetAsync(pcount, 0, nb * sizeof(double), s));
  PMGB_CUDA(cudaMemsetAsync(ksum, 0, nb * sizeof(double), s));
  const int64_t total = (int64_t)nx * ny * (nz / 2 + 1);
  const double twopi = 6.283185307179586;
  double inv_norm = 1.0 / ((double)nx * ny * nz);
  // (2 pi * n) / L as written in the reference
  power_kernel<<<grid_for(total, 256, 4), 256, 3 * nb * sizeof(double), s>>>(
      static_cast<const float2 *>(spec), nx, ny, nz, twopi * nx / bx, twopi * ny / by,
      twopi * nz / bz, edges, n_edges, inv_norm, psum, pcount, ksum);
  PMGB_LAUNCHED("power_kernel");
  return PMGB_OK;
}

}  // namespace pmgb
