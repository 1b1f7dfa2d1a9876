// cuFFT wrappers with a process-wide plan cache.
//
// The reference's fft3d/ifft3d (jaxpm/distributed.py:37-42) are C2C
// transforms of real fields; here the forward transform is R2C (the half
// spectrum carries the same information) and the inverse C2R, which equals
// ifft3d(x).real for a Hermitian spectrum.  cuFFT stays a library call:
// plans are created on first use per (device, shape, batch, direction),
// kept for the life of the process, and guarded by one mutex that is also
// held across cufftSetStream + cufftExec so concurrent callers on different
// streams cannot race on a shared plan.
#include <cufft.h>

#include <map>
#include <mutex>
#include <tuple>

#include "common.cuh"
#include "kernels.cuh"

namespace pmgb {
namespace {

// dev, nx (0 for a batch of 2-D plane transforms), ny, nz, batch, type, pitch
using Key = std::tuple<int, int, int, int, int, int, int>;

std::mutex g_mu;
std::map<Key, cufftHandle> g_plans;

const char *cufft_name(cufftResult r) {
  switch (r) {
    case CUFFT_SUCCESS: return "CUFFT_SUCCESS";
    case CUFFT_INVALID_PLAN: return "CUFFT_INVALID_PLAN";
    case CUFFT_ALLOC_FAILED: return "CUFFT_ALLOC_FAILED";
    case CUFFT_INVALID_VALUE: return "CUFFT_INVALID_VALUE";
    case CUFFT_INTERNAL_ERROR: return "CUFFT_INTERNAL_ERROR";
    case CUFFT_EXEC_FAILED: return "CUFFT_EXEC_FAILED";
    case CUFFT_SETUP_FAILED: return "CUFFT_SETUP_FAILED";
    case CUFFT_INVALID_SIZE: return "CUFFT_INVALID_SIZE";
    default: return "cufft error";
  }
}

// Returns the cached plan (creating it); g_mu must be held.
int plan_for(int nx, int ny, int nz, int batch, cufftType type, cufftHandle *out) {
  int dev = 0;
  PMGB_CUDA(cudaGetDevice(&dev));
  Key k{dev, nx, ny, nz, batch, (int)type, 0};
  auto it = g_plans.find(k);
  if (it != g_plans.end()) {
    *out = it->second;
    return PMGB_OK;
  }
  cufftHandle h;
  cufftResult r = cufftCreate(&h);
  if (r != CUFFT_SUCCESS) return fail(PMGB_ERR_CUFFT, std::string("cufftCreate: ") + cufft_name(r));
  int n[3] = {nx, ny, nz};
  size_t work = 0;
  r = cufftMakePlanMany(h, 3, n, nullptr, 1, 0, nullptr, 1, 0, type, batch, &work);
  if (r != CUFFT_SUCCESS) {
    cufftDestroy(h);
    return fail(PMGB_ERR_CUFFT, std::string("cufftMakePlanMany: ") + cufft_name(r));
  }
  g_plans[k] = h;
  *out = h;
  return PMGB_OK;
}

// Batched 2-D (y, z) transforms of x-planes with padded half-spectrum rows
// ([plane][ny][pitch] complex); g_mu must be held.
int plane_plan_for(int nplanes, int ny, int nz, int pitch, cufftType type, cufftHandle *out) {
  int dev = 0;
  PMGB_CUDA(cudaGetDevice(&dev));
  Key k{dev, 0, ny, nz, nplanes, (int)type, pitch};
  auto it = g_plans.find(k);
  if (it != g_plans.end()) {
    *out = it->second;
    return PMGB_OK;
  }
  cufftHandle h;
  cufftResult r = cufftCreate(&h);
  if (r != CUFFT_SUCCESS) return fail(PMGB_ERR_CUFFT, std::string("cufftCreate: ") + cufft_name(r));
  int n[2] = {ny, nz};
  int real_embed[2] = {ny, nz}, spec_embed[2] = {ny, pitch};
  const bool fwd = type == CUFFT_R2C;
  size_t work = 0;
  r = cufftMakePlanMany(h, 2, n, fwd ? real_embed : spec_embed, 1,
                        fwd ? ny * nz : ny * pitch, fwd ? spec_embed : real_embed, 1,
                        fwd ? ny * pitch : ny * nz, type, nplanes, &work);
  if (r != CUFFT_SUCCESS) {
    cufftDestroy(h);
    return fail(PMGB_ERR_CUFFT, std::string("cufftMakePlanMany (planes): ") + cufft_name(r));
  }
  g_plans[k] = h;
  *out = h;
  return PMGB_OK;
}

__global__ void scale_kernel(float *__restrict__ x, int64_t n, float s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= s;
}

}  // namespace

int fft_r2c(const float *in, void *out, int nx, int ny, int nz, int batch, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_mu);
  cufftHandle h;
  PMGB_TRY(plan_for(nx, ny, nz, batch, CUFFT_R2C, &h));
  cufftResult r = cufftSetStream(h, s);
  if (r == CUFFT_SUCCESS)
    r = cufftExecR2C(h, const_cast<cufftReal *>(in), static_cast<cufftComplex *>(out));
  if (r != CUFFT_SUCCESS) return fail(PMGB_ERR_CUFFT, std::string("cufftExecR2C: ") + cufft_name(r));
  return PMGB_OK;
}

int fft_prepare(int nx, int ny, int nz, int batch, int r2c) {
  std::lock_guard<std::mutex> lk(g_mu);
  cufftHandle h;
  return plan_for(nx, ny, nz, batch, r2c ? CUFFT_R2C : CUFFT_C2R, &h);
}

int fft_c2r(void *in, float *out, int nx, int ny, int nz, int batch, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_mu);
  cufftHandle h;
  PMGB_TRY(plan_for(nx, ny, nz, batch, CUFFT_C2R, &h));
  cufftResult r = cufftSetStream(h, s);
  if (r == CUFFT_SUCCESS) r = cufftExecC2R(h, static_cast<cufftComplex *>(in), out);
  if (r != CUFFT_SUCCESS) return fail(PMGB_ERR_CUFFT, std::string("cufftExecC2R: ") + cufft_name(r));
  return PMGB_OK;
}

int fft_planes_r2c(const float *in, void *out, int nplanes, int ny, int nz, int pitch,
                   cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_mu);
  cufftHandle h;
  PMGB_TRY(plane_plan_for(nplanes, ny, nz, pitch, CUFFT_R2C, &h));
  cufftResult r = cufftSetStream(h, s);
  if (r == CUFFT_SUCCESS)
    r = cufftExecR2C(h, const_cast<cufftReal *>(in), static_cast<cufftComplex *>(out));
  if (r != CUFFT_SUCCESS) return fail(PMGB_ERR_CUFFT, std::string("cufftExecR2C: ") + cufft_name(r));
  return PMGB_OK;
}

int fft_planes_c2r(void *in, float *out, int nplanes, int ny, int nz, int pitch,
                   cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_mu);
  cufftHandle h;
  PMGB_TRY(plane_plan_for(nplanes, ny, nz, pitch, CUFFT_C2R, &h));
  cufftResult r = cufftSetStream(h, s);
  if (r == CUFFT_SUCCESS) r = cufftExecC2R(h, static_cast<cufftComplex *>(in), out);
  if (r != CUFFT_SUCCESS) return fail(PMGB_ERR_CUFFT, std::string("cufftExecC2R: ") + cufft_name(r));
  return PMGB_OK;
}

int scale_inplace(float *x, int64_t n, float scale, cudaStream_t s) {
  if (n == 0) return PMGB_OK;
  scale_kernel<<<wave_grid(scale_kernel, n, 256), 256, 0, s>>>(x, n, scale);
  PMGB_LAUNCHED("scale_kernel");
  return PMGB_OK;
}

}  // namespace pmgb
