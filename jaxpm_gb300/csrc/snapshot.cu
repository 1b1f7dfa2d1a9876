// Snapshot output: arrays in device memory written to NumPy .npy files
// without holding up the GPU (the reference saves fields with np.save,
// notebooks/05-MultiHost_PM.py:151-177, after gathering them to the host).
//
// pmgb_snapshot_begin_npy records the array's state in stream order -- a
// device-to-device copy into a caller-provided staging buffer (HBM speed),
// or, without staging, an event the caller promises not to overwrite the
// array before -- and returns at once.  A host thread then streams the
// array to the file through two pinned chunks on its own stream (device to
// host copy of one chunk overlapping the write of the other).
// pmgb_snapshot_wait joins the thread and returns its status.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace pmgb {

namespace {

constexpr size_t CHUNK = 32u << 20;  // bytes per pinned chunk

}  // namespace

// .npy format 1.0 header: magic, version, little-endian header length, and a
// Python-literal dict padded with spaces to a multiple of 64 bytes (ending in
// a newline).
size_t npy_header(const char *descr, const int64_t *shape, int ndim, char *buf, size_t cap) {
  std::string dict = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': (";
  for (int i = 0; i < ndim; ++i) {
    dict += std::to_string(shape[i]);
    if (ndim == 1 || i + 1 < ndim) dict += ",";
    if (i + 1 < ndim) dict += " ";
  }
  dict += "), }";
  size_t total = 10 + dict.size() + 1;
  const size_t padded = (total + 63) / 64 * 64;
  dict.append(padded - total, ' ');
  dict += '\n';
  if (buf && cap >= padded) {
    const uint16_t hl = (uint16_t)(padded - 10);
    std::memcpy(buf, "\x93NUMPY\x01\x00", 8);
    buf[8] = (char)(hl & 0xff);
    buf[9] = (char)(hl >> 8);
    std::memcpy(buf + 10, dict.data(), dict.size());
  }
  return padded;
}

struct Snapshot {
  std::thread worker;
  int status = PMGB_OK;
  std::string error;
};

namespace {

void write_worker(Snapshot *snap, std::string path, const char *src, size_t bytes,
                  std::vector<char> header, cudaEvent_t ready, int device) {
  auto fail_with = [&](const std::string &m) {
    snap->status = PMGB_ERR_CUDA;
    snap->error = m;
  };
  cudaSetDevice(device);
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) {
    snap->status = PMGB_ERR_INVALID_ARGUMENT;
    snap->error = "cannot open " + path + " for writing";
    cudaEventDestroy(ready);
    return;
  }
  cudaStream_t st = nullptr;
  char *pin[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  bool ok = std::fwrite(header.data(), 1, header.size(), f) == header.size();
  if (!ok) fail_with("write failed: " + path);
  if (ok && (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
             cudaHostAlloc((void **)&pin[0], CHUNK, cudaHostAllocDefault) != cudaSuccess ||
             cudaHostAlloc((void **)&pin[1], CHUNK, cudaHostAllocDefault) != cudaSuccess ||
             cudaEventCreateWithFlags(&done[0], cudaEventDisableTiming) != cudaSuccess ||
             cudaEventCreateWithFlags(&done[1], cudaEventDisableTiming) != cudaSuccess ||
             cudaStreamWaitEvent(st, ready, 0) != cudaSuccess)) {
    ok = false;
    fail_with(std::string("snapshot staging: ") + cudaGetErrorString(cudaGetLastError()));
  }
  // chunk i goes to pinned buffer i % 2; its copy is issued while chunk i-1
  // is being written
  const size_t nchunks = (bytes + CHUNK - 1) / CHUNK;
  for (size_t i = 0; ok && i <= nchunks; ++i) {
    if (i < nchunks) {
      const size_t off = i * CHUNK, n = std::min(CHUNK, bytes - off);
      if (cudaMemcpyAsync(pin[i & 1], src + off, n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaEventRecord(done[i & 1], st) != cudaSuccess) {
        ok = false;
        fail_with(std::string("snapshot copy: ") + cudaGetErrorString(cudaGetLastError()));
        break;
      }
    }
    if (i > 0) {
      const size_t j = i - 1, off = j * CHUNK, n = std::min(CHUNK, bytes - off);
      if (cudaEventSynchronize(done[j & 1]) != cudaSuccess) {
        ok = false;
        fail_with(std::string("snapshot copy: ") + cudaGetErrorString(cudaGetLastError()));
        break;
      }
      if (std::fwrite(pin[j & 1], 1, n, f) != n) {
        ok = false;
        fail_with("write failed: " + path);
      }
    }
  }
  if (st) cudaStreamSynchronize(st);
  if (std::fclose(f) != 0 && ok) fail_with("close failed: " + path);
  for (int b = 0; b < 2; ++b) {
    if (pin[b]) cudaFreeHost(pin[b]);
    if (done[b]) cudaEventDestroy(done[b]);
  }
  if (st) cudaStreamDestroy(st);
  cudaEventDestroy(ready);
}

}  // namespace

int snapshot_begin_npy(const char *path, const void *dev, const char *descr, int itemsize,
                       const int64_t *shape, int ndim, void *staging, size_t staging_bytes,
                       cudaStream_t s, Snapshot **out) {
  int64_t count = 1;
  for (int i = 0; i < ndim; ++i) {
    PMGB_REQUIRE(shape[i] >= 0, "negative extent in shape");
    count *= shape[i];
  }
  const size_t bytes = (size_t)count * (size_t)itemsize;
  if (staging && staging_bytes < bytes)
    return fail(PMGB_ERR_WORKSPACE, "snapshot staging needs " + std::to_string(bytes) +
                                        " bytes, got " + std::to_string(staging_bytes));
  const size_t hlen = npy_header(descr, shape, ndim, nullptr, 0);
  std::vector<char> header(hlen);
  npy_header(descr, shape, ndim, header.data(), hlen);
  const char *src = static_cast<const char *>(dev);
  if (staging && bytes > 0) {
    PMGB_CUDA(cudaMemcpyAsync(staging, dev, bytes, cudaMemcpyDeviceToDevice, s));
    src = static_cast<const char *>(staging);
  }
  cudaEvent_t ready;
  PMGB_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ready, s);
  if (e != cudaSuccess) {
    cudaEventDestroy(ready);
    return fail(PMGB_ERR_CUDA, std::string("snapshot event: ") + cudaGetErrorString(e));
  }
  int device = 0;
  PMGB_CUDA(cudaGetDevice(&device));
  Snapshot *snap = new Snapshot();
  snap->worker = std::thread(write_worker, snap, std::string(path), src, bytes,
                             std::move(header), ready, device);
  *out = snap;
  return PMGB_OK;
}

int snapshot_wait(Snapshot *snap) {
  if (!snap) return fail(PMGB_ERR_INVALID_ARGUMENT, "snapshot is NULL");
  if (snap->worker.joinable()) snap->worker.join();
  const int st = snap->status;
  const std::string msg = snap->error;
  delete snap;
  if (st != PMGB_OK) return fail(st, msg);
  return PMGB_OK;
}

}  // namespace pmgb
