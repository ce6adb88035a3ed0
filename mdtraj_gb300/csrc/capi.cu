// C-ABI plumbing: error reporting, device queries, host<->device row copies.
#include <stdarg.h>
#include <stdio.h>

#include <atomic>
#include <thread>
#include <vector>

#include "capi_internal.h"

namespace gb {

namespace {
thread_local char g_last_error[1024] = "";

// Per-device attributes, filled on first use.  Host threads may race on the
// first fill: both store the same values, smem before sm, and a reader that
// sees sm != 0 (acquire) also sees smem.
struct DevCache {
  std::atomic<int> sm{0};
  std::atomic<int> smem{0};
};
DevCache g_dev[64];
}  // namespace

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

void clear_error() { g_last_error[0] = '\0'; }

int cuda_status(cudaError_t e, const char* what) {
  return set_error(GBRMSD_E_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

static DevCache& dev_cache() {
  int d = 0;
  cudaGetDevice(&d);
  DevCache& c = g_dev[(d >= 0 && d < 64) ? d : 0];
  if (c.sm.load(std::memory_order_acquire) == 0) {
    int sm = 0, smem = 0;
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, d);
    cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, d);
    c.smem.store(smem, std::memory_order_relaxed);
    c.sm.store(sm > 0 ? sm : 1, std::memory_order_release);
  }
  return c;
}

int sm_count() { return dev_cache().sm.load(std::memory_order_relaxed); }
int max_dyn_smem() { return dev_cache().smem.load(std::memory_order_relaxed); }

}  // namespace gb

extern "C" {

int gbrmsd_version(void) { return 1; }

const char* gbrmsd_last_error(void) { return gb::g_last_error; }

int gbrmsd_device_supported(void) {
  int d = 0, major = 0, minor = 0;
  if (cudaGetDevice(&d) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, d) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, d) != cudaSuccess) return 0;
  return (major == 10 && minor == 3) ? 1 : 0;
}

int gbrmsd_device_caps(int32_t* caps, int32_t n) {
  gb::clear_error();
  int d = 0;
  GB_CUDA_TRY(cudaGetDevice(&d), "cudaGetDevice");
  const cudaDeviceAttr attrs[] = {cudaDevAttrComputeCapabilityMajor,
                                  cudaDevAttrComputeCapabilityMinor,
                                  cudaDevAttrMultiProcessorCount,
                                  cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                  cudaDevAttrPageableMemoryAccess,
                                  cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                                  cudaDevAttrConcurrentManagedAccess,
                                  cudaDevAttrHostRegisterSupported,
                                  cudaDevAttrDirectManagedMemAccessFromHost,
                                  cudaDevAttrL2CacheSize,
                                  cudaDevAttrClockRate,
                                  cudaDevAttrMemoryClockRate};
  const int na = (int)(sizeof(attrs) / sizeof(attrs[0]));
  for (int i = 0; i < n && i < na; ++i) {
    int v = -1;
    if (cudaDeviceGetAttribute(&v, attrs[i], d) != cudaSuccess) v = -1;
    caps[i] = v;
  }
  return na;
}

int gbrmsd_copy_rows(void* dst, size_t dst_pitch, const void* src, size_t src_pitch,
                     size_t row_bytes, size_t n_rows, int32_t kind, void* stream) {
  gb::clear_error();
  if (n_rows == 0 || row_bytes == 0) return GBRMSD_OK;
  if (!dst || !src) return gb::set_error(GBRMSD_E_INVALID, "copy_rows: null pointer");
  if (dst_pitch < row_bytes || src_pitch < row_bytes)
    return gb::set_error(GBRMSD_E_INVALID, "copy_rows: pitch smaller than row");
  cudaMemcpyKind k;
  switch (kind) {
    case 1: k = cudaMemcpyHostToDevice; break;
    case 2: k = cudaMemcpyDeviceToHost; break;
    case 3: k = cudaMemcpyDeviceToDevice; break;
    default: return gb::set_error(GBRMSD_E_INVALID, "copy_rows: bad kind %d", kind);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dst_pitch == row_bytes && src_pitch == row_bytes) {
    GB_CUDA_TRY(cudaMemcpyAsync(dst, src, row_bytes * n_rows, k, s), "cudaMemcpyAsync");
  } else {
    GB_CUDA_TRY(cudaMemcpy2DAsync(dst, dst_pitch, src, src_pitch, row_bytes, n_rows, k, s),
                "cudaMemcpy2DAsync");
  }
  return GBRMSD_OK;
}

int gbrmsd_host_subtract_centroids(float* x, int64_t n_frames, int32_t n_atoms, int64_t frame_stride,
                                    const float* centroids, int32_t n_threads) {
  gb::clear_error();
  if (n_frames <= 0 || n_atoms <= 0) return GBRMSD_OK;
  if (!x || !centroids) return gb::set_error(GBRMSD_E_INVALID, "host_subtract_centroids: null pointer");
  if (frame_stride < 3LL * n_atoms) return gb::set_error(GBRMSD_E_INVALID, "host_subtract_centroids: frame_stride too small");
  int64_t nt = n_threads > 0 ? n_threads : (int64_t)std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  // Below ~4 MB the thread start-up costs more than the subtraction.
  const int64_t bytes = n_frames * (int64_t)n_atoms * 12;
  const int64_t by_size = bytes / (4LL << 20) + 1;
  if (nt > by_size) nt = by_size;
  if (nt > n_frames) nt = n_frames;
  auto work = [=](int64_t f0, int64_t f1) {
    for (int64_t f = f0; f < f1; ++f) {
      float* p = x + f * frame_stride;
      const float mx = centroids[3 * f], my = centroids[3 * f + 1], mz = centroids[3 * f + 2];
      for (int32_t k = 0; k < n_atoms; ++k) {
        p[3 * k] -= mx;
        p[3 * k + 1] -= my;
        p[3 * k + 2] -= mz;
      }
    }
  };
  if (nt == 1) {
    work(0, n_frames);
    return GBRMSD_OK;
  }
  std::vector<std::thread> pool;
  pool.reserve((size_t)nt);
  for (int64_t t = 0; t < nt; ++t) {
    const int64_t f0 = n_frames * t / nt, f1 = n_frames * (t + 1) / nt;
    pool.emplace_back(work, f0, f1);
  }
  for (auto& th : pool) th.join();
  return GBRMSD_OK;
}

}  // extern "C"
