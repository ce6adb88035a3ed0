// Host <-> device movement for the drop-in's host-buffer path.
//
// On GB300 the GPU reaches the Grace host's pageable memory through the
// host page tables over NVLink-C2C (cudaDevAttrPageableMemoryAccess = 1 with
// cudaDevAttrPageableMemoryAccessUsesHostPageTables = 1), so the coordinates
// of a numpy array can be read by a kernel directly, without the driver's
// staged pageable memcpy, and the reference's in-place centring can be
// written straight back into the caller's array.  Both kernels use plain
// 4-byte loads/stores (coalesced per warp); padding atoms of the device
// layout are written as zeros.  Where the device cannot access pageable
// memory the entry points refuse unregistered host pointers instead of
// touching them.
#include "capi_internal.h"
#include "common.cuh"

namespace gb {
namespace {

// dst row r (dst_pitch floats apart) = src row r (src_pitch floats apart),
// row_floats values, then zeros up to dst_fill floats.  One warp per row,
// U independent loads in flight per lane.
__global__ void __launch_bounds__(256) copy_rows_kernel(float* __restrict__ dst, int64_t dst_pitch,
                                                        const float* __restrict__ src, int64_t src_pitch,
                                                        int64_t row_floats, int64_t dst_fill, int64_t n_rows) {
  constexpr int U = 8;
  const int lane = threadIdx.x & 31;
  const int64_t W = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n_rows; r += W) {
    const float* s = src + r * src_pitch;
    float* d = dst + r * dst_pitch;
    const int32_t nr = (int32_t)row_floats, nf = (int32_t)dst_fill;
    int32_t i = lane;
    for (; i + 32 * (U - 1) < nr; i += 32 * U) {
      float v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] = s[i + 32 * u];
#pragma unroll
      for (int u = 0; u < U; ++u) d[i + 32 * u] = v[u];
    }
    for (; i < nr; i += 32) d[i] = s[i];
    for (int32_t j = nr + lane; j < nf; j += 32) d[j] = 0.f;
  }
}

// host[f][k][c] = dev[f][k][c] - centroid[f][c] for an atom-major device
// frame (dev_stride floats apart) written into an unpadded host frame.
__global__ void __launch_bounds__(256) write_centred_kernel(float* __restrict__ host, const float* __restrict__ dev,
                                                            int64_t dev_stride, const float* __restrict__ cent,
                                                            int64_t n_frames, int32_t n_atoms) {
  constexpr int U = 8;
  const int lane = threadIdx.x & 31;
  const int64_t W = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int32_t n = 3 * n_atoms;
  for (int64_t f = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); f < n_frames; f += W) {
    const float* s = dev + f * dev_stride;
    float* d = host + f * (int64_t)n;
    const float mu[3] = {cent[3 * f], cent[3 * f + 1], cent[3 * f + 2]};
    uint32_t i = lane;
    for (; i + 32 * (U - 1) < (uint32_t)n; i += 32 * U) {
      float v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] = s[i + 32 * u];
#pragma unroll
      for (int u = 0; u < U; ++u) d[i + 32 * u] = __fsub_rn(v[u], mu[(i + 32 * u) % 3u]);
    }
    for (; i < (uint32_t)n; i += 32) d[i] = __fsub_rn(s[i], mu[i % 3u]);
  }
}

int host_access_ok(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged || at.type == cudaMemoryTypeHost) return 1;
  // unregistered host memory: only through the host page tables
  int d = 0, pageable = 0;
  cudaGetDevice(&d);
  cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, d);
  return pageable == 1 ? 1 : 0;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

int gbrmsd_pageable_access(void) {
  int d = 0, pageable = 0, uses_pt = 0;
  if (cudaGetDevice(&d) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, d);
  cudaDeviceGetAttribute(&uses_pt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, d);
  return (pageable == 1 && uses_pt == 1) ? 1 : 0;
}

int gbrmsd_copy_rows_kernel(float* dst, int64_t dst_pitch, const float* src, int64_t src_pitch, int64_t row_floats,
                            int64_t dst_fill, int64_t n_rows, void* stream) {
  clear_error();
  if (n_rows <= 0) return GBRMSD_OK;
  if (!dst || !src) return set_error(GBRMSD_E_INVALID, "copy_rows_kernel: null pointer");
  if (row_floats < 0 || dst_fill < row_floats || dst_pitch < dst_fill || src_pitch < row_floats ||
      dst_fill > (1LL << 30))
    return set_error(GBRMSD_E_INVALID, "copy_rows_kernel: inconsistent pitches");
  if (!host_access_ok(src) || !host_access_ok(dst))
    return set_error(GBRMSD_E_UNSUPPORTED, "copy_rows_kernel: the device cannot access this host memory");
  const int grid = sm_count() * 8;
  copy_rows_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(dst, dst_pitch, src, src_pitch, row_floats,
                                                                        dst_fill, n_rows);
  GB_CUDA_TRY(cudaGetLastError(), "launch copy_rows_kernel");
  return GBRMSD_OK;
}

int gbrmsd_write_centred(float* host, const float* dev, int64_t dev_frame_stride, const float* centroids,
                         int64_t n_frames, int32_t n_atoms, void* stream) {
  clear_error();
  if (n_frames <= 0 || n_atoms <= 0) return GBRMSD_OK;
  if (!host || !dev || !centroids) return set_error(GBRMSD_E_INVALID, "write_centred: null pointer");
  if (dev_frame_stride < 3LL * n_atoms || n_atoms > (1 << 28))
    return set_error(GBRMSD_E_INVALID, "write_centred: bad frame stride / atom count");
  if (!host_access_ok(host))
    return set_error(GBRMSD_E_UNSUPPORTED, "write_centred: the device cannot access this host memory");
  const int grid = sm_count() * 8;
  write_centred_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(host, dev, dev_frame_stride, centroids,
                                                                            n_frames, n_atoms);
  GB_CUDA_TRY(cudaGetLastError(), "launch write_centred_kernel");
  return GBRMSD_OK;
}

}  // extern "C"
