// Host <-> device movement for the drop-in's host-buffer path.
//
// On GB300 the GPU reaches the Grace host's pageable memory through the
// host page tables over NVLink-C2C (cudaDevAttrPageableMemoryAccess = 1 with
// cudaDevAttrPageableMemoryAccessUsesHostPageTables = 1), so the coordinates
// of a numpy array can be read by a kernel directly, without the driver's
// staged pageable memcpy, and the reference's in-place centring can be
// written straight back into the caller's array.  Where the device cannot
// access pageable memory the entry points refuse unregistered host pointers
// instead of touching them.
//
// The host side of a copy is contiguous (rows of `row` floats back to back),
// so the kernels sweep it as one flat array: at any moment the whole grid
// works inside a window of a few MB of host memory, which keeps the
// translations of the link's page walks warm, and 16-byte accesses are used
// whenever rows and pointers allow.  The device side has rows `pitch` floats
// apart (the padded layout).  Measured on GB300 with 2.4 GB of pageable
// memory: one warp per row reached 188 GB/s host->device and 137 GB/s
// device->host; the flat 16-byte sweep 208 and 175 GB/s.  The grid is two
// blocks per SM so that an inbound copy, an outbound copy and the RMSD
// kernel of neighbouring chunks are resident together: both directions of
// the link then run at once (273 GB/s combined, against 208 GB/s when each
// copy kernel fills the GPU and they take turns).
#include "capi_internal.h"
#include "common.cuh"

namespace gb {
namespace {

constexpr int HOSTIO_THREADS = 256;
constexpr int HOSTIO_BLOCKS_PER_SM = 2;
constexpr int HOSTIO_UNROLL = 4;

template <int VEC>
struct VecT;
template <>
struct VecT<1> {
  using T = float;
};
template <>
struct VecT<4> {
  using T = float4;
};

__device__ __forceinline__ float sub_mu(float v, const float* mu, uint32_t c) { return __fsub_rn(v, mu[c]); }
__device__ __forceinline__ float4 sub_mu(float4 v, const float* mu, uint32_t c) {
  // 4 = 1 (mod 3): the four floats of a 16-byte group at row offset 4*o are
  // coordinates o, o+1, o+2, o (mod 3)
  const uint32_t c1 = c == 2 ? 0 : c + 1, c2 = c == 0 ? 2 : c - 1;
  return make_float4(__fsub_rn(v.x, mu[c]), __fsub_rn(v.y, mu[c1]), __fsub_rn(v.z, mu[c2]), __fsub_rn(v.w, mu[c]));
}

// INBOUND: pitched[r][o] = flat[r * row + o] for o < row, and zeros at
// [row, fill) of every pitched row.  Outbound: flat[r * row + o] =
// pitched[r][o] (- cent[r][o mod 3] with CENTRE).  Units of VEC floats:
// row, pitch and fill are given in those units; the zero fill in floats.
template <bool INBOUND, bool CENTRE, int VEC>
__global__ void __launch_bounds__(HOSTIO_THREADS) flat_rows_kernel(typename VecT<VEC>::T* __restrict__ pitched,
                                                                   int64_t pitch, typename VecT<VEC>::T* __restrict__ flat,
                                                                   int64_t row, int64_t n_rows,
                                                                   const float* __restrict__ cent, int32_t fill_floats) {
  using T = typename VecT<VEC>::T;
  constexpr int64_t CH = 32 * HOSTIO_UNROLL;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (int64_t)blockIdx.x * (HOSTIO_THREADS / 32) + (threadIdx.x >> 5);
  const int64_t W = (int64_t)gridDim.x * (HOSTIO_THREADS / 32);
  const int64_t total = row * n_rows;
  const uint32_t urow = (uint32_t)row;
  for (int64_t c0 = warp * CH; c0 < total; c0 += W * CH) {
    const int64_t r0 = c0 / row;
    const uint32_t o0 = (uint32_t)(c0 - r0 * row);
    T v[HOSTIO_UNROLL];
#pragma unroll
    for (int u = 0; u < HOSTIO_UNROLL; ++u) {
      const int64_t i = c0 + lane + 32 * u;
      if (i < total) {
        const uint32_t o = o0 + lane + 32 * u;
        const uint32_t q = o / urow;
        v[u] = INBOUND ? flat[i] : pitched[(r0 + q) * pitch + (o - q * urow)];
      }
    }
#pragma unroll
    for (int u = 0; u < HOSTIO_UNROLL; ++u) {
      const int64_t i = c0 + lane + 32 * u;
      if (i < total) {
        const uint32_t o = o0 + lane + 32 * u;
        const uint32_t q = o / urow;
        const uint32_t oo = o - q * urow;
        if (INBOUND) {
          pitched[(r0 + q) * pitch + oo] = v[u];
        } else if (CENTRE) {
          flat[i] = sub_mu(v[u], cent + 3 * (r0 + q), oo % 3u);
        } else {
          flat[i] = v[u];
        }
      }
    }
  }
  if (INBOUND && fill_floats > 0) {
    // padding of the pitched rows (at most a few floats per row)
    float* p = reinterpret_cast<float*>(pitched);
    const int64_t T0 = (int64_t)blockIdx.x * HOSTIO_THREADS + threadIdx.x;
    const int64_t NT = (int64_t)gridDim.x * HOSTIO_THREADS;
    const int64_t pad0 = row * VEC, pitchf = pitch * VEC;
    for (int64_t t = T0; t < n_rows * fill_floats; t += NT) {
      const int64_t r = t / fill_floats;
      p[r * pitchf + pad0 + (t - r * fill_floats)] = 0.f;
    }
  }
}

template <bool INBOUND, bool CENTRE>
void launch_flat(float* pitched, int64_t pitch, float* flat, int64_t row, int64_t n_rows, const float* cent,
                 int32_t fill_floats, cudaStream_t st) {
  const int grid = sm_count() * HOSTIO_BLOCKS_PER_SM;
  const bool vec = (row % 4 == 0) && (pitch % 4 == 0) && ((uintptr_t)pitched % 16 == 0) && ((uintptr_t)flat % 16 == 0);
  if (vec) {
    flat_rows_kernel<INBOUND, CENTRE, 4><<<grid, HOSTIO_THREADS, 0, st>>>(
        reinterpret_cast<float4*>(pitched), pitch / 4, reinterpret_cast<float4*>(flat), row / 4, n_rows, cent,
        fill_floats);
  } else {
    flat_rows_kernel<INBOUND, CENTRE, 1><<<grid, HOSTIO_THREADS, 0, st>>>(pitched, pitch, flat, row, n_rows, cent,
                                                                          fill_floats);
  }
}

// General strided rows (neither side contiguous): one warp per row.
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

int gbrmsd_host_register(void* p, size_t bytes) {
  clear_error();
  if (!p || bytes == 0) return set_error(GBRMSD_E_INVALID, "host_register: null pointer or empty range");
  const cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();  // not sticky: the caller continues on pageable access
    return set_error(GBRMSD_E_UNSUPPORTED, "host_register: %s", cudaGetErrorString(e));
  }
  return GBRMSD_OK;
}

int gbrmsd_host_unregister(void* p) {
  clear_error();
  if (!p) return set_error(GBRMSD_E_INVALID, "host_unregister: null pointer");
  const cudaError_t e = cudaHostUnregister(p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(GBRMSD_E_UNSUPPORTED, "host_unregister: %s", cudaGetErrorString(e));
  }
  return GBRMSD_OK;
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
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (src_pitch == row_floats) {
    launch_flat<true, false>(dst, dst_pitch, const_cast<float*>(src), row_floats, n_rows, nullptr,
                             (int32_t)(dst_fill - row_floats), st);
  } else if (dst_pitch == row_floats && dst_fill == row_floats) {
    launch_flat<false, false>(const_cast<float*>(src), src_pitch, dst, row_floats, n_rows, nullptr, 0, st);
  } else {
    copy_rows_kernel<<<sm_count() * 8, 256, 0, st>>>(dst, dst_pitch, src, src_pitch, row_floats, dst_fill, n_rows);
  }
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
  launch_flat<false, true>(const_cast<float*>(dev), dev_frame_stride, host, 3LL * n_atoms, n_frames, centroids, 0,
                           static_cast<cudaStream_t>(stream));
  GB_CUDA_TRY(cudaGetLastError(), "launch write_centred_kernel");
  return GBRMSD_OK;
}

}  // extern "C"
