// All-pairs RMSD matrix on GB300.
//
//   allpairs_prep_kernel  warp per frame: exact centroid (compensated sums),
//                         centred float rows X32[3i+c][k], trace G_i, and the
//                         split BF16 planes hi = bf16(x), lo = bf16(x - hi)
//                         used by the tensor-core kernel (allpairs_tc.cu).
//   allpairs_fp32_kernel  plain FP32 CUDA-core tiles (48 x 48 frames per
//                         CTA, 3 x 3 frames per thread, cp.async double
//                         buffering): the yardstick for the tensor path.
//   pair epilogue         FP32 QCP on the quartic normalised by its upper
//                         bound; msd = 2 lam0 (1 - x) / n.  Pairs closer than
//                         0.25 * scale / sqrt(n) (scale = (Ga + Gb) / 2n)
//                         are queued for allpairs_refine_kernel.
//   allpairs_refine_kernel warp per queued pair: compensated M, FP64 QCP,
//                         then the direct residual |R a_i - a_j|^2.
#include <cuda.h>
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include "allpairs.cuh"
#include "capi_internal.h"
#include "common.cuh"
#include "qcp.cuh"
#include "stream.cuh"

namespace gb {

size_t allpairs_tc_tiles_bytes(int64_t F);  // allpairs_tc.cu

namespace {

// ---------------------------------------------------------------------------
// Preparation
// ---------------------------------------------------------------------------

__device__ __forceinline__ float frame_coord(const float* fr, int32_t layout, int32_t Ap, int32_t k, int c) {
  return layout == ATOM_MAJOR ? fr[3 * k + c] : fr[(size_t)c * Ap + k];
}

__global__ void __launch_bounds__(256) allpairs_prep_kernel(const float* __restrict__ x, int64_t F, int32_t A,
                                                            int32_t Ap, int64_t fstride, int32_t layout,
                                                            int32_t centre, int32_t kpad, float* __restrict__ X32,
                                                            __nv_bfloat16* __restrict__ Xhi,
                                                            __nv_bfloat16* __restrict__ Xlo, double* __restrict__ G) {
  const int lane = threadIdx.x & 31;
  const int64_t W = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t f = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); f < F; f += W) {
    const float* fr = x + f * fstride;
    float mu[3] = {0.f, 0.f, 0.f};
    if (centre) {
      CF s[3] = {cf_zero(), cf_zero(), cf_zero()};
      for (int32_t k = lane; k < A; k += 32)
        for (int c = 0; c < 3; ++c) cf_add(s[c], frame_coord(fr, layout, Ap, k, c));
      for (int c = 0; c < 3; ++c) {
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) {
          CF o;
          o.hi = __shfl_xor_sync(FULL_MASK, s[c].hi, m);
          o.lo = __shfl_xor_sync(FULL_MASK, s[c].lo, m);
          s[c] = cf_add2(s[c], o);
        }
        mu[c] = (float)(cf_to_double(s[c]) / (double)A);
      }
    }
    CF g = cf_zero();
    for (int32_t k = lane; k < kpad; k += 32) {
      for (int c = 0; c < 3; ++c) {
        float v = 0.f;
        if (k < A) v = __fsub_rn(frame_coord(fr, layout, Ap, k, c), mu[c]);
        const size_t idx = (size_t)(3 * f + c) * kpad + k;
        X32[idx] = v;
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        Xhi[idx] = h;
        Xlo[idx] = __float2bfloat16_rn(__fsub_rn(v, __bfloat162float(h)));
        cf_add(g, __fmul_rn(v, v));
      }
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
      CF o;
      o.hi = __shfl_xor_sync(FULL_MASK, g.hi, m);
      o.lo = __shfl_xor_sync(FULL_MASK, g.lo, m);
      g = cf_add2(g, o);
    }
    if (lane == 0) G[f] = cf_to_double(g);
  }
}

// ---------------------------------------------------------------------------
// FP32 CUDA-core tiles
// ---------------------------------------------------------------------------

constexpr int TBF = 48;            // frames per tile side
constexpr int TROWS = 3 * TBF;     // rows of X per tile side
constexpr int KB = 32;             // atoms per k block
constexpr int LDS_STRIDE = KB + 4; // padded shared row (floats): conflict-free float4 reads
constexpr int FP32_TILE_SMEM = 2 * 2 * TROWS * LDS_STRIDE * 4;

__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  const uint32_t d = smem_addr(dst);
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Upper-triangle tile t -> (bi, bj), bi <= bj, row-major over bi.
__device__ __forceinline__ void tri_tile(int64_t t, int64_t nb, int64_t& bi, int64_t& bj) {
  const double b = 2.0 * (double)nb + 1.0;
  int64_t r = (int64_t)floor((b - sqrt(b * b - 8.0 * (double)t)) * 0.5);
  if (r < 0) r = 0;
  if (r > nb - 1) r = nb - 1;
  auto start = [nb](int64_t q) { return q * nb - q * (q - 1) / 2; };
  while (r > 0 && start(r) > t) --r;
  while (r + 1 < nb && start(r + 1) <= t) ++r;
  bi = r;
  bj = r + (t - start(r));
}

__global__ void __launch_bounds__(256, 1) allpairs_fp32_kernel(const float* __restrict__ X32,
                                                               const double* __restrict__ G, int64_t F, int32_t A,
                                                               int32_t kpad, int64_t nb, float* __restrict__ out,
                                                               PairRefine* rl, int* rc, int rcap, int* err) {
  extern __shared__ __align__(16) float sm[];
  float* sA = sm;                                  // [2][TROWS][LDS_STRIDE]
  float* sB = sm + 2 * TROWS * LDS_STRIDE;         // [2][TROWS][LDS_STRIDE]
  int64_t bi, bj;
  tri_tile(blockIdx.x, nb, bi, bj);
  const int tid = threadIdx.x;
  const int ty = tid >> 4, tx = tid & 15;
  const int64_t rowsA = bi * TROWS, rowsB = bj * TROWS, nrows = 3 * F;

  auto load_block = [&](int buf, int kb) {
    for (int idx = tid; idx < TROWS * (KB / 4); idx += 256) {
      const int r = idx / (KB / 4), c4 = idx % (KB / 4);
      const int64_t ga = rowsA + r, gbr = rowsB + r;
      const size_t col = (size_t)kb * KB + 4 * c4;
      cp_async16(&sA[(buf * TROWS + r) * LDS_STRIDE + 4 * c4], X32 + (ga < nrows ? (size_t)ga * kpad + col : 0),
                 ga < nrows);
      cp_async16(&sB[(buf * TROWS + r) * LDS_STRIDE + 4 * c4], X32 + (gbr < nrows ? (size_t)gbr * kpad + col : 0),
                 gbr < nrows);
    }
    cp_async_commit();
  };

  float acc[3][3][9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int t = 0; t < 9; ++t) acc[a][b][t] = 0.f;

  const int nkb = kpad / KB;
  load_block(0, 0);
  for (int kb = 0; kb < nkb; ++kb) {
    const int buf = kb & 1;
    cp_async_wait0();
    __syncthreads();
    if (kb + 1 < nkb) load_block(buf ^ 1, kb + 1);
    const float* pa = &sA[(buf * TROWS + ty * 9) * LDS_STRIDE];
    const float* pb = &sB[(buf * TROWS + tx * 9) * LDS_STRIDE];
#pragma unroll 2
    for (int kk = 0; kk < KB; kk += 4) {
      float4 a[9], b[9];
#pragma unroll
      for (int r = 0; r < 9; ++r) {
        a[r] = *reinterpret_cast<const float4*>(pa + r * LDS_STRIDE + kk);
        b[r] = *reinterpret_cast<const float4*>(pb + r * LDS_STRIDE + kk);
      }
#pragma unroll
      for (int fa = 0; fa < 3; ++fa)
#pragma unroll
        for (int fb = 0; fb < 3; ++fb)
#pragma unroll
          for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
              float s = acc[fa][fb][3 * c + d];
              const float4 u = a[3 * fa + c], v = b[3 * fb + d];
              s = fmaf(u.x, v.x, s);
              s = fmaf(u.y, v.y, s);
              s = fmaf(u.z, v.z, s);
              s = fmaf(u.w, v.w, s);
              acc[fa][fb][3 * c + d] = s;
            }
    }
    __syncthreads();
  }

  const float inv_n = 1.0f / (float)A;
#pragma unroll
  for (int fa = 0; fa < 3; ++fa)
#pragma unroll
    for (int fb = 0; fb < 3; ++fb) {
      const int64_t i = bi * TBF + ty * 3 + fa, j = bj * TBF + tx * 3 + fb;
      if (i < F && j < F && i <= j) pair_epilogue(i, j, acc[fa][fb], G, inv_n, F, out, rl, rc, rcap, err);
    }
}

// ---------------------------------------------------------------------------
// Refinement of near-identical pairs (warp per pair)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) allpairs_refine_kernel(const float* __restrict__ X32,
                                                              const double* __restrict__ G, int64_t F, int32_t A,
                                                              int32_t kpad, const PairRefine* rl, const int* rc,
                                                              int rcap, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t W = (int64_t)gridDim.x * (blockDim.x >> 5);
  int n = *reinterpret_cast<const volatile int*>(rc);
  if (n > rcap) n = rcap;
  for (int64_t e = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < n; e += W) {
    const int64_t i = rl[e].i, j = rl[e].j;
    const float* ai[3] = {X32 + (size_t)(3 * i) * kpad, X32 + (size_t)(3 * i + 1) * kpad, X32 + (size_t)(3 * i + 2) * kpad};
    const float* bj[3] = {X32 + (size_t)(3 * j) * kpad, X32 + (size_t)(3 * j + 1) * kpad, X32 + (size_t)(3 * j + 2) * kpad};
    // compensated 3x3 inner product
    CF v[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) v[t] = cf_zero();
    for (int32_t k0 = 0; k0 < A; k0 += 32 * 4) {
      float part[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int32_t k = k0 + lane + 32 * u;
        if (k < A) {
          const float a[3] = {ai[0][k], ai[1][k], ai[2][k]};
          const float b[3] = {bj[0][k], bj[1][k], bj[2][k]};
#pragma unroll
          for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int d = 0; d < 3; ++d) part[3 * c + d] = fmaf(a[c], b[d], part[3 * c + d]);
        }
      }
#pragma unroll
      for (int t = 0; t < 9; ++t) cf_add(v[t], part[t]);
    }
    warp_xpose_reduce16(v, lane);
    double m[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const float hi = __shfl_sync(FULL_MASK, v[0].hi, 2 * t);
      const float lo = __shfl_sync(FULL_MASK, v[0].lo, 2 * t);
      m[t] = (double)hi + (double)lo;
    }
    const double ga = G[i], gb = G[j];
    int iters = 0;
    const double lam = qcp_lambda_max(m, ga, gb, &iters);
    double rot[9];
    qcp_rotation(m, lam, rot);
    float R[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) R[t] = (float)rot[t];
    CF acc = cf_zero();
    for (int32_t k0 = 0; k0 < A; k0 += 32 * 4) {
      float part = 0.f;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int32_t k = k0 + lane + 32 * u;
        if (k < A) {
          const float a0 = ai[0][k], a1 = ai[1][k], a2 = ai[2][k];
          const float rx = fmaf(R[0], a0, fmaf(R[1], a1, R[2] * a2)) - bj[0][k];
          const float ry = fmaf(R[3], a0, fmaf(R[4], a1, R[5] * a2)) - bj[1][k];
          const float rz = fmaf(R[6], a0, fmaf(R[7], a1, R[8] * a2)) - bj[2][k];
          part = fmaf(rx, rx, fmaf(ry, ry, fmaf(rz, rz, part)));
        }
      }
      cf_add(acc, part);
    }
#pragma unroll
    for (int mm = 16; mm >= 1; mm >>= 1) {
      CF o;
      o.hi = __shfl_xor_sync(FULL_MASK, acc.hi, mm);
      o.lo = __shfl_xor_sync(FULL_MASK, acc.lo, mm);
      acc = cf_add2(acc, o);
    }
    if (lane == 0) {
      double msd = cf_to_double(acc) / (double)A;
      if (!(msd > 0.0)) msd = 0.0;
      const float r = (float)sqrt(msd);
      out[i * F + j] = r;
      out[j * F + i] = r;
    }
  }
}

struct ApWs {
  size_t x32, hi, lo, g, rl, total;
  int rcap;
};

ApWs ap_ws(int64_t F, int32_t A) {
  const int32_t kpad = (A + 63) / 64 * 64;
  const size_t rows = (size_t)3 * F;
  ApWs w;
  w.x32 = 256;
  w.hi = align_up(w.x32 + rows * kpad * 4, 256);
  w.lo = align_up(w.hi + rows * kpad * 2, 256);
  w.g = align_up(w.lo + rows * kpad * 2, 256);
  w.rl = align_up(w.g + (size_t)F * 8, 256);
  const int64_t pairs = F * (F - 1) / 2;
  w.rcap = (int)(pairs < (1 << 22) ? (pairs > 0 ? pairs : 1) : (1 << 22));
  w.total = align_up(w.rl + (size_t)w.rcap * sizeof(PairRefine), 256) + allpairs_tc_tiles_bytes(F);
  return w;
}

}  // namespace

// Implemented in allpairs_tc.cu: split-BF16 tcgen05 tiles.
int launch_allpairs_tc(const __nv_bfloat16* Xhi, const __nv_bfloat16* Xlo, const double* G, int64_t F, int32_t A,
                       int32_t kpad, float* out, PairRefine* rl, int* rc, int rcap, int* err, cudaStream_t st);

}  // namespace gb

using namespace gb;

extern "C" {

size_t gbrmsd_allpairs_workspace_bytes(int64_t n_frames, int32_t n_atoms) {
  if (n_frames < 0 || n_atoms < 0) return 0;
  return ap_ws(n_frames, n_atoms).total;
}

int gbrmsd_allpairs_status(const void* ws, int32_t* refined_pairs, void* stream) {
  clear_error();
  if (!ws) return set_error(GBRMSD_E_INVALID, "allpairs_status: null workspace");
  int h[2] = {0, 0};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  GB_CUDA_TRY(cudaMemcpyAsync(h, ws, sizeof(h), cudaMemcpyDeviceToHost, st), "copy allpairs header");
  GB_CUDA_TRY(cudaStreamSynchronize(st), "sync");
  if (refined_pairs) *refined_pairs = h[1];
  if (h[0]) return set_error(GBRMSD_E_DEVICE, "allpairs device error word 0x%x (1 = wait expired, 4 = refinement list full)", h[0]);
  return GBRMSD_OK;
}

int gbrmsd_allpairs(const float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded, int64_t frame_stride,
                    int32_t layout, int32_t centre, int32_t method, float* out, void* ws, size_t ws_bytes,
                    void* stream) {
  clear_error();
  if (n_frames < 0 || n_atoms < 0) return set_error(GBRMSD_E_INVALID, "allpairs: negative sizes");
  if (layout != ATOM_MAJOR && layout != AXIS_MAJOR) return set_error(GBRMSD_E_INVALID, "allpairs: bad layout");
  if (n_padded < n_atoms || frame_stride < 3LL * n_padded)
    return set_error(GBRMSD_E_INVALID, "allpairs: n_padded / frame_stride too small");
  if (method != 0 && method != 1) return set_error(GBRMSD_E_INVALID, "allpairs: method must be 0 (fp32) or 1 (tensor)");
  if (n_frames > (1LL << 31) / 3) return set_error(GBRMSD_E_INVALID, "allpairs: too many frames");
  if (n_frames == 0) return GBRMSD_OK;
  if (!x || !out) return set_error(GBRMSD_E_INVALID, "allpairs: null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_atoms == 0) {
    GB_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * n_frames * n_frames, st), "memset out");
    return GBRMSD_OK;
  }
  const ApWs L = ap_ws(n_frames, n_atoms);
  if (!ws || ws_bytes < L.total || !aligned16(ws))
    return set_error(GBRMSD_E_WORKSPACE, "allpairs: workspace needs %zu bytes", L.total);
  const int32_t kpad = (n_atoms + 63) / 64 * 64;
  unsigned char* w = static_cast<unsigned char*>(ws);
  int* hdr = reinterpret_cast<int*>(w);  // [0] err, [1] refine count
  float* X32 = reinterpret_cast<float*>(w + L.x32);
  __nv_bfloat16* Xhi = reinterpret_cast<__nv_bfloat16*>(w + L.hi);
  __nv_bfloat16* Xlo = reinterpret_cast<__nv_bfloat16*>(w + L.lo);
  double* G = reinterpret_cast<double*>(w + L.g);
  PairRefine* rl = reinterpret_cast<PairRefine*>(w + L.rl);
  GB_CUDA_TRY(cudaMemsetAsync(hdr, 0, 8, st), "memset allpairs header");
  allpairs_prep_kernel<<<sm_count() * 8, 256, 0, st>>>(x, n_frames, n_atoms, n_padded, frame_stride, layout,
                                                       centre ? 1 : 0, kpad, X32, Xhi, Xlo, G);
  GB_CUDA_TRY(cudaGetLastError(), "launch allpairs_prep_kernel");
  if (method == 0) {
    const int64_t nb = (n_frames + TBF - 1) / TBF;
    const int64_t tiles = nb * (nb + 1) / 2;
    if (tiles > 0x7fffffffLL) return set_error(GBRMSD_E_INVALID, "allpairs: too many tiles");
    GB_CUDA_TRY(cudaFuncSetAttribute(allpairs_fp32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, FP32_TILE_SMEM),
                "cudaFuncSetAttribute(allpairs_fp32_kernel)");
    prof_begin(st);
    allpairs_fp32_kernel<<<(unsigned)tiles, 256, FP32_TILE_SMEM, st>>>(X32, G, n_frames, n_atoms, kpad, nb, out, rl,
                                                                       hdr + 1, L.rcap, hdr);
    GB_CUDA_TRY(cudaGetLastError(), "launch allpairs_fp32_kernel");
    prof_end(st);
  } else {
    prof_begin(st);
    const int rc = launch_allpairs_tc(Xhi, Xlo, G, n_frames, n_atoms, kpad, out, rl, hdr + 1, L.rcap, hdr, st);
    if (rc) return rc;
    prof_end(st);
  }
  allpairs_refine_kernel<<<sm_count() * 4, 256, 0, st>>>(X32, G, n_frames, n_atoms, kpad, rl, hdr + 1, L.rcap, out);
  GB_CUDA_TRY(cudaGetLastError(), "launch allpairs_refine_kernel");
  return GBRMSD_OK;
}

}  // extern "C"
