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
//                         0.75 * scale / sqrt(n) (scale = (Ga + Gb) / 2n)
//                         are queued for allpairs_refine_kernel (marked NaN
//                         in the output when the queue is full).
//   allpairs_refine_kernel warp per queued (or marked) pair: compensated M,
//                         FP64 QCP, then the direct residual |R a_i - a_j|^2.
#include <cuda.h>
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

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

// Arguments of the FP32 tile kernel.  All-pairs: X32b == X32, one upper-
// triangle tile per CTA.  Cross: rows from a database set, columns from a
// query set, tiles from a list.
struct Fp32Args {
  const float* X32;   // row frames
  const double* G;
  int64_t F;          // row frames
  const float* X32b;  // column frames
  const double* Gb;
  int64_t Fb;         // column frames (capacity of the query set)
  int32_t A, kpad;
  int64_t nb;         // all-pairs: frame blocks per side
  float* out;         // all-pairs output
  const int2* tiles;  // cross: (row block, column block)
  const gbrmsd_cross_request_t* reqs;
  const int32_t* colreq;
  PairRefine* rl;
  int* rc;
  int rcap;
  int* err;
};

template <bool CROSS>
__global__ void __launch_bounds__(256, 1) allpairs_fp32_kernel(const Fp32Args p) {
  extern __shared__ __align__(16) float sm[];
  float* sA = sm;                                  // [2][TROWS][LDS_STRIDE]
  float* sB = sm + 2 * TROWS * LDS_STRIDE;         // [2][TROWS][LDS_STRIDE]
  int64_t bi, bj;
  if (CROSS) {
    const int2 t = p.tiles[blockIdx.x];
    bi = t.x;
    bj = t.y;
  } else {
    tri_tile(blockIdx.x, p.nb, bi, bj);
  }
  const float* __restrict__ X32 = p.X32;
  const float* __restrict__ X32b = p.X32b;
  const int32_t kpad = p.kpad;
  const int tid = threadIdx.x;
  const int ty = tid >> 4, tx = tid & 15;
  const int64_t rowsA = bi * TROWS, rowsB = bj * TROWS, nrows = 3 * p.F, nrowsb = 3 * p.Fb;

  auto load_block = [&](int buf, int kb) {
    for (int idx = tid; idx < TROWS * (KB / 4); idx += 256) {
      const int r = idx / (KB / 4), c4 = idx % (KB / 4);
      const int64_t ga = rowsA + r, gbr = rowsB + r;
      const size_t col = (size_t)kb * KB + 4 * c4;
      cp_async16(&sA[(buf * TROWS + r) * LDS_STRIDE + 4 * c4], X32 + (ga < nrows ? (size_t)ga * kpad + col : 0),
                 ga < nrows);
      cp_async16(&sB[(buf * TROWS + r) * LDS_STRIDE + 4 * c4], X32b + (gbr < nrowsb ? (size_t)gbr * kpad + col : 0),
                 gbr < nrowsb);
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

  const float inv_n = 1.0f / (float)p.A;
  if (CROSS) {
#pragma unroll
    for (int fb = 0; fb < 3; ++fb) {
      const int64_t j = bj * TBF + tx * 3 + fb;
      const CrossCol cv = cross_col(p.reqs, p.colreq, j, p.Fb);
      if (cv.row == nullptr) continue;
#pragma unroll
      for (int fa = 0; fa < 3; ++fa) {
        const int64_t i = bi * TBF + ty * 3 + fa;
        if (i >= cv.db0 && i < cv.db1 && i < p.F)
          cross_pair(i, j, acc[fa][fb], (float)p.G[i], (float)p.Gb[j], inv_n, cv.row + (i - cv.db0), p.rl, p.rc,
                     p.rcap, p.err);
      }
    }
  } else {
#pragma unroll
    for (int fa = 0; fa < 3; ++fa)
#pragma unroll
      for (int fb = 0; fb < 3; ++fb) {
        const int64_t i = bi * TBF + ty * 3 + fa, j = bj * TBF + tx * 3 + fb;
        if (i < p.F && j < p.F && i <= j)
          pair_epilogue(i, j, acc[fa][fb], p.G, inv_n, p.F, p.out, p.rl, p.rc, p.rcap, p.err);
      }
  }
}

// ---------------------------------------------------------------------------
// Refinement of near-identical pairs (warp per pair)
// ---------------------------------------------------------------------------

// One pair (i, j), the whole warp: compensated M, FP64 QCP, then the direct
// residual |R a_i - a_j|^2 with R rounded to float.  Cross: i indexes X32/G
// (database), j indexes X32b/Gb (query set) and the result goes to the
// request's output row; all-pairs: X32b == X32, both triangles written.
template <bool CROSS>
__device__ __forceinline__ void refine_pair(int64_t i, int64_t j, int lane, const float* __restrict__ X32,
                                            const double* __restrict__ G, int64_t F, int32_t A, int32_t kpad,
                                            float* __restrict__ out, const float* __restrict__ X32b,
                                            const double* __restrict__ Gb, int64_t Fb,
                                            const gbrmsd_cross_request_t* reqs, const int32_t* colreq) {
  const float* ai[3] = {X32 + (size_t)(3 * i) * kpad, X32 + (size_t)(3 * i + 1) * kpad, X32 + (size_t)(3 * i + 2) * kpad};
  const float* bj[3] = {X32b + (size_t)(3 * j) * kpad, X32b + (size_t)(3 * j + 1) * kpad,
                        X32b + (size_t)(3 * j + 2) * kpad};
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
  const double ga = G[i], gb = Gb[j];
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
    if (CROSS) {
      const CrossCol cv = cross_col(reqs, colreq, j, Fb);
      if (cv.row != nullptr) cv.row[i - cv.db0] = r;
    } else {
      out[i * F + j] = r;
      out[j * F + i] = r;
    }
  }
}

// Refinement, one warp per pair: first the queued pairs, then, when the
// list overflowed (count above rcap), every output slot holding the
// refine_marker() NaN -- all-pairs: the upper triangle row by row; cross:
// each request's output row by query column.  *refined receives the number
// of pairs refined by both.
template <bool CROSS>
__global__ void __launch_bounds__(256) allpairs_refine_kernel(const float* __restrict__ X32,
                                                              const double* __restrict__ G, int64_t F, int32_t A,
                                                              int32_t kpad, const PairRefine* rl, const int* rc,
                                                              int rcap, float* __restrict__ out,
                                                              const float* __restrict__ X32b,
                                                              const double* __restrict__ Gb, int64_t Fb,
                                                              const gbrmsd_cross_request_t* reqs,
                                                              const int32_t* colreq, unsigned long long* refined) {
  const int lane = threadIdx.x & 31;
  const int64_t W = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int n_all = *reinterpret_cast<const volatile int*>(rc);
  const int n = n_all < rcap ? n_all : rcap;
  if (gw == 0 && lane == 0 && n > 0) atomicAdd(refined, (unsigned long long)n);
  for (int64_t e = gw; e < n; e += W)
    refine_pair<CROSS>(rl[e].i, rl[e].j, lane, X32, G, F, A, kpad, out, X32b, Gb, Fb, reqs, colreq);
  if (n_all <= rcap) return;
  unsigned long long found = 0;
  if (!CROSS) {
    for (int64_t i = gw; i < F; i += W) {
      const float* row = out + i * F;
      for (int64_t j0 = i + 1; j0 < F; j0 += 32) {
        const int64_t j = j0 + lane;
        unsigned hit = __ballot_sync(FULL_MASK, j < F && isnan(row[j]));
        while (hit) {
          const int b = __ffs(hit) - 1;
          hit &= hit - 1;
          refine_pair<false>(i, j0 + b, lane, X32, G, F, A, kpad, out, X32b, Gb, Fb, reqs, colreq);
          ++found;
        }
      }
    }
  } else {
    for (int64_t j = gw; j < Fb; j += W) {
      const CrossCol cv = cross_col(reqs, colreq, j, Fb);
      if (cv.row == nullptr) continue;
      const int64_t end = cv.db1 < F ? cv.db1 : F;
      for (int64_t i0 = cv.db0; i0 < end; i0 += 32) {
        const int64_t i = i0 + lane;
        unsigned hit = __ballot_sync(FULL_MASK, i < end && isnan(cv.row[i - cv.db0]));
        while (hit) {
          const int b = __ffs(hit) - 1;
          hit &= hit - 1;
          refine_pair<true>(i0 + b, j, lane, X32, G, F, A, kpad, out, X32b, Gb, Fb, reqs, colreq);
          ++found;
        }
      }
    }
  }
  if (lane == 0 && found) atomicAdd(refined, found);
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
int launch_cross_tc(const __nv_bfloat16* Ahi, const __nv_bfloat16* Alo, const double* Ga, int64_t n_a, int64_t cap_a,
                    const __nv_bfloat16* Bhi, const __nv_bfloat16* Blo, const double* Gb, int64_t cap_b, int32_t A,
                    int32_t kpad, const gbrmsd_cross_request_t* reqs, const int32_t* colreq, const int2* tiles,
                    int64_t max_tiles, const int64_t* n_tiles_dev, PairRefine* rl, int* rc, int rcap, int* err,
                    cudaStream_t st);
int cross_tc_block_frames(int* rows, int* cols);

namespace {

// Frame set: [X32 (3 cap x kpad floats) | hi | lo (BF16) | G (cap doubles)].
struct FsLayout {
  size_t x32, hi, lo, g, total;
  int32_t kpad;
};

FsLayout fs_layout(int64_t cap, int32_t A) {
  FsLayout l;
  l.kpad = (A + 63) / 64 * 64;
  const size_t rows = (size_t)3 * (size_t)cap;
  l.x32 = 0;
  l.hi = align_up(rows * l.kpad * 4, 256);
  l.lo = align_up(l.hi + rows * l.kpad * 2, 256);
  l.g = align_up(l.lo + rows * l.kpad * 2, 256);
  l.total = align_up(l.g + (size_t)cap * 8, 256);
  return l;
}

// Cross workspace: [header | requests | column -> request | tiles | refinement list].
struct CrossWs {
  size_t reqs, colreq, tiles, rl, act, cnt, ntl, total;
  int64_t max_tiles;
  int rcap;
};

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

CrossWs cross_ws(int64_t n_db, int64_t qcap, int32_t n_req) {
  int fm = 1, fn = 1;
  cross_tc_block_frames(&fm, &fn);
  CrossWs w;
  w.max_tiles = std::max(ceil_div(n_db, fm) * ceil_div(qcap, fn), ceil_div(n_db, TBF) * ceil_div(qcap, TBF));
  w.reqs = 256;
  w.colreq = align_up(w.reqs + (size_t)n_req * sizeof(gbrmsd_cross_request_t), 256);
  w.tiles = align_up(w.colreq + (size_t)qcap * sizeof(int32_t), 256);
  w.rl = align_up(w.tiles + (size_t)w.max_tiles * sizeof(int2), 256);
  const int64_t pairs = n_db * qcap;
  w.rcap = (int)(pairs < (1 << 22) ? (pairs > 0 ? pairs : 1) : (1 << 22));
  // device tile builder: active column blocks (16 B each), per-row-block
  // counts / offsets, tile count
  w.act = align_up(w.rl + (size_t)w.rcap * sizeof(PairRefine), 256);
  w.cnt = align_up(w.act + (size_t)ceil_div(qcap, fn) * 16, 256);
  w.ntl = align_up(w.cnt + (size_t)(ceil_div(n_db, fm) + 1) * sizeof(int64_t), 256);
  w.total = align_up(w.ntl + sizeof(int64_t), 256);
  return w;
}

// Column blocks of a cross call that hold requested pairs, with the row
// blocks between the lowest and highest database frame their requests ask
// for (inclusive).
struct ActiveBlock {
  int32_t cb, lo, hi, pad;
};

struct CrossColumns {
  std::vector<int32_t> colreq;      // query row -> request (-1: none)
  std::vector<ActiveBlock> active;  // ascending column block
  int64_t rmin = 0, n_rb = 0;       // row blocks [rmin, rmin + n_rb)
  int64_t max_tiles = 0;            // n_rb * active.size(): an upper bound of the tile count
};

// Validates the requests and fills the column -> request map and the active
// column blocks.
int build_cross_columns(const gbrmsd_cross_request_t* reqs, int32_t n_req, int64_t n_db, int64_t qcap, int fr_rows,
                        int fr_cols, CrossColumns& cc) {
  cc.colreq.assign((size_t)qcap, -1);
  const int64_t ncb = ceil_div(qcap, fr_cols);
  std::vector<int64_t> lo((size_t)ncb, INT64_MAX), hi((size_t)ncb, -1);
  for (int32_t r = 0; r < n_req; ++r) {
    const gbrmsd_cross_request_t& q = reqs[r];
    if (q.n_query < 0 || q.pool0 < 0 || q.pool0 + q.n_query > qcap || q.db0 < 0 || q.db1 < q.db0 || q.db1 > n_db)
      return set_error(GBRMSD_E_INVALID,
                       "cross: request %d needs 0 <= pool0, pool0 + n_query <= query capacity and "
                       "0 <= db0 <= db1 <= n_db",
                       r);
    if (q.n_query == 0 || q.db1 == q.db0) continue;
    if (!q.out) return set_error(GBRMSD_E_INVALID, "cross: request %d has no output buffer", r);
    for (int64_t j = q.pool0; j < q.pool0 + q.n_query; ++j) {
      if (cc.colreq[(size_t)j] >= 0)
        return set_error(GBRMSD_E_INVALID, "cross: requests %d and %d share query row %lld", cc.colreq[(size_t)j], r,
                         (long long)j);
      cc.colreq[(size_t)j] = r;
    }
    const int64_t rb0 = q.db0 / fr_rows, rb1 = (q.db1 - 1) / fr_rows;
    for (int64_t cb = q.pool0 / fr_cols; cb <= (q.pool0 + q.n_query - 1) / fr_cols; ++cb) {
      lo[(size_t)cb] = std::min(lo[(size_t)cb], rb0);
      hi[(size_t)cb] = std::max(hi[(size_t)cb], rb1);
    }
  }
  cc.active.clear();
  int64_t rmin = INT64_MAX, rmax = -1;
  for (int64_t cb = 0; cb < ncb; ++cb)
    if (hi[(size_t)cb] >= 0) {
      cc.active.push_back(ActiveBlock{(int32_t)cb, (int32_t)lo[(size_t)cb], (int32_t)hi[(size_t)cb], 0});
      rmin = std::min(rmin, lo[(size_t)cb]);
      rmax = std::max(rmax, hi[(size_t)cb]);
    }
  cc.rmin = cc.active.empty() ? 0 : rmin;
  cc.n_rb = cc.active.empty() ? 0 : rmax - rmin + 1;
  cc.max_tiles = cc.n_rb * (int64_t)cc.active.size();
  return GBRMSD_OK;
}

// The (row block, column block) tiles that hold at least one requested pair,
// row-block-major so that CTAs running at the same time share database rows
// in L2.  Host version, for the FP32 tiles (whose grid is one CTA per tile).
void host_cross_tiles(const CrossColumns& cc, std::vector<int2>& tiles) {
  tiles.clear();
  for (int64_t i = 0; i < cc.n_rb; ++i) {
    const int64_t rb = cc.rmin + i;
    for (const ActiveBlock& b : cc.active)
      if (rb >= b.lo && rb <= b.hi) tiles.push_back(make_int2((int)rb, b.cb));
  }
}

// The same list built on the device (tensor path), so that neither the host
// loop over up to millions of tiles nor their pageable upload holds the host
// up: count the tiles of every row block, scan the counts, write each row
// block's tiles at its offset.  Same order as host_cross_tiles.
__global__ void __launch_bounds__(256) cross_tile_count_kernel(const ActiveBlock* __restrict__ act, int32_t n_act,
                                                              int64_t rmin, int64_t n_rb, int64_t* __restrict__ cnt) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_rb; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t rb = rmin + i;
    int64_t c = 0;
    for (int32_t k = 0; k < n_act; ++k) c += (rb >= act[k].lo && rb <= act[k].hi) ? 1 : 0;
    cnt[i] = c;
  }
}

// In-place exclusive scan of cnt[0, n) by one block; *total = the sum.
__global__ void __launch_bounds__(1024) cross_tile_scan_kernel(int64_t* __restrict__ cnt, int64_t n,
                                                              int64_t* __restrict__ total) {
  __shared__ int64_t part[1024];
  int64_t carry = 0;
  for (int64_t base = 0; base < n; base += 1024) {
    const int64_t i = base + threadIdx.x;
    const int64_t v = i < n ? cnt[i] : 0;
    part[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      const int64_t t = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
      __syncthreads();
      part[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n) cnt[i] = carry + part[threadIdx.x] - v;
    carry += part[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(256) cross_tile_fill_kernel(const ActiveBlock* __restrict__ act, int32_t n_act,
                                                             int64_t rmin, int64_t n_rb, const int64_t* __restrict__ off,
                                                             int2* __restrict__ tiles) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_rb; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t rb = rmin + i;
    int64_t p = off[i];
    for (int32_t k = 0; k < n_act; ++k)
      if (rb >= act[k].lo && rb <= act[k].hi) tiles[p++] = make_int2((int)rb, act[k].cb);
  }
}

}  // namespace

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
  // header: [0] error word, [1] list count (saturates near the list's
  // capacity), [2..3] pairs refined (list and overflow scan)
  int h[4] = {0, 0, 0, 0};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  GB_CUDA_TRY(cudaMemcpyAsync(h, ws, sizeof(h), cudaMemcpyDeviceToHost, st), "copy allpairs header");
  GB_CUDA_TRY(cudaStreamSynchronize(st), "sync");
  if (refined_pairs) {
    unsigned long long total;
    memcpy(&total, h + 2, sizeof(total));
    *refined_pairs = (int32_t)std::min<unsigned long long>(total, (unsigned long long)INT32_MAX);
  }
  if (h[0]) return set_error(GBRMSD_E_DEVICE, "allpairs device error word 0x%x (1 = wait expired)", h[0]);
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
  int* hdr = reinterpret_cast<int*>(w);  // [0] err, [1] list count, [2..3] pairs refined
  float* X32 = reinterpret_cast<float*>(w + L.x32);
  __nv_bfloat16* Xhi = reinterpret_cast<__nv_bfloat16*>(w + L.hi);
  __nv_bfloat16* Xlo = reinterpret_cast<__nv_bfloat16*>(w + L.lo);
  double* G = reinterpret_cast<double*>(w + L.g);
  PairRefine* rl = reinterpret_cast<PairRefine*>(w + L.rl);
  GB_CUDA_TRY(cudaMemsetAsync(hdr, 0, 16, st), "memset allpairs header");
  allpairs_prep_kernel<<<sm_count() * 8, 256, 0, st>>>(x, n_frames, n_atoms, n_padded, frame_stride, layout,
                                                       centre ? 1 : 0, kpad, X32, Xhi, Xlo, G);
  GB_CUDA_TRY(cudaGetLastError(), "launch allpairs_prep_kernel");
  if (method == 0) {
    const int64_t nb = (n_frames + TBF - 1) / TBF;
    const int64_t tiles = nb * (nb + 1) / 2;
    if (tiles > 0x7fffffffLL) return set_error(GBRMSD_E_INVALID, "allpairs: too many tiles");
    GB_CUDA_TRY(cudaFuncSetAttribute(allpairs_fp32_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     FP32_TILE_SMEM),
                "cudaFuncSetAttribute(allpairs_fp32_kernel)");
    Fp32Args fa;
    memset(&fa, 0, sizeof(fa));
    fa.X32 = X32;
    fa.G = G;
    fa.F = n_frames;
    fa.X32b = X32;
    fa.Gb = G;
    fa.Fb = n_frames;
    fa.A = n_atoms;
    fa.kpad = kpad;
    fa.nb = nb;
    fa.out = out;
    fa.rl = rl;
    fa.rc = hdr + 1;
    fa.rcap = L.rcap;
    fa.err = hdr;
    prof_begin(st);
    allpairs_fp32_kernel<false><<<(unsigned)tiles, 256, FP32_TILE_SMEM, st>>>(fa);
    GB_CUDA_TRY(cudaGetLastError(), "launch allpairs_fp32_kernel");
    prof_end(st);
  } else {
    prof_begin(st);
    const int rc = launch_allpairs_tc(Xhi, Xlo, G, n_frames, n_atoms, kpad, out, rl, hdr + 1, L.rcap, hdr, st);
    if (rc) return rc;
    prof_end(st);
  }
  allpairs_refine_kernel<false><<<sm_count() * 4, 256, 0, st>>>(X32, G, n_frames, n_atoms, kpad, rl, hdr + 1, L.rcap,
                                                                 out, X32, G, n_frames, nullptr, nullptr,
                                                                 reinterpret_cast<unsigned long long*>(hdr + 2));
  GB_CUDA_TRY(cudaGetLastError(), "launch allpairs_refine_kernel");
  return GBRMSD_OK;
}

size_t gbrmsd_frameset_bytes(int64_t capacity, int32_t n_atoms) {
  if (capacity < 0 || n_atoms < 1) return 0;
  return fs_layout(capacity, n_atoms).total;
}

int gbrmsd_frameset_prepare(const float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded,
                            int64_t frame_stride, int32_t layout, int32_t centre, void* set, int64_t capacity,
                            int64_t first, void* stream) {
  clear_error();
  if (n_frames < 0 || n_atoms < 1 || first < 0 || first + n_frames > capacity)
    return set_error(GBRMSD_E_INVALID, "frameset_prepare: need n_atoms >= 1 and 0 <= first <= first + n_frames <= capacity");
  if (layout != ATOM_MAJOR && layout != AXIS_MAJOR) return set_error(GBRMSD_E_INVALID, "frameset_prepare: bad layout");
  if (n_padded < n_atoms || frame_stride < 3LL * n_padded)
    return set_error(GBRMSD_E_INVALID, "frameset_prepare: n_padded / frame_stride too small");
  if (capacity > (1LL << 31) / 3) return set_error(GBRMSD_E_INVALID, "frameset_prepare: capacity too large");
  if (n_frames == 0) return GBRMSD_OK;
  if (!x || !set || !aligned16(set)) return set_error(GBRMSD_E_INVALID, "frameset_prepare: null or misaligned pointer");
  const FsLayout L = fs_layout(capacity, n_atoms);
  unsigned char* b = static_cast<unsigned char*>(set);
  const size_t row0 = (size_t)3 * (size_t)first * L.kpad;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t blocks = std::min<int64_t>((int64_t)sm_count() * 8, (n_frames + 7) / 8);
  allpairs_prep_kernel<<<(unsigned)blocks, 256, 0, st>>>(
      x, n_frames, n_atoms, n_padded, frame_stride, layout, centre ? 1 : 0, L.kpad,
      reinterpret_cast<float*>(b + L.x32) + row0, reinterpret_cast<__nv_bfloat16*>(b + L.hi) + row0,
      reinterpret_cast<__nv_bfloat16*>(b + L.lo) + row0, reinterpret_cast<double*>(b + L.g) + first);
  GB_CUDA_TRY(cudaGetLastError(), "launch frameset prep kernel");
  return GBRMSD_OK;
}

size_t gbrmsd_cross_workspace_bytes(int64_t n_db, int64_t query_capacity, int32_t n_requests) {
  if (n_db < 0 || query_capacity < 0 || n_requests < 0) return 0;
  return cross_ws(n_db, query_capacity, n_requests).total;
}

int gbrmsd_cross_rmsd(const void* db_set, int64_t db_capacity, int64_t n_db, const void* query_set,
                      int64_t query_capacity, int32_t n_atoms, const gbrmsd_cross_request_t* requests,
                      int32_t n_requests, int32_t method, void* ws, size_t ws_bytes, void* stream) {
  clear_error();
  if (n_atoms < 1 || n_db < 0 || n_db > db_capacity || query_capacity < 0 || n_requests < 0)
    return set_error(GBRMSD_E_INVALID, "cross: need n_atoms >= 1, 0 <= n_db <= db_capacity, query_capacity >= 0");
  if (db_capacity > (1LL << 31) / 3 || query_capacity > (1LL << 31) / 3)
    return set_error(GBRMSD_E_INVALID, "cross: set capacity too large");
  if (method != 0 && method != 1) return set_error(GBRMSD_E_INVALID, "cross: method must be 0 (fp32) or 1 (tensor)");
  if (n_requests > 0 && !requests) return set_error(GBRMSD_E_INVALID, "cross: null request table");
  if (!db_set || !query_set || !aligned16(db_set) || !aligned16(query_set))
    return set_error(GBRMSD_E_INVALID, "cross: null or misaligned frame set");
  const CrossWs W = cross_ws(n_db, query_capacity, n_requests);
  if (!ws || ws_bytes < W.total || !aligned16(ws))
    return set_error(GBRMSD_E_WORKSPACE, "cross: workspace needs %zu bytes", W.total);
  int fm = TBF, fn = TBF;
  if (method == 1) cross_tc_block_frames(&fm, &fn);
  CrossColumns cc;
  int rc = build_cross_columns(requests, n_requests, n_db, query_capacity, fm, fn, cc);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* w = static_cast<unsigned char*>(ws);
  int* hdr = reinterpret_cast<int*>(w);
  GB_CUDA_TRY(cudaMemsetAsync(hdr, 0, 16, st), "memset cross header");
  if (cc.max_tiles == 0) return GBRMSD_OK;
  auto* dreq = reinterpret_cast<gbrmsd_cross_request_t*>(w + W.reqs);
  auto* dcol = reinterpret_cast<int32_t*>(w + W.colreq);
  auto* dtiles = reinterpret_cast<int2*>(w + W.tiles);
  auto* rl = reinterpret_cast<PairRefine*>(w + W.rl);
  GB_CUDA_TRY(cudaMemcpyAsync(dreq, requests, sizeof(gbrmsd_cross_request_t) * n_requests, cudaMemcpyHostToDevice, st),
              "upload cross requests");
  GB_CUDA_TRY(cudaMemcpyAsync(dcol, cc.colreq.data(), sizeof(int32_t) * cc.colreq.size(), cudaMemcpyHostToDevice, st),
              "upload column map");
  std::vector<int2> tiles;  // host tile list (FP32 tiles only)
  int64_t* d_ntl = nullptr;
  if (method == 0) {
    host_cross_tiles(cc, tiles);
    GB_CUDA_TRY(cudaMemcpyAsync(dtiles, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice, st),
                "upload cross tiles");
  } else {
    auto* dact = reinterpret_cast<ActiveBlock*>(w + W.act);
    auto* dcnt = reinterpret_cast<int64_t*>(w + W.cnt);
    d_ntl = reinterpret_cast<int64_t*>(w + W.ntl);
    GB_CUDA_TRY(cudaMemcpyAsync(dact, cc.active.data(), sizeof(ActiveBlock) * cc.active.size(), cudaMemcpyHostToDevice,
                                st),
                "upload active column blocks");
    const int32_t n_act = (int32_t)cc.active.size();
    const int blocks = (int)std::min<int64_t>(ceil_div(cc.n_rb, 256), (int64_t)sm_count() * 4);
    cross_tile_count_kernel<<<blocks, 256, 0, st>>>(dact, n_act, cc.rmin, cc.n_rb, dcnt);
    cross_tile_scan_kernel<<<1, 1024, 0, st>>>(dcnt, cc.n_rb, d_ntl);
    cross_tile_fill_kernel<<<blocks, 256, 0, st>>>(dact, n_act, cc.rmin, cc.n_rb, dcnt, dtiles);
    GB_CUDA_TRY(cudaGetLastError(), "launch cross tile builder");
  }
  const FsLayout La = fs_layout(db_capacity, n_atoms), Lb = fs_layout(query_capacity, n_atoms);
  const unsigned char* a = static_cast<const unsigned char*>(db_set);
  const unsigned char* b = static_cast<const unsigned char*>(query_set);
  const float* X32a = reinterpret_cast<const float*>(a + La.x32);
  const float* X32b = reinterpret_cast<const float*>(b + Lb.x32);
  const double* Ga = reinterpret_cast<const double*>(a + La.g);
  const double* Gb = reinterpret_cast<const double*>(b + Lb.g);
  if (method == 0) {
    GB_CUDA_TRY(cudaFuncSetAttribute(allpairs_fp32_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     FP32_TILE_SMEM),
                "cudaFuncSetAttribute(cross_fp32_kernel)");
    Fp32Args fa;
    memset(&fa, 0, sizeof(fa));
    fa.X32 = X32a;
    fa.G = Ga;
    fa.F = n_db;
    fa.X32b = X32b;
    fa.Gb = Gb;
    fa.Fb = query_capacity;
    fa.A = n_atoms;
    fa.kpad = La.kpad;
    fa.tiles = dtiles;
    fa.reqs = dreq;
    fa.colreq = dcol;
    fa.rl = rl;
    fa.rc = hdr + 1;
    fa.rcap = W.rcap;
    fa.err = hdr;
    prof_begin(st);
    allpairs_fp32_kernel<true><<<(unsigned)tiles.size(), 256, FP32_TILE_SMEM, st>>>(fa);
    GB_CUDA_TRY(cudaGetLastError(), "launch cross_fp32_kernel");
    prof_end(st);
  } else {
    prof_begin(st);
    rc = launch_cross_tc(reinterpret_cast<const __nv_bfloat16*>(a + La.hi), reinterpret_cast<const __nv_bfloat16*>(a + La.lo),
                         Ga, n_db, db_capacity, reinterpret_cast<const __nv_bfloat16*>(b + Lb.hi),
                         reinterpret_cast<const __nv_bfloat16*>(b + Lb.lo), Gb, query_capacity, n_atoms, La.kpad, dreq,
                         dcol, dtiles, cc.max_tiles, d_ntl, rl, hdr + 1, W.rcap, hdr, st);
    if (rc) return rc;
    prof_end(st);
  }
  allpairs_refine_kernel<true><<<sm_count() * 4, 256, 0, st>>>(X32a, Ga, n_db, n_atoms, La.kpad, rl, hdr + 1, W.rcap,
                                                                nullptr, X32b, Gb, query_capacity, dreq, dcol,
                                                                reinterpret_cast<unsigned long long*>(hdr + 2));
  GB_CUDA_TRY(cudaGetLastError(), "launch cross refine kernel");
  return GBRMSD_OK;
}

}  // extern "C"
