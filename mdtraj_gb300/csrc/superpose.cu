// Superposition on GB300: applying per-frame rotations, RMSF, and the
// rotated (align-on-one-set, measure-on-another) MSD.
//
//   apply_rotations_kernel  x <- R_f (x - mu_f) + offset for every atom of every
//                           frame, in place (Trajectory.superpose,
//                           mdtraj/core/trajectory.py:1127-1165, with
//                           rot_atom_major, src/rotation_generic.h:29-44)
//   rmsf_partial_kernel     per (frame chunk, atom): compensated sums of the
//   rmsf_final_kernel       rotated positions about a per-atom shift, then the
//                           mean and mean squared deviation per atom (rmsf,
//                           mdtraj/rmsd/_rmsd.pyx:419-451)
//   rotated_msd_kernel      warp per frame: sum |R_f a_k - b_k|^2 / n
//                           (rot_msd_atom_major, src/rotation_generic.h:47-103,
//                           as used by getMultipleAlignDisplaceRMSDs_atom_major,
//                           _rmsd.pyx:677-759)
//   center_weighted_kernel  warp per frame: x <- x - sum_k w_k x_k in place
//                           (Trajectory.center_coordinates(mass_weighted=True),
//                           mdtraj/core/trajectory.py:2133-2134)
//
// Rotations come from gbrmsd_rotations (row-major R, aligned = R x).  All
// four kernels are HBM-bound streaming passes over float32 coordinates.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "capi_internal.h"
#include "common.cuh"

namespace gb {
namespace {

// float(double(x) + d) computed in FP32 from the split d = hi + lo (hi =
// float(d), lo = float(d - hi)): within one float ulp of the FP64 form and free
// of GB300's slow FP64 pipe.
__device__ __forceinline__ float add_split(float x, float hi, float lo) { return (x + hi) + lo; }

constexpr int APPLY_THREADS = 128;

// Per-frame constants of the apply pass: R and -mu split into float hi + lo.
struct ApplyFrame {
  float r[9];
  float mh[3], ml[3];
};

__device__ __forceinline__ void apply_one(const ApplyFrame& p, const float (&oh)[3], const float (&ol)[3], float& x,
                                          float& y, float& z, bool& nz) {
  const float dx = add_split(x, p.mh[0], p.ml[0]);
  const float dy = add_split(y, p.mh[1], p.ml[1]);
  const float dz = add_split(z, p.mh[2], p.ml[2]);
  const float rx = fmaf(p.r[0], dx, fmaf(p.r[1], dy, p.r[2] * dz));
  const float ry = fmaf(p.r[3], dx, fmaf(p.r[4], dy, p.r[5] * dz));
  const float rz = fmaf(p.r[6], dx, fmaf(p.r[7], dy, p.r[8] * dz));
  nz = nz || (rx != 0.f) || (ry != 0.f) || (rz != 0.f);
  x = add_split(rx, oh[0], ol[0]);
  y = add_split(ry, oh[1], ol[1]);
  z = add_split(rz, oh[2], ol[2]);
}

// One CTA per (frame, block of 4 * APPLY_THREADS atoms); each thread moves one
// 4-atom quad with three 128-bit loads and stores when the frame is 16-byte
// aligned (VEC), else atom by atom.
template <bool VEC>
__global__ void __launch_bounds__(APPLY_THREADS) apply_rotations_kernel(float* __restrict__ x, int64_t F, int32_t A,
                                                                       int64_t fs, const float* __restrict__ rot,
                                                                       const double* __restrict__ mu, float oh0,
                                                                       float oh1, float oh2, float ol0, float ol1,
                                                                       float ol2, int32_t* nonzero0) {
  __shared__ ApplyFrame sp;
  constexpr int ATOMS_PER_CTA = 4 * APPLY_THREADS;
  const int32_t nab = (A + ATOMS_PER_CTA - 1) / ATOMS_PER_CTA;
  const int64_t f = blockIdx.x / nab;
  const int32_t k0 = (int32_t)(blockIdx.x - f * nab) * ATOMS_PER_CTA;
  if (threadIdx.x < 9) sp.r[threadIdx.x] = rot[9 * f + threadIdx.x];
  if (threadIdx.x >= 16 && threadIdx.x < 19) {
    const int c = threadIdx.x - 16;
    const double m = mu ? mu[3 * f + c] : 0.0;
    const float hi = -(float)m;
    sp.mh[c] = hi;
    sp.ml[c] = -(float)(m + (double)hi);
  }
  __syncthreads();
  const float oh[3] = {oh0, oh1, oh2}, ol[3] = {ol0, ol1, ol2};
  bool nz = false;
  float* fr = x + f * fs;
  const int32_t k = k0 + 4 * threadIdx.x;
  if (VEC && k + 3 < A) {
    float4* q = reinterpret_cast<float4*>(fr + 3 * (int64_t)k);
    float4 a = q[0], b = q[1], c = q[2];
    apply_one(sp, oh, ol, a.x, a.y, a.z, nz);
    apply_one(sp, oh, ol, a.w, b.x, b.y, nz);
    apply_one(sp, oh, ol, b.z, b.w, c.x, nz);
    apply_one(sp, oh, ol, c.y, c.z, c.w, nz);
    q[0] = a;
    q[1] = b;
    q[2] = c;
  } else {
    for (int t = 0; t < 4; ++t) {
      if (k + t < A) {
        float* p = fr + 3 * (int64_t)(k + t);
        float px = p[0], py = p[1], pz = p[2];
        apply_one(sp, oh, ol, px, py, pz, nz);
        p[0] = px;
        p[1] = py;
        p[2] = pz;
      }
    }
  }
  if (nonzero0 && f == 0 && __any_sync(FULL_MASK, nz) && (threadIdx.x & 31) == 0) atomicOr(nonzero0, 1);
}

// ---- RMSF ---------------------------------------------------------------

constexpr int RMSF_THREADS = 128;
constexpr int RMSF_FOLD = 16;  // frames per FP32 partial before it is folded into a TwoSum pair

__device__ __forceinline__ void rotate(const float* r, float ax, float ay, float az, float& bx, float& by, float& bz) {
  bx = fmaf(r[0], ax, fmaf(r[1], ay, r[2] * az));
  by = fmaf(r[3], ax, fmaf(r[4], ay, r[5] * az));
  bz = fmaf(r[6], ax, fmaf(r[7], ay, r[8] * az));
}

constexpr int RMSF_ILP = 4;  // frames whose loads a thread issues together

// One frame of an atom: d = R x - s (or x - s without a rotation) added to
// the FP32 partial sums a[0..2] and |d|^2 to a[3].
__device__ __forceinline__ void rmsf_accum(const float* r, float px, float py, float pz, const float (&s)[3],
                                           float (&a)[4]) {
  float bx = px, by = py, bz = pz;
  if (r) rotate(r, px, py, pz, bx, by, bz);
  const float dx = bx - s[0], dy = by - s[1], dz = bz - s[2];
  a[0] += dx;
  a[1] += dy;
  a[2] += dz;
  a[3] = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, a[3])));
}

// part[(chunk * A + k) * 4 + {0,1,2,3}] = sums over the chunk's frames of
// d = R_f x_fk - s_k (3 components) and |d|^2, s_k = R_0 x_0k.
__global__ void __launch_bounds__(RMSF_THREADS) rmsf_partial_kernel(const float* __restrict__ x, int64_t F, int32_t A,
                                                                   int64_t fs, const float* __restrict__ rot,
                                                                   int64_t fch, double* __restrict__ part) {
  __shared__ float sr[RMSF_FOLD * 9];
  const int32_t k = blockIdx.x * RMSF_THREADS + threadIdx.x;
  const int64_t f0 = (int64_t)blockIdx.y * fch;
  const int64_t f1 = min(F, f0 + fch);
  float s[3] = {0.f, 0.f, 0.f};
  if (k < A) {
    const float* p = x + 3 * (int64_t)k;
    if (rot) rotate(rot, p[0], p[1], p[2], s[0], s[1], s[2]);
    else { s[0] = p[0]; s[1] = p[1]; s[2] = p[2]; }
  }
  CF acc[4] = {cf_zero(), cf_zero(), cf_zero(), cf_zero()};
  for (int64_t fb = f0; fb < f1; fb += RMSF_FOLD) {
    const int nf = (int)(f1 - fb < RMSF_FOLD ? f1 - fb : RMSF_FOLD);
    __syncthreads();
    if (rot)
      for (int t = threadIdx.x; t < nf * 9; t += RMSF_THREADS) sr[t] = rot[9 * fb + t];
    __syncthreads();
    float a[4] = {0.f, 0.f, 0.f, 0.f};
    if (k < A) {
      // frames in groups of RMSF_ILP: all their loads are issued before any
      // is used, so a thread keeps RMSF_ILP frames in flight (one at a time
      // left the pass latency-bound at ~4 TB/s); the sums still run in frame
      // order, so the results do not change
      int i = 0;
      for (; i + RMSF_ILP <= nf; i += RMSF_ILP) {
        float px[RMSF_ILP], py[RMSF_ILP], pz[RMSF_ILP];
#pragma unroll
        for (int u = 0; u < RMSF_ILP; ++u) {
          const float* p = x + (fb + i + u) * fs + 3 * (int64_t)k;
          px[u] = p[0];
          py[u] = p[1];
          pz[u] = p[2];
        }
#pragma unroll
        for (int u = 0; u < RMSF_ILP; ++u)
          rmsf_accum(rot ? sr + 9 * (i + u) : nullptr, px[u], py[u], pz[u], s, a);
      }
      for (; i < nf; ++i) {
        const float* p = x + (fb + i) * fs + 3 * (int64_t)k;
        rmsf_accum(rot ? sr + 9 * i : nullptr, p[0], p[1], p[2], s, a);
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) cf_add(acc[j], a[j]);
  }
  if (k < A) {
    double* o = part + ((int64_t)blockIdx.y * A + k) * 4;
#pragma unroll
    for (int j = 0; j < 4; ++j) o[j] = cf_to_double(acc[j]);
  }
}

__global__ void __launch_bounds__(256) rmsf_final_kernel(const double* __restrict__ part, int32_t n_chunks, int32_t A,
                                                        int64_t F, float* __restrict__ out) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A) return;
  double t[4] = {0.0, 0.0, 0.0, 0.0};
  for (int32_t c = 0; c < n_chunks; ++c)
    for (int j = 0; j < 4; ++j) t[j] += part[((int64_t)c * A + k) * 4 + j];
  const double inv = 1.0 / (double)F;
  const double mx = t[0] * inv, my = t[1] * inv, mz = t[2] * inv;
  double var = t[3] * inv - (mx * mx + my * my + mz * mz);
  if (!(var > 0.0)) var = 0.0;
  out[k] = (float)sqrt(var);
}

struct RmsfPlan {
  int64_t fch;
  int32_t n_chunks;
  size_t bytes;
};

RmsfPlan rmsf_plan(int64_t F, int32_t A) {
  RmsfPlan p;
  // enough frame chunks to fill the GPU when there are few atoms, at most 65,535
  const int64_t atom_blocks = ((int64_t)A + RMSF_THREADS - 1) / RMSF_THREADS;
  int64_t want = (8LL * 152 + atom_blocks - 1) / (atom_blocks > 0 ? atom_blocks : 1);
  if (want < 1) want = 1;
  int64_t fch = (F + want - 1) / want;
  if (fch < 64) fch = 64;
  if ((F + fch - 1) / fch > 65535) fch = (F + 65534) / 65535;
  p.fch = fch;
  p.n_chunks = (int32_t)((F + fch - 1) / fch);
  if (p.n_chunks < 1) p.n_chunks = 1;
  p.bytes = align_up((size_t)p.n_chunks * (size_t)A * 4 * sizeof(double), 256);
  return p;
}

// ---- rotated MSD (align-displace) -----------------------------------------

__global__ void __launch_bounds__(256) rotated_msd_kernel(const float* __restrict__ x, int64_t F, int32_t A,
                                                         int64_t fs, const float* __restrict__ rot,
                                                         const float* __restrict__ ref, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t W = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t f = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); f < F; f += W) {
    float r[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) r[i] = rot[9 * f + i];
    const float* p = x + f * fs;
    CF acc = cf_zero();
    for (int32_t k0 = 0; k0 < A; k0 += 32 * 8) {
      float part = 0.f;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int32_t k = k0 + lane + 32 * u;
        if (k < A) {
          float bx, by, bz;
          rotate(r, p[3 * k], p[3 * k + 1], p[3 * k + 2], bx, by, bz);
          const float dx = bx - ref[3 * k], dy = by - ref[3 * k + 1], dz = bz - ref[3 * k + 2];
          part = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, part)));
        }
      }
      cf_add(acc, part);
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
      CF o;
      o.hi = __shfl_xor_sync(FULL_MASK, acc.hi, m);
      o.lo = __shfl_xor_sync(FULL_MASK, acc.lo, m);
      acc = cf_add2(acc, o);
    }
    if (lane == 0) {
      double msd = A > 0 ? cf_to_double(acc) / (double)A : 0.0;
      if (!(msd > 0.0)) msd = (msd == msd) ? 0.0 : msd;
      out[f] = sqrtf((float)msd);
    }
  }
}

// ---------------------------------------------------------------------------
// Mass-weighted centring (Trajectory.center_coordinates(mass_weighted=True))
// ---------------------------------------------------------------------------

constexpr int CW_THREADS = 256;  // 8 warps: one frame each per round
constexpr int CW_CHUNK = 2048;   // weights staged per round as float pairs (16 KB)

// x_f <- x_f - com_f in place, com_f = sum_k w_k x_fk with the caller's
// (normalised) weights, one warp per frame.  The reference forms com in FP64
// (mdtraj/geometry/distance.py:366-384, x.astype(float64).T.dot(masses)) and
// subtracts it from the float32 coordinates through numpy's float64 loop
// (mdtraj/core/trajectory.py:2133-2134), i.e. x <- float(double(x) - com).
// Here the weights are split into float pairs (hi + lo) once per CTA round,
// products w x are formed error-free in FP32 (FMA residual), summed in
// float pairs (~48 bits), and the subtraction float(x - (ch + cl)) is taken
// through TwoSum: the same float as the FP64 form except where x - com lies
// within ~2^-40 of a rounding midpoint.  No FP64 per atom (GB300's FP64
// pipe is narrow).  Pass 2 re-reads the frame, which a warp has just read
// (L1/L2).
__global__ void __launch_bounds__(CW_THREADS) center_weighted_kernel(float* __restrict__ x, int64_t F, int32_t A,
                                                                    int64_t fs, const double* __restrict__ w,
                                                                    double* __restrict__ com_out) {
  __shared__ float2 sw[CW_CHUNK];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int WPB = CW_THREADS / 32;
  const int64_t rounds = (F + WPB - 1) / WPB;
  for (int64_t b = blockIdx.x; b < rounds; b += gridDim.x) {
    const int64_t f = b * WPB + warp;
    const bool live = f < F;
    float* fr = x + (live ? f : 0) * fs;
    CF s[3] = {cf_zero(), cf_zero(), cf_zero()};
    for (int32_t k0 = 0; k0 < A; k0 += CW_CHUNK) {
      const int n = min(CW_CHUNK, A - k0);
      __syncthreads();  // the previous chunk's weights are no longer read
      for (int i = threadIdx.x; i < n; i += CW_THREADS) {
        const double d = w[k0 + i];
        const float hi = (float)d;
        sw[i] = make_float2(hi, (float)(d - (double)hi));
      }
      __syncthreads();
      if (live) {
        for (int i = lane; i < n; i += 32) {
          const float2 ww = sw[i];
          const float* p = fr + 3 * (size_t)(k0 + i);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float v = p[c];
            const float ph = __fmul_rn(ww.x, v);  // not contracted into the sums below
            float pl = fmaf(ww.y, v, fmaf(ww.x, v, -ph));  // w x - ph to ~2^-48
            if (!isfinite(ph)) pl = 0.f;  // inf - inf: an infinite product carries no low part
            cf_add(s[c], ph);
            cf_add(s[c], pl);
          }
        }
      }
    }
    if (!live) continue;
    float ch[3], cl[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      CF v = s[c];
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) {
        CF o;
        o.hi = __shfl_xor_sync(FULL_MASK, v.hi, m);
        o.lo = __shfl_xor_sync(FULL_MASK, v.lo, m);
        v = cf_add2(v, o);
      }
      ch[c] = v.hi;
      cl[c] = isfinite(v.hi) ? v.lo : 0.f;  // an infinite com carries no low part
    }
    if (lane == 0 && com_out)
      for (int c = 0; c < 3; ++c) com_out[3 * f + c] = (double)ch[c] + (double)cl[c];
    __syncwarp();
    for (int32_t k = lane; k < A; k += 32) {
      float* p = fr + 3 * (size_t)k;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float v = p[c];
        float sh, sl;
        two_sum(v, -ch[c], sh, sl);  // v - ch exactly
        p[c] = isfinite(ch[c]) ? __fadd_rn(sh, __fsub_rn(sl, cl[c])) : __fsub_rn(v, ch[c]);
      }
    }
  }
}

int check_rows(const void* x, int64_t F, int32_t A, int64_t fs, const char* who) {
  if (F < 0 || A < 0) return set_error(GBRMSD_E_INVALID, "%s: negative sizes", who);
  if (fs < 3LL * A) return set_error(GBRMSD_E_INVALID, "%s: frame_stride must be >= 3 * n_atoms", who);
  if (F > 0 && A > 0 && !x) return set_error(GBRMSD_E_INVALID, "%s: null coordinates", who);
  return GBRMSD_OK;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

int gbrmsd_apply_rotations(float* x, int64_t n_frames, int32_t n_atoms, int64_t frame_stride, const float* rot,
                           const double* centroids, const double* offset3, int32_t* nonzero0, void* stream) {
  clear_error();
  int rc = check_rows(x, n_frames, n_atoms, frame_stride, "apply_rotations");
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (nonzero0) GB_CUDA_TRY(cudaMemsetAsync(nonzero0, 0, sizeof(int32_t), st), "memset nonzero flag");
  if (n_frames == 0 || n_atoms == 0) return GBRMSD_OK;
  if (!rot) return set_error(GBRMSD_E_INVALID, "apply_rotations: null rotations");
  const int64_t nab = (n_atoms + 4 * APPLY_THREADS - 1) / (4 * APPLY_THREADS);
  if (n_frames * nab > 0x7fffffffLL) return set_error(GBRMSD_E_INVALID, "apply_rotations: too many frames");
  float oh[3], ol[3];
  for (int c = 0; c < 3; ++c) {
    const double o = offset3 ? offset3[c] : 0.0;
    oh[c] = (float)o;
    ol[c] = (float)(o - (double)oh[c]);
  }
  const bool vec = aligned16(x) && (frame_stride % 4) == 0;
  const unsigned grid = (unsigned)(n_frames * nab);
  if (vec)
    apply_rotations_kernel<true><<<grid, APPLY_THREADS, 0, st>>>(x, n_frames, n_atoms, frame_stride, rot, centroids,
                                                                 oh[0], oh[1], oh[2], ol[0], ol[1], ol[2], nonzero0);
  else
    apply_rotations_kernel<false><<<grid, APPLY_THREADS, 0, st>>>(x, n_frames, n_atoms, frame_stride, rot, centroids,
                                                                  oh[0], oh[1], oh[2], ol[0], ol[1], ol[2], nonzero0);
  GB_CUDA_TRY(cudaGetLastError(), "launch apply_rotations_kernel");
  return GBRMSD_OK;
}

size_t gbrmsd_rmsf_workspace_bytes(int64_t n_frames, int32_t n_atoms) {
  if (n_frames < 0 || n_atoms < 0) return 0;
  return rmsf_plan(n_frames, n_atoms).bytes;
}

int gbrmsd_rmsf(const float* x, int64_t n_frames, int32_t n_atoms, int64_t frame_stride, const float* rot,
                float* out_rmsf, void* ws, size_t ws_bytes, void* stream) {
  clear_error();
  int rc = check_rows(x, n_frames, n_atoms, frame_stride, "rmsf");
  if (rc) return rc;
  if (n_atoms == 0) return GBRMSD_OK;
  if (!out_rmsf) return set_error(GBRMSD_E_INVALID, "rmsf: null output");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_frames == 0) {
    // the reference divides the zero sums by n_frames: 0/0 -> NaN
    return set_error(GBRMSD_E_INVALID, "rmsf: need at least one frame");
  }
  const RmsfPlan P = rmsf_plan(n_frames, n_atoms);
  if (!ws || ws_bytes < P.bytes) return set_error(GBRMSD_E_WORKSPACE, "rmsf: workspace needs %zu bytes", P.bytes);
  double* part = static_cast<double*>(ws);
  dim3 grid((unsigned)((n_atoms + RMSF_THREADS - 1) / RMSF_THREADS), (unsigned)P.n_chunks);
  prof_begin(st);
  rmsf_partial_kernel<<<grid, RMSF_THREADS, 0, st>>>(x, n_frames, n_atoms, frame_stride, rot, P.fch, part);
  GB_CUDA_TRY(cudaGetLastError(), "launch rmsf_partial_kernel");
  prof_end(st);
  rmsf_final_kernel<<<(n_atoms + 255) / 256, 256, 0, st>>>(part, P.n_chunks, n_atoms, n_frames, out_rmsf);
  GB_CUDA_TRY(cudaGetLastError(), "launch rmsf_final_kernel");
  return GBRMSD_OK;
}

int gbrmsd_rotated_rmsd(const float* x, int64_t n_frames, int32_t n_atoms, int64_t frame_stride, const float* rot,
                        const float* ref_frame, float* out_rmsd, void* stream) {
  clear_error();
  int rc = check_rows(x, n_frames, n_atoms, frame_stride, "rotated_rmsd");
  if (rc) return rc;
  if (n_frames == 0) return GBRMSD_OK;
  if (!rot || !out_rmsd || (n_atoms > 0 && !ref_frame))
    return set_error(GBRMSD_E_INVALID, "rotated_rmsd: null rotations, reference or output");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t warps = (int64_t)sm_count() * 32;
  const int64_t blocks = std::min<int64_t>((n_frames + 7) / 8, warps / 8);
  rotated_msd_kernel<<<(unsigned)(blocks > 0 ? blocks : 1), 256, 0, st>>>(x, n_frames, n_atoms, frame_stride, rot,
                                                                          ref_frame, out_rmsd);
  GB_CUDA_TRY(cudaGetLastError(), "launch rotated_msd_kernel");
  return GBRMSD_OK;
}

int gbrmsd_center_weighted_inplace(float* x, int64_t n_frames, int32_t n_atoms, int64_t frame_stride,
                                   const double* weights, double* out_com, void* stream) {
  clear_error();
  int rc = check_rows(x, n_frames, n_atoms, frame_stride, "center_weighted_inplace");
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_frames == 0) return GBRMSD_OK;
  if (n_atoms == 0) {
    // the reference's dot product over no atoms is 0: nothing moves
    if (out_com) GB_CUDA_TRY(cudaMemsetAsync(out_com, 0, sizeof(double) * 3 * n_frames, st), "memset com");
    return GBRMSD_OK;
  }
  if (!weights) return set_error(GBRMSD_E_INVALID, "center_weighted_inplace: null weights");
  const int64_t rounds = (n_frames + CW_THREADS / 32 - 1) / (CW_THREADS / 32);
  const int64_t blocks = std::min<int64_t>(rounds, (int64_t)sm_count() * 8);
  prof_begin(st);
  center_weighted_kernel<<<(unsigned)blocks, CW_THREADS, 0, st>>>(x, n_frames, n_atoms, frame_stride, weights,
                                                                  out_com);
  GB_CUDA_TRY(cudaGetLastError(), "launch center_weighted_kernel");
  prof_end(st);
  return GBRMSD_OK;
}

}  // extern "C"
