// Device helpers shared by the uniform streaming kernel (stream.cu) and the
// ragged batch kernel (ragged.cu): reference preparation, per-quad loads and
// accumulation, per-frame QCP finish, refinement residuals.
#pragma once

#include <math.h>

#include "common.cuh"
#include "qcp.cuh"
#include "stream.cuh"

namespace gb {

constexpr int HDR_BYTES = 256;  // workspace header: err word, refine count

struct WsHeader {
  int err;
  int refine_count;
};

constexpr int PREP_THREADS = 1024;

__device__ __forceinline__ double block_sum_d(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum_d(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
    t = warp_sum_d(t);
    if (lane == 0) red[0] = t;
  }
  __syncthreads();
  t = red[0];
  __syncthreads();
  return t;
}

// Body of the reference preparation, run by one CTA of PREP_THREADS threads
// (red: 32 doubles, part: 3 * PREP_THREADS doubles of shared memory).
__device__ __forceinline__ void prepare_reference_block(const float* __restrict__ raw, int32_t A, int32_t Ap,
                                                        int32_t layout, int32_t centre, float* __restrict__ out,
                                                        RefInfo* __restrict__ info, double* __restrict__ prefix,
                                                        double* red, double* part) {
  const int tid = threadIdx.x;
  // 1. centroid: double accumulation, rounded to float (center_generic.h:19-29)
  float mu[3] = {0.f, 0.f, 0.f};
  if (centre) {
    double s[3] = {0.0, 0.0, 0.0};
    for (int k = tid; k < A; k += blockDim.x)
      for (int c = 0; c < 3; ++c) s[c] += (double)raw[3 * k + c];
    for (int c = 0; c < 3; ++c) {
      const double t = block_sum_d(s[c], red);
      mu[c] = (float)(t / (double)A);
    }
  }
  // 2. centred (float subtraction) reference in the requested layout
  double g = 0.0, sb[3] = {0.0, 0.0, 0.0};
  for (int k = tid; k < Ap; k += blockDim.x) {
    for (int c = 0; c < 3; ++c) {
      float v = 0.f;
      if (k < A) v = __fsub_rn(raw[3 * k + c], mu[c]);
      if (layout == ATOM_MAJOR)
        out[3 * (size_t)k + c] = v;
      else
        out[(size_t)c * Ap + k] = v;
      g += (double)v * (double)v;
      sb[c] += (double)v;
    }
  }
  g = block_sum_d(g, red);
  for (int c = 0; c < 3; ++c) sb[c] = block_sum_d(sb[c], red);
  // 3. prefix sums over quads (for splitting frames across warps)
  const int Q = (A + 3) >> 2;
  const int per = (Q + PREP_THREADS - 1) / PREP_THREADS;
  const int q_lo = min(Q, tid * per), q_hi = min(Q, q_lo + per);
  double loc[3] = {0.0, 0.0, 0.0};
  for (int q = q_lo; q < q_hi; ++q)
    for (int t = 0; t < 4; ++t) {
      const int k = 4 * q + t;
      if (k < A)
        for (int c = 0; c < 3; ++c) loc[c] += (double)__fsub_rn(raw[3 * k + c], mu[c]);
    }
  for (int c = 0; c < 3; ++c) part[3 * tid + c] = loc[c];
  __syncthreads();
  if (tid == 0) {
    double run[3] = {0.0, 0.0, 0.0};
    for (int t = 0; t < PREP_THREADS; ++t)
      for (int c = 0; c < 3; ++c) {
        const double v = part[3 * t + c];
        part[3 * t + c] = run[c];
        run[c] += v;
      }
  }
  __syncthreads();
  double run[3] = {part[3 * tid], part[3 * tid + 1], part[3 * tid + 2]};
  for (int q = q_lo; q < q_hi; ++q) {
    for (int c = 0; c < 3; ++c) prefix[3 * (size_t)q + c] = run[c];
    for (int t = 0; t < 4; ++t) {
      const int k = 4 * q + t;
      if (k < A)
        for (int c = 0; c < 3; ++c) run[c] += (double)__fsub_rn(raw[3 * k + c], mu[c]);
    }
  }
  if (q_lo < q_hi && q_hi == Q)
    for (int c = 0; c < 3; ++c) prefix[3 * (size_t)Q + c] = run[c];
  if (Q == 0 && tid == 0)
    for (int c = 0; c < 3; ++c) prefix[c] = 0.0;
  if (tid == 0) {
    info->g = g;
    info->g_hi = (float)g;
    info->g_lo = (float)(g - (double)info->g_hi);
    for (int c = 0; c < 3; ++c) {
      info->sum[c] = sb[c];
      info->sum_hi[c] = (float)sb[c];
      info->sum_lo[c] = (float)(sb[c] - (double)info->sum_hi[c]);
      info->centroid[c] = mu[c];
    }
    info->n_atoms = A;
    info->n_padded = Ap;
    info->layout = layout;
    info->centred = centre;
  }
}


// Axis-major stages are a sequence of 64-quad boxes [x 256 | y 256 | z 256]
// (3 KB), each moved by one 3-D tensor copy of the box (256 atoms, 3 axes, 1
// frame); atom-major stages are one contiguous 1-D bulk copy.
constexpr int BOX_QUADS = 64;
constexpr int BOX_BYTES = BOX_QUADS * 48;


// Loads quad i of a stage (or of the reference) as x[4], y[4], z[4].
template <int LAYOUT, int CQ>
__device__ __forceinline__ void load_stage_quad(const float* st, int i, float (&x)[4], float (&y)[4],
                                                float (&z)[4]) {
  if (LAYOUT == ATOM_MAJOR) {
    const float4 t0 = lds4(st + 12 * i), t1 = lds4(st + 12 * i + 4), t2 = lds4(st + 12 * i + 8);
    x[0] = t0.x; y[0] = t0.y; z[0] = t0.z; x[1] = t0.w;
    y[1] = t1.x; z[1] = t1.y; x[2] = t1.z; y[2] = t1.w;
    z[2] = t2.x; x[3] = t2.y; y[3] = t2.z; z[3] = t2.w;
  } else {
    const float* b = st + (i / BOX_QUADS) * (BOX_BYTES / 4) + 4 * (i % BOX_QUADS);
    const float4 tx = lds4(b), ty = lds4(b + 4 * BOX_QUADS), tz = lds4(b + 8 * BOX_QUADS);
    x[0] = tx.x; x[1] = tx.y; x[2] = tx.z; x[3] = tx.w;
    y[0] = ty.x; y[1] = ty.y; y[2] = ty.z; y[3] = ty.w;
    z[0] = tz.x; z[1] = tz.y; z[2] = tz.z; z[3] = tz.w;
  }
}

template <int LAYOUT, bool SMEM>
__device__ __forceinline__ void load_ref_quad(const float* ref, int32_t Ap, int32_t gq, float (&x)[4],
                                              float (&y)[4], float (&z)[4]) {
  float4 t0, t1, t2;
  if (LAYOUT == ATOM_MAJOR) {
    const float* q = ref + (size_t)gq * 12;
    if (SMEM) { t0 = lds4(q); t1 = lds4(q + 4); t2 = lds4(q + 8); }
    else { t0 = ldg4(q); t1 = ldg4(q + 4); t2 = ldg4(q + 8); }
    x[0] = t0.x; y[0] = t0.y; z[0] = t0.z; x[1] = t0.w;
    y[1] = t1.x; z[1] = t1.y; x[2] = t1.z; y[2] = t1.w;
    z[2] = t2.x; x[3] = t2.y; y[3] = t2.z; z[3] = t2.w;
  } else {
    const float* q = ref + (size_t)gq * 4;
    if (SMEM) { t0 = lds4(q); t1 = lds4(q + Ap); t2 = lds4(q + 2 * (size_t)Ap); }
    else { t0 = ldg4(q); t1 = ldg4(q + Ap); t2 = ldg4(q + 2 * (size_t)Ap); }
    x[0] = t0.x; x[1] = t0.y; x[2] = t0.z; x[3] = t0.w;
    y[0] = t1.x; y[1] = t1.y; y[2] = t1.z; y[3] = t1.w;
    z[0] = t2.x; z[1] = t2.y; z[2] = t2.z; z[3] = t2.w;
  }
}

// Number of level-1 sums per mode.
template <int MODE>
struct NSums {
  static constexpr int value = MODE == MODE_CENTER ? 13 : MODE == MODE_PRECENTERED ? 9 : MODE == MODE_NOSUPERPOSE ? 1 : 3;
};

// Level-1 accumulation of one quad (4 atoms).  MASKED handles the last quad
// of a frame whose atom count is not a multiple of 4 (nv valid atoms).
template <int MODE, bool MASKED, int NV>
__device__ __forceinline__ void accum_quad(float (&acc)[NV], const float (&ax)[4], const float (&ay)[4],
                                           const float (&az)[4], const float (&bx)[4], const float (&by)[4],
                                           const float (&bz)[4], const float (&shift)[3], int nv) {
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    float dx, dy, dz;
    if constexpr (MODE == MODE_CENTER) {
      dx = ax[t] - shift[0]; dy = ay[t] - shift[1]; dz = az[t] - shift[2];
    } else if constexpr (MODE == MODE_NOSUPERPOSE) {
      dx = ax[t] - bx[t]; dy = ay[t] - by[t]; dz = az[t] - bz[t];
    } else {
      dx = ax[t]; dy = ay[t]; dz = az[t];
    }
    if constexpr (MASKED) {
      if (t >= nv) { dx = 0.f; dy = 0.f; dz = 0.f; }
    }
    if constexpr (MODE == MODE_NOSUPERPOSE) {
      acc[0] = fmaf(dx, dx, acc[0]);
      acc[0] = fmaf(dy, dy, acc[0]);
      acc[0] = fmaf(dz, dz, acc[0]);
    } else {
      acc[0] = fmaf(dx, bx[t], acc[0]);
      acc[1] = fmaf(dx, by[t], acc[1]);
      acc[2] = fmaf(dx, bz[t], acc[2]);
      acc[3] = fmaf(dy, bx[t], acc[3]);
      acc[4] = fmaf(dy, by[t], acc[4]);
      acc[5] = fmaf(dy, bz[t], acc[5]);
      acc[6] = fmaf(dz, bx[t], acc[6]);
      acc[7] = fmaf(dz, by[t], acc[7]);
      acc[8] = fmaf(dz, bz[t], acc[8]);
      if constexpr (MODE == MODE_CENTER) {
        acc[9] += dx;
        acc[10] += dy;
        acc[11] += dz;
        float gg = acc[12];
        gg = fmaf(dx, dx, gg);
        gg = fmaf(dy, dy, gg);
        gg = fmaf(dz, dz, gg);
        acc[12] = gg;
      }
    }
  }
}


// Per-frame QCP finish shared by the uniform and ragged paths: FP64
// recombination of the frame's S split records with exact re-centring,
//   mu = sum_j (sd_j + n_j s_j) / A
//   Ga = sum_j (g_j + 2 (s_j - mu) . sd_j + n_j |s_j - mu|^2)
//   M  = sum_j (m_j + (s_j - mu) B_j^T),  B_j = sum of the reference over split j,
// QCP (FP32 Newton + float-float polish), outputs, and the refinement queue.
struct FrameCtx {
  const double* recs;      // S records of SUMS_STRIDE doubles
  int32_t S, A, mode;
  double inv_a;            // 1 / A, computed once by the caller (FP64 division is slow on GB300)
  const RefInfo* ref_info;
  const double* ref_prefix;
  float g_target;          // MODE_PRECENTERED: supplied trace of this frame
  float g_ref;             // MODE_PRECENTERED: supplied reference trace
  bool self;               // the frame's storage is the reference's
  int64_t out_idx;         // index into the outputs
  int64_t refine_frame;    // frame id recorded for refinement
  int32_t refine_seg;      // segment id recorded for refinement (ragged)
  float* out_rot;          // optional: rotation R (row-major, R (a - mu) ~ b) per frame, 9 floats
  double* out_mu;          // optional with out_rot: FP64 centroid per frame, 3 doubles
};

// Split records are read through L2 (ld.global.cg): the streaming kernel's
// in-kernel finish reads records other warps of its CTA have just written.
__device__ __forceinline__ double ldrec(const double* p) { return __ldcg(p); }

// A frame that needs the refinement pass is queued in refine[] (refine_count
// the queue's length), or, when `held` is given, handed back in *held with
// *pending set, for the caller to refine at once.
__device__ __forceinline__ void finish_frame(const FrameCtx& c, float* out_rmsd, float* out_centroid,
                                             float* out_trace, RefineEntry* refine, int* refine_count, int* err,
                                             RefineEntry* held = nullptr, bool* pending = nullptr) {
  const int32_t A = c.A, S = c.S;
  const int32_t Q = (A + 3) >> 2;
  const double* base = c.recs;
  const double dA = (double)A;
  const double invA = c.inv_a;  // no FP64 division per frame: GB300's FP64 pipe is narrow
  const int64_t f = c.out_idx;

  if (c.mode == MODE_NOSUPERPOSE) {
    double g = 0.0;
    for (int j = 0; j < S; ++j) g += ldrec(base + j * SUMS_STRIDE + 12);
    double msd = g * invA;
    if (!(msd > 0.0)) msd = 0.0;
    out_rmsd[f] = (float)sqrt(msd);
    return;
  }
  if (c.mode == MODE_TRACE) {
    for (int k = 0; k < 3; ++k) {
      double s = 0.0;
      for (int j = 0; j < S; ++j) s += ldrec(base + j * SUMS_STRIDE + 9 + k);
      out_centroid[3 * f + k] = (float)(s * invA);
    }
    return;
  }

  double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  double ga, gb, mu[3] = {0.0, 0.0, 0.0};
  if (c.mode == MODE_PRECENTERED) {
    for (int j = 0; j < S; ++j)
      for (int i = 0; i < 9; ++i) m[i] += ldrec(base + j * SUMS_STRIDE + i);
    ga = (double)c.g_target;
    gb = (double)c.g_ref;
  } else {
    double sa[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < S; ++j) {
      const double* r = base + j * SUMS_STRIDE;
      const int32_t q0 = (int32_t)(((int64_t)j * Q) / S), q1 = (int32_t)(((int64_t)(j + 1) * Q) / S);
      const double nj = (double)(min(4 * q1, A) - 4 * q0);
      for (int k = 0; k < 3; ++k) sa[k] += ldrec(r + 9 + k) + nj * ldrec(r + 16 + k);
    }
    for (int k = 0; k < 3; ++k) mu[k] = sa[k] * invA;
    ga = 0.0;
    for (int j = 0; j < S; ++j) {
      const double* r = base + j * SUMS_STRIDE;
      const int32_t q0 = (int32_t)(((int64_t)j * Q) / S), q1 = (int32_t)(((int64_t)(j + 1) * Q) / S);
      const double nj = (double)(min(4 * q1, A) - 4 * q0);
      double ds[3], bj[3];
      for (int k = 0; k < 3; ++k) {
        ds[k] = ldrec(r + 16 + k) - mu[k];
        bj[k] = c.ref_prefix[3 * (size_t)q1 + k] - c.ref_prefix[3 * (size_t)q0 + k];
      }
      ga += ldrec(r + 12) + 2.0 * (ds[0] * ldrec(r + 9) + ds[1] * ldrec(r + 10) + ds[2] * ldrec(r + 11)) +
            nj * (ds[0] * ds[0] + ds[1] * ds[1] + ds[2] * ds[2]);
      for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) m[3 * i + k] += ldrec(r + 3 * i + k) + ds[i] * bj[k];
    }
    gb = c.ref_info->g;
    if (out_centroid)
      for (int k = 0; k < 3; ++k) out_centroid[3 * f + k] = (float)mu[k];
    if (out_trace) out_trace[f] = (float)ga;
  }

  bool self = c.self;
  if (self && c.mode == MODE_PRECENTERED) self = (c.g_target == c.g_ref);
  if (self && !c.out_rot) {  // a rotation is still computed for superposition
    out_rmsd[f] = 0.f;
    return;
  }
  bool finite = isfinite(ga) && isfinite(gb);
  for (int i = 0; i < 9; ++i) finite = finite && isfinite(m[i]);
  if (!finite) {
    // Non-finite coordinates.  The reference's msd is then NaN and its clamp
    // `if (rmsd2 > 0.0f)` returns 0 (src/theobald_rmsd.cpp:275-277), so the
    // RMSD is 0 here too; the error word records that it happened.  Its
    // rotation is NaN (qsqr < 1e-11f is false for NaN), as here.
    atomicOr(err, DEV_ERR_NONFINITE);
    out_rmsd[f] = 0.f;
    if (c.out_rot)
      for (int i = 0; i < 9; ++i) c.out_rot[9 * f + i] = nanf("");
    if (out_centroid && (refine || held) && c.mode == MODE_CENTER) {
      // The shifted one-pass sums turn an infinite coordinate into NaN, where
      // the reference's double sum gives +-inf: the refinement pass recomputes
      // this frame's centroid by plain FP64 sums (marked by seg = -1).
      RefineEntry e;
      e.frame = c.refine_frame;
      for (int i = 0; i < 9; ++i) e.rot[i] = 0.f;
      for (int k = 0; k < 3; ++k) { e.mu_hi[k] = 0.f; e.mu_lo[k] = 0.f; }
      e.seg = -1;
      if (held) {
        *held = e;
        *pending = true;
      } else {
        refine[atomicAdd(refine_count, 1)] = e;
      }
    }
    return;
  }
  int iters = 0;
  bool short_ = false;
  double lam = qcp_lambda_max_df(m, ga, gb, &iters, &short_);
  if (short_) lam = qcp_newton_fp64(m, lam);  // (near) double root: rare, FP64
  double msd = (ga + gb - 2.0 * lam) * invA;
  if (!(msd > 0.0) || self) msd = 0.0;
  out_rmsd[f] = sqrtf((float)msd);
  if (c.out_rot) {
    double rot[9];
    qcp_rotation(m, lam, rot);
    for (int i = 0; i < 9; ++i) c.out_rot[9 * f + i] = (float)rot[i];
    if (c.out_mu)
      for (int k = 0; k < 3; ++k) c.out_mu[3 * f + k] = mu[k];
  }
  if (self) return;

  // One-pass sums resolve msd to about 1e-7 * scale / sqrt(A); below
  // (0.1 * scale / sqrt(A))^2 the direct residual is recomputed by the
  // refinement kernel.  scale = (G_a + G_b) / (2 A).
  const double scale = (ga + gb) * (0.5 * invA);
  if (msd * dA < 0.01 * scale * scale && A > 0) {
    RefineEntry e;
    qcp_rotation_refine(m, lam, e.rot);
    e.frame = c.refine_frame;
    for (int k = 0; k < 3; ++k) {
      e.mu_hi[k] = (float)mu[k];
      e.mu_lo[k] = (float)(mu[k] - (double)e.mu_hi[k]);
    }
    e.seg = c.refine_seg;
    if (held) {
      *held = e;
      *pending = true;
    } else {
      refine[atomicAdd(refine_count, 1)] = e;
    }
  }
}

// Records of the in-kernel finish (one unit per frame) hold float pairs in
// the unit's SUMS_STRIDE slot: sum j as (hi, lo) at floats [2j, 2j + 1]
// (j < 13: M, then MODE_CENTER's coordinate sum and trace about the shift),
// MODE_CENTER's float shift at [DFREC_SHIFT, +3).
constexpr int DFREC_SHIFT = 26;
// Floats per record slot of the in-kernel finish when the records are kept
// in shared memory (13 float pairs and the float shift, padded).
constexpr int FREC_FLOATS = 32;

// The reference's trace and coordinate sums as float pairs, read once per
// thread before its frames (MODE_CENTER).
struct RefDF {
  DF g;
  DF sum[3];
};

// finish_frame for such a record, with no FP64 instruction on the common
// path (GB300 issues one FP64 instruction per ~64 cycles of a sub-partition;
// the FP64 recombination and conversions were half of finish_frame's
// latency): the re-centring of a whole frame, with s the shift, sd = sum (a - s)
// and sdA = sd / A,
//   mu = s + sdA,  Ga = g - sdA . sd,  M = m - sdA (sum_k b_k)^T,
// runs in float pairs and feeds qcp_lambda_max_dfm directly.  FP64 remains
// for the double-root polish and for building a refinement entry (rare).
// rec: the frame's record, in shared memory or in the workspace (written by
// warps of the same CTA before a __syncthreads, so plain loads see it).
__device__ __forceinline__ void finish_frame_df(const float* rec, int64_t f, const FinishArgs& a, DF inv,
                                                const RefDF& rv, RefineEntry* held, bool* pending) {
  const int32_t A = a.n_atoms;
  DF m[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) m[i] = DF{rec[2 * i], rec[2 * i + 1]};
  DF ga, gb, mu[3] = {DF{0.f, 0.f}, DF{0.f, 0.f}, DF{0.f, 0.f}};
  if (a.mode == MODE_PRECENTERED) {
    ga = DF{a.g_target[f], 0.f};
    gb = DF{a.g_ref_override, 0.f};
  } else {
    DF sd[3], sdA[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      sd[k] = DF{rec[18 + 2 * k], rec[19 + 2 * k]};
      sdA[k] = df_mul(sd[k], inv);
      mu[k] = df_add_f(sdA[k], rec[DFREC_SHIFT + k]);
    }
    const DF g = DF{rec[24], rec[25]};
    ga = df_sub(g, df_add(df_add(df_mul(sdA[0], sd[0]), df_mul(sdA[1], sd[1])), df_mul(sdA[2], sd[2])));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
      for (int i = 0; i < 3; ++i) m[3 * i + k] = df_sub(m[3 * i + k], df_mul(sdA[i], rv.sum[k]));
    }
    gb = rv.g;
    if (a.out_centroid)
      for (int k = 0; k < 3; ++k) a.out_centroid[3 * f + k] = __fadd_rn(mu[k].hi, mu[k].lo);
    if (a.out_trace) a.out_trace[f] = __fadd_rn(ga.hi, ga.lo);
  }
  bool self = (f == a.self_index);
  if (self && a.mode == MODE_PRECENTERED) self = (a.g_target[f] == a.g_ref_override);
  if (self) {
    a.out_rmsd[f] = 0.f;
    return;
  }
  bool finite = isfinite(ga.hi) && isfinite(ga.lo) && isfinite(gb.hi) && isfinite(gb.lo);
#pragma unroll
  for (int i = 0; i < 9; ++i) finite = finite && isfinite(m[i].hi) && isfinite(m[i].lo);
  if (!finite) {
    // as finish_frame: the reference's clamp of a NaN msd gives 0, and the
    // centroid is recomputed by plain FP64 sums in the refinement pass
    atomicOr(a.err, DEV_ERR_NONFINITE);
    a.out_rmsd[f] = 0.f;
    if (a.out_centroid && a.mode == MODE_CENTER) {
      RefineEntry e;
      e.frame = f;
      for (int i = 0; i < 9; ++i) e.rot[i] = 0.f;
      for (int k = 0; k < 3; ++k) { e.mu_hi[k] = 0.f; e.mu_lo[k] = 0.f; }
      e.seg = -1;
      *held = e;
      *pending = true;
    }
    return;
  }
  int iters = 0;
  bool short_ = false;
  DF lam = qcp_lambda_max_dfm(m, df_mul_f(df_add(ga, gb), 0.5f), &iters, &short_);
  if (short_) {  // (near) double root: rare, FP64
    double md[9];
    for (int i = 0; i < 9; ++i) md[i] = df_to_double(m[i]);
    lam = df_from_double(qcp_newton_fp64(md, df_to_double(lam)));
  }
  const DF t = df_sub(df_add(ga, gb), df_mul_f(lam, 2.0f));
  const DF msd_df = df_mul(t, inv);
  float msd = __fadd_rn(msd_df.hi, msd_df.lo);
  if (!(msd > 0.0f)) msd = 0.0f;
  a.out_rmsd[f] = sqrtf(msd);
  // One-pass sums resolve msd to about 1e-7 * scale / sqrt(A); below
  // (0.1 * scale / sqrt(A))^2 the direct residual is recomputed.
  const float scale = __fmul_rn(__fadd_rn(ga.hi, gb.hi), 0.5f * inv.hi);
  if (msd * (float)A < 0.01f * scale * scale && A > 0) {
    RefineEntry e;
    qcp_rotation_refine_dfm(m, lam, e.rot);
    e.frame = f;
    for (int k = 0; k < 3; ++k) {
      e.mu_hi[k] = mu[k].hi;
      e.mu_lo[k] = mu[k].lo;
    }
    e.seg = 0;
    *held = e;
    *pending = true;
  }
}

template <int LAYOUT>
__device__ __forceinline__ void load_frame_quad(const float* fr, int32_t Ap, int32_t q, float (&x)[4], float (&y)[4],
                                                float (&z)[4]) {
  if (LAYOUT == ATOM_MAJOR) {
    const float4 t0 = ldg4(fr + 12 * (size_t)q), t1 = ldg4(fr + 12 * (size_t)q + 4),
                 t2 = ldg4(fr + 12 * (size_t)q + 8);
    x[0] = t0.x; y[0] = t0.y; z[0] = t0.z; x[1] = t0.w;
    y[1] = t1.x; z[1] = t1.y; x[2] = t1.z; y[2] = t1.w;
    z[2] = t2.x; x[3] = t2.y; y[3] = t2.z; z[3] = t2.w;
  } else {
    const float4 tx = ldg4(fr + 4 * (size_t)q), ty = ldg4(fr + Ap + 4 * (size_t)q),
                 tz = ldg4(fr + 2 * (size_t)Ap + 4 * (size_t)q);
    x[0] = tx.x; x[1] = tx.y; x[2] = tx.z; x[3] = tx.w;
    y[0] = ty.x; y[1] = ty.y; y[2] = ty.z; y[3] = ty.w;
    z[0] = tz.x; z[1] = tz.y; z[2] = tz.z; z[3] = tz.w;
  }
}

// sum over valid atoms of |R (a - mu) - b|^2 for one quad
__device__ __forceinline__ float residual_quad(const RefineEntry& en, const float (&ax)[4], const float (&ay)[4],
                                               const float (&az)[4], const float (&bx)[4], const float (&by)[4],
                                               const float (&bz)[4], int nv) {
  float part = 0.f;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    if (t < nv) {
      const float dx = (ax[t] - en.mu_hi[0]) - en.mu_lo[0];
      const float dy = (ay[t] - en.mu_hi[1]) - en.mu_lo[1];
      const float dz = (az[t] - en.mu_hi[2]) - en.mu_lo[2];
      const float rx = fmaf(en.rot[0], dx, fmaf(en.rot[1], dy, en.rot[2] * dz)) - bx[t];
      const float ry = fmaf(en.rot[3], dx, fmaf(en.rot[4], dy, en.rot[5] * dz)) - by[t];
      const float rz = fmaf(en.rot[6], dx, fmaf(en.rot[7], dy, en.rot[8] * dz)) - bz[t];
      part = fmaf(rx, rx, part);
      part = fmaf(ry, ry, part);
      part = fmaf(rz, rz, part);
    }
  }
  return part;
}


}  // namespace gb
