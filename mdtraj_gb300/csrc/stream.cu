// Single-reference streaming RMSD on GB300 (sm_103a).
//
// Work per call (all on one stream, no host synchronisation):
//   1. stream_kernel   one pass over the frames.  Persistent CTAs (one per
//                      SM), 8 or 16 warps each (kCfgs); every warp owns a ring of
//                      shared-memory stages fed by 1-D bulk async copies
//                      (cp.async.bulk + mbarrier, issued by lane 0) and
//                      walks a static round-robin list of (frame, split)
//                      units.  Per 4-atom quad a lane reads 3 x 128-bit
//                      words of the frame and of the reference (the
//                      reference lives in shared memory when it fits) and
//                      accumulates, relative to a per-unit shift, the 3x3
//                      inner product, the coordinate sum and the trace in
//                      FP32 over one stage, then folds those into
//                      error-free (TwoSum) float pairs.  A warp transpose
//                      reduction turns the 13 sums into one record per unit.
//   2. the finish      one thread per frame: combines the split records
//                      (exact re-centring), solves QCP (Newton on the
//                      quartic) and writes rmsd / centroid / trace.  Frames
//                      whose msd is below what the one-pass sums can resolve
//                      (near-identical structures) are then refined by a
//                      whole warp: msd = sum |R (a - mu) - b|^2 / n with the
//                      QCP rotation, which has no cancellation as rmsd -> 0.
//                      With one unit per frame (the usual case) the finish
//                      runs at the end of stream_kernel itself, in float-pair
//                      arithmetic, 32 frames per warp (stream_fin_tail);
//                      otherwise finish_refine_kernel runs it on FP64
//                      records.  (The rotation call keeps the two-kernel form,
//                      finish_kernel + refine_kernel over a queue.)
//
// Reference algorithm (CPU): mdtraj/rmsd/_rmsd.pyx:211-224 (centre, then
// msd_atom_major per frame), src/center_generic.h:3-44 (centring),
// src/theobald_rmsd_generic.h:7-119 (3x3 inner products),
// src/theobald_rmsd.cpp:217-334 (QCP).
#include <cuda.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>

#include "capi_internal.h"
#include "common.cuh"
#include "qcp.cuh"
#include "stream.cuh"
#include "stream_deal.cuh"
#include "stream_dev.cuh"

namespace gb {

namespace {

// ---------------------------------------------------------------------------
// Reference preparation (one CTA)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(PREP_THREADS) ref_prepare_kernel(
    const float* __restrict__ raw, int32_t A, int32_t Ap, int32_t layout, int32_t centre,
    float* __restrict__ out, RefInfo* __restrict__ info, double* __restrict__ prefix) {
  __shared__ double red[32];
  __shared__ double part[PREP_THREADS * 3];
  prepare_reference_block(raw, A, Ap, layout, centre, out, info, prefix, red, part);
}

// ---------------------------------------------------------------------------
// Refinement: direct residual for near-identical frames (warp per frame)
// ---------------------------------------------------------------------------

struct RefineArgs {
  const float* x;
  int32_t n_atoms;
  int32_t n_padded;
  int64_t frame_stride;
  const float* ref;
  const RefineEntry* list;
  const int* count;
  float* out_rmsd;
  float* out_centroid;  // entries with seg = -1: centroid of a non-finite frame
};

// One queued frame, by the whole warp (every lane calls it with the same
// entry): msd = sum |R (a - mu) - b|^2 / n with the entry's rotation and
// split-float centroid, or (seg = -1) the centroid of a frame with
// non-finite coordinates by plain FP64 sums.
template <int LAYOUT>
__device__ __forceinline__ void refine_one(const RefineArgs& r, const RefineEntry& en, int lane) {
  constexpr int U = 4;  // quads in flight per lane (8 measured slower: more code to fetch cold)
  const int32_t A = r.n_atoms, Ap = r.n_padded, Q = (A + 3) >> 2;
  const float* fr = r.x + en.frame * r.frame_stride;
  if (en.seg < 0) {
    // centroid of a frame with non-finite coordinates as the reference
    // computes it (src/center_generic.h: double sum, divide, round to
    // float), which keeps +-inf where the shifted sums give NaN
    double s[3] = {0.0, 0.0, 0.0};
    for (int32_t q = lane; q < Q; q += 32) {
      float ax[4], ay[4], az[4];
      load_frame_quad<LAYOUT>(fr, Ap, q, ax, ay, az);
      const int nv = A - 4 * q;
#pragma unroll
      for (int t = 0; t < 4; ++t)
        if (t < nv) { s[0] += ax[t]; s[1] += ay[t]; s[2] += az[t]; }
    }
    for (int k = 0; k < 3; ++k) s[k] = warp_sum_d(s[k]);
    if (lane == 0 && r.out_centroid)
      for (int k = 0; k < 3; ++k) r.out_centroid[3 * en.frame + k] = (float)(s[k] / (double)A);
    return;
  }
  CF acc = cf_zero();
  int32_t q = lane;
  for (; q + 32 * (U - 1) < Q; q += 32 * U) {
    float ax[U][4], ay[U][4], az[U][4];
#pragma unroll
    for (int u = 0; u < U; ++u) load_frame_quad<LAYOUT>(fr, Ap, q + 32 * u, ax[u], ay[u], az[u]);
    float part = 0.f;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      float bx[4], by[4], bz[4];
      load_ref_quad<LAYOUT, false>(r.ref, Ap, q + 32 * u, bx, by, bz);
      part += residual_quad(en, ax[u], ay[u], az[u], bx, by, bz, A - 4 * (q + 32 * u));
    }
    cf_add(acc, part);
  }
  for (; q < Q; q += 32) {
    float ax[4], ay[4], az[4], bx[4], by[4], bz[4];
    load_frame_quad<LAYOUT>(fr, Ap, q, ax, ay, az);
    load_ref_quad<LAYOUT, false>(r.ref, Ap, q, bx, by, bz);
    cf_add(acc, residual_quad(en, ax, ay, az, bx, by, bz, A - 4 * q));
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    CF o;
    o.hi = __shfl_xor_sync(FULL_MASK, acc.hi, m);
    o.lo = __shfl_xor_sync(FULL_MASK, acc.lo, m);
    acc = cf_add2(acc, o);
  }
  if (lane == 0) {
    // in FP32: the sum is exact to ~1e-12 and the output is a float (an FP64
    // division and square root are long FP64 sequences on GB300)
    float msd = __fadd_rn(acc.hi, acc.lo) * (1.0f / (float)A);
    if (!(msd > 0.0f)) msd = 0.0f;
    r.out_rmsd[en.frame] = sqrtf(msd);
  }
}

// ---------------------------------------------------------------------------
// Streaming pass
// ---------------------------------------------------------------------------

struct Cursor {
  int64_t unit;
  int64_t frame;
  int32_t q0, q1;  // quad range of the unit
  int32_t c;       // chunk index within the unit
};

template <int CQ>
__device__ __forceinline__ void cursor_unit(Cursor& cur, int64_t u, int32_t S, int32_t Q) {
  cur.unit = u;
  cur.c = 0;
  if (S == 1) {
    cur.frame = u;
    cur.q0 = 0;
    cur.q1 = Q;
    return;
  }
  cur.frame = u / S;
  const int32_t s = (int32_t)(u - cur.frame * S);
  cur.q0 = (int32_t)(((int64_t)s * Q) / S);
  cur.q1 = (int32_t)(((int64_t)(s + 1) * Q) / S);
}

// The unit dealt at round position v (stream_deal.cuh), from the launch's
// dealing parameters (kernel arguments: no registers held for them).
__device__ __forceinline__ int64_t place_unit(int64_t v, const StreamArgs& p) {
  return deal_place(v, p.full_units, p.part_shift, p.n_frames * p.splits);
}

// Advances to the next chunk; returns true when a new unit starts.
template <int CQ>
__device__ __forceinline__ bool cursor_next(Cursor& cur, int64_t W, int32_t S, int32_t Q, const StreamArgs& p) {
  cur.c += 1;
  if (cur.q0 + cur.c * CQ >= cur.q1) {
    cursor_unit<CQ>(cur, deal_next(cur.unit, W, p.full_units, p.part_shift, p.n_frames * p.splits), S, Q);
    return true;
  }
  return false;
}

template <int LAYOUT, int CQ>
__device__ __forceinline__ void issue_chunk(const StreamArgs& p, const void* tmap, const Cursor& cur,
                                            unsigned char* stage, uint64_t* bar) {
  // failure-detection test hook: this chunk is never issued, so the wait on
  // its stage runs out (nothing is put in flight for it)
  if (cur.c == 0 && cur.unit == p.skip_unit) return;
  const int32_t qb = cur.q0 + cur.c * CQ;
  const int32_t nq = min(CQ, cur.q1 - qb);
  if (LAYOUT == ATOM_MAJOR) {
    const float* fbase = p.x + cur.frame * p.frame_stride;
    mbar_arrive_expect_tx(bar, (uint32_t)nq * 48u);
    bulk_g2s(stage, fbase + (size_t)qb * 12, (uint32_t)nq * 48u, bar);
  } else {
    const int nbox = (nq + BOX_QUADS - 1) / BOX_QUADS;
    mbar_arrive_expect_tx(bar, (uint32_t)(nbox * BOX_BYTES));
    for (int b = 0; b < nbox; ++b)
      tma_load_3d(stage + b * BOX_BYTES, tmap, 4 * (qb + b * BOX_QUADS), 0, (int32_t)cur.frame, bar);
  }
}

// In-kernel finish (FIN), used when every frame is one unit (S = 1): after
// its last frame each warp meets the rest of its CTA at a barrier, and the
// CTA solves QCP for all of its frames, 32 at a time (one frame per lane,
// finish_frame_df: no FP64 on the common path), spread over its warps, so
// that a 10,000-frame call ends one QCP batch (~6 us) after its last byte
// is read instead of a second launch later.  Frames that need the direct
// residual are queued in the CTA's slice of the refinement list and refined
// after a second barrier, one after another, each by the whole CTA.
//
// CTA-local frame i of CTA b belongs to warp w = i % WARPS, round
// r = i / WARPS: unit b * WARPS + w + r * W (W warps in the grid).
// Bytes of the in-kernel finish's state in shared memory (refinement count,
// 16 bytes, then one float pair per warp), 16-byte aligned; the host's
// fin_smem_bytes gives the same figure.
template <int WARPS>
constexpr size_t kFinStateBytes = (16 + 8 * (size_t)WARPS + 15) / 16 * 16;

// This CTA's frames and their local order (stream_deal.cuh).
__device__ __forceinline__ FinSlice fin_slice(int64_t F, int warps) {
  return fin_slice_of(F, gridDim.x, blockIdx.x, warps);
}

__device__ __forceinline__ int64_t fin_frame(const FinSlice& s, int64_t i, int warps) {
  return fin_frame_of(s, i, gridDim.x, blockIdx.x, warps);
}

// Direct residual of one queued frame by the whole CTA (WARPS warps): every
// thread takes quads t, t + T, ... (T = WARPS * 32, up to 4 in flight), each
// warp reduces its compensated partial, and thread 0 sums the WARPS partials
// in warp order (deterministic).  One CTA-wide pass of a 1,000-atom frame is
// a single round trip to memory; a warp alone needs several.
template <int LAYOUT, int WARPS>
__device__ __forceinline__ void refine_one_cta(const RefineArgs& r, const RefineEntry& en, CF* part, int warp,
                                               int lane) {
  constexpr int U = 4;
  constexpr int T = WARPS * 32;
  const int32_t A = r.n_atoms, Ap = r.n_padded, Q = (A + 3) >> 2;
  const float* fr = r.x + en.frame * r.frame_stride;
  CF acc = cf_zero();
  int32_t q = threadIdx.x;
  for (; q + T * (U - 1) < Q; q += T * U) {
    float ax[U][4], ay[U][4], az[U][4];
#pragma unroll
    for (int u = 0; u < U; ++u) load_frame_quad<LAYOUT>(fr, Ap, q + T * u, ax[u], ay[u], az[u]);
    float pp = 0.f;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      float bx[4], by[4], bz[4];
      load_ref_quad<LAYOUT, false>(r.ref, Ap, q + T * u, bx, by, bz);
      pp += residual_quad(en, ax[u], ay[u], az[u], bx, by, bz, A - 4 * (q + T * u));
    }
    cf_add(acc, pp);
  }
  for (; q < Q; q += T) {
    float ax[4], ay[4], az[4], bx[4], by[4], bz[4];
    load_frame_quad<LAYOUT>(fr, Ap, q, ax, ay, az);
    load_ref_quad<LAYOUT, false>(r.ref, Ap, q, bx, by, bz);
    cf_add(acc, residual_quad(en, ax, ay, az, bx, by, bz, A - 4 * q));
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    CF o;
    o.hi = __shfl_xor_sync(FULL_MASK, acc.hi, m);
    o.lo = __shfl_xor_sync(FULL_MASK, acc.lo, m);
    acc = cf_add2(acc, o);
  }
  if (lane == 0) part[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    CF sum = part[0];
    for (int w = 1; w < WARPS; ++w) sum = cf_add2(sum, part[w]);
    // in FP32, as refine_one
    float msd = __fadd_rn(sum.hi, sum.lo) * (1.0f / (float)A);
    if (!(msd > 0.0f)) msd = 0.0f;
    r.out_rmsd[en.frame] = sqrtf(msd);
  }
  __syncthreads();  // part[] is reused by the next entry
}

// Called by every thread of the CTA once its records are written and
// visible (after a __syncthreads).  nref and part (WARPS partial sums) live
// in the kernel's dynamic shared memory, after the barriers (fin_smem_bytes);
// with a.rec_smem the records follow them (srec, FREC_FLOATS per frame, in
// the CTA's local frame order).
template <int LAYOUT, int WARPS>
__device__ __noinline__ void stream_fin_tail(const FinishArgs& a, const RefineArgs& r, int* nref, CF* part,
                                             const float* srec, int warp, int lane) {
  const FinSlice sl = fin_slice(a.n_frames, WARPS);
  const DF inv = DF{a.inv_hi, a.inv_lo};
  RefDF rv;
  rv.g = DF{0.f, 0.f};
  for (int k = 0; k < 3; ++k) rv.sum[k] = DF{0.f, 0.f};
  if (a.mode != MODE_PRECENTERED) {
    const RefInfo* ri = a.ref_info;
    rv.g = DF{ri->g_hi, ri->g_lo};
    for (int k = 0; k < 3; ++k) rv.sum[k] = DF{ri->sum_hi[k], ri->sum_lo[k]};
  }
  for (int64_t k = warp; k * 32 < sl.n; k += WARPS) {
    const int64_t i = k * 32 + lane;
    RefineEntry held;
    bool pending = false;
    if (i < sl.n) {
      const int64_t f = fin_frame(sl, i, WARPS);
      const float* rec = a.rec_smem ? srec + i * FREC_FLOATS : reinterpret_cast<const float*>(a.sums + f * SUMS_STRIDE);
      finish_frame_df(rec, f, a, inv, rv, &held, &pending);
    }
    if (pending) a.refine[sl.base + atomicAdd_block(nref, 1)] = held;
  }
  __syncthreads();
  const int n = *reinterpret_cast<volatile int*>(nref);
  for (int e = 0; e < n; ++e) {
    const RefineEntry en = a.refine[sl.base + e];
    if (en.seg >= 0) refine_one_cta<LAYOUT, WARPS>(r, en, part, warp, lane);  // same entry CTA-wide: uniform
  }
  // non-finite frames' centroids (plain FP64 sums), a warp each
  for (int e = warp; e < n; e += WARPS)
    if (a.refine[sl.base + e].seg < 0) refine_one<LAYOUT>(r, a.refine[sl.base + e], lane);
}

// Streaming pass.  WARPS warps per CTA, each with a private ring of NSTAGE
// shared-memory stages of CQ quads, fed by bulk async copies that lane 0
// issues NSTAGE chunks ahead.  FP32 level-1 sums cover at most 4 quads per
// lane (16 atoms) before they are folded into TwoSum pairs, which bounds the
// rounding error of the one-pass sums independently of the atom count.
// With FIN the call's finish runs at the end of the kernel (stream_fin_tail).
template <int LAYOUT, int MODE, int CQ, int NSTAGE, bool REF_SMEM, int WARPS, bool FIN>
__global__ void __launch_bounds__(WARPS * 32, 1)
    stream_kernel(const StreamArgs p, const __grid_constant__ CUtensorMap tmap, const FinishArgs fa,
                  const RefineArgs ra) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int STAGE_BYTES = CQ * 48;
  constexpr int NV = NSums<MODE>::value;
  constexpr bool USE_REF = MODE != MODE_TRACE;
  constexpr int QPL = CQ / 32;  // quads per lane per full chunk
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int32_t A = p.n_atoms;
  const int32_t Ap = p.n_padded;
  const int32_t Q = (A + 3) >> 2;
  const int32_t S = p.splits;
  const bool ragged_tail = (A & 3) != 0;
  const size_t ref_al = (REF_SMEM && USE_REF) ? align_up((size_t)Ap * 12, 128) : 0;
  float* sref = reinterpret_cast<float*>(smem);
  unsigned char* stages = smem + ref_al + (size_t)warp * NSTAGE * STAGE_BYTES;
  uint64_t* bars =
      reinterpret_cast<uint64_t*>(smem + ref_al + (size_t)WARPS * NSTAGE * STAGE_BYTES) + warp * NSTAGE;
  // the reference's copy into shared memory completes on its own barrier,
  // after the warps' stage barriers (16 bytes reserved)
  uint64_t* ref_bar = reinterpret_cast<uint64_t*>(smem + ref_al + (size_t)WARPS * NSTAGE * (STAGE_BYTES + 8));
  // FIN: refinement entries the CTA's finish queued, then the CTA-wide
  // refinement's per-warp partial sums (16-byte aligned)
  int* fin_nref = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(ref_bar) + 16);
  CF* fin_part = reinterpret_cast<CF*>(fin_nref + 4);
  float* fin_rec = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(fin_nref) + kFinStateBytes<WARPS>);
  int32_t fin_done = 0;  // frames this warp has recorded

  // The reference goes to shared memory as one bulk copy, issued before any
  // frame chunk, so that it is in flight while the warps start; every
  // thread waits for it (bounded) before its first chunk.
  if constexpr (REF_SMEM && USE_REF) {
    if (threadIdx.x == 0) {
      const uint32_t ref_bytes = (uint32_t)Ap * 12u;
      mbar_init(ref_bar, 1);
      fence_mbar_init();
      mbar_arrive_expect_tx(ref_bar, ref_bytes);
      bulk_g2s(sref, p.ref, ref_bytes, ref_bar);
    }
  }
  if (lane == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  if constexpr (FIN)
    if (threadIdx.x == 0) *fin_nref = 0;
  __syncthreads();
  const float* rbase = REF_SMEM ? sref : p.ref;

  const int64_t n_units = p.n_frames * S;
  const int64_t W = (int64_t)gridDim.x * WARPS;
  const int64_t gw = (int64_t)blockIdx.x * WARPS + warp;

  // Cursors: consumer (cc) and bulk copies into shared memory (pc, NSTAGE
  // chunks ahead).
  const void* tm = &tmap;
  Cursor pc, cc;
  cursor_unit<CQ>(pc, place_unit(gw, p), S, Q);
  cursor_unit<CQ>(cc, place_unit(gw, p), S, Q);
  int64_t issued = 0, consumed = 0;
#pragma unroll 1
  for (int s = 0; s < NSTAGE; ++s) {
    if (pc.unit < n_units) {
      if (lane == 0) issue_chunk<LAYOUT, CQ>(p, tm, pc, stages + s * STAGE_BYTES, &bars[s]);
      cursor_next<CQ>(pc, W, S, Q, p);
      ++issued;
    }
  }
  __syncwarp();

  uint32_t phases = 0;
  int slot = 0;
  bool failed = false;
  if constexpr (REF_SMEM && USE_REF) failed = !mbar_wait_timed(ref_bar, 0u, p.err, p.wait_ns);
  CF acc2[NV];
  float acc1[NV];
  int pending = 0;  // quads per lane in acc1 since the last fold
  float shift[3] = {0.f, 0.f, 0.f};

#pragma unroll 1
  while (!failed && cc.unit < n_units) {
    const bool unit_start = (cc.c == 0);
    if (unit_start) {
#pragma unroll
      for (int j = 0; j < NV; ++j) { acc2[j] = cf_zero(); acc1[j] = 0.f; }
      pending = 0;
    }
    const int32_t qb = cc.q0 + cc.c * CQ;
    const int32_t nq = min(CQ, cc.q1 - qb);
    if (!mbar_wait_timed(&bars[slot], (phases >> slot) & 1u, p.err, p.wait_ns)) {
      failed = true;
      break;
    }
    phases ^= 1u << slot;
    ++consumed;
    const float* st = reinterpret_cast<const float*>(stages + slot * STAGE_BYTES);

    if (MODE == MODE_CENTER && unit_start) {
      // Shift = mean of the unit's first atoms (each lane's first quad).
      float sx = 0.f, sy = 0.f, sz = 0.f, cnt = 0.f;
      if (lane < nq) {
        float x[4], y[4], z[4];
        load_stage_quad<LAYOUT, CQ>(st, lane, x, y, z);
        const int nv = A - 4 * (qb + lane);
#pragma unroll
        for (int t = 0; t < 4; ++t)
          if (t < nv) { sx += x[t]; sy += y[t]; sz += z[t]; cnt += 1.f; }
      }
      sx = warp_sum(sx); sy = warp_sum(sy); sz = warp_sum(sz); cnt = warp_sum(cnt);
      shift[0] = sx / cnt; shift[1] = sy / cnt; shift[2] = sz / cnt;
    }

    // The frame's padded last quad can only be the chunk's last quad.
    const bool has_tail = ragged_tail && (qb + nq == Q);
    if (nq == CQ && !has_tail) {
#pragma unroll
      for (int kq = 0; kq < QPL; ++kq) {
        const int i = lane + 32 * kq;
        const int32_t gq = qb + i;
        float ax[4], ay[4], az[4];
        load_stage_quad<LAYOUT, CQ>(st, i, ax, ay, az);
        if constexpr (MODE == MODE_TRACE) {
#pragma unroll
          for (int t = 0; t < 4; ++t) { cf_add(acc2[0], ax[t]); cf_add(acc2[1], ay[t]); cf_add(acc2[2], az[t]); }
        } else {
          float bx[4], by[4], bz[4];
          load_ref_quad<LAYOUT, REF_SMEM>(rbase, Ap, gq, bx, by, bz);
          accum_quad<MODE, false, NV>(acc1, ax, ay, az, bx, by, bz, shift, 4);
        }
      }
    } else {
#pragma unroll
      for (int kq = 0; kq < QPL; ++kq) {
        const int i = lane + 32 * kq;
        if (i < nq) {
          const int32_t gq = qb + i;
          const int nv = A - 4 * gq;
          float ax[4], ay[4], az[4];
          load_stage_quad<LAYOUT, CQ>(st, i, ax, ay, az);
          if constexpr (MODE == MODE_TRACE) {
#pragma unroll
            for (int t = 0; t < 4; ++t)
              if (t < nv) { cf_add(acc2[0], ax[t]); cf_add(acc2[1], ay[t]); cf_add(acc2[2], az[t]); }
          } else {
            float bx[4], by[4], bz[4];
            load_ref_quad<LAYOUT, REF_SMEM>(rbase, Ap, gq, bx, by, bz);
            if (nv < 4)
              accum_quad<MODE, true, NV>(acc1, ax, ay, az, bx, by, bz, shift, nv);
            else
              accum_quad<MODE, false, NV>(acc1, ax, ay, az, bx, by, bz, shift, 4);
          }
        }
      }
    }
    pending += QPL;

    // Release the stage and refill it with the chunk NSTAGE ahead.
    __syncwarp();
    if (pc.unit < n_units) {
      if (lane == 0) {
        fence_proxy_async_smem();
        issue_chunk<LAYOUT, CQ>(p, tm, pc, stages + slot * STAGE_BYTES, &bars[slot]);
      }
      cursor_next<CQ>(pc, W, S, Q, p);
      ++issued;
    }
    slot = (slot + 1 == NSTAGE) ? 0 : slot + 1;

    const int64_t unit = cc.unit;
    const bool unit_end = cursor_next<CQ>(cc, W, S, Q, p);
    if constexpr (MODE != MODE_TRACE) {
      if (pending >= 4 || unit_end) {
#pragma unroll
        for (int j = 0; j < NV; ++j) { cf_add(acc2[j], acc1[j]); acc1[j] = 0.f; }
        pending = 0;
      }
    }
    if (unit_end) {
      double* rec = p.sums + unit * SUMS_STRIDE;
      float* recf = reinterpret_cast<float*>(rec);
      if constexpr (FIN) {
        if (fa.rec_smem)
          recf = fin_rec + fin_local_index(fin_done, warp, p.full_rounds, p.part_shift, blockIdx.x, WARPS) * FREC_FLOATS;
        ++fin_done;
      }
      if constexpr (NV == 1) {
        CF v = acc2[0];
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) {
          CF o;
          o.hi = __shfl_xor_sync(FULL_MASK, v.hi, m);
          o.lo = __shfl_xor_sync(FULL_MASK, v.lo, m);
          v = cf_add2(v, o);
        }
        if (lane == 0) rec[12] = cf_to_double(v);
      } else if constexpr (NV == 3) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          CF v = acc2[j];
#pragma unroll
          for (int m = 16; m >= 1; m >>= 1) {
            CF o;
            o.hi = __shfl_xor_sync(FULL_MASK, v.hi, m);
            o.lo = __shfl_xor_sync(FULL_MASK, v.lo, m);
            v = cf_add2(v, o);
          }
          if (lane == 0) rec[9 + j] = cf_to_double(v);
        }
      } else {
        CF v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = (j < NV) ? acc2[j < NV ? j : 0] : cf_zero();
        warp_xpose_reduce16(v, lane);
        const int idx = lane >> 1;
        if ((lane & 1) == 0 && idx < NV) {
          if constexpr (FIN) {
            // float pair (finish_frame_df's record), normalised
            const DF d = df_two_sum(v[0].hi, v[0].lo);
            recf[2 * idx] = d.hi;
            recf[2 * idx + 1] = d.lo;
          } else {
            rec[idx] = cf_to_double(v[0]);
          }
        }
      }
      if (lane == 0 && MODE == MODE_CENTER) {
        if constexpr (FIN) {
          recf[DFREC_SHIFT] = shift[0];
          recf[DFREC_SHIFT + 1] = shift[1];
          recf[DFREC_SHIFT + 2] = shift[2];
        } else {
          rec[16] = shift[0];
          rec[17] = shift[1];
          rec[18] = shift[2];
        }
      }
    }
  }

  if (failed) {
    // Wait (bounded) on every stage this warp still has outstanding, the one
    // that timed out included, so that no copy is left in flight into shared
    // memory when the CTA exits; a stage whose copy never arrives costs one
    // more bounded wait and does not stop the others from being drained.
    // The same for the reference's copy (at once when it has landed).
    if constexpr (REF_SMEM && USE_REF) mbar_wait_timed(ref_bar, 0u, nullptr, p.wait_ns);
    const int64_t outstanding = issued - consumed;
    for (int64_t i = 0; i < outstanding; ++i) {
      mbar_wait_timed(&bars[slot], (phases >> slot) & 1u, nullptr, p.wait_ns);
      phases ^= 1u << slot;
      slot = (slot + 1 == NSTAGE) ? 0 : slot + 1;
    }
  }
  if constexpr (FIN) {
    // every record of the CTA is written (a warp whose wait ran out leaves
    // some unwritten: the error word already marks the call's results)
    __syncthreads();
    stream_fin_tail<LAYOUT, WARPS>(fa, ra, fin_nref, fin_part, fin_rec, warp, lane);
  }
}

// ---------------------------------------------------------------------------
// QCP finish: one thread per frame
// ---------------------------------------------------------------------------

// Threads per finish block: the QCP solve is FP64 (a narrow pipe on GB300),
// so batches of fewer than ~2 frames per thread slot of the whole GPU are
// spread over every SM with 64-thread blocks instead of packing 256 frames
// into each of a few blocks.
int finish_threads(int64_t n_frames) { return n_frames >= 256LL * 2 * sm_count() ? 256 : 64; }

void launch_finish(const FinishArgs& fa, int64_t n_frames, cudaStream_t st);

__global__ void __launch_bounds__(256) finish_kernel(const FinishArgs a) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= a.n_frames) return;
  FrameCtx c;
  c.recs = a.sums + f * (int64_t)a.splits * SUMS_STRIDE;
  c.S = a.splits;
  c.A = a.n_atoms;
  c.inv_a = a.inv_atoms;
  c.mode = a.mode;
  c.ref_info = a.ref_info;
  c.ref_prefix = a.ref_prefix;
  c.g_target = (a.mode == MODE_PRECENTERED) ? a.g_target[f] : 0.f;
  c.g_ref = a.g_ref_override;
  c.self = (f == a.self_index);
  c.out_idx = f;
  c.refine_frame = f;
  c.refine_seg = 0;
  c.out_rot = a.out_rot;
  c.out_mu = a.out_mu;
  finish_frame(c, a.out_rmsd, a.out_centroid, a.out_trace, a.refine, a.refine_count, a.err);
}

void launch_finish(const FinishArgs& fa, int64_t n_frames, cudaStream_t st) {
  const int t = finish_threads(n_frames);
  finish_kernel<<<(unsigned)((n_frames + t - 1) / t), t, 0, st>>>(fa);
}

// Refinement of a queue filled by finish_kernel: one warp per entry.
template <int LAYOUT>
__global__ void __launch_bounds__(256) refine_kernel(const RefineArgs r) {
  const int lane = threadIdx.x & 31;
  const int64_t W = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int n = *reinterpret_cast<const volatile int*>(r.count);
  for (int64_t e = gw; e < n; e += W) refine_one<LAYOUT>(r, r.list[e], lane);
}

// Finish and refinement in one launch (the single-reference call): thread j
// of block b finishes frame b * per_block + j; the frames of a warp that need
// the refinement pass are then refined by that warp, one after the other
// with all 32 lanes.  Blocks take equal shares of the frames, one block per
// SM while there are at most 128 frames per SM: the FP64 QCP is the cost
// here (GB300's FP64 pipe is narrow), so the SM with the most frames sets
// the time, and a second launch for the refinement would cost as much again
// as its (usually empty) work.
template <int LAYOUT>
__global__ void __launch_bounds__(128) finish_refine_kernel(const FinishArgs a, const RefineArgs r,
                                                           int32_t per_block) {
  const int j = threadIdx.x;
  const int lane = j & 31;
  const int64_t f = (int64_t)blockIdx.x * per_block + j;
  RefineEntry held;
  bool pending = false;
  if (j < per_block && f < a.n_frames) {
    FrameCtx c;
    c.recs = a.sums + f * (int64_t)a.splits * SUMS_STRIDE;
    c.S = a.splits;
    c.A = a.n_atoms;
    c.inv_a = a.inv_atoms;
    c.mode = a.mode;
    c.ref_info = a.ref_info;
    c.ref_prefix = a.ref_prefix;
    c.g_target = (a.mode == MODE_PRECENTERED) ? a.g_target[f] : 0.f;
    c.g_ref = a.g_ref_override;
    c.self = (f == a.self_index);
    c.out_idx = f;
    c.refine_frame = f;
    c.refine_seg = 0;
    c.out_rot = nullptr;
    c.out_mu = nullptr;
    finish_frame(c, a.out_rmsd, a.out_centroid, a.out_trace, nullptr, nullptr, a.err, &held, &pending);
  }
  unsigned todo = __ballot_sync(FULL_MASK, pending);
  while (todo) {
    const int src = __ffs(todo) - 1;
    todo &= todo - 1;
    RefineEntry en;
    en.frame = __shfl_sync(FULL_MASK, held.frame, src);
#pragma unroll
    for (int i = 0; i < 9; ++i) en.rot[i] = __shfl_sync(FULL_MASK, held.rot[i], src);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      en.mu_hi[k] = __shfl_sync(FULL_MASK, held.mu_hi[k], src);
      en.mu_lo[k] = __shfl_sync(FULL_MASK, held.mu_lo[k], src);
    }
    en.seg = __shfl_sync(FULL_MASK, held.seg, src);
    refine_one<LAYOUT>(r, en, lane);
  }
}

// ---------------------------------------------------------------------------
// In-place centring write-back (warp per frame)
// ---------------------------------------------------------------------------

template <int LAYOUT>
__global__ void __launch_bounds__(256) center_writeback_kernel(float* x, int64_t F, int32_t A, int32_t Ap,
                                                               int64_t frame_stride, float* centroid,
                                                               float* traces) {
  const int lane = threadIdx.x & 31;
  const int64_t W = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int32_t Q = (A + 3) >> 2;
  for (int64_t f = gw; f < F; f += W) {
    float* fr = x + f * frame_stride;
    float mx = centroid[3 * f], my = centroid[3 * f + 1], mz = centroid[3 * f + 2];
    if (!(isfinite(mx) && isfinite(my) && isfinite(mz))) {
      // non-finite coordinates: the shifted one-pass sums give NaN where the
      // reference's double sum gives +-inf (src/center_generic.h), so this
      // frame's centroid is recomputed the reference's way first
      double s[3] = {0.0, 0.0, 0.0};
      for (int32_t q = lane; q < Q; q += 32) {
        float ax[4], ay[4], az[4];
        load_frame_quad<LAYOUT>(fr, Ap, q, ax, ay, az);
        const int nv = A - 4 * q;
#pragma unroll
        for (int t = 0; t < 4; ++t)
          if (t < nv) { s[0] += ax[t]; s[1] += ay[t]; s[2] += az[t]; }
      }
      for (int k = 0; k < 3; ++k) s[k] = warp_sum_d(s[k]);
      mx = (float)(s[0] / (double)A);
      my = (float)(s[1] / (double)A);
      mz = (float)(s[2] / (double)A);
      __syncwarp();
      if (lane == 0) {
        centroid[3 * f] = mx;
        centroid[3 * f + 1] = my;
        centroid[3 * f + 2] = mz;
      }
    }
    CF acc = cf_zero();
    for (int32_t q = lane; q < Q; q += 32) {
      const int nv = A - 4 * q;
      float part = 0.f;
      if (LAYOUT == ATOM_MAJOR) {
        float4* p4 = reinterpret_cast<float4*>(fr + 12 * (size_t)q);
        float v[12];
        float4 t0 = p4[0], t1 = p4[1], t2 = p4[2];
        v[0] = t0.x; v[1] = t0.y; v[2] = t0.z; v[3] = t0.w; v[4] = t1.x; v[5] = t1.y;
        v[6] = t1.z; v[7] = t1.w; v[8] = t2.x; v[9] = t2.y; v[10] = t2.z; v[11] = t2.w;
        const float mu[3] = {mx, my, mz};
#pragma unroll
        for (int e = 0; e < 12; ++e) {
          if (e / 3 < nv) {
            v[e] = __fsub_rn(v[e], mu[e % 3]);
            // float square, then extended-precision accumulation (center_arm.h:78-86)
            cf_add(acc, __fmul_rn(v[e], v[e]));
          }
        }
        p4[0] = make_float4(v[0], v[1], v[2], v[3]);
        p4[1] = make_float4(v[4], v[5], v[6], v[7]);
        p4[2] = make_float4(v[8], v[9], v[10], v[11]);
      } else {
        const float mu[3] = {mx, my, mz};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float4* p4 = reinterpret_cast<float4*>(fr + (size_t)c * Ap + 4 * (size_t)q);
          float4 t = *p4;
          float v[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            if (e < nv) {
              v[e] = __fsub_rn(v[e], mu[c]);
              cf_add(acc, __fmul_rn(v[e], v[e]));
            }
          }
          *p4 = make_float4(v[0], v[1], v[2], v[3]);
        }
      }
      (void)part;
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
      CF o;
      o.hi = __shfl_xor_sync(FULL_MASK, acc.hi, m);
      o.lo = __shfl_xor_sync(FULL_MASK, acc.lo, m);
      acc = cf_add2(acc, o);
    }
    if (lane == 0) traces[f] = (float)cf_to_double(acc);
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

struct StreamCfg {
  int warps;
  int cq;
  int nstage;
  bool ref_smem;
};

// Candidate launch configurations, in order of preference; the first whose
// shared memory fits is used unless gbrmsd_stream_config_select() forced one.
constexpr int kNumCfg = 7;
constexpr StreamCfg kCfgs[kNumCfg] = {
    {16, 128, 2, true},   // small frames: 2 x 6 KB stages per warp
    {16, 64, 3, true},    // medium frames
    {16, 64, 2, true},    // reference up to ~130 KB in shared memory
    {16, 64, 4, false},   // reference through L1/L2
    {8, 128, 3, true},
    {8, 64, 4, true},
    {8, 128, 4, false},
};
int g_forced_cfg = -1;

// Shared memory of the in-kernel finish: the refinement count (16 bytes)
// and one float pair per warp (the CTA-wide refinement's partial sums).
constexpr size_t kFinSmemPerWarp = sizeof(float) * 2;
size_t fin_smem_bytes(int warps) { return align_up(16 + kFinSmemPerWarp * (size_t)warps, 16); }

// Record slots of the in-kernel finish for the CTA with the most frames
// (fin_slice: CTA 0), when they are kept in shared memory.
size_t fin_rec_bytes(int64_t F, int warps, int grid) {
  return (size_t)fin_max_frames(F, grid, warps) * FREC_FLOATS * sizeof(float);
}

size_t stream_smem_bytes(const StreamCfg& c, int32_t Ap, bool use_ref, bool fin = false, size_t rec_bytes = 0) {
  const size_t ref = (c.ref_smem && use_ref) ? align_up((size_t)Ap * 12, 128) : 0;
  const size_t fin_state = fin ? fin_smem_bytes(c.warps) + rec_bytes : 0;
  // stages, their barriers, the reference copy's barrier (16 bytes)
  return ref + (size_t)c.warps * c.nstage * c.cq * 48 + (size_t)c.warps * c.nstage * 8 + 16 + fin_state;
}

// The in-kernel finish keeps its records in shared memory when the largest
// CTA's slots fit beside the reference and the copy stages (no L2 round
// trip per frame in the finish); otherwise in the workspace.
bool fin_rec_smem(const StreamCfg& c, int32_t Ap, int64_t F) {
  return stream_smem_bytes(c, Ap, true, true, fin_rec_bytes(F, c.warps, sm_count())) <= (size_t)max_dyn_smem();
}

// The in-kernel finish is built for the 16-warp configurations of the
// single-reference RMSD modes with one unit per frame.
bool fin_usable(const StreamCfg& c, int mode, int32_t S, int32_t Ap) {
  return S == 1 && c.warps == 16 && (mode == MODE_CENTER || mode == MODE_PRECENTERED) &&
         stream_smem_bytes(c, Ap, true, true) <= (size_t)max_dyn_smem();
}

bool cfg_fits(const StreamCfg& c, int32_t Ap, bool use_ref) {
  return stream_smem_bytes(c, Ap, use_ref) <= (size_t)max_dyn_smem();
}

StreamCfg choose_cfg(int32_t Ap, bool use_ref) {
  if (g_forced_cfg >= 0 && cfg_fits(kCfgs[g_forced_cfg], Ap, use_ref)) return kCfgs[g_forced_cfg];
  for (int i = 0; i < kNumCfg; ++i) {
    if (!use_ref && kCfgs[i].ref_smem) continue;
    if (cfg_fits(kCfgs[i], Ap, use_ref)) return kCfgs[i];
  }
  return kCfgs[6];
}

int grid_warps(const StreamCfg& c) { return sm_count() * c.warps; }

constexpr int64_t kUnitsPerWarpCap = 4;

// Splits per frame: frames are cut into S units of Q/S quads so that every
// warp gets work, but each unit also costs a fixed epilogue (shift, warp
// reduction of 13 compensated sums, record).  S minimises the busiest warp's
// time, ceil(F S / warps) * (Q/S * kCyclesPerQuad + kCyclesPerUnit): ~35
// cycles per 48-byte quad is a warp's share of the HBM bandwidth with 16
// warps per SM, ~3,400 cycles the per-unit epilogue (about 850 warp
// instructions at a quarter of an SMSP's issue rate; measured with ncu at
// 10,000 x 1,000 atoms, where S = 4 spent 1,000 instructions per 62-quad
// unit and ran at 0.3 of the copy peak).
int32_t choose_splits(int64_t F, int32_t Q, int gwarps) {
  constexpr double kCyclesPerQuad = 35.0, kCyclesPerUnit = 3400.0;
  if (F <= 0 || gwarps <= 0) return 1;
  int64_t smax = Q / 32;
  if (smax < 1) smax = 1;
  // F * S <= max(F, 4 * warps): more than a few units per warp only adds
  // epilogues, and the cap keeps the record count a monotone bound of F
  // (rmsd_units_bound)
  const int64_t scap = (kUnitsPerWarpCap * gwarps) / F;
  if (smax > scap) smax = scap < 1 ? 1 : scap;
  int32_t best_s = 1;
  double best = 0.0;
  for (int64_t s = 1; s <= smax; ++s) {
    const double per_warp = (double)((F * s + gwarps - 1) / gwarps);
    const double cost = per_warp * ((double)Q / (double)s * kCyclesPerQuad + kCyclesPerUnit);
    if (s == 1 || cost < best * 0.999) {
      best = cost;
      best_s = (int32_t)s;
    }
  }
  return best_s;
}

template <int LAYOUT, int MODE, int CQ, int NSTAGE, bool REF_SMEM, int WARPS, bool FIN>
int launch_stream_t(const StreamArgs& a, const CUtensorMap& tmap, const FinishArgs& fa, const RefineArgs& ra,
                    size_t smem, int grid, cudaStream_t st) {
  auto k = stream_kernel<LAYOUT, MODE, CQ, NSTAGE, REF_SMEM, WARPS, FIN>;
  GB_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
              "cudaFuncSetAttribute(stream_kernel)");
  k<<<grid, WARPS * 32, smem, st>>>(a, tmap, fa, ra);
  GB_CUDA_TRY(cudaGetLastError(), "launch stream_kernel");
  return GBRMSD_OK;
}

template <int LAYOUT, int MODE>
int launch_stream_m(const StreamArgs& a, const CUtensorMap& tm, const StreamCfg& c, const FinishArgs* fin,
                    const RefineArgs* rfin, size_t smem, int grid, cudaStream_t st) {
  const FinishArgs fa = fin ? *fin : FinishArgs{};
  const RefineArgs ra = rfin ? *rfin : RefineArgs{};
#define GB_CFG(W, CQ_, NS, RS, FIN_)                                                            \
  if (c.warps == W && c.cq == CQ_ && c.nstage == NS && c.ref_smem == RS)                       \
    return launch_stream_t<LAYOUT, MODE, CQ_, NS, RS, W, FIN_>(a, tm, fa, ra, smem, grid, st);
  if constexpr (MODE == MODE_CENTER || MODE == MODE_PRECENTERED) {
    if (fin) {
      GB_CFG(16, 128, 2, true, true)
      GB_CFG(16, 64, 3, true, true)
      GB_CFG(16, 64, 2, true, true)
      GB_CFG(16, 64, 4, false, true)
      return set_error(GBRMSD_E_INVALID, "no in-kernel finish for this configuration");
    }
  }
  GB_CFG(16, 128, 2, true, false)
  GB_CFG(16, 64, 3, true, false)
  GB_CFG(16, 64, 2, true, false)
  GB_CFG(16, 64, 4, false, false)
  GB_CFG(8, 128, 3, true, false)
  GB_CFG(8, 64, 4, true, false)
  GB_CFG(8, 128, 4, false, false)
#undef GB_CFG
  return set_error(GBRMSD_E_INVALID, "no streaming kernel for this configuration");
}

template <int LAYOUT>
int launch_stream_l(int mode, const StreamArgs& a, const CUtensorMap& tm, const StreamCfg& c,
                    const FinishArgs* fin, const RefineArgs* rfin, size_t smem, int grid, cudaStream_t st) {
  switch (mode) {
    case MODE_CENTER: return launch_stream_m<LAYOUT, MODE_CENTER>(a, tm, c, fin, rfin, smem, grid, st);
    case MODE_PRECENTERED: return launch_stream_m<LAYOUT, MODE_PRECENTERED>(a, tm, c, fin, rfin, smem, grid, st);
    case MODE_NOSUPERPOSE: return launch_stream_m<LAYOUT, MODE_NOSUPERPOSE>(a, tm, c, nullptr, nullptr, smem, grid, st);
    default: return launch_stream_m<LAYOUT, MODE_TRACE>(a, tm, c, nullptr, nullptr, smem, grid, st);
  }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn lookup_encode_tiled() {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return reinterpret_cast<EncodeTiledFn>(p);
}

int encode_axis_map(CUtensorMap* tm, const StreamArgs& a) {
  // looked up once per process (a function-local static is initialised
  // exactly once even when host threads call concurrently)
  static const EncodeTiledFn fn = lookup_encode_tiled();
  if (!fn) return set_error(GBRMSD_E_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
  // (atoms, axes, frames); box = 256 atoms x 3 axes x 1 frame
  const cuuint64_t dims[3] = {(cuuint64_t)a.n_padded, 3, (cuuint64_t)a.n_frames};
  const cuuint64_t strides[2] = {(cuuint64_t)a.n_padded * 4, (cuuint64_t)a.frame_stride * 4};
  const cuuint32_t box[3] = {4 * BOX_QUADS, 3, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = fn(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(a.x), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(GBRMSD_E_INVALID, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return GBRMSD_OK;
}

// fin / rfin non-null: the call's finish runs inside the streaming kernel
// (fin_usable must hold); otherwise the caller launches the finish.
int launch_stream(int layout, int mode, const StreamArgs& args, const StreamCfg& c, cudaStream_t st,
                  const FinishArgs* fin = nullptr, const RefineArgs* rfin = nullptr) {
  StreamArgs a = args;
  a.wait_ns = wait_limit_ns();
  a.skip_unit = skip_unit_hook();
  const int grid = sm_count();
  {
    const Deal d = make_deal(a.n_frames * a.splits, (int64_t)grid * c.warps);
    a.full_rounds = d.full_rounds;
    a.full_units = d.full_units;
    a.part_shift = d.part_shift;
  }
  const bool use_ref = mode != MODE_TRACE;
  // bulk copies need 16-byte aligned sources (the prepared reference)
  if (use_ref && !aligned16(a.ref)) return set_error(GBRMSD_E_INVALID, "reference workspace must be 16-byte aligned");
  const size_t rec_bytes = (fin && fin->rec_smem) ? fin_rec_bytes(a.n_frames, c.warps, sm_count()) : 0;
  const size_t smem = stream_smem_bytes(c, a.n_padded, use_ref, fin != nullptr, rec_bytes);
  alignas(64) CUtensorMap tm;
  memset(&tm, 0, sizeof(tm));
  if (layout == AXIS_MAJOR) {
    const int rc = encode_axis_map(&tm, a);
    if (rc) return rc;
    return launch_stream_l<AXIS_MAJOR>(mode, a, tm, c, fin, rfin, smem, grid, st);
  }
  return launch_stream_l<ATOM_MAJOR>(mode, a, tm, c, fin, rfin, smem, grid, st);
}

struct WsLayout {
  size_t sums_off, refine_off, cent_off, total;
};

// F frames cut into `units` (frame, split) records
WsLayout ws_layout(int64_t F, int64_t units) {
  WsLayout w;
  w.sums_off = HDR_BYTES;
  w.refine_off = align_up(w.sums_off + (size_t)units * SUMS_STRIDE * sizeof(double), 256);
  w.cent_off = align_up(w.refine_off + (size_t)F * sizeof(RefineEntry), 256);
  w.total = align_up(w.cent_off + (size_t)F * 3 * sizeof(float), 256);
  return w;
}

struct RefWsLayout {
  size_t info_off, coords_off, prefix_off, total;
};

RefWsLayout ref_ws_layout(int32_t A, int32_t Ap) {
  RefWsLayout r;
  r.info_off = 0;
  r.coords_off = 256;
  r.prefix_off = align_up(r.coords_off + (size_t)Ap * 12, 256);
  const size_t Q = (size_t)((A + 3) / 4);
  r.total = align_up(r.prefix_off + (Q + 1) * 3 * sizeof(double), 256);
  return r;
}

int check_frames(const float* x, int64_t F, int32_t A, int32_t Ap, int64_t frame_stride, int32_t layout) {
  if (F < 0 || A < 0) return set_error(GBRMSD_E_INVALID, "negative n_frames/n_atoms");
  if (layout != ATOM_MAJOR && layout != AXIS_MAJOR) return set_error(GBRMSD_E_INVALID, "bad layout %d", layout);
  if (Ap < A || (Ap & 3)) return set_error(GBRMSD_E_INVALID, "n_padded (%d) must be >= n_atoms (%d) and a multiple of 4", Ap, A);
  if (frame_stride < 3LL * Ap || (frame_stride & 3))
    return set_error(GBRMSD_E_INVALID, "frame_stride (%lld) must be >= 3*n_padded and a multiple of 4", (long long)frame_stride);
  if (F > 0 && A > 0 && (!x || !aligned16(x))) return set_error(GBRMSD_E_INVALID, "coordinates must be a 16-byte aligned device pointer");
  return GBRMSD_OK;
}

}  // namespace

// Upper bound of F' * S over every call with F' <= F frames, any mode and any
// launch configuration: choose_splits keeps F' * S <= min(max(F', 4 * warps),
// F' * Q / 32), which grows with F' and with the warp count, so a workspace
// sized for F frames also serves every smaller call (the last chunk of a
// stream, a partial batch).
int64_t rmsd_units_bound(int64_t F, int32_t A) {
  int gw = 0;
  for (int i = 0; i < kNumCfg; ++i) gw = gw > grid_warps(kCfgs[i]) ? gw : grid_warps(kCfgs[i]);
  int64_t smax = ((A + 3) / 4) / 32;
  if (smax < 1) smax = 1;
  const int64_t cap = F > kUnitsPerWarpCap * gw ? F : kUnitsPerWarpCap * gw;
  return F * smax < cap ? F * smax : cap;
}

// Optional CUDA-event timing of the dominant kernel of each profiled call
// (streaming kernel, all-pairs tile kernel, ...): one event pair per call,
// recorded on its launch stream, kept in a ring of up to kProfMax calls.
namespace {
constexpr int kProfMax = 4096;
int g_prof_cap = 0;
int g_prof_n = 0;
cudaEvent_t g_ev[kProfMax][2];
}  // namespace

// Failure-detection settings (gbrmsd_set_wait_limit_ns, gbrmsd_test_skip_copy).
namespace {
constexpr uint64_t kDefaultWaitNs = 2000000000ull;  // 2 s per bounded wait
std::atomic<uint64_t> g_wait_ns{kDefaultWaitNs};
std::atomic<int64_t> g_skip_unit{-1};
}  // namespace

uint64_t wait_limit_ns() { return g_wait_ns.load(std::memory_order_relaxed); }
int64_t skip_unit_hook() { return g_skip_unit.load(std::memory_order_relaxed); }

void prof_begin(cudaStream_t st) {
  if (g_prof_n < g_prof_cap) cudaEventRecord(g_ev[g_prof_n][0], st);
}

void prof_end(cudaStream_t st) {
  if (g_prof_n < g_prof_cap) {
    cudaEventRecord(g_ev[g_prof_n][1], st);
    ++g_prof_n;
  }
}

}  // namespace gb

// Scratch of gbrmsd_rmsd_to_reference_noalloc: a fixed device array that
// exists on every GPU that loads this library, for the life of the process.
// 16 MiB covers the partial-sum records, refinement list and centroids of
// gbrmsd_noalloc_max_frames(n_atoms) frames: about 68,700 of any atom count on
// a 152-SM GB300 (244 bytes per frame).
constexpr size_t kNoallocScratchBytes = 16u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];
static std::atomic<void*> g_noalloc_scratch_addr[64] = {};

using namespace gb;

// Device address of g_noalloc_scratch on the current device.  In host code
// the array's name stands for a host-side shadow, not for device memory, so
// the address is looked up once per device, with that device current, and
// kept for the life of the process (a cudaDeviceReset destroys the context
// it belongs to: the entry point must not be used after one).
static int noalloc_scratch(void** out) {
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= 64) return set_error(GBRMSD_E_UNSUPPORTED, "rmsd_to_reference_noalloc: device %d", dev);
  void* scratch = g_noalloc_scratch_addr[dev].load(std::memory_order_acquire);
  if (!scratch) {
    GB_CUDA_TRY(cudaGetSymbolAddress(&scratch, g_noalloc_scratch), "cudaGetSymbolAddress(g_noalloc_scratch)");
    if (!scratch) return set_error(GBRMSD_E_CUDA, "rmsd_to_reference_noalloc: null scratch address");
    g_noalloc_scratch_addr[dev].store(scratch, std::memory_order_release);
  }
  *out = scratch;
  return GBRMSD_OK;
}

extern "C" {

size_t gbrmsd_reference_workspace_bytes(int32_t n_atoms, int32_t n_padded) {
  if (n_atoms < 0 || n_padded < n_atoms) return 0;
  return ref_ws_layout(n_atoms, n_padded).total;
}

int gbrmsd_prepare_reference(const float* ref_xyz, int32_t n_atoms, int32_t n_padded, int32_t layout,
                             int32_t centre, void* ref_ws, size_t ref_ws_bytes, void* stream) {
  clear_error();
  if (n_atoms < 0 || n_padded < n_atoms || (n_padded & 3))
    return set_error(GBRMSD_E_INVALID, "prepare_reference: n_padded must be >= n_atoms and a multiple of 4");
  if (layout != ATOM_MAJOR && layout != AXIS_MAJOR) return set_error(GBRMSD_E_INVALID, "prepare_reference: bad layout");
  const RefWsLayout L = ref_ws_layout(n_atoms, n_padded);
  if (!ref_ws || ref_ws_bytes < L.total)
    return set_error(GBRMSD_E_WORKSPACE, "prepare_reference: workspace needs %zu bytes", L.total);
  if (n_atoms > 0 && !ref_xyz) return set_error(GBRMSD_E_INVALID, "prepare_reference: null reference");
  unsigned char* w = static_cast<unsigned char*>(ref_ws);
  ref_prepare_kernel<<<1, PREP_THREADS, 0, static_cast<cudaStream_t>(stream)>>>(
      ref_xyz, n_atoms, n_padded, layout, centre ? 1 : 0, reinterpret_cast<float*>(w + L.coords_off),
      reinterpret_cast<RefInfo*>(w + L.info_off), reinterpret_cast<double*>(w + L.prefix_off));
  GB_CUDA_TRY(cudaGetLastError(), "launch ref_prepare_kernel");
  return GBRMSD_OK;
}

int gbrmsd_reference_info(const void* ref_ws, float* host_trace, float* host_centroid3, void* stream) {
  clear_error();
  if (!ref_ws) return set_error(GBRMSD_E_INVALID, "reference_info: null workspace");
  RefInfo ri;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  GB_CUDA_TRY(cudaMemcpyAsync(&ri, ref_ws, sizeof(RefInfo), cudaMemcpyDeviceToHost, st), "copy RefInfo");
  GB_CUDA_TRY(cudaStreamSynchronize(st), "sync RefInfo");
  if (host_trace) *host_trace = (float)ri.g;
  if (host_centroid3)
    for (int c = 0; c < 3; ++c) host_centroid3[c] = ri.centroid[c];
  return GBRMSD_OK;
}

size_t gbrmsd_rotations_workspace_bytes(int64_t n_frames, int32_t n_atoms) {
  if (n_frames < 0 || n_atoms < 0) return 0;
  return align_up(ws_layout(n_frames, rmsd_units_bound(n_frames, n_atoms)).total, 256) +
         align_up((size_t)n_frames * sizeof(float), 256);
}

size_t gbrmsd_rmsd_workspace_bytes(int64_t n_frames, int32_t n_atoms) {
  if (n_frames < 0 || n_atoms < 0) return 0;
  return ws_layout(n_frames, rmsd_units_bound(n_frames, n_atoms)).total;
}

int gbrmsd_rmsd_to_reference(const float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded,
                             int64_t frame_stride, int32_t layout, int32_t mode, const void* ref_ws,
                             const float* g_target, float g_ref, int64_t self_index, float* out_rmsd,
                             float* out_centroid, float* out_trace, void* ws, size_t ws_bytes,
                             void* stream) {
  clear_error();
  int rc = check_frames(x, n_frames, n_atoms, n_padded, frame_stride, layout);
  if (rc) return rc;
  if (mode != MODE_CENTER && mode != MODE_PRECENTERED && mode != MODE_NOSUPERPOSE)
    return set_error(GBRMSD_E_INVALID, "rmsd_to_reference: bad mode %d", mode);
  if (n_frames == 0) return GBRMSD_OK;
  if (!out_rmsd) return set_error(GBRMSD_E_INVALID, "rmsd_to_reference: null out_rmsd");
  if (!ref_ws) return set_error(GBRMSD_E_INVALID, "rmsd_to_reference: null reference workspace");
  if (mode == MODE_PRECENTERED && !g_target) return set_error(GBRMSD_E_INVALID, "precentered mode needs g_target");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_atoms == 0) {
    // The reference divides 0/0 and clamps NaN to 0 (theobald_rmsd.cpp:275-277).
    GB_CUDA_TRY(cudaMemsetAsync(out_rmsd, 0, sizeof(float) * n_frames, st), "memset rmsd");
    if (out_centroid) GB_CUDA_TRY(cudaMemsetAsync(out_centroid, 0, sizeof(float) * 3 * n_frames, st), "memset");
    if (out_trace) GB_CUDA_TRY(cudaMemsetAsync(out_trace, 0, sizeof(float) * n_frames, st), "memset");
    return GBRMSD_OK;
  }
  const StreamCfg cfg = choose_cfg(n_padded, true);
  const int32_t S = choose_splits(n_frames, (n_atoms + 3) / 4, grid_warps(cfg));
  const WsLayout L = ws_layout(n_frames, n_frames * S);
  if (!ws || ws_bytes < L.total || !aligned16(ws))
    return set_error(GBRMSD_E_WORKSPACE, "rmsd_to_reference: workspace needs %zu bytes (16-byte aligned)", L.total);
  const RefWsLayout RL = ref_ws_layout(n_atoms, n_padded);
  const unsigned char* rw = static_cast<const unsigned char*>(ref_ws);
  unsigned char* w = static_cast<unsigned char*>(ws);
  WsHeader* hdr = reinterpret_cast<WsHeader*>(w);
  GB_CUDA_TRY(cudaMemsetAsync(hdr, 0, sizeof(WsHeader), st), "memset workspace header");

  StreamArgs sa;
  sa.x = x;
  sa.n_frames = n_frames;
  sa.n_atoms = n_atoms;
  sa.n_padded = n_padded;
  sa.frame_stride = frame_stride;
  sa.ref = reinterpret_cast<const float*>(rw + RL.coords_off);
  sa.splits = S;
  sa.sums = reinterpret_cast<double*>(w + L.sums_off);
  sa.err = &hdr->err;

  FinishArgs fa{};
  fa.n_frames = n_frames;
  fa.n_atoms = n_atoms;
  fa.inv_atoms = 1.0 / (double)n_atoms;
  fa.splits = S;
  fa.sums = sa.sums;
  fa.ref_info = reinterpret_cast<const RefInfo*>(rw + RL.info_off);
  fa.ref_prefix = reinterpret_cast<const double*>(rw + RL.prefix_off);
  fa.g_target = g_target;
  fa.g_ref_override = g_ref;
  fa.self_index = self_index;
  fa.out_rmsd = out_rmsd;
  fa.out_centroid = out_centroid;
  fa.out_trace = out_trace;
  fa.refine = reinterpret_cast<RefineEntry*>(w + L.refine_off);
  fa.refine_count = &hdr->refine_count;
  fa.err = &hdr->err;
  fa.mode = mode;
  fa.out_rot = nullptr;
  fa.out_mu = nullptr;

  RefineArgs ra;
  ra.x = x;
  ra.n_atoms = n_atoms;
  ra.n_padded = n_padded;
  ra.frame_stride = frame_stride;
  ra.ref = sa.ref;
  ra.list = fa.refine;
  ra.count = fa.refine_count;
  ra.out_rmsd = out_rmsd;
  ra.out_centroid = out_centroid;

  // One launch when every frame is one unit: each CTA solves its own
  // frames at the end of the streaming kernel (no second kernel).
  fa.inv_hi = (float)fa.inv_atoms;
  fa.inv_lo = (float)(fa.inv_atoms - (double)fa.inv_hi);
  const bool fin = fin_usable(cfg, mode, S, n_padded);
  fa.rec_smem = fin && fin_rec_smem(cfg, n_padded, n_frames) ? 1 : 0;
  prof_begin(st);
  rc = fin ? launch_stream(layout, mode, sa, cfg, st, &fa, &ra) : launch_stream(layout, mode, sa, cfg, st);
  if (rc) return rc;
  prof_end(st);
  if (fin) return GBRMSD_OK;

  // equal shares of at most 128 frames per block, one block per SM while
  // they fit
  const int64_t sms = sm_count();
  const int32_t per_block = (int32_t)std::min<int64_t>(128, (n_frames + sms - 1) / sms);
  const unsigned blocks = (unsigned)((n_frames + per_block - 1) / per_block);
  const int threads = (per_block + 31) & ~31;
  if (layout == ATOM_MAJOR)
    finish_refine_kernel<ATOM_MAJOR><<<blocks, threads, 0, st>>>(fa, ra, per_block);
  else
    finish_refine_kernel<AXIS_MAJOR><<<blocks, threads, 0, st>>>(fa, ra, per_block);
  GB_CUDA_TRY(cudaGetLastError(), "launch finish_refine_kernel");
  return GBRMSD_OK;
}

int gbrmsd_rotations(const float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded, int64_t frame_stride,
                     int32_t layout, int32_t mode, const void* ref_ws, const float* g_target, float g_ref,
                     float* out_rot, double* out_centroid, float* out_rmsd, void* ws, size_t ws_bytes,
                     void* stream) {
  clear_error();
  int rc = check_frames(x, n_frames, n_atoms, n_padded, frame_stride, layout);
  if (rc) return rc;
  if (mode != MODE_CENTER && mode != MODE_PRECENTERED)
    return set_error(GBRMSD_E_INVALID, "rotations: mode must be CENTER or PRECENTERED");
  if (n_frames == 0) return GBRMSD_OK;
  if (!out_rot || !ref_ws) return set_error(GBRMSD_E_INVALID, "rotations: null out_rot or reference workspace");
  if (mode == MODE_PRECENTERED && !g_target) return set_error(GBRMSD_E_INVALID, "precentered mode needs g_target");
  if (n_atoms == 0) return set_error(GBRMSD_E_INVALID, "rotations: need at least one alignment atom");
  const StreamCfg cfg = choose_cfg(n_padded, true);
  const int32_t S = choose_splits(n_frames, (n_atoms + 3) / 4, grid_warps(cfg));
  const WsLayout L = ws_layout(n_frames, n_frames * S);
  const size_t scratch_off = align_up(L.total, 256);
  if (!ws || ws_bytes < scratch_off + align_up((size_t)n_frames * sizeof(float), 256) || !aligned16(ws))
    return set_error(GBRMSD_E_WORKSPACE, "rotations: workspace needs %zu bytes (16-byte aligned)",
                     scratch_off + align_up((size_t)n_frames * sizeof(float), 256));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const RefWsLayout RL = ref_ws_layout(n_atoms, n_padded);
  const unsigned char* rw = static_cast<const unsigned char*>(ref_ws);
  unsigned char* w = static_cast<unsigned char*>(ws);
  WsHeader* hdr = reinterpret_cast<WsHeader*>(w);
  GB_CUDA_TRY(cudaMemsetAsync(hdr, 0, sizeof(WsHeader), st), "memset workspace header");
  StreamArgs sa;
  sa.x = x;
  sa.n_frames = n_frames;
  sa.n_atoms = n_atoms;
  sa.n_padded = n_padded;
  sa.frame_stride = frame_stride;
  sa.ref = reinterpret_cast<const float*>(rw + RL.coords_off);
  sa.splits = S;
  sa.sums = reinterpret_cast<double*>(w + L.sums_off);
  sa.err = &hdr->err;
  rc = launch_stream(layout, mode, sa, cfg, st);
  if (rc) return rc;
  FinishArgs fa{};
  fa.n_frames = n_frames;
  fa.n_atoms = n_atoms;
  fa.inv_atoms = 1.0 / (double)n_atoms;
  fa.splits = S;
  fa.sums = sa.sums;
  fa.ref_info = reinterpret_cast<const RefInfo*>(rw + RL.info_off);
  fa.ref_prefix = reinterpret_cast<const double*>(rw + RL.prefix_off);
  fa.g_target = g_target;
  fa.g_ref_override = g_ref;
  fa.self_index = -1;
  fa.out_rmsd = out_rmsd ? out_rmsd : reinterpret_cast<float*>(w + scratch_off);
  fa.refine = reinterpret_cast<RefineEntry*>(w + L.refine_off);
  fa.refine_count = &hdr->refine_count;
  fa.err = &hdr->err;
  fa.mode = mode;
  fa.out_rot = out_rot;
  fa.out_mu = mode == MODE_CENTER ? out_centroid : nullptr;
  launch_finish(fa, n_frames, st);
  GB_CUDA_TRY(cudaGetLastError(), "launch finish_kernel (rotations)");
  if (out_rmsd) {  // exact rmsd for near-identical frames, as gbrmsd_rmsd_to_reference
    RefineArgs ra;
    ra.x = x;
    ra.n_atoms = n_atoms;
    ra.n_padded = n_padded;
    ra.frame_stride = frame_stride;
    ra.ref = sa.ref;
    ra.list = fa.refine;
    ra.count = fa.refine_count;
    ra.out_rmsd = out_rmsd;
    ra.out_centroid = nullptr;
    if (layout == ATOM_MAJOR)
      refine_kernel<ATOM_MAJOR><<<sm_count() * 4, 256, 0, st>>>(ra);
    else
      refine_kernel<AXIS_MAJOR><<<sm_count() * 4, 256, 0, st>>>(ra);
    GB_CUDA_TRY(cudaGetLastError(), "launch refine_kernel (rotations)");
  }
  return GBRMSD_OK;
}

// For callers that cannot allocate device memory when they need RMSDs -- for
// example code running inside another runtime's memory pool (the pool owns
// the device memory and must not see a cudaMalloc behind its back), a plugin
// whose host application hands it buffers but no allocator, or a
// latency-bound loop that must not call cudaMalloc/cudaFree (they can
// synchronise the whole device) -- this variant of gbrmsd_rmsd_to_reference takes no workspace: its scratch is
// g_noalloc_scratch above.  It calls no cudaMalloc/cudaFree.  The first call
// on a device looks up the array's device address (cudaGetSymbolAddress) with
// that device current; make that first call before any stream capture.  All
// calls share the one array and it keeps the last call's contents (the
// per-call header is cleared on the stream before use), so calls whose work
// overlaps on the GPU -- concurrent streams or threads -- race; serialise them.
int gbrmsd_rmsd_to_reference_noalloc(const float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded,
                                     int64_t frame_stride, int32_t layout, int32_t mode, const void* ref_ws,
                                     const float* g_target, float g_ref, int64_t self_index, float* out_rmsd,
                                     float* out_centroid, float* out_trace, void* stream) {
  clear_error();
  void* scratch = nullptr;
  const int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  if (n_frames < 0 || n_atoms < 0) return set_error(GBRMSD_E_INVALID, "negative n_frames/n_atoms");
  const size_t need = gbrmsd_rmsd_workspace_bytes(n_frames, n_atoms);
  if (need > kNoallocScratchBytes)
    return set_error(GBRMSD_E_WORKSPACE,
                     "rmsd_to_reference_noalloc: %lld frames of %d atoms need %zu bytes of scratch but the static "
                     "scratch holds %zu (at most %lld frames of %d atoms per call); split the call or use "
                     "gbrmsd_rmsd_to_reference with a workspace",
                     (long long)n_frames, n_atoms, need, kNoallocScratchBytes,
                     (long long)gbrmsd_noalloc_max_frames(n_atoms), n_atoms);
  return gbrmsd_rmsd_to_reference(x, n_frames, n_atoms, n_padded, frame_stride, layout, mode, ref_ws, g_target,
                                  g_ref, self_index, out_rmsd, out_centroid, out_trace, scratch,
                                  kNoallocScratchBytes, stream);
}

int gbrmsd_center_inplace(float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded, int64_t frame_stride,
                          int32_t layout, float* out_traces, float* out_centroids, void* ws, size_t ws_bytes,
                          void* stream) {
  clear_error();
  int rc = check_frames(x, n_frames, n_atoms, n_padded, frame_stride, layout);
  if (rc) return rc;
  if (n_frames == 0) return GBRMSD_OK;
  if (!out_traces) return set_error(GBRMSD_E_INVALID, "center_inplace: null out_traces");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_atoms == 0) {
    GB_CUDA_TRY(cudaMemsetAsync(out_traces, 0, sizeof(float) * n_frames, st), "memset traces");
    if (out_centroids) GB_CUDA_TRY(cudaMemsetAsync(out_centroids, 0, sizeof(float) * 3 * n_frames, st), "memset");
    return GBRMSD_OK;
  }
  const StreamCfg cfg = choose_cfg(n_padded, false);
  const int32_t S = choose_splits(n_frames, (n_atoms + 3) / 4, grid_warps(cfg));
  const WsLayout L = ws_layout(n_frames, n_frames * S);
  const size_t need = L.total;
  if (!ws || ws_bytes < need || !aligned16(ws))
    return set_error(GBRMSD_E_WORKSPACE, "center_inplace: workspace needs %zu bytes", need);
  unsigned char* w = static_cast<unsigned char*>(ws);
  WsHeader* hdr = reinterpret_cast<WsHeader*>(w);
  float* cent = out_centroids ? out_centroids : reinterpret_cast<float*>(w + L.cent_off);
  GB_CUDA_TRY(cudaMemsetAsync(hdr, 0, sizeof(WsHeader), st), "memset workspace header");
  StreamArgs sa;
  sa.x = x;
  sa.n_frames = n_frames;
  sa.n_atoms = n_atoms;
  sa.n_padded = n_padded;
  sa.frame_stride = frame_stride;
  sa.ref = nullptr;
  sa.splits = S;
  sa.sums = reinterpret_cast<double*>(w + L.sums_off);
  sa.err = &hdr->err;
  rc = launch_stream(layout, MODE_TRACE, sa, cfg, st);
  if (rc) return rc;
  FinishArgs fa{};
  fa.n_frames = n_frames;
  fa.n_atoms = n_atoms;
  fa.inv_atoms = 1.0 / (double)n_atoms;
  fa.splits = S;
  fa.sums = sa.sums;
  fa.out_centroid = cent;
  fa.err = &hdr->err;
  fa.mode = MODE_TRACE;
  fa.self_index = -1;
  launch_finish(fa, n_frames, st);
  GB_CUDA_TRY(cudaGetLastError(), "launch finish_kernel(trace)");
  const int grid = sm_count() * 4;
  if (layout == ATOM_MAJOR)
    center_writeback_kernel<ATOM_MAJOR><<<grid, 256, 0, st>>>(x, n_frames, n_atoms, n_padded, frame_stride, cent, out_traces);
  else
    center_writeback_kernel<AXIS_MAJOR><<<grid, 256, 0, st>>>(x, n_frames, n_atoms, n_padded, frame_stride, cent, out_traces);
  GB_CUDA_TRY(cudaGetLastError(), "launch center_writeback_kernel");
  return GBRMSD_OK;
}

int gbrmsd_stream_config_count(void) { return kNumCfg; }

int gbrmsd_stream_config_select(int32_t index) {
  clear_error();
  if (index < -1 || index >= kNumCfg)
    return set_error(GBRMSD_E_INVALID, "stream_config_select: index must be -1 or in [0, %d)", kNumCfg);
  g_forced_cfg = index;
  return GBRMSD_OK;
}

int gbrmsd_stream_config_describe(int32_t index, int32_t n_atoms, int32_t* out5) {
  int32_t* out4 = out5;
  clear_error();
  if (index < 0 || index >= kNumCfg || !out4)
    return set_error(GBRMSD_E_INVALID, "stream_config_describe: bad arguments");
  const StreamCfg& c = kCfgs[index];
  out4[0] = c.warps;
  out4[1] = c.cq;
  out4[2] = c.nstage;
  out4[3] = c.ref_smem ? 1 : 0;
  out4[4] = 0;
  return cfg_fits(c, (n_atoms + 3) / 4 * 4, true) ? 1 : 0;
}

int gbrmsd_profile_enable(int32_t max_calls) {
  clear_error();
  if (max_calls < 0 || max_calls > kProfMax)
    return set_error(GBRMSD_E_INVALID, "profile_enable: max_calls must be in [0, %d]", kProfMax);
  for (int i = g_prof_cap; i < max_calls; ++i) {
    GB_CUDA_TRY(cudaEventCreate(&g_ev[i][0]), "cudaEventCreate");
    GB_CUDA_TRY(cudaEventCreate(&g_ev[i][1]), "cudaEventCreate");
  }
  if (max_calls > g_prof_cap) g_prof_cap = max_calls;
  if (max_calls == 0) g_prof_cap = 0;
  g_prof_n = 0;
  return GBRMSD_OK;
}

int gbrmsd_profile_read(float* stream_kernel_ms, int32_t capacity) {
  clear_error();
  if (!stream_kernel_ms && capacity > 0) return set_error(GBRMSD_E_INVALID, "profile_read: null output");
  const int n = g_prof_n < capacity ? g_prof_n : capacity;
  for (int i = 0; i < n; ++i) {
    GB_CUDA_TRY(cudaEventSynchronize(g_ev[i][1]), "cudaEventSynchronize");
    GB_CUDA_TRY(cudaEventElapsedTime(&stream_kernel_ms[i], g_ev[i][0], g_ev[i][1]), "cudaEventElapsedTime");
  }
  g_prof_n = 0;
  return n;
}

int gbrmsd_workspace_error_word(const void* ws, int32_t* word, void* stream) {
  clear_error();
  if (!ws || !word) return set_error(GBRMSD_E_INVALID, "workspace_error_word: null workspace or output");
  WsHeader h;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  GB_CUDA_TRY(cudaMemcpyAsync(&h, ws, sizeof(h), cudaMemcpyDeviceToHost, st), "copy header");
  GB_CUDA_TRY(cudaStreamSynchronize(st), "sync");
  *word = h.err;
  return GBRMSD_OK;
}

int gbrmsd_workspace_status(const void* ws, void* stream) {
  int32_t word = 0;
  const int rc = gbrmsd_workspace_error_word(ws, &word, stream);
  if (rc) return rc;
  if (word)
    return set_error(GBRMSD_E_DEVICE, "device error word 0x%x (1 = bounded wait expired, 2 = non-finite input)",
                     word);
  return GBRMSD_OK;
}

int gbrmsd_noalloc_status(int32_t* word, void* stream) {
  clear_error();
  void* scratch = nullptr;
  const int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  int32_t w = 0;
  const int rc2 = gbrmsd_workspace_error_word(scratch, &w, stream);
  if (rc2) return rc2;
  if (word) *word = w;
  if (w)
    return set_error(GBRMSD_E_DEVICE,
                     "rmsd_to_reference_noalloc: device error word 0x%x (1 = bounded wait expired, 2 = non-finite "
                     "input)", w);
  return GBRMSD_OK;
}

int64_t gbrmsd_noalloc_max_frames(int32_t n_atoms) {
  if (n_atoms < 0) return -1;
  // the scratch a call needs grows with the frame count: largest F that fits
  int64_t lo = 0, hi = (int64_t)kNoallocScratchBytes;  // a frame needs more than one byte
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo + 1) / 2;
    if (gbrmsd_rmsd_workspace_bytes(mid, n_atoms) <= kNoallocScratchBytes)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

int gbrmsd_set_wait_limit_ns(uint64_t ns) {
  clear_error();
  if (ns == 0) ns = kDefaultWaitNs;
  if (ns < 1000ull || ns > 60000000000ull)
    return set_error(GBRMSD_E_INVALID, "set_wait_limit_ns: limit must be 0 (default) or in [1 us, 60 s]");
  g_wait_ns.store(ns, std::memory_order_relaxed);
  return GBRMSD_OK;
}

int gbrmsd_test_skip_copy(int64_t unit) {
  clear_error();
  if (unit < -1) return set_error(GBRMSD_E_INVALID, "test_skip_copy: unit must be -1 (off) or >= 0");
  if (unit >= 0 && wait_limit_ns() > 100000000ull)
    return set_error(GBRMSD_E_INVALID, "test_skip_copy: set a wait limit of at most 100 ms first");
  g_skip_unit.store(unit, std::memory_order_relaxed);
  return GBRMSD_OK;
}

}  // extern "C"
