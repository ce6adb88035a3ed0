// Ragged batch: many trajectories with different atom and frame counts,
// each scored against its own frame 0 (md.rmsd(t, t, 0) per trajectory,
// mdtraj/rmsd/_rmsd.pyx:211-224), in ONE persistent launch.
//
// Layout: segment s holds F_s frames of n_padded_s atoms, atom-major, padded
// to 4 atoms, starting at float offset x_off_s of the packed buffer (16-byte
// aligned).  Work units are (segment, frame, split) with at most
// `max_unit_quads` quads per unit; the unit sequence is cut into one
// contiguous range per CTA of equal estimated cost, so the warps of a CTA
// mostly stream the same segment and share its reference through L1.
//
//   ragged_ref_kernel     one CTA per segment: centred reference from frame 0
//   ragged_stream_kernel  persistent: bulk-copy staged quads, compensated sums
//   ragged_finish_kernel  one thread per global frame: FP64 QCP
//   ragged_refine_kernel  warp per near-identical frame: direct residual
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "capi_internal.h"
#include "common.cuh"
#include "qcp.cuh"
#include "stream.cuh"
#include "stream_dev.cuh"

namespace gb {
namespace {

struct RaggedSeg {
  int64_t x_off;    // float offset of frame 0 in the packed buffer
  int64_t unit0;    // first unit
  int64_t frame0;   // first global frame (output index)
  int64_t ref_off;  // byte offset of the segment's prepared reference in the workspace
  int32_t n_atoms, n_padded, splits, n_frames;
  double inv_atoms;  // 1 / n_atoms
};

struct RaggedArgs {
  const float* x;
  const RaggedSeg* segs;
  int32_t n_seg;
  const int64_t* cta_begin;  // [grid + 1] unit ranges
  const unsigned char* ref_base;
  double* sums;
  int* err;
  uint64_t wait_ns;  // limit of each bounded wait (gbrmsd_set_wait_limit_ns)
};

constexpr size_t REF_INFO_BYTES = 256;

__host__ __device__ inline size_t ref_coords_off() { return REF_INFO_BYTES; }
__host__ __device__ inline size_t ref_prefix_off(int32_t Ap) { return align_up(REF_INFO_BYTES + (size_t)Ap * 12, 256); }
__host__ __device__ inline size_t ref_bytes(int32_t A, int32_t Ap) {
  return align_up(ref_prefix_off(Ap) + (size_t)((A + 3) / 4 + 1) * 3 * sizeof(double), 256);
}

__device__ __forceinline__ int find_seg_by_unit(const RaggedSeg* segs, int n, int64_t u) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (segs[mid].unit0 <= u) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int find_seg_by_frame(const RaggedSeg* segs, int n, int64_t gf) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (segs[mid].frame0 <= gf) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(PREP_THREADS) ragged_ref_kernel(const float* __restrict__ x,
                                                                  const RaggedSeg* __restrict__ segs,
                                                                  unsigned char* __restrict__ ref_base) {
  __shared__ double red[32];
  __shared__ double part[PREP_THREADS * 3];
  const RaggedSeg sg = segs[blockIdx.x];
  unsigned char* r = ref_base + sg.ref_off;
  prepare_reference_block(x + sg.x_off, sg.n_atoms, sg.n_padded, ATOM_MAJOR, 1,
                          reinterpret_cast<float*>(r + ref_coords_off()), reinterpret_cast<RefInfo*>(r),
                          reinterpret_cast<double*>(r + ref_prefix_off(sg.n_padded)), red, part);
}

// Producer cursor over the unit sequence of one warp: units u, u + WARPS,
// u + 2 WARPS, ... of the CTA's range.  Within a segment units are ordered
// split-major (unit = unit0 + j * F + f for split j of frame f), so the warps
// of a CTA stream consecutive frames over the same reference slice and the
// slice is served from L1.  Stepping is incremental: the binary search over the
// segment table runs once per warp; afterwards segments are entered by a
// forward scan, and frame/split advance by additions.
struct RCursor {
  int64_t u, uend, seg_uend, unit0, x_seg;
  const float* ref;
  int32_t seg, A, Ap, F, S, Q, f, j, q0, q1, c;
};

__device__ __forceinline__ void rc_split_range(RCursor& w) {
  w.q0 = (int32_t)(((int64_t)w.j * w.Q) / w.S);
  w.q1 = (int32_t)(((int64_t)(w.j + 1) * w.Q) / w.S);
}

__device__ __forceinline__ void rc_enter(RCursor& w, const RaggedArgs& p) {
  const RaggedSeg sg = p.segs[w.seg];
  w.unit0 = sg.unit0;
  w.A = sg.n_atoms;
  w.Ap = sg.n_padded;
  w.F = sg.n_frames;
  w.S = sg.splits;
  w.Q = (sg.n_atoms + 3) >> 2;
  w.seg_uend = sg.unit0 + (int64_t)sg.splits * sg.n_frames;
  w.x_seg = sg.x_off;
  w.ref = reinterpret_cast<const float*>(p.ref_base + sg.ref_off + ref_coords_off());
  const int64_t lu = w.u - sg.unit0;
  w.j = (int32_t)(lu / w.F);
  w.f = (int32_t)(lu - (int64_t)w.j * w.F);
  rc_split_range(w);
}

__device__ __forceinline__ void rc_start(RCursor& w, const RaggedArgs& p, int64_t u, int64_t uend) {
  w.u = u;
  w.uend = uend;
  w.c = 0;
  if (u >= uend) return;
  w.seg = find_seg_by_unit(p.segs, p.n_seg, u);
  rc_enter(w, p);
}

template <int WARPS>
__device__ __forceinline__ void rc_next_unit(RCursor& w, const RaggedArgs& p) {
  w.u += WARPS;
  w.c = 0;
  if (w.u >= w.uend) return;
  if (w.u < w.seg_uend) {
    w.f += WARPS;
    if (w.f >= w.F) {
      do { w.f -= w.F; ++w.j; } while (w.f >= w.F);
      rc_split_range(w);
    }
    return;
  }
  do { ++w.seg; } while (w.seg + 1 < p.n_seg && p.segs[w.seg + 1].unit0 <= w.u);
  rc_enter(w, p);
}

#ifndef GB_RAGGED_X2
#define GB_RAGGED_X2 1
#endif

// Packed float pairs (sm_100+ f32x2 arithmetic): the level-1 sums of a lane
// run on atom pairs, even atoms in the low half and odd atoms in the high
// half, so one instruction does the work of two.
__device__ __forceinline__ uint64_t pk2(float a, float b) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float sum2(uint64_t v) {
  float a, b;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
  return a + b;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// The 13 centred sums of one quad on atom pairs (0, 1) and (2, 3); atoms
// at or beyond nv (MASKED, the frame's last quad) contribute zeros.
template <bool MASKED>
__device__ __forceinline__ void accum_quad_x2(uint64_t (&acc)[13], const float (&ax)[4], const float (&ay)[4],
                                              const float (&az)[4], const float (&bx)[4], const float (&by)[4],
                                              const float (&bz)[4], const float (&shift)[3], int nv) {
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    float d[2][3];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int t = 2 * p + h;
      d[h][0] = ax[t] - shift[0];
      d[h][1] = ay[t] - shift[1];
      d[h][2] = az[t] - shift[2];
      if (MASKED && t >= nv) d[h][0] = d[h][1] = d[h][2] = 0.f;
    }
    const uint64_t dx = pk2(d[0][0], d[1][0]), dy = pk2(d[0][1], d[1][1]), dz = pk2(d[0][2], d[1][2]);
    const uint64_t qx = pk2(bx[2 * p], bx[2 * p + 1]), qy = pk2(by[2 * p], by[2 * p + 1]),
                   qz = pk2(bz[2 * p], bz[2 * p + 1]);
    acc[0] = fma2(dx, qx, acc[0]);
    acc[1] = fma2(dx, qy, acc[1]);
    acc[2] = fma2(dx, qz, acc[2]);
    acc[3] = fma2(dy, qx, acc[3]);
    acc[4] = fma2(dy, qy, acc[4]);
    acc[5] = fma2(dy, qz, acc[5]);
    acc[6] = fma2(dz, qx, acc[6]);
    acc[7] = fma2(dz, qy, acc[7]);
    acc[8] = fma2(dz, qz, acc[8]);
    acc[9] = add2(acc[9], dx);
    acc[10] = add2(acc[10], dy);
    acc[11] = add2(acc[11], dz);
    acc[12] = fma2(dx, dx, acc[12]);
    acc[12] = fma2(dy, dy, acc[12]);
    acc[12] = fma2(dz, dz, acc[12]);
  }
}

// Per-stage description of the staged chunk, written by the issuing lane
// before its arrive (release) and read by the warp after the wait (acquire).
struct ChunkMeta {
  const float* ref;  // reference quads of the chunk's first quad
  int64_t rec;       // sums record of the unit
  int32_t arem;      // atoms from the chunk's first quad to the end of the frame
  int32_t nq;        // quads in the chunk
  int32_t flags;     // 1: first chunk of its unit, 2: last chunk of its unit
  int32_t pad;
};
static_assert(sizeof(ChunkMeta) == 32, "ChunkMeta is 32 bytes");

// Issues the cursor's current chunk into `stage` (all lanes advance the
// cursor; lane 0 writes the metadata and starts the copy).
template <int CQ, int WARPS>
__device__ __forceinline__ void rc_issue(RCursor& w, const RaggedArgs& p, int lane, unsigned char* stage,
                                         ChunkMeta* meta, uint64_t* bar) {
  const int32_t qb = w.q0 + w.c * CQ;
  const int32_t nq = min(CQ, w.q1 - qb);
  const bool last = qb + nq >= w.q1;
  if (lane == 0) {
    ChunkMeta m;
    m.ref = w.ref + (size_t)qb * 12;
    m.rec = w.unit0 + (int64_t)w.f * w.S + w.j;
    m.arem = w.A - 4 * qb;
    m.nq = nq;
    m.flags = (w.c == 0 ? 1 : 0) | (last ? 2 : 0);
    m.pad = 0;
    *meta = m;
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, (uint32_t)nq * 48u);
    bulk_g2s(stage, p.x + w.x_seg + (int64_t)w.f * 3 * w.Ap + (size_t)qb * 12, (uint32_t)nq * 48u, bar);
  }
  if (last) rc_next_unit<WARPS>(w, p);
  else w.c += 1;
}

template <int CQ, int NSTAGE, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, 1) ragged_stream_kernel(const RaggedArgs p) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int STAGE_BYTES = CQ * 48;
  constexpr int NV = 13;
  constexpr int QPL = CQ / 32;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  unsigned char* stages = smem + (size_t)warp * NSTAGE * STAGE_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)WARPS * NSTAGE * STAGE_BYTES) + warp * NSTAGE;
  ChunkMeta* metas = reinterpret_cast<ChunkMeta*>(smem + (size_t)WARPS * NSTAGE * (STAGE_BYTES + 8)) +
                     warp * NSTAGE;
  if (lane == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  RCursor pc;
  rc_start(pc, p, p.cta_begin[blockIdx.x] + warp, p.cta_begin[blockIdx.x + 1]);
  int issued = 0, consumed = 0;
  for (int s = 0; s < NSTAGE && pc.u < pc.uend; ++s) {
    rc_issue<CQ, WARPS>(pc, p, lane, stages + s * STAGE_BYTES, &metas[s], &bars[s]);
    ++issued;
  }
  __syncwarp();

  uint32_t phases = 0;
  int slot = 0;
  bool failed = false;
  CF acc2[NV];
#if GB_RAGGED_X2
  uint64_t acc1[NV];
#else
  float acc1[NV];
#endif
  int pending = 0;
  float shift[3] = {0.f, 0.f, 0.f};

  while (consumed < issued) {
    if (!mbar_wait_timed(&bars[slot], (phases >> slot) & 1u, p.err, p.wait_ns)) {
      failed = true;
      break;
    }
    phases ^= 1u << slot;
    ++consumed;
    const ChunkMeta m = metas[slot];
    const float* st = reinterpret_cast<const float*>(stages + slot * STAGE_BYTES);
    if (m.flags & 1) {
#pragma unroll
      for (int j = 0; j < NV; ++j) { acc2[j] = cf_zero(); acc1[j] = 0; }
      pending = 0;
      float sx = 0.f, sy = 0.f, sz = 0.f, cnt = 0.f;
      if (lane < m.nq) {
        float xx[4], yy[4], zz[4];
        load_stage_quad<ATOM_MAJOR, CQ>(st, lane, xx, yy, zz);
        const int nv = m.arem - 4 * lane;
#pragma unroll
        for (int t = 0; t < 4; ++t)
          if (t < nv) { sx += xx[t]; sy += yy[t]; sz += zz[t]; cnt += 1.f; }
      }
      sx = warp_sum(sx); sy = warp_sum(sy); sz = warp_sum(sz); cnt = warp_sum(cnt);
      shift[0] = sx / cnt; shift[1] = sy / cnt; shift[2] = sz / cnt;
    }
#pragma unroll
    for (int kq = 0; kq < QPL; ++kq) {
      const int i = lane + 32 * kq;
      if (i < m.nq) {
        float ax[4], ay[4], az[4], bx[4], by[4], bz[4];
        load_stage_quad<ATOM_MAJOR, CQ>(st, i, ax, ay, az);
        load_ref_quad<ATOM_MAJOR, false>(m.ref, 0, i, bx, by, bz);
        const int nv = m.arem - 4 * i;
#if GB_RAGGED_X2
        if (nv < 4)
          accum_quad_x2<true>(acc1, ax, ay, az, bx, by, bz, shift, nv);
        else
          accum_quad_x2<false>(acc1, ax, ay, az, bx, by, bz, shift, 4);
#else
        if (nv < 4)
          accum_quad<MODE_CENTER, true, NV>(acc1, ax, ay, az, bx, by, bz, shift, nv);
        else
          accum_quad<MODE_CENTER, false, NV>(acc1, ax, ay, az, bx, by, bz, shift, 4);
#endif
      }
    }
    pending += QPL;

    __syncwarp();
    if (pc.u < pc.uend) {
      rc_issue<CQ, WARPS>(pc, p, lane, stages + slot * STAGE_BYTES, &metas[slot], &bars[slot]);
      ++issued;
    }
    slot = (slot + 1 == NSTAGE) ? 0 : slot + 1;

    const bool unit_end = (m.flags & 2) != 0;
    if (pending >= 4 || unit_end) {
#pragma unroll
#if GB_RAGGED_X2
      for (int j = 0; j < NV; ++j) { cf_add(acc2[j], sum2(acc1[j])); acc1[j] = 0; }
#else
      for (int j = 0; j < NV; ++j) { cf_add(acc2[j], acc1[j]); acc1[j] = 0.f; }
#endif
      pending = 0;
    }
    if (unit_end) {
      double* rec = p.sums + m.rec * SUMS_STRIDE;
      CF v[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = (j < NV) ? acc2[j < NV ? j : 0] : cf_zero();
      warp_xpose_reduce16(v, lane);
      const int idx = lane >> 1;
      if ((lane & 1) == 0 && idx < NV) rec[idx] = cf_to_double(v[0]);
      if (lane == 0) {
        rec[16] = shift[0];
        rec[17] = shift[1];
        rec[18] = shift[2];
      }
    }
  }
  if (failed) {
    // bounded wait on every outstanding stage (the one that timed out
    // included) so that no copy is in flight into shared memory at exit
    const int outstanding = issued - consumed;
    for (int i = 0; i < outstanding; ++i) {
      mbar_wait_timed(&bars[slot], (phases >> slot) & 1u, nullptr, p.wait_ns);
      phases ^= 1u << slot;
      slot = (slot + 1 == NSTAGE) ? 0 : slot + 1;
    }
  }
}

struct RaggedFinishArgs {
  const RaggedSeg* segs;
  int32_t n_seg;
  int64_t total_frames;
  const unsigned char* ref_base;
  const double* sums;
  float* out;
  RefineEntry* refine;
  int* refine_count;
  int* err;
};

__global__ void __launch_bounds__(256) ragged_finish_kernel(const RaggedFinishArgs a) {
  const int64_t gf = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gf >= a.total_frames) return;
  const int s = find_seg_by_frame(a.segs, a.n_seg, gf);
  const RaggedSeg sg = a.segs[s];
  const int64_t f = gf - sg.frame0;
  const unsigned char* r = a.ref_base + sg.ref_off;
  FrameCtx c;
  c.recs = a.sums + (sg.unit0 + f * sg.splits) * SUMS_STRIDE;
  c.S = sg.splits;
  c.A = sg.n_atoms;
  c.inv_a = sg.inv_atoms;
  c.mode = MODE_CENTER;
  c.ref_info = reinterpret_cast<const RefInfo*>(r);
  c.ref_prefix = reinterpret_cast<const double*>(r + ref_prefix_off(sg.n_padded));
  c.g_target = 0.f;
  c.g_ref = 0.f;
  c.self = (f == 0);  // each trajectory is scored against its own frame 0
  c.out_idx = gf;
  c.refine_frame = gf;
  c.refine_seg = s;
  c.out_rot = nullptr;
  c.out_mu = nullptr;
  finish_frame(c, a.out, nullptr, nullptr, a.refine, a.refine_count, a.err);
}

__global__ void __launch_bounds__(256) ragged_refine_kernel(const float* __restrict__ x, const RaggedSeg* segs,
                                                            const unsigned char* ref_base, const RefineEntry* list,
                                                            const int* count, float* out) {
  constexpr int U = 4;
  const int lane = threadIdx.x & 31;
  const int64_t W = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int n = *reinterpret_cast<const volatile int*>(count);
  for (int64_t e = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < n; e += W) {
    const RefineEntry en = list[e];
    const RaggedSeg sg = segs[en.seg];
    const int64_t f = en.frame - sg.frame0;
    const float* fr = x + sg.x_off + f * 3 * (int64_t)sg.n_padded;
    const float* ref = reinterpret_cast<const float*>(ref_base + sg.ref_off + ref_coords_off());
    const int32_t A = sg.n_atoms, Q = (A + 3) >> 2;
    CF acc = cf_zero();
    int32_t q = lane;
    for (; q + 32 * (U - 1) < Q; q += 32 * U) {
      float ax[U][4], ay[U][4], az[U][4];
#pragma unroll
      for (int u = 0; u < U; ++u) load_frame_quad<ATOM_MAJOR>(fr, sg.n_padded, q + 32 * u, ax[u], ay[u], az[u]);
      float part = 0.f;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        float bx[4], by[4], bz[4];
        load_ref_quad<ATOM_MAJOR, false>(ref, sg.n_padded, q + 32 * u, bx, by, bz);
        part += residual_quad(en, ax[u], ay[u], az[u], bx, by, bz, A - 4 * (q + 32 * u));
      }
      cf_add(acc, part);
    }
    for (; q < Q; q += 32) {
      float ax[4], ay[4], az[4], bx[4], by[4], bz[4];
      load_frame_quad<ATOM_MAJOR>(fr, sg.n_padded, q, ax, ay, az);
      load_ref_quad<ATOM_MAJOR, false>(ref, sg.n_padded, q, bx, by, bz);
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
      double msd = cf_to_double(acc) / (double)A;
      if (!(msd > 0.0)) msd = 0.0;
      out[en.frame] = (float)sqrt(msd);
    }
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

struct RCfg {
  int warps, cq, nstage;
};
constexpr int kNumRCfg = 5;
constexpr RCfg kRCfgs[kNumRCfg] = {{16, 128, 2}, {16, 64, 4}, {16, 64, 3}, {8, 128, 4}, {8, 64, 4}};

size_t rcfg_smem(const RCfg& c) {
  return (size_t)c.warps * c.nstage * c.cq * 48 + (size_t)c.warps * c.nstage * (8 + sizeof(ChunkMeta));
}

template <int CQ, int NS, int W>
int launch_ragged_t(const RaggedArgs& a, int grid, cudaStream_t st) {
  auto k = ragged_stream_kernel<CQ, NS, W>;
  const size_t smem = rcfg_smem(RCfg{W, CQ, NS});
  GB_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
              "cudaFuncSetAttribute(ragged_stream_kernel)");
  k<<<grid, W * 32, smem, st>>>(a);
  GB_CUDA_TRY(cudaGetLastError(), "launch ragged_stream_kernel");
  return GBRMSD_OK;
}

int launch_ragged(int cfg, const RaggedArgs& a, int grid, cudaStream_t st) {
  switch (cfg) {
    case 0: return launch_ragged_t<128, 2, 16>(a, grid, st);
    case 1: return launch_ragged_t<64, 4, 16>(a, grid, st);
    case 2: return launch_ragged_t<64, 3, 16>(a, grid, st);
    case 3: return launch_ragged_t<128, 4, 8>(a, grid, st);
    default: return launch_ragged_t<64, 4, 8>(a, grid, st);
  }
}

struct RaggedTables {
  std::vector<RaggedSeg> segs;
  std::vector<int64_t> cta;
  int64_t total_frames = 0, total_units = 0;
  size_t ref_total = 0;
};

// Estimated time of one unit of q quads, in units of a warp's share of HBM
// per quad (~35 cycles with 16 warps per SM): a unit either streams at that
// rate, or, when it is small, is held up by its own instructions (~9.4 cycles
// per quad) plus the per-unit epilogue (shift, warp reduction of 13
// compensated sums, record: ~3,400 cycles).  Calibrated on single-segment
// runs: 64-atom frames (16-quad units) stream at 0.93 TB/s, 14% of the copy
// peak, which this model puts at 16 / (0.27 * 16 + 97) = 16%.
inline double unit_cost(double q) {
  const double mem = q, issue = 0.27 * q + 97.0;
  return mem > issue ? mem : issue;
}

int build_tables(const int64_t* x_off, const int32_t* atoms, const int32_t* padded, const int64_t* frames, int32_t n,
                 int32_t max_unit_quads, int grid, RaggedTables& t) {
  t.segs.resize(n);
  std::vector<double> cost(n);
  std::vector<int64_t> upf(n);
  for (int s = 0; s < n; ++s) {
    if (atoms[s] < 1 || padded[s] < atoms[s] || (padded[s] & 3) || frames[s] < 1 || (x_off[s] & 3) || x_off[s] < 0)
      return set_error(GBRMSD_E_INVALID,
                       "ragged: segment %d needs n_atoms >= 1, n_padded >= n_atoms (multiple of 4), n_frames >= 1 "
                       "and a 16-byte aligned offset",
                       s);
    RaggedSeg& g = t.segs[s];
    g.x_off = x_off[s];
    g.n_atoms = atoms[s];
    g.inv_atoms = 1.0 / (double)atoms[s];
    g.n_padded = padded[s];
    g.n_frames = (int32_t)frames[s];
    const int32_t Q = (atoms[s] + 3) / 4;
    int32_t sp = (Q + max_unit_quads - 1) / max_unit_quads;
    if (sp < 1) sp = 1;
    g.splits = sp;
    g.unit0 = t.total_units;
    g.frame0 = t.total_frames;
    g.ref_off = (int64_t)t.ref_total;
    t.ref_total += ref_bytes(atoms[s], padded[s]);
    upf[s] = sp;
    t.total_units += (int64_t)sp * frames[s];
    t.total_frames += frames[s];
    cost[s] = unit_cost((double)Q / sp);
  }
  // contiguous unit ranges of equal cost per CTA
  std::vector<double> seg_cost_prefix(n + 1, 0.0);
  for (int s = 0; s < n; ++s) seg_cost_prefix[s + 1] = seg_cost_prefix[s] + cost[s] * (double)(upf[s] * frames[s]);
  const double total = seg_cost_prefix[n];
  t.cta.assign(grid + 1, 0);
  int s = 0;
  for (int c = 1; c < grid; ++c) {
    const double target = total * c / grid;
    while (s < n - 1 && seg_cost_prefix[s + 1] < target) ++s;
    int64_t u = t.segs[s].unit0 + (int64_t)((target - seg_cost_prefix[s]) / cost[s]);
    const int64_t lim = t.segs[s].unit0 + upf[s] * frames[s];
    if (u > lim) u = lim;
    if (u < t.cta[c - 1]) u = t.cta[c - 1];
    t.cta[c] = u;
  }
  t.cta[grid] = t.total_units;
  return GBRMSD_OK;
}

struct RaggedWs {
  size_t segs, cta, ref, sums, refine, total;
};

RaggedWs ragged_ws(int32_t n, int grid, size_t ref_total, int64_t units, int64_t frames) {
  RaggedWs w;
  w.segs = HDR_BYTES;
  w.cta = align_up(w.segs + (size_t)n * sizeof(RaggedSeg), 256);
  w.ref = align_up(w.cta + (size_t)(grid + 1) * sizeof(int64_t), 256);
  w.sums = align_up(w.ref + ref_total, 256);
  w.refine = align_up(w.sums + (size_t)units * SUMS_STRIDE * sizeof(double), 256);
  w.total = align_up(w.refine + (size_t)frames * sizeof(RefineEntry), 256);
  return w;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

int gbrmsd_ragged_plan(const int64_t* seg_x_offsets, const int32_t* seg_atoms, const int32_t* seg_padded,
                       const int64_t* seg_frames, int32_t n_seg, int32_t config, int32_t max_unit_quads,
                       gbrmsd_ragged_plan_t* plan) {
  clear_error();
  if (!plan || n_seg < 1 || !seg_x_offsets || !seg_atoms || !seg_padded || !seg_frames)
    return set_error(GBRMSD_E_INVALID, "ragged_plan: need at least one segment and all arrays");
  if (config < 0 || config >= kNumRCfg) config = 0;
  if (max_unit_quads <= 0) max_unit_quads = 512;
  if (max_unit_quads < 32) max_unit_quads = 32;
  const RCfg c = kRCfgs[config];
  if ((size_t)max_dyn_smem() < rcfg_smem(c)) return set_error(GBRMSD_E_UNSUPPORTED, "ragged_plan: config needs more shared memory");
  const int grid = sm_count();
  RaggedTables t;
  int rc = build_tables(seg_x_offsets, seg_atoms, seg_padded, seg_frames, n_seg, max_unit_quads, grid, t);
  if (rc) return rc;
  const RaggedWs w = ragged_ws(n_seg, grid, t.ref_total, t.total_units, t.total_frames);
  memset(plan, 0, sizeof(*plan));
  plan->n_seg = n_seg;
  plan->config = config;
  plan->max_unit_quads = max_unit_quads;
  plan->grid = grid;
  plan->total_frames = t.total_frames;
  plan->total_units = t.total_units;
  plan->ws_bytes = w.total;
  return GBRMSD_OK;
}

int gbrmsd_ragged_setup(const float* x, const int64_t* seg_x_offsets, const int32_t* seg_atoms,
                        const int32_t* seg_padded, const int64_t* seg_frames, const gbrmsd_ragged_plan_t* plan,
                        void* ws, size_t ws_bytes, void* stream) {
  clear_error();
  if (!plan || !x || !aligned16(x)) return set_error(GBRMSD_E_INVALID, "ragged_setup: null plan or misaligned frames");
  RaggedTables t;
  int rc = build_tables(seg_x_offsets, seg_atoms, seg_padded, seg_frames, plan->n_seg, plan->max_unit_quads,
                        plan->grid, t);
  if (rc) return rc;
  if (t.total_units != plan->total_units || t.total_frames != plan->total_frames)
    return set_error(GBRMSD_E_INVALID, "ragged_setup: segments differ from the plan");
  const RaggedWs w = ragged_ws(plan->n_seg, plan->grid, t.ref_total, t.total_units, t.total_frames);
  if (!ws || ws_bytes < w.total || !aligned16(ws))
    return set_error(GBRMSD_E_WORKSPACE, "ragged_setup: workspace needs %zu bytes", w.total);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* b = static_cast<unsigned char*>(ws);
  GB_CUDA_TRY(cudaMemcpyAsync(b + w.segs, t.segs.data(), t.segs.size() * sizeof(RaggedSeg), cudaMemcpyHostToDevice, st),
              "upload segment table");
  GB_CUDA_TRY(cudaMemcpyAsync(b + w.cta, t.cta.data(), t.cta.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st),
              "upload CTA ranges");
  ragged_ref_kernel<<<plan->n_seg, PREP_THREADS, 0, st>>>(x, reinterpret_cast<const RaggedSeg*>(b + w.segs), b + w.ref);
  GB_CUDA_TRY(cudaGetLastError(), "launch ragged_ref_kernel");
  GB_CUDA_TRY(cudaStreamSynchronize(st), "sync ragged setup");
  return GBRMSD_OK;
}

int gbrmsd_ragged_rmsd(const float* x, float* out, const gbrmsd_ragged_plan_t* plan, void* ws, size_t ws_bytes,
                       void* stream) {
  clear_error();
  if (!plan || !x || !out || !ws) return set_error(GBRMSD_E_INVALID, "ragged_rmsd: null argument");
  if (ws_bytes < plan->ws_bytes) return set_error(GBRMSD_E_WORKSPACE, "ragged_rmsd: workspace smaller than the plan's");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* b = static_cast<unsigned char*>(ws);
  // region offsets are recomputed from the plan's totals (ref area size is
  // the distance between the CTA table and the sums, fixed at setup)
  const size_t segs_off = HDR_BYTES;
  const size_t cta_off = align_up(segs_off + (size_t)plan->n_seg * sizeof(RaggedSeg), 256);
  const size_t ref_off = align_up(cta_off + (size_t)(plan->grid + 1) * sizeof(int64_t), 256);
  const size_t refine_bytes = align_up((size_t)plan->total_frames * sizeof(RefineEntry), 256);
  const size_t sums_bytes = align_up((size_t)plan->total_units * SUMS_STRIDE * sizeof(double), 256);
  const size_t refine_off = plan->ws_bytes - refine_bytes;
  const size_t sums_off = refine_off - sums_bytes;
  WsHeader* hdr = reinterpret_cast<WsHeader*>(b);
  GB_CUDA_TRY(cudaMemsetAsync(hdr, 0, sizeof(WsHeader), st), "memset ragged header");
  RaggedArgs a;
  a.x = x;
  a.segs = reinterpret_cast<const RaggedSeg*>(b + segs_off);
  a.n_seg = plan->n_seg;
  a.cta_begin = reinterpret_cast<const int64_t*>(b + cta_off);
  a.ref_base = b + ref_off;
  a.sums = reinterpret_cast<double*>(b + sums_off);
  a.err = &hdr->err;
  a.wait_ns = wait_limit_ns();
  prof_begin(st);
  int rc = launch_ragged(plan->config, a, plan->grid, st);
  if (rc) return rc;
  prof_end(st);
  RaggedFinishArgs fa;
  fa.segs = a.segs;
  fa.n_seg = plan->n_seg;
  fa.total_frames = plan->total_frames;
  fa.ref_base = a.ref_base;
  fa.sums = a.sums;
  fa.out = out;
  fa.refine = reinterpret_cast<RefineEntry*>(b + refine_off);
  fa.refine_count = &hdr->refine_count;
  fa.err = &hdr->err;
  ragged_finish_kernel<<<(unsigned)((plan->total_frames + 255) / 256), 256, 0, st>>>(fa);
  GB_CUDA_TRY(cudaGetLastError(), "launch ragged_finish_kernel");
  ragged_refine_kernel<<<sm_count() * 4, 256, 0, st>>>(x, a.segs, a.ref_base, fa.refine, fa.refine_count, out);
  GB_CUDA_TRY(cudaGetLastError(), "launch ragged_refine_kernel");
  return GBRMSD_OK;
}

int gbrmsd_ragged_config_count(void) { return kNumRCfg; }

}  // extern "C"
