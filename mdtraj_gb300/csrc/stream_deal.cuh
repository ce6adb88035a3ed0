// Dealing of the streaming kernel's units (frames, or parts of frames) to
// its warps, and the per-CTA frame order of the in-kernel finish.  Plain
// integer arithmetic, __host__ __device__: the kernel evaluates it with
// gridDim / blockIdx, and tests/stream_deal_check.cu on the host checks that
// every unit is dealt exactly once and that each CTA's local order maps back
// to the frames its warps streamed.
//
// W = grid x warps warps take the units in rounds: warp g takes g, g + W,
// g + 2W, ... (full_rounds = units / W rounds).  The partial last round
// (units - full_units units) goes to the highest warps: warp g >= part_shift
// takes unit full_units + g - part_shift, so frames near the start (in
// md.rmsd's use often the ones closest to the reference, which the finish
// refines) sit in CTAs that stream one round less.
#pragma once

#include <stdint.h>

namespace gb {

#if defined(__CUDACC__)
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD inline
#endif

struct Deal {
  int64_t units;        // units to deal
  int64_t full_rounds;  // units / W
  int64_t full_units;   // full_rounds * W
  int64_t part_shift;   // W - (units - full_units): first warp with a partial-round unit
};

GB_HD Deal make_deal(int64_t units, int64_t W) {
  Deal d;
  d.units = units;
  d.full_rounds = units / W;
  d.full_units = d.full_rounds * W;
  d.part_shift = W - (units - d.full_units);
  return d;
}

// The unit dealt at round position v = g + k W (warp g, round k); `units`
// (one past the last) when warp g has no unit in that round.
GB_HD int64_t deal_place(int64_t v, int64_t full_units, int64_t part_shift, int64_t units) {
  if (v < full_units) return v;
  const int64_t g = v - full_units;  // < W for every round position a warp reaches
  return g >= part_shift ? v - part_shift : units;
}

// The unit a warp takes after unit u (a unit of the partial round is a
// warp's last).
GB_HD int64_t deal_next(int64_t u, int64_t W, int64_t full_units, int64_t part_shift, int64_t units) {
  return u >= full_units ? units : deal_place(u + W, full_units, part_shift, units);
}

// One CTA's frames with one unit per frame (the in-kernel finish): warp w's
// k-th frame is b0 + w + k W for k < full, and in the partial round (warps
// w >= w0 only) full W + b0 + w - shift.  Local index i (the order of the
// CTA's records and of its finish): w + k warps for k < full, then
// full warps + w - w0.
struct FinSlice {
  int64_t n;      // frames of this CTA
  int64_t base;   // first refinement-list entry of this CTA (frames of lower CTAs)
  int64_t full;   // full rounds
  int64_t shift;  // W - (frames of the partial round)
  int64_t w0;     // first warp of this CTA with a frame in the partial round
};

GB_HD int64_t deal_min(int64_t a, int64_t b) { return a < b ? a : b; }
GB_HD int64_t deal_max(int64_t a, int64_t b) { return a > b ? a : b; }

GB_HD FinSlice fin_slice_of(int64_t F, int64_t grid, int64_t block, int warps) {
  const int64_t W = grid * warps;
  const int64_t b0 = block * warps;
  FinSlice s;
  s.full = F / W;
  s.shift = W - (F - s.full * W);
  s.w0 = deal_min((int64_t)warps, deal_max((int64_t)0, s.shift - b0));
  s.n = s.full * warps + (warps - s.w0);
  s.base = s.full * warps * block + deal_max((int64_t)0, b0 - s.shift);
  return s;
}

// Frame of local index i of CTA `block`.
GB_HD int64_t fin_frame_of(const FinSlice& s, int64_t i, int64_t grid, int64_t block, int warps) {
  const int64_t W = grid * warps;
  const int64_t b0 = block * warps;
  if (i < s.full * warps) return b0 + (i % warps) + (i / warps) * W;
  return s.full * W + b0 + (i - s.full * warps + s.w0) - s.shift;
}

// Local index of the k-th frame streamed by warp `warp` of CTA `block`.
GB_HD int64_t fin_local_index(int64_t k, int warp, int64_t full_rounds, int64_t part_shift, int64_t block,
                              int warps) {
  if (k < full_rounds) return warp + k * warps;
  const int64_t w0 = deal_min((int64_t)warps, deal_max((int64_t)0, part_shift - block * warps));
  return full_rounds * warps + warp - w0;
}

// Record slots of the CTA with the most frames (fin_slice_of's n is largest
// for the CTAs whose warps all have a partial-round frame).
GB_HD int64_t fin_max_frames(int64_t F, int64_t grid, int warps) {
  const int64_t W = grid * warps;
  return (F / W) * warps + deal_min((int64_t)warps, F % W);
}

#undef GB_HD

}  // namespace gb
