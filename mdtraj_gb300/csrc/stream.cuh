// Single-reference streaming RMSD path: declarations shared between the
// kernel translation unit and the C-ABI layer.
#pragma once

#include <stdint.h>

namespace gb {

enum Layout : int { ATOM_MAJOR = 0, AXIS_MAJOR = 1 };

// What the streaming pass accumulates per frame.
enum Mode : int {
  MODE_CENTER = 0,       // md.rmsd default: centroid + trace + M in one pass
  MODE_PRECENTERED = 1,  // frames already centred, traces supplied: M only
  MODE_NOSUPERPOSE = 2,  // sum |a - b|^2, no alignment
  MODE_TRACE = 3,        // exact centroid only (first pass of in-place centring)
};

constexpr int SUMS_STRIDE = 20;   // doubles per (frame, split) partial record

// Per-reference information produced by the reference preparation kernel.
struct RefInfo {
  double g;          // sum |b_k|^2 of the (centred) reference, FP64
  double sum[3];     // sum b_k, FP64 (not exactly zero after float centring)
  float centroid[3]; // float centroid that was subtracted (0 when not centred)
  int32_t n_atoms;
  int32_t n_padded;
  int32_t layout;
  int32_t centred;
  float g_hi, g_lo;          // g and sum as float pairs (hi + lo), for
  float sum_hi[3], sum_lo[3];  // finishes that use no FP64
};

// A frame whose QCP msd is too small for the one-pass sums to resolve; the
// refinement pass recomputes it as sum |R (a - mu) - b|^2 / n directly.
struct RefineEntry {
  int64_t frame;   // frame index (global frame index on the ragged path)
  float rot[9];
  float mu_hi[3];
  float mu_lo[3];
  int32_t seg;     // segment of the frame (ragged path; 0 otherwise)
};

struct StreamArgs {
  const float* x;        // frames, padded layout, 16-byte aligned
  int64_t n_frames;
  int32_t n_atoms;
  int32_t n_padded;      // atoms per frame in memory (multiple of 4)
  int64_t frame_stride;  // floats between consecutive frames (multiple of 4)
  const float* ref;      // prepared reference in the same layout (zero padded)
  int32_t splits;        // partial records per frame
  double* sums;          // [n_frames * splits][SUMS_STRIDE]
  int* err;
  uint64_t wait_ns;      // limit of each bounded wait (gbrmsd_set_wait_limit_ns)
  int64_t skip_unit;     // failure-detection test hook: the first chunk of this
                         // unit is never issued (-1: off)
  // Dealing of the units to the warps (stream_deal.cuh, make_deal), set by
  // the launcher.
  int64_t full_units;
  int64_t part_shift;
  int64_t full_rounds;
};

// Process-wide settings of the failure-detection hooks (stream.cu).
uint64_t wait_limit_ns();
int64_t skip_unit_hook();

struct FinishArgs {
  int64_t n_frames;
  int32_t n_atoms;
  double inv_atoms;           // 1 / n_atoms
  int32_t splits;
  const double* sums;
  const RefInfo* ref_info;
  const double* ref_prefix;   // (quads + 1) x 3 prefix sums of the reference
  const float* g_target;      // MODE_PRECENTERED: supplied per-frame traces
  float g_ref_override;       // MODE_PRECENTERED: supplied reference trace
  int64_t self_index;         // frame that aliases the reference (-1: none)
  float* out_rmsd;
  float* out_centroid;        // optional, n_frames x 3
  float* out_trace;           // optional, n_frames
  RefineEntry* refine;
  int* refine_count;
  int* err;
  int32_t mode;
  float* out_rot;             // optional, n_frames x 9 (superposition)
  double* out_mu;             // optional with out_rot, n_frames x 3
  float inv_hi, inv_lo;       // 1 / n_atoms as a float pair (in-kernel finish)
  int32_t rec_smem;           // in-kernel finish: records in shared memory (1) or in sums (0)
};

}  // namespace gb
