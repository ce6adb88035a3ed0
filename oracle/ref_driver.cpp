/*
 * ORACLE — test infrastructure only (never part of the product path).
 *
 * Thin C driver over mdtraj's own compiled CPU kernels (built from the
 * reference's sources by oracle/Makefile into oracle/_ref/): it reproduces the
 * loops that mdtraj/rmsd/_rmsd.pyx runs around them, so the reference can be
 * called without Cython:
 *   ref_md_rmsd              <- _rmsd.pyx:211-224 (centre target + reference
 *                               frame in place, prange msd_atom_major, sqrtf)
 *   ref_multiple_axis_major  <- _rmsd.pyx:546-550
 *   ref_multiple_atom_major  <- _rmsd.pyx:606-609
 *   ref_center_inplace       <- _rmsd.pyx:487-491
 * The kernels themselves (inplace_center_and_trace_atom_major, msd_atom_major,
 * msd_axis_major) are the reference's, declared in its include/center.h and
 * include/theobald_rmsd.h.
 */
#include <math.h>
#include <stdint.h>
#include <vector>

#include "center.h"
#include "theobald_rmsd.h"

extern "C" {

void ref_md_rmsd(float* target, int64_t n_frames, int32_t n_atoms, float* ref_frame, float* out) {
  std::vector<float> g((size_t)n_frames);
  float ref_g = 0.0f;
  inplace_center_and_trace_atom_major(target, g.data(), (int)n_frames, n_atoms);
  inplace_center_and_trace_atom_major(ref_frame, &ref_g, 1, n_atoms);
  int64_t i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n_frames; ++i) {
    const float msd = msd_atom_major(n_atoms, n_atoms, target + i * 3 * (int64_t)n_atoms, ref_frame, g[i], ref_g, 0, nullptr);
    out[i] = sqrtf(msd);
  }
}

void ref_multiple_axis_major(float* xyz1, float* xyz2, float* g1, float* g2, int64_t frame, int64_t n_frames,
                             int32_t n_atoms, float* out) {
  int64_t i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n_frames; ++i) {
    const float msd = msd_axis_major(n_atoms, n_atoms, n_atoms, xyz1 + frame * 3 * (int64_t)n_atoms,
                                     xyz2 + i * 3 * (int64_t)n_atoms, g1[frame], g2[i]);
    out[i] = sqrtf(msd);
  }
}

void ref_multiple_atom_major(float* xyz1, float* xyz2, float* g1, float* g2, int64_t frame, int64_t n_frames,
                             int32_t n_atoms, float* out) {
  int64_t i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n_frames; ++i) {
    const float msd = msd_atom_major(n_atoms, n_atoms, xyz1 + frame * 3 * (int64_t)n_atoms,
                                     xyz2 + i * 3 * (int64_t)n_atoms, g1[frame], g2[i], 0, nullptr);
    out[i] = sqrtf(msd);
  }
}

void ref_center_inplace(float* xyz, int64_t n_frames, int32_t n_atoms, float* traces) {
  inplace_center_and_trace_atom_major(xyz, traces, (int)n_frames, n_atoms);
}

}  // extern "C"
