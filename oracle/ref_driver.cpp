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
 *   ref_superpose_atom_major <- _rmsd.pyx:664-674 (prange msd_atom_major with
 *                               computeRot = 1, then rot_atom_major)
 *   ref_rmsf_rotated         <- _rmsd.pyx:419-451 (prange rotations of the
 *                               displaced copy, per-atom mean and mean squared
 *                               deviation in float, sqrtf)
 * The kernels themselves (inplace_center_and_trace_atom_major, msd_atom_major,
 * msd_axis_major, rot_atom_major) are the reference's, declared in its
 * include/center.h, include/theobald_rmsd.h and include/rotation.h.
 */
#include <math.h>
#include <stdint.h>
#include <vector>

#include "center.h"
#include "rotation.h"
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

void ref_superpose_atom_major(const float* align_target_frame, const float* align_mobile, float g_target,
                              const float* g_mobile, float* displace, int64_t n_frames, int32_t n_align,
                              int32_t n_displace) {
  std::vector<float> rot((size_t)n_frames * 9);
  int64_t i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n_frames; ++i) {
    msd_atom_major(n_align, n_align, align_mobile + i * 3 * (int64_t)n_align, align_target_frame, g_target,
                   g_mobile[i], 1, rot.data() + 9 * i);
    rot_atom_major(n_displace, displace + i * 3 * (int64_t)n_displace, rot.data() + 9 * i);
  }
}

void ref_rmsf_rotated(const float* centred, const float* ref_frame, float ref_g, const float* g, float* displaced,
                      int64_t n_frames, int32_t n_atoms, int32_t rotate, float* out) {
  std::vector<float> rot((size_t)n_frames * 9);
  std::vector<float> avg((size_t)n_atoms * 3, 0.0f);
  int64_t i;
  if (rotate) {
#pragma omp parallel for schedule(static)
    for (i = 0; i < n_frames; ++i) {
      msd_atom_major(n_atoms, n_atoms, centred + i * 3 * (int64_t)n_atoms, ref_frame, ref_g, g[i], 1,
                     rot.data() + 9 * i);
      rot_atom_major(n_atoms, displaced + i * 3 * (int64_t)n_atoms, rot.data() + 9 * i);
    }
  }
  const int nf = (int)n_frames;
  int32_t j;
#pragma omp parallel for schedule(static)
  for (j = 0; j < n_atoms; ++j) {
    for (int64_t f = 0; f < n_frames; ++f)
      for (int c = 0; c < 3; ++c) avg[3 * j + c] += displaced[(f * n_atoms + j) * 3 + c] / nf;
    float fl = 0.0f;
    for (int64_t f = 0; f < n_frames; ++f) {
      const float* p = displaced + (f * n_atoms + j) * 3;
      fl += ((p[0] - avg[3 * j]) * (p[0] - avg[3 * j]) + (p[1] - avg[3 * j + 1]) * (p[1] - avg[3 * j + 1]) +
             (p[2] - avg[3 * j + 2]) * (p[2] - avg[3 * j + 2])) / nf;
    }
    out[j] = sqrtf(fl);
  }
}

}  // extern "C"
