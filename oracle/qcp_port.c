/*
 * ORACLE — test infrastructure only.  Never linked into or called by the
 * product path (mdtraj_gb300/).  Used by tests/ as a checker and by
 * bench.py as the timed CPU baseline ("port") when the reference's own
 * sources are not available to compile.
 *
 * A plain-C restatement of mdtraj's CPU RMSD path, float32 as in the
 * reference, OpenMP over frames:
 *   port_center_and_trace   <- mdtraj/rmsd/src/center_generic.h:3-44
 *   port_msd_atom_major     <- mdtraj/rmsd/src/theobald_rmsd_generic.h:63-119
 *   port_msd_axis_major     <- mdtraj/rmsd/src/theobald_rmsd_generic.h:7-60
 *   port_msd_from_m_and_g   <- mdtraj/rmsd/src/theobald_rmsd.cpp:217-277
 *   port_quartic_max_root   <- mdtraj/rmsd/src/theobald_rmsd.cpp:81-193
 *                              (largest root via the resolvent cubic, double)
 *   port_md_rmsd            <- mdtraj/rmsd/_rmsd.pyx:211-224 (centre target and
 *                              reference frame, then msd per frame, sqrtf)
 *   port_multiple_axis_major<- mdtraj/rmsd/_rmsd.pyx:546-550
 *   port_nosuperpose        <- mdtraj/rmsd/_rmsd.pyx:762-793
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

/* Centre each frame in place: mean accumulated in double and rounded to
 * float, subtracted in float; trace = sum of float squares, in double. */
void port_center_and_trace(float* coords, float* traces, int64_t n_frames, int32_t n_atoms) {
  int64_t f;
#pragma omp parallel for schedule(static)
  for (f = 0; f < n_frames; ++f) {
    float* c = coords + f * (int64_t)n_atoms * 3;
    double sx = 0.0, sy = 0.0, sz = 0.0, tr = 0.0;
    for (int32_t k = 0; k < n_atoms; ++k) {
      sx += c[3 * k];
      sy += c[3 * k + 1];
      sz += c[3 * k + 2];
    }
    const float mx = (float)(sx / n_atoms), my = (float)(sy / n_atoms), mz = (float)(sz / n_atoms);
    for (int32_t k = 0; k < n_atoms; ++k) {
      c[3 * k] -= mx;
      c[3 * k + 1] -= my;
      c[3 * k + 2] -= mz;
      tr += c[3 * k] * c[3 * k] + c[3 * k + 1] * c[3 * k + 1] + c[3 * k + 2] * c[3 * k + 2];
    }
    if (traces) traces[f] = (float)tr;
  }
}

/* Largest real root of the monic cubic y^3 + b y^2 + c y + d (Cardano /
 * trigonometric form). */
static double largest_cubic_root(double b, double c, double d) {
  const double q = c / 3.0 - b * b / 9.0;
  const double r = (b * c - 3.0 * d) / 6.0 - b * b * b / 27.0;
  const double disc = q * q * q + r * r;
  if (disc > 0.0) {
    const double s = sqrt(disc);
    return cbrt(r + s) + cbrt(r - s) - b / 3.0;
  }
  if (disc < 0.0) {
    const double theta = acos(r / sqrt(-q * q * q)) / 3.0;
    return 2.0 * sqrt(-q) * cos(theta) - b / 3.0;
  }
  return 2.0 * cbrt(r) - b / 3.0;
}

/* Largest root of x^4 + p x^2 + q x + r (Ferrari: (x^2 + y/2)^2 =
 * (y - p) x^2 - q x + y^2/4 - r with y the largest resolvent root).  Like the
 * reference, a complex pair contributes its real part. */
double port_quartic_max_root(double p, double q, double r) {
  const double y = largest_cubic_root(-p, -4.0 * r, 4.0 * p * r - q * q);
  const double r2 = y - p;
  double R = r2 > 0.0 ? sqrt(r2) : 0.0;
  double dd, ee;
  if (R != 0.0) {
    dd = -r2 - 2.0 * p - 2.0 * q / R;
    ee = -r2 - 2.0 * p + 2.0 * q / R;
  } else {
    const double t = 2.0 * sqrt(y * y - 4.0 * r);
    dd = -2.0 * p + t;
    ee = -2.0 * p - t;
  }
  double best = -INFINITY, v;
  if (dd >= 0.0) {
    const double D = sqrt(dd);
    v = 0.5 * R - 0.5 * D; best = v > best ? v : best;
    v = 0.5 * R + 0.5 * D; best = v > best ? v : best;
  } else {
    v = 0.5 * R; best = v > best ? v : best;
  }
  if (ee >= 0.0) {
    const double E = sqrt(ee);
    v = -0.5 * R - 0.5 * E; best = v > best ? v : best;
    v = -0.5 * R + 0.5 * E; best = v > best ? v : best;
  } else {
    v = -0.5 * R; best = v > best ? v : best;
  }
  return best;
}

/* QCP msd from the float 3x3 inner product M (row-major, M[3i+j] =
 * sum a_i b_j) and float traces, coefficients formed in float. */
float port_msd_from_m_and_g(const float* M, float ga, float gb, int32_t n_atoms) {
  const float k00 = M[0] + M[4] + M[8];
  const float k01 = M[5] - M[7];
  const float k02 = M[6] - M[2];
  const float k03 = M[1] - M[3];
  const float k11 = M[0] - M[4] - M[8];
  const float k12 = M[1] + M[3];
  const float k13 = M[6] + M[2];
  const float k22 = -M[0] + M[4] - M[8];
  const float k23 = M[5] + M[7];
  const float k33 = -M[0] - M[4] + M[8];
  float c2 = 0.0f;
  for (int i = 0; i < 9; ++i) c2 += M[i] * M[i];
  c2 *= -2.0f;
  const float det_m = M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) +
                      M[2] * (M[3] * M[7] - M[4] * M[6]);
  /* det K by complementary 2x2 minors of rows {0,1} and {2,3} */
  const float s01 = k00 * k11 - k01 * k01, s02 = k00 * k12 - k02 * k01, s03 = k00 * k13 - k03 * k01;
  const float s12 = k01 * k12 - k02 * k11, s13 = k01 * k13 - k03 * k11, s23 = k02 * k13 - k03 * k12;
  const float c01 = k02 * k13 - k12 * k03, c02 = k02 * k23 - k22 * k03, c03 = k02 * k33 - k23 * k03;
  const float c12 = k12 * k23 - k22 * k13, c13 = k12 * k33 - k23 * k13, c23 = k22 * k33 - k23 * k23;
  const float det_k = s01 * c23 - s02 * c13 + s03 * c12 + s12 * c03 - s13 * c02 + s23 * c01;
  const float c1 = -8.0f * det_m;
  const float lam = (float)port_quartic_max_root((double)c2, (double)c1, (double)det_k);
  const float msd = (ga + gb - 2.0f * lam) / (float)n_atoms;
  return msd > 0.0f ? msd : 0.0f;
}

float port_msd_atom_major(int32_t n_atoms, const float* a, const float* b, float ga, float gb) {
  if (a == b && ga == gb) return 0.0f;
  float m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int32_t k = 0; k < n_atoms; ++k) {
    const float ax = a[3 * k], ay = a[3 * k + 1], az = a[3 * k + 2];
    const float bx = b[3 * k], by = b[3 * k + 1], bz = b[3 * k + 2];
    m[0] += ax * bx; m[1] += ax * by; m[2] += ax * bz;
    m[3] += ay * bx; m[4] += ay * by; m[5] += ay * bz;
    m[6] += az * bx; m[7] += az * by; m[8] += az * bz;
  }
  return port_msd_from_m_and_g(m, ga, gb, n_atoms);
}

float port_msd_axis_major(int32_t n_atoms, int32_t rowstride, const float* a, const float* b, float ga,
                          float gb) {
  if (a == b && ga == gb) return 0.0f;
  float m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int32_t k = 0; k < n_atoms; ++k) {
    const float ax = a[k], ay = a[rowstride + k], az = a[2 * rowstride + k];
    const float bx = b[k], by = b[rowstride + k], bz = b[2 * rowstride + k];
    m[0] += ax * bx; m[1] += ax * by; m[2] += ax * bz;
    m[3] += ay * bx; m[4] += ay * by; m[5] += ay * bz;
    m[6] += az * bx; m[7] += az * by; m[8] += az * bz;
  }
  return port_msd_from_m_and_g(m, ga, gb, n_atoms);
}

/* md.rmsd(target, reference, frame) with precentered=False: centres the
 * target frames and the reference frame in place, then rmsd per frame. */
void port_md_rmsd(float* target, int64_t n_frames, int32_t n_atoms, float* ref_frame, float* out) {
  float ref_g = 0.0f;
  float* traces = out; /* traces are written to out first, then overwritten */
  port_center_and_trace(target, traces, n_frames, n_atoms);
  port_center_and_trace(ref_frame, &ref_g, 1, n_atoms);
  int64_t f;
#pragma omp parallel for schedule(static)
  for (f = 0; f < n_frames; ++f) {
    const float ga = traces[f];
    const float msd = port_msd_atom_major(n_atoms, target + f * (int64_t)n_atoms * 3, ref_frame, ga, ref_g);
    out[f] = sqrtf(msd);
  }
}

/* getMultipleRMSDs_axis_major: rmsd of xyz1[frame] to every xyz2[i]. */
void port_multiple_axis_major(const float* xyz1, const float* xyz2, const float* g1, const float* g2,
                              int64_t frame, int64_t n_frames, int32_t n_atoms, float* out) {
  const float* a = xyz1 + frame * 3 * (int64_t)n_atoms;
  int64_t i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n_frames; ++i) {
    const float msd = port_msd_axis_major(n_atoms, n_atoms, a, xyz2 + i * 3 * (int64_t)n_atoms, g1[frame], g2[i]);
    out[i] = sqrtf(msd);
  }
}

/* getMultipleRMSDs_atom_major. */
void port_multiple_atom_major(const float* xyz1, const float* xyz2, const float* g1, const float* g2,
                              int64_t frame, int64_t n_frames, int32_t n_atoms, float* out) {
  const float* a = xyz1 + frame * 3 * (int64_t)n_atoms;
  int64_t i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n_frames; ++i) {
    const float msd = port_msd_atom_major(n_atoms, a, xyz2 + i * 3 * (int64_t)n_atoms, g1[frame], g2[i]);
    out[i] = sqrtf(msd);
  }
}

/* md.rmsd(..., superpose=False): plain float mean square deviation. */
void port_nosuperpose(const float* target, int64_t n_frames, int32_t n_atoms, const float* ref_frame, float* out) {
  int64_t f;
#pragma omp parallel for schedule(static)
  for (f = 0; f < n_frames; ++f) {
    const float* a = target + f * 3 * (int64_t)n_atoms;
    float s = 0.0f;
    for (int32_t k = 0; k < n_atoms; ++k)
      for (int c = 0; c < 3; ++c) {
        const float d = a[3 * k + c] - ref_frame[3 * k + c];
        s += d * d;
      }
    out[f] = sqrtf(s / n_atoms);
  }
}
