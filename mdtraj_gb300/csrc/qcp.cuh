// Quaternion characteristic polynomial (QCP) solve, FP64, one structure pair
// per thread.
//
// Follows Theobald, Acta Cryst. A61:478 (2005) as used by mdtraj's
// msdFromMandG (mdtraj/rmsd/src/theobald_rmsd.cpp:217-334): the 4x4 key
// matrix K is built from the 3x3 inner-product matrix M = sum_k a_k b_k^T,
// its characteristic polynomial is
//     P(l) = l^4 + C2 l^2 + C1 l + C0,  C2 = -2 |M|_F^2, C1 = -8 det M, C0 = det K,
// and msd = (G_a + G_b - 2 lambda_max) / n_atoms.  The reference forms the
// coefficients in float32 and solves the quartic in closed form
// (theobald_rmsd.cpp:81-193); here everything is FP64 and lambda_max is found
// by Newton's method from the upper bound (G_a + G_b) / 2, which converges
// monotonically from above (all roots lie below the start).
#pragma once

#include "common.cuh"

namespace gb {

struct Key4 {
  double k00, k01, k02, k03, k11, k12, k13, k22, k23, k33;
};

// K(M) with M row-major, M[3*i + j] = sum_k a_k[i] * b_k[j]
// (same entry layout as theobald_rmsd.cpp:227-236).
__host__ __device__ __forceinline__ Key4 key_matrix(const double* m) {
  Key4 k;
  k.k00 = m[0] + m[4] + m[8];
  k.k01 = m[5] - m[7];
  k.k02 = m[6] - m[2];
  k.k03 = m[1] - m[3];
  k.k11 = m[0] - m[4] - m[8];
  k.k12 = m[1] + m[3];
  k.k13 = m[6] + m[2];
  k.k22 = -m[0] + m[4] - m[8];
  k.k23 = m[5] + m[7];
  k.k33 = -m[0] - m[4] + m[8];
  return k;
}

// Determinant of a symmetric 4x4 via complementary 2x2 minors of rows {0,1}
// and {2,3}.
__host__ __device__ __forceinline__ double det_sym4(const Key4& k) {
  const double r0[4] = {k.k00, k.k01, k.k02, k.k03};
  const double r1[4] = {k.k01, k.k11, k.k12, k.k13};
  const double r2[4] = {k.k02, k.k12, k.k22, k.k23};
  const double r3[4] = {k.k03, k.k13, k.k23, k.k33};
  const double s01 = r0[0] * r1[1] - r0[1] * r1[0];
  const double s02 = r0[0] * r1[2] - r0[2] * r1[0];
  const double s03 = r0[0] * r1[3] - r0[3] * r1[0];
  const double s12 = r0[1] * r1[2] - r0[2] * r1[1];
  const double s13 = r0[1] * r1[3] - r0[3] * r1[1];
  const double s23 = r0[2] * r1[3] - r0[3] * r1[2];
  const double c01 = r2[0] * r3[1] - r2[1] * r3[0];
  const double c02 = r2[0] * r3[2] - r2[2] * r3[0];
  const double c03 = r2[0] * r3[3] - r2[3] * r3[0];
  const double c12 = r2[1] * r3[2] - r2[2] * r3[1];
  const double c13 = r2[1] * r3[3] - r2[3] * r3[1];
  const double c23 = r2[2] * r3[3] - r2[3] * r3[2];
  return s01 * c23 - s02 * c13 + s03 * c12 + s12 * c03 - s13 * c02 + s23 * c01;
}

__host__ __device__ __forceinline__ double det3(const double* m) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}

// Largest eigenvalue of K(M), by Newton on the characteristic quartic.
// Returns the iteration count through *iters (capped at max_iter).
__host__ __device__ __forceinline__ double qcp_lambda_max(const double* m, double ga, double gb,
                                                          int* iters, int max_iter = 60) {
  const Key4 k = key_matrix(m);
  double c2 = 0.0;
#pragma unroll
  for (int i = 0; i < 9; ++i) c2 += m[i] * m[i];
  c2 *= -2.0;
  const double c1 = -8.0 * det3(m);
  const double c0 = det_sym4(k);
  double lam = 0.5 * (ga + gb);
  int it = 0;
  for (; it < max_iter; ++it) {
    const double l2 = lam * lam;
    const double b = (l2 + c2) * lam;
    const double a = b + c1;
    const double p = a * lam + c0;            // P(lam)
    const double dp = 2.0 * l2 * lam + b + a; // P'(lam)
    if (!(dp != 0.0)) break;
    // P(lam) at its rounding floor: lam is a root to working precision (at
    // a double root, as for collinear structures, P' is rounding noise too
    // and a step would be noise over noise)
    if (fabs(p) <= 32.0 * 2.220446049250313e-16 * (l2 * l2 + fabs(c2) * l2 + fabs(c1 * lam) + fabs(c0))) break;
    const double step = p / dp;
    lam -= step;
    if (!(fabs(step) > 1e-15 * fabs(lam))) {
      ++it;
      break;
    }
  }
  if (iters) *iters = it;
  return lam;
}

// Same root, cheaper on GB300's narrow FP64 pipe: Newton runs in FP32 on
// the quartic normalised by its upper bound lam0 = (G_a + G_b) / 2 (so the
// root is near 1 and nothing overflows), then FP64 Newton steps on the
// original FP64 coefficients polish it to double precision (quadratic
// convergence from a 1e-7-accurate start: usually one or two steps).
// No FP64 division: the normalisation only has to be close to 1 / lam0 (the
// polish works on the unnormalised quartic), and a polish step of relative
// size ~1e-7 needs its quotient to FP32 precision only (an error of 1e-7 in
// a step of 1e-7 * lam moves lam by 1e-14 relative), so both use an FP32
// reciprocal; FP64 division remains only where FP32 would over- or
// underflow.
__host__ __device__ __forceinline__ double qcp_lambda_max_mixed(const double* m, double ga, double gb,
                                                                int* iters, int max_iter = 60) {
  const Key4 k = key_matrix(m);
  double c2 = 0.0;
#pragma unroll
  for (int i = 0; i < 9; ++i) c2 += m[i] * m[i];
  c2 *= -2.0;
  const double c1 = -8.0 * det3(m);
  const double c0 = det_sym4(k);
  const double lam0 = 0.5 * (ga + gb);
  if (!(lam0 > 0.0)) {
    if (iters) *iters = 0;
    return 0.0;
  }
  const float lam0f = (float)lam0;
  double inv = (double)(1.0f / lam0f);
  if (!(lam0f > 1e-30f) || !(lam0f < 1e30f)) inv = 1.0 / lam0;
  const double inv2 = inv * inv;
  const float a2 = (float)(c2 * inv2);
  const float a1 = (float)(c1 * inv2 * inv);
  const float a0 = (float)(c0 * inv2 * inv2);
  // start at the tighter of the upper bounds 1 and sqrt(3) |M|_F / lam0 =
  // sqrt(-1.5 a2) (K is traceless: lambda_max <= sqrt(3/4 tr K^2)), nudged
  // up by 2^-20 against rounding; Newton from above converges monotonically
  float x = fminf(1.0f, sqrtf(-1.5f * a2) * 1.00000095f);
  int it = 0;
  for (; it < 40; ++it) {
    const float x2 = x * x;
    const float b = (x2 + a2) * x;
    const float a = b + a1;
    const float pv = a * x + a0;
    const float dp = 2.0f * x2 * x + b + a;
    if (!(dp != 0.0f)) break;
    // at the rounding floor of P: x is a root to FP32 precision (see the
    // FP64 loop below); starting from the upper bound, it is the largest
    if (fabsf(pv) <= 32.0f * 1.1920929e-7f * (x2 * x2 + fabsf(a2) * x2 + fabsf(a1 * x) + fabsf(a0))) break;
#ifdef __CUDA_ARCH__
    const float step = __fdividef(pv, dp);
#else
    const float step = pv / dp;
#endif
    x -= step;
    if (!(fabsf(step) > 3e-7f * fabsf(x))) break;
  }
  double lam = (double)x * lam0;
  int jt = 0;
  for (; jt < max_iter; ++jt) {
    const double l2 = lam * lam;
    const double b = (l2 + c2) * lam;
    const double a = b + c1;
    const double pv = a * lam + c0;
    const double dp = 2.0 * l2 * lam + b + a;
    if (!(dp != 0.0)) break;
    // P(lam) at its rounding floor: lam is a root to working precision (at
    // a double root, as for collinear structures, P' is rounding noise too
    // and a step would be noise over noise)
    if (fabs(pv) <= 32.0 * 2.220446049250313e-16 * (l2 * l2 + fabs(c2) * l2 + fabs(c1 * lam) + fabs(c0))) break;
    const float dpf = (float)fabs(dp);
    const double step = (dpf > 1e-30f && dpf < 1e30f) ? pv * (double)(1.0f / (float)dp) : pv / dp;
    lam -= step;
    if (!(fabs(step) > 1e-15 * fabs(lam))) {
      ++jt;
      break;
    }
  }
  if (iters) *iters = it + jt;
  return lam;
}

// ---------------------------------------------------------------------------
// The same solve with no FP64 arithmetic past the inputs.  On GB300 an FP64
// instruction (conversions included) costs ~64 cycles of its SM sub-
// partition's pipe, against ~4.6 for FP32 (measured: dependent DFMA chains
// 64 cycles per operation, FFMA 4.6), and the coefficient build above is
// ~70 of them: it made the per-frame finish ~20 us of the 10,000-frame
// call.  Here the coefficients and the final Newton steps run in
// float-float arithmetic (an unevaluated sum hi + lo of two floats, ~48
// significant bits, error-free transformations with FMA: Dekker, Knuth),
// which is ample: msd = (Ga + Gb - 2 lambda) / n loses at most ~1e4 of
// relative accuracy to cancellation before the finish sends a frame to the
// direct residual, and 2^-44 * 1e4 is far below float32's 6e-8.
// ---------------------------------------------------------------------------

struct DF {
  float hi, lo;
};

// Rounded float operations that the compiler may not fuse into an FMA (a
// fused product would break the error-free transformations below).  The
// host build (tests only) is compiled with contraction off.
#ifdef __CUDA_ARCH__
#define GB_FADD(a, b) __fadd_rn((a), (b))
#define GB_FSUB(a, b) __fsub_rn((a), (b))
#define GB_FMUL(a, b) __fmul_rn((a), (b))
#else
#define GB_FADD(a, b) ((a) + (b))
#define GB_FSUB(a, b) ((a) - (b))
#define GB_FMUL(a, b) ((a) * (b))
#endif

// s + e == a + b exactly (Knuth)
__host__ __device__ __forceinline__ DF df_two_sum(float a, float b) {
  const float s = GB_FADD(a, b);
  const float bb = GB_FSUB(s, a);
  return DF{s, GB_FADD(GB_FSUB(a, GB_FSUB(s, bb)), GB_FSUB(b, bb))};
}
// the same for |a| >= |b| (Dekker)
__host__ __device__ __forceinline__ DF df_fast_two_sum(float a, float b) {
  const float s = GB_FADD(a, b);
  return DF{s, GB_FSUB(b, GB_FSUB(s, a))};
}
__host__ __device__ __forceinline__ DF df_from_double(double d) {
  const float h = (float)d;
  return DF{h, (float)(d - (double)h)};
}
__host__ __device__ __forceinline__ double df_to_double(DF a) { return (double)a.hi + (double)a.lo; }
__host__ __device__ __forceinline__ DF df_neg(DF a) { return DF{-a.hi, -a.lo}; }
__host__ __device__ __forceinline__ DF df_add(DF a, DF b) {
  DF s = df_two_sum(a.hi, b.hi);
  return df_fast_two_sum(s.hi, GB_FADD(s.lo, GB_FADD(a.lo, b.lo)));
}
__host__ __device__ __forceinline__ DF df_sub(DF a, DF b) { return df_add(a, df_neg(b)); }
__host__ __device__ __forceinline__ DF df_add_f(DF a, float b) {
  DF s = df_two_sum(a.hi, b);
  return df_fast_two_sum(s.hi, GB_FADD(s.lo, a.lo));
}
// product with the exact error of hi * hi from an FMA
__host__ __device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = GB_FMUL(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}
__host__ __device__ __forceinline__ DF df_mul_f(DF a, float b) {
  const float p = GB_FMUL(a.hi, b);
  const float e = fmaf(a.lo, b, fmaf(a.hi, b, -p));
  return df_fast_two_sum(p, e);
}
// a b - c d
__host__ __device__ __forceinline__ DF df_det2(DF a, DF b, DF c, DF d) { return df_sub(df_mul(a, b), df_mul(c, d)); }
__host__ __device__ __forceinline__ float df_abs_hi(DF a) { return fabsf(a.hi); }

// FP64 Newton on the quartic from a start above (or at) the largest root,
// until P reaches its FP64 rounding floor: the polish of
// qcp_lambda_max_df's result where that one stops short (below).
__host__ __device__ __forceinline__ double qcp_newton_fp64(const double* m, double lam, int max_iter = 60) {
  double c2 = 0.0;
#pragma unroll
  for (int i = 0; i < 9; ++i) c2 += m[i] * m[i];
  c2 *= -2.0;
  const double c1 = -8.0 * det3(m);
  const double c0 = det_sym4(key_matrix(m));
  for (int it = 0; it < max_iter; ++it) {
    const double l2 = lam * lam;
    const double b = (l2 + c2) * lam;
    const double a = b + c1;
    const double p = a * lam + c0;
    const double dp = 2.0 * l2 * lam + b + a;
    if (!(dp != 0.0)) break;
    if (fabs(p) <= 32.0 * 2.220446049250313e-16 * (l2 * l2 + fabs(c2) * l2 + fabs(c1 * lam) + fabs(c0))) break;
    const double step = p / dp;
    lam -= step;
    if (!(fabs(step) > 1e-15 * fabs(lam))) break;
  }
  return lam;
}

// lambda_max as qcp_lambda_max_mixed, on float-float coefficients: FP32
// Newton on the normalised quartic, then float-float Newton steps on P
// (float-float P, float P') until P reaches its rounding floor or the step
// is below 2^-44 lambda.  M and lam0 = (G_a + G_b) / 2 come as float pairs
// and lambda is returned as one: no FP64 instruction at all.
// At a (near) double largest root, as for (nearly) collinear structures,
// Newton converges only linearly and P's floor stops it ~sqrt(2^-44) ~ 1e-6
// (relative) short of the root, 8x further than FP64's floor does; *short_
// is then set (the last step was still above 1e-9 lambda, or the steps ran
// out) and the caller polishes with qcp_newton_fp64.
__host__ __device__ __forceinline__ DF qcp_lambda_max_dfm(const DF (&m)[9], DF lam0, int* iters, bool* short_,
                                                         int max_iter = 24) {
  *short_ = false;
  if (!(lam0.hi > 0.0f)) {
    if (iters) *iters = 0;
    return DF{0.0f, 0.0f};
  }
  // K (theobald_rmsd.cpp:227-236 entry layout)
  const DF k00 = df_add(df_add(m[0], m[4]), m[8]), k01 = df_sub(m[5], m[7]), k02 = df_sub(m[6], m[2]);
  const DF k03 = df_sub(m[1], m[3]), k11 = df_sub(df_sub(m[0], m[4]), m[8]), k12 = df_add(m[1], m[3]);
  const DF k13 = df_add(m[6], m[2]), k22 = df_sub(df_sub(m[4], m[0]), m[8]), k23 = df_add(m[5], m[7]);
  const DF k33 = df_sub(df_sub(m[8], m[0]), m[4]);
  DF c2 = df_mul(m[0], m[0]);
#pragma unroll
  for (int i = 1; i < 9; ++i) c2 = df_add(c2, df_mul(m[i], m[i]));
  c2 = df_mul_f(c2, -2.0f);
  const DF d3 = df_add(df_sub(df_mul(m[0], df_det2(m[4], m[8], m[5], m[7])), df_mul(m[1], df_det2(m[3], m[8], m[5], m[6]))),
                       df_mul(m[2], df_det2(m[3], m[7], m[4], m[6])));
  const DF c1 = df_mul_f(d3, -8.0f);
  // det K from the complementary 2x2 minors of rows {0,1} and {2,3}
  const DF s01 = df_det2(k00, k11, k01, k01), s02 = df_det2(k00, k12, k02, k01), s03 = df_det2(k00, k13, k03, k01);
  const DF s12 = df_det2(k01, k12, k02, k11), s13 = df_det2(k01, k13, k03, k11), s23 = df_det2(k02, k13, k03, k12);
  const DF q01 = df_det2(k02, k13, k12, k03), q02 = df_det2(k02, k23, k22, k03), q03 = df_det2(k02, k33, k23, k03);
  const DF q12 = df_det2(k12, k23, k22, k13), q13 = df_det2(k12, k33, k23, k13), q23 = df_det2(k22, k33, k23, k23);
  DF c0 = df_mul(s01, q23);
  c0 = df_sub(c0, df_mul(s02, q13));
  c0 = df_add(c0, df_mul(s03, q12));
  c0 = df_add(c0, df_mul(s12, q03));
  c0 = df_sub(c0, df_mul(s13, q02));
  c0 = df_add(c0, df_mul(s23, q01));
  // FP32 Newton on the quartic normalised by lam0 (root near 1, no overflow)
  const float inv = 1.0f / lam0.hi;
  const float inv2 = inv * inv;
  const float a2 = c2.hi * inv2;
  const float a1 = c1.hi * inv2 * inv;
  const float a0 = c0.hi * inv2 * inv2;
  float x = fminf(1.0f, sqrtf(-1.5f * a2) * 1.00000095f);
  int it = 0;
  for (; it < 40; ++it) {
    const float x2 = x * x;
    const float b = (x2 + a2) * x;
    const float a = b + a1;
    const float pv = a * x + a0;
    const float dp = 2.0f * x2 * x + b + a;
    if (!(dp != 0.0f)) break;
    if (fabsf(pv) <= 32.0f * 1.1920929e-7f * (x2 * x2 + fabsf(a2) * x2 + fabsf(a1 * x) + fabsf(a0))) break;
    const float step = pv / dp;
    x -= step;
    if (!(fabsf(step) > 3e-7f * fabsf(x))) break;
  }
  DF lam = df_mul_f(lam0, x);
  int jt = 0;
  float last = 0.0f;
  bool done = false;
  for (; jt < max_iter; ++jt) {
    const DF l2 = df_mul(lam, lam);
    const DF pv = df_add(df_mul(df_add(df_mul(df_add(l2, c2), lam), c1), lam), c0);
    const float lf = lam.hi, l2f = l2.hi;
    const float dp = 4.0f * l2f * lf + 2.0f * c2.hi * lf + c1.hi;
    if (!(dp != 0.0f)) break;
    // P at its rounding floor (~2^-44 of its terms): lam is a root to
    // working precision; at a double root P' is noise too and a step would
    // be noise over noise.  Converged when the last step was already tiny
    // or the Newton correction P / P' is (a simple root reached in one
    // step, as from FP32 Newton's 1e-7 start); at a (near) double root P'
    // is as small as P's noise allows and the correction stays large.
    if (fabsf(pv.hi) <= 4.5e-13f * (l2f * l2f + fabsf(c2.hi) * l2f + fabsf(c1.hi * lf) + fabsf(c0.hi))) {
      done = !(fabsf(last) > 1e-9f * fabsf(lf)) || fabsf(pv.hi + pv.lo) <= 1e-9f * fabsf(lf * dp);
      break;
    }
    const float step = (pv.hi + pv.lo) / dp;
    lam = df_add_f(lam, -step);
    last = step;
    if (!(fabsf(step) > 5.7e-14f * fabsf(lam.hi))) {
      ++jt;
      done = true;
      break;
    }
  }
  *short_ = !done;
  if (iters) *iters = it + jt;
  return lam;
}

// The same from FP64 inputs, converted once (33 FP64 operations).
__host__ __device__ __forceinline__ double qcp_lambda_max_df(const double* md, double gad, double gbd, int* iters,
                                                             bool* short_, int max_iter = 24) {
  DF m[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) m[i] = df_from_double(md[i]);
  const DF lam0 = df_mul_f(df_add(df_from_double(gad), df_from_double(gbd)), 0.5f);
  return df_to_double(qcp_lambda_max_dfm(m, lam0, iters, short_, max_iter));
}

// Rotation R (row-major) minimising sum_k |R a_k - b_k|^2 for the given
// lambda_max: the quaternion is the null vector of B = K - lambda I, taken as
// the row of adj(B) with the largest diagonal entry (adj(B) = c v v^T when
// lambda is a simple eigenvalue, so that row is c v_i v with the largest
// |v_i|).  The adjugate entries come from the twelve 2x2 minors of rows
// {0,1} and {2,3} (Laplace expansion), ~70 FP64 operations instead of the 16
// 3x3 cofactors (~220).  Returns false when B has no well-defined null vector
// (all four diagonal cofactors vanish even after the shift below), in which
// case R is the identity.
__host__ __device__ __forceinline__ double qcp_adj_row(const Key4& k, double lam, double (&q)[4]) {
  const double b00 = k.k00 - lam, b11 = k.k11 - lam, b22 = k.k22 - lam, b33 = k.k33 - lam;
  const double b01 = k.k01, b02 = k.k02, b03 = k.k03, b12 = k.k12, b13 = k.k13, b23 = k.k23;
  const double u0 = b00 * b11 - b01 * b01, u1 = b00 * b12 - b01 * b02, u2 = b00 * b13 - b01 * b03;
  const double u3 = b01 * b12 - b11 * b02, u4 = b01 * b13 - b11 * b03, u5 = b02 * b13 - b12 * b03;
  const double w5 = b22 * b33 - b23 * b23, w4 = b12 * b33 - b13 * b23, w3 = b12 * b23 - b13 * b22;
  const double w2 = b02 * b33 - b03 * b23, w1 = b02 * b23 - b03 * b22, w0 = b02 * b13 - b03 * b12;
  const double a00 = b11 * w5 - b12 * w4 + b13 * w3;
  const double a11 = b00 * w5 - b02 * w2 + b03 * w1;
  const double a22 = b03 * u4 - b13 * u2 + b33 * u0;
  const double a33 = b02 * u3 - b12 * u1 + b22 * u0;
  double best = fabs(a00);
  q[0] = a00;
  q[1] = -b01 * w5 + b02 * w4 - b03 * w3;
  q[2] = b13 * u5 - b23 * u4 + b33 * u3;
  q[3] = -b12 * u5 + b22 * u4 - b23 * u3;
  if (fabs(a11) > best) {
    best = fabs(a11);
    q[0] = -b01 * w5 + b12 * w2 - b13 * w1;
    q[1] = a11;
    q[2] = -b03 * u5 + b23 * u2 - b33 * u1;
    q[3] = b02 * u5 - b22 * u2 + b23 * u1;
  }
  if (fabs(a22) > best) {
    best = fabs(a22);
    q[0] = b01 * w4 - b11 * w2 + b13 * w0;
    q[1] = -b00 * w4 + b01 * w2 - b03 * w0;
    q[2] = a22;
    q[3] = -b02 * u4 + b12 * u2 - b23 * u0;
  }
  if (fabs(a33) > best) {
    q[0] = -b01 * w3 + b11 * w1 - b12 * w0;
    q[1] = b00 * w3 - b01 * w1 + b02 * w0;
    q[2] = -b03 * u3 + b13 * u1 - b23 * u0;
    q[3] = a33;
  }
  return best;
}

__host__ __device__ __forceinline__ bool qcp_rotation(const double* m, double lam, double* rot) {
  const Key4 k = key_matrix(m);
  double q[4];
  const double best = qcp_adj_row(k, lam, q);
  // When the largest eigenvalue of K is double (collinear structures, every
  // 2-atom selection) and lam sits on it to rounding (exact copies: lam is
  // the upper bound (G_a + G_b) / 2 itself), every cofactor of K - lam I is
  // rounding noise and so would be the rotation.  Shifted by
  // eps = 1e-9 * |K|, the adjugate is eps * c * (v1 v1^T + v2 v2^T) + O(eps^2)
  // with v1, v2 spanning the eigenspace, so its rows give an optimal
  // rotation; where the two top eigenvalues differ by g < 1e-12 |K| the
  // shift changes the residual by at most ~2 g / n_atoms.  Other cases keep
  // the unshifted row.
  const double sk = fabs(lam) + fabs(k.k00) + fabs(k.k11) + fabs(k.k22) + fabs(k.k33);
  if (sk > 0.0 && best < 1e-12 * sk * sk * sk) qcp_adj_row(k, lam + 1e-9 * sk, q);
  const double n = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  if (!(n > 0.0) || !(n < 1e300)) {
    rot[0] = rot[4] = rot[8] = 1.0;
    rot[1] = rot[2] = rot[3] = rot[5] = rot[6] = rot[7] = 0.0;
    return false;
  }
  const double inv = 1.0 / sqrt(n);
  const double qw = q[0] * inv, qx = q[1] * inv, qy = q[2] * inv, qz = q[3] * inv;
  const double ww = qw * qw, xx = qx * qx, yy = qy * qy, zz = qz * qz;
  const double xy = qx * qy, wz = qw * qz, zx = qz * qx, wy = qw * qy, yz = qy * qz, wx = qw * qx;
  rot[0] = ww + xx - yy - zz;
  rot[1] = 2.0 * (xy - wz);
  rot[2] = 2.0 * (zx + wy);
  rot[3] = 2.0 * (xy + wz);
  rot[4] = ww - xx + yy - zz;
  rot[5] = 2.0 * (yz - wx);
  rot[6] = 2.0 * (zx - wy);
  rot[7] = 2.0 * (yz + wx);
  rot[8] = ww - xx - yy + zz;
  return true;
}

// FP32 core of the refinement rotation: B = K - lam I with its diagonal
// (b00..b33, already rounded past the subtraction of lam) and M in float.
// Returns false, leaving rot untouched, where the adjugate is FP32 rounding
// noise (top eigenvalue (nearly) double) and the FP64 rotation is needed.
__host__ __device__ __forceinline__ bool qcp_rotation_refine_f32(float b00, float b11, float b22, float b33,
                                                                 const float (&mf)[9], float* rot) {
  const float b01 = mf[5] - mf[7], b02 = mf[6] - mf[2], b03 = mf[1] - mf[3];
  const float b12 = mf[1] + mf[3], b13 = mf[6] + mf[2], b23 = mf[5] + mf[7];
  const float u0 = b00 * b11 - b01 * b01, u1 = b00 * b12 - b01 * b02, u2 = b00 * b13 - b01 * b03;
  const float u3 = b01 * b12 - b11 * b02, u4 = b01 * b13 - b11 * b03, u5 = b02 * b13 - b12 * b03;
  const float w5 = b22 * b33 - b23 * b23, w4 = b12 * b33 - b13 * b23, w3 = b12 * b23 - b13 * b22;
  const float w2 = b02 * b33 - b03 * b23, w1 = b02 * b23 - b03 * b22, w0 = b02 * b13 - b03 * b12;
  const float a00 = b11 * w5 - b12 * w4 + b13 * w3;
  const float a11 = b00 * w5 - b02 * w2 + b03 * w1;
  const float a22 = b03 * u4 - b13 * u2 + b33 * u0;
  const float a33 = b02 * u3 - b12 * u1 + b22 * u0;
  float q[4];
  float best = fabsf(a00);
  q[0] = a00;
  q[1] = -b01 * w5 + b02 * w4 - b03 * w3;
  q[2] = b13 * u5 - b23 * u4 + b33 * u3;
  q[3] = -b12 * u5 + b22 * u4 - b23 * u3;
  if (fabsf(a11) > best) {
    best = fabsf(a11);
    q[0] = -b01 * w5 + b12 * w2 - b13 * w1;
    q[1] = a11;
    q[2] = -b03 * u5 + b23 * u2 - b33 * u1;
    q[3] = b02 * u5 - b22 * u2 + b23 * u1;
  }
  if (fabsf(a22) > best) {
    best = fabsf(a22);
    q[0] = b01 * w4 - b11 * w2 + b13 * w0;
    q[1] = -b00 * w4 + b01 * w2 - b03 * w0;
    q[2] = a22;
    q[3] = -b02 * u4 + b12 * u2 - b23 * u0;
  }
  if (fabsf(a33) > best) {
    best = fabsf(a33);
    q[0] = -b01 * w3 + b11 * w1 - b12 * w0;
    q[1] = b00 * w3 - b01 * w1 + b02 * w0;
    q[2] = -b03 * u3 + b13 * u1 - b23 * u0;
    q[3] = a33;
  }
  // adj(B) = c v v^T with c the product of the other three eigenvalues of B:
  // far above FP32 noise (~1e-6 sk^3) unless the top eigenvalue is (nearly)
  // double
  const float sk = fabsf(b00) + fabsf(b11) + fabsf(b22) + fabsf(b33);
  const float n = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  if (!(best > 1e-4f * sk * sk * sk) || !(n > 1e-30f) || !(n < 1e30f)) return false;
  const float inv = 1.0f / sqrtf(n);
  const float qw = q[0] * inv, qx = q[1] * inv, qy = q[2] * inv, qz = q[3] * inv;
  const float ww = qw * qw, xx = qx * qx, yy = qy * qy, zz = qz * qz;
  const float xy = qx * qy, wz = qw * qz, zx = qz * qx, wy = qw * qy, yz = qy * qz, wx = qw * qx;
  rot[0] = ww + xx - yy - zz;
  rot[1] = 2.0f * (xy - wz);
  rot[2] = 2.0f * (zx + wy);
  rot[3] = 2.0f * (xy + wz);
  rot[4] = ww - xx + yy - zz;
  rot[5] = 2.0f * (yz - wx);
  rot[6] = 2.0f * (zx - wy);
  rot[7] = 2.0f * (yz + wx);
  rot[8] = ww - xx - yy + zz;
  return true;
}

// Rotation for the refinement pass (near-identical frames), in FP32 past the
// subtraction of lam: the refined residual sum |R (a - mu) - b|^2 is at its
// minimum over rotations, so an error e in R changes it by O(e^2), and a
// float adjugate (e ~ 1e-7 where the top eigenvalue is simple) suffices.
// Where it is (nearly) double, the adjugate is rounding noise in FP32 and
// the FP64 qcp_rotation (with its shift) is used instead.  ~25 FP64
// operations against ~200 (the FP64 rotation's sqrt and division alone are
// software sequences of FP64 operations).
__host__ __device__ __forceinline__ void qcp_rotation_refine(const double* m, double lam, float* rot) {
  const float b00 = (float)((m[0] + m[4] + m[8]) - lam), b11 = (float)((m[0] - m[4] - m[8]) - lam);
  const float b22 = (float)((m[4] - m[0] - m[8]) - lam), b33 = (float)((m[8] - m[0] - m[4]) - lam);
  float mf[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) mf[i] = (float)m[i];
  if (qcp_rotation_refine_f32(b00, b11, b22, b33, mf, rot)) return;
  double r64[9];
  qcp_rotation(m, lam, r64);
#pragma unroll
  for (int i = 0; i < 9; ++i) rot[i] = (float)r64[i];
}

// The same from float-pair M and lam (the in-kernel finish): the diagonal of
// B in float pairs, no FP64 instruction unless the FP64 fallback is needed
// (GB300 issues an FP64 instruction per ~64 cycles of a sub-partition, and
// the ~25 of qcp_rotation_refine held a refined frame's lane ~2 us).
__host__ __device__ __forceinline__ void qcp_rotation_refine_dfm(const DF (&m)[9], DF lam, float* rot) {
  const DF k00 = df_add(df_add(m[0], m[4]), m[8]), k11 = df_sub(df_sub(m[0], m[4]), m[8]);
  const DF k22 = df_sub(df_sub(m[4], m[0]), m[8]), k33 = df_sub(df_sub(m[8], m[0]), m[4]);
  const DF d0 = df_sub(k00, lam), d1 = df_sub(k11, lam), d2 = df_sub(k22, lam), d3 = df_sub(k33, lam);
  float mf[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) mf[i] = GB_FADD(m[i].hi, m[i].lo);
  if (qcp_rotation_refine_f32(GB_FADD(d0.hi, d0.lo), GB_FADD(d1.hi, d1.lo), GB_FADD(d2.hi, d2.lo),
                              GB_FADD(d3.hi, d3.lo), mf, rot))
    return;
  double md[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) md[i] = df_to_double(m[i]);
  double r64[9];
  qcp_rotation(md, df_to_double(lam), r64);
#pragma unroll
  for (int i = 0; i < 9; ++i) rot[i] = (float)r64[i];
}

}  // namespace gb
