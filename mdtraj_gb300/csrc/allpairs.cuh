// All-pairs RMSD matrix: shared declarations.
//
// Work = the reference's clustering loop `for i: D[i] = md.rmsd(traj, traj,
// i, precentered=True)` (mdtraj examples/clustering.ipynb, cell 6) done as
// one symmetric matrix: frames are centred once (Trajectory.center_coordinates,
// mdtraj/core/trajectory.py:2114-2137), stacked as X (3F x A) with row 3i+c =
// axis c of frame i, and P = X X^T; the 3x3 block (i, j) of P is the inner
// product matrix M_ij of msd_atom_major (mdtraj/rmsd/src/theobald_rmsd_generic.h:63-119),
// fed to QCP per pair.
#pragma once

#include <stdint.h>

#include "../../include/gbrmsd.h"
#include "common.cuh"

namespace gb {

// Refinement record for a pair whose msd is too small for the per-pair FP32
// QCP to resolve.
struct PairRefine {
  int32_t i, j;
};

struct AllPairsDims {
  int64_t n_frames;
  int32_t n_atoms;
  int32_t k_pad;   // atoms padded to a multiple of 64 (BF16 K blocks)
  int64_t rows;    // 3 * n_frames
};

// Result slot of a pair that needs refinement but found the refinement list
// full: a quiet NaN, which the refinement kernel finds by scanning the output
// (a non-finite input gives NaN as well; refining it again gives NaN again).
__device__ __forceinline__ float refine_marker() { return __int_as_float(0x7fc00000); }

// Explicitly rounded FP32 operations for the pair epilogue.  The epilogue is
// inlined at several points of the tile kernels (inside the fold loop, after
// it, at the end of a CTA's tiles), and with implicit contraction the
// compiler is free to fuse a product into an FMA at one point and not at
// another; a pair would then round differently depending on where in its
// CTA's tile sequence it was finished, and a query served in a mixed batch
// could differ in the last bit from the same query served alone.  The _rn
// intrinsics are never contracted, so every copy computes the same bits.
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rn_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// a b - c d
__device__ __forceinline__ float rn_det2(float a, float b, float c, float d) { return rn_fma(a, b, rn_mul(-c, d)); }
// a0 b0 + a1 b1 + a2 b2 (+ a3 b3)
__device__ __forceinline__ float rn_dot3(float a0, float b0, float a1, float b1, float a2, float b2) {
  return rn_fma(a2, b2, rn_fma(a1, b1, rn_mul(a0, b0)));
}
__device__ __forceinline__ float rn_dot4(float a0, float b0, float a1, float b1, float a2, float b2, float a3,
                                         float b3) {
  return rn_fma(a3, b3, rn_fma(a2, b2, rn_fma(a1, b1, rn_mul(a0, b0))));
}

// FP32 QCP on the quartic normalised by lam0 = (Ga + Gb) / 2 (root near 1).
// Returns msd = 2 lam0 (1 - x) / n, x = normalised lambda_max.
//
// `unresolved` is set when the FP32 result cannot be trusted to 2e-5 nm.
// That happens at (nearly) double roots: when one of the two structures is
// (nearly) collinear, as every 2-atom selection is, M has rank ~1 and K's
// top eigenvalue is doubled, and in FP32 the quartic fixes such a root only
// to ~sqrt(eps): Newton steps become rounding noise over rounding noise and
// x can land anywhere, and the adjugate behind the Rayleigh polish is noise
// too (an FP32 emulation of this routine gave errors up to 0.5 nm on 2-atom
// pairs and NaN on exact collinear copies).  Two tests, both a posteriori:
//   * Newton did not converge (30 steps, last step above 1e-5, or NaN);
//   * the polish's own error estimate is too large for the pair's rmsd: the
//     polish removes an error ~dx from x and leaves ~dx^2 / gap, gap ~
//     P'(x) / (P''(x) / 2), so rmsd error ~ lam0 dx^2 |P''/2| / (n |P'| r).
//   * M has rank ~1 and the pair's rmsd is small against the structures'
//     size (below).
// The caller sends such pairs to the exact FP64 refinement, whose QCP
// handles double roots.  In the same emulation (3,000 sampled pairs each of
// 2,000-atom metastable, 300-atom chain and 100-atom cube frames; 1,500 each
// of 3- to 2,000-atom collinear and nearly collinear frames with 0.01-0.2 nm
// noise) the three tests together flagged every pair off by more than
// 2e-5 nm and none of the generic pairs.
__device__ __forceinline__ float qcp_msd_f32(const float (&m)[9], float ga, float gb, float inv_n,
                                             bool& unresolved) {
  unresolved = false;
  const float lam0 = rn_mul(0.5f, rn_add(ga, gb));
  if (!(lam0 > 0.f)) return 0.f;
  const float inv = __fdiv_rn(1.0f, lam0);
  float mm[9];
#pragma unroll
  for (int t = 0; t < 9; ++t) mm[t] = rn_mul(m[t], inv);
  const float k00 = rn_add(rn_add(mm[0], mm[4]), mm[8]), k01 = rn_sub(mm[5], mm[7]);
  const float k02 = rn_sub(mm[6], mm[2]), k03 = rn_sub(mm[1], mm[3]);
  const float k11 = rn_sub(rn_sub(mm[0], mm[4]), mm[8]), k12 = rn_add(mm[1], mm[3]), k13 = rn_add(mm[6], mm[2]);
  const float k22 = rn_sub(rn_sub(mm[4], mm[0]), mm[8]), k23 = rn_add(mm[5], mm[7]);
  const float k33 = rn_sub(rn_sub(mm[8], mm[0]), mm[4]);
  float c2 = 0.f;
#pragma unroll
  for (int t = 0; t < 9; ++t) c2 = rn_fma(mm[t], mm[t], c2);
  c2 = rn_mul(c2, -2.f);
  const float cf00 = rn_det2(mm[4], mm[8], mm[5], mm[7]), cf01 = rn_det2(mm[3], mm[8], mm[5], mm[6]);
  const float cf02 = rn_det2(mm[3], mm[7], mm[4], mm[6]);
  const float detm = rn_dot3(mm[0], cf00, -mm[1], cf01, mm[2], cf02);
  // |cof M|_F^2 = s1^2 s2^2 + s1^2 s3^2 + s2^2 s3^2 (singular values of M):
  // near 0 when M has rank ~1, i.e. when a structure is (nearly) collinear
  float cof2 = rn_fma(cf02, cf02, rn_fma(cf01, cf01, rn_mul(cf00, cf00)));
  {
    const float c10 = rn_det2(mm[1], mm[8], mm[2], mm[7]), c11 = rn_det2(mm[0], mm[8], mm[2], mm[6]);
    const float c12 = rn_det2(mm[0], mm[7], mm[1], mm[6]), c20 = rn_det2(mm[1], mm[5], mm[2], mm[4]);
    const float c21 = rn_det2(mm[0], mm[5], mm[2], mm[3]), c22 = rn_det2(mm[0], mm[4], mm[1], mm[3]);
    cof2 = rn_fma(c10, c10, cof2);
    cof2 = rn_fma(c11, c11, cof2);
    cof2 = rn_fma(c12, c12, cof2);
    cof2 = rn_fma(c20, c20, cof2);
    cof2 = rn_fma(c21, c21, cof2);
    cof2 = rn_fma(c22, c22, cof2);
  }
  const float c1 = rn_mul(-8.f, detm);
  const float s01 = rn_det2(k00, k11, k01, k01), s02 = rn_det2(k00, k12, k02, k01), s03 = rn_det2(k00, k13, k03, k01);
  const float s12 = rn_det2(k01, k12, k02, k11), s13 = rn_det2(k01, k13, k03, k11), s23 = rn_det2(k02, k13, k03, k12);
  const float q01 = rn_det2(k02, k13, k12, k03), q02 = rn_det2(k02, k23, k22, k03), q03 = rn_det2(k02, k33, k23, k03);
  const float q12 = rn_det2(k12, k23, k22, k13), q13 = rn_det2(k12, k33, k23, k13), q23 = rn_det2(k22, k33, k23, k23);
  float c0 = rn_mul(s01, q23);
  c0 = rn_fma(-s02, q13, c0);
  c0 = rn_fma(s03, q12, c0);
  c0 = rn_fma(s12, q03, c0);
  c0 = rn_fma(-s13, q02, c0);
  c0 = rn_fma(s23, q01, c0);
  // Newton from above converges monotonically to the largest root; start at
  // the smaller of the two upper bounds 1 = (Ga + Gb) / 2 / lam0 and
  // sqrt(3/4 tr K^2) = sqrt(3) |M|_F = sqrt(-1.5 c2) (K is traceless, so
  // lambda_max <= sqrt((n-1)/n tr K^2) for n = 4), nudged up by 2^-20 against
  // rounding.  Far-apart structures start much closer: 17.9 -> 6.2
  // iterations on the all-pairs workload in an FP32 emulation, same errors.
  float x = fminf(1.0f, rn_mul(sqrtf(rn_mul(-1.5f, c2)), 1.00000095f));
  // Then one Laguerre step, x -= 4P / (P' + sqrt(3 (3P'^2 - 4 P P''))): for a
  // polynomial with real roots (K is symmetric) it goes from above to the
  // largest root without passing it, and cubically near it, where Newton
  // starts with steps of ~x/4.  Should rounding carry it past the root
  // (P < 0 there), Newton starts from the bound instead.  With Newton's stop
  // at 1e-6 (the polish below takes x the rest of the way), the slowest lane
  // of a warp needs 6.7 Newton steps instead of 12.0 on 300-atom chains and
  // 2.1 instead of 4.2 on the all-pairs workload (FP32 emulation; the same
  // pairs flagged, the largest error of the others unchanged on both and
  // within 1.2e-5 nm on nearly collinear 40-atom frames).
  {
    const float x2 = rn_mul(x, x);
    const float b = rn_mul(rn_add(x2, c2), x);
    const float a = rn_add(b, c1);
    const float pv = rn_fma(a, x, c0);
    const float dp = rn_add(rn_fma(rn_mul(2.0f, x2), x, b), a);
    const float d2 = rn_fma(rn_mul(12.0f, x), x, rn_mul(2.0f, c2));
    const float g = fmaxf(rn_mul(3.0f, rn_fma(rn_mul(3.0f, dp), dp, rn_mul(rn_mul(-4.0f, pv), d2))), 0.0f);
    float sg;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(sg) : "f"(g));
    const float den = rn_add(dp, sg);
    if (den > 0.0f) {
      const float x1 = rn_sub(x, __fdividef(rn_mul(4.0f, pv), den));
      const float p1 = rn_fma(rn_add(rn_mul(rn_add(rn_mul(x1, x1), c2), x1), c1), x1, c0);
      if (p1 >= 0.0f) x = x1;  // false for NaN
    }
  }
  float last = 0.f;      // last Newton step
  bool converged = false;
#pragma unroll 1
  for (int it = 0; it < 30; ++it) {
    const float x2 = rn_mul(x, x);
    const float b = rn_mul(rn_add(x2, c2), x);
    const float a = rn_add(b, c1);
    const float pv = rn_fma(a, x, c0);
    const float dp = rn_add(rn_fma(rn_mul(2.0f, x2), x, b), a);
    if (!(dp != 0.0f)) break;
    const float step = __fdividef(pv, dp);
    x = rn_sub(x, step);
    last = step;
    if (fabsf(step) <= 1e-6f) {  // false for NaN: a NaN step runs to the cap
      converged = true;
      break;
    }
  }
  unresolved = !converged && !(fabsf(last) <= 1e-5f);
  // P'(x) and P''(x) / 2 at Newton's x, for the polish's error estimate
  float slope, curv;
  {
    const float x2 = rn_mul(x, x);
    const float b = rn_mul(rn_add(x2, c2), x);
    const float a = rn_add(b, c1);
    slope = fabsf(rn_add(rn_fma(rn_mul(2.0f, x2), x, b), a));
    curv = fabsf(rn_fma(6.0f, x2, c2));
  }
  float dx = 0.f;
  // The quartic's largest root is ill-conditioned when the top eigenvalues of
  // K are close (far-apart structures): FP32 Newton stalls ~1e-6 away from it.
  // The eigenvalue itself is well-conditioned, so polish x with the Rayleigh
  // quotient of v = the row of adj(K - x I) with the largest diagonal
  // cofactor (parallel to the top eigenvector; the quotient's error is
  // quadratic in v's): x += v^T (K - x I) v / v^T v.  The adjugate comes from
  // the 2x2 complementary minors of rows {0,1} and {2,3} (Laplace expansion).
  {
    const float b00 = rn_sub(k00, x), b11 = rn_sub(k11, x), b22 = rn_sub(k22, x), b33 = rn_sub(k33, x);
    const float b01 = k01, b02 = k02, b03 = k03, b12 = k12, b13 = k13, b23 = k23;
    const float u0 = rn_det2(b00, b11, b01, b01), u1 = rn_det2(b00, b12, b01, b02), u2 = rn_det2(b00, b13, b01, b03);
    const float u3 = rn_det2(b01, b12, b11, b02), u4 = rn_det2(b01, b13, b11, b03), u5 = rn_det2(b02, b13, b12, b03);
    const float w5 = rn_det2(b22, b33, b23, b23), w4 = rn_det2(b12, b33, b13, b23), w3 = rn_det2(b12, b23, b13, b22);
    const float w2 = rn_det2(b02, b33, b03, b23), w1 = rn_det2(b02, b23, b03, b22), w0 = rn_det2(b02, b13, b03, b12);
    const float a00 = rn_dot3(b11, w5, -b12, w4, b13, w3);
    const float a11 = rn_dot3(b00, w5, -b02, w2, b03, w1);
    const float a22 = rn_dot3(b03, u4, -b13, u2, b33, u0);
    const float a33 = rn_dot3(b02, u3, -b12, u1, b22, u0);
    float v0, v1, v2, v3, best = fabsf(a00);
    v0 = a00;
    v1 = rn_dot3(-b01, w5, b02, w4, -b03, w3);
    v2 = rn_dot3(b13, u5, -b23, u4, b33, u3);
    v3 = rn_dot3(-b12, u5, b22, u4, -b23, u3);
    if (fabsf(a11) > best) {
      best = fabsf(a11);
      v0 = rn_dot3(-b01, w5, b12, w2, -b13, w1);
      v1 = a11;
      v2 = rn_dot3(-b03, u5, b23, u2, -b33, u1);
      v3 = rn_dot3(b02, u5, -b22, u2, b23, u1);
    }
    if (fabsf(a22) > best) {
      best = fabsf(a22);
      v0 = rn_dot3(b01, w4, -b11, w2, b13, w0);
      v1 = rn_dot3(-b00, w4, b01, w2, -b03, w0);
      v2 = a22;
      v3 = rn_dot3(-b02, u4, b12, u2, -b23, u0);
    }
    if (fabsf(a33) > best) {
      v0 = rn_dot3(-b01, w3, b11, w1, -b12, w0);
      v1 = rn_dot3(b00, w3, -b01, w1, b02, w0);
      v2 = rn_dot3(-b03, u3, b13, u1, -b23, u0);
      v3 = a33;
    }
    const float bv0 = rn_dot4(b00, v0, b01, v1, b02, v2, b03, v3);
    const float bv1 = rn_dot4(b01, v0, b11, v1, b12, v2, b13, v3);
    const float bv2 = rn_dot4(b02, v0, b12, v1, b22, v2, b23, v3);
    const float bv3 = rn_dot4(b03, v0, b13, v1, b23, v2, b33, v3);
    const float vv = rn_dot4(v0, v0, v1, v1, v2, v2, v3, v3);
    dx = __fdiv_rn(rn_dot4(v0, bv0, v1, bv1, v2, bv2, v3, bv3), vv);
    if (vv > 1e-30f && fabsf(dx) < 1e-3f) x = rn_add(x, dx);
  }
  float msd = rn_mul(rn_mul(rn_mul(2.0f, lam0), rn_sub(1.0f, x)), inv_n);
  msd = msd > 0.f ? msd : 0.f;
  // rmsd error estimate lam0 dx^2 curv / (n slope r) <= 2e-5 nm, without a
  // division (false for NaN or an infinite dx: such pairs are refined too)
  const float lhs = rn_mul(rn_mul(rn_mul(lam0, inv_n), rn_mul(dx, dx)), curv);
  const float rhs = rn_mul(rn_mul(2e-5f, sqrtf(msd)), slope);
  if (!(lhs <= rhs)) unresolved = true;
  // M of rank ~1 (q = |cof M|^2 / |M|_F^4 small) with an rmsd small against
  // the structures' size: q (r / scale)^2 < 2e-7, scale = lam0 / n.  The
  // emulation needed 1e-7 to catch every pair off by more than 2e-5 nm, and
  // the first generic pair (300-atom chains) came at 1e-6.
  const float i1 = rn_mul(-0.5f, c2);  // |M|_F^2 of the normalised M
  const float sc = rn_mul(lam0, inv_n);
  if (!(rn_mul(cof2, msd) >= rn_mul(rn_mul(2e-7f, rn_mul(i1, i1)), rn_mul(sc, sc)))) unresolved = true;
  return msd;
}

// Refinement threshold of a pair: r < 0.75 * scale * sqrt(1/n), scale =
// (Ga + Gb) / 2n (explicitly rounded for the same reason as the QCP above).
// The msd error of the split-BF16 M grows like scale / sqrt(n): summing the
// three BF16 products exactly it stays below 3.4e-5 * scale / sqrt(n) (all
// 44,850 pairs each of 300 noisy rotated copies of 257 and of 1,000 atoms,
// 0.001-0.4 nm noise), and the tensor core's FP32 accumulation doubles it.
// The rmsd error is the msd error over 2 r, so above the threshold it stays
// below ~4.5e-5 nm (measured 1.2-1.4e-4 nm at the former 0.25).
__device__ __forceinline__ bool pair_needs_refine(float r, float ga, float gb, float inv_n) {
  const float scale = rn_mul(rn_mul(0.5f, rn_add(ga, gb)), inv_n);
  return r < rn_mul(rn_mul(0.75f, scale), sqrtf(inv_n));
}

// Writes the pair's rmsd to both triangles (i < j) or 0 on the diagonal and
// queues pairs the FP32 QCP cannot resolve, or that lie below the refinement
// threshold, for exact refinement.  When the list is full the pair's two
// slots get refine_marker() instead, and the refinement kernel scans for it.
// (ga, gb: the two frames' traces rounded to float.)
__device__ __forceinline__ void pair_epilogue_g(int64_t i, int64_t j, const float (&m)[9], float ga, float gb,
                                                float inv_n, int64_t F, float* __restrict__ out, PairRefine* rl,
                                                int* rc, int rcap, int* err) {
  if (i == j) {
    out[i * F + i] = 0.f;
    return;
  }
  bool unresolved;
  const float msd = qcp_msd_f32(m, ga, gb, inv_n, unresolved);
  float r = sqrtf(msd);
  if (unresolved || pair_needs_refine(r, ga, gb, inv_n)) {
    // the count is read first so that it stops growing once the list is
    // full (it exceeds rcap by at most the pairs in flight)
    const int slot = *reinterpret_cast<volatile int*>(rc) < rcap ? atomicAdd(rc, 1) : rcap;
    if (slot < rcap)
      rl[slot] = PairRefine{(int32_t)i, (int32_t)j};
    else
      r = refine_marker();
  }
  out[i * F + j] = r;
  out[j * F + i] = r;
}

__device__ __forceinline__ void pair_epilogue(int64_t i, int64_t j, const float (&m)[9], const double* __restrict__ G,
                                              float inv_n, int64_t F, float* __restrict__ out, PairRefine* rl,
                                              int* rc, int rcap, int* err) {
  pair_epilogue_g(i, j, m, (float)G[i], (float)G[j], inv_n, F, out, rl, rc, rcap, err);
}

// Cross RMSD (query set against a database): the output row and database
// range of one query-set column, or row == nullptr when the column belongs to
// no request of the call.
struct CrossCol {
  float* row;  // out_r + q * (db1 - db0)
  int64_t db0, db1;
};

__device__ __forceinline__ CrossCol cross_col(const gbrmsd_cross_request_t* __restrict__ reqs,
                                              const int32_t* __restrict__ colreq, int64_t j, int64_t n_cols) {
  CrossCol c;
  c.row = nullptr;
  c.db0 = 0;
  c.db1 = 0;
  if (j < n_cols) {
    const int32_t r = colreq[j];
    if (r >= 0) {
      const gbrmsd_cross_request_t q = reqs[r];
      c.row = q.out + (j - q.pool0) * (q.db1 - q.db0);
      c.db0 = q.db0;
      c.db1 = q.db1;
    }
  }
  return c;
}

// Cross pair (database frame i, query row j): FP32 QCP, result to *dst, and
// the same refinement rule as pair_epilogue.
__device__ __forceinline__ void cross_pair(int64_t i, int64_t j, const float (&m)[9], float ga, float gb,
                                           float inv_n, float* dst, PairRefine* rl, int* rc, int rcap, int* err) {
  bool unresolved;
  const float msd = qcp_msd_f32(m, ga, gb, inv_n, unresolved);
  float r = sqrtf(msd);
  if (unresolved || pair_needs_refine(r, ga, gb, inv_n)) {
    // the count is read first so that it stops growing once the list is
    // full (it exceeds rcap by at most the pairs in flight)
    const int slot = *reinterpret_cast<volatile int*>(rc) < rcap ? atomicAdd(rc, 1) : rcap;
    if (slot < rcap)
      rl[slot] = PairRefine{(int32_t)i, (int32_t)j};
    else
      r = refine_marker();
  }
  *dst = r;
}

}  // namespace gb
