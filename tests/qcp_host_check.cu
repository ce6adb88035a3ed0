// Host build of the QCP solve shared by every kernel's finish
// (mdtraj_gb300/csrc/qcp.cuh is __host__ __device__), for tests/test_qcp_host.py.
//
// Reads cases from stdin: "A" then A lines "ax ay az bx by bz" (float32
// coordinates of the moving frame a and the reference frame b).  For each
// case prints: lambda (mixed FP32/FP64 solve), lambda (FP64 solve), the
// upper bound (Ga + Gb) / 2, the QCP msd, whether the finish would refine
// the frame, the direct residual rmsd with the QCP rotation, lambda from
// the float-float solve (the one the finish kernels use), the direct
// residual rmsd with the refinement pass's FP32 rotation, and the same with
// the in-kernel finish's rotation from float-pair M and lambda
// (qcp_rotation_refine_dfm).
#include <cmath>
#include <cstdio>

#include "../mdtraj_gb300/csrc/qcp.cuh"

using namespace gb;

int main() {
  int A = 0;
  static float a[1 << 16][3], b[1 << 16][3];
  while (std::scanf("%d", &A) == 1) {
    if (A <= 0 || A > (1 << 16)) return 2;
    for (int k = 0; k < A; ++k)
      if (std::scanf("%f %f %f %f %f %f", &a[k][0], &a[k][1], &a[k][2], &b[k][0], &b[k][1], &b[k][2]) != 6) return 3;
    double ma[3] = {0, 0, 0}, mb[3] = {0, 0, 0};
    for (int k = 0; k < A; ++k)
      for (int c = 0; c < 3; ++c) {
        ma[c] += a[k][c];
        mb[c] += b[k][c];
      }
    for (int c = 0; c < 3; ++c) {
      ma[c] /= A;
      mb[c] /= A;
    }
    double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, ga = 0, gb = 0;
    for (int k = 0; k < A; ++k) {
      double x[3], y[3];
      for (int c = 0; c < 3; ++c) {
        x[c] = a[k][c] - ma[c];
        y[c] = b[k][c] - mb[c];
        ga += x[c] * x[c];
        gb += y[c] * y[c];
      }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m[3 * i + j] += x[i] * y[j];
    }
    int it1 = 0, it2 = 0;
    const double lam = qcp_lambda_max_mixed(m, ga, gb, &it1);
    const double lam64 = qcp_lambda_max(m, ga, gb, &it2);
    int it3 = 0;
    bool short_ = false;
    double lamdf = qcp_lambda_max_df(m, ga, gb, &it3, &short_);
    if (short_) lamdf = qcp_newton_fp64(m, lamdf);
    double msd = (ga + gb - 2.0 * lamdf) / A;
    if (!(msd > 0.0)) msd = 0.0;
    const double scale = (ga + gb) * 0.5 / A;
    const int refine = msd * A < 0.01 * scale * scale;
    double rot[9];
    qcp_rotation(m, lamdf, rot);
    double s = 0.0;
    for (int k = 0; k < A; ++k) {
      double x[3], y[3];
      for (int c = 0; c < 3; ++c) {
        x[c] = a[k][c] - ma[c];
        y[c] = b[k][c] - mb[c];
      }
      for (int i = 0; i < 3; ++i) {
        const double r = rot[3 * i] * x[0] + rot[3 * i + 1] * x[1] + rot[3 * i + 2] * x[2] - y[i];
        s += r * r;
      }
    }
    float rf[9];
    qcp_rotation_refine(m, lamdf, rf);
    double s2 = 0.0;
    for (int k = 0; k < A; ++k) {
      double x[3], y[3];
      for (int c = 0; c < 3; ++c) {
        x[c] = a[k][c] - ma[c];
        y[c] = b[k][c] - mb[c];
      }
      for (int i = 0; i < 3; ++i) {
        const double r = rf[3 * i] * x[0] + rf[3 * i + 1] * x[1] + rf[3 * i + 2] * x[2] - y[i];
        s2 += r * r;
      }
    }
    // the in-kernel finish's refinement rotation, from float-pair M and lambda
    DF mdf[9];
    for (int i = 0; i < 9; ++i) mdf[i] = df_from_double(m[i]);
    int it4 = 0;
    bool sh4 = false;
    DF lam_pair = qcp_lambda_max_dfm(mdf, df_mul_f(df_add(df_from_double(ga), df_from_double(gb)), 0.5f), &it4, &sh4);
    if (sh4) lam_pair = df_from_double(qcp_newton_fp64(m, df_to_double(lam_pair)));
    float rp[9];
    qcp_rotation_refine_dfm(mdf, lam_pair, rp);
    double s3 = 0.0;
    for (int k = 0; k < A; ++k) {
      double x[3], y[3];
      for (int c = 0; c < 3; ++c) {
        x[c] = a[k][c] - ma[c];
        y[c] = b[k][c] - mb[c];
      }
      for (int i = 0; i < 3; ++i) {
        const double r = rp[3 * i] * x[0] + rp[3 * i + 1] * x[1] + rp[3 * i + 2] * x[2] - y[i];
        s3 += r * r;
      }
    }
    std::printf("%.17g %.17g %.17g %.17g %d %.17g %.17g %.17g %.17g\n", lam, lam64, 0.5 * (ga + gb), msd, refine,
                std::sqrt(s / A), lamdf, std::sqrt(s2 / A), std::sqrt(s3 / A));
  }
  return 0;
}
