// Pointwise LDA exchange-correlation shared by the grid kernels.
#pragma once

namespace derek {

// Spin-unpolarised LDA: Slater exchange + Perdew-Wang 92 correlation, written
// from libxc 6.2.2's maple sources (maple/util.mpl:58-94 for the exchange
// prefactor, maple/lda_exc/lda_c_pw.mpl:34-37 for G(rs), parameters of
// src/lda_c_pw.c:41-50, first column).  Densities below 1e-15 give zero
// (src/work_lda_inc.c:50); exchange is screened when n/2 <= 1e-15.
__device__ __forceinline__ void lda_point(double rho, double &exc, double &vxc) {
  const double thr = 1e-15;
  if (!(rho >= thr)) {
    exc = 0.0;
    vxc = 0.0;
    return;
  }
  const double n = rho;
  const double pi = 3.141592653589793238462643383279502884;
  double ex = -0.75 * cbrt(3.0 / pi) * cbrt(n);
  if (!(0.5 * n > thr)) ex = 0.0;
  const double vx = 4.0 / 3.0 * ex;
  const double rs = cbrt(3.0 / (4.0 * pi * n));
  const double a = 0.031091, alpha1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382,
               b4 = 0.49294;
  const double srs = sqrt(rs);
  const double q0 = -2.0 * a * (1.0 + alpha1 * rs);
  const double q1 = 2.0 * a * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  const double dq1 = a * (b1 / srs + 2.0 * b2 + 3.0 * b3 * srs + 4.0 * b4 * rs);
  const double lg = log(1.0 + 1.0 / q1);
  const double ec = q0 * lg;
  const double dec = -2.0 * a * alpha1 * lg - q0 * dq1 / (q1 * q1 + q1);
  const double vc = ec - rs / 3.0 * dec;
  exc = ex + ec;
  vxc = vx + vc;
}

}  // namespace derek
