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

// PW92 G_k(rs) and dG_k/drs for parameter column k of src/lda_c_pw.c:41-50
// (k = 0: eps_c(rs, 0); 1: eps_c(rs, 1); 2: -alpha_c(rs)).
__device__ __forceinline__ void pw92_g(int k, double rs, double srs, double &g, double &dg) {
  const double A[3] = {0.031091, 0.015545, 0.016887}, AL[3] = {0.21370, 0.20548, 0.11125},
               B1[3] = {7.5957, 14.1189, 10.357}, B2[3] = {3.5876, 6.1977, 3.6231},
               B3[3] = {1.6382, 3.3662, 0.88026}, B4[3] = {0.49294, 0.62517, 0.49671};
  const double a = A[k], al = AL[k];
  const double q0 = -2.0 * a * (1.0 + al * rs);
  const double q1 = 2.0 * a * (B1[k] * srs + B2[k] * rs + B3[k] * rs * srs + B4[k] * rs * rs);
  const double dq1 = a * (B1[k] / srs + 2.0 * B2[k] + 3.0 * B3[k] * srs + 4.0 * B4[k] * rs);
  const double lg = log(1.0 + 1.0 / q1);
  g = q0 * lg;
  dg = -2.0 * a * al * lg - q0 * dq1 / (q1 * q1 + q1);
}

// Spin-polarised LDA (Slater exchange + PW92 with the spin interpolation of
// maple/lda_exc/lda_c_pw.mpl:42-44): energy per particle exc and the
// potentials va = d(n exc)/dn_up, vb = d(n exc)/dn_down.  libxc 6.2.2's
// screening: each spin density raised to 1e-15, zeros when na + nb < 1e-15
// (src/work_lda_inc.c:48-55), 1 +/- zeta kept >= DBL_EPSILON
// (maple/util.mpl:77-82), an exchange channel with n_s <= 1e-15 dropped
// (maple/util.mpl:101-110).  1 +/- zeta are formed as 2 n_s / n, which keeps
// full digits next to full polarisation.
__device__ __forceinline__ void lsda_point(double rho_a, double rho_b, double &exc, double &va,
                                           double &vb) {
  const double thr = 1e-15, zt = 2.220446049250313e-16;
  exc = va = vb = 0.0;
  if (!(rho_a + rho_b >= thr)) return;
  const double na = fmax(rho_a, thr), nb = fmax(rho_b, thr);
  const double n = na + nb;
  double opz = 2.0 * na / n, omz = 2.0 * nb / n;
  if (opz <= zt) {
    opz = zt;
    omz = 2.0 - zt;
  } else if (omz <= zt) {
    omz = zt;
    opz = 2.0 - zt;
  }
  const double z = opz - 1.0;
  const double pi = 3.141592653589793238462643383279502884;
  const double cx = -0.75 * cbrt(3.0 / pi);
  const double n13 = cbrt(n);
  const double c43a = cbrt(opz) * opz, c43b = cbrt(omz) * omz;   // (1 +/- z)^{4/3}
  double ex = 0.0;
  if (na > thr) {
    ex += 0.5 * cx * n13 * c43a;
    va = -cbrt(6.0 * na / pi);
  }
  if (nb > thr) {
    ex += 0.5 * cx * n13 * c43b;
    vb = -cbrt(6.0 * nb / pi);
  }
  const double rs = cbrt(3.0 / (4.0 * pi * n));
  const double srs = sqrt(rs);
  double g1, d1, g2, d2, g3, d3;
  pw92_g(0, rs, srs, g1, d1);
  pw92_g(1, rs, srs, g2, d2);
  pw92_g(2, rs, srs, g3, d3);
  const double fz20 = 1.709921;
  const double den = 0.5198420997897464;   // 2^{4/3} - 2
  const double fz = (c43a + c43b - 2.0) / den;
  const double dfz = (4.0 / 3.0) * (cbrt(opz) - cbrt(omz)) / den;
  const double z3 = z * z * z, z4 = z3 * z;
  const double stiff = g2 - g1 + g3 / fz20;
  const double ec = g1 + z4 * fz * stiff - fz * g3 / fz20;
  const double de_rs = d1 + z4 * fz * (d2 - d1 + d3 / fz20) - fz * d3 / fz20;
  const double de_z = (4.0 * z3 * fz + z4 * dfz) * stiff - dfz * g3 / fz20;
  const double base = ec - rs / 3.0 * de_rs;
  exc = ex + ec;
  va += base + omz * de_z;
  vb += base - opz * de_z;
}

}  // namespace derek
