/* Flat C entry points over the compiled libxc subset: evaluate the Slater
 * exchange (XC_LDA_X, id 1) and Perdew-Wang 92 correlation (XC_LDA_C_PW,
 * id 12) on n densities.  ex/ec are energies per particle (libxc "zk"),
 * vx/vc the potentials d(n eps)/dn_s (libxc "vrho").  The polarised entry
 * takes rho as n (rho_up, rho_down) pairs and returns vx/vc as n pairs.
 * Return 0 on success. */
#include "xc.h"

int ref_lda_unpol(long n, const double *rho, double *ex, double *vx,
                  double *ec, double *vc) {
  xc_func_type fx, fc;
  if (xc_func_init(&fx, XC_LDA_X, XC_UNPOLARIZED) != 0) return 1;
  if (xc_func_init(&fc, XC_LDA_C_PW, XC_UNPOLARIZED) != 0) return 2;
  xc_lda_exc_vxc(&fx, (size_t)n, rho, ex, vx);
  xc_lda_exc_vxc(&fc, (size_t)n, rho, ec, vc);
  xc_func_end(&fx);
  xc_func_end(&fc);
  return 0;
}

int ref_lda_pol(long n, const double *rho, double *ex, double *vx,
                double *ec, double *vc) {
  xc_func_type fx, fc;
  if (xc_func_init(&fx, XC_LDA_X, XC_POLARIZED) != 0) return 1;
  if (xc_func_init(&fc, XC_LDA_C_PW, XC_POLARIZED) != 0) return 2;
  xc_lda_exc_vxc(&fx, (size_t)n, rho, ex, vx);
  xc_lda_exc_vxc(&fc, (size_t)n, rho, ec, vc);
  xc_func_end(&fx);
  xc_func_end(&fc);
  return 0;
}
