// Launchers of the grid-level SCF kernels (scf_kernels.cu).
#pragma once

#include <algorithm>

#include "subspace.cuh"

namespace derek {

// Grids of the non-collinear SCF (all systems spinor), passed by value to the
// grid kernels; on == 0 for scalar batches.  Three-component grids are
// component-major with component stride tg (the batch's total grid points);
// 2x2 potentials hold V11, V21, V12, V22 per point.
struct SpinGrids {
  int on;
  long long tg;
  const double2 *vnc_ext;   // external nc_pot (set_nc_pot / V_ext on the diagonal)
  double *mag_in;           // m_in, mixed
  const double *mag_out;    // m_out of the density pass
  double *bxc;              // xc field b = (v_up - v_down)/2 m_in/|m_in|
  double2 *vnc64;           // the H.psi potential, FP64 and FP32 copies
  float2 *vnc32;
  double *min_hist, *mres_hist;   // mixing history, 3 x (hist slots x nr) per system
};

template <typename R>
// start vectors: hashed random entries, or (pw_entry non-null) band b of item
// i on entry pw_entry[i] plus a small hashed perturbation
void launch_init_psi(const Tables &t, int nitems, void *X, unsigned long long seed, const int *pw_entry,
                     cudaStream_t st);
void launch_filter_coef(const Tables &t, int nks, const double *eig, const SysState *st, Axpby *coef,
                        int m, cudaStream_t s);
// t is the band view: a spinor band holds one electron and its density
// weight goes to both of its items
void launch_occupations(const Tables &t, int nsys, const double *eig, double *occ, double *occw,
                        SysState *st, cudaStream_t s);
void launch_energies(const Tables &t, int nsys, const double *vhxc, const double *rho_in,
                     const double *rho_out, const double2 *cgrid, double *part, SysState *st,
                     SysDev *sys_rw, const int *ks_status, const SpinGrids &sg, cudaStream_t s);
void launch_mix(const Tables &t, int nsys, int max_nr, double *rho_in, const double *rho_out,
                double *nin_hist, double *res_hist, const long long *hist_off, SysState *st, int H,
                double *part, double2 *cgrid, double alpha, double q0, int max_n, const SpinGrids &sg,
                cudaStream_t s);
void launch_potential(const Tables &t, int nsys, int max_nr, int max_n, const double *rho_in,
                      double2 *cgrid, const double *vext, double *vhxc, double *vloc, float *vloc32,
                      double *part, SysState *st, int all, const SpinGrids &sg, cudaStream_t s);
void launch_lsda(long n, const double *rho_a, const double *rho_b, double *exc, double *va, double *vb,
                 cudaStream_t s);
void launch_density_fft(const Tables &t, int nsys, int max_nr, int max_n, const double *rho,
                        double2 *cgrid, cudaStream_t s);
void launch_hf_gradient(const Tables &t, int nsys, const double *rho, const double *wells,
                        const int *well_off, const double *cells, double *part, int max_wells,
                        double *grad, cudaStream_t s);
void launch_hartree_only(const Tables &t, int nsys, int max_nr, int max_n, const double *rho,
                         double2 *cgrid, cudaStream_t s);
void launch_fxc(long long n, const double *rho, double *fxc, cudaStream_t s);
void launch_uniform_density(const Tables &t, int nsys, int max_nr, double *rho, cudaStream_t s);

}  // namespace derek
