// Launchers of the subspace kernels (subspace.cu) and the SCF grid kernels
// (scf_kernels.cu).
#pragma once

#include "kernels.cuh"

namespace derek {

constexpr int kMaxBands = 128;   // per k-set (rotation kernel register tile)
constexpr int kOverlapSplit = 2048;      // default split-K (complex coefficients per CTA)
constexpr int kOverlapSplitMin = 512;    // smallest split the partial buffers hold

template <typename R>
void launch_overlap(const Tables &t, int ks_begin, int nks, int max_nb, int max_npw, int ksplit,
                    const cplx<R> *A, const cplx<R> *B, double2 *part, const long long *part_off,
                    double2 *out, const long long *mat_off, int hermitize, cudaStream_t st);
void launch_overlap_reduce(const Tables &t, int ks_begin, int nks, const double2 *part,
                           const long long *part_off, int ksplit, double2 *out,
                           const long long *mat_off, int hermitize, cudaStream_t st);
// split-BF16 tcgen05 overlap (complex64 inputs, nb <= 128), same partial layout
size_t overlap_tc_smem(int max_nb);
void launch_overlap_tc(const Tables &t, int ks_begin, int nks, int max_nb, int max_npw, int ksplit,
                       const float2 *X, const float2 *Y, double2 *part, const long long *part_off,
                       double2 *out, const long long *mat_off, int hermitize, int *status,
                       cudaStream_t st);
// split-BF16 tcgen05 rotation X <- X C (complex64, nb <= 128), in place
// img: rotate_tc_image_bytes(max_nb) bytes per k-set of scratch for the
// converted B operand
size_t rotate_tc_image_bytes(int max_nb);
void launch_rotate_tc(const Tables &t, int ks_begin, int nks, int max_nb, int max_npw, float2 *X,
                      const double2 *C, const long long *mat_off, unsigned char *img, int *status,
                      cudaStream_t st);
// try limit of the tensor-core kernels' pipeline-stage waits (< 0: default)
int set_stage_wait_limit(long iterations);
template <typename R>
void launch_rotate(const Tables &t, int ks_begin, int nks, int max_nb, int max_npw, cplx<R> *X,
                   const double2 *C, const long long *mat_off, cudaStream_t st);
bool cholesky_fits_smem(int max_nb);
void launch_cholesky_inv(const Tables &t, int ks_begin, int nks, int max_nb, const double2 *S,
                         double2 *C, const long long *mat_off, double2 *scratch, int *status,
                         cudaStream_t st);
// fp32_vectors: accumulate the eigenvectors in FP32 (A stays FP64); single:
// one CTA per k-set even where the two-CTA cluster kernel fits
void launch_jacobi(const Tables &t, int ks_begin, int nks, int max_nb, const double2 *Hs,
                   double2 *C, const long long *mat_off, double *eig, double2 *scratch,
                   int max_sweeps, double tol, int fp32_vectors, int *sweeps_out, cudaStream_t st,
                   int single = 0);

// Per-system SCF scalars kept on the device.
constexpr int kMaxHist = 16;
struct SysState {
  double mu, entropy, e_band, e_dc, e_h, e_xc, energy, free, free_prev, delta;
  double vmax;             // max V_loc (filter upper bound)
  double etol;
  double rtol;             // density residual tolerance (0 = off)
  double resid;            // max|n_out - n_in|
  int iter;
  int converged;
  int status;
  int nhist;               // stored mixing pairs
  int slot;                // slot of the newest pair
  int pad;
  double gram[kMaxHist * kMaxHist];
  double coef[kMaxHist];
};

}  // namespace derek
