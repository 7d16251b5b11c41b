// Device tables shared by the kernels and the launcher declarations.
#pragma once

#include "common.cuh"

namespace derek {

// Read-only tables describing a batch (one copy in device memory).
struct Tables {
  const SysDev *sys;
  const KSetDev *ks;
  const int *item_ks;     // item -> k-set
  const int *item_band;   // item -> band
  const double *kin64;    // sphere entry (column order) -> 1/2|k+G|^2
  const float *kin32;
  const int *ent_col;     // sphere entry -> its column (local index)
  const short *ent_ix;    // sphere entry -> FFT index along x
  const int *col_start;   // per column: first entry (local), ncol + 1 per k-set
  const short *col_y;     // per column: FFT indices along y and z
  const short *col_z;
  const short *col_x0;    // per column: centred Miller x of its first entry
  const short *rows;      // per k-set: the y rows holding columns
  const double2 *tw64;    // twiddle tables exp(-2 pi i t/n)
  const float2 *tw32;
  const int *item_list;   // optional: block x -> item (one grid-size class)
  const double *item_shift;  // optional: per-item extra beta in the H.psi epilogue
};

template <typename R> __device__ __forceinline__ const cplx<R> *twtab(const Tables &t);
template <> __device__ __forceinline__ const float2 *twtab<float>(const Tables &t) { return t.tw32; }
template <> __device__ __forceinline__ const double2 *twtab<double>(const Tables &t) { return t.tw64; }
template <typename R> __device__ __forceinline__ const R *kintab(const Tables &t);
template <> __device__ __forceinline__ const float *kintab<float>(const Tables &t) { return t.kin32; }
template <> __device__ __forceinline__ const double *kintab<double>(const Tables &t) { return t.kin64; }

// Per-k-set coefficients of the fused H.psi epilogue:
//   out = alpha * (tk T psi + V psi) + (beta + shift[item]) * psi + gamma * prev
// (tk = 1 is H; tk = 0 applies the potential alone).
struct Axpby {
  double alpha, beta, gamma, tk;
};

// ---- H.psi and density pipeline (hpsi4.cu) --------------------------------
// Launch geometry: items [item_begin, item_begin + nitems) of the batch.
template <typename R>
void launch_x_inv(const Tables &t, int item_begin, int nitems, int max_nchunk, int max_n1,
                  int min_n1, int max_m, const cplx<R> *psi, cplx<R> *abuf, const double *occ_skip,
                  cudaStream_t st);
// (y,z)-plane pass; a compile-time kernel is used when every system has
// n2 = n3 = N for N in {32, 36, 48, 54, 64, 72}
// max_m: largest |centred Miller index| (x, y or z) of a sphere entry among the items
template <typename R>
void launch_plane(const Tables &t, int item_begin, int nitems, int max_n1, int max_n2, int max_n3,
                  int min_n2, int min_n3, int max_m, cplx<R> *abuf, const R *vloc, cudaStream_t st);
template <typename R>
void launch_x_fwd(const Tables &t, int item_begin, int nitems, int max_nchunk, int max_n1,
                  int min_n1, int max_m, const cplx<R> *abuf, const cplx<R> *psi, const cplx<R> *prev,
                  cplx<R> *out, const Axpby *coef, cudaStream_t st);
template <typename R>
void launch_density_plane(const Tables &t, int ks_begin, int nks, int max_n1, int max_n2, int max_n3,
                          int min_n2, int min_n3, int max_m, const cplx<R> *abuf, const double *occ,
                          double *partial, const long long *partial_off, cudaStream_t st);
// The x passes on shared-memory lines only (the layout k_plane and the
// spinor passes read), never the FP32 register kernels' row layouts.
template <typename R>
void launch_x_inv_lines(const Tables &t, int item_begin, int nitems, int max_nchunk, int max_n1,
                        int min_n1, const cplx<R> *psi, cplx<R> *abuf, const double *occ_skip,
                        cudaStream_t st);
template <typename R>
void launch_x_fwd_lines(const Tables &t, int item_begin, int nitems, int max_nchunk, int max_n1,
                        int min_n1, const cplx<R> *abuf, const cplx<R> *psi, const cplx<R> *prev,
                        cplx<R> *out, const Axpby *coef, cudaStream_t st);

// Non-collinear spinors (spinor.cu).  Band b of a spinor system is items 2b
// (up) and 2b + 1 (down), so a launch covers an even number of items starting
// on a pair.  vnc holds the 2x2 potential per grid point as four complex
// numbers V11, V21, V12, V22 (the reference's nc_pot(n, i, j) order).
template <typename R>
void launch_plane_spinor(const Tables &t, int item_begin, int nitems, const int n[3], cplx<R> *abuf,
                         const cplx<R> *vnc, cudaStream_t st);
// Charge and magnetisation partials per k-set: four planes (n, mx, my, mz)
// of nr values at partial + partial_off[k-set], from the x-line buffer the
// x_inv pass filled for the items with nonzero weight.
template <typename R>
void launch_density_spinor(const Tables &t, int nks, const int max_n[3], const cplx<R> *abuf,
                           const double *occ, double *partial, const long long *partial_off,
                           cudaStream_t st);
size_t spinor_plane_smem(int n2, int n3, size_t elem);

constexpr int kColChunk = 64;   // columns per x-line chunk (kCC in hpsi4.cu)

// FP32 (y,z)-plane passes with register-resident line transforms
// (hpsi_reg.cu), for cubic-plane lengths n in {24, 27, 32, 36, 48, 54, 64, 72};
// they return false for any other n.
bool launch_plane_reg(const Tables &t, int item_begin, int nitems, int max_n1, int n, int max_m,
                      float2 *abuf, const float *vloc, cudaStream_t st);
bool launch_xinv_reg(const Tables &t, int item_begin, int nitems, int max_ncol, int n, int max_m,
                     const float2 *psi, float2 *abuf, const double *occ_skip, cudaStream_t st);
bool launch_xfwd_reg(const Tables &t, int item_begin, int nitems, int max_ncol, int n, int max_m,
                     const float2 *abuf, const float2 *psi, const float2 *prev, float2 *out,
                     const Axpby *coef, cudaStream_t st);
bool launch_density_reg(const Tables &t, int ks_begin, int nks, int max_n1, int n, int max_m,
                        const float2 *abuf, const double *occ, double *partial,
                        const long long *partial_off, cudaStream_t st);

// ---- full-grid FFT (grid.cu) -----------------------------------------------
// In-place unnormalised 3D FFT of one complex FP64 grid per system in
// [sys_begin, sys_begin + nsys); grid s starts at data + sys[s].grid_off.
void launch_fft3d_grid(const Tables &t, int sys_begin, int nsys, int max_n, double2 *data,
                       int sign, cudaStream_t st);

void launch_lda(long n, const double *rho, double *exc, double *vxc, cudaStream_t st);

}  // namespace derek
