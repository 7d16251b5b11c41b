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
  const int *pidx;        // sphere entry -> position iy*n3 + iz in its x-plane
  const double *kin64;    // sphere entry -> 1/2|k+G|^2
  const float *kin32;
  const int *xstart;      // per plane: first sphere entry (local), nxr+1 per k-set
  const int *rowstart;    // per plane: first active row (local), nxr+1 per k-set
  const short *rows;      // active y rows of each plane
  const double2 *tw64;    // twiddle tables exp(-2 pi i t/n)
  const float2 *tw32;
};

template <typename R> __device__ __forceinline__ const cplx<R> *twtab(const Tables &t);
template <> __device__ __forceinline__ const float2 *twtab<float>(const Tables &t) { return t.tw32; }
template <> __device__ __forceinline__ const double2 *twtab<double>(const Tables &t) { return t.tw64; }
template <typename R> __device__ __forceinline__ const R *kintab(const Tables &t);
template <> __device__ __forceinline__ const float *kintab<float>(const Tables &t) { return t.kin32; }
template <> __device__ __forceinline__ const double *kintab<double>(const Tables &t) { return t.kin64; }

// Per-k-set coefficients of the fused H.psi epilogue:
//   out = alpha * (H psi) + beta * psi + gamma * prev
struct Axpby {
  double alpha, beta, gamma;
};

// ---- H.psi and density pipeline (hpsi.cu) ---------------------------------
// Launch geometry: items [item_begin, item_begin + nitems) of the batch.
//   inv_yz : scatter sphere -> backward z and y transforms -> plane buffer
//   vmul_x : backward x transform, V(r) multiply, forward x transform
//   fwd_yz : forward y and z transforms -> gather sphere, kinetic, epilogue
template <typename R>
void launch_inv_yz(const Tables &t, int item_begin, int nitems, int max_nxr, int max_plane,
                   const cplx<R> *psi, cplx<R> *planes, const double *occ_skip,
                   cudaStream_t st);
template <typename R>
void launch_vmul_x(const Tables &t, int item_begin, int nitems, int max_n1, int max_n2,
                   int max_n3, cplx<R> *planes, const R *vloc, cudaStream_t st);
template <typename R>
void launch_fwd_yz(const Tables &t, int item_begin, int nitems, int max_nxr, int max_plane,
                   const cplx<R> *planes, const cplx<R> *psi, const cplx<R> *prev,
                   cplx<R> *out, const Axpby *coef, cudaStream_t st);
// density: per (k-set, y) loop over bands, accumulate occ-weighted |psi(r)|^2
template <typename R>
void launch_density_x(const Tables &t, int ks_begin, int nks, int max_n1, int max_n2,
                      int max_n3, const cplx<R> *planes, const double *occ,
                      double *partial, const long long *partial_off, cudaStream_t st);

// ---- full-grid FFT (grid.cu) -----------------------------------------------
// In-place unnormalised 3D FFT of one complex FP64 grid per system in
// [sys_begin, sys_begin + nsys); grid s starts at data + sys[s].grid_off.
void launch_fft3d_grid(const Tables &t, int sys_begin, int nsys, int max_n, double2 *data,
                       int sign, cudaStream_t st);

void launch_lda(long n, const double *rho, double *exc, double *vxc, cudaStream_t st);

}  // namespace derek
