// Shared types and helpers for the DEReK GB300 library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "derek_gpu.h"

namespace derek {

// Complex element type per precision: float2 (FP32 path) or double2 (FP64).
template <typename R> struct CT;
template <> struct CT<float>  { using T = float2; };
template <> struct CT<double> { using T = double2; };
template <typename R> using cplx = typename CT<R>::T;

template <typename R> __host__ __device__ __forceinline__ cplx<R> mk(R x, R y) {
  cplx<R> c; c.x = x; c.y = y; return c;
}
template <typename R> __host__ __device__ __forceinline__ cplx<R> cadd(cplx<R> a, cplx<R> b) {
  return mk<R>(a.x + b.x, a.y + b.y);
}
template <typename R> __host__ __device__ __forceinline__ cplx<R> csub(cplx<R> a, cplx<R> b) {
  return mk<R>(a.x - b.x, a.y - b.y);
}
template <typename R> __host__ __device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) {
  return mk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
template <typename R> __host__ __device__ __forceinline__ cplx<R> cmulc(cplx<R> a, cplx<R> b) {
  return mk<R>(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <typename R> __host__ __device__ __forceinline__ cplx<R> cscale(cplx<R> a, R s) {
  return mk<R>(a.x * s, a.y * s);
}

constexpr int kMaxRadices = 8;
constexpr int kMaxDim = 128;       // largest FFT length along one axis

// Radix plan of one FFT length (product of radices == n).
struct FftPlan {
  int n;
  int nstages;
  int radix[kMaxRadices];
  long long tw_off;   // offset of this length's twiddle table (n entries)
};

// Factorisation of one transform length for the four-step line kernels:
// n = a * b with a, b <= 16; group = lines per warp (32 / max(a, b)).
struct LinePlan {
  int n, a, b, group;
  long long tw_off;        // twiddle table exp(-2 pi i t / n), t < n
};

// One independent Kohn-Sham system of a batch.
struct SysDev {
  int n[3];
  int nr;
  int nk;
  int nb;                  // bands carried (requested + buffer), x nspinor
  int nbr;                 // bands requested and reported, x nspinor
  int ks0;                 // first k-set index of this system
  int active;              // 0 once converged (work items exit early)
  int nspinor;             // 1, or 2: band b is items 2b (up) and 2b + 1 (down)
  double volume;
  double B[9];             // inv_cell, row-major: G_i = sum_j B[i*3+j] m_j
  double ecut;
  double nelec;
  double kT;
  long long grid_off;      // offset of this system's grids (nr entries)
  FftPlan plan[3];         // Stockham plans (full-grid transforms)
  LinePlan lp[3];          // four-step plans (H.psi and density)
};

// One (system, k-point) pair: its plane-wave sphere and buffers.  The
// sphere's coefficients are stored in column order: the ncol (y,z) columns
// the sphere occupies, each a contiguous run of increasing Miller x.
struct KSetDev {
  int sys;
  int kidx;
  int npw;
  int npw_pad;
  int nb;                  // bands carried (requested + buffer), x nspinor
  int nbr;                 // bands requested and reported, x nspinor
  int ncol;                // (y,z) columns of the sphere
  int ncol_pad;
  int nrow;                // distinct y rows holding columns
  int item0;               // first (k-set, band) item of this k-set
  long long psi_off;       // element offset of band 0 in psi-shaped buffers
  long long ent_off;       // offset into per-sphere-entry tables
  long long col_off;       // offset into per-column tables (ncol + 1 entries)
  long long row_off;       // offset into the active-row lists
  long long a_off;         // element offset in the x-line buffer (nb * n1 * ncol_pad)
  double wk;
  double kfrac[3];
};

// Host-side count of kernel launches issued by the library (every launch
// site calls note_launch; a CUDA graph replay adds its captured kernel count).
void note_launch(long long n = 1);
unsigned long long launch_total();

// Error codes mirrored from the C ABI.
enum Status : int {
  OK = DEREK_OK,
  BAD_ARG = DEREK_ERR_BAD_ARG,
  OOM = DEREK_ERR_OOM,
  CUDA = DEREK_ERR_CUDA,
  NOT_CONVERGED = DEREK_ERR_NOT_CONVERGED,
  CHOLESKY = DEREK_ERR_CHOLESKY,
  NAN_DETECTED = DEREK_ERR_NAN,
  TIMEOUT = DEREK_ERR_TIMEOUT,
  UNSUPPORTED = DEREK_ERR_UNSUPPORTED,
};

}  // namespace derek
