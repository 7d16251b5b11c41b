// Fine-grid kernels: full 3D FFT of density-like grids and the LDA
// exchange-correlation evaluation.
#include "fft_smem.cuh"
#include "kernels.cuh"

namespace derek {

// Pass 1 of a full-grid transform: for one x, the contiguous (y,z) plane:
// z-transform of every row, then y-transform of every column.
template <int SIGN>
__global__ void __launch_bounds__(256) k_grid_yz(Tables t, int sys_begin, double2 *__restrict__ data) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const SysDev &S = t.sys[sys_begin + blockIdx.y];
  const int x = blockIdx.x;
  const int n1 = S.n[0], n2 = S.n[1], n3 = S.n[2];
  if (x >= n1) return;
  const int np = n2 * n3;
  double2 *bufA = reinterpret_cast<double2 *>(smem_raw);
  double2 *bufB = bufA + np;
  double2 *twy = bufB + np;
  double2 *twz = twy + n2;
  for (int i = threadIdx.x; i < n2; i += blockDim.x) twy[i] = t.tw64[S.plan[1].tw_off + i];
  for (int i = threadIdx.x; i < n3; i += blockDim.x) twz[i] = t.tw64[S.plan[2].tw_off + i];
  double2 *g = data + S.grid_off + (long long)x * np;
  for (int i = threadIdx.x; i < np; i += blockDim.x) bufA[i] = g[i];
  __syncthreads();
  double2 *res = fft_lines<double, SIGN, false>(bufA, bufB, S.plan[2], n2, n3, 1, twz, nullptr);
  double2 *oth = res == bufA ? bufB : bufA;
  res = fft_lines<double, SIGN, true>(res, oth, S.plan[1], n3, 1, n3, twy, nullptr);
  for (int i = threadIdx.x; i < np; i += blockDim.x) g[i] = res[i];
}

// Pass 2: for one y, the (x,z) plane: x-transform of every column.
template <int SIGN>
__global__ void __launch_bounds__(256) k_grid_x(Tables t, int sys_begin, double2 *__restrict__ data) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const SysDev &S = t.sys[sys_begin + blockIdx.y];
  const int y = blockIdx.x;
  const int n1 = S.n[0], n2 = S.n[1], n3 = S.n[2];
  if (y >= n2) return;
  const int np = n1 * n3;
  double2 *bufA = reinterpret_cast<double2 *>(smem_raw);
  double2 *bufB = bufA + np;
  double2 *twx = bufB + np;
  for (int i = threadIdx.x; i < n1; i += blockDim.x) twx[i] = t.tw64[S.plan[0].tw_off + i];
  double2 *g = data + S.grid_off + (long long)y * n3;
  const long long xs = (long long)n2 * n3;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const int x = i / n3, z = i - x * n3;
    bufA[i] = g[x * xs + z];
  }
  __syncthreads();
  double2 *res = fft_lines<double, SIGN, true>(bufA, bufB, S.plan[0], n3, 1, n3, twx, nullptr);
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const int x = i / n3, z = i - x * n3;
    g[x * xs + z] = res[i];
  }
}

void launch_fft3d_grid(const Tables &t, int sys_begin, int nsys, int max_n, double2 *data, int sign,
                       cudaStream_t st) {
  if (nsys <= 0) return;
  const size_t sm = (2 * (size_t)max_n * max_n + 2 * kMaxDim) * sizeof(double2);
  dim3 grid(max_n, nsys);
  if (sign < 0) {
    cudaFuncSetAttribute(k_grid_yz<-1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaFuncSetAttribute(k_grid_x<-1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_grid_yz<-1><<<grid, 256, sm, st>>>(t, sys_begin, data);
    k_grid_x<-1><<<grid, 256, sm, st>>>(t, sys_begin, data);
  } else {
    cudaFuncSetAttribute(k_grid_yz<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaFuncSetAttribute(k_grid_x<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_grid_yz<1><<<grid, 256, sm, st>>>(t, sys_begin, data);
    k_grid_x<1><<<grid, 256, sm, st>>>(t, sys_begin, data);
  }
}

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

__global__ void k_lda(long n, const double *__restrict__ rho, double *__restrict__ exc,
                      double *__restrict__ vxc) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double e, v;
    lda_point(rho[i], e, v);
    if (exc) exc[i] = e;
    if (vxc) vxc[i] = v;
  }
}

void launch_lda(long n, const double *rho, double *exc, double *vxc, cudaStream_t st) {
  if (n <= 0) return;
  long blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_lda<<<(int)blocks, 256, 0, st>>>(n, rho, exc, vxc);
}

}  // namespace derek
