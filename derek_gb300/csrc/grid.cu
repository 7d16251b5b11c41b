// Fine-grid kernels: full 3D FFT of density-like grids and the LDA
// exchange-correlation evaluation.
#include "fft_smem.cuh"
#include "kernels.cuh"
#include "xc.cuh"

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
    derek::note_launch(), k_grid_yz<-1><<<grid, 256, sm, st>>>(t, sys_begin, data);
    derek::note_launch(), k_grid_x<-1><<<grid, 256, sm, st>>>(t, sys_begin, data);
  } else {
    cudaFuncSetAttribute(k_grid_yz<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaFuncSetAttribute(k_grid_x<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    derek::note_launch(), k_grid_yz<1><<<grid, 256, sm, st>>>(t, sys_begin, data);
    derek::note_launch(), k_grid_x<1><<<grid, 256, sm, st>>>(t, sys_begin, data);
  }
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
  derek::note_launch(), k_lda<<<(int)blocks, 256, 0, st>>>(n, rho, exc, vxc);
}

}  // namespace derek
