// Overlap S = X^H Y that allocates nothing.
//
// Some callers cannot call cudaMalloc.  A Fortran driver, for example, may
// run inside a code that owns the device memory pool or forbids allocation
// once its set-up phase is over.  A library thread may be running while
// another thread captures a CUDA graph.  Such callers pass device pointers for
// the inputs and the output only.  The split-K partial sums that the handle
// path keeps in its own buffer live here instead, in one file-scope device
// array.  Every GPU that loads the library holds that array until the
// process exits.
//
// The entry point derek_gpu_overlap_noalloc shares the array between calls.
// Two calls whose kernels overlap on the GPU (different streams, or threads
// without ordering) race on it and give wrong results.  Every partial is
// written before it is read in the same call, so nothing needs clearing.
//
// The array's device address is looked up once per device, on the first call
// with that device current, and cached.  The cache does not survive a
// cudaDeviceReset: a caller that resets a device must not call this entry
// point again in the same process.  Each launch's own status is taken from
// cudaLaunchKernel, so an error left pending by unrelated earlier work is
// neither reported as this call's nor cleared.
#include <mutex>

#include "common.cuh"

namespace derek {
namespace {

// scratch: up to kStaticSplits K-splits of a kStaticMaxBands^2 complex matrix
constexpr int kStaticMaxBands = 128;
constexpr int kStaticSplits = 16;
constexpr int kStaticSplitK = 4096;  // complex coefficients per split
constexpr long long kStaticElems = (long long)kStaticSplits * kStaticMaxBands * kStaticMaxBands;

__device__ __align__(256) double2 g_overlap_scratch[kStaticElems];  // 4 MiB

constexpr int ST = 16, SKC = 32;

template <typename R>
__global__ void __launch_bounds__(256) k_overlap_partial_flat(const cplx<R> *__restrict__ X,
                                                              const cplx<R> *__restrict__ Y, int nb,
                                                              int npw, long long ld,
                                                              double2 *__restrict__ part) {
  __shared__ cplx<R> As[ST][SKC + 1];
  __shared__ cplx<R> Bs[ST][SKC + 1];
  const int nt = (nb + ST - 1) / ST;
  const int ti = blockIdx.x / nt, tj = blockIdx.x % nt;
  const int split = blockIdx.y;
  const int g0 = split * kStaticSplitK, g1 = min(npw, g0 + kStaticSplitK);
  const int ty = threadIdx.x / ST, tx = threadIdx.x % ST;
  const int i0 = ti * ST, j0 = tj * ST;
  double ar = 0, ai = 0;
  for (int k0 = g0; k0 < g1; k0 += SKC) {
    for (int e = threadIdx.x; e < ST * SKC; e += blockDim.x) {
      const int r = e / SKC, c = e % SKC, g = k0 + c;
      As[r][c] = (i0 + r < nb && g < g1) ? X[(long long)(i0 + r) * ld + g] : mk<R>(0, 0);
      Bs[r][c] = (j0 + r < nb && g < g1) ? Y[(long long)(j0 + r) * ld + g] : mk<R>(0, 0);
    }
    __syncthreads();
    R cr = 0, ci = 0;
    for (int c = 0; c < SKC; ++c) {
      const cplx<R> a = As[ty][c], b = Bs[tx][c];
      cr += a.x * b.x + a.y * b.y;
      ci += a.x * b.y - a.y * b.x;
    }
    ar += (double)cr;
    ai += (double)ci;
    __syncthreads();
  }
  const int i = i0 + ty, j = j0 + tx;
  if (i < nb && j < nb) part[((long long)split * nb + i) * nb + j] = make_double2(ar, ai);
}

__global__ void k_overlap_reduce_flat(const double2 *__restrict__ part, int nb, int nsplit,
                                      double2 *__restrict__ S) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nb * nb; e += gridDim.x * blockDim.x) {
    double x = 0, y = 0;
    for (int s = 0; s < nsplit; ++s) {
      const double2 v = part[(long long)s * nb * nb + e];
      x += v.x;
      y += v.y;
    }
    S[e] = make_double2(x, y);
  }
}

// device address of the scratch array, looked up once per device
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double2 *g_scratch_ptr[kMaxDevices] = {};

int scratch_for_current_device(double2 **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DEREK_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_overlap_scratch) != cudaSuccess || !p) return DEREK_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double2 *>(p);
  }
  *out = g_scratch_ptr[dev];
  return DEREK_OK;
}

}  // namespace
}  // namespace derek

extern "C" int derek_gpu_overlap_noalloc(const void *x, const void *y, int nb, int npw, long ld,
                                         int precision, void *s, void *stream) {
  using namespace derek;
  if (!x || !y || !s || nb <= 0 || npw <= 0 || ld < npw) return DEREK_ERR_BAD_ARG;
  if (precision != DEREK_PREC_FP64 && precision != DEREK_PREC_MIXED) return DEREK_ERR_BAD_ARG;
  const int nsplit = (npw + kStaticSplitK - 1) / kStaticSplitK;
  if (nb > kStaticMaxBands || nsplit > kStaticSplits) return DEREK_ERR_UNSUPPORTED;
  double2 *scratch = nullptr;
  int st = scratch_for_current_device(&scratch);
  if (st) return st;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const int nt = (nb + ST - 1) / ST;
  dim3 grid(nt * nt, nsplit);
  long long ldl = ld;
  void *pargs[] = {const_cast<void **>(&x), const_cast<void **>(&y), &nb, &npw, &ldl, &scratch};
  const void *partial = precision == DEREK_PREC_FP64
                            ? reinterpret_cast<const void *>(&k_overlap_partial_flat<double>)
                            : reinterpret_cast<const void *>(&k_overlap_partial_flat<float>);
  derek::note_launch();
  cudaError_t e = cudaLaunchKernel(partial, grid, dim3(256), pargs, 0, cs);
  if (e == cudaSuccess) {
    void *rargs[] = {&scratch, &nb, const_cast<int *>(&nsplit), &s};
    derek::note_launch();
    e = cudaLaunchKernel(reinterpret_cast<const void *>(&k_overlap_reduce_flat),
                         dim3((nb * nb + 255) / 256), dim3(256), rargs, 0, cs);
  }
  if (e != cudaSuccess) {
    (void)cudaGetLastError();  // this call's own launch error, recorded just now
    return DEREK_ERR_CUDA;
  }
  return DEREK_OK;
}
