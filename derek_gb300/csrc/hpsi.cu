// Fused H.psi and density kernels.
//
// H psi(G) = 1/2|k+G|^2 psi(G) + (1/N) F[ V(r) F^-1[psi] ](G) on the plane-wave
// sphere of one k-point (the product the reference leaves as a stub in
// pot_apply_wfn, Source/pot.f90:344-382).  F^-1 / F are the unnormalised
// backward / forward transforms of Source/fft.f90:204-212 on the fine grid.
//
// The 3D transforms are split so that each kernel keeps a 2D plane of one
// band in shared memory and touches global memory once per plane:
//   inv_yz  (per band, per x-plane of the sphere): scatter the sphere entries
//           of that x into a (y,z) plane, backward z-transform on the rows
//           holding entries, backward y-transform on all columns, store.
//   vmul_x  (per band, per y): gather the (x,z) plane from the stored
//           x-planes (x outside the sphere's span is zero), backward
//           x-transform, multiply by V(r), forward x-transform, store back
//           only the x-planes the sphere spans (in place).
//   fwd_yz  (per band, per x-plane): forward y-transform, forward
//           z-transform on the rows the sphere needs, gather the sphere,
//           add the kinetic term and apply the filter epilogue
//           out = alpha H psi + beta psi + gamma prev.
// The stored planes hold only the x range the sphere spans, so the
// intermediate traffic shrinks by n1 / nxr.
#include "fft_smem.cuh"
#include "kernels.cuh"

namespace derek {

template <typename R>
__device__ __forceinline__ void load_twiddles(cplx<R> *dst, const cplx<R> *src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

template <typename R>
__global__ void __launch_bounds__(256) k_inv_yz(Tables t, int item_begin, const cplx<R> *__restrict__ psi,
                                                cplx<R> *__restrict__ planes,
                                                const double *__restrict__ occ_skip) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int item = item_begin + blockIdx.x;
  const int j = blockIdx.y;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  if (j >= K.nxr) return;
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  if (occ_skip && occ_skip[item] == 0.0) return;
  const int b = t.item_band[item];
  const int n2 = S.n[1], n3 = S.n[2];
  const int np = n2 * n3;
  cplx<R> *bufA = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *bufB = bufA + np;
  cplx<R> *twy = bufB + np;
  cplx<R> *twz = twy + n2;
  const cplx<R> zero = mk<R>(0, 0);
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    bufA[i] = zero;
    bufB[i] = zero;
  }
  load_twiddles<R>(twy, twtab<R>(t) + S.plan[1].tw_off, n2);
  load_twiddles<R>(twz, twtab<R>(t) + S.plan[2].tw_off, n3);
  __syncthreads();
  const int *xs = t.xstart + K.plane_off;
  const int e0 = xs[j], e1 = xs[j + 1];
  const int *pidx = t.pidx + K.ent_off;
  const cplx<R> *src = psi + K.psi_off + (long long)b * K.npw_pad;
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) bufA[pidx[e]] = src[e];
  __syncthreads();
  const int *rs = t.rowstart + K.plane_off;
  const int r0 = rs[j], r1 = rs[j + 1];
  const short *rows = t.rows + K.row_off + r0;
  cplx<R> *res = fft_lines<R, +1, false>(bufA, bufB, S.plan[2], r1 - r0, n3, 1, twz, rows);
  cplx<R> *oth = res == bufA ? bufB : bufA;
  res = fft_lines<R, +1, true>(res, oth, S.plan[1], n3, 1, n3, twy, nullptr);
  cplx<R> *dst = planes + K.t_off + ((long long)b * K.nxr + j) * np;
  for (int i = threadIdx.x; i < np; i += blockDim.x) dst[i] = res[i];
}

template <typename R>
__global__ void __launch_bounds__(256) k_vmul_x(Tables t, int item_begin, cplx<R> *__restrict__ planes,
                                                const R *__restrict__ vloc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int item = item_begin + blockIdx.x;
  const int y = blockIdx.y;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int n1 = S.n[0], n2 = S.n[1], n3 = S.n[2];
  if (y >= n2) return;
  const int b = t.item_band[item];
  const int np = n1 * n3;
  cplx<R> *bufA = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *bufB = bufA + np;
  cplx<R> *twx = bufB + np;
  const cplx<R> zero = mk<R>(0, 0);
  const int nxr = K.nxr;
  for (int i = threadIdx.x; i < np; i += blockDim.x) bufA[i] = zero;
  load_twiddles<R>(twx, twtab<R>(t) + S.plan[0].tw_off, n1);
  __syncthreads();
  cplx<R> *base = planes + K.t_off + (long long)b * nxr * n2 * n3 + (long long)y * n3;
  const long long pstride = (long long)n2 * n3;
  for (int i = threadIdx.x; i < nxr * n3; i += blockDim.x) {
    const int jj = i / n3, z = i - jj * n3;
    int x = (K.mx_min + jj) % n1;
    if (x < 0) x += n1;
    bufA[x * n3 + z] = base[jj * pstride + z];
  }
  __syncthreads();
  cplx<R> *res = fft_lines<R, +1, true>(bufA, bufB, S.plan[0], n3, 1, n3, twx, nullptr);
  const R *v = vloc + S.grid_off;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const int x = i / n3, z = i - x * n3;
    const R vv = v[((long long)x * n2 + y) * n3 + z];
    res[i] = cscale<R>(res[i], vv);
  }
  __syncthreads();
  cplx<R> *oth = res == bufA ? bufB : bufA;
  res = fft_lines<R, -1, true>(res, oth, S.plan[0], n3, 1, n3, twx, nullptr);
  for (int i = threadIdx.x; i < nxr * n3; i += blockDim.x) {
    const int jj = i / n3, z = i - jj * n3;
    int x = (K.mx_min + jj) % n1;
    if (x < 0) x += n1;
    base[jj * pstride + z] = res[x * n3 + z];
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_fwd_yz(Tables t, int item_begin, const cplx<R> *__restrict__ planes,
                                                const cplx<R> *__restrict__ psi,
                                                const cplx<R> *__restrict__ prev,
                                                cplx<R> *__restrict__ out,
                                                const Axpby *__restrict__ coef) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int item = item_begin + blockIdx.x;
  const int j = blockIdx.y;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  if (j >= K.nxr) return;
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int b = t.item_band[item];
  const int n2 = S.n[1], n3 = S.n[2];
  const int np = n2 * n3;
  cplx<R> *bufA = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *bufB = bufA + np;
  cplx<R> *twy = bufB + np;
  cplx<R> *twz = twy + n2;
  load_twiddles<R>(twy, twtab<R>(t) + S.plan[1].tw_off, n2);
  load_twiddles<R>(twz, twtab<R>(t) + S.plan[2].tw_off, n3);
  const cplx<R> *src = planes + K.t_off + ((long long)b * K.nxr + j) * np;
  for (int i = threadIdx.x; i < np; i += blockDim.x) bufA[i] = src[i];
  __syncthreads();
  cplx<R> *res = fft_lines<R, -1, true>(bufA, bufB, S.plan[1], n3, 1, n3, twy, nullptr);
  cplx<R> *oth = res == bufA ? bufB : bufA;
  const int *rs = t.rowstart + K.plane_off;
  const int r0 = rs[j], r1 = rs[j + 1];
  const short *rows = t.rows + K.row_off + r0;
  res = fft_lines<R, -1, false>(res, oth, S.plan[2], r1 - r0, n3, 1, twz, rows);
  const int *xs = t.xstart + K.plane_off;
  const int e0 = xs[j], e1 = xs[j + 1];
  const int *pidx = t.pidx + K.ent_off;
  const R *kin = kintab<R>(t) + K.ent_off;
  const long long off = K.psi_off + (long long)b * K.npw_pad;
  const R inv_n = (R)(1.0 / (double)S.nr);
  R a = 1, bb = 0, g = 0;
  if (coef) {
    a = (R)coef[ksi].alpha;
    bb = (R)coef[ksi].beta;
    g = (R)coef[ksi].gamma;
  }
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const cplx<R> p = psi[off + e];
    const cplx<R> f = res[pidx[e]];
    const R k = kin[e];
    R hx = f.x * inv_n + k * p.x;
    R hy = f.y * inv_n + k * p.y;
    R ox = a * hx + bb * p.x;
    R oy = a * hy + bb * p.y;
    if (prev) {
      const cplx<R> q = prev[off + e];
      ox += g * q.x;
      oy += g * q.y;
    }
    out[off + e] = mk<R>(ox, oy);
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_density_x(Tables t, int ks_begin, const cplx<R> *__restrict__ planes,
                                                   const double *__restrict__ occ,
                                                   double *__restrict__ partial,
                                                   const long long *__restrict__ partial_off) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ksi = ks_begin + blockIdx.x;
  const int y = blockIdx.y;
  const KSetDev &K = t.ks[ksi];
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int n1 = S.n[0], n2 = S.n[1], n3 = S.n[2];
  if (y >= n2) return;
  const int np = n1 * n3;
  double *acc = reinterpret_cast<double *>(smem_raw);
  cplx<R> *bufA = reinterpret_cast<cplx<R> *>(acc + np);
  cplx<R> *bufB = bufA + np;
  cplx<R> *twx = bufB + np;
  const cplx<R> zero = mk<R>(0, 0);
  for (int i = threadIdx.x; i < np; i += blockDim.x) acc[i] = 0.0;
  load_twiddles<R>(twx, twtab<R>(t) + S.plan[0].tw_off, n1);
  const int nxr = K.nxr;
  const long long pstride = (long long)n2 * n3;
  for (int b = 0; b < K.nb; ++b) {
    const double w = occ[K.item0 + b];
    if (w == 0.0) continue;
    __syncthreads();
    for (int i = threadIdx.x; i < np; i += blockDim.x) bufA[i] = zero;
    __syncthreads();
    const cplx<R> *base = planes + K.t_off + (long long)b * nxr * pstride + (long long)y * n3;
    for (int i = threadIdx.x; i < nxr * n3; i += blockDim.x) {
      const int jj = i / n3, z = i - jj * n3;
      int x = (K.mx_min + jj) % n1;
      if (x < 0) x += n1;
      bufA[x * n3 + z] = base[jj * pstride + z];
    }
    __syncthreads();
    cplx<R> *res = fft_lines<R, +1, true>(bufA, bufB, S.plan[0], n3, 1, n3, twx, nullptr);
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
      const cplx<R> c = res[i];
      acc[i] += w * ((double)c.x * (double)c.x + (double)c.y * (double)c.y);
    }
  }
  __syncthreads();
  double *dst = partial + partial_off[ksi];
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const int x = i / n3, z = i - x * n3;
    dst[((long long)x * n2 + y) * n3 + z] = acc[i];
  }
}

template <typename R> static size_t smem_yz(int max_plane) {
  return (2 * (size_t)max_plane + 2 * kMaxDim) * sizeof(cplx<R>);
}

template <typename R>
void launch_inv_yz(const Tables &t, int item_begin, int nitems, int max_nxr, int max_plane,
                   const cplx<R> *psi, cplx<R> *planes, const double *occ_skip, cudaStream_t st) {
  if (nitems <= 0) return;
  size_t sm = smem_yz<R>(max_plane);
  cudaFuncSetAttribute(k_inv_yz<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid(nitems, max_nxr);
  derek::note_launch(), k_inv_yz<R><<<grid, 256, sm, st>>>(t, item_begin, psi, planes, occ_skip);
}

template <typename R>
void launch_vmul_x(const Tables &t, int item_begin, int nitems, int max_n1, int max_n2, int max_n3,
                   cplx<R> *planes, const R *vloc, cudaStream_t st) {
  if (nitems <= 0) return;
  size_t sm = (2 * (size_t)max_n1 * max_n3 + kMaxDim) * sizeof(cplx<R>);
  cudaFuncSetAttribute(k_vmul_x<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid(nitems, max_n2);
  derek::note_launch(), k_vmul_x<R><<<grid, 256, sm, st>>>(t, item_begin, planes, vloc);
}

template <typename R>
void launch_fwd_yz(const Tables &t, int item_begin, int nitems, int max_nxr, int max_plane,
                   const cplx<R> *planes, const cplx<R> *psi, const cplx<R> *prev, cplx<R> *out,
                   const Axpby *coef, cudaStream_t st) {
  if (nitems <= 0) return;
  size_t sm = smem_yz<R>(max_plane);
  cudaFuncSetAttribute(k_fwd_yz<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid(nitems, max_nxr);
  derek::note_launch(), k_fwd_yz<R><<<grid, 256, sm, st>>>(t, item_begin, planes, psi, prev, out, coef);
}

template <typename R>
void launch_density_x(const Tables &t, int ks_begin, int nks, int max_n1, int max_n2, int max_n3,
                      const cplx<R> *planes, const double *occ, double *partial,
                      const long long *partial_off, cudaStream_t st) {
  if (nks <= 0) return;
  size_t np = (size_t)max_n1 * max_n3;
  size_t sm = np * sizeof(double) + (2 * np + kMaxDim) * sizeof(cplx<R>);
  cudaFuncSetAttribute(k_density_x<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid(nks, max_n2);
  derek::note_launch(), k_density_x<R><<<grid, 256, sm, st>>>(t, ks_begin, planes, occ, partial, partial_off);
}

#define DEREK_INST(R)                                                                          \
  template void launch_inv_yz<R>(const Tables &, int, int, int, int, const cplx<R> *, cplx<R> *, \
                                 const double *, cudaStream_t);                                \
  template void launch_vmul_x<R>(const Tables &, int, int, int, int, int, cplx<R> *, const R *, \
                                 cudaStream_t);                                                \
  template void launch_fwd_yz<R>(const Tables &, int, int, int, int, const cplx<R> *,          \
                                 const cplx<R> *, const cplx<R> *, cplx<R> *, const Axpby *,   \
                                 cudaStream_t);                                                \
  template void launch_density_x<R>(const Tables &, int, int, int, int, int, const cplx<R> *,  \
                                    const double *, double *, const long long *, cudaStream_t);
DEREK_INST(float)
DEREK_INST(double)
#undef DEREK_INST

}  // namespace derek
