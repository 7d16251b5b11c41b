// Non-collinear spinor H.psi and density.
//
// The reference's wavefunction always carries two spinor components,
// coeff(gvec, kpt, band, 1:2) (Source/wave.f90:30,164), and its potential a
// 2x2 matrix per fine-grid point, nc_pot(:, 2, 2) (Source/pot.f90:33,88),
// whose V / B decomposition Source/xsf.f90:44-51 writes as
//   nc_pot = V I + mu_B (Bx sigma_x + By sigma_y + Bz sigma_z),  mu_B = 1/2.
// Its density holds the charge and a three-component spin density,
// den%charge(nr) and den%spin(nr, 3) (Source/density.f90:63-64).  The
// products themselves are empty stubs (pot_apply_wfn, Source/pot.f90:344-382;
// density_calculate, Source/density.f90:101-130); this file defines them:
//   (H psi)_s(G) = 1/2|k+G|^2 psi_s(G) + (1/N) F[ sum_s' V_ss'(r) psi_s'(r) ](G)
//   n(r)  = sum_b w_b (|u_b|^2 + |d_b|^2)
//   m(r)  = sum_b w_b psi_b^H sigma psi_b
//         = sum_b w_b (2 Re u* d, 2 Im u* d, |u|^2 - |d|^2)
// with psi_b(r) = (u_b(r), d_b(r)) = F^-1 of the two coefficient sets.
//
// Layout: band b of a spinor system is two consecutive items, 2b (up) and
// 2b + 1 (down), with coefficient rows 2b and 2b + 1 of the k-set.  A band's
// vector is therefore one contiguous run of 2 npw_pad coefficients, so
// overlaps and rotations see a spinor band as a longer scalar band.  The
// x-line passes of hpsi4.cu run per item unchanged; only the (y,z)-plane
// pass couples the two components, so this file holds that pass (both
// components' planes in shared memory, the 2x2 product in place) and the
// density pass that accumulates n and m.
#include "fft4.cuh"
#include "kernels.cuh"

namespace derek {

size_t spinor_plane_smem(int n2, int n3, size_t elem) {
  return (2 * (size_t)n2 * (n3 + 1) + (size_t)n2 + n3) * elem;
}

template <typename R>
__device__ __forceinline__ void load_lines_tw(cplx<R> *dst, const cplx<R> *src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// Scatter the sphere columns of both components at plane x into the zeroed
// planes P0 (up) and P1 (down), then backward z (rows holding columns) and
// backward y (every column) on both.
template <typename R>
__device__ __forceinline__ void spinor_planes_backward(const Tables &t, const KSetDev &K, const SysDev &S,
                                                       const cplx<R> *a0, const cplx<R> *a1, cplx<R> *P0,
                                                       cplx<R> *P1, const cplx<R> *twy, const cplx<R> *twz) {
  const int n2 = S.n[1], n3 = S.n[2], pz = n3 + 1;
  for (int i = threadIdx.x; i < 2 * n2 * pz; i += blockDim.x) P0[i] = mk<R>(0, 0);
  __syncthreads();
  const short *cy = t.col_y + K.col_off;
  const short *cz = t.col_z + K.col_off;
  for (int c = threadIdx.x; c < K.ncol; c += blockDim.x) {
    const int o = cy[c] * pz + cz[c];
    P0[o] = a0[c];
    P1[o] = a1[c];
  }
  __syncthreads();
  const short *rows = t.rows + K.row_off;
  fft4_lines<R, +1>(P0, S.lp[2], K.nrow, pz, 1, rows, twz);
  fft4_lines<R, +1>(P1, S.lp[2], K.nrow, pz, 1, rows, twz);
  fft4_lines<R, +1>(P0, S.lp[1], n3, 1, pz, nullptr, twy);
  fft4_lines<R, +1>(P1, S.lp[1], n3, 1, pz, nullptr, twy);
}

// (y,z)-plane pass of one band (items 2q, 2q + 1 of the launch) at x-plane
// blockIdx.y: backward yz of both components, the 2x2 product, forward yz,
// columns written back in place.
template <typename R>
__global__ void __launch_bounds__(512) k_plane_spinor(Tables t, int item_begin, cplx<R> *__restrict__ abuf,
                                                      const cplx<R> *__restrict__ vnc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int slot = 2 * blockIdx.x;
  const int item = t.item_list ? t.item_list[slot] : item_begin + slot;
  const int x = blockIdx.y;
  const KSetDev &K = t.ks[t.item_ks[item]];
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int n1 = S.n[0], n2 = S.n[1], n3 = S.n[2];
  const int b = t.item_band[item];
  if (x >= n1 || (b & 1)) return;   // b is the up component; b + 1 < K.nb is the down one
  const int pz = n3 + 1;
  cplx<R> *P0 = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *P1 = P0 + n2 * pz;
  cplx<R> *twy = P1 + n2 * pz;
  cplx<R> *twz = twy + n2;
  load_lines_tw<R>(twy, twtab<R>(t) + S.lp[1].tw_off, n2);
  load_lines_tw<R>(twz, twtab<R>(t) + S.lp[2].tw_off, n3);
  const long long plane = (long long)n1 * K.ncol_pad;
  cplx<R> *a0 = abuf + K.a_off + (long long)b * plane + (long long)x * K.ncol_pad;
  cplx<R> *a1 = a0 + plane;
  spinor_planes_backward<R>(t, K, S, a0, a1, P0, P1, twy, twz);
  const cplx<R> *v = vnc + 4 * (S.grid_off + (long long)x * n2 * n3);
  for (int i = threadIdx.x; i < n2 * n3; i += blockDim.x) {
    const int y = i / n3, z = i - y * n3;
    const int o = y * pz + z;
    const cplx<R> u = P0[o], d = P1[o];
    const cplx<R> v11 = v[4 * i], v21 = v[4 * i + 1], v12 = v[4 * i + 2], v22 = v[4 * i + 3];
    P0[o] = cadd<R>(cmul<R>(v11, u), cmul<R>(v12, d));
    P1[o] = cadd<R>(cmul<R>(v21, u), cmul<R>(v22, d));
  }
  __syncthreads();
  const short *rows = t.rows + K.row_off;
  fft4_lines<R, -1>(P0, S.lp[1], n3, 1, pz, nullptr, twy);
  fft4_lines<R, -1>(P1, S.lp[1], n3, 1, pz, nullptr, twy);
  fft4_lines<R, -1>(P0, S.lp[2], K.nrow, pz, 1, rows, twz);
  fft4_lines<R, -1>(P1, S.lp[2], K.nrow, pz, 1, rows, twz);
  const short *cy = t.col_y + K.col_off;
  const short *cz = t.col_z + K.col_off;
  for (int c = threadIdx.x; c < K.ncol; c += blockDim.x) {
    const int o = cy[c] * pz + cz[c];
    a0[c] = P0[o];
    a1[c] = P1[o];
  }
}

// Density pass per (k-set, x-plane): n, mx, my, mz of the k-set's bands
// with per-item weights occ (equal on both items of a band), written as four
// planes of nr values at partial + partial_off[k-set].  Each thread owns the
// same grid points in every band, so the sums need no synchronisation.
template <typename R>
__global__ void __launch_bounds__(512) k_density_spinor(Tables t, const cplx<R> *__restrict__ abuf,
                                                        const double *__restrict__ occ,
                                                        double *__restrict__ partial,
                                                        const long long *__restrict__ partial_off) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ksi = blockIdx.x;
  const int x = blockIdx.y;
  const KSetDev &K = t.ks[ksi];
  const SysDev &S = t.sys[K.sys];
  if (!S.active || S.nspinor != 2) return;
  const int n1 = S.n[0], n2 = S.n[1], n3 = S.n[2];
  if (x >= n1) return;
  const int pz = n3 + 1;
  cplx<R> *P0 = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *P1 = P0 + n2 * pz;
  cplx<R> *twy = P1 + n2 * pz;
  cplx<R> *twz = twy + n2;
  load_lines_tw<R>(twy, twtab<R>(t) + S.lp[1].tw_off, n2);
  load_lines_tw<R>(twz, twtab<R>(t) + S.lp[2].tw_off, n3);
  const long long nr = S.nr;
  double *dst = partial + partial_off[ksi] + (long long)x * n2 * n3;
  for (int i = threadIdx.x; i < n2 * n3; i += blockDim.x) {
    dst[i] = 0.0;
    dst[nr + i] = 0.0;
    dst[2 * nr + i] = 0.0;
    dst[3 * nr + i] = 0.0;
  }
  const long long plane = (long long)n1 * K.ncol_pad;
  for (int b = 0; b + 1 < K.nb; b += 2) {
    const double w = occ[K.item0 + b];
    if (w == 0.0) continue;
    __syncthreads();   // the previous band's planes are read to the end
    const cplx<R> *a0 = abuf + K.a_off + (long long)b * plane + (long long)x * K.ncol_pad;
    spinor_planes_backward<R>(t, K, S, a0, a0 + plane, P0, P1, twy, twz);
    for (int i = threadIdx.x; i < n2 * n3; i += blockDim.x) {
      const int y = i / n3, z = i - y * n3;
      const cplx<R> u = P0[y * pz + z], d = P1[y * pz + z];
      const double ux = u.x, uy = u.y, dx = d.x, dy = d.y;
      const double uu = ux * ux + uy * uy, dd = dx * dx + dy * dy;
      dst[i] += w * (uu + dd);
      dst[nr + i] += 2.0 * w * (ux * dx + uy * dy);
      dst[2 * nr + i] += 2.0 * w * (ux * dy - uy * dx);
      dst[3 * nr + i] += w * (uu - dd);
    }
  }
}

template <typename R>
void launch_plane_spinor(const Tables &t, int item_begin, int nitems, const int n[3], cplx<R> *abuf,
                         const cplx<R> *vnc, cudaStream_t st) {
  if (nitems <= 1) return;
  const size_t sm = spinor_plane_smem(n[1], n[2], sizeof(cplx<R>));
  cudaFuncSetAttribute(k_plane_spinor<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  derek::note_launch(), k_plane_spinor<R><<<dim3(nitems / 2, n[0]), 512, sm, st>>>(t, item_begin, abuf, vnc);
}

template <typename R>
void launch_density_spinor(const Tables &t, int nks, const int max_n[3], const cplx<R> *abuf,
                           const double *occ, double *partial, const long long *partial_off,
                           cudaStream_t st) {
  if (nks <= 0) return;
  const size_t sm = spinor_plane_smem(max_n[1], max_n[2], sizeof(cplx<R>));
  cudaFuncSetAttribute(k_density_spinor<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  derek::note_launch(), k_density_spinor<R><<<dim3(nks, max_n[0]), 512, sm, st>>>(t, abuf, occ, partial, partial_off);
}

#define DEREK_INST(R)                                                                                  \
  template void launch_plane_spinor<R>(const Tables &, int, int, const int *, cplx<R> *, const cplx<R> *, \
                                       cudaStream_t);                                                  \
  template void launch_density_spinor<R>(const Tables &, int, const int *, const cplx<R> *,            \
                                         const double *, double *, const long long *, cudaStream_t);
DEREK_INST(float)
DEREK_INST(double)
#undef DEREK_INST

}  // namespace derek
