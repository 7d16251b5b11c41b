// Fused H.psi and density kernels on the x-first decomposition.
//
// H psi(G) = 1/2|k+G|^2 psi(G) + (1/N) F[ V(r) F^-1[psi] ](G) on the sphere of
// one k-point -- the product the reference leaves as a stub in pot_apply_wfn
// (Source/pot.f90:344-382); F^-1 / F are the unnormalised backward / forward
// transforms of Source/fft.f90:204-212 on the fine grid.
//
// Inside the library the sphere coefficients of a k-point are kept in
// column order: the (y,z) columns the sphere occupies one after another, each
// column's entries in increasing Miller x (a contiguous run).  The reference
// order (x outermost, Source/basis.f90:125-135) is restored at the C ABI.
// With that order the transform splits into three passes that each keep a
// whole 1D line set or 2D plane of one band in shared memory:
//   x_inv  (band, chunk of columns): scatter each column's entries into an
//          x-line, backward x transform, store line values per x-plane
//          (buffer A[band][x][column]).
//   plane  (band, x-plane): gather the columns of that x into a (y,z) plane,
//          backward z on the rows holding columns, backward y on every
//          column, multiply by V(r), forward y, forward z on those rows,
//          scatter the columns back into A (in place).
//   x_fwd  (band, chunk of columns): forward x transform of each column,
//          gather the sphere, add the kinetic term, filter epilogue
//          out = alpha H psi + beta psi + gamma prev.
// Intermediate traffic per band is 2 x (x-lines of the sphere's columns)
// instead of full (y,z) planes.
#include "fft4.cuh"
#include "kernels.cuh"

namespace derek {

constexpr int kCC = kColChunk;

template <typename R>
__device__ __forceinline__ void load_tw(cplx<R> *dst, const cplx<R> *src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// ---- pass 1: backward x transforms of the sphere's columns ----------------
template <typename R, int NX>
__global__ void __launch_bounds__(256) k_x_inv(Tables t, int item_begin, const cplx<R> *__restrict__ psi,
                                               cplx<R> *__restrict__ abuf,
                                               const double *__restrict__ occ_skip) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int item = t.item_list ? t.item_list[blockIdx.x] : item_begin + blockIdx.x;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  const int c0 = blockIdx.y * kCC;
  if (c0 >= K.ncol) return;
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  if (occ_skip && occ_skip[item] == 0.0) return;
  const int b = t.item_band[item];
  const int n1 = NX ? NX : S.n[0];
  const int pl = n1 + 1;  // odd line pitch
  const int nc = min(kCC, K.ncol - c0);
  cplx<R> *L = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *tw = L + kCC * pl;
  for (int i = threadIdx.x; i < nc * pl; i += blockDim.x) L[i] = mk<R>(0, 0);
  load_tw<R>(tw, twtab<R>(t) + S.lp[0].tw_off, n1);
  __syncthreads();
  const int *cs = t.col_start + K.col_off;
  const int e0 = cs[c0], e1 = cs[c0 + nc];
  const cplx<R> *src = psi + K.psi_off + (long long)b * K.npw_pad;
  const int *ecol = t.ent_col + K.ent_off;
  const short *eix = t.ent_ix + K.ent_off;
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) L[(ecol[e] - c0) * pl + eix[e]] = src[e];
  __syncthreads();
  if (NX)
    fft4_fixed<R, +1, NX ? NX : 1, 1, NX + 1>(L, nc, nullptr, tw);
  else
    fft4_lines<R, +1>(L, S.lp[0], nc, pl, 1, nullptr, tw);
  cplx<R> *dst = abuf + K.a_off + (long long)b * n1 * K.ncol_pad + c0;
  for (int i = threadIdx.x; i < n1 * nc; i += blockDim.x) {
    const int x = i / nc, c = i - x * nc;
    dst[(long long)x * K.ncol_pad + c] = L[c * pl + x];
  }
}

// ---- pass 2: (y,z) planes: backward yz, V(r), forward yz ------------------
template <typename R>
__global__ void __launch_bounds__(512) k_plane(Tables t, int item_begin, cplx<R> *__restrict__ abuf,
                                               const R *__restrict__ vloc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int item = t.item_list ? t.item_list[blockIdx.x] : item_begin + blockIdx.x;
  const int x = blockIdx.y;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int n1 = S.n[0], n2 = S.n[1], n3 = S.n[2];
  if (x >= n1) return;
  const int b = t.item_band[item];
  const int pz = n3 + 1;  // odd row pitch
  cplx<R> *P = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *twy = P + n2 * pz;
  cplx<R> *twz = twy + n2;
  for (int i = threadIdx.x; i < n2 * pz; i += blockDim.x) P[i] = mk<R>(0, 0);
  load_tw<R>(twy, twtab<R>(t) + S.lp[1].tw_off, n2);
  load_tw<R>(twz, twtab<R>(t) + S.lp[2].tw_off, n3);
  __syncthreads();
  cplx<R> *a = abuf + K.a_off + ((long long)b * n1 + x) * K.ncol_pad;
  const short *cy = t.col_y + K.col_off;
  const short *cz = t.col_z + K.col_off;
  for (int c = threadIdx.x; c < K.ncol; c += blockDim.x) P[cy[c] * pz + cz[c]] = a[c];
  __syncthreads();
  const short *rows = t.rows + K.row_off;
  fft4_lines<R, +1>(P, S.lp[2], K.nrow, pz, 1, rows, twz);      // z, rows with columns
  fft4_lines<R, +1>(P, S.lp[1], n3, 1, pz, nullptr, twy);       // y, every column
  const R *v = vloc + S.grid_off + (long long)x * n2 * n3;
  for (int i = threadIdx.x; i < n2 * n3; i += blockDim.x) {
    const int y = i / n3, z = i - y * n3;
    P[y * pz + z] = cscale<R>(P[y * pz + z], v[i]);
  }
  __syncthreads();
  fft4_lines<R, -1>(P, S.lp[1], n3, 1, pz, nullptr, twy);
  fft4_lines<R, -1>(P, S.lp[2], K.nrow, pz, 1, rows, twz);
  for (int c = threadIdx.x; c < K.ncol; c += blockDim.x) a[c] = P[cy[c] * pz + cz[c]];
}

// Same pass for n2 = n3 = N known at compile time (cubic grids).
template <typename R, int N>
__global__ void __launch_bounds__(512) k_plane_fixed(Tables t, int item_begin, cplx<R> *__restrict__ abuf,
                                                     const R *__restrict__ vloc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int PZ = N + 1;
  const int item = t.item_list ? t.item_list[blockIdx.x] : item_begin + blockIdx.x;
  const int x = blockIdx.y;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int n1 = S.n[0];
  if (x >= n1) return;
  const int b = t.item_band[item];
  cplx<R> *P = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *tw = P + N * PZ;
  for (int i = threadIdx.x; i < N * PZ; i += blockDim.x) P[i] = mk<R>(0, 0);
  load_tw<R>(tw, twtab<R>(t) + S.lp[1].tw_off, N);
  __syncthreads();
  cplx<R> *a = abuf + K.a_off + ((long long)b * n1 + x) * K.ncol_pad;
  const short *cy = t.col_y + K.col_off;
  const short *cz = t.col_z + K.col_off;
  for (int c = threadIdx.x; c < K.ncol; c += blockDim.x) P[cy[c] * PZ + cz[c]] = a[c];
  __syncthreads();
  const short *rows = t.rows + K.row_off;
  fft4_fixed<R, +1, N, 1, PZ>(P, K.nrow, rows, tw);
  fft4_fixed<R, +1, N, PZ, 1>(P, N, nullptr, tw);
  const R *v = vloc + S.grid_off + (long long)x * N * N;
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) {
    const int y = i / N, z = i - y * N;
    P[y * PZ + z] = cscale<R>(P[y * PZ + z], v[i]);
  }
  __syncthreads();
  fft4_fixed<R, -1, N, PZ, 1>(P, N, nullptr, tw);
  fft4_fixed<R, -1, N, 1, PZ>(P, K.nrow, rows, tw);
  for (int c = threadIdx.x; c < K.ncol; c += blockDim.x) a[c] = P[cy[c] * PZ + cz[c]];
}

// (y,z) pass for n2 = n3 = N known at compile time, with the backward and
// forward y transforms of a column fused around V(r).  The backward transform
// uses N = A * B (step 1 radix A, step 2 radix B); its step-2 thread for k1
// holds X[k1 + A k2], k2 < B, which is exactly the step-1 input of a forward
// transform factored the other way (N = B * A, n2' = k1, n1' = k2).  So the
// column goes  step1_bwd -> [smem] -> step2_bwd * V -> step1_fwd -> [smem]
// -> step2_fwd  with V(r) applied in registers and no block barrier between.
template <typename R, int N, int NT>
__global__ void __launch_bounds__(NT) k_plane_fused(Tables t, int item_begin, cplx<R> *__restrict__ abuf,
                                                    const R *__restrict__ vloc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int PZ = N + 1;
  constexpr int A = plan_a(N);
  constexpr int B = N / A;
  constexpr int SPAN = A > B ? A : B;
  constexpr int G = 32 / SPAN;
  const int item = t.item_list ? t.item_list[blockIdx.x] : item_begin + blockIdx.x;
  const int x = blockIdx.y;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int n1 = S.n[0];
  if (x >= n1) return;
  const int b = t.item_band[item];
  cplx<R> *P = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *tw = P + N * PZ;
  for (int i = threadIdx.x; i < N * PZ; i += NT) P[i] = mk<R>(0, 0);
  for (int i = threadIdx.x; i < N; i += NT) tw[i] = twtab<R>(t)[S.lp[1].tw_off + i];
  __syncthreads();
  cplx<R> *a = abuf + K.a_off + ((long long)b * n1 + x) * K.ncol_pad;
  const short *cy = t.col_y + K.col_off;
  const short *cz = t.col_z + K.col_off;
  for (int c = threadIdx.x; c < K.ncol; c += NT) P[cy[c] * PZ + cz[c]] = a[c];
  __syncthreads();
  const short *rows = t.rows + K.row_off;
  fft4_fixed<R, +1, N, 1, PZ>(P, K.nrow, rows, tw);  // backward z on the rows with columns
  const R *v = vloc + S.grid_off + (long long)x * N * N;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane / SPAN, r = lane - g * SPAN;
  for (int l0 = warp * G; l0 < N; l0 += (NT / 32) * G) {
    const int z = l0 + g;
    const bool live = g < G && z < N;
    cplx<R> *col = P + (live ? z : 0);
    // backward step 1: radix A over n1 for n2 = r
    if (live && r < B) {
      cplx<R> u[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) u[n1] = col[(B * n1 + r) * PZ];
      Dft<R, A, +1>::run(u);
#pragma unroll
      for (int k1 = 1; k1 < A; ++k1) {
        cplx<R> w = tw[(r * k1) % N];
        w.y = -w.y;
        u[k1] = cmul<R>(u[k1], w);
      }
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) col[(B * k1 + r) * PZ] = u[k1];
    }
    __syncwarp();
    // backward step 2 (radix B) for k1 = r, times V, forward step 1 (radix B)
    cplx<R> u[B];
    const bool act = live && r < A;
    if (act) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) u[n2] = col[(B * r + n2) * PZ];
    }
    __syncwarp();
    if (act) {
      Dft<R, B, +1>::run(u);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) u[k2] = cscale<R>(u[k2], v[(r + A * k2) * N + z]);
      Dft<R, B, -1>::run(u);
#pragma unroll
      for (int k1 = 1; k1 < B; ++k1) u[k1] = cmul<R>(u[k1], tw[(r * k1) % N]);
#pragma unroll
      for (int k1 = 0; k1 < B; ++k1) col[(A * k1 + r) * PZ] = u[k1];
    }
    __syncwarp();
    // forward step 2 (radix A) for k1' = r < B: natural-order output r + B k2
    cplx<R> q[A];
    const bool act2 = live && r < B;
    if (act2) {
#pragma unroll
      for (int n2 = 0; n2 < A; ++n2) q[n2] = col[(A * r + n2) * PZ];
    }
    __syncwarp();
    if (act2) {
      Dft<R, A, -1>::run(q);
#pragma unroll
      for (int k2 = 0; k2 < A; ++k2) col[(r + B * k2) * PZ] = q[k2];
    }
    __syncwarp();
  }
  __syncthreads();
  fft4_fixed<R, -1, N, 1, PZ>(P, K.nrow, rows, tw);  // forward z on the rows needed
  for (int c = threadIdx.x; c < K.ncol; c += NT) a[c] = P[cy[c] * PZ + cz[c]];
}

// ---- pass 3: forward x transforms, gather, kinetic, epilogue --------------
template <typename R, int NX>
__global__ void __launch_bounds__(256) k_x_fwd(Tables t, int item_begin, const cplx<R> *__restrict__ abuf,
                                               const cplx<R> *__restrict__ psi,
                                               const cplx<R> *__restrict__ prev,
                                               cplx<R> *__restrict__ out,
                                               const Axpby *__restrict__ coef) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int item = t.item_list ? t.item_list[blockIdx.x] : item_begin + blockIdx.x;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  const int c0 = blockIdx.y * kCC;
  if (c0 >= K.ncol) return;
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int b = t.item_band[item];
  const int n1 = NX ? NX : S.n[0];
  const int pl = n1 + 1;
  const int nc = min(kCC, K.ncol - c0);
  cplx<R> *L = reinterpret_cast<cplx<R> *>(smem_raw);
  cplx<R> *tw = L + kCC * pl;
  load_tw<R>(tw, twtab<R>(t) + S.lp[0].tw_off, n1);
  const cplx<R> *src = abuf + K.a_off + (long long)b * n1 * K.ncol_pad + c0;
  for (int i = threadIdx.x; i < n1 * nc; i += blockDim.x) {
    const int x = i / nc, c = i - x * nc;
    L[c * pl + x] = src[(long long)x * K.ncol_pad + c];
  }
  __syncthreads();
  if (NX)
    fft4_fixed<R, -1, NX ? NX : 1, 1, NX + 1>(L, nc, nullptr, tw);
  else
    fft4_lines<R, -1>(L, S.lp[0], nc, pl, 1, nullptr, tw);
  const int *cs = t.col_start + K.col_off;
  const int e0 = cs[c0], e1 = cs[c0 + nc];
  const int *ecol = t.ent_col + K.ent_off;
  const short *eix = t.ent_ix + K.ent_off;
  const R *kin = kintab<R>(t) + K.ent_off;
  const long long off = K.psi_off + (long long)b * K.npw_pad;
  const R inv_n = (R)(1.0 / (double)S.nr);
  R al = 1, be = 0, ga = 0, tk = 1;
  if (coef) {
    al = (R)coef[ksi].alpha;
    be = (R)coef[ksi].beta;
    ga = (R)coef[ksi].gamma;
    tk = (R)coef[ksi].tk;
  }
  if (t.item_shift) be += (R)t.item_shift[item];
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const cplx<R> p = psi[off + e];
    const cplx<R> f = L[(ecol[e] - c0) * pl + eix[e]];
    const R k = tk * kin[e];
    const R hx = f.x * inv_n + k * p.x;
    const R hy = f.y * inv_n + k * p.y;
    R ox = al * hx + be * p.x;
    R oy = al * hy + be * p.y;
    if (prev) {
      const cplx<R> q = prev[off + e];
      ox += ga * q.x;
      oy += ga * q.y;
    }
    out[off + e] = mk<R>(ox, oy);
  }
}

// ---- density: per (k-set, x-plane), loop over bands ------------------------
// FP64 accumulators of one plane, rounded up to an even count so that the
// complex planes after them start on a 16-byte boundary (a double2 needs it)
__host__ __device__ constexpr int density_acc_count(int points) { return (points + 1) & ~1; }

template <typename R>
__global__ void __launch_bounds__(512) k_density_plane(Tables t, int ks_begin, const cplx<R> *__restrict__ abuf,
                                                       const double *__restrict__ occ,
                                                       double *__restrict__ partial,
                                                       const long long *__restrict__ partial_off) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ksi = ks_begin + blockIdx.x;
  const int x = blockIdx.y;
  const KSetDev &K = t.ks[ksi];
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int n1 = S.n[0], n2 = S.n[1], n3 = S.n[2];
  if (x >= n1) return;
  const int pz = n3 + 1;
  double *acc = reinterpret_cast<double *>(smem_raw);
  // the planes start on a 16-byte boundary: an even count of accumulators
  cplx<R> *P = reinterpret_cast<cplx<R> *>(acc + density_acc_count(n2 * n3));
  cplx<R> *twy = P + n2 * pz;
  cplx<R> *twz = twy + n2;
  for (int i = threadIdx.x; i < n2 * n3; i += blockDim.x) acc[i] = 0.0;
  load_tw<R>(twy, twtab<R>(t) + S.lp[1].tw_off, n2);
  load_tw<R>(twz, twtab<R>(t) + S.lp[2].tw_off, n3);
  const short *cy = t.col_y + K.col_off;
  const short *cz = t.col_z + K.col_off;
  const short *rows = t.rows + K.row_off;
  for (int b = 0; b < K.nb; ++b) {
    const double w = occ[K.item0 + b];
    if (w == 0.0) continue;
    __syncthreads();
    for (int i = threadIdx.x; i < n2 * pz; i += blockDim.x) P[i] = mk<R>(0, 0);
    __syncthreads();
    const cplx<R> *a = abuf + K.a_off + ((long long)b * n1 + x) * K.ncol_pad;
    for (int c = threadIdx.x; c < K.ncol; c += blockDim.x) P[cy[c] * pz + cz[c]] = a[c];
    __syncthreads();
    fft4_lines<R, +1>(P, S.lp[2], K.nrow, pz, 1, rows, twz);
    fft4_lines<R, +1>(P, S.lp[1], n3, 1, pz, nullptr, twy);
    for (int i = threadIdx.x; i < n2 * n3; i += blockDim.x) {
      const int y = i / n3, z = i - y * n3;
      const cplx<R> c = P[y * pz + z];
      acc[i] += w * ((double)c.x * (double)c.x + (double)c.y * (double)c.y);
    }
  }
  __syncthreads();
  double *dst = partial + partial_off[ksi] + (long long)x * n2 * n3;
  for (int i = threadIdx.x; i < n2 * n3; i += blockDim.x) dst[i] = acc[i];
}

// Density pass for n2 = n3 = N known at compile time.
template <typename R, int N, int NT>
__global__ void __launch_bounds__(NT) k_density_fixed(Tables t, int ks_begin, const cplx<R> *__restrict__ abuf,
                                                      const double *__restrict__ occ,
                                                      double *__restrict__ partial,
                                                      const long long *__restrict__ partial_off) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int PZ = N + 1;
  const int ksi = ks_begin + blockIdx.x;
  const int x = blockIdx.y;
  const KSetDev &K = t.ks[ksi];
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int n1 = S.n[0];
  if (x >= n1) return;
  double *acc = reinterpret_cast<double *>(smem_raw);
  cplx<R> *P = reinterpret_cast<cplx<R> *>(acc + density_acc_count(N * N));
  cplx<R> *tw = P + N * PZ;
  for (int i = threadIdx.x; i < N * N; i += NT) acc[i] = 0.0;
  for (int i = threadIdx.x; i < N; i += NT) tw[i] = twtab<R>(t)[S.lp[1].tw_off + i];
  const short *cy = t.col_y + K.col_off;
  const short *cz = t.col_z + K.col_off;
  const short *rows = t.rows + K.row_off;
  for (int b = 0; b < K.nb; ++b) {
    const double w = occ[K.item0 + b];
    if (w == 0.0) continue;
    __syncthreads();
    for (int i = threadIdx.x; i < N * PZ; i += NT) P[i] = mk<R>(0, 0);
    __syncthreads();
    const cplx<R> *a = abuf + K.a_off + ((long long)b * n1 + x) * K.ncol_pad;
    for (int c = threadIdx.x; c < K.ncol; c += NT) P[cy[c] * PZ + cz[c]] = a[c];
    __syncthreads();
    fft4_fixed<R, +1, N, 1, PZ>(P, K.nrow, rows, tw);
    fft4_fixed<R, +1, N, PZ, 1>(P, N, nullptr, tw);
    for (int i = threadIdx.x; i < N * N; i += NT) {
      const int y = i / N, z = i - y * N;
      const cplx<R> c = P[y * PZ + z];
      acc[i] += w * ((double)c.x * (double)c.x + (double)c.y * (double)c.y);
    }
  }
  __syncthreads();
  double *dst = partial + partial_off[ksi] + (long long)x * N * N;
  for (int i = threadIdx.x; i < N * N; i += NT) dst[i] = acc[i];
}

// ---- launchers --------------------------------------------------------------
template <typename R> static size_t smem_x(int max_n1) {
  return ((size_t)kCC * (max_n1 + 1) + kMaxDim) * sizeof(cplx<R>);
}
template <typename R> static size_t smem_plane(int max_n2, int max_n3) {
  return ((size_t)max_n2 * (max_n3 + 1) + 2 * kMaxDim) * sizeof(cplx<R>);
}


template <typename R, int NX>
static void x_inv_go(const Tables &t, int item_begin, int nitems, int max_nchunk, int max_n1,
                     const cplx<R> *psi, cplx<R> *abuf, const double *occ_skip, cudaStream_t st) {
  const size_t sm = smem_x<R>(max_n1);
  cudaFuncSetAttribute(k_x_inv<R, NX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  derek::note_launch(), k_x_inv<R, NX><<<dim3(nitems, max_nchunk), 256, sm, st>>>(t, item_begin, psi, abuf, occ_skip);
}

// compile-time x length when every item has the same n1 in {32, 36, 48, 54, 64, 72}
template <typename R>
void launch_x_inv(const Tables &t, int item_begin, int nitems, int max_nchunk, int max_n1,
                  int min_n1, int max_m, const cplx<R> *psi, cplx<R> *abuf, const double *occ_skip,
                  cudaStream_t st) {
  if (nitems <= 0) return;
  if constexpr (std::is_same<R, float>::value) {
    if (max_n1 == min_n1 &&
        launch_xinv_reg(t, item_begin, nitems, max_nchunk * kCC, max_n1, max_m, psi, abuf, occ_skip, st))
      return;
  }
  launch_x_inv_lines<R>(t, item_begin, nitems, max_nchunk, max_n1, min_n1, psi, abuf, occ_skip, st);
}

template <typename R>
void launch_x_inv_lines(const Tables &t, int item_begin, int nitems, int max_nchunk, int max_n1,
                        int min_n1, const cplx<R> *psi, cplx<R> *abuf, const double *occ_skip,
                        cudaStream_t st) {
  if (nitems <= 0) return;
  const int n = max_n1 == min_n1 ? max_n1 : 0;
  if (n == 72) x_inv_go<R, 72>(t, item_begin, nitems, max_nchunk, max_n1, psi, abuf, occ_skip, st);
  else if (n == 54) x_inv_go<R, 54>(t, item_begin, nitems, max_nchunk, max_n1, psi, abuf, occ_skip, st);
  else if (n == 36) x_inv_go<R, 36>(t, item_begin, nitems, max_nchunk, max_n1, psi, abuf, occ_skip, st);
  else if (n == 64) x_inv_go<R, 64>(t, item_begin, nitems, max_nchunk, max_n1, psi, abuf, occ_skip, st);
  else if (n == 48) x_inv_go<R, 48>(t, item_begin, nitems, max_nchunk, max_n1, psi, abuf, occ_skip, st);
  else if (n == 32) x_inv_go<R, 32>(t, item_begin, nitems, max_nchunk, max_n1, psi, abuf, occ_skip, st);
  else x_inv_go<R, 0>(t, item_begin, nitems, max_nchunk, max_n1, psi, abuf, occ_skip, st);
}

template <typename R, int NX>
static void x_fwd_go(const Tables &t, int item_begin, int nitems, int max_nchunk, int max_n1,
                     const cplx<R> *abuf, const cplx<R> *psi, const cplx<R> *prev, cplx<R> *out,
                     const Axpby *coef, cudaStream_t st) {
  const size_t sm = smem_x<R>(max_n1);
  cudaFuncSetAttribute(k_x_fwd<R, NX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  derek::note_launch(), k_x_fwd<R, NX><<<dim3(nitems, max_nchunk), 256, sm, st>>>(t, item_begin, abuf, psi, prev, out, coef);
}

template <typename R>
void launch_x_fwd(const Tables &t, int item_begin, int nitems, int max_nchunk, int max_n1,
                  int min_n1, int max_m, const cplx<R> *abuf, const cplx<R> *psi, const cplx<R> *prev,
                  cplx<R> *out, const Axpby *coef, cudaStream_t st) {
  if (nitems <= 0) return;
  if constexpr (std::is_same<R, float>::value) {
    if (max_n1 == min_n1 &&
        launch_xfwd_reg(t, item_begin, nitems, max_nchunk * kCC, max_n1, max_m, abuf, psi, prev, out, coef, st))
      return;
  }
  launch_x_fwd_lines<R>(t, item_begin, nitems, max_nchunk, max_n1, min_n1, abuf, psi, prev, out, coef, st);
}

template <typename R>
void launch_x_fwd_lines(const Tables &t, int item_begin, int nitems, int max_nchunk, int max_n1,
                        int min_n1, const cplx<R> *abuf, const cplx<R> *psi, const cplx<R> *prev,
                        cplx<R> *out, const Axpby *coef, cudaStream_t st) {
  if (nitems <= 0) return;
  const int n = max_n1 == min_n1 ? max_n1 : 0;
  if (n == 72) x_fwd_go<R, 72>(t, item_begin, nitems, max_nchunk, max_n1, abuf, psi, prev, out, coef, st);
  else if (n == 54) x_fwd_go<R, 54>(t, item_begin, nitems, max_nchunk, max_n1, abuf, psi, prev, out, coef, st);
  else if (n == 36) x_fwd_go<R, 36>(t, item_begin, nitems, max_nchunk, max_n1, abuf, psi, prev, out, coef, st);
  else if (n == 64) x_fwd_go<R, 64>(t, item_begin, nitems, max_nchunk, max_n1, abuf, psi, prev, out, coef, st);
  else if (n == 48) x_fwd_go<R, 48>(t, item_begin, nitems, max_nchunk, max_n1, abuf, psi, prev, out, coef, st);
  else if (n == 32) x_fwd_go<R, 32>(t, item_begin, nitems, max_nchunk, max_n1, abuf, psi, prev, out, coef, st);
  else x_fwd_go<R, 0>(t, item_begin, nitems, max_nchunk, max_n1, abuf, psi, prev, out, coef, st);
}

template <typename R, int N>
static bool try_plane_fixed(const Tables &t, int item_begin, int nitems, int max_n1, int max_n2,
                            int max_n3, int min_n2, int min_n3, cplx<R> *abuf, const R *vloc,
                            cudaStream_t st) {
  if (max_n2 != N || max_n3 != N || min_n2 != N || min_n3 != N) return false;
  const size_t sm = ((size_t)N * (N + 1) + N) * sizeof(cplx<R>);
  constexpr int NT = 384;
  cudaFuncSetAttribute(k_plane_fused<R, N, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  derek::note_launch(), k_plane_fused<R, N, NT><<<dim3(nitems, max_n1), NT, sm, st>>>(t, item_begin, abuf, vloc);
  return true;
}

template <typename R>
void launch_plane(const Tables &t, int item_begin, int nitems, int max_n1, int max_n2, int max_n3,
                  int min_n2, int min_n3, int max_m, cplx<R> *abuf, const R *vloc, cudaStream_t st) {
  if (nitems <= 0) return;
  if constexpr (std::is_same<R, float>::value) {
    if (max_n2 == max_n3 && min_n2 == max_n2 && min_n3 == max_n3 &&
        launch_plane_reg(t, item_begin, nitems, max_n1, max_n2, max_m, abuf, vloc, st))
      return;
  }
  if (try_plane_fixed<R, 72>(t, item_begin, nitems, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, vloc, st) ||
      try_plane_fixed<R, 54>(t, item_begin, nitems, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, vloc, st) ||
      try_plane_fixed<R, 36>(t, item_begin, nitems, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, vloc, st) ||
      try_plane_fixed<R, 64>(t, item_begin, nitems, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, vloc, st) ||
      try_plane_fixed<R, 48>(t, item_begin, nitems, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, vloc, st) ||
      try_plane_fixed<R, 32>(t, item_begin, nitems, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, vloc, st))
    return;
  const size_t sm = smem_plane<R>(max_n2, max_n3);
  cudaFuncSetAttribute(k_plane<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  derek::note_launch(), k_plane<R><<<dim3(nitems, max_n1), 512, sm, st>>>(t, item_begin, abuf, vloc);
}


template <typename R, int N>
static bool try_density_fixed(const Tables &t, int ks_begin, int nks, int max_n1, int max_n2,
                              int max_n3, int min_n2, int min_n3, const cplx<R> *abuf,
                              const double *occ, double *partial, const long long *partial_off,
                              cudaStream_t st) {
  if (max_n2 != N || max_n3 != N || min_n2 != N || min_n3 != N) return false;
  constexpr int NT = 384;
  const size_t sm = (size_t)density_acc_count(N * N) * sizeof(double) + ((size_t)N * (N + 1) + N) * sizeof(cplx<R>);
  cudaFuncSetAttribute(k_density_fixed<R, N, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  derek::note_launch(), k_density_fixed<R, N, NT><<<dim3(nks, max_n1), NT, sm, st>>>(t, ks_begin, abuf, occ, partial, partial_off);
  return true;
}

template <typename R>
void launch_density_plane(const Tables &t, int ks_begin, int nks, int max_n1, int max_n2, int max_n3,
                          int min_n2, int min_n3, int max_m, const cplx<R> *abuf, const double *occ,
                          double *partial, const long long *partial_off, cudaStream_t st) {
  if (nks <= 0) return;
  if constexpr (std::is_same<R, float>::value) {
    if (max_n2 == max_n3 && min_n2 == max_n2 && min_n3 == max_n3 &&
        launch_density_reg(t, ks_begin, nks, max_n1, max_n2, max_m, abuf, occ, partial, partial_off, st))
      return;
  }
  if (try_density_fixed<R, 72>(t, ks_begin, nks, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, occ, partial, partial_off, st) ||
      try_density_fixed<R, 54>(t, ks_begin, nks, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, occ, partial, partial_off, st) ||
      try_density_fixed<R, 36>(t, ks_begin, nks, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, occ, partial, partial_off, st) ||
      try_density_fixed<R, 64>(t, ks_begin, nks, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, occ, partial, partial_off, st) ||
      try_density_fixed<R, 48>(t, ks_begin, nks, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, occ, partial, partial_off, st) ||
      try_density_fixed<R, 32>(t, ks_begin, nks, max_n1, max_n2, max_n3, min_n2, min_n3, abuf, occ, partial, partial_off, st))
    return;
  const size_t sm = (size_t)density_acc_count(max_n2 * max_n3) * sizeof(double) + smem_plane<R>(max_n2, max_n3);
  cudaFuncSetAttribute(k_density_plane<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  derek::note_launch(), k_density_plane<R><<<dim3(nks, max_n1), 512, sm, st>>>(t, ks_begin, abuf, occ, partial, partial_off);
}

#define DEREK_INST(R)                                                                             \
  template void launch_x_inv<R>(const Tables &, int, int, int, int, int, int, const cplx<R> *,   \
                                cplx<R> *, const double *, cudaStream_t);                         \
  template void launch_plane<R>(const Tables &, int, int, int, int, int, int, int, int, cplx<R> *, \
                                const R *, cudaStream_t);                                         \
  template void launch_x_fwd<R>(const Tables &, int, int, int, int, int, int, const cplx<R> *,   \
                                const cplx<R> *, const cplx<R> *, cplx<R> *, const Axpby *,      \
                                cudaStream_t);                                                    \
  template void launch_x_inv_lines<R>(const Tables &, int, int, int, int, int, const cplx<R> *,   \
                                      cplx<R> *, const double *, cudaStream_t);                   \
  template void launch_x_fwd_lines<R>(const Tables &, int, int, int, int, int, const cplx<R> *,   \
                                      const cplx<R> *, const cplx<R> *, cplx<R> *, const Axpby *, \
                                      cudaStream_t);                                              \
  template void launch_density_plane<R>(const Tables &, int, int, int, int, int, int, int, int,   \
                                        const cplx<R> *, const double *, double *,                \
                                        const long long *, cudaStream_t);
DEREK_INST(float)
DEREK_INST(double)
#undef DEREK_INST

}  // namespace derek
