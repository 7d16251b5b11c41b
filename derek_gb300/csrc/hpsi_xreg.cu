// FP32 x passes of H.psi with one thread per sphere column: the column's
// x-line of N points is transformed in registers (regfft.cuh).
//   x_inv: the block's columns are scattered from the sphere into zeroed
//          shared-memory lines (row pitch N | 1, so consecutive columns hit
//          distinct banks), each thread loads its line, transforms it
//          backward and writes it to the x-plane buffer A[band][x][column]:
//          consecutive threads write consecutive columns.
//   x_fwd: each thread reads its column's line from A (coalesced), transforms
//          it forward and stores the line in shared memory; the sphere
//          entries are then gathered in entry order with the kinetic term
//          and the filter epilogue out = alpha H psi + beta psi + gamma prev.
#include "kernels.cuh"
#include "regfft.cuh"

namespace derek {

constexpr int kXCols = 96;   // columns (threads) per block

template <int N>
__global__ void __launch_bounds__(kXCols, 4) k_xinv_reg(Tables t, int item_begin, const float2 *__restrict__ psi,
                                                        float2 *__restrict__ abuf,
                                                        const double *__restrict__ occ_skip) {
  constexpr int PL = N | 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *L = reinterpret_cast<float2 *>(smem_raw);
  const int item = t.item_list ? t.item_list[blockIdx.x] : item_begin + blockIdx.x;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  const int c0 = blockIdx.y * kXCols;
  if (c0 >= K.ncol) return;
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  if (occ_skip && occ_skip[item] == 0.0) return;
  const int b = t.item_band[item];
  const int nc = min(kXCols, K.ncol - c0);
  const int tid = threadIdx.x;
  for (int i = tid; i < nc * PL; i += kXCols) L[i] = make_float2(0.f, 0.f);
  __syncthreads();
  const int *cs = t.col_start + K.col_off;
  const int e0 = cs[c0], e1 = cs[c0 + nc];
  const float2 *src = psi + K.psi_off + (long long)b * K.npw_pad;
  const int *ecol = t.ent_col + K.ent_off;
  const short *eix = t.ent_ix + K.ent_off;
  for (int e = e0 + tid; e < e1; e += kXCols) L[(ecol[e] - c0) * PL + eix[e]] = src[e];
  __syncthreads();
  if (tid < nc) {
    float2 v[N];
    static_for<0, N>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      v[j] = L[tid * PL + j];
    });
    reg_fft<N, +1, 0>(v);
    const long long ld = K.ncol_pad;
    float2 *dst = abuf + K.a_off + (long long)b * N * ld + c0 + tid;
    static_for<0, N>([&](auto mc) {
      constexpr int m = decltype(mc)::value;
      dst[m * ld] = v[line_slot<N>(m, 1)];
    });
  }
}

template <int N>
__global__ void __launch_bounds__(kXCols, 4) k_xfwd_reg(Tables t, int item_begin, const float2 *__restrict__ abuf,
                                                        const float2 *__restrict__ psi,
                                                        const float2 *__restrict__ prev,
                                                        float2 *__restrict__ out,
                                                        const Axpby *__restrict__ coef) {
  constexpr int PL = N | 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *L = reinterpret_cast<float2 *>(smem_raw);
  const int item = t.item_list ? t.item_list[blockIdx.x] : item_begin + blockIdx.x;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  const int c0 = blockIdx.y * kXCols;
  if (c0 >= K.ncol) return;
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int b = t.item_band[item];
  const int nc = min(kXCols, K.ncol - c0);
  const int tid = threadIdx.x;
  if (tid < nc) {
    const long long ld = K.ncol_pad;
    const float2 *src = abuf + K.a_off + (long long)b * N * ld + c0 + tid;
    float2 v[N];
    static_for<0, N>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      v[j] = src[j * ld];
    });
    reg_fft<N, -1, 0>(v);
    static_for<0, N>([&](auto mc) {
      constexpr int m = decltype(mc)::value;
      L[tid * PL + m] = v[line_slot<N>(m, 1)];
    });
  }
  __syncthreads();
  const int *cs = t.col_start + K.col_off;
  const int e0 = cs[c0], e1 = cs[c0 + nc];
  const int *ecol = t.ent_col + K.ent_off;
  const short *eix = t.ent_ix + K.ent_off;
  const float *kin = t.kin32 + K.ent_off;
  const long long off = K.psi_off + (long long)b * K.npw_pad;
  const float inv_n = 1.0f / (float)S.nr;
  float al = 1, be = 0, ga = 0, tk = 1;
  if (coef) {
    al = (float)coef[ksi].alpha;
    be = (float)coef[ksi].beta;
    ga = (float)coef[ksi].gamma;
    tk = (float)coef[ksi].tk;
  }
  if (t.item_shift) be += (float)t.item_shift[item];
  for (int e = e0 + tid; e < e1; e += kXCols) {
    const float2 p = psi[off + e];
    const float2 f = L[(ecol[e] - c0) * PL + eix[e]];
    const float k = tk * kin[e];
    const float hx = f.x * inv_n + k * p.x;
    const float hy = f.y * inv_n + k * p.y;
    float ox = al * hx + be * p.x;
    float oy = al * hy + be * p.y;
    if (prev) {
      const float2 q = prev[off + e];
      ox += ga * q.x;
      oy += ga * q.y;
    }
    out[off + e] = make_float2(ox, oy);
  }
}

template <int N>
static void xinv_go(const Tables &t, int item_begin, int nitems, int max_ncol, const float2 *psi,
                    float2 *abuf, const double *occ_skip, cudaStream_t st) {
  const int nchunk = (max_ncol + kXCols - 1) / kXCols;
  const int sm = kXCols * (N | 1) * (int)sizeof(float2);
  cudaFuncSetAttribute(k_xinv_reg<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  derek::note_launch(), k_xinv_reg<N><<<dim3(nitems, nchunk), kXCols, sm, st>>>(t, item_begin, psi, abuf, occ_skip);
}

template <int N>
static void xfwd_go(const Tables &t, int item_begin, int nitems, int max_ncol, const float2 *abuf,
                    const float2 *psi, const float2 *prev, float2 *out, const Axpby *coef, cudaStream_t st) {
  const int nchunk = (max_ncol + kXCols - 1) / kXCols;
  const int sm = kXCols * (N | 1) * (int)sizeof(float2);
  cudaFuncSetAttribute(k_xfwd_reg<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  derek::note_launch(), k_xfwd_reg<N><<<dim3(nitems, nchunk), kXCols, sm, st>>>(t, item_begin, abuf, psi, prev, out, coef);
}

bool launch_xinv_reg(const Tables &t, int item_begin, int nitems, int max_ncol, int n, const float2 *psi,
                     float2 *abuf, const double *occ_skip, cudaStream_t st) {
  switch (n) {
    case 72: xinv_go<72>(t, item_begin, nitems, max_ncol, psi, abuf, occ_skip, st); return true;
    case 64: xinv_go<64>(t, item_begin, nitems, max_ncol, psi, abuf, occ_skip, st); return true;
    case 54: xinv_go<54>(t, item_begin, nitems, max_ncol, psi, abuf, occ_skip, st); return true;
    case 48: xinv_go<48>(t, item_begin, nitems, max_ncol, psi, abuf, occ_skip, st); return true;
    case 36: xinv_go<36>(t, item_begin, nitems, max_ncol, psi, abuf, occ_skip, st); return true;
    case 32: xinv_go<32>(t, item_begin, nitems, max_ncol, psi, abuf, occ_skip, st); return true;
    case 27: xinv_go<27>(t, item_begin, nitems, max_ncol, psi, abuf, occ_skip, st); return true;
    case 24: xinv_go<24>(t, item_begin, nitems, max_ncol, psi, abuf, occ_skip, st); return true;
    default: return false;
  }
}

bool launch_xfwd_reg(const Tables &t, int item_begin, int nitems, int max_ncol, int n, const float2 *abuf,
                     const float2 *psi, const float2 *prev, float2 *out, const Axpby *coef,
                     cudaStream_t st) {
  switch (n) {
    case 72: xfwd_go<72>(t, item_begin, nitems, max_ncol, abuf, psi, prev, out, coef, st); return true;
    case 64: xfwd_go<64>(t, item_begin, nitems, max_ncol, abuf, psi, prev, out, coef, st); return true;
    case 54: xfwd_go<54>(t, item_begin, nitems, max_ncol, abuf, psi, prev, out, coef, st); return true;
    case 48: xfwd_go<48>(t, item_begin, nitems, max_ncol, abuf, psi, prev, out, coef, st); return true;
    case 36: xfwd_go<36>(t, item_begin, nitems, max_ncol, abuf, psi, prev, out, coef, st); return true;
    case 32: xfwd_go<32>(t, item_begin, nitems, max_ncol, abuf, psi, prev, out, coef, st); return true;
    case 27: xfwd_go<27>(t, item_begin, nitems, max_ncol, abuf, psi, prev, out, coef, st); return true;
    case 24: xfwd_go<24>(t, item_begin, nitems, max_ncol, abuf, psi, prev, out, coef, st); return true;
    default: return false;
  }
}

}  // namespace derek
