// FP32 x passes of H.psi with one thread per sphere column: the column's
// x-line of N points is transformed in registers (regfft.cuh).
//
// A column's sphere entries are one contiguous run of increasing Miller x
// (column order, see the per-k-set tables), so a thread knows the entry of
// line position j from the run's first entry, its length and the centred x
// of its first entry (col_x0): entry = first + (mx(j) - x0) when that lies in
// the run.  x_inv loads its column's entries straight into its registers,
// one predicated access per possible line position, with no shared-memory
// staging and no block barrier: a thread keeps tens of independent loads in
// flight.  x_fwd writes its run's transformed values into shared memory and
// the block then walks its contiguous range of entries coalesced.
// Line positions with |mx| > RX hold no entry of any column (host check on
// the largest |Miller index| of the spheres); they are compile-time zeros.
//   x_inv: load the column's entries, backward x transform, write the line
//          to the x-plane buffer A[band][x][column] (consecutive threads,
//          consecutive columns).
//   x_fwd: read the line from A, forward x transform, then per entry the
//          kinetic term and the filter epilogue
//          out = alpha (1/N F[V psi] + tk T psi) + beta psi + gamma prev.
#include "kernels.cuh"
#include "regfft.cuh"

namespace derek {

constexpr int kXThreads = 128;   // columns (threads) per block

template <int N> __host__ __device__ constexpr int mx_of(int j) { return j > N / 2 ? j - N : j; }

// L2 prefetch of [p, p + bytes) on 16-byte boundaries: the start rounded
// down (the buffers start on 256-byte boundaries), the end rounded down so
// the range never passes the end of the run
__device__ __forceinline__ void prefetch_l2(const void *p, int bytes) {
  const unsigned long long a = reinterpret_cast<unsigned long long>(p);
  const unsigned long long lo = a & ~15ull, hi = (a + (unsigned)bytes) & ~15ull;
  if (hi > lo)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo), "r"((unsigned)(hi - lo)) : "memory");
}
template <int N, int RX> __host__ __device__ constexpr bool x_kept(int j) {
  return mx_of<N>(j) >= -RX && mx_of<N>(j) <= RX;
}
// the x-line positions a sphere column can occupy, as a reg_fft input policy
template <int N, int RX> struct XKept {
  __host__ __device__ static constexpr bool kept(int j) { return x_kept<N, RX>(j); }
};

template <int N, int RX>
__global__ void __launch_bounds__(kXThreads, 3) k_xinv_reg(Tables t, int item_begin, const float2 *__restrict__ psi,
                                                           float2 *__restrict__ abuf,
                                                           const double *__restrict__ occ_skip) {
  const int item = t.item_list ? t.item_list[blockIdx.x] : item_begin + blockIdx.x;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  const int c = blockIdx.y * kXThreads + threadIdx.x;
  if (c >= K.ncol) return;   // no barriers below: threads leave independently
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  if (occ_skip && occ_skip[item] == 0.0) return;
  const int b = t.item_band[item];
  const int *cs = t.col_start + K.col_off;
  const int e0 = cs[c], cnt = cs[c + 1] - e0, x0 = t.col_x0[K.col_off + c];
  const float2 *src = psi + K.psi_off + (long long)b * K.npw_pad + e0;
  float2 v[N];
  static_for<0, N>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    v[j] = make_float2(0.f, 0.f);
    if constexpr (x_kept<N, RX>(j)) {
      const int d = mx_of<N>(j) - x0;
      if ((unsigned)d < (unsigned)cnt) v[j] = src[d];
    }
  });
  reg_fft<N, +1, 0, XKept<N, RX>>(v);
  const long long ld = K.ncol_pad;
  float2 *dst = abuf + K.a_off + (long long)b * N * ld + c;
  static_for<0, N>([&](auto mc) {
    constexpr int m = decltype(mc)::value;
    dst[m * ld] = v[line_slot<N>(m, 1)];
  });
}

// x_fwd: the block's 128 columns own one contiguous range [E0, E1) of the
// sphere's entries.  Each thread transforms its column and writes its run's
// values (already scaled by 1/N) into shared memory at their entry offsets;
// after one barrier the block walks [E0, E1) with consecutive threads on
// consecutive entries, so the epilogue's loads of psi, prev and the kinetic
// energies and its store of out are coalesced (a thread's own run would make
// every warp access touch up to 32 cache lines).
template <int N, int RX>
__global__ void __launch_bounds__(kXThreads, 3) k_xfwd_reg(Tables t, int item_begin, const float2 *__restrict__ abuf,
                                                           const float2 *__restrict__ psi,
                                                           const float2 *__restrict__ prev,
                                                           float2 *__restrict__ out,
                                                           const Axpby *__restrict__ coef) {
  extern __shared__ __align__(16) float2 run_vals[];   // kXThreads * (2 RX + 1)
  const int item = t.item_list ? t.item_list[blockIdx.x] : item_begin + blockIdx.x;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  const int c0 = blockIdx.y * kXThreads;
  if (c0 >= K.ncol) return;   // uniform: the whole block leaves
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;      // uniform
  const int b = t.item_band[item];
  const long long ld = K.ncol_pad;
  const int *cs = t.col_start + K.col_off;
  const int cend = min(K.ncol, c0 + kXThreads);
  const int E0 = cs[c0], E1 = cs[cend];
  const long long row = K.psi_off + (long long)b * K.npw_pad;
  const float *kin = t.kin32 + K.ent_off;
  if (threadIdx.x == 0) {
    // the epilogue's ranges into L2 while the x-line loads and the transform run
    prefetch_l2(psi + row + E0, (E1 - E0) * (int)sizeof(float2));
    if (prev) prefetch_l2(prev + row + E0, (E1 - E0) * (int)sizeof(float2));
    prefetch_l2(kin + E0, (E1 - E0) * (int)sizeof(float));
  }
  const int c = c0 + threadIdx.x;
  if (c < cend) {
    const int e0 = cs[c], cnt = cs[c + 1] - e0, x0 = t.col_x0[K.col_off + c];
    const float2 *src = abuf + K.a_off + (long long)b * N * ld + c;
    float2 v[N];
    static_for<0, N>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      v[j] = src[j * ld];
    });
    reg_fft<N, -1, 0>(v);
    const float inv_n = 1.0f / (float)S.nr;
    float2 *dst = run_vals + (e0 - E0);
    static_for<0, N>([&](auto mc) {
      constexpr int m = decltype(mc)::value;
      if constexpr (x_kept<N, RX>(m)) {
        const int d = mx_of<N>(m) - x0;
        if ((unsigned)d < (unsigned)cnt) {
          const float2 f = v[line_slot<N>(m, 1)];
          dst[d] = make_float2(f.x * inv_n, f.y * inv_n);
        }
      }
    });
  }
  float al = 1, be = 0, ga = 0, tk = 1;
  if (coef) {
    al = (float)coef[ksi].alpha;
    be = (float)coef[ksi].beta;
    ga = (float)coef[ksi].gamma;
    tk = (float)coef[ksi].tk;
  }
  if (t.item_shift) be += (float)t.item_shift[item];
  __syncthreads();
  for (int e = E0 + threadIdx.x; e < E1; e += kXThreads) {
    const float2 p = psi[row + e];
    const float2 f = run_vals[e - E0];
    const float k = tk * kin[e];
    const float hx = f.x + k * p.x;
    const float hy = f.y + k * p.y;
    float ox = al * hx + be * p.x;
    float oy = al * hy + be * p.y;
    if (prev) {
      const float2 q = prev[row + e];
      ox += ga * q.x;
      oy += ga * q.y;
    }
    out[row + e] = make_float2(ox, oy);
  }
}

// |Miller x| bounds of the compact and tight kernels (as the planes' row
// bounds; no tight kernels below N = 48)
template <int N> constexpr int compact_rx() { return N / 4 + 1; }
template <int N> constexpr int tight_rx() { return N >= 48 ? N / 4 - 2 : 0; }

template <int N, int RX>
static void xinv_go(const Tables &t, int item_begin, int nitems, int max_ncol, const float2 *psi,
                    float2 *abuf, const double *occ_skip, cudaStream_t st) {
  const int nchunk = (max_ncol + kXThreads - 1) / kXThreads;
  derek::note_launch(), k_xinv_reg<N, RX><<<dim3(nitems, nchunk), kXThreads, 0, st>>>(t, item_begin, psi, abuf, occ_skip);
}

template <int N, int RX>
static void xfwd_go(const Tables &t, int item_begin, int nitems, int max_ncol, const float2 *abuf,
                    const float2 *psi, const float2 *prev, float2 *out, const Axpby *coef, cudaStream_t st) {
  const int nchunk = (max_ncol + kXThreads - 1) / kXThreads;
  // every column of a block holds at most 2 RX + 1 entries (|mx| <= RX)
  const int smem = kXThreads * (2 * RX + 1) * (int)sizeof(float2);
  auto kern = k_xfwd_reg<N, RX>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  derek::note_launch(), kern<<<dim3(nitems, nchunk), kXThreads, smem, st>>>(t, item_begin, abuf, psi, prev, out, coef);
}

template <int N>
static void xinv_n(const Tables &t, int item_begin, int nitems, int max_ncol, int max_m, const float2 *psi,
                   float2 *abuf, const double *occ_skip, cudaStream_t st) {
  if constexpr (tight_rx<N>() > 0) {
    if (max_m <= tight_rx<N>()) {
      xinv_go<N, tight_rx<N>()>(t, item_begin, nitems, max_ncol, psi, abuf, occ_skip, st);
      return;
    }
  }
  if (max_m <= compact_rx<N>())
    xinv_go<N, compact_rx<N>()>(t, item_begin, nitems, max_ncol, psi, abuf, occ_skip, st);
  else
    xinv_go<N, N / 2>(t, item_begin, nitems, max_ncol, psi, abuf, occ_skip, st);
}

template <int N>
static void xfwd_n(const Tables &t, int item_begin, int nitems, int max_ncol, int max_m, const float2 *abuf,
                   const float2 *psi, const float2 *prev, float2 *out, const Axpby *coef, cudaStream_t st) {
  if constexpr (tight_rx<N>() > 0) {
    if (max_m <= tight_rx<N>()) {
      xfwd_go<N, tight_rx<N>()>(t, item_begin, nitems, max_ncol, abuf, psi, prev, out, coef, st);
      return;
    }
  }
  if (max_m <= compact_rx<N>())
    xfwd_go<N, compact_rx<N>()>(t, item_begin, nitems, max_ncol, abuf, psi, prev, out, coef, st);
  else
    xfwd_go<N, N / 2>(t, item_begin, nitems, max_ncol, abuf, psi, prev, out, coef, st);
}

bool launch_xinv_reg(const Tables &t, int item_begin, int nitems, int max_ncol, int n, int max_m,
                     const float2 *psi, float2 *abuf, const double *occ_skip, cudaStream_t st) {
  switch (n) {
    case 72: xinv_n<72>(t, item_begin, nitems, max_ncol, max_m, psi, abuf, occ_skip, st); return true;
    case 64: xinv_n<64>(t, item_begin, nitems, max_ncol, max_m, psi, abuf, occ_skip, st); return true;
    case 54: xinv_n<54>(t, item_begin, nitems, max_ncol, max_m, psi, abuf, occ_skip, st); return true;
    case 48: xinv_n<48>(t, item_begin, nitems, max_ncol, max_m, psi, abuf, occ_skip, st); return true;
    case 36: xinv_n<36>(t, item_begin, nitems, max_ncol, max_m, psi, abuf, occ_skip, st); return true;
    case 32: xinv_n<32>(t, item_begin, nitems, max_ncol, max_m, psi, abuf, occ_skip, st); return true;
    case 27: xinv_n<27>(t, item_begin, nitems, max_ncol, max_m, psi, abuf, occ_skip, st); return true;
    case 24: xinv_n<24>(t, item_begin, nitems, max_ncol, max_m, psi, abuf, occ_skip, st); return true;
    default: return false;
  }
}

bool launch_xfwd_reg(const Tables &t, int item_begin, int nitems, int max_ncol, int n, int max_m,
                     const float2 *abuf, const float2 *psi, const float2 *prev, float2 *out,
                     const Axpby *coef, cudaStream_t st) {
  switch (n) {
    case 72: xfwd_n<72>(t, item_begin, nitems, max_ncol, max_m, abuf, psi, prev, out, coef, st); return true;
    case 64: xfwd_n<64>(t, item_begin, nitems, max_ncol, max_m, abuf, psi, prev, out, coef, st); return true;
    case 54: xfwd_n<54>(t, item_begin, nitems, max_ncol, max_m, abuf, psi, prev, out, coef, st); return true;
    case 48: xfwd_n<48>(t, item_begin, nitems, max_ncol, max_m, abuf, psi, prev, out, coef, st); return true;
    case 36: xfwd_n<36>(t, item_begin, nitems, max_ncol, max_m, abuf, psi, prev, out, coef, st); return true;
    case 32: xfwd_n<32>(t, item_begin, nitems, max_ncol, max_m, abuf, psi, prev, out, coef, st); return true;
    case 27: xfwd_n<27>(t, item_begin, nitems, max_ncol, max_m, abuf, psi, prev, out, coef, st); return true;
    case 24: xfwd_n<24>(t, item_begin, nitems, max_ncol, max_m, abuf, psi, prev, out, coef, st); return true;
    default: return false;
  }
}

}  // namespace derek
