// FP32 density pass over (y,z) planes with every line transform held in one
// thread's registers (regfft.cuh): per k-set and group of x-planes, band
// after band, the sphere columns go into the planes, the backward z and y
// transforms run, and f_b |psi_b(r)|^2 accumulates per grid point.
#include "planes.cuh"

namespace derek {

// Density of one k-set over XP x-planes: loop over bands, accumulate
// f_b |psi_b(r)|^2 per point in FP32 for up to kFlush bands, then add that
// sum into the FP64 per-k-set partial grid (each point owned by one thread).
constexpr int kFlush = 8;

template <int N, int RY, int XP, int NT>
__global__ void __launch_bounds__(NT, 1) k_density_rows(Tables t, int ks_begin, const float2 *__restrict__ abuf,
                                                        const double *__restrict__ occ,
                                                        double *__restrict__ partial,
                                                        const long long *__restrict__ partial_off) {
  using Lay = RowsLayout<N, RY>;
  constexpr int PZ = Lay::PZ, PP = Lay::PP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *P = reinterpret_cast<float2 *>(smem_raw);
  float *acc = reinterpret_cast<float *>(P + XP * PP);
  short *rows_s = reinterpret_cast<short *>(acc + XP * N * N);
  const int ksi = ks_begin + blockIdx.x;
  const KSetDev &K = t.ks[ksi];
  const SysDev &S = t.sys[K.sys];
  if (!S.active) return;
  const int n1 = S.n[0];
  const int x0 = blockIdx.y * XP;
  if (x0 >= n1) return;
  const int np = min(XP, n1 - x0);
  const int tid = threadIdx.x;
  for (int i = tid; i < np * PP; i += NT) P[i] = make_float2(0.f, 0.f);
  const bool owner = tid < np * N;
  const int p = owner ? tid / N : 0;
  const int z = owner ? tid - p * N : 0;
  float *accz = acc + p * N * N + z;
  if (owner)
    static_for<0, N>([&](auto mc) { accz[decltype(mc)::value * N] = 0.f; });
  double *dst = partial + partial_off[ksi] + (long long)(x0 + p) * N * N + z;
  const int nrow = K.nrow;
  const long long ld = K.ncol_pad;
  const short *cy = t.col_y + K.col_off;
  const short *cz = t.col_z + K.col_off;
  const short *rows = t.rows + K.row_off;
  for (int l = tid; l < nrow; l += NT) rows_s[l] = (short)Lay::row_of(rows[l]);
  int pending = 0;     // bands summed in acc since the last flush
  bool first = true;   // dst not yet written
  for (int b = 0; b < K.nb; ++b) {
    const double w = occ[K.item0 + b];
    if (w == 0.0) continue;
    __syncthreads();   // previous band's column reads done; P's rows are zero again
    float2 *a0 = const_cast<float2 *>(abuf) + K.a_off + ((long long)b * n1 + x0) * ld;
    if (tid == 0 && b + 1 < K.nb) {
      // the next band's x-plane rows (np consecutive rows of ld columns,
      // 128-byte aligned, ld a multiple of 16) into L2 while this band runs
      const float2 *nxt = a0 + (long long)n1 * ld;
      const unsigned bytes = (unsigned)((long long)np * ld * sizeof(float2));
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(nxt), "r"(bytes) : "memory");
    }
    move_columns<N, RY, XP, NT, true>(P, a0, ld, np, K.ncol, cy, cz);
    __syncthreads();
    z_pass<N, RY, +1>(P, np, nrow, rows);
    __syncthreads();
    if (owner) {
      float2 *col = P + p * PP + z;
      float2 v[N];
      load_column<N, RY>(v, col);
      // clear this column's rows for the next band's gather
      for (int l = 0; l < nrow; ++l) col[rows_s[l] * PZ] = make_float2(0.f, 0.f);
      reg_fft<N, +1, 0, Lay>(v);
      const float wf = (float)w;
      static_for<0, N>([&](auto mc) {
        constexpr int m = decltype(mc)::value;
        const float2 e = v[line_slot<N>(m, 1)];
        accz[m * N] += wf * (e.x * e.x + e.y * e.y);
      });
      if (++pending == kFlush) {
        static_for<0, N>([&](auto mc) {
          constexpr int m = decltype(mc)::value;
          const double s = (double)accz[m * N];
          dst[m * N] = first ? s : dst[m * N] + s;
          accz[m * N] = 0.f;
        });
        first = false;
        pending = 0;
      }
    }
  }
  if (owner && (pending || first)) {
    static_for<0, N>([&](auto mc) {
      constexpr int m = decltype(mc)::value;
      const double s = (double)accz[m * N];
      dst[m * N] = first ? s : dst[m * N] + s;
    });
  }
}

template <int N, int RY>
static void density_rows_go(const Tables &t, int ks_begin, int nks, int max_n1, const float2 *abuf,
                            const double *occ, double *partial, const long long *partial_off,
                            cudaStream_t st) {
  using Sh = RowsShape<N, RY, true>;
  auto kern = k_density_rows<N, RY, Sh::XP, Sh::NT>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Sh::SMEM);
  const int ng = (max_n1 + Sh::XP - 1) / Sh::XP;
  derek::note_launch(), kern<<<dim3(nks, ng), Sh::NT, Sh::SMEM, st>>>(t, ks_begin, abuf, occ, partial, partial_off);
}

template <int N>
static void density_go(const Tables &t, int ks_begin, int nks, int max_n1, int max_m, const float2 *abuf,
                       const double *occ, double *partial, const long long *partial_off, cudaStream_t st) {
  if constexpr (tight_ry<N>() > 0) {
    if (max_m <= tight_ry<N>()) {
      density_rows_go<N, tight_ry<N>()>(t, ks_begin, nks, max_n1, abuf, occ, partial, partial_off, st);
      return;
    }
  }
  if (max_m <= compact_ry<N>())
    density_rows_go<N, compact_ry<N>()>(t, ks_begin, nks, max_n1, abuf, occ, partial, partial_off, st);
  else
    density_rows_go<N, N / 2>(t, ks_begin, nks, max_n1, abuf, occ, partial, partial_off, st);
}

bool launch_density_reg(const Tables &t, int ks_begin, int nks, int max_n1, int n, int max_m,
                        const float2 *abuf, const double *occ, double *partial,
                        const long long *partial_off, cudaStream_t st) {
  switch (n) {
    case 72: density_go<72>(t, ks_begin, nks, max_n1, max_m, abuf, occ, partial, partial_off, st); return true;
    case 64: density_go<64>(t, ks_begin, nks, max_n1, max_m, abuf, occ, partial, partial_off, st); return true;
    case 54: density_go<54>(t, ks_begin, nks, max_n1, max_m, abuf, occ, partial, partial_off, st); return true;
    case 48: density_go<48>(t, ks_begin, nks, max_n1, max_m, abuf, occ, partial, partial_off, st); return true;
    case 36: density_go<36>(t, ks_begin, nks, max_n1, max_m, abuf, occ, partial, partial_off, st); return true;
    case 32: density_go<32>(t, ks_begin, nks, max_n1, max_m, abuf, occ, partial, partial_off, st); return true;
    case 27: density_go<27>(t, ks_begin, nks, max_n1, max_m, abuf, occ, partial, partial_off, st); return true;
    case 24: density_go<24>(t, ks_begin, nks, max_n1, max_m, abuf, occ, partial, partial_off, st); return true;
    default: return false;
  }
}

}  // namespace derek
