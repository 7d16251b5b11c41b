// FP32 (y,z)-plane passes with every line transform held in one thread's
// registers (regfft.cuh).
//
// A block works on XP consecutive x-planes: of one k-set, band after band
// (density), or of a sequence of items (apply H, one block per SM keeping its
// group of x-planes and its V(r) planes).  Each plane sits in shared memory
// as the rows of centred Miller
// index my in [-RY, RY] (row my + RY), PZ elements per row: the rows a
// sphere's columns can occupy.  Every other y row of the plane is zero after
// the backward z transforms and is not needed after the forward y
// transforms, so it is never stored: the y transforms take those inputs as
// compile-time zeros and drop those outputs.  RY = N / 2 keeps every row.
//   z pass:  one thread per (plane, row holding sphere columns): load the
//            row, transform it in registers, store it back.
//   y pass:  one thread per (plane, z): load the column, backward transform,
//            multiply by V(r), forward transform, store it back (apply H), or
//            backward transform and accumulate f |psi(r)|^2 (density).
// Consecutive threads walk consecutive rows (z pass) or consecutive columns
// (y pass), so no shared-memory access has a bank conflict, and a whole line
// costs one load and one store per element.  The V(r) planes of the block
// are copied into shared memory with cp.async while the columns are gathered
// and the z transforms run, and stay there while the system is unchanged.
#include "planes.cuh"

namespace derek {

// ---- H.psi (y,z) pass ----------------------------------------------------------
// Block b keeps x-group g = b mod ng and walks the items r, r + R, ... with
// r = b div ng, R = gridDim.x / ng.  Its V(r) planes stay in shared memory
// while consecutive items belong to the same system.  While the forward z
// transforms of a tile run (most threads idle), the threads without a z line
// load the next tile's columns into registers and, when its k-set differs
// from the one whose offsets their buffer holds, stage its column and row
// offsets (per k-set data: consecutive tiles of a block mostly share one).
struct PlaneTileSm {
  long long a_base;    // offset of (band, x0) in the x-plane buffer
  long long ld;        // x-plane buffer row pitch
  long long vbase;     // offset of plane x0 in V(r)
  int sys, ncol, nrow, np, valid, ks;
};

template <int N, int XP>
__device__ __forceinline__ void plane_tile_describe(const Tables &t, int item_begin, int it, int g,
                                                    PlaneTileSm &m) {
  const int item = t.item_list ? t.item_list[it] : item_begin + it;
  const KSetDev &K = t.ks[t.item_ks[item]];
  const SysDev &S = t.sys[K.sys];
  const int n1 = S.n[0];
  const int x0 = g * XP;
  m.valid = S.active && x0 < n1;
  if (!m.valid) return;
  const int b = t.item_band[item];
  m.sys = K.sys;
  m.ks = t.item_ks[item];
  m.np = min(XP, n1 - x0);
  m.ld = K.ncol_pad;
  m.a_base = K.a_off + ((long long)b * n1 + x0) * K.ncol_pad;
  m.vbase = S.grid_off + (long long)x0 * N * N;
  m.ncol = K.ncol;
  m.nrow = K.nrow;
}

// column offsets (row_of(y) PZ + z) and row offsets (row_of(y) PZ) of item
// it's k-set, by the threads [t0, NT)
template <int N, int RY, int NT>
__device__ __forceinline__ void stage_offsets(const Tables &t, int item_begin, int it, int ncol, int nrow,
                                              short *coff, short *roff, int t0) {
  using Lay = RowsLayout<N, RY>;
  const int tid = threadIdx.x - t0, nthr = NT - t0;
  if (tid < 0) return;
  const int item = t.item_list ? t.item_list[it] : item_begin + it;
  const KSetDev &K = t.ks[t.item_ks[item]];
  const short *cy = t.col_y + K.col_off;
  const short *cz = t.col_z + K.col_off;
  const short *rows = t.rows + K.row_off;
#pragma unroll 4
  for (int c = tid; c < ncol; c += nthr) coff[c] = (short)(Lay::row_of(cy[c]) * Lay::PZ + cz[c]);
  for (int l = tid; l < nrow; l += nthr) roff[l] = (short)(Lay::row_of(rows[l]) * Lay::PZ);
}

// values (columns x planes) per idle thread the persistent plane pass
// prefetches for the next tile
constexpr int kPrefetchValues = 32;

template <int N, int RY, int XP, int NT>
__global__ void __launch_bounds__(NT, 1) k_plane_persist(Tables t, int item_begin, int nitems, int ng,
                                                         float2 *__restrict__ abuf,
                                                         const float *__restrict__ vloc) {
  using Lay = RowsLayout<N, RY>;
  constexpr int PZ = Lay::PZ, PP = Lay::PP, VP = Lay::VP;
  constexpr int MAXC = Lay::NRW * Lay::NRW, MAXR = Lay::NRW;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *P = reinterpret_cast<float2 *>(smem_raw);
  float *Vs = reinterpret_cast<float *>(smem_raw + (((size_t)XP * PP * sizeof(float2) + 15) & ~(size_t)15));
  short *offs = reinterpret_cast<short *>(Vs + XP * VP);   // [2][MAXC + MAXR]
  __shared__ PlaneTileSm meta[2];
  __shared__ int v_sys;      // system whose V(r) planes are in Vs (-1: none)
  __shared__ int offs_ks[2];   // k-set whose offsets each offset buffer holds
  const int tid = threadIdx.x;
  const int g = blockIdx.x % ng;
  const int R = gridDim.x / ng;
  int it = blockIdx.x / ng;
  if (it >= nitems || blockIdx.x >= R * ng) return;   // whole block leaves together
  if (tid == 0) {
    plane_tile_describe<N, XP>(t, item_begin, it, g, meta[0]);
    v_sys = -1;
    offs_ks[0] = meta[0].valid ? meta[0].ks : -1;
    offs_ks[1] = -1;
  }
  __syncthreads();
  if (meta[0].valid)
    stage_offsets<N, RY, NT>(t, item_begin, it, meta[0].ncol, meta[0].nrow, offs, offs + MAXC, 0);
  int cur = 0;
  // columns of the next tile loaded into registers by the threads idle in
  // the forward z transforms: thread tid >= pf_t0 holds columns
  // (tid - pf_t0) + j * (NT - pf_t0), j < kPrefetchCols, for every plane
  constexpr int PFC = kPrefetchValues / XP > 0 ? kPrefetchValues / XP : 1;
  float2 pf[PFC][XP];
  int pf_t0 = -1;   // -1: this tile's columns were not prefetched
  for (; it < nitems; it += R) {
    const int valid = meta[cur].valid;
    const short *coff = offs + cur * (MAXC + MAXR);
    for (int i = tid; i < XP * PP; i += NT) P[i] = make_float2(0.f, 0.f);
    __syncthreads();   // offsets staged, P zero
    if (valid) {
      const int sys = meta[cur].sys, np = meta[cur].np;
      if (sys != v_sys) {   // uniform: new system, stage its V(r) planes
        const float *vsrc = vloc + meta[cur].vbase;
        if (N % 4 == 0 && (reinterpret_cast<uintptr_t>(vsrc) & 15) == 0) {
          constexpr int Q = N * N / 4;
          for (int i = tid; i < np * Q; i += NT) {
            const int p = i / Q, r = i - p * Q;
            cp_async16(Vs + p * VP + 4 * r, vsrc + (long long)p * N * N + 4 * r);
          }
        } else {
          for (int i = tid; i < np * N * N; i += NT) {
            const int p = i / (N * N), r = i - p * (N * N);
            cp_async4(Vs + p * VP + r, vsrc + (long long)p * N * N + r);
          }
        }
        cp_async_commit();
      }
      const int ncol = meta[cur].ncol;
      if (pf_t0 >= 0) {
        if (tid >= pf_t0) {
          const int nthr = NT - pf_t0;
#pragma unroll
          for (int j = 0; j < PFC; ++j) {
            const int c = tid - pf_t0 + j * nthr;
            if (c < ncol) {
              const int off = coff[c];
#pragma unroll
              for (int p = 0; p < XP; ++p)
                if (p < np) P[p * PP + off] = pf[j][p];
            }
          }
        }
      } else {
        float2 *a0 = abuf + meta[cur].a_base;
        const long long ld = meta[cur].ld;
#pragma unroll 4
        for (int c = tid; c < ncol; c += NT) {
          const int off = coff[c];
#pragma unroll
          for (int p = 0; p < XP; ++p)
            if (p < np) P[p * PP + off] = a0[p * ld + c];
        }
      }
    }
    // the prefetched values are consumed: end their live range before the
    // transforms (they are reloaded after the forward z transforms)
#pragma unroll
    for (int j = 0; j < PFC; ++j)
#pragma unroll
      for (int p = 0; p < XP; ++p) pf[j][p] = make_float2(0.f, 0.f);
    __syncthreads();
    int zoff = -1, zthr = 0;
    if (valid) {
      const int nrow = meta[cur].nrow;
      zthr = meta[cur].np * nrow;
      if (tid < zthr) {
        const int p = tid / nrow;
        zoff = p * PP + coff[MAXC + tid - p * nrow];
      }
    }
    if (zoff >= 0) {
      float2 *line = P + zoff;
      float2 v[N];
      static_for<0, N>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        if constexpr (Lay::kept(j))
          v[j] = line[j];
        else
          v[j] = make_float2(0.f, 0.f);
      });
      reg_fft<N, +1, 0, Lay>(v);
      store_line<N, 1>(v, line, 1);
    }
    const int next = it + R;
    if (tid == NT - 1) {
      if (next < nitems)
        plane_tile_describe<N, XP>(t, item_begin, next, g, meta[cur ^ 1]);
      else
        meta[cur ^ 1].valid = 0;
      if (valid) v_sys = meta[cur].sys;
    }
    cp_async_wait_all();
    __syncthreads();
    if (valid && tid < meta[cur].np * N) {
      const int p = tid / N;
      const int z = tid - p * N;
      float2 *col = P + p * PP + z;
      const float *vz = Vs + p * VP + z;
      float2 v[N];
      load_column<N, RY>(v, col);
      reg_fft<N, +1, 0, Lay>(v);
      static_for<0, N>([&](auto mc) {
        constexpr int mm = decltype(mc)::value;
        const float w = vz[mm * N];
        float2 &e = v[line_slot<N>(mm, 1)];
        e.x *= w;
        e.y *= w;
      });
      reg_fft<N, -1, 1>(v);
      static_for<0, N>([&](auto mc) {
        constexpr int mm = decltype(mc)::value;
        if constexpr (Lay::kept(mm)) col[Lay::row_of(mm) * PZ] = v[line_slot<N>(mm, 2)];
      });
    }
    __syncthreads();   // the next tile's description is visible
    if (zoff >= 0) {
      float2 *line = P + zoff;
      float2 v[N];
      load_line<N>(v, line, 1);
      reg_fft<N, -1, 0>(v);
      static_for<0, N>([&](auto mc) {
        constexpr int mm = decltype(mc)::value;
        if constexpr (Lay::kept(mm)) line[mm] = v[line_slot<N>(mm, 1)];
      });
    }
    // the next tile's columns into registers (threads past the z lines, when
    // they can hold all of them)
    pf_t0 = -1;
    {
      const int t0 = zthr < NT - 32 ? (zthr + 31) / 32 * 32 : 0;
      if (t0 > 0 && meta[cur ^ 1].valid && meta[cur ^ 1].ncol <= PFC * (NT - t0)) {
        pf_t0 = t0;
        if (tid >= t0) {
          const int nthr = NT - t0;
          const float2 *a0n = abuf + meta[cur ^ 1].a_base;
          const long long ldn = meta[cur ^ 1].ld;
          const int ncn = meta[cur ^ 1].ncol, npn = meta[cur ^ 1].np;
#pragma unroll
          for (int j = 0; j < PFC; ++j) {
            const int c = tid - t0 + j * nthr;
#pragma unroll
            for (int p = 0; p < XP; ++p)
              pf[j][p] = (c < ncn && p < npn) ? a0n[p * ldn + c] : make_float2(0.f, 0.f);
          }
        }
      }
    }
    // the next tile's offsets, unless its offset buffer already holds its
    // k-set: staged by the threads without a z line (whole warps past the
    // last z line) while the z transforms run, or by every thread after its
    // z line when nearly all threads have one
    const bool restage = meta[cur ^ 1].valid && offs_ks[cur ^ 1] != meta[cur ^ 1].ks;
    if (restage) {
      const int t0 = zthr < NT - 32 ? (zthr + 31) / 32 * 32 : 0;
      if (tid >= t0) {
        short *nco = offs + (cur ^ 1) * (MAXC + MAXR);
        stage_offsets<N, RY, NT>(t, item_begin, next, meta[cur ^ 1].ncol, meta[cur ^ 1].nrow, nco,
                                 nco + MAXC, t0);
      }
    }
    __syncthreads();
    if (tid == 0 && restage) offs_ks[cur ^ 1] = meta[cur ^ 1].ks;
    if (valid) {
      float2 *a0 = abuf + meta[cur].a_base;
      const long long ld = meta[cur].ld;
      const int ncol = meta[cur].ncol, np = meta[cur].np;
#pragma unroll 4
      for (int c = tid; c < ncol; c += NT) {
        const int off = coff[c];
#pragma unroll
        for (int p = 0; p < XP; ++p)
          if (p < np) a0[p * ld + c] = P[p * PP + off];
      }
    }
    __syncthreads();   // every scatter read of P done before the next tile zeroes it
    cur ^= 1;
  }
}

// ---- launch shapes -----------------------------------------------------------
template <int N, int RY>
static void plane_persist_go(const Tables &t, int item_begin, int nitems, int max_n1, float2 *abuf,
                             const float *vloc, cudaStream_t st) {
  using Lay = RowsLayout<N, RY>;
  constexpr size_t OFFS = 2 * (size_t)(Lay::NRW * Lay::NRW + Lay::NRW) * sizeof(short);
  constexpr int PLANE = Lay::PP * 8 + Lay::VP * 4;
  constexpr int BYS = (int)((kSmemMax - 256 - OFFS) / PLANE);
  constexpr int XP0 = BYS < kThreadsMax / N ? BYS : kThreadsMax / N;
  constexpr int XP = XP0 < 1 ? 1 : XP0;
  constexpr int NT = (N * XP + 31) / 32 * 32;
  const size_t smem = (size_t)XP * PLANE + OFFS + 16;
  auto kern = k_plane_persist<N, RY, XP, NT>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int ng = (max_n1 + XP - 1) / XP;
  int R = sm_count() / ng;
  if (R < 1) R = 1;
  if (R > nitems) R = nitems;
  derek::note_launch(), kern<<<ng * R, NT, smem, st>>>(t, item_begin, nitems, ng, abuf, vloc);
}

template <int N>
static void plane_go(const Tables &t, int item_begin, int nitems, int max_n1, int max_m, float2 *abuf,
                     const float *vloc, cudaStream_t st) {
  if constexpr (tight_ry<N>() > 0) {
    if (max_m <= tight_ry<N>()) {
      plane_persist_go<N, tight_ry<N>()>(t, item_begin, nitems, max_n1, abuf, vloc, st);
      return;
    }
  }
  if (max_m <= compact_ry<N>())
    plane_persist_go<N, compact_ry<N>()>(t, item_begin, nitems, max_n1, abuf, vloc, st);
  else
    plane_persist_go<N, N / 2>(t, item_begin, nitems, max_n1, abuf, vloc, st);
}

bool launch_plane_reg(const Tables &t, int item_begin, int nitems, int max_n1, int n, int max_m,
                      float2 *abuf, const float *vloc, cudaStream_t st) {
  switch (n) {
    case 72: plane_go<72>(t, item_begin, nitems, max_n1, max_m, abuf, vloc, st); return true;
    case 64: plane_go<64>(t, item_begin, nitems, max_n1, max_m, abuf, vloc, st); return true;
    case 54: plane_go<54>(t, item_begin, nitems, max_n1, max_m, abuf, vloc, st); return true;
    case 48: plane_go<48>(t, item_begin, nitems, max_n1, max_m, abuf, vloc, st); return true;
    case 36: plane_go<36>(t, item_begin, nitems, max_n1, max_m, abuf, vloc, st); return true;
    case 32: plane_go<32>(t, item_begin, nitems, max_n1, max_m, abuf, vloc, st); return true;
    case 27: plane_go<27>(t, item_begin, nitems, max_n1, max_m, abuf, vloc, st); return true;
    case 24: plane_go<24>(t, item_begin, nitems, max_n1, max_m, abuf, vloc, st); return true;
    default: return false;
  }
}

}  // namespace derek
