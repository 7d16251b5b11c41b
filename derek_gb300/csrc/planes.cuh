// Shared pieces of the FP32 (y,z)-plane kernels that keep every line
// transform in one thread's registers: the plane row layout, line loads and
// stores, the z pass and column moves of the density pass, launch shapes
// (hpsi_reg.cu: H.psi plane pass; hpsi_density.cu: density pass).
#pragma once
#include "kernels.cuh"
#include "regfft.cuh"

namespace derek {

// Shared-memory layout of one plane (rows my in [-RY, RY]) and of one V(r)
// plane.  The plane pitch PP is congruent to N mod 16 and the V pitch VP to N
// mod 32, so a warp straddling two planes still reads consecutive banks.
// kept(j): line index j (0 <= j < N) has a centred index within [-RY, RY];
// the same bound holds for the z index of every sphere column.
template <int N, int RY> struct RowsLayout {
  static_assert(RY >= 0 && 2 * RY + 1 <= N + 1, "row bound");
  static constexpr int NRW = 2 * RY + 1;
  static constexpr int PZ = N | 1;
  static constexpr int PP0 = NRW * PZ;
  static constexpr int PP = PP0 + ((N - PP0) % 16 + 16) % 16;
  static constexpr int VP = N * N + ((N - N * N) % 32 + 32) % 32;
  // centred index of line index j (0 <= j < N)
  __host__ __device__ static constexpr int my_of(int j) { return j > N / 2 ? j - N : j; }
  __host__ __device__ static constexpr bool kept(int j) { return my_of(j) >= -RY && my_of(j) <= RY; }
  __host__ __device__ static constexpr int row_of(int j) { return my_of(j) + RY; }
};

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void load_line(float2 (&v)[N], const float2 *p, int stride) {
  static_for<0, N>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    v[j] = p[j * stride];
  });
}

// store X[m] (slot line_slot(m, L)) to p[m * stride]
template <int N, int L>
__device__ __forceinline__ void store_line(const float2 (&v)[N], float2 *p, int stride) {
  static_for<0, N>([&](auto mc) {
    constexpr int m = decltype(mc)::value;
    p[m * stride] = v[line_slot<N>(m, L)];
  });
}

// column z of a plane: the kept rows from shared memory, zeros elsewhere
template <int N, int RY>
__device__ __forceinline__ void load_column(float2 (&v)[N], const float2 *col) {
  using Lay = RowsLayout<N, RY>;
  static_for<0, N>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    if constexpr (Lay::kept(j))
      v[j] = col[Lay::row_of(j) * Lay::PZ];
    else
      v[j] = make_float2(0.f, 0.f);
  });
}

// z transforms of the rows holding columns, planes [0, np).  The backward
// transform reads only the z positions a sphere column can occupy (the rest
// of the row is zero); the forward one stores only those positions.
template <int N, int RY, int SIGN>
__device__ __forceinline__ void z_pass(float2 *P, int np, int nrow, const short *__restrict__ rows) {
  using Lay = RowsLayout<N, RY>;
  const int tid = threadIdx.x;
  if (tid < np * nrow) {
    const int p = tid / nrow;
    const int l = tid - p * nrow;
    float2 *line = P + p * Lay::PP + Lay::row_of(rows[l]) * Lay::PZ;
    float2 v[N];
    if (SIGN > 0) {
      static_for<0, N>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        if constexpr (Lay::kept(j))
          v[j] = line[j];
        else
          v[j] = make_float2(0.f, 0.f);
      });
      reg_fft<N, SIGN, 0, Lay>(v);
      store_line<N, 1>(v, line, 1);
    } else {
      load_line<N>(v, line, 1);
      reg_fft<N, SIGN, 0>(v);
      static_for<0, N>([&](auto mc) {
        constexpr int m = decltype(mc)::value;
        if constexpr (Lay::kept(m)) line[m] = v[line_slot<N>(m, 1)];
      });
    }
  }
}

// columns of the item's sphere into (IN) or out of the planes
template <int N, int RY, int XP, int NT, bool IN>
__device__ __forceinline__ void move_columns(float2 *P, float2 *a0, long long ld, int np, int ncol,
                                             const short *__restrict__ cy, const short *__restrict__ cz) {
  using Lay = RowsLayout<N, RY>;
  for (int c = threadIdx.x; c < ncol; c += NT) {
    const int off = Lay::row_of(cy[c]) * Lay::PZ + cz[c];
#pragma unroll
    for (int p = 0; p < XP; ++p) {
      if (p < np) {
        if (IN)
          P[p * Lay::PP + off] = a0[p * ld + c];
        else
          a0[p * ld + c] = P[p * Lay::PP + off];
      }
    }
  }
}

// Row bound of the compact kernels: a fine grid of N points along y holds the
// sphere's |my| <= N / 4 + 1 whenever the grid is about twice the sphere's
// diameter (the density cutoff); other spheres use every row (RY = N / 2).
template <int N> constexpr int compact_ry() { return N / 4 + 1; }
// A tighter bound for the larger grids: a grid chosen as the first {2,3}-smooth
// size above four sphere radii leaves the sphere at |m| <= N / 4 - 2 or so
// (72^3 for |m| <= 16); those spheres prune six more rows of every line.
// Zero where no tight kernels are compiled (N < 48).
template <int N> constexpr int tight_ry() { return N >= 48 ? N / 4 - 2 : 0; }

constexpr int kSmemMax = 227 * 1024;
constexpr int kThreadsMax = 384;

// planes per block: as many as fit the shared memory and kThreadsMax threads
template <int N, int RY, bool DENSITY> struct RowsShape {
  using Lay = RowsLayout<N, RY>;
  static constexpr int PLANE = Lay::PP * 8 + (DENSITY ? N * N * 4 : Lay::VP * 4);
  static constexpr int BY_SMEM = (kSmemMax - 2 * N - 16) / PLANE;
  static constexpr int BY_THREADS = kThreadsMax / N;
  static constexpr int XP0 = BY_SMEM < BY_THREADS ? BY_SMEM : BY_THREADS;
  static constexpr int XP = XP0 < 1 ? 1 : XP0;
  static constexpr int NT = (N * XP + 31) / 32 * 32;
  static constexpr size_t SMEM = (size_t)XP * PLANE + 2 * N + 16;
};

inline int sm_count() {
  static int n = [] {
    int dev = 0, c = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    return c > 0 ? c : 1;
  }();
  return n;
}

}  // namespace derek
