// Four-step line DFTs in shared memory, one warp per group of lines.
//
// A line of length N = A * B is transformed as
//   step 1: for each n2 < B:  y[n2][k1] = W_N^{n2 k1} sum_{n1} x[B n1 + n2] W_A^{n1 k1}
//   step 2: for each k1 < A:  X[k1 + A k2] = sum_{n2} y[n2][k1] W_B^{n2 k2}
// (Cooley-Tukey with the twiddle folded into step 1).  Step 1 writes y[n2][k1]
// back into the slots x[B k1 + n2] it read, so it is in place per thread;
// step 2 reads the B values y[.][k1] of one k1 and writes them to the
// natural-order slots k1 + A k2, which only the threads of the same line
// touch.  A warp owns G = floor(32 / max(A, B)) whole lines, so the only
// synchronisation inside a transform is __syncwarp -- no block barrier.
// SIGN = -1 is the forward transform (exponent -i, FFTW_FORWARD), +1 the
// backward one; neither is normalised (Source/fft.f90:204-212).
#pragma once

#include "fft_smem.cuh"

namespace derek {

template <typename R_, int R, int SIGN>
__device__ __forceinline__ void dft_r(cplx<R_> *v) {
  Dft<R_, R, SIGN>::run(v);
}

// Step 1 for one (line, n2): radix-A DFT over n1, twiddle, store in place.
template <typename R_, int SIGN, int A>
__device__ __noinline__ void step1(cplx<R_> *line, int es, int B, int N, int n2,
                                      const cplx<R_> *__restrict__ tw) {
  cplx<R_> v[A];
#pragma unroll
  for (int n1 = 0; n1 < A; ++n1) v[n1] = line[(B * n1 + n2) * es];
  dft_r<R_, A, SIGN>(v);
  int idx = 0;
#pragma unroll
  for (int k1 = 1; k1 < A; ++k1) {
    idx += n2;
    if (idx >= N) idx -= N;
    cplx<R_> w = tw[idx];
    if (SIGN > 0) w.y = -w.y;
    v[k1] = cmul<R_>(v[k1], w);
  }
#pragma unroll
  for (int k1 = 0; k1 < A; ++k1) line[(B * k1 + n2) * es] = v[k1];
}

// Step 2 for one (line, k1): load B values, warp-sync, radix-B DFT, store.
template <typename R_, int SIGN, int B>
__device__ __noinline__ void step2(cplx<R_> *line, int es, int A, int k1, bool active) {
  cplx<R_> v[B];
  if (active) {
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) v[n2] = line[(B * k1 + n2) * es];
  }
  __syncwarp();
  if (active) {
    dft_r<R_, B, SIGN>(v);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) line[(k1 + A * k2) * es] = v[k2];
  }
}

template <typename R_, int SIGN>
__device__ __forceinline__ void step1_dispatch(int A, cplx<R_> *line, int es, int B, int N, int n2,
                                               const cplx<R_> *tw) {
  switch (A) {
    case 1: {
      break;
    }
    case 2: step1<R_, SIGN, 2>(line, es, B, N, n2, tw); break;
    case 3: step1<R_, SIGN, 3>(line, es, B, N, n2, tw); break;
    case 4: step1<R_, SIGN, 4>(line, es, B, N, n2, tw); break;
    case 5: step1<R_, SIGN, 5>(line, es, B, N, n2, tw); break;
    case 6: step1<R_, SIGN, 6>(line, es, B, N, n2, tw); break;
    case 7: step1<R_, SIGN, 7>(line, es, B, N, n2, tw); break;
    case 8: step1<R_, SIGN, 8>(line, es, B, N, n2, tw); break;
    case 9: step1<R_, SIGN, 9>(line, es, B, N, n2, tw); break;
    case 10: step1<R_, SIGN, 10>(line, es, B, N, n2, tw); break;
    case 11: step1<R_, SIGN, 11>(line, es, B, N, n2, tw); break;
    case 12: step1<R_, SIGN, 12>(line, es, B, N, n2, tw); break;
    case 13: step1<R_, SIGN, 13>(line, es, B, N, n2, tw); break;
    case 14: step1<R_, SIGN, 14>(line, es, B, N, n2, tw); break;
    case 15: step1<R_, SIGN, 15>(line, es, B, N, n2, tw); break;
    case 16: step1<R_, SIGN, 16>(line, es, B, N, n2, tw); break;
    default: break;
  }
}

template <typename R_, int SIGN>
__device__ __forceinline__ void step2_dispatch(int B, cplx<R_> *line, int es, int A, int k1,
                                               bool active) {
  switch (B) {
    case 1: __syncwarp(); break;
    case 2: step2<R_, SIGN, 2>(line, es, A, k1, active); break;
    case 3: step2<R_, SIGN, 3>(line, es, A, k1, active); break;
    case 4: step2<R_, SIGN, 4>(line, es, A, k1, active); break;
    case 5: step2<R_, SIGN, 5>(line, es, A, k1, active); break;
    case 6: step2<R_, SIGN, 6>(line, es, A, k1, active); break;
    case 7: step2<R_, SIGN, 7>(line, es, A, k1, active); break;
    case 8: step2<R_, SIGN, 8>(line, es, A, k1, active); break;
    case 9: step2<R_, SIGN, 9>(line, es, A, k1, active); break;
    case 10: step2<R_, SIGN, 10>(line, es, A, k1, active); break;
    case 11: step2<R_, SIGN, 11>(line, es, A, k1, active); break;
    case 12: step2<R_, SIGN, 12>(line, es, A, k1, active); break;
    case 13: step2<R_, SIGN, 13>(line, es, A, k1, active); break;
    case 14: step2<R_, SIGN, 14>(line, es, A, k1, active); break;
    case 15: step2<R_, SIGN, 15>(line, es, A, k1, active); break;
    case 16: step2<R_, SIGN, 16>(line, es, A, k1, active); break;
    default: __syncwarp(); break;
  }
}

// In-place transform of `nlines` lines held in shared memory: line l (or
// lines[l] when a list is given) starts at buf + line * ldist, element i at
// + i * es.  All threads of the block call it; it ends with __syncthreads().
template <typename R_, int SIGN>
__device__ void fft4_lines(cplx<R_> *buf, const LinePlan &p, int nlines, int ldist, int es,
                           const short *lines, const cplx<R_> *__restrict__ tw) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  const int A = p.a, B = p.b, N = p.n, G = p.group;
  const int span = A > B ? A : B;          // lanes per line
  const int g = lane / span;               // line within the warp's group
  const int r = lane - g * span;           // lane within the line
  for (int l0 = warp * G; l0 < nlines; l0 += nwarps * G) {
    const int l = l0 + g;
    const bool live = g < G && l < nlines;
    cplx<R_> *line = buf;
    if (live) line = buf + (long)(lines ? (int)lines[l] : l) * ldist;
    if (live && r < B) step1_dispatch<R_, SIGN>(A, line, es, B, N, r, tw);
    __syncwarp();
    step2_dispatch<R_, SIGN>(B, line, es, A, r, live && r < A);
    __syncwarp();
  }
  __syncthreads();
}

}  // namespace derek

namespace derek {

// ---- compile-time variant: n = A * B, element stride ES and line distance
// LD known at compile time (the (y,z) planes of cubic grids).
constexpr int plan_a(int n) {
  int best = 0, span = 1 << 30, p2 = 0;
  for (int x = 1; x <= 16; ++x) {
    if (n % x) continue;
    const int y = n / x;
    if (y > 16) continue;
    const int s = x > y ? x : y;
    const int q = ((x & (x - 1)) == 0 && x > 1) ? 1 : 0;
    if (s < span || (s == span && q > p2)) {
      best = x;
      span = s;
      p2 = q;
    }
  }
  return best;
}

template <typename R_, int SIGN, int N, int ES, int LD>
__device__ __forceinline__ void fft4_fixed(cplx<R_> *buf, int nlines, const short *lines,
                                           const cplx<R_> *__restrict__ tw) {
  constexpr int A = plan_a(N);
  constexpr int B = N / A;
  constexpr int SPAN = A > B ? A : B;
  constexpr int G = 32 / SPAN;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  const int g = lane / SPAN;
  const int r = lane - g * SPAN;
  for (int l0 = warp * G; l0 < nlines; l0 += nwarps * G) {
    const int l = l0 + g;
    const bool live = g < G && l < nlines;
    cplx<R_> *line = buf + (live ? (lines ? (int)lines[l] : l) * LD : 0);
    if (live && r < B && A > 1) {
      cplx<R_> v[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) v[n1] = line[(B * n1 + r) * ES];
      Dft<R_, A, SIGN>::run(v);
#pragma unroll
      for (int k1 = 1; k1 < A; ++k1) {
        cplx<R_> w = tw[(r * k1) % N];
        if (SIGN > 0) w.y = -w.y;
        v[k1] = cmul<R_>(v[k1], w);
      }
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) line[(B * k1 + r) * ES] = v[k1];
    }
    __syncwarp();
    if (B > 1) {
      cplx<R_> v[B];
      const bool act = live && r < A;
      if (act) {
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) v[n2] = line[(B * r + n2) * ES];
      }
      __syncwarp();
      if (act) {
        Dft<R_, B, SIGN>::run(v);
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) line[(r + A * k2) * ES] = v[k2];
      }
    }
    __syncwarp();
  }
  __syncthreads();
}

}  // namespace derek
