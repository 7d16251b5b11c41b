// Line DFTs held entirely in one thread's registers.
//
// A line of length N = A * B (A, B <= 16) is transformed, for a split with a
// common factor (Cooley-Tukey), as
//   step 1: for each n2 < B:  y[n2][k1] = W_N^{n2 k1} sum_{n1} x[B n1 + n2] W_A^{n1 k1}
//   step 2: for each k1 < A:  X[k1 + A k2] = sum_{n2} y[n2][k1] W_B^{n2 k2}
// with every index a compile-time constant, so the N complex values stay in
// registers and every twiddle is an immediate operand.  Both steps work in
// place on register slots: step 1 writes y[n2][k1] to the slot that held
// x[B k1 + n2], step 2 writes X[k1 + A k2] to the slot that held
// y[k2][k1] (slot B k1 + k2).  So a transform whose input x[j] sits in slot
// s(j) leaves X[m] in slot s(perm(m)), perm(m) = B (m mod A) + m div A.  The
// slot map after L transforms is perm applied L times; callers load and
// store through that compile-time map instead of moving registers.
// When A and B are coprime (72 = 8 x 9, 48 = 3 x 16, 36 = 4 x 9, 24 = 3 x 8)
// the prime-factor mapping (Good-Thomas) is used instead: input x[(B n1 +
// A n2) mod N] and output X[m] with (m mod A, m mod B) = (k1, k2) turn the
// transform into a plain A x B two-dimensional DFT with no twiddles; the
// index maps are again compile-time slot permutations.
// SIGN = -1 is the forward transform (exponent -i), +1 the backward one;
// neither is normalised (Source/fft.f90:204-212).
#pragma once

#include "fft4.cuh"

namespace derek {

template <int V> struct IC {
  static constexpr int value = V;
};

// f(IC<I>), f(IC<I+1>), ..., f(IC<E-1>) with each index a constant expression.
template <int I, int E, typename F> __device__ __forceinline__ void static_for(F &&f) {
  if constexpr (I < E) {
    f(IC<I>{});
    static_for<I + 1, E>(f);
  }
}

// cos and sin of 2 pi m / n at compile time: reduce to the first octant with
// exact integer arithmetic, then Taylor series (|phi| <= pi/4, 13 terms, error
// far below one double ulp of the result).
struct CosSin {
  double c, s;
};
__host__ __device__ constexpr double taylor_sin(double x) {
  double term = x, sum = x;
  for (int k = 1; k < 14; ++k) {
    term *= -x * x / ((2.0 * k) * (2.0 * k + 1.0));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double taylor_cos(double x) {
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 14; ++k) {
    term *= -x * x / ((2.0 * k - 1.0) * (2.0 * k));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr CosSin turn_cs(int m, int n) {
  const double half_pi = 1.57079632679489661923132169163975144;
  m %= n;
  if (m < 0) m += n;
  const int q = (4 * m) / n;      // quadrant
  const int r = 4 * m - q * n;    // angle = q pi/2 + (pi/2) r / n
  double c = 0, s = 0;
  if (2 * r <= n) {
    const double phi = half_pi * (double)r / (double)n;
    c = taylor_cos(phi);
    s = taylor_sin(phi);
  } else {
    const double psi = half_pi * (double)(n - r) / (double)n;
    c = taylor_sin(psi);
    s = taylor_cos(psi);
  }
  for (int i = 0; i < q; ++i) {
    const double tmp = c;
    c = -s;
    s = tmp;
  }
  return CosSin{c, s};
}

constexpr int gcd_int(int a, int b) { return b == 0 ? a : gcd_int(b, a % b); }

// Split N = A * B (A, B <= 16) for the register transforms: a coprime pair
// when one exists (prime-factor algorithm, no twiddles), the smaller larger
// factor first; otherwise the four-step split plan_a (Cooley-Tukey).
constexpr int reg_split_a(int n) {
  int best = 0, span = 1 << 30;
  for (int x = 2; x <= 16; ++x) {
    if (n % x) continue;
    const int y = n / x;
    if (y > 16 || y < 2 || gcd_int(x, y) != 1) continue;
    const int s = x > y ? x : y;
    if (s < span) {
      best = x;
      span = s;
    }
  }
  return best ? best : plan_a(n);
}

template <int N> struct LineSplit {
  static constexpr int A = reg_split_a(N);
  static constexpr int B = N / A;
  static constexpr bool PFA = A > 1 && B > 1 && gcd_int(A, B) == 1;
  static_assert(A >= 1 && A * B == N && A <= 16 && B <= 16, "line length must split into two factors <= 16");
  // input index of (n1, n2) in step 1, and the slot step 2 writes X[k1, k2] to
  __host__ __device__ static constexpr int in_index(int n1, int n2) {
    return PFA ? (B * n1 + A * n2) % N : B * n1 + n2;
  }
};

// Slot (relative to the input slot map) that holds X[m] after a transform.
// Cooley-Tukey: X[k1 + A k2] is written where x[B k1 + k2] was.  Prime
// factor (Good-Thomas): X[m] with k1 = m mod A, k2 = m mod B is written where
// x[(B k1 + A k2) mod N] was.
template <int N> __host__ __device__ constexpr int line_perm(int m) {
  using S = LineSplit<N>;
  return S::PFA ? (S::B * (m % S::A) + S::A * (m % S::B)) % N : S::B * (m % S::A) + m / S::A;
}
// slot holding element j after L transforms
template <int N> __host__ __device__ constexpr int line_slot(int j, int L) {
  for (int i = 0; i < L; ++i) j = line_perm<N>(j);
  return j;
}

// In-place transform of v (input x[j] in slot line_slot(j, L)).
//   Cooley-Tukey: step 1 over n1 of x[B n1 + n2], twiddle W_N^{n2 k1};
//   step 2 over n2 of y[n2][k1] -> X[k1 + A k2].
//   Prime factor (gcd(A, B) = 1): x[(B n1 + A n2) mod N] and
//   X[CRT(k1 mod A, k2 mod B)] make the transform a plain A x B 2D DFT:
//   W_N^{nk} = W_A^{n1 k1} W_B^{n2 k2}, so there are no twiddles.
template <int N, int SIGN, int L>
__device__ __forceinline__ void reg_fft(float2 (&v)[N]) {
  using S = LineSplit<N>;
  constexpr int A = S::A;
  constexpr int B = S::B;
  static_for<0, B>([&](auto n2c) {
    constexpr int n2 = decltype(n2c)::value;
    float2 t[A];
    static_for<0, A>([&](auto n1c) {
      constexpr int n1 = decltype(n1c)::value;
      t[n1] = v[line_slot<N>(S::in_index(n1, n2), L)];
    });
    Dft<float, A, SIGN>::run(t);
    if constexpr (!S::PFA) {
      static_for<1, A>([&](auto k1c) {
        constexpr int k1 = decltype(k1c)::value;
        constexpr int m = (n2 * k1) % N;
        if constexpr (m != 0) {
          constexpr CosSin w = turn_cs(m, N);
          constexpr float wc = (float)w.c;
          constexpr float ws = (float)(SIGN * w.s);
          const float2 a = t[k1];
          t[k1] = make_float2(a.x * wc - a.y * ws, a.x * ws + a.y * wc);
        }
      });
    }
    static_for<0, A>([&](auto k1c) {
      constexpr int k1 = decltype(k1c)::value;
      v[line_slot<N>(S::in_index(k1, n2), L)] = t[k1];
    });
  });
  static_for<0, A>([&](auto k1c) {
    constexpr int k1 = decltype(k1c)::value;
    float2 t[B];
    static_for<0, B>([&](auto n2c) {
      constexpr int n2 = decltype(n2c)::value;
      t[n2] = v[line_slot<N>(S::in_index(k1, n2), L)];
    });
    Dft<float, B, SIGN>::run(t);
    static_for<0, B>([&](auto k2c) {
      constexpr int k2 = decltype(k2c)::value;
      v[line_slot<N>(S::in_index(k1, k2), L)] = t[k2];
    });
  });
}

// Shared-memory layout of the (y,z) planes of the register-line kernels:
// rows of PZ elements (PZ odd, so a warp walking 32 consecutive rows at the
// same z hits distinct banks) and a plane pitch congruent to N mod 16 (a warp
// that straddles two planes at the same y keeps consecutive bank pairs).
template <int N> struct PlaneLayout {
  static constexpr int PZ = N | 1;
  static constexpr int PP0 = N * PZ;
  static constexpr int PP = PP0 + ((N - PP0) % 16 + 16) % 16;
};

}  // namespace derek
