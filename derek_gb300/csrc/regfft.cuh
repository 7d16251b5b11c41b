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

// ---- DFTs with compile-time zero inputs -------------------------------------
// DftZ<R_, R, SIGN, M> computes the same DFT as Dft<R_, R, SIGN> when bit j
// of M marks the inputs that may be nonzero and every other input is zero.
// Zero inputs are never read and the arithmetic they would enter is left
// out (IEEE rules keep the compiler from dropping x + 0 or x * 0 on its
// own).  Every output is written.  A full mask runs Dft itself, so dense
// transforms are unchanged.
constexpr unsigned dz_full(int r) { return r >= 32 ? 0xffffffffu : (1u << r) - 1u; }
constexpr bool dz_bit(unsigned m, int i) { return ((m >> i) & 1u) != 0; }
constexpr int dz_popc(unsigned m) {
  int c = 0;
  for (; m; m &= m - 1) ++c;
  return c;
}
constexpr int dz_low(unsigned m) {
  int i = 0;
  while (!((m >> i) & 1u)) ++i;
  return i;
}

template <typename R_, bool A, bool B> __device__ __forceinline__ cplx<R_> zadd(cplx<R_> a, cplx<R_> b) {
  if constexpr (A && B)
    return cadd<R_>(a, b);
  else if constexpr (A)
    return a;
  else if constexpr (B)
    return b;
  else
    return mk<R_>((R_)0, (R_)0);
}
template <typename R_, bool A, bool B> __device__ __forceinline__ cplx<R_> zsub(cplx<R_> a, cplx<R_> b) {
  if constexpr (A && B)
    return csub<R_>(a, b);
  else if constexpr (A)
    return a;
  else if constexpr (B)
    return mk<R_>(-b.x, -b.y);
  else
    return mk<R_>((R_)0, (R_)0);
}

// a * exp(SIGN 2 pi i m / R); the quarter turns are exact moves
template <typename R_, int R, int SIGN, int M0> __device__ __forceinline__ cplx<R_> turn(cplx<R_> a) {
  constexpr int m = ((M0 % R) + R) % R;
  if constexpr (m == 0) {
    return a;
  } else if constexpr (4 * m == R) {
    return mul_si<R_, SIGN>(a);
  } else if constexpr (2 * m == R) {
    return mk<R_>(-a.x, -a.y);
  } else if constexpr (4 * m == 3 * R) {
    return mul_si<R_, -SIGN>(a);
  } else {
    constexpr CosSin w = turn_cs(m, R);
    return cmul<R_>(a, mk<R_>((R_)w.c, (R_)(SIGN * w.s)));
  }
}

template <typename R_, int R, int SIGN, unsigned M> struct DftZPart;

template <typename R_, int R, int SIGN, unsigned M> struct DftZ {
  __device__ __forceinline__ static void run(cplx<R_> *v) {
    if constexpr (M == dz_full(R)) {
      Dft<R_, R, SIGN>::run(v);
    } else if constexpr (M == 0) {
      static_for<0, R>([&](auto kc) { v[decltype(kc)::value] = mk<R_>((R_)0, (R_)0); });
    } else if constexpr (dz_popc(M) == 1) {
      constexpr int J = dz_low(M);   // X_k = x_J W^{J k}
      const cplx<R_> x = v[J];
      static_for<0, R>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        v[k] = turn<R_, R, SIGN, J * k>(x);
      });
    } else {
      DftZPart<R_, R, SIGN, M>::run(v);
    }
  }
};

// two of three inputs (the radix-3 butterfly of Dft<3>)
template <typename R_, int SIGN, unsigned M> struct DftZPart<R_, 3, SIGN, M> {
  __device__ __forceinline__ static void run(cplx<R_> *v) {
    constexpr bool a = dz_bit(M, 0), b = dz_bit(M, 1), c = dz_bit(M, 2);
    const R_ h = (R_)0.86602540378443864676;  // sqrt(3)/2
    const cplx<R_> t1 = zadd<R_, b, c>(v[1], v[2]);
    const cplx<R_> t2 = cscale<R_>(mul_si<R_, SIGN>(zsub<R_, b, c>(v[1], v[2])), h);
    cplx<R_> m;
    if constexpr (a)
      m = mk<R_>(v[0].x - (R_)0.5 * t1.x, v[0].y - (R_)0.5 * t1.y);
    else
      m = mk<R_>((R_)-0.5 * t1.x, (R_)-0.5 * t1.y);
    v[0] = zadd<R_, a, true>(v[0], t1);
    v[1] = cadd<R_>(m, t2);
    v[2] = csub<R_>(m, t2);
  }
};

// two or three of four inputs (Dft<4>)
template <typename R_, int SIGN, unsigned M> struct DftZPart<R_, 4, SIGN, M> {
  __device__ __forceinline__ static void run(cplx<R_> *v) {
    constexpr bool b0 = dz_bit(M, 0), b1 = dz_bit(M, 1), b2 = dz_bit(M, 2), b3 = dz_bit(M, 3);
    constexpr bool e = b0 || b2, o = b1 || b3;
    const cplx<R_> a = zadd<R_, b0, b2>(v[0], v[2]);
    const cplx<R_> b = zsub<R_, b0, b2>(v[0], v[2]);
    const cplx<R_> c = zadd<R_, b1, b3>(v[1], v[3]);
    const cplx<R_> d = mul_si<R_, SIGN>(zsub<R_, b1, b3>(v[1], v[3]));
    v[0] = zadd<R_, e, o>(a, c);
    v[2] = zsub<R_, e, o>(a, c);
    v[1] = zadd<R_, e, o>(b, d);
    v[3] = zsub<R_, e, o>(b, d);
  }
};

// Dft<8>'s even/odd split with the zeros carried into both halves
template <typename R_, int SIGN, unsigned M> struct DftZPart<R_, 8, SIGN, M> {
  __device__ __forceinline__ static void run(cplx<R_> *v) {
    constexpr unsigned me = (M & 1u) | ((M >> 1) & 2u) | ((M >> 2) & 4u) | ((M >> 3) & 8u);
    constexpr unsigned mo = ((M >> 1) & 1u) | ((M >> 2) & 2u) | ((M >> 3) & 4u) | ((M >> 4) & 8u);
    constexpr bool E = me != 0, O = mo != 0;
    cplx<R_> e[4] = {v[0], v[2], v[4], v[6]};
    cplx<R_> o[4] = {v[1], v[3], v[5], v[7]};
    DftZ<R_, 4, SIGN, me>::run(e);
    DftZ<R_, 4, SIGN, mo>::run(o);
    const R_ r = (R_)0.70710678118654752440;
    const cplx<R_> w1 = mk<R_>(r, (R_)SIGN * r);
    const cplx<R_> w3 = mk<R_>(-r, (R_)SIGN * r);
    const cplx<R_> o1 = cmul<R_>(o[1], w1);
    const cplx<R_> o2 = mul_si<R_, SIGN>(o[2]);
    const cplx<R_> o3 = cmul<R_>(o[3], w3);
    v[0] = zadd<R_, E, O>(e[0], o[0]);
    v[4] = zsub<R_, E, O>(e[0], o[0]);
    v[1] = zadd<R_, E, O>(e[1], o1);
    v[5] = zsub<R_, E, O>(e[1], o1);
    v[2] = zadd<R_, E, O>(e[2], o2);
    v[6] = zsub<R_, E, O>(e[2], o2);
    v[3] = zadd<R_, E, O>(e[3], o3);
    v[7] = zsub<R_, E, O>(e[3], o3);
  }
};

// other lengths: the direct sum over the nonzero inputs (prime R) or
// DftGen's split R = P Q with the zero inputs and zero sub-transforms left out
template <typename R_, int R, int SIGN, unsigned M> struct DftZPart {
  static constexpr int P = smallest_factor(R);
  static constexpr int Q = R / P;
  static constexpr unsigned group(int n2) {
    unsigned g = 0;
    for (int n1 = 0; n1 < P; ++n1)
      if (dz_bit(M, Q * n1 + n2)) g |= 1u << n1;
    return g;
  }
  static constexpr unsigned groups() {
    unsigned g = 0;
    for (int n2 = 0; n2 < Q; ++n2)
      if (group(n2)) g |= 1u << n2;
    return g;
  }
  __device__ __forceinline__ static void run(cplx<R_> *v) {
    if constexpr (P == R) {
      cplx<R_> out[R];
      static_for<0, R>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        R_ ax = 0, ay = 0;
        static_for<0, R>([&](auto jc) {
          constexpr int j = decltype(jc)::value;
          if constexpr (dz_bit(M, j)) {
            constexpr int m = (j * k) % R;
            const R_ c = (R_)RadixConst<R>::c(m);
            const R_ s = (R_)(SIGN * RadixConst<R>::s(m));
            ax += v[j].x * c - v[j].y * s;
            ay += v[j].x * s + v[j].y * c;
          }
        });
        out[k] = mk<R_>(ax, ay);
      });
      static_for<0, R>([&](auto kc) { v[decltype(kc)::value] = out[decltype(kc)::value]; });
    } else {
      cplx<R_> y[R];
      static_for<0, Q>([&](auto n2c) {
        constexpr int n2 = decltype(n2c)::value;
        constexpr unsigned G = group(n2);
        cplx<R_> t[P];
        static_for<0, P>([&](auto n1c) {
          constexpr int n1 = decltype(n1c)::value;
          if constexpr (dz_bit(G, n1))
            t[n1] = v[Q * n1 + n2];
          else
            t[n1] = mk<R_>((R_)0, (R_)0);
        });
        DftZ<R_, P, SIGN, G>::run(t);
        static_for<0, P>([&](auto k1c) {
          constexpr int k1 = decltype(k1c)::value;
          constexpr int m = (n2 * k1) % R;
          if constexpr (m == 0 || G == 0) {
            y[n2 * P + k1] = t[k1];
          } else {
            const cplx<R_> w = mk<R_>((R_)RadixConst<R>::c(m), (R_)(SIGN * RadixConst<R>::s(m)));
            y[n2 * P + k1] = cmul<R_>(t[k1], w);
          }
        });
      });
      constexpr unsigned G2 = groups();
      static_for<0, P>([&](auto k1c) {
        constexpr int k1 = decltype(k1c)::value;
        cplx<R_> t[Q];
        static_for<0, Q>([&](auto n2c) {
          constexpr int n2 = decltype(n2c)::value;
          t[n2] = y[n2 * P + k1];
        });
        DftZ<R_, Q, SIGN, G2>::run(t);
        static_for<0, Q>([&](auto k2c) {
          constexpr int k2 = decltype(k2c)::value;
          v[k1 + P * k2] = t[k2];
        });
      });
    }
  }
};

// Which line positions of a register transform's input may be nonzero:
// every one (AllKept), or kept(j) of a layout policy (the row bound of a
// plane, the |mx| bound of an x-line).
struct AllKept {
  __host__ __device__ static constexpr bool kept(int) { return true; }
};

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
// Z::kept(j) false: input x[j] is zero (its slot is not read).  The step-1
// transforms skip those inputs, and a step-1 group with no kept input
// yields zeros that step 2 leaves out in turn.
template <int N, class Z> __host__ __device__ constexpr unsigned step1_mask(int n2) {
  using S = LineSplit<N>;
  unsigned m = 0;
  for (int n1 = 0; n1 < S::A; ++n1)
    if (Z::kept(S::in_index(n1, n2))) m |= 1u << n1;
  return m;
}
template <int N, class Z> __host__ __device__ constexpr unsigned step2_mask() {
  using S = LineSplit<N>;
  unsigned m = 0;
  for (int n2 = 0; n2 < S::B; ++n2)
    if (step1_mask<N, Z>(n2)) m |= 1u << n2;
  return m;
}

template <int N, int SIGN, int L, class Z = AllKept>
__device__ __forceinline__ void reg_fft(float2 (&v)[N]) {
  using S = LineSplit<N>;
  constexpr int A = S::A;
  constexpr int B = S::B;
  static_for<0, B>([&](auto n2c) {
    constexpr int n2 = decltype(n2c)::value;
    constexpr unsigned M1 = step1_mask<N, Z>(n2);
    if constexpr (M1 != 0) {
      float2 t[A];
      static_for<0, A>([&](auto n1c) {
        constexpr int n1 = decltype(n1c)::value;
        if constexpr (dz_bit(M1, n1))
          t[n1] = v[line_slot<N>(S::in_index(n1, n2), L)];
        else
          t[n1] = make_float2(0.f, 0.f);
      });
      DftZ<float, A, SIGN, M1>::run(t);
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
    }
  });
  constexpr unsigned M2 = step2_mask<N, Z>();
  static_for<0, A>([&](auto k1c) {
    constexpr int k1 = decltype(k1c)::value;
    float2 t[B];
    static_for<0, B>([&](auto n2c) {
      constexpr int n2 = decltype(n2c)::value;
      if constexpr (dz_bit(M2, n2))
        t[n2] = v[line_slot<N>(S::in_index(k1, n2), L)];
      else
        t[n2] = make_float2(0.f, 0.f);
    });
    DftZ<float, B, SIGN, M2>::run(t);
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
