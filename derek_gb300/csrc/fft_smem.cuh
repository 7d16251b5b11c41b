// Mixed-radix Stockham DFTs over lines held in shared memory.
//
// A "plane" is a 2D tile in shared memory; its rows or columns are the lines
// transformed.  Each stage of radix R combines R sub-transforms of span Ns:
//   v_r = src[j + r n/R] * w^{(j mod Ns) r n/(Ns R)},  v <- DFT_R(v),
//   dst[(j div Ns) Ns R + (j mod Ns) + r Ns] = v_r
// (autosort Stockham, natural-order output), ping-ponging two buffers.
// SIGN = -1 is the forward transform (FFTW_FORWARD), +1 the backward one.
// Neither is normalised, as the reference's FFTW plans (Source/fft.f90:204-212).
#pragma once

#include "common.cuh"

namespace derek {

// cos/sin(2 pi m / R) for the generic radices, m = 0..R-1.
template <int R> struct RadixConst;
template <> struct RadixConst<5> {
  __device__ __forceinline__ static double c(int m) {
    constexpr double t[5] = {1.0, 0.309016994374947424102, -0.809016994374947424102, -0.809016994374947424102, 0.309016994374947424102};
    return t[m];
  }
  __device__ __forceinline__ static double s(int m) {
    constexpr double t[5] = {0.0, 0.951056516295153572116, 0.587785252292473129169, -0.587785252292473129169, -0.951056516295153572116};
    return t[m];
  }
};
template <> struct RadixConst<6> {
  __device__ __forceinline__ static double c(int m) {
    constexpr double t[6] = {1.0, 0.5, -0.5, -1.0, -0.5, 0.5};
    return t[m];
  }
  __device__ __forceinline__ static double s(int m) {
    constexpr double t[6] = {0.0, 0.866025403784438646764, 0.866025403784438646764, 0.00000000000000000000000000000000000000000041340642196527976473, -0.866025403784438646764, -0.866025403784438646764};
    return t[m];
  }
};
template <> struct RadixConst<7> {
  __device__ __forceinline__ static double c(int m) {
    constexpr double t[7] = {1.0, 0.623489801858733530525, -0.222520933956314404289, -0.900968867902419126236, -0.900968867902419126236, -0.222520933956314404289, 0.623489801858733530525};
    return t[m];
  }
  __device__ __forceinline__ static double s(int m) {
    constexpr double t[7] = {0.0, 0.781831482468029808708, 0.974927912181823607018, 0.433883739117558120476, -0.433883739117558120476, -0.974927912181823607018, -0.781831482468029808708};
    return t[m];
  }
};
template <> struct RadixConst<9> {
  __device__ __forceinline__ static double c(int m) {
    constexpr double t[9] = {1.0, 0.766044443118978035202, 0.173648177666930348852, -0.5, -0.939692620785908384054, -0.939692620785908384054, -0.5, 0.173648177666930348852, 0.766044443118978035202};
    return t[m];
  }
  __device__ __forceinline__ static double s(int m) {
    constexpr double t[9] = {0.0, 0.642787609686539326323, 0.984807753012208059367, 0.866025403784438646764, 0.342020143325668733044, -0.342020143325668733044, -0.866025403784438646764, -0.984807753012208059367, -0.642787609686539326323};
    return t[m];
  }
};
template <> struct RadixConst<10> {
  __device__ __forceinline__ static double c(int m) {
    constexpr double t[10] = {1.0, 0.809016994374947424102, 0.309016994374947424102, -0.309016994374947424102, -0.809016994374947424102, -1.0, -0.809016994374947424102, -0.309016994374947424102, 0.309016994374947424102, 0.809016994374947424102};
    return t[m];
  }
  __device__ __forceinline__ static double s(int m) {
    constexpr double t[10] = {0.0, 0.587785252292473129169, 0.951056516295153572116, 0.951056516295153572116, 0.587785252292473129169, 0.00000000000000000000000000000000000000000041340642196527976473, -0.587785252292473129169, -0.951056516295153572116, -0.951056516295153572116, -0.587785252292473129169};
    return t[m];
  }
};
template <> struct RadixConst<11> {
  __device__ __forceinline__ static double c(int m) {
    constexpr double t[11] = {1.0, 0.841253532831181168862, 0.415415013001886425529, -0.142314838273285140444, -0.654860733945285064057, -0.95949297361449738989, -0.95949297361449738989, -0.654860733945285064057, -0.142314838273285140444, 0.415415013001886425529, 0.841253532831181168862};
    return t[m];
  }
  __device__ __forceinline__ static double s(int m) {
    constexpr double t[11] = {0.0, 0.540640817455597582108, 0.909631995354518371412, 0.989821441880932732376, 0.755749574354258283774, 0.281732556841429697711, -0.281732556841429697711, -0.755749574354258283774, -0.989821441880932732376, -0.909631995354518371412, -0.540640817455597582108};
    return t[m];
  }
};
template <> struct RadixConst<12> {
  __device__ __forceinline__ static double c(int m) {
    constexpr double t[12] = {1.0, 0.866025403784438646764, 0.5, 0.000000000000000000000000000000000000000000206703210982639882365, -0.5, -0.866025403784438646764, -1.0, -0.866025403784438646764, -0.5, 0.0000000000000000000000000000000000000000223387644065498832429, 0.5, 0.866025403784438646764};
    return t[m];
  }
  __device__ __forceinline__ static double s(int m) {
    constexpr double t[12] = {0.0, 0.5, 0.866025403784438646764, 1.0, 0.866025403784438646764, 0.5, 0.00000000000000000000000000000000000000000041340642196527976473, -0.5, -0.866025403784438646764, -1.0, -0.866025403784438646764, -0.5};
    return t[m];
  }
};
template <> struct RadixConst<13> {
  __device__ __forceinline__ static double c(int m) {
    constexpr double t[13] = {1.0, 0.8854560256532098959, 0.568064746731155802512, 0.120536680255323053349, -0.35460488704253562597, -0.748510748171101098635, -0.970941817426052027157, -0.970941817426052027157, -0.748510748171101098635, -0.35460488704253562597, 0.120536680255323053349, 0.568064746731155802512, 0.8854560256532098959};
    return t[m];
  }
  __device__ __forceinline__ static double s(int m) {
    constexpr double t[13] = {0.0, 0.464723172043768545656, 0.82298386589365639458, 0.992708874098053992801, 0.93501624268541482344, 0.663122658240795202377, 0.239315664287557767149, -0.239315664287557767149, -0.663122658240795202377, -0.93501624268541482344, -0.992708874098053992801, -0.82298386589365639458, -0.464723172043768545656};
    return t[m];
  }
};
template <> struct RadixConst<14> {
  __device__ __forceinline__ static double c(int m) {
    constexpr double t[14] = {1.0, 0.900968867902419126236, 0.623489801858733530525, 0.222520933956314404289, -0.222520933956314404289, -0.623489801858733530525, -0.900968867902419126236, -1.0, -0.900968867902419126236, -0.623489801858733530525, -0.222520933956314404289, 0.222520933956314404289, 0.623489801858733530525, 0.900968867902419126236};
    return t[m];
  }
  __device__ __forceinline__ static double s(int m) {
    constexpr double t[14] = {0.0, 0.433883739117558120476, 0.781831482468029808708, 0.974927912181823607018, 0.974927912181823607018, 0.781831482468029808708, 0.433883739117558120476, 0.00000000000000000000000000000000000000000041340642196527976473, -0.433883739117558120476, -0.781831482468029808708, -0.974927912181823607018, -0.974927912181823607018, -0.781831482468029808708, -0.433883739117558120476};
    return t[m];
  }
};
template <> struct RadixConst<15> {
  __device__ __forceinline__ static double c(int m) {
    constexpr double t[15] = {1.0, 0.913545457642600895502, 0.669130606358858213826, 0.309016994374947424102, -0.1045284632676534714, -0.5, -0.809016994374947424102, -0.978147600733805637929, -0.978147600733805637929, -0.809016994374947424102, -0.5, -0.1045284632676534714, 0.309016994374947424102, 0.669130606358858213826, 0.913545457642600895502};
    return t[m];
  }
  __device__ __forceinline__ static double s(int m) {
    constexpr double t[15] = {0.0, 0.406736643075800207754, 0.743144825477394235015, 0.951056516295153572116, 0.994521895368273336923, 0.866025403784438646764, 0.587785252292473129169, 0.207911690817759337102, -0.207911690817759337102, -0.587785252292473129169, -0.866025403784438646764, -0.994521895368273336923, -0.951056516295153572116, -0.743144825477394235015, -0.406736643075800207754};
    return t[m];
  }
};
template <> struct RadixConst<16> {
  __device__ __forceinline__ static double c(int m) {
    constexpr double t[16] = {1.0, 0.923879532511286756128, 0.707106781186547524401, 0.382683432365089771728, 0.000000000000000000000000000000000000000000206703210982639882365, -0.382683432365089771728, -0.707106781186547524401, -0.923879532511286756128, -1.0, -0.923879532511286756128, -0.707106781186547524401, -0.382683432365089771728, 0.0000000000000000000000000000000000000000223387644065498832429, 0.382683432365089771728, 0.707106781186547524401, 0.923879532511286756128};
    return t[m];
  }
  __device__ __forceinline__ static double s(int m) {
    constexpr double t[16] = {0.0, 0.382683432365089771728, 0.707106781186547524401, 0.923879532511286756128, 1.0, 0.923879532511286756128, 0.707106781186547524401, 0.382683432365089771728, 0.00000000000000000000000000000000000000000041340642196527976473, -0.382683432365089771728, -0.707106781186547524401, -0.923879532511286756128, -1.0, -0.923879532511286756128, -0.707106781186547524401, -0.382683432365089771728};
    return t[m];
  }
};

// In-register DFT of length R with exponent sign SIGN.  Prime lengths use the
// direct O(R^2) sum; composite lengths R = P * Q (P the smallest prime
// factor) split Cooley-Tukey style into P-point and Q-point DFTs with
// compile-time twiddles; 2, 3, 4 and 8 are written out below.
constexpr int smallest_factor(int r) {
  for (int p = 2; p * p <= r; ++p)
    if (r % p == 0) return p;
  return r;
}

template <typename R_, int R, int SIGN, bool PRIME = (smallest_factor(R) == R)> struct DftGen;

template <typename R_, int R, int SIGN> struct DftGen<R_, R, SIGN, true> {
  __device__ __forceinline__ static void run(cplx<R_> *v) {
    cplx<R_> out[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
      R_ ax = v[0].x, ay = v[0].y;
#pragma unroll
      for (int j = 1; j < R; ++j) {
        const int m = (j * k) % R;
        const R_ c = (R_)RadixConst<R>::c(m);
        const R_ s = (R_)(SIGN * RadixConst<R>::s(m));
        ax += v[j].x * c - v[j].y * s;
        ay += v[j].x * s + v[j].y * c;
      }
      out[k] = mk<R_>(ax, ay);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = out[k];
  }
};

template <typename R_, int R, int SIGN> struct Dft;

template <typename R_, int R, int SIGN> struct DftGen<R_, R, SIGN, false> {
  static constexpr int P = smallest_factor(R);
  static constexpr int Q = R / P;
  __device__ __forceinline__ static void run(cplx<R_> *v) {
    // y[n2][k1] = W_R^{n2 k1} sum_{n1} x[Q n1 + n2] W_P^{n1 k1}
    cplx<R_> y[R];
#pragma unroll
    for (int n2 = 0; n2 < Q; ++n2) {
      cplx<R_> t[P];
#pragma unroll
      for (int n1 = 0; n1 < P; ++n1) t[n1] = v[Q * n1 + n2];
      Dft<R_, P, SIGN>::run(t);
#pragma unroll
      for (int k1 = 0; k1 < P; ++k1) {
        const int m = (n2 * k1) % R;
        if (m == 0) {
          y[n2 * P + k1] = t[k1];
        } else {
          const cplx<R_> w = mk<R_>((R_)RadixConst<R>::c(m), (R_)(SIGN * RadixConst<R>::s(m)));
          y[n2 * P + k1] = cmul<R_>(t[k1], w);
        }
      }
    }
    // X[k1 + P k2] = sum_{n2} y[n2][k1] W_Q^{n2 k2}
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
      cplx<R_> t[Q];
#pragma unroll
      for (int n2 = 0; n2 < Q; ++n2) t[n2] = y[n2 * P + k1];
      Dft<R_, Q, SIGN>::run(t);
#pragma unroll
      for (int k2 = 0; k2 < Q; ++k2) v[k1 + P * k2] = t[k2];
    }
  }
};

template <typename R_, int R, int SIGN> struct Dft {
  __device__ __forceinline__ static void run(cplx<R_> *v) { DftGen<R_, R, SIGN>::run(v); }
};

template <typename R_, int SIGN> struct Dft<R_, 1, SIGN> {
  __device__ __forceinline__ static void run(cplx<R_> *) {}
};

template <typename R_, int SIGN> struct Dft<R_, 2, SIGN> {
  __device__ __forceinline__ static void run(cplx<R_> *v) {
    cplx<R_> a = v[0], b = v[1];
    v[0] = cadd<R_>(a, b);
    v[1] = csub<R_>(a, b);
  }
};

// multiply by SIGN * i
template <typename R_, int SIGN> __device__ __forceinline__ cplx<R_> mul_si(cplx<R_> a) {
  return SIGN > 0 ? mk<R_>(-a.y, a.x) : mk<R_>(a.y, -a.x);
}

template <typename R_, int SIGN> struct Dft<R_, 3, SIGN> {
  __device__ __forceinline__ static void run(cplx<R_> *v) {
    const R_ h = (R_)0.86602540378443864676;  // sqrt(3)/2
    cplx<R_> t1 = cadd<R_>(v[1], v[2]);
    cplx<R_> t2 = cscale<R_>(mul_si<R_, SIGN>(csub<R_>(v[1], v[2])), h);
    cplx<R_> m = mk<R_>(v[0].x - (R_)0.5 * t1.x, v[0].y - (R_)0.5 * t1.y);
    v[0] = cadd<R_>(v[0], t1);
    v[1] = cadd<R_>(m, t2);
    v[2] = csub<R_>(m, t2);
  }
};

template <typename R_, int SIGN> struct Dft<R_, 4, SIGN> {
  __device__ __forceinline__ static void run(cplx<R_> *v) {
    cplx<R_> a = cadd<R_>(v[0], v[2]);
    cplx<R_> b = csub<R_>(v[0], v[2]);
    cplx<R_> c = cadd<R_>(v[1], v[3]);
    cplx<R_> d = mul_si<R_, SIGN>(csub<R_>(v[1], v[3]));
    v[0] = cadd<R_>(a, c);
    v[2] = csub<R_>(a, c);
    v[1] = cadd<R_>(b, d);
    v[3] = csub<R_>(b, d);
  }
};

template <typename R_, int SIGN> struct Dft<R_, 8, SIGN> {
  __device__ __forceinline__ static void run(cplx<R_> *v) {
    cplx<R_> e[4] = {v[0], v[2], v[4], v[6]};
    cplx<R_> o[4] = {v[1], v[3], v[5], v[7]};
    Dft<R_, 4, SIGN>::run(e);
    Dft<R_, 4, SIGN>::run(o);
    const R_ r = (R_)0.70710678118654752440;
    // w8^k for k = 0..3 with exponent sign SIGN
    cplx<R_> w1 = mk<R_>(r, (R_)SIGN * r);
    cplx<R_> w3 = mk<R_>(-r, (R_)SIGN * r);
    cplx<R_> o1 = cmul<R_>(o[1], w1);
    cplx<R_> o2 = mul_si<R_, SIGN>(o[2]);
    cplx<R_> o3 = cmul<R_>(o[3], w3);
    v[0] = cadd<R_>(e[0], o[0]);
    v[4] = csub<R_>(e[0], o[0]);
    v[1] = cadd<R_>(e[1], o1);
    v[5] = csub<R_>(e[1], o1);
    v[2] = cadd<R_>(e[2], o2);
    v[6] = csub<R_>(e[2], o2);
    v[3] = cadd<R_>(e[3], o3);
    v[7] = csub<R_>(e[3], o3);
  }
};

// One Stockham stage of radix R over a set of lines.
//   element (line, i) at buf[line * ldist + i * istride]
//   LINES_FAST: consecutive threads walk consecutive lines (column transforms,
//   where lines are adjacent in memory); otherwise they walk along a line.
//   rows: optional list mapping line slot -> line index (pruned transforms).
template <typename R_, int R, int SIGN, bool LINES_FAST>
__device__ __forceinline__ void stockham_stage(const cplx<R_> *__restrict__ src,
                                               cplx<R_> *__restrict__ dst, int n, int Ns,
                                               int nlines, int ldist, int istride,
                                               const cplx<R_> *__restrict__ tw,
                                               const short *__restrict__ rows) {
  const int nq = n / R;
  const int total = nlines * nq;
  const int twstep = n / (Ns * R);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int slot, j;
    if (LINES_FAST) {
      slot = t % nlines;
      j = t / nlines;
    } else {
      slot = t / nq;
      j = t - slot * nq;
    }
    const int line = rows ? (int)rows[slot] : slot;
    const cplx<R_> *s = src + (long)line * ldist;
    cplx<R_> *d = dst + (long)line * ldist;
    cplx<R_> v[R];
    const int jm = j % Ns;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      cplx<R_> x = s[(j + r * nq) * istride];
      if (r > 0 && jm != 0) {
        cplx<R_> w = tw[jm * r * twstep];
        if (SIGN > 0) w.y = -w.y;
        x = cmul<R_>(x, w);
      }
      v[r] = x;
    }
    Dft<R_, R, SIGN>::run(v);
    const int base = (j / Ns) * Ns * R + jm;
#pragma unroll
    for (int r = 0; r < R; ++r) d[(base + r * Ns) * istride] = v[r];
  }
}

// Full 1D transform of `nlines` lines.  Data starts in `a`; `b` is scratch of
// the same layout.  Returns the buffer that holds the result.  All threads of
// the block must call it; it ends with a __syncthreads().
template <typename R_, int SIGN, bool LINES_FAST>
__device__ cplx<R_> *fft_lines(cplx<R_> *a, cplx<R_> *b, const FftPlan &p, int nlines,
                               int ldist, int istride, const cplx<R_> *tw,
                               const short *rows) {
  int Ns = 1;
  cplx<R_> *src = a, *dst = b;
  for (int s = 0; s < p.nstages; ++s) {
    const int R = p.radix[s];
    switch (R) {
      case 2: stockham_stage<R_, 2, SIGN, LINES_FAST>(src, dst, p.n, Ns, nlines, ldist, istride, tw, rows); break;
      case 3: stockham_stage<R_, 3, SIGN, LINES_FAST>(src, dst, p.n, Ns, nlines, ldist, istride, tw, rows); break;
      case 4: stockham_stage<R_, 4, SIGN, LINES_FAST>(src, dst, p.n, Ns, nlines, ldist, istride, tw, rows); break;
      case 5: stockham_stage<R_, 5, SIGN, LINES_FAST>(src, dst, p.n, Ns, nlines, ldist, istride, tw, rows); break;
      case 7: stockham_stage<R_, 7, SIGN, LINES_FAST>(src, dst, p.n, Ns, nlines, ldist, istride, tw, rows); break;
      case 8: stockham_stage<R_, 8, SIGN, LINES_FAST>(src, dst, p.n, Ns, nlines, ldist, istride, tw, rows); break;
      case 11: stockham_stage<R_, 11, SIGN, LINES_FAST>(src, dst, p.n, Ns, nlines, ldist, istride, tw, rows); break;
      case 13: stockham_stage<R_, 13, SIGN, LINES_FAST>(src, dst, p.n, Ns, nlines, ldist, istride, tw, rows); break;
      default: break;
    }
    __syncthreads();
    Ns *= R;
    cplx<R_> *tmp = src; src = dst; dst = tmp;
  }
  return src;
}

}  // namespace derek
