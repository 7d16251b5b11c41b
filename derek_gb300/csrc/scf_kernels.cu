// Grid-level kernels of the SCF iteration: start vectors, Chebyshev filter
// coefficients, Fermi-Dirac occupations, energies, Pulay/Kerker mixing and
// the local potential V_ext + V_H + v_xc.  Every kernel is deterministic:
// reductions use a fixed block count per system and a fixed summation order.
//
// The reference's SCF loop (Source/electronic.f90:86-175) is a stub; the
// formulas here are textbook plane-wave Kohn-Sham DFT in Hartree units:
//   f = 2 / (1 + exp((e - mu)/kT)),  sum_k w_k sum_n f_nk = N_e
//   S = -2 sum_k w_k sum_n [f~ ln f~ + (1-f~) ln(1-f~)],  f~ = f/2
//   n(G) = F[n]/N,  V_H(G) = 4 pi n(G)/|G|^2 (G = 0 dropped),
//   E_H = Omega/2 sum_G 4 pi |n(G)|^2/|G|^2
//   E = E_band - int V_Hxc[n_in] n_out + E_H[n_out] + E_xc[n_out],  F = E - kT S
#include "scf_kernels.cuh"
#include "xc.cuh"

namespace derek {

constexpr int RB = 64;  // reduction blocks per system
constexpr int EP = 8;   // partial slots per block: 0-2 energies, 3 residual, 4 V max

__device__ __forceinline__ double block_sum(double v, double *red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double gsq(const SysDev &S, long long r) {
  const int n1 = S.n[0], n2 = S.n[1], n3 = S.n[2];
  const int iz = (int)(r % n3);
  const int iy = (int)((r / n3) % n2);
  const int ix = (int)(r / ((long long)n2 * n3));
  const double m0 = ix < n1 - n1 / 2 ? ix : ix - n1;
  const double m1 = iy < n2 - n2 / 2 ? iy : iy - n2;
  const double m2 = iz < n3 - n3 / 2 ? iz : iz - n3;
  double g2 = 0.0;
  for (int i = 0; i < 3; ++i) {
    const double g = S.B[3 * i] * m0 + S.B[3 * i + 1] * m1 + S.B[3 * i + 2] * m2;
    g2 += g * g;
  }
  return g2;
}

// ---- start vectors: real r - 0.5 per (band, G) like wave_initialise_wfn
// (Source/wave.f90:873-886), from a splitmix64 counter hash
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ULL;
  unsigned long long z = x;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

template <typename R>
__global__ void k_init_psi(const Tables t, cplx<R> *__restrict__ X, unsigned long long seed,
                           const int *__restrict__ pw_entry) {
  const int item = blockIdx.x;
  const int ksi = t.item_ks[item];
  const KSetDev &K = t.ks[ksi];
  const int b = t.item_band[item];
  const unsigned long long key = (seed * 0x100000001B3ULL) ^ ((unsigned long long)K.sys << 40) ^
                                 ((unsigned long long)K.kidx << 24);
  cplx<R> *dst = X + K.psi_off + (long long)b * K.npw_pad;
  // plane-wave start: one entry 1, the rest a small perturbation
  const int e1 = pw_entry ? pw_entry[item] : -1;
  const double amp = pw_entry ? 1e-3 : 1.0;
  for (int g = threadIdx.x; g < K.npw_pad; g += blockDim.x) {
    R v = 0;
    if (g < K.npw) {
      const unsigned long long h = splitmix64(key + (unsigned long long)b * (1ULL << 20) + g);
      v = (R)(amp * ((double)(h >> 11) * (1.0 / 9007199254740992.0) - 0.5) + (g == e1 ? 1.0 : 0.0));
    }
    dst[g] = mk<R>(v, 0);
  }
}

// ---- Chebyshev filter coefficients (scaled filter of Zhou, Saad, Tiago and
// Chelikowsky, J. Comput. Phys. 219 (2006) 172): damp [a, b], scale at a0.
__global__ void k_filter_coef(const Tables t, int nks, const double *__restrict__ eig,
                              const SysState *__restrict__ st, Axpby *__restrict__ coef, int m) {
  const int ksi = blockIdx.x * blockDim.x + threadIdx.x;
  if (ksi >= nks) return;
  const KSetDev &K = t.ks[ksi];
  const SysDev &S = t.sys[K.sys];
  double a0 = eig[K.item0];
  double a = eig[K.item0 + K.nb - 1];
  const double b = S.ecut + st[K.sys].vmax + 0.01 * fabs(S.ecut);
  if (!(a < b)) a = b - 0.1 * fabs(b - a0) - 1e-3;
  if (!(a0 < a)) a0 = a - 1e-3;
  const double e = 0.5 * (b - a), c = 0.5 * (b + a);
  const double sigma1 = e / (a0 - c);
  double sigma = sigma1;
  coef[ksi] = Axpby{sigma1 / e, -c * sigma1 / e, 0.0, 1.0};
  for (int i = 1; i < m; ++i) {
    const double sn = 1.0 / (2.0 / sigma1 - sigma);
    const double al = 2.0 * sn / e;
    coef[(long long)i * nks + ksi] = Axpby{al, -c * al, -sigma * sn, 1.0};
    sigma = sn;
  }
}

// ---- Fermi-Dirac occupations, one block per system
__global__ void __launch_bounds__(1024) k_occupations(const Tables t, const double *__restrict__ eig,
                                                      double *__restrict__ occ,
                                                      double *__restrict__ occw,
                                                      SysState *__restrict__ st) {
  __shared__ double red[1024];
  __shared__ double s_lo, s_hi, s_mu;
  __shared__ int s_done;
  const int s = blockIdx.x;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  // only the requested bands are occupied; the buffer bands get f = 0.  A
  // scalar band holds up to two electrons, a spinor band one; t is the band
  // view, so band j's eigenvalue is eig[item0 + j] either way
  const int nsp = S.nspinor;
  const double g = nsp == 2 ? 1.0 : 2.0;
  const int nb = S.nbr / nsp, nk = S.nk;
  const int ntot = nb * nk;
  const double kT = S.kT, ne = S.nelec;
  // bracket
  double lo = 1e300, hi = -1e300;
  for (int i = threadIdx.x; i < ntot; i += blockDim.x) {
    const KSetDev &K = t.ks[S.ks0 + i / nb];
    const double e = eig[K.item0 + i % nb];
    lo = fmin(lo, e);
    hi = fmax(hi, e);
  }
  red[threadIdx.x] = lo;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmin(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) s_lo = red[0] - 40.0 * kT - 1.0;
  __syncthreads();
  red[threadIdx.x] = hi;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    s_hi = red[0] + 40.0 * kT + 1.0;
    // from the previous SCF iteration's Fermi level when there is one (the
    // state is reset at SCF start, so every run takes the same path)
    const double prev = st[s].mu;
    s_mu = st[s].iter > 0 && prev > s_lo && prev < s_hi ? prev : 0.5 * (s_lo + s_hi);
    s_done = 0;
  }
  // each thread's eigenvalues and weights in registers (up to kOccReg per
  // thread), read once instead of once per Newton step
  constexpr int kOccReg = 6;
  const bool in_reg = ntot <= kOccReg * (int)blockDim.x;
  // slots of this thread: i = threadIdx.x + q blockDim.x < ntot for q < nq
  const int nq = (int)threadIdx.x < ntot ? (ntot - 1 - (int)threadIdx.x) / (int)blockDim.x + 1 : 0;
  double er[kOccReg], wr[kOccReg];
#pragma unroll
  for (int q = 0; q < kOccReg; ++q) {
    const int i = threadIdx.x + q * (int)blockDim.x;
    er[q] = 0.0;
    wr[q] = 0.0;
    if (in_reg && q < nq) {
      const KSetDev &K = t.ks[S.ks0 + i / nb];
      er[q] = eig[K.item0 + i % nb];
      wr[q] = K.wk * g;
    }
  }
  __syncthreads();
  // safeguarded Newton on N(mu) - Ne
  for (int it = 0; it < 200; ++it) {
    const double mu = s_mu;
    double cnt = 0, der = 0;
    if (in_reg) {
#pragma unroll
      for (int q = 0; q < kOccReg; ++q) {
        if (q < nq) {
          const double x = fmin(fmax((er[q] - mu) / kT, -200.0), 200.0);
          const double f = 1.0 / (1.0 + exp(x));
          cnt += wr[q] * f;
          der += wr[q] * f * (1.0 - f) / kT;
        }
      }
    } else {
      for (int i = threadIdx.x; i < ntot; i += blockDim.x) {
        const KSetDev &K = t.ks[S.ks0 + i / nb];
        const double x = fmin(fmax((eig[K.item0 + i % nb] - mu) / kT, -200.0), 200.0);
        const double f = 1.0 / (1.0 + exp(x));
        cnt += K.wk * g * f;
        der += K.wk * g * f * (1.0 - f) / kT;
      }
    }
    cnt = block_sum(cnt, red);
    der = block_sum(der, red);
    if (threadIdx.x == 0) {
      const double r = cnt - ne;
      if (r < 0)
        s_lo = mu;
      else
        s_hi = mu;
      double nmu = der > 0 ? mu - r / der : 0.5 * (s_lo + s_hi);
      if (!(nmu > s_lo && nmu < s_hi)) nmu = 0.5 * (s_lo + s_hi);
      if (fabs(r) <= 1e-14 * ne || (s_hi - s_lo) <= 1e-15 * fmax(1.0, fabs(mu))) s_done = 1;
      s_mu = s_done ? mu : nmu;
    }
    __syncthreads();
    if (s_done) break;
  }
  const double mu = s_mu;
  // S.nb items per k-set (both components of a spinor band are items)
  for (int i = threadIdx.x; i < nk * S.nb; i += blockDim.x) {
    const KSetDev &K = t.ks[S.ks0 + i / S.nb];
    occ[K.item0 + i % S.nb] = 0.0;
    occw[K.item0 + i % S.nb] = 0.0;
  }
  __syncthreads();
  double ent = 0, eb = 0;
  for (int i = threadIdx.x; i < ntot; i += blockDim.x) {
    const KSetDev &K = t.ks[S.ks0 + i / nb];
    const int j = i % nb;
    const double e = eig[K.item0 + j];
    const double x = fmin(fmax((e - mu) / kT, -200.0), 200.0);
    const double f = 1.0 / (1.0 + exp(x));
    occ[K.item0 + j] = g * f;
    if (nsp == 2) {
      occw[K.item0 + 2 * j] = K.wk * f / S.volume;
      occw[K.item0 + 2 * j + 1] = K.wk * f / S.volume;
    } else {
      occw[K.item0 + j] = K.wk * g * f / S.volume;
    }
    if (f > 0.0 && f < 1.0) ent += K.wk * (f * log(f) + (1.0 - f) * log1p(-f));
    eb += K.wk * g * f * e;
  }
  ent = block_sum(ent, red);
  eb = block_sum(eb, red);
  if (threadIdx.x == 0) {
    st[s].mu = mu;
    st[s].entropy = -g * ent;
    st[s].e_band = eb;
  }
}

// ---- energies of the output density.  cgrid holds F[n_out] (unnormalised).
__global__ void __launch_bounds__(256) k_energy_partials(const Tables t, const double *__restrict__ vhxc,
                                                         const double *__restrict__ rho_in,
                                                         const double *__restrict__ rho_out,
                                                         const double2 *__restrict__ cgrid,
                                                         double *__restrict__ part, const SpinGrids sg) {
  __shared__ double red[256];
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  const long long n = S.nr;
  const long long chunk = (n + RB - 1) / RB;
  const long long r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
  double q0 = 0, q1 = 0, q2 = 0, q3 = 0;
  for (long long r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const double nr = rho_out[S.grid_off + r];
    q3 = fmax(q3, fabs(nr - rho_in[S.grid_off + r]));
    q0 += vhxc[S.grid_off + r] * nr;
    double e, v;
    if (sg.on) {
      // non-collinear: double counting tr(V_Hxc rho_out) = v n + b.m, and
      // E_xc of (n, |m|) as spin densities (n +/- |m|)/2
      const long long i = S.grid_off + r;
      double m2 = 0.0;
      for (int c = 0; c < 3; ++c) {
        const double mo = sg.mag_out[c * sg.tg + i];
        q0 += sg.bxc[c * sg.tg + i] * mo;
        q3 = fmax(q3, fabs(mo - sg.mag_in[c * sg.tg + i]));
        m2 += mo * mo;
      }
      const double am = sqrt(m2);
      double va, vb;
      lsda_point(0.5 * (nr + am), 0.5 * (nr - am), e, va, vb);
    } else {
      lda_point(nr, e, v);
    }
    q1 += nr * e;
    const double g2 = gsq(S, r);
    if (g2 > 0) {
      const double2 c = cgrid[S.grid_off + r];
      q2 += (c.x * c.x + c.y * c.y) / g2;
    }
  }
  q0 = block_sum(q0, red);
  q1 = block_sum(q1, red);
  q2 = block_sum(q2, red);
  red[threadIdx.x] = q3;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double *p = part + ((long long)s * RB + blockIdx.x) * EP;
    p[0] = q0;
    p[1] = q1;
    p[2] = q2;
    p[3] = red[0];
  }
}

__global__ void k_energy_final(const Tables t, int nsys, const double *__restrict__ part,
                               SysState *__restrict__ st, SysDev *__restrict__ sys_rw,
                               const int *__restrict__ ks_status) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  double q0 = 0, q1 = 0, q2 = 0, q3 = 0;
  for (int b = 0; b < RB; ++b) {
    const double *p = part + ((long long)s * RB + b) * EP;
    q0 += p[0];
    q1 += p[1];
    q2 += p[2];
    q3 = fmax(q3, p[3]);
  }
  const double dv = S.volume / S.nr;
  const double four_pi = 12.566370614359172953850573533118;
  SysState &X = st[s];
  X.resid = q3;
  X.e_dc = dv * q0;
  X.e_xc = dv * q1;
  X.e_h = 0.5 * S.volume * four_pi * q2 / ((double)S.nr * (double)S.nr);
  X.energy = X.e_band - X.e_dc + X.e_h + X.e_xc;
  const double F = X.energy - S.kT * X.entropy;
  X.iter += 1;
  X.delta = X.iter > 1 ? fabs(F - X.free) : 1e300;
  X.free_prev = X.free;
  X.free = F;
  int status = 0;
  for (int k = 0; k < S.nk; ++k)
    if (ks_status[S.ks0 + k]) status = ks_status[S.ks0 + k];
  // a k-set's own failure (a wait that timed out, a singular overlap) is
  // the cause of a NaN that follows it, so it is the status reported
  if (!(F == F) && !status) status = DEREK_ERR_NAN;
  X.status = status;
  if (X.iter > 1 && X.delta < X.etol && (X.rtol <= 0.0 || X.resid < X.rtol)) X.converged = 1;
  if (X.converged || status) sys_rw[s].active = 0;
}

// ---- Pulay mixing with optional Kerker preconditioning
__global__ void __launch_bounds__(256) k_mix_store(const Tables t, const double *__restrict__ rho_in,
                                                   const double *__restrict__ rho_out,
                                                   double *__restrict__ nin_hist,
                                                   double *__restrict__ res_hist,
                                                   const long long *__restrict__ hist_off,
                                                   const SysState *__restrict__ st, int H) {
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  const int slot = (st[s].slot + 1) % H;
  double *ni = nin_hist + hist_off[s] + (long long)slot * S.nr;
  double *re = res_hist + hist_off[s] + (long long)slot * S.nr;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < S.nr;
       r += (long long)gridDim.x * blockDim.x) {
    const double a = rho_in[S.grid_off + r];
    ni[r] = a;
    re[r] = rho_out[S.grid_off + r] - a;
  }
}

__global__ void __launch_bounds__(256) k_mix_gram_partials(const Tables t, const double *__restrict__ res_hist,
                                                           const long long *__restrict__ hist_off,
                                                           const SysState *__restrict__ st, int H,
                                                           double *__restrict__ part) {
  __shared__ double red[256];
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  const int slot = (st[s].slot + 1) % H;
  const int m = min(st[s].nhist + 1, H);
  const long long n = S.nr;
  const long long chunk = (n + RB - 1) / RB;
  const long long r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
  const double *rs = res_hist + hist_off[s] + (long long)slot * n;
  for (int j = 0; j < m; ++j) {
    const double *rj = res_hist + hist_off[s] + (long long)j * n;
    double q = 0;
    for (long long r = r0 + threadIdx.x; r < r1; r += blockDim.x) q += rs[r] * rj[r];
    q = block_sum(q, red);
    if (threadIdx.x == 0) part[((long long)s * RB + blockIdx.x) * kMaxHist + j] = q;
  }
}

__global__ void k_mix_solve(const Tables t, int nsys, const double *__restrict__ part,
                            SysState *__restrict__ st, int H) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  SysState &X = st[s];
  const int slot = (X.slot + 1) % H;
  const int m = min(X.nhist + 1, H);
  for (int j = 0; j < m; ++j) {
    double q = 0;
    for (int b = 0; b < RB; ++b) q += part[((long long)s * RB + b) * kMaxHist + j];
    X.gram[slot * kMaxHist + j] = q;
    X.gram[j * kMaxHist + slot] = q;
  }
  X.slot = slot;
  X.nhist = m;
  // [G 1; 1^T 0] [c; lambda] = [0; 1], G scaled by its largest diagonal
  double A[(kMaxHist + 1) * (kMaxHist + 1)];
  double rhs[kMaxHist + 1];
  const int N = m + 1;
  double gmax = 0;
  for (int j = 0; j < m; ++j) gmax = fmax(gmax, X.gram[j * kMaxHist + j]);
  if (!(gmax > 0)) gmax = 1;
  for (int i = 0; i < m; ++i) {
    for (int j = 0; j < m; ++j) A[i * N + j] = X.gram[i * kMaxHist + j] / gmax;
    A[i * N + m] = 1.0;
    A[m * N + i] = 1.0;
    rhs[i] = 0.0;
  }
  A[m * N + m] = 0.0;
  rhs[m] = 1.0;
  bool ok = true;
  for (int c = 0; c < N && ok; ++c) {
    int piv = c;
    for (int r = c + 1; r < N; ++r)
      if (fabs(A[r * N + c]) > fabs(A[piv * N + c])) piv = r;
    if (!(fabs(A[piv * N + c]) > 1e-14)) {
      ok = false;
      break;
    }
    if (piv != c) {
      for (int j = 0; j < N; ++j) {
        const double tmp = A[c * N + j];
        A[c * N + j] = A[piv * N + j];
        A[piv * N + j] = tmp;
      }
      const double tmp = rhs[c];
      rhs[c] = rhs[piv];
      rhs[piv] = tmp;
    }
    for (int r = c + 1; r < N; ++r) {
      const double f = A[r * N + c] / A[c * N + c];
      for (int j = c; j < N; ++j) A[r * N + j] -= f * A[c * N + j];
      rhs[r] -= f * rhs[c];
    }
  }
  double x[kMaxHist + 1];
  if (ok) {
    for (int r = N - 1; r >= 0; --r) {
      double v = rhs[r];
      for (int j = r + 1; j < N; ++j) v -= A[r * N + j] * x[j];
      x[r] = v / A[r * N + r];
    }
  }
  for (int j = 0; j < kMaxHist; ++j) X.coef[j] = 0.0;
  if (ok) {
    for (int j = 0; j < m; ++j) X.coef[j] = x[j];
  } else {
    X.coef[slot] = 1.0;
  }
}

// rho_in <- sum c_j nin_j + (kerker ? 0 : alpha sum c_j R_j); cgrid <- sum c_j R_j
__global__ void __launch_bounds__(256) k_mix_combine(const Tables t, double *__restrict__ rho_in,
                                                     const double *__restrict__ nin_hist,
                                                     const double *__restrict__ res_hist,
                                                     const long long *__restrict__ hist_off,
                                                     const SysState *__restrict__ st,
                                                     double2 *__restrict__ cgrid, double alpha,
                                                     int kerker) {
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  const int m = st[s].nhist;
  double c[kMaxHist];
  for (int j = 0; j < kMaxHist; ++j) c[j] = j < m ? st[s].coef[j] : 0.0;
  const long long n = S.nr;
  const double *ni = nin_hist + hist_off[s];
  const double *re = res_hist + hist_off[s];
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x) {
    double a = 0, b = 0;
    for (int j = 0; j < m; ++j) {
      a += c[j] * ni[(long long)j * n + r];
      b += c[j] * re[(long long)j * n + r];
    }
    if (kerker) {
      rho_in[S.grid_off + r] = a;
      cgrid[S.grid_off + r] = make_double2(b, 0.0);
    } else {
      rho_in[S.grid_off + r] = a + alpha * b;
    }
  }
}

// ---- non-collinear: the magnetisation joins the Pulay vector (n, m).  Its
// history holds 3 x nr values per slot at 3 hist_off[s]; its residual dots
// add to the charge's Gram partials; it combines with the same coefficients
// (no Kerker: that preconditions the charge alone).
__global__ void __launch_bounds__(256) k_mix_store_m(const Tables t, const SpinGrids sg,
                                                     const long long *__restrict__ hist_off,
                                                     const SysState *__restrict__ st, int H) {
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  const int slot = (st[s].slot + 1) % H;
  const long long n = S.nr;
  double *ni = sg.min_hist + 3 * hist_off[s] + (long long)slot * 3 * n;
  double *re = sg.mres_hist + 3 * hist_off[s] + (long long)slot * 3 * n;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < 3 * n;
       r += (long long)gridDim.x * blockDim.x) {
    const long long c = r / n, i = S.grid_off + (r - c * n);
    const double a = sg.mag_in[c * sg.tg + i];
    ni[r] = a;
    re[r] = sg.mag_out[c * sg.tg + i] - a;
  }
}

__global__ void __launch_bounds__(256) k_mix_gram_m(const Tables t, const SpinGrids sg,
                                                    const long long *__restrict__ hist_off,
                                                    const SysState *__restrict__ st, int H,
                                                    double *__restrict__ part) {
  __shared__ double red[256];
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  const int slot = (st[s].slot + 1) % H;
  const int m = min(st[s].nhist + 1, H);
  const long long n = 3 * (long long)S.nr;
  const long long chunk = (n + RB - 1) / RB;
  const long long r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
  const double *rs = sg.mres_hist + 3 * hist_off[s] + (long long)slot * n;
  for (int j = 0; j < m; ++j) {
    const double *rj = sg.mres_hist + 3 * hist_off[s] + (long long)j * n;
    double q = 0;
    for (long long r = r0 + threadIdx.x; r < r1; r += blockDim.x) q += rs[r] * rj[r];
    q = block_sum(q, red);
    if (threadIdx.x == 0) part[((long long)s * RB + blockIdx.x) * kMaxHist + j] += q;
  }
}

__global__ void __launch_bounds__(256) k_mix_combine_m(const Tables t, const SpinGrids sg,
                                                       const long long *__restrict__ hist_off,
                                                       const SysState *__restrict__ st, double alpha) {
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  const int m = st[s].nhist;
  double c[kMaxHist];
  for (int j = 0; j < kMaxHist; ++j) c[j] = j < m ? st[s].coef[j] : 0.0;
  const long long n = 3 * (long long)S.nr;
  const double *ni = sg.min_hist + 3 * hist_off[s];
  const double *re = sg.mres_hist + 3 * hist_off[s];
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x) {
    double a = 0, b = 0;
    for (int j = 0; j < m; ++j) {
      a += c[j] * ni[(long long)j * n + r];
      b += c[j] * re[(long long)j * n + r];
    }
    const long long cc = r / S.nr, i = S.grid_off + (r - cc * S.nr);
    sg.mag_in[cc * sg.tg + i] = a + alpha * b;
  }
}

// cgrid <- alpha G^2/(G^2 + q0^2) cgrid / N (the /N undoes the unnormalised pair)
__global__ void __launch_bounds__(256) k_kerker_scale(const Tables t, double2 *__restrict__ cgrid,
                                                      double alpha, double q0) {
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  const double invn = 1.0 / S.nr;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < S.nr;
       r += (long long)gridDim.x * blockDim.x) {
    const double g2 = gsq(S, r);
    const double f = alpha * g2 / (g2 + q0 * q0) * invn;
    double2 &c = cgrid[S.grid_off + r];
    c.x *= f;
    c.y *= f;
  }
}

__global__ void __launch_bounds__(256) k_add_real(const Tables t, double *__restrict__ rho,
                                                  const double2 *__restrict__ cgrid) {
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!S.active) return;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < S.nr;
       r += (long long)gridDim.x * blockDim.x)
    rho[S.grid_off + r] += cgrid[S.grid_off + r].x;
}

// ---- potential
__global__ void __launch_bounds__(256) k_real_to_complex(const Tables t, const double *__restrict__ a,
                                                         double2 *__restrict__ c, int all) {
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!all && !S.active) return;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < S.nr;
       r += (long long)gridDim.x * blockDim.x)
    c[S.grid_off + r] = make_double2(a[S.grid_off + r], 0.0);
}

__global__ void __launch_bounds__(256) k_hartree_scale(const Tables t, double2 *__restrict__ c, int all) {
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!all && !S.active) return;
  const double four_pi = 12.566370614359172953850573533118;
  const double invn = 1.0 / S.nr;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < S.nr;
       r += (long long)gridDim.x * blockDim.x) {
    const double g2 = gsq(S, r);
    const double f = g2 > 0 ? four_pi / g2 * invn : 0.0;
    double2 &v = c[S.grid_off + r];
    v.x *= f;
    v.y *= f;
  }
}

__global__ void __launch_bounds__(256) k_build_vloc(const Tables t, const double *__restrict__ rho_in,
                                                    const double2 *__restrict__ vh,
                                                    const double *__restrict__ vext,
                                                    double *__restrict__ vhxc,
                                                    double *__restrict__ vloc,
                                                    float *__restrict__ vloc32,
                                                    double *__restrict__ part, int all, const SpinGrids sg) {
  __shared__ double red[256];
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  if (!all && !S.active) return;
  const long long n = S.nr;
  const long long chunk = (n + RB - 1) / RB;
  const long long r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
  double vm = -1e300;
  for (long long r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const long long i = S.grid_off + r;
    double e, v;
    if (sg.on) {
      // non-collinear: V = V_ext + (V_H + (v_up + v_down)/2) I + b.sigma with
      // b = (v_up - v_down)/2 m/|m|, spin densities (n +/- |m|)/2 of n_in, m_in
      const long long tg = sg.tg;
      const double mx = sg.mag_in[i], my = sg.mag_in[tg + i], mz = sg.mag_in[2 * tg + i];
      const double am = sqrt(mx * mx + my * my + mz * mz);
      const double n = rho_in[i];
      double va, vb;
      lsda_point(0.5 * (n + am), 0.5 * (n - am), e, va, vb);
      const double hx = vh[i].x + 0.5 * (va + vb);
      const double sc = am > 0.0 ? 0.5 * (va - vb) / am : 0.0;
      const double bx = sc * mx, by = sc * my, bz = sc * mz;
      sg.bxc[i] = bx;
      sg.bxc[tg + i] = by;
      sg.bxc[2 * tg + i] = bz;
      vhxc[i] = hx;
      const double2 *x = sg.vnc_ext + 4 * i;
      const double2 w[4] = {make_double2(x[0].x + hx + bz, x[0].y), make_double2(x[1].x + bx, x[1].y + by),
                            make_double2(x[2].x + bx, x[2].y - by), make_double2(x[3].x + hx - bz, x[3].y)};
      for (int c = 0; c < 4; ++c) {
        sg.vnc64[4 * i + c] = w[c];
        if (sg.vnc32) sg.vnc32[4 * i + c] = make_float2((float)w[c].x, (float)w[c].y);
      }
      const double vl = 0.5 * (w[0].x + w[3].x);
      vloc[i] = vl;
      if (vloc32) vloc32[i] = (float)vl;
      // filter bound: largest eigenvalue of the Hermitian part of V
      const double ore = 0.5 * (w[2].x + w[1].x), oim = 0.5 * (w[2].y - w[1].y);
      const double hd = 0.5 * (w[0].x - w[3].x);
      vm = fmax(vm, vl + sqrt(hd * hd + ore * ore + oim * oim));
      continue;
    }
    lda_point(rho_in[i], e, v);
    const double hx = vh[i].x + v;
    vhxc[i] = hx;
    const double vl = vext[i] + hx;
    vloc[i] = vl;
    if (vloc32) vloc32[i] = (float)vl;
    vm = fmax(vm, vl);
  }
  red[threadIdx.x] = vm;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[((long long)s * RB + blockIdx.x) * EP + 4] = red[0];
}

__global__ void k_vmax_final(const Tables t, int nsys, const double *__restrict__ part,
                             SysState *__restrict__ st, int all) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  if (!all && !t.sys[s].active) return;
  double vm = -1e300;
  for (int b = 0; b < RB; ++b) vm = fmax(vm, part[((long long)s * RB + b) * EP + 4]);
  st[s].vmax = vm;
}

__global__ void __launch_bounds__(256) k_uniform_density(const Tables t, double *__restrict__ rho) {
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  const double v = S.nelec / S.volume;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < S.nr;
       r += (long long)gridDim.x * blockDim.x)
    rho[S.grid_off + r] = v;
}

// ---------------------------------------------------------------------------
template <typename R>
void launch_init_psi(const Tables &t, int nitems, void *X, unsigned long long seed, const int *pw_entry,
                     cudaStream_t st) {
  derek::note_launch(), k_init_psi<R><<<nitems, 256, 0, st>>>(t, (cplx<R> *)X, seed, pw_entry);
}
template void launch_init_psi<float>(const Tables &, int, void *, unsigned long long, const int *, cudaStream_t);
template void launch_init_psi<double>(const Tables &, int, void *, unsigned long long, const int *, cudaStream_t);

void launch_filter_coef(const Tables &t, int nks, const double *eig, const SysState *st, Axpby *coef,
                        int m, cudaStream_t s) {
  derek::note_launch(), k_filter_coef<<<(nks + 127) / 128, 128, 0, s>>>(t, nks, eig, st, coef, m);
}

void launch_occupations(const Tables &t, int nsys, const double *eig, double *occ, double *occw,
                        SysState *st, cudaStream_t s) {
  derek::note_launch(), k_occupations<<<nsys, 1024, 0, s>>>(t, eig, occ, occw, st);
}

void launch_energies(const Tables &t, int nsys, const double *vhxc, const double *rho_in,
                     const double *rho_out, const double2 *cgrid, double *part, SysState *st,
                     SysDev *sys_rw, const int *ks_status, const SpinGrids &sg, cudaStream_t s) {
  derek::note_launch(), k_energy_partials<<<dim3(RB, nsys), 256, 0, s>>>(t, vhxc, rho_in, rho_out, cgrid, part, sg);
  derek::note_launch(), k_energy_final<<<(nsys + 63) / 64, 64, 0, s>>>(t, nsys, part, st, sys_rw, ks_status);
}

void launch_mix(const Tables &t, int nsys, int max_nr, double *rho_in, const double *rho_out,
                double *nin_hist, double *res_hist, const long long *hist_off, SysState *st, int H,
                double *part, double2 *cgrid, double alpha, double q0, int max_n, const SpinGrids &sg,
                cudaStream_t s) {
  const int gx = (int)std::min<long long>(((long long)max_nr + 255) / 256, 256);
  derek::note_launch(), k_mix_store<<<dim3(gx, nsys), 256, 0, s>>>(t, rho_in, rho_out, nin_hist, res_hist, hist_off, st, H);
  if (sg.on) derek::note_launch(), k_mix_store_m<<<dim3(gx, nsys), 256, 0, s>>>(t, sg, hist_off, st, H);
  derek::note_launch(), k_mix_gram_partials<<<dim3(RB, nsys), 256, 0, s>>>(t, res_hist, hist_off, st, H, part);
  if (sg.on) derek::note_launch(), k_mix_gram_m<<<dim3(RB, nsys), 256, 0, s>>>(t, sg, hist_off, st, H, part);
  derek::note_launch(), k_mix_solve<<<(nsys + 63) / 64, 64, 0, s>>>(t, nsys, part, st, H);
  const int kerker = q0 > 0;
  derek::note_launch(), k_mix_combine<<<dim3(gx, nsys), 256, 0, s>>>(t, rho_in, nin_hist, res_hist, hist_off, st, cgrid,
                                               alpha, kerker);
  if (sg.on) derek::note_launch(), k_mix_combine_m<<<dim3(gx, nsys), 256, 0, s>>>(t, sg, hist_off, st, alpha);
  if (kerker) {
    launch_fft3d_grid(t, 0, nsys, max_n, cgrid, -1, s);
    derek::note_launch(), k_kerker_scale<<<dim3(gx, nsys), 256, 0, s>>>(t, cgrid, alpha, q0);
    launch_fft3d_grid(t, 0, nsys, max_n, cgrid, +1, s);
    derek::note_launch(), k_add_real<<<dim3(gx, nsys), 256, 0, s>>>(t, rho_in, cgrid);
  }
}

void launch_potential(const Tables &t, int nsys, int max_nr, int max_n, const double *rho_in,
                      double2 *cgrid, const double *vext, double *vhxc, double *vloc, float *vloc32,
                      double *part, SysState *st, int all, const SpinGrids &sg, cudaStream_t s) {
  const int gx = (int)std::min<long long>(((long long)max_nr + 255) / 256, 256);
  derek::note_launch(), k_real_to_complex<<<dim3(gx, nsys), 256, 0, s>>>(t, rho_in, cgrid, all);
  launch_fft3d_grid(t, 0, nsys, max_n, cgrid, -1, s);
  derek::note_launch(), k_hartree_scale<<<dim3(gx, nsys), 256, 0, s>>>(t, cgrid, all);
  launch_fft3d_grid(t, 0, nsys, max_n, cgrid, +1, s);
  derek::note_launch(), k_build_vloc<<<dim3(RB, nsys), 256, 0, s>>>(t, rho_in, cgrid, vext, vhxc, vloc, vloc32, part, all, sg);
  derek::note_launch(), k_vmax_final<<<(nsys + 63) / 64, 64, 0, s>>>(t, nsys, part, st, all);
}

__global__ void k_lsda(long n, const double *__restrict__ ra, const double *__restrict__ rb,
                       double *__restrict__ exc, double *__restrict__ va, double *__restrict__ vb) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double e, a, b;
    lsda_point(ra[i], rb[i], e, a, b);
    exc[i] = e;
    va[i] = a;
    vb[i] = b;
  }
}

void launch_lsda(long n, const double *rho_a, const double *rho_b, double *exc, double *va, double *vb,
                 cudaStream_t s) {
  const int blocks = (int)std::min<long>((n + 255) / 256, 152 * 8);
  derek::note_launch(), k_lsda<<<blocks, 256, 0, s>>>(n, rho_a, rho_b, exc, va, vb);
}

void launch_density_fft(const Tables &t, int nsys, int max_nr, int max_n, const double *rho,
                        double2 *cgrid, cudaStream_t s) {
  const int gx = (int)std::min<long long>(((long long)max_nr + 255) / 256, 256);
  derek::note_launch(), k_real_to_complex<<<dim3(gx, nsys), 256, 0, s>>>(t, rho, cgrid, 0);
  launch_fft3d_grid(t, 0, nsys, max_n, cgrid, -1, s);
}

void launch_uniform_density(const Tables &t, int nsys, int max_nr, double *rho, cudaStream_t s) {
  const int gx = (int)std::min<long long>(((long long)max_nr + 255) / 256, 256);
  derek::note_launch(), k_uniform_density<<<dim3(gx, nsys), 256, 0, s>>>(t, rho);
}

}  // namespace derek

namespace derek {

// ---- Hellmann-Feynman gradient of the free energy with respect to the
// Gaussian-well parameters: dF/dp = int n(r) dV_ext/dp dr at self-consistency.
// V_ext = 0.5 Ne / N - sum_w U_w exp(-|r - R_w|^2 / (2 s_w^2)), r sampled at
// frac = (i+1)/n (the reference's real grid, Source/basis.f90:156-188) with
// the minimum-image displacement d = frac - c - rint(frac - c), r = cell d:
//   dV/dU   = -e,   dV/ds = -U e |r|^2 / s^3,
//   dV/dc_a = -U e (r . a_a) / s^2   (a_a = lattice vector a, c fractional).
// Output per well: (dF/dcx, dF/dcy, dF/dcz, dF/dU, dF/ds).
__global__ void __launch_bounds__(256) k_hf_partials(const Tables t, const double *__restrict__ rho,
                                                     const double *__restrict__ wells,
                                                     const int *__restrict__ well_off,
                                                     const double *__restrict__ cells,
                                                     double *__restrict__ part, int max_wells) {
  __shared__ double red[256];
  const int s = blockIdx.y;
  const SysDev &S = t.sys[s];
  const int n1 = S.n[0], n2 = S.n[1], n3 = S.n[2];
  const long long n = S.nr;
  const long long chunk = (n + RB - 1) / RB;
  const long long r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
  const double *cell = cells + 9 * s;  // column-major
  const int w0 = well_off[s], nw = well_off[s + 1] - w0;
  for (int w = 0; w < nw; ++w) {
    const double *p = wells + 5 * (w0 + w);
    const double cx = p[0], cy = p[1], cz = p[2], U = p[3], sw = p[4];
    const double inv2 = 1.0 / (2.0 * sw * sw);
    double q[5] = {0, 0, 0, 0, 0};
    for (long long r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      const int iz = (int)(r % n3), iy = (int)((r / n3) % n2), ix = (int)(r / ((long long)n2 * n3));
      double dx = (double)(ix + 1) / n1 - cx;
      dx -= nearbyint(dx);
      double dy = (double)(iy + 1) / n2 - cy;
      dy -= nearbyint(dy);
      double dz = (double)(iz + 1) / n3 - cz;
      dz -= nearbyint(dz);
      double rv[3], r2 = 0.0;
      for (int i = 0; i < 3; ++i) {
        rv[i] = cell[i] * dx + cell[3 + i] * dy + cell[6 + i] * dz;
        r2 += rv[i] * rv[i];
      }
      const double e = exp(-r2 * inv2);
      const double nr = rho[S.grid_off + r];
      for (int a = 0; a < 3; ++a) {
        const double ra = rv[0] * cell[3 * a] + rv[1] * cell[3 * a + 1] + rv[2] * cell[3 * a + 2];
        q[a] += nr * (-U * e * ra / (sw * sw));
      }
      q[3] += nr * (-e);
      q[4] += nr * (-U * e * r2 / (sw * sw * sw));
    }
    for (int a = 0; a < 5; ++a) {
      const double v = block_sum(q[a], red);
      if (threadIdx.x == 0) part[(((long long)s * RB + blockIdx.x) * max_wells + w) * 5 + a] = v;
    }
  }
}

__global__ void k_hf_final(const Tables t, int nsys, const double *__restrict__ part,
                           const int *__restrict__ well_off, double *__restrict__ grad,
                           int max_wells) {
  const int s = blockIdx.x;
  if (s >= nsys) return;
  const SysDev &S = t.sys[s];
  const int w0 = well_off[s], nw = well_off[s + 1] - w0;
  const double dv = S.volume / S.nr;
  for (int e = threadIdx.x; e < nw * 5; e += blockDim.x) {
    double acc = 0;
    for (int b = 0; b < RB; ++b) acc += part[((long long)s * RB + b) * max_wells * 5 + e];
    grad[5 * w0 + e] = dv * acc;
  }
}

void launch_hf_gradient(const Tables &t, int nsys, const double *rho, const double *wells,
                        const int *well_off, const double *cells, double *part, int max_wells,
                        double *grad, cudaStream_t s) {
  if (max_wells <= 0) return;
  derek::note_launch(), k_hf_partials<<<dim3(RB, nsys), 256, 0, s>>>(t, rho, wells, well_off, cells, part, max_wells);
  derek::note_launch(), k_hf_final<<<nsys, 128, 0, s>>>(t, nsys, part, well_off, grad, max_wells);
}

}  // namespace derek

namespace derek {

// V_H[rho] into cgrid (.x), every system (FP64 grids).
void launch_hartree_only(const Tables &t, int nsys, int max_nr, int max_n, const double *rho,
                         double2 *cgrid, cudaStream_t s) {
  const int gx = (int)std::min<long long>(((long long)max_nr + 255) / 256, 256);
  derek::note_launch(), k_real_to_complex<<<dim3(gx, nsys), 256, 0, s>>>(t, rho, cgrid, 1);
  launch_fft3d_grid(t, 0, nsys, max_n, cgrid, -1, s);
  derek::note_launch(), k_hartree_scale<<<dim3(gx, nsys), 256, 0, s>>>(t, cgrid, 1);
  launch_fft3d_grid(t, 0, nsys, max_n, cgrid, +1, s);
}

// dv_xc/dn at rho (central difference, relative step 1e-4; zero below 1e-10)
__global__ void k_fxc(long long n, const double *__restrict__ rho, double *__restrict__ fxc) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double r = rho[i];
    double f = 0.0;
    if (r > 1e-10) {
      const double h = 1e-4 * r;
      double e1, v1, e2, v2;
      lda_point(r + h, e1, v1);
      lda_point(r - h, e2, v2);
      f = (v1 - v2) / (2.0 * h);
    }
    fxc[i] = f;
  }
}

void launch_fxc(long long n, const double *rho, double *fxc, cudaStream_t s) {
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 8);
  derek::note_launch(), k_fxc<<<blocks, 256, 0, s>>>(n, rho, fxc);
}

}  // namespace derek
