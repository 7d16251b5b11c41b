// Subspace kernels of the Chebyshev-filtered subspace iteration:
//   overlaps  A^H B (split-K, batched over k-sets)        -> FP64 matrices
//   rotation  X <- X C (in place, batched over k-sets)
//   Cholesky of the overlap and the inverse factor C = L^-H (FP64)
//   Hermitian Jacobi eigensolver of the projected Hamiltonian (FP64)
// These replace the empty wave_dot_* routines (Source/wave.f90:929-1036)
// with the full matrices a Rayleigh-Ritz step needs.
#include <cstdio>

#include "subspace.cuh"

#include <cooperative_groups.h>

namespace derek {

// ---------------------------------------------------------------------------
// Overlap: part[ks][split] = sum_{G in split} conj(A_i(G)) B_j(G)
// ---------------------------------------------------------------------------
constexpr int OT = 16;   // output tile
constexpr int OKC = 32;  // K chunk staged in shared memory

template <typename R>
__global__ void __launch_bounds__(256) k_overlap_partial(const Tables t, int ks_begin,
                                                         const cplx<R> *__restrict__ A,
                                                         const cplx<R> *__restrict__ B,
                                                         double2 *__restrict__ part,
                                                         const long long *__restrict__ part_off,
                                                         int ksplit) {
  __shared__ cplx<R> As[OT][OKC + 1];
  __shared__ cplx<R> Bs[OT][OKC + 1];
  const int ksi = ks_begin + blockIdx.z;
  const KSetDev &K = t.ks[ksi];
  if (!t.sys[K.sys].active) return;
  const int nb = K.nb;
  const int nt = (nb + OT - 1) / OT;
  const int ti = blockIdx.x / nt, tj = blockIdx.x - (blockIdx.x / nt) * nt;
  if (ti >= nt) return;
  const int split = blockIdx.y;
  const int g0 = split * ksplit;
  if (g0 >= K.npw) return;
  const int g1 = min(K.npw, g0 + ksplit);
  const int ty = threadIdx.x / OT, tx = threadIdx.x % OT;
  const int i0 = ti * OT, j0 = tj * OT;
  const cplx<R> *Ab = A + K.psi_off;
  const cplx<R> *Bb = B + K.psi_off;
  R ar = 0, ai = 0;
  for (int k0 = g0; k0 < g1; k0 += OKC) {
    for (int e = threadIdx.x; e < OT * OKC; e += blockDim.x) {
      const int r = e / OKC, c = e % OKC;
      const int g = k0 + c;
      const int ia = i0 + r, jb = j0 + r;
      As[r][c] = (ia < nb && g < g1) ? Ab[(long long)ia * K.npw_pad + g] : mk<R>(0, 0);
      Bs[r][c] = (jb < nb && g < g1) ? Bb[(long long)jb * K.npw_pad + g] : mk<R>(0, 0);
    }
    __syncthreads();
#pragma unroll 8
    for (int c = 0; c < OKC; ++c) {
      const cplx<R> a = As[ty][c], b = Bs[tx][c];
      ar += a.x * b.x + a.y * b.y;
      ai += a.x * b.y - a.y * b.x;
    }
    __syncthreads();
  }
  const int i = i0 + ty, j = j0 + tx;
  if (i < nb && j < nb)
    part[part_off[ksi] + ((long long)split * nb + i) * nb + j] = make_double2((double)ar, (double)ai);
}

__global__ void k_overlap_reduce(const Tables t, int ks_begin, const double2 *__restrict__ part,
                                 const long long *__restrict__ part_off, int ksplit,
                                 double2 *__restrict__ out, const long long *__restrict__ mat_off,
                                 int hermitize) {
  const int ksi = ks_begin + blockIdx.x;
  const KSetDev &K = t.ks[ksi];
  if (!t.sys[K.sys].active) return;
  const int nb = K.nb;
  const int nsplit = (K.npw + ksplit - 1) / ksplit;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    double x = 0, y = 0;
    for (int s = 0; s < nsplit; ++s) {
      const double2 v = part[part_off[ksi] + (long long)s * nb * nb + e];
      x += v.x;
      y += v.y;
    }
    out[mat_off[ksi] + e] = make_double2(x, y);
  }
  if (hermitize) {
    __syncthreads();
    double2 *M = out + mat_off[ksi];
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
      const int i = e / nb, j = e % nb;
      if (i < j) {
        const double2 a = M[i * nb + j], b = M[j * nb + i];
        const double2 h = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
        M[i * nb + j] = h;
        M[j * nb + i] = make_double2(h.x, -h.y);
      } else if (i == j) {
        M[e].y = 0.0;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Rotation: X[:, j] <- sum_i X[:, i] C[i][j], in place per G tile
// ---------------------------------------------------------------------------
constexpr int RG = 32;   // G columns per block
constexpr int RI = 32;   // rows of C staged per chunk
constexpr int RJ = 16;   // max output bands per thread (nb <= 8 * RJ = 128)

template <typename R>
__global__ void __launch_bounds__(256) k_rotate(const Tables t, int ks_begin, cplx<R> *__restrict__ X,
                                                const double2 *__restrict__ C,
                                                const long long *__restrict__ mat_off) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ksi = ks_begin + blockIdx.y;
  const KSetDev &K = t.ks[ksi];
  if (!t.sys[K.sys].active) return;
  const int g0 = blockIdx.x * RG;
  if (g0 >= K.npw) return;
  const int nb = K.nb;
  cplx<R> *Xs = reinterpret_cast<cplx<R> *>(smem_raw);   // [RI][RG]
  cplx<R> *Cs = Xs + RI * RG;                            // [RI][nb]
  const int g = threadIdx.x % RG, jg = threadIdx.x / RG;  // 8 j-groups
  cplx<R> acc[RJ];
#pragma unroll
  for (int q = 0; q < RJ; ++q) acc[q] = mk<R>(0, 0);
  cplx<R> *Xb = X + K.psi_off;
  const double2 *Cb = C + mat_off[ksi];
  for (int i0 = 0; i0 < nb; i0 += RI) {
    const int ni = min(RI, nb - i0);
    for (int e = threadIdx.x; e < RI * RG; e += blockDim.x) {
      const int r = e / RG, c = e % RG;
      const int gg = g0 + c;
      Xs[e] = (r < ni && gg < K.npw) ? Xb[(long long)(i0 + r) * K.npw_pad + gg] : mk<R>(0, 0);
    }
    for (int e = threadIdx.x; e < ni * nb; e += blockDim.x) {
      const int r = e / nb, c = e % nb;
      const double2 v = Cb[(long long)(i0 + r) * nb + c];
      Cs[r * nb + c] = mk<R>((R)v.x, (R)v.y);
    }
    __syncthreads();
    for (int r = 0; r < ni; ++r) {
      const cplx<R> x = Xs[r * RG + g];
#pragma unroll
      for (int q = 0; q < RJ; ++q) {
        const int j = jg + 8 * q;
        if (j < nb) {
          const cplx<R> c = Cs[r * nb + j];
          acc[q].x += x.x * c.x - x.y * c.y;
          acc[q].y += x.x * c.y + x.y * c.x;
        }
      }
    }
    __syncthreads();
  }
  const int gg = g0 + g;
  if (gg < K.npw) {
#pragma unroll
    for (int q = 0; q < RJ; ++q) {
      const int j = jg + 8 * q;
      if (j < nb) Xb[(long long)j * K.npw_pad + gg] = acc[q];
    }
  }
}

// ---------------------------------------------------------------------------
// Cholesky S = L L^H and C = L^-H (upper triangular), one block per k-set.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zmulc(double2 a, double2 b) {  // a * conj(b)
  return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

__global__ void __launch_bounds__(256) k_cholesky_inv(const Tables t, int ks_begin,
                                                      const double2 *__restrict__ S,
                                                      double2 *__restrict__ Cout,
                                                      const long long *__restrict__ mat_off,
                                                      double2 *__restrict__ scratch,
                                                      int *__restrict__ status, int use_smem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ksi = ks_begin + blockIdx.x;
  const KSetDev &K = t.ks[ksi];
  if (!t.sys[K.sys].active) return;
  const int n = K.nb;
  double2 *M = use_smem ? reinterpret_cast<double2 *>(smem_raw) : scratch + 2 * mat_off[ksi];
  double2 *Li = M + n * n;
  __shared__ double s_diag;
  __shared__ int s_fail;
  const double2 *Sb = S + mat_off[ksi];
  double dmax = 0.0;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    M[e] = Sb[e];
    Li[e] = make_double2(0, 0);
  }
  if (threadIdx.x == 0) s_fail = 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) dmax = fmax(dmax, M[i * n + i].x);
    s_diag = dmax;
  }
  __syncthreads();
  const double thr = 1e-13 * s_diag;
  for (int j = 0; j < n; ++j) {
    if (threadIdx.x == 0) {
      const double d = M[j * n + j].x;
      if (!(d > thr)) s_fail = 1;
      M[j * n + j] = make_double2(sqrt(fmax(d, thr)), 0.0);
    }
    __syncthreads();
    const double inv = 1.0 / M[j * n + j].x;
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) {
      M[i * n + j].x *= inv;
      M[i * n + j].y *= inv;
    }
    __syncthreads();
    // trailing update of the lower triangle: M[i][k] -= L[i][j] conj(L[k][j]), j < k <= i
    const int m = n - j - 1;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int i = j + 1 + e / m, k = j + 1 + e % m;
      if (k <= i) {
        const double2 p = zmulc(M[i * n + j], M[k * n + j]);
        M[i * n + k].x -= p.x;
        M[i * n + k].y -= p.y;
      }
    }
    __syncthreads();
  }
  // inverse of L: column c solves L x = e_c (forward substitution), one thread per column
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    for (int i = c; i < n; ++i) {
      double2 acc = make_double2(i == c ? 1.0 : 0.0, 0.0);
      for (int p = c; p < i; ++p) {
        const double2 q = zmul(M[i * n + p], Li[p * n + c]);
        acc.x -= q.x;
        acc.y -= q.y;
      }
      const double d = 1.0 / M[i * n + i].x;
      Li[i * n + c] = make_double2(acc.x * d, acc.y * d);
    }
  }
  __syncthreads();
  // C[i][j] = conj(Linv[j][i])
  double2 *Cb = Cout + mat_off[ksi];
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e % n;
    const double2 v = Li[j * n + i];
    Cb[e] = make_double2(v.x, -v.y);
  }
  // keep an earlier failure of this k-set (a timed-out overlap wait)
  if (threadIdx.x == 0 && s_fail && status[ksi] == 0) status[ksi] = DEREK_ERR_CHOLESKY;
}

// ---------------------------------------------------------------------------
// Hermitian Jacobi eigensolver (parallel cyclic, round-robin pair ordering).
// Each round rotates np = ne/2 disjoint index pairs (p, q) at once:
//   A <- U^H A U,  V <- V U,  U = diag(1, e^{-i phi}) [[c, s], [-s, c]] per pair.
// Entry (i, j) of U^H A U depends only on the 2x2 block of A at the pairs
// holding i and j, so a round is one pass over the blocks (a <= b) of pairs:
// A'_ab = U_a^H A_ab U_b, with A'_ba = A'_ab^H written by the same thread.
// That touches half of A, with all arithmetic on A in FP64.  The
// eigenvectors accumulate in VT (FP64, or FP32 on the mixed-precision path,
// whose wavefunctions are FP32), stored one eigenvector per row so that a
// warp updates consecutive addresses.  Eigenvalues ascending go to
// eig[item0 + j]; eigenvectors (columns) to C.
// ---------------------------------------------------------------------------
// pair k of round r in the circle schedule over ne positions (position 0
// fixed, the others advance one place per round)
// Rotation that zeroes the Hermitian 2x2 block [[a, b], [conj(b), d]]: the
// phase ph = b / |b|, then the real symmetric rotation (c, s) of
// [[a, |b|], [|b|, d]] with t = sign(tau) / (|tau| + sqrt(1 + tau^2)),
// tau = (d - a) / (2 |b|), c = 1 / sqrt(1 + t^2), s = t c (Rutishauser).
// Written as two reciprocal square roots, one square root and one division:
// the dependent FP64 chain every Jacobi round waits on.  The entries are bounded by the matrix norm, so |b| needs
// no hypot scaling.  False (no rotation) when |b| <= skip.
__device__ __forceinline__ bool jacobi_rotation(double a, double d, double2 b, double skip, double &c,
                                                double &s, double2 &ph) {
  const double e2 = b.x * b.x + b.y * b.y;
  if (!(e2 > skip * skip)) return false;
  const double ie = rsqrt(e2);
  ph = make_double2(b.x * ie, b.y * ie);
  const double tau = (d - a) * (0.5 * ie);
  const double tt = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
  c = rsqrt(1.0 + tt * tt);
  s = tt * c;
  return true;
}

__device__ __forceinline__ void rr_pair(int k, int r, int ne, int &p, int &q) {
  const int m = ne - 1;
  const int a = k == 0 ? 0 : 1 + (k - 1 + r) % m;
  const int b = 1 + (ne - 2 - k + r) % m;
  p = min(a, b);
  q = max(a, b);
}

template <typename VT>
__global__ void __launch_bounds__(256) k_jacobi(const Tables t, int ks_begin,
                                                const double2 *__restrict__ Hs,
                                                double2 *__restrict__ Cout,
                                                const long long *__restrict__ mat_off,
                                                double *__restrict__ eig,
                                                double2 *__restrict__ scratch, int max_sweeps,
                                                double tol, int a_in_smem, int v_in_smem,
                                                int *__restrict__ sweeps_out) {
  using V2 = cplx<VT>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ksi = ks_begin + blockIdx.x;
  const KSetDev &K = t.ks[ksi];
  if (!t.sys[K.sys].active) return;
  const int n = K.nb;
  const int ne = n + (n & 1);  // even count for the tournament; index n is a dummy
  const int np = ne / 2;
  const int nblk = np * (np + 1) / 2;
  unsigned char *sp = smem_raw;
  double2 *A = a_in_smem ? reinterpret_cast<double2 *>(sp) : scratch + 2 * mat_off[ksi] + (long long)n * n;
  if (a_in_smem) sp += (size_t)n * n * sizeof(double2);
  V2 *Vt = v_in_smem ? reinterpret_cast<V2 *>(sp) : reinterpret_cast<V2 *>(scratch + 2 * mat_off[ksi]);
  if (v_in_smem) sp += ((size_t)n * n * sizeof(V2) + 15) / 16 * 16;
  double2 *rph = reinterpret_cast<double2 *>(sp);  // [np]
  double *rc = reinterpret_cast<double *>(rph + np);
  double *rs = rc + np;
  int *pp = reinterpret_cast<int *>(rs + np);
  int *pq = pp + np;
  int *act = pq + np;
  short2 *blk = reinterpret_cast<short2 *>(act + np);  // [nblk]: (a, b), a <= b
  __shared__ double red[256];
  __shared__ double red2[256];
  const double2 *Hb = Hs + mat_off[ksi];
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    A[e] = Hb[e];
    const int i = e / n, j = e % n;
    V2 one;
    one.x = (VT)(i == j ? 1 : 0);
    one.y = (VT)0;
    Vt[e] = one;
  }
  for (int w = threadIdx.x; w < nblk; w += blockDim.x) {
    // w -> (a, b) with a <= b, rows of the upper triangle in order
    int a = 0, rem = w;
    while (rem >= np - a) {
      rem -= np - a;
      ++a;
    }
    blk[w] = make_short2((short)a, (short)(a + rem));
  }
  __syncthreads();
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    // convergence: sum of |offdiag|^2 vs sum of |A|^2, both summed directly
    double off = 0, tot = 0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const double m2 = A[e].x * A[e].x + A[e].y * A[e].y;
      tot += m2;
      if (e / n != e % n) off += m2;
    }
    red[threadIdx.x] = off;
    red2[threadIdx.x] = tot;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        red[threadIdx.x] += red[threadIdx.x + s];
        red2[threadIdx.x] += red2[threadIdx.x + s];
      }
      __syncthreads();
    }
    const bool done = red[0] <= tol * tol * red2[0];
    // skip rotations whose element cannot matter for the convergence test
    // (threshold Jacobi): |a_pq| below tol * ||A||_F / (4 n)
    const double skip = tol * sqrt(red2[0]) / (4.0 * n);
    __syncthreads();
    if (done) break;
    for (int round = 0; round < ne - 1; ++round) {
      for (int k = threadIdx.x; k < np; k += blockDim.x) {
        int p, q;
        rr_pair(k, round, ne, p, q);
        pp[k] = p;
        pq[k] = q;
        double c = 1.0, s = 0.0;
        double2 ph = make_double2(1.0, 0.0);
        int on = 0;
        if (q < n) {
          on = jacobi_rotation(A[p * n + p].x, A[q * n + q].x, A[p * n + q], skip, c, s, ph) ? 1 : 0;
        }
        rc[k] = c;
        rs[k] = s;
        rph[k] = ph;
        act[k] = on;
      }
      __syncthreads();
      // blocks of A: left by U_a^H (new row p = c A_p - s ph A_q, new row
      // q = s A_p + c ph A_q), right by U_b (new col p = c X_p - s conj(ph) X_q,
      // new col q = s X_p + c conj(ph) X_q)
      for (int w = threadIdx.x; w < nblk; w += blockDim.x) {
        const short2 ab = blk[w];
        const int ia = ab.x, ib = ab.y;
        const int on_a = act[ia], on_b = act[ib];
        if (!on_a && !on_b) continue;
        const int pa = pp[ia], qa = pq[ia], pb = pp[ib], qb = pq[ib];
        const bool qa_ok = qa < n, qb_ok = qb < n;
        const double2 z = make_double2(0.0, 0.0);
        double2 x00 = A[pa * n + pb];
        double2 x01 = qb_ok ? A[pa * n + qb] : z;
        double2 x10 = qa_ok ? A[qa * n + pb] : z;
        double2 x11 = (qa_ok && qb_ok) ? A[qa * n + qb] : z;
        if (on_a) {
          const double c = rc[ia], s = rs[ia];
          const double2 ph = rph[ia];
          const double2 t0 = zmul(ph, x10), t1 = zmul(ph, x11);
          const double2 n00 = make_double2(c * x00.x - s * t0.x, c * x00.y - s * t0.y);
          const double2 n01 = make_double2(c * x01.x - s * t1.x, c * x01.y - s * t1.y);
          x10 = make_double2(s * x00.x + c * t0.x, s * x00.y + c * t0.y);
          x11 = make_double2(s * x01.x + c * t1.x, s * x01.y + c * t1.y);
          x00 = n00;
          x01 = n01;
        }
        if (on_b) {
          const double c = rc[ib], s = rs[ib];
          const double2 phc = make_double2(rph[ib].x, -rph[ib].y);
          const double2 t0 = zmul(phc, x01), t1 = zmul(phc, x11);
          const double2 n00 = make_double2(c * x00.x - s * t0.x, c * x00.y - s * t0.y);
          const double2 n10 = make_double2(c * x10.x - s * t1.x, c * x10.y - s * t1.y);
          x01 = make_double2(s * x00.x + c * t0.x, s * x00.y + c * t0.y);
          x11 = make_double2(s * x10.x + c * t1.x, s * x10.y + c * t1.y);
          x00 = n00;
          x10 = n10;
        }
        if (ia == ib) {
          // the pair's own 2x2 block is now diagonal and real
          A[pa * n + pa] = make_double2(x00.x, 0.0);
          A[qa * n + qa] = make_double2(x11.x, 0.0);
          A[pa * n + qa] = z;
          A[qa * n + pa] = z;
          continue;
        }
        A[pa * n + pb] = x00;
        A[pb * n + pa] = make_double2(x00.x, -x00.y);
        if (qb_ok) {
          A[pa * n + qb] = x01;
          A[qb * n + pa] = make_double2(x01.x, -x01.y);
        }
        if (qa_ok) {
          A[qa * n + pb] = x10;
          A[pb * n + qa] = make_double2(x10.x, -x10.y);
        }
        if (qa_ok && qb_ok) {
          A[qa * n + qb] = x11;
          A[qb * n + qa] = make_double2(x11.x, -x11.y);
        }
      }
      // eigenvectors: Vt[col][row], new col p = c X_p - s conj(ph) X_q,
      // new col q = s X_p + c conj(ph) X_q
      for (int w = threadIdx.x; w < np * n; w += blockDim.x) {
        const int k = w / n, row = w - (w / n) * n;
        if (!act[k]) continue;
        const VT c = (VT)rc[k], s = (VT)rs[k];
        const VT phx = (VT)rph[k].x, phy = (VT)-rph[k].y;
        V2 &xp = Vt[pp[k] * n + row];
        V2 &xq = Vt[pq[k] * n + row];
        const V2 a = xp, b = xq;
        const VT tx = phx * b.x - phy * b.y, ty = phx * b.y + phy * b.x;
        xp.x = c * a.x - s * tx;
        xp.y = c * a.y - s * ty;
        xq.x = s * a.x + c * tx;
        xq.y = s * a.y + c * ty;
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0 && sweeps_out) sweeps_out[ksi] = sweep;
  // sort eigenvalues ascending (selection by rank; ties broken by index)
  double *ev = rc;  // reuse: np * 2 >= n entries (rc and rs are adjacent)
  for (int i = threadIdx.x; i < n; i += blockDim.x) ev[i] = A[i * n + i].x;
  __syncthreads();
  double2 *Cb = Cout + mat_off[ksi];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double vi = ev[i];
    int rank = 0;
    for (int j = 0; j < n; ++j) rank += (ev[j] < vi) || (ev[j] == vi && j < i);
    eig[K.item0 + rank] = vi;
    for (int r = 0; r < n; ++r) {
      const V2 v = Vt[i * n + r];
      Cb[r * n + rank] = make_double2((double)v.x, (double)v.y);
    }
  }
}

// ---------------------------------------------------------------------------
// The same Jacobi eigensolver on a cluster of two CTAs per k-set, so the FP64
// work of a round is split over two SMs.  Each CTA keeps a full copy of A and
// computes every rotation (the two copies are equal, so both take the same
// decisions); it updates half of the 2x2 blocks of a round and writes each
// result into its own A and, through distributed shared memory, into its
// partner's, then updates its half of the eigenvector rows.  One cluster
// barrier per round makes the partner's writes visible before the next
// round reads A.
// ---------------------------------------------------------------------------
template <typename VT>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(256)
    k_jacobi_pair(const Tables t, int ks_begin, const double2 *__restrict__ Hs,
                  double2 *__restrict__ Cout, const long long *__restrict__ mat_off,
                  double *__restrict__ eig, int max_sweeps, double tol, int *__restrict__ sweeps_out) {
  using V2 = cplx<VT>;
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int crank = (int)cluster.block_rank();
  const int ksi = ks_begin + blockIdx.x / 2;
  const KSetDev &K = t.ks[ksi];
  if (!t.sys[K.sys].active) return;   // both CTAs of the cluster leave together
  const int n = K.nb;
  const int ne = n + (n & 1);
  const int np = ne / 2;
  const int nblk = np * (np + 1) / 2;
  const int hv = (n + 1) / 2;                  // eigenvector rows per CTA
  const int r0 = crank * hv, r1 = min(n, r0 + hv);
  unsigned char *sp = smem_raw;
  double2 *A = reinterpret_cast<double2 *>(sp);
  sp += (size_t)n * n * sizeof(double2);
  V2 *Vt = reinterpret_cast<V2 *>(sp);          // [n][hv]: eigenvector i, rows r0..r1
  sp += ((size_t)n * hv * sizeof(V2) + 15) / 16 * 16;
  double2 *rph = reinterpret_cast<double2 *>(sp);
  double *rc = reinterpret_cast<double *>(rph + np);
  double *rs = rc + np;
  int *pp = reinterpret_cast<int *>(rs + np);
  int *pq = pp + np;
  int *act = pq + np;
  short2 *blk = reinterpret_cast<short2 *>(act + np);
  __shared__ double red[256];
  __shared__ double red2[256];
  double2 *Ap = cluster.map_shared_rank(A, crank ^ 1);   // the partner's copy of A
  const double2 *Hb = Hs + mat_off[ksi];
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) A[e] = Hb[e];
  for (int e = threadIdx.x; e < n * hv; e += blockDim.x) {
    const int i = e / hv, r = r0 + e % hv;
    V2 one;
    one.x = (VT)(i == r ? 1 : 0);
    one.y = (VT)0;
    Vt[e] = one;
  }
  for (int w = threadIdx.x; w < nblk; w += blockDim.x) {
    int a = 0, rem = w;
    while (rem >= np - a) {
      rem -= np - a;
      ++a;
    }
    blk[w] = make_short2((short)a, (short)(a + rem));
  }
  cluster.sync();   // both CTAs running and initialised before any remote write
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    double off = 0, tot = 0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const double m2 = A[e].x * A[e].x + A[e].y * A[e].y;
      tot += m2;
      if (e / n != e % n) off += m2;
    }
    red[threadIdx.x] = off;
    red2[threadIdx.x] = tot;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        red[threadIdx.x] += red[threadIdx.x + s];
        red2[threadIdx.x] += red2[threadIdx.x + s];
      }
      __syncthreads();
    }
    const bool done = red[0] <= tol * tol * red2[0];
    const double skip = tol * sqrt(red2[0]) / (4.0 * n);
    __syncthreads();
    if (done) break;
    for (int round = 0; round < ne - 1; ++round) {
      for (int k = threadIdx.x; k < np; k += blockDim.x) {
        int p, q;
        rr_pair(k, round, ne, p, q);
        pp[k] = p;
        pq[k] = q;
        double c = 1.0, s = 0.0;
        double2 ph = make_double2(1.0, 0.0);
        int on = 0;
        if (q < n) {
          on = jacobi_rotation(A[p * n + p].x, A[q * n + q].x, A[p * n + q], skip, c, s, ph) ? 1 : 0;
        }
        rc[k] = c;
        rs[k] = s;
        rph[k] = ph;
        act[k] = on;
      }
      __syncthreads();
      for (int w = crank + 2 * (int)threadIdx.x; w < nblk; w += 2 * blockDim.x) {
        const short2 ab = blk[w];
        const int ia = ab.x, ib = ab.y;
        const int on_a = act[ia], on_b = act[ib];
        if (!on_a && !on_b) continue;
        const int pa = pp[ia], qa = pq[ia], pb = pp[ib], qb = pq[ib];
        const bool qa_ok = qa < n, qb_ok = qb < n;
        const double2 z = make_double2(0.0, 0.0);
        double2 x00 = A[pa * n + pb];
        double2 x01 = qb_ok ? A[pa * n + qb] : z;
        double2 x10 = qa_ok ? A[qa * n + pb] : z;
        double2 x11 = (qa_ok && qb_ok) ? A[qa * n + qb] : z;
        if (on_a) {
          const double c = rc[ia], s = rs[ia];
          const double2 ph = rph[ia];
          const double2 t0 = zmul(ph, x10), t1 = zmul(ph, x11);
          const double2 n00 = make_double2(c * x00.x - s * t0.x, c * x00.y - s * t0.y);
          const double2 n01 = make_double2(c * x01.x - s * t1.x, c * x01.y - s * t1.y);
          x10 = make_double2(s * x00.x + c * t0.x, s * x00.y + c * t0.y);
          x11 = make_double2(s * x01.x + c * t1.x, s * x01.y + c * t1.y);
          x00 = n00;
          x01 = n01;
        }
        if (on_b) {
          const double c = rc[ib], s = rs[ib];
          const double2 phc = make_double2(rph[ib].x, -rph[ib].y);
          const double2 t0 = zmul(phc, x01), t1 = zmul(phc, x11);
          const double2 n00 = make_double2(c * x00.x - s * t0.x, c * x00.y - s * t0.y);
          const double2 n10 = make_double2(c * x10.x - s * t1.x, c * x10.y - s * t1.y);
          x01 = make_double2(s * x00.x + c * t0.x, s * x00.y + c * t0.y);
          x11 = make_double2(s * x10.x + c * t1.x, s * x10.y + c * t1.y);
          x00 = n00;
          x10 = n10;
        }
        // each entry goes to both copies of A
        auto put = [&](int idx, double2 v) {
          A[idx] = v;
          Ap[idx] = v;
        };
        if (ia == ib) {
          put(pa * n + pa, make_double2(x00.x, 0.0));
          put(qa * n + qa, make_double2(x11.x, 0.0));
          put(pa * n + qa, z);
          put(qa * n + pa, z);
          continue;
        }
        put(pa * n + pb, x00);
        put(pb * n + pa, make_double2(x00.x, -x00.y));
        if (qb_ok) {
          put(pa * n + qb, x01);
          put(qb * n + pa, make_double2(x01.x, -x01.y));
        }
        if (qa_ok) {
          put(qa * n + pb, x10);
          put(pb * n + qa, make_double2(x10.x, -x10.y));
        }
        if (qa_ok && qb_ok) {
          put(qa * n + qb, x11);
          put(qb * n + qa, make_double2(x11.x, -x11.y));
        }
      }
      // eigenvector rows r0..r1 of this CTA
      const int nr = r1 - r0;
      for (int w = threadIdx.x; w < np * nr; w += blockDim.x) {
        const int k = w / nr, row = w - (w / nr) * nr;
        if (!act[k]) continue;
        const VT c = (VT)rc[k], s = (VT)rs[k];
        const VT phx = (VT)rph[k].x, phy = (VT)-rph[k].y;
        V2 &xp = Vt[pp[k] * hv + row];
        V2 &xq = Vt[pq[k] * hv + row];
        const V2 a = xp, b = xq;
        const VT tx = phx * b.x - phy * b.y, ty = phx * b.y + phy * b.x;
        xp.x = c * a.x - s * tx;
        xp.y = c * a.y - s * ty;
        xq.x = s * a.x + c * tx;
        xq.y = s * a.y + c * ty;
      }
      cluster.sync();   // both halves of the round written into both copies of A
    }
  }
  if (threadIdx.x == 0 && crank == 0 && sweeps_out) sweeps_out[ksi] = sweep;
  double *ev = rc;
  for (int i = threadIdx.x; i < n; i += blockDim.x) ev[i] = A[i * n + i].x;
  __syncthreads();
  double2 *Cb = Cout + mat_off[ksi];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double vi = ev[i];
    int rank = 0;
    for (int j = 0; j < n; ++j) rank += (ev[j] < vi) || (ev[j] == vi && j < i);
    if (crank == 0) eig[K.item0 + rank] = vi;
    for (int r = r0; r < r1; ++r) {
      const V2 v = Vt[i * hv + (r - r0)];
      Cb[r * n + rank] = make_double2((double)v.x, (double)v.y);
    }
  }
  cluster.sync();   // neither CTA leaves while its partner could still address it
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename R>
void launch_overlap(const Tables &t, int ks_begin, int nks, int max_nb, int max_npw, int ksplit,
                    const cplx<R> *A, const cplx<R> *B, double2 *part, const long long *part_off,
                    double2 *out, const long long *mat_off, int hermitize, cudaStream_t st) {
  if (nks <= 0) return;
  const int nt = (max_nb + OT - 1) / OT;
  dim3 grid(nt * nt, (max_npw + ksplit - 1) / ksplit, nks);
  derek::note_launch(), k_overlap_partial<R><<<grid, 256, 0, st>>>(t, ks_begin, A, B, part, part_off, ksplit);
  launch_overlap_reduce(t, ks_begin, nks, part, part_off, ksplit, out, mat_off, hermitize, st);
}

void launch_overlap_reduce(const Tables &t, int ks_begin, int nks, const double2 *part,
                           const long long *part_off, int ksplit, double2 *out,
                           const long long *mat_off, int hermitize, cudaStream_t st) {
  derek::note_launch(), k_overlap_reduce<<<nks, 256, 0, st>>>(t, ks_begin, part, part_off, ksplit, out, mat_off, hermitize);
}

template <typename R>
void launch_rotate(const Tables &t, int ks_begin, int nks, int max_nb, int max_npw, cplx<R> *X,
                   const double2 *C, const long long *mat_off, cudaStream_t st) {
  if (nks <= 0) return;
  const size_t sm = (RI * RG + (size_t)RI * max_nb) * sizeof(cplx<R>);
  cudaFuncSetAttribute(k_rotate<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid((max_npw + RG - 1) / RG, nks);
  derek::note_launch(), k_rotate<R><<<grid, 256, sm, st>>>(t, ks_begin, X, C, mat_off);
}

bool cholesky_fits_smem(int max_nb) { return 2 * (size_t)max_nb * max_nb * 16 <= 200 * 1024; }
void launch_cholesky_inv(const Tables &t, int ks_begin, int nks, int max_nb, const double2 *S,
                         double2 *C, const long long *mat_off, double2 *scratch, int *status,
                         cudaStream_t st) {
  if (nks <= 0) return;
  const int use_smem = cholesky_fits_smem(max_nb);
  const size_t sm = use_smem ? 2 * (size_t)max_nb * max_nb * sizeof(double2) : 0;
  cudaFuncSetAttribute(k_cholesky_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  derek::note_launch(), k_cholesky_inv<<<nks, 256, sm, st>>>(t, ks_begin, S, C, mat_off, scratch, status, use_smem);
}

// shared memory of the Jacobi kernel: A (FP64) when it fits, the eigenvector
// matrix when it also fits, and the pair and block tables
static size_t jacobi_tables(int max_nb) {
  const size_t np = (size_t)(max_nb + 1) / 2;
  return np * (sizeof(double2) + 2 * sizeof(double) + 3 * sizeof(int)) + np * (np + 1) / 2 * 4 + 64;
}
constexpr size_t kJacobiSmem = 227 * 1024 - 4096;   // static reduction arrays take 4 KB

void launch_jacobi(const Tables &t, int ks_begin, int nks, int max_nb, const double2 *Hs,
                   double2 *C, const long long *mat_off, double *eig, double2 *scratch,
                   int max_sweeps, double tol, int fp32_vectors, int *sweeps_out, cudaStream_t st,
                   int single) {
  if (nks <= 0) return;
  const size_t nn = (size_t)max_nb * max_nb;
  const size_t tab = jacobi_tables(max_nb);
  const size_t vbytes = (nn * (fp32_vectors ? sizeof(float2) : sizeof(double2)) + 15) / 16 * 16;
  const int a_smem = nn * sizeof(double2) + tab <= kJacobiSmem;
  const int v_smem = a_smem && nn * sizeof(double2) + vbytes + tab <= kJacobiSmem;
  const size_t sm = (a_smem ? nn * sizeof(double2) : 0) + (v_smem ? vbytes : 0) + tab;
  // two CTAs per k-set when A and half of the eigenvector rows fit
  const size_t hv = (size_t)(max_nb + 1) / 2;
  const size_t vhalf = ((size_t)max_nb * hv * (fp32_vectors ? sizeof(float2) : sizeof(double2)) + 15) / 16 * 16;
  const size_t sm_pair = nn * sizeof(double2) + vhalf + tab;
  if (!single && sm_pair <= kJacobiSmem) {
    if (fp32_vectors) {
      cudaFuncSetAttribute(k_jacobi_pair<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_pair);
      derek::note_launch(), k_jacobi_pair<float><<<2 * nks, 256, sm_pair, st>>>(t, ks_begin, Hs, C, mat_off, eig,
                                                                             max_sweeps, tol, sweeps_out);
    } else {
      cudaFuncSetAttribute(k_jacobi_pair<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_pair);
      derek::note_launch(), k_jacobi_pair<double><<<2 * nks, 256, sm_pair, st>>>(t, ks_begin, Hs, C, mat_off, eig,
                                                                              max_sweeps, tol, sweeps_out);
    }
    return;
  }
  if (fp32_vectors) {
    cudaFuncSetAttribute(k_jacobi<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    derek::note_launch(), k_jacobi<float><<<nks, 256, sm, st>>>(t, ks_begin, Hs, C, mat_off, eig, scratch, max_sweeps,
                                                                tol, a_smem, v_smem, sweeps_out);
  } else {
    cudaFuncSetAttribute(k_jacobi<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    derek::note_launch(), k_jacobi<double><<<nks, 256, sm, st>>>(t, ks_begin, Hs, C, mat_off, eig, scratch, max_sweeps,
                                                                 tol, a_smem, v_smem, sweeps_out);
  }
}

#define DEREK_INST(R)                                                                          \
  template void launch_overlap<R>(const Tables &, int, int, int, int, int, const cplx<R> *,    \
                                  const cplx<R> *, double2 *, const long long *, double2 *,   \
                                  const long long *, int, cudaStream_t);                      \
  template void launch_rotate<R>(const Tables &, int, int, int, int, cplx<R> *,               \
                                 const double2 *, const long long *, cudaStream_t);
DEREK_INST(float)
DEREK_INST(double)
#undef DEREK_INST

}  // namespace derek
