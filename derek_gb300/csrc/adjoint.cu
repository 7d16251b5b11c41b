// Adjoint gradient of a density-matching loss through the converged SCF.
//
//   L(p) = sum_r (n(r) - n_target(r))^2 dV,   p = Gaussian-well parameters
//   dL/dp = dV sum_r u(r) dV_ext/dp(r),   u = chi [2 (n - n_target)]
//
// chi, the self-consistent density response (symmetric for a real
// perturbation), is applied once: u solves u = chi0 [g + v_H[u] + f_xc u]
// with g = 2 (n - n_target), iterated with Anderson mixing.  chi0 of the
// smeared (metallic) ground state is written as density-functional
// perturbation theory for metals (S. de Gironcoli, Phys. Rev. B 51, 6773
// (1995)) split at a subspace M of each k-set: its leading bands that are
// converged eigenvectors (Ritz residual below kRitzConv), and at least every
// band with occupation above 1e-12:
//   dn = sum_k w_k/Omega [ sum_{n,m in M} w_nm psi_n^* psi_m V_mn
//                        + sum_n 2 f_n Re psi_n^* x_n ]  - dmu n_F,
//   w_nm = (f_n - f_m)/(e_n - e_m) (f'_n when degenerate), V_mn = <m|dV|n>,
//   (H - e_n) x_n = -P_c dV psi_n on the complement of M (Sternheimer,
//   preconditioned conjugate gradients batched over every band),
//   dmu = sum w_k f'_n V_nn / sum w_k f'_n,  n_F = sum w_k/Omega f'_n |psi_n|^2.
// The real cross density Re psi^* xi is formed as (|psi + xi|^2 - |psi - xi|^2)/4
// with the density kernels.  FP64 path only.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "handle.h"
#include "scf_kernels.cuh"

namespace derek {
namespace {

__global__ void k_lincomb(long long n, double a, const double2 *__restrict__ X, double b,
                          const double2 *__restrict__ Y, double2 *__restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double2 x = X[i];
    const double2 y = Y ? Y[i] : make_double2(0, 0);
    out[i] = make_double2(a * x.x + b * y.x, a * x.y + b * y.y);
  }
}

// d[item] = Re <X_item | Y_item>
__global__ void k_item_dot(const Tables t, const double2 *__restrict__ X, const double2 *__restrict__ Y,
                           double *__restrict__ d) {
  __shared__ double red[256];
  const int item = blockIdx.x;
  const KSetDev &K = t.ks[t.item_ks[item]];
  const long long off = K.psi_off + (long long)t.item_band[item] * K.npw_pad;
  double s = 0;
  for (int g = threadIdx.x; g < K.npw; g += blockDim.x) {
    const double2 x = X[off + g], y = Y[off + g];
    s += x.x * y.x + x.y * y.y;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) d[item] = red[0];
}

// Y_item += sign * c[item] * X_item   (or, with xpay, Y = X + c Y)
__global__ void k_item_axpy(const Tables t, const double *__restrict__ c, double sign,
                            const double2 *__restrict__ X, double2 *__restrict__ Y, int xpay) {
  const int item = blockIdx.x;
  const KSetDev &K = t.ks[t.item_ks[item]];
  const long long off = K.psi_off + (long long)t.item_band[item] * K.npw_pad;
  const double a = sign * c[item];
  for (int g = threadIdx.x; g < K.npw; g += blockDim.x) {
    const double2 x = X[off + g];
    double2 y = Y[off + g];
    if (xpay) {
      y = make_double2(x.x + a * y.x, x.y + a * y.y);
    } else {
      y.x += a * x.x;
      y.y += a * x.y;
    }
    Y[off + g] = y;
  }
}

// Z = R / (1/2|k+G|^2 + 1), rows of items with mask[item] == 0 set to zero
__global__ void k_precond(const Tables t, const double2 *__restrict__ R, const double *__restrict__ mask,
                          double2 *__restrict__ Z) {
  const int item = blockIdx.x;
  const KSetDev &K = t.ks[t.item_ks[item]];
  const long long off = K.psi_off + (long long)t.item_band[item] * K.npw_pad;
  const double *kin = t.kin64 + K.ent_off;
  const double m = mask ? mask[item] : 1.0;
  for (int g = threadIdx.x; g < K.npw; g += blockDim.x) {
    const double2 r = R[off + g];
    const double p = m / (kin[g] + 1.0);
    Z[off + g] = make_double2(p * r.x, p * r.y);
  }
}

// Y[:, j] -= sum_i Psi[:, i] C[i][j] per k-set (all buffers FP64 complex)
__global__ void __launch_bounds__(256) k_gemm_sub(const Tables t, const double2 *__restrict__ Psi,
                                                  const double2 *__restrict__ C,
                                                  const long long *__restrict__ mat_off,
                                                  double2 *__restrict__ Y) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ksi = blockIdx.y;
  const KSetDev &K = t.ks[ksi];
  const int g0 = blockIdx.x * 32;
  if (g0 >= K.npw) return;
  const int nb = K.nb;
  double2 *Cs = reinterpret_cast<double2 *>(smem_raw);  // nb x nb
  const double2 *Cb = C + mat_off[ksi];
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) Cs[e] = Cb[e];
  __syncthreads();
  const int g = g0 + (threadIdx.x & 31);
  if (g >= K.npw) return;
  for (int j = threadIdx.x >> 5; j < nb; j += blockDim.x >> 5) {
    double ax = 0, ay = 0;
    for (int i = 0; i < nb; ++i) {
      const double2 p = Psi[K.psi_off + (long long)i * K.npw_pad + g];
      const double2 c = Cs[i * nb + j];
      ax += p.x * c.x - p.y * c.y;
      ay += p.x * c.y + p.y * c.x;
    }
    double2 &y = Y[K.psi_off + (long long)j * K.npw_pad + g];
    y.x -= ax;
    y.y -= ay;
  }
}

// W[m][n] = w_nm V[m][n] with w_nm = (f_n - f_m)/(e_n - e_m), f'_n when degenerate
__global__ void k_pair_weights(const Tables t, const double *__restrict__ eig,
                               const double *__restrict__ occ, const double2 *__restrict__ V,
                               const long long *__restrict__ mat_off, double2 *__restrict__ W) {
  const int ksi = blockIdx.x;
  const KSetDev &K = t.ks[ksi];
  const SysDev &S = t.sys[K.sys];
  const int nb = K.nb;
  const double kT = S.kT;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int m = e / nb, n = e % nb;
    const double em = eig[K.item0 + m], en = eig[K.item0 + n];
    const double fm = occ[K.item0 + m], fn = occ[K.item0 + n];
    double w;
    if (fabs(en - em) > 1e-9 * kT) {
      w = (fn - fm) / (en - em);
    } else {
      const double ft = 0.5 * fn;  // per-spin occupation
      w = -2.0 * ft * (1.0 - ft) / kT;
    }
    const double2 v = V[mat_off[ksi] + e];
    W[mat_off[ksi] + e] = make_double2(w * v.x, w * v.y);
  }
}

// CG scalar updates per item: alpha = rz / pAp (masked), beta = rz_new / rz
__global__ void k_cg_ratio(int n, const double *__restrict__ num, const double *__restrict__ den,
                           const double *__restrict__ mask, double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = den[i];
  out[i] = (mask[i] != 0.0 && d != 0.0) ? num[i] / d : 0.0;
}

__global__ void k_scale_grid(long long n, const double *__restrict__ a, double sa,
                             const double *__restrict__ b, double sb, double *__restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = sa * a[i] + (b ? sb * b[i] : 0.0);
}

// dV = g + V_H[dn] + f_xc dn
__global__ void k_response_potential(long long n, const double *__restrict__ g,
                                     const double2 *__restrict__ vh, const double *__restrict__ fxc,
                                     const double *__restrict__ dn, double *__restrict__ dv) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dv[i] = g[i] + vh[i].x + fxc[i] * dn[i];
}

template <typename T> cudaError_t dmalloc(T **p, size_t n) {
  return cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T));
}

struct Work {
  double2 *phi = nullptr, *xi = nullptr, *sp = nullptr, *sm = nullptr;
  double2 *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *ap = nullptr;
  double *w = nullptr, *mask = nullptr, *rz = nullptr, *rz2 = nullptr, *pap = nullptr,
         *alpha = nullptr, *beta = nullptr, *shift = nullptr;
  double *g = nullptr, *fxc = nullptr, *dn = nullptr, *dv = nullptr, *tmp = nullptr, *nf = nullptr,
         *dn_out = nullptr;
  Axpby *vcoef = nullptr;
  ~Work() {
    void *ptrs[] = {phi, xi, sp, sm, x, r, z, p, ap, w, mask, rz, rz2, pap, alpha, beta, shift,
                    g, fxc, dn, dv, tmp, nf, dn_out, vcoef};
    for (void *q : ptrs)
      if (q) cudaFree(q);
  }
};

}  // namespace
}  // namespace derek

using namespace derek;

extern "C" int derek_gpu_grad_density_loss(derek_gpu_t *h, int s, const double *n_target,
                                           double *loss, double *grad, int max_iter, double tol) {
  if (!h || s < 0 || s >= h->nsys || !n_target || !grad) return DEREK_ERR_BAD_ARG;
  if (reject_spinor(h, "grad_density_loss")) return DEREK_ERR_UNSUPPORTED;
  if (h->prec != DEREK_PREC_FP64 || h->nsys != 1) {
    h->last_error = "the adjoint gradient needs an FP64 handle over one system";
    return DEREK_ERR_UNSUPPORTED;
  }
  const int nw = h->well_off[s + 1] - h->well_off[s];
  if (nw == 0 || !h->wells_define_vext[s]) {
    h->last_error = "system has no Gaussian wells defining its external potential";
    return DEREK_ERR_BAD_ARG;
  }
  if (!h->scf_started) {
    h->last_error = "run the SCF first";
    return DEREK_ERR_BAD_ARG;
  }
  if (max_iter <= 0) max_iter = 60;
  if (!(tol > 0)) tol = 1e-9;
  const SysDev &S = h->sys[s];
  const long long nr = S.nr, np = h->total_psi;
  const int ni = h->nitems;
  cudaStream_t st = h->stream;
  const Tables &t = h->tab;
  Work W;
#define CKA(call)                                                    \
  do {                                                               \
    cudaError_t _e = (call);                                         \
    if (_e != cudaSuccess) return cuda_status(_e, h, #call);         \
  } while (0)
  CKA(dmalloc(&W.phi, np));
  CKA(dmalloc(&W.xi, np));
  CKA(dmalloc(&W.sp, np));
  CKA(dmalloc(&W.sm, np));
  CKA(dmalloc(&W.x, np));
  CKA(dmalloc(&W.r, np));
  CKA(dmalloc(&W.z, np));
  CKA(dmalloc(&W.p, np));
  CKA(dmalloc(&W.ap, np));
  for (double **q : {&W.w, &W.mask, &W.rz, &W.rz2, &W.pap, &W.alpha, &W.beta, &W.shift})
    CKA(dmalloc(q, ni));
  for (double **q : {&W.g, &W.fxc, &W.dn, &W.dv, &W.tmp, &W.nf, &W.dn_out}) CKA(dmalloc(q, nr));
  CKA(dmalloc(&W.vcoef, h->nks));
  // every system active for the duration (converged systems are masked off)
  std::vector<SysDev> saved(h->nsys), all = h->sys;
  CKA(cudaMemcpyAsync(saved.data(), h->d_sys, saved.size() * sizeof(SysDev), cudaMemcpyDeviceToHost, st));
  CKA(cudaStreamSynchronize(st));
  for (auto &x : all) x.active = 1;
  CKA(cudaMemcpyAsync(h->d_sys, all.data(), all.size() * sizeof(SysDev), cudaMemcpyHostToDevice, st));

  const double2 *psi = (const double2 *)h->cur_psi();
  const double dvol = S.volume / nr;
  // host copies of the ground state scalars
  std::vector<double> eig(ni), occ(ni), rho(nr), nt(n_target, n_target + nr);
  CKA(cudaMemcpyAsync(eig.data(), h->d_eig, ni * sizeof(double), cudaMemcpyDeviceToHost, st));
  CKA(cudaMemcpyAsync(occ.data(), h->d_occ, ni * sizeof(double), cudaMemcpyDeviceToHost, st));
  CKA(cudaMemcpyAsync(rho.data(), h->d_rho_out + S.grid_off, nr * sizeof(double), cudaMemcpyDeviceToHost, st));
  CKA(cudaStreamSynchronize(st));
  double L = 0;
  std::vector<double> g(nr);
  for (long long i = 0; i < nr; ++i) {
    const double d = rho[i] - nt[i];
    L += d * d;
    g[i] = 2.0 * d;
  }
  if (loss) *loss = L * dvol;
  CKA(cudaMemcpyAsync(W.g, g.data(), nr * sizeof(double), cudaMemcpyHostToDevice, st));
  launch_fxc(nr, h->d_rho_out + S.grid_off, W.fxc, st);

  // The split subspace M of each k-set: its leading bands whose Ritz
  // residual |(H - e_m) psi_m| is below kRitzConv, and at least every band
  // with occupation above 1e-12.  The pair sum over M and the Sternheimer
  // solve on its complement add up to the exact response only when M is an
  // invariant subspace; the top carried bands of an SCF are not converged
  // eigenvectors, so they go to the complement, where the Sternheimer solve
  // treats them with H itself.
  std::vector<double> shift(ni);
  for (int it = 0; it < ni; ++it) shift[it] = -eig[it];
  CKA(cudaMemcpyAsync(W.shift, shift.data(), ni * sizeof(double), cudaMemcpyHostToDevice, st));
  std::vector<double> rres(ni);
  {
    Tables ts = t;
    ts.item_shift = W.shift;
    int e0 = apply_h_items_ex(h, ts, 0, ni, psi, nullptr, W.ap, nullptr, h->d_vloc);
    if (e0) return e0;
    derek::note_launch(), k_item_dot<<<ni, 256, 0, st>>>(t, W.ap, W.ap, W.pap);
    CKA(cudaMemcpyAsync(rres.data(), W.pap, ni * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKA(cudaStreamSynchronize(st));
  }
  constexpr double kRitzConv = 1e-7;
  std::vector<int> nsplit(h->nks, 0);
  {
    std::vector<int> lead(h->nks, 0), last_occ(h->nks, -1);
    std::vector<char> broken(h->nks, 0);
    for (int it = 0; it < ni; ++it) {
      const int ksi = h->item_ks[it], b = h->item_band[it];
      if (!broken[ksi] && std::sqrt(rres[it]) < kRitzConv && b == lead[ksi]) ++lead[ksi];
      else if (b == lead[ksi]) broken[ksi] = 1;
      if (occ[it] > 1e-12) last_occ[ksi] = std::max(last_occ[ksi], b);
    }
    for (int k = 0; k < h->nks; ++k) nsplit[k] = std::max({lead[k], last_occ[k] + 1, 1});
  }
  std::vector<KSetDev> ks_split(h->ks);
  for (int k = 0; k < h->nks; ++k) ks_split[k].nb = nsplit[k];
  KSetDev *d_ks_split = nullptr;
  CKA(dmalloc(&d_ks_split, ks_split.size()));
  struct FreeKs {
    KSetDev *p;
    ~FreeKs() {
      if (p) cudaFree(p);
    }
  } free_ks{d_ks_split};
  CKA(cudaMemcpyAsync(d_ks_split, ks_split.data(), ks_split.size() * sizeof(KSetDev), cudaMemcpyHostToDevice, st));
  Tables tM = t;   // the split subspace: k-set tables with nb = |M|
  tM.ks = d_ks_split;

  // item weights (bands outside M take no pair or Sternheimer term)
  const double kT = S.kT;
  std::vector<double> w_pair(ni), w_stern(ni), w_fermi(ni), mask(ni);
  double fsum = 0;
  std::vector<double> fprime(ni);
  for (int it = 0; it < ni; ++it) {
    const KSetDev &K = h->ks[h->item_ks[it]];
    const bool inM = h->item_band[it] < nsplit[h->item_ks[it]];
    const double ft = 0.5 * occ[it];
    fprime[it] = -2.0 * ft * (1.0 - ft) / kT;
    w_pair[it] = inM ? 0.25 * K.wk / S.volume : 0.0;                  // (|psi+xi|^2 - |psi-xi|^2)/4
    w_stern[it] = inM ? 0.25 * 2.0 * occ[it] * K.wk / S.volume : 0.0;  // 2 f Re psi* x
    w_fermi[it] = fprime[it] * K.wk / S.volume;
    mask[it] = inM && occ[it] > 1e-12 ? 1.0 : 0.0;
    fsum += K.wk * fprime[it];
  }
  CKA(cudaMemcpyAsync(W.mask, mask.data(), ni * sizeof(double), cudaMemcpyHostToDevice, st));
  std::vector<Axpby> vc(h->nks, Axpby{1.0, 0.0, 0.0, 0.0});
  CKA(cudaMemcpyAsync(W.vcoef, vc.data(), vc.size() * sizeof(Axpby), cudaMemcpyHostToDevice, st));

  auto density_with = [&](const double2 *buf, const std::vector<double> &wts, double *out) -> int {
    CKA(cudaMemcpyAsync(h->d_occw, wts.data(), ni * sizeof(double), cudaMemcpyHostToDevice, st));
    int e = density_items(h, buf, out);
    return e;
  };
  auto cross_density = [&](const double2 *a, const double2 *b, const std::vector<double> &wts,
                           double *out) -> int {
    const int blocks = 152 * 8;
    derek::note_launch(), k_lincomb<<<blocks, 256, 0, st>>>(np, 1.0, a, 1.0, b, W.sp);
    derek::note_launch(), k_lincomb<<<blocks, 256, 0, st>>>(np, 1.0, a, -1.0, b, W.sm);
    int e = density_with(W.sp, wts, h->d_rho_in);  // scratch grid
    if (e) return e;
    derek::note_launch(), k_scale_grid<<<152, 256, 0, st>>>(nr, h->d_rho_in + S.grid_off, 1.0, nullptr, 0.0, W.tmp);
    e = density_with(W.sm, wts, h->d_rho_in);
    if (e) return e;
    derek::note_launch(), k_scale_grid<<<152, 256, 0, st>>>(nr, W.tmp, 1.0, h->d_rho_in + S.grid_off, -1.0, out);
    return 0;
  };
  // P_c y = y - Psi (Psi^H y)
  auto project = [&](double2 *y) {
    launch_overlap<double>(tM, 0, h->nks, h->max_nb, h->max_npw, h->tune.ksplit, psi, y, h->d_opart,
                           h->d_opart_off, h->d_S, h->d_mat_off, 0, st);
    const size_t sm = (size_t)h->max_nb * h->max_nb * sizeof(double2);
    cudaFuncSetAttribute(k_gemm_sub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    derek::note_launch(), k_gemm_sub<<<dim3((h->max_npw + 31) / 32, h->nks), 256, sm, st>>>(tM, psi, h->d_S, h->d_mat_off, y);
  };
  // Fermi-level density n_F (fixed for the whole solve); rho_in and the item
  // weights are used as scratch and restored at the end
  std::vector<double> occw_saved(ni);
  CKA(cudaMemcpyAsync(occw_saved.data(), h->d_occw, ni * sizeof(double), cudaMemcpyDeviceToHost, st));
  std::vector<double> rho_in_saved(nr);
  CKA(cudaMemcpyAsync(rho_in_saved.data(), h->d_rho_in + S.grid_off, nr * sizeof(double), cudaMemcpyDeviceToHost, st));
  int e = density_with(psi, w_fermi, h->d_rho_in);
  if (e) return e;
  CKA(cudaMemcpyAsync(W.nf, h->d_rho_in + S.grid_off, nr * sizeof(double), cudaMemcpyDeviceToDevice, st));

  // Anderson mixing state (host)
  const int hist = 8;
  std::vector<std::vector<double>> Xin, Res;
  std::vector<double> dn(nr, 0.0), dn_out(nr), vnn(ni);
  int status = DEREK_OK;
  bool converged = false;
  for (int iter = 0; iter < max_iter && !converged; ++iter) {
    CKA(cudaMemcpyAsync(W.dn, dn.data(), nr * sizeof(double), cudaMemcpyHostToDevice, st));
    launch_hartree_only(t, 1, (int)nr, h->max_nmax, W.dn, h->d_cgrid, st);
    derek::note_launch(), k_response_potential<<<152, 256, 0, st>>>(nr, W.g, h->d_cgrid, W.fxc, W.dn, W.dv);
    // phi = dV psi
    {
      int e2 = apply_h_items_ex(h, t, 0, ni, psi, nullptr, W.phi, W.vcoef, W.dv);
      if (e2) return e2;
    }
    // V_mn and the pair orbitals xi = psi W
    launch_overlap<double>(tM, 0, h->nks, h->max_nb, h->max_npw, h->tune.ksplit, psi, W.phi, h->d_opart,
                           h->d_opart_off, h->d_Hs, h->d_mat_off, 1, st);
    derek::note_launch(), k_pair_weights<<<h->nks, 256, 0, st>>>(tM, h->d_eig, h->d_occ, h->d_Hs, h->d_mat_off, h->d_C);
    CKA(cudaMemcpyAsync(W.xi, psi, np * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    launch_rotate<double>(tM, 0, h->nks, h->max_nb, h->max_npw, W.xi, h->d_C, h->d_mat_off, st);
    e = cross_density(psi, W.xi, w_pair, W.dn_out);
    if (e) return e;
    // diagonal V_nn for the Fermi shift
    {
      std::vector<double2> vm(h->mat_off.back() + (long long)h->ks.back().nb * h->ks.back().nb);
      CKA(cudaMemcpyAsync(vm.data(), h->d_Hs, vm.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
      CKA(cudaStreamSynchronize(st));
      for (int it = 0; it < ni; ++it) {
        const int ksi = h->item_ks[it], b = h->item_band[it];
        vnn[it] = b < nsplit[ksi] ? vm[h->mat_off[ksi] + (long long)b * nsplit[ksi] + b].x : 0.0;
      }
    }
    double dmu_num = 0;
    for (int it = 0; it < ni; ++it) dmu_num += h->ks[h->item_ks[it]].wk * fprime[it] * vnn[it];
    const double dmu = fsum != 0 ? dmu_num / fsum : 0.0;
    // Sternheimer: b = -P_c phi on occupied bands; CG for (H - e_n) x = b on P_c
    CKA(cudaMemcpyAsync(W.r, W.phi, np * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    project(W.r);
    {
      // r = -mask * P_c phi  (k_precond with unit scaling is not a copy; do it explicitly)
      std::vector<double> negmask(ni);
      for (int it = 0; it < ni; ++it) negmask[it] = -mask[it];
      CKA(cudaMemcpyAsync(W.alpha, negmask.data(), ni * sizeof(double), cudaMemcpyHostToDevice, st));
      CKA(cudaMemsetAsync(W.x, 0, np * sizeof(double2), st));
      // x = 0 + (-mask) * r  -> x holds b; then r = b
      derek::note_launch(), k_item_axpy<<<ni, 256, 0, st>>>(t, W.alpha, 1.0, W.r, W.x, 0);
      CKA(cudaMemcpyAsync(W.r, W.x, np * sizeof(double2), cudaMemcpyDeviceToDevice, st));
      CKA(cudaMemsetAsync(W.x, 0, np * sizeof(double2), st));
    }
    derek::note_launch(), k_item_dot<<<ni, 256, 0, st>>>(t, W.r, W.r, W.rz2);  // |b|^2
    std::vector<double> bnorm(ni), rnorm(ni);
    CKA(cudaMemcpyAsync(bnorm.data(), W.rz2, ni * sizeof(double), cudaMemcpyDeviceToHost, st));
    derek::note_launch(), k_precond<<<ni, 256, 0, st>>>(t, W.r, W.mask, W.z);
    project(W.z);
    CKA(cudaMemcpyAsync(W.p, W.z, np * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    derek::note_launch(), k_item_dot<<<ni, 256, 0, st>>>(t, W.r, W.z, W.rz);
    const double cg_tol = std::max(std::min(1e-6, tol * 0.1), 1e-12);
    for (int cg = 0; cg < 200; ++cg) {
      // ap = P_c (H - e_n) p
      {
        Tables ts = t;
        ts.item_shift = W.shift;
        int e2 = apply_h_items_ex(h, ts, 0, ni, W.p, nullptr, W.ap, nullptr, h->d_vloc);
        if (e2) return e2;
      }
      project(W.ap);
      derek::note_launch(), k_item_dot<<<ni, 256, 0, st>>>(t, W.p, W.ap, W.pap);
      derek::note_launch(), k_cg_ratio<<<(ni + 127) / 128, 128, 0, st>>>(ni, W.rz, W.pap, W.mask, W.alpha);
      derek::note_launch(), k_item_axpy<<<ni, 256, 0, st>>>(t, W.alpha, 1.0, W.p, W.x, 0);
      derek::note_launch(), k_item_axpy<<<ni, 256, 0, st>>>(t, W.alpha, -1.0, W.ap, W.r, 0);
      derek::note_launch(), k_item_dot<<<ni, 256, 0, st>>>(t, W.r, W.r, W.pap);
      CKA(cudaMemcpyAsync(rnorm.data(), W.pap, ni * sizeof(double), cudaMemcpyDeviceToHost, st));
      CKA(cudaStreamSynchronize(st));
      bool done = true;
      for (int it = 0; it < ni; ++it)
        if (mask[it] != 0.0 && rnorm[it] > cg_tol * cg_tol * std::max(bnorm[it], 1e-300)) done = false;
      if (done) break;
      derek::note_launch(), k_precond<<<ni, 256, 0, st>>>(t, W.r, W.mask, W.z);
      project(W.z);
      derek::note_launch(), k_item_dot<<<ni, 256, 0, st>>>(t, W.r, W.z, W.rz2);
      derek::note_launch(), k_cg_ratio<<<(ni + 127) / 128, 128, 0, st>>>(ni, W.rz2, W.rz, W.mask, W.beta);
      derek::note_launch(), k_item_axpy<<<ni, 256, 0, st>>>(t, W.beta, 1.0, W.z, W.p, 1);
      std::swap(W.rz, W.rz2);
    }
    e = cross_density(psi, W.x, w_stern, W.tmp);
    if (e) return e;
    // dn_out = pair + Sternheimer - dmu n_F
    derek::note_launch(), k_scale_grid<<<152, 256, 0, st>>>(nr, W.dn_out, 1.0, W.tmp, 1.0, W.dn_out);
    derek::note_launch(), k_scale_grid<<<152, 256, 0, st>>>(nr, W.dn_out, 1.0, W.nf, -dmu, W.dn_out);
    CKA(cudaMemcpyAsync(dn_out.data(), W.dn_out, nr * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKA(cudaStreamSynchronize(st));
    // convergence and Anderson update on the host
    std::vector<double> res(nr);
    double rn = 0, on = 0;
    for (long long i = 0; i < nr; ++i) {
      res[i] = dn_out[i] - dn[i];
      rn += res[i] * res[i];
      on += dn_out[i] * dn_out[i];
    }
    if (rn <= tol * tol * std::max(on, 1e-300)) {
      converged = true;
      break;
    }
    Xin.push_back(dn);
    Res.push_back(res);
    if ((int)Xin.size() > hist) {
      Xin.erase(Xin.begin());
      Res.erase(Res.begin());
    }
    const int m = (int)Res.size();
    std::vector<double> A((m + 1) * (m + 1), 0.0), rhs(m + 1, 0.0);
    for (int i = 0; i < m; ++i) {
      for (int j = 0; j < m; ++j) {
        double q = 0;
        for (long long r = 0; r < nr; ++r) q += Res[i][r] * Res[j][r];
        A[i * (m + 1) + j] = q;
      }
      A[i * (m + 1) + m] = 1.0;
      A[m * (m + 1) + i] = 1.0;
    }
    rhs[m] = 1.0;
    // Gaussian elimination with partial pivoting
    std::vector<double> c(m + 1, 0.0);
    {
      const int N = m + 1;
      std::vector<double> M = A, b = rhs;
      bool ok = true;
      for (int col = 0; col < N && ok; ++col) {
        int piv = col;
        for (int rr = col + 1; rr < N; ++rr)
          if (std::fabs(M[rr * N + col]) > std::fabs(M[piv * N + col])) piv = rr;
        if (std::fabs(M[piv * N + col]) < 1e-300) {
          ok = false;
          break;
        }
        if (piv != col) {
          for (int j = 0; j < N; ++j) std::swap(M[col * N + j], M[piv * N + j]);
          std::swap(b[col], b[piv]);
        }
        for (int rr = col + 1; rr < N; ++rr) {
          const double f = M[rr * N + col] / M[col * N + col];
          for (int j = col; j < N; ++j) M[rr * N + j] -= f * M[col * N + j];
          b[rr] -= f * b[col];
        }
      }
      if (ok) {
        for (int rr = N - 1; rr >= 0; --rr) {
          double v = b[rr];
          for (int j = rr + 1; j < N; ++j) v -= M[rr * N + j] * c[j];
          c[rr] = v / M[rr * N + rr];
        }
      } else {
        std::fill(c.begin(), c.end(), 0.0);
        c[m - 1] = 1.0;
      }
    }
    const double beta_mix = 0.5;
    for (long long r = 0; r < nr; ++r) {
      double a = 0, b = 0;
      for (int i = 0; i < m; ++i) {
        a += c[i] * Xin[i][r];
        b += c[i] * Res[i][r];
      }
      dn[r] = a + beta_mix * b;
    }
  }
  if (!converged) status = DEREK_ERR_NOT_CONVERGED;
  // gradient: dV sum u dV_ext/dp with u = dn_out
  CKA(cudaMemcpyAsync(W.dn_out, dn_out.data(), nr * sizeof(double), cudaMemcpyHostToDevice, st));
  // the Hellmann-Feynman kernel reads a grid at grid_off; the handle has one system
  launch_hf_gradient(t, h->nsys, W.dn_out - S.grid_off, h->d_wells, h->d_well_off, h->d_cells,
                     h->d_hfpart, h->max_wells, h->d_hfgrad, st);
  CKA(cudaMemcpyAsync(grad, h->d_hfgrad + 5 * h->well_off[s], (size_t)nw * 5 * sizeof(double),
                      cudaMemcpyDeviceToHost, st));
  // restore scratch grids and the active flags
  CKA(cudaMemcpyAsync(h->d_rho_in + S.grid_off, rho_in_saved.data(), nr * sizeof(double), cudaMemcpyHostToDevice, st));
  CKA(cudaMemcpyAsync(h->d_occw, occw_saved.data(), ni * sizeof(double), cudaMemcpyHostToDevice, st));
  CKA(cudaMemcpyAsync(h->d_sys, saved.data(), saved.size() * sizeof(SysDev), cudaMemcpyHostToDevice, st));
  CKA(cudaStreamSynchronize(st));
  CKA(cudaGetLastError());
#undef CKA
  return status;
}
