// SCF driver: Chebyshev-filtered subspace iteration inside a self-consistent
// density loop, batched over every k-point and every system of the handle.
//
// The reference's electronic_scf (Source/electronic.f90:86-175) loops until
// |E - E_prev| < energy_tol but never builds a Hamiltonian.  One iteration
// here is
//   filter    Y = p_m(H) X             (m fused H.psi applications)
//   CholQR    S = Y^H Y = L L^H, X = Y L^-H
//   RR        Hs = X^H H X = U diag(e) U^H (Jacobi), X <- X U
//   occupations (Fermi-Dirac), n_out(r), energies of n_out, |dF| test
//   Pulay (+Kerker) mixing -> n_in, V_loc = V_ext + V_H[n_in] + v_xc[n_in]
// with every scalar kept on the device, so a steady-state iteration is one
// CUDA graph launch followed by a small state read-back.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "handle.h"
#include "scf_kernels.cuh"

using namespace derek;

namespace {

template <typename T> cudaError_t dalloc(T **p, size_t n) {
  return cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T));
}

}  // namespace

// -- pieces of an iteration -------------------------------------------------
namespace derek {

// the tensor-core kernels serve complex64 scalar bands, nb <= 128, when the
// options allow them: use_tensor_cores 1 (overlaps) or 2 (overlaps and
// rotations) at any subspace size, -1 (the default) overlaps and rotations
// for subspaces of kTcMinBands or more carried bands
bool tc_capable(const derek_gpu *h) {
  if (h->prec != DEREK_PREC_MIXED || !h->opts.use_tensor_cores || h->max_nb > kMaxBands || h->any_spinor)
    return false;
  return h->opts.use_tensor_cores > 0 || h->max_nb_band >= kTcMinBands;
}
bool use_tc_overlap(const derek_gpu *h) {
  return tc_capable(h) && (h->tune.overlap_tc >= 0 ? h->tune.overlap_tc == 1 : true);
}
bool use_tc_rotate(const derek_gpu *h) {
  return tc_capable(h) && h->opts.use_tensor_cores != 1 &&
         (h->tune.rotate_tc >= 0 ? h->tune.rotate_tc == 1 : true);
}

int overlap_all(derek_gpu *h, const void *A, const void *B, double2 *out, int hermitize) {
  const int ks = h->tune.ksplit;
  if (use_tc_overlap(h))
    launch_overlap_tc(h->tab_band, 0, h->nks, h->max_nb_band, h->max_npw_band, ks, (const float2 *)A,
                      (const float2 *)B, h->d_opart, h->d_opart_off, out, h->d_mat_off, hermitize,
                      h->d_status, h->stream);
  else if (h->prec == DEREK_PREC_FP64)
    launch_overlap<double>(h->tab_band, 0, h->nks, h->max_nb_band, h->max_npw_band, ks,
                           (const double2 *)A, (const double2 *)B, h->d_opart, h->d_opart_off, out,
                           h->d_mat_off, hermitize, h->stream);
  else
    launch_overlap<float>(h->tab_band, 0, h->nks, h->max_nb_band, h->max_npw_band, ks,
                          (const float2 *)A, (const float2 *)B, h->d_opart, h->d_opart_off, out,
                          h->d_mat_off, hermitize, h->stream);
  return DEREK_OK;
}

int rotate_all(derek_gpu *h, void *X, const double2 *C) {
  if (use_tc_rotate(h))
    launch_rotate_tc(h->tab_band, 0, h->nks, h->max_nb_band, h->max_npw_band, (float2 *)X, C, h->d_mat_off,
                     h->d_rot_img, h->d_status, h->stream);
  else if (h->prec == DEREK_PREC_FP64)
    launch_rotate<double>(h->tab_band, 0, h->nks, h->max_nb_band, h->max_npw_band, (double2 *)X, C, h->d_mat_off,
                          h->stream);
  else
    launch_rotate<float>(h->tab_band, 0, h->nks, h->max_nb_band, h->max_npw_band, (float2 *)X, C, h->d_mat_off,
                         h->stream);
  return DEREK_OK;
}

}  // namespace derek

namespace {

// orthonormalise buf(cur) and do Rayleigh-Ritz; leaves Ritz values in d_eig
int cholqr_rr(derek_gpu *h) {
  void *X = h->cur_psi();
  overlap_all(h, X, X, h->d_S, 1);
  launch_cholesky_inv(h->tab_band, 0, h->nks, h->max_nb_band, h->d_S, h->d_C, h->d_mat_off, h->d_scratch,
                      h->d_status, h->stream);
  rotate_all(h, X, h->d_C);
  int st = apply_h_items(h, 0, h->nitems, X, nullptr, h->d_HX, nullptr);
  if (st) return st;
  overlap_all(h, X, h->d_HX, h->d_Hs, 1);
  // Off-diagonal Frobenius target relative to ||Hs||: 1e-14 on the FP64 path;
  // on the mixed path Hs itself carries the FP32 H.psi error (~1e-7
  // relative), so 1e-10 leaves eigenvalue errors of order 1e-20 / gap while
  // saving about one of the four sweeps near convergence.
  const double jtol = h->prec == DEREK_PREC_FP64 ? 1e-14 : 1e-10;
  launch_jacobi(h->tab_band, 0, h->nks, h->max_nb_band, h->d_Hs, h->d_C, h->d_mat_off, h->d_eig,
                h->d_scratch, 30, jtol, 0, h->d_sweeps, h->stream, h->tune.jacobi_single);
  rotate_all(h, X, h->d_C);
  return DEREK_OK;
}

int filter(derek_gpu *h, int m) {
  launch_filter_coef(h->tab_band, h->nks, h->d_eig, h->d_state, h->d_coef_all, m, h->stream);
  int in = h->cur, prev = -1;
  for (int i = 0; i < m; ++i) {
    const int out = prev < 0 ? (in + 1) % 3 : 3 - in - prev;
    int st = apply_h_items(h, 0, h->nitems, h->buf(in), prev < 0 ? nullptr : h->buf(prev),
                           h->buf(out), h->d_coef_all + (size_t)i * h->nks);
    if (st) return st;
    prev = in;
    in = out;
  }
  h->cur = in;
  return DEREK_OK;
}

int subspace_step(derek_gpu *h, int m) {
  int st = filter(h, m);
  if (st) return st;
  return cholqr_rr(h);
}

// the non-collinear SCF's grids (on = 0 for scalar batches)
SpinGrids spin_grids(const derek_gpu *h) {
  SpinGrids g{};
  g.on = h->all_spinor && h->d_mag_in != nullptr;
  if (!g.on) return g;
  g.tg = h->total_grid;
  g.vnc_ext = h->d_vnc_ext;
  g.mag_in = h->d_mag_in;
  g.mag_out = h->d_mag;
  g.bxc = h->d_bxc;
  g.vnc64 = h->d_vnc64;
  g.vnc32 = h->prec == DEREK_PREC_FP64 ? nullptr : h->d_vnc32;
  g.min_hist = h->d_min_hist;
  g.mres_hist = h->d_mres_hist;
  return g;
}

// a batch mixing spinor and scalar systems runs no SCF
bool reject_mixed(derek_gpu *h, const char *what) {
  if (!h->any_spinor || h->all_spinor) return false;
  h->last_error = std::string(what) + ": a batch mixing spinor and scalar systems";
  return true;
}

int finish_iteration(derek_gpu *h) {
  const SpinGrids sg = spin_grids(h);
  launch_occupations(h->tab_band, h->nsys, h->d_eig, h->d_occ, h->d_occw, h->d_state, h->stream);
  int st = sg.on ? density_spinor_items(h, h->cur_psi(), h->d_rho_out)
                 : density_items(h, h->cur_psi(), h->d_rho_out);
  if (st) return st;
  launch_density_fft(h->tab, h->nsys, (int)h->max_nr, h->max_nmax, h->d_rho_out, h->d_cgrid,
                     h->stream);
  launch_energies(h->tab, h->nsys, h->d_vhxc, h->d_rho_in, h->d_rho_out, h->d_cgrid, h->d_epart, h->d_state,
                  h->d_sys, h->d_status, sg, h->stream);
  launch_mix(h->tab, h->nsys, (int)h->max_nr, h->d_rho_in, h->d_rho_out, h->d_nin_hist,
             h->d_res_hist, h->d_hist_off, h->d_state, h->hist, h->d_gpart, h->d_cgrid,
             h->opts.mix_alpha, h->opts.kerker_q0, h->max_nmax, sg, h->stream);
  launch_potential(h->tab, h->nsys, (int)h->max_nr, h->max_nmax, h->d_rho_in, h->d_cgrid,
                   h->d_vext, h->d_vhxc, h->d_vloc, h->prec == DEREK_PREC_FP64 ? nullptr : h->d_vloc32,
                   h->d_epart, h->d_state, 0, sg, h->stream);
  DEREK_CUDA(h, cudaGetLastError());
  return DEREK_OK;
}

void drop_graphs(derek_gpu *h) {
  for (auto &g : h->graph_exec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

// back to the full work lists; true when some class had a compacted one
bool reset_lists(derek_gpu *h) {
  bool any = false;
  for (const auto &c : h->classes) any |= c.active_count >= 0;
  reset_classes(h);
  return any;
}

// Once the still-active systems hold at most 60 % of the items the H.psi
// and density passes launch over, those passes get lists of the active
// systems' items only (the graphs captured with the longer lists are
// dropped and recaptured): a converged system's items otherwise still cost
// their blocks' exits and the plane pass's per-tile barriers every iteration.
void maybe_compact(derek_gpu *h, const std::vector<SysState> &st) {
  std::vector<int> act(h->nsys);
  for (int s = 0; s < h->nsys; ++s) act[s] = !st[s].converged && !st[s].status;
  long long live = 0, launched = 0;
  for (int it = 0; it < h->nitems; ++it) live += act[h->ks[h->item_ks[it]].sys];
  for (const auto &c : h->classes) launched += c.launch_count();
  if (live > 0 && live * 10 <= launched * 6 && compact_classes(h, act)) drop_graphs(h);
}

// Start vectors in buf(cur): hashed entries (init_vectors 0) or plane waves
// (1) in X; with 2 the wavefunctions stored by set_wfn (a restart from a
// saved state) keep their bands and the buffer bands get plane-wave start
// vectors.
int start_vectors(derek_gpu *h) {
  const int init = h->opts.init_vectors;
  const int *pw = init >= 1 ? h->d_pw_entry : nullptr;
  const int dst = init == 2 ? (h->cur + 1) % 3 : 0;
  if (h->prec == DEREK_PREC_FP64)
    launch_init_psi<double>(h->tab, h->nitems, h->buf(dst), h->opts.seed, pw, h->stream);
  else
    launch_init_psi<float>(h->tab, h->nitems, h->buf(dst), h->opts.seed, pw, h->stream);
  if (init == 2) {
    // the reported bands of a k-set are its first nbr rows of npw_pad coefficients
    const size_t es = h->elem_size();
    for (const auto &K : h->ks)
      DEREK_CUDA(h, cudaMemcpyAsync((char *)h->buf(dst) + (size_t)K.psi_off * es,
                                    (const char *)h->cur_psi() + (size_t)K.psi_off * es,
                                    (size_t)K.nbr * K.npw_pad * es, cudaMemcpyDeviceToDevice, h->stream));
  }
  h->cur = dst;
  DEREK_CUDA(h, cudaGetLastError());
  return DEREK_OK;
}

int scf_start(derek_gpu *h, double etol) {
  // reset state: all systems active, uniform start density, start vectors
  for (auto &s : h->sys) s.active = 1;
  if (reset_lists(h)) drop_graphs(h);
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_sys, h->sys.data(), h->sys.size() * sizeof(SysDev),
                                cudaMemcpyHostToDevice, h->stream));
  std::vector<SysState> st(h->nsys);
  for (int s = 0; s < h->nsys; ++s) {
    SysState &x = st[s];
    std::memset(&x, 0, sizeof(x));
    x.slot = -1;
    x.etol = h->opts.etol_per_electron ? etol * h->sys[s].nelec : etol;
    x.rtol = h->opts.density_tol;
    x.free = 0.0;
  }
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_state, st.data(), st.size() * sizeof(SysState),
                                cudaMemcpyHostToDevice, h->stream));
  DEREK_CUDA(h, cudaMemsetAsync(h->d_status, 0, h->nks * sizeof(int), h->stream));
  launch_uniform_density(h->tab, h->nsys, (int)h->max_nr, h->d_rho_in, h->stream);
  for (int s = 0; s < h->nsys && s < (int)h->start_rho.size(); ++s)
    if (!h->start_rho[s].empty())
      DEREK_CUDA(h, cudaMemcpyAsync(h->d_rho_in + h->sys[s].grid_off, h->start_rho[s].data(),
                                    h->start_rho[s].size() * sizeof(double), cudaMemcpyHostToDevice,
                                    h->stream));
  const SpinGrids sg = spin_grids(h);
  if (sg.on) {
    DEREK_CUDA(h, cudaMemsetAsync(h->d_mag_in, 0, 3 * (size_t)h->total_grid * sizeof(double), h->stream));
    for (int s = 0; s < h->nsys && s < (int)h->start_mag.size(); ++s)
      if (!h->start_mag[s].empty())
        for (int c = 0; c < 3; ++c)
          DEREK_CUDA(h, cudaMemcpyAsync(h->d_mag_in + c * h->total_grid + h->sys[s].grid_off,
                                        h->start_mag[s].data() + (size_t)c * h->sys[s].nr,
                                        (size_t)h->sys[s].nr * sizeof(double), cudaMemcpyHostToDevice,
                                        h->stream));
  }
  launch_potential(h->tab, h->nsys, (int)h->max_nr, h->max_nmax, h->d_rho_in, h->d_cgrid,
                   h->d_vext, h->d_vhxc, h->d_vloc, h->prec == DEREK_PREC_FP64 ? nullptr : h->d_vloc32,
                   h->d_epart, h->d_state, 1, sg, h->stream);
  int s = start_vectors(h);
  if (s) return s;
  s = cholqr_rr(h);
  if (s) return s;
  for (int p = 0; p < h->opts.first_passes; ++p) {
    s = subspace_step(h, h->opts.first_degree);
    if (s) return s;
  }
  h->scf_started = true;
  return DEREK_OK;
}

int steady_iteration(derek_gpu *h) {
  const int m = h->opts.cheb_degree;
  if (!h->opts.use_graph) {
    int s = subspace_step(h, m);
    if (s) return s;
    return finish_iteration(h);
  }
  if (h->graph_degree != m) {
    for (auto &g : h->graph_exec)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
    h->graph_degree = m;
  }
  const int start = h->cur;
  if (!h->graph_exec[start]) {
    cudaGraph_t g = nullptr;
    const unsigned long long before = launch_total();
    DEREK_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int s = subspace_step(h, m);
    if (!s) s = finish_iteration(h);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    // captured launches run only when the graph is replayed
    note_launch(-(long long)(launch_total() - before));
    if (s) {
      if (g) cudaGraphDestroy(g);
      return s;
    }
    if (e != cudaSuccess) return cuda_status(e, h, "graph capture");
    size_t nodes = 0;
    cudaGraphGetNodes(g, nullptr, &nodes);
    h->graph_nodes[start] = (long long)nodes;
    e = cudaGraphInstantiate(&h->graph_exec[start], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_status(e, h, "graph instantiate");
  }
  DEREK_CUDA(h, cudaGraphLaunch(h->graph_exec[start], h->stream));
  note_launch(h->graph_nodes[start]);
  h->cur = (start + m) % 3;
  return DEREK_OK;
}

void fill_reports(derek_gpu *h, const std::vector<SysState> &st, derek_scf_report *rep) {
  if (!rep) return;
  for (int s = 0; s < h->nsys; ++s) {
    const SysState &x = st[s];
    derek_scf_report &r = rep[s];
    r.energy = x.energy;
    r.free_energy = x.free;
    r.delta = x.delta;
    r.efermi = x.mu;
    r.entropy = x.entropy;
    r.e_band = x.e_band;
    r.e_hartree = x.e_h;
    r.e_xc = x.e_xc;
    r.e_dc = x.e_dc;
    r.residual = x.resid;
    r.iterations = x.iter;
    r.converged = x.converged;
  }
}

int read_state(derek_gpu *h, std::vector<SysState> &st) {
  st.resize(h->nsys);
  DEREK_CUDA(h, cudaMemcpyAsync(st.data(), h->d_state, st.size() * sizeof(SysState),
                                cudaMemcpyDeviceToHost, h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

int one_iteration(derek_gpu *h, double etol) {
  int s;
  if (!h->scf_started) {
    s = scf_start(h, etol);
    if (s) return s;
    s = finish_iteration(h);
  } else {
    s = steady_iteration(h);
  }
  return s;
}

}  // namespace

extern "C" int derek_scf_alloc(derek_gpu_t *h) {
  h->hist = std::max(1, std::min(h->opts.pulay_history, kMaxHist));
  h->max_degree = std::max({h->opts.cheb_degree, h->opts.first_degree, 1});
  if (h->max_nb > kMaxBands) {
    h->last_error = "more than 128 bands per k-point";
    return DEREK_ERR_UNSUPPORTED;
  }
  long long moff = 0, poff = 0;
  std::vector<long long> opart_off;
  for (const auto &K : h->ks) {
    h->mat_off.push_back(moff);
    moff += (long long)K.nb * K.nb;
    opart_off.push_back(poff);
    poff += (long long)((K.npw + kOverlapSplitMin - 1) / kOverlapSplitMin) * K.nb * K.nb;
    h->max_npw = std::max(h->max_npw, K.npw);
  }
  for (const auto &K : h->ks_band) {
    h->max_nb_band = std::max(h->max_nb_band, K.nb);
    h->max_npw_band = std::max(h->max_npw_band, K.npw);
  }
  std::vector<long long> hist_off;
  long long hoff = 0;
  for (const auto &S : h->sys) {
    hist_off.push_back(hoff);
    hoff += (long long)h->hist * S.nr;
    h->max_nr = std::max<long long>(h->max_nr, S.nr);
  }
  cudaError_t e;
#define A(call)                                                  \
  if ((e = (call)) != cudaSuccess) return cuda_status(e, h, #call);
  A(dalloc(&h->d_state, h->nsys));
  A(dalloc(&h->d_S, moff));
  A(dalloc(&h->d_Hs, moff));
  A(dalloc(&h->d_C, moff));
  A(dalloc(&h->d_scratch, 2 * moff));
  A(dalloc(&h->d_opart, poff));
  A(dalloc(&h->d_mat_off, h->mat_off.size()));
  A(dalloc(&h->d_opart_off, opart_off.size()));
  A(dalloc(&h->d_hist_off, hist_off.size()));
  A(dalloc(&h->d_status, h->nks));
  A(dalloc(&h->d_sweeps, h->nks));
  if (tc_capable(h)) A(dalloc(&h->d_rot_img, h->nks * rotate_tc_image_bytes(h->max_nb)));
  A(dalloc(&h->d_coef_all, (size_t)h->max_degree * h->nks));
  A(dalloc(&h->d_nin_hist, hoff));
  A(dalloc(&h->d_res_hist, hoff));
  A(dalloc(&h->d_epart, (size_t)h->nsys * 64 * 8));
  A(dalloc(&h->d_gpart, (size_t)h->nsys * 64 * kMaxHist));
  if (h->all_spinor) {
    A(dalloc(&h->d_mag_in, 3 * (size_t)h->total_grid));
    A(dalloc(&h->d_bxc, 3 * (size_t)h->total_grid));
    A(dalloc(&h->d_min_hist, 3 * (size_t)hoff));
    A(dalloc(&h->d_mres_hist, 3 * (size_t)hoff));
    A(cudaMemset(h->d_mag_in, 0, 3 * (size_t)h->total_grid * sizeof(double)));
    A(cudaMemset(h->d_bxc, 0, 3 * (size_t)h->total_grid * sizeof(double)));
  }
  A(cudaMemcpy(h->d_mat_off, h->mat_off.data(), h->mat_off.size() * sizeof(long long),
               cudaMemcpyHostToDevice));
  A(cudaMemcpy(h->d_opart_off, opart_off.data(), opart_off.size() * sizeof(long long),
               cudaMemcpyHostToDevice));
  A(cudaMemcpy(h->d_hist_off, hist_off.data(), hist_off.size() * sizeof(long long),
               cudaMemcpyHostToDevice));
  A(cudaMemset(h->d_status, 0, h->nks * sizeof(int)));
  A(cudaMemset(h->d_state, 0, h->nsys * sizeof(SysState)));
#undef A
  return DEREK_OK;
}

extern "C" void derek_scf_free(derek_gpu_t *h) {
  for (auto &g : h->graph_exec)
    if (g) cudaGraphExecDestroy(g);
  void *ptrs[] = {h->d_state,  h->d_S,      h->d_Hs,       h->d_C,        h->d_scratch,
                  h->d_opart,  h->d_mat_off, h->d_opart_off, h->d_hist_off, h->d_status,
                  h->d_sweeps, h->d_coef_all, h->d_nin_hist, h->d_res_hist, h->d_epart,
                  h->d_gpart,  h->d_rot_img, h->d_mag_in, h->d_bxc, h->d_min_hist, h->d_mres_hist};
  for (void *p : ptrs)
    if (p) cudaFree(p);
}

extern "C" {

int derek_gpu_overlap(derek_gpu_t *h, int s, int k, double *out) {
  if (!h || s < 0 || s >= h->nsys || k < 0 || k >= h->sys[s].nk || !out) return DEREK_ERR_BAD_ARG;
  if (int st = activate_all(h)) return st;   // an SCF leaves converged systems masked off
  const int ki = h->sys[s].ks0 + k;
  const KSetDev &K = h->ks[ki];
  if (h->sys[s].nspinor == 2) {
    // a spinor band is one contiguous run of 2 npw_pad coefficients (up, then
    // down, zero padded), so the overlap summed over spinors (wave_dot_wfn,
    // Source/wave.f90:955) is the scalar overlap of nb / 2 such rows
    const int nb = K.nb / 2, nbr = K.nbr / 2;
    const long ld = 2L * K.npw_pad;
    const char *x = (const char *)h->cur_psi() + (size_t)K.psi_off * h->elem_size();
    int st = derek_gpu_overlap_noalloc(x, x, nb, (int)ld, ld, h->prec, h->d_S + h->mat_off[ki], h->stream);
    if (st) {
      if (st == DEREK_ERR_UNSUPPORTED) h->last_error = "overlap: spinor bands need nb <= 128 and 2 npw_pad <= 65536";
      return st;
    }
    DEREK_CUDA(h, cudaMemcpy2DAsync(out, (size_t)nbr * sizeof(double2), h->d_S + h->mat_off[ki],
                                    (size_t)nb * sizeof(double2), (size_t)nbr * sizeof(double2), nbr,
                                    cudaMemcpyDeviceToHost, h->stream));
    DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
    return DEREK_OK;
  }
  if (use_tc_overlap(h)) {
    DEREK_CUDA(h, cudaMemsetAsync(h->d_status + ki, 0, sizeof(int), h->stream));
    launch_overlap_tc(h->tab, ki, 1, K.nb, K.npw, h->tune.ksplit, (const float2 *)h->cur_psi(),
                      (const float2 *)h->cur_psi(), h->d_opart, h->d_opart_off, h->d_S, h->d_mat_off,
                      0, h->d_status, h->stream);
    int ks_status = 0;
    DEREK_CUDA(h, cudaMemcpyAsync(&ks_status, h->d_status + ki, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (ks_status) {
      // a bounded wait ran out: the CTA gave up, drained its own MMAs and
      // freed its tensor memory; the handle stays usable
      DEREK_CUDA(h, cudaMemsetAsync(h->d_status + ki, 0, sizeof(int), h->stream));
      h->last_error = "overlap: tensor-core pipeline wait timed out";
      return ks_status;
    }
  }
  else if (h->prec == DEREK_PREC_FP64)
    launch_overlap<double>(h->tab, ki, 1, K.nb, K.npw, h->tune.ksplit, (const double2 *)h->cur_psi(),
                           (const double2 *)h->cur_psi(), h->d_opart, h->d_opart_off, h->d_S,
                           h->d_mat_off, 0, h->stream);
  else
    launch_overlap<float>(h->tab, ki, 1, K.nb, K.npw, h->tune.ksplit, (const float2 *)h->cur_psi(),
                          (const float2 *)h->cur_psi(), h->d_opart, h->d_opart_off, h->d_S,
                          h->d_mat_off, 0, h->stream);
  DEREK_CUDA(h, cudaGetLastError());
  // leading nbr x nbr block of the nb x nb matrix
  DEREK_CUDA(h, cudaMemcpy2DAsync(out, (size_t)K.nbr * sizeof(double2), h->d_S + h->mat_off[ki],
                                  (size_t)K.nb * sizeof(double2), (size_t)K.nbr * sizeof(double2),
                                  K.nbr, cudaMemcpyDeviceToHost, h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

int derek_gpu_set_wait_limit(long iterations) { return set_stage_wait_limit(iterations); }

int derek_gpu_scf_iterate(derek_gpu_t *h, derek_scf_report *rep) {
  if (!h) return DEREK_ERR_BAD_ARG;
  if (reject_mixed(h, "scf_iterate")) return DEREK_ERR_UNSUPPORTED;
  int s = one_iteration(h, 0.0);
  if (s) return s;
  std::vector<SysState> st;
  s = read_state(h, st);
  if (s) return s;
  fill_reports(h, st, rep);
  for (const auto &x : st)
    if (x.status) return x.status;
  return DEREK_OK;
}

int derek_gpu_nscf_run(derek_gpu_t *h, int max_iter, double eig_tol, int nconv, int *iterations) {
  if (!h || max_iter <= 0 || !(eig_tol > 0) || nconv < 0) return DEREK_ERR_BAD_ARG;
  if (reject_mixed(h, "nscf_run")) return DEREK_ERR_UNSUPPORTED;
  // frozen potential: the filter's upper bound from max V_loc of each system
  for (auto &s : h->sys) s.active = 1;
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_sys, h->sys.data(), h->sys.size() * sizeof(SysDev),
                                cudaMemcpyHostToDevice, h->stream));
  std::vector<SysState> st(h->nsys);
  for (int s = 0; s < h->nsys; ++s) {
    std::memset(&st[s], 0, sizeof(SysState));
    st[s].slot = -1;
    const SysDev &S = h->sys[s];
    if (S.nspinor == 2) {
      // largest eigenvalue of the Hermitian part of nc_pot over the grid
      std::vector<double2> v((size_t)4 * S.nr);
      DEREK_CUDA(h, cudaMemcpy(v.data(), h->d_vnc64 + 4 * S.grid_off, v.size() * sizeof(double2),
                               cudaMemcpyDeviceToHost));
      double vmax = -1e300;
      for (long long i = 0; i < S.nr; ++i) {
        const double a = v[4 * i].x, d = v[4 * i + 3].x;
        const double br = 0.5 * (v[4 * i + 2].x + v[4 * i + 1].x), bi = 0.5 * (v[4 * i + 2].y - v[4 * i + 1].y);
        vmax = std::max(vmax, 0.5 * (a + d) + std::sqrt(0.25 * (a - d) * (a - d) + br * br + bi * bi));
      }
      st[s].vmax = vmax;
      continue;
    }
    std::vector<double> v(S.nr);
    DEREK_CUDA(h, cudaMemcpy(v.data(), h->d_vloc + S.grid_off, v.size() * sizeof(double),
                             cudaMemcpyDeviceToHost));
    st[s].vmax = *std::max_element(v.begin(), v.end());
  }
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_state, st.data(), st.size() * sizeof(SysState),
                                cudaMemcpyHostToDevice, h->stream));
  DEREK_CUDA(h, cudaMemsetAsync(h->d_status, 0, h->nks * sizeof(int), h->stream));
  int s = start_vectors(h);
  if (s) return s;
  s = cholqr_rr(h);
  if (s) return s;
  // the lowest nconv reported bands of every k-set (0: all reported): a band
  // close below the subspace's top converges slowly under the filter, whose
  // damped interval reaches up to Ecut + max V
  std::vector<double> eig(h->nitems), prev;
  auto status = [&]() -> int {
    std::vector<int> stat(h->nks);
    DEREK_CUDA(h, cudaMemcpy(stat.data(), h->d_status, stat.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (int x : stat)
      if (x) return x;
    return DEREK_OK;
  };
  int it = 0;
  bool converged = false;
  double last = -1.0;   // largest change of the last iteration
  int last_ks = -1, last_b = -1;
  for (; it < max_iter; ++it) {
    s = subspace_step(h, h->opts.cheb_degree);
    if (s) return s;
    DEREK_CUDA(h, cudaMemcpyAsync(eig.data(), h->d_eig, eig.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                  h->stream));
    DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
    if ((s = status())) return s;
    if (!prev.empty()) {
      double d = 0;
      for (int q = 0; q < h->nks; ++q) {
        const auto &K = h->ks_band[q];
        for (int b = 0; b < (nconv > 0 ? std::min(nconv, K.nbr) : K.nbr); ++b) {
          const double x = std::fabs(eig[K.item0 + b] - prev[K.item0 + b]);
          if (x > d) {
            d = x;
            last_ks = q;
            last_b = b;
          }
        }
      }
      last = d;
      if (d < eig_tol) {
        converged = true;
        ++it;
        break;
      }
    }
    prev = eig;
  }
  if (iterations) *iterations = it;
  if (!converged)
    h->last_error = "largest eigenvalue change " + std::to_string(last) + " Ha after " + std::to_string(it) +
                    " iterations (k-set " + std::to_string(last_ks) + ", band " + std::to_string(last_b) + ")";
  return converged ? DEREK_OK : DEREK_ERR_NOT_CONVERGED;
}

int derek_gpu_scf_run(derek_gpu_t *h, int max_scf, double etol, derek_scf_report *rep) {
  if (!h || max_scf <= 0 || !(etol > 0)) return DEREK_ERR_BAD_ARG;
  if (reject_mixed(h, "scf_run")) return DEREK_ERR_UNSUPPORTED;
  h->scf_started = false;
  std::vector<SysState> st;
  for (int it = 0; it < max_scf; ++it) {
    int s = one_iteration(h, etol);
    if (s) return s;
    s = read_state(h, st);
    if (s) return s;
    bool all_done = true;
    for (const auto &x : st) {
      if (x.status) {
        fill_reports(h, st, rep);
        h->last_error = derek_gpu_strerror(x.status);
        if (reset_lists(h)) drop_graphs(h);
        return x.status;
      }
      all_done &= x.converged != 0;
    }
    if (all_done) break;
    if (h->nsys > 1) maybe_compact(h, st);
  }
  // the other entry points (H.psi, NSCF, gradients) work on every item
  if (reset_lists(h)) drop_graphs(h);
  fill_reports(h, st, rep);
  for (const auto &x : st)
    if (!x.converged) return DEREK_ERR_NOT_CONVERGED;
  return DEREK_OK;
}

static int get_items(derek_gpu_t *h, int s, const double *src, double *out) {
  if (!h || s < 0 || s >= h->nsys || !out) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  // first nbr entries of each k-point (the buffer bands are not reported); a
  // spinor k-set keeps band j's entry at item0 + j
  const KSetDev &K0 = h->ks[S.ks0];
  const int nbr = S.nbr / S.nspinor;
  DEREK_CUDA(h, cudaMemcpy2DAsync(out, (size_t)nbr * sizeof(double), src + K0.item0,
                                  (size_t)S.nb * sizeof(double), (size_t)nbr * sizeof(double),
                                  S.nk, cudaMemcpyDeviceToHost, h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

int derek_gpu_get_eigenvalues(derek_gpu_t *h, int s, double *e) { return get_items(h, s, h ? h->d_eig : nullptr, e); }
int derek_gpu_get_occupations(derek_gpu_t *h, int s, double *o) { return get_items(h, s, h ? h->d_occ : nullptr, o); }

int derek_gpu_get_magnetisation(derek_gpu_t *h, int s, double *mag) {
  if (!h || s < 0 || s >= h->nsys || !mag) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  if (S.nspinor != 2 || !h->d_mag) {
    h->last_error = "get_magnetisation: system is not a spinor system";
    return DEREK_ERR_BAD_ARG;
  }
  for (int c = 0; c < 3; ++c)
    DEREK_CUDA(h, cudaMemcpyAsync(mag + (size_t)c * S.nr, h->d_mag + c * h->total_grid + S.grid_off,
                                  (size_t)S.nr * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

int derek_gpu_set_start_magnetisation(derek_gpu_t *h, int s, const double *mag) {
  if (!h || s < 0 || s >= h->nsys) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  if (S.nspinor != 2) {
    h->last_error = "set_start_magnetisation: system is not a spinor system";
    return DEREK_ERR_BAD_ARG;
  }
  if ((int)h->start_mag.size() < h->nsys) h->start_mag.resize(h->nsys);
  if (!mag)
    h->start_mag[s].clear();
  else
    h->start_mag[s].assign(mag, mag + 3 * (size_t)S.nr);
  h->scf_started = false;
  return DEREK_OK;
}

int derek_gpu_get_density(derek_gpu_t *h, int s, double *rho) {
  if (!h || s < 0 || s >= h->nsys || !rho) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  DEREK_CUDA(h, cudaMemcpyAsync(rho, h->d_rho_out + S.grid_off, (size_t)S.nr * sizeof(double),
                                cudaMemcpyDeviceToHost, h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

int derek_gpu_grad_wells(derek_gpu_t *h, int s, double *grad) {
  if (!h || s < 0 || s >= h->nsys || !grad) return DEREK_ERR_BAD_ARG;
  if (reject_spinor(h, "grad_wells")) return DEREK_ERR_UNSUPPORTED;
  const int nw = h->well_off[s + 1] - h->well_off[s];
  if (nw == 0 || !h->wells_define_vext[s]) {
    h->last_error = "system has no Gaussian wells defining its external potential";
    return DEREK_ERR_BAD_ARG;
  }
  launch_hf_gradient(h->tab, h->nsys, h->d_rho_out, h->d_wells, h->d_well_off, h->d_cells,
                     h->d_hfpart, h->max_wells, h->d_hfgrad, h->stream);
  DEREK_CUDA(h, cudaGetLastError());
  DEREK_CUDA(h, cudaMemcpyAsync(grad, h->d_hfgrad + 5 * h->well_off[s], (size_t)nw * 5 * sizeof(double),
                                cudaMemcpyDeviceToHost, h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

}  // extern "C"
