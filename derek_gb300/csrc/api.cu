// Handle creation and the primitive C-ABI entry points (tables, FFT, H.psi,
// density, XC).  The SCF entry points live in scf.cu.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <new>

#include "basis.h"
#include "handle.h"
#include "scf_kernels.cuh"

using derek::KSetDev;
using derek::SysDev;

namespace derek {

static std::atomic<unsigned long long> g_launches{0};
void note_launch(long long n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }
unsigned long long launch_total() { return g_launches.load(std::memory_order_relaxed); }

int cuda_status(cudaError_t e, derek_gpu *h, const char *what) {
  if (h) h->last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? DEREK_ERR_OOM : DEREK_ERR_CUDA;
}

__global__ void k_reduce_partials(const SysDev *__restrict__ sys, const KSetDev *__restrict__ ks,
                                  int s, const double *__restrict__ partial,
                                  const long long *__restrict__ poff, double *__restrict__ rho) {
  const SysDev &S = sys[s];
  if (!S.active) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < S.nr;
       i += (long long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int k = 0; k < S.nk; ++k) acc += partial[poff[S.ks0 + k] + i];
    rho[S.grid_off + i] = acc;
  }
}

__global__ void k_to_float(long long n, const double *__restrict__ a, float *__restrict__ b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// The three stage kernels of H.psi over one grid-size class.  max_m is the
// row bound the kernels are dispatched with (a class's tuned disp_m); with
// tune.generic_lines the shared-memory kernels with runtime line splits run.
template <typename R>
static void apply_h_class(derek_gpu *h, const Tables &t, int item_begin, int nitems, int nchunk,
                          const int n[3], int max_m, const void *in, const void *prev, void *out,
                          const Axpby *coef, const R *vloc) {
  launch_x_inv<R>(t, item_begin, nitems, nchunk, n[0], disp_min(h, n[0]), max_m, (const cplx<R> *)in,
                  (cplx<R> *)h->d_abuf, nullptr, h->stream);
  launch_plane<R>(t, item_begin, nitems, n[0], n[1], n[2], disp_min(h, n[1]), disp_min(h, n[2]), max_m,
                  (cplx<R> *)h->d_abuf, vloc, h->stream);
  launch_x_fwd<R>(t, item_begin, nitems, nchunk, n[0], disp_min(h, n[0]), max_m, (const cplx<R> *)h->d_abuf,
                  (const cplx<R> *)in, (const cplx<R> *)prev, (cplx<R> *)out, coef, h->stream);
}

// H.psi over items [item_begin, item_begin + nitems): all items (one launch
// per grid-size class) or the items of one k-set (a single class)
template <typename R>
static void apply_h_t(derek_gpu *h, const Tables &base, int item_begin, int nitems, const void *in,
                      const void *prev, void *out, const Axpby *coef, const R *vloc) {
  if (item_begin == 0 && nitems == h->nitems) {
    // a class in chunks of tune.hpsi_chunk items: a chunk's x-plane buffer
    // (~0.47 MB per item at 72^3) can stay in L2 between the three stages
    for (const auto &c : h->classes) {
      const int *list = c.launch_list();
      const int count = c.launch_count();
      const int step = h->tune.hpsi_chunk > 0 ? h->tune.hpsi_chunk : count;
      for (int i0 = 0; i0 < count; i0 += step) {
        Tables t = base;
        t.item_list = list ? list + i0 : nullptr;
        apply_h_class<R>(h, t, list ? 0 : i0, std::min(step, count - i0), c.nchunk, c.n, c.disp_m, in,
                         prev, out, coef, vloc);
      }
    }
    return;
  }
  const KSetDev &K = h->ks[h->item_ks[item_begin]];
  const SysDev &S = h->sys[K.sys];
  apply_h_class<R>(h, base, item_begin, nitems, (K.ncol + kColChunk - 1) / kColChunk, S.n,
                   h->ks_max_m[h->item_ks[item_begin]], in, prev, out, coef, vloc);
}

int apply_h_items(derek_gpu *h, int item_begin, int nitems, const void *in, const void *prev,
                  void *out, const Axpby *coef) {
  if (h->any_spinor) {
    // spinor items pair up within a k-set: all items of an all-spinor batch,
    // or one spinor k-set (mixed batches run per k-set)
    if (item_begin == 0 && nitems == h->nitems) {
      if (h->all_spinor) return apply_spinor_items(h, item_begin, nitems, in, prev, out, coef);
      h->last_error = "H.psi over a batch mixing spinor and scalar systems";
      return DEREK_ERR_UNSUPPORTED;
    }
    if (h->sys[h->ks[h->item_ks[item_begin]].sys].nspinor == 2)
      return apply_spinor_items(h, item_begin, nitems, in, prev, out, coef);
  }
  if (h->prec == DEREK_PREC_FP64)
    apply_h_t<double>(h, h->tab, item_begin, nitems, in, prev, out, coef, h->d_vloc);
  else
    apply_h_t<float>(h, h->tab, item_begin, nitems, in, prev, out, coef, h->d_vloc32);
  DEREK_CUDA(h, cudaGetLastError());
  return DEREK_OK;
}

bool compact_classes(derek_gpu *h, const std::vector<int> &sys_active) {
  bool changed = false;
  for (auto &c : h->classes) {
    std::vector<int> keep;
    keep.reserve(c.items.size());
    for (int it : c.items)
      if (sys_active[h->ks[h->item_ks[it]].sys]) keep.push_back(it);
    if ((int)keep.size() == c.launch_count()) continue;
    if (!keep.empty() && cudaMemcpyAsync(c.d_active, keep.data(), keep.size() * sizeof(int),
                                         cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
      continue;   // keep the previous list: still a superset of the active items
    c.active_count = (int)keep.size();
    changed = true;
  }
  return changed;
}

void reset_classes(derek_gpu *h) {
  for (auto &c : h->classes) c.active_count = -1;
}

int activate_all(derek_gpu *h) {
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_sys, h->sys.data(), h->sys.size() * sizeof(SysDev),
                                cudaMemcpyHostToDevice, h->stream));
  return DEREK_OK;
}

int apply_h_items_ex(derek_gpu *h, const Tables &base, int item_begin, int nitems, const void *in,
                     const void *prev, void *out, const Axpby *coef, const void *vloc) {
  if (h->prec == DEREK_PREC_FP64)
    apply_h_t<double>(h, base, item_begin, nitems, in, prev, out, coef, (const double *)vloc);
  else
    apply_h_t<float>(h, base, item_begin, nitems, in, prev, out, coef, (const float *)vloc);
  DEREK_CUDA(h, cudaGetLastError());
  return DEREK_OK;
}

template <typename R> static void density_t(derek_gpu *h, const void *psi) {
  for (const auto &c : h->classes) {
    Tables t = h->tab;
    t.item_list = c.launch_list();
    launch_x_inv<R>(t, 0, c.launch_count(), c.nchunk, c.n[0], disp_min(h, c.n[0]), c.disp_m,
                    (const cplx<R> *)psi, (cplx<R> *)h->d_abuf, h->d_occw, h->stream);
  }
  launch_density_plane<R>(h->tab, 0, h->nks, h->max_n[0], h->max_n[1], h->max_n[2], disp_min(h, h->min_n[1]),
                          disp_min(h, h->min_n[2]), h->max_m_all, (const cplx<R> *)h->d_abuf, h->d_occw,
                          h->d_partial, h->d_partial_off, h->stream);
}

int density_items(derek_gpu *h, const void *psi, double *rho) {
  if (h->prec == DEREK_PREC_FP64)
    density_t<double>(h, psi);
  else
    density_t<float>(h, psi);
  for (int s = 0; s < h->nsys; ++s)
    derek::note_launch(), k_reduce_partials<<<152, 256, 0, h->stream>>>(h->d_sys, h->d_ks, s, h->d_partial,
                                                  h->d_partial_off, rho);
  DEREK_CUDA(h, cudaGetLastError());
  return DEREK_OK;
}

// Spinor H.psi over one grid-size class: x-line passes per component, the
// 2x2 plane pass per band, the filter epilogue per component
template <typename R>
static void apply_spinor_class(derek_gpu *h, const Tables &t, int item_begin, int nitems, int nchunk,
                               const int n[3], const void *in, const void *prev, void *out,
                               const Axpby *coef) {
  const cplx<R> *vnc;
  if constexpr (std::is_same<R, double>::value)
    vnc = h->d_vnc64;
  else
    vnc = h->d_vnc32;
  launch_x_inv_lines<R>(t, item_begin, nitems, nchunk, n[0], n[0], (const cplx<R> *)in,
                        (cplx<R> *)h->d_abuf, nullptr, h->stream);
  launch_plane_spinor<R>(t, item_begin, nitems, n, (cplx<R> *)h->d_abuf, vnc, h->stream);
  launch_x_fwd_lines<R>(t, item_begin, nitems, nchunk, n[0], n[0], (const cplx<R> *)h->d_abuf,
                        (const cplx<R> *)in, (const cplx<R> *)prev, (cplx<R> *)out, coef, h->stream);
}

template <typename R>
static void apply_spinor_t(derek_gpu *h, int item_begin, int nitems, const void *in, const void *prev,
                           void *out, const Axpby *coef) {
  if (item_begin == 0 && nitems == h->nitems) {
    for (const auto &c : h->classes) {
      Tables t = h->tab;
      t.item_list = c.d_list;
      apply_spinor_class<R>(h, t, 0, c.count, c.nchunk, c.n, in, prev, out, coef);
    }
    return;
  }
  const KSetDev &K = h->ks[h->item_ks[item_begin]];
  apply_spinor_class<R>(h, h->tab, item_begin, nitems, (K.ncol + kColChunk - 1) / kColChunk,
                        h->sys[K.sys].n, in, prev, out, coef);
}

int apply_spinor_items(derek_gpu *h, int item_begin, int nitems, const void *in, const void *prev,
                       void *out, const Axpby *coef) {
  if (h->prec == DEREK_PREC_FP64)
    apply_spinor_t<double>(h, item_begin, nitems, in, prev, out, coef);
  else
    apply_spinor_t<float>(h, item_begin, nitems, in, prev, out, coef);
  DEREK_CUDA(h, cudaGetLastError());
  return DEREK_OK;
}

// n and m of every active spinor system from psi and per-item weights
// h->d_occw: rho gets n, h->d_mag the three components of m
template <typename R> static void density_spinor_t(derek_gpu *h, const void *psi) {
  for (const auto &c : h->classes) {
    Tables t = h->tab;
    t.item_list = c.d_list;
    launch_x_inv_lines<R>(t, 0, c.count, c.nchunk, c.n[0], c.n[0], (const cplx<R> *)psi,
                          (cplx<R> *)h->d_abuf, h->d_occw, h->stream);
  }
  launch_density_spinor<R>(h->tab, h->nks, h->max_n, (const cplx<R> *)h->d_abuf, h->d_occw,
                           h->d_partial, h->d_partial_off, h->stream);
}

int density_spinor_items(derek_gpu *h, const void *psi, double *rho) {
  if (h->prec == DEREK_PREC_FP64)
    density_spinor_t<double>(h, psi);
  else
    density_spinor_t<float>(h, psi);
  for (int s = 0; s < h->nsys; ++s) {
    const SysDev &S = h->sys[s];
    if (S.nspinor != 2) continue;
    for (int c = 0; c < 4; ++c)
      derek::note_launch(),
          k_reduce_partials<<<152, 256, 0, h->stream>>>(h->d_sys, h->d_ks, s, h->d_partial + c * (long long)S.nr,
                                                       h->d_partial_off,
                                                       c == 0 ? rho : h->d_mag + (c - 1) * h->total_grid);
  }
  DEREK_CUDA(h, cudaGetLastError());
  return DEREK_OK;
}

bool reject_spinor(derek_gpu *h, const char *what) {
  if (!h->any_spinor) return false;
  h->last_error = std::string(what) + ": spinor (nspinor = 2) systems support H.psi, overlaps and densities only";
  return true;
}

int refresh_vloc32(derek_gpu *h) {
  if (h->prec != DEREK_PREC_FP64)
    derek::note_launch(), k_to_float<<<152 * 4, 256, 0, h->stream>>>(h->total_grid, h->d_vloc, h->d_vloc32);
  DEREK_CUDA(h, cudaGetLastError());
  return DEREK_OK;
}

}  // namespace derek

using namespace derek;

static thread_local std::string g_create_error;

template <typename T> static cudaError_t upload(T **d, const std::vector<T> &v) {
  size_t bytes = std::max<size_t>(v.size(), 1) * sizeof(T);
  cudaError_t e = cudaMalloc((void **)d, bytes);
  if (e != cudaSuccess) return e;
  if (!v.empty()) return cudaMemcpy(*d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  return cudaSuccess;
}

extern "C" int derek_scf_alloc(derek_gpu_t *);
extern "C" void derek_scf_free(derek_gpu_t *);

extern "C" {

void derek_gpu_default_opts(derek_scf_opts *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->precision = DEREK_PREC_FP64;
  o->mix_alpha = 0.3;
  o->kerker_q0 = 0.0;
  o->pulay_history = 8;
  o->cheb_degree = 8;
  o->first_passes = 4;
  o->first_degree = 10;
  o->seed = 20240101ULL;
  o->use_graph = 1;
  o->use_tensor_cores = -1;
  o->density_tol = 0.0;
  o->buffer_bands = -1;
  o->etol_per_electron = 0;
  o->init_vectors = 0;
}

const char *derek_gpu_strerror(int s) {
  switch (s) {
    case DEREK_OK: return "ok";
    case DEREK_ERR_BAD_ARG: return "invalid argument";
    case DEREK_ERR_OOM: return "out of device memory";
    case DEREK_ERR_CUDA: return "CUDA error";
    case DEREK_ERR_NOT_CONVERGED: return "SCF not converged";
    case DEREK_ERR_CHOLESKY: return "overlap matrix not positive definite (Cholesky failed)";
    case DEREK_ERR_NAN: return "NaN detected";
    case DEREK_ERR_TIMEOUT: return "device wait timed out";
    case DEREK_ERR_UNSUPPORTED: return "unsupported configuration";
    default: return "unknown status";
  }
}

const char *derek_gpu_last_error(derek_gpu_t *h) {
  return h ? h->last_error.c_str() : g_create_error.c_str();
}

int derek_gpu_destroy(derek_gpu_t *h) {
  if (!h) return DEREK_ERR_BAD_ARG;
  void *ptrs[] = {h->d_sys,   h->d_ks,      h->d_item_ks, h->d_item_band, h->d_ent_col,
                  h->d_col_start, h->d_ent_ix, h->d_col_y, h->d_col_z, h->d_col_x0, h->d_rows, h->d_pw_entry, h->d_kin64,     h->d_kin32,
                  h->d_tw64,  h->d_tw32,    h->d_vext,    h->d_vloc,      h->d_vhxc,
                  h->d_vloc32, h->d_rho_in, h->d_rho_out, h->d_exc,       h->d_vxc,
                  h->d_cgrid, h->d_partial, h->d_partial_off, h->d_X,     h->d_Y,
                  h->d_Yp,    h->d_HX,      h->d_abuf,    h->d_occw,      h->d_eig,
                  h->d_occ,   h->d_coef,    h->d_cells,   h->d_wells,     h->d_well_off,
                  h->d_hfpart, h->d_hfgrad, h->d_vnc64, h->d_vnc32, h->d_mag, h->d_ks_band,
                  h->d_vnc_ext};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (auto &c : h->classes) {
    if (c.d_list) cudaFree(c.d_list);
    if (c.d_active) cudaFree(c.d_active);
  }
  derek_scf_free(h);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return DEREK_OK;
}

#define FAIL(code, msg)          \
  do {                           \
    g_create_error = (msg);      \
    derek_gpu_destroy(h);        \
    return (code);               \
  } while (0)

#define CK(call)                                                         \
  do {                                                                   \
    cudaError_t _e = (call);                                             \
    if (_e != cudaSuccess) {                                             \
      int _c = _e == cudaErrorMemoryAllocation ? DEREK_ERR_OOM : DEREK_ERR_CUDA; \
      FAIL(_c, std::string(#call) + ": " + cudaGetErrorString(_e));     \
    }                                                                    \
  } while (0)

int derek_gpu_create(derek_gpu_t **out, const derek_sys_desc *desc, int nsys,
                     const derek_scf_opts *opts) {
  if (!out || !desc || nsys <= 0) return DEREK_ERR_BAD_ARG;
  *out = nullptr;
  derek_gpu *h = new (std::nothrow) derek_gpu();
  if (!h) return DEREK_ERR_OOM;
  if (opts)
    h->opts = *opts;
  else
    derek_gpu_default_opts(&h->opts);
  h->prec = h->opts.precision;
  if (h->prec != DEREK_PREC_FP64 && h->prec != DEREK_PREC_MIXED) FAIL(DEREK_ERR_BAD_ARG, "precision");
  h->nsys = nsys;

  std::vector<int> ent_col, col_start;
  std::vector<short> ent_ix, col_y, col_z, col_x0, rows;
  std::vector<int> pw_entry;
  std::vector<float> kin32;
  std::vector<double> tw64;
  std::map<int, long long> tw_of;  // n -> offset
  std::vector<long long> partial_off;

  long long grid_off = 0, psi_off = 0, ent_off = 0, col_off = 0, row_off = 0, a_off = 0,
            part_off = 0;
  for (int s = 0; s < nsys; ++s) {
    const derek_sys_desc &d = desc[s];
    if (d.nspinor != 1 && d.nspinor != 2) FAIL(DEREK_ERR_UNSUPPORTED, "nspinor must be 1 or 2");
    if (d.nk <= 0 || !d.kpts || d.nbands <= 0 || d.ecut <= 0 || !(d.kT > 0) || d.nelec <= 0)
      FAIL(DEREK_ERR_BAD_ARG, "system " + std::to_string(s) + ": bad sizes");
    // a scalar band holds two electrons, a spinor band one
    if (d.nelec > (3 - d.nspinor) * (double)d.nbands) FAIL(DEREK_ERR_BAD_ARG, "more electrons than the bands hold");
    SysDev S{};
    double inv[9];
    bool have_inv = false;
    for (int i = 0; i < 9; ++i) have_inv |= d.inv_cell[i] != 0.0;
    if (have_inv)
      std::memcpy(inv, d.inv_cell, sizeof(inv));
    else
      inverse_cell(d.cell, inv);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S.B[i * 3 + j] = inv[3 * j + i];
    int nstd[3], nfine[3];
    grid_sizes(d.cell, d.ecut, d.g_fine_scale > 0 ? d.g_fine_scale : 2.0, d.grid_policy, nstd, nfine);
    if (d.n_fine[0] > 0 && d.n_fine[1] > 0 && d.n_fine[2] > 0)
      for (int i = 0; i < 3; ++i) nfine[i] = d.n_fine[i];
    for (int i = 0; i < 3; ++i) {
      if (nfine[i] < 2 || nfine[i] > kMaxDim)
        FAIL(DEREK_ERR_UNSUPPORTED, "grid size outside 2.." + std::to_string(kMaxDim));
      // the sphere must fit without wrapping onto itself
      if (nfine[i] < nstd[i]) FAIL(DEREK_ERR_BAD_ARG, "fine grid smaller than standard box");
    }
    {
      // density planes hold an FP64 accumulator plus one (y,z) plane
      const size_t es = h->prec == DEREK_PREC_FP64 ? 16 : 8;
      const size_t need = (size_t)((nfine[1] * nfine[2] + 1) & ~1) * 8 + ((size_t)nfine[1] * (nfine[2] + 1) + 2 * kMaxDim) * es;
      if (need > 227 * 1024) FAIL(DEREK_ERR_UNSUPPORTED, "grid planes exceed shared memory");
      // spinor passes hold both components' planes
      if (d.nspinor == 2 && spinor_plane_smem(nfine[1], nfine[2], es) > 227 * 1024)
        FAIL(DEREK_ERR_UNSUPPORTED, "spinor grid planes exceed shared memory");
    }
    for (int i = 0; i < 3; ++i) {
      S.n[i] = nfine[i];
      h->n_std.push_back(nstd[i]);
      h->max_n[i] = std::max(h->max_n[i], nfine[i]);
      h->min_n[i] = s == 0 ? nfine[i] : std::min(h->min_n[i], nfine[i]);
      h->max_nmax = std::max(h->max_nmax, nfine[i]);
      FftPlan &p = S.plan[i];
      p.n = nfine[i];
      if (!radix_plan(nfine[i], p.radix, &p.nstages))
        FAIL(DEREK_ERR_UNSUPPORTED, "grid size " + std::to_string(nfine[i]) + " not 13-smooth");
      LinePlan &lp = S.lp[i];
      lp.n = nfine[i];
      if (!line_plan(nfine[i], &lp.a, &lp.b))
        FAIL(DEREK_ERR_UNSUPPORTED, "grid size " + std::to_string(nfine[i]) + " has no a*b <= 16*16 split");
      lp.group = 32 / std::max(lp.a, lp.b);
      auto it = tw_of.find(nfine[i]);
      if (it == tw_of.end()) {
        std::vector<double> w;
        twiddles(nfine[i], w);
        long long off = (long long)tw64.size() / 2;
        tw64.insert(tw64.end(), w.begin(), w.end());
        tw_of[nfine[i]] = off;
        p.tw_off = off;
      } else {
        p.tw_off = it->second;
      }
      S.lp[i].tw_off = p.tw_off;
    }
    S.nr = nfine[0] * nfine[1] * nfine[2];
    S.nk = d.nk;
    const int nbuf = h->opts.buffer_bands >= 0 ? h->opts.buffer_bands : std::max(4, (d.nbands + 19) / 20);
    // a spinor band is two items (up, down): counts below are items
    const int nbi = d.nspinor * (d.nbands + nbuf);
    S.nb = nbi;
    S.nbr = d.nspinor * d.nbands;
    S.nspinor = d.nspinor;
    h->any_spinor |= d.nspinor == 2;
    h->all_spinor &= d.nspinor == 2;
    S.ks0 = (int)h->ks.size();
    S.active = 1;
    S.volume = cell_volume(d.cell);
    S.ecut = d.ecut;
    S.nelec = d.nelec;
    S.kT = d.kT;
    S.grid_off = grid_off;
    grid_off += S.nr;
    h->max_nb = std::max(h->max_nb, nbi);

    std::vector<double> v;
    if (d.vext)
      v.assign(d.vext, d.vext + S.nr);
    else
      build_vext(d.cell, nfine, d.nelec, d.nwells, d.wells, v);
    h->well_off.push_back((int)(h->wells_host.size() / 5));
    if (d.nwells > 0 && d.wells) h->wells_host.insert(h->wells_host.end(), d.wells, d.wells + 5 * d.nwells);
    h->wells_define_vext.push_back(d.vext == nullptr);
    h->max_wells = std::max(h->max_wells, d.nwells > 0 && d.wells ? d.nwells : 0);
    h->vext_host.insert(h->vext_host.end(), v.begin(), v.end());

    for (int k = 0; k < d.nk; ++k) {
      Sphere sp;
      build_sphere(inv, d.ecut, d.kpts + 3 * k, nstd, sp);
      const int npw = (int)sp.box_row.size();
      if (npw < nbi) FAIL(DEREK_ERR_BAD_ARG, "fewer plane waves than bands");
      KSetDev K{};
      K.sys = s;
      K.kidx = k;
      K.npw = npw;
      K.npw_pad = (npw + 31) / 32 * 32;
      K.nb = nbi;
      K.nbr = S.nbr;
      K.wk = d.wk ? d.wk[k] : 1.0 / d.nk;
      for (int i = 0; i < 3; ++i) K.kfrac[i] = d.kpts[3 * k + i];
      if (sp.mx.back() - sp.mx.front() + 1 > nfine[0]) FAIL(DEREK_ERR_BAD_ARG, "sphere wider than the fine grid");
      K.item0 = h->nitems;
      K.psi_off = psi_off;
      K.ent_off = ent_off;
      K.col_off = col_off;
      K.row_off = row_off;
      K.a_off = a_off;
      // column order: (y,z) columns sorted by centred (my, mz), each a run of
      // increasing mx (for a sphere the run is contiguous)
      std::map<std::pair<int, int>, std::vector<int>> cols;
      for (int i = 0; i < npw; ++i) cols[{sp.my[i], sp.mz[i]}].push_back(i);
      K.ncol = (int)cols.size();
      K.ncol_pad = (K.ncol + 15) / 16 * 16;
      int c = 0, e = 0, last_row = -1, max_m = 0;
      std::vector<short> krows;
      for (auto &kv : cols) {
        const int iy = ((kv.first.first % nfine[1]) + nfine[1]) % nfine[1];
        const int iz = ((kv.first.second % nfine[2]) + nfine[2]) % nfine[2];
        col_start.push_back(e);
        col_y.push_back((short)iy);
        col_z.push_back((short)iz);
        col_x0.push_back((short)sp.mx[kv.second.front()]);
        for (int ref : kv.second) {
          max_m = std::max(max_m, std::abs(sp.mx[ref]));
          const int ix = ((sp.mx[ref] % nfine[0]) + nfine[0]) % nfine[0];
          ent_col.push_back(c);
          ent_ix.push_back((short)ix);
          h->perm.push_back(ref);
          h->kin_col.push_back(sp.kinetic[ref]);
          kin32.push_back((float)sp.kinetic[ref]);
          ++e;
        }
        max_m = std::max(max_m, std::max(std::abs(kv.first.first), std::abs(kv.first.second)));
        if (kv.first.first != last_row) {
          krows.push_back((short)iy);
          last_row = kv.first.first;
        }
        ++c;
      }
      col_start.push_back(e);
      // keep col_y / col_z aligned with col_start (ncol + 1 entries per k-set)
      col_y.push_back(0);
      col_z.push_back(0);
      col_x0.push_back(0);
      K.nrow = (int)krows.size();
      h->ks_max_m.push_back(max_m);
      h->max_m_all = std::max(h->max_m_all, max_m);
      rows.insert(rows.end(), krows.begin(), krows.end());
      for (int i = 0; i < npw; ++i) {
        const int ix = ((sp.mx[i] % nfine[0]) + nfine[0]) % nfine[0];
        const int iy = ((sp.my[i] % nfine[1]) + nfine[1]) % nfine[1];
        const int iz = ((sp.mz[i] % nfine[2]) + nfine[2]) % nfine[2];
        h->box_rows.push_back(sp.box_row[i]);
        h->fft_index.push_back((ix * nfine[1] + iy) * nfine[2] + iz);
        h->kin64.push_back(sp.kinetic[i]);
      }
      h->max_nchunk = std::max(h->max_nchunk, (K.ncol + kColChunk - 1) / kColChunk);
      ent_off += npw;
      col_off += K.ncol + 1;
      row_off += K.nrow;
      psi_off += (long long)nbi * K.npw_pad;
      a_off += (long long)nbi * nfine[0] * K.ncol_pad;
      partial_off.push_back(part_off);
      part_off += (d.nspinor == 2 ? 4 : 1) * (long long)S.nr;
      {
        // plane-wave start vectors: the nbi lowest kinetic energies of the
        // k-point (ties by entry index), entries in column order
        std::vector<int> order(npw);
        for (int i = 0; i < npw; ++i) order[i] = i;
        const double *kc = h->kin_col.data() + K.ent_off;
        std::partial_sort(order.begin(), order.begin() + nbi, order.end(), [kc](int a, int b) {
          return kc[a] < kc[b] || (kc[a] == kc[b] && a < b);
        });
        for (int b = 0; b < nbi; ++b) pw_entry.push_back(order[b]);
      }
      for (int b = 0; b < nbi; ++b) {
        h->item_ks.push_back((int)h->ks.size());
        h->item_band.push_back(b);
      }
      h->nitems += nbi;
      h->ks.push_back(K);
    }
    h->sys.push_back(S);
  }
  h->well_off.push_back((int)(h->wells_host.size() / 5));
  h->nks = (int)h->ks.size();
  h->total_psi = psi_off;
  h->total_abuf = a_off;
  h->total_grid = grid_off;
  std::vector<float> tw32(tw64.begin(), tw64.end());

  CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  CK(upload(&h->d_sys, h->sys));
  CK(upload(&h->d_ks, h->ks));
  h->ks_band = h->ks;
  for (auto &K : h->ks_band)
    if (h->sys[K.sys].nspinor == 2) {
      K.nb /= 2;
      K.nbr /= 2;
      K.npw_pad *= 2;
      K.npw = K.npw_pad;
    }
  CK(upload(&h->d_ks_band, h->ks_band));
  CK(upload(&h->d_item_ks, h->item_ks));
  CK(upload(&h->d_item_band, h->item_band));
  CK(upload(&h->d_ent_col, ent_col));
  CK(upload(&h->d_ent_ix, ent_ix));
  CK(upload(&h->d_col_start, col_start));
  CK(upload(&h->d_col_y, col_y));
  CK(upload(&h->d_col_z, col_z));
  CK(upload(&h->d_col_x0, col_x0));
  CK(upload(&h->d_rows, rows));
  CK(upload(&h->d_pw_entry, pw_entry));
  CK(upload(&h->d_kin64, h->kin_col));
  CK(upload(&h->d_kin32, kin32));
  {
    std::vector<double2> t(tw64.size() / 2);
    std::vector<float2> t32(tw64.size() / 2);
    for (size_t i = 0; i < t.size(); ++i) {
      t[i] = make_double2(tw64[2 * i], tw64[2 * i + 1]);
      t32[i] = make_float2((float)tw64[2 * i], (float)tw64[2 * i + 1]);
    }
    CK(upload(&h->d_tw64, t));
    CK(upload(&h->d_tw32, t32));
  }
  CK(upload(&h->d_vext, h->vext_host));
  {
    std::vector<double> cells;
    for (int s = 0; s < nsys; ++s) cells.insert(cells.end(), desc[s].cell, desc[s].cell + 9);
    CK(upload(&h->d_cells, cells));
    CK(upload(&h->d_wells, h->wells_host));
    CK(upload(&h->d_well_off, h->well_off));
    CK(cudaMalloc((void **)&h->d_hfpart, (size_t)nsys * 64 * std::max(h->max_wells, 1) * 5 * sizeof(double)));
    CK(cudaMalloc((void **)&h->d_hfgrad, std::max<size_t>(h->wells_host.size(), 1) * sizeof(double)));
  }
  CK(upload(&h->d_partial_off, partial_off));
  const size_t gbytes = (size_t)grid_off * sizeof(double);
  CK(cudaMalloc((void **)&h->d_vloc, gbytes));
  CK(cudaMemcpy(h->d_vloc, h->d_vext, gbytes, cudaMemcpyDeviceToDevice));
  CK(cudaMalloc((void **)&h->d_vhxc, gbytes));
  CK(cudaMemset(h->d_vhxc, 0, gbytes));
  CK(cudaMalloc((void **)&h->d_vloc32, (size_t)grid_off * sizeof(float)));
  CK(cudaMalloc((void **)&h->d_rho_in, gbytes));
  CK(cudaMalloc((void **)&h->d_rho_out, gbytes));
  CK(cudaMalloc((void **)&h->d_exc, gbytes));
  CK(cudaMalloc((void **)&h->d_vxc, gbytes));
  CK(cudaMalloc((void **)&h->d_cgrid, (size_t)grid_off * sizeof(double2)));
  CK(cudaMalloc((void **)&h->d_partial, (size_t)std::max<long long>(part_off, 1) * sizeof(double)));
  if (h->any_spinor) {
    // nc_pot starts as V_ext on the diagonal (Source/pot.f90:133-166)
    std::vector<double2> vnc((size_t)4 * grid_off, make_double2(0.0, 0.0));
    for (int s = 0; s < nsys; ++s) {
      const SysDev &S = h->sys[s];
      if (S.nspinor != 2) continue;
      for (long long i = 0; i < S.nr; ++i) {
        const double v = h->vext_host[S.grid_off + i];
        vnc[4 * (S.grid_off + i)] = make_double2(v, 0.0);
        vnc[4 * (S.grid_off + i) + 3] = make_double2(v, 0.0);
      }
    }
    std::vector<float2> vnc32(vnc.size());
    for (size_t i = 0; i < vnc.size(); ++i) vnc32[i] = make_float2((float)vnc[i].x, (float)vnc[i].y);
    CK(upload(&h->d_vnc64, vnc));
    CK(upload(&h->d_vnc32, vnc32));
    CK(upload(&h->d_vnc_ext, vnc));
    CK(cudaMalloc((void **)&h->d_mag, (size_t)3 * grid_off * sizeof(double)));
  }
  const size_t pbytes = (size_t)h->total_psi * h->elem_size();
  CK(cudaMalloc(&h->d_X, pbytes));
  CK(cudaMalloc(&h->d_Y, pbytes));
  CK(cudaMalloc(&h->d_Yp, pbytes));
  CK(cudaMalloc(&h->d_HX, pbytes));
  CK(cudaMemset(h->d_X, 0, pbytes));
  CK(cudaMemset(h->d_Y, 0, pbytes));
  CK(cudaMemset(h->d_Yp, 0, pbytes));
  CK(cudaMemset(h->d_HX, 0, pbytes));
  CK(cudaMalloc(&h->d_abuf, (size_t)std::max<long long>(h->total_abuf, 1) * h->elem_size()));
  CK(cudaMalloc((void **)&h->d_occw, (size_t)h->nitems * sizeof(double)));
  CK(cudaMalloc((void **)&h->d_eig, (size_t)h->nitems * sizeof(double)));
  CK(cudaMalloc((void **)&h->d_occ, (size_t)h->nitems * sizeof(double)));
  CK(cudaMemset(h->d_eig, 0, (size_t)h->nitems * sizeof(double)));
  CK(cudaMemset(h->d_occ, 0, (size_t)h->nitems * sizeof(double)));
  CK(cudaMalloc((void **)&h->d_coef, (size_t)h->nks * sizeof(Axpby)));

  h->tab.sys = h->d_sys;
  h->tab.ks = h->d_ks;
  h->tab.item_ks = h->d_item_ks;
  h->tab.item_band = h->d_item_band;
  h->tab.ent_col = h->d_ent_col;
  h->tab.ent_ix = h->d_ent_ix;
  h->tab.col_start = h->d_col_start;
  h->tab.col_y = h->d_col_y;
  h->tab.col_z = h->d_col_z;
  h->tab.col_x0 = h->d_col_x0;
  h->tab.kin64 = h->d_kin64;
  h->tab.kin32 = h->d_kin32;
  h->tab.rows = h->d_rows;
  h->tab.tw64 = h->d_tw64;
  h->tab.tw32 = h->d_tw32;
  h->tab.item_list = nullptr;
  h->tab.item_shift = nullptr;
  h->tab_band = h->tab;
  h->tab_band.ks = h->d_ks_band;
  {
    // group items by grid size; a single class over all items needs no list
    std::map<std::array<int, 3>, std::vector<int>> groups;
    std::map<std::array<int, 3>, int> chunks, mys;
    for (int it = 0; it < h->nitems; ++it) {
      const KSetDev &K = h->ks[h->item_ks[it]];
      const SysDev &S = h->sys[K.sys];
      const std::array<int, 3> key = {S.n[0], S.n[1], S.n[2]};
      groups[key].push_back(it);
      chunks[key] = std::max(chunks[key], (K.ncol + kColChunk - 1) / kColChunk);
      mys[key] = std::max(mys[key], h->ks_max_m[h->item_ks[it]]);
    }
    for (auto &g : groups) {
      derek_gpu::ItemClass c{};
      for (int i = 0; i < 3; ++i) c.n[i] = g.first[i];
      c.count = (int)g.second.size();
      c.nchunk = chunks[g.first];
      c.max_m = mys[g.first];
      c.disp_m = c.max_m;
      c.d_list = nullptr;
      if (groups.size() > 1) CK(upload(&c.d_list, g.second));
      c.items = g.second;
      CK(cudaMalloc((void **)&c.d_active, std::max<size_t>(c.items.size(), 1) * sizeof(int)));
      h->classes.push_back(c);
    }
  }
  if (refresh_vloc32(h) != DEREK_OK) FAIL(DEREK_ERR_CUDA, h->last_error);
  int st = derek_scf_alloc(h);
  if (st != DEREK_OK) FAIL(st, h->last_error);
  CK(cudaStreamSynchronize(h->stream));
  *out = h;
  return DEREK_OK;
}

static int check_sys(derek_gpu_t *h, int s) { return h && s >= 0 && s < h->nsys; }

static int ks_index(derek_gpu_t *h, int s, int k) {
  if (!check_sys(h, s) || k < 0 || k >= h->sys[s].nk) return -1;
  return h->sys[s].ks0 + k;
}

int derek_gpu_grid(derek_gpu_t *h, int s, int n_fine[3], int n_std[3]) {
  if (!check_sys(h, s)) return DEREK_ERR_BAD_ARG;
  for (int i = 0; i < 3; ++i) {
    if (n_fine) n_fine[i] = h->sys[s].n[i];
    if (n_std) n_std[i] = h->n_std[3 * s + i];
  }
  return DEREK_OK;
}

int derek_gpu_bands(derek_gpu_t *h, int s, int *nb, int *nbi) {
  if (!check_sys(h, s)) return DEREK_ERR_BAD_ARG;
  if (nb) *nb = h->sys[s].nbr / h->sys[s].nspinor;
  if (nbi) *nbi = h->sys[s].nb / h->sys[s].nspinor;
  return DEREK_OK;
}

int derek_gpu_npw(derek_gpu_t *h, int s, int k, int *npw) {
  int ki = ks_index(h, s, k);
  if (ki < 0 || !npw) return DEREK_ERR_BAD_ARG;
  *npw = h->ks[ki].npw;
  return DEREK_OK;
}

int derek_gpu_gsphere(derek_gpu_t *h, int s, int k, int32_t *box_rows, int32_t *fft_index,
                      double *kinetic) {
  int ki = ks_index(h, s, k);
  if (ki < 0) return DEREK_ERR_BAD_ARG;
  const KSetDev &K = h->ks[ki];
  for (int i = 0; i < K.npw; ++i) {
    if (box_rows) box_rows[i] = h->box_rows[K.ent_off + i];
    if (fft_index) fft_index[i] = h->fft_index[K.ent_off + i];
    if (kinetic) kinetic[i] = h->kin64[K.ent_off + i];
  }
  return DEREK_OK;
}

int derek_gpu_fft3d(derek_gpu_t *h, int s, double *inout, int dir) {
  if (!check_sys(h, s) || !inout || (dir != 1 && dir != -1)) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  double2 *g = h->d_cgrid + S.grid_off;
  DEREK_CUDA(h, cudaMemcpyAsync(g, inout, (size_t)S.nr * sizeof(double2), cudaMemcpyHostToDevice,
                                h->stream));
  // dir = +1 is the forward transform, exponent -i
  launch_fft3d_grid(h->tab, s, 1, h->max_nmax, h->d_cgrid, dir == 1 ? -1 : +1, h->stream);
  DEREK_CUDA(h, cudaGetLastError());
  DEREK_CUDA(h, cudaMemcpyAsync(inout, g, (size_t)S.nr * sizeof(double2), cudaMemcpyDeviceToHost,
                                h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

// write system s's 2x2 potential, given per point as V11, V21, V12, V22: the
// H.psi potential and, with ext, the SCF's external potential too
static int upload_nc(derek_gpu_t *h, int s, const std::vector<double2> &vnc, bool ext = false) {
  const SysDev &S = h->sys[s];
  if (ext)
    DEREK_CUDA(h, cudaMemcpyAsync(h->d_vnc_ext + 4 * S.grid_off, vnc.data(), vnc.size() * sizeof(double2),
                                  cudaMemcpyHostToDevice, h->stream));
  std::vector<float2> v32(vnc.size());
  for (size_t i = 0; i < vnc.size(); ++i) v32[i] = make_float2((float)vnc[i].x, (float)vnc[i].y);
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_vnc64 + 4 * S.grid_off, vnc.data(), vnc.size() * sizeof(double2),
                                cudaMemcpyHostToDevice, h->stream));
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_vnc32 + 4 * S.grid_off, v32.data(), v32.size() * sizeof(float2),
                                cudaMemcpyHostToDevice, h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

int derek_gpu_set_vloc(derek_gpu_t *h, int s, const double *v) {
  if (!check_sys(h, s) || !v) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_vloc + S.grid_off, v, (size_t)S.nr * sizeof(double),
                                cudaMemcpyHostToDevice, h->stream));
  int st = refresh_vloc32(h);
  if (st) return st;
  if (S.nspinor == 2) {
    // a spin-independent potential: V on the diagonal of nc_pot
    std::vector<double2> vnc((size_t)4 * S.nr, make_double2(0.0, 0.0));
    for (long long i = 0; i < S.nr; ++i) vnc[4 * i] = vnc[4 * i + 3] = make_double2(v[i], 0.0);
    return upload_nc(h, s, vnc);
  }
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

int derek_gpu_set_nc_pot(derek_gpu_t *h, int s, const double *nc_pot) {
  if (!check_sys(h, s) || !nc_pot) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  if (S.nspinor != 2) {
    h->last_error = "set_nc_pot: system is not a spinor system (nspinor = 1)";
    return DEREK_ERR_BAD_ARG;
  }
  // reference order nc_pot(n, i, j): component c = i + 2 j is plane c of nr values
  std::vector<double2> vnc((size_t)4 * S.nr);
  for (int c = 0; c < 4; ++c)
    for (long long i = 0; i < S.nr; ++i)
      vnc[4 * i + c] = make_double2(nc_pot[2 * (c * S.nr + i)], nc_pot[2 * (c * S.nr + i) + 1]);
  h->scf_started = false;
  return upload_nc(h, s, vnc, true);
}

// copy system s's 2x2 potential (H.psi's, or the SCF's external one) out in
// the reference's nc_pot(nr, 2, 2) order
static int read_nc(derek_gpu_t *h, int s, double *nc_pot, bool ext) {
  if (!check_sys(h, s) || !nc_pot) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  if (S.nspinor != 2) {
    h->last_error = "nc_pot: system is not a spinor system (nspinor = 1)";
    return DEREK_ERR_BAD_ARG;
  }
  std::vector<double2> vnc((size_t)4 * S.nr);
  DEREK_CUDA(h, cudaMemcpyAsync(vnc.data(), (ext ? h->d_vnc_ext : h->d_vnc64) + 4 * S.grid_off,
                                vnc.size() * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  for (int c = 0; c < 4; ++c)
    for (long long i = 0; i < S.nr; ++i) {
      nc_pot[2 * (c * S.nr + i)] = vnc[4 * i + c].x;
      nc_pot[2 * (c * S.nr + i) + 1] = vnc[4 * i + c].y;
    }
  return DEREK_OK;
}

int derek_gpu_get_nc_pot(derek_gpu_t *h, int s, double *nc_pot) { return read_nc(h, s, nc_pot, false); }
int derek_gpu_get_nc_ext(derek_gpu_t *h, int s, double *nc_pot) { return read_nc(h, s, nc_pot, true); }

int derek_gpu_set_start_density(derek_gpu_t *h, int s, const double *rho) {
  if (!check_sys(h, s)) return DEREK_ERR_BAD_ARG;
  if ((int)h->start_rho.size() < h->nsys) h->start_rho.resize(h->nsys);
  if (!rho) {
    h->start_rho[s].clear();
    return DEREK_OK;
  }
  const SysDev &S = h->sys[s];
  h->start_rho[s].assign(rho, rho + S.nr);
  return DEREK_OK;
}

int derek_gpu_get_vloc(derek_gpu_t *h, int s, double *v) {
  if (!check_sys(h, s) || !v) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  DEREK_CUDA(h, cudaMemcpyAsync(v, h->d_vloc + S.grid_off, (size_t)S.nr * sizeof(double),
                                cudaMemcpyDeviceToHost, h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

// copy between a host complex128 [nspinor][nbr][npw] slice in the
// reference's G order (coeff(gvec, band, spinor) of one k-point) and the
// padded, column-ordered device buffer, where band b's spinor s is row
// nspinor * b + s (only the requested bands; buffer bands stay on the device)
static int copy_slice(derek_gpu_t *h, int ki, void *dev_base, double *host, bool to_dev) {
  const KSetDev &K = h->ks[ki];
  const size_t es = h->elem_size();
  char *dev = (char *)dev_base + (size_t)K.psi_off * es;
  const int nb = K.nbr;
  const int nsp = h->sys[K.sys].nspinor;
  auto host_row = [nb, nsp](int p) { return nsp == 1 ? p : (p % 2) * (nb / 2) + p / 2; };
  const size_t n = (size_t)nb * K.npw_pad;
  const int32_t *perm = h->perm.data() + K.ent_off;
  const bool f64 = h->prec == DEREK_PREC_FP64;
  std::vector<double> t64(f64 ? 2 * n : 0, 0.0);
  std::vector<float> t32(f64 ? 0 : 2 * n, 0.0f);
  if (to_dev) {
    for (int b = 0; b < nb; ++b)
      for (int g = 0; g < K.npw; ++g) {
        const size_t src = 2 * ((size_t)host_row(b) * K.npw + perm[g]);
        const size_t dst = 2 * ((size_t)b * K.npw_pad + g);
        if (f64) {
          t64[dst] = host[src];
          t64[dst + 1] = host[src + 1];
        } else {
          t32[dst] = (float)host[src];
          t32[dst + 1] = (float)host[src + 1];
        }
      }
    DEREK_CUDA(h, cudaMemcpyAsync(dev, f64 ? (void *)t64.data() : (void *)t32.data(), n * es,
                                  cudaMemcpyHostToDevice, h->stream));
    DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  } else {
    DEREK_CUDA(h, cudaMemcpyAsync(f64 ? (void *)t64.data() : (void *)t32.data(), dev, n * es,
                                  cudaMemcpyDeviceToHost, h->stream));
    DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
    for (int b = 0; b < nb; ++b)
      for (int g = 0; g < K.npw; ++g) {
        const size_t dst = 2 * ((size_t)host_row(b) * K.npw + perm[g]);
        const size_t src = 2 * ((size_t)b * K.npw_pad + g);
        host[dst] = f64 ? t64[src] : (double)t32[src];
        host[dst + 1] = f64 ? t64[src + 1] : (double)t32[src + 1];
      }
  }
  return DEREK_OK;
}

int derek_gpu_set_wfn(derek_gpu_t *h, int s, int k, const double *psi) {
  int ki = ks_index(h, s, k);
  if (ki < 0 || !psi) return DEREK_ERR_BAD_ARG;
  return copy_slice(h, ki, h->cur_psi(), const_cast<double *>(psi), true);
}

int derek_gpu_get_wfn(derek_gpu_t *h, int s, int k, double *psi) {
  int ki = ks_index(h, s, k);
  if (ki < 0 || !psi) return DEREK_ERR_BAD_ARG;
  return copy_slice(h, ki, h->cur_psi(), psi, false);
}

int derek_gpu_apply_h(derek_gpu_t *h, int s, int k, double *hpsi) {
  int ki = ks_index(h, s, k);
  if (ki < 0 || !hpsi) return DEREK_ERR_BAD_ARG;
  const KSetDev &K = h->ks[ki];
  // an SCF leaves its converged systems masked off on the device
  int st = activate_all(h);
  if (st) return st;
  st = apply_h_items(h, K.item0, K.nb, h->cur_psi(), nullptr, h->d_HX, nullptr);
  if (st) return st;
  return copy_slice(h, ki, h->d_HX, hpsi, false);
}

int derek_gpu_density(derek_gpu_t *h, int s, const double *occ, double *rho) {
  if (!check_sys(h, s) || !occ || !rho) return DEREK_ERR_BAD_ARG;
  if (h->sys[s].nspinor == 2) return derek_gpu_density_spinor(h, s, occ, rho, nullptr);
  const SysDev &S = h->sys[s];
  // per-item weights w_k f / Omega for this system, zero elsewhere
  std::vector<double> w(h->nitems, 0.0);
  for (int k = 0; k < S.nk; ++k) {
    const KSetDev &K = h->ks[S.ks0 + k];
    for (int b = 0; b < K.nbr; ++b) w[K.item0 + b] = K.wk * occ[(size_t)k * S.nbr + b] / S.volume;
  }
  // other systems are masked off for the duration of the call
  std::vector<SysDev> masked = h->sys;
  for (int i = 0; i < h->nsys; ++i) masked[i].active = (i == s) && h->sys[i].active;
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_sys, masked.data(), masked.size() * sizeof(SysDev),
                                cudaMemcpyHostToDevice, h->stream));
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_occw, w.data(), w.size() * sizeof(double),
                                cudaMemcpyHostToDevice, h->stream));
  int st = density_items(h, h->cur_psi(), h->d_rho_out);
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_sys, h->sys.data(), h->sys.size() * sizeof(SysDev),
                                cudaMemcpyHostToDevice, h->stream));
  if (st) return st;
  DEREK_CUDA(h, cudaMemcpyAsync(rho, h->d_rho_out + S.grid_off, (size_t)S.nr * sizeof(double),
                                cudaMemcpyDeviceToHost, h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

int derek_gpu_density_spinor(derek_gpu_t *h, int s, const double *occ, double *rho, double *mag) {
  if (!check_sys(h, s) || !occ || (!rho && !mag)) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  if (S.nspinor != 2) {
    h->last_error = "density_spinor: system is not a spinor system (nspinor = 1)";
    return DEREK_ERR_BAD_ARG;
  }
  // per-item weights w_k f / Omega, equal on both components of a band
  const int nbr = S.nbr / 2;
  std::vector<double> w(h->nitems, 0.0);
  for (int k = 0; k < S.nk; ++k) {
    const KSetDev &K = h->ks[S.ks0 + k];
    for (int b = 0; b < nbr; ++b)
      w[K.item0 + 2 * b] = w[K.item0 + 2 * b + 1] = K.wk * occ[(size_t)k * nbr + b] / S.volume;
  }
  std::vector<SysDev> masked = h->sys;
  for (int i = 0; i < h->nsys; ++i) masked[i].active = (i == s) && h->sys[i].active;
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_sys, masked.data(), masked.size() * sizeof(SysDev),
                                cudaMemcpyHostToDevice, h->stream));
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_occw, w.data(), w.size() * sizeof(double),
                                cudaMemcpyHostToDevice, h->stream));
  int st = density_spinor_items(h, h->cur_psi(), h->d_rho_out);
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_sys, h->sys.data(), h->sys.size() * sizeof(SysDev),
                                cudaMemcpyHostToDevice, h->stream));
  if (st) return st;
  if (rho)
    DEREK_CUDA(h, cudaMemcpyAsync(rho, h->d_rho_out + S.grid_off, (size_t)S.nr * sizeof(double),
                                  cudaMemcpyDeviceToHost, h->stream));
  if (mag)
    for (int c = 0; c < 3; ++c)
      DEREK_CUDA(h, cudaMemcpyAsync(mag + (size_t)c * S.nr, h->d_mag + c * h->total_grid + S.grid_off,
                                    (size_t)S.nr * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  return DEREK_OK;
}

int derek_gpu_xc_lsda(derek_gpu_t *h, long n, const double *rho_a, const double *rho_b, double *exc,
                      double *va, double *vb) {
  if (!h || n <= 0 || !rho_a || !rho_b || !exc || !va || !vb) return DEREK_ERR_BAD_ARG;
  double *d = nullptr;
  DEREK_CUDA(h, cudaMalloc((void **)&d, 5 * (size_t)n * sizeof(double)));
  cudaMemcpyAsync(d, rho_a, n * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  cudaMemcpyAsync(d + n, rho_b, n * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  launch_lsda(n, d, d + n, d + 2 * n, d + 3 * n, d + 4 * n, h->stream);
  cudaMemcpyAsync(exc, d + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  cudaMemcpyAsync(va, d + 3 * n, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  cudaMemcpyAsync(vb, d + 4 * n, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_status(e, h, "xc_lsda");
  return DEREK_OK;
}

int derek_gpu_xc_lda(derek_gpu_t *h, long n, const double *rho, double *exc, double *vxc) {
  if (!h || n <= 0 || !rho || (!exc && !vxc)) return DEREK_ERR_BAD_ARG;
  double *d = nullptr;
  DEREK_CUDA(h, cudaMalloc((void **)&d, 3 * (size_t)n * sizeof(double)));
  cudaMemcpyAsync(d, rho, n * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  launch_lda(n, d, d + n, d + 2 * n, h->stream);
  if (exc) cudaMemcpyAsync(exc, d + n, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (vxc) cudaMemcpyAsync(vxc, d + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_status(e, h, "xc_lda");
  return DEREK_OK;
}

int derek_host_prime_fact(int n) { return n > 0 ? prime_fact_round(n) : -1; }

int derek_host_grid_sizes(const double cell[9], double ecut, double g_fine_scale, int policy,
                          int n_std[3], int n_fine[3]) {
  if (!cell || !n_std || !n_fine || !(ecut > 0)) return DEREK_ERR_BAD_ARG;
  grid_sizes(cell, ecut, g_fine_scale > 0 ? g_fine_scale : 2.0, policy, n_std, n_fine);
  return DEREK_OK;
}

int derek_host_gsphere(const double inv_cell[9], double ecut, const double kfrac[3],
                       const int n_std[3], int capacity, int32_t *box_rows, int *npw) {
  if (!inv_cell || !kfrac || !n_std || !npw || !(ecut > 0)) return DEREK_ERR_BAD_ARG;
  Sphere sp;
  build_sphere(inv_cell, ecut, kfrac, n_std, sp);
  *npw = (int)sp.box_row.size();
  if (box_rows)
    for (int i = 0; i < *npw && i < capacity; ++i) box_rows[i] = sp.box_row[i];
  return DEREK_OK;
}

int derek_gpu_set_vext(derek_gpu_t *h, int s, const double *v) {
  if (!check_sys(h, s) || !v) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_vext + S.grid_off, v, (size_t)S.nr * sizeof(double),
                                cudaMemcpyHostToDevice, h->stream));
  std::copy(v, v + S.nr, h->vext_host.begin() + S.grid_off);
  h->scf_started = false;
  if (S.nspinor == 2) {
    // the spinor SCF's external potential: V_ext on the diagonal, no field
    std::vector<double2> vnc((size_t)4 * S.nr, make_double2(0.0, 0.0));
    for (long long i = 0; i < S.nr; ++i) vnc[4 * i] = vnc[4 * i + 3] = make_double2(v[i], 0.0);
    return upload_nc(h, s, vnc, true);
  }
  return DEREK_OK;
}

int derek_gpu_get_vext(derek_gpu_t *h, int s, double *v) {
  if (!check_sys(h, s) || !v) return DEREK_ERR_BAD_ARG;
  const SysDev &S = h->sys[s];
  std::copy(h->vext_host.begin() + S.grid_off, h->vext_host.begin() + S.grid_off + S.nr, v);
  return DEREK_OK;
}

void *derek_gpu_stream(derek_gpu_t *h) { return h ? (void *)h->stream : nullptr; }

unsigned long long derek_gpu_launch_count(void) { return launch_total(); }

int derek_gpu_time_apply_h(derek_gpu_t *h, int nrep, double *ms_apply, double *ms_stage) {
  if (!h || nrep <= 0) return DEREK_ERR_BAD_ARG;
  if (h->any_spinor) {
    // an all-spinor batch: the whole 2x2 H.psi timed as one (its x passes
    // and 2x2 plane pass interleave per class); the stage times are zero
    if (!h->all_spinor) {
      h->last_error = "time_apply_h: a batch mixing spinor and scalar systems";
      return DEREK_ERR_UNSUPPORTED;
    }
    for (auto &s : h->sys) s.active = 1;
    DEREK_CUDA(h, cudaMemcpyAsync(h->d_sys, h->sys.data(), h->sys.size() * sizeof(SysDev),
                                  cudaMemcpyHostToDevice, h->stream));
    cudaEvent_t e0, e1;
    DEREK_CUDA(h, cudaEventCreate(&e0));
    DEREK_CUDA(h, cudaEventCreate(&e1));
    int st = apply_spinor_items(h, 0, h->nitems, h->cur_psi(), nullptr, h->d_HX, nullptr);   // warm-up
    cudaEventRecord(e0, h->stream);
    for (int r = 0; r < nrep && !st; ++r)
      st = apply_spinor_items(h, 0, h->nitems, h->cur_psi(), nullptr, h->d_HX, nullptr);
    cudaEventRecord(e1, h->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    DEREK_CUDA(h, cudaGetLastError());
    if (ms_apply) *ms_apply = ms / nrep;
    if (ms_stage)
      for (int k = 0; k < 3; ++k) ms_stage[k] = 0.0;
    return DEREK_OK;
  }
  // converged systems are masked off on the device; time every system
  std::vector<SysDev> all = h->sys;
  for (auto &s : all) s.active = 1;
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_sys, all.data(), all.size() * sizeof(SysDev),
                                cudaMemcpyHostToDevice, h->stream));
  // the chunks apply_h_items runs, with events around each stage of each chunk
  struct Chunk {
    const derek_gpu::ItemClass *c;
    int i0, n;
  };
  std::vector<Chunk> chunks;
  for (const auto &c : h->classes) {
    const int step = h->tune.hpsi_chunk > 0 ? h->tune.hpsi_chunk : c.count;
    for (int i0 = 0; i0 < c.count; i0 += step) chunks.push_back({&c, i0, std::min(step, c.count - i0)});
  }
  std::vector<cudaEvent_t> ev(4 * chunks.size());
  for (auto &e : ev) DEREK_CUDA(h, cudaEventCreate(&e));
  double tot[3] = {0, 0, 0};
  const void *in = h->cur_psi();
  for (int r = 0; r < nrep; ++r) {
    for (size_t q = 0; q < chunks.size(); ++q) {
      const auto &ch = chunks[q];
      const auto &c = *ch.c;
      Tables t = h->tab;
      t.item_list = c.d_list ? c.d_list + ch.i0 : nullptr;
      const int ib = c.d_list ? 0 : ch.i0;
      cudaEventRecord(ev[4 * q], h->stream);
      if (h->prec == DEREK_PREC_FP64)
        launch_x_inv<double>(t, ib, ch.n, c.nchunk, c.n[0], disp_min(h, c.n[0]), c.disp_m, (const double2 *)in,
                             (double2 *)h->d_abuf, nullptr, h->stream);
      else
        launch_x_inv<float>(t, ib, ch.n, c.nchunk, c.n[0], disp_min(h, c.n[0]), c.disp_m, (const float2 *)in,
                            (float2 *)h->d_abuf, nullptr, h->stream);
      cudaEventRecord(ev[4 * q + 1], h->stream);
      if (h->prec == DEREK_PREC_FP64)
        launch_plane<double>(t, ib, ch.n, c.n[0], c.n[1], c.n[2], disp_min(h, c.n[1]), disp_min(h, c.n[2]),
                             c.disp_m, (double2 *)h->d_abuf, h->d_vloc, h->stream);
      else
        launch_plane<float>(t, ib, ch.n, c.n[0], c.n[1], c.n[2], disp_min(h, c.n[1]), disp_min(h, c.n[2]),
                            c.disp_m, (float2 *)h->d_abuf, h->d_vloc32, h->stream);
      cudaEventRecord(ev[4 * q + 2], h->stream);
      if (h->prec == DEREK_PREC_FP64)
        launch_x_fwd<double>(t, ib, ch.n, c.nchunk, c.n[0], disp_min(h, c.n[0]), c.disp_m,
                             (const double2 *)h->d_abuf, (const double2 *)in, nullptr, (double2 *)h->d_HX,
                             nullptr, h->stream);
      else
        launch_x_fwd<float>(t, ib, ch.n, c.nchunk, c.n[0], disp_min(h, c.n[0]), c.disp_m,
                            (const float2 *)h->d_abuf, (const float2 *)in, nullptr, (float2 *)h->d_HX,
                            nullptr, h->stream);
      cudaEventRecord(ev[4 * q + 3], h->stream);
    }
    DEREK_CUDA(h, cudaEventSynchronize(ev.back()));
    for (size_t q = 0; q < chunks.size(); ++q)
      for (int k = 0; k < 3; ++k) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ev[4 * q + k], ev[4 * q + k + 1]);
        tot[k] += ms;
      }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  DEREK_CUDA(h, cudaGetLastError());
  if (ms_apply) *ms_apply = (tot[0] + tot[1] + tot[2]) / nrep;
  if (ms_stage)
    for (int k = 0; k < 3; ++k) ms_stage[k] = tot[k] / nrep;
  return DEREK_OK;
}

}  // extern "C"
