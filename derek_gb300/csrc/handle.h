// The handle behind derek_gpu_t: host copies of the batch description and
// the device arrays, laid out once at creation.
#pragma once

#include <cstdio>
#include <string>
#include <vector>

#include "subspace.cuh"

struct derek_gpu {
  // ---- configuration
  derek_scf_opts opts;
  int prec = DEREK_PREC_FP64;
  int nsys = 0;
  int nks = 0;
  int nitems = 0;
  int max_n[3] = {0, 0, 0};
  int min_n[3] = {0, 0, 0};
  int max_nmax = 0;        // max over all axes and systems
  int max_nchunk = 0;      // column chunks of the largest sphere
  int max_nb = 0;
  long long total_psi = 0; // elements per psi-shaped buffer
  long long total_abuf = 0;
  long long total_grid = 0;

  // ---- host copies
  std::vector<derek::SysDev> sys;
  std::vector<derek::KSetDev> ks;
  std::vector<int> n_std;          // 3 per system
  std::vector<int> item_ks, item_band;
  std::vector<int32_t> box_rows, fft_index;  // per sphere entry, reference order
  std::vector<double> kin64;                 // reference order
  std::vector<int32_t> perm;                 // column-order entry -> reference entry
  std::vector<double> kin_col;               // kinetic energies, column order
  std::vector<double> vext_host;   // per system grid, concatenated

  // ---- device tables
  derek::Tables tab{};
  // band view for the subspace kernels (overlaps, Cholesky, Jacobi,
  // rotations, filter bounds): equal to tab except that a spinor k-set's
  // band is one row of 2 npw_pad coefficients (nb, nbr halved; npw = npw_pad
  // = 2 npw_pad), its eigenvalue j at eig[item0 + j]
  derek::Tables tab_band{};
  std::vector<derek::KSetDev> ks_band;
  derek::KSetDev *d_ks_band = nullptr;
  int max_nb_band = 0, max_npw_band = 0;
  derek::SysDev *d_sys = nullptr;
  derek::KSetDev *d_ks = nullptr;
  int *d_item_ks = nullptr, *d_item_band = nullptr;
  int *d_ent_col = nullptr, *d_col_start = nullptr;
  short *d_ent_ix = nullptr, *d_col_y = nullptr, *d_col_z = nullptr, *d_col_x0 = nullptr, *d_rows = nullptr;
  int *d_pw_entry = nullptr;   // per item: entry of its band's start plane wave
  double *d_kin64 = nullptr;
  float *d_kin32 = nullptr;
  double2 *d_tw64 = nullptr;
  float2 *d_tw32 = nullptr;

  // ---- device grids (FP64, grid_off per system)
  double *d_vext = nullptr, *d_vloc = nullptr, *d_vhxc = nullptr;
  float *d_vloc32 = nullptr;
  double *d_rho_in = nullptr, *d_rho_out = nullptr;
  // non-collinear systems: 2x2 potential per point (V11, V21, V12, V22) and
  // the magnetisation (mx, my, mz grids of total_grid values each)
  bool any_spinor = false;
  bool all_spinor = true;         // every system has nspinor = 2
  double2 *d_vnc64 = nullptr;
  float2 *d_vnc32 = nullptr;
  double *d_mag = nullptr;
  // non-collinear SCF: external nc_pot, mixed input magnetisation, xc field,
  // mixing history of m, per-system start magnetisation (empty = zero)
  double2 *d_vnc_ext = nullptr;
  double *d_mag_in = nullptr, *d_bxc = nullptr, *d_min_hist = nullptr, *d_mres_hist = nullptr;
  std::vector<std::vector<double>> start_mag;
  std::vector<std::vector<double>> start_rho;   // per system: SCF start density (empty = uniform)
  double *d_exc = nullptr, *d_vxc = nullptr;
  double2 *d_cgrid = nullptr;      // complex work grid
  double *d_partial = nullptr;     // per-k-set density partials
  long long *d_partial_off = nullptr;

  // ---- device psi-shaped buffers (element type by precision)
  void *d_X = nullptr, *d_Y = nullptr, *d_Yp = nullptr, *d_HX = nullptr;
  void *d_abuf = nullptr;          // x-line buffer of the H.psi passes
  double *d_occw = nullptr;        // per item: w_k f / Omega (density weights)
  double *d_eig = nullptr;         // per item
  double *d_occ = nullptr;         // per item: f in [0, 2]
  derek::Axpby *d_coef = nullptr;  // per k-set filter coefficients

  // ---- SCF state (scf.cu)
  derek::SysState *d_state = nullptr;
  double2 *d_S = nullptr, *d_Hs = nullptr, *d_C = nullptr, *d_scratch = nullptr;
  double2 *d_opart = nullptr;                  // overlap split-K partials
  long long *d_mat_off = nullptr, *d_opart_off = nullptr, *d_hist_off = nullptr;
  int *d_status = nullptr, *d_sweeps = nullptr;
  unsigned char *d_rot_img = nullptr;   // tensor-core rotation operands (mixed path)
  derek::Axpby *d_coef_all = nullptr;
  int max_degree = 0;
  double *d_nin_hist = nullptr, *d_res_hist = nullptr;
  double *d_epart = nullptr, *d_gpart = nullptr;
  int hist = 8;
  int max_npw = 0;
  long long max_nr = 0;
  int cur = 0;                                 // psi buffer holding the current subspace
  bool scf_started = false;
  std::vector<long long> mat_off;
  cudaGraphExec_t graph_exec[3] = {nullptr, nullptr, nullptr};  // keyed by starting buffer
  int graph_degree = -1;
  long long graph_nodes[3] = {0, 0, 0};

  // ---- Gaussian wells (Hellmann-Feynman gradient)
  std::vector<double> wells_host;   // 5 per well, all systems
  std::vector<int> well_off;        // nsys + 1
  std::vector<int> wells_define_vext;
  int max_wells = 0;
  double *d_wells = nullptr, *d_cells = nullptr, *d_hfpart = nullptr, *d_hfgrad = nullptr;
  int *d_well_off = nullptr;

  // ---- items grouped by grid size (one launch per class on uneven batches)
  struct ItemClass {
    int n[3];
    int count;
    int nchunk;
    int max_m;     // largest |centred Miller index| (x, y or z) of a sphere entry in the class
    int disp_m;    // row bound the stage kernels are dispatched with (>= max_m; autotuned)
    int *d_list;   // nullptr when the class is the contiguous range of all items
    // the class's items of the still-active systems, used by the SCF's H.psi
    // and density passes once many systems have converged (active_count < 0:
    // the full list)
    std::vector<int> items;
    int *d_active = nullptr;
    int active_count = -1;
    const int *launch_list() const { return active_count >= 0 ? d_active : d_list; }
    int launch_count() const { return active_count >= 0 ? active_count : count; }
  };
  std::vector<ItemClass> classes;
  std::vector<int> ks_max_m;    // per k-set: largest |centred Miller index| of its sphere
  int max_m_all = 0;

  // ---- plan choices the autotuner (autotune.cu) may change; the defaults
  // are the untuned plan
  struct Tune {
    int ksplit = 2048;       // overlap split-K: complex coefficients per CTA (>= kOverlapSplit)
    int overlap_tc = -1;     // -1: opts.use_tensor_cores decides; 0/1: CUDA cores / tensor cores
    int rotate_tc = -1;
    int jacobi_single = 0;   // 1: one CTA per k-set even where the two-CTA cluster fits
    int generic_lines = 0;   // 1: shared-memory line kernels with the runtime splits sys[].lp
    int hpsi_chunk = 0;      // H.psi items per chunk of the three stage launches (0: a class at once)
    std::string source = "default";   // "default", "tuned" or "cache"
  } tune;

  cudaStream_t stream = nullptr;
  std::string last_error;

  void *buf(int i) const { return i == 0 ? d_X : (i == 1 ? d_Y : d_Yp); }
  void *cur_psi() const { return buf(cur); }

  size_t elem_size() const { return prec == DEREK_PREC_FP64 ? sizeof(double2) : sizeof(float2); }
};

namespace derek {

int cuda_status(cudaError_t e, derek_gpu *h, const char *what);
#define DEREK_CUDA(h, call)                                   \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return derek::cuda_status(_e, h, #call); \
  } while (0)

// Runs H.psi for items [item_begin, item_begin+nitems) on `in`, writing
// `out` = alpha H in + beta in + gamma prev with per-k-set coefficients
// (coef = nullptr: plain H in).
int apply_h_items(derek_gpu *h, int item_begin, int nitems, const void *in, const void *prev,
                  void *out, const Axpby *coef);
// Same with a caller-provided table copy (item_shift) and potential (element
// type of the handle's precision).
int apply_h_items_ex(derek_gpu *h, const Tables &base, int item_begin, int nitems, const void *in,
                     const void *prev, void *out, const Axpby *coef, const void *vloc);
// Density of every active system from psi buffer `psi` and per-item weights
// h->d_occw into rho (FP64 grids).
int density_items(derek_gpu *h, const void *psi, double *rho);
// Spinor systems: H.psi over items [item_begin, item_begin + nitems) (all
// items of an all-spinor batch, or the items of one spinor k-set) with the
// same epilogue as apply_h_items, and n, m of every active spinor system
// (rho, h->d_mag).
int apply_spinor_items(derek_gpu *h, int item_begin, int nitems, const void *in, const void *prev,
                       void *out, const Axpby *coef);
// True (with last_error set) when h holds a spinor system: the SCF, NSCF,
// gradients and timing entry points run scalar systems only.
bool reject_spinor(derek_gpu *h, const char *what);
// Subspace pieces of the SCF (scf.cu) the autotuner times: tensor-core
// availability and choice, overlaps S = A^H B and rotations X <- X C over all
// k-sets, with the handle's tuned split and paths.
// Smallest subspace (carried bands per k-set) that the default
// use_tensor_cores = -1 and the autotuner give the tensor cores.  The
// split-BF16 products carry ~2^-16 relative error per element of a rotated
// band: on a 12-band subspace (8 electrons) that left the SCF's free energy
// moving by ~4e-6 Ha per iteration after 200 iterations (measured), and on the
// uneven batch (at most 44 bands) the CUDA-core paths kept 251 of 256
// systems within 1e-6 Ha/e of the FP64 path against 241 with tensor cores;
// at kpts64's 84 bands the tensor cores are faster and within 2.5e-7 Ha/e.
constexpr int kTcMinBands = 64;
bool tc_capable(const derek_gpu *h);
bool use_tc_overlap(const derek_gpu *h);
bool use_tc_rotate(const derek_gpu *h);
int overlap_all(derek_gpu *h, const void *A, const void *B, double2 *out, int hermitize);
int rotate_all(derek_gpu *h, void *X, const double2 *C);
// The host copy of the system table (every system active) back on the
// device: the SCF masks converged systems off there, the primitives
// (apply_h, overlap) work on any system.
int activate_all(derek_gpu *h);
// SCF work lists: compact_classes keeps, per grid class, the items of the
// systems still active (sys_active[s] != 0) and returns true when a list
// changed; reset_classes goes back to the full lists.  Only the all-items
// H.psi and the density pass use them (set while an SCF runs).
bool compact_classes(derek_gpu *h, const std::vector<int> &sys_active);
void reset_classes(derek_gpu *h);
// minimum first argument of the stage launchers: the class's own size, or -1
// to force the shared-memory kernels with runtime line splits
inline int disp_min(const derek_gpu *h, int n) { return h->tune.generic_lines ? -1 : n; }
int density_spinor_items(derek_gpu *h, const void *psi, double *rho);

}  // namespace derek
