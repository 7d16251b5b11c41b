/*
 * derek_gpu.h -- C ABI of the GB300 plane-wave Kohn-Sham hot path.
 *
 * The DEReK Fortran driver binds these through iso_c_binding, the same way
 * Source/fft.f90:57-132 binds FFTW: opaque handle as type(c_ptr), scalars by
 * value, arrays as assumed-size C_DOUBLE / C_DOUBLE_COMPLEX buffers.  Every
 * entry point returns an int status (0 = DEREK_OK); derek_gpu_strerror maps a
 * status to text for io_errors (Source/io.f90:885-930).
 *
 * Conventions
 *   units       Hartree atomic units (Ha, bohr), as after io_convert_all
 *               (Source/io.f90:324-358).
 *   cell        column-major like the Fortran cell(3,3): cell[3*j + i] is
 *               cell(i+1, j+1); column j is lattice vector j
 *               (r = cell . frac, Source/basis.f90:166-167).
 *   inv_cell    transpose(2 pi cell^-1) as Source/io.f90:1954, same storage.
 *   grids       flat z-fastest order, index (ix*ny + iy)*nz + iz
 *               (Source/fft.f90:260,273).
 *   G order     the reference's centred standard-box order, x outermost and
 *               z innermost (Source/basis.f90:125-135); a k-point's sphere is
 *               the ordered subsequence with 1/2|k+G|^2 <= ecut.
 *   psi         [band][npw] interleaved complex, G fastest (the reference's
 *               coeff(gvec, kpt, band, spinor) slice for one k, nspinor = 1).
 *   ownership   host arrays stay owned by the caller and are copied; device
 *               memory belongs to the handle.
 *   threading   one host thread per handle; all work runs on the handle's
 *               own CUDA stream.
 */
#ifndef DEREK_GPU_H
#define DEREK_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define DEREK_OK                 0
#define DEREK_ERR_BAD_ARG        1
#define DEREK_ERR_OOM            2
#define DEREK_ERR_CUDA           3
#define DEREK_ERR_NOT_CONVERGED  4
#define DEREK_ERR_CHOLESKY       5
#define DEREK_ERR_NAN            6
#define DEREK_ERR_TIMEOUT        7
#define DEREK_ERR_UNSUPPORTED    8

/* precision modes */
#define DEREK_PREC_FP64   0   /* complex128 psi, FP64 FFTs and contractions */
#define DEREK_PREC_MIXED  1   /* complex64 psi, FP32 FFTs and H.psi, split-BF16
                                 tensor-core contractions (hi + lo per operand,
                                 four products, FP32 accumulation); FP64
                                 Cholesky, Jacobi, occupations, densities,
                                 energies */

/* grid policies for n_fine = 0 */
#define DEREK_GRID_REFERENCE 0  /* basis_prime_fact: {2,3,5,7,11,13}-smooth */
#define DEREK_GRID_SMOOTH23  1  /* {2,3}-smooth */

/* derek_gpu_autotune flags */
#define DEREK_TUNE_RETUNE    1  /* time every candidate even where the cache holds a choice */

typedef struct derek_gpu derek_gpu_t;

/* One independent system.  Mirrors the fields of current_structure /
 * current_params the hot path reads (Source/io.f90:63-114,171-194). */
typedef struct {
  double cell[9];          /* bohr, column-major cell(3,3) */
  double inv_cell[9];      /* transpose(2 pi cell^-1); all zero = derive */
  double ecut;             /* cut_off_energy, Ha */
  double g_fine_scale;     /* Source/io.f90:73 default 2.0 */
  int    n_fine[3];        /* fine FFT grid; zeros = derive (grid_policy) */
  int    grid_policy;      /* DEREK_GRID_* */
  int    nk;               /* number of k-points */
  const double *kpts;      /* nk*3 fractional (reciprocal basis) */
  const double *wk;        /* nk weights summing to 1; NULL = uniform */
  int    nbands;           /* n_electrons + conduction_bands (io.f90:316) */
  int    nspinor;          /* 1, or 2: non-collinear spinor bands */
  double nelec;            /* n_electrons */
  double kT;               /* electronic_temp converted to Ha, > 0 */
  const double *vext;      /* nr FP64 values, or NULL to build from wells */
  int    nwells;           /* Gaussian wells: jellium + sum of wells */
  const double *wells;     /* nwells*5: cx cy cz (fractional) depth width */
} derek_sys_desc;

/* SCF options (keys the reference lacks; defaults in derek_gpu_default_opts). */
typedef struct {
  int    precision;        /* DEREK_PREC_* */
  double mix_alpha;        /* Pulay/linear mixing amplitude */
  double kerker_q0;        /* Kerker wavevector (1/bohr); 0 = no Kerker */
  int    pulay_history;    /* stored (n_in, residual) pairs, <= 16 */
  int    cheb_degree;      /* Chebyshev filter degree per SCF iteration */
  int    first_passes;     /* filter passes in the first SCF iteration */
  int    first_degree;     /* filter degree of those passes */
  uint64_t seed;           /* start-vector hash seed */
  int    use_graph;        /* capture each SCF iteration in a CUDA graph */
  int    use_tensor_cores; /* mixed mode: -1 (default) = tcgen05 split-BF16
                              overlaps and rotations for subspaces of 64
                              or more carried bands, CUDA cores below;
                              2 = tensor-core overlaps and rotations, 1 =
                              overlaps only, at any size; 0 = CUDA cores */
  double density_tol;      /* also require max|n_out - n_in| < density_tol
                              (0 = energy criterion only, as the reference) */
  int    buffer_bands;     /* extra unreported bands carried by the filtered
                              subspace (-1 = max(4, nbands/20)) */
  int    etol_per_electron;/* 1: scf_run's etol is per electron (each system
                              stops at |dF| < etol * nelec) */
  int    init_vectors;     /* start vectors: 0 = hashed random entries; 1 = band
                              b on the b-th lowest-kinetic-energy plane wave of
                              its k-point, plus a 1e-3 hashed perturbation;
                              2 = the wavefunctions stored with set_wfn (a
                              restart from a saved state, as state_write keeps
                              model%wfn, Source/state.f90:612), buffer bands
                              as in 1 */
} derek_scf_opts;

/* Per-system SCF report (Source/electronic.f90:143-146 table row). */
typedef struct {
  double energy;           /* Kohn-Sham total energy of the output density */
  double free_energy;      /* energy - kT * entropy (the converged quantity) */
  double delta;            /* |F - F_prev| of the last iteration */
  double efermi;           /* Fermi level */
  double entropy;
  double e_band, e_hartree, e_xc, e_dc;
  double residual;         /* max|n_out - n_in| of the last iteration */
  int    iterations;
  int    converged;
} derek_scf_report;

void derek_gpu_default_opts(derek_scf_opts *opts);
const char *derek_gpu_strerror(int status);
/* Detail text of the last failure on h (h = NULL: the last failed create). */
const char *derek_gpu_last_error(derek_gpu_t *h);

/* Create a handle over nsys independent systems.  Replaces the set-up the
 * reference spreads over basis_init (Source/basis.f90:65-241), fft_init
 * (Source/fft.f90:139-219), state_init (Source/state.f90:59-168) and
 * pot_external_pot (Source/pot.f90:104-190). */
int derek_gpu_create(derek_gpu_t **h, const derek_sys_desc *sys, int nsys,
                     const derek_scf_opts *opts);
int derek_gpu_destroy(derek_gpu_t *h);

/* Sizes: fine grid, standard box and sphere size of (sys, k); bands as
 * requested and as carried internally (requested + buffer). */
int derek_gpu_grid(derek_gpu_t *h, int sys, int n_fine[3], int n_std[3]);
int derek_gpu_bands(derek_gpu_t *h, int sys, int *nbands, int *nbands_internal);
int derek_gpu_npw(derek_gpu_t *h, int sys, int k, int *npw);

/* Sphere of (sys, k): 0-based row numbers into the standard-box G list
 * (basis.f90:125-135) and the flat fine-grid FFT index of each entry.
 * Parity hook for the G tables (Source/basis.f90:125-149). */
int derek_gpu_gsphere(derek_gpu_t *h, int sys, int k, int32_t *box_rows,
                      int32_t *fft_index, double *kinetic);

/* In-place unnormalised 3D c2c FFT of one fine-grid array of system sys.
 * dir = +1 forward (exponent -i), -1 backward (+i).  Replaces fft_3d with
 * grid='FINE' (Source/fft.f90:222-303). */
int derek_gpu_fft3d(derek_gpu_t *h, int sys, double *inout_interleaved, int dir);

/* Local potential used by H.psi: V_ext + V_H + v_xc on the fine grid (FP64). */
int derek_gpu_set_vloc(derek_gpu_t *h, int sys, const double *vloc);
int derek_gpu_get_vloc(derek_gpu_t *h, int sys, double *vloc);

/* Wavefunction slice of (sys, k): nb bands x npw interleaved complex128. */
int derek_gpu_set_wfn(derek_gpu_t *h, int sys, int k, const double *psi);
int derek_gpu_get_wfn(derek_gpu_t *h, int sys, int k, double *psi);

/* H.psi on the handle's stored wavefunctions of (sys, k) with the current
 * local potential; result copied to hpsi (nb x npw complex128).
 * Replaces pot_apply_wfn (Source/pot.f90:344-382) plus the kinetic term. */
int derek_gpu_apply_h(derek_gpu_t *h, int sys, int k, double *hpsi);

/* n(r) = sum_k w_k sum_b occ[k][b] |psi_kb(r)|^2 / Omega from the stored
 * wavefunctions.  Replaces density_calculate (Source/density.f90:101-130);
 * occ is occ(nbands, nk) as state_data%occ (Source/state.f90:43). */
int derek_gpu_density(derek_gpu_t *h, int sys, const double *occ, double *rho);

/* Non-collinear spinor systems (nspinor = 2).  The reference carries two
 * spinor components in every wavefunction, coeff(gvec, kpt, band, 1:2)
 * (Source/wave.f90:30,164), a 2x2 potential nc_pot(nr, 2, 2)
 * (Source/pot.f90:33,88) and a spin density den%spin(nr, 3)
 * (Source/density.f90:63-64); the products on them are empty stubs there
 * (pot_apply_wfn, Source/pot.f90:344-382; density_calculate,
 * Source/density.f90:101-130).  On a spinor system:
 *   set_wfn / get_wfn / apply_h take coeff(gvec, band, spinor) of one k,
 *     complex128 [2][nbands][npw];
 *   apply_h: (H psi)_s = T psi_s + sum_s' V_ss' psi_s' with V = nc_pot;
 *   overlap: <psi_i|psi_j> summed over both spinors (wave_dot_wfn,
 *     Source/wave.f90:955);
 *   density(_spinor): n = sum w |u|^2 + |d|^2 and the magnetisation
 *     m = sum w psi^H sigma psi = (2 Re u*d, 2 Im u*d, |u|^2 - |d|^2),
 *     mag = [3][nr] real (den%spin(:, 1:3));
 *   set_vloc(v) sets nc_pot = diag(v, v) (H.psi only); set_nc_pot takes the reference's
 *     nc_pot(nr, 2, 2) complex128 (element (n, i, j) at n + nr (i + 2 j)),
 *     nc_pot = V I + mu_B sigma.B with mu_B = 1/2 (Source/xsf.f90:44-51);
 *     it is also the SCF's external potential (set_vext: diag(V_ext));
 *   scf_run / scf_iterate: the non-collinear SCF.  A band holds one
 *     electron; V = nc_ext + (V_H + (v_up + v_down)/2) I + b.sigma with
 *     b = (v_up - v_down)/2 m/|m| from the spin-polarised LDA (Slater + PW92)
 *     of the spin densities (n +/- |m|)/2; Pulay mixing of (n, m); the
 *     energy's double counting is int (V_Hxc n + b.m).  The start
 *     magnetisation is zero unless set_start_magnetisation gives one;
 *     get_magnetisation returns m of the last density pass;
 *   nscf_run: band energies in the frozen nc_pot.
 * A batch mixing spinor and scalar systems runs no SCF or NSCF; the
 * gradient and timing entry points run scalar batches only
 * (DEREK_ERR_UNSUPPORTED). */
int derek_gpu_set_nc_pot(derek_gpu_t *h, int sys, const double *nc_pot);
int derek_gpu_get_nc_pot(derek_gpu_t *h, int sys, double *nc_pot);
/* the SCF's external nc_pot (set_nc_pot, or V_ext on the diagonal) */
int derek_gpu_get_nc_ext(derek_gpu_t *h, int sys, double *nc_pot);
int derek_gpu_density_spinor(derek_gpu_t *h, int sys, const double *occ /* nk*nbands */,
                             double *rho /* nr, or NULL */, double *mag /* 3*nr, or NULL */);
int derek_gpu_get_magnetisation(derek_gpu_t *h, int sys, double *mag /* 3*nr */);
int derek_gpu_set_start_magnetisation(derek_gpu_t *h, int sys, const double *mag /* 3*nr, NULL = zero */);
/* Spin-polarised LDA_X + LDA_C_PW (libxc 6.2.2 conventions) on n points:
 * energy per particle and d(n exc)/dn_up, d(n exc)/dn_down. */
int derek_gpu_xc_lsda(derek_gpu_t *h, long n, const double *rho_up, const double *rho_down,
                      double *exc, double *v_up, double *v_down);

/* LDA (Slater exchange + Perdew-Wang 92 correlation, libxc ids 1 + 12),
 * spin-unpolarised: exc = energy per particle, vxc = potential. */
int derek_gpu_xc_lda(derek_gpu_t *h, long n, const double *rho, double *exc,
                     double *vxc);

/* Overlap S = psi^H psi of the stored wavefunctions of (sys, k):
 * nb x nb complex128, row-major S[i*nb + j] = <psi_i|psi_j>.
 * The reference's wave_dot_* (Source/wave.f90:929-1036), as a full matrix. */
int derek_gpu_overlap(derek_gpu_t *h, int sys, int k, double *s);

/* Overlap S = X^H Y that allocates nothing, for callers that cannot call
 * cudaMalloc (a host code that owns the device memory pool, or that forbids
 * allocation once its set-up is done).  No counterpart in the reference: the
 * handle path above allocates its split-K scratch at derek_gpu_create, this
 * variant keeps it in a 4 MiB file-scope device array instead.
 *   x, y     device pointers, nb rows of npw coefficients, row stride ld
 *            (complex128 for DEREK_PREC_FP64, complex64 for DEREK_PREC_MIXED)
 *   s        device pointer, nb x nb complex128, s[i*nb + j] = <x_i|y_j>
 *   stream   cudaStream_t to launch on (NULL = default stream)
 * Limits: nb <= 128 and npw <= 16 * 4096 = 65536, else DEREK_ERR_UNSUPPORTED.
 * The first call on a device looks up the array's device address, so make
 * that first call before any stream capture.  That address is cached per
 * device and does not survive cudaDeviceReset: do not call this again after
 * resetting a device.  Calls share the array: calls that overlap on the GPU
 * race and give wrong results.  DEREK_ERR_CUDA means one of this call's own
 * launches failed; an error pending from other work is left as it was. */
int derek_gpu_overlap_noalloc(const void *x, const void *y, int nb, int npw, long ld,
                              int precision, void *s, void *stream);

/* Self-consistent field.  scf_iterate runs one iteration on every active
 * system; scf_run iterates until |dF| < etol or max_scf iterations
 * (Source/electronic.f90:86-175).  rep has one entry per system. */
int derek_gpu_scf_iterate(derek_gpu_t *h, derek_scf_report *rep);

/* Try limit of the tensor-core kernels' pipeline-stage waits, for every
 * handle in the process (< 0: the default).  With a small limit a stage wait
 * runs out: the kernel records DEREK_ERR_TIMEOUT, drains its own MMAs (that
 * wait keeps the default limit), frees its tensor memory and returns; the
 * overlap or SCF call reports DEREK_ERR_TIMEOUT and the handle stays usable.
 * For tests of that path; no counterpart in the reference. */
int derek_gpu_set_wait_limit(long iterations);
int derek_gpu_scf_run(derek_gpu_t *h, int max_scf, double etol,
                      derek_scf_report *rep);

/* Replace the external potential of sys (nr FP64 values); the next SCF run
 * starts from it.  The reference's pot_external_pot (Source/pot.f90:104-190)
 * fills ext_pot the same way before state_init hands it to the SCF. */
int derek_gpu_set_vext(derek_gpu_t *h, int sys, const double *vext);
int derek_gpu_get_vext(derek_gpu_t *h, int sys, double *vext);

/* Measurement hooks.  derek_gpu_stream returns the handle's cudaStream_t;
 * derek_gpu_launch_count the number of kernels the library has launched in
 * this process (graph replays count their kernels); derek_gpu_time_apply_h
 * runs H.psi on every band of every k-point nrep times and returns the mean
 * device time per application and per stage kernel (3 values: backward x
 * lines, (y,z) planes with V(r), forward x lines + gather + kinetic; zero
 * for an all-spinor batch, whose 2x2 H.psi is timed as one). */
void *derek_gpu_stream(derek_gpu_t *h);
unsigned long long derek_gpu_launch_count(void);
int derek_gpu_time_apply_h(derek_gpu_t *h, int nrep, double *ms_apply, double *ms_stage);

/* Autotuner.  Times the candidate plans of this handle's shapes on its own
 * tables and buffers and keeps the fastest: the radix sequence of every
 * grid-FFT length, register/fixed-length line kernels against shared-memory
 * four-step kernels with a runtime split per length, the row layout of each
 * grid class's H.psi kernels, tensor or CUDA cores and the split-K length of
 * the overlaps, the rotation path and the Jacobi launch shape.  Every
 * candidate computes the same result.  With cache_path (NULL: no cache) the
 * choices are read from and written to a JSON file keyed by device and
 * shape; DEREK_TUNE_RETUNE re-times what the cache holds.  It overwrites the
 * wavefunction buffers and subspace matrices, so call it right after
 * derek_gpu_create (an SCF starts from its own start vectors).  Scalar
 * systems only.  Replaces the reference's FFTW_ESTIMATE planning
 * (Source/fft.f90:204-212), which chooses without timing.
 * derek_gpu_plan writes the handle's current plan as a JSON object (len
 * bytes available; DEREK_ERR_BAD_ARG when it does not fit). */
int derek_gpu_autotune(derek_gpu_t *h, const char *cache_path, int flags);
int derek_gpu_plan(derek_gpu_t *h, char *buf, int len);
/* Host-only pieces of the autotuner: derek_host_tune_cache_normalise parses
 * a cache file's text and writes it back in the library's own layout
 * (DEREK_ERR_BAD_ARG when it does not parse or fit); derek_host_radix_candidates
 * lists the radix sequences tried for length n as "8x3x3;3x3x8;..." (empty
 * when n has a prime factor above 13). */
int derek_host_tune_cache_normalise(const char *text, char *out, int len);
int derek_host_radix_candidates(int n, char *out, int len);

/* Hellmann-Feynman gradient of the converged free energy with respect to the
 * Gaussian-well parameters of sys: dF/dp = int n(r) dV_ext/dp dr.  Writes
 * (dF/dcx, dF/dcy, dF/dcz, dF/ddepth, dF/dwidth) per well (nwells*5).  The
 * reference parses these wells ($data gaussian_pot, Source/io.f90:1888-1922)
 * but never uses them (Source/pot.f90:165-166).  Needs a system whose V_ext
 * was built from its wells and a converged SCF. */
int derek_gpu_grad_wells(derek_gpu_t *h, int sys, double *grad);

/* Gradient of the density-matching loss L = sum_r (n - n_target)^2 dV with
 * respect to the Gaussian-well parameters of sys, through the converged SCF:
 * one self-consistent linear-response (adjoint) solve: a sum over pairs of
 * the converged leading bands of each k-point (Ritz residual below 1e-7,
 * every occupied band included) and Sternheimer equations on their
 * complement, which takes the unconverged top bands.  No counterpart in the
 * reference.  Needs an FP64 handle over one system and a converged SCF;
 * n_target has nr values; writes L to *loss and nwells*5 derivatives
 * (cx, cy, cz, depth, width order) to grad.  max_iter <= 0 and tol <= 0
 * take defaults (60, 1e-9 relative response residual). */
int derek_gpu_grad_density_loss(derek_gpu_t *h, int sys, const double *n_target, double *loss,
                                double *grad, int max_iter, double tol);

/* Results of the last SCF iteration. */
int derek_gpu_get_eigenvalues(derek_gpu_t *h, int sys, double *eig /* nk*nb */);
int derek_gpu_get_occupations(derek_gpu_t *h, int sys, double *occ /* nk*nb */);
int derek_gpu_get_density(derek_gpu_t *h, int sys, double *rho /* nr */);

/* Non-self-consistent eigenvalues (the bandstructure and dos tasks, whose
 * routines are empty in the reference: Source/spectral.f90:33-44; task
 * keys Source/io.f90:519-527, DOS grid key dos_kpt_mp_grid io.f90:111):
 * Chebyshev-filtered subspace iterations of degree cheb_degree in the
 * potential set with derek_gpu_set_vloc (e.g. a converged one), from the
 * start vectors of init_vectors, until none of the lowest nconv reported
 * eigenvalues (0: all reported) of any k-point moves by eig_tol between
 * iterations.  Bands just below the top of the carried subspace converge
 * slowly (raise buffer_bands for them).  On the mixed path the split-BF16
 * tensor-core products (about 16 significant bits per operand) make the
 * Ritz values move by ~1e-5 relative between iterations; use_tensor_cores
 * = 0 (FP32 CUDA-core products, ~1e-7) allows tighter eig_tol.  On failure
 * the last error names the largest remaining change.  Eigenvalues through
 * derek_gpu_get_eigenvalues.  *iterations may be NULL. */
int derek_gpu_nscf_run(derek_gpu_t *h, int max_iter, double eig_tol, int nconv, int *iterations);

/* Restart: the next scf_run starts system `sys` from this density (nr FP64
 * values, the reference's flat z-fastest order) instead of the uniform one;
 * NULL clears it.  Pairs with derek_io_read_den for a .den restart
 * (Source/state.f90 state_restart, which the reference leaves disabled at
 * Source/derek.f90:71-74). */
int derek_gpu_set_start_density(derek_gpu_t *h, int sys, const double *rho);

/* The reference's output files, host only (no GPU needed).  Binary files are
 * one big-endian Fortran sequential record each (gfortran with
 * -fconvert=big-endian, Source/Makefile:86; 4-byte length markers,
 * subrecords past 2^31 - 9 bytes with negated continuation markers):
 *   .den   n_std(3), charge(nr), spin(nr,3), .true.  Source/density.f90:128-160
 *   .pot   n_std(3), nc_pot(nr,2,2), .true.          Source/pot.f90:194-224
 *   .potex as .pot (the external potential)          Source/state.f90:203-232
 *   .wvfn  n_std(3), coeff(nbox,nk,nb,nspinor), nbands, kpts, .true.
 *                                                     Source/wave.f90:893-921
 * Complex arrays are interleaved (re, im) doubles, column-major; n_std is
 * the standard grid written in the header (the readers require it to
 * match, as pot_read does at Source/pot.f90:329-331); nr is the number of
 * fine-grid points.  NULL spin writes zeros; NULL outputs skip a field. */
int derek_io_write_den(const char *path, const int n_std[3], long long nr, const double *charge,
                       const double *spin);
int derek_io_read_den(const char *path, const int n_std[3], long long nr, double *charge, double *spin);
int derek_io_write_pot(const char *path, const int n_std[3], long long nr, const double *nc_pot);
int derek_io_read_pot(const char *path, const int n_std[3], long long nr, double *nc_pot);
int derek_io_write_wvfn(const char *path, const int n_std[3], long long nbox, int nk, int nb, int nspinor,
                        const double *coeff);
int derek_io_read_wvfn(const char *path, const int n_std[3], long long nbox, int nk, int nb, int nspinor,
                       double *coeff);
/* XSF grid file (Source/xsf.f90:67-128): cell rows in F20.10, one value per
 * line in E20.10, in the array's flat order as the reference writes it. */
int derek_io_write_xsf(const char *path, const double cell[9], const int n_fine[3], const double *data);
/* Formatted grid tables (.fden, .fpot, .fpotex): density_writef
 * (Source/density.f90:165-211) and pot_writef (Source/pot.f90:228-287) row
 * for row, F9.4 values, x outermost; the banner of io_out_file_header is
 * replaced by two comment lines of this library.  charge: nr reals; spin:
 * 3 nr reals (component-major) or NULL for zeros; nc_pot: the reference's
 * nc_pot(nr, 2, 2) complex128. */
int derek_io_write_fden(const char *path, const int n_fine[3], const double *charge, const double *spin);
int derek_io_write_fpot(const char *path, const int n_fine[3], const double *nc_pot);
/* Test hook: largest subrecord in bytes (0 = gfortran's 2147483639). */
int derek_io_set_subrecord_limit(long long bytes);

/* A .info parameter file read as the reference reads it (Source/io.f90
 * io_read_param 360-830, io_freeform_read 836-882, io_block_parse
 * 1765-1937, spell check 2545-2630, io_initialise 299-353 with
 * Source/units.f90 and CODATA 2018, Source/constants.f90:70-104): every key
 * of io.f90:116-162 with its default, the lattice and gaussian_pot /
 * lorentzian_pot blocks, keys within Levenshtein distance 1-2 corrected,
 * output_level's write flags, and the unit conversions.  Units accepted:
 * length bohr m cm mm mum nm A pm; energy Ha mHa eV meV Ry mRy J Hz MHz GHz
 * THz cm-1; K; fields Ha/Bohr/e eV/A/e N/C T G agr.  On error the message
 * holds the reference's error text; on success the keys it corrected. */
typedef struct {
  int    check, debugging, n_electrons, max_scf, conduction_bands, nbands, iprint, random_seed;
  int    write_wvfn, soc, write_density, write_potential, write_state, write_spec, write_memory,
         write_formatted_potential, write_potex, write_formatted_density, restart,
         write_formatted_potex, write_xsf;
  int    kpt_mp_grid[3], periodic_pot_grid[3], dos_kpt_mp_grid[3];
  double energy_tol, cut_off_energy, g_fine_scale;       /* Ha, Ha, - */
  double electronic_temp;                                /* kT in Ha */
  double finite_barrier_height, finite_barrier_width[3], periodic_pot_amp;   /* Ha, bohr, Ha */
  double ext_efield[3], ext_bfield[3];                   /* atomic units */
  char   xc_functional[32], task[32], scf_method[32], external_pot[32], output_level[32],
         unit_energy[32], unit_length[32], unit_efield[32], unit_bfield[32],
         out_energy_unit[32], out_len_unit[32], out_efield_unit[32], out_bfield_unit[32];
  double cell[9];          /* bohr, column-major cell(3,3), cell(i,:) lattice vector i */
  int    n_pots;           /* rows of a gaussian_pot / lorentzian_pot block (<= 64) */
  double pot_centres[3 * 64], pot_heights[64], pot_widths[64];   /* fractional, Ha, bohr */
  int    n_corrected;      /* keys corrected by the spell check */
} derek_info;
int derek_info_read(const char *path, derek_info *out, char *message, int message_len);

/* Host-only helpers (no GPU needed): the grid and sphere rules the handle
 * uses, exposed so drivers and tests can check them on any machine. */
int derek_host_prime_fact(int n);  /* Source/basis.f90:257-309 */
int derek_host_grid_sizes(const double cell[9], double ecut, double g_fine_scale,
                          int grid_policy, int n_std[3], int n_fine[3]);
/* Sphere of one k-point; writes at most `capacity` rows, returns the count
 * in *npw (call with capacity 0 to size). */
int derek_host_gsphere(const double inv_cell[9], double ecut, const double kfrac[3],
                       const int n_std[3], int capacity, int32_t *box_rows, int *npw);

#ifdef __cplusplus
}
#endif

#endif /* DEREK_GPU_H */
