"""DEReK GB300: the plane-wave Kohn-Sham hot path of DEReK on one GB300 GPU.

The compute path is ``libderek_gpu.so`` (hand-written sm_103a CUDA behind the
C ABI in ``include/derek_gpu.h``).  This package is a thin ctypes mirror of
that ABI, named after the reference's Fortran module routines it replaces
(fft_3d, pot_apply_wfn, density_calculate, wave_dot, electronic_scf).  There
is no CPU fallback: loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _abi
from ._abi import (DEREK_PREC_FP64, DEREK_PREC_MIXED, DEREK_GRID_REFERENCE,  # noqa: F401
                   DEREK_GRID_SMOOTH23, DerekError, lib, lib_path)

__all__ = ["Handle", "SystemSpec", "DerekError", "lib", "lib_path", "host_grid_sizes",
           "host_gsphere", "host_prime_fact", "DEREK_PREC_FP64", "DEREK_PREC_MIXED",
           "DEREK_GRID_REFERENCE", "DEREK_GRID_SMOOTH23"]


class SystemSpec:
    """One independent system (the fields of current_structure/current_params
    the hot path reads, Source/io.f90:63-114,171-194), in Ha/bohr."""

    def __init__(self, cell, ecut, kpts, nbands, nelec, kT=0.01, wk=None, vext=None,
                 wells=None, n_fine=None, grid_policy=DEREK_GRID_SMOOTH23, g_fine_scale=2.0,
                 inv_cell=None, nspinor=1):
        self.cell = np.asarray(cell, dtype=np.float64).reshape(3, 3)
        self.inv_cell = None if inv_cell is None else np.asarray(inv_cell, dtype=np.float64).reshape(3, 3)
        self.ecut = float(ecut)
        self.kpts = np.ascontiguousarray(np.asarray(kpts, dtype=np.float64).reshape(-1, 3))
        self.wk = None if wk is None else np.ascontiguousarray(np.asarray(wk, dtype=np.float64))
        self.nbands = int(nbands)
        self.nelec = float(nelec)
        self.kT = float(kT)
        self.vext = None if vext is None else np.ascontiguousarray(np.asarray(vext, dtype=np.float64))
        self.wells = (np.zeros((0, 5)) if wells is None
                      else np.ascontiguousarray(np.asarray(wells, dtype=np.float64).reshape(-1, 5)))
        self.n_fine = (0, 0, 0) if n_fine is None else tuple(int(x) for x in n_fine)
        self.grid_policy = int(grid_policy)
        self.g_fine_scale = float(g_fine_scale)
        self.nspinor = int(nspinor)

    @classmethod
    def from_info(cls, path):
        """The system a .info file describes (read_info), with the
        reference's own grid rule (Source/basis.f90:87-105) and its
        Monkhorst-Pack k-points (Source/io.f90:2016-2031).  A gaussian_pot
        block's rows (centre, height, width) become this build's Gaussian
        wells of depth `height`; the reference evaluates that potential to
        zero (Source/pot.f90:165-166).  kT must be positive here (Fermi
        smearing), so electronic_temp 0, the reference default, is refused."""
        p = read_info(path)
        if not p["electronic_temp"] > 0:
            raise ValueError("electronic_temp must be > 0 (the SCF uses Fermi-Dirac occupations)")
        from .workloads import mp_grid
        wells = None
        if p["external_pot"] == "gaussian_pot" and p["n_pots"] > 0:
            n = p["n_pots"]
            c = np.asarray(p["pot_centres"][:3 * n]).reshape(n, 3)
            wells = np.column_stack([c, p["pot_heights"][:n], p["pot_widths"][:n]])
        return cls(np.asarray(p["cell"]).reshape(3, 3, order="F"), p["cut_off_energy"],
                   mp_grid(p["kpt_mp_grid"]), p["nbands"], float(p["n_electrons"]), kT=p["electronic_temp"],
                   wells=wells, grid_policy=DEREK_GRID_REFERENCE, g_fine_scale=p["g_fine_scale"])

    def to_desc(self, keep):
        d = _abi.SysDesc()
        # column-major storage of cell(3,3): cell[3*j+i] = cell(i+1, j+1)
        for i in range(3):
            for j in range(3):
                d.cell[3 * j + i] = self.cell[i, j]
                if self.inv_cell is not None:
                    d.inv_cell[3 * j + i] = self.inv_cell[i, j]
        d.ecut = self.ecut
        d.g_fine_scale = self.g_fine_scale
        for i in range(3):
            d.n_fine[i] = self.n_fine[i]
        d.grid_policy = self.grid_policy
        d.nk = len(self.kpts)
        keep.append(self.kpts)
        d.kpts = self.kpts.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        if self.wk is not None:
            keep.append(self.wk)
            d.wk = self.wk.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.nbands = self.nbands
        d.nspinor = self.nspinor
        d.nelec = self.nelec
        d.kT = self.kT
        if self.vext is not None:
            keep.append(self.vext)
            d.vext = self.vext.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.nwells = len(self.wells)
        keep.append(self.wells)
        d.wells = self.wells.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        return d


def _check(status, h=None, what=""):
    if status != 0:
        detail = lib.derek_gpu_last_error(h).decode() if lib is not None else ""
        raise DerekError(status, f"{what}: {lib.derek_gpu_strerror(status).decode()} {detail}".strip())


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Handle:
    """Owns one derek_gpu_t over a batch of systems."""

    def __init__(self, systems, precision=DEREK_PREC_FP64, **opts):
        if isinstance(systems, SystemSpec):
            systems = [systems]
        self.systems = list(systems)
        o = _abi.ScfOpts()
        lib.derek_gpu_default_opts(ctypes.byref(o))
        o.precision = int(precision)
        for k, v in opts.items():
            if not hasattr(o, k):
                raise TypeError(f"unknown option {k}")
            setattr(o, k, v)
        self.opts = o
        keep = []
        arr = (_abi.SysDesc * len(self.systems))(*[s.to_desc(keep) for s in self.systems])
        h = ctypes.c_void_p()
        st = lib.derek_gpu_create(ctypes.byref(h), arr, len(self.systems), ctypes.byref(o))
        if st != 0:
            raise DerekError(st, f"derek_gpu_create: {lib.derek_gpu_strerror(st).decode()} "
                                 f"{lib.derek_gpu_last_error(None).decode()}")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib.derek_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- sizes and tables
    def grid(self, sys=0):
        nf = (ctypes.c_int * 3)()
        ns = (ctypes.c_int * 3)()
        _check(lib.derek_gpu_grid(self._h, sys, nf, ns), self._h, "grid")
        return tuple(nf), tuple(ns)

    def bands(self, sys=0):
        """(requested bands, bands carried internally including the buffer)."""
        a, b = ctypes.c_int(), ctypes.c_int()
        _check(lib.derek_gpu_bands(self._h, sys, ctypes.byref(a), ctypes.byref(b)), self._h, "bands")
        return a.value, b.value

    def npw(self, sys=0, k=0):
        n = ctypes.c_int()
        _check(lib.derek_gpu_npw(self._h, sys, k, ctypes.byref(n)), self._h, "npw")
        return n.value

    def gsphere(self, sys=0, k=0):
        n = self.npw(sys, k)
        rows = np.zeros(n, dtype=np.int32)
        fidx = np.zeros(n, dtype=np.int32)
        kin = np.zeros(n, dtype=np.float64)
        _check(lib.derek_gpu_gsphere(self._h, sys, k, rows.ctypes.data_as(ctypes.c_void_p),
                                     fidx.ctypes.data_as(ctypes.c_void_p), _dptr(kin)),
               self._h, "gsphere")
        return rows, fidx, kin

    # ---- reference-facing operations
    def fft_3d(self, grid_values, direction, sys=0):
        """fft_3d(in_grid, 'FINE', dir) of Source/fft.f90:222-303 (unnormalised)."""
        a = np.ascontiguousarray(np.asarray(grid_values, dtype=np.complex128)).copy()
        _check(lib.derek_gpu_fft3d(self._h, sys, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   int(direction)), self._h, "fft3d")
        return a

    def set_vloc(self, v, sys=0):
        v = np.ascontiguousarray(np.asarray(v, dtype=np.float64))
        _check(lib.derek_gpu_set_vloc(self._h, sys, _dptr(v)), self._h, "set_vloc")

    def get_vloc(self, sys=0):
        nf, _ = self.grid(sys)
        v = np.zeros(int(np.prod(nf)))
        _check(lib.derek_gpu_get_vloc(self._h, sys, _dptr(v)), self._h, "get_vloc")
        return v

    def set_wfn(self, psi, sys=0, k=0):
        psi = np.ascontiguousarray(np.asarray(psi, dtype=np.complex128))
        _check(lib.derek_gpu_set_wfn(self._h, sys, k, psi.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
               self._h, "set_wfn")

    def _wfn_shape(self, sys, k):
        """(nbands, npw), or (2, nbands, npw) = coeff(gvec, band, spinor) of
        one k-point for a spinor system (Source/wave.f90:30)."""
        s = self.systems[sys]
        shape = (s.nbands, self.npw(sys, k))
        return shape if s.nspinor == 1 else (2,) + shape

    def get_wfn(self, sys=0, k=0):
        psi = np.zeros(self._wfn_shape(sys, k), dtype=np.complex128)
        _check(lib.derek_gpu_get_wfn(self._h, sys, k, psi.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
               self._h, "get_wfn")
        return psi

    def pot_apply_wfn(self, sys=0, k=0):
        """H psi of the stored wavefunctions (pot_apply_wfn + kinetic)."""
        out = np.zeros(self._wfn_shape(sys, k), dtype=np.complex128)
        _check(lib.derek_gpu_apply_h(self._h, sys, k, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
               self._h, "apply_h")
        return out

    def density_calculate(self, occ, sys=0):
        """n(r) from the stored wavefunctions and occ(nbands, nk)."""
        s = self.systems[sys]
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.float64).reshape(len(s.kpts), s.nbands))
        nf, _ = self.grid(sys)
        rho = np.zeros(int(np.prod(nf)))
        _check(lib.derek_gpu_density(self._h, sys, _dptr(occ), _dptr(rho)), self._h, "density")
        return rho

    def density_spinor(self, occ, sys=0):
        """(n, m) of a spinor system: n(r) and the magnetisation m = (mx, my,
        mz)(r), shape (3, nr), the reference's den%charge / den%spin
        (Source/density.f90:63-64)."""
        s = self.systems[sys]
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.float64).reshape(len(s.kpts), s.nbands))
        nf, _ = self.grid(sys)
        nr = int(np.prod(nf))
        rho = np.zeros(nr)
        mag = np.zeros((3, nr))
        _check(lib.derek_gpu_density_spinor(self._h, sys, _dptr(occ), _dptr(rho), _dptr(mag)),
               self._h, "density_spinor")
        return rho, mag

    def set_nc_pot(self, nc_pot, sys=0):
        """The 2x2 potential of a spinor system, nc_pot[n, i, j] (nr, 2, 2)
        complex as Source/pot.f90:33 holds it: V I + mu_B sigma.B."""
        a = np.asarray(nc_pot, dtype=np.complex128)
        f = np.ascontiguousarray(a.reshape(-1, 2, 2).transpose(2, 1, 0))   # [j][i][n]: n fastest
        _check(lib.derek_gpu_set_nc_pot(self._h, sys, f.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
               self._h, "set_nc_pot")

    def get_nc_pot(self, sys=0, external=False):
        """nc_pot[n, i, j] of a spinor system: the H.psi potential (after an
        SCF, its last input potential), or with external=True the SCF's
        external potential."""
        nf, _ = self.grid(sys)
        nr = int(np.prod(nf))
        f = np.zeros((2, 2, nr), dtype=np.complex128)
        fn = lib.derek_gpu_get_nc_ext if external else lib.derek_gpu_get_nc_pot
        _check(fn(self._h, sys, f.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), self._h, "get_nc_pot")
        return np.ascontiguousarray(f.transpose(2, 1, 0))

    def magnetisation(self, sys=0):
        """m(r) of a spinor system's last density pass, shape (3, nr)."""
        nf, _ = self.grid(sys)
        mag = np.zeros((3, int(np.prod(nf))))
        _check(lib.derek_gpu_get_magnetisation(self._h, sys, _dptr(mag)), self._h, "get_magnetisation")
        return mag

    def set_start_magnetisation(self, mag, sys=0):
        """Start magnetisation (3, nr) of a spinor system's SCF (None: zero)."""
        if mag is None:
            _check(lib.derek_gpu_set_start_magnetisation(self._h, sys, None), self._h, "set_start_magnetisation")
            return
        m = np.ascontiguousarray(np.asarray(mag, dtype=np.float64))
        _check(lib.derek_gpu_set_start_magnetisation(self._h, sys, _dptr(m)), self._h, "set_start_magnetisation")

    def xc_lsda(self, rho_up, rho_down):
        """(eps_xc, v_up, v_down) of the spin-polarised LDA on the GPU."""
        a = np.ascontiguousarray(np.asarray(rho_up, dtype=np.float64))
        b = np.ascontiguousarray(np.asarray(rho_down, dtype=np.float64))
        e, va, vb = np.zeros_like(a), np.zeros_like(a), np.zeros_like(a)
        _check(lib.derek_gpu_xc_lsda(self._h, ctypes.c_long(a.size), _dptr(a), _dptr(b), _dptr(e), _dptr(va),
                                     _dptr(vb)), self._h, "xc_lsda")
        return e, va, vb

    def xc_lda(self, rho):
        rho = np.ascontiguousarray(np.asarray(rho, dtype=np.float64))
        exc = np.zeros_like(rho)
        vxc = np.zeros_like(rho)
        _check(lib.derek_gpu_xc_lda(self._h, ctypes.c_long(rho.size), _dptr(rho), _dptr(exc), _dptr(vxc)),
               self._h, "xc_lda")
        return exc, vxc

    def wave_dot(self, sys=0, k=0):
        """Full overlap matrix S = psi^H psi of the stored wavefunctions."""
        nb = self.systems[sys].nbands
        s = np.zeros((nb, nb), dtype=np.complex128)
        _check(lib.derek_gpu_overlap(self._h, sys, k, s.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
               self._h, "overlap")
        return s

    # ---- SCF
    def electronic_scf(self, max_scf=100, etol=1e-8):
        """Run the SCF to |dF| < etol (Source/electronic.f90:86-175)."""
        rep = (_abi.ScfReport * len(self.systems))()
        st = lib.derek_gpu_scf_run(self._h, int(max_scf), float(etol), rep)
        if st not in (0, _abi.DEREK_ERR_NOT_CONVERGED):
            _check(st, self._h, "scf_run")
        return [_abi.report_dict(r) for r in rep]

    def scf_iterate(self):
        rep = (_abi.ScfReport * len(self.systems))()
        _check(lib.derek_gpu_scf_iterate(self._h, rep), self._h, "scf_iterate")
        return [_abi.report_dict(r) for r in rep]

    def grad_wells(self, sys=0):
        """Hellmann-Feynman dF/d(cx, cy, cz, depth, width) per well, (nwells, 5)."""
        nw = len(self.systems[sys].wells)
        g = np.zeros((nw, 5))
        _check(lib.derek_gpu_grad_wells(self._h, sys, _dptr(g)), self._h, "grad_wells")
        return g

    def grad_density_loss(self, n_target, sys=0, max_iter=60, tol=1e-9):
        """(L, dL/d(cx, cy, cz, depth, width) per well) for L = sum (n - n_target)^2 dV,
        via the adjoint linear-response solve (FP64 handle, converged SCF)."""
        nt = np.ascontiguousarray(np.asarray(n_target, dtype=np.float64))
        nw = len(self.systems[sys].wells)
        g = np.zeros((nw, 5))
        loss = ctypes.c_double()
        _check(lib.derek_gpu_grad_density_loss(self._h, sys, _dptr(nt), ctypes.byref(loss), _dptr(g),
                                               int(max_iter), float(tol)), self._h, "grad_density_loss")
        return loss.value, g

    def eigenvalues(self, sys=0):
        s = self.systems[sys]
        e = np.zeros((len(s.kpts), s.nbands))
        _check(lib.derek_gpu_get_eigenvalues(self._h, sys, _dptr(e)), self._h, "eigenvalues")
        return e

    def occupations(self, sys=0):
        s = self.systems[sys]
        e = np.zeros((len(s.kpts), s.nbands))
        _check(lib.derek_gpu_get_occupations(self._h, sys, _dptr(e)), self._h, "occupations")
        return e

    def set_vext(self, v, sys=0):
        v = np.ascontiguousarray(np.asarray(v, dtype=np.float64))
        _check(lib.derek_gpu_set_vext(self._h, sys, _dptr(v)), self._h, "set_vext")

    def get_vext(self, sys=0):
        nf, _ = self.grid(sys)
        v = np.zeros(int(np.prod(nf)))
        _check(lib.derek_gpu_get_vext(self._h, sys, _dptr(v)), self._h, "get_vext")
        return v

    def stream(self):
        """The handle's cudaStream_t as an integer (for external event timing)."""
        return int(lib.derek_gpu_stream(self._h) or 0)

    def time_apply_h(self, nrep=5):
        """Mean device ms of one H.psi over every band and k-point, and of its
        three stage kernels."""
        tot = ctypes.c_double()
        stage = (ctypes.c_double * 3)()
        _check(lib.derek_gpu_time_apply_h(self._h, int(nrep), ctypes.byref(tot), stage), self._h,
               "time_apply_h")
        return tot.value, list(stage)

    def autotune(self, cache_path=None, retune=False):
        """Time the candidate FFT radix plans, line splits, row layouts and
        subspace-kernel shapes on this handle and keep the fastest
        (derek_gpu_autotune); with cache_path the choices are read from and
        written to that JSON file.  Call it right after creating the handle:
        it overwrites the wavefunction buffers.  Returns the plan."""
        path = None if cache_path is None else os.fspath(cache_path).encode()
        _check(lib.derek_gpu_autotune(self._h, path, _abi.DEREK_TUNE_RETUNE if retune else 0), self._h,
               "autotune")
        return self.plan()

    def plan(self):
        """The handle's current plan (radices, line kernels, row layouts,
        overlap/rotation paths, Jacobi shape) as a dict."""
        import json
        buf = ctypes.create_string_buffer(1 << 16)
        _check(lib.derek_gpu_plan(self._h, buf, len(buf)), self._h, "plan")
        return json.loads(buf.value.decode())

    def density(self, sys=0):
        nf, _ = self.grid(sys)
        rho = np.zeros(int(np.prod(nf)))
        _check(lib.derek_gpu_get_density(self._h, sys, _dptr(rho)), self._h, "density")
        return rho

    # ---- bandstructure and dos (non-self-consistent)
    def nscf(self, max_iter=200, eig_tol=1e-9, nconv=0):
        """Eigenvalues (nk, nbands) per system in the potential set with
        set_vloc (set_nc_pot on spinor systems), the lowest nconv bands (0:
        all) converged to eig_tol Ha; returns (eigenvalues list, iterations)."""
        it = ctypes.c_int()
        _check(lib.derek_gpu_nscf_run(self._h, int(max_iter), float(eig_tol), int(nconv), ctypes.byref(it)),
               self._h, "nscf_run")
        return [self.eigenvalues(s) for s in range(len(self.systems))], it.value

    def dos(self, energies, sigma=0.01, sys=0):
        """Density of states per Ha (both spins) of the last eigenvalues:
        sum_k w_k sum_b g g_sigma(E - e_kb), Gaussian of width sigma Ha, with
        g = 2 for scalar bands and 1 for spinor bands."""
        s = self.systems[sys]
        eig = self.eigenvalues(sys)
        wk = np.full(len(s.kpts), 1.0 / len(s.kpts)) if s.wk is None else np.asarray(s.wk)
        return dos_gaussian(eig, wk, energies, sigma, degeneracy=2.0 / s.nspinor)

    # ---- files and restart
    def set_start_density(self, rho, sys=0):
        """The next electronic_scf starts system sys from this density (None:
        the uniform start again)."""
        if rho is None:
            _check(lib.derek_gpu_set_start_density(self._h, sys, None), self._h, "set_start_density")
            return
        rho = np.ascontiguousarray(np.asarray(rho, dtype=np.float64))
        _check(lib.derek_gpu_set_start_density(self._h, sys, _dptr(rho)), self._h, "set_start_density")

    def wavefunction_box(self, sys=0):
        """All wavefunctions in the reference's wavefunction%coeff layout:
        (n_std product, nk, nbands, 2) complex128, the sphere's coefficients
        at their box rows (Source/basis.f90:125-149 order), zeros elsewhere
        and, for a scalar system, in the second spinor component
        (Source/wave.f90:164)."""
        s = self.systems[sys]
        _, ns = self.grid(sys)
        nbox = int(np.prod(ns))
        c = np.zeros((nbox, len(s.kpts), s.nbands, 2), dtype=np.complex128, order="F")
        for k in range(len(s.kpts)):
            rows, _, _ = self.gsphere(sys, k)
            psi = self.get_wfn(sys, k)
            if s.nspinor == 1:
                c[rows, k, :, 0] = psi.T
            else:
                for sp in range(2):
                    c[rows, k, :, sp] = psi[sp].T
        return c

    def write_state(self, seed, sys=0):
        """seed.den, seed.pot, seed.potex and seed.wvfn of system sys as the
        reference writes them (Source/state.f90:203-232 and the type-bound
        writers): the last density, the local potential and the external
        potential (on the spin diagonal for a scalar system; a spinor system
        writes its magnetisation as den%spin and its 2x2 potentials), and the
        wavefunctions."""
        nf, ns = self.grid(sys)
        nr = int(np.prod(nf))
        spinor = self.systems[sys].nspinor == 2
        spin = self.magnetisation(sys).T.astype(np.complex128) if spinor else None
        write_den(seed + ".den", ns, self.density(sys).astype(np.complex128), spin)
        if spinor:
            write_pot(seed + ".pot", ns, self.get_nc_pot(sys))
            write_pot(seed + ".potex", ns, self.get_nc_pot(sys, external=True))
        else:
            for ext, v in ((".pot", self.get_vloc(sys)), (".potex", self.get_vext(sys))):
                nc = np.zeros((nr, 2, 2), dtype=np.complex128, order="F")
                nc[:, 0, 0] = v
                nc[:, 1, 1] = v
                write_pot(seed + ext, ns, nc)
        write_wvfn(seed + ".wvfn", ns, self.wavefunction_box(sys))

    def restart_density(self, path, sys=0):
        """Start the next SCF of system sys from the charge (and, for a
        spinor system, the magnetisation) in a .den file."""
        nf, ns = self.grid(sys)
        charge, spin = read_den(path, ns, int(np.prod(nf)))
        self.set_start_density(charge.real, sys)
        if self.systems[sys].nspinor == 2:
            self.set_start_magnetisation(np.ascontiguousarray(spin.real.T), sys)


def dos_gaussian(eig, wk, energies, sigma, degeneracy=2.0):
    """sum_k w_k sum_b d exp(-(E - e_kb)^2 / (2 sigma^2)) / (sigma sqrt(2 pi)),
    d = degeneracy (2 for scalar bands, 1 for spinor bands)."""
    e = np.asarray(energies, dtype=np.float64)[:, None, None]
    g = np.exp(-0.5 * ((e - np.asarray(eig)[None]) / sigma) ** 2) / (sigma * np.sqrt(2 * np.pi))
    return degeneracy * np.einsum("ekb,k->e", g, np.asarray(wk, dtype=np.float64))


def read_info(path):
    """A .info parameter file read as the reference reads it (derek_info_read):
    every parameter by name, in Ha and bohr after the unit conversions;
    'corrected' lists the keys the spell check corrected.  Raises DerekError
    with the reference's message on a bad file."""
    p = _abi.InfoParams()
    msg = ctypes.create_string_buffer(512)
    st = lib.derek_info_read(str(path).encode(), ctypes.byref(p), msg, 512)
    if st != 0:
        raise DerekError(st, f"read_info: {msg.value.decode()}")
    out = {}
    for name, t in _abi.InfoParams._fields_:
        v = getattr(p, name)
        if t is _abi._c32:
            out[name] = bytes(v).split(b"\0", 1)[0].decode()
        elif hasattr(v, "__len__"):
            out[name] = list(v)
        else:
            out[name] = v
    out["corrected"] = msg.value.decode()
    return out


# ---- the reference's files (host only)
def _ns(n_std):
    return (ctypes.c_int * 3)(*[int(x) for x in n_std])


def _cplx(a, shape):
    a = np.asarray(a, dtype=np.complex128).reshape(shape, order="F")
    return np.ascontiguousarray(a.ravel(order="F").view(np.float64))


def write_den(path, n_std, charge, spin=None):
    """Binary .den (Source/density.f90:128-160): charge (nr,) and spin (nr, 3)."""
    nr = int(np.size(charge))
    c = _cplx(charge, (nr,))
    sp = None if spin is None else _dptr(_cplx(spin, (nr, 3)))
    _check(lib.derek_io_write_den(str(path).encode(), _ns(n_std), nr, _dptr(c), sp), None, "write_den")


def read_den(path, n_std, nr):
    c = np.zeros(2 * nr)
    sp = np.zeros(6 * nr)
    _check(lib.derek_io_read_den(str(path).encode(), _ns(n_std), int(nr), _dptr(c), _dptr(sp)), None,
           "read_den")
    return c.view(np.complex128), sp.view(np.complex128).reshape((nr, 3), order="F")


def write_pot(path, n_std, nc_pot):
    """Binary .pot / .potex (Source/pot.f90:194-224): nc_pot (nr, 2, 2)."""
    nr = np.asarray(nc_pot).shape[0]
    v = _cplx(nc_pot, (nr, 2, 2))
    _check(lib.derek_io_write_pot(str(path).encode(), _ns(n_std), nr, _dptr(v)), None, "write_pot")


def read_pot(path, n_std, nr):
    v = np.zeros(8 * nr)
    _check(lib.derek_io_read_pot(str(path).encode(), _ns(n_std), int(nr), _dptr(v)), None, "read_pot")
    return v.view(np.complex128).reshape((nr, 2, 2), order="F")


def write_wvfn(path, n_std, coeff):
    """Binary .wvfn (Source/wave.f90:893-921): coeff (nbox, nk, nbands, nspinor)."""
    shape = np.asarray(coeff).shape
    c = _cplx(coeff, shape)
    _check(lib.derek_io_write_wvfn(str(path).encode(), _ns(n_std), shape[0], shape[1], shape[2], shape[3],
                                   _dptr(c)), None, "write_wvfn")


def read_wvfn(path, n_std, nbox, nk, nb, nspinor=2):
    c = np.zeros(2 * nbox * nk * nb * nspinor)
    _check(lib.derek_io_read_wvfn(str(path).encode(), _ns(n_std), int(nbox), int(nk), int(nb), int(nspinor),
                                  _dptr(c)), None, "read_wvfn")
    return c.view(np.complex128).reshape((nbox, nk, nb, nspinor), order="F")


def write_xsf(path, cell, n_fine, data):
    """XSF grid file of real values (Source/xsf.f90:67-128)."""
    cm = (ctypes.c_double * 9)(*np.asarray(cell, dtype=np.float64).reshape(3, 3).ravel(order="F"))
    d = np.ascontiguousarray(np.asarray(data, dtype=np.float64))
    _check(lib.derek_io_write_xsf(str(path).encode(), cm, _ns(n_fine), _dptr(d)), None, "write_xsf")


def write_fden(path, n_fine, charge, spin=None):
    """Formatted density table (.fden, Source/density.f90:165-211): charge
    (nr,) real and spin (3, nr) real or None."""
    c = np.ascontiguousarray(np.asarray(charge, dtype=np.float64).real)
    sp = None if spin is None else _dptr(np.ascontiguousarray(np.asarray(spin, dtype=np.float64).real))
    _check(lib.derek_io_write_fden(str(path).encode(), _ns(n_fine), _dptr(c), sp), None, "write_fden")


def write_fpot(path, n_fine, nc_pot):
    """Formatted potential table (.fpot / .fpotex, Source/pot.f90:228-287):
    nc_pot (nr, 2, 2) complex."""
    nr = np.asarray(nc_pot).shape[0]
    v = _cplx(nc_pot, (nr, 2, 2))
    _check(lib.derek_io_write_fpot(str(path).encode(), _ns(n_fine), _dptr(v)), None, "write_fpot")


def set_subrecord_limit(nbytes=0):
    """Largest Fortran subrecord written (0: gfortran's 2^31 - 9 bytes)."""
    _check(lib.derek_io_set_subrecord_limit(int(nbytes)), None, "subrecord_limit")


def launch_count() -> int:
    """Kernels launched by the library in this process (graph replays included)."""
    return int(lib.derek_gpu_launch_count())


def host_prime_fact(n: int) -> int:
    return int(lib.derek_host_prime_fact(int(n)))


def host_grid_sizes(cell, ecut, g_fine_scale=2.0, policy=DEREK_GRID_REFERENCE):
    c = (ctypes.c_double * 9)()
    cell = np.asarray(cell, dtype=np.float64).reshape(3, 3)
    for i in range(3):
        for j in range(3):
            c[3 * j + i] = cell[i, j]
    ns = (ctypes.c_int * 3)()
    nf = (ctypes.c_int * 3)()
    _check(lib.derek_host_grid_sizes(c, float(ecut), float(g_fine_scale), int(policy), ns, nf),
           None, "grid_sizes")
    return tuple(ns), tuple(nf)


def host_gsphere(inv_cell, ecut, kfrac, n_std):
    c = (ctypes.c_double * 9)()
    inv_cell = np.asarray(inv_cell, dtype=np.float64).reshape(3, 3)
    for i in range(3):
        for j in range(3):
            c[3 * j + i] = inv_cell[i, j]
    k = (ctypes.c_double * 3)(*[float(x) for x in kfrac])
    ns = (ctypes.c_int * 3)(*[int(x) for x in n_std])
    n = ctypes.c_int()
    _check(lib.derek_host_gsphere(c, float(ecut), k, ns, 0, None, ctypes.byref(n)), None, "gsphere")
    rows = np.zeros(n.value, dtype=np.int32)
    _check(lib.derek_host_gsphere(c, float(ecut), k, ns, n.value, rows.ctypes.data_as(ctypes.c_void_p),
                                  ctypes.byref(n)), None, "gsphere")
    return rows
