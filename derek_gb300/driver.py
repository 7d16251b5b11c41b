"""The reference's program flow on the GPU library: read seed.info, build the
system, run the SCF, the task's non-self-consistent step, and write the files
the parameters ask for.

Follows Source/derek.f90:58-113 (initialise, electronic_minimise,
state_finalise), Source/pot.f90:104-190 (pot_external_pot) and
Source/state.f90:172-480 (the files state_finalise writes, with their
names).  The control flow is host code; every H.psi, density, subspace and
SCF step runs in libderek_gpu.
"""
from __future__ import annotations

import os

import numpy as np

from . import (DEREK_GRID_REFERENCE, DEREK_PREC_MIXED, Handle, SystemSpec, dos_gaussian,
               host_grid_sizes, read_info, read_pot, write_den, write_fden, write_fpot, write_pot,
               write_wvfn, write_xsf)
from .workloads import mp_grid

MU_B = 0.5   # Bohr magneton, atomic units (Source/constants.f90:102)

# file-name tags of the preset external potentials (Source/state.f90:208-219)
POT_TAG = {"finite_barrier": "FB", "periodic_pot": "PP", "jelly": "jelly",
           "gaussian_pot": "local", "lorentzian_pot": "local"}


def frac_points(n_fine):
    """The reference's real grid, frac = i/n with i = 1..n
    (Source/basis.f90:156-188), z fastest, shape (N, 3)."""
    f = [np.arange(1, n + 1, dtype=np.float64) / n for n in n_fine]
    fx, fy, fz = np.meshgrid(*f, indexing="ij")
    return np.stack([fx.ravel(), fy.ravel(), fz.ravel()], axis=1)


def external_potential(p, n_fine):
    """nc_pot of the external potential as pot_external_pot builds it
    (Source/pot.f90:104-190), shape (nr, 2, 2) complex:
      jelly          0.5 Ne / N on the diagonal;
      finite_barrier 0.5 height where every |frac - 1/2| < width / 2 (the
                     width, converted to bohr, is compared with fractional
                     coordinates, as the reference does);
      periodic_pot   0.5 amp sin(2 pi g1 x) sin(2 pi g2 x) sin(2 pi g3 x),
                     all three factors on the x coordinate, as the
                     reference writes them;
      gaussian_pot, lorentzian_pot  zero (the block's rows are read, the
                     potential is left unset);
      a .potex file  its nc_pot, read back.
    The uniform external field ext_bfield adds mu_B sigma.B."""
    nr = int(np.prod(n_fine))
    kind = p["external_pot"]
    nc = np.zeros((nr, 2, 2), dtype=np.complex128)
    if kind == "jelly":
        v = np.full(nr, 0.5 * p["n_electrons"] / nr)
    elif kind == "finite_barrier":
        t = frac_points(n_fine) - 0.5
        inside = np.all(np.abs(t) < np.asarray(p["finite_barrier_width"]) / 2.0, axis=1)
        v = np.where(inside, 0.5 * p["finite_barrier_height"], 0.0)
    elif kind == "periodic_pot":
        x = frac_points(n_fine)[:, 0]
        g = p["periodic_pot_grid"]
        v = 0.5 * p["periodic_pot_amp"] * np.sin(2 * np.pi * g[0] * x) * np.sin(2 * np.pi * g[1] * x) * \
            np.sin(2 * np.pi * g[2] * x)
    elif kind in ("gaussian_pot", "lorentzian_pot"):
        v = np.zeros(nr)
    else:
        raise ValueError(f"{kind} is not a preset external potential: read the .potex with read_pot")
    nc[:, 0, 0] = v
    nc[:, 1, 1] = v
    b = np.asarray(p["ext_bfield"], dtype=np.float64)
    nc[:, 0, 0] += MU_B * b[2]
    nc[:, 1, 1] -= MU_B * b[2]
    nc[:, 0, 1] += MU_B * (b[0] - 1j * b[1])
    nc[:, 1, 0] += MU_B * (b[0] + 1j * b[1])
    return nc


def _spinor_needed(nc):
    """A collinear, spin-independent nc_pot runs on scalar bands."""
    return bool(np.any(nc[:, 0, 1]) or np.any(nc[:, 1, 0]) or np.any(nc[:, 0, 0] != nc[:, 1, 1])
                or np.any(nc[:, 0, 0].imag))


def system_from_params(p, nc, nspinor):
    """The system of the parameters: the reference's nbands (n_electrons +
    conduction_bands, Source/io.f90:316) bands, which are spinor bands in a
    non-collinear run, as the reference's own always are."""
    cell = np.asarray(p["cell"]).reshape(3, 3, order="F")
    return SystemSpec(cell, p["cut_off_energy"], mp_grid(p["kpt_mp_grid"]), p["nbands"],
                      float(p["n_electrons"]), kT=p["electronic_temp"], vext=nc[:, 0, 0].real.copy(),
                      grid_policy=DEREK_GRID_REFERENCE, g_fine_scale=p["g_fine_scale"], nspinor=nspinor)


def run(seed, precision=DEREK_PREC_MIXED, dos_energies=None, dos_sigma=0.01, **opts):
    """Run seed.info as program derek does; returns a dict with the SCF
    report, the band energies, the DOS (task dos) and the files written.

    A spinor (non-collinear) calculation runs when the external potential
    couples or splits the spins (ext_bfield, or a .potex with a field).
    electronic_temp must be positive (Fermi-Dirac occupations).  The band
    energies of the dos / bandstructure step converge to 1e-6 Ha (mixed) or
    1e-9 Ha (FP64) on CUDA-core subspace contractions."""
    p = read_info(seed + ".info")
    if not p["electronic_temp"] > 0:
        raise ValueError("electronic_temp must be > 0 (the SCF uses Fermi-Dirac occupations)")
    cell = np.asarray(p["cell"]).reshape(3, 3, order="F")
    n_std, n_fine = host_grid_sizes(cell, p["cut_off_energy"], p["g_fine_scale"], DEREK_GRID_REFERENCE)
    kind = p["external_pot"]
    if kind in POT_TAG:
        nc = external_potential(p, n_fine)
    else:
        nc = read_pot(kind, n_std, int(np.prod(n_fine)))
    nspinor = 2 if _spinor_needed(nc) else 1
    spec = system_from_params(p, nc, nspinor)
    out = {"nspinor": nspinor, "n_fine": tuple(n_fine), "n_std": tuple(n_std), "files": []}
    with Handle(spec, precision=precision, **opts) as h:
        if nspinor == 2:
            h.set_nc_pot(nc)
        rep = h.electronic_scf(max_scf=p["max_scf"], etol=p["energy_tol"])[0]
        out["report"] = rep
        out["eigenvalues"] = h.eigenvalues()
        if p["task"] in ("dos", "bandstructure"):
            kpts = mp_grid(p["dos_kpt_mp_grid"]) if p["task"] == "dos" else spec.kpts
            nspec = SystemSpec(cell, spec.ecut, kpts, spec.nbands, spec.nelec, kT=spec.kT, vext=spec.vext,
                               grid_policy=DEREK_GRID_REFERENCE, g_fine_scale=spec.g_fine_scale,
                               nspinor=nspinor)
            nopts = dict(opts)
            nopts["use_tensor_cores"] = 0
            with Handle(nspec, precision=precision, **nopts) as g:
                if nspinor == 2:
                    g.set_nc_pot(h.get_nc_pot())
                else:
                    g.set_vloc(h.get_vloc())
                eig = g.nscf(max_iter=300, eig_tol=1e-6 if precision == DEREK_PREC_MIXED else 1e-9,
                             nconv=spec.nbands)[0][0]
            out["nscf_eigenvalues"] = eig
            if p["task"] == "dos":
                e = dos_energies if dos_energies is not None else \
                    np.linspace(eig.min() - 5 * dos_sigma, eig.max() + 5 * dos_sigma, 400)
                wk = np.full(len(kpts), 1.0 / len(kpts))
                out["dos"] = (e, dos_gaussian(eig, wk, e, dos_sigma, degeneracy=2.0 / nspinor))
        out["files"] = _write_files(h, p, seed, nc, n_std, n_fine, cell, nspinor)
    return out


def _nc_of(h, nspinor, which):
    if nspinor == 2:
        return h.get_nc_pot(external=(which == "ext"))
    v = h.get_vloc() if which == "tot" else h.get_vext()
    nc = np.zeros((v.size, 2, 2), dtype=np.complex128)
    nc[:, 0, 0] = v
    nc[:, 1, 1] = v
    return nc


def _xsf_components(path_stem, nc, cell, n_fine, written):
    """-V, -Bx, -By, -Bz .xsf files of an nc_pot (Source/xsf.f90:44-51)."""
    comps = {"V": (nc[:, 0, 0] + nc[:, 1, 1]) / 2.0,
             "Bx": (nc[:, 0, 1] + nc[:, 1, 0]) / (MU_B * 2.0),
             "By": (nc[:, 0, 1] - nc[:, 1, 0]) / (-MU_B * 2j),
             "Bz": (nc[:, 0, 0] - nc[:, 1, 1]) / (2.0 * MU_B)}
    for tag, data in comps.items():
        f = f"{path_stem}-{tag}.xsf"
        write_xsf(f, cell, n_fine, np.ascontiguousarray(data.real))
        written.append(f)


def _write_files(h, p, seed, nc_ext, n_std, n_fine, cell, nspinor):
    """The files of state_finalise (Source/state.f90:203-480).  A formatted
    potential is written as XSF components when write_xsf is set, else as a
    .fpot / .fpotex table; .fpotex goes to its own file (the reference's
    formatted branch writes to the binary .potex unit instead)."""
    written = []
    preset = p["external_pot"] in POT_TAG
    ext_stem = f"{seed}-{POT_TAG[p['external_pot']]}" if preset else seed
    if p["write_potex"]:
        f = ext_stem + ".potex"
        write_pot(f, n_std, _nc_of(h, nspinor, "ext") if nspinor == 2 else nc_ext)
        written.append(f)
    if p["write_formatted_potex"]:
        if p["write_xsf"]:
            _xsf_components(ext_stem, nc_ext, cell, n_fine, written)
        else:
            f = ext_stem + ".fpotex"
            write_fpot(f, n_fine, nc_ext)
            written.append(f)
    if p["write_potential"]:
        f = seed + ".pot"
        write_pot(f, n_std, _nc_of(h, nspinor, "tot"))
        written.append(f)
    if p["write_formatted_potential"]:
        if p["write_xsf"]:
            _xsf_components(seed, _nc_of(h, nspinor, "tot"), cell, n_fine, written)
        else:
            f = seed + ".fpot"
            write_fpot(f, n_fine, _nc_of(h, nspinor, "tot"))
            written.append(f)
    if p["write_density"]:
        f = seed + ".den"
        spin = h.magnetisation().T.astype(np.complex128) if nspinor == 2 else None
        write_den(f, n_std, h.density().astype(np.complex128), spin)
        written.append(f)
    if p["write_formatted_density"]:
        f = seed + ".fden"
        write_fden(f, n_fine, h.density(), h.magnetisation() if nspinor == 2 else None)
        written.append(f)
    if p["write_wvfn"]:
        f = seed + ".wvfn"
        write_wvfn(f, n_std, h.wavefunction_box())
        written.append(f)
    return [os.path.basename(f) for f in written]
