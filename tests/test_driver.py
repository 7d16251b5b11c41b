"""derek_gb300.driver: a .info seed run end to end as program derek runs it
(read the parameters, build the external potential, SCF, the dos task,
write the files state_finalise writes).

CPU: the external potentials against the oracle's point-by-point
restatement of pot_external_pot (Source/pot.f90:128-166), quirks included.
GPU: runs of small seeds: the SCF equals a direct handle run, the files read
back as the handle's state, the DOS integrates to the band count, and a
uniform field gives a spinor run whose moment opposes the field.
"""
import os

import numpy as np
import pytest

LATTICE = "$DATA LATTICE\n6.0 0.0 0.0\n0.0 6.0 0.0\n0.0 0.0 6.0\n$ENDDATA LATTICE\n"
BASE = ("unit_energy : Ha\nunit_length : bohr\ncut_off_energy : 4.0\nn_electrons : 2\nconduction_bands : 4\n"
        "electronic_temp : 6000\nmax_scf : 80\nenergy_tol : 1e-10\n")


def write_seed(tmp_path, name, extra):
    seed = str(tmp_path / name)
    with open(seed + ".info", "w") as f:
        f.write(BASE + extra + LATTICE)
    return seed


@pytest.mark.parametrize("extra", [
    "external_pot : jelly\n",
    "external_pot : finite_barrier\nfinite_barrier_height : 2.0\nfinite_barrier_width : 0.6 0.4 0.5\n",
    "external_pot : periodic_pot\nperiodic_pot_amp : 1.5\nperiodic_pot_grid : 1 2 3\n",
    "external_pot : jelly\nunit_bfield : agr\next_bfield : 0.1 -0.2 0.3\n",
])
def test_external_potential_matches_oracle(oracle, tmp_path, extra):
    import derek_gb300 as dg
    from derek_gb300 import driver
    seed = write_seed(tmp_path, "pot", extra)
    p = dg.read_info(seed + ".info")
    n_fine = (10, 8, 6)
    got = driver.external_potential(p, n_fine)
    ref = oracle.external_nc_pot(p, n_fine)
    assert np.max(np.abs(got - ref)) < 1e-15
    assert driver._spinor_needed(got) == bool(np.any(np.asarray(p["ext_bfield"])))


@pytest.mark.gpu
def test_run_finite_barrier_dos_and_files(tmp_path):
    import derek_gb300 as dg
    from derek_gb300 import driver
    seed = write_seed(tmp_path, "fb",
                      "external_pot : finite_barrier\nfinite_barrier_height : -3.0\n"
                      "finite_barrier_width : 0.5 0.5 0.5\ntask : dos\ndos_kpt_mp_grid : 2 2 2\n"
                      "output_level : all\nwrite_xsf : true\n")
    out = driver.run(seed, precision=dg.DEREK_PREC_FP64)
    rep = out["report"]
    assert rep["converged"] and out["nspinor"] == 1
    p = dg.read_info(seed + ".info")
    nc = driver.external_potential(p, out["n_fine"])
    spec = driver.system_from_params(p, nc, 1)
    with dg.Handle(spec) as h:
        r = h.electronic_scf(max_scf=80, etol=1e-10)[0]
        rho = h.density()
    assert abs(r["free_energy"] - rep["free_energy"]) < 1e-10
    names = set(out["files"])
    assert {"fb-FB.potex", "fb.pot", "fb.den", "fb.wvfn", "fb-V.xsf", "fb-FB-V.xsf"} <= names
    nr = int(np.prod(out["n_fine"]))
    charge, _ = dg.read_den(seed + ".den", out["n_std"], nr)
    assert np.max(np.abs(charge.real - rho)) < 1e-9
    assert np.array_equal(dg.read_pot(os.path.join(tmp_path, "fb-FB.potex"), out["n_std"], nr), nc)
    e, d = out["dos"]
    integral = float(np.sum((d[1:] + d[:-1]) * np.diff(e)) / 2.0)
    assert abs(integral - 2 * p["nbands"]) < 1e-3 * p["nbands"]


@pytest.mark.gpu
def test_run_uniform_field_is_spinor(tmp_path):
    import derek_gb300 as dg
    from derek_gb300 import driver
    seed = write_seed(tmp_path, "b", "external_pot : jelly\nunit_bfield : agr\next_bfield : 0.0 0.0 0.4\n"
                                     "write_density : true\n")
    out = driver.run(seed, precision=dg.DEREK_PREC_FP64)
    assert out["nspinor"] == 2 and out["report"]["converged"]
    nr = int(np.prod(out["n_fine"]))
    _, spin = dg.read_den(seed + ".den", out["n_std"], nr)
    moment = spin.real.sum(axis=0)
    assert moment[2] < 0 and abs(moment[0]) < 1e-8 * abs(moment[2]) and abs(moment[1]) < 1e-8 * abs(moment[2])


class _StateStub:
    """The handle methods _write_files reads, over fixed arrays (no GPU)."""

    def __init__(self, nr, nbox, nspinor, rng):
        self.n = rng.uniform(0, 1, nr)
        self.m = rng.standard_normal((3, nr))
        self.v = rng.standard_normal(nr)
        self.vx = rng.standard_normal(nr)
        self.nc = rng.standard_normal((nr, 2, 2)) + 1j * rng.standard_normal((nr, 2, 2))
        self.nc_ext = rng.standard_normal((nr, 2, 2)) + 1j * rng.standard_normal((nr, 2, 2))
        self.box = rng.standard_normal((nbox, 1, 3, 2)) + 0j

    def density(self, sys=0):
        return self.n

    def magnetisation(self, sys=0):
        return self.m

    def get_vloc(self, sys=0):
        return self.v

    def get_vext(self, sys=0):
        return self.vx

    def get_nc_pot(self, sys=0, external=False):
        return self.nc_ext if external else self.nc

    def wavefunction_box(self, sys=0):
        return np.asfortranarray(self.box)


@pytest.mark.parametrize("extra,nspinor,expect", [
    ("external_pot : jelly\noutput_level : all\n", 1,
     {"s-jelly.potex", "s-jelly.fpotex", "s.pot", "s.fpot", "s.den", "s.fden", "s.wvfn"}),
    ("external_pot : finite_barrier\nwrite_potex : true\nwrite_formatted_potex : true\nwrite_xsf : true\n", 1,
     {"s-FB.potex", "s-FB-V.xsf", "s-FB-Bx.xsf", "s-FB-By.xsf", "s-FB-Bz.xsf"}),
    ("external_pot : jelly\nwrite_potential : true\nwrite_formatted_potential : true\n"
     "write_xsf : true\nwrite_density : true\n", 2,
     {"s.pot", "s-V.xsf", "s-Bx.xsf", "s-By.xsf", "s-Bz.xsf", "s.den"}),
])
def test_state_file_names_and_contents(oracle, tmp_path, extra, nspinor, expect):
    """state_finalise's files (Source/state.f90:203-480): which flags write
    which file under which name, and what each holds.  (An output_level line
    would override the single flags, Source/io.f90:763-826.)"""
    import derek_gb300 as dg
    from derek_gb300 import driver
    seed = write_seed(tmp_path, "s", extra)
    p = dg.read_info(seed + ".info")
    n_fine, n_std = (4, 3, 2), (2, 2, 2)
    nr = int(np.prod(n_fine))
    h = _StateStub(nr, int(np.prod(n_std)), nspinor, np.random.default_rng(1))
    nc_ext = driver.external_potential(p, n_fine)
    cell = np.eye(3) * 6.0
    names = driver._write_files(h, p, seed, nc_ext, n_std, n_fine, cell, nspinor)
    assert set(names) == expect
    d = str(tmp_path)
    if "s.den" in expect:
        charge, spin = dg.read_den(os.path.join(d, "s.den"), n_std, nr)
        assert np.array_equal(charge.real, h.n)
        assert np.array_equal(spin.real, h.m.T if nspinor == 2 else np.zeros((nr, 3)))
    if "s.pot" in expect:
        got = dg.read_pot(os.path.join(d, "s.pot"), n_std, nr)
        if nspinor == 2:
            assert np.array_equal(got, h.nc)
        else:
            assert np.array_equal(got[:, 0, 0], h.v + 0j) and not np.any(got[:, 0, 1])
    if "s-V.xsf" in expect:
        nc = h.nc if nspinor == 2 else None
        text = open(os.path.join(d, "s-Bz.xsf")).read()
        from oracle import fortran_records as F
        bz = ((nc[:, 0, 0] - nc[:, 1, 1]) / (2 * oracle.MU_B)).real
        assert text == F.xsf_text(cell, n_fine, bz)
    if "s-jelly.fpotex" in expect:
        from oracle import fortran_records as F
        assert open(os.path.join(d, "s-jelly.fpotex")).read() == F.fpot_text(n_fine, nc_ext)
    if "s.fden" in expect:
        from oracle import fortran_records as F
        assert open(os.path.join(d, "s.fden")).read() == F.fden_text(n_fine, h.n)
    if "s-FB.potex" in expect:
        assert np.array_equal(dg.read_pot(os.path.join(d, "s-FB.potex"), n_std, nr), nc_ext)
